// Host check of sdim_gb300/csrc/planes3.cuh against integer arithmetic mod 3:
// every pair of residues in every lane for add / sub / mul / neg / half,
// scalar multiples, lane get / set, the exclusive prefix and the
// deterministic-outcome word sums on random words.  Prints "ok" or the
// first mismatch; exit status 0 only when every check passes.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../sdim_gb300/csrc/planes3.cuh"

using namespace sdim;

static P3 pack(const int* r) {
  P3 a = p3_zero();
  for (int j = 0; j < 32; ++j) a = p3_set(a, j, r[j]);
  return a;
}

static int fail(const char* what, int x, int y) {
  std::printf("mismatch in %s (%d, %d)\n", what, x, y);
  return 1;
}

int main() {
  // every (a, b) pair in every lane position
  for (int j = 0; j < 32; ++j)
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) {
        const P3 a = p3_set(p3_zero(), j, x), b = p3_set(p3_zero(), j, y);
        if (p3_get(a, j) != x) return fail("get/set", x, y);
        if (p3_get(p3_add(a, b), j) != (x + y) % 3) return fail("add", x, y);
        if (p3_get(p3_sub(a, b), j) != (x - y + 3) % 3) return fail("sub", x, y);
        if (p3_get(p3_mul(a, b), j) != (x * y) % 3) return fail("mul", x, y);
        if (p3_get(p3_neg(a), j) != (3 - x) % 3) return fail("neg", x, y);
        if (p3_get(p3_mulc(a, y), j) != (x * y) % 3) return fail("mulc", x, y);
        if (p3_get(p3_half(a), j) != (x * (x - 1) / 2) % 3) return fail("half", x, y);
        if (p3_get(p3_splat(x), j) != x) return fail("splat", x, y);
        const P3 s = p3_add(a, b);
        if ((s.p0 & s.p1) != 0u) return fail("add encoding", x, y);
      }
  std::mt19937 rng(12345);
  for (int rep = 0; rep < 20000; ++rep) {
    int ra[32], rb[32], rf[32], rx[32], rz[32];
    for (int j = 0; j < 32; ++j) {
      ra[j] = (int)(rng() % 3);
      rb[j] = (int)(rng() % 3);
      rf[j] = (int)(rng() % 3);
      rx[j] = (int)(rng() % 3);
      rz[j] = (int)(rng() % 3);
    }
    const P3 a = pack(ra), b = pack(rb);
    int sum = 0, pre = 0;
    const P3 e = p3_prefix(a);
    for (int j = 0; j < 32; ++j) {
      if (p3_get(e, j) != pre) return fail("prefix", rep, j);
      if (p3_get(p3_add(a, b), j) != (ra[j] + rb[j]) % 3) return fail("add words", rep, j);
      pre = (pre + ra[j]) % 3;
      sum += ra[j];
    }
    if (p3_rsum(a) != sum) return fail("rsum", rep, sum);
    // deterministic-outcome sums over a row of two words against the
    // per-residue loop (acc += f x pre, pre += f z; dd += h x z)
    int rf2[32], rx2[32], rz2[32];
    for (int j = 0; j < 32; ++j) {
      rf2[j] = (int)(rng() % 3);
      rx2[j] = (int)(rng() % 3);
      rz2[j] = (int)(rng() % 3);
    }
    int acc = 0, p = 0, dref = 0;
    for (int w = 0; w < 2; ++w)
      for (int j = 0; j < 32; ++j) {
        const int f = w ? rf2[j] : rf[j], x = w ? rx2[j] : rx[j], z = w ? rz2[j] : rz[j];
        acc = (acc + f * x * p) % 3;
        p = (p + f * z) % 3;
        dref = (dref + (f * (f - 1) / 2) * x * z) % 3;
      }
    int t = 0, dd = 0, carry = 0;
    const P3 f1 = pack(rf), f2 = pack(rf2);
    carry = p3_det_word(f1, p3_half(f1), pack(rx), pack(rz), carry, t, dd);
    carry = p3_det_word(f2, p3_half(f2), pack(rx2), pack(rz2), carry, t, dd);
    if (t % 3 != acc || dd % 3 != dref || carry != p) return fail("det words", rep, t % 3);
  }
  std::printf("ok\n");
  return 0;
}
