// Host check of sdim_gb300/csrc/nibbles.cuh against integer arithmetic mod d
// for d = 5 and 7: every pair of residues in every lane for add / sub /
// neg / mul / half / scalar multiples, lane get / set / non-zero masks, and
// random words for the lane sums.  Prints "ok" or the first mismatch.
#include <cstdio>
#include <random>

#include "../../sdim_gb300/csrc/nibbles.cuh"

using namespace sdim;

template <int D>
int check() {
  using M = N4<D>;
  for (int j = 0; j < 8; ++j)
    for (int x = 0; x < D; ++x)
      for (int y = 0; y < D; ++y) {
        // the other lanes hold other residues, to catch carries across lanes
        uint32_t a = 0u, b = 0u;
        for (int k = 0; k < 8; ++k) {
          a = M::set(a, k, k == j ? x : (x + k) % D);
          b = M::set(b, k, k == j ? y : (y + 2 * k) % D);
        }
        for (int k = 0; k < 8; ++k) {
          const int xa = M::get(a, k), yb = M::get(b, k);
          if (M::get(M::add(a, b), k) != (xa + yb) % D) return std::printf("add d=%d %d %d\n", D, xa, yb), 1;
          if (M::get(M::sub(a, b), k) != (xa - yb + D) % D) return std::printf("sub d=%d\n", D), 1;
          if (M::get(M::neg(a), k) != (D - xa) % D) return std::printf("neg d=%d\n", D), 1;
          if (M::get(M::mul(a, b), k) != (xa * yb) % D) return std::printf("mul d=%d\n", D), 1;
          if (M::get(M::half(a), k) != ((xa * (xa - 1)) / 2) % D) return std::printf("half d=%d\n", D), 1;
          if (M::get(M::mulc(a, y), k) != (xa * y) % D) return std::printf("mulc d=%d\n", D), 1;
          if (((M::nz(a) >> (4 * k)) & 1u) != (xa != 0 ? 1u : 0u)) return std::printf("nz d=%d\n", D), 1;
        }
      }
  std::mt19937 rng(7 + D);
  for (int rep = 0; rep < 100000; ++rep) {
    uint32_t a = 0u;
    int s = 0;
    for (int k = 0; k < 8; ++k) {
      const int v = (int)(rng() % D);
      a = M::set(a, k, v);
      s += v;
    }
    if (M::rsum(a) != s) return std::printf("rsum d=%d\n", D), 1;
  }
  return 0;
}

int main() {
  if (check<5>() || check<7>()) return 1;
  std::printf("ok\n");
  return 0;
}
