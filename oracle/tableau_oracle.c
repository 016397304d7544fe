/*
 * CPU oracle for the prime-dimension stabilizer-tableau path of sdim.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it; the product never
 * does.  It is a plain-C restatement of sdim's ExtendedTableau and of the
 * per-shot loop of Program._simulate_tableau, kept deliberately close to the
 * reference's own arithmetic:
 *
 *   - int64 blocks in the reference layout block[qudit][generator]
 *     (sdim/tableau/dataclasses.py:30-39, sdim/tableau/tableau_prime.py:76-86);
 *   - lazy reduction: values are reduced only every 64 instructions of a
 *     circuit and inside measure() (sdim/program.py:317-318, 351;
 *     sdim/tableau/tableau_prime.py:284-289);
 *   - X, X_INV, Z, Z_INV, CZ, CZ_INV, SWAP and M_X are applied as the same
 *     compositions of H/P/CNOT the reference uses
 *     (sdim/tableau/tableau_gates.py:27-137, 229-261, 280-329);
 *   - RESET = measure, then X applied (-m mod d) times (sdim/program.py:335-339).
 *
 * Random outcomes and N1 noise come from the Philox4x32-10 stream described in
 * oracle/philox.py (seed, shot, ordinal, domain).  Noise applies X^a then Z^b
 * after the N1 instruction, as the reference's (deprecated) tableau noise
 * function does (sdim/tableau/tableau_gates.py:387-391).
 *
 * Signed overflow is checked on every product and sum; the run reports
 * ORACLE_OVERFLOW instead of continuing with wrapped values.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_OK 0
#define ORACLE_EBADARG -1
#define ORACLE_ENOMEM -2
#define ORACLE_OVERFLOW -3
#define ORACLE_EBADGATE -4

/* gate ids, sdim/gatedata.py:55-102 and sdim/program.py:13-32 */
enum {
  G_I = 0, G_X, G_X_INV, G_Z, G_Z_INV, G_H, G_H_INV, G_P, G_P_INV, G_CNOT,
  G_CNOT_INV, G_CZ, G_CZ_INV, G_SWAP, G_M, G_M_X, G_RESET, G_N1
};

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al., SC'11)                               */
/* ------------------------------------------------------------------ */
void oracle_philox(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void stream(uint64_t seed, int64_t shot, uint32_t ordinal, uint32_t domain, uint32_t out[4]) {
  uint32_t ctr[4] = {ordinal, (uint32_t)((uint64_t)shot & 0xffffffffu),
                     (uint32_t)((uint64_t)shot >> 32), domain};
  uint32_t key[2] = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  oracle_philox(ctr, key, out);
}

static inline int64_t mulshift(uint32_t w, int64_t m) {
  return (int64_t)(((uint64_t)w * (uint64_t)m) >> 32);
}

/* ------------------------------------------------------------------ */
/* Python integer semantics                                           */
/* ------------------------------------------------------------------ */
static inline int64_t pymod(int64_t a, int64_t m) {
  int64_t r = a % m;
  return r < 0 ? r + m : r;
}
static inline int64_t pyfloordiv(int64_t a, int64_t b) { /* b > 0 */
  return (a - pymod(a, b)) / b;
}

typedef struct {
  int n, d, order, phase_order, even;
  int64_t *x, *z, *ph, *dx, *dz, *dph;  /* x[q*n + i]: qudit q, generator i */
  int overflow;
} tab_t;

static inline int64_t ck_mul(tab_t *t, int64_t a, int64_t b) {
  int64_t r;
  if (__builtin_mul_overflow(a, b, &r)) t->overflow = 1;
  return r;
}
static inline int64_t ck_add(tab_t *t, int64_t a, int64_t b) {
  int64_t r;
  if (__builtin_add_overflow(a, b, &r)) t->overflow = 1;
  return r;
}
static inline int64_t ck_sub(tab_t *t, int64_t a, int64_t b) {
  int64_t r;
  if (__builtin_sub_overflow(a, b, &r)) t->overflow = 1;
  return r;
}

#define X(t, q, i) ((t)->x[(size_t)(q) * (t)->n + (i)])
#define Z(t, q, i) ((t)->z[(size_t)(q) * (t)->n + (i)])
#define DX(t, q, i) ((t)->dx[(size_t)(q) * (t)->n + (i)])
#define DZ(t, q, i) ((t)->dz[(size_t)(q) * (t)->n + (i)])

static int tab_alloc(tab_t *t, int n, int d) {
  size_t nn = (size_t)n * n;
  t->n = n; t->d = d;
  t->even = (d % 2 == 0);
  t->order = t->even ? 2 * d : d;          /* dataclasses.py:88-96 */
  t->phase_order = t->even ? 2 : 1;        /* dataclasses.py:98-106 */
  t->overflow = 0;
  t->x = malloc(sizeof(int64_t) * (4 * nn + 2 * (size_t)n));
  if (!t->x) return ORACLE_ENOMEM;
  t->z = t->x + nn; t->dx = t->z + nn; t->dz = t->dx + nn;
  t->ph = t->dz + nn; t->dph = t->ph + n;
  return ORACLE_OK;
}

/* z = I, x = 0, destab_x = I, destab_z = 0, phases 0 (dataclasses.py:30-39, tableau_prime.py:76-86) */
static void tab_reset(tab_t *t) {
  int n = t->n;
  size_t nn = (size_t)n * n;
  memset(t->x, 0, sizeof(int64_t) * (4 * nn + 2 * (size_t)n));
  for (int q = 0; q < n; ++q) { Z(t, q, q) = 1; DX(t, q, q) = 1; }
  t->overflow = 0;
}

/* ExtendedTableau.modulo (tableau_prime.py:88-95, dataclasses.py:41-47) */
static void tab_modulo(tab_t *t) {
  size_t nn = (size_t)t->n * t->n;
  for (size_t k = 0; k < nn; ++k) {
    t->x[k] = pymod(t->x[k], t->d); t->z[k] = pymod(t->z[k], t->d);
    t->dx[k] = pymod(t->dx[k], t->d); t->dz[k] = pymod(t->dz[k], t->d);
  }
  for (int i = 0; i < t->n; ++i) {
    t->ph[i] = pymod(t->ph[i], t->order); t->dph[i] = pymod(t->dph[i], t->order);
  }
}

/* hadamard_optimized (tableau_optimized.py:5-30) */
static void hadamard(tab_t *t, int q) {
  for (int i = 0; i < t->n; ++i) {
    int64_t nx = ck_sub(t, 0, Z(t, q, i)), nz = X(t, q, i);
    t->ph[i] = ck_add(t, t->ph[i], ck_mul(t, ck_mul(t, t->phase_order, nx), nz));
    X(t, q, i) = nx; Z(t, q, i) = nz;
  }
  for (int i = 0; i < t->n; ++i) {
    int64_t nx = ck_sub(t, 0, DZ(t, q, i)), nz = DX(t, q, i);
    t->dph[i] = ck_add(t, t->dph[i], ck_mul(t, ck_mul(t, t->phase_order, nx), nz));
    DX(t, q, i) = nx; DZ(t, q, i) = nz;
  }
}

/* hadamard_inv_optimized (tableau_optimized.py:33-58) */
static void hadamard_inv(tab_t *t, int q) {
  for (int i = 0; i < t->n; ++i) {
    int64_t nx = Z(t, q, i), nz = ck_sub(t, 0, X(t, q, i));
    t->ph[i] = ck_add(t, t->ph[i], ck_mul(t, ck_mul(t, t->phase_order, nx), nz));
    X(t, q, i) = nx; Z(t, q, i) = nz;
  }
  for (int i = 0; i < t->n; ++i) {
    int64_t nx = DZ(t, q, i), nz = ck_sub(t, 0, DX(t, q, i));
    t->dph[i] = ck_add(t, t->dph[i], ck_mul(t, ck_mul(t, t->phase_order, nx), nz));
    DX(t, q, i) = nx; DZ(t, q, i) = nz;
  }
}

/* phase term: x^2 for even d, x(x-1)//2 for odd d (tableau_optimized.py:62-77) */
static inline int64_t p_term(tab_t *t, int64_t x) {
  if (t->even) return ck_mul(t, x, x);
  return pyfloordiv(ck_mul(t, x, ck_sub(t, x, 1)), 2);
}

/* phase_optimized / phase_inv_optimized (tableau_optimized.py:62-96) */
static void phase(tab_t *t, int q, int sign) {
  for (int i = 0; i < t->n; ++i) {
    int64_t x = X(t, q, i), dxv = DX(t, q, i);
    if (sign > 0) {
      t->ph[i] = ck_add(t, t->ph[i], p_term(t, x));
      t->dph[i] = ck_add(t, t->dph[i], p_term(t, dxv));
      Z(t, q, i) = ck_add(t, Z(t, q, i), x);
      DZ(t, q, i) = ck_add(t, DZ(t, q, i), dxv);
    } else {
      t->ph[i] = ck_sub(t, t->ph[i], p_term(t, x));
      t->dph[i] = ck_sub(t, t->dph[i], p_term(t, dxv));
      Z(t, q, i) = ck_sub(t, Z(t, q, i), x);
      DZ(t, q, i) = ck_sub(t, DZ(t, q, i), dxv);
    }
  }
}

/* cnot_optimized / cnot_inv_optimized (tableau_optimized.py:99-118) */
static void cnot(tab_t *t, int c, int tg, int sign) {
  int64_t dm1 = t->d - 1;
  for (int i = 0; i < t->n; ++i) {
    if (sign > 0) {
      X(t, tg, i) = ck_add(t, X(t, tg, i), X(t, c, i));
      Z(t, c, i) = ck_add(t, Z(t, c, i), ck_mul(t, Z(t, tg, i), dm1));
    } else {
      X(t, tg, i) = ck_sub(t, X(t, tg, i), X(t, c, i));
      Z(t, c, i) = ck_sub(t, Z(t, c, i), ck_mul(t, Z(t, tg, i), dm1));
    }
  }
  for (int i = 0; i < t->n; ++i) {
    if (sign > 0) {
      DX(t, tg, i) = ck_add(t, DX(t, tg, i), DX(t, c, i));
      DZ(t, c, i) = ck_add(t, DZ(t, c, i), ck_mul(t, DZ(t, tg, i), dm1));
    } else {
      DX(t, tg, i) = ck_sub(t, DX(t, tg, i), DX(t, c, i));
      DZ(t, c, i) = ck_sub(t, DZ(t, c, i), ck_mul(t, DZ(t, tg, i), dm1));
    }
  }
}

/* apply_X / apply_X_inv / apply_Z / apply_Z_inv compositions (tableau_gates.py:27-137) */
static void apply_x(tab_t *t, int q) {
  if (t->even) { hadamard(t, q); phase(t, q, 1); phase(t, q, 1); hadamard(t, q); }
  else { hadamard(t, q); phase(t, q, -1); hadamard(t, q); hadamard(t, q); phase(t, q, 1); hadamard(t, q); }
}
static void apply_x_inv(tab_t *t, int q) {
  if (t->even) { hadamard(t, q); phase(t, q, 1); phase(t, q, 1); hadamard(t, q); }
  else { hadamard(t, q); phase(t, q, 1); hadamard(t, q); hadamard(t, q); phase(t, q, -1); hadamard(t, q); }
}
static void apply_z(tab_t *t, int q) {
  if (t->even) { phase(t, q, 1); phase(t, q, 1); }
  else { phase(t, q, -1); hadamard(t, q); hadamard(t, q); phase(t, q, 1); hadamard(t, q); hadamard(t, q); }
}
static void apply_z_inv(tab_t *t, int q) {
  if (t->even) { phase(t, q, -1); phase(t, q, -1); }
  else { phase(t, q, 1); hadamard_inv(t, q); hadamard_inv(t, q); phase(t, q, -1); hadamard_inv(t, q); hadamard_inv(t, q); }
}

static int64_t modinv(int64_t a, int64_t m) { /* m prime, 0 < a < m */
  int64_t r = 1, b = a, e = m - 2;
  while (e > 0) { if (e & 1) r = (r * b) % m; b = (b * b) % m; e >>= 1; }
  return r;
}

/* column dot products over qudits k (np.dot over block[:, i]) */
static int64_t coldot(tab_t *t, const int64_t *a, int ia, const int64_t *b, int ib) {
  int64_t s = 0;
  for (int k = 0; k < t->n; ++k)
    s = ck_add(t, s, ck_mul(t, a[(size_t)k * t->n + ia], b[(size_t)k * t->n + ib]));
  return s;
}

/* ExtendedTableau.exponentiate (tableau_prime.py:365-380) */
static void exponentiate(tab_t *t, int col, int64_t e) {
  int64_t dot = coldot(t, t->x, col, t->z, col);
  t->ph[col] = ck_mul(t, t->ph[col], e);
  t->ph[col] = ck_add(t, t->ph[col],
                      ck_mul(t, pyfloordiv(ck_mul(t, ck_mul(t, dot, e), e - 1), 2), t->phase_order));
  for (int k = 0; k < t->n; ++k) {
    X(t, k, col) = ck_mul(t, X(t, k, col), e);
    Z(t, k, col) = ck_mul(t, Z(t, k, col), e);
  }
  t->ph[col] = pymod(t->ph[col], t->order);
}

/* rowsum of generator column p into column i of the given block pair
 * (one iteration of _random_measurement, tableau_prime.py:308-322) */
static void rowsum(tab_t *t, int64_t *bx, int64_t *bz, int64_t *bph, int i, int p, int64_t f) {
  int n = t->n, d = t->d;
  int64_t cp = 0;
  for (int k = 0; k < n; ++k)
    cp = ck_add(t, cp, ck_mul(t, bz[(size_t)k * n + i], ck_mul(t, X(t, k, p), f)));
  int64_t s = coldot(t, t->x, p, t->z, p);
  cp = ck_add(t, cp, ck_mul(t, pyfloordiv(ck_mul(t, ck_mul(t, s, f), f - 1), 2), t->phase_order));
  for (int k = 0; k < n; ++k) {
    bx[(size_t)k * n + i] = pymod(ck_add(t, bx[(size_t)k * n + i], ck_mul(t, X(t, k, p), f)), d);
    bz[(size_t)k * n + i] = pymod(ck_add(t, bz[(size_t)k * n + i], ck_mul(t, Z(t, k, p), f)), d);
  }
  bph[i] = pymod(ck_add(t, ck_add(t, bph[i], ck_mul(t, t->ph[p], f)), ck_mul(t, t->phase_order, cp)),
                 t->order);
}

/* ExtendedTableau.measure + _random_measurement + _det_measurement
 * (tableau_prime.py:262-363).  Returns the outcome; *det gets the flag. */
static int64_t measure(tab_t *t, int q, uint64_t seed, int64_t shot, uint32_t ordinal, int *det) {
  int n = t->n, d = t->d;
  int first = -1;
  for (int i = 0; i < n; ++i) {
    int64_t xp = pymod(X(t, q, i), d);
    if (xp > 0) {
      first = i;
      if (xp != 1) exponentiate(t, first, modinv(xp, d));
      break;
    }
  }
  tab_modulo(t); /* the full reduction inside measure, tableau_prime.py:284-289 */
  if (first >= 0) {
    int p = first;
    for (int i = 0; i < n; ++i) {
      if (DX(t, q, i) != 0) rowsum(t, t->dx, t->dz, t->dph, i, p, pymod(-DX(t, q, i), d));
      if (X(t, q, i) != 0 && i != p) rowsum(t, t->x, t->z, t->ph, i, p, pymod(-X(t, q, i), d));
    }
    for (int k = 0; k < n; ++k) {
      DX(t, k, p) = X(t, k, p);
      DZ(t, k, p) = Z(t, k, p);
    }
    t->dph[p] = t->ph[p];
    for (int k = 0; k < n; ++k) { Z(t, k, p) = 0; X(t, k, p) = 0; }
    Z(t, q, p) = 1;
    uint32_t w[4];
    stream(seed, shot, ordinal, 0, w);
    int64_t m = mulshift(w[0], d);
    t->ph[p] = pymod(-m * t->phase_order, t->order);
    *det = 0;
    return m;
  }
  /* deterministic: ancilla accumulation (tableau_prime.py:348-362) */
  int64_t *ax = calloc((size_t)2 * n, sizeof(int64_t));
  int64_t *az = ax + n;
  int64_t aph = 0;
  for (int i = 0; i < n; ++i) {
    int64_t f = pymod(DX(t, q, i), d);
    if (f == 0) continue;
    int64_t cp = 0;
    for (int k = 0; k < n; ++k) cp = ck_add(t, cp, ck_mul(t, az[k], ck_mul(t, f, X(t, k, i))));
    int64_t s = coldot(t, t->x, i, t->z, i);
    cp = ck_add(t, cp, ck_mul(t, pyfloordiv(ck_mul(t, ck_mul(t, s, f), f - 1), 2), t->phase_order));
    for (int k = 0; k < n; ++k) {
      ax[k] = ck_add(t, ax[k], ck_mul(t, X(t, k, i), f));
      az[k] = ck_add(t, az[k], ck_mul(t, Z(t, k, i), f));
    }
    aph = ck_add(t, aph, ck_add(t, ck_mul(t, f, t->ph[i]), ck_mul(t, t->phase_order, cp)));
  }
  free(ax);
  aph = pymod(aph, t->order);
  *det = 1;
  return pymod(pyfloordiv(-aph, t->phase_order), d);
}

static void snapshot(const tab_t *t, int8_t *dst) {
  size_t nn = (size_t)t->n * t->n;
  const int64_t *blocks[4] = {t->x, t->z, t->dx, t->dz};
  /* order: x, z, ph, dx, dz, dph -- all reduced */
  int8_t *o = dst;
  for (int b = 0; b < 2; ++b) for (size_t k = 0; k < nn; ++k) *o++ = (int8_t)pymod(blocks[b][k], t->d);
  for (int i = 0; i < t->n; ++i) *o++ = (int8_t)pymod(t->ph[i], t->order);
  for (int b = 2; b < 4; ++b) for (size_t k = 0; k < nn; ++k) *o++ = (int8_t)pymod(blocks[b][k], t->d);
  for (int i = 0; i < t->n; ++i) *o++ = (int8_t)pymod(t->dph[i], t->order);
}

size_t oracle_tableau_bytes(int n) { return (size_t)4 * n * n + 2 * (size_t)n; }

/*
 * Runs nshots shots of one program.
 *   ops: nops rows of 5 int64: gate_id, qudit, target, time-in-circuit, channel
 *        (channel: 0 none, 1 'd', 2 'f', 3 'p'); noise_thr: nops thresholds
 *        (identity iff word0 < thr; thr may be 2^32).
 *   out: nshots x nmeas bytes, value | (deterministic << 7).
 *   final_tab: NULL or nshots x oracle_tableau_bytes(n) reduced tableaux.
 *   snaps: NULL or nops x oracle_tableau_bytes(n): state of shot shot0 after
 *          each instruction (including RESET corrections and noise).
 */
int oracle_simulate(int n, int d, int64_t nops, const int64_t *ops, const int64_t *noise_thr,
                    uint64_t seed, int64_t shot0, int64_t nshots, int noise_on, int64_t nmeas,
                    uint8_t *out, int8_t *final_tab, int8_t *snaps, int nthreads) {
  if (n < 1 || d < 2 || d > 127 || nops < 0 || nshots < 0) return ORACLE_EBADARG;
  for (int64_t g = 0; g < nops; ++g) {
    int64_t id = ops[g * 5], q = ops[g * 5 + 1], tg = ops[g * 5 + 2];
    if (id < 0 || id > G_N1) return ORACLE_EBADGATE;
    if (q < 0 || q >= n) return ORACLE_EBADARG;
    if ((id >= G_CNOT && id <= G_SWAP) && (tg < 0 || tg >= n)) return ORACLE_EBADARG;
  }
  int status = ORACLE_OK;
  size_t tb = oracle_tableau_bytes(n);
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
#endif
  {
    tab_t t;
    int local = tab_alloc(&t, n, d);
    if (local != ORACLE_OK) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
      status = local;
    } else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
      for (int64_t s = 0; s < nshots; ++s) {
        int64_t shot = shot0 + s;
        tab_reset(&t);
        uint32_t mord = 0, nord = 0;
        for (int64_t g = 0; g < nops; ++g) {
          int id = (int)ops[g * 5], q = (int)ops[g * 5 + 1], tg = (int)ops[g * 5 + 2];
          int64_t time = ops[g * 5 + 3];
          if (time % 64 == 0) tab_modulo(&t);
          int det = 0;
          int64_t m = -1;
          switch (id) {
            case G_I: break;
            case G_X: apply_x(&t, q); break;
            case G_X_INV: apply_x_inv(&t, q); break;
            case G_Z: apply_z(&t, q); break;
            case G_Z_INV: apply_z_inv(&t, q); break;
            case G_H: hadamard(&t, q); break;
            case G_H_INV: hadamard_inv(&t, q); break;
            case G_P: phase(&t, q, 1); break;
            case G_P_INV: phase(&t, q, -1); break;
            case G_CNOT: cnot(&t, q, tg, 1); break;
            case G_CNOT_INV: cnot(&t, q, tg, -1); break;
            case G_CZ: hadamard_inv(&t, tg); cnot(&t, q, tg, 1); hadamard(&t, tg); break;
            case G_CZ_INV: hadamard_inv(&t, tg); cnot(&t, q, tg, -1); hadamard(&t, tg); break;
            case G_SWAP:
              cnot(&t, q, tg, 1); hadamard(&t, q); hadamard(&t, tg); cnot(&t, q, tg, 1);
              hadamard(&t, q); hadamard(&t, tg); cnot(&t, q, tg, 1); hadamard(&t, tg); hadamard(&t, tg);
              break;
            case G_M: m = measure(&t, q, seed, shot, mord, &det); break;
            case G_M_X: hadamard_inv(&t, q); m = measure(&t, q, seed, shot, mord, &det); break;
            case G_RESET: {
              m = measure(&t, q, seed, shot, mord, &det);
              int64_t steps = pymod(-m, d);
              for (int64_t k = 0; k < steps; ++k) apply_x(&t, q);
              break;
            }
            case G_N1: {
              if (noise_on) {
                /* coin: word (j & 3) of block j >> 2, domain 1; choice: word 0 of
                 * block j, domain 2, drawn only when the coin fires */
                uint32_t cb[4], w[4];
                stream(seed, shot, nord >> 2, 1, cb);
                int64_t thr = noise_thr[g];
                int64_t chan = ops[g * 5 + 4];
                int64_t a = 0, b = 0;
                if ((int64_t)cb[nord & 3] >= thr) {
                  stream(seed, shot, nord, 2, w);
                  if (chan == 1) { int64_t r = 1 + mulshift(w[0], (int64_t)d * d - 1); a = r % d; b = r / d; }
                  else if (chan == 2) { a = 1 + mulshift(w[0], d - 1); }
                  else if (chan == 3) { b = 1 + mulshift(w[0], d - 1); }
                }
                for (int64_t k = 0; k < a; ++k) apply_x(&t, q);
                for (int64_t k = 0; k < b; ++k) apply_z(&t, q);
              }
              nord++;
              break;
            }
            default: break;
          }
          if (m >= 0) {
            if ((int64_t)mord < nmeas) out[s * nmeas + mord] = (uint8_t)(m | (det ? 0x80 : 0));
            mord++;
          }
          if (snaps && s == 0) {
            /* reduced state after the instruction; the reduction is a copy */
            snapshot(&t, snaps + (size_t)g * tb);
          }
        }
        tab_modulo(&t);
        if (final_tab) snapshot(&t, final_tab + (size_t)s * tb);
        if (t.overflow) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
          status = ORACLE_OVERFLOW;
        }
      }
      free(t.x);
    }
  }
  return status;
}
