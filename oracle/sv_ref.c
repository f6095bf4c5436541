/* Plain-C complex128 restatement of the reference statevector kernels.
 *
 * TEST INFRASTRUCTURE ONLY: the large-state oracle (28 qubits = 4 GiB of
 * complex128) for the GPU parity tests and nothing else.  The product library
 * never links it.  Built by oracle/build.py into oracle/_build/.
 *
 * Conventions follow TyxonQ's src/tyxonq/libs/quantum_library/kernels:
 *   - a state is 2^n complex128 amplitudes (interleaved re, im); viewed C-order
 *     as (2,)*n, axis q is qubit q, so qubit q is index bit n-1-q
 *     (statevector.py:28-59);
 *   - a 2q matrix U acts on the index 2*bit(q0) + bit(q1)
 *     (statevector.py:45-59, gates.py:82-160); q0 == q1 leaves psi unchanged
 *     (statevector.py:46-47);
 *   - a Pauli string has codes 0..3 = I, X, Y, Z per qubit, qubit 0 leftmost in
 *     the Kronecker product (pauli.py:65-87).
 * Loops are OpenMP-parallel over disjoint amplitude sets; every reduction sums
 * per-thread partials in thread order (static schedule), so results do not
 * depend on timing.
 */
#include <omp.h>
#include <stdint.h>
#include <string.h>

typedef struct {
  double re, im;
} zc;

static inline zc zmul(zc a, zc b) {
  zc r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}
static inline zc zadd(zc a, zc b) {
  zc r = {a.re + b.re, a.im + b.im};
  return r;
}

/* init_statevector (statevector.py:19-25), generalised to |basis>. */
void orc_init(zc* psi, int n, int64_t basis) {
  const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) {
    psi[i].re = 0.0;
    psi[i].im = 0.0;
  }
  psi[basis].re = 1.0;
}

/* apply_1q_statevector (statevector.py:28-42): psi'[..a..] = sum_b U[a][b]
 * psi[..b..] on axis q.  U is row-major 2x2 complex (8 doubles). */
void orc_apply_1q(zc* psi, int n, int q, const double* Ud) {
  const zc* U = (const zc*)Ud;
  const int b = n - 1 - q;
  const int64_t half = (int64_t)1 << (n - 1);
  const int64_t lo = ((int64_t)1 << b) - 1;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < half; ++k) {
    const int64_t i0 = ((k & ~lo) << 1) | (k & lo);
    const int64_t i1 = i0 | ((int64_t)1 << b);
    const zc a0 = psi[i0], a1 = psi[i1];
    psi[i0] = zadd(zmul(U[0], a0), zmul(U[1], a1));
    psi[i1] = zadd(zmul(U[2], a0), zmul(U[3], a1));
  }
}

/* apply_2q_statevector (statevector.py:45-59): U (row-major 4x4 complex, 32
 * doubles) on the index 2*bit(q0) + bit(q1). */
void orc_apply_2q(zc* psi, int n, int q0, int q1, const double* Ud) {
  if (q0 == q1) return;
  const zc* U = (const zc*)Ud;
  const int b0 = n - 1 - q0, b1 = n - 1 - q1;
  const int blo = b0 < b1 ? b0 : b1, bhi = b0 < b1 ? b1 : b0;
  const int64_t quarter = (int64_t)1 << (n - 2);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < quarter; ++k) {
    int64_t i = k;
    i = ((i >> blo) << (blo + 1)) | (i & (((int64_t)1 << blo) - 1));
    i = ((i >> bhi) << (bhi + 1)) | (i & (((int64_t)1 << bhi) - 1));
    int64_t idx[4];
    for (int s = 0; s < 4; ++s)
      idx[s] = i | ((int64_t)((s >> 1) & 1) << b0) | ((int64_t)(s & 1) << b1);
    zc a[4];
    for (int s = 0; s < 4; ++s) a[s] = psi[idx[s]];
    for (int r = 0; r < 4; ++r) {
      zc acc = {0.0, 0.0};
      for (int c = 0; c < 4; ++c) acc = zadd(acc, zmul(U[r * 4 + c], a[c]));
      psi[idx[r]] = acc;
    }
  }
}

/* probabilities |psi_i|^2 (engine.py:377-465 before normalisation; the GPU
 * engine returns them unnormalised, as StatevectorEngine.probability does,
 * engine.py:1041-1047). */
void orc_probs(const zc* psi, int n, double* p) {
  const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; ++i) p[i] = psi[i].re * psi[i].re + psi[i].im * psi[i].im;
}

static double sum_partials(const double* part, int nt) {
  double s = 0.0;
  for (int t = 0; t < nt; ++t) s += part[t];
  return s;
}

/* Re <psi|P|psi> for one Pauli string, P = kron of codes[0..n-1] with qubit 0
 * leftmost (pauli_string_to_matrix, pauli.py:65-71), applied without forming
 * it: per qubit, X flips the bit, Z gives (-1)^bit, Y flips with i*(-1)^bit. */
static double term_expectation(const zc* psi, int n, const uint8_t* codes, double* part, int nt) {
  int64_t flip = 0, zy = 0;
  int ny = 0;
  for (int q = 0; q < n; ++q) {
    const int64_t bit = (int64_t)1 << (n - 1 - q);
    if (codes[q] == 1 || codes[q] == 2) flip |= bit;
    if (codes[q] == 2 || codes[q] == 3) zy |= bit;
    if (codes[q] == 2) ++ny;
  }
  /* P|j> = i^ny (-1)^popcount(j & zy) |j ^ flip>, so
   * <psi|P|psi> = i^ny sum_j conj(psi[j ^ flip]) (-1)^popcount(j & zy) psi[j]. */
  const int64_t N = (int64_t)1 << n;
  for (int t = 0; t < nt; ++t) part[t] = 0.0;
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num();
    const int T = omp_get_num_threads();
    const int64_t chunk = (N + T - 1) / T;
    const int64_t j0 = chunk * t, j1 = j0 + chunk < N ? j0 + chunk : N;
    double sr = 0.0, si = 0.0;
    for (int64_t j = j0; j < j1; ++j) {
      const zc a = psi[j ^ flip], b = psi[j];
      /* conj(a) * b */
      double re = a.re * b.re + a.im * b.im, im = a.re * b.im - a.im * b.re;
      if (__builtin_popcountll((uint64_t)(j & zy)) & 1) {
        re = -re;
        im = -im;
      }
      sr += re;
      si += im;
    }
    part[t] = 0.0;
    /* i^ny * (sr + i si): real part */
    switch (ny & 3) {
      case 0: part[t] = sr; break;
      case 1: part[t] = -si; break;
      case 2: part[t] = -sr; break;
      default: part[t] = si; break;
    }
  }
  return sum_partials(part, nt);
}

/* E = Re <psi|H|psi>, H = sum_k coeffs[k] P_k (pauli_string_sum_dense +
 * dynamics.expectation, pauli.py:74-87, dynamics.py:117-126), term by term in
 * input order.  codes: n_terms x n bytes.  part: scratch of >= nt doubles. */
double orc_pauli_expectation(const zc* psi, int n, int n_terms, const uint8_t* codes, const double* coeffs,
                             double* part, int nt) {
  double e = 0.0;
  for (int k = 0; k < n_terms; ++k) e += coeffs[k] * term_expectation(psi, n, codes + (size_t)k * n, part, nt);
  return e;
}

int orc_max_threads(void) { return omp_get_max_threads(); }
