// UCC excitations.  Statevector form (k_exc_*): each excitation rotates the
// pairs of basis states it changes (tq_excitation in tq_sv.h).
// CI-space form: the state restricted to determinants with fixed alpha / beta
// electron counts (real amplitudes).  Each excitation j maps determinant i to
// perm_j[i] with a sign, and evolves
//   c <- c + (1 - cos t_j) f2_j * c + sin t_j * f_j * c[perm_j]
// (reference: chem_libs/quantum_chem_library/civector_ops.py:334-350); the
// reverse sweep un-applies the excitations to ket and bra and takes
// grad_j = sum_i bra_i f_j[i] ket[perm_j[i]] (civector_ops.py:141-200).
// The Hamiltonian is applied in the full statevector: tq_ci_embed scatters the
// CI vector to basis indices (determinant bitstring = basis index), the Pauli
// sum kernels run there, and tq_ci_gather reads the CI components back.
#include "common.cuh"

namespace tq {

__global__ void k_ci_step(const double* __restrict__ in, double* __restrict__ out, int64_t D,
                          const int32_t* __restrict__ perm, const int8_t* __restrict__ ph,
                          const int8_t* __restrict__ ph2, double s, double omc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const double c = in[i];
    out[i] = c + omc * (double)ph2[i] * c + s * (double)ph[i] * in[perm[i]];
  }
}

// Both vectors un-evolved by one excitation (sin -> -sin).
__global__ void k_ci_step2(const double* __restrict__ kin, double* __restrict__ kout, const double* __restrict__ bin,
                           double* __restrict__ bout, int64_t D, const int32_t* __restrict__ perm,
                           const int8_t* __restrict__ ph, const int8_t* __restrict__ ph2, double s, double omc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    const double f2 = omc * (double)ph2[i], f = s * (double)ph[i];
    const int32_t p = perm[i];
    const double k = kin[i], b = bin[i];
    kout[i] = k + f2 * k + f * kin[p];
    bout[i] = b + f2 * b + f * bin[p];
  }
}

__device__ double ci_block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// partials[blockIdx.x] = sum over the block's indices of b[i] * ph[i] * k[perm[i]]
__global__ void k_ci_dot_perm(const double* __restrict__ k, const double* __restrict__ b, int64_t D,
                              const int32_t* __restrict__ perm, const int8_t* __restrict__ ph, double* partials) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
    acc += b[i] * (double)ph[i] * k[perm[i]];
  acc = ci_block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// out[o] = sum_b partials[o * nblk + b] (one block per output, fixed order)
__global__ void k_ci_finalize(const double* partials, int nblk, double* out) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += partials[(int64_t)blockIdx.x * nblk + b];
  acc = ci_block_sum(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

__global__ void k_ci_dot(const double* __restrict__ a, const double* __restrict__ b, int64_t D, double* partials) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  acc = ci_block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

template <typename R>
__global__ void k_ci_embed(const double* __restrict__ civ, const uint64_t* __restrict__ strings, int64_t D,
                           typename C2<R>::T* psi) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
    typename C2<R>::T v;
    v.x = (R)civ[i];
    v.y = R(0);
    psi[strings[i]] = v;
  }
}

template <typename R>
__global__ void k_ci_gather(const typename C2<R>::T* __restrict__ psi, const uint64_t* __restrict__ strings,
                            int64_t D, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)psi[strings[i]].x;
}

// ---------------------------------------------------------------------------
// H in the CI space as CSR (row_ptr[D + 1], col, val): one warp per row, lanes
// stride over the row's entries, fixed shuffle tree (deterministic).
__device__ __forceinline__ double ci_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_ci_spmv(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                          const double* __restrict__ val, int64_t D, const double* __restrict__ x,
                          double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < D; r += nw) {
    double acc = 0.0;
    for (int64_t q = rp[r] + lane; q < rp[r + 1]; q += 32) acc += val[q] * x[col[q]];
    acc = ci_warp_sum(acc);
    if (lane == 0) y[r] = acc;
  }
}

// ---------------------------------------------------------------------------
// One-CTA sweeps over excitation PAIRS.  Excitation j changes only the
// determinants i with fphase_j[i] != 0; they come in pairs (i, p = perm_j[i])
// with fphase_j[p] = -fphase_j[i] and f2phase = -1 on both, and every other
// amplitude is left as it is.  One thread updates both members of a pair in
// place:
//   c_i <- c_i - omc c_i + sin phi c_p,   c_p <- c_p - omc c_p - sin phi c_i
// (phi = fphase_j[i]), so the work per excitation is the pair count, not D.
// Pair entry (int2): x = i, y = (p << 1) | (phi < 0).  pair_start[j] ..
// pair_start[j + 1] index excitation j's pairs; a barrier separates
// excitations.  The entries of the next two excitations are prefetched into
// registers while the current one is applied.
//
// The CTA has NT = 256 or 1024 threads (256 when no excitation has more than
// 512 pairs: a shorter barrier per excitation).
// FP64 issues at a small fraction of the FP32 rate on this GPU (and a CTA
// runs on one SM), so signs are applied by flipping the sign bit with integer
// operations and cross-thread sums are left to k_ci_segsum on many SMs: each
// thread stores its in-thread partial of grad_j (and of the energy) to
// part[part_start[...] + tid].

__device__ __forceinline__ double ci_neg_if(double x, unsigned neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((long long)neg << 63));
}

template <int IT, int NT>
__device__ __forceinline__ void ci_load_pairs(int2 (&r)[IT], const int2* __restrict__ pairs,
                                              const int64_t* ps, int j, int n_ex) {
  if (j < 0 || j >= n_ex) return;
  const int64_t a = ps[j], np = ps[j + 1] - a;
#pragma unroll
  for (int m = 0; m < IT; ++m) {
    const int64_t k = threadIdx.x + (int64_t)m * NT;
    r[m] = k < np ? __ldg(pairs + a + k) : make_int2(-1, 0);
  }
}

template <int IT>
__device__ __forceinline__ void ci_rotate(int2 (&a)[IT], int2 (&b)[IT], int2 (&c)[IT]) {
#pragma unroll
  for (int m = 0; m < IT; ++m) {
    a[m] = b[m];
    b[m] = c[m];
  }
}

// c <- U_j c for one pair (sign = +1 forward, -1 to un-apply).
__device__ __forceinline__ void ci_pair_update(double* c, int i, int p, double t, double mo) {
  const double ci = c[i], cp = c[p];
  c[i] = fma(t, cp, fma(mo, ci, ci));
  c[p] = fma(ci_neg_if(t, 1u), ci, fma(mo, cp, cp));
}

__device__ __forceinline__ bool ci_pair_ok(int2 e, int D) {
  return e.x >= 0 && e.x < D && (e.y >> 1) >= 0 && (e.y >> 1) < D;
}

// Shared memory layout of both sweeps: [vectors][sin, omc per excitation][pair_start][part_start].
template <int IT, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_ci_forward(int D, int init, int n_ex, const int2* __restrict__ pairs, const int64_t* __restrict__ pair_start,
                 const double* __restrict__ sin_omc, double* __restrict__ ket) {
  extern __shared__ double sm[];
  double* c = sm;
  double* so = sm + D;
  int64_t* ps = (int64_t*)(so + 2 * n_ex);
  const int tid = threadIdx.x;
  for (int i = tid; i < 2 * n_ex; i += NT) so[i] = sin_omc[i];
  for (int i = tid; i <= n_ex; i += NT) ps[i] = pair_start[i];
  for (int i = tid; i < D; i += NT) c[i] = (i == init) ? 1.0 : 0.0;
  __syncthreads();
  int2 cur[IT], nx1[IT], nx2[IT];
  ci_load_pairs<IT, NT>(cur, pairs, ps, 0, n_ex);
  ci_load_pairs<IT, NT>(nx1, pairs, ps, 1, n_ex);
  for (int j = 0; j < n_ex; ++j) {
    ci_load_pairs<IT, NT>(nx2, pairs, ps, j + 2, n_ex);
    const double s = so[2 * j], mo = ci_neg_if(so[2 * j + 1], 1u);
#pragma unroll
    for (int m = 0; m < IT; ++m)
      if (ci_pair_ok(cur[m], D)) ci_pair_update(c, cur[m].x, cur[m].y >> 1, ci_neg_if(s, cur[m].y & 1), mo);
    __syncthreads();
    ci_rotate<IT>(cur, nx1, nx2);
  }
  for (int i = tid; i < D; i += NT) ket[i] = c[i];
}

// Energy partials <ket, bra> and, when grad != 0, the reverse sweep: un-apply
// excitation j to ket and bra, then grad_j partial = sum over j's pairs of
// b_i phi k_p - b_p phi k_i (= sum_i bra_i fphase_j[i] ket[fperm_j[i]]).
template <int IT, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_ci_reverse(int D, int n_ex, int grad, const int2* __restrict__ pairs, const int64_t* __restrict__ pair_start,
                 const int64_t* __restrict__ part_start, const double* __restrict__ sin_omc,
                 const double* __restrict__ ket, const double* __restrict__ bra, double* __restrict__ part) {
  extern __shared__ double sm[];
  double* k = sm;
  double* b = sm + D;
  double* so = sm + 2 * D;
  int64_t* ps = (int64_t*)(so + 2 * n_ex);
  const int tid = threadIdx.x;
  for (int i = tid; i < 2 * n_ex; i += NT) so[i] = sin_omc[i];
  for (int i = tid; i <= n_ex; i += NT) ps[i] = pair_start[i];
  double e = 0.0;
  for (int i = tid; i < D; i += NT) {
    const double kv = ket[i], bv = bra[i];
    k[i] = kv;
    b[i] = bv;
    e = fma(kv, bv, e);
  }
  if (tid < (D < NT ? D : NT)) part[part_start[0] + tid] = e;
  if (!grad) return;
  __syncthreads();
  int2 cur[IT], nx1[IT], nx2[IT];
  ci_load_pairs<IT, NT>(cur, pairs, ps, n_ex - 1, n_ex);
  ci_load_pairs<IT, NT>(nx1, pairs, ps, n_ex - 2, n_ex);
  for (int j = n_ex - 1; j >= 0; --j) {
    ci_load_pairs<IT, NT>(nx2, pairs, ps, j - 2, n_ex);
    const double s = ci_neg_if(so[2 * j], 1u), mo = ci_neg_if(so[2 * j + 1], 1u);
    double acc = 0.0;
#pragma unroll
    for (int m = 0; m < IT; ++m) {
      if (!ci_pair_ok(cur[m], D)) continue;
      const int i = cur[m].x, p = cur[m].y >> 1;
      const unsigned neg = cur[m].y & 1;
      const double t = ci_neg_if(s, neg);
      ci_pair_update(k, i, p, t, mo);
      ci_pair_update(b, i, p, t, mo);
      // pairs of one excitation are disjoint: this thread's own updates are the values it reads
      acc = fma(ci_neg_if(b[i], neg), k[p], acc);
      acc = fma(ci_neg_if(b[p], neg ^ 1u), k[i], acc);
    }
    const int64_t np = ps[j + 1] - ps[j];
    if (tid < np) part[part_start[1 + j] + tid] = acc;
    __syncthreads();
    ci_rotate<IT>(cur, nx1, nx2);
  }
}

// out[o] = sum of part[seg[o] .. seg[o + 1]) in index order (one block per output).
__global__ void k_ci_segsum(const double* __restrict__ part, const int64_t* __restrict__ seg, double* out) {
  __shared__ double sh[32];
  const int64_t a = seg[blockIdx.x], z = seg[blockIdx.x + 1];
  double acc = 0.0;
  for (int64_t q = a + threadIdx.x; q < z; q += blockDim.x) acc += part[q];
  acc = ci_block_sum(acc, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

static size_t ci_sweep_smem(int64_t vectors, int64_t D, int n_ex) {
  return sizeof(double) * ((size_t)vectors * D + (size_t)2 * n_ex) + sizeof(int64_t) * (size_t)(n_ex + 1);
}

static int ci_smem_optin() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return v;
}

// ---------------------------------------------------------------------------
// Statevector excitations.  Thread t of the pair range [0, 2^(n-k)) spreads t
// over the non-excitation bits (a zero inserted at each excitation bit,
// ascending), forms s_neg / s_pos and rotates the pair; every other amplitude
// is untouched.
__device__ __forceinline__ bool exc_ok(const tq_excitation& e, int n) {
  if (e.k != 2 && e.k != 4) return false;
  uint64_t all = 0;
  int prev = -1;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    if (b < e.k) {
      if (e.bits[b] <= prev || e.bits[b] >= n) return false;
      prev = e.bits[b];
      all |= 1ull << e.bits[b];
    }
  }
  return (e.m_neg | e.m_pos) == all && (e.m_neg & e.m_pos) == 0 && (e.zmask & all) == 0;
}

__device__ __forceinline__ uint64_t exc_spread(uint64_t x, const tq_excitation& e) {
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    if (b < e.k) {
      const int p = e.bits[b];
      x = ((x >> p) << (p + 1)) | (x & ((1ull << p) - 1));
    }
  }
  return x;
}

template <typename R>
__global__ void k_exc_apply(typename C2<R>::T* __restrict__ psi, int n, const tq_excitation* __restrict__ exc, int j,
                            const double* __restrict__ sincos, int reverse) {
  const tq_excitation e = exc[j];
  if (!exc_ok(e, n)) return;
  const R s = (R)(reverse ? -sincos[2 * j] : sincos[2 * j]), c = (R)sincos[2 * j + 1];
  const uint64_t np = 1ull << (n - e.k);
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < np; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t base = exc_spread(t, e), sn = base | e.m_neg, sp = base | e.m_pos;
    const R f = (__popcll(sn & e.zmask) & 1) ? (e.sign > 0 ? s : -s) : (e.sign > 0 ? -s : s);
    const typename C2<R>::T a = psi[sn], b = psi[sp];
    typename C2<R>::T a2, b2;
    a2.x = c * a.x + f * b.x;
    a2.y = c * a.y + f * b.y;
    b2.x = c * b.x - f * a.x;
    b2.y = c * b.y - f * a.y;
    psi[sn] = a2;
    psi[sp] = b2;
  }
}

// Un-apply excitation j to psi and lam, then this block's part of
// Re sum conj(lam) F psi = sum over pairs phi (Re conj(lam_n) psi_p - Re conj(lam_p) psi_n).
template <typename R>
__global__ void k_exc_adjoint(typename C2<R>::T* __restrict__ psi, typename C2<R>::T* __restrict__ lam, int n,
                              const tq_excitation* __restrict__ exc, int j, const double* __restrict__ sincos,
                              double* __restrict__ part) {
  __shared__ double sh[32];
  const tq_excitation e = exc[j];
  double acc = 0.0;
  if (exc_ok(e, n)) {
    const R s = (R)(-sincos[2 * j]), c = (R)sincos[2 * j + 1];
    const uint64_t np = 1ull << (n - e.k);
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < np;
         t += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t base = exc_spread(t, e), sn = base | e.m_neg, sp = base | e.m_pos;
      const bool odd = __popcll(sn & e.zmask) & 1;
      const bool phi_pos = odd == (e.sign > 0);
      const R f = phi_pos ? s : -s;
      typename C2<R>::T a = psi[sn], b = psi[sp], la = lam[sn], lb = lam[sp];
      typename C2<R>::T a2, b2, la2, lb2;
      a2.x = c * a.x + f * b.x;
      a2.y = c * a.y + f * b.y;
      b2.x = c * b.x - f * a.x;
      b2.y = c * b.y - f * a.y;
      la2.x = c * la.x + f * lb.x;
      la2.y = c * la.y + f * lb.y;
      lb2.x = c * lb.x - f * la.x;
      lb2.y = c * lb.y - f * la.y;
      psi[sn] = a2;
      psi[sp] = b2;
      lam[sn] = la2;
      lam[sp] = lb2;
      const double g = (double)la2.x * (double)b2.x + (double)la2.y * (double)b2.y -
                       ((double)lb2.x * (double)a2.x + (double)lb2.y * (double)a2.y);
      acc += phi_pos ? g : -g;
    }
  }
  acc = ci_block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

static int exc_blocks(int n) {
  // one grid size for every excitation of a state (fixed partial count per excitation)
  const int64_t pairs = n >= 2 ? (1ll << (n - 2)) : 1;
  int64_t b = (pairs + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return (int)(b < 1 ? 1 : b);
}

static int ci_blocks(int64_t D) {
  int64_t b = (D + 255) / 256;
  if (b > 1216) b = 1216;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace tq

using namespace tq;

extern "C" int tq_ci_apply_excitations(double* civ, double* tmp, int64_t D, const int32_t* fperm, const int8_t* fphase,
                                       const int8_t* f2phase, const double* sin_t, const double* omc_t, int n_ex,
                                       int reverse, void* stream) {
  if (D < 1 || n_ex < 0) return fail(TQ_ERR_ARG, "tq_ci_apply_excitations: D=%lld, n_ex=%d", (long long)D, n_ex);
  if (n_ex == 0) return TQ_OK;
  if (!civ || !tmp || !fperm || !fphase || !f2phase || !sin_t || !omc_t)
    return fail(TQ_ERR_ARG, "tq_ci_apply_excitations: NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = ci_blocks(D);
  double* a = civ;
  double* b = tmp;
  for (int k = 0; k < n_ex; ++k) {
    const int j = reverse ? n_ex - 1 - k : k;
    const double sj = reverse ? -sin_t[j] : sin_t[j];
    k_ci_step<<<nb, 256, 0, s>>>(a, b, D, fperm + (int64_t)j * D, fphase + (int64_t)j * D, f2phase + (int64_t)j * D,
                                 sj, omc_t[j]);
    double* t = a;
    a = b;
    b = t;
  }
  if (a != civ) {
    cudaError_t e = cudaMemcpyAsync(civ, a, sizeof(double) * D, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e, "tq_ci_apply_excitations: copy");
  }
  TQ_CHECK_LAUNCH("tq_ci_apply_excitations");
  return TQ_OK;
}

extern "C" size_t tq_ci_adjoint_workspace_bytes(int64_t D, int n_ex) {
  if (D < 1 || n_ex < 0) return 0;
  return sizeof(double) * ((size_t)4 * D + (size_t)ci_blocks(D) * (size_t)(n_ex > 0 ? n_ex : 1));
}

extern "C" int tq_ci_adjoint(const double* ket, const double* bra, int64_t D, const int32_t* fperm,
                             const int8_t* fphase, const int8_t* f2phase, const double* sin_t, const double* omc_t,
                             int n_ex, double* grads, void* ws, size_t ws_bytes, void* stream) {
  if (D < 1 || n_ex < 0) return fail(TQ_ERR_ARG, "tq_ci_adjoint: D=%lld, n_ex=%d", (long long)D, n_ex);
  if (n_ex == 0) return TQ_OK;
  if (!ket || !bra || !fperm || !fphase || !f2phase || !sin_t || !omc_t || !grads)
    return fail(TQ_ERR_ARG, "tq_ci_adjoint: NULL pointer");
  const size_t need = tq_ci_adjoint_workspace_bytes(D, n_ex);
  if (!ws || ws_bytes < need) return fail(TQ_ERR_WORKSPACE, "tq_ci_adjoint: workspace of %zu bytes < %zu", ws_bytes, need);
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = ci_blocks(D);
  double* k0 = (double*)ws;
  double* b0 = k0 + D;
  double* k1 = b0 + D;
  double* b1 = k1 + D;
  double* part = b1 + D;
  cudaError_t e = cudaMemcpyAsync(k0, ket, sizeof(double) * D, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b0, bra, sizeof(double) * D, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_status(e, "tq_ci_adjoint: copy");
  for (int j = n_ex - 1; j >= 0; --j) {
    const int32_t* pj = fperm + (int64_t)j * D;
    const int8_t* phj = fphase + (int64_t)j * D;
    k_ci_step2<<<nb, 256, 0, s>>>(k0, k1, b0, b1, D, pj, phj, f2phase + (int64_t)j * D, -sin_t[j], omc_t[j]);
    k_ci_dot_perm<<<nb, 256, 0, s>>>(k1, b1, D, pj, phj, part + (int64_t)j * nb);
    double* t = k0;
    k0 = k1;
    k1 = t;
    t = b0;
    b0 = b1;
    b1 = t;
  }
  k_ci_finalize<<<n_ex, 256, 0, s>>>(part, nb, grads);
  TQ_CHECK_LAUNCH("tq_ci_adjoint");
  return TQ_OK;
}

extern "C" size_t tq_ci_dot_workspace_bytes(int64_t D) { return D < 1 ? 0 : sizeof(double) * (size_t)ci_blocks(D); }

extern "C" int tq_ci_dot(const double* a, const double* b, int64_t D, double* out_dev, void* ws, size_t ws_bytes,
                         void* stream) {
  if (D < 1) return fail(TQ_ERR_ARG, "tq_ci_dot: D=%lld", (long long)D);
  if (!a || !b || !out_dev) return fail(TQ_ERR_ARG, "tq_ci_dot: NULL pointer");
  if (!ws || ws_bytes < tq_ci_dot_workspace_bytes(D)) return fail(TQ_ERR_WORKSPACE, "tq_ci_dot: workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = ci_blocks(D);
  k_ci_dot<<<nb, 256, 0, s>>>(a, b, D, (double*)ws);
  k_ci_finalize<<<1, 256, 0, s>>>((const double*)ws, nb, out_dev);
  TQ_CHECK_LAUNCH("tq_ci_dot");
  return TQ_OK;
}

extern "C" int tq_ci_embed(const double* civ, const uint64_t* strings, int64_t D, void* psi, int n, int dtype,
                           void* stream) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (D < 1 || !civ || !strings || !psi) return fail(TQ_ERR_ARG, "tq_ci_embed: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t S = dtype == TQ_C64 ? 8 : 16;
  cudaError_t e = cudaMemsetAsync(psi, 0, S << n, s);
  if (e != cudaSuccess) return cuda_status(e, "tq_ci_embed: clear");
  if (dtype == TQ_C64)
    k_ci_embed<float><<<ci_blocks(D), 256, 0, s>>>(civ, strings, D, (float2*)psi);
  else
    k_ci_embed<double><<<ci_blocks(D), 256, 0, s>>>(civ, strings, D, (double2*)psi);
  TQ_CHECK_LAUNCH("tq_ci_embed");
  return TQ_OK;
}

extern "C" int tq_ci_gather(const void* psi, const uint64_t* strings, int64_t D, int dtype, double* out, void* stream) {
  if (dtype != TQ_C64 && dtype != TQ_C128) return fail(TQ_ERR_ARG, "tq_ci_gather: bad dtype %d", dtype);
  if (D < 1 || !psi || !strings || !out) return fail(TQ_ERR_ARG, "tq_ci_gather: bad argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TQ_C64)
    k_ci_gather<float><<<ci_blocks(D), 256, 0, s>>>((const float2*)psi, strings, D, out);
  else
    k_ci_gather<double><<<ci_blocks(D), 256, 0, s>>>((const double2*)psi, strings, D, out);
  TQ_CHECK_LAUNCH("tq_ci_gather");
  return TQ_OK;
}

extern "C" int tq_ci_spmv(const int64_t* row_ptr, const int32_t* col, const double* val, int64_t D, const double* x,
                          double* y, void* stream) {
  if (D < 1 || !row_ptr || !col || !val || !x || !y) return fail(TQ_ERR_ARG, "tq_ci_spmv: bad argument");
  int64_t nb = (D + 7) / 8;
  if (nb > 152 * 16) nb = 152 * 16;
  k_ci_spmv<<<(int)nb, 256, 0, (cudaStream_t)stream>>>(row_ptr, col, val, D, x, y);
  TQ_CHECK_LAUNCH("tq_ci_spmv");
  return TQ_OK;
}

extern "C" int64_t tq_ci_pairs_max_dim(int n_ex) {
  if (n_ex < 0) return 0;
  const int64_t optin = ci_smem_optin();
  const int64_t fixed = (int64_t)ci_sweep_smem(0, 0, n_ex);
  const int64_t d = (optin - fixed) / (2 * (int64_t)sizeof(double));
  return d > 0 ? d : 0;
}

extern "C" size_t tq_ci_energy_grad_workspace_bytes(int64_t D, int64_t n_partials) {
  if (D < 1 || n_partials < 0) return 0;
  return sizeof(double) * ((size_t)2 * D + (size_t)n_partials);
}

extern "C" int tq_ci_energy_grad(int64_t D, int64_t init_index, int n_ex, const int32_t* pairs,
                                 const int64_t* pair_start, int64_t max_pairs, const int64_t* part_start,
                                 int64_t n_partials, const double* sin_omc, const int64_t* row_ptr, const int32_t* col,
                                 const double* val, int grad, int threads, double* ket_out, double* out, void* ws,
                                 size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_ci_energy_grad");
  if (D < 1 || n_ex < 0 || init_index < 0 || init_index >= D || max_pairs < 0 || n_partials < 1)
    return fail(TQ_ERR_ARG, "tq_ci_energy_grad: D=%lld, n_ex=%d, init=%lld, max_pairs=%lld, n_partials=%lld",
                (long long)D, n_ex, (long long)init_index, (long long)max_pairs, (long long)n_partials);
  if (D > tq_ci_pairs_max_dim(n_ex))
    return fail(TQ_ERR_RANGE, "tq_ci_energy_grad: D=%lld above the one-CTA limit %lld for %d excitations",
                (long long)D, (long long)tq_ci_pairs_max_dim(n_ex), n_ex);
  if (threads != 256 && threads != 1024)
    return fail(TQ_ERR_ARG, "tq_ci_energy_grad: %d threads per sweep (256 or 1024)", threads);
  if (max_pairs > 2 * (int64_t)threads)
    return fail(TQ_ERR_RANGE, "tq_ci_energy_grad: %lld pairs in one excitation (at most %d with %d threads)",
                (long long)max_pairs, 2 * threads, threads);
  if (!pair_start || !part_start || !row_ptr || !col || !val || !out || (n_ex > 0 && (!pairs || !sin_omc)))
    return fail(TQ_ERR_ARG, "tq_ci_energy_grad: NULL pointer");
  const size_t need = tq_ci_energy_grad_workspace_bytes(D, n_partials);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_ci_energy_grad: workspace of %zu bytes < %zu", ws_bytes, need);
  cudaStream_t s = (cudaStream_t)stream;
  double* ket = ket_out ? ket_out : (double*)ws;
  double* bra = (double*)ws + D;
  double* part = bra + D;
  const int2* pr = (const int2*)pairs;
  const size_t smem_f = ci_sweep_smem(1, D, n_ex), smem_r = ci_sweep_smem(2, D, n_ex);
#define TQ_CI_SWEEPS(IT, NT)                                                                                     \
  do {                                                                                                           \
    cudaError_t e = cudaFuncSetAttribute(k_ci_forward<IT, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                         (int)smem_f);                                                           \
    if (e == cudaSuccess)                                                                                        \
      e = cudaFuncSetAttribute(k_ci_reverse<IT, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_r); \
    if (e != cudaSuccess) return cuda_status(e, "tq_ci_energy_grad: shared memory");                             \
    k_ci_forward<IT, NT><<<1, NT, smem_f, s>>>((int)D, (int)init_index, n_ex, pr, pair_start, sin_omc, ket);     \
    k_ci_spmv<<<spmv_blocks, 256, 0, s>>>(row_ptr, col, val, D, ket, bra);                                      \
    k_ci_reverse<IT, NT><<<1, NT, smem_r, s>>>((int)D, n_ex, grad, pr, pair_start, part_start, sin_omc, ket,     \
                                               bra, part);                                                       \
  } while (0)
  int64_t spmv_blocks = (D + 7) / 8;
  if (spmv_blocks > 152 * 16) spmv_blocks = 152 * 16;
  if (threads == 256) {
    if (max_pairs <= 256)
      TQ_CI_SWEEPS(1, 256);
    else
      TQ_CI_SWEEPS(2, 256);
  } else {
    if (max_pairs <= 1024)
      TQ_CI_SWEEPS(1, 1024);
    else
      TQ_CI_SWEEPS(2, 1024);
  }
#undef TQ_CI_SWEEPS
  k_ci_segsum<<<grad ? 1 + n_ex : 1, 256, 0, s>>>(part, part_start, out);
  TQ_CHECK_LAUNCH("tq_ci_energy_grad");
  return TQ_OK;
}

extern "C" int tq_sv_apply_excitations(void* psi, int n, int dtype, const tq_excitation* exc, int n_ex,
                                       const double* sincos, int reverse, void* stream) {
  TQ_RANGE("tq_sv_apply_excitations");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_ex < 0 || n < 2) return fail(TQ_ERR_ARG, "tq_sv_apply_excitations: n=%d, n_ex=%d", n, n_ex);
  if (n_ex == 0) return TQ_OK;
  if (!psi || !exc || !sincos) return fail(TQ_ERR_ARG, "tq_sv_apply_excitations: NULL pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = exc_blocks(n);
  for (int q = 0; q < n_ex; ++q) {
    const int j = reverse ? n_ex - 1 - q : q;
    if (dtype == TQ_C64)
      k_exc_apply<float><<<nb, 256, 0, s>>>((float2*)psi, n, exc, j, sincos, reverse);
    else
      k_exc_apply<double><<<nb, 256, 0, s>>>((double2*)psi, n, exc, j, sincos, reverse);
  }
  TQ_CHECK_LAUNCH("tq_sv_apply_excitations");
  return TQ_OK;
}

extern "C" size_t tq_sv_excitation_adjoint_workspace_bytes(int n, int n_ex) {
  if (n < 2 || n_ex < 0) return 0;
  return sizeof(double) * (size_t)exc_blocks(n) * (size_t)(n_ex > 0 ? n_ex : 1);
}

extern "C" int tq_sv_excitation_adjoint(void* psi, void* lam, int n, int dtype, const tq_excitation* exc, int n_ex,
                                        const double* sincos, double* grads, void* ws, size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_excitation_adjoint");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_ex < 0 || n < 2) return fail(TQ_ERR_ARG, "tq_sv_excitation_adjoint: n=%d, n_ex=%d", n, n_ex);
  if (n_ex == 0) return TQ_OK;
  if (!psi || !lam || !exc || !sincos || !grads) return fail(TQ_ERR_ARG, "tq_sv_excitation_adjoint: NULL pointer");
  const size_t need = tq_sv_excitation_adjoint_workspace_bytes(n, n_ex);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_excitation_adjoint: workspace of %zu bytes < %zu", ws_bytes, need);
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = exc_blocks(n);
  double* part = (double*)ws;
  for (int j = n_ex - 1; j >= 0; --j) {
    if (dtype == TQ_C64)
      k_exc_adjoint<float><<<nb, 256, 0, s>>>((float2*)psi, (float2*)lam, n, exc, j, sincos, part + (int64_t)j * nb);
    else
      k_exc_adjoint<double><<<nb, 256, 0, s>>>((double2*)psi, (double2*)lam, n, exc, j, sincos,
                                               part + (int64_t)j * nb);
  }
  k_ci_finalize<<<n_ex, 256, 0, s>>>(part, nb, grads);
  TQ_CHECK_LAUNCH("tq_sv_excitation_adjoint");
  return TQ_OK;
}
