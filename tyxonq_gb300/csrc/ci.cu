// CI-space UCC: the state restricted to determinants with fixed alpha / beta
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
