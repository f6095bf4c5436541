// Batches of Kraus trajectories.
//
// The reference unravels a noisy circuit one trajectory per run: each Kraus
// channel draws a status, computes the Born weights ||K_i psi||^2 of every
// operator and keeps K_i psi / ||K_i psi|| for the first i whose cumulative
// normalised weight reaches the status
// (libs/quantum_library/kernels/statevector.py:132-218, engine.py:145-155).
// Here T trajectories of an n-qubit circuit live in one buffer of T states
// (trajectory t at offset t * 2^n; for T a power of two this is one state of
// n + log2 T qubits whose leading qubits index the trajectory, so the unitary
// segments between channels run as one fused program over every trajectory).
// A channel on qubit q is three launches with no host round trip: the 2x2
// reduced density matrix of q in every trajectory (fixed-order sums), the
// selection of each trajectory's operator from its status on the device, and
// one 2x2 per trajectory applied to its own amplitudes.
#include "common.cuh"

namespace tq {

constexpr int kMaxKrausOps = 16;

template <typename R>
__device__ __forceinline__ cplx<R> ldt(const typename C2<R>::T* p, int64_t i) {
  const typename C2<R>::T v = p[i];
  return cplx<R>(v.x, v.y);
}

// partials[((t * nbx) + bx) * 4 + k]: sum |a|^2, sum |b|^2, Re sum a conj(b),
// Im sum a conj(b) over the block's pairs (a = bit clear, b = bit set) of
// trajectory t = blockIdx.y.
template <typename R>
__global__ void k_rdm_traj(const typename C2<R>::T* __restrict__ psi, int n, int bit, double* partials) {
  __shared__ double sh[4][32];
  const int64_t half = int64_t(1) << (n - 1);
  const typename C2<R>::T* st = psi + ((int64_t)blockIdx.y << n);
  const int64_t lo = (int64_t(1) << bit) - 1;
  double s[4] = {0, 0, 0, 0};
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < half; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = ((p >> bit) << (bit + 1)) | (p & lo);
    const cplx<R> a = ldt<R>(st, i), b = ldt<R>(st, i | (int64_t(1) << bit));
    s[0] += (double)(a.x * a.x + a.y * a.y);
    s[1] += (double)(b.x * b.x + b.y * b.y);
    s[2] += (double)(a.x * b.x + a.y * b.y);
    s[3] += (double)(a.y * b.x - a.x * b.y);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double v = s[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
    partials[((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * 4 + threadIdx.x] = v;
  }
}

// out[t * 4 + k] = sum over the nbx block partials of trajectory t, in order.
__global__ void k_rdm_traj_finalize(const double* __restrict__ partials, int nbx, int n_traj, double* out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_traj * 4) return;
  const int t = idx >> 2, k = idx & 3;
  double v = 0;
  for (int b = 0; b < nbx; ++b) v += partials[((int64_t)t * nbx + b) * 4 + k];
  out[idx] = v;
}

// Per trajectory: Born weights p_i = Tr(K_i rho K_i^dagger) from its reduced
// density matrix rho (4 doubles: rho00, rho11, Re rho01, Im rho01), the first
// operator whose cumulative normalised weight reaches the status (and whose
// weight is positive), and the matrix K_i / sqrt(p_i) (8 doubles, row-major
// (re, im)).  chosen[t] = i.
__global__ void k_kraus_select(const double* __restrict__ rdm, const double* __restrict__ kraus, int n_ops,
                               const double* __restrict__ status, int n_traj, double* mats, int32_t* chosen) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_traj) return;
  // rho = [[r00, r01], [conj(r01), r11]] with r01 = sum a conj(b) = rre + i rim
  const double r00 = rdm[4 * t], r11 = rdm[4 * t + 1], rre = rdm[4 * t + 2], rim = rdm[4 * t + 3];
  double p[kMaxKrausOps];
  double total = 0;
  for (int i = 0; i < n_ops; ++i) {
    const double* K = kraus + 8 * i;
    // ||K_i psi||^2 = sum_r (|K_r0|^2 r00 + |K_r1|^2 r11 + 2 Re(conj(K_r0) K_r1 conj(r01)))
    double w = 0;
    for (int r = 0; r < 2; ++r) {
      const double ax = K[4 * r], ay = K[4 * r + 1], bx = K[4 * r + 2], by = K[4 * r + 3];
      const double cx = ax * bx + ay * by, cy = ax * by - ay * bx;  // conj(K_r0) K_r1
      w += (ax * ax + ay * ay) * r00 + (bx * bx + by * by) * r11 + 2.0 * (cx * rre + cy * rim);
    }
    p[i] = w;
    total += w;
  }
  int sel = 0;
  double cum = 0;
  for (int i = 0; i < n_ops; ++i) {
    cum += p[i] / total;
    if (status[t] <= cum && p[i] > 0) {
      sel = i;
      break;
    }
  }
  const double inv = p[sel] > 0 ? 1.0 / sqrt(p[sel]) : 0.0;
  for (int e = 0; e < 8; ++e) mats[8 * t + e] = kraus[8 * sel + e] * inv;
  chosen[t] = sel;
}

// psi_t <- M_t psi_t on qubit bit, M_t = mats[8 t .. 8 t + 8) (row-major (re, im)).
template <typename R>
__global__ void k_apply_1q_traj(typename C2<R>::T* psi, int n, int bit, int64_t total_pairs,
                                const double* __restrict__ mats) {
  const int64_t lo = (int64_t(1) << bit) - 1;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total_pairs;
       g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = g >> (n - 1), p = g & ((int64_t(1) << (n - 1)) - 1);
    typename C2<R>::T* st = psi + (t << n);
    const int64_t i = ((p >> bit) << (bit + 1)) | (p & lo), j = i | (int64_t(1) << bit);
    const double* M = mats + 8 * t;
    const cplx<R> u0((R)M[0], (R)M[1]), u1((R)M[2], (R)M[3]), u2((R)M[4], (R)M[5]), u3((R)M[6], (R)M[7]);
    const cplx<R> a = ldt<R>(st, i), b = ldt<R>(st, j);
    const cplx<R> x = cfma(u1, b, cmul(u0, a)), y = cfma(u3, b, cmul(u2, a));
    st[i].x = x.x;
    st[i].y = x.y;
    st[j].x = y.x;
    st[j].y = y.y;
  }
}

static int traj_blocks(int n) {
  const int64_t half = int64_t(1) << (n - 1);
  int64_t b = (half + 255) / 256;
  if (b > 64) b = 64;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace tq

using namespace tq;

extern "C" size_t tq_traj_kraus_workspace_bytes(int n, int n_traj) {
  if (n < 1 || n > TQ_MAX_QUBITS || n_traj < 1) return 0;
  return sizeof(double) * 4 * (size_t)traj_blocks(n) * (size_t)n_traj   // block partials
         + sizeof(double) * 4 * (size_t)n_traj                          // reduced density matrices
         + sizeof(double) * 8 * (size_t)n_traj                          // chosen matrices
         + 64;
}

extern "C" int tq_traj_kraus(void* psi, int n, int n_traj, int dtype, int qubit, const double* kraus_dev, int n_ops,
                             const double* status_dev, int32_t* chosen_dev, void* ws, size_t ws_bytes,
                             void* stream) {
  TQ_RANGE("tq_traj_kraus");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n < 1) return fail(TQ_ERR_ARG, "tq_traj_kraus: a channel needs at least one qubit");
  if ((rc = check_qubit(n, qubit))) return rc;
  if (n_traj < 1 || n_ops < 1 || n_ops > kMaxKrausOps)
    return fail(TQ_ERR_ARG, "tq_traj_kraus: %d trajectories, %d operators (1..%d)", n_traj, n_ops, kMaxKrausOps);
  if ((int64_t)n_traj << n > (int64_t(1) << TQ_MAX_QUBITS))
    return fail(TQ_ERR_RANGE, "tq_traj_kraus: %d trajectories of %d qubits exceed 2^%d amplitudes", n_traj, n,
                TQ_MAX_QUBITS);
  if (!psi || !kraus_dev || !status_dev || !chosen_dev) return fail(TQ_ERR_ARG, "tq_traj_kraus: NULL pointer");
  const size_t need = tq_traj_kraus_workspace_bytes(n, n_traj);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_traj_kraus: workspace of %zu bytes < %zu", ws_bytes, need);
  const int nbx = traj_blocks(n);
  double* part = static_cast<double*>(ws);
  double* rdm = part + 4 * (size_t)nbx * n_traj;
  double* mats = rdm + 4 * (size_t)n_traj;
  const int bit = tq_bit(n, qubit);
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 grid(nbx, n_traj);
  if (dtype == TQ_C64)
    k_rdm_traj<float><<<grid, 256, 0, s>>>((const float2*)psi, n, bit, part);
  else
    k_rdm_traj<double><<<grid, 256, 0, s>>>((const double2*)psi, n, bit, part);
  k_rdm_traj_finalize<<<(n_traj * 4 + 255) / 256, 256, 0, s>>>(part, nbx, n_traj, rdm);
  k_kraus_select<<<(n_traj + 127) / 128, 128, 0, s>>>(rdm, kraus_dev, n_ops, status_dev, n_traj, mats, chosen_dev);
  const int64_t pairs = (int64_t)n_traj << (n - 1);
  if (dtype == TQ_C64)
    k_apply_1q_traj<float><<<grid_for(pairs, 256), 256, 0, s>>>((float2*)psi, n, bit, pairs, mats);
  else
    k_apply_1q_traj<double><<<grid_for(pairs, 256), 256, 0, s>>>((double2*)psi, n, bit, pairs, mats);
  TQ_CHECK_LAUNCH("tq_traj_kraus");
  return TQ_OK;
}
