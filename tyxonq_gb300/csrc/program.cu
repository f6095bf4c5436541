// Fused gate programs as shared-memory tile passes (forward and adjoint).
//
// Per pass, every tile (2^t amplitudes sharing the non-local bits) is read
// from HBM once with 128-bit loads in runs of 2^nlow contiguous amplitudes,
// all the pass's gates are applied in shared memory, and the tile is written
// back once: algorithmic bytes 2*N*S per pass (4*N*S for the adjoint pass,
// which carries psi and lambda), however many gates the pass holds.
#include "stage.cuh"
#include "staged_io.cuh"

namespace tq {

static const int kTileGridCap = 152 * 8;

static PassArgs to_args(const tq_tile_pass& p, int n) {
  PassArgs a;
  a.n = n;
  a.t = p.t;
  a.nlow = p.nlow;
  a.op_begin = p.op_begin;
  a.op_end = p.op_end;
  for (int i = 0; i < TQ_TILE_MAX_BITS; ++i) a.pos[i] = p.pos[i];
  return a;
}

// Tile <-> global copies.  complex64 moves two amplitudes per 16-byte access.
template <typename R>
__device__ __forceinline__ void tile_load(cplx<R>* s, const typename C2<R>::T* psi, int64_t base, const int64_t* hoff,
                                          const PassArgs& P);
template <>
__device__ __forceinline__ void tile_load<float>(cplx<float>* s, const float2* psi, int64_t base, const int64_t* hoff,
                                                 const PassArgs& P) {
  const int nv = 1 << (P.t - 1);
  const int lm = (1 << P.nlow) - 1;
  const float4* g4 = reinterpret_cast<const float4*>(psi);
  float4* s4 = reinterpret_cast<float4*>(s);
  for (int v = threadIdx.x; v < nv; v += blockDim.x) {
    const int j = 2 * v;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + 2 <= (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    s4[v] = g4[gi >> 1];
  }
}
template <>
__device__ __forceinline__ void tile_load<double>(cplx<double>* s, const double2* psi, int64_t base,
                                                  const int64_t* hoff, const PassArgs& P) {
  const int N = 1 << P.t;
  const int lm = (1 << P.nlow) - 1;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi < (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    const double2 v = psi[gi];
    s[j] = cplx<double>(v.x, v.y);
  }
}
template <typename R>
__device__ __forceinline__ void tile_store(const cplx<R>* s, typename C2<R>::T* psi, int64_t base, const int64_t* hoff,
                                           const PassArgs& P);
template <>
__device__ __forceinline__ void tile_store<float>(const cplx<float>* s, float2* psi, int64_t base, const int64_t* hoff,
                                                  const PassArgs& P) {
  const int nv = 1 << (P.t - 1);
  const int lm = (1 << P.nlow) - 1;
  float4* g4 = reinterpret_cast<float4*>(psi);
  const float4* s4 = reinterpret_cast<const float4*>(s);
  for (int v = threadIdx.x; v < nv; v += blockDim.x) {
    const int j = 2 * v;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + 2 <= (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    g4[gi >> 1] = s4[v];
  }
}
template <>
__device__ __forceinline__ void tile_store<double>(const cplx<double>* s, double2* psi, int64_t base,
                                                   const int64_t* hoff, const PassArgs& P) {
  const int N = 1 << P.t;
  const int lm = (1 << P.nlow) - 1;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi < (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    psi[gi] = make_double2(s[j].x, s[j].y);
  }
}

template <typename R>
__global__ void k_tile_forward(typename C2<R>::T* psi, int n, const PassArgs P, const tq_tile_op* __restrict__ ops,
                               const double* __restrict__ theta) {
  extern __shared__ __align__(16) unsigned char smem[];
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem);
  int64_t* hoff = reinterpret_cast<int64_t*>(smem + (sizeof(cplx<R>) << P.t));
  build_hoff(hoff, P);
  __syncthreads();
  const int64_t ntiles = int64_t(1) << (n - P.t);
  for (int64_t g = blockIdx.x; g < ntiles; g += gridDim.x) {
    const int64_t base = tile_base(g, P);
    tile_load<R>(s, psi, base, hoff, P);
    __syncthreads();
    for (int k = P.op_begin; k < P.op_end; ++k) {
      tile_apply<R>(s, P.t, ops[k], threadIdx.x, blockDim.x, false, theta, (uint64_t)base);
      __syncthreads();
    }
    tile_store<R>(s, psi, base, hoff, P);
    __syncthreads();
  }
}

// Adjoint pass: psi and lam tiles; per op: gradient term then un-apply.
// Per-block slot sums go to partials[block * n_slots + slot].
constexpr int kAdjChunk = 64;  // ops per gradient-partial flush in k_tile_adjoint

template <typename R>
__global__ void k_tile_adjoint(typename C2<R>::T* psi, typename C2<R>::T* lam, int n, const PassArgs P,
                               const tq_tile_op* __restrict__ ops, const double* __restrict__ theta, int n_slots,
                               double* partials) {
  extern __shared__ __align__(16) unsigned char smem[];
  const size_t tb = sizeof(cplx<R>) << P.t;
  cplx<R>* sp = reinterpret_cast<cplx<R>*>(smem);
  cplx<R>* sl = reinterpret_cast<cplx<R>*>(smem + tb);
  int64_t* hoff = reinterpret_cast<int64_t*>(smem + 2 * tb);
  double* acc = reinterpret_cast<double*>(smem + 2 * tb + (sizeof(int64_t) << (P.t - P.nlow)));
  const int nops = P.op_end - P.op_begin;
  // per-warp gradient partials of up to kAdjChunk ops, summed over warps once per chunk
  R* wpart = reinterpret_cast<R*>(acc + nops);
  const int nwarps = (int)(blockDim.x >> 5), warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  build_hoff(hoff, P);
  for (int k = threadIdx.x; k < nops; k += blockDim.x) acc[k] = 0.0;
  __syncthreads();
  const int64_t ntiles = int64_t(1) << (n - P.t);
  for (int64_t g = blockIdx.x; g < ntiles; g += gridDim.x) {
    const int64_t base = tile_base(g, P);
    tile_load<R>(sp, psi, base, hoff, P);
    tile_load<R>(sl, lam, base, hoff, P);
    __syncthreads();
    for (int k = 0; k < nops; ++k) {
      const tq_tile_op& o = ops[P.op_begin + k];
      if (o.slot >= 0) {
        // warp sums in the working precision (FP64 issues slowly on this GPU);
        // warps are added in order at the end of the chunk
        const R phr[4] = {R(1), R(0), R(-1), R(0)}, phi[4] = {R(0), R(1), R(0), R(-1)};
        const cplx<R> ph(phr[o.gny & 3], phi[o.gny & 3]);
        R v = zsign<R>(o, (uint64_t)base, 0) *
              tile_grad_partial<R>(sp, sl, P.t, o.gxm, o.gzm, o.gcm, ph, threadIdx.x, blockDim.x);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
        if (lane == 0) wpart[(k % kAdjChunk) * nwarps + warp] = v;
      }
      tile_apply<R>(sp, P.t, o, threadIdx.x, blockDim.x, true, theta, (uint64_t)base);
      tile_apply<R>(sl, P.t, o, threadIdx.x, blockDim.x, true, theta, (uint64_t)base);
      __syncthreads();
      if (k % kAdjChunk == kAdjChunk - 1 || k == nops - 1) {  // the barrier above published wpart
        const int k0 = k - k % kAdjChunk;
        for (int q = threadIdx.x; q <= k - k0; q += blockDim.x) {
          if (ops[P.op_begin + k0 + q].slot < 0) continue;
          R sum = R(0);
          for (int w = 0; w < nwarps; ++w) sum += wpart[q * nwarps + w];
          acc[k0 + q] += (double)sum;
        }
        __syncthreads();
      }
    }
    tile_store<R>(sp, psi, base, hoff, P);
    tile_store<R>(sl, lam, base, hoff, P);
    __syncthreads();
  }
  for (int k = threadIdx.x; k < nops; k += blockDim.x) {
    const int slot = ops[P.op_begin + k].slot;
    if (slot >= 0) partials[(int64_t)blockIdx.x * n_slots + slot] = acc[k];
  }
}

__global__ void k_finalize_slots(const double* partials, int nblk, int nslots, double* out) {
  __shared__ double sh[32];
  const int o = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += partials[(int64_t)b * nslots + o];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    out[o] = s;
  }
}

static int tile_threads(int t) {
  int nt = 1 << (t - 1);
  if (nt > 512) nt = 512;
  if (nt < 32) nt = 32;
  return nt;
}

static int check_passes(int n, int dtype, const tq_tile_pass* passes, int n_passes, int max_t, const char* name) {
  for (int p = 0; p < n_passes; ++p) {
    const tq_tile_pass& P = passes[p];
    if (P.t < 1 || P.t > n || P.t > max_t)
      return fail(TQ_ERR_ARG, "%s: pass %d has t=%d (n=%d, max %d)", name, p, P.t, n, max_t);
    if (P.nlow < 1 || P.nlow > P.t) return fail(TQ_ERR_ARG, "%s: pass %d has nlow=%d", name, p, P.nlow);
    for (int j = 0; j < P.t; ++j) {
      if (P.pos[j] < 0 || P.pos[j] >= n) return fail(TQ_ERR_RANGE, "%s: pass %d pos out of range", name, p);
      if (j < P.nlow && P.pos[j] != j) return fail(TQ_ERR_ARG, "%s: pass %d low positions not 0..nlow-1", name, p);
      if (j > 0 && P.pos[j] <= P.pos[j - 1]) return fail(TQ_ERR_ARG, "%s: pass %d pos not ascending", name, p);
    }
    if (P.op_begin < 0 || P.op_end < P.op_begin) return fail(TQ_ERR_ARG, "%s: pass %d op range", name, p);
  }
  (void)dtype;
  return TQ_OK;
}

static int max_bits(int dtype, bool adjoint) {
  // complex64: 2^14 * 8 B = 128 KiB; complex128: 2^13 * 16 B = 128 KiB per tile
  const int f = (dtype == TQ_C64) ? 14 : 13;
  return adjoint ? f - 1 : f;
}

template <typename R>
static int run_fwd(void* psi, int n, const tq_tile_pass* passes, int n_passes, const tq_tile_op* ops,
                   const double* theta, cudaStream_t s) {
  for (int p = 0; p < n_passes; ++p) {
    const PassArgs P = to_args(passes[p], n);
    if (P.op_end == P.op_begin) continue;
    const size_t smem = (sizeof(cplx<R>) << P.t) + (sizeof(int64_t) << (P.t - P.nlow));
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_tile_forward<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_status(e, "tq_sv_run_tiles: smem attribute");
    }
    const int64_t ntiles = int64_t(1) << (n - P.t);
    const unsigned grid = (unsigned)(ntiles < kTileGridCap ? ntiles : kTileGridCap);
    k_tile_forward<R><<<grid, tile_threads(P.t), smem, s>>>((typename C2<R>::T*)psi, n, P, ops, theta);
    TQ_CHECK_LAUNCH("tq_sv_run_tiles");
  }
  return TQ_OK;
}

static unsigned adjoint_grid(int n, const tq_tile_pass* passes, int n_passes) {
  int64_t g = 1;
  for (int p = 0; p < n_passes; ++p) {
    const int64_t nt = int64_t(1) << (n - passes[p].t);
    if (nt > g) g = nt;
  }
  return (unsigned)(g < kTileGridCap ? g : kTileGridCap);
}

template <typename R>
static int run_adj(void* psi, void* lam, int n, const tq_tile_pass* passes, int n_passes, const tq_tile_op* ops,
                   const double* theta,
                   int n_slots, double* slot_out, double* partials, cudaStream_t s) {
  const unsigned grid = adjoint_grid(n, passes, n_passes);
  if (n_slots > 0) cudaMemsetAsync(partials, 0, sizeof(double) * (size_t)grid * n_slots, s);
  for (int p = 0; p < n_passes; ++p) {
    const PassArgs P = to_args(passes[p], n);
    const int nops = P.op_end - P.op_begin;
    if (nops == 0) continue;
    const size_t smem = 2 * (sizeof(cplx<R>) << P.t) + (sizeof(int64_t) << (P.t - P.nlow)) + sizeof(double) * nops +
                        sizeof(R) * kAdjChunk * (tile_threads(P.t) / 32);
    if (smem > 227 * 1024) return fail(TQ_ERR_ARG, "tq_sv_adjoint_tiles: pass %d needs %zu B shared memory", p, smem);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_tile_adjoint<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return cuda_status(e, "tq_sv_adjoint_tiles: smem attribute");
    }
    k_tile_adjoint<R><<<grid, tile_threads(P.t), smem, s>>>((typename C2<R>::T*)psi, (typename C2<R>::T*)lam, n, P,
                                                            ops, theta, n_slots, partials);
    TQ_CHECK_LAUNCH("tq_sv_adjoint_tiles");
  }
  if (n_slots > 0) {
    k_finalize_slots<<<n_slots, 256, 0, s>>>(partials, (int)grid, n_slots, slot_out);
    TQ_CHECK_LAUNCH("tq_sv_adjoint_tiles: finalize");
  }
  return TQ_OK;
}

}  // namespace tq

using namespace tq;

extern "C" int tq_sv_tile_max_bits(int dtype) { return (dtype == TQ_C64 || dtype == TQ_C128) ? max_bits(dtype, false) : 0; }

extern "C" int tq_sv_run_tiles(void* psi, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                               const tq_tile_op* ops, const double* theta, void* stream) {
  TQ_RANGE("tq_sv_run_tiles");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_passes < 0) return fail(TQ_ERR_ARG, "tq_sv_run_tiles: negative pass count");
  if (n_passes == 0) return TQ_OK;
  if (!psi || !passes || !ops) return fail(TQ_ERR_ARG, "tq_sv_run_tiles: NULL pointer");
  if ((rc = check_passes(n, dtype, passes, n_passes, max_bits(dtype, false), "tq_sv_run_tiles"))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == TQ_C64 ? run_fwd<float>(psi, n, passes, n_passes, ops, theta, s)
                         : run_fwd<double>(psi, n, passes, n_passes, ops, theta, s);
}

extern "C" size_t tq_sv_adjoint_tiles_workspace_bytes(int n, int n_slots) {
  if (n < 1 || n > TQ_MAX_QUBITS || n_slots < 0) return 0;
  return sizeof(double) * (size_t)kTileGridCap * (size_t)(n_slots > 0 ? n_slots : 1);
}

extern "C" int tq_sv_adjoint_tiles(void* psi, void* lam, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                                   const tq_tile_op* ops, const double* theta, int n_slots, double* slot_out,
                                   void* ws, size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_adjoint_tiles");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_passes < 0 || n_slots < 0) return fail(TQ_ERR_ARG, "tq_sv_adjoint_tiles: negative count");
  if (!psi || !lam || (n_passes > 0 && (!passes || !ops)) || (n_slots > 0 && !slot_out))
    return fail(TQ_ERR_ARG, "tq_sv_adjoint_tiles: NULL pointer");
  if (psi == lam) return fail(TQ_ERR_ARG, "tq_sv_adjoint_tiles: psi aliases lam");
  if ((rc = check_passes(n, dtype, passes, n_passes, max_bits(dtype, true), "tq_sv_adjoint_tiles"))) return rc;
  const size_t need = tq_sv_adjoint_tiles_workspace_bytes(n, n_slots);
  if (n_slots > 0 && (!ws || ws_bytes < need))
    return fail(TQ_ERR_WORKSPACE, "tq_sv_adjoint_tiles: workspace of %zu bytes < %zu", ws_bytes, need);
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == TQ_C64
             ? run_adj<float>(psi, lam, n, passes, n_passes, ops, theta, n_slots, slot_out, (double*)ws, s)
             : run_adj<double>(psi, lam, n, passes, n_passes, ops, theta, n_slots, slot_out, (double*)ws, s);
}

// ----------------------------------------------------------------- generator term (plain reverse sweep)
namespace tq {
template <typename R>
__global__ void k_generator_im(const typename C2<R>::T* psi, const typename C2<R>::T* lam, int64_t N, uint64_t xm,
                               uint64_t zm, uint64_t cm, cplx<R> ph, double* partials) {
  __shared__ double red[32];
  double acc = 0.0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  while (i < N) {
    R loc = 0;
    for (int u = 0; u < 8 && i < N; ++u, i += stride) {
      if (((uint64_t)i & cm) != cm) continue;
      const typename C2<R>::T pv = psi[i];
      const typename C2<R>::T lv = lam[i ^ (int64_t)xm];
      const cplx<R> v = cmul(ph, cplx<R>(pv.x, pv.y));
      const R sg = (__popcll((uint64_t)i & zm) & 1) ? R(-1) : R(1);
      loc += sg * (lv.x * v.y - lv.y * v.x);
    }
    acc += (double)loc;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    partials[blockIdx.x] = s;
  }
}
}  // namespace tq

extern "C" int tq_sv_generator_im(const void* psi, const void* lam, int n, int dtype, uint64_t xm, uint64_t zm,
                                  uint64_t cm, double* out_dev, void* ws, size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_generator_im");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi || !lam || !out_dev) return fail(TQ_ERR_ARG, "tq_sv_generator_im: NULL pointer");
  const uint64_t full = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  if ((xm | zm | cm) & ~full) return fail(TQ_ERR_RANGE, "tq_sv_generator_im: mask has bits above n=%d", n);
  const int64_t N = int64_t(1) << n;
  int64_t nb = (N + 4095) / 4096;
  if (nb > 1216) nb = 1216;
  if (!ws || ws_bytes < sizeof(double) * nb)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_generator_im: workspace of %zu bytes < %zu", ws_bytes, sizeof(double) * nb);
  const int ny = __builtin_popcountll(xm & zm) & 3;
  const double phr[4] = {1, 0, -1, 0}, phi[4] = {0, 1, 0, -1};
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TQ_C64)
    k_generator_im<float><<<(unsigned)nb, 256, 0, s>>>((const float2*)psi, (const float2*)lam, N, xm, zm, cm,
                                                        cplx<float>((float)phr[ny], (float)phi[ny]), (double*)ws);
  else
    k_generator_im<double><<<(unsigned)nb, 256, 0, s>>>((const double2*)psi, (const double2*)lam, N, xm, zm, cm,
                                                         cplx<double>(phr[ny], phi[ny]), (double*)ws);
  k_finalize_slots<<<1, 256, 0, s>>>((const double*)ws, (int)nb, 1, out_dev);
  TQ_CHECK_LAUNCH("tq_sv_generator_im");
  return TQ_OK;
}

// ----------------------------------------------------------------- register-staged forward passes
namespace tq {

// Shared memory: one or two padded tiles | offset table | compiled ops.
template <typename R>
__global__ void __launch_bounds__(sizeof(R) == 4 ? 512 : 256, 1)
    k_staged_forward(typename C2<R>::T* psi, int n, const PassArgs P, const tq_tile_stage* __restrict__ stages,
                     const tq_tile_op* __restrict__ ops, const double* __restrict__ theta, int dbuf) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int PT = padded_len(P.t);
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem);
  cplx<R>* buf1 = buf0 + (dbuf ? PT : 0);
  int64_t* hoff = reinterpret_cast<int64_t*>(smem + (size_t)(dbuf ? 2 : 1) * PT * sizeof(cplx<R>));
  ROp<R>* rops = reinterpret_cast<ROp<R>*>(reinterpret_cast<unsigned char*>(hoff) + staged_hoff_bytes(P.t, P.nlow));
  build_hoff(hoff, P);
  // compile the whole pass once when it fits, else stage by stage per tile
  const int op0 = P.op_end > P.op_begin ? stages[P.op_begin].op_begin : 0;
  const int nops = P.op_end > P.op_begin ? stages[P.op_end - 1].op_end - op0 : 0;
  const bool resident = nops <= kStagedRopCap;
  if (resident) rops_build<R>(rops, ops, op0, op0 + nops, theta, false, false);
  __syncthreads();
  const int64_t ntiles = int64_t(1) << (n - P.t);
  int64_t g = blockIdx.x;
  if (g < ntiles) staged_issue_load<R>(buf0, psi, tile_base(g, P), hoff, P);
  cp_async_commit();
  int cur = 0;
  for (; g < ntiles; g += gridDim.x) {
    const int64_t gn = g + gridDim.x;
    cplx<R>* s = cur ? buf1 : buf0;
    if (dbuf) {
      if (gn < ntiles) staged_issue_load<R>(cur ? buf0 : buf1, psi, tile_base(gn, P), hoff, P);
      cp_async_commit();
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_group<0>();
    }
    __syncthreads();
    run_stages<R>(s, rops, resident, op0, stages, P.op_begin, P.op_end, ops, theta, (uint64_t)tile_base(g, P));
    staged_store<R>(s, psi, tile_base(g, P), hoff, P);
    __syncthreads();
    if (!dbuf && gn < ntiles) {
      staged_issue_load<R>(buf0, psi, tile_base(gn, P), hoff, P);
      cp_async_commit();
    }
    cur ^= dbuf;
  }
  cp_async_wait_group<0>();
}

static int staged_max_bits(int dtype) { return dtype == TQ_C64 ? 13 : 12; }

template <typename R>
static int run_staged(void* psi, int n, const tq_tile_pass* passes, int n_passes, const tq_tile_stage* stages,
                      const tq_tile_op* ops, const double* theta, cudaStream_t s) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int p = 0; p < n_passes; ++p) {
    const PassArgs P = to_args(passes[p], n);
    if (P.op_end == P.op_begin) continue;
    const int64_t ntiles = int64_t(1) << (n - P.t);
    const int dbuf = ntiles > sms ? 1 : 0;
    const size_t smem = (size_t)(dbuf ? 2 : 1) * padded_len(P.t) * sizeof(cplx<R>) +
                        staged_hoff_bytes(P.t, P.nlow) + kStagedRopCap * sizeof(ROp<R>);
    cudaError_t e = cudaFuncSetAttribute(k_staged_forward<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "tq_sv_run_staged: smem attribute");
    const unsigned grid = (unsigned)(ntiles < sms ? ntiles : sms);
    k_staged_forward<R><<<grid, 1 << (P.t - kRB), smem, s>>>((typename C2<R>::T*)psi, n, P, stages, ops, theta, dbuf);
    TQ_CHECK_LAUNCH("tq_sv_run_staged");
  }
  return TQ_OK;
}

}  // namespace tq

extern "C" int tq_sv_run_staged(void* psi, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                                const tq_tile_stage* stages, const tq_tile_op* ops, const double* theta,
                                void* stream) {
  TQ_RANGE("tq_sv_run_staged");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n_passes < 0) return fail(TQ_ERR_ARG, "tq_sv_run_staged: negative pass count");
  if (n_passes == 0) return TQ_OK;
  if (!psi || !passes || !stages || !ops) return fail(TQ_ERR_ARG, "tq_sv_run_staged: NULL pointer");
  if ((rc = check_passes(n, dtype, passes, n_passes, staged_max_bits(dtype), "tq_sv_run_staged"))) return rc;
  for (int p = 0; p < n_passes; ++p)
    if (passes[p].t < 9) return fail(TQ_ERR_ARG, "tq_sv_run_staged: pass %d has t=%d < 9", p, passes[p].t);
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == TQ_C64 ? run_staged<float>(psi, n, passes, n_passes, stages, ops, theta, s)
                         : run_staged<double>(psi, n, passes, n_passes, stages, ops, theta, s);
}
TQ_CHECK_UNIT(program)
