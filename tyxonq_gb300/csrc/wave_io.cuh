// Work items of the L2-resident waves: pass arguments, the offset table of a
// tile, tile loads (cp.async into padded shared memory) and stores.  Device
// code only, shared by the library's wave kernels (wave.cu) and the
// runtime-compiled wave kernels (jit_wave.cuh).
#pragma once

#include "stage.cuh"

namespace tq {

// tmask: the global bits of local bits nlow .. t-1 (ascending), kept as one
// mask so that the per-item deposits below run in registers (an indexed
// position array would live in local memory).
struct WPass {
  int t, nlow, op_begin, op_end;
  uint64_t tmask;
  int n;  // qubits of the item's instance (index checks of checked builds)
};

__device__ __forceinline__ WPass wload_pass(const tq_tile_pass* p, int n) {
  WPass s;
  s.n = n;
  s.t = p->t;
  s.nlow = p->nlow;
  s.op_begin = p->op_begin;
  s.op_end = p->op_end;
  uint64_t m = 0;
#pragma unroll
  for (int i = 0; i < TQ_TILE_MAX_BITS; ++i)
    if (i >= s.nlow && i < s.t) m |= uint64_t(1) << p->pos[i];
  s.tmask = m;
  return s;
}

__device__ __forceinline__ void w_hoff(int64_t* hoff, const WPass& P) {
  const int nh = 1 << (P.t - P.nlow);
  for (int h = threadIdx.x; h < nh; h += blockDim.x) {
    int64_t off = 0;
    uint64_t m = P.tmask;
    for (int k = 0; m; ++k) {
      const uint64_t low = m & (~m + 1);  // lowest remaining tile bit
      m ^= low;
      if ((h >> k) & 1) off |= (int64_t)low;
    }
    hoff[h] = off;
  }
}

// Passes of a wave keep at least kWaveMinNlow contiguous low bits, so the
// offset table has at most 2^(t - kWaveMinNlow) entries.
constexpr int kWaveMinNlow = 4;
__host__ __device__ __forceinline__ size_t w_hoff_bytes(int t) { return sizeof(int64_t) << (t - kWaveMinNlow); }

__device__ __forceinline__ int64_t w_base(int64_t g, const WPass& P) {
  int64_t x = g << P.nlow;
  for (uint64_t m = P.tmask; m; m &= m - 1) x = insert_zero(x, __ffsll((long long)m) - 1);
  return x;
}

__device__ __forceinline__ void w_commit_wait() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

template <typename R>
__device__ __forceinline__ void w_load(cplx<R>* s, const typename C2<R>::T* g, int64_t base, const int64_t* hoff,
                                       const WPass& P) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + A <= (int64_t(1) << P.n), TQ_SITE_WAVE_TILE, gi, continue);
    cp_async16(&s[pphys(j)], &g[gi]);
  }
}

template <typename R>
__device__ __forceinline__ void w_store(const cplx<R>* s, typename C2<R>::T* g, int64_t base, const int64_t* hoff,
                                        const WPass& P) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + A <= (int64_t(1) << P.n), TQ_SITE_WAVE_TILE, gi, continue);
    *reinterpret_cast<float4*>(&g[gi]) = *reinterpret_cast<const float4*>(&s[pphys(j)]);
  }
}

}  // namespace tq
