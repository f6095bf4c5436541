// Tile passes of the register-staged forward kernels: pass arguments, the
// global offset table of a tile, asynchronous tile loads into padded shared
// memory and the stores back.  Device code only, shared by the kernels built
// with the library (program.cu) and the runtime-compiled pass kernels
// (jit_staged.cuh).
#pragma once

#include "stage.cuh"

namespace tq {

struct PassArgs {
  int t, nlow;
  int op_begin, op_end;
  int pos[TQ_TILE_MAX_BITS];
  int n;  // qubits of the state (index checks of checked builds)
};

// hoff[h] = global offset of local index (h << nlow).
__device__ __forceinline__ void build_hoff(int64_t* hoff, const PassArgs& P) {
  const int nh = 1 << (P.t - P.nlow);
  for (int h = threadIdx.x; h < nh; h += blockDim.x) {
    int64_t off = 0;
    for (int k = 0; k < P.t - P.nlow; ++k)
      if ((h >> k) & 1) off |= int64_t(1) << P.pos[P.nlow + k];
    hoff[h] = off;
  }
}

__device__ __forceinline__ int64_t tile_base(int64_t g, const PassArgs& P) {
  int64_t x = g << P.nlow;
  for (int k = P.nlow; k < P.t; ++k) x = insert_zero(x, P.pos[k]);
  return x;
}

// Issue (without waiting) the async copy of one tile into a padded buffer.
template <typename R>
__device__ __forceinline__ void staged_issue_load(cplx<R>* s, const typename C2<R>::T* g, int64_t base,
                                                  const int64_t* hoff, const PassArgs& P) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + A <= (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    cp_async16(&s[pphys(j)], &g[gi]);
  }
}

template <typename R>
__device__ __forceinline__ void staged_store(const cplx<R>* s, typename C2<R>::T* g, int64_t base,
                                             const int64_t* hoff, const PassArgs& P) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    TQ_DCHECK(gi + A <= (int64_t(1) << P.n), TQ_SITE_TILE, gi, continue);
    *reinterpret_cast<float4*>(&g[gi]) = *reinterpret_cast<const float4*>(&s[pphys(j)]);
  }
}

// Compiled ops of one pass kept in shared memory for all its tiles.
constexpr int kStagedRopCap = 256;

// Offset-table bytes of a staged pass, rounded up to 16 (the compiled ops follow it).
__host__ __device__ __forceinline__ size_t staged_hoff_bytes(int t, int nlow) {
  return ((sizeof(int64_t) << (t - nlow)) + 15) & ~size_t(15);
}

}  // namespace tq
