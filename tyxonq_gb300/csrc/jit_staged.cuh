// Runtime-specialised register-staged forward passes.
//
// The library's k_staged_forward interprets each pass's op list: every op is
// a switch over its compiled code, and every op writes all 16 registers of
// the other register array, so a pass of a random circuit spends most of its
// instructions on dispatch and register moves.  Here the op list of a pass is
// turned into straight-line code instead (tyxonq_gb300/jit.py writes one body
// per pass and this header wraps it; the source is compiled at run time by
// NVRTC, csrc/jit.cu).  Register bits, stage layouts and op shapes become
// compile-time constants: permutations (CX, SWAP) are register renames, CZ a
// few sign flips, rotations their FMAs.  Coefficients are still compiled
// from the op table and theta into op records (rop_build, by the library's
// k_rops_compile once per program run) that each CTA copies to shared memory,
// so one body serves every angle vector of the same circuit structure.
#pragma once

#include "staged_io.cuh"

namespace tq {

// In-place dense 4x4 on register bits (A = matrix high bit, B = low bit) of
// NR registers.
template <typename R, int NR, int A, int B>
__device__ __forceinline__ void j_u2(cplx<R>* x, const tq_tile_op& o) {
  cplx<R> u[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) u[e] = op_m<R>(o, e);
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if (((i >> A) & 1) || ((i >> B) & 1)) continue;
    const int id[4] = {i, i | (1 << B), i | (1 << A), i | (1 << A) | (1 << B)};
    const cplx<R> v[4] = {x[id[0]], x[id[1]], x[id[2]], x[id[3]]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      cplx<R> acc = cmul(u[4 * r], v[0]);
      acc = cfma(u[4 * r + 1], v[1], acc);
      acc = cfma(u[4 * r + 2], v[2], acc);
      acc = cfma(u[4 * r + 3], v[3], acc);
      x[id[r]] = acc;
    }
  }
}

// In-place real 2x2 [[u0, u1], [u2, u3]] on register bit K of NR registers
// (Hadamard, Y rotations and their products): 4 FP32 instructions per amplitude
// instead of 8 for a complex matrix.
template <typename R, int NR, int K>
__device__ __forceinline__ void j_ureal(cplx<R>* x, R u0, R u1, R u2, R u3) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    const cplx<R> a = x[i], b = x[j];
    x[i] = cplx<R>(fma(u1, b.x, u0 * a.x), fma(u1, b.y, u0 * a.y));
    x[j] = cplx<R>(fma(u3, b.x, u2 * a.x), fma(u3, b.y, u2 * a.y));
  }
}

// In-place Pauli rotation exp(-i a/2 P) on register bits: X/Y bits XM, Z/Y bits
// ZM, control bits CM (all compile-time), coefficients c = m0 (real part used,
// as the library's t_prot) and w = sign * m1.
template <typename R, int NR, int XM, int ZM, int CM>
__device__ __forceinline__ void j_prot(cplx<R>* x, cplx<R> c, cplx<R> w) {
  if constexpr (XM == 0) {
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      if ((i & CM) != CM) continue;
      const R sg = (__popc(i & ZM) & 1) ? R(-1) : R(1);
      x[i] = cmul(cplx<R>(c.x + sg * w.x, sg * w.y), x[i]);
    }
  } else {
    constexpr int H = (XM & 16) ? 4 : (XM & 8) ? 3 : (XM & 4) ? 2 : (XM & 2) ? 1 : 0;
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      if ((i >> H) & 1) continue;
      if ((i & CM) != CM) continue;
      const int j = i ^ XM;
      const R si = (__popc(i & ZM) & 1) ? R(-1) : R(1);
      const R sj = (__popc(j & ZM) & 1) ? R(-1) : R(1);
      const cplx<R> a = x[i], b = x[j];
      x[i] = cfma(cplx<R>(w.x * sj, w.y * sj), b, cplx<R>(c.x * a.x, c.x * a.y));
      x[j] = cfma(cplx<R>(w.x * si, w.y * si), a, cplx<R>(c.x * b.x, c.x * b.y));
    }
  }
}

// Pass geometry known when the kernel is generated (struct G: tile bits T,
// contiguous low bits NLOW, POS[k] = global bit of local bit k, THREADS).
// Local index -> offset from the tile base: a bit deposit, so it is additive
// over disjoint bit sets and a thread's part is computed once per kernel.
template <typename G>
__device__ __forceinline__ int64_t geo_off(int64_t j) {
  int64_t off = j & ((int64_t(1) << G::NLOW) - 1);
#pragma unroll
  for (int k = G::NLOW; k < G::T; ++k) off |= ((j >> k) & 1) << G::POS[k];
  return off;
}

// Global index of local index 0 of tile g (the tile's bits cleared).
template <typename G>
__device__ __forceinline__ int64_t geo_base(int64_t g) {
  int64_t x = g << G::NLOW;
#pragma unroll
  for (int k = G::NLOW; k < G::T; ++k) x = insert_zero(x, G::POS[k]);
  return x;
}

// The tile loop of one forward pass with the geometry compiled in: thread
// tid moves the 16-byte chunks tid + i * THREADS (i < PER); chunk i's global
// offset is the thread's part plus a constant and its shared-memory index the
// thread's padded index plus a constant, so a chunk costs one copy instruction
// and its address arithmetic folds into immediates.  Memory schedule and
// shared-memory layout as the library's k_staged_forward: persistent CTAs,
// cp.async double buffering when a CTA owns several tiles, the pass's op
// records in shared memory (the offset table region is left unused).  body(s, rops, gbase, on_free, gt): with G::DIRECT the body's last
// stage stores to gt = psi + gbase and calls on_free once its inputs are read.
template <typename R, typename G, typename Body>
__device__ __forceinline__ void jit_staged_forward_g(typename C2<R>::T* psi, int n, const PassArgs& P,
                                                     const tq_tile_stage* __restrict__ stages,
                                                     const ROp<R>* __restrict__ rops_g, int dbuf, Body body) {
  typedef typename C2<R>::T T2;
  constexpr int A = 16 / sizeof(cplx<R>);
  constexpr int NC = (1 << G::T) / A;
  static_assert(NC % G::THREADS == 0, "chunks per tile must be a multiple of the threads");
  constexpr int PER = NC / G::THREADS;
  constexpr int S = A * G::THREADS;
  extern __shared__ __align__(16) unsigned char smem[];
  const int PT = padded_len(G::T);
  cplx<R>* buf0 = reinterpret_cast<cplx<R>*>(smem);
  cplx<R>* buf1 = buf0 + (dbuf ? PT : 0);
  ROp<R>* rops = reinterpret_cast<ROp<R>*>(smem + (size_t)(dbuf ? 2 : 1) * PT * sizeof(cplx<R>) +
                                           staged_hoff_bytes(G::T, G::NLOW));
  const int op0 = stages[P.op_begin].op_begin;
  const int nwords = (stages[P.op_end - 1].op_end - op0) * (int)(sizeof(ROp<R>) / 16);
  const uint4* src = reinterpret_cast<const uint4*>(rops_g + op0);
  uint4* dst = reinterpret_cast<uint4*>(rops);
  for (int w = threadIdx.x; w < nwords; w += blockDim.x) dst[w] = __ldg(&src[w]);
  const int j0 = A * (int)threadIdx.x;
  const int64_t toff = geo_off<G>(j0);
  const int sp0 = pphys(j0);
  auto load = [&](cplx<R>* s, int64_t base) {
    const T2* gp = psi + base + toff;
#pragma unroll
    for (int i = 0; i < PER; ++i) cp_async16(&s[sp0 + pphys(i * S)], &gp[geo_off<G>((int64_t)i * S)]);
  };
  auto store = [&](const cplx<R>* s, int64_t base) {
    T2* gp = psi + base + toff;
#pragma unroll
    for (int i = 0; i < PER; ++i)
      *reinterpret_cast<float4*>(&gp[geo_off<G>((int64_t)i * S)]) =
          *reinterpret_cast<const float4*>(&s[sp0 + pphys(i * S)]);
  };
  __syncthreads();
  const int64_t ntiles = int64_t(1) << (n - G::T);
  int64_t g = blockIdx.x;
  if (g < ntiles) load(buf0, geo_base<G>(g));
  cp_async_commit();
  int cur = 0;
  for (; g < ntiles; g += gridDim.x) {
    const int64_t gn = g + gridDim.x;
    cplx<R>* s = cur ? buf1 : buf0;
    if (dbuf) {
      if (gn < ntiles) load(cur ? buf0 : buf1, geo_base<G>(gn));
      cp_async_commit();
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_group<0>();
    }
    __syncthreads();
    const int64_t gbase = geo_base<G>(g);
    if constexpr (G::DIRECT) {
      // the body's last stage reads its registers, calls on_free (a single
      // buffer then takes the next tile while the stage computes) and stores
      // its results to psi itself
      auto on_free = [&]() {
        if (!dbuf && gn < ntiles) {
          load(buf0, geo_base<G>(gn));
          cp_async_commit();
        }
      };
      body(s, rops, (uint64_t)gbase, on_free, psi + gbase);
    } else {
      body(s, rops, (uint64_t)gbase, []() {}, psi + gbase);
      store(s, gbase);
      __syncthreads();
      if (!dbuf && gn < ntiles) {
        load(buf0, geo_base<G>(gn));
        cp_async_commit();
      }
    }
    cur ^= dbuf;
  }
  cp_async_wait_group<0>();
}

}  // namespace tq
