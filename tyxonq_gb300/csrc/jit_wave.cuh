// Runtime-specialised wave kernels (forward and adjoint passes of the
// L2-resident waves of a batch).
//
// k_wave_forward / k_wave_adjoint (wave.cu) interpret each item's pass: a
// switch per op, runtime register-bit indices for the ops without a register
// routine, and register moves after every dispatch.  Here one kernel is
// generated per distinct pass body of the batch (tyxonq_gb300/jit.py): the
// items of a wave phase are grouped by body, and each group is launched with
// its kernel, whose stages are straight-line register code.  The memory
// schedule, the op records (rop_build per item, with the item's theta offset)
// and the fixed-order gradient partials are those of the library kernels.
#pragma once

#include "jit_staged.cuh"  // register routines shared with the staged passes
#include "wave_io.cuh"

namespace tq {

// In-place adjoint of a dense 4x4 on register bits (A high, B low): U^dagger.
template <typename R, int NR, int A, int B>
__device__ __forceinline__ void j_u2_adj(cplx<R>* x, const tq_tile_op& o) {
  cplx<R> u[16];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const cplx<R> v = op_m<R>(o, 4 * c + r);
      u[4 * r + c] = cplx<R>(v.x, -v.y);
    }
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if (((i >> A) & 1) || ((i >> B) & 1)) continue;
    const int id[4] = {i, i | (1 << B), i | (1 << A), i | (1 << A) | (1 << B)};
    const cplx<R> v[4] = {x[id[0]], x[id[1]], x[id[2]], x[id[3]]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      cplx<R> acc(R(0), R(0));
      acc = cfma(u[4 * r], v[0], acc);
      acc = cfma(u[4 * r + 1], v[1], acc);
      acc = cfma(u[4 * r + 2], v[2], acc);
      acc = cfma(u[4 * r + 3], v[3], acc);
      x[id[r]] = acc;
    }
  }
}

// Im <y|G|x> over the thread's registers for a general generator
// G|i> = [i & CM == CM] ph (-1)^{popc(i & ZM)} |i ^ XM> (register bits; the
// caller applies the sign of Z factors outside the registers).
template <typename R, int NR, int XM, int ZM, int CM>
__device__ __forceinline__ R j_grad(const cplx<R>* x, const cplx<R>* y, cplx<R> ph) {
  R acc = 0;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i & CM) != CM) continue;
    const R sg = (__popc(i & ZM) & 1) ? R(-1) : R(1);
    const cplx<R> v = cmul(ph, x[i]);
    const cplx<R> l = y[i ^ XM];
    acc += sg * (l.x * v.y - l.y * v.x);
  }
  return acc;
}

// Warp sum of a gradient term; lane 0 stores it (fixed order, as the library kernel).
template <typename R>
__device__ __forceinline__ void j_part(R part, R* wpart, int slot, int nwarps, int warp, int lane) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xffffffffu, part, off);
  if (lane == 0) wpart[slot * nwarps + warp] = part;
}

// The item's op records in shared memory: copied from the records compiled once
// per evaluation (tq_wave_rops; rops_g + item.group_begin records), or built
// here when there are none.
template <typename R>
__device__ __forceinline__ void wave_rops(ROp<R>* rops, const void* __restrict__ rops_g, const tq_wave_item& I,
                                          const tq_tile_op* __restrict__ ops, int op0, int nops,
                                          const double* __restrict__ theta, bool adj) {
  if (rops_g != nullptr) {
    // asynchronous 16-byte copies: they complete with the item's tile loads
    // (the caller's commit and wait), so no load round trip of their own
    constexpr int W = (int)(sizeof(ROp<R>) / 16);
    const uint4* src = reinterpret_cast<const uint4*>(rops_g) + (size_t)I.group_begin * W;
    uint4* dst = reinterpret_cast<uint4*>(rops);
    for (int w = threadIdx.x; w < nops * W; w += blockDim.x) cp_async16(&dst[w], &src[w]);
  } else {
    rops_build<R>(rops, ops, op0, op0 + nops, theta + I.theta_off, adj, adj);
  }
}

// Forward pass items: k_wave_forward with the stage loop replaced by
// body(s, rops, gbase) (ends with a barrier after the last stage).
template <typename R, typename Body>
__device__ __forceinline__ void jit_wave_forward(const tq_wave_item* __restrict__ items, int n_items,
                                                 const tq_tile_pass* __restrict__ passes,
                                                 const tq_tile_stage* __restrict__ stages,
                                                 const tq_tile_op* __restrict__ ops, const double* __restrict__ theta,
                                                 const void* __restrict__ rops_g, void* pool, int max_ops, Body body) {
  extern __shared__ __align__(16) unsigned char smem[];
  typedef typename C2<R>::T T2;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const tq_wave_item I = items[it];
    const WPass P = wload_pass(&passes[I.pass], I.n);
    // with compiled records the item carries its op count (group_count); the
    // first op index is needed only to build the records here
    const int op0 = rops_g == nullptr && P.op_end > P.op_begin ? stages[P.op_begin].op_begin : 0;
    const int nops = rops_g != nullptr ? I.group_count
                                       : (P.op_end > P.op_begin ? stages[P.op_end - 1].op_end - op0 : 0);
    if (P.nlow < kWaveMinNlow || nops > max_ops) continue;
    cplx<R>* s = reinterpret_cast<cplx<R>*>(smem);
    int64_t* hoff = reinterpret_cast<int64_t*>(smem + padded_len(P.t) * sizeof(cplx<R>));
    ROp<R>* rops = reinterpret_cast<ROp<R>*>(smem + padded_len(P.t) * sizeof(cplx<R>) + w_hoff_bytes(P.t));
    T2* psi = reinterpret_cast<T2*>(pool) + I.psi_off;
    __syncthreads();
    w_hoff(hoff, P);
    __syncthreads();
    const int64_t base = w_base(I.tile, P);
    // the tile streams in (cp.async) while the op records are compiled
    if (I.basis_lo < 0) w_load<R>(s, psi, base, hoff, P);
    wave_rops<R>(rops, rops_g, I, ops, op0, nops, theta, false);
    if (I.basis_lo >= 0) {
      const int N = 1 << P.t;
      const int lm = (1 << P.nlow) - 1;
      for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
        s[pphys(j)] = cplx<R>(gi == (int64_t)I.basis_lo ? R(1) : R(0), R(0));
      }
    }
    w_commit_wait();  // the tile and the op records
    __syncthreads();
    body(s, rops, (uint64_t)base);
    w_store<R>(s, psi, base, hoff, P);
  }
}

// Adjoint pass items (4-bit stages): k_wave_adjoint with the stage loop replaced
// by body(sp, sl, rops, wpart, gbase, nwarps, warp, lane).
template <typename R, typename Body>
__device__ __forceinline__ void jit_wave_adjoint(const tq_wave_item* __restrict__ items, int n_items,
                                                 const tq_tile_pass* __restrict__ passes,
                                                 const tq_tile_stage* __restrict__ stages,
                                                 const tq_tile_op* __restrict__ ops, const double* __restrict__ theta,
                                                 const void* __restrict__ rops_g, void* pool, double* partials,
                                                 int max_ops, Body body) {
  extern __shared__ __align__(16) unsigned char smem[];
  typedef typename C2<R>::T T2;
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const tq_wave_item I = items[it];
    const WPass P = wload_pass(&passes[I.pass], I.n);
    // with compiled records the item carries its op count (group_count); the
    // first op index is needed only to build the records here
    const int op0 = rops_g == nullptr && P.op_end > P.op_begin ? stages[P.op_begin].op_begin : 0;
    const int nops = rops_g != nullptr ? I.group_count
                                       : (P.op_end > P.op_begin ? stages[P.op_end - 1].op_end - op0 : 0);
    if (P.nlow < kWaveMinNlow || nops > max_ops) continue;
    const int PT = padded_len(P.t);
    cplx<R>* sp = reinterpret_cast<cplx<R>*>(smem);
    cplx<R>* sl = sp + PT;
    unsigned char* tail = smem + 2 * PT * sizeof(cplx<R>);
    int64_t* hoff = reinterpret_cast<int64_t*>(tail);
    ROp<R>* rops = reinterpret_cast<ROp<R>*>(tail + w_hoff_bytes(P.t));
    R* wpart = reinterpret_cast<R*>(tail + w_hoff_bytes(P.t) + (size_t)max_ops * sizeof(ROp<R>));
    T2* psi = reinterpret_cast<T2*>(pool) + I.psi_off;
    T2* lam = reinterpret_cast<T2*>(pool) + I.lam_off;
    __syncthreads();
    w_hoff(hoff, P);
    __syncthreads();
    const int64_t base = w_base(I.tile, P);
    // psi and lam tiles stream in (cp.async) while the op records are compiled
    w_load<R>(sp, psi, base, hoff, P);
    w_load<R>(sl, lam, base, hoff, P);
    for (int k = threadIdx.x; k < nops * nwarps; k += blockDim.x) wpart[k] = R(0);
    wave_rops<R>(rops, rops_g, I, ops, op0, nops, theta, true);
    w_commit_wait();
    __syncthreads();
    body(sp, sl, rops, wpart, (uint64_t)base, nwarps, warp, lane);
    w_store<R>(sp, psi, base, hoff, P);
    w_store<R>(sl, lam, base, hoff, P);
    for (int k = threadIdx.x; k < nops; k += blockDim.x) {
      double s = 0;
      for (int w = 0; w < nwarps; ++w) s += (double)wpart[k * nwarps + w];
      partials[I.part_off + k] = s;
    }
  }
}

}  // namespace tq
