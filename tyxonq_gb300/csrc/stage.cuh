// Register-staged application of tile ops.
//
// A stage names 4 local bit positions (its "register bits").  Thread tid of
// a 2^(t-4)-thread CTA holds the 16 amplitudes whose other local bits spell
// tid; every op of the stage acts on register bits only, so it is applied to
// those 16 registers without touching shared memory.  Shared memory is read
// and written once per stage instead of once per op.  Register-bit indices
// are runtime values; each op kind dispatches to code instantiated for every
// bit combination so the register array is only ever indexed by constants.
//
// Shared-memory tiles are padded by 2 amplitudes per 16 (phys = j + 2*(j>>4)):
// the pad keeps 16-byte chunks aligned for cp.async and spreads the
// stride-16 access pattern of low register bits over the banks.
#pragma once

#include "tile.cuh"

namespace tq {

constexpr int kRB = 4;            // register bits per stage
constexpr int kNR = 1 << kRB;     // amplitudes per thread

__device__ __forceinline__ int pphys(int j) { return j + ((j >> 4) << 1); }
__host__ __device__ __forceinline__ int padded_len(int t) { return (1 << t) + ((1 << t) >> 3); }

template <typename R, int K>
__device__ __forceinline__ void r_u1(cplx<R>* x, cplx<R> u0, cplx<R> u1, cplx<R> u2, cplx<R> u3) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    const cplx<R> a = x[i], b = x[j];
    x[i] = cfma(u1, b, cmul(u0, a));
    x[j] = cfma(u3, b, cmul(u2, a));
  }
}

template <typename R, int K>
__device__ __forceinline__ void r_d1(cplx<R>* x, cplx<R> d0, cplx<R> d1, bool lo_id) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if ((i >> K) & 1)
      x[i] = cmul(d1, x[i]);
    else if (!lo_id)
      x[i] = cmul(d0, x[i]);
  }
}

template <typename R, int A, int B>
__device__ __forceinline__ void r_u2(cplx<R>* x, const tq_tile_op& o, bool adj) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if (((i >> A) & 1) || ((i >> B) & 1)) continue;
    const int id[4] = {i, i | (1 << B), i | (1 << A), i | (1 << A) | (1 << B)};
    const cplx<R> v0 = x[id[0]], v1 = x[id[1]], v2 = x[id[2]], v3 = x[id[3]];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      cplx<R> u[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        u[c] = adj ? op_m<R>(o, 4 * c + r) : op_m<R>(o, 4 * r + c);
        if (adj) u[c].y = -u[c].y;
      }
      cplx<R> acc = cmul(u[0], v0);
      acc = cfma(u[1], v1, acc);
      acc = cfma(u[2], v2, acc);
      acc = cfma(u[3], v3, acc);
      x[id[r]] = acc;
    }
  }
}

// MODE 0 CX (control A, target B), 1 SWAP, 2 CZ
template <typename R, int MODE, int A, int B>
__device__ __forceinline__ void r_perm(cplx<R>* x) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if (((i >> A) & 1) || ((i >> B) & 1)) continue;
    if (MODE == 0) {
      const int p = i | (1 << A), q = p | (1 << B);
      const cplx<R> tmp = x[p];
      x[p] = x[q];
      x[q] = tmp;
    } else if (MODE == 1) {
      const int p = i | (1 << A), q = i | (1 << B);
      const cplx<R> tmp = x[p];
      x[p] = x[q];
      x[q] = tmp;
    } else {
      const int q = i | (1 << A) | (1 << B);
      x[q] = cplx<R>(-x[q].x, -x[q].y);
    }
  }
}

// exp(-i a/2 P) on register bits: flip mask XM (compile time), sign mask zm and
// control mask cm (runtime), coefficients c (real part used) and w.
template <typename R, int XM>
__device__ __forceinline__ void r_prot(cplx<R>* x, uint32_t zm, uint32_t cm, cplx<R> c, cplx<R> w) {
  if (XM == 0) {
#pragma unroll
    for (int i = 0; i < kNR; ++i) {
      if ((i & cm) != cm) continue;
      const R sg = (__popc(i & zm) & 1) ? R(-1) : R(1);
      x[i] = cmul(cplx<R>(c.x + sg * w.x, sg * w.y), x[i]);
    }
  } else {
    constexpr int H = (XM & 8) ? 3 : (XM & 4) ? 2 : (XM & 2) ? 1 : 0;
#pragma unroll
    for (int i = 0; i < kNR; ++i) {
      if ((i >> H) & 1) continue;
      const int j = i ^ XM;
      if ((i & cm) != cm) continue;
      const cplx<R> a = x[i], b = x[j];
      const R si = (__popc(i & zm) & 1) ? R(-1) : R(1);
      const R sj = (__popc(j & zm) & 1) ? R(-1) : R(1);
      x[i] = cfma(cplx<R>(w.x * sj, w.y * sj), b, cplx<R>(c.x * a.x, c.x * a.y));
      x[j] = cfma(cplx<R>(w.x * si, w.y * si), a, cplx<R>(c.x * b.x, c.x * b.y));
    }
  }
}

#define TQ_CASE_AB(FN, ...)                                          \
  switch (o.a * 4 + o.b) {                                            \
    case 1: FN<__VA_ARGS__, 0, 1>(x); break;                          \
    case 2: FN<__VA_ARGS__, 0, 2>(x); break;                          \
    case 3: FN<__VA_ARGS__, 0, 3>(x); break;                          \
    case 4: FN<__VA_ARGS__, 1, 0>(x); break;                          \
    case 6: FN<__VA_ARGS__, 1, 2>(x); break;                          \
    case 7: FN<__VA_ARGS__, 1, 3>(x); break;                          \
    case 8: FN<__VA_ARGS__, 2, 0>(x); break;                          \
    case 9: FN<__VA_ARGS__, 2, 1>(x); break;                          \
    case 11: FN<__VA_ARGS__, 2, 3>(x); break;                         \
    case 12: FN<__VA_ARGS__, 3, 0>(x); break;                         \
    case 13: FN<__VA_ARGS__, 3, 1>(x); break;                         \
    case 14: FN<__VA_ARGS__, 3, 2>(x); break;                         \
    default: break;                                                   \
  }

template <typename R>
__device__ __forceinline__ void r_u2_dispatch(cplx<R>* x, const tq_tile_op& o, bool adj) {
  switch (o.a * 4 + o.b) {
    case 1: r_u2<R, 0, 1>(x, o, adj); break;
    case 2: r_u2<R, 0, 2>(x, o, adj); break;
    case 3: r_u2<R, 0, 3>(x, o, adj); break;
    case 4: r_u2<R, 1, 0>(x, o, adj); break;
    case 6: r_u2<R, 1, 2>(x, o, adj); break;
    case 7: r_u2<R, 1, 3>(x, o, adj); break;
    case 8: r_u2<R, 2, 0>(x, o, adj); break;
    case 9: r_u2<R, 2, 1>(x, o, adj); break;
    case 11: r_u2<R, 2, 3>(x, o, adj); break;
    case 12: r_u2<R, 3, 0>(x, o, adj); break;
    case 13: r_u2<R, 3, 1>(x, o, adj); break;
    case 14: r_u2<R, 3, 2>(x, o, adj); break;
    default: break;
  }
}

// Apply one op (bit indices in register space 0..3) to the 16 registers.
template <typename R>
__device__ __forceinline__ void r_apply(cplx<R>* x, const tq_tile_op& o, const double* theta, bool adj,
                                        R zs = R(1)) {
  switch (o.kind) {
    case TOP_U1: {
      cplx<R> u0 = op_m<R>(o, 0), u1 = op_m<R>(o, 1), u2 = op_m<R>(o, 2), u3 = op_m<R>(o, 3);
      if (adj) {
        const cplx<R> t1 = u1;
        u0 = cplx<R>(u0.x, -u0.y);
        u1 = cplx<R>(u2.x, -u2.y);
        u2 = cplx<R>(t1.x, -t1.y);
        u3 = cplx<R>(u3.x, -u3.y);
      }
      switch (o.a) {
        case 0: r_u1<R, 0>(x, u0, u1, u2, u3); break;
        case 1: r_u1<R, 1>(x, u0, u1, u2, u3); break;
        case 2: r_u1<R, 2>(x, u0, u1, u2, u3); break;
        default: r_u1<R, 3>(x, u0, u1, u2, u3); break;
      }
      break;
    }
    case TOP_D1: {
      cplx<R> d0 = op_m<R>(o, 0), d1 = op_m<R>(o, 1);
      if (o.pidx >= 0 && theta != nullptr) {
        R c, sn;
        rot_cs(2.0 * o.pscale * theta[o.pidx], c, sn);
        d0 = cplx<R>(R(1), R(0));
        d1 = cplx<R>(c, sn);
      }
      if (adj) {
        d0.y = -d0.y;
        d1.y = -d1.y;
      }
      const bool lo_id = (d0.x == R(1) && d0.y == R(0));
      switch (o.a) {
        case 0: r_d1<R, 0>(x, d0, d1, lo_id); break;
        case 1: r_d1<R, 1>(x, d0, d1, lo_id); break;
        case 2: r_d1<R, 2>(x, d0, d1, lo_id); break;
        default: r_d1<R, 3>(x, d0, d1, lo_id); break;
      }
      break;
    }
    case TOP_U2:
      r_u2_dispatch<R>(x, o, adj);
      break;
    case TOP_CX: TQ_CASE_AB(r_perm, R, 0) break;
    case TOP_SWAP: TQ_CASE_AB(r_perm, R, 1) break;
    case TOP_CZ: TQ_CASE_AB(r_perm, R, 2) break;
    case TOP_PROT: {
      cplx<R> c, w;
      prot_coeffs<R>(o, theta, c, w);
      // zs: sign of the Z factors outside the stage (zsign); adjoint flips the sin term
      const R ws = adj ? -zs : zs;
      w = cplx<R>(ws * w.x, ws * w.y);
      const uint32_t zm = o.zm, cm = o.cm;
      switch (o.xm & 15) {
        case 0: r_prot<R, 0>(x, zm, cm, c, w); break;
        case 1: r_prot<R, 1>(x, zm, cm, c, w); break;
        case 2: r_prot<R, 2>(x, zm, cm, c, w); break;
        case 3: r_prot<R, 3>(x, zm, cm, c, w); break;
        case 4: r_prot<R, 4>(x, zm, cm, c, w); break;
        case 5: r_prot<R, 5>(x, zm, cm, c, w); break;
        case 6: r_prot<R, 6>(x, zm, cm, c, w); break;
        case 7: r_prot<R, 7>(x, zm, cm, c, w); break;
        case 8: r_prot<R, 8>(x, zm, cm, c, w); break;
        case 9: r_prot<R, 9>(x, zm, cm, c, w); break;
        case 10: r_prot<R, 10>(x, zm, cm, c, w); break;
        case 11: r_prot<R, 11>(x, zm, cm, c, w); break;
        case 12: r_prot<R, 12>(x, zm, cm, c, w); break;
        case 13: r_prot<R, 13>(x, zm, cm, c, w); break;
        case 14: r_prot<R, 14>(x, zm, cm, c, w); break;
        default: r_prot<R, 15>(x, zm, cm, c, w); break;
      }
      break;
    }
    default: break;
  }
}

// Per-thread register <-> padded shared-memory index of register i for a stage
// with register bits b[0..3] (ascending local positions).
struct StageMap {
  int base;       // local index with all register bits zero
  int m[kRB];     // 1 << bits[k]
  __device__ __forceinline__ int idx(int i) const {  // i is a compile-time constant at every call
    return base | ((i & 1) ? m[0] : 0) | ((i & 2) ? m[1] : 0) | ((i & 4) ? m[2] : 0) | ((i & 8) ? m[3] : 0);
  }
};

__device__ __forceinline__ StageMap stage_map(const tq_tile_stage& st, int tid) {
  StageMap m;
  int b = tid;
#pragma unroll
  for (int k = 0; k < kRB; ++k) b = insz(b, st.bits[k]);
  m.base = b;
#pragma unroll
  for (int k = 0; k < kRB; ++k) m.m[k] = 1 << st.bits[k];
  return m;
}

// Run stages[s0..s1) on the padded tile s (2^(t-4) threads).
template <typename R>
__device__ __forceinline__ void run_stages(cplx<R>* s, const tq_tile_stage* __restrict__ stages, int s0, int s1,
                                           const tq_tile_op* __restrict__ ops, const double* theta, bool adj,
                                           uint64_t gbase) {
  const int tid = threadIdx.x;
  for (int si = s0; si < s1; ++si) {
    const tq_tile_stage st = stages[si];
    const StageMap m = stage_map(st, tid);
    cplx<R> x[kNR];
#pragma unroll
    for (int i = 0; i < kNR; ++i) x[i] = s[pphys(m.idx(i))];
    for (int k = st.op_begin; k < st.op_end; ++k) {
      const tq_tile_op& o = ops[k];
      r_apply<R>(x, o, theta, adj, zsign<R>(o, gbase, m.base));
    }
#pragma unroll
    for (int i = 0; i < kNR; ++i) s[pphys(m.idx(i))] = x[i];
    __syncthreads();
  }
}

}  // namespace tq
