// Shared-memory tile machinery: gate application on a 2^t-amplitude tile held
// in shared memory, addressed by *local* bit positions 0..t-1.
//
// A tile pass picks t "local" global bit positions pos[0..t-1] (ascending,
// pos[j] = j for the nlow lowest ones so global accesses come in contiguous
// runs of 2^nlow amplitudes).  Tile g holds the 2^t amplitudes whose
// non-local bits spell g.  Every gate whose qubits are all local is applied
// inside shared memory; the tile is read from and written to HBM once per pass.
#pragma once

#include "common.cuh"

namespace tq {

enum TileOpKind : int32_t {
  TOP_U1 = 1,    // dense 2x2 on bit a
  TOP_D1 = 2,    // diag(m0, m1) on bit a
  TOP_U2 = 3,    // dense 4x4 on (a = high, b = low)
  TOP_CX = 4,    // control a, target b
  TOP_CZ = 5,
  TOP_SWAP = 6,
  TOP_PROT = 7,  // exp(-i theta/2 P), P given by local masks xm/zm; m0 = cos, m1 = -i sin * i^ny
};

__device__ __forceinline__ int insz(int i, int p) { return ((i >> p) << (p + 1)) | (i & ((1 << p) - 1)); }

template <typename R>
__device__ __forceinline__ cplx<R> op_m(const tq_tile_op& o, int e);
template <>
__device__ __forceinline__ cplx<float> op_m<float>(const tq_tile_op& o, int e) {
  return cplx<float>(o.mf[2 * e], o.mf[2 * e + 1]);
}
template <>
__device__ __forceinline__ cplx<double> op_m<double>(const tq_tile_op& o, int e) {
  return cplx<double>(o.md[2 * e], o.md[2 * e + 1]);
}

__device__ __forceinline__ void rot_cs(double a, float& c, float& s) { sincosf((float)(0.5 * a), &s, &c); }
__device__ __forceinline__ void rot_cs(double a, double& c, double& s) { sincos(0.5 * a, &s, &c); }

// (m0, m1) of a kind-7 op: fixed, or built from theta for parametrised ops.
template <typename R>
__device__ __forceinline__ void prot_coeffs(const tq_tile_op& o, const double* theta, cplx<R>& m0, cplx<R>& m1) {
  if (o.pidx < 0 || theta == nullptr) {
    m0 = op_m<R>(o, 0);
    m1 = op_m<R>(o, 1);
    return;
  }
  R c, s;
  rot_cs(o.pscale * theta[o.pidx], c, s);
  const int ny = __popc(o.xm & o.zm) & 3;
  // -i s i^ny: ny = 0 -> (0, -s), 1 -> (s, 0), 2 -> (0, s), 3 -> (-s, 0)
  const R sg = (ny >= 2) ? -s : s;
  m0 = cplx<R>(c, R(0));
  m1 = (ny & 1) ? cplx<R>(sg, R(0)) : cplx<R>(R(0), -sg);
}

// Sign of a Pauli rotation's Z factors that lie outside the amplitudes being
// updated together: zg over the tile's non-local bits (fixed by the tile base
// index gbase) and zo over local bits outside a register stage (fixed by the
// thread's local base index tbase).
template <typename R>
__device__ __forceinline__ R zsign(const tq_tile_op& o, uint64_t gbase, int tbase) {
  const int par = (__popcll(gbase & o.zg) + __popc((unsigned)tbase & o.zo)) & 1;
  return par ? R(-1) : R(1);
}

// Apply one op to tile s[0..2^t) with `nt` cooperating threads (index tid).
// `adj` = apply the inverse (U^dagger).  No barrier inside: the caller syncs.
// theta: device angles for ops with pidx >= 0 (may be NULL otherwise);
// gbase: global index of the tile's first amplitude (non-local Z signs).
template <typename R>
__device__ __forceinline__ void tile_apply(cplx<R>* s, int t, const tq_tile_op& o, int tid, int nt, bool adj,
                                           const double* theta = nullptr, uint64_t gbase = 0) {
  const int kind = o.kind;
  const int a = o.a, b = o.b;
  if (kind == TOP_U1) {
    cplx<R> u0 = op_m<R>(o, 0), u1 = op_m<R>(o, 1), u2 = op_m<R>(o, 2), u3 = op_m<R>(o, 3);
    if (adj) {
      cplx<R> t1 = u1;
      u0 = cplx<R>(u0.x, -u0.y);
      u1 = cplx<R>(u2.x, -u2.y);
      u2 = cplx<R>(t1.x, -t1.y);
      u3 = cplx<R>(u3.x, -u3.y);
    }
    const int np = 1 << (t - 1);
    for (int p = tid; p < np; p += nt) {
      const int j0 = insz(p, a), j1 = j0 | (1 << a);
      const cplx<R> x = s[j0], y = s[j1];
      s[j0] = cfma(u1, y, cmul(u0, x));
      s[j1] = cfma(u3, y, cmul(u2, x));
    }
  } else if (kind == TOP_D1) {
    cplx<R> d0 = op_m<R>(o, 0), d1 = op_m<R>(o, 1);
    if (o.pidx >= 0 && theta != nullptr) {  // phase(a) = diag(1, e^{ia})
      R c, sn;
      rot_cs(2.0 * o.pscale * theta[o.pidx], c, sn);
      d0 = cplx<R>(R(1), R(0));
      d1 = cplx<R>(c, sn);
    }
    if (adj) {
      d0.y = -d0.y;
      d1.y = -d1.y;
    }
    const int np = 1 << (t - 1);
    const bool lo_id = (d0.x == R(1) && d0.y == R(0));
    for (int p = tid; p < np; p += nt) {
      const int j0 = insz(p, a), j1 = j0 | (1 << a);
      if (!lo_id) s[j0] = cmul(d0, s[j0]);
      s[j1] = cmul(d1, s[j1]);
    }
  } else if (kind == TOP_U2) {
    const int plo = a < b ? a : b, phi = a < b ? b : a;
    const int nq = 1 << (t - 2);
    for (int p = tid; p < nq; p += nt) {
      const int j = insz(insz(p, plo), phi);
      const int idx[4] = {j, j | (1 << b), j | (1 << a), j | (1 << a) | (1 << b)};
      cplx<R> x[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) x[r] = s[idx[r]];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        cplx<R> acc(0, 0);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          cplx<R> u = adj ? op_m<R>(o, 4 * c + r) : op_m<R>(o, 4 * r + c);
          if (adj) u.y = -u.y;
          acc = cfma(u, x[c], acc);
        }
        s[idx[r]] = acc;
      }
    }
  } else if (kind == TOP_CX || kind == TOP_CZ || kind == TOP_SWAP) {
    const int plo = a < b ? a : b, phi = a < b ? b : a;
    const int nq = 1 << (t - 2);
    for (int p = tid; p < nq; p += nt) {
      const int j = insz(insz(p, plo), phi);
      if (kind == TOP_CX) {
        const int i0 = j | (1 << a), i1 = i0 | (1 << b);
        const cplx<R> x = s[i0];
        s[i0] = s[i1];
        s[i1] = x;
      } else if (kind == TOP_SWAP) {
        const int i0 = j | (1 << a), i1 = j | (1 << b);
        const cplx<R> x = s[i0];
        s[i0] = s[i1];
        s[i1] = x;
      } else {
        const int i = j | (1 << a) | (1 << b);
        s[i] = cplx<R>(-s[i].x, -s[i].y);
      }
    }
  } else if (kind == TOP_PROT) {
    // psi_i <- c psi_i + w * (-1)^{popc(j & zm)} psi_j  with j = i ^ xm, on (i & cm) == cm
    cplx<R> c, w;
    prot_coeffs<R>(o, theta, c, w);
    // exp(+i t/2 P): the sin term flips sign; non-local Z factors give one sign per tile
    const R zs = zsign<R>(o, gbase, 0) * (adj ? R(-1) : R(1));
    w = cplx<R>(zs * w.x, zs * w.y);
    const uint32_t xm = o.xm, zm = o.zm, cm = o.cm;
    if (xm == 0) {
      const int N = 1 << t;
      for (int i = tid; i < N; i += nt) {
        if ((i & cm) != cm) continue;
        const R sg = (__popc(i & zm) & 1) ? R(-1) : R(1);
        s[i] = cmul(cplx<R>(c.x + sg * w.x, sg * w.y), s[i]);
      }
    } else {
      const int h = 31 - __clz(xm);
      const int np = 1 << (t - 1);
      for (int p = tid; p < np; p += nt) {
        const int i = insz(p, h), j = i ^ (int)xm;
        if ((i & cm) != cm) continue;
        const cplx<R> x = s[i], y = s[j];
        const R si = (__popc(i & zm) & 1) ? R(-1) : R(1);
        const R sj = (__popc(j & zm) & 1) ? R(-1) : R(1);
        s[i] = cfma(cplx<R>(w.x * sj, w.y * sj), y, cplx<R>(c.x * x.x, c.x * x.y));
        s[j] = cfma(cplx<R>(w.x * si, w.y * si), x, cplx<R>(c.x * y.x, c.x * y.y));
      }
    }
  }
}

// f(i) = sum_t w_t (-1)^{popc(i & zy_t)} over a Pauli group's terms.
template <typename R>
__device__ __forceinline__ cplx<R> group_f(const tq_pauli_term* __restrict__ terms, int first, int cnt, uint64_t i) {
  R fr = 0, fi = 0;
  for (int t = 0; t < cnt; ++t) {
    const uint64_t zy = __ldg(&terms[first + t].zy);
    const cplx<R> w_ = term_w<R>(&terms[first + t]);
    const R wr = w_.x, wi = w_.y;
    const bool neg = __popcll(i & zy) & 1;
    fr += neg ? -wr : wr;
    fi += neg ? -wi : wi;
  }
  return cplx<R>(fr, fi);
}

// 16-byte global -> shared asynchronous copy (cp.async, L2-only caching).
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"((unsigned long long)gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Thread-partial of Im <lam| G |psi> over the tile, G|i> = [i & cm == cm]
// i^{ny} (-1)^{popc(i & zy)} |i ^ xm> (a Pauli string with optional control
// projector), ph = i^{ny} passed in.  All masks are local.
template <typename R>
__device__ __forceinline__ R tile_grad_partial(const cplx<R>* psi, const cplx<R>* lam, int t, uint32_t xm,
                                               uint32_t zy, uint32_t cm, cplx<R> ph, int tid, int nt) {
  const int N = 1 << t;
  R acc = 0;
  for (int i = tid; i < N; i += nt) {
    if ((i & cm) != cm) continue;
    const R sg = (__popc(i & zy) & 1) ? R(-1) : R(1);
    // conj(lam_{i^xm}) * ph * sg * psi_i
    const cplx<R> v = cmul(ph, psi[i]);
    const cplx<R> l = lam[i ^ xm];
    acc += sg * (l.x * v.y - l.y * v.x);
  }
  return acc;
}

}  // namespace tq
