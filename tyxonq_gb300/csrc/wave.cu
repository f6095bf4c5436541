// L2-resident waves of large batched instances.
//
// A wave is a set of instances whose psi and lam fit in L2 together.  Each
// phase of a wave (a forward pass, H psi, an adjoint pass) is one launch over
// work items = (instance, tile), so every SM works on the same few states and
// their re-reads (tile passes, the partner reads of H psi) are served by L2.
//   kind 0  forward: register-staged tile pass on psi (the instance's first
//           pass also writes the initial basis state, so no separate init);
//   kind 1  H psi: one output tile of 2^hbits amplitudes per item, partner
//           amplitudes psi[i ^ flip] read from source tiles staged once in
//           shared memory per distinct high part of the flip, accumulators in
//           registers;
//           the item's share of <psi|H psi> goes to partials[part_off];
//   kind 2  adjoint: register-staged un-apply of psi and lam with the
//           gradient terms Im <lam|G|psi> reduced per warp in a fixed order,
//           partials[part_off + k] per op k of the pass.
// Gradient and energy partials are summed by tq_wave_reduce in a fixed order.
#include "stage.cuh"
#include "wave_io.cuh"

namespace tq {

// ------------------------------------------------------------------ forward
// Shared memory: padded tile | offset table (8 << (t - kWaveMinNlow) bytes) |
// the pass's compiled ops (max_ops records, built once per item before any
// register holds amplitudes).
template <typename R>
__global__ void __launch_bounds__(sizeof(R) == 4 ? 512 : 256)
    k_wave_forward(const tq_wave_item* __restrict__ items, int n_items, const tq_tile_pass* __restrict__ passes,
                   const tq_tile_stage* __restrict__ stages, const tq_tile_op* __restrict__ ops,
                   const double* __restrict__ theta, void* pool, int max_ops) {
  extern __shared__ __align__(16) unsigned char smem[];
  typedef typename C2<R>::T T2;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const tq_wave_item I = items[it];
    const WPass P = wload_pass(&passes[I.pass], I.n);
    const int op0 = P.op_end > P.op_begin ? stages[P.op_begin].op_begin : 0;
    const int nops = P.op_end > P.op_begin ? stages[P.op_end - 1].op_end - op0 : 0;
    // tables that would not fit the shared memory sized by the host (never planned)
    if (P.nlow < kWaveMinNlow || nops > max_ops) continue;
    cplx<R>* s = reinterpret_cast<cplx<R>*>(smem);
    int64_t* hoff = reinterpret_cast<int64_t*>(smem + padded_len(P.t) * sizeof(cplx<R>));
    ROp<R>* rops = reinterpret_cast<ROp<R>*>(smem + padded_len(P.t) * sizeof(cplx<R>) + w_hoff_bytes(P.t));
    T2* psi = reinterpret_cast<T2*>(pool) + I.psi_off;
    __syncthreads();  // previous item's readers of s / hoff / rops are done
    w_hoff(hoff, P);
    __syncthreads();
    const int64_t base = w_base(I.tile, P);
    // the tile streams in (cp.async) while the op records are compiled
    if (I.basis_lo < 0) w_load<R>(s, psi, base, hoff, P);
    rops_build<R>(rops, ops, op0, op0 + nops, theta + I.theta_off, false, false);
    if (I.basis_lo >= 0) {
      // first pass of the instance: the tile of |basis> (psi was never written)
      const int N = 1 << P.t;
      const int lm = (1 << P.nlow) - 1;
      for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
        s[pphys(j)] = cplx<R>(gi == (int64_t)I.basis_lo ? R(1) : R(0), R(0));
      }
    } else {
      w_commit_wait();
    }
    __syncthreads();
    run_stages<R>(s, rops, true, op0, stages, P.op_begin, P.op_end, ops, theta + I.theta_off, (uint64_t)base);
    w_store<R>(s, psi, base, hoff, P);
  }
}

// ------------------------------------------------------------------ H psi
// acc[k] += (-1)^popc(k & C) sw * pv[k] (IM: times i) for the one-term groups.
template <typename R, int PER, int C, bool IM>
__device__ __forceinline__ void hpsi_one_term_c(cplx<R>* acc, const cplx<R>* pv, R sw) {
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const R s = (__builtin_popcount(k & C) & 1) ? -sw : sw;
    if (IM) {
      acc[k].x = fma(-s, pv[k].y, acc[k].x);
      acc[k].y = fma(s, pv[k].x, acc[k].y);
    } else {
      acc[k].x = fma(s, pv[k].x, acc[k].x);
      acc[k].y = fma(s, pv[k].y, acc[k].y);
    }
  }
}

template <typename R, int PER, bool IM>
__device__ __forceinline__ void hpsi_one_term(cplx<R>* acc, const cplx<R>* pv, R sw, int c) {
  switch (c) {
#define TQ_HC(C_) \
  case C_: if constexpr (C_ < PER) hpsi_one_term_c<R, PER, C_, IM>(acc, pv, sw); break;
    TQ_HC(0) TQ_HC(1) TQ_HC(2) TQ_HC(3) TQ_HC(4) TQ_HC(5) TQ_HC(6) TQ_HC(7)
    TQ_HC(8) TQ_HC(9) TQ_HC(10) TQ_HC(11) TQ_HC(12) TQ_HC(13) TQ_HC(14) TQ_HC(15)
#undef TQ_HC
    default: break;
  }
}

// A run of one-term groups whose term has sign class C (Z/Y bits 8 .. 11), from
// group g on; returns the first group after the run.  Partner loads by byte
// offset: output j = tid | k << 8, partner (tid ^ ml) ^ (k << 8) in the source
// buffer at byte offset bo.  The group records are software-pipelined: while
// group g computes, the term of group g + 1 and the record of group g + 2 are
// in flight (every index comes from a record already read, none is guessed).
template <typename R, int PER, int C>
__device__ __forceinline__ int hpsi_run_c(cplx<R>* acc, const unsigned char* smem, int bo, int g, int ge, int HN,
                                          int64_t tbase, const tq_pauli_group* __restrict__ groups,
                                          const tq_pauli_term* __restrict__ terms) {
  constexpr int SH = sizeof(cplx<R>) == 8 ? 3 : 4;
  auto rec = [&](int i) { return __ldg(reinterpret_cast<const int4*>(&groups[i])); };
  int4 gr = rec(g);
  uint64_t zy = __ldg(&terms[gr.z].zy);
  cplx<R> w = term_w<R>(&terms[gr.z]);
  int4 gr1 = g + 1 < ge ? rec(g + 1) : make_int4(0, 0, 0, 0);
  for (;;) {
    if (gr.w != 1 || ((int)(zy >> 8) & (PER - 1)) != C) break;
    // next loads: the term of group g + 1, the record of group g + 2
    uint64_t zy1 = 0;
    cplx<R> w1(0, 0);
    const bool has1 = g + 1 < ge && gr1.w >= 1;
    if (has1) {
      zy1 = __ldg(&terms[gr1.z].zy);
      w1 = term_w<R>(&terms[gr1.z]);
    }
    const int4 gr2 = g + 2 < ge ? rec(g + 2) : make_int4(0, 0, 0, 0);
    const uint64_t m = (uint64_t)(uint32_t)gr.x | ((uint64_t)(uint32_t)gr.y << 32);
    const int ml = (int)(m & (uint64_t)(HN - 1));
    const int ab = ((((int)threadIdx.x ^ ml)) << SH) | bo;
    cplx<R> pv[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) pv[k] = *reinterpret_cast<const cplx<R>*>(smem + (ab ^ (k << (8 + SH))));
    const int p0 = __popcll((uint64_t)(tbase ^ (int64_t)m) & zy) & 1;
    if (w.x != R(0)) hpsi_one_term_c<R, PER, C, false>(acc, pv, p0 ? -w.x : w.x);
    if (w.y != R(0)) hpsi_one_term_c<R, PER, C, true>(acc, pv, p0 ? -w.y : w.y);
    ++g;
    if (!has1) break;
    gr = gr1;
    zy = zy1;
    w = w1;
    gr1 = gr2;
  }
  return g;
}

// Item = output tile of HN = 2^hb amplitudes (256 threads x PER).  The partner
// of output i under a group with flip m is psi[i ^ m]: it lies in source tile
// (tile ^ (m >> hb)) at offset (i ^ m) mod HN.  Groups are visited in the order
// of the table (the host sorts them by m >> hb), and each distinct source tile
// is copied once into shared memory, where every group that shares it reads
// its partners.
constexpr int kHpsiThreads = 256;  // every launch of k_wave_hpsi: output j = tid + 256 k
// Groups of up to this many terms apply each term with constant-sign FMAs; larger
// ones sum the terms per sign class and take a Walsh-Hadamard transform.
constexpr int kHpsiFewTerms = 4;

template <typename R, int PER>
__global__ void __launch_bounds__(kHpsiThreads) k_wave_hpsi(const tq_wave_item* __restrict__ items, int n_items, int hbits,
                                                   const tq_pauli_group* __restrict__ groups,
                                                   const tq_pauli_term* __restrict__ terms, void* pool,
                                                   void* lam_pool, double* partials, double* norm_partials) {
  typedef typename C2<R>::T T2;
  extern __shared__ __align__(16) unsigned char smem[];
  cplx<R>* src = reinterpret_cast<cplx<R>*>(smem);
  __shared__ double red[32];
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const tq_wave_item I = items[it];
    const int hb = I.n < hbits ? I.n : hbits;
    const int HN = 1 << hb;
    const T2* psi = reinterpret_cast<const T2*>(pool) + I.psi_off;
    T2* lam = lam_pool ? reinterpret_cast<T2*>(lam_pool) + I.lam_off : nullptr;  // null: energy partials only
    const int64_t tile = I.tile;
    const int64_t t0 = tile << hb;
    cplx<R> acc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) acc[k] = cplx<R>(0, 0);
    const bool full = (HN == PER * kHpsiThreads);
    const int gend = I.group_begin + I.group_count;
    // source tiles double-buffered: the next run's tile streams in while this run computes
    auto issue = [&](cplx<R>* dst, int64_t h) {
      TQ_DCHECK((tile ^ h) < (int64_t(1) << (I.n - hb)), TQ_SITE_HPSI, tile ^ h, h = 0);
      const T2* sp = psi + ((tile ^ h) << hb);
      constexpr int A = 16 / sizeof(cplx<R>);
      if (HN >= A) {
        for (int c = threadIdx.x; c < HN / A; c += blockDim.x) cp_async16(&dst[c * A], &sp[c * A]);
      } else {
        for (int j = threadIdx.x; j < HN; j += blockDim.x) dst[j] = cplx<R>(sp[j].x, sp[j].y);
      }
      cp_async_commit();
    };
    int buf = 0;
    if (I.group_count > 0) issue(src, (int64_t)(__ldg(&groups[I.group_begin].flip) >> hb));
    for (int g = I.group_begin; g < gend;) {
      const int64_t h = (int64_t)(__ldg(&groups[g].flip) >> hb);
      int ge = g + 1;
      while (ge < gend && (int64_t)(__ldg(&groups[ge].flip) >> hb) == h) ++ge;
      cplx<R>* cb = src + (buf ? HN : 0);
      if (ge < gend) issue(src + (buf ? 0 : HN), (int64_t)(__ldg(&groups[ge].flip) >> hb));
      else cp_async_commit();
      cp_async_wait_group<1>();
      __syncthreads();
      for (; g < ge; ++g) {
        // the 16-byte group record {flip, first_term, n_terms} in one load
        const int4 gr = __ldg(reinterpret_cast<const int4*>(&groups[g]));
        if (full && gr.w == 1) {
          // a run of one-term groups of one sign class (the host orders them so):
          // one dispatch on the class for the whole run
          const int c = (int)(__ldg(&terms[gr.z].zy) >> 8) & (PER - 1);
          const int bo = (buf ? HN : 0) * (int)sizeof(cplx<R>);
          const int64_t tb = t0 | (int64_t)threadIdx.x;
          int gn = g + 1;
          switch (c) {
#define TQ_HR(C_) \
  case C_: if constexpr (C_ < PER) gn = hpsi_run_c<R, PER, C_>(acc, smem, bo, g, ge, HN, tb, groups, terms); break;
            TQ_HR(0) TQ_HR(1) TQ_HR(2) TQ_HR(3) TQ_HR(4) TQ_HR(5) TQ_HR(6) TQ_HR(7)
            TQ_HR(8) TQ_HR(9) TQ_HR(10) TQ_HR(11) TQ_HR(12) TQ_HR(13) TQ_HR(14) TQ_HR(15)
#undef TQ_HR
            default: break;
          }
          g = gn - 1;
          continue;
        }
        const uint64_t m = (uint64_t)(uint32_t)gr.x | ((uint64_t)(uint32_t)gr.y << 32);
        const int first = gr.z, cnt = gr.w;
        const int ml = (int)(m & (uint64_t)(HN - 1));
        cplx<R> pv[PER], W[PER];
        if (full) {
          // output j = tid | k << 8 (disjoint bits), so its partner j ^ ml is
          // (tid ^ ml) ^ (k << 8); as a byte offset into the dynamic shared
          // memory (source buffer base HN or 0 is a disjoint high bit), one XOR
          // with a constant per amplitude and the buffer base an immediate
          constexpr int SH = sizeof(cplx<R>) == 8 ? 3 : 4;
          const int ab = ((((int)threadIdx.x ^ ml)) << SH) | ((buf ? HN : 0) << SH);
#pragma unroll
          for (int k = 0; k < PER; ++k) pv[k] = *reinterpret_cast<const cplx<R>*>(smem + (ab ^ (k << (8 + SH))));
        } else {
#pragma unroll
          for (int k = 0; k < PER; ++k) {
            const int j = threadIdx.x + k * kHpsiThreads;
            pv[k] = j < HN ? cb[j ^ ml] : cplx<R>(0, 0);
          }
        }
        // src_k = (t0 | tid | k << 8) ^ m with disjoint bit fields (t0 is a multiple
        // of 2^hb = PER * 256), so parity(src_k & zy) = parity(((t0 | tid) ^ m) & zy)
        // XOR parity(k & c) with c = (zy >> 8) & (PER - 1): one popcount per term
        // and thread.
        const uint64_t sbase = (uint64_t)((t0 | (int64_t)threadIdx.x) ^ (int64_t)m);
        if (cnt <= kHpsiFewTerms) {
          // few terms (most groups of a random Pauli sum have one): each term adds
          // (-1)^(p0 + popc(k & c)) w pv[k] to amplitude k, p0 per thread and c =
          // the term's Z/Y bits among the k bits (the same for every thread), so a
          // uniform switch over c selects code whose per-k signs are constants; a
          // real weight (or the real part) is two FMAs per amplitude, an imaginary
          // one (or part) two more.  Weights c * i^ny of a Pauli sum are one or the
          // other.
          for (int tt = 0; tt < cnt; ++tt) {
            const uint64_t zy = __ldg(&terms[first + tt].zy);
            const cplx<R> w_ = term_w<R>(&terms[first + tt]);
            const int p0 = __popcll(sbase & zy) & 1;
            const int c = (int)(zy >> 8) & (PER - 1);
            if (w_.x != R(0)) hpsi_one_term<R, PER, false>(acc, pv, p0 ? -w_.x : w_.x, c);
            if (w_.y != R(0)) hpsi_one_term<R, PER, true>(acc, pv, p0 ? -w_.y : w_.y, c);
          }
          continue;
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) W[k] = cplx<R>(0, 0);
        {
          // many terms: sum per class c (W_c), then f_k = sum_c W_c (-1)^{popc(k & c)},
          // a PER-point Walsh-Hadamard transform.  Terms sorted by c make the class
          // switches rare; the result does not depend on the order.
          int cur = 0;
          R sr = 0, si = 0;
          for (int tt = 0; tt < cnt; ++tt) {
            const uint64_t zy = __ldg(&terms[first + tt].zy);
            const cplx<R> w_ = term_w<R>(&terms[first + tt]);
            const R wr = w_.x, wi = w_.y;
            const int c = (int)(zy >> 8) & (PER - 1);
            if (c != cur) {  // same for every thread: the term is shared
#pragma unroll
              for (int q = 0; q < PER; ++q)
                if (q == cur) W[q] = cplx<R>(W[q].x + sr, W[q].y + si);
              cur = c;
              sr = si = 0;
            }
            const bool neg = __popcll(sbase & zy) & 1;
            sr += neg ? -wr : wr;
            si += neg ? -wi : wi;
          }
#pragma unroll
          for (int q = 0; q < PER; ++q)
            if (q == cur) W[q] = cplx<R>(W[q].x + sr, W[q].y + si);
#pragma unroll
          for (int hh = 1; hh < PER; hh <<= 1) {
#pragma unroll
            for (int q = 0; q < PER; ++q) {
              if (q & hh) continue;
              const cplx<R> a = W[q], b = W[q + hh];
              W[q] = cplx<R>(a.x + b.x, a.y + b.y);
              W[q + hh] = cplx<R>(a.x - b.x, a.y - b.y);
            }
          }
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) acc[k] = cfma(W[k], pv[k], acc[k]);
      }
      __syncthreads();  // readers of cb are done before it is refilled
      buf ^= 1;
    }
    cp_async_wait_group<0>();
    R eloc = 0, nloc = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int j = threadIdx.x + k * kHpsiThreads;
      if (j < HN) {
        const T2 a = psi[t0 + j];
        eloc += a.x * acc[k].x + a.y * acc[k].y;
        nloc += a.x * a.x + a.y * a.y;
        T2 o;
        o.x = acc[k].x;
        o.y = acc[k].y;
        if (lam) lam[t0 + j] = o;
      }
    }
    double v = (double)eloc, nv = (double)nloc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_down_sync(0xffffffffu, v, o);
      nv += __shfl_down_sync(0xffffffffu, nv, o);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = v;
      red[16 + (threadIdx.x >> 5)] = nv;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0, q = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        s += red[w];
        q += red[16 + w];
      }
      partials[I.part_off] = s;
      // <psi|psi> of the tile: the energy of a complex64 state is divided by it
      // (tq_wave_normalize), which removes the norm drift of rounded rotations
      if (norm_partials) norm_partials[I.part_off] = q;
    }
  }
}

// ------------------------------------------------------------------ adjoint
// Shared memory: psi tile | lam tile | offset table | the pass's compiled ops
// (max_ops records, built at item start) | per-warp gradient partials
// (max_ops x warps, in R; summed over warps in FP64 in a fixed order).
template <typename R, int RB>
__global__ void __launch_bounds__(sizeof(R) == 4 ? 512 : 256, RB == 3 ? 2 : 1)
    k_wave_adjoint(const tq_wave_item* __restrict__ items, int n_items, const tq_tile_pass* __restrict__ passes,
                   const tq_tile_stage* __restrict__ stages, const tq_tile_op* __restrict__ ops,
                   const double* __restrict__ theta, void* pool, double* partials, int max_ops) {
  extern __shared__ __align__(16) unsigned char smem[];
  typedef typename C2<R>::T T2;
  constexpr int NR = 1 << RB;  // amplitudes of psi (and of lam) per thread
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const tq_wave_item I = items[it];
    const WPass P = wload_pass(&passes[I.pass], I.n);
    const int op0 = P.op_end > P.op_begin ? stages[P.op_begin].op_begin : 0;
    const int nops = P.op_end > P.op_begin ? stages[P.op_end - 1].op_end - op0 : 0;
    // tables that would not fit the shared memory sized by the host (never planned)
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
    const double* th = theta + I.theta_off;
    __syncthreads();
    w_hoff(hoff, P);
    __syncthreads();
    const int64_t base = w_base(I.tile, P);
    // psi and lam tiles stream in (cp.async) while the op records are compiled
    w_load<R>(sp, psi, base, hoff, P);
    w_load<R>(sl, lam, base, hoff, P);
    for (int k = threadIdx.x; k < nops * nwarps; k += blockDim.x) wpart[k] = R(0);
    rops_build<R>(rops, ops, op0, op0 + nops, th, true, true);
    w_commit_wait();
    __syncthreads();
    for (int si = P.op_begin; si < P.op_end; ++si) {
      const tq_tile_stage st = stages[si];
      const StageMap<RB> mp = stage_map<RB>(st, threadIdx.x);
      cplx<R> x[NR], y[NR];
      {
        int ad[NR];
        mp.addrs(ad);
#pragma unroll
        for (int i = 0; i < NR; ++i) {
          x[i] = sp[ad[i]];
          y[i] = sl[ad[i]];
        }
      }
      for (int k = st.op_begin; k < st.op_end; ++k) {
        const ROp<R>& r = rops[k - op0];
        const R zs = rop_sign<R>(r, (uint64_t)base, mp.base);
        R part = 0;
        if (rop_is_cold(r)) {  // same for every thread: the record is shared
#pragma unroll
          for (int i = 0; i < NR; ++i) {
            const int j = mp.phys(i);
            sp[j] = x[i];
            sl[j] = y[i];
          }
          const tq_tile_op& o = ops[r.op];
          if (r.gcode != RG_NONE) part = zs * s_cold_grad<R, RB>(sp, sl, mp, o);
          s_cold_apply<R, RB>(sp, mp, o, r, true, zs);
          s_cold_apply<R, RB>(sl, mp, o, r, true, zs);
#pragma unroll
          for (int i = 0; i < NR; ++i) {
            const int j = mp.phys(i);
            x[i] = sp[j];
            y[i] = sl[j];
          }
          if (r.code != RC_U2 && r.code != RC_PROT) rop_apply<R, 2, NR>(x, y, r, ops, true, zs);
        } else {
          if (r.gcode != RG_NONE) part = zs * rop_grad<R, NR>(x, y, r, ops);
          rop_apply<R, 2, NR>(x, y, r, ops, true, zs);
        }
        if (r.gcode != RG_NONE) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xffffffffu, part, off);
          if (lane == 0) wpart[(k - op0) * nwarps + warp] = part;
        }
      }
      {
        int ad[NR];
        mp.addrs(ad);
#pragma unroll
        for (int i = 0; i < NR; ++i) {
          sp[ad[i]] = x[i];
          sl[ad[i]] = y[i];
        }
      }
      __syncthreads();
    }
    w_store<R>(sp, psi, base, hoff, P);
    w_store<R>(sl, lam, base, hoff, P);
    for (int k = threadIdx.x; k < nops; k += blockDim.x) {
      double s = 0;
      for (int w = 0; w < nwarps; ++w) s += (double)wpart[k * nwarps + w];
      partials[I.part_off + k] = s;
    }
  }
}

__global__ void k_wave_reduce(const double* __restrict__ partials, const int32_t* __restrict__ first,
                              const int32_t* __restrict__ count, const int32_t* __restrict__ stride,
                              const double* __restrict__ scale, const int32_t* __restrict__ out_index, int n_out,
                              double* out, int accumulate) {
  // one warp per output: lane l sums partials l, l + 32, ... in order, then a
  // fixed shuffle tree (the same order on every launch)
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_out; r += warps) {
    double s = 0;
    const int f = first[r], c = count[r], st = stride[r];
    for (int j = lane; j < c; j += 32) s += partials[(int64_t)f + (int64_t)j * st];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      s *= scale[r];
      if (accumulate)
        out[out_index[r]] += s;
      else
        out[out_index[r]] = s;
    }
  }
}

template <typename R>
static size_t fwd_smem(int t, int max_ops) {
  return padded_len(t) * sizeof(cplx<R>) + w_hoff_bytes(t) + (size_t)max_ops * sizeof(ROp<R>);
}
template <typename R>
static size_t adj_smem(int t, int rb, int max_ops) {
  return 2 * padded_len(t) * sizeof(cplx<R>) + w_hoff_bytes(t) + (size_t)max_ops * sizeof(ROp<R>) +
         sizeof(R) * (size_t)max_ops * ((1 << (t - rb)) / 32);
}

template <typename R>
static int wave_launch(int kind, const tq_wave_item* items, int n_items, int t, int hbits, int rb,
                       const tq_tile_pass* passes, const tq_tile_stage* stages, const tq_tile_op* ops,
                       const tq_pauli_group* groups, const tq_pauli_term* terms, const double* theta, void* pool,
                       double* partials, double* norm_partials, int max_ops, cudaStream_t s) {
  if (kind == 1) {
    if (hbits < 8 || hbits > 12) return fail(TQ_ERR_ARG, "tq_wave_run: hbits %d outside [8, 12]", hbits);
    const int grid = n_items;
    const size_t sm = 2 * (sizeof(cplx<R>) << hbits);  // two source tiles
    cudaError_t e = cudaSuccess;
#define TQ_HPSI(PER_)                                                                                          \
  e = cudaFuncSetAttribute(k_wave_hpsi<R, PER_>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);        \
  if (e != cudaSuccess) return cuda_status(e, "tq_wave_run: smem attribute");                                  \
  k_wave_hpsi<R, PER_><<<grid, 256, sm, s>>>(items, n_items, hbits, groups, terms, pool, pool, partials,       \
                                             norm_partials);
    switch (hbits) {
      case 8: TQ_HPSI(1) break;
      case 9: TQ_HPSI(2) break;
      case 10: TQ_HPSI(4) break;
      case 11: TQ_HPSI(8) break;
      default: TQ_HPSI(16) break;
    }
#undef TQ_HPSI
    TQ_CHECK_LAUNCH("tq_wave_run (H psi)");
    return TQ_OK;
  }
  if (t < 9 || t > (sizeof(R) == 4 ? 13 : 12)) return fail(TQ_ERR_ARG, "tq_wave_run: t=%d", t);
  if (kind == 0 ? rb != kRB : (rb != 3 && rb != 4))
    return fail(TQ_ERR_ARG, "tq_wave_run: %d register bits per stage (forward 4, adjoint 3 or 4)", rb);
  const int threads = 1 << (t - rb);
  if (threads > (sizeof(R) == 4 ? 512 : 256))
    return fail(TQ_ERR_ARG, "tq_wave_run: t=%d with %d-bit stages needs %d threads per CTA", t, rb, threads);
  const int grid = n_items;
  if (kind == 0) {
    const size_t smem = fwd_smem<R>(t, max_ops);
    if (smem > 227 * 1024) return fail(TQ_ERR_ARG, "tq_wave_run: forward needs %zu B shared memory", smem);
    cudaError_t e = cudaFuncSetAttribute(k_wave_forward<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "tq_wave_run: smem attribute");
    k_wave_forward<R><<<grid, threads, smem, s>>>(items, n_items, passes, stages, ops, theta, pool, max_ops);
  } else {
    const size_t smem = adj_smem<R>(t, rb, max_ops);
    if (smem > 227 * 1024) return fail(TQ_ERR_ARG, "tq_wave_run: adjoint needs %zu B shared memory", smem);
    cudaError_t e = rb == 3 ? cudaFuncSetAttribute(k_wave_adjoint<R, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem)
                            : cudaFuncSetAttribute(k_wave_adjoint<R, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "tq_wave_run: smem attribute");
    if (rb == 3)
      k_wave_adjoint<R, 3><<<grid, threads, smem, s>>>(items, n_items, passes, stages, ops, theta, pool, partials,
                                                        max_ops);
    else
      k_wave_adjoint<R, 4><<<grid, threads, smem, s>>>(items, n_items, passes, stages, ops, theta, pool, partials,
                                                        max_ops);
  }
  TQ_CHECK_LAUNCH("tq_wave_run");
  return TQ_OK;
}

// ---------------------------------------------------------------------------
// One state through k_wave_hpsi: items = (output tile, group slice).  Slice s
// of tile t writes its partial H psi to buf[s] (straight to out when there is
// one slice; nowhere for the energy alone) and its energy partial to
// partials[t * S + s].
constexpr int kTiledHb = 12;

__global__ void k_tiled_items(tq_wave_item* items, int n, int tiles, int slices, int n_groups, int64_t slice_stride) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= tiles * slices) return;
  const int t = it / slices, sl = it % slices;
  const int g0 = (int)((int64_t)n_groups * sl / slices), g1 = (int)((int64_t)n_groups * (sl + 1) / slices);
  tq_wave_item I;
  I.psi_off = 0;
  I.lam_off = (int64_t)sl * slice_stride;
  I.pass = 0;
  I.tile = t;
  I.theta_off = 0;
  I.part_off = it;
  I.n = n;
  I.group_begin = g0;
  I.group_count = g1 - g0;
  I.basis_lo = -1;
  items[it] = I;
}

template <typename R>
__global__ void k_slice_sum(const typename C2<R>::T* __restrict__ buf, int slices, int64_t N,
                            typename C2<R>::T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    typename C2<R>::T a = buf[i];
    for (int sl = 1; sl < slices; ++sl) {
      const typename C2<R>::T b = buf[(int64_t)sl * N + i];
      a.x += b.x;
      a.y += b.y;
    }
    out[i] = a;
  }
}

__global__ void k_sum_partials(const double* __restrict__ p, int n, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += p[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    out[0] = s;
  }
}

static void tiled_shape(int n, int n_groups, int& tiles, int& slices) {
  tiles = 1 << (n - kTiledHb);
  slices = (2 * 152 + tiles - 1) / tiles;
  if (slices > 16) slices = 16;
  if (slices > n_groups) slices = n_groups;
  if (slices < 1) slices = 1;
}

static size_t tiled_buf_amps(int n, int slices, bool have_out) {
  return (have_out && slices > 1) ? (size_t)slices << n : 0;
}

}  // namespace tq

using namespace tq;

extern "C" size_t tq_sv_pauli_sum_tiled_workspace_bytes(int n, int dtype, int n_groups, int with_out) {
  if (n < kTiledHb || n > 40 || (dtype != TQ_C64 && dtype != TQ_C128) || n_groups < 0) return 0;
  int tiles, slices;
  tiled_shape(n, n_groups, tiles, slices);
  const size_t S = dtype == TQ_C64 ? 8 : 16;
  const size_t items = (size_t)tiles * slices;
  size_t b = items * sizeof(tq_wave_item);
  b = (b + 255) & ~(size_t)255;
  b += items * sizeof(double);
  b = (b + 255) & ~(size_t)255;
  return b + S * tiled_buf_amps(n, slices, with_out != 0);
}

extern "C" int tq_sv_pauli_sum_tiled(const void* psi, void* out, int n, int dtype, const tq_pauli_group* groups,
                                     int n_groups, const tq_pauli_term* terms, int n_terms, double* energy_out,
                                     void* ws, size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_pauli_sum_tiled");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n < kTiledHb) return fail(TQ_ERR_ARG, "tq_sv_pauli_sum_tiled: n=%d below %d", n, kTiledHb);
  if (!psi || (!out && !energy_out)) return fail(TQ_ERR_ARG, "tq_sv_pauli_sum_tiled: nothing to compute");
  if (out == psi) return fail(TQ_ERR_ARG, "tq_sv_pauli_sum_tiled: out aliases psi");
  if (n_groups < 0 || n_terms < 0 || (n_groups > 0 && (!groups || !terms)))
    return fail(TQ_ERR_ARG, "tq_sv_pauli_sum_tiled: bad Pauli tables");
  const size_t need = tq_sv_pauli_sum_tiled_workspace_bytes(n, dtype, n_groups, out != nullptr);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_pauli_sum_tiled: workspace of %zu bytes < %zu", ws_bytes, need);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t S = dtype == TQ_C64 ? 8 : 16;
  const int64_t N = int64_t(1) << n;
  if (n_groups == 0) {
    cudaError_t e = cudaSuccess;
    if (out) e = cudaMemsetAsync(out, 0, S * (size_t)N, s);
    if (e == cudaSuccess && energy_out) e = cudaMemsetAsync(energy_out, 0, sizeof(double), s);
    if (e != cudaSuccess) return cuda_status(e, "tq_sv_pauli_sum_tiled: clear");
    return TQ_OK;
  }
  int tiles, slices;
  tiled_shape(n, n_groups, tiles, slices);
  const int items = tiles * slices;
  unsigned char* w = (unsigned char*)ws;
  tq_wave_item* it = (tq_wave_item*)w;
  size_t off = ((size_t)items * sizeof(tq_wave_item) + 255) & ~(size_t)255;
  double* part = (double*)(w + off);
  off = (off + (size_t)items * sizeof(double) + 255) & ~(size_t)255;
  void* buf = tiled_buf_amps(n, slices, out != nullptr) ? (void*)(w + off) : out;  // null: energy only
  k_tiled_items<<<(items + 255) / 256, 256, 0, s>>>(it, n, tiles, slices, n_groups, N);
  const size_t sm = 2 * (S << kTiledHb);
  cudaError_t e;
  if (dtype == TQ_C64) {
    e = cudaFuncSetAttribute(k_wave_hpsi<float, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e, "tq_sv_pauli_sum_tiled: smem attribute");
    k_wave_hpsi<float, 16><<<items, 256, sm, s>>>(it, items, kTiledHb, groups, terms, const_cast<void*>(psi), buf,
                                                  part, nullptr);
    if (out && buf != out)
      k_slice_sum<float><<<grid_for(N, 256), 256, 0, s>>>((const float2*)buf, slices, N, (float2*)out);
  } else {
    e = cudaFuncSetAttribute(k_wave_hpsi<double, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_status(e, "tq_sv_pauli_sum_tiled: smem attribute");
    k_wave_hpsi<double, 16><<<items, 256, sm, s>>>(it, items, kTiledHb, groups, terms, const_cast<void*>(psi), buf,
                                                   part, nullptr);
    if (out && buf != out)
      k_slice_sum<double><<<grid_for(N, 256), 256, 0, s>>>((const double2*)buf, slices, N, (double2*)out);
  }
  if (energy_out) k_sum_partials<<<1, 256, 0, s>>>(part, items, energy_out);
  TQ_CHECK_LAUNCH("tq_sv_pauli_sum_tiled");
  return TQ_OK;
}

extern "C" int tq_wave_run(int kind, int dtype, const tq_wave_item* items, int n_items, int t, int hbits,
                           int stage_bits, const tq_tile_pass* passes, const tq_tile_stage* stages,
                           const tq_tile_op* ops, const tq_pauli_group* groups, const tq_pauli_term* terms,
                           const double* theta, void* pool, double* partials, double* norm_partials,
                           int max_pass_ops, void* stream) {
  TQ_RANGE("tq_wave_run");
  if (dtype != TQ_C64 && dtype != TQ_C128) return fail(TQ_ERR_ARG, "tq_wave_run: bad dtype %d", dtype);
  if (kind < 0 || kind > 2) return fail(TQ_ERR_ARG, "tq_wave_run: bad kind %d", kind);
  if (n_items < 0) return fail(TQ_ERR_ARG, "tq_wave_run: negative item count");
  if (n_items == 0) return TQ_OK;
  if (!items || !pool) return fail(TQ_ERR_ARG, "tq_wave_run: NULL pointer");
  if (kind != 1 && (!passes || !stages || !ops || !theta)) return fail(TQ_ERR_ARG, "tq_wave_run: NULL table");
  if (kind == 1 && (!groups || !terms || !partials)) return fail(TQ_ERR_ARG, "tq_wave_run: NULL Pauli table");
  if (kind == 2 && !partials) return fail(TQ_ERR_ARG, "tq_wave_run: adjoint partials");
  if (kind != 1 && max_pass_ops < 1) return fail(TQ_ERR_ARG, "tq_wave_run: max_pass_ops %d < 1", max_pass_ops);
  cudaStream_t s = (cudaStream_t)stream;
  return dtype == TQ_C64 ? wave_launch<float>(kind, items, n_items, t, hbits, stage_bits, passes, stages, ops, groups,
                                              terms, theta, pool, partials, norm_partials, max_pass_ops, s)
                         : wave_launch<double>(kind, items, n_items, t, hbits, stage_bits, passes, stages, ops,
                                               groups, terms, theta, pool, partials, norm_partials, max_pass_ops, s);
}

// Energies and gradients of complex64 / complex128 states divided by <psi|psi>:
// row r covers instance inst[r], whose norm partials are
// norm_partials[first[r] .. first[r] + count[r]) (summed in order) and whose
// gradient entries are grads[goff[r] .. goff[r] + gcount[r]).
// One warp per row: lane l sums partials l, l + 32, ... in order, then a fixed
// shuffle tree; the result does not depend on the launch, so replays are
// bit-identical.
__global__ void k_wave_normalize(const double* __restrict__ norm_partials, const int32_t* __restrict__ first,
                                 const int32_t* __restrict__ count, const int32_t* __restrict__ inst,
                                 const int32_t* __restrict__ goff, const int32_t* __restrict__ gcount, int n_rows,
                                 double* energies, double* grads) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_rows; r += warps) {
    double q = 0;
    const int f = first[r], c = count[r];
    for (int j = lane; j < c; j += 32) q += norm_partials[f + j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    const double inv = q > 0 ? 1.0 / q : 1.0;
    if (lane == 0) energies[inst[r]] *= inv;
    const int g0 = goff[r], gc = gcount[r];
    for (int j = lane; j < gc; j += 32) grads[g0 + j] *= inv;
  }
}

extern "C" int tq_wave_normalize(const double* norm_partials, const int32_t* first, const int32_t* count,
                                 const int32_t* inst, const int32_t* goff, const int32_t* gcount, int n_rows,
                                 double* energies, double* grads, void* stream) {
  TQ_RANGE("tq_wave_normalize");
  if (n_rows < 0) return fail(TQ_ERR_ARG, "tq_wave_normalize: negative count");
  if (n_rows == 0) return TQ_OK;
  if (!norm_partials || !first || !count || !inst || !goff || !gcount || !energies || !grads)
    return fail(TQ_ERR_ARG, "tq_wave_normalize: NULL pointer");
  k_wave_normalize<<<(n_rows + 3) / 4, 128, 0, (cudaStream_t)stream>>>(norm_partials, first, count, inst, goff,
                                                                        gcount, n_rows, energies, grads);
  TQ_CHECK_LAUNCH("tq_wave_normalize");
  return TQ_OK;
}

extern "C" int tq_wave_reduce(const double* partials, const int32_t* first, const int32_t* count,
                              const int32_t* stride, const double* scale, const int32_t* out_index, int n_out,
                              double* out, int accumulate, void* stream) {
  TQ_RANGE("tq_wave_reduce");
  if (n_out < 0) return fail(TQ_ERR_ARG, "tq_wave_reduce: negative count");
  if (n_out == 0) return TQ_OK;
  if (!partials || !first || !count || !stride || !scale || !out_index || !out)
    return fail(TQ_ERR_ARG, "tq_wave_reduce: NULL pointer");
  const int threads = 256;
  const int64_t want = ((int64_t)n_out * 32 + threads - 1) / threads;  // a warp per output
  const int grid = (int)(want < 4096 ? want : 4096);
  k_wave_reduce<<<grid, threads, 0, (cudaStream_t)stream>>>(partials, first, count, stride, scale, out_index, n_out,
                                                            out, accumulate);
  TQ_CHECK_LAUNCH("tq_wave_reduce");
  return TQ_OK;
}
TQ_CHECK_UNIT(wave)
