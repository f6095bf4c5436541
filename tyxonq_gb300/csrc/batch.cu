// Batched VQE energy + adjoint gradient: one persistent launch per size class.
//
// CTAs pull instance indices from a device counter (cost-sorted work list, so
// the largest instances start first and the tail is short).
//   resident  (small n): psi and lam = H psi live in shared memory for the whole
//             evaluation; a CTA runs G independent thread groups (named
//             barriers), one instance each.  HBM traffic is only the op,
//             Hamiltonian and parameter tables plus the outputs.
//   streamed  (large n): psi and lam live in the caller's pool; forward tile
//             passes, a tile-blocked H psi (partner tiles grouped by the high
//             part of each flip mask, one load per distinct high part) and
//             adjoint tile passes, all issued by one CTA with cp.async loads.
// No spin-waits: the only inter-CTA interaction is the atomic work counter.
#include "tile.cuh"

namespace tq {

struct BatchArgs {
  const tq_batch_inst* insts;
  const int32_t* work;
  int n_work;
  int groups;
  const tq_tile_pass* passes;
  const tq_tile_op* ops;
  const tq_pauli_group* pgroups;
  const tq_pauli_term* terms;
  const double* theta;
  void* pool;
  double* energies;
  double* grads;
  int32_t* counter;
  int hbits;  // streamed H psi tile bits
};

__device__ __forceinline__ void gsync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

// Sum over a thread group; every thread of the group gets the result.
__device__ __forceinline__ double group_sum(double v, double* red, int gtid, int gsize, int bar) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((gtid & 31) == 0) red[gtid >> 5] = v;
  gsync(bar, gsize);
  double s = 0;
  const int nw = gsize >> 5;
  for (int w = 0; w < nw; ++w) s += red[w];
  gsync(bar, gsize);
  return s;
}

template <typename R>
__device__ __forceinline__ cplx<R> gen_phase(int gny) {
  const R re[4] = {R(1), R(0), R(-1), R(0)}, im[4] = {R(0), R(1), R(0), R(-1)};
  return cplx<R>(re[gny & 3], im[gny & 3]);
}

// ------------------------------------------------------------------ resident
template <typename R>
__device__ void eval_resident(const BatchArgs& A, const tq_batch_inst& I, int inst_id, cplx<R>* psi, cplx<R>* lam,
                              double* red, int gtid, int gsize, int bar) {
  const int n = I.n;
  const int N = 1 << n;
  const double* th = A.theta + I.theta_offset;
  for (int j = gtid; j < N; j += gsize) psi[j] = cplx<R>((int64_t)j == I.basis ? R(1) : R(0), R(0));
  gsync(bar, gsize);
  for (int k = I.fwd_begin; k < I.fwd_begin + I.fwd_count; ++k) {
    tile_apply<R>(psi, n, A.ops[k], gtid, gsize, false, th);
    gsync(bar, gsize);
  }
  // lam = H psi, and E = Re <psi|lam>.  Thread owns j = gtid + k * gsize (k < N / gsize
  // <= 8 for every size class); the term sign parity splits as in k_wave_hpsi.
  R eloc = 0, nloc = 0;
  const int lg = 31 - __clz(gsize);
  const int per = N >> lg;
  if (per >= 1 && per <= 8 && (gsize << lg) != 0) {
    cplx<R> acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = cplx<R>(0, 0);
    for (int g = I.group_begin; g < I.group_begin + I.group_count; ++g) {
      const int m = (int)__ldg(&A.pgroups[g].flip);
      const int first = __ldg(&A.pgroups[g].first_term), cnt = __ldg(&A.pgroups[g].n_terms);
      cplx<R> f[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) f[k] = cplx<R>(0, 0);
      const int sbase = gtid ^ m;
      for (int tt = 0; tt < cnt; ++tt) {
        const int zy = (int)__ldg(&A.terms[first + tt].zy);
        const cplx<R> w_ = term_w<R>(&A.terms[first + tt]);
        const R wr = w_.x, wi = w_.y;
        const int p0 = __popc(sbase & zy) & 1;
        const int kz = zy >> lg;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int kp = k & kz;
          const int par = p0 ^ ((kp ^ (kp >> 1) ^ (kp >> 2)) & 1);
          f[k].x += par ? -wr : wr;
          f[k].y += par ? -wi : wi;
        }
      }
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < per) acc[k] = cfma(f[k], psi[(gtid + (k << lg)) ^ m], acc[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < per) {
        const int j = gtid + (k << lg);
        lam[j] = acc[k];
        eloc += psi[j].x * acc[k].x + psi[j].y * acc[k].y;
        nloc += psi[j].x * psi[j].x + psi[j].y * psi[j].y;
      }
  } else {
    for (int j = gtid; j < N; j += gsize) {
      cplx<R> acc(0, 0);
      for (int g = I.group_begin; g < I.group_begin + I.group_count; ++g) {
        const int k = j ^ (int)__ldg(&A.pgroups[g].flip);
        const cplx<R> f =
            group_f<R>(A.terms, __ldg(&A.pgroups[g].first_term), __ldg(&A.pgroups[g].n_terms), (uint64_t)k);
        acc = cfma(f, psi[k], acc);
      }
      lam[j] = acc;
      eloc += psi[j].x * acc.x + psi[j].y * acc.y;
      nloc += psi[j].x * psi[j].x + psi[j].y * psi[j].y;
    }
  }
  // E = <psi|H|psi> / <psi|psi>: exact for unitary circuits, and for complex64
  // states it removes the norm drift of rounded rotation coefficients; the
  // gradient terms are divided by the same norm
  const double Q = group_sum((double)nloc, red, gtid, gsize, bar);
  const double inv = Q > 0 ? 1.0 / Q : 1.0;
  const double E = group_sum((double)eloc, red, gtid, gsize, bar) * inv;
  // reverse sweep
  double* grad = A.grads + I.grad_offset;
  for (int k = I.adj_begin; k < I.adj_begin + I.adj_count; ++k) {
    const tq_tile_op& o = A.ops[k];
    if (o.slot >= 0) {
      const R part = tile_grad_partial<R>(psi, lam, n, o.gxm, o.gzm, o.gcm, gen_phase<R>(o.gny), gtid, gsize);
      const double s = group_sum((double)part, red, gtid, gsize, bar);
      if (gtid == 0) grad[o.slot] += o.gcoef * s * inv;
    }
    tile_apply<R>(psi, n, o, gtid, gsize, true, th);
    tile_apply<R>(lam, n, o, gtid, gsize, true, th);
    gsync(bar, gsize);
  }
  if (gtid == 0) A.energies[inst_id] = E;
}

template <typename R>
__global__ void __launch_bounds__(1024, 1) k_batch_resident(const BatchArgs A, int region_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int G = A.groups;
  const int gsize = blockDim.x / G;
  const int gid = threadIdx.x / gsize, gtid = threadIdx.x % gsize;
  const int bar = gid + 1;
  unsigned char* base = smem + (size_t)gid * region_bytes;
  double* red = reinterpret_cast<double*>(base);
  int* slot = reinterpret_cast<int*>(base + 32 * sizeof(double));
  cplx<R>* psi = reinterpret_cast<cplx<R>*>(base + 32 * sizeof(double) + 16);
  while (true) {
    if (gtid == 0) *slot = atomicAdd(A.counter, 1);
    gsync(bar, gsize);
    const int w = *slot;
    gsync(bar, gsize);
    if (w >= A.n_work) break;
    const int id = A.work[w];
    const tq_batch_inst I = A.insts[id];
    cplx<R>* lam = psi + (1 << I.n);
    eval_resident<R>(A, I, id, psi, lam, red, gtid, gsize, bar);
  }
}

// ------------------------------------------------------------------ streamed
struct SPass {
  int t, nlow, op_begin, op_end;
  int pos[TQ_TILE_MAX_BITS];
};

__device__ __forceinline__ SPass load_pass(const tq_tile_pass* p) {
  SPass s;
  s.t = p->t;
  s.nlow = p->nlow;
  s.op_begin = p->op_begin;
  s.op_end = p->op_end;
  for (int i = 0; i < TQ_TILE_MAX_BITS; ++i) s.pos[i] = p->pos[i];
  return s;
}

__device__ __forceinline__ void s_build_hoff(int64_t* hoff, const SPass& P) {
  const int nh = 1 << (P.t - P.nlow);
  for (int h = threadIdx.x; h < nh; h += blockDim.x) {
    int64_t off = 0;
    for (int k = 0; k < P.t - P.nlow; ++k)
      if ((h >> k) & 1) off |= int64_t(1) << P.pos[P.nlow + k];
    hoff[h] = off;
  }
}

__device__ __forceinline__ int64_t s_tile_base(int64_t g, const SPass& P) {
  int64_t x = g << P.nlow;
  for (int k = P.nlow; k < P.t; ++k) x = insert_zero(x, P.pos[k]);
  return x;
}

// async tile load: 16-byte chunks (2 complex64 or 1 complex128 amplitude)
template <typename R>
__device__ __forceinline__ void s_tile_load(cplx<R>* s, const typename C2<R>::T* g, int64_t base, const int64_t* hoff,
                                            const SPass& P) {
  constexpr int A = 16 / sizeof(cplx<R>);  // amplitudes per chunk
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    cp_async16(&s[j], &g[gi]);
  }
  cp_async_wait_all();
}
template <typename R>
__device__ __forceinline__ void s_tile_store(const cplx<R>* s, typename C2<R>::T* g, int64_t base,
                                             const int64_t* hoff, const SPass& P) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << P.t) / A;
  const int lm = (1 << P.nlow) - 1;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) {
    const int j = c * A;
    const int64_t gi = base + hoff[j >> P.nlow] + (j & lm);
    *reinterpret_cast<float4*>(&g[gi]) = *reinterpret_cast<const float4*>(&s[j]);
  }
}
// contiguous block of 2^b amplitudes starting at index `start`
template <typename R>
__device__ __forceinline__ void s_block_load(cplx<R>* s, const typename C2<R>::T* g, int64_t start, int b) {
  constexpr int A = 16 / sizeof(cplx<R>);
  const int nc = (1 << b) / A;
  for (int c = threadIdx.x; c < nc; c += blockDim.x) cp_async16(&s[c * A], &g[start + c * A]);
  cp_async_wait_all();
}

template <typename R>
__device__ void eval_streamed(const BatchArgs& A, const tq_batch_inst& I, int inst_id, unsigned char* smem,
                              size_t smem_bytes) {
  typedef typename C2<R>::T T2;
  const int n = I.n;
  const int64_t N = int64_t(1) << n;
  const double* th = A.theta + I.theta_offset;
  T2* psiG = reinterpret_cast<T2*>(A.pool) + I.scratch_offset;
  T2* lamG = psiG + N;
  const int tid = threadIdx.x, nt = blockDim.x;
  double* red = reinterpret_cast<double*>(smem);
  unsigned char* work = smem + 32 * sizeof(double);
  __shared__ double norm_inv;
  for (int64_t i = tid; i < N; i += nt) {
    T2 v;
    v.x = (i == I.basis) ? R(1) : R(0);
    v.y = R(0);
    psiG[i] = v;
  }
  __syncthreads();
  // ---- forward passes
  for (int p = I.fwd_begin; p < I.fwd_begin + I.fwd_count; ++p) {
    const SPass P = load_pass(&A.passes[p]);
    cplx<R>* s = reinterpret_cast<cplx<R>*>(work);
    int64_t* hoff = reinterpret_cast<int64_t*>(work + (sizeof(cplx<R>) << P.t));
    s_build_hoff(hoff, P);
    __syncthreads();
    const int64_t ntiles = int64_t(1) << (n - P.t);
    for (int64_t g = 0; g < ntiles; ++g) {
      const int64_t base = s_tile_base(g, P);
      s_tile_load<R>(s, psiG, base, hoff, P);
      __syncthreads();
      for (int k = P.op_begin; k < P.op_end; ++k) {
        tile_apply<R>(s, P.t, A.ops[k], tid, nt, false, th, (uint64_t)base);
        __syncthreads();
      }
      s_tile_store<R>(s, psiG, base, hoff, P);
      __syncthreads();
    }
  }
  // ---- lam = H psi over contiguous tiles of 2^hb amplitudes
  const int hb = n < A.hbits ? n : A.hbits;
  const int HN = 1 << hb;
  {
    cplx<R>* ps = reinterpret_cast<cplx<R>*>(work);
    cplx<R>* ls = ps + HN;
    R eloc = 0, nloc = 0;
    const int64_t ntile = N >> hb;
    for (int64_t T = 0; T < ntile; ++T) {
      for (int j = tid; j < HN; j += nt) ls[j] = cplx<R>(0, 0);
      int64_t cur = -1;
      for (int g = I.group_begin; g < I.group_begin + I.group_count; ++g) {
        const uint64_t m = __ldg(&A.pgroups[g].flip);
        const int64_t src = T ^ (int64_t)(m >> hb);
        const int ml = (int)(m & (uint64_t)(HN - 1));
        if (src != cur) {
          __syncthreads();
          s_block_load<R>(ps, psiG, src << hb, hb);
          __syncthreads();
          cur = src;
        }
        const int first = __ldg(&A.pgroups[g].first_term), cnt = __ldg(&A.pgroups[g].n_terms);
        for (int j = tid; j < HN; j += nt) {
          const int kl = j ^ ml;
          const cplx<R> f = group_f<R>(A.terms, first, cnt, (uint64_t)((src << hb) | kl));
          ls[j] = cfma(f, ps[kl], ls[j]);
        }
      }
      __syncthreads();
      if (cur != T) {
        s_block_load<R>(ps, psiG, T << hb, hb);
        __syncthreads();
      }
      for (int j = tid; j < HN; j += nt) {
        const cplx<R> a = ps[j], l = ls[j];
        eloc += a.x * l.x + a.y * l.y;
        nloc += a.x * a.x + a.y * a.y;
        T2 v;
        v.x = l.x;
        v.y = l.y;
        lamG[(T << hb) + j] = v;
      }
      __syncthreads();
    }
    // block sums of eloc and of <psi|psi> (the energy and the gradient terms are
    // divided by the norm: see eval_resident)
    double v = (double)eloc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double s = 0;
      for (int w = 0; w < (nt >> 5); ++w) s += red[w];
      A.energies[inst_id] = s;
    }
    __syncthreads();
    v = (double)nloc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
      double q = 0;
      for (int w = 0; w < (nt >> 5); ++w) q += red[w];
      const double inv = q > 0 ? 1.0 / q : 1.0;
      A.energies[inst_id] *= inv;
      norm_inv = inv;
    }
    __syncthreads();
  }
  // ---- adjoint passes
  double* grad = A.grads + I.grad_offset;
  for (int p = I.adj_begin; p < I.adj_begin + I.adj_count; ++p) {
    const SPass P = load_pass(&A.passes[p]);
    const size_t tb = sizeof(cplx<R>) << P.t;
    cplx<R>* sp = reinterpret_cast<cplx<R>*>(work);
    cplx<R>* sl = reinterpret_cast<cplx<R>*>(work + tb);
    int64_t* hoff = reinterpret_cast<int64_t*>(work + 2 * tb);
    double* acc = reinterpret_cast<double*>(work + 2 * tb + (sizeof(int64_t) << (P.t - P.nlow)));
    const int nops = P.op_end - P.op_begin;
    s_build_hoff(hoff, P);
    for (int k = tid; k < nops; k += nt) acc[k] = 0.0;
    __syncthreads();
    const int64_t ntiles = int64_t(1) << (n - P.t);
    for (int64_t g = 0; g < ntiles; ++g) {
      const int64_t base = s_tile_base(g, P);
      s_tile_load<R>(sp, psiG, base, hoff, P);
      s_tile_load<R>(sl, lamG, base, hoff, P);
      __syncthreads();
      for (int k = 0; k < nops; ++k) {
        const tq_tile_op& o = A.ops[P.op_begin + k];
        if (o.slot >= 0) {
          const R part = zsign<R>(o, (uint64_t)base, 0) *
                         tile_grad_partial<R>(sp, sl, P.t, o.gxm, o.gzm, o.gcm, gen_phase<R>(o.gny), tid, nt);
          double v = (double)part;
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
          if ((tid & 31) == 0) red[tid >> 5] = v;
          __syncthreads();
          if (tid == 0) {
            double s = 0;
            for (int w = 0; w < (nt >> 5); ++w) s += red[w];
            acc[k] += s;
          }
          __syncthreads();
        }
        tile_apply<R>(sp, P.t, o, tid, nt, true, th, (uint64_t)base);
        tile_apply<R>(sl, P.t, o, tid, nt, true, th, (uint64_t)base);
        __syncthreads();
      }
      s_tile_store<R>(sp, psiG, base, hoff, P);
      s_tile_store<R>(sl, lamG, base, hoff, P);
      __syncthreads();
    }
    if (tid == 0)
      for (int k = 0; k < nops; ++k) {
        const tq_tile_op& o = A.ops[P.op_begin + k];
        if (o.slot >= 0) grad[o.slot] += o.gcoef * acc[k] * norm_inv;
      }
    __syncthreads();
  }
  (void)smem_bytes;
}

template <typename R>
__global__ void __launch_bounds__(1024, 1) k_batch_streamed(const BatchArgs A, size_t smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int slot;
  while (true) {
    if (threadIdx.x == 0) slot = atomicAdd(A.counter, 1);
    __syncthreads();
    const int w = slot;
    __syncthreads();
    if (w >= A.n_work) break;
    const int id = A.work[w];
    const tq_batch_inst I = A.insts[id];
    eval_streamed<R>(A, I, id, smem, smem_bytes);
    __syncthreads();
  }
}

static size_t region_bytes(int dtype, int max_n) {
  const size_t S = dtype == TQ_C64 ? 8 : 16;
  const size_t b = 32 * sizeof(double) + 16 + 2 * (S << max_n);
  return (b + 127) & ~size_t(127);
}

static size_t streamed_bytes(int dtype, int t) {
  const size_t S = dtype == TQ_C64 ? 8 : 16;
  // 2 tiles + hoff (nlow >= 1) + 512 op accumulators + reduction scratch
  return 32 * sizeof(double) + 2 * (S << t) + (sizeof(int64_t) << (t - 1)) + 512 * sizeof(double) + 256;
}

}  // namespace tq

using namespace tq;

extern "C" size_t tq_batch_smem_bytes(int dtype, int max_resident_n, int groups_per_cta, int streamed_t) {
  if (dtype != TQ_C64 && dtype != TQ_C128) return 0;
  if (streamed_t > 0) return streamed_bytes(dtype, streamed_t);
  if (max_resident_n < 1 || max_resident_n > 16 || groups_per_cta < 1) return 0;
  return region_bytes(dtype, max_resident_n) * (size_t)groups_per_cta;
}

extern "C" int tq_batch_run(int dtype, const tq_batch_inst* insts, const int32_t* work, int n_work, int streamed,
                            int groups_per_cta, int threads_per_cta, int grid, size_t smem_bytes,
                            const tq_tile_pass* passes, const tq_tile_op* ops, const tq_pauli_group* groups,
                            const tq_pauli_term* terms, const double* theta, void* pool, double* energies,
                            double* grads, int32_t* counter, void* stream) {
  TQ_RANGE("tq_batch_run");
  if (dtype != TQ_C64 && dtype != TQ_C128) return fail(TQ_ERR_ARG, "tq_batch_run: bad dtype %d", dtype);
  if (n_work < 0) return fail(TQ_ERR_ARG, "tq_batch_run: negative work count");
  if (n_work == 0) return TQ_OK;
  if (!insts || !work || !ops || !groups || !terms || !theta || !energies || !grads || !counter)
    return fail(TQ_ERR_ARG, "tq_batch_run: NULL pointer");
  if (streamed && (!pool || !passes)) return fail(TQ_ERR_ARG, "tq_batch_run: streamed class needs pool and passes");
  if (groups_per_cta < 1 || groups_per_cta > 8 || (streamed && groups_per_cta != 1))
    return fail(TQ_ERR_ARG, "tq_batch_run: groups_per_cta %d", groups_per_cta);
  if (threads_per_cta < 32 || threads_per_cta > 1024 || threads_per_cta % (32 * groups_per_cta))
    return fail(TQ_ERR_ARG, "tq_batch_run: threads_per_cta %d", threads_per_cta);
  if (grid < 1) return fail(TQ_ERR_ARG, "tq_batch_run: grid %d", grid);
  if (smem_bytes > 227 * 1024) return fail(TQ_ERR_ARG, "tq_batch_run: %zu B shared memory", smem_bytes);
  BatchArgs A;
  A.insts = insts;
  A.work = work;
  A.n_work = n_work;
  A.groups = groups_per_cta;
  A.passes = passes;
  A.ops = ops;
  A.pgroups = groups;
  A.terms = terms;
  A.theta = theta;
  A.pool = pool;
  A.energies = energies;
  A.grads = grads;
  A.counter = counter;
  A.hbits = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (streamed) {
    // H psi tile: two 2^hbits tiles must fit next to the reduction scratch
    const size_t S = dtype == TQ_C64 ? 8 : 16;
    int hb = 1;
    while (hb < 16 && 32 * sizeof(double) + 2 * (S << (hb + 1)) <= smem_bytes) ++hb;
    A.hbits = hb;
    if (dtype == TQ_C64) {
      cudaError_t e = cudaFuncSetAttribute(k_batch_streamed<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes);
      if (e != cudaSuccess) return cuda_status(e, "tq_batch_run: smem attribute");
      k_batch_streamed<float><<<grid, threads_per_cta, smem_bytes, s>>>(A, smem_bytes);
    } else {
      cudaError_t e = cudaFuncSetAttribute(k_batch_streamed<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes);
      if (e != cudaSuccess) return cuda_status(e, "tq_batch_run: smem attribute");
      k_batch_streamed<double><<<grid, threads_per_cta, smem_bytes, s>>>(A, smem_bytes);
    }
  } else {
    const int region = (int)(smem_bytes / groups_per_cta) & ~127;
    if (dtype == TQ_C64) {
      cudaError_t e = cudaFuncSetAttribute(k_batch_resident<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes);
      if (e != cudaSuccess) return cuda_status(e, "tq_batch_run: smem attribute");
      k_batch_resident<float><<<grid, threads_per_cta, smem_bytes, s>>>(A, region);
    } else {
      cudaError_t e = cudaFuncSetAttribute(k_batch_resident<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_bytes);
      if (e != cudaSuccess) return cuda_status(e, "tq_batch_run: smem attribute");
      k_batch_resident<double><<<grid, threads_per_cta, smem_bytes, s>>>(A, region);
    }
  }
  TQ_CHECK_LAUNCH("tq_batch_run");
  return TQ_OK;
}
