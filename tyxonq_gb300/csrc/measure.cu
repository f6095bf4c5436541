// Read-side kernels: norms, inner products, <Z_q>, probabilities, Pauli-sum
// expectation and H*psi, and Z-basis shot sampling.
//
// Accumulation: a thread sums a short run of products in the state's own
// precision and folds it into an FP64 accumulator; blocks write FP64 partials
// into caller-provided workspace and a single-block finalize kernel adds them
// in a fixed order, so every result is bit-identical run to run.
#include <cmath>

#include "common.cuh"

namespace tq {

static const int kRedThreads = 256;

template <typename R>
__device__ __forceinline__ cplx<R> ldc(const typename C2<R>::T* p, int64_t i) {
  typename C2<R>::T v = p[i];
  return cplx<R>(v.x, v.y);
}

// Sum of v over the block; result valid in thread 0. `sh` needs 32 doubles.
__device__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = (l < nw) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// Number of partial-sum blocks for a reduction over N amplitudes (a function
// of n only, so the summation order is fixed).
static int red_blocks(int n) {
  const int64_t N = int64_t(1) << n;
  int64_t b = (N + 4095) / 4096;
  if (b > 1216) b = 1216;
  if (b < 1) b = 1;
  return (int)b;
}

// out[o] = sum_b partials[b * nout + o] for o < nout (one block per output).
__global__ void k_finalize(const double* partials, int nblk, int nout, double* out) {
  __shared__ double sh[32];
  const int o = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += partials[(int64_t)b * nout + o];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) out[o] = acc;
}

// ----------------------------------------------------------------- one-qubit reduced density matrix
// Over the pairs (a, b) = (psi_i, psi_{i | bit}) with the bit clear:
// partials[blk * 4 + {0,1,2,3}] = sum |a|^2, sum |b|^2, Re sum a conj(b), Im sum a conj(b).
template <typename R>
__global__ void k_qubit_rdm(const typename C2<R>::T* psi, int64_t half, int bit, double* partials) {
  __shared__ double sh[32];
  R s00 = 0, s11 = 0, sre = 0, sim = 0;
  const int64_t lo = (int64_t(1) << bit) - 1;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < half; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = ((p >> bit) << (bit + 1)) | (p & lo);
    const cplx<R> a = ldc<R>(psi, i), b = ldc<R>(psi, i | (int64_t(1) << bit));
    s00 += a.x * a.x + a.y * a.y;
    s11 += b.x * b.x + b.y * b.y;
    sre += a.x * b.x + a.y * b.y;
    sim += a.y * b.x - a.x * b.y;
  }
  const R v[4] = {s00, s11, sre, sim};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double t = block_sum((double)v[k], sh);
    if (threadIdx.x == 0) partials[(int64_t)blockIdx.x * 4 + k] = t;
  }
}

// ----------------------------------------------------------------- norm / inner
template <typename R>
__global__ void k_inner_re(const typename C2<R>::T* a, const typename C2<R>::T* b, int64_t N,
                           double* partials) {
  __shared__ double sh[32];
  double acc = 0.0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  while (i < N) {
    R loc = 0;
#pragma unroll 4
    for (int u = 0; u < 8 && i < N; ++u, i += stride) {
      cplx<R> x = ldc<R>(a, i), y = b ? ldc<R>(b, i) : x;
      loc += x.x * y.x + x.y * y.y;
    }
    acc += (double)loc;
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// ----------------------------------------------------------------- <Z_q> for all q
// Block = chunk of CH = min(N, 8192) contiguous amplitudes, 256 threads.
// Thread t reads i = base + t + 256*k.  Bits below LB = log2(min(256, CH))
// are fixed by t, bits LB..log2(CH)-1 come from k, bits above from the block.
template <typename R>
__global__ void k_expect_z(const typename C2<R>::T* psi, int n, int lch, double* partials) {
  __shared__ double sh[32];
  const int64_t CH = int64_t(1) << lch;
  const int64_t base = int64_t(blockIdx.x) << lch;
  const int LB = lch < 8 ? lch : 8;
  const int KB = lch - LB;
  const int nk = 1 << KB;
  const int t = threadIdx.x;
  R tot = 0;
  R kacc[5] = {0, 0, 0, 0, 0};
  if (t < (1 << LB)) {
    for (int k = 0; k < nk; ++k) {
      cplx<R> a = ldc<R>(psi, base + t + (int64_t(k) << LB));
      const R p = a.x * a.x + a.y * a.y;
      tot += p;
#pragma unroll
      for (int j = 0; j < 5; ++j)
        if (j < KB) kacc[j] += ((k >> j) & 1) ? -p : p;
    }
  }
  (void)CH;
  // reduce: total, per low bit (from t), per k bit
  double btot = block_sum((double)tot, sh);
  __shared__ double res[TQ_MAX_QUBITS + 1];
  if (t == 0) res[TQ_MAX_QUBITS] = btot;
  for (int pos = 0; pos < LB; ++pos) {
    double v = block_sum((double)(((t >> pos) & 1) ? -tot : tot), sh);
    if (t == 0) res[pos] = v;
  }
  for (int j = 0; j < KB; ++j) {
    double v = block_sum((double)kacc[j], sh);
    if (t == 0) res[LB + j] = v;
  }
  __syncthreads();
  if (t == 0) {
    const double bt = res[TQ_MAX_QUBITS];
    for (int pos = lch; pos < n; ++pos) res[pos] = ((base >> pos) & 1) ? -bt : bt;
    // partial layout [block][qubit]: qubit q <-> bit n-1-q
    for (int q = 0; q < n; ++q) partials[(int64_t)blockIdx.x * n + q] = res[n - 1 - q];
  }
}

// ----------------------------------------------------------------- probabilities
__global__ void k_probs_c64(const float4* psi4, float2* probs2, int64_t items) {
  for (int64_t v = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < items; v += int64_t(gridDim.x) * blockDim.x) {
    float4 a = psi4[v];
    probs2[v] = make_float2(a.x * a.x + a.y * a.y, a.z * a.z + a.w * a.w);
  }
}
__global__ void k_probs_c64_one(const float2* psi, float* probs) {
  if (threadIdx.x == 0) probs[0] = psi[0].x * psi[0].x + psi[0].y * psi[0].y;
}
__global__ void k_probs_c128(const double2* psi, double* probs, int64_t N) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x) {
    double2 a = psi[i];
    probs[i] = a.x * a.x + a.y * a.y;
  }
}

// ----------------------------------------------------------------- Pauli sums
// f_g(i) = sum_{t in g} w_t (-1)^{popc(i & zy_t)}
template <typename R>
__device__ __forceinline__ cplx<R> pauli_f(const tq_pauli_term* __restrict__ terms, int first, int cnt,
                                          uint64_t i) {
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

// Grid (nchunk, n_groups).  Group g with flip m != 0 sums over the N/2 indices i
// with bit h(m) clear: 2 Re[conj(psi_{i^m}) psi_i f(i)]; m == 0 sums |psi_i|^2 f(i).
template <typename R>
__global__ void k_pauli_expect(const typename C2<R>::T* psi, int n, const tq_pauli_group* __restrict__ groups,
                               const tq_pauli_term* __restrict__ terms, double* partials, int nchunk) {
  __shared__ double sh[32];
  const int g = blockIdx.y;
  const uint64_t m = groups[g].flip;
  const int first = groups[g].first_term, cnt = groups[g].n_terms;
  const int64_t N = int64_t(1) << n;
  const int64_t items = m ? N / 2 : N;
  const int h = m ? 63 - __clzll((long long)m) : 0;
  const int64_t per = (items + nchunk - 1) / nchunk;
  const int64_t lo = per * blockIdx.x;
  int64_t hi = lo + per;
  if (hi > items) hi = items;
  double acc = 0.0;
  int64_t v = lo + threadIdx.x;
  while (v < hi) {
    R loc = 0;
    for (int u = 0; u < 8 && v < hi; ++u, v += blockDim.x) {
      const int64_t i = m ? insert_zero(v, h) : v;
      const cplx<R> f = pauli_f<R>(terms, first, cnt, (uint64_t)i);
      const cplx<R> a = ldc<R>(psi, i);
      if (m) {
        const cplx<R> b = ldc<R>(psi, i ^ (int64_t)m);
        const cplx<R> z = cconjmul(b, a);  // conj(psi_j) psi_i
        loc += R(2) * (z.x * f.x - z.y * f.y);
      } else {
        loc += (a.x * a.x + a.y * a.y) * f.x;
      }
    }
    acc += (double)loc;
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[(int64_t)g * nchunk + blockIdx.x] = acc;
}

// out_i = sum_g psi_{i^m_g} f_g(i^m_g)
template <typename R>
__global__ void k_apply_pauli_sum(const typename C2<R>::T* psi, typename C2<R>::T* out, int64_t N,
                                  const tq_pauli_group* __restrict__ groups, int ngroups,
                                  const tq_pauli_term* __restrict__ terms) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x) {
    cplx<R> acc(0, 0);
    for (int g = 0; g < ngroups; ++g) {
      const uint64_t m = __ldg(&groups[g].flip);
      const int64_t k = i ^ (int64_t)m;
      const cplx<R> f = pauli_f<R>(terms, __ldg(&groups[g].first_term), __ldg(&groups[g].n_terms), (uint64_t)k);
      acc = cfma(f, ldc<R>(psi, k), acc);
    }
    typename C2<R>::T o;
    o.x = acc.x;
    o.y = acc.y;
    out[i] = o;
  }
}

// ----------------------------------------------------------------- sampling
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): counter (ctr, 0, 0), key = seed.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}
__device__ __forceinline__ float u01_open_hi(uint32_t x) {  // [0, 1)
  return (float)(x >> 8) * (1.0f / 16777216.0f);
}

static const int kSampCH = 4096;     // amplitudes per chunk
static const int kSampThreads = 256;
static const int kSpacePerBlock = 2048;  // shots per spacing block (256 threads x 8)

// chunk c: sums[c] = sum |psi|^2 over the chunk (FP64)
template <typename R>
__global__ void k_chunk_sums(const typename C2<R>::T* psi, int64_t N, double* sums) {
  __shared__ double sh[32];
  const int64_t base = int64_t(blockIdx.x) * kSampCH;
  R loc = 0;
  for (int k = threadIdx.x; k < kSampCH; k += blockDim.x) {
    const int64_t i = base + k;
    if (i < N) {
      cplx<R> a = ldc<R>(psi, i);
      loc += a.x * a.x + a.y * a.y;
    }
  }
  double acc = block_sum((double)loc, sh);
  if (threadIdx.x == 0) sums[blockIdx.x] = acc;
}

// In-place exclusive scan of x[0..cnt) with x[cnt] = total, one block of 1024.
__global__ void k_scan_excl(double* x, int64_t cnt) {
  __shared__ double seg[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int64_t per = (cnt + T - 1) / T;
  const int64_t lo = per * t;
  const int64_t hi = (lo + per < cnt) ? lo + per : cnt;
  double s = 0;
  for (int64_t i = lo; i < hi; ++i) s += x[i];
  seg[t] = s;
  __syncthreads();
  if (t == 0) {
    double run = 0;
    for (int j = 0; j < T; ++j) {
      const double v = seg[j];
      seg[j] = run;
      run += v;
    }
    x[cnt] = run;
  }
  __syncthreads();
  double run = seg[t];
  for (int64_t i = lo; i < hi; ++i) {
    const double v = x[i];
    x[i] = run;
    run += v;
  }
}

// Exponential spacings E_k = -log(1-u_k), k in [0, M] (M = shots): within-block
// inclusive scan into tgt[k] (k < M), block totals into bsum[block].
__global__ void k_spacings(double* tgt, int64_t M, uint64_t seed, double* bsum) {
  __shared__ double sh[kSampThreads];
  const int t = threadIdx.x;
  const int64_t k0 = int64_t(blockIdx.x) * kSpacePerBlock + int64_t(t) * 8;
  float e[8];
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint64_t ctr = (uint64_t)(k0 + 4 * h) >> 2;
    uint4 r = philox4x32_10(make_uint4((uint32_t)ctr, (uint32_t)(ctr >> 32), 0x5A4D504Cu, 0u), key);
    const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) e[4 * h + j] = -log1pf(-u01_open_hi(rr[j]));
  }
  double loc[8];
  double s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const bool valid = (k0 + j) <= M;
    s += valid ? (double)e[j] : 0.0;
    loc[j] = s;
  }
  sh[t] = s;
  __syncthreads();
  // inclusive scan of per-thread sums (Hillis-Steele, 256 entries)
  for (int o = 1; o < kSampThreads; o <<= 1) {
    double v = (t >= o) ? sh[t - o] : 0.0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  const double before = (t > 0) ? sh[t - 1] : 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (k0 + j < M) tgt[k0 + j] = before + loc[j];
  if (t == kSampThreads - 1) bsum[blockIdx.x] = sh[t];
}

// tgt[k] = min((tgt[k] + bsum_excl[block]) / S_total * T, prev(T))
__global__ void k_targets(double* tgt, int64_t M, const double* bsum_excl, int64_t nsb, const double* prefix,
                          int64_t nchunks) {
  const double S = bsum_excl[nsb];
  const double T = prefix[nchunks];
  const double cap = nextafter(T, 0.0);
  for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < M; k += int64_t(gridDim.x) * blockDim.x) {
    double v = (tgt[k] + bsum_excl[k / kSpacePerBlock]) / S * T;
    tgt[k] = v < cap ? v : cap;
  }
}

__device__ __forceinline__ int64_t lower_bound_d(const double* a, int64_t cnt, double x) {
  int64_t lo = 0, hi = cnt;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <typename R>
__global__ void k_resolve(const typename C2<R>::T* psi, int64_t N, const double* prefix, int64_t nchunks,
                          const double* tgt, int64_t M, int64_t* out) {
  __shared__ R cum[kSampCH];
  __shared__ int64_t range[2];
  __shared__ int last_nz;
  const int64_t c = blockIdx.x;
  if (threadIdx.x == 0) {
    range[0] = lower_bound_d(tgt, M, prefix[c]);
    range[1] = (c == nchunks - 1) ? M : lower_bound_d(tgt, M, prefix[c + 1]);
    last_nz = -1;
  }
  __syncthreads();
  const int64_t lo = range[0], hi = range[1];
  if (lo >= hi) return;
  const int64_t base = c * kSampCH;
  const int len = (int)((N - base) < kSampCH ? (N - base) : kSampCH);
  // per-thread contiguous segment scan
  const int T = blockDim.x, t = threadIdx.x;
  const int per = (len + T - 1) / T;
  const int s0 = per * t, s1 = (s0 + per < len) ? s0 + per : len;
  R run = 0;
  int my_last = -1;
  for (int j = s0; j < s1; ++j) {
    cplx<R> a = ldc<R>(psi, base + j);
    const R p = a.x * a.x + a.y * a.y;
    if (p > R(0)) my_last = j;
    run += p;
    cum[j] = run;
  }
  if (my_last >= 0) atomicMax(&last_nz, my_last);
  __shared__ R segsum[kSampThreads];
  segsum[t] = run;
  __syncthreads();
  if (t == 0) {
    R r = 0;
    for (int j = 0; j < T; ++j) {
      const R v = segsum[j];
      segsum[j] = r;
      r += v;
    }
  }
  __syncthreads();
  const R off = segsum[t];
  for (int j = s0; j < s1; ++j) cum[j] += off;
  __syncthreads();
  const double p0 = prefix[c];
  const int lnz = last_nz;
  for (int64_t k = lo + t; k < hi; k += T) {
    const R x = (R)(tgt[k] - p0);
    // first j with cum[j] > x
    int a = 0, b = len;
    while (a < b) {
      const int mid = (a + b) >> 1;
      if (cum[mid] > x) b = mid;
      else a = mid + 1;
    }
    int j = (a < len) ? a : lnz;
    if (j > lnz) j = lnz;
    TQ_DCHECK(base + (j < 0 ? 0 : j) < N, TQ_SITE_SAMPLE, base + j, j = -1);
    out[k] = base + (j < 0 ? 0 : j);
  }
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace tq

using namespace tq;
#define STREAM(s) ((cudaStream_t)(s))

// ----------------------------------------------------------------- C ABI
extern "C" size_t tq_sv_norm_workspace_bytes(int n) {
  if (n < 0 || n > TQ_MAX_QUBITS) return 0;
  return sizeof(double) * red_blocks(n);
}
extern "C" size_t tq_sv_inner_workspace_bytes(int n) { return tq_sv_norm_workspace_bytes(n); }

static int inner_impl(const void* a, const void* b, int n, int dtype, double* out, void* ws, size_t ws_bytes,
                      void* stream, const char* name) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!a || !out) return fail(TQ_ERR_ARG, "%s: NULL pointer", name);
  const int nb = red_blocks(n);
  if (!ws || ws_bytes < sizeof(double) * nb)
    return fail(TQ_ERR_WORKSPACE, "%s: workspace of %zu bytes < %zu", name, ws_bytes, sizeof(double) * nb);
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  double* part = (double*)ws;
  if (dtype == TQ_C64)
    k_inner_re<float><<<nb, kRedThreads, 0, s>>>((const float2*)a, (const float2*)b, N, part);
  else
    k_inner_re<double><<<nb, kRedThreads, 0, s>>>((const double2*)a, (const double2*)b, N, part);
  k_finalize<<<1, 1024, 0, s>>>(part, nb, 1, out);
  TQ_CHECK_LAUNCH(name);
  return TQ_OK;
}

extern "C" int tq_sv_norm2(const void* psi, int n, int dtype, double* out_dev, void* ws, size_t ws_bytes,
                           void* stream) {
  TQ_RANGE("tq_sv_norm2");
  return inner_impl(psi, nullptr, n, dtype, out_dev, ws, ws_bytes, stream, "tq_sv_norm2");
}
extern "C" int tq_sv_inner_re(const void* a, const void* b, int n, int dtype, double* out_dev, void* ws,
                              size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_inner_re");
  if (!b) return fail(TQ_ERR_ARG, "tq_sv_inner_re: b is NULL");
  return inner_impl(a, b, n, dtype, out_dev, ws, ws_bytes, stream, "tq_sv_inner_re");
}

static int lch_for(int n) { return n < 13 ? n : 13; }

extern "C" size_t tq_sv_expect_z_workspace_bytes(int n) {
  if (n < 1 || n > TQ_MAX_QUBITS) return 0;
  const int64_t nb = (int64_t(1) << n) >> lch_for(n);
  return sizeof(double) * nb * n;
}

extern "C" int tq_sv_expect_z_all(const void* psi, int n, int dtype, double* out_dev, void* ws, size_t ws_bytes,
                                  void* stream) {
  TQ_RANGE("tq_sv_expect_z_all");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (n == 0) return TQ_OK;
  if (!psi || !out_dev) return fail(TQ_ERR_ARG, "tq_sv_expect_z_all: NULL pointer");
  const size_t need = tq_sv_expect_z_workspace_bytes(n);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_expect_z_all: workspace of %zu bytes < %zu", ws_bytes, need);
  const int lch = lch_for(n);
  const int64_t nb = (int64_t(1) << n) >> lch;
  if (nb > 0x7fffffff) return fail(TQ_ERR_RANGE, "state too large");
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_expect_z<float><<<(unsigned)nb, 256, 0, s>>>((const float2*)psi, n, lch, (double*)ws);
  else
    k_expect_z<double><<<(unsigned)nb, 256, 0, s>>>((const double2*)psi, n, lch, (double*)ws);
  k_finalize<<<n, 1024, 0, s>>>((const double*)ws, (int)nb, n, out_dev);
  TQ_CHECK_LAUNCH("tq_sv_expect_z_all");
  return TQ_OK;
}

extern "C" size_t tq_sv_qubit_rdm_workspace_bytes(int n) {
  if (n < 1 || n > TQ_MAX_QUBITS) return 0;
  return sizeof(double) * 4 * (size_t)red_blocks(n - 1);
}

extern "C" int tq_sv_qubit_rdm(const void* psi, int n, int dtype, int qubit, double* out_dev, void* ws,
                               size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_qubit_rdm");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if ((rc = check_qubit(n, qubit))) return rc;
  if (!psi || !out_dev) return fail(TQ_ERR_ARG, "tq_sv_qubit_rdm: NULL pointer");
  const size_t need = tq_sv_qubit_rdm_workspace_bytes(n);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_qubit_rdm: workspace of %zu bytes < %zu", ws_bytes, need);
  const int nb = red_blocks(n - 1);
  const int64_t half = int64_t(1) << (n - 1);
  const int bit = tq_bit(n, qubit);
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_qubit_rdm<float><<<nb, 256, 0, s>>>((const float2*)psi, half, bit, (double*)ws);
  else
    k_qubit_rdm<double><<<nb, 256, 0, s>>>((const double2*)psi, half, bit, (double*)ws);
  k_finalize<<<4, 1024, 0, s>>>((const double*)ws, nb, 4, out_dev);
  TQ_CHECK_LAUNCH("tq_sv_qubit_rdm");
  return TQ_OK;
}

extern "C" int tq_sv_probabilities(const void* psi, int n, int dtype, void* probs, void* stream) {
  TQ_RANGE("tq_sv_probabilities");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi || !probs) return fail(TQ_ERR_ARG, "tq_sv_probabilities: NULL pointer");
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64) {
    if (N >= 2)
      k_probs_c64<<<grid_for(N / 2, 256), 256, 0, s>>>((const float4*)psi, (float2*)probs, N / 2);
    else
      k_probs_c64_one<<<1, 32, 0, s>>>((const float2*)psi, (float*)probs);
  } else {
    k_probs_c128<<<grid_for(N, 256), 256, 0, s>>>((const double2*)psi, (double*)probs, N);
  }
  TQ_CHECK_LAUNCH("tq_sv_probabilities");
  return TQ_OK;
}

static int pauli_nchunk(int n) {
  const int64_t N = int64_t(1) << n;
  int64_t c = (N + 2047) / 2048;
  if (c > 2048) c = 2048;
  if (c < 1) c = 1;
  return (int)c;
}

extern "C" size_t tq_sv_pauli_expectation_workspace_bytes(int n, int n_groups) {
  if (n < 0 || n > TQ_MAX_QUBITS || n_groups < 0) return 0;
  return sizeof(double) * (size_t)pauli_nchunk(n) * (size_t)(n_groups > 0 ? n_groups : 1);
}

extern "C" int tq_sv_pauli_expectation(const void* psi, int n, int dtype, const tq_pauli_group* groups, int n_groups,
                                       const tq_pauli_term* terms, int n_terms, double* out_dev, void* ws,
                                       size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_pauli_expectation");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi || !out_dev) return fail(TQ_ERR_ARG, "tq_sv_pauli_expectation: NULL pointer");
  if (n_groups < 0 || n_terms < 0 || n_groups > 65535)
    return fail(TQ_ERR_ARG, "tq_sv_pauli_expectation: %d groups (max 65535)", n_groups);
  cudaStream_t s = STREAM(stream);
  if (n_groups == 0) {
    cudaMemsetAsync(out_dev, 0, sizeof(double), s);
    TQ_CHECK_LAUNCH("tq_sv_pauli_expectation");
    return TQ_OK;
  }
  if (!groups || !terms) return fail(TQ_ERR_ARG, "tq_sv_pauli_expectation: NULL table");
  const size_t need = tq_sv_pauli_expectation_workspace_bytes(n, n_groups);
  if (!ws || ws_bytes < need)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_pauli_expectation: workspace of %zu bytes < %zu", ws_bytes, need);
  const int nch = pauli_nchunk(n);
  dim3 grid(nch, n_groups);
  if (dtype == TQ_C64)
    k_pauli_expect<float><<<grid, 256, 0, s>>>((const float2*)psi, n, groups, terms, (double*)ws, nch);
  else
    k_pauli_expect<double><<<grid, 256, 0, s>>>((const double2*)psi, n, groups, terms, (double*)ws, nch);
  k_finalize<<<1, 1024, 0, s>>>((const double*)ws, nch * n_groups, 1, out_dev);
  TQ_CHECK_LAUNCH("tq_sv_pauli_expectation");
  return TQ_OK;
}

extern "C" int tq_sv_apply_pauli_sum(const void* psi, void* out, int n, int dtype, const tq_pauli_group* groups,
                                     int n_groups, const tq_pauli_term* terms, int n_terms, void* stream) {
  TQ_RANGE("tq_sv_apply_pauli_sum");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi || !out) return fail(TQ_ERR_ARG, "tq_sv_apply_pauli_sum: NULL pointer");
  if (psi == out) return fail(TQ_ERR_ARG, "tq_sv_apply_pauli_sum: out aliases psi");
  if (n_groups < 0 || n_terms < 0) return fail(TQ_ERR_ARG, "tq_sv_apply_pauli_sum: negative count");
  if (n_groups > 0 && (!groups || !terms)) return fail(TQ_ERR_ARG, "tq_sv_apply_pauli_sum: NULL table");
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_apply_pauli_sum<float><<<grid_for(N, 256), 256, 0, s>>>((const float2*)psi, (float2*)out, N, groups, n_groups,
                                                               terms);
  else
    k_apply_pauli_sum<double><<<grid_for(N, 256), 256, 0, s>>>((const double2*)psi, (double2*)out, N, groups,
                                                                n_groups, terms);
  TQ_CHECK_LAUNCH("tq_sv_apply_pauli_sum");
  return TQ_OK;
}

// Workspace layout for sampling: [prefix: nchunks+1][tgt: shots][bsum: nsb+1]
struct SampLayout {
  int64_t nchunks, nsb;
  size_t off_prefix, off_tgt, off_bsum, total;
};
static SampLayout samp_layout(int n, int64_t shots) {
  SampLayout L;
  const int64_t N = int64_t(1) << n;
  L.nchunks = (N + kSampCH - 1) / kSampCH;
  L.nsb = (shots + 1 + kSpacePerBlock - 1) / kSpacePerBlock;
  L.off_prefix = 0;
  L.off_tgt = align256(sizeof(double) * (L.nchunks + 1));
  L.off_bsum = L.off_tgt + align256(sizeof(double) * (shots > 0 ? shots : 1));
  L.total = L.off_bsum + align256(sizeof(double) * (L.nsb + 1));
  return L;
}

extern "C" size_t tq_sv_sample_workspace_bytes(int n, int64_t shots) {
  if (n < 0 || n > TQ_MAX_QUBITS || shots < 0) return 0;
  return samp_layout(n, shots).total;
}

extern "C" int tq_sv_sample(const void* psi, int n, int dtype, int64_t shots, uint64_t seed, int64_t* out_indices,
                            void* ws, size_t ws_bytes, void* stream) {
  TQ_RANGE("tq_sv_sample");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (shots < 0) return fail(TQ_ERR_ARG, "tq_sv_sample: negative shots");
  if (shots == 0) return TQ_OK;
  if (!psi || !out_indices) return fail(TQ_ERR_ARG, "tq_sv_sample: NULL pointer");
  const SampLayout L = samp_layout(n, shots);
  if (!ws || ws_bytes < L.total)
    return fail(TQ_ERR_WORKSPACE, "tq_sv_sample: workspace of %zu bytes < %zu", ws_bytes, L.total);
  if (L.nchunks > 0x7fffffffLL || L.nsb > 0x7fffffffLL) return fail(TQ_ERR_RANGE, "tq_sv_sample: too large");
  const int64_t N = int64_t(1) << n;
  char* w = (char*)ws;
  double* prefix = (double*)(w + L.off_prefix);
  double* tgt = (double*)(w + L.off_tgt);
  double* bsum = (double*)(w + L.off_bsum);
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_chunk_sums<float><<<(unsigned)L.nchunks, kSampThreads, 0, s>>>((const float2*)psi, N, prefix);
  else
    k_chunk_sums<double><<<(unsigned)L.nchunks, kSampThreads, 0, s>>>((const double2*)psi, N, prefix);
  k_scan_excl<<<1, 1024, 0, s>>>(prefix, L.nchunks);
  k_spacings<<<(unsigned)L.nsb, kSampThreads, 0, s>>>(tgt, shots, seed, bsum);
  k_scan_excl<<<1, 1024, 0, s>>>(bsum, L.nsb);
  k_targets<<<grid_for(shots, 256), 256, 0, s>>>(tgt, shots, bsum, L.nsb, prefix, L.nchunks);
  if (dtype == TQ_C64)
    k_resolve<float><<<(unsigned)L.nchunks, kSampThreads, 0, s>>>((const float2*)psi, N, prefix, L.nchunks, tgt,
                                                                   shots, out_indices);
  else
    k_resolve<double><<<(unsigned)L.nchunks, kSampThreads, 0, s>>>((const double2*)psi, N, prefix, L.nchunks, tgt,
                                                                    shots, out_indices);
  TQ_CHECK_LAUNCH("tq_sv_sample");
  return TQ_OK;
}

// ----------------------------------------------------------------- sampling without allocation
// Scratch for tq_sv_sample_noalloc: a fixed device array that lives as long as
// the library is loaded, one copy per GPU that uses it.  Host code cannot
// use the symbol itself as a device address, so the address is looked up
// once per device with cudaGetSymbolAddress and cached.
#define TQ_NOALLOC_SCRATCH_BYTES (size_t(8) << 20)
static __device__ __align__(256) unsigned char g_sample_scratch[TQ_NOALLOC_SCRATCH_BYTES];

#include <cuda.h>
#include <mutex>

namespace tq {
// The scratch array's device address, cached per device ordinal together with
// the CUDA context it was looked up in.  A device reset (or a primary context
// released and created again) reloads the module, so the address is looked up
// again whenever the current context differs from the cached one.
struct ScratchAddr {
  CUcontext ctx;
  void* ptr;
};
static std::mutex g_scratch_mu;
static ScratchAddr g_scratch_addr[64] = {};
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

static CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(f);
  }
  return fn;
}
}  // namespace tq

extern "C" int tq_sv_sample_noalloc(const void* psi, int n, int dtype, int64_t shots, uint64_t seed,
                                    int64_t* out_indices, void* stream) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (shots < 0) return fail(TQ_ERR_ARG, "tq_sv_sample_noalloc: negative shots");
  const size_t need = tq_sv_sample_workspace_bytes(n, shots);
  if (need > TQ_NOALLOC_SCRATCH_BYTES)
    return fail(TQ_ERR_RANGE,
                "tq_sv_sample_noalloc: n=%d with %lld shots needs %zu bytes of scratch, above the fixed %zu bytes; "
                "use tq_sv_sample with a caller-provided workspace",
                n, (long long)shots, need, (size_t)TQ_NOALLOC_SCRATCH_BYTES);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "tq_sv_sample_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(TQ_ERR_RANGE, "tq_sv_sample_noalloc: device ordinal %d", dev);
  // a thread whose context the runtime has not made current yet reads a null
  // context: the address is then looked up again (which also makes it current)
  CUcontext ctx = nullptr;
  if (CtxGetCurrentFn f = ctx_get_current()) {
    if (f(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    ScratchAddr& a = g_scratch_addr[dev];
    if (!a.ptr || !ctx || a.ctx != ctx) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_sample_scratch);
      if (e != cudaSuccess) return cuda_status(e, "tq_sv_sample_noalloc: cudaGetSymbolAddress");
      a.ptr = p;
      a.ctx = ctx;
    }
    scratch = a.ptr;
  }
  // Every scratch word the sampler reads is written earlier in the same call
  // (chunk sums, scans, spacings), so the previous call's contents need no clearing.
  return tq_sv_sample(psi, n, dtype, shots, seed, out_indices, scratch, TQ_NOALLOC_SCRATCH_BYTES, stream);
}
TQ_CHECK_UNIT(measure)
