// Single-gate kernels of the plain (one launch per gate) engine.
//
// Each kernel is one streaming pass over the amplitudes the gate can change,
// HBM-bound at the algorithmic bytes:
//   dense 1q              2*N*S      (every amplitude read + written once)
//   diag1 with d0 == 1    2*(N/2)*S
//   CX / SWAP             2*(N/2)*S
//   CZ                    2*(N/4)*S
//   dense 2q / kq         2*N*S
// (N = 2^n amplitudes, S = 8 B for complex64, 16 B for complex128).
// complex64 kernels move two neighbouring amplitudes per 128-bit access
// whenever the gate's lowest bit position is >= 1, so every warp access is a
// fully used 512 B segment.
#include <cmath>

#include "common.cuh"

namespace tq {

// ----------------------------------------------------------------- helpers
template <typename R>
__device__ __forceinline__ cplx<R> ld(const typename C2<R>::T* p, int64_t i) {
  typename C2<R>::T v = p[i];
  return cplx<R>(v.x, v.y);
}
template <typename R>
__device__ __forceinline__ void st(typename C2<R>::T* p, int64_t i, cplx<R> a) {
  typename C2<R>::T v;
  v.x = a.x;
  v.y = a.y;
  p[i] = v;
}
__device__ __forceinline__ void split4(float4 v, cplx<float>& a, cplx<float>& b) {
  a = cplx<float>(v.x, v.y);
  b = cplx<float>(v.z, v.w);
}
__device__ __forceinline__ float4 join4(cplx<float> a, cplx<float> b) {
  return make_float4(a.x, a.y, b.x, b.y);
}
template <typename R>
__device__ __forceinline__ void mv2(const Mat2<R>& u, cplx<R>& a0, cplx<R>& a1) {
  cplx<R> z(0, 0);
  cplx<R> o0 = cfma(u.m[1], a1, cmul(u.m[0], a0));
  cplx<R> o1 = cfma(u.m[3], a1, cmul(u.m[2], a0));
  (void)z;
  a0 = o0;
  a1 = o1;
}
template <typename R>
__device__ __forceinline__ void mv4(const Mat4<R>& u, cplx<R>& a0, cplx<R>& a1, cplx<R>& a2,
                                    cplx<R>& a3) {
  cplx<R> o[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    cplx<R> acc = cmul(u.m[4 * r + 0], a0);
    acc = cfma(u.m[4 * r + 1], a1, acc);
    acc = cfma(u.m[4 * r + 2], a2, acc);
    acc = cfma(u.m[4 * r + 3], a3, acc);
    o[r] = acc;
  }
  a0 = o[0];
  a1 = o[1];
  a2 = o[2];
  a3 = o[3];
}

#define GRID_STRIDE(v, count) \
  for (int64_t v = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; v < (count); v += int64_t(gridDim.x) * blockDim.x)

// ----------------------------------------------------------------- init
template <typename R>
__global__ void k_init_basis(typename C2<R>::T* psi, int64_t N, int64_t basis) {
  GRID_STRIDE(i, N) {
    typename C2<R>::T v;
    v.x = (i == basis) ? R(1) : R(0);
    v.y = R(0);
    psi[i] = v;
  }
}

// ----------------------------------------------------------------- dense 1q
// complex64, bit p >= 1: item v covers the pairs of amplitudes (2v, 2v+1 after
// inserting a zero at p) -> two float4 loads, two float4 stores.
__global__ void k_1q_c64_vec(float4* psi4, int64_t items, int p, Mat2<float> u) {
  GRID_STRIDE(v, items) {
    const int64_t i0 = insert_zero(2 * v, p);
    const int64_t i1 = i0 | (int64_t(1) << p);
    TQ_DCHECK((i1 >> 1) < 2 * items, TQ_SITE_GATE, i1, continue);
    float4 A = psi4[i0 >> 1], B = psi4[i1 >> 1];
    cplx<float> a0, a1, b0, b1;
    split4(A, a0, a1);
    split4(B, b0, b1);
    mv2(u, a0, b0);
    mv2(u, a1, b1);
    psi4[i0 >> 1] = join4(a0, a1);
    psi4[i1 >> 1] = join4(b0, b1);
  }
}
// complex64, bit 0: one float4 holds both amplitudes of a pair.
__global__ void k_1q_c64_p0(float4* psi4, int64_t items, Mat2<float> u) {
  GRID_STRIDE(v, items) {
    cplx<float> a0, a1;
    split4(psi4[v], a0, a1);
    mv2(u, a0, a1);
    psi4[v] = join4(a0, a1);
  }
}
template <typename R>
__global__ void k_1q_scalar(typename C2<R>::T* psi, int64_t items, int p, Mat2<R> u) {
  GRID_STRIDE(v, items) {
    const int64_t i0 = insert_zero(v, p);
    const int64_t i1 = i0 | (int64_t(1) << p);
    TQ_DCHECK(i1 < 2 * items, TQ_SITE_GATE, i1, continue);
    cplx<R> a0 = ld<R>(psi, i0), a1 = ld<R>(psi, i1);
    mv2(u, a0, a1);
    st<R>(psi, i0, a0);
    st<R>(psi, i1, a1);
  }
}

// ----------------------------------------------------------------- diagonal 1q
// Only the |1> half when d0 == 1 (phase-type gates).
__global__ void k_diag_hi_c64_vec(float4* psi4, int64_t items, int p, cplx<float> d1) {
  GRID_STRIDE(v, items) {
    const int64_t i1 = insert_zero(2 * v, p) | (int64_t(1) << p);
    TQ_DCHECK((i1 >> 1) < 2 * items, TQ_SITE_GATE, i1, continue);
    cplx<float> a, b;
    split4(psi4[i1 >> 1], a, b);
    psi4[i1 >> 1] = join4(cmul(d1, a), cmul(d1, b));
  }
}
template <typename R>
__global__ void k_diag_hi_scalar(typename C2<R>::T* psi, int64_t items, int p, cplx<R> d1) {
  GRID_STRIDE(v, items) {
    const int64_t i1 = insert_zero(v, p) | (int64_t(1) << p);
    TQ_DCHECK(i1 < 2 * items, TQ_SITE_GATE, i1, continue);
    st<R>(psi, i1, cmul(d1, ld<R>(psi, i1)));
  }
}
__global__ void k_diag_c64_vec(float4* psi4, int64_t items, int p, cplx<float> d0, cplx<float> d1) {
  GRID_STRIDE(v, items) {
    cplx<float> a, b;
    split4(psi4[v], a, b);
    const int64_t i = 2 * v;
    a = cmul(((i >> p) & 1) ? d1 : d0, a);
    b = cmul((((i + 1) >> p) & 1) ? d1 : d0, b);
    psi4[v] = join4(a, b);
  }
}
template <typename R>
__global__ void k_diag_scalar(typename C2<R>::T* psi, int64_t N, int p, cplx<R> d0, cplx<R> d1) {
  GRID_STRIDE(i, N) { st<R>(psi, i, cmul(((i >> p) & 1) ? d1 : d0, ld<R>(psi, i))); }
}

// ----------------------------------------------------------------- dense 2q
// pa = bit of the matrix-high qubit, pb = bit of the matrix-low qubit.
__global__ void k_2q_c64_vec(float4* psi4, int64_t items, int pa, int pb, int plo, int phi,
                             Mat4<float> u) {
  GRID_STRIDE(v, items) {
    const int64_t b = insert_zero2(2 * v, plo, phi);
    const int64_t ia = int64_t(1) << pa, ib = int64_t(1) << pb;
    const int64_t idx[4] = {b, b | ib, b | ia, b | ia | ib};
    TQ_DCHECK((idx[3] >> 1) < 4 * items, TQ_SITE_GATE, idx[3], continue);
    cplx<float> x[4], y[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) split4(psi4[idx[r] >> 1], x[r], y[r]);
    mv4(u, x[0], x[1], x[2], x[3]);
    mv4(u, y[0], y[1], y[2], y[3]);
#pragma unroll
    for (int r = 0; r < 4; ++r) psi4[idx[r] >> 1] = join4(x[r], y[r]);
  }
}
template <typename R>
__global__ void k_2q_scalar(typename C2<R>::T* psi, int64_t items, int pa, int pb, int plo, int phi,
                            Mat4<R> u) {
  GRID_STRIDE(v, items) {
    const int64_t b = insert_zero2(v, plo, phi);
    const int64_t ia = int64_t(1) << pa, ib = int64_t(1) << pb;
    TQ_DCHECK((b | ia | ib) < 4 * items, TQ_SITE_GATE, b | ia | ib, continue);
    cplx<R> a0 = ld<R>(psi, b), a1 = ld<R>(psi, b | ib), a2 = ld<R>(psi, b | ia),
            a3 = ld<R>(psi, b | ia | ib);
    mv4(u, a0, a1, a2, a3);
    st<R>(psi, b, a0);
    st<R>(psi, b | ib, a1);
    st<R>(psi, b | ia, a2);
    st<R>(psi, b | ia | ib, a3);
  }
}

// ----------------------------------------------------------------- permutation / sign 2q
// mode 0 = CX (swap |c=1,t=0> <-> |c=1,t=1>), 1 = SWAP (|01> <-> |10>),
// 2 = CZ (negate |11>).  pa = control / first qubit bit, pb = target / second.
template <int MODE>
__global__ void k_perm2_c64_vec(float4* psi4, int64_t items, int pa, int pb, int plo, int phi) {
  GRID_STRIDE(v, items) {
    const int64_t b = insert_zero2(2 * v, plo, phi);
    const int64_t ia = int64_t(1) << pa, ib = int64_t(1) << pb;
    TQ_DCHECK(((b | ia | ib) >> 1) < 4 * items, TQ_SITE_GATE, b | ia | ib, continue);
    if (MODE == 0) {
      float4 x = psi4[(b | ia) >> 1], y = psi4[(b | ia | ib) >> 1];
      psi4[(b | ia) >> 1] = y;
      psi4[(b | ia | ib) >> 1] = x;
    } else if (MODE == 1) {
      float4 x = psi4[(b | ia) >> 1], y = psi4[(b | ib) >> 1];
      psi4[(b | ia) >> 1] = y;
      psi4[(b | ib) >> 1] = x;
    } else {
      float4 x = psi4[(b | ia | ib) >> 1];
      psi4[(b | ia | ib) >> 1] = make_float4(-x.x, -x.y, -x.z, -x.w);
    }
  }
}
template <int MODE, typename R>
__global__ void k_perm2_scalar(typename C2<R>::T* psi, int64_t items, int pa, int pb, int plo,
                               int phi) {
  GRID_STRIDE(v, items) {
    const int64_t b = insert_zero2(v, plo, phi);
    const int64_t ia = int64_t(1) << pa, ib = int64_t(1) << pb;
    TQ_DCHECK((b | ia | ib) < 4 * items, TQ_SITE_GATE, b | ia | ib, continue);
    if (MODE == 0) {
      typename C2<R>::T x = psi[b | ia], y = psi[b | ia | ib];
      psi[b | ia] = y;
      psi[b | ia | ib] = x;
    } else if (MODE == 1) {
      typename C2<R>::T x = psi[b | ia], y = psi[b | ib];
      psi[b | ia] = y;
      psi[b | ib] = x;
    } else {
      typename C2<R>::T x = psi[b | ia | ib];
      x.x = -x.x;
      x.y = -x.y;
      psi[b | ia | ib] = x;
    }
  }
}

// ----------------------------------------------------------------- dense k-qubit
template <typename R, int K>
struct KqParams {
  int sp[K];           // target bit positions, ascending (for zero insertion)
  int64_t offs[1 << K];  // offset of matrix index j (MSB = first listed qubit)
  cplx<R> u[(1 << K) * (1 << K)];
};

__device__ __forceinline__ void ld_pair(const cplx<float>* p, cplx<float>& a, cplx<float>& b) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = cplx<float>(v.x, v.y);
  b = cplx<float>(v.z, v.w);
}
__device__ __forceinline__ void ld_pair(const cplx<double>* p, cplx<double>& a, cplx<double>& b) {
  a = p[0];
  b = p[1];
}

// The matrix is copied once per CTA into shared memory and read two entries per
// 16-byte load (the same address in every lane: a broadcast); two accumulators
// per output row halve the dependent FMA chain.  Rows are not unrolled (all 32
// rows at once would need 32 accumulators next to the 32 inputs).
template <typename R, int K>
__global__ void k_kq(typename C2<R>::T* psi, int64_t items, const __grid_constant__ KqParams<R, K> P) {
  constexpr int D = 1 << K;
  constexpr bool SMEM = K >= 4;  // up to 8x8 the constant-bank operands measured faster
  __shared__ __align__(16) cplx<R> su[SMEM ? D * D : 2];
  if constexpr (SMEM) {
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) su[e] = P.u[e];
    __syncthreads();
  }
  GRID_STRIDE(v, items) {
    int64_t b = v;
#pragma unroll
    for (int r = 0; r < K; ++r) b = insert_zero(b, P.sp[r]);
    TQ_DCHECK((b | P.offs[D - 1]) < (items << K), TQ_SITE_GATE, b | P.offs[D - 1], continue);
    cplx<R> x[D];
#pragma unroll
    for (int j = 0; j < D; ++j) x[j] = ld<R>(psi, b + P.offs[j]);
    if constexpr (!SMEM) {
#pragma unroll 1
      for (int r = 0; r < D; ++r) {
        cplx<R> acc(0, 0);
#pragma unroll
        for (int c = 0; c < D; ++c) acc = cfma(P.u[r * D + c], x[c], acc);
        st<R>(psi, b + P.offs[r], acc);
      }
      continue;
    }
#pragma unroll 1
    for (int r = 0; r < D; ++r) {
      const cplx<R>* row = su + r * D;
      cplx<R> a0(0, 0), a1(0, 0);
#pragma unroll
      for (int c = 0; c < D; c += 2) {
        cplx<R> m0, m1;
        ld_pair(row + c, m0, m1);
        a0 = cfma(m0, x[c], a0);
        a1 = cfma(m1, x[c + 1], a1);
      }
      st<R>(psi, b + P.offs[r], cplx<R>(a0.x + a1.x, a0.y + a1.y));
    }
  }
}

// ----------------------------------------------------------------- Pauli rotation
// psi <- cos(t/2) psi - i sin(t/2) P psi with P|i> = ph (-1)^{popc(i&zy)} |i^m>.
template <typename R>
__global__ void k_pauli_rot(typename C2<R>::T* psi, int64_t items, uint64_t m, uint64_t zy, int h,
                            cplx<R> ph, R c, R s) {
  // -i*s*ph
  const cplx<R> w(s * ph.y, -s * ph.x);
  GRID_STRIDE(v, items) {
    if (m == 0) {
      const int64_t i = v;
      const R sg = (__popcll((unsigned long long)i & zy) & 1) ? R(-1) : R(1);
      cplx<R> a = ld<R>(psi, i);
      // (c + w*sg) * a
      st<R>(psi, i, cmul(cplx<R>(c + sg * w.x, sg * w.y), a));
    } else {
      const int64_t i = insert_zero(v, h);
      const int64_t j = i ^ (int64_t)m;
      TQ_DCHECK(i < 2 * items && j < 2 * items, TQ_SITE_GATE, i > j ? i : j, continue);
      cplx<R> a = ld<R>(psi, i), b = ld<R>(psi, j);
      const R si = (__popcll((unsigned long long)i & zy) & 1) ? R(-1) : R(1);
      const R sj = (__popcll((unsigned long long)j & zy) & 1) ? R(-1) : R(1);
      cplx<R> na(c * a.x, c * a.y), nb(c * b.x, c * b.y);
      // P psi at i = ph * sj * psi_j ; at j = ph * si * psi_i
      na = cfma(cplx<R>(w.x * sj, w.y * sj), b, na);
      nb = cfma(cplx<R>(w.x * si, w.y * si), a, nb);
      st<R>(psi, i, na);
      st<R>(psi, j, nb);
    }
  }
}

template <typename R>
__global__ void k_scale(typename C2<R>::T* psi, int64_t N, cplx<R> f) {
  GRID_STRIDE(i, N) { st<R>(psi, i, cmul(f, ld<R>(psi, i))); }
}

static const int kThreads = 256;

template <typename R>
static Mat2<R> mat2_from(const double* u) {
  Mat2<R> m;
  for (int i = 0; i < 4; ++i) m.m[i] = cplx<R>((R)u[2 * i], (R)u[2 * i + 1]);
  return m;
}
template <typename R>
static Mat4<R> mat4_from(const double* u) {
  Mat4<R> m;
  for (int i = 0; i < 16; ++i) m.m[i] = cplx<R>((R)u[2 * i], (R)u[2 * i + 1]);
  return m;
}

template <typename R, int K>
static void launch_kq(void* psi, int n, const int* pos, const double* u, cudaStream_t s) {
  KqParams<R, K> P;
  int sp[K];
  for (int r = 0; r < K; ++r) sp[r] = pos[r];
  for (int a = 0; a < K; ++a)
    for (int b = a + 1; b < K; ++b)
      if (sp[b] < sp[a]) {
        int t = sp[a];
        sp[a] = sp[b];
        sp[b] = t;
      }
  for (int r = 0; r < K; ++r) P.sp[r] = sp[r];
  const int D = 1 << K;
  for (int j = 0; j < D; ++j) {
    int64_t o = 0;
    for (int r = 0; r < K; ++r)
      if ((j >> (K - 1 - r)) & 1) o |= int64_t(1) << pos[r];
    P.offs[j] = o;
  }
  for (int e = 0; e < D * D; ++e) P.u[e] = cplx<R>((R)u[2 * e], (R)u[2 * e + 1]);
  const int64_t items = (int64_t(1) << n) >> K;
  const int threads = (sizeof(R) == 8 && K >= 4) ? 64 : 128;
  // persistent-sized grid where every CTA copies the matrix once
  unsigned grid = grid_for(items, threads);
  if (K >= 4 && grid > 152u * 16u) grid = 152u * 16u;
  k_kq<R, K><<<grid, threads, 0, s>>>((typename C2<R>::T*)psi, items, P);
}

}  // namespace tq

using namespace tq;

#define STREAM(s) ((cudaStream_t)(s))

extern "C" int tq_sv_init_basis(void* psi, int n, int dtype, int64_t basis, void* stream) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  const int64_t N = int64_t(1) << n;
  if (basis < 0 || basis >= N) return fail(TQ_ERR_RANGE, "basis index %lld out of range", (long long)basis);
  if (!psi) return fail(TQ_ERR_ARG, "psi is NULL");
  if (dtype == TQ_C64)
    k_init_basis<float><<<grid_for(N, kThreads), kThreads, 0, STREAM(stream)>>>((float2*)psi, N, basis);
  else
    k_init_basis<double><<<grid_for(N, kThreads), kThreads, 0, STREAM(stream)>>>((double2*)psi, N, basis);
  TQ_CHECK_LAUNCH("tq_sv_init_basis");
  return TQ_OK;
}

extern "C" int tq_sv_apply_1q(void* psi, int n, int dtype, int qubit, const double* u, void* stream) {
  TQ_RANGE("tq_sv_apply_1q");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if ((rc = check_qubit(n, qubit))) return rc;
  if (!psi || !u) return fail(TQ_ERR_ARG, "NULL pointer");
  const int p = tq_bit(n, qubit);
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64) {
    Mat2<float> m = mat2_from<float>(u);
    if (p == 0)
      k_1q_c64_p0<<<grid_for(N / 2, kThreads), kThreads, 0, s>>>((float4*)psi, N / 2, m);
    else
      k_1q_c64_vec<<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((float4*)psi, N / 4, p, m);
  } else {
    k_1q_scalar<double><<<grid_for(N / 2, kThreads), kThreads, 0, s>>>((double2*)psi, N / 2, p,
                                                                         mat2_from<double>(u));
  }
  TQ_CHECK_LAUNCH("tq_sv_apply_1q");
  return TQ_OK;
}

extern "C" int tq_sv_apply_diag1(void* psi, int n, int dtype, int qubit, const double* d, void* stream) {
  TQ_RANGE("tq_sv_apply_diag1");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if ((rc = check_qubit(n, qubit))) return rc;
  if (!psi || !d) return fail(TQ_ERR_ARG, "NULL pointer");
  const int p = tq_bit(n, qubit);
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  const bool hi_only = (d[0] == 1.0 && d[1] == 0.0);
  if (dtype == TQ_C64) {
    cplx<float> d0((float)d[0], (float)d[1]), d1((float)d[2], (float)d[3]);
    if (hi_only && p >= 1)
      k_diag_hi_c64_vec<<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((float4*)psi, N / 4, p, d1);
    else
      k_diag_c64_vec<<<grid_for(N / 2, kThreads), kThreads, 0, s>>>((float4*)psi, N / 2, p, d0, d1);
  } else {
    cplx<double> d0(d[0], d[1]), d1(d[2], d[3]);
    if (hi_only)
      k_diag_hi_scalar<double><<<grid_for(N / 2, kThreads), kThreads, 0, s>>>((double2*)psi, N / 2, p, d1);
    else
      k_diag_scalar<double><<<grid_for(N, kThreads), kThreads, 0, s>>>((double2*)psi, N, p, d0, d1);
  }
  TQ_CHECK_LAUNCH("tq_sv_apply_diag1");
  return TQ_OK;
}

extern "C" int tq_sv_apply_2q(void* psi, int n, int dtype, int q0, int q1, const double* u, void* stream) {
  TQ_RANGE("tq_sv_apply_2q");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if ((rc = check_qubit(n, q0)) || (rc = check_qubit(n, q1))) return rc;
  if (!psi || !u) return fail(TQ_ERR_ARG, "NULL pointer");
  if (q0 == q1) return TQ_OK;  // statevector.py:46-47
  const int pa = tq_bit(n, q0), pb = tq_bit(n, q1);
  const int plo = pa < pb ? pa : pb, phi = pa < pb ? pb : pa;
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64) {
    Mat4<float> m = mat4_from<float>(u);
    if (plo >= 1)
      k_2q_c64_vec<<<grid_for(N / 8, kThreads), kThreads, 0, s>>>((float4*)psi, N / 8, pa, pb, plo, phi, m);
    else
      k_2q_scalar<float><<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((float2*)psi, N / 4, pa, pb, plo, phi, m);
  } else {
    k_2q_scalar<double><<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((double2*)psi, N / 4, pa, pb, plo, phi,
                                                                         mat4_from<double>(u));
  }
  TQ_CHECK_LAUNCH("tq_sv_apply_2q");
  return TQ_OK;
}

template <int MODE>
static int perm2(void* psi, int n, int dtype, int q0, int q1, void* stream, const char* name) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if ((rc = check_qubit(n, q0)) || (rc = check_qubit(n, q1))) return rc;
  if (!psi) return fail(TQ_ERR_ARG, "psi is NULL");
  if (q0 == q1) return TQ_OK;
  const int pa = tq_bit(n, q0), pb = tq_bit(n, q1);
  const int plo = pa < pb ? pa : pb, phi = pa < pb ? pb : pa;
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64) {
    if (plo >= 1)
      k_perm2_c64_vec<MODE><<<grid_for(N / 8, kThreads), kThreads, 0, s>>>((float4*)psi, N / 8, pa, pb, plo, phi);
    else
      k_perm2_scalar<MODE, float><<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((float2*)psi, N / 4, pa, pb, plo,
                                                                                   phi);
  } else {
    k_perm2_scalar<MODE, double><<<grid_for(N / 4, kThreads), kThreads, 0, s>>>((double2*)psi, N / 4, pa, pb, plo,
                                                                                  phi);
  }
  TQ_CHECK_LAUNCH(name);
  return TQ_OK;
}

extern "C" int tq_sv_apply_cx(void* psi, int n, int dtype, int control, int target, void* stream) {
  TQ_RANGE("tq_sv_apply_cx");
  return perm2<0>(psi, n, dtype, control, target, stream, "tq_sv_apply_cx");
}
extern "C" int tq_sv_apply_swap(void* psi, int n, int dtype, int q0, int q1, void* stream) {
  TQ_RANGE("tq_sv_apply_swap");
  return perm2<1>(psi, n, dtype, q0, q1, stream, "tq_sv_apply_swap");
}
extern "C" int tq_sv_apply_cz(void* psi, int n, int dtype, int q0, int q1, void* stream) {
  TQ_RANGE("tq_sv_apply_cz");
  return perm2<2>(psi, n, dtype, q0, q1, stream, "tq_sv_apply_cz");
}

extern "C" int tq_sv_apply_kq(void* psi, int n, int dtype, const int* qubits, int k, const double* u,
                              void* stream) {
  TQ_RANGE("tq_sv_apply_kq");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi || !qubits || !u) return fail(TQ_ERR_ARG, "NULL pointer");
  if (k < 1 || k > TQ_MAX_KQ || k > n) return fail(TQ_ERR_ARG, "k=%d outside [1, min(%d, n)]", k, TQ_MAX_KQ);
  int pos[TQ_MAX_KQ];
  for (int r = 0; r < k; ++r) {
    if ((rc = check_qubit(n, qubits[r]))) return rc;
    for (int t = 0; t < r; ++t)
      if (qubits[t] == qubits[r]) return fail(TQ_ERR_ARG, "repeated qubit %d in k-qubit unitary", qubits[r]);
    pos[r] = tq_bit(n, qubits[r]);
  }
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64) {
    switch (k) {
      case 1: launch_kq<float, 1>(psi, n, pos, u, s); break;
      case 2: launch_kq<float, 2>(psi, n, pos, u, s); break;
      case 3: launch_kq<float, 3>(psi, n, pos, u, s); break;
      case 4: launch_kq<float, 4>(psi, n, pos, u, s); break;
      default: launch_kq<float, 5>(psi, n, pos, u, s); break;
    }
  } else {
    switch (k) {
      case 1: launch_kq<double, 1>(psi, n, pos, u, s); break;
      case 2: launch_kq<double, 2>(psi, n, pos, u, s); break;
      case 3: launch_kq<double, 3>(psi, n, pos, u, s); break;
      case 4: launch_kq<double, 4>(psi, n, pos, u, s); break;
      default: launch_kq<double, 5>(psi, n, pos, u, s); break;
    }
  }
  TQ_CHECK_LAUNCH("tq_sv_apply_kq");
  return TQ_OK;
}

extern "C" int tq_sv_apply_pauli_rotation(void* psi, int n, int dtype, uint64_t x_mask, uint64_t z_mask,
                                          double theta, void* stream) {
  TQ_RANGE("tq_sv_apply_pauli_rotation");
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi) return fail(TQ_ERR_ARG, "psi is NULL");
  const uint64_t full = (n >= 64) ? ~0ull : ((1ull << n) - 1);
  if ((x_mask & ~full) || (z_mask & ~full)) return fail(TQ_ERR_RANGE, "Pauli mask has bits above n=%d", n);
  const int64_t N = int64_t(1) << n;
  const int ny = __builtin_popcountll(x_mask & z_mask);
  // i^ny
  const double phr[4] = {1, 0, -1, 0}, phi_[4] = {0, 1, 0, -1};
  const double c = cos(0.5 * theta), sn = sin(0.5 * theta);
  int h = 0;
  if (x_mask) h = 63 - __builtin_clzll(x_mask);
  const int64_t items = x_mask ? N / 2 : N;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_pauli_rot<float><<<grid_for(items, kThreads), kThreads, 0, s>>>(
        (float2*)psi, items, x_mask, z_mask, h, cplx<float>((float)phr[ny & 3], (float)phi_[ny & 3]), (float)c,
        (float)sn);
  else
    k_pauli_rot<double><<<grid_for(items, kThreads), kThreads, 0, s>>>(
        (double2*)psi, items, x_mask, z_mask, h, cplx<double>(phr[ny & 3], phi_[ny & 3]), c, sn);
  TQ_CHECK_LAUNCH("tq_sv_apply_pauli_rotation");
  return TQ_OK;
}

extern "C" int tq_sv_scale(void* psi, int n, int dtype, double re, double im, void* stream) {
  int rc = check_n(n, dtype);
  if (rc) return rc;
  if (!psi) return fail(TQ_ERR_ARG, "psi is NULL");
  const int64_t N = int64_t(1) << n;
  cudaStream_t s = STREAM(stream);
  if (dtype == TQ_C64)
    k_scale<float><<<grid_for(N, kThreads), kThreads, 0, s>>>((float2*)psi, N, cplx<float>((float)re, (float)im));
  else
    k_scale<double><<<grid_for(N, kThreads), kThreads, 0, s>>>((double2*)psi, N, cplx<double>(re, im));
  TQ_CHECK_LAUNCH("tq_sv_scale");
  return TQ_OK;
}
TQ_CHECK_UNIT(gates)
