// Shared device/host helpers for the tyxonq_gb300 statevector library.
//
// Basis convention (mirrors the reference engine): qubit q of an n-qubit
// register is bit (n-1-q) of the basis index, i.e. qubit 0 is the most
// significant bit (kernels/statevector.py:32,49; engine.py:454,1050-1057).
// Every kernel in this library works on *bit positions*; the C-ABI entry
// points translate qubit indices with tq_bit(n, q) exactly once.
#pragma once

#ifdef __CUDACC_RTC__
// Runtime-compiled kernels (tyxonq_gb300/csrc/jit.cu) see only device code:
// fixed-width integer types without the host headers.
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#endif

#include "tq_sv.h"

namespace tq {

// ----------------------------------------------------------------- complex
template <typename R> struct C2;
template <> struct C2<float>  { typedef float2  T; };
template <> struct C2<double> { typedef double2 T; };

template <typename R>
struct cplx {
  R x, y;
  __host__ __device__ cplx() {}
  __host__ __device__ cplx(R a, R b) : x(a), y(b) {}
};

template <typename R>
__device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return cplx<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc + a*b
template <typename R>
__device__ __forceinline__ cplx<R> cfma(cplx<R> a, cplx<R> b, cplx<R> acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// conj(a)*b
template <typename R>
__device__ __forceinline__ cplx<R> cconjmul(cplx<R> a, cplx<R> b) {
  return cplx<R>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Weight of a Pauli term in the working precision: complex64 kernels read the
// float copies, so no double -> float conversion (an FP64-pipe instruction)
// runs per term and thread.
template <typename R> struct TermW;
template <> struct TermW<float> {
  static __device__ __forceinline__ cplx<float> get(const tq_pauli_term* t) {
    return cplx<float>(__ldg(&t->f_re), __ldg(&t->f_im));
  }
};
template <> struct TermW<double> {
  static __device__ __forceinline__ cplx<double> get(const tq_pauli_term* t) {
    return cplx<double>(__ldg(&t->w_re), __ldg(&t->w_im));
  }
};
template <typename R>
__device__ __forceinline__ cplx<R> term_w(const tq_pauli_term* t) { return TermW<R>::get(t); }

// 2x2 and 4x4 complex matrices passed by value as kernel parameters.
template <typename R> struct Mat2 { cplx<R> m[4]; };
template <typename R> struct Mat4 { cplx<R> m[16]; };

// ----------------------------------------------------------------- bits
__host__ __device__ __forceinline__ int64_t insert_zero(int64_t i, int p) {
  const int64_t lo = i & ((int64_t(1) << p) - 1);
  return ((i >> p) << (p + 1)) | lo;
}
// Insert zeros at two positions plo < phi (positions in the *result*).
__host__ __device__ __forceinline__ int64_t insert_zero2(int64_t i, int plo, int phi) {
  return insert_zero(insert_zero(i, plo), phi);
}

// ----------------------------------------------------------------- checked builds
// With -DTQ_CHECKED (the library's checked variant) device-side index checks
// guard the accesses whose indices kernels compute: a failing check records
// the first failing site (TQ_SITE_*) and its index in this translation unit's
// status words and skips the access instead of trapping, and the host reads
// and clears them with tq_check_status.  Unchecked builds compile the checks
// away.  TQ_DCHECK(cond, site, index, action): action (continue, return, ...)
// runs after a failing check.
#if defined(TQ_CHECKED) && !defined(__CUDACC_RTC__)
static __device__ unsigned long long tq_check_word[2];
static __device__ __noinline__ void tq_check_fail(unsigned site, long long index) {
  if (atomicCAS(&tq_check_word[0], 0ull, (unsigned long long)site) == 0ull) tq_check_word[1] = (unsigned long long)index;
}
#define TQ_DCHECK(cond, site, index, action)                        \
  do {                                                              \
    if (!(cond)) {                                                  \
      ::tq::tq_check_fail((unsigned)(site), (long long)(index));    \
      action;                                                       \
    }                                                               \
  } while (0)
// Host reader of this translation unit's status words (name: the unit).
#define TQ_CHECK_UNIT(name)                                                                         \
  extern "C" int tq_check_read_##name(unsigned long long* out) {                                   \
    cudaError_t e = cudaMemcpyFromSymbol(out, ::tq::tq_check_word, sizeof(unsigned long long) * 2); \
    if (e != cudaSuccess) return (int)e;                                                            \
    const unsigned long long zero[2] = {0ull, 0ull};                                                \
    return (int)cudaMemcpyToSymbol(::tq::tq_check_word, zero, sizeof(zero));                        \
  }
#else
#define TQ_DCHECK(cond, site, index, action) \
  do {                                       \
  } while (0)
#define TQ_CHECK_UNIT(name)
#endif

#ifndef __CUDACC_RTC__
// ----------------------------------------------------------------- tracing
// One NVTX range per entry point (kernel class): header-only NVTX v3, a no-op
// unless a tool (nsys, ncu) is attached.
}  // namespace tq
#include <nvtx3/nvToolsExt.h>
namespace tq {
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define TQ_RANGE(name) ::tq::NvtxRange tq_nvtx_range_(name)

// ----------------------------------------------------------------- errors
// Host-side error reporting: each failing entry point records a message that
// tq_last_error() returns (thread-local, like errno).
// fail() records (code, message) and returns code.
int fail(int code, const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define TQ_CHECK_LAUNCH(where)                                   \
  do {                                                           \
    cudaError_t _e = cudaGetLastError();                         \
    if (_e != cudaSuccess) return ::tq::cuda_status(_e, where);  \
  } while (0)

inline int check_n(int n, int dtype) {
  if (n < 0 || n > TQ_MAX_QUBITS)
    return fail(TQ_ERR_ARG, "num_qubits %d outside [0, %d]", n, TQ_MAX_QUBITS);
  if (dtype != TQ_C64 && dtype != TQ_C128)
    return fail(TQ_ERR_ARG, "dtype tag %d is neither TQ_C64 nor TQ_C128", dtype);
  return TQ_OK;
}
inline int check_qubit(int n, int q) {
  if (q < 0 || q >= n)
    return fail(TQ_ERR_RANGE, "qubit index %d out of range for %d qubits", q, n);
  return TQ_OK;
}
inline int tq_bit(int n, int q) { return n - 1 - q; }

// Grid for an elementwise loop over `items` work items with `threads`
// threads per block (each thread handles one item; the grid is capped and
// kernels use a grid-stride loop beyond the cap).
inline unsigned grid_for(int64_t items, int threads) {
  int64_t b = (items + threads - 1) / threads;
  if (b < 1) b = 1;
  const int64_t cap = int64_t(152) * 64;  // 152 SMs x 64 resident blocks worth
  return (unsigned)(b < cap ? b : cap);
}

#endif  // __CUDACC_RTC__

}  // namespace tq
