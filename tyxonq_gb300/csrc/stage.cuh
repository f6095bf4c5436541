// Register-staged application of tile ops.
//
// A stage names 4 local bit positions (its "register bits").  Thread tid of
// a 2^(t-4)-thread CTA holds the 16 amplitudes whose other local bits spell
// tid; every op of the stage acts on register bits only, so it is applied to
// those 16 registers without touching shared memory.  Shared memory is read
// and written once per stage instead of once per op.
//
// Before a stage runs, its ops are compiled (one thread per op) into compact
// shared-memory records (ROp): angles are turned into coefficients, the
// adjoint is folded in, and the op's shape picks a specialised routine --
// a real or imaginary single-bit rotation costs 8 FMAs per amplitude pair
// instead of a dense complex 2x2.  Register-bit indices are runtime values;
// each routine is instantiated for every bit (combination) and the record's
// code selects one, so the register array is only ever indexed by constants.
//
// Shared-memory tiles are padded by 2 amplitudes per 16 (phys = j + 2*(j>>4)):
// the pad keeps 16-byte chunks aligned for cp.async and spreads the
// stride-16 access pattern of low register bits over the banks.
#pragma once

#include "tile.cuh"

namespace tq {

constexpr int kRB = 4;            // register bits per stage
constexpr int kNR = 1 << kRB;     // amplitudes per thread
constexpr int kRopCap = 64;       // compiled ops held in shared memory at once

__device__ __forceinline__ int pphys(int j) { return j + ((j >> 4) << 1); }
__host__ __device__ __forceinline__ int padded_len(int t) { return (1 << t) + ((1 << t) >> 3); }

// ------------------------------------------------------------------ register routines
template <typename R, int NR, int K>
__device__ __forceinline__ void r_u1(cplx<R>* x, cplx<R> u0, cplx<R> u1, cplx<R> u2, cplx<R> u3) {
  if constexpr (!((1 << K) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    const cplx<R> a = x[i], b = x[j];
    x[i] = cfma(u1, b, cmul(u0, a));
    x[j] = cfma(u3, b, cmul(u2, a));
  }
  }
}

// [[c, a01], [a10, c]] with real entries
template <typename R, int NR, int K>
__device__ __forceinline__ void r_rr(cplx<R>* x, R c, R a01, R a10) {
  if constexpr (!((1 << K) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    const cplx<R> u = x[i], v = x[j];
    x[i] = cplx<R>(fma(a01, v.x, c * u.x), fma(a01, v.y, c * u.y));
    x[j] = cplx<R>(fma(a10, u.x, c * v.x), fma(a10, u.y, c * v.y));
  }
  }
}

// [[c, i b01], [i b10, c]] with c, b01, b10 real
template <typename R, int NR, int K>
__device__ __forceinline__ void r_ri(cplx<R>* x, R c, R b01, R b10) {
  if constexpr (!((1 << K) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    const cplx<R> u = x[i], v = x[j];
    x[i] = cplx<R>(fma(-b01, v.y, c * u.x), fma(b01, v.x, c * u.y));
    x[j] = cplx<R>(fma(-b10, u.y, c * v.x), fma(b10, u.x, c * v.y));
  }
  }
}

template <typename R, int NR, int K>
__device__ __forceinline__ void r_d1(cplx<R>* x, cplx<R> d0, cplx<R> d1) {
  if constexpr (!((1 << K) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i) x[i] = cmul(((i >> K) & 1) ? d1 : d0, x[i]);
  }
}

template <typename R, int NR, int K>
__device__ __forceinline__ void r_dh(cplx<R>* x, cplx<R> d1) {
  if constexpr (!((1 << K) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i)
    if ((i >> K) & 1) x[i] = cmul(d1, x[i]);
  }
}

// MODE 0 CX (control A, target B), 1 SWAP, 2 CZ
template <typename R, int NR, int MODE, int A, int B>
__device__ __forceinline__ void r_perm(cplx<R>* x) {
  if constexpr (!((1 << A) < NR && (1 << B) < NR)) {
    return;
  } else {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
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
}

// G flips bit K, Z factors only on K (sign w1 on the bit-K-set half):
// Im(ph (sum conj(y_j) x_i + w1 sum conj(y_i) x_j)), i = j ^ (1 << K), bit K of i clear.
template <typename R, int NR, int K>
__device__ __forceinline__ R g_pair(const cplx<R>* x, const cplx<R>* y, cplx<R> ph, R w1) {
  if constexpr (!((1 << K) < NR)) {
    return R(0);
  } else {
  R ax = 0, ay = 0, bx = 0, by = 0;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    ax = fma(y[j].x, x[i].x, fma(y[j].y, x[i].y, ax));
    ay = fma(y[j].x, x[i].y, fma(-y[j].y, x[i].x, ay));
    bx = fma(y[i].x, x[j].x, fma(y[i].y, x[j].y, bx));
    by = fma(y[i].x, x[j].y, fma(-y[i].y, x[j].x, by));
  }
  const R zx = fma(w1, bx, ax), zy = fma(w1, by, ay);
  return ph.x * zy + ph.y * zx;
  }
}

// Diagonal G: weight w0 where bit K is clear, w1 where it is set.
template <typename R, int NR, int K>
__device__ __forceinline__ R g_diag(const cplx<R>* x, const cplx<R>* y, cplx<R> ph, R w0, R w1) {
  if constexpr (!((1 << K) < NR)) {
    return R(0);
  } else {
  R s0x = 0, s0y = 0, s1x = 0, s1y = 0;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    if ((i >> K) & 1) {
      s1x = fma(y[i].x, x[i].x, fma(y[i].y, x[i].y, s1x));
      s1y = fma(y[i].x, x[i].y, fma(-y[i].y, x[i].x, s1y));
    } else {
      s0x = fma(y[i].x, x[i].x, fma(y[i].y, x[i].y, s0x));
      s0y = fma(y[i].x, x[i].y, fma(-y[i].y, x[i].x, s0y));
    }
  }
  const R zx = fma(w1, s1x, w0 * s0x), zy = fma(w1, s1y, w0 * s0y);
  return ph.x * zy + ph.y * zx;
  }
}

// ------------------------------------------------------------------ compiled ops
enum RCode : int32_t {
  RC_NOP = 0,
  RC_U1 = 1,     // + K: dense 2x2 m0..m3; the per-thread sign scales m1, m2
  RC_RR = 5,     // + K: [[c, a01], [a10, c]] real: m0.x, m1.x, m2.x
  RC_RI = 9,     // + K: [[c, i b01], [i b10, c]]: m0.x, m1.y, m2.y
  RC_D = 13,     // + K: diag(m0, m1); a negative sign swaps the two
  RC_DH = 17,    // + K: diag(1, m1)
  RC_CX = 21,    // + pair index 4 a + b (a != b)
  RC_SWAP = 37,
  RC_CZ = 53,
  RC_U2 = 69,    // dense 4x4 read from the op table
  RC_PROT = 70,  // general Pauli rotation: c = m0, w = m1, masks from the op table
};
enum RGCode : int32_t { RG_NONE = -1, RG_GEN = 0, RG_PAIR = 1, RG_DIAG = 5 };

template <typename R>
struct __align__(16) ROp {
  int32_t code;   // RCode (+ register bit or pair index)
  int32_t gcode;  // RGCode (+ register bit); RG_NONE: no gradient slot
  int32_t op;     // index of the source op in the op table
  uint32_t zo;    // local bits outside the stage whose parity signs the op
  uint64_t zg;    // global bits outside the tile whose parity signs the op
  int32_t skip;   // 1 + ops folded into this one (the next op to run is op + skip)
  int32_t pad;
  cplx<R> m[4];
  cplx<R> gph;    // i^ny of the generator
  R gw0, gw1;
};

// ordered pair (a, b), a != b, of register bits -> 4 a + b
__device__ __forceinline__ int pair_index(int a, int b) { return 4 * a + b; }

__device__ __forceinline__ bool one_bit(uint32_t m) { return m != 0 && (m & (m - 1)) == 0; }

// Forward 2x2 matrix u (row-major) and register bit K of an op that acts on
// one register bit with no sign from outside the stage; false otherwise.
template <typename R>
__device__ __forceinline__ bool op_mat2(const tq_tile_op& o, const double* theta, cplx<R>* u, int& K) {
  if (o.zo != 0u || o.zg != 0ull) return false;
  const cplx<R> z(R(0), R(0));
  switch (o.kind) {
    case TOP_U1:
      K = o.a & 3;
      for (int e = 0; e < 4; ++e) u[e] = op_m<R>(o, e);
      return true;
    case TOP_D1: {
      K = o.a & 3;
      cplx<R> d0 = op_m<R>(o, 0), d1 = op_m<R>(o, 1);
      if (o.pidx >= 0 && theta != nullptr) {
        R c, sn;
        rot_cs(2.0 * o.pscale * theta[o.pidx], c, sn);
        d0 = cplx<R>(R(1), R(0));
        d1 = cplx<R>(c, sn);
      }
      u[0] = d0;
      u[1] = u[2] = z;
      u[3] = d1;
      return true;
    }
    case TOP_PROT: {
      const uint32_t xm = o.xm & 15, zm = o.zm & 15;
      if ((o.cm & 15) != 0) return false;
      cplx<R> c, w;
      prot_coeffs<R>(o, theta, c, w);
      if (one_bit(xm) && (zm & ~xm) == 0) {
        K = __ffs(xm) - 1;
        u[0] = u[3] = c;
        u[1] = (zm & xm) ? cplx<R>(-w.x, -w.y) : w;
        u[2] = w;
        return true;
      }
      if (xm == 0 && one_bit(zm)) {
        K = __ffs(zm) - 1;
        u[0] = cplx<R>(c.x + w.x, c.y + w.y);
        u[1] = u[2] = z;
        u[3] = cplx<R>(c.x - w.x, c.y - w.y);
        return true;
      }
      return false;
    }
    default: return false;
  }
}

// Compile op k of the table into r.  adj: the record applies ops[k]^dagger;
// grad: fill the gradient routine of an op with a slot.  Forward records of
// an op with fuse_next = m > 0 multiply in the next m ops (same register bit)
// and skip them.
template <typename R>
__device__ __forceinline__ void rop_build(ROp<R>& r, const tq_tile_op* __restrict__ ops, int k, const double* theta,
                                          bool adj, bool grad) {
  const tq_tile_op& o = ops[k];
  ROp<R> q;
  q.code = RC_NOP;
  q.gcode = RG_NONE;
  q.op = k;
  q.zo = o.zo;
  q.zg = o.zg;
  q.skip = 1;
  q.pad = 0;
  const cplx<R> z(R(0), R(0));
  q.m[0] = q.m[1] = q.m[2] = q.m[3] = z;
  q.gph = z;
  q.gw0 = q.gw1 = R(0);
  const int a = o.a & 3, b = o.b & 3;
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
      q.code = RC_U1 + a;
      q.m[0] = u0;
      q.m[1] = u1;
      q.m[2] = u2;
      q.m[3] = u3;
      break;
    }
    case TOP_D1: {
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
      q.code = (d0.x == R(1) && d0.y == R(0)) ? RC_DH + a : RC_D + a;
      q.m[0] = d0;
      q.m[1] = d1;
      break;
    }
    case TOP_U2: q.code = RC_U2; break;
    case TOP_CX: q.code = a != b ? RC_CX + pair_index(a, b) : RC_NOP; break;
    case TOP_SWAP: q.code = a != b ? RC_SWAP + pair_index(a, b) : RC_NOP; break;
    case TOP_CZ: q.code = a != b ? RC_CZ + pair_index(a, b) : RC_NOP; break;
    case TOP_PROT: {
      cplx<R> c, w;
      prot_coeffs<R>(o, theta, c, w);
      if (adj) w = cplx<R>(-w.x, -w.y);  // exp(+i t/2 P): the sin term flips sign
      const uint32_t xm = o.xm & 15, zm = o.zm & 15, cm = o.cm & 15;
      if (cm == 0 && one_bit(xm) && (zm & ~xm) == 0) {
        // pair (i, j = i | bit K): x_i' = c x_i + w (-1)^{zK} x_j, x_j' = w x_i + c x_j
        const int K = __ffs(xm) - 1;
        const cplx<R> w01 = (zm & xm) ? cplx<R>(-w.x, -w.y) : w;
        q.m[0] = c;
        q.m[1] = w01;
        q.m[2] = w;
        q.m[3] = c;
        if (c.y == R(0) && w.y == R(0))
          q.code = RC_RR + K;
        else if (c.y == R(0) && w.x == R(0))
          q.code = RC_RI + K;
        else
          q.code = RC_U1 + K;
      } else if (cm == 0 && xm == 0 && one_bit(zm)) {
        // diag(c + w, c - w) on bit K
        q.code = RC_D + (__ffs(zm) - 1);
        q.m[0] = cplx<R>(c.x + w.x, c.y + w.y);
        q.m[1] = cplx<R>(c.x - w.x, c.y - w.y);
      } else {
        q.code = RC_PROT;
        q.m[0] = c;
        q.m[1] = w;
      }
      break;
    }
    default: break;
  }
  if (!adj && o.fuse_next > 0) {
    cplx<R> u[4];
    int K = -1;
    if (op_mat2<R>(o, theta, u, K)) {
      int j = 1;
      for (; j <= o.fuse_next && j < 16; ++j) {
        cplx<R> v[4];
        int Kj = -1;
        if (!op_mat2<R>(ops[k + j], theta, v, Kj) || Kj != K) break;
        const cplx<R> p0 = cfma(v[1], u[2], cmul(v[0], u[0])), p1 = cfma(v[1], u[3], cmul(v[0], u[1]));
        const cplx<R> p2 = cfma(v[3], u[2], cmul(v[2], u[0])), p3 = cfma(v[3], u[3], cmul(v[2], u[1]));
        u[0] = p0;
        u[1] = p1;
        u[2] = p2;
        u[3] = p3;
      }
      q.code = RC_U1 + K;
      for (int e = 0; e < 4; ++e) q.m[e] = u[e];
      q.skip = j;
    }
  }
  if (grad && o.slot >= 0) {
    const R re[4] = {R(1), R(0), R(-1), R(0)}, im[4] = {R(0), R(1), R(0), R(-1)};
    q.gph = cplx<R>(re[o.gny & 3], im[o.gny & 3]);
    const uint32_t gx = o.gxm, gz = o.gzm, gc = o.gcm;
    if (gc == 0 && one_bit(gx) && gx < 16 && (gz & ~gx) == 0) {
      q.gcode = RG_PAIR + (__ffs(gx) - 1);
      q.gw0 = (gz & gx) ? R(-1) : R(1);
    } else if (gx == 0 && gc == 0 && one_bit(gz) && gz < 16) {
      q.gcode = RG_DIAG + (__ffs(gz) - 1);
      q.gw0 = R(1);
      q.gw1 = R(-1);
    } else if (gx == 0 && gz == 0 && one_bit(gc) && gc < 16) {
      q.gcode = RG_DIAG + (__ffs(gc) - 1);
      q.gw0 = R(0);
      q.gw1 = R(1);
    } else {
      q.gcode = RG_GEN;
    }
  }
  r = q;
}

// Compile ops [k0, k1) into rops[0 .. k1-k0) (all threads of the CTA).
template <typename R>
__device__ __forceinline__ void rops_build(ROp<R>* rops, const tq_tile_op* __restrict__ ops, int k0, int k1,
                                           const double* theta, bool adj, bool grad) {
  for (int k = k0 + (int)threadIdx.x; k < k1; k += blockDim.x) rop_build<R>(rops[k - k0], ops, k, theta, adj, grad);
}

// Sign of the op's Z factors outside the registers: tile base gbase, thread base tbase.
template <typename R>
__device__ __forceinline__ R rop_sign(const ROp<R>& r, uint64_t gbase, int tbase) {
  const uint32_t zo = r.zo;
  const uint64_t zg = r.zg;
  if ((zo | zg) == 0) return R(1);
  const int par = (__popcll(gbase & zg) + __popc((unsigned)tbase & zo)) & 1;
  return par ? R(-1) : R(1);
}

#define TQ_RK_CASES(BASE, FN, ...)                                                               \
  case BASE + 0: FN<R, NR, 0>(x, __VA_ARGS__); if (NA == 2) FN<R, NR, 0>(y, __VA_ARGS__); break; \
  case BASE + 1: FN<R, NR, 1>(x, __VA_ARGS__); if (NA == 2) FN<R, NR, 1>(y, __VA_ARGS__); break; \
  case BASE + 2: FN<R, NR, 2>(x, __VA_ARGS__); if (NA == 2) FN<R, NR, 2>(y, __VA_ARGS__); break; \
  case BASE + 3: FN<R, NR, 3>(x, __VA_ARGS__); if (NA == 2) FN<R, NR, 3>(y, __VA_ARGS__); break;

#define TQ_PAIR_CASE(BASE, MODE, A, B) \
  case BASE + 4 * A + B: r_perm<R, NR, MODE, A, B>(x); if (NA == 2) r_perm<R, NR, MODE, A, B>(y); break;
#define TQ_PAIR_CASES(BASE, MODE)                                                                      \
  TQ_PAIR_CASE(BASE, MODE, 0, 1) TQ_PAIR_CASE(BASE, MODE, 0, 2) TQ_PAIR_CASE(BASE, MODE, 0, 3)           \
  TQ_PAIR_CASE(BASE, MODE, 1, 0) TQ_PAIR_CASE(BASE, MODE, 1, 2) TQ_PAIR_CASE(BASE, MODE, 1, 3)           \
  TQ_PAIR_CASE(BASE, MODE, 2, 0) TQ_PAIR_CASE(BASE, MODE, 2, 1) TQ_PAIR_CASE(BASE, MODE, 2, 3)           \
  TQ_PAIR_CASE(BASE, MODE, 3, 0) TQ_PAIR_CASE(BASE, MODE, 3, 1) TQ_PAIR_CASE(BASE, MODE, 3, 2)

// Apply compiled op r to x (and to y when NA == 2) with sign s; NR
// amplitudes per array (2^stage bits).  Codes for register bits >= log2(NR)
// never occur and compile to nothing.
template <typename R, int NA, int NR>
__device__ __forceinline__ void rop_apply(cplx<R>* x, cplx<R>* y, const ROp<R>& r,
                                          const tq_tile_op* __restrict__ ops, bool adj, R s) {
  switch (r.code) {
    TQ_RK_CASES(RC_U1, r_u1, r.m[0], cplx<R>(s * r.m[1].x, s * r.m[1].y), cplx<R>(s * r.m[2].x, s * r.m[2].y),
                r.m[3])
    TQ_RK_CASES(RC_RR, r_rr, r.m[0].x, s * r.m[1].x, s * r.m[2].x)
    TQ_RK_CASES(RC_RI, r_ri, r.m[0].x, s * r.m[1].y, s * r.m[2].y)
    TQ_RK_CASES(RC_D, r_d1, s < R(0) ? r.m[1] : r.m[0], s < R(0) ? r.m[0] : r.m[1])
    TQ_RK_CASES(RC_DH, r_dh, r.m[1])
    TQ_PAIR_CASES(RC_CX, 0)
    TQ_PAIR_CASES(RC_SWAP, 1)
    TQ_PAIR_CASES(RC_CZ, 2)
    default: break;  // RC_U2 / RC_PROT: cold path (s_cold_apply)
  }
}

// Gradient partial Im <y|G|x> of compiled op r (unsigned; the caller applies the op's sign).
template <typename R, int NR>
__device__ __forceinline__ R rop_grad(const cplx<R>* x, const cplx<R>* y, const ROp<R>& r,
                                      const tq_tile_op* __restrict__ ops) {
  switch (r.gcode) {
    case RG_PAIR + 0: return g_pair<R, NR, 0>(x, y, r.gph, r.gw0);
    case RG_PAIR + 1: return g_pair<R, NR, 1>(x, y, r.gph, r.gw0);
    case RG_PAIR + 2: return g_pair<R, NR, 2>(x, y, r.gph, r.gw0);
    case RG_PAIR + 3: return g_pair<R, NR, 3>(x, y, r.gph, r.gw0);
    case RG_DIAG + 0: return g_diag<R, NR, 0>(x, y, r.gph, r.gw0, r.gw1);
    case RG_DIAG + 1: return g_diag<R, NR, 1>(x, y, r.gph, r.gw0, r.gw1);
    case RG_DIAG + 2: return g_diag<R, NR, 2>(x, y, r.gph, r.gw0, r.gw1);
    case RG_DIAG + 3: return g_diag<R, NR, 3>(x, y, r.gph, r.gw0, r.gw1);
    default: return R(0);  // RG_GEN: cold path (s_cold_grad)
  }
}

// ------------------------------------------------------------------ stage mapping
// Per-thread register <-> padded shared-memory index of register i for a stage
// with RB register bits b[0..RB) (ascending local positions).  pphys is
// additive over disjoint bit sets (j + 2 (j >> 4) has no carries between them),
// so the padded address of register i is p0 + sum of pm[k] over i's bits.
template <int RB>
struct StageMap {
  int base;       // local index with all register bits zero
  int p0;         // pphys(base)
  int pm[RB];     // pphys(1 << bits[k])
  __device__ __forceinline__ int phys(int i) const {  // i is a compile-time constant at most calls
    int v = p0;
#pragma unroll
    for (int k = 0; k < RB; ++k) v += ((i >> k) & 1) ? pm[k] : 0;
    return v;
  }
  // addr[i] = phys(i) for every register: one add each
  __device__ __forceinline__ void addrs(int* addr) const {
    addr[0] = p0;
#pragma unroll
    for (int i = 1; i < (1 << RB); ++i) {
      const int low = i & -i;
      const int k = low == 1 ? 0 : low == 2 ? 1 : low == 4 ? 2 : 3;
      addr[i] = addr[i ^ low] + pm[k];
    }
  }
};

template <int RB>
__device__ __forceinline__ StageMap<RB> stage_map(const tq_tile_stage& st, int tid) {
  StageMap<RB> m;
  int b = tid;
#pragma unroll
  for (int k = 0; k < RB; ++k) b = insz(b, st.bits[k]);
  m.base = b;
  m.p0 = pphys(b);
#pragma unroll
  for (int k = 0; k < RB; ++k) m.pm[k] = pphys(1 << st.bits[k]);
  return m;
}

// Ops without a register routine: general dense 4x4 (RC_U2), Pauli rotations
// with several flip bits or a control (RC_PROT), and general gradient
// generators (RG_GEN).  The thread moves its registers to its own slots of the
// shared-memory tile (no other thread touches them, so no barrier is needed),
// applies the op there with runtime register-bit indices and reloads.
template <typename R>
__device__ __forceinline__ bool rop_is_cold(const ROp<R>& r) {
  return r.code == RC_U2 || r.code == RC_PROT || r.gcode == RG_GEN;
}

template <int RB>
__device__ __forceinline__ int slot_of(const StageMap<RB>& mp, int i) {
  return mp.phys(i);
}

template <typename R, int RB>
__device__ void s_cold_apply(cplx<R>* s, const StageMap<RB>& mp, const tq_tile_op& o, const ROp<R>& r, bool adj,
                             R sgn) {
  constexpr int NR = 1 << RB;
  if (r.code == RC_U2) {
    const int A = o.a, B = o.b, plo = A < B ? A : B, phi = A < B ? B : A;
    for (int q = 0; q < NR / 4; ++q) {
      const int i = insz(insz(q, plo), phi);
      const int id[4] = {slot_of<RB>(mp, i), slot_of<RB>(mp, i | (1 << B)), slot_of<RB>(mp, i | (1 << A)),
                         slot_of<RB>(mp, i | (1 << A) | (1 << B))};
      const cplx<R> v[4] = {s[id[0]], s[id[1]], s[id[2]], s[id[3]]};
      for (int rr = 0; rr < 4; ++rr) {
        cplx<R> acc(R(0), R(0));
        for (int c = 0; c < 4; ++c) {
          cplx<R> u = adj ? op_m<R>(o, 4 * c + rr) : op_m<R>(o, 4 * rr + c);
          if (adj) u.y = -u.y;
          acc = cfma(u, v[c], acc);
        }
        s[id[rr]] = acc;
      }
    }
  } else if (r.code == RC_PROT) {
    const cplx<R> c = r.m[0], w(sgn * r.m[1].x, sgn * r.m[1].y);
    const uint32_t xm = o.xm & (NR - 1), zm = o.zm, cm = o.cm;
    if (xm == 0) {
      for (int i = 0; i < NR; ++i) {
        if ((i & cm) != cm) continue;
        const R sg = (__popc(i & zm) & 1) ? R(-1) : R(1);
        const int a = slot_of<RB>(mp, i);
        s[a] = cmul(cplx<R>(c.x + sg * w.x, sg * w.y), s[a]);
      }
    } else {
      const int h = 31 - __clz(xm);
      for (int i = 0; i < NR; ++i) {
        if ((i >> h) & 1) continue;
        const int j = i ^ (int)xm;
        if ((i & cm) != cm) continue;
        const int ai = slot_of<RB>(mp, i), aj = slot_of<RB>(mp, j);
        const cplx<R> a = s[ai], b = s[aj];
        const R si = (__popc(i & zm) & 1) ? R(-1) : R(1);
        const R sj = (__popc(j & zm) & 1) ? R(-1) : R(1);
        s[ai] = cfma(cplx<R>(w.x * sj, w.y * sj), b, cplx<R>(c.x * a.x, c.x * a.y));
        s[aj] = cfma(cplx<R>(w.x * si, w.y * si), a, cplx<R>(c.x * b.x, c.x * b.y));
      }
    }
  }
  // any other code of a cold record (a hot op with a general generator) is applied by the caller
}

// Im <lam|G|psi> over the thread's slots (sp = psi, sl = lam), G from the op's
// generator masks: G|i> = [i & gcm == gcm] i^gny (-1)^{popc(i & gzm)} |i ^ gxm>.
template <typename R, int RB>
__device__ R s_cold_grad(const cplx<R>* sp, const cplx<R>* sl, const StageMap<RB>& mp, const tq_tile_op& o) {
  constexpr int NR = 1 << RB;
  const R re[4] = {R(1), R(0), R(-1), R(0)}, im[4] = {R(0), R(1), R(0), R(-1)};
  const cplx<R> ph(re[o.gny & 3], im[o.gny & 3]);
  const uint32_t xm = o.gxm & (NR - 1), zm = o.gzm, cm = o.gcm;
  R acc = 0;
  for (int i = 0; i < NR; ++i) {
    if ((i & cm) != cm) continue;
    const R sg = (__popc(i & zm) & 1) ? R(-1) : R(1);
    const cplx<R> v = cmul(ph, sp[slot_of<RB>(mp, i)]);
    const cplx<R> l = sl[slot_of<RB>(mp, i ^ (int)xm)];
    acc += sg * (l.x * v.y - l.y * v.x);
  }
  return acc;
}

// ------------------------------------------------------------------ out-of-place forms
// The forward path alternates between two register arrays: every op reads
// array a and writes all 16 amplitudes of array b.  No value has to be moved
// back into its input register after a dispatch, which an in-place update of
// a register pair cannot avoid.
template <typename R, int K>
__device__ __forceinline__ void t_u1(const cplx<R>* a, cplx<R>* b, cplx<R> u0, cplx<R> u1, cplx<R> u2, cplx<R> u3) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    b[i] = cfma(u1, a[j], cmul(u0, a[i]));
    b[j] = cfma(u3, a[j], cmul(u2, a[i]));
  }
}

template <typename R, int K>
__device__ __forceinline__ void t_rr(const cplx<R>* a, cplx<R>* b, R c, R a01, R a10) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    b[i] = cplx<R>(fma(a01, a[j].x, c * a[i].x), fma(a01, a[j].y, c * a[i].y));
    b[j] = cplx<R>(fma(a10, a[i].x, c * a[j].x), fma(a10, a[i].y, c * a[j].y));
  }
}

template <typename R, int K>
__device__ __forceinline__ void t_ri(const cplx<R>* a, cplx<R>* b, R c, R b01, R b10) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if ((i >> K) & 1) continue;
    const int j = i | (1 << K);
    b[i] = cplx<R>(fma(-b01, a[j].y, c * a[i].x), fma(b01, a[j].x, c * a[i].y));
    b[j] = cplx<R>(fma(-b10, a[i].y, c * a[j].x), fma(b10, a[i].x, c * a[j].y));
  }
}

template <typename R, int K>
__device__ __forceinline__ void t_d1(const cplx<R>* a, cplx<R>* b, cplx<R> d0, cplx<R> d1) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) b[i] = cmul(((i >> K) & 1) ? d1 : d0, a[i]);
}

template <typename R, int K>
__device__ __forceinline__ void t_dh(const cplx<R>* a, cplx<R>* b, cplx<R> d1) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) b[i] = ((i >> K) & 1) ? cmul(d1, a[i]) : a[i];
}

// MODE 0 CX (control A, target B), 1 SWAP, 2 CZ
template <typename R, int MODE, int A, int B>
__device__ __forceinline__ void t_perm(const cplx<R>* a, cplx<R>* b) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    const int ba = (i >> A) & 1, bb = (i >> B) & 1;
    if (MODE == 0) {
      b[i] = a[ba ? i ^ (1 << B) : i];
    } else if (MODE == 1) {
      b[i] = a[ba != bb ? i ^ (1 << A) ^ (1 << B) : i];
    } else {
      b[i] = (ba && bb) ? cplx<R>(-a[i].x, -a[i].y) : a[i];
    }
  }
}

template <typename R, int A, int B>
__device__ __forceinline__ void t_u2(const cplx<R>* a, cplx<R>* b, const tq_tile_op& o) {
#pragma unroll
  for (int i = 0; i < kNR; ++i) {
    if (((i >> A) & 1) || ((i >> B) & 1)) continue;
    const int id[4] = {i, i | (1 << B), i | (1 << A), i | (1 << A) | (1 << B)};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      cplx<R> acc = cmul(op_m<R>(o, 4 * r), a[id[0]]);
      acc = cfma(op_m<R>(o, 4 * r + 1), a[id[1]], acc);
      acc = cfma(op_m<R>(o, 4 * r + 2), a[id[2]], acc);
      acc = cfma(op_m<R>(o, 4 * r + 3), a[id[3]], acc);
      b[id[r]] = acc;
    }
  }
}

template <typename R, int XM>
__device__ __forceinline__ void t_prot(const cplx<R>* a, cplx<R>* b, uint32_t zm, uint32_t cm, cplx<R> c,
                                       cplx<R> w) {
  if (XM == 0) {
#pragma unroll
    for (int i = 0; i < kNR; ++i) {
      const R sg = (__popc(i & zm) & 1) ? R(-1) : R(1);
      b[i] = ((i & cm) == cm) ? cmul(cplx<R>(c.x + sg * w.x, sg * w.y), a[i]) : a[i];
    }
  } else {
    constexpr int H = (XM & 8) ? 3 : (XM & 4) ? 2 : (XM & 2) ? 1 : 0;
#pragma unroll
    for (int i = 0; i < kNR; ++i) {
      if ((i >> H) & 1) continue;
      const int j = i ^ XM;
      const bool on = (i & cm) == cm;
      const R si = (__popc(i & zm) & 1) ? R(-1) : R(1);
      const R sj = (__popc(j & zm) & 1) ? R(-1) : R(1);
      const cplx<R> ni = cfma(cplx<R>(w.x * sj, w.y * sj), a[j], cplx<R>(c.x * a[i].x, c.x * a[i].y));
      const cplx<R> nj = cfma(cplx<R>(w.x * si, w.y * si), a[i], cplx<R>(c.x * a[j].x, c.x * a[j].y));
      b[i] = on ? ni : a[i];
      b[j] = on ? nj : a[j];
    }
  }
}

#define TQ_TK_CASES(BASE, FN, ...)                       \
  case BASE + 0: FN<R, 0>(a, b, __VA_ARGS__); break;     \
  case BASE + 1: FN<R, 1>(a, b, __VA_ARGS__); break;     \
  case BASE + 2: FN<R, 2>(a, b, __VA_ARGS__); break;     \
  case BASE + 3: FN<R, 3>(a, b, __VA_ARGS__); break;
#define TQ_TPAIR_CASE(BASE, MODE, A, B) case BASE + 4 * A + B: t_perm<R, MODE, A, B>(a, b); break;
#define TQ_TPAIR_CASES(BASE, MODE)                                                                          \
  TQ_TPAIR_CASE(BASE, MODE, 0, 1) TQ_TPAIR_CASE(BASE, MODE, 0, 2) TQ_TPAIR_CASE(BASE, MODE, 0, 3)            \
  TQ_TPAIR_CASE(BASE, MODE, 1, 0) TQ_TPAIR_CASE(BASE, MODE, 1, 2) TQ_TPAIR_CASE(BASE, MODE, 1, 3)            \
  TQ_TPAIR_CASE(BASE, MODE, 2, 0) TQ_TPAIR_CASE(BASE, MODE, 2, 1) TQ_TPAIR_CASE(BASE, MODE, 2, 3)            \
  TQ_TPAIR_CASE(BASE, MODE, 3, 0) TQ_TPAIR_CASE(BASE, MODE, 3, 1) TQ_TPAIR_CASE(BASE, MODE, 3, 2)

// b = (compiled forward op r) a, with sign s.
template <typename R>
__device__ __forceinline__ void rop_apply_to(const cplx<R>* a, cplx<R>* b, const ROp<R>& r,
                                             const tq_tile_op* __restrict__ ops, R s) {
  switch (r.code) {
    TQ_TK_CASES(RC_U1, t_u1, r.m[0], cplx<R>(s * r.m[1].x, s * r.m[1].y), cplx<R>(s * r.m[2].x, s * r.m[2].y),
                r.m[3])
    TQ_TK_CASES(RC_RR, t_rr, r.m[0].x, s * r.m[1].x, s * r.m[2].x)
    TQ_TK_CASES(RC_RI, t_ri, r.m[0].x, s * r.m[1].y, s * r.m[2].y)
    TQ_TK_CASES(RC_D, t_d1, s < R(0) ? r.m[1] : r.m[0], s < R(0) ? r.m[0] : r.m[1])
    TQ_TK_CASES(RC_DH, t_dh, r.m[1])
    TQ_TPAIR_CASES(RC_CX, 0)
    TQ_TPAIR_CASES(RC_SWAP, 1)
    TQ_TPAIR_CASES(RC_CZ, 2)
    case RC_U2: {
      const tq_tile_op& o = ops[r.op];
      switch (o.a * 4 + o.b) {
        case 1: t_u2<R, 0, 1>(a, b, o); break;
        case 2: t_u2<R, 0, 2>(a, b, o); break;
        case 3: t_u2<R, 0, 3>(a, b, o); break;
        case 4: t_u2<R, 1, 0>(a, b, o); break;
        case 6: t_u2<R, 1, 2>(a, b, o); break;
        case 7: t_u2<R, 1, 3>(a, b, o); break;
        case 8: t_u2<R, 2, 0>(a, b, o); break;
        case 9: t_u2<R, 2, 1>(a, b, o); break;
        case 11: t_u2<R, 2, 3>(a, b, o); break;
        case 12: t_u2<R, 3, 0>(a, b, o); break;
        case 13: t_u2<R, 3, 1>(a, b, o); break;
        case 14: t_u2<R, 3, 2>(a, b, o); break;
        default:
#pragma unroll
          for (int i = 0; i < kNR; ++i) b[i] = a[i];
          break;
      }
      break;
    }
    case RC_PROT: {
      const tq_tile_op& o = ops[r.op];
      const cplx<R> w(s * r.m[1].x, s * r.m[1].y), c = r.m[0];
      const uint32_t zm = o.zm, cm = o.cm;
      switch (o.xm & 15) {
        case 0: t_prot<R, 0>(a, b, zm, cm, c, w); break;
        case 1: t_prot<R, 1>(a, b, zm, cm, c, w); break;
        case 2: t_prot<R, 2>(a, b, zm, cm, c, w); break;
        case 3: t_prot<R, 3>(a, b, zm, cm, c, w); break;
        case 4: t_prot<R, 4>(a, b, zm, cm, c, w); break;
        case 5: t_prot<R, 5>(a, b, zm, cm, c, w); break;
        case 6: t_prot<R, 6>(a, b, zm, cm, c, w); break;
        case 7: t_prot<R, 7>(a, b, zm, cm, c, w); break;
        case 8: t_prot<R, 8>(a, b, zm, cm, c, w); break;
        case 9: t_prot<R, 9>(a, b, zm, cm, c, w); break;
        case 10: t_prot<R, 10>(a, b, zm, cm, c, w); break;
        case 11: t_prot<R, 11>(a, b, zm, cm, c, w); break;
        case 12: t_prot<R, 12>(a, b, zm, cm, c, w); break;
        case 13: t_prot<R, 13>(a, b, zm, cm, c, w); break;
        case 14: t_prot<R, 14>(a, b, zm, cm, c, w); break;
        default: t_prot<R, 15>(a, b, zm, cm, c, w); break;
      }
      break;
    }
    default:
#pragma unroll
      for (int i = 0; i < kNR; ++i) b[i] = a[i];
      break;
  }
}

// Run stages[s0..s1) forward on the padded tile s (2^(t-4) threads).
// rops: the pass's compiled ops when `resident` (rops[k - op0] is op k),
// else room for kRopCap ops compiled chunk by chunk.  The caller
// synchronises before the first stage.
template <typename R>
__device__ __forceinline__ void run_stages(cplx<R>* s, ROp<R>* rops, bool resident, int op0,
                                           const tq_tile_stage* __restrict__ stages, int s0, int s1,
                                           const tq_tile_op* __restrict__ ops, const double* theta,
                                           uint64_t gbase) {
  for (int si = s0; si < s1; ++si) {
    const tq_tile_stage st = stages[si];
    const StageMap<kRB> m = stage_map<kRB>(st, threadIdx.x);
    cplx<R> x[kNR], x2[kNR];
    {
      int ad[kNR];
      m.addrs(ad);
#pragma unroll
      for (int i = 0; i < kNR; ++i) x[i] = s[ad[i]];
    }
    for (int k0 = st.op_begin; k0 < st.op_end;) {
      const int k1 = resident ? st.op_end : min(k0 + kRopCap, st.op_end);
      const ROp<R>* rr = rops - (resident ? op0 : k0);
      if (!resident) {
        if (k0 != st.op_begin) __syncthreads();  // readers of the previous chunk are done
        rops_build<R>(rops, ops, k0, k1, theta, false, false);
        __syncthreads();
      }
      // a fused record may reach past k1; the next chunk starts after it
      int k = k0;
      while (k < k1) {
        const ROp<R>& ra = rr[k];
        rop_apply_to<R>(x, x2, ra, ops, rop_sign<R>(ra, gbase, m.base));
        k += ra.skip;
        if (k >= k1) {
#pragma unroll
          for (int i = 0; i < kNR; ++i) x[i] = x2[i];
          break;
        }
        const ROp<R>& rb = rr[k];
        rop_apply_to<R>(x2, x, rb, ops, rop_sign<R>(rb, gbase, m.base));
        k += rb.skip;
      }
      k0 = k;
    }
    {
      int ad[kNR];
      m.addrs(ad);
#pragma unroll
      for (int i = 0; i < kNR; ++i) s[ad[i]] = x[i];
    }
    __syncthreads();
  }
}

}  // namespace tq
