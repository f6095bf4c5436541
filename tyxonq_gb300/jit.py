"""Circuit-specialised register-staged passes (runtime-compiled CUDA).

A staged forward program (``program.encode_staged``) is normally run by the
library's interpreting kernel, which dispatches every op through a switch and
moves all 16 registers per op.  ``specialise`` writes CUDA C++ in which each
pass is straight-line register code: the stage layouts, register bits and op
shapes are literals, permutations are register renames, and only the
coefficients (compiled from the op table and theta on the device, exactly as
the interpreter does) remain data.  The source is compiled for sm_103a in
process by NVRTC (``tq_jit_build``, one kernel per distinct pass, built in
parallel threads), cached as cubins on disk and per process, so programs with
the same gate structure and different angles share the kernels.

Coverage: every op code of the forward register stages (dense / real /
imaginary / diagonal single-bit ops, runs fused on the device, CX / SWAP / CZ,
dense 4x4, general Pauli rotations, Z signs from outside the stage).  A pass
with more than 256 ops keeps the interpreter.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import threading
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _native as nat

CSRC = Path(__file__).resolve().parent / "csrc"
INCLUDE = Path(__file__).resolve().parent.parent / "include"
ROP_CAP = 256  # kStagedRopCap

TOP_U1, TOP_D1, TOP_U2, TOP_CX, TOP_CZ, TOP_SWAP, TOP_PROT = 1, 2, 3, 4, 5, 6, 7


def _one_bit(m: int) -> bool:
    return m != 0 and (m & (m - 1)) == 0


def _ffs(m: int) -> int:
    return (m & -m).bit_length() - 1


def _insz(b: str, p: int) -> str:
    return f"b = ((b >> {p}) << {p + 1}) | (b & {(1 << p) - 1});"


def _pphys(j: int) -> int:
    return j + ((j >> 4) << 1)


def _mat(o, e: int, double: bool) -> complex:
    m = o["md"] if double else o["mf"]
    return complex(m[2 * e], m[2 * e + 1])


def _op_code(o, double: bool) -> tuple:
    """(routine, args) the device compiles op record o into (rop_build, forward,
    not fused); routine None = no-op.  Register bits as encoded (0..rb-1)."""
    kind = int(o["kind"])
    a, b = int(o["a"]), int(o["b"])
    if kind == TOP_U1:
        return _u1_routine(o, double)
    if kind == TOP_D1:
        if int(o["pidx"]) >= 0:
            return "dh", a
        d0 = _mat(o, 0, double)
        return ("dh" if (d0.real == 1.0 and d0.imag == 0.0) else "d", a)
    if kind == TOP_U2:
        return ("u2", (int(o["a"]), int(o["b"]))) if o["a"] != o["b"] else (None, None)
    if kind in (TOP_CX, TOP_SWAP, TOP_CZ):
        mode = {TOP_CX: 0, TOP_SWAP: 1, TOP_CZ: 2}[kind]
        return ("perm", (mode, a, b)) if a != b else (None, None)
    if kind == TOP_PROT:
        xm, zm, cm = int(o["xm"]) & 15, int(o["zm"]) & 15, int(o["cm"]) & 15
        if cm == 0 and _one_bit(xm) and (zm & ~xm) == 0:
            K = _ffs(xm)
            if int(o["pidx"]) >= 0:
                ny = bin(int(o["xm"]) & int(o["zm"])).count("1") & 3
                return ("rr" if ny & 1 else "ri"), K
            c, w = _mat(o, 0, double), _mat(o, 1, double)
            if c.imag == 0.0 and w.imag == 0.0:
                return "rr", K
            if c.imag == 0.0 and w.real == 0.0:
                return "ri", K
            return "u1", K
        if cm == 0 and xm == 0 and _one_bit(zm):
            return "d", _ffs(zm)
        if int(o["cm"]) >= 16:
            return None, None  # the interpreter's (i & cm) == cm never holds: no-op
        return "prot", (xm, int(o["zm"]) & 15, int(o["cm"]))
    return None, None


def _shape2(o, double: bool) -> str | None:
    """Shape of the 2x2 an op contributes to a fused run, as the device builds
    it (op_mat2): "diag" (off-diagonals zero), "real" (all entries real),
    "dense", or None when the values are only known on the device."""
    kind = int(o["kind"])
    if kind == TOP_U1:
        m = [_mat(o, e, double) for e in range(4)]
        if m[1] == 0 and m[2] == 0:
            return "diag"
        return "real" if all(v.imag == 0 for v in m) else "dense"
    if kind == TOP_D1:
        return "diag"
    if kind == TOP_PROT:
        xm, zm = int(o["xm"]) & 15, int(o["zm"]) & 15
        if xm == 0:
            return "diag"
        if int(o["pidx"]) >= 0:
            ny = bin(int(o["xm"]) & int(o["zm"])).count("1") & 3
            return "real" if ny & 1 else "dense"
        m = [_mat(o, e, double) for e in range(2)]
        return "real" if all(v.imag == 0 for v in m) else "dense"
    return None


def _has_complex_diag(ops, k: int, j: int, double: bool) -> bool:
    """Whether a diagonal factor of ops[k:k+j] may be complex (device angles or
    complex entries): then a product with real factors is not real."""
    for i in range(j):
        o = ops[k + i]
        if _shape2(o, double) != "diag":
            continue
        kind = int(o["kind"])
        if kind == TOP_U1:
            if _mat(o, 0, double).imag != 0 or _mat(o, 3, double).imag != 0:
                return True
        elif kind == TOP_D1:
            if int(o["pidx"]) >= 0 or _mat(o, 0, double).imag != 0 or _mat(o, 1, double).imag != 0:
                return True
        else:
            return True  # a Z rotation: c +- w with imaginary w
    return False


def _u1_routine(o, double: bool) -> tuple:
    """Cheapest register routine for a fixed single-bit 2x2 (TOP_U1): the
    record holds the matrix m0..m3."""
    m = [_mat(o, e, double) for e in range(4)]
    a = int(o["a"])
    if m[1] == 0 and m[2] == 0:
        return "d03", a
    if all(v.imag == 0 for v in m):
        return "ureal", a
    if m[0] == m[3] and m[0].imag == 0 and m[1].real == 0 and m[2].real == 0:
        return "ri", a
    return "u1", a


def _single_bit(o) -> int | None:
    """Register bit of a fusable op (device op_mat2), else None."""
    if int(o["zo"]) or int(o["zg"]):
        return None
    kind = int(o["kind"])
    if kind in (TOP_U1, TOP_D1):
        return int(o["a"])
    if kind == TOP_PROT:
        xm, zm, cm = int(o["xm"]) & 15, int(o["zm"]) & 15, int(o["cm"]) & 15
        if cm:
            return None
        if _one_bit(xm) and (zm & ~xm) == 0:
            return _ffs(xm)
        if xm == 0 and _one_bit(zm):
            return _ffs(zm)
    return None


def _emit_op(lines: list, k_rel: int, o, routine: str, arg, signed: bool) -> None:
    r = f"rops[{k_rel}]"
    s = "sg * " if signed else ""
    pre = f"const ROp<R>& r = {r}; " + ("const R sg = rop_sign<R>(r, gbase, b); " if signed else "")
    if routine == "u1":
        call = (f"r_u1<R, NR, {arg}>(x, r.m[0], cplx<R>({s}r.m[1].x, {s}r.m[1].y), "
                f"cplx<R>({s}r.m[2].x, {s}r.m[2].y), r.m[3]);")
    elif routine == "rr":
        call = f"r_rr<R, NR, {arg}>(x, r.m[0].x, {s}r.m[1].x, {s}r.m[2].x);"
    elif routine == "ri":
        call = f"r_ri<R, NR, {arg}>(x, r.m[0].x, {s}r.m[1].y, {s}r.m[2].y);"
    elif routine == "d":
        if signed:
            call = f"r_d1<R, NR, {arg}>(x, sg < R(0) ? r.m[1] : r.m[0], sg < R(0) ? r.m[0] : r.m[1]);"
        else:
            call = f"r_d1<R, NR, {arg}>(x, r.m[0], r.m[1]);"
    elif routine == "dh":
        call = f"r_dh<R, NR, {arg}>(x, r.m[1]);"
    elif routine == "d03":  # diagonal held as a dense 2x2: diag(m0, m3)
        call = f"r_d1<R, NR, {arg}>(x, r.m[0], r.m[3]);"
    elif routine == "ureal":
        call = f"j_ureal<R, NR, {arg}>(x, r.m[0].x, r.m[1].x, r.m[2].x, r.m[3].x);"
    elif routine == "perm":
        mode, a, b = arg
        call = f"r_perm<R, NR, {mode}, {a}, {b}>(x);"
        pre = ""
    elif routine == "u2":
        A, B = arg
        call = f"j_u2<R, NR, {A}, {B}>(x, ops[r.op]);"
    elif routine == "prot":
        xm, zm, cm = arg
        call = f"j_prot<R, NR, {xm}, {zm}, {cm}>(x, r.m[0], cplx<R>({s}r.m[1].x, {s}r.m[1].y));"
    else:
        return
    lines.append(f"    {{ {pre}{call} }}")


def _geo_off(j: int, nlow: int, pos: list) -> int:
    """Offset from the tile base of local index j (the device's geo_off)."""
    off = j & ((1 << nlow) - 1)
    for k in range(nlow, len(pos)):
        if (j >> k) & 1:
            off |= 1 << pos[k]
    return off


# The last stage stores its registers straight to global memory when none of its
# register bits is below this one.  With register bits 0 or 1 a warp store fills
# half of each 32-byte sector (the other half comes from another register's
# store, merged in L2); measured on the 28-qubit circuit (5-bit stages), storing
# every pass's last stage this way was the fastest: 13-qubit tiles 32.7 ->
# 31.5 ms, 14-qubit tiles 31.9 -> 30.9 ms against a threshold of 2, and 35.9 /
# 40.4 ms with no direct stores at all.
DIRECT_MIN_BIT = 0


def direct_last_ok(stages: np.ndarray, p, stage_bits: list | None = None) -> bool:
    """Whether pass p's last stage may store its registers directly to global memory."""
    se = int(p.op_end)
    if se <= int(p.op_begin):
        return False
    bits = [int(v) for v in (stage_bits[se - 1] if stage_bits is not None else stages[se - 1]["bits"])]
    return all(v >= DIRECT_MIN_BIT for v in bits)


def _pass_body(stages: np.ndarray, ops: np.ndarray, p, double: bool, stage_bits: list | None = None,
               rb: int = 4, direct_geo: tuple | None = None) -> list[str] | None:
    """Body lines of one pass (stages[p.op_begin:p.op_end]) with rb-bit register
    stages (stage_bits: every stage's bits, needed for rb > 4), or None if the
    interpreter must run it.  direct_geo = (nlow, pos): the last stage reads its
    registers, releases the tile buffer (barrier, then on_free() issues the next
    tile's load) and stores its results straight to the tile in global memory
    (gt) at offsets from the compiled-in geometry."""
    NR = 1 << rb
    sb, se = int(p.op_begin), int(p.op_end)
    if se <= sb:
        return None
    op0 = int(stages[sb]["op_begin"])
    nops = int(stages[se - 1]["op_end"]) - op0
    if nops <= 0 or nops > ROP_CAP:
        return None
    lines = []
    for si in range(sb, se):
        st = stages[si]
        bits = [int(v) for v in (stage_bits[si] if stage_bits is not None else st["bits"])]
        if len(bits) != rb or any(v < 0 for v in bits) or sorted(bits) != bits:
            return None
        lines.append(f"  {{  // stage bits {bits}")
        lines.append("    int b = tid;")
        for bb in bits:
            lines.append("    " + _insz("b", bb))
        lines.append("    const int p0 = b + ((b >> 4) << 1);")
        offs = []
        for i in range(NR):
            j = 0
            for k in range(rb):
                if (i >> k) & 1:
                    j |= 1 << bits[k]
            offs.append(_pphys(j))
        lines.append("    " + " ".join(f"x[{i}] = s[p0 + {offs[i]}];" for i in range(NR)))
        last_direct = direct_geo is not None and si == se - 1
        if last_direct:
            lines.append("    __syncthreads();  // every register read: the buffer takes the next tile")
            lines.append("    on_free();")
        k, k1 = int(st["op_begin"]), int(st["op_end"])
        while k < k1:
            o = ops[k]
            fuse = int(o["fuse_next"])
            if fuse > 0 and _single_bit(o) is not None:
                K = _single_bit(o)
                j = 1
                while j <= fuse and j < 16 and k + j < len(ops) and _single_bit(ops[k + j]) == K:
                    j += 1
                # the product's shape from its factors: diagonal or real products stay so
                shapes = {_shape2(ops[k + i], double) for i in range(j)}
                if shapes <= {"diag"}:
                    routine = "d03"
                elif shapes <= {"diag", "real"} and not ("diag" in shapes and _has_complex_diag(ops, k, j, double)):
                    routine = "ureal"
                else:
                    routine = "u1"
                _emit_op(lines, k - op0, o, routine, K, False)
                k += j
                continue
            routine, arg = _op_code(o, double)
            signed = bool(int(o["zo"]) or int(o["zg"]))
            _emit_op(lines, k - op0, o, routine, arg, signed)
            k += 1
        if last_direct:
            nlow, pos = direct_geo
            gofs = []
            for i in range(NR):
                j = 0
                for kk in range(rb):
                    if (i >> kk) & 1:
                        j |= 1 << bits[kk]
                gofs.append(_geo_off(j, nlow, pos))
            lines.append("    const int64_t g0 = geo_off<JitGeom>(b);")
            lines.append("    " + " ".join(f"gt[g0 + {gofs[i]}LL] = {{x[{i}].x, x[{i}].y}};" for i in range(NR)))
        else:
            lines.append("    " + " ".join(f"s[p0 + {offs[i]}] = x[{i}];" for i in range(NR)))
            lines.append("    __syncthreads();")
        lines.append("  }")
    return lines


def _grad_code(o) -> tuple:
    """Gradient routine of an adjoint record with a slot (rop_build, grad)."""
    gx, gz, gc = int(o["gxm"]), int(o["gzm"]), int(o["gcm"])
    if gc == 0 and _one_bit(gx) and gx < 16 and (gz & ~gx) == 0:
        return "pair", _ffs(gx)
    if gx == 0 and gc == 0 and _one_bit(gz) and gz < 16:
        return "diag", _ffs(gz)
    if gx == 0 and gz == 0 and _one_bit(gc) and gc < 16:
        return "diag", _ffs(gc)
    return "gen", (gx & 15, gz & 15, gc)


def _emit_adj_op(lines: list, k_rel: int, o, double: bool) -> None:
    """One adjoint op on psi (x) and lam (y) registers: the gradient term
    Im <lam|G|psi> first (when the op has a slot), then the un-apply."""
    routine, arg = _op_code(o, double)
    if routine == "u2":
        routine = "u2adj"
    has_grad = int(o["slot"]) >= 0
    signed = bool(int(o["zo"]) or int(o["zg"]))
    body = [f"const ROp<R>& r = rops[{k_rel}];"]
    if signed:
        body.append("const R sg = rop_sign<R>(r, gbase, b);")
    s = "sg * " if signed else ""
    if has_grad:
        gk, garg = _grad_code(o)
        if gk == "pair":
            g = f"g_pair<R, NR, {garg}>(x, y, r.gph, r.gw0)"
        elif gk == "diag":
            g = f"g_diag<R, NR, {garg}>(x, y, r.gph, r.gw0, r.gw1)"
        else:
            g = f"j_grad<R, NR, {garg[0]}, {garg[1]}, {garg[2]}>(x, y, r.gph)"
        body.append(f"const R part = {s}{g};")
    for arr in ("x", "y"):
        if routine == "u1":
            body.append(f"r_u1<R, NR, {arg}>({arr}, r.m[0], cplx<R>({s}r.m[1].x, {s}r.m[1].y), "
                        f"cplx<R>({s}r.m[2].x, {s}r.m[2].y), r.m[3]);")
        elif routine == "rr":
            body.append(f"r_rr<R, NR, {arg}>({arr}, r.m[0].x, {s}r.m[1].x, {s}r.m[2].x);")
        elif routine == "ri":
            body.append(f"r_ri<R, NR, {arg}>({arr}, r.m[0].x, {s}r.m[1].y, {s}r.m[2].y);")
        elif routine == "d":
            if signed:
                body.append(f"r_d1<R, NR, {arg}>({arr}, sg < R(0) ? r.m[1] : r.m[0], sg < R(0) ? r.m[0] : r.m[1]);")
            else:
                body.append(f"r_d1<R, NR, {arg}>({arr}, r.m[0], r.m[1]);")
        elif routine == "dh":
            body.append(f"r_dh<R, NR, {arg}>({arr}, r.m[1]);")
        elif routine == "d03":
            body.append(f"r_d1<R, NR, {arg}>({arr}, r.m[0], r.m[3]);")
        elif routine == "ureal":
            body.append(f"j_ureal<R, NR, {arg}>({arr}, r.m[0].x, r.m[1].x, r.m[2].x, r.m[3].x);")
        elif routine == "perm":
            mode, a, b = arg
            body.append(f"r_perm<R, NR, {mode}, {a}, {b}>({arr});")
        elif routine == "u2adj":
            A, B = arg
            body.append(f"j_u2_adj<R, NR, {A}, {B}>({arr}, ops[r.op]);")
        elif routine == "prot":
            xm, zm, cm = arg
            body.append(f"j_prot<R, NR, {xm}, {zm}, {cm}>({arr}, r.m[0], cplx<R>({s}r.m[1].x, {s}r.m[1].y));")
    if has_grad:
        body.append(f"j_part<R>(part, wpart, {k_rel}, nwarps, warp, lane);")
    lines.append("    { " + " ".join(body) + " }")


def _adj_body(stages: np.ndarray, ops: np.ndarray, p, double: bool, max_ops: int) -> list[str] | None:
    """Body lines of one adjoint pass (4-bit stages), or None (library kernel)."""
    sb, se = int(p[2]), int(p[3])
    if se <= sb:
        return None
    op0 = int(stages[sb]["op_begin"])
    nops = int(stages[se - 1]["op_end"]) - op0
    if nops <= 0 or nops > max_ops:
        return None
    lines = []
    for si in range(sb, se):
        st = stages[si]
        bits = [int(v) for v in st["bits"]]
        if any(v < 0 for v in bits) or sorted(bits) != bits:
            return None
        lines.append(f"  {{  // stage bits {bits}")
        lines.append("    int b = tid;")
        for bb in bits:
            lines.append("    " + _insz("b", bb))
        lines.append("    const int p0 = b + ((b >> 4) << 1);")
        offs = []
        for i in range(16):
            j = 0
            for k in range(4):
                if (i >> k) & 1:
                    j |= 1 << bits[k]
            offs.append(_pphys(j))
        lines.append("    " + " ".join(f"x[{i}] = sp[p0 + {offs[i]}]; y[{i}] = sl[p0 + {offs[i]}];"
                                       for i in range(16)))
        for k in range(int(st["op_begin"]), int(st["op_end"])):
            _emit_adj_op(lines, k - op0, ops[k], double)
        lines.append("    " + " ".join(f"sp[p0 + {offs[i]}] = x[{i}]; sl[p0 + {offs[i]}] = y[{i}];"
                                       for i in range(16)))
        lines.append("    __syncthreads();")
        lines.append("  }")
    return lines


WAVE_FWD_KERNEL = "tq_jit_wave_forward"
WAVE_ADJ_KERNEL = "tq_jit_wave_adjoint"


def wave_source(kind: int, t: int, body: str, double: bool) -> str:
    """Source of one wave kernel: kind 0 forward (body over s), 2 adjoint
    (body over sp, sl)."""
    R = "double" if double else "float"
    threads = 1 << (t - 4)
    head = ['#include "jit_wave.cuh"', "", "namespace tq {", "template <typename R>"]
    if kind == 0:
        head.append("__device__ __forceinline__ void jit_body(cplx<R>* __restrict__ s, const ROp<R>* __restrict__ rops, "
                    "const tq_tile_op* __restrict__ ops, uint64_t gbase) {")
        head += ["  const int tid = threadIdx.x;", "  constexpr int NR = 16;", "  cplx<R> x[NR];"]
    else:
        head.append("__device__ __forceinline__ void jit_body(cplx<R>* __restrict__ sp, cplx<R>* __restrict__ sl, "
                    "const ROp<R>* __restrict__ rops, const tq_tile_op* __restrict__ ops, R* __restrict__ wpart, "
                    "uint64_t gbase, int nwarps, int warp, int lane) {")
        head += ["  const int tid = threadIdx.x;", "  constexpr int NR = 16;", "  cplx<R> x[NR], y[NR];"]
    src = head + [body, "}", "}  // namespace tq", ""]
    common = ("const tq_wave_item* __restrict__ items, int n_items, const tq_tile_pass* __restrict__ passes, "
              "const tq_tile_stage* __restrict__ stages, const tq_tile_op* __restrict__ ops, "
              "const double* __restrict__ theta, const void* __restrict__ rops_g, void* pool")
    if kind == 0:
        src.append(f'extern "C" __global__ void __launch_bounds__({threads}) {WAVE_FWD_KERNEL}({common}, int max_ops) {{')
        src.append(f"  tq::jit_wave_forward<{R}>(items, n_items, passes, stages, ops, theta, rops_g, pool, max_ops, "
                   f"[&](tq::cplx<{R}>* s, const tq::ROp<{R}>* rops, uint64_t gbase) "
                   f"{{ tq::jit_body<{R}>(s, rops, ops, gbase); }});")
    else:
        minb = 2 if threads <= 256 else 1
        src.append(f'extern "C" __global__ void __launch_bounds__({threads}, {minb}) {WAVE_ADJ_KERNEL}({common}, '
                   "double* partials, int max_ops) {")
        src.append(f"  tq::jit_wave_adjoint<{R}>(items, n_items, passes, stages, ops, theta, rops_g, pool, partials, "
                   "max_ops, "
                   f"[&](tq::cplx<{R}>* sp, tq::cplx<{R}>* sl, const tq::ROp<{R}>* rops, {R}* wpart, uint64_t gbase, "
                   f"int nwarps, int warp, int lane) "
                   f"{{ tq::jit_body<{R}>(sp, sl, rops, ops, wpart, gbase, nwarps, warp, lane); }});")
    src.append("}")
    return "\n".join(src) + "\n"


def wave_kernels(kind: int, t: int, stages: np.ndarray, ops: np.ndarray, pass_rows: dict, double: bool,
                 max_ops: int, device) -> dict:
    """{pass id: kernel handle} for the given wave passes (pass id -> (t, nlow,
    op_begin, op_end, pos) rows); passes without a body are left out."""
    srcs = {}
    for pid, row in pass_rows.items():
        if kind == 0:
            class _P:
                pass
            pp = _P()
            pp.op_begin, pp.op_end, pp.t = row[2], row[3], row[0]
            lines = _pass_body(stages, ops, pp, double)
            if lines is not None:
                nops = int(stages[row[3] - 1]["op_end"]) - int(stages[row[2]]["op_begin"])
                if nops > max_ops:
                    lines = None
        else:
            lines = _adj_body(stages, ops, row, double, max_ops)
        if lines is not None:
            srcs[pid] = wave_source(kind, t, "\n".join(lines), double)
    uniq = list(dict.fromkeys(srcs.values()))
    handles = dict(zip(uniq, kernels_for(uniq, device, names=[WAVE_FWD_KERNEL if kind == 0 else WAVE_ADJ_KERNEL]
                                         * len(uniq))))
    return {pid: handles[src] for pid, src in srcs.items()}


@dataclass
class JitStaged:
    """Specialised kernels of one staged segment: per pass a kernel handle
    (0: the interpreting kernel runs that pass) and the op-record workspace."""

    kernels: ctypes.Array
    n_kernels: int
    ws: torch.Tensor | None = None
    rb: int = 4


_kernels: dict = {}  # (source hash, device) -> kernel handle
_lock = threading.Lock()


def cache_dir() -> Path:
    """Cubin cache: $TQ_JIT_CACHE, else ~/.cache/tyxonq_gb300/jit."""
    d = os.environ.get("TQ_JIT_CACHE")
    return Path(d) if d else Path.home() / ".cache" / "tyxonq_gb300" / "jit"


def pass_source(p, body: str, double: bool, rb: int = 4, direct: bool = False) -> str:
    """Source of one staged pass kernel: p is the pass (TilePass: t, nlow, pos),
    whose geometry is compiled in (tile loads and stores with constant
    offsets); direct: the body's last stage stores to global memory itself
    (_pass_body with direct_geo)."""
    R = "double" if double else "float"
    T2 = "double2" if double else "float2"
    t, nlow = int(p.t), int(p.nlow)
    pos = [int(p.pos[k]) for k in range(t)]
    return "\n".join([
        '#include "jit_staged.cuh"',
        "",
        "namespace tq {",
        "struct JitGeom {",
        f"  static constexpr int T = {t}, NLOW = {nlow}, THREADS = {1 << (t - rb)};",
        f"  static constexpr bool DIRECT = {'true' if direct else 'false'};",
        f"  static constexpr int POS[{t}] = {{{', '.join(map(str, pos))}}};",
        "};",
        "template <typename R, typename F>",
        "__device__ __forceinline__ void jit_body(cplx<R>* __restrict__ s, const ROp<R>* __restrict__ rops, "
        "const tq_tile_op* __restrict__ ops, uint64_t gbase, F&& on_free, typename C2<R>::T* __restrict__ gt) {",
        "  const int tid = threadIdx.x;",
        f"  constexpr int NR = {1 << rb};",
        "  cplx<R> x[NR];",
        body,
        "}",
        "}  // namespace tq",
        "",
        f'extern "C" __global__ void __launch_bounds__({1 << (t - rb)}, {2 if (t - rb) <= 8 else 1}) '
        f'{KERNEL_NAME}({T2}* psi, int n, '
        "const tq::PassArgs P, const tq_tile_stage* __restrict__ stages, "
        f"const tq_tile_op* __restrict__ ops, const tq::ROp<{R}>* __restrict__ rops_g, int dbuf) {{",
        f"  tq::jit_staged_forward_g<{R}, tq::JitGeom>(psi, n, P, stages, rops_g, dbuf, "
        f"[&](tq::cplx<{R}>* s, const tq::ROp<{R}>* rops, uint64_t gbase, auto&& on_free, {T2}* gt) "
        f"{{ tq::jit_body<{R}>(s, rops, ops, gbase, on_free, gt); }});",
        "}",
        "",
    ])


KERNEL_NAME = "tq_jit_staged_pass"


def _headers_digest() -> str:
    h = hashlib.sha256()
    for f in sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")):
        h.update(f.name.encode())
        h.update(f.read_bytes())
    return h.hexdigest()[:16]


def _build_cubin(source: str) -> bytes:
    lib = nat.load()
    inc = [str(CSRC).encode(), str(INCLUDE).encode()]
    inc_arr = (ctypes.c_char_p * len(inc))(*inc)
    out, size = ctypes.c_void_p(), ctypes.c_size_t()
    log = ctypes.create_string_buffer(8192)
    rc = lib.tq_jit_build(source.encode(), inc_arr, len(inc), ctypes.byref(out), ctypes.byref(size), log, len(log))
    if rc != 0:
        _, msg = nat.last_error()
        raise nat.TqError(rc, msg + "\n" + log.value.decode(errors="replace")[:4000])
    try:
        return ctypes.string_at(out.value, size.value)
    finally:
        lib.tq_jit_free_host(out)


def kernels_for(sources: list[str], device, names: list[str] | None = None) -> list[int]:
    """Kernel handles for the given sources on `device` (built in parallel,
    cubins cached on disk by source and header digest); names: the kernel of
    each source (default the staged pass kernel)."""
    names = names or [KERNEL_NAME] * len(sources)
    dev = torch.device(device)
    digest = _headers_digest()
    keys = [hashlib.sha256((digest + "\0" + src).encode()).hexdigest() for src in sources]
    cdir = cache_dir()
    need = [i for i, k in enumerate(keys) if (k, dev.index) not in _kernels]
    blobs: dict[int, bytes] = {}
    todo = []
    for i in need:
        f = cdir / f"{keys[i]}.cubin"
        if f.exists():
            blobs[i] = f.read_bytes()
        else:
            todo.append(i)
    if todo:
        with ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 1, 32)) as ex:
            for i, blob in zip(todo, ex.map(lambda j: _build_cubin(sources[j]), todo)):
                blobs[i] = blob
                try:
                    cdir.mkdir(parents=True, exist_ok=True)
                    tmp = cdir / f"{keys[i]}.{os.getpid()}.tmp"
                    tmp.write_bytes(blob)
                    os.replace(tmp, cdir / f"{keys[i]}.cubin")
                except OSError:
                    pass  # an unwritable cache only costs a rebuild
    lib = nat.load()
    with _lock, torch.cuda.device(dev):
        for i in need:
            if (keys[i], dev.index) in _kernels:
                continue
            h = ctypes.c_void_p()
            blob = blobs[i]
            nat.check(lib.tq_jit_load(blob, len(blob), names[i].encode(), ctypes.byref(h)))
            _kernels[(keys[i], dev.index)] = h.value
        return [_kernels[(k, dev.index)] for k in keys]


def specialise(enc, dtype, device="cuda") -> JitStaged | None:
    """Specialised kernels for the passes of an EncodedStaged program; None
    when no pass qualifies (with stages wider than 4 bits: None unless every
    pass qualifies, since the library kernel takes at most 4)."""
    double = dtype == torch.complex128
    rb = int(getattr(enc, "rb", 4))
    tmax = (12 if double else 13) + (1 if rb == 5 else 0)
    srcs, where = [], []
    for pi in range(enc.n_passes):
        p = enc.passes[pi]
        if not (9 <= int(p.t) <= tmax) or int(p.t) - rb < 5:
            continue
        direct = direct_last_ok(enc.stages_host, p, enc.stage_bits)
        geo = (int(p.nlow), [int(p.pos[k]) for k in range(int(p.t))]) if direct else None
        lines = _pass_body(enc.stages_host, enc.ops_host, p, double, enc.stage_bits, rb, direct_geo=geo)
        if lines is None:
            continue
        srcs.append(pass_source(p, "\n".join(lines), double, rb, direct=direct))
        where.append(pi)
    if not srcs or (rb > 4 and len(srcs) < sum(1 for pi in range(enc.n_passes)
                                               if enc.passes[pi].op_end > enc.passes[pi].op_begin)):
        return None
    uniq = list(dict.fromkeys(srcs))
    handles = dict(zip(uniq, kernels_for(uniq, device)))
    arr = (ctypes.c_void_p * max(enc.n_passes, 1))()
    for pi, src in zip(where, srcs):
        arr[pi] = handles[src]
    return JitStaged(arr, len(where), rb=rb)


def specialise_wide(enc, dtype, device="cuda"):
    """The segment re-encoded with 5-bit register stages and specialised kernels
    for every pass, or None (an op the 5-bit records cannot express: Pauli
    rotations with register masks above bit 3, or a pass without a kernel)."""
    from .program import encode_staged

    if enc.source is None:
        return None
    plans, gates, params, slots, n = enc.source
    if slots is not None:
        return None
    wide = encode_staged(n, plans, gates, params=params, rb=5)
    ops = wide.ops_host
    prot = ops[ops["kind"] == TOP_PROT]
    if len(prot) and int(((prot["xm"] | prot["zm"] | prot["cm"]) >= 16).sum()):
        return None
    js = specialise(wide, dtype, device)
    if js is None:
        return None
    wide.jit = js
    return wide


def run_staged(js: JitStaged, enc, psi: torch.Tensor, n: int, dtag: int, theta_ptr, stream,
               ws: dict | None = None) -> None:
    """Launch every pass of enc (specialised kernels; the interpreter for passes
    without one).  The op records of a call live in a workspace: `ws` (a dict
    owned by the caller, keyed by segment) when given -- programs shared by
    callers that run concurrently on different streams need one each -- else
    the segment's own."""
    st_d, ops_d = enc.device_tables(psi.device)
    lib = nat.load()
    n_ops = len(enc.ops_host)
    need = int(lib.tq_jit_rops_bytes(dtag, n_ops))
    buf = ws.get(id(enc)) if ws is not None else js.ws
    if buf is None or buf.numel() < need or buf.device != psi.device:
        buf = torch.empty(max(need, 16), dtype=torch.uint8, device=psi.device)
        if ws is not None:
            ws[id(enc)] = buf
        else:
            js.ws = buf
    P = ctypes.c_void_p
    nat.call("tq_jit_run_staged", js.kernels, js.rb, P(psi.data_ptr()), n, dtag, enc.passes, enc.n_passes,
             enc.stages_host.ctypes.data_as(P), P(st_d.data_ptr()), P(ops_d.data_ptr()), n_ops, theta_ptr,
             P(buf.data_ptr()), buf.numel(), stream)
