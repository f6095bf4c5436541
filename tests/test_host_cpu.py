"""Host-side logic on CPU: the C ABI library exports every declared symbol,
the tile planner and fusion preserve circuit semantics, the tile-op encoding
matches the device layout, and Hamiltonian packing matches the reference's
dense Pauli matrices.  No GPU compute."""
import ctypes
import math
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import sv
from tyxonq_gb300 import _build, _native
from tyxonq_gb300 import program as P
from tyxonq_gb300.hamiltonian import PauliSum, random_pauli_sum
from tyxonq_gb300.ir import Gate, lower_ops
from tyxonq_gb300.workloads import random_circuit

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        for m in re.finditer(r"TQ_API\s+[\w\s\*]+?\b(tq_\w+)\s*\(", h.read_text()):
            syms.add(m.group(1))
    return syms


def test_library_builds_and_exports_every_declared_symbol():
    lib_path = _build.build()
    lib = ctypes.CDLL(str(lib_path))
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/*.h but not exported"
    # and the Python binding covers exactly the declared ABI
    assert syms == set(_native.SIGNATURES), syms ^ set(_native.SIGNATURES)


def test_host_validation_without_gpu():
    lib = _native.load()
    # argument checks run before any device work
    assert lib.tq_sv_init_basis(None, 99, 0, 0, None) == -1
    assert lib.tq_sv_apply_1q(ctypes.c_void_p(16), 4, 0, 7, (ctypes.c_double * 8)(), None) == -3
    assert lib.tq_sv_apply_1q(ctypes.c_void_p(16), 4, 5, 0, (ctypes.c_double * 8)(), None) == -1
    code, msg = _native.last_error()
    assert code == -1 and "dtype" in msg
    assert lib.tq_sv_sample_workspace_bytes(20, 8192) > 0
    assert lib.tq_sv_tile_max_bits(0) == 14 and lib.tq_sv_tile_max_bits(1) == 13


class _CTileOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32), ("slot", ctypes.c_int32),
                ("xm", ctypes.c_uint32), ("zm", ctypes.c_uint32), ("cm", ctypes.c_uint32), ("gxm", ctypes.c_uint32),
                ("gzm", ctypes.c_uint32), ("gcm", ctypes.c_uint32), ("gny", ctypes.c_int32), ("pidx", ctypes.c_int32),
                ("pscale", ctypes.c_double), ("gcoef", ctypes.c_double), ("zo", ctypes.c_uint32),
                ("fuse_next", ctypes.c_int32), ("zg", ctypes.c_uint64), ("mf", ctypes.c_float * 32),
                ("md", ctypes.c_double * 32)]


def test_tile_op_layout_matches_c_struct():
    assert ctypes.sizeof(_CTileOp) == P.TILE_OP_DTYPE.itemsize
    for name in P.TILE_OP_DTYPE.names:
        assert getattr(_CTileOp, name).offset == P.TILE_OP_DTYPE.fields[name][1], name
    assert ctypes.sizeof(P.TilePass) == 80


def _oracle_apply(psi, g: Gate, n):
    if g.kind in ("u1", "d1", "u2", "uk"):
        return sv.apply_kq(psi, g.mat, list(g.qubits), n)
    if g.kind in ("cx", "cz", "swap"):
        return sv.apply_kq(psi, sv.gate_matrix(g.kind), list(g.qubits), n)
    if g.kind == "prot":
        U = sv.g_rot(g.rot[1], np.kron(*[sv.PAULI[p] for _, p in g.pauli]) if len(g.pauli) == 2 else sv.PAULI[g.pauli[0][1]])
        return sv.apply_kq(psi, U, list(g.qubits), n)
    raise KeyError(g.kind)


class _C:
    def __init__(self, n, ops):
        self.num_qubits = n
        self.ops = ops


@pytest.mark.parametrize("n,t", [(6, 4), (10, 7), (12, 8), (14, 9)])
def test_planner_preserves_semantics(n, t):
    ops = random_circuit(n, 12, seed=n)
    gates, _ = lower_ops(_C(n, ops), mode="run")
    ref = sv.init_state(n)
    for g in gates:
        ref = _oracle_apply(ref, g, n)
    segs = P.plan_passes(gates, n, t, nlow=3)
    psi = sv.init_state(n)
    seen = []
    for s in segs:
        assert s.kind == "tiles"
        for pp in s.passes:
            low = set(range(n - pp.nlow, n))
            assert pp.nlow >= 1 and len(pp.qubits) <= t and low <= set(pp.qubits)
            for i in pp.gates:
                assert set(gates[i].qubits) <= set(pp.qubits)
                psi = _oracle_apply(psi, gates[i], n)
                seen.append(i)
    assert sorted(seen) == list(range(len(gates)))
    np.testing.assert_allclose(psi, ref, atol=1e-12)


def test_fusion_preserves_semantics():
    n = 6
    ops = random_circuit(n, 10, seed=9)
    gates, _ = lower_ops(_C(n, ops), mode="run")
    ref = sv.init_state(n)
    for g in gates:
        ref = _oracle_apply(ref, g, n)
    fused = P.fuse_pass(gates)
    assert len(fused) < len(gates)
    psi = sv.init_state(n)
    for g in fused:
        psi = _oracle_apply(psi, g, n)
    np.testing.assert_allclose(psi, ref, atol=1e-12)


def _emulate_tiles(psi, n, enc):
    """NumPy emulation of k_tile_forward on encoded passes (complex128 path)."""
    psi = psi.copy()
    ops = enc.ops_host
    for p in range(enc.n_passes):
        pa = enc.passes[p]
        t = pa.t
        pos = [pa.pos[j] for j in range(t)]
        nonloc = [b for b in range(n) if b not in pos]
        for g in range(1 << (n - t)):
            base = sum(((g >> k) & 1) << b for k, b in enumerate(nonloc))
            idx = np.array([base + sum(((j >> k) & 1) << pos[k] for k in range(t)) for j in range(1 << t)])
            s = psi[idx]
            for o in ops[pa.op_begin:pa.op_end]:
                s = _apply_local(s, o, t, _zs(o, base))
            psi[idx] = s
    return psi


def _emulate_staged(psi, n, enc):
    """NumPy emulation of k_staged_forward: per stage, every thread's 16
    register amplitudes get the stage's ops in register-bit space."""
    psi = psi.copy()
    for p in range(enc.n_passes):
        pa = enc.passes[p]
        t = pa.t
        pos = [pa.pos[j] for j in range(t)]
        nonloc = [b for b in range(n) if b not in pos]
        for g in range(1 << (n - t)):
            base = sum(((g >> k) & 1) << b for k, b in enumerate(nonloc))
            idx = np.array([base + sum(((j >> k) & 1) << pos[k] for k in range(t)) for j in range(1 << t)])
            s = psi[idx]
            for st in enc.stages_host[pa.op_begin:pa.op_end]:
                bits = [int(b) for b in st["bits"]]
                rest = [b for b in range(t) if b not in bits]
                for tid in range(1 << (t - 4)):
                    b0 = sum(((tid >> k) & 1) << b for k, b in enumerate(rest))
                    ridx = np.array([b0 + sum(((i >> k) & 1) << bits[k] for k in range(4)) for i in range(16)])
                    v = s[ridx]
                    for o in enc.ops_host[st["op_begin"]:st["op_end"]]:
                        v = _apply_local(v, o, 4, _zs(o, base, b0))
                    s[ridx] = v
            psi[idx] = s
    return psi


def _zs(o, gbase, tbase=0):
    par = (bin(int(gbase) & int(o["zg"])).count("1") + bin(int(tbase) & int(o["zo"])).count("1")) & 1
    return -1.0 if par else 1.0


def _apply_local(s, o, t, zs=1.0):
    s = s.copy()
    if True:
        if True:
            if True:
                m = o["md"][0::2] + 1j * o["md"][1::2]
                a, b = int(o["a"]), int(o["b"])
                j = np.arange(1 << t)
                if o["kind"] == 1:
                    lo = j[((j >> a) & 1) == 0]
                    hi = lo | (1 << a)
                    x, y = s[lo].copy(), s[hi].copy()
                    s[lo], s[hi] = m[0] * x + m[1] * y, m[2] * x + m[3] * y
                elif o["kind"] == 2:
                    s = np.where((j >> a) & 1, m[1], m[0]) * s
                elif o["kind"] == 3:
                    base4 = j[(((j >> a) & 1) == 0) & (((j >> b) & 1) == 0)]
                    ids = [base4, base4 | (1 << b), base4 | (1 << a), base4 | (1 << a) | (1 << b)]
                    X = np.stack([s[i] for i in ids])
                    Y = m[:16].reshape(4, 4) @ X
                    for r in range(4):
                        s[ids[r]] = Y[r]
                elif o["kind"] in (4, 5, 6):
                    base4 = j[(((j >> a) & 1) == 0) & (((j >> b) & 1) == 0)]
                    if o["kind"] == 4:
                        i0, i1 = base4 | (1 << a), base4 | (1 << a) | (1 << b)
                        s[i0], s[i1] = s[i1].copy(), s[i0].copy()
                    elif o["kind"] == 6:
                        i0, i1 = base4 | (1 << a), base4 | (1 << b)
                        s[i0], s[i1] = s[i1].copy(), s[i0].copy()
                    else:
                        s[base4 | (1 << a) | (1 << b)] *= -1
                elif o["kind"] == 7:
                    xm, zm, cm = int(o["xm"]), int(o["zm"]), int(o["cm"])
                    c, w = m[0], m[1] * zs
                    sgn = np.array([-1 if bin(int(x) & zm).count("1") % 2 else 1 for x in j])
                    on = (j & cm) == cm
                    new = c * s + w * sgn[j ^ xm] * s[j ^ xm]
                    s = np.where(on, new, s)
                else:
                    raise AssertionError("unexpected op kind")
    return s


def _op_matrix_local(o, theta, t):
    """Dense 2^t x 2^t action of one encoded op (register or tile space), with
    device-side angles taken from theta."""
    dim = 1 << t
    M = np.zeros((dim, dim), dtype=np.complex128)
    o = o.copy()
    if o["pidx"] >= 0:
        a = o["pscale"] * theta[o["pidx"]]
        if o["kind"] == 7:
            ny = bin(int(o["xm"]) & int(o["zm"])).count("1") & 3
            w = -1j * np.sin(a / 2) * (1j ** ny)
            o["md"][0:4] = [np.cos(a / 2), 0, w.real, w.imag]
        elif o["kind"] == 2:
            o["md"][0:4] = [1, 0, np.cos(a), np.sin(a)]
    for c in range(dim):
        e = np.zeros(dim, dtype=np.complex128)
        e[c] = 1
        M[:, c] = _apply_local(e, o, t)
    return M


@pytest.mark.parametrize("rb", [3, 4])
def test_staged_adjoint_encoding_emulated_matches_oracle_gradient(rb):
    """Reverse sweep over register stages (rb bits, 2^rb amplitudes per thread)
    as the wave adjoint kernel runs it."""
    from tyxonq_gb300.batch import structure_gates
    from tyxonq_gb300.workloads import batched_vqe

    inst = batched_vqe(1, seed=17, n_range=(10, 10), depth_range=(2, 2), terms_range=(20, 20))[0]
    n = inst.n
    gates, params = structure_gates(inst.structure())
    rg = list(reversed(gates))
    G = len(gates)
    rparams = {G - 1 - gi: v for gi, v in params.items()}
    slots = {ri: rparams[ri][0] for ri in rparams}
    e_ref, g_ref = sv.grad_adjoint(n, [(nm, list(qs), p, 1.0) for nm, qs, p in inst.structure()], inst.theta,
                                   inst.H.codes, inst.H.coeffs)
    psi, _ = sv.run_ops(n, inst.ops())
    lam = sv.apply_pauli_sum(psi, inst.H.codes, inst.H.coeffs)
    grad = np.zeros(inst.n_params)
    for s in P.plan_passes(rg, n, 9, max_ops=64):
        for pp in s.passes:
            enc = P.encode_staged(n, [pp], rg, params=rparams, slots=slots, rb=rb)
            pa = enc.passes[0]
            t = pa.t
            pos = [pa.pos[j] for j in range(t)]
            nonloc = [b for b in range(n) if b not in pos]
            for gidx in range(1 << (n - t)):
                base = sum(((gidx >> k) & 1) << b for k, b in enumerate(nonloc))
                idx = np.array([base + sum(((j >> k) & 1) << pos[k] for k in range(t)) for j in range(1 << t)])
                sp, sl = psi[idx], lam[idx]
                for st in enc.stages_host[pa.op_begin:pa.op_end]:
                    bits = [int(b) for b in st["bits"]][:rb]
                    assert all(b >= 0 for b in bits) and all(int(b) == -1 for b in st["bits"][rb:])
                    rest = [b for b in range(t) if b not in bits]
                    ops = enc.ops_host[st["op_begin"]:st["op_end"]]
                    mats = [_op_matrix_local(o, inst.theta, rb) for o in ops]
                    for tid in range(1 << (t - rb)):
                        b0 = sum(((tid >> k) & 1) << b for k, b in enumerate(rest))
                        ridx = np.array([b0 + sum(((i >> k) & 1) << bits[k] for k in range(rb)) for i in range(1 << rb)])
                        x, y = sp[ridx], sl[ridx]
                        for o, M in zip(ops, mats):
                            if o["slot"] >= 0:
                                i = np.arange(1 << rb)
                                on = (i & int(o["gcm"])) == int(o["gcm"])
                                sg = np.array([-1 if bin(k & int(o["gzm"])).count("1") % 2 else 1 for k in i])
                                v = (1j ** int(o["gny"])) * sg * x
                                grad[o["slot"]] += o["gcoef"] * np.sum(np.imag(np.conj(y[i ^ int(o["gxm"])]) * v)[on])
                            x = M.conj().T @ x
                            y = M.conj().T @ y
                        sp[ridx], sl[ridx] = x, y
                psi[idx], lam[idx] = sp, sl
    np.testing.assert_allclose(grad, g_ref, atol=1e-10)


@pytest.mark.parametrize("staged", [False, True])
def test_wide_pauli_rotations_with_nonlocal_z_emulated(staged):
    """UCC rotations carry long Z strings: only their X/Y qubits are made
    local, the other Z factors enter as per-tile / per-thread signs."""
    from tyxonq_gb300 import chem
    from tyxonq_gb300.ir import pauli_rotation

    n_orb = 5
    n = 2 * n_orb
    pg, npar, ex = chem.uccsd_param_gates(n_orb, 2)
    rng = np.random.default_rng(3)
    th = rng.uniform(-0.7, 0.7, npar)
    gates = [pauli_rotation(p.gate.pauli, p.scale * th[p.param]) for p in pg][:120]
    psi0 = sv.init_state(n, chem.hf_basis(n, 1))
    ref = psi0.copy()
    for g in gates:
        M = np.array([[1.0 + 0j]])
        for q, s in g.pauli:
            M = np.kron(M, sv.PAULI[s])
        a = g.rot[1]
        ref = sv.apply_kq(ref, np.cos(a / 2) * np.eye(M.shape[0]) - 1j * np.sin(a / 2) * M, [q for q, _ in g.pauli], n)
    t = 9 if staged else 6
    segs = P.plan_passes(gates, n, t, nlow=2)
    assert all(s.kind == "tiles" for s in segs)
    psi = psi0.copy()
    wide = 0
    for s in segs:
        if staged:
            enc = P.encode_staged(n, s.passes, gates)
            wide += int((enc.ops_host["zg"] != 0).sum() + (enc.ops_host["zo"] != 0).sum())
            psi = _emulate_staged(psi, n, enc)
        else:
            enc, _ = P.encode_passes(n, s.passes, gates, fuse=False, nlow=2)
            wide += int((enc.ops_host["zg"] != 0).sum())
            psi = _emulate_tiles(psi, n, enc)
    assert wide > 0
    np.testing.assert_allclose(psi, ref, atol=1e-12)


def test_staged_encoding_emulated_matches_oracle():
    n = 10
    ops = random_circuit(n, 5, seed=12)
    ops += [("rxx", 0, 9, 0.4), ("cry", 3, 8, 1.3), ("iswap", 2, 7)]
    gates, _ = lower_ops(_C(n, ops), mode="run")
    ref = sv.init_state(n)
    for g in gates:
        ref = _oracle_apply(ref, g, n) if g.kind != "u2" or g.rot is None else sv.apply_kq(ref, g.mat, list(g.qubits), n)
    segs = P.plan_passes(gates, n, 9, nlow=3)
    psi = sv.init_state(n)
    for s in segs:
        enc = P.encode_staged(n, s.passes, [P._canon(g) for g in gates])
        assert len(enc.stages_host) < sum(len(pp.gates) for pp in s.passes)
        psi = _emulate_staged(psi, n, enc)
    np.testing.assert_allclose(psi, ref, atol=1e-12)


@pytest.mark.parametrize("fuse", [False, True])
def test_encoded_tiles_emulated_match_oracle(fuse):
    n = 8
    ops = random_circuit(n, 6, seed=4)
    gates, _ = lower_ops(_C(n, ops), mode="run")
    ref = sv.init_state(n)
    for g in gates:
        ref = _oracle_apply(ref, g, n)
    segs = P.plan_passes(gates, n, 5, nlow=2)
    psi = sv.init_state(n)
    for s in segs:
        enc, _ = P.encode_passes(n, s.passes, gates, fuse=fuse, nlow=2)
        psi = _emulate_tiles(psi, n, enc)
    np.testing.assert_allclose(psi, ref, atol=1e-12)


def test_pauli_packing_matches_dense_reference_matrices():
    rng = np.random.default_rng(11)
    n = 5
    H = random_pauli_sum(n, 30, rng)
    g, t = H.pack()
    assert int(g["n_terms"].sum()) == 30
    Hd = sv.dense_hamiltonian(H.codes, H.coeffs)
    # rebuild the operator from packed masks: P|i> = w (-1)^{popc(i&zy)} |i^flip>
    M = np.zeros_like(Hd)
    for gr in g:
        for k in range(gr["first_term"], gr["first_term"] + gr["n_terms"]):
            w = t[k]["w_re"] + 1j * t[k]["w_im"]
            for i in range(1 << n):
                sgn = -1 if bin(i & int(t[k]["zy"])).count("1") % 2 else 1
                M[i ^ int(gr["flip"]), i] += w * sgn
    np.testing.assert_allclose(M, Hd, atol=1e-12)


def test_term_formats_agree():
    terms = [(0.5, [("X", 0), ("Z", 2)]), (-1.25, [("Y", 1)]), (2.0, [])]
    A = PauliSum.from_terms(3, terms)
    B = PauliSum.from_codes([[1, 0, 3], [0, 2, 0], [0, 0, 0]], [0.5, -1.25, 2.0])
    C = PauliSum.from_qubit_operator_terms(3, {((0, "X"), (2, "Z")): 0.5, ((1, "Y"),): -1.25, (): 2.0})
    for X in (B, C):
        np.testing.assert_array_equal(np.sort(A.codes, axis=0), np.sort(X.codes, axis=0))
        assert math.isclose(A.one_norm(), X.one_norm())


def test_lowering_follows_reference_dispatch():
    ops = [("h", 0), ("y", 1), ("z", 1), ("t", 0), ("cry", 0, 1, 0.3), ("measure_z", 0), ("barrier", 0, 1),
           ("rz", 1, 0.7), ("cx", 1, 1), ("foo", 0)]
    g_state, m_state = lower_ops(_C(2, ops), mode="state")
    g_run, m_run = lower_ops(_C(2, ops), mode="run")
    assert [g.kind for g in g_state] == ["u1", "d1"]  # y/z/t/cry ignored, cx(q,q) no-op
    assert [g.kind for g in g_run] == ["u1", "u2", "d1"]  # run() has cry
    assert m_run == [0] and m_state == []
    # a Kraus op whose operators are not cached is skipped (engine.py:150-151); pulses are not supported
    assert lower_ops(_C(1, [("kraus", 0, "k")]), mode="run")[0] == []
    c = _C(1, [("kraus", 0, "k", 0.3)])
    c._kraus_cache = {"k": [np.eye(2)]}
    (g,), _ = lower_ops(c, mode="state")
    assert g.kind == "kraus" and g.qubits == (0,) and g.status == 0.3 and len(g.kraus) == 1
    with pytest.raises(NotImplementedError):
        lower_ops(_C(1, [("pulse", 0, "p")]), mode="run")


def test_excitation_records_layout_and_masks():
    """tq_excitation records: the C struct's 48-byte layout, masks splitting
    the excitation bits, ascending bit list, Z mask disjoint from them."""
    from tyxonq_gb300 import chem
    from tyxonq_gb300.excitation import EXCITATION_DTYPE, excitation_records

    assert EXCITATION_DTYPE.itemsize == 48
    n = 12
    ex, _ = chem.uccsd_excitations(2, 4)
    rec = excitation_records(n, ex)
    for r, f in zip(rec, ex):
        allbits = sum(1 << x for x in f)
        assert int(r["m_neg"]) | int(r["m_pos"]) == allbits and int(r["m_neg"]) & int(r["m_pos"]) == 0
        assert int(r["zmask"]) & allbits == 0 and r["sign"] in (-1, 1) and r["k"] == len(f)
        assert list(r["bits"][:len(f)]) == sorted(f)
    with pytest.raises(ValueError):
        excitation_records(n, [(0, 0)])
    with pytest.raises(ValueError):
        excitation_records(n, [(0, 1, 2)])


def test_staged_adjoint_cold_gate_classification():
    """Gates that may lack a register routine in the staged adjoint: rotations
    with two or more X/Y qubits, ZZ rotations, controlled rotations, dense
    two-qubit unitaries."""
    from tyxonq_gb300.adjoint import _cold_in_staged_adjoint
    from tyxonq_gb300.ir import Gate, _rot_gate, pauli_rotation
    from tyxonq_gb300.program import _canon

    assert not _cold_in_staged_adjoint(_canon(_rot_gate("ry", (0,), 0.3)))
    assert _cold_in_staged_adjoint(_canon(_rot_gate("rzz", (0, 3), 0.3)))
    assert not _cold_in_staged_adjoint(_canon(_rot_gate("rz", (2,), 0.3)))
    assert not _cold_in_staged_adjoint(_canon(Gate("cx", (0, 1))))
    assert not _cold_in_staged_adjoint(_canon(pauli_rotation(((0, "X"), (2, "Z"), (5, "Z")), 0.2)))
    assert _cold_in_staged_adjoint(_canon(_rot_gate("rxx", (0, 3), 0.3)))
    assert _cold_in_staged_adjoint(_canon(pauli_rotation(((0, "X"), (2, "Z"), (5, "Y")), 0.2)))


def test_staged_reverse_tables_cover_every_parametrised_op():
    """Host tables of the single-state staged reverse sweep (built on the CPU
    here): one work item per (adjoint pass, tile), disjoint partial ranges, a
    reduction row for every parametrised op, and reduction launches that never
    write one gradient twice (a parameter shared by several rotations)."""
    import torch

    from tyxonq_gb300.adjoint import ParamGate, _StagedReverse
    from tyxonq_gb300.ir import Gate, _rot_gate, pauli_rotation
    from tyxonq_gb300.waves import WAVE_ITEM_DTYPE

    n = 15
    pg, p = [], 0
    for layer in range(2):
        for q in range(n):
            pg.append(ParamGate(_rot_gate("ry", (q,), 0.0), p))
            p += 1
        for q in range(n - 1):
            pg.append(ParamGate(Gate("cx", (q, q + 1))))
    shared = p
    pg.append(ParamGate(pauli_rotation(((0, "X"), (7, "Z")), 0.0), shared, 2.0))
    pg.append(ParamGate(pauli_rotation(((3, "Y"), (9, "Z")), 0.0), shared, -1.0))
    p += 1
    sr = _StagedReverse(n, pg, p, torch.complex64, "cpu")
    items = np.frombuffer(sr.items_dev.numpy().tobytes(), dtype=WAVE_ITEM_DTYPE)
    assert sr.t == 13 and len(items) == sum(c for _, c in sr.runs) == len(sr.runs) * (1 << (n - sr.t))
    assert np.all(items["psi_off"] == 0) and np.all(items["lam_off"] == 1 << n)
    # every tile of every pass owns its own block of partial slots
    ranges = sorted(zip(items["part_off"], items["pass"]))
    assert len({int(o) for o, _ in ranges}) == len(items)
    first = sr.r_first.numpy()
    count, stride, out = sr.r_count.numpy(), sr.r_stride.numpy(), sr.r_out.numpy()
    assert np.all(count == 1 << (n - sr.t))
    assert np.all(first + (count - 1) * stride < sr.partials.numel())
    # one row per parametrised op; the shared parameter has two rows in different launches
    assert len(out) == sum(1 for g in pg if g.param is not None)
    for b, c in sr.layers:
        lay = out[b:b + c]
        assert len(set(lay.tolist())) == len(lay)
    assert sorted(set(out.tolist())) == list(range(p))


def test_specialised_sources_compile_with_nvrtc():
    """Circuit-specialised kernels are generated on the host and compiled by the
    library's NVRTC entry point (no GPU needed): a staged pass of a 28-qubit
    random circuit (real, diagonal, i-symmetric and general 2x2 routines), the
    same pass re-encoded with 5-bit stages, and the wave forward and adjoint
    bodies of an HEA pass."""
    import collections
    import time

    import torch

    from tyxonq_gb300 import jit as J
    from tyxonq_gb300.workloads import hea_rz_ops_params

    class _C:
        def __init__(self, n, o):
            self.num_qubits, self.ops = n, o

    gates, _ = lower_ops(_C(28, random_circuit(28, 40, seed=1)), mode="run")
    prog = P.compile_forward(gates, 28, torch.complex64, t=13)
    enc = [o for k, o in prog.segments if k == "staged"][0]
    used = collections.Counter()
    srcs = []
    for pi in range(enc.n_passes):
        lines = J._pass_body(enc.stages_host, enc.ops_host, enc.passes[pi], False, enc.stage_bits, 4)
        assert lines is not None
        for ln in lines:
            used.update(re.findall(r"([a-z_0-9]+)<R, NR", ln))
        if pi == 3:
            srcs.append(J.pass_source(enc.passes[pi], "\n".join(lines), False, 4))
    # real and diagonal single-qubit products take the cheap routines
    assert used["j_ureal"] > 0 and used["r_d1"] > 0 and used["r_perm"] > 0
    plans, g, params, slots, n = enc.source
    wide = P.encode_staged(n, plans, g, params=params, rb=5)
    p = wide.passes[0]
    srcs.append(J.pass_source(p, "\n".join(J._pass_body(wide.stages_host, wide.ops_host, p, False,
                                                                 wide.stage_bits, 5)), False, 5))
    n = 16
    struct = hea_rz_ops_params(n, 2)
    th = np.random.default_rng(0).uniform(-1, 1, 64)
    ops = [(nm, *qs) if pp is None else (nm, *qs, float(th[pp])) for nm, qs, pp in struct]
    hg, _ = lower_ops(_C(n, ops), mode="run")
    henc = [o for k, o in P.compile_forward(hg, n, torch.complex64, t=13).segments if k == "staged"][0]
    hp = henc.passes[0]
    row = (int(hp.t), 0, int(hp.op_begin), int(hp.op_end), 0)
    srcs.append(J.wave_source(0, 13, "\n".join(J._pass_body(henc.stages_host, henc.ops_host, hp, False)), False))
    srcs.append(J.wave_source(2, 13, "\n".join(J._adj_body(henc.stages_host, henc.ops_host, row, False, 10**6)),
                              False))
    from concurrent.futures import ThreadPoolExecutor

    t0 = time.time()
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        blobs = list(ex.map(J._build_cubin, srcs))
    assert all(len(b) > 1000 for b in blobs)
    assert time.time() - t0 < 300


def test_commuted_diagonals_preserve_the_state_and_meet_their_neighbours():
    """commute_diagonals moves diagonal single-qubit gates only past gates they
    commute with (CZ, CX on its control, other qubits, other diagonals): the
    state is the oracle's for the original order, and most diagonals of the
    28-qubit random-circuit generator end next to a single-qubit gate on their
    qubit (so the encoder fuses them)."""
    n = 9
    gates, _ = lower_ops(_C(n, random_circuit(n, 24, seed=4)), mode="run")
    order = P.commute_diagonals(gates)
    assert sorted(order) == list(range(len(gates)))
    psi0 = np.zeros(1 << n, dtype=np.complex128)
    psi0[0] = 1
    a, b = psi0.copy(), psi0.copy()
    for g in gates:
        a = _oracle_apply(a, g, n)
    for i in order:
        b = _oracle_apply(b, gates[i], n)
    np.testing.assert_allclose(b, a, atol=1e-12)
    moved = [gates[i] for i in order]
    d1 = [k for k, g in enumerate(moved) if g.kind == "d1"]
    near = sum(1 for k in d1 if any(0 <= k + d < len(moved) and moved[k + d].kind == "u1"
                                    and moved[k + d].qubits == moved[k].qubits for d in (-1, 1)))
    assert near >= len(d1) // 2


def test_checked_variant_builds_and_reports_status():
    """The -DTQ_CHECKED variant compiles and exports every declared symbol; the
    normal build answers tq_check_status with 0 (nothing recorded, unchecked)."""
    lib = _native.load()
    site, index = ctypes.c_uint(7), ctypes.c_longlong(7)
    assert lib.tq_check_status(ctypes.byref(site), ctypes.byref(index)) == 0
    assert site.value == 0 and index.value == 0
    path = _build.build(checked=True)
    chk = ctypes.CDLL(str(path))
    for name in header_symbols():
        assert hasattr(chk, name), name


def test_tuned_tile_widths_are_read_from_the_cache_file(tmp_path, monkeypatch):
    """tile_bits_for reads the single-state tuner's cache file once per process
    (TYXONQ_GB300_TUNE) and falls back to the shared-memory defaults."""
    import json

    import torch

    from tyxonq_gb300 import autotune as A

    f = tmp_path / "tune.json"
    f.write_text(json.dumps({"fwd:24:c64": 11, "adj:24:c64": 10}))
    monkeypatch.setenv("TYXONQ_GB300_TUNE", str(f))
    monkeypatch.setattr(A, "_TUNED", {})
    monkeypatch.setattr(A, "_LOADED", False)
    assert A.tile_bits_for(24, torch.complex64) == 11
    assert A.tile_bits_for(24, torch.complex64, adjoint=True) == 10
    assert A.tile_bits_for(22, torch.complex64) == 13  # untuned: 2^13 complex64 amplitudes
    assert A.tile_bits_for(22, torch.complex128, adjoint=True) == 11
    A.set_tile_bits(9, torch.complex64, False, 7)
    out = tmp_path / "out.json"
    A.save(out)
    assert json.loads(out.read_text())["fwd:9:c64"] == 7


def test_op_record_jobs_one_per_pass_and_instance():
    """rop_jobs: one job per distinct (kind, pass, instance angles) of the
    forward and adjoint launches, consecutive record ranges, and every item
    pointing at its job's records (group_begin) with its op count (group_count);
    H psi items are left alone."""
    from tyxonq_gb300.program import STAGE_DTYPE
    from tyxonq_gb300.waves import rop_jobs

    stages = np.zeros(6, dtype=STAGE_DTYPE)
    stages["op_begin"] = [0, 3, 5, 9, 12, 20]
    stages["op_end"] = [3, 5, 9, 12, 20, 21]
    passes = [(12, 5, 0, 2, [0] * 16), (12, 5, 2, 4, [0] * 16), (12, 5, 4, 6, [0] * 16)]
    # items: (psi_off, lam_off, pass, tile, theta_off, part_off, n, group_begin, group_count, basis_lo)
    items = [(0, 0, 0, t, 0, 0, 14, 0, 0, -1) for t in range(4)]  # instance A, pass 0
    items += [(0, 0, 0, t, 40, 0, 14, 0, 0, -1) for t in range(4)]  # instance B (other angles), pass 0
    items += [(0, 0, 0, t, 0, t, 14, 7, 3, -1) for t in range(4)]  # H psi items
    items += [(0, 0, 2, t, 0, 0, 14, 0, 0, -1) for t in range(4)]  # instance A, adjoint pass 2
    launches = [("run", 0, 0, 8), ("run", 1, 8, 4), ("run", 2, 12, 4)]
    out, jobs = rop_jobs(items, launches, passes, stages)
    assert len(jobs) == 3
    assert list(jobs["op_begin"]) == [0, 0, 12] and list(jobs["n_ops"]) == [5, 5, 9]
    assert list(jobs["theta_off"]) == [0, 40, 0] and list(jobs["flags"]) == [0, 0, 1]
    assert list(jobs["out_record"]) == [0, 5, 10]
    assert all(r[7] == 0 and r[8] == 5 for r in out[0:4])
    assert all(r[7] == 5 and r[8] == 5 for r in out[4:8])
    assert out[8:12] == items[8:12]  # H psi items keep their group fields
    assert all(r[7] == 10 and r[8] == 9 for r in out[12:16])


def test_tile_group_order_keeps_partner_runs_and_groups_one_term_classes():
    """order_groups_for_tiles only permutes groups: partner-tile runs (flip >> 12)
    stay contiguous, and inside a run one-term groups come ordered by their
    term's Z/Y bits 8..11, the multi-term groups after them."""
    from tyxonq_gb300.hamiltonian import order_groups_for_tiles, random_pauli_sum, sort_terms_by_class

    H = random_pauli_sum(16, 400, np.random.default_rng(3))
    g, t = H.pack()
    t = sort_terms_by_class(g, t, 12)
    o = order_groups_for_tiles(g, t, 12)
    assert sorted(map(tuple, o.tolist())) == sorted(map(tuple, g.tolist()))
    hi = o["flip"] >> np.uint64(12)
    assert (np.diff(hi.astype(np.int64)) >= 0).all()
    for h in np.unique(hi):
        run = o[hi == h]
        one = run["n_terms"] == 1
        cls = np.where(one, (t["zy"][run["first_term"]] >> np.uint64(8)) & np.uint64(15), 16).astype(np.int64)
        assert (np.diff(cls) >= 0).all()


def test_parametrised_program_with_commuted_diagonals_emulated_matches_oracle():
    """compile_forward of a parametrised circuit (angles read from theta on the
    device) reorders diagonal gates and remaps the parameter table; the staged
    program, emulated with the device-side angle formulas, gives the oracle's
    state up to a global phase."""
    import torch

    from tyxonq_gb300.batch import structure_gates

    n, depth = 10, 3
    rng = np.random.default_rng(7)
    struct = []
    for layer in range(depth):
        for q in range(n):
            struct.append(("h", (q,), None))
        for q in range(0, n - 1, 2 if layer % 2 else 1):
            struct.append(("cz" if q % 3 else "cx", (q, q + 1), None))
        for q in range(n):  # diagonals behind CZ / CX controls: moved back to the H of their qubit
            struct.append(("rz", (q,), len(struct)))
    # parameter indices 0, 1, ... in gate order
    struct2, n_par = [], 0
    for nm, qs, p in struct:
        struct2.append((nm, qs, None if p is None else n_par))
        n_par += p is not None
    theta = rng.uniform(-3, 3, n_par)
    gates, params = structure_gates(struct2)
    order = P.commute_diagonals([P._canon(g) for g in gates])
    assert order != list(range(len(gates)))  # the diagonals do move here
    prog = P.compile_forward(gates, n, torch.complex128, t=9, params=params)
    psi = sv.init_state(n)
    for kind, enc in prog.segments:
        assert kind == "staged"
        psi = psi.copy()
        for pi in range(enc.n_passes):
            pa = enc.passes[pi]
            t = pa.t
            pos = [pa.pos[j] for j in range(t)]
            nonloc = [b for b in range(n) if b not in pos]
            for g in range(1 << (n - t)):
                base = sum(((g >> k) & 1) << b for k, b in enumerate(nonloc))
                idx = np.array([base + sum(((j >> k) & 1) << pos[k] for k in range(t)) for j in range(1 << t)])
                s = psi[idx]
                for st in enc.stages_host[pa.op_begin:pa.op_end]:
                    bits = [int(b) for b in st["bits"]]
                    rest = [b for b in range(t) if b not in bits]
                    for tid in range(1 << (t - 4)):
                        b0 = sum(((tid >> k) & 1) << b for k, b in enumerate(rest))
                        ridx = np.array([b0 + sum(((i >> k) & 1) << bits[k] for k in range(4)) for i in range(16)])
                        v = s[ridx]
                        for o in enc.ops_host[st["op_begin"]:st["op_end"]]:
                            v = _op_matrix_local(o, theta, 4) @ v if o["pidx"] >= 0 else \
                                _apply_local(v, o, 4, _zs(o, base, b0))
                        s[ridx] = v
                psi[idx] = s
    ops = [(nm, *qs) if p is None else (nm, *qs, float(theta[p])) for nm, qs, p in struct2]
    ref, _ = sv.run_ops(n, ops, mode="run")
    assert abs(abs(np.vdot(ref, psi)) - 1.0) < 1e-10


@pytest.mark.parametrize("ops,routine", [
    ([("h", 9), ("ry", 9, 0.3)], "j_ureal<"),  # real factors: a real 2x2
    ([("rz", 9, 0.2), ("s", 9)], "r_d1<"),  # diagonal factors: a diagonal
    ([("rx", 9, 0.4)], "r_ri<"),  # c I - i s X
    ([("h", 9), ("rz", 9, 0.7)], "r_u1<"),  # a complex diagonal times a real matrix: general
])
def test_specialised_routine_follows_the_factors_shapes(ops, routine):
    """The generated pass body applies a run of single-qubit ops on one register
    bit with the cheapest routine its factors allow (register-routine choice of
    the circuit-specialised kernels)."""
    import torch

    from tyxonq_gb300 import jit as J

    n = 10
    gates, _ = lower_ops(_C(n, ops), mode="run")
    prog = P.compile_forward(gates, n, torch.complex64, t=9)
    enc = [o for k, o in prog.segments if k == "staged"][0]
    body = "\n".join(J._pass_body(enc.stages_host, enc.ops_host, enc.passes[0], False))
    names = set(re.findall(r"([a-z_0-9]+<)R, NR", body))
    assert names == {routine}, names


def test_fused_program_cache_keys_tell_circuits_apart():
    """The engine's fused-program cache is keyed by every gate's kind, qubits,
    matrix and angle: circuits that differ in one angle, one qubit or one gate
    kind get different keys; the same circuit lowered twice gets the same key."""
    def key(ops, n=4):
        gates, _ = lower_ops(_C(n, ops), mode="run")
        return tuple(P._gate_key(P._canon(g)) for g in gates)

    base = [("h", 0), ("rx", 1, 0.3), ("cx", 0, 1), ("rz", 2, 0.7)]
    assert key(base) == key(list(base))
    assert key(base) != key([("h", 0), ("rx", 1, 0.30001), ("cx", 0, 1), ("rz", 2, 0.7)])
    assert key(base) != key([("h", 0), ("rx", 2, 0.3), ("cx", 0, 1), ("rz", 2, 0.7)])
    assert key(base) != key([("h", 0), ("ry", 1, 0.3), ("cx", 0, 1), ("rz", 2, 0.7)])
    assert key(base) != key([("h", 0), ("rx", 1, 0.3), ("cz", 0, 1), ("rz", 2, 0.7)])
