"""NumPy restatement of the reference statevector engine (test oracle only).

Conventions (reference):
  * state = complex128 vector of length 2^n viewed C-order as (2,)*n, axis q
    is qubit q, so qubit 0 is the most significant index bit
    (kernels/statevector.py:28-59).
  * gate matrices: kernels/gates.py:11-287; 2q index = 2*bit(q0) + bit(q1).
All references are relative to TyxonQ's ``src/tyxonq``.
"""
from __future__ import annotations

import math
from typing import Any, Sequence

import numpy as np

# ------------------------------------------------------------------ gates (gates.py)
I2 = np.eye(2, dtype=np.complex128)
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
PAULI = {0: I2, 1: X, 2: Y, 3: Z, "I": I2, "X": X, "Y": Y, "Z": Z}


def g_h():  # gates.py:11-16
    return np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2.0)


def g_phase(t):  # gates.py:68-79
    return np.array([[1, 0], [0, np.exp(1j * t)]], dtype=np.complex128)


def g_rot(t, P):  # cos(t/2) I - i sin(t/2) P  (gates.py:19-48, 203-249)
    return math.cos(t / 2) * np.eye(P.shape[0]) + (-1j * math.sin(t / 2)) * P


def g_ry(t):  # gates.py:51-65
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def g_cx():  # gates.py:82-91
    return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)


def g_cz():  # gates.py:98-107
    return np.diag([1, 1, 1, -1]).astype(np.complex128)


def g_swap():  # gates.py:136-160
    return np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def g_iswap():  # gates.py:110-133
    return np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def g_cry(t):  # gates.py:252-284
    U = np.eye(4, dtype=np.complex128)
    U[2:, 2:] = g_ry(t)
    return U


def gate_matrix(name: str, theta: float | None = None) -> np.ndarray:
    name = name.lower()
    if name == "h":
        return g_h()
    if name == "x":
        return X.copy()
    if name == "y":
        return Y.copy()
    if name == "z":
        return Z.copy()
    if name == "s":
        return g_phase(math.pi / 2)
    if name == "sdg":
        return g_phase(-math.pi / 2)
    if name == "t":
        return g_phase(math.pi / 4)
    if name == "tdg":
        return g_phase(-math.pi / 4)
    if name == "rx":
        return g_rot(theta, X)
    if name == "ry":
        return g_ry(theta)
    if name == "rz":
        return g_rot(theta, Z)
    if name == "phase":
        return g_phase(theta)
    if name in ("cx", "cnot"):
        return g_cx()
    if name == "cz":
        return g_cz()
    if name == "cy":
        U = np.eye(4, dtype=np.complex128)
        U[2:, 2:] = Y
        return U
    if name == "swap":
        return g_swap()
    if name == "iswap":
        return g_iswap()
    if name == "rxx":
        return g_rot(theta, np.kron(X, X))
    if name == "ryy":
        return g_rot(theta, np.kron(Y, Y))
    if name == "rzz":
        return g_rot(theta, np.kron(Z, Z))
    if name == "cry":
        return g_cry(theta)
    raise KeyError(name)


# ------------------------------------------------------------------ kernels (statevector.py)
def init_state(n: int, basis: int = 0) -> np.ndarray:
    """init_statevector (statevector.py:19-25), generalised to |basis>."""
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[basis] = 1.0
    return psi


def apply_1q(psi: np.ndarray, U: np.ndarray, q: int, n: int) -> np.ndarray:
    """apply_1q_statevector (statevector.py:28-42): contract U's column index
    with axis q of the (2,)*n view (tensordot instead of the 26-letter einsum)."""
    t = psi.reshape((2,) * n)
    out = np.tensordot(U, t, axes=([1], [q]))  # new axis 0 = qubit q
    return np.moveaxis(out, 0, q).reshape(-1)


def apply_kq(psi: np.ndarray, U: np.ndarray, qubits: Sequence[int], n: int) -> np.ndarray:
    """apply_kqubit_unitary (statevector.py:71-129): move target axes last (in
    the listed order), (2^{n-k}, 2^k) @ U^T, inverse permutation."""
    k = len(qubits)
    if k == 0:
        return psi
    qs = [int(q) for q in qubits]
    keep = [a for a in range(n) if a not in qs]
    perm = keep + qs
    inv = np.argsort(perm)
    m = psi.reshape((2,) * n).transpose(perm).reshape(1 << (n - k), 1 << k)
    m = m @ np.asarray(U, dtype=np.complex128).reshape(1 << k, 1 << k).T
    return m.reshape((2,) * n).transpose(inv).reshape(-1)


def apply_2q(psi: np.ndarray, U: np.ndarray, q0: int, q1: int, n: int) -> np.ndarray:
    """apply_2q_statevector (statevector.py:45-59); q0 == q1 leaves psi unchanged."""
    if q0 == q1:
        return psi
    return apply_kq(psi, U, [q0, q1], n)


def expect_z(psi: np.ndarray, q: int, n: int) -> float:
    """expect_z_statevector (statevector.py:62-68)."""
    s = np.moveaxis(psi.reshape((2,) * n), q, 0).reshape(2, -1)
    p = (np.abs(s) ** 2).sum(axis=1)
    return float(p[0] - p[1])


def project_z(psi: np.ndarray, q: int, keep: int, n: int) -> np.ndarray:
    """StatevectorEngine._project_z (engine.py:1075-1086)."""
    t = np.moveaxis(psi.reshape((2,) * n).copy(), q, 0)
    t[1 - int(keep), ...] = 0
    out = np.moveaxis(t, 0, q).reshape(-1)
    nrm = np.linalg.norm(out)
    return out / nrm if nrm > 0 else out


# ------------------------------------------------------------------ engine dispatch (engine.py)
RUN_OPS = {"h", "rz", "rx", "ry", "cx", "cry", "cz", "iswap", "swap", "rxx", "ryy", "rzz", "x", "s", "sdg",
           "measure_z", "barrier", "project_z", "reset", "unitary", "kraus"}
# state() lacks cry/y/z/t/tdg/cy/measure_z/barrier branches (engine.py:914-1039)
STATE_OPS = {"h", "rz", "rx", "ry", "cx", "cz", "iswap", "swap", "rxx", "ryy", "rzz", "x", "s", "sdg",
             "project_z", "reset", "unitary", "kraus"}


def apply_kraus(psi: np.ndarray, ops: Sequence[np.ndarray], q: int, n: int, status: float) -> np.ndarray:
    """apply_kraus_statevector (kernels/statevector.py:132-218): Born weights
    p_i = ||K_i psi||^2, normalised cumulative sums, the first i with
    status <= cum_i (0 if none), then K_i psi / ||K_i psi||."""
    outs = [apply_1q(psi, np.asarray(k, dtype=np.complex128), q, n) for k in ops]
    p = np.array([float(np.real(np.vdot(o, o))) for o in outs])
    cum = np.cumsum(p / p.sum())
    sel = 0
    for i, c in enumerate(cum):
        if status <= float(c):
            sel = i
            break
    out = outs[sel]
    return out / np.sqrt(np.real(np.vdot(out, out)))


# gates that feed use_noise's Z attenuation (engine.py:56-143)
ATTENUATED_OPS = {"h", "rz", "rx", "ry", "cx", "cry", "cz", "iswap", "swap", "rxx", "ryy", "rzz", "x", "s", "sdg",
                  "unitary"}


def z_attenuation(n: int, ops: Sequence[Any], noise: dict, unitary_cache: dict | None = None) -> np.ndarray:
    """_attenuate (engine.py:488-494) over the run() gate loop: depolarizing p
    multiplies the factor of every wire a gate touches by max(0, 1 - 4p/3)."""
    att = np.ones(n)
    if str(noise.get("type", "")).lower() != "depolarizing":
        return att
    f = max(0.0, 1.0 - 4.0 * float(noise.get("p", 0.0)) / 3.0)
    cache = unitary_cache or {}
    for op in ops:
        if not isinstance(op, (list, tuple)) or not op or op[0] not in ATTENUATED_OPS:
            continue
        if op[0] in ("h", "rz", "rx", "ry", "x", "s", "sdg"):
            wires = [int(op[1])]
        elif op[0] == "unitary":
            if len(op) == 3 and cache.get(str(op[2])) is not None:
                wires = [int(op[1])]
            elif len(op) == 4 and cache.get(str(op[3])) is not None:
                wires = [int(op[1]), int(op[2])]
            else:
                continue
        else:
            wires = [int(op[1]), int(op[2])]
        for q in wires:
            att[q] *= f
    return att


def noisy_probabilities(psi: np.ndarray, n: int, noise: dict) -> np.ndarray:
    """The sampled distribution of run(use_noise=True) (engine.py:377-414):
    |psi|^2, then readout (kron of per-qubit calibration matrices, identity
    where absent) or depolarizing mixing (1 - a) p + a / 2^n, a = min(1, 4p/3);
    clip to [0, 1], renormalise, uniform if nothing is left."""
    p = np.abs(psi) ** 2
    ntype = str(noise.get("type", "")).lower()
    if ntype == "readout":
        cals = noise.get("cals", {}) or {}
        A = None
        for q in range(n):
            m = np.asarray(cals.get(q, np.eye(2)), dtype=float)
            A = m if A is None else np.kron(A, m)
        p = A @ p
    elif ntype == "depolarizing":
        a = max(0.0, min(1.0, 4.0 * float(noise.get("p", 0.0)) / 3.0))
        p = (1.0 - a) * p + a / p.size
    p = np.clip(p, 0.0, 1.0)
    s = float(p.sum())
    p = p / (s if s > 1e-12 else 1.0)
    return p / p.sum() if p.sum() > 0 else np.full(p.size, 1.0 / p.size)


def run_ops(n: int, ops: Sequence[Any], *, mode: str = "state", unitary_cache: dict | None = None,
            initial: np.ndarray | None = None, kraus_cache: dict | None = None) -> tuple[np.ndarray, list[int]]:
    """Gate loop of StatevectorEngine.run (engine.py:52-374) / .state
    (engine.py:914-1039).  Returns (psi, measured qubits).  Kraus ops need an
    explicit status here (the reference draws a missing one at random)."""
    psi = init_state(n) if initial is None else np.asarray(initial, dtype=np.complex128).reshape(-1).copy()
    allowed = RUN_OPS if mode == "run" else STATE_OPS
    measures: list[int] = []
    for op in ops:
        if not isinstance(op, (list, tuple)) or not op:
            continue
        name = op[0]
        if name not in allowed:
            continue  # ignored, as in the reference
        if name in ("h", "x", "s", "sdg"):
            psi = apply_1q(psi, gate_matrix(name), int(op[1]), n)
        elif name in ("rx", "ry", "rz"):
            psi = apply_1q(psi, gate_matrix(name, float(op[2])), int(op[1]), n)
        elif name in ("cx", "cz", "swap", "iswap"):
            psi = apply_2q(psi, gate_matrix(name), int(op[1]), int(op[2]), n)
        elif name in ("rxx", "ryy", "rzz", "cry"):
            psi = apply_2q(psi, gate_matrix(name, float(op[3])), int(op[1]), int(op[2]), n)
        elif name == "measure_z":
            measures.append(int(op[1]))
        elif name == "project_z":
            psi = project_z(psi, int(op[1]), int(op[2]), n)
        elif name == "reset":
            psi = project_z(psi, int(op[1]), 0, n)
        elif name == "kraus":  # engine.py:145-155
            kops = (kraus_cache or {}).get(str(op[2]))
            if kops is not None:
                psi = apply_kraus(psi, kops, int(op[1]), n, float(op[3]))
        elif name == "unitary":
            cache = unitary_cache or {}
            if len(op) == 3:
                U = cache.get(str(op[2]))
                if U is not None:
                    psi = apply_kq(psi, U, [int(op[1])], n)
            elif len(op) == 4:
                U = cache.get(str(op[3]))
                if U is not None:
                    psi = apply_kq(psi, U, [int(op[1]), int(op[2])], n)
    return psi, measures


# ------------------------------------------------------------------ Pauli sums
def pauli_string_matrix(codes: Sequence[int]) -> np.ndarray:
    """pauli_string_to_matrix (kernels/pauli.py:65-71): kron, qubit 0 leftmost."""
    out = np.array([[1.0 + 0j]])
    for c in codes:
        out = np.kron(out, PAULI[int(c)])
    return out


def dense_hamiltonian(codes: np.ndarray, coeffs: np.ndarray) -> np.ndarray:
    """pauli_string_sum_dense (kernels/pauli.py:74-87); small n only."""
    n = codes.shape[1]
    H = np.zeros((1 << n, 1 << n), dtype=np.complex128)
    for c, w in zip(codes, coeffs):
        H += float(w) * pauli_string_matrix(c)
    return H


def apply_pauli_term(psi: np.ndarray, codes: Sequence[int], n: int) -> np.ndarray:
    """P psi for one Pauli string by per-qubit 2x2 application (same operator as
    pauli_string_to_matrix, without forming it)."""
    out = psi
    for q, c in enumerate(codes):
        if int(c):
            out = apply_1q(out, PAULI[int(c)], q, n)
    return out


def apply_pauli_sum(psi: np.ndarray, codes: np.ndarray, coeffs: np.ndarray) -> np.ndarray:
    n = codes.shape[1]
    out = np.zeros_like(psi)
    for c, w in zip(codes, coeffs):
        out += float(w) * apply_pauli_term(psi, c, n)
    return out


def pauli_expectation(psi: np.ndarray, codes: np.ndarray, coeffs: np.ndarray) -> float:
    """Re <psi|H|psi> = dynamics.expectation(psi, H) (dynamics.py:117-126)."""
    return float(np.real(np.vdot(psi, apply_pauli_sum(psi, codes, coeffs))))


def terms_to_codes(n: int, terms) -> tuple[np.ndarray, np.ndarray]:
    """[(coeff, [(P, q), ...])] -> codes/coeffs, last Pauli wins per qubit
    (hea_numeric_runtime.py:36-53)."""
    m = {"X": 1, "Y": 2, "Z": 3}
    codes = np.zeros((len(terms), n), dtype=np.int8)
    coeffs = np.zeros(len(terms))
    for k, (c, ops) in enumerate(terms):
        coeffs[k] = float(c)
        for p, q in ops:
            codes[k, int(q)] = m[str(p).upper()]
    return codes, coeffs


# ------------------------------------------------------------------ gradients
def energy(n: int, ops_fn, theta: np.ndarray, codes, coeffs) -> float:
    psi, _ = run_ops(n, ops_fn(theta), mode="state")
    return pauli_expectation(psi, codes, coeffs)


def grad_forward_fd(n, ops_fn, theta, codes, coeffs, eps: float = 1e-6) -> tuple[float, np.ndarray]:
    """NumPy backend value_and_grad: forward differences, eps 1e-6
    (numerics/backends/numpy_backend.py:386-454)."""
    theta = np.asarray(theta, dtype=np.float64)
    e0 = energy(n, ops_fn, theta, codes, coeffs)
    g = np.zeros_like(theta)
    for k in range(theta.size):
        t = theta.copy()
        t[k] += eps
        g[k] = (energy(n, ops_fn, t, codes, coeffs) - e0) / eps
    return e0, g


def grad_central_fd(n, ops_fn, theta, codes, coeffs, h: float = 1e-4) -> np.ndarray:
    theta = np.asarray(theta, dtype=np.float64)
    g = np.zeros_like(theta)
    for k in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        g[k] = (energy(n, ops_fn, tp, codes, coeffs) - energy(n, ops_fn, tm, codes, coeffs)) / (2 * h)
    return g


def grad_param_shift(n, ops_fn, theta, codes, coeffs) -> np.ndarray:
    """Parameter shift g = (E(t+pi/2) - E(t-pi/2)) / 2 for parameters that enter
    exactly one Pauli rotation each (compiler/gradients/parameter_shift.py:9-36,
    kernels/common.py:11-23)."""
    theta = np.asarray(theta, dtype=np.float64)
    g = np.zeros_like(theta)
    s = math.pi / 2
    for k in range(theta.size):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += s
        tm[k] -= s
        g[k] = 0.5 * (energy(n, ops_fn, tp, codes, coeffs) - energy(n, ops_fn, tm, codes, coeffs))
    return g


def grad_adjoint(n, gates, theta, codes, coeffs) -> tuple[float, np.ndarray]:
    """Reverse-sweep adjoint gradient in the form of the reference's CI-space
    energy_and_grad_civector (chem_libs/quantum_chem_library/civector_ops.py:141-200):
    ket, bra = H ket; walk gates backwards, un-apply on both, grad = <bra|dU ket>.
    `gates` = list of (name, qubits, param_index or None, scale) with angle =
    scale * theta[param_index]; rotations exp(-i a/2 P) give dE/da = Im<bra|P|ket>."""
    theta = np.asarray(theta, dtype=np.float64)
    psi = init_state(n)
    mats = []
    for name, qs, pidx, sc in gates:
        ang = sc * theta[pidx] if pidx is not None else None
        U = gate_matrix(name, ang)
        mats.append(U)
        psi = apply_kq(psi, U, qs, n)
    lam = apply_pauli_sum(psi, codes, coeffs)
    e = float(np.real(np.vdot(psi, lam)))
    g = np.zeros_like(theta)
    gens = {"rx": [X], "ry": [Y], "rz": [Z], "rxx": [X, X], "ryy": [Y, Y], "rzz": [Z, Z]}
    for (name, qs, pidx, sc), U in zip(reversed(gates), reversed(mats)):
        if pidx is not None:
            if name not in gens:
                raise NotImplementedError(name)
            P = gens[name][0] if len(qs) == 1 else np.kron(gens[name][0], gens[name][1])
            Ppsi = apply_kq(psi, P, qs, n)
            g[pidx] += 2.0 * sc * float(np.real(np.vdot(lam, -0.5j * Ppsi)))
        Ud = U.conj().T
        psi = apply_kq(psi, Ud, qs, n)
        lam = apply_kq(lam, Ud, qs, n)
    return e, g


# ------------------------------------------------------------------ shot estimates
def group_by_basis(codes: np.ndarray, coeffs: np.ndarray) -> tuple[float, dict]:
    """group_hamiltonian_pauli_terms (hamiltonian_grouping.py:120-138): terms
    with identical product bases share a group; identity terms add to a constant."""
    inv = "IXYZ"
    const, groups = 0.0, {}
    for row, c in zip(np.asarray(codes), np.asarray(coeffs)):
        term = tuple((q, inv[int(x)]) for q, x in enumerate(row) if x)
        if not term:
            const += float(c)
            continue
        groups.setdefault(tuple(inv[int(x)] for x in row), []).append((term, float(c)))
    return const, groups


def term_expectation_from_counts(counts: dict, idxs) -> float:
    """counts_expval.py:7-20: mean of prod_q (+1 if bit q is 0 else -1)."""
    total = sum(counts.values()) or 1
    acc = 0.0
    for b, cnt in counts.items():
        s = 1.0
        for q in idxs:
            s *= 1.0 if b[q] == "0" else -1.0
        acc += s * cnt
    return acc / total


def expval_pauli_sum(counts: dict, items, identity_const: float = 0.0) -> float:
    """counts_expval.py:96-130 (counts path): identity + sum coeff * <Z...Z>."""
    e = float(identity_const)
    for term, c in items:
        e += c * term_expectation_from_counts(counts, [q for q, _ in term])
    return e


# ------------------------------------------------------------------ sampling
def probabilities(psi: np.ndarray) -> np.ndarray:
    """engine.py:377-414: |psi|^2 renormalised."""
    p = np.abs(psi) ** 2
    s = p.sum()
    return p / s if s > 0 else np.full(p.size, 1.0 / p.size)


def sample_counts(psi: np.ndarray, shots: int, rng: np.random.Generator) -> dict[str, int]:
    """engine.py:381-463: choice + bincount + big-endian bitstrings."""
    n = int(psi.size).bit_length() - 1
    p = probabilities(psi)
    idx = rng.choice(p.size, size=shots, p=p)
    cnt = np.bincount(idx, minlength=p.size)
    return {format(i, f"0{n}b"): int(c) for i, c in enumerate(cnt) if c}


def chi2_pvalue(counts: dict[str, int], probs: np.ndarray, min_expected: float = 5.0) -> float:
    """Pearson chi^2 goodness of fit of counts against exact probabilities;
    bins with expected count < min_expected are pooled."""
    from scipy import stats

    shots = sum(counts.values())
    n = int(probs.size).bit_length() - 1
    obs = np.zeros(probs.size)
    for b, c in counts.items():
        obs[int(b, 2) if n else 0] += c
    exp = probs * shots
    big = exp >= min_expected
    o = list(obs[big])
    e = list(exp[big])
    if (~big).any():
        o.append(obs[~big].sum())
        e.append(exp[~big].sum())
    o, e = np.array(o), np.array(e)
    keep = e > 0
    if (o[~keep] > 0).any():
        return 0.0
    o, e = o[keep], e[keep]
    if len(o) < 2:
        return 1.0
    chi2 = ((o - e) ** 2 / e).sum()
    return float(stats.chi2.sf(chi2, len(o) - 1))
