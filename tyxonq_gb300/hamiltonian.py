"""Pauli-sum Hamiltonians packed for the GPU kernels.

Input formats accepted (all from the reference):
  * list of ``(coeff, [(pauli_char, qubit), ...])`` — the HEA runtime format
    (tyxonq/applications/chem/runtimes/hea_numeric_runtime.py:36-53);
  * Pauli code lists + weights, codes 0..3 = I, X, Y, Z, qubit 0 first
    (tyxonq/libs/quantum_library/kernels/pauli.py:65-87);
  * a dict ``{((q, 'X'), ...): coeff}`` as in openfermion's ``QubitOperator.terms``.

Packing: term P = prod_q sigma_q acts as P|i> = i^{ny} (-1)^{popc(i & zy)} |i ^ flip>
with flip = X/Y bits, zy = Y/Z bits (qubit q <-> bit n-1-q).  Terms are
sorted by flip mask into groups so the kernels sweep the state once per
distinct mask.  Repeated qubits inside one term keep the last Pauli, as the
reference's ``term[qubit_idx] = code`` does (hea_numeric_runtime.py:45-47).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

GROUP_DTYPE = np.dtype([("flip", "<u8"), ("first_term", "<i4"), ("n_terms", "<i4")])
TERM_DTYPE = np.dtype([("zy", "<u8"), ("w_re", "<f8"), ("w_im", "<f8"), ("f_re", "<f4"), ("f_im", "<f4")])
_CODE = {"I": 0, "X": 1, "Y": 2, "Z": 3}
_I_POW = [(1.0, 0.0), (0.0, 1.0), (-1.0, 0.0), (0.0, -1.0)]


@dataclass
class PauliSum:
    """H = sum_k coeff_k * P_k on n qubits; codes[k, q] in {0,1,2,3}."""

    n: int
    codes: np.ndarray  # (K, n) int8
    coeffs: np.ndarray  # (K,) float64
    _packed: tuple | None = field(default=None, repr=False)
    _device_cache: dict = field(default_factory=dict, repr=False)

    # ------------------------------------------------------------ constructors
    @classmethod
    def from_terms(cls, n: int, terms: Iterable) -> "PauliSum":
        terms = list(terms)
        codes = np.zeros((len(terms), n), dtype=np.int8)
        coeffs = np.zeros(len(terms), dtype=np.float64)
        for k, (c, ops) in enumerate(terms):
            coeffs[k] = float(c)
            for p, q in ops:
                q = int(q)
                if q < 0 or q >= n:
                    raise ValueError(f"qubit {q} out of range for {n} qubits")
                codes[k, q] = _CODE[str(p).upper()]
        return cls(n, codes, coeffs)

    @classmethod
    def from_codes(cls, ls: Sequence[Sequence[int]], weights: Sequence[float] | None = None) -> "PauliSum":
        arr = np.asarray(ls, dtype=np.int8)
        if arr.ndim != 2:
            raise ValueError("Pauli code list must be 2-D (terms x qubits)")
        if np.any((arr < 0) | (arr > 3)):
            raise ValueError("Pauli codes must be in 0..3")
        w = np.ones(arr.shape[0]) if weights is None else np.asarray(weights, dtype=np.float64)
        return cls(arr.shape[1], arr.copy(), w.astype(np.float64))

    @classmethod
    def from_qubit_operator_terms(cls, n: int, terms: dict) -> "PauliSum":
        items = []
        for key, c in terms.items():
            if abs(complex(c).imag) > 1e-12:
                raise ValueError("non-Hermitian term coefficient")
            items.append((complex(c).real, [(p, q) for (q, p) in key]))
        return cls.from_terms(n, items)

    # ------------------------------------------------------------ views
    @property
    def n_terms(self) -> int:
        return int(self.codes.shape[0])

    def terms(self) -> list:
        inv = "IXYZ"
        out = []
        for k in range(self.n_terms):
            out.append((float(self.coeffs[k]), [(inv[c], q) for q, c in enumerate(self.codes[k]) if c]))
        return out

    def masks(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(flip, zy, ny) per term as uint64/uint64/int."""
        n = self.n
        bits = (np.uint64(1) << (np.uint64(n - 1) - np.arange(n, dtype=np.uint64))) if n else np.zeros(0, np.uint64)
        c = self.codes
        xy = (c == 1) | (c == 2)
        yz = (c == 2) | (c == 3)
        flip = np.bitwise_or.reduce(np.where(xy, bits, np.uint64(0)), axis=1) if n else np.zeros(len(c), np.uint64)
        zy = np.bitwise_or.reduce(np.where(yz, bits, np.uint64(0)), axis=1) if n else np.zeros(len(c), np.uint64)
        ny = (c == 2).sum(axis=1)
        return flip.astype(np.uint64), zy.astype(np.uint64), ny.astype(np.int64)

    def pack(self) -> tuple[np.ndarray, np.ndarray]:
        """(groups, terms) structured arrays matching tq_pauli_group / tq_pauli_term."""
        if self._packed is not None:
            return self._packed
        flip, zy, ny = self.masks()
        order = np.lexsort((zy, flip))
        pw = np.array(_I_POW)[ny[order] & 3]
        terms = np.zeros(self.n_terms, dtype=TERM_DTYPE)
        terms["zy"] = zy[order]
        terms["w_re"] = self.coeffs[order] * pw[:, 0] if self.n_terms else 0
        terms["w_im"] = self.coeffs[order] * pw[:, 1] if self.n_terms else 0
        terms["f_re"] = terms["w_re"]  # float copies for the complex64 kernels
        terms["f_im"] = terms["w_im"]
        fs = flip[order]
        starts = np.flatnonzero(np.r_[True, fs[1:] != fs[:-1]]) if self.n_terms else np.zeros(0, np.int64)
        g = np.zeros(len(starts), dtype=GROUP_DTYPE)
        g["flip"] = fs[starts]
        g["first_term"] = starts
        g["n_terms"] = np.diff(np.r_[starts, self.n_terms])
        self._packed = (g, terms)
        return self._packed

    @property
    def n_groups(self) -> int:
        return int(self.pack()[0].shape[0])

    def to_device(self, device):
        """Device copies of the packed tables (uint8 tensors), cached per device."""
        import torch

        key = str(device)
        hit = self._device_cache.get(key)
        if hit is not None:
            return hit
        g, t = self.pack()
        gd = torch.from_numpy(np.frombuffer(g.tobytes() or b"\0" * 16, dtype=np.uint8).copy()).to(device)
        td = torch.from_numpy(np.frombuffer(t.tobytes() or b"\0" * 32, dtype=np.uint8).copy()).to(device)
        out = (gd, td, int(g.shape[0]), int(t.shape[0]))
        self._device_cache[key] = out
        return out

    def to_device_classed(self, device, hbits: int = 12):
        """Like to_device, with each group's terms sorted by bits 8 .. hbits-1 of
        zy (the order the tiled H psi kernel reads fastest), cached per device."""
        import torch

        key = f"classed{hbits}:{device}"
        hit = self._device_cache.get(key)
        if hit is not None:
            return hit
        g, t = self.pack()
        t = sort_terms_by_class(g, t, hbits)
        g = order_groups_for_tiles(g, t, hbits)
        gd = torch.from_numpy(np.frombuffer(g.tobytes() or b"\0" * 16, dtype=np.uint8).copy()).to(device)
        td = torch.from_numpy(np.frombuffer(t.tobytes() or b"\0" * 32, dtype=np.uint8).copy()).to(device)
        out = (gd, td, int(g.shape[0]), int(t.shape[0]))
        self._device_cache[key] = out
        return out

    def one_norm(self) -> float:
        return float(np.abs(self.coeffs).sum())


def sort_terms_by_class(groups: np.ndarray, terms: np.ndarray, hbits: int) -> np.ndarray:
    """Order each group's terms by their Z/Y bits 8 .. hbits-1 (the bits that
    tell apart the amplitudes one thread of the wave H psi kernel holds), so
    the kernel's per-class sums switch class at most 2^(hbits-8) - 1 times per
    group.  Groups keep their term ranges; only the order inside changes."""
    if len(terms) == 0 or hbits <= 8:
        return terms
    gid = np.repeat(np.arange(len(groups)), groups["n_terms"])
    first = np.repeat(groups["first_term"], groups["n_terms"])
    order_in = np.arange(len(terms)) - first  # position inside the group (groups are contiguous, in order)
    cls = (terms["zy"] >> np.uint64(8)) & np.uint64((1 << (hbits - 8)) - 1)
    idx = np.lexsort((order_in, cls.astype(np.int64), gid))
    return terms[idx]


def order_groups_for_tiles(groups: np.ndarray, terms: np.ndarray, hbits: int) -> np.ndarray:
    """Groups in the order the tiled H psi kernel reads fastest: by the flip
    bits above the output tile (groups that read the same partner tile are
    neighbours), then one-term groups by the Z/Y bits 8 .. 11 of their term
    (runs of equal class share one code path), then the others; by flip last.
    Only the summation order depends on it."""
    if len(groups) == 0:
        return groups
    hi = groups["flip"] >> np.uint64(hbits)
    one = groups["n_terms"] == 1
    zy_first = terms["zy"][np.minimum(groups["first_term"], max(len(terms) - 1, 0))] if len(terms) else \
        np.zeros(len(groups), np.uint64)
    cls = np.where(one, ((zy_first >> np.uint64(8)) & np.uint64(15)).astype(np.int64), 16)
    return groups[np.lexsort((groups["flip"], cls, hi))]


def as_pauli_sum(H, n: int | None = None) -> PauliSum:
    """Coerce any accepted Hamiltonian format to PauliSum."""
    if isinstance(H, PauliSum):
        return H
    if isinstance(H, dict):
        if n is None:
            raise ValueError("n is required for dict Hamiltonians")
        return PauliSum.from_qubit_operator_terms(n, H)
    if hasattr(H, "terms") and isinstance(getattr(H, "terms"), dict):
        if n is None:
            raise ValueError("n is required for QubitOperator Hamiltonians")
        return PauliSum.from_qubit_operator_terms(n, H.terms)
    if isinstance(H, tuple) and len(H) == 2 and not isinstance(H[0], (int, float)):
        return PauliSum.from_codes(H[0], H[1])
    if n is None:
        raise ValueError("n is required for term-list Hamiltonians")
    return PauliSum.from_terms(n, H)


# ---------------------------------------------------------------- generators
def tfim_terms(n: int, hx: float = 1.0, hzz: float = 1.0, pbc: bool = False) -> list:
    """H = -hzz sum Z_i Z_{i+1} - hx sum X_i (open chain unless pbc); the
    term set of tyxonq/libs/circuits_library/hamiltonians.py:17-27."""
    terms = []
    for i in range(n - 1 + (1 if pbc and n > 2 else 0)):
        terms.append((-hzz, [("Z", i), ("Z", (i + 1) % n)]))
    for i in range(n):
        terms.append((-hx, [("X", i)]))
    return terms


def random_pauli_sum(n: int, n_terms: int, rng: np.random.Generator, max_weight: int = 4) -> PauliSum:
    """Random H: n_terms terms, weight uniform in 1..max_weight on distinct
    random qubits, Paulis uniform in {X,Y,Z}, coefficients N(0,1)."""
    w = rng.integers(1, min(max_weight, n) + 1, size=n_terms)
    # the first w[k] entries of a random permutation of the qubits are the support
    perm = np.argsort(rng.random((n_terms, n)), axis=1)
    rank = np.empty_like(perm)
    np.put_along_axis(rank, perm, np.arange(n)[None, :].repeat(n_terms, 0), axis=1)
    on = rank < w[:, None]
    codes = np.where(on, rng.integers(1, 4, size=(n_terms, n)), 0).astype(np.int8)
    coeffs = rng.standard_normal(n_terms)
    return PauliSum(n, codes, coeffs)
