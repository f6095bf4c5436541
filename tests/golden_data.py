"""Loader for the committed golden vectors (produced by tests/golden/make_golden.py
from the reference itself)."""
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


@lru_cache(maxsize=1)
def load():
    arrays = dict(np.load(GOLDEN / "golden.npz"))
    meta = json.loads((GOLDEN / "golden.json").read_text())
    return arrays, meta


def circuit_cases():
    arrays, meta = load()
    out = []
    for c in meta["circuits"]:
        ucache = {u: arrays[f"{c['name']}_{u}"] for u in c["unitaries"]}
        ops = [tuple(o) for o in c["ops"]]
        out.append((c["name"], c["n"], ops, ucache, arrays[f"{c['name']}_state"], arrays[f"{c['name']}_runz"]))
    return out


def kraus_sets():
    _, meta = load()
    return {k: [np.array([complex(re, im) for re, im in m], dtype=np.complex128).reshape(2, 2) for m in v]
            for k, v in meta["kraus_sets"].items()}


def noise_cases():
    """(name, n, ops, kraus_cache, state, run <Z>, run <Z> under use_noise depolarizing p=0.05)."""
    arrays, meta = load()
    sets = kraus_sets()
    out = []
    for c in meta["noise"]:
        kc = {key: sets[name] for key, name in c["kraus"].items()}
        ops = [tuple(o) for o in c["ops"]]
        out.append((c["name"], c["n"], ops, kc, arrays[f"{c['name']}_state"], arrays[f"{c['name']}_runz"],
                    arrays[f"{c['name']}_runz_depol"]))
    return out


def counts_cases():
    """(n, counts, items [(term, coeff)], energy, expvals) from the reference's expval_pauli_sum."""
    _, meta = load()
    return [(c["n"], c["counts"], [(tuple((int(q), p) for q, p in t), float(w)) for t, w in c["items"]],
             c["energy"], c["expvals"]) for c in meta["counts"]]
