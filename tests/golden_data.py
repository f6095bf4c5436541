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
