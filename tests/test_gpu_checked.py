"""The checked library variant (-DTQ_CHECKED): device-side index checks on
every instrumented site stay silent over exhaustive tiny cases (every gate kind
on every qubit, qubit pair and several triples of 1..6-qubit states, both
precisions) and larger fused, H psi, sampling and batched runs, whose results
match the oracle.  Runs in a child process: the library variant is chosen at
load time."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.gpu
def test_checked_build_is_silent_and_matches_the_oracle():
    env = dict(os.environ, TYXONQ_GB300_CHECKED="1", TYXONQ_GB300_JIT="0")
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "checked_child.py")], env=env, capture_output=True,
                       text=True, timeout=1800)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
    out = json.loads(line)
    print(json.dumps(out["err"], indent=1))
    assert out["checked"] is True and out["library"].endswith("libtyxonq_gb300_checked.so")
    assert out["site"] == 0, f"check site {out['site']} failed at index {out['index']}"
    err = out["err"]
    for k, v in err.items():
        if k.endswith("_c128"):
            assert v < 1e-12, (k, v)
        elif k.endswith("_c64") and k != "batched_energy_c64":
            assert v < 2e-6, (k, v)
    assert err["batched_energy_c64"] < 1e-5
    assert err["sample_in_range"] == 0.0
