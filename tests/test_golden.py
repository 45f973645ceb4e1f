"""The oracle against the committed golden fixtures (CPU).

The fixtures in tests/golden are oracle outputs written by
tests/golden/make_golden.py (the reference itself cannot be run here); this
test keeps the oracle pinned to them: fields after 4 steps to 1e-12 relative
L2 (libm may differ by an ulp between machines), iteration counts, the
recycling map and lamda."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import CASES, STEPS, run_oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, f"{name}.npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_golden(name):
    g = load(name)
    d, counts = run_oracle(name)
    for f in ("u", "v", "w", "p"):
        assert rel(d[f], g[f]) <= 1e-12, (f, rel(d[f], g[f]))
    for q in range(STEPS):
        c = g["counts"][q]
        assert counts[q] == [int(x) for x in c[c >= 0]], q
    assert np.array_equal(d["newk"], g["newk"])
    assert d["lamda"] == pytest.approx(float(g["lamda"]), rel=1e-12)
    assert d["nstep"] == int(g["nstep"])
