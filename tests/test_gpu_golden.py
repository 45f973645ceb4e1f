"""The GPU library against the committed golden fixtures (oracle outputs,
tests/golden): the three programs' variants, 4 steps from the seeded start,
fields to 1e-12 relative L2, iteration counts, recycling map and lamda."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import CASES, STEPS, case_setup

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_matches_golden(name):
    from turbulentbl_gb300.lib import TblGpu
    g = dict(np.load(os.path.join(HERE, f"{name}.npz")))
    mesh, rp, st = case_setup(name)
    gpu = TblGpu(mesh, rp)
    gpu.upload(st)
    for q in range(STEPS):
        gpu.step(1)
        c = g["counts"][q]
        assert gpu.last_counts() == [int(x) for x in c[c >= 0]], q
    d = gpu.download()
    for f in ("u", "v", "w", "p"):
        assert rel(d[f], g[f]) <= 1e-12, (f, rel(d[f], g[f]))
    assert np.array_equal(d["newk"], g["newk"])
    assert d["lamda"] == pytest.approx(float(g["lamda"]), rel=1e-12)
