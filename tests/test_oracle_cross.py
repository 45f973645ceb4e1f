"""The C++ oracle against the independent NumPy restatement (CPU only).

Both restate dnstbl2/dnstbl.f90's time step with P virtual ranks; they were
written separately (loops vs array slicing), so agreement to round-off pins
the restatement's reading of the reference.
"""
import numpy as np
import pytest

from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner
from oracle.np_oracle import NpOracle


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("nx,nzs,nyw,P,steps", [(16, 8, 14, 2, 7), (14, 6, 17, 3, 6), (12, 10, 11, 1, 6),
                                                 (20, 4, 16, 2, 3), (22, 5, 16, 2, 3)])
def test_cpp_equals_numpy(nx, nzs, nyw, P, steps):
    """Including the smallest span (4 rows, the periodic wrap of the span
    stencils on the fewest points) and 5 rows."""
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw, kmax=10)
    mesh, rp, st = make_state(wl, nproc=P)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    n = NpOracle(mesh, rp)
    n.upload(st)
    for s in range(steps):
        o.step(1)
        counts = o.last_counts()
        cn = n.step(counts)
        assert cn == counts
        d = o.download()
        for f, x in (("u", n.U[0]), ("v", n.U[1]), ("w", n.U[2]), ("p", n.P), ("pcorr", n.PC)):
            assert rel(x, d[f]) < 1e-12, (s, f, rel(x, d[f]))
        assert np.array_equal(d["newk"], n.newk)
        assert d["lamda"] == pytest.approx(n.lamda, rel=1e-13)
        assert np.allclose(d["wt"], n.Wt, rtol=1e-13, atol=1e-15)


def test_oracle_free_running_counts_match_numpy():
    """Without replay the NumPy restatement picks the same GS/GMRES counts."""
    wl = small_workload(nx=16, nz_span=8, ny_wall=14, kmax=10)
    mesh, rp, st = make_state(wl, nproc=2)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    n = NpOracle(mesh, rp)
    n.upload(st)
    o.step(1)
    assert n.step(None) == o.last_counts()
