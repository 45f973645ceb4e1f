"""Restart file round trips in the reference's 3D.tp format (CPU)."""
import numpy as np

from turbulentbl_gb300 import tpfile
from turbulentbl_gb300.synth import small_workload, make_state


def test_fortran_e_format():
    assert tpfile.fortran_e(1.0) == " 0.100000000000000E+01"
    assert tpfile.fortran_e(-0.5) == "-0.500000000000000E+00"
    assert tpfile.fortran_e(0.0) == " 0.000000000000000E+00"
    assert tpfile.fortran_e(123.456) == " 0.123456000000000E+03"
    assert tpfile.fortran_e(9.9999999999999999e-3) == " 0.100000000000000E-01"
    for v in (1e-30, -3.25e17, 0.999999999999999, 7.0 / 3.0):
        assert len(tpfile.fortran_e(v)) == 22
        assert float(tpfile.fortran_e(v)) == float(f"{v:.14e}") or abs(float(tpfile.fortran_e(v)) - v) <= 1e-14 * abs(v)


def test_merged_roundtrip(tmp_path):
    wl = small_workload(nx=10, nz_span=6, ny_wall=9)
    mesh, rp, st = make_state(wl, nproc=2)
    p = tmp_path / "3D.tp"
    tpfile.write_tp(p, mesh, st, time=1.25, nstep=37)
    back, t, n = tpfile.read_tp(p)
    assert t == 1.25 and n == 37
    for c in ("u", "v", "w", "p", "uf", "vf", "wf"):
        assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300)
    for c in ("usum2", "vsum2", "wsum2", "wt"):
        assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300)
    assert np.array_equal(back["newk"], st["newk"])


def test_rank_split_and_merge(tmp_path):
    """Per-rank files (j = 2..ny-1, own k range) merged as dnstbl/restart.f90 does."""
    wl = small_workload(nx=8, nz_span=6, ny_wall=13)
    mesh, rp, st = make_state(wl, nproc=3)
    tpfile.write_rank_files(tmp_path, mesh, st, time=0.5, nstep=4, nproc=3)
    tpfile.merge_rank_files(tmp_path, mesh.nz, 3)
    back, t, n = tpfile.read_tp(tmp_path / "3D.tp")
    assert (t, n) == (0.5, 4)
    for c in ("u", "v", "w"):  # ghost rows rebuilt by periodic copy
        assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300)
    assert np.allclose(back["p"][:, 1:-1], st["p"][:, 1:-1], rtol=1e-14, atol=1e-300)
    assert np.array_equal(back["newk"], st["newk"])
    ranges = tpfile.rank_ranges(mesh.nz, 3)
    assert ranges[0][0] == 0 and ranges[-1][1] == mesh.nz - 1
    assert all(ranges[q][1] + 1 == ranges[q + 1][0] for q in range(2))


def test_counters(tmp_path):
    tpfile.write_counters(tmp_path, 64, 3, 8, 1234)
    assert tpfile.read_counters(tmp_path) == (64, 3, 8, 1234)
