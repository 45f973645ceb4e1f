"""Restart files (CPU): the library's C++ readers and writers
(tbl_restart.cpp, through turbulentbl_gb300/tpfile.py) against the Python
restatement of the formats (oracle/tp_format.py), byte for byte, for the
three programs' formats; round trips; the per-rank split and merge; the
counter files and dnssetbl's statData.dat."""
import numpy as np
import pytest

from turbulentbl_gb300 import tpfile
from turbulentbl_gb300.synth import small_workload, make_state
from oracle import tp_format as ref

FMTS = [0, 1, 2]


def _case(nx=10, nzs=6, nyw=9, P=2):
    wl = small_workload(nx=nx, nz_span=nzs, ny_wall=nyw)
    mesh, rp, st = make_state(wl, nproc=P)
    return mesh, rp, st


def test_fortran_e_format():
    assert ref.fortran_e(1.0) == " 0.100000000000000E+01"
    assert ref.fortran_e(-0.5) == "-0.500000000000000E+00"
    assert ref.fortran_e(0.0) == " 0.000000000000000E+00"
    assert ref.fortran_e(123.456) == " 0.123456000000000E+03"
    assert ref.fortran_e(9.9999999999999999e-3) == " 0.100000000000000E-01"
    assert ref.fortran_e(2.5e120) == " 0.250000000000000+121"
    for v in (1e-30, -3.25e17, 0.999999999999999, 7.0 / 3.0):
        assert len(ref.fortran_e(v)) == 22
        assert abs(float(ref.fortran_e(v)) - v) <= 5e-15 * abs(v)  # 15 significant digits


@pytest.mark.parametrize("fmt", FMTS)
def test_writer_bytes_match_the_restatement(tmp_path, fmt):
    mesh, rp, st = _case()
    rng = np.random.default_rng(1)
    st = dict(st)
    st["p"] = np.asfortranarray(rng.normal(size=st["u"].shape) * 10.0 ** rng.integers(-40, 40, size=st["u"].shape))
    st["u"] = np.asfortranarray(st["u"].copy())
    st["u"][0, 0, 0] = -0.0
    st["u"][1, 0, 0] = 1e-310  # subnormal
    for header in (0, 1, 2):
        a, b = tmp_path / f"c{header}.tp", tmp_path / f"p{header}.tp"
        tpfile.write_tp(a, mesh, st, 1.25, 37, j_range=(1, mesh.ny - 2), k_range=(2, 5), header=header, fmt=fmt,
                        nproc=3)
        ref.write_tp(b, mesh, st, 1.25, 37, j_range=(1, mesh.ny - 2), k_range=(2, 5), header=header, fmt=fmt,
                     nproc=3)
        assert a.read_bytes() == b.read_bytes(), (fmt, header)


@pytest.mark.parametrize("fmt", FMTS)
def test_merged_roundtrip(tmp_path, fmt):
    mesh, rp, st = _case()
    p = tmp_path / "3D.tp"
    tpfile.write_tp(p, mesh, st, time=1.25, nstep=37, header=2, fmt=fmt)
    back, t, n = tpfile.read_tp(p, mesh.nx, mesh.ny, mesh.nz, fmt=fmt)
    assert t == 1.25 and n == 37
    cols = ("u", "v", "w", "p") + (("uf", "vf", "wf") if fmt == 0 else ())
    for c in cols:
        assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300), c
    if fmt == 0:
        for c in ("usum2", "vsum2", "wsum2", "wt"):
            assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300), c
        assert np.array_equal(back["newk"], st["newk"])
    for c, x in (("x1", mesh.x1), ("x2", mesh.x2), ("x3", mesh.x3)):
        assert np.allclose(back[c], x, atol=5e-7), c  # F10.6
    pb, _, _ = ref.read_tp(p, fmt=fmt)
    for c in cols:
        assert np.array_equal(pb[c], back[c]), c


@pytest.mark.parametrize("fmt", FMTS)
@pytest.mark.parametrize("P", [2, 3])
def test_rank_split_and_merge(tmp_path, fmt, P):
    """Per-rank files (j = 2..ny-1, each rank's k range) and their merge, as
    the reference's mergers do; both byte-identical to the restatement."""
    mesh, rp, st = _case(nx=8, nzs=6, nyw=13, P=P)
    (tmp_path / "c").mkdir()
    (tmp_path / "p").mkdir()
    tpfile.write_rank_files(tmp_path / "c", mesh, st, time=0.5, nstep=4, nproc=P, fmt=fmt)
    ref.write_rank_files(tmp_path / "p", mesh, st, time=0.5, nstep=4, nproc=P, fmt=fmt)
    for r in range(P):
        name = ref.rank_name(r, fmt)
        assert (tmp_path / "c" / name).read_bytes() == (tmp_path / "p" / name).read_bytes(), name
    tpfile.merge_rank_files(tmp_path / "c", mesh.nz, P, fmt=fmt)
    ref.merge_rank_files(tmp_path / "p", mesh.nz, P, fmt=fmt)
    assert (tmp_path / "c" / "3D.tp").read_bytes() == (tmp_path / "p" / "3D.tp").read_bytes()
    back, t, n = tpfile.read_tp(tmp_path / "c" / "3D.tp", mesh.nx, mesh.ny, mesh.nz, fmt=fmt)
    assert (t, n) == (0.5, 4)
    for c in ("u", "v", "w"):  # ghost rows rebuilt by periodic copy
        assert np.allclose(back[c], st[c], rtol=1e-14, atol=1e-300)
    assert np.allclose(back["p"][:, 1:-1], st["p"][:, 1:-1], rtol=1e-14, atol=1e-300)
    if fmt == 0:
        assert np.array_equal(back["newk"], st["newk"])
    ranges = ref.rank_ranges(mesh.nz, P, fmt)
    assert ranges[0][0] == 0 and ranges[-1][1] == mesh.nz - 1
    assert all(ranges[q][1] + 1 == ranges[q + 1][0] for q in range(P - 1))


def test_counters(tmp_path):
    tpfile.write_counters(tmp_path, 64, 3, 8, 1234)
    assert tpfile.read_counters(tmp_path) == (64, 3, 8, 1234)
    (tmp_path / "r").mkdir()
    ref.write_counters(tmp_path / "r", 64, 3, 8, 1234)
    for f in ("cnt", "cnt2"):
        assert (tmp_path / f).read_bytes() == (tmp_path / "r" / f).read_bytes()


def test_statdata_roundtrip_rounds_to_seven_decimals(tmp_path):
    mesh, rp, st = _case()
    p, q = tmp_path / "statData.dat", tmp_path / "ref.dat"
    tpfile.write_statdata(p, st, rp.irec)
    ref.write_statdata(q, st, rp.irec)
    assert p.read_bytes() == q.read_bytes()
    back = {n: np.zeros_like(st[n], order="F") for n in ("usum2", "vsum2", "wsum2", "wt")}
    back["newk"] = np.zeros_like(st["newk"], dtype=np.int32)
    tpfile.read_statdata(p, back, rp.irec)
    ir = rp.irec - 1
    for n in ("usum2", "vsum2", "wsum2"):
        assert np.allclose(back[n][ir], st[n][ir], atol=5.001e-8, rtol=0), n
    assert np.allclose(back["wt"][0], st["wt"][0], atol=5.001e-8, rtol=0)
    assert np.array_equal(back["newk"], st["newk"])


def test_bad_arguments_and_missing_files(tmp_path):
    from turbulentbl_gb300.runner import TblError
    mesh, rp, st = _case()
    with pytest.raises(TblError):
        tpfile.read_tp(tmp_path / "missing.tp", mesh.nx, mesh.ny, mesh.nz)
    with pytest.raises(TblError):
        tpfile.write_tp(tmp_path / "x.tp", mesh, st, 0.0, 0, fmt=7)
    with pytest.raises(TblError):
        tpfile.write_tp(tmp_path / "x.tp", mesh, st, 0.0, 0, k_range=(3, mesh.nz))
    p = tmp_path / "3D.tp"
    tpfile.write_tp(p, mesh, st, 0.0, 0, header=2)
    with pytest.raises(TblError):  # zone does not match the grid
        tpfile.read_tp(p, mesh.nx + 1, mesh.ny, mesh.nz)
    p.write_text(p.read_text()[: len(p.read_text()) // 2])  # truncated
    with pytest.raises(TblError):
        tpfile.read_tp(p, mesh.nx, mesh.ny, mesh.nz)


@pytest.mark.parametrize("P", [2, 3])
def test_restart_through_files_continues_the_run(tmp_path, P):
    """Checkpoint/resume: 3 steps, the per-rank files, merge and counters
    written by the library, read back, and 3 more steps, against resuming
    from the in-memory arrays.  A restart starts a new program run
    (dnstbl2/dnstbl.f90:147-159, 350-358, 434-445): PCorr, lamda, cont and the
    statistics sums start afresh, and the restart file carries 15
    significant digits, so both resumes agree to that rounding."""
    from oracle.bind import OracleRunner
    wl = small_workload(nx=16, nz_span=8, ny_wall=14, kmax=10)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.cum = 4
    o = OracleRunner(mesh, rp)
    o.upload(st)
    o.step(3)
    d = o.download()
    d["ume1"], d["bltkns"] = st["ume1"], st["bltkns"]
    tpfile.write_rank_files(tmp_path, mesh, d, d["time"], d["nstep"], nproc=P)
    tpfile.merge_rank_files(tmp_path, mesh.nz, P)
    tpfile.write_counters(tmp_path, mesh.nz, 1, P, d["cnt2"])
    back, t, n = tpfile.read_tp(tmp_path / "3D.tp", mesh.nx, mesh.ny, mesh.nz)
    nz_, cnt, nproc, cnt2 = tpfile.read_counters(tmp_path)
    assert (n, nz_, nproc, cnt2) == (d["nstep"], mesh.nz, P, 3)
    assert t == pytest.approx(d["time"], abs=5.001e-11)  # the title's F20.10
    fresh = dict(lamda=1.0, cont=0, pcorr=None, ume1=st["ume1"], bltkns=st["bltkns"], ksep=d["ksep"])
    runs = []
    for src in (dict(d, **fresh), dict(back, time=t, nstep=n, cnt2=cnt2, **fresh)):
        r = OracleRunner(mesh, rp)
        r.upload(src)
        r.step(3)
        runs.append(r.download())
    for f in ("u", "v", "w", "p"):
        err = np.linalg.norm(runs[1][f] - runs[0][f]) / np.linalg.norm(runs[0][f])
        assert err <= 1e-9, (f, err)
    assert runs[1]["nstep"] == runs[0]["nstep"] == d["nstep"] + 3


def test_inflow_profile_round_trip(tmp_path):
    """U_innerdns.dat written from a profile and read back: 8 significant
    digits (E18.8), byte-identical to the Python restatement, record 37
    repeated above plane 37."""
    wl = small_workload(nx=10, nz_span=6, ny_wall=48)
    mesh, rp, st = make_state(wl, nproc=2)
    p = tmp_path / "U_innerdns.dat"
    tpfile.write_inflow_profile(p, mesh.x3, st["ume1"])
    assert p.read_text() == ref.inflow_profile_text(mesh.x3, st["ume1"])
    back = tpfile.read_inflow_profile(p, mesh.nz)
    assert np.array_equal(back, ref.read_inflow_profile(p.read_text(), mesh.nz))
    np.testing.assert_allclose(back[:37], st["ume1"][:37], rtol=5e-8, atol=0)
    assert np.all(back[37:] == back[36])


def test_inflow_profile_fortran_input_forms(tmp_path):
    """Fields as a Fortran READ(…,'(24X,E18.8)') takes them: exponent letters
    E and D, a bare-sign exponent, no decimal point (8 implied decimals),
    embedded blanks ignored, an empty field read as zero; a short record is
    padded with blanks."""
    fields = ["0.12345678E+01", "1.5D-02", "  .5E0", "12345678", "-0.25+01", "", "1 .5", "3.0E 1"]
    want = [1.2345678, 0.015, 0.5, 0.12345678, -2.5, 0.0, 1.5, 30.0]
    recs = [("x" * 24 + f.rjust(18)) for f in fields] + ["x" * 24 + "0.9E0"] * (37 - len(fields))
    text = "\n".join(recs) + "\n"
    p = tmp_path / "U_innerdns.dat"
    p.write_text(text)
    got = tpfile.read_inflow_profile(p, 40)
    np.testing.assert_allclose(got[:len(want)], want, rtol=1e-15, atol=0)
    assert np.all(got[len(want):] == 0.9)
    assert np.array_equal(got, ref.read_inflow_profile(text, 40))
    short = tmp_path / "short.dat"
    short.write_text("\n".join(recs[:36]) + "\n")
    with pytest.raises(Exception):
        tpfile.read_inflow_profile(short, 40)
    bad = tmp_path / "bad.dat"
    bad.write_text("\n".join(["x" * 24 + "abc"] + recs[1:]) + "\n")
    with pytest.raises(Exception):
        tpfile.read_inflow_profile(bad, 40)
