"""Monitor files (CPU): the library's C++ writers (tbl_monitor_* in
tbl_restart.cpp, through turbulentbl_gb300/monitor.py) against the Python
restatement of the reference's formats (oracle/tp_format.py), byte for byte,
and the Monitor's schedule over a run of the oracle that crosses a rescaling
at a multiple of 100 steps and the end of a 500-step wall-shear window."""
import numpy as np
import pytest

from turbulentbl_gb300 import abi, monitor
from turbulentbl_gb300.synth import small_workload, make_state
from oracle import tp_format as ref

EDGE = [0.0, -1e-9, 1.0, -2.5, 1234567.25, 12345678.0, -1234567.0, 7.0 / 3.0, 0.123456749999, np.nan, np.inf]


def test_fortran_f_format():
    assert ref.fortran_f(1.5, 15, 7) == "      1.5000000"
    assert ref.fortran_f(-1e-9, 15, 7) == "     -0.0000000"
    assert ref.fortran_f(12345678.0, 15, 7) == "*" * 15
    assert ref.fortran_f(-1234567.0, 15, 7) == "*" * 15  # 16 characters
    assert ref.fortran_f(1234567.25, 15, 7) == "1234567.2500000"
    assert ref.fortran_f(np.nan, 15, 7) == "            NaN"
    assert ref.fortran_f(-np.inf, 20, 10) == "           -Infinity"
    assert ref.fortran_f(0.5, 20, 10) == "        0.5000000000"


def _s(path):
    return str(path).encode()


def _d(a):
    return abi.dptr(np.asfortranarray(a, dtype=np.float64))


def test_writers_match_the_restatement(tmp_path):
    rng = np.random.default_rng(3)
    nx, ny, nz = 7, 6, 5
    x1 = np.linspace(0.0, 3.0, nx)
    x3 = np.linspace(0.0, 2.0, nz)
    a, b, c = (np.asfortranarray(rng.normal(size=(nx, nz)) * 10.0 ** rng.integers(-3, 4, size=(nx, nz)))
               for _ in range(3))
    a[0, 0], a[1, 0], a[2, 0], b[0, 0] = -1e-12, 1e9, np.nan, 0.5e-7
    ub = np.array(EDGE[:5])
    tw = rng.normal(size=nx)
    bl = [rng.uniform(0, 5, size=nx) for _ in range(6)]
    newk = np.array([3, 1, 4, 1, 5], dtype=np.int32)
    eta = np.array([1.0, 1.1, 0.9, np.inf, 0.0])
    L = monitor._lib()
    cases = [
        ("massflow.xy", True, lambda p: L.tbl_monitor_massflow(_s(p), 0.125, _d(ub)), ref.massflow_text(0.125, ub)),
        ("numrcltauwall.xy", True, lambda p: L.tbl_monitor_tauwall(_s(p), 2.5, nx, ny, 19.798, _d(x1), _d(tw)),
         ref.tauwall_text(2.5, nx, ny, 19.798, x1, tw)),
        ("kineticenergy.dat", True, lambda p: L.tbl_monitor_kinetic_energy(_s(p), 0.0005, -3.25e-7),
         ref.kinetic_energy_text(0.0005, -3.25e-7)),
        ("lamda.dat", True, lambda p: L.tbl_monitor_lamda(_s(p), 1e-4, 1.0123, -np.inf),
         ref.lamda_text(1e-4, 1.0123, -np.inf)),
        ("W.dat", False, lambda p: L.tbl_monitor_blend(_s(p), nx, nz, _d(x1), _d(x3), _d(a)), ref.blend_text(x1, x3, a)),
        ("boundarylthickness.dat", False,
         lambda p: L.tbl_monitor_bl_thickness(_s(p), 3.0, nx, _d(x1), *(_d(q) for q in bl[:5])),
         ref.bl_thickness_text(3.0, x1, *bl[:5])),
        ("k.dat", True, lambda p: L.tbl_monitor_knew(_s(p), nz, abi.iptr(newk), _d(eta)), ref.knew_text(newk, eta)),
        ("meanvalues.dat", True, lambda p: L.tbl_monitor_meanvalues(_s(p), nx, nz, _d(x1), _d(x3), _d(a), _d(b), _d(c)),
         ref.meanvalues_text(x1, x3, a, b, c)),
        ("Umeanvalues.dat", False,
         lambda p: L.tbl_monitor_umeanvalues(_s(p), nx, nz, _d(x1), _d(x3), _d(a), _d(b), _d(c), 150.92),
         ref.meanvalues_text(x1, x3, a, b, c, re=150.92)),
        ("means", False, lambda p: L.tbl_monitor_averages(_s(p), nx, nz, _d(a), _d(b), _d(c)), ref.averages_text(a, b, c)),
    ]
    for name, append, write, text in cases:
        p = tmp_path / name
        assert write(p) == abi.TBL_OK, name
        assert write(p) == abi.TBL_OK, name
        assert p.read_text() == (text + text if append else text), name


def test_writers_reject_bad_arguments(tmp_path):
    L = monitor._lib()
    assert L.tbl_monitor_massflow(_s(tmp_path / "m"), 0.0, None) == abi.TBL_ERR_BAD_ARG
    assert L.tbl_monitor_tauwall(_s(tmp_path / "t"), 0.0, 2, 6, 1.0, _d(np.zeros(2)), _d(np.zeros(2))) == abi.TBL_ERR_BAD_ARG
    assert L.tbl_monitor_lamda(None, 0.0, 1.0, 1.0) == abi.TBL_ERR_BAD_ARG
    assert L.tbl_monitor_kinetic_energy(_s(tmp_path / "no" / "such" / "dir"), 0.0, 1.0) == abi.TBL_ERR_IO


def _numbers(path):
    return [float(x) for x in path.read_text().split()]


def test_monitor_schedule_over_an_oracle_run(tmp_path):
    from oracle.bind import OracleRunner
    wl = small_workload(nx=24, nz_span=12, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    st = dict(st, nstep=495, time=0.0495, cont=0)  # steps 496..506: window end at 500, rescalings at cont 5, 10
    r = OracleRunner(mesh, rp)
    r.upload(st)
    mon = monitor.Monitor(r, tmp_path)
    status, recs = mon.step(11)
    assert status == abi.TBL_OK
    assert [q["nstep"] for q in recs] == list(range(496, 507))
    cum_steps = [q["nstep"] for q in recs if q["cum_step"]]
    assert cum_steps == [500, 505]
    nx, ny, nz = mesh.nx, mesh.ny, mesh.nz
    # every step: massflow.xy, with the last step's fluxes in its last record
    lines = (tmp_path / "massflow.xy").read_text().splitlines()
    assert len(lines) == 11
    stats = r.download_stats()
    assert lines[-1] + "\n" == ref.massflow_text(recs[-1]["time"], stats["ubulk"])
    # one wall-shear window closed (step 500): nx-2 records
    tw = _numbers(tmp_path / "numrcltauwall.xy")
    assert len(tw) == 4 * (nx - 2)
    np.testing.assert_allclose(tw[0], recs[4]["time"], atol=1e-7)
    np.testing.assert_allclose(tw[2::4], stats["tauw_window"][1:-1] / (ny - 2), rtol=1e-6, atol=1e-7)
    # KE on every step (recycling started long before)
    ke = np.array(_numbers(tmp_path / "kineticenergy.dat")).reshape(-1, 2)
    np.testing.assert_allclose(ke[:, 1], [q["ke"] for q in recs], rtol=1e-9)
    # two rescalings: lamda.dat appended twice, k.dat and meanvalues.dat once (step 500)
    lam = np.array(_numbers(tmp_path / "lamda.dat")).reshape(-1, 3)
    assert lam.shape == (2, 3)
    np.testing.assert_allclose(lam[:, 1], [recs[4]["lamda"], recs[9]["lamda"]], atol=1e-10)
    np.testing.assert_allclose(lam[1, 2], stats["lamda03"], atol=1e-10)
    assert len((tmp_path / "k.dat").read_text().splitlines()) == nz
    assert len((tmp_path / "meanvalues.dat").read_text().splitlines()) == nx * nz
    # the rewritten files hold the second rescaling's values
    s = r.download(fields=("usum2", "vsum2", "wsum2", "wt"))
    avg = r.download_averages()
    for q, name in (("u", "usum2"), ("v", "vsum2"), ("w", "wsum2")):
        np.testing.assert_array_equal(avg[q], s[name])  # the same division of the same sums
    assert (tmp_path / "means").read_text() == ref.averages_text(avg["u"], avg["v"], avg["w"])
    assert (tmp_path / "medians").read_text() == ref.averages_text(avg["uu"], avg["vv"], avg["ww"])
    assert (tmp_path / "taustress").read_text() == ref.averages_text(avg["uv"], avg["uw"], avg["vw"])
    assert np.all(avg["uu"] >= 0.0) and np.any(avg["uu"] > 0.0)
    assert (tmp_path / "Umeanvalues.dat").read_text() == ref.meanvalues_text(mesh.x1, mesh.x3, s["usum2"], s["vsum2"],
                                                                           s["wsum2"], re=rp.re)
    assert (tmp_path / "W.dat").read_text() == ref.blend_text(mesh.x1, mesh.x3, s["wt"])
    assert (tmp_path / "boundarylthickness.dat").read_text() == ref.bl_thickness_text(
        recs[9]["time"], mesh.x1, s["bltkns"], stats["deltastar"], stats["theta"], stats["ht"], stats["reth"])
    r.close()


def test_monitor_follows_the_variant_window_and_recycling_start(tmp_path):
    """originalTBL closes its wall-shear window every 1000 steps (not 500)
    and its fluctuation energy starts after its recycling start (1000)."""
    from oracle.bind import OracleRunner
    wl = small_workload(nx=24, nz_span=12, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    rp.use_variant(1)
    st = dict(st, nstep=998, time=0.0998, cont=0, cnt2=0)  # steps 999..1001: 1000 closes the window
    r = OracleRunner(mesh, rp)
    r.upload(st)
    mon = monitor.Monitor(r, tmp_path)
    assert mon.window == 1000
    status, recs = mon.step(3)
    assert status == abi.TBL_OK and [q["nstep"] for q in recs] == [999, 1000, 1001]
    tw = _numbers(tmp_path / "numrcltauwall.xy")
    assert len(tw) == 4 * (mesh.nx - 2) and tw[0] == pytest.approx(recs[1]["time"], abs=1e-7)
    ke = _numbers(tmp_path / "kineticenergy.dat")
    assert len(ke) == 2 and ke[0] == pytest.approx(recs[2]["time"], rel=1e-9)  # nstep 1001 > 1000 only
    assert len((tmp_path / "massflow.xy").read_text().splitlines()) == 3
    r.close()
