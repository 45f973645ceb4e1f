"""Monitor files of a GPU run (GB300): the same 11 steps (a 500-step
wall-shear window closing, two rescalings, one of them at a multiple of 100
steps) monitored on the GPU and on the oracle write the same files.  Values
agree to 1e-12 relative, so the formatted numbers agree to the last printed
digit (one unit of it where a value sits on a rounding boundary); the device's
averaged sums of the last rescaling match the oracle's to 1e-12."""
import numpy as np
import pytest

from turbulentbl_gb300 import abi, monitor
from turbulentbl_gb300.synth import small_workload, make_state
from oracle.bind import OracleRunner

pytestmark = pytest.mark.gpu

# last printed digit: F15.7 -> 1e-7, F20.10 -> 1e-10, E20.10 -> 1e-10 relative
DIGIT = {"kineticenergy.dat": ("rel", 2e-10), "lamda.dat": ("abs", 2e-10), "boundarylthickness.dat": ("abs", 2e-10),
         "k.dat": ("abs", 2e-10)}


def _numbers(path):
    return np.array([float(x) for x in path.read_text().split()])


def test_gpu_monitor_files_match_the_oracle(tmp_path):
    from turbulentbl_gb300.lib import TblGpu
    wl = small_workload(nx=24, nz_span=12, ny_wall=20)
    mesh, rp, st = make_state(wl, nproc=2)
    st = dict(st, nstep=495, time=0.0495, cont=0)
    out = {}
    avgs = {}
    for name, cls in (("gpu", TblGpu), ("oracle", OracleRunner)):
        d = tmp_path / name
        d.mkdir()
        r = cls(mesh, rp)
        r.upload(st)
        status, recs = monitor.Monitor(r, d).step(11)
        assert status == abi.TBL_OK, name
        avgs[name] = r.download_averages()
        r.close()
        out[name] = d
    for q in avgs["gpu"]:
        a, b = avgs["gpu"][q], avgs["oracle"][q]
        assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1e-300), q
    for f in monitor.Monitor.FILES:
        pg, po = out["gpu"] / f, out["oracle"] / f
        assert pg.exists() and po.exists(), f
        tg, to = pg.read_text(), po.read_text()
        assert len(tg.splitlines()) == len(to.splitlines()), f
        a, b = _numbers(pg), _numbers(po)
        assert a.shape == b.shape, f
        kind, tol = DIGIT.get(f, ("abs", 2e-7))
        # one unit of the last printed digit, plus the 1e-12 relative difference of large values
        bound = tol * np.abs(b) if kind == "rel" else tol + 1e-11 * np.abs(b)
        assert np.all(np.abs(a - b) <= bound), (f, np.max(np.abs(a - b)))
