"""The allocation-free divergence diagnostic (tbl_div_diag_noalloc).

Callers that cannot allocate device memory (a host code whose own pool owns
the GPU's memory, or a time loop where an allocation could synchronise the
device) use this entry point with fields they already hold on the device.
It must give the same value as the divergence diagnostic tbl_step reports,
on two calls in a row (the scratch it keeps between calls must not leak into
the next result), and refuse grids larger than its fixed scratch.  This file
is collected last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

from turbulentbl_gb300 import abi
from turbulentbl_gb300.synth import small_workload, make_state

pytestmark = pytest.mark.gpu
TOL = 1e-12  # relative; only the order of the grid reduction differs


def _bind(lib):
    f = lib.tbl_div_diag_noalloc
    f.argtypes = [C.POINTER(abi.TblConfig)] + [C.c_void_p] * 5
    f.restype = C.c_int
    return f


@pytest.mark.parametrize("variant", [abi.TBL_VARIANT_DNSTBL2, abi.TBL_VARIANT_ORIGINAL])
def test_noalloc_matches_step_diagnostic_twice(variant):
    """The default program prints |sum div U|/N, originalTBL its square root."""
    import torch
    from turbulentbl_gb300.lib import TblGpu, load
    wl = small_workload(nx=40, nz_span=34, ny_wall=33)
    mesh, rp, st = make_state(wl, nproc=4)
    rp.variant = variant
    g = TblGpu(mesh, rp)
    g.upload(st)
    f = _bind(load())
    for step in range(2):
        status, rec = g.step(1)
        ref = rec[0]["div_diag"]
        d = g.download(fields=("u", "v", "w"))
        dev = torch.device("cuda", torch.cuda.current_device())
        fields = [torch.from_numpy(np.asarray(d[c]).reshape(-1, order="F").copy()).to(dev) for c in ("u", "v", "w")]
        jinv = torch.from_numpy(1.0 / mesh.jac).to(dev)
        out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
        cfg = g._cfg
        for call in range(2):
            out.fill_(-1.0)
            torch.cuda.synchronize()
            s = f(C.byref(cfg), jinv.data_ptr(), fields[0].data_ptr(), fields[1].data_ptr(), fields[2].data_ptr(),
                  out.data_ptr())
            torch.cuda.synchronize()
            assert s == abi.TBL_OK, s
            val = float(out.item())
            assert abs(val - ref) <= TOL * abs(ref), (step, call, val, ref)


def test_noalloc_rejects_grids_beyond_its_scratch():
    from turbulentbl_gb300.lib import load
    f = _bind(load())
    cfg = abi.TblConfig()
    cfg.nx, cfg.ny, cfg.nz = 4098, 4098, 8
    cfg.dx = cfg.dy = cfg.dxi = 1.0
    s = f(C.byref(cfg), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), C.c_void_p(16))
    assert s == abi.TBL_ERR_TOO_LARGE
