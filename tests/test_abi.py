"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/tbl_gpu.h (no device work: this runs on CPU)."""
import ctypes as C
import os
import re

import pytest

from turbulentbl_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "tbl_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tbl_[a-z_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return C.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("tbl_create", "tbl_upload_state", "tbl_step", "tbl_download_state", "tbl_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layout_matches_c(tmp_path):
    """The ctypes mirror has the C compiler's layout of every ABI struct."""
    import subprocess
    prog = tmp_path / "sz.c"
    structs = ["tbl_config", "tbl_mesh", "tbl_state", "tbl_step_stats", "tbl_stats_out", "tbl_window_config",
               "tbl_fields", "tbl_adjoint_stats"]
    body = "".join(f'printf("%zu\\n", sizeof({t}));' for t in structs)
    prog.write_text('#include <stdio.h>\n#include "tbl_gpu.h"\nint main(void){' + body + "return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    mirror = [abi.TblConfig, abi.TblMesh, abi.TblState, abi.TblStepStats, abi.TblStatsOut, abi.TblWindowConfig,
              abi.TblFields, abi.TblAdjointStats]
    assert sizes == [C.sizeof(m) for m in mirror]


def test_bad_arguments_are_rejected_without_a_device(lib):
    lib.tbl_create.restype = C.c_int
    lib.tbl_step.restype = C.c_int
    h = C.c_void_p()
    assert lib.tbl_create(None, None, C.byref(h)) == abi.TBL_ERR_BAD_ARG
    assert lib.tbl_step(None, 1, None) == abi.TBL_ERR_BAD_ARG
    lib.tbl_status_string.restype = C.c_char_p
    assert lib.tbl_status_string(abi.TBL_ERR_TIMEOUT)
    for f in (lib.tbl_set_wall_control, lib.tbl_forward_window, lib.tbl_backward_window):
        f.restype = C.c_int
    assert lib.tbl_set_wall_control(None, None) == abi.TBL_ERR_BAD_ARG
    assert lib.tbl_forward_window(None, 1, None, None, None) == abi.TBL_ERR_BAD_ARG
    assert lib.tbl_backward_window(None, C.c_double(1.0), None, None, None, None) == abi.TBL_ERR_BAD_ARG
