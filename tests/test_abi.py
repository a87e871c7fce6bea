"""The C-ABI library loads (no GPU needed) and exports every function that
include/mhd_gpu.h declares; host-side helpers behave; errors are codes."""
import ctypes as C
import os
import re

import numpy as np

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mhd_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\*?\s*(mhd_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(M):
    names = declared_functions()
    assert len(names) >= 30, names
    lib = C.CDLL(M.LIBPATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_errstr_and_bad_arguments(M):
    L = M.lib()
    assert L.mhd_errstr(M.MHD_ERR_DT).decode().startswith("stop due to small dt")
    h = C.c_void_p()
    # NULL grid / odd phi count are argument errors, reported before any CUDA call
    assert L.mhd_create(None, C.byref(M.default_params()), C.byref(h)) == -1
    s = M.MhdGridSpec()
    assert L.mhd_gridspec_disc(32, 15, 32, C.byref(s)) == -1
    assert L.mhd_gridspec_disc(8, 16, 32, C.byref(s)) == -1


def test_params_default_are_the_reference_values(M):
    p = M.default_params()
    assert p.cfl == 0.4 and p.dtmin == 1.0e-9 and p.prcr == 0.015 and p.rhocr == 1.0e-4
    assert p.betacr == 0.1 and p.armnum == 2 and p.scheme == 2
    assert p.tausp == 200.0 * 1.0e+6 * 3.1536e+7 / 4.7058e+15
    assert p.pitch == 15.0 * np.pi / 180.0


def test_initial_condition_is_seeded_and_consistent(M):
    g = M.Grid.disc(16, 8, 16)
    U1, V1 = g.ic_disc(beta=10.0, amp=0.01, seed=0)
    U2, V2 = g.ic_disc(beta=10.0, amp=0.01, seed=0)
    U3, V3 = g.ic_disc(beta=10.0, amp=0.01, seed=1)
    assert np.array_equal(U1, U2) and np.array_equal(V1, V2)
    assert not np.array_equal(V1, V3)
    rho = V1[0]
    assert np.all(rho > 0) and np.allclose(V1[7], 0.01 * rho, rtol=0, atol=0)
    assert np.allclose(V1[5], np.sqrt(2 * V1[7] / 10.0))
    assert np.all(np.abs(V1[2] - 1.0) <= 0.01) and np.all(np.abs(V1[1]) <= 0.01)
    # U = VtoU(V) (vtou.h:44-52)
    x = g.arr("x", g.ixmax).reshape(-1, 1, 1)
    assert np.array_equal(U1[2], x * V1[0] * V1[2])


def test_grid_storage_layout(M):
    g = M.Grid.disc(24, 12, 20)
    x = g.arr("x", g.ixmax)
    dx = g.arr("dx", g.ixmax)
    assert np.allclose(x[1], 0.1 + 0.5 * 1.4 / 24) and np.all(dx == dx[0])
    assert g.irin == int(0.1 / (1.4 / 24))
    z = g.arr("z", g.kzmax)
    assert np.isclose(z[1], -0.5 + 0.5 / 20) and np.isclose(z[-2], 0.5 - 0.5 / 20)


def test_device_selection_errors_are_codes(M):
    L = M.lib()
    d = C.c_int(-1)
    rc0 = L.mhd_use_device(0)
    if rc0 == -7:          # no CUDA device here: every call says so, none crashes
        assert L.mhd_use_device(-1) == -7 and L.mhd_current_device(C.byref(d)) == -7
    else:
        assert rc0 == 0 and L.mhd_use_device(-1) == -1 and L.mhd_use_device(1 << 20) == -1
        assert L.mhd_current_device(C.byref(d)) == 0 and d.value == 0
    assert L.mhd_current_device(None) == -1


def test_binding_precision_codes_match_the_header(M):
    """The binding's precision names map to the header's MHD_PREC_* codes."""
    src = open(os.path.join(ROOT, "include", "mhd_gpu.h")).read()
    codes = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define MHD_PREC_(\w+) (\d+)", src)}
    assert codes == {"FP64": 0, "FP32": 1, "FP32X2": 2}
    assert M.PREC == {k.lower(): v for k, v in codes.items()}
