"""Device-resident stepping (mhd_run: one CUDA graph per step, dt and the psi
factor on the device) and the FP64 diagnostics (mhd_diagnostics)."""
import numpy as np
import pytest

from mhdcase import diagnostics_np, make_case, rel_l1

pytestmark = pytest.mark.gpu


def fp32(M, params):
    d = params.as_dict()
    d.pop("precision")
    return M.default_params(precision="fp32", **d)


@pytest.mark.parametrize("variant", ["rk3_minmod_hlld", "rk3_mc_hlld_grav_cool", "rk2_minmod_hlld"])
def test_run_matches_host_stepping(M, variant):
    """mhd_run(n) against n mhd_step calls of the same precision-form disc:
    the only difference is exp() of the psi factor on the device (rounded to
    FP32 either way), so the states agree to 1e-6 relative L1."""
    grid, params, U, V = make_case(M, variant, (24, 16, 20))
    p = fp32(M, params)
    a = M.Disc(grid, p)
    b = M.Disc(grid, p)
    a.upload(U, V)
    b.upload(U, V)
    t = 0.0
    for _ in range(7):
        rc, t, *_ = a.step(t)
        assert rc == 0
    tb = b.run(3, 0.0)
    tb = b.run(4, tb)
    assert abs(t - tb) <= 1e-12 * t
    Ua, Va = a.download()
    Ub, Vb = b.download()
    assert np.all(rel_l1(Ub[:8], Ua[:8]) < 1e-6)
    n0 = b.launches()
    b.run(2, tb)
    nst = 3 if variant.startswith("rk3") else 2
    assert b.launches() - n0 >= 2 * (2 * nst + 2)    # per stage: stage + ghost; setdt, scalars
    a.close()
    b.close()


def test_run_dt_guard_freezes_state(M):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (16, 16, 16), dtmin=1.0e3)
    d = M.Disc(grid, fp32(M, params))
    d.upload(U, V)
    U0, V0 = d.download()
    with pytest.raises(M.MhdError) as e:
        d.run(3, 0.0)
    assert e.value.code == M.MHD_ERR_DT
    U1, V1 = d.download()
    assert np.array_equal(U0, U1)
    d.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_diagnostics(M, prec):
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", (24, 16, 20))
    p = params if prec == "fp64" else fp32(M, params)
    d = M.Disc(grid, p)
    d.upload(U, V)
    t = 0.0
    for _ in range(3):
        rc, t, *_ = d.step(t)
    Ug, _ = d.download()
    got = d.diagnostics()
    want = diagnostics_np(grid, Ug)
    for k in want:
        assert abs(got[k] - want[k]) <= 1e-12 * max(abs(want[k]), 1e-300), (k, got[k], want[k])
    d.close()


def test_invalid_cell_stops_the_precision_form(M):
    """A NaN in the state: the precision form's CFL reduction counts its rate as
    infinite, so the dt guard fires before any step is taken (mhd_step and
    mhd_run); the plain form keeps the reference's Setdt, where a NaN rate never
    wins the comparison (setdt.h:57,60), and steps on."""
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (24, 16, 20))
    Vb = V.copy()
    Vb[7, 5, 7, 9] = np.nan          # a pressure inside the CFL range (i < ixmax - 11)
    d = M.Disc(grid, fp32(M, params))
    d.upload(U, Vb)
    rc, t, dt, ch, cnt = d.step(0.0)
    assert rc == M.MHD_ERR_DT and t == 0.0
    d.upload(U, Vb)
    with pytest.raises(M.MhdError) as e:
        d.run(1, 0.0)
    assert e.value.code == M.MHD_ERR_DT
    d.close()
    d64 = M.Disc(grid, params)
    d64.upload(U, Vb)
    rc, t, dt, ch, cnt = d64.step(0.0)
    assert rc == 0 and np.isfinite(dt) and dt > 0
    d64.close()
