"""Host transfers of the precision form (staged through device buffers on
several copy streams): pinned and pageable host arrays must give the same
bits; a buffer pinned only in part makes CUDA refuse the copy, and the
context stays usable afterwards."""
import numpy as np
import pytest

from mhdcase import make_case, rel_l1

pytestmark = pytest.mark.gpu


def fp32(M, params):
    d = params.as_dict()
    d.pop("precision")
    return M.default_params(precision="fp32", **d)


@pytest.mark.parametrize("pin", ["none", "full", "half"])
def test_pinned_and_staged_transfers_agree(M, pin):
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", (40, 24, 70))
    p = fp32(M, params)
    ref = M.Disc(grid, p)
    ref.upload(U, V)
    t = ref.run(2, 0.0)
    Ur, Vr = ref.download()
    ref.close()
    d = M.Disc(grid, p)
    d.upload(U, V)
    Uh, Vh = U.copy(), V.copy()
    Uo, Vo = np.zeros_like(U), np.zeros_like(V)
    pinned = []
    if pin != "none":
        for a in (Uh, Vh, Uo, Vo):
            nbytes = a.nbytes if pin == "full" else (a.nbytes // 2) & ~4095
            assert M.lib().mhd_pin(a.ctypes.data, nbytes, 1) == M.MHD_OK
            pinned.append(a)
    if pin == "half":
        # not wholly pinned: no direct access; CUDA itself refuses a copy over
        # a partly registered buffer (an ordinary, non-sticky error)
        with pytest.raises(M.MhdError):
            d.upload_state(Uh, Vh)
        for a in pinned:
            assert M.lib().mhd_pin(a.ctypes.data, 1, 0) == M.MHD_OK
        pinned = []
    d.upload_state(Uh, Vh)
    t2 = d.run(2, 0.0)
    d.download_into(Uo, Vo)
    for a in pinned:
        assert M.lib().mhd_pin(a.ctypes.data, 1, 0) == M.MHD_OK
    assert t2 == t
    assert np.array_equal(Uo, Ur) and np.array_equal(Vo, Vr)
    d.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_state_upload_without_primitives(M, prec):
    """mhd_upload_state(U, NULL) forms V = UtoV(U) on the device; a host that
    keeps only the conserved state moves half the bytes.  The V read back is
    UtoV(U) to rounding; a step from U alone is bit-identical to the step from
    U and that V; in the plain form it also matches the step from U and the
    initial condition's own V to 1e-12 relative L1."""
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (24, 16, 20))
    d = M.Disc(grid, M.default_params(**{k: v for k, v in params.as_dict().items() if k != "precision"},
                                      precision=prec))
    d.upload(U, V)
    d.upload_state(U, None)
    _, Vd = d.download()
    # the device's UtoV of the uploaded U: V to rounding.  In the precision
    # form U is held in FP32, so E carries a relative error of 2^-24 and the
    # pressure (gamma-1)(E - KE - ME) an absolute one of that order of
    # (gamma-1)|E| (gamma = 5/3): the pressure is checked against that scale.
    err = rel_l1(Vd, V)
    if prec == "fp32":
        err[7] = np.abs(Vd[7] - V[7]).sum() / ((5.0 / 3.0 - 1.0) * np.abs(U[7]).sum())
    assert np.all(err <= (1e-14 if prec == "fp64" else 1e-6)), err

    def step_from(Vh):
        d.upload_state(U, Vh)
        rc, t, *_ = d.step(0.0)
        assert rc == M.MHD_OK
        Uo = np.zeros_like(U)
        d.download_into(Uo, None)
        return t, Uo

    t1, Ua = step_from(None)
    t2, Ub = step_from(Vd)
    assert t1 == t2 and np.array_equal(Ua, Ub)
    if prec == "fp64":
        t3, Uc = step_from(V)
        err = rel_l1(Ua, Uc)
        err[[3, 4, 6, 8]] = [np.abs(Ua[m] - Uc[m]).sum() / max(np.abs(Uc[4:7]).sum(), 1e-300) for m in (3, 4, 6, 8)]
        assert np.all(err <= 1e-12), err
        assert abs(t1 - t3) <= 1e-9 * t3
    d.close()
