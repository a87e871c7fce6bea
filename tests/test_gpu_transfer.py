"""Host transfers of the precision form (staged through device buffers on
several copy streams): pinned and pageable host arrays must give the same
bits; a buffer pinned only in part makes CUDA refuse the copy, and the
context stays usable afterwards."""
import numpy as np
import pytest

from mhdcase import make_case

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
