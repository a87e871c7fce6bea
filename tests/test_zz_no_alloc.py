"""The allocation-free CFL reduction (mhd_setdt_noalloc) against the context's
mhd_setdt on the same state, through the C-ABI.

It serves callers that may not allocate device memory when they need a step
size; its scratch is a fixed device array inside the library.  Both entry
points evaluate the same FP64 kernel and fold the partial maxima with the same
rule, so dt, ch and the argmax cell must be identical (the plain FP64 form's
tolerance everywhere in this suite is exact equality).  Two calls in a row on
different states check that the shared array's leftovers do not leak into the
next result.  Collected last on purpose (file name)."""
import ctypes as C

import numpy as np
import pytest

from mhdcase import make_case

pytestmark = pytest.mark.gpu


def _noalloc(M, grid, params, Vdev, mldev, stream):
    dt, ch = C.c_double(), C.c_double()
    ijk = np.zeros(3, dtype=np.int32)
    rc = M.lib().mhd_setdt_noalloc(C.c_void_p(Vdev), C.c_void_p(mldev), grid.ix, grid.jy, grid.kz,
                                   params.cfl, grid.g.minminlength, params.cooling, C.c_void_p(stream),
                                   C.byref(dt), C.byref(ch), ijk)
    return rc, dt.value, ch.value, tuple(int(v) for v in ijk)


def test_noalloc_setdt_matches_context_setdt(M):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", (40, 32, 24))
    ml = grid.arr("minlength", grid.ixmax * grid.kzmax)
    mldev = torch.from_numpy(ml).cuda()
    d = M.Disc(grid, params)
    d.upload(U, V)
    stream = torch.cuda.current_stream().cuda_stream
    t = 0.0
    for call in range(2):
        _, Vcur = d.download()
        Vdev = torch.from_numpy(np.ascontiguousarray(Vcur)).cuda()
        torch.cuda.synchronize()
        rc, dt, ch, ijk = _noalloc(M, grid, params, Vdev.data_ptr(), mldev.data_ptr(), stream)
        assert rc == M.MHD_OK, M.lib().mhd_errstr(rc)
        dt_ref, ch_ref, ijk_ref = d.setdt()
        assert (dt, ch, ijk) == (dt_ref, ch_ref, ijk_ref), "call %d" % call
        rc, t, *_ = d.step(t)       # a different state for the second call
        assert rc == 0
    d.close()


def test_noalloc_rejects_grids_beyond_its_scratch(M):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (16, 16, 16))
    dt, ch = C.c_double(), C.c_double()
    ijk = np.zeros(3, dtype=np.int32)
    # 2048x1024x128: CFL range far beyond 8192 blocks of 256x64 cells; the
    # pointers are never dereferenced because the size check comes first
    rc = M.lib().mhd_setdt_noalloc(C.c_void_p(16), C.c_void_p(16), 2048, 1024, 128, 0.4, 1.0, 0,
                                   None, C.byref(dt), C.byref(ch), ijk)
    assert rc == M.MHD_ERR_ARG
