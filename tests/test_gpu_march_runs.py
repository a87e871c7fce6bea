"""The marched r and phi flux kernels at every run length the launcher picks.

A thread marches over a run of faces and reconstructs each cell once; the run
is 16 faces where that still leaves several blocks per SM, 4 or 1 on smaller
grids.  On a 152-SM GB300: 24x16x20 runs 1 face per thread, 96x96x64 runs 4,
160x160x64 runs 16.  Plain FP64 form, two steps, bit for bit against the
oracle (dt, ch, floor counters and the state), with the MC limiter (periodic
r/phi face fills) and van Leer (free r faces, fixed phi faces) so the edge
faces of every run length are covered.
"""
import os

import numpy as np
import pytest

from mhdcase import make_case, oracle_for, run_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(24, 16, 20), (96, 96, 64), (160, 160, 64)])
@pytest.mark.parametrize("variant", ["rk3_mc_hlld_grav_cool", "rk2_vanleer_hlld_grav_cool"])
def test_march_run_lengths_bitwise(M, P, dims, variant):
    nsteps = 2
    grid, params, U, V = make_case(M, variant, dims)
    o = oracle_for(M, P, grid, params, threads=os.cpu_count())
    Uo, Vo, log_o, _ = run_oracle(o, U, V, nsteps)
    o.close()
    d = M.Disc(grid, params)
    d.upload(U, V)
    t = 0.0
    log = []
    for _ in range(nsteps):
        rc, t, dt, ch, cnt = d.step(t)
        assert rc == 0
        log.append((dt, ch, tuple(int(c) for c in cnt)))
    Ug, Vg = d.download()
    d.close()
    assert log == log_o
    assert np.array_equal(Ug, Uo) and np.array_equal(Vg, Vo)
