"""The plain FP64 single-disc configuration at its full size: 256x256x128,
beta 1, MC limiter, HLLD, spiral gravity (2 arms, 15 degrees, 3 percent,
pattern speed 0.5) + axisymmetric gravity, cooling on, TVD-RK3, 100 steps --
the GPU against the oracle (bit-identical to the reference C), every step's
dt, ch and floor counters and the final state bit for bit.  The oracle runs on
all host cores (about 2-3 minutes on a 16-core host)."""
import os

import numpy as np
import pytest

from mhdcase import make_case, oracle_for

pytestmark = pytest.mark.gpu

NSTEPS = 100


def test_config2_256x256x128_100_steps_bitwise(M, P):
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", (256, 256, 128))
    o = oracle_for(M, P, grid, params, threads=os.cpu_count())
    o.load(U, V)
    d = M.Disc(grid, params)
    d.upload(U, V)
    to = tg = 0.0
    for n in range(NSTEPS):
        ro = o.step(to)
        rg = d.step(tg)
        assert ro[0] == 0 and rg[0] == 0
        assert ro[1:4] == rg[1:4], "step %d: t, dt, ch" % n
        assert list(ro[4]) == list(rg[4]), "step %d: floor counters" % n
        to, tg = ro[1], rg[1]
    Uo, Vo, _ = o.store()
    Ug, Vg = d.download()
    assert np.array_equal(Ug, Uo) and np.array_equal(Vg, Vo)
    o.close()
    d.close()
