"""Pin the oracle: its C restatement (oracle/mhd_oracle.c) against the
reference's own C compiled in place (oracle/_ref/), bit for bit, on the
scheme variants, plus the product's host-side grid and gravity tables against
the reference's.  Runs where the reference tree exists (this container)."""
import numpy as np
import pytest

from conftest import reference_tree_present
from mhdcase import VARIANTS, make_case, oracle_for

pytestmark = pytest.mark.skipif(not reference_tree_present(), reason="reference tree not present")

DIMS = (16, 16, 16)


def ref_for(M, P, grid, params):
    r = P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params))
    if params.gravity:
        r.initial_gravity()
    return r


def test_grid_tables_match_reference(M, P):
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", DIMS)
    r = ref_for(M, P, grid, params)
    o = oracle_for(M, P, grid, params)
    gr, go = r.grid1d(), o.grid1d()
    for k in gr:
        assert np.array_equal(np.asarray(gr[k]), np.asarray(go[k])), k
    mr, mo = r.metric(), o.metric()
    for k in mr:
        assert np.array_equal(mr[k], mo[k]), k
    # the product's host-side CylindricalGrid / InitialGravity
    for name, n in [("x", grid.ixmax), ("xm", grid.ixmax), ("dx", grid.ixmax), ("dxm", grid.ixmax),
                    ("oneox", grid.ixmax), ("oneodx", grid.ixmax), ("y", grid.jymax), ("z", grid.kzmax),
                    ("zm", grid.kzmax), ("dz", grid.kzmax), ("dzm", grid.kzmax), ("oneodz", grid.kzmax)]:
        assert np.array_equal(grid.arr(name, n), gr[name]), name
    assert grid.g.minminlength == gr["minminlength"] and grid.g.dy == gr["dy"]
    gflat = np.stack([grid.arr("g%d" % (n + 1), (grid.ixmax - 1) * (grid.kzmax - 1)) for n in range(6)])
    gflat = gflat.reshape(6, grid.ixmax - 1, 1, grid.kzmax - 1)
    assert np.array_equal(mr["g"][:, :, 1:, :], np.broadcast_to(gflat, mr["g"][:, :, 1:, :].shape))
    assert np.array_equal(grid.arr("x_absorb_factor", 11), mr["xabs"])
    assert np.array_equal(grid.arr("z_absorb_factor", 11), mr["zabs"])
    assert np.array_equal(grid.arr("c_absorb_factor", (grid.irin + 1) * grid.kzmax), mr["cabs"].ravel())
    axi_r, _ = r.gravity()
    assert np.array_equal(axi_r, grid.gravity_axi_cells())


@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_steps_match_reference(M, P, variant):
    grid, params, U, V = make_case(M, variant, DIMS)
    r = ref_for(M, P, grid, params)
    o = oracle_for(M, P, grid, params, threads=4)
    r.load(U, V)
    o.load(U, V)
    tr = to = 0.0
    for n in range(4):
        rr = r.step(tr)
        ro = o.step(to)
        tr, to = rr[1], ro[1]
        assert rr[0] == ro[0] == 0
        assert rr[2] == ro[2] and rr[3] == ro[3], "dt/ch step %d" % n
        assert np.array_equal(rr[4], ro[4]), "floor counters step %d" % n
    Ur, Vr, U1r = r.store()
    Uo, Vo, U1o = o.store()
    assert np.array_equal(Ur, Uo)
    assert np.array_equal(Vr, Vo)
    assert np.array_equal(U1r, U1o)


@pytest.mark.parametrize("variant", ["rk3_minmod_hlld", "rk3_mc_hlld_grav_cool", "rk3_minmod_hll"])
def test_probes_match_reference(M, P, variant):
    grid, params, U, V = make_case(M, variant, DIMS)
    r = ref_for(M, P, grid, params)
    o = oracle_for(M, P, grid, params)
    r.load(U, V)
    o.load(U, V)
    dt_r, ch_r, _ = r.setdt()
    dt_o, ch_o, _ = o.setdt()
    assert (dt_r, ch_r) == (dt_o, ch_o)
    r.set_dtch(dt_r, ch_r)
    o.set_dtch(dt_r, ch_r)
    for d in range(3):
        a, b = r.limiter(d), o.limiter(d)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), d
        assert np.array_equal(r.flux(d), o.flux(d)), d
    r.spiral(0.37)
    o.spiral(0.37)
    assert np.array_equal(r.gravity()[1], o.gravity()[1])
    assert np.array_equal(r.source(), o.source())


def test_cooling_function_matches_reference(M, P):
    """Cooling (cooling.h:22) as an int on a sweep of temperatures, including
    the band edges a=0.031 and b=0.054 where its sign factors are 0/0."""
    grid, params, _, _ = make_case(M, "rk3_mc_hlld_grav_cool", DIMS)
    r = ref_for(M, P, grid, params)
    lib = P.Oracle.lib()
    for rho in (0.5, 1.0, 3.0):
        for T in np.concatenate([np.linspace(0.0, 0.3, 301), [0.031, 0.054, 0.078, 0.235, 1e-9]]):
            pr = T * rho
            assert r.lib.ref_cooling(rho, pr) == lib.orc_cooling(rho, pr), (rho, T)
