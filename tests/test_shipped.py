"""The reference's shipped production case, pinned against the reference C
built on its own stretched grid (input.h:45-76, via -DREF_SHIPPED):

* the product's CylindricalGrid tables on the stretched grid,
* the product's GalacticDisc3 (model.h:149-327): V, U after the z=0 fills,
  the initial arrays, floors and the axisymmetric gravity,
* the oracle's live RK2 steps (halfstep.h/fullstep.h, Z antisymmetric/free
  boundaries, spiral gravity, cooling) against the reference's.

The reduced grid keeps the shipped spacing and stretching rules and is long
enough to reach the stretched zones in r (beyond r = 2) and z (beyond 0.03).
All comparisons are bit for bit."""
import numpy as np
import pytest

from conftest import reference_tree_present
from mhdcase import make_shipped, oracle_for

pytestmark = pytest.mark.skipif(not reference_tree_present(), reason="reference tree not present")

REDUCED = (220, 8, 120)
FULL = (240, 64, 200)


def ref_shipped(M, P, grid, params):
    return P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params), shipped=True)


@pytest.mark.parametrize("dims", [REDUCED, FULL])
def test_shipped_grid_and_galactic_disc3_match_reference(M, P, dims):
    grid, params, U, V, Ui, Vi, rf = make_shipped(M, dims)
    assert grid.arr("dx", grid.ixmax)[-1] > grid.arr("dx", grid.ixmax)[1]      # stretched in r
    assert grid.arr("dz", grid.kzmax)[-1] > grid.arr("dz", grid.kzmax)[1]      # and in z
    r = ref_shipped(M, P, grid, params)
    gr = r.grid1d()
    for name, n in [("x", grid.ixmax), ("xm", grid.ixmax), ("dx", grid.ixmax), ("dxm", grid.ixmax),
                    ("oneox", grid.ixmax), ("oneodx", grid.ixmax), ("y", grid.jymax), ("z", grid.kzmax),
                    ("zm", grid.kzmax), ("dz", grid.kzmax), ("dzm", grid.kzmax), ("oneodz", grid.kzmax)]:
        assert np.array_equal(grid.arr(name, n), gr[name]), name
    assert grid.g.minminlength == gr["minminlength"]
    mr = r.metric()
    gflat = np.stack([grid.arr("g%d" % (n + 1), (grid.ixmax - 1) * (grid.kzmax - 1)) for n in range(6)])
    gflat = gflat.reshape(6, grid.ixmax - 1, 1, grid.kzmax - 1)
    assert np.array_equal(mr["g"][:, :, 1:, :], np.broadcast_to(gflat, mr["g"][:, :, 1:, :].shape))
    assert np.array_equal(grid.arr("c_absorb_factor", (grid.irin + 1) * grid.kzmax), mr["cabs"].ravel())
    r.galactic_disc3()
    Ur, Vr, _ = r.store()
    Uir, Vir, rfr = r.get_initial()
    assert np.array_equal(V, Vr)
    assert np.array_equal(U, Ur)
    assert np.array_equal(Ui, Uir) and np.array_equal(Vi, Vir) and np.array_equal(rf, rfr)
    axi_r, _ = r.gravity()
    assert np.array_equal(axi_r, grid.gravity_axi_cells())


def test_shipped_rk2_oracle_matches_reference(M, P):
    grid, params, U, V, Ui, Vi, rf = make_shipped(M, REDUCED)
    r = ref_shipped(M, P, grid, params)
    r.galactic_disc3()
    o = oracle_for(M, P, grid, params, threads=4)
    o.load(U, V, Ui, Vi, rf)
    tr = to = 0.0
    for n in range(3):
        rr = r.step(tr)
        ro = o.step(to)
        assert rr[0] == 0 and ro[0] == 0
        assert rr[1:4] == ro[1:4], "step %d t/dt/ch" % n
        assert list(rr[4]) == list(ro[4]), "step %d floor counters" % n
        tr, to = rr[1], ro[1]
    Ur, Vr, _ = r.store()
    Uo, Vo, _ = o.store()
    assert np.array_equal(Ur, Uo) and np.array_equal(Vr, Vo)
    o.close()
