"""The TMA-staged update (precision form): each tile of 128 cells is loaded into
shared memory with tensor copies before the update runs, against the update
that loads its inputs thread by thread.

Both paths run update_core on the same values, so they may differ only
through FMA contraction choices: per-variable relative L1 of U <= 1e-6 after
5 steps (the initially-zero components against the momentum and field
scales); of V <= 1e-5, since the pressure is the small difference
(gamma-1)(E - rho v^2/2 - B^2/2) and magnifies the rounding of E (measured
1.5e-6 at 40x24x70).  The thread loads are the default; the staged
path is available wherever the layout allows it (cells per variable a
multiple of 4) and is refused elsewhere; mhd_run's captured graphs follow a
change of path.
"""
import numpy as np
import pytest

from mhdcase import make_case, rel_l1

pytestmark = pytest.mark.gpu

# (nr, nphi, nz): tiles that straddle rows, planes and the last interior plane
SHAPES = [(24, 16, 20), (40, 24, 70)]


def fp32(M, params):
    return M.default_params(**{k: v for k, v in params.as_dict().items() if k != "precision"}, precision="fp32")


def run_path(M, grid, params, U, V, nsteps, tma, use_run=False):
    d = M.Disc(grid, params)
    if tma is not None:
        d.set_update_path(tma)
    d.upload(U, V)
    path = d.update_path()
    log = []
    if use_run:
        d.run(nsteps, 0.0)
    else:
        t = 0.0
        for _ in range(nsteps):
            rc, t, dt, ch, cnt = d.step(t)
            assert rc == 0
            log.append((dt, ch, tuple(int(c) for c in cnt)))
    Ug, Vg = d.download()
    d.close()
    return Ug, Vg, log, path


def field_scaled_err(grid, Ua, Ub):
    err = rel_l1(Ua, Ub)
    x = grid.arr("x", grid.ixmax)[:, None, None]
    mscale = np.abs(Ub[2] / x).sum()
    bscale = max(np.abs(Ub[4:7]).sum(), 1e-300)
    err[3] = np.abs(Ua[3] - Ub[3]).sum() / mscale
    for m in (4, 6, 8):
        err[m] = np.abs(Ua[m] - Ub[m]).sum() / bscale
    return err


@pytest.mark.parametrize("variant", ["rk3_mc_hlld_grav_cool", "rk2_mc_hll_grav_cool", "rk3_vanleer_hlld"])
@pytest.mark.parametrize("dims", SHAPES)
def test_staged_update_matches_loads(M, variant, dims):
    grid, params, U, V = make_case(M, variant, dims)
    p32 = fp32(M, params)
    Ut, Vt, logt, path = run_path(M, grid, p32, U, V, 5, 1)
    assert path == 1
    Ul, Vl, logl, path0 = run_path(M, grid, p32, U, V, 5, None)
    assert path0 == 0, "thread loads are the default"
    assert [c for _, _, c in logt] == [c for _, _, c in logl], "floor counters"
    assert np.all(field_scaled_err(grid, Ut, Ul) <= 1e-6)
    assert np.all(field_scaled_err(grid, Vt, Vl) <= 1e-5)


def test_run_graphs_follow_update_path(M):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld_axi_cool", (40, 24, 70))
    p32 = fp32(M, params)
    Ua, Va, _, _ = run_path(M, grid, p32, U, V, 4, 1, use_run=True)
    d = M.Disc(grid, p32)
    d.upload(U, V)
    d.run(1, 0.0)                      # graphs captured with the thread-load update
    d.set_update_path(1)               # must drop them
    d.upload(U, V)
    d.run(4, 0.0)
    Ub, Vb = d.download()
    d.close()
    assert np.array_equal(Ua, Ub) and np.array_equal(Va, Vb)


def test_staged_update_refused_where_unavailable(M):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (24, 16, 20))
    d = M.Disc(grid, params)           # plain FP64 form: loads only
    assert d.update_path() == 0
    with pytest.raises(M.MhdError) as e:
        d.set_update_path(1)
    assert e.value.code == M.MHD_ERR_ARG
    d.close()
    # 15 x 10 x 15 = 2250 cells per variable (not a multiple of 4): rows of the
    # tensor view would not start on 16-byte boundaries, so the precision form
    # keeps the loads
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (13, 8, 13))
    d = M.Disc(grid, fp32(M, params))
    assert d.update_path() == 0
    with pytest.raises(M.MhdError):
        d.set_update_path(1)
    d.upload(U, V)
    t = 0.0
    for _ in range(2):
        rc, t, *_ = d.step(t)
        assert rc == 0
    d.close()


@pytest.mark.parametrize("dims", SHAPES + [(13, 8, 13)])
def test_prefetching_update_is_bitwise_the_loads(M, dims):
    """Path 2: the same thread loads, with each block prefetching the block one
    wave ahead into L2 -- the same arithmetic, so the same bits."""
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", dims)
    p32 = fp32(M, params)
    Up, Vp, logp, path = run_path(M, grid, p32, U, V, 5, 2)
    assert path == 2
    Ul, Vl, logl, _ = run_path(M, grid, p32, U, V, 5, 0)
    assert logp == logl
    assert np.array_equal(Up, Ul) and np.array_equal(Vp, Vl)
    d = M.Disc(grid, params)           # plain FP64 form: not offered
    with pytest.raises(M.MhdError):
        d.set_update_path(2)
    d.close()


@pytest.mark.parametrize("path", [4, 6])
@pytest.mark.parametrize("variant", ["rk3_mc_hlld_grav_cool", "rk2_mc_hll_grav_cool"])
def test_primitives_from_state_match_loads(M, variant, path):
    """Paths 4 and 6: the update forms the cell's input primitives as UtoV of
    its input state U^(k) instead of loading V (which holds UtoV of the same
    state, corrected by Check where a floor fired), 6 with the L2 prefetch of
    path 2.  Same values up to rounding where floors fired."""
    grid, params, U, V = make_case(M, variant, (40, 24, 70))
    p32 = fp32(M, params)
    Uw, Vw, logw, p = run_path(M, grid, p32, U, V, 5, path)
    assert p == path
    Ul, Vl, logl, _ = run_path(M, grid, p32, U, V, 5, 0)
    assert [c for _, _, c in logw] == [c for _, _, c in logl], "floor counters"
    assert np.all(field_scaled_err(grid, Uw, Ul) <= 1e-6)
    assert np.all(field_scaled_err(grid, Vw, Vl) <= 1e-5)
