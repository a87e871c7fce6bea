"""The fused stage kernel (fluxes + update in one launch, fluxes kept on chip)
against the split kernels (flux r/phi/z to device memory, then update) and
against the oracle.

Plain FP64 form: both stage shapes must give the same bits as the oracle, so
they are compared bit for bit, at tile and run shapes that leave partial tiles
in every direction.  Precision form: the two shapes may differ only through
FMA contraction choices, so per-variable relative L1 <= 1e-6 after 5 steps
(the initially-zero components against the momentum and field scales).
"""
import numpy as np
import pytest

from mhdcase import VARIANTS, make_case, oracle_for, rel_l1, run_oracle

pytestmark = pytest.mark.gpu

# (nr, nphi, nz): one tile; ragged tiles in k (70 = 2x32 + 6) and j; runs in r
SHAPES = [(20, 12, 14), (40, 24, 70)]
# (fused, tj, seg): 1 = one fused stage kernel, 2 = z fluxes fused into the update, 0 = split,
# 3 = split kernels pipelined over seg slabs of i planes (uneven slabs, one slab, more slabs than planes)
STAGE = [(1, 7, 32), (1, 7, 5), (1, 7, 1), (2, 7, 32), (0, 7, 32), (3, 7, 3), (3, 7, 1), (3, 7, 64)]


def same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def run_disc(M, grid, params, U, V, nsteps, shape):
    d = M.Disc(grid, params)
    d.set_stage_shape(*shape)
    d.upload(U, V)
    t = 0.0
    log = []
    for _ in range(nsteps):
        rc, t, dt, ch, cnt = d.step(t)
        assert rc == 0
        log.append((dt, ch, tuple(int(c) for c in cnt)))
    Ug, Vg = d.download()
    d.close()
    return Ug, Vg, log


@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("dims", SHAPES)
def test_fp64_stage_shapes_bitwise(M, P, variant, dims):
    nsteps = 3
    grid, params, U, V = make_case(M, variant, dims)
    o = oracle_for(M, P, grid, params)
    Uo, Vo, log_o, _ = run_oracle(o, U, V, nsteps)
    o.close()
    for shape in STAGE:
        Ug, Vg, log = run_disc(M, grid, params, U, V, nsteps, shape)
        assert log == log_o, "shape %s: dt/ch/counters" % (shape,)
        assert same(Ug, Uo), "shape %s: U differs" % (shape,)
        assert same(Vg, Vo), "shape %s: V differs" % (shape,)


@pytest.mark.parametrize("variant", ["rk3_minmod_hlld", "rk2_mc_hll_grav_cool"])
def test_fp32_fused_matches_split(M, variant):
    grid, params, U, V = make_case(M, variant, (40, 24, 70))
    p32 = M.default_params(**{k: v for k, v in params.as_dict().items() if k != "precision"}, precision="fp32")
    Us, Vs, _ = run_disc(M, grid, p32, U, V, 5, (0, 7, 32))
    for shape in [sh for sh in STAGE if sh[0] != 0]:
        Uf, Vf, _ = run_disc(M, grid, p32, U, V, 5, shape)
        err = rel_l1(Uf, Us)
        # m_z, B_r, B_z, psi start at (or near) zero: measured against the
        # momentum and field scales
        x = grid.arr("x", grid.ixmax)[:, None, None]
        mscale = np.abs(Us[2] / x).sum()
        bscale = max(np.abs(Us[4:7]).sum(), 1e-300)
        err[3] = np.abs(Uf[3] - Us[3]).sum() / mscale
        for m in (4, 6, 8):
            err[m] = np.abs(Uf[m] - Us[m]).sum() / bscale
        assert np.all(err <= 1e-6), (shape, err)


def test_fp32_run_graph_follows_shape(M):
    """mhd_run captures the step as a graph; changing the stage shape must
    rebuild it (the result then matches a context created with that shape)."""
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (40, 24, 70))
    p32 = M.default_params(**{k: v for k, v in params.as_dict().items() if k != "precision"}, precision="fp32")
    ref = M.Disc(grid, p32)
    ref.set_stage_shape(0, 7, 32)
    ref.upload(U, V)
    ref.run(2, 0.0)
    Ur, _ = ref.download()
    ref.close()
    d = M.Disc(grid, p32)
    d.set_stage_shape(1, 7, 32)
    d.upload(U, V)
    d.run(1, 0.0)                      # graph built with the fused shape
    d.set_stage_shape(0, 7, 32)
    d.upload(U, V)
    d.run(2, 0.0)                      # must run the split kernels now
    Ud, _ = d.download()
    d.close()
    assert same(Ud, Ur)


def test_stage_shape_rejects_bad_arguments(M):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (20, 12, 14))
    d = M.Disc(grid, params)
    for bad in [(4, 7, 32), (1, 3, 32), (1, 7, 0), (3, 7, 65), (3, 7, 0)]:
        assert M.lib().mhd_set_stage_shape(d.h, *bad) == M.MHD_ERR_ARG
    d.close()
