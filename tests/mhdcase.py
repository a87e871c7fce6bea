"""Test cases shared by the CPU and GPU parity tests: named scheme variants on
small seeded disc grids, run through the oracle and/or the GPU library."""
import numpy as np

# variant -> (workload, overrides)
VARIANTS = {
    "rk3_minmod_hlld": ("disc1", {}),
    "rk2_minmod_hlld": ("disc1", {"scheme": 2}),
    "rk3_mc_hlld_grav_cool": ("disc2", {}),
    "rk3_minmod_hll": ("disc1", {"solver": "hll"}),
    "rk2_mc_hll_grav_cool": ("disc2", {"scheme": 2, "solver": "hll"}),
    "rk3_vanleer_hlld": ("disc1", {"limiter": "vanleer"}),
    "rk2_vanleer_hlld_grav_cool": ("disc2", {"scheme": 2, "limiter": "vanleer"}),
    "rk3_superbee_hll_grav_cool": ("disc2", {"solver": "hll", "limiter": "superbee"}),
    "rk2_superbee_hlld": ("disc1", {"scheme": 2, "limiter": "superbee"}),
    "rk3_minmod_hlld_axi_cool": ("disc2", {"limiter": "minmod", "source": "axi"}),
    "rk2_minmod_hll_axi": ("disc2", {"scheme": 2, "solver": "hll", "cooling": 0, "source": "axi"}),
    "rk2_mc_hlld_uniformgz": ("disc1", {"scheme": 2, "limiter": "mc", "source": "uniformgz"}),
    "rk3_vanleer_hll_nosource": ("disc1", {"solver": "hll", "limiter": "vanleer", "source": "none"}),
}


def make_case(M, variant, dims, **extra):
    """Grid, params and seeded initial state for one variant at `dims`."""
    wl, over = VARIANTS[variant]
    over = dict(over)
    over.update(extra)
    (nr, nphi, nz), params, ic = M.workload(wl, nr=dims[0], nphi=dims[1], nz=dims[2], **over)
    grid = M.Grid.disc(nr, nphi, nz)
    if params.gravity:
        grid.set_initial_gravity()
    U, V = grid.ic_disc(**ic)
    return grid, params, U, V


def oracle_for(M, P, grid, params, threads=None):
    o = P.Oracle(grid.spec.as_dict(), M.oracle_params(params), threads=threads)
    if params.gravity:
        o.initial_gravity()
    return o


def run_oracle(o, U, V, nsteps, t=0.0):
    o.load(U, V)
    log = []
    for _ in range(nsteps):
        rc, t, dt, ch, cnt = o.step(t)
        assert rc == 0
        log.append((dt, ch, tuple(int(c) for c in cnt)))
    Uo, Vo, _ = o.store()
    return Uo, Vo, log, t


def rel_l1(a, b):
    """per-variable relative L1 of a against b over all cells"""
    out = []
    for m in range(a.shape[0]):
        den = np.abs(b[m]).sum()
        num = np.abs(a[m] - b[m]).sum()
        out.append(num / den if den > 0 else num)
    return np.array(out)


def diagnostics_np(grid, U):
    """The library's mhd_diagnostics definition restated in numpy (FP64)."""
    x = grid.arr("x", grid.ixmax)
    xm = grid.arr("xm", grid.ixmax)
    dzm = grid.arr("dzm", grid.kzmax)
    z = grid.arr("z", grid.kzmax)
    dy = grid.g.dy
    dv = 0.5 * (xm[1:-1] ** 2 - xm[:-2] ** 2)[:, None] * dy * dzm[:-2][None, :]
    dv = dv[:, None, :]
    I = (slice(1, -1),) * 3
    out = {"mass": float((U[0][I] * dv).sum()), "angmom": float((U[2][I] * dv).sum()),
           "energy": float((U[7][I] * dv).sum()), "psi": float((np.abs(U[8][I]) * dv).sum())}
    xi = x[1:-1][:, None, None]
    xp = x[2:][:, None, None]
    xn = x[:-2][:, None, None]
    br, bp, bz = U[4], U[5], U[6]
    divb = ((xp * br[2:, 1:-1, 1:-1] - xn * br[:-2, 1:-1, 1:-1]) / (xi * (xp - xn))
            + (bp[1:-1, 2:, 1:-1] - bp[1:-1, :-2, 1:-1]) / (xi * 2.0 * dy)
            + (bz[1:-1, 1:-1, 2:] - bz[1:-1, 1:-1, :-2]) / (z[2:] - z[:-2])[None, None, :])
    out["maxdivb"] = float(np.abs(divb).max())
    return out


def make_shipped(M, dims=None, **over):
    """The reference's shipped production case: its stretched grid (240x64x200,
    or other cell counts with the same spacing rules), GalacticDisc3, the
    reference's own knobs (live RK2, minmod, HLLD, spiral gravity, cooling)."""
    grid = M.Grid.shipped(*(dims or (None, None, None)))
    grid.set_initial_gravity()
    params = M.default_params(**over)
    U, V, Ui, Vi, rf = grid.ic_galactic_disc3(params)
    return grid, params, U, V, Ui, Vi, rf
