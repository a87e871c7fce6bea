"""Checkpoint files and the restart sequence (host side, no GPU).

The product's BinaryOutput must write the same bytes as the reference's own
BinaryOutput (output.h:1202-1414) for the same state, and its restart
sequence (main.c:244-270: RestartRead(0), SaveInitial, RestartRead(nout),
each RestartRead = files + VtoU + Check) must leave the same U, V, initial
arrays, floors and floor counters as the reference's RestartRead."""
import os

import numpy as np
import pytest

from conftest import reference_tree_present
from mhdcase import make_case

DIMS = (16, 16, 16)
NAMES = ["GridTime.dat", "r", "phi", "z", "rho", "vr", "vphi", "vz", "br", "bphi", "bz", "pr", "psi"]

needs_ref = pytest.mark.skipif(not reference_tree_present(), reason="reference tree not present")


class chdir:
    def __init__(self, d):
        self.d = d

    def __enter__(self):
        self.old = os.getcwd()
        os.chdir(self.d)

    def __exit__(self, *a):
        os.chdir(self.old)


def evolved_state(M, P, variant="rk3_mc_hlld_grav_cool", nsteps=3):
    grid, params, U, V = make_case(M, variant, DIMS)
    r = P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params))
    if params.gravity:
        r.initial_gravity()
    r.load(U, V)
    t = 0.0
    for _ in range(nsteps):
        rc, t, *_ = r.step(t)
        assert rc == 0
    Ur, Vr, _ = r.store()
    return grid, params, U, V, Vr, t


@needs_ref
def test_binary_output_bytes_match_reference(M, P, tmp_path):
    grid, params, U0, V0, V, t = evolved_state(M, P)
    r = P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params))
    r.load(M.vtou(grid, V), V)
    a, b = tmp_path / "ref", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    with chdir(a):
        r.binary_output(7, t)
    M.binary_output(b, 7, t, grid, V)
    for name in NAMES:
        ra, rb = (a / "7" / name).read_bytes(), (b / "7" / name).read_bytes()
        assert ra == rb, name
    assert (b / "7" / "GridTime.dat").read_text() == "%d\t%d\t%d\t%.3e" % (grid.ixmax, grid.jymax, grid.kzmax, t)
    assert len((b / "7" / "rho").read_bytes()) == 8 * grid.ixmax * grid.jymax * grid.kzmax


def plant_floor_cases(grid, V, seed=3):
    """A copy of V with cells that each Check floor catches."""
    V = V.copy()
    rng = np.random.default_rng(seed)
    cells = [tuple(rng.integers(0, n) for n in grid.cell) for _ in range(12)]
    for n, c in enumerate(cells):
        if n % 3 == 0:
            V[(0,) + c] = 1e-12               # below rhofloor
        elif n % 3 == 1:
            V[(7,) + c] = -1e-3               # negative pressure
        else:
            V[(4,) + c] = 5.0                 # plasma beta below betacr
    return V


@needs_ref
def test_restart_matches_reference(M, P, tmp_path):
    grid, params, U0, V0, V, t = evolved_state(M, P)
    Vp = plant_floor_cases(grid, V)
    M.binary_output(tmp_path, 0, 0.0, grid, V0)
    M.binary_output(tmp_path, 2, t, grid, Vp)
    # the reference: fresh globals (zero floors), then main.c:250-258
    r = P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params))
    with chdir(tmp_path):
        c0 = r.restart_read(0)
        r.save_initial()
        c2 = r.restart_read(2)
    Ur, Vr, _ = r.store()
    Uir, Vir, rfr = r.get_initial()
    # the product, step by step and in one call
    V0p = M.restart_read(tmp_path, 0, grid)
    U0p = M.vtou(grid, V0p)
    d0 = M.check_floors(grid, params, U0p, V0p, np.zeros(grid.cell))
    assert list(d0) == list(c0)
    V2p = M.restart_read(tmp_path, 2, grid)
    U2p = M.vtou(grid, V2p)
    rf = U0p[0] * params.rhocr
    d2 = M.check_floors(grid, params, U2p, V2p, rf)
    assert list(d2) == list(c2) and sum(d2) >= 12
    assert np.array_equal(U2p, Ur) and np.array_equal(V2p, Vr)
    U, Vv, Ui, Vi, rfp, tt, tout = M.restart(tmp_path, 2, 0.05, grid, params)
    assert np.array_equal(U, Ur) and np.array_equal(Vv, Vr)
    assert np.array_equal(Ui, Uir) and np.array_equal(Vi, Vir) and np.array_equal(rfp, rfr)
    assert tt == 2 * 0.05 and tout == 3 * 0.05


def test_binary_output_round_trip(M, tmp_path):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (12, 8, 12))
    M.binary_output(tmp_path, 4, 1.25, grid, V)
    assert np.array_equal(M.restart_read(tmp_path, 4, grid), V)
    assert np.array_equal(np.fromfile(tmp_path / "4" / "r"), grid.arr("x", grid.ixmax))
    assert np.array_equal(np.fromfile(tmp_path / "4" / "phi"), grid.arr("y", grid.jymax))
    assert np.array_equal(np.fromfile(tmp_path / "4" / "z"), grid.arr("z", grid.kzmax))
    # an existing output directory is reused, as mkdir in output.h:1208 allows
    M.binary_output(tmp_path, 4, 1.25, grid, V)


def test_restart_errors(M, tmp_path):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (12, 8, 12))
    with pytest.raises(M.MhdError) as e:
        M.restart_read(tmp_path, 9, grid)            # no such output
    assert e.value.code == M.MHD_ERR_IO
    M.binary_output(tmp_path, 1, 0.0, grid, V)
    (tmp_path / "1" / "pr").write_bytes(b"\0" * 16)   # truncated file
    with pytest.raises(M.MhdError) as e:
        M.restart_read(tmp_path, 1, grid)
    assert e.value.code == M.MHD_ERR_IO
    x = grid.arr("x", grid.ixmax)
    assert M.lib().mhd_binary_output_arrays(b"x", -1, 0.0, 12, 8, 12, x, x, x, V) == M.MHD_ERR_ARG
    assert M.lib().mhd_restart_read(str(tmp_path).encode(), 1, 0, 8, 12, V) == M.MHD_ERR_ARG


@needs_ref
def test_text_outputs_match_reference(M, P, tmp_path):
    """GNUOutputCylinder / GDLOutputCylinder: the same files, byte for byte, on
    the shipped grid family (the reference cuts at radial index 160)."""
    from mhdcase import make_shipped
    grid, params, U, V, Ui, Vi, rf = make_shipped(M, (220, 8, 120))
    r = P.RefOracle(grid.ix, grid.jy, grid.kz, M.oracle_params(params), shipped=True)
    r.galactic_disc3()
    Ur, Vr, _ = r.store()
    a, b = tmp_path / "ref", tmp_path / "lib"
    a.mkdir()
    b.mkdir()
    with chdir(a):
        r.text_output(5, 1234, 0.25)
    M.text_output(b, 5, 1234, 0.25, grid, Ur, Vr)
    names = sorted(p.name for p in a.iterdir())
    assert names == sorted(p.name for p in b.iterdir()) and len(names) == 10
    for name in names:
        assert (a / name).read_bytes() == (b / name).read_bytes(), name
    small, params2, U2, V2 = make_case(M, "rk3_minmod_hlld", (64, 8, 12))
    with pytest.raises(M.MhdError) as e:
        M.text_output(b, 1, 0, 0.0, small, U2, V2)      # no radial index 160 on this grid
    assert e.value.code == M.MHD_ERR_ARG
