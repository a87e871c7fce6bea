"""The C host program (host/mhd_disc_main.c: the reference's main.c on the
C-ABI) end to end on the GPU: GalacticDisc3 on the shipped grid family, live
RK2, outputs through the asynchronous checkpoint, and the restart branch --
every output file against the oracle run the same way, bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import PKG
from mhdcase import make_shipped, oracle_for

pytestmark = pytest.mark.gpu

EXE = os.path.join(PKG, "lib", "mhd_disc")
DIMS = (220, 8, 120)
TINT = 1e-12          # every step is past the next output time: one output per step


def run_exe(*args):
    r = subprocess.run([EXE, "--grid", "%dx%dx%d" % DIMS, "--quiet"] + [str(a) for a in args],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_host_program_fresh_start_and_restart(M, P, tmp_path):
    run_exe("--root", tmp_path, "--nstop", 3, "--tint", TINT)      # nstop+1 = 4 steps (main.c:316)
    grid, params, U, V, Ui, Vi, rf = make_shipped(M, DIMS)
    assert np.array_equal(M.restart_read(tmp_path, 0, grid), V)    # the initial BinaryOutput
    o = oracle_for(M, P, grid, params)
    o.load(U, V, Ui, Vi, rf)
    t = 0.0
    for n in range(1, 5):
        rc, t, *_ = o.step(t)
        assert rc == 0
        _, Vo, _ = o.store()
        assert np.array_equal(M.restart_read(tmp_path, n, grid), Vo), "output %d" % n
        assert (tmp_path / str(n) / "GridTime.dat").read_text().endswith("%.3e" % t)
    o.close()
    # restart from output 2 (main.c:244-272: t = 2*tint), two more steps
    rdir = tmp_path / "restart"
    rdir.mkdir()
    for n in (0, 2):
        shutil.copytree(tmp_path / str(n), rdir / str(n))
    run_exe("--root", rdir, "--restart", 2, "--nstop", 1, "--tint", TINT)
    Ur, Vr, Uir, Vir, rfr, tr, _ = M.restart(rdir, 2, TINT, grid, params)
    o = oracle_for(M, P, grid, params)
    o.load(Ur, Vr, Uir, Vir, rfr)
    for n in (3, 4):
        rc, tr, *_ = o.step(tr)
        assert rc == 0
        _, Vo, _ = o.store()
        assert np.array_equal(M.restart_read(rdir, n, grid), Vo), "restart output %d" % n
    o.close()


def test_host_program_precision_form(M, P, tmp_path):
    """--fp32 --sync-output: two steps; rho, v_phi, B_phi and p of the last
    output within 1e-5 relative L1 of the FP64 oracle."""
    run_exe("--root", tmp_path, "--nstop", 1, "--tint", TINT, "--fp32", "--sync-output")
    grid, params, U, V, Ui, Vi, rf = make_shipped(M, DIMS)
    o = oracle_for(M, P, grid, params)
    o.load(U, V, Ui, Vi, rf)
    t = 0.0
    for _ in range(2):
        rc, t, *_ = o.step(t)
        assert rc == 0
    _, Vo, _ = o.store()
    o.close()
    Vg = M.restart_read(tmp_path, 2, grid)
    for m in (0, 2, 5, 7):
        err = np.abs(Vg[m] - Vo[m]).sum() / np.abs(Vo[m]).sum()
        assert err < 1e-5, (m, err)
