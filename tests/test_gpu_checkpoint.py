"""Asynchronous checkpoint (mhd_checkpoint_begin/wait) and a restart from its
files, on the GPU.

Plain FP64 form: the files written while the disc keeps stepping hold the
state of the step the checkpoint was taken at, bit for bit (against the
oracle), and a run restarted from them (the reference's restart sequence)
continues bit-identically to the oracle run restarted the same way.
Precision form: the files equal the FP64 download of the state at that step.
"""
import numpy as np
import pytest

from mhdcase import make_case, oracle_for, run_oracle

pytestmark = pytest.mark.gpu

DIMS = (16, 16, 16)


def test_checkpoint_overlaps_steps_and_restarts_bitwise(M, P, tmp_path):
    grid, params, U, V = make_case(M, "rk3_mc_hlld_grav_cool", DIMS)
    o = oracle_for(M, P, grid, params)
    Uo3, Vo3, _, t3 = run_oracle(o, U, V, 3)
    d = M.Disc(grid, params)
    d.upload(U, V)
    M.binary_output(tmp_path, 0, 0.0, grid, V)          # main.c:304, the initial output
    t = 0.0
    for _ in range(3):
        rc, t, *_ = d.step(t)
        assert rc == 0
    assert t == t3
    d.checkpoint_begin(tmp_path, 1, t)
    for _ in range(3):                                  # keeps stepping while the copy runs
        rc, t, *_ = d.step(t)
        assert rc == 0
    d.checkpoint_wait()
    Vf = M.restart_read(tmp_path, 1, grid)
    assert np.array_equal(Vf, Vo3)
    assert (tmp_path / "1" / "GridTime.dat").read_text() == "%d\t%d\t%d\t%.3e" % (
        grid.ixmax, grid.jymax, grid.kzmax, t3)
    # restart from output 1 on a fresh context and on the oracle
    Ur, Vr, Ui, Vi, rf, tr, tout = M.restart(tmp_path, 1, t3, grid, params)
    d2 = M.Disc(grid, params)
    d2.upload(Ur, Vr, Ui, Vi, rf)
    o2 = oracle_for(M, P, grid, params)
    o2.load(Ur, Vr, Ui, Vi, rf)
    tg = to = tr
    for _ in range(3):
        rc, tg, *_ = d2.step(tg)
        assert rc == 0
        rc, to, *_ = o2.step(to)
        assert rc == 0
    Ug, Vg = d2.download()
    Uo, Vo, _ = o2.store()
    assert tg == to
    assert np.array_equal(Ug, Uo) and np.array_equal(Vg, Vo)
    d.close()
    d2.close()
    o.close()
    o2.close()


def test_checkpoint_precision_form_matches_download(M, tmp_path):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", (24, 16, 20))
    p32 = M.default_params(**{k: v for k, v in params.as_dict().items() if k != "precision"}, precision="fp32")
    d = M.Disc(grid, p32)
    d.upload(U, V)
    t = d.run(4, 0.0)
    _, Vd = d.download()
    d.checkpoint_begin(tmp_path, 2, t)
    t = d.run(2, t)
    d.checkpoint_begin(tmp_path, 3, t)                   # waits for output 2 first
    _, Vd3 = d.download()
    d.checkpoint_wait()
    assert np.array_equal(M.restart_read(tmp_path, 2, grid), Vd)
    assert np.array_equal(M.restart_read(tmp_path, 3, grid), Vd3)
    d.close()


def test_checkpoint_reports_write_failure(M, tmp_path):
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", DIMS)
    d = M.Disc(grid, params)
    d.upload(U, V)
    blocker = tmp_path / "7"
    blocker.write_text("a file where the output directory should go")
    d.checkpoint_begin(tmp_path, 7, 0.0)
    with pytest.raises(M.MhdError) as e:
        d.checkpoint_wait()
    assert e.value.code == M.MHD_ERR_IO
    d.checkpoint_begin(tmp_path, 8, 0.0)                 # the context is still usable
    d.checkpoint_wait()
    assert np.array_equal(M.restart_read(tmp_path, 8, grid), V)
    d.close()
