"""The batched form: uneven discs in one persistent launch per RK stage.

Each disc of a batch must follow the same trajectory as the same disc stepped
alone by the device-resident single-disc path (mhd_run) -- the same per-cell
code, the same device-side dt -- to 1e-6 relative L1, and stay within the
precision form's tolerance of its own plain FP64 run."""
import numpy as np
import pytest

from mhdcase import rel_l1

pytestmark = pytest.mark.gpu

SIZES = [(16, 16, 16), (24, 8, 20), (32, 12, 14), (20, 16, 24)]


def make_discs(M, fp="fp32", dtmin_bad=None):
    cases = []
    for d, dims in enumerate(SIZES):
        over = dict(precision=fp, epssp0=0.01 * (d + 1), omegapattern=0.3 + 0.1 * d, beta=1.0 + 10 * d,
                    limiter="minmod" if d % 2 == 0 else "mc")
        if dtmin_bad is not None and d == dtmin_bad:
            over["dtmin"] = 1.0e3
        (nr, nphi, nz), params, ic = M.workload("disc2", nr=dims[0], nphi=dims[1], nz=dims[2], **over)
        ic["seed"] = 50 + d
        grid = M.Grid.disc(nr, nphi, nz)
        grid.set_initial_gravity()
        U, V = grid.ic_disc(**ic)
        cases.append((grid, params, U, V))
    return cases


def test_batch_matches_single_disc_runs(M):
    cases = make_discs(M)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t = np.zeros(len(cases))
    t, st = b.step(3, t)
    t, st = b.step(2, t)
    assert np.all(st == 0)
    for d, (g, p, U, V) in enumerate(cases):
        s = M.Disc(g, p)
        s.upload(U, V)
        ts = s.run(5, 0.0)
        Us, _ = s.download()
        Ub, _ = b.download(d)
        # the default (persistent) mode's flux kernels compute the same faces
        # with other FP32 roundings: dt follows the state to the form's precision
        assert abs(ts - t[d]) <= 1e-7 * ts, d
        err = rel_l1(Ub[:8], Us[:8])
        # B_r, B_z start at zero in these discs: against the field scale
        bscale = np.abs(Us[4:7]).sum()
        for m in (4, 6):
            err[m] = np.abs(Ub[m] - Us[m]).sum() / bscale
        assert np.all(err <= 1e-6), (d, err)
        s.close()
    b.close()


def test_batch_against_fp64(M):
    """Every disc of the batch against its own plain FP64 run after 4 steps, on
    all nine conserved variables: within 3x that disc's FP32-storage floor
    (FP64 arithmetic, U and V rounded to FP32 after every stage, rounded
    start) plus 1e-7 -- after 4 steps both are single realisations of
    rounding noise a few times 1e-7 -- and within 1e-4 on the order-one
    components."""
    cases = make_discs(M)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(4, np.zeros(len(cases)))

    def run64(g, pd, U0, V0, round_state):
        s = M.Disc(g, M.default_params(precision="fp64", **pd))
        if round_state:
            s.set_state_rounding(True)
        s.upload(U0, V0)
        tt = 0.0
        for _ in range(4):
            rc, tt, *_ = s.step(tt)
        Uf, _ = s.download()
        s.close()
        return Uf

    for d, (g, p, U, V) in enumerate(cases):
        pd = p.as_dict()
        pd.pop("precision")
        U64 = run64(g, pd, U, V, False)
        Ufl = run64(g, pd, U.astype(np.float32).astype(np.float64), V.astype(np.float32).astype(np.float64), True)
        Ub, _ = b.download(d)
        err, floor = rel_l1(Ub, U64), rel_l1(Ufl, U64)
        assert np.all(err <= 3.0 * floor + 1e-7), (d, err, floor)
        assert np.all(err[[0, 1, 2, 5, 7]] <= 1e-4), (d, err)
    b.close()


def test_batch_per_disc_dt_guard(M):
    cases = make_discs(M, dtmin_bad=2)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(3, np.zeros(len(cases)))
    assert st[2] == M.MHD_ERR_DT and t[2] == 0.0
    assert all(st[d] == 0 and t[d] > 0 for d in (0, 1, 3))
    U2, _ = b.download(2)
    # frozen: the uploaded state as the precision form stores it (FP32)
    assert np.array_equal(U2, cases[2][2].astype(np.float32).astype(np.float64))
    b.close()


def test_batch_tune_restores_state(M):
    cases = make_discs(M)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(2, np.zeros(len(cases)))
    before = [b.download(d) for d in range(len(cases))]
    best = b.tune()
    if best[4] == 2:
        assert best[0] in (2, 3, 4)          # branches, capped at the 4 discs here
    else:
        assert best[3] in (64, 128, 256, 512) and best[2] > 0 and best[4] in (0, 1)
    for d in range(len(cases)):
        Ua, Va = b.download(d)
        assert np.array_equal(Ua, before[d][0]) and np.array_equal(Va, before[d][1])
    t2, st2 = b.step(2, t)
    assert np.all(st2 == 0) and np.all(t2 > t)
    b.close()


def test_batch_plain_fp64_is_bitwise_per_disc(M):
    cases = make_discs(M, fp="fp64")[:2]
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(2, np.zeros(2))
    for d, (g, p, U, V) in enumerate(cases):
        s = M.Disc(g, p)
        s.upload(U, V)
        tt = 0.0
        for _ in range(2):
            rc, tt, *_ = s.step(tt)
        Us, _ = s.download()
        Ub, _ = b.download(d)
        assert np.array_equal(Us, Ub)
        s.close()
    b.close()


@pytest.mark.parametrize("mode,arg", [(2, 3), (2, 1), (1, 0), (0, 0)])
def test_batch_modes_match_single_disc_runs(M, mode, arg):
    """Each mode against the discs stepped alone (mhd_run).  The disc graph
    runs the single-disc kernels themselves: bit for bit; the persistent and
    phased kernels (one thread per face, other FP32 roundings) to the
    precision form's 1e-6, and dt to 1e-7."""
    cases = make_discs(M)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    b.set_mode(mode, arg)
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(3, np.zeros(len(cases)))
    t, st = b.step(2, t)
    assert np.all(st == 0)
    for d, (g, p, U, V) in enumerate(cases):
        s = M.Disc(g, p)
        s.upload(U, V)
        ts = s.run(5, 0.0)
        Us, _ = s.download()
        Ub, _ = b.download(d)
        assert abs(ts - t[d]) <= (0.0 if mode == 2 else 1e-7) * ts, d
        if mode == 2:
            assert ts == t[d] and np.array_equal(Ub, Us), d
        else:
            err = rel_l1(Ub[:8], Us[:8])
            bscale = np.abs(Us[4:7]).sum()
            for m in (4, 6):
                err[m] = np.abs(Ub[m] - Us[m]).sum() / bscale
            assert np.all(err <= 1e-6), (d, err)
        s.close()
    with pytest.raises(M.MhdError):
        b.set_mode(2, 0)
    b.close()


def test_batch_bounded_wait_times_out_and_recovers(M):
    """The persistent kernel's waits are bounded: a flux count that is never
    reached (test hook) ends the step with MHD_ERR_TIMEOUT after the short
    limit, with no fault; with the hook cleared and the state uploaded again
    the batch steps normally."""
    cases = make_discs(M)
    b = M.Batch([c[0] for c in cases], [c[1] for c in cases])
    b.set_mode(0, 0)
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    b.debug_stall(1, 4096)
    with pytest.raises(M.MhdError) as e:
        b.step(1, np.zeros(len(cases)))
    assert e.value.code == M.MHD_ERR_TIMEOUT
    b.debug_stall(-1)
    for d, (g, p, U, V) in enumerate(cases):
        b.upload(d, U, V)
    t, st = b.step(2, np.zeros(len(cases)))
    assert np.all(st == 0)
    for d, (g, p, U, V) in enumerate(cases):
        s = M.Disc(g, p)
        s.upload(U, V)
        ts = s.run(2, 0.0)
        Us, _ = s.download()
        Ub, _ = b.download(d)
        assert abs(ts - t[d]) <= 1e-12 * ts
        err = rel_l1(Ub[:8], Us[:8])
        bscale = np.abs(Us[4:7]).sum()
        for m in (4, 6):
            err[m] = np.abs(Ub[m] - Us[m]).sum() / bscale
        assert np.all(err <= 1e-6), (d, err)
        s.close()
    b.close()
