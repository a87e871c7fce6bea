"""Golden vectors made by the reference C itself (tests/golden/make_golden.py)
pin the oracle and the GPU path where the reference tree is absent.

Conserved variables after 4 steps of each scheme variant on a 12x4x12 grid:
the oracle must match within 1e-12 relative L1 per variable (bit-identical on
the machine that made the vectors; across CPU architectures the C library's
transcendental functions may differ in the last bit), with identical floor
counters.  The GPU path (plain FP64) is held to the same bar."""
import os

import numpy as np
import pytest

from mhdcase import VARIANTS, rel_l1

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_case(P, name):
    inp = np.load(os.path.join(HERE, "golden_input.npz"))
    gold = np.load(os.path.join(HERE, "golden_%s.npz" % name))
    gs = dict(zip(P.GRIDSPEC_FIELDS, inp["gridspec"]))
    for k in ("ix", "jy", "kz"):
        gs[k] = int(gs[k])
    params = dict(zip(P.PARAM_FIELDS, gold["params"]))
    params.update(dict(zip(P.FLAG_FIELDS, (int(v) for v in gold["flags"]))))
    return inp["U"], inp["V"], gs, params, gold


@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_oracle_against_golden(P, name):
    U, V, gs, params, gold = load_case(P, name)
    o = P.Oracle(gs, params, threads=2)
    if params["gravity"]:
        o.initial_gravity()
    o.load(U, V)
    t = 0.0
    for n in range(len(gold["dt"])):
        rc, t, dt, ch, cnt = o.step(t)
        assert rc == 0
        assert abs(dt - gold["dt"][n]) <= 1e-14 * abs(gold["dt"][n])
        assert np.array_equal(cnt, gold["counters"][n])
    Uo, _, _ = o.store()
    err = rel_l1(Uo, gold["U"])
    assert np.all(err <= 1e-12), err
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_gpu_against_golden(M, P, name):
    import ctypes as C
    U, V, gs, params, gold = load_case(P, name)
    spec = M.MhdGridSpec(**{k: (int(v) if k in ("ix", "jy", "kz") else float(v)) for k, v in gs.items()})
    grid = M.Grid(spec)
    p = M.default_params(**{k: (int(params[k]) if k in P.FLAG_FIELDS or k == "armnum" else float(params[k]))
                            for k in list(P.PARAM_FIELDS) + list(P.FLAG_FIELDS)})
    if p.gravity:
        grid.set_initial_gravity()
    d = M.Disc(grid, p)
    d.upload(U, V)
    t = 0.0
    for n in range(len(gold["dt"])):
        rc, t, dt, ch, cnt = d.step(t)
        assert rc == 0
        assert np.array_equal(cnt, gold["counters"][n])
    Ug, _ = d.download()
    err = rel_l1(Ug, gold["U"])
    assert np.all(err <= 1e-12), err
    d.close()
