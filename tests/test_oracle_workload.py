"""The CPU legs' own copy of the disc workloads (oracle/pyoracle.py:
workload, gridspec_disc, Oracle.ic_disc) against the product's host helpers,
so that the reference arm and the CPU baseline, which load no product
library, time the same grid, knobs and initial state."""
import numpy as np
import pytest


@pytest.mark.parametrize("name", ["disc1", "disc2", "disc3", "disc5"])
def test_workload_params_match(M, P, name):
    dims, params, ic = M.workload(name, nr=32, nphi=16, nz=24)
    odims, oparams, oic = P.workload(name, nr=32, nphi=16, nz=24)
    assert tuple(dims) == tuple(odims)
    assert ic == oic
    want = M.oracle_params(params)
    for k, v in oparams.items():
        assert want[k] == v, k


@pytest.mark.parametrize("dims", [(24, 16, 20), (512, 512, 256), (100, 36, 14)])
def test_gridspec_matches(M, P, dims):
    spec = M.Grid.disc(*dims).spec.as_dict()
    assert spec == P.gridspec_disc(*dims)


@pytest.mark.parametrize("name", ["disc1", "disc5"])
def test_ic_disc_bitwise(M, P, name):
    (nr, nphi, nz), params, ic = M.workload(name, nr=24, nphi=16, nz=20)
    grid = M.Grid.disc(nr, nphi, nz)
    U, V = grid.ic_disc(**ic)
    _, oparams, oic = P.workload(name, nr=24, nphi=16, nz=20)
    o = P.Oracle(P.gridspec_disc(nr, nphi, nz), oparams, threads=2)
    o.ic_disc(**oic)
    Uo, Vo, _ = o.store()
    # the oracle's step from its own state equals its step from the product's state
    o2 = P.Oracle(P.gridspec_disc(nr, nphi, nz), oparams, threads=2)
    o2.load(U, V)
    r1 = o.step(0.0)
    r2 = o2.step(0.0)
    U1, V1, _ = o.store()
    U2, V2, _ = o2.store()
    o.close()
    o2.close()
    assert np.array_equal(Uo, U) and np.array_equal(Vo, V)
    assert r1[0] == 0 and r1[2] == r2[2]
    assert np.array_equal(U1, U2) and np.array_equal(V1, V2)
