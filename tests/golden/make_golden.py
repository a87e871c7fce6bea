"""Generate the golden vectors in this directory from the reference C itself.

Runs only where the reference tree exists: builds the reference in place
(oracle/build_ref.py) for a 12x4x12 grid, and for each scheme variant runs 4
steps of the reference's own step (ref_harness.c: Setdt, SpiralGravity, TVDRK
as in main.c:319-351) from one seeded initial state.  Writes
golden_input.npz (the initial state and grid spec) and golden_<variant>.npz
(U after the steps, per-step dt, ch and floor counters).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

DIMS = (12, 4, 12)
NSTEPS = 4


def main():
    from conftest import load_mhdgpu
    from mhdcase import VARIANTS, make_case
    import pyoracle
    M = load_mhdgpu()
    grid, params, U, V = make_case(M, "rk3_minmod_hlld", DIMS)
    gs = grid.spec.as_dict()
    np.savez_compressed(os.path.join(HERE, "golden_input.npz"), U=U, V=V,
                        gridspec=np.array([gs[k] for k in pyoracle.GRIDSPEC_FIELDS], dtype=np.float64))
    for name in sorted(VARIANTS):
        _, p, _, _ = make_case(M, name, DIMS)
        op = M.oracle_params(p)
        r = pyoracle.RefOracle(*DIMS, op)
        if p.gravity:
            r.initial_gravity()
        r.load(U, V)
        t = 0.0
        dts, chs, cnts = [], [], []
        for _ in range(NSTEPS):
            rc, t, dt, ch, cnt = r.step(t)
            assert rc == 0
            dts.append(dt)
            chs.append(ch)
            cnts.append(cnt.copy())
        Uo, Vo, _ = r.store()
        np.savez_compressed(os.path.join(HERE, "golden_%s.npz" % name), U=Uo, dt=np.array(dts),
                            ch=np.array(chs), counters=np.array(cnts),
                            params=np.array([op[f] for f in pyoracle.PARAM_FIELDS]),
                            flags=np.array([op[f] for f in pyoracle.FLAG_FIELDS], dtype=np.int32))
        print(name, "dt", dts[-1], "counters", cnts[-1])


if __name__ == "__main__":
    main()
