#!/usr/bin/env python
"""Benchmark: zone-updates/s of the cylindrical GLM-MHD TVD-RK3 step.

Default workload (``disc5``): one 512x512x256 disc (67.1 M zones), beta = 1,
cooling on, HLLD, minmod, RK3, CFL 0.4; seeded synthetic initial state (no
dataset exists for this benchmark).  A "step" is one full RK3 step: CFL
reduction, dt guard, three stages.

* ``value``     the FP32 + FP64-repair form, state resident in HBM.
* ``fp64``      the plain FP64 form (bit-identical to the reference C), same
                workload, fewer steps; its own per-kernel times and an
                end-to-end figure through the C-ABI.
* ``e2e``       the FP32 form through the C-ABI with the reference host's own
                FP64 arrays: every step uploads U, V from pinned host memory
                (mhd_upload_state), steps, and downloads U, V (mhd_download).
* ``roofline``  the kernel with the largest share of device time, timed live
                with CUDA events around every launch on the context's stream;
                ``kernel_roofline`` the same for every kernel.
* ``host_link`` the plain pinned copy rate of this machine's host link.
* ``cpu_baseline`` the oracle (C restatement of the reference algorithm) on
                the host cores, on the full grid, a bounded number of steps.

``--impl reference`` times that CPU implementation alone (the reference's
own C cannot travel to the GPU machine; the restatement is bit-identical to it);
it loads nothing of the product.
The state is larger than L2 (129 MB), so timed steps run without a flush.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "zone-updates/s per RK3 step, FP32+FP64-repair vs plain FP64 on 1 GB300; HBM GB/s"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        if not sm:
            return None
        mx = max(float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_product():
    import __graft_entry__ as ge
    b = ge._load("mhd_build", os.path.join(ge.PKG, "build.py"))
    b.build()
    return ge._load("mhdgpu", os.path.join(ge.PKG, "mhdgpu.py"))


def make_state(M, workload, dims):
    (nr, nphi, nz), params, ic = M.workload(workload, nr=dims[0], nphi=dims[1], nz=dims[2])
    grid = M.Grid.disc(nr, nphi, nz)
    if params.gravity:
        grid.set_initial_gravity()
    U, V = grid.ic_disc(**ic)
    return grid, params, U, V


def with_precision(M, params, prec):
    d = params.as_dict()
    d.pop("precision")
    return M.default_params(precision=prec, **d)


def time_steps(M, disc, steps, warmup, prof=False, clocks=False):
    t = 0.0
    for _ in range(warmup):
        rc, t, dt, ch, cnt = disc.step(t)
        if rc != 0:
            raise RuntimeError("dt guard fired in warm-up")
    if prof:
        disc.prof(True)
    sampler = ClockSampler() if clocks else None
    if sampler:
        sampler.start()
        time.sleep(0.5)
    n0 = disc.launches()
    disc.timer_start()
    w0 = time.perf_counter()
    for _ in range(steps):
        rc, t, dt, ch, cnt = disc.step(t)
        if rc != 0:
            raise RuntimeError("dt guard fired")
    ms = disc.timer_stop()
    wall = time.perf_counter() - w0
    launches = disc.launches() - n0
    ck = sampler.stop() if sampler else None
    kern = disc.prof_read() if prof else None
    if prof:
        disc.prof(False)
    return ms, wall, launches, kern, ck


def time_run(M, disc, steps, warmup, clocks=False):
    """The precision form's timed region: K steps through mhd_run (each step one
    CUDA graph launch: CFL reduction, dt/ch/psi factor on the device, arm-phase
    table, all stages and ghost fills), bracketed by CUDA events on the
    context's stream after W warm-up steps."""
    t = disc.run(warmup, 0.0)
    sampler = ClockSampler() if clocks else None
    if sampler:
        sampler.start()
        time.sleep(0.5)
    n0 = disc.launches()
    disc.timer_start()
    w0 = time.perf_counter()
    t = disc.run(steps, t)
    ms = disc.timer_stop()
    wall = time.perf_counter() - w0
    launches = disc.launches() - n0
    ck = sampler.stop() if sampler else None
    return ms, wall, launches, ck


def cpu_baseline(workload, dims, steps=2, warmup=1):
    """The CPU baseline: the oracle (the reference algorithm restated in C,
    bit-identical to the reference C; oracle/) on all host cores, on the FULL
    grid of the workload, for a bounded number of steps -- the loop of the
    reference's main.c:316-393 (Setdt, the dt guard, SpiralGravity when
    gravity is on, the RK stages).  Grid, knobs and the seeded initial state
    come from oracle/pyoracle.py, so no product library is loaded."""
    import pyoracle
    threads = os.cpu_count() or 1
    (nr, nphi, nz), prm, ic = pyoracle.workload(workload, *dims)
    w0 = time.perf_counter()
    o = pyoracle.Oracle(pyoracle.gridspec_disc(nr, nphi, nz), prm, threads=threads)
    if prm["gravity"]:
        o.initial_gravity()
    o.ic_disc(**ic)
    t = 0.0
    for _ in range(warmup):
        rc, t, *_ = o.step(t)
        if rc != 0:
            raise RuntimeError("dt guard fired in the CPU warm-up")
    setup = time.perf_counter() - w0
    w0 = time.perf_counter()
    for _ in range(steps):
        rc, t, *_ = o.step(t)
        if rc != 0:
            raise RuntimeError("dt guard fired in the CPU run")
    el = time.perf_counter() - w0
    o.close()
    zones = nr * nphi * nz
    return {"value": zones * steps / el, "unit": "zone-updates/s", "cores": threads, "kind": "port",
            "sample": "%d timed RK3 steps (after %d untimed) of the full %dx%dx%d grid (%d zones), the oracle "
                      "C restatement of the reference algorithm (bit-identical to the reference C) with "
                      "OpenMP on %d threads" % (steps, warmup, nr, nphi, nz, zones, threads),
            "seconds": el, "seconds_per_step": el / steps, "setup_seconds": setup}


def precision_report(args):
    """FP32 + FP64-repair form against the plain FP64 form (bit-identical to the
    reference C, checked on smaller grids by the tests) after N steps from the
    same state: per conserved variable relative L1 and Linf, and the drift of
    the totals and max|div B| of both forms.  Two plain-form runs give the
    floors: fp64_twin starts from the FP32-rounded state (what one rounding of
    the start produces by itself), fp32_storage_floor also rounds U and V to
    FP32 after every stage with FP64 arithmetic (what FP32 state storage alone
    produces -- no form that stores FP32 state does better).  m_r, m_z
    (against sum |rho v_phi|) and B_r, B_z, psi (against sum |B|) are also
    reported relative to the flow's scales."""
    M = load_product()
    dims = tuple(int(v) for v in args.size.split("x")) if args.size else (256, 256, 128)
    (nr, nphi, nz), params, ic = M.workload(args.workload, nr=dims[0], nphi=dims[1], nz=dims[2],
                                             **({"solver": args.solver} if args.solver else {}))
    grid = M.Grid.disc(nr, nphi, nz)
    if params.gravity:
        grid.set_initial_gravity()
    U, V = grid.ic_disc(**ic)
    out = {"report": "precision", "workload": args.workload, "dims": dims, "steps": args.precision_report,
           "solver": "hll" if params.solver == 1 else "hlld"}
    res = {}
    # fp64_twin: the plain form from the initial state rounded to FP32 -- how far
    # a rounding-sized perturbation of the start alone carries in N steps
    U32 = U.astype(np.float32).astype(np.float64)
    V32 = V.astype(np.float32).astype(np.float64)
    for prec in ("fp64", "fp32", "fp32x2", "fp64_twin", "fp32_storage_floor"):
        d = M.Disc(grid, with_precision(M, params, prec if prec in ("fp32", "fp32x2") else "fp64"))
        if prec == "fp32_storage_floor":
            d.set_state_rounding(True)
        if prec in ("fp64_twin", "fp32_storage_floor"):
            d.upload(U32, V32)
        else:
            d.upload(U, V)
        d0 = d.diagnostics()
        t = 0.0
        w0 = time.perf_counter()
        maxdivb = d0["maxdivb"]
        psi_max = 0.0
        for n in range(args.precision_report):
            rc, t, dt, ch, cnt = d.step(t)
            if rc != 0:
                raise RuntimeError("dt guard fired at step %d" % n)
            if (n + 1) % 10 == 0 or n + 1 == args.precision_report:
                dg = d.diagnostics()
                maxdivb = max(maxdivb, dg["maxdivb"])
                psi_max = max(psi_max, dg["psi"])
        wall = time.perf_counter() - w0
        d1 = d.diagnostics()
        Uf, _ = d.download()
        d.close()
        res[prec] = Uf
        out[prec] = {"t": t, "wall_s": wall,
                     "drift": {k: (d1[k] - d0[k]) / abs(d0[k]) if d0[k] else d1[k] for k in ("mass", "angmom", "energy")},
                     "maxdivb_end": d1["maxdivb"], "maxdivb_max": maxdivb, "psi_total_max": psi_max}
    names = ["rho", "m_r", "r*m_phi", "m_z", "B_r", "B_phi", "B_z", "E", "psi"]
    b = res["fp64"]
    x = grid.arr("x", grid.ixmax)[:, None, None]
    mscale = np.abs(b[2] / x).sum()          # sum |rho v_phi|: the momentum scale
    bscale = np.abs(b[4:7]).sum()            # sum |B|: the field scale

    def compare(a):
        rl1, linf, scaled = {}, {}, {}
        for m in range(9):
            diff = np.abs(a[m] - b[m])
            den = np.abs(b[m]).sum()
            rl1[names[m]] = float(diff.sum() / den) if den > 0 else float(diff.sum())
            sc = np.abs(b[m]).max()
            linf[names[m]] = float(diff.max() / sc) if sc > 0 else float(diff.max())
            # components that start at (or near) zero, against the flow's scales
            if m in (1, 3):
                scaled[names[m]] = float(diff.sum() / mscale)
            elif m in (4, 6, 8):
                scaled[names[m]] = float(diff.sum() / bscale)
        return {"rel_l1": rl1, "rel_linf": linf, "rel_l1_of_scale": scaled}

    out["fp32_vs_fp64"] = compare(res["fp32"])
    out["fp32x2_vs_fp64"] = compare(res["fp32x2"])
    out["fp64_twin_vs_fp64"] = compare(res["fp64_twin"])
    out["fp32_storage_floor_vs_fp64"] = compare(res["fp32_storage_floor"])
    print(json.dumps(out))
    return 0


def monitor_run(args):
    """A long run with both Riemann solvers (and, on request, both forms):
    max|div B|, sum|psi| dV and the conservation totals (FP64 diagnostics on the
    device) every args.monitor_every steps, and the device time per step.  The
    precision form runs mhd_run (device-resident dt, one graph per step)
    between diagnostics; the plain form runs mhd_step."""
    M = load_product()
    dims = tuple(int(v) for v in args.size.split("x")) if args.size else (512, 512, 256)
    out = {"report": "monitor", "workload": args.workload, "dims": dims, "steps": args.monitor}
    runs = [(s_, p_) for p_ in args.monitor_forms.split(",") for s_ in args.monitor_solvers.split(",")]
    for solver, prec in runs:
        (nr, nphi, nz), params, ic = M.workload(args.workload, nr=dims[0], nphi=dims[1], nz=dims[2], solver=solver,
                                                 precision=prec)
        grid = M.Grid.disc(nr, nphi, nz)
        if params.gravity:
            grid.set_initial_gravity()
        U, V = grid.ic_disc(**ic)
        d = M.Disc(grid, params)
        d.upload(U, V)
        d0 = d.diagnostics()
        rows = [{"step": 0, "t": 0.0, "maxdivb": d0["maxdivb"], "psi": d0["psi"], "mass": d0["mass"],
                 "angmom": d0["angmom"], "energy": d0["energy"]}]
        t, done, dev_ms = 0.0, 0, 0.0
        while done < args.monitor:
            n = min(args.monitor_every, args.monitor - done)
            d.timer_start()
            if prec == "fp32":
                t = d.run(n, t)
            else:
                for _ in range(n):       # the plain form steps with host exp/sincos
                    rc, t, *_ = d.step(t)
                    if rc != 0:
                        raise RuntimeError("dt guard fired")
            dev_ms += d.timer_stop()
            done += n
            dg = d.diagnostics()
            rows.append({"step": done, "t": t, "maxdivb": dg["maxdivb"], "psi": dg["psi"], "mass": dg["mass"],
                         "angmom": dg["angmom"], "energy": dg["energy"]})
        d.close()
        zones = nr * nphi * nz
        out[solver + "_" + prec] = {"ms_per_step": dev_ms / args.monitor,
                                    "zone_updates_per_s": zones * args.monitor / (dev_ms / 1e3), "rows": rows}
    print(json.dumps(out))
    return 0


def batch_bench(args):
    """Batched workload: 64 uneven discs (sizes from seed 7), precision form.
    value = all zones of all discs x steps / device time of the persistent
    batched step (after mhd_batch_tune); sequential = the same discs stepped
    one after another with the single-disc device-resident path (mhd_run).
    --batch-check N adds each disc's error against its own plain FP64 run
    after N steps."""
    M = load_product()
    n = int(args.workload[5:] or 64)
    wl = M.batch_workload(n=n, seed=7)
    grids, params, states = [], [], []
    for dims, p, ic in wl:
        g = M.Grid.disc(*dims)
        g.set_initial_gravity()
        U, V = g.ic_disc(**ic)
        grids.append(g)
        params.append(p)
        states.append((U, V))
    zones = sum(g.ix * g.jy * g.kz for g in grids)
    b = M.Batch(grids, params)
    for d, (U, V) in enumerate(states):
        b.upload(d, U, V)
    t = np.zeros(n)
    t, st = b.step(1, t)
    w0 = time.perf_counter()
    best = b.tune()
    tune_s = time.perf_counter() - w0
    # every mode the tuner chooses among, timed on its own over a few steps
    mode_ms = {}
    for name, mode, arg in ([("persistent_%d" % c, 0, c) for c in range(8)] +
                            [("phased", 1, 0)] + [("disc_graph_%d" % k, 2, k) for k in (4, 16)]):
        bm = M.Batch(grids, params)
        for d, (U, V) in enumerate(states):
            bm.upload(d, U, V)
        bm.set_mode(mode, arg)
        tm, _ = bm.step(2, np.zeros(n))
        w0 = time.perf_counter()
        bm.step(5, tm)
        mode_ms[name] = (time.perf_counter() - w0) / 5 * 1e3
        bm.close()
    t, st = b.step(args.warmup, t)
    sampler = ClockSampler()
    sampler.start()
    time.sleep(0.3)
    w0 = time.perf_counter()
    t, st = b.step(args.steps, t)
    wall = time.perf_counter() - w0
    clocks = sampler.stop()
    stopped = int((st != 0).sum())
    b.close()
    # sequential single-disc device-resident path
    seq_wall = 0.0
    for d in range(n):
        disc = M.Disc(grids[d], params[d])
        disc.upload(*states[d])
        tt = disc.run(1 + args.warmup, 0.0)
        w0 = time.perf_counter()
        disc.run(args.steps, tt)
        seq_wall += time.perf_counter() - w0
        disc.close()
    out = {"metric": "zone-updates/s, batched discs (FP32 + FP64 repair)", "workload": "batch%d" % n,
           "discs": n, "zones": zones, "steps": args.steps, "warmup": args.warmup,
           "value": zones * args.steps / wall, "unit": "zone-updates/s", "ms_per_step": wall / args.steps * 1e3,
           "sequential_single_disc": {"value": zones * args.steps / seq_wall, "ms_per_step": seq_wall / args.steps * 1e3},
           "tuned": ({"mode": "disc_graph", "branches": best[0], "tune_seconds": tune_s} if best[4] == 2 else
                     {"mode": "phased", "tune_seconds": tune_s} if best[4] == 1 else
                     {"mode": "persistent", "slab_planes": best[0], "queue_lag": best[1],
                      "registers_per_thread": best[2], "threads": best[3], "tune_seconds": tune_s}),
           "modes_ms_per_step": mode_ms,
           "discs_stopped_by_dt_guard": stopped, "clocks": clocks,
           "sizes": [list(dims) for dims, _, _ in wl]}
    if args.batch_check:
        errs, twin, floor = [], [], []
        b = M.Batch(grids, params)
        for d, (U, V) in enumerate(states):
            b.upload(d, U, V)
        mode = args.batch_check_mode
        if mode == "tuned":
            b.set_mode(best[4], best[0] if best[4] == 2 else 0)
        else:
            mm, _, arg = mode.partition(":")
            b.set_mode(int(mm), int(arg or 0))
        _, st32 = b.step(args.batch_check, np.zeros(n))
        stopped64 = {"fp64": 0, "twin": 0, "floor": 0}

        def run64(d, U, V, what):
            pd = params[d].as_dict()
            pd.pop("precision")
            s64 = M.Disc(grids[d], M.default_params(precision="fp64", **pd))
            if what == "floor":
                s64.set_state_rounding(True)
            s64.upload(U, V)
            tt = 0.0
            for _ in range(args.batch_check):
                rc, tt, *_ = s64.step(tt)
                if rc != 0:          # dt guard: this disc stops, as in the batch
                    stopped64[what] += 1
                    break
            Uo, _ = s64.download()
            s64.close()
            return Uo

        def rel(a, ref):
            return [float(np.abs(a[m] - ref[m]).sum() / max(np.abs(ref[m]).sum(), 1e-300)) for m in range(9)]

        for d in range(n):
            U, V = states[d]
            U64 = run64(d, U, V, "fp64")
            Ub, _ = b.download(d)
            errs.append(rel(Ub, U64))
            # the plain form from the FP32-rounded start (twin), and with the
            # state also rounded to FP32 after every stage (the storage floor)
            U32, V32 = U.astype(np.float32).astype(np.float64), V.astype(np.float32).astype(np.float64)
            twin.append(rel(run64(d, U32, V32, "twin"), U64))
            floor.append(rel(run64(d, U32, V32, "floor"), U64))
        b.close()
        errs, twin, floor = np.array(errs), np.array(twin), np.array(floor)
        names = ["rho", "m_r", "r*m_phi", "m_z", "B_r", "B_phi", "B_z", "E", "psi"]
        ratio = errs / np.maximum(floor, 1e-300)
        out["fp64_check"] = {"steps": args.batch_check, "mode": mode,
                             "stopped_by_dt_guard": {"batch": int(np.count_nonzero(st32)), **stopped64},
                             "max_over_discs_rel_l1": dict(zip(names, errs.max(axis=0).tolist())),
                             "median_over_discs_rel_l1": dict(zip(names, np.median(errs, axis=0).tolist())),
                             "storage_floor_median_over_discs_rel_l1": dict(zip(names, np.median(floor, axis=0).tolist())),
                             "storage_floor_max_over_discs_rel_l1": dict(zip(names, floor.max(axis=0).tolist())),
                             "fp64_twin_median_over_discs_rel_l1": dict(zip(names, np.median(twin, axis=0).tolist())),
                             "fp64_twin_max_over_discs_rel_l1": dict(zip(names, twin.max(axis=0).tolist())),
                             "err_over_floor_median": dict(zip(names, np.median(ratio, axis=0).tolist())),
                             "err_over_floor_max": dict(zip(names, ratio.max(axis=0).tolist())),
                             "worst_disc_by_rho": int(np.argmax(errs[:, 0]))}
    print(json.dumps(out))
    return 0


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_init(world):
    """One process per GPU under torchrun: a gloo group for the barrier and
    the max-over-ranks timing only (the replicas exchange no data)."""
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x):
    """The largest of every rank's x (x itself on one process)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def select_device(M, local, world):
    """One process per GPU: bind this rank's device -- its local rank among
    the visible devices -- before any context exists.  Returns the ordinal
    (None on one process, which keeps the current device)."""
    if world <= 1:
        return None
    M.use_device(local)
    return M.current_device()


def kernel_bytes(dims, s, pair=False):
    """Algorithmic bytes per launch of each kernel: its unique inputs and
    outputs, s bytes per value (4 in the precision form, 8 in the plain form).
    A flux kernel reads each cell's 9 primitives once and writes 9 fluxes per
    face (18 values per face); the update reads V, the three fluxes (27 values
    with their lower neighbours), U^n, U^(k) in two of the three RK3 stages and
    the density floor, and writes U and V (70 values per cell averaged over
    the stages); the CFL reduction reads 8 primitives of the cells of its
    range (i < ixmax-11).  pair: the pair-state form, whose update also moves
    the low words of U^n, U^(k) and U (94 values per cell averaged: 82, 100,
    100 by stage)."""
    nx, ny, nz = dims
    zones = nx * ny * nz
    return {"flux_r": (nx + 1) * ny * nz * 18 * s,
            "flux_phi": nx * (ny + 1) * nz * 18 * s,
            "flux_z": nx * ny * (nz + 1) * 18 * s,      # every z face (the row walk and the last face of each row)
            "update": zones * (94 if pair else 70) * s,
            "setdt": (nx - 10) * ny * nz * 8 * s,
            "ghost": 0, "trig": 0, "convert": 0,
            "stage": zones * (9 + 9 + 1 + 9 + 9 + 6) * s,
            "zupdate": zones * (70 - 9) * s}


def kernel_rooflines(kern, nbytes, peak):
    """Per kernel: algorithmic bytes per launch / mean CUDA-event launch time,
    against the HBM peak."""
    out = {}
    for k, (ms, n) in kern.items():
        if not n or not nbytes.get(k):
            continue
        gbs = nbytes[k] / (ms / n / 1e3) / 1e9
        out[k] = {"launch_ms": ms / n, "bytes_per_launch": nbytes[k], "gbs": gbs, "frac_hbm": gbs / peak,
                  "launches": n}
    return out


def e2e_steps(M, disc, U, V, steps, warmup, dist=None, with_v=True):
    """The metric end to end through the C-ABI: each step uploads the state
    from pinned FP64 host arrays (mhd_upload_state), steps (mhd_step) and
    downloads it (mhd_download); each step timed on the context's stream on
    its own.  with_v=False moves the conserved state U alone: the device forms
    V = UtoV(U) after the upload, half the bytes each way."""
    Uh = np.ascontiguousarray(U.copy())
    Vh = np.ascontiguousarray(V.copy()) if with_v else None
    M.pin(Uh)
    if with_v:
        M.pin(Vh)
    t = 0.0
    for _ in range(warmup):
        disc.upload_state(Uh, Vh)
        rc, t, *_ = disc.step(t)
        disc.download_into(Uh, Vh)
    step_ms = []
    if dist:
        dist.barrier()
    for _ in range(steps):
        disc.timer_start()
        disc.upload_state(Uh, Vh)
        rc, t, *_ = disc.step(t)
        if rc != 0:
            raise RuntimeError("dt guard fired")
        disc.download_into(Uh, Vh)
        step_ms.append(disc.timer_stop())
    M.pin(Uh, False)
    if with_v:
        M.pin(Vh, False)
    return step_ms


def host_link(M, disc, U, V, reps=2):
    """Plain pinned host<->device copy rate on this machine: the plain form's
    mhd_upload_state / mhd_download move U and V with one cudaMemcpyAsync each
    (no conversion), timed on the context's stream."""
    Uh = np.ascontiguousarray(U.copy())
    Vh = np.ascontiguousarray(V.copy())
    M.pin(Uh)
    M.pin(Vh)
    nb = Uh.nbytes + Vh.nbytes
    up, down = [], []
    for _ in range(reps + 1):
        disc.timer_start()
        disc.upload_state(Uh, Vh)
        up.append(disc.timer_stop())
        disc.timer_start()
        disc.download_into(Uh, Vh)
        down.append(disc.timer_stop())
    M.pin(Uh, False)
    M.pin(Vh, False)
    return {"h2d_gbs": nb / (min(up[1:]) / 1e3) / 1e9, "d2h_gbs": nb / (min(down[1:]) / 1e3) / 1e9,
            "bytes": nb, "what": "pinned FP64 U, V: one cudaMemcpyAsync per array (plain form's "
                                 "mhd_upload_state / mhd_download), best of %d" % reps}


def reference_arm(args, dims, cfg):
    """--impl reference: the reference's algorithm on the CPU (the oracle),
    full grid, a bounded number of steps; loads no product library."""
    steps = max(1, min(args.steps, 3))
    warmup = min(max(args.warmup, 0), 1)
    cb = cpu_baseline(args.workload, dims, steps=steps, warmup=warmup)
    out = {"metric": METRIC, "value": cb["value"], "unit": "zone-updates/s", "n_gpus": args.gpus,
           "steps": steps, "warmup": warmup, "ms_per_step": cb["seconds_per_step"] * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded disc initial state; no public dataset exists)", "impl": "reference",
           "config": cfg,
           "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
           "e2e": {"value": cb["value"], "unit": "zone-updates/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "note": "each step is a full RK3 step of the stated grid; the arm times min(steps, 3) of them "
                   "after min(warmup, 1) untimed ones so the run stays within a few minutes"}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="disc5")
    ap.add_argument("--size", default=None, help="NRxNPHIxNZ override")
    ap.add_argument("--fp64-steps", type=int, default=None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision-report", type=int, default=0, metavar="NSTEPS",
                    help="run both forms NSTEPS steps and report the FP32 form's error")
    ap.add_argument("--solver", default=None, help="hlld or hll")
    ap.add_argument("--monitor", type=int, default=0, metavar="NSTEPS",
                    help="long precision-form run with both solvers, diagnostics every --monitor-every steps")
    ap.add_argument("--monitor-every", type=int, default=100)
    ap.add_argument("--monitor-forms", default="fp32", help="fp32, fp64 or fp32,fp64")
    ap.add_argument("--monitor-solvers", default="hlld,hll")
    ap.add_argument("--batch-check", type=int, default=0, metavar="NSTEPS")
    ap.add_argument("--batch-check-mode", default="tuned",
                    help="batch mode of the checked run: tuned, 0 (persistent), 1 (phased), 2:B (disc graph, B branches)")
    args = ap.parse_args()
    if args.precision_report:
        return precision_report(args)
    if args.monitor:
        return monitor_run(args)
    if args.workload.startswith("batch"):
        return batch_bench(args)
    rank, world, local = rank_info()
    dims = tuple(int(v) for v in args.size.split("x")) if args.size else (512, 512, 256)
    zones = dims[0] * dims[1] * dims[2]
    cfg = {"workload": "%s: single disc %dx%dx%d (r in [0.1,1.5], phi in [0,2pi), z in [-0.5,0.5]), "
                       "beta=1, cooling on, HLLD, minmod, TVD-RK3, CFL 0.4, seeded 1%% perturbation"
                       % (args.workload, dims[0], dims[1], dims[2]),
           "zones": zones, "l2": "state (>=2.5 GB) larger than L2; no flush needed"}
    timed_path = ("value: mhd_run, one CUDA graph per RK3 step (CFL reduction and dt on the device); "
                  "kernel shares/rooflines: a separate mhd_step pass with events around each launch; "
                  "e2e: mhd_upload_state + mhd_step + mhd_download per step")

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args, dims, cfg)

    dist = dist_init(world)
    M = load_product()
    device = select_device(M, local, world)
    grid, params, U, V = make_state(M, args.workload, dims)
    hbm_peak, peak_kind = load_peaks()

    # ---- FP32 + FP64-repair form, resident ----
    p32 = with_precision(M, params, "fp32")
    d32 = M.Disc(grid, p32)
    d32.upload(U, V)
    if dist:
        dist.barrier()
    ms, wall, launches, clocks = time_run(M, d32, args.steps, args.warmup, clocks=(rank == 0))
    # per-kernel CUDA-event times (for the shares and the rooflines) from a
    # separate pass of the same steps through mhd_step, events around each launch
    nprof = max(3, min(args.steps, 5))
    d32.upload(U, V)
    _, _, _, kern, _ = time_steps(M, d32, nprof, 1, prof=True)
    ms = max_over_ranks(dist, ms)
    value = zones * args.steps * world / (ms / 1e3)

    nb32 = kernel_bytes(dims, 4)
    per_kernel = kernel_rooflines(kern, nb32, hbm_peak)
    tot = sum(v[0] for v in kern.values())
    dom = max(kern, key=lambda k: kern[k][0])
    # DRAM bytes (read + write) per zone per launch from the ncu captures at
    # 256x256x128 (profiles/), scaled here by the zones of this workload
    measured_traffic = {"update": (1.613262e9 + 0.632994e9) / 8388608,
                        "flux_r": (0.384357e9 + 0.262446e9) / 8388608,
                        "flux_phi": (0.382199e9 + 0.262957e9) / 8388608}
    traffic = measured_traffic[dom] * zones if dom in measured_traffic else None
    pk = per_kernel.get(dom, {})
    roof = {"bound": "hbm", "kernel": dom, "achieved": pk.get("gbs"), "peak": hbm_peak, "unit": "GB/s",
            "frac": pk.get("frac_hbm"), "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 256x256x128, "
                              "scaled by zones" if traffic else None,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "algorithmic_bytes_per_launch": pk.get("bytes_per_launch"), "avg_launch_ms": pk.get("launch_ms")}
    shares = {k: round(v[0] / tot, 4) for k, v in kern.items() if v[1]}
    step_ms = ms / args.steps
    split_bytes = sum(nb32.get(k, 0) * kern[k][1] for k in kern) / nprof   # bytes the split kernels move per step

    # ---- e2e through the C-ABI with host FP64 buffers ----
    e2e = None
    nb = 2 * 9 * grid.ixmax * grid.jymax * grid.kzmax * 8     # U and V, FP64
    if not args.no_e2e:
        # the host keeps the conserved state U (FP64); V is formed on the device
        sms = e2e_steps(M, d32, U, V, args.steps, args.warmup, dist, with_v=False)
        ems = max_over_ranks(dist, sum(sms))
        e2e = {"value": zones * args.steps * world / (ems / 1e3), "unit": "zone-updates/s",
               "h2d_bytes_per_step": nb // 2, "d2h_bytes_per_step": nb // 2, "ms_per_step": ems / args.steps,
               "step_ms_min": min(sms), "step_ms_max": max(sms),
               "what": "mhd_upload_state(U, NULL: V formed on the device) + mhd_step + mhd_download(U), "
                       "FP64 pinned host array"}
        # the reference host's own pair of arrays, U and V both ways
        n_uv = max(2, min(args.steps, 5))
        sms = e2e_steps(M, d32, U, V, n_uv, 1, dist, with_v=True)
        ems = max_over_ranks(dist, sum(sms))
        e2e["with_v"] = {"value": zones * n_uv * world / (ems / 1e3), "unit": "zone-updates/s",
                         "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "ms_per_step": ems / n_uv,
                         "what": "mhd_upload_state(U,V) + mhd_step + mhd_download(U,V)"}
    d32.close()

    # ---- pair-state precision form (FP32 fluxes, state as FP32 pairs), resident ----
    p2 = with_precision(M, params, "fp32x2")
    d2 = M.Disc(grid, p2)
    d2.upload(U, V)
    if dist:
        dist.barrier()
    ms2, _, _, _ = time_run(M, d2, args.steps, args.warmup, clocks=False)
    d2.upload(U, V)
    _, _, _, kern2, _ = time_steps(M, d2, nprof, 1, prof=True)
    ms2 = max_over_ranks(dist, ms2)
    pair = {"value": zones * args.steps * world / (ms2 / 1e3), "unit": "zone-updates/s",
            "ms_per_step": ms2 / args.steps,
            "kernels": kernel_rooflines(kern2, kernel_bytes(dims, 4, pair=True), hbm_peak),
            "what": "MHD_PREC_FP32X2 through mhd_run: the FP32 form's fluxes and primitives, the conserved "
                    "state as FP32 pairs (hi + lo)"}
    d2.close()

    # ---- plain FP64 form ----
    f64_steps = args.fp64_steps or max(2, min(args.steps, 5))
    p64 = with_precision(M, params, "fp64")
    d64 = M.Disc(grid, p64)
    d64.upload(U, V)
    if dist:
        dist.barrier()
    ms64, wall64, l64, kern64, _ = time_steps(M, d64, f64_steps, 1, prof=True)
    ms64 = max_over_ranks(dist, ms64)
    v64 = zones * f64_steps * world / (ms64 / 1e3)
    fp64 = {"value": v64, "unit": "zone-updates/s", "steps": f64_steps, "ms_per_step": ms64 / f64_steps,
            "speedup_fp32_over_fp64": value / v64, "speedup_pair_over_fp64": pair["value"] / v64,
            "kernels": kernel_rooflines(kern64, kernel_bytes(dims, 8), hbm_peak),
            "bound": "FP64 pipe: the flux kernels keep it 86 % active (ncu, profiles/flux_fp64_256x256x128.md); "
                     "frac_hbm is each kernel's HBM fraction only"}
    link = None
    if not args.no_e2e:
        d64.upload(U, V)
        n64e = max(2, min(args.steps, 3))
        sms = e2e_steps(M, d64, U, V, n64e, 1, dist)
        ems = max_over_ranks(dist, sum(sms))
        fp64["e2e"] = {"value": zones * n64e * world / (ems / 1e3), "unit": "zone-updates/s",
                       "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "steps": n64e,
                       "ms_per_step": ems / n64e,
                       "what": "mhd_upload_state(U,V) + mhd_step + mhd_download(U,V), plain FP64 form"}
        link = host_link(M, d64, U, V)
    d64.close()

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(args.workload, dims, steps=2, warmup=1)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "zone-updates/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded disc initial state; no public dataset exists)",
               "config": cfg, "timed_path": timed_path, "e2e": e2e, "roofline": roof, "cpu_baseline": cb,
               "clocks": clocks,
               "gpu_launches": launches,
               "kernel_share": shares,
               "kernel_roofline": per_kernel,
               "fp64": fp64,
               "pair": pair,
               "host_link": link,
               "step_traffic": {
                   "split_kernels_gbs": split_bytes / (step_ms / 1e3) / 1e9,
                   "split_kernels_bytes_per_zone": split_bytes / zones,
                   "fused_minimum_bytes_per_zone": 300,
                   "fused_minimum_gbs": 300 * zones / (step_ms / 1e3) / 1e9,
                   "fused_minimum_frac_hbm": 300 * zones / (step_ms / 1e3) / 1e9 / hbm_peak},
               "device": device}
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
