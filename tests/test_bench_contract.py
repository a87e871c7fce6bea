"""bench.py's default flow and its JSON line, on the CPU.

The disc context needs a GB300, so here a stand-in replaces mhdgpu.Disc (and
the host-memory pinning) with fixed timings; everything else -- the workload
set-up through the library's host functions, the timing bookkeeping, the
roofline, e2e and CPU-baseline blocks, the printed line -- is bench.py's own
code.  This guards the keys and arithmetic of the line the benchmark contract
asks for, not any measured value.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class StandInDisc:
    """Fixed 2 ms per step, 1 ms per state upload or download, 5 kernels per
    stage, 1 ms per kernel launch."""
    PROF_KINDS = ["flux_r", "flux_phi", "flux_z", "update", "ghost", "setdt", "trig", "convert", "stage",
                  "zupdate"]

    def __init__(self, grid, params):
        self.n = 0
        self.ms = 0.0
        self.profiling = False
        self.prof_steps = 0

    def upload(self, U, V):
        pass

    def upload_state(self, U, V):
        self.ms += 1.0

    def download_into(self, U, V):
        self.ms += 1.0

    def run(self, nsteps, t):
        self.n += 21 * nsteps
        self.ms += 2.0 * nsteps
        return t + 1e-3 * nsteps

    def step(self, t):
        self.n += 21
        self.ms += 2.0
        if self.profiling:
            self.prof_steps += 1
        return 0, t + 1e-3, 1e-3, 1.0, np.zeros(3, dtype=np.int32)

    def timer_start(self):
        self.t0 = self.ms

    def timer_stop(self):
        return self.ms - self.t0

    def launches(self):
        return self.n

    def prof(self, on=True):
        self.profiling = on
        if on:
            self.prof_steps = 0

    def prof_read(self):
        s = self.prof_steps
        out = {k: (0.0, 0) for k in self.PROF_KINDS}
        for k, w in (("flux_r", 1.0), ("flux_phi", 1.0), ("flux_z", 1.0), ("update", 3.0), ("ghost", 0.1)):
            out[k] = (3 * s * w, 3 * s)
        out["setdt"] = (0.5 * s, s)
        return out

    def close(self):
        pass


@pytest.fixture
def bench_with_stand_in(monkeypatch):
    import bench
    real = bench.load_product

    def fake_load():
        M = real()
        monkeypatch.setattr(M, "Disc", StandInDisc)
        monkeypatch.setattr(M, "pin", lambda a, on=True: None)
        return M

    monkeypatch.setattr(bench, "load_product", fake_load)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    return bench


def test_default_line_has_the_contract_keys(bench_with_stand_in, monkeypatch, capsys):
    bench = bench_with_stand_in
    monkeypatch.setattr(sys, "argv", ["bench.py", "--size", "24x16x20", "--steps", "4", "--warmup", "3"])
    assert bench.main() == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks",
              "gpu_launches"):
        assert k in d, k
    zones = 24 * 16 * 20
    assert d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3
    assert d["ms_per_step"] == pytest.approx(2.0)
    assert d["value"] == pytest.approx(zones / 2e-3)
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["config"]["workload"].startswith("disc5") and d["config"]["zones"] == zones
    assert d["gpu_launches"] == 4 * 21
    e = d["e2e"]
    assert e["unit"] == d["unit"] and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 9 * 26 * 18 * 22 * 8
    assert e["with_v"]["h2d_bytes_per_step"] == 2 * 9 * 26 * 18 * 22 * 8
    assert e["ms_per_step"] == pytest.approx(4.0) and e["value"] == pytest.approx(zones / 4e-3)
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["kernel"] == "update"
    assert r["avg_launch_ms"] == pytest.approx(3.0)
    assert r["achieved"] == pytest.approx(zones * 70 * 4 / 3e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["traffic"] == pytest.approx((1.613262e9 + 0.632994e9) / 8388608 * zones)
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] > 0 and cb["unit"] == "zone-updates/s"
    assert "24x16x20" in cb["sample"]
    assert abs(sum(d["kernel_share"].values()) - 1.0) < 1e-3
    kr = d["kernel_roofline"]
    for k in ("flux_r", "flux_phi", "flux_z", "update", "setdt"):
        assert kr[k]["frac_hbm"] == pytest.approx(kr[k]["gbs"] / r["peak"])
    assert kr["flux_r"]["bytes_per_launch"] == 25 * 16 * 20 * 18 * 4
    assert kr["flux_z"]["bytes_per_launch"] == 24 * 16 * 21 * 18 * 4   # every z face, the boundary ones too
    assert kr["setdt"]["bytes_per_launch"] == 14 * 16 * 20 * 8 * 4
    p2 = d["pair"]
    assert p2["unit"] == d["unit"] and p2["ms_per_step"] == pytest.approx(2.0)
    assert p2["value"] == pytest.approx(zones / 2e-3)
    assert p2["kernels"]["update"]["bytes_per_launch"] == zones * 94 * 4
    assert f_speedups_ok(d)
    f = d["fp64"]
    assert f["e2e"]["unit"] == d["unit"] and f["e2e"]["h2d_bytes_per_step"] == e["with_v"]["h2d_bytes_per_step"]
    assert f["kernels"]["update"]["bytes_per_launch"] == zones * 70 * 8
    hl = d["host_link"]
    assert hl["bytes"] == e["with_v"]["h2d_bytes_per_step"] and hl["h2d_gbs"] == pytest.approx(hl["bytes"] / 1e-3 / 1e9)
    st = d["step_traffic"]
    assert st["fused_minimum_gbs"] == pytest.approx(300 * zones / 2e-3 / 1e9)


def f_speedups_ok(d):
    f = d["fp64"]
    return (f["speedup_fp32_over_fp64"] == pytest.approx(d["value"] / f["value"])
            and f["speedup_pair_over_fp64"] == pytest.approx(d["pair"]["value"] / f["value"]))


def test_reference_arm_line(monkeypatch, capsys):
    import bench

    def no_product():
        raise AssertionError("the reference arm must not load the product library")

    monkeypatch.setattr(bench, "load_product", no_product)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--size", "24x16x20", "--steps", "5",
                                      "--warmup", "2"])
    assert bench.main() == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    d = json.loads(lines[-1])
    assert d["impl"] == "reference" and d["value"] == d["cpu_baseline"]["value"] == d["e2e"]["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # full grid of the stated workload, a bounded number of steps
    assert d["config"]["zones"] == 24 * 16 * 20 and "24x16x20" in d["cpu_baseline"]["sample"]
    assert d["steps"] == 3 and d["warmup"] == 1
