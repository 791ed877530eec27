"""Host logic of bench.py that needs no GPU: the child processes that measure
the other workloads after the headline line (their command lines, and how a
failed, silent or timed-out child is recorded), and the bit-identity count of
the reference-arithmetic leg."""
import json
import os
import subprocess
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_children_run_each_other_workload_without_recursing(monkeypatch):
    calls = []

    def fake_run(cmd, capture_output, text, timeout):
        calls.append(cmd)
        c = int(cmd[cmd.index("--config") + 1])
        if c == 3:
            return types.SimpleNamespace(returncode=1, stdout="", stderr="boom")
        if c == 4:
            raise subprocess.TimeoutExpired(cmd, timeout)
        if c == 5:
            return types.SimpleNamespace(returncode=0, stdout="no json here\n", stderr="")
        line = {"metric": "m", "unit": "u", "value": float(c), "ms_per_step": 1.0, "data": "synthetic",
                "autotune": {"block": 128, "table": [[1, 2, 3, 4.0]]}}
        return types.SimpleNamespace(returncode=0, stdout="log line\n" + json.dumps(line) + "\n", stderr="")

    monkeypatch.setattr(bench.subprocess, "run", fake_run)
    args = types.SimpleNamespace(workloads="auto", steps=20, warmup=5)
    out = bench.run_workloads(args)
    assert sorted(out) == ["1", "3", "4", "5", "6"]
    for cmd in calls:
        # children never spawn children, measure briefly, and keep the warm-up rule
        assert cmd[cmd.index("--workloads") + 1] == "none" and "--brief" in cmd
        assert cmd[cmd.index("--warmup") + 1] == "3" and cmd[cmd.index("--steps") + 1] == "3"
    assert out["1"]["value"] == 1.0 and "metric" not in out["1"] and "table" not in out["1"]["autotune"]
    assert out["1"]["autotune"]["block"] == 128
    assert out["3"]["error"].startswith("exit 1") and "boom" in out["3"]["error"]
    assert "timed out" in out["4"]["error"]
    assert out["5"]["error"].startswith("exit 0")
    assert all(v["wall_s"] >= 0 for v in out.values())


def test_workload_list_is_parsed(monkeypatch):
    seen = []
    monkeypatch.setattr(bench.subprocess, "run", lambda cmd, **k: seen.append(cmd[cmd.index("--config") + 1])
                        or types.SimpleNamespace(returncode=0, stdout='{"value": 1}', stderr=""))
    out = bench.run_workloads(types.SimpleNamespace(workloads="5, 3", steps=2, warmup=3))
    assert seen == ["5", "3"] and sorted(out) == ["3", "5"]


def test_bitexact_vs_oracle_counts_identical_trajectories():
    """bench.bitexact_vs_oracle on the oracle's own REF results with correctly
    rounded powers is 1.0, and a one-ulp change in one trajectory's saveat
    value, or one extra rejected step, takes exactly that trajectory out."""
    import bench
    import __graft_entry__ as g
    cfg = dict(bench.CONFIGS[2], n=64)
    u0, p = cfg["inputs"](64, 3)
    sv = np.linspace(cfg["tspan"][0], cfg["tspan"][1], cfg["nsave"])
    ref = g.oracle().solve(cfg["alg"], cfg["rhs"], u0, p, cfg["tspan"], cfg["dt"], rounding="ref", controller="ref",
                           abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv, nthreads=4)
    res = {k: ref[k].copy() for k in ("u_final", "naccept", "nreject", "us")}
    assert bench.bitexact_vs_oracle(cfg, u0, p, sv, res)["frac_bit_identical"] == 1.0
    res["us"][50, 1, 7] = np.nextafter(res["us"][50, 1, 7], np.inf)
    res["nreject"][9] += 1
    assert bench.bitexact_vs_oracle(cfg, u0, p, sv, res)["frac_bit_identical"] == 62 / 64
