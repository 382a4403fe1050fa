"""bench.py's reference arm (the compiled C restatement on the host cores)
prints one JSON line with the contract's keys; it needs no GPU."""

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def run_reference(*args):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1", *args],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


@pytest.mark.parametrize("args", [(), ("--workload", "grids", "--instances", "40")],
                         ids=["adder_mc", "grids"])
def test_reference_arm_prints_the_contract_line(args):
    line = run_reference(*args)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    base = line["cpu_baseline"]
    assert base["value"] == line["value"] and base["kind"] == "port" and base["cores"] >= 1
    if args:
        assert "first 32 of the 40 grids" in base["sample"]
    else:
        assert "grids" not in base["sample"]


@pytest.mark.parametrize("name,instances", [("adder_mc", 8), ("grid100", 1), ("grids", 40)])
def test_cpu_legs_report_a_bounded_sample(name, instances):
    sys.path.insert(0, str(ROOT))
    import bench
    w = bench.WORKLOADS[name]
    n_t = 5 if w.analysis == "transient" else 1
    base = bench.cpu_baseline(w, n_t, instances, min_seconds=0.2)
    assert base["kind"] == "port" and base["cores"] == 1 and base["value"] > 0
    assert ("first 32 of the 40 grids" in base["sample"]) == (name == "grids")
    lu = bench.cpu_superlu(w, instances, min_seconds=0.2)
    if w.analysis == "dc":
        assert lu["kind"] == "superlu" and lu["value"] > 0
        grids = min(instances, bench.CPU_GRIDS) if name == "grids" else 1
        unknowns = int(lu["sample"].split("of the ")[1].split("-unknown")[0])
        assert (unknowns > 200_000) == (grids > 1)
    else:
        assert lu is None


def test_clock_summary_reads_throttle_reasons():
    sys.path.insert(0, str(ROOT))
    import bench
    clk = bench.Clocks()
    assert clk.summary()["reasons"] == ["unsampled"]
    row = "0, {sm}, 2070, 900.0, 0x0, Not Active, {hw}, Not Active, {pc}"
    for sm, hw, pc in [(1965, "Not Active", "Active"), (2070, "Not Active", "Not Active"),
                       (1980, "Active", "Not Active")]:
        clk.rows.append([x.strip() for x in row.format(sm=sm, hw=hw, pc=pc).split(",")])
    s = clk.summary()
    assert s["sm_mhz"] == 1980 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


@pytest.mark.parametrize("name", ["adder_mc", "ring101", "grid100"])
def test_oracle_check_accepts_oracle_results_and_rejects_a_planted_error(name):
    """bench.py's oracle_check on CPU: trajectories the oracle produced
    itself pass; the same trajectories with one node voltage moved by 10 uV
    at one time point fail both the 1e-9 match and the Newton-step test."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    from oracle import cbase
    from voltax_gb300 import symbolic
    w = bench.WORKLOADS[name]
    c = w.circuit(3 if name == "adder_mc" else 1)
    ts = w.times()[:51]  # the workload's own time step, first 50 steps
    ic = w.ic(c)
    z0 = None if isinstance(ic, str) else ic.numpy()
    st = symbolic.structure(c)
    z = np.stack([cbase.CSystem(c, st, st.plan, b).run(
        ts if w.analysis == "transient" else ts[:1], z0=z0, method=w.method or "be",
        dc_first=z0 is None)[0] for b in range(c.batch)])
    good = bench.oracle_check(w, c, z, ts, ic, count=3)
    assert good["pass"] and good["max_rel_node_v"] == 0.0
    assert good["max_newton_step_ratio"] <= 1.0 and good["instances"] == c.batch
    bad = z.copy()
    bad[0, -1, 1] += 1e-5
    worse = bench.oracle_check(w, c, bad, ts, ic, count=3)
    assert not worse["pass"] and worse["max_newton_step_ratio"] > 1.0
