"""Host-side pieces of bench.py that need no GPU: the clock record's
summary (from NVML samples or nvidia-smi lines) and the committed
per-launch DRAM traffic it reports beside the roofline."""
import bench


def test_nvml_samples_summary():
    c = bench.ClockSampler(0)
    c.max_mhz = 2070.0
    # idle (0x1) and application-clock (0x2) bits are not throttling; power
    # cap (0x4) in one sample; hardware slowdown with its thermal cause in another
    c.samples = [(2070.0, 0x0), (2055.0, 0x1 | 0x2), (1980.0, 0x4), (2070.0, 0x8 | 0x40)]
    s = c.summary()
    assert s["sm_mhz"] == 2062.5
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap"]
    assert s["samples"] == 4 and s["source"].startswith("nvml")


def test_nvidia_smi_lines_summary():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 812.3, 0x0000000000000000, Not Active, Not Active, Not Active, "
               "Not Active",
               "0, 1965, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, "
               "Active",
               "garbled"]
    s = c.summary()
    assert s["sm_mhz"] == (2070 + 1965) / 2
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 2 and s["source"].startswith("nvidia-smi")


def test_no_samples_gives_no_record():
    assert bench.ClockSampler(0).summary() is None


def test_committed_traffic_of_the_fused_kernels():
    # the T=200 capture scaled to T=3500, as profiles/traffic.txt states
    assert bench.committed_traffic("seq_bwd_tape_kernel") == 6941428480
    assert bench.committed_traffic("seq_bwd_fused_kernel") == 1040063360
    assert bench.committed_traffic("no_such_kernel") is None


def test_committed_instruction_counts():
    """Warp instructions per time step of the fused kernels' launches, read
    from the committed ncu summary for the issue roofline."""
    n = bench.committed_count("seq_bwd_tape_kernel")
    assert n is None or n > 0
    assert bench.committed_count("no_such_kernel") is None


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the reference's CPU path restated, on the
    host cores) prints one JSON line with the keys the benchmark contract
    asks of that arm; a batch of 2 keeps the run to a few seconds."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--batch", "2"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "cell-steps/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    # the unmodified reference's own CPU path beside the port, where its
    # install (baseline/_ref) is present
    ref = d["cpu_baseline_reference"]
    if os.path.isdir(os.path.join(root, "baseline", "_ref", "wavetorch")):
        assert ref["kind"] == "reference" and ref["value"] > 0 and ref["cores"] >= 1
    else:
        assert ref is None


def test_other_workloads_keep_going_after_a_failure(monkeypatch):
    """The compact pass over the other workloads records each one's result
    line under its name, and a workload that raises records its error while
    the rest still run (and print nothing of their own)."""
    import argparse
    import json

    def ok(name):
        def run(a):
            print("some log line")
            print(json.dumps({"metric": name, "value": 1.0, "steps": a.steps, "warmup": a.warmup}))
        return run

    def boom(a):
        raise RuntimeError("out of memory")

    monkeypatch.setattr(bench, "run_lens", ok("lens"))
    monkeypatch.setattr(bench, "run_nonlinear", boom)
    monkeypatch.setattr(bench, "run_ragged", ok("ragged"))
    monkeypatch.setattr(bench, "run_fields", ok("fields"))
    monkeypatch.setattr(bench, "run_holey", ok("holey"))
    out = bench.other_workloads(argparse.Namespace(steps=5, warmup=3, workload="batched"))
    assert list(out) == ["lens", "nonlinear", "ragged", "fields", "holey"]
    assert out["lens"]["metric"] == "lens" and out["lens"]["steps"] == 2
    assert out["lens"]["warmup"] == 3 and out["lens"]["wall_s"] >= 0
    assert out["nonlinear"]["error"].startswith("RuntimeError: out of memory")
    assert out["holey"]["value"] == 1.0
