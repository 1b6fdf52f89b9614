"""bench.py's reference arm runs the CPU restatement of the reference cycle
(no GPU) and prints one JSON line with the fields the benchmark contract
names; a small workload keeps it to seconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "disk",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["n_bodies"] == 1000
    # the full workload, described by the same config object the GPU arm prints
    import bench

    assert d["cpu_baseline"]["full_workload"] is True
    assert d["config"] == bench.config_of("disk", 1000, 1, 1)


def test_default_workload_is_timed_whole_on_the_cpu():
    """The headline workload is one the CPU restatement runs in full, so both
    arms measure the same 131,072-body job."""
    import bench

    assert "plummer_disk" in bench.CPU_FULL
    sims, what = bench.cpu_sample("plummer_disk", 64)
    assert len(sims) == 1 and len(sims[0]["x"]) == 128 and "full workload" in what


def test_roofline_traffic_comes_from_the_summary_of_the_kernel_that_ran():
    """The `traffic` of a bench line is read from the committed ncu summary
    of the kernel and workload: the one-sided kernel on the headline
    workload, the symmetric kernel on the uniform ball."""
    sys.path.insert(0, ROOT)
    import bench

    assert bench.traffic_from_profiles("plummer_disk") == 100160512
    assert bench.traffic_from_profiles("uniform", "k_pair_sym") == 1.64e10
    assert bench.traffic_from_profiles("uniform") is None  # no one-sided summary of that workload
