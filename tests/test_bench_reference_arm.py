"""bench.py --impl reference on the CPU: one JSON line with the benchmark's keys, the CPU port of the
reference's algorithm timed on the workload's whole raster, and no host-device bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "accu_1k", "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["unit"] == "Mcells/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "accu_1k"


def test_committed_profiles_carry_the_lines_the_bench_reads():
    """bench.py takes the accu call's DRAM traffic and the multi-step kinematic wave's instructions per
    cell step from the committed ncu summaries under profiles/: both lines exist and are plausible."""
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.remove(ROOT)
    traffic = bench.profile_traffic("accu_f32_tiles")
    assert traffic is not None
    nbytes, cells = traffic
    assert 9.0 <= nbytes / cells <= 40.0  # at least the algorithmic 9 B/cell
    ipcs = bench.profile_value("warp_instructions_per_cell_step", "k_stage_flow_kw")
    assert ipcs is not None and 1.0 < ipcs[0][0] < 100.0
    fma = bench.profile_value("fma_pipe_pct", "k_stage_flow_kw")
    assert fma is not None and 0.0 < fma[0][0] <= 100.0
