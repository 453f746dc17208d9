"""bench.py's reference arm on the CPU: one JSON line with the contract's keys, the oracle port timed
on the host cores, and nothing copied to or from a device."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-steps", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["config"]["workload"] and d["config"]["lattice"] == [128, 128, 128]


def test_fp64_rooflines_arithmetic():
    """FP64 form at 128^3 with friction: 240 B/pt and 6 * 5 N log2 N + 60 N flops per step (the 18 axis
    transforms of a friction step are 6 3D-transform equivalents); without friction 176 B/pt and 4."""
    sys.path.insert(0, ROOT)
    import bench
    n = 128 ** 3
    peak = (1.5, "measured")
    r = bench.fp64_rooflines(100.0, n, peak, qf=True)
    assert r["hbm"]["achieved"] == 240 * n * 100.0 / 1e9
    assert r["fp64_alu"]["flops_per_step"] == 6 * 5.0 * n * 21 + 60.0 * n
    assert abs(r["fp64_alu"]["achieved"] - r["fp64_alu"]["flops_per_step"] * 100.0 / 1e12) < 1e-12
    assert r["fp64_alu"]["frac"] == r["fp64_alu"]["achieved"] / 1.5
    assert r["fp64_alu"]["peak_kind"] == "measured"
    plain = bench.fp64_rooflines(100.0, n, peak, qf=False)
    assert plain["hbm"]["achieved"] == 176 * n * 100.0 / 1e9
    assert plain["fp64_alu"]["flops_per_step"] == 4 * 5.0 * n * 21 + 60.0 * n
    json.dumps(r)


def test_traffic_summary_is_read_with_its_label(tmp_path, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "pass_kernel_traffic.txt").write_text("# comment\nfp32_ufg_qf_rte_128 1.5e8 steady state, cache-control none\n")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.traffic_from_profiles(128) == (1.5e8, "steady state, cache-control none")
    assert bench.traffic_from_profiles(256) == (None, None)
