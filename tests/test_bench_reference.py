"""The reference arm of bench.py (`--impl reference`): the CPU restatement of
the reference's step timed on the host cores, printing the same JSON line as
the GPU arm.  Run here on the small plain-fluid workload (no GPU needed)."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload", "plain32",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "MPCD particle-steps/s" and d["unit"] == "particle-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 3
    assert d["config"]["workload"].startswith("plain32: 32^3 cells x 10 fluid")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "2 MPC steps" in cb["sample"]


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--workload", "plain32",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=REPO,
                       env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_roofline_uses_the_algorithmic_bytes_and_the_measured_peak():
    """frac = particles x 112 B (float64: read + write of the reference's
    56 B state) / the fluid kernel's average launch time / MEASURED_PEAKS
    hbm_gbs; the build's own 96 B layout is reported beside it."""
    sys.path.insert(0, REPO)
    import bench

    nf = 2621440
    kernels = {"fluid": (1.34, 10), "cell": (0.5, 10), "md": (2.2, 10), "bead": (0.0, 0), "sort": (0.0, 0)}
    r = bench.roofline(nf, kernels, "fp64")
    hbm, kind = bench.peaks()
    achieved = nf * 112 / 0.134e-3 / 1e9
    assert abs(r["achieved"] - achieved) < 1e-6 * achieved and abs(r["frac"] - achieved / hbm) < 1e-9
    assert r["peak"] == hbm and r["peak_kind"] == kind and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["frac_state_bytes"] - nf * 96 / 0.134e-3 / 1e9 / hbm) < 1e-9
    assert r["traffic"] == bench.TRAFFIC_B_PER_PARTICLE["fp64"] * nf
    r32 = bench.roofline(nf, kernels, "fp32")
    assert abs(r32["achieved"] - nf * 64 / 0.134e-3 / 1e9) < 1e-6 * r32["achieved"]
