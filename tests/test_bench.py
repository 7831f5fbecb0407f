"""bench.py's command-line contract on the CPU: the reference arm (the CPU
restatement of the reference timed on the host cores, by default on the
headline 3D problem) prints one JSON line with the metric, unit, CPU-baseline
and end-to-end keys; workloads the reference does not have print an
`unavailable` line; fewer than 3 warm-up steps are refused."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout, r.stderr


def last_json(out):
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    return json.loads(lines[0])


def test_reference_arm_line():
    rc, out, err = run("--impl", "reference", "--n", "64", "--steps", "2", "--warmup", "3")
    assert rc == 0, err
    d = last_json(out)
    assert d["impl"] == "reference" and d["metric"] == "T_eff" and d["unit"] == "GB/s"
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3
    assert d["higher_is_better"] is True and d["config"]["workload"] == "3d_nonlin_512"
    assert d["config"]["shape"] == [64, 64, 64]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_unavailable_for_new_workloads():
    for w in ("batch_linstep_256", "adjoint_3d_256"):
        rc, out, err = run("--impl", "reference", "--workload", w)
        assert rc == 0, err
        d = last_json(out)
        assert d["impl"] == "reference" and "unavailable" in d


def test_reference_arm_2d_workload():
    rc, out, err = run("--impl", "reference", "--workload", "2d_nonlin_4096", "--n", "96", "--steps", "1",
                       "--warmup", "3")
    assert rc == 0, err
    d = last_json(out)
    assert d["config"] == {"workload": "2d_nonlin_4096", "shape": [96, 96],
                           "protocol": "fixed PT iterations of physical step 2"}


def test_warmup_below_three_is_refused():
    rc, out, err = run("--impl", "reference", "--warmup", "2")
    assert rc != 0 and "--warmup must be >= 3" in err
