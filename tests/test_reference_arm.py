"""The bench's reference arm and CPU baseline: the oracle's spec-mode step
(the reference's si_nlist/si_force restated, on the host cores) on the
bench's cascade, timed with the bench's warm-up and step counts, set up from
the oracle alone. Small slabs, so that it runs in seconds here."""
from __future__ import annotations

import json
import math
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def test_reference_run_honours_warmup_and_steps(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    calls = []
    real = bench._oracle_sample

    def counted(o, sample_steps, nthreads):
        calls.append((o.spec_scalars()["time"], sample_steps))
        return real(o, sample_steps, nthreads)

    monkeypatch.setattr(bench, "_oracle_sample", counted)
    value, cb = bench.cpu_reference_run((4, 4, 4), 0.6, 2, 3, 2, nthreads=2)
    # two untimed and three timed samples of two steps each, the cascade
    # going on from sample to sample
    assert [c[1] for c in calls] == [2] * 5
    assert calls[0][0] == 0.0 and all(b[0] > a[0] for a, b in zip(calls, calls[1:]))
    assert math.isfinite(value) and value > 0
    assert cb["value"] == value and cb["cores"] == 2 and cb["kind"] == "port"
    assert "median of 3" in cb["sample"] and "2 untimed" in cb["sample"]


def test_cpu_baseline_after_an_untimed_sample(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    calls = []
    real = bench._oracle_sample

    def counted(o, sample_steps, nthreads):
        calls.append(sample_steps)
        return real(o, sample_steps, nthreads)

    monkeypatch.setattr(bench, "_oracle_sample", counted)
    cb = bench.cpu_baseline((4, 4, 4), 0.6, 3, nthreads=2)
    assert calls == [1, 3]
    assert cb["value"] > 0 and cb["unit"] == "atom-steps/s"


def test_oracle_workload_equals_gpu_workload():
    """The reference arm's slab (oracle restatements) is the GPU arm's slab."""
    sys.path.insert(0, str(ROOT))
    import bench

    a = bench.make_workload((5, 5, 4), list_skin_A=0.6)
    b = bench.oracle_workload((5, 5, 4), list_skin_A=0.6)
    for k in ("X", "V", "Xi", "mass", "atype", "xsides", "tags"):
        assert np.array_equal(a[k], b[k]), k
    assert a["params"].remove_z == b["params"].remove_z
    assert a["params"].list_skin == b["params"].list_skin


def test_reference_arm_loads_no_gpu_package(tmp_path):
    """`bench.py --impl reference` on a small slab prints the arm's JSON line
    with the GPU arm's config object, and its process never imports the GPU
    package nor maps libfibmd_gpu.so."""
    code = (
        "import runpy, sys, json\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', '--steps', '2', '--warmup', '1',"
        f" '--cells', '3,3,3', '--cpu-sample-steps', '8']\n"
        "try:\n"
        f"    runpy.run_path({str(ROOT / 'bench.py')!r}, run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'pkg': 'fib_md_gb300' in sys.modules,"
        " 'so': 'libfibmd_gpu' in maps}))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    line, probe = json.loads(lines[0]), json.loads(lines[-1])
    assert probe == {"pkg": False, "so": False}
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["atoms"] == 8 * 27 + 1 and line["config"]["mode"] == "spec"
    assert line["cpu_baseline"]["kind"] == "port"
