"""bench.py's reference arm runs on the CPU: its JSON line carries the keys
the benchmark contract asks for, and its oracle results match the per-job
oracle on a sample of the batched workload."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                         timeout=600, check=True).stdout.strip().splitlines()
    line = json.loads(out[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e", "impl"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in line["config"]


def test_batched_oracle_matches_per_job_oracle():
    sys.path.insert(0, ROOT)
    from gpu_workgroup_managment_gb300.batch import batch_workload
    from oracle import oracle
    gs, jobs, _ = batch_workload(n_graphs=24, seed=11, mu=9.0, sigma=1.5, lo=8, hi=12)
    a = oracle.BatchArena(gs, jobs)
    d = a.run()
    for k, (gi, algo, src) in enumerate(jobs):
        want = oracle.lonestar_bfs(gs[gi], src) if algo == "bfs" else \
            oracle.lonestar_sssp(gs[gi], src)
        assert np.array_equal(d[a.dist_off[k]:a.dist_off[k] + a.V[k]], want), k


def test_oracle_workload_equals_product_workload():
    """The reference arm's inputs (oracle/workload.py) are the GPU arm's,
    array for array."""
    sys.path.insert(0, ROOT)
    from gpu_workgroup_managment_gb300 import graphs as G
    from gpu_workgroup_managment_gb300.batch import batch_workload
    from oracle import workload as W
    for scale, ef, seed in ((8, 5, 3), (13, 11, 2024007)):
        a, b = W.rmat(scale, ef, seed=seed), G.rmat(scale, ef, seed=seed)
        assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)
        assert np.array_equal(a.weights, b.weights)
    a, b = W.grid(17, 29), G.grid(17, 29)
    assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)
    kw = dict(n_graphs=40, seed=5, mu=10.0, sigma=2.0, lo=8, hi=13)
    ga, ja, ma = W.batch_workload(**kw)
    gb, jb, mb = batch_workload(**kw)
    assert ja == jb and ma == mb
    for x, y in zip(ga, gb):
        assert np.array_equal(x.row_ptr, y.row_ptr) and np.array_equal(x.col, y.col)
        assert (x.weights is None) == (y.weights is None)
        if x.weights is not None:
            assert np.array_equal(x.weights, y.weights)


def test_reference_arm_loads_no_product_library():
    """--impl reference maps only oracle/ libraries: it never imports the
    package and never loads libwgm.so."""
    code = (
        "import runpy, sys\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']\n"
        "try:\n"
        f"    runpy.run_path({os.path.join(ROOT, 'bench.py')!r}, run_name='__main__')\n"
        "except SystemExit as e:\n"
        "    assert not e.code, e.code\n"
        "assert not any(m.startswith('gpu_workgroup_managment_gb300') for m in sys.modules)\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libwgm.so' not in maps\n"
        "print('CLEAN')\n")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    assert lines[-1] == "CLEAN"
    ref = json.loads(lines[-2])
    assert ref["warmup"] == 3 and ref["steps"] == 1
