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
