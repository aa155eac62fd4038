"""Host-side checks of bench.py (no GPU): the DRAM figures it reads from the committed ncu
summaries, and the CPU reference arm, which must print the GPU arm's workload config and load
only the oracle's library."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("name", ["k_step_1m_particles.md", "k_step_ensemble_4096_replicas.md"])
def test_profiled_traffic_reads_the_committed_summaries(name):
    t = bench.profiled_traffic(name, 1000)
    assert t is not None and 50e3 < t < 500e3  # bytes per 1,000 particles: 50-500 B per particle
    assert bench.profiled_traffic("no_such_summary.md", 1000) is None


def test_workload_config_is_a_function_of_the_workload():
    prm = bench.workload_params(1000.0)
    a = bench.workload_config(327680, prm, "0123456789abcdef")
    b = bench.workload_config(327680, dict(prm), "0123456789abcdef")
    assert a == b and a["particles"] == bench.N_1M and a["mesh_sha16"] == "0123456789abcdef"
    assert "l2" not in a and "state" not in a  # how an arm runs it stays outside the config


def test_mesh_hash_changes_with_the_mesh():
    a = dict(v3=np.zeros((3, 3)), f3=np.array([[0, 1, 2]]), uv=np.zeros((3, 2)), fuv=np.array([[0, 1, 2]]))
    b = dict(a, v3=np.ones((3, 3)))
    assert bench.mesh_sha16(a) == bench.mesh_sha16(dict(a)) != bench.mesh_sha16(b)


def test_reference_arm_runs_on_the_oracle_alone():
    """One warm-up and one timed FP64 oracle step of the 1M-particle workload on the host cores."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "maps = open('/proc/self/maps').read();"
            "print('GPU_LIB_MAPPED', 'lib2dtissue_gb300' in maps)")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    d = json.loads(lines[-1])
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    arrays, area = bench.load_workload_mesh()
    assert d["config"] == bench.workload_config(len(arrays["f3"]), bench.workload_params(area),
                                                bench.mesh_sha16(arrays))
    assert "GPU_LIB_MAPPED False" in r.stdout
