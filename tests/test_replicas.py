"""The multi-rank path of bench.py, on CPU with gloo (world size 2, 127.0.0.1).

The deposition path does not shard: N ranks run N independent replicas, each on
its own GPU, joined only by a barrier around the timed region and a max over
ranks of the step time (no data-path collective). These tests run that host
logic without a GPU: the barrier and the max across two gloo ranks, and the
reference arm under torchrun, where rank 0 alone does the work and prints the
one JSON line and the other rank exits 0 without output; and the reference
arm's line in one process (the keys of the benchmark line, and the GB300 arm's
metric and workload).
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = """
import sys
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
d.barrier()
m = d.max(0.5 + d.rank)
d.barrier()
d.close()
print("RESULT", d.rank, d.ws, m, flush=True)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_barrier_and_max_over_two_gloo_ranks():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT)], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    results = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=180)
            assert p.returncode == 0, err[-2000:]
            line = [l for l in out.splitlines() if l.startswith("RESULT")][0].split()
            results.append((int(line[1]), int(line[2]), float(line[3])))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    assert sorted(results) == [(0, 2, 1.5), (1, 2, 1.5)]


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "3", "--warmup", "3", "--ppc", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 3 and d["warmup"] == 3
    assert d["unit"] == "particles/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] and d["config"]["particles"] == 1024 * 1024
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_single_process_line_keeps_the_contract():
    sys.path.insert(0, ROOT)
    import bench

    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3", "--ppc",
                        "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert k in d, k
    # the same metric, unit and direction as the GB300 arm, so that the two lines compare
    assert d["metric"] == bench.METRIC and d["unit"] == "particles/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["config"]["workload"] == bench.WORKLOAD
    assert d["ms_per_step"] > 0 and d["value"] > 0
