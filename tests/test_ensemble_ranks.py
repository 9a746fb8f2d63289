"""An ensemble split over ranks (pic_gb300.partition_members / run_ensemble_ranks).

Each rank runs its share of the members as one batched ensemble on its own GPU;
the one exchange is a final gather of the energy histories to rank 0. These
tests run the host logic without a GPU: the partition is exact, complete and
balanced, and two gloo ranks (127.0.0.1) merge to the histories one process
gives, through a stand-in batch that keeps the library's reordering of members
by grid size. The GPU test checks the property the split rests on: a member's
history does not depend on the other members of its batch.
"""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pic-deposition_gb300")
sys.path.insert(0, ROOT)
sys.path.insert(0, PKG)

import pic_gb300 as pg  # noqa: E402  (host module; the library loads only on first use)

FAKE = """
import numpy as np
import pic_gb300 as pg


class StandInBatch(pg.Ensemble):
    '''Members advanced by a closed formula of (N, ppc, seed, dt, step), in the
    library's order (a stable sort by grid size), without a GPU.'''

    def __init__(self, runs, dt=0.1, **cfg):
        self.h = None
        self.runs = list(runs)
        self.nruns = len(runs)
        self.order = sorted(range(len(runs)), key=lambda i: int(runs[i][0]))
        self.dt = dt

    def close(self):
        pass

    def run(self, steps):
        s = np.arange(steps)[:, None]
        mem = [self.runs[i] for i in self.order]
        n = np.array([m[0] for m in mem], float)[None, :]
        p = np.array([m[1] for m in mem], float)[None, :]
        seed = np.array([m[2] for m in mem], float)[None, :]
        fe = np.cos(0.37 * seed + self.dt * s) * n + p
        ke = np.sin(0.11 * seed * p + s) + n * p
        return fe, ke
"""


def members(count=37, seed=5):
    rng = np.random.default_rng(seed)
    return [(int(n), int(p), int(100 + i)) for i, (n, p) in
            enumerate(zip(rng.choice([128, 256, 512, 1024], count), rng.choice([4, 16, 64, 256], count)))]


@pytest.mark.parametrize("world_size", [1, 2, 3, 4, 8])
def test_partition_exact_complete_balanced(world_size):
    runs = members()
    parts = pg.partition_members(runs, world_size)
    assert len(parts) == world_size
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(runs)))
    sizes = [n * n * p for n, p, _ in runs]
    loads = [sum(sizes[i] for i in p) for p in parts]
    # largest-first greedy: no rank exceeds the mean by more than the largest member
    assert max(loads) <= sum(sizes) / world_size + max(sizes)
    assert all(p == sorted(p) for p in parts)
    assert parts == pg.partition_members(runs, world_size)  # deterministic


def test_partition_more_ranks_than_members():
    parts = pg.partition_members([(128, 4, 1), (256, 4, 2)], 4)
    assert sorted(i for p in parts for i in p) == [0, 1] and sum(1 for p in parts if not p) == 2


def test_member_order_mapping_single_process():
    ns = {}
    exec(FAKE, ns)
    runs = members(11)
    fe, ke = pg.run_ensemble_ranks(runs, 7, ensemble=ns["StandInBatch"], dt=0.05)
    for i, (n, p, s) in enumerate(runs):
        want = np.cos(0.37 * s + 0.05 * np.arange(7)) * n + p
        assert np.array_equal(fe[:, i], want)


RANK_SCRIPT = """
import os, sys
sys.path.insert(0, {root!r}); sys.path.insert(0, {pkg!r})
import numpy as np
import torch.distributed as dist
{fake}
sys.path.insert(0, {tests!r})
from test_ensemble_ranks import members
dist.init_process_group("gloo")
rank, ws = dist.get_rank(), dist.get_world_size()
out = pg.run_ensemble_ranks(members(), 9, rank, ws, ensemble=StandInBatch, dt=0.05)
if rank == 0:
    np.savez({out!r}, fe=out[0], ke=out[1])
else:
    assert out is None
dist.destroy_process_group()
print("DONE", rank, flush=True)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_merge_to_single_process_histories(tmp_path):
    out = str(tmp_path / "merged.npz")
    script = RANK_SCRIPT.format(root=ROOT, pkg=PKG, tests=os.path.join(ROOT, "tests"), fake=FAKE, out=out)
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", script], env=env, cwd=ROOT, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    try:
        for p in procs:
            so, se = p.communicate(timeout=180)
            assert p.returncode == 0, se[-2000:]
            assert "DONE" in so
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    got = np.load(out)
    ns = {}
    exec(FAKE, ns)
    fe, ke = pg.run_ensemble_ranks(members(), 9, ensemble=ns["StandInBatch"], dt=0.05)
    assert np.array_equal(got["fe"], fe) and np.array_equal(got["ke"], ke)


@pytest.mark.gpu
def test_split_batches_equal_one_batch(pg):
    """The two halves of a partition, run as separate batches one after the
    other, give every member's field-energy history bit for bit as one batch of
    all members does, and the kinetic energy (FP32 partial sums) to 1e-6."""
    runs = [(256, 4, 11), (128, 16, 12), (128, 4, 13), (256, 16, 14), (128, 8, 15)]
    cfg = dict(dt=0.1, sort_interval=3, use_graph=True)
    fe1, ke1 = pg.run_ensemble_ranks(runs, 8, **cfg)
    parts = pg.partition_members(runs, 2)
    fe2 = np.full_like(fe1, np.nan)
    ke2 = np.full_like(ke1, np.nan)
    for mine in parts:
        with pg.Ensemble([runs[i] for i in mine], **cfg) as e:
            f, k = e.run_member_order(8)
        fe2[:, mine], ke2[:, mine] = f, k
    assert np.array_equal(fe1, fe2)
    assert np.allclose(ke1, ke2, rtol=1e-6)
