"""The multi-GPU path is replicas only (species and members are independent;
no exchange step): under torchrun every rank runs its own replica, times
are combined by a max over ranks, and rank 0 alone prints the JSON line.
These run on the CPU with the gloo backend and world size 2."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, values, out):
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, str(ROOT))
        import bench
        out.put((rank, bench.max_over_ranks(values[rank])))
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    vals = [3.5, 7.25]
    ps = [mp.Process(target=_worker, args=(r, 2, port, vals, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 7.25, 1: 7.25}


def test_reference_arm_under_torchrun():
    """bench.py --impl reference as the driver launches it for N = 2: rank 0
    times the reference's CPU path and prints one line, rank 1 exits
    cleanly."""
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--workload", "single_h"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    # the reference's own routines (translated) where they are available here
    import refrun
    kind = "reference" if refrun.build() is not None else "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == kind


def test_member_partition_covers_and_balances():
    """Ensemble members over ranks by work (species x length): every member
    exactly once, and the heaviest rank within Graham's 4/3 bound of the
    ideal share."""
    from ramgpu import shard, workload as W

    ens = W.make_ensemble(256)
    work = shard.member_work(ens.species, ens.length)
    for world in (1, 2, 3, 8):
        parts = shard.partition_members(work, world)
        flat = sorted(m for p in parts for m in p)
        assert flat == list(range(256))
        loads = [sum(work[m] for m in p) for p in parts]
        assert max(loads) <= 4.0 / 3.0 * max(sum(work) / world, max(work)) + 1e-9
    with pytest.raises(ValueError):
        shard.partition_members(work, 0)


def _shard_worker(rank, world, port, out):
    import numpy as np
    import torch
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, str(ROOT / "ram-scb_gb300"))
        from ramgpu import shard, workload as W

        ens = W.make_ensemble(48, seed=77)
        sums = [float(np.sum(a)) for a in ens.base.f2]
        parts = shard.partition_members(shard.member_work(ens.species, ens.length), world)
        # each rank's diagnostic rows for its own members only
        rows = {m: [sums[s] * float(ens.scale[m]) for s in ens.species[m]] for m in parts[rank]}
        allrows = shard.gather_member_rows(rows, world, rank, ens.members, torch.distributed)
        out.put((rank, parts, allrows))
    finally:
        torch.distributed.destroy_process_group()


def test_member_shards_gather_gloo():
    """Two ranks each advance their own members (here: the members' initial
    diagnostics) and every rank gathers all rows, in member order, each
    exactly once -- the host side of the ensemble split over GPUs."""
    torch = pytest.importorskip("torch")
    import numpy as np
    sys.path.insert(0, str(ROOT / "ram-scb_gb300"))
    from ramgpu import workload as W

    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict((r, (parts, rows)) for r, parts, rows in (q.get(timeout=180) for _ in ps))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    ens = W.make_ensemble(48, seed=77)
    sums = [float(np.sum(a)) for a in ens.base.f2]
    expect = [[sums[s] * float(ens.scale[m]) for s in ens.species[m]] for m in range(48)]
    parts0, rows0 = got[0]
    parts1, rows1 = got[1]
    assert parts0 == parts1 and sorted(parts0[0] + parts0[1]) == list(range(48))
    assert parts0[0] and parts0[1]
    assert rows0 == rows1 == expect
