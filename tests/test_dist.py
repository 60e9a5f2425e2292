"""The multi-process path of bench.py on CPU (gloo, world size 2): one process
per GPU, independent batches per rank (weak scaling, no data-path
collective), a barrier and the max over ranks around the timed region, and
the reference arm printing from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    d.init("gloo")
    d.barrier()
    m = d.max(10.0 * (rank + 1))  # e.g. each rank's elapsed ms
    d.barrier()
    q.put((rank, m, bench.rank_batch(rank)["seed"]))
    d.done()


def test_dist_barrier_and_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [20.0, 20.0]   # both ranks see the slowest rank's time
    assert got[0][2] != got[1][2]                # each rank solves its own batch


def test_rank_batches():
    import bench
    b = [bench.rank_batch(r) for r in range(4)]
    assert len({x["seed"] for x in b}) == 4
    assert all(x["N"] == b[0]["N"] and x["n"] == b[0]["n"] for x in b)


def test_reference_arm_two_ranks():
    """torchrun with 2 ranks: rank 0 times the CPU reference and prints one
    JSON line, rank 1 exits without work."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--ref-sample", "512"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["value"] > 0 and out["n_gpus"] == 2
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["cpu_baseline"]["cores"] >= 1


@pytest.mark.parametrize("parts", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("block_cnt", [0, 1, 7, 2048, 2051])
def test_partition_blocks_covers_every_block_once(block_cnt, parts):
    """ves_partition_blocks (host code): contiguous, disjoint, in order, every
    block exactly once, part sizes differing by at most one (ragged tails)."""
    import ves
    got = [ves.partition_blocks(block_cnt, parts, p) for p in range(parts)]
    nxt = 0
    for first, nb in got:
        assert first == nxt and nb >= 0
        nxt = first + nb
    assert nxt == block_cnt
    sizes = [nb for _, nb in got]
    assert max(sizes) - min(sizes) <= 1


def test_partition_blocks_rejects_bad_arguments():
    import ves
    for args in ((-1, 2, 0), (8, 0, 0), (8, 2, 2), (8, 2, -1)):
        with pytest.raises(ves.VesError):
            ves.partition_blocks(*args)


def _split_rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    import ves
    dist.init_process_group("gloo")
    first, nb = ves.partition_blocks(2051, world, rank)
    mine = torch.arange(first, first + nb, dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([nb], dtype=torch.int64))
    allb = [torch.zeros(int(s.item()), dtype=torch.int64) for s in sizes]
    if all(int(s.item()) == nb for s in sizes):
        dist.all_gather(allb, mine)
    else:  # gloo all_gather needs equal sizes: pad
        m = max(int(s.item()) for s in sizes)
        pad = torch.full((m,), -1, dtype=torch.int64)
        pad[:nb] = mine
        bufs = [torch.zeros(m, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(bufs, pad)
        allb = [b[b >= 0] for b in bufs]
    q.put((rank, sorted(torch.cat(allb).tolist())))
    dist.destroy_process_group()


def test_split_batch_two_ranks_gloo():
    """Two ranks (gloo): the parts each rank takes cover the batch's blocks
    exactly once, as every rank sees them."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_split_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for _ in range(2):
        _, blocks = q.get(timeout=10)
        assert blocks == list(range(2051))
