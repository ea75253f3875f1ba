"""bench.py's multi-rank path on CPU: N > 1 runs independent replicas (one per
GPU, no collective on the data path); the only cross-rank steps are the
barrier and the max over ranks of the timed value.  Two gloo ranks stand in
for the GPUs here."""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    dist = bench.dist_init(w, "gloo")
    value = bench.max_over_ranks(dist, 10.0 + rank)  # rank 1 is the slowest replica
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, local, value))


def test_max_over_ranks_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[3] == 11.0 for o in out)
    assert [o[2] for o in out] == [0, 1]


def test_batched_instances_shard_by_footprint():
    """The batched lambda-path sample is dealt to ranks by device footprint: every
    instance lands on exactly one rank, and no rank carries more than the
    average load plus its largest instance (greedy largest-first)."""
    sys.path.insert(0, ROOT)
    import bench
    fp = bench.batch_footprints(64)
    for world in (1, 2, 3, 8):
        shards = bench.shard_by_footprint(fp, world)
        assert sorted(i for s in shards for i in s) == list(range(64))
        loads = [sum(fp[i] for i in s) for s in shards]
        assert max(loads) <= sum(fp) / world + max(fp)
    assert bench.shard_by_footprint(fp[:2], 4)[2:] == [[], []]  # more ranks than instances
    # a rank's shard is the same instances the whole sample holds
    insts, lams = bench.batch_sample(6, only=[1, 4])
    full, flams = bench.batch_sample(6)
    assert [x.n for x in insts] == [full[1].n, full[4].n] and lams.shape == (2, 16)
    assert (lams == flams[[1, 4]]).all()


def _sum_rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist = bench.dist_init(world, "gloo")
    total = bench.sum_over_ranks(dist, 16.0 * (rank + 1))  # solves of each rank's shard
    slowest = bench.max_over_ranks(dist, 1.0 + rank)
    dist.destroy_process_group()
    q.put((rank, total, slowest))


def test_sharded_batched_totals_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_sum_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(o[1] == 48.0 and o[2] == 2.0 for o in out)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "lasso_m2e3_n1e4", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
