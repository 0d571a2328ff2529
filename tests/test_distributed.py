"""Multi-process host logic on CPU (gloo, world size 2): photon sharding, the gather of
per-photon results, and the bench's max/sum-over-ranks timing reductions. The sharded trace
runs the oracle (the CPU checker) on each rank's slice, standing in for a rank's GPU, and
gathers the traced states."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys

    import torch
    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), BENCH_BACKEND="gloo")
    import bench
    from excalibur_tool_gb300.distributed import gather_rows, shard_range

    r, w, _ = bench.dist_setup(world)
    n = 11
    a, b = shard_range(n, r, w)
    rows = torch.arange(a * 3, b * 3, dtype=torch.float64).reshape(-1, 3)   # a stand-in for traced outputs
    full = gather_rows(rows, n)
    bench.barrier(w)
    mx = bench.max_over_ranks(float(r + 1) * 1.5, w)
    sm = bench.sum_over_ranks(float(b - a), w)
    out[rank] = (full.numpy().tolist(), mx, sm, (a, b))
    dist.destroy_process_group()


def test_shard_range_partitions():
    from excalibur_tool_gb300.distributed import shard_range

    for n in (0, 1, 7, 65536):
        for w in (1, 2, 3, 8):
            cuts = [shard_range(n, r, w) for r in range(w)]
            assert cuts[0][0] == 0 and cuts[-1][1] == n
            assert all(cuts[i][1] == cuts[i + 1][0] for i in range(w - 1))
            sizes = [b - a for a, b in cuts]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_gather_and_timing_reductions():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    want = np.arange(33, dtype=np.float64).reshape(11, 3).tolist()
    for r in range(2):
        full, mx, sm, cut = out[r]
        assert full == want
        assert mx == 3.0 and sm == 11.0
    assert out[0][3] == (0, 6) and out[1][3] == (6, 11)


def _shard_worker(rank, world, port, out):
    import sys

    import torch
    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), BENCH_BACKEND="gloo")
    import bench
    from excalibur_tool_gb300.distributed import gather_rows, shard_range
    from oracle import oracle as O
    from test_gpu_parity import _flrw_patch_case

    r, w, _ = bench.dist_setup(world)
    spec, st, cfg = _flrw_patch_case(16, 5)          # 25 rays through a 16^3 lens-plus-random-field box
    a, b = shard_range(len(st), r, w)
    mine = O.trace(spec, st[a:b], cfg, threads=1)
    cols = np.concatenate([mine.state, mine.status[:, None], mine.n_steps[:, None], mine.obs], axis=1)
    full = gather_rows(torch.from_numpy(cols), len(st))
    out[rank] = full.numpy()
    dist.destroy_process_group()


def test_two_rank_sharded_trace_gathers_the_whole_batch():
    """Each rank traces its shard_range slice of one batch; the gathered rows (final states,
    statuses, step counts, observables) are those of a single-process trace, on every rank."""
    import sys

    import torch.multiprocessing as mp

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle import oracle as O
    from test_gpu_parity import _flrw_patch_case

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs)
    spec, st, cfg = _flrw_patch_case(16, 5)
    whole = O.trace(spec, st, cfg, threads=1)
    want = np.concatenate([whole.state, whole.status[:, None], whole.n_steps[:, None], whole.obs], axis=1)
    for r in range(2):
        assert np.array_equal(out[r], want, equal_nan=True)
    assert (whole.status == 1).all()      # every ray left the box
