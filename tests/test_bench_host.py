"""CPU tests of bench.py's multi-process host logic (replicas): a gloo
world of 2 ranks agrees on the max-over-ranks time and passes barriers."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), QS3G_BENCH_BACKEND="gloo")
    import bench
    r, w, lr, dist = bench.dist_setup()
    try:
        bench.barrier(dist)
        m = bench.max_over_ranks(1.5 + r, dist)
        q.put((r, w, m))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]


def test_single_process_defaults():
    import bench
    for k in ("WORLD_SIZE", "RANK"):
        os.environ.pop(k, None)
    r, w, lr, dist = bench.dist_setup()
    assert (r, w, dist) == (0, 1, None)
    assert bench.max_over_ranks(3.0, None) == 3.0


def test_peaks_and_traffic_records():
    """The roofline denominators and the ncu traffic records the bench line
    cites: measured peaks when present, and a traffic entry for each kernel
    it reports a roofline for."""
    import bench
    hbm, kind = bench.peaks()
    assert hbm > 1000.0 and kind in ("measured", "fallback")
    assert bench.peaks_bf16() > 100.0
    tr = bench.traffic_record()
    for k in ("hv_chain64", "hv_tab_real_f32"):
        assert tr[k]["dram_bytes_per_launch"] > 1e9 and "ncu" in tr[k]["source"]


def test_arguments_of_the_optional_legs():
    """--batch, --cfg5, --dsf and --no-table parse; the default runs the
    ground-state solve with the connection table."""
    import sys
    import bench
    old = sys.argv
    try:
        sys.argv = ["bench.py"]
        a = bench.parse_args()
        assert a.solve and a.table and not a.batch and not a.cfg5 and a.batch_n == 256
        sys.argv = ["bench.py", "--batch", "--batch-n", "64", "--no-table", "--cfg5", "--dsf", "--no-solve"]
        a = bench.parse_args()
        assert a.batch and a.batch_n == 64 and not a.table and a.cfg5 and a.dsf and not a.solve
    finally:
        sys.argv = old
