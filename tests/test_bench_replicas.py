"""Host logic of bench.py's multi-GPU (replica) mode, world size 2 on gloo,
CPU only: the process group comes up from the torchrun environment
variables, the timing reduction takes the slowest rank, the barrier
releases both ranks, every rank starts at a different pose, and the job
value counts every rank's rays.  Rays are independent, so replicas exchange
nothing on the data path."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    try:
        os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                           "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
        sys.path.insert(0, ROOT)
        import bench
        w, r, local = bench._dist()
        mx = bench._max_over_ranks(w, 10.0 + 5.0 * r)
        bench._barrier(w)
        poses = bench.rank_poses(r, 8)
        import torch.distributed as dist
        dist.destroy_process_group()
        q.put((r, w, local, mx, poses))
    except Exception as e:  # report instead of hanging the parent
        q.put((rank, "error", repr(e)))


def test_two_gloo_ranks_reduce_max_and_split_poses():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = {}
    try:
        for _ in range(2):
            item = q.get(timeout=120)
            assert item[1] != "error", item
            res[item[0]] = item
    finally:
        for p in ps:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    assert sorted(res) == [0, 1]
    for r, (rank, w, local, mx, poses) in res.items():
        assert (rank, w, local) == (r, 2, r)
        assert mx == 15.0                       # the slower rank's time
        assert sorted(poses) == list(range(8))  # each rank cycles all poses
    assert res[0][4][0] != res[1][4][0]         # from different starting poses


def test_job_value_counts_all_ranks():
    sys.path.insert(0, ROOT)
    import bench
    # 2 ranks x 4 frames of 921,600 rays in 10 ms (slowest rank) = 737.28 Mrays/s
    assert bench.job_value(2, 921600, 4, 10.0) == pytest.approx(737.28)
    assert bench.job_value(1, 921600, 4, 10.0) == pytest.approx(368.64)
