"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1) run
independent replicas.  Checked: the per-rank seeds and packings differ, the
only collective is the clock reduction (maximum over ranks), and the
whole-job throughput is every rank's steps over the slowest rank's time."""
import json
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        env_ws, env_rank, _ = bench.dist_env()
        local_seconds = 1.0 + 0.5 * rank  # rank 1 is the slowest replica
        seconds = bench.max_over_ranks(local_seconds, env_ws, dist, torch, torch.device("cpu"))
        cfg = bench._configs()
        pos, radii, L = cfg.packing(16, 0.2, 0.05, bench.replica_seed(env_rank), sweeps=5)
        res = {"rank": env_rank, "ws": env_ws, "seconds": seconds,
               "value": bench.replica_throughput(env_ws, 3, seconds), "pos0": pos[0].tolist()}
        with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fp:
            json.dump(res, fp)
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    ws = 2
    mp.start_processes(_rank, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(ws)]
    assert [r["rank"] for r in res] == [0, 1] and all(r["ws"] == ws for r in res)
    # the clock reduction gives every rank the slowest replica's time
    assert all(r["seconds"] == pytest.approx(1.5) for r in res)
    assert all(r["value"] == pytest.approx(ws * 3 / 1.5) for r in res)
    # independent systems: different seeds, different packings
    assert not np.allclose(res[0]["pos0"], res[1]["pos0"])


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(2.5, 1, None, None, None) == 2.5
    assert bench.replica_throughput(1, 4, 2.0) == 2.0
    assert bench.replica_seed(0) != bench.replica_seed(1)
