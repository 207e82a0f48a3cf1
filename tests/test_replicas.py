"""bench.py's replica path (one process per GPU, no collective on the data path) on two
gloo ranks on the CPU: the max-over-ranks time and the whole-job throughput."""
import json
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init(world)
    bench.barrier(w)
    ms_local = 100.0 + 50.0 * r  # rank 1 is the slow one
    value, ms = bench.replica_value(1e9, 4, ms_local, w)
    import torch.distributed as td
    td.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump({"rank": r, "world": w, "value": value, "ms": ms}, f)


def test_two_replicas_report_max_time_and_summed_throughput(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % k))) for k in range(2)]
    for r in res:
        assert r["world"] == 2
        assert r["ms"] == pytest.approx(150.0)  # the slowest rank's time
        # 2 ranks x 4 steps x 1e9 units in 0.15 s
        assert r["value"] == pytest.approx(2 * 4 * 1e9 / 0.15 / 1e9)


def test_single_process_is_its_own_max(tmp_path):
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.replica_value(2e9, 10, 500.0, 1)
    assert ms == 500.0 and value == pytest.approx(2e9 * 10 / 0.5 / 1e9)
