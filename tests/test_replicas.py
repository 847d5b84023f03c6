"""The N > 1 path of bench.py: N independent replicas, one per rank, whose
timings are combined as the maximum over the ranks (gloo, two processes on the
CPU)."""
import json
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        # each replica reports its own (device, end-to-end) times
        got = bench.replica_max([1.0 + rank, 5.0 - rank], dist)
        with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
            json.dump(got, f)
    finally:
        dist.destroy_process_group()


def test_replica_timings_take_the_maximum_over_ranks(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = []
    for r in range(world):
        with open(tmp_path / f"rank{r}.json") as f:
            res.append(json.load(f))
    assert res[0] == res[1] == [2.0, 5.0]


def test_replica_max_on_one_rank_is_identity():
    import bench
    assert bench.replica_max([0.25, 3]) == [0.25, 3.0]


def test_rank_keeps_the_launchers_gpu_list():
    """A rank takes the LOCAL_RANK-th GPU of a CUDA_VISIBLE_DEVICES list the
    launcher set, and the bare local rank only when no list was set."""
    import bench
    assert bench.visible_device_for_rank(1, "4,5") == "5"
    assert bench.visible_device_for_rank(0, " 4, 5") == "4"
    assert bench.visible_device_for_rank(1, "GPU-aa,GPU-bb") == "GPU-bb"
    assert bench.visible_device_for_rank(1, None) == "1"
    assert bench.visible_device_for_rank(1, "") == "1"
    with pytest.raises(ValueError):
        bench.visible_device_for_rank(2, "4,5")
