"""Multi-GPU path of the bench on CPU: independent replicas, one per rank,
joined over a world_size-2 gloo process group (no GPU, no data-path
collective).  The whole-job value is N steps per slowest rank's step time,
for the device-timed value and for e2e."""
import json
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    line = {"ms_per_step": 2.0 + rank, "value": 1e3 / (2.0 + rank), "n_gpus": 1,
            "e2e": {"value": 100.0 - 10 * rank, "unit": "SR steps/s"}}
    dist.barrier()
    bench.aggregate_replicas(line, world)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(line, f)


def test_replicas_aggregate_over_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(world):
        line = json.load(open(tmp_path / f"rank{r}.json"))
        assert line["n_gpus"] == 2
        assert line["ms_per_step"] == 3.0                    # slowest rank
        assert abs(line["value"] - 2 * 1e3 / 3.0) < 1e-9
        assert abs(line["e2e"]["value"] - 2 * 90.0) < 1e-9   # slowest rank's e2e, times N
