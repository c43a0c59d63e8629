"""The replica path of bench.py (N > 1 under torchrun) on CPU: two gloo ranks,
world_size 2, rendezvous on 127.0.0.1.  Each rank times its own problem; the
job's time is the maximum over ranks, which every rank must agree on."""

import json
import os
import socket
import sys
from pathlib import Path

import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, out_dir: str) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist, r, world, local = bench.dist_setup()
    assert dist is not None and dist.get_backend() == "gloo"
    ms = bench.reduce_max(dist, 10.0 + 5.0 * rank, torch.device("cpu"))
    units = bench.reduce_max(dist, float(rank), torch.device("cpu"))
    Path(out_dir, f"{rank}.json").write_text(json.dumps({"rank": r, "world": world, "local": local,
                                                          "max_ms": ms, "max_rank": units}))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_max_time(tmp_path):
    mp.spawn(_rank, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    out = [json.loads((tmp_path / f"{r}.json").read_text()) for r in range(2)]
    assert [o["rank"] for o in out] == [0, 1]
    assert all(o["world"] == 2 for o in out)
    assert all(o["max_ms"] == 15.0 for o in out)
    assert all(o["max_rank"] == 1.0 for o in out)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    dist, rank, world, local = bench.dist_setup()
    assert dist is None and (rank, world, local) == (0, 1, 0)
    assert bench.reduce_max(None, 7.5, torch.device("cpu")) == 7.5
