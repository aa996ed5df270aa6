"""The replica path of bench.py (one stripe of the image per rank, no data exchange, job time = the
slowest rank's) with two gloo ranks on CPU: the stripes tile the range, every rank's stripe is the
same per-bin computation as a single-process run of that stripe (the oracle stands in for the GPU),
and the reduction gives every rank the maximum."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle as orc
    from viltrum_gb300 import scenes
    rmin, rmax = bench.stripe(rank, world)
    bins, _ = orc.port().per_bin_adaptive_nested(scenes.SCENE2, scenes.scene2(7), rmin, rmax, [8, 8],
                                                 orc.Nested.make(), 15)
    worst = bench.max_over_ranks(10.0 + rank, device="cpu")
    np.savez(os.path.join(out_dir, f"r{rank}.npz"), bins=bins, rmin=rmin, rmax=rmax, worst=worst)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    from oracle import oracle as orc
    from viltrum_gb300 import scenes
    got = [np.load(tmp_path / f"r{r}.npz") for r in range(world)]
    # stripes tile [0,1]^2 along y without overlap
    assert got[0]["rmin"][1] == 0.0 and got[-1]["rmax"][1] == 1.0
    for a, b in zip(got, got[1:]):
        assert a["rmax"][1] == b["rmin"][1]
    for r, g in enumerate(got):
        assert float(g["worst"]) == 10.0 + world - 1
        ref, _ = orc.port().per_bin_adaptive_nested(scenes.SCENE2, scenes.scene2(7), g["rmin"], g["rmax"], [8, 8],
                                                    orc.Nested.make(), 15)
        assert np.array_equal(ref, g["bins"])
