"""The multi-GPU dealing of stacks (the reference launcher's rule, script/HDoG_gpu.py:67-98)
and its use by one process per GPU, checked on CPU with two gloo ranks."""
import json
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import hdog
from hdog import launch


def fake_tree(root, sizes):
    """{root}/{Y}/{Y}_{X}/{Z}.bin with the given slice counts; returns the stack dirs."""
    dirs = []
    for i, n in enumerate(sizes):
        y = "%06d" % (100000 + 1000 * (i // 3))
        d = os.path.join(root, y, "%s_%06d" % (y, 200000 + 1000 * (i % 3)))
        os.makedirs(d)
        for z in range(n):
            np.zeros(4, np.uint16).tofile(os.path.join(d, "%06d.bin" % z))
        dirs.append(d)
    return dirs


def test_assign_is_sorted_round_robin(tmp_path):
    dirs = fake_tree(str(tmp_path), [5, 9, 7, 3, 9, 1])
    stacks = launch.list_stacks(str(tmp_path))
    assert sorted(n for _, n in stacks) == [1, 3, 5, 7, 9, 9]
    by_gpu = launch.assign_stacks(stacks, [0, 1])
    counts = {g: [dict(stacks)[d] for d in v] for g, v in by_gpu.items()}
    # largest first, dealt alternately
    assert counts[0][0] == 9 and counts[1][0] == 9
    assert sorted(counts[0] + counts[1]) == [1, 3, 5, 7, 9, 9]
    assert counts[0] == sorted(counts[0], reverse=True) and counts[1] == sorted(counts[1], reverse=True)
    assert set(by_gpu[0]) | set(by_gpu[1]) == set(dirs) and not set(by_gpu[0]) & set(by_gpu[1])
    # zmin/zmax limit the slices counted
    assert sorted(n for _, n in launch.list_stacks(str(tmp_path), 1, 4)) == [0, 2, 3, 3, 3, 3]


def test_gpu_param_files_load_in_the_library(tmp_path):
    src = tmp_path / "src"
    fake_tree(str(src), [4, 2, 3])
    params = {"devID": 0, "gpus": [0, 1], "verbose": 0,
              "input_image_info": {"width": 2, "height": 2, "left_margin": 0, "right_margin": 0,
                                   "top_margin": 0, "bottom_margin": 0},
              "coordinate_info": {"scale_x": 1.0, "scale_y": 1.0, "scale_z": 1.0},
              "HDoG_param": {"depth": 32, "extra_depth_margin": 3, "radius_norm": {"xy_large": 20, "z_large": 5},
                             "min_intensity": 50, "gamma_n": 1.0,
                             "sigma_dog": {"xy_small": 2.0, "z_small": 1.5, "xy_large": 3.2, "z_large": 2.4},
                             "min_size": 0}}
    by_gpu = launch.assign_stacks(launch.list_stacks(str(src)), [0, 1])
    files = launch.write_gpu_param_files(params, by_gpu, str(tmp_path / "dst"), str(tmp_path))
    assert [os.path.basename(f) for f in files] == ["param_gpu00.json", "param_gpu01.json"]
    for gpu, f in zip((0, 1), files):
        d = json.load(open(f))
        assert d["devID"] == gpu and len(d["stacks"]) == len(by_gpu[gpu])
        p = hdog.load_param_file(f)     # the library's own reader accepts it
        assert p.dev_id == gpu and p.depth == 32
    n = sum(len(json.load(open(f))["stacks"]) for f in files)
    assert n == 3


def _rank_main(rank, world, port, stacks, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = launch.shard_for_rank(stacks, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    # the bench's timing rule: the job takes as long as its slowest rank
    t = torch.tensor([float(sum(dict(stacks)[d] for d in mine))], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        with open(out, "w") as f:
            json.dump({"shards": gathered, "max_slices": float(t.item())}, f)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_partition_the_stacks(tmp_path):
    stacks = [("stack%02d" % i, n) for i, n in enumerate([128, 512, 64, 300, 300, 96, 480])]
    out = str(tmp_path / "shards.json")
    mp.spawn(_rank_main, args=(2, _free_port(), stacks, out), nprocs=2, join=True)
    res = json.load(open(out))
    a, b = res["shards"]
    assert set(a) | set(b) == {s for s, _ in stacks} and not set(a) & set(b)
    assert a == launch.assign_stacks(stacks, [0, 1])[0] and b == launch.assign_stacks(stacks, [0, 1])[1]
    slices = dict(stacks)
    assert res["max_slices"] == max(sum(slices[s] for s in a), sum(slices[s] for s in b))
