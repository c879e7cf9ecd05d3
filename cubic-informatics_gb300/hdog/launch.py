"""Dealing stacks to GPUs, as the reference's launcher does (script/HDoG_gpu.py:39-103).

A brain is many independent stacks (one per camera tile), so the work shards by stack with
no exchange between GPUs: stacks are sorted by slice count (largest first) and dealt
round-robin to the GPUs, and each GPU gets its own parameter file with its `devID` and its
`stacks` list.  The same assignment serves one process per GPU under torch.distributed
(`shard_for_rank`), where rank r plays the part of the r-th GPU of the list.
"""
import copy
import glob
import json
import os


def list_stacks(src_basedir, zmin=None, zmax=None):
    """[(stack_dir, n_slices)] for the layout {src_basedir}/{Y}/{Y}_{X}/{Z}.bin
    (HDoG_gpu.py:57-66), slices [zmin:zmax] of each stack."""
    out = []
    for d in glob.glob(os.path.join(src_basedir, "*", "*")):
        out.append((d, len(sorted(glob.glob(os.path.join(d, "*.bin")))[zmin:zmax])))
    return out


def assign_stacks(stacks, gpus):
    """{gpu: [stack_dir, ...]}: stacks sorted by slice count, largest first, then stack i
    goes to gpus[i % len(gpus)] (HDoG_gpu.py:67-77).  Equal counts keep their given order."""
    order = sorted(stacks, key=lambda s: s[1], reverse=True)
    out = {g: [] for g in gpus}
    for i, (path, _) in enumerate(order):
        out[gpus[i % len(gpus)]].append(path)
    return out


def shard_for_rank(stacks, rank, world_size):
    """The stacks rank `rank` of `world_size` processes handles (the assignment above with
    gpus = 0 .. world_size-1)."""
    return assign_stacks(stacks, list(range(world_size)))[rank]


def write_gpu_param_files(params, stacks_by_gpu, dst_dir, out_dir, zmin=None, zmax=None):
    """One parameter file per GPU, param_gpuNN.json in out_dir (HDoG_gpu.py:79-98): a copy of
    `params` (the parsed JSON of the whole run) with devID set and a `stacks` list of
    {dst_path: dst_dir/{Y}_{X}.bin, src_paths: sorted slices}.  Returns the file paths."""
    paths = []
    for gpu, dirs in stacks_by_gpu.items():
        p = copy.deepcopy(params)
        p["devID"] = gpu
        p["stacks"] = []
        for d in dirs:
            yx = os.path.basename(os.path.normpath(d))
            src = sorted(glob.glob(os.path.join(d, "*.bin")))[zmin:zmax]
            p["stacks"].append({"dst_path": os.path.join(dst_dir, "%s.bin" % yx), "src_paths": src})
        path = os.path.join(out_dir, "param_gpu%02d.json" % gpu)
        with open(path, "w") as f:
            json.dump(p, f, indent=4)
        paths.append(path)
    return paths
