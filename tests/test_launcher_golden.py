"""The launcher path against the reference's own launcher, script/HDoG_gpu.py.

tests/golden/launcher_param_files.json holds the per-GPU parameter files the reference's
launcher wrote for the tree of tests/launcher_tree.py (make_launcher_golden.py ran it with
its executable replaced by a stub).  On CPU, this package's restatement of the launcher
(hdog.launch) must write the same files for the same tree.  On the GPU, hdog_main runs on
the reference launcher's files as they are -- except devID, set to 0 here where one GPU
is visible -- and each result file must hold the oracle's records of its stack.
"""
import json
import os
import subprocess

import numpy as np
import pytest

import hdog
import launcher_tree
from hdog import launch
from oracle import oracle as orc

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "launcher_param_files.json")))


def test_restated_launcher_writes_the_reference_launchers_files(tmp_path):
    root = str(tmp_path)
    param_file = launcher_tree.build(root)
    params = json.load(open(param_file))
    stacks = launch.list_stacks(params["src_basedir"])
    by_gpu = launch.assign_stacks(stacks, params["gpus"])
    out = tmp_path / "out"
    out.mkdir()
    paths = launch.write_gpu_param_files(params, by_gpu, params["dst_basedir"], str(out))
    assert sorted(os.path.basename(p) for p in paths) == sorted(GOLDEN["param_files"])
    for p in paths:
        got = json.load(open(p))
        want = launcher_tree.absolute(GOLDEN["param_files"][os.path.basename(p)], root)
        assert got == want, os.path.basename(p)


@pytest.mark.gpu
def test_hdog_main_on_the_reference_launchers_files(tmp_path):
    root = str(tmp_path)
    launcher_tree.build(root)
    os.makedirs(os.path.join(root, "result"))
    op = orc.params_from(launcher_tree.params())
    lengths = {"%s_%s" % (y, x): (n, seed) for y, x, n, seed in launcher_tree.STACKS}
    done = 0
    for name, content in sorted(GOLDEN["param_files"].items()):
        d = launcher_tree.absolute(content, root)
        d["devID"] = 0
        path = os.path.join(root, name)
        with open(path, "w") as f:
            json.dump(d, f, indent=4)
        r = subprocess.run([hdog.MAIN_PATH, path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode == 0, r.stdout
        for s in d["stacks"]:
            yx = os.path.basename(s["dst_path"])[:-4]
            n, seed = lengths[yx]
            got = np.fromfile(s["dst_path"], dtype=hdog.DT_LOCAL)
            want = orc.stack(op, launcher_tree.stack_volume(n, seed))
            assert len(got) == len(want) > 0, yx
            for f in ("local_x", "local_y", "local_z", "intensity", "size"):
                assert np.array_equal(got[f], want[f]), (yx, f)
            done += 1
    assert done == len(launcher_tree.STACKS)
