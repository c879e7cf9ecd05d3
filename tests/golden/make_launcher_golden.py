"""Writes launcher_param_files.json: the per-GPU parameter files the reference's own
launcher, script/HDoG_gpu.py, writes for a small synthetic tree
{src_basedir}/{Y}/{Y}_{X}/{Z}.bin (its run of the executable replaced by a stub that keeps a
copy of each file it is given).  The reference checkout is read from HDOG_REFERENCE or the
first argument; docopt, absent from this image, is stood in for by launcher_stub/docopt.py.

    python tests/golden/make_launcher_golden.py [REFERENCE_DIR]
"""
import glob
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cubic-informatics_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import launcher_tree  # noqa: E402


def main(ref):
    script = os.path.join(ref, "script", "HDoG_gpu.py")
    tmp = tempfile.mkdtemp(prefix="hdog_launcher_")
    try:
        param_file = launcher_tree.build(tmp)
        capture = os.path.join(tmp, "captured")
        os.makedirs(capture)
        stub = os.path.join(tmp, "exec_stub.sh")
        with open(stub, "w") as f:
            f.write("#!/bin/sh\ncp \"$1\" %s/\necho stub ran \"$1\"\n" % capture)
        os.chmod(stub, 0o755)
        env = dict(os.environ, PYTHONPATH=os.path.join(HERE, "launcher_stub"))
        subprocess.run([sys.executable, script, param_file, "--exec", stub], check=True, env=env, cwd=tmp)
        files = {}
        for p in sorted(glob.glob(os.path.join(capture, "param_gpu*.json"))):
            d = json.load(open(p))
            files[os.path.basename(p)] = launcher_tree.relative(d, tmp)
        out = {"generator": "tests/golden/make_launcher_golden.py", "script": "script/HDoG_gpu.py",
               "tree": launcher_tree.STACKS, "param_files": files}
        with open(os.path.join(HERE, "launcher_param_files.json"), "w") as f:
            json.dump(out, f, indent=1)
        print("wrote %d parameter files" % len(files))
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HDOG_REFERENCE", "/root/reference"))
