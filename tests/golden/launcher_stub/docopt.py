"""A minimal stand-in for the docopt package (absent from this image), enough for the
reference launcher's usage line `HDoG_gpu PARAM_FILE [single <xname> <yname>] [--zmin <ZMIN>]
[--zmax <ZMAX>] [--exec <path>]`.  Used only by make_launcher_golden.py."""
import sys


def docopt(doc, argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    out = {"PARAM_FILE": None, "single": False, "<xname>": None, "<yname>": None, "--zmin": None, "--zmax": None,
           "--exec": "/usr/local/bin/HDoG3D_main"}
    pos = []
    i = 0
    while i < len(argv):
        a = argv[i]
        if a in ("--zmin", "--zmax", "--exec"):
            out[a] = argv[i + 1]
            i += 2
            continue
        pos.append(a)
        i += 1
    out["PARAM_FILE"] = pos[0]
    if len(pos) >= 4 and pos[1] == "single":
        out["single"], out["<xname>"], out["<yname>"] = True, pos[2], pos[3]
    return out
