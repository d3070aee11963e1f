"""Golden parses of the NAMELIST configs under tests/golden/configs/, made by
the reference's own Python reader (ses3dpy.namelist.namelist2dict).

The reader is Python 2 code; importing it here under Python 3 needs only the
old StringIO module name, which is supplied from io. Run from the repository
root with SES3D_NT_REFERENCE naming a checkout of the reference:
    SES3D_NT_REFERENCE=path/to/Ses3d-NT python tests/golden/make_config_golden.py
"""
import glob
import io
import json
import os
import sys
import types

REFERENCE = os.environ.get("SES3D_NT_REFERENCE", "")


def reference_reader():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "ses3dpy")):
        raise SystemExit("set SES3D_NT_REFERENCE to a checkout of the reference (it holds ses3dpy/)")
    m = types.ModuleType("StringIO")
    m.StringIO = io.StringIO
    sys.modules.setdefault("StringIO", m)
    sys.path.insert(0, REFERENCE)
    from ses3dpy import namelist
    return namelist.namelist2dict


def main():
    read = reference_reader()
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "configs")
    for conf in sorted(glob.glob(os.path.join(here, "*.conf"))):
        d = read(conf)
        out = conf[:-5] + ".json"
        with open(out, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        print("wrote", out)


if __name__ == "__main__":
    main()
