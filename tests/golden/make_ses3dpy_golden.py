"""Golden GLL knots and point coordinates made by the reference's own Python
package (ses3dpy/ses3dpy.py: get_knots, generate_coordinates, with the
configs parsed by ses3dpy/namelist.py) for the NAMELIST configs under
tests/golden/configs/.

ses3dpy is Python 2 code; importing it under Python 3 needs the old StringIO
module name (supplied from io) and its own directory on the path (its config
reader imports `namelist` as a top-level module). Run from the repository
root with SES3D_NT_REFERENCE naming a checkout of the reference:
    SES3D_NT_REFERENCE=path/to/Ses3d-NT python tests/golden/make_ses3dpy_golden.py
"""
import glob
import io
import json
import os
import sys
import types

REFERENCE = os.environ.get("SES3D_NT_REFERENCE", "")


def reference_module():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "ses3dpy")):
        raise SystemExit("set SES3D_NT_REFERENCE to a checkout of the reference (it holds ses3dpy/)")
    m = types.ModuleType("StringIO")
    m.StringIO = io.StringIO
    sys.modules.setdefault("StringIO", m)
    sys.path[:0] = [REFERENCE, os.path.join(REFERENCE, "ses3dpy")]
    from ses3dpy import ses3dpy
    return ses3dpy


def main():
    s = reference_module()
    out = {"knots": {str(lpd): [float(x) for x in s.get_knots(lpd)] for lpd in range(2, 8)}, "configs": {}}
    here = os.path.dirname(os.path.abspath(__file__))
    from namelist import namelist2dict
    for conf in sorted(glob.glob(os.path.join(here, "configs", "*.conf"))):
        # the parameters ses3dpy.read_config_file derives (ses3dpy.py:69-78); that
        # function itself also wants the older format's `pml` key, which these
        # configs (the current format, taper_width) do not have
        c = namelist2dict(conf)
        g, m = c["grid"][0], c["model"][0]
        par = {"nX_global": (g["nx"], g["ny"], g["nz"]), "lpd": g["lpd"],
               "minX": (90.0 - m["lat_max"], m["lon_min"], m["rad_min"]),
               "maxX": (90.0 - m["lat_min"], m["lon_max"], m["rad_max"])}
        theta, phi, r = s.generate_coordinates(par)
        out["configs"][os.path.basename(conf)] = {
            "nX_global": [int(n) for n in par["nX_global"]], "lpd": int(par["lpd"]),
            "minX": [float(x) for x in par["minX"]], "maxX": [float(x) for x in par["maxX"]],
            "theta": [float(x) for x in theta], "phi": [float(x) for x in phi], "r": [float(x) for x in r]}
    path = os.path.join(here, "ses3dpy_geometry.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main()
