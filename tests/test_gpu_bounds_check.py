"""The bounds-check build (-DSESNT_BOUNDS_CHECK): every global index of the
step kernels is checked against its buffer; an index out of range sets a bit
of the handle's error word (no device assert, no trap), which the next
synchronising call returns as SESNT_ERANGE. This is the stand-in for a
memory sanitizer: the library is rebuilt with the checks, and a subprocess
runs every kernel variant (degrees 2-7, elastic and SLS, anisotropy,
batches, FP32 and FP64, the staged, persistent, column (one and two
simulations per thread) and tensor-core element kernels, compensated stress
integration, the tuner's sweep, strain and rotation state, every receiver
channel, snapshot fields, the kinetic energy) on small grids."""
import os
import subprocess
import sys

import pytest

import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "ses3d-nt_gb300")

SCRIPT = r"""
import sys
sys.path[:0] = [%r, %r]
import numpy as np
import sesnt, workloads
from test_gpu_parity import small_workload, with_grid

ALL = 0xFFFF
C, CS, SR = sesnt.ELEMENT_COLUMNS, sesnt.ELEMENT_COLUMNS_STAGED, sesnt.ELEMENT_STAGE_REG
CP = sesnt.ELEMENT_COLUMNS_PAIR
cases = [  # lpd, n_sls, aniso, kind, flags, batch[, (variant, arg, piece) or "tune"[, precision]]
    (2, 0, False, sesnt.SOURCE_MT, 0, 1),
    (3, 3, False, sesnt.SOURCE_SF, 0, 2),
    (4, 3, True, sesnt.SOURCE_MT, sesnt.FLAG_STRAIN | sesnt.FLAG_ROTATION, 2),
    (4, 3, False, sesnt.SOURCE_MT, sesnt.FLAG_PERSISTENT_ELEMENT, 3),
    (4, 0, True, sesnt.SOURCE_SF, sesnt.FLAG_TC_TF32X3, 1),
    (5, 0, False, sesnt.SOURCE_MT, sesnt.FLAG_KAHAN, 1),
    (6, 3, False, sesnt.SOURCE_MT, sesnt.FLAG_TC_BF16X3, 1),
    (7, 0, True, sesnt.SOURCE_MT, sesnt.FLAG_PERSISTENT_ELEMENT, 1),
    (4, 3, False, sesnt.SOURCE_MT, 0, 1),
    (5, 3, True, sesnt.SOURCE_SF, 0, 2),
    (6, 3, False, sesnt.SOURCE_MT, 0, 2),
    (7, 3, False, sesnt.SOURCE_MT, sesnt.FLAG_KAHAN, 1),
    (2, 0, False, sesnt.SOURCE_MT, 0, 5, (C, 12, 0)),
    (4, 0, True, sesnt.SOURCE_SF, 0, 3, (C, 1, 0)),
    (4, 0, False, sesnt.SOURCE_MT, 0, 6, (CS, 9, 4096)),
    (7, 0, True, sesnt.SOURCE_MT, 0, 3, (CS, 15, 0)),
    (6, 0, False, sesnt.SOURCE_MT, 0, 2, (C, 0, 0), 8),
    (5, 3, False, sesnt.SOURCE_MT, 0, 2, (SR, 0, 4096)),
    (4, 0, False, sesnt.SOURCE_MT, 0, 4, "tune"),
    (4, 3, False, sesnt.SOURCE_MT, 0, 1, "tune", 8),
    (4, 3, False, sesnt.SOURCE_MT, sesnt.FLAG_FORCE64, 2),
    (4, 0, False, sesnt.SOURCE_SF, sesnt.FLAG_FORCE64, 4, (C, 1, 0)),
    (4, 3, True, sesnt.SOURCE_MT, 0, 3, (sesnt.ELEMENT_STAGE, 7, 0)),
    (6, 3, False, sesnt.SOURCE_MT, 0, 1, (SR, 6, 8192), 8),
    (4, 0, False, sesnt.SOURCE_MT, 0, 4, (CP, 9, 0)),
    (7, 0, True, sesnt.SOURCE_SF, 0, 2, (CP, 0, 0)),
    (3, 0, False, sesnt.SOURCE_MT, 0, 6, (CP, 10, 0), 8),
    (4, 3, False, sesnt.SOURCE_MT, sesnt.FLAG_KAHAN_STRESS, 2),
    (3, 3, True, sesnt.SOURCE_SF, sesnt.FLAG_KAHAN_STRESS, 1),
    (6, 0, False, sesnt.SOURCE_MT, sesnt.FLAG_KAHAN_STRESS, 1, None, 8),
]
for case in cases:
    lpd, n_sls, aniso, kind, flags, batch = case[:6]
    variant = case[6] if len(case) > 6 else None
    precision = case[7] if len(case) > 7 else 4
    wl = small_workload(lpd, n_sls=n_sls, aniso=aniso, kind=kind, nt=40)
    src = wl.sources[0]
    wl.receivers.insert(0, workloads.Receiver(lat=src.lat, lon=src.lon, depth=src.depth))
    g = with_grid(wl, flags=flags, batch=batch, precision=precision).grid
    with sesnt.Simulation(g) as sim:
        m = wl.model
        sim.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
        for s in range(batch):
            elem, vm = sesnt.locate_point(g, src.lat, src.lon, src.depth)
            stf = sesnt.source_signature(src.wavelet, src.onset, src.width, g.dt, g.nt)
            sim.add_source(s, elem, vm, kind, np.asarray(src.comp, np.float32), stf)
        for r in wl.receivers:
            elem, vm = sesnt.locate_point(g, r.lat, r.lon, r.depth)
            sim.add_receiver(elem, vm, ALL)
        sim.add_snapshot("pressure", 10, 10, 30, prefix=%r + "/",
                         attribute="p%%d_%%d_%%d" %% (lpd, flags, cases.index(case)))
        if variant == "tune":
            sim.tune()
        elif variant is not None:
            sim.set_element_variant(*variant)
        sim.run(1, 40)
        sim.synchronize()
        sim.wait_snapshots()
        for name in ("vz", "sxy", "pressure"):
            sim.field(name, sim=batch - 1)
        if flags & sesnt.FLAG_STRAIN:
            sim.field("exy")
        if flags & sesnt.FLAG_ROTATION:
            sim.field("rot_vz")
        for b in range(16):
            sim.trace(0, 1 << b, sim=batch - 1)
        sim.kinetic_energy(batch - 1)
        sim.synchronize()
    print("case", case, "clean")
print("OK", len(cases))
"""


def test_every_kernel_in_bounds(gpu, tmp_path):
    lib_dir = tmp_path / "bounds-check"
    build.build(extra_nvcc=["-DSESNT_BOUNDS_CHECK"], out_dir=str(lib_dir))
    env = dict(os.environ, SESNT_LIBRARY=str(lib_dir / "libsesnt.so"), SESNT_TUNE_CACHE=str(tmp_path / "tune.txt"))
    code = SCRIPT % (PKG, HERE, str(tmp_path))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "OK 30" in r.stdout
