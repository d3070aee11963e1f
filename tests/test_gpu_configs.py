"""Oracle parity at the sizes of the named workloads, through the C ABI.

- The heterogeneous visco-elastic section at full size (48x48x24 elements,
  lpd 4, 3 SLS, 64 receivers), 900 steps (past the peak of the 60 s Ricker
  wavelet at 90 s): seismograms and the final velocity, stress and all 18
  memory-variable fields against the FP32 oracle, each error also stated
  against the FP64 build of the same kernels. A shorter FP64 run checks the
  FP64 build against the FP64 oracle on the same grid.
- The batched grid (64x64x32 elements, lpd 4, 3 SLS) with 4 of its 64
  seeded sources in one batch, each simulation against its own oracle run.
  The 4 are the shallowest of the 64 (their positions and moment tensors
  as seeded), with the wavelets shortened to a width of 16 s (the grid's
  resolved period, 1/f_c) and onset 24 s, so that the pulse reaches the
  surface receivers within the 250 steps the oracle can afford here; from
  the deeper seeded sources (up to 300 km) nothing arrives in 25 s, and
  relative errors of pre-arrival noise say nothing. The FP64 build of the
  same batch is the anchor each error is also stated against.
- The precision workload's generator (lpd 6, 3 SLS) on a 16x16x8 grid, dt
  0.15 s (Courant number 0.22 on this coarser grid), 1000 steps (150 s):
  the FP32 CUDA-core kernel, the Kahan-compensated update and the two
  tensor-core contraction variants against the FP32 oracle, and the FP64
  build against the FP64 oracle. Seismograms over all 1000 steps;
  wavefields at step 650 (97.5 s, the field's largest extent, just after the
  wavelet's peak at 90 s). By step 1000 the taper has absorbed most of the
  pulse, and there, as in any FP32 run of a decayed field, the relative
  error of a wavefield is set by rounding (both the GPU and the oracle sit
  near 1e-4 of FP64 there).

Tolerances: 1e-4 relative L2 for FP32 results (the required FP32 misfit), 1e-3
for the BF16x3 contractions (a split into three bfloat16 products keeps about
16 significant bits per product), 1e-10 for FP64 wavefields against the FP64
oracle, float32 output rounding (1e-7) for FP64 seismograms.
"""
import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import rel_l2, with_grid

pytestmark = pytest.mark.gpu

TOL = 1e-4
STATE = {"vx": 0, "vy": 1, "vz": 2, "sxx": 3, "sxy": 4, "sxz": 5, "syy": 6, "syz": 7, "szz": 8}
MEMORY = {"m%d" % x: sesnt.MEMORY_FIELD0 + x for x in range(18)}


def gpu_run(wl, steps):
    """Open handle after `steps` steps (the caller closes it)."""
    sim = sesnt.Simulation(wl.grid)
    workloads.setup(sim, wl)
    sim.run(1, steps)
    sim.synchronize()
    return sim


def oracle_run(oracle_mod, wl, steps, precision=4, sim=0):
    o = oracle_mod.Oracle(wl.grid, precision)
    oracle_mod.load_workload(o, wl, sim=sim)
    o.run(steps)
    return o


def check_fields(label, g32, o32, g64, names, tol, sim=0):
    """Field by field (one at a time, to keep host memory small): GPU FP32 vs
    oracle FP32 within tol; the GPU FP32 and oracle FP32 errors against the
    GPU FP64 build are printed."""
    worst = 0.0
    for name, code in names.items():
        a = g32.field(code, sim=sim, precision=8)
        b = o32.field(code).astype(np.float64)
        assert np.abs(b).max() > 0, (label, name)
        e = rel_l2(a, b)
        line = "%s %s: GPU-FP32 vs oracle-FP32 %.2e" % (label, name, e)
        if g64 is not None:
            c = g64.field(code, sim=sim, precision=8)
            line += ", GPU-FP32 vs FP64 %.2e, oracle-FP32 vs FP64 %.2e" % (rel_l2(a, c), rel_l2(b, c))
        print(line)
        worst = max(worst, e)
        assert e < tol, (label, name, e)
    return worst


def test_config2_full_grid_matches_oracle(gpu, sesnt_lib, oracle_mod):
    steps = 900
    wl = workloads.config2(nt=steps)
    g32 = gpu_run(wl, steps)
    g64 = gpu_run(with_grid(wl, precision=8), steps)
    try:
        o32 = oracle_run(oracle_mod, wl, steps)
        assert o32.visco()
        s32, s64, so = g32.seismograms()[0], g64.seismograms()[0], o32.seismograms()
        assert np.abs(so).max() > 0
        e = rel_l2(s32, so)
        print("config2 %d steps seismograms: GPU-FP32 vs oracle-FP32 %.2e, GPU-FP32 vs FP64 %.2e, "
              "oracle-FP32 vs FP64 %.2e" % (steps, e, rel_l2(s32, s64), rel_l2(so, s64)))
        assert e < TOL
        for c in range(3):
            assert rel_l2(s32[:, c], so[:, c]) < TOL, c
        check_fields("config2", g32, o32, g64, STATE, TOL)
        check_fields("config2", g32, o32, g64, MEMORY, TOL)
        o32.close()
    finally:
        g32.close()
        g64.close()


def test_config2_full_grid_fp64_equals_fp64_oracle(gpu, sesnt_lib, oracle_mod):
    steps = 150
    wl = with_grid(workloads.config2(nt=steps), precision=8)
    g = gpu_run(wl, steps)
    try:
        o = oracle_run(oracle_mod, wl, steps, precision=8)
        e = rel_l2(g.seismograms()[0].astype(np.float64), o.seismograms())
        print("config2 FP64 %d steps: seismograms vs FP64 oracle %.2e (float32 output)" % (steps, e))
        assert e < 1e-6
        for name, code in {**STATE, "m0": MEMORY["m0"], "m9": MEMORY["m9"], "m17": MEMORY["m17"]}.items():
            b = o.field(code)
            assert np.abs(b).max() > 0, name
            ef = rel_l2(g.field(code, precision=8), b)
            print("config2 FP64 %s vs FP64 oracle %.2e" % (name, ef))
            assert ef < 1e-10, name
        o.close()
    finally:
        g.close()


def test_config4_grid_batched_sources_match_oracle(gpu, sesnt_lib, oracle_mod):
    steps, batch = 250, 4
    wl = workloads.config4(nt=steps)  # the 64 seeded sources
    shallow = sorted(wl.sources, key=lambda x: x.depth)[:batch]
    wl.grid.batch = batch
    wl.sources = []
    for q, src in enumerate(shallow):
        src.sim, src.width, src.onset = q, 16.0, 24.0
        wl.sources.append(src)
    print("config4 grid: batch of the %d shallowest seeded sources, depths %s km"
          % (batch, ", ".join("%.0f" % (x.depth / 1e3) for x in wl.sources)))
    g = gpu_run(wl, steps)
    g64 = gpu_run(with_grid(wl, precision=8), steps)
    try:
        seis, seis64 = g.seismograms(), g64.seismograms()
        for s in range(batch):
            o = oracle_run(oracle_mod, wl, steps, sim=s)
            so = o.seismograms()
            assert np.abs(so).max() > 0
            e = rel_l2(seis[s], so)
            print("config4 grid, batch member %d, %d steps: seismograms GPU-FP32 vs oracle-FP32 %.2e, "
                  "GPU-FP32 vs FP64 %.2e, oracle-FP32 vs FP64 %.2e"
                  % (s, steps, e, rel_l2(seis[s], seis64[s]), rel_l2(so, seis64[s])))
            assert e < TOL
            check_fields("config4 sim %d" % s, g, o, g64,
                         {k: STATE[k] for k in ("vx", "vz", "sxz", "szz")} |
                         {k: MEMORY[k] for k in ("m0", "m8", "m17")}, TOL, sim=s)
            o.close()
    finally:
        g.close()
        g64.close()


def test_config3_generator_lpd6_variants_match_oracle(gpu, sesnt_lib, oracle_mod):
    steps, mid = 1000, 650
    names = ("vx", "vz", "sxx", "syz")
    wl = workloads.config3(nt=steps, nx=16, ny=16, nz=8)
    wl.grid.dt = 0.15

    def oracle(precision):
        o = oracle_mod.Oracle(wl.grid, precision)
        oracle_mod.load_workload(o, wl)
        o.run(mid)
        f = {k: o.field(STATE[k]).astype(np.float64) for k in names}
        o.run(steps - mid)
        s = o.seismograms()
        o.close()
        return s, f

    def gpu(grid):
        with sesnt.Simulation(grid) as sim:
            workloads.setup(sim, workloads.Workload(wl.name, grid, wl.model, wl.sources, wl.receivers))
            sim.run(1, mid)
            f = {k: sim.field(k, precision=8) for k in names}
            sim.run(mid + 1, steps - mid)
            return sim.seismograms()[0].astype(np.float64), f

    so, fo = oracle(4)
    so64, fo64 = oracle(8)
    assert np.abs(so).max() > 0
    print("config3 generator 16x16x8 lpd 6, %d steps: oracle-FP32 vs oracle-FP64 %.2e" % (steps, rel_l2(so, so64)))
    s64, f64 = gpu(with_grid(wl, precision=8).grid)
    e = rel_l2(s64, so64)
    print("  FP64 build: seismograms vs FP64 oracle %.2e" % e)
    assert e < 1e-6
    for k in names:
        assert rel_l2(f64[k], fo64[k]) < 1e-10, k
    variants = (("FP32", 0, TOL), ("Kahan", sesnt.FLAG_KAHAN, TOL), ("FP64 force", sesnt.FLAG_FORCE64, TOL),
                ("TF32x3", sesnt.FLAG_TC_TF32X3, TOL),
                ("BF16x3", sesnt.FLAG_TC_BF16X3, 1e-3))
    for label, flags, tol in variants:
        s, f = gpu(with_grid(wl, flags=flags).grid)
        e, e64 = rel_l2(s, so), rel_l2(s, so64)
        print("  %s: seismograms vs oracle-FP32 %.2e, vs FP64 %.2e" % (label, e, e64))
        assert e < tol, label
        for k in names:
            ef = rel_l2(f[k], fo[k])
            print("  %s: step-%d %s vs oracle-FP32 %.2e, vs FP64 %.2e, oracle-FP32 vs FP64 %.2e"
                  % (label, mid, k, ef, rel_l2(f[k], f64[k]), rel_l2(fo[k], fo64[k])))
            assert ef < tol, (label, k)
