"""Compensated (Kahan) stress integration, SESNT_FLAG_KAHAN_STRESS.

On coarse grids the FP32 error against FP64 over long runs comes almost
entirely from the rounding of the stored stress at each step: rounding only
the stored stress of an FP64 oracle run to FP32 reproduces the whole FP32
error of the config-3 generator on 16x16x8 elements, while rounding the
strain, the stress rates or the memory variables instead gives less than 1%
of it. With six compensation
terms per point the integration keeps the low-order part the stored stress
loses.

- On the config-3 generator (lpd 6, 3 SLS, staged kernel) at config 3's
  time step and length, the compensated FP32 run's seismograms are at least
  twice as close to the FP64 build as the plain FP32 run's (2.8x measured:
  7.1e-6 -> 2.4e-6 over 4000 steps), also with the velocity update
  compensated too (SESNT_FLAG_KAHAN), and within the FP32 bound 1e-4 of the
  FP32 oracle. (On config 3's full 96x96x48 grid the stress rounding is no
  longer the dominant term and the flag gains nothing there.)
- On small degree-4 SLS (staged kernel), elastic and degree-3 SLS
  (one point per thread) workloads, batches included, it stays within the
  FP32 bound of the FP64 build.
- FP64 handles with the flag equal plain FP64 to rounding.
- The tensor-core, persistent and strain flags are refused with it.
"""
import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import rel_l2, small_workload, with_grid

pytestmark = pytest.mark.gpu

TOL = 1e-4


def run(wl, steps):
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        name, _ = sim.element_kernel()
        sim.run(1, steps)
        return sim.seismograms().astype(np.float64), sim.field("vz", precision=8), name


def test_compensated_stress_config3_generator(gpu, sesnt_lib, oracle_mod):
    # config 3's time step and length: the stress-rounding error grows with the
    # number of steps (at 5x the time step over 1000 steps it is a small part)
    steps = 4000
    wl = workloads.config3(nt=steps, nx=16, ny=16, nz=8)
    s64, v64, _ = run(with_grid(wl, precision=8), steps)
    sp, vp, name_p = run(wl, steps)
    sk, vk, name_k = run(with_grid(wl, flags=sesnt.FLAG_KAHAN_STRESS), steps)
    sb, vb, _ = run(with_grid(wl, flags=sesnt.FLAG_KAHAN_STRESS | sesnt.FLAG_KAHAN), steps)
    o = oracle_mod.Oracle(wl.grid, 4)
    oracle_mod.load_workload(o, wl)
    o.run(steps)
    so = o.seismograms()
    o.close()
    ep, ek = rel_l2(sp, s64), rel_l2(sk, s64)
    evp, evk = rel_l2(vp, v64), rel_l2(vk, v64)
    print("config3 generator 16x16x8 lpd 6, dt 0.03, %d steps, vs FP64: plain FP32 seismograms %.2e vz %.2e (%s), "
          "compensated stress %.2e vz %.2e (%s), compensated stress and velocity %.2e vz %.2e; "
          "compensated stress vs FP32 oracle %.2e"
          % (steps, ep, evp, name_p, ek, evk, name_k, rel_l2(sb, s64), rel_l2(vb, v64), rel_l2(sk[0], so)))
    assert name_k == "k_element_stage (register stores)"
    assert np.abs(s64).max() > 0
    # seismograms at least twice as close; the final vz (a decayed field, whose
    # relative error has a larger rounding floor) closer
    assert ek < 0.5 * ep and evk < evp
    assert rel_l2(sb, s64) < 0.5 * ep
    assert rel_l2(sk[0], so) < TOL


@pytest.mark.parametrize("case", ["sls_lpd4_batch2", "elastic_lpd4", "sls_lpd3", "sls_lpd6_aniso"])
def test_compensated_stress_small_workloads(gpu, sesnt_lib, case):
    wl = {"sls_lpd4_batch2": lambda: small_workload(4, n_sls=3, nt=300),
          "elastic_lpd4": lambda: small_workload(4, nt=300),
          "sls_lpd3": lambda: small_workload(3, n_sls=3, nt=300),
          "sls_lpd6_aniso": lambda: small_workload(6, n_sls=3, aniso=True, nt=300)}[case]()
    if case.endswith("batch2"):
        wl = with_grid(wl, batch=2)
        src = workloads.Source(**{**wl.sources[0].__dict__})
        src.sim, src.lat = 1, src.lat + 1.0
        wl.sources = wl.sources + [src]
    s64, _, _ = run(with_grid(wl, precision=8), 300)
    sp, _, _ = run(wl, 300)
    sk, _, name = run(with_grid(wl, flags=sesnt.FLAG_KAHAN_STRESS), 300)
    expect = "k_element_stage (register stores)" if wl.grid.n_sls and wl.grid.lpd >= 4 else "k_element"
    for s in range(wl.grid.batch):
        ep, ek = rel_l2(sp[s], s64[s]), rel_l2(sk[s], s64[s])
        print("%s sim %d vs FP64: plain FP32 %.2e, compensated stress %.2e (%s)" % (case, s, ep, ek, name))
        assert np.abs(s64[s]).max() > 0
        assert ek < TOL
    assert name == expect


def test_fp64_with_compensation_equals_fp64(gpu, sesnt_lib):
    wl = with_grid(small_workload(4, n_sls=3, nt=200), precision=8)
    d, vd, _ = run(wl, 200)
    k, vk, _ = run(with_grid(wl, flags=sesnt.FLAG_KAHAN_STRESS), 200)
    assert rel_l2(k, d) < 1e-10 and rel_l2(vk, vd) < 1e-10


def test_incompatible_flags_are_refused(gpu, sesnt_lib):
    wl = small_workload(4, nt=10)
    for other in (sesnt.FLAG_TC_TF32X3, sesnt.FLAG_PERSISTENT_ELEMENT, sesnt.FLAG_STRAIN):
        with pytest.raises(sesnt.SesntError) as ex:
            sesnt.Simulation(with_grid(wl, flags=sesnt.FLAG_KAHAN_STRESS | other).grid)
        assert ex.value.code == sesnt.EUNSUPPORTED
