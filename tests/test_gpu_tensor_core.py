"""The tensor-core (tcgen05) element kernel: the velocity-gradient and
weak-divergence contractions as split-precision MMA products with FP32
accumulation, everything else as in the CUDA-core kernel.

Tolerances, relative L2 over all seismogram samples after 200 steps:
TF32x3 (three products of 11-bit parts, about 22 significant bits) stays
within the FP32 tolerance of 1e-4 of the FP64 build; BF16x3 (8-bit parts,
about 16 significant bits) within 1e-3 of the FP64 build.
"""
import copy

import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import TOL, rel_l2, run_gpu, run_oracle, small_workload, with_grid

MODES = {"tf32x3": (sesnt.FLAG_TC_TF32X3, TOL), "bf16x3": (sesnt.FLAG_TC_BF16X3, 1e-3)}


def test_flags_are_validated(sesnt_lib):
    g = small_workload(4).grid
    g.precision = 8
    g.flags = sesnt.FLAG_TC_TF32X3
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.Simulation(g)
    assert e.value.code == sesnt.EUNSUPPORTED
    g.precision = 4
    g.flags = sesnt.FLAG_TC_TF32X3 | sesnt.FLAG_TC_BF16X3
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.Simulation(g)
    assert e.value.code == sesnt.EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("lpd,n_sls,aniso", [(4, 0, False), (4, 3, False), (4, 0, True), (2, 0, False),
                                              (3, 3, False), (5, 0, False), (6, 3, True), (7, 0, False)])
def test_tensor_core_kernel_matches_fp64(gpu, sesnt_lib, mode, lpd, n_sls, aniso):
    flag, tol = MODES[mode]
    wl = small_workload(lpd, n_sls=n_sls, aniso=aniso, nt=200)
    ref, fref, _ = run_gpu(with_grid(wl, precision=8), 200)
    cc, fcc, _ = run_gpu(wl, 200)
    tc, ftc, _ = run_gpu(with_grid(wl, flags=flag), 200)
    assert np.abs(ref).max() > 0
    e_tc, e_cc = rel_l2(tc, ref), rel_l2(cc, ref)
    print("lpd %d sls %d aniso %d %s: vs FP64 %.2e (CUDA-core FP32 %.2e)" % (lpd, n_sls, aniso, mode, e_tc, e_cc))
    assert e_tc < tol
    for k in fref:
        assert rel_l2(ftc[k], fref[k]) < 10 * tol, k


@pytest.mark.gpu
@pytest.mark.parametrize("mode", sorted(MODES))
def test_tensor_core_config1_against_oracle(gpu, sesnt_lib, oracle_mod, mode):
    """Homogeneous elastic 12x12x8 lpd 4, 600 steps (the largest field in
    the section) against the FP32 oracle."""
    flag, tol = MODES[mode]
    wl = workloads.config1(nt=600)
    got, _, _ = run_gpu(with_grid(wl, flags=flag), 600)
    want, _, o = run_oracle(oracle_mod, wl, 600)
    o.close()
    e = rel_l2(got[0], want)
    print("config 1, 600 steps, %s vs FP32 oracle: %.2e" % (mode, e))
    assert e < tol


@pytest.mark.gpu
def test_tensor_core_batch_and_graph(gpu, sesnt_lib):
    """Batched simulations (one block per element and simulation) through the
    graph replay give the traces of separate ungraphed runs."""
    wl = small_workload(4, n_sls=3, nt=100)
    g = copy.copy(wl.grid)
    g.batch, g.flags = 3, sesnt.FLAG_TC_TF32X3
    srcs = []
    for s in range(3):
        src = copy.copy(wl.sources[0])
        src.sim, src.lat, src.lon = s, 34.0 + s, 3.5 + 1.5 * s
        srcs.append(src)
    gs, _, _ = run_gpu(workloads.Workload("batch3", g, wl.model, srcs, wl.receivers), 100, fields=())
    for s in range(3):
        one = workloads.Workload("one", with_grid(wl, flags=sesnt.FLAG_TC_TF32X3 | sesnt.FLAG_NO_GRAPH).grid,
                                 wl.model, [copy.copy(srcs[s])], wl.receivers)
        one.sources[0].sim = 0
        os_, _, _ = run_gpu(one, 100, fields=())
        assert rel_l2(gs[s], os_[0]) < 1e-5


@pytest.mark.gpu
def test_completion_wait_runs_out_and_reports(gpu, sesnt_lib):
    """Failure detection without a fault: with the completion signal dropped
    the kernel's bounded mbarrier waits run out, the error word is set and
    synchronising returns SESNT_ETIMEOUT; after sesnt_reset the handle steps
    normally again."""
    wl = small_workload(4, nt=40)
    g = with_grid(wl, flags=sesnt.FLAG_TC_TF32X3)
    with sesnt.Simulation(g.grid) as sim:
        workloads.setup(sim, g)
        sim.set_wait_limit(64, drop_completion=True)
        sim.run(1, 2)
        with pytest.raises(sesnt.SesntError) as e:
            sim.synchronize()
        assert e.value.code == sesnt.ETIMEOUT
        with pytest.raises(sesnt.SesntError) as e:
            sim.seismograms()
        assert e.value.code == sesnt.ETIMEOUT
        sim.set_wait_limit(1 << 22)
        sim.reset()
        sim.run(1, 40)
        again = sim.seismograms()
    fresh, _, _ = run_gpu(g, 40, fields=())
    assert rel_l2(again, fresh) < 1e-6
