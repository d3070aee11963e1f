"""Element-kernel variants and the tuner, through the C ABI.

- The column kernel (one thread per (i, j) column, z contractions in
  registers) and its two-simulations-per-thread form compute the step of the
  one-thread-per-point kernel: FP64 to 1e-12 relative L2, FP32 to 1e-5 (the
  order of the atomic adds differs), for every degree, with and without
  anisotropy, in batches; and the column kernel matches the oracle within the
  FP32 bound 1e-4.
- sesnt_tune keeps one of the variants that compute the step; the tuned
  handle's seismograms and wavefield equal the default handle's (FP32 to
  1e-5, FP64 to 1e-12); the choice is cached per GPU and grid and reused by
  SESNT_FLAG_AUTOTUNE; tuning after stepping is refused.
"""
import os

import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import rel_l2, run_oracle, small_workload, with_grid

pytestmark = pytest.mark.gpu


def run(wl, steps, variant=None, arg=0, piece=8192, tune=False):
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        report = sim.tune() if tune else None
        if variant is not None:
            sim.set_element_variant(variant, arg, piece)
        name, choice = sim.element_kernel()
        sim.run(1, steps)
        return sim.seismograms(), sim.field("vz", precision=8), name, choice, report


def batch_of(wl, batch):
    w = with_grid(wl, batch=batch)
    w.sources = []
    for s in range(batch):
        src = workloads.Source(**{**wl.sources[0].__dict__})
        src.sim, src.lat, src.lon = s, 34.0 + 0.7 * s, 3.5 + 1.1 * s
        w.sources.append(src)
    return w


@pytest.mark.parametrize("lpd", [2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("precision", [4, 8])
def test_column_kernel_matches_point_kernel(gpu, sesnt_lib, lpd, precision):
    tol = 1e-5 if precision == 4 else 1e-12
    for aniso, batch in ((False, 1), (True, 1), (False, 3), (True, 4)):
        wl = batch_of(with_grid(small_workload(lpd, aniso=aniso, nt=120), precision=precision), batch)
        sp, vp, name_p, _, _ = run(wl, 120, sesnt.ELEMENT_POINT)
        assert name_p == "k_element"
        for variant, kname in ((sesnt.ELEMENT_COLUMNS, "k_element_cols"),
                               (sesnt.ELEMENT_COLUMNS_STAGED, "k_element_cols (staged stress)")):
            for arg in ((0, 1, 2, 3, 5, 10, 15) if precision == 4 else (0, 6)):
                sc, vcol, name_c, choice, _ = run(wl, 120, variant, arg, piece=0 if arg % 2 else 4096)
                assert name_c == kname and choice[:2] == (variant, arg)
                e, ev = rel_l2(sc, sp), rel_l2(vcol, vp)
                print("lpd %d prec %d aniso %d batch %d %s arg %d: columns vs point seismograms %.2e, vz %.2e"
                      % (lpd, precision, aniso, batch, kname, arg, e, ev))
                assert np.abs(sp).max() > 0
                assert e < tol and ev < tol


@pytest.mark.parametrize("lpd", [2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("precision", [4, 8])
def test_paired_column_kernel_matches_point_kernel(gpu, sesnt_lib, lpd, precision):
    tol = 1e-5 if precision == 4 else 1e-12
    for aniso, batch in ((False, 2), (True, 4), (False, 6)):
        wl = batch_of(with_grid(small_workload(lpd, aniso=aniso, nt=120), precision=precision), batch)
        sp, vp, name_p, _, _ = run(wl, 120, sesnt.ELEMENT_POINT)
        assert name_p == "k_element"
        for arg in ((0, 1, 2, 3, 8, 9, 10) if precision == 4 else (0, 8)):
            sc, vcol, name_c, choice, _ = run(wl, 120, sesnt.ELEMENT_COLUMNS_PAIR, arg)
            assert name_c == "k_element_cols2" and choice[:2] == (sesnt.ELEMENT_COLUMNS_PAIR, arg)
            e = [rel_l2(sc[s], sp[s]) for s in range(batch)]
            ev = rel_l2(vcol, vp)
            print("lpd %d prec %d aniso %d batch %d arg %d: paired columns vs point seismograms %.2e, vz %.2e"
                  % (lpd, precision, aniso, batch, arg, max(e), ev))
            assert all(np.abs(sp[s]).max() > 0 for s in range(batch))
            assert max(e) < tol and ev < tol
    # an odd batch has no simulation pairs: the launch rules' kernel runs
    wl = batch_of(with_grid(small_workload(lpd, nt=20), precision=precision), 3)
    _, _, name, choice, _ = run(wl, 20, sesnt.ELEMENT_COLUMNS_PAIR, 0)
    assert name == "k_element" and choice[0] == sesnt.ELEMENT_COLUMNS_PAIR


@pytest.mark.parametrize("lpd", [4, 5, 6, 7])
def test_staged_kernel_wait_modes_agree(gpu, sesnt_lib, lpd):
    """The staged SLS kernel with the stage's wait polled by every thread or
    by one lane per warp, with and without the L2 prefetch of the state
    ahead, with bulk and register stores: the same step."""
    for precision in (4, 8):
        tol = 1e-5 if precision == 4 else 1e-12
        wl = batch_of(with_grid(small_workload(lpd, n_sls=3, nt=100), precision=precision), 2)
        base, vb, name_b, _, _ = run(wl, 100, sesnt.ELEMENT_STAGE, 0, 8192)
        assert name_b == "k_element_stage"
        for variant in (sesnt.ELEMENT_STAGE, sesnt.ELEMENT_STAGE_REG):
            for arg in (1, 2, 4, 7):
                s, v, _, choice, _ = run(wl, 100, variant, arg, 0)
                e, ev = rel_l2(s, base), rel_l2(v, vb)
                print("lpd %d prec %d variant %d arg %d: %.2e, vz %.2e" % (lpd, precision, variant, arg, e, ev))
                assert choice[:2] == (variant, arg) and e < tol and ev < tol


def test_lane_zero_stage_wait_runs_out_and_reports(gpu, sesnt_lib):
    """The one-lane-per-warp stage wait is bounded like the all-thread one."""
    wl = small_workload(4, n_sls=3, nt=40)
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        sim.set_element_variant(sesnt.ELEMENT_STAGE, 1, 0)
        sim.set_wait_limit(64, drop_completion=True)
        sim.run(1, 2)
        with pytest.raises(sesnt.SesntError) as e:
            sim.synchronize()
        assert e.value.code == sesnt.ETIMEOUT
        sim.set_wait_limit(1 << 22)
        sim.reset()
        sim.run(1, 40)
        again = sim.seismograms()
    fresh, _, _, _, _ = run(wl, 40, sesnt.ELEMENT_POINT)
    assert rel_l2(again, fresh) < 1e-5


def test_staged_column_wait_runs_out_and_reports(gpu, sesnt_lib):
    """The staged column kernel's one mbarrier wait per block is bounded:
    with its bulk load dropped the wait runs out, synchronising returns
    SESNT_ETIMEOUT, and after sesnt_reset the handle steps normally again."""
    wl = batch_of(small_workload(4, nt=40), 2)
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        sim.set_element_variant(sesnt.ELEMENT_COLUMNS_STAGED, 0, 0)
        sim.set_wait_limit(64, drop_completion=True)
        sim.run(1, 2)
        with pytest.raises(sesnt.SesntError) as e:
            sim.synchronize()
        assert e.value.code == sesnt.ETIMEOUT
        sim.set_wait_limit(1 << 22)
        sim.reset()
        sim.run(1, 40)
        again = sim.seismograms()
    fresh, _, _, _, _ = run(wl, 40, sesnt.ELEMENT_POINT)
    assert rel_l2(again, fresh) < 1e-5


def test_column_kernel_matches_oracle(gpu, sesnt_lib, oracle_mod):
    for lpd in (4, 6):
        wl = small_workload(lpd, nt=300)
        sc, _, _, _, _ = run(wl, 300, sesnt.ELEMENT_COLUMNS)
        so, _, _ = run_oracle(oracle_mod, wl, 300)
        e = rel_l2(sc[0], so)
        print("lpd %d columns vs oracle %.2e" % (lpd, e))
        assert e < 1e-4


@pytest.mark.parametrize("case", ["elastic_batch4", "sls_lpd4", "sls_lpd6", "sls_lpd5_fp64"])
def test_tuned_choice_computes_the_default_step(gpu, sesnt_lib, tmp_path, monkeypatch, case):
    monkeypatch.setenv("SESNT_TUNE_CACHE", str(tmp_path / "tune.txt"))
    if case == "elastic_batch4":
        wl = batch_of(small_workload(4, nt=150, nx=12, ny=12, nz=8), 4)
    elif case == "sls_lpd4":
        wl = small_workload(4, n_sls=3, nt=150, nx=12, ny=12, nz=8)
    elif case == "sls_lpd6":
        wl = small_workload(6, n_sls=3, nt=150)
    else:
        wl = with_grid(small_workload(5, n_sls=3, aniso=True, nt=150), precision=8)
    tol = 1e-12 if wl.grid.precision == 8 else 1e-5
    sd, vd, name_d, _, _ = run(wl, 150)
    st, vt, name_t, choice, report = run(wl, 150, tune=True)
    print(report)
    print("%s: default %s, tuned %s %s" % (case, name_d, name_t, choice))
    assert "chosen" in report and choice[0] != sesnt.ELEMENT_AUTO
    e, ev = rel_l2(st, sd), rel_l2(vt, vd)
    print("%s: tuned vs default seismograms %.2e, vz %.2e" % (case, e, ev))
    assert e < tol and ev < tol
    # the cache now holds the choice; an autotuned handle of the same grid reuses it
    lines = open(str(tmp_path / "tune.txt")).read().splitlines()
    assert len(lines) == 1
    g = with_grid(wl, flags=wl.grid.flags | sesnt.FLAG_AUTOTUNE).grid
    with sesnt.Simulation(g) as sim:
        workloads.setup(sim, workloads.Workload(wl.name, g, wl.model, wl.sources, wl.receivers))
        name_a, choice_a = sim.element_kernel()
    assert (name_a, choice_a) == (name_t, choice)
    assert len(open(str(tmp_path / "tune.txt")).read().splitlines()) == 1


def test_autotune_without_a_cache_entry_tunes_and_caches(gpu, sesnt_lib, tmp_path, monkeypatch):
    path = tmp_path / "fresh.txt"
    monkeypatch.setenv("SESNT_TUNE_CACHE", str(path))
    wl = small_workload(4, n_sls=3, nt=50)
    g = with_grid(wl, flags=sesnt.FLAG_AUTOTUNE).grid
    with sesnt.Simulation(g) as sim:
        workloads.setup(sim, workloads.Workload(wl.name, g, wl.model, wl.sources, wl.receivers))
        name, choice = sim.element_kernel()
        sim.run(1, 50)
        s = sim.seismograms()
    assert choice[0] != sesnt.ELEMENT_AUTO
    assert os.path.exists(path) and len(open(path).read().splitlines()) == 1
    sd, _, _, _, _ = run(wl, 50)
    assert rel_l2(s, sd) < 1e-5


def test_tuning_after_stepping_and_bad_variants_are_refused(gpu, sesnt_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("SESNT_TUNE_CACHE", str(tmp_path / "t.txt"))
    wl = small_workload(4, nt=20)
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        sim.run(1, 5)
        with pytest.raises(sesnt.SesntError) as ex:
            sim.tune()
        assert ex.value.code == sesnt.ESTATE
        sim.reset()
        sim.tune()  # after a reset the wavefield is zero again
        for bad in ((99, 0, 0), (sesnt.ELEMENT_COLUMNS, 16, 0), (sesnt.ELEMENT_STAGE, 8, 0),
                    (sesnt.ELEMENT_STAGE, 0, 100)):
            with pytest.raises(sesnt.SesntError) as ex:
                sim.set_element_variant(*bad)
            assert ex.value.code == sesnt.EINVAL
        # a variant the configuration lacks falls back to the launch rules
        sim.set_element_variant(sesnt.ELEMENT_STAGE)
        assert sim.element_kernel()[0] == "k_element"
