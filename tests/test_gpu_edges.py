"""Edge cases of the step through the C ABI: empty source and receiver sets,
the smallest grid the reference accepts, the shortest run, no taper, a
batch in which some simulations have no source, receivers added after
stepping, and sources on element faces. Each is compared with the oracle or
with an invariant that holds exactly."""
import copy

import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import TOL, rel_l2, run_gpu, run_oracle, small_workload, with_grid

pytestmark = pytest.mark.gpu


def test_no_sources_no_receivers(gpu, sesnt_lib):
    """A run without sources keeps the zero wavefield exactly; one without
    receivers runs and returns empty seismograms."""
    wl = small_workload(4, n_sls=3, nt=40)
    with sesnt.Simulation(wl.grid) as sim:
        m = wl.model
        sim.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
        sim.run(1, 40)
        assert sim.seismograms().size == 0
        for k in ("vx", "vz", "sxx", "syz"):
            assert not np.any(sim.field(k))
        assert sim.v_ptp(0) == (0.0, 0.0)


@pytest.mark.parametrize("lpd", [2, 7])
def test_smallest_grid_and_shortest_run(gpu, sesnt_lib, oracle_mod, lpd):
    """nx = ny = nz = 4 (the reference's minimum), taper width 1, nt = 2:
    step 1 injects nothing (the source slab acts from step 2)."""
    wl = small_workload(lpd, nt=2, nx=4, ny=4, nz=4)
    got, gf, _ = run_gpu(with_grid(wl, precision=8), 2)
    want, of, o = run_oracle(oracle_mod, wl, 2, precision=8)
    o.close()
    assert not np.any(got[0][:, :, 0])  # step 1: zero
    assert np.abs(gf["vz"]).max() > 0
    for k in gf:  # FP64 step, fields read back as float32
        assert rel_l2(gf[k], of[k]) < 1e-6, k


def test_no_taper(gpu, sesnt_lib, oracle_mod):
    wl = with_grid(small_workload(4, nt=120), taper_width=0)
    got, gf, _ = run_gpu(wl, 120)
    want, of, o = run_oracle(oracle_mod, wl, 120)
    o.close()
    assert rel_l2(got[0], want) < TOL
    assert rel_l2(gf["vz"], of["vz"]) < TOL


@pytest.mark.parametrize("batch", [3, 4])
def test_batch_with_idle_simulations(gpu, sesnt_lib, batch):
    """Only simulation 1 has a source: the others stay exactly zero, and
    simulation 1 equals the same source run alone (odd batch: one
    simulation per thread; even batch: the paired kernel)."""
    wl = small_workload(4, nt=100)
    g = copy.copy(wl.grid)
    g.batch = batch
    src = copy.copy(wl.sources[0])
    src.sim = 1
    bw = workloads.Workload("idle", g, wl.model, [src], wl.receivers)
    seis, _, _ = run_gpu(bw, 100, fields=())
    for s in range(batch):
        if s != 1:
            assert not np.any(seis[s])
    alone, _, _ = run_gpu(wl, 100, fields=())
    assert np.abs(seis[1]).max() > 0
    assert rel_l2(seis[1], alone[0]) < 1e-5


def test_receivers_added_after_stepping(gpu, sesnt_lib):
    """A receiver added after 30 steps records from step 31 on; the earlier
    receivers keep their first 30 samples."""
    wl = small_workload(4, nt=80)
    full, _, _ = run_gpu(wl, 80, fields=())
    first, later = wl.receivers[:3], wl.receivers[3:]
    with sesnt.Simulation(wl.grid) as sim:
        m = wl.model
        sim.set_model(m["rhoinv"], m["lambda"], m["mu"])
        s = wl.sources[0]
        elem, vm = sesnt.locate_point(wl.grid, s.lat, s.lon, s.depth)
        sim.add_source(0, elem, vm, s.kind, np.asarray(s.comp, np.float32),
                       sesnt.source_signature(s.wavelet, s.onset, s.width, wl.grid.dt, wl.grid.nt))
        for r in first:
            sim.add_receiver(*sesnt.locate_point(wl.grid, r.lat, r.lon, r.depth))
        sim.run(1, 30)
        for r in later:
            sim.add_receiver(*sesnt.locate_point(wl.grid, r.lat, r.lon, r.depth))
        sim.run(31, 50)
        got = sim.seismograms()[0]
    # two FP32 runs: equal up to the order of the atomic adds
    assert rel_l2(got[:3], full[0][:3]) < TOL
    assert not np.any(got[3:, :, :30])
    assert rel_l2(got[3:, :, 30:], full[0][3:, :, 30:]) < TOL


def test_source_on_element_faces(gpu, sesnt_lib, oracle_mod):
    """A source exactly on an element corner (shared by eight elements) is
    located as the reference locates it and injected identically."""
    wl = small_workload(4, nt=150)
    g = wl.grid
    # element corner: colatitude and longitude on the element grid, depth at an element boundary
    dlat = (g.lat_max - g.lat_min) / g.nx
    dlon = (g.lon_max - g.lon_min) / g.ny
    drad = (g.rad_max - g.rad_min) / g.nz
    src = copy.copy(wl.sources[0])
    src.lat, src.lon, src.depth = g.lat_max - 3 * dlat, g.lon_min + 3 * dlon, 2 * drad
    w = workloads.Workload("corner", g, wl.model, [src], wl.receivers)
    got, _, _ = run_gpu(w, 150, fields=())
    want, _, o = run_oracle(oracle_mod, w, 150)
    o.close()
    assert np.abs(want).max() > 0
    assert rel_l2(got[0], want) < TOL
