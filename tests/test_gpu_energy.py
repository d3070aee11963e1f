"""Kinetic energy (sesnt_kinetic_energy) against the oracle's restatement of
the reference's kinetic_energy (src/elastic_vars.F90:218-246), and the energy
of the config-1 run staying bounded once its source has stopped.

Tolerances: FP64 GPU equals the FP64 oracle to 1e-10 relative (the sums run
in a different order: unique points against element-local copies); FP32
wavefields within 1e-5 of the FP64 oracle's energy (the energy is quadratic
in v, whose FP32 error is a few 1e-7 on these runs); the FP32 oracle itself
sums millions of float32 terms, so against it the bound is 1e-4.
"""
import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import small_workload, with_grid

pytestmark = pytest.mark.gpu


def gpu_energies(wl, steps, every):
    out = []
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        assert sim.kinetic_energy() == 0.0  # zero wavefield after set_model
        it = 1
        while it <= steps:
            sim.run(it, every)
            it += every
            out.append([sim.kinetic_energy(s) for s in range(wl.grid.batch)])
    return np.array(out)


def oracle_energies(oracle_mod, wl, steps, every, precision, sim=0):
    o = oracle_mod.Oracle(wl.grid, precision)
    oracle_mod.load_workload(o, wl, sim=sim)
    out = []
    for _ in range(steps // every):
        o.run(every)
        out.append(o.kinetic_energy())
    o.close()
    return np.array(out)


@pytest.mark.parametrize("n_sls,lpd", [(0, 4), (3, 4), (3, 6)])
def test_kinetic_energy_matches_oracle(gpu, sesnt_lib, oracle_mod, n_sls, lpd):
    wl = small_workload(lpd, n_sls=n_sls, nt=200)
    e64 = gpu_energies(with_grid(wl, precision=8), 200, 40)[:, 0]
    e32 = gpu_energies(wl, 200, 40)[:, 0]
    o64 = oracle_energies(oracle_mod, wl, 200, 40, 8)
    o32 = oracle_energies(oracle_mod, wl, 200, 40, 4)
    assert o64.max() > 0
    r64 = np.abs(e64 - o64) / o64.max()
    r32 = np.abs(e32 - o64) / o64.max()
    ro = np.abs(e32 - o32) / o64.max()
    print("kinetic energy lpd %d n_sls %d: FP64 GPU vs FP64 oracle %.2e, FP32 GPU vs FP64 oracle %.2e, "
          "vs FP32 oracle %.2e" % (lpd, n_sls, r64.max(), r32.max(), ro.max()))
    assert r64.max() < 1e-10
    assert r32.max() < 1e-5
    assert ro.max() < 1e-4


def test_kinetic_energy_of_a_batch(gpu, sesnt_lib):
    """Each simulation of a batch has its own energy; a simulation without a
    source stays at exactly zero."""
    wl = small_workload(4, n_sls=3, nt=80)
    g = with_grid(wl, batch=3).grid
    src = [workloads.Source(lat=s.lat, lon=s.lon, depth=s.depth, kind=s.kind, comp=s.comp, width=s.width,
                            onset=s.onset, sim=q) for q, s in ((0, wl.sources[0]), (2, wl.sources[0]))]
    b = workloads.Workload("batch3", g, wl.model, src, wl.receivers)
    e = gpu_energies(b, 80, 40)
    one = gpu_energies(wl, 80, 40)[:, 0]
    assert np.all(e[:, 1] == 0.0)
    assert np.allclose(e[:, 0], one, rtol=1e-5, atol=0) and np.allclose(e[:, 2], one, rtol=1e-5, atol=0)


def test_kinetic_energy_config1_is_bounded(gpu, sesnt_lib, oracle_mod):
    """Config 1 (homogeneous elastic 12x12x8, lpd 4, 2000 steps): the source
    wavelet is over by about step 720, after which the absorbing taper only
    removes energy. Sampled every 50 steps, the kinetic energy (which swaps
    with the potential energy within a period) falls by windows, ends more
    than 100x below its peak, and follows the FP64 oracle's curve."""
    wl = workloads.config1(nt=2000)
    e = gpu_energies(wl, 2000, 50)[:, 0]
    o = oracle_energies(oracle_mod, wl, 2000, 50, 8)
    assert np.all(np.isfinite(e))
    peak = e.max()
    rel = np.abs(e - o) / o.max()
    print("config1 kinetic energy: peak %.4e J at step %d, final/peak %.2e, FP32 GPU vs FP64 oracle %.2e"
          % (peak, 50 * (int(np.argmax(e)) + 1), e[-1] / peak, rel.max()))
    assert rel.max() < 1e-4
    late = e[16:]  # steps 850 .. 2000
    assert late.max() < peak
    windows = [late[q:q + 8].mean() for q in range(0, len(late) - 7, 8)]
    assert all(b < a for a, b in zip(windows, windows[1:])), windows
    assert e[-1] < 1e-2 * peak
