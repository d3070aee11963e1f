"""The request server: requests of different grids, degrees, step counts and
source counts submitted at once under a device budget that forces queueing
and source splitting. Each result must be the same as the request run alone,
in the mix, within the stated tolerance."""
import copy

import numpy as np
import pytest

import sesnt
import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-5  # same kernels, same inputs: only the order of the atomic adds differs


def alone(wl):
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        sim.run(1, wl.grid.nt)
        return sim.seismograms()


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_results_are_the_same_alone_and_in_the_mix(gpu, sesnt_lib):
    stream = workloads.served_stream(8, seed=11, lateral=(6, 10), radial=(4, 6), steps=(60, 160), sources=(1, 3),
                                     receivers=8)
    budget = 2 * max(sesnt.footprint_bytes(w.grid) for w in stream)  # about two requests at a time
    with sesnt.Server(device_bytes=budget, max_active=3, chunk_steps=16, max_batch=2) as srv:
        ids = [srv.submit(workloads.request_of(w)) for w in stream]
        for rid in ids:
            assert srv.wait(rid, 300.0) == sesnt.OK
        st = srv.stats()
        assert st["completed"] == len(stream) and st["failed"] == 0
        assert 0 < st["latency_p50"] <= st["latency_p99"] <= st["latency_max"]
        assert st["updates_per_second"] > 0 and st["device_bytes_used"] == 0
        for w, rid in zip(stream, ids):
            got, latency, wait = srv.result(rid)
            assert latency >= wait >= 0
            want = alone(w)
            assert np.abs(want).max() > 0
            assert rel(got, want) < TOL, w.name
            srv.release(rid)


def test_cancel_and_oversized_requests(gpu, sesnt_lib):
    stream = workloads.served_stream(3, seed=5, lateral=(6, 8), radial=(4, 5), steps=(400, 500), sources=(1, 1),
                                     receivers=4)
    one = max(sesnt.footprint_bytes(w.grid) for w in stream)
    with sesnt.Server(device_bytes=int(1.2 * one), max_active=1, chunk_steps=8) as srv:
        ids = [srv.submit(workloads.request_of(w)) for w in stream]
        # the last request is still queued behind the first: it can be cancelled
        assert srv.cancel(ids[-1]) == sesnt.OK
        assert srv.wait(ids[0], 300.0) == sesnt.OK
        assert srv.wait(ids[-1], 1.0) != sesnt.OK  # cancelled requests report failure
        big = copy.copy(stream[0])
        big.grid = copy.copy(stream[0].grid)
        big.grid.nx, big.grid.ny, big.grid.nz = 40, 40, 20
        big.model = workloads.homogeneous_model(big.grid)
        big.sources = big.sources[:1]
        with pytest.raises(sesnt.SesntError) as e:
            srv.submit(workloads.request_of(big))
        assert e.value.code == sesnt.ENOMEM
        assert srv.wait(ids[1], 300.0) == sesnt.OK
