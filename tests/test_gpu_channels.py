"""Receiver channels beyond the velocity and volume-snapshot fields, against
the oracle (the reference's channel classes and get_field restated):

- rot_vx/rot_vy/rot_vz and n receiver channels, recorded source-field
  channels mxx..mzz / fx..fz;
- pressure, strain (displacement gradient, SESNT_FLAG_STRAIN) and rotation
  fields;
- snapshots written behind the steps to <prefix><attribute>_<it>.vol.

Tolerances: FP64 fields against the FP64 oracle 1e-9 relative L2 (same
algorithm, different summation order); FP64 traces within float32 rounding
(1e-6: traces are returned as float32, like the reference's REAL32 channel
data); FP32 against the FP32 oracle 1e-4 relative to the field's (or
trace's) norm; snapshot files (float32) against the FP64 oracle 1e-6.
"""
import os

import numpy as np
import pytest

import sesnt
import workloads
from test_gpu_parity import rel_l2, small_workload, with_grid

ROT = sesnt.CH_ROT_VX | sesnt.CH_ROT_VY | sesnt.CH_ROT_VZ
MOMENT = (sesnt.CH_MXX | sesnt.CH_MXY | sesnt.CH_MXZ | sesnt.CH_MYY | sesnt.CH_MYZ | sesnt.CH_MZZ)
FORCE = sesnt.CH_FX | sesnt.CH_FY | sesnt.CH_FZ


def test_field_names(sesnt_lib):
    L = sesnt.lib()
    for name, code in sesnt.FIELDS.items():
        if name == "mass":
            continue
        assert L.sesnt_field_id(name.encode()) == code
        assert L.sesnt_field_name(code).decode() == name
    assert L.sesnt_field_id(b" ROT_VZ ") == sesnt.FIELDS["rot_vz"]
    assert L.sesnt_field_id(b"grad_rho") == -1 and L.sesnt_field_name(99) is None


def channel_workload(kind=sesnt.SOURCE_MT, n_sls=0, nt=200):
    """Small section; receiver 0 shares the source's element (records the
    source fields), the others sit elsewhere."""
    wl = small_workload(4, n_sls=n_sls, kind=kind, nt=nt)
    src = wl.sources[0]
    wl.receivers.insert(0, workloads.Receiver(lat=src.lat + 0.05, lon=src.lon - 0.05, depth=src.depth))
    return wl


def masks_for(wl, extra):
    return [sesnt.CH_VX | sesnt.CH_VY | sesnt.CH_VZ | extra for _ in wl.receivers]


def gpu_traces(wl, masks, nsteps, fields=(), flags=0):
    g = with_grid(wl, flags=wl.grid.flags | flags)
    out, f = {}, {}
    with sesnt.Simulation(g.grid) as sim:
        m = wl.model
        sim.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
        for s in wl.sources:
            elem, vm = sesnt.locate_point(g.grid, s.lat, s.lon, s.depth)
            stf = sesnt.source_signature(s.wavelet, s.onset, s.width, g.grid.dt, g.grid.nt)
            sim.add_source(s.sim, elem, vm, s.kind, np.asarray(s.comp, np.float32), stf)
        for r, mask in zip(wl.receivers, masks):
            elem, vm = sesnt.locate_point(g.grid, r.lat, r.lon, r.depth)
            sim.add_receiver(elem, vm, mask)
        sim.run(1, nsteps)
        for q, mask in enumerate(masks):
            for b in range(16):
                if mask >> b & 1:
                    out[(q, 1 << b)] = sim.trace(q, 1 << b).astype(np.float64)
        for k in fields:
            f[k] = sim.field(k, precision=8)
    return out, f


def oracle_traces(oracle_mod, wl, masks, nsteps, precision, fields=(), strain=False):
    o = oracle_mod.Oracle(wl.grid, precision)
    if strain:
        o.keep_strain()
    oracle_mod.load_workload(o, wl, masks=masks)
    o.run(nsteps)
    out = {}
    for q, mask in enumerate(masks):
        for b in range(16):
            if mask >> b & 1:
                out[(q, 1 << b)] = o.trace(q, 1 << b).astype(np.float64)
    f = {k: o.field(sesnt.FIELDS[k]).astype(np.float64) for k in fields}
    o.close()
    return out, f


def compare_traces(got, want, tol):
    """Each trace relative to its own norm; all-zero traces must be zero."""
    worst = {}
    for key, w in want.items():
        g = got[key]
        scale = np.linalg.norm(w)
        if scale == 0.0:
            assert np.abs(g).max() == 0.0, key
            continue
        err = np.linalg.norm(g - w) / scale
        worst[key[1]] = max(worst.get(key[1], 0.0), err)
        assert err < tol, (key, err)
    print("worst relative L2 per channel:", {k: "%.1e" % v for k, v in sorted(worst.items())})


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(8, 1e-6), (4, 1e-4)])
def test_rotation_and_n_channels(gpu, sesnt_lib, oracle_mod, precision, tol):
    wl = with_grid(channel_workload(n_sls=3), precision=precision)
    masks = masks_for(wl, ROT | sesnt.CH_N)
    got, _ = gpu_traces(wl, masks, 200)
    want, _ = oracle_traces(oracle_mod, wl, masks, 200, precision)
    assert np.abs(want[(1, sesnt.CH_ROT_VZ)]).max() > 0
    compare_traces(got, want, tol)
    # n is -vx
    for q in range(len(masks)):
        assert np.array_equal(got[(q, sesnt.CH_N)], -got[(q, sesnt.CH_VX)])


@pytest.mark.gpu
@pytest.mark.parametrize("kind,bits", [(sesnt.SOURCE_MT, MOMENT), (sesnt.SOURCE_SF, FORCE)])
def test_recorded_source_channels(gpu, sesnt_lib, oracle_mod, kind, bits):
    wl = with_grid(channel_workload(kind=kind), precision=8)
    masks = masks_for(wl, bits)
    got, _ = gpu_traces(wl, masks, 120)
    want, _ = oracle_traces(oracle_mod, wl, masks, 120, 8)
    # receiver 0 is in the source element and sees the slab; the others see zero
    assert max(np.abs(want[(0, b)]).max() for b in (1 << q for q in range(16)) if bits & b) > 0
    compare_traces(got, want, 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(8, 1e-9), (4, 1e-4)])
def test_snapshot_fields(gpu, sesnt_lib, oracle_mod, precision, tol):
    wl = with_grid(channel_workload(n_sls=3), precision=precision)
    masks = masks_for(wl, 0)
    names = ("pressure", "exx", "exy", "exz", "eyy", "eyz", "ezz", "rot_vx", "rot_vy", "rot_vz", "lambda", "mu")
    _, got = gpu_traces(wl, masks, 150, fields=names, flags=sesnt.FLAG_STRAIN | sesnt.FLAG_ROTATION)
    _, want = oracle_traces(oracle_mod, wl, masks, 150, precision, fields=names, strain=True)
    for k in names:
        assert np.abs(want[k]).max() > 0, k
        assert rel_l2(got[k], want[k]) < tol, (k, rel_l2(got[k], want[k]))


@pytest.mark.gpu
def test_strain_and_rotation_need_their_flags(gpu, sesnt_lib):
    wl = channel_workload(nt=10)
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        sim.run(1, 3)
        for name in ("exx", "rot_vz"):
            with pytest.raises(sesnt.SesntError) as e:
                sim.field(name)
            assert e.value.code == sesnt.ESTATE
        with pytest.raises(sesnt.SesntError):
            sim.add_snapshot("exx", 1, 1)
        with pytest.raises(sesnt.SesntError) as e:
            sim.trace(0, sesnt.CH_ROT_VX)  # not requested
        assert e.value.code == sesnt.EINVAL


@pytest.mark.gpu
def test_snapshots_written_behind_the_steps(gpu, sesnt_lib, oracle_mod, tmp_path):
    """Snapshots every 40 steps from step 20 to 180 through the graph path
    (runs of 32 steps are replayed): vx, pressure, rotation (computed on the
    due steps only) and strain, compared with the FP64 oracle at each step."""
    wl = with_grid(channel_workload(n_sls=3, nt=200), precision=8, flags=sesnt.FLAG_STRAIN)
    prefix = str(tmp_path) + "/"
    names = ("vx", "pressure", "rot_vz", "exy")
    steps = list(range(20, 181, 40))
    with sesnt.Simulation(wl.grid) as sim:
        workloads.setup(sim, wl)
        for k in names:
            sim.add_snapshot(k, 20, 40, 180, prefix=prefix)
        with pytest.raises(sesnt.SesntError) as e:
            sim.add_snapshot("vx", 0, 10)
        assert e.value.code == sesnt.ERANGE
        with pytest.raises(sesnt.SesntError):
            sim.add_snapshot("vx", 10, 0)
        with pytest.raises(sesnt.SesntError):
            sim.add_snapshot("vx", 50, 10, 40)
        sim.run(1, 200)
        sim.wait_snapshots()
    files = sorted(os.listdir(tmp_path))
    assert files == sorted("%s_%d.vol" % (k, it) for k in names for it in steps)
    o = oracle_mod.Oracle(wl.grid, 8)
    o.keep_strain()
    oracle_mod.load_workload(o, wl)
    done = 0
    for it in steps:
        o.run(it - done)
        done = it
        for k in names:
            got = sesnt.read_raw_field(os.path.join(prefix, "%s_%d.vol" % (k, it)), wl.grid).astype(np.float64)
            want = o.field(sesnt.FIELDS[k]).astype(np.float64)
            assert rel_l2(got, want) < 1e-6, (k, it, rel_l2(got, want))
    o.close()


@pytest.mark.gpu
def test_snapshot_override(gpu, sesnt_lib, tmp_path):
    wl = channel_workload(nt=20)
    prefix = str(tmp_path) + "/"
    for override, ok in ((False, True), (False, False), (True, True)):
        with sesnt.Simulation(wl.grid) as sim:
            workloads.setup(sim, wl)
            sim.add_snapshot("vz", 5, 5, prefix=prefix, override=override)
            sim.run(1, 20)
            if ok:
                sim.wait_snapshots()
            else:
                with pytest.raises(sesnt.SesntError):
                    sim.wait_snapshots()
    assert sorted(os.listdir(tmp_path)) == ["vz_10.vol", "vz_15.vol", "vz_20.vol", "vz_5.vol"]
