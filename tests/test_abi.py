"""The C ABI library loads, exports every function include/sesnt.h declares,
and its host-only entry points (no GPU needed) agree bit for bit with the
oracle's restatement of the reference."""
import ctypes as C

import numpy as np
import pytest


def test_exports_every_declared_symbol(sesnt_lib):
    import sesnt
    names = sesnt.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(sesnt_lib, n)]
    assert not missing, missing


def test_locate_point_matches_oracle(sesnt_lib, oracle_mod):
    import sesnt
    import workloads
    rng = np.random.default_rng(11)
    for wl in (workloads.config1(nt=4), workloads.config2(nt=4, nx=12, ny=12, nz=8, n_sls=0)):
        g = wl.grid
        pts = [(p.lat, p.lon, p.depth) for p in wl.sources + wl.receivers]
        # element faces and corners (points of the float32 lattice) and random points
        for a in range(0, g.nx + 1, 3):
            for b in range(0, g.ny + 1, 4):
                pts.append((g.lat_min + (g.lat_max - g.lat_min) * a / g.nx,
                            g.lon_min + (g.lon_max - g.lon_min) * b / g.ny, 75000.0 * (a % 3)))
        pts += [(float(rng.uniform(g.lat_min, g.lat_max)), float(rng.uniform(g.lon_min, g.lon_max)),
                 float(rng.uniform(0, g.rad_max - g.rad_min))) for _ in range(300)]
        hits = 0
        for lat, lon, dep in pts:
            e_ref, v_ref = oracle_mod.locate(g, np.float32(lat), np.float32(lon), np.float32(dep))
            try:
                e, v = sesnt.locate_point(g, lat, lon, dep)
            except sesnt.SesntError as err:
                assert e_ref is None or not (0 <= e_ref[0] < g.nx and 0 <= e_ref[1] < g.ny and 0 <= e_ref[2] < g.nz), (lat, lon, dep, err)
                continue
            assert e == e_ref, (lat, lon, dep)
            assert np.array_equal(v, v_ref), (lat, lon, dep)
            hits += 1
        assert hits > 200


@pytest.mark.parametrize("wavelet", ["DELTA", "RICKER", "GAUSS", "SIN**3", "BRUNE"])
def test_source_signature_matches_oracle(sesnt_lib, oracle_mod, wavelet):
    import sesnt
    code = sesnt.WAVELETS[wavelet]
    for onset, width, dt, nt in [(90.0, 60.0, 0.25, 2000), (7.5, 3.0, 0.125, 400)]:
        a = sesnt.source_signature(wavelet, onset, width, dt, nt)
        b = oracle_mod.stf(code, onset, width, dt, nt)
        assert np.array_equal(a, b)
    assert np.abs(sesnt.source_signature("RICKER", 90.0, 60.0, 0.25, 2000)).max() > 0.9


def test_invalid_arguments_are_rejected(sesnt_lib):
    import sesnt
    g = sesnt.Grid(nx=3, ny=12, nz=8, lpd=4, lat_min=30, lat_max=50, lon_min=0, lon_max=20,
                   rad_min=5771000.0, rad_max=6371000.0, dt=0.25, nt=100)
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.Simulation(g)
    assert e.value.code == sesnt.EINVAL and "at least 4" in str(e.value)
    g.nx = 12
    g.lpd = 9
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.Simulation(g)
    assert e.value.code == sesnt.EUNSUPPORTED
    g.lpd = 4
    g.taper_width = 6
    with pytest.raises(sesnt.SesntError):
        sesnt.Simulation(g)
    g.taper_width = 3
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.locate_point(g, 10.0, 10.0, 0.0)  # latitude outside the section
    assert e.value.code == sesnt.ENOTFOUND
    with pytest.raises(sesnt.SesntError) as e:
        sesnt.locate_point(g, 95.0, 10.0, 0.0)
    assert e.value.code == sesnt.EINVAL


def test_footprint_and_algorithmic_bytes(sesnt_lib):
    import sesnt
    import workloads
    g = workloads.config2(nt=10, nx=12, ny=12, nz=8).grid
    fp = sesnt.footprint_bytes(g)
    # sigma + 18 memory variables + lambda, mu, tau per local point, 7 per unique point
    assert fp > g.n_loc * 4 * 27
    assert fp < g.n_loc * 4 * 40 + g.n_uni * 4 * 10 + (2 << 20)


def test_binding_constants_match_the_header():
    """Every value #defined in include/sesnt.h (error codes, flags, source
    kinds, wavelets, receiver channel bits, field ids) equals the Python
    binding's constant of the same name; every flag and channel bit has one."""
    import re

    import sesnt
    defines = {}
    for line in open(sesnt.HEADER):
        m = re.match(r"#define\s+SESNT_([A-Z0-9_]+)\s+\(?(-?\d+)u?\)?", line)
        if m:
            defines[m.group(1)] = int(m.group(2))
    assert defines["FLAG_NO_STAGE"] == 256 and defines["ENONFINITE"] == -9
    for name, value in defines.items():
        if name.startswith("FIELD_"):
            key = name[len("FIELD_"):].lower()
            if key == "memory":
                assert sesnt.MEMORY_FIELD0 == value
            else:
                assert sesnt.FIELDS[key] == value, name
        elif name.startswith("WAVELET_"):
            key = name[len("WAVELET_"):]
            assert sesnt.WAVELETS["SIN**3" if key == "SIN3" else key] == value, name
        else:
            assert getattr(sesnt, name) == value, name
    for prefix in ("FLAG_", "CH_"):
        assert {n for n in dir(sesnt) if n.startswith(prefix)} == {n for n in defines if n.startswith(prefix)}
