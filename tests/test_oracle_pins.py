"""Pins the oracle (and the library's host-side set-up) to the reference.

The reference's own tests for this path are the serial unit programs under
src/examples/ (gll_test.f90, coordinates_test.f90, interpolation_test.f90);
each is restated here against the oracle. The GLL points and weights are
further checked against independently computed Gauss-Lobatto-Legendre nodes,
and the committed golden fixture (tests/golden/, made by
tests/golden/make_golden.py) freezes the oracle's config-1 output. The GLL
knots and the point coordinates are also checked against output of the
reference's own Python package (ses3dpy), made by
tests/golden/make_ses3dpy_golden.py.
"""
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_gll_sizes(oracle_mod):
    # src/examples/gll_test.f90:20-33: sizes of get_knots/get_weights for lpd -2..10
    L = oracle_mod.lib()
    got = [L.oracle_gll_size(i) for i in range(-2, 11)]
    want = [0, 0] + [(i + 1) * 1000 + (i + 1) for i in range(0, 11)]
    assert got == want


@pytest.mark.parametrize("lpd", range(1, 8))
def test_gll_points_known_answers(oracle_mod, lpd):
    k, w, d = oracle_mod.gll(lpd, precision=8)
    # GLL nodes are -1, 1 and the roots of P'_N; weights 2/(N(N+1) P_N(x)^2)
    c = np.zeros(lpd + 1)
    c[-1] = 1.0
    P = np.polynomial.legendre.Legendre(c)
    ref = np.concatenate([[-1.0], np.sort(P.deriv().roots().real), [1.0]]) if lpd > 1 else np.array([-1.0, 1.0])
    assert np.allclose(k, ref, rtol=0, atol=2e-15 if lpd < 7 else 1e-15 + 1e-15 * 10)
    wref = 2.0 / (lpd * (lpd + 1) * P(ref) ** 2)
    if lpd == 1:
        # the reference tabulates placeholder weights for lpd 1
        # (src/gll_mod.f90:63-67, "@todo check if those dummy values work")
        assert np.array_equal(w, [0.5, 0.5])
    else:
        assert np.allclose(w, wref, rtol=1e-14, atol=1e-15)
        assert abs(w.sum() - 2.0) < 1e-13
    # derivative matrix: sum over the basis at any point is d/dx 1 = 0, and
    # it differentiates x exactly
    assert np.allclose(d.sum(axis=0), 0.0, atol=1e-12)
    assert np.allclose(k @ d, 1.0, atol=1e-12)


def test_knots_and_coordinates_match_ses3dpy(oracle_mod):
    """GLL knots and 1-D point coordinates against the reference's own Python
    package: tests/golden/ses3dpy_geometry.json, made by
    tests/golden/make_ses3dpy_golden.py with ses3dpy.get_knots and
    ses3dpy.generate_coordinates. generate_coordinates leaves out the first
    point of every element (the shared ones, and the very first) and works in
    float64 from the config's degrees and metres; the oracle's construction is
    float32, as the reference's Fortran."""
    import json
    with open(os.path.join(GOLDEN, "ses3dpy_geometry.json")) as f:
        d = json.load(f)
    assert sorted(d["knots"]) == [str(n) for n in range(2, 8)]
    for lpd, knots in d["knots"].items():
        k, _, _ = oracle_mod.gll(int(lpd), precision=8)
        assert np.allclose(k, knots, rtol=0, atol=1e-15), lpd
        # the float32 tables fold the closed forms in float32 (a few roundings,
        # pinned exactly by test_gll_float32_matches_float32_closed_forms)
        k32, _, _ = oracle_mod.gll(int(lpd), precision=4)
        assert np.allclose(k32, knots, rtol=0, atol=2.5e-7), lpd
    assert d["configs"]
    for name, c in d["configs"].items():
        for axis, key in enumerate(("theta", "phi", "r")):
            n = c["nX_global"][axis]
            x = oracle_mod.coordinates_1d(n, c["lpd"], c["minX"][axis], c["maxX"][axis])
            want = np.asarray(c[key])
            assert want.size == n * c["lpd"], (name, key)
            assert np.allclose(x[:, 1:].ravel(), want, rtol=2e-7, atol=0), (name, key)


@pytest.mark.parametrize("lpd", range(1, 8))
def test_gll_float32_matches_float32_closed_forms(oracle_mod, lpd):
    """The float32 tables are the closed forms of src/gll_mod.f90 folded in
    float32 (each operation rounded once)."""
    k, w, _ = oracle_mod.gll(lpd, precision=4)
    f = np.float32
    sq = lambda x: np.sqrt(f(x), dtype=f)
    if lpd == 4:
        a = sq(f(3) / f(7))
        assert np.array_equal(k, np.array([-1, -a, 0, a, 1], f))
        assert np.array_equal(w, np.array([f(1) / f(10), f(49) / f(90), f(32) / f(45), f(49) / f(90), f(1) / f(10)], f))
    if lpd == 6:
        r15, r33 = sq(15), sq(33)
        a = np.sqrt(f(2) * r15 + f(15), dtype=f) / r33
        b = np.sqrt(f(15) - f(2) * r15, dtype=f) / r33
        assert np.array_equal(k, np.array([-1, -a, -b, 0, b, a, 1], f))
    assert k[0] == -1 and k[-1] == 1


def test_coordinates_bounds_exact(oracle_mod):
    # src/examples/coordinates_test.f90:29-40
    c_min, c_max = np.float32(-1.234136), np.float32(14.237239)
    for elms in range(1, 14, 3):
        for lpd in range(1, 8):
            c = oracle_mod.coordinates_1d(elms, lpd, c_min, c_max)
            assert c[0, 0] == c_min and c[elms - 1, lpd] == c_max


def test_coordinates_integer_boundaries(oracle_mod):
    # src/examples/coordinates_test.f90:43-54
    for elms in range(1, 51, 7):
        for lpd in range(1, 8):
            c = oracle_mod.coordinates_1d(elms, lpd, np.float32(0.0), np.float32(elms))
            packed = np.concatenate([c[:, 0], [c[-1, -1]]])
            assert np.array_equal(packed, np.arange(elms + 1, dtype=np.float32))


def test_coordinates_connect_bit_exactly(oracle_mod):
    # src/examples/coordinates_test.f90:56-65: coords(i,lpd+1) == coords(i+1,1)
    for elms in range(1, 236, 43):
        for lpd in range(1, 8):
            c = oracle_mod.coordinates_1d(elms, lpd, np.float32(-1.1), np.float32(1.3))
            assert np.array_equal(c[:-1, lpd], c[1:, 0])


def _interp(oracle_mod, knots, f, x):
    return np.array([np.dot(oracle_mod.lagrange(xi, knots), f) for xi in x], np.float64)


def test_interpolation(oracle_mod):
    """src/examples/interpolation_test.f90:24-96 with seeded perturbations.
    The reference compares linear and sin interpolants against the constant 1
    (a check that always passes); here each is compared with its own function."""
    rng = np.random.default_rng(7)
    f32 = np.float32
    knots = np.array([-1, 0, 1], f32)
    x = np.arange(-50, 51, dtype=f32)
    x[1:-1] += rng.random(x.size - 2, dtype=f32) - f32(0.5)
    x /= np.abs(x).max()
    assert np.all(np.abs(_interp(oracle_mod, knots, np.ones(3, f32), x) - 1.0) < 0.01)
    knots = np.array([-1, 1], f32)
    x = np.arange(-3, 4, dtype=f32)
    x[1:-1] += rng.random(x.size - 2, dtype=f32) - f32(0.5)
    x /= np.abs(x).max()
    assert np.all(np.abs(_interp(oracle_mod, knots, knots, x) - x) < 0.01)
    n = 10
    knots = (np.arange(-n // 2, n // 2 + 1, dtype=f32) / f32(n // 2) * f32(math.pi)).astype(f32)
    x = np.arange(-24, 25, dtype=f32)
    x[1:-1] += rng.random(x.size - 2, dtype=f32) - f32(0.5)
    x = (x / np.abs(x).max() * f32(math.pi)).astype(f32)
    assert np.all(np.abs(_interp(oracle_mod, knots, np.sin(knots), x) - np.sin(x)) < 0.01)
    # exact at the knots (l_j(x_i) = delta_ij)
    for i, xi in enumerate(knots):
        l = oracle_mod.lagrange(xi, knots)
        assert l[i] == 1.0 and np.count_nonzero(l) == 1


def test_assembly_is_unique_point_sum(oracle_mod):
    """communicate_local_boundaries (src/communicate_fields.F90:48-79) on one
    rank equals summing all copies of each unique GLL point and writing the
    sum back: the unique numbering gx = ex*lpd + i used by the GPU library is
    the reference's assembly map. Integer data make the check bit-exact."""
    import workloads
    from sesnt import Grid
    for (nx, ny, nz, lpd) in [(4, 5, 4, 2), (5, 4, 6, 4), (4, 4, 4, 6)]:
        g = Grid(nx=nx, ny=ny, nz=nz, lpd=lpd, lat_min=0, lat_max=10, lon_min=0, lon_max=10,
                 rad_min=5e6, rad_max=6e6, dt=0.1, nt=10, taper_width=1)
        rng = np.random.default_rng(nx * 100 + lpd)
        f = rng.integers(-1000, 1000, size=g.shape).astype(np.float32)
        f = np.asfortranarray(f)
        ref = oracle_mod.assemble(f, g)
        gx, gy, gz = workloads.local_index(g)
        uni = np.zeros((nx * lpd + 1, ny * lpd + 1, nz * lpd + 1), np.float64)
        np.add.at(uni, (gx, gy, gz), f.astype(np.float64))
        mine = uni[gx, gy, gz].astype(np.float32)
        assert np.array_equal(ref, mine)


def test_taper_is_identical_on_shared_points(oracle_mod):
    """The GPU stores v once per unique point and tapers it with the copy of
    the lowest element; that is exact only if every copy carries the same
    taper value (coordinates of shared points are bit-identical)."""
    import workloads
    for wl in (workloads.config1(nt=4),):
        o = oracle_mod.Oracle(wl.grid)
        m = wl.model
        o.set_model(m["rhoinv"], m["lambda"], m["mu"])
        t = o.field(9)
        gx, gy, gz = workloads.local_index(wl.grid)
        g = wl.grid
        lo = np.full((g.nx * g.lpd + 1, g.ny * g.lpd + 1, g.nz * g.lpd + 1), np.inf, np.float32)
        hi = np.full_like(lo, -np.inf)
        np.minimum.at(lo, (gx, gy, gz), t)
        np.maximum.at(hi, (gx, gy, gz), t)
        assert np.array_equal(lo, hi)


def test_golden_config1(oracle_mod):
    """The oracle reproduces the committed golden seismograms and wavefield of
    config 1 (first 300 steps)."""
    path = os.path.join(GOLDEN, "config1_300steps.npz")
    gold = np.load(path)
    import workloads
    wl = workloads.config1(nt=int(gold["nt"]))
    o = oracle_mod.Oracle(wl.grid)
    oracle_mod.load_workload(o, wl)
    o.run(int(gold["nt"]))
    s = o.seismograms()
    ref = gold["seismograms"]
    err = np.linalg.norm(s - ref) / np.linalg.norm(ref)
    assert err < 1e-6, err
    vz = o.field(2)
    assert np.linalg.norm(vz[::2, ::2, ::2, ::2, ::2, ::2] - gold["vz_sub"]) / np.linalg.norm(gold["vz_sub"]) < 1e-6
