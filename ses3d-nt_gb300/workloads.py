"""Seeded synthetic workloads for the time step: domains, Earth models,
sources and receivers in the reference raw layout.

The reference ships no benchmark inputs; these are built from the workload
descriptions the project measures on (a homogeneous elastic section; a
heterogeneous visco-elastic section with depth gradients, +-5% smooth random
perturbations and per-element Q; a high-order precision case; a batched
multi-source case; a served request stream). Everything is seeded with
numpy PCG64. Choices the descriptions leave open are fixed here and listed in
`OPEN_CHOICES`.

Models are evaluated on the unique GLL points and then copied to every
element-local copy, so shared points of neighbouring elements carry identical
values (a continuous model), as the reference's own model writers produce
(examples/*/make_model.py write per-point values of smooth functions).
"""
import math
from dataclasses import dataclass, field

import numpy as np

from sesnt import Grid, SOURCE_MT, WAVELETS

EARTH_RADIUS = 6371000.0

OPEN_CHOICES = {
    "taper_width": 3,
    "taper_slope": 1.2,
    "ricker_onset_over_width": 1.5,  # onset = 1.5 * width (90 s for the 60 s wavelet)
    "dt_config2": 0.12,
    "dt_config3": 0.03,
    "dt_config4": 0.1,
    "model_generator_configs_3_5": "config 2 generator (gradients + 5% smooth perturbations + per-element Q)",
    "perturbation_field": "white noise on a 25 km grid, Gaussian kernel (sigma = L/2, L = 200 km), "
                          "scaled to max |dv/v| = 5%, trilinear to GLL points; independent fields for vp, vs, rho",
}


def gll_points_f64(lpd):
    """GLL points in float64 (only used to place model values)."""
    if lpd == 1:
        return np.array([-1.0, 1.0])
    # roots of (1-x^2) P'_N(x)
    c = np.zeros(lpd + 1)
    c[-1] = 1.0
    inner = np.polynomial.legendre.Legendre(c).deriv().roots()
    return np.concatenate([[-1.0], np.sort(inner.real), [1.0]])


def unique_axes(grid):
    """float64 colatitude [rad], longitude [rad], radius [m] of the unique GLL
    lines (ex*lpd+i), as the reference builds them (radius decreasing)."""
    n = grid.lpd
    xi = 0.5 * (1.0 + gll_points_f64(n))
    x0, x1 = math.radians(90.0 - grid.lat_max), math.radians(90.0 - grid.lat_min)
    y0, y1 = math.radians(grid.lon_min), math.radians(grid.lon_max)
    z0, z1 = grid.rad_max, grid.rad_min

    def axis(e, lo, hi):
        d = (hi - lo) / e
        pts = [lo + (k + xi[i]) * d for k in range(e) for i in range(n)] + [hi]
        return np.array(pts)

    return axis(grid.nx, x0, x1), axis(grid.ny, y0, y1), axis(grid.nz, z0, z1)


def local_index(grid):
    """For every element-local point (Fortran order of the raw layout), the
    unique-point coordinates (gx, gy, gz)."""
    n, p = grid.lpd, grid.lpd + 1
    ex, ey, ez, i, j, k = np.meshgrid(np.arange(grid.nx), np.arange(grid.ny), np.arange(grid.nz),
                                      np.arange(p), np.arange(p), np.arange(p), indexing="ij")
    return ex * n + i, ey * n + j, ez * n + k


def to_local(grid, uni):
    """Unique-point field uni[gx, gy, gz] -> raw-layout array (nx,ny,nz,P,P,P)."""
    gx, gy, gz = local_index(grid)
    return np.asfortranarray(uni[gx, gy, gz].astype(np.float32))


def smooth_noise(rng, extent_km, corr_km=200.0, h_km=25.0):
    """Gaussian-filtered white noise on a regular grid covering extent_km
    (3 lengths), normalised to max |f| = 1. Returns (field, spacing)."""
    pad = corr_km
    shape = [int(math.ceil((e + 2 * pad) / h_km)) + 1 for e in extent_km]
    w = rng.standard_normal(shape)
    sig = corr_km / 2.0 / h_km
    spec = np.fft.rfftn(w)
    ks = [np.fft.fftfreq(s) for s in shape[:-1]] + [np.fft.rfftfreq(shape[-1])]
    kk = np.meshgrid(*ks, indexing="ij")
    g = np.exp(-2.0 * (math.pi * sig) ** 2 * sum(x * x for x in kk))
    f = np.fft.irfftn(spec * g, s=shape, axes=(0, 1, 2))
    f /= np.abs(f).max()
    return f, h_km, pad


def trilinear(f, h, pad, x, y, z):
    """Sample grid field f (origin at -pad, spacing h) at km coordinates."""
    out = []
    coords = [(np.asarray(c) + pad) / h for c in (x, y, z)]
    i0 = [np.clip(np.floor(c).astype(int), 0, s - 2) for c, s in zip(coords, f.shape)]
    t = [c - i for c, i in zip(coords, i0)]
    acc = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wgt = ((t[0] if dx else 1 - t[0]) * (t[1] if dy else 1 - t[1]) * (t[2] if dz else 1 - t[2]))
                acc = acc + wgt * f[i0[0] + dx, i0[1] + dy, i0[2] + dz]
    out = acc
    return out


def homogeneous_model(grid, rho=3300.0, vp=8000.0, vs=4500.0):
    """rhoinv, lambda, mu for a homogeneous elastic medium (SI units)."""
    shape = grid.shape
    mu = rho * vs * vs
    lam = rho * (vp * vp - 2.0 * vs * vs)
    f = lambda v: np.full(shape, v, dtype=np.float32, order="F")
    return {"rhoinv": f(1.0 / rho), "lambda": f(lam), "mu": f(mu)}


def gradient_model(grid, seed, q=True, depth_top=None):
    """Config-2 generator: vp 8.0->8.9 km/s, vs 4.5->4.9 km/s, rho 3.3->3.6
    g/cm^3 linear in depth across the section, times (1 + 5% smooth noise,
    200 km correlation), and Q_mu ~ U[80, 600] per element."""
    rng = np.random.Generator(np.random.PCG64(seed))
    th, ph, r = unique_axes(grid)
    depth = (grid.rad_max - r) / (grid.rad_max - grid.rad_min)  # 0 at top, 1 at bottom
    r0 = grid.rad_max / 1000.0
    x_km = (th - th[0]) * r0
    y_km = (ph - ph[0]) * r0 * math.sin(0.5 * (th[0] + th[-1]))
    z_km = (grid.rad_max - r) / 1000.0
    ext = (x_km[-1], y_km[-1], z_km[-1])
    X, Y, Z = np.meshgrid(x_km, y_km, z_km, indexing="ij")
    D = np.broadcast_to(depth[None, None, :], X.shape)
    pert = []
    for _ in range(3):
        f, h, pad = smooth_noise(rng, ext)
        pert.append(0.05 * trilinear(f, h, pad, X, Y, Z))
    vp = (8.0 + 0.9 * D) * (1.0 + pert[0]) * 1000.0
    vs = (4.5 + 0.4 * D) * (1.0 + pert[1]) * 1000.0
    rho = (3.3 + 0.3 * D) * (1.0 + pert[2]) * 1000.0
    mu = rho * vs * vs
    lam = rho * (vp * vp - 2.0 * vs * vs)
    out = {"rhoinv": to_local(grid, 1.0 / rho), "lambda": to_local(grid, lam), "mu": to_local(grid, mu)}
    if q:
        qe = rng.uniform(80.0, 600.0, size=(grid.nx, grid.ny, grid.nz)).astype(np.float32)
        p = grid.lpd + 1
        out["q"] = np.asfortranarray(np.broadcast_to(qe[:, :, :, None, None, None],
                                                     (grid.nx, grid.ny, grid.nz, p, p, p)).astype(np.float32))
    return out


@dataclass
class Source:
    lat: float
    lon: float
    depth: float
    kind: int = SOURCE_MT
    comp: tuple = (1e18, 0.0, 0.0, 1e18, 0.0, 1e18)  # Mxx Mxy Mxz Myy Myz Mzz
    wavelet: str = "RICKER"
    width: float = 60.0
    onset: float = 90.0
    sim: int = 0


@dataclass
class Receiver:
    lat: float
    lon: float
    depth: float = 0.0


@dataclass
class Workload:
    name: str
    grid: Grid
    model: dict
    sources: list = field(default_factory=list)
    receivers: list = field(default_factory=list)


def interior_latlon(grid, margin_elems):
    """Latitude/longitude bounds strictly inside the taper strips."""
    dlat = (grid.lat_max - grid.lat_min) / grid.nx
    dlon = (grid.lon_max - grid.lon_min) / grid.ny
    return (grid.lat_min + margin_elems * dlat, grid.lat_max - margin_elems * dlat,
            grid.lon_min + margin_elems * dlon, grid.lon_max - margin_elems * dlon)


def config1(nt=2000, precision=4):
    """Plain method, small: 12x12x8 elements, lpd 4, homogeneous elastic,
    one moment-tensor Ricker source at 50 km depth in the centre, 16 surface
    receivers along the central meridian."""
    g = Grid(nx=12, ny=12, nz=8, lpd=4, lat_min=30.0, lat_max=50.0, lon_min=0.0, lon_max=20.0,
             rad_min=5771000.0, rad_max=6371000.0, dt=0.25, nt=nt, taper_width=3, taper_slope=1.2,
             precision=precision)
    src = [Source(lat=40.0, lon=10.0, depth=50000.0)]
    rec = [Receiver(lat=35.5 + 0.6 * q, lon=10.0, depth=0.0) for q in range(16)]
    return Workload("config1_plain_12x12x8_lpd4", g, homogeneous_model(g), src, rec)


def surface_array(grid, n_lat, n_lon, margin=3.5):
    la0, la1, lo0, lo1 = interior_latlon(grid, margin)
    out = []
    for a in range(n_lat):
        for b in range(n_lon):
            out.append(Receiver(lat=la0 + (la1 - la0) * (a + 0.5) / n_lat,
                                lon=lo0 + (lo1 - lo0) * (b + 0.5) / n_lon, depth=0.0))
    return out


def config2(nt=6000, seed=2, precision=4, nx=48, ny=48, nz=24, n_sls=3):
    """Heterogeneous visco-elastic: 48x48x24, lpd 4, gradient + perturbed
    model, 3 SLS with per-element Q, 64 surface receivers."""
    g = Grid(nx=nx, ny=ny, nz=nz, lpd=4, lat_min=30.0, lat_max=50.0, lon_min=0.0, lon_max=20.0,
             rad_min=5771000.0, rad_max=6371000.0, dt=OPEN_CHOICES["dt_config2"], nt=nt,
             taper_width=3, taper_slope=1.2, n_sls=n_sls, precision=precision)
    src = [Source(lat=40.0, lon=10.0, depth=50000.0)]
    return Workload("config2_hetero_sls_%dx%dx%d_lpd4" % (nx, ny, nz), g,
                    gradient_model(g, seed, q=n_sls > 0), src, surface_array(g, 8, 8))


def config3(nt=4000, seed=3, precision=4, nx=96, ny=96, nz=48, flags=0):
    """Precision variant: 96x96x48, lpd 6, config-2 generator, 3 SLS."""
    g = Grid(nx=nx, ny=ny, nz=nz, lpd=6, lat_min=30.0, lat_max=50.0, lon_min=0.0, lon_max=20.0,
             rad_min=5771000.0, rad_max=6371000.0, dt=OPEN_CHOICES["dt_config3"], nt=nt,
             taper_width=3, taper_slope=1.2, n_sls=3, precision=precision, flags=flags)
    src = [Source(lat=40.0, lon=10.0, depth=50000.0)]
    return Workload("config3_precision_%dx%dx%d_lpd6" % (nx, ny, nz), g, gradient_model(g, seed), src,
                    surface_array(g, 8, 8))


def random_sources(grid, n, rng, first_sim=0):
    la0, la1, lo0, lo1 = interior_latlon(grid, grid.taper_width + 0.5)
    out = []
    for s in range(n):
        m = rng.normal(0.0, 1e18, size=(3, 3))
        m = 0.5 * (m + m.T)
        out.append(Source(lat=float(rng.uniform(la0, la1)), lon=float(rng.uniform(lo0, lo1)),
                          depth=float(rng.uniform(10e3, 300e3)),
                          comp=(m[0, 0], m[0, 1], m[0, 2], m[1, 1], m[1, 2], m[2, 2]),
                          width=float(rng.uniform(40.0, 100.0)), sim=first_sim + s))
        out[-1].onset = 1.5 * out[-1].width
    return out


def config4(nt=3000, seed=4, batch=64, precision=4, nx=64, ny=64, nz=32):
    """Batched multi-source: one model on 64x64x32, lpd 4, 3 SLS; 64
    independent simulations (one per source), 128 shared receivers."""
    g = Grid(nx=nx, ny=ny, nz=nz, lpd=4, lat_min=30.0, lat_max=50.0, lon_min=0.0, lon_max=20.0,
             rad_min=5771000.0, rad_max=6371000.0, dt=OPEN_CHOICES["dt_config4"], nt=nt,
             taper_width=3, taper_slope=1.2, n_sls=3, precision=precision, batch=batch)
    rng = np.random.Generator(np.random.PCG64(seed))
    model = gradient_model(g, seed)
    src = random_sources(g, batch, rng)
    return Workload("config4_batched_%dsrc_%dx%dx%d_lpd4" % (batch, nx, ny, nz), g, model, src,
                    surface_array(g, 16, 8))


def setup(sim, wl):
    """Load a workload into a sesnt.Simulation: model, sources, receivers."""
    m = wl.model
    sim.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
    setup_sources_receivers(sim, wl)


def setup_sources_receivers(sim, wl):
    """The sources and receivers of a workload, located and registered."""
    from sesnt import locate_point, source_signature
    g = wl.grid
    for s in wl.sources:
        elem, vm = locate_point(g, s.lat, s.lon, s.depth)
        stf = source_signature(s.wavelet, s.onset, s.width, g.dt, g.nt)
        sim.add_source(s.sim, elem, vm, s.kind, np.asarray(s.comp, np.float32), stf)
    for r in wl.receivers:
        elem, vm = locate_point(g, r.lat, r.lon, r.depth)
        sim.add_receiver(elem, vm)


def request_of(wl):
    """A sesnt.Request (model, located sources with their STFs, receivers)
    for a workload whose sources are numbered 0..n-1 by `sim`."""
    import sesnt
    g = wl.grid
    srcs = []
    for s in sorted(wl.sources, key=lambda x: x.sim):
        elem, vm = sesnt.locate_point(g, s.lat, s.lon, s.depth)
        stf = sesnt.source_signature(s.wavelet, s.onset, s.width, g.dt, g.nt)
        srcs.append((elem, vm, s.kind, np.asarray(s.comp, np.float32), stf))
    recs = [sesnt.locate_point(g, r.lat, r.lon, r.depth) for r in wl.receivers]
    return sesnt.Request(g, wl.model, srcs, recs)


def served_stream(n_requests, seed, lateral=(16, 96), radial=(8, 48), lpds=(4, 6), steps=(500, 8000),
                  sources=(1, 32), receivers=16):
    """Seeded request stream of the served workload: per request a horizontal
    element count uniform in `lateral` per direction, radial in `radial`, lpd
    from `lpds`, step count log-uniform in `steps`, a config-2-generator model
    with its own seed and 1..n random moment-tensor sources. Returns a list of
    Workload objects (grid.batch = number of sources)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for q in range(n_requests):
        nx = int(rng.integers(lateral[0], lateral[1] + 1))
        ny = int(rng.integers(lateral[0], lateral[1] + 1))
        nz = int(rng.integers(radial[0], radial[1] + 1))
        lpd = int(rng.choice(lpds))
        nt = int(round(math.exp(rng.uniform(math.log(steps[0]), math.log(steps[1])))))
        ns = int(rng.integers(sources[0], sources[1] + 1))
        # dt for a Courant number ~0.25 at the smallest GLL spacing: element
        # sizes at the bottom of the section (r = 5771 km, colatitude 40 deg
        # for phi) times the smallest GLL interval of the degree
        elem_km = min(600.0 / nz, 5771.0 * math.radians(20.0) / nx,
                      5771.0 * math.sin(math.radians(40.0)) * math.radians(20.0) / ny)
        frac = float(np.diff(gll_points_f64(lpd)).min() / 2.0)
        dt = float(min(0.25, 0.25 * elem_km * 1e3 * frac / 9400.0))
        g = Grid(nx=nx, ny=ny, nz=nz, lpd=lpd, lat_min=30.0, lat_max=50.0, lon_min=0.0, lon_max=20.0,
                 rad_min=5771000.0, rad_max=6371000.0, dt=dt, nt=nt,
                 taper_width=min(2, (min(nx, ny, nz) - 1) // 2), taper_slope=1.2, n_sls=3, batch=ns)
        model = gradient_model(g, int(rng.integers(1 << 30)))
        srcs = random_sources(g, ns, rng)
        for s in srcs:  # pulse early enough to be recorded in short runs
            s.width = float(min(s.width, 0.1 * nt * dt + 4 * dt))
            s.onset = 1.5 * s.width
        out.append(Workload("request%d_%dx%dx%d_lpd%d_%dsrc_%dsteps" % (q, nx, ny, nz, lpd, ns, nt), g, model, srcs,
                            surface_array(g, 4, receivers // 4, margin=2.5)))
    return out
