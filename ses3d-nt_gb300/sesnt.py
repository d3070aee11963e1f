"""Python binding of libsesnt (include/sesnt.h) through ctypes.

This is the host-side mirror of the reference driver's interface for the time
step: a `Simulation` owns one library handle (one Earth model, `batch`
simulations) and exposes the calls the Fortran driver makes around
`ses3d_evolution` (src/ses3d-nt.F90:84-275): model set-up, point location,
sources, receivers, stepping and readback. Arrays use the reference raw
layout: numpy arrays of shape (nx, ny, nz, lpd+1, lpd+1, lpd+1) in Fortran
order (element x index fastest).

There is no CPU path: if libsesnt.so is missing or was built without a GPU
visible, every call fails with a clear error.
"""
import ctypes as C
import os
import re
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# SESNT_LIBRARY selects another build of the library (e.g. the bounds-check build)
LIB_PATH = os.environ.get("SESNT_LIBRARY") or os.path.join(HERE, "libsesnt.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "sesnt.h")

OK = 0
EINVAL, ECUDA, ENOMEM, ESTATE, ERANGE, ETIMEOUT, ENOTFOUND, EUNSUPPORTED, ENONFINITE = range(-1, -10, -1)
FLAG_KAHAN = 1
FLAG_NO_GRAPH = 2
FLAG_PERSISTENT_ELEMENT = 4
FLAG_TC_TF32X3 = 8
FLAG_TC_BF16X3 = 16
FLAG_STRAIN = 32
FLAG_ROTATION = 64
FLAG_NO_PAIR = 128
FLAG_NO_STAGE = 256
FLAG_AUTOTUNE = 512
FLAG_FORCE64 = 1024
FLAG_KAHAN_STRESS = 2048
(ELEMENT_AUTO, ELEMENT_POINT, ELEMENT_PAIR, ELEMENT_STAGE, ELEMENT_STAGE_REG, ELEMENT_PERSISTENT, ELEMENT_COLUMNS,
 ELEMENT_COLUMNS_STAGED, ELEMENT_COLUMNS_PAIR) = range(9)
SOURCE_MT, SOURCE_SF = 0, 1
WAVELETS = {"DELTA": 0, "RICKER": 1, "GAUSS": 2, "SIN**3": 3, "BRUNE": 4}
CH_VX, CH_VY, CH_VZ, CH_N = 1, 2, 4, 8
CH_ROT_VX, CH_ROT_VY, CH_ROT_VZ = 16, 32, 64
CH_MXX, CH_MXY, CH_MXZ, CH_MYY, CH_MYZ, CH_MZZ = 128, 256, 512, 1024, 2048, 4096
CH_FX, CH_FY, CH_FZ = 8192, 16384, 32768
# receiver attributes of the reference (construct_channel_container_receiver)
CHANNELS = {"vx": CH_VX, "vy": CH_VY, "e": CH_VY, "vz": CH_VZ, "z": CH_VZ, "n": CH_N,
            "rot_vx": CH_ROT_VX, "rot_vy": CH_ROT_VY, "rot_vz": CH_ROT_VZ,
            "mxx": CH_MXX, "mxy": CH_MXY, "myx": CH_MXY, "mxz": CH_MXZ, "mzx": CH_MXZ, "myy": CH_MYY,
            "myz": CH_MYZ, "mzy": CH_MYZ, "mzz": CH_MZZ, "fx": CH_FX, "fy": CH_FY, "fz": CH_FZ}
FIELDS = {"vx": 0, "vy": 1, "vz": 2, "sxx": 3, "sxy": 4, "sxz": 5, "syy": 6, "syz": 7, "szz": 8,
          "taper": 9, "mass": 10, "pressure": 40, "exx": 41, "exy": 42, "exz": 43, "eyy": 44, "eyz": 45,
          "ezz": 46, "rot_vx": 47, "rot_vy": 48, "rot_vz": 49, "lambda": 50, "mu": 51, "a": 52, "b": 53,
          "c": 54}
MEMORY_FIELD0 = 13


class SesntError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("sesnt error %d: %s" % (code, msg))
        self.code = code


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("lpd", C.c_int),
                ("taper_width", C.c_int), ("taper_slope", C.c_float),
                ("lat_min", C.c_float), ("lat_max", C.c_float), ("lon_min", C.c_float),
                ("lon_max", C.c_float), ("rad_min", C.c_float), ("rad_max", C.c_float),
                ("dt", C.c_float), ("nt", C.c_int), ("n_sls", C.c_int), ("precision", C.c_int),
                ("batch", C.c_int), ("flags", C.c_uint)]


@dataclass
class Grid:
    """Values of the reference NAMELIST groups &grid, &model, &time plus the
    GPU build choices (n_sls, precision, batch, flags)."""
    nx: int
    ny: int
    nz: int
    lpd: int
    lat_min: float
    lat_max: float
    lon_min: float
    lon_max: float
    rad_min: float
    rad_max: float
    dt: float
    nt: int
    taper_width: int = 3
    taper_slope: float = 1.2
    n_sls: int = 0
    precision: int = 4
    batch: int = 1
    flags: int = 0

    def c(self):
        return _Grid(self.nx, self.ny, self.nz, self.lpd, self.taper_width, self.taper_slope,
                     self.lat_min, self.lat_max, self.lon_min, self.lon_max, self.rad_min,
                     self.rad_max, self.dt, self.nt, self.n_sls, self.precision, self.batch,
                     self.flags)

    @property
    def shape(self):
        p = self.lpd + 1
        return (self.nx, self.ny, self.nz, p, p, p)

    @property
    def n_loc(self):
        return self.nx * self.ny * self.nz * (self.lpd + 1) ** 3

    @property
    def n_uni(self):
        n = self.lpd
        return (self.nx * n + 1) * (self.ny * n + 1) * (self.nz * n + 1)


class _SacInfo(C.Structure):
    _fields_ = [("lat", C.c_float), ("lon", C.c_float), ("depth", C.c_float), ("dt", C.c_float),
                ("network", C.c_char * 8), ("station", C.c_char * 8), ("location", C.c_char * 8),
                ("channel", C.c_char * 8), ("event", C.c_char * 16), ("override", C.c_int),
                ("date_time", C.c_int * 8)]


_lib = None


def header_functions():
    """Names of every function declared in include/sesnt.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sesnt_[a-z_0-9]+)\s*\(", txt)))


def lib():
    """Load libsesnt.so (built in place by build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SesntError(EUNSUPPORTED, "libsesnt.so not found at %s; run __graft_entry__.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P, I, F, U = C.c_void_p, C.c_int, C.c_float, C.c_uint
    fp = C.POINTER(C.c_float)
    ip = C.POINTER(C.c_int)
    G = C.POINTER(_Grid)
    sig = {
        "sesnt_create": (I, [G, C.POINTER(C.c_void_p)]),
        "sesnt_destroy": (I, [P]),
        "sesnt_last_error": (C.c_char_p, [P]),
        "sesnt_set_model": (I, [P, fp, fp, fp, fp, fp, fp, fp]),
        "sesnt_locate_point": (I, [G, F, F, F, ip, fp]),
        "sesnt_source_signature": (I, [I, F, F, F, I, fp]),
        "sesnt_add_source": (I, [P, I, I, I, I, fp, I, fp, fp, I]),
        "sesnt_add_receiver": (I, [P, I, I, I, fp, U]),
        "sesnt_step": (I, [P, I]),
        "sesnt_run": (I, [P, I, I]),
        "sesnt_run_timed": (I, [P, I, I, fp]),
        "sesnt_synchronize": (I, [P]),
        "sesnt_run_profiled": (I, [P, I, I, fp]),
        "sesnt_get_samples": (I, [P, I, fp]),
        "sesnt_reset": (I, [P]),
        "sesnt_get_seismograms": (I, [P, fp]),
        "sesnt_get_field": (I, [P, I, I, P, I]),
        "sesnt_v_ptp": (I, [P, I, fp]),
        "sesnt_kinetic_energy": (I, [P, I, C.POINTER(C.c_double)]),
        "sesnt_tune": (I, [P, C.c_char_p, I]),
        "sesnt_set_element_variant": (I, [P, I, I, I]),
        "sesnt_element_kernel": (I, [P, C.c_char_p, I, ip]),
        "sesnt_assemble_field": (I, [P, fp]),
        "sesnt_info": (I, [P, C.POINTER(C.c_longlong)]),
        "sesnt_footprint_bytes": (C.c_longlong, [G]),
        "sesnt_stream": (P, [P]),
        "sesnt_io_last_error": (C.c_char_p, []),
        "sesnt_config_last_error": (C.c_char_p, []),
        "sesnt_read_raw_field": (I, [C.c_char_p, I, I, I, I, fp]),
        "sesnt_write_raw_field": (I, [C.c_char_p, I, I, I, I, fp, I]),
        "sesnt_write_sac": (I, [C.c_char_p, C.POINTER(_SacInfo), fp, I]),
        "sesnt_sac_file_name": (I, [C.POINTER(_SacInfo), C.c_char_p, I]),
        "sesnt_day_of_year": (I, [I, I, I]),
        "sesnt_courant": (I, [G, fp, fp, fp, fp]),
        "sesnt_config_load": (I, [C.c_char_p, C.POINTER(C.c_void_p)]),
        "sesnt_config_free": (I, [P]),
        "sesnt_config_count": (I, [P, C.c_char_p]),
        "sesnt_config_grid": (I, [P, G]),
        "sesnt_config_get": (I, [P, C.c_char_p, I, C.c_char_p, C.c_char_p, I]),
        "sesnt_config_json": (I, [P, C.c_char_p, C.c_longlong, C.POINTER(C.c_longlong)]),
        "sesnt_forward": (I, [C.c_char_p, I, C.POINTER(C.c_int)]),
        "sesnt_get_trace": (I, [P, I, I, U, fp]),
        "sesnt_set_wait_limit": (I, [P, I, I]),
        "sesnt_state_bytes": (C.c_longlong, [P]),
        "sesnt_save_state": (I, [P, P]),
        "sesnt_load_state": (I, [P, P]),
        "sesnt_add_snapshot": (I, [P, I, I, I, I, I, C.c_char_p, C.c_char_p, I]),
        "sesnt_snapshots_wait": (I, [P]),
        "sesnt_field_name": (C.c_char_p, [I]),
        "sesnt_field_id": (I, [C.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f32(a, n=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F") if np.ndim(a) > 1
                             else np.asarray(a, dtype=np.float32))
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


def _check(rc, h=None):
    if rc < 0:
        msg = lib().sesnt_last_error(h)
        raise SesntError(rc, msg.decode() if msg else "")
    return rc


def locate_point(grid, lat, lon, depth):
    """(ex, ey, ez), vanderm[(lpd+1)^3] for a point (construct_point_cls)."""
    p = grid.lpd + 1
    elem = (C.c_int * 3)()
    vm = np.zeros(p ** 3, np.float32)
    g = grid.c()
    _check(lib().sesnt_locate_point(C.byref(g), lat, lon, depth, elem, _fptr(vm)))
    return (elem[0], elem[1], elem[2]), vm


def source_signature(wavelet, onset, width, dt, nt):
    code = WAVELETS[wavelet] if isinstance(wavelet, str) else int(wavelet)
    out = np.zeros(nt, np.float32)
    _check(lib().sesnt_source_signature(code, onset, width, dt, nt, _fptr(out)))
    return out


def footprint_bytes(grid):
    g = grid.c()
    return lib().sesnt_footprint_bytes(C.byref(g))


class Simulation:
    """One handle: an Earth model on the GPU and `grid.batch` wavefields."""

    def __init__(self, grid):
        self.grid = grid
        self._h = C.c_void_p()
        g = grid.c()
        _check(lib().sesnt_create(C.byref(g), C.byref(self._h)))
        self.receivers = 0

    def close(self):
        if self._h:
            lib().sesnt_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _c(self, rc):
        return _check(rc, self._h)

    def set_model(self, rhoinv, lam, mu, a=None, b=None, c=None, q=None):
        n = self.grid.n_loc
        arrs = [None if x is None else _f32(x, n) for x in (rhoinv, lam, mu, a, b, c, q)]
        ptrs = [None if x is None else _fptr(x) for x in arrs]
        self._c(lib().sesnt_set_model(self._h, *ptrs))

    def add_source(self, sim, elem, vanderm, kind, comp, stf):
        vm = _f32(vanderm, (self.grid.lpd + 1) ** 3)
        cp = _f32(comp)
        st = _f32(stf, self.grid.nt)
        self._c(lib().sesnt_add_source(self._h, sim, elem[0], elem[1], elem[2], _fptr(vm), kind, _fptr(cp),
                                       _fptr(st), st.size))

    def add_receiver(self, elem, vanderm, channels=CH_VX | CH_VY | CH_VZ):
        vm = _f32(vanderm, (self.grid.lpd + 1) ** 3)
        r = self._c(lib().sesnt_add_receiver(self._h, elem[0], elem[1], elem[2], _fptr(vm), channels))
        self.receivers += 1
        return r

    def step(self, it):
        self._c(lib().sesnt_step(self._h, it))

    def run(self, it0, nsteps):
        self._c(lib().sesnt_run(self._h, it0, nsteps))

    def run_timed(self, it0, nsteps):
        ms = C.c_float()
        self._c(lib().sesnt_run_timed(self._h, it0, nsteps, C.byref(ms)))
        return ms.value

    def run_profiled(self, it0, nsteps):
        """Device milliseconds summed per kernel: element, sources, node, receivers."""
        ms = np.zeros(4, np.float32)
        self._c(lib().sesnt_run_profiled(self._h, it0, nsteps, _fptr(ms)))
        return ms

    def samples(self, it, out=None):
        """Receiver samples of step it, [batch][nrec][3]."""
        if out is None:
            out = np.zeros((self.grid.batch, self.receivers, 3), np.float32)
        if self.receivers:
            self._c(lib().sesnt_get_samples(self._h, it, _fptr(out)))
        return out

    def synchronize(self):
        self._c(lib().sesnt_synchronize(self._h))

    def save_state(self):
        """Checkpoint of the time-stepping state (bytes)."""
        n = self._c(lib().sesnt_state_bytes(self._h))
        buf = np.zeros(n, np.uint8)
        self._c(lib().sesnt_save_state(self._h, buf.ctypes.data_as(C.c_void_p)))
        return buf

    def load_state(self, buf):
        buf = np.ascontiguousarray(buf, np.uint8)
        self._c(lib().sesnt_load_state(self._h, buf.ctypes.data_as(C.c_void_p)))

    def set_wait_limit(self, polls, drop_completion=False):
        self._c(lib().sesnt_set_wait_limit(self._h, polls, 1 if drop_completion else 0))

    def reset(self):
        self._c(lib().sesnt_reset(self._h))

    def seismograms(self):
        out = np.zeros((self.grid.batch, self.receivers, 3, self.grid.nt), np.float32)
        if self.receivers:
            self._c(lib().sesnt_get_seismograms(self._h, _fptr(out)))
        return out

    def trace(self, receiver, channel, sim=0):
        """One receiver channel (CH_* bit or attribute name), float32 [nt]."""
        ch = CHANNELS[channel] if isinstance(channel, str) else int(channel)
        out = np.zeros(self.grid.nt, np.float32)
        self._c(lib().sesnt_get_trace(self._h, sim, receiver, ch, _fptr(out)))
        return out

    def add_snapshot(self, field, start, increment, end=0, prefix="./", attribute=None, sim=0, override=False):
        """Volume snapshot of `field` (name or FIELD code) written to
        <prefix><attribute>_<it>.vol after every due step (written by a
        background thread; wait_snapshots() waits for the files)."""
        code = FIELDS[field] if isinstance(field, str) else int(field)
        return self._c(lib().sesnt_add_snapshot(self._h, sim, code, start, increment, end,
                                                prefix.encode() if prefix else None,
                                                attribute.encode() if attribute else None, 1 if override else 0))

    def wait_snapshots(self):
        self._c(lib().sesnt_snapshots_wait(self._h))

    def field(self, which, sim=0, precision=4):
        code = FIELDS[which] if isinstance(which, str) else int(which)
        dt = np.float64 if precision == 8 else np.float32
        out = np.zeros(self.grid.n_loc, dt)
        self._c(lib().sesnt_get_field(self._h, sim, code, out.ctypes.data_as(C.c_void_p), precision))
        return out.reshape(self.grid.shape, order="F")

    def v_ptp(self, sim=0):
        out = np.zeros(2, np.float32)
        self._c(lib().sesnt_v_ptp(self._h, sim, _fptr(out)))
        return float(out[0]), float(out[1])

    def tune(self):
        """Tune the element kernel on this grid (after set_model, before stepping); returns the report."""
        buf = C.create_string_buffer(8192)
        self._c(lib().sesnt_tune(self._h, buf, len(buf)))
        return buf.value.decode()

    def set_element_variant(self, variant, arg=0, piece=8192):
        self._c(lib().sesnt_set_element_variant(self._h, variant, arg, piece))

    def element_kernel(self):
        """(name of the element kernel a step launches, (variant, arg, piece))."""
        buf = C.create_string_buffer(128)
        ch = (C.c_int * 3)()
        self._c(lib().sesnt_element_kernel(self._h, buf, len(buf), ch))
        return buf.value.decode(), tuple(ch)

    def kinetic_energy(self, sim=0):
        """Kinetic energy of simulation `sim` in joules (elastic_vars.F90:218-246)."""
        out = C.c_double(0.0)
        self._c(lib().sesnt_kinetic_energy(self._h, sim, C.byref(out)))
        return out.value

    def assemble(self, field):
        f = _f32(field, self.grid.n_loc).copy()
        self._c(lib().sesnt_assemble_field(self._h, _fptr(f)))
        return f.reshape(self.grid.shape, order="F")

    def info(self):
        out = (C.c_longlong * 6)()
        self._c(lib().sesnt_info(self._h, out))
        keys = ("elements", "n_loc", "n_uni", "device_bytes", "algorithmic_bytes_per_step", "launches_per_step")
        return dict(zip(keys, list(out)))


# ---------------------------------------------------------------------------
# files and configuration
# ---------------------------------------------------------------------------
def _io_check(rc, which="io"):
    if rc < 0:
        m = lib().sesnt_io_last_error() if which == "io" else lib().sesnt_config_last_error()
        raise SesntError(rc, m.decode() if m else "")
    return rc


def read_raw_field(path, grid):
    """A raw model/field file in the reference layout, with the size check."""
    out = np.zeros(grid.n_loc, np.float32)
    _io_check(lib().sesnt_read_raw_field(os.fsencode(path), grid.nx, grid.ny, grid.nz, grid.lpd, _fptr(out)))
    return out.reshape(grid.shape, order="F")


def write_raw_field(path, grid, field, override=False):
    f = _f32(field, grid.n_loc)
    _io_check(lib().sesnt_write_raw_field(os.fsencode(path), grid.nx, grid.ny, grid.nz, grid.lpd, _fptr(f),
                                          int(bool(override))))


def sac_info(lat, lon, depth, dt, network="Ses3d-NT", station="", location="", channel="", event="ses3d-nt event",
             override=False, date_time=(2000, 1, 1, 0, 0, 0, 0, 0)):
    i = _SacInfo()
    i.lat, i.lon, i.depth, i.dt = lat, lon, depth, dt
    i.network, i.station, i.location = network.encode()[:8], station.encode()[:8], location.encode()[:8]
    i.channel, i.event = channel.encode()[:8], event.encode()[:16]
    i.override = int(bool(override))
    for q in range(8):
        i.date_time[q] = int(date_time[q])
    return i


def write_sac(path, info, data):
    d = np.ascontiguousarray(data, np.float32)
    _io_check(lib().sesnt_write_sac(os.fsencode(path), C.byref(info), _fptr(d), d.size))


def sac_file_name(info):
    buf = C.create_string_buffer(256)
    _io_check(lib().sesnt_sac_file_name(C.byref(info), buf, 256))
    return buf.value.decode()


def day_of_year(y, m, d):
    return lib().sesnt_day_of_year(y, m, d)


def courant(grid, rhoinv, lam, mu):
    """(Courant number, maximum resolved frequency in Hz) of a model."""
    out = np.zeros(2, np.float32)
    g = grid.c()
    n = grid.n_loc
    arrs = [_f32(x, n) for x in (rhoinv, lam, mu)]
    _io_check(lib().sesnt_courant(C.byref(g), *[_fptr(a) for a in arrs], _fptr(out)))
    return float(out[0]), float(out[1])


class Config:
    """A reference configuration file (NAMELIST groups)."""

    def __init__(self, path):
        self._c = C.c_void_p()
        _io_check(lib().sesnt_config_load(os.fsencode(path), C.byref(self._c)), "config")

    def close(self):
        if self._c:
            lib().sesnt_config_free(self._c)
            self._c = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def count(self, group):
        return lib().sesnt_config_count(self._c, group.encode())

    def get(self, group, key, idx=0):
        buf = C.create_string_buffer(1 << 16)
        rc = lib().sesnt_config_get(self._c, group.encode(), idx, key.encode(), buf, 1 << 16)
        if rc == ENOTFOUND:
            return None
        _io_check(rc, "config")
        return buf.value.decode()

    def json(self):
        import json as _json
        need = C.c_longlong()
        _io_check(lib().sesnt_config_json(self._c, None, 0, C.byref(need)), "config")
        buf = C.create_string_buffer(need.value)
        _io_check(lib().sesnt_config_json(self._c, buf, need.value, None), "config")
        return _json.loads(buf.value.decode())

    def grid(self):
        g = _Grid()
        _io_check(lib().sesnt_config_grid(self._c, C.byref(g)), "config")
        return Grid(nx=g.nx, ny=g.ny, nz=g.nz, lpd=g.lpd, lat_min=g.lat_min, lat_max=g.lat_max,
                    lon_min=g.lon_min, lon_max=g.lon_max, rad_min=g.rad_min, rad_max=g.rad_max, dt=g.dt,
                    nt=g.nt, taper_width=g.taper_width, taper_slope=g.taper_slope, n_sls=g.n_sls)


def forward(config_path, precision=4):
    """Run the reference forward workflow from a config file on the GPU;
    returns the number of SAC traces written."""
    n = C.c_int()
    rc = lib().sesnt_forward(os.fsencode(config_path), precision, C.byref(n))
    if rc < 0:
        m = lib().sesnt_config_last_error()
        raise SesntError(rc, m.decode() if m else "")
    return n.value


# ---------------------------------------------------------------------------
# request server
# ---------------------------------------------------------------------------
class _ServerConfig(C.Structure):
    _fields_ = [("device_bytes", C.c_longlong), ("max_active", C.c_int), ("chunk_steps", C.c_int),
                ("max_batch", C.c_int)]


class _Request(C.Structure):
    _fields_ = [("grid", _Grid)] + [(k, C.POINTER(C.c_float)) for k in
                                    ("rhoinv", "lambda_", "mu", "a", "b", "c", "q")] + [
        ("n_sources", C.c_int), ("src_elem", C.POINTER(C.c_int)), ("src_kind", C.POINTER(C.c_int)),
        ("src_vanderm", C.POINTER(C.c_float)), ("src_comp", C.POINTER(C.c_float)),
        ("src_stf", C.POINTER(C.c_float)), ("n_receivers", C.c_int), ("rec_elem", C.POINTER(C.c_int)),
        ("rec_vanderm", C.POINTER(C.c_float)), ("rec_mask", C.POINTER(C.c_uint))]


class _ServerStats(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in ("completed", "failed", "queued", "active", "device_bytes_used",
                                            "device_bytes_budget", "total_updates")] + [
        (k, C.c_double) for k in ("latency_p50", "latency_p99", "latency_max", "queue_wait_p50", "wall_seconds",
                                  "updates_per_second")]


def _server_lib():
    L = lib()
    if not getattr(L, "_server_ready", False):
        P = C.c_void_p
        for name, res, args in [
                ("sesnt_server_create", C.c_int, [C.POINTER(_ServerConfig), C.POINTER(P)]),
                ("sesnt_server_destroy", C.c_int, [P]),
                ("sesnt_server_submit", C.c_int, [P, C.POINTER(_Request), C.POINTER(C.c_longlong)]),
                ("sesnt_server_wait", C.c_int, [P, C.c_longlong, C.c_double]),
                ("sesnt_server_result", C.c_int, [P, C.c_longlong, C.POINTER(C.c_float),
                                                  C.POINTER(C.c_double)]),
                ("sesnt_server_release", C.c_int, [P, C.c_longlong]),
                ("sesnt_server_cancel", C.c_int, [P, C.c_longlong]),
                ("sesnt_server_stats", C.c_int, [P, C.POINTER(_ServerStats)]),
                ("sesnt_server_last_error", C.c_char_p, [P])]:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        L._server_ready = True
    return L


class Request:
    """Host arrays of one request (model, located sources, receivers)."""

    def __init__(self, grid, model, sources, receivers):
        # sources: list of (elem(3), vanderm, kind, comp(6 or 3), stf(nt)); receivers: list of (elem, vanderm)
        self.grid = grid
        self.model = [None if model.get(k) is None else _f32(model[k], grid.n_loc)
                      for k in ("rhoinv", "lambda", "mu", "a", "b", "c", "q")]
        ns, nr = len(sources), len(receivers)
        NP = (grid.lpd + 1) ** 3
        self.src_elem = np.ascontiguousarray([s[0] for s in sources], np.int32).reshape(ns, 3)
        self.src_vm = np.ascontiguousarray([s[1] for s in sources], np.float32).reshape(ns, NP)
        self.src_kind = np.ascontiguousarray([s[2] for s in sources], np.int32)
        comp = np.zeros((ns, 6), np.float32)
        for i, s in enumerate(sources):
            comp[i, :len(s[3])] = s[3]
        self.src_comp = comp
        self.src_stf = np.ascontiguousarray([s[4] for s in sources], np.float32).reshape(ns, grid.nt)
        self.rec_elem = np.ascontiguousarray([r[0] for r in receivers], np.int32).reshape(nr, 3)
        self.rec_vm = np.ascontiguousarray([r[1] for r in receivers], np.float32).reshape(nr, NP)

    def c(self):
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        r = _Request()
        r.grid = self.grid.c()
        for name, arr in zip(("rhoinv", "lambda_", "mu", "a", "b", "c", "q"), self.model):
            setattr(r, name, _fptr(arr) if arr is not None else C.POINTER(C.c_float)())
        r.n_sources = len(self.src_kind)
        r.src_elem, r.src_kind = ip(self.src_elem), ip(self.src_kind)
        r.src_vanderm, r.src_comp, r.src_stf = _fptr(self.src_vm), _fptr(self.src_comp), _fptr(self.src_stf)
        r.n_receivers = len(self.rec_elem)
        r.rec_elem, r.rec_vanderm = ip(self.rec_elem), _fptr(self.rec_vm)
        r.rec_mask = C.POINTER(C.c_uint)()
        return r


class Server:
    """Queue of forward requests served concurrently on the current GPU."""

    def __init__(self, device_bytes=0, max_active=16, chunk_steps=64, max_batch=0):
        L = _server_lib()
        self._s = C.c_void_p()
        cfg = _ServerConfig(device_bytes, max_active, chunk_steps, max_batch)
        _check(L.sesnt_server_create(C.byref(cfg), C.byref(self._s)))
        self._req = {}

    def submit(self, request):
        rid = C.c_longlong()
        cr = request.c()
        rc = _server_lib().sesnt_server_submit(self._s, C.byref(cr), C.byref(rid))
        if rc < 0:
            raise SesntError(rc, (_server_lib().sesnt_server_last_error(self._s) or b"").decode())
        self._req[rid.value] = request
        return rid.value

    def wait(self, rid, timeout=600.0):
        return _server_lib().sesnt_server_wait(self._s, rid, timeout)

    def result(self, rid):
        r = self._req[rid]
        g = r.grid
        out = np.zeros((len(r.src_kind), len(r.rec_elem), 3, g.nt), np.float32)
        times = (C.c_double * 2)()
        rc = _server_lib().sesnt_server_result(self._s, rid, _fptr(out), times)
        if rc < 0:
            raise SesntError(rc, (_server_lib().sesnt_server_last_error(self._s) or b"").decode())
        return out, times[0], times[1]

    def release(self, rid):
        self._req.pop(rid, None)
        return _server_lib().sesnt_server_release(self._s, rid)

    def cancel(self, rid):
        return _server_lib().sesnt_server_cancel(self._s, rid)

    def stats(self):
        st = _ServerStats()
        _check(_server_lib().sesnt_server_stats(self._s, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def close(self):
        if self._s:
            _server_lib().sesnt_server_destroy(self._s)
            self._s = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
