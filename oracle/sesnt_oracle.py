"""Python wrapper of the oracle (oracle.cpp): the CPU restatement of the
reference time step, used only as the checker by tests/, by
__graft_entry__.smoke() and by the CPU-baseline leg of bench.py.

build() compiles oracle.cpp with g++ into oracle/_build/liboracle.so (OpenMP,
-ffp-contract=off so REAL32 expressions round as the reference writes them).
The reference itself is Fortran + MPI and cannot be compiled here (no Fortran
compiler), so there is no oracle/_ref build of it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", LIB + ".tmp", SRC]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + p.stdout)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Cfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("lpd", C.c_int),
                ("taper_width", C.c_int), ("nt", C.c_int), ("precision", C.c_int),
                ("taper_slope", C.c_float), ("lat_min", C.c_float), ("lat_max", C.c_float),
                ("lon_min", C.c_float), ("lon_max", C.c_float), ("rad_min", C.c_float),
                ("rad_max", C.c_float), ("dt", C.c_float)]


_L = None


def lib():
    global _L
    if _L is None:
        _L = C.CDLL(build())
        fp = C.POINTER(C.c_float)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        V = C.c_void_p
        _L.oracle_create.restype = V
        _L.oracle_create.argtypes = [C.POINTER(_Cfg)]
        _L.oracle_set_model.argtypes = [V, fp, fp, fp, fp, fp, fp, fp]
        _L.oracle_locate_cfg.argtypes = [C.POINTER(_Cfg), C.c_float, C.c_float, C.c_float, ip, fp]
        _L.oracle_add_source.argtypes = [V, C.c_int, C.c_int, C.c_int, fp, C.c_int, fp, fp]
        _L.oracle_add_receiver.argtypes = [V, C.c_int, C.c_int, C.c_int, fp]
        _L.oracle_add_receiver_mask.argtypes = [V, C.c_int, C.c_int, C.c_int, fp, C.c_uint]
        _L.oracle_keep_strain.argtypes = [V]
        _L.oracle_get_trace.argtypes = [V, C.c_int, C.c_int, V]
        _L.oracle_run.argtypes = [V, C.c_int]
        _L.oracle_get_field.argtypes = [V, C.c_int, V]
        _L.oracle_get_seismograms.argtypes = [V, V]
        _L.oracle_destroy.argtypes = [V]
        _L.oracle_is_visco.argtypes = [V]
        _L.oracle_kinetic_energy.argtypes = [V, dp]
        _L.oracle_gll_f32.argtypes = [C.c_int, fp, fp, fp]
        _L.oracle_gll_f64.argtypes = [C.c_int, dp, dp, dp]
        _L.oracle_coordinates_1d.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, fp]
        _L.oracle_lagrange.argtypes = [C.c_float, C.c_int, fp, fp]
        _L.oracle_assemble_f32.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, fp]
        _L.oracle_stf.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, fp]
        _L.oracle_threads.argtypes = [C.c_int]
        _L.oracle_courant.argtypes = [V, fp]
    return _L


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def cfg_of(grid, precision=None):
    return _Cfg(grid.nx, grid.ny, grid.nz, grid.lpd, grid.taper_width, grid.nt,
                precision or grid.precision, grid.taper_slope, grid.lat_min, grid.lat_max,
                grid.lon_min, grid.lon_max, grid.rad_min, grid.rad_max, grid.dt)


def threads(n=0):
    return lib().oracle_threads(n)


def gll(lpd, precision=4):
    p = lpd + 1
    if precision == 8:
        k, w, d = np.zeros(p), np.zeros(p), np.zeros(p * p)
        lib().oracle_gll_f64(lpd, *(x.ctypes.data_as(C.POINTER(C.c_double)) for x in (k, w, d)))
    else:
        k, w, d = (np.zeros(n, np.float32) for n in (p, p, p * p))
        lib().oracle_gll_f32(lpd, _fp(k), _fp(w), _fp(d))
    return k, w, d.reshape(p, p)


def coordinates_1d(elms, lpd, lo, hi):
    out = np.zeros(elms * (lpd + 1), np.float32)
    lib().oracle_coordinates_1d(elms, lpd, lo, hi, _fp(out))
    return out.reshape(elms, lpd + 1)


def lagrange(x, knots):
    k = np.ascontiguousarray(knots, np.float32)
    out = np.zeros(k.size, np.float32)
    lib().oracle_lagrange(x, k.size, _fp(k), _fp(out))
    return out


def assemble(field, grid):
    f = np.array(np.asarray(field, np.float32).ravel(order="F"), copy=True)
    lib().oracle_assemble_f32(grid.nx, grid.ny, grid.nz, grid.lpd, _fp(f))
    return f.reshape(grid.shape, order="F")


def stf(kind, onset, width, dt, nt):
    out = np.zeros(nt, np.float32)
    lib().oracle_stf(kind, onset, width, dt, nt, _fp(out))
    return out


def locate(grid, lat, lon, depth):
    cfg = cfg_of(grid)
    e = (C.c_int * 3)()
    vm = np.zeros((grid.lpd + 1) ** 3, np.float32)
    rc = lib().oracle_locate_cfg(C.byref(cfg), lat, lon, depth, e, _fp(vm))
    if rc != 0:
        return None, None
    return (e[0], e[1], e[2]), vm


class Oracle:
    """One reference-layout simulation on the CPU (single source set)."""

    def __init__(self, grid, precision=4):
        self.grid = grid
        self.precision = precision
        self._cfg = cfg_of(grid, precision)
        self._h = lib().oracle_create(C.byref(self._cfg))
        self.nrec = 0

    def close(self):
        if self._h:
            lib().oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_model(self, rhoinv, lam, mu, a=None, b=None, c=None, q=None):
        keep = []

        def p(x):
            if x is None:
                return None
            x = np.ascontiguousarray(np.asarray(x, np.float32).ravel(order="F"))
            keep.append(x)
            return _fp(x)

        lib().oracle_set_model(self._h, p(rhoinv), p(lam), p(mu), p(a), p(b), p(c), p(q))

    def add_source(self, elem, vm, kind, comp, stf_):
        vm = np.ascontiguousarray(vm, np.float32)
        comp = np.ascontiguousarray(comp, np.float32)
        stf_ = np.ascontiguousarray(stf_, np.float32)
        lib().oracle_add_source(self._h, elem[0], elem[1], elem[2], _fp(vm), kind, _fp(comp), _fp(stf_))

    def add_receiver(self, elem, vm, mask=7):
        """mask: channel bits as the GPU library's SESNT_CH_* (vx vy vz always recorded)."""
        vm = np.ascontiguousarray(vm, np.float32)
        lib().oracle_add_receiver_mask(self._h, elem[0], elem[1], elem[2], _fp(vm), mask)
        self.nrec += 1

    def keep_strain(self):
        """Integrate the displacement gradient (before set_model)."""
        lib().oracle_keep_strain(self._h)

    def trace(self, receiver, channel):
        """One receiver channel (a single SESNT_CH_* bit), [nt]."""
        bit = int(channel).bit_length() - 1
        dt = np.float64 if self.precision == 8 else np.float32
        out = np.zeros(self.grid.nt, dt)
        if lib().oracle_get_trace(self._h, receiver, bit, out.ctypes.data_as(C.c_void_p)) != 0:
            raise ValueError("channel %d of receiver %d unavailable" % (channel, receiver))
        return out

    def run(self, nsteps):
        lib().oracle_run(self._h, nsteps)

    def field(self, which):
        dt = np.float64 if self.precision == 8 else np.float32
        out = np.zeros(self.grid.n_loc, dt)
        rc = lib().oracle_get_field(self._h, which, out.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise ValueError("field %d unavailable" % which)
        return out.reshape(self.grid.shape, order="F")

    def seismograms(self):
        dt = np.float64 if self.precision == 8 else np.float32
        out = np.zeros((self.nrec, 3, self.grid.nt), dt)
        lib().oracle_get_seismograms(self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def courant(self):
        out = np.zeros(2, np.float32)
        lib().oracle_courant(self._h, _fp(out))
        return float(out[0]), float(out[1])

    def visco(self):
        return bool(lib().oracle_is_visco(self._h))

    def kinetic_energy(self):
        """kinetic_energy of src/elastic_vars.F90:218-246 in the oracle's precision."""
        out = C.c_double(0.0)
        lib().oracle_kinetic_energy(self._h, C.byref(out))
        return out.value


def load_workload(o, wl, sim=0, masks=None):
    """Model, the sources of simulation `sim`, and all receivers of a workload,
    located with the oracle's own point location. masks: per-receiver channel
    bits (default vx vy vz)."""
    m = wl.model
    o.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
    kinds = {"DELTA": 0, "RICKER": 1, "GAUSS": 2, "SIN**3": 3, "BRUNE": 4}
    g = wl.grid
    for s in wl.sources:
        if s.sim != sim:
            continue
        elem, vm = locate(g, s.lat, s.lon, s.depth)
        o.add_source(elem, vm, s.kind, np.asarray(s.comp, np.float32),
                     stf(kinds[s.wavelet], s.onset, s.width, g.dt, g.nt))
    for q, r in enumerate(wl.receivers):
        elem, vm = locate(g, r.lat, r.lon, r.depth)
        o.add_receiver(elem, vm, 7 if masks is None else masks[q])
