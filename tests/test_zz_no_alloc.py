"""sesnt_assemble_field_noalloc, the assembly entry point for callers that
cannot allocate device memory when they call it (for example inside a time
loop that must not synchronise the whole device the way cudaMalloc/cudaFree
may, or in a program that reserved all device memory up front). It must give the same
sums as the allocating sesnt_assemble_field, call after call, although every
call reuses one fixed device array.

Collected last (file name) so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import sesnt

pytestmark = pytest.mark.gpu


def _grid(nx=6, ny=5, nz=4, lpd=4):
    return sesnt.Grid(nx=nx, ny=ny, nz=nz, lpd=lpd, lat_min=30.0, lat_max=40.0, lon_min=0.0, lon_max=10.0,
                      rad_min=5971000.0, rad_max=6371000.0, dt=0.1, nt=10, taper_width=1)


def _noalloc(sim, d_in, d_out):
    f = sesnt.lib().sesnt_assemble_field_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    return f(sim.handle, C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()))


def test_noalloc_assembly_matches_allocating_entry_point(gpu, sesnt_lib):
    torch = pytest.importorskip("torch")
    for lpd in (4, 6):
        g = _grid(lpd=lpd)
        with sesnt.Simulation(g) as sim:
            rng = np.random.default_rng(20 + lpd)
            for call in range(2):  # two calls in a row: the shared array is cleared each time
                f = np.asfortranarray(rng.integers(-2048, 2048, size=g.shape).astype(np.float32))
                want = sim.assemble(f)  # allocating entry point, host buffers
                d_in = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).to("cuda")
                d_out = torch.full_like(d_in, float("nan"))
                torch.cuda.synchronize()
                rc = _noalloc(sim, d_in, d_out)
                assert rc == sesnt.OK, sesnt.lib().sesnt_last_error(sim.handle)
                got = d_out.cpu().numpy().reshape(g.shape, order="F")
                # integer-valued data: the sums are exact in any order
                assert np.array_equal(got, want), (lpd, call)
            # in place (d_out == d_in)
            f = np.asfortranarray(rng.integers(-2048, 2048, size=g.shape).astype(np.float32))
            d = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).to("cuda")
            torch.cuda.synchronize()
            assert _noalloc(sim, d, d) == sesnt.OK
            assert np.array_equal(d.cpu().numpy().reshape(g.shape, order="F"), sim.assemble(f))


def test_noalloc_on_an_fp64_handle_sums_in_float32(gpu, sesnt_lib):
    """On an FP64 handle the allocating entry point sums in float64 and the
    no-allocation one in float32: with non-integer data they agree to float32
    rounding of sums of up to 8 copies of values in [-1, 1]: at most 7
    float32 additions per point, each rounding by at most 2^-24 of a partial
    sum below 8, i.e. 3.4e-6 absolute; the test bounds the difference by 2e-6
    of the largest sum (about 5 on this grid)."""
    torch = pytest.importorskip("torch")
    g = _grid(lpd=5)
    g.precision = 8
    with sesnt.Simulation(g) as sim:
        rng = np.random.default_rng(31)
        for call in range(2):
            f = np.asfortranarray(rng.uniform(-1.0, 1.0, size=g.shape).astype(np.float32))
            want = sim.assemble(f)
            d_in = torch.from_numpy(np.ascontiguousarray(f.ravel(order="F"))).to("cuda")
            d_out = torch.full_like(d_in, float("nan"))
            torch.cuda.synchronize()
            assert _noalloc(sim, d_in, d_out) == sesnt.OK, sesnt.lib().sesnt_last_error(sim.handle)
            got = d_out.cpu().numpy().reshape(g.shape, order="F")
            err = float(np.abs(got.astype(np.float64) - want).max() / np.abs(want).max())
            print("FP64 handle, call %d: no-allocation vs allocating assembly %.2e of the largest sum"
                  % (call, err))
            assert err < 2e-6, call


def test_noalloc_rejects_grids_beyond_the_fixed_scratch(gpu, sesnt_lib):
    torch = pytest.importorskip("torch")
    g = _grid(nx=64, ny=64, nz=16, lpd=4)  # 257*257*65 = 4.29M unique points > 4,194,304
    with sesnt.Simulation(g) as sim:
        d = torch.zeros(g.n_loc, dtype=torch.float32, device="cuda")
        rc = _noalloc(sim, d, d)
        assert rc == sesnt.ERANGE
        assert b"unique points" in sesnt.lib().sesnt_last_error(sim.handle)
