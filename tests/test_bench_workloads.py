"""bench.py host logic (no GPU): the element kernel named in the roofline
for each kind of grid and --element choice (it selects the profiles/
traffic file), and smaller cases of the configs for ncu captures (--grid)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
import sesnt  # noqa: E402


def grid(lpd=4, n_sls=3, batch=1, flags=0):
    return sesnt.Grid(nx=4, ny=4, nz=4, lpd=lpd, lat_min=30.0, lat_max=40.0, lon_min=0.0, lon_max=10.0,
                      rad_min=5971000.0, rad_max=6371000.0, dt=0.1, nt=10, taper_width=1, taper_slope=1.2,
                      n_sls=n_sls, batch=batch, flags=flags)


@pytest.mark.parametrize("kw,element,kernel", [
    (dict(n_sls=0), "simple", "k_element"),                       # config 1
    (dict(), "simple", "k_element_stage"),                         # configs 2 and 4
    (dict(), "unstaged", "k_element"),
    (dict(), "persistent", "k_element_tma"),
    (dict(), "tc_tf32x3", "k_element_tc"),
    (dict(lpd=6), "simple", "k_element_stage"),                    # config 3
    (dict(lpd=3), "simple", "k_element"),                          # several elements per block
    (dict(flags=sesnt.FLAG_STRAIN), "simple", "k_element"),        # displacement gradient kept
    (dict(n_sls=0, batch=64), "simple", "k_element_pair"),         # config-1 grid, 64 sources
    (dict(n_sls=0, batch=64), "columns:5", "k_element_cols"),
    (dict(n_sls=0, batch=64), "columns_pair:1", "k_element_cols2"),
    (dict(n_sls=0, batch=3), "columns_pair:1", "k_element"),       # odd batch: no simulation pairs
    (dict(flags=sesnt.FLAG_KAHAN_STRESS), "simple", "k_element_stage"),
    (dict(n_sls=0, batch=2, flags=sesnt.FLAG_KAHAN_STRESS), "simple", "k_element"),
])
def test_element_kernel_name(kw, element, kernel):
    assert bench.element_kernel_name(element, grid(**kw)) == kernel


def test_profiles_hold_the_traffic_of_the_default_kernels():
    for workload in ("config2", "config1_batch64"):
        wl = bench.make_workload(workload, 10)
        name = "%s_%s.traffic.json" % (bench.element_kernel_name("simple", wl.grid), wl.name)
        assert os.path.exists(os.path.join(ROOT, "profiles", name)), name
    name = "k_element_stage_config3_precision_96x96x48_lpd6.traffic.json"
    assert os.path.exists(os.path.join(ROOT, "profiles", name))


def test_smaller_case_of_a_config():
    wl = bench.make_workload("config3", 10, (4, 4, 2))
    assert (wl.grid.nx, wl.grid.ny, wl.grid.nz, wl.grid.lpd, wl.grid.n_sls) == (4, 4, 2, 6, 3)
    assert wl.name == "config3_precision_4x4x2_lpd6"
    with pytest.raises(SystemExit):
        bench.make_workload("config1", 10, (8, 8, 4))
