#!/usr/bin/env python3
"""Benchmark of the GB300 spectral-element time step.

Default workload: the heterogeneous visco-elastic section (48x48x24 elements,
lpd 4, three standard linear solids, seeded gradient + 5% perturbation model,
per-element Q, one moment-tensor source, 64 surface receivers). A "step" is
one time step of the whole section. `value` is GLL-point-updates/s
(element-local points x steps x simulations / device seconds) over exactly K
timed steps, measured with CUDA events on the library's own stream; the
per-step working set (about 1.5 GB) is larger than L2, so no flush is needed.

Also reported on the same line: the roofline of the dominant kernel (the
element kernel; its algorithmic bytes over its event-timed duration), the
end-to-end rate through the C ABI with host buffers, the FP32 error against
the FP64 build, the oracle timed on the host cores, and SM clocks sampled
during the timed region.

--impl reference times the CPU implementation of the path instead: the
reference is Fortran + MPI with no compiler on either machine, so the oracle's
restatement of it runs on all host cores.

With torchrun (N>1) every rank runs an independent replica of the workload
(the path has no data-parallel split: every element lives on one GPU) and
rank 0 prints the aggregate.
"""
import argparse
import copy
import json
import os
import shutil
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "ses3d-nt_gb300"), os.path.join(ROOT, "oracle")]

RANK = int(os.environ.get("RANK", "0"))
WORLD = int(os.environ.get("WORLD_SIZE", "1"))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
    # one GPU per rank; set before the library's first CUDA call
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

METRIC = "GLL-point-updates/s"


# ---------------------------------------------------------------------------
# ranks (host-side only: barrier and reductions over gloo)
# ---------------------------------------------------------------------------
_pg = None


def dist_init():
    global _pg
    if WORLD > 1 and _pg is None:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29511")
        dist.init_process_group("gloo", rank=RANK, world_size=WORLD)
        _pg = dist
    return _pg


def barrier():
    if WORLD > 1:
        dist_init().barrier()


def reduce(x, op):
    """max / sum of a float over ranks (gloo)."""
    if WORLD == 1:
        return float(x)
    import torch
    d = dist_init()
    t = torch.tensor([float(x)], dtype=torch.float64)
    d.all_reduce(t, op=d.ReduceOp.MAX if op == "max" else d.ReduceOp.SUM)
    return float(t.item())


def aggregate(units, ms):
    """Whole-job rate of the replicas: the units all ranks processed over the
    slowest rank's time. Returns (units/s, slowest ms)."""
    ms_max = reduce(ms, "max")
    total = reduce(units, "sum")
    return total / (ms_max / 1e3), ms_max


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.reader = None

    def start(self):
        exe = shutil.which("nvidia-smi")
        if not exe:
            return
        self.proc = subprocess.Popen([exe, "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                      "-lms", "200", "-i", str(self.device)],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.reader.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "power_w_max": max(power), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def make_workload(name, nt_needed, grid=None):
    """The named workload; `grid` = (nx, ny, nz) scales configs 2-4 down to a
    small case of the same generator and kernels (ncu captures)."""
    import workloads
    size = dict(zip(("nx", "ny", "nz"), grid)) if grid else {}
    if grid and name not in ("config2", "config3", "config4", "config4_plain"):
        raise SystemExit("--grid applies to config2, config3, config4 and config4_plain")
    if name == "config2":
        wl = workloads.config2(nt=6000, **size)
    elif name == "config1":
        wl = workloads.config1(nt=2000)
    elif name == "config3":
        wl = workloads.config3(nt=4000, **size)
    elif name == "config4":
        wl = workloads.config4(nt=3000, **size)
    elif name == "config4_plain":  # the config-4 grid and model with one source
        wl = workloads.config4(nt=3000, batch=1, **size)
    elif name == "config1_batch64":  # the config-1 grid and model with 64 random sources
        import numpy as _np
        wl = workloads.config1(nt=2000)
        wl.grid.batch = 64
        wl.sources = workloads.random_sources(wl.grid, 64, _np.random.Generator(_np.random.PCG64(1)))
        wl.name = "config1_batched_64src_12x12x8_lpd4"
    else:
        raise SystemExit("unknown workload " + name)
    wl.grid.nt = max(wl.grid.nt, nt_needed)
    return wl


def element_kernel_bytes(g, aniso=False):
    """Algorithmic bytes of one element-kernel launch: stress R+W (48),
    memory variables R+W (48 per mechanism), lambda+mu (8), tau (4, with
    attenuation), A,B,C (12, anisotropic) per element-local point and the
    velocity read (12) per unique point and simulation."""
    e = g.precision // 4
    S = g.batch
    per_loc = (48 + 48 * g.n_sls) * S + 8 + (4 if g.n_sls else 0) + (12 if aniso else 0)
    return (g.n_loc * per_loc + g.n_uni * 12 * S) * e


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_oracle_rate(wl, budget_s, max_steps=None, warm=2):
    """Time the oracle (CPU restatement) on the workload's first simulation:
    `warm` untimed steps, then steps until budget_s elapses."""
    import sesnt_oracle
    threads = sesnt_oracle.threads(os.cpu_count() or 1)
    o = sesnt_oracle.Oracle(wl.grid, 4)
    sesnt_oracle.load_workload(o, wl, sim=0)
    o.run(warm)
    n, t0 = 0, time.perf_counter()
    while True:
        o.run(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (max_steps and n >= max_steps):
            break
    o.close()
    return wl.grid.n_loc * n / el, n, el, threads


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def element_kernel_name(element, g):
    """The element kernel the library's launch rules pick for this grid and an
    --element choice other than tuned/columns (kernels.cuh:plan_element); a
    run reads the kernel it actually launched from the library."""
    import sesnt
    if g.flags & sesnt.FLAG_KAHAN_STRESS:  # compensated stress: staged (SLS, degrees 4-7) or point kernel
        return "k_element_stage" if g.n_sls > 0 and g.lpd >= 4 else "k_element"
    if element.startswith("columns"):
        if g.n_sls:
            return element_kernel_name("simple", g)
        if element.startswith("columns_pair"):
            return "k_element_cols2" if g.batch >= 2 and g.batch % 2 == 0 else element_kernel_name("simple", g)
        return "k_element_cols (staged stress)" if element.startswith("columns_staged") else "k_element_cols"
    if element.startswith("tc_"):
        return "k_element_tc"
    if element == "persistent":
        return "k_element_tma"
    if g.n_sls == 0 and g.batch >= 2 and g.batch % 2 == 0:
        return "k_element_pair"
    if g.n_sls > 0 and g.lpd >= 4 and element != "unstaged" and not (g.flags & sesnt.FLAG_STRAIN):
        return "k_element_stage"
    return "k_element"


def graph_launches(K, per_step):
    """Kernels a run of K steps launches: per_step per step, the step-counter
    set at the start, and one counter advance per replayed graph that ends
    before the run does (runs of 32 steps, then graphs of 16, 8, 4 and 2, the
    last single step without an advance; the rules of run_steps in
    sesnt_api.cu once a handle's graphs exist, as sesnt_run_timed makes sure)."""
    graphs, left = K // 32, K % 32
    for n in (16, 8, 4, 2):
        if left >= n:
            graphs += 1
            left -= n
    return int(K * per_step + 1 + graphs)


def run_ours(args):
    import numpy as np

    import sesnt
    import workloads

    K, W = args.steps, args.warmup
    KP = args.profile_steps
    wl = make_workload(args.workload, W + K + KP + 1, args.grid)
    g = wl.grid
    g.flags |= {"persistent": sesnt.FLAG_PERSISTENT_ELEMENT, "tc_tf32x3": sesnt.FLAG_TC_TF32X3,
                "tc_bf16x3": sesnt.FLAG_TC_BF16X3, "unstaged": sesnt.FLAG_NO_STAGE}.get(args.element, 0)
    if args.force64:
        g.flags |= sesnt.FLAG_FORCE64
    if args.kahan_stress:
        g.flags |= sesnt.FLAG_KAHAN_STRESS
    S = g.batch
    hbm, peak_kind = peaks()

    sim = sesnt.Simulation(g)
    workloads.setup(sim, wl)
    tune_report = choose_element(sim, args.element)
    kname, choice = sim.element_kernel()
    info = sim.info()
    aniso = False
    if W > 0:
        sim.run(1, W)
    sim.synchronize()

    barrier()
    clocks = Clocks(0)
    clocks.start()
    ms = sim.run_timed(W + 1, K)
    clk = clocks.stop()
    barrier()
    value, ms_max = aggregate(float(g.n_loc) * K * S, ms)

    # per-kernel event timing of the same step sequence (dominant kernel)
    prof = sim.run_profiled(W + K + 1, KP) if KP > 0 else None
    seis_ok = bool(np.isfinite(sim.seismograms()).all())
    sim.close()

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": WORLD, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if g.precision == 4 else "f64",
        "data": "synthetic: seeded (PCG64) gradient + 5% perturbation Earth model, per-element Q, "
                "moment-tensor Ricker source",
        "config": {"workload": wl.name, "elements": [g.nx, g.ny, g.nz], "lpd": g.lpd, "n_sls": g.n_sls,
                   "batch": S, "dt": g.dt, "n_loc": g.n_loc, "n_uni": g.n_uni,
                   "receivers": len(wl.receivers),
                   "algorithmic_bytes_per_step": info["algorithmic_bytes_per_step"],
                   "l2": "inputs larger than L2 (%.2f GB touched per step vs 0.13 GB L2)"
                         % (info["algorithmic_bytes_per_step"] / 1e9),
                   "graph": not (g.flags & sesnt.FLAG_NO_GRAPH), "element": args.element,
                   "force_assembly": "fp64" if args.force64 else "fp32",
                   "stress_integration": "compensated" if args.kahan_stress else "plain",
                   "element_kernel": {"name": kname, "variant": choice[0], "arg": choice[1], "piece": choice[2],
                                      "tuning": tune_report.strip().splitlines()[1:] if tune_report else None},
                   "parallelism": "replicas" if WORLD > 1 else "single GPU"},
        "gpu_launches": graph_launches(K, info["launches_per_step"]),
        "clocks": clk,
        "step_alg_hbm_gbs": info["algorithmic_bytes_per_step"] * K / (ms_max / 1e3) / 1e9,
        "finite": seis_ok,
    }
    if prof is not None:
        eb = element_kernel_bytes(g, aniso)
        t_el = float(prof[0]) / KP / 1e3
        ach = eb / t_el / 1e9
        prof = [float(x) for x in prof]
        line["kernels_ms_per_step"] = {"element": prof[0] / KP, "sources": prof[1] / KP, "node": prof[2] / KP,
                                       "receivers": prof[3] / KP}
        traffic = None
        tr_path = os.path.join(ROOT, "profiles", "%s_%s.traffic.json" % (kname.split()[0], wl.name))
        if os.path.exists(tr_path):
            try:
                with open(tr_path) as f:
                    tr = json.load(f)
                if tr.get("workload") == wl.name:
                    traffic = tr.get("dram_bytes_per_launch")
                    if "tensor_pipe_active_pct" in tr:
                        line["tensor_pipe_active_pct"] = tr["tensor_pipe_active_pct"]  # from the ncu capture
            except Exception:
                traffic = None
        line["roofline"] = {"bound": "hbm", "kernel": kname, "achieved": ach, "peak": hbm,
                            "peak_source": peak_kind, "unit": "GB/s", "frac": ach / hbm,
                            "traffic": traffic, "alg_bytes_per_launch": eb,
                            "traffic_source": ("stored ncu capture of this kernel and workload, "
                                               "profiles/" + os.path.basename(tr_path)) if traffic else None}
    if args.e2e and RANK == 0:
        line["e2e"] = e2e(args, wl)
    if args.accuracy_steps > 0 and RANK == 0:
        line["accuracy_vs_fp64"] = accuracy(args, wl)
    if args.batched and RANK == 0 and WORLD == 1 and args.workload == "config2" and not args.grid:
        line["batched"] = batched_headline(args)
    if RANK == 0 and WORLD == 1 and args.cpu_seconds > 0:
        rate, n, el, threads = cpu_oracle_rate(wl, args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": METRIC, "cores": threads, "kind": "port",
                                "sample": "%d time steps of the full %s grid (oracle, %d OpenMP threads, %.1f s)"
                                          % (n, wl.name, threads, el)}
    return line


def choose_element(sim, element):
    """Apply an --element choice that is not a grid flag: `tuned` runs the
    library's tuner on this grid (sesnt_tune, which also caches the choice
    for SESNT_FLAG_AUTOTUNE handles), `columns*` force a column kernel.
    Returns the tuning report or None."""
    import sesnt
    if element == "tuned":
        return sim.tune()
    if element.startswith("columns"):
        kind, _, arg = element.partition(":")
        v = {"columns": sesnt.ELEMENT_COLUMNS, "columns_staged": sesnt.ELEMENT_COLUMNS_STAGED,
             "columns_pair": sesnt.ELEMENT_COLUMNS_PAIR}[kind]
        sim.set_element_variant(v, int(arg or 0), 0)
    return None


def timed_rate(wl, K, W, KP=0, element="tuned"):
    """Steps of one workload: W untimed, K timed with CUDA events on the
    library's stream, then KP steps with per-kernel events. Returns
    (GLL-point-updates/s, ms/step, info, per-step ms of the element, source,
    node and receiver kernels or None, element kernel name)."""
    import sesnt
    import workloads
    g = wl.grid
    with sesnt.Simulation(g) as sim:
        workloads.setup(sim, wl)
        choose_element(sim, element)
        kname = sim.element_kernel()[0]
        info = sim.info()
        sim.run(1, W)
        sim.synchronize()
        ms = sim.run_timed(W + 1, K)
        prof = [float(x) / KP for x in sim.run_profiled(W + K + 1, KP)] if KP > 0 else None
    return g.n_loc * K * g.batch / (ms / 1e3), ms / K, info, prof, kname


def batched_headline(args):
    """The batched form against the plain one-source step on the same grid
    and model: 64 simulations (one per seeded source) in one handle, whose
    steps read the shared material, metric and mass once per element block,
    against one simulation. Three grids: the batched workload's own
    (64x64x32, lpd 4, 3 SLS), the plain workload's (12x12x8, lpd 4, elastic)
    and the served workload's smallest request (16x16x8, lpd 4, 3 SLS, 32
    sources). For
    each: the batched and plain rates, their ratio, the batched element
    kernel's algorithmic bytes over its event-timed duration as a fraction
    of the measured HBM bandwidth, and the whole step's algorithmic bytes over
    the step time as the same fraction. The target is at least 2x the plain
    rate at at least 0.7 of HBM."""
    import numpy as np
    import workloads
    hbm, peak_kind = peaks()
    out = {"peak_gbs": hbm, "peak_source": peak_kind, "target": {"vs_plain": 2.0, "hbm_frac": 0.7}}
    def config1_grid(nt):
        wl = workloads.config1(nt=nt)
        wl.grid.batch = 64
        wl.sources = workloads.random_sources(wl.grid, 64, np.random.Generator(np.random.PCG64(1)))
        return wl

    def smallest_request(nt):
        # the served workload's smallest request shape: 16x16 lateral and 8 radial elements,
        # lpd 4, 3 SLS, the config-2 model generator, its largest source count (32)
        wl = workloads.config4(nt=nt, batch=32, nx=16, ny=16, nz=8)
        wl.name = "served_smallest_request_32src_16x16x8_lpd4"
        return wl

    cases = (("config4_batched_64src_64x64x32_lpd4", lambda nt: workloads.config4(nt=nt), 4, 2, 3),
             ("config1_grid_batched_64src_12x12x8_lpd4", config1_grid, 100, 5, 10),
             ("served_smallest_request_32src_16x16x8_lpd4", smallest_request, 100, 5, 10))
    for name, make, K, W, KP in cases:
        nt = max(W + K + KP + 1, 416)
        wl = make(nt)
        rate, ms, info, prof, kname = timed_rate(wl, K, W, KP)
        t_el = prof[0]
        plain = copy.copy(wl)
        plain.grid = copy.copy(wl.grid)
        plain.grid.batch = 1
        plain.sources = [copy.copy(wl.sources[0])]
        plain.sources[0].sim = 0
        Kp = 40 if wl.grid.n_loc * wl.grid.batch > 1e9 else 400
        plain.grid.nt = max(plain.grid.nt, 5 + Kp + 1)
        prate, pms, pinfo, _, pname = timed_rate(plain, Kp, 5)
        eb = element_kernel_bytes(wl.grid)
        el_frac = eb / (t_el / 1e3) / 1e9 / hbm
        step_frac = info["algorithmic_bytes_per_step"] / (ms / 1e3) / 1e9 / hbm
        out[name] = {
            "batch": wl.grid.batch, "steps": K, "warmup": W, "ms_per_step": ms, "value": rate,
            "element_kernel": kname,
            "plain": {"ms_per_step": pms, "value": prate, "steps": Kp, "element_kernel": pname,
                      "l2": "inputs larger than L2" if pinfo["algorithmic_bytes_per_step"] > 129e6
                      else "%.0f MB per step: L2-resident, as in a real run (no flush)"
                           % (pinfo["algorithmic_bytes_per_step"] / 1e6)},
            "vs_plain": rate / prate,
            "element_kernel_ms": t_el, "element_kernel_hbm_frac": el_frac, "step_hbm_frac": step_frac,
            "node_kernel_ms": prof[2],
            # the replayed step's time outside the two kernels on its critical path (the source and
            # receiver kernels overlap them on a side stream): all that one persistent launch over
            # steps could remove
            "outside_kernels_frac": 1.0 - (prof[0] + prof[2]) / ms,
            "target_met": bool(rate / prate >= 2.0 and step_frac >= 0.7),
        }
    return out


def accuracy(args, wl):
    """FP32 (plain, Kahan-compensated velocity update, compensated stress
    integration, both, force assembled in FP64, tensor-core contractions) against
    the FP64 build of the same
    kernels: relative L2 of the seismograms of the first simulation and of
    its final vz after accuracy_steps steps."""
    import numpy as np

    import sesnt
    import workloads
    n = min(args.accuracy_steps, wl.grid.nt)
    res = {}
    for name, prec, flags in (("fp32", 4, 0), ("fp32_kahan", 4, sesnt.FLAG_KAHAN),
                              ("fp32_kahan_stress", 4, sesnt.FLAG_KAHAN_STRESS),
                              ("fp32_kahan_stress_and_v", 4, sesnt.FLAG_KAHAN_STRESS | sesnt.FLAG_KAHAN),
                              ("fp32_force64", 4, sesnt.FLAG_FORCE64),
                              ("fp32_tc_tf32x3", 4, sesnt.FLAG_TC_TF32X3),
                              ("fp32_tc_bf16x3", 4, sesnt.FLAG_TC_BF16X3), ("fp64", 8, 0)):
        w = copy.copy(wl)
        w.grid = copy.copy(wl.grid)
        w.grid.precision = prec
        w.grid.flags = flags
        w.grid.batch = 1
        w.sources = [s for s in wl.sources if s.sim == 0]
        with sesnt.Simulation(w.grid) as sim:
            workloads.setup(sim, w)
            sim.run(1, n)
            res[name] = (sim.seismograms()[0].astype(np.float64), sim.field("vz", precision=8))
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    out = {"steps": n}
    for name in ("fp32", "fp32_kahan", "fp32_kahan_stress", "fp32_kahan_stress_and_v", "fp32_force64",
                 "fp32_tc_tf32x3", "fp32_tc_bf16x3"):
        out[name] = {"seismogram_rel_l2": rel(res[name][0], res["fp64"][0]),
                     "vz_rel_l2": rel(res[name][1], res["fp64"][1])}
    return out


def e2e(args, wl, jobs=3):
    """The drop-in call pattern through the C ABI with host buffers: create,
    set_model from host arrays (H2D), register sources/receivers, then the K
    steps in runs of 32 (sesnt_run, graph replay) with every step's receiver
    samples read back to the host (one D2H read per step, sesnt_get_samples).
    The samples of a run are read while the next run executes: a read waits
    only for its own step. One untimed warm-up job, then the whole job runs
    `jobs` times; the value is the median job. (The first jobs of a process
    on a box that has just run other work spent 5-28 ms in the model upload
    against 1.6 ms later.)"""
    warm = e2e_job(args, wl)
    runs = [e2e_job(args, wl) for _ in range(jobs)]
    out = dict(sorted(runs, key=lambda r: r["seconds"])[len(runs) // 2])
    out["seconds_per_job"] = [r["seconds"] for r in runs]
    out["seconds_create_model_setup_steps_per_job"] = [r["seconds_create_model_setup_steps"] for r in runs]
    out["warmup_job_seconds"] = warm["seconds"]
    out["includes"] += "; one untimed warm-up job, then the median of %d jobs" % jobs
    return out


def e2e_job(args, wl):
    """One end-to-end job (see e2e)."""
    import numpy as np

    import sesnt
    import workloads
    K = args.steps
    g = wl.grid
    model_bytes = sum(int(np.asarray(v).nbytes) for v in wl.model.values())
    if args.element == "tuned":
        # a user's handle: the tuner's choice comes from the tuning cache that
        # the measured run's sesnt_tune wrote (SESNT_FLAG_AUTOTUNE)
        g = copy.copy(g)
        g.flags |= sesnt.FLAG_AUTOTUNE
        wl = workloads.Workload(wl.name, g, wl.model, wl.sources, wl.receivers)
    t0 = time.perf_counter()
    sim = sesnt.Simulation(g)
    t_create = time.perf_counter()
    m = wl.model
    sim.set_model(m["rhoinv"], m["lambda"], m["mu"], m.get("a"), m.get("b"), m.get("c"), m.get("q"))
    t_model = time.perf_counter()
    workloads.setup_sources_receivers(sim, wl)
    t_setup = time.perf_counter()
    buf = np.zeros((g.batch, len(wl.receivers), 3), np.float32)
    chunk, it, pending, reads = 32, 1, [], 0
    while it <= K or pending:
        if it <= K:
            n = min(chunk, K - it + 1)
            sim.run(it, n)
            pending.append((it, n))
            it += n
        if len(pending) > 1 or (it > K and pending):
            i0, n0 = pending.pop(0)
            for q in range(i0, i0 + n0):
                sim.samples(q, buf)
                reads += 1
    sim.synchronize()
    el = time.perf_counter() - t0
    sim.close()
    assert reads == K
    return {"value": g.n_loc * K * g.batch / el, "unit": METRIC,
            "h2d_bytes_per_step": model_bytes / K, "d2h_bytes_per_step": int(buf.nbytes),
            "seconds": el,
            "seconds_create_model_setup_steps": [t_create - t0, t_model - t_create, t_setup - t_model,
                                                 el - (t_setup - t0)],
            "includes": "handle create, model upload, source/receiver set-up, K steps in runs of 32, "
                        "a D2H read of every step's samples overlapping the next run"}


def run_served(args):
    """Served stream: seeded requests (own grid, degree, step count, model
    and 1..n sources) arriving as a Poisson process, served concurrently by
    the request server, against the plain path (every source of every request
    run alone, one after another). Sizes are the served workload's ranges
    scaled down (see `ranges`, set by --lateral, --radial, --step-range and
    --sources) so that the run ends in minutes."""
    import threading as _th

    import numpy as np

    import sesnt
    import workloads
    ranges = dict(lateral=tuple(args.lateral), radial=tuple(args.radial), lpds=(4, 6), steps=tuple(args.step_range),
                  sources=tuple(args.sources), receivers=16)
    stream = workloads.served_stream(args.requests, seed=5, **ranges)
    reqs = [workloads.request_of(w) for w in stream]
    hbm, peak_kind = peaks()

    def alg_bytes(w):
        g = w.grid
        per_step = g.n_loc * (48 + 48 * g.n_sls + 8 + 4) * g.batch + g.n_uni * (24 * g.batch + 4)
        return per_step * g.nt

    total_updates = sum(w.grid.n_loc * w.grid.nt * w.grid.batch for w in stream)
    total_bytes = sum(alg_bytes(w) for w in stream)
    # plain: one source at a time, one request after another
    t0 = time.perf_counter()
    for w in stream:
        for s in w.sources:
            g1 = copy.copy(w.grid)
            g1.batch = 1
            one = copy.copy(s)
            one.sim = 0
            with sesnt.Simulation(g1) as sim:
                workloads.setup(sim, workloads.Workload(w.name, g1, w.model, [one], w.receivers))
                sim.run(1, g1.nt)
                sim.seismograms()
    plain_s = time.perf_counter() - t0
    out = {"requests": len(stream), "ranges": {k: (list(v) if isinstance(v, tuple) else v) for k, v in ranges.items()},
           "total_updates": total_updates, "plain": {"seconds": plain_s, "value": total_updates / plain_s}}
    rng = np.random.default_rng(17)
    for rate in args.rates:
        gaps = rng.exponential(1.0 / rate, size=len(reqs))
        with sesnt.Server(max_active=args.max_active, chunk_steps=64, max_batch=0) as srv:
            ids = []

            def feed():
                for r, gap in zip(reqs, gaps):
                    time.sleep(gap)
                    ids.append(srv.submit(r))

            t0 = time.perf_counter()
            th = _th.Thread(target=feed)
            th.start()
            th.join()
            for rid in ids:
                srv.wait(rid, 3600.0)
            wall = time.perf_counter() - t0
            st = srv.stats()
        out["served_rate_%g" % rate] = {
            "arrival_rate_per_s": rate, "seconds": wall, "value": total_updates / wall,
            "vs_plain": plain_s / wall, "latency_p50_s": st["latency_p50"], "latency_p99_s": st["latency_p99"],
            "queue_wait_p50_s": st["queue_wait_p50"], "completed": st["completed"],
            "hbm_frac_of_measured": total_bytes / wall / 1e9 / hbm}
    return {"metric": METRIC + " (served stream)", "value": max(v["value"] for k, v in out.items()
                                                                 if k.startswith("served")),
            "unit": METRIC, "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic seeded request stream", "peak_source": peak_kind, "served": out}


def run_reference(args):
    """CPU implementation of the path on the host cores (the oracle's
    restatement of the Fortran reference), same workload and metric."""
    if RANK != 0:
        return None
    K, W = args.steps, args.warmup
    wl = make_workload(args.workload, W + K + 1, args.grid)
    budget = args.ref_seconds
    rate, n, el, threads = cpu_oracle_rate(wl, budget, max_steps=K, warm=min(W, 2))
    return {"impl": "reference", "metric": METRIC, "value": rate, "unit": METRIC, "n_gpus": WORLD, "steps": K,
            "warmup": W, "ms_per_step": el / n * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (same seeded workload as the GPU arm)",
            "config": {"workload": wl.name, "elements": [wl.grid.nx, wl.grid.ny, wl.grid.nz], "lpd": wl.grid.lpd,
                       "n_sls": wl.grid.n_sls},
            "cpu_baseline": {"value": rate, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": "%d of %d requested time steps of the full grid after %d warm-up steps "
                                       "(bounded to %.0f s); reference Fortran+MPI has no compiler here"
                                       % (n, K, min(W, 2), budget)},
            "e2e": {"value": rate, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2",
                    choices=["config1", "config2", "config3", "config4", "config4_plain", "config1_batch64",
                             "served"])
    ap.add_argument("--grid", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="elements of a smaller case of configs 2-4 (same generator and kernels), e.g. for ncu")
    ap.add_argument("--requests", type=int, default=40, help="served stream: number of requests")
    ap.add_argument("--rates", type=float, nargs="+", default=[2.0, 8.0], help="served stream: arrivals per second")
    ap.add_argument("--max-active", type=int, default=16, help="served stream: concurrent batches")
    ap.add_argument("--lateral", type=int, nargs=2, default=[16, 48], help="served stream: lateral elements")
    ap.add_argument("--radial", type=int, nargs=2, default=[8, 24], help="served stream: radial elements")
    ap.add_argument("--step-range", type=int, nargs=2, default=[300, 1500], help="served stream: steps")
    ap.add_argument("--sources", type=int, nargs=2, default=[1, 8], help="served stream: sources per request")
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--accuracy-steps", type=int, default=1500)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=60.0)
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--kahan-stress", action="store_true",
                    help="compensated stress integration (SESNT_FLAG_KAHAN_STRESS) in the measured run")
    ap.add_argument("--force64", action="store_true",
                    help="assemble the force in FP64 (SESNT_FLAG_FORCE64) in the measured run")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the batched-against-plain comparison of the default run")
    ap.add_argument("--element", default="tuned",
                    choices=["tuned", "simple", "persistent", "unstaged", "tc_tf32x3", "tc_bf16x3"] +
                            ["columns:%d" % q for q in range(16)] + ["columns_staged:%d" % q for q in range(16)] +
                            ["columns_pair:%d" % q for q in range(16)],
                    help="element kernel variant (all compute the full step): tuned = the library's tuner "
                         "picks on this grid; simple = the launch rules; tc_*: tcgen05 contractions")
    args = ap.parse_args()
    # the tuning cache of this run (sesnt_tune writes it, SESNT_FLAG_AUTOTUNE handles read it)
    import tempfile
    os.environ.setdefault("SESNT_TUNE_CACHE", os.path.join(tempfile.mkdtemp(prefix="sesnt_bench_"), "tune.txt"))
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        line = run_reference(args)
    elif args.workload == "served":
        line = run_served(args) if RANK == 0 else None
    else:
        line = run_ours(args)
    if RANK == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if _pg is not None:
        _pg.destroy_process_group()


if __name__ == "__main__":
    main()
