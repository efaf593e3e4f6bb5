#!/usr/bin/env python
"""Benchmark of the TURBINS fractional-step hot path on GB300.

Metric: Mcell-steps/s of the full coupled TVD-RK2 step (ENO convection of
u, v, w and two sediment fractions, implicit viscous/diffusive solves with
immersed-boundary rows, pressure Poisson solve + projection) on the
512x256x256 y-stretched turbidity current over 16 seeded Gaussian bumps,
Re=5000, dt=2.5e-4, every step checked to max|div u| <= 1e-10.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs independent replicas (the step has no exchange between GPUs),
one rank per GPU, and reports the aggregate over ranks.  ``value`` is the
device-timed throughput with all fields resident in HBM (steps 4-13); ``e2e``
is the same step driven through the C ABI with the state copied host->device
before and device->host after every step (turb_step_host), and the arms time
the guess and precision methods in turn; both start again from the initial
state, so that every timed step lies within the first 20 (on this bed the
reference's immersed-boundary stencils let a spanwise-velocity mode grow from
about step 25 at 512x256x256, in the oracle as on the GPU).  The reference arm times the CPU oracle port
of the same step on the whole grid, split into one x-slab per host core,
each stepped in its own process (the reference parallelises only over MPI
ranks), for at most about 4 minutes of timed steps.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s at 512x256x256 (div≤1e-10): learned+mixed vs plain FP64 MG-CG"
UNIT = "Mcell-steps/s"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
HBM_FALLBACK = 6800.0
SAMPLE = (128, 64, 64)   # bounded CPU sample of the same workload


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--pmode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--guess", default="learned", choices=["previous", "extrapolate", "learned", "project"])
    ap.add_argument("--galerkin", type=int, default=1,
                    help="learned guess: fit the network candidate together with the stage's last two solutions")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--kv", type=int, default=None,
                    help="kernel variants (turb_set_sweep_kernels flags; default: the library's)")
    ap.add_argument("--host-copy", default=None, choices=["dma", "kernel"],
                    help="how page-locked host arrays move in the e2e leg (turb_set_host_copy; default: the library's)")
    ap.add_argument("--mg-sweeps", default=None,
                    help="red-black sweeps (pre = post) of the mixed V-cycle: finest,next,coarser (e.g. 4,5,12)")
    ap.add_argument("--mg-cluster", type=int, default=None,
                    help="one-cluster V-cycle from the first level of at most this many cells (turb_set_mg_cluster)")
    ap.add_argument("--analytic-geometry", action="store_true",
                    help="keep the analytic-sdf immersed geometry instead of the reference construction")
    ap.add_argument("--cmp-steps", type=int, default=5,
                    help="rounds of one step per arm (learned, previous guess, plain FP64) timed in turn")
    ap.add_argument("--poisson-rhs", type=int, default=16,
                    help="Fourier right-hand sides per grid for the Poisson-alone comparison (0: skip)")
    ap.add_argument("--train-seeds", type=int, default=8, help="learned guess: training runs (one bump field each)")
    ap.add_argument("--train-steps", type=int, default=125, help="learned guess: steps per training run")
    ap.add_argument("--guess-stages", type=int, default=2,
                    help="learned guess: RK stages that try it (bit 0 first, bit 1 second)")
    ap.add_argument("--train-iters", type=int, default=3000, help="learned guess: Adam steps")
    ap.add_argument("--net-params", default=None, help="learned guess: .npy parameters instead of training")
    ap.add_argument("--save-net-params", default=None, help="learned guess: write the trained parameters (.npy)")
    return ap.parse_args()


class Dist:
    """Minimal torch.distributed wrapper (gloo: barrier + max/sum on host)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.td = td
            self.pg = True

    def barrier(self):
        if self.pg:
            self.td.barrier()

    def allmax(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


def bf16_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops)"
    except Exception:
        return 1900.0, "fallback"


def host_cpu():
    """the host's core count and CPU model (model name, or the Arm part
    number, from /proc/cpuinfo)"""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read().splitlines()
        for key in ("model name", "CPU part"):
            for line in info:
                if line.lower().startswith(key.lower()):
                    model = line.split(":", 1)[1].strip()
                    break
            if model:
                break
    except OSError:
        pass
    arm = {"0xd4f": "Arm Neoverse-V2", "0xd40": "Arm Neoverse-V1", "0xd0c": "Arm Neoverse-N1"}
    if model in arm:
        model = "%s (CPU part %s)" % (arm[model], model)
    return {"nproc": os.cpu_count(), "model": model}


def hbm_peak():
    try:
        with open(PEAKS) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.p = None
        # raw samples: $TURB_CLOCKS_DIR if set, else the system's temporary directory
        self.path = os.path.join(os.environ.get("TURB_CLOCKS_DIR", tempfile.gettempdir()),
                                 "clocks_bench_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.p is None:
            return out
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for ln in open(self.path):
                f = [x.strip() for x in ln.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        except OSError:
            pass
        if sm:
            out.update(sm_mhz=float(np.median(sm)), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


# ---------------------------------------------------------------------------
# CPU legs (the oracle port of the same step; never part of the GPU path)
# ---------------------------------------------------------------------------
def _cpu_sample_step(args, keep=False):
    nx, ny, nz, nsteps = args
    from oracle.oracle import Oracle
    from turbins_gb300 import workload as W
    case = W.multi_bump_case(nx, ny, nz)
    o = Oracle(case.grid, case.params)
    s = {k: v.copy() for k, v in case.state.items()}
    o.step(s, case.dt)            # warm the caches / first-touch
    t = time.perf_counter()
    for _ in range(nsteps):
        o.step(s, case.dt)
    el = time.perf_counter() - t
    return (el, s) if keep else el


def cpu_sample_throughput(procs, nsteps=1, keep=None):
    """Mcell-steps/s of `procs` concurrent oracle processes, each running
    `nsteps` steps of the SAMPLE-size version of the workload (after one
    untimed step).  keep (procs == 1): a dict that receives the final state."""
    nx, ny, nz = SAMPLE
    nc = nx * ny * nz
    if procs == 1:
        dt, s = _cpu_sample_step((nx, ny, nz, nsteps), keep=True)
        if keep is not None:
            keep.update(s)
        return nc * nsteps / dt / 1e6, dt
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        times = pool.map(_cpu_sample_step, [(nx, ny, nz, nsteps)] * procs)
        _ = time.perf_counter() - t0
    worst = max(times)
    return procs * nc * nsteps / worst / 1e6, worst


def _slab_worker(conn, nx, ny, nz, nslab, slab):
    """one host process of the reference arm: the slab `slab` of `nslab`
    x-slabs of the nx x ny x nz workload (its own x extent, the full y and z,
    the full case's spacing), one untimed step for first touch, then one
    oracle step per request, replying with the step's wall time"""
    from oracle.oracle import Oracle
    from turbins_gb300 import workload as W
    sx = nx // nslab
    case = W.multi_bump_case(sx, ny, nz, seed=4 + slab, lx=32.0 * sx / 512.0,
                             nbump=max(1, int(round(16.0 * sx / 512.0))))
    o = Oracle(case.grid, case.params)
    s = {k: v.copy() for k, v in case.state.items()}
    o.step(s, case.dt)
    conn.send(("ready", sx * ny * nz))
    while True:
        msg = conn.recv()
        if msg != "step":
            break
        t = time.perf_counter()
        o.step(s, case.dt)
        conn.send(("done", time.perf_counter() - t))
    conn.close()


def run_reference(a, dist):
    """The CPU path of the reference on the headline grid: the 512x256x256
    workload decomposed into one x-slab per host core, as the reference runs
    over MPI ranks (each rank its sub-domain, single-threaded), every slab
    stepped by the oracle port in its own process.  No halo exchange is
    timed, so this favours the CPU.  A step's time is the slowest slab's."""
    if dist.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    procs = os.cpu_count() or 1
    nslab = max(d for d in (1, 2, 4, 8, 16, 32, 64) if d <= procs and (a.nx // d) % 8 == 0)
    ctx = mp.get_context("spawn")
    pipes, workers = [], []
    for i in range(nslab):
        here, there = ctx.Pipe()
        w = ctx.Process(target=_slab_worker, args=(there, a.nx, a.ny, a.nz, nslab, i), daemon=True)
        w.start()
        pipes.append(here)
        workers.append(w)
    cells = sum(pp.recv()[1] for pp in pipes)
    def step():
        for pp in pipes:
            pp.send("step")
        return max(pp.recv()[1] for pp in pipes)
    for _ in range(min(a.warmup, 1)):    # the workers' first-touch step already ran
        step()
    # a bounded sample: the timed steps stop once about 4 minutes have gone
    t0 = time.perf_counter()
    times = []
    while len(times) < a.steps and (not times or time.perf_counter() - t0 < 240.0):
        times.append(step())
    wall = time.perf_counter() - t0
    for pp in pipes:
        pp.send("stop")
    for w in workers:
        w.join(10)
    v = cells * len(times) / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": len(times),
            "steps_requested": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * wall / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "turbidity current %dx%dx%d y-stretched (tanh 1.5), seeded Gaussian bumps "
                                   "(immersed), 2 fractions (Vs 0.005, 0.02), Re=5000, dt=2.5e-4, ENO-3"
                                   % (a.nx, a.ny, a.nz),
                       "decomposition": "%d x-slabs of %dx%dx%d, one host process each" % (
                           nslab, a.nx // nslab, a.ny, a.nz)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nslab, "kind": "port", "host": host_cpu(),
                             "sample": "every step of the whole %dx%dx%d grid, split into %d x-slabs stepped "
                                       "in parallel processes without halo exchange (the reference "
                                       "parallelises over MPI ranks only)" % (a.nx, a.ny, a.nz, nslab)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
# FP64-pipe instructions per DA point of one launch of the group's kernel:
# ncu's sm__pipe_fp64_cycles_active share x launch duration x the DFMA rate
# measured here, divided by the launch's points, on single launches at
# 256x128x128 (profiles/fp64_pipe_multi_bump_256x128x128.md); this counts the
# compares and moves the FP64 pipe executes besides DADD / DMUL / DFMA.  A
# pass advected by a bilinear transpose of another velocity costs 21.4
# (y / z) or 21.8 (x) per point, a self-advected one 15.0; a step's passes
# mix them 4:6 (y / z) and 2:3 (x).  The jacobi group's kernel is the FP64
# Helmholtz residual.  Since that capture the y passes divide by the
# stretched y spacings with the two-term quotient alone (every y spacing of
# this workload passes the set-up's check): 3 divisions x 2 DFMA fewer per
# point in half of the y / z launches, 17.6 - 3.0.
FP64_OPS = {"eno_yz": 14.6, "eno_x": 17.7, "jacobi": 12.1}

# DRAM bytes of one V-cycle of the mixed method at 512x256x256 (all its
# kernels, dram__bytes_read.sum + dram__bytes_write.sum, one ncu pass;
# profiles/vcycle_dram_multi_bump_512x256x256.md): 7.18 GB over its 198
# launches, against 8.42 GB of algorithmic bytes (the coarse levels stay in
# L2).  Per launch, as the roofline's traffic of the mg group.
MG_TRAFFIC_PER_LAUNCH = 7.18e9 / 198


def step_arm(ctx, api, dt, mode, guess, guess_stages=None):
    """one step of an arm, timed with events on the context stream"""
    ctx.set_pressure_mode(mode)
    ctx.set_pressure_guess(guess)
    if guess_stages is not None:
        ctx.set_guess_stages(guess_stages)
    api.event_record(ctx, 2)
    st = ctx.step(dt)
    api.event_record(ctx, 3)
    return api.event_elapsed(ctx, 2, 3), st


def group_table(prof, pbytes, peak_hbm, fp64_rate, npts, ncell):
    """per kernel group: event ms, launches, algorithmic GB, GB/s and the
    fraction of the HBM peak; for FP64-bound groups with measured op counts,
    the fraction of the FP64 pipe rate"""
    out = {}
    for g_, (ms, nl) in prof.items():
        gb = pbytes.get(g_, 0.0) / 1e9
        row = {"ms": ms, "launches": nl, "gbytes": gb}
        if ms > 0 and gb > 0:
            row["gbs"] = gb / (ms / 1e3)
            row["hbm_frac"] = row["gbs"] / peak_hbm
        ops = FP64_OPS.get(g_)
        if ops and ms > 0 and fp64_rate:
            # every launch of these groups is one pass over the DA points
            row["fp64_frac"] = ops * npts * nl / (ms / 1e3) / fp64_rate
        out[g_] = row
    return out


def main():
    a = parse()
    dist = Dist()
    if dist.world > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(dist.local)
    if a.impl == "reference":
        run_reference(a, dist)
        dist.close()
        return
    from turbins_gb300 import api, build
    from turbins_gb300 import workload as W
    build.build()
    # the end-to-end arm's host buffers (7 flow fields + 2 fractions), page-
    # locked at start-up as an application allocates its I/O buffers
    pinned = [] if a.no_e2e else [api.host_empty((a.nz + 1, a.ny + 1, a.nx + 1)) for _ in range(9)]
    learned_info, params = None, None
    if a.guess == "learned":
        from turbins_gb300 import learned as LN
        if a.net_params:
            params = np.load(a.net_params)
            learned_info = {"params": os.path.basename(a.net_params)}
        else:
            # training domains at the full case's grid spacing: a quarter of
            # its x and z extents, the whole height (8 x 125 steps = 2000
            # solves of snapshots)
            tn = (max(16, a.nx // 4), a.ny, max(16, a.nz // 4))
            params, learned_info = LN.train_default(LN.multi_bump_train_case(*tn, full=(a.nx, a.ny, a.nz)),
                                                    seeds=a.train_seeds, steps=a.train_steps, iters=a.train_iters)
            learned_info["train_grid"] = list(tn)
            if a.save_net_params:
                np.save(a.save_net_params, params)
        learned_info["guess_stages"] = a.guess_stages
    case = W.multi_bump_case(a.nx, a.ny, a.nz)
    # the immersed-boundary geometry of the reference's own construction
    # (level-set reinitialised sdf, Immersed.c stencils), built on the GPU
    geom = None
    if not a.analytic_geometry:
        from turbins_gb300 import geometry as GM
        geom = GM.reference_geometry(case)
    g = case.grid
    nc = g.nx * g.ny * g.nz
    npts = g.npts
    ctx = api.Context(g, case.params)
    ctx.load_state(case.state)
    # every Poisson solve of every arm also reaches max|div u| <= 1e-10 after
    # the projection (the metric's gate), not only its relative residual
    ctx.set_divergence_gate(1e-10)
    if a.kv is not None:
        ctx.set_sweep_kernels(a.kv)
    if a.mg_cluster is not None:
        ctx.set_mg_cluster(a.mg_cluster)
    if a.mg_sweeps is not None:
        s0, s1, s2 = (int(v) for v in a.mg_sweeps.split(","))
        ctx.set_pressure_mode(api.PMODE_MIXED)
        ctx.set_mg_sweeps(s0, s0)
        ctx.set_mg_coarse_sweeps(1, s1, s1)
        ctx.set_mg_coarse_sweeps(2, s2, s2)
    if a.host_copy is not None:
        ctx.set_host_copy(api.HOST_COPY_DMA if a.host_copy == "dma" else api.HOST_COPY_KERNEL)
    pmode = api.PMODE_MIXED if a.pmode == "mixed" else api.PMODE_FP64
    ctx.set_pressure_mode(pmode)
    guess = {"previous": api.GUESS_PREVIOUS, "extrapolate": api.GUESS_EXTRAPOLATE, "learned": api.GUESS_LEARNED,
             "project": api.GUESS_PROJECT}[a.guess]
    net = None
    if guess == api.GUESS_LEARNED:
        net = LN.attach(ctx, params)
        ctx.set_guess_stages(a.guess_stages)
        ctx.set_guess_galerkin(a.galerkin)
    elif guess != api.GUESS_PREVIOUS:
        ctx.set_pressure_guess(guess)
    fp64_rate = api.measure_fp64_rate()
    dt = case.dt
    for _ in range(a.warmup):
        ctx.step(dt)
    # ---- timed region: device-resident state --------------------------------
    clocks = Clocks(0 if dist.world == 1 else dist.local)
    api.profile_enable(ctx, True)
    l0 = api.kernel_launches(ctx)
    dist.barrier()
    ctx.synchronize()
    clocks.start()
    api.event_record(ctx, 0)
    stats = []
    for _ in range(a.steps):
        stats.append(ctx.step(dt))
    api.event_record(ctx, 1)
    ctx.synchronize()
    ms = api.event_elapsed(ctx, 0, 1)
    clk = clocks.stop()
    dist.barrier()
    launches = api.kernel_launches(ctx) - l0
    prof = api.profile_read(ctx)
    pbytes = api.profile_bytes(ctx)
    api.profile_enable(ctx, False)
    ms_max = dist.allmax(ms)
    value = dist.world * nc * a.steps / (ms_max / 1e3) / 1e6
    divmax = max(max(s["div_max"]) for s in stats)
    assert divmax <= 1e-10, "divergence gate failed: %g" % divmax
    # The later legs start again from the initial state: on this bed the
    # reference's immersed-boundary stencils let a spanwise-velocity mode grow
    # from about step 25 at 512x256x256 (the oracle shows the same growth on
    # the same stencils), so every timed leg stays within the first 20 steps.
    def restart():
        ctx.load_state(case.state)
        ctx.reset_pressure_history()

    # ---- end to end through the C ABI with host buffers ---------------------
    e2e = None
    if not a.no_e2e:
        restart()
        keys = [("u", api.F_U), ("v", api.F_V), ("w", api.F_W), ("phi", api.F_PHI), ("dpx", api.F_DPX),
                ("dpy", api.F_DPY), ("dpz", api.F_DPZ)] + [("c%d" % i, api.F_C0 + i) for i in range(case.params.nconc)]
        # the step's inputs and outputs in page-locked host memory
        host = {}
        for (k, f), buf in zip(keys, pinned):
            host[k] = buf
            ctx.download_many([(f, host[k])])
        ne = max(1, min(a.steps, 3))
        pairs = [(f, host[k]) for k, f in keys]
        # one untimed round first
        ctx.upload_many(pairs)
        ctx.step(dt)
        ctx.download_many(pairs)
        ctx.step_host(dt, pairs)
        dist.barrier()
        # one call per step: the state up, the step, the state down
        # (turb_step_host: the late fields' copies overlap the step)
        t0 = time.perf_counter()
        for _ in range(ne):
            ctx.step_host(dt, pairs)
        ctx.synchronize()
        te = dist.allmax(time.perf_counter() - t0)
        # the same as three calls in turn, for the breakdown
        tu = ts = td = 0.0
        for _ in range(ne):
            t1 = time.perf_counter()
            ctx.upload_many(pairs)
            t2 = time.perf_counter()
            ctx.step(dt)
            ctx.synchronize()
            t3 = time.perf_counter()
            ctx.download_many(pairs)
            t4 = time.perf_counter()
            tu, ts, td = tu + t2 - t1, ts + t3 - t2, td + t4 - t3
        nbytes = sum(arr.nbytes for arr in host.values())
        e2e = {"value": dist.world * nc * ne / te / 1e6, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": ne, "call": "turb_step_host",
               "ms_per_step": 1e3 * te / ne,
               "separate_calls_ms_per_step": {"upload": 1e3 * tu / ne, "step": 1e3 * ts / ne,
                                              "download": 1e3 * td / ne}}
    # ---- the arms side by side: one step of each in turn, cmp_steps rounds --
    arms = [("mixed_previous_guess", api.PMODE_MIXED, api.GUESS_PREVIOUS, None),
            ("mixed_projection_guess", api.PMODE_MIXED, api.GUESS_PROJECT, 3),
            ("plain_fp64", api.PMODE_FP64, api.GUESS_PREVIOUS, None)]
    if guess == api.GUESS_LEARNED:
        arms.insert(0, ("learned_mixed", api.PMODE_MIXED, api.GUESS_LEARNED, a.guess_stages))
    cmp = {}
    if a.cmp_steps > 0:
        restart()
        for nm, md, gs, stg in arms:            # each arm once untimed (graphs of its mode)
            step_arm(ctx, api, dt, md, gs, stg)
        restart()                               # the rounds then cover steps 1-20
        rec = {nm: [] for nm, _, _, _ in arms}
        failed = {}
        for rnd in range(a.cmp_steps):
            for nm, md, gs, stg in arms:
                if nm in failed:
                    continue
                try:
                    rec[nm].append(step_arm(ctx, api, dt, md, gs, stg))
                except api.TurbError as e:   # the arm stops; the others go on from the state it left
                    failed[nm] = {"round": rnd, "error": str(e), "stats": getattr(e, "stats", None)}
                    print("arm %s failed in round %d: %s %s" % (nm, rnd, e, failed[nm]["stats"]), file=sys.stderr)
        for nm, info in failed.items():
            cmp[nm] = {"failed": info, "steps": len(rec[nm])}
        for nm, lst in rec.items():
            if nm in failed or not lst:
                continue
            t = dist.allmax(sum(x[0] for x in lst))
            cmp[nm] = {"value": dist.world * nc * len(lst) / (t / 1e3) / 1e6, "ms_per_step": t / len(lst),
                       "steps": len(lst), "p_iters": [x[1]["p_iters"] for x in lst],
                       "div_max": max(max(x[1]["div_max"]) for x in lst)}
            assert cmp[nm]["div_max"] <= 1e-10, (nm, cmp[nm]["div_max"])
        ctx.set_pressure_mode(pmode)
        ctx.set_pressure_guess(guess)
        if guess == api.GUESS_LEARNED:
            ctx.set_guess_stages(a.guess_stages)
    # ---- roofline: every group, and the dominant one -------------------------
    peak, peak_src = hbm_peak()
    groups = group_table(prof, pbytes, peak, fp64_rate, npts, nc)
    dom = max(groups, key=lambda k: groups[k]["ms"])
    d = groups[dom]
    roof = {"bound": "tensor" if dom == "net" else "hbm", "kernel_group": dom,
            "achieved": d.get("gbs"), "peak": peak, "unit": "GB/s", "frac": d.get("hbm_frac"),
            "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_src,
            "traffic": MG_TRAFFIC_PER_LAUNCH if dom == "mg" and (a.nx, a.ny, a.nz) == (512, 256, 256) else None,
            "traffic_source": "ncu dram bytes of one V-cycle at 512x256x256, per launch" if dom == "mg" else None,
            "algorithmic_bytes_per_launch": pbytes.get(dom, 0.0) / max(d["launches"], 1),
            "ms_per_launch": d["ms"] / max(d["launches"], 1), "launches": d["launches"],
            "fp64_rate_dfma_per_s": fp64_rate, "groups": groups}
    if learned_info is not None and prof["net"][1]:
        # the network's tensor-core work: 2 * 27 * cin * cout FLOP per voxel and conv
        # (25920 MAC per finest cell over the 11 convolutions), per guess
        nguess = prof["net"][1] / 26.0
        flops = 2.0 * 25920 * nc
        net_ms = prof["net"][0] / nguess
        learned_info.update({"guesses": nguess, "guess_ms": net_ms, "forward_tflop": flops / 1e12,
                             "tensor_tflops": flops / (net_ms / 1e3) / 1e12,
                             "frac_of_bf16_peak": flops / (net_ms / 1e3) / 1e12 / bf16_peak()[0],
                             "bf16_peak_source": bf16_peak()[1],
                             "guess_residual_ratio": ctx.pressure_guess_ratio()})
    gate_n = ctx.divergence_gate_count()
    gate_floor = ctx.divergence_gate_floor_count()
    ctx.close()
    if net is not None:
        net.close()
    # ---- pressure solves alone: mixed vs plain FP64 on Fourier divergences --
    poisson = None
    if a.poisson_rhs > 0 and dist.rank == 0:
        from turbins_gb300 import poisson as PS
        poisson = {}
        for nm, ((px, py, pz), lens, q) in PS.SHAPES.items():
            recs = PS.solve_set(W.poisson_case(px, py, pz, lens, q), range(a.poisson_rhs))
            poisson[nm] = PS.summary(recs)
    # ---- CPU baseline, and the GPU on the same sample from the same state ---
    cpu, parity = None, None
    if dist.rank == 0 and dist.world == 1 and not a.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        ref = {}
        v, dtc = cpu_sample_throughput(1, 1, keep=ref)
        sx, sy, sz = SAMPLE
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "host": host_cpu(),
               "sample": "one TVD-RK2 step of the %dx%dx%d version of the same workload (%.1f s)" % (sx, sy, sz, dtc)}
        sc = W.multi_bump_case(sx, sy, sz)
        sctx = api.Context(sc.grid, sc.params)
        sctx.set_pressure_mode(api.PMODE_MIXED)
        sctx.load_state(sc.state)
        for _ in range(2):               # the oracle's untimed and timed steps
            sctx.step(sc.dt)
        got = sctx.state()
        sctx.close()
        vsc = max(np.abs(ref[k]).max() for k in "uvw")
        parity = {"sample": "%dx%dx%d, 2 steps from the same state" % (sx, sy, sz),
                  "max_abs_diff_rel": {k: float(np.abs(got[k] - ref[k]).max() / (vsc if k in "uvw" else
                                                                                    max(np.abs(ref[k]).max(), 1.0)))
                                       for k in ["u", "v", "w"] + ["c%d" % i for i in range(sc.params.nconc)]}}
    if dist.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded workload generator)",
                "config": {"workload": "turbidity current %dx%dx%d y-stretched (tanh 1.5), 16 seeded Gaussian bumps "
                                       "(immersed), 2 fractions (Vs 0.005, 0.02), Re=5000, dt=2.5e-4, ENO-3"
                                       % (a.nx, a.ny, a.nz),
                           "geometry": "analytic sdf" if geom is None else
                                       "reference construction on the GPU (level-set sdf, Immersed.c stencils)",
                           "pressure": "%s MG-CG (FP64 CG, %s V-cycles), rtol 1e-10" % (
                               a.pmode, "FP32" if a.pmode == "mixed" else "FP64"),
                           "learned_warm_start": a.guess == "learned", "pressure_guess": a.guess,
                           "guess_galerkin": bool(a.galerkin) if a.guess == "learned" else None,
                           "divergence_gate": 1e-10,
                           "l2": "inputs larger than L2: each FP64 field is %.0f MB" % (npts * 8 / 1e6),
                           "parallelism": "replicas" if dist.world > 1 else "single GPU"},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "arms": cmp, "plain_fp64": cmp.get("plain_fp64"),
                "mixed_previous_guess": cmp.get("mixed_previous_guess"), "learned": learned_info,
                "geometry_setup": geom, "poisson_alone": poisson, "parity": parity,
                "solver": {"p_iters": [s["p_iters"] for s in stats], "vel_iters": stats[-1]["vel_iters"],
                           "gate_tightened": gate_n, "gate_at_floor": gate_floor,
                           "conc_iters": stats[-1]["conc_iters"], "div_max": divmax}}
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()
