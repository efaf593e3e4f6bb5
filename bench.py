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
device-timed throughput with all fields resident in HBM; ``e2e`` is the same
step driven through the C ABI with the state copied host->device before and
device->host after every step.  The reference arm times the CPU oracle port
of the same step on a bounded sample of the workload, one process per host
core (the reference parallelises only over MPI ranks).
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
    ap.add_argument("--guess", default="learned", choices=["previous", "extrapolate", "learned"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-geometry", action="store_true", help="skip timing the device geometry set-up")
    ap.add_argument("--plain-steps", type=int, default=3, help="timed steps of the plain FP64 MG-CG variant")
    ap.add_argument("--prev-steps", type=int, default=3,
                    help="timed steps of mixed MG-CG with the previous-pressure guess (learned runs)")
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
def _cpu_sample_step(args):
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
    return time.perf_counter() - t


def cpu_sample_throughput(procs, nsteps=1):
    """Mcell-steps/s of `procs` concurrent oracle processes, each running
    `nsteps` steps of the SAMPLE-size version of the workload."""
    nx, ny, nz = SAMPLE
    nc = nx * ny * nz
    if procs == 1:
        dt = _cpu_sample_step((nx, ny, nz, nsteps))
        return nc * nsteps / dt / 1e6, dt
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        times = pool.map(_cpu_sample_step, [(nx, ny, nz, nsteps)] * procs)
        _ = time.perf_counter() - t0
    worst = max(times)
    return procs * nc * nsteps / worst / 1e6, worst


def run_reference(a, dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    procs = os.cpu_count() or 1
    for _ in range(a.warmup):
        cpu_sample_throughput(procs, 1)
    vals = []
    t0 = time.perf_counter()
    for _ in range(a.steps):
        v, _dt = cpu_sample_throughput(procs, 1)
        vals.append(v)
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    nx, ny, nz = SAMPLE
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * wall / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "turbidity current, 16 seeded Gaussian bumps, 2 fractions, Re=5000, dt=2.5e-4, "
                                   "sampled at %dx%dx%d per host process" % (nx, ny, nz)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "kind": "port", "host": host_cpu(),
                             "sample": "one step of the %dx%dx%d version of the workload in each of %d processes "
                                       "(the reference parallelises over MPI ranks only)" % (nx, ny, nz, procs)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def algorithmic_bytes(group, npts, nl_levels=None):
    """Algorithmic bytes of ONE launch of the group's kernel (each array read
    or written once per launch; status masks at 1 byte)."""
    if group == "jacobi":     # read x, b, status; write x_new
        return npts * (8 + 8 + 1 + 8)
    if group == "eno_yz":     # read q, advecting velocity, conv; write conv
        return npts * (8 + 8 + 8 + 8)
    if group == "eno_x":      # read q, advecting velocity; write conv
        return npts * (8 + 8 + 8)
    return None


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
    g = case.grid
    nc = g.nx * g.ny * g.nz
    npts = g.npts
    ctx = api.Context(g, case.params)
    ctx.load_state(case.state)
    ctx.set_pressure_mode(api.PMODE_MIXED if a.pmode == "mixed" else api.PMODE_FP64)
    guess = {"previous": api.GUESS_PREVIOUS, "extrapolate": api.GUESS_EXTRAPOLATE, "learned": api.GUESS_LEARNED}[a.guess]
    net = None
    if guess == api.GUESS_LEARNED:
        net = LN.attach(ctx, params)
        ctx.set_guess_stages(a.guess_stages)
    elif guess != api.GUESS_PREVIOUS:
        ctx.set_pressure_guess(guess)
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
    api.profile_enable(ctx, False)
    ms_max = dist.allmax(ms)
    value = dist.world * nc * a.steps / (ms_max / 1e3) / 1e6
    divmax = max(max(s["div_max"]) for s in stats)
    assert divmax <= 1e-10, "divergence gate failed: %g" % divmax
    # ---- mixed MG-CG with the previous-pressure guess (what the network adds) --
    mixed_prev = None
    if guess == api.GUESS_LEARNED and a.prev_steps > 0:
        ctx.set_pressure_guess(api.GUESS_PREVIOUS)
        ctx.step(dt)
        api.event_record(ctx, 4)
        mst = [ctx.step(dt) for _ in range(a.prev_steps)]
        api.event_record(ctx, 5)
        mms = dist.allmax(api.event_elapsed(ctx, 4, 5))
        mixed_prev = {"value": dist.world * nc * a.prev_steps / (mms / 1e3) / 1e6, "ms_per_step": mms / a.prev_steps,
                      "p_iters": [s["p_iters"] for s in mst], "steps": a.prev_steps}
        ctx.set_pressure_guess(guess)
    # ---- plain FP64 MG-CG on the same state --------------------------------
    plain = None
    if a.plain_steps > 0:
        ctx.set_pressure_mode(api.PMODE_FP64)
        ctx.set_pressure_guess(api.GUESS_PREVIOUS)   # the plain method: previous-pressure guess
        ctx.step(dt)
        api.event_record(ctx, 2)
        pst = [ctx.step(dt) for _ in range(a.plain_steps)]
        api.event_record(ctx, 3)
        pms = dist.allmax(api.event_elapsed(ctx, 2, 3))
        plain = {"value": dist.world * nc * a.plain_steps / (pms / 1e3) / 1e6, "ms_per_step": pms / a.plain_steps,
                 "p_iters": [s["p_iters"] for s in pst], "steps": a.plain_steps}
        ctx.set_pressure_mode(api.PMODE_MIXED if a.pmode == "mixed" else api.PMODE_FP64)
        ctx.set_pressure_guess(guess)
    # ---- end to end through the C ABI with host buffers ---------------------
    e2e = None
    if not a.no_e2e:
        keys = [("u", api.F_U), ("v", api.F_V), ("w", api.F_W), ("phi", api.F_PHI), ("dpx", api.F_DPX),
                ("dpy", api.F_DPY), ("dpz", api.F_DPZ)] + [("c%d" % i, api.F_C0 + i) for i in range(case.params.nconc)]
        # the step's inputs and outputs in page-locked host memory
        host = {}
        for (k, f), buf in zip(keys, pinned):
            host[k] = buf
            ctx.download_many([(f, host[k])])
        ne = max(1, min(a.steps, 3))
        pairs = [(f, host[k]) for k, f in keys]
        # one untimed round first: the pressure mode switched back after the
        # plain FP64 steps, and its graphs are captured again on first use
        ctx.upload_many(pairs)
        ctx.step(dt)
        ctx.download_many(pairs)
        dist.barrier()
        t0 = time.perf_counter()
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
        ctx.synchronize()
        te = dist.allmax(time.perf_counter() - t0)
        nbytes = sum(arr.nbytes for arr in host.values())
        e2e = {"value": dist.world * nc * ne / te / 1e6, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": ne,
               "ms_per_step": {"upload": 1e3 * tu / ne, "step": 1e3 * ts / ne, "download": 1e3 * td / ne}}
    # ---- roofline of the dominant kernel group -----------------------------
    peak, peak_src = hbm_peak()
    dom = max(("jacobi", "eno_yz", "eno_x"), key=lambda k: prof[k][0])
    gms, gnl = prof[dom]
    bpl = algorithmic_bytes(dom, npts)
    ach = bpl / (gms / gnl / 1e3) / 1e9 if gnl else None
    # DRAM traffic per launch of the ENO y/z pass from one ncu capture of a
    # y pass at 256x128x128 (dram__bytes_read.sum + dram__bytes_write.sum =
    # 68.73 MB + 0.89 MB for 257*129*129 points), scaled by the points of a
    # launch here; at that size the conv writes still sat in L2 when the
    # kernel ended, so the figure counts reads
    traffic = (68.734720e6 + 0.888064e6) / (257 * 129 * 129) * npts if dom == "eno_yz" else None
    roof = {"bound": "hbm", "kernel_group": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": (ach / peak) if ach else None, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "traffic_source": "ncu, one y pass at 256x128x128, scaled by points"
            if traffic else None, "bytes_per_launch": bpl, "launches": gnl, "ms_per_launch": gms / gnl if gnl else None,
            "groups_ms": {k: v[0] for k, v in prof.items()}, "groups_launches": {k: v[1] for k, v in prof.items()}}
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
    # the immersed-boundary set-up of the same bed on the device (reference
    # level-set reinitialisation, statuses, ghost-cell stencils), timed once
    # after the steps; the stepped case keeps its own geometry
    geom = None
    if not a.no_geometry:
        from turbins_gb300 import geometry as GM
        r = GM.device_geometry(g, case.params, GM.bed_heights(g, case.bed), apply=False, ctx=ctx)
        geom = {"seconds": r["seconds"], "reinit_steps": r["steps"],
                "ib_nodes": {q: int(r["stencils"][q]["n"]) for q in "uvwc"}}
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not a.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        v, dtc = cpu_sample_throughput(1, 1)
        nx, ny, nz = SAMPLE
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "host": host_cpu(),
               "sample": "one TVD-RK2 step of the %dx%dx%d version of the same workload (%.1f s)" % (nx, ny, nz, dtc)}
    if dist.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded workload generator)",
                "config": {"workload": "turbidity current %dx%dx%d y-stretched (tanh 1.5), 16 seeded Gaussian bumps "
                                       "(immersed), 2 fractions (Vs 0.005, 0.02), Re=5000, dt=2.5e-4, ENO-3"
                                       % (a.nx, a.ny, a.nz),
                           "pressure": "%s MG-CG (FP64 CG, %s V-cycles), rtol 1e-10" % (
                               a.pmode, "FP32" if a.pmode == "mixed" else "FP64"),
                           "learned_warm_start": a.guess == "learned", "pressure_guess": a.guess,
                           "l2": "inputs larger than L2: each FP64 field is %.0f MB" % (npts * 8 / 1e6),
                           "parallelism": "replicas" if dist.world > 1 else "single GPU"},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "plain_fp64": plain, "mixed_previous_guess": mixed_prev, "learned": learned_info,
                "geometry_setup": geom,
                "solver": {"p_iters": [s["p_iters"] for s in stats], "guess_tried_taken": ctx.pressure_guess_stats(),
                           "vel_iters": stats[-1]["vel_iters"],
                           "conc_iters": stats[-1]["conc_iters"], "div_max": divmax}}
        print(json.dumps(line))
    ctx.close()
    if net is not None:
        net.close()
    dist.close()


if __name__ == "__main__":
    main()
