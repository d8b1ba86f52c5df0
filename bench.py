"""Benchmark of the GB300 FDTD engine.

Workload (N = 1): the 2-D elastic P-SV batch -- 1000 x 3000 cells at 5 m,
40-cell CPML (43 padded cells per face as in the reference), 16 shots,
4000 steps, Ricker 12 Hz explosive sources, 601 vx/vz receivers per shot.
One bench step is one full forward modelling of the batch (update!(pa)).

  value  Gcell-updates/s with all inputs resident on the GPU (gpi_run only)
  e2e    the same metric through the public API with host buffers: upload
         of the medium and wavelets, the run, download of all records
  roofline  algorithmic bytes (60 B per cell update) / kernel time against
         the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (C restatement of the reference, OpenMP on
         all host cores) on a bounded sample of the same workload

Other workloads (--workload): acoustic2d (201 x 301 at 5 m, 2000 steps, 36 B
per cell update), elastic3d (600^3 at 10 m, npml 23, 2500 steps, 104 B) and
acoustic3d (48 B); the default line is the elastic 2-D batch.

--impl reference times the CPU restatement of the reference on the host
cores (the reference is Julia and cannot run here).  Multi-GPU: one process
per GPU, each rank models its own batch of shots (shots are independent,
weak scaling, no data-path collective).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "geophyinv.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gcell-updates/s"

# algorithmic bytes per cell update: 4 B x (2 x state arrays + coefficient arrays)
WORKLOADS = {
    "elastic2d": {"name": "elastic2d_psv_1000x3000_5m_16shots_4000steps", "bpc": 60, "nshots": 16, "nt": 4000,
                  "kernel": "k_e2 (fused elastic step), algorithmic 60 B/cell, launch time = run time / nt"},
    "acoustic2d": {"name": "acoustic2d_layers_201x301_5m_2000steps", "bpc": 36, "nshots": 1, "nt": 2000,
                   "kernel": "k_a2 (fused acoustic step), algorithmic 36 B/cell, launch time = run time / nt"},
    "elastic3d": {"name": "elastic3d_600x600x600_10m_npml23_2500steps", "bpc": 104, "nshots": 1, "nt": 2500,
                  "kernel": "k3_vel_e + k3_str_e (two fused passes), algorithmic 104 B/cell"},
    "acoustic3d": {"name": "acoustic3d_600x600x600_10m_npml23_2500steps", "bpc": 48, "nshots": 1, "nt": 2500,
                   "kernel": "k3_vel_a + k3_str_a (two fused passes), algorithmic 48 B/cell"},
    # one bench step = one gradient!: forward_save (36 B) + adjoint step with
    # the imaging condition (76 B fused) per cell and time step; the engine's
    # fused adjoint moves 84 B (per-velocity-cell rho sums in place of g_rho)
    "acoustic2d_grad": {"name": "acoustic2d_fwi_gradient_500x1500_10m_32shots_3000steps", "bpc": 112, "nshots": 32,
                        "nt": 3000,
                        "kernel": "forward_save (k_a2<m,1>) + fused adjoint (k_a2<m,2>: both wavefields and the "
                                  "imaging condition), algorithmic 36 + 76 B/cell"},
    # the same gradient through the checkpointed adjoint, a checkpoint every
    # 100 steps (30 state slots): forward_save (36 B) + the schedule's
    # recomputed steps (36 B each) + per step a turn: forward step (36 B),
    # velocity half step (20 B), imaging condition (52 B), adjoint step (36 B)
    "acoustic2d_grad_ckpt": {"name": "acoustic2d_fwi_gradient_checkpointed_500x1500_10m_32shots_3000steps_30slots",
                             "bpc": None, "nshots": 32, "nt": 3000, "slots": 30,
                             "kernel": "checkpointed gradient (k_a2 forward, recompute and turns, k_grad_a2), "
                                       "algorithmic 36 x (2 + recomputed/nt) + 108 B/cell"},
    # 3-D acoustic gradient on the 3-D workload's grid (646^3 extended), 500
    # of its 2500 steps, 8 state slots (5.1 GB each): forward_save (48 B) +
    # recomputed steps (48 B) + turns: copies (32 B), forward step (48 B),
    # velocity half step (40 B), imaging condition (64 B), adjoint step (48 B)
    "acoustic3d_grad_ckpt": {"name": "acoustic3d_gradient_checkpointed_600x600x600_10m_npml23_500steps_8slots",
                             "bpc": None, "nshots": 1, "nt": 500, "slots": 8,
                             "kernel": "checkpointed gradient (k3 passes, recompute and turns, k_grad_a3), "
                                       "algorithmic 48 x (2 + recomputed/nt) + 184 B/cell"},
    # 3-D elastic gradient (invlambda, invmu, rho) on the 3-D workload's grid,
    # 500 of its 2500 steps, 8 state slots: forward_save (104 B) + recomputed
    # steps (104 B) + turns: copies of the 9 fields (72 B), velocity half
    # step (60 B), imaging condition (144 B), adjoint step (104 B)
    "elastic3d_grad_ckpt": {"name": "elastic3d_gradient_checkpointed_600x600x600_10m_npml23_500steps_8slots",
                            "bpc": None, "nshots": 1, "nt": 500, "slots": 8,
                            "kernel": "checkpointed gradient (k3 elastic passes, recompute and turns, k_grad_e3), "
                                      "algorithmic 104 x (2 + recomputed/nt) + 276 B/cell"},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="elastic2d", choices=sorted(WORKLOADS) + ["serving"])
    ap.add_argument("--requests", type=int, default=24, help="serving: requests in the stream")
    ap.add_argument("--dist", default="full", choices=["full", "small"],
                    help="serving: request sizes of the 2000-request stream (sides 200-2000, 1000-6000 steps) "
                         "or a small one (sides 200-800, 500-2000 steps)")
    ap.add_argument("--rate", type=float, default=32.0, help="serving: arrival rate, requests/s")
    ap.add_argument("--rates", default="", help="serving: also sweep these arrival rates (comma list)")
    ap.add_argument("--nt", type=int, default=None)
    ap.add_argument("--nshots", type=int, default=None)
    ap.add_argument("--side", type=int, default=None, help="3-D workloads: a side^3 sub-grid (profiling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--order", type=int, default=4, choices=[2, 4, 6, 8],
                    help="forward workloads: stencil order (orders other than 4 run the generic per-cell steps)")
    ap.add_argument("--graph", type=int, default=2, choices=[0, 1, 2],
                    help="forward workloads: CUDA graphs (0 plain, 1 whole run, 2 replayed 16-step chunks)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(kind, nt=None, nshots=None, side=None):
    """The workload; `side` shrinks a 3-D grid to side^3 (CPU samples)."""
    from geophyinv_gb300 import configs

    kw = {} if nt is None else {"nt": nt}
    if side and "3d" in kind:
        kw.update(nz=side, ny=side, nx=side)
    if kind == "elastic2d":
        return configs.elastic2d_batch(nshots=nshots or 16, **kw)
    if kind in ("acoustic2d_grad", "acoustic2d_grad_ckpt"):
        return configs.acoustic2d_fwi(nshots=nshots or 32, anomaly=False, **kw)
    if kind == "acoustic3d_grad_ckpt":
        kw.setdefault("nt", WORKLOADS[kind]["nt"])
        return configs.acoustic3d(rfields=("vz",), src_field="p", **kw)
    if kind == "elastic3d_grad_ckpt":
        kw.setdefault("nt", WORKLOADS[kind]["nt"])
        return configs.elastic3d(rfields=("vx", "vz"), **kw)
    if kind == "acoustic2d":
        wl = configs.acoustic2d_layers(**kw)
    elif kind == "elastic3d":
        wl = configs.elastic3d(**kw)
    else:
        wl = configs.acoustic3d(**kw)
    if nshots and nshots > 1:
        wl.shots = wl.shots * nshots
    return wl


def config_json(kind, wl, n_gpus, shots_per_gpu=None, order=4):
    npml = wl.npml if wl.npml is not None else 43
    nsh = shots_per_gpu if shots_per_gpu is not None else len(wl.shots)
    state = {"elastic2d": 5, "acoustic2d": 3, "elastic3d": 9, "acoustic3d": 4, "acoustic2d_grad": 6,
             "acoustic2d_grad_ckpt": 6, "acoustic3d_grad_ckpt": 8, "elastic3d_grad_ckpt": 18}[kind]
    return {"workload": WORKLOADS[kind]["name"],
            "grid": [len(g) for g in wl.grid], "extended_grid": [len(g) + 2 * npml for g in wl.grid],
            "shots_per_gpu": nsh, "nt": wl.nt, "dt": wl.tgrid.step, "order": order,
            "receivers_per_shot": len(wl.shots[0][1]), "rfields": wl.rfields,
            "parallelism": "shot replicas x%d" % n_gpus,
            "l2": "not flushed: per-step working set %.2f GB >> 129 MB L2" % (
                2 * state * wl.cells() * nsh * 4 / 1e9)}


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# DRAM bytes per cell update of the step-kernel family, a CONSTANT taken
# from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum of the
# four tile-class launches of one step, divided by the cells they update):
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
#       --clock-control none -k regex:k_e2 -s 16 -c 4 --csv python bench.py --nt 10
#       --nshots 4 --steps 1 --warmup 3 --graph 0 --no-cpu-baseline
# (the batch's grid with 4 shots: 13.4 M cells, 633 MB per step; traffic per
# cell changes with the shot count only through the L2 reuse of the shared
# coefficient columns).  The bench cannot measure it in the run; the value
# is re-taken when the kernel changes.
TRAFFIC_B_PER_CELL = {"elastic2d": (47.2, "ncu dram bytes of the four k_e2 launches of one step, batch grid with 4 shots")}


def traffic_per_cell(kind):
    return TRAFFIC_B_PER_CELL.get(kind, (None, None))


def cpu_sample(kind, nt_cap=None, target_s=12.0, order=4):
    """The CPU oracle (all host threads) on one shot of the workload for a
    bounded number of time steps; returns (Gcell-updates/s, threads, sample).
    Gradient workloads time the whole gradient (forward_save and adjoint;
    the 3-D one through the oracle's history mode, the reference having no
    3-D gradient)."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1

    grad = "grad" in kind
    # 3-D: a 160^3 sub-grid (+ CPML) of the 600^3 model; 96^3 for the 3-D
    # gradient, whose oracle keeps the whole forward history in memory
    side = (96 if grad else 160) if "3d" in kind else None

    def run(nt):
        wl = workload(kind, nt, 1, side)
        ex = wl.as_dict()
        ex["order"] = order
        prep = O.Prepared(ex, np.float32)
        cells = int(np.prod(prep.shape))
        if grad:
            nr = len(wl.shots[0][1])
            dobs = {f: np.zeros((1, nt, nr), np.float32) for f in wl.rfields}
            t0 = time.perf_counter()
            O.gradient(ex, dobs, nthreads=threads, history="3d" in kind)
            return cells, time.perf_counter() - t0
        orc = O.Oracle(prep, nthreads=threads)
        src, rec = O._shot_inputs(prep, ex["shots"][0])
        t0 = time.perf_counter()
        orc.shot(0, 0, src, rec)
        t = time.perf_counter() - t0
        orc.close()
        return cells, t

    cells, t = run(4)
    per_step = t / 4
    nt = int(max(8, min(nt_cap or WORKLOADS[kind]["nt"], target_s / max(per_step, 1e-6))))
    cells, t = run(nt)
    rate = cells * nt / t / 1e9
    return rate, threads, "1 of %d shots, %d of %d steps, %d extended cells%s, %.1f s%s" % (
        WORKLOADS[kind]["nshots"], nt, WORKLOADS[kind]["nt"], cells, " (%d^3 sub-grid)" % side if side else "", t,
        ", whole gradient (forward_save + adjoint)" if grad else "")


def engine_arm(args, rank, world, local):
    import torch

    from geophyinv_gb300 import _lib, update

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        # host-side sums (misfits, source frequencies) go over gloo, the
        # timing maximum over NCCL
        dist.init_process_group("cpu:gloo,cuda:nccl", device_id=torch.device("cuda", local))
    # a stream of the plan's own (graphs cannot be captured on the legacy
    # default stream); the CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    # N ranks model a survey of N x the per-GPU shot count; each rank holds
    # its contiguous chunk of it (the reference's sschunks split), so the
    # work per GPU stays fixed (weak scaling)
    nsh = (args.nshots or WORKLOADS[args.workload]["nshots"]) * world
    wl = workload(args.workload, args.nt, nsh, args.side)
    pa = wl.expt(stream=stream.cuda_stream, shard=world > 1, order=args.order)
    pa.set_graph(args.graph)
    medium = wl.medium()
    srcwav = wl.srcwav()
    cells = pa.nss * int(np.prod([len(g) for g in pa.exgrid]))
    units = cells * pa.nt  # cell updates per bench step on this rank

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # --- value: inputs resident, one gpi_run per step ---
    for _ in range(args.warmup):
        pa.run(_lib.FORWARD)
    barrier()
    clocks = Clocks(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    launches = 0
    for _ in range(args.steps):
        pa.run(_lib.FORWARD)
        launches += pa.launches()
    ev1.record(stream)
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms)
    value = world * units / (ms * 1e-3) / 1e9

    # --- e2e: public API, host buffers in and out, every step ---
    update(pa, medium)
    update(pa, srcwav, [1])
    update(pa)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        update(pa, medium)        # H2D medium (padding, derived parameters)
        update(pa, srcwav, [1])   # H2D wavelets and spray matrices
        update(pa)                # run + D2H records
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps)
    e2e = world * units / (e2e_ms * 1e-3) / 1e9
    h2d = sum(int(np.prod(v.shape)) * 4 for v in pa.mod.values()) + sum(
        s.d[f].size * 4 for s in pa.srcwav[0] for f in s.fields)
    d2h = sum(pa.data[0][i].d[f].size * 4 for i in range(pa.nss) for f in pa.rfields)

    peak, peak_kind = peaks()
    W = WORKLOADS[args.workload]
    achieved = W["bpc"] * cells / (ms * 1e-3 / pa.nt) / 1e9  # per launch, all time charged to it
    tpc, tpc_src = traffic_per_cell(args.workload) if args.order == 4 else (None, None)
    kernel = W["kernel"] if args.order == 4 else (
        "generic order-%d steps (k_gvel, k_gstress_*: one thread per cell, derivatives in registers, two "
        "passes), algorithmic %d B/cell (the fused one-pass minimum)" % (args.order, W["bpc"]))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Gcell/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded gradient + smoothed perturbation model)",
        "config": dict(config_json(args.workload, wl, world, pa.nss, args.order),
                       cuda_graphs={0: "off", 1: "whole run", 2: "replayed 16-step chunks"}[args.graph]),
        "e2e": {"value": round(e2e, 3), "unit": "Gcell/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms, 3)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": None if tpc is None else round(tpc * cells),
                     "traffic_source": tpc_src,
                     "kernel": kernel,
                     "peak_source": peak_kind + " hbm_gbs"},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    return line, dist


def gradient_arm(args, world, local, kind="acoustic2d_grad"):
    """One bench step = gradient!(g, m, L2DistLoss(), dobs, pa) over all shots:
    forward_save, adjoint sources, adjoint run with the imaging condition.
    2-D: the observed data are modelled once (not timed) on the model with
    the Gaussian anomaly; the starting model omits it.  3-D: zero observed
    data (the misfit is the energy of the records).  The checkpointed kinds
    run the same gradient through a plan with state slots."""
    import ctypes

    import torch

    from geophyinv_gb300 import L2DistLoss, Recs, _lib, configs, get_modelvector, gradient, update

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    W = WORKLOADS[kind]
    kw = {} if args.nt is None else {"nt": args.nt}
    nsh = args.nshots or W["nshots"]
    wl = workload(kind, args.nt, nsh, args.side)
    if kind.startswith("acoustic2d"):
        true = configs.acoustic2d_fwi(nshots=nsh, **kw)
        pt = true.expt(stream=stream.cuda_stream)
        update(pt)
        # observed records in the Recs layout (nt x nr, column-major)
        dobs = [Recs(r.n, r.grid, r.fields, {f: np.array(r.d[f], order="F") for f in r.fields}) for r in pt.data[0]]
        del pt
    else:
        dobs = [Recs(len(s[1]), wl.tgrid, list(wl.rfields),
                     {f: np.zeros((wl.nt, len(s[1])), np.float32) for f in wl.rfields}) for s in wl.shots]
    slots = W.get("slots", 0)
    pa = wl.expt(mode="forward_save", stream=stream.cuda_stream, checkpoints=slots)
    pa.set_graph(args.graph)
    cells = pa.nss * int(np.prod([len(g) for g in pa.exgrid]))
    units = cells * pa.nt
    params = ["invlambda", "invmu", "rho"] if wl.physics == "elastic" else ["invK", "rho"]
    m0 = get_modelvector(pa, params)
    g = np.zeros_like(m0)
    for _ in range(args.warmup):
        gradient(g, m0, L2DistLoss(), dobs, pa, params)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    t0 = time.perf_counter()
    launches = 0
    for _ in range(args.steps):
        gradient(g, m0, L2DistLoss(), dobs, pa, params)
        launches += pa.launches()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    clk = clocks.stop()
    value = world * units / (ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    bpc = W["bpc"]
    sched = None
    if slots:
        adv, turns, stored = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        _lib.load().gpi_checkpoint_schedule(pa.nt, slots, ctypes.byref(adv), ctypes.byref(turns), ctypes.byref(stored))
        sched = {"slots": slots, "recomputed_steps": adv.value, "turns": turns.value,
                 "slot_gb": round(pa.plan_bytes() / 1e9, 2) if hasattr(pa, "plan_bytes") else None}
        base, turn = {"acoustic2d": (36, 108), "acoustic3d": (48, 184), "elastic3d": (104, 276)}[kind.split("_")[0]]
        bpc = base * (2 + adv.value / pa.nt) + turn
    achieved = bpc * cells / (ms * 1e-3 / pa.nt) / 1e9
    return {"metric": METRIC, "value": round(value, 3), "unit": "Gcell/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (layered + Gaussian anomaly, zero-anomaly start)" if kind.startswith("acoustic2d")
            else "synthetic (linear-gradient medium with a smoothed perturbation; zero observed data)",
            "config": dict(config_json(kind, wl, world), checkpoints=sched,
                           cuda_graphs={0: "off", 1: "whole run", 2: "replayed 16-step chunks"}[args.graph]),
            "e2e": {"value": round(value, 3), "unit": "Gcell/s", "note": "gradient! is the public call; host buffers"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": None, "kernel": W["kernel"],
                         "peak_source": peak_kind + " hbm_gbs"},
            "gpu_launches": int(launches), "clocks": clk}


def serving_arm(args):
    """The mixed request stream (50 % acoustic forward, 30 % elastic forward,
    20 % acoustic gradient; Poisson arrivals) through the continuous-batching
    loop, one shot at a time with plain launches (the baseline the serving
    target is quoted against) and one request at a time with its shots
    batched.  The requests follow the size distribution of the 2000-request
    stream (sides 200-2000, 1000-6000 steps, 1-8 shots; --dist small: sides
    200-800, 500-2000 steps); fewer requests than 2000 so that the three arms
    finish in minutes (the count is in the line).  Request payloads (models,
    geometry) are built before the clock starts: they arrive with the
    request."""
    from geophyinv_gb300 import serving

    sides, steps = SERVING_DIST[args.dist]
    reqs = serving.make_stream(args.requests, rate=args.rate, seed=4, sides=sides, steps=steps, shots=(1, 8))
    for r in reqs:
        r.payload()
    warm = serving.make_stream(6, rate=1000.0, seed=5, sides=(100, 150), steps=(50, 60), shots=(1, 2))
    serving.serve(warm, realtime=False)
    serving.serve_plain(warm, realtime=False, per_shot=True)
    clocks = Clocks(0)
    clocks.start()
    _, st = serving.serve(reqs, max_inflight=8)
    clk = clocks.stop()
    _, pl = serving.serve_plain(reqs, per_shot=True)
    _, pr = serving.serve_plain(reqs)
    return {"metric": "shots/s", "value": round(st["shots_per_s"], 3), "unit": "shots/s", "n_gpus": 1,
            "steps": 1, "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic request stream (seed 4)",
            "config": {"workload": "serving_stream_%d_requests_%g_per_s" % (len(reqs), args.rate),
                       "sides": list(sides), "steps": list(steps), "shots": [1, 8],
                       "mix": "50 % acoustic forward, 30 % elastic forward, 20 % acoustic gradient",
                       "max_inflight": 8},
            "serving": {k: round(v, 4) if isinstance(v, float) else v for k, v in st.items()},
            "plain_one_shot_at_a_time": {k: round(v, 4) if isinstance(v, float) else v for k, v in pl.items()},
            "plain_one_request_at_a_time": {k: round(v, 4) if isinstance(v, float) else v for k, v in pr.items()},
            "speedup_shots_per_s": round(st["shots_per_s"] / pl["shots_per_s"], 3),
            "speedup_vs_request_at_a_time": round(st["shots_per_s"] / pr["shots_per_s"], 3), "clocks": clk,
            "sweep": [rate_point(float(r), args.dist) for r in args.rates.split(",") if r] or None}


SERVING_DIST = {"full": ((200, 2000), (1000, 6000)), "small": ((200, 800), (500, 2000))}


def rate_point(rate, dist):
    """Serving against one shot at a time at one arrival rate: 8 s of
    arrivals (16 to 48 requests), shots/s, p50 and p99 of both."""
    from geophyinv_gb300 import serving

    n = int(max(16, min(48, 8 * rate)))
    sides, steps = SERVING_DIST[dist]
    reqs = serving.make_stream(n, rate=rate, seed=6, sides=sides, steps=steps, shots=(1, 8))
    for r in reqs:
        r.payload()
    _, st = serving.serve(reqs, max_inflight=8)
    _, pl = serving.serve_plain(reqs, per_shot=True)
    keep = ("shots_per_s", "p50_s", "p99_s")
    return {"rate": rate, "requests": n, "serving": {k: round(st[k], 4) for k in keep},
            "plain_one_shot_at_a_time": {k: round(pl[k], 4) for k in keep}}


def reference_arm(args):
    """CPU restatement of the reference (the oracle) on all host cores."""
    if args.workload not in WORKLOADS:
        return {"impl": "reference", "unavailable": "the serving loop has no counterpart in the reference"}
    rates = []
    sample = ""
    threads = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        rate, threads, sample = cpu_sample(args.workload, nt_cap=60, target_s=6.0, order=args.order)
        if i >= args.warmup:
            rates.append(rate)
    v = float(np.mean(rates))
    return {"metric": METRIC, "value": round(v, 4), "unit": "Gcell/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload]["name"], "order": args.order, "sample": sample},
            "cpu_baseline": {"value": round(v, 4), "unit": "Gcell/s", "cores": threads, "kind": "port",
                             "sample": sample + "; C restatement of the reference time loop (Julia is absent)"},
            "e2e": {"value": round(v, 4), "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args)))
        return
    if args.workload == "serving":
        print(json.dumps(serving_arm(args)))
        return
    if args.workload in ("acoustic2d_grad", "acoustic2d_grad_ckpt", "acoustic3d_grad_ckpt", "elastic3d_grad_ckpt"):
        if args.order != 4:
            raise SystemExit("gradients run at stencil order 4 only")
        line, dist = gradient_arm(args, world, local, args.workload), None
    else:
        line, dist = engine_arm(args, rank, world, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            rate, threads, sample = cpu_sample(args.workload, order=args.order)
            line["cpu_baseline"] = {"value": round(rate, 4), "unit": "Gcell/s", "cores": threads, "kind": "port",
                                    "sample": sample}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
