"""Continuous-batching serving loop for forward and gradient shot requests.

Requests of uneven grid sizes, step counts and shot counts arrive over time.
The server admits a request as soon as an in-flight slot is free and its
plan fits the HBM budget, prepares it on a host worker thread (model, CPML
profiles, projections, a plan of its own with stream-ordered device
allocations) while other requests run, then launches it on its own CUDA
stream (all of its shots in one multi-shot launch per step; optionally the
whole time loop as one CUDA graph, worth it for plans that run more than
once) and keeps its wavefields, boundary store and records resident until it
completes.  Requests on the GPU overlap, and the host work of one request
overlaps the device work of the others.  A gradient request runs forward_save, builds its adjoint
sources from the residuals and runs the adjoint (gradient!,
src/fdtd/func_grad.jl:11-49).

A request carries its payload (model, geometry, wavelets: `Request.payload`,
built by the client before it is sent); the server's own work starts at
admission.  The baselines (`serve_plain`) take the same stream one shot at a
time (a single-shot plan per shot, plain launches, no overlap), or one
request at a time with its shots batched.  Results do not depend on what else
runs: every request's arithmetic is its own and deterministic.
"""
import copy
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib, configs
from .fdtd import L2DistLoss, Recs, Srcs, update

KINDS = ("acoustic_forward", "elastic_forward", "acoustic_gradient")


@dataclass
class Request:
    """One modelling request: `kind` in KINDS, grid nz x nx, nt steps, nshots
    supersources, arrival time in seconds from the start of the stream."""
    rid: int
    kind: str
    nz: int
    nx: int
    nt: int
    nshots: int
    arrival: float = 0.0
    seed: int = 0
    _payload: object = field(default=None, repr=False, compare=False)

    def payload(self):
        """The request's workload (built once, then kept)."""
        if self._payload is None:
            self._payload = self.workload()
        return self._payload

    def workload(self):
        nrec = max(8, self.nx // 4)
        if self.kind == "acoustic_forward":
            wl = configs.acoustic2d_layers(nz=self.nz, nx=self.nx, nt=self.nt, nrec=nrec, seed=self.seed,
                                           rfields=("p", "vz"))
            src, rec = wl.shots[0]
            xm = wl.grid[1].last
            wl.shots = [(np.array([[src[0, 0], x]]), rec) for x in np.linspace(0.0, xm, self.nshots + 2)[1:-1]]
            return wl
        if self.kind == "elastic_forward":
            return configs.elastic2d_batch(nz=self.nz, nx=self.nx, nt=self.nt, nshots=self.nshots, nrec=nrec,
                                           seed=self.seed)
        return configs.acoustic2d_fwi(nz=self.nz, nx=self.nx, nt=self.nt, nshots=self.nshots, nrec=nrec,
                                      seed=self.seed, anomaly=False)

    def cells(self):
        return (self.nz + 86) * (self.nx + 86) * self.nshots * self.nt


def make_stream(n, rate, seed=4, sides=(200, 2000), steps=(1000, 6000), shots=(1, 8), mix=(0.5, 0.3, 0.2)):
    """A seeded request stream: Poisson arrivals at `rate` requests/s, grid
    sides and step counts uniform in the given ranges, 50 / 30 / 20 %
    acoustic forward / elastic forward / acoustic gradient."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        kind = KINDS[int(rng.choice(3, p=np.asarray(mix) / np.sum(mix)))]
        out.append(Request(i, kind, int(rng.integers(sides[0], sides[1] + 1)), int(rng.integers(sides[0], sides[1] + 1)),
                           int(rng.integers(steps[0], steps[1] + 1)), int(rng.integers(shots[0], shots[1] + 1)), t,
                           seed=int(rng.integers(0, 1 << 30))))
    return out


def plan_bytes_estimate(req):
    """Device bytes of a request's plan (state, CPML strips, coefficients,
    records, boundary store), from the layout of the engine."""
    nz, nx = req.nz + 86, req.nx + 86
    nzp = (nz + 124 + 12 + 31) // 32 * 32
    f = nzp * (nx + 15) * 4
    ela = req.kind == "elastic_forward"
    npw = 2 if req.kind == "acoustic_gradient" else 1
    state = (5 if ela else 3) * 2 * npw * req.nshots * f
    coef = ((5 if ela else 3) + 3) * f
    psi = (8 if ela else 4) * 2 * npw * req.nshots * 88 * max(nzp, nx + 15) * 4
    rec = req.nt * (req.nx // 4 + 8) * 2 * req.nshots * 4
    store = (req.nt * 6 * (nz + nx) + 3 * nzp * (nx + 15)) * 4 * req.nshots if npw == 2 else 0
    return state + coef + psi + rec + store + npw * 2 * req.nshots * f


@dataclass
class Result:
    rid: int
    kind: str
    records: list = field(default_factory=list)
    gradient: dict = None
    loss: float = None
    t_admit: float = 0.0
    t_done: float = 0.0


class _Job:
    """The life of one request on the server (a small state machine)."""

    def __init__(self, req, graphs, stream, shot=None):
        self.req = req
        self.wl = req.payload()
        if shot is not None:
            self.wl = copy.copy(self.wl)
            self.wl.shots = [self.wl.shots[shot]]
        mode = "forward_save" if req.kind == "acoustic_gradient" else "forward"
        self.pa = self.wl.expt(mode=mode, stream=stream)
        if graphs:
            # forward runs as replays of one captured 16-step chunk; a
            # whole-run graph would cost more to capture than one run saves
            self.pa.set_graph(2)
        self.res = Result(req.rid, req.kind)
        self.phase = 0
        self.busy = None  # a launch still being issued on a worker thread
        self.error = None

    def launch(self):
        pa = self.pa
        if self.req.kind == "acoustic_gradient":
            if self.phase == 0:
                update(pa, pa.srcwav, [1, 0])
                pa.run(_lib.FORWARD_SAVE)
            else:
                pa.run(_lib.ADJOINT)
        else:
            pa.run(_lib.FORWARD)

    def finish_phase(self, pool=None):
        """Called when the device work of the current phase is done; returns
        True when the request is complete.  The next phase is issued on a
        worker thread of `pool` when one is given."""
        pa = self.pa
        recs = [{f: pa.records(i, f) for f in pa.rfields} for i in range(pa.nss)]
        if self.req.kind != "acoustic_gradient":
            self.res.records = recs
            return True
        if self.phase == 0:
            # adjoint sources: deriv(L2DistLoss(), dobs, dcal) reversed in time,
            # with zero observed data (func_grad.jl:19-31)
            loss = L2DistLoss()
            adj = []
            total = 0.0
            for i in range(pa.nss):
                s = Srcs(pa.ageom[i].nr, pa.tgrid, pa.rfields)
                for f in pa.rfields:
                    obs = np.zeros_like(recs[i][f])
                    total += loss.value(obs, recs[i][f])
                    s.d[f] = loss.deriv(obs, recs[i][f])[::-1].copy()
                adj.append(s)
            self.res.records = recs
            self.res.loss = total
            pa.srcwav[1] = adj
            update(pa, pa.srcwav, [-1, 1])
            self.phase = 1
            if pool is None:
                self.launch()
            else:
                self.busy = pool.submit(self.launch)
                self.busy.add_done_callback(self._issued)
            return False
        self.res.gradient = {"invK": pa.gradient_raw(0), "rho": pa.gradient_raw(1)}
        return True

    def _issued(self, fut):
        self.error = fut.exception()
        self.busy = None

    def close(self):
        self.pa.close() if hasattr(self.pa, "close") else None
        self.pa = None


def _prepare(req, graphs, stream):
    job = _Job(req, graphs, stream)
    job.launch()
    return job


def _streams(n):
    import torch

    return [torch.cuda.Stream() for _ in range(n)]


def serve(requests, hbm_budget=64 << 30, max_inflight=8, graphs=True, realtime=True, prep_threads=4):
    """Continuous batching: admit arrived requests while slots and HBM budget
    allow, prepare them on host threads, launch them when ready, poll the
    in-flight ones, launch their next phase or collect their results.
    Returns (results by id, stats)."""
    from concurrent.futures import ThreadPoolExecutor

    import torch

    streams = _streams(max_inflight)
    free = list(range(max_inflight))
    pending = sorted(requests, key=lambda r: r.arrival)
    preparing = {}
    inflight = {}
    results = {}
    used = 0
    pool = ThreadPoolExecutor(max_workers=prep_threads)
    t0 = time.perf_counter()
    while pending or preparing or inflight:
        now = time.perf_counter() - t0
        # admission: arrival order, HBM budget, a free stream
        while pending and free and (not realtime or pending[0].arrival <= now):
            need = plan_bytes_estimate(pending[0])
            if (inflight or preparing) and used + need > hbm_budget:
                break
            req = pending.pop(0)
            slot = free.pop()
            preparing[req.rid] = (pool.submit(_prepare, req, graphs, streams[slot].cuda_stream), slot, need,
                                  time.perf_counter() - t0)
            used += need
        for rid in list(preparing):
            fut, slot, need, t_admit = preparing[rid]
            if fut.done():
                job = fut.result()
                job.res.t_admit = t_admit
                inflight[rid] = (job, slot, need)
                del preparing[rid]
        done_any = False
        for rid in list(inflight):
            job, slot, need = inflight[rid]
            if job.error is not None:
                raise job.error
            if job.busy is None and job.pa.done():
                done_any = True
                if job.finish_phase(pool):
                    job.res.t_done = time.perf_counter() - t0
                    results[rid] = job.res
                    job.close()
                    del inflight[rid]
                    free.append(slot)
                    used -= need
        if not done_any:
            time.sleep(0.0002)
    pool.shutdown()
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    return results, _stats(requests, results, time.perf_counter() - t0)


def _run_plain(job):
    import torch

    job.launch()
    while True:
        torch.cuda.synchronize()
        if job.finish_phase():
            break
    res = job.res
    job.close()
    return res


def serve_plain(requests, realtime=True, per_shot=False):
    """The baseline: one request at a time, or with `per_shot` one shot at a
    time (a single-shot plan per shot), plain launches, each to completion.
    A request's result collects its shots' records in order (and sums their
    gradients and losses)."""
    results = {}
    t0 = time.perf_counter()
    for req in sorted(requests, key=lambda r: r.arrival):
        if realtime:
            wait = req.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        t_admit = time.perf_counter() - t0
        if not per_shot:
            res = _run_plain(_Job(req, False, None))
        else:
            res = Result(req.rid, req.kind)
            for i in range(req.nshots):
                one = _run_plain(_Job(req, False, None, shot=i))
                res.records += one.records
                if one.gradient is not None:
                    res.loss = one.loss if res.loss is None else res.loss + one.loss
                    res.gradient = one.gradient if res.gradient is None else \
                        {k: res.gradient[k] + one.gradient[k] for k in one.gradient}
        res.t_admit = t_admit
        res.t_done = time.perf_counter() - t0
        results[req.rid] = res
    return results, _stats(requests, results, time.perf_counter() - t0)


def _stats(requests, results, wall):
    lat = np.array([results[r.rid].t_done - r.arrival for r in requests])
    shots = sum(r.nshots for r in requests)
    return {"requests": len(requests), "shots": shots, "wall_s": wall, "shots_per_s": shots / wall,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "gcells_per_s": sum(r.cells() for r in requests) / wall / 1e9}
