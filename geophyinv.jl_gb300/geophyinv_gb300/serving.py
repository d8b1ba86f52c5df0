"""Continuous-batching serving loop for forward and gradient shot requests.

Requests of uneven grid sizes, step counts and shot counts arrive over time.
`serve` hands each one, when it arrives, to the engine's C server
(gpi_server_*, csrc/gpi_server.cu): the client builds the request's arrays
(padding, CPML profiles, projections: `RequestBuffers`) on a pool of host
threads, the server admits requests in arrival order while its worker
slots and HBM budget allow, runs each on its own CUDA stream (all of its
shots in one multi-shot launch per step, forward runs replayed as captured
16-step chunks) and returns records and gradients.  Requests on the GPU
overlap, and the host work of one overlaps the device work of the others.
A gradient request runs forward_save, builds its adjoint sources from the
residuals and runs the adjoint (gradient!, src/fdtd/func_grad.jl:11-49).

A request carries its payload (model, geometry, wavelets: `Request.payload`,
built by the client before it is sent).  The baselines (`serve_plain`) take
the same stream one shot at a time (a single-shot plan per shot, plain
launches, no overlap), or one request at a time with its shots batched.
Results do not depend on what else runs: every request's arithmetic is its
own and deterministic.
"""
import copy
import ctypes
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


class RequestBuffers:
    """The arrays of one request as the C server takes them (gpi_request):
    the host set-up of the reference's PFdtd constructor (padding, derived
    parameters, peak frequency and CPML profiles, projection matrices), in
    the same steps as SeisForwExpt, without creating a plan."""

    def __init__(self, req, graphs=True):
        from . import setup as S

        wl = req.payload()
        gradient = req.kind == "acoustic_gradient"
        npml = wl.npml if wl.npml is not None else 43
        mask = S.face_mask(wl.pml_faces)
        exgrid = S.padgrid(wl.grid, npml, mask)
        vp = S.padarray(wl.vp, npml, mask)
        rho = S.padarray(wl.rho, npml, mask)
        if wl.physics == "acoustic":
            mod = [S.invK(vp, rho), rho]
        else:
            vs = S.padarray(wl.vs, npml, mask)
            mod = [S.invlambda(vp, vs, rho), S.invmu(vs, rho), rho]
        self.mod = [np.asfortranarray(m, np.float32) for m in mod]
        d = _lib.PlanDesc()
        d.physics = _lib.ACOUSTIC if wl.physics == "acoustic" else _lib.ELASTIC
        d.ndim, d.order = 2, 4
        d.nz, d.ny, d.nx = len(exgrid[0]), 1, len(exgrid[1])
        d.dz, d.dy, d.dx = wl.grid[0].step, 1.0, wl.grid[1].step
        d.npml, d.nbound = npml, 3
        d.pml_faces = mask
        d.rigid_faces = mask
        d.free_faces = S.face_mask(wl.stressfree_faces)
        d.nt, d.nshots = wl.nt, len(wl.shots)
        d.npw = 2 if gradient else 1
        d.dt = wl.tgrid.step
        srcwav = wl.srcwav()
        peaks = [np.mean([S.findfreq_peak(np.asarray(s.d[f], np.float32), d.dt) for f in s.fields]) for s in srcwav]
        _, vb = S.ref_bounds(vp)
        velavg = np.float32((vb[0] + vb[1]) / np.float32(2.0))
        pml = S.cpml_all(wl.physics, 2, 4, wl.grid, mask, np.float32(d.dt), velavg, np.float32(np.mean(peaks)), npml)
        self.pml = np.ascontiguousarray(np.concatenate([np.concatenate(x) for x in pml]), np.float32)
        self.keep = []
        src, rec = [], []
        ageom = wl.ageom()
        for iss, (a, sw) in enumerate(zip(ageom, srcwav)):
            for f in sw.fields:
                cp, rv, nz = S.projection(f, exgrid, a.points("s", 2), 4)
                w = np.asfortranarray(sw.d[f], np.float32)
                src.append((iss, f, len(cp) - 1, cp, rv, nz, w))
            for f in wl.rfields:
                cp, rv, nz = S.projection(f, exgrid, a.points("r", 2), 4)
                rec.append((iss, f, len(cp) - 1, cp, rv, nz, None))
        self.src_entries, self.rec_entries = src, rec

        def projs(entries):
            arr = (_lib.Proj * len(entries))()
            for i, (iss, f, n, cp, rv, nz, data) in enumerate(entries):
                self.keep += [cp, rv, nz] + ([data] if data is not None else [])
                arr[i].shot, arr[i].field, arr[i].n = iss, _lib.FIELD[f], n
                arr[i].colptr, arr[i].rowval, arr[i].nzval = cp.ctypes.data, rv.ctypes.data, nz.ctypes.data
                arr[i].data = data.ctypes.data if data is not None else None
            return arr

        self.src_arr, self.rec_arr = projs(src), projs(rec)
        self.mod_ptrs = (ctypes.c_void_p * len(self.mod))(*[m.ctypes.data for m in self.mod])
        r = _lib.Request()
        r.plan = d
        r.gradient = int(gradient)
        r.nsrc, r.nrec = len(src), len(rec)
        # forward runs replay a captured 16-step chunk (a whole-run graph
        # costs more to capture than one run saves)
        r.graph = 2 if graphs else 0
        r.mod = ctypes.cast(self.mod_ptrs, ctypes.c_void_p)
        r.pml = self.pml.ctypes.data
        r.src, r.rec = self.src_arr, self.rec_arr
        self.request = r
        self.desc = d
        self.rfields = list(wl.rfields)
        self.nt = wl.nt
        self.nshots = len(wl.shots)


def request_bytes(req):
    """Device bytes the server charges a request against its HBM budget (the
    plan's pool by gpi_plan_estimate plus its record buffers)."""
    L = _lib.load()
    rb = RequestBuffers(req)
    b = ctypes.c_size_t()
    _lib.check(L.gpi_plan_estimate(ctypes.byref(rb.desc), ctypes.byref(b)))
    recs = sum(rb.nt * e[2] for e in rb.rec_entries)
    return b.value + recs * 4 * (3 if req.kind == "acoustic_gradient" else 2)


class Server:
    """The C ABI server (gpi_server_*): requests in, results out."""

    def __init__(self, max_inflight=8, hbm_budget=64 << 30, device=0, max_batch=0):
        self.L = _lib.load()
        d = _lib.ServerDesc()
        d.device, d.max_inflight, d.hbm_budget, d.max_batch = device, max_inflight, hbm_budget, max_batch
        h = ctypes.c_void_p()
        rc = self.L.gpi_server_create(ctypes.byref(d), ctypes.byref(h))
        if rc:
            raise _lib.EngineError("gpi_server_create: %s" % self.L.gpi_server_message(None, 0).decode())
        self.h = h

    def submit(self, rb):
        i = ctypes.c_int64()
        rc = self.L.gpi_server_submit(self.h, ctypes.byref(rb.request), ctypes.byref(i))
        if rc:
            raise _lib.EngineError("gpi_server_submit: %s" % self.L.gpi_server_message(self.h, 0).decode())
        return i.value

    def _check(self, rc, sid):
        if rc:
            raise _lib.EngineError("request %d: %s: %s" % (sid, _lib.STATUS.get(rc, rc),
                                                          self.L.gpi_server_message(self.h, sid).decode()))

    def result(self, sid, req, rb):
        L = self.L
        self._check(L.gpi_server_wait(self.h, sid), sid)
        res = Result(req.rid, req.kind)
        for iss in range(rb.nshots):
            per = {}
            for (s, f, n, *_rest) in rb.rec_entries:
                if s == iss:
                    out = np.zeros((rb.nt, n), np.float32, order="F")
                    self._check(L.gpi_server_records(self.h, sid, iss, _lib.FIELD[f], out.ctypes.data), sid)
                    per[f] = out
            res.records.append(per)
        if req.kind == "acoustic_gradient":
            n = [rb.desc.nz, rb.desc.nx]
            res.gradient = {}
            loss = ctypes.c_double()
            for q, k in enumerate(("invK", "rho")):
                g = np.zeros(n, np.float32, order="F")
                self._check(L.gpi_server_gradient(self.h, sid, q, g.ctypes.data, ctypes.byref(loss)), sid)
                res.gradient[k] = g
            res.loss = loss.value
        t = (ctypes.c_double * 3)()
        self._check(L.gpi_server_times(self.h, sid, t), sid)
        res.t_admit, res.t_done = t[1], t[2]
        L.gpi_server_release(self.h, sid)
        return res

    def close(self):
        if self.h:
            self.L.gpi_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def serve(requests, hbm_budget=64 << 30, max_inflight=8, graphs=True, realtime=True, prep_threads=4, max_batch=0):
    """Continuous batching through the C server: each request is handed to
    it when it arrives (its host set-up -- padding, CPML profiles,
    projections -- on one of `prep_threads` client threads), the server
    admits it while slots and the HBM budget allow -- 2-D forward requests
    into the batch of their physics, advanced by shared launches (max_batch
    members, 0: the server's default, -1: no batches), the others on their
    own streams overlapping -- and returns its records (and gradient).
    Returns (results by id, stats); admission and completion times are on
    the stream's clock (seconds from its start)."""
    from concurrent.futures import ThreadPoolExecutor

    srv = Server(max_inflight=max_inflight, hbm_budget=hbm_budget, max_batch=max_batch)
    pool = ThreadPoolExecutor(max_workers=prep_threads)
    pending = sorted(requests, key=lambda r: r.arrival)
    # the stream's clock starts with the server's (gpi_server_times)
    t0 = time.perf_counter()

    def hand_in(req):
        rb = RequestBuffers(req, graphs)
        return rb, srv.submit(rb)

    futs = []
    for req in pending:
        if realtime:
            wait = req.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        futs.append((req, pool.submit(hand_in, req)))
    results = {}
    for req, fut in futs:
        rb, sid = fut.result()
        results[req.rid] = srv.result(sid, req, rb)
    pool.shutdown()
    wall = time.perf_counter() - t0
    srv.close()
    return results, _stats(requests, results, wall)


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
