"""ctypes driver of the CPU ORACLE (test infrastructure only).

Runs the C restatement of the reference time loop (libgpo.so, built from
oracle/fdtd_oracle_*.c by oracle/Makefile) on a plain-dict experiment
description and returns records and gradients.  It mirrors the control flow
of the reference drivers:

  * forward          -> update!(pa)            (src/fdtd/propagate.jl:74-135)
  * gradient         -> gradient!(g, m, ...)   (src/fdtd/func_grad.jl:11-49)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.

Experiment description (all positions in metres, arrays Float32):
  physics      "acoustic" | "elastic"
  ndim         2 | 3
  order        stencil order (4)
  grid         physical grid [(start, step, n)] per axis (z, [y,] x)
  vp, rho, vs  physical media (vs for elastic)
  pml_faces, rigid_faces, free_faces   bit masks (setup_ref.FACE_BITS)
  dt, nt
  shots        list of {"src": {field: (positions, wavelets nt x ns)},
                        "rec": positions}
  rfields      list of recorded fields
"""
import ctypes
import os
import subprocess

import numpy as np

from . import setup_ref as S

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    """Compile libgpo.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "libgpo.so")
        if not os.path.exists(path):
            build()
        _LIB = ctypes.CDLL(path)
        for sfx in ("f32", "f64"):
            getattr(_LIB, "gpo_create_" + sfx).restype = ctypes.c_void_p
            getattr(_LIB, "gpo_create_" + sfx).argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            getattr(_LIB, "gpo_shot_" + sfx).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                        ctypes.c_void_p]
            getattr(_LIB, "gpo_get_field_" + sfx).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
            getattr(_LIB, "gpo_destroy_" + sfx).argtypes = [ctypes.c_void_p]
        _LIB.gpo_get_dmod_f32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_int)]
    return _LIB


class _Desc(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int), ("ndim", ctypes.c_int), ("order", ctypes.c_int),
                ("nz", ctypes.c_int), ("ny", ctypes.c_int), ("nx", ctypes.c_int),
                ("npml", ctypes.c_int), ("nbound", ctypes.c_int), ("pml_faces", ctypes.c_int),
                ("rigid_faces", ctypes.c_int), ("free_faces", ctypes.c_int), ("nt", ctypes.c_int),
                ("nthreads", ctypes.c_int),
                ("dt", ctypes.c_double), ("dz", ctypes.c_double), ("dy", ctypes.c_double), ("dx", ctypes.c_double)]


class _Proj(ctypes.Structure):
    _fields_ = [("field", ctypes.c_int), ("n", ctypes.c_int), ("colptr", ctypes.c_void_p),
                ("rowval", ctypes.c_void_p), ("nzval", ctypes.c_void_p), ("data", ctypes.c_void_p)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Prepared:
    """Everything the time loop needs, derived from an experiment description
    exactly as the reference constructor does (PFdtd, src/fdtd/fdtd.jl:61-297)."""

    def __init__(self, ex, dtype=np.float32, ref_compat=True):
        self.ex = ex
        self.dtype = dtype
        self.physics = ex["physics"]
        self.ndim = ex["ndim"]
        self.order = ex.get("order", 4)
        self.h = self.order - 1
        self.npml = int(ex["npml"]) if ex.get("npml") is not None else S.npml_of(self.order)
        self.faces = ex["pml_faces"]
        self.rigid = ex.get("rigid_faces", self.faces) | self.faces
        self.free = ex.get("free_faces", 0)
        self.nt = ex["nt"]
        self.dt = ex["dt"]
        self.grid = ex["grid"]
        self.exgrid = S.padmgrid(self.grid, self.npml, self.faces)
        vp = S.padarray(np.asarray(ex["vp"], np.float32), self.npml, self.faces)
        rho = S.padarray(np.asarray(ex["rho"], np.float32), self.npml, self.faces)
        if self.physics == "acoustic":
            self.mod = S.derived_acoustic(vp, rho)
        else:
            vs = S.padarray(np.asarray(ex["vs"], np.float32), self.npml, self.faces)
            self.mod = S.derived_elastic(vp, vs, rho)
        _, vb = S.bounds(vp)
        self.velavg = np.float32((vb[0] + vb[1]) / np.float32(2))
        # wavelets of wavefield 1 set the peak frequency (fill_wavelets!, source.jl:24-58)
        peaks = []
        for shot in ex["shots"]:
            fp = [S.findfreq_peak(w, self.dt) for (_, w) in shot["src"].values()]
            peaks.append(np.mean(fp))
        self.fpeak = np.float32(np.mean(peaks))
        self.pml = S.pml_all(self.physics, self.ndim, self.order, self.grid, self.faces,
                             np.float32(self.dt), self.velavg, self.fpeak, self.npml)
        self.ref_compat = ref_compat
        self.shape = [g[2] for g in self.exgrid]

    def desc(self, nthreads=0):
        d = _Desc()
        d.physics = 0 if self.physics == "acoustic" else 1
        d.ndim = self.ndim
        d.order = self.order
        n = self.shape
        d.nz, d.ny, d.nx = (n[0], n[1], n[2]) if self.ndim == 3 else (n[0], 1, n[1])
        st = [g[1] for g in self.grid]
        d.dz, d.dy, d.dx = (st[0], st[1], st[2]) if self.ndim == 3 else (st[0], 1.0, st[1])
        d.npml = self.npml
        d.nbound = 3
        d.pml_faces = self.faces
        d.rigid_faces = self.rigid
        d.free_faces = self.free
        d.nt = self.nt
        d.nthreads = nthreads
        d.dt = self.dt
        return d

    def proj(self, field, points):
        return S.proj_matrix(field, self.exgrid, points, self.ndim, self.order, self.ref_compat)


class Oracle:
    """Owns one oracle context (wavefields, boundary stores)."""

    def __init__(self, prep, nthreads=0):
        self.p = prep
        self.sfx = "f32" if prep.dtype == np.float32 else "f64"
        L = lib()
        self.L = L
        self._keep = []
        mods = [np.ascontiguousarray(m.astype(prep.dtype).reshape(-1, order="F")) for m in prep.mod]
        pml = []
        for a, b, k in prep.pml:
            pml += [np.ascontiguousarray(a.astype(prep.dtype)), np.ascontiguousarray(b.astype(prep.dtype)),
                    np.ascontiguousarray(k.astype(prep.dtype))]
        self._keep += mods + pml
        mp = (ctypes.c_void_p * len(mods))(*[m.ctypes.data for m in mods])
        pp = (ctypes.c_void_p * len(pml))(*[x.ctypes.data for x in pml])
        self.d = prep.desc(nthreads)
        self.ctx = getattr(L, "gpo_create_" + self.sfx)(ctypes.byref(self.d), mp, pp, len(prep.ex["shots"]))

    def close(self):
        if self.ctx:
            getattr(self.L, "gpo_destroy_" + self.sfx)(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def _projs(self, items, nt):
        arrs = (_Proj * max(1, len(items)))()
        for i, (field, (cp, rv, nz), data) in enumerate(items):
            nzv = np.ascontiguousarray(nz.astype(self.p.dtype))
            self._keep += [cp, rv, nzv, data]
            arrs[i].field = S.FIELD_ID[field]
            arrs[i].n = len(cp) - 1
            arrs[i].colptr = cp.ctypes.data
            arrs[i].rowval = rv.ctypes.data
            arrs[i].nzval = nzv.ctypes.data
            arrs[i].data = data.ctypes.data
        return arrs

    def shot(self, ishot, mode, src, rec, adj=(), grads=None):
        """src: list of (field, csc, wavelets nt x n Fortran); rec: list of
        (field, csc) -> returns {field: records nt x nr}."""
        nt = self.p.nt
        dt = self.p.dtype
        srcs = [(f, csc, np.asfortranarray(np.asarray(w, dt))) for f, csc, w in src]
        outs = {}
        recs = []
        for f, csc in rec:
            out = np.zeros((nt, len(csc[0]) - 1), dtype=dt, order="F")
            outs[f] = out
            recs.append((f, csc, out))
        adjs = [(f, csc, np.asfortranarray(np.asarray(w, dt))) for f, csc, w in adj]
        sp = self._projs(srcs, nt)
        rp = self._projs(recs, nt)
        ap = self._projs(adjs, nt)
        gs = [None, None, None]
        if grads is not None:
            for i, g in enumerate(grads):
                gs[i] = g
        rc = getattr(self.L, "gpo_shot_" + self.sfx)(
            self.ctx, ishot, mode, len(srcs), sp, len(recs), rp, len(adjs), ap,
            *[None if g is None else g.ctypes.data for g in gs])
        self._keep = self._keep[: 0]
        if rc != 0:
            raise RuntimeError("oracle shot failed: %d" % rc)
        return outs

    def field(self, name, ipw=1):
        from ctypes import byref, c_int
        n1, n2, n3 = c_int(), c_int(), c_int()
        L = self.L
        L.gpo_field_shape.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                      ctypes.POINTER(c_int)]
        L.gpo_field_shape(ctypes.byref(self.d), S.FIELD_ID[name], byref(n1), byref(n2), byref(n3))
        out = np.zeros(n1.value * n2.value * n3.value, dtype=self.p.dtype)
        rc = getattr(L, "gpo_get_field_" + self.sfx)(self.ctx, ipw, S.FIELD_ID[name], out.ctypes.data)
        if rc != 0:
            raise RuntimeError("no field %s" % name)
        shp = (n1.value, n3.value) if self.p.ndim == 2 else (n1.value, n2.value, n3.value)
        return out.reshape(shp, order="F")

    def dmod(self, idx):
        from ctypes import byref, c_int
        n1, n2, n3 = c_int(), c_int(), c_int()
        if self.L.gpo_get_dmod_f32(self.ctx, idx, None, byref(n1), byref(n2), byref(n3)) != 0:
            raise IndexError(idx)
        out = np.zeros(n1.value * n2.value * n3.value, dtype=np.float32)
        self.L.gpo_get_dmod_f32(self.ctx, idx, out.ctypes.data, byref(n1), byref(n2), byref(n3))
        shp = (n1.value, n3.value) if self.p.ndim == 2 else (n1.value, n2.value, n3.value)
        return out.reshape(shp, order="F")


def _shot_inputs(prep, shot, src_types=1):
    src = []
    for f, (pos, w) in shot["src"].items():
        w = np.asarray(w, np.float32)
        if w.ndim == 1:
            w = w[:, None]
        if src_types == -1:
            w = S.source_reverse(w)
        src.append((f, prep.proj(f, pos), w))
    rec = [(f, prep.proj(f, shot["rec"])) for f in prep.ex["rfields"]]
    return src, rec


def forward(ex, dtype=np.float32, nthreads=0, ref_compat=True, return_oracle=False, snaps=None, mod=None,
            illum=False):
    """update!(pa) in :forward mode: records[field] of shape (nshots, nt, nr).
    snaps = (field, [steps]) also returns res["snaps"][shot][k], the field at
    the end of step steps[k] (1-based; snaps_save!).  illum=True also returns
    res["illum"], pac.illum_stack with illum_flag (compute_illum!, stack_illums!,
    src/fdtd/fdtd.jl:556-582): the shot sum of sum_t p^2 on the physical
    grid, FP64.  mod: extended-grid
    medium parameters replacing the ones padded from ex (as after
    update!(pa, m, mparams), which leaves the PML cells as they were)."""
    prep = Prepared(ex, dtype, ref_compat)
    if mod is not None:
        prep.mod = [np.asarray(m, np.float64 if dtype == np.float64 else np.float32) for m in mod]
    orc = Oracle(prep, nthreads)
    if snaps is not None:
        its = (ctypes.c_int * len(snaps[1]))(*snaps[1])
        sfx = orc.sfx
        fn = getattr(orc.L, "gpo_set_snaps_" + sfx)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        assert fn(orc.ctx, S.FIELD_ID[snaps[0]], len(snaps[1]), its) == 0
    if illum:
        fn = getattr(orc.L, "gpo_set_illum_" + orc.sfx)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
        assert fn(orc.ctx, 1) == 0
    out = {f: [] for f in ex["rfields"]}
    stack = None
    for i, shot in enumerate(ex["shots"]):
        src, rec = _shot_inputs(prep, shot)
        r = orc.shot(i, 0, src, rec)
        for f in ex["rfields"]:
            out[f].append(r[f])
        if illum:
            shape = orc.field("p").shape
            a = np.zeros(int(np.prod(shape)), np.float64)
            get = getattr(orc.L, "gpo_get_illum_" + orc.sfx)
            get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            assert get(orc.ctx, i, a.ctypes.data) == 0
            gss = a.reshape(shape, order="F")[_inner(prep, shape)]
            stack = (np.zeros_like(gss) if stack is None else stack) + gss  # illums += gss
    res = {f: np.stack(v) for f, v in out.items()}
    if illum:
        res["illum"] = stack
    if snaps is not None:
        shape = orc.field(snaps[0]).shape
        get = getattr(orc.L, "gpo_get_snap_" + orc.sfx)
        get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        res["snaps"] = []
        for i in range(len(ex["shots"])):
            per = []
            for k in range(len(snaps[1])):
                a = np.zeros(int(np.prod(shape)), dtype=prep.dtype)
                assert get(orc.ctx, i, k, a.ctypes.data) == 0
                per.append(a.reshape(shape, order="F"))
            res["snaps"].append(per)
    if return_oracle:
        return res, orc
    orc.close()
    return res


def gradient(ex, dobs, dtype=np.float32, nthreads=0, ref_compat=True, history=False, imaging=0, mod=None):
    """gradient!(g, m, L2DistLoss(), dobs, pa) for 2-D acoustic
    (src/fdtd/func_grad.jl:11-49).  Returns (loss, {"invK": g, "rho": g},
    dcal) with g the chain-ruled gradient on the inner (non-PML) grid and the
    raw per-cell accumulations on the extended grid.

    history=True takes wavefield 1 from the stored forward history instead
    of rebuilding it by time reversal (GPO_FORWARD_HIST / GPO_ADJOINT_HIST):
    the gradient of a checkpointed adjoint; 2-D and 3-D acoustic.

    imaging selects the rho term of the imaging condition (gpo_set_imaging):
    0 the reference's, 1 the finite-difference-consistent one.

    mod: extended-grid medium parameters that replace the ones padded from
    ex (update!(pa, m, mparams) keeps the PML cells of the old medium)."""
    prep = Prepared(ex, dtype, ref_compat)
    if mod is not None:
        prep.mod = [np.asarray(m, np.float64 if dtype == np.float64 else np.float32) for m in mod]
    if prep.physics == "elastic" and not history:
        raise ValueError("elastic gradients: history mode only (no boundary store in 3-D)")
    orc = Oracle(prep, nthreads)
    if imaging:
        fn = getattr(orc.L, "gpo_set_imaging_" + orc.sfx)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
        assert fn(orc.ctx, int(imaging)) == 0
    shape = prep.shape
    names = ["invK", "rho"] if prep.physics == "acoustic" else ["invlambda", "invmu", "rho"]
    gs = [np.zeros(shape, dtype=dtype, order="F") for _ in names]
    dcal = {f: [] for f in ex["rfields"]}
    # forward_save with src_types [1, 0]
    for i, shot in enumerate(ex["shots"]):
        src, rec = _shot_inputs(prep, shot, 1)
        r = orc.shot(i, 3 if history else 1, src, rec)
        for f in ex["rfields"]:
            dcal[f].append(r[f])
    dcal = {f: np.stack(v) for f, v in dcal.items()}
    loss = sum(S.l2_value(dobs[f], dcal[f]) for f in ex["rfields"])
    # adjoint with src_types [-1, 1] (history mode: the forward sources, for
    # the source terms of the elastic imaging condition)
    for i, shot in enumerate(ex["shots"]):
        src, _ = _shot_inputs(prep, shot, 1 if history else -1)
        adj = []
        for f in ex["rfields"]:
            a = S.l2_deriv(dobs[f][i], dcal[f][i])[::-1].copy()
            adj.append((f, prep.proj(f, shot["rec"]), a))
        orc.shot(i, 4 if history else 2, src, [], adj, gs)
    orc.close()
    raw = {k: g.copy() for k, g in zip(names, gs)}
    inner = _inner(prep, shape)
    g = {k: (raw[k] * prep.mod[i])[inner] for i, k in enumerate(names)}
    return loss, g, dcal, raw


def _inner(prep, shape):
    """Slices of the physical grid in an extended-grid array (the padding
    sits on the PML faces only)."""
    inner = []
    axes = "zyx" if prep.ndim == 3 else "zx"
    for i, d in enumerate(axes):
        lo = prep.npml if prep.faces & S.FACE_BITS[d + "min"] else 0
        hi = prep.npml if prep.faces & S.FACE_BITS[d + "max"] else 0
        inner.append(slice(lo, shape[i] - hi))
    return tuple(inner)


def born(ex, dinvK, drho, dtype=np.float32, nthreads=0):
    """Born (linearised) records for the medium perturbation (dinvK, drho)
    given on the extended grid (update!(pa, medium, medium_pert) forms it as
    the padded perturbed medium minus the medium, src/fdtd/medium.jl:103-126):
    records[field] of shape (nshots, nt, nr) of the scattered wavefield
    (GPO_BORN, acoustic)."""
    prep = Prepared(ex, dtype)
    orc = Oracle(prep, nthreads)
    a = np.ascontiguousarray(np.asarray(dinvK, dtype).reshape(-1, order="F"))
    b = np.ascontiguousarray(np.asarray(drho, dtype).reshape(-1, order="F"))
    fn = getattr(orc.L, "gpo_set_born_" + orc.sfx)
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert fn(orc.ctx, a.ctypes.data, b.ctypes.data) == 0
    out = {f: [] for f in ex["rfields"]}
    for i, shot in enumerate(ex["shots"]):
        src, rec = _shot_inputs(prep, shot)
        r = orc.shot(i, 5, src, rec)
        for f in ex["rfields"]:
            out[f].append(r[f])
    orc.close()
    return {f: np.stack(v) for f, v in out.items()}
