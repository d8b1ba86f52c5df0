"""Host mirror of GeoPhyInv's FDTD experiment API on top of the C ABI.

    pa = SeisForwExpt(FdtdAcoustic(), medium=..., ageom=..., srcwav=...,
                      tgrid=..., rfields=["p"], pml_faces=[...])
    update(pa)                    # update!(pa)            (src/fdtd/propagate.jl:74-135)
    pa["data"]                    # records, one Recs per supersource
    update(pa, medium)            # update!(pa, medium)    (src/fdtd/medium.jl:128-140)
    update(pa, srcwav, [1])       # update!(pa, srcwav, src_types) (src/fdtd/source.jl:192-246)
    gradient(g, m, loss, dobs, pa, ["invK", "rho"])   (src/fdtd/func_grad.jl:11-49)
    lossvalue(m, loss, dobs, pa, mparams)             (src/fdtd/func_grad.jl:1-9)

The constructor follows PFdtd (src/fdtd/fdtd.jl:61-297): checks, padding,
derived parameters, plan allocation, wavelets and peak frequency, CPML
profiles, projection matrices.  All supersources of an experiment run in one
plan (the reference distributes them over Distributed workers).
"""
import ctypes
import copy
import warnings

import numpy as np

from . import _lib
from . import setup as S
from . import shots as _shots
from .setup import Grid

ALL_FACES = ["zmin", "zmax", "ymin", "ymax", "xmax", "xmin"]


class FdtdAcoustic:
    """FdtdAcoustic{FullWave}(mode, npw) (src/physics_types.jl:25-49)."""
    physics = "acoustic"

    def __init__(self, mode="forward", npw=None):
        self.mode = mode
        self.npw = npw if npw is not None else (1 if mode == "forward" else 2)


class FdtdElastic(FdtdAcoustic):
    physics = "elastic"


class FdtdAcousticBorn(FdtdAcoustic):
    """FdtdAcoustic{Born}(mode, npw = 2) (src/physics_types.jl:25-49):
    wavefield 1 the background, wavefield 2 the Born (single-scattering)
    field of the perturbation set by update(pa, medium, medium_pert); its
    records are pa.data[1]."""
    born = True

    def __init__(self, mode="forward", npw=2):
        super().__init__(mode, 2)


class AcousticMedium:
    """AcousticMedium (src/media/media.jl:40-51): grid per axis, vp, rho (Float32)."""
    params = ("vp", "rho")

    def __init__(self, grid, vp, rho):
        self.grid = list(grid)
        self.vp = np.asarray(vp, np.float32)
        self.rho = np.asarray(rho, np.float32)
        assert self.vp.shape == tuple(len(g) for g in self.grid) == self.rho.shape

    @property
    def ndim(self):
        return len(self.grid)

    def copy(self):
        return copy.deepcopy(self)


class ElasticMedium(AcousticMedium):
    params = ("vp", "vs", "rho")

    def __init__(self, grid, vp, vs, rho):
        super().__init__(grid, vp, rho)
        self.vs = np.asarray(vs, np.float32)
        assert self.vs.shape == self.vp.shape


class AGeomss:
    """Positions of one supersource (src/ageom/ageom.jl:4-16): s and r map
    axis names to coordinate arrays."""

    def __init__(self, s, r):
        self.s = {k: np.atleast_1d(np.asarray(v, np.float64)) for k, v in s.items()}
        self.r = {k: np.atleast_1d(np.asarray(v, np.float64)) for k, v in r.items()}
        self.ns = len(next(iter(self.s.values())))
        self.nr = len(next(iter(self.r.values())))

    def points(self, which, ndim):
        d = self.s if which == "s" else self.r
        return np.stack([d[a] for a in S.axis_names(ndim)], 1)


class Srcs:
    """Srcs / Recs (src/database/database.jl:18-43): d[field] is nt x n."""

    def __init__(self, n, grid, fields, d=None):
        self.n = n
        self.grid = grid
        self.fields = list(fields)
        self.d = d if d is not None else {f: np.zeros((len(grid), n), np.float32) for f in self.fields}

    def copy(self):
        return copy.deepcopy(self)


Recs = Srcs


def Fields(attrib, ndim):
    """Non-derivative fields of a physics (src/fields.jl:9-25)."""
    v = ["vx", "vz"] if ndim == 2 else ["vx", "vy", "vz"]
    if attrib.physics == "acoustic":
        return ["p"] + v
    t = ["tauxx", "tauzz", "tauxz"] if ndim == 2 else ["tauxx", "tauyy", "tauzz", "tauxy", "tauxz", "tauyz"]
    return t + v


class L2DistLoss:
    """LossFunctions 0.11.2 L2DistLoss: value (output - target)^2 and
    deriv 2 (output - target), called as loss(dobs, dcal)."""

    def value(self, output, target):
        r = np.subtract(np.asarray(output), np.asarray(target), dtype=np.float64).ravel(order="K")
        return float(np.dot(r, r))

    def deriv(self, output, target):
        return (np.float32(2) * (np.asarray(output, np.float32) - np.asarray(target, np.float32))).astype(np.float32)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class SeisForwExpt:
    """PFdtd (src/fdtd/fdtd.jl:61-297) driving one libgpi_fdtd plan."""

    def __init__(self, attrib, *, medium, ageom, srcwav, tgrid, rfields=("vz",), pml_faces=ALL_FACES,
                 rigid_faces=None, stressfree_faces=(), order=4, ref_compat_proj=True, stream=None, verbose=False,
                 npml=None, checkpoints=0, tsnaps=None, snaps_field=None, shard=False, ref_compat_grad=True,
                 illum_flag=False, jobname="forward_propagation", backprop_flag=None, nworker=None):
        L = _lib.load()
        self.L = L
        self.attrib = attrib
        # PFdtd keywords kept for their meaning only: the run mode (attrib)
        # selects the boundary store, one process drives one device
        self.jobname = jobname
        self.backprop_flag = backprop_flag
        self.nworker = nworker
        self.illum_flag = bool(illum_flag)
        if self.illum_flag and attrib.physics != "acoustic":
            raise ValueError("illum_flag: the illumination sums p^2 (acoustic media only)")
        self.order = order
        self.h = order - 1
        # the reference pads by 40 + h cells (_fd_npml, GeoPhyInv.jl:90); a smaller CPML
        # (npml = n + h) may be asked for explicitly
        self.npml = int(npml) if npml is not None else 40 + self.h
        self.nbound = 3
        N = medium.ndim
        self.ndim = N
        self.tgrid = tgrid
        self.nt = len(tgrid)
        self.dt = tgrid.step
        self.rfields = list(rfields)
        fields = Fields(attrib, N)
        for f in self.rfields:
            assert f in fields, "receiver field %s not in %s" % (f, fields)
        if isinstance(ageom, AGeomss):
            ageom = [ageom]
        ageom = list(ageom)
        srcwav = list(srcwav) if isinstance(srcwav, (list, tuple)) else [srcwav]
        assert len(ageom) == len(srcwav), "ageom and srcwav mismatch"
        for s in srcwav:
            for f in s.fields:
                assert f in fields, "source field %s not in %s" % (f, fields)
        # shard=True under an initialised torch.distributed group: this rank
        # holds only its contiguous chunk of the supersources (sschunks,
        # src/fdtd/fdtd.jl:246-255); gradients and misfits are summed over
        # the ranks once per gradient! / lossvalue (sum_grads!,
        # src/fdtd/gradient.jl:2-12).  Lists indexed by supersource that the
        # caller passes later (srcwav, dobs) may cover all of them.
        self.nss_global = len(ageom)
        self.shot_ids = list(range(len(ageom)))
        self.shard = False
        if shard:
            rank, world = _shots.rank_world()
            if world > 1:
                self.shot_ids = list(_shots.my_shots(len(ageom), rank, world))
                if not self.shot_ids:
                    raise ValueError("rank %d of %d holds no supersource (%d in all)" % (rank, world, len(ageom)))
                ageom = [ageom[i] for i in self.shot_ids]
                srcwav = [srcwav[i] for i in self.shot_ids]
                self.shard = True
        self.ageom = ageom
        self.nss = len(ageom)
        # adjoint geometry/wavelets of the second wavefield (fdtd.jl:90-99)
        self.srcwav = [[s.copy() for s in srcwav]]
        if attrib.npw == 2:
            self.srcwav.append([Srcs(a.nr, tgrid, self.rfields) for a in ageom])
        self._check_inside(medium)
        self.pml_mask = S.face_mask(pml_faces)
        rigid = pml_faces if rigid_faces is None else rigid_faces
        self.rigid_mask = S.face_mask(rigid) | self.pml_mask
        self.free_mask = S.face_mask(stressfree_faces)
        self.ref_compat_proj = ref_compat_proj
        self.medium = medium.copy()
        self._set_exmedium(self.medium)
        n = [len(g) for g in self.exgrid]
        d = _lib.PlanDesc()
        d.physics = _lib.ACOUSTIC if attrib.physics == "acoustic" else _lib.ELASTIC
        d.ndim = N
        d.order = order
        d.nz, d.ny, d.nx = (n[0], n[1], n[2]) if N == 3 else (n[0], 1, n[1])
        st = [g.step for g in medium.grid]
        d.dz, d.dy, d.dx = (st[0], st[1], st[2]) if N == 3 else (st[0], 1.0, st[1])
        d.npml = self.npml
        d.nbound = self.nbound
        d.pml_faces = self.pml_mask
        d.rigid_faces = self.rigid_mask
        d.free_faces = self.free_mask
        d.nt = self.nt
        d.nshots = self.nss
        d.npw = attrib.npw
        # checkpointed adjoint (no counterpart in the reference): this many
        # device slots of wavefield-1 states replace the boundary store
        d.checkpoints = int(checkpoints) if attrib.npw == 2 else 0
        self.checkpoints = d.checkpoints
        # rho term of the imaging condition: the reference's
        # (src/fdtd/gradient.jl:31-56) or, with ref_compat_grad=False, the
        # gradient of the discrete model (agrees with finite differences)
        d.imaging = 0 if ref_compat_grad else 1
        d.dt = self.dt
        self.desc = d
        plan = ctypes.c_void_p()
        rc = L.gpi_plan_create(ctypes.byref(d), ctypes.byref(plan))
        if rc != 0:
            raise _lib.EngineError("gpi_plan_create: %s: %s" % (_lib.STATUS.get(rc, rc), L.gpi_last_error(None).decode()))
        self.plan = plan
        self.stream = stream
        if stream is not None:
            self._check(L.gpi_set_stream(plan, ctypes.c_void_p(stream)))
        self._upload_medium()
        self._set_receivers()
        self._src_types = [1] * attrib.npw
        update(self, self.srcwav[0] if attrib.npw == 1 else [self.srcwav[0], self.srcwav[1]],
               [1] if attrib.npw == 1 else [1, 0], _pml=False)
        self._update_pml()
        self.check_stability(verbose)
        self.data = [[Recs(a.nr, tgrid, self.rfields) for a in ageom] for _ in range(attrib.npw)]
        self.gradients = None
        # snapshots at the steps nearest to tsnaps (fdtd.jl:179-187; default
        # time: the middle of tgrid)
        self.snaps_field = snaps_field
        self.itsnaps = []
        if snaps_field is not None:
            assert snaps_field in fields, "snapshot field %s not in %s" % (snaps_field, fields)
            t = tgrid.values()
            ts = [0.5 * (t[0] + t[-1])] if tsnaps is None else list(tsnaps)
            self.tsnaps = ts
            self.itsnaps = [int(np.argmin(np.abs(t - x))) + 1 for x in ts]
            its = (ctypes.c_int32 * len(self.itsnaps))(*self.itsnaps)
            self._check(L.gpi_set_snapshots(self.plan, _lib.FIELD[snaps_field], len(self.itsnaps), its))
        if self.illum_flag:
            self._check(L.gpi_set_illum(self.plan, 1))

    # ------------------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            raise _lib.EngineError("%s: %s" % (_lib.STATUS.get(rc, rc), self.L.gpi_last_error(self.plan).decode()))

    def __del__(self):
        p = getattr(self, "plan", None)
        if p:
            self.L.gpi_plan_destroy(p)
            self.plan = None

    def close(self):
        self.__del__()

    def _check_inside(self, medium):
        g = medium.grid
        names = S.axis_names(medium.ndim)
        for a in self.ageom:
            for which in ("s", "r"):
                P = a.points(which, medium.ndim)
                for i in range(medium.ndim):
                    if np.any((P[:, i] - g[i].first) * (g[i].last - P[:, i]) < 0.0):
                        raise ValueError("sources or receivers not inside medium (%s)" % names[i])

    def _set_exmedium(self, medium):
        """padarray + MediumParameters (fdtd.jl:137-153, media.jl:260-304)."""
        self.exgrid = S.padgrid(medium.grid, self.npml, self.pml_mask)
        vp = S.padarray(medium.vp, self.npml, self.pml_mask)
        rho = S.padarray(medium.rho, self.npml, self.pml_mask)
        self.exvp = vp
        if self.attrib.physics == "acoustic":
            self.mparams = ["invK", "rho"]
            self.mod = {"invK": S.invK(vp, rho), "rho": rho}
        else:
            vs = S.padarray(medium.vs, self.npml, self.pml_mask)
            self.exvs = vs
            self.mparams = ["invlambda", "invmu", "rho"]
            self.mod = {"invlambda": S.invlambda(vp, vs, rho), "invmu": S.invmu(vs, rho), "rho": rho}
        self.ref_mod = {k: S.ref_bounds(v)[0] for k, v in self.mod.items()}

    def _upload_medium(self):
        arrs = [np.asfortranarray(self.mod[k], np.float32) for k in self.mparams]
        self._mod_keep = arrs
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        self._check(self.L.gpi_set_medium(self.plan, ptrs, 0))

    def _proj(self, field, points):
        return S.projection(field, self.exgrid, points, self.order, self.ref_compat_proj)

    def _set_receivers(self):
        self._rproj = []
        for iss, a in enumerate(self.ageom):
            pts = a.points("r", self.ndim)
            per = {}
            for f in self.rfields:
                cp, rv, nz = self._proj(f, pts)
                per[f] = (cp, rv, nz)
                self._check(self.L.gpi_set_receivers(self.plan, iss, _lib.FIELD[f], a.nr, _ptr(cp), _ptr(rv), _ptr(nz)))
            self._rproj.append(per)

    def _update_pml(self):
        """update_pml! (src/fdtd/cpml.jl:144-155), once, with the peak frequency
        of the wavelets."""
        _, vb = S.ref_bounds(self.exvp)
        velavg = np.float32((vb[0] + vb[1]) / np.float32(2.0))
        self.pml = S.cpml_all(self.attrib.physics, self.ndim, self.order, self.medium.grid, self.pml_mask,
                              np.float32(self.dt), velavg, np.float32(self.freqpeak), self.npml)
        for q, (a, b, k) in enumerate(self.pml):
            self._check(self.L.gpi_set_pml(self.plan, q, len(a), _ptr(a), _ptr(b), _ptr(k)))

    def check_stability(self, verbose=False):
        """check_stability (src/fdtd/stability.jl:8-60): warnings only.
        Spatial sampling: at least H = 20 / order points per minimum
        wavelength at the highest source frequency (vmin: the smallest
        non-zero vs for elastic media, the lower vp bound otherwise); time
        sampling: the Courant limit dt <= d_min / (sqrt(ndim) vmax), vmax
        = sqrt(vp_max^2 + vs_max^2) for elastic media.  As in the reference,
        the limits are compared as %0.2e strings first."""
        H = 20 // self.order
        _, vb = S.ref_bounds(self.medium.vp)
        vmin, vmax = float(vb[0]), float(vb[1])
        if self.attrib.physics == "elastic":
            _, vsb = S.ref_bounds(self.medium.vs)
            vs = np.asarray(self.medium.vs)
            vmin = float(vs[vs != 0].min())
            vmax = float(np.sqrt(vb[1] ** 2 + vsb[1] ** 2))
        steps = [g.step for g in self.medium.grid]
        fmax = getattr(self, "freqmax", None)
        if fmax and np.isfinite(fmax) and fmax > 0:
            ds_temp = round(vmin / H / fmax, 2)
            s1, s2 = "%0.2e" % max(steps), "%0.2e" % ds_temp
            if s1 != s2:
                if max(steps) > ds_temp:
                    warnings.warn("decrease maximum spatial sampling (%s) below %s" % (s1, s2))
                elif verbose:
                    print("spatial sampling (%s) can be as high as %s" % (s1, s2))
        dtmax = (1.0 / np.sqrt(self.ndim)) * min(steps) / vmax
        s1, s2 = "%0.2e" % self.dt, "%0.2e" % dtmax
        if s1 != s2:
            if self.dt > dtmax:
                warnings.warn("decrease time sampling (%s) below %s" % (s1, s2))
            elif verbose:
                print("time sampling (%s) can be as high as %s" % (s1, s2))

    def __getitem__(self, key):
        if isinstance(key, tuple) and key[0] == "snaps":
            return self.snaps(key[1] if len(key) > 1 else 0)
        if key == "snaps":
            return self.snaps(0)
        if key == "data":
            return self.data[0]
        if key == "srcwav":
            return self.srcwav
        if key == "illum":
            return self.illum_stack
        raise KeyError(key)

    @property
    def illum_stack(self):
        """pac.illum_stack (src/fdtd/fdtd.jl:177, stack_illums! :556-566):
        the sum over the supersources of sum_t p^2 of the last run, FP64 on
        the physical grid (illum_flag=True; the reference declares it but its
        calls are commented out, so there it stays zero)."""
        if not self.illum_flag:
            raise ValueError("illum_flag=False")
        out = np.zeros([len(g) for g in self.medium.grid], np.float64, order="F")
        self._check(self.L.gpi_get_illum(self.plan, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0))
        return _shots.reduce_gradient(out) if self.shard else out

    # ------------------------------------------------------------------
    def run(self, mode):
        self._check(self.L.gpi_run(self.plan, mode))

    def set_graph(self, enable=True):
        """CUDA graphs: True / 1 replays each run as one graph (captured on
        first use); 2 replays forward runs as chunks of 16 captured steps
        (pays off for a plan that runs once); False / 0 plain launches."""
        kind = int(enable) if not isinstance(enable, bool) else int(enable)
        self._check(self.L.gpi_set_graph(self.plan, kind))

    def done(self):
        """True when every run issued so far has finished on the device."""
        v = ctypes.c_int32()
        self._check(self.L.gpi_query(self.plan, ctypes.byref(v)))
        return bool(v.value)

    def snaps(self, iss=0, ipw=1):
        """pa[:snaps, iss] (getprop.jl:10-29): the snapshots of the last run,
        in the order of tsnaps (0-based shot index)."""
        name = self.snaps_field
        n = [len(g) for g in self.exgrid]
        kinds = S.FIELD_KINDS[name]
        shape = []
        for ax, g in enumerate(n):
            k = kinds[ax if self.ndim == 3 else (0 if ax == 0 else 2)]
            shape.append(g + self.h if k == S.KV else g - self.h if k == S.KH else g - 2 * self.h if k == S.KI else g)
        out = []
        for k in range(len(self.itsnaps)):
            a = np.zeros(shape, np.float32, order="F")
            self._check(self.L.gpi_get_snapshot(self.plan, ipw, k, iss, _ptr(a), 0))
            out.append(a)
        return out

    def records(self, iss, field):
        out = np.zeros((self.nt, self.ageom[iss].nr), np.float32, order="F")
        self._check(self.L.gpi_get_records(self.plan, iss, _lib.FIELD[field], _ptr(out), 0))
        return out

    def field(self, name, ipw=1, iss=0):
        n = [len(g) for g in self.exgrid]
        kinds = S.FIELD_KINDS[name]
        shape = []
        for ax, g in enumerate(n):
            k = kinds[ax if self.ndim == 3 else (0 if ax == 0 else 2)]
            shape.append(g + self.h if k == S.KV else g - self.h if k == S.KH else g - 2 * self.h if k == S.KI else g)
        out = np.zeros(shape, np.float32, order="F")
        self._check(self.L.gpi_get_field(self.plan, ipw, iss, _lib.FIELD[name], _ptr(out), 0))
        return out

    def gradient_raw(self, param):
        n = [len(g) for g in self.exgrid]
        out = np.zeros(n, np.float32, order="F")
        self._check(self.L.gpi_get_gradient(self.plan, param, _ptr(out), 0))
        return out

    def launches(self):
        v = ctypes.c_int64()
        self._check(self.L.gpi_last_launches(self.plan, ctypes.byref(v)))
        return v.value


# ----------------------------------------------------------------------
# update! dispatch
# ----------------------------------------------------------------------
def update(pa, *args, _pml=True, **kw):
    """update!(pa) / update!(pa, medium) / update!(pa, srcwav, src_types) /
    update!(pa, m, mparams) / update!(pa, medium, medium_pert) (Born)."""
    if not args:
        return _update_run(pa)
    a0 = args[0]
    if isinstance(a0, AcousticMedium) and len(args) > 1 and isinstance(args[1], AcousticMedium):
        return _update_born(pa, a0, args[1])
    if isinstance(a0, AcousticMedium):
        return _update_medium(pa, a0)
    if isinstance(a0, np.ndarray) and a0.ndim == 1:
        return _update_modelvector(pa, a0, args[1])
    return _update_srcwav(pa, a0, args[1] if len(args) > 1 else None)


def _update_run(pa):
    """update!(pa) (src/fdtd/propagate.jl:74-135)."""
    if getattr(pa.attrib, "born", False) and pa.attrib.mode == "forward":
        return _born_run(pa)
    mode = {"forward": _lib.FORWARD, "forward_save": _lib.FORWARD_SAVE, "adjoint": _lib.ADJOINT}[pa.attrib.mode]
    if pa.attrib.npw == 1:
        mode = _lib.FORWARD
    pa.run(mode)
    if mode != _lib.ADJOINT:
        for iss in range(pa.nss):
            for f in pa.rfields:
                pa.data[0][iss].d[f] = pa.records(iss, f)
    return pa


def update_batch(pas, max_steps=256, stream=None):
    """update!(pa) for several forward experiments at once (2-D, one
    physics, npw = 1): the engine advances them together, one launch per
    tile class and time step over the tiles of all of them (gpi_batch_*);
    experiments with fewer steps finish first.  Each experiment's records
    equal those of its own update!(pa) bit for bit.  No counterpart in the
    reference, which runs one experiment per worker at a time."""
    if not pas:
        return pas
    L = _lib.load()
    import torch

    dev = torch.cuda.current_device()
    b = ctypes.c_void_p()
    rc = L.gpi_batch_create(dev, ctypes.c_void_p(stream) if stream else None, ctypes.byref(b))
    if rc:
        raise _lib.EngineError("batch: %s" % L.gpi_batch_error(None).decode())
    try:
        for pa in pas:
            if pa.attrib.mode != "forward" or getattr(pa.attrib, "born", False):
                raise ValueError("update_batch takes forward experiments")
            rc = L.gpi_batch_add(b, pa.plan)
            if rc:
                raise _lib.EngineError("batch: %s" % L.gpi_batch_error(b).decode())
        active = ctypes.c_int32(len(pas))
        while active.value > 0:
            rc = L.gpi_batch_advance(b, max_steps, ctypes.byref(active))
            if rc:
                raise _lib.EngineError("batch: %s" % L.gpi_batch_error(b).decode())
        for pa in pas:
            for iss in range(pa.nss):
                for f in pa.rfields:
                    pa.data[0][iss].d[f] = pa.records(iss, f)
    finally:
        L.gpi_batch_destroy(b)
        for pa in pas:
            pa._check(L.gpi_set_stream(pa.plan, ctypes.c_void_p(pa.stream) if pa.stream else None))
    return pas


def _update_medium(pa, medium):
    """update!(pa, medium) (src/fdtd/medium.jl:128-140): no new allocation,
    PML not recomputed."""
    pa.medium = medium.copy()
    pa._set_exmedium(pa.medium)
    pa._upload_medium()
    return pa


def _update_born(pa, medium, medium_pert):
    """update!(pa, medium, medium_pert) (src/fdtd/medium.jl:103-126): the
    background medium, then dmod = padded medium_pert - padded medium on the
    extended grid (invK and rho)."""
    _update_medium(pa, medium)
    vp = S.padarray(medium_pert.vp, pa.npml, pa.pml_mask)
    rho = S.padarray(medium_pert.rho, pa.npml, pa.pml_mask)
    pert = {"invK": S.invK(vp, rho), "rho": rho}
    set_born_perturbation(pa, [(pert[k] - pa.mod[k]).astype(np.float32) for k in ("invK", "rho")])
    return pa


def set_born_perturbation(pa, dmod):
    """dmod = [dinvK, drho] on the extended grid (pac.δmod of the reference)."""
    arrs = [np.asfortranarray(np.asarray(a, np.float32).reshape([len(g) for g in pa.exgrid], order="F")) for a in dmod]
    pa._born_keep = arrs
    ptrs = (ctypes.c_void_p * 2)(*[a.ctypes.data for a in arrs])
    pa._check(pa.L.gpi_set_born(pa.plan, ptrs, 0))


def _born_run(pa):
    """Born run: the background with the plan's sources, the scattered
    wavefield's records into pa.data[1]."""
    pa._check(pa.L.gpi_clear_sources(pa.plan, 2, -1))
    pa.run(_lib.BORN)
    for iss in range(pa.nss):
        for f in pa.rfields:
            pa.data[1][iss].d[f] = pa.records(iss, f)
    return pa


class BornMap:
    """LinearMap(pa) of a Born experiment (src/fdtd/func_grad.jl:53-120):
    F x -> the Born records of every supersource for x = [dinvK; drho] on
    the extended grid (column-major, flattened), and its transpose
    F' y -> the imaging gradient with y as the adjoint sources.  The
    transpose needs a plan created with checkpoints > 0 and
    ref_compat_grad=False (the exact adjoint of the discrete scheme)."""

    def __init__(self, pa):
        self.pa = pa
        self.nm = 2 * int(np.prod([len(g) for g in pa.exgrid]))
        self.nd = sum(pa.nt * a.nr * len(pa.rfields) for a in pa.ageom)
        self.shape = (self.nd, self.nm)

    def _split(self, x):
        n = [len(g) for g in self.pa.exgrid]
        x = np.asarray(x, np.float32)
        h = len(x) // 2
        return [x[:h].reshape(n, order="F"), x[h:].reshape(n, order="F")]

    def matvec(self, x):
        pa = self.pa
        set_born_perturbation(pa, self._split(x))
        update(pa, pa.srcwav[0], [1, 0])
        _born_run(pa)
        return np.concatenate([pa.data[1][i].d[f].ravel(order="F") for i in range(pa.nss) for f in pa.rfields])

    def rmatvec(self, y):
        """F' y: the adjoint sources are y (time-reversed, as gradient!
        does); the result is -(raw imaging accumulations), since the
        imaging condition returns dJ/dm for adjoint sources -dJ/dd."""
        pa = self.pa
        mode_save = pa.attrib.mode
        y = np.asarray(y, np.float32)
        pa.attrib.mode = "forward_save"
        update(pa, pa.srcwav[0], [1, 0])
        update(pa)
        adj, k = [], 0
        for a in pa.ageom:
            s = Srcs(a.nr, pa.tgrid, pa.rfields)
            for f in pa.rfields:
                n = pa.nt * a.nr
                s.d[f] = y[k:k + n].reshape(pa.nt, a.nr, order="F")[::-1].copy()
                k += n
            adj.append(s)
        update(pa, [pa.srcwav[0], adj], [1 if pa.checkpoints else -1, 1])
        pa.attrib.mode = "adjoint"
        update(pa)
        pa.attrib.mode = mode_save
        return -np.concatenate([pa.gradient_raw(0).ravel(order="F"), pa.gradient_raw(1).ravel(order="F")])


def _update_srcwav(pa, srcwav, src_types=None, ipws=None):
    """update!(pa, srcwav, src_types) (src/fdtd/source.jl:192-246); `ipws`
    limits the engine update to those wavefields (0-based)."""
    if isinstance(srcwav, Srcs):
        srcwav = [[srcwav]]
    elif srcwav and isinstance(srcwav[0], Srcs):
        srcwav = [srcwav]
    if src_types is None:
        src_types = [1] * len(srcwav)
    assert len(srcwav) == len(pa.srcwav) or len(srcwav) == 1
    for ipw, sw in enumerate(srcwav):
        pa.srcwav[ipw] = [s.copy() for s in _local(pa, sw)]
    peaks = []
    fmaxs = []
    for ipw in range(pa.attrib.npw):
        if ipws is not None and ipw not in ipws:
            continue
        st = src_types[ipw] if ipw < len(src_types) else 0
        pa._check(pa.L.gpi_clear_sources(pa.plan, ipw + 1, -1))
        for iss in range(pa.nss):
            sw = pa.srcwav[ipw][iss]
            fpeaks = []
            for f in sw.fields:
                w = np.asarray(sw.d[f], np.float32)
                if st == 0:
                    w = np.zeros_like(w)
                elif st == -1:
                    if f not in ("vx", "vy", "vz"):
                        raise ValueError("time-reversed sources act on velocities only (source.jl:8-19)")
                    w = S.reverse_source(w)
                if np.all(w == 0):
                    continue
                # frequency bounds come from the first wavefield only
                # (source.jl:231-246); the adjoint sources need no spectrum
                if ipw == 0:
                    fpeaks.append(S.findfreq_peak(w, pa.dt))
                    fmaxs.append(S.findfreq(w, pa.dt, "max"))
                wf = np.asfortranarray(w, np.float32)
                if ipw == 0:
                    cp, rv, nz = pa._proj(f, pa.ageom[iss].points("s", pa.ndim))
                    pa._check(pa.L.gpi_set_sources(pa.plan, 1, iss, _lib.FIELD[f], sw.n, _ptr(cp), _ptr(rv),
                                                   _ptr(nz), _ptr(wf)))
                else:
                    pa._check(pa.L.gpi_set_sources(pa.plan, 2, iss, _lib.FIELD[f], sw.n, None, None, None,
                                                   _ptr(wf)))
            if fpeaks and ipw == 0:
                peaks.append(np.mean(fpeaks))
    if pa.shard:
        # the peak frequency (it sets the CPML alpha) and the highest
        # frequency come from the sources of every rank, as on one host
        n = _shots.reduce_scalar(len(peaks))
        tot = _shots.reduce_scalar(float(np.sum(np.asarray(peaks, np.float64))))
        peaks = [tot / n] if n else []
        fm = -_shots.reduce_scalar(-(min(fmaxs) if fmaxs else np.inf), op="max")
        fmaxs = [fm] if np.isfinite(fm) else []
    if fmaxs:
        pa.freqmax = float(min(fmaxs))  # fill_wavelets! (src/fdtd/source.jl:46-53)
    if peaks:
        pa.freqpeak = np.float32(np.mean(peaks))
    elif not hasattr(pa, "freqpeak"):
        pa.freqpeak = np.float32(0.0)
    pa._src_types = list(src_types)
    return pa


# ----------------------------------------------------------------------
# model vector (log-parameterised inner grid) and the FWI gradient
# ----------------------------------------------------------------------
def _inner(pa):
    sl = []
    names = S.axis_names(pa.ndim)
    for g, d in zip(pa.exgrid, names):
        lo = pa.npml if pa.pml_mask & S.FACE_BITS[d + "min"] else 0
        hi = pa.npml if pa.pml_mask & S.FACE_BITS[d + "max"] else 0
        sl.append(slice(lo, len(g) - hi))
    return tuple(sl)


def get_modelvector(pa, mparams):
    """m = log(mod / ref) on the inner grid (src/fdtd/medium.jl:3-7, :55-76)."""
    inn = _inner(pa)
    return np.concatenate([np.log(pa.mod[k][inn] * (np.float32(1) / pa.ref_mod[k])).astype(np.float32).ravel(order="F")
                           for k in mparams])


def _update_modelvector(pa, m, mparams):
    """update!(pa, m, mparams) (src/fdtd/medium.jl:31-52)."""
    inn = _inner(pa)
    chunks = np.split(np.asarray(m, np.float32), len(mparams))
    for k, x in zip(mparams, chunks):
        view = pa.mod[k][inn]
        pa.mod[k][inn] = (np.exp(x.reshape(view.shape, order="F")) * pa.ref_mod[k]).astype(np.float32)
    pa._upload_medium()
    return pa


def lossvalue(m, loss, dobs, pa, mparams=("invK", "rho")):
    """lossvalue (src/fdtd/func_grad.jl:1-9)."""
    update(pa, m, list(mparams))
    mode_save = pa.attrib.mode
    pa.attrib.mode = "forward_save"
    update(pa, pa.srcwav, [1, 0])
    update(pa)
    pa.attrib.mode = mode_save
    return _loss(loss, dobs, pa)


def _local(pa, lst):
    """The entries of this rank's supersources from a list over all of them
    (unchanged when the experiment is not sharded or `lst` is local)."""
    if pa.shard and len(lst) == pa.nss_global:
        return [lst[i] for i in pa.shot_ids]
    return lst


def _on_device(loss, pa):
    """L2DistLoss on a plan with an adjoint wavefield and velocity records:
    misfit and adjoint sources are computed on the device."""
    return type(loss) is L2DistLoss and pa.attrib.npw == 2 and all(f in ("vx", "vy", "vz") for f in pa.rfields)


def _device_l2(pa, dobs, dobs_dev=None):
    """Adjoint sources 2 (dobs - dcal) reversed and the misfit sum
    (dobs - dcal)^2 from the records of the last run, on the device
    (gpi_set_adjoint_l2); the misfit summed over the ranks.  dobs_dev: the
    same observed data already on the device (per local shot, per field, a
    tensor in the Recs layout)."""
    pa._check(pa.L.gpi_clear_sources(pa.plan, 2, -1))
    J = 0.0
    for iss, o in enumerate(_local(pa, dobs)):
        for f in pa.rfields:
            mis = ctypes.c_double()
            if dobs_dev is not None:
                ptr = ctypes.cast(dobs_dev[iss][f].data_ptr(), ctypes.POINTER(ctypes.c_float))
                pa._check(pa.L.gpi_set_adjoint_l2(pa.plan, iss, _lib.FIELD[f], ptr, 1, ctypes.byref(mis)))
            else:
                d = np.asfortranarray(o.d[f], dtype=np.float32)
                pa._check(pa.L.gpi_set_adjoint_l2(pa.plan, iss, _lib.FIELD[f], _ptr(d), 0, ctypes.byref(mis)))
            J += mis.value
    return _shots.reduce_scalar(J) if pa.shard else J


def _loss(loss, dobs, pa):
    """Misfit of the last forward records against dobs, summed over the
    ranks of a sharded experiment."""
    if _on_device(loss, pa):
        return _device_l2(pa, dobs)
    J = sum(loss.value(o.d[f], c.d[f]) for o, c in zip(_local(pa, dobs), pa.data[0]) for f in o.fields)
    return _shots.reduce_scalar(J) if pa.shard else J


def gradient(g, m, loss, dobs, pa, mparams=("invK", "rho")):
    """gradient!(g, m, loss, dobs, pa, mparams) (src/fdtd/func_grad.jl:11-49):
    forward_save, adjoint sources deriv(loss, dobs, dcal) reversed in time,
    adjoint run with src_types [-1, 1], chain rule g * exp(m) * ref.  With
    L2DistLoss the adjoint sources and the misfit are computed on the device
    from the records there (gpi_set_adjoint_l2); pa.srcwav[2] then keeps its
    previous host contents.  On a plan with its own stream (and no
    checkpoints) the host's copies run beside the device work: the observed
    data go up on a second stream during the forward_save run, and the
    records of that run come down on it during the adjoint run (which
    records nothing)."""
    if _on_device(loss, pa) and pa.stream is not None and not pa.checkpoints:
        gv = _gradient_overlapped(pa, m, loss, dobs, mparams)
    else:
        _forward_save(pa, m, mparams)
        gv = _adjoint(pa, m, loss, dobs, mparams)
    if g is not None:
        g[:] = gv
    J = getattr(pa, "_device_misfit", None)
    return J if J is not None else _loss(loss, dobs, pa)


def _gradient_overlapped(pa, m, loss, dobs, mparams):
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    main = torch.cuda.ExternalStream(pa.stream, device=dev)
    side = torch.cuda.Stream(device=dev)
    _forward_save(pa, m, mparams, read_records=False)
    fwd = torch.cuda.Event()
    fwd.record(main)
    with torch.cuda.stream(side):
        dobs_dev = [{f: torch.from_numpy(np.ravel(np.asarray(o.d[f], np.float32), order="F")).to(dev, non_blocking=True)
                     for f in pa.rfields} for o in _local(pa, dobs)]
    up = torch.cuda.Event()
    up.record(side)
    main.wait_event(up)

    def records_beside():
        # the plan's record buffers on the second stream, after the
        # forward_save run, while the adjoint run goes on
        side.wait_event(fwd)
        pa._check(pa.L.gpi_set_stream(pa.plan, ctypes.c_void_p(side.cuda_stream)))
        try:
            for iss in range(pa.nss):
                for f in pa.rfields:
                    pa.data[0][iss].d[f] = pa.records(iss, f)
        finally:
            pa._check(pa.L.gpi_set_stream(pa.plan, ctypes.c_void_p(pa.stream)))

    gv = _adjoint(pa, m, loss, dobs, mparams, dobs_dev=dobs_dev, after_launch=records_beside)
    main.synchronize()  # the observed data stay alive until the adjoint sources are formed
    del dobs_dev
    return gv


def _forward_save(pa, m, mparams, read_records=True):
    """The first half of gradient!: update!(pa, m), forward_save run (the
    boundary store, or the checkpoints of a checkpointed plan, stay on the
    device); without read_records the run is only launched."""
    update(pa, m, list(mparams))
    mode_save = pa.attrib.mode
    pa.attrib.mode = "forward_save"
    update(pa, pa.srcwav, [1, 0])
    if read_records:
        update(pa)
    else:
        pa.run(_lib.FORWARD_SAVE)
    pa.attrib.mode = mode_save


def _adjoint(pa, m, loss, dobs, mparams, scale=1.0, dobs_dev=None, after_launch=None):
    """The second half of gradient!: adjoint sources from the records of the
    last forward_save run, the adjoint run, the chain rule onto m (times
    `scale`).  after_launch runs on the host once the adjoint run is
    queued."""
    mparams = list(mparams)
    # a checkpointed plan recomputes wavefield 1 forward in time, with the
    # sources of its forward_save run (no time-reversed copy is needed)
    st1 = 1 if pa.checkpoints else -1
    pa._device_misfit = None
    if _on_device(loss, pa):
        # adjoint sources 2 (dobs - dcal) reversed, and the misfit, on the
        # device from the records there
        pa._device_misfit = _device_l2(pa, dobs, dobs_dev)
        _update_srcwav(pa, [pa.srcwav[0]], [st1], ipws=(0,))
    else:
        adj = []
        for o, c in zip(_local(pa, dobs), pa.data[0]):
            s = Srcs(o.n, pa.tgrid, pa.rfields)
            for f in pa.rfields:
                # reverse!(srcwav[2]), laid out as the engine takes wavelets
                s.d[f] = np.asfortranarray(loss.deriv(o.d[f], c.d[f])[::-1])
            adj.append(s)
        pa.srcwav[1] = adj
        update(pa, pa.srcwav, [st1, 1])
    mode_save = pa.attrib.mode
    pa.attrib.mode = "adjoint"
    update(pa)
    pa.attrib.mode = mode_save
    if after_launch is not None:
        after_launch()
    inn = _inner(pa)
    chunks = np.split(np.asarray(m, np.float32), len(mparams))
    out = []
    pidx = {"invK": 0, "rho": 1} if pa.attrib.physics == "acoustic" else {"invlambda": 0, "invmu": 1, "rho": 2}
    raw = {}
    for k, x in zip(mparams, chunks):
        gr = pa.gradient_raw(pidx[k])
        raw[k] = gr
        gm = gr[inn]
        gm = gm * np.exp(x.reshape(gm.shape, order="F")) * pa.ref_mod[k]
        out.append(gm.astype(np.float32).ravel(order="F"))
    pa.gradients = raw
    gv = np.concatenate(out)
    if pa.shard:
        _shots.reduce_gradient(gv)
    return gv if scale == 1.0 else (gv * np.float32(scale)).astype(np.float32)
