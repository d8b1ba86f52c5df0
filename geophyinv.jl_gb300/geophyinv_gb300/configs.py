"""Synthetic workloads of the benchmark configurations.

No external data is used: models are seeded layered / gradient media with a
Gaussian-smoothed random perturbation, wavelets are Ricker wavelets.

  acoustic2d_layers  2-D acoustic forward, 201 x 301 at 5 m, 2000 steps
                     (3 layers, sigma 8 cells, +-5 %, Ricker 15 Hz on p)
  elastic2d_batch    2-D elastic P-SV forward, 1000 x 3000 at 5 m, 16 shots,
                     4000 steps (linear vp 1800->4500, vs = vp/1.8, Gardner rho,
                     sigma 15 cells, +-8 %, Ricker 12 Hz explosive)
  acoustic2d_fwi     2-D acoustic gradient, 500 x 1500 at 10 m, 32 shots,
                     3000 steps (layers + 200 m Gaussian anomaly of +10 %)
  elastic3d          3-D elastic forward, 600^3 at 10 m, 20-cell CPML (npml 23),
                     2500 steps (linear vp 2000->5000, vs = vp/1.75, Gardner rho,
                     sigma 10 cells, +-5 %, Ricker 10 Hz explosive at 50 m,
                     121 x 121 surface receivers)
  acoustic3d         the same medium, acoustic, p source

Every builder accepts overrides (sizes, steps, shot count) so tests can run
reduced versions with the same shapes of inputs.
"""
import numpy as np

from .setup import Grid, ricker


def smooth_noise(shape, sigma, seed):
    """N(0,1) smoothed by a Gaussian of `sigma` cells, scaled to peak 1."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    f = gaussian_filter(rng.standard_normal(shape), sigma, mode="reflect")
    return f / np.max(np.abs(f))


class Workload:
    """A complete forward (or gradient) experiment in plain arrays."""

    def __init__(self, name, physics, grid, vp, rho, vs=None, shots=(), tgrid=None, wavelet=None,
                 rfields=("vz",), pml_faces=("zmin", "zmax", "ymin", "ymax", "xmin", "xmax"),
                 stressfree_faces=(), src_field="p", npml=None):
        self.name = name
        self.physics = physics
        self.grid = grid
        self.vp = np.asarray(vp, np.float32)
        self.rho = np.asarray(rho, np.float32)
        self.vs = None if vs is None else np.asarray(vs, np.float32)
        self.shots = list(shots)  # list of (src points (ns, ndim), rec points (nr, ndim))
        self.tgrid = tgrid
        self.wavelet = np.asarray(wavelet, np.float32)
        self.rfields = list(rfields)
        self.pml_faces = list(pml_faces)
        self.stressfree_faces = list(stressfree_faces)
        self.src_field = src_field
        self.npml = npml

    @property
    def ndim(self):
        return len(self.grid)

    @property
    def nt(self):
        return len(self.tgrid)

    def cells(self, npml=None):
        npml = npml if npml is not None else (self.npml if self.npml is not None else 43)
        n = 1
        for g in self.grid:
            n *= len(g) + 2 * npml
        return n

    # --- product side ---
    def medium(self):
        from .fdtd import AcousticMedium, ElasticMedium

        if self.physics == "acoustic":
            return AcousticMedium(self.grid, self.vp, self.rho)
        return ElasticMedium(self.grid, self.vp, self.vs, self.rho)

    def ageom(self):
        from .fdtd import AGeomss

        names = "zyx" if self.ndim == 3 else "zx"
        out = []
        for s, r in self.shots:
            s = np.atleast_2d(s)
            r = np.atleast_2d(r)
            out.append(AGeomss({a: s[:, i] for i, a in enumerate(names)}, {a: r[:, i] for i, a in enumerate(names)}))
        return out

    def srcwav(self):
        from .fdtd import Srcs

        out = []
        for s, _ in self.shots:
            ns = len(np.atleast_2d(s))
            out.append(Srcs(ns, self.tgrid, [self.src_field],
                            {self.src_field: np.repeat(self.wavelet[:, None], ns, 1).astype(np.float32)}))
        return out

    def expt(self, mode="forward", **kw):
        from .fdtd import FdtdAcoustic, FdtdElastic, SeisForwExpt

        attrib = (FdtdAcoustic if self.physics == "acoustic" else FdtdElastic)(mode)
        if self.npml is not None:
            kw.setdefault("npml", self.npml)
        return SeisForwExpt(attrib, medium=self.medium(), ageom=self.ageom(), srcwav=self.srcwav(),
                            tgrid=self.tgrid, rfields=self.rfields, pml_faces=self.pml_faces,
                            stressfree_faces=self.stressfree_faces, **kw)

    # --- plain description (as consumed by a CPU checker) ---
    def as_dict(self):
        from .setup import face_mask

        shots = []
        for s, r in self.shots:
            s = np.atleast_2d(s)
            ns = len(s)
            shots.append({"src": {self.src_field: ([tuple(p) for p in s], np.repeat(self.wavelet[:, None], ns, 1))},
                          "rec": [tuple(p) for p in np.atleast_2d(r)]})
        d = {"physics": self.physics, "ndim": self.ndim, "order": 4,
             "grid": [(g.start, g.step, g.n) for g in self.grid], "vp": self.vp, "rho": self.rho,
             "pml_faces": face_mask(self.pml_faces), "free_faces": face_mask(self.stressfree_faces),
             "dt": self.tgrid.step, "nt": self.nt, "shots": shots, "rfields": self.rfields}
        if self.vs is not None:
            d["vs"] = self.vs
        if self.npml is not None:
            d["npml"] = int(self.npml)
        return d


def _layers(nz, nx, vps, rhos):
    vp = np.empty((nz, nx), np.float32)
    rho = np.empty((nz, nx), np.float32)
    bounds = np.linspace(0, nz, len(vps) + 1).round().astype(int)
    for i, (v, r) in enumerate(zip(vps, rhos)):
        vp[bounds[i]:bounds[i + 1]] = v
        rho[bounds[i]:bounds[i + 1]] = r
    return vp, rho


def acoustic2d_layers(nz=201, nx=301, d=5.0, nt=2000, dt=0.0005, nrec=101, seed=0, f0=15.0,
                      rfields=("p", "vx", "vz"), src_field="p"):
    """2-D acoustic forward on three flat layers with a smooth perturbation."""
    vp, rho = _layers(nz, nx, (1500.0, 2500.0, 3500.0), (1000.0, 2000.0, 2500.0))
    pert = 0.05 * smooth_noise((nz, nx), 8.0, seed)
    vp = (vp * (1 + pert)).astype(np.float32)
    rho = (rho * (1 + pert)).astype(np.float32)
    grid = [Grid(0.0, d, nz), Grid(0.0, d, nx)]
    tgrid = Grid(0.0, dt, nt)
    xm = grid[1].last
    src = np.array([[min(10.0, grid[0].last), 0.5 * xm]])
    rec = np.stack([np.zeros(nrec), np.linspace(0.0, xm, nrec)], 1)
    return Workload("acoustic2d_layers", "acoustic", grid, vp, rho, shots=[(src, rec)], tgrid=tgrid,
                    wavelet=ricker(f0, tgrid), rfields=rfields, src_field=src_field)


def gardner(vp):
    return (310.0 * vp ** 0.25).astype(np.float32)


def elastic2d_batch(nz=1000, nx=3000, d=5.0, nt=4000, dt=0.0004, nshots=16, nrec=601, seed=1, f0=12.0,
                    rfields=("vx", "vz"), src_field="tauxx"):
    """2-D elastic P-SV forward, a batch of surface shots."""
    z = np.linspace(0.0, 1.0, nz)[:, None]
    vp = np.broadcast_to(1800.0 + (4500.0 - 1800.0) * z, (nz, nx)).astype(np.float32)
    pert = 0.08 * smooth_noise((nz, nx), 15.0, seed)
    vp = (vp * (1 + pert)).astype(np.float32)
    vs = (vp / 1.8).astype(np.float32)
    rho = gardner(vp)
    grid = [Grid(0.0, d, nz), Grid(0.0, d, nx)]
    tgrid = Grid(0.0, dt, nt)
    xm = grid[1].last
    zs = min(10.0, grid[0].last)
    xs = np.linspace(0.0, xm, nshots + 2)[1:-1]
    rec = np.stack([np.zeros(nrec), np.linspace(0.0, xm, nrec)], 1)
    shots = [(np.array([[zs, x]]), rec) for x in xs]
    return Workload("elastic2d_batch", "elastic", grid, vp, rho, vs=vs, shots=shots, tgrid=tgrid,
                    wavelet=ricker(f0, tgrid), rfields=rfields, src_field=src_field)


def acoustic2d_fwi(nz=500, nx=1500, d=10.0, nt=3000, dt=0.001, nshots=32, nrec=None, seed=0, f0=8.0,
                   anomaly=True, radius=200.0, amp=0.10):
    """2-D acoustic FWI gradient workload: layered model (+ anomaly)."""
    vp, rho = _layers(nz, nx, (1500.0, 2500.0, 3500.0), (1000.0, 2000.0, 2500.0))
    pert = 0.05 * smooth_noise((nz, nx), 8.0, seed)
    vp = (vp * (1 + pert)).astype(np.float32)
    rho = (rho * (1 + pert)).astype(np.float32)
    if anomaly:
        zz = np.arange(nz)[:, None] * d
        xx = np.arange(nx)[None, :] * d
        zc, xc = 0.5 * (nz - 1) * d, 0.5 * (nx - 1) * d
        g = np.exp(-((zz - zc) ** 2 + (xx - xc) ** 2) / (2 * radius ** 2))
        vp = (vp * (1 + amp * g)).astype(np.float32)
    grid = [Grid(0.0, d, nz), Grid(0.0, d, nx)]
    tgrid = Grid(0.0, dt, nt)
    xm = grid[1].last
    nrec = nrec or nx
    rec = np.stack([np.full(nrec, min(2 * d, grid[0].last)), np.linspace(0.0, xm, nrec)], 1)
    xs = np.linspace(0.0, xm, nshots + 2)[1:-1]
    shots = [(np.array([[min(2 * d, grid[0].last), x]]), rec) for x in xs]
    return Workload("acoustic2d_fwi", "acoustic", grid, vp, rho, shots=shots, tgrid=tgrid,
                    wavelet=ricker(f0, tgrid), rfields=("vz",), src_field="vz")


def _media3d(nz, ny, nx, d, seed, vp0=2000.0, vp1=5000.0, pert=0.05, sigma=10.0, vsr=1.75):
    z = np.linspace(0.0, 1.0, nz)[:, None, None]
    vp = np.broadcast_to(vp0 + (vp1 - vp0) * z, (nz, ny, nx)).astype(np.float32)
    vp = (vp * (1 + pert * smooth_noise((nz, ny, nx), sigma, seed))).astype(np.float32)
    return vp, (vp / vsr).astype(np.float32), gardner(vp)


def _surface_receivers(grid, nside):
    ym, xm = grid[1].last, grid[2].last
    yy, xx = np.meshgrid(np.linspace(0.0, ym, nside), np.linspace(0.0, xm, nside), indexing="ij")
    return np.stack([np.zeros(yy.size), yy.ravel(), xx.ravel()], 1)


def elastic3d(nz=600, ny=600, nx=600, d=10.0, nt=2500, dt=0.0008, npml=23, nrec_side=121, seed=3, f0=10.0,
              zsrc=50.0, rfields=("vz",), src_field="tauxx"):
    """3-D elastic forward: explosive source centred at zsrc, surface grid of
    receivers."""
    vp, vs, rho = _media3d(nz, ny, nx, d, seed)
    grid = [Grid(0.0, d, nz), Grid(0.0, d, ny), Grid(0.0, d, nx)]
    tgrid = Grid(0.0, dt, nt)
    src = np.array([[min(zsrc, grid[0].last), 0.5 * grid[1].last, 0.5 * grid[2].last]])
    rec = _surface_receivers(grid, nrec_side)
    return Workload("elastic3d", "elastic", grid, vp, rho, vs=vs, shots=[(src, rec)], tgrid=tgrid,
                    wavelet=ricker(f0, tgrid), rfields=rfields, src_field=src_field, npml=npml)


def acoustic3d(nz=600, ny=600, nx=600, d=10.0, nt=2500, dt=0.0008, npml=23, nrec_side=121, seed=3, f0=10.0,
               zsrc=50.0, rfields=("p", "vz"), src_field="p"):
    """3-D acoustic forward on the medium of elastic3d."""
    vp, _, rho = _media3d(nz, ny, nx, d, seed)
    grid = [Grid(0.0, d, nz), Grid(0.0, d, ny), Grid(0.0, d, nx)]
    tgrid = Grid(0.0, dt, nt)
    src = np.array([[min(zsrc, grid[0].last), 0.5 * grid[1].last, 0.5 * grid[2].last]])
    rec = _surface_receivers(grid, nrec_side)
    return Workload("acoustic3d", "acoustic", grid, vp, rho, shots=[(src, rec)], tgrid=tgrid,
                    wavelet=ricker(f0, tgrid), rfields=rfields, src_field=src_field, npml=npml)
