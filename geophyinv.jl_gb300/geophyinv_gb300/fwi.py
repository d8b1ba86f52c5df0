"""Full-waveform inversion driver over the engine's gradient.

Mirrors the reference's SeisInvExpt (src/fwi/fwi.jl:10-36) and its misfit
on an inversion grid (src/fwi/func_grad.jl:1-62): the model vector lives on
a coarse inversion grid, one linear-interpolation matrix per axis maps it to
the modelling grid (get_proj_matrix / bilinear_interp, src/proj_mat.jl:
69-247, applied axis by axis as apply_proj_matrix!), the gradient comes back
through the transposed matrices, and `update(paw)` runs L-BFGS on the pair
(the reference calls Optim.LBFGS, src/fwi/fwi.jl:131-143; here
scipy.optimize's L-BFGS-B without bounds).

Model vectors are log(m / ref) as in get_modelvector (medium.jl:3-7).
"""
import numpy as np

from .fdtd import L2DistLoss, get_modelvector, gradient, lossvalue


def _neighbours(arr, val):
    """get_neighbour_indices (src/proj_mat.jl:69-79), 0-based."""
    n = len(arr)
    idx = int(np.searchsorted(arr, val, side="left"))  # searchsortedfirst - 1
    if idx == 0:
        return 0, 1
    if idx >= n - 1:
        return n - 2, n - 1
    return idx - 1, idx


def interp_matrix(grid, points):
    """Column j: the 1-D linear-interpolation weights of points[j] on `grid`
    (bilinear_interp(x, xi), src/proj_mat.jl:168-203: clamped to the end
    values outside the grid).  Shape (len(grid), len(points))."""
    grid = np.asarray(grid, np.float64)
    out = np.zeros((len(grid), len(points)), np.float32)
    lo_v, hi_v = grid.min(), grid.max()
    for j, x in enumerate(points):
        i1, i2 = _neighbours(grid, x)
        if x < lo_v:
            dx = 0.0
        elif x > hi_v:
            dx = 1.0
        else:
            dx = (x - grid[i1]) / (grid[i2] - grid[i1])
        out[i1, j] += np.float32(1.0 - dx)
        out[i2, j] += np.float32(dx)
    return out


def _apply(m, mats):
    """apply_proj_matrix!: m1[i, j(, o)] = sum P[k, i] m[k, l(, n)] Q[l, j] (R[n, o])."""
    out = np.asarray(m, np.float64)
    for ax, P in enumerate(mats):
        out = np.moveaxis(np.tensordot(np.asarray(P, np.float64), np.moveaxis(out, ax, 0), axes=([0], [0])), 0, ax)
    return out


class SeisInvExpt:
    """SeisInvExpt(paf, dobs, migrid, mparams; loss) (src/fwi/fwi.jl:10-36).
    `migrid`: one coordinate array per axis, or a list of cell counts
    (spread over the modelling grid less 4 cells at each end, as the
    reference's Nigrid form, src/fwi/fwi.jl:39-46)."""

    def __init__(self, paf, dobs, migrid=None, mparams=("invK", "rho"), loss=None):
        self.paf = paf
        self.dobs = dobs
        self.mparams = list(mparams)
        self.loss = loss if loss is not None else L2DistLoss()
        mm = [g.values() if hasattr(g, "values") else np.asarray(g, np.float64) for g in paf.medium.grid]
        self.mmgrid = mm
        if migrid is None:
            migrid = mm
        elif all(np.isscalar(n) for n in migrid):
            migrid = [np.linspace(g[0] + 4 * (g[1] - g[0]), g[-1] - 4 * (g[1] - g[0]), int(n))
                      for g, n in zip(mm, migrid)]
        self.migrid = [np.asarray(g, np.float64) for g in migrid]
        # inversion grid -> modelling grid, and the restriction used for the
        # starting model (fwi.jl:12-16, func_grad.jl:1-22)
        self.P = [interp_matrix(mi, mmx) for mi, mmx in zip(self.migrid, mm)]
        self.R = [interp_matrix(mmx, mi) for mi, mmx in zip(self.migrid, mm)]
        self.mfull = get_modelvector(paf, self.mparams)
        self.gmfull = np.zeros_like(self.mfull)
        self.history = []

    @property
    def nm(self):
        return len(self.mparams) * int(np.prod([len(g) for g in self.migrid]))

    def _to_full(self, m):
        shp_i = tuple(len(g) for g in self.migrid)
        shp_m = tuple(len(g) for g in self.mmgrid)
        out = []
        for mc in np.split(np.asarray(m, np.float64), len(self.mparams)):
            out.append(_apply(mc.reshape(shp_i, order="F"), self.P).astype(np.float32).ravel(order="F"))
        assert out[0].size == int(np.prod(shp_m))
        return np.concatenate(out)

    def _to_inv(self, gfull):
        shp_m = tuple(len(g) for g in self.mmgrid)
        out = []
        for gc in np.split(np.asarray(gfull, np.float64), len(self.mparams)):
            out.append(_apply(gc.reshape(shp_m, order="F"), [P.T for P in self.P]).ravel(order="F"))
        return np.concatenate(out)


def get_modelvector_inv(paw):
    """get_modelvector(pa::SeisInvExpt) (src/fwi/func_grad.jl:1-22): the
    modelling-grid model restricted to the inversion grid."""
    mfull = get_modelvector(paw.paf, paw.mparams)
    shp_m = tuple(len(g) for g in paw.mmgrid)
    out = []
    for mc in np.split(np.asarray(mfull, np.float64), len(paw.mparams)):
        out.append(_apply(mc.reshape(shp_m, order="F"), paw.R).ravel(order="F"))
    return np.concatenate(out).astype(np.float32)


def lossvalue_inv(m, paw):
    """lossvalue(m, pa::SeisInvExpt) (src/fwi/func_grad.jl:24-40)."""
    paw.mfull = paw._to_full(m)
    return lossvalue(paw.mfull, paw.loss, paw.dobs, paw.paf, paw.mparams)


def gradient_inv(g, m, paw):
    """gradient!(g, m, pa::SeisInvExpt) (src/fwi/func_grad.jl:42-62): the
    modelling-grid gradient brought back through the transposed
    interpolation matrices."""
    paw.mfull = paw._to_full(m)
    J = gradient(paw.gmfull, paw.mfull, paw.loss, paw.dobs, paw.paf, paw.mparams)
    gi = paw._to_inv(paw.gmfull)
    if g is not None:
        g[:] = gi
    return J, gi


def update(paw, maxiter=10, m0=None, callback=None):
    """update!(paw) (src/fwi/fwi.jl:131-143): L-BFGS on lossvalue /
    gradient!; the model ends in paw.paf.  Returns the scipy result; the
    misfit of every evaluation is in paw.history."""
    from scipy.optimize import minimize

    m0 = get_modelvector_inv(paw) if m0 is None else np.asarray(m0, np.float32)

    def fg(x):
        J, gi = gradient_inv(None, x.astype(np.float32), paw)
        paw.history.append(J)
        return float(J), gi.astype(np.float64)

    res = minimize(fg, m0.astype(np.float64), jac=True, method="L-BFGS-B",
                   options={"maxiter": int(maxiter), "gtol": 1e-25, "ftol": 0.0}, callback=callback)
    paw.mfull = paw._to_full(res.x.astype(np.float32))
    lossvalue(paw.mfull, paw.loss, paw.dobs, paw.paf, paw.mparams)
    return res
