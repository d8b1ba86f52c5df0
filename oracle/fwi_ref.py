"""Inversion-grid misfit and gradient of SeisInvExpt, restated for the CPU
oracle (test infrastructure only).

src/fwi/func_grad.jl:1-62 and src/fwi/fwi.jl:10-46: one 1-D interpolation
matrix per axis maps a model on the inversion grid to the modelling grid
(apply_proj_matrix! with P, the 1-D form of bilinear_interp and
get_neighbour_indices, src/proj_mat.jl:69-203); the gradient on the
inversion grid is the modelling-grid gradient brought back with the
transposed matrices; update!(pa, m, mparams) replaces only the inner
(non-PML) cells of the extended medium (src/fdtd/medium.jl:31-52).
"""
import numpy as np

from . import setup_ref as S


def interp_1d(grid, points):
    """(len(grid), len(points)) weights: column j interpolates points[j]
    linearly between its two neighbours on `grid`, clamped outside."""
    grid = np.asarray(grid, np.float64)
    out = np.zeros((len(grid), len(points)), np.float64)
    for j, x in enumerate(points):
        i1, i2 = S._neighbours(grid, x)
        f = S._frac(grid, x, i1, i2)
        out[i1, j] += 1.0 - f
        out[i2, j] += f
    return out.astype(np.float32)


def along_axes(m, mats):
    """m'[i, j, ...] = sum_k,l P[k, i] Q[l, j] ... m[k, l, ...]."""
    out = np.asarray(m, np.float64)
    for ax, P in enumerate(mats):
        out = np.moveaxis(np.tensordot(np.asarray(P, np.float64).T, np.moveaxis(out, ax, 0), axes=1), 0, ax)
    return out


def inversion_matrices(mmgrid, migrid):
    """P per axis (inversion grid -> modelling grid)."""
    return [interp_1d(mi, mm) for mm, mi in zip(mmgrid, migrid)]


def to_full(m, P, mparams):
    """Model vector on the inversion grid -> model vector on the modelling
    grid (lossvalue / gradient! of SeisInvExpt)."""
    ni = tuple(P_.shape[0] for P_ in P)
    return np.concatenate([along_axes(c.reshape(ni, order="F"), P).astype(np.float32).ravel(order="F")
                           for c in np.split(np.asarray(m, np.float64), len(mparams))])


def to_inversion(gfull, P, mparams):
    """Gradient on the modelling grid -> gradient on the inversion grid."""
    nm = tuple(P_.shape[1] for P_ in P)
    return np.concatenate([along_axes(c.reshape(nm, order="F"), [P_.T for P_ in P]).ravel(order="F")
                           for c in np.split(np.asarray(gfull, np.float64), len(mparams))])


def medium_from_modelvector(prep, mfull, mparams, ref):
    """update!(pa, m, mparams): the extended medium with its inner cells
    replaced by ref * exp(m) (ref: the parameters' reference values); the
    PML cells keep their padded values."""
    inner = []
    names = "zyx" if prep.ndim == 3 else "zx"
    for i, d in enumerate(names):
        lo = prep.npml if prep.faces & S.FACE_BITS[d + "min"] else 0
        hi = prep.npml if prep.faces & S.FACE_BITS[d + "max"] else 0
        inner.append(slice(lo, prep.shape[i] - hi))
    inner = tuple(inner)
    idx = {"invK": 0, "rho": 1}
    mod = [m.copy() for m in prep.mod]
    for k, c in zip(mparams, np.split(np.asarray(mfull, np.float32), len(mparams))):
        view = mod[idx[k]][inner]
        mod[idx[k]][inner] = (np.exp(c.reshape(view.shape, order="F")) * np.float32(ref[k])).astype(np.float32)
    return mod
