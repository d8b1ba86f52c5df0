"""The FWI driver's host parts (no GPU): the inversion-grid interpolation
matrices (bilinear_interp in 1-D, src/proj_mat.jl:168-203, clamped outside
the grid) and the projection / transposed projection pair."""
import numpy as np

from geophyinv_gb300 import fwi


def test_interp_matrix_is_linear_interpolation_clamped_outside():
    grid = np.linspace(0.0, 10.0, 6)  # 0, 2, ..., 10
    pts = np.array([-1.0, 0.0, 1.0, 3.5, 10.0, 12.0])
    M = fwi.interp_matrix(grid, pts)
    assert M.shape == (6, 6)
    np.testing.assert_allclose(M.sum(0), 1.0, rtol=0, atol=1e-7)
    f = 3.0 * grid + 1.0
    vals = f @ M
    np.testing.assert_allclose(vals, [1.0, 1.0, 4.0, 11.5, 31.0, 31.0], rtol=1e-6)


def test_projection_and_its_transpose_are_adjoint():
    class _G:
        def __init__(self, v):
            self.v = v

        def values(self):
            return self.v

    rng = np.random.default_rng(0)
    paw = fwi.SeisInvExpt.__new__(fwi.SeisInvExpt)
    paw.mparams = ["invK", "rho"]
    paw.mmgrid = [np.linspace(0, 100, 21), np.linspace(0, 200, 31)]
    paw.migrid = [np.linspace(10, 90, 5), np.linspace(20, 180, 7)]
    paw.P = [fwi.interp_matrix(mi, mm) for mi, mm in zip(paw.migrid, paw.mmgrid)]
    x = rng.standard_normal(2 * 5 * 7)
    y = rng.standard_normal(2 * 21 * 31)
    # <P x, y> = <x, P^T y>
    lhs = float(paw._to_full(x).astype(np.float64) @ y)
    rhs = float(x @ paw._to_inv(y))
    assert abs(lhs - rhs) <= 1e-5 * abs(rhs)


def test_projections_match_the_oracle_restatement():
    """The product's inversion-grid matrices and projections against the
    oracle's restatement of SeisInvExpt (oracle/fwi_ref.py)."""
    from oracle import fwi_ref as R

    rng = np.random.default_rng(3)
    mm = [np.linspace(0, 100, 21), np.linspace(0, 200, 31)]
    mi = [np.linspace(10, 90, 5), np.linspace(20, 180, 7)]
    P = R.inversion_matrices(mm, mi)
    paw = fwi.SeisInvExpt.__new__(fwi.SeisInvExpt)
    paw.mparams = ["invK", "rho"]
    paw.mmgrid, paw.migrid = mm, mi
    paw.P = [fwi.interp_matrix(a, b) for a, b in zip(mi, mm)]
    for A, B in zip(paw.P, P):
        np.testing.assert_array_equal(A, B)
    x = rng.standard_normal(2 * 5 * 7).astype(np.float32)
    y = rng.standard_normal(2 * 21 * 31).astype(np.float32)
    np.testing.assert_allclose(paw._to_full(x), R.to_full(x, P, paw.mparams), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(paw._to_inv(y), R.to_inversion(y, P, paw.mparams), rtol=1e-6, atol=1e-6)
