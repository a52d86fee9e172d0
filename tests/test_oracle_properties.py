"""Property tests of the oracle for the kernels whose spread values no
reference golden pins (IB_3, IB_4, IB_6, PIECEWISE_CUBIC, BSPLINE_4):
partition of unity, vanishing first moment, conservation of the spread force
and adjointness of spreading and interpolation on a periodic grid.  CPU only."""

import numpy as np
import pytest

KERNELS = ["PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4"]


@pytest.mark.parametrize("kernel", KERNELS)
def test_partition_of_unity_and_first_moment(oracle, kernel):
    rng = np.random.default_rng(3)
    dx, x_lower, ilower, iupper = 1.0 / 64, 0.0, 0, 63
    for X in rng.uniform(0.2, 0.8, size=500):
        base, start, stop, w = oracle.stencil_1d(kernel, X, 0.0, x_lower, dx, ilower, iupper, 8)
        # getStencilSize reports 4 for IB_3, whose support has 3 points
        width = 3 if kernel == "IB_3" else oracle.stencil_size(kernel)
        assert start == 0 and stop == width - 1
        ww = w[start:stop + 1]
        xc = x_lower + (base + np.arange(start, stop + 1) - ilower + 0.5) * dx
        assert abs(ww.sum() - 1.0) <= 1e-12
        assert abs(np.dot(ww, xc - X)) <= 1e-12 * dx


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("centering", [0, 1])
def test_spread_interp_adjoint_and_conservation(oracle, dim, kernel, centering):
    rng = np.random.default_rng(100 + dim)
    N = [16, 12, 8][:dim] if dim == 3 else [24, 20]
    n = 60
    X = rng.uniform(0.0, 1.0, size=n * dim)
    ncomp = dim if centering == 1 else 2
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + N[::-1])
    f, U = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=ncomp)
    h = np.prod([1.0 / v for v in N])
    # <S F, u> h^d == <F, S* u>
    lhs = float((f * u).sum()) * h
    rhs = float(np.dot(F, U))
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(rhs))
    # the total spread force equals the total marker force, per component
    for c in range(ncomp):
        assert abs(f[c].sum() * h - F[c::ncomp].sum()) <= 1e-12 * max(1.0, np.abs(F).sum())


def _quad_mesh(m, rng, lo=0.3, hi=0.7, dim=2):
    """Perturbed structured QUAD4 (2D) / HEX8 (3D) mesh of [lo, hi]^dim in
    libMesh's node order."""
    g = np.linspace(lo, hi, m + 1)
    idx = np.stack(np.meshgrid(*([np.arange(m + 1)] * dim), indexing="ij"), axis=-1).reshape(-1, dim)
    X = g[idx] + rng.uniform(-0.25, 0.25, size=idx.shape) * ((hi - lo) / m)
    stride = [(m + 1) ** (dim - 1 - d) for d in range(dim)]
    nid = lambda c: sum(int(c[d]) * stride[d] for d in range(dim))
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)][: 2 ** dim]
    E = []
    for cell in np.ndindex(*([m] * dim)):
        E += [nid([cell[d] + c[d] for d in range(dim)]) for c in corners]
    return np.array(E, dtype=np.int32), X.reshape(-1)


def test_fe_q1_jxw_integrates_the_cells_exactly(oracle):
    """QUAD4: the 2x2 Gauss rule integrates the bilinear map's Jacobian
    exactly, so each cell's JxW sum is the quadrilateral's area (shoelace
    formula); HEX8: an affine (sheared, scaled) cube gives |det A| per cell
    and constant JxW; the basis is a partition of unity."""
    rng = np.random.default_rng(5)
    E, X = _quad_mesh(6, rng)
    g = 1 / np.sqrt(3)
    pts = np.array([[-g, -g], [g, -g], [g, g], [-g, g]])
    _, _, J = oracle.fe_quadrature_points(2, E, X, pts, np.ones(4), elem_type=oracle.FE_TENSOR_Q1)
    J = J.reshape(-1, 4)
    P = X.reshape(-1, 2)[E.reshape(-1, 4)]  # [cell, corner, xy], counter-clockwise
    area = 0.5 * np.abs(np.sum(P[:, :, 0] * np.roll(P[:, :, 1], -1, 1) - np.roll(P[:, :, 0], -1, 1) * P[:, :, 1], 1))
    assert np.max(np.abs(J.sum(1) - area)) <= 1e-14
    # HEX8 cells of an affinely mapped grid (x -> A x): each cell's JxW sum
    # is |det A| times the cell's reference volume
    A = np.array([[1.1, 0.2, 0.0], [0.1, 0.9, 0.3], [0.0, 0.05, 1.2]])
    E3, _ = _quad_mesh(3, np.random.default_rng(6), dim=3)
    grid = np.stack(np.meshgrid(*([np.linspace(0, 1, 4)] * 3), indexing="ij"), -1).reshape(-1, 3)
    Xa = (grid @ A.T).reshape(-1)
    pts3 = np.array([[sx * g, sy * g, sz * g] for sz in (-1, 1) for sy in (-1, 1) for sx in (-1, 1)])
    _, _, J3 = oracle.fe_quadrature_points(3, E3, Xa, pts3, np.ones(8), elem_type=oracle.FE_TENSOR_Q1)
    cell = abs(np.linalg.det(A)) * (1 / 3) ** 3
    assert np.max(np.abs(J3.reshape(-1, 8).sum(1) - cell)) <= 1e-14
    phi, dphi = oracle._fe_q1_basis(3, pts3)
    assert np.max(np.abs(phi.sum(1) - 1.0)) <= 1e-15 and np.max(np.abs(dphi.sum(1))) <= 1e-15
