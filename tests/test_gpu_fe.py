"""The finite-element quadrature-point path (FEDataManager::spread / interp,
ibtk/src/lagrangian/FEDataManager.cpp:1088-1219, 1873-2005) for first-order
Lagrange meshes (TRI3 / TET4 simplices and QUAD4 / HEX8 cells), on the
device: quadrature-point positions, F * JxW and JxW bit-identical to the
oracle's restatement; the spread of those values (the raw-array
LEInteractor::spread) and the interpolation at the quadrature points followed
by the right-hand-side assembly within 1e-12 of the oracle."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# libMesh-style rules on the reference simplex (weights sum to its measure):
# the 3-point rule exact for quadratics on triangles, the 4-point rule exact
# for quadratics on tetrahedra.
A3, B3 = 0.1381966011250105, 0.5854101966249685
RULES = {
    2: (np.array([[1 / 6, 1 / 6], [2 / 3, 1 / 6], [1 / 6, 2 / 3]]), np.full(3, 1 / 6)),
    3: (np.array([[A3, A3, A3], [B3, A3, A3], [A3, B3, A3], [A3, A3, B3]]), np.full(4, 1 / 24)),
}


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def mesh(dim, m, rng):
    """A perturbed simplex mesh of the box [0.3, 0.7]^dim: m^dim cells, two
    triangles (2D) or six tetrahedra (3D) per cell."""
    g = np.linspace(0.3, 0.7, m + 1)
    if dim == 2:
        I, J = np.meshgrid(np.arange(m + 1), np.arange(m + 1), indexing="ij")
        X = np.stack([g[I], g[J]], axis=-1).reshape(-1, 2)
        nid = lambda i, j: i * (m + 1) + j
        E = []
        for i in range(m):
            for j in range(m):
                a, b, c, d = nid(i, j), nid(i + 1, j), nid(i, j + 1), nid(i + 1, j + 1)
                E += [[a, b, d], [a, d, c]]
    else:
        I, J, K = np.meshgrid(np.arange(m + 1), np.arange(m + 1), np.arange(m + 1), indexing="ij")
        X = np.stack([g[I], g[J], g[K]], axis=-1).reshape(-1, 3)
        nid = lambda i, j, k: (i * (m + 1) + j) * (m + 1) + k
        E = []
        for i in range(m):
            for j in range(m):
                for k in range(m):
                    v = [nid(i + (s & 1), j + ((s >> 1) & 1), k + ((s >> 2) & 1)) for s in range(8)]
                    # Kuhn triangulation: the six paths from corner 0 to corner 7
                    for p in ([1, 2, 4], [1, 4, 2], [2, 1, 4], [2, 4, 1], [4, 1, 2], [4, 2, 1]):
                        c1 = p[0]
                        c2 = p[0] | p[1]
                        E.append([v[0], v[c1], v[c2], v[7]])
    X = X + rng.uniform(-0.3, 0.3, size=X.shape) * (0.4 / m)
    return np.array(E, dtype=np.int32).reshape(-1), X.reshape(-1)


@pytest.mark.parametrize("dim,m", [(2, 24), (3, 8)])
def test_quadrature_points_bit_identical(ibx, oracle, dim, m):
    rng = np.random.default_rng(40 + dim)
    E, X = mesh(dim, m, rng)
    pts, w = RULES[dim]
    n_vars = dim
    F = rng.standard_normal(X.size // dim * n_vars)
    Xq_ref, Fq_ref, J_ref = oracle.fe_quadrature_points(dim, E, X, pts, w, F=F, n_vars=n_vars)
    Xq, Fq, J = ibx.fe_quadrature_points(dim, torch.tensor(E, device="cuda"), torch.tensor(X, device="cuda"), pts,
                                         w, F=torch.tensor(F, device="cuda"), n_vars=n_vars)
    assert np.array_equal(Xq.cpu().numpy(), Xq_ref)
    assert np.array_equal(J.cpu().numpy(), J_ref)
    assert np.array_equal(Fq.cpu().numpy(), Fq_ref)
    # the quadrature weights add up to the mesh's measure (the box's, up to
    # the perturbation of the boundary nodes)
    vol = 0.4 ** dim
    assert abs(J.sum().item() - vol) <= 2e-2 * vol


@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "BSPLINE_4"])
@pytest.mark.parametrize("dim,m,N", [(2, 24, 64), (3, 8, 32)])
def test_fe_spread_and_interp_against_oracle(ibx, oracle, dim, m, N, kernel):
    """FEDataManager::spread: F * JxW at the quadrature points spread from
    their positions (plain FP64 and mixed forms); FEDataManager::interp:
    the field interpolated at the quadrature points and the projection's
    right-hand side assembled."""
    rng = np.random.default_rng(7 * dim + len(kernel))
    E, X = mesh(dim, m, rng)
    pts, w = RULES[dim]
    F = rng.standard_normal(X.size)
    Xq_ref, Fq_ref, _ = oracle.fe_quadrature_points(dim, E, X, pts, w, F=F, n_vars=dim)
    u = rng.standard_normal([dim] + [N] * dim)
    f_ref, U_ref = oracle.periodic_problem(dim, [N] * dim, kernel, Xq_ref, F=Fq_ref, u=u, centering=1)
    rhs_ref = oracle.fe_assemble_rhs(dim, E, X, pts, w, U_ref, dim)
    E_t, X_t = torch.tensor(E, device="cuda"), torch.tensor(X, device="cuda")
    Xq, Fq, _ = ibx.fe_quadrature_points(dim, E_t, X_t, pts, w, F=torch.tensor(F, device="cuda"), n_vars=dim)
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [N - 1] * dim,
                                       [1.0 / N] * dim, [0.0] * dim, [1.0] * dim, q, Xq, Q)
    # spread, plain FP64
    f = [torch.zeros([N] * dim, dtype=torch.float64, device="cuda") for _ in range(dim)]
    ibx.spread(mk(f, Fq), kernel, ibx.FP64)
    torch.cuda.synchronize()
    fs = np.stack([t.cpu().numpy() for t in f])
    assert np.max(np.abs(fs - f_ref)) <= 1e-12 * np.max(np.abs(f_ref))
    # spread, mixed (binned plan)
    f32 = [torch.zeros([N] * dim, dtype=torch.float32, device="cuda") for _ in range(dim)]
    plan = ibx.Plan(mk(f32, Fq.float()), kernel, ibx.MIXED)
    plan.bin()
    plan.spread()
    torch.cuda.synchronize()
    assert plan.status() == ibx.OK
    fm = np.stack([t.double().cpu().numpy() for t in f32])
    assert np.max(np.abs(fm - f_ref)) <= 1e-5 * np.max(np.abs(f_ref))
    plan.close()
    # interpolation at the quadrature points, then the right-hand side
    u_t = [torch.tensor(u[a], device="cuda") for a in range(dim)]
    Uq = torch.zeros(Xq.numel(), dtype=torch.float64, device="cuda")
    ibx.interpolate(mk(u_t, Uq), kernel, ibx.FP64)
    rhs = torch.zeros(X.size, dtype=torch.float64, device="cuda")
    ibx.fe_assemble_rhs(dim, E_t, X_t, pts, w, Uq, dim, rhs)
    torch.cuda.synchronize()
    assert np.max(np.abs(Uq.cpu().numpy() - U_ref)) <= 1e-12 * np.max(np.abs(U_ref))
    assert np.max(np.abs(rhs.cpu().numpy() - rhs_ref)) <= 1e-12 * np.max(np.abs(rhs_ref))


def test_fe_rhs_of_a_constant_field(ibx):
    """For U = 1 at every quadrature point the right-hand side sums to the
    mesh's measure per variable (partition of unity of the basis)."""
    rng = np.random.default_rng(3)
    E, X = mesh(3, 6, rng)
    pts, w = RULES[3]
    n_qp = E.size // 4 * w.size
    U = torch.ones(n_qp * 2, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(X.size // 3 * 2, dtype=torch.float64, device="cuda")
    ibx.fe_assemble_rhs(3, torch.tensor(E, device="cuda"), torch.tensor(X, device="cuda"), pts, w, U, 2, rhs)
    torch.cuda.synchronize()
    r = rhs.cpu().numpy().reshape(-1, 2)
    from oracle import ibx_oracle

    vol = float(np.sum(ibx_oracle._fe_abs_det(3, E, X))) / 6.0
    assert abs(r[:, 0].sum() - vol) <= 1e-12 * vol and abs(r[:, 1].sum() - vol) <= 1e-12 * vol


def q1_mesh(dim, m, rng, lo=0.3, hi=0.7):
    """Perturbed structured QUAD4 (2D) / HEX8 (3D) mesh of [lo, hi]^dim in
    libMesh's node order (counter-clockwise per z layer, z = lo first)."""
    g = np.linspace(lo, hi, m + 1)
    idx = np.stack(np.meshgrid(*([np.arange(m + 1)] * dim), indexing="ij"), axis=-1).reshape(-1, dim)
    X = g[idx] + rng.uniform(-0.25, 0.25, size=idx.shape) * ((hi - lo) / m)
    stride = [(m + 1) ** (dim - 1 - d) for d in range(dim)]
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)][: 2 ** dim]
    E = []
    for cell in np.ndindex(*([m] * dim)):
        E += [sum((cell[d] + c[d]) * stride[d] for d in range(dim)) for c in corners]
    return np.array(E, dtype=np.int32), X.reshape(-1)


def gauss_rule(dim, n):
    """Tensor-product Gauss rule with n points per axis on [-1, 1]^dim."""
    x, w = np.polynomial.legendre.leggauss(n)
    P = np.stack(np.meshgrid(*([x] * dim), indexing="ij"), -1).reshape(-1, dim)
    W = np.prod(np.stack(np.meshgrid(*([w] * dim), indexing="ij"), -1).reshape(-1, dim), axis=1)
    return P, W


@pytest.mark.parametrize("n_gauss", [2, 3])
@pytest.mark.parametrize("dim,m", [(2, 20), (3, 6)])
def test_q1_quadrature_points_bit_identical(ibx, oracle, dim, m, n_gauss):
    """QUAD4 / HEX8 cells: positions, F * JxW and JxW (the Jacobian taken at
    every point) bit-identical to the oracle's restatement."""
    rng = np.random.default_rng(60 + dim + n_gauss)
    E, X = q1_mesh(dim, m, rng)
    pts, w = gauss_rule(dim, n_gauss)
    F = rng.standard_normal(X.size)
    Xq_ref, Fq_ref, J_ref = oracle.fe_quadrature_points(dim, E, X, pts, w, F=F, n_vars=dim,
                                                        elem_type=oracle.FE_TENSOR_Q1)
    Xq, Fq, J = ibx.fe_quadrature_points(dim, torch.tensor(E, device="cuda"), torch.tensor(X, device="cuda"), pts,
                                         w, F=torch.tensor(F, device="cuda"), n_vars=dim,
                                         elem_type=ibx.FE_TENSOR_Q1)
    assert np.array_equal(Xq.cpu().numpy(), Xq_ref)
    assert np.array_equal(J.cpu().numpy(), J_ref)
    assert np.array_equal(Fq.cpu().numpy(), Fq_ref)


@pytest.mark.parametrize("dim,m,N", [(2, 20, 64), (3, 6, 32)])
def test_q1_spread_and_interp_against_oracle(ibx, oracle, dim, m, N):
    """A QUAD4 / HEX8 structure through FEDataManager's path: spread of
    F * JxW from the quadrature points, interpolation there and the
    projection's right-hand side, against the oracle (FP64 within 1e-12)."""
    rng = np.random.default_rng(70 + dim)
    E, X = q1_mesh(dim, m, rng)
    pts, w = gauss_rule(dim, 2)
    F = rng.standard_normal(X.size)
    Q1 = oracle.FE_TENSOR_Q1
    Xq_ref, Fq_ref, _ = oracle.fe_quadrature_points(dim, E, X, pts, w, F=F, n_vars=dim, elem_type=Q1)
    u = rng.standard_normal([dim] + [N] * dim)
    f_ref, U_ref = oracle.periodic_problem(dim, [N] * dim, "IB_4", Xq_ref, F=Fq_ref, u=u, centering=1)
    rhs_ref = oracle.fe_assemble_rhs(dim, E, X, pts, w, U_ref, dim, elem_type=Q1)
    E_t, X_t = torch.tensor(E, device="cuda"), torch.tensor(X, device="cuda")
    Xq, Fq, _ = ibx.fe_quadrature_points(dim, E_t, X_t, pts, w, F=torch.tensor(F, device="cuda"), n_vars=dim,
                                         elem_type=ibx.FE_TENSOR_Q1)
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [N - 1] * dim,
                                       [1.0 / N] * dim, [0.0] * dim, [1.0] * dim, q, Xq, Q)
    f = [torch.zeros([N] * dim, dtype=torch.float64, device="cuda") for _ in range(dim)]
    ibx.spread(mk(f, Fq), "IB_4", ibx.FP64)
    u_t = [torch.tensor(u[a], device="cuda") for a in range(dim)]
    Uq = torch.zeros(Xq.numel(), dtype=torch.float64, device="cuda")
    ibx.interpolate(mk(u_t, Uq), "IB_4", ibx.FP64)
    rhs = torch.zeros(X.size, dtype=torch.float64, device="cuda")
    ibx.fe_assemble_rhs(dim, E_t, X_t, pts, w, Uq, dim, rhs, elem_type=ibx.FE_TENSOR_Q1)
    torch.cuda.synchronize()
    fs = np.stack([t.cpu().numpy() for t in f])
    assert np.max(np.abs(fs - f_ref)) <= 1e-12 * np.max(np.abs(f_ref))
    assert np.max(np.abs(Uq.cpu().numpy() - U_ref)) <= 1e-12 * np.max(np.abs(U_ref))
    assert np.max(np.abs(rhs.cpu().numpy() - rhs_ref)) <= 1e-12 * np.max(np.abs(rhs_ref))
