"""Device spring forces (ibx_spring_forces) against a sequential restatement
of the reference loop (IBStandardForceGen::computeLagrangianSpringForce with
the default linear spring), and the 2D ellipse workload's closed-loop
springs feeding the spread in one stream."""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def reference_springs(X, dim, mastr, slave, K, R0, F):
    """src/IB/IBStandardForceGen.cpp:825-900, sequentially."""
    Xv = X.reshape(-1, dim)
    Fv = F.reshape(-1, dim)
    for k in range(mastr.size):
        D = Xv[slave[k]] - Xv[mastr[k]]
        R = np.sqrt(np.sum(D * D))
        if R < np.finfo(np.float64).eps:
            continue
        T_over_R = K[k] * (R - R0[k]) / R
        Fv[mastr[k]] += T_over_R * D
        Fv[slave[k]] -= T_over_R * D
    return F


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("dim", [2, 3])
def test_spring_forces_match_reference_loop(ibx, dim, dtype):
    rng = np.random.default_rng(3 + dim)
    n, ns = 500, 1500
    X = rng.uniform(0, 1, size=n * dim)
    mastr = rng.integers(0, n, size=ns).astype(np.int32)
    slave = ((mastr + rng.integers(1, n, size=ns)) % n).astype(np.int32)
    slave[:5] = mastr[:5]  # zero-length springs are skipped
    K = rng.uniform(0.5, 2.0, size=ns)
    R0 = rng.uniform(0.0, 0.1, size=ns)
    F0 = rng.standard_normal(n * dim)
    F_ref = reference_springs(X, dim, mastr, slave, K, R0, F0.copy())
    tdt = torch.float64 if dtype == "float64" else torch.float32
    F_t = torch.tensor(F0, dtype=tdt, device="cuda")
    dev = lambda a: torch.tensor(a, device="cuda")
    st = ibx.spring_forces(dim, dev(X), dev(mastr), dev(slave), dev(K), dev(R0), F_t, accumulate=True)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    tol = 1e-12 if dtype == "float64" else 1e-5
    assert cases.rel_err(F_t.double().cpu().numpy(), F_ref) <= tol
    # accumulate = False zeroes F first
    F_t.fill_(123.0)
    ibx.spring_forces(dim, dev(X), dev(mastr), dev(slave), dev(K), dev(R0), F_t)
    F_ref2 = reference_springs(X, dim, mastr, slave, K, R0, np.zeros(n * dim))
    torch.cuda.synchronize()
    assert cases.rel_err(F_t.double().cpu().numpy(), F_ref2) <= tol


def test_bad_node_index_is_reported(ibx):
    dev = lambda a: torch.tensor(a, device="cuda")
    X = dev(np.zeros(6))
    F = torch.zeros(6, dtype=torch.float64, device="cuda")
    st = ibx.spring_forces(2, X, dev(np.array([0, 5], np.int32)), dev(np.array([1, 2], np.int32)),
                           dev(np.ones(2)), dev(np.zeros(2)), F)
    torch.cuda.synchronize()
    assert int(st.item()) & 1


def test_ellipse_springs_then_spread(ibx, oracle):
    """The 2D ellipse workload (256 markers, closed loop, K = 1, rest 0):
    forces on the device, spread on the same stream, against the oracle
    spreading the workload's host-computed forces."""
    from ibamr_gb300 import workloads

    X, F_host = workloads.ellipse_springs(256)
    n = X.size // 2
    mastr = np.arange(n, dtype=np.int32)
    slave = ((mastr + 1) % n).astype(np.int32)
    dev = lambda a: torch.tensor(a, device="cuda")
    X_t = dev(X)
    F_t = torch.zeros(n * 2, dtype=torch.float64, device="cuda")
    ibx.spring_forces(2, X_t, dev(mastr), dev(slave), dev(np.ones(n)), dev(np.zeros(n)), F_t)
    f_t = [torch.zeros(64, 64, dtype=torch.float64, device="cuda") for _ in range(2)]
    prob = ibx.make_problem(2, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [63, 63], [1 / 64] * 2, [0, 0], [1, 1], f_t,
                            X_t, F_t)
    ibx.spread(prob, "IB_4")
    torch.cuda.synchronize()
    assert cases.rel_err(F_t.cpu().numpy(), F_host) <= 1e-12
    f_ref, _ = oracle.periodic_side_problem(2, [64, 64], "IB_4", X, F=F_host)
    f = np.stack([t.cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= 1e-12


def reference_beams(X, dim, mastr, nxt, prv, K, D2X0, F):
    """src/IB/IBStandardForceGen.cpp:1037-1147, sequentially."""
    Xv = X.reshape(-1, dim)
    Fv = F.reshape(-1, dim)
    C = D2X0.reshape(-1, dim)
    for k in range(mastr.size):
        f = K[k] * (((Xv[nxt[k]] + Xv[prv[k]]) - 2.0 * Xv[mastr[k]]) - C[k])
        Fv[mastr[k]] += 2.0 * f
        Fv[nxt[k]] -= f
        Fv[prv[k]] -= f
    return F


def reference_targets(X, U, dim, node, kappa, eta, X0, F):
    """src/IB/IBStandardForceGen.cpp:1201-1299, sequentially; returns the
    largest displacement too."""
    Xv, Uv, Fv, T = X.reshape(-1, dim), U.reshape(-1, dim), F.reshape(-1, dim), X0.reshape(-1, dim)
    md = 0.0
    for k in range(node.size):
        i = node[k]
        Fv[i] += kappa[k] * (T[k] - Xv[i]) - eta[k] * Uv[i]
        md = max(md, float(np.sqrt(np.sum((T[k] - Xv[i]) * (T[k] - Xv[i])))))
    return F, md


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("dim", [2, 3])
def test_beam_forces_match_reference_loop(ibx, dim, dtype):
    """Beams along closed fibres (every node a master once and a neighbour
    twice, so contributions meet at the nodes) against the sequential loop;
    a fibre whose nodes each appear in one beam only is bit-exact."""
    rng = np.random.default_rng(13 + dim)
    n_fib, per = 20, 50
    n = n_fib * per
    X = rng.uniform(0, 1, size=n * dim)
    base = np.repeat(np.arange(n_fib) * per, per)
    j = np.tile(np.arange(per), n_fib)
    mastr = (base + j).astype(np.int32)
    nxt = (base + (j + 1) % per).astype(np.int32)
    prv = (base + (j - 1) % per).astype(np.int32)
    K = rng.uniform(0.5, 2.0, size=n)
    D2X0 = rng.standard_normal(n * dim) * 1e-3
    F0 = rng.standard_normal(n * dim)
    F_ref = reference_beams(X, dim, mastr, nxt, prv, K, D2X0, F0.copy())
    tdt = torch.float64 if dtype == "float64" else torch.float32
    F_t = torch.tensor(F0, dtype=tdt, device="cuda")
    dev = lambda a: torch.tensor(a, device="cuda")
    st = ibx.beam_forces(dim, dev(X), dev(mastr), dev(nxt), dev(prv), dev(K), dev(D2X0), F_t, accumulate=True)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    tol = 1e-12 if dtype == "float64" else 1e-5
    assert cases.rel_err(F_t.double().cpu().numpy(), F_ref) <= tol
    # disjoint beams (nodes 3k, 3k+1, 3k+2): one addition per node, bit-exact in FP64
    nb = n // 3
    m2 = (3 * np.arange(nb)).astype(np.int32)
    a2, b2 = m2 + 1, m2 + 2
    F_ref2 = reference_beams(X, dim, m2, a2, b2, K[:nb], D2X0[:nb * dim], np.zeros(n * dim))
    F2 = torch.full((n * dim,), 7.0, dtype=torch.float64, device="cuda")
    st = ibx.beam_forces(dim, dev(X), dev(m2), dev(a2), dev(b2), dev(K[:nb]), dev(D2X0[:nb * dim]), F2)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert np.array_equal(F2.cpu().numpy(), F_ref2)
    # out-of-range node: skipped and reported
    bad = mastr.copy()
    bad[3] = n + 5
    st = ibx.beam_forces(dim, dev(X), dev(bad), dev(nxt), dev(prv), dev(K), dev(D2X0), F_t, accumulate=True)
    torch.cuda.synchronize()
    assert int(st.item()) == 1


@pytest.mark.parametrize("dim", [2, 3])
def test_target_point_forces_match_reference_loop(ibx, dim):
    """Target points at distinct nodes (bit-exact) and the logged largest
    displacement; with zero velocities (U = NULL) the damping term vanishes."""
    rng = np.random.default_rng(17 + dim)
    n, npt = 800, 300
    X = rng.uniform(0, 1, size=n * dim)
    U = rng.standard_normal(n * dim)
    node = rng.choice(n, size=npt, replace=False).astype(np.int32)
    kappa = rng.uniform(1.0, 1e3, size=npt)
    eta = rng.uniform(0.0, 5.0, size=npt)
    X0 = X.reshape(-1, dim)[node].reshape(-1) + rng.standard_normal(npt * dim) * 1e-2
    F0 = rng.standard_normal(n * dim)
    F_ref, md_ref = reference_targets(X, U, dim, node, kappa, eta, X0, F0.copy())
    dev = lambda a: torch.tensor(a, device="cuda")
    F_t = dev(F0)
    md = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = ibx.target_point_forces(dim, dev(X), dev(U), dev(node), dev(kappa), dev(eta), dev(X0), F_t,
                                 accumulate=True, max_displacement=md)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    assert np.array_equal(F_t.cpu().numpy(), F_ref)
    assert float(md.item()) == md_ref
    F_ref0, _ = reference_targets(X, np.zeros_like(U), dim, node, kappa, eta, X0, np.zeros(n * dim))
    F_t = torch.full((n * dim,), 3.0, dtype=torch.float64, device="cuda")
    ibx.target_point_forces(dim, dev(X), None, dev(node), dev(kappa), dev(eta), dev(X0), F_t)
    torch.cuda.synchronize()
    assert np.array_equal(F_t.cpu().numpy(), F_ref0)


@pytest.mark.parametrize("dim", [2, 3])
def test_body_forces_by_structure(ibx, dim):
    """Uniform body forces: every node of a structure with a force gets it,
    nodes of other structures and out-of-range ids nothing."""
    rng = np.random.default_rng(19 + dim)
    n, ns = 1000, 6
    sid = rng.integers(-1, ns + 1, size=n).astype(np.int32)
    force = rng.standard_normal(ns * dim)
    has = np.array([1, 0, 1, 1, 0, 1], dtype=np.int32)
    F0 = rng.standard_normal(n * dim)
    F_ref = F0.reshape(-1, dim).copy()
    for i in range(n):
        if 0 <= sid[i] < ns and has[sid[i]]:
            F_ref[i] += force.reshape(-1, dim)[sid[i]]
    dev = lambda a: torch.tensor(a, device="cuda")
    F_t = dev(F0)
    ibx.body_forces(dim, dev(sid), dev(force), F_t, has_force=dev(has))
    torch.cuda.synchronize()
    assert np.array_equal(F_t.cpu().numpy(), F_ref.reshape(-1))
