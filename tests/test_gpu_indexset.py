"""LIndexSetData::cacheLocalIndices on the device (ibx_cache_local_indices,
ibtk/src/lagrangian/LIndexSetData.cpp:50-140) against the oracle's
restatement (ibxo_cache_local_indices): the same local marker indices, the
same periodic shifts (+-N dx on periodic sides only), the same order, bit for
bit -- for the ghost-box lists and the interior lists, patches that touch
periodic boundaries on some sides or none, and positions on and one ulp
around every cell face of the patch and its ghost box."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def case(rng, dim, n):
    """A patch of a periodic level [0, L) with N cells per dimension, the
    patch touching the lower / upper boundary on random sides; markers over
    the whole domain, half of them on or one ulp around cell faces."""
    N = rng.integers(12, 40, size=dim)
    dx = rng.uniform(0.01, 0.1, size=dim)
    lo = np.array([int(rng.integers(0, N[d] - 4)) if rng.uniform() < 0.6 else 0 for d in range(dim)])
    hi = np.array([min(N[d] - 1, lo[d] + int(rng.integers(3, 12))) if rng.uniform() < 0.6 else N[d] - 1
                   for d in range(dim)])
    periodic = rng.integers(0, 2, size=dim)
    X = rng.uniform(0.0, 1.0, size=(n, dim)) * (N * dx)[None, :]
    faces = rng.integers(0, N + 1, size=(n // 2, dim)) * dx[None, :]
    ulp = rng.integers(-1, 2, size=(n // 2, dim))
    X[: n // 2] = np.where(ulp < 0, np.nextafter(faces, -np.inf), np.where(ulp > 0, np.nextafter(faces, np.inf),
                                                                           faces))
    X = np.mod(X, (N * dx)[None, :])
    return N, dx, lo, hi, periodic, X.reshape(-1)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("seed", range(6))
def test_cache_local_indices_bit_exact(ibx, oracle, dim, seed):
    rng = np.random.default_rng(1000 + 10 * dim + seed)
    N, dx, lo, hi, periodic, X = case(rng, dim, 3000)
    ghost = [int(rng.integers(1, 5))] * dim
    x_lower = lo * dx
    x_upper = (hi + 1) * dx
    # SAMRAI: a patch touches a periodic boundary where it meets the domain
    # boundary along a periodic dimension; the shift is the domain's cells
    tl = [int(periodic[d] and lo[d] == 0) for d in range(dim)]
    tu = [int(periodic[d] and hi[d] == N[d] - 1) for d in range(dim)]
    shift = [int(N[d]) if periodic[d] else 0 for d in range(dim)]
    P = oracle.make_patch(dim, lo, hi, x_lower, x_upper, dx=dx, periodic=periodic, domain_lo=[0] * dim,
                          domain_hi=list(N - 1))
    X_t = torch.tensor(X, device="cuda")
    for want_ghost in (1, 0):
        idx_ref, sh_ref = oracle.cache_local_indices(P, shift, ghost, want_ghost, X)
        idx, sh, cells = ibx.cache_local_indices(dim, lo, hi, x_lower, x_upper, dx, tl, tu, shift, ghost,
                                                 want_ghost, X_t)
        idx = idx.cpu().numpy()
        sh = sh.cpu().numpy()
        assert idx_ref.size > 0
        assert np.array_equal(idx, idx_ref), (want_ghost, idx.size, idx_ref.size)
        assert np.array_equal(sh, sh_ref)
        # the image cells lie in the selected box, interior ones in the patch box
        c = cells.cpu().numpy().reshape(-1, dim)
        g = np.array(ghost) if want_ghost else 0
        assert np.all(c >= lo - g) and np.all(c <= hi + g)
        # shifts are +-N dx on periodic sides only
        s = sh.reshape(-1, dim)
        for d in range(dim):
            allowed = {0.0, N[d] * dx[d], -N[d] * dx[d]} if periodic[d] else {0.0}
            assert set(np.unique(s[:, d]).tolist()) <= allowed


def test_cache_local_indices_capacity(ibx):
    X = torch.tensor(np.full(3 * 10, 0.5), device="cuda")
    with pytest.raises(ibx.IbxError) as e:
        ibx.cache_local_indices(3, [0] * 3, [9] * 3, [0.0] * 3, [1.0] * 3, [0.1] * 3, [1] * 3, [1] * 3, [10] * 3,
                                [2] * 3, 1, X, capacity=5)
    assert e.value.status == ibx.E_TOO_LARGE
