"""Marker redistribution over the patches of a level (ibx_redistribute):
owners bit-identical to the reference's getCellIndex rule (the oracle's
restatement) evaluated with each patch's geometry, markers grouped by owner
by the counting sort, unowned markers last."""

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


def level_boxes(dim, N, splits):
    """A level over [0, 1]^dim with N cells per dim, cut into splits[d] patches
    per dim; each patch's x_lower / x_upper computed from its own box."""
    dx = [1.0 / n for n in N]
    cuts = [np.linspace(0, N[d], splits[d] + 1).astype(int) for d in range(dim)]
    boxes = []
    for idx in np.ndindex(*splits):
        ilo = [int(cuts[d][idx[d]]) for d in range(dim)]
        ihi = [int(cuts[d][idx[d] + 1]) - 1 for d in range(dim)]
        xl = [ilo[d] * dx[d] for d in range(dim)]
        xu = [(ihi[d] + 1) * dx[d] for d in range(dim)]
        boxes.append((ilo, ihi, xl, xu, dx))
    return boxes


def oracle_owner(oracle, dim, boxes, X):
    n = X.size // dim
    own = np.full(n, -1, dtype=np.int64)
    idx = (oracle.ctypes.c_int * 3)()
    for s in range(n):
        for p, (ilo, ihi, xl, xu, dx) in enumerate(boxes):
            oracle.lib().ibxo_get_cell_index(dim, oracle.dptr(np.ascontiguousarray(X[dim * s: dim * s + dim])),
                                             oracle.dptr(np.asarray(xl, np.float64)),
                                             oracle.dptr(np.asarray(xu, np.float64)),
                                             oracle.dptr(np.asarray(dx, np.float64)), oracle.ivec(ilo),
                                             oracle.ivec(ihi), idx)
            if all(ilo[d] <= idx[d] <= ihi[d] for d in range(dim)):
                own[s] = p
                break
    return own


@pytest.mark.parametrize("dim,N,splits", [(2, [32, 24], [3, 2]), (3, [16, 12, 10], [2, 3, 2])])
def test_redistribute_matches_get_cell_index(ibx, oracle, dim, N, splits):
    rng = np.random.default_rng(9 + dim)
    boxes = level_boxes(dim, N, splits)
    n = 1500
    X = rng.uniform(-0.05, 1.05, size=(n, dim))
    # positions on patch faces and one ulp either side of them
    for k in range(0, 300, 3):
        d = k % dim
        b = boxes[k % len(boxes)]
        x = b[2][d] if k % 2 else b[3][d]
        X[k, d], X[k + 1, d], X[k + 2, d] = x, np.nextafter(x, -1.0), np.nextafter(x, 2.0)
    X = X.reshape(-1)
    own_ref = oracle_owner(oracle, dim, boxes, X)
    owner, order, offs = ibx.redistribute(dim, boxes, torch.tensor(X, device="cuda"))
    torch.cuda.synchronize()
    owner, order, offs = owner.cpu().numpy(), order.cpu().numpy(), offs.cpu().numpy()
    assert np.array_equal(owner, own_ref)
    assert np.array_equal(np.sort(order), np.arange(n))
    counts = np.bincount(np.where(owner < 0, len(boxes), owner), minlength=len(boxes) + 1)
    assert offs[0] == 0 and np.array_equal(np.diff(offs), counts) and offs[-1] == n
    for p in range(len(boxes) + 1):
        seg = order[offs[p]:offs[p + 1]]
        assert np.all(np.where(owner[seg] < 0, len(boxes), owner[seg]) == p)
