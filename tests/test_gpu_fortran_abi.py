"""The Fortran-ABI entry points (include/ibx_fortran.h) against the oracle's
restatement of the same Fortran routines, called with the same arguments in
the same order: host arrays (copied in and out by the library) and device
arrays (used in place).  Bar: 1e-12 relative, the plain-form tolerance."""

import ctypes

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KERNELS = {"PIECEWISE_LINEAR": "piecewise_linear", "PIECEWISE_CUBIC": "piecewise_cubic", "IB_3": "ib_3",
           "IB_4": "ib_4", "IB_6": "ib_6", "BSPLINE_4": "bspline_4"}
TOL = 1e-12


@pytest.fixture(scope="module")
def libibx():
    from ibamr_gb300 import ibx

    assert torch.cuda.is_available()
    return ibx.lib()


def ptr(a):
    if isinstance(a, torch.Tensor):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_int(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def call(libibx, name, op, dim, case, depth, u, idx, sh, X, V):
    f = getattr(libibx, "lagrangian_%s_%s%dd_" % (name, op, dim))
    dx = np.asarray(case["dx"], np.float64)
    xl = np.asarray(case["x_lower"], np.float64)
    xu = np.asarray(case["x_upper"], np.float64)
    box = []
    for d in range(dim):
        box += [ref_int(case["ilower"][d]), ref_int(case["iupper"][d])]
    gw = [ref_int(case["gcw"][d]) for d in range(dim)]
    n = len(idx)
    if op == "interp":
        f(ptr(dx), ptr(xl), ptr(xu), ref_int(depth), *box, *gw, ptr(u), ptr(idx), ptr(sh), ref_int(n), ptr(X),
          ptr(V))
    else:
        f(ptr(dx), ptr(xl), ptr(xu), ref_int(depth), ptr(idx), ptr(sh), ref_int(n), ptr(X), ptr(V), *box, *gw,
          ptr(u))


@pytest.mark.parametrize("device_arrays", [False, True])
@pytest.mark.parametrize("depth", [1, 2])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", list(KERNELS))
def test_fortran_abi_matches_oracle(libibx, oracle, kernel, dim, depth, device_arrays):
    rng = np.random.default_rng(31 * dim + 7 * depth + list(KERNELS).index(kernel) + 500 * device_arrays)
    case = cases.random_patch_case(rng, dim, kernel, 0, q_depth=depth, n_markers=80)
    shape = [depth] + [case["iupper"][d] - case["ilower"][d] + 1 + 2 * case["gcw"][d] for d in range(dim)][::-1]
    u = rng.standard_normal(shape)
    X, idx, sh = case["X"], case["indices"], case["shifts"]
    V = rng.standard_normal(case["n_markers"] * depth)
    name = KERNELS[kernel]

    def args(a):
        return torch.tensor(a, device="cuda") if device_arrays else np.ascontiguousarray(a).copy()

    def back(a):
        return a.cpu().numpy() if isinstance(a, torch.Tensor) else a

    # interpolation overwrites V at the listed markers only
    V_ref = V.copy()
    oracle.fortran_interp(kernel, dim, case["dx"], case["x_lower"], case["x_upper"], depth, case["ilower"],
                          case["iupper"], case["gcw"], u, idx, sh, X, V_ref)
    V_gpu = args(V)
    call(libibx, name, "interp", dim, case, depth, args(u), args(idx), args(sh), args(X), V_gpu)
    assert cases.rel_err(back(V_gpu), V_ref) <= TOL
    # spreading adds into u
    u_ref = u.copy()
    oracle.fortran_spread(kernel, dim, case["dx"], case["x_lower"], case["x_upper"], depth, idx, sh, X, V,
                          case["ilower"], case["iupper"], case["gcw"], u_ref)
    u_gpu = args(u)
    call(libibx, name, "spread", dim, case, depth, u_gpu, args(idx), args(sh), args(X), args(V))
    assert cases.rel_err(back(u_gpu), u_ref) <= TOL
