"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle (``ibx_oracle.cpp``) restates IBAMR's Fortran interaction routines
and the LEInteractor wrapper layer on the CPU.  Only the test-suite, the smoke
check and the CPU-baseline leg of the benchmark import this module; the
product path (``ibamr_gb300``) never does.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libibx_oracle.so")

KERNELS = {"PIECEWISE_LINEAR": 0, "PIECEWISE_CUBIC": 1, "IB_3": 2, "IB_4": 3, "IB_6": 4, "BSPLINE_4": 5}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Patch(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("ilower", ctypes.c_int * 3), ("iupper", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3), ("x_lower", ctypes.c_double * 3), ("x_upper", ctypes.c_double * 3),
        ("touches_regular_lower", ctypes.c_int * 3), ("touches_regular_upper", ctypes.c_int * 3),
        ("touches_periodic_lower", ctypes.c_int * 3), ("touches_periodic_upper", ctypes.c_int * 3),
    ]


class PatchData(ctypes.Structure):
    _fields_ = [("ptr", _dp * 3), ("gcw", ctypes.c_int * 3), ("depth", ctypes.c_int), ("centering", ctypes.c_int)]


def build(force=False):
    """Compile the oracle with the flags its header asks for."""
    src = os.path.join(HERE, "ibx_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ibx_oracle.h"))):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-o", tmp, src,
                               "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.ibxo_stencil_size.argtypes = [ctypes.c_int]
        L.ibxo_min_ghost_width.argtypes = [ctypes.c_int]
        L.ibxo_kernel_from_name.argtypes = [ctypes.c_char_p]
        L.ibxo_nint.argtypes = [ctypes.c_double]
        L.ibxo_stencil_1d.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _ip, _ip, _dp]
        L.ibxo_fortran_interp.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, _ip, _ip, _dp,
                                          _ip, _dp, ctypes.c_int, _dp, _dp]
        L.ibxo_fortran_spread.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, _dp,
                                          ctypes.c_int, _dp, _dp, _ip, _ip, _ip, _dp]
        L.ibxo_get_cell_index.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _ip, _ip, _ip]
        L.ibxo_build_local_indices.argtypes = [ctypes.POINTER(Patch), _ip, _ip, _dp, ctypes.c_int, _ip]
        L.ibxo_cache_local_indices.argtypes = [ctypes.POINTER(Patch), _ip, _ip, ctypes.c_int, _dp, ctypes.c_int,
                                               ctypes.c_int, _ip, _dp]
        L.ibxo_lei_interpolate_raw.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.POINTER(PatchData),
                                               ctypes.POINTER(Patch), _ip, _ip, ctypes.c_int]
        L.ibxo_lei_spread_raw.argtypes = [ctypes.POINTER(PatchData), _dp, ctypes.c_int, _dp, ctypes.c_int,
                                          ctypes.POINTER(Patch), _ip, _ip, ctypes.c_int]
        L.ibxo_lei_interpolate_idx.argtypes = [_dp, ctypes.c_int, _dp, _ip, _dp, ctypes.c_int,
                                               ctypes.POINTER(PatchData), ctypes.POINTER(Patch), ctypes.c_int]
        L.ibxo_lei_spread_idx.argtypes = [ctypes.POINTER(PatchData), _dp, ctypes.c_int, _dp, _ip, _dp, ctypes.c_int,
                                          ctypes.POINTER(Patch), ctypes.c_int]
        L.ibxo_accumulate_ghosts_single_patch.argtypes = [ctypes.POINTER(PatchData), ctypes.POINTER(Patch), _ip, _ip,
                                                          _ip]
        L.ibxo_fill_periodic_ghosts.argtypes = [ctypes.POINTER(PatchData), ctypes.POINTER(Patch)]
        L.ibxo_mt19937_uniform.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp]
        L.ibxo_cpu_plan_create.argtypes = [ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                           ctypes.c_int]
        L.ibxo_cpu_plan_create.restype = ctypes.c_void_p
        L.ibxo_cpu_plan_patches.argtypes = [ctypes.c_void_p]
        L.ibxo_cpu_plan_step.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp]
        L.ibxo_cpu_plan_destroy.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def dptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def iptr(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


def ivec(v):
    return (ctypes.c_int * 3)(*(list(v) + [0] * (3 - len(v))))


def kernel_id(name):
    return KERNELS[name] if isinstance(name, str) else int(name)


def stencil_size(kernel):
    return lib().ibxo_stencil_size(kernel_id(kernel))


def min_ghost_width(kernel):
    return lib().ibxo_min_ghost_width(kernel_id(kernel))


def nint(a):
    return lib().ibxo_nint(float(a))


def stencil_1d(kernel, X, Xshift, x_lower, dx, ilower, iupper, ghost):
    """(base, start, stop, weights[6]) of one dimension (Fortran rules)."""
    b, st, sp = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    w = np.zeros(6)
    rc = lib().ibxo_stencil_1d(kernel_id(kernel), float(X), float(Xshift), float(x_lower), float(dx), int(ilower),
                               int(iupper), int(ghost), ctypes.byref(b), ctypes.byref(st), ctypes.byref(sp), dptr(w))
    assert rc == 0
    return b.value, st.value, sp.value, w


def mt19937_uniform(seed, n, a=0.0, b=1.0):
    out = np.empty(n, dtype=np.float64)
    lib().ibxo_mt19937_uniform(seed, n, a, b, dptr(out))
    return out


def make_patch(dim, ilower, iupper, x_lower, x_upper, dx=None, periodic=(0, 0, 0), domain_lo=None, domain_hi=None):
    """Patch geometry; boundary flags follow from the domain box (default: the patch)."""
    P = Patch()
    P.dim = dim
    domain_lo = list(domain_lo if domain_lo is not None else ilower)
    domain_hi = list(domain_hi if domain_hi is not None else iupper)
    for d in range(dim):
        P.ilower[d] = int(ilower[d])
        P.iupper[d] = int(iupper[d])
        P.x_lower[d] = float(x_lower[d])
        P.x_upper[d] = float(x_upper[d])
        P.dx[d] = float(dx[d]) if dx is not None else (P.x_upper[d] - P.x_lower[d]) / (P.iupper[d] - P.ilower[d] + 1)
        at_lo = int(ilower[d]) == int(domain_lo[d])
        at_hi = int(iupper[d]) == int(domain_hi[d])
        per = bool(periodic[d]) if d < len(periodic) else False
        P.touches_regular_lower[d] = int(at_lo and not per)
        P.touches_regular_upper[d] = int(at_hi and not per)
        P.touches_periodic_lower[d] = int(at_lo and per)
        P.touches_periodic_upper[d] = int(at_hi and per)
    return P


def data_shape(P, centering, gcw, axis=0):
    """Shape (Fortran order, x fastest => numpy reversed) of one ghosted array."""
    n = []
    for d in range(P.dim):
        extra = 1 if (centering == 1 and d == axis) else 0
        n.append(P.iupper[d] - P.ilower[d] + 1 + extra + 2 * gcw[d])
    return n


class GhostedData:
    """SAMRAI CellData/SideData stand-in: numpy arrays with ghosts, depth slowest."""

    def __init__(self, P, centering, gcw, depth=1):
        self.P = P
        self.centering = centering
        self.gcw = list(gcw) + [0] * (3 - len(gcw))
        self.depth = depth
        ncomp = 1 if centering == 0 else P.dim
        self.arrays = []
        for a in range(ncomp):
            n = data_shape(P, centering, self.gcw, a)
            self.arrays.append(np.zeros([depth] + n[::-1], dtype=np.float64))
        self.struct = PatchData()
        for a in range(ncomp):
            self.struct.ptr[a] = dptr(self.arrays[a])
        for d in range(3):
            self.struct.gcw[d] = self.gcw[d]
        self.struct.depth = depth
        self.struct.centering = centering

    def lower(self, axis=0):
        """Index of element [0,...,0] of array `axis` (per dim, x first)."""
        return [self.P.ilower[d] - self.gcw[d] for d in range(self.P.dim)]

    def value(self, axis, idx, depth=0):
        lo = self.lower(axis)
        k = tuple(idx[d] - lo[d] for d in range(self.P.dim))[::-1]
        return self.arrays[axis][(depth,) + k]


def spread_raw(q, Q, Q_depth, X, box_lo, box_hi, kernel):
    n = X.size // q.P.dim
    return lib().ibxo_lei_spread_raw(ctypes.byref(q.struct), dptr(Q), Q_depth, dptr(X), n, ctypes.byref(q.P),
                                     ivec(box_lo), ivec(box_hi), kernel_id(kernel))


def interpolate_raw(Q, Q_depth, X, q, box_lo, box_hi, kernel):
    n = X.size // q.P.dim
    return lib().ibxo_lei_interpolate_raw(dptr(Q), Q_depth, dptr(X), n, ctypes.byref(q.struct), ctypes.byref(q.P),
                                          ivec(box_lo), ivec(box_hi), kernel_id(kernel))


def spread_idx(q, Q, Q_depth, X, idx, shifts, kernel):
    return lib().ibxo_lei_spread_idx(ctypes.byref(q.struct), dptr(Q), Q_depth, dptr(X), iptr(idx), dptr(shifts),
                                     int(idx.size), ctypes.byref(q.P), kernel_id(kernel))


def interpolate_idx(Q, Q_depth, X, idx, shifts, q, kernel):
    return lib().ibxo_lei_interpolate_idx(dptr(Q), Q_depth, dptr(X), iptr(idx), dptr(shifts), int(idx.size),
                                          ctypes.byref(q.struct), ctypes.byref(q.P), kernel_id(kernel))


def cache_local_indices(P, periodic_shift, ghost_width, want_ghost_box, X):
    n = X.size // P.dim
    cap = 27 * max(n, 1)
    idx = np.empty(cap, dtype=np.int32)
    sh = np.empty(cap * P.dim, dtype=np.float64)
    cnt = lib().ibxo_cache_local_indices(ctypes.byref(P), ivec(periodic_shift), ivec(ghost_width),
                                         int(want_ghost_box), dptr(X), n, cap, iptr(idx), dptr(sh))
    return idx[:cnt].copy(), sh[: cnt * P.dim].copy()


def fortran_interp(kernel, dim, dx, x_lower, x_upper, depth, ilower, iupper, nugc, u, indices, Xshift, X, V):
    return lib().ibxo_fortran_interp(kernel_id(kernel), dim, dptr(np.asarray(dx, np.float64)),
                                     dptr(np.asarray(x_lower, np.float64)), dptr(np.asarray(x_upper, np.float64)),
                                     depth, ivec(ilower), ivec(iupper), ivec(nugc), dptr(u), iptr(indices),
                                     dptr(Xshift), int(indices.size), dptr(X), dptr(V))


def fortran_spread(kernel, dim, dx, x_lower, x_upper, depth, indices, Xshift, X, V, ilower, iupper, nugc, u):
    return lib().ibxo_fortran_spread(kernel_id(kernel), dim, dptr(np.asarray(dx, np.float64)),
                                     dptr(np.asarray(x_lower, np.float64)), dptr(np.asarray(x_upper, np.float64)),
                                     depth, iptr(indices), dptr(Xshift), int(indices.size), dptr(X), dptr(V),
                                     ivec(ilower), ivec(iupper), ivec(nugc), dptr(u))


def fill_periodic_ghosts(q):
    return lib().ibxo_fill_periodic_ghosts(ctypes.byref(q.struct), ctypes.byref(q.P))


def accumulate_ghosts_single_patch(q, domain_lo, domain_hi, periodic):
    return lib().ibxo_accumulate_ghosts_single_patch(ctypes.byref(q.struct), ctypes.byref(q.P), ivec(domain_lo),
                                                     ivec(domain_hi), ivec(periodic))


# ---------------------------------------------------------------------------
# Periodic single-patch problems in the compact layout the CUDA path uses.
# ---------------------------------------------------------------------------

def periodic_problem(dim, N, kernel, X, F=None, u=None, centering=1, depth=1):
    """Reference flow on one periodic patch covering [0,1)^dim (LDataManager):
    spread F of the ghost-box markers (with periodic shifts) into zeroed patch
    data and keep the interior; interpolate u (ghosts filled periodically) at
    the interior markers.  f/u are compact periodic arrays of shape
    (ncomp,) + N[::-1] where ncomp = dim for side data (face N == face 0) and
    depth for cell data.  Returns (f, U) (None for the parts not requested)."""
    Nl = list(N)
    P = make_patch(dim, [0] * dim, [n - 1 for n in Nl], [0.0] * dim, [1.0] * dim, dx=[1.0 / n for n in Nl],
                   periodic=[1] * dim)
    g = min_ghost_width(kernel)
    gw = [g] * dim
    Q_depth = dim if centering == 1 else depth
    q_depth = 1 if centering == 1 else depth
    ncomp = dim if centering == 1 else depth
    f_out = U_out = None

    def comp_view(q, c):
        # side: array c, depth 0; cell: array 0, depth c
        return q.arrays[c][0] if centering == 1 else q.arrays[0][c]

    if F is not None:
        idx, sh = cache_local_indices(P, Nl, gw, 1, X)
        q = GhostedData(P, centering, gw, depth=q_depth)
        rc = spread_idx(q, F, Q_depth, X, idx, sh, kernel)
        assert rc == 0, rc
        f_out = np.empty([ncomp] + Nl[::-1])
        sl = tuple(slice(g, g + n) for n in Nl[::-1])
        for c in range(ncomp):
            f_out[c] = comp_view(q, c)[sl]
    if u is not None:
        q = GhostedData(P, centering, gw, depth=q_depth)
        for c in range(ncomp):
            arr = comp_view(q, c)
            grids = np.meshgrid(*[np.arange(arr.shape[k]) for k in range(dim)], indexing="ij")
            src = []
            for k in range(dim):  # numpy axis k <-> dim (dim-1-k)
                src.append((grids[k] - g) % Nl[dim - 1 - k])
            arr[...] = u[c][tuple(src)]
        idx, sh = cache_local_indices(P, Nl, gw, 0, X)
        U_out = np.zeros((X.size // dim) * Q_depth)
        rc = interpolate_idx(U_out, Q_depth, X, idx, sh, q, kernel)
        assert rc == 0, rc
    return f_out, U_out


def periodic_side_problem(dim, N, kernel, X, F=None, u=None):
    return periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)


class CpuPlan:
    """Multi-threaded per-patch CPU baseline (see ibxo_cpu_plan_create):
    ``threads`` host threads working through ``boxes`` box patches (default:
    one patch for one thread, else four patches per thread)."""

    def __init__(self, dim, N, kernel, X, threads=1, boxes=None):
        self.X = np.ascontiguousarray(X, dtype=np.float64)
        self.dim = dim
        if boxes is None:
            boxes = 1 if threads == 1 else 4 * threads
        self.h = lib().ibxo_cpu_plan_create(dim, ivec(N), kernel_id(kernel), self.X.size // dim, dptr(self.X),
                                            int(threads), int(boxes))
        if not self.h:
            raise ValueError("bad CPU plan arguments")
        self.threads = int(threads)
        self.patches = lib().ibxo_cpu_plan_patches(self.h)

    def step(self, F, f, u, U):
        rc = lib().ibxo_cpu_plan_step(self.h, dptr(F), dptr(f), dptr(u), dptr(U))
        assert rc == 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().ibxo_cpu_plan_destroy(self.h)
            self.h = None


# ---------------------------------------------------------------------------
# Finite-element quadrature points (FEDataManager, first-order Lagrange
# simplices TRI3 / TET4 and tensor-product cells QUAD4 / HEX8).
# ---------------------------------------------------------------------------
FE_SIMPLEX_P1, FE_TENSOR_Q1 = 0, 1

# Reference-cell corner of each QUAD4 / HEX8 node in libMesh's order (0: -1,
# 1: +1 along each axis): counter-clockwise per z layer, z = -1 first.
_Q1_CORNER = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def _fe_npe(dim, elem_type):
    return (4 if dim == 2 else 8) if elem_type == FE_TENSOR_Q1 else dim + 1


def _fe_q1_basis(dim, points):
    """QUAD4 / HEX8 basis at the reference points: phi_k = prod_c L(xi_c)
    with L = (1 - xi) / 2 or (1 + xi) / 2 by the node's corner, the product in
    axis order; dphi_k / dxi_c the same product with the derivative +-1/2 on
    axis c.  Returns (phi [n_qp, npe], dphi [n_qp, npe, dim])."""
    P = np.asarray(points, dtype=np.float64).reshape(-1, dim)
    npe = 4 if dim == 2 else 8
    phi = np.zeros((P.shape[0], npe))
    dphi = np.zeros((P.shape[0], npe, dim))
    for k in range(npe):
        L = [np.where(_Q1_CORNER[k, c], 0.5 * (1.0 + P[:, c]), 0.5 * (1.0 - P[:, c])) for c in range(dim)]
        dL = [np.full(P.shape[0], 0.5 if _Q1_CORNER[k, c] else -0.5) for c in range(dim)]
        p = L[0]
        for c in range(1, dim):
            p = p * L[c]
        phi[:, k] = p
        for c in range(dim):
            g = dL[0] if c == 0 else L[0]
            for a in range(1, dim):
                g = g * (dL[a] if a == c else L[a])
            dphi[:, k, c] = g
    return phi, dphi


def _det(dim, J):
    """det of J[..., r, c], the products and differences in a fixed order."""
    if dim == 2:
        return J[..., 0, 0] * J[..., 1, 1] - J[..., 0, 1] * J[..., 1, 0]
    m0 = J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1]
    m1 = J[..., 1, 0] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 0]
    m2 = J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]
    return (J[..., 0, 0] * m0 - J[..., 0, 1] * m1) + J[..., 0, 2] * m2


def _fe_q1_jxw(dim, elem_nodes, X, points, weights):
    """JxW [n_elems, n_qp] of a QUAD4 / HEX8 mesh: |det J(q)| w(q) with
    J(q)_rc = sum_k X_k[r] dphi_k/dxi_c (q), summed from zero in node order."""
    npe = 4 if dim == 2 else 8
    E = np.asarray(elem_nodes).reshape(-1, npe)
    Xn = np.asarray(X, dtype=np.float64).reshape(-1, dim)
    _, dphi = _fe_q1_basis(dim, points)
    nq = dphi.shape[0]
    J = np.zeros((E.shape[0], nq, dim, dim))
    for r in range(dim):
        for c in range(dim):
            v = np.zeros((E.shape[0], nq))
            for k in range(npe):
                v = v + Xn[E[:, k], r][:, None] * dphi[None, :, k, c]
            J[:, :, r, c] = v
    w = np.asarray(weights, dtype=np.float64).reshape(-1)
    return np.abs(_det(dim, J)) * w[None, :]

def _fe_phi(dim, points):
    """Barycentric basis at the reference points: phi_0 = 1 - (xi_0 + ... ),
    phi_d = xi_d (first-order Lagrange TRI3 / TET4)."""
    P = np.asarray(points, dtype=np.float64).reshape(-1, dim)
    s = np.zeros(P.shape[0])
    for d in range(dim):
        s = s + P[:, d]
    return np.concatenate([(1.0 - s)[:, None], P], axis=1)  # [n_qp, dim + 1]


def _fe_abs_det(dim, elem_nodes, X):
    E = np.asarray(elem_nodes).reshape(-1, dim + 1)
    Xn = np.asarray(X, dtype=np.float64).reshape(-1, dim)
    J = np.stack([Xn[E[:, c + 1]] - Xn[E[:, 0]] for c in range(dim)], axis=2)  # J[e, r, c]
    if dim == 2:
        det = J[:, 0, 0] * J[:, 1, 1] - J[:, 0, 1] * J[:, 1, 0]
    else:
        m0 = J[:, 1, 1] * J[:, 2, 2] - J[:, 1, 2] * J[:, 2, 1]
        m1 = J[:, 1, 0] * J[:, 2, 2] - J[:, 1, 2] * J[:, 2, 0]
        m2 = J[:, 1, 0] * J[:, 2, 1] - J[:, 1, 1] * J[:, 2, 0]
        det = (J[:, 0, 0] * m0 - J[:, 0, 1] * m1) + J[:, 0, 2] * m2
    return np.abs(det)


def fe_quadrature_points(dim, elem_nodes, X, points, weights, F=None, n_vars=0, elem_type=FE_SIMPLEX_P1):
    """FEDataManager::spread's quadrature-point values
    (ibtk/src/lagrangian/FEDataManager.cpp:1088-1219 with
    sum_weighted_elem_solution :824-858): X_q = sum_k X_k phi_k(q) and
    F_q = (sum_k F_k phi_k(q)) * JxW(q), the sums from zero over the basis in
    order, JxW(q) = |det J(q)| * w(q).  Returns (X_qp, F_qp or None, JxW),
    entries e * n_qp + q."""
    npe = _fe_npe(dim, elem_type)
    E = np.asarray(elem_nodes).reshape(-1, npe)
    Xn = np.asarray(X, dtype=np.float64).reshape(-1, dim)
    w = np.asarray(weights, dtype=np.float64).reshape(-1)
    if elem_type == FE_TENSOR_Q1:
        phi, _ = _fe_q1_basis(dim, points)
        jxw = _fe_q1_jxw(dim, elem_nodes, X, points, weights)
    else:
        phi = _fe_phi(dim, points)
        jxw = _fe_abs_det(dim, elem_nodes, X)[:, None] * w[None, :]
    nq = w.size
    ne = E.shape[0]
    X_qp = np.zeros((ne, nq, dim))
    for k in range(npe):
        X_qp = X_qp + Xn[E[:, k]][:, None, :] * phi[None, :, k, None]
    F_qp = None
    if F is not None:
        Fn = np.asarray(F, dtype=np.float64).reshape(-1, n_vars)
        acc = np.zeros((ne, nq, n_vars))
        for k in range(npe):
            acc = acc + Fn[E[:, k]][:, None, :] * phi[None, :, k, None]
        F_qp = (acc * jxw[:, :, None]).reshape(-1)
    return X_qp.reshape(-1), F_qp, jxw.reshape(-1)


def fe_assemble_rhs(dim, elem_nodes, X, points, weights, U_qp, n_vars, elem_type=FE_SIMPLEX_P1):
    """FEDataManager::interp's right-hand side (FEDataManager.cpp:1873-2005,
    integrate_elem_rhs :1569-1604): rhs[node_k] += sum_q U_q * (phi_k(q) *
    JxW(q)) per element, the element sums in point order, the elements added
    in order.  Returns rhs [n_nodes * n_vars]."""
    npe = _fe_npe(dim, elem_type)
    E = np.asarray(elem_nodes).reshape(-1, npe)
    n_nodes = np.asarray(X).size // dim
    w = np.asarray(weights, dtype=np.float64).reshape(-1)
    nq = w.size
    if elem_type == FE_TENSOR_Q1:
        phi, _ = _fe_q1_basis(dim, points)
        jxw = _fe_q1_jxw(dim, elem_nodes, X, points, weights)
    else:
        phi = _fe_phi(dim, points)
        det = _fe_abs_det(dim, elem_nodes, X)
        jxw = np.stack([det * w[q] for q in range(nq)], axis=1)
    U = np.asarray(U_qp, dtype=np.float64).reshape(E.shape[0], nq, n_vars)
    rhs = np.zeros((n_nodes, n_vars))
    for k in range(npe):
        acc = np.zeros((E.shape[0], n_vars))
        for q in range(nq):
            p_jxw = phi[q, k] * jxw[:, q]
            acc = acc + U[:, q, :] * p_jxw[:, None]
        np.add.at(rhs, E[:, k], acc)
    return rhs.reshape(-1)
