"""Python binding of libibx (include/ibx.h) over ctypes.

This is host plumbing for tests, benchmarks and Python users: device memory
comes from torch tensors, calls go straight to the C ABI.  There is no CPU
fallback: importing works without a GPU, but every compute call needs the
CUDA library and a device, and raises otherwise.
"""

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("IBX_LIB_PATH") or os.path.join(PKG, "lib", "libibx.so")

PIECEWISE_LINEAR, PIECEWISE_CUBIC, IB_3, IB_4, IB_6, BSPLINE_4 = range(6)
KERNELS = {"PIECEWISE_LINEAR": 0, "PIECEWISE_CUBIC": 1, "IB_3": 2, "IB_4": 3, "IB_6": 4, "BSPLINE_4": 5}
FP64, MIXED = 0, 1
CELL, SIDE = 0, 1
MODE_PATCH, MODE_PERIODIC = 0, 1

OK = 0
E_BAD_KERNEL, E_GHOST_WIDTH, E_DEPTH, E_ARG, E_CUDA, E_OOM, E_TIMEOUT, E_NONFINITE, E_TOO_LARGE = range(1, 10)


class IbxError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__("%s: %s (status %d)" % (where or "libibx", status_string(status), status))


class Problem(ctypes.Structure):
    """ibx_problem (include/ibx.h)."""

    _fields_ = [
        ("dim", ctypes.c_int), ("centering", ctypes.c_int), ("mode", ctypes.c_int),
        ("ilower", ctypes.c_int * 3), ("iupper", ctypes.c_int * 3), ("gcw", ctypes.c_int * 3),
        ("dx", ctypes.c_double * 3), ("x_lower", ctypes.c_double * 3), ("x_upper", ctypes.c_double * 3),
        ("touches_physical_lower", ctypes.c_int * 3), ("touches_physical_upper", ctypes.c_int * 3),
        ("q_depth", ctypes.c_int), ("q", ctypes.c_void_p * 3),
        ("X", ctypes.c_void_p), ("Q", ctypes.c_void_p), ("Q_depth", ctypes.c_int),
        ("n_markers", ctypes.c_int), ("indices", ctypes.c_void_p), ("n_indices", ctypes.c_int),
        ("Xshift", ctypes.c_void_p),
    ]


_lib = None


def lib():
    """The loaded libibx.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libibx.so is missing (%s): build it with python -m ibamr_gb300.build" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(Problem)
        L.ibx_get_stencil_size.argtypes = [ctypes.c_int]
        L.ibx_get_minimum_ghost_width.argtypes = [ctypes.c_int]
        L.ibx_kernel_from_name.argtypes = [ctypes.c_char_p]
        L.ibx_status_string.argtypes = [ctypes.c_int]
        L.ibx_status_string.restype = ctypes.c_char_p
        L.ibx_kernel_launches.restype = ctypes.c_longlong
        L.ibx_spring_forces.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.ibx_beam_forces.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + \
            [ctypes.c_void_p] * 6 + [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.ibx_target_point_forces.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int] + [ctypes.c_void_p] * 5 + \
            [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.ibx_body_forces.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.ibx_cache_local_indices.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                              ctypes.c_void_p]
        L.ibx_fe_quadrature_points.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]
        L.ibx_fe_assemble_rhs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
        L.ibx_redistribute.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for name in ("ibx_accumulate_ghosts", "ibx_fill_ghosts"):
            getattr(L, name).argtypes = [P, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
        for name in ("ibx_interpolate", "ibx_spread"):
            getattr(L, name).argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        if hasattr(L, "ibx_plan_create"):
            L.ibx_plan_create.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_void_p)]
            L.ibx_plan_create2.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]
            L.ibx_plan_create3.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]
            L.ibx_plan_tile_shape.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
            for name in ("ibx_plan_bin", "ibx_plan_spread", "ibx_plan_interpolate", "ibx_plan_step"):
                getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            T = ctypes.POINTER(Transfer)
            L.ibx_plan_step_io.argtypes = [ctypes.c_void_p, T, ctypes.c_int, T, ctypes.c_int, T, ctypes.c_int,
                                           ctypes.c_void_p]
            L.ibx_plan_graph.argtypes = [ctypes.c_void_p, T, ctypes.c_int, T, ctypes.c_int, T, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
            L.ibx_graph_launch.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.ibx_graph_kernels.argtypes = [ctypes.c_void_p]
            L.ibx_graph_destroy.argtypes = [ctypes.c_void_p]
            L.ibx_plan_tma_problems.argtypes = [ctypes.c_void_p]
            L.ibx_plan_scratch_bytes.argtypes = [ctypes.c_void_p]
            L.ibx_plan_scratch_bytes.restype = ctypes.c_longlong
            L.ibx_plan_destroy.argtypes = [ctypes.c_void_p]
            ip = ctypes.POINTER(ctypes.c_int)
            L.ibx_plan_get_bins.argtypes = [ctypes.c_void_p, ip, ip, ip, ip, ip]
            L.ibx_plan_status.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ip]
            L.ibx_plan_n_tiles.argtypes = [ctypes.c_void_p]
            L.ibx_plan_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
            L.ibx_plan_get_tuning.argtypes = [ctypes.c_void_p, ip, ip, ip]
            L.ibx_plan_set_visit_kernel.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.ibx_plan_get_visit_kernel.argtypes = [ctypes.c_void_p]
            L.ibx_plan_set_interp_kernel.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.ibx_plan_get_interp_kernel.argtypes = [ctypes.c_void_p]
            L.ibx_plan_set_step_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.ibx_plan_get_step_mode.argtypes = [ctypes.c_void_p]
            L.ibx_plan_set_unit_cap.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.ibx_plan_get_unit_cap.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def status_string(status):
    try:
        return lib().ibx_status_string(int(status)).decode()
    except Exception:  # library missing
        return "status %d" % status


def kernel_launches():
    """Number of CUDA kernels libibx has launched in this process."""
    return int(lib().ibx_kernel_launches())


def kernel_id(kernel):
    if isinstance(kernel, str):
        k = lib().ibx_kernel_from_name(kernel.encode())
        if k < 0:
            raise IbxError(E_BAD_KERNEL, "unknown kernel %r" % kernel)
        return k
    return int(kernel)


def get_stencil_size(kernel):
    return lib().ibx_get_stencil_size(kernel_id(kernel))


def get_minimum_ghost_width(kernel):
    return lib().ibx_get_minimum_ghost_width(kernel_id(kernel))


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream_handle(stream):
    if stream is None:
        import torch

        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(getattr(stream, "cuda_stream", stream))


def make_problem(dim, centering, mode, ilower, iupper, dx, x_lower, x_upper, q, X, Q, Q_depth=None, q_depth=1,
                 gcw=(0, 0, 0), indices=None, Xshift=None, touches_physical_lower=(0, 0, 0),
                 touches_physical_upper=(0, 0, 0), n_markers=None):
    """Build an ibx_problem from torch tensors (device memory).  ``q`` is a
    tensor (cell data) or a list of one tensor per axis (side data)."""
    P = Problem()
    P.dim = dim
    P.centering = centering
    P.mode = mode
    for d in range(3):
        P.ilower[d] = int(ilower[d]) if d < dim else 0
        P.iupper[d] = int(iupper[d]) if d < dim else 0
        P.gcw[d] = int(gcw[d]) if d < len(gcw) else 0
        P.dx[d] = float(dx[d]) if d < dim else 1.0
        P.x_lower[d] = float(x_lower[d]) if d < dim else 0.0
        P.x_upper[d] = float(x_upper[d]) if d < dim else 1.0
        P.touches_physical_lower[d] = int(touches_physical_lower[d]) if d < len(touches_physical_lower) else 0
        P.touches_physical_upper[d] = int(touches_physical_upper[d]) if d < len(touches_physical_upper) else 0
    qs = q if isinstance(q, (list, tuple)) else [q]
    for a, t in enumerate(qs):
        P.q[a] = t.data_ptr()
    P.q_depth = q_depth
    P.X = X.data_ptr()
    P.Q = Q.data_ptr()
    P.Q_depth = Q_depth if Q_depth is not None else (dim if centering == SIDE else q_depth)
    P.n_markers = int(n_markers if n_markers is not None else X.numel() // dim)
    if indices is not None:
        P.indices = indices.data_ptr()
        P.n_indices = int(indices.numel())
    if Xshift is not None:
        P.Xshift = Xshift.data_ptr()
    P._keep = (qs, X, Q, indices, Xshift)  # keep tensors alive with the descriptor
    return P


def _array(problems):
    if isinstance(problems, Problem):
        problems = [problems]
    arr = (Problem * len(problems))(*problems)
    return arr, len(problems)


def spread(problems, kernel, precision=FP64, stream=None):
    arr, n = _array(problems)
    rc = lib().ibx_spread(arr, n, kernel_id(kernel), precision, _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_spread")


def interpolate(problems, kernel, precision=FP64, stream=None):
    arr, n = _array(problems)
    rc = lib().ibx_interpolate(arr, n, kernel_id(kernel), precision, _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_interpolate")


class PatchBox(ctypes.Structure):
    """ibx_patch_box: one patch of a level (cell box and geometry)."""

    _fields_ = [("ilower", ctypes.c_int * 3), ("iupper", ctypes.c_int * 3), ("x_lower", ctypes.c_double * 3),
                ("x_upper", ctypes.c_double * 3), ("dx", ctypes.c_double * 3)]


def redistribute(dim, boxes, X, stream=None):
    """Owner patch of every marker and the markers grouped by owner
    (ibx_redistribute).  boxes: [(ilower, iupper, x_lower, x_upper, dx), ...];
    X: device float64 tensor.  Returns (owner, order, patch_offsets) device
    int32 tensors."""
    import torch

    arr = (PatchBox * max(1, len(boxes)))()
    for k, (ilo, ihi, xl, xu, dx) in enumerate(boxes):
        for d in range(dim):
            arr[k].ilower[d], arr[k].iupper[d] = int(ilo[d]), int(ihi[d])
            arr[k].x_lower[d], arr[k].x_upper[d], arr[k].dx[d] = float(xl[d]), float(xu[d]), float(dx[d])
    n = X.numel() // dim
    owner = torch.empty(n, dtype=torch.int32, device=X.device)
    order = torch.empty(n, dtype=torch.int32, device=X.device)
    offsets = torch.empty(len(boxes) + 2, dtype=torch.int32, device=X.device)
    rc = lib().ibx_redistribute(int(dim), arr, len(boxes), _ptr(X), int(n), _ptr(owner), _ptr(order), _ptr(offsets),
                                _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_redistribute")
    return owner, order, offsets


class PatchGeometry(ctypes.Structure):
    """ibx_patch_geometry: cell box, geometry and periodic boundary flags."""

    _fields_ = [("dim", ctypes.c_int), ("ilower", ctypes.c_int * 3), ("iupper", ctypes.c_int * 3),
                ("x_lower", ctypes.c_double * 3), ("x_upper", ctypes.c_double * 3), ("dx", ctypes.c_double * 3),
                ("touches_periodic_lower", ctypes.c_int * 3), ("touches_periodic_upper", ctypes.c_int * 3)]


def cache_local_indices(dim, ilower, iupper, x_lower, x_upper, dx, touches_periodic_lower, touches_periodic_upper,
                        periodic_shift, ghost_width, want_ghost_box, X, capacity=None, stream=None):
    """LIndexSetData::cacheLocalIndices on the device (ibx_cache_local_indices):
    returns (local_indices int32, periodic_shifts float64 [dim per entry],
    cells int32 [dim per entry]) device tensors.  X: device float64 tensor."""
    import torch

    G = PatchGeometry()
    G.dim = dim
    for d in range(dim):
        G.ilower[d], G.iupper[d] = int(ilower[d]), int(iupper[d])
        G.x_lower[d], G.x_upper[d], G.dx[d] = float(x_lower[d]), float(x_upper[d]), float(dx[d])
        G.touches_periodic_lower[d] = int(touches_periodic_lower[d])
        G.touches_periodic_upper[d] = int(touches_periodic_upper[d])
    ps = (ctypes.c_int * 3)(*([int(v) for v in periodic_shift] + [0] * (3 - len(periodic_shift))))
    gw = (ctypes.c_int * 3)(*([int(v) for v in ghost_width] + [0] * (3 - len(ghost_width))))
    n = X.numel() // dim
    cap = (3 ** dim) * max(n, 1) if capacity is None else int(capacity)
    idx = torch.empty(max(cap, 1), dtype=torch.int32, device=X.device)
    sh = torch.empty(max(cap, 1) * dim, dtype=torch.float64, device=X.device)
    cells = torch.empty(max(cap, 1) * dim, dtype=torch.int32, device=X.device)
    cnt = ctypes.c_int(0)
    rc = lib().ibx_cache_local_indices(ctypes.byref(G), ps, gw, int(want_ghost_box), _ptr(X), int(n), int(cap),
                                       _ptr(idx), _ptr(sh), _ptr(cells), ctypes.byref(cnt), _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_cache_local_indices")
    m = cnt.value
    return idx[:m], sh[: m * dim], cells[: m * dim]


FE_SIMPLEX_P1, FE_TENSOR_Q1 = 0, 1


class FeMesh(ctypes.Structure):
    """ibx_fe_mesh: first-order Lagrange mesh of one element family (device
    arrays)."""

    _fields_ = [("dim", ctypes.c_int), ("n_nodes", ctypes.c_int), ("n_elems", ctypes.c_int),
                ("elem_nodes", ctypes.c_void_p), ("X", ctypes.c_void_p), ("elem_type", ctypes.c_int)]


def fe_nodes_per_elem(dim, elem_type):
    return (4 if dim == 2 else 8) if elem_type == FE_TENSOR_Q1 else dim + 1


class QuadRule(ctypes.Structure):
    """ibx_quad_rule: reference points and weights (host arrays)."""

    _fields_ = [("n_points", ctypes.c_int), ("points", ctypes.c_void_p), ("weights", ctypes.c_void_p)]


def _fe_args(dim, elem_nodes, X, points, weights, elem_type=FE_SIMPLEX_P1):
    import numpy as np

    M = FeMesh()
    M.dim = dim
    M.elem_type = elem_type
    M.n_nodes = X.numel() // dim
    M.n_elems = elem_nodes.numel() // fe_nodes_per_elem(dim, elem_type)
    M.elem_nodes = _ptr(elem_nodes).value
    M.X = _ptr(X).value
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
    w = np.ascontiguousarray(weights, dtype=np.float64).reshape(-1)
    R = QuadRule()
    R.n_points = w.size
    R.points = pts.ctypes.data
    R.weights = w.ctypes.data
    return M, R, (pts, w)


def fe_quadrature_points(dim, elem_nodes, X, points, weights, F=None, n_vars=0, elem_type=FE_SIMPLEX_P1,
                         stream=None):
    """FEDataManager::spread's quadrature points (ibx_fe_quadrature_points):
    returns (X_qp, F_JxW_qp or None, JxW) float64 device tensors."""
    import torch

    M, R, keep = _fe_args(dim, elem_nodes, X, points, weights, elem_type)
    nq = M.n_elems * R.n_points
    X_qp = torch.empty(max(nq, 1) * dim, dtype=torch.float64, device=X.device)
    JxW = torch.empty(max(nq, 1), dtype=torch.float64, device=X.device)
    F_qp = torch.empty(max(nq, 1) * max(n_vars, 1), dtype=torch.float64, device=X.device) if F is not None else None
    status = torch.zeros(1, dtype=torch.int32, device=X.device)
    rc = lib().ibx_fe_quadrature_points(ctypes.byref(M), ctypes.byref(R), _ptr(F), int(n_vars), _ptr(X_qp),
                                        _ptr(F_qp), _ptr(JxW), _ptr(status), _stream_handle(stream))
    del keep
    if rc:
        raise IbxError(rc, "ibx_fe_quadrature_points")
    if int(status.item()):
        raise IbxError(E_ARG, "ibx_fe_quadrature_points: negative node index")
    return X_qp[: nq * dim], None if F_qp is None else F_qp[: nq * n_vars], JxW[:nq]


def fe_assemble_rhs(dim, elem_nodes, X, points, weights, U_qp, n_vars, rhs, elem_type=FE_SIMPLEX_P1, stream=None):
    """FEDataManager::interp's right-hand side (ibx_fe_assemble_rhs): adds into
    rhs (float64 device tensor, n_vars per node)."""
    M, R, keep = _fe_args(dim, elem_nodes, X, points, weights, elem_type)
    rc = lib().ibx_fe_assemble_rhs(ctypes.byref(M), ctypes.byref(R), _ptr(U_qp), int(n_vars), _ptr(rhs),
                                   _stream_handle(stream))
    del keep
    if rc:
        raise IbxError(rc, "ibx_fe_assemble_rhs")


def spring_forces(dim, X, master, slave, stiffness, rest_length, F, accumulate=False, status=None, stream=None):
    """Linear spring forces into F (ibx_spring_forces).  Device tensors: X
    float64 (dim per marker), master/slave int32, stiffness/rest_length
    float64, F float64 (plain form) or float32 (mixed form).  Returns the
    status tensor (bit 0: a node index was out of range)."""
    import torch

    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device=X.device)
    precision = FP64 if F.dtype == torch.float64 else MIXED
    rc = lib().ibx_spring_forces(int(dim), int(F.numel() // dim), _ptr(X), int(master.numel()), _ptr(master),
                                 _ptr(slave), _ptr(stiffness), _ptr(rest_length), _ptr(F), precision,
                                 1 if accumulate else 0, _ptr(status), _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_spring_forces")
    return status


def beam_forces(dim, X, master, next_, prev, rigidity, curvature, F, accumulate=False, status=None, stream=None):
    """Beam (bending) forces into F (ibx_beam_forces).  Device tensors: X and
    curvature (dim per beam) float64, master/next_/prev int32, rigidity
    float64, F float64 or float32.  Returns the status tensor."""
    import torch

    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device=X.device)
    precision = FP64 if F.dtype == torch.float64 else MIXED
    rc = lib().ibx_beam_forces(int(dim), int(F.numel() // dim), _ptr(X), int(master.numel()), _ptr(master),
                               _ptr(next_), _ptr(prev), _ptr(rigidity), _ptr(curvature), _ptr(F), precision,
                               1 if accumulate else 0, _ptr(status), _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_beam_forces")
    return status


def target_point_forces(dim, X, U, node, kappa, eta, X_target, F, accumulate=False, max_displacement=None,
                        status=None, stream=None):
    """Target-point forces into F (ibx_target_point_forces).  U may be None
    (zero velocities); max_displacement, a one-element float64 device tensor
    or None, receives the largest |X_target - X|.  Returns the status
    tensor."""
    import torch

    if status is None:
        status = torch.zeros(1, dtype=torch.int32, device=X.device)
    precision = FP64 if F.dtype == torch.float64 else MIXED
    rc = lib().ibx_target_point_forces(int(dim), int(F.numel() // dim), _ptr(X), _ptr(U) if U is not None else None,
                                       int(node.numel()), _ptr(node), _ptr(kappa), _ptr(eta), _ptr(X_target),
                                       _ptr(F), precision, 1 if accumulate else 0,
                                       _ptr(max_displacement) if max_displacement is not None else None,
                                       _ptr(status), _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_target_point_forces")
    return status


def body_forces(dim, structure, force, F, has_force=None, stream=None):
    """Uniform body forces of structures added into F (ibx_body_forces):
    structure int32 per marker, force float64 (dim per structure id),
    has_force int32 per structure id or None (every structure)."""
    import torch

    precision = FP64 if F.dtype == torch.float64 else MIXED
    rc = lib().ibx_body_forces(int(dim), int(F.numel() // dim), _ptr(structure), int(force.numel() // dim),
                               _ptr(force), _ptr(has_force) if has_force is not None else None, _ptr(F), precision,
                               _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_body_forces")


def accumulate_ghosts(problem, periodic, stream=None):
    """SAMRAIGhostDataAccumulator on one IBX_MODE_PATCH patch covering the
    domain (ibx_accumulate_ghosts); periodic: per-dimension flags."""
    per = (ctypes.c_int * 3)(*([int(v) for v in periodic] + [0] * (3 - len(periodic))))
    rc = lib().ibx_accumulate_ghosts(ctypes.byref(problem), per, _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_accumulate_ghosts")


def fill_ghosts(problem, periodic, stream=None):
    """Periodic ghost fill of one IBX_MODE_PATCH patch covering the domain."""
    per = (ctypes.c_int * 3)(*([int(v) for v in periodic] + [0] * (3 - len(periodic))))
    rc = lib().ibx_fill_ghosts(ctypes.byref(problem), per, _stream_handle(stream))
    if rc:
        raise IbxError(rc, "ibx_fill_ghosts")


class Transfer(ctypes.Structure):
    """ibx_transfer: one copy of ibx_plan_step_io."""
    _fields_ = [("dst", ctypes.c_void_p), ("src", ctypes.c_void_p), ("bytes", ctypes.c_size_t)]


def _transfers(pairs):
    """ctypes array of ibx_transfer for (dst, src) tensor pairs."""
    pairs = list(pairs)
    if not pairs:
        return None
    arr = (Transfer * len(pairs))()
    for k, (dst, src) in enumerate(pairs):
        nb = dst.numel() * dst.element_size()
        if src.numel() * src.element_size() != nb or not dst.is_contiguous() or not src.is_contiguous():
            raise ValueError("a transfer needs two contiguous tensors of the same byte size")
        arr[k] = Transfer(dst.data_ptr(), src.data_ptr(), nb)
    return arr


class Graph:
    """A plan step captured into a CUDA graph by ibx_plan_graph (the plan's
    stream priorities kept); launch() replays it on a stream."""

    def __init__(self, plan, in_X=(), in_Q=(), out_Q=(), capture_stream=None):
        import torch

        s = capture_stream if capture_stream is not None else torch.cuda.Stream()
        # the capture stream starts after the work already queued on the current one
        s.wait_stream(torch.cuda.current_stream())
        arrs = [_transfers(pairs) for pairs in (in_X, in_Q, out_Q)]
        h = ctypes.c_void_p()
        rc = lib().ibx_plan_graph(plan.h, arrs[0], len(in_X), arrs[1], len(in_Q), arrs[2], len(out_Q),
                                  _stream_handle(s), ctypes.byref(h))
        if rc:
            raise IbxError(rc, "ibx_plan_graph")
        self.h = h
        self._keep = (plan, arrs, in_X, in_Q, out_Q)  # the buffers the graph addresses

    @property
    def kernels(self):
        """Library kernels one launch runs."""
        return int(lib().ibx_graph_kernels(self.h))

    def launch(self, stream=None):
        rc = lib().ibx_graph_launch(self.h, _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_graph_launch")

    def close(self):
        if self.h:
            lib().ibx_graph_destroy(self.h)
            self.h = None
            self._keep = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Binned spread/interpolate pipeline over fixed IBX_MODE_PERIODIC problems."""

    def __init__(self, problems, kernel, precision=MIXED, interp_problems=None, tile_shape=0):
        arr, n = _array(problems)
        self._problems = (problems, interp_problems)
        self._arr = arr
        h = ctypes.c_void_p()
        if interp_problems is None:
            arr2 = arr
        else:
            arr2, n2 = _array(interp_problems)
            self._arr2 = arr2
            if n2 != n:
                raise IbxError(E_ARG, "ibx_plan_create3")
        rc = lib().ibx_plan_create3(arr, arr2, n, kernel_id(kernel), precision, int(tile_shape), ctypes.byref(h))
        if rc:
            raise IbxError(rc, "ibx_plan_create")
        self.h = h

    @property
    def separate_interp(self):
        """True when the plan interpolates into its own targets (interp_problems
        given); otherwise interpolation reads the spread targets and writes
        the spread sources."""
        return self._problems[1] is not None

    def bin(self, stream=None):
        rc = lib().ibx_plan_bin(self.h, _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_plan_bin")

    def step(self, stream=None):
        """bin, then spread and interpolate concurrently (ibx_plan_step)."""
        rc = lib().ibx_plan_step(self.h, _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_plan_step")

    def step_io(self, in_X=(), in_Q=(), out_Q=(), stream=None):
        """One step with its host transfers (ibx_plan_step_io): each argument
        a list of (dst, src) tensor pairs of equal byte size -- in_X copied
        first, in_Q behind it beside the binning (the spread waits for it),
        out_Q as soon as the interpolation ends.  Host tensors should be
        pinned."""
        arrs = [_transfers(pairs) for pairs in (in_X, in_Q, out_Q)]
        rc = lib().ibx_plan_step_io(self.h, arrs[0], len(in_X), arrs[1], len(in_Q), arrs[2], len(out_Q),
                                    _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_plan_step_io")

    def graph(self, in_X=(), in_Q=(), out_Q=(), capture_stream=None):
        """One step (with the host transfers of step_io, if any) captured into
        a CUDA graph that keeps the plan's stream priorities (Graph).  Close
        the graph before the plan."""
        return Graph(self, in_X, in_Q, out_Q, capture_stream)

    def spread(self, stream=None):
        rc = lib().ibx_plan_spread(self.h, _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_plan_spread")

    def interpolate(self, stream=None):
        rc = lib().ibx_plan_interpolate(self.h, _stream_handle(stream))
        if rc:
            raise IbxError(rc, "ibx_plan_interpolate")

    def status(self, stream=None):
        st = ctypes.c_int(0)
        rc = lib().ibx_plan_status(self.h, _stream_handle(stream), ctypes.byref(st))
        if rc:
            raise IbxError(rc, "ibx_plan_status")
        return st.value

    def set_tuning(self, item_units=None, dense_min=None, dense_blocks_per_sm=None):
        """Spread tuning knobs (see ibx_plan_set_tuning); None keeps a value."""
        cur = self.tuning()
        vals = [cur[0] if item_units is None else item_units, cur[1] if dense_min is None else dense_min,
                cur[2] if dense_blocks_per_sm is None else dense_blocks_per_sm]
        rc = lib().ibx_plan_set_tuning(self.h, *[int(v) for v in vals])
        if rc:
            raise IbxError(rc, "ibx_plan_set_tuning")

    @property
    def tile_shape(self):
        """(shape id, tile edges per dimension)."""
        e = (ctypes.c_int * 3)()
        sh = lib().ibx_plan_tile_shape(self.h, e)
        return sh, tuple(e)

    @property
    def visit_kernel(self):
        """Form of the per-visit spread kernel (see ibx_plan_set_visit_kernel)."""
        return lib().ibx_plan_get_visit_kernel(self.h)

    @visit_kernel.setter
    def visit_kernel(self, form):
        rc = lib().ibx_plan_set_visit_kernel(self.h, int(form))
        if rc:
            raise IbxError(rc, "ibx_plan_set_visit_kernel")

    @property
    def interp_kernel(self):
        """Form of the interpolation (see ibx_plan_set_interp_kernel)."""
        return lib().ibx_plan_get_interp_kernel(self.h)

    @interp_kernel.setter
    def interp_kernel(self, form):
        rc = lib().ibx_plan_set_interp_kernel(self.h, int(form))
        if rc:
            raise IbxError(rc, "ibx_plan_set_interp_kernel")

    @property
    def step_mode(self):
        """Order of spread and interpolation in step() (see ibx_plan_set_step_mode)."""
        return lib().ibx_plan_get_step_mode(self.h)

    @step_mode.setter
    def step_mode(self, mode):
        rc = lib().ibx_plan_set_step_mode(self.h, int(mode))
        if rc:
            raise IbxError(rc, "ibx_plan_set_step_mode")

    @property
    def unit_cap(self):
        """Most markers per home unit (see ibx_plan_set_unit_cap)."""
        return lib().ibx_plan_get_unit_cap(self.h)

    @unit_cap.setter
    def unit_cap(self, cap):
        rc = lib().ibx_plan_set_unit_cap(self.h, int(cap))
        if rc:
            raise IbxError(rc, "ibx_plan_set_unit_cap")

    def tuning(self):
        """(item_units, dense_min, dense_blocks_per_sm)."""
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        rc = lib().ibx_plan_get_tuning(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        if rc:
            raise IbxError(rc, "ibx_plan_get_tuning")
        return a.value, b.value, c.value

    @property
    def n_tiles(self):
        return lib().ibx_plan_n_tiles(self.h)

    def bins(self, n_markers):
        """(base_c, base_s, home_tile, tile_start, home_list) as numpy arrays."""
        import numpy as np

        ip = ctypes.POINTER(ctypes.c_int)
        bc = np.zeros(3 * n_markers, dtype=np.int32)
        bs = np.zeros(3 * n_markers, dtype=np.int32)
        ht = np.zeros(n_markers, dtype=np.int32)
        ts = np.zeros(self.n_tiles + 1, dtype=np.int32)
        hl = np.zeros(n_markers, dtype=np.int32)
        rc = lib().ibx_plan_get_bins(self.h, *(a.ctypes.data_as(ip) for a in (bc, bs, ht, ts, hl)))
        if rc:
            raise IbxError(rc, "ibx_plan_get_bins")
        return bc, bs, ht, ts, hl

    @property
    def tma_problems(self):
        """Problems whose interpolation sources load by tensor copies in the
        staged interpolation forms (see ibx_plan_tma_problems)."""
        return lib().ibx_plan_tma_problems(self.h)

    @property
    def scratch_bytes(self):
        return lib().ibx_plan_scratch_bytes(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().ibx_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
