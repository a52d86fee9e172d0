"""CPU checks of the C-ABI boundary: libibx.so loads, exports every function
that include/*.h declares, the host-only queries answer like the reference's
LEInteractor (ibtk/src/lagrangian/LEInteractor.cpp:184-235), and the C++
LEInteractor layer (include/ibx_leinteractor.h) compiles in 2D and 3D."""

import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="session")
def libibx():
    from ibamr_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    return build.LIB


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h") or f == "ibx_leinteractor.h":
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        names.update(re.findall(r"\b(ibx_[a-z0-9_]+)\s*\(", text))
        # the Fortran-ABI routines are declared through IBX_FORTRAN_* macros
        names.update(re.findall(r"\bIBX_FORTRAN_(?:INTERP|SPREAD)[23]D\((lagrangian_[a-z0-9_]+_)\)", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(libibx):
    names = declared_functions()
    assert "ibx_spread" in names and "ibx_plan_create2" in names and "ibx_spread_noalloc" in names
    assert len([n for n in names if n.startswith("lagrangian_")]) == 24
    out = subprocess.run(["nm", "-D", "--defined-only", libibx], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = ctypes.CDLL(libibx)
    for n in names:
        getattr(L, n)


def test_plan_knobs_reject_a_null_plan(libibx):
    """The plan setters validate on the host (no device call): a null plan is
    an argument error, the getters answer -1."""
    L = ctypes.CDLL(libibx)
    E_ARG = 4
    for setter in ("ibx_plan_set_visit_kernel", "ibx_plan_set_interp_kernel", "ibx_plan_set_step_mode",
                   "ibx_plan_set_unit_cap"):
        fn = getattr(L, setter)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int]
        assert fn(None, 1) == E_ARG, setter
    for getter in ("ibx_plan_get_visit_kernel", "ibx_plan_get_interp_kernel", "ibx_plan_get_step_mode",
                   "ibx_plan_get_unit_cap"):
        fn = getattr(L, getter)
        fn.argtypes = [ctypes.c_void_p]
        assert fn(None) == -1, getter
    L.ibx_plan_set_tuning.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    assert L.ibx_plan_set_tuning(None, 128, 32, 2) == E_ARG
    L.ibx_plan_step_io.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p, ctypes.c_int] * 3 + [ctypes.c_void_p]
    assert L.ibx_plan_step_io(None, None, 0, None, 0, None, 0, None) == E_ARG
    # the graph entry points: no plan, no graph pointer or the legacy stream
    L.ibx_plan_graph.argtypes = ([ctypes.c_void_p] + [ctypes.c_void_p, ctypes.c_int] * 3 +
                                 [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)])
    h = ctypes.c_void_p(1234)
    assert L.ibx_plan_graph(None, None, 0, None, 0, None, 0, ctypes.c_void_p(1), ctypes.byref(h)) == E_ARG
    assert h.value is None  # cleared before the arguments are refused
    assert L.ibx_plan_graph(None, None, 0, None, 0, None, 0, ctypes.c_void_p(1), None) == E_ARG
    for name in ("ibx_graph_launch", "ibx_graph_kernels", "ibx_graph_destroy"):
        getattr(L, name).argtypes = [ctypes.c_void_p] + ([ctypes.c_void_p] if name == "ibx_graph_launch" else [])
    assert L.ibx_graph_launch(None, None) == E_ARG
    assert L.ibx_graph_kernels(None) == -1
    assert L.ibx_graph_destroy(None) == 0


def test_force_entry_points_validate_on_the_host(libibx):
    """Argument errors of the Lagrangian force entry points are found before
    any device call: a bad dimension, a missing status word, missing arrays;
    empty inputs succeed without a launch."""
    L = ctypes.CDLL(libibx)
    E_ARG = 4
    vp = ctypes.c_void_p
    L.ibx_beam_forces.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int] + [vp] * 6 + [ctypes.c_int,
                                                                                             ctypes.c_int, vp, vp]
    assert L.ibx_beam_forces(4, 0, None, 0, None, None, None, None, None, None, 0, 1, None, None) == E_ARG
    assert L.ibx_beam_forces(2, 0, None, 0, None, None, None, None, None, None, 0, 1, None, None) == E_ARG
    L.ibx_target_point_forces.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int] + [vp] * 5 + [
        ctypes.c_int, ctypes.c_int, vp, vp, vp]
    assert L.ibx_target_point_forces(2, 0, None, None, 3, None, None, None, None, None, 0, 1, None, None,
                                     None) == E_ARG
    L.ibx_body_forces.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, vp]
    assert L.ibx_body_forces(3, 0, None, 0, None, None, None, 0, None) == 0
    assert L.ibx_body_forces(3, 10, None, 2, None, None, None, 0, None) == E_ARG


def test_host_queries(libibx):
    L = ctypes.CDLL(libibx)
    L.ibx_status_string.restype = ctypes.c_char_p
    # LEInteractor::getStencilSize / getMinimumGhostWidth
    expect = {b"PIECEWISE_LINEAR": (2, 2), b"PIECEWISE_CUBIC": (4, 3), b"IB_3": (4, 3),
              b"IB_4": (4, 3), b"IB_6": (6, 4), b"BSPLINE_4": (4, 3)}
    for name, (width, ghost) in expect.items():
        k = L.ibx_kernel_from_name(name)
        assert k >= 0
        assert L.ibx_get_stencil_size(k) == width
        assert L.ibx_get_minimum_ghost_width(k) == ghost
    assert L.ibx_kernel_from_name(b"IB_5") == -1
    assert L.ibx_get_stencil_size(99) == -1
    assert L.ibx_status_string(0) == b"success"
    assert L.ibx_status_string(1) == b"unknown kernel function"


CPP_TEST = os.path.join(ROOT, "tests", "cpp", "leinteractor_test.cpp")


def compile_cpp_test(libibx, dim, out):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(libibx)
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-DNDIM=%d" % dim, "-I", INCLUDE, CPP_TEST,
           "-L", libdir, "-libx", "-Wl,-rpath," + libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_cpp_leinteractor_layer_compiles(libibx, tmp_path, dim):
    compile_cpp_test(libibx, dim, str(tmp_path / ("lei%d" % dim)))
