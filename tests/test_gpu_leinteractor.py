"""The C++ LEInteractor layer (include/ibx_leinteractor.h) on the GPU,
replaying the reference's own tests through the reference's call signatures:
tests/interpolate/interpolate_01.cpp (use_exact) for every kernel in 2D and
3D, and tests/IBTK/ghost_accumulation_01 (3D, spread, one 8^3 patch) for cell
and side data against the golden outputs."""

import re

import pytest

from golden_replay import load
from test_abi import compile_cpp_test, libibx  # noqa: F401  (fixture)

KERNELS = ["PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4"]


@pytest.fixture(scope="module")
def programs(libibx, tmp_path_factory):  # noqa: F811
    d = tmp_path_factory.mktemp("lei")
    return {dim: compile_cpp_test(libibx, dim, str(d / ("lei%d" % dim))) for dim in (2, 3)}


def run(exe, *args):
    import subprocess

    r = subprocess.run([exe] + list(args), capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", KERNELS)
def test_interpolate_01_exact(programs, dim, kernel):
    assert run(programs[dim], "kat", kernel).strip() == "OK"


def parse(out):
    arrays, comp = {}, None
    for line in out.splitlines():
        m = re.match(r"Array (?:side normal|depth) = (\d+)", line)
        if m:
            comp = int(m.group(1))
            continue
        m = re.match(r"array\(([-\d,]+)\) = (\S+)", line)
        if m:
            idx = tuple(int(v) for v in m.group(1).split(","))
            arrays[(comp, idx)] = float(m.group(2))
    return arrays


@pytest.mark.gpu
@pytest.mark.parametrize("centering", ["cell", "side"])
def test_ghost_accumulation_01_3d_spread(programs, centering):
    case = [c for c in load("ghost_accumulation_01.json")
            if c["name"] == "ghost_accumulation_01_3d.%s.spread.a" % centering][0]
    got = parse(run(programs[3], "spread", centering))
    patch = case["patches"][0]
    n = 0
    for comp_s, entries in patch["values"].items():
        for e in entries:
            v = got[(int(comp_s), tuple(e[:3]))]
            assert abs(v - e[3]) <= 1e-13 * max(1.0, abs(e[3])), (comp_s, e, v)
            n += 1
    assert n == len(got) and n > 0


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("centering,depth", [("side", 1), ("cell", 2)])
@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "PIECEWISE_CUBIC", "BSPLINE_4"])
def test_ldata_index_set_forms(programs, oracle, tmp_path, dim, centering, depth, kernel):
    """The reference's LData / LIndexSetData signatures (SAMRAI::tbox::Pointer
    handles, LIndexSetData::cacheLocalIndices on the device) against the
    oracle's reference flow on a periodic patch (LDataManager::spread over
    the ghost box, interp over the patch box) within 1e-12, and an
    interpolation over a sub-box (buildLocalIndices' general path) equal to
    the oracle's over the markers whose cell lies in it."""
    import numpy as np

    N = 32 if dim == 2 else 16
    rng = np.random.default_rng(77 + dim + 3 * KERNELS.index(kernel) + (centering == "cell"))
    n = 900
    X = np.concatenate([rng.uniform(0.0, 1.0, size=(n // 2, dim)),
                        np.mod(rng.uniform(-0.06, 0.06, size=(n - n // 2, dim)), 1.0)]).reshape(-1)
    Q_depth = dim if centering == "side" else depth
    ncomp = Q_depth
    F = rng.standard_normal(n * Q_depth)
    u = rng.standard_normal([ncomp] + [N] * dim)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as fh:
        fh.write(np.array([n, depth], dtype=np.int32).tobytes())
        fh.write(X.tobytes())
        fh.write(F.tobytes())
        fh.write(u.reshape(-1).tobytes())
    txt = run(programs[dim], "ldata", centering, kernel, str(N), str(inp), str(out))
    assert txt.startswith("OK")
    res = np.fromfile(out, dtype=np.float64)
    f = res[: ncomp * N ** dim].reshape([ncomp] + [N] * dim)
    U = res[ncomp * N ** dim: ncomp * N ** dim + n * Q_depth]
    U_sub = res[ncomp * N ** dim + n * Q_depth:]
    cen = 1 if centering == "side" else 0
    f_ref, U_ref = oracle.periodic_problem(dim, [N] * dim, kernel, X, F=F, u=u, centering=cen, depth=depth)
    assert np.max(np.abs(f - f_ref)) <= 1e-12 * np.max(np.abs(f_ref))
    assert np.max(np.abs(U - U_ref)) <= 1e-12 * np.max(np.abs(U_ref))
    # sub-box: the interior markers whose cell lies in [2, N - 3]^dim
    cells = np.floor(X.reshape(n, dim) * N).astype(int)
    inside = np.all((cells >= 2) & (cells <= N - 3), axis=1)
    Us = U_sub.reshape(n, Q_depth)
    Ur = U_ref.reshape(n, Q_depth)
    assert np.all(Us[~inside] == 7.0)
    assert np.max(np.abs(Us[inside] - Ur[inside])) <= 1e-12 * np.max(np.abs(Ur))
