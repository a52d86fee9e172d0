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
