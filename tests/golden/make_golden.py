"""Build the golden fixtures in this folder from the reference's own tests.

Run from the repository root, with the IBAMR source tree available:

    python tests/golden/make_golden.py /path/to/IBAMR

It reads, as text, the reference test decks and their checked-in outputs:

* ``tests/IBTK/ghost_accumulation_01_{2d,3d}.{cell,side}.spread.{a,b}.{input,output}``:
  100 markers drawn with ``std::mt19937(42)`` / ``uniform_real_distribution(0,1)``
  (first Q, then X), spread with PIECEWISE_LINEAR on every patch of the finest
  level, ghost data accumulated, patch values printed to 16 digits
  (driver ``tests/IBTK/ghost_accumulation_01.cpp:115-160``);
* ``tests/interpolate/interpolate_01_{2d,3d}.<kernel>.exact.input``: the
  polynomial-reproduction known-answer tests (driver
  ``tests/interpolate/interpolate_01.cpp:146-212``), whose outputs only say OK.

The marker inputs are drawn with the oracle's ``ibxo_mt19937_uniform`` (libstdc++
``std::mt19937`` + ``std::uniform_real_distribution<double>``, the generator the
reference tests use) and stored next to the expected values, so the fixtures are
self-contained.  Writes ``ghost_accumulation_01.json`` and ``interpolate_01_exact.json``.
"""

import ctypes
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

KERNELS = ["PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4"]


def load_oracle():
    tmp = tempfile.mkdtemp()
    so = os.path.join(tmp, "libibx_oracle.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", "-o", so,
                           os.path.join(REPO, "oracle", "ibx_oracle.cpp"), "-lpthread"])
    lib = ctypes.CDLL(so)
    lib.ibxo_mt19937_uniform.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.POINTER(ctypes.c_double)]
    return lib


def mt_uniform(lib, seed, n, a, b):
    buf = (ctypes.c_double * n)()
    lib.ibxo_mt19937_uniform(seed, n, a, b, buf)
    return list(buf)


def strip_comments(text):
    return "\n".join(line.split("//")[0] for line in text.splitlines())


def parse_input(path):
    txt = strip_comments(open(path).read())
    out = {}
    m = re.search(r"\bN\s*=\s*(\d+)", txt)
    out["N"] = int(m.group(1))
    m = re.search(r'IB_DELTA_FUNCTION\s*=\s*"(\w+)"', txt)
    out["kernel"] = m.group(1)
    m = re.search(r"periodic_dimension\s*=\s*([\d,\s]+)", txt)
    out["periodic"] = [int(v) for v in m.group(1).replace(" ", "").strip(",").split(",") if v]
    m = re.search(r"max_levels\s*=\s*(\d+)", txt)
    out["max_levels"] = int(m.group(1))
    m = re.search(r"ratio_to_coarser\s*\{\s*level_1\s*=\s*([\d,\s]+)\}", txt)
    out["ratio"] = [int(v) for v in m.group(1).replace(" ", "").strip(",").split(",") if v]
    m = re.search(r"ghost_width\s*=\s*(\d+)", txt)
    out["ghost_width"] = int(m.group(1)) if m else None
    m = re.search(r'var_type\s*=\s*"(\w+)"', txt)
    out["var_type"] = m.group(1) if m else None
    m = re.search(r'function\s*=\s*"([^"]+)"', txt)
    out["function"] = m.group(1) if m else None
    return out


def parse_output(path, dim):
    """Patches printed by ghost_accumulation_01: x lower / x upper and every
    array(i,j[,k]) value of the patch box, per side normal (or depth)."""
    lines = open(path).read().splitlines()
    patches = []
    cur = None
    comp = None
    side_normal = None
    k = 0
    while k < len(lines):
        line = lines[k].strip()
        if line.startswith("Rank:"):
            cur = {"x_lower": [], "x_upper": [], "arrays": {}}
            side_normal = None
            patches.append(cur)
        elif line == "x lower:":
            cur["x_lower"] = [float(lines[k + 1 + d]) for d in range(dim)]
            k += dim
        elif line == "x upper:":
            cur["x_upper"] = [float(lines[k + 1 + d]) for d in range(dim)]
            k += dim
        elif line.startswith("Array side normal"):
            side_normal = int(line.split("=")[1])
        elif line.startswith("Array depth"):
            depth = int(line.split("=")[1])
            comp = side_normal if side_normal is not None else depth
        elif line.startswith("array("):
            m = re.match(r"array\(([-\d,]+)\)\s*=\s*(\S+)", line)
            idx = [int(v) for v in m.group(1).split(",")]
            cur["arrays"].setdefault(comp if comp is not None else 0, []).append(idx + [float(m.group(2))])
        k += 1
    return patches


def ghost_accumulation_cases(ref, lib):
    cases = []
    base = os.path.join(ref, "tests", "IBTK")
    for dim in (2, 3):
        for cent in ("cell", "side"):
            for variant in ("a", "b"):
                stem = f"ghost_accumulation_01_{dim}d.{cent}.spread.{variant}"
                inp = parse_input(os.path.join(base, stem + ".input"))
                patches = parse_output(os.path.join(base, stem + ".output"), dim)
                centering = 1 if cent == "side" else 0
                out_patches = []
                for p in patches:
                    comps = sorted(p["arrays"].keys())
                    # Cell box from the printed indices (side arrays carry one extra face).
                    lo = [min(e[d] for c in comps for e in p["arrays"][c]) for d in range(dim)]
                    hi = []
                    for d in range(dim):
                        if centering == 1:
                            hi.append(max(e[d] for e in p["arrays"][(d + 1) % dim]))
                        else:
                            hi.append(max(e[d] for e in p["arrays"][0]))
                    dx = [(p["x_upper"][d] - p["x_lower"][d]) / (hi[d] - lo[d] + 1) for d in range(dim)]
                    out_patches.append({
                        "ilower": lo, "iupper": hi, "x_lower": p["x_lower"], "x_upper": p["x_upper"], "dx": dx,
                        "values": {str(c): p["arrays"][c] for c in comps},
                    })
                n_fine = inp["N"]
                for _ in range(inp["max_levels"] - 1):
                    n_fine *= inp["ratio"][0]
                q_depth = 1 if centering == 0 else dim
                Q = mt_uniform(lib, 42, q_depth * 100, 0.0, 1.0)
                # The reference draws Q first, then X, from the same generator.
                allv = mt_uniform(lib, 42, q_depth * 100 + dim * 100, 0.0, 1.0)
                assert allv[: len(Q)] == Q
                X = allv[len(Q):]
                cases.append({
                    "name": stem, "dim": dim, "centering": centering, "kernel": inp["kernel"],
                    "ghost_width": inp["ghost_width"], "periodic": inp["periodic"],
                    "domain_cells": [n_fine] * dim, "Q_depth": q_depth, "Q": Q, "X": X,
                    "patches": out_patches,
                    "source": f"tests/IBTK/{stem}.output",
                })
    return cases


def interpolate_exact_cases(ref, lib):
    cases = []
    base = os.path.join(ref, "tests", "interpolate")
    for dim in (2, 3):
        for kname in KERNELS:
            stem = f"interpolate_01_{dim}d.{kname.lower()}.exact"
            path = os.path.join(base, stem + ".input")
            if not os.path.exists(path):
                continue
            inp = parse_input(path)
            assert inp["kernel"] == kname, (stem, inp["kernel"])
            assert open(os.path.join(base, stem + ".output")).read().strip() == "OK"
            txt = strip_comments(open(path).read())
            m = re.search(r"level_0\s*=\s*\[\(([^)]*)\),\s*\(([^)]*)\)\]", txt)
            N = inp["N"]
            lo0 = [int(eval(v, {"N": N})) for v in m.group(1).split(",")]
            hi0 = [int(eval(v, {"N": N})) for v in m.group(2).split(",")]
            r = inp["ratio"][0]
            ilower = [v * r for v in lo0]
            iupper = [(v + 1) * r - 1 for v in hi0]
            dx = 1.0 / (N * r)
            x_lower = [ilower[d] * dx for d in range(dim)]
            x_upper = [(iupper[d] + 1) * dx for d in range(dim)]
            X = mt_uniform(lib, 42, dim * 100, x_lower[0], x_upper[0])
            cases.append({
                "name": stem, "dim": dim, "kernel": kname, "function": inp["function"],
                "ilower": ilower, "iupper": iupper, "dx": [dx] * dim, "x_lower": x_lower, "x_upper": x_upper,
                "periodic": inp["periodic"], "X": X, "Q_depth": dim,
                "tolerance": 1e-10 if kname == "IB_6" else 1e-12,
                "source": f"tests/interpolate/{stem}.input",
            })
    return cases


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("IBAMR_SOURCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py /path/to/IBAMR")
    lib = load_oracle()
    ga = ghost_accumulation_cases(ref, lib)
    ie = interpolate_exact_cases(ref, lib)
    with open(os.path.join(HERE, "ghost_accumulation_01.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": ga}, f, separators=(",", ":"))
    with open(os.path.join(HERE, "interpolate_01_exact.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": ie}, f, indent=0)
    print(f"wrote {len(ga)} ghost-accumulation cases, {len(ie)} interpolation KATs")


if __name__ == "__main__":
    main()
