#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference checkout.

Run once where the reference source tree exists (it does not on GPU hosts):

    make -C oracle ref            # builds oracle/_ref/ref_harness from the
                                  # reference's own hilbert_kernel.hpp / dsfun.hpp
    python tests/golden/make_golden.py [--reference /path/to/halmd]

Outputs (committed; small):
  lj_tables.json        (r, fval, U) rows of test/unit/mdsim/potentials/pair/lennard_jones.cpp:77-211
                        for sharp / shifted / force_shifted / smooth_r4, species AA/AB/BB
  smooth_r4_tables.json near-cutoff rows of test/unit/mdsim/forces/trunc/smooth_r4.cpp:59-149
  other_potential_tables.json  (r, fval, U) rows and parameters of the host tests
                        test/unit/mdsim/potentials/pair/{mie,morse,power_law}.cpp (shifted)
  accumulator.json      expected statistics of test/unit/numeric/accumulator.cpp:28-39
  hilbert_keys.json     keys of the reference's hilbert_kernel::map on seeded points
  dsfun.json            dsadd / dssub / dsmul of the reference's dsfun.hpp on seeded operands
"""
import argparse
import json
import os
import re
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def parse_rows(text):
    rows = re.findall(r"\{\{\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*\}\}", text)
    return [[float(a), float(b), float(c)] for a, b, c in rows]


def lj_tables(ref):
    src = open(os.path.join(ref, "test/unit/mdsim/potentials/pair/lennard_jones.cpp")).read()
    out = {}
    for trunc in ("sharp", "shifted", "force_shifted", "smooth_r4"):
        m = re.search(r"struct results<mdsim::host::potentials::pair::truncations::%s<" % trunc, src)
        body = src[m.end():]
        body = body[: body.find("};\n\ntemplate") if "};\n\ntemplate" in body else len(body)]
        tables = {}
        for pair in ("aa", "ab", "bb"):
            mm = re.search(r"%s\(\)\s*\{\s*return\s*\{\{(.*?)\}\};" % pair, body, re.S)
            tables[pair] = parse_rows(mm.group(1))
            assert len(tables[pair]) == 5, (trunc, pair)
        out[trunc] = tables
    return {
        "source": "test/unit/mdsim/potentials/pair/lennard_jones.cpp:77-211",
        "epsilon": [[1.0, 0.5], [0.5, 0.25]],
        "sigma": [[1.0, 2.0], [2.0, 4.0]],
        "r_cut_sigma": 5.0,
        "h": 0.005,
        "tolerance_eps_double": 5,
        "tables": out,
    }


def _matrix(src, name, cast=float):
    """The 2x2 matrix `name_array <<= a, b, c, d;` of a reference unit test."""
    m = re.search(r"%s_array <<=\s*(.*?);" % name, src, re.S)
    vals = [cast(float(x)) for x in re.findall(r"[-+0-9.eE]+", m.group(1))]
    assert len(vals) == 4, (name, vals)
    return [vals[0:2], vals[2:4]]


def other_potential_tables(ref):
    """(r, fval, U) rows of the host tests of mie, morse and power_law (shifted truncation)."""
    out = {}
    extra = {"mie": [("index_m", int), ("index_n", int)], "morse": [("r_min", float), ("distortion", float)],
             "power_law": [("index", int)]}
    for pot, fields in extra.items():
        path = "test/unit/mdsim/potentials/pair/%s.cpp" % pot
        src = open(os.path.join(ref, path)).read()
        host = src[: src.find("#ifdef HALMD_WITH_GPU", src.find("BOOST_AUTO_TEST_CASE"))]
        entry = {"source": path, "truncation": "shifted",
                 "r_cut_sigma": _matrix(host, "cutoff"), "epsilon": _matrix(host, "epsilon"),
                 "sigma": _matrix(host, "sigma")}
        for name, cast in fields:
            entry[name] = _matrix(host, name, cast)
        tables = {}
        for pair in ("aa", "ab", "bb"):
            mm = re.search(r"results_%s = \{\{(.*?)\}\};" % pair, host, re.S)
            tables[pair] = parse_rows(mm.group(1))
            assert len(tables[pair]) >= 5, (pot, pair)
        entry["tables"] = tables
        out[pot] = entry
    return out


def smooth_r4_tables(ref):
    src = open(os.path.join(ref, "test/unit/mdsim/forces/trunc/smooth_r4.cpp")).read()
    host = src[: src.find("BOOST_AUTO_TEST_SUITE_END() // host")]
    tables = {}
    for pair in ("aa", "ab", "bb"):
        mm = re.search(r"results_%s = \{\{(.*?)\}\};" % pair, host, re.S)
        tables[pair] = parse_rows(mm.group(1))
    return {
        "source": "test/unit/mdsim/forces/trunc/smooth_r4.cpp:59-149",
        "epsilon": [[1.0, 0.5], [0.5, 0.25]],
        "sigma": [[1.0, 2.0], [2.0, 4.0]],
        "r_cut_sigma": [[2.5, 2.0], [2.0, float(np.float32(2.0 ** (1 / 6.0)))]],
        "h": 1.0 / 256,
        "tolerance": "k*eps*(1+rc/(rc-r)), k=8 (aa, ab), k=9 (bb; fval 2x)",
        "tables": tables,
    }


def accumulator_expect(ref):
    src = open(os.path.join(ref, "test/unit/numeric/accumulator.cpp")).read()
    grab = lambda name: float(re.search(r"%s\(a\), ([-+0-9.eE]+)" % name, src).group(1))
    return {
        "source": "test/unit/numeric/accumulator.cpp:28-39",
        "values": list(range(10)),
        "count": 10,
        "mean": grab("mean"),
        "variance": grab("variance"),
        "sigma": grab("sigma"),
        "error_of_mean": grab("error_of_mean"),
        "sum": grab("sum"),
        "tolerance": 1e-14,
    }


def run_harness(harness, text):
    return subprocess.run([harness], input=text, capture_output=True, text=True, check=True).stdout.split("\n")


def hilbert_keys(harness):
    rng = np.random.default_rng(20240501)
    cases = []
    for depth in range(1, 11):
        pts = rng.uniform(-0.5, 0.5, size=(200, 3)).astype(np.float32)
        # edges: cell faces, box faces, the origin and symmetric points
        n = 2 ** depth
        edge = np.array([[-0.5, -0.5, -0.5], [0.0, 0.0, 0.0], [0.49999997, -0.5, 0.25],
                         [1.0 / n - 0.5, 0.5 - 1.0 / n, 0.0], [-1e-9, 1e-9, -0.25]], dtype=np.float32)
        pts = np.concatenate([pts, edge])
        text = "hilbert %d %d\n" % (depth, len(pts)) + "".join("%.9g %.9g %.9g\n" % tuple(p) for p in pts)
        keys = [int(x) for x in run_harness(harness, text) if x.strip()]
        cases.append({"depth": depth, "points": pts.tolist(), "keys": keys})
    return {"source": "halmd/mdsim/sorts/hilbert_kernel.hpp:70-230 (compiled from the reference tree)",
            "cases": cases}


def f2h(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def dsfun_vectors(harness):
    rng = np.random.default_rng(42)
    n = 512
    out = {"source": "halmd/numeric/mp/dsfun.hpp:124-210 (compiled from the reference tree)"}
    a = rng.uniform(-100, 100, n) * 10.0 ** rng.integers(-3, 3, n)
    b = rng.uniform(-100, 100, n) * 10.0 ** rng.integers(-3, 3, n)
    pairs = []
    for x, y in zip(a, b):
        x0 = np.float32(x); x1 = np.float32(x - float(x0))
        y0 = np.float32(y); y1 = np.float32(y - float(y0))
        pairs.append((x0, x1, y0, y1))
    for op in ("add", "sub", "mul"):
        text = "dsfun %s %d\n" % (op, n) + "".join("%08x %08x %08x %08x\n" % tuple(f2h(v) for v in p) for p in pairs)
        res = [line.split() for line in run_harness(harness, text) if line.strip()]
        out[op] = [[f2h(p[0]), f2h(p[1]), f2h(p[2]), f2h(p[3]), int(c0, 16), int(c1, 16)]
                   for p, (c0, c1) in zip(pairs, res)]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("HALMD_REFERENCE"),
                    help="the reference checkout (default: the HALMD_REFERENCE environment variable)")
    ap.add_argument("--harness", default=os.path.join(REPO, "oracle", "_ref", "ref_harness"))
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the reference checkout with --reference or HALMD_REFERENCE")
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REFERENCE=" + args.reference])
    fixtures = {
        "lj_tables.json": lj_tables(args.reference),
        "smooth_r4_tables.json": smooth_r4_tables(args.reference),
        "other_potential_tables.json": other_potential_tables(args.reference),
        "accumulator.json": accumulator_expect(args.reference),
        "hilbert_keys.json": hilbert_keys(args.harness),
        "dsfun.json": dsfun_vectors(args.harness),
    }
    for name, data in fixtures.items():
        with open(os.path.join(HERE, name), "w") as fh:
            json.dump(data, fh, indent=None, separators=(",", ":"))
            fh.write("\n")
        print("wrote", name)


if __name__ == "__main__":
    main()
