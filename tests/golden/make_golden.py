"""Regenerate the golden fixtures in this folder from the reference sources.

Run where a checkout of the reference is available, with its path as the
only argument:  python tests/golden/make_golden.py <reference checkout>.
It is never run by the tests.

Fixtures written:
  tridiag_bdf.json  -- the reference's tridiagonal golden table, both as
                       committed in test/tridiagonalIntegrator.cpp:4-10 (parsed
                       from the text) and as recomputed by running the
                       reference's own generator test/reference/bdf.py
                       (BDFIntegrator / ExactIntegrator) for dt = 0.2, 0.05,
                       0.0125 and the exact solution at t = 1.
  qss_cesium.json   -- initial and final values of the CHEMEQ2 cesium test
                       problem and its settings, parsed from
                       test/old/test_qssintegrator.cpp (YI/YF at lines
                       161-186, EPS list at 112, itermax at 192).
"""
from __future__ import annotations

import importlib.util
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_bdf(ref: str):
    path = os.path.join(ref, "test", "reference", "bdf.py")
    spec = importlib.util.spec_from_file_location("ember_ref_bdf", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def parse_cpp_table(ref: str):
    text = open(os.path.join(ref, "test", "tridiagonalIntegrator.cpp")).read()
    body = text[text.index("soln[6][5] = {"):]
    body = body[:body.index("};")]
    rows = re.findall(r"\{([^{}]+)\}", body)
    return [[float(v) for v in r.split(",")] for r in rows]


def parse_cesium(ref: str):
    text = open(os.path.join(ref, "test", "old", "test_qssintegrator.cpp")).read()
    yi = {int(i): float(v) for i, v in re.findall(r"YI\[(\d+)\]\s*=\s*([-+0-9.eE]+);", text)}
    yf = {int(i): float(v) for i, v in re.findall(r"YF\[(\d+)\]\s*=\s*([-+0-9.eE]+);", text)}
    eps = re.search(r"double EPS\[15\]\s*=\s*\{([^}]*)\}", text).group(1)
    eps = [float(v) for v in eps.replace("\n", " ").split(",")]
    mxcase = int(re.search(r"int MXCASE\s*=\s*(\d+);", text).group(1))
    itermax = int(re.search(r"itermax\s*=\s*(\d+);", text).group(1))
    ti = float(re.search(r"double TI\s*=\s*([-+0-9.eE]+);", text).group(1))
    tf = float(re.search(r"double TF\s*=\s*([-+0-9.eE]+);", text).group(1))
    n = max(yi) + 1
    return {
        "species": ["O2-", "CS+", "CS", "CSO2", "O2", "N2", "NE"][:n],
        "YI": [yi[i] for i in range(n)],
        "YF": [yf[i] for i in range(n)],
        "eps_cases": eps[:mxcase],
        "itermax": itermax,
        "ymin": 1e-20,
        "t_initial": ti,
        "t_final": tf,
        "source": "test/old/test_qssintegrator.cpp:112,161-186,192",
    }


def main(ref: str) -> None:
    bdf = load_bdf(ref)
    y0 = np.array([0, 0.5, 2.0, 1.0, 0])
    k = np.array([0, 0, 0, 0.2, 0.4])
    A = np.array([[-2, 1, 0, 0, 0], [1, -2, 1, 0, 0], [0, 1, -2, 1, 0], [0, 0, 1, -2, 1], [0, 0, 0, 1, -2]],
                 dtype=float)
    out = {
        "source": "test/tridiagonalIntegrator.cpp:4-10 (table) and test/reference/bdf.py (generator)",
        "a": [0, 1, 1, 1, 1], "b": [-2] * 5, "c": [1, 1, 1, 1, 0], "k": k.tolist(), "y0": y0.tolist(),
        "table_cpp": parse_cpp_table(ref),
        "bdf_dt0.2": [y.tolist() for y in bdf.getBdfSolutions(0.20, 1.0, y0.copy(), A, k)],
        "bdf_dt0.05_t1": bdf.getBdfSolutions(0.05, 1.0, y0.copy(), A, k)[-1].tolist(),
        "bdf_dt0.0125_t1": bdf.getBdfSolutions(0.0125, 1.0, y0.copy(), A, k)[-1].tolist(),
        "exact_t1": bdf.ExactIntegrator(y0.copy(), A, k)(1.0).tolist(),
    }
    with open(os.path.join(HERE, "tridiag_bdf.json"), "w") as f:
        json.dump(out, f, indent=1)
    with open(os.path.join(HERE, "qss_cesium.json"), "w") as f:
        json.dump(parse_cesium(ref), f, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
