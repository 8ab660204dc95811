"""Extract the numeric fixtures of jVMC's own test-suite into
``reference_fixtures.json``.

The reference (JAX/Flax) cannot be imported here, so its test files are read
as text and only their literal numbers are taken:

* ``tests/tdvp_test.py``  ground-state energies ``exEs`` (line 32), the
  16-entry CpxRBM(L=4, M=2) weight vector (65-68) and the ZZ(t) series
  ``refZZ`` (122-126);
* ``tests/operator_test.py``  the fermion-model energy (line 254) and
  ``tests/data_ref/fermion_ref.txt`` (its wave-function table);
* ``tests/stats_test.py``  the known answers of ``test_sampled_obs`` (15-39).

Run from the repository root:  python tests/golden/make_golden.py [REF_ROOT]
"""

import ast
import json
import os
import re
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_fixtures.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def array_literal(src, name):
    """Return the first ``name = [...]`` / ``name = jnp.array([...])`` /
    ``name = np.array(\n [...])`` literal as a nested list of floats."""
    m = re.search(name + r"\s*=\s*(?:jnp|np)?\.?(?:array)?\(?\s*(\[[^\]]*(?:\][^\]]*)*?\])", src, re.S)
    if m is None:
        raise RuntimeError(f"{name} not found")
    return ast.literal_eval(m.group(1))


def numeric_expr(expr):
    """Evaluate a bracketed expression of numeric literals like
    ``[[2./3, 1],[1.,14./9]]`` (only numbers, brackets and + - * /)."""
    if not re.fullmatch(r"[\s\d\.\,\[\]\+\-\*/eEj]+", expr):
        raise RuntimeError("not a numeric literal: " + expr)
    return eval(expr, {"__builtins__": {}}, {})


def main():
    fx = {}
    tdvp = read("tests/tdvp_test.py")
    fx["tdvp_exEs"] = array_literal(tdvp, "exEs")
    fx["tdvp_gs_hxs"] = array_literal(tdvp, "hxs")
    fx["rbm_L4_M2_weights"] = array_literal(tdvp, "weights")
    fx["tdvp_refZZ"] = array_literal(tdvp, "refZZ")
    fx["tdvp_source"] = "tests/tdvp_test.py:32,65-68,122-126"

    op = read("tests/operator_test.py")
    m = re.search(r"jnp\.allclose\(Omean,\s*([-\d\.]+)\)", op)
    fx["fermion_energy"] = float(m.group(1))
    tab = np.loadtxt(os.path.join(REF, "tests/data_ref/fermion_ref.txt"), dtype=np.complex128)
    fx["fermion_table_re"] = tab.real.tolist()
    fx["fermion_table_im"] = tab.imag.tolist()
    fx["fermion_source"] = "tests/operator_test.py:189-254, tests/data_ref/fermion_ref.txt"

    st = read("tests/stats_test.py")
    fx["stats_obs1"] = [1, 2, 3]
    fx["stats_obs2"] = [[1, 4], [2, 5], [3, 7]]
    assert "jnp.array([[1, 2, 3]]" in st and "[[[1, 4], [2, 5], [3, 7]]]" in st
    mean1 = re.search(r"assertAlmostEqual\(obs1\.mean\(\)\[0\],\s*([^\)]+)\)", st).group(1)
    var1 = re.search(r"assertAlmostEqual\(obs1\.var\(\)\[0\],\s*([^\)]+)\)", st).group(1)
    cov2 = re.search(r"obs2\.covar\(\),\s*jnp\.array\((\[\[.*?\]\])\)", st).group(1)
    mean2 = re.search(r"obs2\.mean\(\),\s*jnp\.array\((\[.*?\])\)", st).group(1)
    cov12 = re.search(r"obs1\.covar\(obs2\),\s*jnp\.array\((\[.*?\])\)", st).group(1)
    fx["stats_mean1"] = numeric_expr(mean1)
    fx["stats_var1"] = numeric_expr(var1)
    fx["stats_covar2"] = numeric_expr(cov2)
    fx["stats_mean2"] = numeric_expr(mean2)
    fx["stats_covar12"] = numeric_expr(cov12)
    fx["stats_source"] = "tests/stats_test.py:15-39"

    with open(OUT, "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
