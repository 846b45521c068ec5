"""The numpy-only parameter draws (compound_prism_designer/workload.py) positioned by the
oracle give the same designs as the library's synth.random_design: the benchmark's
reference arm, which must not load the library, evaluates the very design the GPU arm
does. No GPU calls."""
import numpy as np

import oracle as O
from compound_prism_designer import synth, workload


def test_oracle_built_draws_equal_library_built_draws():
    for seed, G, B in [(20261204, 6, 64), (7, 3, 32), (11, 2, 128), (13, 5, 16), (17, 4, 64)]:
        d_lib = synth.random_design(np.random.default_rng(seed), G, B)
        d_orc = workload.random_params(np.random.default_rng(seed), G, B, O.accept_params)
        assert d_lib[2] == d_orc[1], (seed, d_lib[2], d_orc[1])
        a, b = d_lib[1], d_orc[0]
        for k in a:
            va, vb = a[k], b[k]
            if isinstance(va, (list, tuple)):
                assert np.array_equal(np.asarray(va, dtype=float), np.asarray(vb, dtype=float)), (seed, k)
            else:
                assert va == vb, (seed, k, va, vb)


def test_workload_module_imports_nothing_from_the_package():
    import ast
    import os

    src = open(os.path.join(os.path.dirname(workload.__file__), "workload.py")).read()
    for node in ast.walk(ast.parse(src)):
        if isinstance(node, ast.ImportFrom):
            assert node.level == 0 and node.module in ("__future__",), node.module
        elif isinstance(node, ast.Import):
            assert all(a.name in ("math", "numpy") for a in node.names)
