"""Golden korder derivative matrices from the reference's own builder (run
where the reference checkout exists): __make_S_by_k__ of
pycbf/gpu/__core_bf_classes__.py, taken out of that module with ast and
executed alone (the module imports cupy, absent here), for the kernel
lengths the tests use.  Stored as float64 and as the float32 copy the
reference's classes hand to their kernels.

    python tests/golden/make_korder_golden.py /path/to/reference
"""
import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
KS = (4, 6, 8, 16, 32)


def reference_builder(ref):
    path = os.path.join(ref, "pycbf", "gpu", "__core_bf_classes__.py")
    with open(path) as fp:
        tree = ast.parse(fp.read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "__make_S_by_k__")
    ns = {}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), path, "exec"), ns)
    return ns["__make_S_by_k__"]


def main(ref):
    make_s = reference_builder(ref)
    out = {}
    for k in KS:
        s = np.asarray(make_s(k), np.float64)
        out[f"S{k}_f64"] = s
        out[f"S{k}"] = s.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "korder_S.npz"), **out)
    print("wrote korder_S.npz:", sorted(out))


def oracle_ref_root() -> str:
    """The reference checkout: $PYCBF_REF, else the default of oracle/Makefile."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    from oracle.oracle import ref_root
    return ref_root()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else oracle_ref_root())
