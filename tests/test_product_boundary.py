"""The product path stands apart from the oracle (CPU only): no package source
imports it, and importing every module of the package, from the repository
root where the oracle is importable, loads nothing from it."""
import ast
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pycbf_gb300")
MODULES = sorted(f[:-3] for f in os.listdir(PKG) if f.endswith(".py") and f != "__init__.py")


def _is_oracle(name: str) -> bool:
    return name == "oracle" or name.startswith("oracle.")


def test_package_sources_do_not_import_the_oracle():
    for m in MODULES + ["__init__"]:
        tree = ast.parse(open(os.path.join(PKG, m + ".py")).read())
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                names = [node.module or ""]
            else:
                continue
            assert not any(_is_oracle(n) for n in names), (m, names)


def test_importing_the_package_loads_no_oracle_module():
    code = ("import importlib, sys\n"
            "for m in sys.argv[1:]:\n"
            "    importlib.import_module('pycbf_gb300.' + m)\n"
            "bad = sorted(m for m in sys.modules if m == 'oracle' or m.startswith('oracle.'))\n"
            "print(bad)\n"
            "sys.exit(1 if bad else 0)\n")
    r = subprocess.run([sys.executable, "-c", code, *MODULES], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
