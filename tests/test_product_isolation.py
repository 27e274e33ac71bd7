"""The product path stands on its own: no module of the package imports, loads or runs the
oracle (or anything outside the package and its compiled library), and the library's build
inputs are the package's own CUDA sources."""
import ast
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "matpl_gb300")


def _py_files():
    for root, _, files in os.walk(PKG):
        if "_build" in root:
            continue
        for f in files:
            if f.endswith(".py"):
                yield os.path.join(root, f)


def test_package_never_imports_the_oracle():
    for path in _py_files():
        tree = ast.parse(open(path).read(), path)
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                mods = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                mods = [node.module or ""] if node.level == 0 else []
            else:
                continue
            for m in mods:
                assert m.split(".")[0] not in ("oracle", "tests", "bench"), (path, m)


def test_package_names_no_oracle_file_or_build_output():
    pat = re.compile(r"oracle[/\\]|_ref[/\\]|libneighconst|libnepneigh|liblammps_neigh")
    for path in _py_files():
        for i, line in enumerate(open(path), 1):
            code = line.split("#", 1)[0]
            assert not pat.search(code), f"{path}:{i}: {line.strip()}"


def test_library_sources_are_the_package_own():
    src = open(os.path.join(PKG, "build.py")).read()
    assert "oracle" not in src.split('"""', 2)[-1]
    for f in os.listdir(os.path.join(PKG, "csrc")):
        txt = open(os.path.join(PKG, "csrc", f), errors="replace").read()
        for inc in re.findall(r'#include\s+"([^"]+)"', txt):
            assert os.path.exists(os.path.join(PKG, "csrc", inc)) or inc == "matpl_gb300.h", \
                (f, inc)
