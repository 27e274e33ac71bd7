"""The product path stands on its own: no module of the package imports, loads or runs the
oracle or the reference comparator (or anything outside the package and its compiled library), and the library's build
inputs are the package's own CUDA sources; the public operators refuse host tensors rather
than fall back to a CPU path."""
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
                assert m.split(".")[0] not in ("oracle", "tests", "bench", "baseline"), (path, m)


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


def test_ops_refuse_cpu_tensors_instead_of_falling_back():
    """Every public operator fails loudly on host tensors: there is no CPU fallback."""
    import pytest
    import torch
    from matpl_gb300 import _lib, nep_ops, ops
    B, N, S = 1, 4, 6
    ln = torch.zeros(B, N, S, dtype=torch.int32)
    dE = torch.zeros(B, N, 4 * S, dtype=torch.float64)
    Rid = torch.zeros(B, N, 4 * S, 3, dtype=torch.float64)
    Rij = torch.zeros(B, N, S, 3, dtype=torch.float64)
    idr = torch.zeros(B, N, S, 4, dtype=torch.float64)
    F = torch.zeros(B, N, 3, dtype=torch.float64)
    NL = torch.full((N, S), -1, dtype=torch.int64)
    Ri = torch.zeros(N, S, 4, dtype=torch.float64)
    calls = [
        lambda: ops.calculateForce(ln, dE, Rid, F, 0),
        lambda: ops.calculateVirial(ln, dE, Rij, Rid, 0),
        lambda: ops.calculateCompress(torch.zeros(5, 1), torch.zeros(5, 25, 6)),
        lambda: ops.env_mat(idr, torch.zeros(N, dtype=torch.int32), torch.zeros(1, 4 * S),
                            torch.ones(1, 4 * S), 0.5, 6.0),
        lambda: ops.find_neighbore(torch.zeros(N, dtype=torch.int32), torch.rand(1, N, 3),
                                   torch.eye(3).unsqueeze(0) * 10, 1, S, 6.0, 6.0),
        lambda: nep_ops.nep_force_virial(NL, torch.zeros(N, S, 4, dtype=torch.float64), Ri, [N]),
        lambda: nep_ops.calculateNepForce(NL, torch.zeros(N, S, 4, dtype=torch.float64),
                                          torch.zeros(N, S, 4, 3, dtype=torch.float64),
                                          torch.zeros(N, 3, dtype=torch.float64)),
    ]
    for call in calls:
        with pytest.raises(_lib.MatplError, match="CUDA"):
            call()
