"""The torch operator library (torch.ops.CalcOps_cuda, libCalcOps_bind.so) on the CPU: it loads
with torch.ops.load_library, registers the reference's operator names with the reference's
schemas (CalcOps_bind.cpp:6-16; compared with the reference's own CPU operator library when
that was built from its sources here), and refuses host tensors (no CPU fallback)."""
import os

import pytest
import torch

from matpl_gb300 import build

SCHEMAS = {
    "calculateForce": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3, Tensor _4) -> Tensor[] _0",
    "calculateVirial": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3, Tensor _4) -> Tensor[] _0",
    "calculateCompress": "(Tensor _0, Tensor _1) -> Tensor[] _0",
    "calculateNepForce": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3) -> Tensor[] _0",
    "calculateNepVirial": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3, Tensor _4) -> Tensor[] _0",
    "calculate_maxneigh": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3, Tensor _4, float _5, "
                          "float _6, int _7, Tensor _8, bool _9) -> Tensor[] _0",
    "calculate_neighbor": "(Tensor _0, Tensor _1, Tensor _2, Tensor _3, Tensor _4, Tensor _5, "
                          "Tensor _6, float _7, float _8, int _9, int _10, bool _11) -> Tensor[] _0",
}


@pytest.fixture(scope="module")
def calcops():
    build.build()
    torch.ops.load_library(build.OPS_LIB)
    return torch.ops.CalcOps_cuda


def test_operator_library_registers_the_reference_schemas(calcops):
    for name, sig in SCHEMAS.items():
        assert str(getattr(calcops, name).default._schema) == f"CalcOps_cuda::{name}{sig}", name


def test_schemas_equal_the_reference_cpu_operator_library(calcops):
    from oracle import ref_build
    if not os.path.exists(ref_build.LIB):
        pytest.skip("the reference's CPU operator library is not built here")
    torch.ops.load_library(ref_build.LIB)
    ref = torch.ops.CalcOps_cpu
    for name in ("calculateForce", "calculateVirial", "calculateCompress", "calculate_maxneigh",
                 "calculate_neighbor"):
        ours = str(getattr(calcops, name).default._schema).split("::", 1)[1]
        theirs = str(getattr(ref, name).default._schema).split("::", 1)[1]
        assert ours == theirs, name


def test_host_tensors_are_refused(calcops):
    ln = torch.zeros(1, 4, 1, 8, dtype=torch.int32)
    with pytest.raises(RuntimeError, match="CUDA tensors expected"):
        calcops.calculateForce(ln, torch.zeros(1, 4, 1, 32), torch.zeros(1, 4, 32, 3),
                               torch.zeros(1, 4, 3), torch.tensor(0))
    with pytest.raises(RuntimeError, match="CUDA tensors expected"):
        calcops.calculateCompress(torch.zeros(5, 1), torch.zeros(5, 25, 6))
