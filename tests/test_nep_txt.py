"""``nep.gpumd_text`` (the nep5 potential file the LAMMPS / GPUMD evaluators read) against the
text MatPL's own converter (utils/nep_to_gpumd.py ``extract_model``) wrote for the same
parameters (tests/golden/nep_txt_*.txt, made by tests/golden/make_nep_txt_golden.py).

The header lines must agree token for token; every parameter line must parse to the same FP32
value (the reader converts each line with ``std::stof``, error.cu:167-179), so the two files
load into identical models."""
import os
import sys

import numpy as np
import pytest

from matpl_gb300 import nep as NP

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_nep_txt_golden as G  # noqa: E402


def _split(text):
    lines = [l for l in text.splitlines() if l.strip()]
    head = [l.split() for l in lines if not _is_number(l)]
    vals = np.array([float(l) for l in lines if _is_number(l)], dtype=np.float64)
    return head, vals.astype(np.float32)


def _is_number(line):
    try:
        float(line)
        return True
    except ValueError:
        return False


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_gpumd_text_matches_the_reference_converter(name):
    cfg, prm, mx = G.case_params(name)
    ours = NP.gpumd_text(cfg, prm, mx)
    ref = open(os.path.join(HERE, "golden", f"nep_txt_{name}.txt")).read()
    h1, v1 = _split(ours)
    h2, v2 = _split(ref)
    assert h1 == h2
    assert v1.shape == v2.shape
    assert np.array_equal(v1.view(np.uint32), v2.view(np.uint32))


def test_gpumd_text_line_count_is_what_the_reader_expects():
    """nep3.cu:327-335: version 5 reads ((dim + 2) * H + 1) * T + 1 network values, then the
    descriptor coefficients and dim q_scaler values."""
    cfg, prm, mx = G.case_params("hfo_l4")
    _, vals = _split(NP.gpumd_text(cfg, prm, mx))
    T, F, H = cfg.ntypes, cfg.feature_nums, cfg.neuron
    n_ann = ((F + 2) * H + 1) * T + 1
    n_c = T * T * (cfg.nr * cfg.kr + cfg.na * cfg.ka)
    assert vals.size == n_ann + n_c + F
