"""The many-body kernels take their repulsion quotients from the reciprocal of
the length (common.cuh: div_by_recip, Markstein's method).  This test builds
a small CUDA program against the same header and checks the result equals the
correctly rounded division (__fdiv_rn) bit for bit on 2^28 sampled pairs."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_markstein_quotient_equals_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "check_quotient")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-o", exe,
                    os.path.join(HERE, "cuda", "check_quotient.cu")], check=True)
    out = subprocess.run([exe, "16"], check=True, capture_output=True, text=True).stdout
    m = re.search(r"pairs=(\d+) mismatches=(\d+)", out)
    assert m and int(m.group(1)) == 1 << 28, out
    assert int(m.group(2)) == 0, out
