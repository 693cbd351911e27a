"""The many-body kernels take their repulsion quotients from the reciprocal of
the length (common.cuh: div_by_recip, Markstein's method), and the length and
its reciprocal from hardware approximations with one FMA correction each
(sqrt_in_range, recip_in_range).  These tests build small CUDA programs
against the same header and check the results equal the correctly rounded
operations bit for bit: the division on 2^28 sampled pairs, the square root
and the reciprocal on every float of their ranges."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _build(tmp_path, name):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / name)
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-o", exe,
                    os.path.join(HERE, "cuda", name + ".cu")], check=True)
    return exe


def test_markstein_quotient_equals_division(tmp_path):
    exe = _build(tmp_path, "check_quotient")
    out = subprocess.run([exe, "16"], check=True, capture_output=True, text=True).stdout
    m = re.search(r"pairs=(\d+) mismatches=(\d+) spring=(\d+)/(\d+)", out)
    # spring operands: about 26/34 of the lengths lie in [1, 2^26]
    assert m and int(m.group(1)) == 1 << 28 and int(m.group(3)) > 1 << 27, out
    assert int(m.group(2)) == 0 and int(m.group(4)) == 0, out


def test_in_range_sqrt_and_recip_equal_correctly_rounded(tmp_path):
    exe = _build(tmp_path, "check_sqrt_recip")
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.search(r"sqrt=(\d+)/(\d+) recip=(\d+)/(\d+)", out)
    assert m, out
    assert int(m.group(1)) == (52 << 23) + 1 and int(m.group(3)) == (26 << 23) + 1, out
    assert int(m.group(2)) == 0 and int(m.group(4)) == 0, out
