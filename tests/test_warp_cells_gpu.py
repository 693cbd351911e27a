"""The warp-cell slot selection (warp_cells.cuh: 32-bit warp minimums, the
hash-threshold filter for cells above 128 points, and its fallback) against
the per-lane top-8 lists, on cells built to reach every path, with tied
hashes, for key offsets 0 and 12345 (the batched engine's per-job offset)."""
import os
import re
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_warp_cells_equal_lists(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "check_warp_cells")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-o", exe,
                    os.path.join(HERE, "cuda", "check_warp_cells.cu")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout
    rows = re.findall(r"koff=(\d+) cells=(\d+) ties=(\d+) fallbacks=(\d+) mismatches=(\d+)", out)
    assert [r[0] for r in rows] == ["0", "12345"], out
    for _, cells, ties, fallbacks, bad in rows:
        assert int(cells) == 16 and int(ties) == 33 and int(fallbacks) == 3, out
        assert int(bad) == 0, out
