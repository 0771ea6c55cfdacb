"""The one-cell and two-cell (packed f32x2) forms of the shifted-space
collision are bit-identical on 2^21 random cells per case (BGK and TRT;
D2Q9, D3Q19, D3Q27): compiled from tests/cuda/lane_identity.cu with nvcc."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_lane1_lane2_bit_identical(tmp_path, lgb):
    from lettuce_gb300 import build
    exe = tmp_path / "lane_identity"
    subprocess.run([build.nvcc_path()] + build.NVCC_FLAGS +
                   ["-o", str(exe), os.path.join(ROOT, "tests", "cuda", "lane_identity.cu")],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "total mismatches 0" in r.stdout
