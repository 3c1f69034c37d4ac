"""Floating-point operations per face of the three fluxes, counted by instantiating the GPU's
flux templates (bes_gb300/csrc/physics.cuh) on the host with a counting scalar
(tests/opcount/flux_opcount.cpp).  The counts are the per-unit FLOPs of the explicit path's
roofline; the test keeps them in step with the code."""
import json
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

EXPECTED = {
    "roe": dict(add=72, mul=109, div=4, sqrt=3, abs=4, cmp=3),
    "roe_harten_one_wave": dict(add=73, mul=113, div=5, sqrt=3, abs=4, cmp=5),
    "slip_wall": dict(add=3, mul=9, div=1, sqrt=0, abs=0, cmp=0),
    "freestream_subsonic_in": dict(add=26, mul=49, div=4, sqrt=1, abs=1, cmp=2),
    "freestream_subsonic_out": dict(add=19, mul=44, div=4, sqrt=1, abs=1, cmp=2),
    "freestream_supersonic_in": dict(add=13, mul=35, div=1, sqrt=1, abs=1, cmp=2),
    "freestream_supersonic_out": dict(add=13, mul=35, div=1, sqrt=1, abs=1, cmp=2),
}


def test_flux_operation_counts(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "opcount")
    subprocess.run(["g++", "-std=c++17", "-O0", os.path.join(HERE, "opcount", "flux_opcount.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.strip().splitlines():
        d = json.loads(line)
        got[d.pop("flux")] = d
    assert got == EXPECTED
