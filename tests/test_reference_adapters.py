"""The reference-side adapters (bes_gb300/adapters): the reference's own Config, Mesh and Gas
with bes_gb300 behind its operator and solver classes.

Needs the reference checkout (environment variable BES_REFERENCE_DIR): the adapters compile
against its headers and link with its sources.  Without a GPU bes_driver builds the
reference's objects from the .besi file and stops, with the reference's error convention,
where the library reports that no CUDA device is present; with one, --operators compares the
GPU adapters with the reference's GradientGreenGauss, LimiterVenkatakrishnan and
TimeStepCalculatorLocal on the same snapshot.
"""
import os
import subprocess

import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("BES_REFERENCE_DIR", "")
DRIVER = os.path.join(ROOT, "oracle", "_ref", "bes_driver")

pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "src"))),
                                reason="BES_REFERENCE_DIR does not name the reference checkout")


def _case(tmp_path):
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    msh = str(tmp_path / "bump.msh")
    meshgen.write_gmsh(mesh, msh)
    besi = tmp_path / "case.besi"
    besi.write_text("\n".join([
        "MESH_FORMAT = GMSH", f"MESH_FILE = {msh}", f"OUTPUT_FOLDER = {tmp_path}",
        "SOLVER_TYPE = EXPLICIT", "LOCAL_TIME_STEP = YES", "COURANT_NUM = 0.8",
        "NUMBER_OF_TIME_STEP = 5", "SAVE_INTERVAL = 100000", "FREESTREAM_MACH = 0.5, 0.0, 0.0",
    ]) + "\n")
    return mesh, str(besi)


def _build():
    nbuild.build()
    subprocess.run(["make", "-C", os.path.join(ROOT, "bes_gb300", "adapters"), f"REF={REF}"],
                   check=True, capture_output=True)
    assert os.path.exists(DRIVER)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_driver_builds_the_reference_objects_and_reaches_the_library(tmp_path):
    _build()
    mesh, besi = _case(tmp_path)
    out = subprocess.run([DRIVER, besi], capture_output=True, text=True, timeout=300)
    assert f"reference objects built: {mesh.n_cells} cells" in out.stdout
    if _has_gpu():
        assert out.returncode == 0, out.stdout[-2000:]
        assert os.path.exists(os.path.join(os.path.dirname(besi), "residual.csv"))
    else:
        # no CUDA device: bes_create reports BES_ERR_CUDA, the adapter exits as the reference
        # does on errors
        assert out.returncode != 0
        assert "ERROR: bes_create returned 2" in out.stdout


@pytest.mark.gpu
def test_operator_adapters_match_the_reference_operators(tmp_path):
    _build()
    _, besi = _case(tmp_path)
    out = subprocess.run([DRIVER, "--operators", besi], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout[-2000:]
    line = [l for l in out.stdout.splitlines() if l.startswith("gradient max rel diff")][0]
    vals = [float(x.strip().split()[-1]) for x in line.split(",")]
    assert vals[0] <= 1e-12 and vals[1] <= 1e-12 and vals[2] <= 1e-12, line
