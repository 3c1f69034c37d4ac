"""Loading of the golden fixtures (produced by tests/golden/make_golden.py from the reference)."""
import ast
import os

import numpy as np

from bes_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

MESHES = {
    "bump_channel_12x4x4_h0.04": lambda: meshgen.bump_channel(12, 4, 4, 0.04),
    "bump_channel_12x4x4_h0.08": lambda: meshgen.bump_channel(12, 4, 4, 0.08),
    "gaussian_box_8x4x8_r1.05": lambda: meshgen.gaussian_box(8, 4, 8),
    "bump_channel_2d_24x8_h0.08": lambda: meshgen.bump_channel_2d(24, 8, 0.08),
    "bump_channel_24x8x6_h0.04": lambda: meshgen.bump_channel(24, 8, 6, 0.04),
}

CASES = ["explicit_bump_local", "explicit_bump_global", "explicit_gauss_pitch",
         "explicit_bump_supersonic", "explicit_bump_ramp", "implicit_bump_jacobi",
         "implicit_bump_ilu0"]

# triangle meshes (the reference's 2-D path); the fixtures pad per-cell data to the 3-D
# layout: five conserved variables (rho w = 0) and four face slots (the fourth -1)
CASES_2D = ["explicit_bump2d_local"]
# the reference's 2-D implicit runs (their 4x4-block systems solved through the linear-solver
# facade as 5x5 blocks with a decoupled spanwise-momentum row)
CASES_2D_IMPLICIT = ["implicit_bump2d_ilu0", "implicit_bump2d_jacobi_global"]
# implicit histories only (no operator dumps): the oracle against the reference's own steps
CASES_IMPLICIT_HISTORY = ["implicit_bump_global", "implicit_gauss_pitch", "implicit_bump_ramp"]
# the rest of the option surface (stage coefficients, limiter and Harten constants, gas
# constants, adaptive-CFL exponents), histories only
CASES_OPTIONS = ["explicit_bump_options", "implicit_bump_options"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    data = {k: z[k] for k in z.files}
    info = ast.literal_eval(str(data.pop("meta")))
    return data, info


def mesh_of(info):
    return MESHES[info["mesh"]]()


def oracle_kwargs(info):
    m = info["meta"]
    kw = dict(solver=0 if m["solver"] == "EXPLICIT" else 1,
              local_dt=1 if m["local"] == "YES" else 0, cfl=m["cfl"], mach=tuple(m["mach"]),
              fs_ramp=m.get("fs_ramp", 0), fs_frac=m.get("fs_frac", 0.5))
    if m["solver"] == "IMPLICIT":
        kw.update(cfl_max=m["cfl_max"], cfl_exp=tuple(m.get("cfl_exp", (1.0, 1.0))),
                  lin_precond=1 if m["smoother"] == "ILU0" else 0, lin_tol=m["lin_tol"],
                  lin_maxiter=m["lin_maxiter"], lin_restart=30)
    kw.update(m.get("oracle", {}))  # the option-surface cases' other keys
    return kw
