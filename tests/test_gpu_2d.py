"""Triangle meshes (the reference's 2-D path) on the GPU.

The explicit path is pinned to the reference's own 2-D run in test_gpu_explicit.py (residual
history and final state within 1e-10) and here against the oracle with a global time step.
The implicit path on triangles is checked against the oracle's restatement (the same
five-variable formulation with zero spanwise momentum, given the GPU's block-ILU(0) order),
which the reference's own 2-D implicit run pins (tests/test_oracle_golden.py; each Jacobian
block added four times in 2-D, the default), and through properties: it converges to the
steady state of the explicit path (the same discrete residual R(U) = 0), the FP32 system
tracks the FP64 one, and the spanwise momentum stays zero.

Tolerances: explicit 1e-10 (as the 3-D path); implicit steps against the oracle 1e-9 with equal
linear-iteration counts (as the 3-D path); steady states of the two solvers 1e-7 relative to
the state's scale (both driven to a residual drop of 1e-11); FP32 defect correction against
FP64 after 15 steps 1e-3.
"""
import numpy as np
import pytest

from bes_gb300 import meshgen
from oracle import pyoracle
from tests._gpu import context, hist_rel_err, rel_err

pytestmark = pytest.mark.gpu

MACH = (0.5, 0.03, 0.0)


def _implicit(mesh, **extra):
    kw = dict(solver_type=1, local_time_step=1, courant_num=10.0, freestream_mach=MACH,
              linear_solver=1, linear_solver_tol=1e-2, linear_solver_max_iter=300,
              gmres_restart=30, cfl_ramp_steps=10, cfl_ramp_start=10.0, cfl_ramp_end=1000.0)
    kw.update(extra)
    return context(mesh, **kw)


def test_2d_implicit_reaches_the_explicit_steady_state():
    """A shallow bump at Mach 0.4, where the reference's own explicit run drives its residual
    down by 1e-13 in 8000 iterations (a 5 % bump at Mach 0.5 stalls near 0.2 in the reference
    and here alike: the limiter's steady state is not reached)."""
    mesh = meshgen.bump_channel_2d(24, 8, 0.02)
    mach = (0.4, 0.0, 0.0)
    imp = _implicit(mesh, freestream_mach=mach)
    # L2 of the unscaled residual R (implicit columns 14-18, explicit 0-4); the implicit
    # solve falls by about 0.86 per step once the CFL ramp is done
    h_imp = imp.implicit_steps(50)
    while h_imp[-1, 14:19].max() > 1e-11 * h_imp[0, 14:19].max() and len(h_imp) < 400:
        h_imp = np.concatenate([h_imp, imp.implicit_steps(50)])
    exp = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8, freestream_mach=mach)
    h_exp = np.concatenate([exp.explicit_iterations(2000) for _ in range(4)])
    drop_imp = h_imp[-1, 14:19].max() / h_imp[0, 14:19].max()
    drop_exp = h_exp[-1, :5].max() / h_exp[0, :5].max()
    assert drop_imp <= 1e-11 and drop_exp <= 1e-11, (len(h_imp), drop_imp, drop_exp)
    u_imp, u_exp = imp.get_state(), exp.get_state()
    assert rel_err(u_imp, u_exp) <= 1e-7
    # no spanwise momentum on a 2-D mesh, and no residual for it
    assert np.abs(u_imp[:, 3]).max() <= 1e-13 and np.abs(u_exp[:, 3]).max() <= 1e-13
    assert h_imp[:, 17].max() <= 1e-13 * h_imp[0, 14:19].max()
    assert h_exp[:, 3].max() <= 1e-13 * h_exp[0, :5].max()


@pytest.mark.parametrize("precond", [0, 1])
def test_2d_fp32_defect_correction_tracks_fp64(precond):
    mesh = meshgen.bump_channel_2d(48, 16, 0.08)
    c64 = _implicit(mesh, linear_solver=precond)
    c32 = _implicit(mesh, linear_solver=precond, precision=1)
    h64 = c64.implicit_steps(15)
    h32 = c32.implicit_steps(15)
    assert rel_err(c32.get_state(), c64.get_state()) <= 1e-3
    assert np.max(np.abs(np.log(h32[:, [0, 1, 2, 4]] / h64[:, [0, 1, 2, 4]]))) <= 0.05
    assert np.abs(c32.get_state()[:, 3]).max() <= 1e-13


def test_2d_explicit_global_dt_matches_oracle():
    mesh = meshgen.bump_channel_2d(24, 8, 0.05)
    ctx = context(mesh, solver_type=0, local_time_step=0, courant_num=0.8, freestream_mach=MACH)
    h = ctx.explicit_iterations(50)
    O = pyoracle.Oracle(mesh, local_dt=0, cfl=0.8, mach=MACH)
    ho = O.explicit_run(50)
    assert hist_rel_err(h, ho) <= 1e-10
    assert rel_err(ctx.get_state(), O.get_state()) <= 1e-10


def test_2d_implicit_steps_match_oracle():
    mesh = meshgen.bump_channel_2d(24, 8, 0.05)
    ctx = _implicit(mesh, cfl_ramp_steps=8, cfl_ramp_end=500.0)
    h = ctx.implicit_steps(10)
    O = pyoracle.Oracle(mesh, solver=1, local_dt=1, cfl=10.0, mach=MACH, lin_precond=1,
                        lin_tol=1e-2, lin_maxiter=300, lin_restart=30, ramp_steps=8,
                        ramp_cfl0=10.0, ramp_cfl1=500.0)
    O.set_ilu_order(ctx.ilu_order())
    ho = O.implicit_run(10)
    assert np.array_equal(h[:, 12], ho[:, 12])
    assert hist_rel_err(h[:, :12], ho[:, :12]) <= 1e-9
    assert rel_err(ctx.get_state(), O.get_state()) <= 1e-9
