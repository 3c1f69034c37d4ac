"""Converged-state parity: the GPU solvers driven to a 1e-10 residual drop against the oracle
driven to the same drop, and the oracle's slip-wall force against bes_wall_force.

The reference logs no force coefficients; they are defined as the slip-wall CSV does
(src/SolutionSnapshot.cpp:268-309): the owner cell's pressure times the dimensional face
normal, summed over the slip-wall faces, over the dynamic pressure 1/2 rho |M|^2 with rho = 1
and a reference area of 1.  Tolerances (the converged-state gate): states 1e-8 relative
(max norm over all cells and variables), force coefficients 1e-8 absolute.

Also here: the implicit path with a freestream ramp (FREESTREAM_RAMP, src/Config.cpp:688-706)
step by step against the oracle, and the first implicit steps on the full 200x60x30-hex
channel (2.16M cells) against the oracle.
"""
import os

import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen
from oracle import pyoracle
from tests._gpu import hist_rel_err, rel_err

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
# a 4 % bump at Mach 0.5: the oracle's FP64 implicit solve falls by 6e-14 in about 80 steps
MESH = (24, 8, 6, 0.04)
MACH = (0.5, 0.0, 0.0)
IMPLICIT = dict(solver_type=1, local_time_step=1, courant_num=10.0, freestream_mach=MACH,
                linear_solver=1, linear_solver_tol=1e-2, linear_solver_max_iter=300,
                gmres_restart=30, cfl_ramp_steps=10, cfl_ramp_start=10.0, cfl_ramp_end=1000.0)
DROP = 1e-10


def _oracle(mesh, order, **kw):
    base = dict(solver=1, local_dt=1, cfl=10.0, mach=MACH, lin_precond=1, lin_tol=1e-2,
                lin_maxiter=300, lin_restart=30, ramp_steps=10, ramp_cfl0=10.0,
                ramp_cfl1=1000.0, threads=THREADS)
    base.update(kw)
    O = pyoracle.Oracle(mesh, **base)
    if order is not None:
        O.set_ilu_order(order)
    return O


def _residual(h):
    return float(np.sqrt(np.sum(np.asarray(h)[14:19] ** 2)))


def _oracle_force(O, U):
    """sum over slip-wall faces of p(owner) S, from the oracle's geometry and a state."""
    g = O.geometry()
    wall = g["face_type"] == 1
    u = U[g["face_owner"][wall]]
    p = 0.4 * (u[:, 4] - 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2 + u[:, 3] ** 2) / u[:, 0])
    return (p[:, None] * g["face_S"][wall]).sum(axis=0)


def _coefficients(F, mach):
    return np.asarray(F) / (0.5 * float(np.sum(np.asarray(mach) ** 2)))


@pytest.fixture(scope="module")
def converged_oracle():
    nbuild.build()
    mesh = meshgen.bump_channel(*MESH)
    ctx = lib.Context(mesh, lib.default_options(**dict(IMPLICIT, precision=0)))
    order = ctx.ilu_order()
    ctx.close()
    O = _oracle(mesh, order)
    r0 = None
    for _ in range(40):
        h = O.implicit_run(5)
        r0 = _residual(h[0]) if r0 is None else r0
        if _residual(h[-1]) <= DROP * r0:
            break
    assert _residual(h[-1]) <= DROP * r0
    U = O.get_state()
    return mesh, U, _oracle_force(O, U)


@pytest.mark.parametrize("precision", [0, 2])
def test_implicit_converged_state_and_force_match_oracle(converged_oracle, precision):
    """The FP64 system, and the defect correction with 16-bit storage (its fixed point is the
    FP64 residual's), solved to the same drop as the oracle."""
    mesh, Uo, Fo = converged_oracle
    ctx = lib.Context(mesh, lib.default_options(**dict(IMPLICIT, precision=precision)))
    r0 = None
    for _ in range(300):
        h = ctx.implicit_steps(1)[0]
        r0 = _residual(h) if r0 is None else r0
        if _residual(h) <= DROP * r0:
            break
    assert _residual(h) <= DROP * r0
    U = ctx.get_state()
    F = ctx.wall_force()
    ctx.close()
    assert rel_err(U, Uo) <= 1e-8
    assert np.abs(_coefficients(F, MACH) - _coefficients(Fo, MACH)).max() <= 1e-8


def test_wall_force_is_the_reference_definition(converged_oracle):
    """bes_wall_force on the oracle's converged state equals the force summed from the
    oracle's own geometry."""
    mesh, Uo, Fo = converged_oracle
    ctx = lib.Context(mesh, lib.default_options(**dict(IMPLICIT, precision=0)))
    ctx.set_state(Uo)
    F = ctx.wall_force()
    ctx.close()
    assert np.abs(F - Fo).max() <= 1e-12 * np.abs(Fo).max()


def test_explicit_converged_state_matches_the_oracle_steady_state(converged_oracle):
    """The explicit multi-step solver has the same fixed point, R(W) = 0: driven to a 1e-10
    drop from the freestream it reaches the oracle's converged state."""
    mesh, Uo, Fo = converged_oracle
    ctx = lib.Context(mesh, lib.default_options(solver_type=0, local_time_step=1,
                                                courant_num=0.8, freestream_mach=MACH))
    r0 = None
    done = False
    for _ in range(200):
        h = ctx.explicit_iterations(500)
        r = np.sqrt((h[:, :5] ** 2).sum(axis=1))
        r0 = r[0] if r0 is None else r0
        if r[-1] <= DROP * r0:
            done = True
            break
    assert done, r[-1] / r0
    U = ctx.get_state()
    F = ctx.wall_force()
    ctx.close()
    assert rel_err(U, Uo) <= 1e-8
    assert np.abs(_coefficients(F, MACH) - _coefficients(Fo, MACH)).max() <= 1e-8


def test_implicit_freestream_ramp_matches_oracle():
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    kw = dict(IMPLICIT, freestream_mach=(0.7, 0.0, 0.0), freestream_ramp=6,
              freestream_ramp_start_frac=0.3, precision=0)
    ctx = lib.Context(mesh, lib.default_options(**kw))
    h = ctx.implicit_steps(10)
    O = _oracle(mesh, ctx.ilu_order(), mach=(0.7, 0.0, 0.0), fs_ramp=6, fs_frac=0.3)
    ho = O.implicit_run(10)
    assert hist_rel_err(h[:, :12], ho[:, :12]) <= 1e-9
    assert np.array_equal(h[:, 12], ho[:, 12])
    assert rel_err(ctx.get_state(), O.get_state()) <= 1e-9
    ctx.close()


def test_full_channel_first_implicit_steps_match_oracle():
    """The benchmark's 200x60x30-hex channel (2.16M cells, Mach 0.84, bump 0.08): the first two
    FP64 implicit steps against the oracle given the GPU's factorisation order."""
    nbuild.build()
    mesh = meshgen.bump_channel(200, 60, 30, 0.08)
    kw = dict(IMPLICIT, freestream_mach=(0.84, 0.0, 0.0), cfl_ramp_steps=50, precision=0)
    ctx = lib.Context(mesh, lib.default_options(**kw))
    h = ctx.implicit_steps(2)
    U = ctx.get_state()
    order = ctx.ilu_order()
    ctx.close()
    O = _oracle(mesh, order, mach=(0.84, 0.0, 0.0), ramp_steps=50)
    ho = O.implicit_run(2)
    assert hist_rel_err(h[:, :12], ho[:, :12]) <= 1e-9
    assert np.array_equal(h[:, 12], ho[:, 12])
    assert rel_err(U, O.get_state()) <= 1e-9
