"""The implicit step as one graph launch: GMRES driven on the device, batched conditions.

* One host synchronisation per implicit step, whatever the number of restart cycles: the
  Arnoldi steps, Givens rotations, restarts and the convergence test run inside the step
  graph's conditional nodes (bes_implicit_stats).
* The device loop over restart cycles has a guard: a solve stopped by the restart-cycle limit
  returns BES_ERR_TIMEOUT, its step is applied, and the context keeps working.
* Frozen conditions of an implicit batch keep their state; a refilled slot
  (bes_set_condition) gives bit for bit the run of a fresh context for its new condition.
"""
import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen

pytestmark = pytest.mark.gpu

MACHS = [(0.5, 0.0, 0.0), (0.7, 0.05, 0.0), meshgen.freestream_mach_vector(0.6, 3.0, -2.0)]
IMPLICIT = dict(solver_type=1, local_time_step=1, courant_num=10.0,
                adaptive_courant_num_max=500.0, linear_solver=1, linear_solver_tol=1e-2,
                linear_solver_max_iter=200)


def _opts(**kw):
    base = dict(IMPLICIT)
    base.update(kw)
    return lib.default_options(**base)


def _single(mesh, mach, n, **kw):
    ctx = lib.Context(mesh, _opts(freestream_mach=mach, **kw))
    h = ctx.implicit_steps(n)
    U = ctx.get_state()
    ctx.close()
    return h, U


@pytest.mark.parametrize("precision", [0, 2])
def test_one_host_sync_per_implicit_step(precision):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    # GMRES(4) to 1e-6: several restart cycles per step
    ctx = lib.Context(mesh, _opts(freestream_mach=MACHS[0], gmres_restart=4,
                                  linear_solver_tol=1e-6, precision=precision))
    h = ctx.implicit_steps(5)
    s = ctx.implicit_stats()
    ctx.close()
    assert s["steps"] == 5
    assert s["host_syncs"] == 5
    assert s["arnoldi_steps"] == int(h[:, 12].sum())
    assert s["restart_cycles"] >= int(np.ceil(h[:, 12] / 4).sum())
    assert np.all(h[:, 13] <= 1e-6)


def test_linear_guard_stops_a_solve_and_the_context_recovers():
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    kw = dict(freestream_mach=MACHS[1], gmres_restart=2, linear_solver_tol=1e-8,
              linear_solver_max_iter=400)
    ctx = lib.Context(mesh, _opts(**kw))
    ctx.set_linear_guard(1)
    with pytest.raises(lib.BesError) as e:
        ctx.implicit_steps(1)
    assert e.value.code == 7  # BES_ERR_TIMEOUT
    assert ctx.implicit_stats()["restart_cycles"] == 1
    U1 = ctx.get_state()
    assert np.all(np.isfinite(U1))
    ctx.set_linear_guard(0)
    h = ctx.implicit_steps(2)  # no limit but the iteration count: more than one cycle each
    assert np.all(h[:, 12] > 2)
    assert np.all(np.isfinite(ctx.get_state()))
    ctx.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_frozen_implicit_condition_keeps_its_state(precision):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    ctx = lib.Context(mesh, _opts(precision=precision), machs=MACHS)
    ctx.implicit_steps(3)
    U3 = ctx.get_state()
    ctx.set_active([1, 0, 1])
    h = ctx.implicit_steps(2)
    U5 = ctx.get_state()
    assert np.array_equal(U5[1], U3[1])
    assert np.all(h[:, 1] == 0.0)
    for b in (0, 2):
        hs, Us = _single(mesh, MACHS[b], 5, precision=precision)
        assert np.array_equal(U5[b], Us)
        assert np.array_equal(h[:, b], hs[3:])
    ctx.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_refilled_slot_matches_a_fresh_context(precision):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    new_mach = meshgen.freestream_mach_vector(0.45, -2.0, 1.0)
    ctx = lib.Context(mesh, _opts(precision=precision, cfl_ramp_steps=4, cfl_ramp_start=10.0,
                                  cfl_ramp_end=200.0), machs=MACHS)
    ctx.implicit_steps(3)
    ctx.set_condition(1, mach=new_mach)
    h = ctx.implicit_steps(4)
    U = ctx.get_state()
    kw = dict(precision=precision, cfl_ramp_steps=4, cfl_ramp_start=10.0, cfl_ramp_end=200.0)
    hs, Us = _single(mesh, new_mach, 4, **kw)
    assert np.array_equal(h[:, 1], hs)
    assert np.array_equal(U[1], Us)
    h0, U0 = _single(mesh, MACHS[0], 7, **kw)
    assert np.array_equal(U[0], U0)
    assert np.array_equal(h[:, 0], h0[3:])
    ctx.close()


def _single_to_drop(mesh, mach, drop, max_steps, **kw):
    ctx = lib.Context(mesh, _opts(freestream_mach=mach, **kw))
    r0 = None
    for k in range(max_steps):
        h = ctx.implicit_steps(1)[0]
        r = float(np.sqrt(np.sum(h[14:19] ** 2)))
        r0 = r if r0 is None else r0
        if r <= drop * r0:
            break
    out = (k + 1, r / r0, ctx.get_state(), ctx.wall_force())
    ctx.close()
    return out


@pytest.mark.parametrize("precision", [0, 2])
def test_sweep_queue_through_slots_matches_single_solves(precision):
    """Five conditions through two slots (bes_implicit_sweep): each gives the steps, final
    residual, state and wall force of its own single-condition solve, bit for bit.  On this
    4 % bump the oracle's FP64 solve reaches a 1e-6 drop in about 65 steps at Mach 0.45, 0.5,
    0.6 and 0.65 and stalls near 1e-3 at Mach 0.55, which ends at the step limit."""
    nbuild.build()
    mesh = meshgen.bump_channel(24, 8, 6, 0.04)
    machs = np.array([(m, 0.0, 0.0) for m in (0.5, 0.55, 0.45, 0.6, 0.65)])
    kw = dict(precision=precision, cfl_ramp_steps=10, cfl_ramp_start=10.0, cfl_ramp_end=1000.0)
    ctx = lib.Context(mesh, _opts(**kw), machs=machs[:2])
    out = ctx.implicit_sweep(machs, drop=1e-6, max_steps=100, states=True)
    ctx.close()
    assert out["steps"][1] == 100 and out["final_res"][1] > 1e-6
    for q, m in enumerate(machs):
        steps, fin, U, F = _single_to_drop(mesh, m, 1e-6, 100, **kw)
        assert out["steps"][q] == steps
        if q != 1:
            assert steps < 100 and fin <= 1e-6
        assert out["final_res"][q] == pytest.approx(fin, rel=1e-14)
        assert np.array_equal(out["U"][q], U)
        assert np.array_equal(out["force"][q], F)
        assert out["seconds"][q] > 0


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_colour_sweep_forms_give_identical_steps(precision):
    """SWEEP_KERNEL 2 (one persistent launch per sweep, grid barrier between colours) and 3
    (one launch per colour, every load of a row issued first; the 16-bit storage) compute each
    row exactly as the per-colour launches (SWEEP_KERNEL 1): identical steps, single and
    batched."""
    nbuild.build()
    mesh = meshgen.bump_channel(24, 8, 6, 0.08)
    runs = {}
    for kern in (1, 2, 3):
        one = lib.Context(mesh, _opts(freestream_mach=MACHS[0], precision=precision,
                                      sweep_kernel=kern))
        bat = lib.Context(mesh, _opts(precision=precision, sweep_kernel=kern), machs=MACHS)
        runs[kern] = (one.implicit_steps(4), one.get_state(), bat.implicit_steps(3),
                      bat.get_state(), one.tuning())
        one.close()
        bat.close()
    for kern in (2, 3):
        rep = runs[kern][4]
        assert "fixed by the options" in rep
        if kern == 2 and (rep.startswith("colour sweep: one launch")
                          or "could not be captured" in rep):
            continue  # the persistent sweep is not available on this device
        if kern == 3:
            assert ("loads first" in rep) == (precision == 2)
        for a, b in zip(runs[1][:4], runs[kern][:4]):
            assert np.array_equal(a, b)


def test_autotuner_reports_its_choice():
    nbuild.build()
    mesh = meshgen.bump_channel(24, 8, 6, 0.08)
    ctx = lib.Context(mesh, _opts(freestream_mach=MACHS[0], precision=2))
    assert ctx.tuning() == ""
    ctx.implicit_steps(1)
    rep = ctx.tuning()
    ctx.close()
    assert rep.startswith("colour sweep:") and "one launch per colour" in rep and "taken:" in rep
