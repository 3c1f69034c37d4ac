"""Batched freestream sweep (bes_create_batch / bes_sweep_run) against single-condition runs.

Every condition of a batch runs the same kernels on the same mesh as a context created for
that condition alone, so its state and residual history must agree bit for bit; the single
runs are themselves pinned to the oracle and the reference by the other GPU tests.
"""
import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen

pytestmark = pytest.mark.gpu

MACHS = [(0.5, 0.0, 0.0), (0.7, 0.05, 0.0), meshgen.freestream_mach_vector(0.6, 3.0, -2.0)]


def _opts(**kw):
    base = dict(solver_type=0, local_time_step=1, courant_num=0.8)
    base.update(kw)
    return lib.default_options(**base)


def _single(mesh, mach, n, **kw):
    ctx = lib.Context(mesh, _opts(freestream_mach=mach, **kw))
    h = ctx.explicit_iterations(n)
    U = ctx.get_state()
    f = ctx.wall_force()
    ctx.close()
    return h, U, f


@pytest.mark.parametrize("kw", [dict(), dict(local_time_step=0),
                                dict(freestream_ramp=6, freestream_ramp_start_frac=0.3)],
                         ids=["local_dt", "global_dt", "freestream_ramp"])
def test_batch_matches_single_condition_runs(kw):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    ctx = lib.Context(mesh, _opts(**kw), machs=MACHS)
    assert ctx.n_cond == 3
    h = ctx.explicit_iterations(15)
    U = ctx.get_state()
    F = ctx.wall_force()
    assert h.shape == (15, 3, 10) and U.shape == (3, ctx.n_cells, 5) and F.shape == (3, 3)
    for b, mach in enumerate(MACHS):
        hs, Us, fs = _single(mesh, mach, 15, **kw)
        assert np.array_equal(h[:, b], hs)
        assert np.array_equal(U[b], Us)
        assert np.array_equal(F[b], fs)
    ctx.close()


def test_frozen_condition_keeps_its_state():
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    ctx = lib.Context(mesh, _opts(), machs=MACHS)
    ctx.explicit_iterations(4)
    U4 = ctx.get_state()
    ctx.set_active([1, 0, 1])
    h = ctx.explicit_iterations(3)  # odd: the ping-pong buffers swap roles
    U7 = ctx.get_state()
    assert np.array_equal(U7[1], U4[1])
    assert np.all(h[:, 1] == 0.0)
    for b in (0, 2):
        hs, Us, _ = _single(mesh, MACHS[b], 7)
        assert np.array_equal(U7[b], Us)
        assert np.array_equal(h[:, b], hs[4:])
    # resumed: the frozen condition continues from its kept state
    ctx.set_active([1, 1, 1])
    ctx.explicit_iterations(2)
    hs, Us, _ = _single(mesh, MACHS[1], 6)
    assert np.array_equal(ctx.get_state()[1], Us)
    ctx.close()


def test_sweep_run_stops_each_condition_at_its_drop():
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    max_iter = 300
    # single runs first: a drop that every condition reaches within 200 iterations
    singles = []
    for mach in MACHS:
        hs, _, _ = _single(mesh, mach, max_iter)
        r = np.sqrt((hs[:, :5] ** 2).sum(axis=1))
        singles.append(r)
    drop = max(float(np.min(r[:200] / r[0])) for r in singles) * (1 + 1e-9)
    ctx = lib.Context(mesh, _opts(), machs=MACHS)
    iters, final = ctx.sweep_run(max_iter, drop=drop, check_every=1)
    U = ctx.get_state()
    for b, mach in enumerate(MACHS):
        r = singles[b]
        hit = np.nonzero(r <= drop * r[0])[0]
        assert hit.size and hit[0] < 200
        assert iters[b] == hit[0] + 1
        assert final[b] == pytest.approx(r[hit[0]] / r[0], rel=1e-12)
        _, Us, _ = _single(mesh, mach, int(iters[b]))
        assert np.array_equal(U[b], Us)  # frozen right after it converged
    ctx.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_implicit_batch_matches_single_condition_runs(precision):
    """Implicit batches step all conditions together (batched Krylov kernels, per-condition
    GMRES state on the device); every condition, with its own adaptive CFL, matches its own
    context bit for bit."""
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    kw = dict(solver_type=1, courant_num=10.0, adaptive_courant_num_max=500.0,
              linear_solver=1, linear_solver_tol=1e-2, linear_solver_max_iter=200,
              precision=precision)
    ctx = lib.Context(mesh, _opts(**kw), machs=MACHS)
    h = ctx.implicit_steps(6)
    U = ctx.get_state()
    assert h.shape == (6, 3, 19)
    for b, mach in enumerate(MACHS):
        single = lib.Context(mesh, _opts(freestream_mach=mach, **kw))
        hs = single.implicit_steps(6)
        assert np.array_equal(h[:, b], hs)
        assert np.array_equal(U[b], single.get_state())
        single.close()
    ctx.close()


def test_batch_rejects_what_it_does_not_run():
    nbuild.build()
    mesh = meshgen.bump_channel(6, 2, 2, 0.08)
    imp = lib.Context(mesh, _opts(solver_type=1, linear_solver=1), machs=MACHS)
    with pytest.raises(lib.BesError, match="BES_ERR_UNSUPPORTED"):
        imp.implicit_assemble(10.0)
    with pytest.raises(lib.BesError, match="BES_ERR_UNSUPPORTED"):
        imp.sweep_run(10)
    imp.close()
    ctx = lib.Context(mesh, _opts(), machs=MACHS[:2])
    with pytest.raises(lib.BesError, match="BES_ERR_UNSUPPORTED"):
        ctx.operators(0.8)
    ctx.close()
