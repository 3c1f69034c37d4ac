"""GPU parity of the explicit residual/update path (through the C ABI) against the oracle
(which is itself pinned to the reference) and against the reference's own golden data.

Tolerances (floating point, FP64 on both sides; the GPU contracts multiply-adds and uses
reciprocals where the reference divides):
  operators (dt, gradient, limiter, face states, fluxes): 1e-12 relative to the array's scale;
  per-iteration residual L2 / max over the first 50 iterations: 1e-10 relative (the parity
  bar of this path), final state 1e-10.
"""
import numpy as np
import pytest

from bes_gb300 import lib, meshgen
from oracle import pyoracle
from tests import _golden as G
from tests._gpu import context, explicit_opts, hist_rel_err, rel_err

pytestmark = pytest.mark.gpu

EXPLICIT = [c for c in G.CASES if c.startswith("explicit")]


@pytest.mark.parametrize("case", EXPLICIT)
def test_operators_match_oracle(case):
    ref, info = G.load(case)
    if "op_state" not in ref:
        pytest.skip("no operator dump")
    mesh = G.mesh_of(info)
    ctx = context(mesh, **explicit_opts(info))
    ctx.set_state(ref["op_state"])
    got = ctx.operators(info["meta"]["cfl"])
    O = pyoracle.Oracle(mesh, **G.oracle_kwargs(info))
    O.set_state(ref["op_state"])
    exp = O.operators(info["meta"]["cfl"])
    for k in ("dt", "grad", "limiter", "face_UL", "face_UR", "face_flux", "residual"):
        assert rel_err(got[k], exp[k]) <= 1e-12, k
    # and against the reference's own dump
    assert rel_err(got["grad"], ref["op_grad"]) <= 1e-12
    assert rel_err(got["face_flux"], ref["op_face_flux"]) <= 1e-12


@pytest.mark.parametrize("case", EXPLICIT + G.CASES_2D)
def test_residual_history_matches_reference(case):
    ref, info = G.load(case)
    mesh = G.mesh_of(info)
    ctx = context(mesh, **explicit_opts(info))
    n = info["steps"]
    h = ctx.explicit_iterations(n)
    refh = ref["residual_history"].reshape(-1, 10)
    assert hist_rel_err(h[:, :5], refh[:, :5]) <= 1e-10  # L2 per variable
    assert hist_rel_err(h[:, 5:], refh[:, 5:]) <= 1e-10  # max norm (the reference's log)
    assert rel_err(ctx.get_state(), ref["final_state"]) <= 1e-10


def test_config1_mesh_first_50_iterations_match_oracle():
    """72,000-tet bump channel (M 0.5, local dt, CFL 0.8): the first 50 iterations."""
    mesh = meshgen.bump_channel(60, 20, 10, 0.04)
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8,
                  freestream_mach=(0.5, 0.0, 0.0))
    h = ctx.explicit_iterations(50)
    O = pyoracle.Oracle(mesh, cfl=0.8, mach=(0.5, 0, 0), threads=16)
    ho = O.explicit_run(50)
    assert hist_rel_err(h, ho) <= 1e-10
    assert rel_err(ctx.get_state(), O.get_state()) <= 1e-10


def test_exact_face_vector_mode_matches_oracle():
    mesh = meshgen.gaussian_box(8, 4, 8)
    mach = meshgen.freestream_mach_vector(0.6, 2.0, 1.0)
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8, freestream_mach=mach,
                  muscl_face_vector=1)
    h = ctx.explicit_iterations(20)
    O = pyoracle.Oracle(mesh, cfl=0.8, mach=mach, muscl_exact=1)
    ho = O.explicit_run(20)
    assert hist_rel_err(h, ho) <= 1e-10


def test_flux_kat_matches_reference():
    for name in ("kat_subsonic", "kat_supersonic"):
        z = np.load(G.GOLDEN + f"/{name}.npz")
        inp, out, mach = z["inputs"], z["outputs"], tuple(z["mach"])
        ctx = context(meshgen.bump_channel(4, 2, 2, 0.04), freestream_mach=mach)
        UL, UR, nh = inp[:, 0:5], inp[:, 5:10], inp[:, 10:13]
        F, JL, JR = ctx.flux_batch(0, UL, UR, nh, jacobians=True)
        assert rel_err(F, out[:, 0:5]) <= 1e-13
        assert rel_err(JL.reshape(-1, 25), out[:, 5:30]) <= 1e-12
        assert rel_err(JR.reshape(-1, 25), out[:, 30:55]) <= 1e-12
        F, JL, _ = ctx.flux_batch(1, UL, UR, nh, jacobians=True)
        assert rel_err(F, out[:, 55:60]) <= 1e-13
        assert rel_err(JL.reshape(-1, 25), out[:, 60:85]) <= 1e-12
        F, JL, _ = ctx.flux_batch(2, UL, UR, nh, jacobians=True)
        assert rel_err(F, out[:, 85:90]) <= 1e-13
        assert rel_err(JL.reshape(-1, 25), out[:, 90:115]) <= 1e-12


def test_nan_flux_is_reported_not_fatal():
    mesh = meshgen.bump_channel(6, 2, 2, 0.04)
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8)
    U = ctx.get_state()
    U[5, 0] = np.nan
    ctx.set_state(U)
    with pytest.raises(lib.BesError) as e:
        ctx.explicit_iterations(1)
    assert e.value.code == 3
    assert "NaN" in str(e.value)
    # the context stays usable
    ctx.set_freestream_state()
    ctx.explicit_iterations(2)


def test_reset_and_repeat_is_deterministic():
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8,
                  freestream_mach=(0.7, 0, 0))
    h1 = ctx.explicit_iterations(10)
    U1 = ctx.get_state()
    ctx.set_freestream_state()
    h2 = ctx.explicit_iterations(10)
    assert np.array_equal(h1, h2)
    assert np.array_equal(U1, ctx.get_state())
