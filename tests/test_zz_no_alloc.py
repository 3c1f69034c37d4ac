"""The allocation-free norms entry point (bes_residual_norms_static) against the explicit
iteration's own logged norms.

Callers that cannot call cudaMalloc (a framework whose caching allocator owns the device
memory, or a loop where cudaMalloc would synchronise the device) use this entry point with
device buffers they already own; the library's scratch for it is a fixed device array.  The
test allocates its buffers with torch, which is the caller's business, not the library's.
This file is collected last on purpose.
"""
import numpy as np
import pytest

from bes_gb300 import lib, meshgen
from tests import _golden as G
from tests._gpu import context

pytestmark = pytest.mark.gpu


def _norms_static(torch, R_host):
    R = torch.tensor(np.ascontiguousarray(R_host), dtype=torch.float64, device="cuda")
    out = torch.full((10,), -1.0, dtype=torch.float64, device="cuda")
    lib.residual_norms_static(R.data_ptr(), R.shape[0], out.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_static_norms_match_explicit_iteration_norms_on_two_calls():
    torch = pytest.importorskip("torch")
    ref, info = G.load("explicit_bump_supersonic")
    mesh = G.mesh_of(info)
    # One stage with coefficient 0: the iteration logs the norms of R(W) at the current state
    # and leaves the state unchanged, so R(W) from bes_compute_operators is the same residual.
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8,
                  freestream_mach=tuple(info["meta"]["mach"]), stage_coeff=(0.0,))
    states = [ref["op_state"].reshape(-1, 5), None]  # a developed state, then freestream
    for st in states:
        if st is None:
            ctx.set_freestream_state()
        else:
            ctx.set_state(st)
        R = ctx.operators(0.8)["residual"]
        hist = ctx.explicit_iterations(1)[0]
        got = _norms_static(torch, R)
        scale = np.maximum(np.abs(hist), 1e-300)
        assert np.all(np.abs(got - hist) / scale <= 1e-12), (got, hist)


def test_static_norms_reject_oversized_input():
    torch = pytest.importorskip("torch")
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(lib.BesError) as e:
        lib.residual_norms_static(buf.data_ptr(), 4194305, buf.data_ptr(), 0)
    assert e.value.code == 1
    assert "4194304" in str(e.value)


@pytest.mark.parametrize("n_cells", [1000, 4194304])
def test_static_norms_match_numpy_at_odd_and_largest_sizes(n_cells):
    # 1000 cells is not a multiple of the 256-cell reduction block; 4,194,304 cells fill the
    # whole scratch array (16,384 blocks of partial sums).  Two calls in a row with different
    # data: the second must not see the first one's partials.
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n_cells)
    for scale in (1.0, 1e-3):
        R = rng.standard_normal((n_cells, 5)) * scale
        got = _norms_static(torch, R)
        l2 = np.sqrt((R * R).sum(axis=0))
        mx = np.abs(R).max(axis=0)
        want = np.concatenate([l2, mx])
        assert np.all(np.abs(got - want) <= 1e-12 * want), (got, want)
