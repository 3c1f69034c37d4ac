"""The learned warm start (bes_mlp_*) on the GPU.

* forward, loss and gradient of one batch against the FP64 restatement
  (oracle/mlp_oracle.py) with the same bfloat16 rounding of the GEMM operands: the remaining
  differences are FP32 accumulation order, so the tolerance is 2e-3 (relative L2 per
  parameter block);
* one AdamW step against the restatement (1e-5 relative);
* trained on solutions of a sweep, the network's prediction for held-out conditions is closer
  to their converged state than the freestream is, and the solver started from it reaches the
  same residual in fewer iterations than from the freestream.
"""
import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _ctx(mesh, machs=None, **kw):
    nbuild.build()
    o = dict(solver_type=0, local_time_step=1, courant_num=0.8, freestream_mach=(0.5, 0, 0))
    o.update(kw)
    return lib.Context(mesh, lib.default_options(**o), machs=machs)


def _blocks(v):
    out, off = {}, 0
    for name, shape in M.layout():
        n = int(np.prod(shape))
        out[name] = v[off:off + n]
        off += n
    return out


@pytest.mark.parametrize("B", [256, 1024])
def test_gradient_matches_oracle(B):
    """B = 1024 also takes the split-K path of the weight-gradient GEMM (two partials of 512
    rows reduced in a fixed order)."""
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    ctx = _ctx(mesh)
    net = lib.WarmStart(ctx, seed=3)
    rng = np.random.default_rng(1)
    p = net.params().astype(np.float64)
    blocks = _blocks(p)
    for l in range(4):  # a FiLM that is not the identity, and nonzero biases
        blocks[f"F{l}"][:] = rng.normal(size=blocks[f"F{l}"].size) * 0.2
        blocks[f"g{l}"][:] = rng.normal(size=blocks[f"g{l}"].size) * 0.1
        blocks[f"b{l}"][:] = rng.normal(size=blocks[f"b{l}"].size) * 0.05
    p = np.concatenate([blocks[n] for n, _ in M.layout()]).astype(np.float32)
    net.set_params(p)
    cells = rng.integers(0, ctx.n_cells, B)
    cond = rng.normal(size=(B, 3))
    tgt = rng.normal(size=(B, 5)) * 0.5
    loss, g, out = net.loss_grad(cells, cond, tgt)
    X = M.encode(net.features().astype(np.float64)[cells])
    lo, go, oo = M.loss_and_grad(p.astype(np.float64), X, cond, tgt, rounded=True)
    assert loss == pytest.approx(lo, rel=2e-3)
    assert np.abs(out - oo).max() <= 2e-3 * np.abs(oo).max()
    gb, gob = _blocks(g.astype(np.float64)), _blocks(go)
    for name, _ in M.layout():
        err = np.linalg.norm(gb[name] - gob[name]) / max(np.linalg.norm(gob[name]), 1e-30)
        assert err <= 2e-3, (name, err)
    net.close()
    ctx.close()


def test_adamw_step_matches_oracle():
    mesh = meshgen.bump_channel(6, 2, 2, 0.08)
    ctx = _ctx(mesh)
    net = lib.WarmStart(ctx, seed=5)
    p0 = net.params().astype(np.float64)
    rng = np.random.default_rng(2)
    g = (rng.normal(size=p0.size) * 1e-2).astype(np.float32)
    net.apply_grad(g, lr=1e-3, weight_decay=1e-2)
    p1 = net.params().astype(np.float64)
    ref, _, _ = M.adamw_step(p0, g.astype(np.float64), np.zeros_like(p0), np.zeros_like(p0), 1,
                             1e-3, 1e-2)
    assert np.abs(p1 - ref).max() <= 1e-5 * np.abs(ref).max()
    net.close()
    ctx.close()


def test_warm_start_beats_freestream_on_held_out_conditions():
    mesh = meshgen.bump_channel(16, 6, 4, 0.08)
    train = np.array([meshgen.freestream_mach_vector(m, a, b)
                      for m, a, b in meshgen.sample_conditions(24, seed=1, mach=(0.4, 0.7))])
    test = np.array([meshgen.freestream_mach_vector(m, a, b)
                     for m, a, b in meshgen.sample_conditions(4, seed=2, mach=(0.45, 0.65))])
    n_it = 1500
    # training data: the batched solver's states after n_it iterations
    sweep = _ctx(mesh, machs=train)
    sweep.explicit_iterations(n_it, history=False)
    states = sweep.get_state()
    sweep.close()
    base = _ctx(mesh)
    net = lib.WarmStart(base, seed=0)
    loss = net.train(train, states, steps=1500, batch=2048, lr=1e-3, weight_decay=1e-4, seed=7)
    assert np.all(np.isfinite(loss)) and loss[-100:].mean() < 0.2 * loss[:10].mean()
    # held-out conditions: reference states, then runs from the freestream and from the network
    ref = _ctx(mesh, machs=test)
    h_fs = ref.explicit_iterations(n_it)
    U_ref = ref.get_state()
    ref.close()
    warm = _ctx(mesh, machs=test)
    used = net.init_state(warm)
    assert used.all()
    U_pred = warm.get_state()
    fs = _ctx(mesh, machs=test)
    U_fs = fs.get_state()
    fs.close()
    err_pred = np.linalg.norm((U_pred - U_ref).reshape(len(test), -1), axis=1)
    err_fs = np.linalg.norm((U_fs - U_ref).reshape(len(test), -1), axis=1)
    assert np.all(err_pred < 0.5 * err_fs), (err_pred, err_fs)
    h_w = warm.explicit_iterations(n_it)
    r_fs = np.sqrt((h_fs[:, :, :5] ** 2).sum(axis=2))
    r_w = np.sqrt((h_w[:, :, :5] ** 2).sum(axis=2))
    target = r_fs[n_it // 2]  # the freestream run's residual half way
    it_fs = np.array([np.argmax(r_fs[:, b] <= target[b]) + 1 for b in range(len(test))])
    it_w = np.array([np.argmax(r_w[:, b] <= target[b]) + 1 if (r_w[:, b] <= target[b]).any()
                     else n_it + 1 for b in range(len(test))])
    assert it_w.sum() < it_fs.sum(), (it_w, it_fs)
    warm.close()
    net.close()
    base.close()
