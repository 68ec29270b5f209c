"""Learned preconditioner: GPU forward/backward against the CPU oracle of the same
network, online training on solver pairs, and the gain over plain GMRES.

Gradient tolerance: the GPU accumulates in FP32 (the oracle in FP64) and both store the
activations in BF16, so a few activations can round to a neighbouring BF16 value;
the loss agrees to 1e-3 and the gradient to 2e-2 relative (cosine >= 0.999)."""
import numpy as np
import pytest

from oracle import gnn_oracle as go
from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _ctx(m):
    rowPtr, colPtr = api.csr_pattern(m.nNo, m.ien)
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, rowPtr, colPtr, 2)
    ctx.gnn_create(api.pipe_node_features(m), seed=7)
    return ctx, rowPtr, colPtr


def test_forward_matches_oracle():
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(3)
    r = rng.standard_normal((m.nNo, 4))
    z = np.zeros((m.nNo, 4))
    ctx.gnn_apply(r, z)
    out, s, _ = go.forward(ctx.gnn_params(), rowPtr, colPtr, r, api.pipe_node_features(m))
    ref = s * out
    assert np.linalg.norm(z - ref) / np.linalg.norm(ref) <= 2e-2


def test_gradient_matches_oracle():
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(4)
    r = rng.standard_normal((m.nNo, 4))
    x = rng.standard_normal((m.nNo, 4))
    loss, g = ctx.gnn_loss_grad(r, x)
    lref, gref = go.loss_grad(ctx.gnn_params(), rowPtr, colPtr, r, x, api.pipe_node_features(m))
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    g = g.astype(np.float64)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) <= 2e-2
    assert g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)) >= 0.999


def test_training_lowers_loss():
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(5)
    # pairs (K e, e) of a smooth field e through a fixed random block operator stand in
    # for solver pairs here; the solver-driven path is exercised below
    for _ in range(4):
        e = np.cumsum(rng.standard_normal((m.nNo, 4)), axis=0) / np.sqrt(m.nNo)
        r = e + 0.1 * rng.standard_normal((m.nNo, 4))
        ctx.gnn_add_pair(r, e)
    l0 = ctx.gnn_train(1, lr=0.0)
    l1 = ctx.gnn_train(200, lr=1e-3)
    l2 = ctx.gnn_train(4, lr=0.0)
    assert l2 < 0.7 * l0, (l0, l1, l2)


def test_learned_initial_guess_ab(golden):
    """A/B of the learned part on the 50k-tet pipe (reference settings: GMRES tolerance
    1e-8, three Newton iterations per step).  Both arms run the multilevel FGMRES of the
    mixed path; arm B also stores its solver pairs for five steps, trains its network
    on them (Adam, lr 1e-3) and then uses it as the initial guess of every solve (solver
    mode 4), with rejection when the guess does not lower the FP64 residual.  Steps 6-10
    are compared: B must stay within 1e-6 of the reference's fields and must not need
    more than 10 % more Krylov iterations than A; the gain (or loss) is printed."""
    import time
    g = golden("pipe50k")
    m = named_pipe("pipe50k")
    ps = eval(str(g["params"]))
    arms = {}
    for arm in ("A", "B"):
        s = api.PipeFluidSolver(m, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                                absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                                newton_tol=ps["newton_tol"], rowPtr=g["rowPtr"], colPtr=g["colPtr"],
                                precision=api.SVGPU_MIXED)
        if arm == "B":
            s.enable_learning()
        s.ctx.set_solver_mode(2)
        its, secs, loss = 0, 0.0, None
        for step in range(1, 11):
            if arm == "B" and step == 6:
                s.ctx.gnn_collect(False)
                loss = (s.ctx.gnn_train(1, 0.0), s.ctx.gnn_train(200, 1e-3), s.ctx.gnn_train(1, 0.0))
                s.ctx.set_solver_mode(4)
            t = time.perf_counter()
            st = s.step(u_mean=ps["u_mean"], u_amp=ps["u_amp"], freq=ps["u_freq"])
            if step > 5:
                secs += time.perf_counter() - t
                its += sum(x["itr"] for x in st)
            assert all(x["suc"] for x in st), (arm, step, st)
        ref = g["Yn_10"]
        ev, ep = rel(s.Yn[:, :3], ref[:, :3]), rel(s.Yn[:, 3], ref[:, 3])
        arms[arm] = dict(its=its, s=secs, ev=ev, ep=ep, loss=loss, rejects=s.ctx.learned_rejects)
        s.ctx.close()
    print("learned initial guess A/B, steps 6-10:", arms)
    for a in arms.values():
        assert a["ev"] <= 1e-6 and a["ep"] <= 1e-6
    assert arms["B"]["its"] <= 1.1 * arms["A"]["its"]
