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


def _trained_like_params(ctx, rng):
    """The seeded parameters with a decoder of the hidden layers' scale, so that the
    output depends on every layer (the initial decoder is near zero)."""
    p = ctx.gnn_params()
    p[go.OFF_WD:go.OFF_WD + go.H * 4] = rng.uniform(-0.3, 0.3, go.H * 4).astype(np.float32)
    ctx.gnn_set_params(p)
    return p


@pytest.mark.parametrize("with_prior", [False, True])
def test_forward_matches_oracle(with_prior):
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(3)
    params = _trained_like_params(ctx, rng)
    r = rng.standard_normal((m.nNo, 4))
    prior = 40.0 * rng.standard_normal((m.nNo, 4)) if with_prior else None
    z = np.zeros((m.nNo, 4))
    ctx.gnn_apply(r, z, prior)
    out, s, _ = go.forward(params, rowPtr, colPtr, r, api.pipe_node_features(m), prior)
    ref = s * out
    if with_prior:
        assert abs(s - np.sqrt(np.mean(np.asarray(prior, np.float32).astype(np.float64) ** 2))) <= 1e-6 * s
    assert np.linalg.norm(z - ref) / np.linalg.norm(ref) <= 2e-2


@pytest.mark.parametrize("with_prior", [False, True])
def test_gradient_matches_oracle(with_prior):
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(4)
    params = _trained_like_params(ctx, rng)
    r = rng.standard_normal((m.nNo, 4))
    x = rng.standard_normal((m.nNo, 4))
    prior = 0.8 * x + 0.3 * rng.standard_normal((m.nNo, 4)) if with_prior else None
    loss, g = ctx.gnn_loss_grad(r, x, prior)
    lref, gref = go.loss_grad(params, rowPtr, colPtr, r, x, api.pipe_node_features(m), prior)
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    g = g.astype(np.float64)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) <= 2e-2
    assert g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)) >= 0.999


def test_pairs_round_trip():
    """Stored triples come back rounded to FP32, oldest first, with a zero prior where
    none was given."""
    m = named_pipe("small")
    ctx, rowPtr, colPtr = _ctx(m)
    rng = np.random.default_rng(6)
    trip = [(rng.standard_normal((m.nNo, 4)), rng.standard_normal((m.nNo, 4)) if k else None,
             rng.standard_normal((m.nNo, 4))) for k in range(3)]
    for r, p, x in trip:
        ctx.gnn_add_pair(r, x, p)
    got = ctx.gnn_pairs()
    assert len(got) == 3
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)  # noqa: E731
    for (r, p, x), (gr, gp, gx) in zip(trip, got):
        assert np.array_equal(gr, f32(r)) and np.array_equal(gx, f32(x))
        assert np.array_equal(gp, np.zeros_like(gp) if p is None else f32(p))


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
    l0 = ctx.gnn_eval()
    l1 = ctx.gnn_train(200, lr=1e-3)
    l2 = ctx.gnn_eval()
    assert abs(l0 - 1.0) < 1e-6  # zero decoder: no correction, the relative error of x is 1
    assert l2 < 0.7 * l0, (l0, l1, l2)


def test_learned_initial_guess_ab(golden):
    """What the learned initial guess gains, on the 50k-tet pipe at the reference's
    settings (GMRES tolerance 1e-8, three Newton iterations per step).  Three arms run
    the multilevel FGMRES of the mixed path from the same start; steps 1-5 are alike
    (the history arms keep each solve's increment, arm L also stores its
    (residual, prior, increment) triples and trains its network on them with Adam,
    lr 1e-3), steps 6-10 differ in the initial guess only:
      A  zero (solver mode 2, the method without the learned part),
      H  the previous step's increment of the same Newton iteration, minimal-residual
         scaled (mode 5, no network),
      L  H plus the network's correction as a second direction (mode 4).
    Every arm stays within 1e-6 of the reference's fields; the history guesses must
    save Krylov iterations against A, and the network must not cost iterations
    against H.  Iterations, guesses kept and training losses are printed."""
    g = golden("pipe50k")
    m = named_pipe("pipe50k")
    ps = eval(str(g["params"]))
    arms = {}
    for arm, mode in (("A", 2), ("H", 5), ("L", 4)):
        s = api.PipeFluidSolver(m, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                                absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                                newton_tol=ps["newton_tol"], rowPtr=g["rowPtr"], colPtr=g["colPtr"],
                                precision=api.SVGPU_MIXED)
        if arm == "L":
            s.enable_learning()
        s.ctx.set_solver_mode(5 if arm == "H" else 2)
        its, loss, x0 = 0, [], []
        for step in range(1, 11):
            if step == 6:
                if arm == "L":
                    s.ctx.gnn_collect(False)
                s.ctx.set_solver_mode(mode)
            st = s.step(u_mean=ps["u_mean"], u_amp=ps["u_amp"], freq=ps["u_freq"])
            assert all(x["suc"] for x in st), (arm, step, st)
            if arm == "L" and 2 <= step <= 5:
                e0 = s.ctx.gnn_eval()
                s.ctx.gnn_train(100, 1e-3)
                loss.append((round(e0, 4), round(s.ctx.gnn_eval(), 4)))
            if step > 5:
                its += sum(x["itr"] for x in st)
                x0.append([round(x["x0_rel"], 3) for x in st])
        ref = g["Yn_10"]
        ev, ep = rel(s.Yn[:, :3], ref[:, :3]), rel(s.Yn[:, 3], ref[:, 3])
        arms[arm] = dict(its=its, ev=ev, ep=ep, loss=loss, x0_rel=x0, guesses=s.ctx.guess_stats)
        s.ctx.close()
    print("initial-guess A/B/C, steps 6-10:", arms)
    for a in arms.values():
        assert a["ev"] <= 1e-6 and a["ep"] <= 1e-6
    assert arms["H"]["its"] < arms["A"]["its"]
    assert arms["L"]["its"] <= 1.05 * arms["H"]["its"]


def _pipe50k_learned(g, ps, **kw):
    m = named_pipe("pipe50k")
    s = api.PipeFluidSolver(m, rowPtr=g["rowPtr"], colPtr=g["colPtr"], precision=api.SVGPU_MIXED, **kw)
    s.enable_learning()
    s.ctx.set_solver_mode(2)
    return s


def _train_then(s, ps, mode, steps=10, switch=6):
    """Steps 1..switch-1 in mode 2 storing the solves' triples (Adam after steps 2..),
    then the given mode with the network frozen."""
    for step in range(1, steps + 1):
        if step == switch:
            s.ctx.gnn_collect(False)
            s.ctx.set_solver_mode(mode)
        st = s.step(u_mean=ps["u_mean"], u_amp=ps["u_amp"], freq=ps["u_freq"])
        assert all(x["suc"] for x in st), (mode, step, st)
        if step < switch and s.ctx.gnn_pair_count() > 0:
            s.ctx.gnn_train(100, 1e-3)
    return s


@pytest.mark.parametrize("mode", [1, 3])
def test_learned_modes_reach_reference_pipe50k(golden, mode):
    """Mode 1 (the trained network as the only right preconditioner of FGMRES) and mode
    3 (the trained network as the V-cycle's finest pre-smoother), at the reference's
    settings on the 50k-tet pipe after 5 steps of online training: the fields after step
    10 within 1e-6 of the reference's own.  Cycles with the network that do not lower
    the FP64 residual are rolled back, those that do not halve it are kept; in either case
    the plain V-cycle finishes the solve.  The network's cycles given up are printed."""
    g = golden("pipe50k")
    ps = eval(str(g["params"]))
    s = _pipe50k_learned(g, ps, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                         absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                         newton_tol=ps["newton_tol"])
    r0 = s.ctx.learned_rejects
    _train_then(s, ps, mode)
    ref = g["Yn_10"]
    ev, ep = rel(s.Yn[:, :3], ref[:, :3]), rel(s.Yn[:, 3], ref[:, 3])
    print(f"mode {mode}: velocity {ev:.2e}, pressure {ep:.2e}, learned cycles rejected "
          f"{s.ctx.learned_rejects - r0}")
    assert ev <= 1e-6 and ep <= 1e-6
    s.ctx.close()


def test_headline_settings_pipe50k(golden):
    """The headline's settings on the 50k-tet pipe: mixed precision, multilevel FGMRES(50)
    from the learned initial guess (mode 4) after 5 steps of online training, tangent
    kept within a step, the extrapolating Newton predictor, linear relative tolerance
    1e-2, Newton to picc's 5e-9 (at most 8 iterations).  Checked against the reference
    run to convergence on the same 10 steps (ref_pipe50k_conv: the compiled reference,
    Newton to 1e-11 within 12 iterations, GMRES to 1e-8): per-field relative L2 within
    1e-6 after step 10.  The reference's fixed-3-iteration run (ref_pipe50k) is itself
    1e-7 (velocity) and 1.4e-6 (pressure) from its converged solution at step 10, so
    the settings are held to the converged one."""
    g = golden("pipe50k")
    gc = golden("pipe50k_conv")
    ps = eval(str(g["params"]))
    s = _pipe50k_learned(g, ps, sD=50, mItr=40, relTol=1e-2, absTol=1e-17, newton_min=1, newton_max=8,
                         newton_tol=5e-9, reuse_tangent=True)
    s.ctx.set_predictor(1)
    _train_then(s, ps, 4)
    ref = gc["Yn_10"]
    ev, ep = rel(s.Yn[:, :3], ref[:, :3]), rel(s.Yn[:, 3], ref[:, 3])
    e3v, e3p = rel(g["Yn_10"][:, :3], ref[:, :3]), rel(g["Yn_10"][:, 3], ref[:, 3])
    print(f"headline settings on pipe50k vs the converged reference: velocity {ev:.2e}, pressure {ep:.2e} "
          f"(the reference's 3-iteration run: {e3v:.2e}, {e3p:.2e}); guesses {s.ctx.guess_stats}")
    assert ev <= 1e-6 and ep <= 1e-6
    s.ctx.close()
