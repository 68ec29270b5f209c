"""Failure detection of the solve, made on the host and ended without a GPU fault.

Each failure is planted in the inputs or the settings, never in a kernel:
  * a NaN written into the residual: svgpu_fsils_solve returns SVGPU_ENAN (the reference
    has no test for it and would iterate on NaN, gmres.cpp:450-629), and the same context
    then solves a clean system to the oracle's answer;
  * a tolerance no solve can meet: the solve ends at its restart cap with suc = 0 and the
    iteration count of gmres_v (ls.suc stays false, ls.itr counts each restart and each
    Arnoldi step, gmres.cpp:481-506,533,590), equal to the oracle's;
  * a guess threshold no initial guess can meet: every history guess is rejected, the
    solves start from zero, and the fields still match the reference's;
  * a network that cannot precondition -- untrained (zero decoder) as the only
    preconditioner (mode 1), or with a NaN decoder weight as the V-cycle's pre-smoother
    (mode 3): its cycles break down, they are rejected, and the method without the
    learned part finishes each solve at the reference's answer.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe

pytestmark = pytest.mark.gpu
SVGPU_ENAN = -5


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _system(name="tiny", seed=2):
    """The fluid system of a pipe at a seeded state (the oracle's assembly) and the
    Dirichlet mask of its inlet and wall."""
    m = named_pipe(name)
    rng = np.random.default_rng(seed)
    Ag = 0.1 * rng.standard_normal((m.nNo, 4))
    Yg = rng.standard_normal((m.nNo, 4))
    rowPtr, colPtr = po.lhsa(m.nNo, m.ien)
    R, Val = po.construct_fluid(po.fluid_params(), m.x, m.ien, Ag, Yg, rowPtr, colPtr)
    nodes, _ = api.dirichlet_nodes(m)
    mask = np.ones((m.nNo, 4))
    mask[nodes, :3] = 0.0
    return m, rowPtr, colPtr, R, Val, mask


def _ctx(m, rowPtr, colPtr, relTol, mItr, sD):
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, rowPtr, colPtr, 2)
    ctx.fsils_bc_create(0, m.faces["inlet"].gN, 3, api.BC_TYPE_Dir)
    ctx.fsils_bc_create(1, m.faces["wall"].gN, 3, api.BC_TYPE_Dir)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, relTol, 1e-17, mItr, sD)
    return ctx


def test_nan_residual_returns_enan_and_context_survives():
    m, rowPtr, colPtr, R, Val, mask = _system()
    ctx = _ctx(m, rowPtr, colPtr, 1e-10, 50, 50)
    bad = R.copy()
    bad[m.nNo // 2, 3] = np.nan
    st = api.LsStats()
    rc = api.lib().svgpu_fsils_solve(ctx._h, 4, bad.ctypes.data_as(C.c_void_p), Val.copy().ctypes.data_as(C.c_void_p),
                                     api.PREC_FSILS, None, None, C.byref(st))
    assert rc == SVGPU_ENAN
    assert "non-finite" in api.lib().svgpu_last_error(ctx._h).decode()
    # the same context, a clean system: the oracle's increment
    x = R.copy()
    st = ctx.fsils_solve(4, x, Val.copy(), api.PREC_FSILS, incL=np.ones(2, np.int32), res=np.zeros(2))
    ref, _, ls = po.fsils_solve_gmres(rowPtr, colPtr, Val, R, mask, sD=50, mItr=50, relTol=1e-10)
    assert st.suc == 1 and ls.suc == 1
    assert rel(x, ref) <= 1e-6
    ctx.close()


def test_nan_state_in_mixed_step_returns_enan():
    """A NaN in the flow state reaches the mixed-precision step's residual: the step
    returns SVGPU_ENAN instead of iterating, and the solver steps on from a clean state."""
    m = named_pipe("small")
    s = api.PipeFluidSolver(m, sD=50, mItr=20, relTol=1e-8, newton_min=1, newton_max=3, newton_tol=1e-6,
                            precision=api.SVGPU_MIXED)
    s.ctx.set_solver_mode(2)
    s.step(10.0, 0.0, 1.0)
    good = (s.Ao.copy(), s.Yo.copy())
    s.Yo[7, 1] = np.nan
    with pytest.raises(RuntimeError, match=r"status -5"):
        s.step(10.0, 0.0, 1.0)
    s.Ao[:], s.Yo[:] = good
    st = s.step(10.0, 0.0, 1.0)
    assert all(q["suc"] for q in st) and np.isfinite(s.Yn).all()
    s.ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_unreachable_tolerance_ends_at_the_cap(precision):
    """relTol 1e-30, 3 restarts of GMRES(10): suc = 0, itr = 3 * (10 + 1) as gmres_v
    counts, and for the FP64 path the oracle's increment, suc and itr."""
    m, rowPtr, colPtr, R, Val, mask = _system()
    sD, mItr = 10, 3
    ctx = _ctx(m, rowPtr, colPtr, 1e-30, mItr, sD)
    ref, _, ls = po.fsils_solve_gmres(rowPtr, colPtr, Val, R, mask, sD=sD, mItr=mItr, relTol=1e-30)
    assert ls.suc == 0 and ls.itr == mItr * (sD + 1)
    if precision == "fp64":
        x = R.copy()
        st = ctx.fsils_solve(4, x, Val.copy(), api.PREC_FSILS, incL=np.ones(2, np.int32), res=np.zeros(2))
        assert st.suc == 0 and st.itr == ls.itr
        assert rel(x, ref) <= 1e-8
        assert abs(st.fNorm - ls.fNorm) <= 1e-6 * ls.iNorm
    else:
        import torch
        # the FP32 tangent resident in the context: the mixed solve of svgpu_fluid_step
        ctx.mesh_create(m.x, m.ien)
        rng = np.random.default_rng(2)
        Ag = torch.from_numpy(0.1 * rng.standard_normal((m.nNo, 4))).cuda()
        Yg = torch.from_numpy(rng.standard_normal((m.nNo, 4))).cuda()
        ctx.construct_fluid(api.fluid_props(), Ag, Yg, precision=api.SVGPU_MIXED)
        st = api.LsStats()
        rc = api.lib().svgpu_fsils_solve(ctx._h, 4, None, None, api.PREC_FSILS, np.ones(2, np.int32).ctypes.data_as(
            C.c_void_p), np.zeros(2).ctypes.data_as(C.c_void_p), C.byref(st))
        assert rc == 0
        assert st.suc == 0 and st.itr == mItr * (sD + 1), (st.suc, st.itr)
    ctx.close()


def _pipe50k_solver(g, mode, learning=False):
    ps = eval(str(g["params"]))
    m = named_pipe("pipe50k")
    s = api.PipeFluidSolver(m, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                            absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                            newton_tol=ps["newton_tol"], rowPtr=g["rowPtr"], colPtr=g["colPtr"],
                            precision=api.SVGPU_MIXED)
    if learning:
        s.enable_learning()
    s.ctx.set_solver_mode(mode)
    return s, ps


def test_rejected_initial_guesses_still_reach_the_reference(golden):
    """Mode 5 (the previous step's increment as the initial guess) with a threshold no
    guess meets (a kept guess must leave less than 1e-9 of the residual): every guess
    from step 2 on is tried and rejected, each solve starts from zero, and the fields
    after step 10 match the reference's within 1e-6."""
    g = golden("pipe50k")
    s, ps = _pipe50k_solver(g, 5)
    assert api.lib().svgpu_guess_options(s.ctx._h, C.c_double(1e-9)) == api.SVGPU_OK
    kept = 0
    for _ in range(10):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert all(q["suc"] for q in st)
        kept += sum(q["x0_kept"] for q in st)
    tried, rejected, _ = s.ctx.guess_stats
    print("guesses tried / rejected:", tried, rejected)
    assert tried > 0 and rejected == tried and kept == 0
    ref = g["Yn_10"]
    assert rel(s.Yn[:, :3], ref[:, :3]) <= 1e-6 and rel(s.Yn[:, 3], ref[:, 3]) <= 1e-6
    s.ctx.close()


@pytest.mark.parametrize("mode", [1, 3])
def test_bad_network_cycles_are_rejected(golden, mode):
    """A network that cannot precondition, in the learned modes.  Mode 1 uses an
    untrained network (zero decoder: every preconditioned vector is zero, so the cycle
    breaks down) as the only right preconditioner of FGMRES; mode 3 uses a network with
    a NaN in its decoder as the V-cycle's finest pre-smoother (every cycle ends with a
    non-finite Arnoldi norm).  Those cycles are rejected (learned_rejects > 0) and each
    solve is finished by the method without the learned part (the plain V-cycle); the fields
    after steps 1 and 2 match the reference's own run (ref_small) within 1e-6."""
    g = golden("small")
    ps = eval(str(g["params"]))
    m = named_pipe("small")
    s = api.PipeFluidSolver(m, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                            absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                            newton_tol=ps["newton_tol"], precision=api.SVGPU_MIXED)
    s.enable_learning(collect=0)
    if mode == 3:
        p = s.ctx.gnn_params()
        p[-3] = np.nan  # a decoder weight
        s.ctx.gnn_set_params(p)
    s.ctx.set_solver_mode(mode)
    for step in (1, 2):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert all(q["suc"] for q in st), (mode, step, st)
        ev = rel(s.Yn, g[f"Yn_{step}"])
        print("mode", mode, "step", step, "Yn rel", ev, "rejects", s.ctx.learned_rejects, "its",
              [q["itr"] for q in st])
        assert ev <= 1e-6
    assert s.ctx.learned_rejects > 0
    s.ctx.close()
