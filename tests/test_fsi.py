"""FSI assembly (construct_fsi, fsi.cpp:48-332) against the reference's own output on
the small pipe (tests/golden/ref_fsi_small.npz, made by make_golden.py from the
compiled reference): 1056 fluid elements integrated in the current configuration
x + D(4..6) with the convection velocity relative to the mesh velocity Y(4..6), and
672 neo-Hookean/ST91 solid elements (legacy struct_3d, dof 4), state arrays of 7 rows,
the FSI equation's generalised-alpha constants (rho_inf 0.5, first order).

Tolerance: relative 1e-12 on R and Val (FP64; the GPU sums the Gauss-point integrand
in another order and uses fused multiply-add)."""
import numpy as np
import pytest

from svfsiplus_gb300.mesh import named_pipe


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fsi_golden_has_both_domains(golden):
    g = golden("fsi_small")
    eid = g["eid"]
    assert set(np.unique(eid)) == {1, 2}
    assert np.isfinite(g["R_asm"]).all() and np.isfinite(g["Val_asm"]).all()


@pytest.mark.gpu
def test_gpu_fsi_assembly_matches_reference(golden):
    from svfsiplus_gb300 import api
    g = golden("fsi_small")
    ps = eval(str(g["params"]))
    m = named_pipe("small")
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, g["rowPtr"], g["colPtr"], 0)
    ctx.mesh_create(m.x, m.ien)
    ctx.mesh_domains(g["eid"])
    fp = api.fluid_props(rho=ps["rho_f"], mu=ps["mu"], dt=ps["dt"], rho_inf=ps["rho_inf"],
                         backflow_beta=ps["backflow_beta"])
    sp = api.solid_props(ps["rho_s"], ps["E"], ps["nu"], ps["dt"], ps["rho_inf"])
    sp.am, sp.af, sp.gam, sp.beta = fp.am, fp.af, fp.gam, fp.beta  # the FSI equation's constants
    R = np.zeros((m.nNo, 4))
    V = np.zeros((g["colPtr"].size, 16))
    ctx.construct_fsi(fp, sp, 7, g["A"], g["Y"], g["D"], R, V)
    er, ev = rel(R, g["R_asm"]), rel(V, g["Val_asm"])
    print("FSI assembly rel err: R", er, "Val", ev)
    assert er <= 1e-12 and ev <= 1e-12


@pytest.mark.gpu
def test_gpu_fsi_mixed_assembly_matches_reference(golden):
    """svgpu_construct_fsi_mixed (the mixed-precision FSI step's assembly: fluid residual
    rows in double-word FP32, fluid tangent in FP32, solid elements in FP64 arithmetic
    with FP32 blocks) against the reference's FP64 system: R within 1e-12 relative (the
    FP64 parity tolerance), Val within 1e-6 relative (FP32 storage and arithmetic)."""
    import ctypes as C
    import torch
    from svfsiplus_gb300 import api
    g = golden("fsi_small")
    ps = eval(str(g["params"]))
    m = named_pipe("small")
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, g["rowPtr"], g["colPtr"], 0)
    ctx.mesh_create(m.x, m.ien)
    ctx.mesh_domains(g["eid"])
    fp = api.fluid_props(rho=ps["rho_f"], mu=ps["mu"], dt=ps["dt"], rho_inf=ps["rho_inf"],
                         backflow_beta=ps["backflow_beta"])
    sp = api.solid_props(ps["rho_s"], ps["E"], ps["nu"], ps["dt"], ps["rho_inf"])
    sp.am, sp.af, sp.gam, sp.beta = fp.am, fp.af, fp.gam, fp.beta
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()  # noqa: E731
    A, Y, D = dev(g["A"]), dev(g["Y"]), dev(g["D"])
    for _ in range(2):  # a second call into cleared arrays gives the same system
        R = torch.zeros((m.nNo, 4), dtype=torch.float64, device="cuda")
        V = torch.zeros((g["colPtr"].size, 16), dtype=torch.float32, device="cuda")
        ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        rc = api.lib().svgpu_construct_fsi_mixed(ctx._h, C.byref(fp), C.byref(sp), 7, ptr(A), ptr(Y), ptr(D), ptr(R),
                                                 ptr(V))
        assert rc == 0, api.lib().svgpu_last_error(ctx._h)
        er = rel(R.cpu().numpy(), g["R_asm"])
        ev = rel(V.cpu().numpy().astype(np.float64), g["Val_asm"])
        print("mixed FSI assembly rel err: R", er, "Val", ev)
        assert er <= 1e-12 and ev <= 1e-6
    ctx.close()


# ---- coupled FSI time steps (iterate_solution with the FSI and mesh equations) -------
# Golden: tests/golden/ref_fsi_run_small.npz, made by make_golden.py from the compiled
# reference (main.cpp's loop with construct_fsi, construct_mesh, b_assem_neu_bc on the
# moving mesh, fsils_solve GMRES/CG and picp/pici/picc) on the FSI pipe 'fsi_small'
# (lumen + 2-ring wall annulus, 2880 tets of which 1152 solid), three time steps of
# three Newton iterations per equation.

def _run_params(g):
    return eval(str(g["params"]))


def test_fsi_run_golden_is_consistent(golden):
    """The reference's run: the equations alternate FSI, mesh, FSI, ... within a step,
    every solve converged, and after a step the solid nodes' mesh rows equal their
    displacement rows (picc, pic.cpp:181-201)."""
    from svfsiplus_gb300.mesh import named_pipe
    g = golden("fsi_run_small")
    log = g["newton_log"]
    assert log.shape[0] == 3 * 6
    assert list(log[:6, 1]) == [0, 1, 0, 1, 0, 1]
    assert np.all(log[:, 6] == 1)
    m = named_pipe("fsi_small")
    solid = np.zeros(m.nNo, bool)
    solid[m.ien[m.eid == 2].ravel()] = True
    for s in (1, 2, 3):
        D = g[f"Dn_{s}"]
        assert np.array_equal(D[solid, 4:7], D[solid, 0:3])
        assert np.abs(D[solid, 0:3]).max() > 0
    assert m.nNo == g["Yn_1"].shape[0] and g["colPtr"].size == g["Val_asm"].shape[0]


@pytest.mark.gpu
def test_gpu_fsi_ale_system_matches_reference(golden):
    """The FSI system of step 2, Newton iteration 3 (the reference dumped it after
    construct_fsi and the outlet's b_assem_neu_bc on the moving mesh): construct_fsi
    + svgpu_neu_bc_fluid_ale from the same Ag/Yg/Dg/Do.  Tolerance 1e-12 relative."""
    from svfsiplus_gb300 import api
    g = golden("fsi_run_small")
    ps = _run_params(g)
    m = named_pipe("fsi_small")
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, g["rowPtr"], g["colPtr"], 0)
    ctx.mesh_create(m.x, m.ien)
    ctx.mesh_domains(m.eid)
    out = m.faces["outlet"]
    ctx.face_create(api.FACE_OUTLET, out.ien, out.gE)
    p = api.fsi_props(ps["rho_f"], ps["mu"], ps["backflow_beta"], ps["rho_s"], ps["E"], ps["nu"], ps["dt"],
                      ps["rho_inf"], ps["mesh_E"], ps["mesh_nu"], ps["mesh_rho"])
    R = np.zeros((m.nNo, 4))
    V = np.zeros((g["colPtr"].size, 16))
    ctx.construct_fsi(p.fluid, p.solid, 7, g["Ag"], g["Yg"], g["Dg"], R, V)
    ctx.b_assem_neu_bc_ale(api.FACE_OUTLET, p.fluid, 0.0, 7, g["Yg"], g["Do"], R, V)
    er, ev = rel(R, g["R_asm"]), rel(V, g["Val_asm"])
    print("FSI ALE system rel err: R", er, "Val", ev)
    assert er <= 1e-12 and ev <= 1e-12
    ctx.close()


@pytest.mark.gpu
def test_gpu_fsi_steps_match_reference(golden):
    """Three coupled time steps through svgpu_fsi_step (C ABI) against the reference's
    fields after every step.  Per-field relative L2 tolerance 1e-8 (both sides solve
    each linear system to relative 1e-10): fluid velocity, pressure, solid displacement
    and mesh displacement.  Every Newton iteration's preconditioned initial residual
    norm within 1e-6 relative, the equation order identical."""
    from svfsiplus_gb300 import api
    g = golden("fsi_run_small")
    ps = _run_params(g)
    m = named_pipe("fsi_small")
    p = api.fsi_props(ps["rho_f"], ps["mu"], ps["backflow_beta"], ps["rho_s"], ps["E"], ps["nu"], ps["dt"],
                      ps["rho_inf"], ps["mesh_E"], ps["mesh_nu"], ps["mesh_rho"])
    s = api.PipeFsiSolver(m, p, newton=(ps["newton_min"], ps["newton_max"], ps["newton_tol"]),
                          mesh_newton=(ps["mesh_newton_min"], ps["mesh_newton_max"], ps["mesh_newton_tol"]),
                          gmres=(ps["ls_rel_tol"], ps["ls_abs_tol"], ps["ls_max_itr"], ps["ls_krylov_dim"]),
                          cg=(ps["mesh_ls_rel_tol"], ps["mesh_ls_abs_tol"], ps["mesh_ls_max_itr"]))
    assert np.array_equal(s.rowPtr, g["rowPtr"]) and np.array_equal(s.colPtr, g["colPtr"])
    solid = np.zeros(m.nNo, bool)
    solid[s.solid_nodes] = True
    fluid = ~solid
    log = g["newton_log"]
    k = 0
    for step in (1, 2, 3):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert [q for q, _ in st] == [int(v) for v in log[k:k + len(st), 1]]
        for q, d in st:
            ref = log[k]
            assert abs(d["iNorm"] - ref[3]) <= 1e-6 * ref[3], (step, q, d["iNorm"], ref[3])
            assert d["suc"] == 1
            k += 1
        Yr, Dr = g[f"Yn_{step}"], g[f"Dn_{step}"]
        errs = {"velocity": rel(s.Yn[fluid, 0:3], Yr[fluid, 0:3]),
                "pressure": rel(s.Yn[:, 3], Yr[:, 3]),
                "solid displacement": rel(s.Dn[solid, 0:3], Dr[solid, 0:3]),
                "mesh displacement": rel(s.Dn[:, 4:7], Dr[:, 4:7]),
                "acceleration": rel(s.An[:, 0:4], g[f"An_{step}"][:, 0:4])}
        print("step", step, {k2: f"{v:.2e}" for k2, v in errs.items()})
        assert max(errs.values()) <= 1e-8, errs
        assert np.array_equal(s.Dn[solid, 4:7], s.Dn[solid, 0:3])
    s.ctx.close()


@pytest.mark.gpu
def test_gpu_fsi_steps_mixed_multilevel(golden):
    """The same three steps with the FSI equation solved in mixed precision (FP32 copy of
    the FP64 tangent in the FP64 defect-correction loop) by multilevel-preconditioned
    FGMRES (solver mode 2); the mesh equation stays FP64 CG.  Per-field relative L2
    tolerance against the reference's FP64 fields: 1e-6."""
    from svfsiplus_gb300 import api
    g = golden("fsi_run_small")
    ps = _run_params(g)
    m = named_pipe("fsi_small")
    p = api.fsi_props(ps["rho_f"], ps["mu"], ps["backflow_beta"], ps["rho_s"], ps["E"], ps["nu"], ps["dt"],
                      ps["rho_inf"], ps["mesh_E"], ps["mesh_nu"], ps["mesh_rho"])
    s = api.PipeFsiSolver(m, p, newton=(3, 3, 1e-11), mesh_newton=(3, 3, 1e-11),
                          gmres=(ps["ls_rel_tol"], ps["ls_abs_tol"], ps["ls_max_itr"], ps["ls_krylov_dim"]),
                          cg=(ps["mesh_ls_rel_tol"], ps["mesh_ls_abs_tol"], ps["mesh_ls_max_itr"]),
                          precision=api.SVGPU_MIXED)
    s.ctx.set_solver_mode(2)
    solid = np.zeros(m.nNo, bool)
    solid[s.solid_nodes] = True
    for step in (1, 2, 3):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert all(d["suc"] == 1 for _, d in st)
        Yr, Dr = g[f"Yn_{step}"], g[f"Dn_{step}"]
        errs = {"velocity": rel(s.Yn[~solid, 0:3], Yr[~solid, 0:3]), "pressure": rel(s.Yn[:, 3], Yr[:, 3]),
                "solid displacement": rel(s.Dn[solid, 0:3], Dr[solid, 0:3]),
                "mesh displacement": rel(s.Dn[:, 4:7], Dr[:, 4:7])}
        its = [d["itr"] for q, d in st if q == 0]
        print("step", step, "FSI Krylov its", its, {k: f"{v:.2e}" for k, v in errs.items()})
        assert max(errs.values()) <= 1e-6, errs
    s.ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [2, 5, 4])
def test_gpu_fsi_steps_mixed_multilevel_mesh_equation(golden, mode):
    """The mixed path with the mesh equation solved by the multilevel FGMRES as well (its
    dof-3 system padded to 4x4 blocks in a solver context of its own): per-field
    relative L2 within 1e-6 of the reference's fields after every step.  Mode 5 starts
    both equations' solves from the previous step's increment of the same Newton
    iteration (kept only where it lowers the FP64 residual); mode 4 adds the learned
    network's correction to the FSI equation's guess, trained on the FSI solves of
    steps 1-2 (stored triples, Adam) and used in step 3."""
    from svfsiplus_gb300 import api
    g = golden("fsi_run_small")
    ps = _run_params(g)
    m = named_pipe("fsi_small")
    p = api.fsi_props(ps["rho_f"], ps["mu"], ps["backflow_beta"], ps["rho_s"], ps["E"], ps["nu"], ps["dt"],
                      ps["rho_inf"], ps["mesh_E"], ps["mesh_nu"], ps["mesh_rho"])
    s = api.PipeFsiSolver(m, p, newton=(3, 3, 1e-11), mesh_newton=(3, 3, 1e-11),
                          gmres=(ps["ls_rel_tol"], ps["ls_abs_tol"], ps["ls_max_itr"], ps["ls_krylov_dim"]),
                          precision=api.SVGPU_MIXED, mesh_gmres=(1e-10, 1e-17, 100, 50))
    if mode == 4:
        s.ctx.gnn_create(api.pipe_node_features(m), 1)
        s.ctx.gnn_collect(1)
    s.ctx.set_solver_mode(5 if mode == 4 else mode)
    solid = np.zeros(m.nNo, bool)
    solid[s.solid_nodes] = True
    for step in (1, 2, 3):
        if mode == 4 and step == 3:
            assert s.ctx.gnn_pair_count() > 0
            s.ctx.gnn_train(100, 1e-3)
            s.ctx.gnn_collect(False)
            s.ctx.set_solver_mode(4)
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert all(d["suc"] == 1 for _, d in st)
        Yr, Dr = g[f"Yn_{step}"], g[f"Dn_{step}"]
        errs = {"velocity": rel(s.Yn[~solid, 0:3], Yr[~solid, 0:3]), "pressure": rel(s.Yn[:, 3], Yr[:, 3]),
                "solid displacement": rel(s.Dn[solid, 0:3], Dr[solid, 0:3]),
                "mesh displacement": rel(s.Dn[:, 4:7], Dr[:, 4:7])}
        mesh_its = [d["itr"] for q, d in st if q == 1]
        print("step", step, "mesh Krylov its", mesh_its, {k: f"{v:.2e}" for k, v in errs.items()})
        assert max(errs.values()) <= 1e-6, errs
    s.ctx.close()


@pytest.mark.gpu
def test_gpu_fsi_kept_tangent_reaches_the_same_solution(golden):
    """svgpu_fsi_opts.reuse_tangent = 1 (the FSI equation's tangent of a step's first
    iteration kept for the later ones, residual rows reassembled every iteration) changes
    the path of the Newton iteration, not its fixed point: with both equations driven to
    picc's 1e-10 (at most 12 iterations each), 3 steps of the mixed multilevel path with
    and without the kept tangent agree within 1e-8 per field."""
    from svfsiplus_gb300 import api
    g = golden("fsi_run_small")
    ps = _run_params(g)
    m = named_pipe("fsi_small")
    p = api.fsi_props(ps["rho_f"], ps["mu"], ps["backflow_beta"], ps["rho_s"], ps["E"], ps["nu"], ps["dt"],
                      ps["rho_inf"], ps["mesh_E"], ps["mesh_nu"], ps["mesh_rho"])
    out = {}
    for reuse in (0, 1):
        s = api.PipeFsiSolver(m, p, newton=(1, 12, 1e-10), mesh_newton=(1, 12, 1e-10),
                              gmres=(1e-4, 1e-17, 100, 50), precision=api.SVGPU_MIXED,
                              mesh_gmres=(1e-6, 1e-17, 100, 50))
        s.opts.reuse_tangent = reuse
        s.ctx.set_solver_mode(2)
        its = []
        for step in (1, 2, 3):
            st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
            assert all(d["suc"] == 1 for _, d in st)
            its.append(sum(1 for q, _ in st if q == 0))
        out[reuse] = (s.Yn.copy(), s.Dn.copy(), its)
        s.ctx.close()
    (Y0, D0, i0), (Y1, D1, i1) = out[0], out[1]
    errs = {"velocity and pressure": rel(Y1[:, :4], Y0[:, :4]), "displacements": rel(D1[:, :7], D0[:, :7])}
    print("FSI Newton iterations per step, reassembled / kept:", i0, i1, {k: f"{v:.2e}" for k, v in errs.items()})
    assert max(errs.values()) <= 1e-8, errs
