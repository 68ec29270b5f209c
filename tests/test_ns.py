"""The FSILS block solver for incompressible flow (fsils_solve with LS_TYPE_NS ->
ns_solver, ns_solver.cpp:167-499) against the reference solver's own output
(tests/golden/ref_{tiny,small}_ns.npz from make_golden.py and the compiled reference):
outer relative tolerance 1e-4, at most 10 outer iterations, inner GMRES and Schur CG at
the reference's NS defaults (GMRES relTol 1e-2, 2 restarts of 50; CG relTol 0.2, 500
iterations).

The GPU sums its dot products in another order, so the iterates differ by rounding
only: equal outer iteration counts, increments within 1e-9 relative (measured 7e-15 on
tiny, 2.5e-12 on small), the increment solving the preconditioned system to the outer
tolerance, and the fields after three Newton steps within 1e-10 (measured 4e-15)."""
import numpy as np
import pytest

from oracle import pyoracle as po


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def preconditioned_residual(g, X):
    """|W (R - K X)| / |W R| with W the diagonal scaling of precond_diag and the
    Dirichlet rows (inlet, wall) removed: the quantity ns_solver's tolerance bounds."""
    from svfsiplus_gb300.mesh import named_pipe
    rowPtr, colPtr, Val, R = g["rowPtr"], g["colPtr"], g["Val_asm"], g["R_asm"]
    nNo = R.shape[0]
    diag = np.zeros((nNo, 4))
    for a in range(nNo):
        k = rowPtr[a] + int(np.searchsorted(colPtr[rowPtr[a]:rowPtr[a + 1]], a))
        diag[a] = Val[k].reshape(4, 4).diagonal()
    diag[diag == 0.0] = 1.0
    W = 1.0 / np.sqrt(np.abs(diag))
    name = "tiny" if nNo < 100 else "small"
    m = named_pipe(name)
    for f in ("inlet", "wall"):
        W[m.faces[f].gN, :3] = 0.0
    # X is the increment of the unscaled system: X = W Xs, so W (R - K X) = Rs - Ks Xs
    KX = po.spar_mul(rowPtr, colPtr, Val, np.ascontiguousarray(X))
    return float(np.linalg.norm(W * (R - KX)) / np.linalg.norm(W * R))


@pytest.mark.parametrize("name", ["tiny_ns"])
def test_reference_ns_increment_meets_its_tolerance(golden, name):
    g = golden(name)
    assert preconditioned_residual(g, g["dX"]) <= 1.5e-4


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny_ns", "small_ns"])
def test_gpu_ns_solve_matches_reference(golden, name):
    from svfsiplus_gb300 import api
    from svfsiplus_gb300.mesh import named_pipe
    g = golden(name)
    ps = eval(str(g["params"]))
    m = named_pipe(name.replace("_ns", ""))
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, g["rowPtr"], g["colPtr"], 2)
    ctx.fsils_bc_create(0, m.faces["inlet"].gN, 3, api.BC_TYPE_Dir)
    ctx.fsils_bc_create(1, m.faces["wall"].gN, 3, api.BC_TYPE_Dir)
    ctx.fsils_ls_create(api.LS_TYPE_NS, ps["ls_rel_tol"], ps["ls_abs_tol"], ps["ls_max_itr"], ps["ls_krylov_dim"])
    Ri = np.array(g["R_asm"], copy=True)
    Val = np.array(g["Val_asm"], copy=True)
    st = ctx.fsils_solve(4, Ri, Val, api.PREC_FSILS, incL=np.ones(2, np.int32), res=np.zeros(2))
    log = g["newton_log"]
    row = [r for r in log if int(r[0]) == ps["dump_step"] and int(r[1]) == ps["dump_iter"]][0]
    print(name, "GPU itr", st.itr, "ref itr", int(row[4]), "GPU fNorm", st.fNorm, "ref", row[3],
          "dX rel", rel(Ri, g["dX"]), "prec. residual", preconditioned_residual(g, Ri))
    assert abs(st.iNorm - row[2]) <= 1e-10 * row[2]
    assert st.suc == 1 and st.itr == int(row[4])
    assert preconditioned_residual(g, Ri) <= 1.5e-4
    assert rel(Ri, g["dX"]) <= 1e-9


@pytest.mark.gpu
def test_gpu_ns_time_steps_match_reference(golden):
    from svfsiplus_gb300 import api
    from svfsiplus_gb300.mesh import named_pipe
    g = golden("small_ns")
    ps = eval(str(g["params"]))
    m = named_pipe("small")
    s = api.PipeFluidSolver(m, sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                            absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                            newton_tol=ps["newton_tol"], rowPtr=g["rowPtr"], colPtr=g["colPtr"],
                            ls_type=api.LS_TYPE_NS)
    for step in range(1, ps["n_steps"] + 1):
        st = s.step(u_mean=ps["u_mean"], u_amp=ps["u_amp"], freq=ps["u_freq"])
        assert all(x["suc"] for x in st)
        ref = g[f"Yn_{step}"]
        ev, ep = rel(s.Yn[:, :3], ref[:, :3]), rel(s.Yn[:, 3], ref[:, 3])
        print("step", step, "velocity", ev, "pressure", ep)
        assert ev <= 1e-10 and ep <= 1e-10
