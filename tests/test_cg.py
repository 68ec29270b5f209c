"""Conjugate gradients (fsils_solve with LS_TYPE_CG -> cgrad_v, cgrad.cpp:166-246) on the
mesh-motion system of the small pipe, against the reference solver's own output
(tests/golden/ref_mesh_cg*_small.npz, made by make_golden.py from the compiled
reference): zero Dirichlet values at the inlet and outlet nodes, FSILS diagonal
preconditioner, CG to 1e-10 (22 iterations) and exactly 7 iterations.

* oracle: bitwise equal (same summation order as the reference);
* GPU: the dot products and norms are summed in another order, so the iterates agree
  to rounding: iteration counts equal, increments within 1e-9 relative after 7
  iterations and within 1e-8 at convergence."""
import numpy as np
import pytest

from oracle import pyoracle as po

CASES = ["mesh_cg_small", "mesh_cg7_small"]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def setup(g):
    nNo = g["R_asm"].shape[0]
    mask = np.ones((nNo, 3))
    mask[g["dir_nodes"]] = 0.0
    return nNo, mask, eval(str(g["params"]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_cg_bitwise(golden, name):
    g = golden(name)
    nNo, mask, P = setup(g)
    X, _, ls = po.fsils_solve_cg(g["rowPtr"], g["colPtr"], g["Val_asm"], g["R_asm"], mask, mItr=P["ls_max_itr"],
                                 relTol=P["ls_rel_tol"], absTol=P["ls_abs_tol"])
    st = g["cg_stats"]
    assert np.array_equal(X, g["dX"])
    assert (ls.iNorm, ls.fNorm, ls.itr, ls.suc, ls.dB) == tuple(st[:2]) + (int(st[2]), int(st[3]), st[4])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_cg_matches_reference(golden, name):
    from svfsiplus_gb300 import api
    g = golden(name)
    nNo, mask, P = setup(g)
    ctx = api.Context(0)
    ctx.fsils_lhs_create(nNo, g["rowPtr"], g["colPtr"], 1)
    ctx.fsils_bc_create(0, g["dir_nodes"], 3, api.BC_TYPE_Dir)
    ctx.fsils_ls_create(api.LS_TYPE_CG, P["ls_rel_tol"], P["ls_abs_tol"], P["ls_max_itr"])
    Ri = np.array(g["R_asm"], copy=True)
    Val = np.array(g["Val_asm"], copy=True)
    st = ctx.fsils_solve(3, Ri, Val, api.PREC_FSILS, incL=np.ones(1, np.int32), res=np.zeros(1))
    ref = g["cg_stats"]
    assert abs(st.iNorm - ref[0]) <= 1e-13 * ref[0]
    assert st.itr == int(ref[2]) and st.suc == int(ref[3])
    assert abs(st.fNorm - ref[1]) <= 1e-3 * ref[1] + 1e-12 * ref[0]
    assert rel(Ri, g["dX"]) <= (1e-9 if name == "mesh_cg7_small" else 1e-8)
