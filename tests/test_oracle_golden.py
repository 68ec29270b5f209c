"""The CPU oracle against golden vectors produced by the reference solver itself
(tests/golden/make_golden.py runs the reference's own construct_fluid, b_assem_neu_bc,
fsils_solve and pic* on procedural pipes).  The oracle follows the reference's
operation order, so these comparisons are bit-for-bit."""
import numpy as np
import pytest

from oracle import pyoracle as po
from svfsiplus_gb300.mesh import named_pipe


@pytest.mark.parametrize("name", ["tiny", "small", "pipe50k"])
def test_csr_pattern_matches_reference_lhsa(golden, name):
    g = golden(name)
    m = named_pipe(name)
    rp, cp = po.lhsa(m.nNo, m.ien)
    assert np.array_equal(rp, g["rowPtr"]) and np.array_equal(cp, g["colPtr"])


@pytest.mark.parametrize("name", ["tiny", "small", "pipe50k"])
def test_assembly_bitwise(golden, name):
    g = golden(name)
    m = named_pipe(name)
    P = po.fluid_params()
    rp, cp = po.lhsa(m.nNo, m.ien)
    R, Val = po.construct_fluid(P, m.x, m.ien, g["Ag"], g["Yg"], rp, cp)
    out = m.faces["outlet"]
    po.neu_backflow(P, out.ien, out.gE, m.ien, m.x, g["Yg"], rp, cp, R, Val)
    assert np.array_equal(R, g["R_asm"])
    if "Val_asm" in g:
        assert np.array_equal(Val, g["Val_asm"])


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_fsils_solve_bitwise(golden, name):
    g = golden(name)
    m = named_pipe(name)
    rp, cp = po.lhsa(m.nNo, m.ien)
    nodes, _ = po.dirichlet_nodes(m)
    mask = np.ones((m.nNo, 4))
    mask[nodes, :3] = 0.0
    dX, _, ls = po.fsils_solve_gmres(rp, cp, g["Val_asm"], g["R_asm"], mask)
    assert np.array_equal(dX, g["dX"])


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_time_steps_bitwise(golden, name):
    g = golden(name)
    m = named_pipe(name)
    ps = eval(str(g["params"]))
    run = po.FluidRun(m, po.fluid_params(), sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                      absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                      newton_tol=ps["newton_tol"])
    log = g["newton_log"]
    k = 0
    for s in range(1, ps["n_steps"] + 1):
        st = run.step(u_mean=ps["u_mean"], u_amp=ps["u_amp"], freq=ps["u_freq"])
        for it in range(st.shape[0]):
            assert st[it, 0] == log[k, 2]   # iNorm
            assert st[it, 2] == log[k, 4]   # Krylov iterations
            k += 1
        assert np.array_equal(run.Yn, g[f"Yn_{s}"])
        assert np.array_equal(run.An, g[f"An_{s}"])


def test_element_is_zero_jacobian_error():
    P = po.fluid_params()
    xl = np.zeros(12)  # degenerate tet
    with pytest.raises(RuntimeError):
        po.fluid_element(P, xl, np.zeros(16), np.zeros(16))
