"""The coupled RCR (Windkessel) outlet of the reference's pipe_RCR_3d case: semi-implicit
0D coupling (set_bc_cpl, RCR_Integ_X, calc_der_cpl_bc; set_bc.cpp:50-790) and the
resistance term of the outlet face in every GMRES product (add_bc_mul.cpp:53).

Golden: tests/golden/ref_small_rcr.npz, made by make_golden.py from the compiled
reference on the small pipe (3 time steps, 3 Newton iterations each, GMRES to 1e-8)
with the reference test's RCR values (Rp 121, C 1.5e-5, Rd 1212, Pd 0, initial 0).

Tolerances: the host 0D integration is bit-exact with the reference (it runs the same
operations in the same order on the same inputs); the GPU steps match the reference's
per-iteration outlet pressures and flow rates to 1e-8 relative, its residual norms to
1e-8 of the step's first, and its fields to 1e-8 (both sides solve each system to
relative 1e-8).
"""
import numpy as np
import pytest

from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _rows(g):
    """Per Newton iteration of the reference's log: dict of its fields."""
    out = []
    for line in str(g["log"]).splitlines():
        t = line.split()
        if t and t[0] == "step":
            out.append({k: float(v) for k, v in zip(t[0::2], t[1::2])})
    return out


def _rcr(ps):
    return dict(Rp=ps["rcr_Rp"], C=ps["rcr_C"], Rd=ps["rcr_Rd"], Pd=ps["rcr_Pd"], Xo=ps["rcr_Xo"])


def test_rcr_0d_model_matches_reference(golden):
    """RCR_Integ_X and calc_der_cpl_bc on the host, fed the reference's own flow rates:
    the outlet pressure of every Newton iteration and the resistance dP/dQ are bitwise
    the reference's; the state carries from step to step (cplBC.xo = xn)."""
    g = golden("small_rcr")
    ps = eval(str(g["params"]))
    c = _rcr(ps)
    r = api.rcr_resistance(c["Rp"], c["C"], c["Rd"], c["Pd"], ps["dt"], c["Xo"], 0.0, 0.0)
    assert r == float(g["rcr_r"])
    rows = _rows(g)
    xo = c["Xo"]
    for k, row in enumerate(rows):
        xn, P = api.rcr_integrate(c["Rp"], c["C"], c["Rd"], c["Pd"], ps["dt"], xo, row["Qo"], row["Qn"])
        assert P == row["P"], (k, P, row["P"])
        if k + 1 < len(rows) and rows[k + 1]["step"] != row["step"]:
            xo = xn
    assert rows[-1]["P"] > 1000.0  # the Windkessel has charged


def test_rcr_face_normal_integrals_golden(golden):
    """The reference's resistance face carries the nodal normal integrals of the outlet:
    axial, summing to the outlet area."""
    g = golden("small_rcr")
    v = g["rcr_face_val"]
    m = named_pipe("small")
    assert v.shape == (m.faces["outlet"].gN.size, 3)
    assert np.abs(v[:, :2]).max() < 1e-12
    area = 0.0
    out = m.faces["outlet"]
    for tri in out.ien:
        p = m.x[tri]
        area += 0.5 * np.linalg.norm(np.cross(p[1] - p[0], p[2] - p[0]))
    assert abs(abs(v[:, 2].sum()) - area) < 1e-12


def _solver(g, precision=api.SVGPU_FP64):
    ps = eval(str(g["params"]))
    m = named_pipe("small")
    s = api.PipeFluidSolver(m, api.fluid_props(rho=ps["rho"], mu=ps["mu"], dt=ps["dt"], rho_inf=ps["rho_inf"],
                                               backflow_beta=ps["backflow_beta"]),
                            sD=ps["ls_krylov_dim"], mItr=ps["ls_max_itr"], relTol=ps["ls_rel_tol"],
                            absTol=ps["ls_abs_tol"], newton_min=ps["newton_min"], newton_max=ps["newton_max"],
                            newton_tol=ps["newton_tol"], precision=precision, rcr=_rcr(ps))
    return s, ps


@pytest.mark.gpu
def test_gpu_rcr_steps_match_reference(golden):
    """Three time steps through svgpu_fluid_step with the RCR outlet (FP64 GMRES with the
    outlet's resistance term) against the reference: every Newton iteration's outlet
    flow rate, pressure and preconditioned residual norm, the fields after each step."""
    g = golden("small_rcr")
    s, ps = _solver(g)
    rows = _rows(g)
    k = 0
    for step in (1, 2, 3):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert len(st) == 3
        first = rows[k]["iNorm"]
        for q in st:
            ref = rows[k]
            # relative to the step's first residual: each solve stops at 1e-8 of its own
            assert abs(q["iNorm"] - ref["iNorm"]) <= 1e-8 * first, (step, q["iNorm"], ref["iNorm"])
            assert q["suc"] == 1
            k += 1
        state = s.ctx.rcr_state()
        ref = rows[k - 1]
        assert abs(state["Qn"] - ref["Qn"]) <= 1e-8 * abs(ref["Qn"]) + 1e-14, (state, ref)
        assert abs(state["P"] - ref["P"]) <= 1e-8 * abs(ref["P"]), (state, ref)
        ev, ea = rel(s.Yn, g[f"Yn_{step}"]), rel(s.An, g[f"An_{step}"])
        print("step", step, "P", state["P"], "Q", state["Qn"], "Yn rel", ev, "An rel", ea)
        assert ev <= 1e-8 and ea <= 1e-8
    assert abs(s.ctx.rcr_state()["r"] - float(g["rcr_r"])) <= 1e-12 * float(g["rcr_r"])
    s.ctx.close()


@pytest.mark.gpu
def test_gpu_rcr_mixed_multilevel(golden):
    """The same steps on the mixed-precision path with the multilevel FGMRES (the
    outlet's resistance term in the FP32 cycles and the FP64 restart residuals): fields
    within 1e-6 of the reference's."""
    g = golden("small_rcr")
    s, ps = _solver(g, api.SVGPU_MIXED)
    s.ctx.set_solver_mode(2)
    for step in (1, 2, 3):
        st = s.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
        assert all(q["suc"] == 1 for q in st)
        ev = rel(s.Yn, g[f"Yn_{step}"])
        print("step", step, "Yn rel", ev, "P", s.ctx.rcr_state()["P"])
        assert ev <= 1e-6
    s.ctx.close()
