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
