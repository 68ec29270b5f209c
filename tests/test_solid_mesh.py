"""Solid (neo-Hookean) and mesh-motion (linear-elastic) assembly: the CPU oracle and
the GPU kernels against golden vectors made by the reference's own construct_dsolid
and construct_mesh (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_oracle_struct_matches_reference(golden):
    g = golden("struct_small")
    m = named_pipe("small")
    ps = eval(str(g["params"]))
    P = po.struct_params(ps["rho"], ps["E"], ps["nu"], ps["C10"], ps["Kpen"], ps["dt"], ps["rho_inf"])
    R, V = po.construct_struct(P, m.x, m.ien, g["A"], g["Y"], g["D"], g["rowPtr"], g["colPtr"])
    assert rel(R, g["R_asm"]) <= 1e-13 and rel(V, g["Val_asm"]) <= 1e-13


def test_oracle_mesh_matches_reference(golden):
    g = golden("mesh_small")
    m = named_pipe("small")
    ps = eval(str(g["params"]))
    R, V = po.construct_mesh(ps["E"], ps["nu"], ps["rho"], ps["dt"], ps["rho_inf"], m.x, m.ien, g["A"], g["D"],
                             g["Do"], g["rowPtr"], g["colPtr"])
    assert rel(R, g["R_asm"]) <= 1e-13 and rel(V, g["Val_asm"]) <= 1e-13


def _ctx(m, g):
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, g["rowPtr"], g["colPtr"], 0)
    ctx.mesh_create(m.x, m.ien)
    return ctx


@pytest.mark.gpu
def test_gpu_struct_matches_reference(golden):
    g = golden("struct_small")
    m = named_pipe("small")
    ps = eval(str(g["params"]))
    ctx = _ctx(m, g)
    props = api.solid_props(ps["rho"], ps["E"], ps["nu"], ps["dt"], ps["rho_inf"])
    R = np.zeros((m.nNo, 3))
    V = np.zeros((g["colPtr"].size, 9))
    ctx.construct_dsolid(props, 3, 3, 0, g["A"], g["Y"], g["D"], R, V)
    assert rel(R, g["R_asm"]) <= 1e-12 and rel(V, g["Val_asm"]) <= 1e-12


@pytest.mark.gpu
def test_gpu_mesh_matches_reference(golden):
    g = golden("mesh_small")
    m = named_pipe("small")
    ps = eval(str(g["params"]))
    ctx = _ctx(m, g)
    R = np.zeros((m.nNo, 3))
    V = np.zeros((g["colPtr"].size, 9))
    ctx.construct_mesh(ps["E"], ps["nu"], ps["rho"], ps["dt"], ps["rho_inf"], 7, 4, g["A"], g["D"], g["Do"], R, V)
    assert rel(R, g["R_asm"]) <= 1e-12 and rel(V, g["Val_asm"]) <= 1e-12
