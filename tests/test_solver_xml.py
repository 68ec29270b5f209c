"""Solver input (svMultiPhysicsFile XML) and VTK mesh/result files.

* the XML reader maps the reference's element names (Parameters.cpp) to settings;
* the Fourier representation of unsteady boundary values is the reference's own
  (fft/ifft, fft.cpp): coefficients and values match the compiled reference's
  (tests/golden/ref_fourier.npz) to rounding;
* VTK XML files round-trip in every encoding VTK writes (ascii, inline base64, appended
  raw; zlib-compressed or not), and a mesh written as the reference's inputs
  (GlobalNodeID / GlobalElementID, 1-based) loads back into the same faces;
* the parabolic profile of bc_ini on the straight pipe equals 1 - r^2/R^2;
* (GPU) a case run from an XML file and .vtu/.vtp meshes gives the reference's fields:
  with the RCR outlet against the compiled reference's own run of the same case
  (tests/golden/ref_small_rcr_steady.npz), with a traction-free outlet against the
  oracle's time loop (oracle/pyoracle.FluidRun) on the same mesh and settings.
"""
import os

import numpy as np
import pytest

from svfsiplus_gb300 import api, solver_xml as sx, vtkio
from svfsiplus_gb300.mesh import named_pipe

CASE_XML = """<?xml version="1.0" encoding="UTF-8" ?>
<svMultiPhysicsFile version="0.1">
<GeneralSimulationParameters>
  <Number_of_spatial_dimensions> 3 </Number_of_spatial_dimensions>
  <Number_of_time_steps> 2 </Number_of_time_steps>
  <Time_step_size> 1e-3 </Time_step_size>
  <Spectral_radius_of_infinite_time_step> 0.50 </Spectral_radius_of_infinite_time_step>
</GeneralSimulationParameters>
<Add_mesh name="pipe" >
  <Mesh_file_path> mesh/mesh-complete.mesh.vtu </Mesh_file_path>
  <Add_face name="inlet"> <Face_file_path> mesh/inlet.vtp </Face_file_path> </Add_face>
  <Add_face name="outlet"> <Face_file_path> mesh/outlet.vtp </Face_file_path> </Add_face>
  <Add_face name="wall"> <Face_file_path> mesh/wall.vtp </Face_file_path> </Add_face>
</Add_mesh>
<Add_equation type="fluid" >
   <Coupled> true </Coupled>
   <Min_iterations> 3 </Min_iterations>
   <Max_iterations> 3 </Max_iterations>
   <Tolerance> 1e-11 </Tolerance>
   <Backflow_stabilization_coefficient> 0.2 </Backflow_stabilization_coefficient>
   <Density> 1.06 </Density>
   <Viscosity model="Constant" > <Value> 0.04 </Value> </Viscosity>
   <LS type="GMRES" >
      <Linear_algebra type="fsils" > <Preconditioner> fsils </Preconditioner> </Linear_algebra>
      <Tolerance> 1e-8 </Tolerance>
      <Absolute_tolerance> 1e-17 </Absolute_tolerance>
      <Max_iterations> 100 </Max_iterations>
      <Krylov_space_dimension> 50 </Krylov_space_dimension>
   </LS>
   <Add_BC name="inlet" >
      <Type> Dir </Type> <Time_dependence> Steady </Time_dependence> <Value> -10.0 </Value>
      <Profile> Parabolic </Profile>
   </Add_BC>
   <Add_BC name="wall" >
      <Type> Dir </Type> <Time_dependence> Steady </Time_dependence> <Value> 0.0 </Value>
   </Add_BC>
   <Add_BC name="outlet" >
      <Type> Neu </Type> <Time_dependence> RCR </Time_dependence>
      <RCR_values>
        <Capacitance> 1.5e-5 </Capacitance> <Distal_resistance> 1212 </Distal_resistance>
        <Proximal_resistance> 121 </Proximal_resistance> <Distal_pressure> 0 </Distal_pressure>
        <Initial_pressure> 0 </Initial_pressure>
      </RCR_values>
   </Add_BC>
</Add_equation>
</svMultiPhysicsFile>
"""


TRACTION_FREE_OUTLET = """   <Add_BC name="outlet" >
      <Type> Neu </Type> <Time_dependence> Steady </Time_dependence> <Value> 0.0 </Value>
   </Add_BC>
</Add_equation>"""


def _write_case(d, traction_free=False):
    m = named_pipe("small")
    vtkio.write_mesh_files(os.path.join(d, "mesh"), m)
    p = os.path.join(d, "solver.xml")
    xml = CASE_XML
    if traction_free:
        a = xml.index('   <Add_BC name="outlet" >')
        b = xml.index("</Add_equation>") + len("</Add_equation>")
        xml = xml[:a] + TRACTION_FREE_OUTLET + xml[b:]
    with open(p, "w") as fh:
        fh.write(xml)
    return m, p


def test_parse_solver_xml(tmp_path):
    _, p = _write_case(str(tmp_path))
    cfg = sx.parse_solver_xml(p)
    assert cfg.n_time_steps == 2 and cfg.dt == 1e-3 and cfg.rho_inf == 0.5
    assert cfg.meshes[0].faces == {"inlet": "mesh/inlet.vtp", "outlet": "mesh/outlet.vtp", "wall": "mesh/wall.vtp"}
    eq = cfg.equations[0]
    assert (eq.type, eq.min_iterations, eq.max_iterations, eq.tolerance) == ("fluid", 3, 3, 1e-11)
    assert (eq.density, eq.viscosity, eq.backflow) == (1.06, 0.04, 0.2)
    assert (eq.ls.type, eq.ls.tolerance, eq.ls.max_iterations, eq.ls.krylov_space_dimension) == ("GMRES", 1e-8, 100, 50)
    names = [(b.name, b.type, b.time_dependence) for b in eq.bcs]
    assert names == [("inlet", "Dir", "Steady"), ("wall", "Dir", "Steady"), ("outlet", "Neu", "RCR")]
    assert eq.bcs[0].value == -10.0 and eq.bcs[0].profile == "Parabolic"
    assert eq.bcs[2].rcr == dict(Rp=121.0, C=1.5e-5, Rd=1212.0, Pd=0.0, Xo=0.0)


@pytest.mark.parametrize("ramp", [0, 1])
def test_fourier_matches_reference(golden, ramp):
    g = golden("fourier")
    f = sx.fourier_fit(g["t"], g["q"], 10, bool(ramp))
    coef = np.concatenate([[f.ti, f.T, f.qi, f.qs], f.r, f.i])
    ref = g[f"coef_ramp{ramp}"]
    assert np.allclose(coef, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    ev = np.array([sx.fourier_eval(f, t) for t in g["times"]])
    er = g[f"eval_ramp{ramp}"]
    assert np.allclose(ev, er, rtol=1e-12, atol=1e-12 * np.abs(er).max())


@pytest.mark.parametrize("encoding,compress", [("appended", False), ("appended", True), ("binary", False),
                                               ("binary", True), ("ascii", False)])
def test_mesh_files_round_trip(tmp_path, encoding, compress):
    m = named_pipe("small")
    vtu, faces = vtkio.write_mesh_files(str(tmp_path), m, encoding=encoding, compress=compress)
    mm = vtkio.load_mesh(vtu, faces)
    assert np.array_equal(mm.x, m.x) and np.array_equal(mm.ien, m.ien)
    for k, f in m.faces.items():
        g = mm.faces[k]
        assert np.array_equal(g.ien, f.ien) and np.array_equal(g.gE, f.gE) and np.array_equal(g.gN, f.gN)


def test_result_vtu_fields(tmp_path):
    """svgpu_write_vtu: the fields and the mesh read back exactly."""
    m = named_pipe("tiny")
    rng = np.random.default_rng(3)
    vel, p = rng.standard_normal((m.nNo, 3)), rng.standard_normal(m.nNo)
    path = str(tmp_path / "result_001.vtu")
    vtkio.write_vtu(path, m.x, m.ien, {"Velocity": vel, "Pressure": p})
    d = vtkio.read_vtk(path)
    assert np.array_equal(d["points"], m.x)
    assert np.array_equal(vtkio.cell_connectivity(d, 4), m.ien)
    assert np.array_equal(d["point_data"]["Velocity"], vel) and np.array_equal(d["point_data"]["Pressure"], p)
    assert set(np.unique(d["cells"]["types"])) == {10}


def test_parabolic_profile_is_the_pipe_profile():
    m = named_pipe("small")
    bc = sx.BcSpec(name="inlet", type="Dir", profile="Parabolic")
    gx = sx.bc_profile(m, "inlet", bc)
    assert np.allclose(gx, m.inlet_profile, atol=1e-12)
    nV = sx.face_unit_normals(m, "inlet")
    assert np.allclose(nV, [0.0, 0.0, -1.0], atol=1e-12)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
def test_gpu_xml_case_matches_reference(tmp_path, golden):
    """The XML case (inlet -10 along the outward normal with the parabolic profile, no-slip
    wall, RCR outlet) through FluidCase against the compiled reference's run of the same
    case (ref_small_rcr_steady): fields after each of 2 steps within 1e-8, the tolerance
    of the reference's RCR steps through the API (test_rcr.py)."""
    g = golden("small_rcr_steady")
    ps = eval(str(g["params"]))
    assert ps["u_amp"] == 0.0 and ps["rcr_Rp"] == 121.0 and ps["n_steps"] == 2
    m, p = _write_case(str(tmp_path))
    case = sx.FluidCase(p)
    for step in (1, 2):
        case.step()
        ev, ea = _rel(case.Yn, g[f"Yn_{step}"]), _rel(case.An, g[f"An_{step}"])
        print("XML case vs reference, step", step, "Yn", ev, "An", ea)
        assert ev <= 1e-8 and ea <= 1e-8
    case.run(1, vtu_prefix=str(tmp_path / "result"), save_every=1)
    d = vtkio.read_vtk(str(tmp_path / "result_003.vtu"))
    assert np.array_equal(d["point_data"]["Pressure"], case.Yn[:, 3])
    case.ctx.close()


@pytest.mark.gpu
def test_gpu_xml_traction_free_case_matches_oracle(tmp_path):
    """The same XML case with a traction-free outlet against the oracle's time loop
    (the reference's Newton loop restated in C) on the same mesh and settings: fields
    after each of 2 steps within 1e-8."""
    from oracle import pyoracle as po
    m, p = _write_case(str(tmp_path), traction_free=True)
    case = sx.FluidCase(p)
    run = po.FluidRun(m, po.fluid_params(), sD=50, mItr=100, relTol=1e-8, absTol=1e-17, newton_min=3,
                      newton_max=3, newton_tol=1e-11)
    for step in (1, 2):
        case.step()
        run.step(10.0, 0.0, 1.0)
        ev, ea = _rel(case.Yn, run.Yn), _rel(case.An, run.An)
        print("XML case vs oracle, step", step, "Yn", ev, "An", ea)
        assert ev <= 1e-8 and ea <= 1e-8
    case.ctx.close()
