"""The reference's solver input file (svMultiPhysicsFile XML, read by Parameters.cpp and
read_files.cpp) for the fluid hot path, and a case driver that runs it on the GPU.

``parse_solver_xml(path)`` reads the general parameters, the meshes with their faces,
and each equation with its domains, linear solver and boundary conditions into plain
dataclasses (the element names of Parameters.cpp).

``FluidCase`` runs a single fluid equation from such a file (the reference's
``fluid/pipe_RCR_3d`` layout): the mesh from its .vtu/.vtp files (``vtkio.load_mesh``),
Dirichlet faces with flat or parabolic profiles, optional flux normalisation and
perimeter zeroing (bc_ini, baf_ini.cpp:270-432), steady or Fourier-interpolated
unsteady values along the face normal (set_bc_dir_l, set_bc.cpp:1005-1045; fft/ifft,
fft.cpp), one Neumann outlet with a steady value or an RCR model, the equation's
generalised-alpha and Newton settings, and its linear solver (GMRES, CG or NS).  Every
time step goes through ``svgpu_fluid_step``.
"""
from __future__ import annotations

import dataclasses
import math
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import api
from . import vtkio


def _text(el, name, default=None, cast=str):
    c = el.find(name) if el is not None else None
    if c is None or c.text is None:
        return default
    t = c.text.strip()
    if cast is bool:
        return t.lower() in ("true", "1")
    if cast is tuple:
        return tuple(float(v) for v in t.strip("()").split(","))
    return cast(t)


@dataclasses.dataclass
class BcSpec:
    name: str
    type: str                      # Dir / Neu
    time_dependence: str = "Steady"
    value: float = 0.0
    profile: str = "Flat"
    impose_flux: bool = False
    zero_out_perimeter: bool | None = None
    temporal_values_file: str | None = None
    ramp: bool = False
    rcr: dict | None = None        # Rp, C, Rd, Pd, Xo
    effective_direction: tuple | None = None


@dataclasses.dataclass
class LsSpec:
    type: str = "GMRES"
    preconditioner: str = "fsils"
    tolerance: float | None = None
    absolute_tolerance: float | None = None
    max_iterations: int | None = None
    krylov_space_dimension: int | None = None
    ns_gm_max_iterations: int | None = None
    ns_cg_max_iterations: int | None = None
    ns_gm_tolerance: float | None = None
    ns_cg_tolerance: float | None = None


@dataclasses.dataclass
class EquationSpec:
    type: str
    coupled: bool = True
    min_iterations: int = 1
    max_iterations: int = 5
    tolerance: float = 1e-6
    density: float | None = None
    viscosity: float | None = None
    backflow: float = 0.2
    domains: list = dataclasses.field(default_factory=list)
    ls: LsSpec = dataclasses.field(default_factory=LsSpec)
    bcs: list = dataclasses.field(default_factory=list)


@dataclasses.dataclass
class MeshSpec:
    name: str
    path: str
    faces: dict
    domain: int | None = None


@dataclasses.dataclass
class SolverConfig:
    n_time_steps: int
    dt: float
    rho_inf: float
    meshes: list
    equations: list
    base: str


def parse_solver_xml(path) -> SolverConfig:
    root = ET.parse(path).getroot()
    base = os.path.dirname(os.path.abspath(path))
    g = root.find("GeneralSimulationParameters")
    meshes = []
    for m in root.findall("Add_mesh"):
        faces = {f.get("name"): _text(f, "Face_file_path") for f in m.findall("Add_face")}
        meshes.append(MeshSpec(m.get("name"), _text(m, "Mesh_file_path"), faces, _text(m, "Domain", None, int)))
    eqs = []
    for e in root.findall("Add_equation"):
        visc = e.find("Viscosity")
        eq = EquationSpec(type=e.get("type"), coupled=_text(e, "Coupled", True, bool),
                          min_iterations=_text(e, "Min_iterations", 1, int),
                          max_iterations=_text(e, "Max_iterations", 5, int),
                          tolerance=_text(e, "Tolerance", 1e-6, float), density=_text(e, "Density", None, float),
                          viscosity=_text(visc, "Value", None, float) if visc is not None else None,
                          backflow=_text(e, "Backflow_stabilization_coefficient", 0.2, float))
        for d in e.findall("Domain"):
            dv = d.find("Viscosity")
            eq.domains.append(dict(id=int(d.get("id")), equation=_text(d, "Equation"),
                                   density=_text(d, "Density", None, float),
                                   viscosity=_text(dv, "Value", None, float) if dv is not None else None,
                                   E=_text(d, "Elasticity_modulus", None, float),
                                   nu=_text(d, "Poisson_ratio", None, float),
                                   backflow=_text(d, "Backflow_stabilization_coefficient", None, float)))
        ls = e.find("LS")
        if ls is not None:
            la = ls.find("Linear_algebra")
            eq.ls = LsSpec(type=ls.get("type", "GMRES"),
                           preconditioner=_text(la, "Preconditioner", "fsils") if la is not None else "fsils",
                           tolerance=_text(ls, "Tolerance", None, float),
                           absolute_tolerance=_text(ls, "Absolute_tolerance", None, float),
                           max_iterations=_text(ls, "Max_iterations", None, int),
                           krylov_space_dimension=_text(ls, "Krylov_space_dimension", None, int),
                           ns_gm_max_iterations=_text(ls, "NS_GM_max_iterations", None, int),
                           ns_cg_max_iterations=_text(ls, "NS_CG_max_iterations", None, int),
                           ns_gm_tolerance=_text(ls, "NS_GM_tolerance", None, float),
                           ns_cg_tolerance=_text(ls, "NS_CG_tolerance", None, float))
        for b in e.findall("Add_BC"):
            rcr = None
            r = b.find("RCR_values")
            if r is not None:
                rcr = dict(Rp=_text(r, "Proximal_resistance", 0.0, float), C=_text(r, "Capacitance", 0.0, float),
                           Rd=_text(r, "Distal_resistance", 0.0, float), Pd=_text(r, "Distal_pressure", 0.0, float),
                           Xo=_text(r, "Initial_pressure", 0.0, float))
            eq.bcs.append(BcSpec(name=b.get("name"), type=_text(b, "Type", "Dir"),
                                 time_dependence=_text(b, "Time_dependence", "Steady"),
                                 value=_text(b, "Value", 0.0, float), profile=_text(b, "Profile", "Flat"),
                                 impose_flux=_text(b, "Impose_flux", False, bool),
                                 zero_out_perimeter=_text(b, "Zero_out_perimeter", None, bool),
                                 temporal_values_file=_text(b, "Temporal_values_file_path"),
                                 ramp=_text(b, "Ramp_function", False, bool), rcr=rcr,
                                 effective_direction=_text(b, "Effective_direction", None, tuple)))
        eqs.append(eq)
    return SolverConfig(n_time_steps=_text(g, "Number_of_time_steps", 1, int),
                        dt=_text(g, "Time_step_size", 1e-3, float),
                        rho_inf=_text(g, "Spectral_radius_of_infinite_time_step", 0.5, float),
                        meshes=meshes, equations=eqs, base=base)


# ---------------------------------------------------------------- temporal values
@dataclasses.dataclass
class Fourier:
    """fcType (ComMod.h:63-103) for one scalar: Fourier coefficients of the part of a
    periodic signal left after its linear trend."""
    ti: float
    T: float
    qi: float
    qs: float
    r: np.ndarray
    i: np.ndarray
    lrmp: bool = False


def fourier_fit(t, q, n: int, lrmp: bool = False) -> Fourier:
    """fft (fft.cpp:36-95): the trend qi + qs t, and n coefficients of the remainder
    from exact integrals of its piecewise-linear interpolant."""
    t = np.asarray(t, dtype=np.float64).copy()
    q = np.asarray(q, dtype=np.float64).copy()
    np_ = t.size
    ti = t[0]
    T = t[np_ - 1] - t[0]
    qi = q[0]
    qs = (q[np_ - 1] - q[0]) / T
    for k in range(np_):
        t[k] = t[k] - ti
        q[k] = q[k] - qi - qs * t[k]
    if lrmp:
        n = 1
    r = np.zeros(n)
    im = np.zeros(n)
    for m in range(n):
        tmp = float(m)
        for k in range(np_ - 1):
            ko = 2.0 * math.pi * tmp * t[k] / T
            kn = 2.0 * math.pi * tmp * t[k + 1] / T
            s = (q[k + 1] - q[k]) / (t[k + 1] - t[k])
            if m == 0:
                r[m] = r[m] + 0.5 * (t[k + 1] - t[k]) * (q[k + 1] + q[k])
            else:
                r[m] = r[m] + s * (math.cos(kn) - math.cos(ko))
                im[m] = im[m] - s * (math.sin(kn) - math.sin(ko))
        if m == 0:
            r[m] = r[m] / T
        else:
            r[m] = 0.5 * r[m] * T / (math.pi * math.pi * tmp * tmp)
            im[m] = 0.5 * im[m] * T / (math.pi * math.pi * tmp * tmp)
    return Fourier(ti, T, qi, qs, r, im, lrmp)


def fourier_eval(f: Fourier, time: float):
    """ifft (fft.cpp:97-140): value and time derivative at `time`."""
    if f.lrmp:
        t = time - f.ti
        t = max(t, 0.0) if t <= 0.0 else min(t, f.T)
        return f.qi + t * f.qs, f.qs
    t = math.fmod(time - f.ti, f.T)
    tmp = 2.0 * math.pi / f.T
    Y = f.qi + t * f.qs
    dY = f.qs
    for k in range(f.r.size):
        dk = tmp * float(k)
        K = t * dk
        Y = Y + f.r[k] * math.cos(K) - f.i[k] * math.sin(K)
        dY = dY - (f.r[k] * math.sin(K) + f.i[k] * math.cos(K)) * dk
    return Y, dY


def read_temporal_values(path, lrmp=False) -> Fourier:
    """read_temporal_values (read_files.cpp:2577-2631): first line 'points modes', then
    'time value' pairs."""
    with open(path) as fh:
        head = fh.readline().split()
        npts, nmodes = int(head[0]), int(head[1])
        if npts < 2 or nmodes == 0:
            raise RuntimeError(f"Error reading the first line of the temporal values file '{path}'.")
        rows = [list(map(float, ln.split())) for ln in fh if ln.strip()]
    if any(len(r) != 2 for r in rows):
        raise RuntimeError(f"Error reading values for the temporal values file '{path}'.")
    rows = np.array(rows)
    return fourier_fit(rows[:npts, 0], rows[:npts, 1], nmodes, lrmp)


# ---------------------------------------------------------------- face geometry
def _tri_normals(x, tri, gE, ien):
    """gnnb's outward, area-weighted normals of face triangles (nn.cpp:727-760)."""
    p0, p1, p2 = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    n = np.cross(p0 - p2, p1 - p2)
    inner = np.array([[v for v in ien[e] if v not in t][0] for e, t in zip(gE, tri)])
    flip = np.einsum("ij,ij->i", n, p0 - x[inner]) < 0.0
    n[flip] *= -1.0
    return n


def face_nodal(x, face, ien):
    """sum_e sum_g N_a w_g n over a face (TRI3, three points): the nodal normal integrals
    (fsi_ls_ini's sV, baf_ini.cpp:738-775)."""
    n = _tri_normals(x, face.ien, face.gE, ien)
    s = 2.0 / 3.0
    t = -0.5 * s + 0.5
    xi = ((t, t), (s, t), (t, s))
    out = np.zeros((x.shape[0], 3))
    for g in range(3):
        N = (xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1])
        for a in range(3):
            np.add.at(out, face.ien[:, a], N[a] * (1.0 / 6.0) * n)
    return out


def face_integral(x, face, ien, s):
    """all_fun::integ of a nodal scalar over a face (all_fun.cpp:561-720)."""
    n = _tri_normals(x, face.ien, face.gE, ien)
    J = np.linalg.norm(n, axis=1)
    s2 = 2.0 / 3.0
    t = -0.5 * s2 + 0.5
    xi = ((t, t), (s2, t), (t, s2))
    tot = 0.0
    for g in range(3):
        N = (xi[g][0], xi[g][1], 1.0 - xi[g][0] - xi[g][1])
        sh = N[0] * s[face.ien[:, 0]] + N[1] * s[face.ien[:, 1]] + N[2] * s[face.ien[:, 2]]
        tot += float(np.sum((1.0 / 6.0) * J * sh))
    return tot


def bc_profile(mesh, face_name, bc: BcSpec):
    """gx of a Dirichlet/Neumann face (bc_ini, baf_ini.cpp:270-432): flat or parabolic,
    zero on the nodes other faces share (Dir default), divided by its face integral when
    the flux is imposed."""
    f = mesh.faces[face_name]
    x = mesh.x
    s = np.zeros(mesh.nNo)
    if bc.profile == "Parabolic":
        area = face_integral(x, f, mesh.ien, np.ones(mesh.nNo))
        center = np.array([face_integral(x, f, mesh.ien, x[:, i]) / area for i in range(3)])
        others = np.zeros(mesh.nNo, bool)
        for name, g in mesh.faces.items():
            if name != face_name:
                others[g.gN] = True
        perim = f.gN[others[f.gN]]
        if perim.size == 0:
            raise RuntimeError(f"Face '{face_name}' has no perimeter.")
        sV = x[perim] - center
        sVl = sV / np.sqrt(np.sum(sV * sV, axis=1))[:, None]
        nV = x[f.gN] - center
        i = np.argmax(nV @ sVl.T, axis=1)
        s[f.gN] = 1.0 - np.sum(nV * nV, axis=1) / np.sum(sV[i] * sV[i], axis=1)
    else:
        s[f.gN] = 1.0
    zp = bc.zero_out_perimeter if bc.zero_out_perimeter is not None else bc.type == "Dir"
    if zp:
        for name, g in mesh.faces.items():
            if name != face_name:
                s[g.gN] = 0.0
    tmp = 1.0
    if bc.impose_flux:
        tmp = face_integral(x, f, mesh.ien, s)
        if tmp == 0.0:
            raise RuntimeError(f"Face '{face_name}' used for a BC has no non-zero node.")
    return s[f.gN] / tmp


def face_unit_normals(mesh, face_name):
    """lFa.nV: the nodal normal integrals normalised (face_ini, baf_ini.cpp:470-520)."""
    f = mesh.faces[face_name]
    sV = face_nodal(mesh.x, f, mesh.ien)[f.gN]
    return sV / np.sqrt(np.sum(sV * sV, axis=1))[:, None]


# ---------------------------------------------------------------- the case driver
class FluidCase:
    """A fluid solver.xml case on the GPU through svgpu_fluid_step."""

    def __init__(self, xml_path, mesh=None, device=0, precision=api.SVGPU_FP64):
        cfg = parse_solver_xml(xml_path)
        self.cfg = cfg
        fluid = [e for e in cfg.equations if e.type == "fluid"]
        if len(cfg.equations) != 1 or not fluid:
            raise ValueError("FluidCase runs a single fluid equation")
        eq = self.eq = fluid[0]
        if mesh is None:
            if len(cfg.meshes) != 1:
                raise ValueError("FluidCase reads one mesh")
            ms = cfg.meshes[0]
            faces = {k: os.path.join(cfg.base, v) for k, v in ms.faces.items()}
            mesh = vtkio.load_mesh(os.path.join(cfg.base, ms.path), faces)
        self.mesh = mesh
        am, af, gam, beta = api.genalpha_first_order(cfg.rho_inf)
        self.props = api.FluidProps(eq.density if eq.density is not None else 1.0,
                                    eq.viscosity if eq.viscosity is not None else 0.0, (api.C.c_double * 3)(0, 0, 0),
                                    0.0, eq.backflow, cfg.dt, am, af, gam, beta)
        dirs = [b for b in eq.bcs if b.type == "Dir"]
        neus = [b for b in eq.bcs if b.type == "Neu"]
        if len(neus) > 1:
            raise ValueError("FluidCase supports one Neumann (outlet) face")
        rcr = neus[0].rcr if neus and neus[0].time_dependence == "RCR" else None
        self.ctx = api.Context(device)
        nNo = mesh.nNo
        rowPtr, colPtr = api.csr_pattern(nNo, mesh.ien)
        self.rowPtr, self.colPtr = rowPtr, colPtr
        nfaces = len(dirs) + (1 if rcr else 0)
        self.ctx.fsils_lhs_create(nNo, rowPtr, colPtr, nfaces)
        for k, b in enumerate(dirs):  # fsi_ls_ini order: the equation's BCs in turn
            self.ctx.fsils_bc_create(k, mesh.faces[b.name].gN, 3, api.BC_TYPE_Dir)
        ls = eq.ls
        ls_type = {"GMRES": api.LS_TYPE_GMRES, "CG": api.LS_TYPE_CG, "NS": api.LS_TYPE_NS}[ls.type]
        self.ctx.fsils_ls_create(ls_type, -1.0 if ls.tolerance is None else ls.tolerance,
                                 -1.0 if ls.absolute_tolerance is None else ls.absolute_tolerance,
                                 -1 if ls.max_iterations is None else ls.max_iterations,
                                 -1 if ls.krylov_space_dimension is None else ls.krylov_space_dimension)
        self.ctx.mesh_create(mesh.x, mesh.ien)
        outlet = -1
        self.outletH = 0.0
        if neus:
            f = mesh.faces[neus[0].name]
            self.ctx.face_create(api.FACE_OUTLET, f.ien, f.gE)
            outlet = api.FACE_OUTLET
            if rcr:
                self.ctx.rcr_create(api.FACE_OUTLET, len(dirs), rcr["Rp"], rcr["C"], rcr["Rd"], rcr["Pd"], rcr["Xo"],
                                    cfg.dt, 0.0)
            elif neus[0].time_dependence == "Steady":
                self.outletH = -neus[0].value  # hg = -h gx with a flat gx (set_bc.cpp:1402-1411)
            else:
                raise ValueError("Neumann face: Steady or RCR")
        # Dirichlet nodes in BC order; later faces overwrite shared nodes (set_bc_dir)
        self.dir_specs = []
        for b in dirs:
            gx = bc_profile(mesh, b.name, b)
            nV = face_unit_normals(mesh, b.name)
            four = None
            if b.time_dependence == "Unsteady":
                four = read_temporal_values(os.path.join(cfg.base, b.temporal_values_file), b.ramp)
            elif b.time_dependence != "Steady":
                raise ValueError(f"Dirichlet face {b.name}: Steady or Unsteady")
            self.dir_specs.append((mesh.faces[b.name].gN, gx, nV, b, four))
        nodes = np.unique(np.concatenate([s[0] for s in self.dir_specs])) if dirs else np.zeros(0, np.int32)
        self.dir_nodes = nodes.astype(np.int32)
        self.ctx.set_dirichlet(self.dir_nodes)
        self.opts = api.NewtonOpts(eq.min_iterations, eq.max_iterations, eq.tolerance, precision, outlet,
                                   self.outletH)
        z = lambda: np.zeros((nNo, 4))  # noqa: E731
        self.Ao, self.Yo, self.Do, self.An, self.Yn, self.Dn = z(), z(), z(), z(), z(), z()
        self.norms = [0.0, 0.0]
        self.time = 0.0
        self.cTS = 0

    def dirichlet_values(self, time):
        """set_bc_dir_l (set_bc.cpp:1005-1045): Y = g(t) gx nV, A = dg/dt gx nV per node."""
        pos = {int(a): k for k, a in enumerate(self.dir_nodes)}
        Y = np.zeros((self.dir_nodes.size, 3))
        A = np.zeros((self.dir_nodes.size, 3))
        for gN, gx, nV, b, four in self.dir_specs:
            if four is None:
                g, dg = b.value, 0.0
            else:
                g, dg = fourier_eval(four, time)
            idx = np.array([pos[int(a)] for a in gN])
            Y[idx] = (g * gx)[:, None] * nV
            A[idx] = (dg * gx)[:, None] * nV
        return Y, A

    def step(self):
        self.time += self.cfg.dt
        self.cTS += 1
        Y, A = self.dirichlet_values(self.time)
        st = self.ctx.fluid_step(self.props, self.opts, Y, A, self.Ao, self.Yo, self.Do, self.An, self.Yn, self.Dn,
                                 self.norms)
        self.Ao[:] = self.An
        self.Yo[:] = self.Yn
        return st

    def run(self, n_steps=None, vtu_prefix=None, save_every=0):
        """n_steps (default: the file's) time steps; with vtu_prefix, a result file every
        save_every steps (vtk_xml.cpp write_vtus' Velocity and Pressure)."""
        out = []
        for k in range(n_steps or self.cfg.n_time_steps):
            out.append(self.step())
            if vtu_prefix and save_every and self.cTS % save_every == 0:
                vtkio.write_vtu(f"{vtu_prefix}_{self.cTS:03d}.vtu", self.mesh.x, self.mesh.ien,
                                {"Velocity": self.Yn[:, :3], "Pressure": self.Yn[:, 3]})
        return out
