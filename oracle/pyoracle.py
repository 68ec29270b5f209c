"""ctypes binding of the C oracle (svoracle.c) -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker / CPU baseline; the GPU product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, -ffp-contract=off so results match across hosts), with
    OpenMP for the threaded CPU baseline where the compiler has it (one thread, the
    default, is the reference's sequential order either way)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "svoracle.c")
    hdr = os.path.join(HERE, "svoracle.h")
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr))
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        base = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"]
        if subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True).returncode != 0:
            subprocess.run(base, check=True)
    return LIB_PATH


class FluidParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("rho", "mu", "fx", "fy", "fz", "k_inv_darcy", "backflow_beta",
                 "dt", "am", "af", "gam", "beta")]


class StructParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("rho", "damping", "fx", "fy", "fz", "C10", "Kpen")] + \
               [("volType", C.c_int)] + [(n, C.c_double) for n in ("dt", "am", "af", "gam", "beta")]


def genalpha_second_order(rho_inf):
    am = (2.0 - rho_inf) / (1.0 + rho_inf)
    af = 1.0 / (1.0 + rho_inf)
    beta = 0.25 * (1.0 + am - af) ** 2
    gam = 0.5 + am - af
    return am, af, gam, beta


def struct_params(rho, E, nu, C10, Kpen, dt, rho_inf, volType=1):
    am, af, gam, beta = genalpha_second_order(rho_inf)
    return StructParams(rho, 0.0, 0.0, 0.0, 0.0, C10, Kpen, volType, dt, am, af, gam, beta)


def construct_struct(P, x, ien, A, Y, D, rowPtr, colPtr):
    nNo = x.shape[0]
    R = np.zeros((nNo, 3))
    Val = np.zeros((colPtr.size, 9))
    rc = lib().or_construct_struct(C.byref(P), nNo, ien.shape[0], _p(np.ascontiguousarray(ien, dtype=np.int32)),
                                   _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(A)),
                                   _p(np.ascontiguousarray(Y)), _p(np.ascontiguousarray(D)),
                                   _p(rowPtr), _p(colPtr), _p(R), _p(Val))
    if rc != 0:
        raise RuntimeError("zero Jacobian")
    return R, Val


def construct_mesh(E, nu, rho, dt, rho_inf, x, ien, A, D, Do, rowPtr, colPtr):
    am, af, gam, beta = genalpha_second_order(rho_inf)
    nNo = x.shape[0]
    R = np.zeros((nNo, 3))
    Val = np.zeros((colPtr.size, 9))
    rc = lib().or_construct_mesh(*(C.c_double(v) for v in (E, nu, rho, dt, am, af, beta)), nNo, ien.shape[0],
                                 _p(np.ascontiguousarray(ien, dtype=np.int32)), _p(np.ascontiguousarray(x)),
                                 _p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(D)),
                                 _p(np.ascontiguousarray(Do)), _p(rowPtr), _p(colPtr), _p(R), _p(Val))
    if rc != 0:
        raise RuntimeError("zero Jacobian")
    return R, Val


class LS(C.Structure):
    _fields_ = [("sD", C.c_int), ("mItr", C.c_int), ("relTol", C.c_double), ("absTol", C.c_double),
                ("iNorm", C.c_double), ("fNorm", C.c_double), ("dB", C.c_double),
                ("itr", C.c_int), ("suc", C.c_int), ("t_precond", C.c_double), ("t_krylov", C.c_double)]


class FluidProblem(C.Structure):
    _fields_ = [("nNo", C.c_int), ("nEl", C.c_int), ("nFa", C.c_int),
                ("ien", C.c_void_p), ("x", C.c_void_p), ("fien", C.c_void_p), ("fgE", C.c_void_p),
                ("rowPtr", C.c_void_p), ("colPtr", C.c_void_p), ("nnz", C.c_long),
                ("nDir", C.c_int), ("dirNodes", C.c_void_p), ("dirMask", C.c_void_p),
                ("minItr", C.c_int), ("maxItr", C.c_int), ("tol", C.c_double)]


class NewtonState(C.Structure):
    _fields_ = [("iNorm", C.c_double), ("pNorm", C.c_double),
                ("t_assembly", C.c_double), ("t_solve", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.or_lhsa.restype = C.c_long
        _lib.or_construct_fluid.restype = C.c_int
        _lib.or_fluid_element.restype = C.c_int
        _lib.or_fluid_step.restype = C.c_int
        _lib.or_dot.restype = C.c_double
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def fluid_params(rho=1.06, mu=0.04, dt=1e-3, rho_inf=0.5, backflow_beta=0.2, k_inv_darcy=0.0,
                 f=(0.0, 0.0, 0.0)) -> FluidParams:
    am, af, gam, beta = (C.c_double() for _ in range(4))
    lib().or_genalpha_first_order(C.c_double(rho_inf), C.byref(am), C.byref(af), C.byref(gam), C.byref(beta))
    return FluidParams(rho, mu, f[0], f[1], f[2], k_inv_darcy, backflow_beta, dt,
                       am.value, af.value, gam.value, beta.value)


def set_threads(n: int) -> int:
    """Host threads of the oracle's loops (n < 1: every processor); returns the count in
    use.  1 is the reference's sequential order, bit for bit."""
    return int(lib().or_set_threads(int(n)))


def color_elements(nNo: int, ien: np.ndarray):
    """Greedy element colouring: (perm, color_start) for construct_fluid_coloured."""
    ien = np.ascontiguousarray(ien, dtype=np.int32)
    perm = np.zeros(ien.shape[0], dtype=np.int32)
    start = np.zeros(129, dtype=np.int32)
    nc = lib().or_color_elements(int(nNo), int(ien.shape[0]), _p(ien), _p(perm), _p(start))
    if nc < 0:
        raise RuntimeError("more than 128 element colours")
    return perm, start[:nc + 1].copy()


def construct_fluid_coloured(P, x, ien, Ag, Yg, rowPtr, colPtr, perm, color_start, R=None, Val=None):
    """construct_fluid over the elements colour by colour, threads inside a colour."""
    nNo = x.shape[0]
    R = np.zeros((nNo, 4)) if R is None else R
    Val = np.zeros((colPtr.size, 16)) if Val is None else Val
    x, ien, Ag, Yg = (np.ascontiguousarray(a) for a in (x, ien, Ag, Yg))
    rc = lib().or_construct_fluid_coloured(C.byref(P), nNo, ien.shape[0], _p(ien), _p(x), _p(Ag), _p(Yg),
                                           _p(rowPtr), _p(colPtr), _p(R), _p(Val), _p(perm), _p(color_start),
                                           int(color_start.size - 1))
    if rc != 0:
        raise RuntimeError(f"zero Jacobian in element {-1 - rc}")
    return R, Val


def lhsa(nNo: int, ien: np.ndarray):
    ien = np.ascontiguousarray(ien, dtype=np.int32)
    rowPtr = np.zeros(nNo + 1, dtype=np.int32)
    nnz = lib().or_lhsa(nNo, ien.shape[0], ien.shape[1], _p(ien), _p(rowPtr), None)
    colPtr = np.zeros(nnz, dtype=np.int32)
    lib().or_lhsa(nNo, ien.shape[0], ien.shape[1], _p(ien), _p(rowPtr), _p(colPtr))
    return rowPtr, colPtr


def construct_fluid(P, x, ien, Ag, Yg, rowPtr, colPtr, R=None, Val=None):
    nNo = x.shape[0]
    R = np.zeros((nNo, 4)) if R is None else R
    Val = np.zeros((colPtr.size, 16)) if Val is None else Val
    x, ien, Ag, Yg = (np.ascontiguousarray(a) for a in (x, ien, Ag, Yg))
    rc = lib().or_construct_fluid(C.byref(P), nNo, ien.shape[0], _p(ien), _p(x), _p(Ag), _p(Yg), None,
                                  _p(rowPtr), _p(colPtr), _p(R), _p(Val))
    if rc != 0:
        raise RuntimeError(f"zero Jacobian in element {-1 - rc}")
    return R, Val


def fluid_element(P, xl, al, yl, bfl=None):
    lR = np.zeros(16)
    lK = np.zeros(256)
    bfl = np.zeros(12) if bfl is None else np.ascontiguousarray(bfl, dtype=np.float64)
    xl, al, yl = (np.ascontiguousarray(a, dtype=np.float64) for a in (xl, al, yl))
    rc = lib().or_fluid_element(C.byref(P), _p(xl), _p(al), _p(yl), _p(bfl), _p(lR), _p(lK))
    if rc != 0:
        raise RuntimeError("zero Jacobian")
    return lR.reshape(4, 4), lK.reshape(4, 4, 16)  # lR[a, i], lK[b, a, i]


def neu_backflow(P, fien, fgE, ien, x, Yg, rowPtr, colPtr, R, Val, h=0.0):
    fien, fgE = (np.ascontiguousarray(a, dtype=np.int32) for a in (fien, fgE))
    lib().or_neu_backflow(C.byref(P), fien.shape[0], _p(fien), _p(fgE), _p(ien), _p(x), _p(Yg),
                          C.c_double(h), _p(rowPtr), _p(colPtr), _p(R), _p(Val))


def spar_mul(rowPtr, colPtr, K, U, dof=4):
    nNo = rowPtr.size - 1
    KU = np.zeros((nNo, dof))
    lib().or_spar_mul(nNo, dof, _p(rowPtr), _p(colPtr), _p(np.ascontiguousarray(K)),
                      _p(np.ascontiguousarray(U)), _p(KU))
    return KU


def dot(u, v):
    return lib().or_dot(C.c_long(u.size), _p(u), _p(v))


def axpy(r, U, V):
    lib().or_axpy(C.c_long(U.size), C.c_double(r), _p(U), _p(V))


def fsils_solve_gmres(rowPtr, colPtr, Val, R, dirMask, sD=50, mItr=100, relTol=1e-8, absTol=1e-17, dof=4):
    """Returns (increment, scaled Val, LS stats). Val and R are copied, not modified."""
    nNo = rowPtr.size - 1
    Val = np.array(Val, dtype=np.float64, order="C", copy=True)
    R = np.array(R, dtype=np.float64, order="C", copy=True)
    ls = LS(sD, mItr, relTol, absTol, 0.0, 0.0, 0.0, 0, 0, 0.0, 0.0)
    mask = None if dirMask is None else _p(np.ascontiguousarray(dirMask, dtype=np.float64))
    lib().or_fsils_solve_gmres(nNo, dof, _p(rowPtr), _p(colPtr), _p(Val), _p(R), mask, C.byref(ls))
    return R, Val, ls


def fsils_solve_cg(rowPtr, colPtr, Val, R, dirMask, mItr=1000, relTol=1e-2, absTol=1e-10, dof=3):
    """fsils_solve with LS_TYPE_CG; returns (increment, scaled Val, LS stats)."""
    nNo = rowPtr.size - 1
    Val = np.array(Val, dtype=np.float64, order="C", copy=True)
    R = np.array(R, dtype=np.float64, order="C", copy=True)
    ls = LS(0, mItr, relTol, absTol, 0.0, 0.0, 0.0, 0, 0, 0.0, 0.0)
    mask = None if dirMask is None else _p(np.ascontiguousarray(dirMask, dtype=np.float64))
    lib().or_fsils_solve_cg(nNo, dof, _p(rowPtr), _p(colPtr), _p(Val), _p(R), mask, C.byref(ls))
    return R, Val, ls


class FluidRun:
    """The reference's fluid time loop on one pipe mesh (oracle side)."""

    def __init__(self, mesh, P, sD=50, mItr=100, relTol=1e-8, absTol=1e-17,
                 newton_min=3, newton_max=3, newton_tol=1e-11):
        self.mesh = mesh
        self.P = P
        nNo = mesh.nNo
        self.x = np.ascontiguousarray(mesh.x, dtype=np.float64)
        self.ien = np.ascontiguousarray(mesh.ien, dtype=np.int32)
        self.rowPtr, self.colPtr = lhsa(nNo, self.ien)
        out = mesh.faces["outlet"]
        self.fien = np.ascontiguousarray(out.ien, dtype=np.int32)
        self.fgE = np.ascontiguousarray(out.gE, dtype=np.int32)
        self.dir_nodes, self.dir_prof = dirichlet_nodes(mesh)
        self.dirMask = np.ones((nNo, 4))
        self.dirMask[self.dir_nodes, 0:3] = 0.0
        self.pb = FluidProblem(nNo, mesh.nEl, self.fien.shape[0], _p(self.ien).value, _p(self.x).value,
                               _p(self.fien).value, _p(self.fgE).value, _p(self.rowPtr).value,
                               _p(self.colPtr).value, self.colPtr.size, self.dir_nodes.size,
                               _p(self.dir_nodes).value, _p(self.dirMask).value,
                               newton_min, newton_max, newton_tol)
        self.ls = LS(sD, mItr, relTol, absTol, 0.0, 0.0, 0.0, 0, 0, 0.0, 0.0)
        self.ns = NewtonState(0.0, 0.0, 0.0, 0.0)
        self.newton_max = newton_max
        z = lambda: np.zeros((nNo, 4))  # noqa: E731
        self.Ao, self.Yo, self.Do, self.An, self.Yn, self.Dn = z(), z(), z(), z(), z(), z()
        self.time = 0.0

    def step(self, u_mean=10.0, u_amp=0.0, freq=1.0):
        self.time += self.P.dt
        dirY, dirA = dirichlet_values(self.dir_prof, self.time, u_mean, u_amp, freq)
        stats = np.zeros(5 * self.newton_max)
        it = lib().or_fluid_step(C.byref(self.pb), C.byref(self.P), C.byref(self.ls), C.byref(self.ns),
                                 _p(dirY), _p(dirA), _p(self.Ao), _p(self.Yo), _p(self.Do),
                                 _p(self.An), _p(self.Yn), _p(self.Dn), _p(stats))
        self.Ao[:] = self.An
        self.Yo[:] = self.Yn
        return stats[:5 * it].reshape(it, 5)


def dirichlet_nodes(mesh):
    """Velocity-Dirichlet nodes: wall and inlet; profile value per node (0 on walls)."""
    inlet, wall = mesh.faces["inlet"], mesh.faces["wall"]
    nodes = np.union1d(inlet.gN, wall.gN).astype(np.int32)
    prof = np.zeros(nodes.size)
    pos = np.searchsorted(nodes, inlet.gN)
    prof[pos] = mesh.inlet_profile
    return nodes, prof


def dirichlet_values(prof, time, u_mean, u_amp, freq):
    w = 2.0 * np.pi * freq
    uc = u_mean + u_amp * np.sin(w * time)
    duc = u_amp * w * np.cos(w * time)
    dirY = np.zeros((prof.size, 3))
    dirA = np.zeros((prof.size, 3))
    dirY[:, 2] = uc * prof
    dirA[:, 2] = duc * prof
    return dirY, dirA
