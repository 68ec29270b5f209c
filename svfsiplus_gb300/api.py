"""Python mirror of the reference interface over the svgpu C ABI (include/svgpu.h).

Names, argument meaning and error behaviour follow the reference:
``fsils_lhs_create`` (liner_solver/lhs.cpp:57), ``fsils_bc_create`` (bc.cpp:45),
``fsils_ls_create`` (ls.cpp:40), ``fsils_solve`` (solve.cpp:50), ``construct_fluid``
(solver/fluid.cpp:464), ``b_assem_neu_bc`` (eq_assem.cpp:58) and one fluid time step
of ``iterate_solution`` (main.cpp:292-762).  Errors raise ``RuntimeError`` with the
library's message, as the reference throws ``std::runtime_error``.

Arrays are numpy (host) or torch CUDA tensors (device); the library accepts either.
Layouts: node-major ``(nNo, dof)`` arrays are the reference's column-major
``Array<double>(dof, nNo)``; ``Val`` is ``(nnz, dof*dof)``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import mesh as _mesh

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsvgpu.so")

SVGPU_OK = 0
SVGPU_FP64, SVGPU_MIXED = 0, 1
BC_TYPE_Dir, BC_TYPE_Neu = 0, 1
LS_TYPE_GMRES = 2
LS_TYPE_CG = 3
LS_TYPE_NS = 4
PREC_NONE, PREC_FSILS = 0, 1

_lib = None


def lib():
    """Load libsvgpu.so.  There is no fallback: without the CUDA library nothing runs."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"svgpu CUDA library not built ({LIB_PATH}); run __graft_entry__.build()")
        _lib = C.CDLL(LIB_PATH)
        _lib.svgpu_last_error.restype = C.c_char_p
        _lib.svgpu_kernel_launches.restype = C.c_longlong
    return _lib


class LsStats(C.Structure):
    _fields_ = [("iNorm", C.c_double), ("fNorm", C.c_double), ("dB", C.c_double), ("callD", C.c_double),
                ("itr", C.c_int), ("suc", C.c_int), ("true_rel", C.c_double), ("x0_rel", C.c_double),
                ("x0_kept", C.c_int), ("pad_", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class FluidProps(C.Structure):
    _fields_ = [("rho", C.c_double), ("mu", C.c_double), ("f", C.c_double * 3), ("k_inv_darcy", C.c_double),
                ("backflow_beta", C.c_double), ("dt", C.c_double), ("am", C.c_double), ("af", C.c_double),
                ("gam", C.c_double), ("beta", C.c_double)]


class SolidProps(C.Structure):
    _fields_ = [("rho", C.c_double), ("damping", C.c_double), ("f", C.c_double * 3), ("C10", C.c_double),
                ("Kpen", C.c_double), ("volType", C.c_int), ("dt", C.c_double), ("am", C.c_double),
                ("af", C.c_double), ("gam", C.c_double), ("beta", C.c_double)]


def genalpha_second_order(rho_inf: float):
    """eq.am/af/gam/beta of a second-order equation (struct, mesh; initialize.cpp:426-465)."""
    am = (2.0 - rho_inf) / (1.0 + rho_inf)
    af = 1.0 / (1.0 + rho_inf)
    beta = 0.25 * (1.0 + am - af) ** 2
    gam = 0.5 + am - af
    return am, af, gam, beta


def solid_props(rho=1.2, E=1.0e6, nu=0.45, dt=1e-3, rho_inf=0.5, volType=1, damping=0.0):
    """Neo-Hookean solid from E, nu: C10 = mu/2, Kpen = bulk modulus."""
    am, af, gam, beta = genalpha_second_order(rho_inf)
    C10 = E / (4.0 * (1.0 + nu))
    Kpen = E / (3.0 * (1.0 - 2.0 * nu))
    return SolidProps(rho, damping, (C.c_double * 3)(0.0, 0.0, 0.0), C10, Kpen, volType, dt, am, af, gam, beta)


class FsiProps(C.Structure):
    _fields_ = [("fluid", FluidProps), ("solid", SolidProps), ("mesh_E", C.c_double), ("mesh_nu", C.c_double),
                ("mesh_rho", C.c_double), ("mesh_am", C.c_double), ("mesh_af", C.c_double),
                ("mesh_gam", C.c_double), ("mesh_beta", C.c_double)]


class FsiOpts(C.Structure):
    _fields_ = [("minItr", C.c_int * 2), ("maxItr", C.c_int * 2), ("tol", C.c_double * 2), ("lsType", C.c_int * 2),
                ("relTol", C.c_double * 2), ("absTol", C.c_double * 2), ("lsMaxItr", C.c_int * 2),
                ("dimKry", C.c_int * 2), ("incL", C.c_void_p * 2), ("outletFace", C.c_int), ("outletH", C.c_double),
                ("precision", C.c_int), ("reuse_tangent", C.c_int)]


class DirichletSet(C.Structure):
    _fields_ = [("n", C.c_int), ("nodes", C.c_void_p), ("Y", C.c_void_p), ("A", C.c_void_p)]


class NewtonOpts(C.Structure):
    _fields_ = [("minItr", C.c_int), ("maxItr", C.c_int), ("tol", C.c_double), ("precision", C.c_int),
                ("outletFace", C.c_int), ("outletH", C.c_double), ("reuse_tangent", C.c_int)]


def genalpha_first_order(rho_inf: float):
    """eq.am/af/gam/beta of a first-order equation (initialize.cpp:426-465)."""
    am = 0.5 * (3.0 - rho_inf) / (1.0 + rho_inf)
    af = 1.0 / (1.0 + rho_inf)
    beta = 0.25 * (1.0 + am - af) ** 2
    gam = 0.5 + am - af
    return am, af, gam, beta


def fluid_props(rho=1.06, mu=0.04, dt=1e-3, rho_inf=0.5, backflow_beta=0.2, k_inv_darcy=0.0, f=(0.0, 0.0, 0.0)):
    am, af, gam, beta = genalpha_first_order(rho_inf)
    return FluidProps(rho, mu, (C.c_double * 3)(*f), k_inv_darcy, backflow_beta, dt, am, af, gam, beta)


def _ptr(a):
    """Data pointer of a numpy array or a torch tensor (host or CUDA)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return C.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One svgpu context (a GPU and a stream): holds the FSILS handles, the mesh and
    the resident linear system."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().svgpu_create(C.byref(self._h), int(device))
        if rc != SVGPU_OK:
            raise RuntimeError(f"svgpu_create failed ({rc}): no usable CUDA device")

    def close(self):
        if self._h:
            lib().svgpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc < 0:
            msg = lib().svgpu_last_error(self._h).decode()
            raise RuntimeError(f"{what}: {msg} (status {rc})")
        return rc

    @property
    def kernel_launches(self) -> int:
        return int(lib().svgpu_kernel_launches(self._h))

    # ---- FSILS set-up
    def fsils_lhs_create(self, nNo, rowPtr, colPtr, nFaces):
        rowPtr = np.ascontiguousarray(rowPtr, dtype=np.int32)
        colPtr = np.ascontiguousarray(colPtr, dtype=np.int32)
        self.nNo, self.nnz = int(nNo), int(colPtr.size)
        self._check(lib().svgpu_lhs_create(self._h, self.nNo, self.nNo, self.nnz, None, _ptr(rowPtr), _ptr(colPtr),
                                           int(nFaces)), "fsils_lhs_create")

    def fsils_bc_create(self, faIn, gNodes, dof, bc_type, val=None):
        gNodes = np.ascontiguousarray(gNodes, dtype=np.int32)
        if val is not None:
            val = np.ascontiguousarray(val, dtype=np.float64)
        self._check(lib().svgpu_bc_create(self._h, int(faIn), int(gNodes.size), int(dof), int(bc_type),
                                          _ptr(gNodes), _ptr(val)), "fsils_bc_create")

    def fsils_ls_create(self, ls_type=LS_TYPE_GMRES, relTol=-1.0, absTol=-1.0, maxItr=-1, dimKry=-1):
        self._check(lib().svgpu_ls_create(self._h, int(ls_type), C.c_double(relTol), C.c_double(absTol),
                                          int(maxItr), int(dimKry)), "fsils_ls_create")

    def fsils_solve(self, dof, Ri, Val, prec=PREC_FSILS, incL=None, res=None) -> LsStats:
        """In place, as the reference: Ri residual -> increment, Val -> scaled Val."""
        st = LsStats()
        incL_a = None if incL is None else np.ascontiguousarray(incL, dtype=np.int32)
        res_a = None if res is None else np.ascontiguousarray(res, dtype=np.float64)
        self._check(lib().svgpu_fsils_solve(self._h, int(dof), _ptr(Ri), _ptr(Val), int(prec), _ptr(incL_a),
                                            _ptr(res_a), C.byref(st)), "fsils_solve")
        return st

    def spar_mul(self, dof, K, U, KU):
        self._check(lib().svgpu_spar_mul(self._h, int(dof), _ptr(K), _ptr(U), _ptr(KU)), "spar_mul")

    def spar_mul32(self, K, U, KU):
        """FP32 block SpMV (dof 4) on device tensors, enqueued on the library's stream."""
        self._check(lib().svgpu_spar_mul_f32(self._h, _ptr(K), _ptr(U), _ptr(KU)), "spar_mul_f32")

    # ---- mesh and assembly
    def mesh_create(self, x, ien):
        x = np.ascontiguousarray(x, dtype=np.float64)
        ien = np.ascontiguousarray(ien, dtype=np.int32)
        self._check(lib().svgpu_mesh_create(self._h, int(x.shape[0]), int(ien.shape[0]), 4, _ptr(ien), _ptr(x)),
                    "mesh_create")

    def face_create(self, face_id, fien, gE):
        fien = np.ascontiguousarray(fien, dtype=np.int32)
        gE = np.ascontiguousarray(gE, dtype=np.int32)
        self._check(lib().svgpu_face_create(self._h, int(face_id), int(gE.size), _ptr(fien), _ptr(gE)), "face_create")

    def construct_fluid(self, props, Ag, Yg, Bf=None, R=None, Val=None, precision=SVGPU_FP64):
        self._check(lib().svgpu_construct_fluid(self._h, C.byref(props), _ptr(Ag), _ptr(Yg), _ptr(Bf), _ptr(R),
                                                _ptr(Val), int(precision)), "construct_fluid")

    def mesh_domains(self, eId):
        eId = np.ascontiguousarray(eId, dtype=np.int32)
        self._check(lib().svgpu_mesh_domains(self._h, _ptr(eId)), "mesh_domains")

    def construct_fsi(self, fluid, solid, tDof, Ag, Yg, Dg, R, Val):
        self._check(lib().svgpu_construct_fsi(self._h, C.byref(fluid), C.byref(solid), int(tDof), _ptr(Ag), _ptr(Yg),
                                              _ptr(Dg), _ptr(R), _ptr(Val)), "construct_fsi")

    def construct_dsolid(self, props, dof, tDof, s, Ag, Yg, Dg, R, Val):
        self._check(lib().svgpu_construct_dsolid(self._h, C.byref(props), int(dof), int(tDof), int(s), _ptr(Ag),
                                                 _ptr(Yg), _ptr(Dg), _ptr(R), _ptr(Val)), "construct_dsolid")

    def construct_mesh(self, E, nu, rho, dt, rho_inf, tDof, s, Ag, Dg, Do, R, Val):
        am, af, gam, beta = genalpha_second_order(rho_inf)
        self._check(lib().svgpu_construct_mesh(self._h, *(C.c_double(v) for v in (E, nu, rho, dt, am, af, beta)),
                                               int(tDof), int(s), _ptr(Ag), _ptr(Dg), _ptr(Do), _ptr(R), _ptr(Val)),
                    "construct_mesh")

    def get_system(self, R=None, Val=None):
        """Copy the resident R (nNo,4) and Val (nnz,16) out as FP64."""
        self._check(lib().svgpu_get_system(self._h, _ptr(R), _ptr(Val)), "get_system")

    def b_assem_neu_bc(self, face_id, props, h, Yg, R=None, Val=None):
        self._check(lib().svgpu_neu_bc_fluid(self._h, int(face_id), C.byref(props), C.c_double(h), _ptr(Yg),
                                             _ptr(R), _ptr(Val)), "b_assem_neu_bc")

    def rcr_create(self, mesh_face, ls_face, Rp, Cap, Rd, Pd=0.0, Xo=0.0, dt=1e-3, Q0=0.0):
        """A coupled RCR outlet on mesh face `mesh_face` with linear-solver face `ls_face`
        (the reference's RCR Neumann BC, semi-implicit coupling); Cap is the capacitance."""
        self._check(lib().svgpu_rcr_create(self._h, int(mesh_face), int(ls_face),
                                           *(C.c_double(v) for v in (Rp, Cap, Rd, Pd, Xo, dt, Q0))), "rcr_create")

    def rcr_set_state(self, xo):
        """Set the RCR outlet's 0D state (a restart)."""
        self._check(lib().svgpu_rcr_set_state(self._h, C.c_double(xo)), "rcr_set_state")

    def rcr_state(self):
        """{xo, xn, P, Qo, Qn, r} of the RCR outlet after the last Newton iteration."""
        out = (C.c_double * 6)()
        self._check(lib().svgpu_rcr_state(self._h, out), "rcr_state")
        return dict(zip(("xo", "xn", "P", "Qo", "Qn", "r"), list(out)))

    def b_assem_neu_bc_ale(self, face_id, props, h, tDof, Yg, Do, R, Val):
        """b_assem_neu_bc on the moving mesh: face at x + Do(4..6), backflow relative to Yg(4..6)."""
        self._check(lib().svgpu_neu_bc_fluid_ale(self._h, int(face_id), C.byref(props), C.c_double(h), int(tDof),
                                                 _ptr(Yg), _ptr(Do), _ptr(R), _ptr(Val)), "b_assem_neu_bc_ale")

    # ---- learned preconditioner
    def gnn_create(self, node_features, seed=1):
        f = np.ascontiguousarray(node_features, dtype=np.float32)
        self._check(lib().svgpu_gnn_create(self._h, _ptr(f), C.c_ulonglong(seed)), "gnn_create")

    def gnn_params(self):
        n = lib().svgpu_gnn_param_count()
        p = np.zeros(n, dtype=np.float32)
        self._check(lib().svgpu_gnn_get_params(self._h, _ptr(p), n), "gnn_get_params")
        return p

    def gnn_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(lib().svgpu_gnn_set_params(self._h, _ptr(p), int(p.size)), "gnn_set_params")

    def gnn_apply(self, r, z, p=None):
        """z = the network's correction M(r, p) - p (p: the prior, or None)."""
        self._check(lib().svgpu_gnn_apply(self._h, _ptr(r), None if p is None else _ptr(np.ascontiguousarray(p)),
                                          _ptr(z)), "gnn_apply")

    def gnn_loss_grad(self, r, x, p=None):
        n = lib().svgpu_gnn_param_count()
        g = np.zeros(n, dtype=np.float32)
        loss = C.c_double()
        pp = None if p is None else _ptr(np.ascontiguousarray(p))
        self._check(lib().svgpu_gnn_loss_grad(self._h, _ptr(np.ascontiguousarray(r)), pp,
                                              _ptr(np.ascontiguousarray(x)), C.byref(loss), _ptr(g)),
                    "gnn_loss_grad")
        return loss.value, g

    def gnn_add_pair(self, r, x, p=None):
        pp = None if p is None else _ptr(np.ascontiguousarray(p))
        self._check(lib().svgpu_gnn_add_pair(self._h, _ptr(np.ascontiguousarray(r)), pp,
                                             _ptr(np.ascontiguousarray(x))), "gnn_add_pair")

    def gnn_collect(self, on=True):
        """Store the solves' triples: False off, True every solve, 2 only solves with a prior."""
        self._check(lib().svgpu_gnn_collect(self._h, int(on)), "gnn_collect")

    def gnn_eval(self):
        """Mean loss of the network over the stored triples."""
        loss = C.c_double()
        self._check(lib().svgpu_gnn_eval(self._h, C.byref(loss)), "gnn_eval")
        return loss.value

    def gnn_pair_count(self):
        """How many (residual, prior, increment) triples are stored."""
        return int(lib().svgpu_gnn_pair_count(self._h))

    def gnn_pairs(self):
        """The stored (residual, prior, increment) triples of the scaled system, oldest
        first; the prior is zero where a triple has none."""
        out = []
        for k in range(self.gnn_pair_count()):
            r, p, x = (np.zeros((self.nNo, 4)) for _ in range(3))
            self._check(lib().svgpu_gnn_get_pair(self._h, k, _ptr(r), _ptr(p), _ptr(x)), "gnn_get_pair")
            out.append((r, p, x))
        return out

    def history_slot(self, slot):
        self._check(lib().svgpu_history_slot(self._h, int(slot)), "history_slot")

    def history_clear(self):
        self._check(lib().svgpu_history_clear(self._h), "history_clear")

    @property
    def guess_stats(self):
        """(initial guesses tried, rejected, with the network's correction) of modes 4 and 5."""
        u, r, k = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self._check(lib().svgpu_guess_stats(self._h, C.byref(u), C.byref(r), C.byref(k)), "guess_stats")
        return u.value, r.value, k.value

    def gnn_train(self, iters, lr=1e-3):
        loss = C.c_double()
        self._check(lib().svgpu_gnn_train(self._h, int(iters), C.c_float(lr), C.byref(loss)), "gnn_train")
        return loss.value

    def set_solver_mode(self, mode):
        """0 plain GMRES + diagonal, 1 learned FGMRES, 2 multilevel FGMRES, 3 multilevel
        with the learned smoother, 4 multilevel with the learned initial guess (previous
        step's increment + network correction), 5 multilevel with the previous step's
        increment alone as initial guess (modes 1-5 act on the mixed-precision path)."""
        self._check(lib().svgpu_set_solver_mode(self._h, int(mode)), "set_solver_mode")

    def multilevel_options(self, omega=0.7, coarse_sweeps=30, coarsest_nodes=256, pre_sweeps=1):
        self._check(lib().svgpu_multilevel_options(self._h, C.c_double(omega), int(coarse_sweeps),
                                                   int(coarsest_nodes), int(pre_sweeps)), "multilevel_options")

    def multilevel_info(self):
        """[(nodes, blocks)] per level of the hierarchy of the last multilevel solve."""
        nl = C.c_int(0)
        nodes = (C.c_int * 16)()
        blocks = (C.c_longlong * 16)()
        self._check(lib().svgpu_multilevel_info(self._h, C.byref(nl), nodes, blocks, 16), "multilevel_info")
        return [(nodes[i], blocks[i]) for i in range(min(nl.value, 16))]

    @property
    def learned_rejects(self):
        lib().svgpu_learned_rejects.restype = C.c_longlong
        return int(lib().svgpu_learned_rejects(self._h))

    PHASES = ("assembly", "precond", "amg_setup", "learned_guess", "restart", "cycles", "other",
              "cycle_precond", "cycle_spmv", "cycle_ortho", "cycle_coarse", "vcycle_spmv", "vcycle_transfer",
              "mesh_equation")

    def phase_timing(self, on=True):
        self._check(lib().svgpu_phase_timing(self._h, int(bool(on))), "phase_timing")

    def phase_times(self):
        """Accumulated milliseconds and interval counts per phase since the last call."""
        n = len(self.PHASES)
        ms = (C.c_double * n)()
        cnt = (C.c_longlong * n)()
        self._check(lib().svgpu_phase_times(self._h, ms, cnt, n), "phase_times")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.PHASES)}

    def set_dirichlet(self, nodes):
        nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        self._check(lib().svgpu_set_dirichlet(self._h, int(nodes.size), _ptr(nodes)), "set_dirichlet")

    def fluid_step(self, props, opts, dirY, dirA, Ao, Yo, Do, An, Yn, Dn, norms):
        stats = (LsStats * max(1, opts.maxItr))()
        iN = C.c_double(norms[0])
        pN = C.c_double(norms[1])
        it = self._check(lib().svgpu_fluid_step(self._h, C.byref(props), C.byref(opts), _ptr(dirY), _ptr(dirA),
                                                _ptr(Ao), _ptr(Yo), _ptr(Do), _ptr(An), _ptr(Yn), _ptr(Dn),
                                                C.byref(iN), C.byref(pN), stats), "fluid_step")
        norms[0], norms[1] = iN.value, pN.value
        return [stats[i].as_dict() for i in range(it)]


    def set_predictor(self, kind):
        """svgpu_set_predictor: 0 picp, 1 the acceleration extrapolated from the last two steps."""
        self._check(lib().svgpu_set_predictor(self._h, int(kind)), "set_predictor")

    def step_device_ms(self):
        """Device milliseconds of the last fluid/FSI time step, between its inputs'
        arrival on the device and the copy-back of its outputs (svgpu_step_device_ms)."""
        ms = C.c_double()
        self._check(lib().svgpu_step_device_ms(self._h, C.byref(ms)), "step_device_ms")
        return ms.value

    def fsi_step(self, props, opts, dir_fsi, dir_mesh, Ao, Yo, Do, An, Yn, Dn, iNorm, pNorm):
        """svgpu_fsi_step: one coupled FSI + mesh-motion time step.  dir_* are
        (nodes, Y, A) triples; iNorm/pNorm are 2-element lists carried across steps.
        Returns [(equation, stats dict)] per Newton iteration."""
        cap = opts.maxItr[0] + opts.maxItr[1]
        stats = (LsStats * cap)()
        eqs = (C.c_int * cap)()
        keep = []

        def dset(d):
            nodes = np.ascontiguousarray(d[0], dtype=np.int32)
            Y = np.ascontiguousarray(d[1], dtype=np.float64)
            A = np.ascontiguousarray(d[2], dtype=np.float64)
            keep.extend((nodes, Y, A))
            return DirichletSet(int(nodes.size), _ptr(nodes), _ptr(Y), _ptr(A))

        dF, dM = dset(dir_fsi), dset(dir_mesh)
        iN = (C.c_double * 2)(*iNorm)
        pN = (C.c_double * 2)(*pNorm)
        n = self._check(lib().svgpu_fsi_step(self._h, C.byref(props), C.byref(opts), C.byref(dF), C.byref(dM),
                                             _ptr(Ao), _ptr(Yo), _ptr(Do), _ptr(An), _ptr(Yn), _ptr(Dn), iN, pN,
                                             stats, eqs), "fsi_step")
        iNorm[:] = list(iN)
        pNorm[:] = list(pN)
        return [(int(eqs[i]), stats[i].as_dict()) for i in range(n)]


# ------------------------------------------------------------------ host driver
FACE_INLET, FACE_WALL, FACE_OUTLET = 0, 1, 2


def rcr_integrate(Rp, C_, Rd, Pd, dt, xo, Qo, Qn):
    """RCR_Integ_X (set_bc.cpp:460-547) on the host: (xn, P)."""
    xn, P = C.c_double(), C.c_double()
    rc = lib().svgpu_rcr_integrate(*(C.c_double(v) for v in (Rp, C_, Rd, Pd, dt, xo, Qo, Qn)), C.byref(xn), C.byref(P))
    if rc != SVGPU_OK:
        raise RuntimeError(f"rcr_integrate failed ({rc})")
    return xn.value, P.value


def rcr_resistance(Rp, C_, Rd, Pd, dt, xo, Qo, Qn):
    """calc_der_cpl_bc's finite-difference dP/dQ (set_bc.cpp:50-240) on the host."""
    lib().svgpu_rcr_resistance.restype = C.c_double
    return float(lib().svgpu_rcr_resistance(*(C.c_double(v) for v in (Rp, C_, Rd, Pd, dt, xo, Qo, Qn))))


def restart_stamp(nEq, nNo, tDof, dFlag, nX=0, nMsh=1):
    """com_mod.stamp of a one-process run (initialize.cpp:497)."""
    return np.array([1, nEq, nMsh, nNo, nX, tDof, 1 if dFlag else 0], dtype=np.int32)


def write_restart(path, stamp, cTS, time, iNorm, Yn, An, Dn=None, xn=None, cpu_time=0.0):
    """The reference's restart file (output::write_restart) of one process.  Arrays are
    node-major (nNo, tDof) -- the reference's column-major (tDof, nNo)."""
    st = np.ascontiguousarray(stamp, dtype=np.int32)
    iN = np.ascontiguousarray(np.atleast_1d(iNorm), dtype=np.float64)
    x = None if xn is None else np.ascontiguousarray(np.atleast_1d(xn), dtype=np.float64)
    arr = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (Yn, An, Dn)]
    rc = lib().svgpu_write_restart(None, str(path).encode(), _ptr(st), int(cTS), C.c_double(time),
                                   C.c_double(cpu_time), _ptr(iN), _ptr(x), *(_ptr(a) for a in arr))
    if rc != SVGPU_OK:
        raise RuntimeError(f"write_restart failed ({rc}): {path}")


def read_restart(path, stamp):
    """init_from_bin (initialize.cpp:78-245): dict of cTS, time, cpu_time, iNorm, xo, Yo,
    Ao, Do for the given stamp; RuntimeError with the reference's message on a mismatch."""
    st = np.ascontiguousarray(stamp, dtype=np.int32)
    nEq, nNo, nX, tDof, dFlag = int(st[1]), int(st[3]), int(st[4]), int(st[5]), int(st[6])
    out = {"iNorm": np.zeros(nEq), "xo": np.zeros(max(nX, 1)), "Yo": np.zeros((nNo, tDof)),
           "Ao": np.zeros((nNo, tDof)), "Do": np.zeros((nNo, tDof)) if dFlag else None}
    cts, t, cpu = C.c_int(), C.c_double(), C.c_double()
    rc = lib().svgpu_read_restart(None, str(path).encode(), _ptr(st), C.byref(cts), C.byref(t), C.byref(cpu),
                                  _ptr(out["iNorm"]), _ptr(out["xo"]), _ptr(out["Yo"]), _ptr(out["Ao"]),
                                  _ptr(out["Do"]))
    if rc != SVGPU_OK:
        raise RuntimeError(_restart_error(path, st))
    out.update(cTS=cts.value, time=t.value, cpu_time=cpu.value)
    out["xo"] = out["xo"][:nX]
    return out


def _restart_error(path, stamp):
    """The reference's message for a restart file that does not fit (initialize.cpp:213-238)."""
    what = ["The number of processors ", "The number of equations ", "The number of meshes ", "The number of nodes ",
            "The number of ncplBC.x ", "The number of dof ", "The dFlag specification "]
    try:
        t = np.fromfile(path, dtype=np.int32, count=7)
    except OSError:
        return f"read_restart: cannot open {path}"
    for i in range(min(7, t.size)):
        if t[i] != stamp[i]:
            return f"{what[i]} {t[i]} read from '{path}' don't match."
    return f"read_restart: file too short: {path}"


class _PinnedHolder:
    """Owns one page-locked host allocation (svgpu_host_alloc) and frees it."""

    def __init__(self, nbytes):
        self.p = C.c_void_p()
        if lib().svgpu_host_alloc(C.c_size_t(nbytes), C.byref(self.p)) != SVGPU_OK:
            raise RuntimeError(f"svgpu_host_alloc: {nbytes} bytes of page-locked memory not available")

    def __del__(self):
        if self.p:
            lib().svgpu_host_free(self.p)
            self.p = C.c_void_p()


def pinned_zeros(shape, dtype=np.float64):
    """A zeroed numpy array in page-locked host memory: the host state of a time step
    then moves to and from the GPU without staging copies."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    h = _PinnedHolder(nbytes)
    buf = (C.c_char * max(nbytes, 1)).from_address(h.p.value)
    buf._holder = h  # the allocation lives as long as the array's buffer
    a = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)
    a[...] = 0
    return a


def csr_pattern(nNo: int, ien: np.ndarray):
    """lhsa (lhsa.cpp:153): rowPtr/colPtr of the element cliques, sorted columns
    (native svgpu_lhsa)."""
    ien = np.ascontiguousarray(ien, dtype=np.int32)
    rowPtr = np.zeros(nNo + 1, dtype=np.int32)
    nnz = C.c_longlong(0)
    rc = lib().svgpu_lhsa(int(nNo), int(ien.shape[0]), int(ien.shape[1]), _ptr(ien), _ptr(rowPtr), None,
                          C.byref(nnz))
    if rc != SVGPU_OK:
        raise RuntimeError("lhsa: bad connectivity or an isolated node")
    colPtr = np.zeros(nnz.value, dtype=np.int32)
    lib().svgpu_lhsa(int(nNo), int(ien.shape[0]), int(ien.shape[1]), _ptr(ien), _ptr(rowPtr), _ptr(colPtr),
                     C.byref(nnz))
    return rowPtr, colPtr


def dirichlet_nodes(mesh):
    """Velocity-Dirichlet nodes (inlet + wall) and the inlet profile (0 on walls)."""
    inlet, wall = mesh.faces["inlet"], mesh.faces["wall"]
    nodes = np.union1d(inlet.gN, wall.gN).astype(np.int32)
    prof = np.zeros(nodes.size)
    prof[np.searchsorted(nodes, inlet.gN)] = mesh.inlet_profile
    return nodes, prof


def inflow(prof, time, u_mean, u_amp, freq):
    """u_z = u_c(t) * profile on the inlet, u_c = u_mean + u_amp sin(2 pi f t); acceleration du_c/dt * profile."""
    w = 2.0 * np.pi * freq
    uc = u_mean + u_amp * np.sin(w * time)
    duc = u_amp * w * np.cos(w * time)
    dirY = np.zeros((prof.size, 3))
    dirA = np.zeros((prof.size, 3))
    dirY[:, 2] = uc * prof
    dirA[:, 2] = duc * prof
    return dirY, dirA


def pipe_node_features(mesh):
    """Static node features of the learned preconditioner: coordinates scaled to
    [-1, 1] (x/R, y/R, 2z/L - 1) and the normalised distance to the wall 1 - r/r_wall."""
    x = mesh.x
    f = np.zeros((mesh.nNo, 4), dtype=np.float32)
    f[:, 0] = x[:, 0] / mesh.radius
    f[:, 1] = x[:, 1] / mesh.radius
    f[:, 2] = 2.0 * x[:, 2] / mesh.length - 1.0
    r = np.hypot(x[:, 0], x[:, 1])
    wall = mesh.faces["wall"].gN
    # wall radius per axial layer and angle is not stored: use the largest radius of the
    # node's layer as r_wall (exact for the straight pipe)
    zkey = np.round(x[:, 2] * 1e6).astype(np.int64)
    rmax = {}
    for k, rr in zip(zkey[wall], r[wall]):
        rmax[k] = max(rmax.get(k, 0.0), rr)
    rw = np.array([rmax.get(k, mesh.radius) for k in zkey])
    f[:, 3] = np.clip(1.0 - r / rw, 0.0, 1.0)
    return f


class PipeFluidSolver:
    """The fluid pipe case on the GPU: CSR set-up (lhsa + fsils_lhs_create), Dirichlet
    faces (fsils_bc_create, baf_ini.cpp:719-744), the outlet face, GMRES settings, and
    time stepping through svgpu_fluid_step."""

    def __init__(self, mesh: _mesh.PipeMesh, props=None, device=0, sD=50, mItr=100, relTol=1e-8, absTol=1e-17,
                 newton_min=3, newton_max=3, newton_tol=1e-11, precision=SVGPU_FP64, rowPtr=None, colPtr=None,
                 ls_type=LS_TYPE_GMRES, rcr=None, reuse_tangent=False):
        """rcr: None for a traction-free outlet, or dict(Rp, C, Rd, Pd, Xo) for a coupled
        RCR outlet (linear-solver face 2)."""
        self.mesh = mesh
        self.props = props or fluid_props()
        self.ctx = Context(device)
        nNo = mesh.nNo
        if rowPtr is None:
            rowPtr, colPtr = csr_pattern(nNo, mesh.ien)
        self.rowPtr, self.colPtr = rowPtr, colPtr
        self.ctx.fsils_lhs_create(nNo, rowPtr, colPtr, 3 if rcr else 2)
        self.ctx.fsils_bc_create(0, mesh.faces["inlet"].gN, 3, BC_TYPE_Dir)
        self.ctx.fsils_bc_create(1, mesh.faces["wall"].gN, 3, BC_TYPE_Dir)
        self.ctx.fsils_ls_create(ls_type, relTol, absTol, mItr, sD)
        self.ctx.mesh_create(mesh.x, mesh.ien)
        out = mesh.faces["outlet"]
        self.ctx.face_create(FACE_OUTLET, out.ien, out.gE)
        if rcr:
            self.ctx.rcr_create(FACE_OUTLET, 2, rcr["Rp"], rcr["C"], rcr["Rd"], rcr.get("Pd", 0.0), rcr.get("Xo", 0.0),
                                self.props.dt, 0.0)
        self.dir_nodes, self.dir_prof = dirichlet_nodes(mesh)
        self.ctx.set_dirichlet(self.dir_nodes)
        self.opts = NewtonOpts(newton_min, newton_max, newton_tol, precision, FACE_OUTLET, 0.0, int(reuse_tangent))
        z = lambda: pinned_zeros((nNo, 4))  # noqa: E731
        self.Ao, self.Yo, self.Do, self.An, self.Yn, self.Dn = z(), z(), z(), z(), z(), z()
        self.norms = [0.0, 0.0]
        self.time = 0.0
        self.cTS = 0
        self.has_rcr = bool(rcr)

    def _stamp(self):
        return restart_stamp(1, self.mesh.nNo, 4, False, nX=1 if self.has_rcr else 0)

    def save_restart(self, path):
        """The reference's restart file of the current state (output::write_restart)."""
        xn = self.ctx.rcr_state()["xo"] if self.has_rcr else None
        write_restart(path, self._stamp(), self.cTS, self.time, [self.norms[0]], self.Yo, self.Ao, xn=xn)

    def load_restart(self, path):
        """Continue from a restart file (init_from_bin): state, time, step count, the
        equation's iNorm and the 0D state."""
        r = read_restart(path, self._stamp())
        self.Yo[:], self.Ao[:] = r["Yo"], r["Ao"]
        self.time, self.cTS = r["time"], r["cTS"]
        self.norms[0] = float(r["iNorm"][0])
        if self.has_rcr:
            self.ctx.rcr_set_state(float(r["xo"][0]))

    def enable_learning(self, seed=1, collect=2):
        """Create the learned preconditioner and start collecting the solves'
        (residual, prior, increment) triples (2: only solves with a prior)."""
        self.ctx.gnn_create(pipe_node_features(self.mesh), seed)
        self.ctx.gnn_collect(collect)

    def step(self, u_mean=10.0, u_amp=0.0, freq=1.0):
        self.time += self.props.dt
        self.cTS += 1
        dirY, dirA = inflow(self.dir_prof, self.time, u_mean, u_amp, freq)
        stats = self.ctx.fluid_step(self.props, self.opts, dirY, dirA, self.Ao, self.Yo, self.Do,
                                    self.An, self.Yn, self.Dn, self.norms)
        # the new state is the next step's old state: Ao/Yo become the same page-locked
        # arrays as An/Yn instead of copies of them (fluid_step reads every input before
        # it writes an output, so in and out may be one array)
        self.Ao = self.An
        self.Yo = self.Yn
        return stats


# Linear-solver faces of the FSI pipe, numbered as the reference's fsi_ls_ini numbers
# them (baf_ini.cpp:190-227 over the FSI equation's BCs, then the mesh equation's, then
# the structure-node face): 0 lumen inlet, 1 wall inlet ring, 2 wall outlet ring (FSI
# Dirichlet), 3 unused (the outlet's plain Neumann BC has no face), 4 lumen inlet,
# 5 lumen outlet (mesh Dirichlet), 6 every node of the solid domain (mesh).
FSI_LS_FACES = 7
FSI_INCL = (np.array([1, 1, 1, 0, 0, 0, 0], np.int32), np.array([0, 0, 0, 0, 1, 1, 1], np.int32))


def fsi_props(rho_f=1.06, mu=0.04, backflow_beta=0.2, rho_s=1.2, E=1.0e6, nu=0.45, dt=1e-3, rho_inf=0.5,
              mesh_E=1.0, mesh_nu=0.3, mesh_rho=0.0, volType=1):
    """Both domains of the FSI equation carry its first-order constants
    (initialize.cpp:424-430); the mesh equation is second order."""
    fp = fluid_props(rho=rho_f, mu=mu, dt=dt, rho_inf=rho_inf, backflow_beta=backflow_beta)
    sp = solid_props(rho_s, E, nu, dt, rho_inf, volType)
    sp.am, sp.af, sp.gam, sp.beta = fp.am, fp.af, fp.gam, fp.beta
    mam, maf, mgam, mbeta = genalpha_second_order(rho_inf)
    return FsiProps(fp, sp, mesh_E, mesh_nu, mesh_rho, mam, maf, mgam, mbeta)


class PipeFsiSolver:
    """The FSI pipe case on the GPU (lumen plus a neo-Hookean wall annulus, linear-elastic
    mesh motion): CSR set-up, the element domains, the linear-solver faces of both
    equations (FSI_LS_FACES), the outlet face, and time stepping through svgpu_fsi_step
    with parabolic pulsatile inflow, fixed wall rings and no mesh motion at the lumen
    ends."""

    def __init__(self, mesh: _mesh.PipeMesh, props=None, device=0, newton=(3, 3, 1e-11), mesh_newton=(3, 3, 1e-11),
                 gmres=(1e-10, 1e-17, 100, 50), cg=(1e-10, 1e-17, 2000), rowPtr=None, colPtr=None,
                 precision=SVGPU_FP64, mesh_gmres=None):
        """mesh_gmres (relTol, absTol, restarts, Krylov dimension): solve the mesh equation
        by GMRES instead of CG (with precision SVGPU_MIXED: the mixed multilevel FGMRES)."""
        if mesh.eid is None:
            raise ValueError("PipeFsiSolver needs an FSI pipe (mesh.make_pipe with nrs > 0)")
        self.mesh = mesh
        self.props = props or fsi_props()
        self.ctx = Context(device)
        nNo = mesh.nNo
        if rowPtr is None:
            rowPtr, colPtr = csr_pattern(nNo, mesh.ien)
        self.rowPtr, self.colPtr = rowPtr, colPtr
        F = mesh.faces
        self.ctx.fsils_lhs_create(nNo, rowPtr, colPtr, FSI_LS_FACES)
        solid = np.zeros(nNo, bool)
        solid[mesh.ien[mesh.eid == 2].ravel()] = True
        self.solid_nodes = np.nonzero(solid)[0].astype(np.int32)
        for fa, name in ((0, "inlet"), (1, "wall_inlet"), (2, "wall_outlet"), (4, "inlet"), (5, "outlet")):
            self.ctx.fsils_bc_create(fa, F[name].gN, 3, BC_TYPE_Dir)
        self.ctx.fsils_bc_create(6, self.solid_nodes, 3, BC_TYPE_Dir)
        self.ctx.fsils_ls_create(LS_TYPE_GMRES, *gmres)
        self.ctx.mesh_create(mesh.x, mesh.ien)
        self.ctx.mesh_domains(mesh.eid)
        self.ctx.face_create(FACE_OUTLET, F["outlet"].ien, F["outlet"].gE)
        self.opts = FsiOpts()
        for q, (mn, mx, tol) in enumerate((newton, mesh_newton)):
            self.opts.minItr[q], self.opts.maxItr[q], self.opts.tol[q] = mn, mx, tol
        self.opts.lsType[0] = LS_TYPE_GMRES
        self.opts.relTol[0], self.opts.absTol[0], self.opts.lsMaxItr[0], self.opts.dimKry[0] = gmres
        if mesh_gmres:
            self.opts.lsType[1] = LS_TYPE_GMRES
            self.opts.relTol[1], self.opts.absTol[1], self.opts.lsMaxItr[1], self.opts.dimKry[1] = mesh_gmres
        else:
            self.opts.lsType[1] = LS_TYPE_CG
            self.opts.relTol[1], self.opts.absTol[1], self.opts.lsMaxItr[1] = cg
            self.opts.dimKry[1] = -1
        self._incl = FSI_INCL
        self.opts.incL[0] = self._incl[0].ctypes.data
        self.opts.incL[1] = self._incl[1].ctypes.data
        self.opts.outletFace, self.opts.outletH = FACE_OUTLET, 0.0
        self.opts.precision = precision
        # FSI Dirichlet nodes: wall rings (zero) and the lumen inlet (profile, 0 on the ring)
        rings = np.union1d(F["wall_inlet"].gN, F["wall_outlet"].gN)
        self.dirF = np.union1d(rings, F["inlet"].gN).astype(np.int32)
        self.profF = np.zeros(self.dirF.size)
        inl = np.searchsorted(self.dirF, F["inlet"].gN)
        self.profF[inl] = mesh.inlet_profile
        self.dirM = np.union1d(F["inlet"].gN, F["outlet"].gN).astype(np.int32)
        z = lambda: pinned_zeros((nNo, 7))  # noqa: E731
        self.Ao, self.Yo, self.Do, self.An, self.Yn, self.Dn = z(), z(), z(), z(), z(), z()
        self.iNorm, self.pNorm = [0.0, 0.0], [0.0, 0.0]
        self.time = 0.0
        self.cTS = 0

    def save_restart(self, path):
        """The reference's restart file (two equations, tDof 7, dFlag)."""
        write_restart(path, restart_stamp(2, self.mesh.nNo, 7, True), self.cTS, self.time, self.iNorm, self.Yo,
                      self.Ao, Dn=self.Do)

    def load_restart(self, path):
        r = read_restart(path, restart_stamp(2, self.mesh.nNo, 7, True))
        self.Yo[:], self.Ao[:], self.Do[:] = r["Yo"], r["Ao"], r["Do"]
        self.time, self.cTS = r["time"], r["cTS"]
        self.iNorm[:] = [float(v) for v in r["iNorm"]]

    def step(self, u_mean=15.0, u_amp=5.0, freq=1.0):
        self.time += self.props.fluid.dt
        self.cTS += 1
        dY, dA = inflow(self.profF, self.time, u_mean, u_amp, freq)
        zm = np.zeros((self.dirM.size, 3))
        stats = self.ctx.fsi_step(self.props, self.opts, (self.dirF, dY, dA), (self.dirM, zm, zm), self.Ao, self.Yo,
                                  self.Do, self.An, self.Yn, self.Dn, self.iNorm, self.pNorm)
        # the new state becomes the old one by reference (see PipeFluidSolver.step)
        self.Ao = self.An
        self.Yo = self.Yn
        self.Do = self.Dn
        return stats
