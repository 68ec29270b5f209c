"""Generate the golden fixtures by running the reference solver itself.

The reference's own fluid hot path (construct_fluid, b_assem_neu_bc, fsils_solve,
pic*) is compiled from the reference tree by ``oracle/build_ref.sh`` into
``oracle/_ref/ref_harness``; this script writes a procedural pipe case for it, runs
it, and stores what it produced as compressed ``.npz`` fixtures next to this file.
It needs the reference tree and is run only where that exists; the fixtures are
committed so the tests do not need it.

Usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from svfsiplus_gb300.mesh import named_pipe  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# Physics and solver settings of the pipe cases (fluid rho=1.06, mu=0.04, backflow 0.2,
# gen-alpha rho_inf=0.5, dt=1e-3, GMRES + diagonal preconditioner).
BASE = dict(rho=1.06, mu=0.04, backflow_beta=0.2, dt=1e-3, rho_inf=0.5,
            ls_rel_tol=1e-8, ls_abs_tol=1e-17, ls_max_itr=100, ls_krylov_dim=50,
            newton_min=3, newton_max=3, newton_tol=1e-11,
            u_mean=10.0, u_amp=0.0, u_freq=1.0)

CASES = {
    # element-level assembly + one solve on a tiny pipe: Val/R committed in full
    "tiny": dict(mesh="tiny", n_steps=2, dump_step=2, dump_iter=2),
    "small": dict(mesh="small", n_steps=3, dump_step=1, dump_iter=1, u_amp=5.0),
    # the CPU-runnable 50k-tet pipe, 10 time steps, fields after every step
    "pipe50k": dict(mesh="pipe50k", n_steps=10, dump_step=1, dump_iter=1),
    # the same 10 steps with the Newton loop run to convergence (picc's test at 1e-11,
    # up to 12 iterations) instead of the fixed 3 iterations: the reference's converged
    # solution, against which a path with its own Newton tolerance is compared
    "pipe50k_conv": dict(mesh="pipe50k", n_steps=10, dump_step=1, dump_iter=1, newton_min=1, newton_max=12),
    # the NS block solver (ns_solver.cpp:167): 10 outer iterations or relative 1e-4,
    # inner GMRES and Schur CG at the reference's NS defaults
    "tiny_ns": dict(mesh="tiny", n_steps=2, dump_step=2, dump_iter=2, ls_type="ns", ls_rel_tol=1e-4,
                    ls_max_itr=10),
    "small_ns": dict(mesh="small", n_steps=3, dump_step=1, dump_iter=1, u_amp=5.0, ls_type="ns",
                     ls_rel_tol=1e-4, ls_max_itr=10),
    # a coupled RCR (Windkessel) outlet with the reference's pipe_RCR_3d values
    # (tests/cases/fluid/pipe_RCR_3d/solver.xml): semi-implicit coupling, the outlet's
    # resistance term in every GMRES product (add_bc_mul.cpp:53)
    "small_rcr": dict(mesh="small", n_steps=3, dump_step=2, dump_iter=2, u_amp=5.0, rcr=1, rcr_Rp=121.0,
                      rcr_C=1.5e-5, rcr_Rd=1212.0, rcr_Pd=0.0, rcr_Xo=0.0),
    # the same outlet with a steady inflow: the case tests/test_solver_xml.py writes as
    # solver.xml + .vtu/.vtp files and runs through FluidCase
    "small_rcr_steady": dict(mesh="small", n_steps=2, dump_step=2, dump_iter=2, rcr=1, rcr_Rp=121.0,
                             rcr_C=1.5e-5, rcr_Rd=1212.0, rcr_Pd=0.0, rcr_Xo=0.0),
}


# Solid (neo-Hookean + ST91 penalty, E=1e6, nu=0.45, rho=1.2) and mesh-motion
# (linear elastic, nu=0.3) assembly on the small pipe with seeded random state.
SOLID = dict(rho=1.2, E=1.0e6, nu=0.45, dt=1e-3, rho_inf=0.5)
SOLID["C10"] = SOLID["E"] / (4.0 * (1.0 + SOLID["nu"]))            # mu / 2
SOLID["Kpen"] = SOLID["E"] / (3.0 * (1.0 - 2.0 * SOLID["nu"]))     # bulk modulus
MESHMOTION = dict(rho=0.5, E=1.0, nu=0.3, dt=1e-3, rho_inf=0.5)


def run_assembly(name, physics, solve=None):
    """Assembly of one solid or mesh-motion system with seeded random state; with
    `solve` = dict(ls_rel_tol, ls_abs_tol, ls_max_itr) also the reference's CG solve
    (fsils_solve, LS_TYPE_CG, diagonal preconditioner) with zero Dirichlet values at
    the inlet and outlet nodes."""
    mesh = named_pipe("small")
    rng = np.random.default_rng(17)
    nNo = mesh.nNo
    tDof = 3 if physics == "struct" else 7
    params = dict(SOLID if physics == "struct" else MESHMOTION)
    params["mode"] = "assemble_" + physics
    if solve:
        params.update(solve)
        params["solve_cg"] = 1
    scale = 0.01 if physics == "struct" else 0.02
    A = rng.standard_normal((nNo, tDof))
    Y = rng.standard_normal((nNo, tDof))
    D = scale * rng.standard_normal((nNo, tDof))
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        cdir, odir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
        write_case(mesh, cdir, params)
        A.tofile(os.path.join(cdir, "A.bin"))
        Y.tofile(os.path.join(cdir, "Y.bin"))
        D.tofile(os.path.join(cdir, "D.bin"))
        out = {"params": np.array(repr(params)), "A": A, "Y": Y, "D": D}
        if physics == "mesh":
            Do = scale * rng.standard_normal((nNo, tDof))
            Do.tofile(os.path.join(cdir, "Do.bin"))
            out["Do"] = Do
        if solve:
            dirn = np.unique(np.concatenate([mesh.faces["inlet"].gN, mesh.faces["outlet"].gN])).astype(np.int32)
            dirn.tofile(os.path.join(cdir, "dir_nodes.bin"))
            out["dir_nodes"] = dirn
        os.makedirs(odir)
        subprocess.run([HARNESS, cdir, odir], check=True)
        rd = lambda f, dt: np.fromfile(os.path.join(odir, f), dtype=dt)  # noqa: E731
        if solve:
            out["dX"] = rd("dX.bin", np.float64).reshape(nNo, 3)
            with open(os.path.join(odir, "log.txt")) as fh:
                t = fh.read().split()
            out["cg_stats"] = np.array([float(t[2]), float(t[4]), float(t[6]), float(t[8]), float(t[10])])
        out["rowPtr"] = rd("rowPtr.bin", np.int32)
        out["colPtr"] = rd("colPtr.bin", np.int32)
        out["R_asm"] = rd("R_asm.bin", np.float64).reshape(nNo, 3)
        out["Val_asm"] = rd("Val_asm.bin", np.float64).reshape(-1, 9)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, "nNo", nNo, "|R|", np.linalg.norm(out["R_asm"]), "|Val|", np.linalg.norm(out["Val_asm"]))
    finally:
        shutil.rmtree(tmp)


# FSI assembly on the small pipe: elements whose centroid lies outside 0.35 (of the
# radius 0.5) form the solid domain, the rest the fluid; seeded random state with the
# mesh displacement/velocity at rows 4..6 (tDof 7).
FSI = dict(rho_f=1.06, mu=0.04, backflow_beta=0.2, rho_s=1.2, E=1.0e6, nu=0.45, dt=1e-3, rho_inf=0.5)
FSI["C10"] = FSI["E"] / (4.0 * (1.0 + FSI["nu"]))
FSI["Kpen"] = FSI["E"] / (3.0 * (1.0 - 2.0 * FSI["nu"]))


def fsi_domains(mesh):
    """eId per element: bit 0 fluid, bit 1 solid (solid where the centroid radius > 0.35)."""
    cen = mesh.x[mesh.ien].mean(axis=1)
    r = np.hypot(cen[:, 0], cen[:, 1])
    return np.where(r > 0.35, 2, 1).astype(np.int32)


def run_fsi(name):
    mesh = named_pipe("small")
    rng = np.random.default_rng(23)
    nNo, tDof = mesh.nNo, 7
    params = dict(FSI)
    params["mode"] = "assemble_fsi"
    A = rng.standard_normal((nNo, tDof))
    Y = rng.standard_normal((nNo, tDof))
    D = 0.01 * rng.standard_normal((nNo, tDof))
    eid = fsi_domains(mesh)
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        cdir, odir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
        write_case(mesh, cdir, params)
        for k, v in (("A", A), ("Y", Y), ("D", D)):
            v.tofile(os.path.join(cdir, f"{k}.bin"))
        eid.tofile(os.path.join(cdir, "eid.bin"))
        os.makedirs(odir)
        subprocess.run([HARNESS, cdir, odir], check=True)
        rd = lambda f, dt: np.fromfile(os.path.join(odir, f), dtype=dt)  # noqa: E731
        out = {"params": np.array(repr(params)), "A": A, "Y": Y, "D": D, "eid": eid,
               "rowPtr": rd("rowPtr.bin", np.int32), "colPtr": rd("colPtr.bin", np.int32),
               "R_asm": rd("R_asm.bin", np.float64).reshape(nNo, 4),
               "Val_asm": rd("Val_asm.bin", np.float64).reshape(-1, 16)}
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, "nNo", nNo, "solid elements", int((eid == 2).sum()), "of", eid.size,
              "|R|", np.linalg.norm(out["R_asm"]), "|Val|", np.linalg.norm(out["Val_asm"]))
    finally:
        shutil.rmtree(tmp)


# Coupled ALE FSI time steps on the FSI pipe (lumen + 1 mm neo-Hookean/ST91 wall
# annulus, E=1e6, nu=0.45, rho=1.2) with linear-elastic mesh motion (E=1, nu=0.3, no
# mass): FSI equation by GMRES(50) + diagonal preconditioner, mesh equation by CG; three
# Newton iterations per equation per step (tolerance below reach), pulsatile inflow
# 15 + 5 sin(2 pi t) cm/s.
FSI_RUN = dict(FSI)
FSI_RUN.update(mode="fsi_run", mesh_E=1.0, mesh_nu=0.3, mesh_rho=0.0,
               ls_rel_tol=1e-10, ls_abs_tol=1e-17, ls_max_itr=100, ls_krylov_dim=50,
               mesh_ls_rel_tol=1e-10, mesh_ls_abs_tol=1e-17, mesh_ls_max_itr=2000,
               newton_min=3, newton_max=3, newton_tol=1e-11,
               mesh_newton_min=3, mesh_newton_max=3, mesh_newton_tol=1e-11,
               u_mean=15.0, u_amp=5.0, u_freq=1.0, n_steps=3, dump_step=2, dump_iter=3)


def run_fsi_steps(name, mesh_name):
    mesh = named_pipe(mesh_name)
    nNo, tDof = mesh.nNo, 7
    params = dict(FSI_RUN)
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        cdir, odir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
        write_case(mesh, cdir, params)
        mesh.eid.tofile(os.path.join(cdir, "eid.bin"))
        os.makedirs(odir)
        subprocess.run([HARNESS, cdir, odir], check=True)
        rd = lambda f, dt: np.fromfile(os.path.join(odir, f), dtype=dt)  # noqa: E731
        with open(os.path.join(odir, "log.txt")) as fh:
            log = fh.read()
        rows = []
        for line in log.splitlines():
            t = line.split()
            if t and t[0] == "step":  # step S eq E iter I iNorm X fNorm Y itr N suc K
                rows.append([int(t[1]), int(t[3]), int(t[5]), float(t[7]), float(t[9]), int(t[11]), int(t[13])])
        out = {"params": np.array(repr(params)), "log": np.array(log), "newton_log": np.array(rows, dtype=np.float64),
               "rowPtr": rd("rowPtr.bin", np.int32), "colPtr": rd("colPtr.bin", np.int32)}
        # the mesh equation's system at the dump point (dof 3)
        out["R_asm"] = rd("R_asm.bin", np.float64).reshape(nNo, -1)
        out["Val_asm"] = rd("Val_asm.bin", np.float64).reshape(out["colPtr"].size, -1)
        for k in ("Ag", "Yg", "Dg", "Do"):
            out[k] = rd(f"{k}.bin", np.float64).reshape(nNo, tDof)
        for s in range(1, params["n_steps"] + 1):
            for k in ("An", "Yn", "Dn"):
                out[f"{k}_{s}"] = rd(f"{k}_{s}.bin", np.float64).reshape(nNo, tDof)
        out["restart_bin"] = rd("stFile_last.bin", np.uint8)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, "nNo", nNo, "nEl", mesh.nEl, "solid", int((mesh.eid == 2).sum()))
        print(log)
    finally:
        shutil.rmtree(tmp)


# Fourier representation of a pulsatile inflow waveform (fft/ifft, fft.cpp): a seeded
# synthetic flow curve of one period (a cardiac-like pulse: systolic peak, dicrotic
# notch), 10 modes, evaluated at times across three periods; and the ramp variant.
def run_fourier(name):
    rng = np.random.default_rng(31)
    t = np.linspace(0.0, 1.0, 41)
    q = -(5.0 + 20.0 * np.exp(-((t - 0.18) / 0.07) ** 2) + 3.0 * np.exp(-((t - 0.45) / 0.05) ** 2))
    q += 0.2 * rng.standard_normal(t.size)
    q[-1] = q[0]
    times = np.concatenate([np.linspace(0.0, 3.0, 61), [0.0005, 1.2345, 2.999]])
    out = {}
    for ramp in (0, 1):
        tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
        try:
            cdir, odir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
            os.makedirs(cdir)
            os.makedirs(odir)
            np.stack([t, q], axis=1).astype(np.float64).tofile(os.path.join(cdir, "tv.bin"))
            times.astype(np.float64).tofile(os.path.join(cdir, "times.bin"))
            with open(os.path.join(cdir, "params.txt"), "w") as fh:
                fh.write(f"mode=fourier\nn_modes=10\nramp={ramp}\n")
            subprocess.run([HARNESS, cdir, odir], check=True)
            out[f"eval_ramp{ramp}"] = np.fromfile(os.path.join(odir, "eval.bin"), dtype=np.float64).reshape(-1, 2)
            out[f"coef_ramp{ramp}"] = np.fromfile(os.path.join(odir, "coef.bin"), dtype=np.float64)
        finally:
            shutil.rmtree(tmp)
    out.update(t=t, q=q, times=times)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
    print(name, out["coef_ramp0"][:6])


def write_case(mesh, d, params):
    os.makedirs(d, exist_ok=True)
    mesh.x.astype(np.float64).tofile(os.path.join(d, "x.bin"))
    mesh.ien.astype(np.int32).tofile(os.path.join(d, "ien.bin"))
    for name, f in mesh.faces.items():
        f.ien.astype(np.int32).tofile(os.path.join(d, f"{name}_ien.bin"))
        f.gE.astype(np.int32).tofile(os.path.join(d, f"{name}_gE.bin"))
        f.gN.astype(np.int32).tofile(os.path.join(d, f"{name}_gN.bin"))
    mesh.inlet_profile.astype(np.float64).tofile(os.path.join(d, "inlet_prof.bin"))
    with open(os.path.join(d, "params.txt"), "w") as fh:
        for k, v in params.items():
            fh.write(f"{k}={v!r}\n" if isinstance(v, float) else f"{k}={v}\n")


def run_case(name):
    spec = dict(CASES[name])
    mesh = named_pipe(spec.pop("mesh"))
    params = dict(BASE)
    params.update(spec)
    tmp = tempfile.mkdtemp(prefix=f"golden_{name}_")
    try:
        cdir, odir = os.path.join(tmp, "case"), os.path.join(tmp, "out")
        write_case(mesh, cdir, params)
        os.makedirs(odir)
        subprocess.run([HARNESS, cdir, odir], check=True)
        nNo = mesh.nNo
        out = {"params": np.array(repr(params))}
        with open(os.path.join(odir, "log.txt")) as fh:
            log = fh.read()
        out["log"] = np.array(log)
        its = []
        for line in log.splitlines():
            t = line.split()
            if t[0] == "step":
                kv = dict(zip(t[0::2], t[1::2]))
                row = [int(t[1]), int(t[3]), float(t[5]), float(t[7]), int(t[9]), int(t[11])]
                if "gm_itr" in kv:  # NS: inner GMRES and CG iteration totals, dB
                    row += [int(kv["gm_itr"]), int(kv["cg_itr"]), float(kv["dB"])]
                if "P" in kv:  # RCR outlet: coupled pressure and the outlet flows at n and n+1
                    row += [float(kv["P"]), float(kv["Qo"]), float(kv["Qn"])]
                its.append(row)
            elif t[0] == "rcr_r":
                out["rcr_r"] = np.array(float(t[1]))
        out["newton_log"] = np.array(its, dtype=np.float64)
        rd = lambda f, dt: np.fromfile(os.path.join(odir, f), dtype=dt)  # noqa: E731
        out["rowPtr"] = rd("rowPtr.bin", np.int32)
        out["colPtr"] = rd("colPtr.bin", np.int32)
        if params.get("rcr") == 1:
            out["rcr_face_val"] = rd("rcr_face_val.bin", np.float64).reshape(-1, 3)
        # the reference's restart file of the final state (output::write_restart)
        out["restart_bin"] = rd("stFile_last.bin", np.uint8)
        out["Ag"] = rd("Ag.bin", np.float64).reshape(nNo, 4)
        out["Yg"] = rd("Yg.bin", np.float64).reshape(nNo, 4)
        out["R_asm"] = rd("R_asm.bin", np.float64).reshape(nNo, 4)
        out["dX"] = rd("dX.bin", np.float64).reshape(nNo, 4)
        nnz = out["colPtr"].size
        if not name.startswith("pipe50k"):
            out["Val_asm"] = rd("Val_asm.bin", np.float64).reshape(nnz, 16)
        for s in range(1, params["n_steps"] + 1):
            if not name.startswith("pipe50k") or s in (1, 10):
                out[f"Yn_{s}"] = rd(f"Yn_{s}.bin", np.float64).reshape(nNo, 4)
                out[f"An_{s}"] = rd(f"An_{s}.bin", np.float64).reshape(nNo, 4)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, "nNo", nNo, "nEl", mesh.nEl, "nnz", nnz)
        print(log.strip().splitlines()[-1])
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: oracle/build_ref.sh")
    for n in (sys.argv[1:] or list(CASES) + ["struct_small", "mesh_small", "mesh_cg_small", "mesh_cg7_small",
                                             "fsi_small", "fsi_run_small", "fourier"]):
        if n == "fsi_small":
            run_fsi(n)
        elif n == "fsi_run_small":
            run_fsi_steps(n, "fsi_small")
        elif n == "fourier":
            run_fourier(n)
        elif n == "struct_small":
            run_assembly(n, "struct")
        elif n == "mesh_small":
            run_assembly(n, "mesh")
        elif n == "mesh_cg_small":  # CG to 1e-10 (stats: iNorm, fNorm, itr, suc, dB)
            run_assembly(n, "mesh", dict(ls_rel_tol=1e-10, ls_abs_tol=1e-30, ls_max_itr=2000))
        elif n == "mesh_cg7_small":  # exactly 7 CG iterations
            run_assembly(n, "mesh", dict(ls_rel_tol=1e-30, ls_abs_tol=1e-300, ls_max_itr=7))
        else:
            run_case(n)
