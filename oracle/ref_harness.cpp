// Test infrastructure, not product code: a driver that links the reference solver's
// own, unmodified hot-path sources (compiled from the reference tree by
// oracle/build_ref.sh into oracle/_ref) and runs its fluid Newton loop on a mesh
// built in code, so that the CPU restatement and the GPU kernels can be checked
// against the reference itself.
//
// The loop follows iterate_solution (Code/Source/solver/main.cpp:292-762) for a single
// fluid equation:
//   picp (pic.cpp:591) -> strong Dirichlet values -> Newton loop:
//     pici (pic.cpp:486) -> ls_alloc (ls.cpp:51) -> global_eq_assem (eq_assem.cpp:377,
//     construct_fluid fluid.cpp:464) -> outlet Neumann/backflow b_assem_neu_bc
//     (eq_assem.cpp:58) -> ls_solve (ls.cpp:69 -> fsils_solve solve.cpp:50) -> picc
//     (pic.cpp:74)
//   -> Ao = An, Yo = Yn (main.cpp:752-757).
// Dirichlet values are written directly (the role of set_bc_dir, set_bc.cpp:794): the
// inlet gets u_z = u_c(t) * profile, walls get zero velocity; acceleration on the
// inlet is du_c/dt * profile (the Fourier branch of set_bc_dir_l, set_bc.cpp:1033).
//
// Input: a case directory written by tests/golden/make_golden.py (raw little-endian
// arrays + params.txt).  Output: raw arrays for the requested step/iteration.
#include "Simulation.h"
#include "ComMod.h"
#include "eq_assem.h"
#include "fluid.h"
#include "fs.h"
#include "lhsa.h"
#include "ls.h"
#include "nn.h"
#include "pic.h"
#include "FsilsLinearAlgebra.h"
#include "fsils_api.hpp"
#include "commu.h"
#include "lhs.h"
#include "mat_fun.h"
#include "all_fun.h"
#include "baf_ini.h"
#include "set_bc.h"
#include "output.h"
#include "fft.h"

#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>
#include <chrono>

// The reference's own restart file (output::write_restart, output.cpp:202-360) of the
// final state, with the stamp and record length initialize.cpp:488-519 sets up.
static void dump_restart(Simulation& sim, const std::string& out) {
  auto& com = sim.com_mod;
  com.stFileName = out + "/stFile";
  com.stFileRepl = true;
  const int nX = com.cplBC.coupled ? com.cplBC.nX : 0;
  com.stamp = {1, com.nEq, com.nMsh, com.tnNo, nX, com.tDof, com.dFlag ? 1 : 0};
  std::array<double, 3> timeP = {0.0, 0.0, 0.0};
  output::write_restart(&sim, timeP);
}

static std::map<std::string, std::string> read_params(const std::string& dir) {
  std::map<std::string, std::string> p;
  std::ifstream f(dir + "/params.txt");
  std::string line;
  while (std::getline(f, line)) {
    auto eq = line.find('=');
    if (eq == std::string::npos) continue;
    p[line.substr(0, eq)] = line.substr(eq + 1);
  }
  return p;
}

template <typename T>
static std::vector<T> read_raw(const std::string& path) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) throw std::runtime_error("cannot open " + path);
  size_t n = f.tellg();
  f.seekg(0);
  std::vector<T> v(n / sizeof(T));
  f.read(reinterpret_cast<char*>(v.data()), n);
  return v;
}

template <typename T>
static void write_raw(const std::string& path, const T* p, size_t n) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p), n * sizeof(T));
}

static void setup_face(faceType& fa, const std::string& dir, const std::string& name) {
  auto ien = read_raw<int>(dir + "/" + name + "_ien.bin");
  auto gE = read_raw<int>(dir + "/" + name + "_gE.bin");
  auto gN = read_raw<int>(dir + "/" + name + "_gN.bin");
  fa.name = name;
  fa.iM = 0;
  fa.eNoN = 3;
  fa.nEl = (int)gE.size();
  fa.gnEl = fa.nEl;
  fa.nNo = (int)gN.size();
  fa.IEN.resize(3, fa.nEl);
  for (int e = 0; e < fa.nEl; e++)
    for (int a = 0; a < 3; a++) fa.IEN(a, e) = ien[3 * e + a];
  fa.gE.resize(fa.nEl);
  for (int e = 0; e < fa.nEl; e++) fa.gE(e) = gE[e];
  fa.gN.resize(fa.nNo);
  for (int a = 0; a < fa.nNo; a++) fa.gN(a) = gN[a];
  fa.eType = consts::ElementType::TRI3;
  fa.nG = 3;
  fa.w.resize(fa.nG);
  fa.xi.resize(2, fa.nG);
  fa.N.resize(3, fa.nG);
  fa.Nx.resize(2, 3, fa.nG);
  nn::get_gip(nullptr, fa);
  for (int g = 0; g < fa.nG; g++) nn::get_gnn(nullptr, g, fa);
}

// Assembly of one solid (construct_dsolid, sv_struct.cpp:213) or mesh-motion
// (construct_mesh, mesh.cpp:49) system on the case mesh with the given state arrays;
// dumps R and Val.  The mesh equation sits at rows 4..6 of a 7-dof state, as in the
// FSI set-up the reference uses it in (construct_mesh reads Do at rows nsd+1..2nsd).
static int assemble_only(const std::string& dir, const std::string& out, std::map<std::string, std::string>& P) {
  auto getd = [&](const char* k) { return std::stod(P.at(k)); };
  const bool is_mesh = P.at("mode") == "assemble_mesh";
  Simulation sim;
  auto& com = sim.com_mod;
  auto xs = read_raw<double>(dir + "/x.bin");
  auto iens = read_raw<int>(dir + "/ien.bin");
  const int nNo = (int)xs.size() / 3;
  const int nEl = (int)iens.size() / 4;
  const int tDof = is_mesh ? 7 : 3;
  com.nsd = 3;
  com.nsymd = 6;
  com.tnNo = nNo;
  com.gtnNo = nNo;
  com.nMsh = 1;
  com.msh.resize(1);
  com.nEq = 1;
  com.eq.resize(1);
  com.dt = getd("dt");
  com.dFlag = true;
  auto& msh = com.msh[0];
  msh.eNoN = 4;
  msh.nEl = nEl;
  msh.gnEl = nEl;
  msh.nNo = nNo;
  msh.IEN.resize(4, nEl);
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < 4; a++) msh.IEN(a, e) = iens[4 * e + a];
  msh.gN.resize(nNo);
  for (int a = 0; a < nNo; a++) msh.gN(a) = a;
  nn::select_ele(com, msh);
  msh.nFs = 1;
  fs::init_fs_msh(com, msh);
  com.x.resize(3, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < 3; i++) com.x(i, a) = xs[3 * a + i];
  com.Bf.resize(3, nNo);
  auto& eq = com.eq[0];
  eq.phys = is_mesh ? consts::EquationType::phys_mesh : consts::EquationType::phys_struct;
  eq.dof = 3;
  eq.roInf = getd("rho_inf");
  eq.am = (2.0 - eq.roInf) / (1.0 + eq.roInf);  // second-order equation
  eq.af = 1.0 / (1.0 + eq.roInf);
  eq.beta = 0.25 * std::pow((1.0 + eq.am - eq.af), 2.0);
  eq.gam = 0.5 + eq.am - eq.af;
  eq.s = is_mesh ? 4 : 0;
  eq.e = eq.s + 2;
  eq.nDmn = 1;
  eq.dmn.resize(1);
  auto& dmn = eq.dmn[0];
  dmn.Id = -1;
  dmn.phys = eq.phys;
  using PP = consts::PhysicalProperyType;
  dmn.prop[PP::solid_density] = getd("rho");
  dmn.prop[PP::elasticity_modulus] = getd("E");
  dmn.prop[PP::poisson_ratio] = getd("nu");
  dmn.prop[PP::damping] = 0.0;
  dmn.prop[PP::f_x] = 0.0;
  dmn.prop[PP::f_y] = 0.0;
  dmn.prop[PP::f_z] = 0.0;
  if (!is_mesh) {
    dmn.stM.isoType = consts::ConstitutiveModelType::stIso_nHook;
    dmn.stM.volType = consts::ConstitutiveModelType::stVol_ST91;
    dmn.stM.C10 = getd("C10");
    dmn.stM.Kpen = getd("Kpen");
  }
  com.tDof = tDof;
  com.dof = 3;
  int nnz = 0;
  lhsa_ns::lhsa(&sim, nnz);
  com.lhs.nnz = nnz;
  FsilsLinearAlgebra fsils_la;
  eq.linear_algebra = &fsils_la;
  auto A = read_raw<double>(dir + "/A.bin");
  auto Y = read_raw<double>(dir + "/Y.bin");
  auto D = read_raw<double>(dir + "/D.bin");
  Array<double> Ag(tDof, nNo), Yg(tDof, nNo), Dg(tDof, nNo);
  com.Do.resize(tDof, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < tDof; i++) {
      Ag(i, a) = A[tDof * a + i];
      Yg(i, a) = Y[tDof * a + i];
      Dg(i, a) = D[tDof * a + i];
    }
  if (is_mesh) {
    auto Do = read_raw<double>(dir + "/Do.bin");
    for (int a = 0; a < nNo; a++)
      for (int i = 0; i < tDof; i++) com.Do(i, a) = Do[tDof * a + i];
  }
  ls_ns::ls_alloc(com, eq);
  com.R.resize(3, nNo);
  com.R = 0.0;
  com.Val = 0.0;
  com.cEq = 0;
  eq_assem::global_eq_assem(com, sim.get_cep_mod(), msh, Ag, Yg, Dg);
  write_raw(out + "/R_asm.bin", com.R.data(), (size_t)com.R.size());
  write_raw(out + "/Val_asm.bin", com.Val.data(), (size_t)com.Val.size());
  write_raw(out + "/rowPtr.bin", com.rowPtr.data(), (size_t)com.rowPtr.size());
  write_raw(out + "/colPtr.bin", com.colPtr.data(), (size_t)com.colPtr.size());
  if (P.count("solve_cg") && P.at("solve_cg") == "1") {
    // fsils_solve with LS_TYPE_CG (cgrad_v, cgrad.cpp:166) + diagonal preconditioner on
    // the assembled system, Dirichlet rows/cols (zero value) at the listed nodes
    fsi_linear_solver::FSILS_commuType commu;
    fsi_linear_solver::fsils_commu_create(commu, MPI_COMM_WORLD);
    Vector<int> gNodes(nNo);
    for (int a = 0; a < nNo; a++) gNodes(a) = a;
    fsi_linear_solver::fsils_lhs_create(com.lhs, commu, nNo, nNo, nnz, gNodes, com.rowPtr, com.colPtr, 1);
    auto dn = read_raw<int>(dir + "/dir_nodes.bin");
    Vector<int> gN((int)dn.size());
    for (size_t a = 0; a < dn.size(); a++) gN((int)a) = dn[a];
    Array<double> sVl(3, (int)dn.size());
    fsi_linear_solver::fsils_bc_create(com.lhs, 0, (int)dn.size(), 3, fsi_linear_solver::BcType::BC_TYPE_Dir, gN, sVl);
    fsi_linear_solver::fsils_ls_create(eq.FSILS, fsi_linear_solver::LinearSolverType::LS_TYPE_CG,
                                       getd("ls_rel_tol"), getd("ls_abs_tol"), std::stoi(P.at("ls_max_itr")));
    Vector<int> incL(1);
    incL = 1;
    Vector<double> res(1);
    res = 0.0;
    fsi_linear_solver::fsils_solve(com.lhs, eq.FSILS, 3, com.R, com.Val, consts::PreconditionerType::PREC_FSILS, incL,
                                   res);
    write_raw(out + "/dX.bin", com.R.data(), (size_t)com.R.size());
    auto& RI = eq.FSILS.RI;
    std::ofstream log(out + "/log.txt");
    log.precision(17);
    log << "cg iNorm " << RI.iNorm << " fNorm " << RI.fNorm << " itr " << RI.itr << " suc " << RI.suc << " dB "
        << RI.dB << "\n";
  }
  return 0;
}

// FSI assembly (construct_fsi, fsi.cpp:48-332) on the case mesh: every element belongs
// to the fluid domain (eId bit 0) or the solid domain (bit 1); tDof = 7 with the mesh
// equation's displacement and velocity at rows 4..6 (fluid elements are integrated in
// x + Dg(4..6) and convect with the velocity relative to Yg(4..6)).  Dumps R and Val.
static int assemble_fsi(const std::string& dir, const std::string& out, std::map<std::string, std::string>& P) {
  auto getd = [&](const char* k) { return std::stod(P.at(k)); };
  Simulation sim;
  auto& com = sim.com_mod;
  auto xs = read_raw<double>(dir + "/x.bin");
  auto iens = read_raw<int>(dir + "/ien.bin");
  auto eid = read_raw<int>(dir + "/eid.bin");
  const int nNo = (int)xs.size() / 3;
  const int nEl = (int)iens.size() / 4;
  const int tDof = 7;
  com.nsd = 3;
  com.nsymd = 6;
  com.tnNo = nNo;
  com.gtnNo = nNo;
  com.nMsh = 1;
  com.msh.resize(1);
  com.nEq = 1;
  com.eq.resize(1);
  com.dt = getd("dt");
  com.mvMsh = true;
  com.dFlag = true;
  auto& msh = com.msh[0];
  msh.name = "pipe";
  msh.eNoN = 4;
  msh.nEl = nEl;
  msh.gnEl = nEl;
  msh.nNo = nNo;
  msh.gnNo = nNo;
  msh.IEN.resize(4, nEl);
  msh.eId.resize(nEl);
  for (int e = 0; e < nEl; e++) {
    for (int a = 0; a < 4; a++) msh.IEN(a, e) = iens[4 * e + a];
    msh.eId(e) = eid[e];
  }
  msh.gN.resize(nNo);
  for (int a = 0; a < nNo; a++) msh.gN(a) = a;
  nn::select_ele(com, msh);
  msh.nFs = 1;
  fs::init_fs_msh(com, msh);
  com.x.resize(3, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < 3; i++) com.x(i, a) = xs[3 * a + i];
  com.Bf.resize(3, nNo);
  mat_fun::ten_init(3);  // the index table of the legacy tensor products (initialize.cpp)
  auto& eq = com.eq[0];
  eq.phys = consts::EquationType::phys_FSI;
  eq.dof = 4;
  eq.roInf = getd("rho_inf");
  eq.am = 0.5 * (3.0 - eq.roInf) / (1.0 + eq.roInf);  // first-order equation (initialize.cpp:424-430)
  eq.af = 1.0 / (1.0 + eq.roInf);
  eq.beta = 0.25 * std::pow((1.0 + eq.am - eq.af), 2.0);
  eq.gam = 0.5 + eq.am - eq.af;
  eq.s = 0;
  eq.e = 3;
  eq.nDmn = 2;
  eq.dmn.resize(2);
  using PP = consts::PhysicalProperyType;
  auto& fd = eq.dmn[0];
  fd.Id = 0;
  fd.phys = consts::EquationType::phys_fluid;
  fd.prop[PP::fluid_density] = getd("rho_f");
  fd.prop[PP::f_x] = 0.0;
  fd.prop[PP::f_y] = 0.0;
  fd.prop[PP::f_z] = 0.0;
  fd.prop[PP::backflow_stab] = getd("backflow_beta");
  fd.prop[PP::inverse_darcy_permeability] = 0.0;
  fd.fluid_visc.viscType = consts::FluidViscosityModelType::viscType_Const;
  fd.fluid_visc.mu_i = getd("mu");
  auto& sd = eq.dmn[1];
  sd.Id = 1;
  sd.phys = consts::EquationType::phys_struct;
  sd.prop[PP::solid_density] = getd("rho_s");
  sd.prop[PP::elasticity_modulus] = getd("E");
  sd.prop[PP::poisson_ratio] = getd("nu");
  sd.prop[PP::damping] = 0.0;
  sd.prop[PP::f_x] = 0.0;
  sd.prop[PP::f_y] = 0.0;
  sd.prop[PP::f_z] = 0.0;
  sd.stM.isoType = consts::ConstitutiveModelType::stIso_nHook;
  sd.stM.volType = consts::ConstitutiveModelType::stVol_ST91;
  sd.stM.C10 = getd("C10");
  sd.stM.Kpen = getd("Kpen");
  com.tDof = tDof;
  com.dof = 4;
  int nnz = 0;
  lhsa_ns::lhsa(&sim, nnz);
  com.lhs.nnz = nnz;
  FsilsLinearAlgebra fsils_la;
  eq.linear_algebra = &fsils_la;
  auto A = read_raw<double>(dir + "/A.bin");
  auto Y = read_raw<double>(dir + "/Y.bin");
  auto D = read_raw<double>(dir + "/D.bin");
  Array<double> Ag(tDof, nNo), Yg(tDof, nNo), Dg(tDof, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < tDof; i++) {
      Ag(i, a) = A[tDof * a + i];
      Yg(i, a) = Y[tDof * a + i];
      Dg(i, a) = D[tDof * a + i];
    }
  ls_ns::ls_alloc(com, eq);
  com.R.resize(4, nNo);
  com.R = 0.0;
  com.Val = 0.0;
  com.cEq = 0;
  eq_assem::global_eq_assem(com, sim.get_cep_mod(), msh, Ag, Yg, Dg);
  write_raw(out + "/R_asm.bin", com.R.data(), (size_t)com.R.size());
  write_raw(out + "/Val_asm.bin", com.Val.data(), (size_t)com.Val.size());
  write_raw(out + "/rowPtr.bin", com.rowPtr.data(), (size_t)com.rowPtr.size());
  write_raw(out + "/colPtr.bin", com.colPtr.data(), (size_t)com.colPtr.size());
  return 0;
}

// Coupled ALE FSI time steps (iterate_solution, main.cpp:292-762, with two coupled
// equations): the FSI equation (dof 4, rows 0..3 of a 7-row state, fluid domain Id 0
// and legacy struct_3d solid domain Id 1, GMRES) and the mesh equation (dof 3, rows
// 4..6, linear elastic over every element, CG).  Per Newton iteration: pici (all
// equations) -> ls_alloc -> global_eq_assem (construct_fsi / construct_mesh) ->
// outlet b_assem_neu_bc (FSI only; gnnb moves the face by Do(4..6), b_fluid convects
// with the velocity relative to the mesh) -> ls_solve -> picc, which copies the solid
// nodes' An/Yn/Dn(0..2) into rows 4..6 after an FSI solve and alternates the
// equations until both converge.  Linear-solver faces follow baf_ini (fsi_ls_ini,
// baf_ini.cpp:690-790, and the structure-node face, :197-227): 0 lumen inlet, 1 wall
// inlet ring, 2 wall outlet ring (FSI, Dirichlet), 3 (the outlet Neumann BC: no face),
// 4 lumen inlet, 5 lumen outlet (mesh, Dirichlet), 6 every solid-domain node (mesh).
// Dirichlet values are written directly (the role of set_bc_dir, set_bc.cpp:794):
// inlet velocity u_z = u_c(t) * profile and acceleration du_c/dt * profile, zero on
// the wall rings (rows 0..2) and zero mesh motion at the lumen ends (rows 4..6).
static int run_fsi(const std::string& dir, const std::string& out, std::map<std::string, std::string>& P) {
  auto getd = [&](const char* k) { return std::stod(P.at(k)); };
  auto geti = [&](const char* k) { return std::stoi(P.at(k)); };
  Simulation sim;
  auto& com = sim.com_mod;
  auto xs = read_raw<double>(dir + "/x.bin");
  auto iens = read_raw<int>(dir + "/ien.bin");
  auto eid = read_raw<int>(dir + "/eid.bin");
  const int nNo = (int)xs.size() / 3;
  const int nEl = (int)iens.size() / 4;
  const int tDof = 7;
  com.nsd = 3;
  com.nsymd = 6;
  com.tnNo = nNo;
  com.gtnNo = nNo;
  com.nMsh = 1;
  com.msh.resize(1);
  com.nEq = 2;
  com.eq.resize(2);
  com.dt = getd("dt");
  com.mvMsh = true;
  com.dFlag = true;
  com.sstEq = false;
  com.pstEq = false;
  auto& msh = com.msh[0];
  msh.name = "pipe";
  msh.eNoN = 4;
  msh.nEl = nEl;
  msh.gnEl = nEl;
  msh.nNo = nNo;
  msh.gnNo = nNo;
  msh.IEN.resize(4, nEl);
  msh.eId.resize(nEl);
  com.dmnId.resize(nNo);
  for (int a = 0; a < nNo; a++) com.dmnId(a) = 0;
  for (int e = 0; e < nEl; e++) {
    for (int a = 0; a < 4; a++) msh.IEN(a, e) = iens[4 * e + a];
    msh.eId(e) = eid[e];
    for (int a = 0; a < 4; a++) com.dmnId(iens[4 * e + a]) |= eid[e];  // read_msh.cpp:1519-1533
  }
  msh.gN.resize(nNo);
  for (int a = 0; a < nNo; a++) msh.gN(a) = a;
  nn::select_ele(com, msh);
  msh.nFs = 1;
  fs::init_fs_msh(com, msh);
  const char* fnames[4] = {"inlet", "outlet", "wall_inlet", "wall_outlet"};
  msh.fa.resize(4);
  msh.nFa = 4;
  for (int f = 0; f < 4; f++) setup_face(msh.fa[f], dir, fnames[f]);
  com.x.resize(3, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < 3; i++) com.x(i, a) = xs[3 * a + i];
  com.Bf.resize(3, nNo);
  mat_fun::ten_init(3);
  using PP = consts::PhysicalProperyType;
  // equation 0: FSI (first order), initialize.cpp:424-465
  auto& eq = com.eq[0];
  eq.phys = consts::EquationType::phys_FSI;
  eq.sym = "FS";
  eq.dof = 4;
  eq.coupled = true;
  eq.roInf = getd("rho_inf");
  eq.am = 0.5 * (3.0 - eq.roInf) / (1.0 + eq.roInf);
  eq.af = 1.0 / (1.0 + eq.roInf);
  eq.beta = 0.25 * std::pow((1.0 + eq.am - eq.af), 2.0);
  eq.gam = 0.5 + eq.am - eq.af;
  eq.pNorm = std::numeric_limits<double>::max();
  eq.s = 0;
  eq.e = 3;
  eq.minItr = geti("newton_min");
  eq.maxItr = geti("newton_max");
  eq.tol = getd("newton_tol");
  eq.nDmn = 2;
  eq.dmn.resize(2);
  auto& fd = eq.dmn[0];
  fd.Id = 0;
  fd.phys = consts::EquationType::phys_fluid;
  fd.prop[PP::fluid_density] = getd("rho_f");
  fd.prop[PP::f_x] = 0.0;
  fd.prop[PP::f_y] = 0.0;
  fd.prop[PP::f_z] = 0.0;
  fd.prop[PP::backflow_stab] = getd("backflow_beta");
  fd.prop[PP::inverse_darcy_permeability] = 0.0;
  fd.fluid_visc.viscType = consts::FluidViscosityModelType::viscType_Const;
  fd.fluid_visc.mu_i = getd("mu");
  auto& sd = eq.dmn[1];
  sd.Id = 1;
  sd.phys = consts::EquationType::phys_struct;
  sd.prop[PP::solid_density] = getd("rho_s");
  sd.prop[PP::elasticity_modulus] = getd("E");
  sd.prop[PP::poisson_ratio] = getd("nu");
  sd.prop[PP::damping] = 0.0;
  sd.prop[PP::f_x] = 0.0;
  sd.prop[PP::f_y] = 0.0;
  sd.prop[PP::f_z] = 0.0;
  sd.stM.isoType = consts::ConstitutiveModelType::stIso_nHook;
  sd.stM.volType = consts::ConstitutiveModelType::stVol_ST91;
  sd.stM.C10 = getd("C10");
  sd.stM.Kpen = getd("Kpen");
  // equation 1: mesh motion (second order), one domain over every element
  auto& meq = com.eq[1];
  meq.phys = consts::EquationType::phys_mesh;
  meq.sym = "MS";
  meq.dof = 3;
  meq.coupled = true;
  meq.roInf = getd("rho_inf");
  meq.am = (2.0 - meq.roInf) / (1.0 + meq.roInf);
  meq.af = 1.0 / (1.0 + meq.roInf);
  meq.beta = 0.25 * std::pow((1.0 + meq.am - meq.af), 2.0);
  meq.gam = 0.5 + meq.am - meq.af;
  meq.pNorm = std::numeric_limits<double>::max();
  meq.s = 4;
  meq.e = 6;
  meq.minItr = geti("mesh_newton_min");
  meq.maxItr = geti("mesh_newton_max");
  meq.tol = getd("mesh_newton_tol");
  meq.nDmn = 1;
  meq.dmn.resize(1);
  auto& md = meq.dmn[0];
  md.Id = -1;
  md.phys = consts::EquationType::phys_mesh;
  md.prop[PP::solid_density] = getd("mesh_rho");
  md.prop[PP::elasticity_modulus] = getd("mesh_E");
  md.prop[PP::poisson_ratio] = getd("mesh_nu");
  md.prop[PP::damping] = 0.0;
  md.prop[PP::f_x] = 0.0;
  md.prop[PP::f_y] = 0.0;
  md.prop[PP::f_z] = 0.0;
  com.tDof = tDof;
  com.dof = 4;
  com.Ao.resize(tDof, nNo); com.An.resize(tDof, nNo);
  com.Yo.resize(tDof, nNo); com.Yn.resize(tDof, nNo);
  com.Do.resize(tDof, nNo); com.Dn.resize(tDof, nNo);
  Array<double> Ag(tDof, nNo), Yg(tDof, nNo), Dg(tDof, nNo);

  int nnz = 0;
  lhsa_ns::lhsa(&sim, nnz);
  com.lhs.nnz = nnz;
  fsi_linear_solver::FSILS_commuType commu;
  fsi_linear_solver::fsils_commu_create(commu, MPI_COMM_WORLD);
  Vector<int> gNodes(nNo);
  for (int a = 0; a < nNo; a++) gNodes(a) = a;
  const int nFacesLS = 7;
  fsi_linear_solver::fsils_lhs_create(com.lhs, commu, nNo, nNo, nnz, gNodes, com.rowPtr, com.colPtr, nFacesLS);
  auto dir_face = [&](int lsPtr, const faceType& fa) {
    Array<double> sVl(3, fa.nNo);
    Vector<int> gN(fa.nNo);
    for (int a = 0; a < fa.nNo; a++) gN(a) = fa.gN(a);
    fsi_linear_solver::fsils_bc_create(com.lhs, lsPtr, fa.nNo, 3, fsi_linear_solver::BcType::BC_TYPE_Dir, gN, sVl);
  };
  dir_face(0, msh.fa[0]);
  dir_face(1, msh.fa[2]);
  dir_face(2, msh.fa[3]);
  dir_face(4, msh.fa[0]);
  dir_face(5, msh.fa[1]);
  {  // baf_ini.cpp:197-227: every node of a solid domain
    std::vector<int> sn;
    for (int a = 0; a < nNo; a++)
      if (all_fun::is_domain(com, eq, a, consts::EquationType::phys_struct)) sn.push_back(a);
    Vector<int> gN((int)sn.size());
    for (size_t k = 0; k < sn.size(); k++) gN((int)k) = sn[k];
    fsi_linear_solver::fsils_bc_create(com.lhs, nFacesLS - 1, (int)sn.size(), 3, fsi_linear_solver::BcType::BC_TYPE_Dir,
                                       gN);
  }
  fsi_linear_solver::fsils_ls_create(eq.FSILS, fsi_linear_solver::LinearSolverType::LS_TYPE_GMRES, getd("ls_rel_tol"),
                                     getd("ls_abs_tol"), geti("ls_max_itr"), geti("ls_krylov_dim"));
  fsi_linear_solver::fsils_ls_create(meq.FSILS, fsi_linear_solver::LinearSolverType::LS_TYPE_CG,
                                     getd("mesh_ls_rel_tol"), getd("mesh_ls_abs_tol"), geti("mesh_ls_max_itr"), 1);
  FsilsLinearAlgebra la0, la1;
  eq.linear_algebra = &la0;
  meq.linear_algebra = &la1;
  eq.linear_algebra_preconditioner = consts::PreconditionerType::PREC_FSILS;
  meq.linear_algebra_preconditioner = consts::PreconditionerType::PREC_FSILS;

  auto prof = read_raw<double>(dir + "/inlet_prof.bin");
  const double u_mean = getd("u_mean"), u_amp = getd("u_amp"), freq = getd("u_freq");
  const int nSteps = geti("n_steps");
  Vector<int> incL(nFacesLS);
  Vector<double> res(nFacesLS);
  Vector<double> hg(nNo);
  std::ofstream log(out + "/log.txt");
  log.precision(17);
  double time = 0.0;
  for (int cTS = 1; cTS <= nSteps; cTS++) {
    time += com.dt;
    com.cTS = cTS;
    com.time = time;
    com.cEq = 0;
    for (auto& e : com.eq) {
      e.itr = 0;
      e.ok = false;
    }
    pic::picp(&sim);
    const double w = 2.0 * M_PI * freq;
    const double uc = u_mean + u_amp * std::sin(w * time);
    const double duc = u_amp * w * std::cos(w * time);
    for (int f : {2, 3, 0}) {  // FSI equation: wall rings, then the lumen inlet (its profile is 0 on the ring)
      auto& fa = msh.fa[f];
      for (int a = 0; a < fa.nNo; a++) {
        int Ac = fa.gN(a);
        for (int i = 0; i < 3; i++) { com.An(i, Ac) = 0.0; com.Yn(i, Ac) = 0.0; }
        if (f == 0) {
          com.An(2, Ac) = duc * prof[a];
          com.Yn(2, Ac) = uc * prof[a];
        }
      }
    }
    for (int f : {0, 1}) {  // mesh equation: no mesh motion at the lumen ends
      auto& fa = msh.fa[f];
      for (int a = 0; a < fa.nNo; a++)
        for (int i = 4; i < 7; i++) { com.An(i, fa.gN(a)) = 0.0; com.Yn(i, fa.gN(a)) = 0.0; }
    }
    int inner = 1;
    while (true) {
      const int iEq = com.cEq;
      auto& ceq = com.eq[iEq];
      pic::pici(&sim, Ag, Yg, Dg);
      ls_ns::ls_alloc(com, ceq);
      com.R = 0.0;
      com.Val = 0.0;
      eq_assem::global_eq_assem(com, sim.get_cep_mod(), msh, Ag, Yg, Dg);
      incL = 0;
      res = 0.0;
      if (iEq == 0) {
        hg = 0.0;
        eq_assem::b_assem_neu_bc(com, msh.fa[1], hg, Yg);
        incL(0) = incL(1) = incL(2) = 1;
      } else {
        incL(4) = incL(5) = incL(nFacesLS - 1) = 1;
      }
      if (P.count("dump_step") && cTS == geti("dump_step") && inner == geti("dump_iter")) {
        write_raw(out + "/R_asm.bin", com.R.data(), (size_t)com.R.size());
        write_raw(out + "/Val_asm.bin", com.Val.data(), (size_t)com.Val.size());
        write_raw(out + "/Ag.bin", Ag.data(), (size_t)Ag.size());
        write_raw(out + "/Yg.bin", Yg.data(), (size_t)Yg.size());
        write_raw(out + "/Dg.bin", Dg.data(), (size_t)Dg.size());
        write_raw(out + "/Do.bin", com.Do.data(), (size_t)com.Do.size());
        write_raw(out + "/rowPtr.bin", com.rowPtr.data(), (size_t)com.rowPtr.size());
        write_raw(out + "/colPtr.bin", com.colPtr.data(), (size_t)com.colPtr.size());
      }
      ls_ns::ls_solve(com, ceq, incL, res);
      auto& RI = ceq.FSILS.RI;
      log << "step " << cTS << " eq " << iEq << " iter " << ceq.itr << " iNorm " << RI.iNorm << " fNorm " << RI.fNorm
          << " itr " << RI.itr << " suc " << RI.suc << "\n";
      pic::picc(&sim);
      bool all_ok = true;
      for (auto& e : com.eq) all_ok = all_ok && e.ok;
      if (all_ok) break;
      inner++;
    }
    write_raw(out + "/An_" + std::to_string(cTS) + ".bin", com.An.data(), (size_t)com.An.size());
    write_raw(out + "/Yn_" + std::to_string(cTS) + ".bin", com.Yn.data(), (size_t)com.Yn.size());
    write_raw(out + "/Dn_" + std::to_string(cTS) + ".bin", com.Dn.data(), (size_t)com.Dn.size());
    com.Ao = com.An;
    com.Yo = com.Yn;
    com.Do = com.Dn;
  }
  dump_restart(sim, out);
  return 0;
}

// Fourier representation of a temporal values file (fft / ifft, fft.cpp:36-140): the
// coefficients and the value and derivative at the requested times.
static int run_fourier(const std::string& dir, const std::string& out, std::map<std::string, std::string>& P) {
  auto tv = read_raw<double>(dir + "/tv.bin");  // (t, q) pairs
  auto times = read_raw<double>(dir + "/times.bin");
  const int np = (int)tv.size() / 2;
  std::vector<std::vector<double>> temporal_values(np);
  for (int i = 0; i < np; i++) temporal_values[i] = {tv[2 * i], tv[2 * i + 1]};
  Simulation sim;
  fcType gt;
  gt.d = 1;
  gt.n = std::stoi(P.at("n_modes"));
  gt.lrmp = std::stoi(P.at("ramp")) != 0;
  if (gt.lrmp) gt.n = 1;
  gt.qi.resize(1);
  gt.qs.resize(1);
  gt.r.resize(1, gt.n);
  gt.i.resize(1, gt.n);
  fft(np, temporal_values, gt);
  std::vector<double> res;
  Vector<double> Y(1), dY(1);
  for (double t : times) {
    sim.com_mod.time = t;
    ifft(sim.com_mod, gt, Y, dY);
    res.push_back(Y(0));
    res.push_back(dY(0));
  }
  write_raw(out + "/eval.bin", res.data(), res.size());
  std::vector<double> coef = {gt.ti, gt.T, gt.qi(0), gt.qs(0)};
  for (int k = 0; k < gt.n; k++) coef.push_back(gt.r(0, k));
  for (int k = 0; k < gt.n; k++) coef.push_back(gt.i(0, k));
  write_raw(out + "/coef.bin", coef.data(), coef.size());
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s CASE_DIR OUT_DIR\n", argv[0]);
    return 2;
  }
  std::string dir = argv[1], out = argv[2];
  auto P = read_params(dir);
  if (P.count("mode") && P.at("mode") == "assemble_fsi") return assemble_fsi(dir, out, P);
  if (P.count("mode") && P.at("mode") == "fsi_run") return run_fsi(dir, out, P);
  if (P.count("mode") && P.at("mode") == "fourier") return run_fourier(dir, out, P);
  if (P.count("mode") && P.at("mode").rfind("assemble_", 0) == 0) return assemble_only(dir, out, P);
  auto getd = [&](const char* k) { return std::stod(P.at(k)); };
  auto geti = [&](const char* k) { return std::stoi(P.at(k)); };
  double log_rcr_r = 0.0;

  Simulation sim;
  auto& com = sim.com_mod;
  auto xs = read_raw<double>(dir + "/x.bin");
  auto iens = read_raw<int>(dir + "/ien.bin");
  const int nNo = (int)xs.size() / 3;
  const int nEl = (int)iens.size() / 4;

  com.nsd = 3;
  com.nsymd = 6;
  com.tnNo = nNo;
  com.gtnNo = nNo;
  com.nMsh = 1;
  com.msh.resize(1);
  com.nEq = 1;
  com.eq.resize(1);
  com.dt = getd("dt");
  com.mvMsh = false;
  com.dFlag = false;
  com.sstEq = false;
  com.pstEq = false;

  auto& msh = com.msh[0];
  msh.name = "pipe";
  msh.eNoN = 4;
  msh.nEl = nEl;
  msh.gnEl = nEl;
  msh.nNo = nNo;
  msh.gnNo = nNo;
  msh.IEN.resize(4, nEl);
  for (int e = 0; e < nEl; e++)
    for (int a = 0; a < 4; a++) msh.IEN(a, e) = iens[4 * e + a];
  msh.gN.resize(nNo);
  for (int a = 0; a < nNo; a++) msh.gN(a) = a;
  nn::select_ele(com, msh);
  msh.nFs = 1;
  fs::init_fs_msh(com, msh);
  msh.fa.resize(3);
  msh.nFa = 3;
  setup_face(msh.fa[0], dir, "inlet");
  setup_face(msh.fa[1], dir, "wall");
  setup_face(msh.fa[2], dir, "outlet");

  com.x.resize(3, nNo);
  for (int a = 0; a < nNo; a++)
    for (int i = 0; i < 3; i++) com.x(i, a) = xs[3 * a + i];
  com.Bf.resize(3, nNo);

  // Equation: fluid, dof = nsd + 1 (initialize.cpp:426-465 for the gen-alpha constants)
  auto& eq = com.eq[0];
  eq.phys = consts::EquationType::phys_fluid;
  eq.sym = "NS";
  eq.dof = 4;
  eq.roInf = getd("rho_inf");
  eq.am = 0.5 * (3.0 - eq.roInf) / (1.0 + eq.roInf);
  eq.af = 1.0 / (1.0 + eq.roInf);
  eq.beta = 0.25 * std::pow((1.0 + eq.am - eq.af), 2.0);
  eq.gam = 0.5 + eq.am - eq.af;
  eq.pNorm = std::numeric_limits<double>::max();
  eq.s = 0;
  eq.e = 3;
  eq.minItr = geti("newton_min");
  eq.maxItr = geti("newton_max");
  eq.tol = getd("newton_tol");
  eq.nDmn = 1;
  eq.dmn.resize(1);
  auto& dmn = eq.dmn[0];
  dmn.Id = -1;
  dmn.phys = consts::EquationType::phys_fluid;
  using PP = consts::PhysicalProperyType;
  dmn.prop[PP::fluid_density] = getd("rho");
  dmn.prop[PP::f_x] = 0.0;
  dmn.prop[PP::f_y] = 0.0;
  dmn.prop[PP::f_z] = 0.0;
  dmn.prop[PP::backflow_stab] = getd("backflow_beta");
  dmn.prop[PP::inverse_darcy_permeability] = 0.0;
  dmn.fluid_visc.viscType = consts::FluidViscosityModelType::viscType_Const;
  dmn.fluid_visc.mu_i = getd("mu");
  com.tDof = 4;
  com.dof = 4;

  com.Ao.resize(4, nNo); com.An.resize(4, nNo);
  com.Yo.resize(4, nNo); com.Yn.resize(4, nNo);
  com.Do.resize(4, nNo); com.Dn.resize(4, nNo);
  Array<double> Ag(4, nNo), Yg(4, nNo), Dg(4, nNo);

  // CSR pattern (lhsa.cpp:153) and FSILS handles (initialize.cpp:571-574, baf_ini.cpp:719-744)
  int nnz = 0;
  lhsa_ns::lhsa(&sim, nnz);
  com.lhs.nnz = nnz;
  fsi_linear_solver::FSILS_commuType commu;
  fsi_linear_solver::fsils_commu_create(commu, MPI_COMM_WORLD);
  Vector<int> gNodes(nNo);
  for (int a = 0; a < nNo; a++) gNodes(a) = a;
  // rcr=1: the outlet is a coupled RCR (Windkessel) Neumann BC, the reference's
  // pipe_RCR_3d set-up (read_files.cpp:280-306, baf_ini.cpp:119-177): semi-implicit
  // coupling, a resistance face of the linear solver (fsi_ls_ini) and the
  // finite-difference resistance of calc_der_cpl_bc.
  const bool rcr = P.count("rcr") && geti("rcr") == 1;
  const int nFacesLS = rcr ? 3 : 2;
  fsi_linear_solver::fsils_lhs_create(com.lhs, commu, nNo, nNo, nnz, gNodes, com.rowPtr, com.colPtr, nFacesLS);
  for (int f = 0; f < 2; f++) {
    auto& fa = msh.fa[f];
    Array<double> sVl(3, fa.nNo);  // zero: velocity rows/cols removed (baf_ini.cpp:724-742)
    Vector<int> gN(fa.nNo);
    for (int a = 0; a < fa.nNo; a++) gN(a) = fa.gN(a);
    fsi_linear_solver::fsils_bc_create(com.lhs, f, fa.nNo, 3, fsi_linear_solver::BcType::BC_TYPE_Dir, gN, sVl);
  }
  if (rcr) {
    eq.nBc = 1;
    eq.bc.resize(1);
    auto& bc = eq.bc[0];
    bc.iFa = 2;
    bc.iM = 0;
    bc.bType = utils::ibset(bc.bType, consts::iBC_Neu);
    bc.bType = utils::ibset(bc.bType, consts::iBC_RCR);
    bc.RCR.Rp = getd("rcr_Rp");
    bc.RCR.C = getd("rcr_C");
    bc.RCR.Rd = getd("rcr_Rd");
    bc.RCR.Pd = getd("rcr_Pd");
    bc.RCR.Xo = getd("rcr_Xo");
    bc.gx.resize(msh.fa[2].nNo);
    bc.gx = 1.0;
    bc.cplBCptr = 0;
    auto& cpl = com.cplBC;
    cpl.coupled = true;
    cpl.nFa = 1;
    cpl.schm = consts::CplBCType::cplBC_SI;
    cpl.nX = 1;
    cpl.nXp = 2;
    cpl.xo.resize(1);
    cpl.xp.resize(2);
    cpl.xn.resize(1);
    cpl.initRCR = false;
    cpl.fa.resize(1);
    cpl.fa[0].name = "outlet";
    cpl.fa[0].y = 0.0;
    cpl.fa[0].bGrp = consts::CplBCType::cplBC_Neu;
    bc.bType = utils::ibset(bc.bType, consts::iBC_res);
    cpl.fa[0].RCR.Rp = bc.RCR.Rp;
    cpl.fa[0].RCR.C = bc.RCR.C;
    cpl.fa[0].RCR.Rd = bc.RCR.Rd;
    cpl.fa[0].RCR.Pd = bc.RCR.Pd;
    cpl.fa[0].RCR.Xo = bc.RCR.Xo;
    com.Yo = 0.0;
    com.Yn = 0.0;
    set_bc::rcr_init(com, sim.cm_mod);
    set_bc::calc_der_cpl_bc(com, sim.cm_mod);
    int lsPtr = 1;
    baf_ini_ns::fsi_ls_ini(com, sim.cm_mod, bc, msh.fa[2], lsPtr);
    log_rcr_r = bc.r;
  }
  // ls_type: "gmres" (default) or "ns" (ns_solver.cpp:167, with its GM/CG defaults)
  const bool use_ns = P.count("ls_type") && P.at("ls_type") == "ns";
  fsi_linear_solver::fsils_ls_create(eq.FSILS, use_ns ? fsi_linear_solver::LinearSolverType::LS_TYPE_NS
                                                      : fsi_linear_solver::LinearSolverType::LS_TYPE_GMRES,
                                     getd("ls_rel_tol"), getd("ls_abs_tol"), geti("ls_max_itr"), geti("ls_krylov_dim"));
  FsilsLinearAlgebra fsils_la;
  eq.linear_algebra = &fsils_la;
  eq.linear_algebra_preconditioner = consts::PreconditionerType::PREC_FSILS;

  auto prof = read_raw<double>(dir + "/inlet_prof.bin");
  const double u_mean = getd("u_mean"), u_amp = getd("u_amp"), freq = getd("u_freq");
  const int nSteps = geti("n_steps");
  const int dump_step = geti("dump_step");
  const int dump_iter = geti("dump_iter");
  Vector<int> incL(nFacesLS);
  Vector<double> res(nFacesLS);
  Vector<double> hg(nNo);

  std::ofstream log(out + "/log.txt");
  log.precision(17);
  if (rcr) {
    log << "rcr_r " << log_rcr_r << "\n";
    const auto& fv = com.lhs.face[2].val;
    write_raw(out + "/rcr_face_val.bin", fv.data(), (size_t)fv.size());
  }
  double time = 0.0;
  double t_asm = 0.0, t_solve = 0.0;
  auto wall0 = std::chrono::steady_clock::now();
  for (int cTS = 1; cTS <= nSteps; cTS++) {
    time += com.dt;
    com.cTS = cTS;
    com.time = time;
    com.cEq = 0;
    eq.itr = 0;
    eq.ok = false;
    pic::picp(&sim);
    // strong Dirichlet values
    const double w = 2.0 * M_PI * freq;
    const double uc = u_mean + u_amp * std::sin(w * time);
    const double duc = u_amp * w * std::cos(w * time);
    for (int f = 1; f >= 0; f--) {  // wall first, inlet last: the inlet profile is 0 on the wall ring
      auto& fa = msh.fa[f];
      for (int a = 0; a < fa.nNo; a++) {
        int Ac = fa.gN(a);
        for (int i = 0; i < 3; i++) { com.An(i, Ac) = 0.0; com.Yn(i, Ac) = 0.0; }
        if (f == 0) {
          com.An(2, Ac) = duc * prof[a];
          com.Yn(2, Ac) = uc * prof[a];
        }
      }
    }
    int inner = 1;
    while (true) {
      if (rcr) set_bc::set_bc_cpl(com, sim.cm_mod);  // main.cpp:385-392 (Dirichlet values unchanged)
      pic::pici(&sim, Ag, Yg, Dg);
      ls_ns::ls_alloc(com, eq);
      auto t0 = std::chrono::steady_clock::now();
      eq_assem::global_eq_assem(com, sim.get_cep_mod(), msh, Ag, Yg, Dg);
      if (rcr) {
        set_bc::set_bc_neu(com, sim.cm_mod, Yg, Dg);
      } else {
        hg = 0.0;
        eq_assem::b_assem_neu_bc(com, msh.fa[2], hg, Yg);
      }
      auto t1 = std::chrono::steady_clock::now();
      incL = 1;
      res = 0.0;
      if (rcr) res(eq.bc[0].lsPtr) = eq.gam * com.dt * eq.bc[0].r;  // main.cpp:566-573
      if (cTS == dump_step && inner == dump_iter) {
        write_raw(out + "/R_asm.bin", com.R.data(), (size_t)com.R.size());
        write_raw(out + "/Val_asm.bin", com.Val.data(), (size_t)com.Val.size());
        write_raw(out + "/Ag.bin", Ag.data(), (size_t)Ag.size());
        write_raw(out + "/Yg.bin", Yg.data(), (size_t)Yg.size());
        write_raw(out + "/rowPtr.bin", com.rowPtr.data(), (size_t)com.rowPtr.size());
        write_raw(out + "/colPtr.bin", com.colPtr.data(), (size_t)com.colPtr.size());
      }
      ls_ns::ls_solve(com, eq, incL, res);
      auto t2 = std::chrono::steady_clock::now();
      t_asm += std::chrono::duration<double>(t1 - t0).count();
      t_solve += std::chrono::duration<double>(t2 - t1).count();
      auto& RI = eq.FSILS.RI;
      log << "step " << cTS << " iter " << inner << " iNorm " << RI.iNorm << " fNorm " << RI.fNorm
          << " itr " << RI.itr << " suc " << RI.suc;
      if (use_ns) log << " gm_itr " << eq.FSILS.GM.itr << " cg_itr " << eq.FSILS.CG.itr << " dB " << RI.dB;
      if (rcr) log << " P " << eq.bc[0].g << " Qo " << com.cplBC.fa[0].Qo << " Qn " << com.cplBC.fa[0].Qn;
      log << "\n";
      if (cTS == dump_step && inner == dump_iter) {
        write_raw(out + "/dX.bin", com.R.data(), (size_t)com.R.size());
        write_raw(out + "/Val_scaled.bin", com.Val.data(), (size_t)com.Val.size());
      }
      pic::picc(&sim);
      bool all_ok = true;
      for (auto& e : com.eq) all_ok = all_ok && e.ok;
      if (all_ok) break;
      inner++;
    }
    write_raw(out + "/An_" + std::to_string(cTS) + ".bin", com.An.data(), (size_t)com.An.size());
    write_raw(out + "/Yn_" + std::to_string(cTS) + ".bin", com.Yn.data(), (size_t)com.Yn.size());
    com.Ao = com.An;
    com.Yo = com.Yn;
    if (rcr) com.cplBC.xo = com.cplBC.xn;  // main.cpp:758
  }
  dump_restart(sim, out);
  double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
  log << "timing steps " << nSteps << " wall_s " << wall << " assembly_s " << t_asm << " solve_s " << t_solve << "\n";
  return 0;
}
