// Restart files in the reference's binary layout, so that a run can continue from a
// file either code wrote: output::write_restart (output.cpp:202-372) and
// init_from_bin (initialize.cpp:78-245) for one process.
//
// Layout (native byte order, no padding):
//   stamp int32[7] = {processes, equations, meshes, nodes, 0D unknowns, tDof, dFlag}
//   cTS int32, time double, cpu seconds double, eq.iNorm double per equation
//   0D state xn double[nX]; Yn, An double[tDof * nNo] (column-major (tDof, nNo));
//   with dFlag: Dn, and Dn once more (the reference writes it twice when there is
//   neither prestress, nor a velocity-pressure solid, nor cardiac EP; its reader
//   takes the first copy).
#include <cstdio>
#include <string>

#include "internal.h"

namespace {

int fail(svgpu_ctx* ctx, int status, const std::string& msg) {
  return ctx ? svgpu::set_err(ctx, status, msg) : status;
}

}  // namespace

extern "C" int svgpu_write_restart(svgpu_ctx* ctx, const char* path, const int* stamp, int cTS, double time,
                                   double cpu_time, const double* iNorm, const double* xn, const double* Yn,
                                   const double* An, const double* Dn) {
  if (!path || !stamp || !iNorm || !Yn || !An) return fail(ctx, SVGPU_EINVAL, "write_restart: missing argument");
  const int nEq = stamp[1], nNo = stamp[3], nX = stamp[4], tDof = stamp[5], dFlag = stamp[6];
  if (nEq < 1 || nNo < 1 || nX < 0 || tDof < 1 || (nX > 0 && !xn) || (dFlag && !Dn))
    return fail(ctx, SVGPU_EINVAL, "write_restart: bad stamp or missing 0D/displacement state");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(ctx, SVGPU_EINVAL, std::string("write_restart: cannot open ") + path);
  const size_t n = (size_t)tDof * nNo;
  bool ok = std::fwrite(stamp, sizeof(int), 7, f) == 7;
  ok = ok && std::fwrite(&cTS, sizeof(int), 1, f) == 1;
  ok = ok && std::fwrite(&time, sizeof(double), 1, f) == 1;
  ok = ok && std::fwrite(&cpu_time, sizeof(double), 1, f) == 1;
  ok = ok && std::fwrite(iNorm, sizeof(double), nEq, f) == (size_t)nEq;
  if (nX > 0) ok = ok && std::fwrite(xn, sizeof(double), nX, f) == (size_t)nX;
  ok = ok && std::fwrite(Yn, sizeof(double), n, f) == n;
  ok = ok && std::fwrite(An, sizeof(double), n, f) == n;
  if (dFlag) {
    ok = ok && std::fwrite(Dn, sizeof(double), n, f) == n;
    ok = ok && std::fwrite(Dn, sizeof(double), n, f) == n;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SVGPU_OK : fail(ctx, SVGPU_EINVAL, std::string("write_restart: write failed: ") + path);
}

extern "C" int svgpu_read_restart(svgpu_ctx* ctx, const char* path, const int* stamp, int* cTS, double* time,
                                  double* cpu_time, double* iNorm, double* xo, double* Yo, double* Ao, double* Do) {
  if (!path || !stamp || !cTS || !time || !cpu_time || !iNorm || !Yo || !Ao)
    return fail(ctx, SVGPU_EINVAL, "read_restart: missing argument");
  const int nEq = stamp[1], nNo = stamp[3], nX = stamp[4], tDof = stamp[5], dFlag = stamp[6];
  if (nEq < 1 || nNo < 1 || nX < 0 || tDof < 1 || (nX > 0 && !xo) || (dFlag && !Do))
    return fail(ctx, SVGPU_EINVAL, "read_restart: bad stamp or missing 0D/displacement state");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, SVGPU_EINVAL, std::string("read_restart: cannot open ") + path);
  int t[7];
  const size_t n = (size_t)tDof * nNo;
  bool ok = std::fread(t, sizeof(int), 7, f) == 7;
  // the stamp decides how much follows: check it before reading the arrays
  static const char* what[7] = {"The number of processors ", "The number of equations ", "The number of meshes ",
                                "The number of nodes ", "The number of ncplBC.x ", "The number of dof ",
                                "The dFlag specification "};
  if (ok) {
    for (int i = 0; i < 7; i++)
      if (t[i] != stamp[i]) {
        std::fclose(f);
        return fail(ctx, SVGPU_EINVAL,
                    std::string(what[i]) + " " + std::to_string(t[i]) + " read from '" + path + "' don't match.");
      }
  }
  ok = ok && std::fread(cTS, sizeof(int), 1, f) == 1;
  ok = ok && std::fread(time, sizeof(double), 1, f) == 1;
  ok = ok && std::fread(cpu_time, sizeof(double), 1, f) == 1;
  ok = ok && std::fread(iNorm, sizeof(double), nEq, f) == (size_t)nEq;
  if (nX > 0) ok = ok && std::fread(xo, sizeof(double), nX, f) == (size_t)nX;
  ok = ok && std::fread(Yo, sizeof(double), n, f) == n;
  ok = ok && std::fread(Ao, sizeof(double), n, f) == n;
  if (dFlag) ok = ok && std::fread(Do, sizeof(double), n, f) == n;
  std::fclose(f);
  return ok ? SVGPU_OK : fail(ctx, SVGPU_EINVAL, std::string("read_restart: file too short: ") + path);
}
