// Result files for inspection: a VTK XML UnstructuredGrid (.vtu) of the volume mesh
// with point fields, the format of the reference's write_vtus (vtk_xml.cpp:800-1010,
// which goes through the VTK library; that library is not part of this build).  Data
// are stored raw in an appended block (header_type UInt64, little-endian), which VTK
// and ParaView read directly.  Host-only.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "internal.h"

namespace {

int fail(svgpu_ctx* ctx, int status, const std::string& msg) {
  return ctx ? svgpu::set_err(ctx, status, msg) : status;
}

struct Block {
  std::string xml;  // the DataArray element (with its offset)
  const void* data;
  uint64_t bytes;
};

std::string esc(const char* s) {
  std::string o;
  for (const char* p = s; *p; p++) {
    if (*p == '"') o += "&quot;";
    else if (*p == '<') o += "&lt;";
    else if (*p == '&') o += "&amp;";
    else o += *p;
  }
  return o;
}

}  // namespace

extern "C" int svgpu_write_vtu(svgpu_ctx* ctx, const char* path, int nNo, const double* x, int nEl, int eNoN,
                               const int* ien, int nFields, const char* const* names, const int* ncomp,
                               const double* const* data) {
  if (!path || nNo < 1 || nEl < 0 || !x || (nEl > 0 && !ien) || nFields < 0 || (nFields > 0 && (!names || !ncomp || !data)))
    return fail(ctx, SVGPU_EINVAL, "write_vtu: bad arguments");
  if (eNoN != 4 && eNoN != 3) return fail(ctx, SVGPU_EINVAL, "write_vtu: linear tets (4) or triangles (3)");
  for (long k = 0; k < (long)nEl * eNoN; k++)
    if (ien[k] < 0 || ien[k] >= nNo) return fail(ctx, SVGPU_EINVAL, "write_vtu: connectivity out of range");
  std::vector<int64_t> conn((size_t)nEl * eNoN), offs(nEl);
  for (size_t k = 0; k < conn.size(); k++) conn[k] = ien[k];
  for (int e = 0; e < nEl; e++) offs[e] = (int64_t)(e + 1) * eNoN;
  std::vector<uint8_t> types(nEl, eNoN == 4 ? 10 : 5);  // VTK_TETRA, VTK_TRIANGLE
  std::vector<Block> pd, cells;
  uint64_t off = 0;
  auto add = [&](std::vector<Block>& dst, const std::string& head, const void* p, uint64_t bytes) {
    dst.push_back({head + " format=\"appended\" offset=\"" + std::to_string(off) + "\"/>", p, bytes});
    off += 8 + bytes;
  };
  for (int f = 0; f < nFields; f++) {
    if (!names[f] || !data[f] || ncomp[f] < 1) return fail(ctx, SVGPU_EINVAL, "write_vtu: bad field");
    add(pd, "<DataArray type=\"Float64\" Name=\"" + esc(names[f]) + "\" NumberOfComponents=\"" + std::to_string(ncomp[f]) +
                "\"",
        data[f], (uint64_t)ncomp[f] * nNo * sizeof(double));
  }
  std::vector<Block> pts;
  add(pts, "<DataArray type=\"Float64\" Name=\"Points\" NumberOfComponents=\"3\"", x, (uint64_t)3 * nNo * sizeof(double));
  add(cells, "<DataArray type=\"Int64\" Name=\"connectivity\"", conn.data(), conn.size() * sizeof(int64_t));
  add(cells, "<DataArray type=\"Int64\" Name=\"offsets\"", offs.data(), offs.size() * sizeof(int64_t));
  add(cells, "<DataArray type=\"UInt8\" Name=\"types\"", types.data(), types.size());
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(ctx, SVGPU_EINVAL, std::string("write_vtu: cannot open ") + path);
  std::string h = "<?xml version=\"1.0\"?>\n"
                  "<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" "
                  "header_type=\"UInt64\">\n  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" +
                  std::to_string(nNo) + "\" NumberOfCells=\"" + std::to_string(nEl) + "\">\n      <PointData>\n";
  for (auto& b : pd) h += "        " + b.xml + "\n";
  h += "      </PointData>\n      <Points>\n";
  for (auto& b : pts) h += "        " + b.xml + "\n";
  h += "      </Points>\n      <Cells>\n";
  for (auto& b : cells) h += "        " + b.xml + "\n";
  h += "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n  <AppendedData encoding=\"raw\">\n   _";
  bool ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
  for (auto* group : {&pd, &pts, &cells})
    for (auto& b : *group) {
      ok = ok && std::fwrite(&b.bytes, sizeof(uint64_t), 1, fp) == 1;
      ok = ok && (b.bytes == 0 || std::fwrite(b.data, 1, b.bytes, fp) == b.bytes);
    }
  const std::string tail = "\n  </AppendedData>\n</VTKFile>\n";
  ok = ok && std::fwrite(tail.data(), 1, tail.size(), fp) == tail.size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? SVGPU_OK : fail(ctx, SVGPU_EINVAL, std::string("write_vtu: write failed: ") + path);
}
