// CSR pattern of the element cliques (the reference's lhsa, solver/lhsa.cpp:153-380):
// for every node the sorted, unique list of nodes it shares an element with.  Host
// code; counting sort by row, then a small sort per row.
#include <algorithm>
#include <vector>

#include "../../include/svgpu.h"

extern "C" int svgpu_lhsa(int nNo, int nEl, int eNoN, const int* IEN, int* rowPtr, int* colPtr, long long* nnz) {
  if (nNo <= 0 || nEl < 0 || eNoN <= 0 || !IEN || !rowPtr || !nnz) return SVGPU_EINVAL;
  std::vector<long long> cnt((size_t)nNo + 1, 0);
  for (long long e = 0; e < nEl; e++)
    for (int a = 0; a < eNoN; a++) {
      const int r = IEN[eNoN * e + a];
      if (r < 0 || r >= nNo) return SVGPU_EINVAL;
      cnt[r + 1] += eNoN;
    }
  for (int i = 0; i < nNo; i++) cnt[i + 1] += cnt[i];
  std::vector<int> raw((size_t)cnt[nNo]);
  std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
  for (long long e = 0; e < nEl; e++)
    for (int a = 0; a < eNoN; a++) {
      const int r = IEN[eNoN * e + a];
      for (int b = 0; b < eNoN; b++) raw[fill[r]++] = IEN[eNoN * e + b];
    }
  long long total = 0;
  rowPtr[0] = 0;
  for (int r = 0; r < nNo; r++) {
    int* s = raw.data() + cnt[r];
    int* e = raw.data() + cnt[r + 1];
    if (s == e) return SVGPU_EINVAL;  // isolated node
    std::sort(s, e);
    e = std::unique(s, e);
    const long long m = e - s;
    if (colPtr) std::copy(s, e, colPtr + total);
    total += m;
    if (total > 0x7fffffffLL) return SVGPU_EINVAL;
    rowPtr[r + 1] = (int)total;
  }
  *nnz = total;
  return SVGPU_OK;
}
