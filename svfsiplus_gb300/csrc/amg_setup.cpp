// Host set-up of the aggregation hierarchy used by the multilevel preconditioner:
// greedy node aggregation of the block-CSR graph, the coarse block pattern of the
// Galerkin operator P^T K P with piecewise-constant P (one 4x4 identity per fine node
// in its aggregate), and the fine-block -> coarse-block lists the GPU sums.  The
// reference has no multilevel preconditioner in FSILS (its AMG lives in the Trilinos
// back-end, out of scope); this serves the learned/mixed paths only.
#include <algorithm>
#include <numeric>
#include <vector>

#include "amg.h"

namespace svgpu {

// Greedy aggregation (Vanek, Mandel & Brezina 1996, phases 1-3 without strength
// filtering): root nodes whose neighbourhood is untouched form an aggregate with all
// their neighbours; left-over nodes join a neighbouring aggregate; the rest stand alone.
// With labels (one per node), only neighbours of the root's label take part: the
// fluid-only and the solid nodes of the FSI equation, whose rows have different scales
// and physics, never share an aggregate.  clabel receives the aggregates' labels.
int aggregate_nodes(int n, const std::vector<int>& rowPtr, const std::vector<int>& colPtr, std::vector<int>& agg,
                    const std::vector<int>* label, std::vector<int>* clabel) {
  auto same = [&](int i, int j) { return !label || (*label)[i] == (*label)[j]; };
  agg.assign(n, -1);
  int na = 0;
  std::vector<int> root;
  for (int i = 0; i < n; i++) {
    bool free_nbhd = true;
    for (int k = rowPtr[i]; k < rowPtr[i + 1] && free_nbhd; k++)
      free_nbhd = !same(i, colPtr[k]) || agg[colPtr[k]] < 0;
    if (!free_nbhd) continue;
    for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++)
      if (same(i, colPtr[k])) agg[colPtr[k]] = na;
    root.push_back(i);
    na++;
  }
  std::vector<int> agg2 = agg;
  for (int i = 0; i < n; i++) {
    if (agg[i] >= 0) continue;
    for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++)
      if (agg[colPtr[k]] >= 0 && same(i, colPtr[k])) {
        agg2[i] = agg[colPtr[k]];
        break;
      }
  }
  for (int i = 0; i < n; i++)
    if (agg2[i] < 0) {
      agg2[i] = na++;
      root.push_back(i);
    }
  agg.swap(agg2);
  if (clabel) {
    clabel->assign(na, 0);
    if (label)
      for (int c = 0; c < na; c++) (*clabel)[c] = (*label)[root[c]];
  }
  return na;
}

// Coarse pattern of P^T K P and, for every coarse block, the list of fine blocks that
// sum into it (CSR: cPtr / fineIdx), in fixed order so the sums are deterministic.
void coarse_pattern(int n, int nc, const std::vector<int>& rowPtr, const std::vector<int>& colPtr,
                    const std::vector<int>& agg, std::vector<int>& cRow, std::vector<int>& cCol,
                    std::vector<int>& sumPtr, std::vector<int>& sumIdx) {
  const long nnz = rowPtr[n];
  std::vector<long long> key(nnz);
  for (int i = 0; i < n; i++)
    for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++) key[k] = (long long)agg[i] * nc + agg[colPtr[k]];
  std::vector<int> order(nnz);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  cRow.assign(nc + 1, 0);
  cCol.clear();
  sumPtr.clear();
  sumIdx.assign(order.begin(), order.end());
  long long last = -1;
  for (long p = 0; p < nnz; p++) {
    const long long kk = key[order[p]];
    if (kk != last) {
      cCol.push_back((int)(kk % nc));
      sumPtr.push_back((int)p);
      cRow[(int)(kk / nc) + 1]++;
      last = kk;
    }
  }
  sumPtr.push_back((int)nnz);
  for (int c = 0; c < nc; c++) cRow[c + 1] += cRow[c];
}

// Pattern of A P (fine rows x coarse columns) for P the aggregate injection: row i
// holds one block per distinct aggregate among its columns (ascending), and for every
// such block the list of A's blocks of row i whose column lies in that aggregate.
void ap_pattern(int n, const std::vector<int>& rowPtr, const std::vector<int>& colPtr, const std::vector<int>& agg,
                std::vector<int>& apRow, std::vector<int>& apCol, std::vector<int>& sumPtr, std::vector<int>& sumIdx) {
  apRow.assign(n + 1, 0);
  apCol.clear();
  sumPtr.clear();
  sumIdx.clear();
  sumIdx.reserve(rowPtr[n]);
  std::vector<std::pair<int, int>> row;
  for (int i = 0; i < n; i++) {
    row.clear();
    for (int k = rowPtr[i]; k < rowPtr[i + 1]; k++) row.emplace_back(agg[colPtr[k]], k);
    std::sort(row.begin(), row.end());
    int last = -1;
    for (auto& e : row) {
      if (e.first != last) {
        apCol.push_back(e.first);
        sumPtr.push_back((int)sumIdx.size());
        last = e.first;
      }
      sumIdx.push_back(e.second);
    }
    apRow[i + 1] = (int)apCol.size();
  }
  sumPtr.push_back((int)sumIdx.size());
}

}  // namespace svgpu
