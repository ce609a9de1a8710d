// Host-side structure builders: node-block sparsity, the destination-sorted
// element-to-block contribution map used by the atomic-free assembly, and the
// node-to-element incidence used by the residual gather.
//
// The block pattern is the node graph of the element connectivity (two nodes
// are coupled when they share an element), the same graph GraphT::MakeGraph
// builds for the reference's MSR structure (toolbox/src/graph/GraphT.cpp:90,
// MSRBuilderT.cpp:16-175).  Expanded to dofs and restricted to active
// equations it is the reference's MSR pattern exactly.
#include <algorithm>
#include <thread>
#include <vector>

#include "tg_internal.h"

namespace tg {

namespace {
int hw_threads() {
  unsigned n = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(n, 32u));
}

template <typename F>
void parallel_for(int n, F f) {
  int nt = std::min(hw_threads(), std::max(1, n / 4096));
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  int chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    int lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo < hi) th.emplace_back(f, lo, hi);
  }
  for (auto& x : th) x.join();
}
}  // namespace

void build_node_elem(int nnd, int nel, const int* conn, std::vector<int>& ptr, std::vector<int>& list) {
  ptr.assign(nnd + 1, 0);
  for (long long k = 0; k < (long long)nel * 8; ++k) ptr[conn[k] + 1]++;
  for (int i = 0; i < nnd; ++i) ptr[i + 1] += ptr[i];
  list.assign((size_t)nel * 8, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  // ascending (e, a) order per node: deterministic gather order
  for (int e = 0; e < nel; ++e)
    for (int a = 0; a < 8; ++a) list[fill[conn[e * 8 + a]]++] = e * 8 + a;
}

void build_block_pattern(int nnd, int nel, const int* conn, std::vector<int>& rowptr, std::vector<int>& col) {
  std::vector<int> nptr, nlist;
  build_node_elem(nnd, nel, conn, nptr, nlist);
  std::vector<int> count(nnd, 0);
  std::vector<std::vector<int>> rows(nnd);
  parallel_for(nnd, [&](int lo, int hi) {
    std::vector<int> tmp;
    for (int i = lo; i < hi; ++i) {
      tmp.clear();
      for (int k = nptr[i]; k < nptr[i + 1]; ++k) {
        int e = nlist[k] >> 3;
        for (int b = 0; b < 8; ++b) tmp.push_back(conn[e * 8 + b]);
      }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      rows[i] = tmp;
      count[i] = (int)tmp.size();
    }
  });
  rowptr.assign(nnd + 1, 0);
  for (int i = 0; i < nnd; ++i) rowptr[i + 1] = rowptr[i] + count[i];
  col.resize(rowptr[nnd]);
  parallel_for(nnd, [&](int lo, int hi) {
    for (int i = lo; i < hi; ++i) std::copy(rows[i].begin(), rows[i].end(), col.begin() + rowptr[i]);
  });
}

// Contribution (e, a, b) -> block (conn[e][a], conn[e][b]); grouped by
// destination block, ascending (e, a, b) within a block so that the
// segmented reduction adds in a fixed order (bitwise repeatable).
void build_contrib_map(int nnd, int nel, const int* conn, const std::vector<int>& rowptr,
                       const std::vector<int>& col, std::vector<int>& cptr, std::vector<int>& contrib) {
  const long long nnzb = rowptr[nnd];
  std::vector<int> dest((size_t)nel * 64);
  parallel_for(nel, [&](int lo, int hi) {
    for (int e = lo; e < hi; ++e)
      for (int a = 0; a < 8; ++a) {
        int row = conn[e * 8 + a];
        const int* c0 = col.data() + rowptr[row];
        const int* c1 = col.data() + rowptr[row + 1];
        for (int b = 0; b < 8; ++b) {
          const int* p = std::lower_bound(c0, c1, conn[e * 8 + b]);
          dest[(size_t)e * 64 + a * 8 + b] = (int)(p - col.data());
        }
      }
  });
  cptr.assign(nnzb + 1, 0);
  for (size_t k = 0; k < dest.size(); ++k) cptr[dest[k] + 1]++;
  for (long long i = 0; i < nnzb; ++i) cptr[i + 1] += cptr[i];
  contrib.assign(dest.size(), 0);
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (size_t k = 0; k < dest.size(); ++k) contrib[fill[dest[k]]++] = (int)k;
}

// Scalar CSR over the active equations from the node-block pattern: row r
// (equation r+1) lists the equations of the dofs of every node coupled to its
// node, ascending, prescribed dofs left out (and, with upper_only, columns
// below the diagonal).  row_ptr / col_idx may be NULL (count only).
void expand_pattern(int nnd, const int* eq, const std::vector<int>& rowptr, const std::vector<int>& col,
                    bool upper_only, int* row_ptr, int* col_idx, long long* nnz) {
  long long count = 0;
  if (row_ptr) row_ptr[0] = 0;
  int row = 0;
  for (int I = 0; I < nnd; ++I)
    for (int p = 0; p < 3; ++p) {
      const int r = eq[I * 3 + p];
      if (r <= 0) continue;
      for (int k = rowptr[I]; k < rowptr[I + 1]; ++k) {
        const int J = col[k];
        for (int q = 0; q < 3; ++q) {
          const int cc = eq[J * 3 + q];
          if (cc <= 0 || (upper_only && cc < r)) continue;
          if (col_idx) col_idx[count] = cc - 1;
          ++count;
        }
      }
      ++row;
      if (row_ptr) row_ptr[row] = (int)count;
    }
  if (nnz) *nnz = count;
}

}  // namespace tg
