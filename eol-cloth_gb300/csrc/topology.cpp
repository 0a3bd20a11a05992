// Host-side topology build: fixed BSR pattern, per-block contribution lists
// and node -> face incidence.  Runs once per topology (the reference rebuilds
// its triplet lists and re-sorts them every step in setFromTriplets,
// Forces.cpp:925-929; here the pattern is static and only values change).
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "internal.h"

namespace eolc {

std::string build_topology(int n_nodes, const int *tri, int n_tri,
                           const int *hinge, int n_hinge, HostTopology &out) {
  if (n_nodes <= 0 || n_tri < 0 || n_hinge < 0) return "bad sizes";
  if (int64_t(n_tri) + n_hinge >= (int64_t(1) << 26)) return "too many elements";
  for (int64_t k = 0; k < int64_t(n_tri) * 3; ++k)
    if (tri[k] < 0 || tri[k] >= n_nodes) return "triangle index out of range";
  for (int64_t k = 0; k < int64_t(n_hinge) * 4; ++k)
    if (hinge[k] < 0 || hinge[k] >= n_nodes) return "hinge index out of range";
  for (int t = 0; t < n_tri; ++t) {
    const int *v = tri + 3 * t;
    if (v[0] == v[1] || v[1] == v[2] || v[0] == v[2]) return "degenerate triangle";
  }
  for (int e = 0; e < n_hinge; ++e) {
    const int *v = hinge + 4 * e;
    for (int a = 0; a < 4; ++a)
      for (int b = a + 1; b < 4; ++b)
        if (v[a] == v[b]) return "degenerate hinge";
  }
  // One record per (element, row vertex, column vertex); the sequence number
  // keeps the reference's insertion order (faces, then hinges) stable.
  struct Rec {
    uint64_t key;  // row << 32 | col
    uint32_t seq;
    int code;
  };
  size_t n_rec = size_t(n_tri) * 9 + size_t(n_hinge) * 16;
  std::vector<Rec> rec;
  rec.reserve(n_rec);
  uint32_t seq = 0;
  for (int t = 0; t < n_tri; ++t)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        rec.push_back({(uint64_t(uint32_t(tri[3 * t + a])) << 32) |
                           uint32_t(tri[3 * t + b]),
                       seq++, contrib_code(t, false, a, b)});
  for (int e = 0; e < n_hinge; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        rec.push_back({(uint64_t(uint32_t(hinge[4 * e + a])) << 32) |
                           uint32_t(hinge[4 * e + b]),
                       seq++, contrib_code(e, true, a, b)});
  std::sort(rec.begin(), rec.end(), [](const Rec &x, const Rec &y) {
    return x.key < y.key || (x.key == y.key && x.seq < y.seq);
  });
  out = HostTopology();
  out.n_nodes = n_nodes;
  out.n_tri = n_tri;
  out.n_hinge = n_hinge;
  out.rowptr.assign(n_nodes + 1, 0);
  out.contrib.resize(rec.size());
  out.cptr.reserve(rec.size() / 4 + 2);
  out.cptr.push_back(0);
  uint64_t prev = ~uint64_t(0);
  for (size_t k = 0; k < rec.size(); ++k) {
    if (rec[k].key != prev) {
      if (k) out.cptr.push_back(int(k));
      prev = rec[k].key;
      int r = int(rec[k].key >> 32), c = int(rec[k].key & 0xffffffffu);
      out.colidx.push_back(c);
      out.blk_row.push_back(r);
      out.rowptr[r + 1]++;
    }
    out.contrib[k] = rec[k].code;
  }
  out.cptr.push_back(int(rec.size()));
  out.n_blocks = int(out.colidx.size());
  for (int i = 0; i < n_nodes; ++i) out.rowptr[i + 1] += out.rowptr[i];
  out.diag.assign(n_nodes, -1);
  for (int i = 0; i < n_nodes; ++i)
    for (int q = out.rowptr[i]; q < out.rowptr[i + 1]; ++q)
      if (out.colidx[q] == i) out.diag[i] = q;
  for (int i = 0; i < n_nodes; ++i)
    if (out.diag[i] < 0) return "node without any element";
  // node -> incident faces, in face order
  out.nf_ptr.assign(n_nodes + 1, 0);
  for (int t = 0; t < n_tri; ++t)
    for (int a = 0; a < 3; ++a) out.nf_ptr[tri[3 * t + a] + 1]++;
  for (int i = 0; i < n_nodes; ++i) out.nf_ptr[i + 1] += out.nf_ptr[i];
  out.nf_list.resize(size_t(n_tri) * 3);
  std::vector<int> pos(out.nf_ptr.begin(), out.nf_ptr.end() - 1);
  for (int t = 0; t < n_tri; ++t)
    for (int a = 0; a < 3; ++a) out.nf_list[pos[tri[3 * t + a]]++] = (t << 2) | a;
  return "";
}

}  // namespace eolc
