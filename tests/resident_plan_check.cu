// Host-side check of the resident solvers' plan (build_patch_plan in
// eol-cloth_gb300/csrc/patch.cu) for a BSR pattern read from a file:
//   * the device's warp-compacted record and slot positions, replayed on the
//     CPU, stay inside the patch's image and visit every record once;
//   * every record's block lies in its row, with the column / halo node its
//     word names; every internal upper record writes a distinct slot, which
//     is the slot row `col` gathers for column `row`;
//   * image capacities (records, slots, halo nodes) hold;
//   * coarse plan: each patch's own aggregate is its first target, every
//     halo node's aggregate is listed, the contributor lists hold exactly the
//     (patch, target) records of each aggregate pair, patches in order.
// Prints "problems N" and exits 1 when N > 0.  Test infrastructure only.
#include "../eol-cloth_gb300/csrc/patch.cu"

#include <cstdio>

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int N = 0, NB = 0;
  if (fread(&N, 4, 1, f) != 1 || fread(&NB, 4, 1, f) != 1) return 2;
  std::vector<int> rowptr(N + 1), colidx(NB);
  std::vector<double> X(2 * size_t(N));
  if (fread(rowptr.data(), 4, N + 1, f) != size_t(N + 1) ||
      fread(colidx.data(), 4, NB, f) != size_t(NB) ||
      fread(X.data(), 8, 2 * size_t(N), f) != 2 * size_t(N))
    return 2;
  fclose(f);
  using namespace eolc;
  PatchPlan L, L1;
  const std::string why = build_patch_plan(N, rowptr, colidx, &X, 152, L);
  if (!why.empty()) {
    printf("misfit: %s\n", why.c_str());
    return 3;
  }
  long bad = 0;
  // the threaded build equals the single-threaded one, array for array
  if (!build_patch_plan(N, rowptr, colidx, &X, 152, L1, 1).empty()) ++bad;
  const bool same =
      L.G == L1.G && L.perm == L1.perm && L.rowptr == L1.rowptr && L.colidx == L1.colidx &&
      L.src == L1.src && L.tr == L1.tr && L.diag == L1.diag && L.patch_row == L1.patch_row &&
      L.hnptr == L1.hnptr && L.hnode == L1.hnode && L.fptr == L1.fptr && L.fblk == L1.fblk &&
      L.rcnt == L1.rcnt && L.wbase == L1.wbase && L.fword == L1.fword &&
      L.n_agg == L1.n_agg && L.patch_agg == L1.patch_agg && L.hagg == L1.hagg &&
      L.ctgt == L1.ctgt && L.cl_ptr == L1.cl_ptr && L.cl_idx == L1.cl_idx && L.bsl == L1.bsl &&
      L.gsrc == L1.gsrc && L.slice_off == L1.slice_off && L.slice_len == L1.slice_len;
  if (!same) {
    printf("threaded plan differs from the single-threaded plan\n");
    ++bad;
  }
  int max_rec = 0, max_slot = 0;
  std::vector<int> patch_of(N);
  for (int c = 0; c < L.G; ++c)
    for (int i = L.patch_row[c]; i < L.patch_row[c + 1]; ++i) patch_of[i] = c;
  for (int c = 0; c < L.G; ++c) {
    const int p0 = L.patch_row[c], np = L.patch_row[c + 1] - p0;
    const int f0 = L.fptr[c], nrec = L.fptr[c + 1] - f0;
    const int hb = L.hnptr[c], nh = L.hnptr[c + 1] - hb;
    if (np > kMaxRows || nrec > kMaxFwd || nh > kMaxHaloNodes) ++bad;
    int nslot = 0;
    for (int i = 0; i < np; ++i) nslot += (L.rcnt[p0 + i] >> 16) & 0xff;
    if (nslot > kMaxSlots) ++bad;
    max_rec = std::max(max_rec, nrec);
    max_slot = std::max(max_slot, nslot);
    std::vector<int> seen(nrec, 0), writer(nslot, 0), gathered(nslot, -1);
    int fi[kWarps][32], ft[kWarps][32], tc[kWarps][32];
    for (int w = 0; w < kWarps; ++w)
      for (int l = 0; l < 32; ++l) {
        const int i = 32 * w + l, rc = i < np ? L.rcnt[p0 + i] : 0;
        fi[w][l] = rc & 0xff;
        ft[w][l] = (rc >> 8) & 0xff;
        tc[w][l] = (rc >> 16) & 0xff;
      }
    for (int w = 0; w < kWarps; ++w) {  // gather positions: slot -> gathering row
      int sb = L.wbase[2 * (c * kWarps + w) + 1], tmax = 0;
      for (int l = 0; l < 32; ++l) tmax = std::max(tmax, tc[w][l]);
      for (int k = 0; k < tmax; ++k) {
        unsigned act = 0;
        for (int l = 0; l < 32; ++l) if (k < tc[w][l]) act |= 1u << l;
        for (int l = 0; l < 32; ++l) {
          if (!(k < tc[w][l])) continue;
          const int q = sb + __builtin_popcount(act & ((1u << l) - 1u));
          if (q < 0 || q >= nslot || gathered[q] >= 0) { ++bad; continue; }
          gathered[q] = 32 * w + l;
        }
        sb += __builtin_popcount(act);
      }
    }
    for (int w = 0; w < kWarps; ++w) {  // forward records
      int base = L.wbase[2 * (c * kWarps + w)], kmax = 0;
      for (int l = 0; l < 32; ++l) kmax = std::max(kmax, ft[w][l]);
      for (int k = 0; k < kmax; ++k) {
        unsigned act = 0;
        for (int l = 0; l < 32; ++l) if (k < ft[w][l]) act |= 1u << l;
        for (int l = 0; l < 32; ++l) {
          if (!(k < ft[w][l])) continue;
          const int e = base + __builtin_popcount(act & ((1u << l) - 1u));
          if (e < 0 || e >= nrec) { ++bad; continue; }
          seen[e]++;
          const unsigned word = L.fword[f0 + e];
          const int col = int(word & 0xffffu), sl = int(word >> 16), blk = L.fblk[f0 + e];
          const int row = p0 + 32 * w + l;
          if (blk < L.rowptr[row] || blk >= L.rowptr[row + 1]) { ++bad; continue; }
          const int gcol = L.colidx[blk];
          if (col < kMaxRows) {
            if (gcol != p0 + col || col <= 32 * w + l || k >= fi[w][l]) ++bad;
            if (sl == 0xffff || sl >= nslot) { ++bad; continue; }
            writer[sl]++;
            if (gathered[sl] != col) ++bad;  // the row that gathers this slot
          } else {
            const int h = col - kMaxRows;
            if (h >= nh || L.hnode[hb + h] != gcol || sl != 0xffff || k < fi[w][l]) ++bad;
          }
        }
        base += __builtin_popcount(act);
      }
    }
    for (int e = 0; e < nrec; ++e) bad += seen[e] != 1;
    for (int q = 0; q < nslot; ++q) bad += writer[q] != 1;
    // coarse plan
    const int *t = L.ctgt.data() + size_t(c) * kMaxTgt;
    if (t[0] != L.patch_agg[c]) ++bad;
    int nt = 0;
    while (nt < kMaxTgt && t[nt] >= 0) ++nt;
    for (int q = 0; q < nt; ++q) bad += t[q] >= L.n_agg;
    for (int h = hb; h < hb + nh; ++h) {
      const int aj = L.patch_agg[patch_of[L.hnode[h]]];
      if (L.hagg[h] != aj) ++bad;
      bool listed = false;
      for (int q = 0; q < nt; ++q) listed |= t[q] == aj;
      if (!listed) ++bad;
    }
  }
  for (int a = 0; a < L.n_agg; ++a)
    for (int b = 0; b < L.n_agg; ++b) {
      std::vector<int> want;
      for (int c = 0; c < L.G; ++c) {
        if (L.patch_agg[c] != a) continue;
        for (int q = 0; q < kMaxTgt && L.ctgt[size_t(c) * kMaxTgt + q] >= 0; ++q)
          if (L.ctgt[size_t(c) * kMaxTgt + q] == b) want.push_back(c * kMaxTgt + q);
      }
      const int r0 = L.cl_ptr[size_t(a) * L.n_agg + b], r1 = L.cl_ptr[size_t(a) * L.n_agg + b + 1];
      if (r1 - r0 != int(want.size()) || !std::equal(want.begin(), want.end(), L.cl_idx.begin() + r0))
        ++bad;
    }
  printf("patches %d records max %d of %d slots max %d of %d aggregates %d problems %ld\n", L.G,
         max_rec, kMaxFwd, max_slot, kMaxSlots, L.n_agg, bad);
  return bad ? 1 : 0;
}
