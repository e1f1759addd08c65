// Host planner of the windowed band LU-SGS sweep (k_lusgs_window in
// mcfd_implicit.cu), plain C++ so that it also compiles without CUDA.
//
// Input: one sweep's rows in sweep order (positions, level by level), each
// row's entries (column positions, in the row's entry order), and the runs
// of levels that one cluster launch sweeps.  Block k of an nc-block cluster
// owns the cells [k * band_rows, (k + 1) * band_rows).  Each run is cut into
// windows of at most max_levels levels (shortened by a quarter at a time
// where a block's closure would not fit); for window w and block k the plan
// lists, contiguously:
//   level ranges grp[gbase[w] + k * (nl + 1) + m], m = 0..nl (record indices);
//   stage[4 (w nc + k) ..] = first record, records, first external, externals;
//   per record r (8 ints): position (~position for a row of another band),
//     cell, slot | entries << 16, start of its entries' slots in eslot, and
//     its first four entry slots;
//   per external e (2 ints): its slot, its cell.
// The closure of block k's own rows in a window: the rows of any band they
// depend on inside the window (recomputed by k) and the solutions from
// before the window they read (the externals).  Slots number the externals
// first, then the window's rows level by level.
#pragma once

#include <algorithm>
#include <cstddef>
#include <vector>

namespace mcfd {

struct WindowPlanHost {
  int nc = 0, band_rows = 0, n_records = 0;
  bool ok = false;
  std::vector<int> l0, l1, gbase, grp, stage, rec, eslot, ext;
  std::vector<int> run_w0;  // first window of each run (one more entry: the end)
};

struct WindowLimits {
  int max_levels, max_slots, max_rows, max_ext;
};

// runs: (wavefront, first level, end level) per schedule entry; entries
// that are not wavefront runs get no windows.
inline bool plan_windows_host(const std::vector<int>& level_ptr, const std::vector<int>& pos_cell,
                              const std::vector<int>& ent_ptr, const std::vector<int>& ent_pos,
                              const std::vector<int>& runs, int C, int nc, const WindowLimits& lim,
                              WindowPlanHost& W) {
  W = WindowPlanHost{};
  W.nc = nc;
  W.band_rows = std::max(1, (C + nc - 1) / nc);
  const int nlev = (int)level_ptr.size() - 1;
  const int n_runs = (int)runs.size() / 3;
  std::vector<int> lev_of(C);
  for (int l = 0; l < nlev; ++l)
    for (int p = level_ptr[l]; p < level_ptr[l + 1]; ++p) lev_of[p] = l;
  std::vector<int> mark(C, -1), slot_of(C, -1);
  std::vector<std::vector<int>> by_level(lim.max_levels);
  std::vector<int> ext;
  int stamp = 0;
  auto closure = [&](int L0, int L1, int k) {
    ++stamp;
    const int base = level_ptr[L0], nl = L1 - L0;
    for (int m = 0; m < nl; ++m) by_level[m].clear();
    ext.clear();
    for (int m = 0; m < nl; ++m)
      for (int p = level_ptr[L0 + m]; p < level_ptr[L0 + m + 1]; ++p)
        if (pos_cell[p] / W.band_rows == k) {
          mark[p] = stamp;
          by_level[m].push_back(p);
        }
    for (int m = nl - 1; m >= 0; --m)  // dependencies lie on lower levels
      for (size_t x = 0; x < by_level[m].size(); ++x) {
        const int p = by_level[m][x];
        for (int j = ent_ptr[p]; j < ent_ptr[p + 1]; ++j) {
          const int q = ent_pos[j];
          if (mark[q] == stamp) continue;
          mark[q] = stamp;
          if (q >= base) by_level[lev_of[q] - L0].push_back(q);
          else ext.push_back(q);
        }
      }
    size_t rows = 0;
    for (int m = 0; m < nl; ++m) rows += by_level[m].size();
    return rows + ext.size() <= (size_t)lim.max_slots && rows <= (size_t)lim.max_rows &&
           ext.size() <= (size_t)lim.max_ext;
  };
  auto emit = [&](int L0, int L1, int k) {
    const int nl = L1 - L0;
    closure(L0, L1, k);
    std::sort(ext.begin(), ext.end());
    int sl = 0;
    const int r0 = (int)(W.rec.size() / 8), e0 = (int)(W.ext.size() / 2);
    for (int q : ext) {
      slot_of[q] = sl++;
      W.ext.push_back(slot_of[q]);
      W.ext.push_back(pos_cell[q]);
    }
    for (int m = 0; m < nl; ++m) {
      W.grp.push_back((int)(W.rec.size() / 8));
      std::vector<int>& rows = by_level[m];
      std::sort(rows.begin(), rows.end());
      for (int p : rows) {
        slot_of[p] = sl++;
        const int n = ent_ptr[p + 1] - ent_ptr[p];
        W.rec.push_back(pos_cell[p] / W.band_rows == k ? p : ~p);
        W.rec.push_back(pos_cell[p]);
        W.rec.push_back(slot_of[p] | (n << 16));
        W.rec.push_back((int)W.eslot.size());
        for (int q = 0; q < 4; ++q) W.rec.push_back(q < n ? slot_of[ent_pos[ent_ptr[p] + q]] : 0);
        for (int j = ent_ptr[p]; j < ent_ptr[p + 1]; ++j) W.eslot.push_back(slot_of[ent_pos[j]]);
      }
    }
    W.grp.push_back((int)(W.rec.size() / 8));
    W.stage.push_back(r0);
    W.stage.push_back((int)(W.rec.size() / 8) - r0);
    W.stage.push_back(e0);
    W.stage.push_back((int)(W.ext.size() / 2) - e0);
  };
  W.run_w0.assign(n_runs + 1, 0);
  bool ok = lim.max_slots < (1 << 16);  // the record's 16-bit slot
  for (int p = 0; p < C && ok; ++p) ok = ent_ptr[p + 1] - ent_ptr[p] < (1 << 15);  // and entry count
  for (int si = 0; si < n_runs && ok; ++si) {
    W.run_w0[si] = (int)W.l0.size();
    if (!runs[3 * si]) continue;
    const int end = runs[3 * si + 2];
    for (int L = runs[3 * si + 1]; L < end && ok;) {
      int H = std::min(lim.max_levels, end - L);
      for (;;) {
        bool fits = true;
        for (int k = 0; k < nc && fits; ++k) fits = closure(L, L + H, k);
        if (fits) break;
        if (H == 1) {
          ok = false;
          break;
        }
        H = std::max(1, H * 3 / 4);
      }
      if (!ok) break;
      W.l0.push_back(L);
      W.l1.push_back(L + H);
      W.gbase.push_back((int)W.grp.size());
      for (int k = 0; k < nc; ++k) emit(L, L + H, k);
      L += H;
    }
  }
  W.run_w0.back() = (int)W.l0.size();
  for (int si = n_runs; si-- > 0;)  // entries without windows: empty ranges
    if (!runs[3 * si]) W.run_w0[si] = W.run_w0[si + 1];
  W.ok = ok;
  W.n_records = (int)(W.rec.size() / 8);
  return ok;
}

}  // namespace mcfd
