// Host check of the windowed band LU-SGS sweep's plan
// (meshcfd_gb300/csrc/mcfd_window_plan.h): a sweep executed from the plan
// the way k_lusgs_window executes it (per window and block: externals into
// slots, the closure's rows level by level from slots, own rows to the
// global solution) gives the forward substitution of the natural order bit
// for bit, every recomputed row equals its owner's, every row is owned once,
// and the plan keeps its limits.
//
// usage: window_plan_check SEED -> prints "cases=<n> planned=<k> failures=<m>" (k: the cases
// the limits let the planner plan), exits 0 when m == 0.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../meshcfd_gb300/csrc/mcfd_window_plan.h"

typedef unsigned long long u64;
static u64 g_state;
static u64 next_u64() {
  u64 z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double uniform() { return (double)(next_u64() >> 11) * 0x1p-53; }
static u64 bits(double x) {
  u64 b;
  memcpy(&b, &x, 8);
  return b;
}

static long g_cases = 0, g_planned = 0, g_fail = 0;
static void fail(const char* what, int a, int b) {
  if (g_fail < 5) printf("failure: %s (%d, %d)\n", what, a, b);
  ++g_fail;
}

// A lower-triangular pattern on C cells: rows' lower neighbours (ascending).
static std::vector<std::vector<int>> grid_pattern(int nx, int ny, int extra, bool permute) {
  const int C = nx * ny;
  std::vector<int> id(C);
  for (int c = 0; c < C; ++c) id[c] = c;
  if (permute)
    for (int c = C - 1; c > 0; --c) std::swap(id[c], id[next_u64() % (u64)(c + 1)]);
  std::vector<std::vector<int>> nb(C);
  auto link = [&](int a, int b) {  // an undirected coupling between cells a, b
    nb[a].push_back(b);
    nb[b].push_back(a);
  };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      if (i + 1 < nx) link(id[i + nx * j], id[i + 1 + nx * j]);
      if (j + 1 < ny) link(id[i + nx * j], id[i + nx * (j + 1)]);
    }
  for (int e = 0; e < extra; ++e) {  // a few long-range couplings
    const int a = (int)(next_u64() % (u64)C), b = (int)(next_u64() % (u64)C);
    if (a != b) link(a, b);
  }
  std::vector<std::vector<int>> lower(C);
  for (int c = 0; c < C; ++c) {
    for (int d : nb[c])
      if (d < c) lower[c].push_back(d);
    std::sort(lower[c].begin(), lower[c].end());
    lower[c].erase(std::unique(lower[c].begin(), lower[c].end()), lower[c].end());
  }
  return lower;
}

static void run_case(const std::vector<std::vector<int>>& lower, int nc, mcfd::WindowLimits lim, int wide) {
  ++g_cases;
  const int C = (int)lower.size();
  // levels and sweep order (by level, stable in cell id), entries' positions
  std::vector<int> lev(C, 0);
  int nlev = 0;
  for (int c = 0; c < C; ++c) {
    for (int d : lower[c]) lev[c] = std::max(lev[c], lev[d] + 1);
    nlev = std::max(nlev, lev[c] + 1);
  }
  std::vector<int> level_ptr(nlev + 1, 0), pos_cell(C), pos_of(C);
  for (int c = 0; c < C; ++c) level_ptr[lev[c] + 1]++;
  for (int l = 0; l < nlev; ++l) level_ptr[l + 1] += level_ptr[l];
  std::vector<int> fill(level_ptr.begin(), level_ptr.end() - 1);
  for (int c = 0; c < C; ++c) {
    pos_of[c] = fill[lev[c]]++;
    pos_cell[pos_of[c]] = c;
  }
  std::vector<int> ent_ptr(C + 1, 0), ent_pos, ent_cell;
  for (int p = 0; p < C; ++p) {
    for (int d : lower[pos_cell[p]]) {
      ent_pos.push_back(pos_of[d]);
      ent_cell.push_back(d);
    }
    ent_ptr[p + 1] = (int)ent_pos.size();
  }
  // runs: levels wider than `wide` are runs of their own without windows
  std::vector<int> runs;
  for (int l = 0; l < nlev;) {
    if (level_ptr[l + 1] - level_ptr[l] > wide) {
      runs.insert(runs.end(), {0, l, l + 1});
      ++l;
      continue;
    }
    int l1 = l;
    while (l1 < nlev && level_ptr[l1 + 1] - level_ptr[l1] <= wide) ++l1;
    runs.insert(runs.end(), {1, l, l1});
    l = l1;
  }
  mcfd::WindowPlanHost W;
  const bool ok = mcfd::plan_windows_host(level_ptr, pos_cell, ent_ptr, ent_pos, runs, C, nc, lim, W);
  if (!ok) return;  // the sweep would take another engine: nothing to check
  ++g_planned;
  // values: entries, diagonal, right-hand side (4 components)
  std::vector<double> val(ent_pos.size()), diag(C), rhs(4 * (size_t)C);
  for (double& v : val) v = uniform() - 0.5;
  for (double& d : diag) d = 1.0 + 3.0 * uniform();
  for (double& r : rhs) r = uniform() * 2.0 - 1.0;
  // the forward substitution in the natural order: acc = r, acc -= v x per
  // entry in ascending column order, x = acc / d
  std::vector<double> ref(4 * (size_t)C);
  for (int c = 0; c < C; ++c)
    for (int k = 0; k < 4; ++k) {
      const int p = pos_of[c];
      double acc = rhs[4 * (size_t)c + k];
      for (int j = ent_ptr[p]; j < ent_ptr[p + 1]; ++j) acc = acc - val[j] * ref[4 * (size_t)ent_cell[j] + k];
      ref[4 * (size_t)c + k] = acc / diag[c];
    }
  // the plan's execution
  std::vector<double> x(4 * (size_t)C, NAN);
  std::vector<int> owned(C, 0);
  const int n_runs = (int)runs.size() / 3;
  for (int si = 0; si < n_runs; ++si) {
    if (!runs[3 * si]) {  // a wide level: every row from global memory
      for (int p = level_ptr[runs[3 * si + 1]]; p < level_ptr[runs[3 * si + 2]]; ++p) {
        const int c = pos_cell[p];
        ++owned[c];
        for (int k = 0; k < 4; ++k) {
          double acc = rhs[4 * (size_t)c + k];
          for (int j = ent_ptr[p]; j < ent_ptr[p + 1]; ++j) acc = acc - val[j] * x[4 * (size_t)ent_cell[j] + k];
          x[4 * (size_t)c + k] = acc / diag[c];
        }
      }
      if (W.run_w0[si] != W.run_w0[si + 1]) fail("windows on a wide run", si, 0);
      continue;
    }
    for (int w = W.run_w0[si]; w < W.run_w0[si + 1]; ++w) {
      const int nl = W.l1[w] - W.l0[w];
      if (nl < 1 || nl > lim.max_levels) fail("window length", w, nl);
      std::vector<std::vector<double>> ghosts;  // (cell, values) of recomputed rows
      std::vector<int> ghost_cells;
      for (int k = 0; k < nc; ++k) {
        const int r0 = W.stage[4 * (w * nc + k)], nr = W.stage[4 * (w * nc + k) + 1];
        const int e0 = W.stage[4 * (w * nc + k) + 2], ne = W.stage[4 * (w * nc + k) + 3];
        if (nr > lim.max_rows || ne > lim.max_ext) fail("staging limits", nr, ne);
        std::vector<double> sl(4 * (size_t)lim.max_slots, NAN);
        for (int e = e0; e < e0 + ne; ++e) {
          const int slot = W.ext[2 * e], c = W.ext[2 * e + 1];
          if (slot >= lim.max_slots) fail("external slot", slot, c);
          if (level_ptr[W.l0[w]] <= pos_of[c]) fail("external inside the window", c, w);
          for (int q = 0; q < 4; ++q) sl[4 * (size_t)slot + q] = x[4 * (size_t)c + q];
        }
        const int g0 = W.gbase[w] + k * (nl + 1);
        if (W.grp[g0] != r0 || W.grp[g0 + nl] != r0 + nr) fail("level ranges", w, k);
        for (int m = 0; m < nl; ++m)
          for (int r = W.grp[g0 + m]; r < W.grp[g0 + m + 1]; ++r) {
            const int* R = &W.rec[8 * (size_t)r];
            const bool own = R[0] >= 0;
            const int p = own ? R[0] : ~R[0], c = R[1], slot = R[2] & 0xffff, n = R[2] >> 16;
            if (pos_cell[p] != c || n != ent_ptr[p + 1] - ent_ptr[p]) fail("record", r, p);
            if (lev[c] != W.l0[w] + m) fail("record level", r, lev[c]);
            if (own != (c / W.band_rows == k)) fail("ownership", r, k);
            if (slot >= lim.max_slots) fail("slot", r, slot);
            std::vector<double> res(4);
            for (int q = 0; q < 4; ++q) {
              double acc = rhs[4 * (size_t)c + q];
              for (int e = 0; e < n; ++e) {
                const int s = e < 4 ? R[4 + e] : W.eslot[R[3] + e];
                if (s != W.eslot[R[3] + e]) fail("packed entry slot", r, e);
                acc = acc - val[ent_ptr[p] + e] * sl[4 * (size_t)s + q];
              }
              res[q] = acc / diag[c];
              sl[4 * (size_t)slot + q] = res[q];
            }
            if (own) {
              ++owned[c];
              for (int q = 0; q < 4; ++q) x[4 * (size_t)c + q] = res[q];
            } else {
              ghosts.push_back(res);
              ghost_cells.push_back(c);
            }
          }
      }
      for (size_t g = 0; g < ghosts.size(); ++g)  // recomputed rows: the owner's bits
        for (int q = 0; q < 4; ++q)
          if (bits(ghosts[g][q]) != bits(x[4 * (size_t)ghost_cells[g] + q])) fail("recomputed row", ghost_cells[g], q);
    }
  }
  for (int c = 0; c < C; ++c) {
    if (owned[c] != 1) fail("row owned", c, owned[c]);
    for (int q = 0; q < 4; ++q)
      if (bits(x[4 * (size_t)c + q]) != bits(ref[4 * (size_t)c + q])) {
        fail("solution", c, q);
        break;
      }
  }
}

int main(int argc, char** argv) {
  g_state = argc > 1 ? strtoull(argv[1], nullptr, 10) : 1;
  const mcfd::WindowLimits roomy{32, 2048, 560, 512}, tight{16, 96, 60, 40}, tiny{8, 24, 16, 12};
  for (int trial = 0; trial < 6; ++trial) {
    const int nx = 8 + (int)(next_u64() % 60), ny = 4 + (int)(next_u64() % 40);
    for (int extra : {0, 3, 40})
      for (bool permute : {false, true})
        for (int nc : {8, 16})
          for (const mcfd::WindowLimits& lim : {roomy, tight, tiny})
            for (int wide : {1 << 30, 24}) {
              run_case(grid_pattern(nx, ny, extra, permute), nc, lim, wide);
            }
  }
  printf("cases=%ld planned=%ld failures=%ld\n", g_cases, g_planned, g_fail);
  return g_fail ? 1 : 0;
}
