// Host helper: the two-ring stencil of the MUSCL-parabolic reconstruction.
//
// _parabolic_stencil (solver.py:2241-2291) builds, for every cell, the cells
// reached in two steps of the gradient adjacency (entries in the reference's
// order), with the offset accumulated along the path; a (cell, offset) pair
// is visited once, offsets compared after rounding offset / domain_scale to
// 10 decimals (Python's round: the correctly rounded decimal, ties to
// even), and the pairs whose offset is not ~zero are kept in visiting order.
// This is the same breadth-first search per source cell, in C++ and spread
// over host threads (each thread a contiguous range of sources, results
// concatenated in source order), so the output equals the reference's list
// entry for entry.  The decimal rounding is printf("%.10f") followed by
// strtod, both exact; it is only evaluated when two candidates reach the
// same cell, which is the only time the keys are compared.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "../../include/meshcfd_gb300.h"

namespace {

double round10(double x) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.10f", x);
  return std::strtod(buf, nullptr);
}

struct Visit {
  long long cell;
  double x, y;
  bool keyed;
  double kx, ky;
};

struct Out {
  std::vector<long long> s, n;
  std::vector<double> x, y;
};

void stencil_range(long long c0, long long c1, const std::vector<long long>& start,
                   const std::vector<long long>& adj_n, const std::vector<double>& adj_x,
                   const std::vector<double>& adj_y, double scale, Out& out) {
  std::vector<Visit> seen, frontier, next;
  auto key = [&](Visit& v) {
    if (!v.keyed) {
      v.kx = round10(v.x / scale);
      v.ky = round10(v.y / scale);
      v.keyed = true;
    }
  };
  for (long long source = c0; source < c1; ++source) {
    seen.clear();
    frontier.clear();
    seen.push_back(Visit{source, 0.0, 0.0, true, 0.0, 0.0});  // the reference's (source, 0, 0)
    frontier.push_back(Visit{source, 0.0, 0.0, true, 0.0, 0.0});
    for (int depth = 0; depth < 2; ++depth) {
      next.clear();
      for (const Visit& cur : frontier) {
        for (long long k = start[cur.cell]; k < start[cur.cell + 1]; ++k) {
          Visit cand{adj_n[k], cur.x + adj_x[k], cur.y + adj_y[k], false, 0.0, 0.0};
          bool dup = false;
          for (Visit& s : seen) {
            if (s.cell != cand.cell) continue;
            key(s);
            key(cand);
            if (s.kx == cand.kx && s.ky == cand.ky) {  // -0.0 == 0.0, as Python's tuple keys
              dup = true;
              break;
            }
          }
          if (dup) continue;
          seen.push_back(cand);
          next.push_back(cand);
          if (std::hypot(cand.x, cand.y) > scale * 1e-12) {
            out.s.push_back(source);
            out.n.push_back(cand.cell);
            out.x.push_back(cand.x);
            out.y.push_back(cand.y);
          }
        }
      }
      frontier.swap(next);
    }
  }
}

}  // namespace

extern "C" int mcfd_host_parabolic_stencil(int64_t n_cells, int64_t n_entries, const int64_t* sources,
                                           const int64_t* neighbours, const double* dx, const double* dy,
                                           double domain_scale, int64_t capacity, int64_t* out_sources,
                                           int64_t* out_neighbours, double* out_dx, double* out_dy,
                                           int64_t* out_count) {
  if (n_cells < 0 || n_entries < 0 || capacity < 0 || !out_count || !(domain_scale > 0.0)) return MCFD_E_ARG;
  if (n_entries && (!sources || !neighbours || !dx || !dy)) return MCFD_E_ARG;
  for (int64_t e = 0; e < n_entries; ++e)
    if (sources[e] < 0 || sources[e] >= n_cells || neighbours[e] < 0 || neighbours[e] >= n_cells)
      return MCFD_E_GEOMETRY;
  // adjacency in entry order per source (a stable counting sort)
  std::vector<long long> start(n_cells + 1, 0), adj_n(n_entries);
  std::vector<double> adj_x(n_entries), adj_y(n_entries);
  for (int64_t e = 0; e < n_entries; ++e) start[sources[e] + 1]++;
  for (int64_t c = 0; c < n_cells; ++c) start[c + 1] += start[c];
  {
    std::vector<long long> fill(start.begin(), start.end() - 1);
    for (int64_t e = 0; e < n_entries; ++e) {
      const long long k = fill[sources[e]]++;
      adj_n[k] = neighbours[e];
      adj_x[k] = dx[e];
      adj_y[k] = dy[e];
    }
  }
  unsigned hw = std::thread::hardware_concurrency();
  const long long threads = std::max<long long>(1, std::min<long long>(hw ? hw : 1, (n_cells + 4095) / 4096));
  std::vector<Out> parts(threads);
  std::vector<std::thread> pool;
  for (long long t = 0; t < threads; ++t) {
    const long long c0 = n_cells * t / threads, c1 = n_cells * (t + 1) / threads;
    pool.emplace_back(stencil_range, c0, c1, std::cref(start), std::cref(adj_n), std::cref(adj_x),
                      std::cref(adj_y), domain_scale, std::ref(parts[t]));
  }
  for (std::thread& th : pool) th.join();
  int64_t total = 0;
  for (const Out& p : parts) total += (int64_t)p.s.size();
  *out_count = total;
  if (total > capacity) return MCFD_E_ARG;
  if (total && (!out_sources || !out_neighbours || !out_dx || !out_dy)) return MCFD_E_ARG;
  int64_t k = 0;
  for (const Out& p : parts) {
    for (size_t i = 0; i < p.s.size(); ++i, ++k) {
      out_sources[k] = p.s[i];
      out_neighbours[k] = p.n[i];
      out_dx[k] = p.x[i];
      out_dy[k] = p.y[i];
    }
  }
  return MCFD_OK;
}
