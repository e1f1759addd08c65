// Geometry build on the device: the numeric loops of _build_geometry
// (solver.py:1654-2105) as kernels, with the same operation order as the
// host helpers (mcfd_host_cell_geometry / mcfd_host_face_geometry) and the
// NumPy restatement in geometry.py, so the device build gives the host
// build's arrays bit for bit.  The topology (faces of cells, periodic
// matching, boundary classification, the order of the entry lists) stays on
// the host; these kernels take the index lists and fill every float array.
//
// * cell geometry: per cell, the shoelace sum of x0 y1 - x1 y0 in Python's
//   compensated order (Neumaier; CPython >= 3.12 sum()), the centroid sums,
//   centroid = sums / (3 * twice area), area = 0.5 |twice area|;
// * face geometry: per face, length sqrt(fma(ey, ey, ex ex)) (the FMA-based
//   BLAS dot of np.linalg.norm on the reference's platform), the unit normal
//   (ey, -ex) / length turned to point out of the owner by the sign of
//   fma(ny, dy, nx dx), the midpoint;
// * least-squares gradient coefficients (solver.py:2004-2078): per entry the
//   offset to the neighbour (periodic entries across the shift), weight
//   1 / max(|d|^2, 1e-300); per cell the weighted moment sums in the entry
//   order (np.add.at on zeros: 0.0 + first term, then in order), the
//   determinant test det > 1e-14 max(mxx myy, 1e-300) and the inverse; per
//   entry cx = ixx w dx + ixy w dy, cy = ixy w dx + iyy w dy;
// * limiter entries: face centre minus cell centre.
// Compiled with -fmad=false: no product is contracted unless written as fma.
#include <cstdint>

#include "mcfd_device.cuh"
#include "mcfd_internal.h"

namespace mcfd {
namespace {

constexpr int kGeomBlock = 256;

__global__ void __launch_bounds__(kGeomBlock) k_cell_geometry(long long n, const long long* __restrict__ off,
                                                              const long long* __restrict__ nodes,
                                                              const double* __restrict__ pts, double* __restrict__ centers,
                                                              double* __restrict__ areas,
                                                              unsigned long long* __restrict__ bad) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const long long b = off[c], k = off[c + 1] - b;
  double twice = 0.0, comp = 0.0;
  for (long long i = 0; i < k; ++i) {
    const double* p0 = pts + 2 * nodes[b + i];
    const double* p1 = pts + 2 * nodes[b + (i + 1) % k];
    const double x = p0[0] * p1[1] - p1[0] * p0[1];
    if (i == 0) {
      twice = x;
      continue;
    }
    const double t = twice + x;
    if (fabs(twice) >= fabs(x)) comp += (twice - t) + x;
    else comp += (x - t) + twice;
    twice = t;
  }
  if (comp != 0.0 && isfinite(comp)) twice += comp;
  if (!isfinite(twice) || fabs(twice) <= 1e-15) {
    atomicMin(bad, (unsigned long long)c);
    return;
  }
  double xs = 0.0, ys = 0.0;
  for (long long i = 0; i < k; ++i) {
    const double* p0 = pts + 2 * nodes[b + i];
    const double* p1 = pts + 2 * nodes[b + (i + 1) % k];
    const double cross = p0[0] * p1[1] - p1[0] * p0[1];
    xs += (p0[0] + p1[0]) * cross;
    ys += (p0[1] + p1[1]) * cross;
  }
  centers[2 * c] = xs / (3.0 * twice);
  centers[2 * c + 1] = ys / (3.0 * twice);
  areas[c] = 0.5 * fabs(twice);
}

__global__ void __launch_bounds__(kGeomBlock) k_face_geometry(long long n, const long long* __restrict__ fn,
                                                              const double* __restrict__ pts,
                                                              const double* __restrict__ centers,
                                                              const long long* __restrict__ owners,
                                                              double* __restrict__ fc, double* __restrict__ normals,
                                                              double* __restrict__ lengths,
                                                              unsigned long long* __restrict__ bad) {
  const long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (f >= n) return;
  const double* a = pts + 2 * fn[2 * f];
  const double* b = pts + 2 * fn[2 * f + 1];
  const double ex = b[0] - a[0], ey = b[1] - a[1];
  const double length = sqrt(__fma_rn(ey, ey, ex * ex));
  if (!isfinite(length) || length <= 1e-15) {
    atomicMin(bad, (unsigned long long)f);
    return;
  }
  double nx = ey / length, ny = -ex / length;
  const double cx = 0.5 * (a[0] + b[0]), cy = 0.5 * (a[1] + b[1]);
  const double* o = centers + 2 * owners[f];
  const double dx = cx - o[0], dy = cy - o[1];
  if (__fma_rn(ny, dy, nx * dx) < 0.0) {
    nx = -nx;
    ny = -ny;
  }
  fc[2 * f] = cx;
  fc[2 * f + 1] = cy;
  normals[2 * f] = nx;
  normals[2 * f + 1] = ny;
  lengths[f] = length;
}

// Per entry: offset to the neighbour and its weight; the entry list holds the
// interior entries (owner, then neighbour of each interior face) followed by
// the periodic ones (whose neighbour centre is shifted back by the period).
__global__ void __launch_bounds__(kGeomBlock) k_entry_offsets(long long n, long long n_interior_entries,
                                                              const long long* __restrict__ src,
                                                              const long long* __restrict__ nbr,
                                                              const double* __restrict__ centers,
                                                              const double* __restrict__ shift,
                                                              double* __restrict__ gdx, double* __restrict__ gdy,
                                                              double* __restrict__ wdx, double* __restrict__ wdy) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long s = src[e], t = nbr[e];
  double dx, dy;
  if (e < n_interior_entries) {
    // delta = centers[neighbour] - centers[owner], the owner's entry +delta,
    // the neighbour's entry -delta (solver.py:2004-2013)
    const long long own = (e & 1) ? t : s, nb = (e & 1) ? s : t;
    const double ddx = centers[2 * nb] - centers[2 * own], ddy = centers[2 * nb + 1] - centers[2 * own + 1];
    dx = (e & 1) ? -ddx : ddx;
    dy = (e & 1) ? -ddy : ddy;
  } else {
    // pdelta = (centers[b] - shift) - centers[a] for the pair's a entry, its
    // negation for the b entry (solver.py:2015-2021)
    const long long k = (e - n_interior_entries) >> 1;
    const long long a = (e & 1) ? t : s, b = (e & 1) ? s : t;
    const double pdx = (centers[2 * b] - shift[2 * k]) - centers[2 * a];
    const double pdy = (centers[2 * b + 1] - shift[2 * k + 1]) - centers[2 * a + 1];
    dx = (e & 1) ? -pdx : pdx;
    dy = (e & 1) ? -pdy : pdy;
  }
  const double dist2 = dx * dx + dy * dy;
  const double w = 1.0 / (dist2 > 1e-300 || dist2 != dist2 ? dist2 : 1e-300);  // np.maximum
  gdx[e] = dx;
  gdy[e] = dy;
  wdx[e] = w * dx;
  wdy[e] = w * dy;
}

// Per cell: the moment sums over its entries in entry order and the inverse.
__global__ void __launch_bounds__(kGeomBlock) k_lsq_inverse(long long n_cells, const long long* __restrict__ ptr,
                                                            const long long* __restrict__ order,
                                                            const double* __restrict__ gdx,
                                                            const double* __restrict__ gdy,
                                                            const double* __restrict__ wdx,
                                                            const double* __restrict__ wdy,
                                                            double* __restrict__ inv) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  double mxx = 0.0, mxy = 0.0, myy = 0.0;
  for (long long j = ptr[c]; j < ptr[c + 1]; ++j) {
    const long long e = order[j];
    mxx = mxx + wdx[e] * gdx[e];
    mxy = mxy + wdx[e] * gdy[e];
    myy = myy + wdy[e] * gdy[e];
  }
  const double det = mxx * myy - mxy * mxy;
  const double p = mxx * myy;
  const double floor = (p > 1e-300 || p != p) ? p : 1e-300;
  double ixx = 0.0, ixy = 0.0, iyy = 0.0;
  if (det > 1e-14 * floor) {
    ixx = myy / det;
    ixy = -mxy / det;
    iyy = mxx / det;
  }
  inv[3 * c] = ixx;
  inv[3 * c + 1] = ixy;
  inv[3 * c + 2] = iyy;
}

__global__ void __launch_bounds__(kGeomBlock) k_lsq_coefficients(long long n, const long long* __restrict__ src,
                                                                 const double* __restrict__ inv,
                                                                 const double* __restrict__ wdx,
                                                                 const double* __restrict__ wdy,
                                                                 double* __restrict__ cx, double* __restrict__ cy) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const double* m = inv + 3 * src[e];
  cx[e] = m[0] * wdx[e] + m[1] * wdy[e];
  cy[e] = m[1] * wdx[e] + m[2] * wdy[e];
}

// limiter entry offsets: face centre minus the entry cell's centre
__global__ void __launch_bounds__(kGeomBlock) k_limiter_offsets(long long n, const long long* __restrict__ face,
                                                                const long long* __restrict__ cell,
                                                                const double* __restrict__ fc,
                                                                const double* __restrict__ centers,
                                                                double* __restrict__ ldx, double* __restrict__ ldy) {
  const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  ldx[s] = fc[2 * face[s]] - centers[2 * cell[s]];
  ldy[s] = fc[2 * face[s] + 1] - centers[2 * cell[s] + 1];
}

inline unsigned grid_of(long long n) { return (unsigned)((n + kGeomBlock - 1) / kGeomBlock); }

}  // namespace
}  // namespace mcfd

extern "C" {

int mcfd_device_cell_geometry(int64_t n_cells, const int64_t* cell_offsets, const int64_t* cell_nodes,
                              const double* points, double* centers, double* areas, uint64_t* bad_cell,
                              void* stream) {
  if (n_cells <= 0 || !cell_offsets || !cell_nodes || !points || !centers || !areas || !bad_cell) return MCFD_E_ARG;
  mcfd::count_launch(1);
  mcfd::k_cell_geometry<<<mcfd::grid_of(n_cells), mcfd::kGeomBlock, 0, static_cast<cudaStream_t>(stream)>>>(
      n_cells, reinterpret_cast<const long long*>(cell_offsets), reinterpret_cast<const long long*>(cell_nodes),
      points, centers, areas, reinterpret_cast<unsigned long long*>(bad_cell));
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

int mcfd_device_face_geometry(int64_t n_faces, const int64_t* face_nodes, const double* points,
                              const double* centers, const int64_t* owners, double* face_centers, double* normals,
                              double* lengths, uint64_t* bad_face, void* stream) {
  if (n_faces < 0 || !bad_face ||
      (n_faces && (!face_nodes || !points || !centers || !owners || !face_centers || !normals || !lengths)))
    return MCFD_E_ARG;
  if (!n_faces) return MCFD_OK;
  mcfd::count_launch(1);
  mcfd::k_face_geometry<<<mcfd::grid_of(n_faces), mcfd::kGeomBlock, 0, static_cast<cudaStream_t>(stream)>>>(
      n_faces, reinterpret_cast<const long long*>(face_nodes), points, centers,
      reinterpret_cast<const long long*>(owners), face_centers, normals, lengths,
      reinterpret_cast<unsigned long long*>(bad_face));
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

int mcfd_device_gradient_coefficients(int64_t n_cells, int64_t n_entries, int64_t n_interior_entries,
                                      const int64_t* sources, const int64_t* neighbours, const double* centers,
                                      const double* periodic_shifts, const int64_t* cell_entry_ptr,
                                      const int64_t* cell_entry_order, double* dx, double* dy, double* cx,
                                      double* cy, double* scratch, void* stream) {
  if (n_cells <= 0 || n_entries < 0 || n_interior_entries < 0 || n_interior_entries > n_entries ||
      ((n_entries - n_interior_entries) & 1) || !centers || !cell_entry_ptr || !scratch ||
      (n_entries && (!sources || !neighbours || !cell_entry_order || !dx || !dy || !cx || !cy)) ||
      (n_entries > n_interior_entries && !periodic_shifts))
    return MCFD_E_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* wdx = scratch;
  double* wdy = scratch + n_entries;
  double* inv = scratch + 2 * n_entries;  // [n_cells][3]
  const auto* src = reinterpret_cast<const long long*>(sources);
  mcfd::count_launch(n_entries ? 3 : 1);
  if (n_entries)
    mcfd::k_entry_offsets<<<mcfd::grid_of(n_entries), mcfd::kGeomBlock, 0, s>>>(
        n_entries, n_interior_entries, src, reinterpret_cast<const long long*>(neighbours), centers, periodic_shifts,
        dx, dy, wdx, wdy);
  mcfd::k_lsq_inverse<<<mcfd::grid_of(n_cells), mcfd::kGeomBlock, 0, s>>>(
      n_cells, reinterpret_cast<const long long*>(cell_entry_ptr),
      reinterpret_cast<const long long*>(cell_entry_order), dx, dy, wdx, wdy, inv);
  if (n_entries)
    mcfd::k_lsq_coefficients<<<mcfd::grid_of(n_entries), mcfd::kGeomBlock, 0, s>>>(n_entries, src, inv, wdx, wdy,
                                                                                  cx, cy);
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

int mcfd_device_limiter_offsets(int64_t n_slots, const int64_t* slot_faces, const int64_t* slot_cells,
                                const double* face_centers, const double* centers, double* dx, double* dy,
                                void* stream) {
  if (n_slots < 0 || (n_slots && (!slot_faces || !slot_cells || !face_centers || !centers || !dx || !dy)))
    return MCFD_E_ARG;
  if (!n_slots) return MCFD_OK;
  mcfd::count_launch(1);
  mcfd::k_limiter_offsets<<<mcfd::grid_of(n_slots), mcfd::kGeomBlock, 0, static_cast<cudaStream_t>(stream)>>>(
      n_slots, reinterpret_cast<const long long*>(slot_faces), reinterpret_cast<const long long*>(slot_cells),
      face_centers, centers, dx, dy);
  return cudaGetLastError() == cudaSuccess ? MCFD_OK : MCFD_E_CUDA;
}

}  // extern "C"
