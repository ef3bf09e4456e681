// swap_dev.cuh -- device-side views and helpers shared by the sm_103a kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace swapk {

// Error codes written by kernels into the context's device flag (first
// writer wins); the host maps them to SWAP_E* status codes.
enum : int { KERR_NONE = 0, KERR_DOMAIN = 3, KERR_CAPACITY = 4, KERR_MOVE = 7, KERR_WAIT = 8, KERR_RANGE = 10 };

// Grid geometry on the device.  Node arrays are 1-based (element 0 unused)
// so kernel code reads like the reference: qx[i] is qx(i).
struct Geo {
  int nx, ny, nz;
  long long C;  // nodes incl. ghosts
  const double *qx, *qy, *qz;
  const double *dxg, *dyg, *dzg;  // dx_grid ...
  const double *dxc, *dyc, *dzc;  // dx_cell ...
  const double *xr, *yr, *zr;     // xrat ...
  double dy;                      // module dy (gutsp.f:1404)
  double inv_dx, inv_dz;          // guesses for the cell search only
};

__host__ __device__ __forceinline__ long long nidx(const Geo& g, int i, int j, int k) {
  return (long long)(i - 1) + (long long)g.nx * ((long long)(j - 1) + (long long)g.ny * (long long)(k - 1));
}

// Periodic image of a node index (boundary.f:21-22): 1 -> n-1, n -> 2.
__host__ __device__ __forceinline__ int wrapn(int i, int n) { return i == 1 ? n - 1 : (i == n ? 2 : i); }

// Interior thread t -> (i,j,k) in [2, n-1]^3, i fastest.
__device__ __forceinline__ void interior_ijk(const Geo& g, long long t, int& i, int& j, int& k) {
  const long long ix = g.nx - 2, iy = g.ny - 2;
  i = (int)(t % ix) + 2;
  const long long r = t / ix;
  j = (int)(r % iy) + 2;
  k = (int)(r / iy) + 2;
}

__host__ __device__ __forceinline__ long long n_interior(const Geo& g) {
  return (long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
}

// Ghost-shell enumeration: x faces (all j,k), then y faces (interior i, all
// k), then z faces (interior i,j).  Total = n_ghost(g).
__host__ __device__ __forceinline__ long long n_ghost(const Geo& g) {
  return 2LL * g.ny * g.nz + 2LL * (g.nx - 2) * g.nz + 2LL * (g.nx - 2) * (g.ny - 2);
}

__device__ __forceinline__ void ghost_ijk(const Geo& g, long long t, int& i, int& j, int& k) {
  const long long A = 2LL * g.ny * g.nz;
  const long long B = 2LL * (g.nx - 2) * g.nz;
  if (t < A) {
    const long long face = t / ((long long)g.ny * g.nz), r = t % ((long long)g.ny * g.nz);
    i = face == 0 ? 1 : g.nx;
    j = (int)(r % g.ny) + 1;
    k = (int)(r / g.ny) + 1;
  } else if (t < A + B) {
    t -= A;
    const long long per = (long long)(g.nx - 2) * g.nz;
    const long long face = t / per, r = t % per;
    j = face == 0 ? 1 : g.ny;
    i = (int)(r % (g.nx - 2)) + 2;
    k = (int)(r / (g.nx - 2)) + 1;
  } else {
    t -= A + B;
    const long long per = (long long)(g.nx - 2) * (g.ny - 2);
    const long long face = t / per, r = t % per;
    k = face == 0 ? 1 : g.nz;
    i = (int)(r % (g.nx - 2)) + 2;
    j = (int)(r / (g.nx - 2)) + 2;
  }
}

__device__ __forceinline__ void set_err(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// Cell search of get_interp_weights (gutsp.f:1396-1401): the index i with
// q(i) < x <= q(i+1), i.e. one less than the first node with x <= q(node).
// A guess from the uniform spacing is corrected against the node array
// itself, so the result equals the reference's linear search for any
// monotone q.  Returns 0 (invalid) when x <= q(1) or x > q(n).
__device__ __forceinline__ int cell_search(const double* __restrict__ q, int n, double x, double inv_d) {
  if (!(x > q[1]) || x > q[n]) return 0;
  int i = (int)((x - q[1]) * inv_d) + 1;
  i = i < 1 ? 1 : (i > n - 1 ? n - 1 : i);
  while (i > 1 && !(x > q[i])) --i;
  while (i < n - 1 && x > q[i + 1]) ++i;
  return i;
}

// The eight interpolation weights of a particle at (x,y,z) in cell (i,j,k),
// in the reference's order (000,100,001,101,010,110,011,111 over x,z,y;
// gutsp.f:1414-1429).  Units compiled with --fmad=false round every product
// like the Fortran.
__device__ __forceinline__ void weights8(const Geo& g, int i, int j, int k, double x, double y, double z,
                                         double w[8]) {
  const double vol = 1.0 / ((g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]));
  const double x1 = fabs(x - g.qx[i]), x2 = fabs(x - g.qx[i + 1]);
  const double y1 = fabs(y - g.qy[j]), y2 = fabs(y - g.qy[j + 1]);
  const double z1 = fabs(z - g.qz[k]), z2 = fabs(z - g.qz[k + 1]);
  w[0] = x2 * y2 * z2 * vol;
  w[1] = x1 * y2 * z2 * vol;
  w[2] = x2 * y2 * z1 * vol;
  w[3] = x1 * y2 * z1 * vol;
  w[4] = x2 * y1 * z2 * vol;
  w[5] = x1 * y1 * z2 * vol;
  w[6] = x2 * y1 * z1 * vol;
  w[7] = x1 * y1 * z1 * vol;
}

// Deposit target of a raw corner after the periodic fold (gutsp.f:1496-1498,
// 1803-1805) and the ghost overwrite of periodic_scalar/periodic: plane 1 goes
// to plane n-1, plane n is discarded.  Returns -1 for a discarded corner.
__device__ __forceinline__ long long fold_target(const Geo& g, int i, int j, int k) {
  if (i == g.nx || j == g.ny || k == g.nz) return -1;
  return nidx(g, i == 1 ? g.nx - 1 : i, j == 1 ? g.ny - 1 : j, k == 1 ? g.nz - 1 : k);
}

// The folded targets of the eight corners, in the weights' order.
__device__ __forceinline__ void corner_targets(const Geo& g, int i, int j, int k, long long tg[8]) {
  tg[0] = fold_target(g, i, j, k);
  tg[1] = fold_target(g, i + 1, j, k);
  tg[2] = fold_target(g, i, j, k + 1);
  tg[3] = fold_target(g, i + 1, j, k + 1);
  tg[4] = fold_target(g, i, j + 1, k);
  tg[5] = fold_target(g, i + 1, j + 1, k);
  tg[6] = fold_target(g, i, j + 1, k + 1);
  tg[7] = fold_target(g, i + 1, j + 1, k + 1);
}

}  // namespace swapk
