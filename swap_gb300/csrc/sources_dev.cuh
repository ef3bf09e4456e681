// sources_dev.cuh -- the per-draw formulas of the particle sources and sinks,
// shared by the FP64 drop-in (swap_sources.cu) and the FP32 form
// (swap_f32_sources.cu).  FP64 arithmetic in the CPU restatement's operation
// order; the including units are compiled with --fmad=false, so counts equal
// the restatement's.
#pragma once

#include <cmath>

#include "../../include/swap_gpu.h"
#include "philox.h"
#include "swap_dev.cuh"

namespace swapsrc {

using swapk::Geo;

// Ring ion q of Ionize_sw_mp (chem_rates.f:567-608): v = (vsw + vsw cos th,
// vsw sin th, 0), position uniform in (q(1), q(n-1)] per axis.
__device__ __forceinline__ void ionize_state(const Geo& g, const swap_sources& s, long long step, long long q,
                                             double st[6]) {
  const double twopi = 2.0 * 3.14159265358979323846;
  double u[4];
  swapk::source_uniforms(s.seed, swapk::RNG_IONIZE, step, q, 1u, u);
  const double th = u[0] * twopi;
  st[3] = s.vsw + s.vsw * cos(th);
  st[4] = s.vsw * sin(th);
  st[5] = 0.0;
  st[0] = g.qx[1] + (1.0 - u[1]) * (g.qx[g.nx - 1] - g.qx[1]);
  st[1] = g.qy[1] + (1.0 - u[2]) * (g.qy[g.ny - 1] - g.qy[1]);
  st[2] = g.qz[1] + (1.0 - u[3]) * (g.qz[g.nz - 1] - g.qz[1]);
}

// Inflow candidate of slot (ck, cj, p) in the one-cell ghost slab before
// x = q(1): a drifting Maxwellian of the reference's form; returns whether
// its ballistic move over dt enters the box, and its state after the move.
__device__ __forceinline__ bool inflow_candidate(const Geo& g, const swap_sources& s, long long step, long long slot,
                                                 int cj, int ck, double dt, double st[6]) {
  const double pi = 3.14159265358979323846;
  double u[4], v[4], e[4];
  swapk::source_uniforms(s.seed, swapk::RNG_INFLOW, step, slot, 0u, u);
  swapk::source_uniforms(s.seed, swapk::RNG_INFLOW, step, slot, 1u, v);
  swapk::source_uniforms(s.seed, swapk::RNG_INFLOW, step, slot, 2u, e);
  const double vx = s.inflow_ux + s.inflow_vth * sqrt(-log(u[3])) * cos(pi * v[0]);
  const double vy = s.inflow_uy + s.inflow_vth * sqrt(-log(v[1])) * cos(pi * v[2]);
  const double vz = s.inflow_uz + s.inflow_vth * sqrt(-log(v[3])) * cos(pi * e[0]);
  const double x0 = g.qx[1], dxg = g.dxg[1];
  const double xg = x0 - dxg + u[0] * dxg;
  const double xn = xg + dt * vx;
  st[0] = xn;
  st[1] = g.qy[cj + 1] + u[1] * (g.qy[cj + 2] - g.qy[cj + 1]);
  st[2] = g.qz[ck + 1] + u[2] * (g.qz[ck + 2] - g.qz[ck + 1]);
  st[3] = vx; st[4] = vy; st[5] = vz;
  return xn > x0 && !(xn > g.qx[g.nx - 1]);
}

// Whether inflow candidate `slot` enters the box: the draws and operations
// of inflow_candidate that decide it, and nothing else.
__device__ __forceinline__ bool inflow_enters(const Geo& g, const swap_sources& s, long long step, long long slot,
                                              double dt) {
  const double pi = 3.14159265358979323846;
  double u[4], v[4];
  swapk::source_uniforms(s.seed, swapk::RNG_INFLOW, step, slot, 0u, u);
  swapk::source_uniforms(s.seed, swapk::RNG_INFLOW, step, slot, 1u, v);
  const double vx = s.inflow_ux + s.inflow_vth * sqrt(-log(u[3])) * cos(pi * v[0]);
  const double x0 = g.qx[1], dxg = g.dxg[1];
  const double xg = x0 - dxg + u[0] * dxg;
  const double xn = xg + dt * vx;
  return xn > x0 && !(xn > g.qx[g.nx - 1]);
}

// Neutral cloud density n_n(r) = N0/(1+(r/r0)^2).
__device__ __forceinline__ double cloud_density(const swap_sources& s, double x, double y, double z) {
  const double dx = x - s.cloud_x, dy = y - s.cloud_y, dz = z - s.cloud_z;
  const double r2 = (dx * dx + dy * dy + dz * dz) / (s.cloud_r0 * s.cloud_r0);
  return s.cloud_N0 / (1.0 + r2);
}

// New heavy ions of physical cell (ci,cj,ck) (0-based): floor(lambda) plus a
// Bernoulli trial on the remainder, lambda = vol*beta*beta_h*n_n*nu*dt.
__device__ __forceinline__ long long cloud_count(const Geo& g, const swap_sources& s, long long step, double dt,
                                                 double beta, int ci, int cj, int ck, long long cell) {
  const double xc = 0.5 * (g.qx[ci + 1] + g.qx[ci + 2]);
  const double yc = 0.5 * (g.qy[cj + 1] + g.qy[cj + 2]);
  const double zc = 0.5 * (g.qz[ck + 1] + g.qz[ck + 2]);
  const double vol = g.dxg[ci + 1] * g.dyg[cj + 1] * g.dzg[ck + 1];
  const double lam = vol * beta * s.beta_heavy * cloud_density(s, xc, yc, zc) * s.nu_ion * dt;
  long long n = (long long)floor(lam);
  double u[4];
  swapk::source_uniforms(s.seed, swapk::RNG_CLOUD, step, cell, 0u, u);
  if (u[0] < lam - (double)n) ++n;
  return n;
}

// Position of the q-th new ion of a cell, uniform in the cell.
__device__ __forceinline__ void cloud_position(const Geo& g, const swap_sources& s, long long step, int ci, int cj,
                                               int ck, long long cell, long long q, double x[3]) {
  double u[4];
  swapk::source_uniforms(s.seed, swapk::RNG_CLOUD, step, cell, (uint32_t)(1 + q), u);
  x[0] = g.qx[ci + 1] + u[0] * (g.qx[ci + 2] - g.qx[ci + 1]);
  x[1] = g.qy[cj + 1] + u[1] * (g.qy[cj + 2] - g.qy[cj + 1]);
  x[2] = g.qz[ck + 1] + u[2] * (g.qz[ck + 2] - g.qz[ck + 1]);
}

// res_chex's trial for one ion (chem_rates.f:823-840) at draw slot l.
__device__ __forceinline__ bool chex_trial(const swap_sources& s, long long step, long long l, double dt, double x,
                                           double y, double z, double vx, double vy, double vz) {
  const double vrel = sqrt(vx * vx + vy * vy + vz * vz);
  if (!(vrel > 0.0)) return false;
  const double sigma = s.cx_a - s.cx_b * log(vrel);
  if (!(sigma > 0.0)) return false;
  const double prob = dt * cloud_density(s, x, y, z) * sigma * vrel;
  double u[4];
  swapk::source_uniforms(s.seed, swapk::RNG_CHEX, step, l, 0u, u);
  return u[0] < prob;
}

}  // namespace swapsrc
