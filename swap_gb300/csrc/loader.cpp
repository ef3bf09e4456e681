// loader.cpp -- host-side particle loading, the product's replacement for
// load_Maxwellian (part_init.f:146-232).
//
// Differences from the reference, kept on purpose:
//  * stratified: exactly ppc particles in every physical cell, positions
//    uniform inside the cell (the reference draws positions uniformly over the
//    whole box, part_init.f:176-178);
//  * counter-based Philox draws keyed by (seed, stream, particle id) instead of
//    the compiler's random_number seeded by the wall clock (maind.f:156);
//  * the velocity sampler keeps the reference's form
//    v = u + vth*sqrt(-ln U)*cos(pi*U') per component (part_init.f:204-206),
//    i.e. a Gaussian of standard deviation vth/sqrt(2).
// Particles come out cell-sorted: by bricks of 4x4x4 cells (the order of the
// FP32 form) when every axis has a multiple of 4 physical cells, otherwise
// by cell with x fastest.
#include <cmath>
#include <cstdint>

#include "../../include/swap_gpu.h"
#include "philox.h"

extern "C" int swap_load_maxwellian_host(const swap_dims* d, const swap_coords* co, const swap_load_spec* s,
                                         double* xp, double* vp, double* vp1, double* mrat, double* beta_p,
                                         int64_t first, int64_t* count) {
  if (!d || !co || !s || !xp || !vp || !vp1 || !mrat || !beta_p || s->ppc < 0 || first < 0) return SWAP_EINVAL;
  const int64_t ncx = d->nx - 2, ncy = d->ny - 2, ncz = d->nz - 2;
  const int64_t n = ncx * ncy * ncz * (int64_t)s->ppc;
  if (count) *count = n;
  if (first + n > d->ni_max) return SWAP_ECAPACITY;
  const int64_t NM = d->ni_max;
  const double pi = 3.14159265358979323846;
  const bool bricks = ncx % 4 == 0 && ncy % 4 == 0 && ncz % 4 == 0;
  const int64_t nbx = ncx / 4, nby = ncy / 4;
#pragma omp parallel for schedule(static)
  for (int64_t id = 0; id < n; ++id) {
    const int64_t cell = id / s->ppc;
    int ci, cj, ck;
    if (bricks) {
      const int64_t b = cell / 64, l = cell % 64;
      ci = (int)(b % nbx) * 4 + (int)(l & 3);
      cj = (int)((b / nbx) % nby) * 4 + (int)((l >> 2) & 3);
      ck = (int)(b / (nbx * nby)) * 4 + (int)(l >> 4);
    } else {
      ci = (int)(cell % ncx);
      cj = (int)((cell / ncx) % ncy);
      ck = (int)(cell / (ncx * ncy));
    }
    double u[12];
    swapk::particle_uniforms(s->seed, s->stream, (uint64_t)id, 0u, u);
    // cell (i,j,k) spans nodes i..i+1 (1-based), i = ci+1; coords are 0-based
    const double x0 = co->qx[ci], x1 = co->qx[ci + 1];
    const double y0 = co->qy[cj], y1 = co->qy[cj + 1];
    const double z0 = co->qz[ck], z1 = co->qz[ck + 1];
    const int64_t l = first + id;
    xp[l] = x0 + u[0] * (x1 - x0);
    xp[l + NM] = y0 + u[1] * (y1 - y0);
    xp[l + 2 * NM] = z0 + u[2] * (z1 - z0);
    const double vx = s->ux + s->vth * std::sqrt(-std::log(u[3])) * std::cos(pi * u[4]);
    const double vy = s->uy + s->vth * std::sqrt(-std::log(u[5])) * std::cos(pi * u[6]);
    const double vz = s->uz + s->vth * std::sqrt(-std::log(u[7])) * std::cos(pi * u[8]);
    vp[l] = vx; vp[l + NM] = vy; vp[l + 2 * NM] = vz;
    vp1[l] = vx; vp1[l + NM] = vy; vp1[l + 2 * NM] = vz;  // part_init.f:220
    mrat[l] = s->mrat;
    beta_p[l] = s->beta_p;
  }
  return SWAP_OK;
}
