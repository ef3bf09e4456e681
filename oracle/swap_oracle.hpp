// swap_oracle.hpp -- CPU restatement of SWAP's hybrid PIC ion step.
//
// TEST INFRASTRUCTURE ONLY.  This header is the parity oracle: it restates,
// subroutine by subroutine, the Fortran reference (pdelamere/SWAP) so that the
// CUDA path can be checked against it.  Only tests/, __graft_entry__.smoke()
// and the CPU-baseline leg of bench.py may load it.  The product path never
// links or calls anything in oracle/.
//
// Conventions (chosen to read like the reference):
//  * indices are 1-based, grids are column-major (nx,ny,nz[,3]) with x fastest
//    and the vector component slowest; particle arrays are (ni_max,3);
//  * arithmetic follows the Fortran source left to right; the library is
//    compiled with -ffp-contract=off so no multiply-add is fused;
//  * templated on the real type R: float = the reference's own precision
//    (makefile:1, -real-size 32), double = the FP64 oracle.
//
// Parity status: the reference has no Fortran compiler here, so nothing can be
// compared against a reference run.  The only reference golden vector (b0.dat,
// written by initial.f:136-139) pins grd7/grd6_setup/initparameters at FP32;
// everything else is pinned by the known-answer tests in tests/ (exact Boris
// rotation, uniform-load density, div(curl E) = 0, periodic-wrap invariants,
// stationary uniform plasma, Courant rule).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <vector>

#include "../swap_gb300/csrc/philox.h"

#ifdef _OPENMP
#include <omp.h>
#endif

// Loops over nodes or particles in which every iteration writes only its own
// outputs run on `nt` host threads when the CPU baseline is timed; their
// results do not depend on the thread count.  Parity runs use one thread.
#define SWO_PRAGMA(x) _Pragma(#x)
#define SWO_OMP_FOR(nt) SWO_PRAGMA(omp parallel for schedule(static) num_threads(nt) if ((nt) > 1))

namespace swo {

// ---------------------------------------------------------------------------
// Mesh: the /coords/ COMMON block (global.f:27-38) for a run-time grid size.
// Node arrays are stored 1-based (element 0 unused) to keep the restated loops
// literal.
// ---------------------------------------------------------------------------
template <class R>
struct Mesh {
  int nx = 0, ny = 0, nz = 0;
  int nt = 1;         // host threads of the node and particle loops (see SWO_OMP_FOR)
  std::size_t C = 0;  // nodes, ghosts included
  R dx = 0, dy = 0, delz = 0;
  std::vector<R> qx, qy, qz;
  std::vector<R> dx_grid, dy_grid, dz_grid;
  std::vector<R> dx_cell, dy_cell, dz_cell;
  std::vector<R> xrat, yrat, zrat;

  std::size_t n(int i, int j, int k) const {
    return (std::size_t)(i - 1) +
           (std::size_t)nx * ((std::size_t)(j - 1) + (std::size_t)ny * (std::size_t)(k - 1));
  }
};

// grd7 (initial.f:147-301): node coordinates, grid/cell spacings and the
// interpolation ratios.  Stretch factors xsf/zsf are 0 in the reference
// (initial.f:173,209); they are kept as arguments.  The reference's stretch
// loops index below 1 / above nx for small grids (nx < 2*nrgrd); they are
// clamped to the array here, which changes nothing when xsf = zsf = 0.
template <class R>
void grd7(Mesh<R>& g, int nx, int ny, int nz, R dx, R dy, R delz, R xsf = 0, R zsf = 0) {
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.C = (std::size_t)nx * ny * nz;
  g.dx = dx; g.dy = dy; g.delz = delz;
  auto alloc = [](std::vector<R>& v, int n) { v.assign((std::size_t)n + 1, R(0)); };
  alloc(g.qx, nx); alloc(g.qy, ny); alloc(g.qz, nz);
  alloc(g.dx_grid, nx); alloc(g.dy_grid, ny); alloc(g.dz_grid, nz);
  alloc(g.dx_cell, nx); alloc(g.dy_cell, ny); alloc(g.dz_cell, nz);
  alloc(g.xrat, nx); alloc(g.yrat, ny); alloc(g.zrat, nz);
  const int nrgrd = 20;
  const int rk = nz / 2, ri = nx / 2;  // integer division (global.f:30)

  for (int j = 1; j <= ny; ++j) {  // initial.f:159-162
    g.qy[j] = R(j) * dy;
    g.dy_grid[j] = dy;
  }
  auto stretch = [&](std::vector<R>& d, int n, int rc, R base, R sf) {
    // initial.f:175-191 (x) and 211-231 (z)
    for (int i = rc; i <= rc + nrgrd; ++i)
      if (i >= 1 && i <= n) d[i] = base;
    for (int i = rc + nrgrd + 1; i <= n; ++i)
      if (i >= 1) d[i] = base + sf * base * R(i - (rc + nrgrd + 1)) / R(n - (rc + nrgrd + 1));
    for (int i = rc - nrgrd; i <= rc - 1; ++i)
      if (i >= 1 && i <= n) d[i] = base;
    for (int i = 1; i <= rc - nrgrd - 1; ++i) {
      int ind = rc - nrgrd - i;
      if (ind >= 1 && ind <= n)
        d[ind] = base + sf * base * R(rc - nrgrd - 1 - ind) / R(rc - nrgrd - 1);
    }
    for (int i = 1; i <= n; ++i)  // entries never touched by the loops above
      if (d[i] == R(0)) d[i] = base;
  };
  stretch(g.dx_grid, nx, ri, dx, xsf);
  g.qx[1] = dx;  // initial.f:193-201
  for (int i = 2; i <= nx; ++i) g.qx[i] = g.qx[i - 1] + g.dx_grid[i];
  for (int i = 1; i <= nx - 1; ++i) g.dx_grid[i] = g.qx[i + 1] - g.qx[i];
  g.dx_grid[nx] = g.dx_grid[nx - 1];

  stretch(g.dz_grid, nz, rk, delz, zsf);
  g.qz[1] = delz;  // initial.f:233-242
  for (int k = 2; k <= nz; ++k) g.qz[k] = g.qz[k - 1] + g.dz_grid[k];
  for (int k = 1; k <= nz - 1; ++k) g.dz_grid[k] = g.qz[k + 1] - g.qz[k];
  g.dz_grid[nz] = g.dz_grid[nz - 1];

  auto cells = [](const std::vector<R>& q, const std::vector<R>& dgrid, std::vector<R>& dcell,
                  std::vector<R>& rat, int n) {  // initial.f:246-282
    dcell[1] = dgrid[1];
    dcell[n] = dgrid[n];
    rat[1] = R(0.5);
    rat[n] = R(0.5);
    for (int i = 2; i <= n - 1; ++i) {
      dcell[i] = ((q[i + 1] + q[i]) / R(2.0)) - ((q[i] + q[i - 1]) / R(2.0));
      R plus = (q[i + 1] + q[i]) / R(2.0);
      R minus = (q[i] + q[i - 1]) / R(2.0);
      rat[i] = (q[i] - minus) / (plus - minus);
    }
  };
  cells(g.qz, g.dz_grid, g.dz_cell, g.zrat, nz);
  cells(g.qx, g.dx_grid, g.dx_cell, g.xrat, nx);
  cells(g.qy, g.dy_grid, g.dy_cell, g.yrat, ny);
}

// Scalars of the `inputs` module derived by initparameters (inputs.f:125-172)
// for the quantities the B0 golden vector depends on.  Physical constants are
// the reference's PARAMETERs (inputs.f:19,50-57).
template <class R>
struct PhysInputs {
  R b0_init, nf_init, dt_frac, dx_frac, nu_init_frac;
  int ion_amu;
};

template <class R>
struct PhysDerived {
  R mion, omega_p, lambda_i, dx, dy, delz, dt, dtsub_init, nu_init, alpha;
};

template <class R>
PhysDerived<R> initparameters(const PhysInputs<R>& in, int ntsub) {
  const R q = R(1.6e-19);
  const R pi = R(3.14159);
  const R mu0 = pi * R(4.0e-7);
  PhysDerived<R> d;
  d.mion = R(in.ion_amu) * R(1.67e-27);                                    // inputs.f:128
  d.omega_p = q * in.b0_init / d.mion;                                      // inputs.f:130
  d.lambda_i = (R(3e8) / std::sqrt((in.nf_init / R(1e9)) * q * q / (R(8.85e-12) * d.mion))) / R(1e3);  // :132-133
  d.dx = d.lambda_i * in.dx_frac;                                           // inputs.f:135-137
  d.dy = d.lambda_i * in.dx_frac;
  d.delz = d.lambda_i * in.dx_frac;
  d.dt = in.dt_frac * d.mion / (q * in.b0_init);                            // inputs.f:141
  d.dtsub_init = d.dt / R(ntsub);                                          // inputs.f:142
  d.nu_init = in.nu_init_frac * d.omega_p;                                  // inputs.f:168
  d.alpha = (mu0 / R(1e3)) * q * (q / d.mion);                              // inputs.f:170
  return d;
}

// grd6_setup (initial.f:10-142): b0 = (0,0,b0_init*q/mO) everywhere and the
// time levels bt, b12, b1, b1p2 start equal to b0; nu = nu_init.
template <class R>
void grd6_setup(const Mesh<R>& g, R b0_init, R mion, R nu_init, R* b0, R* bt, R* b12, R* b1, R* b1p2,
                R* nu) {
  const R q = R(1.6e-19);
  const R eoverm = q / mion;  // initial.f:36
  const std::size_t C = g.C;
  for (std::size_t n = 0; n < C; ++n) {
    b0[n] = R(0.0);
    b0[n + C] = R(0.0);
    b0[n + 2 * C] = b0_init * eoverm;  // initial.f:61-63
  }
  for (std::size_t n = 0; n < C; ++n) {
    nu[n] = nu_init;  // initial.f:79
    for (int m = 0; m < 3; ++m) {
      const std::size_t o = n + C * m;
      bt[o] = b0[o]; b12[o] = b0[o]; b1[o] = b0[o]; b1p2[o] = b0[o];  // initial.f:82-85
    }
  }
}

// ---------------------------------------------------------------------------
// The implicit state of the Fortran path: module `inputs`/`global` scalars,
// /ion_info/ (ijkp), /weights/ (wght), /dummy/ (a, c, ct), /timestep/.
// ---------------------------------------------------------------------------
template <class R>
struct State {
  Mesh<R> g;
  std::int64_t ni_max = 0;
  R dt = 0, dtsub_init = 0, alpha = 0, beta = 0;
  int ntsub = 10;
  R dtsub = 0, ntf = 0;              // /timestep/ (global.f:76-77); ntf is real there
  R grad_pe = 0;                     // isothermal T_e/m (0 = reference: no pressure term)
  std::vector<std::int32_t> ijkp;    // (ni_max,3)
  std::vector<R> wght;               // (ni_max,8)
  std::vector<R> a, c, ct;           // /dummy/ scratch (global.f:70-71)
  // locals of the subroutines that the reference allocates per call
  std::vector<R> ajc, upc, aa, btcl, curl_E, btp1, btp1mf, btc2, v_tmp;
  int nthreads = 1;                  // >1 only for the CPU baseline timing leg
  std::vector<std::vector<R>> priv;  // per-thread deposit grids, kept between calls

  std::size_t C() const { return g.C; }
};

template <class R>
void state_alloc(State<R>& s, std::int64_t ni_max) {
  s.ni_max = ni_max;
  const std::size_t C3 = 3 * s.g.C;
  s.ijkp.assign((std::size_t)ni_max * 3, 0);
  s.wght.assign((std::size_t)ni_max * 8, R(0));
  for (auto* v : {&s.a, &s.c, &s.ct, &s.ajc, &s.upc, &s.aa, &s.btcl, &s.curl_E, &s.btp1, &s.btp1mf,
                  &s.btc2})
    v->assign(C3, R(0));
  s.v_tmp.assign((std::size_t)ni_max * 3, R(0));
}

// ---------------------------------------------------------------------------
// Boundary fill (boundary.f)
// ---------------------------------------------------------------------------

// periodic (boundary.f:9-52): ghost planes 1 and n copy nodes n-1 and 2, x
// then y then z, for each of the three components in turn -- the scalar fill
// below applied to each component.
template <class R>
void periodic_scalar(const Mesh<R>& g, R* f);

template <class R>
void periodic(const Mesh<R>& g, R* b) {
  for (int m = 0; m < 3; ++m) periodic_scalar(g, b + g.C * m);
}

// periodic_scalar (boundary.f:167-206)
template <class R>
void periodic_scalar(const Mesh<R>& g, R* f) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  SWO_OMP_FOR(g.nt)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      f[g.n(1, j, k)] = f[g.n(nx - 1, j, k)];
      f[g.n(nx, j, k)] = f[g.n(2, j, k)];
    }
  SWO_OMP_FOR(g.nt)
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      f[g.n(i, 1, k)] = f[g.n(i, ny - 1, k)];
      f[g.n(i, ny, k)] = f[g.n(i, 2, k)];
    }
  SWO_OMP_FOR(g.nt)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      f[g.n(i, j, 1)] = f[g.n(i, j, nz - 1)];
      f[g.n(i, j, nz)] = f[g.n(i, j, 2)];
    }
}

// ---------------------------------------------------------------------------
// Staggered-grid interpolation (grid_interp.f)
// ---------------------------------------------------------------------------

// face_to_center (grid_interp.f:136-176).  Note the reference calls
// periodic(v) first, i.e. it overwrites the ghosts of its INPUT.
template <class R>
void face_to_center(const Mesh<R>& g, R* v, R* vc) {
  periodic(g, v);
  const std::size_t C = g.C;
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz; ++k)
    for (int j = 2; j <= g.ny; ++j)
      for (int i = 2; i <= g.nx; ++i) {
        const std::size_t o = g.n(i, j, k);
        vc[o] = g.xrat[i] * (v[o] - v[g.n(i - 1, j, k)]) + v[g.n(i - 1, j, k)];
        vc[o + C] = g.yrat[j] * (v[o + C] - v[g.n(i, j - 1, k) + C]) + v[g.n(i, j - 1, k) + C];
        vc[o + 2 * C] =
            g.zrat[k] * (v[o + 2 * C] - v[g.n(i, j, k - 1) + 2 * C]) + v[g.n(i, j, k - 1) + 2 * C];
      }
  periodic(g, vc);
}

// The cell-centre stencil shared by edge_to_center (grid_interp.f:22-57) and
// edge_to_face (grid_interp.f:80-115).
template <class R>
inline void edge_center_at(const Mesh<R>& g, const R* bt, int i, int j, int k, R* btc) {
  const std::size_t C = g.C;
  const int im = i - 1, jm = j - 1, km = k - 1;
  const std::size_t o = g.n(i, j, k);
  R b1, b2;
  b2 = bt[g.n(i, jm, k)] + g.yrat[j] * (bt[g.n(i, j, k)] - bt[g.n(i, jm, k)]);
  b1 = bt[g.n(i, jm, km)] + g.yrat[j] * (bt[g.n(i, j, km)] - bt[g.n(i, jm, km)]);
  btc[o] = b1 + g.zrat[k] * (b2 - b1);
  b2 = bt[g.n(im, j, k) + C] + g.xrat[i] * (bt[g.n(i, j, k) + C] - bt[g.n(im, j, k) + C]);
  b1 = bt[g.n(im, j, km) + C] + g.xrat[i] * (bt[g.n(i, j, km) + C] - bt[g.n(im, j, km) + C]);
  btc[o + C] = b1 + g.zrat[k] * (b2 - b1);
  b2 = bt[g.n(i, jm, k) + 2 * C] + g.yrat[j] * (bt[g.n(i, j, k) + 2 * C] - bt[g.n(i, jm, k) + 2 * C]);
  b1 = bt[g.n(im, jm, k) + 2 * C] +
       g.yrat[j] * (bt[g.n(im, j, k) + 2 * C] - bt[g.n(im, jm, k) + 2 * C]);
  btc[o + 2 * C] = b1 + g.xrat[i] * (b2 - b1);
}

// edge_to_center (grid_interp.f:10-62); periodic(bt) first, then interior,
// then periodic(btc).
template <class R>
void edge_to_center(const Mesh<R>& g, R* bt, R* btc) {
  periodic(g, bt);
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) edge_center_at(g, bt, i, j, k, btc);
  periodic(g, btc);
}

// edge_to_face (grid_interp.f:67-130).  The reference's final loop runs to
// i = nx (j = ny, k = nz) and reads btc(nx+1,...) past the array there; those
// outputs are ghost nodes, which every consumer (face_to_center) overwrites
// with periodic() before reading.  Only the interior is formed here.
template <class R>
void edge_to_face(const Mesh<R>& g, R* bt, R* btmf, R* btc_local) {
  periodic(g, bt);
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz; ++k)
    for (int j = 2; j <= g.ny; ++j)
      for (int i = 2; i <= g.nx; ++i) edge_center_at(g, bt, i, j, k, btc_local);
  periodic(g, btc_local);
  const std::size_t C = g.C;
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        btmf[o] = R(0.5) * (btc_local[o] + btc_local[g.n(i + 1, j, k)]);
        btmf[o + C] = R(0.5) * (btc_local[o + C] + btc_local[g.n(i, j + 1, k) + C]);
        btmf[o + 2 * C] = R(0.5) * (btc_local[o + 2 * C] + btc_local[g.n(i, j, k + 1) + 2 * C]);
      }
}

// ---------------------------------------------------------------------------
// Field solver (gutsf.f)
// ---------------------------------------------------------------------------

// crossf2 (gutsf.f:40-104): cross product at the cell centre into ct, then
// averaged back to the contravariant (face) positions.
template <class R>
void crossf2(State<R>& s, R* aa, R* btc, R* cc) {
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  R* ct = s.ct.data();
  periodic(g, aa);
  periodic(g, btc);
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        const R ax = aa[o], bx = btc[o], ay = aa[o + C], by = btc[o + C], az = aa[o + 2 * C],
                bz = btc[o + 2 * C];
        ct[o] = ay * bz - az * by;
        ct[o + C] = az * bx - ax * bz;
        ct[o + 2 * C] = ax * by - ay * bx;
      }
  periodic(g, ct);
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        cc[o] = R(0.5) * (ct[o] + ct[g.n(i + 1, j, k)]);
        cc[o + C] = R(0.5) * (ct[o + C] + ct[g.n(i, j + 1, k) + C]);
        cc[o + 2 * C] = R(0.5) * (ct[o + 2 * C] + ct[g.n(i, j, k + 1) + 2 * C]);
      }
  periodic(g, cc);
}

// curlB (gutsf.f:178-244): aj = curl(B)/(ntot*alpha) with backward
// differences over dx_cell etc.; periodic(b1) first.  aj ghosts are left as
// they were (the reference never sets them here).
template <class R>
void curlB(State<R>& s, R* b1, const R* np, R* aj) {
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  periodic(g, b1);
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        R ntot[3], cb[3];
        ntot[0] = R(0.5) * (np[o] + np[g.n(i + 1, j, k)]);
        ntot[1] = R(0.5) * (np[o] + np[g.n(i, j + 1, k)]);
        ntot[2] = R(0.5) * (np[o] + np[g.n(i, j, k + 1)]);
        cb[0] = (b1[o + 2 * C] - b1[g.n(i, j - 1, k) + 2 * C]) / g.dy_cell[j] +
                (b1[g.n(i, j, k - 1) + C] - b1[o + C]) / g.dz_cell[k];
        cb[1] = (b1[o] - b1[g.n(i, j, k - 1)]) / g.dz_cell[k] +
                (b1[g.n(i - 1, j, k) + 2 * C] - b1[o + 2 * C]) / g.dx_cell[i];
        cb[2] = (b1[o + C] - b1[g.n(i - 1, j, k) + C]) / g.dx_cell[i] +
                (b1[g.n(i, j - 1, k)] - b1[o]) / g.dy_cell[j];
        for (int m = 0; m < 3; ++m) aj[o + C * m] = cb[m] / (ntot[m] * s.alpha);
      }
}

// curlE (gutsf.f:249-308): forward differences over dx_grid etc.
template <class R>
void curlE(const Mesh<R>& g, const R* E, R* curl_E) {
  const std::size_t C = g.C;
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        curl_E[o] = (E[g.n(i, j + 1, k) + 2 * C] - E[o + 2 * C]) / g.dy_grid[j] +
                    (E[o + C] - E[g.n(i, j, k + 1) + C]) / g.dz_grid[k];
        curl_E[o + C] = (E[o + 2 * C] - E[g.n(i + 1, j, k) + 2 * C]) / g.dx_grid[i] +
                        (E[g.n(i, j, k + 1)] - E[o]) / g.dz_grid[k];
        curl_E[o + 2 * C] = (E[o] - E[g.n(i, j + 1, k)]) / g.dy_grid[j] +
                            (E[g.n(i + 1, j, k) + C] - E[o + C]) / g.dx_grid[i];
      }
}

// Isothermal electron-pressure term (an extension, off by default: the
// reference keeps it only as a commented "- gradP", gutsf.f:1083,1283).
// gradP_m at the face of component m: T_e/m * (n(node+e_m)-n(node)) /
// (dg_m * n_face), with n_face the face average of np as in curlB.
template <class R>
inline R grad_pe_at(const State<R>& s, const R* np, int i, int j, int k, int m) {
  const Mesh<R>& g = s.g;
  const std::size_t o = g.n(i, j, k);
  std::size_t op;
  R dg;
  if (m == 0) { op = g.n(i + 1, j, k); dg = g.dx_grid[i]; }
  else if (m == 1) { op = g.n(i, j + 1, k); dg = g.dy_grid[j]; }
  else { op = g.n(i, j, k + 1); dg = g.dz_grid[k]; }
  const R nf = R(0.5) * (np[o] + np[op]);
  return s.grad_pe * ((np[op] - np[o]) / dg) / nf;
}

// get_E (gutsf.f:994-1110): E = crossf2(face_to_center(aj-up),
// edge_to_center(bt)) + nu*aj, then periodic(E).
template <class R>
void get_E(State<R>& s, R* E, R* bt, R* aj, const R* up, const R* np, const R* nu) {
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  R* a = s.a.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k) + C * m;
          a[o] = aj[o] - up[o];  // gutsf.f:1059
        }
  face_to_center(g, a, s.aa.data());      // gutsf.f:1073
  edge_to_center(g, bt, s.btcl.data());   // gutsf.f:1074
  crossf2(s, s.aa.data(), s.btcl.data(), s.c.data());  // gutsf.f:1075
  const R* c = s.c.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k);
          E[o + C * m] = c[o + C * m] + nu[o] * aj[o + C * m];  // gutsf.f:1082
          if (s.grad_pe != R(0)) E[o + C * m] = E[o + C * m] - grad_pe_at(s, np, i, j, k, m);
        }
  periodic(g, E);
}

// predict_B (gutsf.f:1115-1169): b1p2 = b12 - 2*dtsub*curl(E(bt)).
template <class R>
void predict_B(State<R>& s, R* b0, R* b1, R* b12, R* b1p2, R* bt, R* E, R* aj, R* up, R* np, R* nu) {
  (void)b0; (void)b1;
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  get_E(s, E, bt, aj, up, np, nu);
  curlE(g, E, s.curl_E.data());
  const R* ce = s.curl_E.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k) + C * m;
          b1p2[o] = b12[o] - R(2.0) * s.dtsub * ce[o];  // gutsf.f:1158-1159
        }
  periodic(g, b1p2);
}

// get_Ep1 (gutsf.f:1174-1304): E at m+1/2 from btp1 = (b1p2+b1)/2, with aj
// recomputed from btp1 and B brought to the centre via edge_to_face then
// face_to_center.
template <class R>
void get_Ep1(State<R>& s, R* E, R* b1, R* b1p2, R* aj, const R* up, const R* np, const R* nu) {
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  R* btp1 = s.btp1.data();
  SWO_OMP_FOR(g.nt)
  for (std::size_t o = 0; o < 3 * C; ++o) btp1[o] = R(0.5) * (b1p2[o] + b1[o]);  // :1210-1219
  curlB(s, btp1, np, aj);  // gutsf.f:1221
  R* a = s.a.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k) + C * m;
          a[o] = aj[o] - up[o];  // gutsf.f:1261
        }
  face_to_center(g, a, s.aa.data());                     // :1267
  edge_to_face(g, btp1, s.btp1mf.data(), s.btc2.data());  // :1268
  face_to_center(g, s.btp1mf.data(), s.btcl.data());     // :1269
  crossf2(s, s.aa.data(), s.btcl.data(), s.c.data());    // :1276
  const R* c = s.c.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k);
          E[o + C * m] = c[o + C * m] + nu[o] * aj[o + C * m];  // :1282
          if (s.grad_pe != R(0)) E[o + C * m] = E[o + C * m] - grad_pe_at(s, np, i, j, k, m);
        }
  periodic(g, E);
}

// correct_B (gutsf.f:1309-1359): b1p2 = b1 - dtsub*curl(E(m+1/2)).
template <class R>
void correct_B(State<R>& s, R* b0, R* b1, R* b1p2, R* E, R* aj, R* up, R* np, R* nu) {
  (void)b0;
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  get_Ep1(s, E, b1, b1p2, aj, up, np, nu);
  curlE(g, E, s.curl_E.data());
  const R* ce = s.curl_E.data();
  SWO_OMP_FOR(g.nt)
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i)
        for (int m = 0; m < 3; ++m) {
          const std::size_t o = g.n(i, j, k) + C * m;
          b1p2[o] = b1[o] - s.dtsub * ce[o];  // gutsf.f:1349-1350
        }
  periodic(g, b1p2);
}

// f_update_tlev (gutsf.f:10-35): bt <- b1p2, b12 <- b1, b1 <- b1p2.
template <class R>
void f_update_tlev(const Mesh<R>& g, R* b1, R* b12, R* b1p2, R* bt) {
  SWO_OMP_FOR(g.nt)
  for (std::size_t o = 0; o < 3 * g.C; ++o) {
    bt[o] = b1p2[o];
    b12[o] = b1[o];
    b1[o] = b1p2[o];
  }
}

// check_time_step (gutsf.f:1776-1822): whistler Courant test at every node
// (ghosts included); every violating node halves dtsub and doubles ntf, in
// loop order i, j, k (k innermost).  Returns the number of halvings.
template <class R>
int check_time_step(State<R>& s, const R* bt, const R* np, R dx) {
  const Mesh<R>& g = s.g;
  const std::size_t C = g.C;
  int halvings = 0;
  for (int i = 1; i <= g.nx; ++i)
    for (int j = 1; j <= g.ny; ++j)
      for (int k = 1; k <= g.nz; ++k) {
        const std::size_t o = g.n(i, j, k);
        const R ak = R(2.) / dx;
        const R btot = std::sqrt(bt[o] * bt[o] + bt[o + C] * bt[o + C] + bt[o + 2 * C] * bt[o + 2 * C]);
        const R a1 = ak * ak * btot / (s.alpha * (np[o]));
        const R a2 = (ak * btot) * (ak * btot) / (s.alpha * (np[o]));
        const R womega = R(0.5) * (a1 + std::sqrt(a1 * a1 + R(4) * a2));
        const R phi = womega / ak;
        const R deltat = dx / phi;
        if (deltat <= R(2.0) * s.dtsub) {
          s.dtsub = s.dtsub / R(2.0);
          s.ntf = s.ntf * R(2.0);
          ++halvings;
        }
      }
  return halvings;
}

// ---------------------------------------------------------------------------
// Particle kernels (gutsp.f)
// ---------------------------------------------------------------------------

// Cell search of get_interp_weights (gutsp.f:1396-1412): i is one less than
// the first node with x <= qx(i) (strict '>' in the loop test); j uses floor.
template <class R>
inline int search_node(const std::vector<R>& q, int n, R x) {
  int i = 0;
  do {
    ++i;
    if (i > n) return n + 1;  // past the array: the reference would read beyond it
  } while (x > q[i]);
  return i - 1;
}

// get_interp_weights (gutsp.f:1378-1435)
template <class R>
void get_interp_weights(State<R>& s, const R* xp, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(s.nthreads) if (s.nthreads > 1) reduction(| : bad)
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    const R x = xp[l], y = xp[l + NM], z = xp[l + 2 * NM];
    const int i = search_node(g.qx, g.nx, x);
    const int j = (int)std::floor(y / g.dy);
    const int k = search_node(g.qz, g.nz, z);
    s.ijkp[l] = i;
    s.ijkp[l + NM] = j;
    s.ijkp[l + 2 * NM] = k;
    if (i < 1 || i >= g.nx || j < 1 || j >= g.ny || k < 1 || k >= g.nz) {
      bad = 1;
      continue;
    }
    const R vol = R(1.0) / ((g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]));
    const R x1 = std::fabs(x - g.qx[i]), x2 = std::fabs(x - g.qx[i + 1]);
    const R y1 = std::fabs(y - g.qy[j]), y2 = std::fabs(y - g.qy[j + 1]);
    const R z1 = std::fabs(z - g.qz[k]), z2 = std::fabs(z - g.qz[k + 1]);
    R* w = s.wght.data();
    w[l + 0 * NM] = x2 * y2 * z2 * vol;
    w[l + 1 * NM] = x1 * y2 * z2 * vol;
    w[l + 2 * NM] = x2 * y2 * z1 * vol;
    w[l + 3 * NM] = x1 * y2 * z1 * vol;
    w[l + 4 * NM] = x2 * y1 * z2 * vol;
    w[l + 5 * NM] = x1 * y1 * z2 * vol;
    w[l + 6 * NM] = x2 * y1 * z1 * vol;
    w[l + 7 * NM] = x1 * y1 * z1 * vol;
  }
  if (bad) throw std::runtime_error("get_interp_weights: particle outside the grid");
}

// The eight interpolation nodes in the reference's weight order
// (gutsp.f:1484-1491): (i,j,k),(ip,j,k),(i,j,kp),(ip,j,kp),(i,jp,k),
// (ip,jp,k),(i,jp,kp),(ip,jp,kp).
template <class R>
inline void corner_nodes(const Mesh<R>& g, int i, int j, int k, std::size_t nd[8]) {
  nd[0] = g.n(i, j, k);         nd[1] = g.n(i + 1, j, k);
  nd[2] = g.n(i, j, k + 1);     nd[3] = g.n(i + 1, j, k + 1);
  nd[4] = g.n(i, j + 1, k);     nd[5] = g.n(i + 1, j + 1, k);
  nd[6] = g.n(i, j + 1, k + 1); nd[7] = g.n(i + 1, j + 1, k + 1);
}

// The periodic fold of the deposit (gutsp.f:1496-1498, 1803-1805): plane 1 is
// added into plane n-1, x then y then z.
template <class R>
void fold_scalar(const Mesh<R>& g, R* f) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  SWO_OMP_FOR(g.nt)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) f[g.n(nx - 1, j, k)] = f[g.n(nx - 1, j, k)] + f[g.n(1, j, k)];
  SWO_OMP_FOR(g.nt)
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) f[g.n(i, ny - 1, k)] = f[g.n(i, ny - 1, k)] + f[g.n(i, 1, k)];
  SWO_OMP_FOR(g.nt)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) f[g.n(i, j, nz - 1)] = f[g.n(i, j, nz - 1)] + f[g.n(i, j, 1)];
}

// Thread-private deposit grids reduced in thread order: the CPU-baseline
// analogue of the reference's particle decomposition plus MPI_ALLREDUCE
// (gutsp.f:1503,1812-1822).  With one thread this is the sequential loop.
template <class R, class F>
void deposit_loop(State<R>& s, std::int64_t ni_tot, std::size_t len, R* out, F&& body) {
  const int T = std::max(1, s.nthreads);
  if (T == 1) {
    for (std::int64_t l = 0; l < ni_tot; ++l) body(l, out);
    return;
  }
#ifdef _OPENMP
  auto& priv = s.priv;
  if (priv.size() < (std::size_t)T) priv.resize((std::size_t)T);
#pragma omp parallel num_threads(T)
  {
    const int t = omp_get_thread_num();
    auto& mine_v = priv[(std::size_t)t];
    if (mine_v.size() < len) mine_v.resize(len);
    std::fill(mine_v.begin(), mine_v.begin() + (std::ptrdiff_t)len, R(0));
    R* mine = mine_v.data();
#pragma omp for schedule(static)
    for (std::int64_t l = 0; l < ni_tot; ++l) body(l, mine);
#pragma omp for schedule(static)
    for (std::int64_t o = 0; o < (std::int64_t)len; ++o) {
      R acc = out[o];
      for (int u = 0; u < T; ++u) acc = acc + priv[(std::size_t)u][(std::size_t)o];
      out[o] = acc;
    }
  }
#else
  for (std::int64_t l = 0; l < ni_tot; ++l) body(l, out);
#endif
}

// update_np (gutsp.f:1441-1512); the MPI_ALLREDUCE of a single rank is the
// identity.  `fold_and_fill` = false returns the raw local sums (the input of
// the reference's allreduce in a multi-rank run).
template <class R>
void update_np(State<R>& s, R* np, const R* beta_p, std::int64_t ni_tot, bool fold_and_fill = true) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  std::fill(np, np + g.C, R(0.0));
  deposit_loop(s, ni_tot, g.C, np, [&](std::int64_t l, R* acc) {
    const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
    const R volb = R(1.0) / (g.dx_grid[i] * g.dy_grid[j] * g.dz_grid[k] * s.beta * beta_p[l]);
    std::size_t nd[8];
    corner_nodes(g, i, j, k, nd);
    for (int c = 0; c < 8; ++c) acc[nd[c]] = acc[nd[c]] + s.wght[l + c * NM] * volb;
  });
  if (!fold_and_fill) return;
  fold_scalar(g, np);
  periodic_scalar(g, np);
}

// update_up (gutsp.f:1649-1842): ct(node) += v*w/(np(node)*volb), fold,
// periodic, face average to up, periodic.
template <class R>
void update_up(State<R>& s, const R* vp, const R* np, R* up, const R* beta_p, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  R* ct = s.ct.data();
  std::fill(up, up + 3 * C, R(0.0));
  std::fill(ct, ct + 3 * C, R(0.0));
  deposit_loop(s, ni_tot, 3 * C, ct, [&](std::int64_t l, R* acc) {
    const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
    const R volb = (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * s.beta *
                   beta_p[l];  // gutsp.f:1692-1693
    std::size_t nd[8];
    corner_nodes(g, i, j, k, nd);
    const R v1 = vp[l], v2 = vp[l + NM], v3 = vp[l + 2 * NM];
    for (int c = 0; c < 8; ++c) {
      const R w = s.wght[l + c * NM];
      const R nvolb = R(1.0) / (np[nd[c]] * volb);
      acc[nd[c]] = acc[nd[c]] + v1 * w * nvolb;
      acc[nd[c] + C] = acc[nd[c] + C] + v2 * w * nvolb;
      acc[nd[c] + 2 * C] = acc[nd[c] + 2 * C] + v3 * w * nvolb;
    }
  });
  for (int m = 0; m < 3; ++m) fold_scalar(g, ct + C * m);  // gutsp.f:1803-1805
  periodic(g, ct);                                          // gutsp.f:1808
  SWO_OMP_FOR(g.nt)
  for (int k = 1; k <= g.nz - 1; ++k)                       // gutsp.f:1825-1836
    for (int j = 1; j <= g.ny - 1; ++j)
      for (int i = 1; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        up[o] = R(0.5) * (ct[o] + ct[g.n(i + 1, j, k)]);
        up[o + C] = R(0.5) * (ct[o + C] + ct[g.n(i, j + 1, k) + C]);
        up[o + 2 * C] = R(0.5) * (ct[o + 2 * C] + ct[g.n(i, j, k + 1) + 2 * C]);
      }
  periodic(g, up);
}

// update_rho (gutsp.f:1517-1590): mass density mnp(node) += (w/mrat)/volb,
// times mion, fold, periodic_scalar.
template <class R>
void update_rho(State<R>& s, R* mnp, const R* mrat, const R* beta_p, std::int64_t ni_tot, R mion) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  std::fill(mnp, mnp + g.C, R(0.0));
  deposit_loop(s, ni_tot, g.C, mnp, [&](std::int64_t l, R* acc) {
    const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
    const R volb = (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * s.beta *
                   beta_p[l];  // gutsp.f:1557-1558
    std::size_t nd[8];
    corner_nodes(g, i, j, k, nd);
    for (int c = 0; c < 8; ++c) acc[nd[c]] = acc[nd[c]] + (s.wght[l + c * NM] / mrat[l]) / volb;
  });
  for (std::size_t o = 0; o < g.C; ++o) mnp[o] = mion * mnp[o];  // gutsp.f:1571
  fold_scalar(g, mnp);                                            // gutsp.f:1574-1576
  periodic_scalar(g, mnp);
}

// get_temperature (gutsp.f:2257-2541): with mvp = v/sqrt(mrat), deposit
// <mvp^2> and <mvp> per node (skipping nodes with np = 0), fold, periodic,
// face-average each, then temp_p = (1/3)*1e6*mion*|<mvp^2> - <mvp>^2|.
template <class R>
void get_temperature(State<R>& s, const R* vp, const R* np, R* temp_p, const R* mrat, const R* beta_p,
                     std::int64_t ni_tot, R mion) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  std::vector<R> up2(3 * C, R(0)), upa(3 * C, R(0));
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<R>& out = pass == 0 ? up2 : upa;
    R* ct = s.ct.data();
    std::fill(ct, ct + 3 * C, R(0.0));
    deposit_loop(s, ni_tot, 3 * C, ct, [&](std::int64_t l, R* acc) {
      const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
      const R volb = (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * s.beta *
                     beta_p[l];  // gutsp.f:2310-2311
      const R sq = std::sqrt(mrat[l]);
      R mv[3];
      for (int m = 0; m < 3; ++m) {
        mv[m] = vp[l + m * NM] / sq;  // gutsp.f:2291
        if (pass == 0) mv[m] = mv[m] * mv[m];
      }
      std::size_t nd[8];
      corner_nodes(g, i, j, k, nd);
      for (int c = 0; c < 8; ++c) {
        if (!(np[nd[c]] > R(0.0))) continue;  // gutsp.f:2313, 2425 etc.
        const R nvolb = np[nd[c]] * volb;
        const R w = s.wght[l + c * NM];
        for (int m = 0; m < 3; ++m) acc[nd[c] + C * m] = acc[nd[c] + C * m] + mv[m] * w / nvolb;
      }
    });
    for (int m = 0; m < 3; ++m) fold_scalar(g, ct + C * m);  // gutsp.f:2373-2375, 2485-2487
    periodic(g, ct);
    SWO_OMP_FOR(g.nt)
    for (int k = 1; k <= g.nz - 1; ++k)  // gutsp.f:2395-2403, 2507-2515
      for (int j = 1; j <= g.ny - 1; ++j)
        for (int i = 1; i <= g.nx - 1; ++i) {
          const std::size_t o = g.n(i, j, k);
          out[o] = R(0.5) * (ct[o] + ct[g.n(i + 1, j, k)]);
          out[o + C] = R(0.5) * (ct[o + C] + ct[g.n(i, j + 1, k) + C]);
          out[o + 2 * C] = R(0.5) * (ct[o + 2 * C] + ct[g.n(i, j, k + 1) + 2 * C]);
        }
    periodic(g, out.data());
  }
  for (std::size_t o = 0; o < C; ++o) {  // gutsp.f:2521-2529
    R a[3];
    for (int m = 0; m < 3; ++m) {
      const R d = up2[o + C * m] - upa[o + C * m] * upa[o + C * m];
      a[m] = d * d;
    }
    temp_p[o] = (R(1.0) / R(3.0)) * R(1e6) * mion * std::sqrt(a[0] + a[1] + a[2]);
  }
}

// extrapol_up (gutsp.f:127-150): deposit v at time level n = 1.5 vp - 0.5 vp1.
template <class R>
void extrapol_up(State<R>& s, R* up, const R* vp, const R* vp1, const R* np, const R* beta_p,
                 std::int64_t ni_tot) {
  const std::int64_t NM = s.ni_max;
  R* vn = s.v_tmp.data();
  for (int m = 0; m < 3; ++m)
    SWO_OMP_FOR(s.g.nt)
    for (std::int64_t l = 0; l < ni_tot; ++l)
      vn[l + m * NM] = R(1.5) * vp[l + m * NM] - R(0.5) * vp1[l + m * NM];
  update_up(s, vn, np, up, beta_p, ni_tot);
}

template <class R>
inline R gather8(const R* f, const std::size_t nd[8], const R* w, std::int64_t l, std::int64_t NM) {
  // Left-to-right sum of the reference's gathers (gutsp.f:218-240).
  return f[nd[0]] * w[l] + f[nd[1]] * w[l + NM] + f[nd[2]] * w[l + 2 * NM] + f[nd[3]] * w[l + 3 * NM] +
         f[nd[4]] * w[l + 4 * NM] + f[nd[5]] * w[l + 5 * NM] + f[nd[6]] * w[l + 6 * NM] +
         f[nd[7]] * w[l + 7 * NM];
}

// get_Ep (gutsp.f:155-276): Ep = ((aj-up) x btc at the particle) * mrat.
template <class R>
void get_Ep(State<R>& s, R* Ep, R* aj, const R* np, R* up, const R* btc, const R* nu, const R* mrat,
            std::int64_t ni_tot) {
  (void)nu;
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  face_to_center(g, aj, s.ajc.data());  // gutsp.f:183
  face_to_center(g, up, s.upc.data());  // gutsp.f:184
  const R* ajc = s.ajc.data();
  const R* upc = s.upc.data();
  R* gpc = nullptr;
  std::vector<R> gradc;
  if (s.grad_pe != R(0)) {
    // centre the face pressure gradient like aj (extension; see grad_pe_at)
    std::vector<R> gface(3 * C, R(0));
    for (int k = 2; k <= g.nz - 1; ++k)
      for (int j = 2; j <= g.ny - 1; ++j)
        for (int i = 2; i <= g.nx - 1; ++i)
          for (int m = 0; m < 3; ++m) gface[g.n(i, j, k) + C * m] = grad_pe_at(s, np, i, j, k, m);
    gradc.assign(3 * C, R(0));
    face_to_center(g, gface.data(), gradc.data());
    gpc = gradc.data();
  }
#pragma omp parallel for schedule(static) num_threads(s.nthreads) if (s.nthreads > 1)
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
    std::size_t nd[8];
    corner_nodes(g, i, j, k, nd);
    R aa[3], bb[3], cc[3];
    for (int m = 0; m < 3; ++m) {
      const R aj3 = gather8(ajc + C * m, nd, s.wght.data(), l, NM);
      const R up3 = gather8(upc + C * m, nd, s.wght.data(), l, NM);
      const R bt3 = gather8(btc + C * m, nd, s.wght.data(), l, NM);
      aa[m] = aj3 - up3;  // gutsp.f:256
      bb[m] = bt3;
    }
    cc[0] = aa[1] * bb[2] - aa[2] * bb[1];
    cc[1] = aa[2] * bb[0] - aa[0] * bb[2];
    cc[2] = aa[0] * bb[1] - aa[1] * bb[0];
    for (int m = 0; m < 3; ++m) {
      R e = cc[m];
      if (gpc) e = e - gather8(gpc + C * m, nd, s.wght.data(), l, NM);
      Ep[l + m * NM] = e * mrat[l];  // gutsp.f:265-270
    }
  }
}

// get_vplus_vminus (gutsp.f:281-402): half electric kick then the analytic
// rotation about B' = mrat*B.
template <class R>
void get_vplus_vminus(State<R>& s, const R* Ep, const R* btc, const R* vp, R* vplus, R* vminus,
                      const R* mrat, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  const R dt = s.dt;
  for (int m = 0; m < 3; ++m)
    SWO_OMP_FOR(g.nt)
    for (std::int64_t l = 0; l < ni_tot; ++l)
      vminus[l + m * NM] = vp[l + m * NM] + R(0.5) * dt * Ep[l + m * NM];  // gutsp.f:302-305
#pragma omp parallel for schedule(static) num_threads(s.nthreads) if (s.nthreads > 1)
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    const int i = s.ijkp[l], j = s.ijkp[l + NM], k = s.ijkp[l + 2 * NM];
    std::size_t nd[8];
    corner_nodes(g, i, j, k, nd);
    R b3[3];
    for (int m = 0; m < 3; ++m) b3[m] = gather8(btc + C * m, nd, s.wght.data(), l, NM);
    const R mr = mrat[l];
    const R vm1 = vminus[l], vm2 = vminus[l + NM], vm3 = vminus[l + 2 * NM];
    R vxb[3];
    vxb[0] = vm2 * b3[2] * mr - vm3 * b3[1] * mr;  // gutsp.f:371-376
    vxb[1] = vm3 * b3[0] * mr - vm1 * b3[2] * mr;
    vxb[2] = vm1 * b3[1] * mr - vm2 * b3[0] * mr;
    const R vdb = vm1 * b3[0] * mr + vm2 * b3[1] * mr + vm3 * b3[2] * mr;  // :378-380
    const R Bx = b3[0] * mr, By = b3[1] * mr, Bz = b3[2] * mr;
    const R B2 = Bx * Bx + By * By + Bz * Bz;
    const R dt2 = dt * dt;
    const R a_d = R(1.0) / (R(1.0) + (R(0.25) * B2 * dt2));  // gutsp.f:389-392
    const R a1 = (R(1) - (R(0.25) * B2 * dt2)) * a_d;
    const R a2 = dt * a_d;
    const R a3 = R(0.5) * dt2 * a_d;
    const R vm[3] = {vm1, vm2, vm3};
    for (int m = 0; m < 3; ++m)
      vplus[l + m * NM] = a1 * vm[m] + a2 * vxb[m] + a3 * vdb * b3[m] * mr;  // :394-397
  }
}

// improve_up (gutsp.f:407-428)
template <class R>
void improve_up(State<R>& s, R* vp1, const R* vplus, const R* vminus, R* up, const R* np, const R* beta_p,
                std::int64_t ni_tot) {
  const std::int64_t NM = s.ni_max;
  for (int m = 0; m < 3; ++m)
    SWO_OMP_FOR(s.g.nt)
    for (std::int64_t l = 0; l < ni_tot; ++l)
      vp1[l + m * NM] = R(0.5) * (vplus[l + m * NM] + vminus[l + m * NM]);
  update_up(s, vp1, np, up, beta_p, ni_tot);
}

// get_vp_final (gutsp.f:433-449)
template <class R>
void get_vp_final(State<R>& s, const R* Ep, R* vp, R* vp1, const R* vplus, std::int64_t ni_tot) {
  const std::int64_t NM = s.ni_max;
  for (int m = 0; m < 3; ++m)
    SWO_OMP_FOR(s.g.nt)
    for (std::int64_t l = 0; l < ni_tot; ++l) {
      vp1[l + m * NM] = vp[l + m * NM];
      vp[l + m * NM] = vplus[l + m * NM] + R(0.5) * s.dt * Ep[l + m * NM];
    }
}

// move_ion_half (gutsp.f:454-570): half-step drift and periodic wrap into
// (q(1), q(n-1)] on each axis.
template <class R>
void move_ion_half(State<R>& s, R* xp, const R* vp, std::int64_t ni_tot, bool x_open = false) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const R dth = s.dt / R(2.);
  SWO_OMP_FOR(g.nt)
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    R x = xp[l] + dth * vp[l];
    R y = xp[l + NM] + dth * vp[l + NM];
    R z = xp[l + 2 * NM] + dth * vp[l + 2 * NM];
    if (!x_open) {
      if (x > g.qx[g.nx - 1]) x = g.qx[1] + (x - g.qx[g.nx - 1]);
      else if (x <= g.qx[1]) x = g.qx[g.nx - 1] - (g.qx[1] - x);
    }
    if (y > g.qy[g.ny - 1]) y = g.qy[1] + (y - g.qy[g.ny - 1]);
    else if (y <= g.qy[1]) y = g.qy[g.ny - 1] - (g.qy[1] - y);
    if (z > g.qz[g.nz - 1]) z = g.qz[1] + (z - g.qz[g.nz - 1]);
    else if (z <= g.qz[1]) z = g.qz[g.nz - 1] - (g.qz[1] - z);
    xp[l] = x; xp[l + NM] = y; xp[l + 2 * NM] = z;
  }
}

// ---------------------------------------------------------------------------
// Diagnostics
// ---------------------------------------------------------------------------

// Energy in normalized units (d_i = 1, Omega_i = 1, v_A = 1, alpha*n0 = 1),
// full 3D, accumulated in double:
//   ekin  = sum_l 0.5 * (1/mrat_l) * |v_l|^2 / (beta*beta_p_l)
//   eb1   = sum_interior 0.5*|b1-b0|^2 * dx_cell*dy_cell*dz_cell / alpha
//   eb    = same with |b1|^2
// The reference's Energy_diag (part_init.f:14-139) sums the j = 2 plane only,
// in SI units, and weights particles by beta_p instead of 1/beta_p
// (part_init.f:82-83, "/beta*beta_p"); energy_ref restates that form.
struct Energy {
  double ekin, eb1, eb, ee;
};

template <class R>
Energy energy_norm(const State<R>& s, const R* vp, const R* b0, const R* b1, const R* E, const R* mrat,
                   const R* beta_p, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  Energy en{0, 0, 0, 0};
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    const double v2 = (double)vp[l] * vp[l] + (double)vp[l + NM] * vp[l + NM] +
                      (double)vp[l + 2 * NM] * vp[l + 2 * NM];
    en.ekin += 0.5 * (1.0 / (double)mrat[l]) * v2 / ((double)s.beta * (double)beta_p[l]);
  }
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        const double vol = (double)g.dx_cell[i] * g.dy_cell[j] * g.dz_cell[k];
        for (int m = 0; m < 3; ++m) {
          const double b = b1[o + C * m], d = (double)b1[o + C * m] - (double)b0[o + C * m];
          en.eb1 += 0.5 * d * d * vol / (double)s.alpha;
          en.eb += 0.5 * b * b * vol / (double)s.alpha;
          en.ee += 0.5 * (double)E[o + C * m] * E[o + C * m] * vol;
        }
      }
  return en;
}

// Energy_diag (part_init.f:14-139) in the reference's own units and with its
// own quirks (j = 2 plane, "/beta*beta_p").  Constants per inputs.f.
template <class R>
Energy energy_ref(const State<R>& s, const R* vp, const R* b0, const R* b1, const R* E, const R* m_arr,
                  const R* beta_p, std::int64_t ni_tot, R mion) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const std::size_t C = g.C;
  const R q = R(1.6e-19), pi = R(3.14159), mu0 = pi * R(4.0e-7), eps = R(8.85e-12), km = R(1e3);
  const R m_q = mion / q;
  R EB1 = 0, EE = 0, Evp = 0;
  for (int i = 1; i <= g.nx - 1; ++i) {
    const int j = 2;
    for (int k = 1; k <= g.nz - 1; ++k) {
      const R vol = g.dx_cell[i] * g.dy_cell[j] * g.dz_cell[k] * km * km * km;
      for (int m = 0; m < 3; ++m) {
        const std::size_t o = g.n(i, j, k) + C * m;
        const R db = m_q * (b1[o] - b0[o]);
        EB1 = EB1 + (vol / (R(2.0) * mu0)) * db * db;
        const R e = m_q * E[o] * km;
        EE = EE + (eps * vol / R(2.0)) * e * e;
      }
    }
  }
  for (std::int64_t l = 0; l < ni_tot; ++l)
    for (int m = 0; m < 3; ++m) {
      const R v = vp[l + m * NM] * km;
      Evp = Evp + R(0.5) * m_arr[l] * v * v / s.beta * beta_p[l];
    }
  return Energy{(double)Evp, (double)EB1, 0.0, (double)EE};
}

// Discrete div B with forward differences over dx_grid etc. -- the divergence
// that annihilates curlE (gutsf.f:288-299), so the B update keeps it constant
// to roundoff.  Returns max over interior nodes of |div B|.
template <class R>
double max_abs_divB(const Mesh<R>& g, const R* b) {
  const std::size_t C = g.C;
  double mx = 0;
  for (int k = 2; k <= g.nz - 1; ++k)
    for (int j = 2; j <= g.ny - 1; ++j)
      for (int i = 2; i <= g.nx - 1; ++i) {
        const std::size_t o = g.n(i, j, k);
        const double d = ((double)b[g.n(i + 1, j, k)] - b[o]) / g.dx_grid[i] +
                         ((double)b[g.n(i, j + 1, k) + C] - b[o + C]) / g.dy_grid[j] +
                         ((double)b[g.n(i, j, k + 1) + 2 * C] - b[o + 2 * C]) / g.dz_grid[k];
        mx = std::max(mx, std::fabs(d));
      }
  return mx;
}

// ---------------------------------------------------------------------------
// Stable counting sort of particles by cell (an addition: the reference never
// sorts).  key = linear index of the particle's cell (i,j,k) with i fastest.
// Returns the permutation perm[new] = old.
// ---------------------------------------------------------------------------
template <class R>
void counting_sort_perm(const Mesh<R>& g, const std::int32_t* ijkp, std::int64_t ni_max, std::int64_t ni_tot,
                        std::vector<std::int64_t>& perm, std::vector<std::int64_t>& counts) {
  const std::size_t ncell = g.C;
  counts.assign(ncell, 0);
  std::vector<std::int64_t> key((std::size_t)ni_tot);
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    key[(std::size_t)l] = (std::int64_t)g.n(ijkp[l], ijkp[l + ni_max], ijkp[l + 2 * ni_max]);
    counts[(std::size_t)key[(std::size_t)l]]++;
  }
  std::vector<std::int64_t> start(ncell + 1, 0);
  for (std::size_t c = 0; c < ncell; ++c) start[c + 1] = start[c] + counts[c];
  perm.assign((std::size_t)ni_tot, 0);
  for (std::int64_t l = 0; l < ni_tot; ++l) perm[(std::size_t)start[(std::size_t)key[(std::size_t)l]]++] = l;
}

}  // namespace swo

// ---------------------------------------------------------------------------
// Particle sources and sinks (chem_rates.f, gutsp.f:12-46) and the
// extensions: x inflow/outflow, cloud ionization, charge exchange.
// The compiler's random_number (misc.f:24) is replaced by Philox4x32-10
// draws keyed by (seed, stream) with counters (step, slot, draw block), so
// the CPU and GPU paths consume identical uniforms.
// ---------------------------------------------------------------------------
namespace swo {

struct Sources {
  std::uint64_t seed;
  double ndot, vsw, beta_pu, mrat_pu, delz_ref;    // Ionize_sw_mp
  int x_open, inflow_ppc;                          // open x axis, inflow
  double inflow_vth, inflow_ux, inflow_uy, inflow_uz;
  double cloud_N0, cloud_r0, cloud_x, cloud_y, cloud_z, nu_ion, mrat_heavy, beta_heavy;  // cloud
  double cx_a, cx_b;                               // res_chex
};

using swapk::RNG_CHEX;
using swapk::RNG_CLOUD;
using swapk::RNG_INFLOW;
using swapk::RNG_IONIZE;

// Four uniforms in (0,1) for (stream, step, a, b): the product's draw.
inline void draw4(const Sources& s, std::uint32_t stream, std::int64_t step, std::int64_t a, std::uint32_t b,
                  double u[4]) {
  swapk::source_uniforms(s.seed, stream, step, a, b, u);
}

// A position drawn inside a cell must lie strictly above the cell's low node
// on the axes whose cell search is strict (x and z, gutsp.f:1396-1412), or
// the search puts it one cell lower, outside the grid at q(1).  Drawn in
// double it always does (the uniforms are at least 2^-33 above 0); rounded to
// float, a draw within half an ulp of the node lands on it, and goes to the
// next float above instead.
template <class R>
inline R above(R x, R lo) {
  return x > lo ? x : std::nextafter(lo, std::numeric_limits<R>::infinity());
}

// Ionize_sw_mp (chem_rates.f:508-646): dNi = ndot*dt*beta*beta_pu*dx*dy*delz*nz
// (:553), a Bernoulli trial when below one (:555-560), nint (:562); ring
// ions v = (vsw + vsw cos th, vsw sin th, 0) placed uniformly in the box
// (:570-577) with mrat, beta_pu (:606-608), appended after Ni_tot (:567,628).
template <class R>
std::int64_t ionize_sw_count(const State<R>& s, const Sources& src, std::int64_t step) {
  const Mesh<R>& g = s.g;
  double dNi = src.ndot * (double)s.dt * (double)s.beta * src.beta_pu * (double)g.dx * (double)g.dy * src.delz_ref *
               (double)g.nz;
  if (dNi < 1.0) {
    double u[4];
    draw4(src, RNG_IONIZE, step, -1, 0, u);
    if (dNi > u[0]) dNi = 1.0;
  }
  return (std::int64_t)std::llround(dNi);  // nint
}

template <class R>
std::int64_t ionize_sw(State<R>& s, const Sources& src, std::int64_t step, R* xp, R* vp, R* vp1, R* mrat, R* beta_p,
                       std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max, n = ionize_sw_count(s, src, step);
  if (ni_tot + n > NM) throw std::runtime_error("Ionize_sw_mp: Ni_max exceeded");
  const double twopi = 2.0 * 3.14159265358979323846;
  for (std::int64_t q = 0; q < n; ++q) {
    double u[4];
    draw4(src, RNG_IONIZE, step, q, 1, u);
    const std::int64_t l = ni_tot + q;
    const R th = (R)(u[0] * twopi);
    vp[l] = (R)src.vsw + (R)src.vsw * std::cos(th);
    vp[l + NM] = (R)src.vsw * std::sin(th);
    vp[l + 2 * NM] = R(0.0);
    xp[l] = above<R>(g.qx[1] + (R(1.0) - (R)u[1]) * (g.qx[g.nx - 1] - g.qx[1]), g.qx[1]);
    xp[l + NM] = g.qy[1] + (R(1.0) - (R)u[2]) * (g.qy[g.ny - 1] - g.qy[1]);
    xp[l + 2 * NM] = above<R>(g.qz[1] + (R(1.0) - (R)u[3]) * (g.qz[g.nz - 1] - g.qz[1]), g.qz[1]);
    for (int m = 0; m < 3; ++m) vp1[l + m * NM] = vp[l + m * NM];
    mrat[l] = (R)src.mrat_pu;
    beta_p[l] = (R)src.beta_pu;
  }
  return n;
}

// Stable removal of every particle with keep[l] == 0: the bulk form of
// remove_ion's order-preserving shift (gutsp.f:29-41).  Returns the new count.
// On more than one host thread the kept ions' destinations come from a
// blocked prefix count and each array moves through the scratch v_tmp, which
// gives the same arrays as the sequential shift.
template <class R>
std::int64_t compact(State<R>& s, const std::vector<char>& keep, R* xp, R* vp, R* vp1, R* mrat, R* beta_p,
                     std::int64_t ni_tot) {
  const std::int64_t NM = s.ni_max;
  const int T = std::max(1, s.g.nt);
  if (T == 1 || ni_tot < 4096) {
    std::int64_t w = 0;
    for (std::int64_t l = 0; l < ni_tot; ++l) {
      if (!keep[(std::size_t)l]) continue;
      if (w != l)
        for (int m = 0; m < 3; ++m) {
          xp[w + m * NM] = xp[l + m * NM];
          vp[w + m * NM] = vp[l + m * NM];
          vp1[w + m * NM] = vp1[l + m * NM];
        }
      mrat[w] = mrat[l];
      beta_p[w] = beta_p[l];
      ++w;
    }
    return w;
  }
  const std::int64_t B = (ni_tot + T - 1) / T;
  std::vector<std::int64_t> off((std::size_t)T + 1, 0);
  SWO_OMP_FOR(T)
  for (int t = 0; t < T; ++t) {
    std::int64_t c = 0;
    for (std::int64_t l = t * B; l < std::min(ni_tot, (t + 1) * B); ++l) c += keep[(std::size_t)l] ? 1 : 0;
    off[(std::size_t)t + 1] = c;
  }
  for (int t = 0; t < T; ++t) off[(std::size_t)t + 1] += off[(std::size_t)t];
  const std::int64_t w = off[(std::size_t)T];
  R* tmp = s.v_tmp.data();
  auto move = [&](R* a) {
    SWO_OMP_FOR(T)
    for (int t = 0; t < T; ++t) {
      std::int64_t d = off[(std::size_t)t];
      for (std::int64_t l = t * B; l < std::min(ni_tot, (t + 1) * B); ++l)
        if (keep[(std::size_t)l]) tmp[d++] = a[l];
    }
    SWO_OMP_FOR(T)
    for (std::int64_t l = 0; l < w; ++l) a[l] = tmp[l];
  };
  for (int m = 0; m < 3; ++m) {
    move(xp + m * NM);
    move(vp + m * NM);
    move(vp1 + m * NM);
  }
  move(mrat);
  move(beta_p);
  return w;
}

// Outflow: after a half move with the x axis open, particles with
// x > q(nx-1) or x <= q(1) leave the box.
template <class R>
std::int64_t remove_outflow_x(State<R>& s, R* xp, R* vp, R* vp1, R* mrat, R* beta_p, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  std::vector<char> keep((std::size_t)ni_tot);
  SWO_OMP_FOR(g.nt)
  for (std::int64_t l = 0; l < ni_tot; ++l) keep[(std::size_t)l] = xp[l] > g.qx[1] && xp[l] <= g.qx[g.nx - 1];
  return compact(s, keep, xp, vp, vp1, mrat, beta_p, ni_tot);
}

// Inflow: a virtual ghost slab one cell deep before x = q(1).  Each face
// cell (j,k) holds inflow_ppc particles, stratified like the load, with
// drifting-Maxwellian velocities of the reference's form; those whose
// ballistic move over one ion step crosses x = q(1) enter the box at their
// moved position.  Counts are exact functions of the draws.
template <class R>
std::int64_t inflow_x(State<R>& s, const Sources& src, std::int64_t step, R* xp, R* vp, R* vp1, R* mrat, R* beta_p,
                      std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  const int ncy = g.ny - 2, ncz = g.nz - 2, ppc = src.inflow_ppc;
  const double pi = 3.14159265358979323846;
  const R x0 = g.qx[1], dxg = g.dx_grid[1];
  std::int64_t w = ni_tot;
  for (int ck = 0; ck < ncz; ++ck)
    for (int cj = 0; cj < ncy; ++cj)
      for (int p = 0; p < ppc; ++p) {
        const std::int64_t slot = ((std::int64_t)ck * ncy + cj) * ppc + p;
        double u[4], v[4], e[4];
        draw4(src, RNG_INFLOW, step, slot, 0, u);
        draw4(src, RNG_INFLOW, step, slot, 1, v);
        draw4(src, RNG_INFLOW, step, slot, 2, e);
        const R vx = (R)(src.inflow_ux + src.inflow_vth * std::sqrt(-std::log(u[3])) * std::cos(pi * v[0]));
        const R vy = (R)(src.inflow_uy + src.inflow_vth * std::sqrt(-std::log(v[1])) * std::cos(pi * v[2]));
        const R vz = (R)(src.inflow_uz + src.inflow_vth * std::sqrt(-std::log(v[3])) * std::cos(pi * e[0]));
        const R xg = x0 - dxg + (R)u[0] * dxg;
        const R xn = xg + s.dt * vx;
        if (!(xn > x0) || xn > g.qx[g.nx - 1]) continue;
        if (w >= NM) throw std::runtime_error("inflow: Ni_max exceeded");
        xp[w] = xn;
        xp[w + NM] = g.qy[cj + 1] + (R)u[1] * (g.qy[cj + 2] - g.qy[cj + 1]);
        xp[w + 2 * NM] = above<R>(g.qz[ck + 1] + (R)u[2] * (g.qz[ck + 2] - g.qz[ck + 1]), g.qz[ck + 1]);
        vp[w] = vx; vp[w + NM] = vy; vp[w + 2 * NM] = vz;
        for (int m = 0; m < 3; ++m) vp1[w + m * NM] = vp[w + m * NM];
        mrat[w] = R(1.0);
        beta_p[w] = R(1.0);
        ++w;
      }
  return w - ni_tot;
}

// Neutral cloud density n_n(r) = N0/(1+(r/r0)^2) about (cx,cy,cz).
inline double cloud_density(const Sources& src, double x, double y, double z) {
  const double dx = x - src.cloud_x, dy = y - src.cloud_y, dz = z - src.cloud_z;
  const double r2 = (dx * dx + dy * dy + dz * dz) / (src.cloud_r0 * src.cloud_r0);
  return src.cloud_N0 / (1.0 + r2);
}

// Cloud ionization, after the per-cell rule of Ionize_pluto_mp
// (chem_rates.f:346-432): in every physical cell, n_new = vol*beta*beta_h*
// n_n(centre)*nu_ion*dt; floor plus a Bernoulli trial on the remainder; new
// heavy ions at rest, uniform in the cell.
template <class R>
std::int64_t cloud_count(const State<R>& s, const Sources& src, std::int64_t step, int ci, int cj, int ck) {
  const Mesh<R>& g = s.g;
  const double xc = 0.5 * ((double)g.qx[ci + 1] + (double)g.qx[ci + 2]);
  const double yc = 0.5 * ((double)g.qy[cj + 1] + (double)g.qy[cj + 2]);
  const double zc = 0.5 * ((double)g.qz[ck + 1] + (double)g.qz[ck + 2]);
  const double vol = (double)g.dx_grid[ci + 1] * (double)g.dy_grid[cj + 1] * (double)g.dz_grid[ck + 1];
  const double lam = vol * (double)s.beta * src.beta_heavy * cloud_density(src, xc, yc, zc) * src.nu_ion * (double)s.dt;
  std::int64_t n = (std::int64_t)std::floor(lam);
  double u[4];
  const std::int64_t cell = ((std::int64_t)ck * (g.ny - 2) + cj) * (g.nx - 2) + ci;
  draw4(src, RNG_CLOUD, step, cell, 0, u);
  if (u[0] < lam - (double)n) ++n;
  return n;
}

template <class R>
std::int64_t ionize_cloud(State<R>& s, const Sources& src, std::int64_t step, R* xp, R* vp, R* vp1, R* mrat,
                          R* beta_p, std::int64_t ni_tot) {
  const Mesh<R>& g = s.g;
  const std::int64_t NM = s.ni_max;
  std::int64_t w = ni_tot;
  for (int ck = 0; ck < g.nz - 2; ++ck)
    for (int cj = 0; cj < g.ny - 2; ++cj)
      for (int ci = 0; ci < g.nx - 2; ++ci) {
        const std::int64_t n = cloud_count(s, src, step, ci, cj, ck);
        const std::int64_t cell = ((std::int64_t)ck * (g.ny - 2) + cj) * (g.nx - 2) + ci;
        for (std::int64_t q = 0; q < n; ++q) {
          if (w >= NM) throw std::runtime_error("cloud ionization: Ni_max exceeded");
          double u[4];
          draw4(src, RNG_CLOUD, step, cell, (std::uint32_t)(1 + q), u);
          xp[w] = above<R>(g.qx[ci + 1] + (R)u[0] * (g.qx[ci + 2] - g.qx[ci + 1]), g.qx[ci + 1]);
          xp[w + NM] = g.qy[cj + 1] + (R)u[1] * (g.qy[cj + 2] - g.qy[cj + 1]);
          xp[w + 2 * NM] = above<R>(g.qz[ck + 1] + (R)u[2] * (g.qz[ck + 2] - g.qz[ck + 1]), g.qz[ck + 1]);
          for (int m = 0; m < 3; ++m) { vp[w + m * NM] = R(0); vp1[w + m * NM] = R(0); }
          mrat[w] = (R)src.mrat_heavy;
          beta_p[w] = (R)src.beta_heavy;
          ++w;
        }
      }
  return w - ni_tot;
}

// Charge exchange, after res_chex (chem_rates.f:823-840): each ion with
// mrat != mrat_heavy exchanges with probability dt*n_n*sigma*v_rel,
// sigma = a - b ln(v_rel); the new ion is heavy and at rest.  Returns the count.
template <class R>
std::int64_t res_chex(State<R>& s, const Sources& src, std::int64_t step, const R* xp, R* vp, R* vp1, R* mrat,
                      std::int64_t ni_tot) {
  const std::int64_t NM = s.ni_max;
  std::int64_t n = 0;
  for (std::int64_t l = 0; l < ni_tot; ++l) {
    if (mrat[l] == (R)src.mrat_heavy) continue;
    const double vx = vp[l], vy = vp[l + NM], vz = vp[l + 2 * NM];
    const double vrel = std::sqrt(vx * vx + vy * vy + vz * vz);
    if (!(vrel > 0.0)) continue;
    const double sigma = src.cx_a - src.cx_b * std::log(vrel);
    if (!(sigma > 0.0)) continue;
    const double prob = (double)s.dt * cloud_density(src, xp[l], xp[l + NM], xp[l + 2 * NM]) * sigma * vrel;
    double u[4];
    draw4(src, RNG_CHEX, step, l, 0, u);
    if (u[0] < prob) {
      for (int m = 0; m < 3; ++m) { vp[l + m * NM] = R(0); vp1[l + m * NM] = R(0); }
      mrat[l] = (R)src.mrat_heavy;
      ++n;
    }
  }
  return n;
}

}  // namespace swo
