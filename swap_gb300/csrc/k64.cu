// k64.cu -- FP64 kernels of the drop-in path, one per reference operator.
//
// This translation unit is compiled with --fmad=false: every multiply and add
// is rounded separately, in the order the Fortran source writes them, so that
// everything except the atomic deposit sums reproduces the FP64 CPU
// restatement bit for bit.  One thread per node (interior nodes for the
// stencils) or per particle.
#include "k64.cuh"

namespace swapk {
namespace {

constexpr int TPB = 256;

inline unsigned nblocks(long long n) {
  long long b = (n + TPB - 1) / TPB;
  return (unsigned)(b < 1 ? 1 : b);
}

#define GRID_STRIDE(t, n) for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (n); \
                               t += (long long)gridDim.x * blockDim.x)

// ---- boundary.f ----------------------------------------------------------

// periodic (boundary.f:9-52) as "every ghost node copies its interior image";
// the reference's x, y, z passes produce exactly that.
__global__ void k_periodic(Geo g, double* __restrict__ b, int ncomp) {
  const long long G = n_ghost(g);
  GRID_STRIDE(t, G) {
    int i, j, k;
    ghost_ijk(g, t, i, j, k);
    const long long dst = nidx(g, i, j, k);
    const long long src = nidx(g, wrapn(i, g.nx), wrapn(j, g.ny), wrapn(k, g.nz));
    for (int m = 0; m < ncomp; ++m) b[dst + g.C * m] = b[src + g.C * m];
  }
}

// ---- grid_interp.f -------------------------------------------------------

// face_to_center (grid_interp.f:150-171), interior nodes.
__global__ void k_face_to_center(Geo g, const double* __restrict__ v, double* __restrict__ vc) {
  const long long N = n_interior(g);
  const long long C = g.C, sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    vc[o] = g.xr[i] * (v[o] - v[o - sx]) + v[o - sx];
    vc[o + C] = g.yr[j] * (v[o + C] - v[o - sy + C]) + v[o - sy + C];
    vc[o + 2 * C] = g.zr[k] * (v[o + 2 * C] - v[o - sz + 2 * C]) + v[o - sz + 2 * C];
  }
}

// edge_to_center (grid_interp.f:22-57), interior nodes.
__global__ void k_edge_to_center(Geo g, const double* __restrict__ bt, double* __restrict__ btc) {
  const long long N = n_interior(g);
  const long long C = g.C, sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double yr = g.yr[j], xr = g.xr[i], zr = g.zr[k];
    double b1, b2;
    // component 1: y then z
    b2 = bt[o - sy] + yr * (bt[o] - bt[o - sy]);
    b1 = bt[o - sy - sz] + yr * (bt[o - sz] - bt[o - sy - sz]);
    btc[o] = b1 + zr * (b2 - b1);
    // component 2: x then z
    const double* b = bt + C;
    b2 = b[o - sx] + xr * (b[o] - b[o - sx]);
    b1 = b[o - sx - sz] + xr * (b[o - sz] - b[o - sx - sz]);
    btc[o + C] = b1 + zr * (b2 - b1);
    // component 3: y then x
    b = bt + 2 * C;
    b2 = b[o - sy] + yr * (b[o] - b[o - sy]);
    b1 = b[o - sx - sy] + yr * (b[o - sx] - b[o - sx - sy]);
    btc[o + 2 * C] = b1 + xr * (b2 - b1);
  }
}

// Face average cc_m = 0.5*(ct_m(node) + ct_m(node+e_m)) of crossf2
// (gutsf.f:94-96) and edge_to_face (grid_interp.f:123-125), interior nodes.
__global__ void k_face_avg(Geo g, const double* __restrict__ ct, double* __restrict__ cc) {
  const long long N = n_interior(g);
  const long long C = g.C, sy = g.nx, sz = (long long)g.nx * g.ny;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    cc[o] = 0.5 * (ct[o] + ct[o + 1]);
    cc[o + C] = 0.5 * (ct[o + C] + ct[o + sy + C]);
    cc[o + 2 * C] = 0.5 * (ct[o + 2 * C] + ct[o + sz + 2 * C]);
  }
}

// Cell-centre cross product of crossf2 (gutsf.f:65-76), interior nodes.
__global__ void k_cross(Geo g, const double* __restrict__ aa, const double* __restrict__ btc,
                        double* __restrict__ ct) {
  const long long N = n_interior(g);
  const long long C = g.C;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double ax = aa[o], bx = btc[o], ay = aa[o + C], by = btc[o + C], az = aa[o + 2 * C],
                 bz = btc[o + 2 * C];
    ct[o] = ay * bz - az * by;
    ct[o + C] = az * bx - ax * bz;
    ct[o + 2 * C] = ax * by - ay * bx;
  }
}

// ---- gutsf.f ---------------------------------------------------------------

// curlB (gutsf.f:202-239), interior nodes.
__global__ void k_curlB(Geo g, const double* __restrict__ b1, const double* __restrict__ np,
                        double* __restrict__ aj, double alpha) {
  const long long N = n_interior(g);
  const long long C = g.C, sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double n0 = np[o];
    const double nt1 = 0.5 * (n0 + np[o + sx]);
    const double nt2 = 0.5 * (n0 + np[o + sy]);
    const double nt3 = 0.5 * (n0 + np[o + sz]);
    const double* B1 = b1;
    const double* B2 = b1 + C;
    const double* B3 = b1 + 2 * C;
    const double c1 = (B3[o] - B3[o - sy]) / g.dyc[j] + (B2[o - sz] - B2[o]) / g.dzc[k];
    const double c2 = (B1[o] - B1[o - sz]) / g.dzc[k] + (B3[o - sx] - B3[o]) / g.dxc[i];
    const double c3 = (B2[o] - B2[o - sx]) / g.dxc[i] + (B1[o - sy] - B1[o]) / g.dyc[j];
    aj[o] = c1 / (nt1 * alpha);
    aj[o + C] = c2 / (nt2 * alpha);
    aj[o + 2 * C] = c3 / (nt3 * alpha);
  }
}

// a = aj - up (gutsf.f:1059, 1261), interior nodes.
__global__ void k_sub(Geo g, const double* __restrict__ aj, const double* __restrict__ up, double* __restrict__ a) {
  const long long N = n_interior(g);
  const long long C = g.C;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    for (int m = 0; m < 3; ++m) a[o + C * m] = aj[o + C * m] - up[o + C * m];
  }
}

// Pressure-gradient extension at faces (see oracle grad_pe_at).
__device__ __forceinline__ double grad_pe_at(const Geo& g, const double* np, double gp, long long o, int i, int j,
                                             int k, int m) {
  long long op;
  double dg;
  if (m == 0) { op = o + 1; dg = g.dxg[i]; }
  else if (m == 1) { op = o + g.nx; dg = g.dyg[j]; }
  else { op = o + (long long)g.nx * g.ny; dg = g.dzg[k]; }
  const double nf = 0.5 * (np[o] + np[op]);
  return gp * ((np[op] - np[o]) / dg) / nf;
}

// E = c + nu*aj (gutsf.f:1082, 1282), interior nodes.
__global__ void k_e_from_c(Geo g, const double* __restrict__ c, const double* __restrict__ nu,
                           const double* __restrict__ aj, const double* __restrict__ np, double gp,
                           double* __restrict__ E) {
  const long long N = n_interior(g);
  const long long C = g.C;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double nuo = nu[o];
    for (int m = 0; m < 3; ++m) {
      double e = c[o + C * m] + nuo * aj[o + C * m];
      if (gp != 0.0) e = e - grad_pe_at(g, np, gp, o, i, j, k, m);
      E[o + C * m] = e;
    }
  }
}

__global__ void k_grad_pe_face(Geo g, const double* __restrict__ np, double gp, double* __restrict__ gf) {
  const long long N = n_interior(g);
  const long long C = g.C;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    for (int m = 0; m < 3; ++m) gf[o + C * m] = grad_pe_at(g, np, gp, o, i, j, k, m);
  }
}

// curlE (gutsf.f:288-299) fused with b1p2 = base - coef*curlE
// (predict_B gutsf.f:1158-1159 with coef = 2*dtsub; correct_B :1349-1350 with
// coef = dtsub), interior nodes.
__global__ void k_curlE_update(Geo g, const double* __restrict__ E, const double* __restrict__ base, double coef,
                               double* __restrict__ b1p2) {
  const long long N = n_interior(g);
  const long long C = g.C, sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double* E1 = E;
    const double* E2 = E + C;
    const double* E3 = E + 2 * C;
    const double ce1 = (E3[o + sy] - E3[o]) / g.dyg[j] + (E2[o] - E2[o + sz]) / g.dzg[k];
    const double ce2 = (E3[o] - E3[o + sx]) / g.dxg[i] + (E1[o + sz] - E1[o]) / g.dzg[k];
    const double ce3 = (E1[o] - E1[o + sy]) / g.dyg[j] + (E2[o + sx] - E2[o]) / g.dxg[i];
    b1p2[o] = base[o] - coef * ce1;
    b1p2[o + C] = base[o + C] - coef * ce2;
    b1p2[o + 2 * C] = base[o + 2 * C] - coef * ce3;
  }
}

// btp1 = 0.5*(b1p2 + b1) over all nodes (gutsf.f:1210-1219).
__global__ void k_half_sum(long long n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ out) {
  GRID_STRIDE(t, n) out[t] = 0.5 * (a[t] + b[t]);
}

// Whistler Courant time of check_time_step (gutsf.f:1785-1792) at every node.
__global__ void k_deltat(Geo g, const double* __restrict__ bt, const double* __restrict__ np, double alpha,
                         double dx, double* __restrict__ dtn) {
  const long long C = g.C;
  GRID_STRIDE(o, C) {
    const double ak = 2. / dx;
    const double b1 = bt[o], b2 = bt[o + C], b3 = bt[o + 2 * C];
    const double btot = sqrt(b1 * b1 + b2 * b2 + b3 * b3);
    const double a1 = ak * ak * btot / (alpha * (np[o]));
    const double a2 = (ak * btot) * (ak * btot) / (alpha * (np[o]));
    const double womega = 0.5 * (a1 + sqrt(a1 * a1 + 4.0 * a2));
    const double phi = womega / ak;
    dtn[o] = dx / phi;
  }
}

// ---- gutsp.f -----------------------------------------------------------------

// get_interp_weights (gutsp.f:1391-1432).
__global__ void k_weights(Geo g, PartDev p, long long N, int* err) {
  GRID_STRIDE(l, N) {
    const double x = p.xp[l], y = p.xp[l + p.NM], z = p.xp[l + 2 * p.NM];
    const int i = cell_search(g.qx, g.nx, x, g.inv_dx);
    const int j = (int)floor(y / g.dy);
    const int k = cell_search(g.qz, g.nz, z, g.inv_dz);
    p.ijk[l] = i;
    p.ijk[l + p.NM] = j;
    p.ijk[l + 2 * p.NM] = k;
    if (i < 1 || j < 1 || j >= g.ny || k < 1) {
      set_err(err, KERR_DOMAIN);
      for (int c = 0; c < 8; ++c) p.wght[l + c * p.NM] = 0.0;
      p.ijk[l] = 1; p.ijk[l + p.NM] = 1; p.ijk[l + 2 * p.NM] = 1;
      continue;
    }
    double w[8];
    weights8(g, i, j, k, x, y, z, w);
    for (int c = 0; c < 8; ++c) p.wght[l + c * p.NM] = w[c];
  }
}

// A cell index triple is usable for node addressing only inside
// [1,n-1] on every axis; anything else is reported and skipped.
__device__ __forceinline__ bool cell_ok(const Geo& g, int i, int j, int k) {
  return i >= 1 && i <= g.nx - 1 && j >= 1 && j <= g.ny - 1 && k >= 1 && k <= g.nz - 1;
}

// The eight corners in the reference's weight order (gutsp.f:1484-1491).
__device__ __forceinline__ void corners(const Geo& g, int i, int j, int k, long long nd[8]) {
  const long long o = nidx(g, i, j, k), sy = g.nx, sz = (long long)g.nx * g.ny;
  nd[0] = o; nd[1] = o + 1; nd[2] = o + sz; nd[3] = o + 1 + sz;
  nd[4] = o + sy; nd[5] = o + 1 + sy; nd[6] = o + sy + sz; nd[7] = o + 1 + sy + sz;
}

// update_np deposit (gutsp.f:1461-1493) into the folded node.
// One value into a deterministic fixed-point sum (Fix64); a value out of
// range or not finite is flagged instead (the conversions saturate).
__device__ __forceinline__ void fix_add(const Fix64& f, long long t, double x, unsigned& bad) {
  bad |= fabs(x) < 0x1p25 ? 0u : 1u;
  const double xs = x * 0x1p28, h = floor(xs);
  atomicAdd(reinterpret_cast<unsigned long long*>(f.h) + t, (unsigned long long)__double2ll_rn(h));
  atomicAdd(f.l + t, __double2ull_rn((xs - h) * 0x1p32));
}

__global__ void k_fix_to_double(long long n, Fix64 f, double* __restrict__ out) {
  GRID_STRIDE(t, n) {
    const unsigned long long l = f.l[t];
    // the sum is hh * 2^32 + (l mod 2^32) units of 2^-60
    const long long hh = f.h[t] + (long long)(l >> 32);
    const double a = (double)hh;            // rounds beyond 2^53
    const long long r = hh - (long long)a;  // exact remainder
    out[t] = fma(a, 0x1p-28, fma((double)r, 0x1p-28, (double)(l & 0xffffffffULL) * 0x1p-60));
  }
}

template <bool DET>
__global__ void k_deposit_np(Geo g, PartDev p, long long N, double beta, double* __restrict__ np, Fix64 fx,
                             int* err) {
  unsigned bad = 0;
  GRID_STRIDE(l, N) {
    const int i = p.ijk[l], j = p.ijk[l + p.NM], k = p.ijk[l + 2 * p.NM];
    if (!cell_ok(g, i, j, k)) {
      set_err(err, KERR_DOMAIN);
      continue;
    }
    const double volb = 1.0 / (g.dxg[i] * g.dyg[j] * g.dzg[k] * beta * p.beta_p[l]);
    long long tg[8];
    corner_targets(g, i, j, k, tg);
    for (int c = 0; c < 8; ++c) {
      if (tg[c] < 0) continue;
      if (DET) fix_add(fx, tg[c], p.wght[l + c * p.NM] * volb, bad);
      else atomicAdd(np + tg[c], p.wght[l + c * p.NM] * volb);
    }
  }
  if (DET && bad) set_err(err, KERR_RANGE);
}

// update_up deposit (gutsp.f:1676-1800) without the per-node 1/np factor,
// which ct_from_sums applies once per node: sum v*w/volb.
template <bool DET>
__global__ void k_deposit_u(Geo g, PartDev p, long long N, double beta, int mode, const double* __restrict__ va,
                            const double* __restrict__ vb, double* __restrict__ out_v1, double* __restrict__ S,
                            Fix64 fx, int* err) {
  const long long C = g.C;
  unsigned bad = 0;
  GRID_STRIDE(l, N) {
    double v[3];
    const double sq = mode >= 3 ? sqrt(p.mrat[l]) : 1.0;
    for (int m = 0; m < 3; ++m) {
      const double a = va[l + m * p.NM];
      if (mode == 0) v[m] = a;
      else if (mode == 1) v[m] = 1.5 * a - 0.5 * vb[l + m * p.NM];  // gutsp.f:144
      else if (mode == 2) {
        v[m] = 0.5 * (a + vb[l + m * p.NM]);  // gutsp.f:422
        out_v1[l + m * p.NM] = v[m];
      } else {
        const double mv = a / sq;  // get_temperature's mvp (gutsp.f:2291)
        v[m] = mode == 3 ? mv * mv : mv;
      }
    }
    const int i = p.ijk[l], j = p.ijk[l + p.NM], k = p.ijk[l + 2 * p.NM];
    if (!cell_ok(g, i, j, k)) {
      set_err(err, KERR_DOMAIN);
      continue;
    }
    const double volb =
        (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * beta * p.beta_p[l];
    const double ivolb = 1.0 / volb;
    long long tg[8];
    corner_targets(g, i, j, k, tg);
    for (int c = 0; c < 8; ++c) {
      if (tg[c] < 0) continue;
      const double w = p.wght[l + c * p.NM] * ivolb;
      if (DET) {
        fix_add(fx, tg[c], v[0] * w, bad);
        fix_add(fx, tg[c] + C, v[1] * w, bad);
        fix_add(fx, tg[c] + 2 * C, v[2] * w, bad);
      } else {
        atomicAdd(S + tg[c], v[0] * w);
        atomicAdd(S + tg[c] + C, v[1] * w);
        atomicAdd(S + tg[c] + 2 * C, v[2] * w);
      }
    }
  }
  if (DET && bad) set_err(err, KERR_RANGE);
}

// update_rho deposit (gutsp.f:1543-1567): (w/mrat)/volb.
__global__ void k_deposit_rho(Geo g, PartDev p, long long N, double beta, double* __restrict__ mnp, int* err) {
  GRID_STRIDE(l, N) {
    const int i = p.ijk[l], j = p.ijk[l + p.NM], k = p.ijk[l + 2 * p.NM];
    if (!cell_ok(g, i, j, k)) {
      set_err(err, KERR_DOMAIN);
      continue;
    }
    const double volb =
        (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * beta * p.beta_p[l];
    long long tg[8];
    corner_targets(g, i, j, k, tg);
    for (int c = 0; c < 8; ++c)
      if (tg[c] >= 0) atomicAdd(mnp + tg[c], (p.wght[l + c * p.NM] / p.mrat[l]) / volb);
  }
}

// f *= a on interior nodes.
__global__ void k_scale_int(Geo g, double* __restrict__ f, double a) {
  GRID_STRIDE(t, n_interior(g)) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    f[o] = a * f[o];
  }
}

// temp_p = (1/3)*1e6*mion*|<mvp^2> - <mvp>^2| at every node (gutsp.f:2521-2527).
__global__ void k_temperature(Geo g, const double* __restrict__ up2, const double* __restrict__ upa, double mion,
                              double* __restrict__ temp) {
  const long long C = g.C;
  GRID_STRIDE(o, C) {
    double a = 0.0;
    for (int m = 0; m < 3; ++m) {
      const double d = up2[o + C * m] - upa[o + C * m] * upa[o + C * m];
      a = a + d * d;
    }
    temp[o] = (1.0 / 3.0) * 1e6 * mion * sqrt(a);
  }
}

// ct = S/np on interior nodes (the reference divides per particle by
// np(node)*volb, gutsp.f:1704; the node factor is taken out of the sum).
__global__ void k_ct_from_sums(Geo g, const double* __restrict__ S, const double* __restrict__ np,
                               double* __restrict__ ct) {
  const long long N = n_interior(g);
  const long long C = g.C;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double n = np[o];
    // A node no particle reaches keeps ct = 0, as in the reference (its
    // sums start at zero and nothing is added).
    if (n == 0.0) {
      ct[o] = 0.0; ct[o + C] = 0.0; ct[o + 2 * C] = 0.0;
      continue;
    }
    ct[o] = S[o] / n;
    ct[o + C] = S[o + C] / n;
    ct[o + 2 * C] = S[o + 2 * C] / n;
  }
}

__device__ __forceinline__ double gather8(const double* __restrict__ f, const long long nd[8],
                                          const double* __restrict__ w, long long l, long long NM) {
  return f[nd[0]] * w[l] + f[nd[1]] * w[l + NM] + f[nd[2]] * w[l + 2 * NM] + f[nd[3]] * w[l + 3 * NM] +
         f[nd[4]] * w[l + 4 * NM] + f[nd[5]] * w[l + 5 * NM] + f[nd[6]] * w[l + 6 * NM] +
         f[nd[7]] * w[l + 7 * NM];
}

// get_Ep particle loop (gutsp.f:189-273).
__global__ void k_get_Ep(Geo g, PartDev p, long long N, const double* __restrict__ ajc,
                         const double* __restrict__ upc, const double* __restrict__ btc,
                         const double* __restrict__ gpc, double* __restrict__ Ep, int* err) {
  const long long C = g.C;
  GRID_STRIDE(l, N) {
    const int i = p.ijk[l], j = p.ijk[l + p.NM], k = p.ijk[l + 2 * p.NM];
    if (!cell_ok(g, i, j, k)) {
      set_err(err, KERR_DOMAIN);
      continue;
    }
    long long nd[8];
    corners(g, i, j, k, nd);
    double aa[3], bb[3];
    for (int m = 0; m < 3; ++m) {
      const double aj3 = gather8(ajc + C * m, nd, p.wght, l, p.NM);
      const double up3 = gather8(upc + C * m, nd, p.wght, l, p.NM);
      bb[m] = gather8(btc + C * m, nd, p.wght, l, p.NM);
      aa[m] = aj3 - up3;
    }
    double cc[3];
    cc[0] = aa[1] * bb[2] - aa[2] * bb[1];
    cc[1] = aa[2] * bb[0] - aa[0] * bb[2];
    cc[2] = aa[0] * bb[1] - aa[1] * bb[0];
    const double mr = p.mrat[l];
    for (int m = 0; m < 3; ++m) {
      double e = cc[m];
      if (gpc) e = e - gather8(gpc + C * m, nd, p.wght, l, p.NM);
      Ep[l + m * p.NM] = e * mr;
    }
  }
}

// get_vplus_vminus (gutsp.f:302-399).
__global__ void k_vplus_vminus(Geo g, PartDev p, long long N, double dt, const double* __restrict__ Ep,
                               const double* __restrict__ btc, const double* __restrict__ vp,
                               double* __restrict__ vplus, double* __restrict__ vminus, int* err) {
  const long long C = g.C, NM = p.NM;
  GRID_STRIDE(l, N) {
    double vm[3];
    for (int m = 0; m < 3; ++m) {
      vm[m] = vp[l + m * NM] + 0.5 * dt * Ep[l + m * NM];
      vminus[l + m * NM] = vm[m];
    }
    const int i = p.ijk[l], j = p.ijk[l + NM], k = p.ijk[l + 2 * NM];
    if (!cell_ok(g, i, j, k)) {
      set_err(err, KERR_DOMAIN);
      continue;
    }
    long long nd[8];
    corners(g, i, j, k, nd);
    double b3[3];
    for (int m = 0; m < 3; ++m) b3[m] = gather8(btc + C * m, nd, p.wght, l, NM);
    const double mr = p.mrat[l];
    double vxb[3];
    vxb[0] = vm[1] * b3[2] * mr - vm[2] * b3[1] * mr;
    vxb[1] = vm[2] * b3[0] * mr - vm[0] * b3[2] * mr;
    vxb[2] = vm[0] * b3[1] * mr - vm[1] * b3[0] * mr;
    const double vdb = vm[0] * b3[0] * mr + vm[1] * b3[1] * mr + vm[2] * b3[2] * mr;
    const double Bx = b3[0] * mr, By = b3[1] * mr, Bz = b3[2] * mr;
    const double B2 = Bx * Bx + By * By + Bz * Bz;
    const double dt2 = dt * dt;
    const double a_d = 1.0 / (1.0 + (0.25 * B2 * dt2));
    const double a1 = (1.0 - (0.25 * B2 * dt2)) * a_d;
    const double a2 = dt * a_d;
    const double a3 = 0.5 * dt2 * a_d;
    for (int m = 0; m < 3; ++m) vplus[l + m * NM] = a1 * vm[m] + a2 * vxb[m] + a3 * vdb * b3[m] * mr;
  }
}

// get_vp_final (gutsp.f:442-446).
__global__ void k_vp_final(PartDev p, long long N, double dt, const double* __restrict__ Ep, double* __restrict__ vp,
                           double* __restrict__ vp1, const double* __restrict__ vplus) {
  GRID_STRIDE(l, N) {
    for (int m = 0; m < 3; ++m) {
      const long long o = l + m * p.NM;
      vp1[o] = vp[o];
      vp[o] = vplus[o] + 0.5 * dt * Ep[o];
    }
  }
}

// move_ion_half (gutsp.f:469-510).
__global__ void k_move_half(Geo g, PartDev p, long long N, double dt, double* __restrict__ xp,
                            const double* __restrict__ vp, bool x_open) {
  const double dth = dt / 2.;
  const long long NM = p.NM;
  GRID_STRIDE(l, N) {
    double x = xp[l] + dth * vp[l];
    double y = xp[l + NM] + dth * vp[l + NM];
    double z = xp[l + 2 * NM] + dth * vp[l + 2 * NM];
    const double qx1 = g.qx[1], qxn = g.qx[g.nx - 1];
    const double qy1 = g.qy[1], qyn = g.qy[g.ny - 1];
    const double qz1 = g.qz[1], qzn = g.qz[g.nz - 1];
    if (!x_open) {
      if (x > qxn) x = qx1 + (x - qxn);
      else if (x <= qx1) x = qxn - (qx1 - x);
    }
    if (y > qyn) y = qy1 + (y - qyn);
    else if (y <= qy1) y = qyn - (qy1 - y);
    if (z > qzn) z = qz1 + (z - qzn);
    else if (z <= qz1) z = qzn - (qz1 - z);
    xp[l] = x;
    xp[l + NM] = y;
    xp[l + 2 * NM] = z;
  }
}

// ---- reductions ----------------------------------------------------------------

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// Non-negative doubles order like their bit patterns.
__global__ void k_min_nonneg(const double* __restrict__ x, long long n, unsigned long long* out) {
  double m = 1.0e308;
  GRID_STRIDE(t, n) m = fmin(m, x[t]);
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMin(out, (unsigned long long)__double_as_longlong(m > 0.0 ? m : 0.0));
}

__global__ void k_energy_particles(PartDev p, long long N, double beta, const double* __restrict__ vp,
                                   double* acc) {
  double s = 0.0;
  GRID_STRIDE(l, N) {
    const double v1 = vp[l], v2 = vp[l + p.NM], v3 = vp[l + 2 * p.NM];
    const double v2s = v1 * v1 + v2 * v2 + v3 * v3;
    s += 0.5 * (1.0 / p.mrat[l]) * v2s / (beta * p.beta_p[l]);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) atomicAdd(acc, s);
}

__global__ void k_energy_fields(Geo g, double alpha, const double* __restrict__ b0, const double* __restrict__ b1,
                                const double* __restrict__ E, double* acc) {
  const long long N = n_interior(g);
  const long long C = g.C;
  double s1 = 0, s2 = 0, s3 = 0, sc[3] = {0, 0, 0};
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double vol = g.dxc[i] * g.dyc[j] * g.dzc[k];
    for (int m = 0; m < 3; ++m) {
      const double b = b1[o + C * m], d = b1[o + C * m] - b0[o + C * m], e = E[o + C * m];
      const double eb = 0.5 * d * d * vol / alpha;
      s1 += eb;
      sc[m] += eb;
      s2 += 0.5 * b * b * vol / alpha;
      s3 += 0.5 * e * e * vol;
    }
  }
  for (int m = 0; m < 3; ++m) {  // per component of |b1-b0|^2 (EB1x, EB1y, EB1z)
    sc[m] = block_sum(sc[m]);
    if (threadIdx.x == 0) atomicAdd(acc + 4 + m, sc[m]);
  }
  s1 = block_sum(s1);
  if (threadIdx.x == 0) atomicAdd(acc + 1, s1);
  s2 = block_sum(s2);
  if (threadIdx.x == 0) atomicAdd(acc + 2, s2);
  s3 = block_sum(s3);
  if (threadIdx.x == 0) atomicAdd(acc + 3, s3);
}

__global__ void k_divb_max(Geo g, const double* __restrict__ b, unsigned long long* out) {
  const long long N = n_interior(g);
  const long long C = g.C, sy = g.nx, sz = (long long)g.nx * g.ny;
  double m = 0.0;
  GRID_STRIDE(t, N) {
    int i, j, k;
    interior_ijk(g, t, i, j, k);
    const long long o = nidx(g, i, j, k);
    const double d = (b[o + 1] - b[o]) / g.dxg[i] + (b[o + sy + C] - b[o + C]) / g.dyg[j] +
                     (b[o + sz + 2 * C] - b[o + 2 * C]) / g.dzg[k];
    m = fmax(m, fabs(d));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_nonfinite(const double* __restrict__ x, long long n, unsigned long long* cnt) {
  unsigned long long c = 0;
  GRID_STRIDE(t, n) c += isfinite(x[t]) ? 0ull : 1ull;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

}  // namespace

// ---- launchers -------------------------------------------------------------------

#define LAUNCH(kern, n, ...)                                     \
  do {                                                           \
    kern<<<nblocks(n), TPB, 0, st>>>(__VA_ARGS__);                \
    return cudaGetLastError();                                   \
  } while (0)

cudaError_t periodic3(const Geo& g, double* b, cudaStream_t st) { LAUNCH(k_periodic, n_ghost(g), g, b, 3); }
cudaError_t periodic1(const Geo& g, double* b, cudaStream_t st) { LAUNCH(k_periodic, n_ghost(g), g, b, 1); }
cudaError_t face_to_center_int(const Geo& g, const double* v, double* vc, cudaStream_t st) {
  LAUNCH(k_face_to_center, n_interior(g), g, v, vc);
}
cudaError_t edge_to_center_int(const Geo& g, const double* bt, double* btc, cudaStream_t st) {
  LAUNCH(k_edge_to_center, n_interior(g), g, bt, btc);
}
cudaError_t face_avg_int(const Geo& g, const double* ct, double* cc, cudaStream_t st) {
  LAUNCH(k_face_avg, n_interior(g), g, ct, cc);
}
cudaError_t cross_int(const Geo& g, const double* aa, const double* btc, double* ct, cudaStream_t st) {
  LAUNCH(k_cross, n_interior(g), g, aa, btc, ct);
}
cudaError_t curlB_int(const Geo& g, const double* b1, const double* np, double* aj, double alpha, cudaStream_t st) {
  LAUNCH(k_curlB, n_interior(g), g, b1, np, aj, alpha);
}
cudaError_t sub_int(const Geo& g, const double* aj, const double* up, double* a, cudaStream_t st) {
  LAUNCH(k_sub, n_interior(g), g, aj, up, a);
}
cudaError_t e_from_c_int(const Geo& g, const double* c, const double* nu, const double* aj, const double* np,
                         double gp, double* E, cudaStream_t st) {
  LAUNCH(k_e_from_c, n_interior(g), g, c, nu, aj, np, gp, E);
}
cudaError_t grad_pe_face_int(const Geo& g, const double* np, double gp, double* gf, cudaStream_t st) {
  LAUNCH(k_grad_pe_face, n_interior(g), g, np, gp, gf);
}
cudaError_t curlE_update_int(const Geo& g, const double* E, const double* base, double coef, double* b1p2,
                             cudaStream_t st) {
  LAUNCH(k_curlE_update, n_interior(g), g, E, base, coef, b1p2);
}
cudaError_t half_sum_all(const Geo& g, const double* a, const double* b, double* out, cudaStream_t st) {
  LAUNCH(k_half_sum, 3 * g.C, 3 * g.C, a, b, out);
}
cudaError_t deltat_all(const Geo& g, const double* bt, const double* np, double alpha, double dx, double* dtn,
                       cudaStream_t st) {
  LAUNCH(k_deltat, g.C, g, bt, np, alpha, dx, dtn);
}
cudaError_t interp_weights(const Geo& g, const PartDev& p, long long N, int* err, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_weights, N, g, p, N, err);
}
cudaError_t deposit_np(const Geo& g, const PartDev& p, long long N, double beta, double* np, int* err,
                       cudaStream_t st, Fix64 fix) {
  if (N <= 0) return cudaSuccess;
  if (fix.h) LAUNCH(k_deposit_np<true>, N, g, p, N, beta, np, fix, err);
  LAUNCH(k_deposit_np<false>, N, g, p, N, beta, np, fix, err);
}
cudaError_t deposit_u(const Geo& g, const PartDev& p, long long N, double beta, int mode, const double* va,
                      const double* vb, double* out_v1, double* S, int* err, cudaStream_t st, Fix64 fix) {
  if (N <= 0) return cudaSuccess;
  if (fix.h) LAUNCH(k_deposit_u<true>, N, g, p, N, beta, mode, va, vb, out_v1, S, fix, err);
  LAUNCH(k_deposit_u<false>, N, g, p, N, beta, mode, va, vb, out_v1, S, fix, err);
}
cudaError_t fix_to_double(long long n, Fix64 fix, double* out, cudaStream_t st) {
  LAUNCH(k_fix_to_double, n, n, fix, out);
}
cudaError_t deposit_rho(const Geo& g, const PartDev& p, long long N, double beta, double* mnp, int* err,
                        cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_deposit_rho, N, g, p, N, beta, mnp, err);
}
cudaError_t scale_interior(const Geo& g, double* f, double a, cudaStream_t st) {
  LAUNCH(k_scale_int, n_interior(g), g, f, a);
}
cudaError_t temperature(const Geo& g, const double* up2, const double* upa, double mion, double* temp,
                        cudaStream_t st) {
  LAUNCH(k_temperature, g.C, g, up2, upa, mion, temp);
}
cudaError_t ct_from_sums(const Geo& g, const double* S, const double* np, double* ct, cudaStream_t st) {
  LAUNCH(k_ct_from_sums, n_interior(g), g, S, np, ct);
}
cudaError_t get_Ep(const Geo& g, const PartDev& p, long long N, const double* ajc, const double* upc,
                   const double* btc, const double* gpc, double* Ep, int* err, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_get_Ep, N, g, p, N, ajc, upc, btc, gpc, Ep, err);
}
cudaError_t vplus_vminus(const Geo& g, const PartDev& p, long long N, double dt, const double* Ep,
                         const double* btc, const double* vp, double* vplus, double* vminus, int* err,
                         cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_vplus_vminus, N, g, p, N, dt, Ep, btc, vp, vplus, vminus, err);
}
cudaError_t vp_final(const PartDev& p, long long N, double dt, const double* Ep, double* vp, double* vp1,
                     const double* vplus, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_vp_final, N, p, N, dt, Ep, vp, vp1, vplus);
}
cudaError_t move_half(const Geo& g, const PartDev& p, long long N, double dt, double* xp, const double* vp,
                      bool x_open, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  LAUNCH(k_move_half, N, g, p, N, dt, xp, vp, x_open);
}
cudaError_t reduce_min(const double* x, long long n, double* d_out, int, cudaStream_t st) {
  const unsigned long long init = (unsigned long long)0x7fefffffffffffffULL;  // DBL_MAX bits
  cudaError_t e = cudaMemcpyAsync(d_out, &init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  LAUNCH(k_min_nonneg, n, x, n, reinterpret_cast<unsigned long long*>(d_out));
}
cudaError_t energy_parts(const Geo& g, const PartDev& p, long long N, double beta, double alpha, const double* vp,
                         const double* b0, const double* b1, const double* E, double* d_acc4, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(d_acc4, 0, 7 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (N > 0) {
    k_energy_particles<<<nblocks(N), TPB, 0, st>>>(p, N, beta, vp, d_acc4);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  LAUNCH(k_energy_fields, n_interior(g), g, alpha, b0, b1, E, d_acc4);
}
cudaError_t divb_max(const Geo& g, const double* b, double* d_max, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(d_max, 0, sizeof(double), st);
  if (e != cudaSuccess) return e;
  LAUNCH(k_divb_max, n_interior(g), g, b, reinterpret_cast<unsigned long long*>(d_max));
}
cudaError_t count_nonfinite(const double* x, long long n, unsigned long long* d_cnt, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  LAUNCH(k_nonfinite, n, x, n, d_cnt);
}

// ---- the caller's 4-byte reals ------------------------------------------------

__global__ void k_widen(const float* __restrict__ in, double* __restrict__ out, long long n) {
  GRID_STRIDE(i, n) out[i] = (double)in[i];
}

__global__ void k_narrow(const double* __restrict__ in, float* __restrict__ out, long long n) {
  GRID_STRIDE(i, n) out[i] = (float)in[i];
}

cudaError_t widen_f32(const float* in, double* out, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_widen<<<nblocks(n), TPB, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t narrow_f64(const double* in, float* out, long long n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_narrow<<<nblocks(n), TPB, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

}  // namespace swapk
