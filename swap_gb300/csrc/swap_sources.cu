// swap_sources.cu -- particle sources and sinks of the ion step: the
// reference's Ionize_sw_mp (chem_rates.f:508-646), remove_ion
// (gutsp.f:12-46) and res_chex (chem_rates.f:805-843), an open x axis with
// inflow and outflow, and per-cell ionization of a neutral cloud (after
// Ionize_pluto_mp, chem_rates.f:290-503).  Random draws are Philox
// (philox.h: source_uniforms) keyed by (seed, rule, step, slot), so counts
// and new-particle positions equal the CPU restatement's.  Compiled with
// --fmad=false like the FP64 drop-in.
#include <algorithm>
#include <cmath>
#include <string>

#include "../../include/swap_gpu.h"
#include "k32.cuh"
#include "k64.cuh"
#include "philox.h"
#include "swap_ctx.h"
#include "swap_ops.h"
#include "swap_prof.h"

using namespace swapk;

namespace {

constexpr int TPB = 256;
inline unsigned nb(long long n) { return (unsigned)((n + TPB - 1) / TPB < 1 ? 1 : (n + TPB - 1) / TPB); }

struct PView {
  double *xp, *vp, *vp1, *mrat, *beta_p;
  long long NM;
};

// Ionize_sw_mp's new ions (chem_rates.f:567-620): ring velocity, uniform
// position in the box, pickup mrat and beta_pu.
__global__ void k_ionize(Geo g, PView p, long long N, long long n, swap_sources s, long long step) {
  const double twopi = 2.0 * 3.14159265358979323846;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    double u[4];
    source_uniforms(s.seed, RNG_IONIZE, step, q, 1u, u);
    const long long l = N + q, NM = p.NM;
    const double th = u[0] * twopi;
    p.vp[l] = s.vsw + s.vsw * cos(th);
    p.vp[l + NM] = s.vsw * sin(th);
    p.vp[l + 2 * NM] = 0.0;
    p.xp[l] = g.qx[1] + (1.0 - u[1]) * (g.qx[g.nx - 1] - g.qx[1]);
    p.xp[l + NM] = g.qy[1] + (1.0 - u[2]) * (g.qy[g.ny - 1] - g.qy[1]);
    p.xp[l + 2 * NM] = g.qz[1] + (1.0 - u[3]) * (g.qz[g.nz - 1] - g.qz[1]);
    for (int m = 0; m < 3; ++m) p.vp1[l + m * NM] = p.vp[l + m * NM];
    p.mrat[l] = s.mrat_pu;
    p.beta_p[l] = s.beta_pu;
  }
}

// Inflow: the ghost-slab candidate of slot (ck, cj, pp); returns whether
// its ballistic move over dt crosses x = q(1) into the box, and the state.
__device__ __forceinline__ bool inflow_candidate(const Geo& g, const swap_sources& s, long long step, long long slot,
                                                 int cj, int ck, double dt, double st[6]) {
  const double pi = 3.14159265358979323846;
  double u[4], v[4], e[4];
  source_uniforms(s.seed, RNG_INFLOW, step, slot, 0u, u);
  source_uniforms(s.seed, RNG_INFLOW, step, slot, 1u, v);
  source_uniforms(s.seed, RNG_INFLOW, step, slot, 2u, e);
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

__global__ void k_inflow_flags(Geo g, swap_sources s, long long step, double dt, int64_t* flag) {
  const int ncy = g.ny - 2, ncz = g.nz - 2, ppc = s.inflow_ppc;
  const long long nslot = (long long)ncy * ncz * ppc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslot; t += (long long)gridDim.x * blockDim.x) {
    const int cj = (int)((t / ppc) % ncy), ck = (int)(t / ((long long)ppc * ncy));
    double st[6];
    flag[t] = inflow_candidate(g, s, step, t, cj, ck, dt, st) ? 1 : 0;
  }
}

__global__ void k_inflow_write(Geo g, PView p, swap_sources s, long long step, double dt, const int64_t* flag,
                               const int64_t* pos, long long N) {
  const int ncy = g.ny - 2, ncz = g.nz - 2, ppc = s.inflow_ppc;
  const long long nslot = (long long)ncy * ncz * ppc, NM = p.NM;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslot; t += (long long)gridDim.x * blockDim.x) {
    if (!flag[t]) continue;
    const int cj = (int)((t / ppc) % ncy), ck = (int)(t / ((long long)ppc * ncy));
    double st[6];
    inflow_candidate(g, s, step, t, cj, ck, dt, st);
    const long long l = N + pos[t];
    p.xp[l] = st[0]; p.xp[l + NM] = st[1]; p.xp[l + 2 * NM] = st[2];
    for (int m = 0; m < 3; ++m) { p.vp[l + m * NM] = st[3 + m]; p.vp1[l + m * NM] = st[3 + m]; }
    p.mrat[l] = 1.0;
    p.beta_p[l] = 1.0;
  }
}

__device__ __forceinline__ double cloud_density(const swap_sources& s, double x, double y, double z) {
  const double dx = x - s.cloud_x, dy = y - s.cloud_y, dz = z - s.cloud_z;
  const double r2 = (dx * dx + dy * dy + dz * dz) / (s.cloud_r0 * s.cloud_r0);
  return s.cloud_N0 / (1.0 + r2);
}

// Cloud ionization: new heavy ions of one cell: floor(lambda) + Bernoulli(remainder).
__global__ void k_cloud_count(Geo g, swap_sources s, long long step, double dt, double beta, int64_t* cnt) {
  const int ncx = g.nx - 2, ncy = g.ny - 2, ncz = g.nz - 2;
  const long long ncell = (long long)ncx * ncy * ncz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c % ncx), cj = (int)((c / ncx) % ncy), ck = (int)(c / ((long long)ncx * ncy));
    const double xc = 0.5 * (g.qx[ci + 1] + g.qx[ci + 2]);
    const double yc = 0.5 * (g.qy[cj + 1] + g.qy[cj + 2]);
    const double zc = 0.5 * (g.qz[ck + 1] + g.qz[ck + 2]);
    const double vol = g.dxg[ci + 1] * g.dyg[cj + 1] * g.dzg[ck + 1];
    const double lam = vol * beta * s.beta_heavy * cloud_density(s, xc, yc, zc) * s.nu_ion * dt;
    long long n = (long long)floor(lam);
    double u[4];
    source_uniforms(s.seed, RNG_CLOUD, step, c, 0u, u);
    if (u[0] < lam - (double)n) ++n;
    cnt[c] = n;
  }
}

__global__ void k_cloud_write(Geo g, PView p, swap_sources s, long long step, const int64_t* cnt, const int64_t* pos,
                              long long N) {
  const int ncx = g.nx - 2, ncy = g.ny - 2, ncz = g.nz - 2;
  const long long ncell = (long long)ncx * ncy * ncz, NM = p.NM;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c % ncx), cj = (int)((c / ncx) % ncy), ck = (int)(c / ((long long)ncx * ncy));
    for (long long q = 0; q < cnt[c]; ++q) {
      double u[4];
      source_uniforms(s.seed, RNG_CLOUD, step, c, (uint32_t)(1 + q), u);
      const long long l = N + pos[c] + q;
      p.xp[l] = g.qx[ci + 1] + u[0] * (g.qx[ci + 2] - g.qx[ci + 1]);
      p.xp[l + NM] = g.qy[cj + 1] + u[1] * (g.qy[cj + 2] - g.qy[cj + 1]);
      p.xp[l + 2 * NM] = g.qz[ck + 1] + u[2] * (g.qz[ck + 2] - g.qz[ck + 1]);
      for (int m = 0; m < 3; ++m) { p.vp[l + m * NM] = 0.0; p.vp1[l + m * NM] = 0.0; }
      p.mrat[l] = s.mrat_heavy;
      p.beta_p[l] = s.beta_heavy;
    }
  }
}

// Charge exchange after res_chex (chem_rates.f:823-840).
__global__ void k_chex(PView p, long long N, swap_sources s, long long step, double dt, unsigned long long* count) {
  const long long NM = p.NM;
  unsigned long long mine = 0;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    if (p.mrat[l] == s.mrat_heavy) continue;
    const double vx = p.vp[l], vy = p.vp[l + NM], vz = p.vp[l + 2 * NM];
    const double vrel = sqrt(vx * vx + vy * vy + vz * vz);
    if (!(vrel > 0.0)) continue;
    const double sigma = s.cx_a - s.cx_b * log(vrel);
    if (!(sigma > 0.0)) continue;
    const double prob = dt * cloud_density(s, p.xp[l], p.xp[l + NM], p.xp[l + 2 * NM]) * sigma * vrel;
    double u[4];
    source_uniforms(s.seed, RNG_CHEX, step, l, 0u, u);
    if (u[0] < prob) {
      for (int m = 0; m < 3; ++m) { p.vp[l + m * NM] = 0.0; p.vp1[l + m * NM] = 0.0; }
      p.mrat[l] = s.mrat_heavy;
      ++mine;
    }
  }
  if (mine) atomicAdd(count, mine);
}

__global__ void k_outflow_flags(Geo g, const double* xp, long long N, int64_t* keep) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    keep[l] = (xp[l] > g.qx[1] && !(xp[l] > g.qx[g.nx - 1])) ? 1 : 0;
}

__global__ void k_keep_all_but(long long N, long long drop, int64_t* keep) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    keep[l] = l == drop ? 0 : 1;
}

// Stable compaction of one component array (8-byte or 4-byte elements).
template <class T>
__global__ void k_compact(const T* __restrict__ src, T* __restrict__ dst, long long N, const int64_t* __restrict__ keep,
                          const int64_t* __restrict__ pos) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x)
    if (keep[l]) dst[pos[l]] = src[l];
}

}  // namespace


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define TRY(x)         \
  do {                 \
    int _r = (x);      \
    if (_r) return _r; \
  } while (0)
#define CU(x)                                           \
  do {                                                  \
    cudaError_t _e = (x);                               \
    if (_e != cudaSuccess) return c->cuda_fail(_e, #x); \
  } while (0)

namespace {

// Scan scratch for n flags (grown on demand), one ni_max buffer of 8-byte
// elements for compaction, and the res_chex counters.
int src_scratch(swap_ctx* c, long long n) {
  if (!c->src_tmp) {
    const std::size_t nm = (std::size_t)(c->dims.ni_max > 0 ? c->dims.ni_max : 1);
    void *t = nullptr, *k = nullptr;
    if (cudaMalloc(&t, nm * 8) != cudaSuccess) return c->fail(SWAP_ECUDA, "allocation of source/sink scratch failed");
    c->src_tmp = t;
    if (cudaMalloc(&k, 4 * sizeof(unsigned long long)) != cudaSuccess)
      return c->fail(SWAP_ECUDA, "allocation of source/sink counters failed");
    c->src_cnt = static_cast<unsigned long long*>(k);
    CU(cudaMemsetAsync(c->src_cnt, 0, 4 * sizeof(unsigned long long), c->st));
  }
  if (n <= c->src_cap) return SWAP_OK;
  CU(cudaStreamSynchronize(c->st));
  for (int64_t* p : {c->src_flag, c->src_pos, c->src_sums})
    if (p) cudaFree(p);
  c->src_flag = c->src_pos = c->src_sums = nullptr;
  c->src_cap = 0;
  const long long cap = n + n / 8 + 1024;
  void *a = nullptr, *b = nullptr, *d = nullptr;
  if (cudaMalloc(&a, (std::size_t)(cap + 1) * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc(&b, (std::size_t)(cap + 1) * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc(&d, (std::size_t)(cap / 1024 + 16) * sizeof(int64_t)) != cudaSuccess) {
    if (a) cudaFree(a);
    if (b) cudaFree(b);
    return c->fail(SWAP_ECUDA, "allocation of source/sink scan scratch failed");
  }
  c->src_flag = static_cast<int64_t*>(a);
  c->src_pos = static_cast<int64_t*>(b);
  c->src_sums = static_cast<int64_t*>(d);
  c->src_cap = cap;
  return SWAP_OK;
}

// Exclusive scan of src_flag[0..n) into src_pos; returns the total.
int scan_count(swap_ctx* c, long long n, long long* total) {
  CU(swapk32::scan_exclusive(c->src_flag, c->src_pos, n, c->src_sums, c->st));
  int64_t t = 0;
  CU(cudaMemcpyAsync(&t, c->src_pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  *total = t;
  return SWAP_OK;
}

PView pview(swap_ctx* c, double* xp, double* vp, double* vp1) {
  return PView{xp, vp, vp1, c->d_mrat, c->d_beta_p, c->dims.ni_max};
}

template <class T>
int compact_one(swap_ctx* c, T* a, long long N, long long kept) {
  T* tmp = static_cast<T*>(c->src_tmp);
  k_compact<T><<<nb(N), TPB, 0, c->st>>>(a, tmp, N, c->src_flag, c->src_pos);
  CU(cudaGetLastError());
  if (kept > 0) CU(cudaMemcpyAsync(a, tmp, (std::size_t)kept * sizeof(T), cudaMemcpyDeviceToDevice, c->st));
  return SWAP_OK;
}

// Stable removal of the particles whose src_flag is 0 from xp, vp, vp1, mrat
// and beta_p: the bulk form of remove_ion's shift (gutsp.f:29-41).  With
// keep_weights the device ijkp/wght are shifted too (gutsp.f:33,37-39);
// otherwise they are marked stale.
int compact_particles(swap_ctx* c, double* xp, double* vp, double* vp1, bool keep_weights) {
  const long long N = c->ntot(), NM = c->dims.ni_max;
  long long kept = 0;
  TRY(scan_count(c, N, &kept));
  if (kept == N) return SWAP_OK;
  for (int m = 0; m < 3; ++m) {
    TRY(compact_one(c, xp + m * NM, N, kept));
    TRY(compact_one(c, vp + m * NM, N, kept));
    TRY(compact_one(c, vp1 + m * NM, N, kept));
  }
  TRY(compact_one(c, c->d_mrat, N, kept));
  TRY(compact_one(c, c->d_beta_p, N, kept));
  if (keep_weights && c->weights_valid && c->weights_n >= N) {
    for (int m = 0; m < 3; ++m) TRY(compact_one(c, c->d_ijk + m * NM, N, kept));
    for (int m = 0; m < 8; ++m) TRY(compact_one(c, c->d_wght + m * NM, N, kept));
    c->weights_n = kept;
  } else {
    c->weights_valid = false;
  }
  CU(cudaStreamSynchronize(c->st));
  *c->ni_tot_ptr = (int32_t)kept;
  return SWAP_OK;
}

// dNi of Ionize_sw_mp (chem_rates.f:551-562) with the Bernoulli draw of
// step m, in the CPU restatement's operation order.
long long ionize_count(const swap_ctx* c, long long m) {
  const swap_sources& s = c->srcs;
  double dNi = s.ndot * c->prm.dt * c->prm.beta * s.beta_pu * c->prm.dx * c->prm.dy * s.delz_ref * (double)c->dims.nz;
  if (dNi < 1.0) {
    double u[4];
    source_uniforms(s.seed, RNG_IONIZE, m, -1, 0u, u);
    if (dNi > u[0]) dNi = 1.0;
  }
  return (long long)std::llround(dNi);
}

int src_ionize(swap_ctx* c, double* xp, double* vp, double* vp1, long long m) {
  const long long N = c->ntot(), n = ionize_count(c, m);
  if (n <= 0) return SWAP_OK;
  if (N + n > c->dims.ni_max) return c->fail(SWAP_ECAPACITY, "Ionize_sw_mp: Ni_max exceeded");
  {
    ProfScope ps(c, "src_ionize", c->st);
    k_ionize<<<nb(n), TPB, 0, c->st>>>(c->g, pview(c, xp, vp, vp1), N, n, c->srcs, m);
  }
  CU(cudaGetLastError());
  *c->ni_tot_ptr = (int32_t)(N + n);
  return SWAP_OK;
}

int src_inflow(swap_ctx* c, double* xp, double* vp, double* vp1, long long m) {
  const swap_sources& s = c->srcs;
  const long long nslot = (long long)(c->dims.ny - 2) * (c->dims.nz - 2) * s.inflow_ppc;
  if (nslot <= 0) return SWAP_OK;
  TRY(src_scratch(c, nslot));
  {
    ProfScope ps(c, "src_inflow_flags", c->st);
    k_inflow_flags<<<nb(nslot), TPB, 0, c->st>>>(c->g, s, m, c->prm.dt, c->src_flag);
  }
  CU(cudaGetLastError());
  long long n = 0;
  TRY(scan_count(c, nslot, &n));
  const long long N = c->ntot();
  if (N + n > c->dims.ni_max) return c->fail(SWAP_ECAPACITY, "inflow: Ni_max exceeded");
  if (n > 0) {
    {
      ProfScope ps(c, "src_inflow_write", c->st);
      k_inflow_write<<<nb(nslot), TPB, 0, c->st>>>(c->g, pview(c, xp, vp, vp1), s, m, c->prm.dt, c->src_flag,
                                                    c->src_pos, N);
    }
    CU(cudaGetLastError());
  }
  *c->ni_tot_ptr = (int32_t)(N + n);
  return SWAP_OK;
}

int src_cloud(swap_ctx* c, double* xp, double* vp, double* vp1, long long m) {
  const long long ncell = (long long)(c->dims.nx - 2) * (c->dims.ny - 2) * (c->dims.nz - 2);
  TRY(src_scratch(c, ncell));
  {
    ProfScope ps(c, "src_cloud_count", c->st);
    k_cloud_count<<<nb(ncell), TPB, 0, c->st>>>(c->g, c->srcs, m, c->prm.dt, c->prm.beta, c->src_flag);
  }
  CU(cudaGetLastError());
  long long n = 0;
  TRY(scan_count(c, ncell, &n));
  const long long N = c->ntot();
  if (N + n > c->dims.ni_max) return c->fail(SWAP_ECAPACITY, "cloud ionization: Ni_max exceeded");
  if (n > 0) {
    {
      ProfScope ps(c, "src_cloud_write", c->st);
      k_cloud_write<<<nb(ncell), TPB, 0, c->st>>>(c->g, pview(c, xp, vp, vp1), c->srcs, m, c->src_flag, c->src_pos,
                                                   N);
    }
    CU(cudaGetLastError());
  }
  *c->ni_tot_ptr = (int32_t)(N + n);
  return SWAP_OK;
}

int src_outflow(swap_ctx* c, double* xp, double* vp, double* vp1, bool keep_weights) {
  const long long N = c->ntot();
  if (N <= 0) return SWAP_OK;
  TRY(src_scratch(c, N));
  {
    ProfScope ps(c, "src_outflow", c->st);
    k_outflow_flags<<<nb(N), TPB, 0, c->st>>>(c->g, xp, N, c->src_flag);
  }
  CU(cudaGetLastError());
  return compact_particles(c, xp, vp, vp1, keep_weights);
}

// res_chex over the live particles; the count of this call goes to
// src_cnt[0] and is added to src_cnt[1].
int src_chex(swap_ctx* c, double* xp, double* vp, double* vp1, long long m) {
  TRY(src_scratch(c, 0));
  const long long N = c->ntot();
  CU(cudaMemsetAsync(c->src_cnt, 0, sizeof(unsigned long long), c->st));
  if (N > 0) {
    {
      ProfScope ps(c, "src_chex", c->st);
      k_chex<<<nb(N), TPB, 0, c->st>>>(pview(c, xp, vp, vp1), N, c->srcs, m, c->prm.dt, c->src_cnt);
    }
    CU(cudaGetLastError());
  }
  return SWAP_OK;
}

__global__ void k_add_count(unsigned long long* cnt) { cnt[1] += cnt[0]; }

bool active(const swap_ctx* c) { return c->have_srcs; }

// mrat and beta_p change with every source and sink.
int touch_scalars(swap_ctx* c) {
  if (!c->h_mrat) return c->fail(SWAP_EINVAL, "swap_bind_particles has not been called");
  double* d;
  TRY(c->use(c->h_mrat, Access::InOut, &d));
  TRY(c->use(c->h_beta_p, Access::InOut, &d));
  return SWAP_OK;
}

}  // namespace

namespace srcops {

bool x_open(const swap_ctx* c) { return c->have_srcs && c->srcs.x_open != 0; }

int step_begin(swap_ctx* c, double* xp, double* vp, double* vp1) {
  if (!active(c)) return SWAP_OK;
  TRY(touch_scalars(c));
  const long long m = c->src_step;
  if (c->srcs.ndot > 0) TRY(src_ionize(c, xp, vp, vp1, m));
  if (c->srcs.nu_ion > 0) TRY(src_cloud(c, xp, vp, vp1, m));
  if (c->srcs.x_open) TRY(src_inflow(c, xp, vp, vp1, m));
  return SWAP_OK;
}

int after_move(swap_ctx* c, double* xp, double* vp, double* vp1) {
  if (!x_open(c)) return SWAP_OK;
  return src_outflow(c, xp, vp, vp1, false);
}

int step_end(swap_ctx* c, double* xp, double* vp, double* vp1) {
  if (!active(c)) return SWAP_OK;
  if (c->srcs.cx_a > 0) {
    TRY(src_chex(c, xp, vp, vp1, c->src_step));
    k_add_count<<<1, 1, 0, c->st>>>(c->src_cnt);
    CU(cudaGetLastError());
  }
  c->src_step++;
  return SWAP_OK;
}

void free_all(swap_ctx* c) {
  for (void* p : {(void*)c->src_flag, (void*)c->src_pos, (void*)c->src_sums, c->src_tmp, (void*)c->src_cnt})
    if (p) cudaFree(p);
  c->src_flag = c->src_pos = c->src_sums = nullptr;
  c->src_tmp = nullptr;
  c->src_cnt = nullptr;
  c->src_cap = 0;
}

}  // namespace srcops

// ---------------------------------------------------------------------------
// C-ABI entries
// ---------------------------------------------------------------------------

extern "C" int swap_set_sources(swap_ctx* c, const swap_sources* s, int64_t step0) {
  if (!c || !s) return SWAP_EINVAL;
  c->err.clear();
  if (s->inflow_ppc < 0) return c->fail(SWAP_EINVAL, "inflow_ppc must be >= 0");
  if (s->nu_ion > 0 && !(s->cloud_r0 > 0)) return c->fail(SWAP_EINVAL, "cloud_r0 must be > 0");
  if (s->cx_a > 0 && !(s->cloud_r0 > 0)) return c->fail(SWAP_EINVAL, "cloud_r0 must be > 0");
  if (c->dims.nx - 2 > 0 && (long long)(c->dims.ny - 2) * (c->dims.nz - 2) * s->inflow_ppc > (1LL << 31))
    return c->fail(SWAP_EINVAL, "inflow slot count out of range");
  TRY(src_scratch(c, 0));
  CU(cudaMemsetAsync(c->src_cnt, 0, 4 * sizeof(unsigned long long), c->st));
  CU(cudaStreamSynchronize(c->st));
  c->srcs = *s;
  c->have_srcs = true;
  c->src_step = step0;
  return SWAP_OK;
}

extern "C" int swap_chex_count(swap_ctx* c, int64_t* count) {
  if (!c || !count) return SWAP_EINVAL;
  *count = 0;
  if (!c->src_cnt) return SWAP_OK;
  unsigned long long h = 0;
  CU(cudaMemcpyAsync(&h, c->src_cnt + 1, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  *count = (int64_t)h;
  return SWAP_OK;
}

static int need_srcs(swap_ctx* c) {
  if (!c->have_srcs) return c->fail(SWAP_EINVAL, "swap_set_sources has not been called");
  return touch_scalars(c);
}

extern "C" int swap_Ionize_sw_mp(swap_ctx* c, double* np, double* vp, double* vp1, double* xp, int32_t m_tstep,
                                 double* input_p, double* up) {
  (void)input_p;  // the reference's input-energy bookkeeping (chem_rates.f:611-617) is diagnostics only
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(need_srcs(c));
  double *dnp, *dvp, *dvp1, *dxp, *dup;
  TRY(c->use(xp, Access::InOut, &dxp));
  TRY(c->use(vp, Access::InOut, &dvp));
  TRY(c->use(vp1, Access::InOut, &dvp1));
  TRY(c->use(np, Access::Out, &dnp));
  TRY(c->use(up, Access::Out, &dup));
  TRY(src_ionize(c, dxp, dvp, dvp1, m_tstep));
  TRY(ops::get_interp_weights(c, dxp));  // chem_rates.f:641-643
  TRY(ops::update_np(c, dnp));
  TRY(ops::update_up_mode(c, 0, dvp, nullptr, nullptr, dnp, dup));
  return c->finish();
}

static int bound_particles(swap_ctx* c, double** dxp, double** dvp, double** dvp1) {
  if (!c->h_xp) return c->fail(SWAP_EINVAL, "swap_bind_particles has not been called");
  TRY(c->use(c->h_xp, Access::InOut, dxp));
  TRY(c->use(c->h_vp, Access::InOut, dvp));
  TRY(c->use(c->h_vp1, Access::InOut, dvp1));
  return SWAP_OK;
}

extern "C" int swap_inflow_x(swap_ctx* c, int32_t m_tstep) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(need_srcs(c));
  double *dxp, *dvp, *dvp1;
  TRY(bound_particles(c, &dxp, &dvp, &dvp1));
  TRY(src_inflow(c, dxp, dvp, dvp1, m_tstep));
  return c->finish();
}

extern "C" int swap_ionize_cloud(swap_ctx* c, int32_t m_tstep) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(need_srcs(c));
  double *dxp, *dvp, *dvp1;
  TRY(bound_particles(c, &dxp, &dvp, &dvp1));
  TRY(src_cloud(c, dxp, dvp, dvp1, m_tstep));
  return c->finish();
}

extern "C" int swap_remove_outflow_x(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(touch_scalars(c));
  double *dxp, *dvp, *dvp1;
  TRY(bound_particles(c, &dxp, &dvp, &dvp1));
  TRY(src_outflow(c, dxp, dvp, dvp1, true));
  return c->finish();
}

extern "C" int swap_remove_ion(swap_ctx* c, double* xp, double* vp, double* vp1, int32_t ion_l) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(touch_scalars(c));
  const long long N = c->ntot();
  if (ion_l < 1 || ion_l > N) return c->fail(SWAP_EINVAL, "remove_ion: index out of range");
  double *dxp, *dvp, *dvp1;
  TRY(c->use(xp, Access::InOut, &dxp));
  TRY(c->use(vp, Access::InOut, &dvp));
  TRY(c->use(vp1, Access::InOut, &dvp1));
  TRY(src_scratch(c, N));
  k_keep_all_but<<<nb(N), TPB, 0, c->st>>>(N, (long long)ion_l - 1, c->src_flag);
  CU(cudaGetLastError());
  TRY(compact_particles(c, dxp, dvp, dvp1, true));
  return c->finish();
}

extern "C" int swap_res_chex(swap_ctx* c, double* xp, double* vp, int32_t m_tstep, int64_t* count) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  TRY(need_srcs(c));
  double *dxp, *dvp, *dvp1;
  TRY(c->use(xp, Access::In, &dxp));
  TRY(c->use(vp, Access::InOut, &dvp));
  TRY(c->use(c->h_vp1, Access::InOut, &dvp1));
  TRY(src_chex(c, dxp, dvp, dvp1, m_tstep));
  unsigned long long h = 0;
  CU(cudaMemcpyAsync(&h, c->src_cnt, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  TRY(c->finish());
  if (count) *count = (int64_t)h;
  return SWAP_OK;
}
