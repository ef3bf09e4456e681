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
#include "swap_dev.cuh"
#include "philox.h"
#include "sources_dev.cuh"
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

// Ionize_sw_mp's new ions (chem_rates.f:567-620), appended after N.
__global__ void k_ionize(Geo g, PView p, long long N, long long n, swap_sources s, long long step) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    double st[6];
    swapsrc::ionize_state(g, s, step, q, st);
    const long long l = N + q, NM = p.NM;
    for (int m = 0; m < 3; ++m) {
      p.xp[l + m * NM] = st[m];
      p.vp[l + m * NM] = st[3 + m];
      p.vp1[l + m * NM] = st[3 + m];
    }
    p.mrat[l] = s.mrat_pu;
    p.beta_p[l] = s.beta_pu;
  }
}

__global__ void k_inflow_flags(Geo g, swap_sources s, long long step, double dt, int64_t* flag) {
  const long long ncy = g.ny - 2, ncz = g.nz - 2, ppc = s.inflow_ppc;
  const long long nslot = (long long)ncy * ncz * ppc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslot; t += (long long)gridDim.x * blockDim.x) {
    flag[t] = swapsrc::inflow_enters(g, s, step, t, dt) ? 1 : 0;
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
    swapsrc::inflow_candidate(g, s, step, t, cj, ck, dt, st);
    const long long l = N + pos[t];
    for (int m = 0; m < 3; ++m) {
      p.xp[l + m * NM] = st[m];
      p.vp[l + m * NM] = st[3 + m];
      p.vp1[l + m * NM] = st[3 + m];
    }
    p.mrat[l] = 1.0;
    p.beta_p[l] = 1.0;
  }
}

// Cloud ionization: per-cell counts (the oracle's cell order, x fastest).
__global__ void k_cloud_count(Geo g, swap_sources s, long long step, double dt, double beta, int64_t* cnt) {
  const int ncx = g.nx - 2, ncy = g.ny - 2, ncz = g.nz - 2;
  const long long ncell = (long long)ncx * ncy * ncz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c % ncx), cj = (int)((c / ncx) % ncy), ck = (int)(c / ((long long)ncx * ncy));
    cnt[c] = swapsrc::cloud_count(g, s, step, dt, beta, ci, cj, ck, c);
  }
}

// New heavy ions at rest, uniform in their cell (mrat_heavy, beta_heavy).
__global__ void k_cloud_write(Geo g, PView p, swap_sources s, long long step, const int64_t* cnt, const int64_t* pos,
                              long long N) {
  const int ncx = g.nx - 2, ncy = g.ny - 2, ncz = g.nz - 2;
  const long long ncell = (long long)ncx * ncy * ncz, NM = p.NM;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(c % ncx), cj = (int)((c / ncx) % ncy), ck = (int)(c / ((long long)ncx * ncy));
    for (long long q = 0; q < cnt[c]; ++q) {
      double x[3];
      swapsrc::cloud_position(g, s, step, ci, cj, ck, c, q, x);
      const long long l = N + pos[c] + q;
      for (int m = 0; m < 3; ++m) {
        p.xp[l + m * NM] = x[m];
        p.vp[l + m * NM] = 0.0;
        p.vp1[l + m * NM] = 0.0;
      }
      p.mrat[l] = s.mrat_heavy;
      p.beta_p[l] = s.beta_heavy;
    }
  }
}

// Charge exchange after res_chex (chem_rates.f:823-840): the new ion is heavy
// and at rest; ions already heavy are skipped.
__global__ void k_chex(PView p, long long N, swap_sources s, long long step, double dt, unsigned long long* count) {
  const long long NM = p.NM;
  unsigned long long mine = 0;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    if (p.mrat[l] == s.mrat_heavy) continue;
    if (swapsrc::chex_trial(s, step, l, dt, p.xp[l], p.xp[l + NM], p.xp[l + 2 * NM], p.vp[l], p.vp[l + NM],
                            p.vp[l + 2 * NM])) {
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

// ---- the FP32 form: new ions staged for the sort ----

using swapk32::G32;
using swapk32::key_of;
using swapk32::offset_in_cell;
using swapk32::pk;

__device__ __forceinline__ void stage_one(swapk32::Part& st, long long q, int ci, int cj, int ck, float ox, float oy,
                                          float oz, const double v[3], uint8_t sp) {
  st.cell[q] = pk(ci, cj, ck);
  st.ox[q] = ox; st.oy[q] = oy; st.oz[q] = oz;
  st.vx[q] = (float)v[0]; st.vy[q] = (float)v[1]; st.vz[q] = (float)v[2];
  st.wx[q] = (float)v[0]; st.wy[q] = (float)v[1]; st.wz[q] = (float)v[2];
  st.sp[q] = sp;
}

// Ring ions anywhere in the box: state and key; ranks follow sequentially.
__global__ void k32_stage_ionize(Geo g64, G32 g, swap_sources s, long long step, long long n, swapk32::Part st,
                                 int32_t* key, uint8_t sp, int* err) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    double x[6];
    swapsrc::ionize_state(g64, s, step, q, x);
    int ci = 0, cj = 0, ck = 0;
    float ox = 0.5f, oy = 0.5f, oz = 0.5f;
    const bool ok = swapk32::split_axis(x[0], g.qx1, g.dx, g.ncx, true, ci, ox) &&
                    swapk32::split_axis(x[1], g.qy1, g.dy, g.ncy, false, cj, oy) &&
                    swapk32::split_axis(x[2], g.qz1, g.dz, g.ncz, true, ck, oz);
    if (!ok) atomicCAS(err, 0, KERR_DOMAIN);
    stage_one(st, q, ci, cj, ck, ox, oy, oz, x + 3, sp);
    key[q] = (int32_t)key_of(g, ci, cj, ck);
  }
}

// Ranks of n staged ions among the new ions of their key, in staging order.
__global__ void k32_rank_seq(long long n, const int32_t* key, int32_t* rank, int32_t* ncount) {
  for (long long q = 0; q < n; ++q) rank[q] = ncount[key[q]]++;
}

// Cloud ions of cell c (the restatement's cell order), staged at base+pos[c].
__global__ void k32_stage_cloud(Geo g64, G32 g, swap_sources s, long long step, const int64_t* cnt,
                                const int64_t* pos, long long base, swapk32::Part st, int32_t* key, int32_t* rank,
                                int32_t* ncount, uint8_t sp) {
  const long long ncell = (long long)g.ncx * g.ncy * g.ncz;
  const double zero[3] = {0.0, 0.0, 0.0};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const long long n = cnt[c];
    if (n == 0) continue;
    const int ci = (int)(c % g.ncx), cj = (int)((c / g.ncx) % g.ncy), ck = (int)(c / ((long long)g.ncx * g.ncy));
    const int32_t X = (int32_t)key_of(g, ci, cj, ck);
    const int32_t r0 = ncount[X];
    for (long long q = 0; q < n; ++q) {
      double x[3];
      swapsrc::cloud_position(g64, s, step, ci, cj, ck, c, q, x);
      const long long o = base + pos[c] + q;
      stage_one(st, o, ci, cj, ck, offset_in_cell(x[0], g.qx1, g.dx, ci, true),
                offset_in_cell(x[1], g.qy1, g.dy, cj, false), offset_in_cell(x[2], g.qz1, g.dz, ck, true), zero, sp);
      key[o] = X;
      rank[o] = r0 + (int32_t)q;
    }
    ncount[X] = r0 + (int32_t)n;
  }
}

// Inflow ions: slot t of face cell f = t / ppc enters physical cell
// (0, cj, ck); staged at base+pos[t]; its rank among the key's new ions
// follows the ones staged before (ncount) and the earlier slots of its face.
__global__ void k32_stage_inflow(Geo g64, G32 g, swap_sources s, long long step, double dt, const int64_t* flag,
                                 const int64_t* pos, long long base, swapk32::Part st, int32_t* key, int32_t* rank,
                                 const int32_t* ncount, uint8_t sp, int* err) {
  const int ppc = s.inflow_ppc;
  const long long nslot = (long long)g.ncy * g.ncz * ppc;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nslot; t += (long long)gridDim.x * blockDim.x) {
    if (!flag[t]) continue;
    const long long f = t / ppc;
    const int cj = (int)(f % g.ncy), ck = (int)(f / g.ncy);
    const int32_t X = (int32_t)key_of(g, 0, cj, ck);
    double x[6];
    swapsrc::inflow_candidate(g64, s, step, t, cj, ck, dt, x);
    if ((x[0] - g.qx1) / g.dx > 1.0) atomicCAS(err, 0, KERR_MOVE);  // entered past the first cell
    const long long o = base + pos[t];
    stage_one(st, o, 0, cj, ck, offset_in_cell(x[0], g.qx1, g.dx, 0, true),
              offset_in_cell(x[1], g.qy1, g.dy, cj, false), offset_in_cell(x[2], g.qz1, g.dz, ck, true), x + 3, sp);
    key[o] = X;
    rank[o] = ncount[X] + (int32_t)(pos[t] - pos[f * ppc]);
  }
}

// After k32_stage_inflow: the inflow ions of each face cell join the count
// of its key.
__global__ void k32_count_inflow(G32 g, int ppc, const int64_t* pos, int32_t* ncount) {
  const long long nface = (long long)g.ncy * g.ncz;
  for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nface; f += (long long)gridDim.x * blockDim.x) {
    const int cj = (int)(f % g.ncy), ck = (int)(f / g.ncy);
    ncount[key_of(g, 0, cj, ck)] += (int32_t)(pos[(f + 1) * ppc] - pos[f * ppc]);
  }
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

unsigned long long* counters(swap_ctx* c) {
  return src_scratch(c, 0) == SWAP_OK ? c->src_cnt : nullptr;
}

bool any_rule(const swap_ctx* c) {
  const swap_sources& s = c->srcs;
  return c->have_srcs && (s.ndot > 0 || s.x_open || s.nu_ion > 0 || s.cx_a > 0);
}

void stage_free(F32Stage& st) {
  swapk32::Part& p = st.part;
  for (void* q : {(void*)p.cell, (void*)p.ox, (void*)p.oy, (void*)p.oz, (void*)p.vx, (void*)p.vy, (void*)p.vz,
                  (void*)p.wx, (void*)p.wy, (void*)p.wz, (void*)p.sp, (void*)st.key, (void*)st.rank, (void*)st.ncount})
    if (q) cudaFree(q);
  st.part = swapk32::Part{};
  st.key = st.rank = st.ncount = nullptr;
  st.cap = st.nkeys = 0;
}

static int stage_reserve(swap_ctx* c, F32Stage& st, long long need, long long nkeys) {
  if (!st.ncount || st.nkeys != nkeys) {
    if (st.ncount) cudaFree(st.ncount);
    st.ncount = nullptr;
    if (cudaMalloc(&st.ncount, (std::size_t)nkeys * sizeof(int32_t)) != cudaSuccess)
      return c->fail(SWAP_ECUDA, "allocation of the new-ion counts failed");
    st.nkeys = nkeys;
  }
  if (need <= st.cap) return SWAP_OK;
  CU(cudaStreamSynchronize(c->st));
  int32_t* nc = st.ncount;
  const long long nk = st.nkeys;
  st.ncount = nullptr;
  stage_free(st);
  st.ncount = nc;
  st.nkeys = nk;
  const long long cap = need + need / 4 + 1024;
  swapk32::Part& p = st.part;
  void** f4[] = {(void**)&p.ox, (void**)&p.oy, (void**)&p.oz, (void**)&p.vx, (void**)&p.vy, (void**)&p.vz,
                 (void**)&p.wx, (void**)&p.wy, (void**)&p.wz, (void**)&p.cell, (void**)&st.key, (void**)&st.rank};
  for (void** a : f4)
    if (cudaMalloc(a, (std::size_t)cap * 4) != cudaSuccess) return c->fail(SWAP_ECUDA, "staging allocation failed");
  if (cudaMalloc((void**)&p.sp, (std::size_t)cap) != cudaSuccess) return c->fail(SWAP_ECUDA, "staging allocation failed");
  st.cap = cap;
  return SWAP_OK;
}

int f32_stage(swap_ctx* c, const swapk32::G32& g, F32Stage& st, long long m, long long* n_host,
              const int64_t** n_dev, long long* n_max) {
  *n_host = 0;
  *n_dev = nullptr;
  *n_max = 0;
  const swap_sources& s = c->srcs;
  if (!any_rule(c)) return SWAP_OK;
  const long long n_ion = s.ndot > 0 ? ionize_count(c, m) : 0;
  const long long ncell = (long long)g.ncx * g.ncy * g.ncz;
  const long long nslot = s.x_open ? (long long)g.ncy * g.ncz * s.inflow_ppc : 0;
  long long n_cloud = 0;
  if (s.nu_ion > 0) {
    TRY(src_scratch(c, ncell));
    {
      ProfScope ps(c, "f32_src_cloud_count", c->st);
      k_cloud_count<<<nb(ncell), TPB, 0, c->st>>>(c->g, s, m, c->prm.dt, c->prm.beta, c->src_flag);
    }
    CU(cudaGetLastError());
    {
      ProfScope ps(c, "f32_src_cloud_scan", c->st, 3);
      TRY(scan_count(c, ncell, &n_cloud));
    }
  }
  TRY(stage_reserve(c, st, n_ion + n_cloud + nslot, g.nkeys));
  CU(cudaMemsetAsync(st.ncount, 0, (std::size_t)g.nkeys * sizeof(int32_t), c->st));
  if (n_ion > 0) {
    ProfScope ps(c, "f32_src_ionize", c->st, 2);
    k32_stage_ionize<<<nb(n_ion), TPB, 0, c->st>>>(c->g, g, s, m, n_ion, st.part, st.key, st.sp_ion, c->d_err);
    k32_rank_seq<<<1, 1, 0, c->st>>>(n_ion, st.key, st.rank, st.ncount);
  }
  CU(cudaGetLastError());
  if (n_cloud > 0) {
    ProfScope ps(c, "f32_src_cloud", c->st);
    k32_stage_cloud<<<nb(ncell), TPB, 0, c->st>>>(c->g, g, s, m, c->src_flag, c->src_pos, n_ion, st.part, st.key,
                                                  st.rank, st.ncount, st.sp_cloud);
  }
  CU(cudaGetLastError());
  if (nslot > 0) {
    TRY(src_scratch(c, nslot));
    {
      ProfScope ps(c, "f32_src_inflow", c->st, 6);  // flags, the scan's 3, stage, count
      k_inflow_flags<<<nb(nslot), TPB, 0, c->st>>>(c->g, s, m, c->prm.dt, c->src_flag);
      CU(cudaGetLastError());
      CU(swapk32::scan_exclusive(c->src_flag, c->src_pos, nslot, c->src_sums, c->st));
      k32_stage_inflow<<<nb(nslot), TPB, 0, c->st>>>(c->g, g, s, m, c->prm.dt, c->src_flag, c->src_pos,
                                                     n_ion + n_cloud, st.part, st.key, st.rank, st.ncount,
                                                     st.sp_inflow, c->d_err);
      CU(cudaGetLastError());
      const long long nface = (long long)g.ncy * g.ncz;
      k32_count_inflow<<<nb(nface), TPB, 0, c->st>>>(g, s.inflow_ppc, c->src_pos, st.ncount);
    }
    CU(cudaGetLastError());
    *n_dev = c->src_pos + nslot;
  }
  *n_host = n_ion + n_cloud;
  *n_max = n_ion + n_cloud + nslot;
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
