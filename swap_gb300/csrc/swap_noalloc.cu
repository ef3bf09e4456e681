// swap_noalloc.cu -- swap_update_up_noalloc: the update_up moment deposit
// (gutsp.f:1649-1842) for callers that cannot allocate device memory.
//
// Who needs it: callers that cannot call cudaMalloc.  One is a host whose
// device memory belongs to another allocator -- for example a process in
// which a framework's caching allocator has already reserved the GPU's
// memory, so a direct cudaMalloc fails or fragments that pool.  Another is a
// caller driving its own asynchronous pipeline: cudaMalloc and cudaFree can
// synchronize the device, which such a caller cannot afford inside its time
// step.  Neither can create a swap_ctx, because swap_init allocates the
// device mirrors and scratch.  This entry takes the caller's own device
// arrays for every input and output and keeps its one scratch array -- the
// per-node velocity sums -- in a file-scope __device__ array instead.
//
// Properties:
//  * scratch is static: every GPU that loads this library holds it
//    (SWAP_NOALLOC_SCRATCH_BYTES) until the process exits;
//  * the first call on a device looks up the scratch address with
//    cudaGetSymbolAddress (no allocation); make that first call before any
//    stream capture;
//  * all calls share the scratch, so calls that overlap on the GPU (two
//    streams, two threads) race; serialize them;
//  * sizes beyond SWAP_NOALLOC_MAX_NODES nodes or SWAP_NOALLOC_MAX_AXIS
//    nodes on an axis are rejected with SWAP_ECAPACITY.
//
// Compiled with --fmad=false like the FP64 drop-in, so the result equals
// swap_update_up up to the order of the atomic sums.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"

namespace {

constexpr long long kMaxNodes = SWAP_NOALLOC_MAX_NODES;
constexpr int kMaxAxis = SWAP_NOALLOC_MAX_AXIS;
constexpr long long kGeoLen = kMaxAxis + 1;  // 1-based node coordinates
// layout: qx | qy | qz (each kGeoLen, 1-based) | S (3 * kMaxNodes)
constexpr long long kScratchDoubles = 3 * kGeoLen + 3 * kMaxNodes;
static_assert(kScratchDoubles * 8 == SWAP_NOALLOC_SCRATCH_BYTES, "header size out of date");

static __device__ __align__(256) double g_scratch[kScratchDoubles];
static __device__ int g_flag;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {};
int* g_flag_addr[kMaxDevices] = {};

// Once per device, with that device current: resolve the device addresses
// of the static scratch and flag.  Host code may not use the symbols
// themselves as addresses (they are host-side stand-ins).
int setup(double** scratch, int** flag) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SWAP_ECUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* s = nullptr;
    void* f = nullptr;
    if (cudaGetSymbolAddress(&s, g_scratch) != cudaSuccess) return SWAP_ECUDA;
    if (cudaGetSymbolAddress(&f, g_flag) != cudaSuccess) return SWAP_ECUDA;
    g_scratch_addr[dev] = static_cast<double*>(s);
    g_flag_addr[dev] = static_cast<int*>(f);
  }
  *scratch = g_scratch_addr[dev];
  *flag = g_flag_addr[dev];
  return SWAP_OK;
}

struct NaGeo {
  int nx, ny, nz;
  long long C;
  const double *qx, *qy, *qz;  // 1-based, in the scratch
  double dy, inv_dx, inv_dz;
};

__device__ __forceinline__ long long na_idx(const NaGeo& g, int i, int j, int k) {
  return (long long)(i - 1) + (long long)g.nx * ((long long)(j - 1) + (long long)g.ny * (long long)(k - 1));
}

// q(i) < x <= q(i+1): the linear search of gutsp.f:1396-1401.
__device__ __forceinline__ int na_search(const double* q, int n, double x, double inv_d) {
  if (!(x > q[1]) || x > q[n]) return 0;
  int i = (int)((x - q[1]) * inv_d) + 1;
  i = i < 1 ? 1 : (i > n - 1 ? n - 1 : i);
  while (i > 1 && !(x > q[i])) --i;
  while (i < n - 1 && x > q[i + 1]) ++i;
  return i;
}

// Folded deposit target (gutsp.f:1803-1805 + periodic): plane 1 -> n-1,
// plane n dropped.
__device__ __forceinline__ long long na_fold(const NaGeo& g, int i, int j, int k) {
  if (i == g.nx || j == g.ny || k == g.nz) return -1;
  return na_idx(g, i == 1 ? g.nx - 1 : i, j == 1 ? g.ny - 1 : j, k == 1 ? g.nz - 1 : k);
}

// Weights (gutsp.f:1414-1429) and the update_up deposit (gutsp.f:1676-1800)
// of one particle into S = sum v*w/volb at folded nodes.
__global__ void k_na_deposit(NaGeo g, const double* __restrict__ xp, const double* __restrict__ vp,
                             const double* __restrict__ beta_p, long long N, long long NM, double beta,
                             double* __restrict__ S, int* flag) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const double x = xp[l], y = xp[l + NM], z = xp[l + 2 * NM];
    const int i = na_search(g.qx, g.nx, x, g.inv_dx);
    const int j = (int)floor(y / g.dy);
    const int k = na_search(g.qz, g.nz, z, g.inv_dz);
    if (i < 1 || j < 1 || j >= g.ny || k < 1) {
      atomicCAS(flag, 0, SWAP_EDOMAIN);
      continue;
    }
    const double vol = 1.0 / ((g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]));
    const double x1 = fabs(x - g.qx[i]), x2 = fabs(x - g.qx[i + 1]);
    const double y1 = fabs(y - g.qy[j]), y2 = fabs(y - g.qy[j + 1]);
    const double z1 = fabs(z - g.qz[k]), z2 = fabs(z - g.qz[k + 1]);
    double w[8];
    w[0] = x2 * y2 * z2 * vol;
    w[1] = x1 * y2 * z2 * vol;
    w[2] = x2 * y2 * z1 * vol;
    w[3] = x1 * y2 * z1 * vol;
    w[4] = x2 * y1 * z2 * vol;
    w[5] = x1 * y1 * z2 * vol;
    w[6] = x2 * y1 * z1 * vol;
    w[7] = x1 * y1 * z1 * vol;
    const long long tg[8] = {na_fold(g, i, j, k),         na_fold(g, i + 1, j, k),
                             na_fold(g, i, j, k + 1),     na_fold(g, i + 1, j, k + 1),
                             na_fold(g, i, j + 1, k),     na_fold(g, i + 1, j + 1, k),
                             na_fold(g, i, j + 1, k + 1), na_fold(g, i + 1, j + 1, k + 1)};
    const double volb =
        (g.qx[i + 1] - g.qx[i]) * (g.qy[j + 1] - g.qy[j]) * (g.qz[k + 1] - g.qz[k]) * beta * beta_p[l];
    const double ivolb = 1.0 / volb;
    const double v0 = vp[l], v1 = vp[l + NM], v2 = vp[l + 2 * NM];
    for (int c = 0; c < 8; ++c) {
      if (tg[c] < 0) continue;
      const double wc = w[c] * ivolb;
      atomicAdd(S + tg[c], v0 * wc);
      atomicAdd(S + tg[c] + g.C, v1 * wc);
      atomicAdd(S + tg[c] + 2 * g.C, v2 * wc);
    }
  }
}

__device__ __forceinline__ int na_wrap(int i, int n) { return i == 1 ? n - 1 : (i == n ? 2 : i); }

// ct(node) = S/np at the node's interior image (zero where np = 0), then the
// face average up_m = 0.5*(ct_m(node) + ct_m(node+e_m)) (gutsp.f:1825-1836)
// on the interior.
__device__ __forceinline__ double na_ct(const NaGeo& g, const double* S, const double* np, int i, int j, int k,
                                        int m) {
  const long long o = na_idx(g, na_wrap(i, g.nx), na_wrap(j, g.ny), na_wrap(k, g.nz));
  const double n = np[o];
  return n == 0.0 ? 0.0 : S[o + g.C * m] / n;
}

__global__ void k_na_up(NaGeo g, const double* __restrict__ S, const double* __restrict__ np,
                        double* __restrict__ up) {
  const long long ix = g.nx - 2, iy = g.ny - 2;
  const long long n_int = ix * iy * (g.nz - 2);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n_int;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % ix) + 2;
    const int j = (int)((t / ix) % iy) + 2;
    const int k = (int)(t / (ix * iy)) + 2;
    const long long o = na_idx(g, i, j, k);
    up[o] = 0.5 * (na_ct(g, S, np, i, j, k, 0) + na_ct(g, S, np, i + 1, j, k, 0));
    up[o + g.C] = 0.5 * (na_ct(g, S, np, i, j, k, 1) + na_ct(g, S, np, i, j + 1, k, 1));
    up[o + 2 * g.C] = 0.5 * (na_ct(g, S, np, i, j, k, 2) + na_ct(g, S, np, i, j, k + 1, 2));
  }
}

// periodic(up) (gutsp.f:1839, boundary.f:9-52): each ghost node copies its
// interior image.
__global__ void k_na_periodic(NaGeo g, double* __restrict__ b) {
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < g.C; o += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(o % g.nx) + 1;
    const int j = (int)((o / g.nx) % g.ny) + 1;
    const int k = (int)(o / ((long long)g.nx * g.ny)) + 1;
    const int wi = na_wrap(i, g.nx), wj = na_wrap(j, g.ny), wk = na_wrap(k, g.nz);
    if (wi == i && wj == j && wk == k) continue;
    const long long s = na_idx(g, wi, wj, wk);
    for (int m = 0; m < 3; ++m) b[o + g.C * m] = b[s + g.C * m];
  }
}

unsigned na_blocks(long long n) {
  const long long b = (n + 255) / 256;
  return (unsigned)(b < 1 ? 1 : (b > 1048576 ? 1048576 : b));
}

}  // namespace

extern "C" int swap_update_up_noalloc(const swap_dims* dims, const swap_params* params, const swap_coords* coords,
                                      const double* xp, const double* vp, const double* beta_p, int64_t ni_tot,
                                      const double* np, double* up, void* stream) {
  if (!dims || !params || !coords || !coords->qx || !coords->qy || !coords->qz || !np || !up) return SWAP_EINVAL;
  if (ni_tot < 0 || ni_tot > dims->ni_max || (ni_tot > 0 && (!xp || !vp || !beta_p))) return SWAP_EINVAL;
  if (dims->nx < 3 || dims->ny < 3 || dims->nz < 3) return SWAP_EINVAL;
  const long long C = (long long)dims->nx * dims->ny * dims->nz;
  if (dims->nx > kMaxAxis || dims->ny > kMaxAxis || dims->nz > kMaxAxis || C > kMaxNodes) return SWAP_ECAPACITY;
  double* scratch = nullptr;
  int* flag = nullptr;
  int r = setup(&scratch, &flag);
  if (r) return r;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* qx = scratch;
  double* qy = scratch + kGeoLen;
  double* qz = scratch + 2 * kGeoLen;
  double* S = scratch + 3 * kGeoLen;
  // The scratch keeps the previous call's contents: load this call's
  // geometry and clear the sums and the flag.
  if (cudaMemcpyAsync(qx + 1, coords->qx, dims->nx * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(qy + 1, coords->qy, dims->ny * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(qz + 1, coords->qz, dims->nz * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(S, 0, 3 * C * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess)
    return SWAP_ECUDA;
  NaGeo g;
  g.nx = dims->nx; g.ny = dims->ny; g.nz = dims->nz;
  g.C = C;
  g.qx = qx; g.qy = qy; g.qz = qz;
  g.dy = params->dy;
  g.inv_dx = 1.0 / (coords->qx[1] - coords->qx[0]);
  g.inv_dz = 1.0 / (coords->qz[1] - coords->qz[0]);
  if (ni_tot > 0) k_na_deposit<<<na_blocks(ni_tot), 256, 0, st>>>(g, xp, vp, beta_p, ni_tot, dims->ni_max,
                                                                    params->beta, S, flag);
  k_na_up<<<na_blocks((long long)(g.nx - 2) * (g.ny - 2) * (g.nz - 2)), 256, 0, st>>>(g, S, np, up);
  k_na_periodic<<<na_blocks(C), 256, 0, st>>>(g, up);
  if (cudaGetLastError() != cudaSuccess) return SWAP_ECUDA;
  int hflag = 0;
  if (cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return SWAP_ECUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return SWAP_ECUDA;
  return hflag ? SWAP_EDOMAIN : SWAP_OK;
}
