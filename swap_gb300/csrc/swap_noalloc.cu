// swap_noalloc.cu -- swap_update_up_noalloc: the update_up moment deposit
// (gutsp.f:1649-1842) for callers that cannot allocate device memory.
//
// Who needs it: callers that cannot call cudaMalloc.  One is a host whose
// device memory belongs to another allocator -- for example a process in
// which a framework's caching allocator has already reserved the GPU's
// memory, so a direct cudaMalloc fails or fragments that pool.  Another is a
// caller driving its own asynchronous pipeline on several streams: cudaMalloc
// and cudaFree can synchronize the whole device, every stream of it, which
// such a caller cannot afford inside its time step.  (This entry waits only
// for the one stream it is given: it returns after that stream has finished
// its work, to read the out-of-grid flag.)  Neither caller can create a
// swap_ctx, because swap_init allocates the device mirrors and scratch.  This
// entry takes the caller's own device arrays for every input and output and
// keeps its one scratch array -- the grid coordinates and the per-node
// velocity sums -- in a file-scope __device__ array instead.
//
// Properties:
//  * scratch is static: every GPU that loads this library holds it
//    (SWAP_NOALLOC_SCRATCH_BYTES) until the process exits;
//  * no call can be captured in a CUDA graph: every call reads the flag back
//    and waits for its stream, which a capture does not allow;
//  * the first call on a device looks up the scratch address with
//    cudaGetSymbolAddress (no allocation) and keeps it for the process; do
//    not call the entry again on a device after cudaDeviceReset on it (the
//    module is loaded anew and the kept address is stale);
//  * all calls share the scratch, so calls that overlap on the GPU (two
//    streams, two threads) race; serialize them.  After an error the entry
//    waits for its stream before it returns, so no work of the failed call
//    is still running when the caller tries again;
//  * sizes beyond SWAP_NOALLOC_MAX_NODES nodes or SWAP_NOALLOC_MAX_AXIS
//    nodes on an axis are rejected with SWAP_ECAPACITY.
//
// The cell search, weights and fold are the FP64 drop-in's own
// (swap_dev.cuh), and the unit is compiled with --fmad=false like it, so the
// result equals swap_update_up up to the order of the atomic sums.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"
#include "swap_dev.cuh"

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

using swapk::Geo;

// Weights (gutsp.f:1414-1429) and the update_up deposit (gutsp.f:1676-1800)
// of one particle into S = sum v*w/volb at folded nodes.
__global__ void k_na_deposit(Geo g, const double* __restrict__ xp, const double* __restrict__ vp,
                             const double* __restrict__ beta_p, long long N, long long NM, double beta,
                             double* __restrict__ S, int* flag) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < N; l += (long long)gridDim.x * blockDim.x) {
    const double x = xp[l], y = xp[l + NM], z = xp[l + 2 * NM];
    const int i = swapk::cell_search(g.qx, g.nx, x, g.inv_dx);
    const int j = (int)floor(y / g.dy);
    const int k = swapk::cell_search(g.qz, g.nz, z, g.inv_dz);
    if (i < 1 || j < 1 || j >= g.ny || k < 1) {
      atomicCAS(flag, 0, SWAP_EDOMAIN);
      continue;
    }
    double w[8];
    swapk::weights8(g, i, j, k, x, y, z, w);
    long long tg[8];
    swapk::corner_targets(g, i, j, k, tg);
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

// ct(node) = S/np at the node's interior image (zero where np = 0), then the
// face average up_m = 0.5*(ct_m(node) + ct_m(node+e_m)) (gutsp.f:1825-1836)
// on the interior.
__device__ __forceinline__ double na_ct(const Geo& g, const double* S, const double* np, int i, int j, int k,
                                        int m) {
  const long long o = swapk::nidx(g, swapk::wrapn(i, g.nx), swapk::wrapn(j, g.ny), swapk::wrapn(k, g.nz));
  const double n = np[o];
  return n == 0.0 ? 0.0 : S[o + g.C * m] / n;
}

__global__ void k_na_up(Geo g, const double* __restrict__ S, const double* __restrict__ np,
                        double* __restrict__ up) {
  const long long n_int = swapk::n_interior(g);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n_int;
       t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    swapk::interior_ijk(g, t, i, j, k);
    const long long o = swapk::nidx(g, i, j, k);
    up[o] = 0.5 * (na_ct(g, S, np, i, j, k, 0) + na_ct(g, S, np, i + 1, j, k, 0));
    up[o + g.C] = 0.5 * (na_ct(g, S, np, i, j, k, 1) + na_ct(g, S, np, i, j + 1, k, 1));
    up[o + 2 * g.C] = 0.5 * (na_ct(g, S, np, i, j, k, 2) + na_ct(g, S, np, i, j, k + 1, 2));
  }
}

// periodic(up) (gutsp.f:1839, boundary.f:9-52): each ghost node copies its
// interior image.
__global__ void k_na_periodic(Geo g, double* __restrict__ b) {
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < g.C; o += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(o % g.nx) + 1;
    const int j = (int)((o / g.nx) % g.ny) + 1;
    const int k = (int)(o / ((long long)g.nx * g.ny)) + 1;
    const int wi = swapk::wrapn(i, g.nx), wj = swapk::wrapn(j, g.ny), wk = swapk::wrapn(k, g.nz);
    if (wi == i && wj == j && wk == k) continue;
    const long long s = swapk::nidx(g, wi, wj, wk);
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
  // geometry and clear the sums and the flag.  Once anything is queued, an
  // error waits for the stream before returning (see the file's notes).
  auto fail_after_enqueue = [st]() {
    cudaStreamSynchronize(st);
    return SWAP_ECUDA;
  };
  if (cudaMemcpyAsync(qx + 1, coords->qx, dims->nx * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(qy + 1, coords->qy, dims->ny * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(qz + 1, coords->qz, dims->nz * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemsetAsync(S, 0, 3 * C * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(flag, 0, sizeof(int), st) != cudaSuccess)
    return fail_after_enqueue();
  Geo g{};
  g.nx = dims->nx; g.ny = dims->ny; g.nz = dims->nz;
  g.C = C;
  g.qx = qx; g.qy = qy; g.qz = qz;
  g.dy = params->dy;
  g.inv_dx = 1.0 / (coords->qx[1] - coords->qx[0]);
  g.inv_dz = 1.0 / (coords->qz[1] - coords->qz[0]);
  if (ni_tot > 0) k_na_deposit<<<na_blocks(ni_tot), 256, 0, st>>>(g, xp, vp, beta_p, ni_tot, dims->ni_max,
                                                                    params->beta, S, flag);
  k_na_up<<<na_blocks(swapk::n_interior(g)), 256, 0, st>>>(g, S, np, up);
  k_na_periodic<<<na_blocks(C), 256, 0, st>>>(g, up);
  if (cudaGetLastError() != cudaSuccess) return fail_after_enqueue();
  int hflag = 0;
  if (cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return fail_after_enqueue();
  if (cudaStreamSynchronize(st) != cudaSuccess) return SWAP_ECUDA;
  return hflag ? SWAP_EDOMAIN : SWAP_OK;
}
