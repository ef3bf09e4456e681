// swap_abi.cu -- the extern "C" drop-in (include/swap_gpu.h): context,
// registry of the caller's host arrays with device mirrors, and one entry per
// reference subroutine built from the FP64 kernels in k64.cu.
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/swap_gpu.h"
#include "k64.cuh"
#include "swap_ctx.h"
#include "swap_ops.h"
#include "swap_prof.h"

using namespace swapk;

// ---------------------------------------------------------------------------
// context helpers
// ---------------------------------------------------------------------------

int swap_ctx::fail(int code, const std::string& msg) {
  err = msg;
  return code;
}

int swap_ctx::cuda_fail(cudaError_t e, const char* where) {
  err = std::string(where) + ": " + cudaGetErrorString(e);
  return SWAP_ECUDA;
}

double* swap_ctx::dalloc(std::size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
  owned.push_back(p);
  return static_cast<double*>(p);
}

Mirror* swap_ctx::find(const void* host) {
  auto it = reg.find(host);
  return it == reg.end() ? nullptr : &it->second;
}

int swap_ctx::add_mirror(void* host, std::size_t bytes, MirrorKind kind, bool real) {
  if (!host) return SWAP_OK;  // optional array not supplied
  if (Mirror* m = find(host)) {
    if (m->bytes != bytes || m->kind != kind) return fail(SWAP_EINVAL, "array registered twice with another size");
    return SWAP_OK;
  }
  Mirror m;
  m.host = host;
  m.bytes = bytes;
  m.kind = kind;
  m.host_f32 = real && real_bytes == 4;
  if (cudaMalloc(&m.dev, bytes) != cudaSuccess) return fail(SWAP_ECUDA, "device allocation of a mirror failed");
  if (bytes && cudaMemsetAsync(m.dev, 0, bytes, st) != cudaSuccess) {  // (ni_max = 0: no memory to clear)
    cudaFree(m.dev);
    return fail(SWAP_ECUDA, "clearing a mirror failed");
  }
  m.host_valid = true;
  m.dev_valid = false;
  reg.emplace(host, m);
  return SWAP_OK;
}

long long swap_ctx::ntot() const { return ni_tot_ptr ? (long long)*ni_tot_ptr : 0; }

// One segment of a 4-byte-real mirror: n floats at host element `off`
// through the staging buffer, converted to or from the device's doubles.
static cudaError_t convert_segment(swap_ctx* c, Mirror& m, std::size_t off, std::size_t n, bool to_dev) {
  if (n == 0) return cudaSuccess;
  if (c->stage32_n < n) {
    if (c->stage32) cudaFree(c->stage32);
    c->stage32 = nullptr;
    c->stage32_n = 0;
    cudaError_t e = cudaMalloc(&c->stage32, n * sizeof(float));
    if (e != cudaSuccess) return e;
    c->stage32_n = n;
  }
  float* h = static_cast<float*>(m.host) + off;
  double* d = static_cast<double*>(m.dev) + off;
  cudaError_t e;
  if (to_dev) {
    e = cudaMemcpyAsync(c->stage32, h, n * sizeof(float), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = swapk::widen_f32(c->stage32, d, (long long)n, c->st);
  } else {
    e = swapk::narrow_f64(d, c->stage32, (long long)n, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, c->stage32, n * sizeof(float), cudaMemcpyDeviceToHost, c->st);
  }
  return e;
}

// Copy the live part of a mirror: particle vectors move three ni_tot segments,
// per-particle scalars one, grids everything.
int swap_ctx::transfer(Mirror& m, bool to_dev) {
  const cudaMemcpyKind kind = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  char* d = static_cast<char*>(m.dev);
  char* h = static_cast<char*>(m.host);
  cudaError_t e = cudaSuccess;
  if (m.host_f32) {
    const bool part = m.kind == MirrorKind::Particle3 || m.kind == MirrorKind::Particle1;
    const std::size_t N = part ? (std::size_t)std::max(0LL, ntot()) : m.bytes / sizeof(double);
    const int ncomp = m.kind == MirrorKind::Particle3 ? 3 : 1;
    for (int q = 0; q < ncomp && e == cudaSuccess; ++q)
      e = convert_segment(this, m, part ? (std::size_t)q * (std::size_t)dims.ni_max : 0, N, to_dev);
    if (e != cudaSuccess) return cuda_fail(e, "transfer (4-byte reals)");
    (to_dev ? h2d_bytes : d2h_bytes) += (long long)(N * ncomp * sizeof(float));
    if (to_dev) m.dev_valid = true;
    else m.host_valid = true;
    return SWAP_OK;
  }
  if (m.kind == MirrorKind::Particle3 || m.kind == MirrorKind::Particle1 || m.kind == MirrorKind::ParticleI3) {
    const long long N = ntot();
    const std::size_t esz = m.kind == MirrorKind::ParticleI3 ? sizeof(int32_t) : sizeof(double);
    const int ncomp = m.kind == MirrorKind::Particle1 ? 1 : 3;
    for (int c = 0; c < ncomp && e == cudaSuccess; ++c) {
      const std::size_t off = (std::size_t)c * (std::size_t)dims.ni_max * esz;
      if (N > 0)
        e = to_dev ? cudaMemcpyAsync(d + off, h + off, (std::size_t)N * esz, kind, st)
                   : cudaMemcpyAsync(h + off, d + off, (std::size_t)N * esz, kind, st);
    }
  } else {
    e = to_dev ? cudaMemcpyAsync(d, h, m.bytes, kind, st) : cudaMemcpyAsync(h, d, m.bytes, kind, st);
  }
  if (e != cudaSuccess) return cuda_fail(e, "transfer");
  const long long moved = (m.kind == MirrorKind::Grid) ? (long long)m.bytes
                          : ntot() * (m.kind == MirrorKind::ParticleI3 ? 12 : m.kind == MirrorKind::Particle1 ? 8 : 24);
  (to_dev ? h2d_bytes : d2h_bytes) += moved;
  if (to_dev) m.dev_valid = true;
  else m.host_valid = true;
  return SWAP_OK;
}

// Resolve a host address handed to an entry to its device mirror; inputs are
// uploaded when the device copy is stale.
int swap_ctx::use(const void* host, Access acc, double** dev) {
  if (!host) return fail(SWAP_EINVAL, "null array argument");
  Mirror* m = find(host);
  if (!m) return fail(SWAP_EINVAL, "array not registered with swap_bind_*");
  if ((acc == Access::In || acc == Access::InOut) && !m->dev_valid) {
    int r = transfer(*m, true);
    if (r) return r;
  }
  if (acc == Access::Out || acc == Access::InOut) touched.push_back(m);
  *dev = static_cast<double*>(m->dev);
  return SWAP_OK;
}

int swap_ctx::use_host(const void* host, Access acc, double** ptr, bool* direct) {
  *direct = false;
  if (!host_direct || acc == Access::InOut || real_bytes != 8) return use(host, acc, ptr);
  if (!host) return fail(SWAP_EINVAL, "null array argument");
  Mirror* m = find(host);
  if (!m) return fail(SWAP_EINVAL, "array not registered with swap_bind_*");
  if (acc == Access::In && m->dev_valid) return use(host, acc, ptr);  // the device copy is current
  if (acc == Access::Out) touched_host.push_back(m);
  *ptr = static_cast<double*>(m->host);
  *direct = true;
  return SWAP_OK;
}

int swap_ctx::begin() {
  touched.clear();
  touched_host.clear();
  err.clear();
  const long long N = ntot();
  if (N < 0 || N > dims.ni_max) return fail(SWAP_ECAPACITY, "Ni_tot exceeds Ni_max");
  return SWAP_OK;
}

// Finish an entry: wait for the stream, read the kernel error flag, and mark
// every output device-current.
int swap_ctx::finish() {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "stream");
  for (Mirror* m : touched) {
    m->dev_valid = true;
    m->host_valid = false;
  }
  touched.clear();
  for (Mirror* m : touched_host) {
    m->host_valid = true;
    m->dev_valid = false;
  }
  touched_host.clear();
  int herr = 0;
  e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "error flag");
  if (herr) {
    cudaMemset(d_err, 0, sizeof(int));
    if (herr == KERR_DOMAIN) return fail(SWAP_EDOMAIN, "a particle lies outside the grid");
    if (herr == KERR_MOVE) return fail(SWAP_EMOVE, "a particle moved more than one cell in one step");
    if (herr == KERR_WAIT) return fail(SWAP_EWAIT, "a device wait reached its iteration limit");
    if (herr == KERR_RANGE)
      return fail(SWAP_ENONFINITE, "a deposited value is not finite or beyond the deterministic sums' range (2^25)");
    return fail(SWAP_ECUDA, "device error flag " + std::to_string(herr));
  }
  return SWAP_OK;
}

int swap_ctx::exchange(void* data, long long count, int kind) {
  if (!xfn) return SWAP_OK;
  const int r = xfn(xuser, data, (int64_t)count, (int32_t)kind, static_cast<void*>(st));
  if (r) return fail(SWAP_EEXCHANGE, "the exchange callback returned " + std::to_string(r));
  return SWAP_OK;
}

PartDev swap_ctx::part_view() {
  PartDev p;
  p.xp = p.vp = p.vp1 = nullptr;
  p.mrat = d_mrat;
  p.beta_p = d_beta_p;
  p.ijk = d_ijk;
  p.wght = d_wght;
  p.NM = dims.ni_max;
  return p;
}

#define TRY(x)                \
  do {                        \
    int _r = (x);             \
    if (_r) return _r;        \
  } while (0)
#define KL(name, x)                        \
  do {                                     \
    ProfScope _ps(c, name, c->st);         \
    cudaError_t _e = (x);                  \
    if (_e != cudaSuccess) return c->cuda_fail(_e, name); \
  } while (0)
#define CU(x)                                          \
  do {                                                 \
    cudaError_t _e = (x);                              \
    if (_e != cudaSuccess) return c->cuda_fail(_e, #x); \
  } while (0)

// ---------------------------------------------------------------------------
// device-side operators shared by the per-subroutine entries and the fused
// step; all arguments are device pointers.
// ---------------------------------------------------------------------------
namespace ops {

int periodic(swap_ctx* c, double* b) {
  KL("periodic", periodic3(c->g, b, c->st));
  return 0;
}

// face_to_center (grid_interp.f:136-176)
int face_to_center(swap_ctx* c, double* v, double* vc) {
  KL("periodic", periodic3(c->g, v, c->st));
  KL("face_to_center_int", face_to_center_int(c->g, v, vc, c->st));
  KL("periodic", periodic3(c->g, vc, c->st));
  return 0;
}

// edge_to_center (grid_interp.f:10-62)
int edge_to_center(swap_ctx* c, double* bt, double* btc) {
  KL("periodic", periodic3(c->g, bt, c->st));
  KL("edge_to_center_int", edge_to_center_int(c->g, bt, btc, c->st));
  KL("periodic", periodic3(c->g, btc, c->st));
  return 0;
}

// edge_to_face (grid_interp.f:67-130): interior faces; ghosts of btmf are
// left for the consumer's periodic() (face_to_center) as in the reference.
int edge_to_face(swap_ctx* c, double* bt, double* btmf) {
  KL("periodic", periodic3(c->g, bt, c->st));
  KL("edge_to_center_int", edge_to_center_int(c->g, bt, c->s_btc2, c->st));
  KL("periodic", periodic3(c->g, c->s_btc2, c->st));
  KL("face_avg_int", face_avg_int(c->g, c->s_btc2, btmf, c->st));
  return 0;
}

// crossf2 (gutsf.f:40-104); aa and btc arrive periodic from their producers.
int crossf2(swap_ctx* c, double* aa, double* btc, double* cc) {
  KL("cross_int", cross_int(c->g, aa, btc, c->s_ct, c->st));
  KL("periodic", periodic3(c->g, c->s_ct, c->st));
  KL("face_avg_int", face_avg_int(c->g, c->s_ct, cc, c->st));
  KL("periodic", periodic3(c->g, cc, c->st));
  return 0;
}

// curlB (gutsf.f:178-244)
int curlB(swap_ctx* c, double* bt, const double* np, double* aj) {
  KL("periodic", periodic3(c->g, bt, c->st));
  KL("curlB_int", curlB_int(c->g, bt, np, aj, c->prm.alpha, c->st));
  return 0;
}

// E = crossf2(face_to_center(aj-up), btc) + nu*aj; periodic(E)
int e_tail(swap_ctx* c, double* E, const double* aj, const double* np, const double* nu) {
  TRY(crossf2(c, c->s_aa, c->s_btcl, c->s_c));
  KL("e_from_c_int", e_from_c_int(c->g, c->s_c, nu, aj, np, c->prm.grad_pe, E, c->st));
  KL("periodic", periodic3(c->g, E, c->st));
  return 0;
}

// get_E (gutsf.f:994-1110)
int get_E(swap_ctx* c, double* E, double* bt, double* aj, const double* up, const double* np, const double* nu) {
  KL("sub_int", sub_int(c->g, aj, up, c->s_a, c->st));
  TRY(face_to_center(c, c->s_a, c->s_aa));
  TRY(edge_to_center(c, bt, c->s_btcl));
  return e_tail(c, E, aj, np, nu);
}

// predict_B (gutsf.f:1115-1169)
int predict_B(swap_ctx* c, double* b12, double* b1p2, double* bt, double* E, double* aj, double* up, double* np,
              double* nu, double dtsub) {
  TRY(get_E(c, E, bt, aj, up, np, nu));
  KL("curlE_update_int", curlE_update_int(c->g, E, b12, 2.0 * dtsub, b1p2, c->st));
  KL("periodic", periodic3(c->g, b1p2, c->st));
  return 0;
}

// get_Ep1 (gutsf.f:1174-1304) + correct_B (gutsf.f:1309-1359)
int correct_B(swap_ctx* c, double* b1, double* b1p2, double* E, double* aj, double* up, double* np, double* nu,
              double dtsub) {
  double* btp1 = c->s_btp1;
  KL("half_sum_all", half_sum_all(c->g, b1p2, b1, btp1, c->st));
  TRY(curlB(c, btp1, np, aj));
  KL("sub_int", sub_int(c->g, aj, up, c->s_a, c->st));
  TRY(face_to_center(c, c->s_a, c->s_aa));
  TRY(edge_to_face(c, btp1, c->s_btmf));
  TRY(face_to_center(c, c->s_btmf, c->s_btcl));
  TRY(e_tail(c, E, aj, np, nu));
  KL("curlE_update_int", curlE_update_int(c->g, E, b1, dtsub, b1p2, c->st));
  KL("periodic", periodic3(c->g, b1p2, c->st));
  return 0;
}

// f_update_tlev (gutsf.f:10-35)
int f_update_tlev(swap_ctx* c, double* b1, double* b12, double* b1p2, double* bt) {
  const std::size_t bytes = 3 * (std::size_t)c->g.C * sizeof(double);
  KL("cudaMemcpyAsync", cudaMemcpyAsync(bt, b1p2, bytes, cudaMemcpyDeviceToDevice, c->st));
  KL("cudaMemcpyAsync", cudaMemcpyAsync(b12, b1, bytes, cudaMemcpyDeviceToDevice, c->st));
  KL("cudaMemcpyAsync", cudaMemcpyAsync(b1, b1p2, bytes, cudaMemcpyDeviceToDevice, c->st));
  return 0;
}

// check_time_step (gutsf.f:1776-1822).  The per-node Courant times are
// formed on the device; when even the smallest leaves the current dtsub
// alone (the normal case) nothing changes.  Otherwise the reference's
// ordered, per-node halving is replayed on the host from the node values.
int check_time_step(swap_ctx* c, const double* bt, const double* np, double* dtsub, double* ntf) {
  KL("deltat_all", deltat_all(c->g, bt, np, c->prm.alpha, c->prm.dx, c->s_dtn, c->st));
  KL("reduce_min", reduce_min(c->s_dtn, c->g.C, c->s_red, 0, c->st));
  double mn = 0;
  KL("cudaMemcpyAsync", cudaMemcpyAsync(&mn, c->s_red, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  if (mn > 2.0 * *dtsub) return 0;
  std::vector<double> dtn((std::size_t)c->g.C);
  CU(cudaMemcpy(dtn.data(), c->s_dtn, dtn.size() * sizeof(double), cudaMemcpyDeviceToHost));
  const Geo& g = c->g;
  for (int i = 1; i <= g.nx; ++i)
    for (int j = 1; j <= g.ny; ++j)
      for (int k = 1; k <= g.nz; ++k) {
        if (dtn[(std::size_t)nidx(g, i, j, k)] <= 2.0 * *dtsub) {
          *dtsub = *dtsub / 2.0;
          *ntf = *ntf * 2.0;
        }
      }
  if (*ntf > 1.0e6) return c->fail(SWAP_ESUBCYCLE, "subcycle count overflow in check_time_step");
  return 0;
}

// get_interp_weights (gutsp.f:1378-1435)
int get_interp_weights(swap_ctx* c, const double* xp) {
  PartDev p = c->part_view();
  p.xp = const_cast<double*>(xp);
  KL("interp_weights", interp_weights(c->g, p, c->ntot(), c->d_err, c->st));
  c->weights_valid = true;
  c->weights_n = c->ntot();
  return 0;
}

// The device ijk/wght cover the particles get_interp_weights saw; a larger
// Ni_tot since then would address cells never computed.
int need_weights(swap_ctx* c) {
  if (!c->weights_valid) return c->fail(SWAP_EINVAL, "get_interp_weights has not been called");
  if (c->ntot() > c->weights_n) return c->fail(SWAP_EINVAL, "Ni_tot grew since get_interp_weights");
  return 0;
}

// update_np (gutsp.f:1441-1512)
// The fixed-point sums of the deterministic deposits, n values, zeroed.
static int fix_sums(swap_ctx* c, long long n, swapk::Fix64* f) {
  if (!c->fix.h) {
    void *h = nullptr, *l = nullptr;
    const std::size_t b = 3 * (std::size_t)c->g.C * 8;
    if (cudaMalloc(&h, b) != cudaSuccess) return c->fail(SWAP_ECUDA, "deterministic deposit sums");
    c->owned.push_back(h);
    if (cudaMalloc(&l, b) != cudaSuccess) return c->fail(SWAP_ECUDA, "deterministic deposit sums");
    c->owned.push_back(l);
    c->fix = swapk::Fix64{static_cast<long long*>(h), static_cast<unsigned long long*>(l)};
  }
  KL("cudaMemsetAsync", cudaMemsetAsync(c->fix.h, 0, (std::size_t)n * 8, c->st));
  KL("cudaMemsetAsync", cudaMemsetAsync(c->fix.l, 0, (std::size_t)n * 8, c->st));
  *f = c->fix;
  return 0;
}

int update_np(swap_ctx* c, double* np) {
  TRY(need_weights(c));
  if (c->deterministic) {
    swapk::Fix64 f;
    TRY(fix_sums(c, c->g.C, &f));
    KL("deposit_np", deposit_np(c->g, c->part_view(), c->ntot(), c->prm.beta, np, c->d_err, c->st, f));
    KL("fix_to_double", fix_to_double(c->g.C, f, np, c->st));
  } else {
    KL("cudaMemsetAsync", cudaMemsetAsync(np, 0, (std::size_t)c->g.C * sizeof(double), c->st));
    KL("deposit_np", deposit_np(c->g, c->part_view(), c->ntot(), c->prm.beta, np, c->d_err, c->st));
  }
  if (c->fused) TRY(c->exchange(np, c->g.C, 8));  // MPI_ALLREDUCE, gutsp.f:1503
  KL("periodic", periodic1(c->g, np, c->st));
  return 0;
}

// update_up (gutsp.f:1649-1842) with the velocity chosen by `mode`
// (0 v, 1 extrapol_up's 1.5v-0.5v1, 2 improve_up's 0.5(v+ + v-)).
int update_up_mode(swap_ctx* c, int mode, const double* va, const double* vb, double* out_v1, const double* np,
                   double* up) {
  TRY(need_weights(c));
  const std::size_t b3 = 3 * (std::size_t)c->g.C * sizeof(double);
  if (c->deterministic) {
    swapk::Fix64 f;
    TRY(fix_sums(c, 3 * c->g.C, &f));
    KL("deposit_u",
       deposit_u(c->g, c->part_view(), c->ntot(), c->prm.beta, mode, va, vb, out_v1, c->s_S, c->d_err, c->st, f));
    KL("fix_to_double", fix_to_double(3 * c->g.C, f, c->s_S, c->st));
  } else {
    KL("cudaMemsetAsync", cudaMemsetAsync(c->s_S, 0, b3, c->st));
    KL("deposit_u",
       deposit_u(c->g, c->part_view(), c->ntot(), c->prm.beta, mode, va, vb, out_v1, c->s_S, c->d_err, c->st));
  }
  if (c->fused) TRY(c->exchange(c->s_S, 3 * c->g.C, 8));  // MPI_ALLREDUCE, gutsp.f:1812-1822
  KL("ct_from_sums", ct_from_sums(c->g, c->s_S, np, c->s_ct, c->st));
  KL("periodic", periodic3(c->g, c->s_ct, c->st));
  KL("face_avg_int", face_avg_int(c->g, c->s_ct, up, c->st));
  KL("periodic", periodic3(c->g, up, c->st));
  return 0;
}

// get_Ep (gutsp.f:155-276)
int get_Ep(swap_ctx* c, double* Ep, double* aj, const double* np, double* up, const double* btc) {
  TRY(need_weights(c));
  TRY(face_to_center(c, aj, c->s_ajc));
  TRY(face_to_center(c, up, c->s_upc));
  const double* gpc = nullptr;
  if (c->prm.grad_pe != 0.0) {
    KL("grad_pe_face_int", grad_pe_face_int(c->g, np, c->prm.grad_pe, c->s_gf, c->st));
    TRY(face_to_center(c, c->s_gf, c->s_gpc));
    gpc = c->s_gpc;
  }
  KL("get_Ep", swapk::get_Ep(c->g, c->part_view(), c->ntot(), c->s_ajc, c->s_upc, btc, gpc, Ep, c->d_err, c->st));
  return 0;
}

int vpm(swap_ctx* c, const double* Ep, const double* btc, const double* vp, double* vplus, double* vminus) {
  TRY(need_weights(c));
  KL("vplus_vminus", vplus_vminus(c->g, c->part_view(), c->ntot(), c->prm.dt, Ep, btc, vp, vplus, vminus, c->d_err, c->st));
  return 0;
}

int vp_final(swap_ctx* c, const double* Ep, double* vp, double* vp1, const double* vplus) {
  KL("vp_final", swapk::vp_final(c->part_view(), c->ntot(), c->prm.dt, Ep, vp, vp1, vplus, c->st));
  return 0;
}

// update_rho (gutsp.f:1517-1590): mion * sum (w/mrat)/volb, folded, periodic.
int update_rho(swap_ctx* c, double* mnp) {
  TRY(need_weights(c));
  KL("cudaMemsetAsync", cudaMemsetAsync(mnp, 0, (std::size_t)c->g.C * sizeof(double), c->st));
  KL("deposit_rho", deposit_rho(c->g, c->part_view(), c->ntot(), c->prm.beta, mnp, c->d_err, c->st));
  KL("scale_interior", scale_interior(c->g, mnp, c->mion, c->st));
  KL("periodic", periodic1(c->g, mnp, c->st));
  return 0;
}

// get_temperature (gutsp.f:2257-2541): the face moments of (v/sqrt(mrat))^2
// and v/sqrt(mrat) through update_up's path, then the temperature per node.
int get_temperature(swap_ctx* c, const double* vp, const double* np, double* temp_p) {
  TRY(update_up_mode(c, 3, vp, nullptr, nullptr, np, c->s_btc2));
  TRY(update_up_mode(c, 4, vp, nullptr, nullptr, np, c->s_btmf));
  KL("temperature", temperature(c->g, c->s_btc2, c->s_btmf, c->mion, temp_p, c->st));
  return 0;
}

int move_ion_half(swap_ctx* c, double* xp, const double* vp) {
  KL("move_half", move_half(c->g, c->part_view(), c->ntot(), c->prm.dt, xp, vp, srcops::x_open(c), c->st));
  return 0;
}

}  // namespace ops

// ---------------------------------------------------------------------------
// lifecycle
// ---------------------------------------------------------------------------

extern "C" int swap_abi_version(void) { return 1; }

extern "C" const char* swap_last_error(const swap_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int swap_init(swap_ctx** out, const swap_dims* d, const swap_params* p, const swap_coords* co) {
  if (!out || !d || !p || !co) return SWAP_EINVAL;
  *out = nullptr;
  if (d->nx < 3 || d->ny < 3 || d->nz < 3 || d->ni_max < 0 || p->ntsub < 1) return SWAP_EINVAL;
  if (d->real_bytes != 0 && d->real_bytes != 4 && d->real_bytes != 8) return SWAP_EINVAL;
  const double* arrs[12] = {co->qx, co->qy, co->qz, co->dx_grid, co->dy_grid, co->dz_grid,
                            co->dx_cell, co->dy_cell, co->dz_cell, co->xrat, co->yrat, co->zrat};
  for (const double* a : arrs)
    if (!a) return SWAP_EINVAL;
  auto* c = new swap_ctx();
  c->dims = *d;
  c->prm = *p;
  c->real_bytes = d->real_bytes == 4 ? 4 : 8;
  c->dims.real_bytes = c->real_bytes;
  {
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess)
      c->host_direct = pageable != 0 && c->real_bytes == 8;
  }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return SWAP_ECUDA;
  }
  // geometry, 1-based on the device
  const int ns[12] = {d->nx, d->ny, d->nz, d->nx, d->ny, d->nz, d->nx, d->ny, d->nz, d->nx, d->ny, d->nz};
  double* dg[12];
  for (int a = 0; a < 12; ++a) {
    std::vector<double> h((std::size_t)ns[a] + 1, 0.0);
    std::memcpy(h.data() + 1, arrs[a], (std::size_t)ns[a] * sizeof(double));
    dg[a] = c->dalloc(h.size());
    if (!dg[a] || cudaMemcpy(dg[a], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      swap_finalize(c);
      return SWAP_ECUDA;
    }
  }
  Geo& g = c->g;
  g.nx = d->nx; g.ny = d->ny; g.nz = d->nz;
  g.C = (long long)d->nx * d->ny * d->nz;
  g.qx = dg[0]; g.qy = dg[1]; g.qz = dg[2];
  g.dxg = dg[3]; g.dyg = dg[4]; g.dzg = dg[5];
  g.dxc = dg[6]; g.dyc = dg[7]; g.dzc = dg[8];
  g.xr = dg[9]; g.yr = dg[10]; g.zr = dg[11];
  g.dy = p->dy;
  g.inv_dx = 1.0 / (co->qx[1] - co->qx[0]);
  g.inv_dz = 1.0 / (co->qz[1] - co->qz[0]);
  c->h_qx.assign(co->qx, co->qx + d->nx);
  c->h_qy.assign(co->qy, co->qy + d->ny);
  c->h_qz.assign(co->qz, co->qz + d->nz);
  // grid scratch (the reference's /dummy/ a, c, ct and subroutine locals)
  const std::size_t C3 = 3 * (std::size_t)g.C;
  double** bufs[] = {&c->s_a, &c->s_aa, &c->s_c, &c->s_ct, &c->s_btcl, &c->s_btc2, &c->s_btmf, &c->s_ajc,
                     &c->s_upc, &c->s_btp1, &c->s_S, &c->s_gf, &c->s_gpc};
  for (double** b : bufs) {
    *b = c->dalloc(C3);
    if (!*b || cudaMemset(*b, 0, C3 * sizeof(double)) != cudaSuccess) {
      swap_finalize(c);
      return SWAP_ECUDA;
    }
  }
  c->s_dtn = c->dalloc((std::size_t)g.C);
  c->s_red = c->dalloc(8);
  int* e = nullptr;
  if (!c->s_dtn || !c->s_red || cudaMalloc(&e, sizeof(int)) != cudaSuccess) {
    swap_finalize(c);
    return SWAP_ECUDA;
  }
  c->owned.push_back(e);
  c->d_err = e;
  if (cudaMemset(e, 0, sizeof(int)) != cudaSuccess || cudaEventCreate(&c->t0) != cudaSuccess ||
      cudaEventCreate(&c->t1) != cudaSuccess) {
    swap_finalize(c);
    return SWAP_ECUDA;
  }
  *out = c;
  return SWAP_OK;
}

extern "C" int swap_finalize(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  if (c->st) cudaStreamSynchronize(c->st);
  swap_f32_free(c);
  swap_diag_free(c);
  srcops::free_all(c);
  for (auto& kv : c->reg) cudaFree(kv.second.dev);
  for (void* p : c->owned) cudaFree(p);
  if (c->stage32) cudaFree(c->stage32);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  c->prof_free();
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// registration
// ---------------------------------------------------------------------------

extern "C" int swap_bind_particles(swap_ctx* c, double* xp, double* vp, double* vp1, double* mrat, double* beta_p,
                                   int32_t* ijkp, int32_t* ni_tot) {
  if (!c || !xp || !vp || !vp1 || !mrat || !beta_p || !ni_tot) return SWAP_EINVAL;
  const std::size_t NM = (std::size_t)c->dims.ni_max;
  TRY(c->add_mirror(xp, 3 * NM * sizeof(double), MirrorKind::Particle3));
  TRY(c->add_mirror(vp, 3 * NM * sizeof(double), MirrorKind::Particle3));
  TRY(c->add_mirror(vp1, 3 * NM * sizeof(double), MirrorKind::Particle3));
  TRY(c->add_mirror(mrat, NM * sizeof(double), MirrorKind::Particle1));
  TRY(c->add_mirror(beta_p, NM * sizeof(double), MirrorKind::Particle1));
  if (ijkp) TRY(c->add_mirror(ijkp, 3 * NM * sizeof(int32_t), MirrorKind::ParticleI3, false));
  c->h_xp = xp; c->h_vp = vp; c->h_vp1 = vp1; c->h_mrat = mrat; c->h_beta_p = beta_p; c->h_ijkp = ijkp;
  c->ni_tot_ptr = ni_tot;
  c->d_mrat = static_cast<double*>(c->find(mrat)->dev);
  c->d_beta_p = static_cast<double*>(c->find(beta_p)->dev);
  if (!c->d_ijk) {
    void* p1 = nullptr;
    void* p2 = nullptr;
    if (cudaMalloc(&p1, 3 * NM * sizeof(int32_t) + 16) != cudaSuccess ||
        cudaMalloc(&p2, 8 * NM * sizeof(double) + 16) != cudaSuccess)
      return c->fail(SWAP_ECUDA, "device allocation of ijkp/wght failed");
    c->owned.push_back(p1);
    c->owned.push_back(p2);
    c->d_ijk = static_cast<int32_t*>(p1);
    c->d_wght = static_cast<double*>(p2);
  }
  return SWAP_OK;
}

extern "C" int swap_bind_fields(swap_ctx* c, double* b0, double* b1, double* b12, double* b1p2, double* bt,
                                double* btc, double* np, double* up, double* aj, double* E, double* nu) {
  if (!c || !b0 || !b1 || !b12 || !b1p2 || !bt || !btc || !np || !up || !aj || !E || !nu) return SWAP_EINVAL;
  const std::size_t C = (std::size_t)c->g.C;
  double* v3[] = {b0, b1, b12, b1p2, bt, btc, up, aj, E};
  for (double* a : v3) TRY(c->add_mirror(a, 3 * C * sizeof(double), MirrorKind::Grid));
  TRY(c->add_mirror(np, C * sizeof(double), MirrorKind::Grid));
  TRY(c->add_mirror(nu, C * sizeof(double), MirrorKind::Grid));
  c->h_b0 = b0; c->h_b1 = b1; c->h_b12 = b12; c->h_b1p2 = b1p2; c->h_bt = bt; c->h_btc = btc;
  c->h_np = np; c->h_up = up; c->h_aj = aj; c->h_E = E; c->h_nu = nu;
  return SWAP_OK;
}

extern "C" int swap_bind_array(swap_ctx* c, void* host, int64_t bytes) {
  if (!c || !host || bytes <= 0) return SWAP_EINVAL;
  if (bytes % c->real_bytes) return c->fail(SWAP_EINVAL, "swap_bind_array: size is not a whole number of reals");
  // the device mirror holds doubles whatever the caller's real size
  const std::size_t dev_bytes = (std::size_t)bytes / (std::size_t)c->real_bytes * sizeof(double);
  const std::size_t NM3 = 3 * (std::size_t)c->dims.ni_max * sizeof(double);
  // a (ni_max,3) real array moves as particle segments
  const MirrorKind k = dev_bytes == NM3 ? MirrorKind::Particle3 : MirrorKind::Grid;
  return c->add_mirror(host, dev_bytes, k);
}

extern "C" int swap_sync_to_device(swap_ctx* c, const void* host) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  if (host) {
    Mirror* m = c->find(host);
    if (!m) return c->fail(SWAP_EINVAL, "array not registered");
    TRY(c->transfer(*m, true));
  } else {
    for (auto& kv : c->reg)
      if (!kv.second.dev_valid) TRY(c->transfer(kv.second, true));
  }
  cudaError_t e = cudaStreamSynchronize(c->st);
  return e == cudaSuccess ? SWAP_OK : c->cuda_fail(e, "sync_to_device");
}

extern "C" int swap_sync_to_host(swap_ctx* c, void* host) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  if (host) {
    Mirror* m = c->find(host);
    if (!m) return c->fail(SWAP_EINVAL, "array not registered");
    if (!m->host_valid) TRY(c->transfer(*m, false));
  } else {
    for (auto& kv : c->reg)
      if (!kv.second.host_valid) TRY(c->transfer(kv.second, false));
  }
  cudaError_t e = cudaStreamSynchronize(c->st);
  return e == cudaSuccess ? SWAP_OK : c->cuda_fail(e, "sync_to_host");
}

extern "C" int swap_set_host_direct(swap_ctx* c, int on) {
  if (!c) return SWAP_EINVAL;
  if (on && c->real_bytes != 8)
    return c->fail(SWAP_EINVAL, "host-direct mode reads 8-byte reals; this context binds 4-byte reals");
  if (on) {
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess || !pageable)
      return c->fail(SWAP_EINVAL, "this device cannot address host memory directly");
  }
  c->host_direct = on != 0;
  return SWAP_OK;
}

extern "C" int swap_set_deterministic(swap_ctx* c, int32_t on) {
  if (!c) return SWAP_EINVAL;
  c->deterministic = on != 0;
  return SWAP_OK;
}

extern "C" int swap_set_wait_limit(swap_ctx* c, uint32_t polls) {
  if (!c) return SWAP_EINVAL;
  c->wait_polls = polls;
  return SWAP_OK;
}

extern "C" int swap_set_exchange(swap_ctx* c, swap_exchange_fn fn, void* user) {
  if (!c) return SWAP_EINVAL;
  c->xfn = fn;
  c->xuser = user;
  return SWAP_OK;
}

extern "C" int swap_transfer_bytes(swap_ctx* c, int64_t* h2d, int64_t* d2h, int reset) {
  if (!c) return SWAP_EINVAL;
  if (h2d) *h2d = c->h2d_bytes;
  if (d2h) *d2h = c->d2h_bytes;
  if (reset) c->h2d_bytes = c->d2h_bytes = 0;
  return SWAP_OK;
}

extern "C" int swap_mark_host_dirty(swap_ctx* c, const void* host) {
  if (!c) return SWAP_EINVAL;
  if (host) {
    Mirror* m = c->find(host);
    if (!m) return c->fail(SWAP_EINVAL, "array not registered");
    m->dev_valid = false;
    m->host_valid = true;
  } else {
    for (auto& kv : c->reg) {
      kv.second.dev_valid = false;
      kv.second.host_valid = true;
    }
  }
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// per-subroutine entries
// ---------------------------------------------------------------------------

#define ENTRY                             \
  if (!c) return SWAP_EINVAL;             \
  TRY(c->begin())

// The implicit per-particle inputs (mrat, beta_p) are uploaded on first use.
static int need_particle_scalars(swap_ctx* c) {
  if (!c->h_mrat) return c->fail(SWAP_EINVAL, "swap_bind_particles has not been called");
  double* d;
  TRY(c->use(c->h_mrat, Access::In, &d));
  TRY(c->use(c->h_beta_p, Access::In, &d));
  return SWAP_OK;
}

extern "C" int swap_get_interp_weights(swap_ctx* c, const double* xp) {
  ENTRY;
  double* dxp;
  TRY(need_particle_scalars(c));
  TRY(c->use(xp, Access::In, &dxp));
  TRY(ops::get_interp_weights(c, dxp));
  int r = c->finish();
  if (r == SWAP_OK && c->h_ijkp) {  // the COMMON ijkp mirror now holds new indices
    Mirror* m = c->find(c->h_ijkp);
    const std::size_t NM = (std::size_t)c->dims.ni_max;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess && c->ntot() > 0; ++k)
      e = cudaMemcpyAsync(static_cast<int32_t*>(m->dev) + k * NM, c->d_ijk + k * NM, (std::size_t)c->ntot() * 4,
                          cudaMemcpyDeviceToDevice, c->st);
    const cudaError_t e2 = cudaStreamSynchronize(c->st);  // also after a failed copy: nothing stays queued
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return c->cuda_fail(e, "ijkp mirror");
    m->dev_valid = true;
    m->host_valid = false;
  }
  return r;
}

extern "C" int swap_update_np(swap_ctx* c, double* np) {
  ENTRY;
  double* dnp;
  TRY(need_particle_scalars(c));
  TRY(c->use(np, Access::Out, &dnp));
  TRY(ops::update_np(c, dnp));
  return c->finish();
}

extern "C" int swap_update_up(swap_ctx* c, const double* vp, const double* np, double* up) {
  ENTRY;
  double *dvp, *dnp, *dup;
  TRY(need_particle_scalars(c));
  TRY(c->use(vp, Access::In, &dvp));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(up, Access::Out, &dup));
  TRY(ops::update_up_mode(c, 0, dvp, nullptr, nullptr, dnp, dup));
  return c->finish();
}

extern "C" int swap_extrapol_up(swap_ctx* c, double* up, const double* vp, const double* vp1, const double* np) {
  ENTRY;
  double *dvp, *dvp1, *dnp, *dup;
  TRY(need_particle_scalars(c));
  TRY(c->use(vp, Access::In, &dvp));
  TRY(c->use(vp1, Access::In, &dvp1));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(up, Access::Out, &dup));
  TRY(ops::update_up_mode(c, 1, dvp, dvp1, nullptr, dnp, dup));
  return c->finish();
}

extern "C" int swap_get_Ep(swap_ctx* c, double* Ep, double* aj, const double* np, double* up, const double* btc,
                           const double* nu) {
  ENTRY;
  double *dEp, *daj, *dnp, *dup, *dbtc, *dnu;
  TRY(need_particle_scalars(c));
  TRY(c->use(aj, Access::InOut, &daj));  // face_to_center() rewrites its ghosts
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(up, Access::InOut, &dup));
  TRY(c->use(btc, Access::In, &dbtc));
  TRY(c->use(nu, Access::In, &dnu));
  TRY(c->use(Ep, Access::Out, &dEp));
  TRY(ops::get_Ep(c, dEp, daj, dnp, dup, dbtc));
  return c->finish();
}

extern "C" int swap_get_vplus_vminus(swap_ctx* c, const double* Ep, const double* btc, const double* vp,
                                     double* vplus, double* vminus) {
  ENTRY;
  double *dEp, *dbtc, *dvp, *dvpl, *dvmi;
  TRY(need_particle_scalars(c));
  TRY(c->use(Ep, Access::In, &dEp));
  TRY(c->use(btc, Access::In, &dbtc));
  TRY(c->use(vp, Access::In, &dvp));
  TRY(c->use(vplus, Access::Out, &dvpl));
  TRY(c->use(vminus, Access::Out, &dvmi));
  TRY(ops::vpm(c, dEp, dbtc, dvp, dvpl, dvmi));
  return c->finish();
}

extern "C" int swap_improve_up(swap_ctx* c, double* vp1, const double* vplus, const double* vminus, double* up,
                               const double* np) {
  ENTRY;
  double *dvp1, *dvpl, *dvmi, *dup, *dnp;
  TRY(need_particle_scalars(c));
  TRY(c->use(vplus, Access::In, &dvpl));
  TRY(c->use(vminus, Access::In, &dvmi));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(vp1, Access::Out, &dvp1));
  TRY(c->use(up, Access::Out, &dup));
  TRY(ops::update_up_mode(c, 2, dvpl, dvmi, dvp1, dnp, dup));
  return c->finish();
}

extern "C" int swap_get_vp_final(swap_ctx* c, const double* Ep, double* vp, double* vp1, const double* vplus) {
  ENTRY;
  double *dEp, *dvp, *dvp1, *dvpl;
  TRY(c->use(Ep, Access::In, &dEp));
  TRY(c->use(vplus, Access::In, &dvpl));
  TRY(c->use(vp, Access::InOut, &dvp));
  TRY(c->use(vp1, Access::Out, &dvp1));
  TRY(ops::vp_final(c, dEp, dvp, dvp1, dvpl));
  return c->finish();
}

extern "C" int swap_move_ion_half(swap_ctx* c, double* xp, const double* vp, const double* vp1, double* input_p) {
  (void)vp1;
  (void)input_p;  // declared but unused by the reference's active code (gutsp.f:454-570)
  ENTRY;
  double *dxp, *dvp;
  TRY(c->use(vp, Access::In, &dvp));
  TRY(c->use(xp, Access::InOut, &dxp));
  TRY(ops::move_ion_half(c, dxp, dvp));
  return c->finish();
}

extern "C" int swap_curlB(swap_ctx* c, double* bt, const double* np, double* aj) {
  ENTRY;
  double *dbt, *dnp, *daj;
  TRY(c->use(bt, Access::InOut, &dbt));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(aj, Access::InOut, &daj));  // ghosts untouched, as in the reference
  TRY(ops::curlB(c, dbt, dnp, daj));
  return c->finish();
}

extern "C" int swap_edge_to_center(swap_ctx* c, double* bt, double* btc) {
  ENTRY;
  double *dbt, *dbtc;
  TRY(c->use(bt, Access::InOut, &dbt));
  TRY(c->use(btc, Access::Out, &dbtc));
  TRY(ops::edge_to_center(c, dbt, dbtc));
  return c->finish();
}

extern "C" int swap_face_to_center(swap_ctx* c, double* v, double* vc) {
  ENTRY;
  double *dv, *dvc;
  TRY(c->use(v, Access::InOut, &dv));
  TRY(c->use(vc, Access::Out, &dvc));
  TRY(ops::face_to_center(c, dv, dvc));
  return c->finish();
}

extern "C" int swap_get_E(swap_ctx* c, double* E, const double* b0, double* bt, double* aj, const double* up,
                          const double* np, const double* nu) {
  (void)b0;  // passed but unused by the reference (gutsf.f:994-1110)
  ENTRY;
  double *dE, *dbt, *daj, *dup, *dnp, *dnu;
  TRY(c->use(bt, Access::InOut, &dbt));
  TRY(c->use(aj, Access::In, &daj));
  TRY(c->use(up, Access::In, &dup));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(nu, Access::In, &dnu));
  TRY(c->use(E, Access::InOut, &dE));
  TRY(ops::get_E(c, dE, dbt, daj, dup, dnp, dnu));
  return c->finish();
}

extern "C" int swap_predict_B(swap_ctx* c, double* b0, double* b1, double* b12, double* b1p2, double* bt,
                              double* E, double* aj, double* up, double* np, double* nu, double dtsub) {
  (void)b0;
  (void)b1;
  ENTRY;
  double *db12, *db1p2, *dbt, *dE, *daj, *dup, *dnp, *dnu;
  TRY(c->use(b12, Access::In, &db12));
  TRY(c->use(bt, Access::InOut, &dbt));
  TRY(c->use(aj, Access::In, &daj));
  TRY(c->use(up, Access::In, &dup));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(nu, Access::In, &dnu));
  TRY(c->use(E, Access::InOut, &dE));
  TRY(c->use(b1p2, Access::InOut, &db1p2));
  TRY(ops::predict_B(c, db12, db1p2, dbt, dE, daj, dup, dnp, dnu, dtsub));
  return c->finish();
}

extern "C" int swap_correct_B(swap_ctx* c, double* b0, double* b1, double* b1p2, double* E, double* aj, double* up,
                              double* np, double* nu, double dtsub) {
  (void)b0;
  ENTRY;
  double *db1, *db1p2, *dE, *daj, *dup, *dnp, *dnu;
  TRY(c->use(b1, Access::In, &db1));
  TRY(c->use(b1p2, Access::InOut, &db1p2));
  TRY(c->use(up, Access::In, &dup));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(nu, Access::In, &dnu));
  TRY(c->use(aj, Access::InOut, &daj));
  TRY(c->use(E, Access::InOut, &dE));
  TRY(ops::correct_B(c, db1, db1p2, dE, daj, dup, dnp, dnu, dtsub));
  return c->finish();
}

extern "C" int swap_f_update_tlev(swap_ctx* c, double* b1, double* b12, double* b1p2, double* bt, const double* b0) {
  (void)b0;
  ENTRY;
  double *db1, *db12, *db1p2, *dbt;
  TRY(c->use(b1p2, Access::In, &db1p2));
  TRY(c->use(b1, Access::InOut, &db1));
  TRY(c->use(b12, Access::Out, &db12));
  TRY(c->use(bt, Access::Out, &dbt));
  TRY(ops::f_update_tlev(c, db1, db12, db1p2, dbt));
  return c->finish();
}

extern "C" int swap_check_time_step(swap_ctx* c, const double* bt, const double* np, double* dtsub, double* ntf) {
  ENTRY;
  if (!dtsub || !ntf) return c->fail(SWAP_EINVAL, "null dtsub/ntf");
  double *dbt, *dnp;
  TRY(c->use(bt, Access::In, &dbt));
  TRY(c->use(np, Access::In, &dnp));
  TRY(ops::check_time_step(c, dbt, dnp, dtsub, ntf));
  return c->finish();
}

extern "C" int swap_periodic(swap_ctx* c, double* b) {
  ENTRY;
  double* db;
  TRY(c->use(b, Access::InOut, &db));
  TRY(ops::periodic(c, db));
  return c->finish();
}

extern "C" int swap_periodic_scalar(swap_ctx* c, double* b) {
  ENTRY;
  double* db;
  TRY(c->use(b, Access::InOut, &db));
  CU(periodic1(c->g, db, c->st));
  return c->finish();
}

extern "C" int swap_update_rho(swap_ctx* c, double* mnp) {
  ENTRY;
  double* d;
  TRY(need_particle_scalars(c));
  TRY(c->use(mnp, Access::Out, &d));
  TRY(ops::update_rho(c, d));
  return c->finish();
}

extern "C" int swap_get_temperature(swap_ctx* c, const double* xp, const double* vp, const double* np,
                                    double* temp_p) {
  ENTRY;
  (void)xp;  // the reference reads positions through ijkp/wght only
  double *dvp, *dnp, *dt;
  TRY(need_particle_scalars(c));
  TRY(c->use(vp, Access::In, &dvp));
  TRY(c->use(np, Access::In, &dnp));
  TRY(c->use(temp_p, Access::Out, &dt));
  TRY(ops::get_temperature(c, dvp, dnp, dt));
  return c->finish();
}

extern "C" int swap_set_mion(swap_ctx* c, double mion) {
  if (!c || !(mion > 0)) return SWAP_EINVAL;
  c->mion = mion;
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// fused, device-resident ion step on the bound arrays (maind.f:385-479)
// ---------------------------------------------------------------------------

namespace {

struct Bound {
  double *xp, *vp, *vp1, *b0, *b1, *b12, *b1p2, *bt, *btc, *np, *up, *aj, *E, *nu;
};

int bound_inputs(swap_ctx* c, Bound& b) {
  if (!c->h_xp || !c->h_b1) return c->fail(SWAP_EINVAL, "swap_bind_particles and swap_bind_fields are required");
  TRY(need_particle_scalars(c));
  TRY(c->use(c->h_xp, Access::InOut, &b.xp));
  TRY(c->use(c->h_vp, Access::InOut, &b.vp));
  TRY(c->use(c->h_vp1, Access::InOut, &b.vp1));
  TRY(c->use(c->h_b0, Access::In, &b.b0));
  TRY(c->use(c->h_b1, Access::InOut, &b.b1));
  TRY(c->use(c->h_b12, Access::InOut, &b.b12));
  TRY(c->use(c->h_b1p2, Access::InOut, &b.b1p2));
  TRY(c->use(c->h_bt, Access::InOut, &b.bt));
  TRY(c->use(c->h_btc, Access::InOut, &b.btc));
  TRY(c->use(c->h_np, Access::InOut, &b.np));
  TRY(c->use(c->h_up, Access::InOut, &b.up));
  TRY(c->use(c->h_aj, Access::InOut, &b.aj));
  TRY(c->use(c->h_E, Access::InOut, &b.E));
  TRY(c->use(c->h_nu, Access::In, &b.nu));
  if (!c->w_Ep) {
    const std::size_t n3 = 3 * (std::size_t)c->dims.ni_max + 2;
    c->w_Ep = c->dalloc(n3);
    c->w_vplus = c->dalloc(n3);
    c->w_vminus = c->dalloc(n3);
    if (!c->w_Ep || !c->w_vplus || !c->w_vminus) return c->fail(SWAP_ECUDA, "allocation of push work arrays");
  }
  return SWAP_OK;
}

// Marks the deposits made in its scope as the fused step's (exchanged).
struct FusedScope {
  swap_ctx* c;
  explicit FusedScope(swap_ctx* cc) : c(cc) { c->fused = true; }
  ~FusedScope() { c->fused = false; }
};

int step_pre(swap_ctx* c, Bound& b) {
  FusedScope fs(c);
  TRY(srcops::step_begin(c, b.xp, b.vp, b.vp1));                            // sources
  TRY(ops::get_interp_weights(c, b.xp));                                     // maind.f:385
  TRY(ops::update_np(c, b.np));                                              // :386
  TRY(ops::update_up_mode(c, 0, b.vp, nullptr, nullptr, b.np, b.up));        // :387
  TRY(ops::curlB(c, b.bt, b.np, b.aj));                                      // :395
  TRY(ops::edge_to_center(c, b.bt, b.btc));                                  // :398
  TRY(ops::update_up_mode(c, 1, b.vp, b.vp1, nullptr, b.np, b.up));          // :399
  TRY(ops::get_Ep(c, c->w_Ep, b.aj, b.np, b.up, b.btc));                     // :400
  TRY(ops::vpm(c, c->w_Ep, b.btc, b.vp, c->w_vplus, c->w_vminus));           // :401
  TRY(ops::update_up_mode(c, 2, c->w_vplus, c->w_vminus, b.vp1, b.np, b.up)); // :402
  TRY(ops::get_Ep(c, c->w_Ep, b.aj, b.np, b.up, b.btc));                     // :404
  TRY(ops::vpm(c, c->w_Ep, b.btc, b.vp, c->w_vplus, c->w_vminus));           // :405
  TRY(ops::vp_final(c, c->w_Ep, b.vp, b.vp1, c->w_vplus));                   // :406
  TRY(ops::move_ion_half(c, b.xp, b.vp));                                    // :408
  TRY(srcops::after_move(c, b.xp, b.vp, b.vp1));                             // outflow
  TRY(ops::get_interp_weights(c, b.xp));                                     // :411
  TRY(ops::update_np(c, b.np));                                              // :412
  TRY(ops::update_up_mode(c, 0, b.vp, nullptr, nullptr, b.np, b.up));        // :413
  return SWAP_OK;
}

int subcycles(swap_ctx* c, Bound& b) {
  double dtsub = c->prm.dt / (double)c->prm.ntsub;  // maind.f:420 (dtsub_init, inputs.f:142)
  double ntf = (double)c->prm.ntsub;                // :421
  TRY(ops::check_time_step(c, b.bt, b.np, &dtsub, &ntf));  // :423
  c->last_dtsub = dtsub;
  c->last_ntf = ntf;
  const int n = (int)ntf;
  for (int s = 0; s < n; ++s) {  // :425-476
    TRY(ops::curlB(c, b.bt, b.np, b.aj));
    TRY(ops::predict_B(c, b.b12, b.b1p2, b.bt, b.E, b.aj, b.up, b.np, b.nu, dtsub));
    TRY(ops::correct_B(c, b.b1, b.b1p2, b.E, b.aj, b.up, b.np, b.nu, dtsub));
    TRY(ops::f_update_tlev(c, b.b1, b.b12, b.b1p2, b.bt));
  }
  return SWAP_OK;
}

// maind.f:479 and the sinks after it (res_chex, maind.f:484).
int step_post(swap_ctx* c, Bound& b) {
  TRY(ops::move_ion_half(c, b.xp, b.vp));
  TRY(srcops::after_move(c, b.xp, b.vp, b.vp1));
  TRY(srcops::step_end(c, b.xp, b.vp, b.vp1));
  return SWAP_OK;
}

}  // namespace

extern "C" int swap_ion_step_pre(swap_ctx* c) {
  ENTRY;
  Bound b;
  TRY(bound_inputs(c, b));
  TRY(step_pre(c, b));
  return c->finish();
}

extern "C" int swap_field_subcycles(swap_ctx* c) {
  ENTRY;
  Bound b;
  TRY(bound_inputs(c, b));
  TRY(subcycles(c, b));
  return c->finish();
}

extern "C" int swap_ion_step_post(swap_ctx* c) {
  ENTRY;
  Bound b;
  TRY(bound_inputs(c, b));
  TRY(step_post(c, b));  // maind.f:479
  return c->finish();
}

extern "C" int swap_ion_step(swap_ctx* c) {
  ENTRY;
  Bound b;
  TRY(bound_inputs(c, b));
  TRY(step_pre(c, b));
  TRY(subcycles(c, b));
  TRY(step_post(c, b));
  return c->finish();
}

extern "C" int swap_run(swap_ctx* c, int32_t nsteps) {
  ENTRY;
  Bound b;
  TRY(bound_inputs(c, b));
  for (int s = 0; s < nsteps; ++s) {
    TRY(step_pre(c, b));
    TRY(subcycles(c, b));
    TRY(step_post(c, b));
  }
  return c->finish();
}

// ---------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------

int ops::energy7(swap_ctx* c, double out[7]) {
  TRY(c->begin());
  Bound b;
  TRY(bound_inputs(c, b));
  CU(energy_parts(c->g, c->part_view(), c->ntot(), c->prm.beta, c->prm.alpha, b.vp, b.b0, b.b1, b.E, c->s_red,
                  c->st));
  CU(cudaMemcpyAsync(out, c->s_red, 7 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  return c->finish();
}

extern "C" int swap_energy(swap_ctx* c, double out[4]) {
  ENTRY;
  if (!out) return c->fail(SWAP_EINVAL, "null output");
  Bound b;
  TRY(bound_inputs(c, b));
  CU(energy_parts(c->g, c->part_view(), c->ntot(), c->prm.beta, c->prm.alpha, b.vp, b.b0, b.b1, b.E, c->s_red,
                  c->st));
  CU(cudaMemcpyAsync(out, c->s_red, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  return c->finish();
}

extern "C" int swap_max_abs_divB(swap_ctx* c, const double* bh, double* out) {
  ENTRY;
  if (!out) return c->fail(SWAP_EINVAL, "null output");
  double* db;
  TRY(c->use(bh, Access::In, &db));
  CU(divb_max(c->g, db, c->s_red, c->st));
  CU(cudaMemcpyAsync(out, c->s_red, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  return c->finish();
}

extern "C" int swap_check_finite(swap_ctx* c) {
  ENTRY;
  CU(cudaMemsetAsync(c->s_red, 0, sizeof(double), c->st));
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c->s_red);
  for (auto& kv : c->reg) {
    Mirror& m = kv.second;
    if (m.kind == MirrorKind::ParticleI3) continue;
    double* d;
    TRY(c->use(m.host, Access::In, &d));
    if (m.kind == MirrorKind::Particle3 || m.kind == MirrorKind::Particle1) {
      const int ncomp = m.kind == MirrorKind::Particle1 ? 1 : 3;
      for (int k = 0; k < ncomp; ++k) CU(count_nonfinite(d + (std::size_t)k * c->dims.ni_max, c->ntot(), cnt, c->st));
    } else {
      CU(count_nonfinite(d, (long long)(m.bytes / sizeof(double)), cnt, c->st));
    }
  }
  unsigned long long h = 0;
  CU(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  TRY(c->finish());
  if (h) return c->fail(SWAP_ENONFINITE, std::to_string(h) + " non-finite values in registered arrays");
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// timing
// ---------------------------------------------------------------------------

extern "C" int swap_timer_start(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  CU(cudaEventRecord(c->t0, c->st));
  return SWAP_OK;
}

extern "C" int swap_timer_stop(swap_ctx* c, double* ms) {
  if (!c || !ms) return SWAP_EINVAL;
  CU(cudaEventRecord(c->t1, c->st));
  CU(cudaEventSynchronize(c->t1));
  float f = 0;
  CU(cudaEventElapsedTime(&f, c->t0, c->t1));
  *ms = f;
  return SWAP_OK;
}
