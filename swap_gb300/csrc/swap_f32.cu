// swap_f32.cu -- the FP32 form of the ion step behind the same context.
//
// swap_f32_begin converts the bound FP64 state (device mirrors) into the
// FP32 form and sorts the particles by brick-major cell key; swap_f32_run
// advances whole ion steps (maind.f:385-479); swap_f32_end writes the state
// back into the bound arrays' device mirrors (particles come back in sorted
// order).  Precision: particle positions as int32 cell + FP32 offset, FP32
// velocities and moments, B accumulated across subcycles in double-float
// (float hi + lo pairs, 48 significant bits).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swap_gpu.h"
#include "k32.cuh"
#include "swap_dev.cuh"
#include "swap_ctx.h"
#include "swap_ops.h"
#include "swap_prof.h"
#include "surrogate.h"

using namespace swapk32;

struct F32State {
  G32 g{};
  Species sp{};
  long long N = 0;
  Part buf[2]{};
  int cur = 0;
  int64_t *start = nullptr, *start_new = nullptr, *count = nullptr, *sums = nullptr;
  uint32_t* dirrank = nullptr;
  uint16_t* dep = nullptr;
  uint16_t* pre = nullptr;
  void* partial = nullptr;  // brick partial tiles, 8 bytes per entry (fixed point or FP32)
  FarList far{};            // pass 3's ions that moved more than one cell
  // the isothermal electron-pressure term (grad_pe != 0): its face gradient
  // for E, and centred per node for the passes' gather
  float gp = 0.0f;
  float* gpf = nullptr;
  float4* kitg = nullptr;
  bool exact = true;        // exact moment sums (swap_f32_set_moment_sums)
  float4* kit = nullptr;
  float *np = nullptr, *S = nullptr, *up = nullptr, *aj = nullptr, *ct = nullptr, *E = nullptr, *nu = nullptr;
  long long np_span = 0;  // floats from np to the end of S (one allocation)
  float *db1 = nullptr, *db1p2 = nullptr, *dbtp1 = nullptr;
  double* b0 = nullptr;  // FP64 b0, for the diagnostics
  // B levels in double-float: hi + lo float pairs (48 significant bits)
  struct DF {
    float *h = nullptr, *l = nullptr;
  } b1, b12, b1p2;
  float* b0c = nullptr;  // 3 floats: the uniform b0
  uint8_t* order = nullptr;  // source-key order table of the incremental sort
  float* dtn = nullptr;  // per-node Courant time
  float* d_min = nullptr;
  double* acc = nullptr;
  double last_dtsub = 0, last_ntf = 0;
  std::vector<void*> owned;
  // species tables (FP64, device) and the particle sources and sinks
  double *tabm = nullptr, *tabb = nullptr;
  srcops::F32Stage stage;
  bool src_on = false, x_open = false, ended = false;
  long long n_out = 0;  // ions written back by swap_f32_end
  uint8_t heavy_of[MAX_SPECIES]{};
  // the learned subcycle surrogate
  swap_surrogate* sur = nullptr;      // attached network
  swap_surrogate* collect = nullptr;  // network collecting training pairs
  int sur_every = 8;
  double sur_bound = 1e-3;
  double sur_bound_db = 0;             // bound on the (B - b0) error too; 0: none
  bool sur_off = false;               // the last judge failed: plain until one passes
  long long sur_step = 0, sur_used = 0, sur_judged = 0, sur_fallbacks = 0;
  double sur_err_b = 0, sur_err_db = 0;
  float *e_sum = nullptr, *vin = nullptr, *ve = nullptr, *jh = nullptr, *jl = nullptr, *jdb = nullptr;
  double* jacc = nullptr;

  // the next step's new ions are staged on a second stream while this step's
  // fields advance (the staging draws in FP64, the field kernels stream HBM)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_side = nullptr;
  // the step's sort runs on the second stream too, beside the field
  // subcycles (it reads only pass 3's outputs and the staging): its end, and
  // the new ion count it copies to pinned host memory
  cudaEvent_t ev_sort = nullptr;
  int64_t* h_n = nullptr;
  bool sort_pending = false;
  ~F32State() {
    if (side) cudaStreamSynchronize(side);
    if (ev_main) cudaEventDestroy(ev_main);
    if (ev_side) cudaEventDestroy(ev_side);
    if (ev_sort) cudaEventDestroy(ev_sort);
    if (h_n) cudaFreeHost(h_n);
    if (side) cudaStreamDestroy(side);
    srcops::stage_free(stage);
    for (void* p : owned) cudaFree(p);
    release_pool();
  }
  // device blocks of a previous state of the same context, handed back in
  // allocation order while their sizes match (swap_f32_begin again on the
  // same grid allocates nothing); the rest are freed by release_pool
  std::vector<std::pair<void*, std::size_t>> pool;
  std::size_t pool_next = 0;
  std::vector<std::size_t> owned_bytes;
  template <class T>
  T* alloc(std::size_t n) {
    const std::size_t bytes = n * sizeof(T) + 64;
    void* p = nullptr;
    if (pool_next < pool.size() && pool[pool_next].second == bytes) {
      p = pool[pool_next++].first;
    } else {
      release_pool();
      if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    }
    owned.push_back(p);
    owned_bytes.push_back(bytes);
    return static_cast<T*>(p);
  }
  void release_pool() {
    for (std::size_t q = pool_next; q < pool.size(); ++q) cudaFree(pool[q].first);
    pool.clear();
    pool_next = 0;
  }
};

static F32State* f32(swap_ctx* c) { return static_cast<F32State*>(c->f32_state); }

bool swap_f32_ended(swap_ctx* c) { return !f32(c) || f32(c)->ended; }

void swap_f32_free(swap_ctx* c) {
  delete f32(c);
  c->f32_state = nullptr;
}

#define TRY(x)             \
  do {                     \
    int _r = (x);          \
    if (_r) return _r;     \
  } while (0)
#define KL(name, x)                                           \
  do {                                                        \
    ProfScope _ps(c, name, c->st);                            \
    cudaError_t _e = (x);                                     \
    if (_e != cudaSuccess) return c->cuda_fail(_e, name);     \
  } while (0)
// a launcher call that launches n kernels
#define KLN(name, n, x)                                       \
  do {                                                        \
    ProfScope _ps(c, name, c->st, n);                         \
    cudaError_t _e = (x);                                     \
    if (_e != cudaSuccess) return c->cuda_fail(_e, name);     \
  } while (0)
#define CU(x)                                                 \
  do {                                                        \
    cudaError_t _e = (x);                                     \
    if (_e != cudaSuccess) return c->cuda_fail(_e, #x);       \
  } while (0)

static int check_err(swap_ctx* c) {
  int herr = 0;
  CU(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  if (herr) {
    cudaMemset(c->d_err, 0, sizeof(int));
    if (herr == swapk::KERR_DOMAIN) return c->fail(SWAP_EDOMAIN, "a particle lies outside the grid");
    if (herr == swapk::KERR_CAPACITY) return c->fail(SWAP_ECAPACITY, "Ni_max exceeded by new ions");
    if (herr == swapk::KERR_MOVE)
      return c->fail(SWAP_EMOVE,
                     "a particle's half move spanned the grid less two cells, or more than 65536 particles "
                     "moved more than one cell per axis in one step");
    if (herr == swapk::KERR_WAIT) return c->fail(SWAP_EWAIT, "a particle chunk copy did not complete within its wait limit");
    if (herr == swapk::KERR_RANGE)
      return c->fail(SWAP_ENONFINITE,
                     "a moment sum is not finite or beyond the exact sums' range (|sum| < 2^15)");
    return c->fail(SWAP_ECUDA, "device error flag " + std::to_string(herr));
  }
  return SWAP_OK;
}

// New ions staged ahead on the second stream (valid: the counts below hold).
struct PreStaged {
  bool valid = false;
  long long n_host = 0, n_max = 0;
  const int64_t* n_dev = nullptr;
};
static int sort_step(swap_ctx* c, F32State* s, long long src_step, bool prepared = false,
                     const PreStaged* pre = nullptr, bool on_side = false);

// ---------------------------------------------------------------------------

extern "C" int swap_f32_begin(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  TRY(c->begin());
  if (!c->h_xp || !c->h_b1) return c->fail(SWAP_EINVAL, "swap_bind_particles and swap_bind_fields are required");
  const int nx = c->dims.nx, ny = c->dims.ny, nz = c->dims.nz;
  const int ncx = nx - 2, ncy = ny - 2, ncz = nz - 2;
  if (ncx % 4 || ncy % 4 || ncz % 4 || ncx < 8 || ncy < 8 || ncz < 8 || ncx > 1024 || ncy > 1024 || ncz > 1024)
    return c->fail(SWAP_EINVAL, "the FP32 form needs 8..1024 physical cells per axis, multiples of 4");
  // uniform spacing per axis
  auto uniform = [](const std::vector<double>& q) {
    const double d = q[1] - q[0];
    for (std::size_t i = 1; i < q.size(); ++i)
      if (std::fabs((q[i] - q[i - 1]) - d) > 1e-9 * std::fabs(d)) return false;
    return true;
  };
  if (!uniform(c->h_qx) || !uniform(c->h_qy) || !uniform(c->h_qz))
    return c->fail(SWAP_EINVAL, "the FP32 form needs a uniform grid on every axis");
  auto* s = new F32State();
  if (F32State* old = f32(c)) {  // reuse its device blocks (same grid: same sizes, same order)
    for (std::size_t q = 0; q < old->owned.size(); ++q) s->pool.emplace_back(old->owned[q], old->owned_bytes[q]);
    for (std::size_t q = old->pool_next; q < old->pool.size(); ++q) s->pool.push_back(old->pool[q]);
    old->owned.clear();
    old->pool.clear();
    swap_f32_free(c);
  }
  c->f32_state = s;
  G32& g = s->g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.ncx = ncx; g.ncy = ncy; g.ncz = ncz;
  g.nbx = ncx / 4; g.nby = ncy / 4; g.nbz = ncz / 4;
  g.C = (long long)nx * ny * nz;
  g.nbricks = (long long)g.nbx * g.nby * g.nbz;
  g.nkeys = g.nbricks * BCELLS;
  const double dx = c->h_qx[1] - c->h_qx[0], dy = c->h_qy[1] - c->h_qy[0], dz = c->h_qz[1] - c->h_qz[0];
  g.dx = (float)dx; g.dy = (float)dy; g.dz = (float)dz;
  g.inv_dx = (float)(1.0 / dx); g.inv_dy = (float)(1.0 / dy); g.inv_dz = (float)(1.0 / dz);
  g.qx1 = c->h_qx[0]; g.qy1 = c->h_qy[0]; g.qz1 = c->h_qz[0];

  // bound FP64 state: the particle vectors are read where they are current
  // (in the caller's memory in host-direct mode), the rest on the device
  double *xp, *vp, *vp1, *mrat, *beta_p, *b0, *b1, *b12, *npd, *nud;
  bool direct[3];
  TRY(c->use_host(c->h_xp, Access::In, &xp, &direct[0]));
  TRY(c->use_host(c->h_vp, Access::In, &vp, &direct[1]));
  TRY(c->use_host(c->h_vp1, Access::In, &vp1, &direct[2]));
  TRY(c->use(c->h_mrat, Access::In, &mrat));
  TRY(c->use(c->h_beta_p, Access::In, &beta_p));
  TRY(c->use(c->h_b0, Access::In, &b0));
  TRY(c->use(c->h_b1, Access::In, &b1));
  TRY(c->use(c->h_b12, Access::In, &b12));
  TRY(c->use(c->h_np, Access::In, &npd));
  TRY(c->use(c->h_nu, Access::In, &nud));
  const long long N = c->ntot(), NM = c->dims.ni_max;
  s->N = N;

  // b0 must be uniform for the FP32 stencils (curl b0 = 0): checked on the device
  double hb0v[3];
  {
    int* flag = s->alloc<int>(1);
    if (!flag) return c->fail(SWAP_ECUDA, "allocation");
    CU(cudaMemsetAsync(flag, 0, sizeof(int), c->st));
    CU(not_uniform(g.C, b0, flag, c->st));
    int hf = 0;
    CU(cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    for (int m = 0; m < 3; ++m)
      CU(cudaMemcpyAsync(&hb0v[m], b0 + m * g.C, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    if (hf) return c->fail(SWAP_EINVAL, "the FP32 form needs a uniform b0");
  }
  const float hb0c[3] = {(float)hb0v[0], (float)hb0v[1], (float)hb0v[2]};

  // species table from the (mrat, beta_p) pairs present, in order of first
  // appearance: found on the device, one pass per species (the first
  // particle whose pair is not yet in the table adds it)
  std::vector<double> tm, tb;
  // sized by ni_max, like every block here, so that the next swap_f32_begin
  // on this grid finds the same sizes in the same order and allocates nothing
  uint8_t* spid = s->alloc<uint8_t>((std::size_t)std::max<long long>(NM, 1));
  double* tabm = s->tabm = s->alloc<double>(MAX_SPECIES);
  double* tabb = s->tabb = s->alloc<double>(MAX_SPECIES);
  int* miss = s->alloc<int>(1);
  if (!spid || !tabm || !tabb || !miss) return c->fail(SWAP_ECUDA, "allocation");
  for (long long first = 0; N > 0 && first >= 0;) {
    double pr[2];
    CU(cudaMemcpyAsync(&pr[0], mrat + first, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CU(cudaMemcpyAsync(&pr[1], beta_p + first, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    if (tm.size() == MAX_SPECIES) return c->fail(SWAP_ECAPACITY, "more than 16 (mrat, beta_p) species");
    tm.push_back(pr[0]);
    tb.push_back(pr[1]);
    CU(cudaMemcpyAsync(tabm, tm.data(), tm.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(tabb, tb.data(), tb.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemsetAsync(miss, 0x7f, sizeof(int), c->st));  // INT_MAX-like: no miss
    CU(assign_species(N, mrat, beta_p, tabm, tabb, (int)tm.size(), spid, miss, c->st));
    int hm = 0;
    CU(cudaMemcpyAsync(&hm, miss, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    first = hm == 0x7f7f7f7f ? -1 : hm;
  }
  if (tm.empty()) { tm.push_back(1.0); tb.push_back(1.0); }
  // species the sources create: ring ions, inflow, cloud ions, and the heavy
  // twin (mrat_heavy, same beta_p) of every species for charge exchange
  s->src_on = srcops::any_rule(c);
  s->x_open = srcops::x_open(c);
  auto species = [&](double m, double bp) -> int {
    for (std::size_t q = 0; q < tm.size(); ++q)
      if (tm[q] == m && tb[q] == bp) return (int)q;
    tm.push_back(m);
    tb.push_back(bp);
    return (int)tm.size() - 1;
  };
  if (s->src_on) {
    const swap_sources& q = c->srcs;
    if (q.ndot > 0) s->stage.sp_ion = (uint8_t)species(q.mrat_pu, q.beta_pu);
    if (q.x_open) s->stage.sp_inflow = (uint8_t)species(1.0, 1.0);
    if (q.nu_ion > 0) s->stage.sp_cloud = (uint8_t)species(q.mrat_heavy, q.beta_heavy);
  }
  for (int q = 0; q < MAX_SPECIES; ++q) s->heavy_of[q] = (uint8_t)q;
  if (s->src_on && c->srcs.cx_a > 0)
    for (std::size_t q = 0, n0 = tm.size(); q < n0; ++q) s->heavy_of[q] = (uint8_t)species(c->srcs.mrat_heavy, tb[q]);
  if (tm.size() > (std::size_t)MAX_SPECIES) return c->fail(SWAP_ECAPACITY, "more than 16 (mrat, beta_p) species");
  s->sp.n = (int)tm.size();
  for (int q = 0; q < s->sp.n; ++q) {
    s->sp.mrat[q] = (float)tm[q];
    s->sp.qw[q] = (float)(1.0 / (dx * dy * dz * c->prm.beta * tb[q]));
  }

  // allocations
  const std::size_t NMs = (std::size_t)std::max<long long>(NM, 1);
  // the passes copy whole 128-ion chunks from 16-aligned starts: pad the arrays
  const std::size_t NMp = NMs + PASS_PAD;
  for (int k = 0; k < 2; ++k) {
    Part& p = s->buf[k];
    p.cell = s->alloc<int32_t>(NMp);
    p.ox = s->alloc<float>(NMp); p.oy = s->alloc<float>(NMp); p.oz = s->alloc<float>(NMp);
    p.vx = s->alloc<float>(NMp); p.vy = s->alloc<float>(NMp); p.vz = s->alloc<float>(NMp);
    p.wx = s->alloc<float>(NMp); p.wy = s->alloc<float>(NMp); p.wz = s->alloc<float>(NMp);
    p.sp = s->alloc<uint8_t>(NMp);
    if (!p.cell || !p.ox || !p.oy || !p.oz || !p.vx || !p.vy || !p.vz || !p.wx || !p.wy || !p.wz || !p.sp)
      return c->fail(SWAP_ECUDA, "FP32 particle allocation failed");
  }
  const std::size_t C = (std::size_t)g.C, nk = (std::size_t)g.nkeys;
  s->start = s->alloc<int64_t>(nk + 1);
  s->start_new = s->alloc<int64_t>(nk + 1);
  s->count = s->alloc<int64_t>(nk + 1);
  s->sums = s->alloc<int64_t>(nk / 1024 + 16);
  s->dirrank = s->alloc<uint32_t>(NMs);
  s->dep = s->alloc<uint16_t>(nk * NDIR);
  s->pre = s->alloc<uint16_t>(nk * NDIR);
  s->order = s->alloc<uint8_t>(BCELLS * NDIR);
  {
    uint8_t ord[BCELLS * NDIR];
    sort_order_table(ord);
    if (!s->order || cudaMemcpy(s->order, ord, sizeof(ord), cudaMemcpyHostToDevice) != cudaSuccess)
      return c->fail(SWAP_ECUDA, "sort order table");
  }
  s->partial = s->alloc<unsigned long long>((std::size_t)g.nbricks * 4 * TNODES);
  s->far.idx = s->alloc<long long>(FAR_CAP);
  s->far.key = s->alloc<long long>(FAR_CAP);
  s->far.dcell = s->alloc<int32_t>(FAR_CAP);
  s->far.o = s->alloc<float>(3 * (std::size_t)FAR_CAP);
  s->far.q = s->alloc<float>(4 * (std::size_t)FAR_CAP);
  s->far.n = s->alloc<int>(1);
  s->far.total = s->alloc<unsigned long long>(1);
  s->kit = s->alloc<float4>(2 * (std::size_t)ncx * ncy * ncz);
  s->gp = (float)c->prm.grad_pe;
  if (s->gp != 0.0f) {
    s->gpf = s->alloc<float>(3 * (std::size_t)C);
    s->kitg = s->alloc<float4>((std::size_t)ncx * ncy * ncz);
    if (!s->gpf || !s->kitg) return c->fail(SWAP_ECUDA, "FP32 grid allocation failed");
    CU(cudaMemsetAsync(s->gpf, 0, 3 * (std::size_t)C * sizeof(float), c->st));
  }
  // np and the velocity sums S in one block (S 128-byte aligned after np), so
  // that one exchange covers a deposit's node sums.  Zeroed once: the gap and
  // S's ghost nodes are never written, and stay zero through the exchanges.
  const std::size_t npad = ((std::size_t)C + 31) / 32 * 32;
  float* nps = s->alloc<float>(npad + 3 * C);
  s->np = nps;
  s->S = nps ? nps + npad : nullptr;
  s->np_span = (long long)(npad + 3 * C);
  if (nps) CU(cudaMemsetAsync(nps, 0, (npad + 3 * C) * sizeof(float), c->st));
  s->up = s->alloc<float>(3 * C);
  s->aj = s->alloc<float>(3 * C); s->ct = s->alloc<float>(3 * C); s->E = s->alloc<float>(3 * C);
  s->nu = s->alloc<float>(C);
  s->db1 = s->alloc<float>(3 * C); s->db1p2 = s->alloc<float>(3 * C); s->dbtp1 = s->alloc<float>(3 * C);
  s->b0 = s->alloc<double>(3 * C);
  for (F32State::DF* d : {&s->b1, &s->b12, &s->b1p2}) {
    d->h = s->alloc<float>(3 * C);
    d->l = s->alloc<float>(3 * C);
  }
  s->b0c = s->alloc<float>(4);
  s->d_min = s->alloc<float>(4);
  s->dtn = s->alloc<float>(C);
  s->acc = s->alloc<double>(4);
  if (!s->start || !s->start_new || !s->count || !s->sums || !s->dirrank || !s->dep || !s->pre || !s->partial || !s->kit ||
      !s->np || !s->S || !s->up || !s->aj || !s->ct || !s->E || !s->nu || !s->db1 || !s->db1p2 || !s->dbtp1 ||
      !s->b0 || !s->b1.l || !s->b12.l || !s->b1p2.l || !s->b0c || !s->d_min || !s->acc || !s->dtn || !s->far.idx ||
      !s->far.key || !s->far.dcell || !s->far.o || !s->far.q || !s->far.n || !s->far.total)
    return c->fail(SWAP_ECUDA, "FP32 grid allocation failed");
  CU(cudaMemsetAsync(s->far.n, 0, sizeof(int), c->st));
  CU(cudaMemsetAsync(s->far.total, 0, sizeof(unsigned long long), c->st));
  CU(cudaMemsetAsync(s->np, 0, C * sizeof(float), c->st));
  for (void* p : {(void*)s->S, (void*)s->up, (void*)s->aj, (void*)s->ct, (void*)s->E})
    CU(cudaMemsetAsync(p, 0, 3 * C * sizeof(float), c->st));
  CU(cudaMemcpyAsync(s->b0c, hb0c, 3 * sizeof(float), cudaMemcpyHostToDevice, c->st));

  // fields: FP64 levels copied, dB = B - b0 in FP32, nu in FP32
  const std::size_t b3 = 3 * C * sizeof(double);
  CU(cudaMemcpyAsync(s->b0, b0, b3, cudaMemcpyDeviceToDevice, c->st));
  CU(split_df(3 * g.C, b1, s->b1.h, s->b1.l, c->st));
  CU(split_df(3 * g.C, b12, s->b12.h, s->b12.l, c->st));
  CU(grid_f64_to_f32(3 * g.C, b1, b0, s->db1, c->st));
  CU(grid_f64_to_f32(g.C, nud, nullptr, s->nu, c->st));

  // particles: convert, assign species, sort by key (host counting sort, once)
  Part& tmp = s->buf[1];
  CU(from_f64(g, N, NM, xp, vp, vp1, mrat, beta_p, s->sp, tmp, c->d_err, c->st));
  for (bool d : direct)
    if (d) c->h2d_bytes += 24 * N;
  if (N > 0) CU(cudaMemcpyAsync(tmp.sp, spid, (std::size_t)N, cudaMemcpyDeviceToDevice, c->st));
  // the full table (with the sources' species) for the conversion back
  CU(cudaMemcpyAsync(tabm, tm.data(), tm.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CU(cudaMemcpyAsync(tabb, tb.data(), tb.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
  TRY(check_err(c));
  int32_t* keys = reinterpret_cast<int32_t*>(s->dirrank);
  CU(keys_of(g, N, tmp.cell, keys, c->st));
  int* unsorted = s->alloc<int>(1);
  if (!unsorted) return c->fail(SWAP_ECUDA, "allocation");
  CU(cudaMemsetAsync(unsorted, 0, sizeof(int), c->st));
  CU(sorted_hist(N, keys, g.nkeys, unsorted, s->count, c->st));
  int hun = 0;
  CU(cudaMemcpyAsync(&hun, unsorted, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  if (hun == 2) return c->fail(SWAP_EDOMAIN, "a particle lies outside the grid");
  if (hun == 0) {
    // already in key order (the product loader and swap_f32_end give that):
    // starts by scan, particles used as they are
    CU(scan_exclusive(s->count, s->start, g.nkeys, s->sums, c->st));
    std::swap(s->buf[0], s->buf[1]);
  } else {
    // arbitrary order: one stable counting sort on the host
    std::vector<int32_t> hk((std::size_t)N);
    CU(cudaMemcpy(hk.data(), keys, N * sizeof(int32_t), cudaMemcpyDeviceToHost));
    std::vector<int64_t> cnt(nk + 1, 0), perm((std::size_t)N);
    for (long long l = 0; l < N; ++l) cnt[(std::size_t)hk[l] + 1]++;
    for (std::size_t k = 0; k < nk; ++k) cnt[k + 1] += cnt[k];
    CU(cudaMemcpy(s->start, cnt.data(), (nk + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    for (long long l = 0; l < N; ++l) perm[(std::size_t)cnt[(std::size_t)hk[l]]++] = l;
    void* pbuf = nullptr;
    CU(cudaMalloc(&pbuf, (std::size_t)std::max<long long>(N, 1) * sizeof(int64_t)));
    cudaError_t e = cudaMemcpy(pbuf, perm.data(), N * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = gather_perm(N, static_cast<int64_t*>(pbuf), tmp, s->buf[0], c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cudaFree(pbuf);
    if (e != cudaSuccess) return c->cuda_fail(e, "initial sort");
  }
  s->cur = 0;
  TRY(check_err(c));
  if (s->src_on) TRY(sort_step(c, s, c->src_step));  // the sources of the first step
  return check_err(c);
}

// Deposit finish: node sums -> np (+ghosts) and up (maind.f:386-387 etc.).
static int finish_deposit(swap_ctx* c, F32State* s, int pass, int nq) {
  KL("f32_node_sum", node_sum(s->g, pass, s->partial, nq, s->exact, s->np, s->S, c->st));
  // the rank sum of the raw node sums (MPI_ALLREDUCE, gutsp.f:1503,1812-1822);
  // pass 2 deposits no density
  if (nq == 4) TRY(c->exchange(s->np, s->np_span, 4));
  else TRY(c->exchange(s->S, 3 * s->g.C, 4));
  KL("f32_ct_up", ct_and_up(s->g, s->np, s->S, s->up, c->st));
  return SWAP_OK;
}

static int subcycles(swap_ctx* c, F32State* s, float* e_acc = nullptr) {
  const G32& g = s->g;
  double dtsub = c->prm.dt / (double)c->prm.ntsub;  // maind.f:420-421
  double ntf = (double)c->prm.ntsub;
  // check_time_step (gutsf.f:1776-1822): per-node Courant times; when even
  // the smallest leaves dtsub alone nothing changes, otherwise the
  // reference's ordered halving (once per violating node, k innermost) is
  // replayed on the host from the node values.
  KL("f32_courant", courant_min(g, s->db1, s->b0c, s->np, (float)c->prm.alpha, g.dx, s->dtn, s->d_min, c->st));
  float mn = 0;
  int herr = 0;
  CU(cudaMemcpyAsync(&mn, s->d_min, sizeof(float), cudaMemcpyDeviceToHost, c->st));
  CU(cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  // a pass that failed (a wait that gave up, an ion outside the grid) ends
  // the step here, before its moments reach the fields
  if (herr) return check_err(c);
  if ((double)mn <= 2.0 * dtsub) {
    std::vector<float> h((std::size_t)g.C);
    CU(cudaMemcpy(h.data(), s->dtn, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int i = 0; i < g.nx; ++i)
      for (int j = 0; j < g.ny; ++j)
        for (int k = 0; k < g.nz; ++k)
          if ((double)h[(std::size_t)i + (std::size_t)g.nx * (j + (std::size_t)g.ny * k)] <= 2.0 * dtsub) {
            dtsub /= 2.0;
            ntf *= 2.0;
          }
    if (ntf > 1.0e6) return c->fail(SWAP_ESUBCYCLE, "subcycle count overflow in check_time_step");
  }
  s->last_dtsub = dtsub;
  s->last_ntf = ntf;
  const int n = (int)ntf;
  const float alpha = (float)c->prm.alpha;
  for (int it = 0; it < n; ++it) {
    const bool last = it == n - 1;
    // predictor: curlB (maind.f:430) and predict_B with its get_E (maind.f:457), plus dB at m+1/2
    KL("f32_aj_ct_pred", aj_ct(g, false, s->db1, s->np, s->up, s->b0c, alpha, s->aj, s->ct, c->st));
    KL("f32_bstep_pred", b_step(g, true, false, s->ct, s->nu, s->aj, s->gpf, s->b12.h, s->b12.l, 2.0 * dtsub, s->b0c,
                                s->b1p2.h, s->b1p2.l, s->db1p2, s->db1, s->dbtp1, s->E, nullptr, c->st));
    // corrector: correct_B (maind.f:462) with its curlB and get_Ep1 at m+1/2
    KL("f32_aj_ct_corr", aj_ct(g, true, s->dbtp1, s->np, s->up, s->b0c, alpha, s->aj, s->ct, c->st));
    KL("f32_bstep_corr", b_step(g, false, last, s->ct, s->nu, s->aj, s->gpf, s->b1.h, s->b1.l, dtsub, s->b0c, s->b1p2.h,
                                s->b1p2.l, s->db1p2, nullptr, nullptr, s->E, e_acc, c->st));
    // f_update_tlev (gutsf.f:10-35): b12 <- b1, b1 <- b1p2 (bt = b1)
    std::swap(s->b12, s->b1);
    std::swap(s->b1, s->b1p2);
    std::swap(s->db1, s->db1p2);
  }
  return SWAP_OK;
}

// The stable incremental counting sort after each step (particles moved at
// most one cell per axis since the last sort).  Removed ions are dropped;
// with src_step >= 0 the new ions of that step's sources are placed after the
// arrivals of their cell, flagged fresh.  prepared: pass 3 already wrote the
// directions, ranks and per-key counts.
static int sort_body(swap_ctx* c, F32State* s, long long src_step, bool prepared, const PreStaged* pre,
                     bool on_side);
static int side_stream(swap_ctx* c, F32State* s);
// on_side: the sort goes to the second stream after the main stream's work
// so far and the staging; sort_join (after the field step) waits for it and
// takes the new count.
static int sort_step(swap_ctx* c, F32State* s, long long src_step, bool prepared, const PreStaged* pre,
                     bool on_side) {
  if (!on_side) return sort_body(c, s, src_step, prepared, pre, false);
  TRY(side_stream(c, s));
  if (!(pre && pre->valid)) {  // no staging ahead of it: order after the main stream here
    CU(cudaEventRecord(s->ev_main, c->st));
    CU(cudaStreamWaitEvent(s->side, s->ev_main, 0));
  }
  cudaStream_t main = c->st;
  c->st = s->side;
  const int r = sort_body(c, s, src_step, prepared, pre, true);
  c->st = main;
  if (r) return r;
  CU(cudaEventRecord(s->ev_sort, s->side));
  s->sort_pending = true;
  return SWAP_OK;
}

static int sort_join(swap_ctx* c, F32State* s) {
  if (!s->sort_pending) return SWAP_OK;
  s->sort_pending = false;
  CU(cudaStreamWaitEvent(c->st, s->ev_sort, 0));
  if (s->src_on) {
    CU(cudaEventSynchronize(s->ev_sort));
    const int64_t n = *s->h_n;
    if (n > c->dims.ni_max) return c->fail(SWAP_ECAPACITY, "Ni_max exceeded by new ions");
    s->N = n;
  }
  return SWAP_OK;
}

static int sort_body(swap_ctx* c, F32State* s, long long src_step, bool prepared, const PreStaged* pre,
                     bool on_side) {
  const G32& g = s->g;
  Part& a = s->buf[s->cur];
  Part& b = s->buf[1 - s->cur];
  long long n_host = 0, n_max = 0;
  const int64_t* n_dev = nullptr;
  if (pre && pre->valid) {
    if (!on_side) CU(cudaStreamWaitEvent(c->st, s->ev_side, 0));
    n_host = pre->n_host;
    n_max = pre->n_max;
    n_dev = pre->n_dev;
  } else if (src_step >= 0 && s->src_on) {
    TRY(srcops::f32_stage(c, g, s->stage, src_step, &n_host, &n_dev, &n_max));
  }
  const bool staged = n_max > 0;
  const long long cap = c->dims.ni_max;
  if (!prepared) KL("f32_sort_prep", sort_prep(g, s->start, a.cell, s->dirrank, s->dep, c->d_err, c->st));
  KL("f32_sort_count", sort_count(g, s->dep, staged ? s->stage.ncount : nullptr, s->order, s->count, s->pre,
                                  c->d_err, c->st));
  if (prepared) KL("f32_far_count", far_count(s->far, s->count, c->st));
  KLN("f32_sort_scan", 3, scan_exclusive(s->count, s->start_new, g.nkeys, s->sums, c->st));
  KL("f32_sort_scatter", sort_scatter(g, s->N, cap, a.cell, s->dirrank, s->pre, s->start_new, a, b, c->d_err, c->st));
  if (prepared)
    KL("f32_far_scatter", far_scatter(g, s->far, staged ? s->stage.ncount : nullptr, s->start_new, a, b, cap,
                                      c->d_err, c->st));
  if (staged)
    KL("f32_new_scatter", new_scatter(g, n_host, n_dev, n_max, s->stage.part, s->stage.key, s->stage.rank,
                                      s->stage.ncount, s->start_new, b, cap, c->d_err, c->st));
  std::swap(s->start, s->start_new);
  s->cur = 1 - s->cur;
  if (on_side) {  // the count, for sort_join
    if (s->src_on) CU(cudaMemcpyAsync(s->h_n, s->start + g.nkeys, sizeof(int64_t), cudaMemcpyDeviceToHost, c->st));
    return SWAP_OK;
  }
  if (s->src_on) {  // the count changed: the host needs it for the next launches
    int64_t n = 0;
    CU(cudaMemcpyAsync(&n, s->start + g.nkeys, sizeof(int64_t), cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    if (n > cap) return c->fail(SWAP_ECAPACITY, "Ni_max exceeded by new ions");
    s->N = n;
  }
  return SWAP_OK;
}

// Step parameters of the particle passes, with the sources and sinks that
// act inside them (open-x outflow, res_chex at the end of the step).
static StepParams step_params(swap_ctx* c, F32State* s) {
  StepParams p{};
  p.dt = (float)c->prm.dt;
  p.x_open = s->x_open ? 1 : 0;
  const swap_sources& q = c->srcs;
  p.chex = (s->src_on && q.cx_a > 0) ? 1 : 0;
  p.chex_step = c->src_step;  // the ion step being taken
  p.seed = q.seed;
  p.cx_a = (float)q.cx_a;
  p.cx_b = (float)q.cx_b;
  p.cloud_N0 = (float)q.cloud_N0;
  p.inv_r0sq = q.cloud_r0 > 0 ? (float)(1.0 / (q.cloud_r0 * q.cloud_r0)) : 0.f;
  p.cloud_x = (float)q.cloud_x;
  p.cloud_y = (float)q.cloud_y;
  p.cloud_z = (float)q.cloud_z;
  for (int k = 0; k < MAX_SPECIES; ++k) p.heavy_of[k] = s->heavy_of[k];
  p.chex_count = p.chex ? srcops::counters(c) + 1 : nullptr;
  p.wait_polls = c->wait_polls;
  return p;
}

// Buffers of the surrogate's field step (allocated on first use).
static int sur_buffers(swap_ctx* c, F32State* s) {
  if (s->e_sum) return SWAP_OK;
  const std::size_t C = (std::size_t)s->g.C, V = (std::size_t)s->g.ncx * s->g.ncy * s->g.ncz;
  s->e_sum = s->alloc<float>(3 * C);
  s->vin = s->alloc<float>((std::size_t)SUR_NIN * V);
  s->ve = s->alloc<float>(3 * V);
  s->jh = s->alloc<float>(3 * C);
  s->jl = s->alloc<float>(3 * C);
  s->jdb = s->alloc<float>(3 * C);
  s->jacc = s->alloc<double>(4);
  if (!s->e_sum || !s->vin || !s->ve || !s->jh || !s->jl || !s->jdb || !s->jacc)
    return c->fail(SWAP_ECUDA, "surrogate buffers");
  return SWAP_OK;
}

// The network's inputs at the start of the subcycles: B, u_p, n_p, p_e and
// E0, the plain E from the first predictor's aj and ct (curlB and the cross
// product of get_E, maind.f:430,457).
static int sur_inputs(swap_ctx* c, F32State* s) {
  const G32& g = s->g;
  KL("f32_sur_inputs", aj_ct(g, false, s->db1, s->np, s->up, s->b0c, (float)c->prm.alpha, s->aj, s->ct, c->st));
  KL("f32_sur_inputs",
     grid_to_voxels(g, s->db1, s->b0c, s->up, s->np, 1.0f, s->ct, s->aj, s->nu, s->gpf, s->b1.h, s->b1.l, s->b12.h,
                    s->b12.l, s->vin, c->st));
  return SWAP_OK;
}

// The network's field advance from the state at the start of the subcycles:
// E = E0 + the predicted correction per node, B into (oh, ol) and its dB
// into odb as B - dt curl E.  The inputs are in s->vin.
static int sur_predict(swap_ctx* c, F32State* s, float* oh, float* ol, float* odb) {
  const G32& g = s->g;
  {
    ProfScope ps(c, "f32_sur_net", c->st, 6);  // the network's own launches (normalise, 4 convs, scale)
    if (surr::predict_e(s->sur, g.ncx, g.ncy, g.ncz, s->vin, s->ve, c->st))
      return c->fail(SWAP_EINVAL, std::string("surrogate: ") + surr::last_error(s->sur));
  }
  KL("f32_sur_E", voxels_to_grid(g, s->ve, s->vin, s->E, c->st));
  KL("f32_sur_B", b_step_given_e(g, s->E, s->b1.h, s->b1.l, c->prm.dt, s->b0c, oh, ol, odb, c->st));
  return SWAP_OK;
}

// maind.f:420-476: the plain subcycles, or the network in their place.  With
// a network attached every sur_every-th step is judged: both run, the plain
// result is kept, and a B error above the bound switches the network off
// until a judged step passes.  Collecting: plain subcycles, and the pair
// (inputs, mean corrector E) joins the network's training set.
static int field_step(swap_ctx* c, F32State* s) {
  const G32& g = s->g;
  const bool judge = s->sur && s->sur_step % s->sur_every == 0;
  const bool use_net = s->sur && !judge && !s->sur_off;
  if (s->sur) ++s->sur_step;
  if (use_net) {
    TRY(sur_buffers(c, s));
    TRY(sur_inputs(c, s));
    TRY(sur_predict(c, s, s->b1p2.h, s->b1p2.l, s->db1p2));
    // b12: B one subcycle before the end of the step, the leapfrog base of the next predictor
    KL("f32_sur_B", df_lerp(g, s->b1p2.h, s->b1p2.l, s->b1.h, 1.0f / (float)c->prm.ntsub, s->b12.h, s->b12.l,
                            c->st));
    std::swap(s->b1, s->b1p2);
    std::swap(s->db1, s->db1p2);
    ++s->sur_used;
    return SWAP_OK;
  }
  const bool collect = s->collect != nullptr;
  if (collect || judge) {
    TRY(sur_buffers(c, s));
    CU(cudaMemsetAsync(s->e_sum, 0, 3 * (std::size_t)g.C * sizeof(float), c->st));
  }
  if (collect || judge) TRY(sur_inputs(c, s));
  if (judge) TRY(sur_predict(c, s, s->jh, s->jl, s->jdb));
  TRY(subcycles(c, s, (collect || judge) ? s->e_sum : nullptr));
  if (collect) {
    KL("f32_sur_target", grid_e_to_voxels(g, s->e_sum, (float)(1.0 / s->last_ntf), s->vin, s->ve, c->st));
    if (surr::add_sample(s->collect, g.ncx, g.ncy, g.ncz, s->vin, s->ve, c->st))
      return c->fail(SWAP_EINVAL, std::string("surrogate: ") + surr::last_error(s->collect));
  }
  if (judge) {
    double h[3];
    KL("f32_sur_judge", judge_sums(g, s->jh, s->jl, s->b1.h, s->b1.l, s->b0c, s->jacc, c->st));
    CU(cudaMemcpyAsync(h, s->jacc, sizeof(h), cudaMemcpyDeviceToHost, c->st));
    CU(cudaStreamSynchronize(c->st));
    s->sur_err_b = std::sqrt(h[0] / std::max(h[1], 1e-300));
    s->sur_err_db = std::sqrt(h[0] / std::max(h[2], 1e-300));
    ++s->sur_judged;
    s->sur_off = s->sur_err_b > s->sur_bound || (s->sur_bound_db > 0 && s->sur_err_db > s->sur_bound_db);
    if (s->sur_off) ++s->sur_fallbacks;
  }
  return SWAP_OK;
}

// The second stream, its events and the pinned count, made once.
static int side_stream(swap_ctx* c, F32State* s) {
  if (s->side) return SWAP_OK;
  CU(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&s->ev_main, cudaEventDisableTiming));
  CU(cudaEventCreateWithFlags(&s->ev_side, cudaEventDisableTiming));
  CU(cudaEventCreateWithFlags(&s->ev_sort, cudaEventDisableTiming));
  CU(cudaMallocHost(&s->h_n, sizeof(int64_t)));
  return SWAP_OK;
}

// Stage the new ions of step m on the second stream, after the main stream's
// work so far (the last sort read the previous staging's buffers).
static int stage_ahead(swap_ctx* c, F32State* s, long long m, PreStaged* pre) {
  TRY(side_stream(c, s));
  CU(cudaEventRecord(s->ev_main, c->st));
  CU(cudaStreamWaitEvent(s->side, s->ev_main, 0));
  cudaStream_t main = c->st;
  c->st = s->side;  // the staging's launches and profile scopes go to the second stream
  const int r = srcops::f32_stage(c, s->g, s->stage, m, &pre->n_host, &pre->n_dev, &pre->n_max);
  c->st = main;
  if (r) return r;
  CU(cudaEventRecord(s->ev_side, s->side));
  pre->valid = true;
  return SWAP_OK;
}

static int one_step_body(swap_ctx* c, F32State* s);
// A step; after a failure the second stream's work (a sort already queued)
// is drained, so that nothing of the step runs on when the caller goes on.
static int one_step(swap_ctx* c, F32State* s) {
  const int r = one_step_body(c, s);
  if (r && s->sort_pending) {
    cudaStreamSynchronize(s->side);
    s->sort_pending = false;
  }
  return r;
}

static int one_step_body(swap_ctx* c, F32State* s) {
  const G32& g = s->g;
  const StepParams sp = step_params(c, s);
  const Part& p = s->buf[s->cur];
  KL("f32_P1", pass(1, g, p, s->sp, sp, s->start, s->kit, s->partial, nullptr, nullptr, c->d_err, s->exact, c->st));  // :385-387,399
  TRY(finish_deposit(c, s, 1, 4));
  KL("f32_curlB", curlB32(g, s->db1, s->np, (float)c->prm.alpha, s->aj, c->st));  // :395
  KL("f32_kit", build_kit(g, s->aj, s->up, s->db1, s->b0c, s->np, s->gp, s->kit, s->kitg, c->st));  // :398, :183-184
  KL("f32_P2", pass(2, g, p, s->sp, sp, s->start, s->kit, s->partial, nullptr, nullptr, c->d_err, s->exact, c->st,
                    nullptr, s->kitg));  // :400-402
  TRY(finish_deposit(c, s, 2, 3));
  KL("f32_kit", build_kit(g, s->aj, s->up, s->db1, s->b0c, s->np, s->gp, s->kit, s->kitg, c->st));  // :404
  // :404-413, the final half move of :479 and res_chex; prepares the sort
  CU(cudaMemsetAsync(s->far.n, 0, sizeof(int), c->st));
  KL("f32_P3", pass(3, g, p, s->sp, sp, s->start, s->kit, s->partial, s->dirrank, s->dep, c->d_err, s->exact,
                    c->st, &s->far, s->kitg));
  KL("f32_far_deposit", far_deposit(g, s->far, s->partial, s->exact, c->d_err, c->st));
  {  // pass 3 wrote the new v into the vp1 arrays and left the old v (the new vp1) in place
    Part& q = s->buf[s->cur];
    std::swap(q.vx, q.wx);
    std::swap(q.vy, q.wy);
    std::swap(q.vz, q.wz);
  }
  PreStaged pre;
  if (s->src_on) TRY(stage_ahead(c, s, c->src_step + 1, &pre));  // the sources of the next step
  // the sort on the second stream, beside the moments' sums and the field
  // subcycles: it reads pass 3's outputs and the staging, they the grids
  TRY(sort_step(c, s, c->src_step + 1, true, &pre, true));
  TRY(finish_deposit(c, s, 3, 4));
  if (s->gpf) KL("f32_gpe", gpe_faces(g, s->np, s->gp, s->gpf, c->st));  // E's pressure term at the new np
  TRY(field_step(c, s));                                                          // :420-476
  TRY(sort_join(c, s));
  if (c->have_srcs) c->src_step++;
  return SWAP_OK;
}

extern "C" int swap_f32_run(swap_ctx* c, int32_t nsteps) {
  if (!c) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  if (s->ended && s->src_on) return c->fail(SWAP_EINVAL, "call swap_f32_begin again after swap_f32_end");
  for (int k = 0; k < nsteps; ++k) TRY(one_step(c, s));
  return check_err(c);
}

extern "C" int swap_f32_end(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  TRY(c->begin());
  // the particle arrays straight into the caller's memory in host-direct
  // mode, the fields into the device copies
  double *xp, *vp, *vp1, *b1, *b12, *b1p2, *bt, *npd, *upd, *Ed, *ajd;
  bool direct[5];
  TRY(c->use_host(c->h_xp, Access::Out, &xp, &direct[0]));
  TRY(c->use_host(c->h_vp, Access::Out, &vp, &direct[1]));
  TRY(c->use_host(c->h_vp1, Access::Out, &vp1, &direct[2]));
  TRY(c->use(c->h_b1, Access::Out, &b1));
  TRY(c->use(c->h_b12, Access::Out, &b12));
  TRY(c->use(c->h_b1p2, Access::Out, &b1p2));
  TRY(c->use(c->h_bt, Access::Out, &bt));
  TRY(c->use(c->h_np, Access::Out, &npd));
  TRY(c->use(c->h_up, Access::Out, &upd));
  TRY(c->use(c->h_E, Access::Out, &Ed));
  TRY(c->use(c->h_aj, Access::Out, &ajd));
  double *mratd, *bpd;
  TRY(c->use_host(c->h_mrat, Access::Out, &mratd, &direct[3]));
  TRY(c->use_host(c->h_beta_p, Access::Out, &bpd, &direct[4]));
  const G32& g = s->g;
  long long n_out = s->N;
  if (s->src_on) {
    // without the ions the last sort staged for the next step (not taken),
    // compacted as they are written; the sort's count arrays are scratch now
    CU(to_f64_kept(g, s->N, c->dims.ni_max, s->buf[s->cur], s->tabm, s->tabb, xp, vp, vp1, mratd, bpd, s->count,
                   s->start_new, s->sums, &n_out, c->st));
  } else {
    CU(to_f64(g, s->N, c->dims.ni_max, s->buf[s->cur], xp, vp, vp1, c->st));
    CU(species_to_f64(s->N, s->buf[s->cur].sp, s->tabm, s->tabb, mratd, bpd, c->st));
  }
  for (int a = 0; a < 5; ++a)
    if (direct[a]) c->d2h_bytes += (a < 3 ? 24 : 8) * n_out;
  *c->ni_tot_ptr = (int32_t)n_out;
  s->n_out = n_out;
  s->ended = true;
  const std::size_t b3 = 3 * (std::size_t)g.C * sizeof(double);
  CU(join_df(3 * g.C, s->b1.h, s->b1.l, b1, c->st));
  CU(cudaMemcpyAsync(bt, b1, b3, cudaMemcpyDeviceToDevice, c->st));
  CU(cudaMemcpyAsync(b1p2, b1, b3, cudaMemcpyDeviceToDevice, c->st));
  CU(join_df(3 * g.C, s->b12.h, s->b12.l, b12, c->st));
  CU(grid_f32_to_f64(g.C, s->np, npd, c->st));
  CU(grid_f32_to_f64(3 * g.C, s->up, upd, c->st));
  CU(grid_f32_to_f64(3 * g.C, s->E, Ed, c->st));
  CU(grid_f32_to_f64(3 * g.C, s->aj, ajd, c->st));
  int r = c->finish();
  c->last_dtsub = s->last_dtsub;
  c->last_ntf = s->last_ntf;
  return r;
}

extern "C" int swap_f32_count(swap_ctx* c, int64_t* n) {
  if (!c || !n) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  // after swap_f32_end the state's ions are those written back (the buffer
  // still holds the next step's staged ions)
  *n = s->ended ? s->n_out : s->N;
  return SWAP_OK;
}

extern "C" int swap_f32_far_movers(swap_ctx* c, int64_t* n) {
  if (!c || !n) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  unsigned long long h = 0;
  CU(cudaMemcpyAsync(&h, s->far.total, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  *n = (int64_t)h;
  return SWAP_OK;
}

extern "C" int swap_f32_set_moment_sums(swap_ctx* c, int exact) {
  if (!c) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  if (!exact && s->gp != 0.0f)
    return c->fail(SWAP_EINVAL, "the electron-pressure term runs with the exact moment sums only");
  s->exact = exact != 0;
  return SWAP_OK;
}

extern "C" int swap_f32_key_starts(swap_ctx* c, int64_t* starts, int64_t n) {
  if (!c || !starts) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s || s->ended) return c->fail(SWAP_EINVAL, "no running FP32 state (swap_f32_begin first)");
  if (n < s->g.nkeys + 1) return c->fail(SWAP_EINVAL, "starts holds fewer than nkeys + 1 entries");
  CU(cudaMemcpyAsync(starts, s->start, (std::size_t)(s->g.nkeys + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                     c->st));
  CU(cudaStreamSynchronize(c->st));
  return SWAP_OK;
}

extern "C" int swap_f32_energy(swap_ctx* c, double out[4]) {
  if (!c || !out) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  const G32& g = s->g;
  const double vol = (double)g.dx * g.dy * g.dz;
  CU(energy32(g, s->N, s->buf[s->cur], s->sp, vol, s->b0, s->b1.h, s->b1.l, s->E, c->prm.alpha, s->acc, c->st));
  CU(cudaMemcpyAsync(out, s->acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  CU(cudaStreamSynchronize(c->st));
  return SWAP_OK;
}

// Validation entry: displace particles idx[q] (current sorted positions) by
// the cell steps of dcell[q] (packed like the cell: dx+1 | (dy+1)<<10 |
// (dz+1)<<20, each step in {-1,0,1}), then run the incremental stable sort
// that follows every ion step.  Lets a test compare the sort with a stable
// counting sort of the same keys.
__global__ void k_displace(G32 g, Part p, long long n, const int64_t* idx, const int32_t* dcell) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long long l = idx[q];
    const int32_t c = p.cell[l], d = dcell[q];
    int i = pk_i(c) + pk_i(d) - 1, j = pk_j(c) + pk_j(d) - 1, k = pk_k(c) + pk_k(d) - 1;
    i = i < 0 ? i + g.ncx : (i >= g.ncx ? i - g.ncx : i);
    j = j < 0 ? j + g.ncy : (j >= g.ncy ? j - g.ncy : j);
    k = k < 0 ? k + g.ncz : (k >= g.ncz ? k - g.ncz : k);
    p.cell[l] = pk(i, j, k);
  }
}

extern "C" int swap_f32_displace_resort(swap_ctx* c, int64_t n, const int64_t* idx, const int32_t* dcell) {
  if (!c || n < 0 || (n > 0 && (!idx || !dcell))) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  for (int64_t q = 0; q < n; ++q) {
    if (idx[q] < 0 || idx[q] >= s->N) return c->fail(SWAP_EINVAL, "particle index out of range");
    if (pk_i(dcell[q]) > 2 || pk_j(dcell[q]) > 2 || pk_k(dcell[q]) > 2 || (dcell[q] >> 30))
      return c->fail(SWAP_EINVAL, "cell steps must be -1, 0 or 1");
  }
  if (n > 0) {
    int64_t* di = s->alloc<int64_t>((std::size_t)n);
    int32_t* dd = s->alloc<int32_t>((std::size_t)n);
    if (!di || !dd) return c->fail(SWAP_ECUDA, "allocation");
    CU(cudaMemcpyAsync(di, idx, n * sizeof(int64_t), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(dd, dcell, n * sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
    k_displace<<<(unsigned)((n + 255) / 256), 256, 0, c->st>>>(s->g, s->buf[s->cur], n, di, dd);
    CU(cudaGetLastError());
  }
  TRY(sort_step(c, s, -1));
  return check_err(c);
}

// ---------------------------------------------------------------------------
// checkpoint of the FP32 state: everything a step reads from the previous one
// ---------------------------------------------------------------------------

namespace {

struct DevBlock {
  const char* name;
  void* dev;
  std::size_t bytes;
};

std::vector<DevBlock> f32_blocks(F32State* s) {
  const std::size_t N = (std::size_t)s->N, C = (std::size_t)s->g.C, nk = (std::size_t)s->g.nkeys;
  Part& p = s->buf[s->cur];
  return {{"cell", p.cell, N * 4},          {"ox", p.ox, N * 4},         {"oy", p.oy, N * 4},
          {"oz", p.oz, N * 4},              {"vx", p.vx, N * 4},         {"vy", p.vy, N * 4},
          {"vz", p.vz, N * 4},              {"wx", p.wx, N * 4},         {"wy", p.wy, N * 4},
          {"wz", p.wz, N * 4},              {"sp", p.sp, N},             {"start", s->start, (nk + 1) * 8},
          {"b1h", s->b1.h, 3 * C * 4},      {"b1l", s->b1.l, 3 * C * 4}, {"b12h", s->b12.h, 3 * C * 4},
          {"b12l", s->b12.l, 3 * C * 4},    {"db1", s->db1, 3 * C * 4},  {"np", s->np, C * 4},
          {"up", s->up, 3 * C * 4},         {"aj", s->aj, 3 * C * 4},    {"E", s->E, 3 * C * 4},
          {"tabm", s->tabm, MAX_SPECIES * 8}, {"tabb", s->tabb, MAX_SPECIES * 8}};
}

}  // namespace

int swap_f32_checkpoint(swap_ctx* c, std::FILE* f, bool write) {
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "no FP32 state");
  struct Meta {
    int64_t N;
    Species sp;
    uint8_t heavy_of[MAX_SPECIES];
    uint8_t sp_ion, sp_cloud, sp_inflow, pad;
  } m{};
  if (write) {
    m.N = s->N;
    m.sp = s->sp;
    std::memcpy(m.heavy_of, s->heavy_of, sizeof(m.heavy_of));
    m.sp_ion = s->stage.sp_ion;
    m.sp_cloud = s->stage.sp_cloud;
    m.sp_inflow = s->stage.sp_inflow;
    if (std::fwrite(&m, sizeof(m), 1, f) != 1) return c->fail(SWAP_EINVAL, "checkpoint write failed");
  } else {
    if (std::fread(&m, sizeof(m), 1, f) != 1) return c->fail(SWAP_EINVAL, "checkpoint read failed");
    if (m.N < 0 || m.N > c->dims.ni_max) return c->fail(SWAP_ECAPACITY, "checkpoint holds more ions than Ni_max");
    s->N = m.N;
    s->sp = m.sp;
    std::memcpy(s->heavy_of, m.heavy_of, sizeof(m.heavy_of));
    s->stage.sp_ion = m.sp_ion;
    s->stage.sp_cloud = m.sp_cloud;
    s->stage.sp_inflow = m.sp_inflow;
  }
  CU(cudaStreamSynchronize(c->st));
  std::vector<char> buf;
  for (const DevBlock& bl : f32_blocks(s)) {
    buf.resize(bl.bytes);
    if (write) {
      if (bl.bytes) CU(cudaMemcpy(buf.data(), bl.dev, bl.bytes, cudaMemcpyDeviceToHost));
      if (bl.bytes && std::fwrite(buf.data(), 1, bl.bytes, f) != bl.bytes)
        return c->fail(SWAP_EINVAL, std::string("checkpoint write failed at ") + bl.name);
    } else {
      if (bl.bytes && std::fread(buf.data(), 1, bl.bytes, f) != bl.bytes)
        return c->fail(SWAP_EINVAL, std::string("checkpoint read failed at ") + bl.name);
      if (bl.bytes) CU(cudaMemcpy(bl.dev, buf.data(), bl.bytes, cudaMemcpyHostToDevice));
    }
  }
  if (!write) s->ended = false;
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// the surrogate on the FP32 form
// ---------------------------------------------------------------------------

extern "C" int swap_surrogate_collect(swap_surrogate* net, swap_ctx* c, int32_t nsteps) {
  if (!net || !c || nsteps < 0) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s || s->ended) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  s->collect = net;
  int r = SWAP_OK;
  for (int k = 0; k < nsteps && !r; ++k) r = one_step(c, s);
  s->collect = nullptr;
  return r ? r : check_err(c);
}

extern "C" int swap_surrogate_attach(swap_ctx* c, swap_surrogate* net, int32_t judge_every, double bound) {
  if (!c) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  if (net && (judge_every < 1 || !(bound > 0))) return c->fail(SWAP_EINVAL, "judge_every >= 1 and bound > 0");
  s->sur = net;
  s->sur_every = judge_every;
  s->sur_bound = bound;
  s->sur_off = false;
  s->sur_step = 0;
  if (net) TRY(sur_buffers(c, s));
  return SWAP_OK;
}

extern "C" int swap_surrogate_set_db_bound(swap_ctx* c, double bound_db) {
  if (!c) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  if (!(bound_db >= 0)) return c->fail(SWAP_EINVAL, "bound_db >= 0");
  s->sur_bound_db = bound_db;
  return SWAP_OK;
}

extern "C" int swap_surrogate_stats(swap_ctx* c, double out[5]) {
  if (!c || !out) return SWAP_EINVAL;
  F32State* s = f32(c);
  if (!s) return c->fail(SWAP_EINVAL, "swap_f32_begin has not been called");
  out[0] = (double)s->sur_used;
  out[1] = (double)s->sur_judged;
  out[2] = (double)s->sur_fallbacks;
  out[3] = s->sur_err_b;
  out[4] = s->sur_err_db;
  return SWAP_OK;
}
