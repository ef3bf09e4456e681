// oracle_capi.cpp -- extern "C" face of the CPU oracle (TEST INFRASTRUCTURE).
//
// Every entry mirrors the argument list of the product's C-ABI entry of the
// same name (include/swap_gpu.h) with the prefix oracle_ (FP64) or oracle32_
// (FP32, the reference's own precision), so one Python replay of maind.f can
// drive either backend.  Arrays are the caller's host arrays; the oracle works
// on them in place, as the Fortran does.
#include <cstdint>
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "swap_oracle.hpp"

namespace {

template <class R>
struct OCtx {
  swo::State<R> s;
  // bound arrays (the Fortran's own arrays)
  R *xp = nullptr, *vp = nullptr, *vp1 = nullptr, *mrat = nullptr, *beta_p = nullptr;
  std::int32_t* ni_tot = nullptr;
  R *b0 = nullptr, *b1 = nullptr, *b12 = nullptr, *b1p2 = nullptr, *bt = nullptr, *btc = nullptr;
  R *np = nullptr, *up = nullptr, *aj = nullptr, *E = nullptr, *nu = nullptr;
  std::vector<R> Ep, vplus, vminus;  // maind.f locals for the fused step
  swo::Sources src{};
  bool have_src = false;
  std::int64_t step = 0;  // ion steps taken by the fused step (RNG counter)
  std::int64_t chex_count = 0;
  std::string err;
  std::int64_t N() const { return ni_tot ? (std::int64_t)*ni_tot : 0; }
};

template <class R, class F>
int guard(OCtx<R>* c, F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    c->err = e.what();
    return 1;
  }
}

template <class R>
struct Api {
  using Ctx = OCtx<R>;

  static Ctx* create(int nx, int ny, int nz, double dx, double dy, double delz, std::int64_t ni_max, double dt,
                     int ntsub, double alpha, double beta, double grad_pe, int nthreads) {
    auto* c = new Ctx();
    swo::grd7<R>(c->s.g, nx, ny, nz, (R)dx, (R)dy, (R)delz);
    c->s.dt = (R)dt;
    c->s.ntsub = ntsub;
    c->s.dtsub_init = (R)dt / (R)ntsub;
    c->s.dtsub = c->s.dtsub_init;
    c->s.ntf = (R)ntsub;
    c->s.alpha = (R)alpha;
    c->s.beta = (R)beta;
    c->s.grad_pe = (R)grad_pe;
    c->s.nthreads = nthreads < 1 ? 1 : nthreads;
    c->s.g.nt = c->s.nthreads;
    swo::state_alloc(c->s, ni_max);
    const std::size_t n3 = (std::size_t)ni_max * 3;
    c->Ep.assign(n3, R(0));
    c->vplus.assign(n3, R(0));
    c->vminus.assign(n3, R(0));
    return c;
  }
};

// The initial ion load of the workloads: ppc ions in every physical cell,
// positions uniform in the cell, each velocity component
// u + vth*sqrt(-ln U)*cos(pi*U') (the form of part_init.f:204-206), vp1 = vp
// (part_init.f:220).  It replaces load_Maxwellian (part_init.f:146-232),
// which draws positions over the whole box from the compiler's
// random_number; here the twelve uniforms of ion `id` are the Philox4x32-10
// block keyed by (seed, stream) with the ion's id as counter (the generator of
// ../swap_gb300/csrc/philox.h).  Ions come out by bricks of 4x4x4 cells, each
// brick's cells x fastest, when every axis has a multiple of 4 physical
// cells, else by cell with x fastest.  Arithmetic is in double, then rounded
// to R (kept above the cell's low node in x and z, see swo::above).
template <class R>
std::int64_t load_maxwellian(const swo::State<R>& s, std::uint64_t seed, std::uint32_t stream, int ppc, double vth,
                             double ux, double uy, double uz, double mrat, double beta_p, std::int64_t first, R* xp,
                             R* vp, R* vp1, R* mr, R* bp) {
  const auto& g = s.g;
  const std::int64_t ncx = g.nx - 2, ncy = g.ny - 2, ncz = g.nz - 2;
  const std::int64_t n = ncx * ncy * ncz * (std::int64_t)ppc;
  const std::int64_t NM = s.ni_max;
  if (ppc < 0 || first < 0) throw std::runtime_error("load_maxwellian: bad arguments");
  if (first + n > NM) throw std::runtime_error("load_maxwellian: Ni_max exceeded");
  const double pi = 3.14159265358979323846;
  const bool bricks = ncx % 4 == 0 && ncy % 4 == 0 && ncz % 4 == 0;
  SWO_OMP_FOR(g.nt)
  for (std::int64_t id = 0; id < n; ++id) {
    const std::int64_t cell = id / ppc;
    std::int64_t ci, cj, ck;
    if (bricks) {
      const std::int64_t b = cell / 64, q = cell % 64, bx = ncx / 4, by = ncy / 4;
      ci = (b % bx) * 4 + (q % 4);
      cj = ((b / bx) % by) * 4 + (q / 4) % 4;
      ck = (b / (bx * by)) * 4 + q / 16;
    } else {
      ci = cell % ncx;
      cj = (cell / ncx) % ncy;
      ck = cell / (ncx * ncy);
    }
    double u[12];
    swapk::particle_uniforms(seed, stream, (std::uint64_t)id, 0u, u);
    // physical cell (ci,cj,ck) spans nodes ci+1..ci+2 of the 1-based mesh
    const double x0 = g.qx[ci + 1], x1 = g.qx[ci + 2];
    const double y0 = g.qy[cj + 1], y1 = g.qy[cj + 2];
    const double z0 = g.qz[ck + 1], z1 = g.qz[ck + 2];
    const std::int64_t l = first + id;
    const double v[3] = {ux + vth * std::sqrt(-std::log(u[3])) * std::cos(pi * u[4]),
                         uy + vth * std::sqrt(-std::log(u[5])) * std::cos(pi * u[6]),
                         uz + vth * std::sqrt(-std::log(u[7])) * std::cos(pi * u[8])};
    xp[l] = swo::above<R>((R)(x0 + u[0] * (x1 - x0)), (R)x0);
    xp[l + NM] = (R)(y0 + u[1] * (y1 - y0));
    xp[l + 2 * NM] = swo::above<R>((R)(z0 + u[2] * (z1 - z0)), (R)z0);
    for (int m = 0; m < 3; ++m) {
      vp[l + m * NM] = (R)v[m];
      vp1[l + m * NM] = (R)v[m];
    }
    mr[l] = (R)mrat;
    bp[l] = (R)beta_p;
  }
  return n;
}

template <class R>
void copy_out(const std::vector<R>& v1based, int n, R* out) {
  for (int i = 1; i <= n; ++i) out[i - 1] = v1based[(std::size_t)i];
}

}  // namespace

#define CTX(T) auto* c = static_cast<OCtx<T>*>(h)

// One macro instantiates the whole API for a real type and prefix.
#define ORACLE_API(T, P)                                                                                   \
  extern "C" void* P##create(int nx, int ny, int nz, double dx, double dy, double delz, std::int64_t ni_max, \
                             double dt, int ntsub, double alpha, double beta, double grad_pe, int nthreads) { \
    try {                                                                                                  \
      return Api<T>::create(nx, ny, nz, dx, dy, delz, ni_max, dt, ntsub, alpha, beta, grad_pe, nthreads);  \
    } catch (...) {                                                                                        \
      return nullptr;                                                                                      \
    }                                                                                                      \
  }                                                                                                        \
  extern "C" void P##destroy(void* h) { delete static_cast<OCtx<T>*>(h); }                                 \
  extern "C" const char* P##last_error(void* h) {                                                          \
    CTX(T);                                                                                                \
    return c->err.c_str();                                                                                 \
  }                                                                                                        \
  extern "C" void P##get_coords(void* h, T* qx, T* qy, T* qz, T* dxg, T* dyg, T* dzg, T* dxc, T* dyc,      \
                                T* dzc, T* xr, T* yr, T* zr) {                                             \
    CTX(T);                                                                                                \
    const auto& g = c->s.g;                                                                                \
    copy_out(g.qx, g.nx, qx); copy_out(g.qy, g.ny, qy); copy_out(g.qz, g.nz, qz);                          \
    copy_out(g.dx_grid, g.nx, dxg); copy_out(g.dy_grid, g.ny, dyg); copy_out(g.dz_grid, g.nz, dzg);        \
    copy_out(g.dx_cell, g.nx, dxc); copy_out(g.dy_cell, g.ny, dyc); copy_out(g.dz_cell, g.nz, dzc);        \
    copy_out(g.xrat, g.nx, xr); copy_out(g.yrat, g.ny, yr); copy_out(g.zrat, g.nz, zr);                    \
  }                                                                                                        \
  extern "C" int P##bind_particles(void* h, T* xp, T* vp, T* vp1, T* mrat, T* beta_p, std::int32_t* ijkp, \
                                   std::int32_t* ni_tot) {                                                 \
    CTX(T);                                                                                                \
    (void)ijkp;                                                                                            \
    c->xp = xp; c->vp = vp; c->vp1 = vp1; c->mrat = mrat; c->beta_p = beta_p; c->ni_tot = ni_tot;          \
    return 0;                                                                                              \
  }                                                                                                        \
  extern "C" int P##bind_fields(void* h, T* b0, T* b1, T* b12, T* b1p2, T* bt, T* btc, T* np, T* up,       \
                                T* aj, T* E, T* nu) {                                                      \
    CTX(T);                                                                                                \
    c->b0 = b0; c->b1 = b1; c->b12 = b12; c->b1p2 = b1p2; c->bt = bt; c->btc = btc;                        \
    c->np = np; c->up = up; c->aj = aj; c->E = E; c->nu = nu;                                              \
    return 0;                                                                                              \
  }                                                                                                        \
  extern "C" void P##get_ijkp(void* h, std::int32_t* out) {                                                \
    CTX(T);                                                                                                \
    std::copy(c->s.ijkp.begin(), c->s.ijkp.end(), out);                                                    \
  }                                                                                                        \
  extern "C" void P##get_wght(void* h, T* out) {                                                           \
    CTX(T);                                                                                                \
    std::copy(c->s.wght.begin(), c->s.wght.end(), out);                                                    \
  }                                                                                                        \
  extern "C" void P##get_timestep(void* h, double* dtsub, double* ntf) {                                   \
    CTX(T);                                                                                                \
    *dtsub = (double)c->s.dtsub; *ntf = (double)c->s.ntf;                                                  \
  }                                                                                                        \
  extern "C" void P##set_nthreads(void* h, int n) {                                                        \
    CTX(T);                                                                                                \
    c->s.nthreads = n < 1 ? 1 : n;                                                                         \
    c->s.g.nt = c->s.nthreads;                                                                             \
  }                                                                                                        \
  /* The stratified Maxwellian load into the bound arrays (see load_maxwellian). */                        \
  extern "C" int P##load_maxwellian(void* h, std::uint64_t seed, std::uint32_t stream, int ppc, double vth,  \
                                    double ux, double uy, double uz, double mrat, double beta_p,           \
                                    std::int64_t first, std::int64_t* count) {                             \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      *count = load_maxwellian<T>(c->s, seed, stream, ppc, vth, ux, uy, uz, mrat, beta_p, first, c->xp,    \
                                  c->vp, c->vp1, c->mrat, c->beta_p);                                      \
      if (c->ni_tot) *c->ni_tot = (std::int32_t)(first + *count);                                          \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##get_interp_weights(void* h, const T* xp) {                                             \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::get_interp_weights(c->s, xp, c->N()); });                                   \
  }                                                                                                        \
  extern "C" int P##update_np(void* h, T* np) {                                                            \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::update_np(c->s, np, c->beta_p, c->N()); });                                 \
  }                                                                                                        \
  extern "C" int P##update_np_local(void* h, T* np) {                                                      \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::update_np(c->s, np, c->beta_p, c->N(), false); });                          \
  }                                                                                                        \
  extern "C" int P##update_up(void* h, const T* vp, const T* np, T* up) {                                  \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::update_up(c->s, vp, np, up, c->beta_p, c->N()); });                         \
  }                                                                                                        \
  extern "C" int P##extrapol_up(void* h, T* up, const T* vp, const T* vp1, const T* np) {                  \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::extrapol_up(c->s, up, vp, vp1, np, c->beta_p, c->N()); });                  \
  }                                                                                                        \
  extern "C" int P##get_Ep(void* h, T* Ep, T* aj, const T* np, T* up, const T* btc, const T* nu) {         \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::get_Ep(c->s, Ep, aj, np, up, btc, nu, c->mrat, c->N()); });                 \
  }                                                                                                        \
  extern "C" int P##get_vplus_vminus(void* h, const T* Ep, const T* btc, const T* vp, T* vplus,            \
                                     T* vminus) {                                                          \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::get_vplus_vminus(c->s, Ep, btc, vp, vplus, vminus, c->mrat, c->N()); });    \
  }                                                                                                        \
  extern "C" int P##improve_up(void* h, T* vp1, const T* vplus, const T* vminus, T* up, const T* np) {     \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::improve_up(c->s, vp1, vplus, vminus, up, np, c->beta_p, c->N()); });        \
  }                                                                                                        \
  extern "C" int P##get_vp_final(void* h, const T* Ep, T* vp, T* vp1, const T* vplus) {                    \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::get_vp_final(c->s, Ep, vp, vp1, vplus, c->N()); });                         \
  }                                                                                                        \
  extern "C" int P##move_ion_half(void* h, T* xp, const T* vp, const T* vp1, T* input_p) {                 \
    CTX(T);                                                                                                \
    (void)vp1; (void)input_p;                                                                              \
    return guard(c, [&] { swo::move_ion_half(c->s, xp, vp, c->N(), c->have_src && c->src.x_open); });      \
  }                                                                                                        \
  extern "C" int P##curlB(void* h, T* bt, const T* np, T* aj) {                                            \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::curlB(c->s, bt, np, aj); });                                                \
  }                                                                                                        \
  extern "C" int P##edge_to_center(void* h, T* bt, T* btc) {                                               \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::edge_to_center(c->s.g, bt, btc); });                                        \
  }                                                                                                        \
  extern "C" int P##face_to_center(void* h, T* v, T* vc) {                                                 \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::face_to_center(c->s.g, v, vc); });                                          \
  }                                                                                                        \
  extern "C" int P##get_E(void* h, T* E, const T* b0, T* bt, T* aj, const T* up, const T* np,              \
                          const T* nu) {                                                                   \
    CTX(T);                                                                                                \
    (void)b0;                                                                                              \
    return guard(c, [&] { swo::get_E(c->s, E, bt, aj, up, np, nu); });                                     \
  }                                                                                                        \
  extern "C" int P##predict_B(void* h, T* b0, T* b1, T* b12, T* b1p2, T* bt, T* E, T* aj, T* up, T* np,    \
                              T* nu, double dtsub) {                                                       \
    CTX(T);                                                                                                \
    c->s.dtsub = (T)dtsub;                                                                                 \
    return guard(c, [&] { swo::predict_B(c->s, b0, b1, b12, b1p2, bt, E, aj, up, np, nu); });              \
  }                                                                                                        \
  extern "C" int P##correct_B(void* h, T* b0, T* b1, T* b1p2, T* E, T* aj, T* up, T* np, T* nu,            \
                              double dtsub) {                                                              \
    CTX(T);                                                                                                \
    c->s.dtsub = (T)dtsub;                                                                                 \
    return guard(c, [&] { swo::correct_B(c->s, b0, b1, b1p2, E, aj, up, np, nu); });                       \
  }                                                                                                        \
  extern "C" int P##f_update_tlev(void* h, T* b1, T* b12, T* b1p2, T* bt, const T* b0) {                   \
    CTX(T);                                                                                                \
    (void)b0;                                                                                              \
    return guard(c, [&] { swo::f_update_tlev(c->s.g, b1, b12, b1p2, bt); });                               \
  }                                                                                                        \
  extern "C" int P##check_time_step(void* h, const T* bt, const T* np, double* dtsub, double* ntf) {       \
    CTX(T);                                                                                                \
    c->s.dtsub = (T)*dtsub;                                                                                \
    c->s.ntf = (T)*ntf;                                                                                    \
    int r = guard(c, [&] { swo::check_time_step(c->s, bt, np, c->s.g.dx); });                              \
    *dtsub = (double)c->s.dtsub;                                                                           \
    *ntf = (double)c->s.ntf;                                                                               \
    return r;                                                                                              \
  }                                                                                                        \
  extern "C" double P##max_abs_divB(void* h, const T* b) {                                                 \
    CTX(T);                                                                                                \
    return swo::max_abs_divB(c->s.g, b);                                                                   \
  }                                                                                                        \
  extern "C" void P##energy(void* h, double* out4) {                                                       \
    CTX(T);                                                                                                \
    auto e = swo::energy_norm(c->s, c->vp, c->b0, c->b1, c->E, c->mrat, c->beta_p, c->N());                \
    out4[0] = e.ekin; out4[1] = e.eb1; out4[2] = e.eb; out4[3] = e.ee;                                     \
  }                                                                                                        \
  extern "C" void P##energy_ref(void* h, const T* m_arr, double mion, double* out4) {                     \
    CTX(T);                                                                                                \
    auto e = swo::energy_ref(c->s, c->vp, c->b0, c->b1, c->E, m_arr, c->beta_p, c->N(), (T)mion);          \
    out4[0] = e.ekin; out4[1] = e.eb1; out4[2] = e.eb; out4[3] = e.ee;                                     \
  }                                                                                                        \
  /* One ion step in the order of maind.f:385-479 on the bound arrays. */                                  \
  extern "C" int P##ion_step(void* h) {                                                                    \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      auto& s = c->s;                                                                                      \
      T* Ep = c->Ep.data(); T* vpl = c->vplus.data(); T* vmi = c->vminus.data();                           \
      if (c->have_src) { /* maind.f:379-383 and the cloud and inflow sources */                                      \
        const auto& q = c->src;                                                                            \
        if (q.ndot > 0)                                                                                    \
          *c->ni_tot += (std::int32_t)swo::ionize_sw(s, q, c->step, c->xp, c->vp, c->vp1, c->mrat,         \
                                                     c->beta_p, c->N());                                   \
        if (q.nu_ion > 0)                                                                                  \
          *c->ni_tot += (std::int32_t)swo::ionize_cloud(s, q, c->step, c->xp, c->vp, c->vp1, c->mrat,      \
                                                        c->beta_p, c->N());                                \
        if (q.x_open)                                                                                      \
          *c->ni_tot += (std::int32_t)swo::inflow_x(s, q, c->step, c->xp, c->vp, c->vp1, c->mrat,          \
                                                    c->beta_p, c->N());                                    \
      }                                                                                                    \
      const bool xo = c->have_src && c->src.x_open;                                                        \
      std::int64_t N = c->N();                                                                             \
      swo::get_interp_weights(s, c->xp, N);                                /* maind.f:385 */               \
      swo::update_np(s, c->np, c->beta_p, N);                              /* :386 */                      \
      swo::update_up(s, c->vp, c->np, c->up, c->beta_p, N);                /* :387 */                      \
      swo::curlB(s, c->bt, c->np, c->aj);                                  /* :395 */                      \
      swo::edge_to_center(s.g, c->bt, c->btc);                             /* :398 */                      \
      swo::extrapol_up(s, c->up, c->vp, c->vp1, c->np, c->beta_p, N);      /* :399 */                      \
      swo::get_Ep(s, Ep, c->aj, c->np, c->up, c->btc, c->nu, c->mrat, N);  /* :400 */                      \
      swo::get_vplus_vminus(s, Ep, c->btc, c->vp, vpl, vmi, c->mrat, N);   /* :401 */                      \
      swo::improve_up(s, c->vp1, vpl, vmi, c->up, c->np, c->beta_p, N);    /* :402 */                      \
      swo::get_Ep(s, Ep, c->aj, c->np, c->up, c->btc, c->nu, c->mrat, N);  /* :404 */                      \
      swo::get_vplus_vminus(s, Ep, c->btc, c->vp, vpl, vmi, c->mrat, N);   /* :405 */                      \
      swo::get_vp_final(s, Ep, c->vp, c->vp1, vpl, N);                     /* :406 */                      \
      swo::move_ion_half(s, c->xp, c->vp, N, xo);                          /* :408 */                      \
      if (xo) {                                                                                            \
        *c->ni_tot = (std::int32_t)swo::remove_outflow_x(s, c->xp, c->vp, c->vp1, c->mrat, c->beta_p, N);  \
        N = c->N();                                                                                        \
      }                                                                                                    \
      swo::get_interp_weights(s, c->xp, N);                                /* :411 */                      \
      swo::update_np(s, c->np, c->beta_p, N);                              /* :412 */                      \
      swo::update_up(s, c->vp, c->np, c->up, c->beta_p, N);                /* :413 */                      \
      s.dtsub = s.dtsub_init;                                              /* :420-421 */                  \
      s.ntf = (T)s.ntsub;                                                                                  \
      swo::check_time_step(s, c->bt, c->np, s.g.dx);                       /* :423 */                      \
      const int nsub = (int)s.ntf;                                                                         \
      for (int n = 1; n <= nsub; ++n) {                                    /* :425-476 */                  \
        swo::curlB(s, c->bt, c->np, c->aj);                                                                \
        swo::predict_B(s, c->b0, c->b1, c->b12, c->b1p2, c->bt, c->E, c->aj, c->up, c->np, c->nu);         \
        swo::correct_B(s, c->b0, c->b1, c->b1p2, c->E, c->aj, c->up, c->np, c->nu);                        \
        swo::f_update_tlev(s.g, c->b1, c->b12, c->b1p2, c->bt);                                            \
      }                                                                                                    \
      swo::move_ion_half(s, c->xp, c->vp, N, xo);                          /* :479 */                      \
      if (xo) *c->ni_tot = (std::int32_t)swo::remove_outflow_x(s, c->xp, c->vp, c->vp1, c->mrat, c->beta_p, N); \
      if (c->have_src && c->src.cx_a > 0) /* :484, res_chex */                                             \
        c->chex_count += swo::res_chex(s, c->src, c->step, c->xp, c->vp, c->vp1, c->mrat, c->N());        \
      c->step++;                                                                                           \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##update_rho(void* h, T* mnp, double mion) {                                            \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::update_rho(c->s, mnp, c->mrat, c->beta_p, c->N(), (T)mion); });             \
  }                                                                                                        \
  extern "C" int P##get_temperature(void* h, const T* xp, const T* vp, const T* np, T* temp_p, double mion) { \
    CTX(T);                                                                                                \
    (void)xp;                                                                                              \
    return guard(c, [&] { swo::get_temperature(c->s, vp, np, temp_p, c->mrat, c->beta_p, c->N(), (T)mion); }); \
  }                                                                                                        \
  extern "C" int P##set_sources(void* h, const swo::Sources* q, std::int64_t step0) {                       \
    CTX(T);                                                                                                \
    c->src = *q;                                                                                           \
    c->have_src = true;                                                                                    \
    c->step = step0;                                                                                       \
    return 0;                                                                                              \
  }                                                                                                        \
  extern "C" std::int64_t P##chex_count(void* h) {                                                         \
    CTX(T);                                                                                                \
    return c->chex_count;                                                                                  \
  }                                                                                                        \
  extern "C" int P##Ionize_sw_mp(void* h, T* np, T* vp, T* vp1, T* xp, std::int32_t m, T* input_p, T* up) { \
    CTX(T);                                                                                                \
    (void)input_p;                                                                                         \
    return guard(c, [&] {                                                                                  \
      *c->ni_tot += (std::int32_t)swo::ionize_sw(c->s, c->src, m, xp, vp, vp1, c->mrat, c->beta_p, c->N()); \
      swo::get_interp_weights(c->s, xp, c->N());                           /* chem_rates.f:641-643 */      \
      swo::update_np(c->s, np, c->beta_p, c->N());                                                         \
      swo::update_up(c->s, vp, np, up, c->beta_p, c->N());                                                 \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##inflow_x(void* h, std::int32_t m) {                                                    \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      *c->ni_tot += (std::int32_t)swo::inflow_x(c->s, c->src, m, c->xp, c->vp, c->vp1, c->mrat, c->beta_p, \
                                                c->N());                                                   \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##ionize_cloud(void* h, std::int32_t m) {                                                \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      *c->ni_tot += (std::int32_t)swo::ionize_cloud(c->s, c->src, m, c->xp, c->vp, c->vp1, c->mrat,        \
                                                    c->beta_p, c->N());                                    \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##remove_outflow_x(void* h) {                                                            \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      *c->ni_tot = (std::int32_t)swo::remove_outflow_x(c->s, c->xp, c->vp, c->vp1, c->mrat, c->beta_p,     \
                                                       c->N());                                            \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##remove_ion(void* h, T* xp, T* vp, T* vp1, std::int32_t ion_l) {                        \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      std::vector<char> keep((std::size_t)c->N(), 1);                                                      \
      if (ion_l < 1 || ion_l > c->N()) throw std::runtime_error("remove_ion: index out of range");         \
      keep[(std::size_t)ion_l - 1] = 0;                                                                    \
      *c->ni_tot = (std::int32_t)swo::compact(c->s, keep, xp, vp, vp1, c->mrat, c->beta_p, c->N());        \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" int P##res_chex(void* h, T* xp, T* vp, std::int32_t m, std::int64_t* count) {                 \
    CTX(T);                                                                                                \
    return guard(c, [&] { *count = swo::res_chex(c->s, c->src, m, xp, vp, c->vp1, c->mrat, c->N()); });    \
  }                                                                                                        \
  extern "C" int P##move_ion_half_open(void* h, T* xp, const T* vp) {                                      \
    CTX(T);                                                                                                \
    return guard(c, [&] { swo::move_ion_half(c->s, xp, vp, c->N(), true); });                             \
  }                                                                                                        \
  extern "C" int P##sort_perm(void* h, std::int64_t* perm, std::int64_t* counts) {                         \
    CTX(T);                                                                                                \
    return guard(c, [&] {                                                                                  \
      std::vector<std::int64_t> p, cnt;                                                                    \
      swo::counting_sort_perm(c->s.g, c->s.ijkp.data(), c->s.ni_max, c->N(), p, cnt);                      \
      std::copy(p.begin(), p.end(), perm);                                                                 \
      std::copy(cnt.begin(), cnt.end(), counts);                                                           \
    });                                                                                                    \
  }                                                                                                        \
  extern "C" void P##initparameters(double b0_init, int ion_amu, double nf_init, double dt_frac,           \
                                    double dx_frac, double nu_init_frac, int ntsub, double* out10) {       \
    swo::PhysInputs<T> in{(T)b0_init, (T)nf_init, (T)dt_frac, (T)dx_frac, (T)nu_init_frac, ion_amu};      \
    auto d = swo::initparameters(in, ntsub);                                                               \
    const T v[10] = {d.mion, d.omega_p, d.lambda_i, d.dx, d.dy, d.delz, d.dt, d.dtsub_init, d.nu_init,     \
                     d.alpha};                                                                             \
    for (int i = 0; i < 10; ++i) out10[i] = (double)v[i];                                                  \
  }                                                                                                        \
  extern "C" void P##grd6_setup(void* h, double b0_init, double mion, double nu_init) {                    \
    CTX(T);                                                                                                \
    swo::grd6_setup(c->s.g, (T)b0_init, (T)mion, (T)nu_init, c->b0, c->bt, c->b12, c->b1, c->b1p2, c->nu); \
  }

ORACLE_API(double, oracle_)
ORACLE_API(float, oracle32_)

// Stable counting sort over arbitrary integer keys in [0, nkeys): perm[new] =
// old, counts[key].  The definition the GPU's incremental sort must match.
extern "C" int oracle_stable_counting_sort(const std::int64_t* keys, std::int64_t n, std::int64_t nkeys,
                                           std::int64_t* perm, std::int64_t* counts) {
  std::vector<std::int64_t> start((std::size_t)nkeys + 1, 0);
  for (std::int64_t l = 0; l < n; ++l) {
    if (keys[l] < 0 || keys[l] >= nkeys) return 1;
    start[(std::size_t)keys[l] + 1]++;
  }
  for (std::int64_t k = 0; k < nkeys; ++k) counts[k] = start[(std::size_t)k + 1];
  for (std::int64_t k = 0; k < nkeys; ++k) start[(std::size_t)k + 1] += start[(std::size_t)k];
  for (std::int64_t l = 0; l < n; ++l) perm[start[(std::size_t)keys[l]]++] = l;
  return 0;
}

// The counter-based generator shared by the oracle and the product
// (swap_gb300/csrc/philox.h), exposed so tests can pin it to the published
// Philox4x32-10 known-answer vectors.
extern "C" void oracle_philox4x32_10(const std::uint32_t ctr[4], const std::uint32_t key[2], std::uint32_t out[4]) {
  swapk::u32x4 c;
  for (int q = 0; q < 4; ++q) c.v[q] = ctr[q];
  const swapk::u32x4 r = swapk::philox4x32_10(c, key[0], key[1]);
  for (int q = 0; q < 4; ++q) out[q] = r.v[q];
}

extern "C" void oracle_source_uniforms(std::uint64_t seed, std::uint32_t stream, std::int64_t step, std::int64_t a,
                                       std::uint32_t b, double u[4]) {
  swapk::source_uniforms(seed, stream, step, a, b, u);
}
