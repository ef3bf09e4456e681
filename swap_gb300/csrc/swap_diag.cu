// swap_diag.cu -- the reference's diagnostic output (maind.f:237-358,
// 498-573) and a checkpoint of the context's state.
//
// Output files are Fortran sequential unformatted: every record is a 4-byte
// length, the payload, and the length again, as the reference's
// `write(unit)` produces and IDL's /f77_unformatted reads (read_para.pro,
// get_fv.pro).  Reals are written at the reference's size (4 bytes, its
// -real-size 32 build) unless 8 is asked for.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"
#include "k64.cuh"
#include "swap_ctx.h"
#include "swap_ops.h"

namespace {

struct Unit {
  int number;
  const char* name;  // file name after out_dir
  FILE* f = nullptr;
};

struct Diag {
  std::string dir;
  swap_diag_spec spec{};
  int ndiag = 0;
  std::vector<Unit> units;
  double* d_temp = nullptr;  // temp_p and mnp on the device
  double* d_mnp = nullptr;
  std::vector<double> h_temp, h_mnp;
};

Diag* diag(swap_ctx* c) { return static_cast<Diag*>(c->diag_state); }

constexpr long long MAX_RECORD = 2147483647LL;

int rec_raw(swap_ctx* c, FILE* f, const void* data, std::size_t bytes) {
  if ((long long)bytes > MAX_RECORD)
    return c->fail(SWAP_ECAPACITY, "a record exceeds 2^31-1 bytes (use 4-byte reals or fewer particles)");
  const int32_t n = (int32_t)bytes;
  if (std::fwrite(&n, 4, 1, f) != 1 || (bytes && std::fwrite(data, 1, bytes, f) != bytes) ||
      std::fwrite(&n, 4, 1, f) != 1)
    return c->fail(SWAP_EINVAL, std::string("diagnostic write failed: ") + std::strerror(errno));
  return SWAP_OK;
}

// One record of reals, converted to the output real size.
int rec_reals(swap_ctx* c, FILE* f, const double* a, std::size_t n, int real_bytes) {
  if (real_bytes == 8) return rec_raw(c, f, a, n * 8);
  std::vector<float> t(n);
  for (std::size_t i = 0; i < n; ++i) t[i] = (float)a[i];
  return rec_raw(c, f, t.data(), n * 4);
}

int rec_int(swap_ctx* c, FILE* f, int32_t m) { return rec_raw(c, f, &m, 4); }

// A record mixing int32 and reals in the given order ('i' / 'r').
int rec_mixed(swap_ctx* c, FILE* f, const char* kinds, const double* v, int real_bytes) {
  std::vector<unsigned char> buf;
  for (int k = 0; kinds[k]; ++k) {
    unsigned char b[8];
    std::size_t n;
    if (kinds[k] == 'i') {
      const int32_t x = (int32_t)v[k];
      std::memcpy(b, &x, 4);
      n = 4;
    } else if (real_bytes == 8) {
      std::memcpy(b, &v[k], 8);
      n = 8;
    } else {
      const float x = (float)v[k];
      std::memcpy(b, &x, 4);
      n = 4;
    }
    buf.insert(buf.end(), b, b + n);
  }
  return rec_raw(c, f, buf.data(), buf.size());
}

// The same for a bound host array: float when the context binds 4-byte reals.
int rec_host(swap_ctx* c, FILE* f, const double* a, std::size_t n, int real_bytes) {
  if (c->real_bytes == 8) return rec_reals(c, f, a, n, real_bytes);
  const float* x = reinterpret_cast<const float*>(a);
  if (real_bytes == 4) return rec_raw(c, f, x, n * 4);
  std::vector<double> t(x, x + n);
  return rec_raw(c, f, t.data(), n * 8);
}

// Element i of a bound host real array, as a double.
inline double hreal(const swap_ctx* c, const double* a, std::size_t i) {
  return c->real_bytes == 4 ? (double)reinterpret_cast<const float*>(a)[i] : a[i];
}

FILE* unit(Diag* d, int number) {
  for (Unit& u : d->units)
    if (u.number == number) return u.f;
  return nullptr;
}

#define TRY(x)         \
  do {                 \
    int _r = (x);      \
    if (_r) return _r; \
  } while (0)

// The field and particle dump of maind.f:512-571.
int dump(swap_ctx* c, Diag* d, int32_t m) {
  const swap_diag_spec& sp = d->spec;
  const int rb = sp.real_bytes;
  const std::size_t C = (std::size_t)c->g.C, NM = (std::size_t)c->dims.ni_max;
  if (sp.rank == 0) {
    // get_temperature and update_rho (maind.f:515-516) on the device
    double *dxp, *dvp, *dnp, *dd;
    TRY(c->begin());
    TRY(c->use(c->h_xp, Access::In, &dxp));
    TRY(c->use(c->h_vp, Access::In, &dvp));
    TRY(c->use(c->h_np, Access::In, &dnp));
    TRY(c->use(c->h_mrat, Access::In, &dd));
    TRY(c->use(c->h_beta_p, Access::In, &dd));
    // the reference uses the weights of maind.f:411; after the FP32 form
    // there are none, so they are taken at the current positions
    if (!c->weights_valid || c->weights_n < c->ntot()) TRY(ops::get_interp_weights(c, dxp));
    TRY(ops::get_temperature(c, dvp, dnp, d->d_temp));
    TRY(ops::update_rho(c, d->d_mnp));
    if (cudaMemcpyAsync(d->h_temp.data(), d->d_temp, C * 8, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
        cudaMemcpyAsync(d->h_mnp.data(), d->d_mnp, C * 8, cudaMemcpyDeviceToHost, c->st) != cudaSuccess)
      return c->fail(SWAP_ECUDA, "diagnostic copy");
    TRY(c->finish());
  }
  TRY(swap_sync_to_host(c, nullptr));
  std::vector<double> zeros3(3 * C, 0.0), t(3 * C);
  if (sp.rank == 0) {
    TRY(rec_int(c, unit(d, 110), m));
    TRY(rec_host(c, unit(d, 110), c->h_np, C, rb));
    TRY(rec_int(c, unit(d, 115), m));
    TRY(rec_reals(c, unit(d, 115), zeros3.data(), C, rb));  // np_b: separate_np is not called (maind.f:513)
    TRY(rec_int(c, unit(d, 120), m));
    TRY(rec_reals(c, unit(d, 120), zeros3.data(), C, rb));  // mixed: no mixing tags in this model
    TRY(rec_int(c, unit(d, 130), m));
    TRY(rec_host(c, unit(d, 130), c->h_bt, 3 * C, rb));
    // current density aj*alpha*np3, np3 the face-averaged density
    const int nx = c->dims.nx, ny = c->dims.ny, nz = c->dims.nz;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const std::size_t o = (std::size_t)i + (std::size_t)nx * (j + (std::size_t)ny * k);
          const std::size_t s[3] = {1, (std::size_t)nx, (std::size_t)nx * ny};
          const bool last[3] = {i == nx - 1, j == ny - 1, k == nz - 1};
          for (int q = 0; q < 3; ++q) {
            const double n3 = last[q] ? hreal(c, c->h_np, o) : 0.5 * (hreal(c, c->h_np, o) + hreal(c, c->h_np, o + s[q]));
            t[o + C * q] = hreal(c, c->h_aj, o + C * q) * c->prm.alpha * n3;
          }
        }
    TRY(rec_int(c, unit(d, 140), m));
    TRY(rec_reals(c, unit(d, 140), t.data(), 3 * C, rb));
    TRY(rec_int(c, unit(d, 150), m));
    TRY(rec_host(c, unit(d, 150), c->h_E, 3 * C, rb));
    TRY(rec_int(c, unit(d, 180), m));
    TRY(rec_host(c, unit(d, 180), c->h_up, 3 * C, rb));
    for (std::size_t o = 0; o < C; ++o) t[o] = d->h_temp[o] / 1.6e-19;  // maind.f:546
    TRY(rec_int(c, unit(d, 300), m));
    TRY(rec_reals(c, unit(d, 300), t.data(), C, rb));
  }
  TRY(rec_int(c, unit(d, 305), m));
  TRY(rec_host(c, unit(d, 305), c->h_xp, 3 * NM, rb));
  TRY(rec_int(c, unit(d, 310), m));
  TRY(rec_host(c, unit(d, 310), c->h_vp, 3 * NM, rb));
  TRY(rec_int(c, unit(d, 315), m));
  TRY(rec_host(c, unit(d, 315), c->h_mrat, NM, rb));
  TRY(rec_int(c, unit(d, 317), m));
  TRY(rec_host(c, unit(d, 317), c->h_beta_p, NM, rb));
  if (sp.rank == 0) {
    TRY(rec_int(c, unit(d, 330), m));
    TRY(rec_reals(c, unit(d, 330), zeros3.data(), 3 * C, rb));  // up_t, up_b: separate_up is not called
    TRY(rec_int(c, unit(d, 340), m));
    TRY(rec_reals(c, unit(d, 340), zeros3.data(), 3 * C, rb));
    TRY(rec_int(c, unit(d, 350), m));
    TRY(rec_reals(c, unit(d, 350), d->h_mnp.data(), C, rb));
  }
  for (Unit& u : d->units)
    if (u.f) std::fflush(u.f);
  return SWAP_OK;
}

}  // namespace

void swap_diag_free(swap_ctx* c) {
  Diag* d = diag(c);
  if (!d) return;
  for (Unit& u : d->units)
    if (u.f) std::fclose(u.f);
  if (d->d_temp) cudaFree(d->d_temp);
  if (d->d_mnp) cudaFree(d->d_mnp);
  delete d;
  c->diag_state = nullptr;
}

extern "C" int swap_diag_open(swap_ctx* c, const char* out_dir, const swap_diag_spec* spec) {
  if (!c || !out_dir || !spec) return SWAP_EINVAL;
  c->err.clear();
  if (spec->real_bytes != 4 && spec->real_bytes != 8) return c->fail(SWAP_EINVAL, "real_bytes must be 4 or 8");
  if (spec->nout < 1 || spec->rank < 0 || spec->rank > 16) return c->fail(SWAP_EINVAL, "nout >= 1, rank 0..16");
  if (!c->h_xp || !c->h_b1) return c->fail(SWAP_EINVAL, "swap_bind_particles and swap_bind_fields are required");
  swap_diag_free(c);
  auto* d = new Diag();
  c->diag_state = d;
  d->dir = out_dir;
  d->spec = *spec;
  c->mion = spec->mion > 0 ? spec->mion : 1.0;
  const std::size_t C = (std::size_t)c->g.C;
  if (cudaMalloc(&d->d_temp, C * 8) != cudaSuccess || cudaMalloc(&d->d_mnp, C * 8) != cudaSuccess)
    return c->fail(SWAP_ECUDA, "diagnostic buffers");
  d->h_temp.assign(C, 0.0);
  d->h_mnp.assign(C, 0.0);
  const int rb = spec->real_bytes;
  if (spec->rank == 0) {
    // para.dat (maind.f:237-256)
    const std::string pth = d->dir + "para.dat";
    FILE* f = std::fopen(pth.c_str(), "wb");
    if (!f) return c->fail(SWAP_EINVAL, "cannot open " + pth);
    const double delz = c->h_qz.size() > 1 ? c->h_qz[1] - c->h_qz[0] : 1.0;
    const double r1[6] = {(double)c->dims.nx, (double)c->dims.ny, (double)c->dims.nz, c->prm.dx, c->prm.dy, delz};
    const double r2[5] = {(double)spec->nt, spec->dtsub_init, (double)c->prm.ntsub, c->prm.dt, (double)spec->nout};
    char od[50];
    std::memset(od, ' ', sizeof(od));
    std::memcpy(od, out_dir, std::min<std::size_t>(std::strlen(out_dir), sizeof(od)));
    const double r4[2] = {spec->vtop, spec->vbottom};
    const double r5[1] = {(double)c->dims.ni_max};
    const double r6[3] = {spec->mion, spec->m_pu, spec->m_heavy};
    const double r7[2] = {spec->np_top, spec->np_bottom};
    const double r8[2] = {spec->b0_top, spec->b0_bottom};
    const double r9[2] = {spec->vth_top, spec->vth_bottom};
    const double r10[2] = {c->prm.alpha, c->prm.beta};
    int r = rec_mixed(c, f, "iiirrr", r1, rb);
    if (!r) r = rec_mixed(c, f, "iriri", r2, rb);
    if (!r) r = rec_raw(c, f, od, sizeof(od));
    if (!r) r = rec_mixed(c, f, "rr", r4, rb);
    if (!r) r = rec_mixed(c, f, "i", r5, rb);
    if (!r) r = rec_mixed(c, f, "rrr", r6, rb);
    if (!r) r = rec_mixed(c, f, "rr", r7, rb);
    if (!r) r = rec_mixed(c, f, "rr", r8, rb);
    if (!r) r = rec_mixed(c, f, "rr", r9, rb);
    if (!r) r = rec_mixed(c, f, "rr", r10, rb);
    std::fclose(f);
    if (r) return r;
    static const struct {
      int n;
      const char* name;
    } files[] = {{110, "c.np.dat"},       {115, "c.np_b.dat"},      {120, "c.mixed.dat"},
                 {130, "c.b1.dat"},       {140, "c.aj.dat"},        {150, "c.E.dat"},
                 {160, "c.energy.dat"},   {180, "c.up.dat"},        {190, "c.momentum.dat"},
                 {192, "c.p_conserve.dat"}, {300, "c.temp_p.dat"},  {305, "c.xp_0.dat"},
                 {310, "c.vp_0.dat"},     {315, "c.mrat_0.dat"},    {317, "c.beta_p_0.dat"},
                 {320, "c.np_wake.dat"},  {330, "c.up_t.dat"},      {340, "c.up_b.dat"},
                 {342, "c.test_part.dat"}, {350, "c.mnp.dat"}};  // maind.f:269-342
    for (const auto& u : files) d->units.push_back(Unit{u.n, u.name});
  } else {
    // ranks > 0 write their own particles (maind.f:344-358)
    static std::string names[4];
    const std::string r = std::to_string(spec->rank);
    names[0] = "c.xp_" + r + ".dat";
    names[1] = "c.vp_" + r + ".dat";
    names[2] = "c.mrat_" + r + ".dat";
    names[3] = "c.beta_p_" + r + ".dat";
    d->units = {Unit{305, names[0].c_str()}, Unit{310, names[1].c_str()}, Unit{315, names[2].c_str()},
                Unit{317, names[3].c_str()}};
  }
  for (Unit& u : d->units) {
    const std::string pth = d->dir + u.name;
    u.f = std::fopen(pth.c_str(), "wb");
    if (!u.f) return c->fail(SWAP_EINVAL, "cannot open " + pth);
  }
  return SWAP_OK;
}

extern "C" int swap_diag_step(swap_ctx* c, int32_t m) {
  if (!c) return SWAP_EINVAL;
  Diag* d = diag(c);
  if (!d) return c->fail(SWAP_EINVAL, "swap_diag_open has not been called");
  if (c->f32_state && !swap_f32_ended(c))
    return c->fail(SWAP_EINVAL, "the FP32 form is active: call swap_f32_end before swap_diag_step");
  const int rb = d->spec.real_bytes;
  if (d->spec.rank == 0) {
    // c.energy.dat and c.momentum.dat every step (maind.f:502-508)
    double e[7] = {0};
    TRY(ops::energy7(c, e));
    int64_t nchex = 0;
    TRY(swap_chex_count(c, &nchex));
    const double en[12] = {0.0, 0.0, e[0], 0.0, e[1], e[4], e[5], e[6], e[3], 0.0, (double)nchex, 0.0};
    TRY(rec_int(c, unit(d, 160), m));
    TRY(rec_reals(c, unit(d, 160), en, 12, rb));
    const double mo[12] = {0};  // Momentum_diag is not called (maind.f:468); input_p is not tracked
    TRY(rec_int(c, unit(d, 190), m));
    TRY(rec_reals(c, unit(d, 190), mo, 12, rb));
  }
  if (++d->ndiag == d->spec.nout) {  // maind.f:510-571
    TRY(dump(c, d, m));
    d->ndiag = 0;
  }
  return SWAP_OK;
}

extern "C" int swap_diag_close(swap_ctx* c) {
  if (!c) return SWAP_EINVAL;
  swap_diag_free(c);
  return SWAP_OK;
}

// ---------------------------------------------------------------------------
// checkpoint / restart
// ---------------------------------------------------------------------------

namespace {

// Layout: header, the bound arrays, the FP32 state when one is running, then
// an 8-byte checksum of everything before it.
constexpr char CK_MAGIC[8] = {'S', 'W', 'A', 'P', 'C', 'K', 'P', '2'};

// A 64-bit checksum of the first `len` bytes of a file, 8-byte words at a time
// (xor, multiply by the FNV prime, fold the high bits down).  Detects a
// truncated or altered checkpoint; not a cryptographic hash.
bool file_checksum(const char* path, long long len, uint64_t* out) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  uint64_t h = 1469598103934665603ULL;
  std::vector<unsigned char> buf((std::size_t)1 << 22);
  long long left = len;
  bool ok = true;
  while (left > 0) {
    const std::size_t want = (std::size_t)std::min<long long>(left, (long long)buf.size());
    if (std::fread(buf.data(), 1, want, f) != want) {
      ok = false;
      break;
    }
    std::size_t i = 0;
    for (; i + 8 <= want; i += 8) {
      uint64_t w;
      std::memcpy(&w, buf.data() + i, 8);
      h = (h ^ w) * 1099511628211ULL;
      h ^= h >> 29;
    }
    for (; i < want; ++i) h = (h ^ buf[i]) * 1099511628211ULL;
    left -= (long long)want;
  }
  std::fclose(f);
  *out = h;
  return ok;
}

struct CkHead {
  char magic[8];
  swap_dims dims;
  swap_params prm;
  int64_t ni_tot, src_step;
  uint64_t chex_total;
  int32_t have_srcs, f32;
  swap_sources srcs;
};

// The bound host real arrays in a fixed order, as (start, element count);
// elements are c->real_bytes wide.
std::vector<std::pair<char*, std::size_t>> host_arrays(swap_ctx* c, std::size_t N) {
  const std::size_t C = (std::size_t)c->g.C, NM = (std::size_t)c->dims.ni_max, rb = (std::size_t)c->real_bytes;
  auto at = [rb](double* a, std::size_t off) { return reinterpret_cast<char*>(a) + off * rb; };
  std::vector<std::pair<char*, std::size_t>> v;
  for (double* a : {c->h_xp, c->h_vp, c->h_vp1})
    for (int m = 0; m < 3; ++m) v.push_back({at(a, m * NM), N});
  v.push_back({at(c->h_mrat, 0), N});
  v.push_back({at(c->h_beta_p, 0), N});
  for (double* a : {c->h_b0, c->h_b1, c->h_b12, c->h_b1p2, c->h_bt, c->h_btc, c->h_up, c->h_aj, c->h_E})
    v.push_back({at(a, 0), 3 * C});
  v.push_back({at(c->h_np, 0), C});
  v.push_back({at(c->h_nu, 0), C});
  return v;
}

}  // namespace

extern "C" int swap_checkpoint_write(swap_ctx* c, const char* path) {
  if (!c || !path) return SWAP_EINVAL;
  if (!c->h_xp || !c->h_b1) return c->fail(SWAP_EINVAL, "swap_bind_particles and swap_bind_fields are required");
  TRY(swap_sync_to_host(c, nullptr));
  CkHead h{};
  std::memcpy(h.magic, CK_MAGIC, 8);
  h.dims = c->dims;
  h.prm = c->prm;
  h.ni_tot = c->ntot();
  h.src_step = c->src_step;
  unsigned long long* cnt = c->have_srcs ? srcops::counters(c) : nullptr;
  if (cnt && cudaMemcpy(&h.chex_total, cnt + 1, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    return c->fail(SWAP_ECUDA, "checkpoint counters");
  h.have_srcs = c->have_srcs ? 1 : 0;
  h.srcs = c->srcs;
  h.f32 = (c->f32_state && !swap_f32_ended(c)) ? 1 : 0;
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return c->fail(SWAP_EINVAL, std::string("cannot open ") + path);
  int r = std::fwrite(&h, sizeof(h), 1, f) == 1 ? SWAP_OK : c->fail(SWAP_EINVAL, "checkpoint write failed");
  for (auto& a : host_arrays(c, (std::size_t)h.ni_tot))
    if (!r && a.second && std::fwrite(a.first, (std::size_t)c->real_bytes, a.second, f) != a.second)
      r = c->fail(SWAP_EINVAL, "checkpoint write failed");
  if (!r && h.f32) r = swap_f32_checkpoint(c, f, true);
  long long len = r ? 0 : (long long)std::ftell(f);
  if (std::fclose(f) != 0 && !r) r = c->fail(SWAP_EINVAL, "checkpoint close failed");
  if (!r) {  // the checksum trailer
    uint64_t sum = 0;
    std::FILE* g = nullptr;
    if (len < 0 || !file_checksum(path, len, &sum) || !(g = std::fopen(path, "ab")) ||
        std::fwrite(&sum, 8, 1, g) != 1)
      r = c->fail(SWAP_EINVAL, "checkpoint checksum write failed");
    if (g && std::fclose(g) != 0 && !r) r = c->fail(SWAP_EINVAL, "checkpoint close failed");
  }
  return r;
}

extern "C" int swap_checkpoint_read(swap_ctx* c, const char* path) {
  if (!c || !path) return SWAP_EINVAL;
  if (!c->h_xp || !c->h_b1) return c->fail(SWAP_EINVAL, "swap_bind_particles and swap_bind_fields are required");
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return c->fail(SWAP_EINVAL, std::string("cannot open ") + path);
  {  // the whole file against its checksum trailer, before anything is read
    uint64_t want = 0, got = 1;
    long long size = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) size = (long long)std::ftell(f);
    const bool ok = size >= (long long)sizeof(CkHead) + 8 && std::fseek(f, size - 8, SEEK_SET) == 0 &&
                    std::fread(&want, 8, 1, f) == 1 && file_checksum(path, size - 8, &got) && want == got;
    if (!ok || std::fseek(f, 0, SEEK_SET) != 0) {
      std::fclose(f);
      return c->fail(SWAP_EINVAL, "checkpoint truncated or corrupted (checksum mismatch)");
    }
  }
  CkHead h{};
  int r = std::fread(&h, sizeof(h), 1, f) == 1 ? SWAP_OK : c->fail(SWAP_EINVAL, "not a checkpoint");
  if (!r && std::memcmp(h.magic, CK_MAGIC, 8) != 0) r = c->fail(SWAP_EINVAL, "not a checkpoint of this library");
  if (!r && (h.dims.nx != c->dims.nx || h.dims.ny != c->dims.ny || h.dims.nz != c->dims.nz))
    r = c->fail(SWAP_EINVAL, "checkpoint grid differs from the context's");
  if (!r && (h.dims.real_bytes == 4 ? 4 : 8) != c->real_bytes)
    r = c->fail(SWAP_EINVAL, "checkpoint real size differs from the context's");
  if (!r && h.ni_tot < 0) r = c->fail(SWAP_EINVAL, "checkpoint holds a negative ion count");
  if (!r && h.ni_tot > c->dims.ni_max) r = c->fail(SWAP_ECAPACITY, "checkpoint holds more ions than Ni_max");
  if (!r) {
    for (auto& a : host_arrays(c, (std::size_t)h.ni_tot))
      if (!r && a.second && std::fread(a.first, (std::size_t)c->real_bytes, a.second, f) != a.second)
        r = c->fail(SWAP_EINVAL, "checkpoint truncated");
  }
  if (!r) {
    *c->ni_tot_ptr = (int32_t)h.ni_tot;
    r = swap_mark_host_dirty(c, nullptr);  // (each failure below still closes the file)
    c->weights_valid = false;
    if (!r && h.have_srcs) r = swap_set_sources(c, &h.srcs, h.src_step);
    if (!r && h.have_srcs) {
      unsigned long long* cnt = srcops::counters(c);
      if (!cnt || cudaMemcpy(cnt + 1, &h.chex_total, 8, cudaMemcpyHostToDevice) != cudaSuccess)
        r = c->fail(SWAP_ECUDA, "checkpoint counters");
    }
  }
  if (!r && h.f32) {
    r = swap_f32_begin(c);
    if (!r) r = swap_f32_checkpoint(c, f, false);
  }
  std::fclose(f);
  return r;
}
