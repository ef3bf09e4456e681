// swap_ctx.h -- host-side state behind a swap_ctx handle.
#pragma once

#include <cstddef>
#include <cstdio>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"
#include "k64.cuh"

enum class MirrorKind { Grid, Particle3, Particle1, ParticleI3 };
enum class Access { In, Out, InOut };

// A caller's host array and its device copy, with which side is current.
struct Mirror {
  void* host = nullptr;
  void* dev = nullptr;
  std::size_t bytes = 0;
  MirrorKind kind = MirrorKind::Grid;
  bool host_valid = true;
  bool dev_valid = false;
  // a real array of a caller built with 4-byte reals: the host copy holds
  // floats, the device mirror doubles; transfers convert (see real_bytes)
  bool host_f32 = false;
};

struct ProfEntry {
  const char* name;
  double ms;
  long long launches;
};

struct swap_ctx {
  swap_dims dims{};
  swap_params prm{};
  swapk::Geo g{};
  cudaStream_t st = nullptr;
  int* d_err = nullptr;
  std::string err;

  // registry of bound host arrays
  std::unordered_map<const void*, Mirror> reg;
  std::vector<Mirror*> touched;
  std::vector<Mirror*> touched_host;  // outputs written straight into the caller's memory
  // On Grace-Blackwell the GPU reads and writes the caller's (pageable or
  // page-locked) memory over NVLink-C2C at the link's speed: the FP32 form's
  // conversions then read and write the FP64 particle arrays in place, with
  // no staging copy through the device mirror.
  bool host_direct = false;
  // Size of the caller's REAL (swap_dims.real_bytes): 8, or 4 for the
  // reference's own build (makefile:1, -real-size 32).  The device state is
  // FP64 either way; with 4, every registered real array is converted on its
  // way to and from the device.
  int real_bytes = 8;
  // multi-rank exchange of the fused entries' deposits (swap_set_exchange)
  swap_exchange_fn xfn = nullptr;
  void* xuser = nullptr;
  bool fused = false;  // inside a fused FP64 step: its deposits are exchanged
  uint32_t wait_polls = 1u << 22;  // bound of the device waits (swap_set_wait_limit)
  // deterministic FP64 deposits (swap_set_deterministic): fixed-point sums
  // for up to 3 C values, allocated on first use
  bool deterministic = false;
  swapk::Fix64 fix{nullptr, nullptr};
  float* stage32 = nullptr;   // device staging of those conversions
  std::size_t stage32_n = 0;  // its capacity in floats
  int64_t h2d_bytes = 0, d2h_bytes = 0;  // bytes moved between the caller's memory and the device
  std::vector<void*> owned;  // device buffers freed at finalize

  // host addresses of the bound arrays (the Fortran's own)
  double *h_xp = nullptr, *h_vp = nullptr, *h_vp1 = nullptr, *h_mrat = nullptr, *h_beta_p = nullptr;
  int32_t* h_ijkp = nullptr;
  int32_t* ni_tot_ptr = nullptr;
  double *h_b0 = nullptr, *h_b1 = nullptr, *h_b12 = nullptr, *h_b1p2 = nullptr, *h_bt = nullptr, *h_btc = nullptr;
  double *h_np = nullptr, *h_up = nullptr, *h_aj = nullptr, *h_E = nullptr, *h_nu = nullptr;
  std::vector<double> h_qx, h_qy, h_qz;

  // device state of the implicit COMMON blocks
  double *d_mrat = nullptr, *d_beta_p = nullptr;
  int32_t* d_ijk = nullptr;   // /ion_info/ ijkp
  double* d_wght = nullptr;   // /weights/ wght
  bool weights_valid = false;
  long long weights_n = 0;

  // grid scratch: /dummy/ a, c, ct and subroutine locals
  double *s_a = nullptr, *s_aa = nullptr, *s_c = nullptr, *s_ct = nullptr, *s_btcl = nullptr, *s_btc2 = nullptr;
  double *s_btmf = nullptr, *s_ajc = nullptr, *s_upc = nullptr, *s_btp1 = nullptr, *s_S = nullptr;
  double *s_gf = nullptr, *s_gpc = nullptr, *s_dtn = nullptr, *s_red = nullptr;
  // particle work arrays of the fused step (maind.f locals Ep, vplus, vminus)
  double *w_Ep = nullptr, *w_vplus = nullptr, *w_vminus = nullptr;
  double last_dtsub = 0, last_ntf = 0;
  double mion = 1.0;  // ion mass of update_rho / get_temperature (normalized units: 1)
  void* f32_state = nullptr;  // the FP32 form (swap_f32.cu)
  void* diag_state = nullptr; // diagnostic output files (swap_diag.cu)

  // particle sources and sinks (swap_sources.cu)
  swap_sources srcs{};
  bool have_srcs = false;
  long long src_step = 0;                    // step counter of the next fused step
  long long src_cap = 0;                     // capacity of the scan scratch
  int64_t *src_flag = nullptr, *src_pos = nullptr, *src_sums = nullptr;
  void* src_tmp = nullptr;                   // ni_max elements of 8 bytes
  unsigned long long* src_cnt = nullptr;     // [0] last res_chex, [1] fused-step total

  cudaEvent_t t0 = nullptr, t1 = nullptr;

  // per-kernel profile (CUDA events), filled by the fused paths
  bool prof_on = false;
  std::vector<ProfEntry> prof;
  struct ProfPending {
    int idx, kernels;
    cudaEvent_t a, b;
  };
  std::vector<ProfPending> prof_pending;
  std::vector<cudaEvent_t> prof_pool;

  int fail(int code, const std::string& msg);
  int cuda_fail(cudaError_t e, const char* where);
  double* dalloc(std::size_t n);
  Mirror* find(const void* host);
  // bytes: the DEVICE mirror's size; real: a real array (float on the host
  // when real_bytes is 4)
  int add_mirror(void* host, std::size_t bytes, MirrorKind kind, bool real = true);
  int transfer(Mirror& m, bool to_dev);
  int use(const void* host, Access acc, double** dev);
  // As use(), but with host_direct an input whose host copy is current, and
  // every output, resolves to the caller's own memory.
  int use_host(const void* host, Access acc, double** ptr, bool* direct);
  int begin();
  int finish();
  // The rank sum of a deposit's raw node sums through the caller's callback
  // (no-op without one).  kind: bytes per real of data.
  int exchange(void* data, long long count, int kind);
  long long ntot() const;
  swapk::PartDev part_view();
  void prof_free();
};

void swap_f32_free(swap_ctx* c);
bool swap_f32_ended(swap_ctx* c);  // the FP32 state was written back by swap_f32_end
void swap_diag_free(swap_ctx* c);
// The FP32 state to or from an open checkpoint file (swap_f32.cu).
int swap_f32_checkpoint(swap_ctx* c, std::FILE* f, bool write);
