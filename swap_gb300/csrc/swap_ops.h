// swap_ops.h -- device-side operators shared between the translation units
// of the FP64 drop-in; every pointer argument is a device pointer.
#pragma once

#include "k32.cuh"
#include "swap_ctx.h"

namespace ops {
int get_interp_weights(swap_ctx* c, const double* xp);
int update_np(swap_ctx* c, double* np);
// update_up with the velocity chosen by mode (0 v, 1 1.5v-0.5v1, 2 0.5(v+ + v-)).
int update_up_mode(swap_ctx* c, int mode, const double* va, const double* vb, double* out_v1, const double* np,
                   double* up);
int update_rho(swap_ctx* c, double* mnp);
// Energies of the bound FP64 state: kinetic, |b1-b0|^2, |b1|^2, |E|^2 and
// the x, y, z parts of |b1-b0|^2 (normalized units, full 3D).
int energy7(swap_ctx* c, double out[7]);
int get_temperature(swap_ctx* c, const double* vp, const double* np, double* temp_p);
}  // namespace ops

// Particle sources and sinks (swap_sources.cu).  Each updates *ni_tot.
namespace srcops {
bool x_open(const swap_ctx* c);
// Start of a fused step: ionization, cloud ionization, inflow.
int step_begin(swap_ctx* c, double* xp, double* vp, double* vp1);
// After each half move: outflow removal when x is open.
int after_move(swap_ctx* c, double* xp, double* vp, double* vp1);
// End of a fused step: res_chex, then the step counter advances.
int step_end(swap_ctx* c, double* xp, double* vp, double* vp1);
void free_all(swap_ctx* c);
// [0] last res_chex, [1] total exchanges (allocated on first use).
unsigned long long* counters(swap_ctx* c);

// New ions of one step staged for the FP32 form's sort: their state, the
// key of their cell, their rank among the new ions of that key, and the
// count per key.  Grown on demand; freed by stage_free.
struct F32Stage {
  swapk32::Part part{};
  int32_t *key = nullptr, *rank = nullptr, *ncount = nullptr;
  long long cap = 0, nkeys = 0;
  uint8_t sp_ion = 0, sp_cloud = 0, sp_inflow = 0;
};
bool any_rule(const swap_ctx* c);
// Stage the new ions of step m: n_host + *n_dev ions (n_dev may be null), at
// most n_max, in staging order ionize, cloud, inflow.
int f32_stage(swap_ctx* c, const swapk32::G32& g, F32Stage& st, long long m, long long* n_host,
              const int64_t** n_dev, long long* n_max);
void stage_free(F32Stage& st);
}  // namespace srcops
