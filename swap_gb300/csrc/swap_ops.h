// swap_ops.h -- device-side operators shared between the translation units
// of the FP64 drop-in; every pointer argument is a device pointer.
#pragma once

#include "swap_ctx.h"

namespace ops {
int get_interp_weights(swap_ctx* c, const double* xp);
int update_np(swap_ctx* c, double* np);
// update_up with the velocity chosen by mode (0 v, 1 1.5v-0.5v1, 2 0.5(v+ + v-)).
int update_up_mode(swap_ctx* c, int mode, const double* va, const double* vb, double* out_v1, const double* np,
                   double* up);
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
}  // namespace srcops
