// k64.cuh -- launchers of the FP64 kernels (k64.cu).  Every launcher enqueues
// on `st` and returns the launch status.  Grids are device arrays in Fortran
// layout (x fastest, component slowest, stride C); particles are (ni_max,3).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "swap_dev.cuh"

namespace swapk {

struct PartDev {  // device mirrors of the particle arrays
  double *xp, *vp, *vp1, *mrat, *beta_p;
  int32_t* ijk;   // (ni_max,3), 1-based cell indices like ijkp
  double* wght;   // (ni_max,8)
  long long NM;   // leading dimension ni_max
};

// boundary.f
cudaError_t periodic3(const Geo& g, double* b, cudaStream_t st);
cudaError_t periodic1(const Geo& g, double* b, cudaStream_t st);

// grid_interp.f / gutsf.f operators on the interior nodes
cudaError_t face_to_center_int(const Geo& g, const double* v, double* vc, cudaStream_t st);
cudaError_t edge_to_center_int(const Geo& g, const double* bt, double* btc, cudaStream_t st);
cudaError_t face_avg_int(const Geo& g, const double* ct, double* cc, cudaStream_t st);
cudaError_t cross_int(const Geo& g, const double* aa, const double* btc, double* ct, cudaStream_t st);
cudaError_t curlB_int(const Geo& g, const double* b1, const double* np, double* aj, double alpha, cudaStream_t st);
cudaError_t sub_int(const Geo& g, const double* aj, const double* up, double* a, cudaStream_t st);
cudaError_t e_from_c_int(const Geo& g, const double* c, const double* nu, const double* aj, const double* np,
                         double grad_pe, double* E, cudaStream_t st);
cudaError_t curlE_update_int(const Geo& g, const double* E, const double* base, double coef, double* b1p2,
                             cudaStream_t st);
cudaError_t half_sum_all(const Geo& g, const double* a, const double* b, double* out, cudaStream_t st);
cudaError_t deltat_all(const Geo& g, const double* bt, const double* np, double alpha, double dx, double* dtn,
                       cudaStream_t st);
cudaError_t grad_pe_face_int(const Geo& g, const double* np, double grad_pe, double* gf, cudaStream_t st);

// gutsp.f particle operators
cudaError_t interp_weights(const Geo& g, const PartDev& p, long long N, int* err, cudaStream_t st);
// Deterministic deposits: each added value x goes into a 128-bit fixed-point
// sum in units of 2^-60, as floor(x * 2^28) into a signed 64-bit word (h)
// and the rest * 2^32, rounded, into an unsigned one (l).  Integer adds are
// exact and commutative, so the sum does not depend on the order of the
// GPU's atomics; |x| < 2^25 per value (SWAP_ENONFINITE otherwise).
struct Fix64 {
  long long* h;
  unsigned long long* l;
};
// fix (h, l null: plain FP64 atomics into np) ...
cudaError_t deposit_np(const Geo& g, const PartDev& p, long long N, double beta, double* np, int* err,
                       cudaStream_t st, Fix64 fix = Fix64{nullptr, nullptr});
// out[t] = the fixed-point sums (h[t], l[t]) rounded to FP64, t < n.
cudaError_t fix_to_double(long long n, Fix64 fix, double* out, cudaStream_t st);
// mode: 0 = v, 1 = 1.5 v - 0.5 v1 (extrapol_up), 2 = 0.5 (a + b) (improve_up, also stores into out_v1),
// 3 = (v/sqrt(mrat))^2 and 4 = v/sqrt(mrat) per component (get_temperature)
cudaError_t deposit_u(const Geo& g, const PartDev& p, long long N, double beta, int mode, const double* va,
                      const double* vb, double* out_v1, double* S, int* err, cudaStream_t st,
                      Fix64 fix = Fix64{nullptr, nullptr});
cudaError_t ct_from_sums(const Geo& g, const double* S, const double* np, double* ct, cudaStream_t st);
// update_rho deposit (folded into the interior), interior scaling, and the
// temperature of get_temperature from the two face moments.
cudaError_t deposit_rho(const Geo& g, const PartDev& p, long long N, double beta, double* mnp, int* err,
                        cudaStream_t st);
cudaError_t scale_interior(const Geo& g, double* f, double a, cudaStream_t st);
cudaError_t temperature(const Geo& g, const double* up2, const double* upa, double mion, double* temp,
                        cudaStream_t st);
cudaError_t get_Ep(const Geo& g, const PartDev& p, long long N, const double* ajc, const double* upc,
                   const double* btc, const double* gpc, double* Ep, int* err, cudaStream_t st);
cudaError_t vplus_vminus(const Geo& g, const PartDev& p, long long N, double dt, const double* Ep,
                         const double* btc, const double* vp, double* vplus, double* vminus, int* err,
                         cudaStream_t st);
cudaError_t vp_final(const PartDev& p, long long N, double dt, const double* Ep, double* vp, double* vp1,
                     const double* vplus, cudaStream_t st);
// x_open: the x axis does not wrap (particles leaving are removed after the
// move by the caller).
cudaError_t move_half(const Geo& g, const PartDev& p, long long N, double dt, double* xp, const double* vp,
                      bool x_open, cudaStream_t st);

// reductions (FP64)
cudaError_t reduce_min(const double* x, long long n, double* d_partial, int nblk, cudaStream_t st);
cudaError_t energy_parts(const Geo& g, const PartDev& p, long long N, double beta, double alpha, const double* vp,
                         const double* b0, const double* b1, const double* E, double* d_acc4, cudaStream_t st);
cudaError_t divb_max(const Geo& g, const double* b, double* d_max, cudaStream_t st);
cudaError_t count_nonfinite(const double* x, long long n, unsigned long long* d_cnt, cudaStream_t st);
// A caller's 4-byte reals to the device's doubles (exact) and back (rounded
// to nearest).
cudaError_t widen_f32(const float* in, double* out, long long n, cudaStream_t st);
cudaError_t narrow_f64(const double* in, float* out, long long n, cudaStream_t st);

}  // namespace swapk
