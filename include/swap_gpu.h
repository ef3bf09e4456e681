/* swap_gpu.h -- C-ABI of the GB300 (sm_103a) hybrid PIC ion step.
 *
 * Drop-in for the particle and field subroutines of SWAP (pdelamere/SWAP):
 * gutsp.f, gutsf.f, grid_interp.f and boundary.f.  A Fortran caller reaches
 * these entries through the bind(C) module in swap_gb300/fortran/, whose
 * wrappers keep the original subroutine names and argument lists; the C
 * entries take the same arguments in the same order plus a context.
 *
 * Data model.
 *   - Arrays are the caller's host arrays in Fortran layout: grids
 *     (nx,ny,nz[,3]) column-major, x fastest, component slowest; particles
 *     (ni_max,3) column-major.  Indices are int32 (-i4, makefile:1).
 *   - Reals are the caller's REAL: swap_dims.real_bytes = 4 for SWAP as its
 *     makefile builds it (makefile:1, -real-size 32: every REAL array is
 *     float), 8 (or 0) for IEEE double.  The device computes in FP64 either
 *     way; with 4, each registered real array is widened on its way to the
 *     device and rounded back to float on its way to the host.  The array
 *     parameters below are declared double*: a caller with 4-byte reals
 *     passes its float arrays there (the entries only use the address to find
 *     the registered array).  Scalars passed by value or through a double*
 *     to a single value (dtsub, ntf, energy sums) are double in both
 *     settings, and so are the coordinate arrays of swap_coords.
 *   - Every host array an entry receives must first be registered
 *     (swap_bind_particles / swap_bind_fields / swap_bind_array).  The context
 *     keeps a device mirror of each and tracks which copy is current: an entry
 *     uploads an input whose device copy is stale, runs on the device, and
 *     marks its outputs device-current.  swap_sync_to_host() brings results
 *     back; swap_mark_host_dirty() tells the context the caller changed a host
 *     array.  The implicit COMMON state of the reference (ijkp, wght,
 *     /dummy/ a,c,ct) lives on the device inside the context.
 *   - Every entry returns 0 on success and a SWAP_E* code otherwise; the
 *     message is in swap_last_error(ctx).  No entry aborts, exits or traps.
 *   - Calls on one context must not run concurrently.  Entries are
 *     synchronous on return.
 *   - This library never calls MPI.  In a multi-rank run the deposit entries
 *     still return the folded, complete moments of the local particles; the
 *     caller keeps its MPI_ALLREDUCE (gutsp.f:1503,1812-1822).
 */
#ifndef SWAP_GPU_H
#define SWAP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SWAP_OK 0
#define SWAP_EINVAL 1        /* bad argument (null, size, unregistered array) */
#define SWAP_ECUDA 2         /* CUDA runtime error (allocation, launch)       */
#define SWAP_EDOMAIN 3       /* a particle lies outside the grid               */
#define SWAP_ECAPACITY 4     /* ni_tot > ni_max or a work buffer too small     */
#define SWAP_ENONFINITE 5    /* non-finite value found by swap_check_finite    */
#define SWAP_ESUBCYCLE 6     /* subcycle count overflow in check_time_step     */
#define SWAP_EMOVE 7         /* a particle moved more than one cell in a step  */
#define SWAP_EWAIT 8         /* a device wait reached its iteration limit      */
#define SWAP_EEXCHANGE 9     /* the caller's exchange callback returned nonzero */

typedef struct swap_ctx swap_ctx;

/* Grid and particle capacity: dimensions.f:5,9 (nx,ny,nz,Ni_max). */
typedef struct swap_dims {
  int32_t nx, ny, nz;
  int32_t real_bytes;  /* size of the caller's REAL: 4, or 8 (0 means 8) */
  int64_t ni_max;
} swap_dims;

/* Scalars of module `inputs`/`global` that the hot path reads. */
typedef struct swap_params {
  double dt;         /* ion step (inputs.f:141)                               */
  double alpha;      /* mu0/1e3*q*q/m (inputs.f:170)                          */
  double beta;       /* particle scale factor (misc.f:462-475)                */
  double dx, dy;     /* module dx, dy; dy enters the y cell index (gutsp.f:1404) */
  double grad_pe;    /* isothermal T_e/m of the electron-pressure extension;
                        0 = the reference's E (no pressure term)              */
  int32_t ntsub;     /* field subcycles per ion step (inputs.f:140)           */
  int32_t flags;     /* reserved, 0                                           */
} swap_params;

/* The /coords/ COMMON block (global.f:27-38) as 0-based copies of the
 * 1-based Fortran arrays: qx[0] holds qx(1).  Lengths nx, ny or nz. */
typedef struct swap_coords {
  const double *qx, *qy, *qz;
  const double *dx_grid, *dy_grid, *dz_grid;
  const double *dx_cell, *dy_cell, *dz_cell;
  const double *xrat, *yrat, *zrat;
} swap_coords;

/* ---- lifecycle ---- */
int swap_init(swap_ctx** ctx, const swap_dims* dims, const swap_params* params, const swap_coords* coords);
int swap_finalize(swap_ctx* ctx);
const char* swap_last_error(const swap_ctx* ctx);
int swap_abi_version(void);

/* ---- multi-rank particle decomposition ---- */
/* The reference decomposes the ions over MPI ranks, each with a full copy of
 * the grid, and sums every moment deposit over the ranks (MPI_ALLREDUCE,
 * gutsp.f:1503,1812-1822; maind.f:140).  A context holds one rank's ions.
 * With an exchange callback set, the fused entries (swap_ion_step_pre,
 * swap_ion_step, swap_run, swap_f32_run) call it after every moment deposit
 * with that rank's raw node sums -- the density and the velocity sums, before
 * the division by the density -- and the callback must replace them in place
 * by their sum over the ranks before it returns.
 *   data:   device array of `count` reals; kind 8 (double, FP64 drop-in) or
 *           4 (float, FP32 form);
 *   stream: the cudaStream_t the deposit's kernels are queued on; the
 *           reduction must come after them: queued on that stream
 *           (ncclAllReduce(data, data, count, ..., stream)) or after
 *           cudaStreamSynchronize(stream).
 * A nonzero return ends the entry with SWAP_EEXCHANGE.  The per-subroutine
 * entries never call it: their caller keeps its own MPI_ALLREDUCE.  With more
 * than one rank, give the sources to one rank (inflow_ppc and nu_ion zero on
 * the others, x_open on all so that every rank's ions flow out) and a
 * different seed per rank for charge exchange.  swap_f32_energy's kinetic
 * term is the rank's own: sum it over the ranks.  fn = NULL switches the
 * exchange off (one rank). */
typedef int (*swap_exchange_fn)(void* user, void* data, int64_t count, int32_t kind, void* stream);
int swap_set_exchange(swap_ctx* ctx, swap_exchange_fn fn, void* user);

/* ---- failure detection ---- */
/* Every device wait of the FP32 form's particle passes (a chunk's bulk copy)
 * polls at most `polls` times (default 4194304, about a second), then the
 * pass stops, lets the copies already started land, and the entry returns
 * SWAP_EWAIT; the context stays usable, the FP32 state does not (call
 * swap_f32_begin again: the bound arrays still hold the state it began from).
 * 0 makes every wait give up at once, to test that path. */
int swap_set_wait_limit(swap_ctx* ctx, uint32_t polls);
/* on != 0: the FP64 drop-in's moment deposits (update_np, update_up and the
 * fused steps') sum in 128-bit fixed point (units of 2^-60, |value| < 2^25
 * per particle and corner, SWAP_ENONFINITE beyond) instead of FP64 atomics,
 * then round once per node.  The result does not depend on the order of the
 * GPU's adds: runs repeat bit for bit and a run resumed from a checkpoint
 * equals the uninterrupted one.  Off by default (FP64 atomics). */
int swap_set_deterministic(swap_ctx* ctx, int32_t on);

/* ---- array registration and data movement ---- */
/* The particle arrays of maind.f:54-59 and global.f:44,96,100; ijkp may be
 * NULL.  ni_tot is the caller's Ni_tot (global.f:41), read at every call. */
int swap_bind_particles(swap_ctx* ctx, double* xp, double* vp, double* vp1, double* mrat, double* beta_p,
                        int32_t* ijkp, int32_t* ni_tot);
/* The grid arrays of maind.f:38-70. */
int swap_bind_fields(swap_ctx* ctx, double* b0, double* b1, double* b12, double* b1p2, double* bt, double* btc,
                     double* np, double* up, double* aj, double* E, double* nu);
/* Any other real array an entry is handed (e.g. Ep, vplus, vminus): bytes
 * is its size in the caller's memory (real_bytes per element). */
int swap_bind_array(swap_ctx* ctx, void* host, int64_t bytes);
/* host = NULL: every registered array. */
int swap_sync_to_device(swap_ctx* ctx, const void* host);
int swap_sync_to_host(swap_ctx* ctx, void* host);
int swap_mark_host_dirty(swap_ctx* ctx, const void* host);
/* On by default where the device addresses host memory directly (Grace-
 * Blackwell, NVLink-C2C): swap_f32_begin then reads the FP64 particle arrays
 * xp, vp, vp1 in the caller's memory when the host copy is current, and
 * swap_f32_end writes xp, vp, vp1, mrat and beta_p straight back (the host
 * copy becomes current, the device copy stale).  0 = always stage through
 * the device mirrors.  SWAP_EINVAL if the device cannot, or if the context
 * binds 4-byte reals (the direct conversions read doubles). */
int swap_set_host_direct(swap_ctx* ctx, int on);
/* Bytes moved from the caller's memory to the device (h2d) and back (d2h)
 * since the last reset: mirror copies and direct reads and writes. */
int swap_transfer_bytes(swap_ctx* ctx, int64_t* h2d, int64_t* d2h, int reset);

/* ---- one entry per reference subroutine (same arguments, same order) ---- */
int swap_get_interp_weights(swap_ctx* ctx, const double* xp);                          /* gutsp.f:1378 */
int swap_update_np(swap_ctx* ctx, double* np);                                          /* gutsp.f:1441 */
int swap_update_up(swap_ctx* ctx, const double* vp, const double* np, double* up);      /* gutsp.f:1649 */
int swap_extrapol_up(swap_ctx* ctx, double* up, const double* vp, const double* vp1,
                     const double* np);                                                 /* gutsp.f:127  */
int swap_get_Ep(swap_ctx* ctx, double* Ep, double* aj, const double* np, double* up, const double* btc,
                const double* nu);                                                      /* gutsp.f:155  */
int swap_get_vplus_vminus(swap_ctx* ctx, const double* Ep, const double* btc, const double* vp,
                          double* vplus, double* vminus);                               /* gutsp.f:281  */
int swap_improve_up(swap_ctx* ctx, double* vp1, const double* vplus, const double* vminus, double* up,
                    const double* np);                                                  /* gutsp.f:407  */
int swap_get_vp_final(swap_ctx* ctx, const double* Ep, double* vp, double* vp1,
                      const double* vplus);                                             /* gutsp.f:433  */
/* x does not wrap when swap_set_sources opened the x axis (x_open). */
int swap_move_ion_half(swap_ctx* ctx, double* xp, const double* vp, const double* vp1,
                       double* input_p);                                                /* gutsp.f:454  */
int swap_curlB(swap_ctx* ctx, double* bt, const double* np, double* aj);                /* gutsf.f:178  */
int swap_edge_to_center(swap_ctx* ctx, double* bt, double* btc);                        /* grid_interp.f:10 */
int swap_face_to_center(swap_ctx* ctx, double* v, double* vc);                          /* grid_interp.f:136 */
int swap_get_E(swap_ctx* ctx, double* E, const double* b0, double* bt, double* aj, const double* up,
               const double* np, const double* nu);                                     /* gutsf.f:994  */
/* dtsub is the module variable of global.f:76 that the Fortran reads. */
int swap_predict_B(swap_ctx* ctx, double* b0, double* b1, double* b12, double* b1p2, double* bt, double* E,
                   double* aj, double* up, double* np, double* nu, double dtsub);       /* gutsf.f:1115 */
int swap_correct_B(swap_ctx* ctx, double* b0, double* b1, double* b1p2, double* E, double* aj, double* up,
                   double* np, double* nu, double dtsub);                               /* gutsf.f:1309 */
int swap_f_update_tlev(swap_ctx* ctx, double* b1, double* b12, double* b1p2, double* bt,
                       const double* b0);                                               /* gutsf.f:10   */
/* dtsub/ntf in and out (global.f:76-77; ntf is real there). */
int swap_check_time_step(swap_ctx* ctx, const double* bt, const double* np, double* dtsub,
                         double* ntf);                                                  /* gutsf.f:1776 */
int swap_periodic(swap_ctx* ctx, double* b);                                            /* boundary.f:9 */
int swap_periodic_scalar(swap_ctx* ctx, double* b);                                     /* boundary.f:167 */
/* Diagnostics moments of the output block (maind.f:515-517), from the
 * ijkp/wght of the last get_interp_weights, as the reference.  mion is the
 * ion mass (swap_set_mion; 1 in normalized units). */
int swap_update_rho(swap_ctx* ctx, double* mnp);                                        /* gutsp.f:1517 */
int swap_get_temperature(swap_ctx* ctx, const double* xp, const double* vp, const double* np,
                         double* temp_p);                                               /* gutsp.f:2257 */
int swap_set_mion(swap_ctx* ctx, double mion);

/* ---- fused, device-resident ion step on the bound arrays ---- */
int swap_ion_step_pre(swap_ctx* ctx);     /* maind.f:385-413 */
int swap_field_subcycles(swap_ctx* ctx);  /* maind.f:420-476 */
int swap_ion_step_post(swap_ctx* ctx);    /* maind.f:479     */
int swap_ion_step(swap_ctx* ctx);         /* maind.f:385-479 */
int swap_run(swap_ctx* ctx, int32_t nsteps);

/* ---- particle sources and sinks (FP64 path) ----
 * Random draws are Philox4x32-10 keyed by (seed, rule) with counters (ion
 * step, slot, draw block), replacing the compiler's random_number
 * (misc.f:24).  Counts are exact functions of the draws.
 *   ndot > 0       Ionize_sw_mp (chem_rates.f:508-646): pickup ring ions.
 *   x_open != 0    x axis open: the moves do not wrap x, ions leaving through
 *                  x <= q(1) or x > q(nx-1) are removed after each move, and
 *                  a drifting Maxwellian enters from a one-cell ghost slab
 *                  (inflow_ppc per face cell) at the start of each step.
 *   nu_ion > 0     ionization of a neutral cloud n_n = N0/(1+(r/r0)^2) per
 *                  cell, after Ionize_pluto_mp (chem_rates.f:290-503); new
 *                  heavy ions (mrat_heavy, beta_heavy) at rest.
 *   cx_a > 0       res_chex (chem_rates.f:805-843): each non-heavy ion turns
 *                  heavy and at rest with probability
 *                  dt*n_n*(cx_a - cx_b ln|v|)*|v|.
 * swap_ion_step / swap_run apply them in this order: ionize, cloud, inflow
 * at the start of a step; outflow removal after both half moves; res_chex
 * after the last move (maind.f:484).  step0 is the step counter of the next
 * fused step; the separate entries take the step number m_tstep. */
typedef struct swap_sources {
  uint64_t seed;
  double ndot, vsw, beta_pu, mrat_pu, delz_ref;   /* Ionize_sw_mp            */
  int32_t x_open, inflow_ppc;                     /* open x axis, inflow      */
  double inflow_vth, inflow_ux, inflow_uy, inflow_uz;
  double cloud_N0, cloud_r0, cloud_x, cloud_y, cloud_z, nu_ion, mrat_heavy, beta_heavy;
  double cx_a, cx_b;                              /* res_chex cross section  */
} swap_sources;
int swap_set_sources(swap_ctx* ctx, const swap_sources* src, int64_t step0);
/* Ions exchanged by res_chex in the fused steps since swap_set_sources. */
int swap_chex_count(swap_ctx* ctx, int64_t* count);
/* Appends the new ions after Ni_tot, then get_interp_weights, update_np,
 * update_up (chem_rates.f:641-643).  input_p is not updated. */
int swap_Ionize_sw_mp(swap_ctx* ctx, double* np, double* vp, double* vp1, double* xp, int32_t m_tstep,
                      double* input_p, double* up);                                     /* chem_rates.f:508 */
/* Order-preserving removal of ion ion_l (1-based), shifting xp, vp, vp1,
 * mrat, beta_p and the device ijkp/wght down by one. */
int swap_remove_ion(swap_ctx* ctx, double* xp, double* vp, double* vp1, int32_t ion_l);   /* gutsp.f:12 */
int swap_res_chex(swap_ctx* ctx, double* xp, double* vp, int32_t m_tstep, int64_t* count); /* chem_rates.f:805 */
int swap_inflow_x(swap_ctx* ctx, int32_t m_tstep);
int swap_ionize_cloud(swap_ctx* ctx, int32_t m_tstep);
int swap_remove_outflow_x(swap_ctx* ctx);

/* ---- diagnostic output (maind.f:237-358, 498-573) ----
 * Fortran sequential unformatted files in out_dir (which must end with a
 * path separator, as the reference's out_dir): para.dat at open; every
 * swap_diag_step writes c.energy.dat and c.momentum.dat; every nout-th step
 * also c.np, c.b1 (bt), c.aj (aj*alpha*face-averaged np), c.E, c.up,
 * c.temp_p (get_temperature/1.6e-19), c.mnp (update_rho), the particle
 * files c.xp_0, c.vp_0, c.mrat_0, c.beta_p_0 (rank > 0: c.xp_<rank> ...),
 * and zero-filled c.np_b, c.mixed, c.up_t, c.up_b, whose producers the
 * reference does not call.  The energy record holds (input_E, input_EeP,
 * Evp, Euf, EB1, EB1x, EB1y, EB1z, EE, EeP, input_chex, input_bill) with
 * the full-3D normalized energies of swap_energy and 0 for fluid terms.
 * Reads the FP64 state: with the FP32 form call swap_f32_end first. */
typedef struct swap_diag_spec {
  int32_t nt;          /* steps of the run (para.dat)                        */
  int32_t nout;        /* dump every nout steps (inputs.dat nout)            */
  int32_t real_bytes;  /* 4 (the reference's -real-size 32) or 8             */
  int32_t rank;        /* 0 writes every file; k > 0 only its particles      */
  double dtsub_init, vtop, vbottom, mion, m_pu, m_heavy, np_top, np_bottom, b0_top, b0_bottom, vth_top,
      vth_bottom;      /* para.dat scalars; mion also sets swap_set_mion      */
} swap_diag_spec;
int swap_diag_open(swap_ctx* ctx, const char* out_dir, const swap_diag_spec* spec);
int swap_diag_step(swap_ctx* ctx, int32_t m);
int swap_diag_close(swap_ctx* ctx);

/* ---- checkpoint / restart (the role of restart.vars, maind.f:208-226,
 * 586-607, in this library's own binary layout) ----
 * write: the bound arrays (synced to the host first), Ni_tot, the sources and
 * their step counter and, when the FP32 form is running, its whole state.
 * read: into a context with the same grid and arrays bound; restores the
 * host arrays and, for an FP32 checkpoint, the FP32 state bit for bit. */
int swap_checkpoint_write(swap_ctx* ctx, const char* path);
int swap_checkpoint_read(swap_ctx* ctx, const char* path);

/* ---- the FP32 form of the fused step ----
 * Particle positions as int32 cell + FP32 offset, FP32 velocities and
 * moments, B accumulated across subcycles in double-float (pairs of floats,
 * 48 significant bits: GB300's FP64 rate is a small fraction of its FP32
 * rate).  The sources and sinks of swap_set_sources apply, with new ions
 * drawn as in the FP64 path and charge exchange drawn per sorted ion.  Needs a uniform grid with
 * 8..1024 physical cells per axis in multiples of 4, a uniform b0, at most 16
 * (mrat, beta_p) species.  An ion that moves more than one cell per axis in
 * a step takes a slower path (listed by pass 3, deposited and sorted apart,
 * at most 65536 per step); a half move that spans the grid less two cells,
 * or more such ions, gives SWAP_EMOVE.
 * begin converts the bound FP64 state; end writes it back into the bound
 * arrays' device mirrors, with the particles in cell-sorted order. */
int swap_f32_begin(swap_ctx* ctx);
int swap_f32_run(swap_ctx* ctx, int32_t nsteps);
int swap_f32_end(swap_ctx* ctx);
int swap_f32_energy(swap_ctx* ctx, double out[4]);
/* Ions in the FP32 state (sources and sinks change it step by step). */
int swap_f32_count(swap_ctx* ctx, int64_t* n);
/* Ions that moved more than one cell per axis in a step and took the slower
 * path, summed since swap_f32_begin. */
int swap_f32_far_movers(swap_ctx* ctx, int64_t* n);
/* Where each sort key's ions start in the FP32 state's sorted order:
 * starts[0..nkeys], nkeys = (cells/4 per axis, multiplied) * 64, key =
 * brick * 64 + cell in the brick (x fastest, bricks x fastest), so key q
 * holds starts[q+1] - starts[q] ions.  n = entries of starts (>= nkeys+1). */
int swap_f32_key_starts(swap_ctx* ctx, int64_t* starts, int64_t n);
/* Moment sums of the FP32 form.  exact = 1 (the default after
 * swap_f32_begin): each warp sums a cell's ions in FP32, and those sums are
 * accumulated per brick and over the bricks as fixed-point integers (units of
 * 2^-32) -- exact, so a node's moment is its warp sums' exact total rounded
 * once to FP32, and the same whatever order the GPU adds in (the FP32 form's
 * steps are then reproducible bit for bit).  A warp sum or node moment of
 * 2^15 or more, or a non-finite one, ends the step with SWAP_ENONFINITE; a
 * brick may hold any number of ions.  exact = 0: FP32 atomics, kept to
 * measure what the exact sums gain. */
int swap_f32_set_moment_sums(swap_ctx* ctx, int exact);
/* Validation: move particles idx[q] of the current (sorted) order by one
 * cell step per axis (dcell[q] = (dx+1) | (dy+1)<<10 | (dz+1)<<20) and run
 * the stable incremental sort that follows each ion step. */
int swap_f32_displace_resort(swap_ctx* ctx, int64_t n, const int64_t* idx, const int32_t* dcell);

/* ---- diagnostics (FP64, device reductions) ---- */
/* out[0] kinetic, out[1] |b1-b0|^2 field, out[2] |b1|^2 field, out[3] |E|^2,
 * in the normalized units of the oracle (part_init.f:14-139 sums the j=2
 * plane only; this is the full-3D form). */
int swap_energy(swap_ctx* ctx, double out[4]);
int swap_max_abs_divB(swap_ctx* ctx, const double* b, double* out);
/* SWAP_ENONFINITE if any registered array holds a NaN or Inf. */
int swap_check_finite(swap_ctx* ctx);

/* ---- particle loading (host, product-side; replaces part_init.f:146-232) ---- */
typedef struct swap_load_spec {
  uint64_t seed;
  uint32_t stream;       /* species / population id mixed into the key   */
  int32_t ppc;           /* particles per physical cell (stratified load) */
  double vth;            /* reference convention: v = vth*sqrt(-ln U)*cos(pi U') */
  double ux, uy, uz;     /* bulk flow                                     */
  double mrat;           /* q/m relative to H+ (global.f:100)             */
  double beta_p;         /* statistical weight factor (global.f:96)       */
} swap_load_spec;
/* Fill particles first .. first+ncell*ppc-1 (0-based) with a stratified
 * Maxwellian over the physical cells of coords; returns the count in *count. */
int swap_load_maxwellian_host(const swap_dims* dims, const swap_coords* coords, const swap_load_spec* spec,
                              double* xp, double* vp, double* vp1, double* mrat, double* beta_p, int64_t first,
                              int64_t* count);

/* ---- allocation-free deposit (no counterpart in the reference) ---- */
/* For callers that cannot call cudaMalloc: a host whose device memory is
 * owned by another allocator, or a caller that cannot let cudaMalloc/cudaFree
 * synchronize the device inside its step.  Such a caller cannot create a
 * swap_ctx.  swap_update_up_noalloc computes the same moment as
 * swap_get_interp_weights + swap_update_up (gutsp.f:1378-1435, 1649-1842)
 * from the caller's DEVICE arrays xp, vp (ni_max,3), beta_p (ni_max), np
 * (nx,ny,nz) into the caller's device array up (nx,ny,nz,3), on `stream`
 * (a cudaStream_t; NULL = default stream), and returns after that stream
 * finishes (it waits on that one stream, not on the device).  coords are
 * host arrays, as for swap_init.
 *   - It allocates nothing.  Its scratch is one file-scope device array of
 *     SWAP_NOALLOC_SCRATCH_BYTES that every GPU loading this library holds
 *     until the process exits.
 *   - No call can be captured in a CUDA graph: each call reads its flag
 *     back and waits for its stream.
 *   - The first call on a device resolves that array's address
 *     (cudaGetSymbolAddress) and keeps it; make no call on a device after
 *     cudaDeviceReset there.  After an error the entry waits for its stream
 *     before returning.
 *   - All calls share the array and each call clears the part it uses first;
 *     calls that overlap on the GPU race, so serialize them.
 *   - More than SWAP_NOALLOC_MAX_NODES nodes, or more than
 *     SWAP_NOALLOC_MAX_AXIS nodes on an axis, returns SWAP_ECAPACITY.  A
 *     particle outside the grid returns SWAP_EDOMAIN. */
#define SWAP_NOALLOC_MAX_NODES (1 << 20)
#define SWAP_NOALLOC_MAX_AXIS 4096
#define SWAP_NOALLOC_SCRATCH_BYTES (8 * (3 * (SWAP_NOALLOC_MAX_AXIS + 1) + 3 * SWAP_NOALLOC_MAX_NODES))
int swap_update_up_noalloc(const swap_dims* dims, const swap_params* params, const swap_coords* coords,
                           const double* xp, const double* vp, const double* beta_p, int64_t ni_tot,
                           const double* np, double* up, void* stream);

/* ---- tensor-core check (no counterpart in the reference) ----
 * D = A * B^T on the 5th-generation tensor cores (tcgen05, BF16 in, FP32
 * accumulate) for device arrays A (128 x K bf16, row-major), B (32 x K bf16,
 * row-major) and D (128 x 32 FP32); K a multiple of 16 up to 256.  The GEMM
 * core of the surrogate's convolutions, exposed so its operand layout can be
 * checked against a CPU product. */
int swap_tc_gemm_check(const void* A, const void* B, float* D, int32_t K);
/* One periodic 3x3x3 convolution layer of the surrogate on the tensor cores:
 * device arrays X [V][cin] bf16 (V = nx*ny*nz voxels, x fastest, a multiple
 * of 128), W [27][cout][cin] bf16 with tap = (dz+1)*9 + (dy+1)*3 + (dx+1),
 * bias [cout] FP32 or NULL; writes Y [V][cout] bf16 (GELU applied when gelu
 * is nonzero) and/or Yf [V][cout] FP32 (before the activation).
 * (cin, cout) in {(16,32), (32,32), (32,16), (16,16)}. */
int swap_conv3_check(int32_t nx, int32_t ny, int32_t nz, int32_t cin, int32_t cout, const void* X, const void* W,
                     const float* bias, void* Y, float* Yf, int32_t gelu);

/* ---- the learned field-subcycle surrogate (FP32 form) ----
 * A 3D convolutional network (swap_surrogate_layers periodic 3x3x3 layers,
 * 14 -> W -> ... -> W -> 3 channels with W = swap_surrogate_width, GELU;
 * BF16 weights and activations, FP32 accumulation on the tensor cores) maps
 * the state at the start of the field subcycles (B, u_p, n_p, p_e, E0, the
 * plain E there, and B - b12, the change over the last subcycle that the
 * leapfrog predictor starts from) to the step's mean corrector E minus E0; B then advances as B - dt curl E, so
 * div B stays where it was.  It is trained on pairs the plain subcycles of
 * swap_surrogate_collect produce, with Adam.
 * Attached to a context, it replaces the subcycles; every judge_every-th
 * step both run, the plain result is kept, and a B rel-L2 difference above
 * bound (or, with swap_surrogate_set_db_bound, a difference relative to
 * B - b0 above that bound) switches the network off until a judged step
 * passes. */
typedef struct swap_surrogate swap_surrogate;
int swap_surrogate_create(swap_surrogate** net, uint64_t seed, int32_t max_samples);
int swap_surrogate_destroy(swap_surrogate* net);
const char* swap_surrogate_last_error(const swap_surrogate* net);
/* nsteps FP32 steps of ctx (after swap_f32_begin) with the plain subcycles,
 * each adding one training pair. */
int swap_surrogate_collect(swap_surrogate* net, swap_ctx* ctx, int32_t nsteps);
int swap_surrogate_samples(swap_surrogate* net, int32_t* n);
/* epochs of Adam over the pairs; loss = mean squared normalised E error of
 * the last epoch, plus curl_w * mean |curl e|^2 / kref2 when a curl weight is
 * set (e the E error, so curl e is the B error per unit dt; kref2 = mean
 * |curl target|^2 of the training pairs, or the value given). */
int swap_surrogate_train(swap_surrogate* net, int32_t epochs, double lr, double* loss);
int swap_surrogate_loss(swap_surrogate* net, double* loss);
int swap_surrogate_set_curl_weight(swap_surrogate* net, double curl_w, double kref2);
/* relative != 0: each pair's loss and gradient scaled by kref2 over its own
 * mean |curl target|^2 (clamped to [0.1, 100]), so every pair counts by its
 * relative error. */
int swap_surrogate_set_pair_weighting(swap_surrogate* net, int32_t relative);
/* cuda_cores != 0: the training's weight gradients on the CUDA cores instead
 * of the tensor cores (the same sums in another order; kept for checking). */
int swap_surrogate_set_weight_grad_cores(swap_surrogate* net, int32_t cuda_cores);
/* The network's depth (conv layers) and the channels of its hidden layers. */
int swap_surrogate_layers(int32_t* n);
int swap_surrogate_width(int32_t* w);
int swap_surrogate_attach(swap_ctx* ctx, swap_surrogate* net, int32_t judge_every, double bound);
/* bound_db > 0: a judged step also falls back when the network's B differs
 * from the subcycles' by more than bound_db relative to the plain B - b0
 * (the field's perturbation, not the field); 0 (the default): B alone. */
int swap_surrogate_set_db_bound(swap_ctx* ctx, double bound_db);
/* [0] steps by the network, [1] judged steps, [2] fallbacks, [3] last judged
 * B rel-L2, [4] last judged (B - b0) rel-L2. */
int swap_surrogate_stats(swap_ctx* ctx, double out[5]);
/* Test access: normalisation (14 input means and stds, output scale) and
 * FP32 master weights of a layer ([27][cout][cin] with (cin, cout) = (16,W)
 * for the first, (W,16) for the last and (W,W) between, W the hidden width
 * of swap_surrogate_width: padded channels zero) with its bias; get or set. */
int swap_surrogate_norm(swap_surrogate* net, float* mean, float* stdv, float* out_mean, float* out_std,
                        int32_t set);
int swap_surrogate_weights(swap_surrogate* net, int32_t layer, float* w, float* b, int32_t set);
/* One forward and backward pass on device inputs [V][14] and targets [V][3]
 * of an nx*ny*nz box: loss = 0.5 mean((out - (tgt - out_mean)/out_std)^2)
 * (plus 0.5 curl_w mean |curl e|^2 / kref2 with a curl weight), gradients of
 * every layer into grads as (gW0, gb0, gW1, gb1, ...). */
int swap_surrogate_grads(swap_surrogate* net, int32_t nx, int32_t ny, int32_t nz, const float* vin, const float* tgt,
                         double* loss, float* grads);

/* ---- timing (CUDA events on the context's stream) ---- */
int swap_timer_start(swap_ctx* ctx);
int swap_timer_stop(swap_ctx* ctx, double* ms);
/* Per-kernel CUDA-event timing of the fused path; names are static strings. */
int swap_profile_enable(swap_ctx* ctx, int on);
int swap_profile_read(swap_ctx* ctx, int32_t max, const char** names, double* total_ms, int64_t* launches,
                      int32_t* n);
int swap_profile_reset(swap_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* SWAP_GPU_H */
