// k32.cuh -- the FP32 form of the ion step: device structures and launchers.
//
// Particles: packed int32 cell (ci | cj<<10 | ck<<20, 0-based physical cells)
// plus FP32 offsets inside the cell, FP32 v and vp1, a species byte.  They
// are kept sorted by a brick-major key (bricks of 4x4x4 cells), so one CTA
// owns one brick's particles as a contiguous range.  Grids keep the
// reference's (nx,ny,nz[,3]) layout with ghosts; B is accumulated in
// double-float (float hi + lo pairs) and its perturbation dB = B - b0 is
// mirrored in FP32 for the stencils.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace swapk32 {

constexpr int BR = 4;                 // brick edge (cells)
constexpr int BCELLS = BR * BR * BR;  // 64 cells per brick
constexpr int TN = BR + 3;            // tile nodes per axis: brick + one-cell mover halo
constexpr int TNODES = TN * TN * TN;  // 343
// Passes 1 and 2 deposit and gather only in their ions' own cells (no move
// before them): a tile of brick + 1 node per axis, origin one node lower.
constexpr int TN_IN = BR + 1;
constexpr int TNODES_IN = TN_IN * TN_IN * TN_IN;  // 125
// Tile nodes per axis of the passes' deposit tiles (and of k_node_sum).
__host__ __device__ constexpr int pass_tile(int pass) { return pass == 3 ? TN : TN_IN; }
constexpr int NDIR = 27;              // displacements in {-1,0,1}^3
constexpr int MAX_SPECIES = 16;
// Inputs per voxel of the field surrogate: B (3), u_p (3), n_p, p_e, E0 (3),
// and B - b12 (3), the change over the last subcycle (the predictor is a
// leapfrog from b12, so the subcycles depend on it as well as on B).
constexpr int SUR_NIN = 14;

struct G32 {
  int nx, ny, nz;     // nodes incl. ghosts
  int ncx, ncy, ncz;  // physical cells
  int nbx, nby, nbz;  // bricks
  long long C;        // nodes
  long long nkeys;    // bricks * 64
  long long nbricks;
  float dx, dy, dz, inv_dx, inv_dy, inv_dz;
  double qx1, qy1, qz1;  // q(1) per axis
};

// Elements past the capacity that every particle array is allocated with:
// the passes copy 128-ion chunks from 16-aligned starts.
constexpr int PASS_PAD = 256;

struct Part {
  int32_t* cell;
  float *ox, *oy, *oz;
  float *vx, *vy, *vz;
  float *wx, *wy, *wz;  // vp1
  uint8_t* sp;
};

struct Species {
  float mrat[MAX_SPECIES];
  float qw[MAX_SPECIES];  // 1/(dx*dy*dz*beta*beta_p): density weight of one particle
  int n;
};

// Flags in the packed cell word.  A dead ion (outflow) is skipped by every
// pass and dropped by the next sort; a fresh ion was created by a source for
// the coming step (P1 clears the flag, or drops the ion at the end of a run).
constexpr int32_t CELL_DEAD = -1;
constexpr int32_t CELL_FRESH = 1 << 30;

struct StepParams {
  float dt;
  int x_open;        // x does not wrap; ions leaving in x are marked dead
  int chex;          // P3: res_chex after the step's last move
  long long chex_step;
  uint64_t seed;
  float cx_a, cx_b, cloud_N0, inv_r0sq, cloud_x, cloud_y, cloud_z;
  uint8_t heavy_of[MAX_SPECIES];     // species after charge exchange
  unsigned long long* chex_count;    // exchanges, accumulated
  uint32_t wait_polls;               // polls of a chunk's copy before a pass gives up
};

// Ions that moved more than one cell per axis in one step (|v| dt > dx: the
// reference handles any move, gutsp.f:454-570, 1378-1435) leave the fast
// path: pass 3 lists them, far_deposit adds their moments to the brick
// partials, and the sort places them after the near arrivals of their new
// key, in array order.  At most FAR_CAP per step; a larger number, or a
// half move of more than the grid's extent less two cells, fails the step.
constexpr int FAR_CAP = 1 << 16;
struct FarList {
  long long* idx;             // the ion's index in the pass's buffer
  long long* key;             // its new key; -1 when it left the grid
  int32_t* dcell;             // packed cell of its deposit position; -1: none
  float* o;                   // deposit offsets, [3][FAR_CAP]
  float* q;                   // qw and qw * v, [4][FAR_CAP]
  int* n;                     // entries this step (above FAR_CAP: the step fails)
  unsigned long long* total;  // ions that took this path since the state began
};

__host__ __device__ __forceinline__ int pk_i(int32_t c) { return c & 1023; }
__host__ __device__ __forceinline__ int pk_j(int32_t c) { return (c >> 10) & 1023; }
__host__ __device__ __forceinline__ int pk_k(int32_t c) { return (c >> 20) & 1023; }
__host__ __device__ __forceinline__ int32_t pk(int i, int j, int k) { return i | (j << 10) | (k << 20); }

__host__ __device__ __forceinline__ long long key_of(const G32& g, int i, int j, int k) {
  const long long b = (long long)(i >> 2) + (long long)g.nbx * ((j >> 2) + (long long)g.nby * (k >> 2));
  return b * BCELLS + (i & 3) + 4 * (j & 3) + 16 * (k & 3);
}
__host__ __device__ __forceinline__ void cell_of_key(const G32& g, long long key, int& i, int& j, int& k) {
  // 32-bit division: keys < 2^30
  const unsigned b = (unsigned)(key / BCELLS), nbx = (unsigned)g.nbx, nby = (unsigned)g.nby;
  const int l = (int)(key % BCELLS);
  const unsigned r = b / nbx, r2 = r / nby;
  const int bi = (int)(b - r * nbx), bj = (int)(r - r2 * nby), bk = (int)r2;
  i = bi * 4 + (l & 3);
  j = bj * 4 + ((l >> 2) & 3);
  k = bk * 4 + (l >> 4);
}

// FP64 position -> (cell, offset): the reference's cell rules on a uniform
// grid (x, z: q(i) < x <= q(i+1); y: floor(y/dy)), offsets in cell units.
__device__ __forceinline__ bool split_axis(double x, double q1, double d, int n, bool upper_closed, int& c, float& o) {
  const double u = (x - q1) / d;  // position in cells from node 1
  int i = upper_closed ? (int)ceil(u) - 1 : (int)floor(u);
  if (i < 0 || i >= n) return false;
  // u - i is exact and lies in (0,1] (upper closed) or [0,1): only the
  // rounding to float can reach the excluded end
  const double f = u - (double)i;
  c = i;
  o = (float)f;
  if (upper_closed && o <= 0.0f) o = 1e-7f;
  if (!upper_closed && o >= 1.0f) o = 0.99999994f;
  return true;
}

// Offset of x inside a known cell c, clamped to (0,1] or [0,1).
__device__ __forceinline__ float offset_in_cell(double x, double q1, double d, int c, bool upper_closed) {
  double f = (x - q1) / d - (double)c;
  float o;
  if (upper_closed) {
    o = (float)(f > 1.0 ? 1.0 : f);
    if (!(o > 0.0f)) o = 1e-7f;
  } else {
    o = (float)(f < 0.0 ? 0.0 : f);
    if (!(o < 1.0f)) o = 0.99999994f;
  }
  return o;
}

// ---- particle passes ----
// Particles lie in their sorted key's cell at P1 and P2; every move happens
// in P3, and the sort that follows restores the order.
// P1: deposit np and up at v_n = 1.5 v - 0.5 vp1 (maind.f:385-387, 399).
// P2: gather, Ep, v-/v+, deposit up at 0.5(v+ + v-) (maind.f:400-402).
// P3: gather, Ep, v-/v+, vp1 = v, v = v+ + dt/2 Ep, half move, deposit np and
//     up there (maind.f:404-413), the second half move (maind.f:479),
//     outflow and res_chex; writes each particle's sort direction and rank
//     (dirrank) and the per-key direction counts (dep, direction-major:
//     dep[dir * nkeys + key]) when those are given, and lists the ions that
//     moved more than one cell in `far` (required for pass 3).
// Moment sums (exact): each warp sums a cell's ions in FP32, and those run
// sums go into the brick tile (two 32-bit words per node), then the brick
// partials (64-bit), as fixed-point integers in units of 2^-32: exact and
// independent of the order of the adds, rounded to FP32 once per node by
// node_sum.  exact = false: FP32 atomics (kept to
// measure what the exact sums gain).  partial: 8 bytes per tile entry.
cudaError_t pass(int which, const G32& g, const Part& p, const Species& sp, const StepParams& sprm,
                 const int64_t* start, const float4* kit, void* partial, uint32_t* dirrank, uint16_t* dep, int* err,
                 bool exact, cudaStream_t st, const FarList* far = nullptr, const float4* kitg = nullptr);
// The moments of pass 3's far list into the brick partials (pass 3's tiles).
cudaError_t far_deposit(const G32& g, const FarList& far, void* partial, bool exact, int* err, cudaStream_t st);
// Add the far list's arrivals to the per-key counts (before the scan).
cudaError_t far_count(const FarList& far, int64_t* count, cudaStream_t st);
// The far list's survivors to start_new[X+1] - ncount[X] - (far arrivals of
// X) + (their rank by array index); ncount may be null.
cudaError_t far_scatter(const G32& g, const FarList& far, const int32_t* ncount, const int64_t* start_new,
                        const Part& src, const Part& dst, long long cap, int* err, cudaStream_t st);
// Sum the brick partial tiles into np and S (interior nodes, (nx,ny,nz) layout).
// pass: the pass (1-3) whose tiles `partial` holds
cudaError_t node_sum(const G32& g, int pass, const void* partial, int nq, bool exact, float* np, float* S,
                     cudaStream_t st);

// ---- fields ----
cudaError_t ct_and_up(const G32& g, const float* np, const float* S, float* up, cudaStream_t st);
// kitg (may be null): the electron-pressure face gradient of np (grad_pe
// gp) centred per node, for the passes' gathered E.
cudaError_t build_kit(const G32& g, const float* aj, const float* up, const float* dbt, const float* b0c,
                      const float* np, float gp, float4* kit, float4* kitg, cudaStream_t st);
// gpf: the electron-pressure gradient at every face (with ghost images),
// which E subtracts (the isothermal extension of gutsf.f:1083,1283).
cudaError_t gpe_faces(const G32& g, const float* np, float gp, float* gpf, cudaStream_t st);
cudaError_t curlB32(const G32& g, const float* dbt, const float* np, float alpha, float* aj, cudaStream_t st);
// One half of a field subcycle in two fused kernels: aj and the cross
// product ct (predictor: B from dB; corrector: B at m+1/2), then E on the
// fly, curlE and B_new = base - coef*curlE in double-float (hi, lo float
// pairs) with its FP32 dB (and, predictor, dB at m+1/2 = (dB_new + dB1)/2).
cudaError_t aj_ct(const G32& g, bool corr, const float* db, const float* np, const float* up, const float* b0c,
                  float alpha, float* aj, float* ct, cudaStream_t st);
// e_acc (may be null): the step's E summed over the correctors.
// gpf (may be null): the electron-pressure face gradient E subtracts.
cudaError_t b_step(const G32& g, bool pred, bool write_e, const float* ct, const float* nu, const float* aj,
                   const float* gpf, const float* bh, const float* bl, double coef, const float* b0c, float* oh,
                   float* ol, float* dbo, const float* db1, float* dbtp1, float* E, float* e_acc, cudaStream_t st);
// The surrogate's field advance: B_new = base - coef * curl E for a given E.
cudaError_t b_step_given_e(const G32& g, const float* E, const float* bh, const float* bl, double coef,
                           const float* b0c, float* oh, float* ol, float* dbo, cudaStream_t st);
// r = b_new + f*(b_old - b_new) (double-float, hi parts of b_old).
cudaError_t df_lerp(const G32& g, const float* nh, const float* nl, const float* oh, float f, float* rh, float* rl,
                    cudaStream_t st);
// Surrogate inputs per interior node, FP32 [V][SUR_NIN]: B, u_p, n_p,
// te*n_p, E0 = ct + nu aj (zero when ct is null) and B - b12 from the
// double-float levels (b1h, b1l) and (b12h, b12l) (zero when b12h is null).
cudaError_t grid_to_voxels(const G32& g, const float* db, const float* b0c, const float* up, const float* np,
                           float te, const float* ct, const float* aj, const float* nu, const float* gpf,
                           const float* b1h, const float* b1l, const float* b12h, const float* b12l, float* out,
                           cudaStream_t st);
// Sums over the interior of |B_a - B_b|^2, |B_b|^2 and |B_b - b0|^2.
cudaError_t judge_sums(const G32& g, const float* ah, const float* al, const float* bh, const float* bl,
                       const float* b0c, double* acc3, cudaStream_t st);
// [V][3] <-> the field layout (ghost images written): E = ev + E0 of vin,
// and ev = f*E - E0 of vin (no E0 when vin is null).
cudaError_t voxels_to_grid(const G32& g, const float* ev, const float* vin, float* E, cudaStream_t st);
cudaError_t grid_e_to_voxels(const G32& g, const float* E, float f, const float* vin, float* ev, cudaStream_t st);
// FP64 <-> double-float (hi + lo).
cudaError_t split_df(long long n, const double* a, float* h, float* l, cudaStream_t st);
cudaError_t join_df(long long n, const float* h, const float* l, double* a, cudaStream_t st);
cudaError_t courant_min(const G32& g, const float* dbt, const float* b0c, const float* np, float alpha, float dx,
                        float* dtn, float* d_min, cudaStream_t st);

// ---- sort ----
// Sort words and the direction-major counts dep[dir * nkeys + key] without pass 3.
cudaError_t sort_prep(const G32& g, const int64_t* start, const int32_t* cell, uint32_t* dirrank, uint16_t* dep,
                      int* err, cudaStream_t st);
// ncount (may be null): new ions per key, placed after the arrivals.  order:
// the BCELLS x NDIR table of sort_order_table on the device.  pre is
// direction-major: pre[dir * nkeys + key].
cudaError_t sort_count(const G32& g, const uint16_t* dep, const int32_t* ncount, const uint8_t* order,
                       int64_t* count, uint16_t* pre, int* err, cudaStream_t st);
// Directions by increasing source key for every place in a brick (host).
void sort_order_table(uint8_t* out);
cudaError_t scan_exclusive(const int64_t* in, int64_t* out, long long n, int64_t* block_sums, cudaStream_t st);
// Survivors to start_new[X] + pre + rank; removed ions are skipped; cap = ni_max.
cudaError_t sort_scatter(const G32& g, long long N, long long cap, const int32_t* cell, const uint32_t* dirrank,
                         const uint16_t* pre, const int64_t* start_new, const Part& src, const Part& dst, int* err,
                         cudaStream_t st);
// Staged new ions q < n_host + *n_dev (n_dev may be null) to
// start_new[X+1] - ncount[X] + rank[q], flagged fresh; cap = ni_max.
cudaError_t new_scatter(const G32& g, long long n_host, const int64_t* n_dev, long long n_max, const Part& stage,
                        const int32_t* key, const int32_t* rank, const int32_t* ncount, const int64_t* start_new,
                        const Part& dst, long long cap, int* err, cudaStream_t st);

// ---- conversions ----
cudaError_t from_f64(const G32& g, long long N, long long NM, const double* xp, const double* vp, const double* vp1,
                     const double* mrat, const double* beta_p, const Species& sp, Part p, int* err,
                     cudaStream_t st);
cudaError_t to_f64(const G32& g, long long N, long long NM, const Part& p, double* xp, double* vp, double* vp1,
                   cudaStream_t st);
// mrat, beta_p from the species ids through the FP64 tables.
cudaError_t species_to_f64(long long N, const uint8_t* spid, const double* tab_mrat, const double* tab_bp,
                           double* mrat, double* beta_p, cudaStream_t st);
cudaError_t keys_of(const G32& g, long long N, const int32_t* cell, int32_t* key, cudaStream_t st);
// The state's ions in FP64 without those created for a step that is not
// taken (CELL_FRESH) or removed, in their order; kept_out: how many.
// bcount, bstart (N / (8 TPB) + 2 each) and sums are scratch.
cudaError_t to_f64_kept(const G32& g, long long N, long long NM, const Part& p, const double* tab_mrat,
                        const double* tab_bp, double* xp, double* vp, double* vp1, double* mrat, double* beta_p,
                        int64_t* bcount, int64_t* bstart, int64_t* sums, long long* kept_out, cudaStream_t st);
cudaError_t gather_perm(long long N, const int64_t* perm, const Part& src, Part dst, cudaStream_t st);
cudaError_t sorted_hist(long long N, const int32_t* key, long long nkeys, int* unsorted, int64_t* count,
                        cudaStream_t st);
cudaError_t grid_f64_to_f32(long long n, const double* a, const double* b, float* out, cudaStream_t st);
cudaError_t grid_f32_to_f64(long long n, const float* a, double* out, cudaStream_t st);
cudaError_t assign_species(long long N, const double* mrat, const double* beta_p, const double* tab_mrat,
                           const double* tab_bp, int n, uint8_t* spid, int* miss, cudaStream_t st);
// flag = 1 when a 3-component grid of C nodes per component is not uniform
// (every node equal to node 0 of its component)
cudaError_t not_uniform(long long C, const double* b, int* flag, cudaStream_t st);
cudaError_t energy32(const G32& g, long long N, const Part& p, const Species& sp, double vol, const double* b0,
                     const float* b1h, const float* b1l, const float* E, double alpha, double* acc4,
                     cudaStream_t st);

}  // namespace swapk32
