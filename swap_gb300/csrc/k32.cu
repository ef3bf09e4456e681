// k32.cu -- kernels of the FP32 form (see k32.cuh for the data layout).
#include <mutex>
#include <type_traits>

#include "k32.cuh"
#include "philox.h"
#include "swap_dev.cuh"
#include "tc05.cuh"

namespace swapk32 {
namespace {

constexpr int TPB = 256;
constexpr int TPB_PASS = 128;  // particle passes: keeps the shared tiles under 48 KB
// Chunk buffers of the particle passes: chunks k+1 .. k+PASS_STAGES-1 are in
// flight while chunk k is processed (more bytes in flight per SM hides more
// of the HBM latency; each stage costs one chunk of shared memory).
#ifndef SWAP_PASS_STAGES
#define SWAP_PASS_STAGES 2
#endif
constexpr int PASS_STAGES = SWAP_PASS_STAGES;
// Polls of a chunk's mbarrier when a pass that gave up lets its copies in
// flight land before it exits (the wait itself is bounded by
// StepParams::wait_polls).
constexpr uint32_t STAGE_WAIT_POLLS = 1u << 22;
// the device error codes of every kernel (swap_dev.cuh), as ints
constexpr int KERR_DOMAIN = swapk::KERR_DOMAIN, KERR_CAPACITY = swapk::KERR_CAPACITY, KERR_MOVE = swapk::KERR_MOVE,
              KERR_WAIT = swapk::KERR_WAIT, KERR_RANGE = swapk::KERR_RANGE;

inline unsigned nblk(long long n, int tpb = TPB) {
  const long long b = (n + tpb - 1) / tpb;
  return (unsigned)(b < 1 ? 1 : b);
}

#define GSTRIDE(t, n) \
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (n); t += (long long)gridDim.x * blockDim.x)

__device__ __forceinline__ void set_err(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// dirrank of ions the 27-direction sort does not place: a failed move,
// removed, and moved more than one cell (placed from the far list)
constexpr uint32_t DR_BAD = 0xffffffffu, DR_DEAD = 0xfffffffeu, DR_FAR = 0xfffffffdu;

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// 0-based linear index of 1-based node (i,j,k) in the (nx,ny,nz) layout
__device__ __forceinline__ long long nid(const G32& g, int i, int j, int k) {
  return (long long)(i - 1) + (long long)g.nx * ((long long)(j - 1) + (long long)g.ny * (long long)(k - 1));
}
// node index of physical node (p,q,r), p in [0,ncx): 1-based i = p + 2
__device__ __forceinline__ long long pid(const G32& g, int p, int q, int r) { return nid(g, p + 2, q + 2, r + 2); }
// interior image of a 1-based node index (ghost 1 -> n-1, ghost n -> 2)
__device__ __forceinline__ int img(int i, int n) { return i == 1 ? n - 1 : (i == n ? 2 : i); }

// Store v at interior node (i,j,k) and at every ghost node whose image it
// is: the periodic fill of boundary.f:9-52 fused into the producer.
template <class T>
__device__ __forceinline__ void store_img(const G32& g, T* f, int i, int j, int k, T v) {
  const int is[2] = {i, i == 2 ? g.nx : (i == g.nx - 1 ? 1 : -1)};
  const int js[2] = {j, j == 2 ? g.ny : (j == g.ny - 1 ? 1 : -1)};
  const int ks[2] = {k, k == 2 ? g.nz : (k == g.nz - 1 ? 1 : -1)};
  for (int a = 0; a < 2; ++a) {
    if (is[a] < 0) continue;
    for (int b = 0; b < 2; ++b) {
      if (js[b] < 0) continue;
      for (int c = 0; c < 2; ++c) {
        if (ks[c] < 0) continue;
        f[nid(g, is[a], js[b], ks[c])] = v;
      }
    }
  }
}

// 32-bit division: t < ncx*ncy*ncz <= 2^30 (64-bit division is a long
// emulated sequence)
__device__ __forceinline__ void interior_of(const G32& g, long long t, int& i, int& j, int& k) {
  const unsigned u = (unsigned)t, nx = (unsigned)g.ncx, ny = (unsigned)g.ncy;
  const unsigned r = u / nx, r2 = r / ny;
  i = (int)(u - r * nx) + 2;
  j = (int)(r - r2 * ny) + 2;
  k = (int)r2 + 2;
}

__host__ __device__ __forceinline__ long long n_int(const G32& g) { return (long long)g.ncx * g.ncy * g.ncz; }

// Move one axis of a (cell, offset) position by d cells.  upper_closed:
// offsets in (0,1] (the '>' cell search of x and z, gutsp.f:1396-1412);
// otherwise [0,1) (the floor of y, gutsp.f:1404).  Periodic in the cell
// index (gutsp.f:490-510, one wrap) when wrap; otherwise the cell may leave
// [0, n).  Returns false on a move that is not finite or spans n - 2 cells
// or more (one wrap then always lands in [0, n)).
__device__ __forceinline__ bool move_axis(int& c, float& o, float d, int n, bool upper_closed, bool wrap = true) {
  if (!(fabsf(d) < (float)(n - 2))) return false;
  o += d;
  // carry whole cells: (0,1] keeps o = 1 in the cell, [0,1) moves it up
  const float k = upper_closed ? ceilf(o) - 1.0f : floorf(o);
  o -= k;
  c += (int)k;
  if (upper_closed) {  // rounding can leave o at 0 or just above 1
    if (o <= 0.0f) { o += 1.0f; --c; }
  } else if (o >= 1.0f) {
    o -= 1.0f;
    ++c;
  }
  if (wrap) c = c < 0 ? c + n : (c >= n ? c - n : c);
  return true;
}

// Offset of a cell from a brick's first cell along one axis, unwrapped
// across the periodic boundary into the brick tile's window [-1, 4] when
// one of the periodic images lies there (n >= 8, so at most one does).
__device__ __forceinline__ int rel_cell(int c, int c0, int n) {
  int r = c - c0;
  if (r < -1) r += n;
  else if (r > 4) r -= n;
  return r;
}

// Step between two cells along one axis, unwrapped into [-1, 1] when one of
// the periodic images lies there.
__device__ __forceinline__ int step_cell(int c, int c0, int n) {
  int r = c - c0;
  if (r < -1) r += n;
  else if (r > 1) r -= n;
  return r;
}

// ---------------------------------------------------------------------------
// particle passes
// ---------------------------------------------------------------------------

__device__ __forceinline__ int dir_index(int dx, int dy, int dz) { return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1); }

// The warp's deposit (gutsp.f:1484-1491, 1704-1756): the 32 particles' 8
// corner weights and 4 moments go to shared memory as value-major rows; lane
// v = (moment q, corner c) then sums w_c * m_q down the runs of particles
// that share a cell (sorted particles: usually one or two runs), with the run
// ends known to the whole warp (tested per group of four particles), and adds
// each run's sum to the brick tile with one shared atomic.  t0: the tile index
// of the particle's lower corner node, -1 when it deposits nothing.  ALL_Q:
// every moment (otherwise the density, q = 0, is skipped).
// MOVERS (pass 3, which deposits after a half move): the runs follow trun,
// the particle's cell before the move (sorted, so runs stay long), and the
// few particles that changed cell (mover) take no part in them; each of
// those then adds its 32 values to the tile directly, one per lane.
// Exact moment sums (EXACT): a run sum x goes into the tile in fixed point,
// units of 2^-32, split over two 32-bit words per node (low words first, then
// the high words of all nodes): the high word takes h = floor(x * 2^16), the
// low word the rest, l = (x * 2^16 - h) * 2^16 rounded, in [0, 2^16].  Both
// are plain integer reductions (no returned value), exact and commutative,
// so a node's tile value sum(h) * 2^16 + sum(l) is the exact sum of its
// rounded run sums whatever order the warps add in.  The brick partials are
// written as 64-bit integers, summed the same way and rounded to FP32 once
// per node (k_node_sum).  Bounds: |x| < 2^15 per run sum and per node (the
// high words wrap, so only the total must fit); a larger or non-finite run
// sum is reported (KERR_RANGE).  A low word takes at most 2^16 per add and
// an ion adds at most once per node, so every CARRY_CHUNKS chunks of a brick
// the low words carry into the high words and any number of ions fits.
// Otherwise (plain): FP32 atomics, whose result depends on the order.
constexpr double FIX_INV = 1.0 / 4294967296.0;  // 2^-32
constexpr float FIX_MAX = 32768.0f;             // 2^15
constexpr int CARRY_CHUNKS = 256;               // 32768 ions: the low words stay below 2^32

// x in units of 2^-32 as the tile holds it: floor(x * 2^16) * 2^16 plus the
// rounded rest (the same two conversions as tile_add).
__device__ __forceinline__ long long to_fixed(float x) {
  const float xs = x * 65536.0f, fh = floorf(xs);
  return (long long)__float2int_rn(fh) * 65536LL + (long long)__float2uint_rn((xs - fh) * 65536.0f);
}

template <bool EXACT, int NT>
__device__ __forceinline__ void tile_add(void* tile, int i, float x, unsigned& bad) {
  if (EXACT) {
    // out of range or not finite: noted here, reported once at the pass's end
    // (a branch to the error word in this loop costs the passes 10%); the
    // conversions saturate, so the adds below stay defined
    bad |= fabsf(x) < FIX_MAX ? 0u : 1u;
    // x * 2^16 and its floor are exact floats; their difference is exact and
    // in [0, 1); only the low part rounds, below 2^-32
    const float xs = x * 65536.0f, fh = floorf(xs);
    unsigned* w = static_cast<unsigned*>(tile);
    atomicAdd(w + i, __float2uint_rn((xs - fh) * 65536.0f));
    atomicAdd(w + NT + i, (unsigned)__float2int_rn(fh));  // two's complement
  } else {
    atomicAdd(static_cast<float*>(tile) + i, x);
  }
}

template <bool ALL_Q, int T, bool MOVERS = false, bool EXACT = true>
__device__ __forceinline__ void warp_deposit(float (*red)[36], bool live, int t0, const float (&w8)[8],
                                             const float (&qdv)[4], void* tile, unsigned& bad, int lane,
                                             int trun = -1, bool mover = false) {
  const bool in_runs = live && !(MOVERS && mover);
#pragma unroll
  for (int c8 = 0; c8 < 8; ++c8) red[c8][lane] = live ? w8[c8] : 0.0f;
#pragma unroll
  for (int q = 0; q < 4; ++q) red[8 + q][lane] = in_runs ? qdv[q] : 0.0f;
  __syncwarp();
  const int key = MOVERS ? trun : t0;
  const int tprev = __shfl_up_sync(0xffffffffu, key, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || key != tprev);
  const unsigned ends = heads >> 1;  // the particle before each head (and, below, the last one)
  const int qv = lane >> 3, cv = lane & 7;
  const int off = (cv & 1) + T * (((cv >> 1) & 1) + T * (cv >> 2));
  const bool add_here = ALL_Q || qv != 0;
  const float4* wrow = reinterpret_cast<const float4*>(red[cv]);
  const float4* mrow = reinterpret_cast<const float4*>(red[8 + qv]);
  float acc = 0.0f;
#pragma unroll
  for (int h = 0; h < 2; ++h) {  // two halves of 16 particles, to bound the registers
    float x[16], m[16];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 v = wrow[4 * h + q], w = mrow[4 * h + q];
      x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
      m[4 * q] = w.x; m[4 * q + 1] = w.y; m[4 * q + 2] = w.z; m[4 * q + 3] = w.w;
    }
#pragma unroll
    for (int g4 = 0; g4 < 4; ++g4) {
      const unsigned e4 = (ends >> (16 * h + 4 * g4)) & 0xfu;
      if (e4 == 0u) {
#pragma unroll
        for (int r = 4 * g4; r < 4 * g4 + 4; ++r) acc = fmaf(x[r], m[r], acc);
      } else {
#pragma unroll
        for (int r = 4 * g4; r < 4 * g4 + 4; ++r) {
          acc = fmaf(x[r], m[r], acc);
          if ((e4 >> (r - 4 * g4)) & 1u) {
            const int tr = __shfl_sync(0xffffffffu, key, 16 * h + r);
            if (add_here && tr >= 0) tile_add<EXACT, 4 * T * T * T>(tile, qv * T * T * T + tr + off, acc, bad);
            acc = 0.0f;
          }
        }
      }
    }
  }
  const int tr = __shfl_sync(0xffffffffu, key, 31);  // the run that ends at the last particle
  if (add_here && tr >= 0) tile_add<EXACT, 4 * T * T * T>(tile, qv * T * T * T + tr + off, acc, bad);
  if (MOVERS) {
    unsigned mv = __ballot_sync(0xffffffffu, live && mover);
    if (mv) {
      __syncwarp();
      if (live && mover) {
#pragma unroll
        for (int q = 0; q < 4; ++q) red[8 + q][lane] = qdv[q];
      }
      __syncwarp();
      while (mv) {
        const int m = __ffs(mv) - 1;
        mv &= mv - 1;
        const int tm = __shfl_sync(0xffffffffu, t0, m);
        if (add_here)
          tile_add<EXACT, 4 * T * T * T>(tile, qv * T * T * T + tm + off, red[cv][m] * red[8 + qv][m], bad);
      }
    }
  }
  __syncwarp();
}

// One CTA per brick; its particles are the contiguous range of the brick's
// keys and lie in their key's cell (every move happens in pass 3, after
// which the sort restores that).
//   P1: deposit np and up at v_n = 1.5 v - 0.5 vp1 (maind.f:385-387, 399).
//   P2: gather, Ep, v-/v+, deposit up at 0.5 (v+ + v-) (maind.f:400-402).
//   P3: gather, Ep, v-/v+, vp1 = v, v = v+ + dt/2 Ep (maind.f:404-406), the
//       half move of maind.f:408 and the deposit of np and up at it
//       (:411-413), then the half move of maind.f:479 (v is unchanged by the
//       field subcycles in between), open-x outflow after each move and
//       res_chex after the second (maind.f:484).  It also prepares the sort:
//       the direction of every particle's new cell from its key's cell and
//       its rank among the particles of that key and direction, in order.
// PGRAD: the isothermal electron-pressure term in the gathered E (kitg:
// its face gradient centred per node, as get_Ep's gradient extension).
template <int PASS, bool CHEX = false, bool EXACT = true, bool PGRAD = false>
__global__ void __launch_bounds__(TPB_PASS, PASS == 3 ? 7 : 8) k_pass(G32 g, Part p, Species sp, StepParams sprm,
                                              const int64_t* __restrict__ start, const float4* __restrict__ kit,
                                              const float4* __restrict__ kitg, void* __restrict__ partial,
                                              uint32_t* __restrict__ dirrank, uint16_t* __restrict__ dep, int* err,
                                              FarList far) {
  // the chunk's particles, copied in by the bulk-copy engine (double-buffered):
  // offsets and v, plus vp1 in P1; cell words; species bytes
  constexpr int NF = PASS == 1 ? 9 : 6, NS = PASS_STAGES;
  __shared__ __align__(128) float s_f[NS][NF][TPB_PASS];
  __shared__ __align__(128) int32_t s_c[NS][TPB_PASS];
  __shared__ __align__(128) uint8_t s_s[NS][TPB_PASS];
  __shared__ uint64_t s_full[NS];
  // the field-gather tile: (aj-up, B_x) and (B_y, B_z) per node
  // deposit tile: T nodes per axis; a cell rx of the brick (rx in [-1,4] for
  // pass 3's movers, [0,3] otherwise) has its lower corner at offset rx + O.
  // The gather happens before any move: its tile is TN_IN wide, origin 0.
  constexpr int T = pass_tile(PASS), TNOD = T * T * T, O = PASS == 3 ? 1 : 0;
  __shared__ float4 s_kitA[PASS == 1 ? 1 : TNODES_IN];
  __shared__ float2 s_kitB[PASS == 1 ? 1 : TNODES_IN];
  __shared__ float4 s_kitG[PGRAD && PASS != 1 ? TNODES_IN : 1];
  // the deposit tile per node and moment: FP32, or (EXACT) fixed point as
  // low words [4 * TNOD] then high words [4 * TNOD]
  __shared__ __align__(8) unsigned s_dep[(EXACT ? 2 : 1) * 4 * TNOD];
  // per warp: [8 weights, 4 moments][particle]; rows padded to 36 floats so
  // that the 8 rows a reducing lane group reads start on different banks
  __shared__ __align__(16) float s_red[TPB_PASS / 32][12][36];
  __shared__ uint16_t s_rank[PASS == 3 ? BCELLS * NDIR : 2];   // running count per (local key, direction)
  const long long b = blockIdx.x;
  const int bi = (int)(b % g.nbx), bj = (int)((b / g.nbx) % g.nby), bk = (int)(b / ((long long)g.nbx * g.nby));
  const int c0x = 4 * bi, c0y = 4 * bj, c0z = 4 * bk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (PASS != 1) {
    for (int t = threadIdx.x; t < TNODES_IN; t += blockDim.x) {
      const int tx = t % TN_IN, ty = (t / TN_IN) % TN_IN, tz = t / (TN_IN * TN_IN);
      const int P = wrapi(c0x - 1 + tx, g.ncx), Q = wrapi(c0y - 1 + ty, g.ncy), R = wrapi(c0z - 1 + tz, g.ncz);
      const long long src = 2 * ((long long)P + (long long)g.ncx * (Q + (long long)g.ncy * R));
      s_kitA[t] = kit[src];
      const float4 hi = kit[src + 1];
      s_kitB[t] = make_float2(hi.x, hi.y);
      if (PGRAD) s_kitG[t] = kitg[src / 2];
    }
  }
  for (int t = threadIdx.x; t < (EXACT ? 2 : 1) * 4 * TNOD; t += blockDim.x) s_dep[t] = 0u;
  if (PASS == 3)
    for (int t = threadIdx.x; t < BCELLS * NDIR; t += blockDim.x) s_rank[t] = 0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < NS; ++q) tc05::mbar_init(&s_full[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const float hdt = 0.5f * sprm.dt;
  const long long first = start[b * BCELLS], last = start[b * BCELLS + BCELLS];
  // chunks of 128 particles from a 16-aligned start (every copy then starts
  // on a 16-byte boundary); lanes outside [first, last) are masked
  const long long a0 = first & ~15LL;
  const int nchunk = last > first ? (int)((last - a0 + TPB_PASS - 1) / TPB_PASS) : 0;
  // one thread copies chunk k's particle arrays into buffer k % NS
  int issued = 0;  // chunks whose copies thread 0 has started
  auto issue = [&](int k) {
    const int u = k % NS;
    issued = k + 1;
    const long long i0 = a0 + (long long)TPB_PASS * k;
    constexpr uint32_t FB = TPB_PASS * 4;
    tc05::mbar_expect_tx(&s_full[u], (NF + 1) * FB + (p.sp ? TPB_PASS : 0));
    tc05::bulk_g2s(s_c[u], p.cell + i0, FB, &s_full[u]);
    const float* src[9] = {p.ox, p.oy, p.oz, p.vx, p.vy, p.vz, p.wx, p.wy, p.wz};
#pragma unroll
    for (int f = 0; f < NF; ++f) tc05::bulk_g2s(s_f[u][f], src[f] + i0, FB, &s_full[u]);
    if (p.sp) tc05::bulk_g2s(s_s[u], p.sp + i0, TPB_PASS, &s_full[u]);
  };
  if (threadIdx.x == 0)
    for (int k = 0; k < NS - 1 && k < nchunk; ++k) issue(k);
  unsigned n_chex = 0;
  unsigned bad = 0;  // EXACT: a run sum beyond the fixed-point range
  // warp-uniform trip count: every lane takes part in the deposit reduction
  for (int kc = 0; kc < nchunk; ++kc) {
    const int u = kc % NS;
    bool got = true;
    if (threadIdx.x == 0) got = tc05::mbar_wait(&s_full[u], (kc / NS) & 1, sprm.wait_polls);
    // the barrier publishes the chunk to every thread and frees the buffer of
    // chunk kc-1, which every thread is done with: chunk kc+NS-1 goes there
    if (__syncthreads_or(!got)) {
      set_err(err, KERR_WAIT);
      // let the copies still in flight land before the CTA's shared memory
      // is released (each wait bounded)
      if (threadIdx.x == 0)
        for (int k = kc; k < issued; ++k) tc05::mbar_wait(&s_full[k % NS], (k / NS) & 1, STAGE_WAIT_POLLS);
      // pass 3: the brick's ions not reached are dropped by the next sort, so
      // that it sees a consistent set of ranks and counts
      if (PASS == 3 && dirrank)
        for (long long q = a0 + (long long)TPB_PASS * kc + threadIdx.x; q < last; q += TPB_PASS)
          if (q >= first) dirrank[q] = DR_DEAD;
      break;
    }
    if (threadIdx.x == 0 && kc + NS - 1 < nchunk) issue(kc + NS - 1);
    const long long l = a0 + (long long)TPB_PASS * kc + threadIdx.x;
    const bool mine = l >= first && l < last;
    const int32_t c = mine ? s_c[u][threadIdx.x] : CELL_DEAD;
    bool live = c >= 0;  // outside the range, or removed
    if (PASS == 3 && dirrank && !live && mine) dirrank[l] = DR_DEAD;
    int t0 = -1;
    int t0o = -1;       // P3: tile index of the cell before the move
    bool mover = false;  // P3: deposits in another cell than its own
    int grp = -1;  // P3: local key * NDIR + direction for the sort, -1 when not sorted
    bool far_ion = false;  // P3: moved more than one cell: placed through the far list
    float w8[8], qdv[4];
    if (live) {
      const bool fresh = (c & CELL_FRESH) != 0;
      int ci = pk_i(c), cj = pk_j(c), ck = pk_k(c);
      const int kl = (ci & 3) + 4 * (cj & 3) + 16 * (ck & 3);  // local key: the particle is in its key's cell
      float ox = s_f[u][0][threadIdx.x], oy = s_f[u][1][threadIdx.x], oz = s_f[u][2][threadIdx.x];
      float vx = s_f[u][3][threadIdx.x], vy = s_f[u][4][threadIdx.x], vz = s_f[u][5][threadIdx.x];
      int s = p.sp ? min((int)s_s[u][threadIdx.x], MAX_SPECIES - 1) : 0;
      float mr = sp.mrat[s], qw = sp.qw[s];
      float dvx = 0.f, dvy = 0.f, dvz = 0.f;  // velocity deposited
      int rx = ci - c0x, ry = cj - c0y, rz = ck - c0z;
      if (PASS == 3) t0o = (rx + 1) + TN * ((ry + 1) + TN * (rz + 1));
      if (PASS == 1) {
        if (fresh) p.cell[l] = c & ~CELL_FRESH;
        // extrapol_up (gutsp.f:144)
        dvx = 1.5f * vx - 0.5f * s_f[u][PASS == 1 ? 6 : 0][threadIdx.x];
        dvy = 1.5f * vy - 0.5f * s_f[u][PASS == 1 ? 7 : 0][threadIdx.x];
        dvz = 1.5f * vz - 0.5f * s_f[u][PASS == 1 ? 8 : 0][threadIdx.x];
      } else {
        // trilinear gather of (ajc-upc, btc) at the 8 corners (gutsp.f:217-251)
        const float wxl = 1.0f - ox, wxu = ox, wyl = 1.0f - oy, wyu = oy, wzl = 1.0f - oz, wzu = oz;
        // (the ion lies in its key's cell; clamped so that a broken sort
        // cannot index outside the tile: the checks below report it)
        const int gx = min(max(rx, 0), 3), gy = min(max(ry, 0), 3), gz = min(max(rz, 0), 3);
        const int tg = gx + TN_IN * (gy + TN_IN * gz);
        float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0, qx = 0, qy = 0, qz = 0;
#pragma unroll
        for (int cz = 0; cz < 2; ++cz)
#pragma unroll
          for (int cy = 0; cy < 2; ++cy)
#pragma unroll
            for (int cx = 0; cx < 2; ++cx) {
              const float w = (cx ? wxu : wxl) * (cy ? wyu : wyl) * (cz ? wzu : wzl);
              const int t = tg + cx + TN_IN * (cy + TN_IN * cz);
              const float4 f0 = s_kitA[t];
              const float2 f1 = s_kitB[t];
              ax = fmaf(w, f0.x, ax); ay = fmaf(w, f0.y, ay); az = fmaf(w, f0.z, az);
              bx = fmaf(w, f0.w, bx); by = fmaf(w, f1.x, by); bz = fmaf(w, f1.y, bz);
              if (PGRAD) {
                const float4 f2 = s_kitG[t];
                qx = fmaf(w, f2.x, qx); qy = fmaf(w, f2.y, qy); qz = fmaf(w, f2.z, qz);
              }
            }
        // Ep = ((aj-up) x B - gradP) * mrat (gutsp.f:260-270; q: gradP, zero without PGRAD)
        const float ex = ((ay * bz - az * by) - qx) * mr, ey = ((az * bx - ax * bz) - qy) * mr,
                    ez = ((ax * by - ay * bx) - qz) * mr;
        // v- and the rotation of get_vplus_vminus (gutsp.f:302-397)
        const float mx = vx + hdt * ex, my = vy + hdt * ey, mz = vz + hdt * ez;
        const float Bx = bx * mr, By = by * mr, Bz = bz * mr;
        const float B2 = Bx * Bx + By * By + Bz * Bz;
        const float dt2 = sprm.dt * sprm.dt;
        const float ad = 1.0f / (1.0f + 0.25f * B2 * dt2);
        const float a1 = (1.0f - 0.25f * B2 * dt2) * ad, a2 = sprm.dt * ad, a3 = 0.5f * dt2 * ad;
        const float mdb = mx * Bx + my * By + mz * Bz;
        const float px = a1 * mx + a2 * (my * Bz - mz * By) + a3 * mdb * Bx;
        const float py = a1 * my + a2 * (mz * Bx - mx * Bz) + a3 * mdb * By;
        const float pz = a1 * mz + a2 * (mx * By - my * Bx) + a3 * mdb * Bz;
        if (PASS == 2) {  // improve_up (gutsp.f:422)
          dvx = 0.5f * (px + mx);
          dvy = 0.5f * (py + my);
          dvz = 0.5f * (pz + mz);
        } else {
          // get_vp_final (gutsp.f:444-445).  vp1 = the old v stays where it
          // is: the new v goes into the vp1 arrays, and the host swaps the
          // two after the pass (12 bytes per ion not written)
          vx = px + hdt * ex;
          vy = py + hdt * ey;
          vz = pz + hdt * ez;
          dvx = vx; dvy = vy; dvz = vz;
          // move_ion_half of maind.f:408 (gutsp.f:473-510): the deposit position
          const float mvx = vx * hdt * g.inv_dx, mvy = vy * hdt * g.inv_dy, mvz = vz * hdt * g.inv_dz;
          bool ok = move_axis(ci, ox, mvx, g.ncx, true, !sprm.x_open);
          ok &= move_axis(cj, oy, mvy, g.ncy, false);
          ok &= move_axis(ck, oz, mvz, g.ncz, true);
          const bool out1 = ci < 0 || ci >= g.ncx;  // outflow through an open x face
          rx = rel_cell(ci, c0x, g.ncx); ry = rel_cell(cj, c0y, g.ncy); rz = rel_cell(ck, c0z, g.ncz);
          float dox = ox, doy = oy, doz = oz;
          // move_ion_half of maind.f:479: the stored position
          int ci2 = ci, cj2 = cj, ck2 = ck;
          bool out2 = out1;
          if (!out1) {
            ok &= move_axis(ci2, ox, mvx, g.ncx, true, !sprm.x_open);
            ok &= move_axis(cj2, oy, mvy, g.ncy, false);
            ok &= move_axis(ck2, oz, mvz, g.ncz, true);
            out2 = ci2 < 0 || ci2 >= g.ncx;
          }
          if (!ok) set_err(err, KERR_MOVE);
          if (CHEX && !out2 && sprm.heavy_of[s] != s) {
            // res_chex (chem_rates.f:823-840) at the end of the step, FP32
            const float x = (float)g.qx1 + ((float)ci2 + ox) * g.dx - sprm.cloud_x;
            const float y = (float)g.qy1 + ((float)cj2 + oy) * g.dy - sprm.cloud_y;
            const float z = (float)g.qz1 + ((float)ck2 + oz) * g.dz - sprm.cloud_z;
            const float vrel = sqrtf(vx * vx + vy * vy + vz * vz);
            const float sigma = vrel > 0.f ? sprm.cx_a - sprm.cx_b * logf(vrel) : 0.f;
            if (sigma > 0.f) {
              const float dens = sprm.cloud_N0 / (1.0f + (x * x + y * y + z * z) * sprm.inv_r0sq);
              const float prob = sprm.dt * dens * sigma * vrel;
              if (swapk::source_uniform_f32(sprm.seed, swapk::RNG_CHEX, sprm.chex_step, l) < prob) {
                vx = vy = vz = 0.f;
                p.vx[l] = 0.f;  // vp1 too
                p.vy[l] = 0.f;
                p.vz[l] = 0.f;
                p.sp[l] = (uint8_t)sprm.heavy_of[s];
                ++n_chex;
              }
            }
          }
          p.wx[l] = vx; p.wy[l] = vy; p.wz[l] = vz;
          if (out2) {
            p.cell[l] = CELL_DEAD;
            if (dirrank) dirrank[l] = DR_DEAD;
          } else {
            p.cell[l] = pk(ci2, cj2, ck2);
            p.ox[l] = ox; p.oy[l] = oy; p.oz[l] = oz;
            const int sx = step_cell(ci2, c0x + (kl & 3), g.ncx), sy = step_cell(cj2, c0y + ((kl >> 2) & 3), g.ncy),
                      sz = step_cell(ck2, c0z + (kl >> 4), g.ncz);
            if (sx < -1 || sx > 1 || sy < -1 || sy > 1 || sz < -1 || sz > 1)
              far_ion = true;
            else
              grp = kl * NDIR + dir_index(sx, sy, sz);
          }
          ox = dox; oy = doy; oz = doz;  // the deposit uses the maind.f:408 position
          if (out1) live = false;
          // a deposit position outside the tile's window also takes the far path
          if (live && (rx < -1 || rx > 4 || ry < -1 || ry > 4 || rz < -1 || rz > 4)) far_ion = true;
          if (far_ion) {
            const int slot = far.n ? atomicAdd(far.n, 1) : FAR_CAP;
            if (slot < FAR_CAP) {
              far.idx[slot] = l;
              far.key[slot] = out2 ? -1LL : key_of(g, ci2, cj2, ck2);
              far.dcell[slot] = live ? pk(ci, cj, ck) : -1;
              far.o[slot] = ox; far.o[FAR_CAP + slot] = oy; far.o[2 * FAR_CAP + slot] = oz;
              far.q[slot] = qw; far.q[FAR_CAP + slot] = qw * dvx;
              far.q[2 * FAR_CAP + slot] = qw * dvy; far.q[3 * FAR_CAP + slot] = qw * dvz;
              atomicAdd(far.total, 1ULL);
              if (!out2 && dirrank) dirrank[l] = DR_FAR;
            } else {
              set_err(err, KERR_MOVE);
              if (!out2 && dirrank) dirrank[l] = DR_BAD;
            }
            grp = -1;
            live = false;  // neither in the tile nor in the ranks
          }
        }
      }
      const bool inside = PASS == 3 ? !(rx < -1 || rx > 4 || ry < -1 || ry > 4 || rz < -1 || rz > 4)
                                    : !(rx < 0 || rx > 3 || ry < 0 || ry > 3 || rz < 0 || rz > 3);
      if (live && !inside) {
        set_err(err, KERR_MOVE);
        live = false;
      }
      if (live) {
        t0 = (rx + O) + T * ((ry + O) + T * (rz + O));
        mover = PASS == 3 && t0 != t0o;
        const float wxl = 1.0f - ox, wxu = ox, wyl = 1.0f - oy, wyu = oy, wzl = 1.0f - oz, wzu = oz;
#pragma unroll
        for (int cc = 0; cc < 8; ++cc)
          w8[cc] = ((cc & 1) ? wxu : wxl) * (((cc >> 1) & 1) ? wyu : wyl) * ((cc >> 2) ? wzu : wzl);
        qdv[0] = qw;
        qdv[1] = qw * dvx;
        qdv[2] = qw * dvy;
        qdv[3] = qw * dvz;
      }
    }
    warp_deposit<PASS != 2, T, PASS == 3, EXACT>(s_red[warp], live, t0, w8, qdv, s_dep, bad, lane, t0o, mover);
    if (PASS == 3 && dirrank) {
      // stable ranks per (key, direction): the warps of the CTA take their
      // turn in order, each adding its particles after the earlier ones
      const unsigned peers = __match_any_sync(0xffffffffu, grp >= 0 ? grp : -1 - lane);
      const unsigned lt = peers & ((1u << lane) - 1u);
      for (int w = 0; w < TPB_PASS / 32; ++w) {
        if (warp == w) {
          const unsigned before = grp >= 0 ? s_rank[grp] : 0u;
          __syncwarp();
          if (grp >= 0) {
            dirrank[l] = ((uint32_t)(grp % NDIR) << 26) | (before + __popc(lt));
            if (lt == 0) s_rank[grp] = (uint16_t)(before + __popc(peers));
          }
        }
        __syncthreads();
      }
    }
    if (EXACT && (kc + 1) % CARRY_CHUNKS == 0 && kc + 1 < nchunk) {
      // a crowded brick: carry the low words into the high words (exact:
      // 2^16 low units are one high unit), so that they never wrap
      __syncthreads();
      for (int t = threadIdx.x; t < 4 * TNOD; t += blockDim.x) {
        const unsigned lo = s_dep[t];
        s_dep[t] = lo & 0xFFFFu;
        s_dep[4 * TNOD + t] += lo >> 16;
      }
      __syncthreads();
    }
  }
  if (EXACT && bad) set_err(err, KERR_RANGE);
  if (CHEX) {
    for (int o = 16; o > 0; o >>= 1) n_chex += __shfl_down_sync(0xffffffffu, n_chex, o);
    if (lane == 0 && n_chex) atomicAdd(sprm.chex_count, (unsigned long long)n_chex);
  }
  __syncthreads();
  if (EXACT) {  // the node's fixed-point value: high words * 2^16 + low words
    long long* out = static_cast<long long*>(partial) + b * (4 * TNOD);
    for (int t = threadIdx.x; t < 4 * TNOD; t += blockDim.x)
      out[t] = (long long)(int)s_dep[4 * TNOD + t] * 65536LL + (long long)s_dep[t];
  } else {
    float* out = static_cast<float*>(partial) + b * (4 * TNOD);
    for (int t = threadIdx.x; t < 4 * TNOD; t += blockDim.x) out[t] = __uint_as_float(s_dep[t]);
  }

  if (PASS == 3 && dep)
    for (int t = threadIdx.x; t < BCELLS * NDIR; t += blockDim.x)  // direction-major: dep[dir][key]
      dep[(long long)(t / BCELLS) * g.nkeys + b * BCELLS + t % BCELLS] =
          (uint16_t)s_rank[(t % BCELLS) * NDIR + t / BCELLS];
}

// Sum, at every interior node, the brick tiles (T nodes per axis) that cover
// it: along each axis node p lies in the tile of brick floor((p+1+O)/4) at
// offset (p+1+O)%4 and in the one before at offset +4 when that is < T
// (O = 1 for the 7-node tiles, whose origin is one node lower).  The density
// is stored with its ghost images (boundary.f:167-206 fused in).
template <int T>
__global__ void k_node_sum(G32 g, const void* __restrict__ partial, int nq, int exact, float* __restrict__ np,
                           float* __restrict__ S) {
  constexpr int O = T == TN ? 1 : 0, TNOD = T * T * T;
  GSTRIDE(t, n_int(g)) {
    int P, Q, R;
    interior_of(g, t, P, Q, R);
    P -= 2;
    Q -= 2;
    R -= 2;
    int bx[2], ox[2], by[2], oy[2], bz[2], oz[2], nxc = 1, nyc = 1, nzc = 1;
    bx[0] = (P + 1 + O) >> 2; ox[0] = (P + 1 + O) & 3;
    if (bx[0] >= g.nbx) bx[0] -= g.nbx;
    if (ox[0] + 4 < T) { bx[1] = bx[0] == 0 ? g.nbx - 1 : bx[0] - 1; ox[1] = ox[0] + 4; nxc = 2; }
    by[0] = (Q + 1 + O) >> 2; oy[0] = (Q + 1 + O) & 3;
    if (by[0] >= g.nby) by[0] -= g.nby;
    if (oy[0] + 4 < T) { by[1] = by[0] == 0 ? g.nby - 1 : by[0] - 1; oy[1] = oy[0] + 4; nyc = 2; }
    bz[0] = (R + 1 + O) >> 2; oz[0] = (R + 1 + O) & 3;
    if (bz[0] >= g.nbz) bz[0] -= g.nbz;
    if (oz[0] + 4 < T) { bz[1] = bz[0] == 0 ? g.nbz - 1 : bz[0] - 1; oz[1] = oz[0] + 4; nzc = 2; }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    long long fix[4] = {0, 0, 0, 0};  // exact: the fixed-point sums (units of 2^-32)
    for (int a = 0; a < nxc; ++a)
      for (int bb = 0; bb < nyc; ++bb)
        for (int cc = 0; cc < nzc; ++cc) {
          const long long brick = bx[a] + (long long)g.nbx * (by[bb] + (long long)g.nby * bz[cc]);
          const long long at = brick * (4 * TNOD) + ox[a] + T * (oy[bb] + T * oz[cc]);
          if (exact) {
            const long long* src = static_cast<const long long*>(partial) + at;
            for (int q = 4 - nq; q < 4; ++q) fix[q] += src[q * TNOD];
          } else {
            const float* src = static_cast<const float*>(partial) + at;
            for (int q = 4 - nq; q < 4; ++q) acc[q] += src[q * TNOD];
          }
        }
    if (exact)  // the one rounding of the exact sum
      for (int q = 0; q < 4; ++q) acc[q] = (float)((double)fix[q] * FIX_INV);
    const long long o = pid(g, P, Q, R);
    if (nq == 4) store_img(g, np, P + 2, Q + 2, R + 2, acc[0]);  // np with its ghost images
    S[o] = acc[1];
    S[o + g.C] = acc[2];
    S[o + 2 * g.C] = acc[3];
  }
}

// ---------------------------------------------------------------------------
// fields (interior nodes, ghost images written by the producer)
// ---------------------------------------------------------------------------

// ct = S/np at the interior image; up_m = 0.5*(ct_m(node) + ct_m(node+e_m))
// (gutsp.f:1825-1836); np and up with ghost images.
// (The fast divide, two ulps: n is a density, far from where it loses accuracy.)
__device__ __forceinline__ float ct_o(const float* np, const float* S, long long o, long long cm) {
  const float n = np[o];
  return n == 0.0f ? 0.0f : __fdividef(S[o + cm], n);
}
__device__ __forceinline__ float ct_at(const G32& g, const float* np, const float* S, int i, int j, int k, int m) {
  return ct_o(np, S, nid(g, img(i, g.nx), img(j, g.ny), img(k, g.nz)), g.C * m);
}

__global__ void k_ct_up(G32 g, float* __restrict__ np, const float* __restrict__ S, float* __restrict__ up) {
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    if (i > 2 && j > 2 && k > 2 && i < g.nx - 1 && j < g.ny - 1 && k < g.nz - 1) {
      // the +1 neighbours interior and no ghost image to store: strides
      const long long C = g.C, o = nid(g, i, j, k), sy = g.nx, sz = (long long)g.nx * g.ny;
      up[o] = 0.5f * (ct_o(np, S, o, 0) + ct_o(np, S, o + 1, 0));
      up[o + C] = 0.5f * (ct_o(np, S, o, C) + ct_o(np, S, o + sy, C));
      up[o + 2 * C] = 0.5f * (ct_o(np, S, o, 2 * C) + ct_o(np, S, o + sz, 2 * C));
      continue;
    }
    const float ux = 0.5f * (ct_at(g, np, S, i, j, k, 0) + ct_at(g, np, S, i + 1, j, k, 0));
    const float uy = 0.5f * (ct_at(g, np, S, i, j, k, 1) + ct_at(g, np, S, i, j + 1, k, 1));
    const float uz = 0.5f * (ct_at(g, np, S, i, j, k, 2) + ct_at(g, np, S, i, j, k + 1, 2));
    store_img(g, up, i, j, k, ux);
    store_img(g, up + g.C, i, j, k, uy);
    store_img(g, up + 2 * g.C, i, j, k, uz);
  }
}

// Cell-centre B from the edge field (edge_to_center, grid_interp.f:35-51)
// with xrat = yrat = zrat = 1/2 (uniform grid), at an interior node.
// I: the offset type, 32-bit unsigned where every offset of the call fits
template <class I = long long>
__device__ __forceinline__ void e2c_o(const G32& g, const float* bt, I o, float& c1, float& c2, float& c3) {
  const I C = (I)g.C, sx = 1, sy = (I)g.nx, sz = (I)g.nx * (I)g.ny;
  float b1, b2;
  b2 = 0.5f * (bt[o] + bt[o - sy]);
  b1 = 0.5f * (bt[o - sz] + bt[o - sy - sz]);
  c1 = 0.5f * (b1 + b2);
  const float* B = bt + C;
  b2 = 0.5f * (B[o] + B[o - sx]);
  b1 = 0.5f * (B[o - sz] + B[o - sx - sz]);
  c2 = 0.5f * (b1 + b2);
  B = bt + 2 * C;
  b2 = 0.5f * (B[o] + B[o - sy]);
  b1 = 0.5f * (B[o - sx] + B[o - sx - sy]);
  c3 = 0.5f * (b1 + b2);
}
__device__ __forceinline__ void e2c(const G32& g, const float* bt, int i, int j, int k, float& c1, float& c2,
                                    float& c3) {
  e2c_o(g, bt, nid(g, i, j, k), c1, c2, c3);
}

// The isothermal electron-pressure gradient at the face of component m
// (node o to o + e_m): grad_pe * (np(o+e_m) - np(o)) / d_m / n_face, n_face
// the face average of np as in curlB.
template <int m, class I = long long>
__device__ __forceinline__ float gpe_face(const G32& g, const float* __restrict__ np, float gp, I o) {
  const I s = m == 0 ? (I)1 : (m == 1 ? (I)g.nx : (I)g.nx * (I)g.ny);
  const float inv = m == 0 ? g.inv_dx : (m == 1 ? g.inv_dy : g.inv_dz);
  return gp * ((np[o + s] - np[o]) * inv) / (0.5f * (np[o] + np[o + s]));
}

// Gather kit per physical node: (ajc - upc, btc) with ajc/upc =
// face_to_center (grid_interp.f:163-170) and btc = edge_to_center of
// dB plus the centred b0.
__global__ void k_kit(G32 g, const float* __restrict__ aj, const float* __restrict__ up,
                      const float* __restrict__ dbt, const float* __restrict__ b0c, const float* __restrict__ np,
                      float gp, float4* __restrict__ kit, float4* __restrict__ kitg) {
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    const long long C = g.C, o = nid(g, i, j, k), sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
    if (kitg)  // the pressure gradient centred like aj (face_to_center), for get_Ep
      kitg[t] = make_float4(0.5f * (gpe_face<0>(g, np, gp, o) + gpe_face<0>(g, np, gp, o - sx)),
                            0.5f * (gpe_face<1>(g, np, gp, o) + gpe_face<1>(g, np, gp, o - sy)),
                            0.5f * (gpe_face<2>(g, np, gp, o) + gpe_face<2>(g, np, gp, o - sz)), 0.0f);
    const float ax = 0.5f * ((aj[o] - up[o]) + (aj[o - sx] - up[o - sx]));
    const float ay = 0.5f * ((aj[o + C] - up[o + C]) + (aj[o - sy + C] - up[o - sy + C]));
    const float az = 0.5f * ((aj[o + 2 * C] - up[o + 2 * C]) + (aj[o - sz + 2 * C] - up[o - sz + 2 * C]));
    float c1, c2, c3;
    e2c(g, dbt, i, j, k, c1, c2, c3);
    kit[2 * t] = make_float4(ax, ay, az, c1 + b0c[0]);
    kit[2 * t + 1] = make_float4(c2 + b0c[1], c3 + b0c[2], 0.0f, 0.0f);
  }
}

// curlB (gutsf.f:202-239) on dB with uniform spacing; curl(b0) = 0.
__global__ void k_curlB(G32 g, const float* __restrict__ b, const float* __restrict__ np, float alpha,
                        float* __restrict__ aj) {
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    const long long C = g.C, o = nid(g, i, j, k), sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
    const float n0 = np[o];
    const float* B1 = b;
    const float* B2 = b + C;
    const float* B3 = b + 2 * C;
    const float c1 = (B3[o] - B3[o - sy]) * g.inv_dy + (B2[o - sz] - B2[o]) * g.inv_dz;
    const float c2 = (B1[o] - B1[o - sz]) * g.inv_dz + (B3[o - sx] - B3[o]) * g.inv_dx;
    const float c3 = (B2[o] - B2[o - sx]) * g.inv_dx + (B1[o - sy] - B1[o]) * g.inv_dy;
    store_img(g, aj, i, j, k, c1 / (0.5f * (n0 + np[o + sx]) * alpha));
    store_img(g, aj + C, i, j, k, c2 / (0.5f * (n0 + np[o + sy]) * alpha));
    store_img(g, aj + 2 * C, i, j, k, c3 / (0.5f * (n0 + np[o + sz]) * alpha));
  }
}

// ---- the field subcycle: two fused kernels per half step ----
//
// Launched over the interior nodes as a 3D grid (no index division).  Every
// field keeps its periodic ghost images (written by store_img), so a value at
// a ghost coordinate is computed at the interior image.

constexpr int FBX = 32, FBY = 4;

#define FIELD_NODE(i, j, k)                                   \
  const int i = blockIdx.x * FBX + threadIdx.x + 2;          \
  const int j = blockIdx.y * FBY + threadIdx.y + 2;          \
  const int k = blockIdx.z + 2;                              \
  if (i > g.ncx + 1 || j > g.ncy + 1) return

// Component m of aj = curl(dB)/(alpha * face-averaged np) at node (i,j,k)
// (curlB, gutsf.f:202-239; curl b0 = 0 for the uniform b0).
template <int m, class I = long long>
__device__ __forceinline__ float aj_o(const G32& g, const float* __restrict__ b, const float* __restrict__ np,
                                      float alpha, I o) {
  const I C = (I)g.C, sx = 1, sy = (I)g.nx, sz = (I)g.nx * (I)g.ny;
  const float* B1 = b;
  const float* B2 = b + C;
  const float* B3 = b + 2 * C;
  float c;
  I s;
  if (m == 0) {
    c = (B3[o] - B3[o - sy]) * g.inv_dy + (B2[o - sz] - B2[o]) * g.inv_dz;
    s = sx;
  } else if (m == 1) {
    c = (B1[o] - B1[o - sz]) * g.inv_dz + (B3[o - sx] - B3[o]) * g.inv_dx;
    s = sy;
  } else {
    c = (B2[o] - B2[o - sx]) * g.inv_dx + (B1[o - sy] - B1[o]) * g.inv_dy;
    s = sz;
  }
  // the fast divide (two ulps): the denominator, a density times alpha, is
  // far from the range where it loses accuracy
  return __fdividef(c, 0.5f * (np[o] + np[o + s]) * alpha);
}

// Linear index of node (i+di, j+dj, k+dk) for |d| <= 1: by strides for a node
// whose neighbours are all interior (INNER), else at the interior image.
template <bool INNER>
__device__ __forceinline__ long long nbr(const G32& g, long long o, int i, int j, int k, int di, int dj, int dk) {
  if (INNER) return o + di + (long long)g.nx * (dj + (long long)g.ny * dk);
  return nid(g, img(i + di, g.nx), img(j + dj, g.ny), img(k + dk, g.nz));
}
// a node at least one node away from every ghost plane
__device__ __forceinline__ bool inner_node(const G32& g, int i, int j, int k) {
  return i > 2 && i < g.nx - 1 && j > 2 && j < g.ny - 1 && k > 2 && k < g.nz - 1;
}
// store at an interior node, with its ghost images unless INNER
template <bool INNER, class T>
__device__ __forceinline__ void put(const G32& g, T* f, long long o, int i, int j, int k, T v) {
  if (INNER) f[o] = v;
  else store_img(g, f, i, j, k, v);
}

// curlB, face_to_center(aj - up) and the cross product of get_E (gutsf.f:
// 1059-1075, crossf2 gutsf.f:65-76): writes aj and ct.  Predictor: B at
// cell centres from edge_to_center of dB (grid_interp.f:35-51).  Corrector:
// B at m+1/2 through edge_to_face then face_to_center (gutsf.f:1268-1269),
// i.e. component m is the 1-2-1 average along axis m of edge_to_center.
template <int m>
__device__ __forceinline__ float aj_comp(const G32& g, const float* __restrict__ b, const float* __restrict__ np,
                                         float alpha, int i, int j, int k) {
  return aj_o<m>(g, b, np, alpha, nid(g, img(i, g.nx), img(j, g.ny), img(k, g.nz)));
}

template <bool CORR>
__global__ void __launch_bounds__(FBX * FBY) k_aj_ct(G32 g, const float* __restrict__ db,
                                                     const float* __restrict__ np, const float* __restrict__ up,
                                                     const float* __restrict__ b0c, float alpha,
                                                     float* __restrict__ aj, float* __restrict__ ct) {
  FIELD_NODE(i, j, k);
  if (inner_node(g, i, j, k)) {
    // every neighbour interior and no ghost image to store: strides, 32-bit
    // offsets (3 C < 2^32), the same arithmetic as below
    using U = unsigned;
    const U C = (U)g.C, o = (U)nid(g, i, j, k), sy = (U)g.nx, sz = (U)g.nx * (U)g.ny;
    const float a1 = aj_o<0, U>(g, db, np, alpha, o);
    const float a2 = aj_o<1, U>(g, db, np, alpha, o);
    const float a3 = aj_o<2, U>(g, db, np, alpha, o);
    const float a1m = aj_o<0, U>(g, db, np, alpha, o - 1);
    const float a2m = aj_o<1, U>(g, db, np, alpha, o - sy);
    const float a3m = aj_o<2, U>(g, db, np, alpha, o - sz);
    aj[o] = a1;
    aj[o + C] = a2;
    aj[o + 2 * C] = a3;
    const float ax = 0.5f * ((a1 - up[o]) + (a1m - up[o - 1]));
    const float ay = 0.5f * ((a2 - up[o + C]) + (a2m - up[o - sy + C]));
    const float az = 0.5f * ((a3 - up[o + 2 * C]) + (a3m - up[o - sz + 2 * C]));
    float bx, by, bz;
    if (!CORR) {
      e2c_o<U>(g, db, o, bx, by, bz);
    } else {
      float c1, c2, c3, m1, m2, m3, p1, p2, p3, d1, d2;
      e2c_o<U>(g, db, o, c1, c2, c3);
      e2c_o<U>(g, db, o - 1, m1, d1, d2);
      e2c_o<U>(g, db, o + 1, p1, d1, d2);
      e2c_o<U>(g, db, o - sy, d1, m2, d2);
      e2c_o<U>(g, db, o + sy, d1, p2, d2);
      e2c_o<U>(g, db, o - sz, d1, d2, m3);
      e2c_o<U>(g, db, o + sz, d1, d2, p3);
      bx = 0.25f * (m1 + 2.0f * c1 + p1);
      by = 0.25f * (m2 + 2.0f * c2 + p2);
      bz = 0.25f * (m3 + 2.0f * c3 + p3);
    }
    bx += b0c[0];
    by += b0c[1];
    bz += b0c[2];
    ct[o] = ay * bz - az * by;
    ct[o + C] = az * bx - ax * bz;
    ct[o + 2 * C] = ax * by - ay * bx;
    return;
  }
  const long long C = g.C, o = nid(g, i, j, k), sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  const float a1 = aj_comp<0>(g, db, np, alpha, i, j, k);
  const float a2 = aj_comp<1>(g, db, np, alpha, i, j, k);
  const float a3 = aj_comp<2>(g, db, np, alpha, i, j, k);
  const float a1m = aj_comp<0>(g, db, np, alpha, i - 1, j, k);
  const float a2m = aj_comp<1>(g, db, np, alpha, i, j - 1, k);
  const float a3m = aj_comp<2>(g, db, np, alpha, i, j, k - 1);
  store_img(g, aj, i, j, k, a1);
  store_img(g, aj + C, i, j, k, a2);
  store_img(g, aj + 2 * C, i, j, k, a3);
  const float ax = 0.5f * ((a1 - up[o]) + (a1m - up[o - sx]));
  const float ay = 0.5f * ((a2 - up[o + C]) + (a2m - up[o - sy + C]));
  const float az = 0.5f * ((a3 - up[o + 2 * C]) + (a3m - up[o - sz + 2 * C]));
  float bx, by, bz;
  if (!CORR) {
    e2c(g, db, i, j, k, bx, by, bz);
  } else {
    float c1, c2, c3, m1, m2, m3, p1, p2, p3, d1, d2;
    e2c(g, db, i, j, k, c1, c2, c3);
    e2c(g, db, img(i - 1, g.nx), j, k, m1, d1, d2);
    e2c(g, db, img(i + 1, g.nx), j, k, p1, d1, d2);
    e2c(g, db, i, img(j - 1, g.ny), k, d1, m2, d2);
    e2c(g, db, i, img(j + 1, g.ny), k, d1, p2, d2);
    e2c(g, db, i, j, img(k - 1, g.nz), d1, d2, m3);
    e2c(g, db, i, j, img(k + 1, g.nz), d1, d2, p3);
    bx = 0.25f * (m1 + 2.0f * c1 + p1);
    by = 0.25f * (m2 + 2.0f * c2 + p2);
    bz = 0.25f * (m3 + 2.0f * c3 + p3);
  }
  bx += b0c[0];
  by += b0c[1];
  bz += b0c[2];
  store_img(g, ct, i, j, k, ay * bz - az * by);
  store_img(g, ct + C, i, j, k, az * bx - ax * bz);
  store_img(g, ct + 2 * C, i, j, k, ax * by - ay * bx);
}

// Component m of E = face average of ct + nu*aj at node (i,j,k) (gutsf.f:
// 94-96, 1082), less the electron-pressure face gradient gpf when given
// (the isothermal extension of the commented "- gradP", gutsf.f:1083,1283).
template <int m>
__device__ __forceinline__ float e_o(const G32& g, const float* __restrict__ ct, const float* __restrict__ nu,
                                     const float* __restrict__ aj, const float* __restrict__ gpf, long long o) {
  const long long C = g.C;
  const long long s = m == 0 ? 1 : (m == 1 ? (long long)g.nx : (long long)g.nx * g.ny);
  const float e = 0.5f * (ct[o + C * m] + ct[o + s + C * m]) + nu[o] * aj[o + C * m];
  return gpf ? e - gpf[o + C * m] : e;
}


// Double-float arithmetic (a pair of floats carrying 48 significant bits):
// the FP32 form accumulates B across subcycles in it, because GB300's FP64
// pipe runs at a small fraction of its FP32 rate.  Dekker/Knuth error-free
// transformations with explicitly rounded operations (never contracted).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (bh + bl) - (ch + cl) * x
__device__ __forceinline__ void df_sub_mul(float bh, float bl, float ch, float cl, float x, float& rh, float& rl) {
  const float p = __fmul_rn(ch, x);
  const float q = __fmaf_rn(cl, x, __fmaf_rn(ch, x, -p));  // low part of the product
  float s, e;
  two_sum(bh, -p, s, e);
  e = __fadd_rn(e, __fsub_rn(bl, q));
  rh = __fadd_rn(s, e);
  rl = __fsub_rn(e, __fsub_rn(rh, s));
}

// E on the fly, curlE (gutsf.f:288-299) and B_new = base - coef*curlE
// (predict_B gutsf.f:1158-1159 with coef = 2 dtsub on b12; correct_B
// gutsf.f:1349-1350 with coef = dtsub on b1) in double-float; dB of the
// result in FP32.  Predictor: only dB at m+1/2 = (dB_new + dB1)/2
// (gutsf.f:1210-1219), the one use of the predicted B.  WRITE_E: store E
// (the step's last corrector).
template <bool PRED, bool WRITE_E, bool INNER>
__device__ __forceinline__ void bstep_node(const G32& g, const float* __restrict__ ct, const float* __restrict__ nu,
                                           const float* __restrict__ aj, const float* __restrict__ gpf,
                                           const float* __restrict__ bh,
                                           const float* __restrict__ bl, float ch, float cl,
                                           const float* __restrict__ b0c, float* __restrict__ oh,
                                           float* __restrict__ ol, float* __restrict__ dbo,
                                           const float* __restrict__ db1, float* __restrict__ dbtp1,
                                           float* __restrict__ E, float* __restrict__ e_acc, int i, int j, int k) {
  const long long C = g.C, o = nid(g, i, j, k);
  const long long ox = nbr<INNER>(g, o, i, j, k, 1, 0, 0), oy = nbr<INNER>(g, o, i, j, k, 0, 1, 0),
                  oz = nbr<INNER>(g, o, i, j, k, 0, 0, 1);
  const float e1 = e_o<0>(g, ct, nu, aj, gpf, o);
  const float e2 = e_o<1>(g, ct, nu, aj, gpf, o);
  const float e3 = e_o<2>(g, ct, nu, aj, gpf, o);
  const float e1y = e_o<0>(g, ct, nu, aj, gpf, oy), e1z = e_o<0>(g, ct, nu, aj, gpf, oz);
  const float e2x = e_o<1>(g, ct, nu, aj, gpf, ox), e2z = e_o<1>(g, ct, nu, aj, gpf, oz);
  const float e3x = e_o<2>(g, ct, nu, aj, gpf, ox), e3y = e_o<2>(g, ct, nu, aj, gpf, oy);
  const float ce[3] = {(e3y - e3) * g.inv_dy + (e2 - e2z) * g.inv_dz,
                       (e3 - e3x) * g.inv_dx + (e1z - e1) * g.inv_dz,
                       (e1 - e1y) * g.inv_dy + (e2x - e2) * g.inv_dx};
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    float rh, rl;
    df_sub_mul(bh[o + C * m], bl[o + C * m], ch, cl, ce[m], rh, rl);
    const float d = __fadd_rn(__fsub_rn(rh, b0c[m]), rl);
    if (PRED) {
      // the predicted B enters the corrector only through dB at m+1/2:
      // the corrector rewrites B and dB from b1
      put<INNER>(g, dbtp1 + C * m, o, i, j, k, 0.5f * (d + db1[o + C * m]));
    } else {
      put<INNER>(g, oh + C * m, o, i, j, k, rh);
      put<INNER>(g, ol + C * m, o, i, j, k, rl);
      put<INNER>(g, dbo + C * m, o, i, j, k, d);
    }
  }
  if (WRITE_E) {
    put<INNER>(g, E, o, i, j, k, e1);
    put<INNER>(g, E + C, o, i, j, k, e2);
    put<INNER>(g, E + 2 * C, o, i, j, k, e3);
  }
  if (e_acc) {  // the sum of the correctors' E over a step: the surrogate's target
    e_acc[o] += e1;
    e_acc[o + C] += e2;
    e_acc[o + 2 * C] += e3;
  }
}

template <bool PRED, bool WRITE_E>
__global__ void __launch_bounds__(FBX * FBY) k_bstep(G32 g, const float* __restrict__ ct,
                                                     const float* __restrict__ nu, const float* __restrict__ aj,
                                                     const float* __restrict__ gpf,
                                                     const float* __restrict__ bh, const float* __restrict__ bl,
                                                     float ch, float cl, const float* __restrict__ b0c,
                                                     float* __restrict__ oh, float* __restrict__ ol,
                                                     float* __restrict__ dbo, const float* __restrict__ db1,
                                                     float* __restrict__ dbtp1, float* __restrict__ E,
                                                     float* __restrict__ e_acc) {
  FIELD_NODE(i, j, k);
  if (inner_node(g, i, j, k))
    bstep_node<PRED, WRITE_E, true>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E, e_acc, i, j,
                                    k);
  else
    bstep_node<PRED, WRITE_E, false>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E, e_acc, i,
                                     j, k);
}

// B_new = base - coef * curl E for a given E (with ghost images), in
// double-float, with its FP32 dB: the field advance of the surrogate, whose
// discrete curl keeps div B where it was.
__global__ void __launch_bounds__(FBX * FBY) k_bstep_given_e(G32 g, const float* __restrict__ E,
                                                             const float* __restrict__ bh,
                                                             const float* __restrict__ bl, float ch, float cl,
                                                             const float* __restrict__ b0c, float* __restrict__ oh,
                                                             float* __restrict__ ol, float* __restrict__ dbo) {
  FIELD_NODE(i, j, k);
  const long long C = g.C, o = nid(g, i, j, k), sx = 1, sy = g.nx, sz = (long long)g.nx * g.ny;
  const float* E1 = E;
  const float* E2 = E + C;
  const float* E3 = E + 2 * C;
  const float ce[3] = {(E3[o + sy] - E3[o]) * g.inv_dy + (E2[o] - E2[o + sz]) * g.inv_dz,
                       (E3[o] - E3[o + sx]) * g.inv_dx + (E1[o + sz] - E1[o]) * g.inv_dz,
                       (E1[o] - E1[o + sy]) * g.inv_dy + (E2[o + sx] - E2[o]) * g.inv_dx};
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    float rh, rl;
    df_sub_mul(bh[o + C * m], bl[o + C * m], ch, cl, ce[m], rh, rl);
    store_img(g, oh + C * m, i, j, k, rh);
    store_img(g, ol + C * m, i, j, k, rl);
    store_img(g, dbo + C * m, i, j, k, __fadd_rn(__fsub_rn(rh, b0c[m]), rl));
  }
}

// b_out = b_new + f * (b_old - b_new) on hi parts, lo of b_new kept: the B
// one subcycle before the end of a surrogate step (the predictor's leapfrog
// base of the next plain subcycle).
__global__ void __launch_bounds__(FBX * FBY) k_df_lerp(G32 g, const float* __restrict__ nh,
                                                       const float* __restrict__ nl, const float* __restrict__ oh,
                                                       float f, float* __restrict__ rh, float* __restrict__ rl) {
  FIELD_NODE(i, j, k);
  const long long C = g.C, o = nid(g, i, j, k);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float d = f * (oh[o + C * m] - nh[o + C * m]);
    float s, e;
    two_sum(nh[o + C * m], d, s, e);
    e = __fadd_rn(e, nl[o + C * m]);
    const float h = __fadd_rn(s, e);
    store_img(g, rh + C * m, i, j, k, h);
    store_img(g, rl + C * m, i, j, k, __fsub_rn(e, __fsub_rn(h, s)));
  }
}

// Block sum (thread 0 holds the result; every thread of the block calls it).
__device__ __forceinline__ double bsum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;
}

// The judge's sums over the interior: |B_a - B_b|^2, |B_b|^2, |B_b - b0|^2
// (double-float levels a and b).
__global__ void k_judge(G32 g, const float* __restrict__ ah, const float* __restrict__ al,
                        const float* __restrict__ bh, const float* __restrict__ bl, const float* __restrict__ b0c,
                        double* acc) {
  double s0 = 0, s1 = 0, s2 = 0;
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    const long long o = nid(g, i, j, k);
    for (int m = 0; m < 3; ++m) {
      const double a = (double)ah[o + g.C * m] + (double)al[o + g.C * m];
      const double b = (double)bh[o + g.C * m] + (double)bl[o + g.C * m];
      s0 += (a - b) * (a - b);
      s1 += b * b;
      s2 += (b - (double)b0c[m]) * (b - (double)b0c[m]);
    }
  }
  // one atomic per block and sum (a grid of a few blocks per SM)
  s0 = bsum(s0);
  if (threadIdx.x == 0) atomicAdd(acc, s0);
  s1 = bsum(s1);
  if (threadIdx.x == 0) atomicAdd(acc + 1, s1);
  s2 = bsum(s2);
  if (threadIdx.x == 0) atomicAdd(acc + 2, s2);
}

// The surrogate's inputs at every interior node (voxel v = x + ncx*(y +
// Surrogate inputs per interior node (v = P + ncx*(Q + ncy*R)), FP32
// [V][SUR_NIN]: B = dB + b0, u_p, n_p, p_e = te * n_p, and E0 = ct + nu aj at
// the faces (the plain E of get_E from the predictor's aj and ct; zero when
// ct is null).
__global__ void k_grid_to_voxels(G32 g, const float* __restrict__ db, const float* __restrict__ b0c,
                                 const float* __restrict__ up, const float* __restrict__ np, float te,
                                 const float* __restrict__ ct, const float* __restrict__ aj,
                                 const float* __restrict__ nu, const float* __restrict__ gpf,
                                 const float* __restrict__ b1h, const float* __restrict__ b1l,
                                 const float* __restrict__ b12h, const float* __restrict__ b12l,
                                 float* __restrict__ out) {
  GSTRIDE(v, n_int(g)) {
    int i, j, k;
    interior_of(g, v, i, j, k);
    const long long C = g.C, o = nid(g, i, j, k);
    float* r = out + v * SUR_NIN;
    r[0] = db[o] + b0c[0];
    r[1] = db[o + C] + b0c[1];
    r[2] = db[o + 2 * C] + b0c[2];
    r[3] = up[o];
    r[4] = up[o + C];
    r[5] = up[o + 2 * C];
    r[6] = np[o];
    r[7] = te * np[o];
    r[8] = ct ? e_o<0>(g, ct, nu, aj, gpf, o) : 0.0f;
    r[9] = ct ? e_o<1>(g, ct, nu, aj, gpf, o) : 0.0f;
    r[10] = ct ? e_o<2>(g, ct, nu, aj, gpf, o) : 0.0f;
#pragma unroll
    for (int m = 0; m < 3; ++m)
      r[11 + m] = b12h ? (b1h[o + C * m] - b12h[o + C * m]) + (b1l[o + C * m] - b12l[o + C * m]) : 0.0f;
  }
}

// E = E0 + the predicted correction ([V][3]) into the field layout with ghost
// images (E0 from the inputs vin, none when vin is null).
__global__ void k_voxels_to_grid(G32 g, const float* __restrict__ ev, const float* __restrict__ vin,
                                 float* __restrict__ E) {
  GSTRIDE(v, n_int(g)) {
    int i, j, k;
    interior_of(g, v, i, j, k);
    for (int m = 0; m < 3; ++m)
      store_img(g, E + g.C * m, i, j, k, ev[v * 3 + m] + (vin ? vin[v * SUR_NIN + 8 + m] : 0.0f));
  }
}

// Grid E (interior) times f into [V][3] per voxel, less E0 from vin (when given).
__global__ void k_grid_e_to_voxels(G32 g, const float* __restrict__ E, float f, const float* __restrict__ vin,
                                   float* __restrict__ ev) {
  GSTRIDE(v, n_int(g)) {
    int i, j, k;
    interior_of(g, v, i, j, k);
    const long long o = nid(g, i, j, k);
    for (int m = 0; m < 3; ++m) ev[v * 3 + m] = f * E[o + g.C * m] - (vin ? vin[v * SUR_NIN + 8 + m] : 0.0f);
  }
}

// FP64 <-> double-float.
__global__ void k_split_df(long long n, const double* __restrict__ a, float* __restrict__ h, float* __restrict__ l) {
  GSTRIDE(t, n) {
    const double v = a[t];
    const float vh = (float)v;
    h[t] = vh;
    l[t] = (float)(v - (double)vh);
  }
}
__global__ void k_join_df(long long n, const float* __restrict__ h, const float* __restrict__ l,
                          double* __restrict__ a) {
  GSTRIDE(t, n) a[t] = (double)h[t] + (double)l[t];
}

// Whistler Courant time at every node, ghosts included, as check_time_step
// loops over them (gutsf.f:1782-1792), plus the smallest value.
__global__ void k_courant(G32 g, const float* __restrict__ dbt, const float* __restrict__ b0c,
                          const float* __restrict__ np, float alpha, float dx, float* __restrict__ dtn, unsigned* out) {
  float mn = 3.0e38f;
  GSTRIDE(o, g.C) {
    const float b1 = dbt[o] + b0c[0], b2 = dbt[o + g.C] + b0c[1], b3 = dbt[o + 2 * g.C] + b0c[2];
    const float btot = sqrtf(b1 * b1 + b2 * b2 + b3 * b3);
    const float ak = 2.0f / dx;
    const float a1 = ak * ak * btot / (alpha * np[o]);
    const float a2 = (ak * btot) * (ak * btot) / (alpha * np[o]);
    const float womega = 0.5f * (a1 + sqrtf(a1 * a1 + 4.0f * a2));
    const float d = dx / (womega / ak);
    dtn[o] = d;
    mn = fminf(mn, d > 0.0f ? d : 0.0f);
  }
  // one atomic per block (a grid of a few per SM): atomics from every warp to
  // the one address serialise in L2
  __shared__ float s_mn[TPB / 32];
  for (int off = 16; off > 0; off >>= 1) mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, off));
  if ((threadIdx.x & 31) == 0) s_mn[threadIdx.x >> 5] = mn;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mn = fminf(mn, s_mn[w]);
    atomicMin(out, __float_as_uint(mn));
  }
}

// ---------------------------------------------------------------------------
// stable counting sort by cell key for particles that moved at most one cell
// per axis since the last sort
// ---------------------------------------------------------------------------

// One warp per old key K: direction of every particle of K and its rank
// among the particles of K with the same direction, in array order.
__global__ void k_sort_prep(G32 g, const int64_t* __restrict__ start, const int32_t* __restrict__ cell,
                            uint32_t* __restrict__ dirrank, uint16_t* __restrict__ dep, int* err) {
  __shared__ unsigned s_cnt[TPB / 32][NDIR];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long K = blockIdx.x * (long long)(blockDim.x >> 5) + w; K < g.nkeys; K += nwarps) {
    if (lane < NDIR) s_cnt[w][lane] = 0;
    __syncwarp();
    int i0, j0, k0;
    cell_of_key(g, K, i0, j0, k0);
    const long long a = start[K], e = start[K + 1];
    for (long long base = a; base < e; base += 32) {
      const long long l = base + lane;
      const bool live = l < e;
      int d = NDIR;  // sentinel for idle lanes
      if (live && cell[l] < 0) {
        d = NDIR + 2;  // removed (outflow): not counted, skipped by the scatter
      } else if (live) {
        const int32_t c = cell[l];
        const int dx = step_cell(pk_i(c), i0, g.ncx), dy = step_cell(pk_j(c), j0, g.ncy),
                  dz = step_cell(pk_k(c), k0, g.ncz);
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) {
          set_err(err, KERR_MOVE);
          d = NDIR + 1;  // not counted; the scatter skips it
        } else {
          d = dir_index(dx, dy, dz);
        }
      }
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const unsigned lt = peers & ((1u << lane) - 1u);
      const int leader = __ffs(peers) - 1;
      const bool counted = live && d < NDIR;
      unsigned basecnt = 0;
      if (counted) basecnt = s_cnt[w][d];
      __syncwarp();
      if (live && !counted) dirrank[l] = d == NDIR + 2 ? DR_DEAD : DR_BAD;
      if (counted) {
        dirrank[l] = ((uint32_t)d << 26) | (basecnt + __popc(lt));
        if (lane == leader) s_cnt[w][d] = basecnt + __popc(peers);
      }
      __syncwarp();
    }
    if (lane < NDIR) dep[(long long)lane * g.nkeys + K] = (uint16_t)s_cnt[w][lane];
    __syncwarp();
  }
}

// The old key from which direction d arrives at the cell of key X.
__device__ __forceinline__ long long src_key(const G32& g, int i, int j, int k, int d) {
  const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
  return key_of(g, wrapi(i - dx, g.ncx), wrapi(j - dy, g.ncy), wrapi(k - dz, g.ncz));
}

// Per new key X: the count of arriving particles and, for every direction d,
// how many of them come from sources earlier in key order than the source of
// d (the stable order), so the scatter needs one lookup per particle.
// For a cell whose 27 source cells need no periodic wrap, the key order of
// the sources depends only on the cell's place in its brick (when there are
// at least 3 bricks along x and y): `order` lists, per place, the directions
// by increasing source key.  Other cells compare the 27 keys directly.
__global__ void __launch_bounds__(TPB) k_sort_count(G32 g, const uint16_t* __restrict__ dep,
                                                    const int32_t* __restrict__ ncount,
                                                    const uint8_t* __restrict__ order, int64_t* __restrict__ count,
                                                    uint16_t* __restrict__ pre, int* err) {
  __shared__ uint8_t s_ord[BCELLS * NDIR];
  __shared__ unsigned s_cnt[NDIR][TPB];  // per thread, indexed by direction
  for (int t = threadIdx.x; t < BCELLS * NDIR; t += blockDim.x) s_ord[t] = order[t];
  __syncthreads();
  const bool bricks_ok = g.nbx >= 3 && g.nby >= 3;
  GSTRIDE(X, g.nkeys) {
    int i, j, k;
    cell_of_key(g, X, i, j, k);
    int64_t n = 0;
#pragma unroll
    for (int d = 0; d < NDIR; ++d) {
      const unsigned c = dep[(long long)d * g.nkeys + src_key(g, i, j, k, d)];
      s_cnt[d][threadIdx.x] = c;
      n += c;
    }
    if (n > 65535) set_err(err, KERR_MOVE);
    if (ncount) n += ncount[X];
    const bool fast = bricks_ok && i > 0 && i < g.ncx - 1 && j > 0 && j < g.ncy - 1 && k > 0 && k < g.ncz - 1;
    if (fast) {
      const uint8_t* ord = s_ord + (X % BCELLS) * NDIR;
      unsigned run = 0;
      for (int r = 0; r < NDIR; ++r) {
        const int d = ord[r];
        pre[(long long)d * g.nkeys + X] = (uint16_t)run;  // direction-major: coalesced
        run += s_cnt[d][threadIdx.x];
      }
    } else {
      int sk[NDIR];  // keys fit in 31 bits (at most 1024^3 cells)
#pragma unroll
      for (int d = 0; d < NDIR; ++d) sk[d] = (int)src_key(g, i, j, k, d);
#pragma unroll
      for (int d = 0; d < NDIR; ++d) {
        unsigned p = 0;
#pragma unroll
        for (int q = 0; q < NDIR; ++q) p += sk[q] < sk[d] ? s_cnt[q][threadIdx.x] : 0u;
        pre[(long long)d * g.nkeys + X] = (uint16_t)p;
      }
    }
    count[X] = n;
  }
}

// dest = start_new[X] + (arrivals from sources earlier in key order) + rank.
__global__ void k_sort_scatter(G32 g, long long N, long long cap, const int32_t* __restrict__ cell,
                               const uint32_t* __restrict__ dirrank, const uint16_t* __restrict__ pre,
                               const int64_t* __restrict__ start_new, Part s, Part d, int* err) {
  GSTRIDE(l, N) {
    const int32_t c = cell[l];
    const uint32_t dr = dirrank[l];
    if (dr == DR_DEAD || dr == DR_FAR) continue;
    // every source field is read before the first store: the source and
    // destination buffers are distinct, and loading them together keeps the
    // ion's reads in flight at once instead of one per store
    const float ox = s.ox[l], oy = s.oy[l], oz = s.oz[l];
    const float vx = s.vx[l], vy = s.vy[l], vz = s.vz[l];
    const float wx = s.wx[l], wy = s.wy[l], wz = s.wz[l];
    const uint8_t spc = s.sp ? s.sp[l] : 0;
    const int dd = (int)(dr >> 26);
    if (dd >= NDIR) {
      set_err(err, KERR_MOVE);
      continue;
    }
    const long long X = key_of(g, pk_i(c), pk_j(c), pk_k(c));
    const long long dst = start_new[X] + pre[(long long)dd * g.nkeys + X] + (dr & ((1u << 26) - 1u));
    if (dst < 0 || dst >= cap) {
      set_err(err, KERR_CAPACITY);
      continue;
    }
    d.cell[dst] = c;
    d.ox[dst] = ox; d.oy[dst] = oy; d.oz[dst] = oz;
    d.vx[dst] = vx; d.vy[dst] = vy; d.vz[dst] = vz;
    d.wx[dst] = wx; d.wy[dst] = wy; d.wz[dst] = wz;
    if (s.sp) d.sp[dst] = spc;
  }
}

// Staged new ions: after the arrivals of their key, in staging order.
__global__ void k_new_scatter(G32 g, long long n_host, const int64_t* __restrict__ n_dev, long long n_max, Part s,
                              const int32_t* __restrict__ key, const int32_t* __restrict__ rank,
                              const int32_t* __restrict__ ncount, const int64_t* __restrict__ start_new, Part d,
                              long long cap, int* err) {
  const long long n = n_host + (n_dev ? *n_dev : 0);
  GSTRIDE(q, n < n_max ? n : n_max) {
    const long long X = key[q];
    const int32_t c = s.cell[q];  // all reads before the first store (see k_sort_scatter)
    const float ox = s.ox[q], oy = s.oy[q], oz = s.oz[q];
    const float vx = s.vx[q], vy = s.vy[q], vz = s.vz[q];
    const float wx = s.wx[q], wy = s.wy[q], wz = s.wz[q];
    const uint8_t spc = s.sp[q];
    const long long dst = start_new[X + 1] - ncount[X] + rank[q];
    if (dst < 0 || dst >= cap) {
      set_err(err, KERR_CAPACITY);
      continue;
    }
    d.cell[dst] = c | CELL_FRESH;
    d.ox[dst] = ox; d.oy[dst] = oy; d.oz[dst] = oz;
    d.vx[dst] = vx; d.vy[dst] = vy; d.vz[dst] = vz;
    d.wx[dst] = wx; d.wy[dst] = wy; d.wz[dst] = wz;
    d.sp[dst] = spc;
  }
}

// three-phase exclusive scan of int64 (block sums, scan of sums, add)
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = TPB * SCAN_ITEMS;

__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* sh, int64_t& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (int)(blockDim.x >> 5)) sh[lane] = s;
  }
  __syncthreads();
  total = sh[(blockDim.x >> 5) - 1];
  const int64_t before = w > 0 ? sh[w - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void k_scan_reduce(const int64_t* __restrict__ in, long long n, int64_t* __restrict__ sums) {
  __shared__ int64_t sh[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  int64_t v = 0;
  for (int q = 0; q < SCAN_ITEMS; ++q) {
    const long long idx = base + threadIdx.x * SCAN_ITEMS + q;
    if (idx < n) v += in[idx];
  }
  int64_t tot;
  block_excl_scan(v, sh, tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int64_t* sums, long long nb) {
  __shared__ int64_t sh[32];
  int64_t carry = 0;
  for (long long base = 0; base < nb; base += blockDim.x) {
    const long long idx = base + threadIdx.x;
    const int64_t v = idx < nb ? sums[idx] : 0;
    int64_t tot;
    const int64_t ex = block_excl_scan(v, sh, tot);
    if (idx < nb) sums[idx] = carry + ex;
    carry += tot;
  }
}

__global__ void k_scan_apply(const int64_t* __restrict__ in, long long n, const int64_t* __restrict__ sums,
                             int64_t* __restrict__ out) {
  __shared__ int64_t sh[32];
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  int64_t v[SCAN_ITEMS], s = 0;
  for (int q = 0; q < SCAN_ITEMS; ++q) {
    const long long idx = base + threadIdx.x * SCAN_ITEMS + q;
    v[q] = idx < n ? in[idx] : 0;
    s += v[q];
  }
  int64_t tot;
  int64_t run = block_excl_scan(s, sh, tot) + sums[blockIdx.x];
  for (int q = 0; q < SCAN_ITEMS; ++q) {
    const long long idx = base + threadIdx.x * SCAN_ITEMS + q;
    if (idx < n) out[idx] = run;
    run += v[q];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = run;
}

// ---------------------------------------------------------------------------
// conversions and diagnostics
// ---------------------------------------------------------------------------

__global__ void k_from_f64(G32 g, long long N, long long NM, const double* __restrict__ xp,
                           const double* __restrict__ vp, const double* __restrict__ vp1,
                           const double* __restrict__ mrat, const double* __restrict__ beta_p, Species sp, Part p,
                           int* err) {
  GSTRIDE(l, N) {
    int ci = 0, cj = 0, ck = 0;
    float ox = 0.5f, oy = 0.5f, oz = 0.5f;
    const bool ok = split_axis(xp[l], g.qx1, g.dx, g.ncx, true, ci, ox) &&
                    split_axis(xp[l + NM], g.qy1, g.dy, g.ncy, false, cj, oy) &&
                    split_axis(xp[l + 2 * NM], g.qz1, g.dz, g.ncz, true, ck, oz);
    if (!ok) set_err(err, KERR_DOMAIN);
    p.cell[l] = pk(ci, cj, ck);
    p.ox[l] = ox; p.oy[l] = oy; p.oz[l] = oz;
    p.vx[l] = (float)vp[l]; p.vy[l] = (float)vp[l + NM]; p.vz[l] = (float)vp[l + 2 * NM];
    p.wx[l] = (float)vp1[l]; p.wy[l] = (float)vp1[l + NM]; p.wz[l] = (float)vp1[l + 2 * NM];
  }
}

__global__ void k_assign_species(long long N, const double* __restrict__ mrat, const double* __restrict__ beta_p,
                                 const double* __restrict__ tab_mrat, const double* __restrict__ tab_bp, int n,
                                 uint8_t* __restrict__ spid, int* miss) {
  GSTRIDE(l, N) {
    int s = -1;
    for (int q = 0; q < n; ++q)
      if (tab_mrat[q] == mrat[l] && tab_bp[q] == beta_p[l]) { s = q; break; }
    if (s < 0) {
      atomicMin(miss, (int)(l & 0x7fffffff));  // the first particle of a pair not in the table
      s = 0;
    }
    spid[l] = (uint8_t)s;
  }
}

__global__ void k_to_f64(G32 g, long long N, long long NM, Part p, double* __restrict__ xp, double* __restrict__ vp,
                         double* __restrict__ vp1) {
  GSTRIDE(l, N) {
    const int32_t c = p.cell[l];
    xp[l] = g.qx1 + ((double)pk_i(c) + (double)p.ox[l]) * (double)g.dx;
    xp[l + NM] = g.qy1 + ((double)pk_j(c) + (double)p.oy[l]) * (double)g.dy;
    xp[l + 2 * NM] = g.qz1 + ((double)pk_k(c) + (double)p.oz[l]) * (double)g.dz;
    vp[l] = p.vx[l]; vp[l + NM] = p.vy[l]; vp[l + 2 * NM] = p.vz[l];
    vp1[l] = p.wx[l]; vp1[l + NM] = p.wy[l]; vp1[l + 2 * NM] = p.wz[l];
  }
}

__global__ void k_species_to_f64(long long N, const uint8_t* __restrict__ spid, const double* __restrict__ tm,
                                 const double* __restrict__ tb, double* __restrict__ mrat, double* __restrict__ beta_p) {
  GSTRIDE(l, N) {
    const int q = min((int)spid[l], MAX_SPECIES - 1);
    mrat[l] = tm[q];
    beta_p[l] = tb[q];
  }
}

// The write-back without the ions staged for a step not taken: tiles of
// KEEP_TILE ions, each block's count of kept ions, then (after a scan of the
// counts) the order-preserving conversion of the kept ones.
constexpr int KEEP_TILE = TPB * 8;
__device__ __forceinline__ bool kept(int32_t c) { return c >= 0 && !(c & CELL_FRESH); }

__global__ void k_keep_count(long long N, const int32_t* __restrict__ cell, int64_t* __restrict__ bcount) {
  __shared__ int64_t sh[32];
  const long long base = (long long)blockIdx.x * KEEP_TILE;
  int64_t n = 0;
  for (int q = 0; q < KEEP_TILE / TPB; ++q) {
    const long long l = base + q * TPB + threadIdx.x;
    n += (l < N && kept(cell[l])) ? 1 : 0;
  }
  int64_t tot;
  block_excl_scan(n, sh, tot);
  if (threadIdx.x == 0) bcount[blockIdx.x] = tot;
}

__global__ void k_to_f64_kept(G32 g, long long N, long long NM, Part p, const int64_t* __restrict__ bstart,
                              const double* __restrict__ tm, const double* __restrict__ tb, double* __restrict__ xp,
                              double* __restrict__ vp, double* __restrict__ vp1, double* __restrict__ mrat,
                              double* __restrict__ beta_p) {
  __shared__ int64_t sh[32];
  const long long base = (long long)blockIdx.x * KEEP_TILE;
  int64_t run = bstart[blockIdx.x];
  for (int q = 0; q < KEEP_TILE / TPB; ++q) {
    const long long l = base + q * TPB + threadIdx.x;
    const int32_t c = l < N ? p.cell[l] : CELL_DEAD;
    const bool k = kept(c);
    int64_t tot;
    const long long d = run + block_excl_scan(k ? 1 : 0, sh, tot);
    run += tot;
    if (!k) continue;
    xp[d] = g.qx1 + ((double)pk_i(c) + (double)p.ox[l]) * (double)g.dx;
    xp[d + NM] = g.qy1 + ((double)pk_j(c) + (double)p.oy[l]) * (double)g.dy;
    xp[d + 2 * NM] = g.qz1 + ((double)pk_k(c) + (double)p.oz[l]) * (double)g.dz;
    vp[d] = p.vx[l]; vp[d + NM] = p.vy[l]; vp[d + 2 * NM] = p.vz[l];
    vp1[d] = p.wx[l]; vp1[d + NM] = p.wy[l]; vp1[d + 2 * NM] = p.wz[l];
    const int s = p.sp ? min((int)p.sp[l], MAX_SPECIES - 1) : 0;
    mrat[d] = tm[s];
    beta_p[d] = tb[s];
  }
}

__global__ void k_keys(G32 g, long long N, const int32_t* __restrict__ cell, int32_t* __restrict__ key) {
  GSTRIDE(l, N) {
    const int32_t c = cell[l];
    key[l] = (int32_t)key_of(g, pk_i(c), pk_j(c), pk_k(c));
  }
}

// Keys non-decreasing?  Counts per key (for the cell starts).
__global__ void k_sorted_hist(long long N, const int32_t* __restrict__ key, long long nkeys, int* unsorted,
                              int64_t* __restrict__ count) {
  GSTRIDE(l, N) {
    const int32_t k = key[l];
    if (l + 1 < N && key[l + 1] < k) atomicExch(unsorted, 1);
    const bool ok = k >= 0 && k < nkeys;
    if (!ok) atomicExch(unsorted, 2);
    // one atomic per group of the warp's lanes with the same key (sorted
    // keys: one or two groups), not one per particle on the same address
    const unsigned peers = __match_any_sync(__activemask(), ok ? k : -1);
    if (ok && (int)(threadIdx.x & 31) == __ffs(peers) - 1)
      atomicAdd(reinterpret_cast<unsigned long long*>(count + k), (unsigned long long)__popc(peers));
  }
}

__global__ void k_gather_perm(long long N, const int64_t* __restrict__ perm, Part s, Part d) {
  GSTRIDE(l, N) {
    const long long q = perm[l];
    const int32_t c = s.cell[q];  // all reads before the first store (see k_sort_scatter)
    const float ox = s.ox[q], oy = s.oy[q], oz = s.oz[q];
    const float vx = s.vx[q], vy = s.vy[q], vz = s.vz[q];
    const float wx = s.wx[q], wy = s.wy[q], wz = s.wz[q];
    const uint8_t spc = s.sp ? s.sp[q] : 0;
    d.cell[l] = c;
    d.ox[l] = ox; d.oy[l] = oy; d.oz[l] = oz;
    d.vx[l] = vx; d.vy[l] = vy; d.vz[l] = vz;
    d.wx[l] = wx; d.wy[l] = wy; d.wz[l] = wz;
    if (s.sp) d.sp[l] = spc;
  }
}

__global__ void k_f64_to_f32(long long n, const double* __restrict__ a, const double* __restrict__ b,
                             float* __restrict__ out) {
  GSTRIDE(t, n) out[t] = (float)(b ? a[t] - b[t] : a[t]);
}

__global__ void k_f32_to_f64(long long n, const float* __restrict__ a, double* __restrict__ out) {
  GSTRIDE(t, n) out[t] = (double)a[t];
}

// kf[q] = 0.5 m_q w_q for species q (m = 1/mrat, w = qw*vol the particle's
// weight 1/(beta*beta_p)): kinetic energy kf * v^2, summed in FP32 per thread
// (a thread sees a few hundred particles) and in FP64 across threads.
struct KinFactor {
  float k[MAX_SPECIES];
};
__global__ void k_energy_p(long long N, Part p, KinFactor kf, double* acc) {
  float sf = 0.0f;
  GSTRIDE(l, N) {
    // every load issued before the test, so that an ion's loads are in
    // flight together (the kernel streams 17 B per ion)
    const int32_t c = p.cell[l];
    const int q = p.sp ? min((int)p.sp[l], MAX_SPECIES - 1) : 0;
    const float vx = p.vx[l], vy = p.vy[l], vz = p.vz[l];
    const float e = kf.k[q] * fmaf(vx, vx, fmaf(vy, vy, vz * vz));
    if (c >= 0 && !(c & CELL_FRESH)) sf += e;  // not removed, not created for the coming step
  }
  const double s = bsum((double)sf);
  if (threadIdx.x == 0) atomicAdd(acc, s);
}

__global__ void k_energy_f(G32 g, const double* __restrict__ b0, const float* __restrict__ b1h,
                           const float* __restrict__ b1l, const float* __restrict__ E, double alpha, double vol,
                           double* acc) {
  // sums of squares per thread, scaled once per block: the FP64 pipe of
  // this part is narrow, and a division per node would dominate the kernel
  double s1 = 0, s2 = 0, s3 = 0;
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    const long long o = nid(g, i, j, k);
    for (int m = 0; m < 3; ++m) {
      const double bb = (double)b1h[o + g.C * m] + (double)b1l[o + g.C * m];
      const double d = bb - b0[o + g.C * m];
      const float e = E[o + g.C * m];
      s1 = fma(d, d, s1);
      s2 = fma(bb, bb, s2);
      s3 += (double)(e * e);
    }
  }
  const double kb = 0.5 * vol / alpha;
  s1 = bsum(s1);
  if (threadIdx.x == 0) atomicAdd(acc + 1, s1 * kb);
  s2 = bsum(s2);
  if (threadIdx.x == 0) atomicAdd(acc + 2, s2 * kb);
  s3 = bsum(s3);
  if (threadIdx.x == 0) atomicAdd(acc + 3, s3 * (0.5 * vol));
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
#define RET(...)                 \
  do {                           \
    __VA_ARGS__;                 \
    return cudaGetLastError();   \
  } while (0)

// One pass launch; the first launch of each form asks for the largest
// shared-memory carve-out, so that the occupancy the launch bounds name (7 or
// 8 CTAs per SM) fits the CTAs' shared tiles.
template <int PASS, bool CHEX, bool EXACT, bool PGRAD = false>
cudaError_t launch_pass(unsigned grid, cudaStream_t st, const G32& g, const Part& p, const Species& sp,
                        const StepParams& s, const int64_t* start, const float4* kit, const float4* kitg,
                        void* partial, uint32_t* dirrank, uint16_t* dep, int* err, const FarList& far) {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_pass<PASS, CHEX, EXACT, PGRAD>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  k_pass<PASS, CHEX, EXACT, PGRAD><<<grid, TPB_PASS, 0, st>>>(g, p, sp, s, start, kit, kitg, partial, dirrank, dep,
                                                               err, far);
  return cudaGetLastError();
}

cudaError_t pass(int which, const G32& g, const Part& p, const Species& sp, const StepParams& s, const int64_t* start,
                 const float4* kit, void* partial, uint32_t* dirrank, uint16_t* dep, int* err, bool exact,
                 cudaStream_t st, const FarList* far, const float4* kitg) {
  const unsigned grid = (unsigned)g.nbricks;
  if (which == 3 && !far) return cudaErrorInvalidValue;
  const FarList none{};
  const FarList& fl = far ? *far : none;
#define PASS_ARGS grid, st, g, p, sp, s, start, kit, kitg, partial, dirrank, dep, err, fl
  if (kitg && which != 1) {  // the electron-pressure term: exact moment sums only
    if (!exact) return cudaErrorInvalidValue;
    if (which == 2) return launch_pass<2, false, true, true>(PASS_ARGS);
    if (s.chex) return launch_pass<3, true, true, true>(PASS_ARGS);
    return launch_pass<3, false, true, true>(PASS_ARGS);
  }
  if (exact) {
    if (which == 1) return launch_pass<1, false, true>(PASS_ARGS);
    if (which == 2) return launch_pass<2, false, true>(PASS_ARGS);
    if (s.chex) return launch_pass<3, true, true>(PASS_ARGS);
    return launch_pass<3, false, true>(PASS_ARGS);
  }
  if (which == 1) return launch_pass<1, false, false>(PASS_ARGS);
  if (which == 2) return launch_pass<2, false, false>(PASS_ARGS);
  if (s.chex) return launch_pass<3, true, false>(PASS_ARGS);
  return launch_pass<3, false, false>(PASS_ARGS);
#undef PASS_ARGS
}
cudaError_t node_sum(const G32& g, int pass, const void* partial, int nq, bool exact, float* np, float* S,
                     cudaStream_t st) {
  const unsigned nb = nblk((long long)g.ncx * g.ncy * g.ncz);
  if (pass_tile(pass) == TN) RET((k_node_sum<TN><<<nb, TPB, 0, st>>>(g, partial, nq, exact ? 1 : 0, np, S)));
  RET((k_node_sum<TN_IN><<<nb, TPB, 0, st>>>(g, partial, nq, exact ? 1 : 0, np, S)));
}
cudaError_t ct_and_up(const G32& g, const float* np, const float* S, float* up, cudaStream_t st) {
  RET((k_ct_up<<<nblk((long long)g.ncx * g.ncy * g.ncz), TPB, 0, st>>>(g, const_cast<float*>(np), S, up)));
}
cudaError_t build_kit(const G32& g, const float* aj, const float* up, const float* dbt, const float* b0c,
                      const float* np, float gp, float4* kit, float4* kitg, cudaStream_t st) {
  RET((k_kit<<<nblk((long long)g.ncx * g.ncy * g.ncz), TPB, 0, st>>>(g, aj, up, dbt, b0c, np, gp, kit, kitg)));
}
__global__ void k_gpe(G32 g, const float* __restrict__ np, float gp, float* __restrict__ gpf) {
  GSTRIDE(t, n_int(g)) {
    int i, j, k;
    interior_of(g, t, i, j, k);
    const long long C = g.C, o = nid(g, i, j, k);
    store_img(g, gpf, i, j, k, gpe_face<0>(g, np, gp, o));
    store_img(g, gpf + C, i, j, k, gpe_face<1>(g, np, gp, o));
    store_img(g, gpf + 2 * C, i, j, k, gpe_face<2>(g, np, gp, o));
  }
}
cudaError_t gpe_faces(const G32& g, const float* np, float gp, float* gpf, cudaStream_t st) {
  RET((k_gpe<<<nblk(n_int(g)), TPB, 0, st>>>(g, np, gp, gpf)));
}
cudaError_t curlB32(const G32& g, const float* dbt, const float* np, float alpha, float* aj, cudaStream_t st) {
  RET((k_curlB<<<nblk((long long)g.ncx * g.ncy * g.ncz), TPB, 0, st>>>(g, dbt, np, alpha, aj)));
}
cudaError_t aj_ct(const G32& g, bool corr, const float* db, const float* np, const float* up, const float* b0c,
                  float alpha, float* aj, float* ct, cudaStream_t st) {
  const dim3 grid((g.ncx + FBX - 1) / FBX, (g.ncy + FBY - 1) / FBY, g.ncz), blk(FBX, FBY);
  if (corr) RET((k_aj_ct<true><<<grid, blk, 0, st>>>(g, db, np, up, b0c, alpha, aj, ct)));
  RET((k_aj_ct<false><<<grid, blk, 0, st>>>(g, db, np, up, b0c, alpha, aj, ct)));
}
cudaError_t b_step(const G32& g, bool pred, bool write_e, const float* ct, const float* nu, const float* aj,
                   const float* gpf, const float* bh, const float* bl, double coef, const float* b0c, float* oh,
                   float* ol, float* dbo, const float* db1, float* dbtp1, float* E, float* e_acc, cudaStream_t st) {
  const dim3 grid((g.ncx + FBX - 1) / FBX, (g.ncy + FBY - 1) / FBY, g.ncz), blk(FBX, FBY);
  const float ch = (float)coef, cl = (float)(coef - (double)ch);
  if (pred && write_e)
    RET((k_bstep<true, true><<<grid, blk, 0, st>>>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E,
                                                   e_acc)));
  if (pred)
    RET((k_bstep<true, false><<<grid, blk, 0, st>>>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E,
                                                    e_acc)));
  if (write_e)
    RET((k_bstep<false, true><<<grid, blk, 0, st>>>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E,
                                                    e_acc)));
  RET((k_bstep<false, false><<<grid, blk, 0, st>>>(g, ct, nu, aj, gpf, bh, bl, ch, cl, b0c, oh, ol, dbo, db1, dbtp1, E,
                                                   e_acc)));
}
cudaError_t b_step_given_e(const G32& g, const float* E, const float* bh, const float* bl, double coef,
                           const float* b0c, float* oh, float* ol, float* dbo, cudaStream_t st) {
  const dim3 grid((g.ncx + FBX - 1) / FBX, (g.ncy + FBY - 1) / FBY, g.ncz), blk(FBX, FBY);
  const float ch = (float)coef, cl = (float)(coef - (double)ch);
  RET((k_bstep_given_e<<<grid, blk, 0, st>>>(g, E, bh, bl, ch, cl, b0c, oh, ol, dbo)));
}
cudaError_t df_lerp(const G32& g, const float* nh, const float* nl, const float* oh, float f, float* rh, float* rl,
                    cudaStream_t st) {
  const dim3 grid((g.ncx + FBX - 1) / FBX, (g.ncy + FBY - 1) / FBY, g.ncz), blk(FBX, FBY);
  RET((k_df_lerp<<<grid, blk, 0, st>>>(g, nh, nl, oh, f, rh, rl)));
}
cudaError_t grid_to_voxels(const G32& g, const float* db, const float* b0c, const float* up, const float* np,
                           float te, const float* ct, const float* aj, const float* nu, const float* gpf,
                           const float* b1h, const float* b1l, const float* b12h, const float* b12l, float* out,
                           cudaStream_t st) {
  RET((k_grid_to_voxels<<<nblk(n_int(g)), TPB, 0, st>>>(g, db, b0c, up, np, te, ct, aj, nu, gpf, b1h, b1l, b12h,
                                                         b12l, out)));
}
cudaError_t judge_sums(const G32& g, const float* ah, const float* al, const float* bh, const float* bl,
                       const float* b0c, double* acc3, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(acc3, 0, 3 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  const unsigned nb = nblk(n_int(g)) < 152u * 8u ? nblk(n_int(g)) : 152u * 8u;
  RET((k_judge<<<nb, TPB, 0, st>>>(g, ah, al, bh, bl, b0c, acc3)));
}
cudaError_t voxels_to_grid(const G32& g, const float* ev, const float* vin, float* E, cudaStream_t st) {
  RET((k_voxels_to_grid<<<nblk(n_int(g)), TPB, 0, st>>>(g, ev, vin, E)));
}
cudaError_t grid_e_to_voxels(const G32& g, const float* E, float f, const float* vin, float* ev, cudaStream_t st) {
  RET((k_grid_e_to_voxels<<<nblk(n_int(g)), TPB, 0, st>>>(g, E, f, vin, ev)));
}
cudaError_t split_df(long long n, const double* a, float* h, float* l, cudaStream_t st) {
  RET((k_split_df<<<nblk(n), TPB, 0, st>>>(n, a, h, l)));
}
cudaError_t join_df(long long n, const float* h, const float* l, double* a, cudaStream_t st) {
  RET((k_join_df<<<nblk(n), TPB, 0, st>>>(n, h, l, a)));
}
cudaError_t courant_min(const G32& g, const float* dbt, const float* b0c, const float* np, float alpha, float dx,
                        float* dtn, float* d_min, cudaStream_t st) {
  const unsigned init = 0x7f7fffffu;  // FLT_MAX
  cudaError_t e = cudaMemcpyAsync(d_min, &init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  const unsigned nb = nblk(g.C) < 152u * 8u ? nblk(g.C) : 152u * 8u;
  RET((k_courant<<<nb, TPB, 0, st>>>(g, dbt, b0c, np, alpha, dx, dtn, reinterpret_cast<unsigned*>(d_min))));
}
// ---------------------------------------------------------------------------
// ions that moved more than one cell in a step (pass 3's far list)
// ---------------------------------------------------------------------------

// Each listed ion's 8 corner weights times (qw, qw v) into the partial tile
// of its deposit cell's brick, as that tile would hold a run of one ion
// (fixed point: 64-bit integer adds, exact and order-independent).
template <bool EXACT>
__global__ void k_far_deposit(G32 g, FarList f, void* __restrict__ partial, int* err) {
  const int n = min(*f.n, FAR_CAP);
  unsigned bad = 0;
  GSTRIDE(i, n) {
    const int32_t c = f.dcell[i];
    if (c < 0) continue;
    const int ci = pk_i(c), cj = pk_j(c), ck = pk_k(c);
    const long long b = (long long)(ci >> 2) + (long long)g.nbx * ((cj >> 2) + (long long)g.nby * (ck >> 2));
    const int t0 = ((ci & 3) + 1) + TN * (((cj & 3) + 1) + TN * ((ck & 3) + 1));
    const float ox = f.o[i], oy = f.o[FAR_CAP + i], oz = f.o[2 * FAR_CAP + i];
    const float wxl = 1.0f - ox, wxu = ox, wyl = 1.0f - oy, wyu = oy, wzl = 1.0f - oz, wzu = oz;
    float q[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) q[m] = f.q[m * FAR_CAP + i];
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
      const float w = ((cc & 1) ? wxu : wxl) * (((cc >> 1) & 1) ? wyu : wyl) * ((cc >> 2) ? wzu : wzl);
      const int t = t0 + (cc & 1) + TN * (((cc >> 1) & 1) + TN * (cc >> 2));
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float x = w * q[m];
        const long long at = b * (4 * TNODES) + m * TNODES + t;
        if (EXACT) {
          bad |= fabsf(x) < FIX_MAX ? 0u : 1u;
          atomicAdd(static_cast<unsigned long long*>(partial) + at, (unsigned long long)to_fixed(x));
        } else {
          atomicAdd(static_cast<float*>(partial) + at, x);
        }
      }
    }
  }
  if (bad) set_err(err, KERR_RANGE);
}

__global__ void k_far_count(FarList f, int64_t* __restrict__ count) {
  const int n = min(*f.n, FAR_CAP);
  GSTRIDE(i, n) {
    const long long X = f.key[i];
    if (X >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(count + X), 1ULL);
  }
}

// Each survivor's rank among the listed arrivals of its key by array index
// (a scan of the whole list: the list is short, and this keeps the order
// deterministic), then a copy after the near arrivals.
__global__ void k_far_scatter(G32 g, FarList f, const int32_t* __restrict__ ncount,
                              const int64_t* __restrict__ start_new, Part s, Part d, long long cap, int* err) {
  const int n = min(*f.n, FAR_CAP);
  GSTRIDE(i, n) {
    const long long X = f.key[i];
    if (X < 0) continue;
    const long long li = f.idx[i];
    int cnt = 0, r = 0;
    for (int j = 0; j < n; ++j)
      if (f.key[j] == X) {
        ++cnt;
        r += f.idx[j] < li ? 1 : 0;
      }
    const long long dst = start_new[X + 1] - (ncount ? ncount[X] : 0) - cnt + r;
    if (dst < 0 || dst >= cap) {
      set_err(err, KERR_CAPACITY);
      continue;
    }
    d.cell[dst] = s.cell[li];
    d.ox[dst] = s.ox[li]; d.oy[dst] = s.oy[li]; d.oz[dst] = s.oz[li];
    d.vx[dst] = s.vx[li]; d.vy[dst] = s.vy[li]; d.vz[dst] = s.vz[li];
    d.wx[dst] = s.wx[li]; d.wy[dst] = s.wy[li]; d.wz[dst] = s.wz[li];
    if (s.sp) d.sp[dst] = s.sp[li];
  }
}

cudaError_t far_deposit(const G32& g, const FarList& far, void* partial, bool exact, int* err, cudaStream_t st) {
  if (exact) RET((k_far_deposit<true><<<64, TPB, 0, st>>>(g, far, partial, err)));
  RET((k_far_deposit<false><<<64, TPB, 0, st>>>(g, far, partial, err)));
}
cudaError_t far_count(const FarList& far, int64_t* count, cudaStream_t st) {
  RET((k_far_count<<<64, TPB, 0, st>>>(far, count)));
}
cudaError_t far_scatter(const G32& g, const FarList& far, const int32_t* ncount, const int64_t* start_new,
                        const Part& src, const Part& dst, long long cap, int* err, cudaStream_t st) {
  RET((k_far_scatter<<<FAR_CAP / TPB, TPB, 0, st>>>(g, far, ncount, start_new, src, dst, cap, err)));
}

cudaError_t sort_prep(const G32& g, const int64_t* start, const int32_t* cell, uint32_t* dirrank, uint16_t* dep,
                      int* err, cudaStream_t st) {
  const long long warps = g.nkeys;
  long long blocks = (warps + (TPB / 32) - 1) / (TPB / 32);
  if (blocks > 65535LL * 16) blocks = 65535LL * 16;
  RET((k_sort_prep<<<(unsigned)blocks, TPB, 0, st>>>(g, start, cell, dirrank, dep, err)));
}
cudaError_t sort_count(const G32& g, const uint16_t* dep, const int32_t* ncount, const uint8_t* order,
                       int64_t* count, uint16_t* pre, int* err, cudaStream_t st) {
  RET((k_sort_count<<<nblk(g.nkeys), TPB, 0, st>>>(g, dep, ncount, order, count, pre, err)));
}
void sort_order_table(uint8_t* out) {
  for (int l = 0; l < BCELLS; ++l) {
    const int li = l & 3, lj = (l >> 2) & 3, lk = l >> 4;
    int rank[NDIR], dirs[NDIR];
    for (int d = 0; d < NDIR; ++d) {
      const int dx = d % 3 - 1, dy = (d / 3) % 3 - 1, dz = d / 9 - 1;
      const int si = li - dx, sj = lj - dy, sk = lk - dz;  // the source cell, relative to this brick
      const int bx = si < 0 ? -1 : (si > 3 ? 1 : 0), by = sj < 0 ? -1 : (sj > 3 ? 1 : 0),
                bz = sk < 0 ? -1 : (sk > 3 ? 1 : 0);
      const int local = (si - 4 * bx) + 4 * (sj - 4 * by) + 16 * (sk - 4 * bz);
      rank[d] = ((bz + 1) * 9 + (by + 1) * 3 + (bx + 1)) * BCELLS + local;
      dirs[d] = d;
    }
    for (int a = 1; a < NDIR; ++a)  // insertion sort by source key
      for (int b = a; b > 0 && rank[dirs[b]] < rank[dirs[b - 1]]; --b) {
        const int t = dirs[b];
        dirs[b] = dirs[b - 1];
        dirs[b - 1] = t;
      }
    for (int r = 0; r < NDIR; ++r) out[l * NDIR + r] = (uint8_t)dirs[r];
  }
}
cudaError_t new_scatter(const G32& g, long long n_host, const int64_t* n_dev, long long n_max, const Part& stage,
                        const int32_t* key, const int32_t* rank, const int32_t* ncount, const int64_t* start_new,
                        const Part& dst, long long cap, int* err, cudaStream_t st) {
  if (n_max <= 0) return cudaSuccess;
  RET((k_new_scatter<<<nblk(n_max), TPB, 0, st>>>(g, n_host, n_dev, n_max, stage, key, rank, ncount, start_new, dst,
                                                  cap, err)));
}

cudaError_t scan_exclusive(const int64_t* in, int64_t* out, long long n, int64_t* sums, cudaStream_t st) {
  const long long nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_reduce<<<(unsigned)(nb < 1 ? 1 : nb), TPB, 0, st>>>(in, n, sums);
  k_scan_sums<<<1, 1024, 0, st>>>(sums, nb < 1 ? 1 : nb);
  RET((k_scan_apply<<<(unsigned)(nb < 1 ? 1 : nb), TPB, 0, st>>>(in, n, sums, out)));
}
cudaError_t sort_scatter(const G32& g, long long N, long long cap, const int32_t* cell, const uint32_t* dirrank,
                         const uint16_t* pre, const int64_t* start_new, const Part& src, const Part& dst, int* err,
                         cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_sort_scatter<<<nblk(N), TPB, 0, st>>>(g, N, cap, cell, dirrank, pre, start_new, src, dst, err)));
}
cudaError_t from_f64(const G32& g, long long N, long long NM, const double* xp, const double* vp, const double* vp1,
                     const double* mrat, const double* beta_p, const Species& sp, Part p, int* err, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_from_f64<<<nblk(N), TPB, 0, st>>>(g, N, NM, xp, vp, vp1, mrat, beta_p, sp, p, err)));
}
cudaError_t assign_species(long long N, const double* mrat, const double* beta_p, const double* tab_mrat,
                           const double* tab_bp, int n, uint8_t* spid, int* miss, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_assign_species<<<nblk(N), TPB, 0, st>>>(N, mrat, beta_p, tab_mrat, tab_bp, n, spid, miss)));
}
__global__ void k_not_uniform(long long C, const double* __restrict__ b, int* flag) {
  GSTRIDE(t, 3 * C) {
    if (b[t] != b[(t / C) * C]) atomicExch(flag, 1);
  }
}
cudaError_t not_uniform(long long C, const double* b, int* flag, cudaStream_t st) {
  RET((k_not_uniform<<<nblk(3 * C), TPB, 0, st>>>(C, b, flag)));
}
cudaError_t to_f64(const G32& g, long long N, long long NM, const Part& p, double* xp, double* vp, double* vp1,
                   cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_to_f64<<<nblk(N), TPB, 0, st>>>(g, N, NM, p, xp, vp, vp1)));
}
cudaError_t species_to_f64(long long N, const uint8_t* spid, const double* tab_mrat, const double* tab_bp,
                           double* mrat, double* beta_p, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_species_to_f64<<<nblk(N), TPB, 0, st>>>(N, spid, tab_mrat, tab_bp, mrat, beta_p)));
}
cudaError_t to_f64_kept(const G32& g, long long N, long long NM, const Part& p, const double* tab_mrat,
                        const double* tab_bp, double* xp, double* vp, double* vp1, double* mrat, double* beta_p,
                        int64_t* bcount, int64_t* bstart, int64_t* sums, long long* kept_out, cudaStream_t st) {
  *kept_out = 0;
  if (N <= 0) return cudaSuccess;
  const long long nb = (N + KEEP_TILE - 1) / KEEP_TILE;
  cudaError_t e;
  k_keep_count<<<(unsigned)nb, TPB, 0, st>>>(N, p.cell, bcount);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = scan_exclusive(bcount, bstart, nb, sums, st)) != cudaSuccess) return e;
  k_to_f64_kept<<<(unsigned)nb, TPB, 0, st>>>(g, N, NM, p, bstart, tab_mrat, tab_bp, xp, vp, vp1, mrat, beta_p);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  int64_t n = 0;
  if ((e = cudaMemcpyAsync(&n, bstart + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *kept_out = n;
  return cudaSuccess;
}
cudaError_t keys_of(const G32& g, long long N, const int32_t* cell, int32_t* key, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_keys<<<nblk(N), TPB, 0, st>>>(g, N, cell, key)));
}
cudaError_t sorted_hist(long long N, const int32_t* key, long long nkeys, int* unsorted, int64_t* count,
                        cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(count, 0, (nkeys + 1) * sizeof(int64_t), st);
  if (e != cudaSuccess) return e;
  if (N <= 0) return cudaSuccess;
  RET((k_sorted_hist<<<nblk(N), TPB, 0, st>>>(N, key, nkeys, unsorted, count)));
}
cudaError_t gather_perm(long long N, const int64_t* perm, const Part& src, Part dst, cudaStream_t st) {
  if (N <= 0) return cudaSuccess;
  RET((k_gather_perm<<<nblk(N), TPB, 0, st>>>(N, perm, src, dst)));
}
cudaError_t grid_f64_to_f32(long long n, const double* a, const double* b, float* out, cudaStream_t st) {
  RET((k_f64_to_f32<<<nblk(n), TPB, 0, st>>>(n, a, b, out)));
}
cudaError_t grid_f32_to_f64(long long n, const float* a, double* out, cudaStream_t st) {
  RET((k_f32_to_f64<<<nblk(n), TPB, 0, st>>>(n, a, out)));
}
cudaError_t energy32(const G32& g, long long N, const Part& p, const Species& sp, double vol, const double* b0,
                     const float* b1h, const float* b1l, const float* E, double alpha, double* acc4,
                     cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(acc4, 0, 4 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  const unsigned cap = 152 * 16;  // many particles per thread, few atomics, the SMs full
  if (N > 0) {
    KinFactor kf{};
    for (int q = 0; q < MAX_SPECIES && q < sp.n; ++q)
      kf.k[q] = (float)(0.5 * (1.0 / (double)sp.mrat[q]) * (double)sp.qw[q] * vol);
    const unsigned nb = nblk(N) < cap ? nblk(N) : cap;
    k_energy_p<<<nb, TPB, 0, st>>>(N, p, kf, acc4);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const long long nn = (long long)g.ncx * g.ncy * g.ncz;
  RET((k_energy_f<<<nblk(nn) < cap ? nblk(nn) : cap, TPB, 0, st>>>(g, b0, b1h, b1l, E, alpha, vol, acc4)));
}

}  // namespace swapk32
