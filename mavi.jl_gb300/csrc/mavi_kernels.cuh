// mavi_kernels.cuh — kernels of libmavi_cuda.so.
//
// Data layout in HBM (all replicas of a handle concatenated):
//  * particles live in chunk-sorted order ("slots" s = 0..M-1): replica-major,
//    then chunk (column-major, as Julia's chunk arrays), then ascending user
//    id inside a chunk — exactly the order of the reference's
//    chunk_particles[:, row, col] lists (src/chunks.jl:144-146);
//  * SoA arrays: FP64 positions/velocities (double2), the user id and the
//    replica (int32), and in the mixed form each particle's offset from its
//    chunk centre in int32 fixed point (int2, 2^-28 chunk units);
//  * chunks in CSR form: count[c], start[c] over all replicas' chunks.
// A step reads the state in "previous order" (*_out arrays, written by the
// last step together with each particle's new chunk and, in the mixed form,
// its new offset; the chunk counts were added up by the same pass), rebuilds
// the chunk lists (scan -> scatter claims places -> deterministic per-chunk
// order + permutation into *_cur) and runs the fused force/update passes.
//
// GB300 executes FP64 at ~1/70 of the FP32 rate, so the per-particle FP64
// work outside the pair loop is kept to a few tens of operations: the
// Julia-exact chunk index is found by verifying a guess with exactly-signed
// FMA residuals, wall tests only run for particles in edge chunks, and the
// mixed form's pair loop is integer + FP32 only.
#pragma once

#include <type_traits>

#include "mavi_device.cuh"

namespace mavi {

#ifndef MAVI_SCAN_ITEMS
#define MAVI_SCAN_ITEMS 4
#endif
constexpr int kFixBits = 28;                       // fixed-point offsets: chunk = 2^28 units
constexpr int kScanThreads = 256;
constexpr int kScanItems = MAVI_SCAN_ITEMS;            // consecutive chunks per thread (int4 loads)
constexpr int kScanTile = kScanThreads * kScanItems;   // chunks per scan tile
constexpr int64_t kScanDirectTiles = 512;  // above this, tile offsets come from k_tile_offsets
constexpr int kTileScanThreads = 1024;     // tiles per group of k_tile_offsets
constexpr int32_t kFixClamp = (1 << 30) - 1;       // |offset| clamp: 4 chunks
constexpr int kPassThreads = 128;                   // threads per block of the pair passes
constexpr int kPassWarps = kPassThreads / 32;
#ifndef MAVI_LJ_SPLIT_SIGMAS
#define MAVI_LJ_SPLIT_SIGMAS 2.0
#endif
constexpr double kLjSplitSigmas = MAVI_LJ_SPLIT_SIGMAS;   // split gather: double-float below this distance (sigmas)
// |offset| allowed in a pair term: two offsets of at most 1.5 chunks and the
// one-chunk stencil shift keep every difference within 4 chunks < 2^31 units
constexpr int32_t kFixRange = 3 << (kFixBits - 1);

// Fixed-point parameters of the pair laws of one (type, type) pair, in units
// u = max(chunk_l, chunk_h) / 2^28 of the replica.
struct FixPair {
    unsigned long long cut2;   // squared cutoff (dist_max / r_max / WCA cutoff), units^2
    long long eq2;             // squared equilibrium distance (dist_eq / r_eq), units^2
    float eq;                  // equilibrium distance, units
    float k_rep, k_atr;        // HarmTrunc constants; Szabo: f_mod below / above r_eq
    float cut2_hi, cut2_lo;    // cut2 * (1 +- 1e-6): FP32 squared distances beyond / below
                               // these are certainly outside / inside the cutoff
    float pad;
    float nb2_hi, nb2_lo;      // rings neighbour threshold (dist_eq * tol)^2 in units^2 * (1 +- 1e-6)
};

struct Ctx {
    // particle arrays in sorted order
    double2 *pos_cur, *pos_mid, *pos_out;
    double2 *vel_cur, *vel_out;
    double *pol_cur, *pol_out;
    int2 *off_cur, *off_mid, *off_out;   // mixed form: fixed-point chunk offsets
    double2 *fd;     // pair-pass force (FP64 form)
    float2 *ff;      // pair-pass force (mixed form)
    double2 *fold_d; // Verlet F(t), FP64 form
    float2 *fold_f;  // Verlet F(t), mixed form
    int32_t *uid_cur, *uid_out, *rep_cur, *rep_out;
    int32_t *cell_cur, *cell_out;
    int32_t *count, *start, *src_of, *slot_of;
    int32_t *key_of, *cell_at;   // per claimed slot: user id and chunk of its particle
    int32_t *rinfo_cur;          // rings: packed ring identity per sorted slot (ring_key), or null
    // rings: the current state and the pair force in user-slot order, where a
    // ring's particles are contiguous, so that k_rings reads them coalesced
    // and without the slot map (null for other models)
    double2 *pos_u;
    int2 *off_u;
    int32_t *cell_u;
    float2 *ff_u;
    double2 *fd_u;
    const int32_t *rkey_user;    // the same per user slot (fixed at creation)
    int32_t *tile_sum;   // chunk counts per scan tile, accumulated with the histogram
    int64_t ntiles;
    // per ring (global ring index)
    double *ring_pol;
    double *ring_area;
    const int32_t *ring_types;
    const int32_t *ring_rep;   // replica of each ring
    const double *cxu, *cyu;   // chunk-centre x per column, y per row, in units of u
    // rings particle neighbour lists (0: off, 1: counts, 2: counts and lists),
    // indexed by user slot; neighbours stored as user slots
    int32_t nb_mode, nb_type_all;
    double nb_tol;
    int32_t *nb_count, *nb_list;
    double2 *ring_cs;          // (cos, sin) of the ring's polarisation angle
    double2 *ring_vc;          // summed particle velocity of the ring in the last update
    // the mixed form keeps both in FP32 (aliases of the same buffers)
    float2 *ring_csf, *ring_vcf;
    // variable number of rings (sources and sinks). var_rings: inactive rings'
    // particles are parked in chunk `park` (after every real chunk), out of
    // every stencil; the step's histogram is then taken by k_count after
    // k_sources instead of inside k_rings.
    int32_t var_rings;
    int64_t park;
    int32_t *ring_active, *ring_uid;   // per ring: VarRingsIds.mask, .uids
    double2 *ring_cms;                 // per ring: RingsInfo.cms
    int32_t *src_ids;                  // per ring slot: VarRingsIds.ids (replica-local, 0-based)
    int32_t *src_state;                // per replica: num_active, max uid
    const SrcEntryD *src_entries;
    const SrcBoxD *src_boxes;
    const double2 *src_spawn;
    const int32_t *src_chunks;
    // descriptors
    const DevRep *reps;
    const MaviSpace *spaces;     // [replica][MAVI_MAX_SPACES]
    const MaviRingsCfg *rcfg;    // [replica]
    const FixPair *fix;          // [replica][MAVI_MAX_TYPES][MAVI_MAX_TYPES]
    DevError *err;
    int64_t M;        // active particles
    int64_t Ctot;     // chunks over all replicas
    int64_t *d_step;  // steps completed (device copy, for the RNG counter)
    const double *noise;
    int32_t noise_mode;
    int32_t num_reps;
    int32_t gather_mode;   // 0: warp-staged window in shared memory, 1: per-chunk global loads,
                           // 2: per-column contiguous global ranges
    uint64_t seed;
};

// ===========================================================================
// Julia-exact chunk index (src/chunks.jl:120-147)
// ===========================================================================
// trunc(Int, div(t, l)) for the numerator t of update_particle_chunk!. For
// t >= 0 Julia's float div is floor(t / l) exactly; it is found by checking
// a guess g: sign(fma(-q, l, t)) is the exact sign of t - q*l (one rounding of
// a nonzero value cannot reach zero at these magnitudes). Particles move far
// less than a chunk per step, so the guess (the current chunk) or a
// neighbour resolves it; otherwise the literal formula runs.
static __device__ __forceinline__ int64_t julia_trunc_div_slow(double t, double l) {
    double q = julia_div(t, l);
    return q < 4e18 ? (int64_t)q : (int64_t)4e18;
}

__device__ __forceinline__ int64_t julia_trunc_div(double t, double l, int64_t g, bool has_guess) {
    if (t < 0) return (t + l > 0) ? 0 : -1;     // div = -0.0 above -l; below it the grid is left
    if (has_guess && g >= 0) {
        double gd = (double)g;
        if (fma(-gd, l, t) >= 0) {
            if (fma(-(gd + 1.0), l, t) < 0) return g;
            if (fma(-(gd + 2.0), l, t) < 0) return g + 1;
        } else if (g >= 1 && fma(-(gd - 1.0), l, t) >= 0) {
            return g - 1;
        }
    }
    return julia_trunc_div_slow(t, l);
}

// Row/col (0-based, with the clamp of index n+1) of a position; the FP64
// numerators tx = x - bl_x and ty = -y + bl_y + H are returned for the
// offset computation.
__device__ __forceinline__ void bin_position(const DevRep& R, double x, double y, int64_t grow, int64_t gcol,
                                             bool has_guess, int64_t& row, int64_t& col, double& tx, double& ty,
                                             bool& finite) {
    tx = __dsub_rn(x, R.bb_blx);
    ty = __dadd_rn(__dadd_rn(-y, R.bb_bly), R.bb_h);
    finite = isfinite(tx) && isfinite(ty);
    if (!finite) { row = 0; col = 0; return; }
    int64_t qr = julia_trunc_div(ty, R.chunk_h, grow, has_guess);
    int64_t qc = julia_trunc_div(tx, R.chunk_l, gcol, has_guess);
    int64_t r = qr + 1, c = qc + 1;
    r -= (r == (int64_t)R.rows + 1) ? 1 : 0;
    c -= (c == (int64_t)R.cols + 1) ? 1 : 0;
    row = r - 1;
    col = c - 1;
}

// Fixed-point offset of a position from the centre of chunk (row, col),
// computed from the binning numerators (x - cx = tx - (col + 1/2) l,
// y - cy = (row + 1/2) h - ty).
// An offset beyond 1.5 chunks (a particle that moved more than a chunk in
// one step) is reported (MAVI_ERR_OFFSET_RANGE) instead of giving wrong pair
// terms; the conversion saturates and the clamp keeps the value finite.
__device__ __forceinline__ int2 fixed_offset(const DevRep& R, int64_t row, int64_t col, double tx, double ty,
                                             DevError* err, int64_t s) {
    double ox = fma(-((double)col + 0.5), R.chunk_l, tx) * R.inv_u;
    double oy = fma((double)row + 0.5, R.chunk_h, -ty) * R.inv_u;
    int32_t ix = min(max(__double2int_rn(ox), -kFixClamp), kFixClamp);
    int32_t iy = min(max(__double2int_rn(oy), -kFixClamp), kFixClamp);
    if (R.has_chunks && (abs(ix) > kFixRange || abs(iy) > kFixRange)) raise_error(err, MAVI_ERR_OFFSET_RANGE, s, 0);
    return make_int2(ix, iy);
}

// Bounds/finite checks; returns the clamped global chunk.
__device__ __forceinline__ int64_t checked_cell(const DevRep& R, int64_t& row, int64_t& col, bool finite,
                                                DevError* err, int64_t s) {
    if (!finite) raise_error(err, MAVI_ERR_NONFINITE, s, 0);
    else if (row < 0 || row >= R.rows || col < 0 || col >= R.cols)
        raise_error(err, MAVI_ERR_OUT_OF_GRID, s, row * 1000003 + col);
    row = row < 0 ? 0 : (row >= R.rows ? R.rows - 1 : row);
    col = col < 0 ? 0 : (col >= R.cols ? R.cols - 1 : col);
    return R.c0 + col * (int64_t)R.rows + row;
}

// Whether the chunk touches the bounding box (walls of the bounding
// rectangle can only act on particles there).
__device__ __forceinline__ bool edge_chunk(const DevRep& R, int64_t row, int64_t col) {
    return row <= 0 || col <= 0 || row >= R.rows - 1 || col >= R.cols - 1;
}

// Warp-aggregated histogram update: lanes with the same chunk share one
// atomic. Must be called by all 32 lanes of the warp.
__device__ __forceinline__ void count_into_chunk(const Ctx& C, bool valid, int64_t s, int64_t cell,
                                                 int32_t cap) {
    // a fire-and-forget add (no rank returned: nothing waits on the atomic);
    // each particle takes its place in the chunk later, in k_scatter
    (void)cap;
    const unsigned full = 0xffffffffu;
    int key = valid ? (int)cell : -1;
    unsigned peers = __match_any_sync(full, key);
    int lane = threadIdx.x & 31;
    if (valid && lane == __ffs(peers) - 1) atomicAdd(&C.count[cell], __popc(peers));
    // scan-tile totals: one atomic per warp and tile (consecutive particles
    // share a tile; per-particle atomics on one address would serialise)
    int tkey = valid ? (int)(cell / kScanTile) : -1;
    unsigned tpeers = __match_any_sync(full, tkey);
    if (valid && lane == __ffs(tpeers) - 1) atomicAdd(&C.tile_sum[tkey], __popc(tpeers));
    if (valid) C.cell_out[s] = (int32_t)cell;
}

// Chunk (and mixed-form offset) of a final position; `guess_cell` is the
// particle's current chunk or -1.
template <int PREC>
__device__ __forceinline__ int64_t bin_final(const Ctx& C, const DevRep& R, int64_t s, double x, double y,
                                            int64_t guess_cell, int32_t uw = -1) {
    // uw >= 0: the offset also goes to the user-order copy (rings)
    if (!R.has_chunks) {
        if constexpr (PREC == kPrecMixed) {
            double tx = __dsub_rn(x, R.bb_blx), ty = __dadd_rn(__dadd_rn(-y, R.bb_bly), R.bb_h);
            const int2 o = fixed_offset(R, 0, 0, tx, ty, C.err, s);
            C.off_out[s] = o;
            if (uw >= 0) C.off_u[uw] = o;
        }
        return R.c0;
    }
    int64_t grow = 0, gcol = 0;
    bool has_guess = guess_cell >= 0;
    if (has_guess) {
        int32_t lc = (int32_t)(guess_cell - R.c0);
        gcol = lc / R.rows;
        grow = lc - gcol * R.rows;
    }
    int64_t row, col;
    double tx, ty;
    bool finite;
    bin_position(R, x, y, grow, gcol, has_guess, row, col, tx, ty, finite);
    int64_t cell = checked_cell(R, row, col, finite, C.err, s);
    if constexpr (PREC == kPrecMixed) {
        const int2 o = fixed_offset(R, row, col, tx, ty, C.err, s);
        C.off_out[s] = o;
        if (uw >= 0) C.off_u[uw] = o;
    }
    return cell;
}

// Chunk of a final position, fast path first: the offset from the centre of
// the current chunk is computed in fixed-point units; when it lies more than
// one unit inside the chunk, the particle is > u/2 (~1e-9 of a chunk) inside,
// far beyond the rounding of the FP64 numerator of the Julia formula (an ulp
// of the position), so the Julia quotient is the current chunk and the exact
// checks are skipped. Returns -1 when the exact path is needed.
template <int PREC>
__device__ __forceinline__ int64_t bin_fast(const Ctx& C, const DevRep& R, int64_t s, double x, double y,
                                           int32_t cell, int32_t uw = -1) {
    if (!R.has_chunks) return -1;
    int32_t lc = (int32_t)(cell - R.c0);
    int32_t col = lc / R.rows, row = lc - col * R.rows;
    // chunk centres in units come from per-column / per-row tables: one FP64
    // FMA and one conversion per coordinate (the FP64 pipe is the scarce one)
    int32_t ix = __double2int_rn(fma(x, R.inv_u, -C.cxu[R.ccol0 + col]));
    int32_t iy = __double2int_rn(fma(y, R.inv_u, -C.cyu[R.crow0 + row]));
    // two-sided tests: a position many chunks away (a periodic wrap) saturates
    // the conversion, and abs(INT_MIN) would pass a one-sided test
    if (ix > 1 - R.half_sx_i && ix < R.half_sx_i - 1 && iy > 1 - R.half_sy_i && iy < R.half_sy_i - 1) {
        if constexpr (PREC == kPrecMixed) {
            C.off_out[s] = make_int2(ix, iy);
            if (uw >= 0) C.off_u[uw] = make_int2(ix, iy);
        }
        return cell;
    }
    return -1;
}

// Standalone histogram of the *_out state (upload, explicit update_chunks!,
// the rings step). The guess of the exact binning: use_guess 1 = the slot's
// chunk in the *_cur order (rings step), 2 = the chunk the slot's particle
// had at the last histogram (after an upload; -1 before the first one).
// src != null: the positions are first gathered from the user-order upload
// buffer into pos_out (an upload's gather fused into its histogram).
template <int PREC>
__global__ void k_count(Ctx C, int32_t use_guess, const double2* __restrict__ src) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = s < C.M;
    int64_t cell = 0;
    int32_t cap = 1 << 30;
    if (valid) {
        const DevRep& R = C.reps[C.num_reps > 1 ? C.rep_out[s] : 0];
        bool parked = false;
        if (C.var_rings) {   // particles of inactive rings take no chunk (update_ids!)
            const int32_t ring = (C.uid_out[s] - (int32_t)R.slot0) / R.nmax;
            parked = C.ring_active[R.ring0 + ring] == 0;
        }
        const int32_t us = (src || C.pos_u) ? C.uid_out[s] : -1;
        const double2 p = src ? src[us] : C.pos_out[s];
        if (src) C.pos_out[s] = p;
        const int32_t uw = C.pos_u ? us : -1;   // rings: the user-order copy too
        if (parked) {
            cell = C.park;
        } else {
            int64_t guess = use_guess == 1 ? (int64_t)C.cell_cur[s] : (use_guess == 2 ? (int64_t)C.cell_out[s] : -1);
            if (guess == C.park) guess = -1;
            // the fixed-point fast path first (a guess is the particle's chunk at
            // the last histogram), the exact Julia formula when it cannot decide
            cell = guess >= 0 ? bin_fast<PREC>(C, R, s, p.x, p.y, (int32_t)guess, uw) : -1;
            if (cell < 0) cell = bin_final<PREC>(C, R, s, p.x, p.y, guess, uw);
            cap = R.has_chunks ? R.cap : (1 << 30);
        }
        if (uw >= 0) {
            C.pos_u[uw] = p;
            C.cell_u[uw] = (int32_t)cell;
        }
    }
    count_into_chunk(C, valid, s, cell, cap);
}

// Chunk counts and scan-tile totals to zero in one launch (a histogram
// replaced before a chunk update consumed it, e.g. by an upload).
static __global__ void k_zero_counts(int32_t* __restrict__ count, int64_t n, int32_t* __restrict__ tile_sum,
                                     int64_t ntiles) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) count[i] = 0;
    if (i < ntiles) tile_sum[i] = 0;
}

// ===========================================================================
// exclusive scan of chunk counts -> start (1024-chunk tiles)
// ===========================================================================
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int& total) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    int nw = blockDim.x >> 5;
    if (warp == 0) {
        int w = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) smem[lane] = w;
    }
    __syncthreads();
    int warp_prefix = warp > 0 ? smem[warp - 1] : 0;
    total = smem[nw - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// Single-kernel exclusive scan: the histogram already accumulated each tile's
// total, so every block sums the tiles before its own and scans its tile;
// with clear it zeroes the counts it consumed (the chunk update instead lets
// k_scatter take them back to zero as it hands out the places).
// With tile_offs (each tile's offset inside its group of kTileScanThreads
// tiles, and at tile_offs[ntiles + g] the total of group g, from
// k_tile_offsets) a block adds the totals of the groups before its own to its
// offset instead of summing every tile before it, which grows quadratically
// with the number of tiles.
static __global__ void k_scan(int32_t* __restrict__ count, int64_t n, const int32_t* __restrict__ tile_sum,
                              int32_t* __restrict__ start, int64_t* d_step, int32_t advance,
                              const int32_t* __restrict__ tile_offs = nullptr, int32_t clear = 1) {
    __shared__ int smem[32];
    int tile_off;
    if (tile_offs) {
        const int64_t ntiles = gridDim.x, grp = (int64_t)blockIdx.x / kTileScanThreads;
        int pre = 0;
        for (int64_t gi = threadIdx.x; gi < grp; gi += blockDim.x) pre += tile_offs[ntiles + gi];
        block_exclusive_scan(pre, smem, tile_off);
        tile_off += tile_offs[blockIdx.x];
    } else {
        int pre = 0;
        for (int64_t t = threadIdx.x; t < (int64_t)blockIdx.x; t += blockDim.x) pre += tile_sum[t];
        block_exclusive_scan(pre, smem, tile_off);
    }
    static_assert(kScanItems % 4 == 0, "int4 loads");
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    const bool full = base + kScanItems <= n;   // count is 16-byte aligned and base a multiple of 4
    // a tile whose total is zero holds only zero counts (sparse grids: a third
    // of the rings workload's tiles): its counts are not read
    const bool empty = tile_sum[blockIdx.x] == 0;
    if (empty) {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) v[k] = 0;
    } else if (full) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; q++) {
            const int4 c = *reinterpret_cast<const int4*>(count + base + 4 * q);
            v[4 * q] = c.x; v[4 * q + 1] = c.y; v[4 * q + 2] = c.z; v[4 * q + 3] = c.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; k++) v[k] = (base + k < n) ? count[base + k] : 0;
    }
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) sum += v[k];
    int total;
    int run = block_exclusive_scan(sum, smem, total) + tile_off;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {   // v becomes the exclusive prefix
        const int c = v[k];
        v[k] = run;
        run += c;
    }
    if (full) {
        // start has n + 1 entries and the same alignment as count
#pragma unroll
        for (int q = 0; q < kScanItems / 4; q++) {
            *reinterpret_cast<int4*>(start + base + 4 * q) = make_int4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            if (clear) *reinterpret_cast<int4*>(count + base + 4 * q) = make_int4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; k++)
            if (base + k < n) { start[base + k] = v[k]; if (clear) count[base + k] = 0; }
    }
    if (threadIdx.x == 0) {
        if (blockIdx.x == gridDim.x - 1) start[n] = tile_off + total;
        if (advance && blockIdx.x == 0) d_step[0] += 1;
    }
}

// Offsets of the tile totals inside groups of kTileScanThreads tiles, one
// block per group (grids with many tiles): tile_offs[t] = exclusive scan
// within the group, tile_offs[ntiles + g] = the group's total.
static __global__ void __launch_bounds__(kTileScanThreads) k_tile_offsets(const int32_t* __restrict__ tile_sum,
                                                                          int64_t ntiles,
                                                                          int32_t* __restrict__ tile_offs) {
    __shared__ int smem[32];
    const int64_t t = (int64_t)blockIdx.x * kTileScanThreads + threadIdx.x;
    const int v = t < ntiles ? tile_sum[t] : 0;
    int total;
    const int ex = block_exclusive_scan(v, smem, total);
    if (t < ntiles) tile_offs[t] = ex;
    if (threadIdx.x == 0) tile_offs[ntiles + blockIdx.x] = total;
}

// ===========================================================================
// scatter: each particle claims a place in its chunk. The scan left the
// counts in place; taking them back down one claim at a time hands out the
// places 0..count-1 (in no particular order: k_permute orders each chunk) and
// leaves the counts at zero for the next histogram.
// ===========================================================================
static __global__ void k_scatter(Ctx C) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < C.ntiles) C.tile_sum[s] = 0;   // k_scan has consumed the tile sums
    if (s >= C.M) return;
    const int32_t c = C.cell_out[s];
    const int32_t r = atomicSub(&C.count[c], 1) - 1;
    const int32_t b = C.start[c];
    if (r == 0 && c != C.park) {
        // chunk capacity (src/chunks.jl:32-34; the reference's BoundsError), once per chunk
        const DevRep& R = C.reps[C.num_reps > 1 ? C.rep_out[s] : 0];
        if (R.has_chunks && C.start[c + 1] - b > R.cap) raise_error(C.err, MAVI_ERR_CHUNK_OVERFLOW, s, c);
    }
    const int32_t dst = b + r;
    // places are < count[c], so dst stays inside [start[c], start[c+1])
    C.src_of[dst] = (int32_t)s;
    C.key_of[dst] = C.uid_out[s];
    C.cell_at[dst] = c;
}

struct RingInfo {
    int32_t ring;   // replica-local ring index
    int32_t p;      // particle index inside the ring
    int32_t type;   // 0-based
};

__device__ __forceinline__ RingInfo ring_info(const Ctx& C, const DevRep& R, int32_t uid) {
    int32_t local = uid - (int32_t)R.slot0;
    RingInfo ri;
    ri.ring = local / R.nmax;
    ri.p = local - ri.ring * R.nmax;
    ri.type = C.ring_types[R.ring0 + ri.ring] - 1;
    return ri;
}

// Ring identity of the particle in sorted slot j, as the pair terms take it:
// the word k_permute keeps beside the position (replica-local ring in bits
// 12-31, index in the ring in bits 2-11, type in bits 0-1: one load instead
// of the user id, a division and the type table), or the user id when the
// rings exceed that packing.
constexpr int kRingKeyMaxNmax = 1 << 10;
constexpr int kRingKeyMaxRings = 1 << 20;
__device__ __forceinline__ int32_t ring_key(const Ctx& C, int32_t j) {
    return C.rinfo_cur ? C.rinfo_cur[j] : C.uid_cur[j];
}
__device__ __forceinline__ RingInfo ring_of_key(const Ctx& C, const DevRep& R, int32_t key) {
    if (C.rinfo_cur) {
        RingInfo r;
        r.type = key & 3;
        r.p = (key >> 2) & (kRingKeyMaxNmax - 1);
        r.ring = (int32_t)((uint32_t)key >> 12);
        return r;
    }
    return ring_info(C, R, key);
}
__device__ __forceinline__ int32_t user_of_key(const Ctx& C, const DevRep& R, int32_t key, const RingInfo& o) {
    return C.rinfo_cur ? (int32_t)R.slot0 + o.ring * R.nmax + o.p : key;
}

// ===========================================================================
// Per claimed slot: the particle's place inside its chunk is its rank by user
// id (the reference appends particles in ascending id, src/chunks.jl:150-161),
// which makes the order deterministic; the state moves into *_cur.
// ===========================================================================
template <int PREC, bool HAS_VEL, bool HAS_POL>
__global__ void k_permute(Ctx C) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= C.M) return;
    // the scatter left each claimed slot's user id and chunk beside it, so the
    // rank loop reads one array and the chunk range needs no gather
    int32_t sm = C.src_of[p];
    int32_t c = C.cell_at[p];
    int32_t u = C.key_of[p];
    int32_t b = C.start[c], e = C.start[c + 1];
    int32_t rank = 0;
    for (int32_t q = b; q < e; q++) rank += (C.key_of[q] < u) ? 1 : 0;
    int32_t dst = b + rank;
    C.pos_cur[dst] = C.pos_out[sm];
    C.uid_cur[dst] = u;
    if (C.num_reps > 1) C.rep_cur[dst] = C.rep_out[sm];   // one replica: stays 0
    C.cell_cur[dst] = c;
    C.slot_of[u] = dst;
    if (C.rinfo_cur) C.rinfo_cur[dst] = C.rkey_user[u];
    if constexpr (HAS_VEL) C.vel_cur[dst] = C.vel_out[sm];
    if constexpr (HAS_POL) C.pol_cur[dst] = C.pol_out[sm];
    if constexpr (PREC == kPrecMixed) C.off_cur[dst] = C.off_out[sm];
}

// ===========================================================================
// pair-force gather. Each thread owns one particle and sums the force exerted
// on it by every candidate of the chunk stencil. The reference evaluates each
// unordered candidate pair once over a half-shell stencil (src/chunks.jl:61-118)
// and applies Newton's third law (src/integration.jl:112-157); summing over the
// full 3x3 neighbourhood visits the same pair set from both sides (the
// half-shell and its mirror form the 8-neighbourhood, clipped at open edges,
// wrapped when periodic with >= 3 chunks per side), so every particle
// receives exactly the reference's pair terms, without atomics and in a fixed
// order (deterministic).
//
// FP64 form: differences of FP64 positions, FP64 pair law.
// Mixed form: differences of fixed-point offsets plus the exact stencil shift
// are exact integers (so are the squared distance, the minimum image and the
// cutoff test); the pair law runs in FP32, with the cancelling term of the
// harmonic laws (dist_eq^2 - d^2) formed exactly in int64 first.
// ===========================================================================


// Rings pair term (src/rings/integration.jl:32-77), FP64: interaction matrix
// by ring type, zero beyond dist_max, bonded neighbours of the same ring
// excluded, attraction only between different rings.
__device__ __forceinline__ double rings_pair_scalar_d(const MaviRingsCfg& rc, int ti, int tj, bool same_ring,
                                                      int32_t pi, int32_t pj, int32_t n_i, double d2) {
    double dmax = rc.inter_dist_max[ti][tj];
    if (d2 > dmax * dmax) return 0.0;
    if (same_ring) {
        int32_t diff = pi > pj ? pi - pj : pj - pi;
        if (diff == 1 || diff == n_i - 1) return 0.0;
    }
    double deq = rc.inter_dist_eq[ti][tj];
    double k;
    if (d2 < deq * deq) k = rc.inter_k_rep[ti][tj];
    else k = same_ring ? 0.0 : rc.inter_k_atr[ti][tj];
    return k * (rsqrt(d2) - 1.0 / deq);
}

// int64 -> float without a 64-bit conversion instruction (those run on the
// FP64 pipe, ~1/70 of the FP32 rate on GB300): hi * 2^32 + lo, hi exact.
__device__ __forceinline__ float i64_to_f32(long long v) {
    int32_t hi = (int32_t)(v >> 32);
    uint32_t lo = (uint32_t)v;
    return fmaf((float)hi, 4294967296.0f, (float)lo);
}
__device__ __forceinline__ float u64_to_f32(unsigned long long v) {
    uint32_t hi = (uint32_t)(v >> 32);
    uint32_t lo = (uint32_t)v;
    return fmaf((float)hi, 4294967296.0f, (float)lo);
}

// Mixed-form pair laws on exact integer differences (units u of the replica).
// dxi, dyi are int32 (|d| < 2^31 units = 8 chunks). The cutoff is tested on
// the FP32 squared distance (relative error < 3e-7) against a 1e-6 band, and
// only pairs inside the band use the exact int64 squared distance; the
// cancelling term of the harmonic laws (dist_eq^2 - d^2) is always formed
// exactly in int64. Returns the force components on i.
template <int DYN>
__device__ __forceinline__ void pair_fixed(const DevRep& R, const FixPair& fp, int32_t dxi, int32_t dyi,
                                           float& fx, float& fy) {
    fx = 0.f;
    fy = 0.f;
    const float dxf = (float)dxi, dyf = (float)dyi;
    const float d2f = fmaf(dxf, dxf, dyf * dyf);
    if (d2f > fp.cut2_hi) return;
    const unsigned long long d2 = (unsigned long long)((long long)dxi * dxi) + (unsigned long long)((long long)dyi * dyi);
    if (d2f >= fp.cut2_lo && d2 > fp.cut2) return;
    if constexpr (DYN == MAVI_DYN_HARM_TRUNC || DYN == MAVI_DYN_RINGS) {
        // f = k (1/d - 1/deq) dr = k (deq^2 - d^2) / (d deq (deq + d)) dr
        const long long D = fp.eq2 - (long long)d2;
        const float k = D > 0 ? fp.k_rep : fp.k_atr;
        const float r = rsqrtf(d2f);
        const float d = d2f * r;
        const float sc = __fdividef(k * i64_to_f32(D) * r, fp.eq * (fp.eq + d));
        fx = sc * dxf;
        fy = sc * dyf;
    } else if constexpr (DYN == MAVI_DYN_SZABO) {
        // f = -f_mod (d - r_eq) dr = -f_mod (d^2 - r_eq^2)/(d + r_eq) dr
        const long long D = (long long)d2 - fp.eq2;
        const float fm = D > 0 ? fp.k_atr : fp.k_rep;
        const float d = d2f * rsqrtf(d2f);
        const float sc = __fdividef(-fm * i64_to_f32(D) * R.u2_f, d + fp.eq);
        fx = sc * dxf;
        fy = sc * dyf;
    }
}

// Whether a pair lies inside the cutoff of fp (FP32 test, exact int64 test
// inside the +-1e-6 band).
__device__ __forceinline__ bool inside_cutoff(const FixPair& fp, int32_t dxi, int32_t dyi) {
    const float dxf = (float)dxi, dyf = (float)dyi;
    const float d2f = fmaf(dxf, dxf, dyf * dyf);
    if (d2f > fp.cut2_hi) return false;
    if (d2f < fp.cut2_lo) return true;
    const unsigned long long d2 = (unsigned long long)((long long)dxi * dxi) + (unsigned long long)((long long)dyi * dyi);
    return d2 <= fp.cut2;
}

// Lennard-Jones force (src/configs.jl:380-397) of the exact integer
// displacement (dxi, dyi), in double-float arithmetic: every value carries a
// float high part and the rounding error of the operation that made it
// (error-free products by fmaf, two-sums), so the result (fxh + fxl,
// fyh + fyl) keeps ~1e-12 relative accuracy with FP32 instructions only. A
// single FP32 evaluation loses ~1e-6 per pair (the r^-14 term amplifies the
// rounding of d^2 sevenfold), which near-cancelling pair sums of a dense
// Lennard-Jones state turn into force errors above 1e-5 of the RMS force.
//   d^2 = S + E (S = fl(dx^2 + dy^2), dx = xh + xl exactly)
//   h + l = d^2 2^-k, t = 1/h, 1/(h + l) = t (1 + e), e = 1 - (h + l) t
//   f/d = (ah + al) (h+l)^-7 - (bh + bl) (h+l)^-4 = t^4 (A t^3 - B) (1 + O(e))
// _rn intrinsics keep the compiler from fusing the products the error terms
// are taken of.
// Hardware reciprocal approximation (about 1 ulp); inputs here are normal
// numbers (scaled squared distances of distinct particles).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void lj_pair_df(const DevRep& R, int32_t dxi, int32_t dyi, float& fxh, float& fxl,
                                           float& fyh, float& fyl) {
    const float xh = (float)dxi, yh = (float)dyi;
    const float xl = (float)(dxi - __float2int_rz(xh)), yl = (float)(dyi - __float2int_rz(yh));
    const float p1 = __fmul_rn(xh, xh), e1 = fmaf(xh, xh, -p1);
    const float p2 = __fmul_rn(yh, yh), e2 = fmaf(yh, yh, -p2);
    const float S = __fadd_rn(p1, p2);
    const float sv = __fsub_rn(S, p1);
    const float E = __fadd_rn(__fsub_rn(p1, __fsub_rn(S, sv)), __fsub_rn(p2, sv)) + e1 + e2 +
                    2.0f * fmaf(xh, xl, yh * yl);
    const float h = __fmul_rn(S, R.lj_sk), l = E * R.lj_sk;   // power-of-two scaling: exact
    // t ~ 1/h to ~1 ulp; e = 1 - (h + l) t is formed exactly enough (the FMA
    // residual) that the first-order correction below absorbs t's error
    const float t = rcp_approx(h);
    const float e = fmaf(-h, t, 1.0f) - l * t;
    const float t2 = __fmul_rn(t, t), t2e = fmaf(t, t, -t2);
    const float t3 = __fmul_rn(t2, t), t3e = fmaf(t2, t, -t3) + t2e * t;
    const float a = __fmul_rn(R.lj_ah, t3);
    const float ae = fmaf(R.lj_ah, t3, -a) + fmaf(R.lj_ah, t3e, R.lj_al * t3);
    const float b = __fsub_rn(a, R.lj_bh);                      // two-sum a + (-bh)
    const float bv = __fsub_rn(b, a);
    const float be = __fadd_rn(__fsub_rn(a, __fsub_rn(b, bv)), __fsub_rn(-R.lj_bh, bv)) + ae - R.lj_bl;
    const float t4 = __fmul_rn(t2, t2), t4e = fmaf(t2, t2, -t4) + 2.0f * t2 * t2e;
    const float sh = __fmul_rn(t4, b);
    float sl = fmaf(t4, b, -sh) + fmaf(t4, be, t4e * b);
    sl = fmaf(e * t4, 7.0f * a - 4.0f * R.lj_bh, sl);         // first order in e
    fxh = __fmul_rn(sh, xh);
    fxl = fmaf(sh, xh, -fxh) + fmaf(sh, xl, sl * xh);
    fyh = __fmul_rn(sh, yh);
    fyl = fmaf(sh, yh, -fyh) + fmaf(sh, yl, sl * yh);
}

// Fixed-point force sums of the tiled (Newton's third law) Lennard-Jones /
// WCA passes. A pair term h + l (double-float) becomes the int64
// round(f 2^32), formed from a coarse part round(h 2^8) and the fine
// remainder (h - coarse 2^-8 + l) 2^32, both int32 conversions. Integer sums
// do not depend on the order of the terms, so shared-memory atomics from any
// thread give the same bits every run; the resolution is 2^-32 per term. A
// term of magnitude 2^22 or more (or not finite) sets `bad`
// (MAVI_ERR_FORCE_RANGE).
constexpr float kFixForceLimit = 1073741824.0f;   // 2^22 * 2^8: |f| < 2^22
__device__ __forceinline__ long long fix_term(float h, float l, bool& bad) {
    const float hs = h * 256.0f;
    bad |= !(fabsf(hs) < kFixForceLimit);
    const float c = rintf(fminf(fmaxf(hs, -kFixForceLimit), kFixForceLimit));
    const float r = __fadd_rn(fmaf(-c, 0.00390625f, h), l);       // f - c 2^-8: |r| <= 2^-9
    return ((long long)__float2int_rn(c) << 24) + (long long)__float2int_rn(r * 4294967296.0f);
}
__device__ __forceinline__ float fix_value(long long v) { return i64_to_f32(v) * 2.3283064365386963e-10f; }

// Force accumulators of the per-particle gathers. Mixed form: FP32,
// Kahan-compensated for Lennard-Jones (no cutoff: tens of terms with
// cancellation), plain for the short-range laws.
template <int PREC, int DYN> struct Acc;
template <int DYN> struct Acc<kPrecFP64, DYN> {
    double x = 0, y = 0;
    int32_t nb = 0;   // rings neighbour count of the lane's particle
    __device__ __forceinline__ double gx() const { return x; }
    __device__ __forceinline__ double gy() const { return y; }
};
template <int DYN> struct Acc<kPrecMixed, DYN> {
    float x = 0, y = 0, cx = 0, cy = 0;
    int32_t nb = 0;   // rings neighbour count of the lane's particle
    __device__ __forceinline__ void add(float fx, float fy) {
        if constexpr (DYN == MAVI_DYN_LEN_JONES) {
            float yx = fx - cx, tx = x + yx;
            cx = (tx - x) - yx;
            x = tx;
            float yy = fy - cy, ty = y + yy;
            cy = (ty - y) - yy;
            y = ty;
        } else {
            x += fx;
            y += fy;
        }
    }
    // a term given as high + low parts (double-float pair laws): the low part
    // goes into the compensation
    __device__ __forceinline__ void add2(float fxh, float fxl, float fyh, float fyl) {
        if constexpr (DYN == MAVI_DYN_LEN_JONES) {
            float yx = fxh - cx, tx = x + yx;
            cx = ((tx - x) - yx) - fxl;
            x = tx;
            float yy = fyh - cy, ty = y + yy;
            cy = ((ty - y) - yy) - fyl;
            y = ty;
        } else {
            x += fxh + fxl;
            y += fyh + fyl;
        }
    }
    __device__ __forceinline__ float gx() const { return x - cx; }
    __device__ __forceinline__ float gy() const { return y - cy; }
};

template <int PREC> struct PartOf { using T = int2; };            // fixed-point offset
template <> struct PartOf<kPrecFP64> { using T = double2; };       // FP64 position

// The particle whose force a lane sums.
template <int PREC, int DYN> struct Me {
    typename PartOf<PREC>::T p;
    int64_t s;        // own sorted slot
    int32_t uid;      // own user slot (rings neighbour lists)
    RingInfo ri;
    int32_t n_ring;
    const FixPair* fixr;
};

template <int PREC, int DYN>
__device__ __forceinline__ Me<PREC, DYN> make_me(const Ctx& C, const DevRep& R, int32_t rep, int64_t s,
                                                 const typename PartOf<PREC>::T* __restrict__ P) {
    Me<PREC, DYN> m;
    m.p = P[s];
    m.s = s;
    m.uid = 0;
    m.ri = RingInfo{0, 0, 0};
    m.n_ring = 0;
    m.fixr = C.fix + (int64_t)rep * MAVI_MAX_TYPES * MAVI_MAX_TYPES;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        m.uid = C.uid_cur[s];
        m.ri = ring_info(C, R, m.uid);
        m.n_ring = C.rcfg[rep].num_particles[m.ri.type];
    }
    return m;
}

// Rings particle neighbour lists (src/rings/neighbors.jl:116-136, called for
// every candidate pair from calc_interaction, src/rings/integration.jl:32-44):
// j is a neighbour of i when dist < max_dist * tol with max_dist =
// 2 * particle_radius = dist_eq of the pair's types, and (type :all or
// different rings). The test uses the reference's FP64 arithmetic on the FP64
// positions (no fused operations), so the sets are exact.
template <int DYN>
__device__ __forceinline__ bool nb_test_fp64(const Ctx& C, const DevRep& R, double dx, double dy, double dist_eq) {
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    return dist < __dmul_rn(2.0 * (dist_eq / 2.0), C.nb_tol);
}

template <class A>
__device__ __forceinline__ void nb_record(const Ctx& C, int32_t me_uid, int32_t other_uid, A& acc) {
    const int32_t k = acc.nb++;
    if (C.nb_mode == 2) {
        if (k < MAVI_MAX_NEIGHBORS) C.nb_list[(int64_t)me_uid * MAVI_MAX_NEIGHBORS + k] = other_uid;
        else raise_error(C.err, MAVI_ERR_NEIGHBOR_OVERFLOW, me_uid, k);
    }
}

// One pair term added to acc: q is the neighbour's position (FP64) or
// offset (mixed), uq its user id (rings), (shx, shy) the stencil shift in
// fixed-point units, mi whether the minimum image applies. The global and the
// staged gathers both call this, in the same order, so they agree bitwise.
// Rings pair law on an exact integer displacement (mixed form): bonded
// neighbours of the same ring excluded, no attraction inside a ring
// (src/rings/integration.jl:32-70).
template <int DYN>
__device__ __forceinline__ void rings_pair_dxy(const DevRep& R, const Me<kPrecMixed, DYN>& me, const RingInfo& o,
                                               int32_t dxi, int32_t dyi, Acc<kPrecMixed, DYN>& acc) {
    const bool same = o.ring == me.ri.ring;
    if (same) {
        int32_t diff = me.ri.p > o.p ? me.ri.p - o.p : o.p - me.ri.p;
        if (diff == 1 || diff == me.n_ring - 1) return;
    }
    FixPair fp = me.fixr[me.ri.type * MAVI_MAX_TYPES + o.type];
    if (same) fp.k_atr = 0.f;
    float fx, fy;
    pair_fixed<DYN>(R, fp, dxi, dyi, fx, fy);
    acc.add(fx, fy);
}

template <int DYN>
__device__ __forceinline__ void pair_term(const Ctx& C, const DevRep& R, int32_t rep, const Me<kPrecFP64, DYN>& me,
                                          double2 q, int32_t uq, int32_t, int32_t, bool mi,
                                          Acc<kPrecFP64, DYN>& acc) {
    double dx = me.p.x - q.x, dy = me.p.y - q.y;
    if (mi) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
    double d2 = dx * dx + dy * dy;
    double sc;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        RingInfo o = ring_of_key(C, R, uq);
        if (C.nb_mode && (C.nb_type_all || o.ring != me.ri.ring) &&
            nb_test_fp64<DYN>(C, R, dx, dy, C.rcfg[rep].inter_dist_eq[me.ri.type][o.type]))
            nb_record(C, me.uid, user_of_key(C, R, uq, o), acc);
        sc = rings_pair_scalar_d(C.rcfg[rep], me.ri.type, o.type, o.ring == me.ri.ring, me.ri.p, o.p, me.n_ring, d2);
    } else {
        sc = pair_scalar<DYN, double>(R.pd, d2);
    }
    acc.x = fma(sc, dx, acc.x);
    acc.y = fma(sc, dy, acc.y);
}

template <int DYN>
__device__ __forceinline__ void pair_term(const Ctx& C, const DevRep& R, int32_t rep, const Me<kPrecMixed, DYN>& me,
                                          int2 oj, int32_t uq, int32_t shx, int32_t shy, bool mi,
                                          Acc<kPrecMixed, DYN>& acc) {
    // offsets are clamped to +-4 chunks and neighbours are <= 1 chunk apart,
    // so the differences fit int32 (wrapping arithmetic)
    int32_t dxi = (int32_t)((uint32_t)me.p.x - (uint32_t)oj.x + (uint32_t)shx);
    int32_t dyi = (int32_t)((uint32_t)me.p.y - (uint32_t)oj.y + (uint32_t)shy);
    if (mi) {   // minimum image (src/integration.jl:43-48) in exact units
        if (abs(dxi) > R.half_bx_i) dxi -= dxi > 0 ? R.bx_i : -R.bx_i;
        if (abs(dyi) > R.half_by_i) dyi -= dyi > 0 ? R.by_i : -R.by_i;
    }
    if constexpr (DYN == MAVI_DYN_LEN_JONES || DYN == MAVI_DYN_RUN_TUMBLE) {
        if constexpr (DYN == MAVI_DYN_RUN_TUMBLE) {
            if (!inside_cutoff(me.fixr[0], dxi, dyi)) return;
        }
        float fxh, fxl, fyh, fyl;
        lj_pair_df(R, dxi, dyi, fxh, fxl, fyh, fyl);
        acc.add2(fxh, fxl, fyh, fyl);
        return;
    }
    if constexpr (DYN == MAVI_DYN_RINGS) {
        RingInfo o = ring_of_key(C, R, uq);
        bool same = o.ring == me.ri.ring;
        if (C.nb_mode && (C.nb_type_all || !same)) {
            // FP32 test on the exact integer displacement; inside the +-1e-6
            // band around the threshold, the reference's FP64 test on positions
            const FixPair& fq = me.fixr[me.ri.type * MAVI_MAX_TYPES + o.type];
            const float dxf = (float)dxi, dyf = (float)dyi;
            const float d2f = fmaf(dxf, dxf, dyf * dyf);
            bool in = d2f < fq.nb2_lo;
            if (!in && d2f <= fq.nb2_hi) {
                const double2 pi = C.pos_cur[me.s], pj = C.pos_cur[C.slot_of[user_of_key(C, R, uq, o)]];
                double ex = pi.x - pj.x, ey = pi.y - pj.y;
                if (R.min_image) { ex = min_image1(ex, R.box_x, R.half_box_x); ey = min_image1(ey, R.box_y, R.half_box_y); }
                in = nb_test_fp64<DYN>(C, R, ex, ey, C.rcfg[rep].inter_dist_eq[me.ri.type][o.type]);
            }
            if (in) nb_record(C, me.uid, user_of_key(C, R, uq, o), acc);
        }
        rings_pair_dxy<DYN>(R, me, o, dxi, dyi, acc);
    } else {
        float fx, fy;
        pair_fixed<DYN>(R, me.fixr[0], dxi, dyi, fx, fy);
        acc.add(fx, fy);
    }
}

// Pair term of a neighbour reached through a wrapped periodic stencil on a
// space without minimum image (periodic walls on a non-rectangular geometry):
// the reference takes the raw difference r1 - r2 there (src/integration.jl:
// 38-52), a vector across the box. FP64 positions give it directly; the
// mixed form forms it from the exact integer offsets and the true chunk
// distance (shx, shy in units, int64) and evaluates the pair law in FP64
// (such pairs are rare and far apart).
template <int DYN>
__device__ __forceinline__ void pair_term_raw(const Ctx& C, const DevRep& R, int32_t rep,
                                              const Me<kPrecFP64, DYN>& me, double2 q, int32_t uq, long long,
                                              long long, Acc<kPrecFP64, DYN>& acc) {
    pair_term<DYN>(C, R, rep, me, q, uq, 0, 0, false, acc);
}

template <int DYN>
__device__ __forceinline__ void pair_term_raw(const Ctx& C, const DevRep& R, int32_t rep,
                                              const Me<kPrecMixed, DYN>& me, int2 oj, int32_t uq, long long shx,
                                              long long shy, Acc<kPrecMixed, DYN>& acc) {
    const double dx = (double)((long long)me.p.x - oj.x + shx) / R.inv_u;
    const double dy = (double)((long long)me.p.y - oj.y + shy) / R.inv_u;
    const double d2 = dx * dx + dy * dy;
    double sc;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        RingInfo o = ring_of_key(C, R, uq);
        if (C.nb_mode && (C.nb_type_all || o.ring != me.ri.ring)) {
            const int32_t uo = user_of_key(C, R, uq, o);
            const double2 pi = C.pos_cur[me.s], pj = C.pos_cur[C.slot_of[uo]];
            if (nb_test_fp64<DYN>(C, R, pi.x - pj.x, pi.y - pj.y, C.rcfg[rep].inter_dist_eq[me.ri.type][o.type]))
                nb_record(C, me.uid, uo, acc);
        }
        sc = rings_pair_scalar_d(C.rcfg[rep], me.ri.type, o.type, o.ring == me.ri.ring, me.ri.p, o.p, me.n_ring, d2);
    } else {
        sc = pair_scalar<DYN, double>(R.pd, d2);
    }
    acc.add((float)(sc * dx), (float)(sc * dy));
}

// Global-memory gather of one lane (also the all-pairs mode without chunks).
template <int PREC, int DYN>
__device__ __forceinline__ void gather_global(const Ctx& C, const DevRep& R, int32_t rep, int64_t s, int32_t cell,
                                              const typename PartOf<PREC>::T* __restrict__ P,
                                              const Me<PREC, DYN>& me, Acc<PREC, DYN>& acc) {
    // own: the particle's own chunk (the only one that holds the particle itself)
    auto visit = [&](auto own, int32_t b, int32_t e, int32_t shx, int32_t shy, bool mi, bool raw = false,
                     long long rshx = 0, long long rshy = 0) {
        for (int32_t j = b; j < e; j++) {
            if constexpr (decltype(own)::value) {
                if (j == (int32_t)s) continue;
            }
            int32_t uq = 0;
            if constexpr (DYN == MAVI_DYN_RINGS) uq = ring_key(C, j);
            if (raw) pair_term_raw<DYN>(C, R, rep, me, P[j], uq, rshx, rshy, acc);
            else pair_term<DYN>(C, R, rep, me, P[j], uq, shx, shy, mi, acc);
        }
    };
    if (!R.has_chunks) {  // all pairs inside the replica (src/integration.jl:197-224): its one chunk
        visit(std::true_type{}, C.start[R.c0], C.start[R.c0 + 1], 0, 0, R.min_image);
        return;
    }
    int32_t lc = (int32_t)(cell - R.c0);
    int32_t col = lc / R.rows, row = lc - col * R.rows;
#pragma unroll 1
    for (int dc = -1; dc <= 1; dc++) {
        int ncol = col + dc;
        bool wrapped = false;
        if (R.periodic) {
            if (ncol < 0) { ncol += R.cols; wrapped = true; }
            else if (ncol >= R.cols) { ncol -= R.cols; wrapped = true; }
        } else if (ncol < 0 || ncol >= R.cols) continue;
#pragma unroll 1
        for (int dr = -1; dr <= 1; dr++) {
            int nrow = row + dr;
            bool wr = wrapped;
            if (R.periodic) {
                if (nrow < 0) { nrow += R.rows; wr = true; }
                else if (nrow >= R.rows) { nrow -= R.rows; wr = true; }
            } else if (nrow < 0 || nrow >= R.rows) continue;
            int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
            // centre of the neighbour chunk relative to ours, in units:
            // x grows with the column, y decreases with the row
            const bool raw = wr && !R.min_image;
            const int32_t b = C.start[nc], e = C.start[nc + 1];
            const bool mi = R.min_image && (wr || R.mi_small);
            if (dc == 0 && dr == 0) visit(std::true_type{}, b, e, 0, 0, mi);
            else visit(std::false_type{}, b, e, -dc * R.sx_i, dr * R.sy_i, mi, raw,
                       -(long long)(ncol - col) * R.sx_u, (long long)(nrow - row) * R.sy_u);
        }
    }
}

// Column-range gather of one lane: in each of the three neighbouring chunk
// columns the rows row-1..row+1 are consecutive chunks, hence one contiguous
// particle range (unless the stencil wraps around the column or is clipped),
// read directly from global memory (neighbouring lanes read overlapping
// ranges, so the loads hit L1). Same terms in the same order as the other
// gathers, so the sums agree bitwise; suits sparse grids (about one particle
// per chunk), where staging a window costs more than it saves.
//
// lane / lanes: with several lanes per particle (k_pass with LANES > 1) lane l
// takes the candidates t = l, l + lanes, ... of the flat loop; outside the
// flat loop lane 0 takes them all. The lanes' partial sums are combined in a
// fixed order by the caller.
template <int PREC, int DYN>
__device__ __forceinline__ void gather_columns(const Ctx& C, const DevRep& R, int32_t rep, int64_t s, int32_t cell,
                                               const typename PartOf<PREC>::T* __restrict__ P,
                                               const Me<PREC, DYN>& me, Acc<PREC, DYN>& acc, int lane = 0,
                                               int lanes = 1) {
    const int32_t lc = (int32_t)(cell - R.c0);
    const int32_t col = lc / R.rows, row = lc - col * R.rows;
    const bool rows_inside = row >= 1 && row + 1 < R.rows;
    if (rows_inside) {
        // all twelve chunk boundaries first (independent loads in flight
        // together), then the three ranges
        int32_t g[3][4];
        int32_t ncl[3];
        bool cws[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            int ncol = col + k - 1;
            bool cw = false, ok = true;
            if (R.periodic) {
                if (ncol < 0) { ncol += R.cols; cw = true; }
                else if (ncol >= R.cols) { ncol -= R.cols; cw = true; }
            } else {
                ok = ncol >= 0 && ncol < R.cols;
            }
            const int64_t cb = R.c0 + (int64_t)(ok ? ncol : col) * R.rows;
#pragma unroll
            for (int q = 0; q < 4; q++) g[k][q] = C.start[cb + row - 1 + q];
            if (!ok) { g[k][0] = 0; g[k][3] = 0; }
            ncl[k] = ncol;
            cws[k] = cw;
        }
        // short-range laws: one loop over the three column ranges in order
        // (the terms and the order of the per-column loops), unrolled so that
        // several neighbour loads are in flight at once (measured 9 % faster
        // for rings; the register-heavy double-float LJ term is faster per
        // column)
        constexpr bool kFlat = DYN != MAVI_DYN_LEN_JONES && DYN != MAVI_DYN_RUN_TUMBLE;
        if (kFlat && (R.min_image || !R.periodic)) {
            const int32_t n0 = g[0][3] - g[0][0], n1 = g[1][3] - g[1][0], n2 = g[2][3] - g[2][0];
            const int32_t n01 = n0 + n1, tot = n01 + n2;
            const bool mi0 = R.min_image && (cws[0] || R.mi_small);
            const bool mi1 = R.min_image && (cws[1] || R.mi_small);
            const bool mi2 = R.min_image && (cws[2] || R.mi_small);
#pragma unroll 4
            for (int32_t t = lane; t < tot; t += lanes) {
                const bool k0 = t < n0, k1 = !k0 && t < n01;
                const int32_t j = k0 ? g[0][0] + t : (k1 ? g[1][0] + (t - n0) : g[2][0] + (t - n01));
                if (j == (int32_t)s) continue;
                const int32_t b1 = k0 ? g[0][1] : (k1 ? g[1][1] : g[2][1]);
                const int32_t b2 = k0 ? g[0][2] : (k1 ? g[1][2] : g[2][2]);
                const int dr = j < b1 ? -1 : (j < b2 ? 0 : 1);
                const int32_t shx = k0 ? R.sx_i : (k1 ? 0 : -R.sx_i);
                const bool mi = k0 ? mi0 : (k1 ? mi1 : mi2);
                int32_t uq = 0;
                if constexpr (DYN == MAVI_DYN_RINGS) uq = ring_key(C, j);
                pair_term<DYN>(C, R, rep, me, P[j], uq, shx, dr * R.sy_i, mi, acc);
            }
            return;
        }
        if (lane != 0) return;
#pragma unroll 1
        for (int k = 0; k < 3; k++) {
            const int dc = k - 1;
            const bool cw = cws[k];
            const bool mi_c = R.min_image && (cw || R.mi_small);
            const int32_t shx = -dc * R.sx_i;
            const long long rshx = -(long long)(ncl[k] - col) * R.sx_u;
            const int32_t g0 = g[k][0], g1 = g[k][1], g2 = g[k][2], g3 = g[k][3];
            const int32_t self = (dc == 0) ? (int32_t)s : -1;
            const bool raw = cw && !R.min_image;
#pragma unroll 2
            for (int32_t j = g0; j < g3; j++) {
                if (j == self) continue;
                const int dr = j < g1 ? -1 : (j < g2 ? 0 : 1);
                int32_t uq = 0;
                if constexpr (DYN == MAVI_DYN_RINGS) uq = ring_key(C, j);
                if (raw) pair_term_raw<DYN>(C, R, rep, me, P[j], uq, rshx, (long long)dr * R.sy_u, acc);
                else pair_term<DYN>(C, R, rep, me, P[j], uq, shx, dr * R.sy_i, mi_c, acc);
            }
        }
        return;
    }
    if (lane != 0) return;
#pragma unroll 1
    for (int dc = -1; dc <= 1; dc++) {
        int ncol = col + dc;
        bool cw = false;
        if (R.periodic) {
            if (ncol < 0) { ncol += R.cols; cw = true; }
            else if (ncol >= R.cols) { ncol -= R.cols; cw = true; }
        } else if (ncol < 0 || ncol >= R.cols) continue;
        const bool mi_c = R.min_image && (cw || R.mi_small);
        const int32_t shx = -dc * R.sx_i;
        const long long rshx = -(long long)(ncol - col) * R.sx_u;
        const int64_t cb = R.c0 + (int64_t)ncol * R.rows;
        // rows row-1..row+1 clipped or wrapped: chunk by chunk
#pragma unroll 1
        for (int dr = -1; dr <= 1; dr++) {
            int nrow = row + dr;
            bool rw = false;
            if (R.periodic) {
                if (nrow < 0) { nrow += R.rows; rw = true; }
                else if (nrow >= R.rows) { nrow -= R.rows; rw = true; }
            } else if (nrow < 0 || nrow >= R.rows) continue;
            const int32_t b = C.start[cb + nrow], e = C.start[cb + nrow + 1];
            const bool mi = mi_c || (R.min_image && rw);
            const bool raw = (cw || rw) && !R.min_image;
            for (int32_t j = b; j < e; j++) {
                if (j == (int32_t)s) continue;
                int32_t uq = 0;
                if constexpr (DYN == MAVI_DYN_RINGS) uq = ring_key(C, j);
                if (raw) pair_term_raw<DYN>(C, R, rep, me, P[j], uq, rshx, (long long)(nrow - row) * R.sy_u, acc);
                else pair_term<DYN>(C, R, rep, me, P[j], uq, shx, dr * R.sy_i, mi, acc);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Warp-staged gather. The 32 particles of a warp are consecutive in chunk
// order, so they sit in a short run of rows [rmin, rmax] of one (or two)
// chunk columns. For each column present, the rows [rmin-1, rmax+1] of the
// three neighbouring columns are at most two contiguous particle ranges each
// (two when a periodic window wraps): the warp copies these <= 6 segments
// into shared memory with coalesced loads, and each lane then reads its own
// neighbour rows there, mapping global particle indices through the segment
// table. Windows that do not fit fall back to the global gather (same terms
// in the same order, bitwise-identical sums).
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Split gather of the mixed Lennard-Jones pass (pass mode 7), over the same
// chunk loops as gather_global. A candidate at r >= 2 sigma (R.lj_near2,
// units^2) is evaluated on the spot in plain FP32: its force is below
// ~0.2 eps / sigma, so the ~10 ulp of that form stay far under the
// double-float error of the close pairs (the first two neighbour shells). A
// closer candidate's exact integer displacement is parked in the thread's
// slots of shared memory (`slots`, stride kPassThreads, kSplitSlots of them)
// and evaluated in double-float afterwards, so the costly term runs ~7-9
// times per particle instead of ~33, with no divergence between the two forms
// inside a warp, and the candidate loop carries no double-float registers. Order: the close terms in candidate order into the
// compensated sum, then the raw wrapped pairs of periodic spaces without
// minimum image (their chunks are set aside in the first loop), then the FP32
// sum of the far ones: fixed, so deterministic. Both particles of a pair see
// the same displacement (negated), hence the same classification and opposite
// forces. A particle with more close candidates than slots takes gather_global
// instead (every term in double-float).
// ---------------------------------------------------------------------------
#ifndef MAVI_SPLIT_SLOTS
#define MAVI_SPLIT_SLOTS 14
#endif
#ifndef MAVI_SPLIT_UNROLL
#define MAVI_SPLIT_UNROLL 1
#endif
constexpr int kSplitSlots = MAVI_SPLIT_SLOTS;   // close candidates parked per particle (8 B each per thread)
constexpr int kSplitUnroll = MAVI_SPLIT_UNROLL;
#ifndef MAVI_SPLIT_NEAR_UNROLL
#define MAVI_SPLIT_NEAR_UNROLL 1
#endif
constexpr int kSplitNearUnroll = MAVI_SPLIT_NEAR_UNROLL;

template <int DYN>
__device__ __forceinline__ void gather_split(const Ctx& C, const DevRep& R, int32_t rep, int64_t s, int32_t cell,
                                             const int2* __restrict__ P, const Me<kPrecMixed, DYN>& me,
                                             Acc<kPrecMixed, DYN>& acc, int2* __restrict__ slots) {
    float fx = 0.f, fy = 0.f;
    int n_near = 0;
    const float near2 = R.lj_near2, sk = R.lj_sk, ah = R.lj_ah, bh = R.lj_bh;
    // one candidate: the FP32 term on the spot, or the displacement parked
    auto term = [&](auto own, int32_t j, int2 oj, int32_t shx, int32_t shy, bool mi) {
        if constexpr (decltype(own)::value) {   // the particle's own chunk holds the particle itself
            if (j == (int32_t)s) return;
        }
        int32_t dxi = (int32_t)((uint32_t)me.p.x - (uint32_t)oj.x + (uint32_t)shx);
        int32_t dyi = (int32_t)((uint32_t)me.p.y - (uint32_t)oj.y + (uint32_t)shy);
        if (mi) {   // minimum image (src/integration.jl:43-48) in exact units
            if (abs(dxi) > R.half_bx_i) dxi -= dxi > 0 ? R.bx_i : -R.bx_i;
            if (abs(dyi) > R.half_by_i) dyi -= dyi > 0 ? R.by_i : -R.by_i;
        }
        const float xf = (float)dxi, yf = (float)dyi;
        const float S = fmaf(xf, xf, yf * yf);
        if (S < near2) {
            if (n_near < kSplitSlots) slots[n_near * kPassThreads] = make_int2(dxi, dyi);
            n_near++;
        } else {
            // (48 eps sigma^12 / r^14 - 24 eps sigma^6 / r^8) d in the scaled units
            const float ti = rcp_approx(S * sk);
            const float t2 = ti * ti;
            const float sh = fmaf(ah, t2 * ti, -bh) * (t2 * t2);
            fx = fmaf(sh, xf, fx);
            fy = fmaf(sh, yf, fy);
        }
    };
    auto visit = [&](auto own, int32_t b, int32_t e, int32_t shx, int32_t shy, bool mi) {
#pragma unroll kSplitUnroll
        for (int32_t j = b; j < e; j++) term(own, j, P[j], shx, shy, mi);
    };
    int32_t col = 0, row = 0;
    uint32_t raw_chunks = 0;   // bit 3 (dc + 1) + (dr + 1): a wrapped chunk without minimum image
    if (!R.has_chunks) {  // all pairs inside the replica (src/integration.jl:197-224): its one chunk
        visit(std::true_type{}, C.start[R.c0], C.start[R.c0 + 1], 0, 0, R.min_image);
    } else {
        const int32_t lc = (int32_t)(cell - R.c0);
        col = lc / R.rows;
        row = lc - col * R.rows;
#pragma unroll 1
        for (int dc = -1; dc <= 1; dc++) {
            int ncol = col + dc;
            bool wrapped = false;
            if (R.periodic) {
                if (ncol < 0) { ncol += R.cols; wrapped = true; }
                else if (ncol >= R.cols) { ncol -= R.cols; wrapped = true; }
            } else if (ncol < 0 || ncol >= R.cols) continue;
#pragma unroll 1
            for (int dr = -1; dr <= 1; dr++) {
                int nrow = row + dr;
                bool wr = wrapped;
                if (R.periodic) {
                    if (nrow < 0) { nrow += R.rows; wr = true; }
                    else if (nrow >= R.rows) { nrow -= R.rows; wr = true; }
                } else if (nrow < 0 || nrow >= R.rows) continue;
                if (wr && !R.min_image) {
                    raw_chunks |= 1u << (3 * (dc + 1) + (dr + 1));
                    continue;
                }
                const int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
                const int32_t b = C.start[nc], e = C.start[nc + 1];
                const bool mi = R.min_image && (wr || R.mi_small);
                if (dc == 0 && dr == 0) visit(std::true_type{}, b, e, 0, 0, mi);
                else visit(std::false_type{}, b, e, -dc * R.sx_i, dr * R.sy_i, mi);
            }
        }
    }
    if (n_near > kSplitSlots) {   // rare: more close candidates than slots
        gather_global<kPrecMixed, DYN>(C, R, rep, s, cell, P, me, acc);
        return;
    }
#pragma unroll kSplitNearUnroll
    for (int k = 0; k < n_near; k++) {
        const int2 d = slots[k * kPassThreads];
        float fxh, fxl, fyh, fyl;
        lj_pair_df(R, d.x, d.y, fxh, fxl, fyh, fyl);
        acc.add2(fxh, fxl, fyh, fyl);
    }
#pragma unroll 1
    while (raw_chunks) {   // periodic spaces without minimum image: the raw difference (src/integration.jl:38-52)
        const int bit = __ffs(raw_chunks) - 1;
        raw_chunks &= raw_chunks - 1;
        const int dc = bit / 3 - 1, dr = bit % 3 - 1;
        int ncol = col + dc, nrow = row + dr;
        ncol += ncol < 0 ? R.cols : (ncol >= R.cols ? -R.cols : 0);
        nrow += nrow < 0 ? R.rows : (nrow >= R.rows ? -R.rows : 0);
        const int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
        const long long rshx = -(long long)(ncol - col) * R.sx_u, rshy = (long long)(nrow - row) * R.sy_u;
        for (int32_t j = C.start[nc]; j < C.start[nc + 1]; j++)
            if (j != (int32_t)s) pair_term_raw<DYN>(C, R, rep, me, P[j], 0, rshx, rshy, acc);
    }
    acc.add(fx, fy);
}

constexpr int kNumGatherModes = 3; // staged window, per-chunk global, per-column global
constexpr int kGatherTiles = 3;      // Lennard-Jones / WCA, mixed form: Newton's-third-law tiles, a CTA per tile
constexpr int kGatherTilesQueue = 4; // the same tiles from a device work queue (persistent CTAs)
constexpr int kGatherLanes2 = 5;      // mixed short-range laws: column gather, 2 lanes per particle
constexpr int kGatherLanes4 = 6;      // the same, 4 lanes per particle
constexpr int kGatherSplit = 7;       // mixed Lennard-Jones: far pairs in FP32, close ones in double-float
constexpr int kNumPassModes = 8;
constexpr int kStageParts = 256;   // staged particles per window

constexpr int kStageRows = 64;     // window rows per column

template <int PREC, int DYN> struct Stage {
    typename PartOf<PREC>::T part[kStageParts];
    int32_t uid[DYN == MAVI_DYN_RINGS ? kStageParts : 1];
    int32_t rbeg[3][kStageRows];   // global first particle of window row w of column k
    int32_t rend[3][kStageRows];   // one past its last particle
};

// Element j of a 6-entry register table (select chain: no local memory).
__device__ __forceinline__ int32_t pick6(const int32_t (&a)[6], int j) {
    int32_t v = a[0];
#pragma unroll
    for (int t = 1; t < 6; t++) v = (j == t) ? a[t] : v;
    return v;
}

// Shared-memory slot of global particle index g of column k (segments 2k and
// 2k+1; g lies in one of them).
__device__ __forceinline__ int seg_map(const int32_t (&sb)[6], const int32_t (&se)[6], const int32_t (&base)[6],
                                       int k, int32_t g) {
    int j = 2 * k;
    if (!(g >= pick6(sb, j) && g < pick6(se, j))) j++;
    return pick6(base, j) + (g - pick6(sb, j));
}

template <int PREC, int DYN>
__device__ __forceinline__ void gather_warp(const Ctx& C, bool valid, int64_t s, int32_t rep, const DevRep& R,
                                            int32_t cell, const typename PartOf<PREC>::T* __restrict__ P,
                                            Stage<PREC, DYN>& st, Acc<PREC, DYN>& acc) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool want = valid && R.has_chunks;
    // all lanes of a staged window must belong to one replica
    unsigned vmask = __ballot_sync(full, valid);
    int first = vmask ? __ffs(vmask) - 1 : 0;
    int32_t rep0 = __shfl_sync(full, rep, first);
    // windows are replica-uniform; the mixed form stages no window whose
    // stencil may wrap without minimum image (raw displacements, see above)
    const bool stageable = PREC == kPrecFP64 || !(R.periodic && !R.min_image);
    bool uniform = __all_sync(full, !valid || (rep == rep0 && stageable));
    Me<PREC, DYN> me;
    if (valid) me = make_me<PREC, DYN>(C, R, rep, s, P);
    int32_t col = 0, row = 0;
    if (want) {
        int32_t lc = (int32_t)(cell - R.c0);
        col = lc / R.rows;
        row = lc - col * R.rows;
    }
    unsigned pending = (uniform && C.gather_mode == 0) ? __ballot_sync(full, want) : 0u;
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int ccur = __shfl_sync(full, col, leader);
        const bool act = ((pending >> lane) & 1u) && col == ccur;
        const unsigned amask = __ballot_sync(full, act);
        const int rmin = __reduce_min_sync(full, act ? row : 0x7fffffff);
        const int rmax = __reduce_max_sync(full, act ? row : -0x7fffffff);
        // the replica of every active lane (windows are replica-uniform)
        const int nrows = __shfl_sync(full, R.rows, leader), ncols = __shfl_sync(full, R.cols, leader);
        const int periodic = __shfl_sync(full, R.periodic, leader);
        const long long c0 = __shfl_sync(full, R.c0, leader);
        const int lo = rmin - 1, hi = rmax + 1;
        const int W = hi - lo + 1;
        bool ok = W <= kStageRows && (!periodic || W <= nrows);
        if (ok) {
            // chunk boundaries of the window rows of the three columns
            for (int q = lane; q < 3 * kStageRows; q += 32) {
                const int k = q / kStageRows, w = q - k * kStageRows;
                if (w >= W) continue;
                int ncol = ccur + k - 1, r = lo + w;
                bool inside = true;
                if (periodic) {
                    ncol = ncol < 0 ? ncol + ncols : (ncol >= ncols ? ncol - ncols : ncol);
                    r = r < 0 ? r + nrows : (r >= nrows ? r - nrows : r);
                } else {
                    inside = ncol >= 0 && ncol < ncols && r >= 0 && r < nrows;
                }
                int32_t b = 0, e = 0;
                if (inside) {
                    const long long ch = c0 + (long long)ncol * nrows + r;
                    b = C.start[ch];
                    e = C.start[ch + 1];
                }
                st.rbeg[k][w] = b;
                st.rend[k][w] = e;
            }
        }
        // segment j = 2k + {0: main, 1: wrapped part}: global [sb, se)
        int32_t sbj = 0, sej = 0;
        if (lane < 6) {
            const int k = lane >> 1, part = lane & 1;
            int ncol = ccur + k - 1;
            bool colok = true;
            if (periodic) ncol = ncol < 0 ? ncol + ncols : (ncol >= ncols ? ncol - ncols : ncol);
            else colok = ncol >= 0 && ncol < ncols;
            int ra, rb;   // row range of this segment, empty when ra > rb
            if (periodic) {
                if (lo < 0) { if (part == 0) { ra = 0; rb = hi; } else { ra = nrows + lo; rb = nrows - 1; } }
                else if (hi >= nrows) { if (part == 0) { ra = lo; rb = nrows - 1; } else { ra = 0; rb = hi - nrows; } }
                else { ra = part == 0 ? lo : 1; rb = part == 0 ? hi : 0; }
            } else {
                ra = part == 0 ? max(lo, 0) : 1;
                rb = part == 0 ? min(hi, nrows - 1) : 0;
            }
            if (colok && ra <= rb) {
                long long cb = c0 + (long long)ncol * nrows;
                sbj = C.start[cb + ra];
                sej = C.start[cb + rb + 1];
            }
        }
        int32_t sb[6], se[6], base[6];
        int total = 0;
#pragma unroll
        for (int j = 0; j < 6; j++) {
            sb[j] = __shfl_sync(full, sbj, j);
            se[j] = __shfl_sync(full, sej, j);
            base[j] = total;
            total += se[j] - sb[j];
        }
        ok = ok && total <= kStageParts;
        if (ok) {
            for (int idx = lane; idx < total; idx += 32) {
                // segment j: the number of segment ends at or below idx
                int j = 0;
#pragma unroll
                for (int t = 0; t < 5; t++) j += idx >= base[t] + (se[t] - sb[t]) ? 1 : 0;
                const int32_t g = pick6(sb, j) + (idx - pick6(base, j));
                st.part[idx] = P[g];
                if constexpr (DYN == MAVI_DYN_RINGS) st.uid[idx] = ring_key(C, g);
            }
        }
        __syncwarp();
        if (act) {
            if (ok) {
#pragma unroll 1
                for (int k = 0; k < 3; k++) {
                    const int dc = k - 1;
                    const int ncol = ccur + dc;
                    bool cw = false;
                    if (periodic) cw = ncol < 0 || ncol >= ncols;
                    else if (ncol < 0 || ncol >= ncols) continue;
                    const bool mi_c = R.min_image && (cw || R.mi_small);
                    const int32_t shx = -dc * R.sx_i;
                    const int w = row - lo;
                    if (row >= 1 && row + 1 < nrows) {
                        // rows row-1..row+1 are consecutive chunks: one contiguous range
                        const int32_t g0 = st.rbeg[k][w - 1], g1 = st.rbeg[k][w];
                        const int32_t g2 = st.rbeg[k][w + 1], g3 = st.rend[k][w + 1];
                        if (g3 == g0) continue;
                        const int b = seg_map(sb, se, base, k, g0);
                        const int b1 = b + (g1 - g0), b2 = b + (g2 - g0), e = b + (g3 - g0);
                        const int self = (dc == 0) ? b1 + (int)(s - g1) : -1;
#pragma unroll 2
                        for (int idx = b; idx < e; idx++) {
                            if (idx == self) continue;
                            const int dr = idx < b1 ? -1 : (idx < b2 ? 0 : 1);
                            int32_t uq = 0;
                            if constexpr (DYN == MAVI_DYN_RINGS) uq = st.uid[idx];
                            pair_term<DYN>(C, R, rep, me, st.part[idx], uq, shx, dr * R.sy_i, mi_c, acc);
                        }
                    } else {
#pragma unroll 1
                        for (int dr = -1; dr <= 1; dr++) {
                            int r = row + dr;
                            bool rw = false;
                            if (periodic) rw = r < 0 || r >= nrows;
                            else if (r < 0 || r >= nrows) continue;
                            const int32_t g0 = st.rbeg[k][w + dr], g1 = st.rend[k][w + dr];
                            if (g1 == g0) continue;
                            const int b = seg_map(sb, se, base, k, g0);
                            const int e = b + (g1 - g0);
                            const int self = (dc == 0 && dr == 0) ? b + (int)(s - g0) : -1;
                            const bool mi = mi_c || (R.min_image && rw);
                            for (int idx = b; idx < e; idx++) {
                                if (idx == self) continue;
                                int32_t uq = 0;
                                if constexpr (DYN == MAVI_DYN_RINGS) uq = st.uid[idx];
                                pair_term<DYN>(C, R, rep, me, st.part[idx], uq, shx, dr * R.sy_i, mi, acc);
                            }
                        }
                    }
                }
            } else {
                gather_global<PREC, DYN>(C, R, rep, s, cell, P, me, acc);
            }
        }
        __syncwarp();
        pending &= ~amask;
    }
    if (valid && (!want || !uniform || C.gather_mode != 0)) {
        if (want && C.gather_mode == 2) gather_columns<PREC, DYN>(C, R, rep, s, cell, P, me, acc);
        else gather_global<PREC, DYN>(C, R, rep, s, cell, P, me, acc);
    }
}

// ===========================================================================
// PotentialWalls forces (src/integration.jl:228-266) and walls!
// (src/integration.jl:268-412) for one particle.
// ===========================================================================
__device__ __forceinline__ double jsign(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

__device__ __forceinline__ void wall_pot_force(const MaviSpace& sp, double drx, double dry, double dist,
                                               double& fx, double& fy) {
    double sc;
    if (sp.pot_kind == MAVI_DYN_LEN_JONES) {
        double sig = sp.pot_params[0], eps = sp.pot_params[1];
        double fm = 4 * eps * (12 * pow(sig, 12.0) / pow(dist, 13.0) - 6 * pow(sig, 6.0) / pow(dist, 7.0));
        sc = fm / dist;
    } else {
        double k_rep = sp.pot_params[0], k_atr = sp.pot_params[1], deq = sp.pot_params[2], dmax = sp.pot_params[3];
        if (dist > dmax) return;
        double fm = dist < deq ? -k_rep * (dist / deq - 1) : -k_atr * (dist / deq - 1);
        sc = fm / dist;
    }
    fx += sc * drx;
    fy += sc * dry;
}

__device__ __forceinline__ double proc_dist(int mode, double dist, double flag) {
    if (mode == MAVI_POTMODE_OUTSIDE) return flag * dist;
    if (mode == MAVI_POTMODE_INSIDE) return -flag * dist;
    return dist;
}

// Mixed form: the force of the pre-checked PotentialWalls circle (truncated
// harmonic potential; inside or repulsion mode) on a particle at the exact
// integer displacement (wx, wy) from the centre, in FP32. signed_pos
// (src/configs.jl:154-163) gives dist - R and the wall vector dr (1 - R/dist);
// dist - R comes from the exact integer r^2 - R^2 divided by (dist + R), so it
// keeps FP32 relative accuracy next to the wall; process_dist and
// potential_force (src/configs.jl:259-261, 354-368) follow.
__device__ __forceinline__ void wall_circle_f32(const DevRep& R, long long wx, long long wy, float wxf, float wyf,
                                                float& fx, float& fy) {
    const __int128 r2 = (__int128)wx * wx + (__int128)wy * wy;
    const __int128 R2 = (__int128)(((unsigned __int128)(unsigned long long)R.wall_R2_hi << 64) | R.wall_R2_lo);
    const __int128 dd = r2 - R2;
    const long long d64 = dd > (__int128)INT64_MAX ? INT64_MAX : (dd < (__int128)INT64_MIN ? INT64_MIN : (long long)dd);
    const float dist_u = sqrtf(fmaf(wxf, wxf, wyf * wyf));
    const float sd_u = i64_to_f32(d64) / (dist_u + R.wall_Ru_f);    // dist - R, units
    const float sd = sd_u * R.u_f;
    const float d = R.wall_precheck == 1 ? -sd : fabsf(sd);         // inside: -(dist - R)
    if (d > R.wall_dmax_f) return;
    const float k = d < R.wall_deq_f ? R.wall_krep_f : R.wall_katr_f;
    const float fm = -k * (d / R.wall_deq_f - 1.0f);
    const float sc = fm / d * (sd_u / dist_u) * R.u_f;              // times dr (units -> length)
    fx += sc * wxf;
    fy += sc * wyf;
}

static __device__ __forceinline__ void add_wall_forces(const Ctx& C, int32_t rep, const DevRep& R, double x, double y,
                                double& fx, double& fy) {
    const MaviSpace* sps = C.spaces + (int64_t)rep * MAVI_MAX_SPACES;
    for (int k = 0; k < R.num_spaces; k++) {
        const MaviSpace& sp = sps[k];
        if (sp.wall != MAVI_WALL_POTENTIAL) continue;
        if (sp.geometry == MAVI_GEOM_CIRCLE) {   // signed_pos (src/configs.jl:154-163)
            double drx = x - sp.cx, dry = y - sp.cy;
            double r2 = drx * drx + dry * dry;
            if (sp.pot_kind == MAVI_DYN_HARM_TRUNC && sp.pot_mode != MAVI_POTMODE_OUTSIDE) {
                // the truncated potential acts only where |dist - radius| <= dist_max
                // (inside and repulsion modes): skip the rest without the sqrt,
                // with a relative margin far above the rounding of dist
                const double dmax = sp.pot_params[3];
                const double lo = sp.radius - dmax, hi = sp.radius + dmax;
                if (lo > 0 && r2 < lo * lo * (1.0 - 1e-9)) continue;
                if (sp.pot_mode == MAVI_POTMODE_REPULSION && r2 > hi * hi * (1.0 + 1e-9)) continue;
            }
            double dist = sqrt(r2);
            double hx = drx / dist, hy = dry / dist;
            drx = drx - hx * sp.radius;
            dry = dry - hy * sp.radius;
            double sd = dist - sp.radius;
            wall_pot_force(sp, drx, dry, proc_dist(sp.pot_mode, fabs(sd), jsign(sd)), fx, fy);
        } else if (sp.geometry == MAVI_GEOM_LINES) {  // signed_pos (src/configs.jl:119-135)
            for (int l = 0; l < sp.num_lines; l++) {
                double p1x = sp.lines[l][0], p1y = sp.lines[l][1], p2x = sp.lines[l][2], p2y = sp.lines[l][3];
                double dx = p2x - p1x, dy = p2y - p1y;
                double norm = sqrt(dx * dx + dy * dy);
                double tx = dx / norm, ty = dy / norm;
                double drx = x - p1x, dry = y - p1y;
                double dt_ = drx * tx + dry * ty;
                if (dt_ > 0) {
                    if (dt_ < norm) { drx = x - (p1x + tx * dt_); dry = y - (p1y + ty * dt_); }
                    else { drx = x - p2x; dry = y - p2y; }
                }
                double dist = sqrt(drx * drx + dry * dry);
                wall_pot_force(sp, drx, dry, proc_dist(sp.pot_mode, dist, 1.0), fx, fy);
            }
        }
    }
}

static __device__ __forceinline__ void apply_walls(const Ctx& C, int32_t rep, const DevRep& R, double radius, double& x, double& y,
                            double& vx, double& vy, bool has_vel) {
    const MaviSpace* sps = C.spaces + (int64_t)rep * MAVI_MAX_SPACES;
    for (int k = 0; k < R.num_spaces; k++) {
        const MaviSpace& sp = sps[k];
        if (sp.wall == MAVI_WALL_RIGID && sp.geometry == MAVI_GEOM_RECTANGLE) {
            if (!has_vel) continue;
            double rx = x - sp.bl_x, ry = y - sp.bl_y;
            bool ox = (rx + radius) > sp.length || (rx - radius) < 0;
            bool oy = (ry + radius) > sp.height || (ry - radius) < 0;
            if (ox) vx = -vx;
            if (oy) vy = -vy;
        } else if (sp.wall == MAVI_WALL_RIGID && sp.geometry == MAVI_GEOM_CIRCLE) {
            if (!has_vel) continue;
            double rr = sp.radius - radius;
            double max_r2 = rr * rr;
            double dx = x - sp.cx, dy = y - sp.cy;
            double d2x = __dmul_rn(dx, dx), d2y = __dmul_rn(dy, dy);
            double r2 = __dadd_rn(d2x, d2y);
            if (r2 <= max_r2) continue;
            double df = __dsub_rn(d2y, d2x);
            double cxy = __dmul_rn(__dmul_rn(2.0, x), y);
            double nvx = __ddiv_rn(__dsub_rn(__dmul_rn(vx, df), __dmul_rn(cxy, vy)), r2);
            double nvy = __ddiv_rn(__dsub_rn(__dmul_rn(-vy, df), __dmul_rn(cxy, vx)), r2);
            vx = nvx;
            vy = nvy;
        } else if (sp.wall == MAVI_WALL_PERIODIC && sp.geometry == MAVI_GEOM_RECTANGLE) {
            double hx = sp.length / 2, hy = sp.height / 2;
            double cx = sp.bl_x + hx, cy = sp.bl_y + hy;
            double dx = x - cx, dy = y - cy;
            if (fabs(dx) > hx) x = __dsub_rn(x, jsign(dx) * (hx * 2));
            if (fabs(dy) > hy) y = __dsub_rn(y, jsign(dy) * (hy * 2));
        } else if (sp.wall == MAVI_WALL_SLIPPERY && sp.geometry == MAVI_GEOM_LINES) {
            double px0 = x, py0 = y;
            for (int l = 0; l < sp.num_lines; l++) {
                double p1x = sp.lines[l][0], p1y = sp.lines[l][1], p2x = sp.lines[l][2], p2y = sp.lines[l][3];
                double dx = p2x - p1x, dy = p2y - p1y;
                double norm = sqrt(dx * dx + dy * dy);
                double nx = -dy / norm, ny = dx / norm, tx = dx / norm, ty = dy / norm;
                double drx = px0 - p1x, dry = py0 - p1y;
                double ds = drx * nx + dry * ny;
                if (fabs(ds) > radius) continue;
                double dtt = drx * tx + dry * ty;
                bool corner = false;
                double cpx = p1x, cpy = p1y;
                if (dtt > 0) {
                    if (dtt > norm) {
                        if (dtt > norm + radius) continue;
                        corner = true; cpx = p2x; cpy = p2y;
                    }
                } else if (dtt > -radius) {
                    corner = true;
                } else {
                    continue;
                }
                if (corner) {
                    double ex = px0 - cpx, ey = py0 - cpy;
                    double nn = sqrt(ex * ex + ey * ey);
                    if (nn > radius) continue;
                    double alpha = radius / nn - 1;
                    x += alpha * ex;
                    y += alpha * ey;
                } else {
                    double sgn = jsign(ds);
                    double alpha = sgn * (radius - sgn * ds);
                    x += alpha * nx;
                    y += alpha * ny;
                }
            }
        } else if (sp.wall == MAVI_WALL_SLIPPERY && sp.geometry == MAVI_GEOM_CIRCLE) {
            double rr = sp.radius + radius;
            double dx = x - sp.cx, dy = y - sp.cy;
            if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
            double d2 = dx * dx + dy * dy;
            if (d2 > rr * rr) continue;
            double dn = sqrt(d2);
            double kk = sp.radius + radius - dn;
            x = x + kk * dx / dn;
            y = y + kk * dy / dn;
        }
    }
}

// ===========================================================================
// fused pair-force passes
// ===========================================================================
constexpr int kPassForce = 0;      // forces only (calc_forces! + optional walls), rings pair pass
constexpr int kPassVerlet1 = 1;    // F(t), x(t+dt) = x + v dt + F dt^2/2
constexpr int kPassVerlet2 = 2;    // F(t+dt) on stale chunks, v update, walls!, histogram
constexpr int kPassOverdamped = 3; // x += mobility F dt, walls!, histogram
constexpr int kPassSzabo = 4;      // update_szabo!, walls!, histogram
constexpr int kPassRTP = 5;        // update_rtp!, walls!, histogram

// walls! then the chunk of the final position. When every wall acts on the
// bounding rectangle only, a particle whose pre-wall chunk is interior cannot
// be touched by a wall, so the walls run for edge-chunk particles only.
template <int PREC>
__device__ __forceinline__ int64_t walls_and_bin(const Ctx& C, int32_t rep, const DevRep& R, int64_t s,
                                                int32_t cell, double& x, double& y, double& vx, double& vy,
                                                bool has_vel) {
    int64_t fast = bin_fast<PREC>(C, R, s, x, y, cell);
    if (fast >= 0) {
        if (!R.has_walls) return fast;
        if (R.walls_edge_only) {
            int32_t lc = (int32_t)(cell - R.c0);
            int32_t col = lc / R.rows, row = lc - col * R.rows;
            if (!edge_chunk(R, row, col)) return fast;   // no bounding-box wall can act
        }
    }
    if (R.has_walls) apply_walls(C, rep, R, R.radius, x, y, vx, vy, has_vel);
    return bin_final<PREC>(C, R, s, x, y, cell);
}

// The end of a pair pass for one particle, after its pair force is summed:
// wall forces, then per pass the force output or the integration (Verlet
// halves, overdamped, Szabo, RTP), walls! and the Julia-exact binning of the
// new position. fx, fy: the pair force in FP64; gx, gy: the mixed form's FP32
// sums (fx, fy widened); nb: rings neighbour count. Returns the new chunk (or
// 0) and sets cap for the histogram.
template <int PREC, int DYN, int PASS, bool HAS_VEL, bool HAS_POL>
__device__ __forceinline__ int64_t pass_epilogue(const Ctx& C, int64_t s, int32_t rep, const DevRep& R, int32_t cell,
                                                 double2 p, double fx, double fy, float gx, float gy, int32_t nb,
                                                 int32_t with_wall_forces, int32_t& cap) {
    (void)gx; (void)gy; (void)nb;
    int64_t new_cell = 0;
    bool walls_f = (PASS != kPassVerlet2) && with_wall_forces && R.has_wall_forces;
    if (walls_f) add_wall_forces(C, rep, R, p.x, p.y, fx, fy);
    const double dt = R.dt;
    if constexpr (PASS == kPassForce && DYN == MAVI_DYN_RINGS) {
        // rings: the force in user order, where k_rings reads a ring's particles together
        const int32_t u = C.uid_cur[s];
        if constexpr (PREC == kPrecFP64) C.fd_u[u] = make_double2(fx, fy);
        else C.ff_u[u] = make_float2(gx, gy);
        if (C.nb_mode) C.nb_count[u] = nb;
    } else if constexpr (PASS == kPassForce) {
        if constexpr (PREC == kPrecFP64) C.fd[s] = make_double2(fx, fy);
        else if (walls_f) C.ff[s] = make_float2((float)fx, (float)fy);
        else C.ff[s] = make_float2(gx, gy);
    } else if constexpr (PASS == kPassVerlet1) {
        // update_verlet! (src/integration.jl:415-431), first half
        double2 v = C.vel_cur[s];
        double term = dt * dt / 2;
        double nx = __dadd_rn(p.x, __dadd_rn(__dmul_rn(v.x, dt), __dmul_rn(fx, term)));
        double ny = __dadd_rn(p.y, __dadd_rn(__dmul_rn(v.y, dt), __dmul_rn(fy, term)));
        C.pos_mid[s] = make_double2(nx, ny);
        if constexpr (PREC == kPrecFP64) C.fold_d[s] = make_double2(fx, fy);
        else {
            C.fold_f[s] = make_float2((float)fx, (float)fy);
            // offsets of x(t+dt) from the (stale) chunk of this step
            int32_t lc = (int32_t)(cell - R.c0);
            int64_t col = lc / R.rows, row = lc - col * R.rows;
            double tx = __dsub_rn(nx, R.bb_blx), ty = __dadd_rn(__dadd_rn(-ny, R.bb_bly), R.bb_h);
            C.off_mid[s] = fixed_offset(R, row, col, tx, ty, C.err, s);
        }
    } else {
        double x = p.x, y = p.y, vx = 0, vy = 0;
        if constexpr (HAS_VEL) { double2 v = C.vel_cur[s]; vx = v.x; vy = v.y; }
        if constexpr (PASS == kPassVerlet2) {
            double ox, oy;
            if constexpr (PREC == kPrecFP64) { double2 o = C.fold_d[s]; ox = o.x; oy = o.y; }
            else { float2 o = C.fold_f[s]; ox = o.x; oy = o.y; }
            double h = dt / 2;
            vx = __dadd_rn(vx, __dmul_rn(h, __dadd_rn(fx, ox)));
            vy = __dadd_rn(vy, __dmul_rn(h, __dadd_rn(fy, oy)));
        } else if constexpr (PASS == kPassOverdamped) {
            if constexpr (PREC == kPrecFP64) {
                x = __dadd_rn(x, __dmul_rn(fx, R.mdt));
                y = __dadd_rn(y, __dmul_rn(fy, R.mdt));
            } else {
                // FP32 displacement (relative error 6e-8 of a step), FP64 position
                x = __dadd_rn(x, f32_to_f64_bits(gx * R.mdt_f));
                y = __dadd_rn(y, f32_to_f64_bits(gy * R.mdt_f));
            }
        } else if constexpr (PASS == kPassSzabo || PASS == kPassRTP) {
            int32_t uid = C.uid_cur[s];
            double theta = C.pol_cur[s];
            double c_, s_;
            sincos(theta, &s_, &c_);
            int64_t step = C.d_step[0] - 1;
            if constexpr (PASS == kPassSzabo) {
                // update_szabo! (src/integration.jl:433-465)
                double wx = __dadd_rn(__dmul_rn(R.vo, c_), __dmul_rn(R.mobility, fx));
                double wy = __dadd_rn(__dmul_rn(R.vo, s_), __dmul_rn(R.mobility, fy));
                double speed = sqrt(fabs(wx) + fabs(wy));
                double cr = speed > 0 ? __ddiv_rn(__dsub_rn(__dmul_rn(c_, wy), __dmul_rn(s_, wx)), speed) : 0.0;
                if (fabs(cr) > 1) cr = jsign(cr);
                double nz;
                if (C.noise_mode == MAVI_NOISE_INJECTED) nz = C.noise[R.noise0 + (uid - R.slot0)];
                else nz = philox_normal(C.seed, (uint64_t)uid, (uint64_t)step);
                double d_theta = 1 / R.relax_time * asin(cr) * dt + sqrt(2 * R.rot_diff * dt) * nz;
                x = __dadd_rn(x, __dmul_rn(wx, dt));
                y = __dadd_rn(y, __dmul_rn(wy, dt));
                theta = theta + d_theta;
            } else {
                // update_rtp! (src/integration.jl:467-498)
                double wx = __dadd_rn(__dmul_rn(R.vo, c_), fx);
                double wy = __dadd_rn(__dmul_rn(R.vo, s_), fy);
                x = __dadd_rn(x, __dmul_rn(wx, dt));
                y = __dadd_rn(y, __dmul_rn(wy, dt));
                double u1, u2;
                if (C.noise_mode == MAVI_NOISE_INJECTED) {
                    int64_t o = R.noise0 + 2 * (int64_t)(uid - R.slot0);
                    u1 = C.noise[o];
                    u2 = C.noise[o + 1];
                } else {
                    Rand2 r2 = philox_uniform2(C.seed, (uint64_t)uid, (uint64_t)step);
                    u1 = r2.a;
                    u2 = r2.b;
                }
                if (u1 < R.tumble_rate * dt) theta = 2 * 3.141592653589793 * u2;
            }
            C.pol_out[s] = theta;
        }
        new_cell = walls_and_bin<PREC>(C, rep, R, s, cell, x, y, vx, vy, HAS_VEL);
        C.pos_out[s] = make_double2(x, y);
        if constexpr (HAS_VEL) C.vel_out[s] = make_double2(vx, vy);
        if constexpr (HAS_POL && !(PASS == kPassSzabo || PASS == kPassRTP)) C.pol_out[s] = C.pol_cur[s];
        C.uid_out[s] = C.uid_cur[s];
        if (C.num_reps > 1) C.rep_out[s] = rep;
        cap = R.has_chunks ? R.cap : (1 << 30);
    }
    return new_cell;
}

#ifndef MAVI_PASS_BLOCKS_MIXED
#define MAVI_PASS_BLOCKS_MIXED 8   // resident pair-pass blocks per SM, mixed form (64 registers)
#endif
#ifndef MAVI_PASS_BLOCKS_FP64
#define MAVI_PASS_BLOCKS_FP64 4    // FP64 form (128 registers)
#endif
#ifndef MAVI_PASS_BLOCKS_RINGS
#define MAVI_PASS_BLOCKS_RINGS 8   // mixed-form rings pair pass
#endif
#ifndef MAVI_PASS_BLOCKS_LJ
#define MAVI_PASS_BLOCKS_LJ 8      // mixed-form Lennard-Jones / WCA passes (double-float pair term)
#endif
template <int PREC, int DYN, int PASS, bool HAS_VEL, bool HAS_POL>
__global__ void __launch_bounds__(kPassThreads,
                                  PREC == kPrecFP64 ? MAVI_PASS_BLOCKS_FP64
                                  : DYN == MAVI_DYN_RINGS ? MAVI_PASS_BLOCKS_RINGS
                                  : (DYN == MAVI_DYN_LEN_JONES || DYN == MAVI_DYN_RUN_TUMBLE) ? MAVI_PASS_BLOCKS_LJ
                                  : MAVI_PASS_BLOCKS_MIXED)
k_pass(Ctx C, int32_t with_wall_forces) {
    __shared__ Stage<PREC, DYN> stage[kPassWarps];
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = s < C.M;
    int64_t new_cell = 0;
    int32_t cap = 1 << 30;
    // one replica: no load in the way of the descriptor (its fields load in
    // parallel with the particle's own state)
    int32_t rep = (valid && C.num_reps > 1) ? C.rep_cur[s] : 0;
    const DevRep& R = C.reps[rep];
    int32_t cell = valid ? C.cell_cur[s] : 0;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        // particles of inactive rings (parked after every real chunk): zero
        // force (clean_forces!), no neighbours, no pair terms
        if (valid && C.var_rings && cell == C.park) {
            if constexpr (PASS == kPassForce) {
                const int32_t u = C.uid_cur[s];
                if constexpr (PREC == kPrecFP64) C.fd_u[u] = make_double2(0.0, 0.0);
                else C.ff_u[u] = make_float2(0.f, 0.f);
                if (C.nb_mode) C.nb_count[u] = 0;
            }
            valid = false;
        }
    }
    const double2* P = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
    // own FP64 position, loaded early so its latency overlaps the gather
    const double2 p = valid ? P[s] : make_double2(0.0, 0.0);
    Acc<PREC, DYN> acc;
    if constexpr (PREC == kPrecFP64) {
        gather_warp<PREC, DYN>(C, valid, s, rep, R, cell, P, stage[threadIdx.x >> 5], acc);
    } else {
        gather_warp<PREC, DYN>(C, valid, s, rep, R, cell, (PASS == kPassVerlet2) ? C.off_mid : C.off_cur,
                               stage[threadIdx.x >> 5], acc);
    }
    if (valid) {
        // FP32 sums widen on the integer pipes (f32_to_f64_bits), not the FP64 one
        double fx, fy;
        float gx = 0.f, gy = 0.f;
        if constexpr (PREC == kPrecFP64) { fx = acc.gx(); fy = acc.gy(); }
        else { gx = acc.gx(); gy = acc.gy(); fx = f32_to_f64_bits(gx); fy = f32_to_f64_bits(gy); }
        new_cell = pass_epilogue<PREC, DYN, PASS, HAS_VEL, HAS_POL>(C, s, rep, R, cell, p, fx, fy, gx, gy, acc.nb,
                                                                  with_wall_forces, cap);
    }
    if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped || PASS == kPassSzabo || PASS == kPassRTP)
        count_into_chunk(C, valid, s, new_cell, cap);
}

// The mixed short-range passes with the column gather (pass mode 2, COLS) or
// the per-chunk gather (pass mode 1): k_pass with that gather called directly
// in place of the warp gathers (the same terms in the same order, so the same
// bits), in a kernel of its own so that its registers serve this gather alone
// (the warp-staged gather's registers made k_pass spill in these loops).
template <int DYN, int PASS, bool HAS_VEL, bool HAS_POL, bool COLS>
__global__ void __launch_bounds__(kPassThreads, DYN == MAVI_DYN_RINGS ? MAVI_PASS_BLOCKS_RINGS : MAVI_PASS_BLOCKS_MIXED)
k_pass_cols(Ctx C, int32_t with_wall_forces) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = s < C.M;
    const int32_t rep = (valid && C.num_reps > 1) ? C.rep_cur[s] : 0;
    const DevRep& R = C.reps[rep];
    const int32_t cell = valid ? C.cell_cur[s] : 0;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        // particles of inactive rings (parked after every real chunk): zero
        // force (clean_forces!), no neighbours, no pair terms
        if (valid && C.var_rings && cell == C.park) {
            const int32_t u = C.uid_cur[s];
            C.ff_u[u] = make_float2(0.f, 0.f);
            if (C.nb_mode) C.nb_count[u] = 0;
            valid = false;
        }
    }
    const int2* P = (PASS == kPassVerlet2) ? C.off_mid : C.off_cur;
    const double2* Pd = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
    const double2 p = valid ? Pd[s] : make_double2(0.0, 0.0);
    int64_t new_cell = 0;
    int32_t cap = 1 << 30;
    if (valid) {
        Acc<kPrecMixed, DYN> acc;
        const Me<kPrecMixed, DYN> me = make_me<kPrecMixed, DYN>(C, R, rep, s, P);
        if (COLS && R.has_chunks) gather_columns<kPrecMixed, DYN>(C, R, rep, s, cell, P, me, acc);
        else gather_global<kPrecMixed, DYN>(C, R, rep, s, cell, P, me, acc);
        const float gx = acc.gx(), gy = acc.gy();
        new_cell = pass_epilogue<kPrecMixed, DYN, PASS, HAS_VEL, HAS_POL>(
            C, s, rep, R, cell, p, f32_to_f64_bits(gx), f32_to_f64_bits(gy), gx, gy, acc.nb, with_wall_forces, cap);
    }
    if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped || PASS == kPassSzabo || PASS == kPassRTP)
        count_into_chunk(C, valid, s, new_cell, cap);
}

template <int DYN, int PASS>
constexpr bool kColsPass = (DYN == MAVI_DYN_HARM_TRUNC && (PASS == kPassForce || PASS == kPassOverdamped ||
                                                          PASS == kPassVerlet1 || PASS == kPassVerlet2)) ||
                           (DYN == MAVI_DYN_SZABO && (PASS == kPassForce || PASS == kPassSzabo)) ||
                           (DYN == MAVI_DYN_RINGS && PASS == kPassForce);

// The mixed Lennard-Jones pass with the split gather (pass mode 7): k_pass
// with gather_split in place of the warp gathers, in a kernel of its own so
// that its registers serve this gather alone.
#ifndef MAVI_PASS_BLOCKS_SPLIT
#define MAVI_PASS_BLOCKS_SPLIT 10   // measured faster than 8 or 12 (start and melted states)
#endif
template <int PASS, bool HAS_VEL, bool HAS_POL>
__global__ void __launch_bounds__(kPassThreads, MAVI_PASS_BLOCKS_SPLIT) k_pass_split(Ctx C, int32_t with_wall_forces) {
    constexpr int DYN = MAVI_DYN_LEN_JONES;
    __shared__ int2 slots[kSplitSlots * kPassThreads];
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = s < C.M;
    const int32_t rep = (valid && C.num_reps > 1) ? C.rep_cur[s] : 0;
    const DevRep& R = C.reps[rep];
    const int32_t cell = valid ? C.cell_cur[s] : 0;
    const int2* P = (PASS == kPassVerlet2) ? C.off_mid : C.off_cur;
    const double2* Pd = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
    const double2 p = valid ? Pd[s] : make_double2(0.0, 0.0);
    int64_t new_cell = 0;
    int32_t cap = 1 << 30;
    if (valid) {
        Acc<kPrecMixed, DYN> acc;
        const Me<kPrecMixed, DYN> me = make_me<kPrecMixed, DYN>(C, R, rep, s, P);
        gather_split<DYN>(C, R, rep, s, cell, P, me, acc, slots + threadIdx.x);
        const float gx = acc.gx(), gy = acc.gy();
        new_cell = pass_epilogue<kPrecMixed, DYN, PASS, HAS_VEL, HAS_POL>(
            C, s, rep, R, cell, p, f32_to_f64_bits(gx), f32_to_f64_bits(gy), gx, gy, 0, with_wall_forces, cap);
    }
    if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped) count_into_chunk(C, valid, s, new_cell, cap);
}

// ===========================================================================
// Several lanes per particle (mixed form, short-range laws). On sparse grids
// (about one particle per chunk) a particle has only ~8 candidates, and one
// lane per particle leaves the pass waiting on three dependent loads (chunk,
// chunk bounds, neighbour offsets) with few pair terms to hide them. Here
// LANES consecutive lanes share a particle: lane l takes the candidates
// l, l + LANES, ... of the column gather's flat loop, and the partial sums are
// combined by an xor butterfly (every lane ends with the same sum, formed in
// the same order each run: deterministic). Lane 0 runs the epilogue.
// ===========================================================================
template <int DYN, int PASS>
constexpr bool kLanesPass = (DYN == MAVI_DYN_HARM_TRUNC && (PASS == kPassForce || PASS == kPassOverdamped)) ||
                            (DYN == MAVI_DYN_SZABO && (PASS == kPassForce || PASS == kPassSzabo));

template <int DYN, int PASS, bool HAS_VEL, bool HAS_POL, int LANES>
__global__ void __launch_bounds__(kPassThreads, MAVI_PASS_BLOCKS_MIXED) k_pass_lanes(Ctx C, int32_t with_wall_forces) {
    static_assert(LANES == 2 || LANES == 4, "2 or 4 lanes per particle");
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s = gt / LANES;
    const int l = (int)(gt & (LANES - 1));
    const bool valid = s < C.M;
    const int32_t rep = (valid && C.num_reps > 1) ? C.rep_cur[s] : 0;
    const DevRep& R = C.reps[rep];
    const int32_t cell = valid ? C.cell_cur[s] : 0;
    const int2* P = (PASS == kPassVerlet2) ? C.off_mid : C.off_cur;
    const double2* Pd = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
    const double2 p = (valid && l == 0) ? Pd[s] : make_double2(0.0, 0.0);
    Acc<kPrecMixed, DYN> acc;
    if (valid) {
        const Me<kPrecMixed, DYN> me = make_me<kPrecMixed, DYN>(C, R, rep, s, P);
        if (R.has_chunks) gather_columns<kPrecMixed, DYN>(C, R, rep, s, cell, P, me, acc, l, LANES);
        else if (l == 0) gather_global<kPrecMixed, DYN>(C, R, rep, s, cell, P, me, acc);
    }
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    const bool lead = valid && l == 0;
    int64_t new_cell = 0;
    int32_t cap = 1 << 30;
    if (lead) {
        const float gx = acc.gx(), gy = acc.gy();
        new_cell = pass_epilogue<kPrecMixed, DYN, PASS, HAS_VEL, HAS_POL>(
            C, s, rep, R, cell, p, f32_to_f64_bits(gx), f32_to_f64_bits(gy), gx, gy, 0, with_wall_forces, cap);
    }
    if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped || PASS == kPassSzabo || PASS == kPassRTP)
        count_into_chunk(C, lead, s, new_cell, cap);
}

// ===========================================================================
// Tiled pair pass with Newton's third law (mixed form, Lennard-Jones / WCA).
//
// The reference evaluates each unordered candidate pair once and adds the
// force to both particles (F[i] += f; F[j] -= f, src/integration.jl:131-132,
// 150-151). Here a CTA owns a tile of whole chunks (w x h chunks of one
// replica; chunk grids are static, so tiles are fixed at creation) and stages
// the fixed-point offsets of the tile and of a one-chunk halo ring (the
// "window") in shared memory, one thread per window chunk. Then every window
// particle gets a thread:
//  * an owned particle evaluates its pairs with owned particles later in the
//    window order (its own chunk and the neighbouring owned chunks), adds the
//    term to its own sum and subtracts it from the partner's;
//  * a halo particle evaluates its pairs with the owned particles next to it
//    and adds each term to the owned partner only (the halo particle's own
//    tile evaluates the same pair for it).
// So every pair with an owned particle is evaluated once per tile, the halo
// work is spread over the halo particles' threads instead of loading the
// tile's edge particles, and each thread runs one flat loop over its
// candidates. Sums are fixed point in shared memory (fix_term): integer
// atomics make them independent of the thread schedule, bit for bit. After a
// barrier the owned particles run the pass's epilogue (integration, walls!,
// binning, histogram).
//
// Tiles are handed to CTAs one per CTA (a grid of tiles) or through a device
// work queue: a persistent grid of CTAs takes the next tile with an atomic
// ticket until the tiles run out, and the last CTA to finish resets the queue
// for the next launch. A tile whose window exceeds the shared-memory arrays
// falls back to per-particle gathers for its owned particles.
// ===========================================================================
struct TileDesc {
    int32_t rep, c0, r0, wh;   // replica, first column and row, w | (h << 8)
};
constexpr int kTileThreads = 256;
constexpr int kTileMaxDim = 12;                       // tile side, chunks
constexpr int kTileWin = kTileMaxDim + 2;             // window side, chunks
constexpr int kTileWinChunks = kTileWin * kTileWin;   // 196 <= kTileThreads
constexpr int kTileMaxWinParts = 1024;                // staged window particles
constexpr int kTileMaxOwn = 640;                      // owned particles with shared sums
#ifndef MAVI_TILE_BLOCKS
#define MAVI_TILE_BLOCKS 4                            // resident tile CTAs per SM (64 registers)
#endif

// The passes that run tiled (Lennard-Jones: forces and both velocity-Verlet
// halves; WCA: forces and the run-and-tumble update); other combinations use
// the per-particle gathers.
template <int DYN, int PASS>
constexpr bool kTiledPass = (DYN == MAVI_DYN_LEN_JONES && (PASS == kPassForce || PASS == kPassVerlet1 ||
                                                          PASS == kPassVerlet2)) ||
                            (DYN == MAVI_DYN_RUN_TUMBLE && (PASS == kPassForce || PASS == kPassRTP));

struct TileSmem {
    int2 off[kTileMaxWinParts];             // fixed-point offsets of the window particles
    unsigned long long acc[2][kTileMaxOwn]; // fixed-point force sums of the owned particles
    int32_t cb[kTileWinChunks];             // window chunk -> first window index
    int32_t ce[kTileWinChunks];             // one past its last
    int32_t gs[kTileWinChunks];             // first global slot of the window chunk
    uint8_t wq[kTileMaxWinParts];           // window chunk of each window particle
    int32_t own0[kTileMaxDim + 1];          // first owned index of each tile column
    int32_t nwin, nown, tile;
    int scan[32];
};

// The fixed-point force on the particle with offset a from the one with
// offset b; (shx, shy): the centre of b's chunk relative to a's, exact units.
// Returns false when the pair lies outside the WCA cutoff.
template <int DYN>
__device__ __forceinline__ bool tile_term(const DevRep& R, const FixPair& fp0, int2 a, int2 b, int32_t shx,
                                          int32_t shy, bool mi, long long& tx, long long& ty, bool& bad) {
    int32_t dxi = (int32_t)((uint32_t)a.x - (uint32_t)b.x + (uint32_t)shx);
    int32_t dyi = (int32_t)((uint32_t)a.y - (uint32_t)b.y + (uint32_t)shy);
    if (mi) {
        if (abs(dxi) > R.half_bx_i) dxi -= dxi > 0 ? R.bx_i : -R.bx_i;
        if (abs(dyi) > R.half_by_i) dyi -= dyi > 0 ? R.by_i : -R.by_i;
    }
    if constexpr (DYN == MAVI_DYN_RUN_TUMBLE) {
        if (!inside_cutoff(fp0, dxi, dyi)) return false;
    }
    float fxh, fxl, fyh, fyl;
    lj_pair_df(R, dxi, dyi, fxh, fxl, fyh, fyl);
    tx = fix_term(fxh, fxl, bad);
    ty = fix_term(fyh, fyl, bad);
    return true;
}

template <int DYN, int PASS, bool HAS_VEL, bool HAS_POL>
__global__ void __launch_bounds__(kTileThreads, MAVI_TILE_BLOCKS)
k_tpass(Ctx C, int32_t with_wall_forces, const TileDesc* __restrict__ tiles, int32_t ntiles,
        int32_t* __restrict__ queue, int32_t persistent) {
    __shared__ TileSmem sm;
    const int2* Po = (PASS == kPassVerlet2) ? C.off_mid : C.off_cur;
    const double2* Pd = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
    const int tid = threadIdx.x;
    int32_t t = blockIdx.x;
    for (;;) {
        if (persistent) {
            __syncthreads();   // the previous tile is done with the shared arrays
            if (tid == 0) sm.tile = atomicAdd(&queue[0], 1);
            __syncthreads();
            t = sm.tile;
        }
        if (t >= ntiles) break;
        const TileDesc td = tiles[t];
        const int32_t rep = td.rep;
        const DevRep& R = C.reps[rep];
        const int w = td.wh & 0xff, h = td.wh >> 8;
        const int H = h + 2, nq = (w + 2) * H;
        // 1. window chunks, column-major: q = k * H + qq is column c0 - 1 + k, row r0 - 1 + qq
        int32_t cnt = 0;
        if (tid < nq) {
            const int k = tid / H, qq = tid - k * H;
            int gc = td.c0 - 1 + k, gr = td.r0 - 1 + qq;
            bool inside = true;
            if (R.periodic) {
                gc = gc < 0 ? gc + R.cols : (gc >= R.cols ? gc - R.cols : gc);
                gr = gr < 0 ? gr + R.rows : (gr >= R.rows ? gr - R.rows : gr);
            } else {
                inside = gc >= 0 && gc < R.cols && gr >= 0 && gr < R.rows;
            }
            int32_t b = 0;
            if (inside) {
                const int64_t ch = R.c0 + (int64_t)gc * R.rows + gr;
                b = C.start[ch];
                cnt = C.start[ch + 1] - b;
            }
            sm.gs[tid] = b;
        }
        int total;
        const int ex = block_exclusive_scan(cnt, sm.scan, total);   // nq <= 196 <= blockDim
        if (tid < nq) { sm.cb[tid] = ex; sm.ce[tid] = ex + cnt; }
        if (tid == 0) sm.nwin = total;
        __syncthreads();
        if (tid <= w) {
            // owned particles: window columns 1..w, rows 1..h, contiguous per column
            int32_t o = 0;
            for (int k = 1; k <= tid; k++) o += sm.ce[k * H + h] - sm.cb[k * H + 1];
            sm.own0[tid] = o;
            if (tid == w) sm.nown = o;
        }
        __syncthreads();
        const int32_t nwin = sm.nwin, nown = sm.nown;
        const bool staged = nwin <= kTileMaxWinParts && nown <= kTileMaxOwn;
        if (staged) {
            if (tid < nq) {   // a thread per window chunk: its particles are consecutive slots
                const int32_t b = sm.cb[tid], e = sm.ce[tid], g0 = sm.gs[tid] - b;
                for (int32_t i = b; i < e; i++) {
                    sm.off[i] = Po[g0 + i];
                    sm.wq[i] = (uint8_t)tid;
                }
            }
            for (int32_t i = tid; i < nown; i += kTileThreads) { sm.acc[0][i] = 0ull; sm.acc[1][i] = 0ull; }
        }
        __syncthreads();
        // 2. pair terms, a thread per window particle, one flat loop over its candidates
        if (staged) {
            const FixPair& fp0 = C.fix[(int64_t)rep * MAVI_MAX_TYPES * MAVI_MAX_TYPES];
            for (int32_t x = tid; x < nwin; x += kTileThreads) {
                const int q = sm.wq[x], k = q / H, qq = q - k * H;
                const bool own_x = k >= 1 && k <= w && qq >= 1 && qq <= h;
                // true grid position of x (a halo position may wrap)
                int gcol = td.c0 - 1 + k, grow = td.r0 - 1 + qq;
                bool xw = false;
                if (R.periodic) {
                    if (gcol < 0) { gcol += R.cols; xw = true; } else if (gcol >= R.cols) { gcol -= R.cols; xw = true; }
                    if (grow < 0) { grow += R.rows; xw = true; } else if (grow >= R.rows) { grow -= R.rows; xw = true; }
                }
                const bool raw = xw && !R.min_image;                 // periodic walls without minimum image
                const bool mi = R.min_image && (xw || R.mi_small);
                const int2 mx = sm.off[x];
                long long X = 0, Y = 0;
                bool bad = false;
                int r = 0, dk = 0, dq = 0;
                int32_t j = 0, e = 0, jown0 = 0;
                for (;;) {
                    while (j >= e && r < 9) {   // next owned neighbour chunk with candidates
                        dk = r / 3 - 1;
                        dq = r - 3 * (r / 3) - 1;
                        r++;
                        const int nk = k + dk, nqq = qq + dq;
                        if (nk < 1 || nk > w || nqq < 1 || nqq > h) continue;
                        const int wqn = nk * H + nqq;
                        j = own_x ? max(sm.cb[wqn], x + 1) : sm.cb[wqn];
                        e = sm.ce[wqn];
                        jown0 = sm.own0[nk - 1] - sm.cb[nk * H + 1];
                    }
                    if (j >= e) break;
                    const int2 mj = sm.off[j];
                    long long tx, ty;
                    if (own_x) {
                        // both owned (never through a wrap): x's term, and its negation for j
                        if (tile_term<DYN>(R, fp0, mx, mj, -dk * R.sx_i, dq * R.sy_i, R.min_image && R.mi_small, tx,
                                           ty, bad)) {
                            X += tx;
                            Y += ty;
                            atomicAdd(&sm.acc[0][jown0 + j], (unsigned long long)(-tx));
                            atomicAdd(&sm.acc[1][jown0 + j], (unsigned long long)(-ty));
                        }
                    } else {
                        // the owned j's term from the halo particle x
                        bool ok = true;
                        if (raw) {
                            const int jcol = td.c0 + k + dk - 1, jrow = td.r0 + qq + dq - 1;
                            const double dx = (double)((long long)mj.x - mx.x - (long long)(gcol - jcol) * R.sx_u) / R.inv_u;
                            const double dy = (double)((long long)mj.y - mx.y + (long long)(grow - jrow) * R.sy_u) / R.inv_u;
                            const double sc = pair_scalar<DYN, double>(R.pd, dx * dx + dy * dy);
                            tx = fix_term((float)(sc * dx), 0.f, bad);
                            ty = fix_term((float)(sc * dy), 0.f, bad);
                        } else {
                            ok = tile_term<DYN>(R, fp0, mj, mx, dk * R.sx_i, -dq * R.sy_i, mi, tx, ty, bad);
                        }
                        if (ok) {
                            atomicAdd(&sm.acc[0][jown0 + j], (unsigned long long)tx);
                            atomicAdd(&sm.acc[1][jown0 + j], (unsigned long long)ty);
                        }
                    }
                    j++;
                }
                if (own_x) {
                    const int32_t o = sm.own0[k - 1] + (x - sm.cb[k * H + 1]);
                    atomicAdd(&sm.acc[0][o], (unsigned long long)X);
                    atomicAdd(&sm.acc[1][o], (unsigned long long)Y);
                }
                if (bad) raise_error(C.err, MAVI_ERR_FORCE_RANGE, sm.gs[q] + (x - sm.cb[q]), 0);
            }
        }
        __syncthreads();
        // 3. epilogue per owned particle (a tile that was not staged gathers its pair sums here);
        // warp-uniform trip counts: the histogram needs whole warps
        for (int32_t base = 0; base < nown; base += kTileThreads) {
            const int32_t o = base + tid;
            const bool valid = o < nown;
            int64_t s = 0, new_cell = 0;
            int32_t cap = 1 << 30;
            if (valid) {
                int kc = 0;
                while (kc + 1 < w && sm.own0[kc + 1] <= o) kc++;
                s = sm.gs[(kc + 1) * H + 1] + (o - sm.own0[kc]);   // owned chunks of a column: consecutive slots
                const int32_t cell = C.cell_cur[s];
                float gx, gy;
                if (staged) {
                    gx = fix_value((long long)sm.acc[0][o]);
                    gy = fix_value((long long)sm.acc[1][o]);
                } else {
                    Acc<kPrecMixed, DYN> acc;
                    const Me<kPrecMixed, DYN> me = make_me<kPrecMixed, DYN>(C, R, rep, s, Po);
                    gather_global<kPrecMixed, DYN>(C, R, rep, s, cell, Po, me, acc);
                    gx = acc.gx();
                    gy = acc.gy();
                }
                new_cell = pass_epilogue<kPrecMixed, DYN, PASS, HAS_VEL, HAS_POL>(
                    C, s, rep, R, cell, Pd[s], f32_to_f64_bits(gx), f32_to_f64_bits(gy), gx, gy, 0, with_wall_forces,
                    cap);
            }
            if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped || PASS == kPassSzabo || PASS == kPassRTP)
                count_into_chunk(C, valid, s, new_cell, cap);
        }
        if (!persistent) break;
    }
    if (persistent && tid == 0) {
        // every CTA has drawn its last ticket before it counts itself done, so
        // the last one may reset the queue for the next launch
        __threadfence();
        if (atomicAdd(&queue[1], 1) == (int32_t)gridDim.x - 1) {
            queue[0] = 0;
            queue[1] = 0;
        }
    }
}

// ===========================================================================
// rings: one warp per ring. Bonded terms (springs src/rings/integration.jl:
// 79-97 & 205-223, area :103-195, bending), wall forces, the overdamped
// active update (:300-351), walls! and the histogram for the next step.
// Positions of the ring are staged in shared memory.
// ===========================================================================
constexpr int kRingMax = 256;     // particles per ring supported
constexpr int kRingWarps = 4;     // rings per block

// Sum of the ring's particle velocities (k_ring_pol divides by n).
template <class V>
__device__ __forceinline__ void ring_vc_store(const Ctx& C, int64_t g, int lane, int32_t do_update, V vcx, V vcy) {
    if (!do_update) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vcx += __shfl_xor_sync(0xffffffffu, vcx, o);
        vcy += __shfl_xor_sync(0xffffffffu, vcy, o);
    }
    if (lane == 0) {
        if constexpr (std::is_same<V, double>::value) C.ring_vc[g] = make_double2(vcx, vcy);
        else C.ring_vcf[g] = make_float2(vcx, vcy);
    }
}

#ifndef MAVI_RINGS_MIN_BLOCKS
#define MAVI_RINGS_MIN_BLOCKS 8    // ring-kernel blocks per SM (64 registers; measured faster than 4, 5 or 6)
#endif
#ifndef MAVI_RINGS_SMALL_BLOCKS
#define MAVI_RINGS_SMALL_BLOCKS 10 // the same for k_rings<mixed, SMALL> (48 registers; faster than 8, level with 12)
#endif
// SMALL (mixed form): every ring of the handle has at most 32 particles and
// no replica takes the minimum image, so every ring takes the exact integer
// path below; the general path is compiled out and its registers with it.
template <int PREC, bool SMALL = false>
__global__ void __launch_bounds__(32 * kRingWarps, SMALL ? MAVI_RINGS_SMALL_BLOCKS : MAVI_RINGS_MIN_BLOCKS)
k_rings(Ctx C, int64_t total_rings, int32_t do_update, int32_t with_walls) {
    static_assert(!SMALL || PREC == kPrecMixed, "the exact integer ring path is the mixed form's");
    constexpr int kRingSlots = SMALL ? 32 : kRingMax;
    __shared__ double2 sp_[kRingWarps][kRingSlots];
    __shared__ int32_t ss_[kRingWarps][kRingSlots];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t g = (int64_t)blockIdx.x * kRingWarps + w;
    if (g >= total_rings) return;   // whole warp exits together
    const int32_t rep = C.ring_rep[g];
    const DevRep& R = C.reps[rep];
    const MaviRingsCfg& rc = C.rcfg[rep];
    const int32_t rl = (int32_t)(g - R.ring0);
    const int t = C.ring_types[g] - 1;
    const int32_t n = rc.num_particles[t];
    if (C.var_rings && C.ring_active[g] == 0) {
        // inactive ring: positions carried over unchanged, no forces
        if (do_update) {
            for (int p = lane; p < n; p += 32) {
                const int32_t u = (int32_t)R.slot0 + rl * R.nmax + p;
                const int32_t s = C.slot_of[u];
                C.pos_out[s] = C.pos_u[u];
                C.uid_out[s] = u;
                C.rep_out[s] = rep;
            }
        }
        return;
    }
    // with sources and sinks the active set changes before the next chunk
    // update, so the histogram is taken afterwards (k_count)
    const bool fused_count = !C.var_rings;
    double2* P = sp_[w];
    int32_t* S = ss_[w];
    const int32_t u0 = (int32_t)R.slot0 + rl * R.nmax;   // user slot of particle 0 (contiguous ring)
    for (int p = lane; p < n; p += 32) {
        S[p] = C.slot_of[u0 + p];
        P[p] = C.pos_u[u0 + p];
    }
    __syncwarp();
    auto diff = [&](double2 a, double2 b) {
        double dx = a.x - b.x, dy = a.y - b.y;
        if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
        return make_double2(dx, dy);
    };
    // overdamped active update parameters; (cos, sin) of the polarisation
    // come from k_ring_pol (one thread per ring, not one warp)
    // the mixed form sums the ring's velocity and forms the position
    // increment in FP32 (FP64 only for x += increment); FP64 form: all double
    using V = typename std::conditional<PREC == kPrecFP64, double, float>::type;
    V pc = 0, ps = 0;
    if (do_update) {
        if constexpr (PREC == kPrecFP64) { const double2 cs = C.ring_cs[g]; pc = cs.x; ps = cs.y; }
        else { const float2 cs = C.ring_csf[g]; pc = cs.x; ps = cs.y; }
    }
    const double vo = rc.vo[t], mu = rc.mobility[t], dt = R.dt;
    V vcx = 0, vcy = 0;
    // pair + wall forces, then the overdamped active update of particle p
    // returns the chunk of the updated position (binning fused here: the
    // histogram of the next step is taken in this kernel)
    const int32_t cap = R.has_chunks ? R.cap : (1 << 30);
    auto finish = [&](int p, double2 xc, V fx, V fy, bool near_wall = true) -> int64_t {
        const int32_t s = S[p], u = u0 + p;
        if constexpr (PREC == kPrecFP64) { double2 f = C.fd_u[u]; fx += f.x; fy += f.y; }
        else { float2 f = C.ff_u[u]; fx += f.x; fy += f.y; }
        if (R.has_wall_forces && near_wall && with_walls) {
            double wx = 0.0, wy = 0.0;
            add_wall_forces(C, rep, R, xc.x, xc.y, wx, wy);
            fx += (V)wx;
            fy += (V)wy;
        }
        if (!do_update) {
            if constexpr (PREC == kPrecFP64) C.fd_u[u] = make_double2(fx, fy);
            else C.ff_u[u] = make_float2(fx, fy);
            return 0;
        }
        double x, y;
        if constexpr (PREC == kPrecFP64) {
            double vx = __dadd_rn(__dmul_rn(vo, pc), __dmul_rn(mu, fx));
            double vy = __dadd_rn(__dmul_rn(vo, ps), __dmul_rn(mu, fy));
            vcx += vx; vcy += vy;
            x = __dadd_rn(xc.x, __dmul_rn(vx, dt));
            y = __dadd_rn(xc.y, __dmul_rn(vy, dt));
        } else {
            const float vx = fmaf(R.ring_vo_f[t], pc, R.ring_mu_f[t] * fx);
            const float vy = fmaf(R.ring_vo_f[t], ps, R.ring_mu_f[t] * fy);
            vcx += vx; vcy += vy;
            x = __dadd_rn(xc.x, f32_to_f64_bits(vx * R.dt_f));
            y = __dadd_rn(xc.y, f32_to_f64_bits(vy * R.dt_f));
        }
        double dvx = 0, dvy = 0;
        if (R.has_walls) apply_walls(C, rep, R, rc.inter_dist_eq[t][t] * 0.5, x, y, dvx, dvy, false);
        int64_t nc = 0;
        if (fused_count) {
            const int32_t cur = C.cell_u[u];
            nc = bin_fast<PREC>(C, R, s, x, y, cur, u);
            if (nc < 0) nc = bin_final<PREC>(C, R, s, x, y, cur, u);
            C.pos_u[u] = make_double2(x, y);
            C.cell_u[u] = (int32_t)nc;
        }
        C.pos_out[s] = make_double2(x, y);
        C.uid_out[s] = u;
        C.rep_out[s] = rep;
        return nc;
    };
    if constexpr (PREC == kPrecMixed) {
        if (SMALL || (n <= 32 && !R.min_image)) {
            // Mixed form, rings of <= 32 particles without minimum image: the
            // ring geometry comes from the exact integer chunk offsets. Each
            // lane's absolute position in units from the centre of chunk
            // (0, 0) is col*sx + ox, -row*sy + oy (int64); bonds are exact
            // integers, the shoelace area of the unwrapped ring is summed
            // exactly in 128-bit integers (update_continuos_pos! + calc_area,
            // src/rings/integration.jl:103-138), and springs, area force and
            // bending run in FP32 on the bond vectors. FP64 is left to the
            // position update and the walls.
            const unsigned full = 0xffffffffu;
            const bool act = lane < n;
            const int p = act ? lane : 0;
            const int pp = p == n - 1 ? 0 : p + 1, pm = p == 0 ? n - 1 : p - 1;
            const int2 off = C.off_u[u0 + p];
            const int32_t lc = C.cell_u[u0 + p] - (int32_t)R.c0;
            const int32_t col = lc / R.rows, row = lc - col * R.rows;
            const long long X = (long long)col * R.sx_u + off.x;
            const long long Y = -(long long)row * R.sy_u + off.y;
            const long long bx = __shfl_sync(full, X, pp) - X;   // bond p: x_{p+1} - x_p (units)
            const long long by = __shfl_sync(full, Y, pp) - Y;
            // unwrapped position of p relative to particle 0: exclusive scan of the bonds
            long long ix = act ? bx : 0, iy = act ? by : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long tx = __shfl_up_sync(full, ix, o), ty = __shfl_up_sync(full, iy, o);
                if (lane >= o) { ix += tx; iy += ty; }
            }
            const long long ux = ix - (act ? bx : 0), uy = iy - (act ? by : 0);
            // shoelace term cross(u_p, u_{p+1}) = cross(u_p, b_p) for p = 0..n-2
            __int128 a2 = (act && p <= n - 2) ? (__int128)ux * by - (__int128)uy * bx : (__int128)0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long lo = (unsigned long long)a2;
                const long long hi = (long long)(a2 >> 64);
                const unsigned long long olo = __shfl_xor_sync(full, lo, o);
                const long long ohi = __shfl_xor_sync(full, hi, o);
                a2 += (__int128)(((unsigned __int128)(unsigned long long)ohi << 64) | olo);
            }
            // area force factor k_area (A - A0) from the exact integer 2A - 2A0 (units^2)
            const __int128 a0x2 = (__int128)(((unsigned __int128)(unsigned long long)R.ring_a0x2_hi[t] << 64) |
                                             R.ring_a0x2_lo[t]);
            const __int128 d2a = a2 - a0x2;
            const long long d2a_c = d2a > (__int128)INT64_MAX ? INT64_MAX
                                  : (d2a < (__int128)INT64_MIN ? INT64_MIN : (long long)d2a);
            const float fa = i64_to_f32(d2a_c) * R.ring_karea_f[t];
            const float uf = R.u_f;
            const float bxf = i64_to_f32(bx) * uf, byf = i64_to_f32(by) * uf;
            const float L = sqrtf(bxf * bxf + byf * byf);
            const float inv = 1.0f / L;
            const long long bmxi = __shfl_sync(full, bx, pm), bmyi = __shfl_sync(full, by, pm);   // bond p-1
            const float bmx = __shfl_sync(full, bxf, pm), bmy = __shfl_sync(full, byf, pm);
            const float invm = __shfl_sync(full, inv, pm);
            const float ks = R.ring_ks_f[t], ls = R.ring_ls_f[t], kbt = R.ring_kb_f[t];
            // Bond components below 2^31 units keep the squares and the cross
            // products of the exact integer bonds inside int64, so the two
            // quantities that cancel near equilibrium are formed exactly: L^2 - l^2
            // of each spring (L ~ l) and the cross product of consecutive bonds
            // (nearly parallel in a smooth ring).
            constexpr long long kLim = 1ll << 31;
            const bool small = bx > -kLim && bx < kLim && by > -kLim && by < kLim && R.ring_ls2_u[t] >= 0;
            const bool exact = __all_sync(full, small);
            // springs: bond p pulls p by s_p b_p, bond p-1 by -s_{p-1} b_{p-1}, with
            // s = k (L - l) / L = k (L^2 - l^2) / ((L + l) L). In a squeezed ring
            // the two terms are large and nearly cancel, so with exact bonds they
            // are formed in float-float and rounded to FP32 only after the sum.
            float fx, fy;
            if (exact) {
                const long long L2 = bx * bx + by * by;
                const FF Lu = ff_sqrt(ff_from_i64(L2));                                   // |b_p|, units
                const FF den = ff_mul(ff_add(Lu, FF{R.ring_lu_h[t], R.ring_lu_l[t]}), Lu);
                const FF sp = ff_div(ff_mul(FF{R.ring_ku_h[t], R.ring_ku_l[t]}, ff_from_i64(L2 - R.ring_ls2_u[t])), den);
                const FF sx = ff_mul(sp, ff_from_i64(bx)), sy = ff_mul(sp, ff_from_i64(by));   // length units
                const FF mx = FF{__shfl_sync(full, sx.h, pm), __shfl_sync(full, sx.l, pm)};
                const FF my = FF{__shfl_sync(full, sy.h, pm), __shfl_sync(full, sy.l, pm)};
                const FF gx = ff_add(sx, ff_neg(mx)), gy = ff_add(sy, ff_neg(my));
                fx = gx.h + gx.l;
                fy = gy.h + gy.l;
            } else {
                const float spf = ks * (L - ls) * inv;
                const float smf = __shfl_sync(full, spf, pm);
                fx = spf * bxf - smf * bmx;
                fy = spf * byf - smf * bmy;
            }
            // area force: dr = x_{p+1} - x_{p-1} = b_p + b_{p-1}
            const long long dbx = bx + bmxi, dby = by + bmyi;
            fx -= fa * (i64_to_f32(dby) * uf * 0.5f);
            fy -= fa * (-i64_to_f32(dbx) * uf * 0.5f);
            // bending, a = bond p-1, b = bond p, c = a.b / (|a||b|):
            //   dc/da = b_perp(a) / (|a||b|) = (a x b) (-a_y, a_x) / (|a|^3 |b|)
            //   dc/db = a_perp(b) / (|a||b|) = -(a x b) (-b_y, b_x) / (|a| |b|^3)
            // (the parts of each bond perpendicular to the other, with no
            // cancellation between nearly equal terms)
            const float iab = invm * inv;
            const float crf = exact ? i64_to_f32(bmxi * by - bmyi * bx) * R.u2_f : bmx * byf - bmy * bxf;
            const float q = crf * iab;
            const float dcax = -q * bmy * (invm * invm), dcay = q * bmx * (invm * invm);
            const float dcbx = q * byf * (inv * inv), dcby = -q * bxf * (inv * inv);
            const float nax = __shfl_sync(full, dcax, pp), nay = __shfl_sync(full, dcay, pp);
            const float pbx = __shfl_sync(full, dcbx, pm), pby = __shfl_sync(full, dcby, pm);
            if (kbt != 0.0f) {
                fx += kbt * (dcax - dcbx) - kbt * nax + kbt * pbx;
                fy += kbt * (dcay - dcby) - kbt * nay + kbt * pby;
            }
            // PotentialWalls circle: float test in units, then the wall force in
            // FP32 on the exact integer displacement (the FP64 one, with its
            // square root and divisions, was most of this kernel's FP64 work)
            bool near_wall = true;
            if (R.wall_precheck) {
                const long long wxl = X - R.wall_cx_u, wyl = Y - R.wall_cy_u;
                const float wx = i64_to_f32(wxl), wy = i64_to_f32(wyl);
                const float r2 = fmaf(wx, wx, wy * wy);
                near_wall = !(r2 < R.wall_lo2_u) && !(R.wall_precheck == 2 && r2 > R.wall_hi2_u);
                if (near_wall && act && with_walls) wall_circle_f32(R, wxl, wyl, wx, wy, fx, fy);
                near_wall = false;
            }
            int64_t nc = 0;
            if (act) nc = finish(p, P[p], fx, fy, near_wall);
            if (do_update && fused_count) count_into_chunk(C, act, S[p], nc, cap);
            ring_vc_store(C, g, lane, do_update, vcx, vcy);
            return;
        }
    }
    // FP64 form: the area of this step's positions in the reference's own
    // operation order (k_ring_area_ref ran before this kernel). Mixed form:
    // unwrapped coordinates relative to particle 0 (update_continuos_pos!):
    // u[p] = sum_{q<p} calc_diff(P[q+1], P[q]); area by the shoelace formula.
    double area2 = 0.0;
    double carry_x = 0.0, carry_y = 0.0;   // u of the first particle of this 32-block
    double prev_last_x = 0.0, prev_last_y = 0.0;
    for (int base = 0; PREC != kPrecFP64 && base < n; base += 32) {
        int p = base + lane;
        double bx = 0, by = 0;
        if (p >= 1 && p < n) { double2 d = diff(P[p], P[p - 1]); bx = d.x; by = d.y; }
        // inclusive scan of bond vectors inside the block of 32
        double ix = bx, iy = by;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double tx = __shfl_up_sync(0xffffffffu, ix, o), ty = __shfl_up_sync(0xffffffffu, iy, o);
            if (lane >= o) { ix += tx; iy += ty; }
        }
        double ux = carry_x + ix, uy = carry_y + iy;
        // shoelace term cross(u[p-1], u[p]) for p in [max(1,base), n)
        double upx = __shfl_up_sync(0xffffffffu, ux, 1), upy = __shfl_up_sync(0xffffffffu, uy, 1);
        if (lane == 0) { upx = prev_last_x; upy = prev_last_y; }
        if (p >= 1 && p < n) area2 += upx * uy - upy * ux;
        prev_last_x = __shfl_sync(0xffffffffu, ux, 31);
        prev_last_y = __shfl_sync(0xffffffffu, uy, 31);
        carry_x = prev_last_x;
        carry_y = prev_last_y;
    }
    // closing term cross(u[n-1], u[0]) vanishes since u[0] = 0
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) area2 += __shfl_xor_sync(0xffffffffu, area2, o);
    const double area = PREC == kPrecFP64 ? C.ring_area[g] : area2 / 2.0;
    const double k_s = rc.k_spring[t], l_s = rc.l_spring[t];
    const double fmod_area = rc.k_area[t] * (area - R.ring_a0sq[t]);
    const double kb = rc.k_bend[t];
    if (n <= 32) {
        // One particle per lane; neighbours' bond data by shuffles. Each bond
        // length and its inverse are formed once (one sqrt and one division
        // per particle), and the bending gradients use the inverse lengths.
        // The mixed form evaluates these ring-internal terms in FP32 on FP64
        // differences; the FP64 form in double.
        using T = typename std::conditional<PREC == kPrecFP64, double, float>::type;
        const unsigned full = 0xffffffffu;
        const bool act = lane < n;
        const int p = act ? lane : 0;
        const int pp = p == n - 1 ? 0 : p + 1, pm = p == 0 ? n - 1 : p - 1;
        const double2 xc = P[p], xp = P[pp], xm = P[pm];
        const double2 bd = diff(xp, xc);                       // bond p: x_{p+1} - x_p
        const T bx = (T)bd.x, by = (T)bd.y;
        const T L = sqrt(bx * bx + by * by);
        const T inv = T(1) / L;
        const T bmx = __shfl_sync(full, bx, pm), bmy = __shfl_sync(full, by, pm);   // bond p-1
        const T invm = __shfl_sync(full, inv, pm);
        T ks, ls, kbt;
        if constexpr (PREC == kPrecFP64) { ks = k_s; ls = l_s; kbt = kb; }
        else { ks = R.ring_ks_f[t]; ls = R.ring_ls_f[t]; kbt = R.ring_kb_f[t]; }
        // springs (p, p+1) and, by a shuffle, (p-1, p); the mixed form forms
        // L - l as (L^2 - l^2) / (L + l) with L^2 - l^2 in FP64, so it keeps its
        // relative accuracy near the rest length
        T sp;
        if constexpr (PREC == kPrecFP64) sp = ks * (L - ls) * inv;
        else sp = ks * (float)(fma(bd.x, bd.x, bd.y * bd.y) - R.ring_ls2_d[t]) / ((L + ls) * L);
        const T sm = __shfl_sync(full, sp, pm);
        T fx = sp * bx - sm * bmx;
        T fy = sp * by - sm * bmy;
        // area: F_p -= k_area (A - A0) * (dr.y, -dr.x)/2, dr = x_{p+1} - x_{p-1}
        {
            const double2 d = diff(xp, xm);
            const T fa = (T)fmod_area;
            if constexpr (PREC == kPrecFP64) {
                fx -= fa * (d.y / 2);
                fy -= fa * (-d.x / 2);
            } else {
                fx -= fa * ((float)d.y * 0.5f);
                fy -= fa * (-(float)d.x * 0.5f);
            }
        }
        // bending: angle at p between a = bond p-1 and b = bond p,
        // c = a.b/(|a||b|); dc/da = b/(|a||b|) - c a/|a|^2, dc/db = a/(|a||b|) - c b/|b|^2
        const T iab = invm * inv;
        T dcax, dcay, dcbx, dcby;
        if constexpr (PREC == kPrecFP64) {
            const T c = (bmx * bx + bmy * by) * iab;
            dcax = bx * iab - c * bmx * (invm * invm); dcay = by * iab - c * bmy * (invm * invm);
            dcbx = bmx * iab - c * bx * (inv * inv); dcby = bmy * iab - c * by * (inv * inv);
        } else {
            // the parts of each bond perpendicular to the other, from the FP64
            // cross product (a x b)(-a_y, a_x) / (|a|^3 |b|) and
            // -(a x b)(-b_y, b_x) / (|a| |b|^3): no cancellation
            const double amx = __shfl_sync(full, bd.x, pm), amy = __shfl_sync(full, bd.y, pm);
            const float q = (float)fma(amx, bd.y, -(amy * bd.x)) * iab;
            dcax = -q * bmy * (invm * invm); dcay = q * bmx * (invm * invm);
            dcbx = q * by * (inv * inv); dcby = -q * bx * (inv * inv);
        }
        const T nax = __shfl_sync(full, dcax, pp), nay = __shfl_sync(full, dcay, pp);   // angle at p+1
        const T pbx = __shfl_sync(full, dcbx, pm), pby = __shfl_sync(full, dcby, pm);   // angle at p-1
        if (kb != 0.0) {
            fx += kbt * (dcax - dcbx) - kbt * nax + kbt * pbx;
            fy += kbt * (dcay - dcby) - kbt * nay + kbt * pby;
        }
        int64_t nc = 0;
        if (act) nc = finish(p, xc, (V)fx, (V)fy);
        if (do_update && fused_count) count_into_chunk(C, act, S[p], nc, cap);
    } else {
        for (int base = 0; base < n; base += 32) {
            const int p = base + lane;
            const bool act = p < n;
            int64_t nc = 0;
            if (act) {
            int pm = p == 0 ? n - 1 : p - 1, pp = p == n - 1 ? 0 : p + 1;
            double2 xc = P[p], xm = P[pm], xp = P[pp];
            double fx = 0, fy = 0;
            // springs: f = -k (d - l) dr/d on (p, p+1) with dr = x_p - x_{p+1};
            // particle p is the first end of spring p and the second of spring p-1
            {
                double2 d = diff(xc, xp);
                double dist = sqrt(d.x * d.x + d.y * d.y);
                double sc = -k_s * (dist - l_s) / dist;
                fx += sc * d.x; fy += sc * d.y;
                double2 e = diff(xm, xc);
                double de = sqrt(e.x * e.x + e.y * e.y);
                double se = -k_s * (de - l_s) / de;
                fx -= se * e.x; fy -= se * e.y;
            }
            // area: F_p -= k_area (A - A0) * (dr.y, -dr.x)/2, dr = x_{p+1} - x_{p-1}
            {
                double2 d = diff(xp, xm);
                fx -= fmod_area * (d.y / 2);
                fy -= fmod_area * (-d.x / 2);
            }
            if (kb != 0.0) {
                // bending: E = kb sum_i (1 - cos theta_i); contributions of the
                // angles at p-1, p and p+1.
                int pmm = pm == 0 ? n - 1 : pm - 1, ppp = pp == n - 1 ? 0 : pp + 1;
                double2 xmm = P[pmm], xpp = P[ppp];
                auto dcos = [&](double2 a, double2 b, double2& dca, double2& dcb) {
                    double la = sqrt(a.x * a.x + a.y * a.y), lb = sqrt(b.x * b.x + b.y * b.y);
                    double c = (a.x * b.x + a.y * b.y) / (la * lb);
                    dca = make_double2(b.x / (la * lb) - c * a.x / (la * la), b.y / (la * lb) - c * a.y / (la * la));
                    dcb = make_double2(a.x / (la * lb) - c * b.x / (lb * lb), a.y / (la * lb) - c * b.y / (lb * lb));
                };
                double2 dca, dcb;
                dcos(diff(xc, xm), diff(xp, xc), dca, dcb);       // angle at p
                fx += kb * (dca.x - dcb.x); fy += kb * (dca.y - dcb.y);
                dcos(diff(xp, xc), diff(xpp, xp), dca, dcb);      // angle at p+1: p is its "i-1"
                fx += -kb * dca.x; fy += -kb * dca.y;
                dcos(diff(xm, xmm), diff(xc, xm), dca, dcb);      // angle at p-1: p is its "i+1"
                fx += kb * dcb.x; fy += kb * dcb.y;
            }
            nc = finish(p, xc, (V)fx, (V)fy);
            }
            if (do_update && fused_count) count_into_chunk(C, act, act ? S[p] : 0, nc, cap);
        }
    }
    ring_vc_store(C, g, lane, do_update, vcx, vcy);
}

// ===========================================================================
// user-order staging <-> sorted state
// ===========================================================================
// Polarisation of each ring (src/rings/integration.jl:340-351), one thread
// per ring: theta += asin(p x v_mean / |v_mean|) / tau dt + sqrt(2 D dt) xi,
// then (cos, sin) of the new angle for the next step. With update == 0 it
// only refreshes (cos, sin) (after an upload). The mixed form takes the
// deterministic increment and (cos, sin) in FP32 (the angle, reduced to
// [-pi, pi] in FP64, stays an FP64 sum); the FP64 transcendental functions
// dominate this kernel otherwise.
template <int PREC>
__global__ void k_ring_pol(Ctx C, int64_t total_rings, int32_t update) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_rings) return;
    if (update && C.var_rings && C.ring_active[g] == 0) return;   // update! runs over active rings
    double theta = C.ring_pol[g];
    if (update) {
        const int32_t rep = C.ring_rep[g];
        const DevRep& R = C.reps[rep];
        const MaviRingsCfg& rc = C.rcfg[rep];
        const int t = C.ring_types[g] - 1;
        const int32_t n = rc.num_particles[t];
        if constexpr (PREC == kPrecFP64) {
            const double2 vs = C.ring_vc[g], cs = C.ring_cs[g];
            const double2 vc = make_double2(vs.x / n, vs.y / n);
            const double dt = R.dt;
            const double speed = sqrt(vc.x * vc.x + vc.y * vc.y);
            double cr = 0.0;
            if (speed != 0) {
                cr = (cs.x * vc.y - cs.y * vc.x) / speed;
                if (fabs(cr) > 1) cr = jsign(cr);
            }
            double nz;
            if (C.noise_mode == MAVI_NOISE_INJECTED) nz = C.noise[R.noise0 + (g - R.ring0)];
            else nz = philox_normal(C.seed, (uint64_t)g, (uint64_t)(C.d_step[0] - 1));
            const double d_theta = 1 / rc.relax_time[t] * asin(cr) * dt + sqrt(2 * rc.rot_diff[t] * dt) * nz;
            theta = theta + d_theta;
        } else {
            const float2 vs = C.ring_vcf[g], cs = C.ring_csf[g];
            const float inv_n = 1.0f / (float)n;
            const float vx = vs.x * inv_n, vy = vs.y * inv_n;
            const float speed = sqrtf(vx * vx + vy * vy);
            float cr = 0.0f;
            if (speed != 0.0f) {
                cr = (cs.x * vy - cs.y * vx) / speed;
                if (fabsf(cr) > 1.0f) cr = copysignf(1.0f, cr);
            }
            double nz;
            if (C.noise_mode == MAVI_NOISE_INJECTED) nz = C.noise[R.noise0 + (g - R.ring0)];
            else nz = f32_to_f64_bits(philox_normal_f(C.seed, (uint64_t)g, (uint64_t)(C.d_step[0] - 1)));
            const double det = f32_to_f64_bits(asinf(cr) * R.ring_dt_tau_f[t]);
            theta = fma(R.ring_noise_amp[t], nz, theta + det);
        }
        C.ring_pol[g] = theta;
    }
    if constexpr (PREC == kPrecFP64) {
        double sn, cn;
        sincos(theta, &sn, &cn);
        C.ring_cs[g] = make_double2(cn, sn);
    } else {
        const double q = rint(theta * 0.15915494309189535);   // 1 / (2 pi)
        const float r = (float)fma(-q, 6.283185307179586, theta);
        float sn, cn;
        sincosf(r, &sn, &cn);
        C.ring_csf[g] = make_float2(cn, sn);
    }
}

// ===========================================================================
// Sources and sinks of the rings model: the head of step!
// (src/rings/integration.jl:522-526) for every replica that has some, one
// block per replica. It runs before the step's chunk update, so the chunk
// lists it reads (start[], the slots in *_cur order) are the previous
// update_chunks!'s, as the reference's ChunksChecker reads them; the current
// positions are in pos_out (same slot order), the previous step's in pos_cur.
// ===========================================================================
constexpr int kSrcThreads = 256;

// is_inside(point, ::RectangleCfg; pad) (src/configs.jl:89-93)
__device__ __forceinline__ bool inside_rect(double x, double y, double blx, double bly, double len, double h,
                                            double pad) {
    const bool ix = (blx - pad <= x) && (x <= blx + len + pad);
    const bool iy = (bly - pad <= y) && (y <= bly + h + pad);
    return ix && iy;
}

// is_inside(point, sink geometry) with pad 0 (src/configs.jl:89-93, 165-168)
__device__ __forceinline__ bool sink_inside(const SrcEntryD& E, double2 c) {
    if (E.geometry == MAVI_GEOM_CIRCLE) {
        const double dx = c.x - E.cx, dy = c.y - E.cy;
        const double rp = E.radius + 0.0;
        return dx * dx + dy * dy <= rp * rp;
    }
    return inside_rect(c.x, c.y, E.bl_x, E.bl_y, E.length, E.height, 0.0);
}

// update_cms! (src/rings/integration.jl:366-372) for one ring: the mean of the
// ring's positions, or with periodic walls of its continuous positions, which
// update_continuos_pos! (:118-138) formed from the previous step's positions.
// Summed in particle order.
__device__ __forceinline__ double2 ring_centre(const Ctx& C, const DevRep& R, int32_t ring, int32_t n) {
    const int32_t u0 = (int32_t)R.slot0 + ring * R.nmax;
    double sx, sy;
    if (R.periodic) {
        double2 prev = C.pos_cur[C.slot_of[u0]];
        double cx = prev.x, cy = prev.y;
        sx = cx; sy = cy;
        for (int32_t p = 1; p < n; p++) {
            const double2 q = C.pos_cur[C.slot_of[u0 + p]];
            double dx = q.x - prev.x, dy = q.y - prev.y;
            if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
            cx = cx + dx; cy = cy + dy;
            sx += cx; sy += cy;
            prev = q;
        }
    } else {
        const double2 q0 = C.pos_out[C.slot_of[u0]];
        sx = q0.x; sy = q0.y;
        for (int32_t p = 1; p < n; p++) {
            const double2 q = C.pos_out[C.slot_of[u0 + p]];
            sx += q.x; sy += q.y;
        }
    }
    return make_double2(sx / n, sy / n);
}

template <int PREC>
__global__ void __launch_bounds__(kSrcThreads) k_sources(Ctx C) {
    const int32_t rep = (int32_t)blockIdx.x;
    const DevRep& R = C.reps[rep];
    if (R.src_ne == 0) return;
    __shared__ int32_t sh_num_active, sh_max_uid, sh_first, sh_hits;
    __shared__ int32_t sh_flag[MAVI_MAX_SPAWN_BOXES];
    __shared__ int smem[32];
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int32_t nr = R.num_rings;
    const MaviRingsCfg& rc = C.rcfg[rep];
    int32_t* ids = C.src_ids + R.ring0;
    int32_t* act = C.ring_active + R.ring0;
    if (tid == 0) {
        sh_num_active = C.src_state[2 * rep];
        sh_max_uid = C.src_state[2 * rep + 1];
        sh_hits = 0;
    }
    __syncthreads();
    if (R.src_has_sink || R.inv_cms) {
        const int32_t na = sh_num_active;
        for (int32_t k = tid; k < na; k += nthr) {
            const int32_t ring = ids[k];
            const int32_t n = rc.num_particles[C.ring_types[R.ring0 + ring] - 1];
            C.ring_cms[R.ring0 + ring] = ring_centre(C, R, ring, n);
        }
    }
    __syncthreads();
    for (int32_t e = 0; e < R.src_ne; e++) {
        const SrcEntryD& E = C.src_entries[R.src_e0 + e];
        if (E.kind == MAVI_SRC_SINK) {
            // process_sink! (src/rings/sources.jl:253-260) over the view
            // ids[1:num_active] taken when the loop starts; every hit
            // decrements num_active (remove_ring!, src/rings/states.jl:176-180)
            const int32_t L = sh_num_active;
            int hits = 0;
            for (int32_t k = tid; k < L; k += nthr) {
                const int32_t ring = ids[k];
                if (sink_inside(E, C.ring_cms[R.ring0 + ring])) { act[ring] = 0; hits++; }
            }
            if (hits) atomicAdd(&sh_hits, hits);
            __syncthreads();
            if (tid == 0) { sh_num_active -= sh_hits; sh_hits = 0; }
            __syncthreads();
            continue;
        }
        // process_source! (src/rings/sources.jl:226-239): which boxes are empty
        // (update_area_empty!, :193-224), all before any ring is added
        const int32_t nb = E.num_boxes;
        for (int32_t b = tid; b < nb; b += nthr) sh_flag[b] = 0;
        __syncthreads();
        for (int32_t b = 0; b < nb; b++) {
            const SrcBoxD& B = C.src_boxes[E.box0 + b];
            bool occ = false;
            if (B.num_chunks < 0) {
                // PosChecker: the active particles of the last update_ids!
                const int32_t lo = C.start[R.c0], hi = C.start[R.c0 + (int64_t)R.rows * R.cols];
                for (int32_t q = lo + tid; q < hi && !occ; q += nthr) {
                    const double2 x = C.pos_out[q];
                    occ = inside_rect(x.x, x.y, B.bl_x, B.bl_y, B.length, B.height, E.pad);
                }
            } else {
                for (int32_t k = tid; k < B.num_chunks && !occ; k += nthr) {
                    const int32_t c = C.src_chunks[B.chunk0 + k];
                    for (int32_t q = C.start[c]; q < C.start[c + 1] && !occ; q++) {
                        const double2 x = C.pos_out[q];
                        occ = inside_rect(x.x, x.y, B.bl_x, B.bl_y, B.length, B.height, E.pad);
                    }
                }
            }
            if (occ) sh_flag[b] = 1;
        }
        __syncthreads();
        for (int32_t b = 0; b < nb; b++) {
            if (sh_flag[b]) continue;   // block-uniform
            const SrcBoxD& B = C.src_boxes[E.box0 + b];
            // add_ring! (src/rings/states.jl:162-174): the first inactive slot
            if (tid == 0) sh_first = 0x7fffffff;
            __syncthreads();
            for (int32_t k = tid; k < nr; k += nthr)
                if (act[k] == 0) { atomicMin(&sh_first, k); break; }
            __syncthreads();
            const int32_t ring = sh_first;
            if (ring == 0x7fffffff) continue;   // no free slot: nothing added (block-uniform)
            const int64_t g = R.ring0 + ring;
            const int32_t n = rc.num_particles[C.ring_types[g] - 1];
            for (int32_t p = tid; p < n; p += nthr)
                C.pos_out[C.slot_of[(int32_t)R.slot0 + ring * R.nmax + p]] = C.src_spawn[B.spawn0 + p];
            if (tid == 0) {
                act[ring] = 1;
                sh_max_uid += 1;
                C.ring_uid[g] = sh_max_uid;
                sh_num_active += 1;
                double pol = E.pol;
                if (E.pol_mode == MAVI_SPAWN_POL_RANDOM) {
                    // get_spawn_pol (src/rings/sources.jl:23-24): rand() * 2 * pi
                    double u;
                    if (C.noise_mode == MAVI_NOISE_INJECTED) u = C.noise[B.noise_idx];
                    else u = philox_uniform2(C.seed, (uint64_t)B.noise_idx + (1ull << 40), (uint64_t)C.d_step[0]).a - 0x1p-53;
                    pol = u * 2.0 * 3.141592653589793;
                }
                C.ring_pol[g] = pol;
                if constexpr (PREC == kPrecFP64) {
                    double sn, cn;
                    sincos(pol, &sn, &cn);
                    C.ring_cs[g] = make_double2(cn, sn);
                } else {
                    const double q = rint(pol * 0.15915494309189535);
                    const float r = (float)fma(-q, 6.283185307179586, pol);
                    float sn, cn;
                    sincosf(r, &sn, &cn);
                    C.ring_csf[g] = make_float2(cn, sn);
                }
                // process_source! sets the new ring's centre: sum(rings_pos[1:n]) / n
                double2 q0 = C.src_spawn[B.spawn0];
                double sx = q0.x, sy = q0.y;
                for (int32_t p = 1; p < n; p++) { const double2 q = C.src_spawn[B.spawn0 + p]; sx += q.x; sy += q.y; }
                C.ring_cms[g] = make_double2(sx / n, sy / n);
            }
            __syncthreads();
        }
    }
    __syncthreads();
    // update_ids! (calc_active_ids!, src/rings/states.jl:200-219): active rings
    // in ascending order; entries past the new count keep their old values
    int32_t base = 0;
    for (int32_t k0 = 0; k0 < nr; k0 += nthr) {
        const int32_t k = k0 + tid;
        const int a = (k < nr && act[k] != 0) ? 1 : 0;
        int total;
        const int ex = block_exclusive_scan(a, smem, total);
        if (a) ids[base + ex] = k;
        base += total;
    }
    if (tid == 0) {
        C.src_state[2 * rep] = base;
        C.src_state[2 * rep + 1] = sh_max_uid;
    }
}

// *_out := *_cur (rings with sources and sinks, after a chunk update outside
// the step): between steps their current state lives in *_out in the slot
// order of *_cur, where k_sources reads it.
static __global__ void k_out_from_cur(Ctx C) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    C.pos_out[s] = C.pos_cur[s];
    C.uid_out[s] = C.uid_cur[s];
    C.rep_out[s] = C.rep_cur[s];
    C.cell_out[s] = C.cell_cur[s];
    if (C.off_out) C.off_out[s] = C.off_cur[s];
}

// Ring areas on demand (RingsInfo.areas, set by area_forces!,
// src/rings/integration.jl:140-160): calc_area (:103-116) of the continuous
// positions (update_continuos_pos!, :118-138: cumulative differences with
// periodic walls, the positions themselves otherwise) of the last force
// evaluation (the *_cur state), FP64, summed in particle order.
// calc_area (src/rings/integration.jl:103-116) of the continuous positions
// (update_continuos_pos!, :118-138: cumulative calc_diff from particle 1 with
// periodic walls, the positions themselves otherwise), in the reference's own
// operation order and rounding: cross products of the continuous coordinates
// added one after the other, no fused operations. The sum cancels (terms of
// order |x|^2, result of order the ring's area), so its rounding depends on
// that order; this keeps the FP64 form's areas bit for bit the reference's.
// at(i): FP64 position of the ring's particle i.
template <class At>
__device__ __forceinline__ double ring_area_reference(const DevRep& R, int32_t n, At at) {
    const double2 c0 = at(0);
    double2 prev = c0, cprev = c0;
    double area = 0.0;
    for (int32_t i = 1; i < n; i++) {
        const double2 q = at(i);
        double2 c = q;
        if (R.periodic) {
            double dx = __dsub_rn(q.x, prev.x), dy = __dsub_rn(q.y, prev.y);
            if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
            c = make_double2(__dadd_rn(cprev.x, dx), __dadd_rn(cprev.y, dy));
        }
        area = __dadd_rn(area, __dsub_rn(__dmul_rn(cprev.x, c.y), __dmul_rn(cprev.y, c.x)));
        prev = q;
        cprev = c;
    }
    area = __dadd_rn(area, __dsub_rn(__dmul_rn(cprev.x, c0.y), __dmul_rn(cprev.y, c0.x)));
    return area / 2.0;
}

static __global__ void k_ring_areas(Ctx C, int64_t ring0, int64_t nrings, double* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrings) return;
    const int64_t g = ring0 + k;
    const DevRep& R = C.reps[C.ring_rep[g]];
    const int32_t rl = (int32_t)(g - R.ring0);
    const int32_t n = C.rcfg[C.ring_rep[g]].num_particles[C.ring_types[g] - 1];
    const int32_t u0 = (int32_t)R.slot0 + rl * R.nmax;
    out[k] = ring_area_reference(R, n, [&](int32_t i) { return C.pos_cur[C.slot_of[u0 + i]]; });
}

// FP64 rings step: each active ring's area at the current positions (user
// order, where the ring is contiguous), one thread per ring, for k_rings.
static __global__ void k_ring_area_ref(Ctx C, int64_t total_rings) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total_rings) return;
    if (C.var_rings && C.ring_active[g] == 0) return;
    const int32_t rep = C.ring_rep[g];
    const DevRep& R = C.reps[rep];
    const int32_t n = C.rcfg[rep].num_particles[C.ring_types[g] - 1];
    const int32_t u0 = (int32_t)R.slot0 + (int32_t)(g - R.ring0) * R.nmax;
    C.ring_area[g] = ring_area_reference(R, n, [&](int32_t i) { return C.pos_u[u0 + i]; });
}

static __global__ void k_gather_user(Ctx C, const double2* __restrict__ pos_user, const double2* __restrict__ vel_user,
                              const double* __restrict__ pol_user) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    int32_t u = C.uid_out[s];
    if (pos_user) C.pos_out[s] = pos_user[u];
    if (vel_user) C.vel_out[s] = vel_user[u];
    if (pol_user) C.pol_out[s] = pol_user[u];
}

static __global__ void k_scatter_user(Ctx C, double2* __restrict__ pos_user, double2* __restrict__ vel_user,
                               double* __restrict__ pol_user) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    int32_t u = C.uid_out[s];
    pos_user[u] = C.pos_out[s];
    if (vel_user) vel_user[u] = C.vel_out[s];
    if (pol_user) pol_user[u] = C.pol_out[s];
}

// forces in sorted order -> user order (double)
template <int PREC>
__global__ void k_forces_to_user(Ctx C, double2* __restrict__ f_user) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    int32_t u = C.uid_cur[s];
    if (C.pos_u) {   // rings keep the force in user order
        if constexpr (PREC == kPrecFP64) f_user[u] = C.fd_u[u];
        else { float2 f = C.ff_u[u]; f_user[u] = make_double2(f.x, f.y); }
        return;
    }
    if constexpr (PREC == kPrecFP64) f_user[u] = C.fd[s];
    else { float2 f = C.ff[s]; f_user[u] = make_double2(f.x, f.y); }
}

// ===========================================================================
// energies: per-particle terms then a deterministic per-replica reduction
// ===========================================================================
static __global__ void k_energy_terms(Ctx C, int32_t dyn, int32_t all_pairs, double* __restrict__ ke_t,
                               double* __restrict__ pe_t, int32_t has_vel) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    const DevRep& R = C.reps[C.rep_cur[s]];
    if (C.var_rings && C.cell_cur[s] == C.park) { ke_t[s] = 0.0; pe_t[s] = 0.0; return; }   // inactive ring
    double ke = 0;
    if (has_vel) { double2 v = C.vel_cur[s]; ke = v.x * v.x + v.y * v.y; }
    ke_t[s] = ke;
    double2 pi = C.pos_cur[s];
    double e[4] = {R.pd[4], R.pd[5], R.pd[6], R.pd[7]};
    if (dyn == MAVI_DYN_HARM_TRUNC) { e[0] = R.pd[0]; e[1] = R.pd[1]; e[2] = R.pd[5]; e[3] = R.pd[6]; }
    double pe = 0, comp = 0;
    auto visit = [&](int32_t b, int32_t e_) {
        for (int32_t j = b; j < e_; j++) {
            if (j == (int32_t)s) continue;
            double2 q = C.pos_cur[j];
            double dx = pi.x - q.x, dy = pi.y - q.y;
            if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
            double u = pair_energy(dyn, e, dx * dx + dy * dy) - comp;
            double t = pe + u;
            comp = (t - pe) - u;
            pe = t;
        }
    };
    if (all_pairs || !R.has_chunks) {
        // the replica's chunked particles (parked ones, of inactive rings, follow every chunk)
        visit(C.start[R.c0], C.start[R.c0 + (int64_t)R.rows * R.cols]);
    } else {
        int64_t lc = C.cell_cur[s] - R.c0;
        int32_t row = (int32_t)(lc % R.rows), col = (int32_t)(lc / R.rows);
        for (int dc = -1; dc <= 1; dc++) {
            int ncol = col + dc;
            if (R.periodic) ncol = ncol < 0 ? ncol + R.cols : (ncol >= R.cols ? ncol - R.cols : ncol);
            else if (ncol < 0 || ncol >= R.cols) continue;
            for (int dr = -1; dr <= 1; dr++) {
                int nrow = row + dr;
                if (R.periodic) nrow = nrow < 0 ? nrow + R.rows : (nrow >= R.rows ? nrow - R.rows : nrow);
                else if (nrow < 0 || nrow >= R.rows) continue;
                int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
                visit(C.start[nc], C.start[nc + 1]);
            }
        }
    }
    pe_t[s] = 0.5 * pe;
}

// One block per replica: Kahan-compensated per-thread sums, fixed-order tree.
static __global__ void k_reduce_per_replica(Ctx C, const double* __restrict__ t, double* __restrict__ out, double scale) {
    __shared__ double sh[256];
    const DevRep& R = C.reps[blockIdx.x];
    double sum = 0, comp = 0;
    for (int64_t s = R.a0 + threadIdx.x; s < R.a0 + R.na; s += blockDim.x) {
        double y = t[s] - comp;
        double tt = sum + y;
        comp = (tt - sum) - y;
        sum = tt;
    }
    sh[threadIdx.x] = sum;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0] * scale;
}

// Pair-distance histogram of the current state (the counts behind the pair
// distribution g(r)): counts[k] += the unordered pairs (i, j) of a replica
// (rep_sel; -1: every replica) with floor(d / dr) == k and d < r_max, where d
// is the length of calc_diff(x_i, x_j) (src/integration.jl:38-52) from the
// FP64 positions, formed with IEEE operations in a fixed order (no fused
// multiply-add) and binned by a correctly rounded division: the counts are
// exact integers, equal to the CPU restatement's. r_max must not exceed the
// chunk sides, so every pair closer than r_max lies in the 3x3 chunk
// neighbourhood; a pair is counted from its lower sorted slot. Bins live in
// shared memory per block (nbins <= kHistMaxBins) and are added to the global
// counts once per block.
constexpr int kHistMaxBins = 4096;
static __global__ void k_pair_hist(Ctx C, int32_t rep_sel, double r_max, double dr, int32_t nbins,
                                   unsigned long long* __restrict__ counts) {
    __shared__ uint32_t bins[kHistMaxBins];
    for (int k = threadIdx.x; k < nbins; k += blockDim.x) bins[k] = 0;
    __syncthreads();
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t rep = (s < C.M && C.num_reps > 1) ? C.rep_cur[s] : 0;
    if (s < C.M && (rep_sel < 0 || rep == rep_sel) && !(C.var_rings && C.cell_cur[s] == C.park)) {
        const DevRep& R = C.reps[rep];
        const double2 pi = C.pos_cur[s];
        auto visit = [&](int32_t b, int32_t e) {
            for (int32_t j = max(b, (int32_t)s + 1); j < e; j++) {
                const double2 q = C.pos_cur[j];
                double dx = __dsub_rn(pi.x, q.x), dy = __dsub_rn(pi.y, q.y);
                if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
                const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
                if (d < r_max) {
                    const int32_t k = min((int32_t)__ddiv_rn(d, dr), nbins - 1);
                    atomicAdd(&bins[k], 1u);
                }
            }
        };
        if (!R.has_chunks) {
            visit(C.start[R.c0], C.start[R.c0 + 1]);
        } else {
            const int64_t lc = C.cell_cur[s] - R.c0;
            const int32_t row = (int32_t)(lc % R.rows), col = (int32_t)(lc / R.rows);
            for (int dc = -1; dc <= 1; dc++) {
                int ncol = col + dc;
                if (R.periodic) ncol = ncol < 0 ? ncol + R.cols : (ncol >= R.cols ? ncol - R.cols : ncol);
                else if (ncol < 0 || ncol >= R.cols) continue;
                for (int drow = -1; drow <= 1; drow++) {
                    int nrow = row + drow;
                    if (R.periodic) nrow = nrow < 0 ? nrow + R.rows : (nrow >= R.rows ? nrow - R.rows : nrow);
                    else if (nrow < 0 || nrow >= R.rows) continue;
                    const int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
                    visit(C.start[nc], C.start[nc + 1]);
                }
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nbins; k += blockDim.x)
        if (bins[k]) atomicAdd(&counts[k], (unsigned long long)bins[k]);
}

// candidate-pair count per particle (roofline accounting)
static __global__ void k_pair_count(Ctx C, unsigned long long* __restrict__ total) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c = 0;
    if (s < C.M) {
        const DevRep& R = C.reps[C.rep_cur[s]];
        if (C.var_rings && C.cell_cur[s] == C.park) c = 0;
        else if (!R.has_chunks) c = C.start[R.c0 + 1] - C.start[R.c0] - 1;
        else {
            int64_t lc = C.cell_cur[s] - R.c0;
            int32_t row = (int32_t)(lc % R.rows), col = (int32_t)(lc / R.rows);
            for (int dc = -1; dc <= 1; dc++) {
                int ncol = col + dc;
                if (R.periodic) ncol = ncol < 0 ? ncol + R.cols : (ncol >= R.cols ? ncol - R.cols : ncol);
                else if (ncol < 0 || ncol >= R.cols) continue;
                for (int dr = -1; dr <= 1; dr++) {
                    int nrow = row + dr;
                    if (R.periodic) nrow = nrow < 0 ? nrow + R.rows : (nrow >= R.rows ? nrow - R.rows : nrow);
                    else if (nrow < 0 || nrow >= R.rows) continue;
                    int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
                    c += C.start[nc + 1] - C.start[nc];
                }
            }
            c -= 1;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

}  // namespace mavi
