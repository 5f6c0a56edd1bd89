// mavi_kernels.cuh — kernels of libmavi_cuda.so.
//
// Data layout in HBM (all replicas of a handle concatenated):
//  * particles live in chunk-sorted order ("slots" s = 0..M-1): replica-major,
//    then chunk (column-major, as Julia's chunk arrays), then ascending user
//    id inside a chunk — exactly the order of the reference's
//    chunk_particles[:, row, col] lists (src/chunks.jl:144-146);
//  * SoA arrays: positions double2, velocities double2, FP32 chunk-centre
//    offsets float2 (mixed form), user id int32, replica int32;
//  * chunks in CSR form: count[c], start[c] over all replicas' chunks.
// A step reads the state in "previous order" (*_out arrays, written by the
// last step together with each particle's new chunk and its rank inside it),
// rebuilds the chunk lists (scan -> scatter -> per-chunk order + permutation
// into *_cur arrays) and runs the fused force/update passes.
#pragma once

#include "mavi_device.cuh"

namespace mavi {

struct Ctx {
    // particle arrays in sorted order
    double2 *pos_cur, *pos_mid, *pos_out;
    double2 *vel_cur, *vel_out;
    double *pol_cur, *pol_out;
    float2 *off_cur, *off_mid;
    double2 *fd;     // pair-pass force (FP64 form)
    float2 *ff;      // pair-pass force (mixed form)
    double2 *fold_d; // Verlet F(t), FP64 form
    float2 *fold_f;  // Verlet F(t), mixed form
    int32_t *uid_cur, *uid_out, *rep_cur, *rep_out;
    int32_t *cell_cur, *cell_out, *rank;
    int32_t *count, *start, *src_of, *slot_of;
    // per ring (global ring index)
    double *ring_pol;
    double *ring_area;
    const int32_t *ring_types;
    // descriptors
    const DevRep *reps;
    const MaviSpace *spaces;     // [replica][MAVI_MAX_SPACES]
    const MaviRingsCfg *rcfg;    // [replica]
    DevError *err;
    int64_t M;        // active particles
    int64_t Ctot;     // chunks over all replicas
    int64_t *d_step;  // steps completed (device copy, for the RNG counter)
    const double *noise;
    int32_t noise_mode;
    int32_t num_reps;
    uint64_t seed;
};

// ===========================================================================
// chunk index of a position, with bounds/finite checks (src/chunks.jl:120-147)
// ===========================================================================
__device__ __forceinline__ int64_t cell_of(const DevRep& R, double x, double y, DevError* err,
                                           int64_t s, bool valid) {
    if (!R.has_chunks) return R.c0;
    int64_t row, col;
    bool finite;
    chunk_row_col(R, x, y, row, col, finite);
    if (valid) {
        if (!finite) raise_error(err, MAVI_ERR_NONFINITE, s, 0);
        else if (row < 0 || row >= R.rows || col < 0 || col >= R.cols)
            raise_error(err, MAVI_ERR_OUT_OF_GRID, s, row * 1000003 + col);
    }
    row = row < 0 ? 0 : (row >= R.rows ? R.rows - 1 : row);
    col = col < 0 ? 0 : (col >= R.cols ? R.cols - 1 : col);
    return R.c0 + col * (int64_t)R.rows + row;
}

// Warp-aggregated histogram update: lanes with the same chunk share one
// atomic; each lane gets its rank of arrival inside the chunk. Must be called
// by all 32 lanes of the warp.
__device__ __forceinline__ void count_into_chunk(const Ctx& C, bool valid, int64_t s, int64_t cell,
                                                 int32_t cap) {
    const unsigned full = 0xffffffffu;
    int key = valid ? (int)cell : -1;
    unsigned peers = __match_any_sync(full, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (valid && lane == leader) base = atomicAdd(&C.count[cell], __popc(peers));
    base = __shfl_sync(full, base, leader);
    if (valid) {
        int r = base + __popc(peers & ((1u << lane) - 1u));
        C.cell_out[s] = (int32_t)cell;
        C.rank[s] = r;
        if (r >= cap) raise_error(C.err, MAVI_ERR_CHUNK_OVERFLOW, s, cell);
    }
}

// Standalone histogram of the *_out state (upload, explicit update_chunks!).
static __global__ void k_count(Ctx C) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = s < C.M;
    int64_t cell = 0;
    int32_t cap = 1 << 30;
    if (valid) {
        const DevRep& R = C.reps[C.rep_out[s]];
        double2 p = C.pos_out[s];
        cell = cell_of(R, p.x, p.y, C.err, s, true);
        cap = R.has_chunks ? R.cap : (1 << 30);
    }
    count_into_chunk(C, valid, s, cell, cap);
}

// ===========================================================================
// exclusive scan of chunk counts -> start (three passes over 2048-chunk tiles)
// ===========================================================================
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

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

static __global__ void k_scan_reduce(const int32_t* __restrict__ count, int64_t n, int32_t* __restrict__ tile_sum) {
    __shared__ int smem[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) v += (base + k < n) ? count[base + k] : 0;
    int total;
    block_exclusive_scan(v, smem, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// Single block: exclusive scan of the tile sums, in 1024-wide rounds.
static __global__ void k_scan_tiles(int32_t* __restrict__ tile_sum, int64_t ntiles, int32_t* __restrict__ start,
                             int64_t n, int64_t* d_step, int32_t advance) {
    __shared__ int smem[32];
    int carry = 0;
    for (int64_t b = 0; b < ntiles; b += blockDim.x) {
        int64_t i = b + threadIdx.x;
        int v = i < ntiles ? tile_sum[i] : 0;
        int total;
        int ex = block_exclusive_scan(v, smem, total);
        if (i < ntiles) tile_sum[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        start[n] = carry;
        if (advance) d_step[0] += 1;
    }
}

static __global__ void k_scan_apply(const int32_t* __restrict__ count, int64_t n, const int32_t* __restrict__ tile_off,
                             int32_t* __restrict__ start) {
    __shared__ int smem[32];
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? count[base + k] : 0;
        sum += v[k];
    }
    int total;
    int ex = block_exclusive_scan(sum, smem, total) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) start[base + k] = ex;
        ex += v[k];
    }
}

// ===========================================================================
// scatter: each particle claims start[cell] + rank
// ===========================================================================
static __global__ void k_scatter(Ctx C) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    int32_t c = C.cell_out[s];
    int32_t dst = C.start[c] + C.rank[s];
    // ranks are < count[c] by construction, so dst stays inside [start[c], start[c+1])
    C.src_of[dst] = (int32_t)s;
}

// ===========================================================================
// per chunk: order members by user id (the reference appends particles in
// ascending id, src/chunks.jl:150-161) and permute the state into *_cur.
// ===========================================================================
constexpr int kSortMax = 64;

template <int PREC, bool HAS_VEL, bool HAS_POL>
__global__ void k_sort_permute(Ctx C) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C.Ctot) return;
    int32_t b = C.start[c], e = C.start[c + 1];
    int32_t k = e - b;
    if (k <= 0) return;
    int32_t src[kSortMax];
    int32_t key[kSortMax];
    bool sorted = k <= kSortMax;
    if (sorted) {
        for (int m = 0; m < k; m++) {
            int32_t sm = C.src_of[b + m];
            int32_t km = C.uid_out[sm];
            int q = m;
            while (q > 0 && key[q - 1] > km) {
                key[q] = key[q - 1];
                src[q] = src[q - 1];
                q--;
            }
            key[q] = km;
            src[q] = sm;
        }
    }
    for (int m = 0; m < k; m++) {
        int32_t sm = sorted ? src[m] : C.src_of[b + m];
        int32_t dst = b + m;
        double2 p = C.pos_out[sm];
        int32_t u = C.uid_out[sm];
        int32_t r = C.rep_out[sm];
        C.pos_cur[dst] = p;
        C.uid_cur[dst] = u;
        C.rep_cur[dst] = r;
        C.cell_cur[dst] = (int32_t)c;
        C.slot_of[u] = dst;
        if constexpr (HAS_VEL) C.vel_cur[dst] = C.vel_out[sm];
        if constexpr (HAS_POL) C.pol_cur[dst] = C.pol_out[sm];
        if constexpr (PREC == kPrecMixed) {
            const DevRep& R = C.reps[r];
            int64_t lc = c - R.c0;
            int64_t row = lc % R.rows, col = lc / R.rows;
            C.off_cur[dst] = make_float2((float)(p.x - chunk_cx(R, col)), (float)(p.y - chunk_cy(R, row)));
        }
    }
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
// ===========================================================================

// Accumulator: FP64, or FP32 with Kahan compensation.
template <int PREC> struct Acc;
template <> struct Acc<kPrecFP64> {
    double x = 0, y = 0;
    __device__ __forceinline__ void add(double fx, double fy) { x += fx; y += fy; }
    __device__ __forceinline__ double gx() const { return x; }
    __device__ __forceinline__ double gy() const { return y; }
};
template <> struct Acc<kPrecMixed> {
    float x = 0, y = 0, cx = 0, cy = 0;
    __device__ __forceinline__ void add(float fx, float fy) {
        float yx = fx - cx, tx = x + yx;
        cx = (tx - x) - yx;
        x = tx;
        float yy = fy - cy, ty = y + yy;
        cy = (ty - y) - yy;
        y = ty;
    }
    __device__ __forceinline__ double gx() const { return (double)x - (double)cx; }
    __device__ __forceinline__ double gy() const { return (double)y - (double)cy; }
};

// Rings pair term (src/rings/integration.jl:32-77): interaction matrix by ring
// type, zero beyond dist_max, bonded neighbours of the same ring excluded,
// attraction only between different rings.
template <typename T>
__device__ __forceinline__ T rings_pair_scalar(const MaviRingsCfg& rc, int ti, int tj, bool same_ring,
                                               int32_t pi, int32_t pj, int32_t n_i, T d2) {
    T dmax = (T)rc.inter_dist_max[ti][tj];
    if (d2 > dmax * dmax) return T(0);
    if (same_ring) {
        int32_t diff = pi > pj ? pi - pj : pj - pi;
        if (diff == 1 || diff == n_i - 1) return T(0);
    }
    T deq = (T)rc.inter_dist_eq[ti][tj];
    T inv_d = rsqrt_<T>(d2);
    T k;
    if (d2 < deq * deq) k = (T)rc.inter_k_rep[ti][tj];
    else k = same_ring ? T(0) : (T)rc.inter_k_atr[ti][tj];
    // fmod/dist = -k (dist/deq - 1)/dist = k (1/dist - 1/deq)
    return k * (inv_d - T(1) / deq);
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

template <int PREC, int DYN>
__device__ __forceinline__ void gather_pair_forces(const Ctx& C, const DevRep& R, int64_t s, int32_t cell,
                                                   const double2* __restrict__ P,
                                                   const float2* __restrict__ O, Acc<PREC>& acc) {
    using T = typename std::conditional<PREC == kPrecFP64, double, float>::type;
    const T* prm;
    if constexpr (PREC == kPrecFP64) prm = R.pd; else prm = R.pf;
    T pix, piy;
    if constexpr (PREC == kPrecFP64) { double2 p = P[s]; pix = p.x; piy = p.y; }
    else { float2 o = O[s]; pix = o.x; piy = o.y; }
    const bool mi = R.min_image;
    T bx, by, hx, hy;
    if constexpr (PREC == kPrecFP64) { bx = R.box_x; by = R.box_y; hx = R.half_box_x; hy = R.half_box_y; }
    else { bx = R.box_xf; by = R.box_yf; hx = R.half_box_xf; hy = R.half_box_yf; }

    RingInfo me{0, 0, 0};
    const MaviRingsCfg* rc = nullptr;
    int32_t n_me = 0;
    if constexpr (DYN == MAVI_DYN_RINGS) {
        me = ring_info(C, R, C.uid_cur[s]);
        rc = &C.rcfg[C.rep_cur[s]];
        n_me = rc->num_particles[me.type];
    }

    auto visit = [&](int32_t b, int32_t e, T shx, T shy) {
        for (int32_t j = b; j < e; j++) {
            if (j == (int32_t)s) continue;
            T dx, dy;
            if constexpr (PREC == kPrecFP64) {
                double2 q = P[j];
                dx = pix - q.x;
                dy = piy - q.y;
            } else {
                float2 q = O[j];
                dx = (pix - q.x) + shx;
                dy = (piy - q.y) + shy;
            }
            if (mi) {
                if constexpr (PREC == kPrecFP64) { dx = min_image1(dx, bx, hx); dy = min_image1(dy, by, hy); }
                else { dx = min_image1f(dx, bx, hx); dy = min_image1f(dy, by, hy); }
            }
            T d2 = dx * dx + dy * dy;
            T sc;
            if constexpr (DYN == MAVI_DYN_RINGS) {
                RingInfo o = ring_info(C, R, C.uid_cur[j]);
                sc = rings_pair_scalar<T>(*rc, me.type, o.type, o.ring == me.ring, me.p, o.p, n_me, d2);
            } else {
                sc = pair_scalar<DYN, T>(prm, d2);
            }
            acc.add(sc * dx, sc * dy);
        }
    };

    if (!R.has_chunks) {  // all pairs inside the replica (src/integration.jl:197-224)
        visit((int32_t)R.a0, (int32_t)(R.a0 + R.na), T(0), T(0));
        return;
    }
    int64_t lc = cell - R.c0;
    int32_t row = (int32_t)(lc % R.rows), col = (int32_t)(lc / R.rows);
    T cl, ch;
    if constexpr (PREC == kPrecFP64) { cl = R.chunk_l; ch = R.chunk_h; } else { cl = R.chunk_lf; ch = R.chunk_hf; }
#pragma unroll 1
    for (int dc = -1; dc <= 1; dc++) {
        int ncol = col + dc;
        if (R.periodic) ncol = ncol < 0 ? ncol + R.cols : (ncol >= R.cols ? ncol - R.cols : ncol);
        else if (ncol < 0 || ncol >= R.cols) continue;
#pragma unroll 1
        for (int dr = -1; dr <= 1; dr++) {
            int nrow = row + dr;
            if (R.periodic) nrow = nrow < 0 ? nrow + R.rows : (nrow >= R.rows ? nrow - R.rows : nrow);
            else if (nrow < 0 || nrow >= R.rows) continue;
            int64_t nc = R.c0 + (int64_t)ncol * R.rows + nrow;
            int32_t b = C.start[nc], e = C.start[nc + 1];
            // offset of the neighbour chunk centre relative to ours:
            // x grows with the column, y decreases with the row.
            T shx = -(T)dc * cl, shy = (T)dr * ch;
            visit(b, e, shx, shy);
        }
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

static __device__ void add_wall_forces(const Ctx& C, int32_t rep, const DevRep& R, double x, double y,
                                double& fx, double& fy) {
    const MaviSpace* sps = C.spaces + (int64_t)rep * MAVI_MAX_SPACES;
    for (int k = 0; k < R.num_spaces; k++) {
        const MaviSpace& sp = sps[k];
        if (sp.wall != MAVI_WALL_POTENTIAL) continue;
        if (sp.geometry == MAVI_GEOM_CIRCLE) {   // signed_pos (src/configs.jl:154-163)
            double drx = x - sp.cx, dry = y - sp.cy;
            double dist = sqrt(drx * drx + dry * dry);
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

static __device__ void apply_walls(const Ctx& C, int32_t rep, const DevRep& R, double radius, double& x, double& y,
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

template <int PREC, int DYN, int PASS, bool HAS_VEL, bool HAS_POL>
__global__ void __launch_bounds__(256) k_pass(Ctx C, int32_t with_wall_forces) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = s < C.M;
    int64_t new_cell = 0;
    int32_t cap = 1 << 30;
    if (valid) {
        int32_t rep = C.rep_cur[s];
        const DevRep& R = C.reps[rep];
        int32_t cell = C.cell_cur[s];
        Acc<PREC> acc;
        const double2* P = (PASS == kPassVerlet2) ? C.pos_mid : C.pos_cur;
        const float2* O = (PASS == kPassVerlet2) ? C.off_mid : C.off_cur;
        gather_pair_forces<PREC, DYN>(C, R, s, cell, P, O, acc);
        double fx = acc.gx(), fy = acc.gy();
        double2 p = P[s];
        bool walls_f = (PASS != kPassVerlet2) && with_wall_forces && R.has_wall_forces;
        if (walls_f) add_wall_forces(C, rep, R, p.x, p.y, fx, fy);
        const double dt = R.dt;
        if constexpr (PASS == kPassForce) {
            if constexpr (PREC == kPrecFP64) C.fd[s] = make_double2(fx, fy);
            else C.ff[s] = make_float2((float)fx, (float)fy);
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
                int64_t lc = cell - R.c0;
                int64_t row = lc % R.rows, col = lc / R.rows;
                C.off_mid[s] = make_float2((float)(nx - chunk_cx(R, col)), (float)(ny - chunk_cy(R, row)));
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
                double mdt = R.mobility * dt;
                x = __dadd_rn(x, __dmul_rn(fx, mdt));
                y = __dadd_rn(y, __dmul_rn(fy, mdt));
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
            apply_walls(C, rep, R, R.radius, x, y, vx, vy, HAS_VEL);
            C.pos_out[s] = make_double2(x, y);
            if constexpr (HAS_VEL) C.vel_out[s] = make_double2(vx, vy);
            if constexpr (HAS_POL && !(PASS == kPassSzabo || PASS == kPassRTP)) C.pol_out[s] = C.pol_cur[s];
            C.uid_out[s] = C.uid_cur[s];
            C.rep_out[s] = rep;
            new_cell = cell_of(R, x, y, C.err, s, true);
            cap = R.has_chunks ? R.cap : (1 << 30);
        }
    }
    if constexpr (PASS == kPassVerlet2 || PASS == kPassOverdamped || PASS == kPassSzabo || PASS == kPassRTP)
        count_into_chunk(C, valid, s, new_cell, cap);
}

// ===========================================================================
// rings: one warp per ring. Bonded terms (springs src/rings/integration.jl:
// 79-97 & 205-223, area :103-195, bending), wall forces, the overdamped
// active update (:300-351), walls! and the histogram for the next step.
// Positions of the ring are staged in shared memory.
// ===========================================================================
constexpr int kRingMax = 256;     // particles per ring supported
constexpr int kRingWarps = 4;     // rings per block

template <int PREC>
__global__ void __launch_bounds__(32 * kRingWarps) k_rings(Ctx C, int64_t total_rings, int32_t do_update) {
    __shared__ double2 sp_[kRingWarps][kRingMax];
    __shared__ int32_t ss_[kRingWarps][kRingMax];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t g = (int64_t)blockIdx.x * kRingWarps + w;
    if (g >= total_rings) return;   // whole warp exits together
    // replica of ring g: binary search over ring offsets
    int lo = 0, hi = C.num_reps - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (C.reps[mid].ring0 <= g) lo = mid; else hi = mid - 1;
    }
    const int32_t rep = lo;
    const DevRep& R = C.reps[rep];
    const MaviRingsCfg& rc = C.rcfg[rep];
    const int32_t rl = (int32_t)(g - R.ring0);
    const int t = C.ring_types[g] - 1;
    const int32_t n = rc.num_particles[t];
    double2* P = sp_[w];
    int32_t* S = ss_[w];
    for (int p = lane; p < n; p += 32) {
        int32_t uid = (int32_t)R.slot0 + rl * R.nmax + p;
        int32_t s = C.slot_of[uid];
        S[p] = s;
        P[p] = C.pos_cur[s];
    }
    __syncwarp();
    auto diff = [&](double2 a, double2 b) {
        double dx = a.x - b.x, dy = a.y - b.y;
        if (R.min_image) { dx = min_image1(dx, R.box_x, R.half_box_x); dy = min_image1(dy, R.box_y, R.half_box_y); }
        return make_double2(dx, dy);
    };
    // unwrapped coordinates relative to particle 0 (update_continuos_pos!):
    // u[p] = sum_{q<p} calc_diff(P[q+1], P[q]); area by the shoelace formula.
    double area2 = 0.0;
    double carry_x = 0.0, carry_y = 0.0;   // u of the first particle of this 32-block
    double prev_last_x = 0.0, prev_last_y = 0.0;
    for (int base = 0; base < n; base += 32) {
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
    const double area = area2 / 2.0;
    if (lane == 0) C.ring_area[g] = area;
    const double k_s = rc.k_spring[t], l_s = rc.l_spring[t];
    const double a0 = n * rc.l_spring[t] / rc.p0[t];
    const double fmod_area = rc.k_area[t] * (area - a0 * a0);
    const double kb = rc.k_bend[t];
    // overdamped active update parameters
    const double theta = C.ring_pol[g];
    double ps, pc;
    sincos(theta, &ps, &pc);
    const double vo = rc.vo[t], mu = rc.mobility[t], dt = R.dt;
    double vcx = 0, vcy = 0;
    for (int p = lane; p < n; p += 32) {
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
        int32_t s = S[p];
        if constexpr (PREC == kPrecFP64) { double2 f = C.fd[s]; fx += f.x; fy += f.y; }
        else { float2 f = C.ff[s]; fx += f.x; fy += f.y; }
        if (R.has_wall_forces) add_wall_forces(C, rep, R, xc.x, xc.y, fx, fy);
        if (!do_update) {
            if constexpr (PREC == kPrecFP64) C.fd[s] = make_double2(fx, fy);
            else C.ff[s] = make_float2((float)fx, (float)fy);
            continue;
        }
        double vx = __dadd_rn(__dmul_rn(vo, pc), __dmul_rn(mu, fx));
        double vy = __dadd_rn(__dmul_rn(vo, ps), __dmul_rn(mu, fy));
        vcx += vx; vcy += vy;
        double x = __dadd_rn(xc.x, __dmul_rn(vx, dt));
        double y = __dadd_rn(xc.y, __dmul_rn(vy, dt));
        double dvx = 0, dvy = 0;
        apply_walls(C, rep, R, rc.inter_dist_eq[t][t] / 2.0, x, y, dvx, dvy, false);
        C.pos_out[s] = make_double2(x, y);
        C.uid_out[s] = C.uid_cur[s];
        C.rep_out[s] = rep;
    }
    if (!do_update) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vcx += __shfl_xor_sync(0xffffffffu, vcx, o);
        vcy += __shfl_xor_sync(0xffffffffu, vcy, o);
    }
    if (lane == 0) {
        vcx /= n;
        vcy /= n;
        double speed = sqrt(vcx * vcx + vcy * vcy);
        double cr = 0.0;
        if (speed != 0) {
            cr = (pc * vcy - ps * vcx) / speed;
            if (fabs(cr) > 1) cr = jsign(cr);
        }
        double nz;
        if (C.noise_mode == MAVI_NOISE_INJECTED) nz = C.noise[R.noise0 + rl];
        else nz = philox_normal(C.seed, (uint64_t)g, (uint64_t)(C.d_step[0] - 1));
        double d_theta = 1 / rc.relax_time[t] * asin(cr) * dt + sqrt(2 * rc.rot_diff[t] * dt) * nz;
        C.ring_pol[g] = theta + d_theta;
    }
}

// ===========================================================================
// user-order staging <-> sorted state
// ===========================================================================
static __global__ void k_gather_user(Ctx C, const double2* __restrict__ pos_user, const double2* __restrict__ vel_user,
                              const double* __restrict__ pol_user) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= C.M) return;
    int32_t u = C.uid_out[s];
    C.pos_out[s] = pos_user[u];
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
        visit((int32_t)R.a0, (int32_t)(R.a0 + R.na));
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

// candidate-pair count per particle (roofline accounting)
static __global__ void k_pair_count(Ctx C, unsigned long long* __restrict__ total) {
    int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c = 0;
    if (s < C.M) {
        const DevRep& R = C.reps[C.rep_cur[s]];
        if (!R.has_chunks) c = R.na - 1;
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
