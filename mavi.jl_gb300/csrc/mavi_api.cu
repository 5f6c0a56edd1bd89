// mavi_api.cu — host runtime and C ABI of libmavi_cuda.so (declared in
// include/mavi_cuda.h). One handle = a batch of independent replicas on one
// GPU, one CUDA stream, all device buffers preallocated at creation.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "mavi_system.cuh"

using namespace mavi;

// ---------------------------------------------------------------------------
// launch sequences shared by both precisions
// ---------------------------------------------------------------------------
// Histogram of the *_out state; with src, the positions are first gathered
// from that user-order buffer (an upload).
static void launch_count(MaviSystem* s, const double2* src = nullptr) {
    record_begin(s, MAVI_KERNEL_BIN_COUNT);
    k_zero_counts<<<nblocks(std::max(s->nscan, s->ntiles)), kBlock, 0, s->stream>>>(s->C.count, s->nscan,
                                                                                  s->C.tile_sum, s->ntiles);
    if (s->prec == MAVI_PREC_FP64) count_fp64(s, 2, src);
    else count_mixed(s, 2, src);
    record_end(s, MAVI_KERNEL_BIN_COUNT);
}

// update_chunks! (src/chunks.jl:150-161): chunk lists from the histogram of the
// *_out state: scan -> scatter -> per-chunk order + permutation into *_cur.
// The scatter takes the counts back to zero as it hands out the places in
// each chunk, and clears the tile sums, so the histogram of the next step
// starts from zero without memset launches.
static void launch_rebin(MaviSystem* s, bool advance) {
    if (!s->counts_valid) launch_count(s);
    record_begin(s, MAVI_KERNEL_BIN_SCAN);
    if (s->tile_offs)   // many tiles: their offsets inside groups of tiles first, a block per group
        k_tile_offsets<<<(unsigned)((s->ntiles + kTileScanThreads - 1) / kTileScanThreads), kTileScanThreads, 0,
                         s->stream>>>(s->C.tile_sum, s->ntiles, s->tile_offs);
    k_scan<<<(unsigned)s->ntiles, kScanThreads, 0, s->stream>>>(s->C.count, s->nscan, s->C.tile_sum, s->C.start,
                                                               s->C.d_step, advance ? 1 : 0, s->tile_offs, 0);
    record_end(s, MAVI_KERNEL_BIN_SCAN);
    record_begin(s, MAVI_KERNEL_BIN_SCATTER);
    k_scatter<<<nblocks(std::max(s->M, s->ntiles)), kBlock, 0, s->stream>>>(s->C);
    record_end(s, MAVI_KERNEL_BIN_SCATTER);
    record_begin(s, MAVI_KERNEL_BIN_SORT);
    if (s->prec == MAVI_PREC_FP64) sort_permute_fp64(s);
    else sort_permute_mixed(s);
    // outside the step, keep the sources' view (current state in *_out, *_cur order)
    if (s->var_rings && !advance) k_out_from_cur<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C);
    record_end(s, MAVI_KERNEL_BIN_SORT);
    s->counts_valid = false;
}

// One whole step; its last kernel leaves the histogram for the next step.
// `due`: replicas whose invasion check falls on this step (eager steps only;
// the check waits for the device).
static int launch_step(MaviSystem* s, const std::vector<int32_t>* due = nullptr) {
    if (s->profiling) {
        cudaEventRecordWithFlags(s->ev.step_a, s->stream, cudaEventRecordExternal);
        s->ev.step_used = 1;
    }
    if (s->var_rings) {
        // step! head: update_cms!, sources and sinks, update_ids!
        // (src/rings/integration.jl:522-526), then the histogram of the active set
        record_begin(s, MAVI_KERNEL_BIN_COUNT);
        if (s->prec == MAVI_PREC_FP64) sources_fp64(s);
        else sources_mixed(s);
        record_end(s, MAVI_KERNEL_BIN_COUNT);
        s->counts_valid = true;
    }
    if (due && !due->empty()) {
        // update_invasions! (src/rings/integration.jl:529-530): after the
        // sources, sinks and update_ids!, before the chunk update and forces
        int rc = run_invasions(s, *due, s->var_rings);
        if (rc) return rc;
    }
    launch_rebin(s, true);
    if (s->prec == MAVI_PREC_FP64) step_body_fp64(s);
    else step_body_mixed(s);
    if (s->profiling) cudaEventRecordWithFlags(s->ev.step_b, s->stream, cudaEventRecordExternal);
    s->counts_valid = !s->var_rings;
    return MAVI_OK;
}

// ---------------------------------------------------------------------------
// host-side configuration helpers
// ---------------------------------------------------------------------------
// particle_radius (src/configs.jl:418-421); rings: minimum over types, as
// get_chunks uses (src/systems.jl:26, src/rings/configs.jl:438-443).
static double particle_radius_of(const MaviReplicaParams& p) {
    const MaviDynamicCfg& d = p.dyn;
    switch (d.kind) {
    case MAVI_DYN_LEN_JONES: return d.sigma * std::pow(2.0, 1.0 / 6.0) / 2;
    case MAVI_DYN_SZABO: return d.r_eq / 2;
    case MAVI_DYN_RUN_TUMBLE: return d.sigma * std::pow(2.0, 1.0 / 6.0) / 2;
    case MAVI_DYN_HARM_TRUNC: return d.dist_eq / 2.0;
    case MAVI_DYN_RINGS: {
        double m = INFINITY;
        for (int t = 0; t < p.rings.num_types; t++) m = std::min(m, p.rings.inter_dist_eq[t][t] / 2.0);
        return m;
    }
    }
    return NAN;
}

static void bbox_of_space(const MaviSpace& sp, double& len, double& h, double& blx, double& bly) {
    if (sp.geometry == MAVI_GEOM_RECTANGLE) {
        len = sp.length; h = sp.height; blx = sp.bl_x; bly = sp.bl_y;
    } else if (sp.geometry == MAVI_GEOM_CIRCLE) {
        double r = sp.radius;
        len = 2 * r; h = 2 * r; blx = sp.cx - r; bly = sp.cy - r;
    } else if (sp.has_bbox) {
        len = sp.bbox_length; h = sp.bbox_height; blx = sp.bbox_bl_x; bly = sp.bbox_bl_y;
    } else {
        double mxx = -INFINITY, mnx = INFINITY, mxy = -INFINITY, mny = INFINITY;
        for (int l = 0; l < sp.num_lines; l++)
            for (int e = 0; e < 2; e++) {
                double x = sp.lines[l][2 * e], y = sp.lines[l][2 * e + 1];
                mxx = std::max(mxx, x); mnx = std::min(mnx, x);
                mxy = std::max(mxy, y); mny = std::min(mny, y);
            }
        len = mxx - mnx; h = mxy - mny; blx = mnx; bly = mny;
    }
}

// get_bounding_box incl. the ManyGeometries fold (src/configs.jl:68-77, 188-229)
static void bbox_of(const MaviReplicaParams& p, double& len, double& h, double& blx, double& bly) {
    bbox_of_space(p.spaces[0], len, h, blx, bly);
    for (int k = 1; k < p.num_spaces; k++) {
        double l2, h2, x2, y2;
        bbox_of_space(p.spaces[k], l2, h2, x2, y2);
        double max_x = std::max(blx + len, x2 + l2), max_y = std::max(bly + h, y2 + h2);
        double min_x = std::min(blx, x2), min_y = std::min(bly, y2);
        h = max_y - min_y; len = max_x - min_x; blx = min_x; bly = min_y;
    }
}

// Chunk grid of one replica with the same arithmetic as mavi_create (bounding
// box, chunk sides, capacity src/chunks.jl:32-34); used by the
// allocation-free chunk-list entry point (mavi_noalloc.cu).
__attribute__((visibility("hidden"))) void replica_chunk_grid(const MaviReplicaParams& p, DevRep& R) {
    R.radius = particle_radius_of(p);
    bbox_of(p, R.bb_len, R.bb_h, R.bb_blx, R.bb_bly);
    R.has_chunks = 1;
    R.rows = p.chunk_rows;
    R.cols = p.chunk_cols;
    R.chunk_l = R.bb_len / R.cols;
    R.chunk_h = R.bb_h / R.rows;
    double nc = (std::ceil(0.5 * R.chunk_l / R.radius) + 1) * (std::ceil(0.5 * R.chunk_h / R.radius) + 1);
    R.cap = (int32_t)std::ceil(nc * 2);
}

// Real particles of a replica (rings: FixRingsIds p_ids, src/rings/states.jl:46-62).
static int64_t active_count(const MaviReplicaParams& p, const int32_t* types) {
    if (p.state_kind != MAVI_STATE_RINGS) return p.num_particles;
    int64_t a = 0;
    for (int r = 0; r < p.rings.num_rings; r++) {
        int t = types ? types[r] - 1 : 0;
        a += p.rings.num_particles[t];
    }
    return a;
}

static int validate(MaviSystem* s, const MaviReplicaParams& p, int idx, const int32_t* types) {
    if (p.num_particles < 1) return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: num_particles must be >= 1", idx);
    if (p.num_spaces < 1 || p.num_spaces > MAVI_MAX_SPACES)
        return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: num_spaces must be in 1..%d", idx, MAVI_MAX_SPACES);
    if (!(p.dt > 0)) return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: dt must be > 0", idx);
    bool sl = p.state_kind == MAVI_STATE_SECOND_LAW, sp_ = p.state_kind == MAVI_STATE_SELF_PROPELLED,
         rg = p.state_kind == MAVI_STATE_RINGS;
    switch (p.step_kind) {
    case MAVI_STEP_NEWTON:
        if (!sl) return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: newton_step! needs a SecondLawState", idx);
        if (p.dyn.kind == MAVI_DYN_RINGS) return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: rings need the rings step", idx);
        break;
    case MAVI_STEP_OVERDAMPED:
        if (!(sl || sp_))
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: overdamped step needs a SecondLaw or SelfPropelled state", idx);
        if (p.dyn.kind == MAVI_DYN_RINGS) return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: rings need the rings step", idx);
        break;
    case MAVI_STEP_SZABO:
        if (!sp_ || p.dyn.kind != MAVI_DYN_SZABO)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: szabo_step! needs SelfPropelledState + SzaboCfg", idx);
        break;
    case MAVI_STEP_RTP:
        if (!sp_ || p.dyn.kind != MAVI_DYN_RUN_TUMBLE)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: rtp_step! needs SelfPropelledState + RunTumbleCfg", idx);
        break;
    case MAVI_STEP_RINGS:
        if (!rg || p.dyn.kind != MAVI_DYN_RINGS)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: rings step needs RingsState + RingsCfg", idx);
        break;
    default:
        return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: unknown step kind %d", idx, p.step_kind);
    }
    if (rg) {
        const MaviRingsCfg& rc = p.rings;
        if (rc.num_types < 1 || rc.num_types > MAVI_MAX_TYPES)
            return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: num_types must be in 1..%d", idx, MAVI_MAX_TYPES);
        if (rc.num_rings < 1 || rc.nmax < 3 || (int64_t)rc.num_rings * rc.nmax != p.num_particles)
            return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: num_particles must equal nmax*num_rings", idx);
        if (rc.nmax > kRingMax)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: rings with more than %d particles", idx, kRingMax);
        for (int t = 0; t < rc.num_types; t++)
            if (rc.num_particles[t] < 3 || rc.num_particles[t] > rc.nmax)
                return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: ring type %d size out of range", idx, t + 1);
        if (types)
            for (int r = 0; r < rc.num_rings; r++)
                if (types[r] < 1 || types[r] > rc.num_types)
                    return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: ring %d has type %d", idx, r, types[r]);
    }
    for (int k = 0; k < p.num_spaces; k++) {
        const MaviSpace& sp = p.spaces[k];
        if (sp.geometry == MAVI_GEOM_LINES && (sp.num_lines < 1 || sp.num_lines > MAVI_MAX_LINES))
            return fail(s, MAVI_ERR_INVALID_ARG, "replica %d: num_lines must be in 1..%d", idx, MAVI_MAX_LINES);
        if (sp.wall == MAVI_WALL_RIGID && !sl)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: RigidWalls reflect velocities; the state has none", idx);
        if (sp.wall == MAVI_WALL_RIGID && sp.geometry == MAVI_GEOM_LINES)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: RigidWalls on LinesCfg is not defined", idx);
        if (sp.wall == MAVI_WALL_PERIODIC && sp.geometry == MAVI_GEOM_LINES)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: PeriodicWalls on LinesCfg is not defined", idx);
        if (sp.wall == MAVI_WALL_POTENTIAL && sp.geometry == MAVI_GEOM_RECTANGLE)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: PotentialWalls need a CircleCfg or LinesCfg", idx);
        if (sp.wall == MAVI_WALL_SLIPPERY && sp.geometry == MAVI_GEOM_RECTANGLE)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: SlipperyWalls need a CircleCfg or LinesCfg", idx);
    }
    bool chunks = p.chunk_cols > 0 && p.chunk_rows > 0;
    if (chunks) {
        if (p.spaces[0].wall == MAVI_WALL_PERIODIC && (p.chunk_cols < 3 || p.chunk_rows < 3))
            return fail(s, MAVI_ERR_UNSUPPORTED,
                        "replica %d: periodic chunk grid needs >= 3 rows and cols (the reference's stencil "
                        "repeats chunks below that)", idx);
        if (p.spaces[0].wall != MAVI_WALL_PERIODIC && p.chunk_cols < 2)
            return fail(s, MAVI_ERR_UNSUPPORTED, "replica %d: open chunk grid needs >= 2 columns", idx);
    }
    return MAVI_OK;
}

// check_inside (src/space_checks.jl:9-37, 53-60): the circle test ignores
// the centre, as the reference does.
static bool outside_space(const MaviReplicaParams& p, const double* pos, const int32_t* types) {
    if (p.num_spaces != 1) return false;
    const MaviSpace& sp = p.spaces[0];
    for (int64_t i = 0; i < p.num_particles; i++) {
        if (p.state_kind == MAVI_STATE_RINGS) {
            int64_t ring = i / p.rings.nmax, k = i % p.rings.nmax;
            int t = types ? types[ring] - 1 : 0;
            if (k >= p.rings.num_particles[t]) continue;
        }
        double x = pos[2 * i], y = pos[2 * i + 1];
        if (sp.geometry == MAVI_GEOM_RECTANGLE) {
            if (x < sp.bl_x || y < sp.bl_y || x > sp.bl_x + sp.length || y > sp.bl_y + sp.height) return true;
        } else if (sp.geometry == MAVI_GEOM_CIRCLE) {
            if (x * x + y * y > sp.radius * sp.radius) return true;
        }
    }
    return false;
}

// Pair-law constants in the packing the kernels expect (mavi_device.cuh).
static void pack_pair_params(const MaviDynamicCfg& d, DevRep& R) {
    for (int k = 0; k < 8; k++) R.pd[k] = 0;
    switch (d.kind) {
    case MAVI_DYN_HARM_TRUNC:
        R.pd[0] = d.k_rep; R.pd[1] = d.k_atr; R.pd[2] = 1.0 / d.dist_eq; R.pd[3] = d.dist_eq * d.dist_eq;
        R.pd[4] = d.dist_max * d.dist_max; R.pd[5] = d.dist_eq; R.pd[6] = d.dist_max;
        break;
    case MAVI_DYN_LEN_JONES:
    case MAVI_DYN_RUN_TUMBLE: {
        double s6 = std::pow(d.sigma, 6.0), s12 = std::pow(d.sigma, 12.0);
        R.pd[0] = 48 * d.epsilon * s12; R.pd[1] = 24 * d.epsilon * s6;
        double cut = std::pow(2.0, 1.0 / 6.0) * d.sigma;
        R.pd[2] = cut * cut;
        R.pd[4] = 4 * d.epsilon; R.pd[5] = s12; R.pd[6] = s6; R.pd[7] = cut * cut;
        break;
    }
    case MAVI_DYN_SZABO:
        R.pd[0] = d.k_rep / (d.r_max - d.r_eq); R.pd[1] = d.k_adh / d.r_eq; R.pd[2] = d.r_eq; R.pd[3] = d.r_max;
        R.pd[4] = d.r_max * d.r_max;
        break;
    }
    for (int k = 0; k < 8; k++) R.pf[k] = (float)R.pd[k];
}


// Fixed-point geometry of the mixed form: unit u = max(chunk_l, chunk_h)/2^28,
// chunk and box sizes in units, and when the minimum image may be skipped for
// neighbours that do not wrap (|dr| < 2 chunks + drift <= L/2 needs >= 6
// chunks per side). Walls run for edge-chunk particles only when every space is
// a rigid or periodic rectangle equal to the chunk bounding box and the
// particle radius is below a chunk.
static void set_fixed_point(const MaviReplicaParams& p, DevRep& R) {
    double u = std::max(R.chunk_l, R.chunk_h) / (double)(1 << kFixBits);
    R.inv_u = 1.0 / u;
    R.u_f = (float)u;
    R.u2_f = (float)(u * u);
    R.u2_d = u * u;
    // centre of chunk (0, 0): the origin of the integer coordinates
    // (col * sx + offset, -row * sy + offset) in units
    R.cx0 = R.bb_blx + 0.5 * R.chunk_l;
    R.cy0 = R.bb_bly + R.bb_h - 0.5 * R.chunk_h;
    // float pre-check of a single PotentialWalls circle with the truncated
    // harmonic potential (the wall force vanishes away from the circle)
    R.wall_precheck = 0;
    if (p.num_spaces == 1 && p.spaces[0].wall == MAVI_WALL_POTENTIAL && p.spaces[0].geometry == MAVI_GEOM_CIRCLE &&
        p.spaces[0].pot_kind == MAVI_DYN_HARM_TRUNC &&
        (p.spaces[0].pot_mode == MAVI_POTMODE_INSIDE || p.spaces[0].pot_mode == MAVI_POTMODE_REPULSION)) {
        const MaviSpace& sp = p.spaces[0];
        const double lo = sp.radius - sp.pot_params[3], hi = sp.radius + sp.pot_params[3];
        if (lo > 0) {
            R.wall_precheck = sp.pot_mode == MAVI_POTMODE_INSIDE ? 1 : 2;
            R.wall_cx_u = std::llround((sp.cx - R.cx0) * R.inv_u);
            R.wall_cy_u = std::llround((sp.cy - R.cy0) * R.inv_u);
            // margins far above the float rounding of the test (relative 1e-7)
            R.wall_lo2_u = (float)(lo * R.inv_u * lo * R.inv_u * (1.0 - 1e-4));
            R.wall_hi2_u = (float)(hi * R.inv_u * hi * R.inv_u * (1.0 + 1e-4));
            // the FP32 wall force of the mixed form: radius^2 in units^2 as an
            // integer (its rounding, <= 0.5 units^2, moves the wall by ~1e-11 units)
            const long double Ru = (long double)sp.radius * (long double)R.inv_u;
            const __int128 R2 = (__int128)(Ru * Ru + 0.5L);
            R.wall_R2_hi = (long long)(R2 >> 64);
            R.wall_R2_lo = (unsigned long long)R2;
            R.wall_Ru_f = (float)Ru;
            R.wall_krep_f = (float)sp.pot_params[0];
            R.wall_katr_f = (float)sp.pot_params[1];
            R.wall_deq_f = (float)sp.pot_params[2];
            R.wall_dmax_f = (float)sp.pot_params[3];
        }
    }
    R.sx_u = std::llround(R.chunk_l / u);
    R.sy_u = std::llround(R.chunk_h / u);
    R.bx_u = R.sx_u * R.cols;
    R.by_u = R.sy_u * R.rows;
    R.half_bx_u = R.bx_u / 2;
    R.half_by_u = R.by_u / 2;
    R.sx_i = (int32_t)R.sx_u;
    R.sy_i = (int32_t)R.sy_u;
    R.half_sx_i = R.sx_i / 2;
    R.half_sy_i = R.sy_i / 2;
    // the minimum image only matters for |dr| > L/2 with dr <= ~2 chunks,
    // i.e. grids of < 6 chunks per side, whose box fits int32 units
    const long long lim = (1ll << 31) - 1;
    R.bx_i = (int32_t)std::min(R.bx_u, lim);
    R.by_i = (int32_t)std::min(R.by_u, lim);
    R.half_bx_i = (int32_t)std::min(R.half_bx_u, lim);
    R.half_by_i = (int32_t)std::min(R.half_by_u, lim);
    R.mi_small = (!R.has_chunks || R.rows < 6 || R.cols < 6) ? 1 : 0;
    bool edge_only = R.has_chunks && p.num_spaces == 1 && R.radius < std::min(R.chunk_l, R.chunk_h);
    const MaviSpace& sp = p.spaces[0];
    edge_only = edge_only && sp.geometry == MAVI_GEOM_RECTANGLE &&
                (sp.wall == MAVI_WALL_RIGID || sp.wall == MAVI_WALL_PERIODIC) && sp.length == R.bb_len &&
                sp.height == R.bb_h && sp.bl_x == R.bb_blx && sp.bl_y == R.bb_bly;
    R.walls_edge_only = edge_only ? 1 : 0;
    if (p.dyn.kind == MAVI_DYN_LEN_JONES || p.dyn.kind == MAVI_DYN_RUN_TUMBLE) {
        // 2^k ~ (sigma/u)^2 so that the scaled d^2 is O(1) at contact
        int k = (int)std::lround(std::log2(p.dyn.sigma * p.dyn.sigma / (u * u)));
        double g = std::ldexp(u * u, k);
        double ad = R.pd[0] * u * std::pow(g, -7.0), bd = R.pd[1] * u * std::pow(g, -4.0);
        R.lj_sk = (float)std::ldexp(1.0, -k);
        R.lj_ah = (float)ad;
        R.lj_al = (float)(ad - (double)R.lj_ah);
        R.lj_bh = (float)bd;
        R.lj_bl = (float)(bd - (double)R.lj_bh);
        const double rn = kLjSplitSigmas * p.dyn.sigma / u;
        R.lj_near2 = (float)(rn * rn);
    }
}

// Fixed-point pair constants (units of the replica) per (type, type).
static void fill_fix_pairs(const MaviReplicaParams& p, const DevRep& R, FixPair* out) {
    double inv_u = R.inv_u;
    auto sq = [&](double len) { double v = len * inv_u; return (unsigned long long)std::llround(v * v); };
    for (int t = 0; t < MAVI_MAX_TYPES * MAVI_MAX_TYPES; t++) out[t] = FixPair{};
    auto bands = [](FixPair& f) {
        f.cut2_hi = (float)((double)f.cut2 * (1.0 + 1e-6));
        f.cut2_lo = (float)((double)f.cut2 * (1.0 - 1e-6));
    };
    const MaviDynamicCfg& d = p.dyn;
    FixPair f{};
    switch (d.kind) {
    case MAVI_DYN_HARM_TRUNC:
        f.cut2 = sq(d.dist_max); f.eq2 = (long long)sq(d.dist_eq); f.eq = (float)(d.dist_eq * inv_u);
        f.k_rep = (float)d.k_rep; f.k_atr = (float)d.k_atr;
        bands(f);
        out[0] = f;
        break;
    case MAVI_DYN_SZABO:
        f.cut2 = sq(d.r_max); f.eq2 = (long long)sq(d.r_eq); f.eq = (float)(d.r_eq * inv_u);
        f.k_rep = (float)(d.k_rep / (d.r_max - d.r_eq)); f.k_atr = (float)(d.k_adh / d.r_eq);
        bands(f);
        out[0] = f;
        break;
    case MAVI_DYN_RUN_TUMBLE:
        f.cut2 = sq(std::pow(2.0, 1.0 / 6.0) * d.sigma);
        bands(f);
        out[0] = f;
        break;
    case MAVI_DYN_RINGS:
        for (int a = 0; a < p.rings.num_types; a++)
            for (int b = 0; b < p.rings.num_types; b++) {
                FixPair g{};
                g.cut2 = sq(p.rings.inter_dist_max[a][b]);
                g.eq2 = (long long)sq(p.rings.inter_dist_eq[a][b]);
                g.eq = (float)(p.rings.inter_dist_eq[a][b] * inv_u);
                g.k_rep = (float)p.rings.inter_k_rep[a][b];
                g.k_atr = (float)p.rings.inter_k_atr[a][b];
                bands(g);
                out[a * MAVI_MAX_TYPES + b] = g;
            }
        break;
    }
}

static int check_device_error(MaviSystem* s);
int mavi::device_error_status(MaviSystem* s) { return check_device_error(s); }

static int check_device_error(MaviSystem* s) {
    DevError e{};
    CUDA_TRY(s, cudaMemcpyAsync(&e, s->C.err, sizeof(DevError), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    if (e.code == 0) return MAVI_OK;
    int32_t uid = -1;
    if (e.slot >= 0 && e.slot < s->M) cudaMemcpy(&uid, s->C.uid_out + e.slot, sizeof(int32_t), cudaMemcpyDeviceToHost);
    DevError z{};
    cudaMemcpy(s->C.err, &z, sizeof(DevError), cudaMemcpyHostToDevice);
    switch (e.code) {
    case MAVI_ERR_OUT_OF_GRID:
        return fail(s, e.code, "particle %d left the chunk grid (row*1000003+col = %lld)", uid, (long long)e.aux);
    case MAVI_ERR_CHUNK_OVERFLOW:
        return fail(s, e.code, "chunk %lld holds more particles than its capacity (particle %d)", (long long)e.aux, uid);
    case MAVI_ERR_NONFINITE:
        return fail(s, e.code, "particle %d has a non-finite position", uid);
    case MAVI_ERR_FORCE_RANGE:
        return fail(s, e.code,
                    "a pair force on particle %d reached 2^22 (particles closer than ~0.37 sigma); the mixed form's "
                    "fixed-point force sums cannot hold it", uid);
    case MAVI_ERR_OFFSET_RANGE:
        return fail(s, e.code,
                    "particle %d is more than 1.5 chunks from the centre of its chunk (it moved more than a chunk "
                    "in one step); the mixed form's fixed-point offsets cannot represent it", uid);
    }
    return fail(s, e.code, "device error %d", e.code);
}

static void drop_graph(MaviSystem* s) {
    if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
    if (s->graph) { cudaGraphDestroy(s->graph); s->graph = nullptr; }
}

// Captures one whole step (assuming a valid histogram, which every step
// leaves behind). With profiling on, the event records are captured too and
// replayed with the graph.
static int ensure_graph(MaviSystem* s) {
    if (s->graph_exec && s->graph_profile_mode == s->profile_mode) return MAVI_OK;
    drop_graph(s);
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++) s->ev.used[k] = 0;
    CUDA_TRY(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    s->counts_valid = true;
    (void)launch_step(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &s->graph);
    if (e != cudaSuccess) return fail(s, MAVI_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    CUDA_TRY(s, cudaGraphInstantiate(&s->graph_exec, s->graph, 0));
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++) {
        s->graph_ev_used[k] = s->ev.used[k];
        s->ev.used[k] = 0;
    }
    s->graph_step_used = s->ev.step_used;
    s->ev.step_used = 0;
    s->graph_profile_mode = s->profile_mode;
    return MAVI_OK;
}

// Pair-gather autotuner: times a force-only pass (it changes no state) with
// each gather and keeps the fastest for the handle's lifetime; graphs are
// captured afterwards and use it. The gathers add the same terms in the same
// order, so the choice never changes results, only speed.
// Pass mode `mode` (MaviOptions.gather_mode 0..7) on the handle: the device
// gather, and the lanes per particle of the mixed short-range passes.
static void set_pass_mode(MaviSystem* s, int mode) {
    s->lanes = mode == kGatherLanes2 ? 2 : (mode == kGatherLanes4 ? 4 : 1);
    s->C.gather_mode = s->lanes > 1 ? 2 : mode;
}
static int pass_mode_of(const MaviSystem* s) {
    return s->lanes == 2 ? kGatherLanes2 : (s->lanes == 4 ? kGatherLanes4 : s->C.gather_mode);
}
static bool lanes_possible(const MaviSystem* s) {
    return s->prec == MAVI_PREC_MIXED && (s->dyn == MAVI_DYN_HARM_TRUNC || s->dyn == MAVI_DYN_SZABO);
}
static bool split_possible(const MaviSystem* s) {
    return s->prec == MAVI_PREC_MIXED && s->dyn == MAVI_DYN_LEN_JONES;
}

static int autotune_gather(MaviSystem* s) {
    cudaEvent_t a = nullptr, b = nullptr;
    CUDA_TRY(s, cudaEventCreate(&a));
    CUDA_TRY(s, cudaEventCreate(&b));
    float best = INFINITY;
    int best_mode = 0;
    for (int mode = 0; mode < kNumPassModes; mode++) {
        // tiles: mixed Lennard-Jones / WCA with chunks; lanes: mixed short-range
        // laws; split: mixed Lennard-Jones
        if ((mode == kGatherTiles || mode == kGatherTilesQueue) && !s->tiles) continue;
        if ((mode == kGatherLanes2 || mode == kGatherLanes4) && !lanes_possible(s)) continue;
        if (mode == kGatherSplit && !split_possible(s)) continue;
        set_pass_mode(s, mode);
        for (int w = 0; w < 2; w++) {
            if (s->prec == MAVI_PREC_FP64) forces_only_fp64(s, 0);
            else forces_only_mixed(s, 0);
        }
        cudaEventRecord(a, s->stream);
        for (int r = 0; r < 5; r++) {
            if (s->prec == MAVI_PREC_FP64) forces_only_fp64(s, 0);
            else forces_only_mixed(s, 0);
        }
        cudaEventRecord(b, s->stream);
        cudaError_t e = cudaEventSynchronize(b);
        float ms = INFINITY;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
        // modes 0..2 give the same bits; a mode that changes them (tiles,
        // lanes, split) must beat the fastest of those by 10 %, so that timing noise
        // cannot make two runs of the same system differ
        const float need = mode < kNumGatherModes ? best : best * 0.9f;
        if (ms < need) {
            best = ms;
            best_mode = mode;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    set_pass_mode(s, best_mode);
    CUDA_TRY(s, cudaGetLastError());
    return check_device_error(s);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int mavi_abi_version(void) { return MAVI_ABI_VERSION; }

const char* mavi_status_string(int st) {
    switch (st) {
    case MAVI_OK: return "ok";
    case MAVI_ERR_INVALID_ARG: return "invalid argument";
    case MAVI_ERR_CUDA: return "CUDA error";
    case MAVI_ERR_OUT_OF_GRID: return "particle outside the chunk grid";
    case MAVI_ERR_CHUNK_OVERFLOW: return "chunk over capacity";
    case MAVI_ERR_NONFINITE: return "non-finite position";
    case MAVI_ERR_OUTSIDE_SPACE: return "particles outside the space";
    case MAVI_ERR_UNSUPPORTED: return "unsupported configuration";
    case MAVI_ERR_NO_DEVICE: return "no CUDA device";
    case MAVI_ERR_NOISE_MISSING: return "noise not supplied";
    case MAVI_ERR_NEIGHBOR_OVERFLOW: return "neighbour list overflow";
    case MAVI_ERR_OFFSET_RANGE: return "particle beyond the mixed form's fixed-point offset range";
    case MAVI_ERR_FORCE_RANGE: return "pair force beyond the mixed form's fixed-point force range";
    }
    return "unknown status";
}

int mavi_destroy(MaviSystem* s) {
    if (!s) return MAVI_OK;
    drop_graph(s);
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++)
        for (int u = 0; u < 4; u++) {
            if (s->ev.a[k][u]) cudaEventDestroy(s->ev.a[k][u]);
            if (s->ev.b[k][u]) cudaEventDestroy(s->ev.b[k][u]);
        }
    if (s->ev.step_a) cudaEventDestroy(s->ev.step_a);
    if (s->ev.step_b) cudaEventDestroy(s->ev.step_b);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void* p : s->allocs) cudaFree(p);
    if (s->series) cudaFree(s->series);
    if (s->hist) cudaFree(s->hist);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return MAVI_OK;
}

int mavi_create(const MaviOptions* opt, int32_t num_replicas, const MaviReplicaParams* replicas,
                const double* pos, const double* vel, const double* pol, const int32_t* ring_types,
                MaviSystem** out) {
    if (!out) return MAVI_ERR_INVALID_ARG;
    *out = nullptr;
    if (!opt || !replicas || num_replicas < 1 || !pos) return MAVI_ERR_INVALID_ARG;
    MaviSystem* s = new MaviSystem();
    s->opt = *opt;
    s->R = num_replicas;
    s->params.assign(replicas, replicas + num_replicas);
    s->prec = opt->precision;
    if ((s->prec != MAVI_PREC_FP64 && s->prec != MAVI_PREC_MIXED) || opt->gather_mode < -1 ||
        opt->gather_mode >= kNumPassModes) {
        delete s;
        return MAVI_ERR_INVALID_ARG;
    }
    const MaviReplicaParams& p0 = replicas[0];
    s->dyn = p0.dyn.kind;
    s->step_kind = p0.step_kind;
    s->state_kind = p0.state_kind;
    // SecondLaw states carry velocities; the overdamped step may run on
    // positions only (vel == NULL), which spares moving dead velocities.
    s->has_vel = s->state_kind == MAVI_STATE_SECOND_LAW && vel != nullptr;
    s->has_pol = s->state_kind == MAVI_STATE_SELF_PROPELLED;
    s->is_rings = s->state_kind == MAVI_STATE_RINGS;
    if (s->state_kind == MAVI_STATE_SECOND_LAW && !vel && s->step_kind != MAVI_STEP_OVERDAMPED) {
        delete s;
        return MAVI_ERR_INVALID_ARG;
    }
    for (int r = 0; r < num_replicas && !s->has_vel; r++)
        for (int k = 0; k < replicas[r].num_spaces; k++)
            if (replicas[r].spaces[k].wall == MAVI_WALL_RIGID) {
                delete s;
                return MAVI_ERR_UNSUPPORTED;   // rigid walls reflect velocities
            }
    if ((s->has_pol || s->is_rings) && !pol) { delete s; return MAVI_ERR_INVALID_ARG; }

    // per-replica layout
    int64_t slot0 = 0, a0 = 0, c0 = 0, ring0 = 0, noise0 = 0;
    const int32_t* types_cursor = ring_types;
    int st = MAVI_OK;
    for (int r = 0; r < num_replicas; r++) {
        const MaviReplicaParams& p = replicas[r];
        if (p.dyn.kind != s->dyn || p.step_kind != s->step_kind || p.state_kind != s->state_kind) {
            st = fail(s, MAVI_ERR_UNSUPPORTED, "all replicas of a handle must share state, dynamics and step kinds");
            break;
        }
        const int32_t* types = s->is_rings ? types_cursor : nullptr;
        if ((st = validate(s, p, r, types))) break;
        if (outside_space(p, pos + 2 * slot0, types)) {
            st = fail(s, MAVI_ERR_OUTSIDE_SPACE, "replica %d: particles outside the space", r);
            break;
        }
        DevRep R{};
        R.slot0 = slot0;
        R.nslots = p.num_particles;
        R.a0 = a0;
        R.na = active_count(p, types);
        R.c0 = c0;
        R.ring0 = ring0;
        R.noise0 = noise0;
        R.dt = p.dt;
        R.num_spaces = p.num_spaces;
        R.radius = particle_radius_of(p);
        bbox_of(p, R.bb_len, R.bb_h, R.bb_blx, R.bb_bly);
        R.has_chunks = p.chunk_cols > 0 && p.chunk_rows > 0;
        if (R.has_chunks) {
            R.rows = p.chunk_rows;
            R.cols = p.chunk_cols;
            R.chunk_l = R.bb_len / R.cols;
            R.chunk_h = R.bb_h / R.rows;
            // capacity (src/chunks.jl:32-34)
            double nc = (std::ceil(0.5 * R.chunk_l / R.radius) + 1) * (std::ceil(0.5 * R.chunk_h / R.radius) + 1);
            R.cap = (int32_t)std::ceil(nc * 2);
        } else {
            R.rows = 1; R.cols = 1;
            R.chunk_l = R.bb_len; R.chunk_h = R.bb_h;
            R.cap = 1 << 30;
        }
        R.periodic = p.spaces[0].wall == MAVI_WALL_PERIODIC;
        R.min_image = p.spaces[0].wall == MAVI_WALL_PERIODIC && p.spaces[0].geometry == MAVI_GEOM_RECTANGLE;
        R.box_x = p.spaces[0].length;
        R.box_y = p.spaces[0].height;
        R.half_box_x = R.box_x / 2;
        R.half_box_y = R.box_y / 2;
        R.chunk_lf = (float)R.chunk_l; R.chunk_hf = (float)R.chunk_h;
        R.box_xf = (float)R.box_x; R.box_yf = (float)R.box_y;
        R.half_box_xf = (float)R.half_box_x; R.half_box_yf = (float)R.half_box_y;
        for (int k = 0; k < p.num_spaces; k++) {
            if (p.spaces[k].wall == MAVI_WALL_POTENTIAL) R.has_wall_forces = 1;
            else R.has_walls = 1;
        }
        pack_pair_params(p.dyn, R);
        set_fixed_point(p, R);
        R.mobility = p.dyn.mobility;
        R.mdt = p.dyn.mobility * p.dt;
        R.mdt_f = (float)R.mdt;
        R.vo = p.dyn.vo;
        R.relax_time = p.dyn.relax_time;
        R.rot_diff = p.dyn.rot_diff;
        R.tumble_rate = p.dyn.tumble_rate;
        if (s->is_rings) {
            R.num_rings = p.rings.num_rings;
            R.nmax = p.rings.nmax;
            for (int t = 0; t < p.rings.num_types && t < MAVI_MAX_TYPES; t++) {
                // area0 (src/rings/configs.jl:221-226)
                const double a0 = p.rings.num_particles[t] * p.rings.l_spring[t] / p.rings.p0[t];
                R.ring_a0sq[t] = a0 * a0;
                // mixed form: 2 A0 / u^2 as an integer (the area is summed exactly in units^2)
                const long double uu = (long double)R.u2_d;
                const __int128 iv = (__int128)(2.0L * (long double)R.ring_a0sq[t] / uu + 0.5L);
                R.ring_a0x2_hi[t] = (long long)(iv >> 64);
                R.ring_a0x2_lo[t] = (unsigned long long)iv;
                R.ring_karea_f[t] = (float)(p.rings.k_area[t] * R.u2_d * 0.5);
                R.ring_ks_f[t] = (float)p.rings.k_spring[t];
                R.ring_ls_f[t] = (float)p.rings.l_spring[t];
                const long double ls2 = (long double)p.rings.l_spring[t] * p.rings.l_spring[t] / uu;
                R.ring_ls2_u[t] = ls2 < 9.0e18L ? (long long)(ls2 + 0.5L) : -1;
                R.ring_ls2_d[t] = p.rings.l_spring[t] * p.rings.l_spring[t];
                const double ku = p.rings.k_spring[t] * std::sqrt(R.u2_d), lu = p.rings.l_spring[t] / std::sqrt(R.u2_d);
                R.ring_ku_h[t] = (float)ku; R.ring_ku_l[t] = (float)(ku - (double)R.ring_ku_h[t]);
                R.ring_lu_h[t] = (float)lu; R.ring_lu_l[t] = (float)(lu - (double)R.ring_lu_h[t]);
                R.ring_kb_f[t] = (float)p.rings.k_bend[t];
                R.ring_vo_f[t] = (float)p.rings.vo[t];
                R.ring_mu_f[t] = (float)p.rings.mobility[t];
                R.ring_dt_tau_f[t] = (float)(p.dt / p.rings.relax_time[t]);
                R.ring_noise_amp[t] = std::sqrt(2 * p.rings.rot_diff[t] * p.dt);
            }
        }
        R.dt_f = (float)p.dt;
        s->reps_h.push_back(R);
        s->rep_active.push_back(R.na);
        slot0 += p.num_particles;
        a0 += R.na;
        c0 += (int64_t)R.rows * R.cols;
        if (s->is_rings) {
            ring0 += p.rings.num_rings;
            if (types_cursor) types_cursor += p.rings.num_rings;
        }
        int64_t nz = 0;
        if (s->step_kind == MAVI_STEP_SZABO) nz = p.num_particles;
        else if (s->step_kind == MAVI_STEP_RTP) nz = 2 * p.num_particles;
        else if (s->step_kind == MAVI_STEP_RINGS) nz = p.rings.num_rings;
        noise0 += nz;
    }
    if (st) {
        std::string msg = s->last_error;
        delete s;
        fprintf(stderr, "mavi_create: %s\n", msg.c_str());
        return st;
    }
    s->Nslots = slot0;
    s->M = a0;
    s->Ctot = c0;
    s->total_rings = ring0;
    s->noise_count = noise0;
    // rings handles scan one more chunk: the parking chunk of inactive rings
    s->nscan = s->Ctot + (s->is_rings ? 1 : 0);
    s->noise_base = s->noise_count;
    s->ntiles = (s->nscan + kScanTile - 1) / kScanTile;
    if (s->Nslots >= (1ll << 31) || s->M >= (1ll << 31) || s->Ctot >= (1ll << 31) - 1) {
        delete s;
        return MAVI_ERR_UNSUPPORTED;
    }
    s->num_steps.assign(num_replicas, 0);
    s->time.assign(num_replicas, 0.0);

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        delete s;
        return MAVI_ERR_NO_DEVICE;
    }
    if (cudaSetDevice(opt->device) != cudaSuccess) {
        delete s;
        return MAVI_ERR_NO_DEVICE;
    }
    auto bail = [&](int code) {
        fprintf(stderr, "mavi_create: %s\n", s->last_error.c_str());
        mavi_destroy(s);
        return code;
    };
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(s, MAVI_ERR_CUDA, "stream creation failed"));

    Ctx& C = s->C;
    const int64_t M = s->M, N = s->Nslots;
#define ALLOC(ptr, n) \
    if (dalloc(s, &(ptr), (n)) != cudaSuccess) return bail(fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for %s", #ptr))
    ALLOC(C.pos_cur, M); ALLOC(C.pos_mid, M); ALLOC(C.pos_out, M);
    if (s->has_vel) { ALLOC(C.vel_cur, M); ALLOC(C.vel_out, M); }
    if (s->has_pol) { ALLOC(C.pol_cur, M); ALLOC(C.pol_out, M); }
    if (s->prec == MAVI_PREC_MIXED) { ALLOC(C.off_cur, M); ALLOC(C.off_mid, M); ALLOC(C.off_out, M); ALLOC(C.ff, M); }
    else { ALLOC(C.fd, M); }
    if (s->step_kind == MAVI_STEP_NEWTON) {
        if (s->prec == MAVI_PREC_MIXED) { ALLOC(C.fold_f, M); } else { ALLOC(C.fold_d, M); }
    }
    ALLOC(C.uid_cur, M); ALLOC(C.uid_out, M); ALLOC(C.rep_cur, M); ALLOC(C.rep_out, M);
    ALLOC(C.cell_cur, M); ALLOC(C.cell_out, M); ALLOC(C.src_of, M);
    ALLOC(C.key_of, M); ALLOC(C.cell_at, M);
    if (s->ntiles > kScanDirectTiles)   // offsets inside groups + one total per group
        ALLOC(s->tile_offs, s->ntiles + (s->ntiles + kTileScanThreads - 1) / kTileScanThreads);
    // no chunk guess before the first histogram
    if (cudaMemset(C.cell_out, 0xff, sizeof(int32_t) * M) != cudaSuccess)
        return bail(fail(s, MAVI_ERR_CUDA, "cudaMemset failed for cell_out"));
    ALLOC(C.slot_of, N);
    ALLOC(C.count, s->nscan); ALLOC(C.start, s->nscan + 1);
    ALLOC(C.tile_sum, s->ntiles);
    int32_t* ring_types_d = nullptr;
    int32_t* ring_rep_d = nullptr;
    if (s->is_rings) {
        // packed ring identity per slot when every replica fits the packing
        bool fits = true;
        for (const DevRep& R : s->reps_h) fits = fits && R.nmax <= kRingKeyMaxNmax && R.num_rings <= kRingKeyMaxRings;
        int32_t* rkey_d = nullptr;
        if (fits) { ALLOC(C.rinfo_cur, M); ALLOC(rkey_d, N); }
        C.rkey_user = rkey_d;
        // user-order state and force of the rings update
        ALLOC(C.pos_u, N); ALLOC(C.cell_u, N);
        if (s->prec == MAVI_PREC_MIXED) { ALLOC(C.off_u, N); ALLOC(C.ff_u, N); } else { ALLOC(C.fd_u, N); }
        ALLOC(C.ring_pol, s->total_rings); ALLOC(C.ring_area, s->total_rings); ALLOC(ring_types_d, s->total_rings);
        ALLOC(ring_rep_d, s->total_rings); ALLOC(C.ring_cs, s->total_rings); ALLOC(C.ring_vc, s->total_rings);
    }
    // chunk-centre tables (units of u) for the fast binning check
    std::vector<double> cxu_h, cyu_h;
    for (int r = 0; r < s->R; r++) {
        DevRep& R = s->reps_h[r];
        R.ccol0 = (int64_t)cxu_h.size();
        R.crow0 = (int64_t)cyu_h.size();
        for (int c = 0; c < R.cols; c++) cxu_h.push_back(std::fma((double)c, R.chunk_l, R.cx0) * R.inv_u);
        for (int q = 0; q < R.rows; q++) cyu_h.push_back(std::fma(-(double)q, R.chunk_h, R.cy0) * R.inv_u);
    }
    double *cxu_d = nullptr, *cyu_d = nullptr;
    DevRep* reps_d = nullptr;
    MaviSpace* spaces_d = nullptr;
    MaviRingsCfg* rcfg_d = nullptr;
    FixPair* fix_d = nullptr;
    ALLOC(reps_d, s->R); ALLOC(spaces_d, (int64_t)s->R * MAVI_MAX_SPACES); ALLOC(rcfg_d, s->R);
    ALLOC(cxu_d, (int64_t)cxu_h.size()); ALLOC(cyu_d, (int64_t)cyu_h.size());
    ALLOC(fix_d, (int64_t)s->R * MAVI_MAX_TYPES * MAVI_MAX_TYPES);
    ALLOC(C.err, 1); ALLOC(C.d_step, 1);
    ALLOC(s->pos_user, N); ALLOC(s->f_user, N);
    if (s->has_vel) { ALLOC(s->vel_user, N); }
    if (s->has_pol) { ALLOC(s->pol_user, N); }
    ALLOC(s->ke_t, M); ALLOC(s->pe_t, M); ALLOC(s->ke_r, s->R); ALLOC(s->pe_r, s->R);
    ALLOC(s->d_pairs, 1);
    if (s->noise_count > 0) { ALLOC(s->noise_cur, s->noise_count); }
#undef ALLOC
    C.ring_csf = reinterpret_cast<float2*>(C.ring_cs);
    C.ring_vcf = reinterpret_cast<float2*>(C.ring_vc);
    C.ring_types = ring_types_d;
    C.ring_rep = ring_rep_d;
    C.reps = reps_d;
    C.cxu = cxu_d;
    C.cyu = cyu_d;
    C.spaces = spaces_d;
    C.rcfg = rcfg_d;
    C.fix = fix_d;
    C.M = M;
    C.Ctot = s->Ctot;
    C.park = s->Ctot;
    C.ntiles = s->ntiles;
    C.noise = s->noise_cur;
    C.noise_mode = opt->noise_mode;
    set_pass_mode(s, opt->gather_mode < 0 ? 0 : opt->gather_mode);
    if (s->lanes > 1 && !lanes_possible(s))
        return bail(fail(s, MAVI_ERR_UNSUPPORTED,
                         "gather modes 5 and 6 (lanes) serve the mixed harmonic-truncated and Szabo passes"));
    if (opt->gather_mode == kGatherSplit && !split_possible(s))
        return bail(fail(s, MAVI_ERR_UNSUPPORTED, "gather mode 7 (split) serves the mixed Lennard-Jones passes"));
    C.num_reps = s->R;
    C.seed = opt->seed;

    // Newton's-third-law tiles (mixed Lennard-Jones / WCA, every replica with
    // chunks): square tiles whose window (tile plus a one-chunk halo) holds
    // about 0.85 kTileThreads particles at the replica's mean chunk
    // occupancy, side 2..kTileMaxDim chunks, column-major per replica
    bool tiled = s->prec == MAVI_PREC_MIXED && (s->dyn == MAVI_DYN_LEN_JONES || s->dyn == MAVI_DYN_RUN_TUMBLE);
    for (int r = 0; r < s->R && tiled; r++) tiled = s->reps_h[r].has_chunks != 0;
    if (!tiled && (opt->gather_mode == kGatherTiles || opt->gather_mode == kGatherTilesQueue))
        return bail(fail(s, MAVI_ERR_UNSUPPORTED,
                         "gather modes 3 and 4 (tiles) serve the mixed Lennard-Jones / WCA passes with chunks"));
    if (tiled) {
        std::vector<TileDesc> th;
        for (int r = 0; r < s->R; r++) {
            const DevRep& R = s->reps_h[r];
            const double per_chunk = std::max(1e-3, (double)R.na / ((double)R.rows * R.cols));
            const int win = (int)std::floor(std::sqrt(0.85 * kTileThreads / per_chunk));
            const int side = std::max(2, std::min(kTileMaxDim, win - 2));
            const int w = std::min(side, (int)R.cols), h = std::min(side, (int)R.rows);
            for (int c0 = 0; c0 < R.cols; c0 += w)
                for (int r0 = 0; r0 < R.rows; r0 += h)
                    th.push_back(TileDesc{r, c0, r0, std::min(w, R.cols - c0) | (std::min(h, R.rows - r0) << 8)});
        }
        s->ntiles_t = (int32_t)th.size();
        if (dalloc(s, &s->tiles, th.size()) != cudaSuccess || dalloc(s, &s->tile_queue, 2) != cudaSuccess)
            return bail(fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the tiles"));
        if (cudaMemcpyAsync(s->tiles, th.data(), sizeof(TileDesc) * th.size(), cudaMemcpyHostToDevice, s->stream) !=
            cudaSuccess)
            return bail(fail(s, MAVI_ERR_CUDA, "tile table upload failed"));
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        s->tile_grid = (unsigned)std::max(1, sms * MAVI_TILE_BLOCKS);
    }

    // descriptors
    std::vector<MaviSpace> spaces_h((size_t)s->R * MAVI_MAX_SPACES);
    std::vector<MaviRingsCfg> rcfg_h(s->R);
    for (int r = 0; r < s->R; r++) {
        for (int k = 0; k < MAVI_MAX_SPACES; k++) spaces_h[(size_t)r * MAVI_MAX_SPACES + k] = replicas[r].spaces[k];
        rcfg_h[r] = replicas[r].rings;
    }
    // the ring kernel specialised to the exact integer path of the mixed form
    s->rings_small = s->is_rings && s->prec == MAVI_PREC_MIXED;
    for (int r = 0; r < s->R && s->rings_small; r++) {
        s->rings_small = !s->reps_h[r].min_image;
        for (int t = 0; t < rcfg_h[r].num_types; t++) s->rings_small = s->rings_small && rcfg_h[r].num_particles[t] <= 32;
    }
    // identity user order over active slots
    std::vector<int32_t> uid_h(M), rep_h(M);
    std::vector<int32_t> types_all, ring_rep_h;
    std::vector<int32_t> rkey_h(C.rkey_user ? N : 0, 0);
    {
        int64_t k = 0;
        const int32_t* tc = ring_types;
        for (int r = 0; r < s->R; r++) {
            const MaviReplicaParams& p = replicas[r];
            const DevRep& R = s->reps_h[r];
            if (s->is_rings) {
                for (int q = 0; q < p.rings.num_rings; q++) {
                    int t = tc ? tc[q] : 1;
                    types_all.push_back(t);
                    ring_rep_h.push_back(r);
                    for (int i = 0; i < p.rings.num_particles[t - 1]; i++) {
                        uid_h[k] = (int32_t)(R.slot0 + (int64_t)q * p.rings.nmax + i);
                        rep_h[k] = r;
                        // ring_key: replica-local ring, index in the ring, 0-based type
                        if (!rkey_h.empty()) rkey_h[uid_h[k]] = (q << 12) | (i << 2) | (t - 1);
                        k++;
                    }
                }
                if (tc) tc += p.rings.num_rings;
            } else {
                for (int64_t i = 0; i < p.num_particles; i++) {
                    uid_h[k] = (int32_t)(R.slot0 + i);
                    rep_h[k] = r;
                    k++;
                }
            }
        }
    }
    CUDA_TRY(s, cudaMemcpyAsync(reps_d, s->reps_h.data(), sizeof(DevRep) * s->R, cudaMemcpyHostToDevice, s->stream));
    if (!rkey_h.empty())
        CUDA_TRY(s, cudaMemcpyAsync(const_cast<int32_t*>(C.rkey_user), rkey_h.data(), sizeof(int32_t) * N,
                                    cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(cxu_d, cxu_h.data(), sizeof(double) * cxu_h.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(cyu_d, cyu_h.data(), sizeof(double) * cyu_h.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(spaces_d, spaces_h.data(), sizeof(MaviSpace) * spaces_h.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(rcfg_d, rcfg_h.data(), sizeof(MaviRingsCfg) * s->R, cudaMemcpyHostToDevice, s->stream));
    std::vector<FixPair> fix_h((size_t)s->R * MAVI_MAX_TYPES * MAVI_MAX_TYPES);
    for (int r = 0; r < s->R; r++) fill_fix_pairs(replicas[r], s->reps_h[r], fix_h.data() + (size_t)r * MAVI_MAX_TYPES * MAVI_MAX_TYPES);
    CUDA_TRY(s, cudaMemcpyAsync(fix_d, fix_h.data(), sizeof(FixPair) * fix_h.size(), cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(C.uid_out, uid_h.data(), sizeof(int32_t) * M, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(C.rep_out, rep_h.data(), sizeof(int32_t) * M, cudaMemcpyHostToDevice, s->stream));
    if (s->is_rings) {
        CUDA_TRY(s, cudaMemcpyAsync(ring_types_d, types_all.data(), sizeof(int32_t) * s->total_rings,
                                    cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(ring_rep_d, ring_rep_h.data(), sizeof(int32_t) * s->total_rings,
                                    cudaMemcpyHostToDevice, s->stream));
    }
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++)
        for (int u = 0; u < 4; u++) {
            cudaEventCreate(&s->ev.a[k][u]);
            cudaEventCreate(&s->ev.b[k][u]);
        }
    cudaEventCreate(&s->ev.step_a);
    cudaEventCreate(&s->ev.step_b);
    int rc = mavi_upload_state(s, pos, vel, pol);
    if (rc) return bail(rc);
    // System() runs the first update_chunks! (src/systems.jl:103-105)
    launch_rebin(s, false);
    rc = check_device_error(s);
    if (rc) return bail(rc);
    if (opt->gather_mode < 0) {
        rc = autotune_gather(s);
        if (rc) return bail(rc);
    }
    *out = s;
    return MAVI_OK;
}

int mavi_upload_state(MaviSystem* s, const double* pos, const double* vel, const double* pol) {
    if (!s || !pos) return MAVI_ERR_INVALID_ARG;
    CUDA_TRY(s, cudaMemcpyAsync(s->pos_user, pos, sizeof(double2) * s->Nslots, cudaMemcpyHostToDevice, s->stream));
    if (s->has_vel && vel)
        CUDA_TRY(s, cudaMemcpyAsync(s->vel_user, vel, sizeof(double2) * s->Nslots, cudaMemcpyHostToDevice, s->stream));
    if (s->has_pol && pol)
        CUDA_TRY(s, cudaMemcpyAsync(s->pol_user, pol, sizeof(double) * s->Nslots, cudaMemcpyHostToDevice, s->stream));
    if (s->is_rings && pol) {
        CUDA_TRY(s, cudaMemcpyAsync(s->C.ring_pol, pol, sizeof(double) * s->total_rings, cudaMemcpyHostToDevice, s->stream));
        if (s->prec == MAVI_PREC_MIXED) k_ring_pol<kPrecMixed><<<nblocks(s->total_rings), kBlock, 0, s->stream>>>(s->C, s->total_rings, 0);
        else k_ring_pol<kPrecFP64><<<nblocks(s->total_rings), kBlock, 0, s->stream>>>(s->C, s->total_rings, 0);
    }
    const double2* vel_src = (s->has_vel && vel) ? s->vel_user : nullptr;
    const double* pol_src = (s->has_pol && pol) ? s->pol_user : nullptr;
    if (vel_src || pol_src)
        k_gather_user<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, nullptr, vel_src, pol_src);
    s->counts_valid = false;
    launch_count(s, s->pos_user);   // positions gathered inside the histogram
    s->counts_valid = true;
    if (s->var_rings) launch_rebin(s, false);   // chunk lists of the uploaded state
    CUDA_TRY(s, cudaGetLastError());
    return MAVI_OK;   // device errors of this state surface at the next synchronising call
}

int mavi_download_state(MaviSystem* s, double* pos, double* vel, double* pol) {
    const int rc = mavi_download_state_async(s, pos, vel, pol);
    if (rc) return rc;
    return check_device_error(s);   // waits for the copies
}

int mavi_synchronize(MaviSystem* s) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    return check_device_error(s);
}

int mavi_download_state_async(MaviSystem* s, double* pos, double* vel, double* pol) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    k_scatter_user<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, s->pos_user, s->has_vel ? s->vel_user : nullptr,
                                                            s->has_pol ? s->pol_user : nullptr);
    CUDA_TRY(s, cudaGetLastError());
    if (pos) CUDA_TRY(s, cudaMemcpyAsync(pos, s->pos_user, sizeof(double2) * s->Nslots, cudaMemcpyDeviceToHost, s->stream));
    if (vel && s->has_vel)
        CUDA_TRY(s, cudaMemcpyAsync(vel, s->vel_user, sizeof(double2) * s->Nslots, cudaMemcpyDeviceToHost, s->stream));
    if (pol && s->has_pol)
        CUDA_TRY(s, cudaMemcpyAsync(pol, s->pol_user, sizeof(double) * s->Nslots, cudaMemcpyDeviceToHost, s->stream));
    if (pol && s->is_rings)
        CUDA_TRY(s, cudaMemcpyAsync(pol, s->C.ring_pol, sizeof(double) * s->total_rings, cudaMemcpyDeviceToHost, s->stream));
    return MAVI_OK;
}

int64_t mavi_noise_count(MaviSystem* s) { return s ? s->noise_count : -1; }

int mavi_set_noise(MaviSystem* s, const double* noise, int64_t count) {
    if (!s || !noise || s->noise_count == 0 || count <= 0 || count % s->noise_count != 0)
        return fail(s, MAVI_ERR_INVALID_ARG, "noise count must be a positive multiple of %lld",
                    (long long)(s ? s->noise_count : 0));
    if (count > s->noise_queue_cap) {
        if (s->noise_queue) {
            cudaStreamSynchronize(s->stream);
            cudaFree(s->noise_queue);
            s->allocs.erase(std::remove(s->allocs.begin(), s->allocs.end(), (void*)s->noise_queue), s->allocs.end());
        }
        if (dalloc(s, &s->noise_queue, count) != cudaSuccess) return fail(s, MAVI_ERR_CUDA, "noise buffer allocation failed");
        s->noise_queue_cap = count;
    }
    CUDA_TRY(s, cudaMemcpyAsync(s->noise_queue, noise, sizeof(double) * count, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    s->noise_queue_len = count / s->noise_count;
    s->noise_queue_pos = 0;
    return MAVI_OK;
}

int mavi_set_seed(MaviSystem* s, uint64_t seed) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    s->opt.seed = seed;
    s->C.seed = seed;
    drop_graph(s);
    return MAVI_OK;
}

int mavi_step(MaviSystem* s, int64_t nsteps) {
    if (!s || nsteps < 0) return MAVI_ERR_INVALID_ARG;
    bool injected = s->noise_count > 0 && s->opt.noise_mode == MAVI_NOISE_INJECTED;
    if (injected && s->noise_queue_len - s->noise_queue_pos < nsteps)
        return fail(s, MAVI_ERR_NOISE_MISSING, "%lld steps need noise; %lld steps of noise supplied",
                    (long long)nsteps, (long long)(s->noise_queue_len - s->noise_queue_pos));
    if (nsteps == 0) return MAVI_OK;
    if (!s->counts_valid && !s->var_rings) {     // after calc_forces/energies/update_chunks
        launch_count(s);
        for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++) s->ev.used[k] = 0;
        s->counts_valid = true;
    }
    if (s->opt.use_graph) {
        int rc = ensure_graph(s);
        if (rc) return rc;
    }
    std::vector<int32_t> due;
    for (int64_t k = 0; k < nsteps; k++) {
        // update_invasions! (src/rings/integration.jl:511-520): which replicas check on this step
        due.clear();
        for (int32_t r = 0; r < (int32_t)s->inv.size(); r++)
            if (s->inv[r].on && s->num_steps[r] - s->inv[r].last_check >= s->inv[r].steps) due.push_back(r);
        if (injected) {
            CUDA_TRY(s, cudaMemcpyAsync(s->noise_cur, s->noise_queue + s->noise_queue_pos * s->noise_count,
                                        sizeof(double) * s->noise_count, cudaMemcpyDeviceToDevice, s->stream));
            s->noise_queue_pos++;
        }
        if (s->graph_exec && due.empty()) {
            CUDA_TRY(s, cudaGraphLaunch(s->graph_exec, s->stream));
            s->counts_valid = !s->var_rings;
            collect_profile(s, s->graph_ev_used);
            collect_step_time(s, s->graph_step_used);
        } else {
            int rc = launch_step(s, &due);
            if (rc) return rc;
            CUDA_TRY(s, cudaGetLastError());
            collect_profile(s, s->ev.used);
            collect_step_time(s, s->ev.step_used);
            for (int q = 0; q < MAVI_NUM_KERNEL_KINDS; q++) s->ev.used[q] = 0;
            s->ev.step_used = 0;
        }
        for (int r = 0; r < s->R; r++) {
            s->num_steps[r] += 1;
            s->time[r] += s->params[r].dt;
        }
        if (s->profiling) s->prof.steps += 1;
    }
    CUDA_TRY(s, cudaGetLastError());
    return MAVI_OK;   // enqueued: device errors of these steps surface at the next synchronising call
}

int mavi_update_chunks(MaviSystem* s) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    s->counts_valid = false;
    launch_rebin(s, false);
    CUDA_TRY(s, cudaGetLastError());
    return check_device_error(s);
}

int mavi_chunk_geometry(MaviSystem* s, int32_t replica, int32_t* rows, int32_t* cols, int32_t* cap) {
    if (!s || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    const DevRep& R = s->reps_h[replica];
    if (!R.has_chunks) return fail(s, MAVI_ERR_INVALID_ARG, "replica %d has no chunks", replica);
    if (rows) *rows = R.rows;
    if (cols) *cols = R.cols;
    if (cap) *cap = R.cap;
    return MAVI_OK;
}

int mavi_get_chunks(MaviSystem* s, int32_t replica, int32_t* num_in_chunk, int32_t* chunk_particles) {
    if (!s || replica < 0 || replica >= s->R || !num_in_chunk || !chunk_particles) return MAVI_ERR_INVALID_ARG;
    const DevRep& R = s->reps_h[replica];
    if (!R.has_chunks) return fail(s, MAVI_ERR_INVALID_ARG, "replica %d has no chunks", replica);
    int rc = mavi_update_chunks(s);
    if (rc) return rc;
    int64_t nch = (int64_t)R.rows * R.cols;
    std::vector<int32_t> start(nch + 1), uid(R.na);
    CUDA_TRY(s, cudaMemcpy(start.data(), s->C.start + R.c0, sizeof(int32_t) * (nch + 1), cudaMemcpyDeviceToHost));
    CUDA_TRY(s, cudaMemcpy(uid.data(), s->C.uid_cur + R.a0, sizeof(int32_t) * R.na, cudaMemcpyDeviceToHost));
    int32_t mx = 0;
    for (int64_t c = 0; c < nch; c++) {
        int32_t b = start[c] - (int32_t)R.a0, e = start[c + 1] - (int32_t)R.a0;
        num_in_chunk[c] = e - b;
        mx = std::max(mx, e - b);
        for (int32_t k = 0; k < R.cap; k++)
            chunk_particles[c * R.cap + k] = (k < e - b) ? uid[b + k] - (int32_t)R.slot0 : -1;
    }
    s->max_chunk_count = mx;
    return MAVI_OK;
}

int mavi_calc_forces(MaviSystem* s, int32_t include_walls, double* forces_out) {
    if (!s || !forces_out) return MAVI_ERR_INVALID_ARG;
    s->counts_valid = false;
    launch_rebin(s, false);
    if (s->prec == MAVI_PREC_FP64) forces_only_fp64(s, include_walls);
    else forces_only_mixed(s, include_walls);
    if (s->is_rings) {
        if (s->prec == MAVI_PREC_FP64) rings_terms_fp64(s, 0, include_walls);
        else rings_terms_mixed(s, 0, include_walls);
    }
    CUDA_TRY(s, cudaMemsetAsync(s->f_user, 0, sizeof(double2) * s->Nslots, s->stream));
    if (s->prec == MAVI_PREC_FP64) forces_to_user_fp64(s);
    else forces_to_user_mixed(s);
    CUDA_TRY(s, cudaGetLastError());
    CUDA_TRY(s, cudaMemcpyAsync(forces_out, s->f_user, sizeof(double2) * s->Nslots, cudaMemcpyDeviceToHost, s->stream));
    return check_device_error(s);
}

// Per-replica kinetic and potential energies of the current state into the
// device arrays ke_out / pe_out (num_replicas doubles each), enqueued.
static void enqueue_energies(MaviSystem* s, int32_t pe_mode, double* ke_out, double* pe_out) {
    s->counts_valid = false;
    launch_rebin(s, false);
    k_energy_terms<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, s->dyn, pe_mode == MAVI_PE_ALL_PAIRS, s->ke_t, s->pe_t,
                                                            s->has_vel ? 1 : 0);
    k_reduce_per_replica<<<s->R, 256, 0, s->stream>>>(s->C, s->ke_t, ke_out, 0.5);
    k_reduce_per_replica<<<s->R, 256, 0, s->stream>>>(s->C, s->pe_t, pe_out, 1.0);
}

int mavi_energies(MaviSystem* s, int32_t pe_mode, double* ke, double* pe) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    enqueue_energies(s, pe_mode, s->ke_r, s->pe_r);
    CUDA_TRY(s, cudaGetLastError());
    if (ke) CUDA_TRY(s, cudaMemcpyAsync(ke, s->ke_r, sizeof(double) * s->R, cudaMemcpyDeviceToHost, s->stream));
    if (pe) CUDA_TRY(s, cudaMemcpyAsync(pe, s->pe_r, sizeof(double) * s->R, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    bool pe_defined = s->dyn == MAVI_DYN_LEN_JONES || s->dyn == MAVI_DYN_HARM_TRUNC || s->dyn == MAVI_DYN_RUN_TUMBLE;
    if (pe && !pe_defined)
        for (int r = 0; r < s->R; r++) pe[r] = NAN;
    return check_device_error(s);
}

int mavi_energy_series(MaviSystem* s, int64_t num_samples, int64_t steps_between, int32_t pe_mode, double* ke,
                       double* pe) {
    if (!s || num_samples < 1 || steps_between < 0 || !ke || !pe) return MAVI_ERR_INVALID_ARG;
    const int64_t need = 2 * num_samples * (int64_t)s->R;
    if (need > s->series_cap) {
        if (s->series) {
            CUDA_TRY(s, cudaStreamSynchronize(s->stream));
            cudaFree(s->series);
            s->series = nullptr;
            s->series_cap = 0;
        }
        CUDA_TRY(s, cudaMalloc((void**)&s->series, sizeof(double) * need));
        s->series_cap = need;
    }
    for (int64_t k = 0; k < num_samples; k++) {
        int rc = mavi_step(s, steps_between);
        if (rc) return rc;
        double* row = s->series + 2 * k * s->R;
        enqueue_energies(s, pe_mode, row, row + s->R);
    }
    CUDA_TRY(s, cudaGetLastError());
    std::vector<double> h(need);
    CUDA_TRY(s, cudaMemcpyAsync(h.data(), s->series, sizeof(double) * need, cudaMemcpyDeviceToHost, s->stream));
    int rc = check_device_error(s);   // waits for the stream
    if (rc) return rc;
    const bool pe_defined = s->dyn == MAVI_DYN_LEN_JONES || s->dyn == MAVI_DYN_HARM_TRUNC || s->dyn == MAVI_DYN_RUN_TUMBLE;
    for (int64_t k = 0; k < num_samples; k++)
        for (int r = 0; r < s->R; r++) {
            ke[k * s->R + r] = h[2 * k * s->R + r];
            pe[k * s->R + r] = pe_defined ? h[2 * k * s->R + s->R + r] : NAN;
        }
    return MAVI_OK;
}

int mavi_pair_distribution(MaviSystem* s, int32_t replica, double r_max, int32_t num_bins, uint64_t* counts) {
    if (!s || !counts || replica < -1 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (num_bins < 1 || num_bins > kHistMaxBins)
        return fail(s, MAVI_ERR_INVALID_ARG, "num_bins must be in 1..%d", kHistMaxBins);
    if (!(r_max > 0) || !std::isfinite(r_max)) return fail(s, MAVI_ERR_INVALID_ARG, "r_max must be positive");
    for (int r = 0; r < s->R; r++) {
        if (replica >= 0 && r != replica) continue;
        const DevRep& R = s->reps_h[r];
        if (R.has_chunks && r_max > std::min(R.chunk_l, R.chunk_h))
            return fail(s, MAVI_ERR_INVALID_ARG, "r_max %g exceeds the chunk sides of replica %d (%g x %g)", r_max, r,
                        R.chunk_l, R.chunk_h);
    }
    if (!s->hist) CUDA_TRY(s, cudaMalloc((void**)&s->hist, sizeof(unsigned long long) * kHistMaxBins));
    s->counts_valid = false;
    launch_rebin(s, false);
    CUDA_TRY(s, cudaMemsetAsync(s->hist, 0, sizeof(unsigned long long) * num_bins, s->stream));
    k_pair_hist<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, replica, r_max, r_max / num_bins, num_bins, s->hist);
    CUDA_TRY(s, cudaGetLastError());
    CUDA_TRY(s, cudaMemcpyAsync(counts, s->hist, sizeof(unsigned long long) * num_bins, cudaMemcpyDeviceToHost,
                                s->stream));
    return check_device_error(s);
}

int mavi_get_time(MaviSystem* s, int64_t* num_steps, double* time) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    if (num_steps) *num_steps = s->num_steps[0];
    if (time) *time = s->time[0];
    return MAVI_OK;
}

int mavi_set_time(MaviSystem* s, int32_t replica, int64_t num_steps, double time) {
    if (!s || replica < 0 || replica >= s->R || num_steps < 0) return MAVI_ERR_INVALID_ARG;
    s->num_steps[replica] = num_steps;
    s->time[replica] = time;
    if (replica == 0) {
        // the noise counter: steps completed, as every step's chunk update advances it
        const int64_t v = num_steps;
        CUDA_TRY(s, cudaMemcpyAsync(s->C.d_step, &v, sizeof(int64_t), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    }
    return MAVI_OK;
}

int mavi_rings_neighbors_config(MaviSystem* s, int32_t enable, int32_t only_count, int32_t type_all, double tol) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    if (!s->is_rings) return fail(s, MAVI_ERR_UNSUPPORTED, "particle neighbour lists belong to the rings model");
    if (!enable) {
        s->C.nb_mode = 0;
        drop_graph(s);
        return MAVI_OK;
    }
    if (!(tol > 0)) return fail(s, MAVI_ERR_INVALID_ARG, "tol must be > 0");
    if (!s->C.nb_count && dalloc(s, &s->C.nb_count, s->Nslots) != cudaSuccess)
        return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the neighbour counts");
    if (!only_count && !s->C.nb_list &&
        dalloc(s, &s->C.nb_list, s->Nslots * (int64_t)MAVI_MAX_NEIGHBORS) != cudaSuccess)
        return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the neighbour lists");
    // squared thresholds (dist_eq * tol)^2 in units^2 with the +-1e-6 band of the FP32 test
    std::vector<FixPair> fix_h((size_t)s->R * MAVI_MAX_TYPES * MAVI_MAX_TYPES);
    for (int r = 0; r < s->R; r++) {
        FixPair* f = fix_h.data() + (size_t)r * MAVI_MAX_TYPES * MAVI_MAX_TYPES;
        fill_fix_pairs(s->params[r], s->reps_h[r], f);
        const MaviRingsCfg& rc = s->params[r].rings;
        for (int a = 0; a < rc.num_types; a++)
            for (int b = 0; b < rc.num_types; b++) {
                const double thr = 2.0 * (rc.inter_dist_eq[a][b] / 2.0) * tol * s->reps_h[r].inv_u;
                f[a * MAVI_MAX_TYPES + b].nb2_hi = (float)(thr * thr * (1.0 + 1e-6));
                f[a * MAVI_MAX_TYPES + b].nb2_lo = (float)(thr * thr * (1.0 - 1e-6));
            }
    }
    CUDA_TRY(s, cudaMemcpyAsync(const_cast<FixPair*>(s->C.fix), fix_h.data(), sizeof(FixPair) * fix_h.size(),
                                cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemsetAsync(s->C.nb_count, 0, sizeof(int32_t) * s->Nslots, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    s->C.nb_mode = only_count ? 1 : 2;
    s->C.nb_type_all = type_all ? 1 : 0;
    s->C.nb_tol = tol;
    drop_graph(s);
    return MAVI_OK;
}

int mavi_rings_neighbors(MaviSystem* s, int32_t replica, int32_t* counts, int32_t* lists) {
    if (!s || !counts || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (!s->C.nb_mode) return fail(s, MAVI_ERR_INVALID_ARG, "neighbour lists are not enabled");
    if (lists && s->C.nb_mode != 2) return fail(s, MAVI_ERR_INVALID_ARG, "only neighbour counts are kept");
    const DevRep& R = s->reps_h[replica];
    const int64_t n = R.nslots;
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    CUDA_TRY(s, cudaMemcpy(counts, s->C.nb_count + R.slot0, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    if (lists) {
        std::vector<int32_t> tmp((size_t)n * MAVI_MAX_NEIGHBORS);
        CUDA_TRY(s, cudaMemcpy(tmp.data(), s->C.nb_list + R.slot0 * MAVI_MAX_NEIGHBORS,
                               sizeof(int32_t) * tmp.size(), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < MAVI_MAX_NEIGHBORS; k++)
                lists[i * MAVI_MAX_NEIGHBORS + k] =
                    k < counts[i] ? tmp[i * MAVI_MAX_NEIGHBORS + k] - (int32_t)R.slot0 : -1;
    }
    return check_device_error(s);
}

// ---------------------------------------------------------------------------
// sources and sinks of the rings model
// ---------------------------------------------------------------------------
// Replaces a device buffer owned by the handle with a copy of `n` host
// elements (nullptr when n == 0). The caller synchronises before the host
// data goes away.
static int replace_buffer(MaviSystem* s, void*& slot, const void* data, size_t bytes, const void** out) {
    if (slot) {
        cudaStreamSynchronize(s->stream);
        cudaFree(slot);
        s->allocs.erase(std::remove(s->allocs.begin(), s->allocs.end(), slot), s->allocs.end());
        slot = nullptr;
    }
    *out = nullptr;
    if (bytes == 0) return MAVI_OK;
    char* d = nullptr;
    if (dalloc(s, &d, bytes) != cudaSuccess) return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the sources");
    slot = d;
    CUDA_TRY(s, cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, s->stream));
    *out = d;
    return MAVI_OK;
}

// Flattens every replica's sources and sinks into the device arrays and the
// replicas' descriptors; random spawn polarisations get their places in the
// step's noise after the replicas' own numbers.
static int upload_sources(MaviSystem* s) {
    std::vector<SrcEntryD> ent;
    std::vector<SrcBoxD> box;
    std::vector<double2> spawn;
    std::vector<int32_t> chunks;
    int64_t noise_idx = s->noise_base;
    for (int r = 0; r < s->R; r++) {
        DevRep& R = s->reps_h[r];
        const MaviSystem::SrcCfg& cfg = s->src_cfg[r];
        R.src_e0 = (int32_t)ent.size();
        R.src_ne = (int32_t)cfg.entries.size();
        R.src_has_sink = 0;
        size_t b = 0, k = 0;
        for (const MaviSourceEntry& e : cfg.entries) {
            SrcEntryD d{};
            d.kind = e.kind; d.num_boxes = e.kind == MAVI_SRC_SOURCE ? e.num_boxes : 0;
            d.pol_mode = e.pol_mode; d.geometry = e.geometry;
            d.box0 = (int32_t)box.size();
            d.pol = e.pol; d.pad = e.pad;
            d.length = e.length; d.height = e.height; d.bl_x = e.bl_x; d.bl_y = e.bl_y;
            d.radius = e.radius; d.cx = e.cx; d.cy = e.cy;
            if (e.kind == MAVI_SRC_SINK) R.src_has_sink = 1;
            for (int32_t q = 0; q < d.num_boxes; q++, b++) {
                const MaviSpawnBox& mb = cfg.boxes[b];
                SrcBoxD bd{};
                bd.bl_x = mb.bl_x; bd.bl_y = mb.bl_y; bd.length = mb.length; bd.height = mb.height;
                bd.num_chunks = mb.num_chunks;
                bd.chunk0 = (int32_t)chunks.size();
                bd.spawn0 = (int64_t)spawn.size();
                bd.noise_idx = e.pol_mode == MAVI_SPAWN_POL_RANDOM ? noise_idx++ : -1;
                for (int32_t p = 0; p < R.nmax; p++)
                    spawn.push_back(make_double2(cfg.spawn_xy[2 * (b * R.nmax + p)], cfg.spawn_xy[2 * (b * R.nmax + p) + 1]));
                for (int32_t c = 0; c < std::max(mb.num_chunks, 0); c++, k++) {
                    const int32_t row = cfg.chunk_rc[2 * k], col = cfg.chunk_rc[2 * k + 1];
                    chunks.push_back((int32_t)(R.c0 + (int64_t)col * R.rows + row));
                }
                box.push_back(bd);
            }
            ent.push_back(d);
        }
    }
    int rc;
    const void* d[4];
    if ((rc = replace_buffer(s, s->src_buf[0], ent.data(), sizeof(SrcEntryD) * ent.size(), &d[0]))) return rc;
    if ((rc = replace_buffer(s, s->src_buf[1], box.data(), sizeof(SrcBoxD) * box.size(), &d[1]))) return rc;
    if ((rc = replace_buffer(s, s->src_buf[2], spawn.data(), sizeof(double2) * spawn.size(), &d[2]))) return rc;
    if ((rc = replace_buffer(s, s->src_buf[3], chunks.data(), sizeof(int32_t) * chunks.size(), &d[3]))) return rc;
    s->C.src_entries = static_cast<const SrcEntryD*>(d[0]);
    s->C.src_boxes = static_cast<const SrcBoxD*>(d[1]);
    s->C.src_spawn = static_cast<const double2*>(d[2]);
    s->C.src_chunks = static_cast<const int32_t*>(d[3]);
    CUDA_TRY(s, cudaMemcpyAsync(const_cast<DevRep*>(s->C.reps), s->reps_h.data(), sizeof(DevRep) * s->R,
                                cudaMemcpyHostToDevice, s->stream));
    // the step's noise grows by the spawn uniforms
    if (noise_idx != s->noise_count) {
        CUDA_TRY(s, cudaStreamSynchronize(s->stream));
        if (s->noise_cur) {
            cudaFree(s->noise_cur);
            s->allocs.erase(std::remove(s->allocs.begin(), s->allocs.end(), (void*)s->noise_cur), s->allocs.end());
            s->noise_cur = nullptr;
        }
        s->noise_count = noise_idx;
        if (s->noise_count > 0 && dalloc(s, &s->noise_cur, s->noise_count) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "noise buffer allocation failed");
        s->C.noise = s->noise_cur;
        s->noise_queue_len = 0;
        s->noise_queue_pos = 0;
    }
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    return MAVI_OK;
}

int mavi_rings_sources(MaviSystem* s, int32_t replica, const int32_t* active_mask, int32_t num_entries,
                       const MaviSourceEntry* entries, const MaviSpawnBox* boxes, const double* spawn_xy,
                       const int32_t* chunk_rc) {
    if (!s || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (!s->is_rings) return fail(s, MAVI_ERR_UNSUPPORTED, "sources and sinks belong to the rings model");
    if (num_entries < 0 || num_entries > MAVI_MAX_SOURCE_ENTRIES || (num_entries > 0 && !entries))
        return fail(s, MAVI_ERR_INVALID_ARG, "num_entries must be in [0, %d]", MAVI_MAX_SOURCE_ENTRIES);
    const DevRep& R = s->reps_h[replica];
    int64_t nbox = 0, nchunk = 0;
    for (int32_t e = 0; e < num_entries; e++) {
        const MaviSourceEntry& E = entries[e];
        if (E.kind == MAVI_SRC_SINK) {
            if (E.geometry != MAVI_GEOM_RECTANGLE && E.geometry != MAVI_GEOM_CIRCLE)
                return fail(s, MAVI_ERR_INVALID_ARG, "entry %d: a sink is a rectangle or a circle", e);
        } else if (E.kind == MAVI_SRC_SOURCE) {
            if (E.num_boxes < 1 || E.num_boxes > MAVI_MAX_SPAWN_BOXES)
                return fail(s, MAVI_ERR_INVALID_ARG, "entry %d: 1..%d spawn boxes", e, MAVI_MAX_SPAWN_BOXES);
            if (E.pol_mode != MAVI_SPAWN_POL_FIXED && E.pol_mode != MAVI_SPAWN_POL_RANDOM)
                return fail(s, MAVI_ERR_INVALID_ARG, "entry %d: unknown spawn polarisation mode", e);
            nbox += E.num_boxes;
        } else {
            return fail(s, MAVI_ERR_INVALID_ARG, "entry %d: unknown kind %d", e, E.kind);
        }
    }
    if (nbox > 0 && (!boxes || !spawn_xy)) return fail(s, MAVI_ERR_INVALID_ARG, "spawn boxes and points required");
    for (int64_t b = 0; b < nbox; b++) {
        if (boxes[b].num_chunks < -1) return fail(s, MAVI_ERR_INVALID_ARG, "box %lld: num_chunks < -1", (long long)b);
        nchunk += std::max(boxes[b].num_chunks, 0);
    }
    if (nchunk > 0 && !chunk_rc) return fail(s, MAVI_ERR_INVALID_ARG, "chunk lists required");
    for (int64_t k = 0; k < nchunk; k++) {
        const int32_t row = chunk_rc[2 * k], col = chunk_rc[2 * k + 1];
        if (row < 0 || row >= R.rows || col < 0 || col >= R.cols)
            return fail(s, MAVI_ERR_INVALID_ARG, "chunk (%d, %d) outside the %d x %d grid", row, col, R.rows, R.cols);
    }
    for (int64_t k = 0; k < 2 * nbox * R.nmax; k++)
        if (!std::isfinite(spawn_xy[k])) return fail(s, MAVI_ERR_INVALID_ARG, "non-finite spawn position");
    if (s->src_cfg.empty()) s->src_cfg.resize(s->R);
    MaviSystem::SrcCfg& cfg = s->src_cfg[replica];
    cfg.entries.assign(entries, entries + num_entries);
    cfg.boxes.assign(boxes, boxes + nbox);
    cfg.spawn_xy.assign(spawn_xy, spawn_xy + 2 * nbox * R.nmax);
    cfg.chunk_rc.assign(chunk_rc, chunk_rc + 2 * nchunk);

    Ctx& C = s->C;
    if (!C.ring_active) {
        // VarRingsIds of every replica: all active, uids 1..num_rings, ids identity
        if (dalloc(s, &C.ring_active, s->total_rings) != cudaSuccess || dalloc(s, &C.ring_uid, s->total_rings) != cudaSuccess ||
            dalloc(s, &C.ring_cms, s->total_rings) != cudaSuccess || dalloc(s, &C.src_ids, s->total_rings) != cudaSuccess ||
            dalloc(s, &C.src_state, 2 * (int64_t)s->R) != cudaSuccess)
            return fail(s, MAVI_ERR_CUDA, "cudaMalloc failed for the rings ids");
        std::vector<int32_t> act(s->total_rings, 1), uid(s->total_rings), ids(s->total_rings), st(2 * s->R);
        for (int r = 0; r < s->R; r++) {
            const DevRep& Q = s->reps_h[r];
            for (int32_t k = 0; k < Q.num_rings; k++) { uid[Q.ring0 + k] = k + 1; ids[Q.ring0 + k] = k; }
            st[2 * r] = Q.num_rings;
            st[2 * r + 1] = Q.num_rings;
        }
        CUDA_TRY(s, cudaMemcpyAsync(C.ring_active, act.data(), sizeof(int32_t) * act.size(), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.ring_uid, uid.data(), sizeof(int32_t) * uid.size(), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.src_ids, ids.data(), sizeof(int32_t) * ids.size(), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.src_state, st.data(), sizeof(int32_t) * st.size(), cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemsetAsync(C.ring_cms, 0, sizeof(double2) * s->total_rings, s->stream));
        CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    }
    {
        // this replica's mask (ActiveState), uids 1..num_rings and ids
        // (calc_active_ids!: active rings ascending, the rest of 1:num_rings after)
        const int32_t nr = R.num_rings;
        std::vector<int32_t> act(nr), uid(nr), ids(nr), st(2);
        int32_t na = 0;
        for (int32_t k = 0; k < nr; k++) {
            act[k] = active_mask ? (active_mask[k] != 0 ? 1 : 0) : 1;
            uid[k] = k + 1;
            ids[k] = k;
        }
        for (int32_t k = 0; k < nr; k++) if (act[k]) ids[na++] = k;
        st[0] = na;
        st[1] = nr;
        CUDA_TRY(s, cudaMemcpyAsync(C.ring_active + R.ring0, act.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.ring_uid + R.ring0, uid.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.src_ids + R.ring0, ids.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaMemcpyAsync(C.src_state + 2 * replica, st.data(), sizeof(int32_t) * 2, cudaMemcpyHostToDevice, s->stream));
        CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    }
    int rc = upload_sources(s);
    if (rc) return rc;
    s->var_rings = true;
    C.var_rings = 1;
    drop_graph(s);
    // chunk lists of the active set (pending histograms were of the old set)
    s->counts_valid = false;
    launch_rebin(s, false);
    CUDA_TRY(s, cudaGetLastError());
    return check_device_error(s);
}

int mavi_rings_active(MaviSystem* s, int32_t replica, int32_t* active_mask, int32_t* uids, int32_t* num_active) {
    if (!s || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (!s->is_rings) return fail(s, MAVI_ERR_UNSUPPORTED, "rings ids belong to the rings model");
    const DevRep& R = s->reps_h[replica];
    const int32_t nr = R.num_rings;
    if (!s->C.ring_active) {
        for (int32_t k = 0; k < nr; k++) {
            if (active_mask) active_mask[k] = 1;
            if (uids) uids[k] = k + 1;
        }
        if (num_active) *num_active = nr;
        return MAVI_OK;
    }
    int32_t st[2] = {0, 0};
    if (active_mask)
        CUDA_TRY(s, cudaMemcpyAsync(active_mask, s->C.ring_active + R.ring0, sizeof(int32_t) * nr, cudaMemcpyDeviceToHost, s->stream));
    if (uids)
        CUDA_TRY(s, cudaMemcpyAsync(uids, s->C.ring_uid + R.ring0, sizeof(int32_t) * nr, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(st, s->C.src_state + 2 * replica, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, s->stream));
    int rc = check_device_error(s);   // waits for the copies
    if (num_active) *num_active = st[0];
    return rc;
}

int mavi_rings_areas(MaviSystem* s, int32_t replica, double* areas) {
    if (!s || !areas || replica < 0 || replica >= s->R) return MAVI_ERR_INVALID_ARG;
    if (!s->is_rings) return fail(s, MAVI_ERR_UNSUPPORTED, "ring areas belong to the rings model");
    const DevRep& R = s->reps_h[replica];
    if (R.num_rings == 0) return MAVI_OK;
    k_ring_areas<<<nblocks(R.num_rings), kBlock, 0, s->stream>>>(s->C, R.ring0, R.num_rings, s->C.ring_area);
    CUDA_TRY(s, cudaGetLastError());
    CUDA_TRY(s, cudaMemcpyAsync(areas, s->C.ring_area, sizeof(double) * R.num_rings, cudaMemcpyDeviceToHost, s->stream));
    return check_device_error(s);   // waits for the copy
}

int mavi_get_stats(MaviSystem* s, MaviStats* st) {
    if (!s || !st) return MAVI_ERR_INVALID_ARG;
    int rc = mavi_update_chunks(s);
    if (rc) return rc;
    CUDA_TRY(s, cudaMemsetAsync(s->d_pairs, 0, sizeof(unsigned long long), s->stream));
    k_pair_count<<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, s->d_pairs);
    unsigned long long pairs = 0;
    CUDA_TRY(s, cudaMemcpyAsync(&pairs, s->d_pairs, sizeof(pairs), cudaMemcpyDeviceToHost, s->stream));
    std::vector<int32_t> start(s->Ctot + 1);
    CUDA_TRY(s, cudaMemcpyAsync(start.data(), s->C.start, sizeof(int32_t) * (s->Ctot + 1), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(s, cudaStreamSynchronize(s->stream));
    int32_t mx = 0;
    for (int64_t c = 0; c < s->Ctot; c++) mx = std::max(mx, start[c + 1] - start[c]);
    st->candidate_pairs = (int64_t)(pairs / 2);
    st->total_particles = s->M;
    st->total_chunks = s->Ctot;
    st->max_chunk_count = mx;
    st->gather_mode = pass_mode_of(s);
    return MAVI_OK;
}

int mavi_profile_enable(MaviSystem* s, int32_t on) {
    if (!s) return MAVI_ERR_INVALID_ARG;
    if (on < 0 || on > 2) return MAVI_ERR_INVALID_ARG;
    s->profiling = on != 0;
    s->profile_mode = on;
    s->prof = MaviProfile{};
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++) s->ev.used[k] = 0;
    return MAVI_OK;
}

int mavi_profile_read(MaviSystem* s, MaviProfile* p) {
    if (!s || !p) return MAVI_ERR_INVALID_ARG;
    *p = s->prof;
    return MAVI_OK;
}

int mavi_last_error(MaviSystem* s, char* buf, int32_t len) {
    if (!s || !buf || len <= 0) return MAVI_ERR_INVALID_ARG;
    snprintf(buf, (size_t)len, "%s", s->last_error.c_str());
    return MAVI_OK;
}

}  // extern "C"
