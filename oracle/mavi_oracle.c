/*
 * mavi_oracle.c — TEST INFRASTRUCTURE ONLY (see mavi_oracle.h).
 *
 * A CPU FP64 restatement of Mavi.jl v1.0.1's step loop. Every function below
 * follows the reference function it names, keeping its loop order (which fixes
 * the FP64 summation order) and its evaluation order of each expression. It is
 * compiled with -ffp-contract=off so that no multiply-add is fused, matching
 * Julia's IEEE semantics without @fastmath.
 *
 * Indices are 0-based here; the reference is 1-based and column-major. A chunk
 * (row, col) has linear index col*rows + row, matching Julia's
 * num_particles_in_chunk[row, col] memory order.
 */
#include "mavi_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y; } V2;

static inline V2 v2(double x, double y) { V2 r = {x, y}; return r; }
static inline V2 vsub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline V2 vadd(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline V2 vscale(double s, V2 a) { return v2(s * a.x, s * a.y); }
static inline double sum_sq(V2 a) { return a.x * a.x + a.y * a.y; }

struct OracleSys {
    MaviReplicaParams p;
    int64_t n;              /* slots */
    double *pos, *vel, *pol;
    int32_t *types;         /* rings: 1-based type per ring */
    double *forces;         /* 2n, get_forces(system) == slice 0 */
    int32_t nthreads;
    double *slices;         /* (nthreads-1) extra slices of 2n for Threaded */
    int64_t *pids; int64_t npids;
    /* chunks (src/chunks.jl:10-25) */
    int has_chunks;
    int32_t rows, cols, cap;
    double chunk_l, chunk_h, bb_len, bb_h, bb_blx, bb_bly;
    int32_t *chunk_particles;   /* [chunk][cap] */
    int32_t *num_in_chunk;      /* [chunk] */
    int32_t *nbr;               /* [chunk][4] */
    int32_t *nbr_cnt;           /* [chunk] */
    /* rings */
    int64_t num_rings; int32_t nmax;
    double *cont_pos;           /* 2*n */
    double *areas;              /* num_rings */
    /* VarRingsIds (src/rings/states.jl:20-40) and RingsInfo.cms */
    int var_ids;
    int32_t *mask, *uids;       /* num_rings */
    int64_t *ids;               /* num_rings: active rings first (update_ids!) */
    int64_t num_active;
    double *cms;                /* 2*num_rings */
    /* sources and sinks (src/rings/sources.jl), in the order of the tuple */
    int32_t src_n;
    MaviSourceEntry *src;
    MaviSpawnBox *boxes;        /* all sources' spawn boxes, in order */
    int64_t nbox;
    double *spawn;              /* nmax points per box */
    int32_t *chunk_rc;          /* (row, col) pairs, 0-based */
    int64_t *box_chunk0;        /* per box: first pair in chunk_rc */
    int64_t n_random;           /* boxes with a random spawn polarisation */
    /* invasions (src/rings/rings.jl:86-100) and the ring chunks of
     * RingsInfo.r_chunks (:189-204) */
    int inv_on;
    int64_t inv_steps, inv_last;
    int32_t rrows, rcols;
    double r_blx, r_bly, r_len, r_h, r_cl, r_ch;
    int32_t *rnbr, *rnbr_cnt, *rcount, *rstart, *rlist;
    MaviInvasion *inv;
    int64_t inv_n, inv_cap;
    /* time_info */
    int64_t num_steps; double time;
    int32_t err;
};

/* ------------------------------------------------------------------------ */
/* Julia Base helpers                                                        */
/* ------------------------------------------------------------------------ */

/* Julia's float `div(x, y)` (RoundToZero): round((x - rem(x, y)) / y) with
 * rem == C fmod and round == round-half-even (Julia Base, base/div.jl; used at
 * src/chunks.jl:129-130). */
double oracle_julia_div(double x, double y) {
    double r = fmod(x, y);
    return nearbyint((x - r) / y);
}

static inline double jsign(double x) { return (x > 0) ? 1.0 : ((x < 0) ? -1.0 : x); }

/* particle_radius (src/configs.jl:418-421; rings src/rings/configs.jl:438-443:
 * the minimum over types is what get_chunks uses, src/systems.jl:26). */
static double particle_radius_of(const MaviReplicaParams* p) {
    const MaviDynamicCfg* d = &p->dyn;
    switch (d->kind) {
    case MAVI_DYN_LEN_JONES: return d->sigma * pow(2.0, 1.0 / 6.0) / 2;
    case MAVI_DYN_SZABO: return d->r_eq / 2;
    case MAVI_DYN_RUN_TUMBLE: return d->sigma * pow(2.0, 1.0 / 6.0) / 2;
    case MAVI_DYN_HARM_TRUNC: return d->dist_eq / 2.0;
    case MAVI_DYN_RINGS: {
        double m = INFINITY;
        for (int t = 0; t < p->rings.num_types; t++) {
            double r = p->rings.inter_dist_eq[t][t] / 2.0;
            if (r < m) m = r;
        }
        return m;
    }
    }
    return NAN;
}

/* Bounding box of a geometry (src/configs.jl:188-229). */
static void bbox_of_space(const MaviSpace* sp, double* len, double* h, double* blx, double* bly) {
    if (sp->geometry == MAVI_GEOM_RECTANGLE) {
        *len = sp->length; *h = sp->height; *blx = sp->bl_x; *bly = sp->bl_y;
    } else if (sp->geometry == MAVI_GEOM_CIRCLE) {
        double r = sp->radius;
        *len = 2 * r; *h = 2 * r; *blx = sp->cx - r; *bly = sp->cy - r;
    } else {
        if (sp->has_bbox) {
            *len = sp->bbox_length; *h = sp->bbox_height; *blx = sp->bbox_bl_x; *bly = sp->bbox_bl_y;
            return;
        }
        double mxx = -INFINITY, mnx = INFINITY, mxy = -INFINITY, mny = INFINITY;
        for (int l = 0; l < sp->num_lines; l++) {
            for (int e = 0; e < 2; e++) {
                double x = sp->lines[l][2 * e], y = sp->lines[l][2 * e + 1];
                if (x > mxx) mxx = x; if (x < mnx) mnx = x;
                if (y > mxy) mxy = y; if (y < mny) mny = y;
            }
        }
        *len = mxx - mnx; *h = mxy - mny; *blx = mnx; *bly = mny;
    }
}

/* ManyGeometries bounding box: fold with `+` (src/configs.jl:68-77, 223-229). */
static void bbox_of(const MaviReplicaParams* p, double* len, double* h, double* blx, double* bly) {
    bbox_of_space(&p->spaces[0], len, h, blx, bly);
    for (int k = 1; k < p->num_spaces; k++) {
        double l2, h2, x2, y2;
        bbox_of_space(&p->spaces[k], &l2, &h2, &x2, &y2);
        double max_x = fmax(*blx + *len, x2 + l2);
        double max_y = fmax(*bly + *h, y2 + h2);
        double min_x = fmin(*blx, x2);
        double min_y = fmin(*bly, y2);
        *h = max_y - min_y; *len = max_x - min_x; *blx = min_x; *bly = min_y;
    }
}

/* ------------------------------------------------------------------------ */
/* calc_diff (src/integration.jl:38-52): the first (wall, geometry) entry     */
/* decides; minimum image only for PeriodicWalls on a RectangleCfg.          */
/* ------------------------------------------------------------------------ */
static inline V2 calc_diff(const OracleSys* s, V2 r1, V2 r2) {
    V2 dr = vsub(r1, r2);
    const MaviSpace* sp = &s->p.spaces[0];
    if (sp->wall == MAVI_WALL_PERIODIC && sp->geometry == MAVI_GEOM_RECTANGLE) {
        double sx = sp->length, sy = sp->height;
        /* dr - (abs.(dr) .> size/2) .* copysign.(size, dr) */
        double mx = (fabs(dr.x) > sx / 2) ? copysign(sx, dr.x) : copysign(0.0, copysign(sx, dr.x));
        double my = (fabs(dr.y) > sy / 2) ? copysign(sy, dr.y) : copysign(0.0, copysign(sy, dr.y));
        dr = v2(dr.x - mx, dr.y - my);
    }
    return dr;
}

static inline V2 P(const OracleSys* s, int64_t i) { return v2(s->pos[2 * i], s->pos[2 * i + 1]); }

/* ------------------------------------------------------------------------ */
/* pair interactions                                                         */
/* ------------------------------------------------------------------------ */

/* potential_force(dr, dist, ::HarmTruncCfg) (src/configs.jl:354-368). */
static inline V2 harm_trunc_force(V2 dr, double dist, double k_rep, double k_atr,
                                  double dist_eq, double dist_max) {
    if (dist > dist_max) return v2(0, 0);
    double fmod_;
    if (dist < dist_eq) fmod_ = -k_rep * (dist / dist_eq - 1);
    else fmod_ = -k_atr * (dist / dist_eq - 1);
    return vscale(fmod_ / dist, dr);
}

/* potential_force(dr, dist, ::LenJonesCfg) (src/configs.jl:389-397): no cutoff. */
static inline V2 len_jones_force(V2 dr, double dist, double sigma, double epsilon) {
    double fmod_ = 4 * epsilon * (12 * pow(sigma, 12) / pow(dist, 13) - 6 * pow(sigma, 6) / pow(dist, 7));
    return vscale(fmod_ / dist, dr);
}

/* Rings pair force: calc_interaction + calc_interaction_force
 * (src/rings/integration.jl:32-77) with InteractionMatrix lookup
 * (src/rings/configs.jl:310-318) and bonded-neighbour exclusion. */
static inline V2 rings_pair_force(const OracleSys* s, int64_t i, int64_t j) {
    const MaviRingsCfg* rc = &s->p.rings;
    int64_t ri = i / s->nmax, rj = j / s->nmax;          /* get_ring_id (src/rings/states.jl:142) */
    int ti = s->types[ri] - 1, tj = s->types[rj] - 1;
    double k_rep = rc->inter_k_rep[ti][tj], k_atr = rc->inter_k_atr[ti][tj];
    double dist_eq = rc->inter_dist_eq[ti][tj], dist_max = rc->inter_dist_max[ti][tj];
    V2 dr = calc_diff(s, P(s, i), P(s, j));
    double dist = sqrt(sum_sq(dr));
    if (dist > dist_max) return v2(0, 0);
    if (ri == rj) {
        int64_t diff = llabs(i - j);
        int64_t num_p = rc->num_particles[ti];
        if (diff == 1 || diff == num_p - 1) return v2(0, 0);
    }
    double fmod_;
    if (dist < dist_eq) fmod_ = -k_rep * (dist / dist_eq - 1);
    else fmod_ = (ri == rj) ? 0.0 : -k_atr * (dist / dist_eq - 1);
    return vscale(fmod_ / dist, dr);
}

/* calc_interaction (src/integration.jl:62-109): force on i exerted by j. */
static inline V2 calc_interaction(const OracleSys* s, int64_t i, int64_t j) {
    const MaviDynamicCfg* d = &s->p.dyn;
    switch (d->kind) {
    case MAVI_DYN_HARM_TRUNC: {          /* :62-66 */
        V2 dr = calc_diff(s, P(s, i), P(s, j));
        return harm_trunc_force(dr, sqrt(sum_sq(dr)), d->k_rep, d->k_atr, d->dist_eq, d->dist_max);
    }
    case MAVI_DYN_LEN_JONES: {           /* :62-66 */
        V2 dr = calc_diff(s, P(s, i), P(s, j));
        return len_jones_force(dr, sqrt(sum_sq(dr)), d->sigma, d->epsilon);
    }
    case MAVI_DYN_SZABO: {               /* :68-87 */
        V2 dr = calc_diff(s, P(s, i), P(s, j));
        double dist = sqrt(sum_sq(dr));
        if (dist > d->r_max) return v2(0, 0);
        double f_mod = (dist > d->r_eq) ? d->k_adh / (d->r_eq) : d->k_rep / (d->r_max - d->r_eq);
        double r = dist - d->r_eq;
        return vscale(-f_mod * r, dr);
    }
    case MAVI_DYN_RUN_TUMBLE: {          /* :89-109 */
        V2 dr = calc_diff(s, P(s, i), P(s, j));
        double dist = sqrt(sum_sq(dr));
        double sigma = d->sigma, epsilon = d->epsilon;
        double cutoff = pow(2.0, 1.0 / 6.0) * sigma;
        if (dist > cutoff) return v2(0, 0);
        double fmod_ = -4 * epsilon * (-12 * pow(sigma, 12) / pow(dist, 13) + 6 * pow(sigma, 6) / pow(dist, 7));
        return vscale(fmod_ / dist, dr);
    }
    case MAVI_DYN_RINGS:
        return rings_pair_force(s, i, j);
    }
    return v2(NAN, NAN);
}

/* ------------------------------------------------------------------------ */
/* chunks (src/chunks.jl)                                                    */
/* ------------------------------------------------------------------------ */

/* get_id inside get_neighbors(…, ::PeriodicWalls) (src/chunks.jl:64-73), 1-based. */
static int64_t periodic_get_id(int64_t x, int64_t num_t) {
    if (x == 0) return num_t;
    if (x % (num_t + 1) == 0) return 1;
    return x;
}

static void add_nbr(int64_t rows, int32_t* nbr, int32_t* cnt, int64_t row1, int64_t col1, int64_t nrow1,
                    int64_t ncol1) {
    int64_t c = (col1 - 1) * rows + (row1 - 1);
    int64_t nc = (ncol1 - 1) * rows + (nrow1 - 1);
    nbr[c * 4 + cnt[c]] = (int32_t)nc;
    cnt[c] += 1;
}

/* get_neighbors: periodic (src/chunks.jl:61-87) and open (:89-118), 0-based
 * column-major chunk ids. An open grid of one column and several rows indexes
 * column 0 (a BoundsError in the reference). */
static int neighbor_table(int64_t R, int64_t C, int periodic, int32_t* nbr, int32_t* cnt) {
    memset(cnt, 0, sizeof(int32_t) * R * C);
    if (periodic) {
        for (int64_t i = 1; i <= R; i++)
            for (int64_t j = 1; j <= C; j++) {
                add_nbr(R, nbr, cnt, i, j, periodic_get_id(i + 1, R), periodic_get_id(j, C));
                add_nbr(R, nbr, cnt, i, j, periodic_get_id(i + 1, R), periodic_get_id(j + 1, C));
                add_nbr(R, nbr, cnt, i, j, periodic_get_id(i, R), periodic_get_id(j + 1, C));
                add_nbr(R, nbr, cnt, i, j, periodic_get_id(i - 1, R), periodic_get_id(j + 1, C));
            }
        return MAVI_OK;
    }
    if (C < 2 && R > 1) return MAVI_ERR_UNSUPPORTED;
    for (int64_t i = 1; i <= R - 1; i++) {
        add_nbr(R, nbr, cnt, i, 1, i + 1, 1);
        add_nbr(R, nbr, cnt, i, 1, i + 1, 2);
        add_nbr(R, nbr, cnt, i, 1, i, 2);
        for (int64_t j = 2; j <= C - 1; j++) {
            add_nbr(R, nbr, cnt, i, j, i + 1, j - 1);
            add_nbr(R, nbr, cnt, i, j, i + 1, j);
            add_nbr(R, nbr, cnt, i, j, i + 1, j + 1);
            add_nbr(R, nbr, cnt, i, j, i, j + 1);
        }
        int64_t cl = (C - 1) * R + (i - 1);
        cnt[cl] = 0;    /* neighbors[i, num_cols] is assigned, not appended */
        add_nbr(R, nbr, cnt, i, C, i + 1, C - 1);
        add_nbr(R, nbr, cnt, i, C, i + 1, C);
    }
    for (int64_t j = 1; j <= C - 1; j++) add_nbr(R, nbr, cnt, R, j, R, j + 1);
    return MAVI_OK;
}

static int build_neighbors(OracleSys* s, int periodic) {
    if (!periodic && s->cols < 2) return MAVI_ERR_UNSUPPORTED; /* reference indexes column 0 (BoundsError) */
    return neighbor_table(s->rows, s->cols, periodic, s->nbr, s->nbr_cnt);
}

/* update_particle_chunk! index computation (src/chunks.jl:120-142). */
int32_t oracle_chunk_of(OracleSys* s, double x, double y, int64_t* row, int64_t* col) {
    double qr = oracle_julia_div(-y + s->bb_bly + s->bb_h, s->chunk_h);
    double qc = oracle_julia_div(x - s->bb_blx, s->chunk_l);
    if (!isfinite(qr) || !isfinite(qc)) return MAVI_ERR_NONFINITE;
    int64_t r = (int64_t)qr + 1;
    int64_t c = (int64_t)qc + 1;
    r -= (r == s->rows + 1) ? 1 : 0;
    c -= (c == s->cols + 1) ? 1 : 0;
    *row = r; *col = c;
    return MAVI_OK;
}

/* update_chunks! (src/chunks.jl:150-161; State-aware variant
 * src/integration.jl:54-59; rings src/rings/integration.jl:18-23):
 * particles are appended in ascending id order. */
int32_t oracle_update_chunks(OracleSys* s) {
    if (!s->has_chunks) return MAVI_OK;
    int64_t nch = (int64_t)s->rows * s->cols;
    memset(s->num_in_chunk, 0, sizeof(int32_t) * nch);
    for (int64_t k = 0; k < s->npids; k++) {
        int64_t i = s->pids[k];
        int64_t r, c;
        int32_t st = oracle_chunk_of(s, s->pos[2 * i], s->pos[2 * i + 1], &r, &c);
        if (st) return s->err = st;
        if (r < 1 || r > s->rows || c < 1 || c > s->cols) return s->err = MAVI_ERR_OUT_OF_GRID;
        int64_t ch = (c - 1) * s->rows + (r - 1);
        int32_t pi = s->num_in_chunk[ch];
        if (pi >= s->cap) return s->err = MAVI_ERR_CHUNK_OVERFLOW;
        s->chunk_particles[ch * s->cap + pi] = (int32_t)i;
        s->num_in_chunk[ch] += 1;
    }
    return MAVI_OK;
}

/* ------------------------------------------------------------------------ */
/* calc_forces!                                                              */
/* ------------------------------------------------------------------------ */

/* Chunk loop body shared by Sequencial (src/integration.jl:112-157) and each
 * thread of Threaded (:159-194): columns [c0, c1). */
static void chunk_force_columns(const OracleSys* s, double* F, int64_t c0, int64_t c1) {
    for (int64_t col = c0; col < c1; col++) {
        for (int64_t row = 0; row < s->rows; row++) {
            int64_t ch = col * s->rows + row;
            int32_t np = s->num_in_chunk[ch];
            const int32_t* chunk = s->chunk_particles + ch * s->cap;
            for (int32_t i = 0; i < np; i++) {
                int64_t p1 = chunk[i];
                for (int32_t j = i + 1; j < np; j++) {
                    int64_t p2 = chunk[j];
                    V2 f1 = calc_interaction(s, p1, p2);
                    F[2 * p1] += f1.x; F[2 * p1 + 1] += f1.y;
                    F[2 * p2] -= f1.x; F[2 * p2 + 1] -= f1.y;
                }
                for (int32_t k = 0; k < s->nbr_cnt[ch]; k++) {
                    int64_t nb = s->nbr[ch * 4 + k];
                    int32_t nnp = s->num_in_chunk[nb];
                    const int32_t* nchunk = s->chunk_particles + nb * s->cap;
                    for (int32_t j = 0; j < nnp; j++) {
                        int64_t p2 = nchunk[j];
                        V2 f1 = calc_interaction(s, p1, p2);
                        F[2 * p1] += f1.x; F[2 * p1 + 1] += f1.y;
                        F[2 * p2] -= f1.x; F[2 * p2 + 1] -= f1.y;
                    }
                }
            }
        }
    }
}

/* calc_forces!(system, ::Nothing, ::Sequencial) (src/integration.jl:197-224). */
static void all_pairs_forces(const OracleSys* s, double* F) {
    for (int64_t a = 0; a < s->npids; a++)
        for (int64_t b = a + 1; b < s->npids; b++) {
            int64_t pi = s->pids[a], pj = s->pids[b];
            V2 f = calc_interaction(s, pi, pj);
            F[2 * pi] += f.x; F[2 * pi + 1] += f.y;
            F[2 * pj] -= f.x; F[2 * pj + 1] -= f.y;
        }
}

static void clean_forces(OracleSys* s) {     /* src/systems.jl:119-123 */
    memset(s->forces, 0, sizeof(double) * 2 * s->n);
    if (s->slices) memset(s->slices, 0, sizeof(double) * 2 * s->n * (s->nthreads - 1));
}

static int32_t calc_forces(OracleSys* s, int32_t mode) {
    if (mode == ORACLE_FORCES_ALL_PAIRS || !s->has_chunks) {
        all_pairs_forces(s, s->forces);
        return MAVI_OK;
    }
    if (mode == ORACLE_FORCES_SEQUENTIAL || s->nthreads <= 1) {
        chunk_force_columns(s, s->forces, 0, s->cols);
        return MAVI_OK;
    }
    /* Threads.@threads :static over columns: contiguous blocks, the first
     * `rem` blocks one column longer; private slices summed in slice order. */
    int nt = s->nthreads;
    int64_t len = s->cols / nt, rem = s->cols % nt;
#pragma omp parallel for schedule(static, 1) num_threads(nt)
    for (int t = 0; t < nt; t++) {
        int64_t f = t * len, l = f + len;
        if (rem > 0) {
            if (t < rem) { f += t; l += t + 1; }
            else { f += rem; l += rem; }
        }
        double* F = (t == 0) ? s->forces : s->slices + (int64_t)(t - 1) * 2 * s->n;
        chunk_force_columns(s, F, f, l);
    }
    /* get_forces(system) .= sum(system.forces) */
    for (int64_t k = 0; k < 2 * s->n; k++) {
        double acc = s->forces[k];
        for (int t = 1; t < nt; t++) acc += s->slices[(int64_t)(t - 1) * 2 * s->n + k];
        s->forces[k] = acc;
    }
    return MAVI_OK;
}

/* ------------------------------------------------------------------------ */
/* calc_walls_forces! (src/integration.jl:228-266)                           */
/* ------------------------------------------------------------------------ */

static double process_dist(int mode, double dist, double inside_flag) {  /* src/configs.jl:259-261 */
    if (mode == MAVI_POTMODE_OUTSIDE) return inside_flag * dist;
    if (mode == MAVI_POTMODE_INSIDE) return -inside_flag * dist;
    return dist;
}

static V2 wall_potential_force(const MaviSpace* sp, V2 dr, double dist) {
    if (sp->pot_kind == MAVI_DYN_LEN_JONES)
        return len_jones_force(dr, dist, sp->pot_params[0], sp->pot_params[1]);
    return harm_trunc_force(dr, dist, sp->pot_params[0], sp->pot_params[1], sp->pot_params[2], sp->pot_params[3]);
}

static void walls_forces_space(OracleSys* s, const MaviSpace* sp) {
    if (sp->wall != MAVI_WALL_POTENTIAL) return;
    for (int64_t k = 0; k < s->npids; k++) {
        int64_t i = s->pids[k];
        V2 pos = P(s, i);
        if (sp->geometry == MAVI_GEOM_CIRCLE) {
            /* signed_pos(point, ::CircleCfg) (src/configs.jl:154-163) */
            V2 dr = vsub(pos, v2(sp->cx, sp->cy));
            double dist = pow(sum_sq(dr), .5);
            V2 dr_hat = v2(dr.x / dist, dr.y / dist);
            dr = vsub(dr, v2(dr_hat.x * sp->radius, dr_hat.y * sp->radius));
            double sign_dist = dist - sp->radius;
            double d2 = process_dist(sp->pot_mode, fabs(sign_dist), jsign(sign_dist));
            V2 f = wall_potential_force(sp, dr, d2);
            s->forces[2 * i] += f.x; s->forces[2 * i + 1] += f.y;
        } else if (sp->geometry == MAVI_GEOM_LINES) {
            for (int l = 0; l < sp->num_lines; l++) {
                /* Line2D (src/configs.jl:102-117) + signed_pos(point, ::Line2D) (:119-135) */
                V2 p1 = v2(sp->lines[l][0], sp->lines[l][1]);
                V2 p2 = v2(sp->lines[l][2], sp->lines[l][3]);
                V2 d = vsub(p2, p1);
                double norm = sqrt(d.x * d.x + d.y * d.y);
                V2 t = v2(d.x / norm, d.y / norm);
                V2 dr = vsub(pos, p1);
                double delta_t = dr.x * t.x + dr.y * t.y;
                if (delta_t > 0) {
                    if (delta_t < norm) {
                        V2 base = vadd(p1, v2(t.x * delta_t, t.y * delta_t));
                        dr = vsub(pos, base);
                    } else {
                        dr = vsub(pos, p2);
                    }
                }
                double dist = sqrt(sum_sq(dr));
                double d2 = process_dist(sp->pot_mode, dist, 1.0);
                V2 f = wall_potential_force(sp, dr, d2);
                s->forces[2 * i] += f.x; s->forces[2 * i + 1] += f.y;
            }
        }
    }
}

static void calc_walls_forces(OracleSys* s) {
    for (int k = 0; k < s->p.num_spaces; k++) walls_forces_space(s, &s->p.spaces[k]);
}

/* ------------------------------------------------------------------------ */
/* walls! (src/integration.jl:268-412)                                       */
/* ------------------------------------------------------------------------ */

/* get_particle_radius (src/systems.jl:131; rings per type src/rings/rings.jl:45-53). */
static double particle_radius_at(const OracleSys* s, int64_t pid) {
    if (s->p.state_kind == MAVI_STATE_RINGS) {
        int t = s->types[pid / s->nmax] - 1;
        return s->p.rings.inter_dist_eq[t][t] / 2.0;
    }
    return particle_radius_of(&s->p);
}

static void walls_space(OracleSys* s, const MaviSpace* sp) {
    double r = particle_radius_of(&s->p);
    if (sp->wall == MAVI_WALL_RIGID && sp->geometry == MAVI_GEOM_RECTANGLE) {   /* :271-285 */
        if (!s->vel) return;
        for (int64_t k = 0; k < s->npids; k++) {
            int64_t i = s->pids[k];
            double rx = s->pos[2 * i] - sp->bl_x, ry = s->pos[2 * i + 1] - sp->bl_y;
            int ox = (rx + r) > sp->length || (rx - r) < 0;
            int oy = (ry + r) > sp->height || (ry - r) < 0;
            if (ox || oy) {
                s->vel[2 * i] = s->vel[2 * i] * (-2 * ox + 1);
                s->vel[2 * i + 1] = s->vel[2 * i + 1] * (-2 * oy + 1);
            }
        }
    } else if (sp->wall == MAVI_WALL_RIGID && sp->geometry == MAVI_GEOM_CIRCLE) {  /* :287-306 */
        if (!s->vel) return;
        double max_r2 = (sp->radius - r) * (sp->radius - r);
        for (int64_t k = 0; k < s->npids; k++) {
            int64_t i = s->pids[k];
            double px = s->pos[2 * i], py = s->pos[2 * i + 1];
            double dx = px - sp->cx, dy = py - sp->cy;
            double d2x = dx * dx, d2y = dy * dy;
            double r2 = d2x + d2y;
            if (r2 <= max_r2) continue;
            double vx = s->vel[2 * i], vy = s->vel[2 * i + 1];
            double nvx = (vx * (d2y - d2x) - 2 * vy * px * py) / r2;
            double nvy = (-vy * (d2y - d2x) - 2 * vx * px * py) / r2;
            s->vel[2 * i] = nvx; s->vel[2 * i + 1] = nvy;
        }
    } else if (sp->wall == MAVI_WALL_PERIODIC && sp->geometry == MAVI_GEOM_RECTANGLE) { /* :309-324 */
        double cx = sp->bl_x + sp->length / 2, cy = sp->bl_y + sp->height / 2;
        double hx = sp->length / 2, hy = sp->height / 2;
        for (int64_t k = 0; k < s->npids; k++) {
            int64_t i = s->pids[k];
            double px = s->pos[2 * i], py = s->pos[2 * i + 1];
            double dx = px - cx, dy = py - cy;
            int ox = fabs(dx) > hx, oy = fabs(dy) > hy;
            if (ox || oy) {
                if (ox) s->pos[2 * i] = px - jsign(dx) * (hx * 2);
                if (oy) s->pos[2 * i + 1] = py - jsign(dy) * (hy * 2);
            }
        }
    } else if (sp->wall == MAVI_WALL_SLIPPERY && sp->geometry == MAVI_GEOM_LINES) {  /* :327-378 */
        for (int64_t k = 0; k < s->npids; k++) {
            int64_t pid = s->pids[k];
            double p_radius = particle_radius_at(s, pid);
            V2 pos_i = P(s, pid);     /* read once, as the reference does */
            for (int l = 0; l < sp->num_lines; l++) {
                V2 p1 = v2(sp->lines[l][0], sp->lines[l][1]);
                V2 p2 = v2(sp->lines[l][2], sp->lines[l][3]);
                V2 d = vsub(p2, p1);
                double norm = sqrt(d.x * d.x + d.y * d.y);
                V2 nrm = v2(-d.y / norm, d.x / norm);
                V2 tan_ = v2(d.x / norm, d.y / norm);
                V2 dr = vsub(pos_i, p1);
                double delta_s = dr.x * nrm.x + dr.y * nrm.y;
                if (fabs(delta_s) > p_radius) continue;
                double delta_t = dr.x * tan_.x + dr.y * tan_.y;
                int is_corner = 0; V2 corner_p = p1;
                if (delta_t > 0) {
                    if (delta_t > norm) {
                        if (delta_t > (norm + p_radius)) continue;
                        is_corner = 1; corner_p = p2;
                    }
                } else if (delta_t > -p_radius) {
                    is_corner = 1; corner_p = p1;
                } else {
                    continue;
                }
                if (is_corner) {
                    V2 drc = vsub(pos_i, corner_p);
                    double nn = sqrt(drc.x * drc.x + drc.y * drc.y);
                    if (nn > p_radius) continue;
                    double alpha = p_radius / nn - 1;
                    s->pos[2 * pid] += alpha * drc.x; s->pos[2 * pid + 1] += alpha * drc.y;
                } else {
                    double sgn = jsign(delta_s);
                    double alpha = sgn * (p_radius - sgn * delta_s);
                    s->pos[2 * pid] += alpha * nrm.x; s->pos[2 * pid + 1] += alpha * nrm.y;
                }
            }
        }
    } else if (sp->wall == MAVI_WALL_SLIPPERY && sp->geometry == MAVI_GEOM_CIRCLE) {  /* :380-401 */
        for (int64_t k = 0; k < s->npids; k++) {
            int64_t pid = s->pids[k];
            V2 p = P(s, pid);
            double pr = particle_radius_at(s, pid);
            double max_r_2 = (sp->radius + pr) * (sp->radius + pr);
            V2 dr = calc_diff(s, p, v2(sp->cx, sp->cy));
            double dr_2 = sum_sq(dr);
            if (dr_2 > max_r_2) continue;
            double dr_norm = sqrt(dr_2);
            double kk = sp->radius + pr - dr_norm;
            s->pos[2 * pid] = p.x + kk * dr.x / dr_norm;
            s->pos[2 * pid + 1] = p.y + kk * dr.y / dr_norm;
        }
    }
}

static void walls(OracleSys* s) {           /* ManyWalls: in order (:404-408) */
    for (int k = 0; k < s->p.num_spaces; k++) walls_space(s, &s->p.spaces[k]);
}

/* ------------------------------------------------------------------------ */
/* rings terms (src/rings/integration.jl)                                    */
/* ------------------------------------------------------------------------ */

static inline int32_t ring_n(const OracleSys* s, int64_t ring) {
    return s->p.rings.num_particles[s->types[ring] - 1];
}

/* get_rings_ids (src/rings/states.jl:35-38, 52-53): the active rings,
 * ascending; every ring without VarRingsIds. */
static inline int64_t rings_count(const OracleSys* s) { return s->var_ids ? s->num_active : s->num_rings; }
static inline int64_t ring_at(const OracleSys* s, int64_t k) { return s->var_ids ? s->ids[k] : k; }

/* update_continuos_pos! (src/rings/integration.jl:118-138): periodic only. */
static void update_continuos_pos(OracleSys* s) {
    const MaviSpace* sp = &s->p.spaces[0];
    int periodic = (sp->wall == MAVI_WALL_PERIODIC);
    for (int64_t k = 0; k < rings_count(s); k++) {
        int64_t ring = ring_at(s, k);
        int64_t base = ring * s->nmax;
        for (int64_t i = 0; i < s->nmax; i++) {
            s->cont_pos[2 * (base + i)] = s->pos[2 * (base + i)];
            s->cont_pos[2 * (base + i) + 1] = s->pos[2 * (base + i) + 1];
        }
        if (!periodic) continue;
        for (int64_t i = 1; i < ring_n(s, ring); i++) {
            V2 dr = calc_diff(s, P(s, base + i), P(s, base + i - 1));
            s->cont_pos[2 * (base + i)] = s->cont_pos[2 * (base + i - 1)] + dr.x;
            s->cont_pos[2 * (base + i) + 1] = s->cont_pos[2 * (base + i - 1) + 1] + dr.y;
        }
    }
}

/* calc_area (src/rings/integration.jl:103-116). */
static double calc_area(const double* rp, int32_t n) {
    double area = 0.0;
    for (int32_t i = 0; i < n - 1; i++)
        area += rp[2 * i] * rp[2 * (i + 1) + 1] - rp[2 * i + 1] * rp[2 * (i + 1)];
    area += rp[2 * (n - 1)] * rp[1] - rp[2 * (n - 1) + 1] * rp[0];
    return area / 2.0;
}

/* forces!: springs (src/rings/integration.jl:79-97, 205-223), area_forces!
 * (:140-195), then the bending term (an addition, zero when k_bend == 0):
 * E = k_bend * sum_i (1 - cos theta_i), theta_i the angle between the bonds
 * entering and leaving particle i. */
static void rings_bonded_forces(OracleSys* s) {
    const MaviRingsCfg* rc = &s->p.rings;
    double* F = s->forces;
    for (int64_t kr = 0; kr < rings_count(s); kr++) {
        int64_t ring = ring_at(s, kr);
        int t = s->types[ring] - 1;
        int32_t n = rc->num_particles[t];
        double k = rc->k_spring[t], l = rc->l_spring[t];
        for (int32_t sid = 0; sid < n; sid++) {
            int64_t p1 = ring * s->nmax + sid;
            int64_t p2 = ring * s->nmax + ((sid == n - 1) ? 0 : sid + 1);
            V2 dr = calc_diff(s, P(s, p1), P(s, p2));
            double dist = sqrt(sum_sq(dr));
            double fmod_ = -k * (dist - l);
            V2 f = vscale(fmod_ / dist, dr);
            F[2 * p1] += f.x; F[2 * p1 + 1] += f.y;
            F[2 * p2] -= f.x; F[2 * p2 + 1] -= f.y;
        }
    }
    for (int64_t kr = 0; kr < rings_count(s); kr++) {
        int64_t ring = ring_at(s, kr);
        int t = s->types[ring] - 1;
        int32_t n = rc->num_particles[t];
        double area = calc_area(s->cont_pos + 2 * ring * s->nmax, n);
        s->areas[ring] = area;
        double k_area = rc->k_area[t], p0 = rc->p0[t], l0 = rc->l_spring[t];
        double a0 = (n * l0 / p0);
        double area0 = a0 * a0;
        for (int32_t i = 0; i < n; i++) {
            double fmod_ = k_area * (area - area0);
            int32_t id1 = (i == 0) ? n - 1 : i - 1;
            int32_t id2 = (i == n - 1) ? 0 : i + 1;
            V2 dr = calc_diff(s, P(s, ring * s->nmax + id2), P(s, ring * s->nmax + id1));
            V2 a_deriv = v2(dr.y / 2, -dr.x / 2);
            int64_t idx = ring * s->nmax + i;
            F[2 * idx] -= fmod_ * a_deriv.x; F[2 * idx + 1] -= fmod_ * a_deriv.y;
        }
    }
    for (int64_t kr = 0; kr < rings_count(s); kr++) {
        int64_t ring = ring_at(s, kr);
        int t = s->types[ring] - 1;
        int32_t n = rc->num_particles[t];
        double kb = rc->k_bend[t];
        if (kb == 0.0) continue;
        for (int32_t i = 0; i < n; i++) {
            int64_t im = ring * s->nmax + ((i == 0) ? n - 1 : i - 1);
            int64_t ic = ring * s->nmax + i;
            int64_t ip = ring * s->nmax + ((i == n - 1) ? 0 : i + 1);
            V2 a = calc_diff(s, P(s, ic), P(s, im));
            V2 b = calc_diff(s, P(s, ip), P(s, ic));
            double la = sqrt(sum_sq(a)), lb = sqrt(sum_sq(b));
            double c = (a.x * b.x + a.y * b.y) / (la * lb);
            /* dc/da = b/(|a||b|) - c a/|a|^2 ; dc/db = a/(|a||b|) - c b/|b|^2 */
            V2 dca = v2(b.x / (la * lb) - c * a.x / (la * la), b.y / (la * lb) - c * a.y / (la * la));
            V2 dcb = v2(a.x / (la * lb) - c * b.x / (lb * lb), a.y / (la * lb) - c * b.y / (lb * lb));
            F[2 * im] += -kb * dca.x;            F[2 * im + 1] += -kb * dca.y;
            F[2 * ic] += kb * (dca.x - dcb.x);   F[2 * ic + 1] += kb * (dca.y - dcb.y);
            F[2 * ip] += kb * dcb.x;             F[2 * ip + 1] += kb * dcb.y;
        }
    }
}

/* update! (src/rings/integration.jl:300-351); noise: one N(0,1) per ring. */
static void rings_update(OracleSys* s, const double* noise) {
    const MaviRingsCfg* rc = &s->p.rings;
    double dt = s->p.dt;
    for (int64_t kr = 0; kr < rings_count(s); kr++) {
        int64_t ring = ring_at(s, kr);
        int t = s->types[ring] - 1;
        int32_t n = rc->num_particles[t];
        double vo = rc->vo[t], relax_time = rc->relax_time[t], mu = rc->mobility[t], dr = rc->rot_diff[t];
        double theta = s->pol[ring];
        V2 pol = v2(cos(theta), sin(theta));
        V2 vel_cm = v2(0, 0);
        for (int32_t i = 0; i < n; i++) {
            int64_t p = ring * s->nmax + i;
            V2 vel = vadd(vscale(vo, pol), vscale(mu, v2(s->forces[2 * p], s->forces[2 * p + 1])));
            vel_cm = vadd(vel_cm, vel);
            s->pos[2 * p] += vel.x * dt; s->pos[2 * p + 1] += vel.y * dt;
        }
        vel_cm = v2(vel_cm.x / n, vel_cm.y / n);
        double speed = sqrt(sum_sq(vel_cm));
        double cross;
        if (speed == 0) cross = 0;
        else {
            cross = (pol.x * vel_cm.y - pol.y * vel_cm.x) / speed;
            if (fabs(cross) > 1) cross = jsign(cross);
        }
        double d_theta = 1 / relax_time * asin(cross) * dt + sqrt(2 * dr * dt) * noise[ring];
        s->pol[ring] += d_theta;
    }
}

/* ------------------------------------------------------------------------ */
/* variable number of rings: sources and sinks (src/rings/sources.jl)        */
/* ------------------------------------------------------------------------ */

/* calc_active_ids! (src/rings/states.jl:200-219): ids and p_ids of the active
 * rings in ascending order; entries of ids past the count keep their values. */
static void update_ids(OracleSys* s) {
    int64_t pointer = 0, p_pointer = 0;
    for (int64_t ring = 0; ring < s->num_rings; ring++) {
        if (!s->mask[ring]) continue;
        s->ids[pointer++] = ring;
        for (int32_t i = 0; i < ring_n(s, ring); i++) s->pids[p_pointer++] = ring * s->nmax + i;
    }
    s->num_active = pointer;
    s->npids = p_pointer;
}

/* update_cms! (src/rings/integration.jl:366-372) with get_continuos_pos
 * (src/rings/rings.jl:31-41): positions, or the continuous positions of the
 * last update_continuos_pos! with periodic walls; summed in particle order. */
static void update_cms(OracleSys* s) {
    const double* src = (s->p.spaces[0].wall == MAVI_WALL_PERIODIC) ? s->cont_pos : s->pos;
    for (int64_t k = 0; k < rings_count(s); k++) {
        int64_t ring = ring_at(s, k);
        int32_t n = ring_n(s, ring);
        const double* rp = src + 2 * ring * s->nmax;
        double sx = rp[0], sy = rp[1];
        for (int32_t i = 1; i < n; i++) { sx += rp[2 * i]; sy += rp[2 * i + 1]; }
        s->cms[2 * ring] = sx / n;
        s->cms[2 * ring + 1] = sy / n;
    }
}

/* is_inside(point, ::RectangleCfg; pad) (src/configs.jl:89-93) */
static int inside_rect(double x, double y, double blx, double bly, double len, double h, double pad) {
    int ix = (blx - pad <= x) && (x <= blx + len + pad);
    int iy = (bly - pad <= y) && (y <= bly + h + pad);
    return ix && iy;
}

/* is_inside(point, sink geometry) (src/configs.jl:89-93, 165-168) */
static int sink_inside(const MaviSourceEntry* e, double x, double y) {
    if (e->geometry == MAVI_GEOM_CIRCLE) {
        double dx = x - e->cx, dy = y - e->cy;
        double rp = e->radius + 0.0;
        return dx * dx + dy * dy <= rp * rp;
    }
    return inside_rect(x, y, e->bl_x, e->bl_y, e->length, e->height, 0.0);
}

/* update_sources! (src/rings/integration.jl:353-358): each sink and source in
 * order. uniforms: one per random-polarisation box, in box order. */
static void process_sources(OracleSys* s, const double* uniforms) {
    int64_t b0 = 0, rnd = 0;
    for (int32_t e = 0; e < s->src_n; e++) {
        const MaviSourceEntry* E = &s->src[e];
        if (E->kind == MAVI_SRC_SINK) {
            /* process_sink! (src/rings/sources.jl:253-260): the view
             * ids[1:num_active] is taken once; remove_ring! decrements num_active */
            int64_t L = s->num_active;
            for (int64_t k = 0; k < L; k++) {
                int64_t ring = s->ids[k];
                if (sink_inside(E, s->cms[2 * ring], s->cms[2 * ring + 1])) {
                    s->mask[ring] = 0;
                    s->num_active -= 1;
                }
            }
            continue;
        }
        /* update_area_empty! (src/rings/sources.jl:193-224) for every box first */
        int32_t nb = E->num_boxes;
        int empty[MAVI_MAX_SPAWN_BOXES];
        for (int32_t b = 0; b < nb; b++) {
            const MaviSpawnBox* B = &s->boxes[b0 + b];
            empty[b] = 1;
            if (B->num_chunks < 0 || !s->has_chunks) {
                /* PosChecker: active particle ids of the last update_ids! */
                for (int64_t k = 0; k < s->npids && empty[b]; k++) {
                    int64_t i = s->pids[k];
                    if (inside_rect(s->pos[2 * i], s->pos[2 * i + 1], B->bl_x, B->bl_y, B->length, B->height, E->pad))
                        empty[b] = 0;
                }
            } else {
                /* ChunksChecker: the chunk lists of the last update_chunks! */
                const int32_t* rc = s->chunk_rc + 2 * s->box_chunk0[b0 + b];
                for (int32_t c = 0; c < B->num_chunks && empty[b]; c++) {
                    int64_t ch = (int64_t)rc[2 * c + 1] * s->rows + rc[2 * c];
                    for (int32_t q = 0; q < s->num_in_chunk[ch] && empty[b]; q++) {
                        int64_t i = s->chunk_particles[ch * s->cap + q];
                        if (inside_rect(s->pos[2 * i], s->pos[2 * i + 1], B->bl_x, B->bl_y, B->length, B->height,
                                        E->pad))
                            empty[b] = 0;
                    }
                }
            }
        }
        /* process_source! (:226-239) */
        for (int32_t b = 0; b < nb; b++) {
            double pol = E->pol;
            if (E->pol_mode == MAVI_SPAWN_POL_RANDOM) pol = uniforms[rnd++] * 2.0 * 3.141592653589793;
            if (!empty[b]) continue;
            /* add_ring! (src/rings/states.jl:162-174): the first inactive slot */
            int64_t ring = -1;
            for (int64_t i = 0; i < s->num_rings; i++)
                if (!s->mask[i]) { ring = i; break; }
            if (ring < 0) continue;
            const double* sp = s->spawn + 2 * (b0 + b) * s->nmax;
            memcpy(s->pos + 2 * ring * s->nmax, sp, sizeof(double) * 2 * s->nmax);
            s->pol[ring] = pol;
            s->mask[ring] = 1;
            int32_t mu = s->uids[0];
            for (int64_t i = 1; i < s->num_rings; i++) if (s->uids[i] > mu) mu = s->uids[i];
            s->uids[ring] = mu + 1;
            s->num_active += 1;
            int32_t n = ring_n(s, ring);
            double sx = sp[0], sy = sp[1];
            for (int32_t i = 1; i < n; i++) { sx += sp[2 * i]; sy += sp[2 * i + 1]; }
            s->cms[2 * ring] = sx / n;
            s->cms[2 * ring + 1] = sy / n;
        }
        b0 += nb;
    }
}

int32_t oracle_rings_sources(OracleSys* s, const int32_t* active_mask, int32_t num_entries,
                             const MaviSourceEntry* entries, const MaviSpawnBox* boxes, const double* spawn_xy,
                             const int32_t* chunk_rc) {
    if (s->p.state_kind != MAVI_STATE_RINGS) return MAVI_ERR_UNSUPPORTED;
    if (num_entries < 0 || num_entries > MAVI_MAX_SOURCE_ENTRIES) return MAVI_ERR_INVALID_ARG;
    if (!s->mask) {
        s->mask = (int32_t*)malloc(sizeof(int32_t) * s->num_rings);
        s->uids = (int32_t*)malloc(sizeof(int32_t) * s->num_rings);
        s->ids = (int64_t*)malloc(sizeof(int64_t) * s->num_rings);
        s->cms = (double*)calloc(2 * s->num_rings, sizeof(double));
    }
    for (int64_t r = 0; r < s->num_rings; r++) {
        s->mask[r] = active_mask ? (active_mask[r] != 0) : 1;
        s->uids[r] = (int32_t)(r + 1);
        s->ids[r] = r;
    }
    free(s->src); free(s->boxes); free(s->spawn); free(s->chunk_rc); free(s->box_chunk0);
    s->src_n = num_entries;
    s->src = (MaviSourceEntry*)malloc(sizeof(MaviSourceEntry) * (num_entries ? num_entries : 1));
    if (num_entries) memcpy(s->src, entries, sizeof(MaviSourceEntry) * num_entries);
    s->nbox = 0;
    s->n_random = 0;
    for (int32_t e = 0; e < num_entries; e++)
        if (entries[e].kind == MAVI_SRC_SOURCE) {
            if (entries[e].num_boxes < 1 || entries[e].num_boxes > MAVI_MAX_SPAWN_BOXES) return MAVI_ERR_INVALID_ARG;
            s->nbox += entries[e].num_boxes;
            if (entries[e].pol_mode == MAVI_SPAWN_POL_RANDOM) s->n_random += entries[e].num_boxes;
        }
    s->boxes = (MaviSpawnBox*)malloc(sizeof(MaviSpawnBox) * (s->nbox ? s->nbox : 1));
    s->box_chunk0 = (int64_t*)malloc(sizeof(int64_t) * (s->nbox ? s->nbox : 1));
    s->spawn = (double*)malloc(sizeof(double) * 2 * s->nmax * (s->nbox ? s->nbox : 1));
    int64_t nchunk = 0;
    for (int64_t b = 0; b < s->nbox; b++) {
        s->boxes[b] = boxes[b];
        s->box_chunk0[b] = nchunk;
        if (boxes[b].num_chunks > 0) nchunk += boxes[b].num_chunks;
    }
    if (s->nbox) memcpy(s->spawn, spawn_xy, sizeof(double) * 2 * s->nmax * s->nbox);
    s->chunk_rc = (int32_t*)malloc(sizeof(int32_t) * 2 * (nchunk ? nchunk : 1));
    if (nchunk) memcpy(s->chunk_rc, chunk_rc, sizeof(int32_t) * 2 * nchunk);
    s->var_ids = 1;
    /* RingsSystem(): update_continuos_pos!, update_ids!, update_chunks_all!
     * (src/rings/rings.jl:280-283) */
    update_ids(s);
    update_continuos_pos(s);
    return oracle_update_chunks(s);
}

int32_t oracle_rings_active(OracleSys* s, int32_t* active_mask, int32_t* uids, int32_t* num_active) {
    for (int64_t r = 0; r < s->num_rings; r++) {
        if (active_mask) active_mask[r] = s->var_ids ? s->mask[r] : 1;
        if (uids) uids[r] = s->var_ids ? s->uids[r] : (int32_t)(r + 1);
    }
    if (num_active) *num_active = (int32_t)rings_count(s);
    return MAVI_OK;
}

/* ------------------------------------------------------------------------ */
/* invasions (src/rings/integration.jl:378-520)                              */
/* ------------------------------------------------------------------------ */

/* point_line_intersect (:378-418): does the ray from p towards +x cross the
 * edge a-b? */
static int point_line_intersect(double px, double py, const double* a, const double* b) {
    double dx = b[0] - a[0];
    double dy = b[1] - a[1];
    if (dx == 0) {
        double x_inter = a[0];
        int check1 = x_inter > px;
        double y1 = a[1], y2 = b[1];
        if (dy < 0) { y1 = b[1]; y2 = a[1]; }
        int check2 = (y1 < py) && (py < y2);
        return check1 & check2;
    }
    if (dy == 0) return 0;
    double c = dy * a[0] - dx * a[1];
    double x_inter = (c + dx * py) / dy;
    int check1 = x_inter > px;
    double y1 = a[1], y2 = b[1];
    if (dy < 0) { y1 = b[1]; y2 = a[1]; }
    double x1 = a[0], x2 = b[0];
    if (dx < 0) { x1 = b[0]; x2 = a[0]; }
    int check2 = ((x1 < x_inter) && (x_inter < x2)) & ((y1 < py) && (py < y2));
    return check1 & check2;
}

/* ring_points (src/rings/rings.jl:31-43): continuous positions with
 * periodic walls, positions otherwise. */
static const double* ring_points(const OracleSys* s, int64_t ring) {
    const double* src = (s->p.spaces[0].wall == MAVI_WALL_PERIODIC) ? s->cont_pos : s->pos;
    return src + 2 * ring * s->nmax;
}

static void push_invasion(OracleSys* s, int64_t invasor, int64_t invaded, int64_t pi) {
    if (s->inv_n == s->inv_cap) {
        s->inv_cap = s->inv_cap ? 2 * s->inv_cap : 64;
        s->inv = (MaviInvasion*)realloc(s->inv, sizeof(MaviInvasion) * s->inv_cap);
    }
    MaviInvasion m;
    memset(&m, 0, sizeof(m));
    m.invasor = (int32_t)(invasor + 1);
    m.invaded = (int32_t)(invaded + 1);
    m.p_id = (int32_t)(invasor * s->nmax + pi + 1);   /* to_scalar_idx (src/rings/states.jl:137-140) */
    s->inv[s->inv_n++] = m;
}

/* polygons_intersect (:420-441) pushed as find_invasions! does (:443-470):
 * the points of ring a inside ring b, ascending. */
static void push_inside(OracleSys* s, int64_t a, int64_t b) {
    const double* pa = ring_points(s, a);
    const double* pb = ring_points(s, b);
    int32_t na = ring_n(s, a), nb = ring_n(s, b);
    for (int32_t id = 0; id < na; id++) {
        int count = 0;
        for (int32_t idx1 = 0; idx1 < nb; idx1++) {
            int32_t idx2 = (idx1 == nb - 1) ? 0 : idx1 + 1;
            if (point_line_intersect(pa[2 * id], pa[2 * id + 1], pb + 2 * idx1, pb + 2 * idx2)) count += 1;
        }
        if (count % 2 != 0) push_invasion(s, a, b, id);
    }
}

static void find_invasions(OracleSys* s, int64_t r1, int64_t r2) {
    /* both lists are formed before either is pushed; pushing does not change them */
    push_inside(s, r1, r2);
    push_inside(s, r2, r1);
}

/* check_invasions! (:472-509). With ring chunks: update_chunks!(r_chunks)
 * (src/rings/integration.jl:18-23 with update_particle_chunk!,
 * src/chunks.jl:120-147, on RingsInfo.cms), then every ring against the later
 * rings of its chunk and all rings of the neighbour chunks; the list is
 * emptied first. Without: ring ids 1:length(get_rings_ids), list kept. */
static int32_t check_invasions(OracleSys* s) {
    if (s->rcols == 0) {
        int64_t L = rings_count(s);
        for (int64_t r1 = 0; r1 < L; r1++)
            for (int64_t r2 = r1 + 1; r2 < L; r2++) find_invasions(s, r1, r2);
        return MAVI_OK;
    }
    s->inv_n = 0;
    int64_t R = s->rrows, C = s->rcols, nch = R * C;
    memset(s->rcount, 0, sizeof(int32_t) * nch);
    int64_t L = rings_count(s);
    int32_t* cell = (int32_t*)malloc(sizeof(int32_t) * (L ? L : 1));
    for (int64_t k = 0; k < L; k++) {
        int64_t ring = ring_at(s, k);
        double x = s->cms[2 * ring], y = s->cms[2 * ring + 1];
        double qr = oracle_julia_div(-y + s->r_bly + s->r_h, s->r_ch);
        double qc = oracle_julia_div(x - s->r_blx, s->r_cl);
        if (!isfinite(qr) || !isfinite(qc) || fabs(qr) >= 4e18 || fabs(qc) >= 4e18) {
            free(cell);
            return MAVI_ERR_NONFINITE;
        }
        int64_t row = (int64_t)qr + 1, col = (int64_t)qc + 1;
        row -= (row == R + 1) ? 1 : 0;
        col -= (col == C + 1) ? 1 : 0;
        if (row < 1 || row > R || col < 1 || col > C) { free(cell); return MAVI_ERR_OUT_OF_GRID; }
        cell[k] = (int32_t)((col - 1) * R + (row - 1));
        s->rcount[cell[k]] += 1;
    }
    int32_t acc = 0;
    for (int64_t c = 0; c < nch; c++) { s->rstart[c] = acc; acc += s->rcount[c]; s->rcount[c] = 0; }
    for (int64_t k = 0; k < L; k++) {
        int32_t c = cell[k];
        s->rlist[s->rstart[c] + s->rcount[c]++] = (int32_t)ring_at(s, k);
    }
    free(cell);
    for (int64_t col = 0; col < C; col++)
        for (int64_t row = 0; row < R; row++) {
            int64_t c = col * R + row;
            int32_t np = s->rcount[c];
            const int32_t* chunk = s->rlist + s->rstart[c];
            for (int32_t i = 0; i < np; i++) {
                int64_t r1 = chunk[i];
                for (int32_t j = i + 1; j < np; j++) find_invasions(s, r1, chunk[j]);
                for (int32_t q = 0; q < s->rnbr_cnt[c]; q++) {
                    int32_t nb = s->rnbr[4 * c + q];
                    for (int32_t j = 0; j < s->rcount[nb]; j++) find_invasions(s, r1, s->rlist[s->rstart[nb] + j]);
                }
            }
        }
    return MAVI_OK;
}

/* update_invasions! (:511-520) */
static int32_t update_invasions(OracleSys* s) {
    if (!s->inv_on) return MAVI_OK;
    if (s->num_steps - s->inv_last < s->inv_steps) return MAVI_OK;
    s->inv_last = s->num_steps;
    return check_invasions(s);
}

int32_t oracle_rings_invasions_config(OracleSys* s, int32_t enable, int64_t steps_to_update, int32_t num_cols,
                                      int32_t num_rows) {
    if (s->p.state_kind != MAVI_STATE_RINGS) return MAVI_ERR_UNSUPPORTED;
    if (num_cols < 0 || num_rows < 0 || ((num_cols == 0) != (num_rows == 0))) return MAVI_ERR_INVALID_ARG;
    free(s->rnbr); free(s->rnbr_cnt); free(s->rcount); free(s->rstart); free(s->rlist);
    s->rnbr = s->rnbr_cnt = s->rcount = s->rstart = s->rlist = NULL;
    s->inv_on = enable != 0;
    s->inv_steps = steps_to_update;
    s->inv_n = 0;
    s->rcols = enable ? num_cols : 0;
    s->rrows = enable ? num_rows : 0;
    if (s->rcols > 0) {
        int64_t nch = (int64_t)s->rrows * s->rcols;
        s->rnbr = (int32_t*)calloc(4 * nch, sizeof(int32_t));
        s->rnbr_cnt = (int32_t*)calloc(nch, sizeof(int32_t));
        s->rcount = (int32_t*)calloc(nch, sizeof(int32_t));
        s->rstart = (int32_t*)calloc(nch, sizeof(int32_t));
        s->rlist = (int32_t*)calloc(s->num_rings ? s->num_rings : 1, sizeof(int32_t));
        int32_t st = neighbor_table(s->rrows, s->rcols, s->p.spaces[0].wall == MAVI_WALL_PERIODIC, s->rnbr,
                                    s->rnbr_cnt);
        if (st) return st;
        bbox_of(&s->p, &s->r_len, &s->r_h, &s->r_blx, &s->r_bly);
        s->r_cl = s->r_len / s->rcols;
        s->r_ch = s->r_h / s->rrows;
    }
    if (!s->cms) s->cms = (double*)calloc(2 * s->num_rings, sizeof(double));
    /* RingsSystem() (src/rings/rings.jl:276-284): last_check = num_steps,
     * update_continuos_pos!, update_cms!, then update_invasions! */
    s->inv_last = s->num_steps;
    update_continuos_pos(s);
    update_cms(s);
    return update_invasions(s);
}

int32_t oracle_rings_invasions(OracleSys* s, MaviInvasion* out, int64_t capacity, int64_t* count,
                               int64_t* last_check) {
    int64_t n = s->inv_n < capacity ? s->inv_n : capacity;
    if (n > 0) memcpy(out, s->inv, sizeof(MaviInvasion) * n);
    if (count) *count = s->inv_n;
    if (last_check) *last_check = s->inv_last;
    return MAVI_OK;
}

/* ------------------------------------------------------------------------ */
/* integrators (src/integration.jl:415-498)                                  */
/* ------------------------------------------------------------------------ */

static void update_szabo(OracleSys* s, const double* noise) {      /* :433-465 */
    const MaviDynamicCfg* d = &s->p.dyn;
    double dt = s->p.dt;
    double vo = d->vo, relax_time = d->relax_time, mu = d->mobility, dr = d->rot_diff;
    for (int64_t i = 0; i < s->n; i++) {
        double theta = s->pol[i];
        V2 pol = v2(cos(theta), sin(theta));
        V2 vel = vadd(vscale(vo, pol), vscale(mu, v2(s->forces[2 * i], s->forces[2 * i + 1])));
        double speed = sqrt(fabs(vel.x) + fabs(vel.y));
        double cross = (speed > 0) ? (pol.x * vel.y - pol.y * vel.x) / speed : 0;
        if (fabs(cross) > 1) cross = jsign(cross);
        double d_theta = 1 / relax_time * asin(cross) * dt + sqrt(2 * dr * dt) * noise[i];
        s->pos[2 * i] += vel.x * dt; s->pos[2 * i + 1] += vel.y * dt;
        s->pol[i] += d_theta;
    }
}

static void update_rtp(OracleSys* s, const double* noise) {        /* :467-498 */
    const MaviDynamicCfg* d = &s->p.dyn;
    double dt = s->p.dt;
    for (int64_t i = 0; i < s->n; i++) {
        double theta = s->pol[i];
        V2 pol = v2(cos(theta), sin(theta));
        V2 vel = vadd(vscale(d->vo, pol), v2(s->forces[2 * i], s->forces[2 * i + 1]));
        s->pos[2 * i] += vel.x * dt; s->pos[2 * i + 1] += vel.y * dt;
        double u = noise[2 * i];
        if (u < d->tumble_rate * dt) s->pol[i] = 2 * M_PI * noise[2 * i + 1];
    }
}

int64_t oracle_noise_count(OracleSys* s) {
    switch (s->p.step_kind) {
    case MAVI_STEP_SZABO: return s->n;
    case MAVI_STEP_RTP: return 2 * s->n;
    case MAVI_STEP_RINGS: return s->num_rings + (s->var_ids ? s->n_random : 0);
    }
    return 0;
}

static void update_time(OracleSys* s) {                            /* :500-503 */
    s->time += s->p.dt;
    s->num_steps += 1;
}

/* One step of the replica's step function. */
static int32_t step_once(OracleSys* s, int32_t fm, const double* noise) {
    int32_t st;
    double dt = s->p.dt;
    switch (s->p.step_kind) {
    case MAVI_STEP_NEWTON: {                                        /* :507-515 */
        clean_forces(s);
        if ((st = oracle_update_chunks(s))) return st;
        calc_forces(s, fm);
        calc_walls_forces(s);
        /* update_verlet! (:415-431) */
        double* old = (double*)malloc(sizeof(double) * 2 * s->n);
        memcpy(old, s->forces, sizeof(double) * 2 * s->n);
        double term = dt * dt / 2;
        for (int64_t k = 0; k < 2 * s->n; k++) s->pos[k] += s->vel[k] * dt + s->forces[k] * term;
        clean_forces(s);
        calc_forces(s, fm);
        for (int64_t k = 0; k < 2 * s->n; k++) s->vel[k] += dt / 2 * (s->forces[k] + old[k]);
        free(old);
        walls(s);
        update_time(s);
        return MAVI_OK;
    }
    case MAVI_STEP_OVERDAMPED: {
        clean_forces(s);
        if ((st = oracle_update_chunks(s))) return st;
        calc_forces(s, fm);
        calc_walls_forces(s);
        double mdt = s->p.dyn.mobility * dt;
        for (int64_t k = 0; k < 2 * s->n; k++) s->pos[k] += s->forces[k] * mdt;
        walls(s);
        update_time(s);
        return MAVI_OK;
    }
    case MAVI_STEP_SZABO:                                           /* :517-525 */
    case MAVI_STEP_RTP:                                             /* :527-535 */
        clean_forces(s);
        if ((st = oracle_update_chunks(s))) return st;
        calc_forces(s, fm);
        calc_walls_forces(s);
        if (s->p.step_kind == MAVI_STEP_SZABO) update_szabo(s, noise);
        else update_rtp(s, noise);
        walls(s);
        update_time(s);
        return MAVI_OK;
    case MAVI_STEP_RINGS:                           /* src/rings/integration.jl:522-543 */
        if (s->var_ids || s->inv_on) update_cms(s);
        if (s->var_ids) {
            process_sources(s, noise ? noise + s->num_rings : NULL);
            update_ids(s);
        }
        if ((st = oracle_update_chunks(s))) return st;
        update_continuos_pos(s);
        if ((st = update_invasions(s))) return st;
        clean_forces(s);
        calc_forces(s, fm);
        rings_bonded_forces(s);
        calc_walls_forces(s);
        rings_update(s, noise);
        walls(s);
        s->num_steps += 1;
        s->time += dt;
        return MAVI_OK;
    }
    return MAVI_ERR_UNSUPPORTED;
}

int32_t oracle_step(OracleSys* s, int64_t nsteps, int32_t force_mode, const double* noise) {
    int64_t nc = oracle_noise_count(s);
    for (int64_t k = 0; k < nsteps; k++) {
        int32_t st = step_once(s, force_mode, noise ? noise + k * nc : NULL);
        if (st) return s->err = st;
    }
    return MAVI_OK;
}

int32_t oracle_calc_forces(OracleSys* s, int32_t mode, int32_t include_walls, double* out) {
    int32_t st;
    clean_forces(s);
    if ((st = oracle_update_chunks(s))) return st;
    if (s->p.state_kind == MAVI_STATE_RINGS) update_continuos_pos(s);
    calc_forces(s, mode);
    if (s->p.state_kind == MAVI_STATE_RINGS) rings_bonded_forces(s);
    if (include_walls) calc_walls_forces(s);
    memcpy(out, s->forces, sizeof(double) * 2 * s->n);
    return MAVI_OK;
}

/* ------------------------------------------------------------------------ */
/* energies (src/quantities.jl)                                              */
/* ------------------------------------------------------------------------ */

/* Pair potential consistent with each force law. LenJones follows
 * src/quantities.jl:46-66; the HarmTrunc energy of the reference
 * (:21-44) reads fields that do not exist, so it is written from the force
 * law: U = k/(2 dist_eq) (d - dist_eq)^2, k = k_rep below dist_eq, k_atr
 * above, 0 beyond dist_max. RunTumble is the unshifted WCA. */
static double pair_energy(const OracleSys* s, int64_t i, int64_t j) {
    const MaviDynamicCfg* d = &s->p.dyn;
    V2 dr = calc_diff(s, P(s, i), P(s, j));
    double dist = sqrt(sum_sq(dr));
    switch (d->kind) {
    case MAVI_DYN_LEN_JONES:
        return pow(d->sigma / dist, 12) - pow(d->sigma / dist, 6);     /* times 4 eps later */
    case MAVI_DYN_HARM_TRUNC: {
        if (dist > d->dist_max) return 0.0;
        double k = dist < d->dist_eq ? d->k_rep : d->k_atr;
        double x = dist - d->dist_eq;
        return k / (2 * d->dist_eq) * x * x;
    }
    case MAVI_DYN_RUN_TUMBLE: {
        if (dist > pow(2.0, 1.0 / 6.0) * d->sigma) return 0.0;
        return pow(d->sigma / dist, 12) - pow(d->sigma / dist, 6);
    }
    }
    return NAN;
}

int32_t oracle_energies(OracleSys* s, int32_t pe_mode, double* ke, double* pe) {
    double k = 0;
    if (s->vel) {
        for (int64_t i = 0; i < s->n; i++) k += s->vel[2 * i] * s->vel[2 * i] + s->vel[2 * i + 1] * s->vel[2 * i + 1];
    }
    *ke = k / 2;
    int kind = s->p.dyn.kind;
    if (kind != MAVI_DYN_LEN_JONES && kind != MAVI_DYN_HARM_TRUNC && kind != MAVI_DYN_RUN_TUMBLE) {
        *pe = NAN;
        return MAVI_OK;
    }
    double pot = 0.0;
    if (pe_mode == MAVI_PE_ALL_PAIRS || !s->has_chunks) {
        for (int64_t a = 0; a < s->npids; a++)
            for (int64_t b = a + 1; b < s->npids; b++) pot += pair_energy(s, s->pids[a], s->pids[b]);
    } else {
        int32_t st = oracle_update_chunks(s);
        if (st) return st;
        for (int64_t col = 0; col < s->cols; col++)
            for (int64_t row = 0; row < s->rows; row++) {
                int64_t ch = col * s->rows + row;
                int32_t np = s->num_in_chunk[ch];
                const int32_t* chunk = s->chunk_particles + ch * s->cap;
                for (int32_t i = 0; i < np; i++) {
                    for (int32_t j = i + 1; j < np; j++) pot += pair_energy(s, chunk[i], chunk[j]);
                    for (int32_t kk = 0; kk < s->nbr_cnt[ch]; kk++) {
                        int64_t nb = s->nbr[ch * 4 + kk];
                        for (int32_t j = 0; j < s->num_in_chunk[nb]; j++)
                            pot += pair_energy(s, chunk[i], s->chunk_particles[nb * s->cap + j]);
                    }
                }
            }
    }
    if (kind != MAVI_DYN_HARM_TRUNC) pot *= 4 * s->p.dyn.epsilon;
    *pe = pot;
    return MAVI_OK;
}

int64_t oracle_count_pairs(OracleSys* s) {
    if (!s->has_chunks) return s->npids * (s->npids - 1) / 2;
    if (oracle_update_chunks(s)) return -1;
    int64_t pairs = 0;
    for (int64_t ch = 0; ch < (int64_t)s->rows * s->cols; ch++) {
        int64_t np = s->num_in_chunk[ch];
        pairs += np * (np - 1) / 2;
        for (int32_t k = 0; k < s->nbr_cnt[ch]; k++) pairs += np * s->num_in_chunk[s->nbr[ch * 4 + k]];
    }
    return pairs;
}

/* Pair-distance histogram (the counts behind the pair distribution g(r)),
 * the definition mavi_pair_distribution implements: every unordered pair of
 * the chunk loop of calc_forces! (src/integration.jl:112-157; all active
 * pairs without chunks, :197-224) whose calc_diff length d is below r_max
 * adds one to bin floor(d / dr), dr = r_max / nbins (the last bin also takes
 * a division that rounds up to nbins). r_max must not exceed the chunk
 * sides, so the chunk loop holds every such pair. */
int32_t oracle_pair_distribution(OracleSys* s, double r_max, int32_t nbins, uint64_t* counts) {
    if (nbins < 1 || !(r_max > 0)) return MAVI_ERR_INVALID_ARG;
    memset(counts, 0, sizeof(uint64_t) * (size_t)nbins);
    const double dr = r_max / nbins;
    #define HIST_PAIR(I, J) do {                                                             \
        V2 d_ = calc_diff(s, P(s, (I)), P(s, (J)));                                          \
        double dd_ = sqrt(sum_sq(d_));                                                       \
        if (dd_ < r_max) {                                                                   \
            int32_t k_ = (int32_t)(dd_ / dr);                                                \
            counts[k_ > nbins - 1 ? nbins - 1 : k_]++;                                       \
        }                                                                                    \
    } while (0)
    if (!s->has_chunks) {
        for (int64_t a = 0; a < s->npids; a++)
            for (int64_t b = a + 1; b < s->npids; b++) HIST_PAIR(s->pids[a], s->pids[b]);
        return MAVI_OK;
    }
    if (oracle_update_chunks(s)) return s->err;
    for (int64_t col = 0; col < s->cols; col++) {
        for (int64_t row = 0; row < s->rows; row++) {
            int64_t ch = col * s->rows + row;
            int32_t np = s->num_in_chunk[ch];
            const int32_t* chunk = s->chunk_particles + ch * s->cap;
            for (int32_t i = 0; i < np; i++) {
                int64_t p1 = chunk[i];
                for (int32_t j = i + 1; j < np; j++) HIST_PAIR(p1, (int64_t)chunk[j]);
                for (int32_t k = 0; k < s->nbr_cnt[ch]; k++) {
                    int64_t nb = s->nbr[ch * 4 + k];
                    const int32_t* nchunk = s->chunk_particles + nb * s->cap;
                    for (int32_t j = 0; j < s->num_in_chunk[nb]; j++) HIST_PAIR(p1, (int64_t)nchunk[j]);
                }
            }
        }
    }
    #undef HIST_PAIR
    return MAVI_OK;
}

/* Particle neighbour lists of the rings model (src/rings/neighbors.jl:116-136,
 * called from calc_interaction, src/rings/integration.jl:32-44): every
 * candidate pair (i, j) of the chunk loop with dist < max_dist * tol, where
 * max_dist = 2 * particle_radius(interaction) = dist_eq of the pair's types,
 * and (type :all or different rings) adds j to i's list and i to j's list,
 * in the loop order of calc_forces! (src/integration.jl:112-157). `lists`
 * (n x max_list, may be NULL) receives 0-based slot ids; a list longer than
 * max_list is an error (the reference's array bound). */
int32_t oracle_rings_neighbors(OracleSys* s, double tol, int32_t type_all, int32_t max_list, int32_t* counts,
                               int32_t* lists) {
    if (s->p.dyn.kind != MAVI_DYN_RINGS || !s->has_chunks) return MAVI_ERR_INVALID_ARG;
    if (oracle_update_chunks(s)) return s->err;
    const MaviRingsCfg* rc = &s->p.rings;
    memset(counts, 0, sizeof(int32_t) * s->n);
    int32_t st = MAVI_OK;
    #define NEIGH_PAIR(I, J) do {                                                          \
        int64_t ri_ = (I) / s->nmax, rj_ = (J) / s->nmax;                                   \
        int ti_ = s->types[ri_] - 1, tj_ = s->types[rj_] - 1;                               \
        V2 dr_ = calc_diff(s, P(s, (I)), P(s, (J)));                                        \
        double dist_ = sqrt(sum_sq(dr_));                                                   \
        double max_dist_ = 2 * (rc->inter_dist_eq[ti_][tj_] / 2.0);                         \
        if (dist_ < max_dist_ * tol && (type_all || ri_ != rj_)) {                          \
            int32_t ci_ = ++counts[(I)], cj_ = ++counts[(J)];                               \
            if (lists) {                                                                    \
                if (ci_ > max_list || cj_ > max_list) st = MAVI_ERR_CHUNK_OVERFLOW;         \
                else { lists[(I) * max_list + ci_ - 1] = (int32_t)(J);                      \
                       lists[(J) * max_list + cj_ - 1] = (int32_t)(I); }                    \
            }                                                                               \
        }                                                                                   \
    } while (0)
    for (int64_t col = 0; col < s->cols; col++) {
        for (int64_t row = 0; row < s->rows; row++) {
            int64_t ch = col * s->rows + row;
            int32_t np = s->num_in_chunk[ch];
            const int32_t* chunk = s->chunk_particles + ch * s->cap;
            for (int32_t i = 0; i < np; i++) {
                int64_t p1 = chunk[i];
                for (int32_t j = i + 1; j < np; j++) NEIGH_PAIR(p1, (int64_t)chunk[j]);
                for (int32_t k = 0; k < s->nbr_cnt[ch]; k++) {
                    int64_t nb = s->nbr[ch * 4 + k];
                    const int32_t* nchunk = s->chunk_particles + nb * s->cap;
                    for (int32_t j = 0; j < s->num_in_chunk[nb]; j++) NEIGH_PAIR(p1, (int64_t)nchunk[j]);
                }
            }
        }
    }
    #undef NEIGH_PAIR
    return st;
}

/* ------------------------------------------------------------------------ */
/* construction                                                              */
/* ------------------------------------------------------------------------ */

/* check_inside (src/space_checks.jl:9-37, 53-60): rectangle bounds; circle
 * tests |p|^2 > R^2 around the origin (the reference ignores the centre). */
static int outside_space(const OracleSys* s) {
    if (s->p.num_spaces != 1) return 0;           /* ManyGeometries: no check */
    const MaviSpace* sp = &s->p.spaces[0];
    for (int64_t k = 0; k < s->npids; k++) {
        int64_t i = s->pids[k];
        double x = s->pos[2 * i], y = s->pos[2 * i + 1];
        if (sp->geometry == MAVI_GEOM_RECTANGLE) {
            if (x < sp->bl_x || y < sp->bl_y || x > sp->bl_x + sp->length || y > sp->bl_y + sp->height) return 1;
        } else if (sp->geometry == MAVI_GEOM_CIRCLE) {
            if (x * x + y * y > sp->radius * sp->radius) return 1;
        }
    }
    return 0;
}

OracleSys* oracle_create(const MaviReplicaParams* p, const double* pos, const double* vel,
                         const double* pol, const int32_t* ring_types, int32_t nthreads,
                         int32_t* status) {
    OracleSys* s = (OracleSys*)calloc(1, sizeof(OracleSys));
    s->p = *p;
    s->n = p->num_particles;
    s->pos = (double*)malloc(sizeof(double) * 2 * s->n);
    memcpy(s->pos, pos, sizeof(double) * 2 * s->n);
    if (p->state_kind == MAVI_STATE_SECOND_LAW && vel) {
        s->vel = (double*)malloc(sizeof(double) * 2 * s->n);
        memcpy(s->vel, vel, sizeof(double) * 2 * s->n);
    }
    s->forces = (double*)calloc(2 * s->n, sizeof(double));
    if (p->state_kind == MAVI_STATE_RINGS) {
        s->num_rings = p->rings.num_rings;
        s->nmax = p->rings.nmax;
        s->types = (int32_t*)malloc(sizeof(int32_t) * s->num_rings);
        for (int64_t r = 0; r < s->num_rings; r++) s->types[r] = ring_types ? ring_types[r] : 1;
        s->pol = (double*)malloc(sizeof(double) * s->num_rings);
        memcpy(s->pol, pol, sizeof(double) * s->num_rings);
        s->cont_pos = (double*)calloc(2 * s->n, sizeof(double));
        s->areas = (double*)calloc(s->num_rings, sizeof(double));
        /* FixRingsIds p_ids (src/rings/states.jl:46-62) */
        s->pids = (int64_t*)malloc(sizeof(int64_t) * s->n);
        s->npids = 0;
        for (int64_t r = 0; r < s->num_rings; r++)
            for (int32_t i = 0; i < ring_n(s, r); i++) s->pids[s->npids++] = r * s->nmax + i;
    } else {
        if (p->state_kind == MAVI_STATE_SELF_PROPELLED) {
            s->pol = (double*)malloc(sizeof(double) * s->n);
            memcpy(s->pol, pol, sizeof(double) * s->n);
        }
        s->pids = (int64_t*)malloc(sizeof(int64_t) * s->n);
        for (int64_t i = 0; i < s->n; i++) s->pids[i] = i;
        s->npids = s->n;
    }
    *status = MAVI_OK;
    if (outside_space(s)) { *status = MAVI_ERR_OUTSIDE_SPACE; }
    s->nthreads = 1;
    oracle_set_threads(s, nthreads);
    if (p->chunk_cols > 0 && p->chunk_rows > 0) {
        /* get_chunks (src/systems.jl:14-28) + Chunks (src/chunks.jl:26-40) */
        s->has_chunks = 1;
        s->rows = p->chunk_rows; s->cols = p->chunk_cols;
        bbox_of(p, &s->bb_len, &s->bb_h, &s->bb_blx, &s->bb_bly);
        s->chunk_l = s->bb_len / s->cols;
        s->chunk_h = s->bb_h / s->rows;
        double pr = particle_radius_of(p);
        double nc = (ceil(0.5 * s->chunk_l / pr) + 1) * ((ceil(0.5 * s->chunk_h / pr) + 1));
        s->cap = (int32_t)ceil(nc * 2);
        int64_t nch = (int64_t)s->rows * s->cols;
        s->chunk_particles = (int32_t*)malloc(sizeof(int32_t) * nch * s->cap);
        s->num_in_chunk = (int32_t*)calloc(nch, sizeof(int32_t));
        s->nbr = (int32_t*)calloc(nch * 4, sizeof(int32_t));
        s->nbr_cnt = (int32_t*)calloc(nch, sizeof(int32_t));
        int32_t st = build_neighbors(s, p->spaces[0].wall == MAVI_WALL_PERIODIC);
        if (st && *status == MAVI_OK) *status = st;
        if (*status == MAVI_OK) {
            st = oracle_update_chunks(s);
            if (st) *status = st;
        }
    }
    return s;
}

int32_t oracle_set_threads(OracleSys* s, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    free(s->slices);
    s->slices = NULL;
    s->nthreads = nthreads;
    if (nthreads > 1) s->slices = (double*)calloc((size_t)(nthreads - 1) * 2 * s->n, sizeof(double));
    return MAVI_OK;
}

void oracle_destroy(OracleSys* s) {
    if (!s) return;
    free(s->pos); free(s->vel); free(s->pol); free(s->types); free(s->forces); free(s->slices);
    free(s->pids); free(s->chunk_particles); free(s->num_in_chunk); free(s->nbr); free(s->nbr_cnt);
    free(s->cont_pos); free(s->areas);
    free(s->rnbr); free(s->rnbr_cnt); free(s->rcount); free(s->rstart); free(s->rlist); free(s->inv);
    free(s->mask); free(s->uids); free(s->ids); free(s->cms);
    free(s->src); free(s->boxes); free(s->spawn); free(s->chunk_rc); free(s->box_chunk0);
    free(s);
}

int32_t oracle_chunk_geometry(OracleSys* s, int32_t* rows, int32_t* cols, int32_t* cap) {
    *rows = s->rows; *cols = s->cols; *cap = s->cap;
    return MAVI_OK;
}

int32_t oracle_get_chunks(OracleSys* s, int32_t* num_in_chunk, int32_t* chunk_particles) {
    if (!s->has_chunks) return MAVI_ERR_INVALID_ARG;
    int64_t nch = (int64_t)s->rows * s->cols;
    memcpy(num_in_chunk, s->num_in_chunk, sizeof(int32_t) * nch);
    for (int64_t c = 0; c < nch; c++)
        for (int32_t k = 0; k < s->cap; k++)
            chunk_particles[c * s->cap + k] = (k < s->num_in_chunk[c]) ? s->chunk_particles[c * s->cap + k] : -1;
    return MAVI_OK;
}

int32_t oracle_get_neighbors(OracleSys* s, int32_t* counts, int32_t* nbr) {
    if (!s->has_chunks) return MAVI_ERR_INVALID_ARG;
    int64_t nch = (int64_t)s->rows * s->cols;
    memcpy(counts, s->nbr_cnt, sizeof(int32_t) * nch);
    memcpy(nbr, s->nbr, sizeof(int32_t) * nch * 4);
    return MAVI_OK;
}

int32_t oracle_get_state(OracleSys* s, double* pos, double* vel, double* pol) {
    if (pos) memcpy(pos, s->pos, sizeof(double) * 2 * s->n);
    if (vel && s->vel) memcpy(vel, s->vel, sizeof(double) * 2 * s->n);
    if (pol && s->pol) {
        int64_t np = (s->p.state_kind == MAVI_STATE_RINGS) ? s->num_rings : s->n;
        memcpy(pol, s->pol, sizeof(double) * np);
    }
    return MAVI_OK;
}

int32_t oracle_set_state(OracleSys* s, const double* pos, const double* vel, const double* pol) {
    if (pos) memcpy(s->pos, pos, sizeof(double) * 2 * s->n);
    if (vel && s->vel) memcpy(s->vel, vel, sizeof(double) * 2 * s->n);
    if (pol && s->pol) {
        int64_t np = (s->p.state_kind == MAVI_STATE_RINGS) ? s->num_rings : s->n;
        memcpy(s->pol, pol, sizeof(double) * np);
    }
    return MAVI_OK;
}

int32_t oracle_get_time(OracleSys* s, int64_t* num_steps, double* time) {
    *num_steps = s->num_steps; *time = s->time;
    return MAVI_OK;
}

/* A System constructed with a time_info (src/systems.jl:84-87). */
int32_t oracle_set_time(OracleSys* s, int64_t num_steps, double time) {
    s->num_steps = num_steps; s->time = time;
    return MAVI_OK;
}

int32_t oracle_get_areas(OracleSys* s, double* areas) {
    if (!s->areas) return MAVI_ERR_INVALID_ARG;
    memcpy(areas, s->areas, sizeof(double) * s->num_rings);
    return MAVI_OK;
}

/* sizeof of the shared ABI structs as this C compiler lays them out, so tests
 * can check the Python ctypes mirror byte for byte. */
int32_t oracle_struct_sizes(int64_t* out) {
    out[0] = (int64_t)sizeof(MaviSpace);
    out[1] = (int64_t)sizeof(MaviRingsCfg);
    out[2] = (int64_t)sizeof(MaviDynamicCfg);
    out[3] = (int64_t)sizeof(MaviReplicaParams);
    out[4] = (int64_t)sizeof(MaviOptions);
    out[5] = (int64_t)sizeof(MaviStats);
    out[6] = (int64_t)sizeof(MaviProfile);
    out[7] = (int64_t)sizeof(MaviSourceEntry);
    out[8] = (int64_t)sizeof(MaviSpawnBox);
    out[9] = (int64_t)sizeof(MaviInvasion);
    return 10;
}
