// mavi_device.cuh — device-side definitions shared by the kernels of
// libmavi_cuda.so: the per-replica descriptor, Julia-exact chunk arithmetic,
// the pair force laws, wall handling and the counter-based RNG.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/mavi_cuda.h"

namespace mavi {

constexpr int kPrecFP64 = MAVI_PREC_FP64;
constexpr int kPrecMixed = MAVI_PREC_MIXED;

// Device error word: the first error code wins; `err_info` keeps the sorted
// slot that raised it. Kernels record and continue with clamped indices so
// that every access stays in bounds; the host reads the word after a step.
struct DevError {
    int32_t code;
    int32_t slot;
    int64_t aux;
};

__device__ __forceinline__ void raise_error(DevError* e, int32_t code, int64_t slot, int64_t aux) {
    if (atomicCAS(&e->code, 0, code) == 0) {
        e->slot = (int32_t)slot;
        e->aux = aux;
    }
}

// A source or sink of the rings model (MaviSourceEntry plus the index of its
// first spawn box in the handle's box array).
struct SrcEntryD {
    int32_t kind, num_boxes, pol_mode, geometry;
    int32_t box0, _pad;
    double pol, pad;
    double length, height, bl_x, bl_y;
    double radius, cx, cy;
};

// A spawn box: Source.bbox[i], its chunk list (global chunk indices
// [chunk0, chunk0 + num_chunks) of the handle's list; num_chunks < 0: every
// chunk of the replica), its nmax spawn points and, for a random
// polarisation, its place in the step's noise (-1: fixed polarisation).
struct SrcBoxD {
    double bl_x, bl_y, length, height;
    int32_t num_chunks, chunk0;
    int64_t spawn0;
    int64_t noise_idx;
};

// Per-replica descriptor, built on the host from MaviReplicaParams.
struct DevRep {
    int64_t a0, na;        // range of this replica's particles in sorted order
    int64_t slot0, nslots; // range of this replica's user slots
    int64_t c0;            // first global chunk of this replica
    int64_t ring0;         // first global ring of this replica
    int64_t noise0;        // first noise number of this replica in a step
    int32_t rows, cols, cap, periodic; // chunk grid; periodic stencil
    int32_t has_chunks;
    int32_t num_rings, nmax;
    // mixed-form circle wall force (the pre-checked PotentialWalls circle):
    // radius^2 in units^2 (128-bit) and in units, HarmTrunc constants
    long long wall_R2_hi;
    unsigned long long wall_R2_lo;
    float wall_Ru_f, wall_krep_f, wall_katr_f, wall_deq_f, wall_dmax_f, _wall_pad;
    // sources and sinks of the rings model: entries [src_e0, src_e0 + src_ne)
    // inv_cms: the step's k_sources keeps RingsInfo.cms for invasion detection
    int32_t src_e0, src_ne, src_has_sink, inv_cms;
    int32_t min_image;     // first space is PeriodicWalls on a RectangleCfg
    int32_t num_spaces;
    int32_t has_wall_forces;
    int32_t has_walls;     // any space that acts in walls!
    int32_t _pad;
    double chunk_l, chunk_h, bb_blx, bb_bly, bb_h, bb_len;
    double box_x, box_y;
    float chunk_lf, chunk_hf, box_xf, box_yf;
    float half_box_xf, half_box_yf;
    double half_box_x, half_box_y;
    double radius;         // particle_radius (walls)
    double dt;
    double pd[8];          // pair-law parameters (double)
    float pf[8];           // same in float
    double mobility, vo, relax_time, rot_diff, tumble_rate;
    // mixed form: fixed-point unit u = max(chunk_l, chunk_h) / 2^28
    double inv_u;          // 1/u
    float u_f, u2_f;       // u, u^2
    long long sx_u, sy_u;  // chunk width / height in units
    long long bx_u, by_u;  // box in units (cols*sx_u, rows*sy_u)
    long long half_bx_u, half_by_u;
    int32_t sx_i, sy_i;    // chunk width / height in units (int32 copies, < 2^29)
    int32_t bx_i, by_i;    // box in units when it fits int32 (minimum image on small grids)
    int32_t half_bx_i, half_by_i;
    int32_t half_sx_i, half_sy_i;  // half chunk in units
    double cx0, cy0;       // centre of chunk (row 0, col 0)
    int64_t ccol0, crow0;  // first entry of this replica in the chunk-centre tables
    double mdt;            // mobility * dt
    float mdt_f;
    int32_t mi_small;      // grid too small to skip the minimum image for unwrapped neighbours
    int32_t walls_edge_only; // every wall acts on the bounding rectangle only
    // mixed-form Lennard-Jones / WCA in double-float: d^2 (units^2) scaled by
    // lj_sk = 2^-k to O(1); (ah + al) = 48 eps sigma^12 u g^-7 and
    // (bh + bl) = 24 eps sigma^6 u g^-4 with g = 2^k u^2
    float lj_sk, lj_ah, lj_al, lj_bh, lj_bl;
    float lj_near2;        // split gather: pairs closer than 2 sigma (units^2) take the double-float term
    // rings, per type: target area A0^2 = (n l / p0)^2 and float copies of the
    // ring-internal constants (mixed form)
    double ring_a0sq[MAVI_MAX_TYPES];
    float ring_ks_f[MAVI_MAX_TYPES], ring_ls_f[MAVI_MAX_TYPES], ring_kb_f[MAVI_MAX_TYPES];
    float ring_vo_f[MAVI_MAX_TYPES], ring_mu_f[MAVI_MAX_TYPES];
    // mixed-form polarisation update: dt / relax_time (FP32) and sqrt(2 D dt)
    float ring_dt_tau_f[MAVI_MAX_TYPES];
    double ring_noise_amp[MAVI_MAX_TYPES];
    float dt_f;
    int32_t _pad3;
    double u2_d;           // u^2 in double (areas from integer units^2)
    // mixed-form rings: 2 A0 / u^2 per type as a 128-bit integer (hi, lo words),
    // k_area * u^2 / 2 in float, and the PotentialWalls circle pre-check in
    // units from the centre of chunk (0, 0): no force where r^2 < wall_lo2
    // (inside mode) or outside [wall_lo2, wall_hi2] (repulsion)
    long long ring_a0x2_hi[MAVI_MAX_TYPES];
    unsigned long long ring_a0x2_lo[MAVI_MAX_TYPES];
    float ring_karea_f[MAVI_MAX_TYPES];
    // springs without cancellation: l^2 / u^2 rounded to an integer (-1 when it
    // does not fit int64; the spring then falls back to FP32 L - l) and l^2
    long long ring_ls2_u[MAVI_MAX_TYPES];
    double ring_ls2_d[MAVI_MAX_TYPES];
    // mixed-form springs in float-float: k_spring * u and l / u as (high, low) pairs
    float ring_ku_h[MAVI_MAX_TYPES], ring_ku_l[MAVI_MAX_TYPES];
    float ring_lu_h[MAVI_MAX_TYPES], ring_lu_l[MAVI_MAX_TYPES];
    int32_t wall_precheck;          // 0 none, 1 inside mode, 2 repulsion
    long long wall_cx_u, wall_cy_u;
    float wall_lo2_u, wall_hi2_u;
};

// ---------------------------------------------------------------------------
// Julia-exact chunk index (src/chunks.jl:120-147). Julia's float div(x, y)
// rounds-to-nearest the exact quotient (x - rem(x, y)) / y, rem == fmod.
// Explicit _rn intrinsics keep the compiler from contracting anything.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double julia_div(double x, double y) {
    double r = fmod(x, y);
    return rint(__ddiv_rn(__dsub_rn(x, r), y));
}

// Returns the 0-based (row, col) before bounds checks, following
// `row = trunc(Int, div(-y + bl_y + H, chunk_h)) + 1` and the one-chunk clamp
// of index n+1. `ok` is false for a non-finite quotient.
__device__ __forceinline__ void chunk_row_col(const DevRep& R, double x, double y,
                                              int64_t& row, int64_t& col, bool& finite) {
    double qr = julia_div(__dadd_rn(__dadd_rn(-y, R.bb_bly), R.bb_h), R.chunk_h);
    double qc = julia_div(__dsub_rn(x, R.bb_blx), R.chunk_l);
    finite = isfinite(qr) && isfinite(qc) && fabs(qr) < 4e18 && fabs(qc) < 4e18;
    int64_t r = finite ? (int64_t)qr + 1 : 1;
    int64_t c = finite ? (int64_t)qc + 1 : 1;
    r -= (r == (int64_t)R.rows + 1) ? 1 : 0;
    c -= (c == (int64_t)R.cols + 1) ? 1 : 0;
    row = r - 1;
    col = c - 1;
}

// Centre of chunk (row, col): the FP32 offsets of the mixed form are taken
// relative to it, so |offset| stays within half a chunk.
__device__ __forceinline__ double chunk_cx(const DevRep& R, int64_t col) {
    return R.bb_blx + ((double)col + 0.5) * R.chunk_l;
}
__device__ __forceinline__ double chunk_cy(const DevRep& R, int64_t row) {
    return R.bb_bly + R.bb_h - ((double)row + 0.5) * R.chunk_h;
}

// ---------------------------------------------------------------------------
// Minimum image (src/integration.jl:43-48):
//   dr - (abs.(dr) .> size/2) .* copysign.(size, dr)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double min_image1(double d, double box, double half) {
    return fabs(d) > half ? d - copysign(box, d) : d;
}
__device__ __forceinline__ float min_image1f(float d, float box, float half) {
    return fabsf(d) > half ? d - copysignf(box, d) : d;
}

// ---------------------------------------------------------------------------
// Pair laws: force on i from j as a scalar s with f = s * dr.
// ---------------------------------------------------------------------------
// Parameter packing (DevRep::pd / pf), set by the host:
//  HarmTrunc: {k_rep, k_atr, 1/dist_eq, dist_eq^2, dist_max^2}
//     fmod/dist = -k (dist/dist_eq - 1)/dist = k (1/dist - 1/dist_eq)
//  LenJones:  {48 eps sigma^12, 24 eps sigma^6}
//     fmod/dist = 4 eps (12 sigma^12/d^14 - 6 sigma^6/d^8) = ir8 (A ir6 - B)
//  Szabo:     {k_rep/(r_max-r_eq), k_adh/r_eq, r_eq, r_max, r_max^2}
//     f = -f_mod (dist - r_eq) dr
//  RunTumble: {48 eps sigma^12, 24 eps sigma^6, cutoff^2}

template <typename T> __device__ __forceinline__ T rcp_(T x);
template <> __device__ __forceinline__ double rcp_<double>(double x) { return 1.0 / x; }
template <> __device__ __forceinline__ float rcp_<float>(float x) { return __frcp_rn(x); }
template <typename T> __device__ __forceinline__ T rsqrt_(T x);
template <> __device__ __forceinline__ double rsqrt_<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float rsqrt_<float>(float x) { return rsqrtf(x); }
template <typename T> __device__ __forceinline__ T sqrt_(T x);
template <> __device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float sqrt_<float>(float x) { return sqrtf(x); }

template <int DYN, typename T>
__device__ __forceinline__ T pair_scalar(const T* prm, T d2) {
    if constexpr (DYN == MAVI_DYN_LEN_JONES) {
        T ir2 = rcp_<T>(d2);
        T ir6 = ir2 * ir2 * ir2;
        return ir6 * ir2 * (prm[0] * ir6 - prm[1]);
    } else if constexpr (DYN == MAVI_DYN_HARM_TRUNC) {
        if (d2 > prm[4]) return T(0);
        T k = d2 < prm[3] ? prm[0] : prm[1];
        return k * (rsqrt_<T>(d2) - prm[2]);
    } else if constexpr (DYN == MAVI_DYN_SZABO) {
        if (d2 > prm[4]) return T(0);
        T dist = sqrt_<T>(d2);
        T f_mod = dist > prm[2] ? prm[1] : prm[0];
        return -f_mod * (dist - prm[2]);
    } else if constexpr (DYN == MAVI_DYN_RUN_TUMBLE) {
        if (d2 > prm[2]) return T(0);
        T ir2 = rcp_<T>(d2);
        T ir6 = ir2 * ir2 * ir2;
        return ir6 * ir2 * (prm[0] * ir6 - prm[1]);
    } else {
        return T(0);
    }
}

// Pair energy consistent with the force law:
// LenJones 4 eps[(s/d)^12-(s/d)^6] (src/quantities.jl:46-66); HarmTrunc
// k/(2 dist_eq) (d - dist_eq)^2 below dist_max; RunTumble unshifted WCA.
__device__ __forceinline__ double pair_energy(int dyn, const double* e, double d2) {
    if (dyn == MAVI_DYN_LEN_JONES) {
        double ir2 = 1.0 / d2;
        double ir6 = ir2 * ir2 * ir2;
        return e[0] * (e[1] * ir6 * ir6 - e[2] * ir6);
    } else if (dyn == MAVI_DYN_HARM_TRUNC) {
        if (d2 > e[3] * e[3]) return 0.0;
        double d = sqrt(d2);
        double k = d < e[2] ? e[0] : e[1];
        double x = d - e[2];
        return k / (2 * e[2]) * x * x;
    } else if (dyn == MAVI_DYN_RUN_TUMBLE) {
        if (d2 > e[3]) return 0.0;
        double ir2 = 1.0 / d2;
        double ir6 = ir2 * ir2 * ir2;
        return e[0] * (e[1] * ir6 * ir6 - e[2] * ir6);
    }
    return 0.0;
}

// ---------------------------------------------------------------------------
// Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC 2011), counter = (a, b, c, d),
// key = 64-bit seed. Uniforms in (0, 1], normals by Box-Muller.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        U4 n;
        n.x = hi1 ^ ctr.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ ctr.w ^ k1;
        n.w = lo0;
        ctr = n;
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

__device__ __forceinline__ double u32_to_unit(uint32_t a, uint32_t b) {
    // 53-bit uniform in (0, 1]
    uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    m &= ((1ull << 53) - 1);
    return ((double)m + 1.0) * (1.0 / 9007199254740992.0);
}

struct Rand2 { double a, b; };

// Two uniforms and a standard normal for (stream id, step).
__device__ __forceinline__ Rand2 philox_uniform2(uint64_t seed, uint64_t id, uint64_t step) {
    U4 c{(uint32_t)id, (uint32_t)(id >> 32), (uint32_t)step, (uint32_t)(step >> 32)};
    U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return Rand2{u32_to_unit(r.x, r.y), u32_to_unit(r.z, r.w)};
}

__device__ __forceinline__ double philox_normal(uint64_t seed, uint64_t id, uint64_t step) {
    Rand2 u = philox_uniform2(seed, id, step);
    return sqrt(-2.0 * log(u.a)) * cospi(2.0 * u.b);
}

// The same Philox counters with the Box-Muller transform in FP32 (24-bit
// uniforms in (0, 1]): the mixed form's noise, a standard normal to FP32
// precision without the FP64 logarithm and cosine.
__device__ __forceinline__ float philox_normal_f(uint64_t seed, uint64_t id, uint64_t step) {
    U4 c{(uint32_t)id, (uint32_t)(id >> 32), (uint32_t)step, (uint32_t)(step >> 32)};
    U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float a = ((float)(r.x >> 8) + 1.0f) * (1.0f / 16777216.0f);
    const float b = ((float)(r.z >> 8) + 1.0f) * (1.0f / 16777216.0f);
    return sqrtf(-2.0f * logf(a)) * cospif(2.0f * b);
}

// float -> double on the integer pipes (the conversion instruction runs on
// the FP64 pipe, the scarce one on this GPU). Exact for normal floats; zero
// and subnormal floats give a signed zero, infinities and NaN stay so.
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xffu;
    const uint32_t sign = b & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    const uint32_t de = (e == 0xffu) ? 0x7ffu : e + 896u;   // rebias 127 -> 1023
    const uint32_t hi = sign | (de << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}


// ---------------------------------------------------------------------------
// Float-float ("double-word") arithmetic on the FP32 pipe: a value is h + l
// with |l| <= ulp(h) / 2, about 44 bits of precision. The error-free
// transformations are Knuth's TwoSum, Dekker's FastTwoSum and the FMA-based
// TwoProd; add, multiply, divide and square root follow the classical
// double-word algorithms (Dekker 1971; Joldes, Muller, Popescu 2017). The _rn
// intrinsics keep the compiler from fusing or reordering the operations whose
// rounding errors are captured.
// ---------------------------------------------------------------------------
struct FF { float h, l; };

__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const FF s = ff_two_sum(a.h, b.h);
    return ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.h, -a.l}; }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q = __fdiv_rn(a.h, b.h);
    const float ph = __fmul_rn(q, b.h), pl = fmaf(q, b.h, -ph);    // q * b.h exactly
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.h, ph), pl), fmaf(-q, b.l, a.l));
    return ff_fast_two_sum(q, __fdiv_rn(r, b.h));
}
__device__ __forceinline__ FF ff_sqrt(FF a) {
    const float s = __fsqrt_rn(a.h);
    const float ph = __fmul_rn(s, s), pl = fmaf(s, s, -ph);        // s^2 exactly
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.h, ph), pl), a.l);
    return ff_fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.0f, s)));
}
// An int64 as float-float: three 24-bit limbs, each exact in FP32.
__device__ __forceinline__ FF ff_from_i64(long long v) {
    const float c0 = (float)(int32_t)(v & 0xffffff);
    const float c1 = (float)(int32_t)((v >> 24) & 0xffffff) * 16777216.0f;     // 2^24
    const float c2 = (float)(int32_t)(v >> 48) * 281474976710656.0f;          // 2^48
    const FF t = ff_fast_two_sum(c2, c1);
    const FF u = ff_two_sum(t.h, c0);
    return ff_fast_two_sum(u.h, __fadd_rn(u.l, t.l));
}

}  // namespace mavi
