// mavi_system.cuh — the handle (MaviSystem) and the launch sequences shared by
// the translation units of libmavi_cuda.so.
#pragma once

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "mavi_kernels.cuh"

namespace mavi {

constexpr int kBlock = 256;

struct ProfEvents {
    cudaEvent_t a[MAVI_NUM_KERNEL_KINDS][4];
    cudaEvent_t b[MAVI_NUM_KERNEL_KINDS][4];
    int used[MAVI_NUM_KERNEL_KINDS];
    cudaEvent_t step_a, step_b;
    int step_used;
};

}  // namespace mavi

// The opaque handle of the C ABI (include/mavi_cuda.h).
struct MaviSystem {
    using DevRep = mavi::DevRep;
    using Ctx = mavi::Ctx;
    using ProfEvents = mavi::ProfEvents;
    MaviOptions opt{};
    int32_t R = 0;
    std::vector<MaviReplicaParams> params;
    std::vector<DevRep> reps_h;
    std::vector<int64_t> rep_active;   // active particles per replica
    int32_t dyn = 0, step_kind = 0, state_kind = 0, prec = 0;
    bool has_vel = false, has_pol = false, is_rings = false;
    bool rings_small = false;   // mixed rings, every ring <= 32 particles, no minimum image: k_rings<mixed, true>
    int64_t M = 0, Nslots = 0, Ctot = 0, total_rings = 0, noise_count = 0, ntiles = 0;
    std::vector<int64_t> num_steps;
    std::vector<double> time;
    cudaStream_t stream = nullptr;
    Ctx C{};
    std::vector<void*> allocs;
    double2 *pos_user = nullptr, *vel_user = nullptr, *f_user = nullptr;
    double* pol_user = nullptr;
    double *ke_t = nullptr, *pe_t = nullptr, *ke_r = nullptr, *pe_r = nullptr;
    unsigned long long* d_pairs = nullptr;
    double* series = nullptr;          // energy series (mavi_energy_series), grown on demand
    int64_t series_cap = 0;            // doubles
    unsigned long long* hist = nullptr;    // pair-distance histogram bins (mavi_pair_distribution)
    // Newton's-third-law tiles of the mixed Lennard-Jones / WCA passes (static:
    // chunk grids do not change), the work-queue tickets and the persistent grid
    mavi::TileDesc* tiles = nullptr;
    int32_t ntiles_t = 0;
    int32_t* tile_queue = nullptr;
    unsigned tile_grid = 0;
    int32_t lanes = 1;             // lanes per particle of the mixed short-range passes (1, 2, 4)
    double* noise_cur = nullptr;
    double* noise_queue = nullptr;
    int64_t noise_queue_cap = 0, noise_queue_len = 0, noise_queue_pos = 0;
    bool counts_valid = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int32_t* tile_offs = nullptr;  // exclusive scan of the tile totals (grids of many tiles)
    bool profiling = false;
    int profile_mode = 0;          // 0 off, 1 per kernel kind + whole step, 2 whole step only
    int graph_profile_mode = 0;    // profile_mode the captured graph was recorded with
    int graph_ev_used[MAVI_NUM_KERNEL_KINDS] = {0};
    int graph_step_used = 0;
    ProfEvents ev{};
    MaviProfile prof{};
    int32_t max_chunk_count = 0;
    int64_t last_pairs = -1;
    std::string last_error;
    // chunks the scan covers: Ctot, plus the parking chunk of rings handles
    int64_t nscan = 0;
    int64_t noise_base = 0;        // noise numbers per step without the spawn uniforms
    // sources and sinks (rings): per replica, as passed to mavi_rings_sources
    bool var_rings = false;
    struct SrcCfg {
        std::vector<MaviSourceEntry> entries;
        std::vector<MaviSpawnBox> boxes;
        std::vector<double> spawn_xy;
        std::vector<int32_t> chunk_rc;
    };
    std::vector<SrcCfg> src_cfg;
    void* src_buf[4] = {nullptr, nullptr, nullptr, nullptr};   // entries, boxes, spawn, chunks
    // invasion detection (rings), per replica
    struct InvCfg {
        bool on = false;
        int64_t steps = 0, last_check = 0;
        int32_t cols = 0, rows = 0;          // ring chunks; 0 x 0: none
        int64_t chunk0 = 0;                  // first ring chunk in the shared arrays
        double blx = 0, bly = 0, len = 0, h = 0, cl = 0, ch = 0;
        std::vector<MaviInvasion> list;
    };
    std::vector<InvCfg> inv;
    struct InvBuffers {
        double2* cont = nullptr;             // continuous ring positions, user order
        double* bb = nullptr;                // per ring: xmin, xmax, ymin, ymax
        int32_t *chunk_of = nullptr, *rank = nullptr, *list = nullptr;   // per ring
        int32_t *count = nullptr, *start = nullptr, *nbr = nullptr;      // per ring chunk (nbr: 4 each)
        int32_t* num_ids = nullptr;          // per replica: rings in get_rings_ids
        void* reps = nullptr;                // the replicas of one check
        void* rec = nullptr;                 // records of one check
        int32_t* nrec = nullptr;
        int64_t rec_cap = 0, nch = 0;
    } invb;
};

namespace mavi {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
inline int fail(MaviSystem* s, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (s) s->last_error = buf;
    return code;
}

#define CUDA_TRY(sys, expr)                                                                  \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(sys, MAVI_ERR_CUDA, "%s failed: %s", #expr, cudaGetErrorString(_e)); \
    } while (0)

template <typename T>
inline cudaError_t dalloc(MaviSystem* s, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e == cudaSuccess) {
        s->allocs.push_back((void*)*p);
        cudaMemsetAsync(*p, 0, sizeof(T) * count, s->stream);
    }
    return e;
}

inline unsigned nblocks(int64_t n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

inline void record_begin(MaviSystem* s, int kind) {
    if (s->profile_mode != 1) return;
    int u = s->ev.used[kind];
    if (u < 4) cudaEventRecordWithFlags(s->ev.a[kind][u], s->stream, cudaEventRecordExternal);
}
inline void record_end(MaviSystem* s, int kind) {
    if (s->profile_mode != 1) return;
    int u = s->ev.used[kind];
    if (u < 4) {
        cudaEventRecordWithFlags(s->ev.b[kind][u], s->stream, cudaEventRecordExternal);
        s->ev.used[kind] = u + 1;
    }
}
// Adds the device time between each begin/end event pair of the last
// launch sequence (eager or graph replay) to the profile.
inline void collect_profile(MaviSystem* s, const int* used) {
    if (!s->profiling) return;
    cudaStreamSynchronize(s->stream);
    for (int k = 0; k < MAVI_NUM_KERNEL_KINDS; k++) {
        for (int u = 0; u < used[k]; u++) {
            float ms = 0;
            if (cudaEventElapsedTime(&ms, s->ev.a[k][u], s->ev.b[k][u]) == cudaSuccess) {
                s->prof.ms[k] += ms;
                s->prof.launches[k] += 1;
            } else {
                cudaGetLastError();   // a missing timing must not poison later error checks
            }
        }
        s->ev.used[k] = 0;
    }
}

// Whole-step device time: an event before the first and after the last launch.
inline void collect_step_time(MaviSystem* s, int used) {
    if (!s->profiling || !used) return;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, s->ev.step_a, s->ev.step_b) == cudaSuccess) {
        s->prof.step_ms += ms;
        s->prof.last_step_ms = ms;
    } else {
        cudaGetLastError();
    }
}


// Per-precision launch sequences (mavi_steps_fp64.cu / mavi_steps_mixed.cu).
void sort_permute_fp64(MaviSystem* s);
void count_fp64(MaviSystem* s, int use_guess, const double2* src);
void count_mixed(MaviSystem* s, int use_guess, const double2* src);
void sort_permute_mixed(MaviSystem* s);
void step_body_fp64(MaviSystem* s);
void step_body_mixed(MaviSystem* s);
void forces_only_fp64(MaviSystem* s, int with_walls);
void forces_only_mixed(MaviSystem* s, int with_walls);
void rings_terms_fp64(MaviSystem* s, int do_update, int with_walls);
void rings_terms_mixed(MaviSystem* s, int do_update, int with_walls);
void forces_to_user_fp64(MaviSystem* s);
void forces_to_user_mixed(MaviSystem* s);
void sources_fp64(MaviSystem* s);
void sources_mixed(MaviSystem* s);
// check_invasions! for the listed replicas (mavi_invasions.cu); waits for the
// device. from_sources: the step's k_sources left RingsInfo.cms.
int run_invasions(MaviSystem* s, const std::vector<int32_t>& due, bool from_sources);
// The mixed short-range passes with s->lanes lanes per particle (mavi_steps_lanes.cu).
void lanes_pass_mixed(MaviSystem* s, int dyn, int pass, int with_walls);
// The mixed Lennard-Jones passes with the split gather (mavi_steps_split.cu).
void split_pass_mixed(MaviSystem* s, int pass, int with_walls);
// The mixed short-range passes with the per-chunk or the column gather (mavi_steps_cols.cu).
void cols_pass_mixed(MaviSystem* s, int dyn, int pass, int with_walls);
// waits for the stream and turns a device error flag into a status (mavi_api.cu)
int device_error_status(MaviSystem* s);

}  // namespace mavi
