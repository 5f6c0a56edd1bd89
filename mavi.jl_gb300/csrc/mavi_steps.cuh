// mavi_steps.cuh — per-precision launch sequences. Included once by
// mavi_steps_fp64.cu (PREC = FP64) and once by mavi_steps_mixed.cu
// (PREC = mixed) so the two sets of kernel instantiations compile in parallel.
#pragma once

#include "mavi_system.cuh"

namespace mavi {
namespace steps {

template <int PREC>
void sort_permute(MaviSystem* s) {
    unsigned g = nblocks(s->M);
    if (s->has_vel) k_permute<PREC, true, false><<<g, kBlock, 0, s->stream>>>(s->C);
    else if (s->has_pol) k_permute<PREC, false, true><<<g, kBlock, 0, s->stream>>>(s->C);
    else k_permute<PREC, false, false><<<g, kBlock, 0, s->stream>>>(s->C);
}

template <int PREC>
void count(MaviSystem* s, int use_guess, const double2* src) {
    k_count<PREC><<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, use_guess, src);
}

// Tiled Newton's-third-law pass (mixed Lennard-Jones / WCA): a CTA per tile,
// or a persistent grid pulling tiles from the device work queue.
template <int DYN, int PASS>
void tpass(MaviSystem* s, int with_walls) {
    const int32_t q = s->C.gather_mode == kGatherTilesQueue ? 1 : 0;
    const unsigned g = q ? s->tile_grid : (unsigned)s->ntiles_t;
    if (s->has_vel)
        k_tpass<DYN, PASS, true, false><<<g, kTileThreads, 0, s->stream>>>(s->C, with_walls, s->tiles, s->ntiles_t,
                                                                           s->tile_queue, q);
    else if (s->has_pol)
        k_tpass<DYN, PASS, false, true><<<g, kTileThreads, 0, s->stream>>>(s->C, with_walls, s->tiles, s->ntiles_t,
                                                                           s->tile_queue, q);
    else
        k_tpass<DYN, PASS, false, false><<<g, kTileThreads, 0, s->stream>>>(s->C, with_walls, s->tiles, s->ntiles_t,
                                                                            s->tile_queue, q);
}

template <int PREC, int DYN, int PASS>
void pass(MaviSystem* s, int with_walls) {
    if constexpr (PREC == kPrecMixed && kTiledPass<DYN, PASS>) {
        if (s->tiles && (s->C.gather_mode == kGatherTiles || s->C.gather_mode == kGatherTilesQueue)) {
            tpass<DYN, PASS>(s, with_walls);
            return;
        }
    }
    if constexpr (PREC == kPrecMixed && DYN == MAVI_DYN_LEN_JONES) {
        if (s->C.gather_mode == kGatherSplit) {
            split_pass_mixed(s, PASS, with_walls);
            return;
        }
    }
    if constexpr (PREC == kPrecMixed && kColsPass<DYN, PASS>) {
        if ((s->C.gather_mode == 1 || s->C.gather_mode == 2) && s->lanes == 1) {
            cols_pass_mixed(s, DYN, PASS, with_walls);
            return;
        }
    }
    if constexpr (PREC == kPrecMixed && kLanesPass<DYN, PASS>) {
        if (s->lanes > 1) {
            lanes_pass_mixed(s, DYN, PASS, with_walls);
            return;
        }
    }
    unsigned g = nblocks(s->M, kPassThreads);
    if (s->has_vel) k_pass<PREC, DYN, PASS, true, false><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else if (s->has_pol) k_pass<PREC, DYN, PASS, false, true><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else k_pass<PREC, DYN, PASS, false, false><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
}

// with_walls: calc_walls_forces! (the step always includes it)
template <int PREC>
void rings_terms(MaviSystem* s, int do_update, int with_walls) {
    unsigned g = (unsigned)((s->total_rings + kRingWarps - 1) / kRingWarps);
    // FP64 form: ring areas in the reference's operation order first
    if constexpr (PREC == kPrecFP64) k_ring_area_ref<<<nblocks(s->total_rings), kBlock, 0, s->stream>>>(s->C, s->total_rings);
    if constexpr (PREC == kPrecMixed) {
        if (s->rings_small) k_rings<PREC, true><<<g, 32 * kRingWarps, 0, s->stream>>>(s->C, s->total_rings, do_update, with_walls);
        else k_rings<PREC, false><<<g, 32 * kRingWarps, 0, s->stream>>>(s->C, s->total_rings, do_update, with_walls);
    } else {
        k_rings<PREC, false><<<g, 32 * kRingWarps, 0, s->stream>>>(s->C, s->total_rings, do_update, with_walls);
    }
    if (do_update) k_ring_pol<PREC><<<nblocks(s->total_rings), kBlock, 0, s->stream>>>(s->C, s->total_rings, 1);
}

// The passes of one step after the chunk rebuild.
template <int PREC, int DYN>
void step_body(MaviSystem* s) {
    switch (s->step_kind) {
    case MAVI_STEP_NEWTON:
        if constexpr (DYN != MAVI_DYN_RINGS) {
            record_begin(s, MAVI_KERNEL_FORCE);
            pass<PREC, DYN, kPassVerlet1>(s, 1);   // F(t) with wall forces, x(t+dt)
            pass<PREC, DYN, kPassVerlet2>(s, 0);   // F(t+dt) on stale chunks, v, walls!
            record_end(s, MAVI_KERNEL_FORCE);
        }
        break;
    case MAVI_STEP_OVERDAMPED:
        if constexpr (DYN != MAVI_DYN_RINGS) {
            record_begin(s, MAVI_KERNEL_FORCE);
            pass<PREC, DYN, kPassOverdamped>(s, 1);
            record_end(s, MAVI_KERNEL_FORCE);
        }
        break;
    case MAVI_STEP_SZABO:
        if constexpr (DYN == MAVI_DYN_SZABO) {
            record_begin(s, MAVI_KERNEL_FORCE);
            pass<PREC, DYN, kPassSzabo>(s, 1);
            record_end(s, MAVI_KERNEL_FORCE);
        }
        break;
    case MAVI_STEP_RTP:
        if constexpr (DYN == MAVI_DYN_RUN_TUMBLE) {
            record_begin(s, MAVI_KERNEL_FORCE);
            pass<PREC, DYN, kPassRTP>(s, 1);
            record_end(s, MAVI_KERNEL_FORCE);
        }
        break;
    case MAVI_STEP_RINGS:
        if constexpr (DYN == MAVI_DYN_RINGS) {
            record_begin(s, MAVI_KERNEL_FORCE);
            pass<PREC, DYN, kPassForce>(s, 0);
            record_end(s, MAVI_KERNEL_FORCE);
            record_begin(s, MAVI_KERNEL_UPDATE);
            rings_terms<PREC>(s, 1, 1);    // ring terms, wall forces, update, walls, binning, histogram
            record_end(s, MAVI_KERNEL_UPDATE);
        }
        break;
    }
}

template <int PREC>
void step_body_dispatch(MaviSystem* s) {
    switch (s->dyn) {
    case MAVI_DYN_HARM_TRUNC: step_body<PREC, MAVI_DYN_HARM_TRUNC>(s); break;
    case MAVI_DYN_LEN_JONES: step_body<PREC, MAVI_DYN_LEN_JONES>(s); break;
    case MAVI_DYN_SZABO: step_body<PREC, MAVI_DYN_SZABO>(s); break;
    case MAVI_DYN_RUN_TUMBLE: step_body<PREC, MAVI_DYN_RUN_TUMBLE>(s); break;
    case MAVI_DYN_RINGS: step_body<PREC, MAVI_DYN_RINGS>(s); break;
    }
}

// calc_forces! (+ calc_walls_forces!) on the current chunks; rings add their
// bonded terms in rings_terms(do_update = 0).
template <int PREC>
void forces_only(MaviSystem* s, int with_walls) {
    switch (s->dyn) {
    case MAVI_DYN_HARM_TRUNC: pass<PREC, MAVI_DYN_HARM_TRUNC, kPassForce>(s, with_walls); break;
    case MAVI_DYN_LEN_JONES: pass<PREC, MAVI_DYN_LEN_JONES, kPassForce>(s, with_walls); break;
    case MAVI_DYN_SZABO: pass<PREC, MAVI_DYN_SZABO, kPassForce>(s, with_walls); break;
    case MAVI_DYN_RUN_TUMBLE: pass<PREC, MAVI_DYN_RUN_TUMBLE, kPassForce>(s, with_walls); break;
    case MAVI_DYN_RINGS: pass<PREC, MAVI_DYN_RINGS, kPassForce>(s, 0); break;
    }
}

// Head of the rings step with sources and sinks: k_sources, then the
// histogram of the (changed) active set for the step's chunk update.
template <int PREC>
void sources(MaviSystem* s) {
    k_sources<PREC><<<(unsigned)s->R, kSrcThreads, 0, s->stream>>>(s->C);
    k_count<PREC><<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, 1, nullptr);
}

template <int PREC>
void forces_to_user(MaviSystem* s) {
    k_forces_to_user<PREC><<<nblocks(s->M), kBlock, 0, s->stream>>>(s->C, s->f_user);
}

}  // namespace steps
}  // namespace mavi

#define MAVI_DEFINE_STEPS(SUFFIX, PREC)                                                      \
    namespace mavi {                                                                         \
    void sort_permute_##SUFFIX(MaviSystem* s) { steps::sort_permute<PREC>(s); }              \
    void count_##SUFFIX(MaviSystem* s, int g, const double2* src) { steps::count<PREC>(s, g, src); } \
    void step_body_##SUFFIX(MaviSystem* s) { steps::step_body_dispatch<PREC>(s); }           \
    void forces_only_##SUFFIX(MaviSystem* s, int w) { steps::forces_only<PREC>(s, w); }      \
    void rings_terms_##SUFFIX(MaviSystem* s, int u, int w) { steps::rings_terms<PREC>(s, u, w); } \
    void forces_to_user_##SUFFIX(MaviSystem* s) { steps::forces_to_user<PREC>(s); }          \
    void sources_##SUFFIX(MaviSystem* s) { steps::sources<PREC>(s); }                        \
    }
