// mavi_steps_cols.cu — the mixed-form short-range pair passes with the
// per-chunk or the column gather (k_pass_cols), in a translation unit of their
// own so that they compile in parallel with the other pass instantiations.
#include "mavi_system.cuh"

namespace mavi {
namespace {

template <int DYN, int PASS, bool COLS>
void launch(MaviSystem* s, int with_walls) {
    const unsigned g = nblocks(s->M, kPassThreads);
    if (s->has_vel) k_pass_cols<DYN, PASS, true, false, COLS><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else if (s->has_pol) k_pass_cols<DYN, PASS, false, true, COLS><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else k_pass_cols<DYN, PASS, false, false, COLS><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
}

template <int DYN, int PASS>
void launch_cols(MaviSystem* s, int with_walls) {
    if (s->C.gather_mode == 2) launch<DYN, PASS, true>(s, with_walls);
    else launch<DYN, PASS, false>(s, with_walls);
}

}  // namespace

void cols_pass_mixed(MaviSystem* s, int dyn, int pass, int with_walls) {
    if (dyn == MAVI_DYN_HARM_TRUNC) {
        if (pass == kPassForce) launch_cols<MAVI_DYN_HARM_TRUNC, kPassForce>(s, with_walls);
        else if (pass == kPassOverdamped) launch_cols<MAVI_DYN_HARM_TRUNC, kPassOverdamped>(s, with_walls);
        else if (pass == kPassVerlet1) launch_cols<MAVI_DYN_HARM_TRUNC, kPassVerlet1>(s, with_walls);
        else if (pass == kPassVerlet2) launch_cols<MAVI_DYN_HARM_TRUNC, kPassVerlet2>(s, with_walls);
    } else if (dyn == MAVI_DYN_SZABO) {
        if (pass == kPassForce) launch_cols<MAVI_DYN_SZABO, kPassForce>(s, with_walls);
        else if (pass == kPassSzabo) launch_cols<MAVI_DYN_SZABO, kPassSzabo>(s, with_walls);
    } else if (dyn == MAVI_DYN_RINGS && pass == kPassForce) {
        launch_cols<MAVI_DYN_RINGS, kPassForce>(s, with_walls);
    }
}

}  // namespace mavi
