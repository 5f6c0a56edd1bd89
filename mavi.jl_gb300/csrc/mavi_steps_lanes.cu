// mavi_steps_lanes.cu — the mixed-form short-range pair passes with two or
// four lanes per particle (k_pass_lanes), in a translation unit of their own
// so that they compile in parallel with the other pass instantiations.
#include "mavi_system.cuh"

namespace mavi {
namespace {

template <int DYN, int PASS, int LANES>
void launch_lanes(MaviSystem* s, int with_walls) {
    const unsigned g = nblocks(s->M * LANES, kPassThreads);
    if (s->has_vel) k_pass_lanes<DYN, PASS, true, false, LANES><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else if (s->has_pol) k_pass_lanes<DYN, PASS, false, true, LANES><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else k_pass_lanes<DYN, PASS, false, false, LANES><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
}

template <int DYN, int PASS>
void lanes(MaviSystem* s, int with_walls) {
    if (s->lanes == 4) launch_lanes<DYN, PASS, 4>(s, with_walls);
    else launch_lanes<DYN, PASS, 2>(s, with_walls);
}

}  // namespace

void lanes_pass_mixed(MaviSystem* s, int dyn, int pass, int with_walls) {
    if (dyn == MAVI_DYN_HARM_TRUNC && pass == kPassForce) lanes<MAVI_DYN_HARM_TRUNC, kPassForce>(s, with_walls);
    else if (dyn == MAVI_DYN_HARM_TRUNC && pass == kPassOverdamped) lanes<MAVI_DYN_HARM_TRUNC, kPassOverdamped>(s, with_walls);
    else if (dyn == MAVI_DYN_SZABO && pass == kPassForce) lanes<MAVI_DYN_SZABO, kPassForce>(s, with_walls);
    else if (dyn == MAVI_DYN_SZABO && pass == kPassSzabo) lanes<MAVI_DYN_SZABO, kPassSzabo>(s, with_walls);
}

}  // namespace mavi
