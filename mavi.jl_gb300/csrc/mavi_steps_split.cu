// mavi_steps_split.cu — the mixed-form Lennard-Jones pair passes with the
// split gather (k_pass_split), in a translation unit of their own so that
// they compile in parallel with the other pass instantiations.
#include "mavi_system.cuh"

namespace mavi {
namespace {

template <int PASS>
void launch_split(MaviSystem* s, int with_walls) {
    const unsigned g = nblocks(s->M, kPassThreads);
    if (s->has_vel) k_pass_split<PASS, true, false><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else if (s->has_pol) k_pass_split<PASS, false, true><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
    else k_pass_split<PASS, false, false><<<g, kPassThreads, 0, s->stream>>>(s->C, with_walls);
}

}  // namespace

void split_pass_mixed(MaviSystem* s, int pass, int with_walls) {
    if (pass == kPassForce) launch_split<kPassForce>(s, with_walls);
    else if (pass == kPassVerlet1) launch_split<kPassVerlet1>(s, with_walls);
    else if (pass == kPassVerlet2) launch_split<kPassVerlet2>(s, with_walls);
    else if (pass == kPassOverdamped) launch_split<kPassOverdamped>(s, with_walls);
}

}  // namespace mavi
