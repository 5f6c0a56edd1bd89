// Mixed-precision instantiation of the per-precision launch sequences.
#include "mavi_steps.cuh"
MAVI_DEFINE_STEPS(mixed, mavi::kPrecMixed)
