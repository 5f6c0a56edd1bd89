// FP64 instantiation of the per-precision launch sequences (the drop-in form).
#include "mavi_steps.cuh"
MAVI_DEFINE_STEPS(fp64, mavi::kPrecFP64)
