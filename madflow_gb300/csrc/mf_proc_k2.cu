// g g > t t~ kernels.
#include "mf_me.cuh"
#include "generated/ttng2.cuh"
#include "mf_proc.cuh"
MF_DEFINE_PROCESS(2)
