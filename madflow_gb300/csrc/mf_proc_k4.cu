// g g > t t~ g g kernels.
#include "mf_me.cuh"
#include "generated/ttng4.cuh"
#include "mf_proc.cuh"
MF_DEFINE_TC(4)
MF_DEFINE_PROCESS(4)
