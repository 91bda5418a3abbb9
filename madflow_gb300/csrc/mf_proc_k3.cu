// g g > t t~ g kernels.
#include "mf_me.cuh"
#include "generated/ttng3.cuh"
#include "mf_proc.cuh"
MF_DEFINE_PROCESS(3)
