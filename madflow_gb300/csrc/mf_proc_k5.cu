// g g > t t~ g g g kernels (120 colour flows; the matrix-element workspace
// lives in global memory).
#include "mf_me.cuh"
#include "generated/ttng5.cuh"
#include "mf_proc.cuh"
MF_DEFINE_TC(5)
MF_DEFINE_PROCESS(5)
