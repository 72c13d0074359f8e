// FP64 plain form of the LB update.  Built with --fmad=false: every addition and
// multiplication rounds separately, in the order the reference source writes them,
// so results are bit-identical to the reference's scalar (non-SSE) build.
#include "lb_kernels.cuh"

HLBG_INSTANTIATE(0)
