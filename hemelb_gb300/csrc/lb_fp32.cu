// FP32-deviation and FP16-storage forms of the LB update (distributions stored as
// f - w_d, collide in FP32).
#include "lb_kernels.cuh"

HLBG_INSTANTIATE(1)
HLBG_INSTANTIATE(2)
