// hx_pass_f32.cu -- FP32-product instances of the pass kernels (the mixed method).
#define HX_T float
#define HX_SUF f32
#include "hx_pass_inst.cuh"
