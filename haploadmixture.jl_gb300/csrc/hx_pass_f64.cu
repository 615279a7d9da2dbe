// hx_pass_f64.cu -- FP64 instances of the pass kernels (the plain method).
#define HX_T double
#define HX_SUF f64
#include "hx_pass_inst.cuh"
