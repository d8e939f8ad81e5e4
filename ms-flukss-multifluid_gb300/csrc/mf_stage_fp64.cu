// mf_stage_fp64.cu - FP64 stage kernels and the precision-independent kernels.
// Built with -fmad=false: no multiply-add is fused, so every FP64 operation
// rounds exactly as in the CPU restatement of the reference.
#define MF_STAGE_COMMON 1
#include "mf_stage_impl.cuh"
