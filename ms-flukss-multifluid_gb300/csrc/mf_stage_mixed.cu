// mf_stage_mixed.cu - stage kernels with FP32 reconstruction and Riemann
// fluxes; state, flux accumulation, pressure recovery, positivity and charge
// exchange stay FP64.
#include "mf_stage_impl.cuh"
