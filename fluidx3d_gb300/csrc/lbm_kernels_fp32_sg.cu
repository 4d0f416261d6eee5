// SUBGRID (Smagorinsky-Lilly) variants of stream_collide for FP32 storage, compiled apart from
// lbm_kernels_fp32.cu so that the two halves build in parallel.
#include "lbm_kernels.cuh"
FX3D_DEFINE_SG_LAUNCHER(fx3d::ST_FP32)
