// SUBGRID (Smagorinsky-Lilly) variants of stream_collide for FP16S storage, compiled apart from
// lbm_kernels_fp16s.cu so that the two halves build in parallel.
#include "lbm_kernels.cuh"
FX3D_DEFINE_SG_LAUNCHER(fx3d::ST_FP16S)
