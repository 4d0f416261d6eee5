// SUBGRID variants of stream_collide, FP16C DDF storage
#include "lbm_kernels.cuh"

FX3D_DEFINE_X_LAUNCHER(fx3d::ST_FP16C, fx3d::EXT_SG)
