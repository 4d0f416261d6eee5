// MOVING_BOUNDARIES variants of stream_collide, FP32 DDF storage
#include "lbm_kernels.cuh"

FX3D_DEFINE_X_LAUNCHER(fx3d::ST_FP32, fx3d::EXT_MB)
