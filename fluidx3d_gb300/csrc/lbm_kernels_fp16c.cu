// Forward-step kernels instantiated for DDF storage FP16C (all velocity sets, collision operators
// and extension combinations). The kernel bodies live in lbm_kernels.cuh.
#include "lbm_kernels.cuh"
FX3D_DEFINE_LAUNCHERS(fp16c, fx3d::ST_FP16C)
