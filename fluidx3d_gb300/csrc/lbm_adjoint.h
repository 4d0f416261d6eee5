// Adjoint launchers (lbm_adjoint.cu) used by the C-ABI driver.
#pragma once
#include "lbm_internal.h"

namespace fx3d {

enum : int { OBJ_KE_PLANE = 1, OBJ_DRAG_X = 2 };
struct AdjArgs {
	const void* state; // f^k, DDFs before step k, in the domain's storage format (objective terms)
	const float* moments; // rho[N] then u[3N] of f^k as step k collides with them (force-shifted, clamped
	                      // velocity; not written at TYPE_E cells, whose presets are a.rho/a.u): the adjoint step's input
	float* lambda;     // q*N adjoint DDFs (FP32), updated in place
	float* grad;       // 3N dJ/dF accumulator
	int obj_kind;
	uint32_t plane_x;
	uint32_t marker;
	float obj_weight;  // weight of the objective term at this time step (0 outside the window)
};
bool adjoint_supported(const Variant& v); // needs VOLUME_FORCE and FORCE_FIELD (F is the design variable)
cudaError_t launch_adjoint_step(const Variant& v, const StepArgs& a, const AdjArgs& j, bool obj_only, cudaStream_t s);
cudaError_t launch_objective_value(const Variant& v, const StepArgs& a, const AdjArgs& j, double* partials, double* J, cudaStream_t s);

} // namespace fx3d
