// Host-side declarations shared by the C-ABI (lbm_capi.cu) and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fx3d {

enum : int { ST_FP32 = 0, ST_FP16S = 1, ST_FP16C = 2 }; // DDF storage formats
enum : int { EXT_VF = 1, EXT_FF = 2, EXT_EQ = 4, EXT_SG = 8, EXT_MB = 16 }; // VOLUME_FORCE, FORCE_FIELD, EQUILIBRIUM_BOUNDARIES, SUBGRID, MOVING_BOUNDARIES

struct GridDesc { // mirrors fx3d::Grid of lbm_scheme.cuh (kept layout-identical)
	uint32_t Nx, Ny, Nz, NxNy;
	uint64_t N;
	uint64_t nx_inv;
};

struct Variant {
	int q;        // 19 or 27
	bool trt;     // false: SRT
	int storage;  // ST_FP32 / ST_FP16S / ST_FP16C
	int ext;      // EXT_* bits, normalised: FF only together with VF
	bool fast;    // fast arithmetic (contracted, regrouped) instead of the reference's exact FP32 operation order
};

// arguments of one stream_collide / update_fields launch
struct StepArgs {
	GridDesc g;
	void* fi;     // DDFs read by the step
	void* fi_dst; // DDFs written by the step: fi (in place) or another array (one-cell and row-staged kernels)
	float* rho;
	float* u;
	const uint8_t* flags;
	const float* F;
	uint64_t t;
	float fx, fy, fz, w;
	int* err; // device error word (KERR_*), set by kernels whose bounded waits time out
	int fields_out; // UPDATE_FIELDS: stream_collide writes the rho/u each cell collides with (not at TYPE_E cells with EQUILIBRIUM_BOUNDARIES)
	float* rho_out; // where those fields go: rho and u (the domain's own, or per-step moment checkpoints of the adjoint)
	float* u_out;
	// collision rates derived from w on the host with the reference's FP32 operations
	// (src/kernel.cpp:1598, 1606-1609): 1-w, fma(w,-0.5,1), 0.5*w, 0.5*wm, fma(w,-0.25,0.5), fma(wm,-0.25,0.5)
	float omw, c_tau, hp, hm, c_taup, c_taum;
};

// relaxation-rate constants of one domain (computed once on the host)
struct Rates { float w, omw, c_tau, hp, hm, c_taup, c_taum; };
Rates make_rates(float w);

constexpr int BLOCK = 256;
constexpr int ROW_TPB_MAX = 512; // threads per CTA of the row-staged stream_collide

// stream_collide implementation: one thread per cell with direct global loads/stores ("cells"), or
// one CTA per x-row with the row's slots staged in shared memory by bulk copies ("rows")
enum : int { PATH_AUTO = 0, PATH_CELLS = 1, PATH_ROWS = 2, PATH_PAIRS = 3, PATH_PIPE = 4 };
// shared-memory plan of the row-staged kernel: bytes of one stage (one x-row's Q DDF rows + its flags)
// and the number of stages; stages==0 if the lattice does not fit its constraints
struct RowPlan { uint32_t stage_bytes, stages; size_t smem; };
RowPlan row_plan(int q, int storage, uint32_t Nx, uint32_t Ny, uint32_t Nz);
inline size_t rows_smem_bytes(const int q, const int storage, const uint32_t Nx, const uint32_t Ny=1u, const uint32_t Nz=1u) {
	return row_plan(q, storage, Nx, Ny, Nz).smem;
}
// persistent-grid size for a kernel: SMs x resident CTAs (cached per kernel, block size and smem)
int persistent_grid(const void* kernel, int threads, size_t smem);

// per-storage launchers (lbm_kernels_<storage>.cu)
#define FX3D_DECLARE_LAUNCHERS(sfx) \
	cudaError_t launch_initialize_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s); \
	cudaError_t launch_stream_collide_##sfx(const Variant& v, const StepArgs& a, int path, cudaStream_t s); \
	cudaError_t launch_update_fields_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s); \
	cudaError_t launch_update_force_field_##sfx(const Variant& v, const StepArgs& a, float* F, cudaStream_t s);
FX3D_DECLARE_LAUNCHERS(fp32)
FX3D_DECLARE_LAUNCHERS(fp16s)
FX3D_DECLARE_LAUNCHERS(fp16c)
#undef FX3D_DECLARE_LAUNCHERS

// storage-independent kernels (lbm_fields.cu)
// kind 0: center-of-mass sums (x,y,z,count), 1: force, 2: torque about c; FP64 partial sums per
// block into partials[blocks*4], then a fixed-order final sum into out[4] (deterministic)
constexpr int REDUCE_BLOCKS = 608; // 4 blocks per SM on 152 SMs
cudaError_t launch_object_sum(const GridDesc& g, const float* F, const uint8_t* flags, uint8_t marker, int kind,
                              double cx, double cy, double cz, double* partials, double* out, cudaStream_t s);
// the same with `blocks` reduction blocks (partials[blocks*4]); blocks == REDUCE_BLOCKS gives the same sums
cudaError_t launch_object_sum_blocks(const GridDesc& g, const float* F, const uint8_t* flags, uint8_t marker, int kind,
                                     double cx, double cy, double cz, int blocks, double* partials, double* out, cudaStream_t s);
// error reporting of the C-ABI (the message lbm_last_error returns), for entry points outside lbm_capi.cu
int capi_fail(int code, const char* message);
int capi_cuda_fail(cudaError_t e, const char* what);
cudaError_t launch_unvoxelize(const GridDesc& g, uint8_t* flags, uint8_t flag, const float* box, cudaStream_t s);
// VTK export packing: count cells from `first` of a dims-component FP32 SoA field, scaled, AoS, big-endian
cudaError_t launch_pack_vtk(const float* src, uint64_t N, uint32_t dims, uint64_t first, uint64_t count, float scale, uint32_t* dst, cudaStream_t s);
// TYPE_MS marking of the cells next to moving solids (src/kernel.cpp:1431-1450)
cudaError_t launch_update_moving_boundaries(int q, const GridDesc& g, const float* u, uint8_t* flags, cudaStream_t s);

// voxelization (lbm_voxelize.cu); bbu: 16 floats in the reference's layout (src/lbm.cpp:280-296)
cudaError_t launch_voxelize(const Variant& v, const GridDesc& g, uint32_t direction, void* fi, float* u, uint8_t* flags, uint64_t t, uint8_t flag,
                            const float* p0, const float* p1, const float* p2, const float* bbu, cudaStream_t s);

} // namespace fx3d
