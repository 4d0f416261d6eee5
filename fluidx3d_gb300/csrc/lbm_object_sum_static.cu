// lbm_object_sum_static: the object reduction of lbm_object_center_of_mass / lbm_object_force /
// lbm_object_torque (k_object_sum + k_object_sum_final: FP64, fixed summation order) over device
// arrays the caller owns, without allocating anything. The block partials and the 4 result values
// live in one file-scope device array of fixed size, so no call reaches cudaMalloc/cudaFree or any
// allocating library routine.
//
// Limits and contract:
//   * at most LBM_OBJECT_SUM_STATIC_MAX_BLOCKS reduction blocks (scratch: (1216+1)*4 doubles =
//     38,944 bytes per device); a larger block count is rejected with LBM_ERR_INVALID_ARGUMENT;
//   * nothing in the scratch must start at zero: every block overwrites its own 4 partial slots and
//     the final block overwrites the 4 result slots, so no clearing is needed before a call;
//   * the scratch is one per device and shared by all calls on it: calls whose kernels overlap on
//     the GPU (issued on different streams, or from several host threads at once) race on it;
//   * the first call on a device resolves the scratch's device address with cudaGetSymbolAddress
//     (with that device current) and caches it; make that first call before any stream capture on
//     the device.
#include <cstdio>
#include <mutex>
#include "lbm_capi.h"
#include "lbm_internal.h"

static constexpr int kMaxBlocks = LBM_OBJECT_SUM_STATIC_MAX_BLOCKS;
// [0, 4*kMaxBlocks): block partials; [4*kMaxBlocks, 4*kMaxBlocks+4): the result
static __device__ __align__(256) double object_sum_scratch[(kMaxBlocks+1)*4];

namespace {

constexpr int kMaxDevices = 64;
std::mutex scratch_mutex;
double* scratch_address[kMaxDevices] = {};

// address of object_sum_scratch on `dev`, which must be the current device; resolved once per device
cudaError_t scratch_of(const int dev, double** p) {
	std::lock_guard<std::mutex> lock(scratch_mutex);
	if(!scratch_address[dev]) {
		void* a = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&a, object_sum_scratch);
		if(e!=cudaSuccess) return e;
		scratch_address[dev] = static_cast<double*>(a);
	}
	*p = scratch_address[dev];
	return cudaSuccess;
}

struct CurrentDevice { // makes `dev` current for the call and restores the caller's device
	int prev = -1;
	bool changed = false;
	cudaError_t err = cudaSuccess;
	explicit CurrentDevice(const int dev) {
		err = cudaGetDevice(&prev);
		if(err==cudaSuccess && prev!=dev) { err = cudaSetDevice(dev); changed = err==cudaSuccess; }
	}
	~CurrentDevice() { if(changed) cudaSetDevice(prev); }
};

} // namespace

extern "C" int lbm_object_sum_static(const int device, const uint32_t Nx, const uint32_t Ny, const uint32_t Nz, const uint8_t* flags, const float* F,
                                     const uint8_t marker, const int kind, const double cx, const double cy, const double cz, const uint32_t blocks,
                                     void* cuda_stream, double out[4]) {
	using namespace fx3d;
	char msg[256];
	if(!out) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: NULL output");
	if(!flags) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: NULL flags array");
	if(kind<0||kind>2) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: kind must be 0 (center of mass), 1 (force) or 2 (torque)");
	if(kind>0&&!F) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: force and torque need the F array");
	const uint64_t N = (uint64_t)Nx*Ny*Nz;
	if(N==0ull) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: grid point number is 0");
	if((uint64_t)Nx*Ny>0xFFFFFFFFull) return capi_fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_sum_static: Nx*Ny must fit in 32 bits");
	if(blocks>(uint32_t)kMaxBlocks) {
		std::snprintf(msg, sizeof(msg), "lbm_object_sum_static: blocks=%u exceeds the static scratch maximum of %d blocks", blocks, kMaxBlocks);
		return capi_fail(LBM_ERR_INVALID_ARGUMENT, msg);
	}
	int count = 0;
	const cudaError_t ec = cudaGetDeviceCount(&count);
	if(ec!=cudaSuccess||count==0) return capi_fail(LBM_ERR_NO_DEVICE, "lbm_object_sum_static: no CUDA device");
	if(device<0||device>=count||device>=kMaxDevices) {
		std::snprintf(msg, sizeof(msg), "lbm_object_sum_static: device %d out of range (%d devices)", device, count);
		return capi_fail(LBM_ERR_INVALID_ARGUMENT, msg);
	}
	CurrentDevice guard(device);
	if(guard.err!=cudaSuccess) return capi_cuda_fail(guard.err, "cudaSetDevice");
	double* scratch = nullptr;
	cudaError_t e = scratch_of(device, &scratch);
	if(e!=cudaSuccess) return capi_cuda_fail(e, "cudaGetSymbolAddress(object_sum_scratch)");
	GridDesc g;
	g.Nx = Nx; g.Ny = Ny; g.Nz = Nz; g.NxNy = Nx*Ny; g.N = N;
	g.nx_inv = Nx==1u ? 0ull : (~0ull)/Nx+1ull;
	const cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
	double* result = scratch+4*kMaxBlocks;
	e = launch_object_sum_blocks(g, kind>0 ? F : nullptr, flags, marker, kind, cx, cy, cz, blocks==0u ? REDUCE_BLOCKS : (int)blocks, scratch, result, s);
	if(e!=cudaSuccess) return capi_cuda_fail(e, "lbm_object_sum_static");
	double h[4];
	e = cudaMemcpyAsync(h, result, sizeof(h), cudaMemcpyDeviceToHost, s);
	if(e!=cudaSuccess) return capi_cuda_fail(e, "cudaMemcpyAsync(object_sum_static)");
	e = cudaStreamSynchronize(s);
	if(e!=cudaSuccess) return capi_cuda_fail(e, "cudaStreamSynchronize");
	if(kind==0) { // mean position and count, as lbm_object_center_of_mass
		for(int i=0; i<3; i++) out[i] = h[3]>0.0 ? h[i]/h[3] : 0.0;
		out[3] = h[3];
	} else {
		for(int i=0; i<3; i++) out[i] = h[i];
		out[3] = 0.0;
	}
	return LBM_OK;
}
