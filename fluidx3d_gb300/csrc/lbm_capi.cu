// C-ABI implementation (include/lbm_capi.h): owns the device buffers of one LBM domain, keeps the
// time step and the lazy-update bookkeeping of the reference's LBM_Domain (src/lbm.cpp:96-332), and
// launches the sm_103a kernels. No entry point exits the process or throws across the ABI.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <new>
#include <filesystem>
#include <system_error>
#include "lbm_capi.h"
#include "lbm_internal.h"
#include "lbm_adjoint.h"

using namespace fx3d;

namespace {

thread_local std::string g_last_error;

int fail(const int code, const char* fmt, ...) {
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_last_error = buf;
	return code;
}
int cuda_fail(const cudaError_t e, const char* what) {
	return fail(e==cudaErrorMemoryAllocation ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}
#define FX3D_CUDA(call, what) do { const cudaError_t e_ = (call); if(e_!=cudaSuccess) return cuda_fail(e_, what); } while(0)

// storage bytes of one DDF
size_t ddf_bytes(const uint32_t storage) { return storage==LBM_FP32 ? 4u : 2u; }

__global__ void k_fill_f32(float* p, const uint64_t n, const float v) {
	for(uint64_t i=(uint64_t)blockIdx.x*blockDim.x+threadIdx.x; i<n; i+=(uint64_t)gridDim.x*blockDim.x) p[i] = v;
}

} // namespace

struct lbm_domain {
	lbm_config cfg;
	Variant v;
	GridDesc g;
	float w;
	Rates rates;
	int device;
	cudaStream_t own_stream = nullptr, stream = nullptr;
	void* fi = nullptr;
	float* rho = nullptr;
	float* u = nullptr;
	uint8_t* flags = nullptr;
	float* F = nullptr;
	double* partials = nullptr; // REDUCE_BLOCKS*4 doubles of reduction scratch
	double* sum_dev = nullptr;  // 4 doubles
	double* sum_host = nullptr; // pinned, 4 doubles
	int* err = nullptr;         // device error word written by kernels with bounded waits
	int path = PATH_AUTO;       // stream_collide implementation
	uint64_t t = 0ull;
	uint64_t t_last_update_fields = UINT64_MAX;
	uint64_t t_last_force_field = UINT64_MAX;
	bool initialized = false;
	bool fused_fields = false; // LBM_EXT_UPDATE_FIELDS: every stream_collide writes rho/u

	StepArgs args() const {
		StepArgs a;
		a.g = g; a.fi = fi; a.fi_dst = fi; a.rho = rho; a.u = u; a.flags = flags; a.F = F;
		a.t = t; a.fx = cfg.fx; a.fy = cfg.fy; a.fz = cfg.fz; a.w = w;
		a.err = err;
		a.fields_out = fused_fields ? 1 : 0;
		a.rho_out = rho; a.u_out = u;
		a.omw = rates.omw; a.c_tau = rates.c_tau; a.hp = rates.hp; a.hm = rates.hm; a.c_taup = rates.c_taup; a.c_taum = rates.c_taum;
		return a;
	}
	size_t field_bytes(const int field) const {
		switch(field) {
			case LBM_FIELD_RHO: return g.N*4u;
			case LBM_FIELD_U: return g.N*12u;
			case LBM_FIELD_FLAGS: return g.N;
			case LBM_FIELD_F: return g.N*12u;
			case LBM_FIELD_FI: return g.N*(size_t)cfg.velocity_set*ddf_bytes(cfg.storage);
			default: return 0u;
		}
	}
	void* field_ptr(const int field) const {
		switch(field) {
			case LBM_FIELD_RHO: return rho;
			case LBM_FIELD_U: return u;
			case LBM_FIELD_FLAGS: return flags;
			case LBM_FIELD_F: return F;
			case LBM_FIELD_FI: return fi;
			default: return nullptr;
		}
	}
};

namespace {

// make the domain's device current for this call (the caller's current device is restored)
struct DeviceGuard {
	int prev = -1;
	bool changed = false;
	cudaError_t err = cudaSuccess;
	explicit DeviceGuard(const int dev) {
		err = cudaGetDevice(&prev);
		if(err==cudaSuccess && prev!=dev) { err = cudaSetDevice(dev); changed = err==cudaSuccess; }
	}
	~DeviceGuard() { if(changed) cudaSetDevice(prev); }
};
#define FX3D_DOMAIN(d) \
	if(!(d)) return fail(LBM_ERR_INVALID_ARGUMENT, "%s: domain is NULL", __func__); \
	DeviceGuard guard_((d)->device); \
	if(guard_.err!=cudaSuccess) return cuda_fail(guard_.err, "cudaSetDevice");

// after a synchronisation: report (and clear) an error a kernel recorded in the error word
int check_kernel_error(lbm_domain* d) {
	int h = 0;
	FX3D_CUDA(cudaMemcpyAsync(&h, d->err, sizeof(int), cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(error word)");
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	if(h==0) return LBM_OK;
	FX3D_CUDA(cudaMemsetAsync(d->err, 0, sizeof(int), d->stream), "cudaMemsetAsync(error word)");
	return fail(LBM_ERR_CUDA, "a kernel gave up waiting for its bulk copies (device error code %d); the affected rows were left unchanged", h);
}

int launch_stream_collide(lbm_domain* d) {
	const StepArgs a = d->args();
	cudaError_t e;
	switch(d->v.storage) {
		case ST_FP32: e = launch_stream_collide_fp32(d->v, a, d->path, d->stream); break;
		case ST_FP16S: e = launch_stream_collide_fp16s(d->v, a, d->path, d->stream); break;
		default: e = launch_stream_collide_fp16c(d->v, a, d->path, d->stream); break;
	}
	return e==cudaSuccess ? LBM_OK : cuda_fail(e, "stream_collide");
}

int ensure_F(lbm_domain* d) {
	if(d->F) return LBM_OK;
	FX3D_CUDA(cudaMalloc(&d->F, d->g.N*12u), "cudaMalloc(F)");
	FX3D_CUDA(cudaMemsetAsync(d->F, 0, d->g.N*12u, d->stream), "cudaMemsetAsync(F)");
	return LBM_OK;
}

int do_update_fields(lbm_domain* d) {
	if(d->fused_fields) return LBM_OK; // the steps keep rho/u current (src/lbm.cpp:184-191 compiles to nothing with UPDATE_FIELDS)
	if(d->t==d->t_last_update_fields) return LBM_OK;
	const StepArgs a = d->args();
	cudaError_t e;
	switch(d->v.storage) {
		case ST_FP32: e = launch_update_fields_fp32(d->v, a, d->stream); break;
		case ST_FP16S: e = launch_update_fields_fp16s(d->v, a, d->stream); break;
		default: e = launch_update_fields_fp16c(d->v, a, d->stream); break;
	}
	if(e!=cudaSuccess) return cuda_fail(e, "update_fields");
	d->t_last_update_fields = d->t;
	return LBM_OK;
}

int do_update_force_field(lbm_domain* d) {
	const int r = ensure_F(d);
	if(r!=LBM_OK) return r;
	if(d->t==d->t_last_force_field) return LBM_OK;
	const StepArgs a = d->args();
	cudaError_t e;
	switch(d->v.storage) {
		case ST_FP32: e = launch_update_force_field_fp32(d->v, a, d->F, d->stream); break;
		case ST_FP16S: e = launch_update_force_field_fp16s(d->v, a, d->F, d->stream); break;
		default: e = launch_update_force_field_fp16c(d->v, a, d->F, d->stream); break;
	}
	if(e!=cudaSuccess) return cuda_fail(e, "update_force_field");
	d->t_last_force_field = d->t;
	return LBM_OK;
}

int object_sum(lbm_domain* d, const int kind, const uint8_t marker, const double cx, const double cy, const double cz, double* out, const int nout) {
	if(kind>0) {
		const int r = do_update_force_field(d);
		if(r!=LBM_OK) return r;
	}
	const float* F = kind>0 ? d->F : nullptr;
	FX3D_CUDA(launch_object_sum(d->g, F, d->flags, marker, kind, cx, cy, cz, d->partials, d->sum_dev, d->stream), "object_sum");
	FX3D_CUDA(cudaMemcpyAsync(d->sum_host, d->sum_dev, 4u*sizeof(double), cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(object_sum)");
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	for(int i=0; i<nout; i++) out[i] = d->sum_host[i];
	return LBM_OK;
}

void release(lbm_domain* d) {
	if(d->fi) cudaFree(d->fi);
	if(d->rho) cudaFree(d->rho);
	if(d->u) cudaFree(d->u);
	if(d->flags) cudaFree(d->flags);
	if(d->F) cudaFree(d->F);
	if(d->partials) cudaFree(d->partials);
	if(d->sum_dev) cudaFree(d->sum_dev);
	if(d->sum_host) cudaFreeHost(d->sum_host);
	if(d->err) cudaFree(d->err);
	if(d->own_stream) cudaStreamDestroy(d->own_stream);
}

} // namespace

namespace fx3d {
// the reference computes these per cell in the kernel (src/kernel.cpp:1598, 1606-1609); the same FP32
// operations on the host (compiled without contraction) give the same values once per domain
Rates make_rates(const float w) {
	Rates r;
	r.w = w;
	r.omw = 1.0f-w;
	r.c_tau = std::fmaf(w, -0.5f, 1.0f);
	const float wm = 1.0f/(0.1875f/(1.0f/w-0.5f)+0.5f);
	r.hp = 0.5f*w;
	r.hm = 0.5f*wm;
	r.c_taup = std::fmaf(w, -0.25f, 0.5f);
	r.c_taum = std::fmaf(wm, -0.25f, 0.5f);
	return r;
}
int capi_fail(const int code, const char* message) { return fail(code, "%s", message); }
int capi_cuda_fail(const cudaError_t e, const char* what) { return cuda_fail(e, what); }
} // namespace fx3d

extern "C" {

const char* lbm_last_error(void) { return g_last_error.c_str(); }

int lbm_host_alloc(const size_t bytes, void** host_ptr) {
	if(!host_ptr) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_host_alloc: NULL output");
	*host_ptr = nullptr;
	if(bytes==0u) return LBM_OK;
	FX3D_CUDA(cudaHostAlloc(host_ptr, bytes, cudaHostAllocPortable), "cudaHostAlloc");
	return LBM_OK;
}
int lbm_host_free(void* host_ptr) {
	if(host_ptr) FX3D_CUDA(cudaFreeHost(host_ptr), "cudaFreeHost");
	return LBM_OK;
}

float lbm_relaxation_rate(const float nu) {
	const float tau = 3.0f*nu+0.5f; // LBM::get_tau (src/lbm.hpp:462)
	char buf[64];
	std::snprintf(buf, sizeof(buf), "%f", (double)(1.0f/tau)); // std::to_string(float) of src/lbm.cpp:374
	return std::strtof(buf, nullptr);
}

uint32_t lbm_bytes_per_cell_device(const lbm_config* c) {
	if(!c) return 0u;
	uint32_t b = c->velocity_set*(uint32_t)ddf_bytes(c->storage)+17u;
	if(c->extensions&LBM_EXT_FORCE_FIELD) b += 12u;
	return b;
}
uint32_t lbm_bandwidth_bytes_per_cell(const lbm_config* c) {
	if(!c) return 0u;
	uint32_t b = c->velocity_set*2u*(uint32_t)ddf_bytes(c->storage)+1u;
	if(c->extensions&LBM_EXT_UPDATE_FIELDS) b += 16u; // rho, u (src/lbm.cpp:53-58)
	if(c->extensions&LBM_EXT_FORCE_FIELD) b += 12u;
	if(c->extensions&LBM_EXT_MOVING_BOUNDARIES) b += c->velocity_set-1u; // neighbour flags (src/lbm.cpp:62-64)
	return b;
}

int lbm_domain_create(const lbm_config* c, lbm_domain** out) {
	if(!c||!out) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_domain_create: NULL argument");
	*out = nullptr;
	const uint64_t N = (uint64_t)c->Nx*c->Ny*c->Nz;
	if(N==0ull) return fail(LBM_ERR_INVALID_ARGUMENT, "Grid point number is 0: %ux%ux%u = 0.", c->Nx, c->Ny, c->Nz);
	if(c->Nz>65535u) return fail(LBM_ERR_INVALID_ARGUMENT, "Nz=%u exceeds 65535 (one launch row of planes per z)", c->Nz);
	if((uint64_t)c->Nx*c->Ny>0xFFFFFFFFull) return fail(LBM_ERR_INVALID_ARGUMENT, "Nx*Ny must fit in 32 bits");
	if(c->velocity_set!=19u&&c->velocity_set!=27u) return fail(LBM_ERR_INVALID_ARGUMENT, "velocity_set must be 19 or 27, got %u", c->velocity_set);
	if(c->collision>LBM_TRT) return fail(LBM_ERR_INVALID_ARGUMENT, "collision must be LBM_SRT or LBM_TRT");
	if(c->storage>LBM_FP16C) return fail(LBM_ERR_INVALID_ARGUMENT, "storage must be LBM_FP32, LBM_FP16S or LBM_FP16C");
	if(c->extensions&~63u) return fail(LBM_ERR_INVALID_ARGUMENT, "unknown extension bits 0x%x", c->extensions&~63u);
	if(c->arithmetic>LBM_ARITH_FAST) return fail(LBM_ERR_INVALID_ARGUMENT, "arithmetic must be LBM_ARITH_AUTO, LBM_ARITH_EXACT or LBM_ARITH_FAST");
	if(!(c->nu>0.0f)) return fail(LBM_ERR_INVALID_ARGUMENT, c->nu==0.0f ? "Viscosity cannot be 0." : "Viscosity cannot be negative.");
	if(!(c->extensions&LBM_EXT_VOLUME_FORCE)&&(c->fx!=0.0f||c->fy!=0.0f||c->fz!=0.0f))
		return fail(LBM_ERR_INVALID_ARGUMENT, "Volume force is set, but LBM_EXT_VOLUME_FORCE is not enabled.");
	int ndev = 0;
	if(cudaGetDeviceCount(&ndev)!=cudaSuccess||ndev==0) { cudaGetLastError(); return fail(LBM_ERR_NO_DEVICE, "no CUDA device available"); }
	int dev = c->device;
	if(dev<0) { if(cudaGetDevice(&dev)!=cudaSuccess) return fail(LBM_ERR_NO_DEVICE, "cudaGetDevice failed"); }
	if(dev>=ndev) return fail(LBM_ERR_INVALID_ARGUMENT, "device %d does not exist (%d devices)", dev, ndev);
	DeviceGuard guard(dev);
	if(guard.err!=cudaSuccess) return cuda_fail(guard.err, "cudaSetDevice");

	const size_t need = (size_t)N*lbm_bytes_per_cell_device(c);
	size_t free_b = 0u, total_b = 0u;
	FX3D_CUDA(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
	if(need>free_b) return fail(LBM_ERR_OUT_OF_MEMORY, "Grid resolution (%u, %u, %u) is too large: %zu MB required, %zu MB available.",
	                            c->Nx, c->Ny, c->Nz, need/1048576u, free_b/1048576u);

	lbm_domain* d = new(std::nothrow) lbm_domain();
	if(!d) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
	d->cfg = *c;
	d->device = dev;
	d->v.q = (int)c->velocity_set;
	d->v.trt = c->collision==LBM_TRT;
	d->v.storage = (int)c->storage;
	int ext = 0;
	if(c->extensions&LBM_EXT_VOLUME_FORCE) ext |= EXT_VF;
	if((c->extensions&LBM_EXT_FORCE_FIELD)&&(c->extensions&LBM_EXT_VOLUME_FORCE)) ext |= EXT_FF; // F acts on the fluid only with VOLUME_FORCE
	if(c->extensions&LBM_EXT_EQUILIBRIUM_BOUNDARIES) ext |= EXT_EQ;
	if(c->extensions&LBM_EXT_SUBGRID) ext |= EXT_SG;
	if(c->extensions&LBM_EXT_MOVING_BOUNDARIES) ext |= EXT_MB;
	d->v.ext = ext;
	d->fused_fields = (c->extensions&LBM_EXT_UPDATE_FIELDS)!=0u;
	d->v.fast = c->arithmetic==LBM_ARITH_FAST || (c->arithmetic==LBM_ARITH_AUTO && c->storage!=LBM_FP32);
	d->g.Nx = c->Nx; d->g.Ny = c->Ny; d->g.Nz = c->Nz; d->g.NxNy = c->Nx*c->Ny; d->g.N = N;
	d->g.nx_inv = c->Nx==1u ? 0ull : (~0ull)/c->Nx+1ull; // ceil(2^64/Nx)
	d->w = lbm_relaxation_rate(c->nu);
	d->rates = make_rates(d->w);
	// stream_collide implementation: FX3D_STREAM_COLLIDE_PATH=cells|rows|pairs|pipe forces one (diagnostics
	// and tests); the default takes the two-cell packed kernel with per-thread prefetch for fast
	// arithmetic on 16-bit storage where the lattice allows it (even Nx, fewer than 2^32 cells), else
	// one thread per cell
	if(const char* p = std::getenv("FX3D_STREAM_COLLIDE_PATH")) {
		if(!std::strcmp(p, "cells")) d->path = PATH_CELLS;
		else if(!std::strcmp(p, "rows")) d->path = PATH_ROWS;
		else if(!std::strcmp(p, "pairs")) d->path = PATH_PAIRS;
		else if(!std::strcmp(p, "pipe")) d->path = PATH_PIPE;
	}

	cudaError_t e = cudaStreamCreateWithFlags(&d->own_stream, cudaStreamNonBlocking);
	if(e==cudaSuccess) { d->stream = d->own_stream; e = cudaMalloc(&d->fi, d->field_bytes(LBM_FIELD_FI)); }
	if(e==cudaSuccess) e = cudaMalloc(&d->rho, N*4u);
	if(e==cudaSuccess) e = cudaMalloc(&d->u, N*12u);
	if(e==cudaSuccess) e = cudaMalloc(&d->flags, (N+15u)&~(uint64_t)15u); // padded: kernels read flags as aligned 4-byte words
	if(e==cudaSuccess && (c->extensions&LBM_EXT_FORCE_FIELD)) e = cudaMalloc(&d->F, N*12u);
	if(e==cudaSuccess) e = cudaMalloc(&d->partials, (size_t)REDUCE_BLOCKS*4u*sizeof(double));
	if(e==cudaSuccess) e = cudaMalloc(&d->sum_dev, 4u*sizeof(double));
	if(e==cudaSuccess) e = cudaMallocHost(&d->sum_host, 4u*sizeof(double));
	if(e==cudaSuccess) e = cudaMalloc(&d->err, sizeof(int));
	if(e==cudaSuccess) e = cudaMemsetAsync(d->err, 0, sizeof(int), d->stream);
	if(e==cudaSuccess) e = cudaMemsetAsync(d->fi, 0, d->field_bytes(LBM_FIELD_FI), d->stream);
	if(e==cudaSuccess) { k_fill_f32<<<1024, 256, 0, d->stream>>>(d->rho, N, 1.0f); e = cudaGetLastError(); } // rho = 1 (src/lbm.cpp:124)
	if(e==cudaSuccess) e = cudaMemsetAsync(d->u, 0, N*12u, d->stream);
	if(e==cudaSuccess) e = cudaMemsetAsync(d->flags, 0, N, d->stream);
	if(e==cudaSuccess && d->F) e = cudaMemsetAsync(d->F, 0, N*12u, d->stream);
	if(e==cudaSuccess) e = cudaStreamSynchronize(d->stream);
	if(e!=cudaSuccess) {
		const int r = cuda_fail(e, "lbm_domain_create");
		release(d);
		delete d;
		return r;
	}
	*out = d;
	return LBM_OK;
}

int lbm_domain_destroy(lbm_domain* d) {
	if(!d) return LBM_OK;
	{
		DeviceGuard guard(d->device);
		if(d->stream) cudaStreamSynchronize(d->stream);
		release(d);
	}
	delete d;
	return LBM_OK;
}

int lbm_set_stream(lbm_domain* d, void* s) {
	FX3D_DOMAIN(d);
	d->stream = s ? (cudaStream_t)s : d->own_stream;
	return LBM_OK;
}
int lbm_get_stream(lbm_domain* d, void** s) {
	FX3D_DOMAIN(d);
	if(!s) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_get_stream: NULL output");
	*s = (void*)d->stream;
	return LBM_OK;
}
int lbm_synchronize(lbm_domain* d) {
	FX3D_DOMAIN(d);
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	return check_kernel_error(d);
}

int lbm_write_field(lbm_domain* d, const int field, const void* host, const size_t bytes) {
	FX3D_DOMAIN(d);
	if(field<LBM_FIELD_RHO||field>LBM_FIELD_FI) return fail(LBM_ERR_INVALID_ARGUMENT, "unknown field %d", field);
	if(field==LBM_FIELD_F) { const int r = ensure_F(d); if(r!=LBM_OK) return r; }
	if(!host) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_write_field: NULL host pointer");
	if(bytes!=d->field_bytes(field)) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_write_field: %zu bytes given, field has %zu", bytes, d->field_bytes(field));
	FX3D_CUDA(cudaMemcpyAsync(d->field_ptr(field), host, bytes, cudaMemcpyHostToDevice, d->stream), "cudaMemcpyAsync(write_field)");
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	if(field==LBM_FIELD_FI) { d->t_last_update_fields = UINT64_MAX; d->t_last_force_field = UINT64_MAX; }
	return LBM_OK;
}

int lbm_read_field(lbm_domain* d, const int field, void* host, const size_t bytes) {
	FX3D_DOMAIN(d);
	if(field<LBM_FIELD_RHO||field>LBM_FIELD_FI) return fail(LBM_ERR_INVALID_ARGUMENT, "unknown field %d", field);
	if(field==LBM_FIELD_F && !d->F) return fail(LBM_ERR_UNSUPPORTED, "F does not exist: enable LBM_EXT_FORCE_FIELD or call lbm_update_force_field");
	if(!host) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_read_field: NULL host pointer");
	if(bytes!=d->field_bytes(field)) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_read_field: %zu bytes given, field has %zu", bytes, d->field_bytes(field));
	if(d->initialized && (field==LBM_FIELD_RHO||field==LBM_FIELD_U)) { const int r = do_update_fields(d); if(r!=LBM_OK) return r; }
	FX3D_CUDA(cudaMemcpyAsync(host, d->field_ptr(field), bytes, cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(read_field)");
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	return check_kernel_error(d);
}

int lbm_field_device_pointer(lbm_domain* d, const int field, void** ptr, size_t* bytes) {
	FX3D_DOMAIN(d);
	if(field<LBM_FIELD_RHO||field>LBM_FIELD_FI) return fail(LBM_ERR_INVALID_ARGUMENT, "unknown field %d", field);
	if(field==LBM_FIELD_F) { const int r = ensure_F(d); if(r!=LBM_OK) return r; }
	if(ptr) *ptr = d->field_ptr(field);
	if(bytes) *bytes = d->field_bytes(field);
	return LBM_OK;
}

int lbm_initialize(lbm_domain* d) {
	FX3D_DOMAIN(d);
	d->t = 1ull; // the initialize kernel stores at odd parity (src/lbm.cpp:904)
	const StepArgs a = d->args();
	cudaError_t e;
	switch(d->v.storage) {
		case ST_FP32: e = launch_initialize_fp32(d->v, a, d->stream); break;
		case ST_FP16S: e = launch_initialize_fp16s(d->v, a, d->stream); break;
		default: e = launch_initialize_fp16c(d->v, a, d->stream); break;
	}
	d->t = 0ull; // src/lbm.cpp:920
	if(e!=cudaSuccess) return cuda_fail(e, "initialize");
	d->t_last_update_fields = d->fused_fields ? 0ull : UINT64_MAX; // src/lbm.cpp:261-266
	d->t_last_force_field = UINT64_MAX;
	d->initialized = true;
	return LBM_OK;
}

int lbm_stream_collide(lbm_domain* d, const uint64_t steps) {
	FX3D_DOMAIN(d);
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_stream_collide: call lbm_initialize first");
	for(uint64_t s=0ull; s<steps; s++) {
		const int r = launch_stream_collide(d);
		if(r!=LBM_OK) return r;
		d->t++;
	}
	if(d->fused_fields) d->t_last_update_fields = d->t; // src/lbm.cpp:255-260
	return LBM_OK;
}

int lbm_update_fields(lbm_domain* d) {
	FX3D_DOMAIN(d);
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_update_fields: call lbm_initialize first");
	return do_update_fields(d);
}

int lbm_get_time_step(lbm_domain* d, uint64_t* t) {
	if(!d||!t) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_get_time_step: NULL argument");
	*t = d->t;
	return LBM_OK;
}
int lbm_set_force(lbm_domain* d, const float fx, const float fy, const float fz) {
	if(!d) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_set_force: domain is NULL");
	if(!(d->cfg.extensions&LBM_EXT_VOLUME_FORCE)&&(fx!=0.0f||fy!=0.0f||fz!=0.0f))
		return fail(LBM_ERR_UNSUPPORTED, "Volume force is set, but LBM_EXT_VOLUME_FORCE is not enabled.");
	d->cfg.fx = fx; d->cfg.fy = fy; d->cfg.fz = fz;
	d->t_last_update_fields = UINT64_MAX;
	return LBM_OK;
}
int lbm_is_initialized(lbm_domain* d, int* initialized) {
	if(!d||!initialized) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_is_initialized: NULL argument");
	*initialized = d->initialized ? 1 : 0;
	return LBM_OK;
}
int lbm_reset(lbm_domain* d) {
	if(!d) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_reset: domain is NULL");
	d->initialized = false;
	return LBM_OK;
}

int lbm_update_force_field(lbm_domain* d) {
	FX3D_DOMAIN(d);
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_update_force_field: call lbm_initialize first");
	return do_update_force_field(d);
}
int lbm_reset_force_field(lbm_domain* d) {
	FX3D_DOMAIN(d);
	const int r = ensure_F(d);
	if(r!=LBM_OK) return r;
	FX3D_CUDA(cudaMemsetAsync(d->F, 0, d->g.N*12u, d->stream), "cudaMemsetAsync(F)");
	d->t_last_force_field = UINT64_MAX;
	return LBM_OK;
}

int lbm_object_center_of_mass(lbm_domain* d, const uint8_t marker, double out[4]) {
	FX3D_DOMAIN(d);
	if(!out) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_center_of_mass: NULL output");
	double s[4];
	const int r = object_sum(d, 0, marker, 0.0, 0.0, 0.0, s, 4);
	if(r!=LBM_OK) return r;
	out[3] = s[3];
	for(int i=0; i<3; i++) out[i] = s[3]>0.0 ? s[i]/s[3] : 0.0;
	return LBM_OK;
}
int lbm_object_force(lbm_domain* d, const uint8_t marker, double out[3]) {
	FX3D_DOMAIN(d);
	if(!out) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_force: NULL output");
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_object_force: call lbm_initialize first");
	return object_sum(d, 1, marker, 0.0, 0.0, 0.0, out, 3);
}
int lbm_object_torque(lbm_domain* d, const uint8_t marker, const double cx, const double cy, const double cz, double out[3]) {
	FX3D_DOMAIN(d);
	if(!out) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_object_torque: NULL output");
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_object_torque: call lbm_initialize first");
	return object_sum(d, 2, marker, cx, cy, cz, out, 3);
}

int lbm_voxelize_mesh(lbm_domain* d, const float* p0, const float* p1, const float* p2, const uint32_t T, const uint8_t flag,
                      const float center[3], const float linear_velocity[3], const float rotational_velocity[3]) {
	FX3D_DOMAIN(d);
	if(T==0u) return LBM_OK;
	if(!p0||!p1||!p2) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_voxelize_mesh: NULL vertex array");
	const float zero[3] = {0.0f, 0.0f, 0.0f};
	const float* c = center ? center : zero;
	const float* lv = linear_velocity ? linear_velocity : zero;
	const float* rv = rotational_velocity ? rotational_velocity : zero;
	// mesh bounds (Mesh::find_bounds, src/utilities.hpp:4458-4469)
	float pmin[3] = {p0[0], p0[1], p0[2]}, pmax[3] = {p0[0], p0[1], p0[2]};
	for(uint32_t i=0u; i<T; i++) {
		for(int k=0; k<3; k++) {
			pmin[k] = fminf(fminf(fminf(p0[3u*i+k], p1[3u*i+k]), p2[3u*i+k]), pmin[k]);
			pmax[k] = fmaxf(fmaxf(fmaxf(p0[3u*i+k], p1[3u*i+k]), p2[3u*i+k]), pmax[k]);
		}
	}
	// bounding box +-2 cells, rotation centre and velocities (src/lbm.cpp:280-296)
	float bbu[16];
	std::memcpy(&bbu[0], &T, 4);
	const float x0 = pmin[0]-2.0f, y0 = pmin[1]-2.0f, z0 = pmin[2]-2.0f, x1 = pmax[0]+2.0f, y1 = pmax[1]+2.0f, z1 = pmax[2]+2.0f;
	bbu[1] = x0; bbu[2] = y0; bbu[3] = z0; bbu[4] = x1; bbu[5] = y1; bbu[6] = z1;
	for(int k=0; k<3; k++) { bbu[7+k] = c[k]; bbu[10+k] = lv[k]; bbu[13+k] = rv[k]; }
	// ray direction (src/lbm.cpp:297-318)
	uint32_t direction = 0u;
	if(sqrtf(rv[0]*rv[0]+rv[1]*rv[1]+rv[2]*rv[2])==0.0f) {
		const float v[3] = {(y1-y0)*(z1-z0), (z1-z0)*(x1-x0), (x1-x0)*(y1-y0)};
		float vmin = v[0];
		for(uint32_t i=1u; i<3u; i++) if(v[i]<vmin) { vmin = v[i]; direction = i; }
	} else {
		const float v[3] = {fabsf(rv[0]), fabsf(rv[1]), fabsf(rv[2])};
		float vmax = v[0];
		for(uint32_t i=1u; i<3u; i++) if(v[i]>vmax) { vmax = v[i]; direction = i; }
	}
	float* dev = nullptr;
	const size_t tb = (size_t)T*12u;
	FX3D_CUDA(cudaMalloc(&dev, 3u*tb+16u*sizeof(float)), "cudaMalloc(mesh)");
	cudaError_t e = cudaMemcpyAsync(dev, p0, tb, cudaMemcpyHostToDevice, d->stream);
	if(e==cudaSuccess) e = cudaMemcpyAsync((char*)dev+tb, p1, tb, cudaMemcpyHostToDevice, d->stream);
	if(e==cudaSuccess) e = cudaMemcpyAsync((char*)dev+2u*tb, p2, tb, cudaMemcpyHostToDevice, d->stream);
	if(e==cudaSuccess) e = cudaMemcpyAsync((char*)dev+3u*tb, bbu, sizeof(bbu), cudaMemcpyHostToDevice, d->stream);
	if(e==cudaSuccess) e = launch_voxelize(d->v, d->g, direction, d->fi, d->u, d->flags, d->t+1ull, flag,
	                                       dev, (const float*)((char*)dev+tb), (const float*)((char*)dev+2u*tb), (const float*)((char*)dev+3u*tb), d->stream);
	// a moving solid marks its fluid neighbours (src/lbm.cpp:1082-1084)
	const bool moving = sqrtf(lv[0]*lv[0]+lv[1]*lv[1]+lv[2]*lv[2])>0.0f || sqrtf(rv[0]*rv[0]+rv[1]*rv[1]+rv[2]*rv[2])>0.0f;
	if(e==cudaSuccess && (d->v.ext&EXT_MB) && (flag&0x03u)==0x01u && moving) // (flag&(TYPE_S|TYPE_E))==TYPE_S
		e = launch_update_moving_boundaries(d->v.q, d->g, d->u, d->flags, d->stream);
	if(e==cudaSuccess) e = cudaStreamSynchronize(d->stream);
	cudaFree(dev);
	if(e!=cudaSuccess) return cuda_fail(e, "voxelize_mesh");
	return LBM_OK;
}

// ---- VTK export
namespace {
struct VtkStaging { // two device + two pinned host chunks, freed on scope exit
	void* dev[2] = {nullptr, nullptr};
	void* host[2] = {nullptr, nullptr};
	cudaEvent_t done[2] = {nullptr, nullptr};
	std::FILE* file = nullptr;
	~VtkStaging() {
		for(int i=0; i<2; i++) {
			if(dev[i]) cudaFree(dev[i]);
			if(host[i]) cudaFreeHost(host[i]);
			if(done[i]) cudaEventDestroy(done[i]);
		}
		if(file) std::fclose(file);
	}
};
} // namespace

int lbm_write_vtk(lbm_domain* d, const int field, const char* filename, const float spacing, const float scale) {
	FX3D_DOMAIN(d);
	if(!filename||!*filename) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_write_vtk: no file name");
	if(field!=LBM_FIELD_RHO&&field!=LBM_FIELD_U&&field!=LBM_FIELD_FLAGS&&field!=LBM_FIELD_F)
		return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_write_vtk: field %d has no VTK form (rho, u, flags or F)", field);
	if(field==LBM_FIELD_F && !d->F) return fail(LBM_ERR_UNSUPPORTED, "F does not exist: enable LBM_EXT_FORCE_FIELD or call lbm_update_force_field");
	if(d->initialized && (field==LBM_FIELD_RHO||field==LBM_FIELD_U)) { const int r = do_update_fields(d); if(r!=LBM_OK) return r; }
	const uint32_t dims = field==LBM_FIELD_U||field==LBM_FIELD_F ? 3u : 1u;
	const bool u8 = field==LBM_FIELD_FLAGS;
	const size_t elem = u8 ? 1u : 4u;
	// header of src/lbm.hpp:308-317: title "FluidX3D <file name>", origin at the box centre, numbers as std::to_string
	const std::string path(filename);
	const size_t slash = path.rfind('/');
	const std::string base = slash==std::string::npos ? path : path.substr(slash+1u);
	const float ox = spacing*(0.5f-0.5f*(float)d->g.Nx), oy = spacing*(0.5f-0.5f*(float)d->g.Ny), oz = spacing*(0.5f-0.5f*(float)d->g.Nz);
	char head[1024];
	const int hl = std::snprintf(head, sizeof(head),
		"# vtk DataFile Version 3.0\nFluidX3D %s\nBINARY\nDATASET STRUCTURED_POINTS\nDIMENSIONS %u %u %u\nORIGIN %f %f %f\nSPACING %f %f %f\n"
		"POINT_DATA %llu\nSCALARS data %s %u\nLOOKUP_TABLE default\n",
		base.c_str(), d->g.Nx, d->g.Ny, d->g.Nz, (double)ox, (double)oy, (double)oz, (double)spacing, (double)spacing, (double)spacing,
		(unsigned long long)d->g.N, u8 ? "unsigned_char" : "float", dims);
	if(hl<=0||hl>=(int)sizeof(head)) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_write_vtk: file name too long");
	if(slash!=std::string::npos && slash>0u) { // create the folder like the reference's create_folder (src/utilities.hpp:4197-4204)
		std::error_code ec;
		std::filesystem::create_directories(path.substr(0u, slash), ec);
	}
	VtkStaging st;
	st.file = std::fopen(filename, "wb");
	if(!st.file) return fail(LBM_ERR_IO, "lbm_write_vtk: cannot open \"%s\" for writing", filename);
	if(std::fwrite(head, 1u, (size_t)hl, st.file)!=(size_t)hl) return fail(LBM_ERR_IO, "lbm_write_vtk: write to \"%s\" failed", filename);
	// chunks of up to 16M values, packed on the GPU (FP32 fields) while the previous chunk is written
	uint64_t chunk_cells = (16ull<<20)/dims;
	if(chunk_cells>d->g.N) chunk_cells = d->g.N;
	const size_t chunk_bytes = (size_t)chunk_cells*dims*elem;
	for(int i=0; i<2; i++) {
		if(!u8) FX3D_CUDA(cudaMalloc(&st.dev[i], chunk_bytes), "cudaMalloc(vtk staging)");
		FX3D_CUDA(cudaHostAlloc(&st.host[i], chunk_bytes, cudaHostAllocDefault), "cudaHostAlloc(vtk staging)");
		FX3D_CUDA(cudaEventCreateWithFlags(&st.done[i], cudaEventDisableTiming), "cudaEventCreate");
	}
	const uint64_t chunks = (d->g.N+chunk_cells-1ull)/chunk_cells;
	const float* src = (const float*)d->field_ptr(field);
	auto issue = [&](const uint64_t k) -> cudaError_t {
		const int b = (int)(k&1ull);
		const uint64_t first = k*chunk_cells, count = first+chunk_cells<=d->g.N ? chunk_cells : d->g.N-first;
		cudaError_t e;
		if(u8) e = cudaMemcpyAsync(st.host[b], d->flags+first, (size_t)count, cudaMemcpyDeviceToHost, d->stream);
		else {
			e = launch_pack_vtk(src, d->g.N, dims, first, count, scale, (uint32_t*)st.dev[b], d->stream);
			if(e==cudaSuccess) e = cudaMemcpyAsync(st.host[b], st.dev[b], (size_t)count*dims*4u, cudaMemcpyDeviceToHost, d->stream);
		}
		if(e==cudaSuccess) e = cudaEventRecord(st.done[b], d->stream);
		return e;
	};
	FX3D_CUDA(issue(0ull), "vtk chunk");
	for(uint64_t k=0ull; k<chunks; k++) {
		if(k+1ull<chunks) FX3D_CUDA(issue(k+1ull), "vtk chunk"); // the buffers of chunk k-1, written out already
		const int b = (int)(k&1ull);
		FX3D_CUDA(cudaEventSynchronize(st.done[b]), "cudaEventSynchronize");
		const uint64_t first = k*chunk_cells, count = first+chunk_cells<=d->g.N ? chunk_cells : d->g.N-first;
		const size_t nb = (size_t)count*dims*elem;
		if(std::fwrite(st.host[b], 1u, nb, st.file)!=nb) {
			cudaStreamSynchronize(d->stream);
			return fail(LBM_ERR_IO, "lbm_write_vtk: write to \"%s\" failed", filename);
		}
	}
	const int rc = std::fclose(st.file);
	st.file = nullptr;
	if(rc!=0) return fail(LBM_ERR_IO, "lbm_write_vtk: closing \"%s\" failed", filename);
	return LBM_OK;
}

int lbm_update_moving_boundaries(lbm_domain* d) {
	FX3D_DOMAIN(d);
	if(!(d->v.ext&EXT_MB)) return fail(LBM_ERR_UNSUPPORTED, "lbm_update_moving_boundaries needs LBM_EXT_MOVING_BOUNDARIES");
	FX3D_CUDA(launch_update_moving_boundaries(d->v.q, d->g, d->u, d->flags, d->stream), "update_moving_boundaries");
	return LBM_OK;
}

int lbm_unvoxelize_mesh(lbm_domain* d, const float pmin[3], const float pmax[3], const uint8_t flag) {
	FX3D_DOMAIN(d);
	if(!pmin||!pmax) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_unvoxelize_mesh: NULL bounds");
	const float box[6] = {pmin[0], pmin[1], pmin[2], pmax[0], pmax[1], pmax[2]};
	FX3D_CUDA(launch_unvoxelize(d->g, d->flags, flag, box, d->stream), "unvoxelize_mesh");
	return LBM_OK;
}

} // extern "C"

// ==================================================================== adjoint driver
namespace {

struct DeviceBuffer { // freed on scope exit
	void* p = nullptr;
	~DeviceBuffer() { if(p) cudaFree(p); }
};

// one forward step in place on a work copy of the DDFs that also writes the rho/u its cells collide
// with (its fused-fields output) into a moment checkpoint: rho at mom[0, N), u at mom[N, 4N)
int step_with_moments(lbm_domain* d, void* work, float* mom, const uint64_t t, cudaStream_t stream) {
	StepArgs a = d->args();
	a.t = t;
	a.fi = work; a.fi_dst = work;
	a.fields_out = mom ? 1 : 0;
	if(mom) { a.rho_out = mom; a.u_out = mom+d->g.N; }
	cudaError_t e;
	switch(d->v.storage) {
		case ST_FP32: e = launch_stream_collide_fp32(d->v, a, d->path, stream); break;
		case ST_FP16S: e = launch_stream_collide_fp16s(d->v, a, d->path, stream); break;
		default: e = launch_stream_collide_fp16c(d->v, a, d->path, stream); break;
	}
	return e==cudaSuccess ? LBM_OK : cuda_fail(e, "stream_collide (recompute)");
}

struct StreamAndEvents { // a second stream and events for the overlapped reverse sweep, released on scope exit
	cudaStream_t stream = nullptr;
	cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
	~StreamAndEvents() {
		if(stream) { cudaStreamSynchronize(stream); cudaStreamDestroy(stream); }
		for(cudaEvent_t& e : ev) if(e) cudaEventDestroy(e);
	}
};

struct EventTimer {
	cudaEvent_t a = nullptr, b = nullptr;
	explicit EventTimer(cudaStream_t s) { cudaEventCreate(&a); cudaEventCreate(&b); cudaEventRecord(a, s); }
	double stop(cudaStream_t s) { float ms = 0.0f; cudaEventRecord(b, s); cudaEventSynchronize(b); cudaEventElapsedTime(&ms, a, b); return ms; }
	~EventTimer() { if(a) cudaEventDestroy(a); if(b) cudaEventDestroy(b); }
};

} // namespace

extern "C" int lbm_run_adjoint(lbm_domain* d, const lbm_adjoint_config* cfg, double* objective, float* gradient, lbm_adjoint_stats* stats) {
	FX3D_DOMAIN(d);
	if(!cfg) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: NULL config");
	if(!d->initialized) return fail(LBM_ERR_NOT_INITIALIZED, "lbm_run_adjoint: call lbm_initialize first");
	if(d->v.ext&EXT_SG) return fail(LBM_ERR_UNSUPPORTED, "lbm_run_adjoint does not support LBM_EXT_SUBGRID (the adjoint has no Smagorinsky-Lilly term)");
	if(d->v.ext&EXT_MB) return fail(LBM_ERR_UNSUPPORTED, "lbm_run_adjoint does not support LBM_EXT_MOVING_BOUNDARIES");
	if(!adjoint_supported(d->v) || !d->F) return fail(LBM_ERR_UNSUPPORTED, "lbm_run_adjoint needs LBM_EXT_VOLUME_FORCE and LBM_EXT_FORCE_FIELD (F is the design variable)");
	if(d->g.N>0xFFFFFFFFull) return fail(LBM_ERR_UNSUPPORTED, "lbm_run_adjoint needs fewer than 2^32 cells (its kernels use 32-bit cell indices)");
	if(cfg->steps==0ull||cfg->checkpoint_interval==0ull) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: steps and checkpoint_interval must be >= 1");
	if(cfg->objective!=LBM_OBJECTIVE_KINETIC_ENERGY_PLANE_X && cfg->objective!=LBM_OBJECTIVE_DRAG_X) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: unknown objective %u", cfg->objective);
	if(cfg->objective==LBM_OBJECTIVE_KINETIC_ENERGY_PLANE_X && cfg->plane_x>=d->g.Nx) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: plane_x outside the lattice");
	if(cfg->window_end<cfg->window_begin) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: empty objective window");
	const uint64_t t0 = d->t, T = cfg->steps, K = cfg->checkpoint_interval, N = d->g.N;
	const size_t SB = d->field_bytes(LBM_FIELD_FI);
	const uint64_t nsnap = (T+K-1ull)/K;
	// objective weight: 1/(window length) (x 1/(fluid cells of the plane) for the kinetic energy)
	double weight = 1.0/(double)(cfg->window_end-cfg->window_begin+1ull);
	if(cfg->objective==LBM_OBJECTIVE_KINETIC_ENERGY_PLANE_X) {
		std::string flags(N, '\0');
		FX3D_CUDA(cudaMemcpyAsync(&flags[0], d->flags, N, cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(flags)");
		FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
		uint64_t cells = 0ull;
		const bool eq = (d->v.ext&EXT_EQ)!=0;
		for(uint64_t n=cfg->plane_x; n<N; n+=d->g.Nx) {
			const uint8_t fl = (uint8_t)flags[n];
			if((fl&3u)!=1u && (fl&0x38u)!=0x20u && !(eq && (fl&3u)==2u)) cells++;
		}
		if(cells==0ull) return fail(LBM_ERR_INVALID_ARGUMENT, "lbm_run_adjoint: plane x=%u has no fluid cells", cfg->plane_x);
		weight /= (double)cells;
	}
	// workspace: DDF snapshots every K steps, one work copy of the DDFs for the recomputation, and
	// moment checkpoints (rho/u, 16 B per cell) of every step of a segment; with room for two moment
	// sets the recomputation of the next segment runs on a second stream while the adjoint steps of
	// this one run. Short of room for one set, two levels: DDF sub-snapshots every K2 steps of a
	// segment, and moments of one sub-segment.
	size_t free_b = 0u, total_b = 0u;
	FX3D_CUDA(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
	const size_t MB = N*16u; // moments of one step
	const size_t fixed = (size_t)d->cfg.velocity_set*N*4u+N*12u+64u;
	size_t margin = 512ull<<20;
	if(cfg->workspace_limit_kib!=0u) { // the caller's cap, within what is free
		const size_t cap = (size_t)cfg->workspace_limit_kib<<10;
		if(cap+margin<=free_b) { free_b = cap; margin = 0u; }
	}
	uint64_t K2 = K; // steps per (sub-)segment with moments
	uint32_t levels = 1u;
	size_t need = (nsnap+1ull)*SB+2ull*K*MB+fixed;
	bool overlap = nsnap>1ull && need+margin<=free_b;
	if(!overlap) need = (nsnap+1ull)*SB+K*MB+fixed;
	if(need+margin>free_b) {
		levels = 2u;
		K2 = 1ull; while(K2*K2<K) K2++;
		need = (nsnap+1ull+(K+K2-1ull)/K2)*SB+K2*MB+fixed;
		if(need+margin>free_b) return fail(LBM_ERR_OUT_OF_MEMORY, "lbm_run_adjoint: %zu MB of workspace needed, %zu MB free; increase checkpoint_interval", need>>20, free_b>>20);
	}
	const uint64_t nsub = levels==2u ? (K+K2-1ull)/K2 : 0ull;
	DeviceBuffer snaps, work, moms, sub, lam, grad, Jd;
	FX3D_CUDA(cudaMalloc(&snaps.p, (size_t)nsnap*SB), "cudaMalloc(snapshots)");
	FX3D_CUDA(cudaMalloc(&work.p, SB), "cudaMalloc(recomputation state)");
	FX3D_CUDA(cudaMalloc(&moms.p, (size_t)(overlap ? 2ull*K : K2)*MB), "cudaMalloc(moment checkpoints)");
	if(levels==2u) FX3D_CUDA(cudaMalloc(&sub.p, (size_t)nsub*SB), "cudaMalloc(sub-snapshots)");
	FX3D_CUDA(cudaMalloc(&lam.p, (size_t)d->cfg.velocity_set*N*4u), "cudaMalloc(adjoint DDFs)");
	FX3D_CUDA(cudaMalloc(&grad.p, N*12u), "cudaMalloc(gradient)");
	FX3D_CUDA(cudaMalloc(&Jd.p, sizeof(double)), "cudaMalloc(J)");
	auto snap = [&](const uint64_t i) { return (void*)((char*)snaps.p+(size_t)i*SB); };
	auto mom = [&](const uint64_t set, const uint64_t i) { return (float*)((char*)moms.p+((size_t)set*K+(size_t)i)*MB); };
	auto subs = [&](const uint64_t i) { return (void*)((char*)sub.p+(size_t)i*SB); };
	AdjArgs j;
	j.lambda = (float*)lam.p; j.grad = (float*)grad.p; j.obj_kind = (int)cfg->objective; j.plane_x = cfg->plane_x; j.marker = cfg->marker;
	j.moments = nullptr;
	auto in_window = [&](const uint64_t t) { return t>=cfg->window_begin && t<=cfg->window_end; };
	auto args_at = [&](const uint64_t t, const void* state) { StepArgs a = d->args(); a.t = t; a.fi = const_cast<void*>(state); return a; };

	// ---- forward sweep (in place on the domain's DDFs), snapshots, objective. With one level, the
	// steps of the last segment write its moment checkpoints themselves (the same kernel on the same
	// states as a recomputation), so the reverse sweep starts without recomputing it; not when the
	// domain's steps already write their fields to rho/u (UPDATE_FIELDS)
	const uint64_t last0 = (nsnap-1ull)*K, last_set = overlap ? ((nsnap-1ull)&1ull) : 0ull;
	const bool forward_moments = levels==1u && !d->fused_fields;
	FX3D_CUDA(cudaMemsetAsync(Jd.p, 0, sizeof(double), d->stream), "cudaMemsetAsync(J)");
	EventTimer tf(d->stream);
	for(uint64_t k=0ull; k<=T; k++) {
		if(k%K==0ull && k<T) FX3D_CUDA(cudaMemcpyAsync(snap(k/K), d->fi, SB, cudaMemcpyDeviceToDevice, d->stream), "cudaMemcpyAsync(snapshot)");
		if(in_window(t0+k)) {
			j.state = d->fi; j.obj_weight = (float)weight;
			FX3D_CUDA(launch_objective_value(d->v, args_at(t0+k, d->fi), j, d->partials, (double*)Jd.p, d->stream), "objective");
		}
		if(k<T) {
			const int r = forward_moments && k>=last0 ? step_with_moments(d, d->fi, mom(last_set, k-last0), t0+k, d->stream) : launch_stream_collide(d);
			if(r!=LBM_OK) return r;
			d->t++;
		}
	}
	const double forward_ms = tf.stop(d->stream);
	// ---- reverse sweep
	double recompute_ms = 0.0, adjoint_ms = 0.0;
	FX3D_CUDA(cudaMemsetAsync(lam.p, 0, (size_t)d->cfg.velocity_set*N*4u, d->stream), "cudaMemsetAsync(lambda)");
	FX3D_CUDA(cudaMemsetAsync(grad.p, 0, N*12u, d->stream), "cudaMemsetAsync(gradient)");
	if(in_window(t0+T)) {
		j.state = d->fi; j.obj_weight = (float)weight;
		FX3D_CUDA(launch_adjoint_step(d->v, args_at(t0+T, d->fi), j, true, d->stream), "adjoint objective");
	}
	// moments of steps k0 .. k1-1 into set `set`, from the DDF state f^{k0} at `start` (work copy)
	auto recompute = [&](const uint64_t k0, const uint64_t k1, const void* start, const uint64_t set, cudaStream_t st) -> int {
		FX3D_CUDA(cudaMemcpyAsync(work.p, start, SB, cudaMemcpyDeviceToDevice, st), "cudaMemcpyAsync(state)");
		for(uint64_t k=k0; k<k1; k++) { const int r = step_with_moments(d, work.p, mom(set, k-k0), t0+k, st); if(r!=LBM_OK) return r; }
		return LBM_OK;
	};
	auto adjoint_steps = [&](const uint64_t k0, const uint64_t k1, const uint64_t set) -> int { // steps k1-1 .. k0
		for(uint64_t k=k1; k-->k0;) {
			j.moments = mom(set, k-k0); j.state = nullptr; j.obj_weight = in_window(t0+k) ? (float)weight : 0.0f;
			FX3D_CUDA(launch_adjoint_step(d->v, args_at(t0+k, nullptr), j, false, d->stream), "adjoint step");
		}
		return LBM_OK;
	};
	EventTimer trev(d->stream);
	StreamAndEvents ov;
	if(overlap) {
		// segment s uses moment set s%2. Stream R recomputes segment s-1 while the domain's stream runs
		// the adjoint steps of segment s; R waits until the adjoint steps of segment s+1 have released
		// the set it refills. The work copy of the DDFs belongs to stream R alone.
		FX3D_CUDA(cudaStreamCreateWithFlags(&ov.stream, cudaStreamNonBlocking), "cudaStreamCreate");
		for(cudaEvent_t& e : ov.ev) FX3D_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
		cudaEvent_t* rec_done = ov.ev; cudaEvent_t* adj_done = ov.ev+2; cudaEvent_t start = ov.ev[4];
		auto recompute_segment = [&](const uint64_t sg, const bool wait_set) -> int {
			const uint64_t k0 = sg*K, k1 = std::min<uint64_t>(k0+K, T);
			if(wait_set) FX3D_CUDA(cudaStreamWaitEvent(ov.stream, adj_done[sg&1ull], 0), "cudaStreamWaitEvent");
			if(!(forward_moments && sg==nsnap-1ull)) { const int r = recompute(k0, k1, snap(sg), sg&1ull, ov.stream); if(r!=LBM_OK) return r; }
			FX3D_CUDA(cudaEventRecord(rec_done[sg&1ull], ov.stream), "cudaEventRecord");
			return LBM_OK;
		};
		FX3D_CUDA(cudaEventRecord(start, d->stream), "cudaEventRecord");
		FX3D_CUDA(cudaStreamWaitEvent(ov.stream, start, 0), "cudaStreamWaitEvent"); // after lambda/grad are cleared
		{ const int r = recompute_segment(nsnap-1ull, false); if(r!=LBM_OK) return r; }
		for(uint64_t sg=nsnap; sg-->0ull;) {
			const uint64_t k0 = sg*K, k1 = std::min<uint64_t>(k0+K, T);
			if(sg>=1ull) { const int r = recompute_segment(sg-1ull, sg+1ull<nsnap); if(r!=LBM_OK) return r; }
			FX3D_CUDA(cudaStreamWaitEvent(d->stream, rec_done[sg&1ull], 0), "cudaStreamWaitEvent");
			{ const int r = adjoint_steps(k0, k1, sg&1ull); if(r!=LBM_OK) return r; }
			FX3D_CUDA(cudaEventRecord(adj_done[sg&1ull], d->stream), "cudaEventRecord");
		}
	}
	for(uint64_t s=nsnap; !overlap && s-->0ull;) {
		const uint64_t k0 = s*K, k1 = std::min<uint64_t>(k0+K, T);
		if(levels==2u) { // DDF sub-snapshots every K2 steps of the segment
			EventTimer tr(d->stream);
			FX3D_CUDA(cudaMemcpyAsync(work.p, snap(s), SB, cudaMemcpyDeviceToDevice, d->stream), "cudaMemcpyAsync(state)");
			for(uint64_t k=k0; k<k1; k++) {
				if((k-k0)%K2==0ull) FX3D_CUDA(cudaMemcpyAsync(subs((k-k0)/K2), work.p, SB, cudaMemcpyDeviceToDevice, d->stream), "cudaMemcpyAsync(sub-snapshot)");
				if(k+1ull<k1) { const int r = step_with_moments(d, work.p, nullptr, t0+k, d->stream); if(r!=LBM_OK) return r; }
			}
			recompute_ms += tr.stop(d->stream);
		}
		const uint64_t nb = levels==2u ? (k1-k0+K2-1ull)/K2 : 1ull;
		for(uint64_t b=nb; b-->0ull;) {
			const uint64_t b0 = levels==2u ? k0+b*K2 : k0, b1 = levels==2u ? std::min<uint64_t>(k0+(b+1ull)*K2, k1) : k1;
			EventTimer tr(d->stream);
			if(!(forward_moments && s==nsnap-1ull)) { const int r = recompute(b0, b1, levels==2u ? subs(b) : snap(s), 0ull, d->stream); if(r!=LBM_OK) return r; }
			recompute_ms += tr.stop(d->stream);
			EventTimer ta(d->stream);
			{ const int r = adjoint_steps(b0, b1, 0ull); if(r!=LBM_OK) return r; }
			adjoint_ms += ta.stop(d->stream);
		}
	}
	const double reverse_ms = trev.stop(d->stream);
	double Jh = 0.0;
	FX3D_CUDA(cudaMemcpyAsync(&Jh, Jd.p, sizeof(double), cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(J)");
	if(gradient) FX3D_CUDA(cudaMemcpyAsync(gradient, grad.p, N*12u, cudaMemcpyDeviceToHost, d->stream), "cudaMemcpyAsync(gradient)");
	FX3D_CUDA(cudaStreamSynchronize(d->stream), "cudaStreamSynchronize");
	{ const int r = check_kernel_error(d); if(r!=LBM_OK) return r; }
	if(objective) *objective = Jh;
	if(stats) {
		stats->forward_ms = forward_ms; stats->recompute_ms = recompute_ms; stats->adjoint_ms = adjoint_ms;
		stats->workspace_bytes = (uint64_t)need; stats->levels = levels; stats->overlapped = overlap ? 1u : 0u;
		stats->reverse_ms = reverse_ms;
	}
	d->t_last_update_fields = d->fused_fields ? d->t : UINT64_MAX;
	d->t_last_force_field = UINT64_MAX;
	return LBM_OK;
}
