// Reference-kernel CPU harness (test infrastructure only; never part of the product path).
//
// Compiles the reference's own OpenCL C kernel text (src/kernel.cpp, extracted by
// extract_kernel_text.cpp) as C++ under opencl_c_shim.hpp and launches its kernels over host
// threads, one work-item per loop iteration, the way src/utilities.hpp:77-93 parallel_for splits a
// range. The variant (velocity set, collision operator, DDF storage, extensions) is fixed at compile
// time through REF_DEFINES, a header that build_ref.py writes following the device defines of
// src/lbm.cpp:334-468; grid size and relaxation rate are runtime values here (the reference bakes
// them in as literals, which changes nothing in the arithmetic).
//
// Built by oracle/ref_harness/build_ref.py into oracle/_ref/; never shipped in the package.
#include <thread>
#include <vector>
#include "opencl_c_shim.hpp"

namespace ocl {
thread_local ulong global_id = 0ull;
static uint g_Nx = 1u, g_Ny = 1u, g_Nz = 1u;
static ulong g_N = 1ull;
static float g_w = 1.0f;
static uint g_threads = 1u;
#include REF_DEFINES
typedef fpxx ddf_t; // storage type of the DDFs in this variant
#include REF_KERNEL_TEXT
} // namespace ocl

typedef ocl::uchar u8; typedef ocl::uint u32; typedef ocl::ulong u64;

template<typename L> static void launch(const u64 items, L&& body) { // contiguous split of [0,items) over g_threads
	const u32 T = ocl::g_threads;
	std::vector<std::thread> pool;
	for(u32 t=0u; t<T; t++) pool.emplace_back([=, &body]() {
		for(u64 n=items*t/T; n<items*(t+1u)/T; n++) { ocl::global_id = n; body(); }
	});
	for(auto& th : pool) th.join();
}

extern "C" {

int ref_velocity_set() { return (int)def_velocity_set; }
int ref_fpxx_bytes() { return (int)sizeof(ocl::ddf_t); }

void ref_configure(const u32 Nx, const u32 Ny, const u32 Nz, const float w, const u32 threads) {
	ocl::g_Nx = Nx; ocl::g_Ny = Ny; ocl::g_Nz = Nz;
	ocl::g_N = (u64)Nx*(u64)Ny*(u64)Nz;
	ocl::g_w = w;
	ocl::g_threads = threads>0u ? threads : 1u;
}

void ref_initialize(void* fi, float* rho, float* u, u8* flags) {
	launch(ocl::g_N, [&]() { ocl::initialize((ocl::ddf_t*)fi, rho, u, flags); });
}

void ref_stream_collide(void* fi, float* rho, float* u, u8* flags, const u64 t, const float fx, const float fy, const float fz, const float* F) {
#ifdef FORCE_FIELD
	launch(ocl::g_N, [&]() { ocl::stream_collide((ocl::ddf_t*)fi, rho, u, flags, t, fx, fy, fz, F); });
#else
	(void)F;
	launch(ocl::g_N, [&]() { ocl::stream_collide((ocl::ddf_t*)fi, rho, u, flags, t, fx, fy, fz); });
#endif
}

void ref_update_fields(const void* fi, float* rho, float* u, const u8* flags, const u64 t, const float fx, const float fy, const float fz, const float* F) {
#ifdef FORCE_FIELD
	launch(ocl::g_N, [&]() { ocl::update_fields((const ocl::ddf_t*)fi, rho, u, flags, t, fx, fy, fz, F); });
#else
	(void)F;
	launch(ocl::g_N, [&]() { ocl::update_fields((const ocl::ddf_t*)fi, rho, u, flags, t, fx, fy, fz); });
#endif
}

int ref_update_force_field(const void* fi, const u8* flags, const u64 t, float* F) {
#ifdef FORCE_FIELD
	launch(ocl::g_N, [&]() { ocl::update_force_field((const ocl::ddf_t*)fi, flags, t, F); });
	return 0;
#else
	(void)fi; (void)flags; (void)t; (void)F;
	return -1;
#endif
}

int ref_update_moving_boundaries(const float* u, u8* flags) {
#ifdef MOVING_BOUNDARIES
	launch(ocl::g_N, [&]() { ocl::update_moving_boundaries(u, flags); });
	return 0;
#else
	(void)u; (void)flags;
	return -1;
#endif
}

void ref_voxelize_mesh(const u32 direction, void* fi, float* u, u8* flags, const u64 t, const u8 flag, const float* p0, const float* p1, const float* p2, const float* bbu) {
	const u64 A = direction==0u ? (u64)ocl::g_Ny*ocl::g_Nz : direction==1u ? (u64)ocl::g_Nz*ocl::g_Nx : (u64)ocl::g_Nx*ocl::g_Ny;
	launch(A, [&]() { ocl::voxelize_mesh(direction, (ocl::ddf_t*)fi, u, flags, t, flag, p0, p1, p2, bbu); });
}

void ref_unvoxelize_mesh(u8* flags, const u8 flag, const float x0, const float y0, const float z0, const float x1, const float y1, const float z1) {
	// the reference kernel has no n<N guard (src/kernel.cpp:2359-2363); the launch stays inside N here
	launch(ocl::g_N, [&]() { ocl::unvoxelize_mesh(flags, flag, x0, y0, z0, x1, y1, z1); });
}

} // extern "C"
