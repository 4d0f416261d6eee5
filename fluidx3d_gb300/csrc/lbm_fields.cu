// Storage-independent kernels: object reductions in FP64 and mesh unvoxelization.
//
//   k_object_sum + k_object_sum_final  src/kernel.cpp:1901-1959 object_center_of_mass/force/torque
//   k_unvoxelize                       src/kernel.cpp:2359-2363 unvoxelize_mesh
//   k_update_moving_boundaries         src/kernel.cpp:1431-1450 update_moving_boundaries
//   k_pack_vtk                         src/lbm.hpp:298-340 write_vtk (unit scaling, AoS, big-endian)
//
// The reference reduces 64-cell work-groups in local memory and adds the group sums into 4 floats
// with float atomics, so its result depends on scheduling. Here each of REDUCE_BLOCKS blocks
// accumulates a fixed, strided subset of cells in FP64 (warp shuffles, then shared memory) into its
// own slot of a partials buffer, and one block adds the partials in a fixed order: the sum is FP64
// and bit-reproducible from run to run.
#include <mutex>
#include "lbm_internal.h"
#include "lbm_scheme.cuh"

namespace fx3d {

constexpr int RB = 256; // threads per reduction block

RowPlan row_plan(const int q, const int storage, const uint32_t Nx, const uint32_t Ny, const uint32_t Nz) {
	RowPlan p{0u, 0u, 0u};
	const size_t elem = storage==ST_FP32 ? 4u : 2u;
	if(Nx%16u!=0u) return p; // bulk copies move whole 16-byte units (the flags row is Nx bytes)
	if((uint64_t)Ny*Nz>0xFFFFFFFFull) return p;
	const size_t stride = (Nx*elem+127u)&~(size_t)127u;
	const size_t stage = (size_t)q*stride+((Nx+127u)&~(size_t)127u);
	const size_t budget2 = 112u*1024u, budget1 = 224u*1024u; // two CTAs per SM, or one
	uint32_t s = 0u;
	for(uint32_t k=4u; k>=2u && s==0u; k--) if(k*stage+128u<=budget2) s = k;
	for(uint32_t k=4u; k>=2u && s==0u; k--) if(k*stage+128u<=budget1) s = k;
	if(s==0u) return p;
	p.stage_bytes = (uint32_t)stage; p.stages = s; p.smem = s*stage+128u;
	return p;
}

int persistent_grid(const void* kernel, const int threads, const size_t smem) {
	struct Entry { const void* k; int threads; size_t smem; int dev; int grid; };
	static Entry cache[64];
	static int count = 0;
	static std::mutex m;
	int dev = 0;
	cudaGetDevice(&dev);
	std::lock_guard<std::mutex> lock(m);
	for(int i=0; i<count; i++) if(cache[i].k==kernel&&cache[i].threads==threads&&cache[i].smem==smem&&cache[i].dev==dev) return cache[i].grid;
	int sms = 0, per_sm = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
	const int grid = sms*(per_sm>0 ? per_sm : 1);
	if(count<64) cache[count++] = Entry{kernel, threads, smem, dev, grid};
	return grid;
}

__device__ __forceinline__ double warp_sum(double v) {
	#pragma unroll
	for(int o=16; o>0; o>>=1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
	return v;
}

// block sum of 4 values into out[0..3] (thread 0 writes); fixed reduction order
__device__ __forceinline__ void block_sum4(double v[4], double* out) {
	__shared__ double sm[RB/32][4];
	const int lane = threadIdx.x&31, warp = threadIdx.x>>5;
	#pragma unroll
	for(int k=0; k<4; k++) v[k] = warp_sum(v[k]);
	if(lane==0) { for(int k=0; k<4; k++) sm[warp][k] = v[k]; }
	__syncthreads();
	if(warp==0) {
		#pragma unroll
		for(int k=0; k<4; k++) {
			double s = lane<RB/32 ? sm[lane][k] : 0.0;
			s = warp_sum(s);
			if(lane==0) out[k] = s;
		}
	}
}

__global__ void __launch_bounds__(RB) k_object_sum(const GridDesc g, const float* __restrict__ F, const uint8_t* __restrict__ flags, const uint8_t marker,
                                                   const int kind, const double cx, const double cy, const double cz, double* __restrict__ partials) {
	double v[4] = {0.0, 0.0, 0.0, 0.0};
	const uint64_t N = g.N, stride = (uint64_t)gridDim.x*RB;
	for(uint64_t n=(uint64_t)blockIdx.x*RB+threadIdx.x; n<N; n+=stride) {
		if(flags[n]!=marker) continue;
		if(kind==1) { v[0] += (double)F[n]; v[1] += (double)F[N+n]; v[2] += (double)F[2ull*N+n]; continue; }
		const uint64_t z = n/g.NxNy;
		const uint32_t xy = (uint32_t)(n-z*g.NxNy);
		const uint32_t y = xy/g.Nx, x = xy-y*g.Nx;
		// cell position in box-centred coordinates, FP32 as the reference's position() (src/kernel.cpp:827-829)
		const double px = (double)__fsub_rn(__fadd_rn((float)x, 0.5f), __fmul_rn(0.5f, (float)g.Nx));
		const double py = (double)__fsub_rn(__fadd_rn((float)y, 0.5f), __fmul_rn(0.5f, (float)g.Ny));
		const double pz = (double)__fsub_rn(__fadd_rn((float)z, 0.5f), __fmul_rn(0.5f, (float)g.Nz));
		if(kind==0) { v[0] += px; v[1] += py; v[2] += pz; v[3] += 1.0; }
		else {
			const double Fx = F[n], Fy = F[N+n], Fz = F[2ull*N+n];
			const double rx = px-cx, ry = py-cy, rz = pz-cz;
			v[0] += ry*Fz-rz*Fy; v[1] += rz*Fx-rx*Fz; v[2] += rx*Fy-ry*Fx;
		}
	}
	block_sum4(v, partials+4ull*blockIdx.x);
}

__global__ void __launch_bounds__(RB) k_object_sum_final(const double* __restrict__ partials, const int blocks, double* __restrict__ out) {
	double v[4] = {0.0, 0.0, 0.0, 0.0};
	for(int b=threadIdx.x; b<blocks; b+=RB) {
		#pragma unroll
		for(int k=0; k<4; k++) v[k] += partials[4*b+k];
	}
	block_sum4(v, out);
}

cudaError_t launch_object_sum(const GridDesc& g, const float* F, const uint8_t* flags, const uint8_t marker, const int kind,
                              const double cx, const double cy, const double cz, double* partials, double* out, cudaStream_t s) {
	k_object_sum<<<REDUCE_BLOCKS, RB, 0, s>>>(g, F, flags, marker, kind, cx, cy, cz, partials);
	k_object_sum_final<<<1, RB, 0, s>>>(partials, REDUCE_BLOCKS, out);
	return cudaGetLastError();
}
cudaError_t launch_object_sum_blocks(const GridDesc& g, const float* F, const uint8_t* flags, const uint8_t marker, const int kind,
                                     const double cx, const double cy, const double cz, const int blocks, double* partials, double* out, cudaStream_t s) {
	if(blocks<1) return cudaErrorInvalidValue;
	k_object_sum<<<blocks, RB, 0, s>>>(g, F, flags, marker, kind, cx, cy, cz, partials);
	k_object_sum_final<<<1, RB, 0, s>>>(partials, blocks, out);
	return cudaGetLastError();
}

// box[6] = x0,y0,z0,x1,y1,z1 (mesh bounds); cells within +-1 lose `flag`
__global__ void __launch_bounds__(BLOCK) k_unvoxelize(const GridDesc g, uint8_t* __restrict__ flags, const uint8_t flag,
                                                      const float x0, const float y0, const float z0, const float x1, const float y1, const float z1) {
	const uint32_t xy = blockIdx.x*(uint32_t)BLOCK+threadIdx.x;
	if(xy>=g.NxNy) return;
	const uint32_t z = blockIdx.y, y = xy/g.Nx, x = xy-y*g.Nx;
	const uint64_t n = (uint64_t)z*g.NxNy+xy;
	// position()+offset of src/kernel.cpp:2361 with zero domain offset
	const float px = __fadd_rn(__fsub_rn(__fadd_rn((float)x, 0.5f), __fmul_rn(0.5f, (float)g.Nx)), __fsub_rn(__fmul_rn(0.5f, (float)(int)g.Nx), 0.5f));
	const float py = __fadd_rn(__fsub_rn(__fadd_rn((float)y, 0.5f), __fmul_rn(0.5f, (float)g.Ny)), __fsub_rn(__fmul_rn(0.5f, (float)(int)g.Ny), 0.5f));
	const float pz = __fadd_rn(__fsub_rn(__fadd_rn((float)z, 0.5f), __fmul_rn(0.5f, (float)g.Nz)), __fsub_rn(__fmul_rn(0.5f, (float)(int)g.Nz), 0.5f));
	if(px>=x0-1.0f&&py>=y0-1.0f&&pz>=z0-1.0f&&px<=x1+1.0f&&py<=y1+1.0f&&pz<=z1+1.0f) flags[n] &= (uint8_t)~flag;
}

cudaError_t launch_unvoxelize(const GridDesc& g, uint8_t* flags, const uint8_t flag, const float* box, cudaStream_t s) {
	const dim3 grid((g.NxNy+BLOCK-1u)/BLOCK, g.Nz, 1u);
	k_unvoxelize<<<grid, BLOCK, 0, s>>>(g, flags, flag, box[0], box[1], box[2], box[3], box[4], box[5]);
	return cudaGetLastError();
}

// TYPE_MS set on cells (not TYPE_S, TYPE_E or TYPE_T) with a TYPE_S neighbour whose velocity is not
// zero, cleared on the others. A neighbour's flags are read only through the TYPE_S test, whose bit
// pattern the marking never produces or removes (00 <-> 11): the result is independent of the order
// in which the cells are marked.
template<int Q> __global__ void __launch_bounds__(BLOCK) k_update_moving_boundaries(const GridDesc gd, const float* __restrict__ u, uint8_t* flags) {
	const Grid& g = reinterpret_cast<const Grid&>(gd);
	const uint32_t xy = blockIdx.x*(uint32_t)BLOCK+threadIdx.x;
	if(xy>=g.NxNy) return;
	const uint32_t z = blockIdx.y, y = div_nx(g, xy), x = xy-y*g.Nx;
	const uint64_t n = (uint64_t)z*g.NxNy+xy, N = g.N;
	const uint8_t flagsn = flags[n], flagsn_bo = flagsn&TYPE_BO;
	if(flagsn_bo==TYPE_S||flagsn_bo==TYPE_E||(flagsn&TYPE_T)) return;
	const Nbr nb(g, x, y, z);
	bool next = false;
	Unroll<1, Q, 1>::run([&](auto ic) {
		const uint64_t j = nb.template j<decltype(ic)::value>();
		next = next||((flags[j]&TYPE_BO)==TYPE_S&&(u[j]!=0.0f||u[N+j]!=0.0f||u[2ull*N+j]!=0.0f));
	});
	flags[n] = next ? (uint8_t)(flagsn|TYPE_MS) : (uint8_t)(flagsn&~TYPE_MS);
}

// VTK export: values [first, first+count) of a field of `dims` FP32 components stored in SoA blocks
// of N, each multiplied by `scale` (the reference's unit conversion, one FP32 multiply), written
// interleaved per cell (x,y,z) and byte-reversed to big-endian, as the legacy VTK binary format wants
__global__ void __launch_bounds__(BLOCK) k_pack_vtk(const float* __restrict__ src, const uint64_t N, const uint32_t dims, const uint64_t first,
                                                    const uint64_t count, const float scale, uint32_t* __restrict__ dst) {
	const uint64_t total = count*dims;
	for(uint64_t k=(uint64_t)blockIdx.x*BLOCK+threadIdx.x; k<total; k+=(uint64_t)gridDim.x*BLOCK) {
		const uint64_t i = k/dims;
		const uint32_t c = (uint32_t)(k-i*dims);
		const float v = __fmul_rn(scale, src[(uint64_t)c*N+first+i]);
		dst[k] = __byte_perm(__float_as_uint(v), 0u, 0x0123u);
	}
}

cudaError_t launch_pack_vtk(const float* src, const uint64_t N, const uint32_t dims, const uint64_t first, const uint64_t count, const float scale,
                            uint32_t* dst, cudaStream_t s) {
	const uint64_t total = count*dims;
	if(total==0ull) return cudaSuccess;
	const uint64_t blocks = (total+BLOCK-1u)/BLOCK;
	k_pack_vtk<<<(unsigned)(blocks<4864ull ? blocks : 4864ull), BLOCK, 0, s>>>(src, N, dims, first, count, scale, dst); // 152 SMs x 32
	return cudaGetLastError();
}

cudaError_t launch_update_moving_boundaries(const int q, const GridDesc& g, const float* u, uint8_t* flags, cudaStream_t s) {
	static_assert(sizeof(GridDesc)==sizeof(Grid), "GridDesc must mirror Grid");
	const dim3 grid((g.NxNy+BLOCK-1u)/BLOCK, g.Nz, 1u);
	if(q==19) k_update_moving_boundaries<19><<<grid, BLOCK, 0, s>>>(g, u, flags);
	else if(q==27) k_update_moving_boundaries<27><<<grid, BLOCK, 0, s>>>(g, u, flags);
	else return cudaErrorInvalidValue;
	return cudaGetLastError();
}

} // namespace fx3d
