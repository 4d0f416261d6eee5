// Ray-parity mesh voxelization (src/kernel.cpp:2267-2357 voxelize_mesh).
//
// One thread per ray through the lattice along the chosen axis. Every thread tests the ray against
// all triangles (Moeller-Trumbore, the reference's f = 1/g form), keeps up to 64 hit distances as
// 16-bit integers, insertion-sorts them and walks the column flipping inside/outside, with the
// reference's two-ray parity error correction. The triangle loop reads each triangle at the same
// address across the warp (one broadcast transaction) and the whole mesh stays L2-resident.
// FP32 without contraction (-fmad=false) and IEEE division: the flags are bit-identical to the FP32
// CPU restatement of the same algorithm.
#include "lbm_internal.h"
#include "lbm_scheme.cuh"

namespace fx3d {

struct V3 { float x, y, z; };
__device__ __forceinline__ V3 vsub(const V3 a, const V3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 vadd(const V3 a, const V3 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 vcross(const V3 a, const V3 b) {
	return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)), __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ float vdot(const V3 a, const V3 b) { return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)); }
// position(xyz)+offset of the reference with zero domain offset
__device__ __forceinline__ V3 cell_point(const Grid& g, const uint32_t x, const uint32_t y, const uint32_t z) {
	const V3 p = {__fsub_rn(__fadd_rn((float)x, 0.5f), __fmul_rn(0.5f, (float)g.Nx)), __fsub_rn(__fadd_rn((float)y, 0.5f), __fmul_rn(0.5f, (float)g.Ny)),
	              __fsub_rn(__fadd_rn((float)z, 0.5f), __fmul_rn(0.5f, (float)g.Nz))};
	const V3 o = {__fsub_rn(__fmul_rn(0.5f, (float)(int)g.Nx), 0.5f), __fsub_rn(__fmul_rn(0.5f, (float)(int)g.Ny), 0.5f), __fsub_rn(__fmul_rn(0.5f, (float)(int)g.Nz), 0.5f)};
	return vadd(p, o);
}
__device__ __forceinline__ int clampi(const int x, const int a, const int b) { return x<a ? a : x>b ? b : x; }

template<int Q, int ST> __global__ void __launch_bounds__(BLOCK) k_voxelize(const GridDesc gd, const uint32_t direction, void* fi, float* __restrict__ u,
                                                                           uint8_t* __restrict__ flags, const uint64_t t, const uint8_t flag,
                                                                           const float* __restrict__ p0, const float* __restrict__ p1, const float* __restrict__ p2,
                                                                           const float* __restrict__ bbu) {
	typedef typename Codec<ST>::T T;
	const Grid& g = reinterpret_cast<const Grid&>(gd);
	const uint32_t Nx = g.Nx, Ny = g.Ny, Nz = g.Nz;
	const uint64_t A = direction==0u ? (uint64_t)Ny*Nz : direction==1u ? (uint64_t)Nz*Nx : (uint64_t)Nx*Ny;
	const uint64_t ai = (uint64_t)blockIdx.x*BLOCK+threadIdx.x;
	if(ai>=A) return;
	const uint32_t a = (uint32_t)ai;
	const uint32_t triangle_number = __float_as_uint(bbu[0]);
	const float x0 = bbu[1], y0 = bbu[2], z0 = bbu[3], x1 = bbu[4], y1 = bbu[5], z1 = bbu[6];
	const float cx = bbu[7], cy = bbu[8], cz = bbu[9], ux = bbu[10], uy = bbu[11], uz = bbu[12], rx = bbu[13], ry = bbu[14], rz = bbu[15];
	const uint32_t hmin = direction==0u ? (uint32_t)clampi((int)x0, 0, (int)Nx-1) : direction==1u ? (uint32_t)clampi((int)y0, 0, (int)Ny-1) : (uint32_t)clampi((int)z0, 0, (int)Nz-1);
	const uint32_t hmax = direction==0u ? (uint32_t)clampi((int)x1, 0, (int)Nx-1) : direction==1u ? (uint32_t)clampi((int)y1, 0, (int)Ny-1) : (uint32_t)clampi((int)z1, 0, (int)Nz-1);
	uint32_t X, Y, Z;
	if(direction==0u) { X = hmin; Y = a%Ny; Z = a/Ny; }
	else if(direction==1u) { X = a/Nz; Y = hmin; Z = a%Nz; }
	else { X = a%Nx; Y = a/Nx; Z = hmin; }
	const V3 o = cell_point(g, X, Y, Z);
	const V3 r_dir = {(float)(direction==0u), (float)(direction==1u), (float)(direction==2u)};
	const bool outside = direction==0u ? o.y<y0||o.z<z0||o.y>=y1||o.z>=z1 : direction==1u ? o.x<x0||o.z<z0||o.x>=x1||o.z>=z1 : o.x<x0||o.y<y0||o.x>=x1||o.y>=y1;
	if(outside) return;
	uint32_t intersections = 0u, intersections_check = 0u;
	uint16_t distances[64];
	#pragma unroll
	for(int i=0; i<64; i++) distances[i] = 0u;
	for(uint32_t i=0u; i<triangle_number; i++) {
		const uint32_t tx = 3u*i;
		const V3 a0 = {__ldg(p0+tx), __ldg(p0+tx+1u), __ldg(p0+tx+2u)}, a1 = {__ldg(p1+tx), __ldg(p1+tx+1u), __ldg(p1+tx+2u)}, a2 = {__ldg(p2+tx), __ldg(p2+tx+1u), __ldg(p2+tx+2u)};
		const V3 eu = vsub(a1, a0), ev = vsub(a2, a0), ew = vsub(o, a0), h = vcross(r_dir, ev), qv = vcross(ew, eu);
		const float gg = vdot(eu, h), f = __fdiv_rn(1.0f, gg), s = __fmul_rn(f, vdot(ew, h)), tt = __fmul_rn(f, vdot(r_dir, qv)), d = __fmul_rn(f, vdot(ev, qv));
		if(gg!=0.0f&&s>=0.0f&&s<1.0f&&tt>=0.0f&&__fadd_rn(s, tt)<1.0f) {
			if(d>0.0f) {
				if(intersections<64u&&d<65536.0f) distances[intersections] = (uint16_t)d;
				intersections++;
			} else {
				intersections_check++;
			}
		}
	}
	const uint32_t nsort = intersections<64u ? intersections : 64u;
	for(uint32_t i=1u; i<nsort; i++) { // insertion sort
		const uint16_t tv = distances[i];
		uint32_t k = i;
		while(k>0u&&distances[k-1u]>tv) { distances[k] = distances[k-1u]; k--; }
		distances[k] = tv;
	}
	bool inside = (intersections%2u)&&(intersections_check%2u);
	uint32_t intersection = (intersections%2u)!=(intersections_check%2u);
	const bool set_u = __fmul_rn(ux, ux)+__fmul_rn(uy, uy)+__fmul_rn(uz, uz)+__fmul_rn(rx, rx)+__fmul_rn(ry, ry)+__fmul_rn(rz, rz)>0.0f;
	const uint32_t h0 = direction==0u ? X : direction==1u ? Y : Z;
	const uint32_t last = intersections-1u<63u ? intersections-1u : 63u;
	const uint32_t hmesh = h0+(uint32_t)distances[last];
	const uint64_t N = g.N;
	for(uint32_t hh=h0; hh<=hmax; hh++) {
		while(intersection<intersections&&hh>h0+(uint32_t)distances[intersection<63u ? intersection : 63u]) { inside = !inside; intersection++; }
		inside = inside&&(intersection<intersections&&hh<hmesh);
		const uint32_t xx = direction==0u ? hh : X, yy = direction==1u ? hh : Y, zz = direction==2u ? hh : Z;
		const uint64_t n = (uint64_t)xx+((uint64_t)yy+(uint64_t)zz*Ny)*(uint64_t)Nx;
		uint8_t flagsn = flags[n];
		const V3 p = cell_point(g, xx, yy, zz);
		const V3 rc = vcross(vsub({cx, cy, cz}, p), {rx, ry, rz});
		const V3 u_set = vadd({ux, uy, uz}, rc);
		if(inside) {
			flagsn = (uint8_t)((flagsn&~TYPE_BO)|flag);
			if(set_u) { u[n] = u_set.x; u[N+n] = u_set.y; u[2ull*N+n] = u_set.z; }
		} else if((flagsn&TYPE_BO)==TYPE_S&&(flagsn&TYPE_XY)==(flag&TYPE_XY)) { // previously solid from this geometry
			const V3 un = {u[n], u[N+n], u[2ull*N+n]};
			if(un.x==u_set.x&&un.y==u_set.y&&un.z==u_set.z) {
				if(set_u) { // solid -> fluid: equilibrium DDFs at rho=1 and the solid's velocity
					const EqState es = eq_state(1.0f, un.x, un.y, un.z);
					float fe[Q];
					fe[0] = feq0<Q>(es);
					Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; feq_pair<Q, i>(es, fe[i], fe[i+1]); });
					const Nbr nb(g, xx, yy, zz);
					store_f<Q, ST>((T*)fi, N, n, nb, (t&1ull)!=0ull, fe);
				}
				flagsn = (flagsn&TYPE_BO)==TYPE_MS ? (uint8_t)(flagsn&~TYPE_MS) : (uint8_t)(flagsn&~flag);
			}
		}
		flags[n] = flagsn;
	}
}

cudaError_t launch_voxelize(const Variant& v, const GridDesc& g, const uint32_t direction, void* fi, float* u, uint8_t* flags, const uint64_t t, const uint8_t flag,
                            const float* p0, const float* p1, const float* p2, const float* bbu, cudaStream_t s) {
	const uint64_t A = direction==0u ? (uint64_t)g.Ny*g.Nz : direction==1u ? (uint64_t)g.Nz*g.Nx : (uint64_t)g.Nx*g.Ny;
	const dim3 grid((unsigned)((A+BLOCK-1u)/BLOCK));
	#define FX3D_VOX(Q, ST) k_voxelize<Q, ST><<<grid, BLOCK, 0, s>>>(g, direction, fi, u, flags, t, flag, p0, p1, p2, bbu)
	if(v.q==19) {
		if(v.storage==ST_FP32) FX3D_VOX(19, ST_FP32); else if(v.storage==ST_FP16S) FX3D_VOX(19, ST_FP16S); else FX3D_VOX(19, ST_FP16C);
	} else {
		if(v.storage==ST_FP32) FX3D_VOX(27, ST_FP32); else if(v.storage==ST_FP16S) FX3D_VOX(27, ST_FP16S); else FX3D_VOX(27, ST_FP16C);
	}
	#undef FX3D_VOX
	return cudaGetLastError();
}

} // namespace fx3d
