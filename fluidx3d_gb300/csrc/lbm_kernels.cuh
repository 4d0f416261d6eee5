// Per-cell LBM kernels (one thread per cell, plane-major launch: blockIdx.y = z, threads cover the
// x-fastest cells of one plane) and their variant dispatch. Included once per DDF storage format by
// lbm_kernels_<storage>.cu, so the three storage formats compile in parallel.
//
// Kernels and the reference functions they replace:
//   k_initialize          src/kernel.cpp:1358-1430 initialize
//   k_stream_collide      src/kernel.cpp:1454-1636 stream_collide
//   k_update_fields       src/kernel.cpp:1794-1870 update_fields
//   k_update_force_field  src/kernel.cpp:1873-1884 update_force_field
#pragma once
#include "lbm_scheme.cuh"
#include "lbm_internal.h"
#include "lbm_bulk.cuh"
#include "lbm_fast.cuh"

namespace fx3d {

static_assert(sizeof(GridDesc)==sizeof(Grid), "GridDesc must mirror Grid");
__device__ __forceinline__ const Grid& grid_of(const GridDesc& g) { return reinterpret_cast<const Grid&>(g); }

struct CellPos { uint32_t x, y, z; uint64_t n; };
// cell of this thread; false for the idle tail threads of a plane
__device__ __forceinline__ bool cell_of_thread(const Grid& g, CellPos& c) {
	const uint32_t xy = blockIdx.x*(uint32_t)BLOCK+threadIdx.x;
	if(xy>=g.NxNy) return false;
	c.z = blockIdx.y;
	c.y = div_nx(g, xy);
	c.x = xy-c.y*g.Nx;
	c.n = (uint64_t)c.z*g.NxNy+xy;
	return true;
}

template<int Q, int ST> __global__ void __launch_bounds__(BLOCK) k_initialize(const StepArgs a) {
	typedef typename Codec<ST>::T T;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n, N = g.N;
	float ux, uy, uz;
	if((a.flags[n]&TYPE_BO)==TYPE_S) { // solid cells start at rest (src/kernel.cpp:1370-1373)
		ux = uy = uz = 0.0f;
		a.u[n] = 0.0f; a.u[N+n] = 0.0f; a.u[2ull*N+n] = 0.0f;
	} else {
		ux = a.u[n]; uy = a.u[N+n]; uz = a.u[2ull*N+n];
	}
	const EqState s = eq_state(a.rho[n], ux, uy, uz);
	float f[Q];
	f[0] = feq0<Q>(s);
	Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; feq_pair<Q, i>(s, f[i], f[i+1]); });
	const Nbr nb(g, c.x, c.y, c.z);
	store_f<Q, ST>((T*)a.fi, N, n, nb, true, f); // odd parity (src/kernel.cpp:1429)
}

// density and velocity of one cell from its streamed DDFs (or the preset TYPE_E values), force
// shifted and clamped exactly as stream_collide / update_fields do
template<int Q, int EXT> __device__ __forceinline__ void cell_rho_u(const StepArgs& a, const uint64_t n, const float* f, const bool is_e,
                                                                    float& rho, float& ux, float& uy, float& uz, float& fx, float& fy, float& fz) {
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0;
	const uint64_t N = a.g.N;
	if(is_e) {
		rho = a.rho[n]; ux = a.u[n]; uy = a.u[N+n]; uz = a.u[2ull*N+n];
	} else {
		float mx, my, mz;
		moments<Q>(f, rho, mx, my, mz);
		ux = __fdiv_rn(mx, rho); uy = __fdiv_rn(my, rho); uz = __fdiv_rn(mz, rho);
	}
	fx = a.fx; fy = a.fy; fz = a.fz;
	if constexpr(FF) { fx = __fadd_rn(fx, a.F[n]); fy = __fadd_rn(fy, a.F[N+n]); fz = __fadd_rn(fz, a.F[2ull*N+n]); }
	shift_clamp<VF>(ux, uy, uz, rho, fx, fy, fz);
}

// one cell step on registers: f in, f out (exact: real units; fast: storage units)
template<int Q, int ST, bool TRT, int EXT, bool FAST> __device__ __forceinline__ void cell_step(float* f, const StepArgs& a, const uint64_t n, const bool is_e) {
	constexpr bool VF = (EXT&EXT_VF)!=0;
	float rho, ux, uy, uz, fx, fy, fz;
	if constexpr(FAST) {
		float rm1, inv;
		cell_rho_u_fast<Q, EXT, ST>(a, n, f, is_e, rho, rm1, inv, ux, uy, uz, fx, fy, fz);
		collide_fast<Q, TRT, VF, ST>(f, rho, rm1, ux, uy, uz, fx, fy, fz, is_e, a);
	} else {
		cell_rho_u<Q, EXT>(a, n, f, is_e, rho, ux, uy, uz, fx, fy, fz);
		collide<Q, TRT, VF>(f, rho, ux, uy, uz, fx, fy, fz, is_e, a);
	}
}
template<int ST, bool FAST> using StepCodec = typename std::conditional<FAST, RawCodec<ST>, Codec<ST>>::type;

template<int Q, int ST, bool TRT, int EXT, bool FAST> __global__ void __launch_bounds__(BLOCK) k_stream_collide(const StepArgs a) {
	typedef typename Codec<ST>::T T;
	constexpr bool EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n;
	const uint8_t flagsn = a.flags[n];
	const uint8_t flagsn_bo = flagsn&TYPE_BO;
	if(flagsn_bo==TYPE_S||(flagsn&TYPE_SU)==TYPE_G) return; // solid or gas: nothing to do
	const Nbr nb(g, c.x, c.y, c.z);
	const bool odd = (a.t&1ull)!=0ull;
	float f[Q];
	load_f<Q, ST, StepCodec<ST, FAST>>((const T*)a.fi, g.N, n, nb, odd, f);
	const bool is_e = EQ && flagsn_bo==TYPE_E;
	cell_step<Q, ST, TRT, EXT, FAST>(f, a, n, is_e);
	store_f<Q, ST, StepCodec<ST, FAST>>((T*)a.fi, g.N, n, nb, odd, f);
}

// Row-staged stream_collide. At either parity the cells of one x-row (y,z) own exactly Q whole
// rows of the DDF array: row (y,z) of array 0 and of the arrays of their "own" slots, and for each
// pair (i,i+1) row (y+c_iy, z+c_iz) of the array of their neighbour slots, rotated by c_ix
// (periodic in x). Rows are owned by exactly one x-row per parity, so x-rows never touch each
// other's DDF rows, and a whole x-row can be moved with Q aligned bulk copies.
//
// Persistent CTAs walk x-rows r = blockIdx.x + j*gridDim.x through a ring of `stages` shared-memory
// stages (one x-row's Q DDF rows + its flags row each): while x-row j is collided from shared memory,
// the bulk loads (cp.async.bulk, completion on the stage's mbarrier) of x-rows j+1..j+P are in flight
// and the bulk stores of x-row j-1 drain. Every global access is a whole 16-byte-aligned row and no
// data in flight occupies registers. Slots of solid cells go back unchanged, so the step may also
// write to a different array than it reads (fi_dst), which the adjoint's recomputation uses.
struct RowStageLayout {
	uint32_t rowbytes, stride, flags_off, stage_bytes;
	__host__ __device__ RowStageLayout(const int q, const uint32_t elem, const uint32_t Nx) {
		rowbytes = Nx*elem; stride = (rowbytes+127u)&~127u;
		flags_off = (uint32_t)q*stride; stage_bytes = flags_off+((Nx+127u)&~127u);
	}
};

// lattice velocities as a table the bulk-copy lanes index at run time
__constant__ int8_t c_vs_tab[3][27] = {
	{0, 1,-1, 0, 0, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1},
	{0, 0, 0, 1,-1, 0, 0, 1,-1, 0, 0, 1,-1,-1, 1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1, 1,-1},
	{0, 0, 0, 0, 0, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0,-1, 1,-1, 1, 1,-1,-1, 1, 1,-1, 1,-1}};

template<int Q, int ST, bool TRT, int EXT, bool FAST> __global__ void __launch_bounds__(ROW_TPB_MAX, (Q==19 ? 2 : 1))
k_stream_collide_rows(const StepArgs a, const uint32_t stages) {
	typedef typename Codec<ST>::T T;
	typedef StepCodec<ST, FAST> CD;
	constexpr bool EQ = (EXT&EXT_EQ)!=0;
	extern __shared__ __align__(128) unsigned char smem[];
	__shared__ int abort_rows;
	const Grid& g = grid_of(a.g);
	const uint32_t Nx = g.Nx, Ny = g.Ny, Nz = g.Nz, rows = Ny*Nz, tid = threadIdx.x;
	const RowStageLayout L(Q, (uint32_t)sizeof(T), Nx);
	uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
	unsigned char* stage0 = smem+128;
	const bool odd = (a.t&1ull)!=0ull;
	const uint64_t N = g.N;
	const T* src = (const T*)a.fi;
	T* dst = (T*)a.fi_dst;
	const uint32_t P = stages>2u ? stages-2u : 1u; // x-rows loaded ahead of the one being collided
	// bulk-copy lanes: lane k<Q of warp 0 moves DDF slot row k of every x-row, lane Q its flags row.
	// Slot row k of x-row (y,z) is row (y+dy, z+dz) of array karr: slot 0 and odd slots (own slots)
	// sit in the x-row itself, slot i+1 (i odd) in the neighbour row along c_i.
	const bool copier = tid<=(uint32_t)Q;
	uint32_t karr = 0u; int dy = 0, dz = 0;
	if(copier && tid<(uint32_t)Q && tid>0u) {
		const uint32_t k = tid;
		if(k%2u==1u) karr = odd ? k : k+1u;
		else { karr = odd ? k : k-1u; dy = c_vs_tab[1][k-1u]; dz = c_vs_tab[2][k-1u]; }
	}
	auto row_of = [&](const uint64_t r, uint32_t& y, uint32_t& z) { z = (uint32_t)(r/Ny); y = (uint32_t)(r-(uint64_t)z*Ny); };
	auto slot_row = [&](const uint32_t y, const uint32_t z) -> uint64_t { // global start of this lane's slot row
		const uint32_t yy = dy>0 ? (y+1u==Ny ? 0u : y+1u) : dy<0 ? (y==0u ? Ny-1u : y-1u) : y;
		const uint32_t zz = dz>0 ? (z+1u==Nz ? 0u : z+1u) : dz<0 ? (z==0u ? Nz-1u : z-1u) : z;
		return (uint64_t)karr*N+((uint64_t)zz*Ny+yy)*Nx;
	};
	auto issue_loads = [&](const uint64_t r, const uint32_t s) { // all lanes of warp 0
		uint32_t y, z; row_of(r, y, z);
		unsigned char* st = stage0+(size_t)s*L.stage_bytes;
		if(tid==0u) mbar_arrive_expect_tx(bars+s, (uint32_t)Q*L.rowbytes+Nx);
		__syncwarp();
		if(tid<(uint32_t)Q) bulk_load(st+(size_t)tid*L.stride, src+slot_row(y, z), L.rowbytes, bars+s);
		else if(tid==(uint32_t)Q) bulk_load(st+L.flags_off, a.flags+((uint64_t)z*Ny+y)*Nx, Nx, bars+s);
	};
	if(tid==0u) {
		for(uint32_t s=0u; s<stages; s++) mbar_init(bars+s, 1u);
		fence_mbar_init();
		abort_rows = 0;
	}
	__syncwarp();
	if(tid<32u) for(uint32_t p=0u; p<P; p++) { const uint64_t r = (uint64_t)blockIdx.x+(uint64_t)p*gridDim.x; if(r<rows) issue_loads(r, p); }
	__syncthreads();
	uint32_t j = 0u;
	for(uint64_t r=blockIdx.x; r<rows; r+=gridDim.x, j++) {
		const uint32_t s = j%stages;
		if(tid<32u) {
			const uint64_t rn = r+(uint64_t)P*gridDim.x;
			if(rn<rows) {
				// the stage of x-row j+P last held x-row j+P-stages: this lane's store of it must have left shared memory
				if(copier) { if(stages-P-1u>=1u) bulk_wait_read_but1(); else bulk_wait_read_all(); }
				issue_loads(rn, (j+P)%stages);
			}
		}
		const bool ok = mbar_wait_bounded(bars+s, (j/stages)&1u, a.err);
		if(!ok) abort_rows = 1;
		unsigned char* st = stage0+(size_t)s*L.stage_bytes;
		auto srow = [&](const int k) { return reinterpret_cast<T*>(st+(size_t)k*L.stride); };
		const uint8_t* fl = st+L.flags_off;
		uint32_t y, z; row_of(r, y, z);
		const uint64_t row0 = ((uint64_t)z*Ny+y)*Nx;
		for(uint32_t x=tid; ok && x<Nx; x+=blockDim.x) {
			const uint8_t flagsn = fl[x];
			const uint8_t flagsn_bo = flagsn&TYPE_BO;
			if(flagsn_bo==TYPE_S||(flagsn&TYPE_SU)==TYPE_G) continue;
			const uint32_t xp = x+1u==Nx ? 0u : x+1u, xm = x==0u ? Nx-1u : x-1u;
			float f[Q];
			f[0] = CD::decode(srow(0)[x]);
			Unroll<1, Q, 2>::run([&](auto ic) {
				constexpr int i = decltype(ic)::value, cx = vs_c(0, i);
				const uint32_t xi = cx>0 ? xp : cx<0 ? xm : x;
				f[i] = CD::decode(srow(i)[x]);
				f[i+1] = CD::decode(srow(i+1)[xi]);
			});
			const bool is_e = EQ && flagsn_bo==TYPE_E;
			cell_step<Q, ST, TRT, EXT, FAST>(f, a, row0+x, is_e);
			srow(0)[x] = CD::encode(f[0]);
			Unroll<1, Q, 2>::run([&](auto ic) {
				constexpr int i = decltype(ic)::value, cx = vs_c(0, i);
				const uint32_t xi = cx>0 ? xp : cx<0 ? xm : x;
				srow(i+1)[xi] = CD::encode(f[i]);
				srow(i)[x] = CD::encode(f[i+1]);
			});
		}
		fence_proxy_async_smem();
		__syncthreads();
		if(abort_rows) { // a bounded wait ran out: store nothing more, drain the copies still in flight
			if(tid==0u) {
				for(uint32_t p=0u; p<=P; p++) {
					const uint64_t rp = r+(uint64_t)p*gridDim.x;
					if(rp<rows) mbar_wait_bounded(bars+(j+p)%stages, ((j+p)/stages)&1u, nullptr);
				}
			}
			if(copier) bulk_wait_all();
			return;
		}
		if(tid<(uint32_t)Q) {
			bulk_store(dst+slot_row(y, z), st+(size_t)tid*L.stride, L.rowbytes);
			bulk_commit();
		}
	}
	if(copier) bulk_wait_all(); // stores complete before the CTA (and its shared memory) goes away
}

template<int Q, int ST, int EXT, bool FAST> __global__ void __launch_bounds__(BLOCK) k_update_fields(const StepArgs a) {
	typedef typename Codec<ST>::T T;
	constexpr bool EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n, N = g.N;
	const uint8_t flagsn = a.flags[n];
	const uint8_t flagsn_bo = flagsn&TYPE_BO;
	if(flagsn_bo==TYPE_S||(flagsn&TYPE_SU)==TYPE_G) return;
	if(EQ && flagsn_bo==TYPE_E) return; // preset rho/u of TYPE_E cells are kept
	const Nbr nb(g, c.x, c.y, c.z);
	float f[Q];
	load_f<Q, ST, StepCodec<ST, FAST>>((const T*)a.fi, N, n, nb, (a.t&1ull)!=0ull, f);
	float rho, ux, uy, uz, fx, fy, fz;
	if constexpr(FAST) {
		float rm1, inv;
		cell_rho_u_fast<Q, EXT&~EXT_EQ, ST>(a, n, f, false, rho, rm1, inv, ux, uy, uz, fx, fy, fz);
		rho *= 1.0f/RawCodec<ST>::K; // R = K*rho, K a power of two
	} else {
		cell_rho_u<Q, EXT&~EXT_EQ>(a, n, f, false, rho, ux, uy, uz, fx, fy, fz);
	}
	a.rho[n] = rho; a.u[n] = ux; a.u[N+n] = uy; a.u[2ull*N+n] = uz;
}

// momentum exchange on TYPE_S cells: F = 2*rho*(m/rho) (the reference reuses calculate_rho_u)
template<int Q, int ST> __global__ void __launch_bounds__(BLOCK) k_update_force_field(const StepArgs a, float* F) {
	typedef typename Codec<ST>::T T;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n, N = g.N;
	if((a.flags[n]&TYPE_BO)!=TYPE_S) return;
	const Nbr nb(g, c.x, c.y, c.z);
	float f[Q];
	load_f<Q, ST>((const T*)a.fi, N, n, nb, (a.t&1ull)!=0ull, f);
	float rho, mx, my, mz;
	moments<Q>(f, rho, mx, my, mz);
	const float s = __fmul_rn(2.0f, rho);
	F[n] = __fmul_rn(s, __fdiv_rn(mx, rho)); F[N+n] = __fmul_rn(s, __fdiv_rn(my, rho)); F[2ull*N+n] = __fmul_rn(s, __fdiv_rn(mz, rho));
}

// ---------------------------------------------------------------- dispatch
inline dim3 cell_grid(const GridDesc& g) { return dim3((g.NxNy+BLOCK-1u)/BLOCK, g.Nz, 1u); }

template<int ST, int Q, bool TRT, int EXT, bool FAST> inline cudaError_t sc_launch_t(const StepArgs& a, const bool rows, cudaStream_t s) {
	if(rows) {
		const RowPlan plan = row_plan(Q, ST, a.g.Nx, a.g.Ny, a.g.Nz);
		if(plan.stages==0u) return cudaErrorInvalidConfiguration;
		auto kernel = k_stream_collide_rows<Q, ST, TRT, EXT, FAST>;
		if(plan.smem>48u*1024u) { // opt in to more than 48 KB of dynamic shared memory (per device, so on every such launch)
			const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem);
			if(e!=cudaSuccess) return e;
		}
		const int tpb = a.g.Nx>=(uint32_t)ROW_TPB_MAX ? ROW_TPB_MAX : (int)((a.g.Nx+31u)&~31u);
		const uint64_t rows_total = (uint64_t)a.g.Ny*a.g.Nz;
		int grid = persistent_grid((const void*)kernel, tpb, plan.smem);
		if((uint64_t)grid>rows_total) grid = (int)rows_total;
		kernel<<<grid, tpb, plan.smem, s>>>(a, plan.stages);
	} else {
		if(a.fi_dst!=a.fi) return cudaErrorInvalidValue; // one thread per cell steps in place only
		k_stream_collide<Q, ST, TRT, EXT, FAST><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
	}
	return cudaGetLastError();
}
template<int ST, int Q, bool TRT, int EXT> inline cudaError_t sc_launch(const StepArgs& a, const bool rows, const bool fast, cudaStream_t s) {
	return fast ? sc_launch_t<ST, Q, TRT, EXT, true>(a, rows, s) : sc_launch_t<ST, Q, TRT, EXT, false>(a, rows, s);
}
template<int ST, int Q, bool TRT> inline cudaError_t sc_ext(const int ext, const StepArgs& a, const bool rows, const bool fast, cudaStream_t s) {
	switch(ext) {
		case 0:                        return sc_launch<ST, Q, TRT, 0>(a, rows, fast, s);
		case EXT_VF:                   return sc_launch<ST, Q, TRT, EXT_VF>(a, rows, fast, s);
		case EXT_VF|EXT_FF:            return sc_launch<ST, Q, TRT, EXT_VF|EXT_FF>(a, rows, fast, s);
		case EXT_EQ:                   return sc_launch<ST, Q, TRT, EXT_EQ>(a, rows, fast, s);
		case EXT_EQ|EXT_VF:            return sc_launch<ST, Q, TRT, EXT_EQ|EXT_VF>(a, rows, fast, s);
		case EXT_EQ|EXT_VF|EXT_FF:     return sc_launch<ST, Q, TRT, EXT_EQ|EXT_VF|EXT_FF>(a, rows, fast, s);
		default: return cudaErrorInvalidValue;
	}
}
template<int ST> cudaError_t launch_stream_collide_t(const Variant& v, const StepArgs& a, const int path, cudaStream_t s) {
	const bool rows_ok = row_plan(v.q, ST, a.g.Nx, a.g.Ny, a.g.Nz).stages!=0u;
	if(path==PATH_ROWS && !rows_ok) return cudaErrorInvalidConfiguration;
	const bool rows = path==PATH_ROWS || (path==PATH_AUTO && rows_ok);
	if(v.q==19) return v.trt ? sc_ext<ST, 19, true>(v.ext, a, rows, v.fast, s) : sc_ext<ST, 19, false>(v.ext, a, rows, v.fast, s);
	if(v.q==27) return v.trt ? sc_ext<ST, 27, true>(v.ext, a, rows, v.fast, s) : sc_ext<ST, 27, false>(v.ext, a, rows, v.fast, s);
	return cudaErrorInvalidValue;
}

template<int ST, int Q, int EXT> inline void uf_launch(const StepArgs& a, const bool fast, cudaStream_t s) {
	if(fast) k_update_fields<Q, ST, EXT, true><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
	else k_update_fields<Q, ST, EXT, false><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
}
template<int ST, int Q> inline bool uf_ext(const int ext, const StepArgs& a, const bool fast, cudaStream_t s) {
	switch(ext) {
		case 0:                        uf_launch<ST, Q, 0>(a, fast, s); return true;
		case EXT_VF:                   uf_launch<ST, Q, EXT_VF>(a, fast, s); return true;
		case EXT_VF|EXT_FF:            uf_launch<ST, Q, EXT_VF|EXT_FF>(a, fast, s); return true;
		case EXT_EQ:                   uf_launch<ST, Q, EXT_EQ>(a, fast, s); return true;
		case EXT_EQ|EXT_VF:            uf_launch<ST, Q, EXT_EQ|EXT_VF>(a, fast, s); return true;
		case EXT_EQ|EXT_VF|EXT_FF:     uf_launch<ST, Q, EXT_EQ|EXT_VF|EXT_FF>(a, fast, s); return true;
		default: return false;
	}
}
template<int ST> cudaError_t launch_update_fields_t(const Variant& v, const StepArgs& a, cudaStream_t s) {
	const bool ok = v.q==19 ? uf_ext<ST, 19>(v.ext, a, v.fast, s) : v.q==27 ? uf_ext<ST, 27>(v.ext, a, v.fast, s) : false;
	return ok ? cudaGetLastError() : cudaErrorInvalidValue;
}

template<int ST> cudaError_t launch_initialize_t(const Variant& v, const StepArgs& a, cudaStream_t s) {
	if(v.q==19) k_initialize<19, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
	else if(v.q==27) k_initialize<27, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
	else return cudaErrorInvalidValue;
	return cudaGetLastError();
}
template<int ST> cudaError_t launch_update_force_field_t(const Variant& v, const StepArgs& a, float* F, cudaStream_t s) {
	if(v.q==19) k_update_force_field<19, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a, F);
	else if(v.q==27) k_update_force_field<27, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a, F);
	else return cudaErrorInvalidValue;
	return cudaGetLastError();
}

} // namespace fx3d

#define FX3D_DEFINE_LAUNCHERS(sfx, ST) \
	namespace fx3d { \
	cudaError_t launch_initialize_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s) { return launch_initialize_t<ST>(v, a, s); } \
	cudaError_t launch_stream_collide_##sfx(const Variant& v, const StepArgs& a, const int path, cudaStream_t s) { return launch_stream_collide_t<ST>(v, a, path, s); } \
	cudaError_t launch_update_fields_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s) { return launch_update_fields_t<ST>(v, a, s); } \
	cudaError_t launch_update_force_field_##sfx(const Variant& v, const StepArgs& a, float* F, cudaStream_t s) { return launch_update_force_field_t<ST>(v, a, F, s); } \
	}
