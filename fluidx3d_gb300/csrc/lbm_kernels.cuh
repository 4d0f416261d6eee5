// Per-cell LBM kernels (one thread per cell, plane-major launch: blockIdx.y = z, threads cover the
// x-fastest cells of one plane) and their variant dispatch. Included once per DDF storage format by
// lbm_kernels_<storage>.cu, so the three storage formats compile in parallel.
//
// Kernels and the reference functions they replace:
//   k_initialize          src/kernel.cpp:1358-1430 initialize
//   k_stream_collide      src/kernel.cpp:1454-1636 stream_collide
//   k_stream_collide_pairs  the same, two x-adjacent cells per thread (fast arithmetic)
//   k_update_fields       src/kernel.cpp:1794-1870 update_fields
//   k_update_force_field  src/kernel.cpp:1873-1884 update_force_field
// MOVING_BOUNDARIES (EXT_MB) adds apply_moving_boundaries (src/kernel.cpp:1104-1113) to
// stream_collide and update_fields and the TYPE_MS marking of initialize (src/kernel.cpp:1378-1387).
// UPDATE_FIELDS (StepArgs::fields_out, a run-time switch) makes stream_collide write rho/u
// (src/kernel.cpp:1565-1573), in every kernel through store_fields.
#pragma once
#include "lbm_scheme.cuh"
#include "lbm_internal.h"
#include "lbm_bulk.cuh"
#include "lbm_fast.cuh"
#include "lbm_index32.cuh"

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

// true if a neighbour of the cell is a TYPE_S cell with u != 0 (src/kernel.cpp:1381-1385, 1441-1447)
template<int Q, class J> __device__ __forceinline__ bool next_to_moving_boundary(const float* __restrict__ u, const uint8_t* flags, const uint64_t N, const J& nbr) {
	bool next = false;
	Unroll<1, Q, 1>::run([&](auto ic) {
		const uint64_t j = nbr(ic);
		next = next||((flags[j]&TYPE_BO)==TYPE_S&&(u[j]!=0.0f||u[N+j]!=0.0f||u[2ull*N+j]!=0.0f));
	});
	return next;
}

// mb: MOVING_BOUNDARIES, where solid cells keep their (wall) velocity unless all their neighbours are
// solid, and the other cells but TYPE_E get TYPE_MS set or cleared. The flags a cell writes are read
// by its neighbours only through the TYPE_S test, whose bit pattern the marking never produces or
// removes (00 <-> 11), so the result does not depend on the order the cells run in.
template<int Q, int ST> __global__ void __launch_bounds__(BLOCK) k_initialize(const StepArgs a, uint8_t* flags, const bool mb) {
	typedef typename Codec<ST>::T T;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n, N = g.N;
	const Nbr nb(g, c.x, c.y, c.z);
	const uint8_t flagsn = flags[n], flagsn_bo = flagsn&TYPE_BO;
	float ux, uy, uz;
	bool rest = flagsn_bo==TYPE_S; // solid cells start at rest (src/kernel.cpp:1370-1377)
	if(mb && rest) {
		Unroll<1, Q, 1>::run([&](auto ic) { rest = rest&&(flags[nb.template j<decltype(ic)::value>()]&TYPE_BO)==TYPE_S; });
	} else if(mb && flagsn_bo!=TYPE_E) {
		const bool next = next_to_moving_boundary<Q>(a.u, flags, N, [&](auto ic) { return nb.template j<decltype(ic)::value>(); });
		flags[n] = next ? (uint8_t)(flagsn|TYPE_MS) : (uint8_t)(flagsn&~TYPE_MS);
	}
	if(rest) {
		ux = uy = uz = 0.0f;
		a.u[n] = 0.0f; a.u[N+n] = 0.0f; a.u[2ull*N+n] = 0.0f;
	} else {
		ux = a.u[n]; uy = a.u[N+n]; uz = a.u[2ull*N+n];
	}
	const EqState s = eq_state(a.rho[n], ux, uy, uz);
	float f[Q];
	f[0] = feq0<Q>(s);
	Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; feq_pair<Q, i>(s, f[i], f[i+1]); });
	store_f<Q, ST>((T*)a.fi, N, n, nb, true, f); // odd parity (src/kernel.cpp:1429)
}

// Moving solid boundaries (src/kernel.cpp:1104-1113 apply_moving_boundaries) on the streamed DDFs of
// a TYPE_MS cell, before its density and velocity are taken: population i (i odd) gains
// -6 w_i (c_{i+1}.u_s) when the neighbour along c_{i+1} is a TYPE_S cell moving at u_s, population
// i+1 gains -6 w_i (c_i.u_s) from the neighbour along c_i (wall density 1). nbr(integral_constant<I>)
// is the neighbour index along c_I. f in real units (scale 1) or in storage units (scale K, a power
// of two: fma(K w6, c.u, K f) is exactly K fma(w6, c.u, f), so both forms add the same correction).
template<int Q, class J> __device__ __forceinline__ void apply_moving_boundaries(float* f, const StepArgs& a, const float scale, const J& nbr) {
	const uint64_t N = a.g.N;
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const float w6 = __fmul_rn(__fmul_rn(-6.0f, vs_w<Q>(i)), scale);
		const uint64_t jb = nbr(std::integral_constant<int, i+1>()), ja = nbr(std::integral_constant<int, i>());
		if((a.flags[jb]&TYPE_BO)==TYPE_S) f[i] = __fmaf_rn(w6, cdot<i+1>(a.u[jb], a.u[N+jb], a.u[2ull*N+jb]), f[i]);
		if((a.flags[ja]&TYPE_BO)==TYPE_S) f[i+1] = __fmaf_rn(w6, cdot<i>(a.u[ja], a.u[N+ja], a.u[2ull*N+ja]), f[i+1]);
	});
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

// UPDATE_FIELDS (src/kernel.cpp:1565-1573): the density and the (force-shifted, clamped) velocity a
// cell collides with, written to rho/u; V = float2 writes cells n and n+1 (n even) as aligned pairs
__device__ __forceinline__ void store_fields(const StepArgs& a, const uint64_t n, const float rho, const float ux, const float uy, const float uz) {
	const uint64_t N = a.g.N;
	a.rho_out[n] = rho; a.u_out[n] = ux; a.u_out[N+n] = uy; a.u_out[2ull*N+n] = uz;
}
__device__ __forceinline__ void store_fields(const StepArgs& a, const uint64_t n, const float2 rho, const float2 ux, const float2 uy, const float2 uz) {
	const uint64_t N = a.g.N;
	*reinterpret_cast<float2*>(a.rho_out+n) = rho; *reinterpret_cast<float2*>(a.u_out+n) = ux;
	*reinterpret_cast<float2*>(a.u_out+N+n) = uy; *reinterpret_cast<float2*>(a.u_out+2ull*N+n) = uz;
}

// one cell step on registers: f in, f out (exact: real units; fast: storage units)
// (SUBGRID: the cell's relaxation rate from the Smagorinsky-Lilly model, src/kernel.cpp:1579-1593)
template<int Q, int ST, bool TRT, int EXT, bool FAST> __device__ __forceinline__ void cell_step(float* f, const StepArgs& a, const uint64_t n, const bool is_e) {
	constexpr bool VF = (EXT&EXT_VF)!=0, SG = (EXT&EXT_SG)!=0;
	float rho, ux, uy, uz, fx, fy, fz;
	if constexpr(FAST) {
		float rm1, inv;
		cell_rho_u_fast<Q, EXT, ST>(a, n, f, is_e, rho, rm1, inv, ux, uy, uz, fx, fy, fz);
		if(a.fields_out && !is_e) store_fields(a, n, __fmul_rn(rho, 1.0f/RawCodec<ST>::K), ux, uy, uz); // rho = R/K exactly
		collide_fast<Q, TRT, VF, ST, SG>(f, rho, rm1, ux, uy, uz, fx, fy, fz, is_e, a);
	} else {
		cell_rho_u<Q, EXT>(a, n, f, is_e, rho, ux, uy, uz, fx, fy, fz);
		if(a.fields_out && !is_e) store_fields(a, n, rho, ux, uy, uz);
		if constexpr(SG) {
			StepArgs b = a; // the same step with this cell's rates
			b.w = subgrid_w_exact<Q>(f, eq_state(rho, ux, uy, uz), a.w);
			cell_rates(b.w, b.omw, b.c_tau, b.hp, b.hm, b.c_taup, b.c_taum);
			collide<Q, TRT, VF>(f, rho, ux, uy, uz, fx, fy, fz, is_e, b);
		} else {
			collide<Q, TRT, VF>(f, rho, ux, uy, uz, fx, fy, fz, is_e, a);
		}
	}
}
template<int ST, bool FAST> using StepCodec = typename std::conditional<FAST, RawCodec<ST>, Codec<ST>>::type;

// the raw slot values of cell n (its Esoteric-Pull slot set at this parity) from src to dst
template<int Q, typename T> __device__ __forceinline__ void copy_slots(const T* __restrict__ src, T* __restrict__ dst, const uint64_t N, const uint64_t n,
                                                                      const Nbr& nb, const bool odd) {
	const uint64_t e = odd ? 0ull : N;
	dst[n] = src[n];
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const uint64_t pa = (uint64_t)i*N+e+n, pb = (uint64_t)(i+1)*N-e+nb.template j<i>();
		dst[pa] = src[pa]; dst[pb] = src[pb];
	});
}

// in place (fi_dst == fi) or out of place (fi_dst != fi: solid and gas cells copy their slots, so
// dst holds the whole next state)
#ifndef FX3D_CELL_MIN_BLOCKS_Q27
#define FX3D_CELL_MIN_BLOCKS_Q27 3 // D3Q27 one-cell: 1.206 ms per step on 512x256x256 FP32 SRT exact, against 1.421 at 2 blocks (110 registers)
#endif
template<int Q, int ST, bool TRT, int EXT, bool FAST> __global__ void __launch_bounds__(BLOCK, (Q==19 ? 4 : FX3D_CELL_MIN_BLOCKS_Q27)) k_stream_collide(const StepArgs a) {
	typedef typename Codec<ST>::T T;
	constexpr bool EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n;
	const uint8_t flagsn = a.flags[n];
	const uint8_t flagsn_bo = flagsn&TYPE_BO;
	const bool odd = (a.t&1ull)!=0ull;
	if(flagsn_bo==TYPE_S||(flagsn&TYPE_SU)==TYPE_G) { // solid or gas: nothing to do in place
		if(a.fi_dst!=a.fi) copy_slots<Q>((const T*)a.fi, (T*)a.fi_dst, g.N, n, Nbr(g, c.x, c.y, c.z), odd);
		return;
	}
	const Nbr nb(g, c.x, c.y, c.z);
	float f[Q];
	load_f<Q, ST, StepCodec<ST, FAST>>((const T*)a.fi, g.N, n, nb, odd, f);
	if constexpr((EXT&EXT_MB)!=0) {
		if(flagsn_bo==TYPE_MS) apply_moving_boundaries<Q>(f, a, FAST ? RawCodec<ST>::K : 1.0f, [&](auto ic) { return nb.template j<decltype(ic)::value>(); });
	}
	const bool is_e = EQ && flagsn_bo==TYPE_E;
	cell_step<Q, ST, TRT, EXT, FAST>(f, a, n, is_e);
	store_f<Q, ST, StepCodec<ST, FAST>>((T*)a.fi_dst, g.N, n, nb, odd, f);
}

// Two x-adjacent cells (x0 even, x0+1) per thread, stepped together with packed FP32x2 arithmetic
// (fast mode; grids with even Nx and fewer than 2^32 cells). A cell's own slots and the neighbour
// slots of directions with c_x = 0 hold the two cells' values side by side at an even index, so they
// move as one aligned 4-byte (FP16) or 8-byte (FP32) access; neighbour slots of directions with
// c_x != 0 are one cell off and move as two scalar accesses. Each warp access so moves 128 bytes of
// FP16 DDFs instead of 64, and the packed instructions halve the arithmetic issued per cell.
// A pair with one solid (or gas) cell steps its other cell alone, on the one-cell path, which gives
// bit-identical results (the arithmetic is the same code in float and float2 form).
template<int ST> struct PairIO;
template<> struct PairIO<ST_FP32> {
	static __device__ __forceinline__ float2 load2(const float* p) { return *reinterpret_cast<const float2*>(p); }
	static __device__ __forceinline__ void store2(float* p, const float2 v) { *reinterpret_cast<float2*>(p) = v; }
};
template<> struct PairIO<ST_FP16S> {
	static __device__ __forceinline__ float2 load2(const uint16_t* p) { return __half22float2(*reinterpret_cast<const __half2*>(p)); }
	static __device__ __forceinline__ void store2(uint16_t* p, const float2 v) { *reinterpret_cast<__half2*>(p) = __float22half2_rn(v); }
};
template<> struct PairIO<ST_FP16C> {
	static __device__ __forceinline__ float2 load2(const uint16_t* p) { return make_float2(RawCodec<ST_FP16C>::decode(p[0]), RawCodec<ST_FP16C>::decode(p[1])); }
	static __device__ __forceinline__ void store2(uint16_t* p, const float2 v) { p[0] = RawCodec<ST_FP16C>::encode(v.x); p[1] = RawCodec<ST_FP16C>::encode(v.y); }
};

template<int Q, int ST, typename T> __device__ __forceinline__ void load_pair(const T* __restrict__ fi, const uint64_t N, const Steps32& sa, const Steps32& sb,
                                                                              const bool odd, float2* f) {
	typedef RawCodec<ST> CD;
	const uint64_t e = odd ? 0ull : N;
	f[0] = PairIO<ST>::load2(fi+sa.n);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const T* pa = fi+((uint64_t)i*N+e);
		const T* pb = fi+((uint64_t)(i+1)*N-e);
		f[i] = PairIO<ST>::load2(pa+sa.n);
		if constexpr(vs_c(0, i)==0) f[i+1] = PairIO<ST>::load2(pb+sa.template j<i>());
		else f[i+1] = make_float2(CD::decode(pb[sa.template j<i>()]), CD::decode(pb[sb.template j<i>()]));
	});
}
template<int Q, int ST, typename T> __device__ __forceinline__ void store_pair(T* __restrict__ fi, const uint64_t N, const Steps32& sa, const Steps32& sb,
                                                                               const bool odd, const float2* f) {
	typedef RawCodec<ST> CD;
	const uint64_t e = odd ? 0ull : N;
	PairIO<ST>::store2(fi+sa.n, f[0]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		T* pa = fi+((uint64_t)i*N+e);
		T* pb = fi+((uint64_t)(i+1)*N-e);
		if constexpr(vs_c(0, i)==0) PairIO<ST>::store2(pb+sa.template j<i>(), f[i]);
		else { pb[sa.template j<i>()] = CD::encode(f[i].x); pb[sb.template j<i>()] = CD::encode(f[i].y); }
		PairIO<ST>::store2(pa+sa.n, f[i+1]);
	});
}

// UPDATE_FIELDS for a pair: both cells as aligned pairs, or each non-TYPE_E cell alone
template<int ST> __device__ __forceinline__ void store_pair_fields(const StepArgs& a, const uint64_t n, const float2 R, const float2 ux, const float2 uy,
                                                                   const float2 uz, const Bool2 is_e, const bool any_e) {
	constexpr float k = 1.0f/RawCodec<ST>::K;
	const float2 rho = v_mul(R, make_float2(k, k)); // exact: K is a power of two
	if(!any_e) { store_fields(a, n, rho, ux, uy, uz); return; }
	if(!is_e.x) store_fields(a, n, rho.x, ux.x, uy.x, uz.x);
	if(!is_e.y) store_fields(a, n+1ull, rho.y, ux.y, uy.y, uz.y);
}

inline dim3 pair_grid(const GridDesc& g) { return dim3((g.NxNy/2u+BLOCK-1u)/BLOCK, g.Nz, 1u); }
inline bool pairs_supported(const GridDesc& g) { return g.Nx%2u==0u && g.N<=0xFFFFFFFFull; }
#ifndef FX3D_PIPE_BLOCK
#define FX3D_PIPE_BLOCK 256
#endif
constexpr int PIPE_BLOCK = FX3D_PIPE_BLOCK; // threads per block of the prefetching two-cell kernel

#ifndef FX3D_PAIRS_MIN_BLOCKS
#define FX3D_PAIRS_MIN_BLOCKS 2 // resident 256-thread blocks per SM the register budget is sized for
#endif
template<int Q, int ST, bool TRT, int EXT> __global__ void __launch_bounds__(BLOCK, FX3D_PAIRS_MIN_BLOCKS) k_stream_collide_pairs(const StepArgs a) {
	typedef typename Codec<ST>::T T;
	constexpr bool EQ = (EXT&EXT_EQ)!=0, VF = (EXT&EXT_VF)!=0;
	const Grid& g = grid_of(a.g);
	const uint32_t xy = 2u*(blockIdx.x*(uint32_t)BLOCK+threadIdx.x);
	if(xy>=g.NxNy) return;
	const uint32_t z = blockIdx.y, y = div_nx(g, xy), x = xy-y*g.Nx;
	const uint32_t n = z*g.NxNy+xy;
	const uint16_t fl = *reinterpret_cast<const uint16_t*>(a.flags+n); // both cells' flags (n even)
	const uint32_t fa = fl&0xFFu, fb = fl>>8;
	const bool skip_a = (fa&TYPE_BO)==TYPE_S||(fa&TYPE_SU)==TYPE_G, skip_b = (fb&TYPE_BO)==TYPE_S||(fb&TYPE_SU)==TYPE_G;
	if(skip_a&&skip_b) return;
	const bool odd = (a.t&1ull)!=0ull;
	if(skip_a||skip_b) { // one cell of the pair steps alone
		const uint32_t c = skip_a ? 1u : 0u;
		const Steps32 s(g, x+c, y, z, n+c);
		float f[Q];
		load_f32<Q, RawCodec<ST>>((const T*)a.fi, g.N, s, odd, f);
		cell_step<Q, ST, TRT, EXT, true>(f, a, n+c, EQ && ((skip_a ? fb : fa)&TYPE_BO)==TYPE_E);
		store_f32<Q, RawCodec<ST>>((T*)a.fi, g.N, s, odd, f);
		return;
	}
	const Steps32 sa(g, x, y, z, n), sb(g, x+1u, y, z, n+1u);
	float2 f[Q];
	load_pair<Q, ST>((const T*)a.fi, g.N, sa, sb, odd, f);
	const Bool2 is_e{EQ && (fa&TYPE_BO)==TYPE_E, EQ && (fb&TYPE_BO)==TYPE_E};
	const bool any_e = is_e.x||is_e.y;
	float2 R, Rm1, inv, ux, uy, uz, fx, fy, fz;
	cell_rho_u_v<Q, EXT, ST, float2>(a, n, f, is_e, any_e, R, Rm1, inv, ux, uy, uz, fx, fy, fz);
	if(a.fields_out) store_pair_fields<ST>(a, n, R, ux, uy, uz, is_e, any_e);
	if(any_e) collide_v<Q, TRT, VF, ST, 2, float2, Bool2, (EXT&EXT_SG)!=0>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
	else collide_v<Q, TRT, VF, ST, 0, float2, Bool2, (EXT&EXT_SG)!=0>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
	store_pair<Q, ST>((T*)a.fi, g.N, sa, sb, odd, f);
}

// Two-cell kernel with per-thread prefetch. A thread walks the pairs (x0, y, z) of a column of z
// planes; while it steps one pair, the DDF words of the next S-1 pairs are already in flight as
// per-thread cp.async copies into its own shared-memory slots (item k of stage s at
// smem[(s*ITEMS + k)*PIPE_BLOCK + thread]), so every warp keeps loads outstanding through its compute and
// store phases without holding them in registers, and no block-wide barrier is needed. Per pair the
// items are: the aligned 4-byte flags word holding both cells' flags, the rest slot, the own slots
// of each direction pair, and for each neighbour slot either one aligned pair word (c_x = 0) or two
// words (c_x != 0): for FP16 the aligned words holding the first cell's value in their upper half
// (index j-1, j odd) and the second cell's value in their lower half (j even), for FP32 the two
// values themselves. Values next to them belong to other cells and are read but never used.
// Slot addresses are per-thread indices onto the launch's slot table (SlotTable). Results are
// bit-identical to the plain two-cell kernel: only where the loads land differs.
// Walk length and block size (measured on 512x256x256 D3Q19 TRT FP16S, GB300): 2 z planes per
// thread in 256-thread blocks, 0.545 ms per step; 4 planes 0.567 ms (128-thread blocks), 8 planes
// 0.586 ms. Shorter walks lose the prefetch of the first pair but even out the blocks' run times.
template<int Q> __host__ __device__ constexpr int pair_nx0() { int c = 0; for(int i=1; i<Q; i+=2) if(vs_c(0, i)==0) c++; return c; }
template<int Q> __host__ __device__ constexpr int pair_items() { return 2+(Q-1)/2+pair_nx0<Q>()+2*((Q-1)/2-pair_nx0<Q>()); }
template<int Q> __host__ __device__ constexpr int pair_b_item(const int i) { // first item of the neighbour slot of pair (i, i+1)
	int k = 2+(Q-1)/2;
	for(int p=1; p<i; p+=2) k += vs_c(0, p)==0 ? 1 : 2;
	return k;
}

// Slot-array addresses of one time step, computed on the host for each launch so that a slot
// address in the kernel is one multiply-add of a per-thread index onto a kernel-parameter base
// instead of a per-direction computation of fi + i N + e: a[0] = fi (rest slots); for each opposite
// pair (i, i+1), i odd, a[i] = fi + i N + e (the array of the cells' own slots) and
// a[i+1] = fi + (i+1) N - e (the array of their neighbours' slots), with e = 0 at odd t and N at
// even t (the Esoteric-Pull slot map of src/kernel.cpp:1326-1339).
struct SlotTable { const void* a[27]; };
template<typename T> inline SlotTable slot_table(const StepArgs& s, const int q) {
	SlotTable tb{};
	const T* fi = (const T*)s.fi;
	const uint64_t N = s.g.N, e = (s.t&1ull) ? 0ull : N;
	tb.a[0] = fi;
	for(int i=1; i<q; i+=2) { tb.a[i] = fi+((uint64_t)i*N+e); tb.a[i+1] = fi+((uint64_t)(i+1)*N-e); }
	return tb;
}
template<int Q, int ST, typename T> __device__ __forceinline__ void issue_pair_t(const SlotTable& tb, const uint8_t* __restrict__ flags,
                                                                                 const Steps32& sa, const Steps32& sb, const uint32_t s0) {
	constexpr uint32_t W = 2u*sizeof(T), STRIDE = PIPE_BLOCK*W;
	auto cpw = [](const uint32_t d, const T* p) { if constexpr(W==4u) cp_async_4(d, p); else cp_async_8(d, p); };
	cp_async_4(s0, flags+(sa.n&~3u));
	cpw(s0+STRIDE, (const T*)tb.a[0]+sa.n);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		constexpr uint32_t ka = 2u+(uint32_t)(i-1)/2u, kb = (uint32_t)pair_b_item<Q>(i);
		const T* pa = (const T*)tb.a[i];
		const T* pb = (const T*)tb.a[i+1];
		cpw(s0+ka*STRIDE, pa+sa.n);
		if constexpr(vs_c(0, i)==0) cpw(s0+kb*STRIDE, pb+sa.template j<i>());
		else if constexpr(W==4u) { cp_async_4(s0+kb*STRIDE, pb+(sa.template j<i>()-1u)); cp_async_4(s0+(kb+1u)*STRIDE, pb+sb.template j<i>()); }
		else { cp_async_4(s0+kb*STRIDE, pb+sa.template j<i>()); cp_async_4(s0+(kb+1u)*STRIDE, pb+sb.template j<i>()); }
	});
}
template<int Q, int ST, typename T> __device__ __forceinline__ void store_pair_t(const SlotTable& tb, const Steps32& sa, const Steps32& sb, const float2* f) {
	typedef RawCodec<ST> CD;
	PairIO<ST>::store2((T*)tb.a[0]+sa.n, f[0]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		T* pa = (T*)tb.a[i];
		T* pb = (T*)tb.a[i+1];
		if constexpr(vs_c(0, i)==0) PairIO<ST>::store2(pb+sa.template j<i>(), f[i]);
		else { pb[sa.template j<i>()] = CD::encode(f[i].x); pb[sb.template j<i>()] = CD::encode(f[i].y); }
		PairIO<ST>::store2(pa+sa.n, f[i+1]);
	});
}

// the pair's values from its staged items (item k of this thread at w[k*PIPE_BLOCK])
template<int ST> struct PairStage;
template<> struct PairStage<ST_FP32> {
	typedef float2 W;
	static __device__ __forceinline__ float2 pair(const W* w, const int k) { return w[k*PIPE_BLOCK]; }
	static __device__ __forceinline__ float2 split(const W* w, const int k) { return make_float2(w[k*PIPE_BLOCK].x, w[(k+1)*PIPE_BLOCK].x); }
	static __device__ __forceinline__ uint32_t flags(const W* w) { return __float_as_uint(w[0].x); }
};
template<> struct PairStage<ST_FP16S> {
	typedef uint32_t W;
	static __device__ __forceinline__ float2 pair(const W* w, const int k) { return __half22float2(__halves2half2(__ushort_as_half((uint16_t)(w[k*PIPE_BLOCK]&0xFFFFu)), __ushort_as_half((uint16_t)(w[k*PIPE_BLOCK]>>16)))); }
	static __device__ __forceinline__ float2 split(const W* w, const int k) { // upper half of item k, lower half of item k+1
		const uint32_t v = __byte_perm(w[k*PIPE_BLOCK], w[(k+1)*PIPE_BLOCK], 0x5432u);
		return __half22float2(__halves2half2(__ushort_as_half((uint16_t)(v&0xFFFFu)), __ushort_as_half((uint16_t)(v>>16))));
	}
	static __device__ __forceinline__ uint32_t flags(const W* w) { return w[0]; }
};
template<> struct PairStage<ST_FP16C> { // the two codes read as 16-bit halves of the staged words
	typedef uint32_t W;
	static __device__ __forceinline__ const uint16_t* h(const W* w, const int k) { return reinterpret_cast<const uint16_t*>(w+k*PIPE_BLOCK); }
	static __device__ __forceinline__ float2 pair(const W* w, const int k) { return make_float2(RawCodec<ST_FP16C>::decode(h(w, k)[0]), RawCodec<ST_FP16C>::decode(h(w, k)[1])); }
	static __device__ __forceinline__ float2 split(const W* w, const int k) { return make_float2(RawCodec<ST_FP16C>::decode(h(w, k)[1]), RawCodec<ST_FP16C>::decode(h(w, k+1)[0])); }
	static __device__ __forceinline__ uint32_t flags(const W* w) { return w[0]; }
};
template<int Q, int ST> __device__ __forceinline__ void read_pair(const typename PairStage<ST>::W* w, float2* f) {
	f[0] = PairStage<ST>::pair(w, 1);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		f[i] = PairStage<ST>::pair(w, 2+(i-1)/2);
		if constexpr(vs_c(0, i)==0) f[i+1] = PairStage<ST>::pair(w, pair_b_item<Q>(i));
		else f[i+1] = PairStage<ST>::split(w, pair_b_item<Q>(i));
	});
}

#ifndef FX3D_PIPE_MIN_THREADS
#define FX3D_PIPE_MIN_THREADS 768 // resident threads per SM the register budget is sized for
#endif
#ifndef FX3D_PIPE_MIN_THREADS_Q27
#define FX3D_PIPE_MIN_THREADS_Q27 512 // D3Q27: 768 spilled 120-156 B and ran at 0.977 ms per step on 512x256x256 FP16S SRT, 512 at 0.828
#endif
#ifndef FX3D_PIPE_MIN_THREADS_SG
#define FX3D_PIPE_MIN_THREADS_SG 512 // SUBGRID variants (768 spilled and ran at 0.976 ms per step)
#endif
#ifndef FX3D_PIPE_STAGES
#define FX3D_PIPE_STAGES 2
#endif
#ifndef FX3D_PIPE_Z_CHUNK
#define FX3D_PIPE_Z_CHUNK 2
#endif
constexpr int PIPE_STAGES = FX3D_PIPE_STAGES; // pairs in flight per thread: PIPE_STAGES-1 ahead of the one stepped
#ifndef FX3D_PIPE_Z_CHUNK_SG
#define FX3D_PIPE_Z_CHUNK_SG 8
#endif
// z planes per thread. The SUBGRID variants run at 2 blocks per SM (124 registers), where the longer
// walk's prefetch pays: 0.627 ms per step on 512x256x256 FP16S TRT with 8 planes, 0.635 with 4, 0.672
// with 2.
template<int EXT> inline uint32_t pipe_z_chunk(const GridDesc& g) {
	const uint32_t zc = (EXT&EXT_SG)!=0 ? (uint32_t)FX3D_PIPE_Z_CHUNK_SG : (uint32_t)FX3D_PIPE_Z_CHUNK;
	return g.Nz<zc ? g.Nz : zc;
}
template<int Q, int ST> inline size_t pipe_smem(const int stages) { return (size_t)stages*pair_items<Q>()*PIPE_BLOCK*2u*sizeof(typename Codec<ST>::T); }

template<int Q, int ST, bool TRT, int EXT, int S> __global__ void __launch_bounds__(PIPE_BLOCK, ((EXT&EXT_SG)!=0 ? FX3D_PIPE_MIN_THREADS_SG : Q==27 ? FX3D_PIPE_MIN_THREADS_Q27 : FX3D_PIPE_MIN_THREADS)/PIPE_BLOCK) k_stream_collide_pairs_pipe(const StepArgs a, const uint32_t zc, const SlotTable tb) {
	typedef typename Codec<ST>::T T;
	typedef typename PairStage<ST>::W SW;
	constexpr bool EQ = (EXT&EXT_EQ)!=0, VF = (EXT&EXT_VF)!=0;
	constexpr int ITEMS = pair_items<Q>();
	extern __shared__ __align__(16) uint8_t pipe_smem_raw[];
	const Grid& g = grid_of(a.g);
	const uint32_t xy = 2u*(blockIdx.x*(uint32_t)PIPE_BLOCK+threadIdx.x);
	if(xy>=g.NxNy) return; // threads never wait on each other
	const uint32_t y = div_nx(g, xy), x = xy-y*g.Nx;
	const uint32_t z0 = blockIdx.y*zc, z1 = min(z0+zc, g.Nz);
	const bool odd = (a.t&1ull)!=0ull;
	SW* const w0 = reinterpret_cast<SW*>(pipe_smem_raw)+threadIdx.x;
	const uint32_t s0 = smem_u32(w0);
	auto issue = [&](const uint32_t z, const int stage) {
		const uint32_t n = z*g.NxNy+xy;
		const Steps32 sa(g, x, y, z, n), sb(g, x+1u, y, z, n+1u);
		issue_pair_t<Q, ST, T>(tb, a.flags, sa, sb, s0+(uint32_t)(stage*ITEMS*PIPE_BLOCK)*(uint32_t)sizeof(SW));
	};
	#pragma unroll
	for(int s=0; s<S-1; s++) {
		if(z0+(uint32_t)s<z1) issue(z0+(uint32_t)s, s);
		cp_async_commit();
	}
	int stage = 0;
	for(uint32_t z=z0; z<z1; z++) {
		const int ahead = stage+S-1<S ? stage+S-1 : stage-1; // the stage the previous pair used
		if(z+(uint32_t)(S-1)<z1) issue(z+(uint32_t)(S-1), ahead);
		cp_async_commit();
		cp_async_wait<S-1>();
		const SW* w = w0+stage*ITEMS*PIPE_BLOCK;
		stage = stage+1<S ? stage+1 : 0;
		const uint32_t n = z*g.NxNy+xy;
		const uint32_t fl = PairStage<ST>::flags(w)>>((n&3u)*8u); // both cells' flags (n even)
		const uint32_t fa = fl&0xFFu, fb = (fl>>8)&0xFFu;
		const bool skip_a = (fa&TYPE_BO)==TYPE_S||(fa&TYPE_SU)==TYPE_G, skip_b = (fb&TYPE_BO)==TYPE_S||(fb&TYPE_SU)==TYPE_G;
		if(skip_a&&skip_b) continue;
		if constexpr((EXT&EXT_MB)!=0) {
			const bool ms_a = (fa&TYPE_BO)==TYPE_MS, ms_b = (fb&TYPE_BO)==TYPE_MS;
			if(ms_a||ms_b) { // next to a moving solid: the pair's cells step one at a time (values read from the stage per cell)
				#pragma unroll 1
				for(uint32_t c=0u; c<2u; c++) {
					if(c ? skip_b : skip_a) continue;
					const Steps32 s(g, x+c, y, z, n+c);
					float2 fp[Q];
					read_pair<Q, ST>(w, fp);
					float f1[Q];
					#pragma unroll
					for(int k=0; k<Q; k++) f1[k] = c ? fp[k].y : fp[k].x;
					if(c ? ms_b : ms_a) apply_moving_boundaries<Q>(f1, a, RawCodec<ST>::K, [&](auto ic) { return (uint64_t)s.template j<decltype(ic)::value>(); });
					cell_step<Q, ST, TRT, EXT, true>(f1, a, n+c, EQ && ((c ? fb : fa)&TYPE_BO)==TYPE_E);
					store_f32<Q, RawCodec<ST>>((T*)a.fi, g.N, s, odd, f1);
				}
				continue;
			}
		}
		float2 f[Q];
		read_pair<Q, ST>(w, f);
		if(skip_a||skip_b) { // one cell of the pair steps alone
			const uint32_t c = skip_a ? 1u : 0u;
			const Steps32 s(g, x+c, y, z, n+c);
			float f1[Q];
			#pragma unroll
			for(int k=0; k<Q; k++) f1[k] = c ? f[k].y : f[k].x;
			cell_step<Q, ST, TRT, EXT, true>(f1, a, n+c, EQ && ((skip_a ? fb : fa)&TYPE_BO)==TYPE_E);
			store_f32<Q, RawCodec<ST>>((T*)a.fi, g.N, s, odd, f1);
			continue;
		}
		const Steps32 sa(g, x, y, z, n), sb(g, x+1u, y, z, n+1u);
		const Bool2 is_e{EQ && (fa&TYPE_BO)==TYPE_E, EQ && (fb&TYPE_BO)==TYPE_E};
		const bool any_e = is_e.x||is_e.y;
		float2 R, Rm1, inv, ux, uy, uz, fx, fy, fz;
		cell_rho_u_v<Q, EXT, ST, float2>(a, n, f, is_e, any_e, R, Rm1, inv, ux, uy, uz, fx, fy, fz);
		if(a.fields_out) store_pair_fields<ST>(a, n, R, ux, uy, uz, is_e, any_e);
		// one collision path per warp (warps holding an inlet or outlet pair ran both): the mixed path
		// gives non-TYPE_E lanes the plain path's values bit for bit (0.541 ms per step on the C2
		// channel, against 0.545 with the per-lane branch)
		const bool any_e_warp = __any_sync(__activemask(), any_e);
		if(any_e_warp) collide_v<Q, TRT, VF, ST, 2, float2, Bool2, (EXT&EXT_SG)!=0>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
		else collide_v<Q, TRT, VF, ST, 0, float2, Bool2, (EXT&EXT_SG)!=0>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
		store_pair_t<Q, ST, T>(tb, sa, sb, f);
	}
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
// write to a different array than it reads (fi_dst).
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

template<int Q, int ST, int EXT, bool FAST> __global__ void __launch_bounds__(BLOCK) k_update_fields(const StepArgs a, const bool mb) {
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
	if(mb && flagsn_bo==TYPE_MS) apply_moving_boundaries<Q>(f, a, FAST ? RawCodec<ST>::K : 1.0f, [&](auto ic) { return nb.template j<decltype(ic)::value>(); });
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

template<int ST, int Q, bool TRT, int EXT, bool FAST> inline cudaError_t sc_launch_t(const StepArgs& a, const int kind, cudaStream_t s) {
	// SUBGRID and MOVING_BOUNDARIES: one thread per cell or the prefetching two-cell kernel
	constexpr bool SG = (EXT&(EXT_SG|EXT_MB))!=0;
	if(kind==PATH_ROWS) {
		if constexpr(SG) return cudaErrorInvalidConfiguration; // (the row kernel serves the adjoint, which has neither)
		else {
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
		}
	} else if(kind==PATH_PAIRS||kind==PATH_PIPE) {
		if constexpr(FAST) {
			if(a.fi_dst!=a.fi||!pairs_supported(a.g)) return cudaErrorInvalidValue; // in place, even Nx, N < 2^32
			if(kind==PATH_PAIRS) {
				if constexpr(SG) return cudaErrorInvalidConfiguration;
				else k_stream_collide_pairs<Q, ST, TRT, EXT><<<pair_grid(a.g), BLOCK, 0, s>>>(a);
			} else {
				constexpr int S = PIPE_STAGES;
				auto kernel = k_stream_collide_pairs_pipe<Q, ST, TRT, EXT, S>;
				const size_t smem = pipe_smem<Q, ST>(S);
				if(smem>48u*1024u) {
					const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
					if(e!=cudaSuccess) return e;
				}
				const uint32_t zc = pipe_z_chunk<EXT>(a.g);
				kernel<<<dim3((a.g.NxNy/2u+PIPE_BLOCK-1u)/PIPE_BLOCK, (a.g.Nz+zc-1u)/zc, 1u), PIPE_BLOCK, smem, s>>>(a, zc, slot_table<typename Codec<ST>::T>(a, Q));
			}
		} else {
			return cudaErrorInvalidConfiguration; // the packed kernel has fast arithmetic only
		}
	} else {
		k_stream_collide<Q, ST, TRT, EXT, FAST><<<cell_grid(a.g), BLOCK, 0, s>>>(a);
	}
	return cudaGetLastError();
}
template<int ST, int Q, bool TRT, int EXT> inline cudaError_t sc_launch(const StepArgs& a, const int kind, const bool fast, cudaStream_t s) {
	return fast ? sc_launch_t<ST, Q, TRT, EXT, true>(a, kind, s) : sc_launch_t<ST, Q, TRT, EXT, false>(a, kind, s);
}
template<int ST, int Q, bool TRT> inline cudaError_t sc_ext(const int ext, const StepArgs& a, const int kind, const bool fast, cudaStream_t s) {
	switch(ext) {
		case 0:                        return sc_launch<ST, Q, TRT, 0>(a, kind, fast, s);
		case EXT_VF:                   return sc_launch<ST, Q, TRT, EXT_VF>(a, kind, fast, s);
		case EXT_VF|EXT_FF:            return sc_launch<ST, Q, TRT, EXT_VF|EXT_FF>(a, kind, fast, s);
		case EXT_EQ:                   return sc_launch<ST, Q, TRT, EXT_EQ>(a, kind, fast, s);
		case EXT_EQ|EXT_VF:            return sc_launch<ST, Q, TRT, EXT_EQ|EXT_VF>(a, kind, fast, s);
		case EXT_EQ|EXT_VF|EXT_FF:     return sc_launch<ST, Q, TRT, EXT_EQ|EXT_VF|EXT_FF>(a, kind, fast, s);
		default: return cudaErrorInvalidValue;
	}
}
// SUBGRID / MOVING_BOUNDARIES variants: instantiated in lbm_kernels_<storage>_<sg|mb|sgmb>.cu, one
// translation unit per combination XB of the two bits (kind already resolved)
template<int ST, int XB> cudaError_t launch_stream_collide_x(const Variant& v, const StepArgs& a, int kind, cudaStream_t s);
#define FX3D_DECLARE_X_LAUNCHERS(ST) \
	template<> cudaError_t launch_stream_collide_x<ST, EXT_SG>(const Variant& v, const StepArgs& a, int kind, cudaStream_t s); \
	template<> cudaError_t launch_stream_collide_x<ST, EXT_MB>(const Variant& v, const StepArgs& a, int kind, cudaStream_t s); \
	template<> cudaError_t launch_stream_collide_x<ST, EXT_SG|EXT_MB>(const Variant& v, const StepArgs& a, int kind, cudaStream_t s);
FX3D_DECLARE_X_LAUNCHERS(ST_FP32)
FX3D_DECLARE_X_LAUNCHERS(ST_FP16S)
FX3D_DECLARE_X_LAUNCHERS(ST_FP16C)
#undef FX3D_DECLARE_X_LAUNCHERS
template<int ST, int Q, bool TRT, int XB> inline cudaError_t sc_ext_x(const int ext, const StepArgs& a, const int kind, const bool fast, cudaStream_t s) {
	switch(ext&~(EXT_SG|EXT_MB)) {
		case 0:                        return sc_launch<ST, Q, TRT, XB>(a, kind, fast, s);
		case EXT_VF:                   return sc_launch<ST, Q, TRT, XB|EXT_VF>(a, kind, fast, s);
		case EXT_VF|EXT_FF:            return sc_launch<ST, Q, TRT, XB|EXT_VF|EXT_FF>(a, kind, fast, s);
		case EXT_EQ:                   return sc_launch<ST, Q, TRT, XB|EXT_EQ>(a, kind, fast, s);
		case EXT_EQ|EXT_VF:            return sc_launch<ST, Q, TRT, XB|EXT_EQ|EXT_VF>(a, kind, fast, s);
		case EXT_EQ|EXT_VF|EXT_FF:     return sc_launch<ST, Q, TRT, XB|EXT_EQ|EXT_VF|EXT_FF>(a, kind, fast, s);
		default: return cudaErrorInvalidValue;
	}
}
template<int ST, int XB> cudaError_t launch_stream_collide_x_t(const Variant& v, const StepArgs& a, const int kind, cudaStream_t s) {
	if((v.ext&(EXT_SG|EXT_MB))!=XB) return cudaErrorInvalidValue;
	if(v.q==19) return v.trt ? sc_ext_x<ST, 19, true, XB>(v.ext, a, kind, v.fast, s) : sc_ext_x<ST, 19, false, XB>(v.ext, a, kind, v.fast, s);
	if(v.q==27) return v.trt ? sc_ext_x<ST, 27, true, XB>(v.ext, a, kind, v.fast, s) : sc_ext_x<ST, 27, false, XB>(v.ext, a, kind, v.fast, s);
	return cudaErrorInvalidValue;
}

template<int ST> cudaError_t launch_stream_collide_t(const Variant& v, const StepArgs& a, const int path, cudaStream_t s) {
	// automatic choice (measured on 512x256x256): for fast arithmetic in place with 16-bit storage the
	// two-cell kernel with per-thread prefetch; otherwise one thread per cell, in place or into another
	// array (FP32 moves enough bytes per access to reach about 90% of the bandwidth that way; it also
	// beat the row-staged kernel out of place)
	const bool rows_ok = row_plan(v.q, ST, a.g.Nx, a.g.Ny, a.g.Nz).stages!=0u;
	const bool pairs_ok = v.fast && pairs_supported(a.g) && a.fi_dst==a.fi;
	int kind = path;
	if(path==PATH_AUTO) kind = pairs_ok && ST!=ST_FP32 ? PATH_PIPE : PATH_CELLS;
	if((kind==PATH_ROWS && !rows_ok) || ((kind==PATH_PAIRS||kind==PATH_PIPE) && !pairs_ok)) return cudaErrorInvalidConfiguration;
	switch(v.ext&(EXT_SG|EXT_MB)) {
		case EXT_SG: return launch_stream_collide_x<ST, EXT_SG>(v, a, kind, s);
		case EXT_MB: return launch_stream_collide_x<ST, EXT_MB>(v, a, kind, s);
		case EXT_SG|EXT_MB: return launch_stream_collide_x<ST, EXT_SG|EXT_MB>(v, a, kind, s);
		default: break;
	}
	if(v.q==19) return v.trt ? sc_ext<ST, 19, true>(v.ext, a, kind, v.fast, s) : sc_ext<ST, 19, false>(v.ext, a, kind, v.fast, s);
	if(v.q==27) return v.trt ? sc_ext<ST, 27, true>(v.ext, a, kind, v.fast, s) : sc_ext<ST, 27, false>(v.ext, a, kind, v.fast, s);
	return cudaErrorInvalidValue;
}

template<int ST, int Q, int EXT> inline void uf_launch(const StepArgs& a, const bool fast, const bool mb, cudaStream_t s) {
	if(fast) k_update_fields<Q, ST, EXT, true><<<cell_grid(a.g), BLOCK, 0, s>>>(a, mb);
	else k_update_fields<Q, ST, EXT, false><<<cell_grid(a.g), BLOCK, 0, s>>>(a, mb);
}
template<int ST, int Q> inline bool uf_ext(const int ext, const StepArgs& a, const bool fast, const bool mb, cudaStream_t s) {
	switch(ext) {
		case 0:                        uf_launch<ST, Q, 0>(a, fast, mb, s); return true;
		case EXT_VF:                   uf_launch<ST, Q, EXT_VF>(a, fast, mb, s); return true;
		case EXT_VF|EXT_FF:            uf_launch<ST, Q, EXT_VF|EXT_FF>(a, fast, mb, s); return true;
		case EXT_EQ:                   uf_launch<ST, Q, EXT_EQ>(a, fast, mb, s); return true;
		case EXT_EQ|EXT_VF:            uf_launch<ST, Q, EXT_EQ|EXT_VF>(a, fast, mb, s); return true;
		case EXT_EQ|EXT_VF|EXT_FF:     uf_launch<ST, Q, EXT_EQ|EXT_VF|EXT_FF>(a, fast, mb, s); return true;
		default: return false;
	}
}
template<int ST> cudaError_t launch_update_fields_t(const Variant& v, const StepArgs& a, cudaStream_t s) {
	const int ext = v.ext&~(EXT_SG|EXT_MB); // SUBGRID changes only the collision; MOVING_BOUNDARIES is a run-time switch here
	const bool mb = (v.ext&EXT_MB)!=0;
	const bool ok = v.q==19 ? uf_ext<ST, 19>(ext, a, v.fast, mb, s) : v.q==27 ? uf_ext<ST, 27>(ext, a, v.fast, mb, s) : false;
	return ok ? cudaGetLastError() : cudaErrorInvalidValue;
}

template<int ST> cudaError_t launch_initialize_t(const Variant& v, const StepArgs& a, cudaStream_t s) {
	uint8_t* flags = const_cast<uint8_t*>(a.flags); // the domain's own flags array: initialize marks TYPE_MS cells
	const bool mb = (v.ext&EXT_MB)!=0;
	if(v.q==19) k_initialize<19, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a, flags, mb);
	else if(v.q==27) k_initialize<27, ST><<<cell_grid(a.g), BLOCK, 0, s>>>(a, flags, mb);
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

#define FX3D_DEFINE_X_LAUNCHER(ST, XB) \
	namespace fx3d { \
	template<> cudaError_t launch_stream_collide_x<ST, XB>(const Variant& v, const StepArgs& a, const int kind, cudaStream_t s) { return launch_stream_collide_x_t<ST, XB>(v, a, kind, s); } \
	}

#define FX3D_DEFINE_LAUNCHERS(sfx, ST) \
	namespace fx3d { \
	cudaError_t launch_initialize_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s) { return launch_initialize_t<ST>(v, a, s); } \
	cudaError_t launch_stream_collide_##sfx(const Variant& v, const StepArgs& a, const int path, cudaStream_t s) { return launch_stream_collide_t<ST>(v, a, path, s); } \
	cudaError_t launch_update_fields_##sfx(const Variant& v, const StepArgs& a, cudaStream_t s) { return launch_update_fields_t<ST>(v, a, s); } \
	cudaError_t launch_update_force_field_##sfx(const Variant& v, const StepArgs& a, float* F, cudaStream_t s) { return launch_update_force_field_t<ST>(v, a, F, s); } \
	}
