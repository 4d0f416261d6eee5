// 32-bit Esoteric-Pull slot addressing for grids of fewer than 2^32 cells.
//
// The slot arrays of one parity start at warp-uniform addresses (fi + i*N + e for the cell's own
// slots, fi + (i+1)*N - e for its neighbours' slots; e = 0 at odd t, N at even t), so a slot
// address is one 32x32->64-bit multiply-add of a per-thread cell index onto a uniform base. The
// neighbour index j_i = n + step_x + step_y + step_z uses per-thread steps that already contain the
// periodic wrap (src/kernel.cpp:904-915 calculate_indices wraps each coordinate): a step of +1 in x
// is 1, or 1-Nx in the last column, and so on. All index arithmetic is modulo 2^32; the true
// neighbour index is in [0, N), so the 32-bit sum equals it whatever the intermediate wraps.
// The slots addressed are exactly those of load_f/store_f (lbm_scheme.cuh).
#pragma once
#include "lbm_scheme.cuh"

namespace fx3d {

struct Steps32 {
	uint32_t n, xp, xm, yp, ym, zp, zm;
	__host__ __device__ __forceinline__ Steps32(const Grid& g, const uint32_t x, const uint32_t y, const uint32_t z, const uint32_t n_) : n(n_) {
		const uint32_t N = (uint32_t)g.N;
		xp = x+1u==g.Nx ? 1u-g.Nx : 1u;
		xm = x==0u ? g.Nx-1u : 0xFFFFFFFFu;
		yp = y+1u==g.Ny ? g.Nx-g.NxNy : g.Nx;
		ym = y==0u ? g.NxNy-g.Nx : 0u-g.Nx;
		zp = z+1u==g.Nz ? g.NxNy-N : g.NxNy;
		zm = z==0u ? N-g.NxNy : 0u-g.NxNy;
	}
	template<int I> __host__ __device__ __forceinline__ uint32_t j() const { // neighbour in direction c_I
		constexpr int a = vs_c(0, I), b = vs_c(1, I), c = vs_c(2, I);
		const uint32_t sx = a>0 ? xp : a<0 ? xm : 0u;
		const uint32_t sy = b>0 ? yp : b<0 ? ym : 0u;
		const uint32_t sz = c>0 ? zp : c<0 ? zm : 0u;
		if constexpr(a!=0 && b!=0 && c!=0) return n+sx+sy+sz;
		else if constexpr(a!=0 && b!=0) return n+sx+sy;
		else if constexpr(a!=0 && c!=0) return n+sx+sz;
		else if constexpr(b!=0 && c!=0) return n+sy+sz;
		else if constexpr(a!=0) return n+sx;
		else if constexpr(b!=0) return n+sy;
		else return n+sz;
	}
};

// Esoteric-Pull load and store (the same slots as load_f/store_f)
template<int Q, class CD, typename T> __device__ __forceinline__ void load_f32(const T* __restrict__ fi, const uint64_t N, const Steps32& s, const bool odd,
                                                                               float* f) {
	const uint64_t e = odd ? 0ull : N;
	f[0] = CD::decode(fi[s.n]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const T* pa = fi+((uint64_t)i*N+e);
		const T* pb = fi+((uint64_t)(i+1)*N-e);
		f[i] = CD::decode(pa[s.n]);
		f[i+1] = CD::decode(pb[s.template j<i>()]);
	});
}
template<int Q, class CD, typename T> __device__ __forceinline__ void store_f32(T* __restrict__ fi, const uint64_t N, const Steps32& s, const bool odd,
                                                                                const float* f) {
	const uint64_t e = odd ? 0ull : N;
	fi[s.n] = CD::encode(f[0]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		T* pa = fi+((uint64_t)i*N+e);
		T* pb = fi+((uint64_t)(i+1)*N-e);
		pb[s.template j<i>()] = CD::encode(f[i]);
		pa[s.n] = CD::encode(f[i+1]);
	});
}

} // namespace fx3d
