// Device-side LBM scheme for sm_103a: velocity sets, DDF storage codecs, Esoteric-Pull slot
// addressing, moments, equilibrium, Guo forcing and the SRT/TRT collision, written so every kernel
// of the library (forward, fields, forces, adjoint) shares one definition of the arithmetic.
//
// Arithmetic contract of this file ("exact" mode): FP32 in the reference's operation order, fmaf()
// exactly where the reference writes fma() (src/kernel.cpp:1004-1101, 1550-1633) and every other
// multiply/add/divide spelled as a rounding intrinsic (__fmul_rn, __fadd_rn, __fdiv_rn), which the
// compiler never contracts, so a kernel's result is bit-identical to the FP32 restatement of the
// scheme on the CPU. The fast mode (lbm_fast.cuh) trades that for about a third of the instructions.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>
#include <type_traits>
#include "lbm_internal.h"

namespace fx3d {

enum : uint8_t {
	TYPE_S = 0x01, TYPE_E = 0x02, TYPE_T = 0x04, TYPE_F = 0x08, TYPE_I = 0x10, TYPE_G = 0x20, TYPE_X = 0x40, TYPE_Y = 0x80,
	TYPE_MS = 0x03, TYPE_BO = 0x03, TYPE_SU = 0x38, TYPE_XY = 0xC0
};

// ---------------------------------------------------------------- velocity sets
// Direction order of src/kernel.cpp:878-887; D3Q19 is the first 19 directions of D3Q27. Pairs
// (i,i+1), i odd, are opposite directions.
__host__ __device__ constexpr int vs_c(const int d, const int i) {
	constexpr int c[3][27] = {
		{0, 1,-1, 0, 0, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1},
		{0, 0, 0, 1,-1, 0, 0, 1,-1, 0, 0, 1,-1,-1, 1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1, 1,-1},
		{0, 0, 0, 0, 0, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0,-1, 1,-1, 1, 1,-1,-1, 1, 1,-1, 1,-1}};
	return c[d][i];
}
// lattice weights as the reference's device defines spell them (src/lbm.cpp:383-393)
template<int Q> __device__ __forceinline__ float vs_w(const int i) {
	if(Q==19) return i==0 ? 1.0f/3.0f : i<7 ? 1.0f/18.0f : 1.0f/36.0f;
	return i==0 ? 1.0f/3.375f : i<7 ? 1.0f/13.5f : i<19 ? 1.0f/54.0f : 1.0f/216.0f;
}

constexpr float DEF_C = 0.57735027f;     // lattice speed of sound (src/lbm.cpp:373)
constexpr float THIRD = 0.33333334f;     // the reference's 1/3 literal (src/kernel.cpp:1096-1099)

// signed sum of the non-zero c_d*v_d in x,y,z order: equals c(i)*vx+c(N+i)*vy+c(2N+i)*vz of the
// reference exactly (c_d in {-1,0,1}), up to the sign of an exact zero
template<int I> __device__ __forceinline__ float csum(const float vx, const float vy, const float vz) {
	constexpr int a = vs_c(0, I), b = vs_c(1, I), c = vs_c(2, I);
	float s = 0.0f; bool first = true;
	if(a!=0) { s = a>0 ? vx : -vx; first = false; }
	if(b!=0) { const float t = b>0 ? vy : -vy; s = first ? t : __fadd_rn(s, t); first = false; }
	if(c!=0) { const float t = c>0 ? vz : -vz; s = first ? t : __fadd_rn(s, t); }
	return s;
}

// c_I.v as the reference writes it in apply_moving_boundaries: c(I)*vx+c(N+I)*vy+c(2N+I)*vz with the
// velocities as FP32 constants, each product rounded (exact), summed left to right
template<int I> __device__ __forceinline__ float cdot(const float vx, const float vy, const float vz) {
	return __fadd_rn(__fadd_rn(__fmul_rn((float)vs_c(0, I), vx), __fmul_rn((float)vs_c(1, I), vy)), __fmul_rn((float)vs_c(2, I), vz));
}

// ---------------------------------------------------------------- DDF storage codecs
template<int ST> struct Codec;
template<> struct Codec<ST_FP32> {
	typedef float T;
	static __device__ __forceinline__ float decode(const float x) { return x; }
	static __device__ __forceinline__ float encode(const float x) { return x; }
	static __device__ __forceinline__ float load(const T* p) { return *p; }
	static __device__ __forceinline__ void store(T* p, const float x) { *p = x; }
};
template<> struct Codec<ST_FP16S> { // IEEE half, range-shifted by 2^15 (src/lbm.cpp:411-414)
	typedef uint16_t T;
	static __device__ __forceinline__ float decode(const uint16_t h) { return __fmul_rn(__half2float(__ushort_as_half(h)), 3.0517578E-5f); }
	static __device__ __forceinline__ uint16_t encode(const float x) { return __half_as_ushort(__float2half_rn(__fmul_rn(x, 32768.0f))); }
	static __device__ __forceinline__ float load(const T* p) { return decode(*p); }
	static __device__ __forceinline__ void store(T* p, const float x) { *p = encode(x); }
};
template<> struct Codec<ST_FP16C> { // custom 1-4-11 format (src/kernel.cpp:848-859), integer bit operations
	typedef uint16_t T;
	static __device__ __forceinline__ float decode(const uint16_t xs) {
		const uint32_t x = xs;
		const uint32_t e = (x&0x7800u)>>11;
		const uint32_t m = (x&0x07FFu)<<12;
		const uint32_t v = __float_as_uint((float)m)>>23;
		return __uint_as_float((x&0x8000u)<<16 | (uint32_t)(e!=0u)*((e+112u)<<23|m) | (uint32_t)((e==0u)&(m!=0u))*((v-37u)<<23|((m<<(150u-v))&0x007FF000u)));
	}
	static __device__ __forceinline__ uint16_t encode(const float xf) {
		const uint32_t b = __float_as_uint(xf)+0x00000800u;
		const uint32_t e = (b&0x7F800000u)>>23;
		const uint32_t m = b&0x007FFFFFu;
		return (uint16_t)((b&0x80000000u)>>16 | (uint32_t)(e>112u)*((((e-112u)<<11)&0x7800u)|m>>12) | (uint32_t)((e<113u)&(e>100u))*((((0x007FF800u+m)>>(124u-e))+1u)>>1));
	}
	static __device__ __forceinline__ float load(const T* p) { return decode(*p); }
	static __device__ __forceinline__ void store(T* p, const float x) { *p = encode(x); }
};

// ---------------------------------------------------------------- lattice geometry
struct Grid {
	uint32_t Nx, Ny, Nz, NxNy;
	uint64_t N;
	uint64_t nx_inv; // ceil(2^64/Nx) (0 when Nx==1): y = xy/Nx without a divide
};
__device__ __forceinline__ uint32_t div_nx(const Grid& g, const uint32_t xy) { return g.nx_inv ? (uint32_t)__umul64hi((uint64_t)xy, g.nx_inv) : xy; }

// periodic neighbour offsets of one cell (src/kernel.cpp:904-915 calculate_indices)
struct Nbr {
	uint32_t x0, xp, xm, y0, yp, ym;
	uint64_t z0, zp, zm;
	__device__ __forceinline__ Nbr(const Grid& g, const uint32_t x, const uint32_t y, const uint32_t z) {
		x0 = x; xp = x+1u==g.Nx ? 0u : x+1u; xm = x==0u ? g.Nx-1u : x-1u;
		y0 = y*g.Nx; yp = (y+1u==g.Ny ? 0u : y+1u)*g.Nx; ym = (y==0u ? g.Ny-1u : y-1u)*g.Nx;
		z0 = (uint64_t)z*g.NxNy; zp = (uint64_t)(z+1u==g.Nz ? 0u : z+1u)*g.NxNy; zm = (uint64_t)(z==0u ? g.Nz-1u : z-1u)*g.NxNy;
	}
	template<int I> __device__ __forceinline__ uint64_t j() const { // neighbour in direction c_I
		constexpr int a = vs_c(0, I), b = vs_c(1, I), c = vs_c(2, I);
		const uint32_t xx = a>0 ? xp : a<0 ? xm : x0;
		const uint32_t yy = b>0 ? yp : b<0 ? ym : y0;
		const uint64_t zz = c>0 ? zp : c<0 ? zm : z0;
		return (uint64_t)(xx+yy)+zz;
	}
};

// ---------------------------------------------------------------- compile-time loop
template<int I, int END, int STEP> struct Unroll {
	template<typename F> static __device__ __forceinline__ void run(F&& f) {
		if constexpr(I<END) { f(std::integral_constant<int, I>()); Unroll<I+STEP, END, STEP>::run(f); }
	}
};

// ---------------------------------------------------------------- Esoteric-Pull (src/kernel.cpp:1326-1339)
// Pair (i,i+1), i odd: slot A = (n, odd ? i : i+1), slot B = (j[i], odd ? i+1 : i). Load reads
// f_i from A and f_{i+1} from B; store writes f_i to B and f_{i+1} to A.
template<int Q, int ST, class CD=Codec<ST>> __device__ __forceinline__ void load_f(const typename Codec<ST>::T* fi, const uint64_t N, const uint64_t n, const Nbr& nb,
                                                                                  const bool odd, float* f) {
	const uint64_t e = odd ? 0ull : N;
	f[0] = CD::decode(fi[n]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		f[i   ] = CD::decode(fi[(uint64_t)i*N+e+n]);
		f[i+1] = CD::decode(fi[(uint64_t)(i+1)*N-e+nb.template j<i>()]);
	});
}
template<int Q, int ST, class CD=Codec<ST>> __device__ __forceinline__ void store_f(typename Codec<ST>::T* fi, const uint64_t N, const uint64_t n, const Nbr& nb,
                                                                                   const bool odd, const float* f) {
	const uint64_t e = odd ? 0ull : N;
	fi[n] = CD::encode(f[0]);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		fi[(uint64_t)(i+1)*N-e+nb.template j<i>()] = CD::encode(f[i]);
		fi[(uint64_t)i*N+e+n] = CD::encode(f[i+1]);
	});
}

// ---------------------------------------------------------------- moments (src/kernel.cpp:1063-1088)
// rho = sum f_i in index order, +1 last; each momentum component alternates +f(positive member)
// -f(negative member) over the pairs in index order
template<int Q, int D> __device__ __forceinline__ float momentum(const float* f) {
	float s = 0.0f; bool first = true;
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		constexpr int c = vs_c(D, i);
		if constexpr(c!=0) {
			const float fp = c>0 ? f[i] : f[i+1], fm = c>0 ? f[i+1] : f[i];
			s = first ? __fsub_rn(fp, fm) : __fsub_rn(__fadd_rn(s, fp), fm);
			first = false;
		}
	});
	return s;
}
template<int Q> __device__ __forceinline__ void moments(const float* f, float& rho, float& mx, float& my, float& mz) {
	rho = f[0];
	#pragma unroll
	for(int i=1; i<Q; i++) rho = __fadd_rn(rho, f[i]);
	rho = __fadd_rn(rho, 1.0f);
	mx = momentum<Q, 0>(f); my = momentum<Q, 1>(f); mz = momentum<Q, 2>(f);
}

// equilibrium of one direction pair (src/kernel.cpp:1004-1061): u_k = 3*(c_i . u)
struct EqState { float rho, rhom1, c3, ux3, uy3, uz3; };
__device__ __forceinline__ EqState eq_state(const float rho, const float ux, const float uy, const float uz) {
	EqState s;
	s.rho = rho; s.rhom1 = __fsub_rn(rho, 1.0f);
	s.c3 = __fmul_rn(-3.0f, __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz)));
	s.ux3 = __fmul_rn(ux, 3.0f); s.uy3 = __fmul_rn(uy, 3.0f); s.uz3 = __fmul_rn(uz, 3.0f);
	return s;
}
template<int Q> __device__ __forceinline__ float feq0(const EqState& s) { return __fmul_rn(vs_w<Q>(0), fmaf(s.rho, __fmul_rn(0.5f, s.c3), s.rhom1)); }
template<int Q, int I> __device__ __forceinline__ void feq_pair(const EqState& s, float& fa, float& fb) {
	const float wi = vs_w<Q>(I);
	const float rhow = __fmul_rn(wi, s.rho), rhom1w = __fmul_rn(wi, s.rhom1);
	const float uk = csum<I>(s.ux3, s.uy3, s.uz3);
	const float quad = fmaf(uk, uk, s.c3);
	fa = fmaf(rhow, fmaf(0.5f, quad,  uk), rhom1w);
	fb = fmaf(rhow, fmaf(0.5f, quad, -uk), rhom1w);
}

// Guo forcing term of direction I (src/kernel.cpp:1091-1101)
template<int Q, int I> __device__ __forceinline__ float forcing_term(const float ux, const float uy, const float uz, const float fx, const float fy, const float fz, const float uF) {
	if constexpr(I==0) return __fmul_rn(__fmul_rn(9.0f, vs_w<Q>(0)), uF);
	else return __fmul_rn(__fmul_rn(9.0f, vs_w<Q>(I)), fmaf(csum<I>(fx, fy, fz), __fadd_rn(csum<I>(ux, uy, uz), THIRD), uF));
}
__device__ __forceinline__ float forcing_uF(const float ux, const float uy, const float uz, const float fx, const float fy, const float fz) {
	return __fmul_rn(-THIRD, fmaf(ux, fx, fmaf(uy, fy, __fmul_rn(uz, fz))));
}

__device__ __forceinline__ float clampc(const float x) { return fminf(fmaxf(x, -DEF_C), DEF_C); }

// force shift and velocity clamp (src/kernel.cpp:1550-1563)
template<bool VF> __device__ __forceinline__ void shift_clamp(float& ux, float& uy, float& uz, const float rho, const float fx, const float fy, const float fz) {
	if constexpr(VF) {
		const float rho2 = __fdiv_rn(0.5f, rho);
		ux = clampc(fmaf(fx, rho2, ux)); uy = clampc(fmaf(fy, rho2, uy)); uz = clampc(fmaf(fz, rho2, uz));
	} else {
		ux = clampc(ux); uy = clampc(uy); uz = clampc(uz);
	}
}

// SRT / TRT collision of all directions in place (src/kernel.cpp:1595-1633). f: streamed DDFs,
// rho/u: after force shift and clamp, fx..fz: total force, is_e: TYPE_E cell (f = feq).
// ---------------------------------------------------------------- SUBGRID (src/kernel.cpp:1579-1593)
// the collision rates of a cell from its relaxation rate w, with the reference's FP32 operations
// (src/kernel.cpp:1598, 1606-1609; the host computes the same once for the uniform rate)
__device__ __forceinline__ void cell_rates(const float w, float& omw, float& c_tau, float& hp, float& hm, float& c_taup, float& c_taum) {
	const float wm = __fdiv_rn(1.0f, __fadd_rn(__fdiv_rn(0.1875f, __fsub_rn(__fdiv_rn(1.0f, w), 0.5f)), 0.5f));
	omw = __fsub_rn(1.0f, w); c_tau = __fmaf_rn(w, -0.5f, 1.0f);
	hp = __fmul_rn(0.5f, w); hm = __fmul_rn(0.5f, wm);
	c_taup = __fmaf_rn(w, -0.25f, 0.5f); c_taum = __fmaf_rn(wm, -0.25f, 0.5f);
}
// Smagorinsky-Lilly: the relaxation rate of a cell from the non-equilibrium stress tensor
// H = sum_i c_i c_i^T (f_i - feq_i) (components xx, yy, zz, xy, xz, yz) and its density:
// w = 2/(tau0 + sqrt(tau0^2 + 0.76421222 sqrt(H:H)/rho)), tau0 = 1/w0, in the reference's order
__device__ __forceinline__ float subgrid_w(const float w0, const float* H, const float rho) {
	const float tau0 = __fdiv_rn(1.0f, w0);
	const float diag = __fadd_rn(__fadd_rn(__fmul_rn(H[0], H[0]), __fmul_rn(H[1], H[1])), __fmul_rn(H[2], H[2]));
	const float offd = __fadd_rn(__fadd_rn(__fmul_rn(H[3], H[3]), __fmul_rn(H[4], H[4])), __fmul_rn(H[5], H[5]));
	const float Qs = __fadd_rn(diag, __fmul_rn(2.0f, offd));
	return __fdiv_rn(2.0f, __fadd_rn(tau0, __fsqrt_rn(__fadd_rn(__fmul_rn(tau0, tau0), __fdiv_rn(__fmul_rn(0.76421222f, __fsqrt_rn(Qs)), rho)))));
}
// add the stress contribution v = f_i - feq_i of direction I (terms with a zero velocity component
// are +-0 in the reference's sums and leave them unchanged, so they are skipped)
template<int I> __device__ __forceinline__ void stress_add(float* H, const float v) {
	constexpr int cx = vs_c(0, I), cy = vs_c(1, I), cz = vs_c(2, I);
	if constexpr(cx!=0) H[0] = __fadd_rn(H[0], v);
	if constexpr(cy!=0) H[1] = __fadd_rn(H[1], v);
	if constexpr(cz!=0) H[2] = __fadd_rn(H[2], v);
	if constexpr(cx!=0 && cy!=0) H[3] = __fadd_rn(H[3], cx*cy>0 ? v : -v);
	if constexpr(cx!=0 && cz!=0) H[4] = __fadd_rn(H[4], cx*cz>0 ? v : -v);
	if constexpr(cy!=0 && cz!=0) H[5] = __fadd_rn(H[5], cy*cz>0 ? v : -v);
}
// the subgrid relaxation rate from the streamed DDFs f and the equilibrium state (exact scheme)
template<int Q> __device__ __forceinline__ float subgrid_w_exact(const float* f, const EqState& s, const float w0) {
	float H[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		float fa, fb;
		feq_pair<Q, i>(s, fa, fb);
		stress_add<i>(H, __fsub_rn(f[i], fa));
		stress_add<i+1>(H, __fsub_rn(f[i+1], fb));
	});
	return subgrid_w(w0, H, s.rho);
}

template<int Q, bool TRT, bool VF> __device__ __forceinline__ void collide(float* f, const float rho, const float ux, const float uy, const float uz,
                                                                          const float fx, const float fy, const float fz, const bool is_e, const StepArgs& a) {
	const float w = a.w;
	const EqState s = eq_state(rho, ux, uy, uz);
	const float uF = VF ? forcing_uF(ux, uy, uz, fx, fy, fz) : 0.0f;
	if constexpr(!TRT) {
		const float omw = a.omw, c_tau = a.c_tau;
		{
			const float fe = feq0<Q>(s);
			const float Fi = VF ? __fmul_rn(forcing_term<Q, 0>(ux, uy, uz, fx, fy, fz, uF), c_tau) : 0.0f;
			f[0] = is_e ? fe : fmaf(omw, f[0], fmaf(w, fe, Fi));
		}
		Unroll<1, Q, 2>::run([&](auto ic) {
			constexpr int i = decltype(ic)::value;
			float fa, fb;
			feq_pair<Q, i>(s, fa, fb);
			const float Fa = VF ? __fmul_rn(forcing_term<Q, i  >(ux, uy, uz, fx, fy, fz, uF), c_tau) : 0.0f;
			const float Fb = VF ? __fmul_rn(forcing_term<Q, i+1>(ux, uy, uz, fx, fy, fz, uF), c_tau) : 0.0f;
			f[i  ] = is_e ? fa : fmaf(omw, f[i  ], fmaf(w, fa, Fa));
			f[i+1] = is_e ? fb : fmaf(omw, f[i+1], fmaf(w, fb, Fb));
		});
	} else {
		const float hp = a.hp, hm = a.hm, c_taup = a.c_taup, c_taum = a.c_taum; // host-computed with the reference's operations
		{ // i = 0: its own opposite
			const float fe = feq0<Q>(s);
			float Fi = 0.0f;
			if constexpr(VF) { const float F0 = forcing_term<Q, 0>(ux, uy, uz, fx, fy, fz, uF); Fi = fmaf(c_taup, __fadd_rn(F0, F0), __fmul_rn(c_taum, __fsub_rn(F0, F0))); }
			const float fh = f[0];
			f[0] = is_e ? fe : fmaf(hp, __fsub_rn(__fadd_rn(__fsub_rn(fe, fh), fe), fh), fmaf(hm, __fadd_rn(__fsub_rn(__fsub_rn(fe, fe), fh), fh), __fadd_rn(fh, Fi)));
		}
		Unroll<1, Q, 2>::run([&](auto ic) {
			constexpr int i = decltype(ic)::value;
			float ea, eb;
			feq_pair<Q, i>(s, ea, eb);
			float Fa = 0.0f, Fb = 0.0f;
			if constexpr(VF) {
				const float Ga = forcing_term<Q, i  >(ux, uy, uz, fx, fy, fz, uF);
				const float Gb = forcing_term<Q, i+1>(ux, uy, uz, fx, fy, fz, uF);
				Fa = fmaf(c_taup, __fadd_rn(Ga, Gb), __fmul_rn(c_taum, __fsub_rn(Ga, Gb)));
				Fb = fmaf(c_taup, __fadd_rn(Gb, Ga), __fmul_rn(c_taum, __fsub_rn(Gb, Ga)));
			}
			const float ha = f[i], hb = f[i+1];
			f[i  ] = is_e ? ea : fmaf(hp, __fsub_rn(__fadd_rn(__fsub_rn(ea, ha), eb), hb), fmaf(hm, __fadd_rn(__fsub_rn(__fsub_rn(ea, eb), ha), hb), __fadd_rn(ha, Fa)));
			f[i+1] = is_e ? eb : fmaf(hp, __fsub_rn(__fadd_rn(__fsub_rn(eb, hb), ea), ha), fmaf(hm, __fadd_rn(__fsub_rn(__fsub_rn(eb, ea), hb), ha), __fadd_rn(hb, Fb)));
		});
	}
}

} // namespace fx3d
