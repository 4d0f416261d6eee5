// Fast arithmetic for one LBM cell step: the reference's scheme (src/kernel.cpp:1454-1636) with the
// freedoms its own GPU build takes (-cl-mad-enable: multiply-adds contracted; OpenCL's default
// non-IEEE division) plus exact algebraic regroupings, at about a third of the issued instructions
// of the operation-for-operation form in lbm_scheme.cuh:
//   * DDFs stay in storage units: FP16S values are used as stored (2^15 times the DDF), so loads and
//     stores are a bare conversion; the density carries the same factor K (R = K*rho), the Guo force
//     terms are scaled by K and the velocity, a ratio, needs no rescaling;
//   * one reciprocal of R per cell instead of four divisions (the velocity gets one Newton correction); rho-1 is the plain sum of the shifted
//     DDFs (the shift is added after summing, as the reference intends with DDF shifting);
//   * moments from pair sums and pair differences (f_i+f_j, f_i-f_j for opposite i,j);
//   * equilibrium of an opposite pair from one shared base term: feq_{i,j} = base +- rho w_i u_k;
//   * TRT in symmetric / antisymmetric parts: with d = feq - f,
//     f_i += hp (d_i+d_j) + hm (d_i-d_j) + F_i,  f_j += hp (d_i+d_j) - hm (d_i-d_j) + F_j,
//     which equals the reference's fma(0.5wp, ..., fma(0.5wm, ..., f+Fin)) in exact arithmetic;
//   * Guo terms of a pair from G_i+G_j = 18 w (c.F)(c.u) + 18 w uF and G_i-G_j = 6 w (c.F).
// Results agree with the exact form to FP32 rounding (tests hold rho/u to 1e-5 relative).
#pragma once
#include "lbm_scheme.cuh"

namespace fx3d {

template<int ST> struct RawCodec; // storage value <-> FP32 in storage units
template<> struct RawCodec<ST_FP32> {
	static constexpr float K = 1.0f;
	static __device__ __forceinline__ float decode(const float x) { return x; }
	static __device__ __forceinline__ float encode(const float x) { return x; }
};
template<> struct RawCodec<ST_FP16S> {
	static constexpr float K = 32768.0f; // the FP16S range shift (src/lbm.cpp:411-414)
	static __device__ __forceinline__ float decode(const uint16_t h) { return __half2float(__ushort_as_half(h)); }
	static __device__ __forceinline__ uint16_t encode(const float x) { return __half_as_ushort(__float2half_rn(x)); }
};
// FP16C (1-4-11, exponent bias 15, src/kernel.cpp:848-859) with the shift trick of IEEE half: the 15
// magnitude bits moved up by 12 form, read as an FP32 bit pattern, the value times 2^-112 for normal
// and denormal codes alike (denormal codes become FP32 denormals), so decoding is a shift and one
// multiply by 2^112 (exact, and equal to the reference's decoder). Encoding multiplies by 2^-112 and
// rounds the 12 dropped bits half up like the reference; for normal values that is the reference's
// encoder bit for bit, for denormal codes it may differ in the last unit.
template<> struct RawCodec<ST_FP16C> {
	static constexpr float K = 1.0f;
	static __device__ __forceinline__ float decode(const uint16_t h) {
		const uint32_t x = h;
		return __uint_as_float(((x&0x7FFFu)<<12)|((x&0x8000u)<<16))*0x1p112f;
	}
	static __device__ __forceinline__ uint16_t encode(const float v) {
		const uint32_t b = __float_as_uint(v);
		const uint32_t y = __float_as_uint(__uint_as_float(b&0x7FFFFFFFu)*0x1p-112f);
		return (uint16_t)((((y+0x800u)>>12)&0x7FFFu)|((b>>16)&0x8000u));
	}
};

// signed sum of v_d over the non-zero components of c_I (any order: fast mode); starts from the
// first non-zero term, since adding to 0.0f cannot be folded away under IEEE rules
template<int I> __device__ __forceinline__ float csum_fast(const float vx, const float vy, const float vz) {
	constexpr int a = vs_c(0, I), b = vs_c(1, I), c = vs_c(2, I);
	const float tx = a>0 ? vx : -vx, ty = b>0 ? vy : -vy, tz = c>0 ? vz : -vz;
	if constexpr(a!=0 && b!=0 && c!=0) return tx+ty+tz;
	else if constexpr(a!=0 && b!=0) return tx+ty;
	else if constexpr(a!=0 && c!=0) return tx+tz;
	else if constexpr(b!=0 && c!=0) return ty+tz;
	else if constexpr(a!=0) return tx;
	else if constexpr(b!=0) return ty;
	else return tz;
}

// accumulate d with sign c into an accumulator that starts unset (no addition to 0.0f)
template<int C> __device__ __forceinline__ void acc_signed(float& m, bool& set, const float d) {
	if constexpr(C!=0) {
		const float t = C>0 ? d : -d;
		m = set ? m+t : t;
		set = true;
	}
}

// S = K*(rho-1) = sum of the shifted DDFs and the momentum (storage units), from pair sums and pair
// differences; the shift K is added only afterwards (R = S+K), so S keeps full precision
template<int Q> __device__ __forceinline__ void moments_fast(const float* f, float& S, float& mx, float& my, float& mz) {
	float s = f[0];
	bool sx = false, sy = false, sz = false;
	mx = 0.0f; my = 0.0f; mz = 0.0f;
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		s += f[i]+f[i+1];
		const float d = f[i]-f[i+1];
		acc_signed<vs_c(0, i)>(mx, sx, d); acc_signed<vs_c(1, i)>(my, sy, d); acc_signed<vs_c(2, i)>(mz, sz, d);
	});
	S = s;
}

// velocity of one cell (storage-unit DDFs or the preset TYPE_E values), force shifted and clamped;
// returns R = K*rho, Rm1 = K*(rho-1) and 1/R
template<int Q, int EXT, int ST> __device__ __forceinline__ void cell_rho_u_fast(const StepArgs& a, const uint64_t n, const float* f, const bool is_e,
                                                                                float& R, float& Rm1, float& inv, float& ux, float& uy, float& uz,
                                                                                float& fx, float& fy, float& fz) {
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0;
	constexpr float K = RawCodec<ST>::K;
	const uint64_t N = a.g.N;
	if(is_e) {
		R = K*a.rho[n]; Rm1 = R-K; inv = __frcp_rn(R);
		ux = a.u[n]; uy = a.u[N+n]; uz = a.u[2ull*N+n];
	} else {
		float mx, my, mz;
		moments_fast<Q>(f, Rm1, mx, my, mz);
		R = Rm1+K;
		inv = __frcp_rn(R);
		// u = m/R from the reciprocal plus one Newton correction (u += (m - u R)/R)
		ux = mx*inv; uy = my*inv; uz = mz*inv;
		ux = fmaf(fmaf(-ux, R, mx), inv, ux); uy = fmaf(fmaf(-uy, R, my), inv, uy); uz = fmaf(fmaf(-uz, R, mz), inv, uz);
	}
	fx = a.fx; fy = a.fy; fz = a.fz;
	if constexpr(FF) { fx += a.F[n]; fy += a.F[N+n]; fz += a.F[2ull*N+n]; }
	if constexpr(VF) {
		const float rho2 = (0.5f*K)*inv; // F/(2 rho) with rho = R/K
		ux = clampc(fmaf(fx, rho2, ux)); uy = clampc(fmaf(fy, rho2, uy)); uz = clampc(fmaf(fz, rho2, uz));
	} else {
		ux = clampc(ux); uy = clampc(uy); uz = clampc(uz);
	}
}

// collision of all directions in place, DDFs in storage units (K scaling); IS_E: TYPE_E cell (f = feq)
template<int Q, bool TRT, bool VF, int ST, bool IS_E> __device__ __forceinline__ void collide_fast_t(float* f, const float R, const float Rm1, const float ux,
                                                                                                 const float uy, const float uz, const float fx, const float fy,
                                                                                                 const float fz, const StepArgs& a) {
	constexpr float K = RawCodec<ST>::K;
	const float c3 = -3.0f*fmaf(ux, ux, fmaf(uy, uy, uz*uz));
	const float ux3 = 3.0f*ux, uy3 = 3.0f*uy, uz3 = 3.0f*uz;
	const float fxK = K*fx, fyK = K*fy, fzK = K*fz; // Guo terms in storage units
	const float uF = VF ? -THIRD*fmaf(ux, fxK, fmaf(uy, fyK, uz*fzK)) : 0.0f;
	{ // center
		const float fe = vs_w<Q>(0)*fmaf(R, 0.5f*c3, Rm1);
		if constexpr(IS_E) f[0] = fe;
		else {
			const float d0 = fe-f[0];
			float g0 = !TRT ? fmaf(a.w, d0, f[0]) : fmaf(2.0f*a.hp, d0, f[0]);
			if constexpr(VF) g0 = fmaf(!TRT ? a.c_tau : 2.0f*a.c_taup, (9.0f*vs_w<Q>(0))*uF, g0);
			f[0] = g0;
		}
	}
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const float wi = vs_w<Q>(i);
		const float rw = wi*R;
		const float uk = csum_fast<i>(ux3, uy3, uz3);
		const float base = fmaf(0.5f*rw, fmaf(uk, uk, c3), wi*Rm1);
		const float ea = fmaf(rw, uk, base), eb = fmaf(-rw, uk, base);
		if constexpr(IS_E) { f[i] = ea; f[i+1] = eb; }
		else {
			const float da = ea-f[i], db = eb-f[i+1];
			float na, nb;
			if constexpr(!TRT) { na = fmaf(a.w, da, f[i]); nb = fmaf(a.w, db, f[i+1]); }
			else {
				const float t = a.hp*(da+db), dd = da-db;
				na = f[i]+fmaf(a.hm, dd, t); nb = f[i+1]+fmaf(-a.hm, dd, t);
			}
			if constexpr(VF) {
				const float cf = csum_fast<i>(fxK, fyK, fzK);
				const float gs = (18.0f*wi)*fmaf(cf, uk*THIRD, uF); // G_i + G_j  (c.u = uk/3)
				const float gd = (6.0f*wi)*cf;                     // G_i - G_j
				if constexpr(!TRT) { na = fmaf(0.5f*a.c_tau, gs+gd, na); nb = fmaf(0.5f*a.c_tau, gs-gd, nb); }
				else { na += fmaf(a.c_taup, gs, a.c_taum*gd); nb += fmaf(a.c_taup, gs, -a.c_taum*gd); }
			}
			f[i] = na; f[i+1] = nb;
		}
	});
}
template<int Q, bool TRT, bool VF, int ST> __device__ __forceinline__ void collide_fast(float* f, const float R, const float Rm1, const float ux, const float uy,
                                                                                      const float uz, const float fx, const float fy, const float fz,
                                                                                      const bool is_e, const StepArgs& a) {
	if(is_e) collide_fast_t<Q, TRT, VF, ST, true>(f, R, Rm1, ux, uy, uz, fx, fy, fz, a);
	else collide_fast_t<Q, TRT, VF, ST, false>(f, R, Rm1, ux, uy, uz, fx, fy, fz, a);
}

} // namespace fx3d
