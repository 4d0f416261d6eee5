// Fast arithmetic for the LBM cell step: the reference's scheme (src/kernel.cpp:1454-1636) with the
// freedoms its own GPU build takes (-cl-mad-enable: multiply-adds fused; OpenCL's default non-IEEE
// division) plus exact algebraic regroupings, at about a third of the issued instructions of the
// operation-for-operation form in lbm_scheme.cuh:
//   * DDFs stay in storage units: FP16S values are used as stored (2^15 times the DDF), so loads and
//     stores are a bare conversion; the density carries the same factor K (R = K*rho), the Guo force
//     terms are scaled by K and the velocity, a ratio, needs no rescaling;
//   * one reciprocal of R per cell instead of four divisions (hardware approximation plus one
//     Newton step; the velocity gets one more Newton correction); rho-1 is the plain sum of the shifted DDFs (the shift is added after summing, as
//     the reference intends with DDF shifting);
//   * moments from pair sums and pair differences (f_i+f_j, f_i-f_j for opposite i,j);
//   * equilibrium of an opposite pair from one shared base term: feq_{i,j} = base +- rho w_i u_k;
//   * TRT in symmetric / antisymmetric parts: with d = feq - f,
//     f_i += hp (d_i+d_j) + hm (d_i-d_j) + F_i,  f_j += hp (d_i+d_j) - hm (d_i-d_j) + F_j,
//     which equals the reference's fma(0.5wp, ..., fma(0.5wm, ..., f+Fin)) in exact arithmetic;
//   * Guo terms of a pair from G_i+G_j = 18 w (c.F)(c.u) + 18 w uF and G_i-G_j = 6 w (c.F).
//
// The arithmetic is written once for a value type V: float (one cell) or float2 (two cells, issued
// as the packed FP32 instructions of sm_100 and later: __fadd2_rn, __fmul2_rn, __ffma2_rn). Every
// operation is explicitly rounded and the packed forms round each component exactly as the scalar
// ones. ptxas fuses a packed multiply whose only use is a packed add into a packed multiply-add
// even with explicit .rn modifiers (the scalar __fmul_rn/__fadd_rn are never fused), so no
// multiply here feeds an add directly: each such pair is written as one fma. One cell then gives
// bit-identical results in either form.
// Results agree with the exact scheme to FP32 rounding (tests hold rho/u to 1e-5 relative).
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
// encoder bit for bit, for denormal codes it may differ in the last unit. Decoding then encoding a
// code gives the code back.
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

// The collision of an opposite pair in pair-sum / pair-difference form (see LaneRates) for 16-bit
// storage, where it saves about a third of the pair's packed instructions and the storage rounding
// dominates the error; FP32 storage keeps the per-direction form, whose error against the FP64
// scheme is an order of magnitude lower (the pair-sum form rounds the large parts twice per step).
template<int ST> __host__ __device__ constexpr bool pair_sum_form() { return ST!=ST_FP32; }

// ---------------------------------------------------------------- one cell (float) or two (float2)
__device__ __forceinline__ float v_add(const float a, const float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float v_sub(const float a, const float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float v_mul(const float a, const float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float v_fma(const float a, const float b, const float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float v_neg(const float a) { return -a; }
__device__ __forceinline__ float2 v_add(const float2 a, const float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 v_mul(const float2 a, const float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 v_neg(const float2 a) { return make_float2(-a.x, -a.y); }
// a-b as fma(b, -1, a): the product is exact, so this is a-b rounded once, with no separate negation
__device__ __forceinline__ float2 v_sub(const float2 a, const float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 v_fma(const float2 a, const float2 b, const float2 c) { return __ffma2_rn(a, b, c); }
template<class V> __device__ __forceinline__ V v_set(const float s);
template<> __device__ __forceinline__ float v_set<float>(const float s) { return s; }
template<> __device__ __forceinline__ float2 v_set<float2>(const float s) { return make_float2(s, s); }
// a per-component function (reciprocal, clamp)
template<class F> __device__ __forceinline__ float v_map(const float a, F&& f) { return f(a); }
template<class F> __device__ __forceinline__ float2 v_map(const float2 a, F&& f) { return make_float2(f(a.x), f(a.y)); }
// per-component choice: b where the lane's flag is set (flags: bool for float, Bool2 for float2)
struct Bool2 { bool x, y; };
__device__ __forceinline__ float v_pick(const float a, const float b, const bool s) { return s ? b : a; }
__device__ __forceinline__ float2 v_pick(const float2 a, const float2 b, const Bool2 s) { return make_float2(s.x ? b.x : a.x, s.y ? b.y : a.y); }
// per-cell float fields (rho, u, F) at cell n (and n+1 for float2; n even, so 8-byte aligned)
__device__ __forceinline__ void v_load(float& v, const float* p) { v = *p; }
__device__ __forceinline__ void v_load(float2& v, const float* p) { v = *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ float v_clampc(const float x) { return fminf(fmaxf(x, -DEF_C), DEF_C); }
template<class V> __device__ __forceinline__ V v_clamp(const V x) { return v_map(x, [](const float t) { return v_clampc(t); }); }
// 1/x: the hardware reciprocal approximation (max. 1 ulp) refined by one Newton step r += r (1 - x r),
// the Newton step in V arithmetic (x is a density of order 1, or 2^15 in FP16S storage units)
template<class V> __device__ __forceinline__ V v_rcp(const V x) {
	const V r = v_map(x, [](const float t) { float y; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(t)); return y; });
	return v_fma(r, v_fma(v_neg(x), r, v_set<V>(1.0f)), r);
}

// signed sum of v_d over the non-zero components of c_I (any order: fast mode): starts from the first
// component with a positive sign and adds or subtracts the others in component order, so that no
// negation is needed (every odd direction of D3Q19/D3Q27 has a positive component); adding to 0
// cannot be folded away under IEEE rules, so no zero start either
template<int I> __host__ __device__ constexpr int csum_first() { return vs_c(0, I)>0 ? 0 : vs_c(1, I)>0 ? 1 : vs_c(2, I)>0 ? 2 : -1; }
template<int I, class V> __device__ __forceinline__ V csum_v(const V vx, const V vy, const V vz) {
	const V v[3] = {vx, vy, vz};
	if constexpr(csum_first<I>()<0) { // no positive component: -(sum of the magnitudes)
		V s = v_set<V>(0.0f);
		bool set = false;
		Unroll<0, 3, 1>::run([&](auto dc) {
			constexpr int d = decltype(dc)::value;
			if constexpr(vs_c(d, I)!=0) { s = set ? v_add(s, v[d]) : v[d]; set = true; }
		});
		return v_neg(s);
	} else {
		V s = v[csum_first<I>()];
		Unroll<0, 3, 1>::run([&](auto dc) {
			constexpr int d = decltype(dc)::value;
			if constexpr(d!=csum_first<I>() && vs_c(d, I)!=0) s = vs_c(d, I)>0 ? v_add(s, v[d]) : v_sub(s, v[d]);
		});
		return s;
	}
}

// accumulate d with sign C into an accumulator that starts unset (no addition to 0)
template<int C, class V> __device__ __forceinline__ void acc_signed(V& m, bool& set, const V d) {
	if constexpr(C!=0) {
		if(set) m = C>0 ? v_add(m, d) : v_sub(m, d);
		else m = C>0 ? d : v_neg(d);
		set = true;
	}
}

// S = K*(rho-1) = sum of the shifted DDFs and the momentum (storage units), from pair sums and pair
// differences; the shift K is added only afterwards (R = S+K), so S keeps full precision. SD: the
// pair sums and differences replace the pair's DDFs in f (f[i] = f_i + f_j, f[i+1] = f_i - f_j for
// the opposite pair (i, j = i+1)), and the collision works on them directly.
template<int Q, bool SD, class V> __device__ __forceinline__ void moments_v(V* f, V& S, V& mx, V& my, V& mz) {
	V s = f[0];
	bool sx = false, sy = false, sz = false;
	mx = v_set<V>(0.0f); my = v_set<V>(0.0f); mz = v_set<V>(0.0f);
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const V p = v_add(f[i], f[i+1]), d = v_sub(f[i], f[i+1]);
		s = v_add(s, p);
		acc_signed<vs_c(0, i)>(mx, sx, d); acc_signed<vs_c(1, i)>(my, sy, d); acc_signed<vs_c(2, i)>(mz, sz, d);
		if constexpr(SD) { f[i] = p; f[i+1] = d; }
	});
	S = s;
}

// velocity of the cell(s) (storage-unit DDFs, or the preset rho/u of TYPE_E cells), force shifted and
// clamped; R = K*rho, Rm1 = K*(rho-1), inv = 1/R. is_e: per-lane TYPE_E flags, any_e: any of them.
// For 16-bit storage the opposite pairs of f leave in pair-sum / pair-difference form (moments_v),
// except for a single TYPE_E cell (float), whose collision does not read f.
template<int Q, int EXT, int ST, class V, class M> __device__ __forceinline__ void cell_rho_u_v(const StepArgs& a, const uint64_t n, V* f, const M is_e,
                                                                                            const bool any_e, V& R, V& Rm1, V& inv, V& ux, V& uy, V& uz,
                                                                                            V& fx, V& fy, V& fz) {
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0;
	constexpr float K = RawCodec<ST>::K;
	const uint64_t N = a.g.N;
	auto from_fields = [&](V& R_, V& Rm1_, V& inv_, V& ux_, V& uy_, V& uz_) {
		V r;
		v_load(r, a.rho+n);
		R_ = v_mul(v_set<V>(K), r); Rm1_ = v_fma(v_set<V>(K), r, v_set<V>(-K)); inv_ = v_rcp(R_);
		v_load(ux_, a.u+n); v_load(uy_, a.u+N+n); v_load(uz_, a.u+2ull*N+n);
	};
	auto from_ddfs = [&]() {
		V mx, my, mz;
		moments_v<Q, pair_sum_form<ST>()>(f, Rm1, mx, my, mz);
		R = v_add(Rm1, v_set<V>(K));
		inv = v_rcp(R);
		// u = m/R from the reciprocal plus one Newton correction (u += (m - u R)/R)
		ux = v_mul(mx, inv); uy = v_mul(my, inv); uz = v_mul(mz, inv);
		const V nR = v_neg(R); // fma(u, -R, m) == fma(-u, R, m)
		ux = v_fma(v_fma(ux, nR, mx), inv, ux); uy = v_fma(v_fma(uy, nR, my), inv, uy); uz = v_fma(v_fma(uz, nR, mz), inv, uz);
	};
	if constexpr(std::is_same<V, float>::value) {
		if(is_e) from_fields(R, Rm1, inv, ux, uy, uz);
		else from_ddfs();
	} else {
		from_ddfs();
		if(any_e) {
			V R2, Rm12, inv2, ux2, uy2, uz2;
			from_fields(R2, Rm12, inv2, ux2, uy2, uz2);
			R = v_pick(R, R2, is_e); Rm1 = v_pick(Rm1, Rm12, is_e); inv = v_pick(inv, inv2, is_e);
			ux = v_pick(ux, ux2, is_e); uy = v_pick(uy, uy2, is_e); uz = v_pick(uz, uz2, is_e);
		}
	}
	fx = v_set<V>(a.fx); fy = v_set<V>(a.fy); fz = v_set<V>(a.fz);
	if constexpr(FF) {
		V Fx, Fy, Fz;
		v_load(Fx, a.F+n); v_load(Fy, a.F+N+n); v_load(Fz, a.F+2ull*N+n);
		fx = v_add(fx, Fx); fy = v_add(fy, Fy); fz = v_add(fz, Fz);
	}
	if constexpr(VF) {
		const V rho2 = v_mul(v_set<V>(0.5f*K), inv); // F/(2 rho) with rho = R/K
		ux = v_clamp(v_fma(fx, rho2, ux)); uy = v_clamp(v_fma(fy, rho2, uy)); uz = v_clamp(v_fma(fz, rho2, uz));
	} else {
		ux = v_clamp(ux); uy = v_clamp(uy); uz = v_clamp(uz);
	}
}

// collision rates as values of V: uniform (the host's rates) or per cell (SUBGRID)
template<class V> struct VRates {
	V w, hp, hm, nhm, half_c_tau, c_taup, c_taum; // per-direction form
	V cs, cb, cd, cu, fp, fm; // pair-sum form: 1/2 - hp, 2 hp, 1/2 - hm, 2 hm, Guo factors of G_i + G_j and G_i - G_j
	V rest_rate, rest_force; // the rest direction's relaxation and Guo factors (SRT: w, c_tau; TRT: 2 hp, 2 c_taup)
};
// Rates of the pair-sum / pair-difference form of the collision. With S = f_i + f_j, D = f_i - f_j
// for an opposite pair, feq_{i,j} = base +- rw uk and d = feq - f, the TRT update
// f_i += hp (d_i + d_j) + hm (d_i - d_j) is, with f_i = (S + D)/2,
//   f_i' = P + M, f_j' = P - M,  P = (1/2 - hp) S + 2 hp base,  M = (1/2 - hm) D + 2 hm rw uk,
// and SRT is the case hp = hm = w/2. The Guo terms add c+ (G_i + G_j) to P and c- (G_i - G_j) to M
// (SRT: c+ = c- = c_tau/2).
struct LaneRates { float w, hp, hm, nhm, half_c_tau, c_taup, c_taum, cs, cb, cd, cu, fp, fm, rest_rate, rest_force; };
template<bool TRT> __device__ __forceinline__ LaneRates lane_rates(const float w, const float hp, const float hm, const float c_tau, const float c_taup,
                                                                 const float c_taum) {
	const float hm_ = TRT ? hm : hp; // hp = w/2
	return LaneRates{w, hp, hm, -hm, 0.5f*c_tau, c_taup, c_taum,
	                 __fsub_rn(0.5f, hp), __fadd_rn(hp, hp), __fsub_rn(0.5f, hm_), __fadd_rn(hm_, hm_), TRT ? c_taup : 0.5f*c_tau, TRT ? c_taum : 0.5f*c_tau,
	                 !TRT ? w : 2.0f*hp, !TRT ? c_tau : 2.0f*c_taup};
}
template<class V> __device__ __forceinline__ VRates<V> v_rates(const LaneRates& a);
template<> __device__ __forceinline__ VRates<float> v_rates<float>(const LaneRates& a) {
	return VRates<float>{a.w, a.hp, a.hm, a.nhm, a.half_c_tau, a.c_taup, a.c_taum, a.cs, a.cb, a.cd, a.cu, a.fp, a.fm, a.rest_rate, a.rest_force};
}
__device__ __forceinline__ VRates<float2> v_rates2(const LaneRates& a, const LaneRates& b) {
	auto p = [](const float x, const float y) { return make_float2(x, y); };
	return VRates<float2>{p(a.w, b.w), p(a.hp, b.hp), p(a.hm, b.hm), p(a.nhm, b.nhm), p(a.half_c_tau, b.half_c_tau), p(a.c_taup, b.c_taup),
	                      p(a.c_taum, b.c_taum), p(a.cs, b.cs), p(a.cb, b.cb), p(a.cd, b.cd), p(a.cu, b.cu), p(a.fp, b.fp), p(a.fm, b.fm),
	                      p(a.rest_rate, b.rest_rate), p(a.rest_force, b.rest_force)};
}
template<> __device__ __forceinline__ VRates<float2> v_rates<float2>(const LaneRates& a) { return v_rates2(a, a); }
// SUBGRID rates of one cell from its stress tensor H (storage units) and 1/R, with the hardware
// approximations of sqrt and 1/x: tau = (tau0 + sqrt(tau0^2 + 0.76421222 sqrt(H:H)/rho))/2,
// w = 1/tau (the reference's 2/(tau0 + ...)), TRT: wm = 1/(0.1875/(tau - 1/2) + 1/2)
__device__ __forceinline__ float approx_rcp(const float x) { float y; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
__device__ __forceinline__ float approx_sqrt(const float x) { float y; asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x)); return y; }
template<bool TRT> __device__ __forceinline__ LaneRates subgrid_lane_rates(const float tau0, const float* H, const float inv) {
	const float diag = __fmaf_rn(H[0], H[0], __fmaf_rn(H[1], H[1], __fmul_rn(H[2], H[2])));
	const float Qs = __fmaf_rn(2.0f, __fmaf_rn(H[3], H[3], __fmaf_rn(H[4], H[4], __fmul_rn(H[5], H[5]))), diag);
	const float S = approx_sqrt(__fmaf_rn(__fmul_rn(0.76421222f, approx_sqrt(Qs)), inv, __fmul_rn(tau0, tau0)));
	const float tau = __fmul_rn(0.5f, __fadd_rn(tau0, S));
	const float w = approx_rcp(tau);
	const float wm = TRT ? approx_rcp(__fmaf_rn(0.1875f, approx_rcp(__fsub_rn(tau, 0.5f)), 0.5f)) : w;
	return lane_rates<TRT>(w, __fmul_rn(0.5f, w), __fmul_rn(0.5f, wm), __fmaf_rn(w, -0.5f, 1.0f), __fmaf_rn(w, -0.25f, 0.5f), __fmaf_rn(wm, -0.25f, 0.5f));
}
// stress contribution of the opposite pair (I, I+1): both directions share c c^T, so their pair sum
// of non-equilibrium parts s enters once
template<int I, class V> __device__ __forceinline__ void stress_add_v(V* H, const V s) {
	constexpr int cx = vs_c(0, I), cy = vs_c(1, I), cz = vs_c(2, I);
	if constexpr(cx!=0) H[0] = v_add(H[0], s);
	if constexpr(cy!=0) H[1] = v_add(H[1], s);
	if constexpr(cz!=0) H[2] = v_add(H[2], s);
	if constexpr(cx!=0 && cy!=0) H[3] = cx*cy>0 ? v_add(H[3], s) : v_sub(H[3], s);
	if constexpr(cx!=0 && cz!=0) H[4] = cx*cz>0 ? v_add(H[4], s) : v_sub(H[4], s);
	if constexpr(cy!=0 && cz!=0) H[5] = cy*cz>0 ? v_add(H[5], s) : v_sub(H[5], s);
}

// collision of all directions in place, DDFs in storage units (K scaling); for 16-bit storage the
// opposite pairs of f are in pair-sum / pair-difference form on entry (moments_v), and f leaves as
// DDFs in either case. EMODE 0: no TYPE_E
// cell; 1: the (single) cell is TYPE_E (f = feq, f not read); 2: mixed lanes, TYPE_E lanes picked by
// is_e. SG: the relaxation rate of each cell from the Smagorinsky-Lilly model
// (src/kernel.cpp:1579-1593); the stress tensor comes from the pair sums S - (feq_i + feq_j),
// feq_i + feq_j = 2 base, and the rate itself from the same scalar operations in either form of V
// (sqrt(H:H)/rho is the same in storage units, H and R both carry the factor K).
template<int Q, bool TRT, bool VF, int ST, int EMODE, class V, class M, bool SG = false> __device__ __forceinline__ void collide_v(V* f, const V R, const V Rm1,
                                                                                                             const V ux, const V uy, const V uz,
                                                                                                             const V fx, const V fy, const V fz,
                                                                                                             const M is_e, const StepArgs& a) {
	constexpr float K = RawCodec<ST>::K;
	constexpr bool SD = pair_sum_form<ST>();
	const V c3 = v_mul(v_set<V>(-3.0f), v_fma(ux, ux, v_fma(uy, uy, v_mul(uz, uz))));
	const V ux3 = v_mul(v_set<V>(3.0f), ux), uy3 = v_mul(v_set<V>(3.0f), uy), uz3 = v_mul(v_set<V>(3.0f), uz);
	V fxK = fx, fyK = fy, fzK = fz, uF = v_set<V>(0.0f); // Guo terms in storage units
	if constexpr(VF) {
		fxK = v_mul(v_set<V>(K), fx); fyK = v_mul(v_set<V>(K), fy); fzK = v_mul(v_set<V>(K), fz);
		uF = v_mul(v_set<V>(-THIRD), v_fma(ux, fxK, v_fma(uy, fyK, v_mul(uz, fzK))));
	}
	// w R / 2 and w (R-K) once per weight class (straight, edge, corner directions): base = w R/2 (uk^2 + c3) + w (R-K)
	constexpr int NC = Q==27 ? 3 : 2;
	V hrc[NC], wmc[NC];
	#pragma unroll
	for(int c=0; c<NC; c++) {
		const float wc = vs_w<Q>(c==0 ? 1 : c==1 ? 7 : 19);
		hrc[c] = v_mul(v_set<V>(0.5f*wc), R); wmc[c] = v_mul(v_set<V>(wc), Rm1);
	}
	auto base_of = [&](auto ic, V& uk) { // the shared equilibrium term of pair (i, i+1)
		constexpr int i = decltype(ic)::value;
		constexpr int c = (vs_c(0, i)!=0)+(vs_c(1, i)!=0)+(vs_c(2, i)!=0)-1;
		uk = csum_v<i>(ux3, uy3, uz3);
		return v_fma(hrc[c], v_fma(uk, uk, c3), wmc[c]);
	};
	VRates<V> r;
	if constexpr(SG) {
		V H[6];
		#pragma unroll
		for(int k=0; k<6; k++) H[k] = v_set<V>(0.0f);
		Unroll<1, Q, 2>::run([&](auto ic) {
			constexpr int i = decltype(ic)::value;
			V uk;
			const V base = base_of(ic, uk);
			stress_add_v<i>(H, v_sub(SD ? f[i] : v_add(f[i], f[i+1]), v_add(base, base)));
		});
		const float tau0 = __fdiv_rn(1.0f, a.w); // uniform
		const V inv = v_rcp(R);
		if constexpr(std::is_same<V, float>::value) {
			r = v_rates<V>(subgrid_lane_rates<TRT>(tau0, H, inv));
		} else {
			const float Ha[6] = {H[0].x, H[1].x, H[2].x, H[3].x, H[4].x, H[5].x}, Hb[6] = {H[0].y, H[1].y, H[2].y, H[3].y, H[4].y, H[5].y};
			r = v_rates2(subgrid_lane_rates<TRT>(tau0, Ha, inv.x), subgrid_lane_rates<TRT>(tau0, Hb, inv.y));
		}
	} else {
		r = v_rates<V>(lane_rates<TRT>(a.w, a.hp, a.hm, a.c_tau, a.c_taup, a.c_taum));
	}
	{ // center: feq_0 = w_0 X; its difference to f_0 as one fused operation
		const V X = v_fma(R, v_mul(v_set<V>(0.5f), c3), Rm1), w0 = v_set<V>(vs_w<Q>(0));
		if constexpr(EMODE==1) f[0] = v_mul(w0, X);
		else {
			const V d0 = v_fma(w0, X, v_neg(f[0]));
			V g0 = v_fma(r.rest_rate, d0, f[0]);
			if constexpr(VF) g0 = v_fma(r.rest_force, v_mul(v_set<V>(9.0f*vs_w<Q>(0)), uF), g0);
			if constexpr(EMODE==2) f[0] = v_pick(g0, v_mul(w0, X), is_e); else f[0] = g0;
		}
	}
	// 2 hm w R per weight class (the factor of uk in M)
	V cuc[NC];
	if constexpr(SD && EMODE!=1) {
		const V cuR = v_mul(r.cu, R);
		#pragma unroll
		for(int c=0; c<NC; c++) cuc[c] = v_mul(v_set<V>(vs_w<Q>(c==0 ? 1 : c==1 ? 7 : 19)), cuR);
	}
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		constexpr int c = (vs_c(0, i)!=0)+(vs_c(1, i)!=0)+(vs_c(2, i)!=0)-1;
		const float wi = vs_w<Q>(i);
		V uk;
		const V base = base_of(ic, uk);
		if constexpr(EMODE==1) { // f = feq = base +- w R uk
			const V rw = v_mul(v_set<V>(wi), R);
			f[i] = v_fma(rw, uk, base); f[i+1] = v_fma(v_neg(rw), uk, base);
		} else if constexpr(!SD) { // per direction: d = feq - f
			const V rw = v_mul(v_set<V>(wi), R);
			const V ea = v_fma(rw, uk, base), eb = v_fma(v_neg(rw), uk, base);
			const V da = v_sub(ea, f[i]), db = v_sub(eb, f[i+1]);
			V na, nb;
			if constexpr(!TRT) { na = v_fma(r.w, da, f[i]); nb = v_fma(r.w, db, f[i+1]); }
			else {
				const V t = v_mul(r.hp, v_add(da, db)), dd = v_sub(da, db);
				na = v_add(f[i], v_fma(r.hm, dd, t)); nb = v_add(f[i+1], v_fma(r.nhm, dd, t));
			}
			if constexpr(VF) {
				const V cf = csum_v<i>(fxK, fyK, fzK);
				const V Y = v_fma(cf, v_mul(uk, v_set<V>(THIRD)), uF);
				const V gd = v_mul(v_set<V>(6.0f*wi), cf);                     // G_i - G_j
				if constexpr(!TRT) { // G_i = gs + gd and G_j = gs - gd, each one fused operation
					na = v_fma(r.half_c_tau, v_fma(v_set<V>(18.0f*wi), Y, gd), na);
					nb = v_fma(r.half_c_tau, v_fma(v_set<V>(18.0f*wi), Y, v_neg(gd)), nb);
				} else {
					const V gs = v_mul(v_set<V>(18.0f*wi), Y);                 // G_i + G_j  (c.u = uk/3)
					const V m = v_mul(r.c_taum, gd);
					na = v_add(na, v_fma(r.c_taup, gs, m)); nb = v_add(nb, v_fma(r.c_taup, gs, v_neg(m)));
				}
			}
			if constexpr(EMODE==2) { f[i] = v_pick(na, ea, is_e); f[i+1] = v_pick(nb, eb, is_e); }
			else { f[i] = na; f[i+1] = nb; }
		} else {
			V P = v_fma(r.cs, f[i], v_mul(r.cb, base));
			V Mn = v_fma(r.cd, f[i+1], v_mul(cuc[c], uk));
			if constexpr(VF) {
				const V cf = csum_v<i>(fxK, fyK, fzK);
				const V Y = v_fma(cf, v_mul(uk, v_set<V>(THIRD)), uF);
				P = v_fma(r.fp, v_mul(v_set<V>(18.0f*wi), Y), P);          // G_i + G_j = 18 w Y  (c.u = uk/3)
				Mn = v_fma(r.fm, v_mul(v_set<V>(6.0f*wi), cf), Mn);         // G_i - G_j = 6 w (c.F)
			}
			const V na = v_add(P, Mn), nb = v_sub(P, Mn);
			if constexpr(EMODE==2) {
				const V rw = v_mul(v_set<V>(wi), R);
				f[i] = v_pick(na, v_fma(rw, uk, base), is_e); f[i+1] = v_pick(nb, v_fma(v_neg(rw), uk, base), is_e);
			} else { f[i] = na; f[i+1] = nb; }
		}
	});
}

// ---------------------------------------------------------------- one cell (the scalar kernels)
template<int Q, int EXT, int ST> __device__ __forceinline__ void cell_rho_u_fast(const StepArgs& a, const uint64_t n, float* f, const bool is_e,
                                                                                float& R, float& Rm1, float& inv, float& ux, float& uy, float& uz,
                                                                                float& fx, float& fy, float& fz) {
	cell_rho_u_v<Q, EXT, ST, float>(a, n, f, is_e, is_e, R, Rm1, inv, ux, uy, uz, fx, fy, fz);
}
template<int Q, bool TRT, bool VF, int ST, bool SG = false> __device__ __forceinline__ void collide_fast(float* f, const float R, const float Rm1, const float ux,
                                                                                                      const float uy, const float uz, const float fx, const float fy,
                                                                                                      const float fz, const bool is_e, const StepArgs& a) {
	if(is_e) collide_v<Q, TRT, VF, ST, 1, float, bool, SG>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
	else collide_v<Q, TRT, VF, ST, 0, float, bool, SG>(f, R, Rm1, ux, uy, uz, fx, fy, fz, is_e, a);
}

} // namespace fx3d
