// Discrete adjoint of stream_collide for dJ/dF, F the per-cell FORCE_FIELD force (no counterpart in
// the reference). One forward step maps the slots of each fluid cell (its Esoteric-Pull slot set at
// the step's parity) to themselves: gather g (load_f), h = Phi(g; F), scatter h (store_f). Its
// adjoint is therefore local and in place, with the forward kernel's memory pattern: lambda is read
// at the store positions (hbar), the cell takes its forward quantities from the moment checkpoint of
// step k and writes gbar = (dPhi/dg)^T hbar (+ dj_k/dg of the objective) at the load positions; solid
// cells map their slots identically. grad accumulates (dPhi/dF)^T hbar plus the objective's direct F
// term. dPhi/dg depends on g only through rho and u0 = m/rho (the collision is affine in g at fixed
// rho, u), so the 16 bytes of (rho, u) that the forward step writes per cell (its fused-fields output)
// replace the saved DDFs: with v = u0 + Ft/(2 rho) and u = clamp(v), v is inside the clamp range
// exactly when |u| < c, and then u0 = u - Ft/(2 rho) (u0 is not needed where the clamp is active).
//
// The chain (forward in lbm_scheme.cuh, reference src/kernel.cpp:1454-1636):
//   rho = sum g + 1, m = sum c g, u0 = m/rho, v = u0 + Ft/(2 rho), u = clamp(v), Ft = (fx,fy,fz) + F
//   feq_i = w_i (rho (0.5 (uk^2 + c3) + uk) + rho - 1), uk = 3 c_i.u, c3 = -3|u|^2
//   G_i = 9 w_i ((c_i.Ft)(c_i.u + 1/3) - u.Ft/3)                      (Guo forcing)
//   SRT: h_i = (1-w) g_i + w feq_i + c_tau G_i
//   TRT: h_i = g_i + hp (d_i + d_j) + hm (d_i - d_j) + c_taup (G_i + G_j) + c_taum (G_i - G_j), d = feq - g
//   TYPE_E: h = feq(rho_preset, clamp(u_preset + Ft/(2 rho_preset)))
// Objectives: OBJ_KE_PLANE, the mean of 1/2 rho |u|^2 over the fluid cells of plane x = X (rho/u as
// update_fields gives them); OBJ_DRAG_X, the x force on cells with flags == marker (2 m_x).
#include "lbm_kernels.cuh"
#include "lbm_adjoint.h"

namespace fx3d {

template<int Q> struct CellState {
	float rho, u0[3], u[3], Ft[3], rho2, c3;
	bool kappa[3];
};

// forward quantities of a fluid (or TYPE_E) cell
// (1/rho from the hardware reciprocal and one Newton step: the adjoint is held to tolerances, not bits)
template<int Q, bool VF> __device__ __forceinline__ void adj_forward(const float* g, const bool is_e, const float rho_p, const float* u_p, const float* Ft,
                                                                    CellState<Q>& s) {
	float inv;
	if(is_e) {
		s.rho = rho_p;
		inv = v_rcp(rho_p);
		for(int d=0; d<3; d++) s.u0[d] = u_p[d];
	} else {
		float rho = g[0];
		#pragma unroll
		for(int i=1; i<Q; i++) rho += g[i];
		rho += 1.0f;
		s.rho = rho;
		inv = v_rcp(rho);
		s.u0[0] = momentum<Q, 0>(g)*inv; s.u0[1] = momentum<Q, 1>(g)*inv; s.u0[2] = momentum<Q, 2>(g)*inv;
	}
	s.rho2 = 0.5f*inv;
	#pragma unroll
	for(int d=0; d<3; d++) {
		s.Ft[d] = Ft[d];
		const float v = VF ? fmaf(Ft[d], s.rho2, s.u0[d]) : s.u0[d];
		s.kappa[d] = v>-DEF_C && v<DEF_C;
		s.u[d] = clampc(v);
	}
	s.c3 = -3.0f*fmaf(s.u[0], s.u[0], fmaf(s.u[1], s.u[1], s.u[2]*s.u[2]));
}

// the same for a TYPE_E cell from its presets (rho_p, u0 = u_p)
template<int Q, bool VF> __device__ __forceinline__ void adj_from_presets(const float rho_p, const float* u_p, const float* Ft, CellState<Q>& s) {
	s.rho = rho_p;
	s.rho2 = 0.5f*v_rcp(rho_p);
	#pragma unroll
	for(int d=0; d<3; d++) {
		s.u0[d] = u_p[d];
		s.Ft[d] = Ft[d];
		const float v = VF ? fmaf(Ft[d], s.rho2, s.u0[d]) : s.u0[d];
		s.kappa[d] = v>-DEF_C && v<DEF_C;
		s.u[d] = clampc(v);
	}
	s.c3 = -3.0f*fmaf(s.u[0], s.u[0], fmaf(s.u[1], s.u[1], s.u[2]*s.u[2]));
}
// the same from the fields a forward step collides a fluid cell with: rho and u = clamp(u0 + Ft/(2 rho))
template<int Q, bool VF> __device__ __forceinline__ void adj_from_fields(const float rho, const float* u, const float* Ft, CellState<Q>& s) {
	s.rho = rho;
	s.rho2 = 0.5f*v_rcp(rho);
	#pragma unroll
	for(int d=0; d<3; d++) {
		s.Ft[d] = Ft[d];
		s.u[d] = u[d];
		s.kappa[d] = u[d]>-DEF_C && u[d]<DEF_C;
		s.u0[d] = VF ? fmaf(-Ft[d], s.rho2, u[d]) : u[d];
	}
	s.c3 = -3.0f*fmaf(s.u[0], s.u[0], fmaf(s.u[1], s.u[1], s.u[2]*s.u[2]));
}

// Adjoint of the collision for one direction pair (i, i+1) (or the rest direction): from hbar the
// collision part of gbar (gi, gj), the equilibrium adjoint (fi, fj) and the Guo-term adjoint (Gi, Gj)
__device__ __forceinline__ void coll_bar_rest(const float h, const bool is_e, const bool trt, const StepArgs& a, float& gb, float& fb, float& Gb) {
	if(is_e) { gb = 0.0f; fb = h; Gb = 0.0f; }
	else if(!trt) { gb = a.omw*h; fb = a.w*h; Gb = a.c_tau*h; }
	else { gb = fmaf(-2.0f*a.hp, h, h); fb = 2.0f*a.hp*h; Gb = 2.0f*a.c_taup*h; }
}
__device__ __forceinline__ void coll_bar_pair(const float x, const float y, const bool is_e, const bool trt, const StepArgs& a,
                                              float& gi, float& gj, float& fi, float& fj, float& Gi, float& Gj) {
	if(is_e) { gi = 0.0f; gj = 0.0f; fi = x; fj = y; Gi = 0.0f; Gj = 0.0f; }
	else if(!trt) { gi = a.omw*x; gj = a.omw*y; fi = a.w*x; fj = a.w*y; Gi = a.c_tau*x; Gj = a.c_tau*y; }
	else {
		const float sp = x+y, sm = x-y;
		const float di = fmaf(a.hp, sp, a.hm*sm), dj = fmaf(a.hp, sp, -a.hm*sm);
		gi = x-di; gj = y-dj; fi = di; fj = dj;
		Gi = fmaf(a.c_taup, sp, a.c_taum*sm); Gj = fmaf(a.c_taup, sp, -a.c_taum*sm);
	}
}
// Moments over the directions of a per-direction weight v_i: m0 = sum v, m1_d = sum v c_d,
// m2 = sum v c c^T (xx, yy, zz, xy, xz, yz). The equilibrium and Guo-term adjoints of all directions
// depend on their per-direction factors only through these moments (below), so a direction costs a
// few signed additions instead of a pass through the full chain rule.
struct DirMoments {
	float m0 = 0.0f, m1[3] = {0.0f, 0.0f, 0.0f}, m2[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
};
template<int I> __device__ __forceinline__ void acc_moments(DirMoments& M, const float v) {
	constexpr int cx = vs_c(0, I), cy = vs_c(1, I), cz = vs_c(2, I);
	M.m0 += v;
	if constexpr(cx!=0) { M.m1[0] += cx>0 ? v : -v; M.m2[0] += v; }
	if constexpr(cy!=0) { M.m1[1] += cy>0 ? v : -v; M.m2[1] += v; }
	if constexpr(cz!=0) { M.m1[2] += cz>0 ? v : -v; M.m2[2] += v; }
	if constexpr(cx!=0 && cy!=0) M.m2[3] += cx*cy>0 ? v : -v;
	if constexpr(cx!=0 && cz!=0) M.m2[4] += cx*cz>0 ? v : -v;
	if constexpr(cy!=0 && cz!=0) M.m2[5] += cy*cz>0 ? v : -v;
}
__device__ __forceinline__ void m2_times(const DirMoments& M, const float* x, float* y) { // y = m2 x
	y[0] = fmaf(M.m2[0], x[0], fmaf(M.m2[3], x[1], M.m2[4]*x[2]));
	y[1] = fmaf(M.m2[3], x[0], fmaf(M.m2[1], x[1], M.m2[5]*x[2]));
	y[2] = fmaf(M.m2[4], x[0], fmaf(M.m2[5], x[1], M.m2[2]*x[2]));
}
// With fb_i = w_i feqbar_i (feq_i = w_i (rho (0.5 (uk^2 + c3) + uk) + rho - 1), uk = 3 c_i.u, c3 = -3 |u|^2):
//   rhobar += sum fb (0.5 (uk^2 + c3) + uk + 1) = 4.5 u.M2 u + (0.5 c3 + 1) M0 + 3 M1.u
//   ubar_d += rho sum fb (3 c_d (uk + 1) - 3 u_d) = rho (9 (M2 u)_d + 3 M1_d - 3 u_d M0)
// and with gb_i = 9 w_i Gbar_i (G_i = 9 w_i ((c_i.Ft)(c_i.u + 1/3) - u.Ft/3)):
//   ubar_d  += sum gb (c.Ft c_d - Ft_d/3)      = (S2 Ft)_d - Ft_d S0/3
//   Ftbar_d += sum gb (c_d (c.u + 1/3) - u_d/3) = (S2 u)_d + S1_d/3 - u_d S0/3
template<int Q> __device__ __forceinline__ void eq_moments_bar(const CellState<Q>& s, const DirMoments& M, float& rhobar, float* ubar) {
	float M2u[3];
	m2_times(M, s.u, M2u);
	const float uM2u = fmaf(s.u[0], M2u[0], fmaf(s.u[1], M2u[1], s.u[2]*M2u[2]));
	const float M1u = fmaf(M.m1[0], s.u[0], fmaf(M.m1[1], s.u[1], M.m1[2]*s.u[2]));
	rhobar += fmaf(4.5f, uM2u, fmaf(fmaf(0.5f, s.c3, 1.0f), M.m0, 3.0f*M1u));
	#pragma unroll
	for(int d=0; d<3; d++) ubar[d] = fmaf(s.rho, fmaf(9.0f, M2u[d], fmaf(3.0f, M.m1[d], -3.0f*s.u[d]*M.m0)), ubar[d]);
}
template<int Q> __device__ __forceinline__ void guo_moments_bar(const CellState<Q>& s, const DirMoments& S, float* ubar, float* Ftbar) {
	float S2F[3], S2u[3];
	m2_times(S, s.Ft, S2F);
	m2_times(S, s.u, S2u);
	#pragma unroll
	for(int d=0; d<3; d++) {
		ubar[d] += fmaf(-s.Ft[d]*THIRD, S.m0, S2F[d]);
		Ftbar[d] += fmaf(-s.u[d]*THIRD, S.m0, fmaf(S.m1[d], THIRD, S2u[d]));
	}
}

// (dh/dg)^T hbar + ke_weight * d(1/2 rho |u|^2)/dg in two passes over the direction pairs, so that
// only hbar stays live: pass 1 accumulates rhobar, ubar and Ftbar (Fbar += Ftbar); afterwards
// gbar_i = (collision part of direction i) + rhobar + c_i.mbar, recomputed per direction and handed
// to put(integral_constant<int, i>, gbar_i)
template<int Q, bool TRT, bool VF, class HB, class PUT> __device__ __forceinline__ void adj_cell(const CellState<Q>& s, const bool is_e, HB&& hbar,
                                                                                     const float ke_weight, const StepArgs& a, float* Fbar, PUT&& put) {
	float rhobar = 0.0f, ubar[3] = {0.0f, 0.0f, 0.0f}, Ftbar[3] = {0.0f, 0.0f, 0.0f};
	DirMoments M, S; // moments of w_i feqbar_i and of 9 w_i Gbar_i
	{
		float gb, fb, Gb;
		coll_bar_rest(hbar(0), is_e, TRT, a, gb, fb, Gb);
		acc_moments<0>(M, vs_w<Q>(0)*fb);
		if constexpr(VF) acc_moments<0>(S, (9.0f*vs_w<Q>(0))*Gb);
	}
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		float gi, gj, fi, fj, Gi, Gj;
		coll_bar_pair(hbar(i), hbar(i+1), is_e, TRT, a, gi, gj, fi, fj, Gi, Gj);
		const float wi = vs_w<Q>(i); // w_{i+1} = w_i
		acc_moments<i>(M, wi*fi); acc_moments<i+1>(M, wi*fj);
		if constexpr(VF) { acc_moments<i>(S, (9.0f*wi)*Gi); acc_moments<i+1>(S, (9.0f*wi)*Gj); }
	});
	eq_moments_bar<Q>(s, M, rhobar, ubar);
	if constexpr(VF) { if(!is_e) guo_moments_bar<Q>(s, S, ubar, Ftbar); }
	if(ke_weight!=0.0f && !is_e) {
		rhobar = fmaf(ke_weight*0.5f, fmaf(s.u[0], s.u[0], fmaf(s.u[1], s.u[1], s.u[2]*s.u[2])), rhobar);
		#pragma unroll
		for(int d=0; d<3; d++) ubar[d] = fmaf(ke_weight*s.rho, s.u[d], ubar[d]);
	}
	float u0bar[3], rho2bar = 0.0f;
	#pragma unroll
	for(int d=0; d<3; d++) {
		const float vbar = s.kappa[d] ? ubar[d] : 0.0f;
		u0bar[d] = vbar;
		if constexpr(VF) { Ftbar[d] = fmaf(vbar, s.rho2, Ftbar[d]); rho2bar = fmaf(vbar, s.Ft[d], rho2bar); }
	}
	float mbar[3] = {0.0f, 0.0f, 0.0f};
	if(!is_e) {
		const float inv = 2.0f*s.rho2; // 1/rho
		rhobar = fmaf(rho2bar, -2.0f*s.rho2*s.rho2, rhobar); // d(0.5/rho)/drho = -0.5/rho^2 = -2 rho2^2
		#pragma unroll
		for(int d=0; d<3; d++) { mbar[d] = u0bar[d]*inv; rhobar = fmaf(-u0bar[d]*inv, s.u0[d], rhobar); }
	} else {
		rhobar = 0.0f; // TYPE_E cells pass nothing back to g
	}
	auto finish = [&](const int cx, const int cy, const int cz, const float gcoll) {
		float gb = gcoll+rhobar;
		if(cx!=0) gb += cx>0 ? mbar[0] : -mbar[0];
		if(cy!=0) gb += cy>0 ? mbar[1] : -mbar[1];
		if(cz!=0) gb += cz>0 ? mbar[2] : -mbar[2];
		return gb;
	};
	{
		float gb, fb, Gb;
		coll_bar_rest(hbar(0), is_e, TRT, a, gb, fb, Gb);
		put(std::integral_constant<int, 0>(), finish(0, 0, 0, gb));
	}
	Unroll<1, Q, 2>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		float gi, gj, fi, fj, Gi, Gj;
		coll_bar_pair(hbar(i), hbar(i+1), is_e, TRT, a, gi, gj, fi, fj, Gi, Gj);
		put(std::integral_constant<int, i>(), finish(vs_c(0, i), vs_c(1, i), vs_c(2, i), gi));
		put(std::integral_constant<int, i+1>(), finish(vs_c(0, i+1), vs_c(1, i+1), vs_c(2, i+1), gj));
	});
	#pragma unroll
	for(int d=0; d<3; d++) Fbar[d] += Ftbar[d];
}

// OBJ_ONLY: add only the objective's dj/dg (lambda += ..., hbar = 0): the final state of the window.
// Slot positions of cell n at the step's parity (32-bit cell indices, N < 2^32): g_0 at n, g_i at
// A_i = i N + e + n, g_{i+1} at B_i = (i+1) N - e + j_i (e = 0 at odd t, N at even t); the forward
// store wrote h_i to B_i and h_{i+1} to A_i, so hbar is read there and gbar written to the load positions.
#ifndef FX3D_ADJ_MIN_BLOCKS
#define FX3D_ADJ_MIN_BLOCKS 4 // 64 registers: measured fastest on the C5 sphere channel despite spills (3 blocks: 2.62 ms per reverse step, 4: 2.48)
#endif
template<int Q, int ST, bool TRT, int EXT, bool OBJ_ONLY> __global__ void __launch_bounds__(BLOCK, FX3D_ADJ_MIN_BLOCKS) k_adjoint_step(const StepArgs a, const AdjArgs j) {
	typedef typename Codec<ST>::T T;
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0, EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint32_t n = (uint32_t)c.n;
	const uint64_t N = g.N, e = (a.t&1ull)!=0ull ? 0ull : N;
	const bool odd = (a.t&1ull)!=0ull;
	const uint8_t fl = a.flags[n];
	const uint8_t bo = fl&TYPE_BO;
	const Steps32 st(g, c.x, c.y, c.z, n);
	float* const L = j.lambda;
	auto A = [&](const int i) -> float& { return (L+((uint64_t)i*N+e))[n]; };
	auto B = [&](auto ic) -> float& { constexpr int i = decltype(ic)::value; return (L+((uint64_t)(i+1)*N-e))[st.template j<i>()]; };
	if(bo==TYPE_S||(fl&TYPE_SU)==TYPE_G) { // identity map; the drag objective lives on these cells
		if(j.obj_kind==OBJ_DRAG_X && j.obj_weight!=0.0f && fl==(uint8_t)j.marker) {
			const float w2 = 2.0f*j.obj_weight;
			Unroll<1, Q, 2>::run([&](auto ic) {
				constexpr int i = decltype(ic)::value, cx = vs_c(0, i);
				if constexpr(cx!=0) { A(i) += cx*w2; B(ic) -= cx*w2; } // g_i at A_i (c_i), g_{i+1} at B_i (-c_i)
			});
		}
		return;
	}
	const bool is_e = EQ && bo==TYPE_E;
	const bool ke = j.obj_kind==OBJ_KE_PLANE && j.obj_weight!=0.0f && c.x==j.plane_x && !is_e;
	if(OBJ_ONLY && !ke) return;
	float hb_[Q];
	if constexpr(OBJ_ONLY) {
		#pragma unroll
		for(int i=0; i<Q; i++) hb_[i] = 0.0f;
	} else {
		hb_[0] = L[n];
		Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; hb_[i] = B(ic); hb_[i+1] = A(i); });
	}
	auto hbar = [&](const int i) { return hb_[i]; };
	CellState<Q> s;
	{
		float Ft[3] = {a.fx, a.fy, a.fz};
		if constexpr(FF) { Ft[0] += a.F[n]; Ft[1] += a.F[N+n]; Ft[2] += a.F[2ull*N+n]; }
		if(is_e) { // the presets
			const float up[3] = {a.u[n], a.u[N+n], a.u[2ull*N+n]};
			adj_from_presets<Q, VF>(a.rho[n], up, Ft, s);
		} else if constexpr(OBJ_ONLY) { // the final state (no step left to write its moments): from its DDFs
			float gv[Q];
			load_f32<Q, Codec<ST>>((const T*)j.state, N, st, odd, gv);
			const float up[3] = {0.0f, 0.0f, 0.0f};
			adj_forward<Q, VF>(gv, false, 1.0f, up, Ft, s);
		} else {
			const float* M = j.moments;
			const float uf[3] = {M[N+n], M[2ull*N+n], M[3ull*N+n]};
			adj_from_fields<Q, VF>(M[n], uf, Ft, s);
		}
	}
	float Fbar[3] = {0.0f, 0.0f, 0.0f};
	// gbar of direction k goes to the load position of g_k: n (k = 0), A_i (k = i odd), B_i (k = i+1)
	adj_cell<Q, TRT, VF>(s, is_e, hbar, ke ? j.obj_weight : 0.0f, a, Fbar, [&](auto kc, const float v) {
		constexpr int k = decltype(kc)::value;
		float* p;
		if constexpr(k==0) p = &L[n];
		else if constexpr((k&1)!=0) p = &A(k);
		else p = &B(std::integral_constant<int, k-1>());
		if constexpr(OBJ_ONLY) *p += v; else *p = v;
	});
	if constexpr(FF) { j.grad[n] += Fbar[0]; j.grad[N+n] += Fbar[1]; j.grad[2ull*N+n] += Fbar[2]; }
}

// objective term of the state at one time step, FP64 partial sums per block (deterministic order)
template<int Q, int ST, int EXT> __global__ void __launch_bounds__(256) k_objective_value(const StepArgs a, const AdjArgs j, double* __restrict__ partials) {
	typedef typename Codec<ST>::T T;
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0, EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	const uint64_t N = g.N;
	double acc = 0.0;
	const bool plane = j.obj_kind==OBJ_KE_PLANE; // only the cells of plane x = plane_x, or every cell (drag)
	const uint64_t M = plane ? (j.plane_x<g.Nx ? (uint64_t)g.Ny*g.Nz : 0ull) : N;
	for(uint64_t k=(uint64_t)blockIdx.x*256u+threadIdx.x; k<M; k+=(uint64_t)gridDim.x*256u) {
		const uint64_t n = plane ? (uint64_t)j.plane_x+k*g.Nx : k;
		const uint8_t fl = a.flags[n];
		const uint64_t z = n/g.NxNy;
		const uint32_t xy = (uint32_t)(n-z*g.NxNy), y = xy/g.Nx, x = xy-y*g.Nx;
		const bool solid = (fl&TYPE_BO)==TYPE_S;
		if(j.obj_kind==OBJ_KE_PLANE) {
			if(x!=j.plane_x||solid||(fl&TYPE_SU)==TYPE_G||(EQ&&(fl&TYPE_BO)==TYPE_E)) continue;
		} else if(fl!=(uint8_t)j.marker) continue;
		const Nbr nb(g, x, y, (uint32_t)z);
		float gv[Q];
		load_f<Q, ST>((const T*)j.state, N, n, nb, (a.t&1ull)!=0ull, gv);
		if(j.obj_kind==OBJ_KE_PLANE) {
			float Ft[3] = {a.fx, a.fy, a.fz};
			if constexpr(FF) { Ft[0] += a.F[n]; Ft[1] += a.F[N+n]; Ft[2] += a.F[2ull*N+n]; }
			const float up[3] = {0.0f, 0.0f, 0.0f};
			CellState<Q> s;
			adj_forward<Q, VF>(gv, false, 1.0f, up, Ft, s);
			acc += 0.5*(double)s.rho*((double)s.u[0]*s.u[0]+(double)s.u[1]*s.u[1]+(double)s.u[2]*s.u[2]);
		} else {
			acc += 2.0*(double)momentum<Q, 0>(gv);
		}
	}
	__shared__ double sm[8];
	for(int o=16; o>0; o>>=1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
	if((threadIdx.x&31u)==0u) sm[threadIdx.x>>5] = acc;
	__syncthreads();
	if(threadIdx.x<32u) {
		double v = threadIdx.x<8u ? sm[threadIdx.x] : 0.0;
		for(int o=16; o>0; o>>=1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
		if(threadIdx.x==0u) partials[blockIdx.x] = v*(double)j.obj_weight;
	}
}
__global__ void __launch_bounds__(256) k_objective_accumulate(const double* __restrict__ partials, const int blocks, double* __restrict__ J) {
	double v = 0.0;
	for(int b=threadIdx.x; b<blocks; b+=256) v += partials[b];
	__shared__ double sm[8];
	for(int o=16; o>0; o>>=1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
	if((threadIdx.x&31u)==0u) sm[threadIdx.x>>5] = v;
	__syncthreads();
	if(threadIdx.x<32u) {
		double t = threadIdx.x<8u ? sm[threadIdx.x] : 0.0;
		for(int o=16; o>0; o>>=1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
		if(threadIdx.x==0u) *J += t;
	}
}

// ---------------------------------------------------------------- dispatch
template<int Q, int ST, bool TRT, int EXT> static void adj_launch(const StepArgs& a, const AdjArgs& j, const bool obj_only, cudaStream_t s) {
	if(obj_only) k_adjoint_step<Q, ST, TRT, EXT, true><<<cell_grid(a.g), BLOCK, 0, s>>>(a, j);
	else k_adjoint_step<Q, ST, TRT, EXT, false><<<cell_grid(a.g), BLOCK, 0, s>>>(a, j);
}
template<int Q, int ST> static bool adj_variant(const Variant& v, const StepArgs& a, const AdjArgs& j, const bool obj_only, cudaStream_t s) {
	const int e = v.ext;
	if(e==(EXT_VF|EXT_FF)) { if(v.trt) adj_launch<Q, ST, true, EXT_VF|EXT_FF>(a, j, obj_only, s); else adj_launch<Q, ST, false, EXT_VF|EXT_FF>(a, j, obj_only, s); return true; }
	if(e==(EXT_VF|EXT_FF|EXT_EQ)) { if(v.trt) adj_launch<Q, ST, true, EXT_VF|EXT_FF|EXT_EQ>(a, j, obj_only, s); else adj_launch<Q, ST, false, EXT_VF|EXT_FF|EXT_EQ>(a, j, obj_only, s); return true; }
	return false;
}
template<int Q, int ST> static bool obj_variant(const Variant& v, const StepArgs& a, const AdjArgs& j, double* partials, cudaStream_t s) {
	if(v.ext==(EXT_VF|EXT_FF)) { k_objective_value<Q, ST, EXT_VF|EXT_FF><<<REDUCE_BLOCKS, 256, 0, s>>>(a, j, partials); return true; }
	if(v.ext==(EXT_VF|EXT_FF|EXT_EQ)) { k_objective_value<Q, ST, EXT_VF|EXT_FF|EXT_EQ><<<REDUCE_BLOCKS, 256, 0, s>>>(a, j, partials); return true; }
	return false;
}
#define FX3D_BY_VARIANT(fn, ...) \
	(v.q==19 ? (v.storage==ST_FP32 ? fn<19, ST_FP32>(__VA_ARGS__) : v.storage==ST_FP16S ? fn<19, ST_FP16S>(__VA_ARGS__) : fn<19, ST_FP16C>(__VA_ARGS__)) \
	         : (v.storage==ST_FP32 ? fn<27, ST_FP32>(__VA_ARGS__) : v.storage==ST_FP16S ? fn<27, ST_FP16S>(__VA_ARGS__) : fn<27, ST_FP16C>(__VA_ARGS__)))

bool adjoint_supported(const Variant& v) { return v.ext==(EXT_VF|EXT_FF) || v.ext==(EXT_VF|EXT_FF|EXT_EQ); }

cudaError_t launch_adjoint_step(const Variant& v, const StepArgs& a, const AdjArgs& j, const bool obj_only, cudaStream_t s) {
	if(!FX3D_BY_VARIANT(adj_variant, v, a, j, obj_only, s)) return cudaErrorInvalidValue;
	return cudaGetLastError();
}
cudaError_t launch_objective_value(const Variant& v, const StepArgs& a, const AdjArgs& j, double* partials, double* J, cudaStream_t s) {
	if(!FX3D_BY_VARIANT(obj_variant, v, a, j, partials, s)) return cudaErrorInvalidValue;
	k_objective_accumulate<<<1, 256, 0, s>>>(partials, REDUCE_BLOCKS, J);
	return cudaGetLastError();
}

} // namespace fx3d
