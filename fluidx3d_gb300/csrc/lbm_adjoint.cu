// Discrete adjoint of stream_collide for dJ/dF, F the per-cell FORCE_FIELD force (no counterpart in
// the reference). One forward step maps the slots of each fluid cell (its Esoteric-Pull slot set at
// the step's parity) to themselves: gather g (load_f), h = Phi(g; F), scatter h (store_f). Its
// adjoint is therefore local and in place, with the forward kernel's memory pattern: lambda is read
// at the store positions (hbar), the cell recomputes its forward quantities from the saved state f^k
// and writes gbar = (dPhi/dg)^T hbar (+ dj_k/dg of the objective) at the load positions; solid cells
// map their slots identically. grad accumulates (dPhi/dF)^T hbar plus the objective's direct F term.
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
template<int Q, bool VF> __device__ __forceinline__ void adj_forward(const float* g, const bool is_e, const float rho_p, const float* u_p, const float* Ft,
                                                                    CellState<Q>& s) {
	if(is_e) {
		s.rho = rho_p;
		for(int d=0; d<3; d++) s.u0[d] = u_p[d];
	} else {
		float rho = g[0];
		#pragma unroll
		for(int i=1; i<Q; i++) rho += g[i];
		rho += 1.0f;
		s.rho = rho;
		const float inv = 1.0f/rho;
		s.u0[0] = momentum<Q, 0>(g)*inv; s.u0[1] = momentum<Q, 1>(g)*inv; s.u0[2] = momentum<Q, 2>(g)*inv;
	}
	s.rho2 = 0.5f/s.rho;
	#pragma unroll
	for(int d=0; d<3; d++) {
		s.Ft[d] = Ft[d];
		const float v = VF ? fmaf(Ft[d], s.rho2, s.u0[d]) : s.u0[d];
		s.kappa[d] = v>-DEF_C && v<DEF_C;
		s.u[d] = clampc(v);
	}
	s.c3 = -3.0f*fmaf(s.u[0], s.u[0], fmaf(s.u[1], s.u[1], s.u[2]*s.u[2]));
}

// gbar = (dh/dg)^T hbar + ke_weight * d(1/2 rho |u|^2)/dg; Fbar += (dh/dFt)^T hbar (+ objective part)
template<int Q, bool TRT, bool VF> __device__ __forceinline__ void adj_cell(const CellState<Q>& s, const bool is_e, const float* hbar, const float ke_weight,
                                                                         const StepArgs& a, float* gbar, float* Fbar) {
	float feqbar[Q], Gbar[Q];
	if(is_e) {
		#pragma unroll
		for(int i=0; i<Q; i++) { gbar[i] = 0.0f; feqbar[i] = hbar[i]; Gbar[i] = 0.0f; }
	} else if constexpr(!TRT) {
		#pragma unroll
		for(int i=0; i<Q; i++) { gbar[i] = a.omw*hbar[i]; feqbar[i] = a.w*hbar[i]; Gbar[i] = a.c_tau*hbar[i]; }
	} else {
		gbar[0] = fmaf(-2.0f*a.hp, hbar[0], hbar[0]); feqbar[0] = 2.0f*a.hp*hbar[0]; Gbar[0] = 2.0f*a.c_taup*hbar[0];
		#pragma unroll
		for(int i=1; i<Q; i+=2) {
			const float x = hbar[i], y = hbar[i+1], sp = x+y, sm = x-y;
			const float di = fmaf(a.hp, sp, a.hm*sm), dj = fmaf(a.hp, sp, -a.hm*sm);
			gbar[i] = x-di; gbar[i+1] = y-dj; feqbar[i] = di; feqbar[i+1] = dj;
			Gbar[i] = fmaf(a.c_taup, sp, a.c_taum*sm); Gbar[i+1] = fmaf(a.c_taup, sp, -a.c_taum*sm);
		}
	}
	// equilibrium
	float rhobar = 0.0f, ubar[3] = {0.0f, 0.0f, 0.0f};
	Unroll<0, Q, 1>::run([&](auto ic) {
		constexpr int i = decltype(ic)::value;
		const float wi = vs_w<Q>(i);
		const float uk = 3.0f*(vs_c(0, i)*s.u[0]+vs_c(1, i)*s.u[1]+vs_c(2, i)*s.u[2]);
		const float fb = feqbar[i]*wi;
		rhobar = fmaf(fb, fmaf(0.5f, fmaf(uk, uk, s.c3), uk+1.0f), rhobar);
		const float fbr = fb*s.rho;
		#pragma unroll
		for(int d=0; d<3; d++) {
			const int cd = d==0 ? vs_c(0, i) : d==1 ? vs_c(1, i) : vs_c(2, i);
			ubar[d] = fmaf(fbr, 3.0f*(cd*(uk+1.0f))-3.0f*s.u[d], ubar[d]);
		}
	});
	float Ftbar[3] = {0.0f, 0.0f, 0.0f};
	if constexpr(VF) {
		if(!is_e) {
			Unroll<0, Q, 1>::run([&](auto ic) {
				constexpr int i = decltype(ic)::value;
				const float wi9 = 9.0f*vs_w<Q>(i)*Gbar[i];
				constexpr int cx = vs_c(0, i), cy = vs_c(1, i), cz = vs_c(2, i);
				const float cf = cx*s.Ft[0]+cy*s.Ft[1]+cz*s.Ft[2], cu = cx*s.u[0]+cy*s.u[1]+cz*s.u[2];
				ubar[0] = fmaf(wi9, cf*cx-s.Ft[0]*THIRD, ubar[0]); Ftbar[0] = fmaf(wi9, cx*(cu+THIRD)-s.u[0]*THIRD, Ftbar[0]);
				ubar[1] = fmaf(wi9, cf*cy-s.Ft[1]*THIRD, ubar[1]); Ftbar[1] = fmaf(wi9, cy*(cu+THIRD)-s.u[1]*THIRD, Ftbar[1]);
				ubar[2] = fmaf(wi9, cf*cz-s.Ft[2]*THIRD, ubar[2]); Ftbar[2] = fmaf(wi9, cz*(cu+THIRD)-s.u[2]*THIRD, Ftbar[2]);
			});
		}
	}
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
	if(!is_e) {
		const float inv = 1.0f/s.rho;
		rhobar = fmaf(rho2bar, -2.0f*s.rho2*s.rho2, rhobar); // d(0.5/rho)/drho = -0.5/rho^2 = -2 rho2^2
		float mbar[3];
		#pragma unroll
		for(int d=0; d<3; d++) { mbar[d] = u0bar[d]*inv; rhobar = fmaf(-u0bar[d]*inv, s.u0[d], rhobar); }
		Unroll<0, Q, 1>::run([&](auto ic) {
			constexpr int i = decltype(ic)::value;
			float gb = gbar[i]+rhobar;
			if constexpr(vs_c(0, i)!=0) gb += vs_c(0, i)>0 ? mbar[0] : -mbar[0];
			if constexpr(vs_c(1, i)!=0) gb += vs_c(1, i)>0 ? mbar[1] : -mbar[1];
			if constexpr(vs_c(2, i)!=0) gb += vs_c(2, i)>0 ? mbar[2] : -mbar[2];
			gbar[i] = gb;
		});
	}
	#pragma unroll
	for(int d=0; d<3; d++) Fbar[d] += Ftbar[d];
}

// load / store positions of the slot set of cell n at the parity of step t:
// load reads g_0 from (n,0), g_i from A_i, g_{i+1} from B_i; store writes h_i to B_i, h_{i+1} to A_i
template<int Q> struct SlotSet {
	uint64_t A[Q], B[Q];
	__device__ __forceinline__ SlotSet(const uint64_t N, const uint64_t n, const Nbr& nb, const bool odd) {
		const uint64_t e = odd ? 0ull : N;
		Unroll<1, Q, 2>::run([&](auto ic) {
			constexpr int i = decltype(ic)::value;
			A[i] = (uint64_t)i*N+e+n;
			B[i] = (uint64_t)(i+1)*N-e+nb.template j<i>();
		});
	}
};

// OBJ_ONLY: add only the objective's dj/dg (lambda += ..., hbar = 0): the final state of the window
template<int Q, int ST, bool TRT, int EXT, bool OBJ_ONLY> __global__ void __launch_bounds__(BLOCK) k_adjoint_step(const StepArgs a, const AdjArgs j) {
	typedef typename Codec<ST>::T T;
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0, EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	CellPos c;
	if(!cell_of_thread(g, c)) return;
	const uint64_t n = c.n, N = g.N;
	const uint8_t fl = a.flags[n];
	const uint8_t bo = fl&TYPE_BO;
	const bool odd = (a.t&1ull)!=0ull;
	const Nbr nb(g, c.x, c.y, c.z);
	if(bo==TYPE_S||(fl&TYPE_SU)==TYPE_G) { // identity map; the drag objective lives on these cells
		if(j.obj_kind==OBJ_DRAG_X && j.obj_weight!=0.0f && fl==(uint8_t)j.marker) {
			const SlotSet<Q> ss(N, n, nb, odd);
			const float w2 = 2.0f*j.obj_weight;
			Unroll<1, Q, 2>::run([&](auto ic) {
				constexpr int i = decltype(ic)::value, cx = vs_c(0, i);
				if constexpr(cx!=0) { j.lambda[ss.A[i]] += cx*w2; j.lambda[ss.B[i]] -= cx*w2; } // g_i at A_i (c_i), g_{i+1} at B_i (-c_i)
			});
		}
		return;
	}
	const bool is_e = EQ && bo==TYPE_E;
	const bool ke = j.obj_kind==OBJ_KE_PLANE && j.obj_weight!=0.0f && c.x==j.plane_x && !is_e;
	if(OBJ_ONLY && !ke) return;
	const SlotSet<Q> ss(N, n, nb, odd);
	float gv[Q], hbar[Q], gbar[Q];
	load_f<Q, ST>((const T*)j.state, N, n, nb, odd, gv);
	if constexpr(OBJ_ONLY) {
		#pragma unroll
		for(int i=0; i<Q; i++) hbar[i] = 0.0f;
	} else {
		hbar[0] = j.lambda[n];
		Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; hbar[i] = j.lambda[ss.B[i]]; hbar[i+1] = j.lambda[ss.A[i]]; });
	}
	float Ft[3] = {a.fx, a.fy, a.fz};
	if constexpr(FF) { Ft[0] += a.F[n]; Ft[1] += a.F[N+n]; Ft[2] += a.F[2ull*N+n]; }
	const float up[3] = {is_e ? a.u[n] : 0.0f, is_e ? a.u[N+n] : 0.0f, is_e ? a.u[2ull*N+n] : 0.0f};
	CellState<Q> s;
	adj_forward<Q, VF>(gv, is_e, is_e ? a.rho[n] : 1.0f, up, Ft, s);
	float Fbar[3] = {0.0f, 0.0f, 0.0f};
	adj_cell<Q, TRT, VF>(s, is_e, hbar, ke ? j.obj_weight : 0.0f, a, gbar, Fbar);
	if constexpr(OBJ_ONLY) {
		j.lambda[n] += gbar[0];
		Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; j.lambda[ss.A[i]] += gbar[i]; j.lambda[ss.B[i]] += gbar[i+1]; });
	} else {
		j.lambda[n] = gbar[0];
		Unroll<1, Q, 2>::run([&](auto ic) { constexpr int i = decltype(ic)::value; j.lambda[ss.A[i]] = gbar[i]; j.lambda[ss.B[i]] = gbar[i+1]; });
	}
	if constexpr(FF) { j.grad[n] += Fbar[0]; j.grad[N+n] += Fbar[1]; j.grad[2ull*N+n] += Fbar[2]; }
}

// objective term of the state at one time step, FP64 partial sums per block (deterministic order)
template<int Q, int ST, int EXT> __global__ void __launch_bounds__(256) k_objective_value(const StepArgs a, const AdjArgs j, double* __restrict__ partials) {
	typedef typename Codec<ST>::T T;
	constexpr bool VF = (EXT&EXT_VF)!=0, FF = (EXT&EXT_FF)!=0, EQ = (EXT&EXT_EQ)!=0;
	const Grid& g = grid_of(a.g);
	const uint64_t N = g.N;
	double acc = 0.0;
	for(uint64_t n=(uint64_t)blockIdx.x*256u+threadIdx.x; n<N; n+=(uint64_t)gridDim.x*256u) {
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
