// CPU ORACLE for the LBM solver path: TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and only as
// the checker or the timed CPU baseline; the product (fluidx3d_gb300) never calls it.
//
// A restatement, in plain C++, of the reference's LBM scheme for one domain:
//   velocity sets, neighbours        src/kernel.cpp:861-958
//   calculate_f_eq                   src/kernel.cpp:1004-1061
//   calculate_rho_u                  src/kernel.cpp:1063-1088
//   calculate_forcing_terms          src/kernel.cpp:1091-1101
//   load_f / store_f (Esoteric-Pull) src/kernel.cpp:1326-1339
//   initialize                       src/kernel.cpp:1358-1430
//   stream_collide (SRT/TRT, TYPE_S, TYPE_E, VOLUME_FORCE, FORCE_FIELD, SUBGRID)  src/kernel.cpp:1454-1636
//   apply_moving_boundaries          src/kernel.cpp:1104-1113
//   UPDATE_FIELDS (rho/u written by stream_collide)  src/kernel.cpp:1565-1573
//   update_moving_boundaries         src/kernel.cpp:1431-1450
//   update_fields                    src/kernel.cpp:1794-1870
//   update_force_field               src/kernel.cpp:1873-1884
//   object_center_of_mass/force/torque (sums done in FP64 here)  src/kernel.cpp:1901-1959
//   voxelize_mesh / unvoxelize_mesh  src/kernel.cpp:2267-2363
//   FP16S / FP16C codecs             src/lbm.cpp:411-414, src/kernel.cpp:848-859
//   relaxation rate literal          src/lbm.cpp:374 (def_w printed with "%f")
//
// Two instantiations:
//   * "f32": FP32 arithmetic in the reference's operation order, with fma() exactly where the
//     reference writes fma() and no other contraction (compiled with -ffp-contract=off); DDFs stored
//     as FP32, FP16S or FP16C. Pinned bit-exact against the reference's own kernel text compiled for
//     the CPU (oracle/ref_harness), and the target the CUDA kernels are compared with.
//   * "f64": the same scheme in FP64 arithmetic and FP64 DDF storage: the error baseline for the FP32,
//     FP16S and FP16C runs.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>
#include "half_ieee.h"

typedef uint8_t u8;
typedef uint16_t u16;
typedef uint32_t u32;
typedef uint64_t u64;

enum { ST_FP32 = 0, ST_FP16S = 1, ST_FP16C = 2 };
enum { EXT_VOLUME_FORCE = 1, EXT_FORCE_FIELD = 2, EXT_EQUILIBRIUM_BOUNDARIES = 4, EXT_SUBGRID = 8, EXT_MOVING_BOUNDARIES = 16, EXT_UPDATE_FIELDS = 32 };
enum { T_S = 0x01, T_E = 0x02, T_T = 0x04, T_BO = 0x03, T_MS = 0x03, T_G = 0x20, T_SU = 0x38, T_XY = 0xC0 };

extern "C" struct OracleConfig {
	u32 Nx, Ny, Nz;
	u32 q;        // 19 or 27
	u32 trt;      // 0: SRT, 1: TRT
	u32 storage;  // ST_*
	u32 ext;      // EXT_* bits
	u32 threads;  // host threads for the per-cell loops
	double w;     // relaxation rate as the kernel sees it
};

// ------------------------------------------------------------------ velocity sets (src/kernel.cpp:878-887)
static const int C19[3][19] = {
	{0, 1,-1, 0, 0, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0},
	{0, 0, 0, 1,-1, 0, 0, 1,-1, 0, 0, 1,-1,-1, 1, 0, 0, 1,-1},
	{0, 0, 0, 0, 0, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0,-1, 1,-1, 1}};
static const int C27[3][27] = {
	{0, 1,-1, 0, 0, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1},
	{0, 0, 0, 1,-1, 0, 0, 1,-1, 0, 0, 1,-1,-1, 1, 0, 0, 1,-1, 1,-1, 1,-1,-1, 1, 1,-1},
	{0, 0, 0, 0, 0, 1,-1, 0, 0, 1,-1, 1,-1, 0, 0,-1, 1,-1, 1, 1,-1,-1, 1, 1,-1, 1,-1}};

static inline int cq(const u32 q, const int d, const u32 i) { return q==19u ? C19[d][i] : C27[d][i]; }

template<typename real> struct Weights { real w0, ws, we, wc; };
template<typename real> static Weights<real> weights(const u32 q) { // weights as the reference's defines spell them
	Weights<real> r;
	if(q==19u) { r.w0 = (real)1/(real)3; r.ws = (real)1/(real)18; r.we = (real)1/(real)36; r.wc = (real)0; }
	else { r.w0 = (real)1/(real)3.375; r.ws = (real)1/(real)13.5; r.we = (real)1/(real)54; r.wc = (real)1/(real)216; }
	return r;
}
template<typename real> static inline real weight(const Weights<real>& W, const u32 i) { return i==0u ? W.w0 : i<7u ? W.ws : i<19u ? W.we : W.wc; }

// ------------------------------------------------------------------ storage codecs
static inline float fp16c_to_float(const u16 x) { // src/kernel.cpp:848-852
	const u32 e = ((u32)x&0x7800u)>>11;
	const u32 m = ((u32)x&0x07FFu)<<12;
	const float mf = (float)m;
	u32 mfb; std::memcpy(&mfb, &mf, 4);
	const u32 v = mfb>>23;
	const u32 r = (((u32)x&0x8000u)<<16) | (u32)(e!=0u)*((e+112u)<<23|m) | (u32)((e==0u)&(m!=0u))*((v-37u)<<23|((m<<(150u-v))&0x007FF000u));
	float f; std::memcpy(&f, &r, 4);
	return f;
}
static inline u16 float_to_fp16c(const float x) { // src/kernel.cpp:853-858
	u32 xb; std::memcpy(&xb, &x, 4);
	const u32 b = xb+0x00000800u;
	const u32 e = (b&0x7F800000u)>>23;
	const u32 m = b&0x007FFFFFu;
	return (u16)((b&0x80000000u)>>16 | (u32)(e>112u)*((((e-112u)<<11)&0x7800u)|m>>12) | (u32)((e<113u)&(e>100u))*((((0x007FF800u+m)>>(124u-e))+1u)>>1));
}

template<typename real> struct Store;
template<> struct Store<double> { // FP64 oracle: DDFs kept in FP64
	static inline double load(const void* p, const u64 o, u32) { return ((const double*)p)[o]; }
	static inline void store(void* p, const u64 o, const double x, u32) { ((double*)p)[o] = x; }
};
template<> struct Store<float> {
	static inline float load(const void* p, const u64 o, const u32 st) {
		if(st==ST_FP16S) return half_bits_to_float(((const u16*)p)[o])*3.0517578E-5f;
		if(st==ST_FP16C) return fp16c_to_float(((const u16*)p)[o]);
		return ((const float*)p)[o];
	}
	static inline void store(void* p, const u64 o, const float x, const u32 st) {
		if(st==ST_FP16S) ((u16*)p)[o] = float_to_half_bits_rne(x*32768.0f);
		else if(st==ST_FP16C) ((u16*)p)[o] = float_to_fp16c(x);
		else ((float*)p)[o] = x;
	}
};

// ------------------------------------------------------------------ lattice helpers
struct Grid {
	u32 Nx, Ny, Nz; u64 N;
	explicit Grid(const OracleConfig* c) : Nx(c->Nx), Ny(c->Ny), Nz(c->Nz), N((u64)c->Nx*c->Ny*c->Nz) {}
	inline void coords(const u64 n, u32& x, u32& y, u32& z) const {
		const u64 t = n%((u64)Nx*Ny);
		x = (u32)(t%Nx); y = (u32)(t/Nx); z = (u32)(n/((u64)Nx*Ny));
	}
	inline u64 index(const u32 x, const u32 y, const u32 z) const { return (u64)x+((u64)y+(u64)z*Ny)*(u64)Nx; }
	// j[i] = periodic neighbour in direction c_i (src/kernel.cpp:904-958)
	inline void neighbors(const u64 n, const u32 q, u64* j) const {
		u32 x, y, z; coords(n, x, y, z);
		j[0] = n;
		for(u32 i=1u; i<q; i++) {
			const u32 xi = (u32)(((int64_t)x+cq(q, 0, i)+Nx)%Nx);
			const u32 yi = (u32)(((int64_t)y+cq(q, 1, i)+Ny)%Ny);
			const u32 zi = (u32)(((int64_t)z+cq(q, 2, i)+Nz)%Nz);
			j[i] = index(xi, yi, zi);
		}
	}
};

template<typename L> static void parallel_cells(const u64 items, const u32 threads, L&& body) {
	const u32 T = threads>0u ? threads : 1u;
	if(T==1u || items<4096ull) { for(u64 n=0ull; n<items; n++) body(n); return; }
	std::vector<std::thread> pool;
	for(u32 t=0u; t<T; t++) pool.emplace_back([=, &body]() { for(u64 n=items*t/T; n<items*(t+1u)/T; n++) body(n); });
	for(auto& th : pool) th.join();
}

// Esoteric-Pull slot of population k for cell n (src/kernel.cpp:1326-1339): the pair (i,i+1), i odd,
// is read from (n, i) and (j[i], i+1) at odd t, from (n, i+1) and (j[i], i) at even t; stores swap.
template<typename real> static void load_f(const u64 n, real* fhn, const void* fi, const u64* j, const u64 t, const u32 q, const u64 N, const u32 st) {
	fhn[0] = Store<real>::load(fi, n, st);
	for(u32 i=1u; i<q; i+=2u) {
		fhn[i   ] = Store<real>::load(fi, (u64)(t%2ull ? i    : i+1u)*N+n   , st);
		fhn[i+1u] = Store<real>::load(fi, (u64)(t%2ull ? i+1u : i   )*N+j[i], st);
	}
}
template<typename real> static void store_f(const u64 n, const real* fhn, void* fi, const u64* j, const u64 t, const u32 q, const u64 N, const u32 st) {
	Store<real>::store(fi, n, fhn[0], st);
	for(u32 i=1u; i<q; i+=2u) {
		Store<real>::store(fi, (u64)(t%2ull ? i+1u : i   )*N+j[i], fhn[i   ], st);
		Store<real>::store(fi, (u64)(t%2ull ? i    : i+1u)*N+n   , fhn[i+1u], st);
	}
}

static inline float fmaT(const float a, const float b, const float c) { return std::fmaf(a, b, c); }
static inline double fmaT(const double a, const double b, const double c) { return std::fma(a, b, c); }

// signed sum of the non-zero terms c_d*v_d in x,y,z order; c_d in {-1,0,1} makes every product exact,
// so this equals the reference's c(i)*vx+c(N+i)*vy+c(2N+i)*vz up to the sign of an exact zero
template<typename real> static inline real csum(const u32 q, const u32 i, const real vx, const real vy, const real vz) {
	const int c[3] = {cq(q, 0, i), cq(q, 1, i), cq(q, 2, i)};
	const real v[3] = {vx, vy, vz};
	bool first = true; real s = (real)0;
	for(int d=0; d<3; d++) {
		if(c[d]==0) continue;
		const real term = c[d]>0 ? v[d] : -v[d];
		s = first ? term : s+term;
		first = false;
	}
	return s;
}

// calculate_f_eq (src/kernel.cpp:1004-1061): pairs (i,i+1) share u_k = 3*(c_i . u)
template<typename real> static void calculate_f_eq(const real rho, real ux, real uy, real uz, real* feq, const u32 q) {
	const Weights<real> W = weights<real>(q);
	const real rhom1 = rho-(real)1;
	const real c3 = (real)(-3)*((ux*ux+uy*uy)+uz*uz);
	uz *= (real)3; ux *= (real)3; uy *= (real)3;
	feq[0] = W.w0*fmaT(rho, (real)0.5*c3, rhom1);
	for(u32 i=1u; i<q; i+=2u) {
		const real wi = weight(W, i);
		const real rhow = wi*rho, rhom1w = wi*rhom1;
		const real uk = csum<real>(q, i, ux, uy, uz);
		feq[i   ] = fmaT(rhow, fmaT((real)0.5, fmaT(uk, uk, c3),  uk), rhom1w);
		feq[i+1u] = fmaT(rhow, fmaT((real)0.5, fmaT(uk, uk, c3), -uk), rhom1w);
	}
}

// calculate_rho_u (src/kernel.cpp:1063-1088): rho sums f_i in index order and adds 1 last; each
// velocity component alternates +f(positive member) -f(negative member) over the pairs in index order
template<typename real> static void moments(const real* f, real& rho, real& mx, real& my, real& mz, const u32 q) {
	rho = f[0];
	for(u32 i=1u; i<q; i++) rho += f[i];
	rho += (real)1;
	real m[3];
	for(int d=0; d<3; d++) {
		bool first = true; real s = (real)0;
		for(u32 i=1u; i<q; i+=2u) {
			const int c = cq(q, d, i);
			if(c==0) continue;
			const real fp = c>0 ? f[i] : f[i+1u], fm = c>0 ? f[i+1u] : f[i];
			s = first ? fp-fm : (s+fp)-fm;
			first = false;
		}
		m[d] = s;
	}
	mx = m[0]; my = m[1]; mz = m[2];
}
template<typename real> static void calculate_rho_u(const real* f, real& rho, real& ux, real& uy, real& uz, const u32 q) {
	real mx, my, mz;
	moments(f, rho, mx, my, mz, q);
	ux = mx/rho; uy = my/rho; uz = mz/rho;
}

template<typename real> static inline real sound_speed();
template<> inline float sound_speed<float>() { return 0.57735027f; } // def_c (src/lbm.cpp:373)
template<> inline double sound_speed<double>() { return 0.57735026918962576; }
template<typename real> static inline real third();
template<> inline float third<float>() { return 0.33333334f; }
template<> inline double third<double>() { return 1.0/3.0; }
template<typename real> static inline real clampT(const real x, const real a, const real b) { return std::fmin(std::fmax(x, a), b); }

// calculate_forcing_terms (src/kernel.cpp:1091-1101), Guo forcing
template<typename real> static void forcing_terms(const real ux, const real uy, const real uz, const real fx, const real fy, const real fz, real* Fin, const u32 q) {
	const Weights<real> W = weights<real>(q);
	const real uF = -third<real>()*fmaT(ux, fx, fmaT(uy, fy, uz*fz));
	Fin[0] = (real)9*W.w0*uF;
	for(u32 i=1u; i<q; i++) {
		Fin[i] = (real)9*weight(W, i)*fmaT(csum<real>(q, i, fx, fy, fz), csum<real>(q, i, ux, uy, uz)+third<real>(), uF);
	}
}

// ------------------------------------------------------------------ kernels
// TYPE_MS marking (src/kernel.cpp:1381-1385, 1441-1447): a cell next to a TYPE_S cell with u != 0
template<typename real> static bool next_to_moving_boundary(const u64* j, const real* u, const u8* flags, const u32 q, const u64 N) {
	bool next = false;
	for(u32 i=1u; i<q; i++) next = next||((flags[j[i]]&T_BO)==T_S&&(u[j[i]]!=(real)0||u[N+j[i]]!=(real)0||u[2ull*N+j[i]]!=(real)0));
	return next;
}

template<typename real> static int initialize_t(const OracleConfig* c, void* fi, real* rho, real* u, u8* flags) {
	const Grid G(c); const u32 q = c->q;
	const bool mb = (c->ext&EXT_MOVING_BOUNDARIES)!=0u;
	// MOVING_BOUNDARIES rewrites flags while neighbours read them; the TYPE_S bit pattern a neighbour
	// tests never changes (00 <-> 11), so marking into a copy gives the reference's result race-free
	std::vector<u8> marked(mb ? G.N : 0ull);
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		u64 j[27]; G.neighbors(n, q, j);
		const u8 flagsn_bo = flags[n]&T_BO;
		if(mb) {
			marked[n] = flags[n];
			if(flagsn_bo==T_S) { // solid cells keep their (wall) velocity unless all their neighbours are solid (src/kernel.cpp:1370-1374)
				bool only_s = true;
				for(u32 i=1u; i<q; i++) only_s = only_s&&(flags[j[i]]&T_BO)==T_S;
				if(only_s) { u[n] = (real)0; u[G.N+n] = (real)0; u[2ull*G.N+n] = (real)0; }
			} else if(flagsn_bo!=T_E) {
				marked[n] = next_to_moving_boundary<real>(j, u, flags, q, G.N) ? (u8)(flags[n]|T_MS) : (u8)(flags[n]&~T_MS);
			}
		} else if(flagsn_bo==T_S) { u[n] = (real)0; u[G.N+n] = (real)0; u[2ull*G.N+n] = (real)0; } // src/kernel.cpp:1370-1377
		real feq[27];
		calculate_f_eq<real>(rho[n], u[n], u[G.N+n], u[2ull*G.N+n], feq, q);
		store_f<real>(n, feq, fi, j, 1ull, q, G.N, c->storage); // odd parity baked in (src/kernel.cpp:1429)
	});
	if(mb) std::memcpy(flags, marked.data(), G.N);
	return 0;
}

// src/kernel.cpp:1431-1450: fluid cells (not TYPE_S, TYPE_E or TYPE_T) next to a moving solid get TYPE_MS
template<typename real> static int update_moving_boundaries_t(const OracleConfig* c, const real* u, u8* flags) {
	const Grid G(c); const u32 q = c->q;
	std::vector<u8> marked(flags, flags+G.N);
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		const u8 flagsn = flags[n], flagsn_bo = flagsn&T_BO;
		if(flagsn_bo==T_S||flagsn_bo==T_E||(flagsn&T_T)) return;
		u64 j[27]; G.neighbors(n, q, j);
		marked[n] = next_to_moving_boundary<real>(j, u, flags, q, G.N) ? (u8)(flagsn|T_MS) : (u8)(flagsn&~T_MS);
	});
	std::memcpy(flags, marked.data(), G.N);
	return 0;
}

// src/kernel.cpp:1104-1113 apply_moving_boundaries: in a TYPE_MS cell, population i gains
// -6 w_i (c_{i+1}.u_s) when the neighbour along c_{i+1} is a TYPE_S cell moving at u_s, population
// i+1 gains -6 w_i (c_i.u_s) from the neighbour along c_i (i odd, wall density 1)
template<typename real> static void apply_moving_boundaries(real* fhn, const u64* j, const real* u, const u8* flags, const u32 q, const u64 N) {
	const Weights<real> W = weights<real>(q);
	auto cu = [&](const u32 k, const u64 s) { return (real)cq(q, 0, k)*u[s]+(real)cq(q, 1, k)*u[N+s]+(real)cq(q, 2, k)*u[2ull*N+s]; };
	for(u32 i=1u; i<q; i+=2u) {
		const real w6 = (real)(-6)*weight(W, i);
		if((flags[j[i+1u]]&T_BO)==T_S) fhn[i] = fmaT(w6, cu(i+1u, j[i+1u]), fhn[i]);
		if((flags[j[i]]&T_BO)==T_S) fhn[i+1u] = fmaT(w6, cu(i, j[i]), fhn[i+1u]);
	}
}

// force shift + clamp shared by stream_collide and update_fields (src/kernel.cpp:1550-1563, 1852-1862)
template<typename real> static inline void shift_clamp(real& ux, real& uy, real& uz, const real rho, const real fx, const real fy, const real fz, const bool vf) {
	const real cs = sound_speed<real>();
	if(vf) {
		const real rho2 = (real)0.5/rho;
		ux = clampT(fmaT(fx, rho2, ux), -cs, cs);
		uy = clampT(fmaT(fy, rho2, uy), -cs, cs);
		uz = clampT(fmaT(fz, rho2, uz), -cs, cs);
	} else {
		ux = clampT(ux, -cs, cs); uy = clampT(uy, -cs, cs); uz = clampT(uz, -cs, cs);
	}
}

template<typename real> static void collide_cell(real* fhn, const real rhon, const real uxn, const real uyn, const real uzn, const real fxn, const real fyn, const real fzn,
                                                 const bool is_e, const OracleConfig* c) {
	const u32 q = c->q;
	const bool vf = (c->ext&EXT_VOLUME_FORCE)!=0u;
	real Fin[27], feq[27];
	if(vf) forcing_terms<real>(uxn, uyn, uzn, fxn, fyn, fzn, Fin, q); else for(u32 i=0u; i<q; i++) Fin[i] = (real)0;
	calculate_f_eq<real>(rhon, uxn, uyn, uzn, feq, q);
	real w = (real)c->w;
	if(c->ext&EXT_SUBGRID) { // Smagorinsky-Lilly relaxation rate of this cell (src/kernel.cpp:1579-1593)
		const real tau0 = (real)1/w;
		real Hxx = 0, Hyy = 0, Hzz = 0, Hxy = 0, Hxz = 0, Hyz = 0; // non-equilibrium stress tensor
		for(u32 i=1u; i<q; i++) {
			const real fneqi = fhn[i]-feq[i];
			const real cxi = (real)cq(q, 0, i), cyi = (real)cq(q, 1, i), czi = (real)cq(q, 2, i);
			Hxx += cxi*cxi*fneqi; Hxy += cxi*cyi*fneqi; Hyy += cyi*cyi*fneqi;
			Hxz += cxi*czi*fneqi; Hyz += cyi*czi*fneqi; Hzz += czi*czi*fneqi;
		}
		const real Qs = Hxx*Hxx+Hyy*Hyy+Hzz*Hzz+(real)2*(Hxy*Hxy+Hxz*Hxz+Hyz*Hyz);
		w = (real)2/(tau0+std::sqrt(tau0*tau0+(real)0.76421222f*std::sqrt(Qs)/rhon));
	}
	if(!c->trt) { // SRT (src/kernel.cpp:1595-1604)
		if(vf) { const real c_tau = fmaT(w, (real)(-0.5), (real)1); for(u32 i=0u; i<q; i++) Fin[i] *= c_tau; }
		for(u32 i=0u; i<q; i++) fhn[i] = is_e ? feq[i] : fmaT((real)1-w, fhn[i], fmaT(w, feq[i], Fin[i]));
	} else { // TRT (src/kernel.cpp:1605-1633)
		const real wp = w;
		const real wm = (real)1/((real)0.1875/((real)1/w-(real)0.5)+(real)0.5);
		if(vf) {
			const real c_taup = fmaT(wp, (real)(-0.25), (real)0.5), c_taum = fmaT(wm, (real)(-0.25), (real)0.5);
			real Fib[27]; Fib[0] = Fin[0];
			for(u32 i=1u; i<q; i+=2u) { Fib[i] = Fin[i+1u]; Fib[i+1u] = Fin[i]; }
			for(u32 i=0u; i<q; i++) Fin[i] = fmaT(c_taup, Fin[i]+Fib[i], c_taum*(Fin[i]-Fib[i]));
		}
		real fhb[27], feb[27];
		fhb[0] = fhn[0]; feb[0] = feq[0];
		for(u32 i=1u; i<q; i+=2u) { fhb[i] = fhn[i+1u]; fhb[i+1u] = fhn[i]; feb[i] = feq[i+1u]; feb[i+1u] = feq[i]; }
		for(u32 i=0u; i<q; i++) {
			fhn[i] = is_e ? feq[i] : fmaT((real)0.5*wp, ((feq[i]-fhn[i])+feb[i])-fhb[i], fmaT((real)0.5*wm, ((feq[i]-feb[i])-fhn[i])+fhb[i], fhn[i]+Fin[i]));
		}
	}
}

template<typename real> static int stream_collide_t(const OracleConfig* c, void* fi, real* rho, real* u, const u8* flags, const u64 t,
                                                    const real fx, const real fy, const real fz, const real* F) {
	const Grid G(c); const u32 q = c->q;
	const bool eq = (c->ext&EXT_EQUILIBRIUM_BOUNDARIES)!=0u, ff = (c->ext&EXT_FORCE_FIELD)!=0u, vf = (c->ext&EXT_VOLUME_FORCE)!=0u;
	const bool mb = (c->ext&EXT_MOVING_BOUNDARIES)!=0u, uf = (c->ext&EXT_UPDATE_FIELDS)!=0u;
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		const u8 flagsn_bo = flags[n]&T_BO;
		if(flagsn_bo==T_S||(flags[n]&T_SU)==T_G) return; // solid (implicit bounce-back through Esoteric-Pull) or gas: nothing
		u64 j[27]; G.neighbors(n, q, j);
		real fhn[27];
		load_f<real>(n, fhn, fi, j, t, q, G.N, c->storage);
		if(mb && flagsn_bo==T_MS) apply_moving_boundaries<real>(fhn, j, u, flags, q, G.N);
		real rhon, uxn, uyn, uzn;
		const bool is_e = eq && flagsn_bo==T_E;
		if(is_e) { rhon = rho[n]; uxn = u[n]; uyn = u[G.N+n]; uzn = u[2ull*G.N+n]; }
		else calculate_rho_u<real>(fhn, rhon, uxn, uyn, uzn, q);
		real fxn = fx, fyn = fy, fzn = fz;
		if(ff) { fxn += F[n]; fyn += F[G.N+n]; fzn += F[2ull*G.N+n]; }
		shift_clamp<real>(uxn, uyn, uzn, rhon, fxn, fyn, fzn, vf);
		if(uf && !is_e) { rho[n] = rhon; u[n] = uxn; u[G.N+n] = uyn; u[2ull*G.N+n] = uzn; } // UPDATE_FIELDS: the fields the cell collides with
		collide_cell<real>(fhn, rhon, uxn, uyn, uzn, fxn, fyn, fzn, is_e, c);
		store_f<real>(n, fhn, fi, j, t, q, G.N, c->storage);
	});
	return 0;
}

template<typename real> static int update_fields_t(const OracleConfig* c, const void* fi, real* rho, real* u, const u8* flags, const u64 t,
                                                   const real fx, const real fy, const real fz, const real* F) {
	const Grid G(c); const u32 q = c->q;
	const bool eq = (c->ext&EXT_EQUILIBRIUM_BOUNDARIES)!=0u, ff = (c->ext&EXT_FORCE_FIELD)!=0u, vf = (c->ext&EXT_VOLUME_FORCE)!=0u;
	const bool mb = (c->ext&EXT_MOVING_BOUNDARIES)!=0u;
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		const u8 flagsn_bo = flags[n]&T_BO;
		if(flagsn_bo==T_S||(flags[n]&T_SU)==T_G) return;
		u64 j[27]; G.neighbors(n, q, j);
		real fhn[27];
		load_f<real>(n, fhn, fi, j, t, q, G.N, c->storage);
		if(mb && flagsn_bo==T_MS) apply_moving_boundaries<real>(fhn, j, u, flags, q, G.N);
		real rhon, uxn, uyn, uzn;
		calculate_rho_u<real>(fhn, rhon, uxn, uyn, uzn, q);
		real fxn = fx, fyn = fy, fzn = fz;
		if(ff) { fxn += F[n]; fyn += F[G.N+n]; fzn += F[2ull*G.N+n]; }
		shift_clamp<real>(uxn, uyn, uzn, rhon, fxn, fyn, fzn, vf);
		if(eq && flagsn_bo==T_E) return; // preset rho/u of TYPE_E cells stay
		rho[n] = rhon; u[n] = uxn; u[G.N+n] = uyn; u[2ull*G.N+n] = uzn;
	});
	return 0;
}

template<typename real> static int update_force_field_t(const OracleConfig* c, const void* fi, const u8* flags, const u64 t, real* F) {
	const Grid G(c); const u32 q = c->q;
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		if((flags[n]&T_BO)!=T_S) return;
		u64 j[27]; G.neighbors(n, q, j);
		real fhn[27];
		load_f<real>(n, fhn, fi, j, t, q, G.N, c->storage);
		real Fb, fx, fy, fz;
		calculate_rho_u<real>(fhn, Fb, fx, fy, fz, q);
		const real s = (real)2*Fb;
		F[n] = s*fx; F[G.N+n] = s*fy; F[2ull*G.N+n] = s*fz;
	});
	return 0;
}

// object reductions: masked sums over flags==marker (src/kernel.cpp:1901-1959), accumulated in FP64
static int object_sum_impl(const OracleConfig* c, const int kind, const float* F, const u8* flags, const u8 marker,
                           const double cx, const double cy, const double cz, double* out) {
	const Grid G(c);
	double s[4] = {0.0, 0.0, 0.0, 0.0};
	for(u64 n=0ull; n<G.N; n++) {
		if(flags[n]!=marker) continue;
		u32 x, y, z; G.coords(n, x, y, z);
		const double px = (double)((float)x+0.5f-0.5f*(float)G.Nx), py = (double)((float)y+0.5f-0.5f*(float)G.Ny), pz = (double)((float)z+0.5f-0.5f*(float)G.Nz);
		if(kind==0) { s[0] += px; s[1] += py; s[2] += pz; s[3] += 1.0; }
		else {
			const double Fx = F[n], Fy = F[G.N+n], Fz = F[2ull*G.N+n];
			if(kind==1) { s[0] += Fx; s[1] += Fy; s[2] += Fz; }
			else {
				const double rx = px-cx, ry = py-cy, rz = pz-cz;
				s[0] += ry*Fz-rz*Fy; s[1] += rz*Fx-rx*Fz; s[2] += rx*Fy-ry*Fx;
			}
		}
	}
	for(int i=0; i<4; i++) out[i] = s[i];
	return 0;
}

// ------------------------------------------------------------------ voxelization (src/kernel.cpp:2267-2357), FP32
struct f3 { float x, y, z; };
static inline f3 sub(const f3 a, const f3 b) { return {a.x-b.x, a.y-b.y, a.z-b.z}; }
static inline f3 add(const f3 a, const f3 b) { return {a.x+b.x, a.y+b.y, a.z+b.z}; }
static inline f3 cross(const f3 a, const f3 b) { return {a.y*b.z-a.z*b.y, a.z*b.x-a.x*b.z, a.x*b.y-a.y*b.x}; }
static inline float dot(const f3 a, const f3 b) { return a.x*b.x+a.y*b.y+a.z*b.z; }
static inline int clampi(const int x, const int a, const int b) { return x<a ? a : x>b ? b : x; }

// rays: the ray indices to cast (NULL: all A rays of the direction), nrays their count
static int voxelize_impl(const OracleConfig* c, const u32 direction, void* fi, float* u, u8* flags, const u64 t, const u8 flag,
                         const float* p0, const float* p1, const float* p2, const float* bbu, const u64* rays = nullptr, const u64 nrays = 0u) {
	const Grid G(c); const u32 q = c->q;
	const u32 Nx = G.Nx, Ny = G.Ny, Nz = G.Nz;
	const u64 A = direction==0u ? (u64)Ny*Nz : direction==1u ? (u64)Nz*Nx : (u64)Nx*Ny;
	u32 triangle_number; std::memcpy(&triangle_number, &bbu[0], 4);
	const float x0=bbu[1], y0=bbu[2], z0=bbu[3], x1=bbu[4], y1=bbu[5], z1=bbu[6];
	const float cx=bbu[7], cy=bbu[8], cz=bbu[9], ux=bbu[10], uy=bbu[11], uz=bbu[12], rx=bbu[13], ry=bbu[14], rz=bbu[15];
	const u32 hmin = direction==0u ? (u32)clampi((int)x0, 0, (int)Nx-1) : direction==1u ? (u32)clampi((int)y0, 0, (int)Ny-1) : (u32)clampi((int)z0, 0, (int)Nz-1);
	const u32 hmax = direction==0u ? (u32)clampi((int)x1, 0, (int)Nx-1) : direction==1u ? (u32)clampi((int)y1, 0, (int)Ny-1) : (u32)clampi((int)z1, 0, (int)Nz-1);
	const f3 offset = {0.5f*(float)(int)Nx-0.5f, 0.5f*(float)(int)Ny-0.5f, 0.5f*(float)(int)Nz-0.5f};
	const f3 r_dir = {(float)(direction==0u), (float)(direction==1u), (float)(direction==2u)};
	const bool set_u = ux*ux+uy*uy+uz*uz+rx*rx+ry*ry+rz*rz>0.0f;
	parallel_cells(rays ? nrays : A, c->threads, [&](const u64 k) {
		const u64 ai = rays ? rays[k] : k;
		if(ai>=A) return;
		const u32 a = (u32)ai;
		u32 X, Y, Z;
		if(direction==0u) { X = hmin; Y = a%Ny; Z = a/Ny; }
		else if(direction==1u) { X = a/Nz; Y = hmin; Z = a%Nz; }
		else { X = a%Nx; Y = a/Nx; Z = hmin; }
		const f3 pos = {(float)X+0.5f-0.5f*(float)Nx, (float)Y+0.5f-0.5f*(float)Ny, (float)Z+0.5f-0.5f*(float)Nz};
		const f3 o = add(pos, offset);
		const bool outside = direction==0u ? o.y<y0||o.z<z0||o.y>=y1||o.z>=z1 : direction==1u ? o.x<x0||o.z<z0||o.x>=x1||o.z>=z1 : o.x<x0||o.y<y0||o.x>=x1||o.y>=y1;
		if(outside) return;
		u32 intersections = 0u, intersections_check = 0u;
		u16 distances[64] = {0};
		for(u32 i=0u; i<triangle_number; i++) {
			const f3 a0 = {p0[3u*i], p0[3u*i+1u], p0[3u*i+2u]}, a1 = {p1[3u*i], p1[3u*i+1u], p1[3u*i+2u]}, a2 = {p2[3u*i], p2[3u*i+1u], p2[3u*i+2u]};
			const f3 eu = sub(a1, a0), ev = sub(a2, a0), ew = sub(o, a0), h = cross(r_dir, ev), qv = cross(ew, eu);
			const float g = dot(eu, h), f = 1.0f/g, s = f*dot(ew, h), tt = f*dot(r_dir, qv), d = f*dot(ev, qv);
			if(g!=0.0f&&s>=0.0f&&s<1.0f&&tt>=0.0f&&s+tt<1.0f) {
				if(d>0.0f) {
					if(intersections<64u&&d<65536.0f) distances[intersections] = (u16)d;
					intersections++;
				} else {
					intersections_check++;
				}
			}
		}
		const u32 nsort = intersections<64u ? intersections : 64u;
		for(u32 i=1u; i<nsort; i++) { // insertion sort
			const u16 tv = distances[i];
			u32 k = i;
			while(k>0u&&distances[k-1u]>tv) { distances[k] = distances[k-1u]; k--; }
			distances[k] = tv;
		}
		bool inside = (intersections%2u)&&(intersections_check%2u);
		u32 intersection = (intersections%2u)!=(intersections_check%2u);
		const u32 h0 = direction==0u ? X : direction==1u ? Y : Z;
		const u32 last = intersections-1u < 63u ? intersections-1u : 63u;
		const u32 hmesh = h0+(u32)distances[last];
		for(u32 hh=h0; hh<=hmax; hh++) {
			while(intersection<intersections&&hh>h0+(u32)distances[intersection<63u ? intersection : 63u]) { inside = !inside; intersection++; }
			inside = inside&&(intersection<intersections&&hh<hmesh);
			const u32 xx = direction==0u ? hh : X, yy = direction==1u ? hh : Y, zz = direction==2u ? hh : Z;
			const u64 n = G.index(xx, yy, zz);
			u8 flagsn = flags[n];
			const f3 p = add({(float)xx+0.5f-0.5f*(float)Nx, (float)yy+0.5f-0.5f*(float)Ny, (float)zz+0.5f-0.5f*(float)Nz}, offset);
			const f3 rc = cross(sub({cx, cy, cz}, p), {rx, ry, rz});
			const f3 u_set = {ux+rc.x, uy+rc.y, uz+rc.z};
			if(inside) {
				flagsn = (u8)((flagsn&~T_BO)|flag);
				if(set_u) { u[n] = u_set.x; u[G.N+n] = u_set.y; u[2ull*G.N+n] = u_set.z; }
			} else if((flagsn&T_BO)==T_S&&(flagsn&T_XY)==(flag&T_XY)) {
				const f3 un = {u[n], u[G.N+n], u[2ull*G.N+n]};
				if(un.x==u_set.x&&un.y==u_set.y&&un.z==u_set.z) {
					if(set_u) {
						u64 j[27]; G.neighbors(n, q, j);
						float feq[27];
						calculate_f_eq<float>(1.0f, un.x, un.y, un.z, feq, q);
						store_f<float>(n, feq, fi, j, t, q, G.N, c->storage);
					}
					flagsn = (flagsn&T_BO)==T_MS ? (u8)(flagsn&~T_MS) : (u8)(flagsn&~flag);
				}
			}
			flags[n] = flagsn;
		}
	});
	return 0;
}

static int unvoxelize_impl(const OracleConfig* c, u8* flags, const u8 flag, const float x0, const float y0, const float z0, const float x1, const float y1, const float z1) {
	const Grid G(c);
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		u32 x, y, z; G.coords(n, x, y, z);
		const float px = ((float)x+0.5f-0.5f*(float)G.Nx)+(0.5f*(float)(int)G.Nx-0.5f);
		const float py = ((float)y+0.5f-0.5f*(float)G.Ny)+(0.5f*(float)(int)G.Ny-0.5f);
		const float pz = ((float)z+0.5f-0.5f*(float)G.Nz)+(0.5f*(float)(int)G.Nz-0.5f);
		if(px>=x0-1.0f&&py>=y0-1.0f&&pz>=z0-1.0f&&px<=x1+1.0f&&py<=y1+1.0f&&pz<=z1+1.0f) flags[n] &= (u8)~flag;
	});
	return 0;
}

static bool valid(const OracleConfig* c) {
	return c && c->Nx>0u && c->Ny>0u && c->Nz>0u && (c->q==19u||c->q==27u) && c->storage<=ST_FP16C;
}

// ------------------------------------------------------------------ C ABI (ctypes)
extern "C" {

// relaxation rate as the reference bakes it into the kernel: "%f"-formatted 1/tau, tau=3*nu+0.5 in FP32
float oracle_kernel_w(const float nu) {
	const float tau = 3.0f*nu+0.5f;
	char buf[64];
	std::snprintf(buf, sizeof(buf), "%f", (double)(1.0f/tau));
	return std::strtof(buf, nullptr);
}

int oracle_initialize_f32(const OracleConfig* c, void* fi, float* rho, float* u, u8* flags) { return valid(c) ? initialize_t<float>(c, fi, rho, u, flags) : -1; }
int oracle_initialize_f64(const OracleConfig* c, double* fi, double* rho, double* u, u8* flags) { return valid(c) ? initialize_t<double>(c, fi, rho, u, flags) : -1; }

int oracle_stream_collide_f32(const OracleConfig* c, void* fi, float* rho, float* u, const u8* flags, const u64 t, const float fx, const float fy, const float fz, const float* F) {
	return valid(c) ? stream_collide_t<float>(c, fi, rho, u, flags, t, fx, fy, fz, F) : -1;
}
int oracle_stream_collide_f64(const OracleConfig* c, double* fi, double* rho, double* u, const u8* flags, const u64 t, const double fx, const double fy, const double fz, const double* F) {
	return valid(c) ? stream_collide_t<double>(c, fi, rho, u, flags, t, fx, fy, fz, F) : -1;
}
// steps consecutive time steps t0, t0+1, ... (the reference's LBM::run loop, src/lbm.cpp:955-975)
int oracle_run_f32(const OracleConfig* c, void* fi, float* rho, float* u, const u8* flags, const u64 t0, const u64 steps, const float fx, const float fy, const float fz, const float* F) {
	if(!valid(c)) return -1;
	for(u64 s=0ull; s<steps; s++) stream_collide_t<float>(c, fi, rho, u, flags, t0+s, fx, fy, fz, F);
	return 0;
}
int oracle_run_f64(const OracleConfig* c, double* fi, double* rho, double* u, const u8* flags, const u64 t0, const u64 steps, const double fx, const double fy, const double fz, const double* F) {
	if(!valid(c)) return -1;
	for(u64 s=0ull; s<steps; s++) stream_collide_t<double>(c, fi, rho, u, flags, t0+s, fx, fy, fz, F);
	return 0;
}

int oracle_update_fields_f32(const OracleConfig* c, const void* fi, float* rho, float* u, const u8* flags, const u64 t, const float fx, const float fy, const float fz, const float* F) {
	return valid(c) ? update_fields_t<float>(c, fi, rho, u, flags, t, fx, fy, fz, F) : -1;
}
int oracle_update_fields_f64(const OracleConfig* c, const double* fi, double* rho, double* u, const u8* flags, const u64 t, const double fx, const double fy, const double fz, const double* F) {
	return valid(c) ? update_fields_t<double>(c, fi, rho, u, flags, t, fx, fy, fz, F) : -1;
}
int oracle_update_moving_boundaries_f32(const OracleConfig* c, const float* u, u8* flags) { return valid(c) ? update_moving_boundaries_t<float>(c, u, flags) : -1; }
int oracle_update_moving_boundaries_f64(const OracleConfig* c, const double* u, u8* flags) { return valid(c) ? update_moving_boundaries_t<double>(c, u, flags) : -1; }
int oracle_update_force_field_f32(const OracleConfig* c, const void* fi, const u8* flags, const u64 t, float* F) {
	return valid(c) ? update_force_field_t<float>(c, fi, flags, t, F) : -1;
}
int oracle_update_force_field_f64(const OracleConfig* c, const double* fi, const u8* flags, const u64 t, double* F) {
	return valid(c) ? update_force_field_t<double>(c, fi, flags, t, F) : -1;
}
// kind 0: center of mass sums (x,y,z,count), 1: force, 2: torque about (cx,cy,cz)
int oracle_object_sum(const OracleConfig* c, const int kind, const float* F, const u8* flags, const u8 marker, const double cx, const double cy, const double cz, double* out) {
	return valid(c) && kind>=0 && kind<=2 ? object_sum_impl(c, kind, F, flags, marker, cx, cy, cz, out) : -1;
}
int oracle_voxelize_mesh(const OracleConfig* c, const u32 direction, void* fi, float* u, u8* flags, const u64 t, const u8 flag,
                         const float* p0, const float* p1, const float* p2, const float* bbu) {
	return valid(c) && direction<3u ? voxelize_impl(c, direction, fi, u, flags, t, flag, p0, p1, p2, bbu) : -1;
}
// the same for a subset of rays (ray index a as in voxelize_mesh: direction 0 a = Y + Z*Ny, 1 a = Z + X*Nz, 2 a = X + Y*Nx)
int oracle_voxelize_rays(const OracleConfig* c, const u32 direction, void* fi, float* u, u8* flags, const u64 t, const u8 flag,
                         const float* p0, const float* p1, const float* p2, const float* bbu, const u64* rays, const u64 nrays) {
	return valid(c) && direction<3u && rays ? voxelize_impl(c, direction, fi, u, flags, t, flag, p0, p1, p2, bbu, rays, nrays) : -1;
}
int oracle_unvoxelize_mesh(const OracleConfig* c, u8* flags, const u8 flag, const float x0, const float y0, const float z0, const float x1, const float y1, const float z1) {
	return valid(c) ? unvoxelize_impl(c, flags, flag, x0, y0, z0, x1, y1, z1) : -1;
}
u16 oracle_fp16s_encode(const float x) { return float_to_half_bits_rne(x*32768.0f); }
float oracle_fp16s_decode(const u16 h) { return half_bits_to_float(h)*3.0517578E-5f; }
u16 oracle_fp16c_encode(const float x) { return float_to_fp16c(x); }
float oracle_fp16c_decode(const u16 h) { return fp16c_to_float(h); }

} // extern "C"

// ==================================================================== adjoint (FP64), no reference
// Discrete adjoint of the forward step above, for dJ/dF with F the per-cell FORCE_FIELD force.
// A step maps the slots of each fluid cell n (its Esoteric-Pull slot set at the step's parity) to
// themselves: gather g (load_f), h = Phi(g; F_n), scatter h (store_f). The adjoint of step k is
// therefore local and in place: with lambda^{k+1} read at the store positions (hbar), the cell
// computes gbar = (dPhi/dg)^T hbar + dj_k/dg and writes it at the load positions; solid cells map
// their slots identically; F_bar accumulates (dPhi/dF)^T hbar. Objectives (averaged over a window
// of time steps k, each term a function of the state after k steps):
//   OBJ_KE_PLANE: mean over fluid cells of plane x=X of 1/2 rho |u|^2, rho/u as update_fields gives;
//   OBJ_DRAG_X:   sum over cells with flags==marker of F_x from update_force_field (= 2 m_x).
extern "C" struct OracleObjective {
	u32 kind;        // 1: OBJ_KE_PLANE, 2: OBJ_DRAG_X
	u32 plane_x;     // OBJ_KE_PLANE
	u32 marker;      // OBJ_DRAG_X
	u32 pad;
	u64 t_begin, t_end; // window [t_begin, t_end] of time steps (inclusive)
};
enum { OBJ_KE_PLANE = 1, OBJ_DRAG_X = 2 };

struct CellFwd { // forward quantities of one fluid cell needed by its adjoint
	double rho, m[3], u0[3], v[3], u[3], Ft[3], rho2, c3;
	bool kappa[3];
};

static void cell_forward_f64(const OracleConfig* c, const double* g, const bool is_e, const double rho_p, const double* u_p, const double* Ft, CellFwd& s) {
	const u32 q = c->q;
	const bool vf = (c->ext&EXT_VOLUME_FORCE)!=0u;
	const double cs = sound_speed<double>();
	if(is_e) { s.rho = rho_p; for(int d=0; d<3; d++) { s.u0[d] = u_p[d]; s.m[d] = 0.0; } }
	else {
		double rho = 0.0; for(u32 i=0u; i<q; i++) rho += g[i]; rho += 1.0;
		s.rho = rho;
		for(int d=0; d<3; d++) { double m = 0.0; for(u32 i=1u; i<q; i++) m += cq(q, d, i)*g[i]; s.m[d] = m; s.u0[d] = m/rho; }
	}
	s.rho2 = 0.5/s.rho;
	for(int d=0; d<3; d++) {
		s.Ft[d] = Ft[d];
		s.v[d] = vf ? s.u0[d]+Ft[d]*s.rho2 : s.u0[d];
		s.kappa[d] = s.v[d]>-cs && s.v[d]<cs;
		s.u[d] = std::fmin(std::fmax(s.v[d], -cs), cs);
	}
	s.c3 = -3.0*(s.u[0]*s.u[0]+s.u[1]*s.u[1]+s.u[2]*s.u[2]);
}

// gbar = (dh/dg)^T hbar (+ objective ke_weight * d(1/2 rho |u|^2)/dg) and Fbar += (dh/dF_total)^T hbar
static void cell_adjoint_f64(const OracleConfig* c, const CellFwd& s, const bool is_e, const double* hbar, const double ke_weight, double* gbar, double* Fbar) {
	const u32 q = c->q;
	const bool vf = (c->ext&EXT_VOLUME_FORCE)!=0u;
	const Weights<double> W = weights<double>(q);
	const double w = c->w;
	const double wm = 1.0/(0.1875/(1.0/w-0.5)+0.5);
	const double hp = 0.5*w, hm = 0.5*wm, c_tau = 1.0-0.5*w, c_taup = 0.5-0.25*w, c_taum = 0.5-0.25*wm;
	double feqbar[27], Gbar[27];
	for(u32 i=0u; i<q; i++) { gbar[i] = 0.0; feqbar[i] = 0.0; Gbar[i] = 0.0; }
	if(is_e) {
		for(u32 i=0u; i<q; i++) feqbar[i] = hbar[i];
	} else if(!c->trt) {
		for(u32 i=0u; i<q; i++) { gbar[i] = (1.0-w)*hbar[i]; feqbar[i] = w*hbar[i]; Gbar[i] = c_tau*hbar[i]; }
	} else {
		gbar[0] = (1.0-2.0*hp)*hbar[0]; feqbar[0] = 2.0*hp*hbar[0]; Gbar[0] = 2.0*c_taup*hbar[0];
		for(u32 i=1u; i<q; i+=2u) {
			const double a = hbar[i], b = hbar[i+1u];
			const double di = hp*(a+b)+hm*(a-b), dj = hp*(a+b)-hm*(a-b);
			gbar[i] = a-di; gbar[i+1u] = b-dj; feqbar[i] = di; feqbar[i+1u] = dj;
			Gbar[i] = c_taup*(a+b)+c_taum*(a-b); Gbar[i+1u] = c_taup*(a+b)-c_taum*(a-b);
		}
	}
	// equilibrium: feq_i = w_i (rho (0.5 (uk^2 + c3) + uk) + rho - 1), uk = 3 c_i.u, c3 = -3 |u|^2
	double rhobar = 0.0, ubar[3] = {0.0, 0.0, 0.0};
	for(u32 i=0u; i<q; i++) {
		const double wi = weight(W, i);
		double uk = 0.0; for(int d=0; d<3; d++) uk += 3.0*cq(q, d, i)*s.u[d];
		rhobar += feqbar[i]*wi*(0.5*(uk*uk+s.c3)+uk+1.0);
		for(int d=0; d<3; d++) ubar[d] += feqbar[i]*wi*s.rho*(3.0*cq(q, d, i)*(uk+1.0)-3.0*s.u[d]);
	}
	// Guo forcing: G_i = 9 w_i (cf (cu + 1/3) + uF), cf = c_i.Ft, cu = c_i.u, uF = -u.Ft/3
	double Ftbar[3] = {0.0, 0.0, 0.0};
	if(vf && !is_e) {
		for(u32 i=0u; i<q; i++) {
			const double wi9 = 9.0*weight(W, i);
			double cf = 0.0, cu = 0.0; for(int d=0; d<3; d++) { cf += cq(q, d, i)*s.Ft[d]; cu += cq(q, d, i)*s.u[d]; }
			for(int d=0; d<3; d++) {
				ubar[d] += Gbar[i]*wi9*(cf*cq(q, d, i)-s.Ft[d]/3.0);
				Ftbar[d] += Gbar[i]*wi9*(cq(q, d, i)*(cu+1.0/3.0)-s.u[d]/3.0);
			}
		}
	}
	if(ke_weight!=0.0 && !is_e) { // objective term 1/2 rho |u|^2 of this cell
		rhobar += ke_weight*0.5*(s.u[0]*s.u[0]+s.u[1]*s.u[1]+s.u[2]*s.u[2]);
		for(int d=0; d<3; d++) ubar[d] += ke_weight*s.rho*s.u[d];
	}
	// clamp, force shift u = u0 + Ft*0.5/rho, u0 = m/rho
	double u0bar[3], rho2bar = 0.0;
	for(int d=0; d<3; d++) {
		const double vbar = s.kappa[d] ? ubar[d] : 0.0;
		u0bar[d] = vbar;
		if(vf) { Ftbar[d] += vbar*s.rho2; rho2bar += vbar*s.Ft[d]; }
	}
	if(!is_e) {
		rhobar += rho2bar*(-0.5/(s.rho*s.rho));
		double mbar[3];
		for(int d=0; d<3; d++) { mbar[d] = u0bar[d]/s.rho; rhobar -= u0bar[d]*s.u0[d]/s.rho; }
		for(u32 i=0u; i<q; i++) {
			gbar[i] += rhobar;
			for(int d=0; d<3; d++) gbar[i] += cq(q, d, i)*mbar[d];
		}
	}
	for(int d=0; d<3; d++) Fbar[d] += Ftbar[d];
}

// objective of the state at time step t (f in FP64 storage), and its gradient added to lambda when lambda != nullptr
static double objective_state_f64(const OracleConfig* c, const OracleObjective* obj, const double* f, const u8* flags, const double* rho_p, const double* u_p,
                                  const double* F, const double fx, const double fy, const double fz, const u64 t, const double weight, double* lambda,
                                  double* grad) {
	const Grid G(c); const u32 q = c->q;
	const bool ff = (c->ext&EXT_FORCE_FIELD)!=0u, eq = (c->ext&EXT_EQUILIBRIUM_BOUNDARIES)!=0u;
	double J = 0.0;
	for(u64 n=0ull; n<G.N; n++) {
		const u8 fl = flags[n];
		u32 x, y, z; G.coords(n, x, y, z);
		const bool solid = (fl&T_BO)==T_S;
		if(obj->kind==OBJ_KE_PLANE) {
			if(x!=obj->plane_x || solid || (fl&T_SU)==T_G || (eq && (fl&T_BO)==T_E)) continue;
		} else {
			if(fl!=(u8)obj->marker) continue;
		}
		u64 j[27]; G.neighbors(n, q, j);
		double g[27]; load_f<double>(n, g, f, j, t, q, G.N, ST_FP32);
		double slot_grad[27];
		if(obj->kind==OBJ_KE_PLANE) {
			CellFwd s;
			const double Ft[3] = {fx+(ff ? F[n] : 0.0), fy+(ff ? F[G.N+n] : 0.0), fz+(ff ? F[2ull*G.N+n] : 0.0)};
			const double up[3] = {u_p[n], u_p[G.N+n], u_p[2ull*G.N+n]};
			cell_forward_f64(c, g, false, rho_p[n], up, Ft, s);
			J += weight*0.5*s.rho*(s.u[0]*s.u[0]+s.u[1]*s.u[1]+s.u[2]*s.u[2]);
			if(!lambda) continue;
			double zero[27] = {0.0}, Fb[3] = {0.0, 0.0, 0.0};
			cell_adjoint_f64(c, s, false, zero, weight, slot_grad, Fb);
			if(ff && grad) { grad[n] += Fb[0]; grad[G.N+n] += Fb[1]; grad[2ull*G.N+n] += Fb[2]; } // the velocity includes F/(2 rho)
		} else {
			double m = 0.0; for(u32 i=1u; i<q; i++) m += cq(q, 0, i)*g[i];
			J += weight*2.0*m;
			if(!lambda) continue;
			for(u32 i=0u; i<q; i++) slot_grad[i] = weight*2.0*cq(q, 0, i);
		}
		// add at the load positions of parity t
		lambda[n] += slot_grad[0];
		for(u32 i=1u; i<q; i+=2u) {
			lambda[(u64)(t%2ull ? i : i+1u)*G.N+n] += slot_grad[i];
			lambda[(u64)(t%2ull ? i+1u : i)*G.N+j[i]] += slot_grad[i+1u];
		}
	}
	return J;
}

static double obj_weight(const OracleObjective* obj, const Grid& G, const u8* flags, const OracleConfig* c, const u64 t) {
	if(t<obj->t_begin||t>obj->t_end) return 0.0;
	const double steps = (double)(obj->t_end-obj->t_begin+1ull);
	if(obj->kind==OBJ_DRAG_X) return 1.0/steps;
	u64 cells = 0ull; // fluid cells of the plane
	const bool eq = (c->ext&EXT_EQUILIBRIUM_BOUNDARIES)!=0u;
	for(u64 n=0ull; n<G.N; n++) {
		u32 x, y, z; G.coords(n, x, y, z);
		const u8 fl = flags[n];
		if(x==obj->plane_x && (fl&T_BO)!=T_S && (fl&T_SU)!=T_G && !(eq && (fl&T_BO)==T_E)) cells++;
	}
	return cells ? 1.0/(steps*(double)cells) : 0.0;
}

// lambda^k = A_k^T lambda^{k+1} in place (fluid cells; solid and gas cells map their slots identically),
// grad += (dPhi_k/dF)^T lambda^{k+1}
static void adjoint_step_f64(const OracleConfig* c, const double* f, double* lambda, const u8* flags, const double* rho_p, const double* u_p,
                             const double* F, const double fx, const double fy, const double fz, const u64 t, double* grad) {
	const Grid G(c); const u32 q = c->q;
	const bool ff = (c->ext&EXT_FORCE_FIELD)!=0u, eq = (c->ext&EXT_EQUILIBRIUM_BOUNDARIES)!=0u;
	parallel_cells(G.N, c->threads, [&](const u64 n) {
		const u8 fl = flags[n];
		if((fl&T_BO)==T_S||(fl&T_SU)==T_G) return;
		u64 j[27]; G.neighbors(n, q, j);
		double g[27], hbar[27], gbar[27];
		load_f<double>(n, g, f, j, t, q, G.N, ST_FP32);
		u64 A[27], B[27];
		hbar[0] = lambda[n];
		for(u32 i=1u; i<q; i+=2u) {
			A[i] = (u64)(t%2ull ? i : i+1u)*G.N+n; B[i] = (u64)(t%2ull ? i+1u : i)*G.N+j[i];
			hbar[i] = lambda[B[i]]; hbar[i+1u] = lambda[A[i]];
		}
		const bool is_e = eq && (fl&T_BO)==T_E;
		const double Ft[3] = {fx+(ff ? F[n] : 0.0), fy+(ff ? F[G.N+n] : 0.0), fz+(ff ? F[2ull*G.N+n] : 0.0)};
		const double up[3] = {u_p[n], u_p[G.N+n], u_p[2ull*G.N+n]};
		CellFwd s;
		cell_forward_f64(c, g, is_e, rho_p[n], up, Ft, s);
		double Fb[3] = {0.0, 0.0, 0.0};
		cell_adjoint_f64(c, s, is_e, hbar, 0.0, gbar, Fb);
		lambda[n] = gbar[0];
		for(u32 i=1u; i<q; i+=2u) { lambda[A[i]] = gbar[i]; lambda[B[i]] = gbar[i+1u]; }
		if(ff && grad) { grad[n] += Fb[0]; grad[G.N+n] += Fb[1]; grad[2ull*G.N+n] += Fb[2]; }
	});
}

extern "C" {

// J of a forward run of `steps` steps from the initialised state f0 (copied, not modified)
double oracle_objective_f64(const OracleConfig* c, const double* f0, const u8* flags, const double* rho_p, const double* u_p, const double* F,
                            const double fx, const double fy, const double fz, const u64 steps, const OracleObjective* obj) {
	const Grid G(c);
	OracleConfig cf = *c; cf.ext &= ~(u32)EXT_UPDATE_FIELDS; // the forward steps leave rho/u alone (they are inputs here)
	std::vector<double> f(f0, f0+(size_t)c->q*G.N);
	double J = 0.0;
	for(u64 t=0ull; t<=steps; t++) {
		const double wgt = obj_weight(obj, G, flags, c, t);
		if(wgt!=0.0) J += objective_state_f64(c, obj, f.data(), flags, rho_p, u_p, F, fx, fy, fz, t, wgt, nullptr, nullptr);
		if(t<steps) stream_collide_t<double>(&cf, f.data(), const_cast<double*>(rho_p), const_cast<double*>(u_p), flags, t, fx, fy, fz, F);
	}
	return J;
}

// J and dJ/dF (grad, 3N, overwritten) by the checkpointed discrete adjoint: snapshots every
// `interval` steps in the forward sweep, each segment recomputed from its snapshot in the reverse sweep
int oracle_adjoint_f64(const OracleConfig* c, const double* f0, const u8* flags, const double* rho_p, const double* u_p, const double* F,
                       const double fx, const double fy, const double fz, const u64 steps, const OracleObjective* obj, const u64 interval,
                       double* J_out, double* grad) {
	if(!valid(c)||interval==0ull) return -1;
	const Grid G(c);
	OracleConfig cf = *c; cf.ext &= ~(u32)EXT_UPDATE_FIELDS; // the forward steps leave rho/u alone (they are inputs here)
	const size_t S = (size_t)c->q*G.N;
	std::vector<std::vector<double>> snaps;
	std::vector<double> f(f0, f0+S);
	double J = 0.0;
	for(u64 t=0ull; t<=steps; t++) {
		if(t%interval==0ull && t<steps) snaps.push_back(f);
		const double wgt = obj_weight(obj, G, flags, c, t);
		if(wgt!=0.0) J += objective_state_f64(c, obj, f.data(), flags, rho_p, u_p, F, fx, fy, fz, t, wgt, nullptr, nullptr);
		if(t<steps) stream_collide_t<double>(&cf, f.data(), const_cast<double*>(rho_p), const_cast<double*>(u_p), flags, t, fx, fy, fz, F);
	}
	std::vector<double> lambda(S, 0.0);
	for(size_t i=0u; i<3u*G.N; i++) grad[i] = 0.0;
	{ const double wgt = obj_weight(obj, G, flags, c, steps); if(wgt!=0.0) objective_state_f64(c, obj, f.data(), flags, rho_p, u_p, F, fx, fy, fz, steps, wgt, lambda.data(), grad); }
	std::vector<std::vector<double>> seg;
	for(u64 s=snaps.size(); s-->0ull;) {
		const u64 k0 = s*interval, k1 = std::min<u64>(k0+interval, steps);
		seg.assign((size_t)(k1-k0), std::vector<double>());
		std::vector<double> w = snaps[(size_t)s];
		for(u64 k=k0; k<k1; k++) {
			seg[(size_t)(k-k0)] = w;
			if(k+1ull<k1) stream_collide_t<double>(&cf, w.data(), const_cast<double*>(rho_p), const_cast<double*>(u_p), flags, k, fx, fy, fz, F);
		}
		for(u64 k=k1; k-->k0;) {
			const std::vector<double>& fk = seg[(size_t)(k-k0)];
			adjoint_step_f64(c, fk.data(), lambda.data(), flags, rho_p, u_p, F, fx, fy, fz, k, grad);
			const double wgt = obj_weight(obj, G, flags, c, k);
			if(wgt!=0.0) objective_state_f64(c, obj, fk.data(), flags, rho_p, u_p, F, fx, fy, fz, k, wgt, lambda.data(), grad);
		}
	}
	*J_out = J;
	return 0;
}

} // extern "C"
