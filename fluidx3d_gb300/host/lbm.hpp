// C++ host layer with the reference's LBM interface (src/lbm.hpp:208-611, src/lbm.cpp:700-1145)
// over the C-ABI of include/lbm_capi.h. Header-only: a setup written against the reference's
// `class LBM` compiles against this header and links libfluidx3d_gb300.so.
//
// The variant is chosen the way the reference chooses it, with macros defined before this header
// is included (src/defines.hpp:5-29): D3Q19 (default) or D3Q27; SRT (default) or TRT; FP16S or
// FP16C DDF storage (default FP32); VOLUME_FORCE, FORCE_FIELD, EQUILIBRIUM_BOUNDARIES, SUBGRID, MOVING_BOUNDARIES;
// and, new here,
// EXACT_ARITHMETIC / FAST_ARITHMETIC (default: exact with FP32 storage, fast with FP16S/FP16C).
//
// Errors: the reference prints and exits (src/utilities.hpp:4159-4166); here a failed call throws
// lbm_error carrying the C-ABI status and message (uncaught, it ends the program the same way).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iterator>
#include <algorithm>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>
#include "lbm_capi.h"

typedef unsigned char uchar;
typedef unsigned int uint;
typedef uint64_t ulong;

#ifndef TYPE_S
#define TYPE_S 0b00000001 // (stationary) solid boundary
#define TYPE_E 0b00000010 // equilibrium boundary (inflow/outflow)
#define TYPE_T 0b00000100 // temperature boundary (not used by this solver core)
#define TYPE_F 0b00001000 // fluid (free surface; not used by this solver core)
#define TYPE_I 0b00010000 // interface (free surface; not used by this solver core)
#define TYPE_G 0b00100000 // gas (free surface; cells are skipped)
#define TYPE_X 0b01000000 // reserved type X
#define TYPE_Y 0b10000000 // reserved type Y
#endif

struct lbm_error : std::runtime_error {
	int status;
	lbm_error(const int s, const std::string& m) : std::runtime_error(m), status(s) {}
};
inline void lbm_check(const int status) {
	if(status!=LBM_OK) throw lbm_error(status, std::string("lbm: ")+lbm_last_error());
}

struct float3 {
	float x = 0.0f, y = 0.0f, z = 0.0f;
	float3() = default;
	explicit float3(const float s) : x(s), y(s), z(s) {}
	float3(const float x, const float y, const float z) : x(x), y(y), z(z) {}
	float3& operator+=(const float3& o) { x += o.x; y += o.y; z += o.z; return *this; }
};
inline float3 operator+(const float3& a, const float3& b) { return float3(a.x+b.x, a.y+b.y, a.z+b.z); }
inline float3 operator-(const float3& a, const float3& b) { return float3(a.x-b.x, a.y-b.y, a.z-b.z); }
inline float3 operator*(const float s, const float3& a) { return float3(s*a.x, s*a.y, s*a.z); }
inline float3 operator/(const float3& a, const float s) { return float3(a.x/s, a.y/s, a.z/s); }
inline float length(const float3& a) { return std::sqrt(a.x*a.x+a.y*a.y+a.z*a.z); }
struct uint3 {
	uint x = 0u, y = 0u, z = 0u;
	uint3() = default;
	uint3(const uint x, const uint y, const uint z) : x(x), y(y), z(z) {}
};

// triangle mesh (src/utilities.hpp:4440-4528)
struct Mesh {
	uint triangle_number = 0u;
	float3 center, pmin, pmax;
	std::vector<float3> p0, p1, p2;
	Mesh(const uint triangle_number, const float3& center) : triangle_number(triangle_number), center(center), pmin(center), pmax(center),
		p0(triangle_number), p1(triangle_number), p2(triangle_number) {}
	void find_bounds() {
		pmin = pmax = p0[0];
		for(uint i=0u; i<triangle_number; i++) {
			const float3 a = p0[i], b = p1[i], c = p2[i];
			pmin.x = std::fmin(std::fmin(std::fmin(a.x, b.x), c.x), pmin.x); pmax.x = std::fmax(std::fmax(std::fmax(a.x, b.x), c.x), pmax.x);
			pmin.y = std::fmin(std::fmin(std::fmin(a.y, b.y), c.y), pmin.y); pmax.y = std::fmax(std::fmax(std::fmax(a.y, b.y), c.y), pmax.y);
			pmin.z = std::fmin(std::fmin(std::fmin(a.z, b.z), c.z), pmin.z); pmax.z = std::fmax(std::fmax(std::fmax(a.z, b.z), c.z), pmax.z);
		}
	}
	void translate(const float3& t) {
		for(uint i=0u; i<triangle_number; i++) { p0[i] += t; p1[i] += t; p2[i] += t; }
		center += t; pmin += t; pmax += t;
	}
};

// binary STL file without rescaling (src/utilities.hpp:4530-4581 read_stl_raw with reposition=false, scale 1)
inline Mesh* read_stl(const std::string& path) {
	std::ifstream file(path, std::ios::in|std::ios::binary);
	if(!file) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+path+"\" does not exist!");
	std::vector<char> data((std::istreambuf_iterator<char>(file)), std::istreambuf_iterator<char>());
	if(data.size()<84u) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+path+"\" is corrupt!");
	uint T = 0u;
	std::memcpy(&T, data.data()+80, 4);
	if(T==0u||data.size()!=84u+50u*(size_t)T) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+path+"\" is corrupt or unsupported! Only binary .stl files are supported.");
	Mesh* mesh = new Mesh(T, float3(0.0f));
	for(uint i=0u; i<T; i++) {
		float v[12];
		std::memcpy(v, data.data()+84u+50u*(size_t)i, 48);
		mesh->p0[i] = float3(v[3], v[4], v[5]); mesh->p1[i] = float3(v[6], v[7], v[8]); mesh->p2[i] = float3(v[9], v[10], v[11]);
	}
	mesh->find_bounds();
	return mesh;
}

// the variant the including setup selected with the reference's macros
inline lbm_config lbm_config_from_defines(const uint Nx, const uint Ny, const uint Nz, const float nu, const float fx, const float fy, const float fz) {
	lbm_config c{};
	c.Nx = Nx; c.Ny = Ny; c.Nz = Nz;
#if defined(D3Q27)
	c.velocity_set = 27u;
#else
	c.velocity_set = 19u;
#endif
#if defined(TRT)
	c.collision = LBM_TRT;
#else
	c.collision = LBM_SRT;
#endif
#if defined(FP16S)
	c.storage = LBM_FP16S;
#elif defined(FP16C)
	c.storage = LBM_FP16C;
#else
	c.storage = LBM_FP32;
#endif
	c.extensions = 0u;
#if defined(VOLUME_FORCE)
	c.extensions |= LBM_EXT_VOLUME_FORCE;
#endif
#if defined(FORCE_FIELD)
	c.extensions |= LBM_EXT_FORCE_FIELD;
#endif
#if defined(EQUILIBRIUM_BOUNDARIES)
	c.extensions |= LBM_EXT_EQUILIBRIUM_BOUNDARIES;
#endif
#if defined(MOVING_BOUNDARIES)
	c.extensions |= LBM_EXT_MOVING_BOUNDARIES;
#endif
#if defined(SUBGRID)
	c.extensions |= LBM_EXT_SUBGRID;
#endif
	c.device = -1;
	c.nu = nu; c.fx = fx; c.fy = fy; c.fz = fz;
#if defined(EXACT_ARITHMETIC)
	c.arithmetic = LBM_ARITH_EXACT; // the reference's FP32 operation order, bit for bit
#elif defined(FAST_ARITHMETIC)
	c.arithmetic = LBM_ARITH_FAST;
#else
	c.arithmetic = LBM_ARITH_AUTO;  // exact with FP32 storage, fast with FP16S/FP16C
#endif
	return c;
}

class LBM {
	uint Nx = 1u, Ny = 1u, Nz = 1u;
	float nu = 1.0f/6.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
	lbm_domain* domain = nullptr;
	bool initialized = false;

public:
	// host buffer of one device field (the reference's Memory_Container, src/lbm.hpp:239-408)
	template<typename T> class Memory_Container {
		LBM* lbm = nullptr;
		int field = 0;
		uint d = 1u;
		ulong N = 0ull;
		std::vector<T> data;
	public:
		class Pointer {
			Memory_Container* m = nullptr;
			uint dim = 0u;
		public:
			Pointer() = default;
			Pointer(Memory_Container* m, const uint dim) : m(m), dim(dim) {}
			T& operator[](const ulong i) { return m->data[i+(ulong)dim*m->N]; }
			const T& operator[](const ulong i) const { return m->data[i+(ulong)dim*m->N]; }
		};
		Pointer x, y, z;
		Memory_Container() = default;
		Memory_Container(LBM* lbm, const int field, const uint d, const T init) : lbm(lbm), field(field), d(d), N(lbm->get_N()), data(N*d, init) {
			x = Pointer(this, 0u);
			if(d>1u) { y = Pointer(this, 1u); z = Pointer(this, 2u); }
		}
		Memory_Container(const Memory_Container&) = delete;
		Memory_Container& operator=(const Memory_Container&) = delete;
		T& operator[](const ulong i) { return data[i]; }
		const T& operator[](const ulong i) const { return data[i]; }
		T operator()(const ulong i, const uint dim) const { return data[i+(ulong)dim*N]; }
		ulong length() const { return N; }
		uint dimensions() const { return d; }
		ulong range() const { return N*(ulong)d; }
		ulong capacity() const { return N*(ulong)d*sizeof(T); }
		T* host() { return data.data(); }
		void reset(const T value=(T)0) { std::fill(data.begin(), data.end(), value); }
		void read_from_device() { lbm_check(lbm_read_field(lbm->domain, field, data.data(), capacity())); } // updates rho/u first when stale
		void write_to_device() { lbm_check(lbm_write_field(lbm->domain, field, data.data(), capacity())); }
	};

	Memory_Container<float> rho, u, F;
	Memory_Container<uchar> flags;

	LBM(const uint Nx, const uint Ny, const uint Nz, const float nu, const float fx=0.0f, const float fy=0.0f, const float fz=0.0f)
		: Nx(Nx), Ny(Ny), Nz(Nz), nu(nu), fx(fx), fy(fy), fz(fz),
		  rho(this, LBM_FIELD_RHO, 1u, 1.0f), u(this, LBM_FIELD_U, 3u, 0.0f), F(this, LBM_FIELD_F, 3u, 0.0f), flags(this, LBM_FIELD_FLAGS, 1u, (uchar)0u) {
		const lbm_config c = lbm_config_from_defines(Nx, Ny, Nz, nu, fx, fy, fz);
		lbm_check(lbm_domain_create(&c, &domain)); // replaces device selection, JIT and allocate() (src/lbm.cpp:96-176)
	}
	LBM(const uint3 N, const float nu, const float fx=0.0f, const float fy=0.0f, const float fz=0.0f) : LBM(N.x, N.y, N.z, nu, fx, fy, fz) {}
	// multi-domain constructor of the reference: one domain per GPU is the only decomposition here
	LBM(const uint Nx, const uint Ny, const uint Nz, const uint Dx, const uint Dy, const uint Dz, const float nu, const float fx=0.0f, const float fy=0.0f, const float fz=0.0f)
		: LBM(Nx, Ny, Nz, nu, fx, fy, fz) {
		if(Dx*Dy*Dz!=1u) throw lbm_error(LBM_ERR_UNSUPPORTED, "lbm: this solver core runs one domain on one GPU (Dx=Dy=Dz=1)");
	}
	LBM(const LBM&) = delete;
	LBM& operator=(const LBM&) = delete;
	~LBM() { lbm_domain_destroy(domain); }

	lbm_domain* handle() const { return domain; }

	void initialize() { // src/lbm.cpp:881-922: host fields to the device, initialize kernel at odd parity, t = 0
		rho.write_to_device();
		u.write_to_device();
		flags.write_to_device();
#ifdef FORCE_FIELD
		F.write_to_device();
#endif
		lbm_check(lbm_initialize(domain));
		initialized = true;
	}
	void run(const ulong steps=1ull, const ulong total_steps=0ull) { // src/lbm.cpp:955-975
		(void)total_steps;
		if(!initialized) initialize();
		lbm_check(lbm_stream_collide(domain, steps));
	}
	void update_fields() { lbm_check(lbm_update_fields(domain)); lbm_check(lbm_synchronize(domain)); }
	void reset() { lbm_check(lbm_reset(domain)); initialized = false; }
	void finish() { lbm_check(lbm_synchronize(domain)); }

	void update_force_field() { lbm_check(lbm_update_force_field(domain)); lbm_check(lbm_synchronize(domain)); }
	void reset_force_field() { lbm_check(lbm_reset_force_field(domain)); }
#if defined(MOVING_BOUNDARIES)
	void update_moving_boundaries() { // src/lbm.cpp:1019-1023
		lbm_check(lbm_update_moving_boundaries(domain));
		if(!initialized) flags.read_from_device();
	}
#endif
	float3 object_center_of_mass(const uchar flag_marker=TYPE_S) {
		double o[4];
		lbm_check(lbm_object_center_of_mass(domain, flag_marker, o));
		return float3((float)o[0], (float)o[1], (float)o[2]);
	}
	float3 object_force(const uchar flag_marker=TYPE_S) {
		double o[3];
		lbm_check(lbm_object_force(domain, flag_marker, o));
		return float3((float)o[0], (float)o[1], (float)o[2]);
	}
	float3 object_torque(const float3& rotation_center, const uchar flag_marker=TYPE_S) {
		double o[3];
		lbm_check(lbm_object_torque(domain, flag_marker, rotation_center.x, rotation_center.y, rotation_center.z, o));
		return float3((float)o[0], (float)o[1], (float)o[2]);
	}

	void voxelize_mesh_on_device(const Mesh* mesh, const uchar flag=TYPE_S, const float3& rotation_center=float3(0.0f),
	                             const float3& linear_velocity=float3(0.0f), const float3& rotational_velocity=float3(0.0f)) { // src/lbm.cpp:1074-1089
		const float c[3] = {rotation_center.x, rotation_center.y, rotation_center.z};
		const float lv[3] = {linear_velocity.x, linear_velocity.y, linear_velocity.z};
		const float rv[3] = {rotational_velocity.x, rotational_velocity.y, rotational_velocity.z};
		lbm_check(lbm_voxelize_mesh(domain, &mesh->p0[0].x, &mesh->p1[0].x, &mesh->p2[0].x, mesh->triangle_number, flag, c, lv, rv));
		if(!initialized) { flags.read_from_device(); u.read_from_device(); }
	}
	void unvoxelize_mesh_on_device(const Mesh* mesh, const uchar flag=TYPE_S) {
		const float lo[3] = {mesh->pmin.x, mesh->pmin.y, mesh->pmin.z}, hi[3] = {mesh->pmax.x, mesh->pmax.y, mesh->pmax.z};
		lbm_check(lbm_unvoxelize_mesh(domain, lo, hi, flag));
	}
	void voxelize_stl(const std::string& path, const uchar flag=TYPE_S) { // file coordinates are lattice coordinates
		Mesh* mesh = read_stl(path);
		flags.write_to_device();
		voxelize_mesh_on_device(mesh, flag);
		delete mesh;
		flags.read_from_device();
	}

	uint get_Nx() const { return Nx; }
	uint get_Ny() const { return Ny; }
	uint get_Nz() const { return Nz; }
	ulong get_N() const { return (ulong)Nx*(ulong)Ny*(ulong)Nz; }
	uint get_D() const { return 1u; }
	float get_nu() const { return nu; }
	float get_tau() const { return 3.0f*nu+0.5f; }
	float get_fx() const { return fx; }
	float get_fy() const { return fy; }
	float get_fz() const { return fz; }
	ulong get_t() const { uint64_t t = 0ull; lbm_check(lbm_get_time_step(domain, &t)); return t; }
	uint get_velocity_set() const {
#if defined(D3Q27)
		return 27u;
#else
		return 19u;
#endif
	}
	void set_f(const float fx, const float fy, const float fz) { lbm_check(lbm_set_force(domain, fx, fy, fz)); this->fx = fx; this->fy = fy; this->fz = fz; }
	void set_fx(const float v) { set_f(v, fy, fz); }
	void set_fy(const float v) { set_f(fx, v, fz); }
	void set_fz(const float v) { set_f(fx, fy, v); }

	void coordinates(const ulong n, uint& x, uint& y, uint& z) const { // src/lbm.hpp:478-483
		const ulong t = n%((ulong)Nx*(ulong)Ny);
		x = (uint)(t%(ulong)Nx); y = (uint)(t/(ulong)Nx); z = (uint)(n/((ulong)Nx*(ulong)Ny));
	}
	ulong index(const uint x, const uint y, const uint z) const { return (ulong)x+((ulong)y+(ulong)z*(ulong)Ny)*(ulong)Nx; }
	float3 position(const uint x, const uint y, const uint z) const { return float3((float)x-0.5f*(float)Nx+0.5f, (float)y-0.5f*(float)Ny+0.5f, (float)z-0.5f*(float)Nz+0.5f); }
	float3 size() const { return float3((float)Nx, (float)Ny, (float)Nz); }
	float3 center() const { return float3(0.5f*(float)Nx-0.5f, 0.5f*(float)Ny-0.5f, 0.5f*(float)Nz-0.5f); }
};
