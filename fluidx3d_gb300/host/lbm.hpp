// C++ host layer with the reference's LBM interface (src/lbm.hpp:208-611, src/lbm.cpp:700-1145)
// over the C-ABI of include/lbm_capi.h. Header-only: a setup written against the reference's
// `class LBM` compiles against this header and links libfluidx3d_gb300.so.
//
// The variant is chosen the way the reference chooses it, with macros defined before this header
// is included (src/defines.hpp:5-29): D3Q19 (default) or D3Q27; SRT (default) or TRT; FP16S or
// FP16C DDF storage (default FP32); VOLUME_FORCE, FORCE_FIELD, EQUILIBRIUM_BOUNDARIES, SUBGRID, MOVING_BOUNDARIES,
// UPDATE_FIELDS;
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
#include <filesystem>
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
inline float3 operator*(const float3& a, const float s) { return float3(a.x*s, a.y*s, a.z*s); }
inline float3 operator-(const float3& a) { return float3(-a.x, -a.y, -a.z); }
// 3x3 matrix, row-major (src/utilities.hpp float3x3); m*v sums each row left to right
struct float3x3 {
	float xx = 1.0f, xy = 0.0f, xz = 0.0f, yx = 0.0f, yy = 1.0f, yz = 0.0f, zx = 0.0f, zy = 0.0f, zz = 1.0f;
	float3x3() = default;
	explicit float3x3(const float s) : xx(s), xy(0.0f), xz(0.0f), yx(0.0f), yy(s), yz(0.0f), zx(0.0f), zy(0.0f), zz(s) {}
	float3x3(const float xx, const float xy, const float xz, const float yx, const float yy, const float yz, const float zx, const float zy, const float zz)
		: xx(xx), xy(xy), xz(xz), yx(yx), yy(yy), yz(yz), zx(zx), zy(zy), zz(zz) {}
};
inline float3 operator*(const float3x3& m, const float3& v) { return float3(m.xx*v.x+m.xy*v.y+m.xz*v.z, m.yx*v.x+m.yy*v.y+m.yz*v.z, m.zx*v.x+m.zy*v.y+m.zz*v.z); }

// unit conversion lattice <-> SI (src/units.hpp:5-75); `units` is the program-wide instance, identity by default
class Units {
public:
	float unit_m = 1.0f, unit_kg = 1.0f, unit_s = 1.0f;
	void set_m_kg_s(const float x, const float u, const float rho, const float si_x, const float si_u, const float si_rho) {
		unit_m = si_x/x;
		unit_kg = si_rho/rho*(unit_m*unit_m*unit_m);
		unit_s = u/si_u*unit_m;
	}
	void set_m_kg_s(const float m, const float kg, const float s) { unit_m = m; unit_kg = kg; unit_s = s; }
	float x(const float si_x) const { return si_x/unit_m; }
	float u(const float si_u) const { return si_u*unit_s/unit_m; }
	float rho(const float si_rho) const { return si_rho*(unit_m*unit_m*unit_m)/unit_kg; }
	float nu(const float si_nu) const { return si_nu*unit_s/(unit_m*unit_m); }
	float F(const float si_F) const { return si_F*(unit_s*unit_s)/(unit_kg*unit_m); }
	ulong t(const float si_t) const { return (ulong)std::fmax(si_t/unit_s+0.5f, 0.5f); }
	float si_x(const float x) const { return x*unit_m; }
	float si_t(const ulong t) const { return (float)t*unit_s; }
	float si_u(const float u) const { return u*unit_m/unit_s; }
	float si_rho(const float rho) const { return rho*unit_kg/(unit_m*unit_m*unit_m); }
	float si_nu(const float nu) const { return nu*(unit_m*unit_m)/unit_s; }
	float si_F(const float F) const { return F*unit_kg*unit_m/(unit_s*unit_s); }
};
inline Units units;

// file names and folders (src/lbm.cpp:85-92, src/utilities.hpp:4197-4207)
inline std::string create_file_extension(const std::string& filename, const std::string& extension) {
	return filename.substr(0, filename.rfind('.'))+(extension.at(0)!='.' ? "." : "")+extension;
}
inline void create_folder(const std::string& path) {
	const size_t slash = path.rfind('/');
	if(slash==std::string::npos||slash==0u) return;
	std::error_code ec;
	std::filesystem::create_directories(path.substr(0u, slash), ec);
}
inline std::string get_exe_path() { // folder of the running executable, with a trailing '/'
	std::error_code ec;
	const std::filesystem::path p = std::filesystem::read_symlink("/proc/self/exe", ec);
	return ec ? std::string("./") : p.parent_path().string()+"/";
}
inline std::string default_filename(const std::string& path, const std::string& name, const std::string& extension, const ulong t) {
	std::string time = "00000000"+std::to_string(t);
	time = time.substr(time.length()-9u, 9u);
	return (path=="" ? get_exe_path()+"export/" : path)+create_file_extension((name=="" ? "file" : name)+"-"+time, extension);
}
template<typename T> inline T reverse_bytes(const T x) {
	T r;
	const unsigned char* a = reinterpret_cast<const unsigned char*>(&x);
	unsigned char* b = reinterpret_cast<unsigned char*>(&r);
	for(size_t i=0u; i<sizeof(T); i++) b[i] = a[sizeof(T)-1u-i];
	return r;
}
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
	float get_max_size() const { return std::fmax(std::fmax(pmax.x-pmin.x, pmax.y-pmin.y), pmax.z-pmin.z); }
	float get_scale_for_box_fit(const float3& b) const { return std::fmin(std::fmin(b.x/(pmax.x-pmin.x), b.y/(pmax.y-pmin.y)), b.z/(pmax.z-pmin.z)); }
};

// binary STL file (src/utilities.hpp:4530-4581 read_stl_raw): vertices rotated, then rescaled (size 0:
// fit box_size; size > 0: longest side = size; size < 0: factor -size) and, with reposition, centred
// on `center`
inline Mesh* read_stl_raw(const std::string& path, const bool reposition, const float3& box_size, const float3& center, const float3x3& rotation, const float size) {
	const std::string filename = create_file_extension(path, ".stl");
	std::ifstream file(filename, std::ios::in|std::ios::binary);
	if(!file) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+filename+"\" does not exist!");
	std::vector<char> data((std::istreambuf_iterator<char>(file)), std::istreambuf_iterator<char>());
	if(data.size()<84u) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+filename+"\" is corrupt!");
	uint T = 0u;
	std::memcpy(&T, data.data()+80, 4);
	if(T==0u||data.size()!=84u+50u*(size_t)T) throw lbm_error(LBM_ERR_INVALID_ARGUMENT, "File \""+filename+"\" is corrupt or unsupported! Only binary .stl files are supported.");
	Mesh* mesh = new Mesh(T, center);
	for(uint i=0u; i<T; i++) {
		float v[12];
		std::memcpy(v, data.data()+84u+50u*(size_t)i, 48);
		mesh->p0[i] = rotation*float3(v[3], v[4], v[5]); mesh->p1[i] = rotation*float3(v[6], v[7], v[8]); mesh->p2[i] = rotation*float3(v[9], v[10], v[11]);
	}
	mesh->find_bounds();
	const float scale = size==0.0f ? mesh->get_scale_for_box_fit(box_size) : size>0.0f ? size/mesh->get_max_size() : -size;
	const float3 offset = reposition ? -(0.5f*(mesh->pmin+mesh->pmax)) : float3(0.0f);
	for(uint i=0u; i<T; i++) {
		mesh->p0[i] = center+scale*(offset+mesh->p0[i]);
		mesh->p1[i] = center+scale*(offset+mesh->p1[i]);
		mesh->p2[i] = center+scale*(offset+mesh->p2[i]);
	}
	mesh->find_bounds();
	return mesh;
}
inline Mesh* read_stl(const std::string& path, const float3& box_size, const float3& center, const float3x3& rotation, const float size) { return read_stl_raw(path, true, box_size, center, rotation, size); }
inline Mesh* read_stl(const std::string& path, const float3& box_size, const float3& center, const float size) { return read_stl_raw(path, true, box_size, center, float3x3(1.0f), size); }
// no rescaling or repositioning: vertices rotated, scaled by |scale| and shifted by offset (file coordinates are lattice coordinates by default)
inline Mesh* read_stl(const std::string& path, const float scale=1.0f, const float3x3& rotation=float3x3(1.0f), const float3& offset=float3(0.0f)) {
	return read_stl_raw(path, false, float3(1.0f), offset, rotation, -std::fabs(scale));
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
#if defined(UPDATE_FIELDS)
	c.extensions |= LBM_EXT_UPDATE_FIELDS;
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
		// binary legacy VTK (src/lbm.hpp:298-340, 401-407), the host copy or straight from the device
		std::string name() const { return field==LBM_FIELD_RHO ? "rho" : field==LBM_FIELD_U ? "u" : field==LBM_FIELD_F ? "F" : "flags"; }
		float si_factor(const bool si) const {
			if(!si) return 1.0f;
			return field==LBM_FIELD_RHO ? units.si_rho(1.0f) : field==LBM_FIELD_U ? units.si_u(1.0f) : field==LBM_FIELD_F ? units.si_F(1.0f) : 1.0f;
		}
		void write_host_to_vtk(const std::string& path="", const bool convert_to_si_units=true) const {
			const std::string filename = create_file_extension(default_filename(path, name(), ".vtk", lbm->get_t()), ".vtk");
			const float spacing = convert_to_si_units ? units.si_x(1.0f) : 1.0f;
			const float factor = si_factor(convert_to_si_units);
			const float3 origin = spacing*float3(0.5f-0.5f*(float)lbm->Nx, 0.5f-0.5f*(float)lbm->Ny, 0.5f-0.5f*(float)lbm->Nz);
			const std::string header = "# vtk DataFile Version 3.0\nFluidX3D "+filename.substr(filename.rfind('/')+1)+"\nBINARY\nDATASET STRUCTURED_POINTS\n"
				"DIMENSIONS "+std::to_string(lbm->Nx)+" "+std::to_string(lbm->Ny)+" "+std::to_string(lbm->Nz)+"\n"
				"ORIGIN "+std::to_string(origin.x)+" "+std::to_string(origin.y)+" "+std::to_string(origin.z)+"\n"
				"SPACING "+std::to_string(spacing)+" "+std::to_string(spacing)+" "+std::to_string(spacing)+"\n"
				"POINT_DATA "+std::to_string(N)+"\n"
				"SCALARS data "+std::string(sizeof(T)==1u ? "unsigned_char" : "float")+" "+std::to_string(d)+"\nLOOKUP_TABLE default\n";
			create_folder(filename);
			std::ofstream file(filename, std::ios::out|std::ios::binary);
			if(!file) throw lbm_error(LBM_ERR_IO, "File \""+filename+"\" cannot be written");
			file.write(header.c_str(), (std::streamsize)header.length());
			std::vector<T> chunk;
			const ulong block = 1ull<<20;
			for(ulong i0=0ull; i0<N; i0+=block) {
				const ulong n1 = i0+block<N ? i0+block : N;
				chunk.resize((size_t)(n1-i0)*d);
				for(ulong i=i0; i<n1; i++) for(uint c=0u; c<d; c++) {
					const T v = data[i+(ulong)c*N];
					chunk[(size_t)(i-i0)*d+c] = sizeof(T)==1u ? v : reverse_bytes((T)(factor*v));
				}
				file.write((const char*)chunk.data(), (std::streamsize)(chunk.size()*sizeof(T)));
			}
		}
		void write_device_to_vtk(const std::string& path="", const bool convert_to_si_units=true) const {
			const std::string filename = create_file_extension(default_filename(path, name(), ".vtk", lbm->get_t()), ".vtk");
			lbm_check(lbm_write_vtk(lbm->domain, field, filename.c_str(), convert_to_si_units ? units.si_x(1.0f) : 1.0f, si_factor(convert_to_si_units)));
		}
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
	void write_mesh_to_vtk(const Mesh* mesh, const std::string& path="", const bool convert_to_si_units=true) const { // src/lbm.cpp:1094-1129
		const std::string filename = default_filename(path, "mesh", ".vtk", get_t());
		const uint T = mesh->triangle_number;
		const std::string header_1 = "# vtk DataFile Version 3.0\nFluidX3D "+filename.substr(filename.rfind('/')+1)+"\nBINARY\nDATASET POLYDATA\nPOINTS "+std::to_string(3u*T)+" float\n";
		const std::string header_2 = "POLYGONS "+std::to_string(T)+" "+std::to_string(4u*T)+"\n";
		const float spacing = convert_to_si_units ? units.si_x(1.0f) : 1.0f;
		const float3 offset = center();
		std::vector<float> points(9u*(size_t)T);
		std::vector<int> triangles(4u*(size_t)T);
		for(uint i=0u; i<T; i++) {
			const float3* p[3] = {&mesh->p0[i], &mesh->p1[i], &mesh->p2[i]};
			for(uint k=0u; k<3u; k++) {
				points[9u*(size_t)i+3u*k   ] = reverse_bytes(spacing*(p[k]->x-offset.x));
				points[9u*(size_t)i+3u*k+1u] = reverse_bytes(spacing*(p[k]->y-offset.y));
				points[9u*(size_t)i+3u*k+2u] = reverse_bytes(spacing*(p[k]->z-offset.z));
			}
			triangles[4u*(size_t)i] = reverse_bytes(3);
			for(uint k=0u; k<3u; k++) triangles[4u*(size_t)i+1u+k] = reverse_bytes(3*(int)i+(int)k);
		}
		create_folder(filename);
		std::ofstream file(filename, std::ios::out|std::ios::binary);
		if(!file) throw lbm_error(LBM_ERR_IO, "File \""+filename+"\" cannot be written");
		file.write(header_1.c_str(), (std::streamsize)header_1.length());
		file.write((const char*)points.data(), (std::streamsize)(4u*9u*(size_t)T));
		file.write(header_2.c_str(), (std::streamsize)header_2.length());
		file.write((const char*)triangles.data(), (std::streamsize)(4u*4u*(size_t)T));
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
