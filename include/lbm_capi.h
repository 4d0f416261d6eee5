/* C-ABI of the GB300 LBM solver core: one LBM domain on one CUDA device.
 *
 * This is the boundary the reference's host code would bind in place of its OpenCL layer
 * (src/opencl.hpp: Device, Memory<T>, Kernel) and the per-domain enqueue calls of LBM_Domain
 * (src/lbm.hpp:94-120, src/lbm.cpp:96-332). Plain pointers and sizes only; every entry point
 * returns an lbm_status and never exits the process (the reference prints and calls exit(1),
 * src/utilities.hpp:4159-4166); lbm_last_error() gives the message of the last failure on the
 * calling thread.
 *
 * Layout of every field is the reference's (src/kernel.cpp:820-826, 861-863, 960-967):
 *   cell index n = x+(y+z*Ny)*Nx; rho float[N]; u float[3N] (SoA: ux, then uy, then uz);
 *   flags uint8[N]; F float[3N] (SoA); DDFs fi[i*N+n] in the storage type of the variant.
 * Flag bits are the reference's TYPE_* values (src/defines.hpp:53-60).
 *
 * Streams: all work is enqueued on the domain's stream (a stream the library creates, or the
 * caller's via lbm_set_stream). Entry points that return host data synchronise that stream.
 */
#ifndef FX3D_LBM_CAPI_H
#define FX3D_LBM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_CAPI_VERSION 1

typedef struct lbm_domain lbm_domain; /* opaque: one LBM_Domain on one GPU */

typedef enum lbm_status {
	LBM_OK = 0,
	LBM_ERR_INVALID_ARGUMENT = 1, /* bad size, pointer, enum or configuration */
	LBM_ERR_OUT_OF_MEMORY = 2,    /* device allocation failed (src/opencl.hpp:375-387 checks the same) */
	LBM_ERR_CUDA = 3,             /* a CUDA runtime call failed */
	LBM_ERR_NOT_INITIALIZED = 4,  /* the call needs lbm_initialize first */
	LBM_ERR_UNSUPPORTED = 5,      /* the variant lacks the extension the call needs */
	LBM_ERR_NO_DEVICE = 6,        /* no CUDA device (the reference exits in get_devices, src/opencl.hpp:222-252) */
	LBM_ERR_IO = 7                /* a file could not be opened or written */
} lbm_status;

/* variant selection: the reference's compile-time switches (src/defines.hpp:5-29) as runtime values */
enum { LBM_SRT = 0, LBM_TRT = 1 };
enum { LBM_FP32 = 0, LBM_FP16S = 1, LBM_FP16C = 2 };
enum {
	LBM_EXT_VOLUME_FORCE = 1,          /* VOLUME_FORCE: global force (fx,fy,fz), Guo forcing */
	LBM_EXT_FORCE_FIELD = 2,           /* FORCE_FIELD: per-cell force F added to (fx,fy,fz) */
	LBM_EXT_EQUILIBRIUM_BOUNDARIES = 4, /* EQUILIBRIUM_BOUNDARIES: TYPE_E cells held at their rho/u */
	LBM_EXT_SUBGRID = 8,               /* SUBGRID: Smagorinsky-Lilly relaxation rate per cell (src/kernel.cpp:1579-1593); not with lbm_run_adjoint */
	LBM_EXT_MOVING_BOUNDARIES = 16,    /* MOVING_BOUNDARIES: TYPE_S cells with u != 0 are moving walls for their TYPE_MS
	                                    * neighbours (src/kernel.cpp:1104-1113, 1378-1387, 1431-1450); not with lbm_run_adjoint */
	LBM_EXT_UPDATE_FIELDS = 32         /* UPDATE_FIELDS: every stream_collide writes the rho/u each cell collides with
	                                    * (src/kernel.cpp:1565-1573; +16 B per cell and step), so reads of rho/u run no
	                                    * update_fields (which becomes a no-op, src/lbm.cpp:184-191); the fields after a
	                                    * step are those of the state the step started from, as in the reference */
};
/* arithmetic of the collision. EXACT evaluates the reference's FP32 operation order with IEEE
 * rounding at every step: bit-identical to the reference's kernel text evaluated on a CPU. FAST
 * contracts multiply-adds and regroups terms the way the reference's own GPU build may
 * (-cl-mad-enable); it agrees with EXACT to FP32 rounding. AUTO (default) is EXACT for FP32 DDF
 * storage and FAST for FP16S/FP16C, where the 16-bit storage rounding dominates either error. */
enum { LBM_ARITH_AUTO = 0, LBM_ARITH_EXACT = 1, LBM_ARITH_FAST = 2 };
enum { LBM_FIELD_RHO = 0, LBM_FIELD_U = 1, LBM_FIELD_FLAGS = 2, LBM_FIELD_F = 3, LBM_FIELD_FI = 4 };
enum { LBM_TYPE_S = 0x01, LBM_TYPE_E = 0x02, LBM_TYPE_T = 0x04, LBM_TYPE_F = 0x08,
       LBM_TYPE_I = 0x10, LBM_TYPE_G = 0x20, LBM_TYPE_X = 0x40, LBM_TYPE_Y = 0x80 };

typedef struct lbm_config {
	uint32_t Nx, Ny, Nz;     /* lattice size; Nz <= 65535, N = Nx*Ny*Nz >= 1 */
	uint32_t velocity_set;   /* 19 (D3Q19) or 27 (D3Q27) */
	uint32_t collision;      /* LBM_SRT or LBM_TRT */
	uint32_t storage;        /* LBM_FP32, LBM_FP16S or LBM_FP16C DDF storage; arithmetic is FP32 */
	uint32_t extensions;     /* LBM_EXT_* bits */
	int32_t device;          /* CUDA device ordinal; -1: the calling thread's current device */
	float nu;                /* kinematic shear viscosity, > 0 */
	float fx, fy, fz;        /* global volume force (needs LBM_EXT_VOLUME_FORCE when non-zero) */
	uint32_t arithmetic;     /* LBM_ARITH_AUTO (0), LBM_ARITH_EXACT or LBM_ARITH_FAST */
} lbm_config;

/* ---- lifetime: replaces LBM_Domain::LBM_Domain + allocate (src/lbm.cpp:96-176) and the
 *      constructor sanity checks (src/lbm.cpp:783-838). rho is filled with 1, u/flags/F with 0. */
int lbm_domain_create(const lbm_config* config, lbm_domain** domain);
int lbm_domain_destroy(lbm_domain* domain);

/* relaxation rate the kernels use: 1/tau, tau = 3*nu+1/2, rounded the way the reference bakes it
 * into its kernel source as a "%f" literal (src/lbm.cpp:374) */
float lbm_relaxation_rate(float nu);
/* bytes per cell: device allocation and per-time-step traffic (src/lbm.cpp:38-72) */
uint32_t lbm_bytes_per_cell_device(const lbm_config* config);
uint32_t lbm_bandwidth_bytes_per_cell(const lbm_config* config);

/* ---- streams and synchronisation (src/opencl.hpp: Device::finish_queue) */
int lbm_set_stream(lbm_domain* domain, void* cuda_stream); /* NULL: back to the domain's own stream */
int lbm_get_stream(lbm_domain* domain, void** cuda_stream);
int lbm_synchronize(lbm_domain* domain);

/* ---- fields: Memory<T>::enqueue_write_to_device / enqueue_read_from_device (src/opencl.hpp:510-531).
 * bytes must equal the field size. Reading rho/u first brings them up to date with lbm_update_fields
 * when the domain is initialised, as Memory_Container::read_from_device does (src/lbm.hpp:390-396).
 * LBM_FIELD_F exists with LBM_EXT_FORCE_FIELD, or after lbm_update_force_field. */
int lbm_write_field(lbm_domain* domain, int field, const void* host, size_t bytes);
int lbm_read_field(lbm_domain* domain, int field, void* host, size_t bytes);
int lbm_field_device_pointer(lbm_domain* domain, int field, void** device_ptr, size_t* bytes);

/* ---- time stepping */
/* initialize kernel at odd parity, then t = 0 (src/lbm.cpp:881-922; src/kernel.cpp:1358-1430) */
int lbm_initialize(lbm_domain* domain);
/* `steps` LBM time steps, each one stream_collide launch and t += 1 (src/lbm.cpp:181-183, 924-975;
 * src/kernel.cpp:1454-1636); no host synchronisation between steps */
int lbm_stream_collide(lbm_domain* domain, uint64_t steps);
/* rho/u from the DDFs at the current t, skipped if already current (src/lbm.cpp:184-191) */
int lbm_update_fields(lbm_domain* domain);
int lbm_get_time_step(lbm_domain* domain, uint64_t* t);
int lbm_set_force(lbm_domain* domain, float fx, float fy, float fz); /* LBM::set_f (src/lbm.hpp:469-473) */
int lbm_is_initialized(lbm_domain* domain, int* initialized);
int lbm_reset(lbm_domain* domain); /* next lbm_initialize starts over (src/lbm.cpp:982-984) */

/* ---- VTK export (src/lbm.hpp:298-340 Memory_Container::write_vtk, 401-407 write_device_to_vtk):
 * writes field rho, u, flags or F as a binary legacy VTK file (STRUCTURED_POINTS, big-endian, one
 * point per cell, x fastest; u and F interleaved per point) with the reference's header: title
 * "FluidX3D <file name>", origin spacing*(0.5-N/2) per axis, `spacing` between points. FP32 values
 * are multiplied by `scale` (the reference's SI unit conversion; 1 for lattice units) on the GPU,
 * where they are also byte-swapped and interleaved, chunk by chunk, while the previous chunk is
 * written to the file. rho/u are brought up to date first (update_fields). The file's folder is
 * created if missing; the caller builds the file name (the reference: <path><name>-<t, 9 digits>.vtk). */
int lbm_write_vtk(lbm_domain* domain, int field, const char* filename, float spacing, float scale);

/* ---- moving boundaries (LBM_EXT_MOVING_BOUNDARIES; src/lbm.cpp:240-244, 1019-1023; src/kernel.cpp:1431-1450):
 * sets TYPE_MS on every cell (not TYPE_S, TYPE_E or TYPE_T) that has a TYPE_S neighbour with u != 0
 * and clears it on the others; call it after changing the velocity of solid cells. lbm_initialize
 * does the same marking (TYPE_T cells included, as the reference's initialize does). */
int lbm_update_moving_boundaries(lbm_domain* domain);

/* ---- forces on solids (src/lbm.cpp:207-229, 991-1015; src/kernel.cpp:1873-1959) */
/* F = momentum exchange on TYPE_S cells at the current t (skipped if already current) */
int lbm_update_force_field(lbm_domain* domain);
int lbm_reset_force_field(lbm_domain* domain);
/* masked sums over cells with flags == marker, accumulated in FP64 on the device:
 * center of mass: out[0..2] = mean cell position (box-centred coordinates), out[3] = cell count;
 * force: out[0..2] = sum F; torque: out[0..2] = sum (p - c) x F */
int lbm_object_center_of_mass(lbm_domain* domain, uint8_t marker, double out[4]);
int lbm_object_force(lbm_domain* domain, uint8_t marker, double out[3]);
int lbm_object_torque(lbm_domain* domain, uint8_t marker, double cx, double cy, double cz, double out[3]);

/* Allocation-free object sums (no counterpart in the reference): the reduction of the three calls
 * above over device arrays the caller owns (flags[N]; F[3N], x|y|z blocks as in a domain), issued on
 * the caller's stream, with its scratch in a fixed static device array instead of an allocation.
 * kind 0: out = mean position (box-centred) and cell count, as lbm_object_center_of_mass;
 * kind 1: out[0..2] = sum F; kind 2: out[0..2] = sum (p - c) x F; out[3] = 0 for kinds 1 and 2.
 * blocks: reduction blocks, 0 = 608 (the count the domain calls use, same summation order);
 * more than LBM_OBJECT_SUM_STATIC_MAX_BLOCKS is LBM_ERR_INVALID_ARGUMENT. Returns once the result
 * is on the host (the stream is synchronised). The first call on a device resolves the scratch's
 * address with cudaGetSymbolAddress: make it before any stream capture on that device. The scratch
 * is shared by all calls on a device: calls that overlap on the GPU race. */
#define LBM_OBJECT_SUM_STATIC_MAX_BLOCKS 1216
int lbm_object_sum_static(int device, uint32_t Nx, uint32_t Ny, uint32_t Nz, const uint8_t* flags_device, const float* F_device,
                          uint8_t marker, int kind, double cx, double cy, double cz, uint32_t blocks, void* cuda_stream, double out[4]);

/* ---- mesh voxelization (src/lbm.cpp:275-327, 1074-1093; src/kernel.cpp:2267-2363).
 * p0/p1/p2: host arrays of `triangles` vertices, xyz interleaved (float3 p0[triangles]), in lattice
 * coordinates; center / linear_velocity / rotational_velocity as in LBM::voxelize_mesh_on_device.
 * Cells inside get flags = (flags & ~(TYPE_S|TYPE_E)) | flag. */
int lbm_voxelize_mesh(lbm_domain* domain, const float* p0, const float* p1, const float* p2, uint32_t triangles, uint8_t flag,
                      const float center[3], const float linear_velocity[3], const float rotational_velocity[3]);
/* With LBM_EXT_MOVING_BOUNDARIES, a solid (flag & (TYPE_S|TYPE_E) == TYPE_S) voxelized with a non-zero
 * velocity also runs lbm_update_moving_boundaries (src/lbm.cpp:1082-1084). */
/* clears `flag` in the mesh bounding box +-1 cell */
int lbm_unvoxelize_mesh(lbm_domain* domain, const float pmin[3], const float pmax[3], uint8_t flag);

/* ---- adjoint (no counterpart in the reference): gradient of an objective J with respect to the
 *      per-cell force field F (LBM_EXT_VOLUME_FORCE and LBM_EXT_FORCE_FIELD required). The forward run
 *      starts at the domain's current time step t0 (after lbm_initialize) and advances it by `steps`,
 *      exactly like lbm_stream_collide; the discrete adjoint then runs backwards through the same steps,
 *      recomputing them from DDF snapshots taken every checkpoint_interval steps. */
enum { LBM_OBJECTIVE_KINETIC_ENERGY_PLANE_X = 1, /* mean of 1/2 rho |u|^2 over the fluid cells of plane x */
       LBM_OBJECTIVE_DRAG_X = 2 };             /* x component of the force on cells with flags == marker */
typedef struct lbm_adjoint_config {
	uint64_t steps;               /* forward time steps */
	uint64_t checkpoint_interval; /* DDF snapshot every this many steps (>= 1) */
	uint32_t objective;           /* LBM_OBJECTIVE_* */
	uint32_t plane_x;             /* KINETIC_ENERGY_PLANE_X: plane */
	uint32_t marker;              /* DRAG_X: flag value of the object's cells */
	uint32_t workspace_limit_kib; /* at most this much device memory for the adjoint's workspace (KiB; 0: what is free,
	                               * less a 512 MiB margin); a smaller limit selects a plan with less overlap or two levels */
	uint64_t window_begin, window_end; /* J is the mean over the states after these time steps (inclusive) */
} lbm_adjoint_config;
typedef struct lbm_adjoint_stats {
	double forward_ms;            /* device time of the forward sweep (steps, snapshots, objective) */
	double recompute_ms, adjoint_ms; /* device time of the recomputation and of the adjoint steps when they run one
	                               * after the other; 0 when they overlap (overlapped = 1): then see reverse_ms */
	uint64_t workspace_bytes;     /* snapshots + recomputation state + moment checkpoints (rho/u, 16 B per cell and
	                               * step) + adjoint DDFs + gradient */
	uint32_t levels;              /* 1: moments of every step of a segment kept; 2: DDF sub-snapshots inside segments */
	uint32_t overlapped;          /* 1: the next segment was recomputed on a second stream during the adjoint steps */
	double reverse_ms;            /* device time of the whole reverse sweep (recomputation and adjoint steps) */
} lbm_adjoint_stats;
/* J (objective, may be NULL), dJ/dF (gradient: host float[3N] SoA, may be NULL), stats (may be NULL) */
int lbm_run_adjoint(lbm_domain* domain, const lbm_adjoint_config* config, double* objective, float* gradient, lbm_adjoint_stats* stats);

/* ---- page-locked host buffers for fast field transfers (the reference's Memory<T> host side,
 *      src/opencl.hpp:342-440, is plain pageable memory) */
int lbm_host_alloc(size_t bytes, void** host_ptr);
int lbm_host_free(void* host_ptr);

/* message of the last failed call on this thread ("" if none) */
const char* lbm_last_error(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* FX3D_LBM_CAPI_H */
