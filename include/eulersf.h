/*
 * eulersf.h - C ABI of the GB300 implementation of EULERSF's coupled
 * solid-fluid step (yunteng/EULERSF).
 *
 * The reference has no FFI: the step sits behind C++ class call surfaces.
 * Each entry point below replaces one of them; the citation names the
 * reference interface it stands in for. All host pointers are plain C
 * arrays; all "device" pointers are CUDA global-memory addresses. No entry
 * point exits, traps or throws: every failure is an esf_status.
 *
 * Grid and indexing follow the reference: node (x, y, z) has index
 * x + y*xRes + z*xRes*yRes (include/geometry/FIELD_3D.h:72); pressure row
 * (cell) c has index x + y*(xRes-1) + z*(xRes-1)*(yRes-1)
 * (COUPLED_INTEGRATOR_3D.cpp:302-306); velocity unknown 3*k+d belongs to the
 * k-th interior node in z, y, x order (COUPLED_INTEGRATOR_3D.cpp:123-131).
 */
#ifndef EULERSF_H
#define EULERSF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ESF_ABI_VERSION 1
#define ESF_MAX_SOLIDS 8

typedef enum esf_status {
  ESF_OK = 0,
  ESF_ERR_INVALID_ARG = 1,   /* bad pointer, size or enum */
  ESF_ERR_STATE = 2,         /* call out of order (e.g. step before init) */
  ESF_ERR_CUDA = 3,          /* a CUDA runtime call failed; see esf_last_error */
  ESF_ERR_OOM = 4,           /* device allocation failed */
  ESF_ERR_IO = 5,            /* config / frame file could not be read or written */
  ESF_ERR_NUMERIC = 6,       /* NaN/Inf met in a solve (the step still returns) */
  ESF_ERR_NO_DEVICE = 7,     /* no CUDA device visible */
  ESF_ERR_UNSUPPORTED = 8
} esf_status;

typedef enum esf_precision {
  ESF_FP64 = 0,   /* plain method: everything in FP64 */
  ESF_MIXED = 1,  /* FP32 inner solves inside FP64 iterative refinement */
  /* As ESF_MIXED, but the pressure solve is one FP32 Krylov run whose
   * correction and search direction are kept at a 48-bit significand
   * (double-float FP32 pairs; operator, residual vectors and stencil in
   * FP32; dot products, alpha/beta and periodic ||b - A x|| checks, into
   * which the correction is folded, in FP64), continued to the FP64
   * tolerance without restarts: about the FP64 solver's iteration count,
   * where the refinement takes 1.3x of it on average (0.4-3.4x per step on
   * a 256^3 scene), for 16 instead of 12 words moved per row and iteration.
   * Grids whose cell rows are not a multiple of 4 cells solve as ESF_MIXED.
   * No reference counterpart. */
  ESF_MIXED_X64 = 2
} esf_precision;

/* Grid of the coupled integrator: COUPLED_INTEGRATOR_3D(int xRes, int yRes,
 * int zRes, Real dh, VEC3F origin) (COUPLED_INTEGRATOR_3D.h:31). */
typedef struct esf_grid {
  int xRes, yRes, zRes;
  double dh;
  double origin[3];
} esf_grid;

/* Every config key the step reads (SIMPLE_PARSER keys, name in quotes).
 * esf_params_default() fills the reference's own defaults. */
typedef struct esf_params {
  double dt;                       /* "dt" (0.01 in the integrator ctor) */
  double fluid_density;            /* "fluid density" (1) */
  double fluid_viscosity;          /* "fluid viscocity" (stored, unused) */
  double vorticity_eps;            /* "vorticity eps" (2.0), raw cfg value */
  double buoyancy;                 /* "buoyancy" (0.1) */
  double gravity;                  /* "gravity" (0) */
  double rayleigh_alpha;           /* "rayleigh alpha" (0) */
  double rayleigh_beta;            /* "rayleigh beta" (0) */
  double implicit_solver_eps;      /* "implicit solver eps" (1e-8) */
  double div_free_solver_eps;      /* "div free solver eps" (1e-8) */
  int cr_max_iterations;           /* "cr max iterations" (10) */
  double mass_sample_dh;           /* "mass sample dh" (dh/10) */
  int tight_border;                /* "tight border" (3) */
  int extrapolation_cells;         /* "extrapolation cells" (20) */
  int particles_per_cell;          /* "number of particles per material cell" (8) */
  double flip_alpha;               /* "flip alpha" (0.95) */
  double contact_safe_distance;    /* "contact safe distance" (dh/2) */
  double wall_thickness;           /* "wall thickness" (1.5 dh) */
  double contact_spring_stiffness; /* "contact spring stiffness" (10000) */
  double friction;                 /* "friction" (0.5) */
  int flip_cutoff;                 /* "flip cutoff" (3) */
  double flow_rate;                /* "flow rate" (0); plasticity only */
  /* GB300 additions (no reference key) */
  int precision;                   /* esf_precision */
  double inner_eps;                /* mixed: FP32 inner relative tolerance (1e-4) */
  int max_refinements;             /* mixed: outer FP64 refinement cap (50) */
} esf_params;

/* One elastic solid: DEFOR_SOLID_3D(xRes, yRes, zRes, dh, origin, restMass)
 * + setMaterial + setMassDensity + setInitialState + setInitialVelocity +
 * loadSurfaceMesh (DEFOR_SOLID_3D.h:43-71; main.cpp:99-160). The mesh is
 * given in its rest pose (as loaded from the OBJ); scaling, rotation and
 * translation are applied as main.cpp:150-154 does. */
typedef struct esf_solid_desc {
  int mass_res[3];            /* rest-pose mass grid (FIELD_3Df "<mesh>.mass") */
  double mass_dh;
  double mass_origin[3];
  const double* rest_mass;    /* mass_res[0]*mass_res[1]*mass_res[2], x fastest */
  double lambda, mu;          /* "material lambda/mu i" */
  double density;             /* "solid mass density i" */
  double rotation[9];         /* row-major 3x3 */
  double translation[3];      /* "solid translation i" */
  double scaling[3];          /* "solid scaling i" */
  double initial_velocity[3]; /* "solid initial velocity i" */
  int num_vertices;
  const double* vertices;     /* num_vertices x 3, rest pose */
  int num_triangles;
  const int* triangles;       /* num_triangles x 3, 0-based */
  double plastic_yield;       /* "solid plastic yield i" (setPlasticYield); <= 0: elastic */
} esf_solid_desc;

/* What one stepImplicit() call did (COUPLED_INTEGRATOR_3D.cpp:377-636). */
typedef struct esf_step_report {
  double dt;                  /* time step taken (CFL-limited) */
  double energy;              /* kinetic + potential + strain (return value) */
  int iterations[3];          /* solid solve 1, pressure solve, solid solve 2 */
  int converged[3];
  double rel_residual[3];     /* ||Ax-b|| / ||b|| at exit */
  int refinements[3];         /* mixed: outer FP64 refinement steps per solve
                                 (ESF_MIXED_X64 pressure solve: its FP64 checks) */
  int fp64_iterations;        /* mixed: FP64 PCR iterations that finished the pressure solve */
  int prone_to_contact;       /* CFL factor 0.6 instead of 1.8 */
  int num_particles;
  int status;                 /* esf_status of the step */
  double device_ms;           /* device time of the step (CUDA events) */
  /* device time per phase, in the order of the reference's TIMING_BREAKDOWN
   * labels (COUPLED_INTEGRATOR_3D.cpp:377-917): 0 broad phase + CFL,
   * 1 solid forces/stiffness/assembly, 2 body forces, 3 solid solve 1,
   * 4 pressure solve, 5 solid solve 2, 6 grid to particle, 7 particle to
   * grid, 8 velocity extension, 9 solid displacement update, 10 solid mass,
   * 11 surface mesh + SDF + particle seeding, 12 fluid advection + walls */
  double phase_ms[13];
  int fp64_stress_cells;      /* mixed: valid cells whose stress was evaluated in FP64
                                 (cond(F) > 1e3); the others use FP32 */
  int valid_cells;            /* valid solid cells of the step's stiffness sweep */
  int solid_contacts;         /* particles that took a solid-solid contact impulse
                                 (DEFOR_SOLID_3D.cpp:967-995) */
} esf_step_report;

/* Field identifiers for esf_get_field / esf_set_field / esf_field_info. */
typedef enum esf_field {
  /* integrator, per node (xRes*yRes*zRes entries) */
  ESF_F_VELOCITY = 0,          /* f64 x3 _velocity */
  ESF_F_INTENSITY = 1,         /* f64 _intensity */
  ESF_F_SOLID_MASS = 2,        /* f64 _solidMass */
  ESF_F_NODE_SOLID_VF = 3,     /* f64 _nodeSolidVolumeFraction */
  ESF_F_DOF_MAP = 4,           /* i32 _gridIdxToSolutionIdx */
  ESF_F_SOLID_DOF_MAP = 5,     /* i32 _gridIdxToSolidIdx */
  /* integrator, per pressure row (cells) */
  ESF_F_PRESSURE = 10,         /* f64 lambda1 (warm-started pressure) */
  ESF_F_JMINVJT_DIAG = 11,     /* f64 _JMInvJTDiag */
  ESF_F_DIV_RHS = 12,          /* f64 _divergenceConstraintsRHS */
  ESF_F_B1 = 13,               /* f64 J v* - rhs */
  /* integrator, per velocity unknown (3 * interior nodes) */
  ESF_F_NZ_MASS_INV = 20,      /* f64 _nzMassVecInv */
  ESF_F_VELOCITY_DT0 = 21,     /* f64 _velocityAtDt0 (v*) */
  ESF_F_VELOCITY_DT1 = 22,     /* f64 _velocityAtDt1 */
  ESF_F_UNIT_FORCE = 23,       /* f64 _unitForce after "*= dt; += mv" */
  /* integrator, per solid unknown (3 * solid nodes) */
  ESF_F_SOLID_UNIT_FORCE = 30, /* f64 _solidUnitForce after "*= dt; += mv" */
  ESF_F_SOLID_VELOCITY_DT0 = 31,
  ESF_F_SOLID_PRESSURE_CORRECTION = 32,
  ESF_F_DAMPED_SOLID_MASS = 33,
  ESF_F_SYSTEM_DIAG = 34,      /* f64 _systemMatrix.diagonal() */
  ESF_F_SYSTEM_BLOCKS = 35,    /* f64 [solid node][27 neighbours][3][3] of _systemMatrix */
  ESF_F_SYSTEM_MASK = 36,      /* i32 [solid node] bit j = structural block j present */
  /* per solid (solid index argument) */
  ESF_F_S_U = 50,              /* f64 x3 per node */
  ESF_F_S_X = 51,              /* f64 x3 per node */
  ESF_F_S_VELOCITY = 52,       /* f64 x3 per node */
  ESF_F_S_VEC_WORKSPACE = 53,  /* f64 x3 per node (previous extended velocity) */
  ESF_F_S_MASS = 54,           /* f64 per node */
  ESF_F_S_PHI = 55,            /* f64 per node */
  ESF_F_S_DET_FINV = 56,       /* f64 per node */
  ESF_F_S_VALID = 57,          /* i8 per cell, (xRes-1)(yRes-1)(zRes-1) */
  ESF_F_S_QUARTER_FRACTIONS = 58, /* f64 8 per node */
  ESF_F_S_PARTICLES = 59,      /* f64 10 per particle: pos, velocity, restPos, mass */
  ESF_F_S_MESH_VERTICES = 60,  /* f64 x3 per vertex (current pose) */
  ESF_F_S_BOXES = 61,          /* i32 12: xmin..zmax, tightMin, tightMax */
  ESF_F_S_FPINV = 62,          /* f64 9 per material cell (row-major 3x3): _FpInv, plastic solids */
  ESF_F_S_FPINV_GRID = 63      /* f64 7: material grid xRes, yRes, zRes, dh, origin (plastic) */
} esf_field;

typedef struct esf_scene esf_scene;

/* ---- library ----------------------------------------------------------- */
int esf_abi_version(void);
/* Text of the last error on this thread (never NULL). */
const char* esf_last_error(void);
/* Fills the reference defaults for a grid (see esf_params). */
esf_status esf_params_default(const esf_grid* grid, esf_params* params);
/* SIMPLE_PARSER::parse + the getInt/getFloat reads of main.cpp:63-141 and of
 * the step path: reads a reference cfg file into grid, params and up to
 * max_solids solid descriptors (mesh/mass paths are returned, not loaded).
 * Replaces SIMPLE_PARSER (src/util/SIMPLE_PARSER.cpp:64-168). */
esf_status esf_parse_config(const char* path, esf_grid* grid, esf_params* params,
                            int* num_solids, char* solid_paths, size_t path_stride,
                            esf_solid_desc* solids, int max_solids);

/* ---- scene lifetime (COUPLED_INTEGRATOR_3D.h:29-78) ---------------------- */
/* COUPLED_INTEGRATOR_3D::COUPLED_INTEGRATOR_3D (COUPLED_INTEGRATOR_3D.cpp:36-78).
 * stream: a cudaStream_t to run on, or NULL for the scene's own stream. */
esf_status esf_create(const esf_grid* grid, const esf_params* params, void* stream,
                      esf_scene** out);
/* ~COUPLED_INTEGRATOR_3D (COUPLED_INTEGRATOR_3D.cpp:79-86): frees everything. */
esf_status esf_destroy(esf_scene* scene);
/* new DEFOR_SOLID_3D + setters + COUPLED_INTEGRATOR_3D::addSolid
 * (main.cpp:99-160; COUPLED_INTEGRATOR_3D.h:44). Copies all inputs. */
esf_status esf_add_solid(esf_scene* scene, const esf_solid_desc* solid);
/* DEFOR_SOLID_3D::loadRestSDF (DEFOR_SOLID_3D.cpp:210-214; main.cpp:146-148):
 * the rest-pose signed distance of solid `solid` from a DT-Grid ".svol" file
 * ("DTG v1.0", SvolLoader_DTTop1.0.h), for solid-solid contact in the
 * particle update. Scenes with more than one solid need it for every solid
 * before their first step (esf_step returns ESF_ERR_STATE otherwise).
 * ESF_ERR_IO on a missing or malformed file, ESF_ERR_UNSUPPORTED for a
 * rotated volume. */
esf_status esf_solid_load_rest_sdf(esf_scene* scene, int solid, const char* svol_path);
/* SPARSE_SDF::signedDistAndCurrentNormal (SPARSE_SDF.cpp:98-117) of a solid
 * at n rest-space points (host arrays, 3 per point): the signed distance, or
 * 1 when the point is farther than safe_dist or its surface point lies under
 * no hashed triangle, and the current unit normal of that triangle (zero
 * when the distance is 1). The contact test of the particle update alone. */
esf_status esf_rest_sdf_query(esf_scene* scene, int solid, int n, const double* points,
                              double safe_dist, double* signed_dist, double* normals);
/* The dense lattice of a ".svol" rest SDF, on the host (no device needed):
 * point (x, y, z) for lo <= (x, y, z) < lo + n at
 * (x - lo[0]) + (y - lo[1]) n[0] + (z - lo[2]) n[0] n[1]; values holds the
 * band values, codes 1 for band points, -1 where the DT-Grid returns its
 * inside constant and 0 where it returns the outside constant (constants[0],
 * constants[1]). Lattice coordinate of a rest point p: (p - translation)/dx.
 * values and codes NULL: size query. */
esf_status esf_svol_read(const char* path, int lo[3], int n[3], double* dx, double translation[3],
                         double constants[2], float* values, signed char* codes, size_t capacity);
/* COUPLED_INTEGRATOR_3D::setFluidDensity / setFluidViscocity (h:45-46). */
esf_status esf_set_fluid(esf_scene* scene, double density, double viscosity);
/* COUPLED_INTEGRATOR_3D::init (COUPLED_INTEGRATOR_3D.cpp:104-135). */
esf_status esf_init(esf_scene* scene);
/* COUPLED_INTEGRATOR_3D::setMaxDt (COUPLED_INTEGRATOR_3D.h:47). */
esf_status esf_set_max_dt(esf_scene* scene, double max_dt);
/* COUPLED_INTEGRATOR_3D::stepImplicit (COUPLED_INTEGRATOR_3D.cpp:377-636).
 * report may be NULL. Synchronises the scene's stream before returning. */
esf_status esf_step(esf_scene* scene, esf_step_report* report);
/* COUPLED_INTEGRATOR_3D::dt() (h:48). */
double esf_dt(const esf_scene* scene);

/* ---- field access (the reference's member access; dumps, noise, I/O) ---- */
/* count = number of elements, elem_bytes = bytes per element (8 f64, 4 i32,
 * 1 i8); a field of 3-vectors counts 3 elements per node. */
esf_status esf_field_info(const esf_scene* scene, esf_field field, int solid,
                          size_t* count, size_t* elem_bytes);
/* Copy a field to host memory (bytes must equal count*elem_bytes). */
esf_status esf_get_field(esf_scene* scene, esf_field field, int solid, void* host,
                         size_t bytes);
/* Overwrite a field from host memory (node/solid fields only). */
esf_status esf_set_field(esf_scene* scene, esf_field field, int solid,
                         const void* host, size_t bytes);

/* ---- solver operator seam ----------------------------------------------- */
/* COUPLED_INTEGRATOR_3D::getMatVecMult (COUPLED_INTEGRATOR_3D.cpp:638-660):
 * out = J diag(mass_inv) J^T in over the (xRes-1)(yRes-1)(zRes-1) pressure
 * rows of `grid`. mass_inv: one value per node (xRes*yRes*zRes, boundary
 * entries ignored). Device pointers, FP64. */
esf_status esf_pressure_apply(const esf_grid* grid, const double* mass_inv_node,
                              const double* in, double* out, void* stream);
/* CONJUGATE_RESIDUAL<JACOBI_PRECONDITIONER>::solvePCR(b, x, getMatVecMult, app)
 * (CONJUGATE_RESIDUAL.inl:109-192) with the pressure operator above and the
 * Jacobi diagonal `diag`. x is the warm start on entry and the solution on
 * exit. Device pointers; FP64 (precision ESF_FP64) or FP32 inner solves in
 * FP64 refinement (ESF_MIXED). iterations/rel_residual may be NULL. */
esf_status esf_pressure_solve(const esf_grid* grid, const double* mass_inv_node,
                              const double* diag, const double* b, double* x,
                              double eps, int max_iterations, int precision,
                              int* iterations, double* rel_residual, void* stream);

/* Batched solver seam: n independent pressure systems solved together, each
 * with its own grid, m^-1, diagonal, right-hand side and warm start (arrays of
 * n device pointers; iterations and rel_residual NULL or arrays of n). No
 * reference counterpart: the reference solves one system per process
 * (solvePCR). At ESF_MIXED the FP32 inner iterations of systems of the same
 * grid shape advance in shared launches (continuous batching, as the server
 * does); each system's FP64 refinement runs on its own stream, driven by its
 * own host thread. Every system gets the same answer, iterations and bits as
 * esf_pressure_solve alone, unless `autotune` is set: the batcher then picks
 * each shape's tile depth by timing (esf_server_config.autotune), and the
 * answers agree to rounding instead. `stats` (may be NULL) receives the batcher's
 * counters (esf_batch_stats, below). Work waits for what is queued on
 * `stream` before the call; the call returns when every solve has finished. */
struct esf_batch_stats;
esf_status esf_pressure_solve_batch(int n, const esf_grid* grids, const double* const* mass_inv_node,
                                    const double* const* diag, const double* const* b,
                                    double* const* x, double eps, int max_iterations, int precision,
                                    int autotune, int* iterations, double* rel_residual,
                                    struct esf_batch_stats* stats, void* stream);

/* Allocation-free variant of esf_pressure_solve at ESF_FP64. It has no
 * counterpart in the reference. It is for callers that must not allocate or
 * free device memory while they solve: a host whose HBM is reserved up front
 * by its own pool (a framework's caching allocator, a serving runtime), where
 * a cudaMalloc can fail or fragment that pool, and callers that keep other
 * streams busy, which the device-wide synchronisation of cudaFree would stall.
 * Same kernels, order and results as esf_pressure_solve(..., ESF_FP64, ...).
 * Its scratch is a file-scope static device array (10.1 MiB per device, part
 * of the loaded module, held by every GPU that loads the library until the
 * process exits) for grids of at most ESF_STATIC_SOLVE_MAX_CELLS cells;
 * larger grids return ESF_ERR_UNSUPPORTED with a message. Nothing is
 * allocated, freed or created (no stream, event or graph). The first call on
 * each device, and the first after that device's context has been re-created
 * (cudaDeviceReset), looks up the array's device address with
 * cudaGetSymbolAddress, which can load the module's device code. One
 * scratch per device: calls
 * that overlap on the same device, from two host threads or two streams, race
 * on it and must be serialised by the caller; each call clears what it needs
 * zeroed. The call synchronises `stream` and returns when the solve has
 * finished on it. */
#define ESF_STATIC_SOLVE_MAX_CELLS (64 * 64 * 64)
#define ESF_STATIC_SOLVE_MAX_DEVICES 64
esf_status esf_pressure_solve_static(const esf_grid* grid, const double* mass_inv_node,
                                     const double* diag, const double* b, double* x,
                                     double eps, int max_iterations, int* iterations,
                                     double* rel_residual, void* stream);

/* Self-test of the kernels' bounded waits; no reference counterpart (the
 * reference has no device code). Runs a one-block kernel that waits, with the
 * same wait the step's kernels use, on something that never happens:
 * kind 0, an mbarrier armed for a TMA copy that is never issued (the wait of
 * the TMA pressure kernels); kind 1, a grid barrier that the other blocks
 * never reach (the wait of the wave sweeps). *gave_up = 1 when the wait ran
 * out and the kernel returned on its own, as it should; *elapsed_ms (may be
 * NULL) is the kernel's device time. The context stays usable afterwards. */
esf_status esf_selftest_bounded_wait(int kind, int* gave_up, double* elapsed_ms);

/* Offline mass baking (projects/rasterizeSolid/main.cpp:20-80, the
 * reference's rasterizeSolid tool) on the GPU: the rest-pose mass grid of a
 * solid from its closed triangle mesh (num_vertices x 3 doubles,
 * num_triangles x 3 vertex indices, 0-based, host memory). The grid is the
 * mesh's bounding box grown by 10 cells on every side, res[k] = (int)(extent
 * / mass_dh), origin = the grown box's minimum; a node carries `density`
 * where its signed distance to the surface is at most mass_dh / 2. The
 * reference reads that distance from a DT-Grid narrow-band SDF (.svol);
 * here it is the exact distance to the triangles, signed by the winding
 * number, so nodes within the SDF's interpolation error of the threshold can
 * differ. Call with mass = NULL to get res and origin; then with a host
 * buffer of res[0]*res[1]*res[2] doubles (x fastest). total_mass (may be
 * NULL) = nodes with mass x density x mass_dh^3, as the tool prints. */
esf_status esf_rasterize_solid(const double* vertices, int num_vertices, const int* triangles,
                               int num_triangles, double mass_dh, double density, int res[3],
                               double origin[3], double* mass, size_t capacity, double* total_mass);

/* ---- serving: many scenes on one GPU -------------------------------------
 * No reference counterpart: the reference runs one scene per process (its
 * function-local statics pin one grid size per process). Requests arrive at
 * any time; a request is admitted when its estimated footprint
 * (esf_scene_footprint) fits what is left of the memory budget and one of
 * max_active slots is free, taking the first request in arrival order that
 * fits. Each admitted scene runs on its own CUDA stream and host thread, so
 * requests that arrive while others run overlap with them on the device.
 * Results stay readable (esf_server_get_field) until esf_server_release,
 * which returns the request's memory to the budget. */
typedef struct esf_server esf_server;
typedef struct esf_server_config {
  size_t hbm_budget_bytes; /* admission budget; 0: 85% of the device's free memory */
  int max_active;          /* scenes stepping at once; 0: 8 */
  int no_batching;         /* 1: each scene runs its inner solves alone on its own stream */
  int autotune;            /* 1: the batcher tunes each lane's tile depth by timing (answers then
                              agree with untuned runs to rounding, not bit for bit) */
} esf_server_config;
typedef struct esf_request {
  esf_grid grid;
  esf_params params;
  int num_solids;
  const esf_solid_desc* solids;  /* copied at submit, with their arrays */
  double fluid_density, fluid_viscosity;
  double smoke_carpet;           /* "smoke carpet thickness" (intensity 0.8 below it); 0: none */
  unsigned long long noise_seed; /* fluid noise U(-a, a) per component at interior nodes */
  double noise_amplitude;        /* without solid mass, added after init; 0: none */
  int steps;                     /* stepImplicit calls */
  const char* const* rest_sdf_paths; /* per solid, a ".svol" rest SDF (esf_solid_load_rest_sdf):
                                        the paths are copied at submit and the files read when
                                        the scene starts; required when num_solids > 1, else NULL */
} esf_request;
typedef enum esf_request_state {
  ESF_REQ_QUEUED = 0,
  ESF_REQ_RUNNING = 1,
  ESF_REQ_DONE = 2,
  ESF_REQ_FAILED = 3
} esf_request_state;
typedef struct esf_request_status {
  int state;               /* esf_request_state */
  int steps_done;
  esf_status status;       /* ESF_ERR_NUMERIC from a step, or the failure */
  double queued_ms;        /* submit -> admitted */
  double latency_ms;       /* submit -> last step done */
  double device_ms;        /* sum of the steps' device time */
  size_t footprint_bytes;  /* admission estimate */
  esf_step_report last;    /* report of the last step */
} esf_request_status;
/* admission estimate of a scene's device memory (fields, solvers, particles) */
size_t esf_scene_footprint(const esf_grid* grid, const esf_params* params, int num_solids,
                           const esf_solid_desc* solids);
esf_status esf_server_create(const esf_server_config* config, esf_server** server);
/* ESF_ERR_OOM if the request alone exceeds the budget */
esf_status esf_server_submit(esf_server* server, const esf_request* request, uint64_t* ticket);
esf_status esf_server_poll(esf_server* server, uint64_t ticket, esf_request_status* status);
/* blocks until the request is done or failed */
esf_status esf_server_wait(esf_server* server, uint64_t ticket, esf_request_status* status);
esf_status esf_server_get_field(esf_server* server, uint64_t ticket, esf_field field, int solid,
                                void* host, size_t bytes);
esf_status esf_server_release(esf_server* server, uint64_t ticket);
/* Continuous batching of the inner solves: the mixed-precision pressure
 * solves of the scenes the server is stepping hand their FP32 inner
 * iterations to one batcher. Scenes of the same grid shape advance their
 * pending inner solves in the same launches (chunks of five iterations of
 * each task), joining and leaving between chunks; each shape has its own
 * lane, and lanes run side by side. A scene whose shape no other active scene
 * shares keeps solving on its own stream. Counters since the server was
 * created. */
struct esf_batch_stats {
  long long launches;        /* launches of the batched iteration kernel */
  long long task_launches;   /* sum over those launches of the tasks they carried */
  long long max_tasks;       /* most tasks in one launch */
  long long inner_solves;    /* inner solves finished through the batcher */
  long long timed_launches;  /* launches timed with CUDA events (every 8th chunk of a lane) */
  long long timed_rows;      /* pressure rows those launches advanced by one iteration */
  double timed_ms;           /* their device time */
};
typedef struct esf_batch_stats esf_batch_stats;
esf_status esf_server_batch_stats(esf_server* server, esf_batch_stats* stats);
/* lets running requests finish their steps, drops queued ones */
esf_status esf_server_destroy(esf_server* server);

/* ---- instrumentation (no reference counterpart beyond TIMING_BREAKDOWN) -- */
/* Number of kernels this library has launched in this process (graph
 * replays count every kernel node). */
uint64_t esf_kernel_launches(void);
/* Average device time (ms) of the pressure-PCR kernels on the scene's
 * current pressure problem, timed with CUDA events on the scene's stream, at
 * the scene's precision (FP32 for ESF_MIXED): the fused update+stencil+dot
 * kernel and the axpy+norm kernel; where one kernel does the whole FP32
 * iteration (ESF_MIXED, cell rows a multiple of 4), update_ms is that kernel
 * and axpy_ms is 0. Leaves the scene's state intact. */
esf_status esf_time_pressure_kernels(esf_scene* scene, int reps, double* update_ms,
                                     double* axpy_ms);

/* ---- frames (COUPLED_INTEGRATOR_3D::writeFrame/readFrame,
 * COUPLED_INTEGRATOR_3D.cpp:977-1012; DEFOR_SOLID_3D.cpp:1299-1370) -------
 * Files "<data_path>frame.NNNN.velocity|.intensity" and, per solid i,
 * "...solid.i.displacement|.velocity|.phi|.obj", in the reference's gz and
 * OBJ formats, so frames move between the reference and this library. The
 * gz fields (and the fluid velocity) are written and read only when
 * frame % 10 == 0 or debug != 0, as in the reference; the .pbrt render
 * export is not written. Reading recomputes X, the boxes, the solid mass and
 * the particles the way readFrame does; the scene's grid must match the
 * files'. Needs zlib (libz.so.1) at run time: ESF_ERR_UNSUPPORTED without it,
 * ESF_ERR_IO on a missing or mismatched file. */
esf_status esf_write_frame(esf_scene* scene, const char* data_path, int frame, int debug);
esf_status esf_read_frame(esf_scene* scene, const char* data_path, int frame, int debug);
/* Asynchronous esf_write_frame: the frame's fields are copied on the scene's
 * stream into pinned host memory, behind the work queued so far, and a host
 * thread compresses and writes the same files once the copies have landed,
 * while the caller goes on stepping (the reference writes its frames
 * synchronously). One frame in flight per scene: the next asynchronous or
 * synchronous write, a read, or esf_destroy first waits for it;
 * esf_frame_wait waits and returns its status. */
esf_status esf_write_frame_async(esf_scene* scene, const char* data_path, int frame, int debug);
esf_status esf_frame_wait(esf_scene* scene);

#ifdef __cplusplus
}
#endif
#endif /* EULERSF_H */
