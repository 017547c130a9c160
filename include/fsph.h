/*
 * fsph.h -- C ABI of the GB300-native fluid step (hashed-grid neighbour search,
 * WCSPH density/pressure/viscosity pass, PBF density-constraint iterations).
 *
 * This ABI replaces the reference's thin C layer between its C++ particle
 * classes and CUDA (the `Cu*` functions declared in rx_cu_funcs.cuh:24-253,
 * fluid subset rx_cu_funcs.cuh:54-135) and carries the operator surface of
 * rxParticleSystemBase (rx_ps.h:55-333) / rxSPH (rx_sph.h:202-426) /
 * rxPBDSPH (rx_sph.h:1027-1274): create + Initialize, SetArrayVBO-style
 * setters, Update(dt), GetArrayVBO-style getters, neighbour access.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Vector arrays are float4 per particle
 *    (x, y, z, w) -- the reference's DIM = 4 stride (rx_ps.h:31-33); scalar
 *    arrays are one float per particle.
 *  - Every call returns an fsph_status; no exception crosses the ABI.  The
 *    text of the last error of a context is fsph_last_error(ctx).
 *  - `stream` arguments are a cudaStream_t passed as void* (NULL = the
 *    context's own stream).  Work is asynchronous on that stream except where
 *    a call says it synchronises (getters into host memory, stats).
 *  - One context per host thread at a time.  There is no CPU fallback: a
 *    context cannot be created without a CUDA device.
 */
#ifndef FSPH_H
#define FSPH_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSPH_ABI_VERSION 1

/* Status codes.  The reference printed CUDA errors and discarded them
 * (RX_CUCHECK / RX_CUERROR, rx_cuda_utils.h:22-54). */
typedef enum fsph_status {
    FSPH_OK = 0,
    FSPH_INVALID_ARG = 1,
    FSPH_OOM = 2,
    FSPH_CUDA_ERROR = 3,
    FSPH_NAN_DETECTED = 4,
    FSPH_TIMEOUT = 5,
    FSPH_NOT_CONVERGED = 6,
    FSPH_NOT_INITIALIZED = 7,
    FSPH_UNSUPPORTED = 8,
    FSPH_NO_DEVICE = 9
} fsph_status;

typedef enum fsph_solver {
    FSPH_SOLVER_WCSPH = 0, /* rxSPH::Update (rx_sph_cpu.cpp:323-380) */
    FSPH_SOLVER_PBF = 1    /* rxPBDSPH::Update (rx_sph_pbd.cpp:377-484) */
} fsph_solver;

/* Density-error definition used by the PBF convergence test.
 * ONE_SIDED = mean(max(rho - rho0, 0) / rho0), the reference GPU form
 * (rx_pbdsph_kernel.cu:431-441); TWO_SIDED = mean(|rho - rho0| / rho0), the
 * reference CPU form (rx_sph_pbd.cpp:448-454). */
typedef enum fsph_error_mode {
    FSPH_ERR_ONE_SIDED = 0,
    FSPH_ERR_TWO_SIDED = 1
} fsph_error_mode;

/* Where a host-side pointer argument lives. */
typedef enum fsph_where {
    FSPH_HOST = 0,
    FSPH_DEVICE = 1
} fsph_where;

/* Particle arrays; numbering follows rxParticleSystemBase::rxParticleArray
 * (rx_ps.h:68-116) so reference callers keep their constants. */
typedef enum fsph_array {
    FSPH_POSITION = 0,        /* float4 */
    FSPH_VELOCITY = 1,        /* float4 */
    FSPH_FORCE = 3,           /* float4, acceleration of the last force pass */
    FSPH_DENSITY = 4,         /* float */
    FSPH_PRESSURE = 5,        /* float, WCSPH only */
    FSPH_ATTRIBUTE = 7,       /* int (stored as 32-bit), user tag carried with the particle */
    FSPH_PREDICT_POS = 8,     /* float4, PBF x* */
    FSPH_PREDICT_VEL = 9,     /* float4, PBF v* */
    FSPH_SCALING_FACTOR = 10, /* float, PBF lambda */
    FSPH_CORRECTION = 11,     /* float4, PBF delta-p of the last iteration */
    FSPH_STEP_CORRECTION = 12,/* float4, x*_final - x*_predicted of the last step (warm start / collect) */
    FSPH_VORTICITY = 18,      /* float4, omega of the last finalize pass */
    FSPH_SORTED_ID = 64,      /* int, device order -> particle index (device_ptr only) */
    FSPH_FEATURES = 65        /* FSPH_MLP_FEATURES floats per particle: warm-start features for the next step */
} fsph_array;

/* Solver parameters.  Mirrors rxSPHEnviroment (rx_sph.h:95-182) after the
 * reference's Initialize has derived h, r and rho0 from it; use
 * fsph_params_from_env for that derivation, or fill the derived values
 * directly (explicit h / rho0 / m, as the benchmark configurations do). */
typedef struct fsph_params {
    int solver;              /* fsph_solver */
    int max_particles;
    float h;                 /* effective (kernel) radius */
    float mass;              /* particle mass */
    float rest_dens;         /* rho0 */
    float particle_radius;   /* wall clearance of the box projection */
    double box_min[3];       /* fluid box (rxSolidBox boundary, rx_sph_pbd.cpp:168) */
    double box_max[3];
    float gravity[3];        /* acceleration, e.g. (0, -9.81, 0) */
    float viscosity;         /* mu; WCSPH viscosity term, PBF pre-pass viscosity */
    float gas_k;             /* WCSPH gas stiffness, p = k (rho - rho0) */
    /* PBF */
    float epsilon;           /* CFM relaxation in lambda = -C / (sum |grad C|^2 + epsilon) */
    float eta;               /* density-error tolerance of the iteration loop */
    int min_iter;
    int max_iter;
    int error_mode;          /* fsph_error_mode */
    int use_ap;              /* tensile-instability correction s_corr on/off */
    float ap_k, ap_n, ap_q;  /* s_corr = -k (W(r) / W(q h))^n dt^2 */
    float xsph_c;            /* XSPH velocity smoothing c (0 = off) */
    float vort_eps;          /* vorticity confinement epsilon (0 = off) */
    /* GPU grid */
    float cell_skin;         /* cell width = h (1 + cell_skin); the grid is rebuilt
                                inside a step only when a particle moved more than
                                half the skin, cell_skin * h / 2, since the last build */
    int use_graph;           /* 1: capture the step (with a device-side while loop) in a CUDA graph */
    int warm_start;          /* 0: plain; 1: learned MLP warm start of the PBF iterations
                                (needs fsph_set_warm_start_model) */
    int clamp_constraint;    /* 0: C = rho/rho0 - 1 as the reference (rx_sph_pbd.cpp:751);
                                1: unilateral C = max(rho/rho0 - 1, 0) (opt-in, not the reference) */
    int walk_cells;          /* 0: PBF passes read per-particle neighbour lists built with
                                each grid (radius = cell width); 1: walk the 27 cells every pass */
    int collect_features;    /* 1: compute FSPH_FEATURES / FSPH_STEP_CORRECTION every step even
                                without a warm start (training-data collection) */
    int compensated_density; /* 1: Kahan-compensated FP32 density sums in the lambda pass */
    int grid_sort;           /* order of the slots by cell at each grid build, both giving the
                                order of the 64-bit key (cell << 32 | previous slot):
                                0: counting sort (atomic ranks, then each cell's slots sorted);
                                1: LSD radix sort of the 64-bit keys, 8 cell bits per pass */
    int mlp_tcgen05;         /* warm-start inference: 0 mma.sync fragments (m16n8k16);
                                1 tcgen05.mma with TMEM accumulators (fsph_mlp_forward_tcgen05),
                                a local-input network's rows brought in by TMA boxes, the default
                                of fsph_params_default; 2 the same MMAs, inputs by per-thread
                                loads (identical results) */
    int reserved[1];
} fsph_params;

/* Scene description in the reference's own terms (rxSPHEnviroment). */
typedef struct fsph_env {
    int solver;
    int max_particles;
    double boundary_cen[3];
    double boundary_ext[3];
    float dens, mass, kernel_particles, viscosity, gas_k;
    float epsilon, eta;
    int min_iter, max_iter;
    int use_ap;
    float ap_k, ap_n, ap_q;
    float gravity_y;
} fsph_env;

/* Per-step statistics (the reference's g_iIterations / g_fEta,
 * rx_sph_pbd.cpp:461-462, plus both error definitions). */
typedef struct fsph_step_stats {
    int iterations;               /* constraint iterations executed */
    int grid_builds;              /* grid builds inside the step (>= 1) */
    float density_error;          /* error of the last iteration, params.error_mode */
    float density_error_one_sided;
    float density_error_two_sided;
    float density_error_max;      /* max_i |rho_i - rho0| / rho0 */
    int status;                   /* FSPH_OK, FSPH_NOT_CONVERGED, FSPH_NAN_DETECTED */
    int kernels;                  /* kernel launches the step executed (PBF graph mode; 0 = not counted) */
    int bounds_bits;              /* a library built with FSPH_DEBUG_BOUNDS (fltk_sph_ice_gb300.build
                                     --debug-bounds): the index checks that failed this step, 1 neighbour
                                     slot, 2 cell row, 8 list count, 16 boundary slot; always 0 otherwise */
    int reserved[1];
} fsph_step_stats;

typedef struct fsph_ctx fsph_ctx;

/* ---- version / errors ---- */
int fsph_abi_version(void);
const char *fsph_status_string(int status);
const char *fsph_last_error(const fsph_ctx *ctx);

/* ---- parameters ---- */
/* rxPBDSPH::Initialize / rxSPH::Initialize derivation (rx_sph_pbd.cpp:102-201,
 * rx_sph_cpu.cpp:92-166): h from kernel_particles, r, rho0 by calRestDensity,
 * box = cen -/+ ext.  Fills the remaining fields with defaults. */
int fsph_params_from_env(const fsph_env *env, fsph_params *out);
/* Defaults for every field (solver PBF, no particles). */
void fsph_params_default(fsph_params *out);

/* ---- context (Initialize / Finalize) ---- */
int fsph_create(const fsph_params *params, fsph_ctx **out);
int fsph_destroy(fsph_ctx *ctx);
int fsph_set_params(fsph_ctx *ctx, const fsph_params *params);
int fsph_get_params(const fsph_ctx *ctx, fsph_params *out);
int fsph_num_particles(const fsph_ctx *ctx);

/* ---- particle data (Set / SetArrayVBO) ---- */
/* Replace all particles: pos4/vel4 hold n float4 in particle order (vel4 may
 * be NULL for zero velocity).  Like rxParticleSystemBase::Set (rx_ps.cpp:30-59)
 * this resets the particle count to n (n <= max_particles). */
int fsph_set_particles(fsph_ctx *ctx, const float *pos4, const float *vel4, int n, int where);
/* Overwrite `count` particles from index `start` of one array
 * (SetArrayVBO, rx_ps.h:260-262).  FSPH_POSITION, FSPH_VELOCITY, FSPH_ATTRIBUTE.
 * Positions and velocities must be finite: a range holding a NaN or an
 * infinity returns FSPH_NAN_DETECTED and leaves the state unchanged.  They
 * land in their particles' device slots and nothing else moves, so writing
 * back what fsph_get_array returned leaves the next steps bit-identical. */
int fsph_set_array(fsph_ctx *ctx, int type, const void *data, int start, int count, int where);

/* ---- step (Update) ---- */
/* Advance one step of dt.  stats may be NULL (then nothing synchronises);
 * otherwise the call waits for the step and fills stats.  Returns
 * FSPH_INVALID_ARG when there are no particles (the reference's Update
 * returns false for N = 0, rx_sph_pbd_gpu.cpp:818). */
int fsph_step(fsph_ctx *ctx, float dt, void *stream, fsph_step_stats *stats);
/* Stats of the last step (synchronises). */
int fsph_last_stats(fsph_ctx *ctx, fsph_step_stats *stats);

/* ---- access (GetArrayVBO / GetParticleDevice) ---- */
/* Copy one array out in particle order (index = the order given to
 * fsph_set_particles).  dst holds n float4 / n floats; where says whether dst
 * is host (synchronises) or device memory. */
int fsph_get_array(fsph_ctx *ctx, int type, void *dst, int where, void *stream);
/* Borrowed device pointer to an internal array, in DEVICE order (see
 * FSPH_SORTED_ID for the device slot -> particle index map); valid until the
 * next fsph_step / fsph_set_particles.  Synchronises the context's own
 * stream first, so work queued without a caller stream (fsph_set_array) is
 * visible through it.  NULL on error. */
const void *fsph_device_ptr(fsph_ctx *ctx, int type);
/* Synchronise the context's stream. */
int fsph_sync(fsph_ctx *ctx);

/* ---- neighbour sets (GetNeights / SetParticlesToCell, rx_sph.h:1196) ---- */
/* Neighbour sets of the current positions under the reference criterion
 * fl32(|x_i - x_j|^2 evaluated in double) <= fl32(h*h), self included
 * (rx_nnsearch.h:487-515).  CSR in particle order: offsets[n+1]; indices
 * (particle indices, ascending within each row) holds at most cap entries;
 * *total receives the number of entries.  Synchronises. */
int fsph_neighbors(fsph_ctx *ctx, int *offsets, int *indices, long long cap, long long *total);
/* The same for any positions (SetParticlesToCell(prts, n, h) + GetNeights,
 * rx_sph_pbd.cpp:1735-1750, rx_nnsearch.h:454-515): pos4 = n float4 (host or
 * device, `where`) whose neighbours among themselves are wanted, or NULL for
 * the context's particles (n ignored); radius <= 0 means params.h, and it
 * may not exceed the grid's cell width h (1 + cell_skin) (FSPH_UNSUPPORTED).
 * dist2 (optional, same length as indices) receives each pair's squared
 * distance as the reference's rxNeigh::Dist2: float coordinates differenced
 * and squared in double, rounded to float.  With indices NULL or cap below
 * the total, only offsets and *total are written.  Synchronises. */
int fsph_neighbors_ex(fsph_ctx *ctx, const float *pos4, int n, float radius, int where, int *offsets,
                      int *indices, float *dist2, long long cap, long long *total);

/* ---- dynamic particle count: inlets and deletion regions ---- */
/* A deleted particle keeps its index: attribute -1, parked at (0, 0, 1e6)
 * with zero velocity (checkDeletePB, rx_pbdsph_kernel.cu:1171-1187), and
 * takes no further part in the steps; fsph_num_particles counts it,
 * fsph_num_active does not.  Writing an attribute of -1 through
 * fsph_set_array deletes a particle the same way, another value revives it. */
int fsph_num_active(const fsph_ctx *ctx);
/* Particles strictly inside [lo, hi] at the end of a step are deleted (the
 * reference applies its regions after the position update,
 * rx_sph_gpu.cpp:875-890; env.delete_region, rx_sph.h:125-126).  At most 64. */
int fsph_add_delete_region(fsph_ctx *ctx, const double *lo, const double *hi);
int fsph_clear_delete_regions(fsph_ctx *ctx);
/* An inlet line (rxInletLine / AddLine, rx_ps.h:41-49, rx_ps.cpp:432-436):
 * when fsph_emit_inlets is called for a step with step % span == 0, the
 * line adds accum rows of n = |pos2 - pos1| / r particles (r the particle
 * radius), spaced l / n along it from (i + 1/2) l / n, jittered by 0.01 of
 * that spacing, rows stacked along `up` by spacing * (l / n), with velocity
 * vel and attribute = the line's index (addParticles, rx_ps.cpp:444-520).
 * Returns the number of lines (> 0) or a negative status. */
int fsph_add_inlet_line(fsph_ctx *ctx, const double *pos1, const double *pos2, const double *vel,
                        const double *up, int accum, int span, double spacing);
int fsph_clear_inlets(fsph_ctx *ctx);
/* The number of inlet lines (the size of the reference's m_vInletLines,
 * rx_ps.h:171; -1 for a NULL context). */
int fsph_num_inlets(const fsph_ctx *ctx);
/* Emit the particles of the lines due at `step` (rxPBDSPH_GPU::Update,
 * rx_sph_pbd_gpu.cpp:795-815, before the step): after the existing
 * particles at first, then from where the last emission ended, wrapping to
 * index 0 past max_particles as the reference does.  *emitted (optional)
 * receives the count.  Synchronises. */
int fsph_emit_inlets(fsph_ctx *ctx, int step, int *emitted);

/* ---- the reference's cell indices ---- */
/* The reference's cell hash z*Gy*Gx + y*Gx + x of each of n positions
 * (float4 stride), for parity of cell indices: rule 0 = the reference's CPU
 * grid (rxNNGrid::Setup / CalGridHash(Vec3), rx_nnsearch.h:174-199, 590-599:
 * power-of-two axis counts, (p - min) / cw in double truncated), rule 1 =
 * its GPU grid (setupCells, rx_sph_pbd_gpu.cpp:1986-2011, and calcGridPos /
 * calcGridHash, rx_cu_common.cu:121-144: floor(L/cw) + 1 cells per axis,
 * float floor); both over the box grown by 1 % (rx_sph_pbd.cpp:188-196) with
 * the context's h, cell coordinates clamped to [0, G-1].  grid[3] and
 * cell_width (either may be NULL) receive the geometry.  This context's own
 * grid is a different, padded one (cell width h(1 + cell_skin)); the
 * neighbour sets do not depend on the grid. */
int fsph_reference_cell_hash(fsph_ctx *ctx, int rule, const float *pos4, int n, int where, unsigned int *hash,
                             int *grid, double *cell_width);

/* ---- density on a lattice, for surface meshing ---- */
/* CalImplicitField / CalImplicitFieldDevice (rx_ps.h:283-285;
 * rxPBDSPH::CalImplicitField -> CalColorField, rx_sph_pbd.cpp:2024-2108;
 * on the GPU pbdsphCalDensityInGrid / sphCalDensityInGrid,
 * rx_pbdsph_kernel.cu:1220-1299, rx_sph_kernel.cu:1038-1085): the density
 * sum_j m W_poly6(|x - x_j|) of the current particles at the nodes of an
 * n[0] x n[1] x n[2] lattice, node (i, j, k) at minp + (i, j, k) d, stored
 * at out[k n0 n1 + j n0 + i] (host or device float array per `where`);
 * nodes outside the simulation range (the box grown by 1 %, as the
 * reference's Initialize sets it) read 0.  The field a marching-cubes mesher
 * consumes (rx_mc_kernel.cu).  Synchronises. */
int fsph_density_grid(fsph_ctx *ctx, const int *n, const double *minp, const double *d, float *out, int where);

/* ---- fields without moving the particles (UpdateWithoutPosAndVel) ---- */
/* rxSPH_GPU::UpdateWithoutPosAndVel (rx_sph_gpu.cpp:925-1060; the pure
 * virtual of rx_ps.h:254): a step's field evaluation without its position
 * and velocity update.  WCSPH: density, pressure and acceleration
 * (calDensity + calForce); PBF: the step's pre-pass, density and the
 * external + viscous acceleration (calDensity + calForceExtAndVisc,
 * rx_sph_pbd.cpp:599-689).  FSPH_DENSITY / FSPH_PRESSURE / FSPH_FORCE then
 * read them; positions and velocities are unchanged.  Synchronises. */
int fsph_step_fields(fsph_ctx *ctx, float dt, void *stream);

/* ---- single passes, for parity checks against the CPU path ---- */
/* PBF lambda pass on the given positions (rxPBDSPH::calScalingFactor,
 * rx_sph_pbd.cpp:699-914): density and scaling factor per particle. Host arrays. */
int fsph_pbf_eval_lambda(fsph_ctx *ctx, const float *pos4, int n, float *dens, float *lambda);
/* PBF position-correction pass (rxPBDSPH::calPositionCorrection,
 * rx_sph_pbd.cpp:925-1026) for given positions and lambdas.  Host arrays. */
int fsph_pbf_eval_correction(fsph_ctx *ctx, const float *pos4, const float *lambda, int n,
                             float dt, float *dp4);
/* The end-of-step passes of a PBF step on given inputs: the XSPH velocity
 * smoothing v_i + c sum_j (m / rho_j)(v_j - v_i) W_ij (xsphVisocosity,
 * rx_pbdsph_kernel.cu:1090-1162, disabled in the reference at
 * rx_sph_pbd_gpu.cpp:926-927) and the vorticity confinement of Macklin &
 * Mueller 2013, eq. 15-16 (only a flag in the reference, rx_ps.h:161,238,
 * the paper cited at rx_sph.h:1281), with params.xsph_c / vort_eps and dt.
 * pos4, vel4 (n float4) and dens (n floats, the densities the passes divide
 * by) in; vel_out4 (the velocity after both) and vort4 (omega) out.  Host
 * arrays; synchronises. */
int fsph_pbf_eval_xsph_vorticity(fsph_ctx *ctx, const float *pos4, const float *vel4, const float *dens, int n,
                                 float dt, float *vel_out4, float *vort4);
/* WCSPH density + force passes (rxSPH::calDensity / calForce,
 * rx_sph_cpu.cpp:495-656).  Host arrays; acc4 receives the acceleration. */
int fsph_sph_eval_forces(fsph_ctx *ctx, const float *pos4, const float *vel4, int n,
                         float *dens, float *pres, float *acc4);

/* ---- allocation-free variant ---- */
/* Largest inputs of fsph_pbf_eval_lambda_noalloc: its scratch is a fixed
 * device array of about 10.3 MB inside the library. */
#define FSPH_NOALLOC_MAX_PARTICLES 65536
#define FSPH_NOALLOC_MAX_CELLS (1 << 20)
/* The lambda pass of fsph_pbf_eval_lambda (density and scaling factor of n
 * particles at the given positions) for callers that cannot allocate device
 * memory: a host application that hands the whole GPU to its own memory
 * pool, or a real-time loop where an allocation's latency or failure is not
 * acceptable.  No counterpart in the reference.
 *   - pos4, dens and lambda are DEVICE pointers owned by the caller
 *     (n float4 in, n floats out each), in particle order.  No context is used,
 *     so static boundary particles (fsph_set_boundary) never enter: the
 *     results equal fsph_pbf_eval_lambda's only for a context without a boundary.
 *   - It allocates nothing: no cudaMalloc / cudaFree / allocating library call.
 *     Its working memory (grid tables, sorted copies) is one file-scope
 *     __device__ array that every GPU loading the library holds until exit.
 *   - n <= FSPH_NOALLOC_MAX_PARTICLES and the wall box padded by one cell of
 *     width h (1 + cell_skin) must span <= FSPH_NOALLOC_MAX_CELLS cells;
 *     larger inputs return FSPH_INVALID_ARG without launching anything.
 *   - The first call on a device looks up that array's device address (once
 *     per device); make that first call before any stream capture.
 *   - Work is enqueued on `stream` (NULL = legacy default stream) and the call
 *     returns without waiting.  Every call shares the one array and leaves its
 *     contents behind, so calls that overlap on the GPU (other streams, other
 *     host threads) race: order them on one stream or synchronise between them. */
int fsph_pbf_eval_lambda_noalloc(const fsph_params *params, const float *pos4, int n, float *dens,
                                 float *lambda, void *stream);

/* ---- static boundary particles (PBF) ---- */
/* Replaces the boundary set-up of rxPBDSPH::Initialize (rx_sph_pbd.cpp:180,
 * 280-297: particles sampled on a solid's surface, then calBoundaryVolumes,
 * rx_sph_pbd.cpp:1061-1090) and rxPBDSPH_GPU::InitBoundary
 * (rx_sph_pbd_gpu.cpp:654-754).  The caller gives the boundary particles'
 * float4 positions (the sampling of a solid is the caller's, e.g. the
 * surface of a box at spacing 1.2 r as rxSolid::GenerateParticlesOnSurf).
 * Each then has a volume psi_b = m / sum_b' m W(r_bb'), adds
 * rho0 psi_b W to the density of fluid neighbours, gets its own lambda_b
 * every pass and enters the position correction (rx_sph_pbd.cpp:624-644,
 * 728-818, 824-913, 977-1019; compiled in by RX_USE_BOUNDARY_PARTICLE).
 * nb = 0 removes the boundary.  The boundary stays fixed. */
typedef enum fsph_boundary_array {
    FSPH_BOUNDARY_POSITION = 0,  /* float4 per boundary particle, as given */
    FSPH_BOUNDARY_VOLUME = 1,    /* psi_b */
    FSPH_BOUNDARY_LAMBDA = 2     /* lambda_b of the last lambda pass */
} fsph_boundary_array;
int fsph_set_boundary(fsph_ctx *ctx, const float *bpos4, int nb, int where);
int fsph_num_boundary(const fsph_ctx *ctx);
/* host dst, the given order of the boundary particles */
int fsph_get_boundary(fsph_ctx *ctx, int which, float *dst);

/* ---- analytic obstacles ---- */
/* SetBoxObstacle / SetSphereObstacle / MoveSphereObstacle /
 * GetSphereObstaclePos (rx_ps.h:266-272; rxPBDSPH_GPU, rx_sph_pbd_gpu.cpp:
 * 2425-2480): at most 10 boxes and 10 spheres (MAX_BOX_NUM /
 * MAX_SPHERE_NUM, rx_cu_common.cuh:135-136).  A particle that the
 * prediction, a position correction or a WCSPH integration leaves inside an
 * obstacle moves to its surface: a box -- centre cen, half extents ext,
 * rotated by the Euler angles ang (degrees; pitch, yaw, roll as
 * EulerToMatrix, rx_sph_commons.h:185-210) -- through its nearest face, a
 * sphere radially (collisionPointBox / collisionPointSphere,
 * rx_cu_common.cu:748-831), obstacles before the box walls.  The velocity
 * is not reflected (the CPU path's reflection is commented out,
 * rx_sph_pbd.cpp:1384); vel is accepted and unused, as in the reference's
 * fluid step; flg = 0 adds nothing.  Obstacles apply to both solvers; the
 * batched scenes take none. */
int fsph_set_box_obstacle(fsph_ctx *ctx, const double *cen, const double *ext, const double *ang,
                          const double *vel, int flg);
int fsph_set_sphere_obstacle(fsph_ctx *ctx, const double *cen, double rad, const double *vel, int flg);
/* moves sphere b (in the order added) by disp; takes effect at the next step */
int fsph_move_sphere_obstacle(fsph_ctx *ctx, int b, const double *disp);
int fsph_get_sphere_obstacle_pos(const fsph_ctx *ctx, int b, double *pos);
int fsph_clear_obstacles(fsph_ctx *ctx);
int fsph_num_obstacles(const fsph_ctx *ctx);

/* Triangle-mesh obstacle (SetPolygonObstacle, rx_ps.h:268;
 * rxPBDSPH_GPU::SetPolygonObstacle, rx_sph_pbd_gpu.cpp:2367-2410): nv
 * vertices (x, y, z doubles, stored as floats as the reference stores them)
 * and nt triangles (three vertex indices into this mesh each), appended to
 * the meshes already set; vel is unused, as in the reference.  The
 * triangles are binned into the cells of the reference's GPU grid they
 * intersect (setPolysToCell, rx_sph_pbd_gpu.cpp:2051-2200).  In the step's
 * prediction (PBF; the WCSPH integration) each particle's segment from its
 * position to its prediction is tested against the triangles of the cells
 * of both ends, and a crossing from a triangle's front side puts the
 * particle back on that side with the velocity component into the triangle
 * removed (pbdsphIntegrateWithPolygon / calCollisionPolygonPB,
 * rx_pbdsph_kernel.cu:916-1030; sphIntegrateWithPolygon,
 * rx_sph_kernel.cu:852-895), before the box and sphere obstacles and the
 * walls.  The reference re-runs that integration after every constraint
 * iteration with zero velocity, where a zero-length segment never crosses,
 * so only the prediction does it here.  Differences from the reference:
 * the triangles of a later mesh index its own vertices (the reference
 * appends them unshifted, so a second mesh points into the first);
 * every non-empty cell of the table is closed (the reference leaves the
 * last one open, dropping its triangles); a zero-area triangle is skipped
 * (the reference reports a hit at a NaN point).  Synchronises. */
int fsph_set_polygon_obstacle(fsph_ctx *ctx, const double *vrts, int nv, const int *tris, int nt,
                              const double *vel);
int fsph_clear_polygon_obstacles(fsph_ctx *ctx);
int fsph_num_polygon_triangles(const fsph_ctx *ctx);
/* The collision of the triangle meshes alone, for parity: for each of n
 * segments x0[i] -> x1[i] (float4 stride) with velocity v[i], x1 and v are
 * updated in place as the prediction does (host or device arrays per
 * `where`).  Synchronises. */
int fsph_polygon_collide(fsph_ctx *ctx, const float *x0_4, float *x1_4, float *v4, int n, float dt, int where);

/* ---- learned warm start ---- */
/* The network: FSPH_MLP_FEATURES -> 64 -> 64 -> 3, ReLU, BF16 tensor-core
 * arithmetic with FP32 accumulation.  Its parameters are one FP32 blob of
 * FSPH_MLP_BLOB_SIZE floats: mu[32], sigma[32] (input standardisation),
 * W1[32][64], b1[64], W2[64][64], b2[64], W3[64][3], b3[3], out_scale[1].
 * Output = (network of (x - mu) / sigma) * out_scale = predicted step
 * correction / h.  An input whose sigma is >= 1e29 carries no weight; when
 * inputs 16-22 (the neighbour means) all carry none, the step neither
 * computes nor reads them.  No counterpart in the reference (its PBF loop always
 * starts from the prediction, rx_sph_pbd.cpp:418-425). */
#define FSPH_MLP_FEATURES 32
#define FSPH_MLP_HIDDEN 64
#define FSPH_MLP_OUTPUTS 3
#define FSPH_MLP_BLOB_SIZE 6532
typedef struct fsph_mlp fsph_mlp;
int fsph_mlp_create(fsph_mlp **out);
int fsph_mlp_destroy(fsph_mlp *m);
int fsph_mlp_set_blob(fsph_mlp *m, const float *blob);            /* host blob; resets Adam */
int fsph_mlp_get_blob(fsph_mlp *m, float *blob);                  /* host blob */
const char *fsph_mlp_last_error(const fsph_mlp *m);
/* The network's calls run on its own stream (or the given one): device
 * inputs written by other streams must be complete before a call (for
 * gradient / train, which take no stream, synchronise the producing stream).
 * y[n][3] = network(x[n][16]); device pointers; stream NULL = synchronous */
int fsph_mlp_forward(fsph_mlp *m, const float *x, int n, float *y, void *stream);
/* The same forward pass on the tcgen05 tensor cores (operands in shared
 * memory, FP32 accumulators in tensor memory), 128 rows per MMA; the
 * accumulation order inside an MMA differs from fsph_mlp_forward's, so the
 * two agree to FP32 rounding of the sums (and the BF16 rounding of a hidden
 * unit that lands between them).  Synchronous; FSPH_TIMEOUT if a bounded wait
 * on an MMA ran out. */
int fsph_mlp_forward_tcgen05(fsph_mlp *m, const float *x, int n, float *y);
/* gradient of the mean squared error mean_i sum_k (y_ik - t_ik)^2 w.r.t. the
 * blob (host, FSPH_MLP_BLOB_SIZE floats; zero for mu, sigma, out_scale);
 * x, t device pointers; *loss receives the loss. Synchronous. */
int fsph_mlp_gradient(fsph_mlp *m, const float *x, const float *t, int n, float *grad, float *loss);
/* Adam (beta 0.9 / 0.999) over `epochs` passes of consecutive minibatches of
 * `batch` rows of (x, t) (device pointers); loss_per_epoch (host, optional). */
int fsph_mlp_train(fsph_mlp *m, const float *x, const float *t, int n, int batch, int epochs, float lr,
                   float *loss_per_epoch);
/* Install a trained blob (host) as the context's warm-start network. */
int fsph_set_warm_start_model(fsph_ctx *ctx, const float *blob);

/* ---- checkpoint / resume ---- */
/* Write everything a step reads to `path`, in device order, so that
 * fsph_load_state into a context of the same solver resumes bit-identically
 * to continuing without the checkpoint: the parameters, the particles'
 * positions, velocities, attributes and slot order, the warm-start history
 * and network, the boundary particles, obstacles, inlet lines (with the
 * ring index of the next emission), deletion regions and the step count.
 * The inlet jitter is a counter-based function of (line, step), so no
 * random-generator state exists to save.  The reference's checkpoint is the
 * particle file alone (OutputParticles / InputParticles, rx_ps.cpp:581-644:
 * uint32 N, positions, velocities), which fsph_particle_system.hpp writes
 * beside this file.  The per-step fields (density, lambda, forces) are not
 * saved: the next step recomputes them.  A file of another build version or
 * a truncated file is rejected with FSPH_INVALID_ARG before the context is
 * changed.  Synchronises. */
int fsph_save_state(fsph_ctx *ctx, const char *path);
int fsph_load_state(fsph_ctx *ctx, const char *path);

/* ---- records and test hooks ---- */
/* Append one JSON line per step to `path` (NULL or "" stops): step number,
 * solver, dt, particle counts, iterations, grid builds, the three density
 * errors, status and the host-timed step in ms.  While a log is open every
 * step waits for its stats.  The reference's per-step figures were the
 * globals g_iIterations / g_fEta (rx_sph_pbd.cpp:461-462) and RXTIMER prints. */
int fsph_set_step_log(fsph_ctx *ctx, const char *path);
/* Device-allocation fault injection, process-wide, for testing the error
 * paths: allocations larger than max_bytes (>= 0) and the allocation
 * numbered fail_at (0 = the next one; < 0 never) fail with FSPH_OOM without
 * calling cudaMalloc.  fsph_set_alloc_fault(-1, -1) switches it off.
 * No counterpart in the reference. */
int fsph_set_alloc_fault(long long max_bytes, long long fail_at);

/* ---- measurement ---- */
typedef enum fsph_pass {
    FSPH_PASS_LAMBDA = 0,      /* one lambda pass (density + constraint + error reduction) */
    FSPH_PASS_CORRECTION = 1,  /* one position-correction pass */
    FSPH_PASS_GRID = 2,        /* one grid build (hash, scan, scatter, cell sort, reorder) */
    FSPH_PASS_LIST = 3,        /* one neighbour-list build on the current grid */
    FSPH_PASS_SPH_DENSITY = 4, /* WCSPH: one density + pressure pass */
    FSPH_PASS_SPH_FORCE = 5    /* WCSPH: one force (pressure + viscosity + gravity) pass */
} fsph_pass;
/* Time `reps` back-to-back launches of one pass of the current state (the
 * PBF passes on a PBF context, the WCSPH passes on a WCSPH one) with CUDA
 * events on the context's stream; *avg_ms receives the mean time of one
 * launch.  A PBF state is advanced as the passes would advance it
 * (corrections are applied), so call it after the steps to be kept; the
 * WCSPH passes leave the particles unchanged.
 * No counterpart in the reference (its timing was the GUI's RXTIMER splits,
 * rx_sph.h:40-58). */
int fsph_time_pass(fsph_ctx *ctx, int pass, int reps, float *avg_ms);

/* ---- batched scenes ---- */
/* Many independent PBF scenes of uneven sizes advanced together: every pass
 * of the step is one persistent launch over all scenes (tiles of one scene
 * per block), and the whole step -- a fixed number of constraint
 * iterations -- is one CUDA graph.  Each scene behaves as its own
 * rxPBDSPH::Update (rx_sph_pbd.cpp:377-484) with its own fsph_params (h,
 * mass, box, ...), run for exactly `iterations` iterations; the reference has
 * no batched form (one rxPBDSPH object per scene, one Update call each).
 * Arrays cross this interface scene after scene, each scene in its own
 * particle order; fsph_batch_offsets gives where each scene starts. */
typedef struct fsph_batch fsph_batch;
typedef struct fsph_batch_config {
    int block;         /* threads per block of the persistent launches: 128, 256 or 512 */
    int lanes;         /* lanes sharing one particle in the constraint passes: 1, 2 or 4 */
    float cell_skin;   /* cell width = h (1 + cell_skin), in [0.02, 0.5] */
    int eager;         /* 1: host-driven iteration loop instead of the CUDA graph (same kernels; profilers) */
} fsph_batch_config;
/* params[s] (PBF) and counts[s] particles for each of the nscenes scenes. */
int fsph_batch_create(const fsph_params *params, const int *counts, int nscenes, int iterations,
                      fsph_batch **out);
int fsph_batch_destroy(fsph_batch *b);
const char *fsph_batch_last_error(const fsph_batch *b);
int fsph_batch_num_particles(const fsph_batch *b);
/* offsets[nscenes + 1]: first particle of each scene in the batched arrays */
int fsph_batch_offsets(const fsph_batch *b, int *offsets);
/* all scenes' float4 positions (and velocities; NULL = zero) back to back */
int fsph_batch_set_particles(fsph_batch *b, const float *pos4, const float *vel4, int where);
/* one step of every scene; stream NULL = the batch's own stream */
int fsph_batch_step(fsph_batch *b, float dt, void *stream);
/* FSPH_POSITION, FSPH_VELOCITY (float4) or FSPH_DENSITY (float), all scenes */
int fsph_batch_get_array(fsph_batch *b, int type, void *dst, int where);
/* the last step's iterations, grid builds and density errors of scene s */
int fsph_batch_scene_stats(fsph_batch *b, int scene, fsph_step_stats *stats);
int fsph_batch_set_config(fsph_batch *b, const fsph_batch_config *cfg);
int fsph_batch_get_config(const fsph_batch *b, fsph_batch_config *cfg);
/* Autotuner: times `steps` steps of dt under every candidate configuration
 * (block x lanes x cell skin) from the current state, restores that state,
 * installs the fastest configuration and returns it with its time per step.
 * The winner is cached per scene-set signature (counts and parameters) for
 * the life of the process, and reused without timing. */
int fsph_batch_autotune(fsph_batch *b, float dt, int steps, fsph_batch_config *best, float *best_ms_per_step);

#ifdef __cplusplus
}
#endif

#endif /* FSPH_H */
