/*
 * tisphi_gb300 - C ABI of the GB300 (sm_103a) SPH step library.
 *
 * The reference (Rabmelon/tiSPHi) has no FFI layer: its hot path is a set of Taichi
 * kernels reached through Python objects.  Each entry point below replaces one of those
 * kernels (or one solver method that launches several); the comment on each names the
 * reference interface it replaces (file:line inside the reference project).  The Python
 * package tisphi_gb300 binds these through ctypes and mirrors the reference's object API
 * (Simulation / ParticleSystem / SPHBase / WCSPHSolver / MUISPHSolver / DPSPHSolver).
 *
 * Conventions
 *  - Every call that launches GPU work takes a CUDA stream (cudaStream_t passed as
 *    void*; NULL = legacy default stream) and is asynchronous unless stated.
 *  - Status: 0 = OK; > 0 = bits of the device error word (TSG_ERR_*); < 0 = API misuse or
 *    a CUDA error (TSG_E_*).  No call aborts the process.
 *  - Particle arrays handed to tsg_upload are row-major host or device arrays:
 *    vectors (n, 3), matrices (n, 3, 3), scalars (n,).  All f64 / int32.
 *  - The handle owns every device buffer; tsg_field returns a view that stays valid until
 *    the next call that reorders particles (tsg_sort / tsg_step) or tsg_destroy.
 */
#ifndef TISPHI_GB300_H
#define TISPHI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tsg_handle tsg_handle;

/* precision forms */
enum { TSG_FP64 = 0, TSG_FP32_MIXED = 1 };

/* tsg_advect selectors */
enum {
    TSG_ADVECT_FULL = 1,       /* advect_SE / advect_LF (eng/solver_sph_base.py:79-87, :106-114) */
    TSG_ADVECT_LF_HALF = 2,    /* advect_LF_half (eng/solver_sph_base.py:96-104) */
    TSG_ADVECT_POS = 3,        /* advect_pos + XSPH (eng/solver_sph_base.py:224-238) */
    TSG_ADVECT_SOMETHING = 4,  /* advect_something (eng/solver_sph_base.py:244-247 + solver overrides) */
    TSG_ENFORCE_BOUNDARY = 5,  /* enforce_boundary (eng/solver_sph_base.py:525-601) */
    TSG_RK_INIT = 6,           /* init_RK (eng/solver_sph_base.py:144-151) */
    TSG_RK_STAGE = 7,          /* advect_RK_4 (eng/solver_sph_base.py:134-142) */
    TSG_RK_FINAL = 8           /* advect_RK (eng/solver_sph_base.py:162-170) */
};

/* device error word bits */
enum {
    TSG_ERR_CELL_OOB = 1,      /* a particle's flattened cell index left [0, grid_num_total) */
    TSG_ERR_NONFINITE = 2,     /* a non-finite density or position was produced */
    TSG_ERR_PACK_RANGE = 4     /* FP32-mixed: a cell coordinate exceeded the packing range */
};

/* negative status codes */
enum {
    TSG_E_ARG = -1, TSG_E_CONFIG = -2, TSG_E_CUDA = -3, TSG_E_STATE = -4, TSG_E_UNSUPPORTED = -5,
    TSG_E_NAME = -6, TSG_E_CAPACITY = -7
};

/* Scene and solver constants, as the reference's Python scope holds them
 * (eng/particle_system.py:14-59, eng/solver_sph_base.py:12-26, solver constructors). */
typedef struct tsg_config {
    int32_t dim;               /* 2 or 3 */
    int32_t solver;            /* 1 WCSPH, 2 mu(I), 3 Drucker-Prager (eng/simulation.py:14-22) */
    int32_t kernel;            /* 0 cubic spline, 1 Wendland C2 */
    int32_t kernel_corr;       /* 0 none, 1 CSPM */
    int32_t time_integration;  /* 1 SE, 2 LF, 4 RK4 */
    int32_t xsph;              /* 0 / 1 */
    int32_t boundary;          /* 0 none, 1 collision, 2 dummy, 3 repulsive, 4 dummy + repulsive */
    int32_t precision;         /* TSG_FP64 or TSG_FP32_MIXED */
    int32_t exponent_is_int;   /* Tait exponent is an integer */
    int32_t init_geostatic;    /* DP: apply init_stress on upload (eng/solver_sph_dp.py:35) */
    int32_t grid_num[3];
    int64_t grid_num_total;
    double vdomain_start[3];
    double domain_start[3];
    double domain_end[3];
    double grid_size;
    double support_radius;
    double smoothing_len;
    double particle_diameter;
    double particle_radius;
    double gravity[3];
    double dt;
    double density0;
    double viscosity;
    double stiffness;
    double exponent;
    double cohesion;           /* Pa */
    double friction;           /* rad */
    double E;                  /* Young's modulus */
    double poisson;
    double dilatancy;          /* rad */
    double damping_eps;        /* viscous damping coefficient (eng/solver_sph_base.py:714) */
    double list_skin;          /* FP32-mixed: neighbour-list skin as a fraction of the support
                                  radius; lists are rebuilt (and particles re-sorted) when a
                                  particle has moved 0.45 skin since the last build; 0 = every
                                  step.  Ignored by the FP64 form, which sorts every step. */
} tsg_config;

/* Initial particle set (eng/particle_system.py:289-314 _add_particles). */
typedef struct tsg_particles {
    int64_t n;
    const double* x;           /* (n, 3) */
    const double* v;           /* (n, 3) */
    const double* density;     /* (n,) */
    const double* mass;        /* (n,) */
    const double* m_V;         /* (n,) */
    const double* pressure;    /* (n,) */
    const double* stress;      /* (n, 3, 3) or NULL (zeros) */
    const int32_t* mat_type;   /* -2 repulsive, -1 dummy, 1 fluid, 2 soil, 11 rigid */
    const int32_t* mat_id;
    const int32_t* obj_id;
    const int32_t* is_dynamic;
} tsg_particles;

/* Strided view of one device field. */
typedef struct tsg_view {
    void* data;                /* device pointer */
    int32_t dtype;             /* 0 f64, 1 f32, 2 i32 */
    int32_t ndim;
    int64_t shape[3];
    int64_t strides[3];        /* in elements */
} tsg_view;

/* Create a solver instance.  Replaces ParticleSystem.__init__'s field allocation
 * (eng/particle_system.py:113-125) and the solver constructors' constant set-up
 * (eng/solver_sph_wc.py:7-21, eng/solver_sph_muI.py:7-25, eng/solver_sph_dp.py:7-35). */
int tsg_create(const tsg_config* cfg, tsg_handle** out);

/* Load the initial particles (host or device pointers, from_device = 0/1) and set
 * id0 = index.  Replaces _add_particles + set_id0 (eng/particle_system.py:208-211,
 * :289-314) and, for DP, init_stress (eng/solver_sph_base.py:249-260). */
int tsg_upload(tsg_handle* h, const tsg_particles* p, int from_device, void* stream);

/* Cell hash + prefix sum + stable counting sort.  Replaces initialize_particle_system
 * (eng/particle_system.py:228-257). */
int tsg_sort(tsg_handle* h, void* stream);

/* Shepard factor for all particles and, when kernel_corr == 1, the CSPM gradient
 * correction matrix.  Replaces calc_kernel_corr (eng/solver_sph_base.py:363-423). */
int tsg_kernel_corr(tsg_handle* h, void* stream);

/* density_tmp = density, v_tmp = v, stress_tmp = stress.  Replaces init_real2tmp
 * (eng/solver_sph_base.py:67-74). */
int tsg_init_tmp(tsg_handle* h, void* stream);

/* One evaluation of the rates.  Replaces WCSPHSolver.one_step (eng/solver_sph_wc.py:82-127),
 * MUISPHSolver.one_step (eng/solver_sph_muI.py:62-131) or DPSPHSolver.one_step
 * (eng/solver_sph_dp.py:210-274), by the configured solver. */
int tsg_one_step(tsg_handle* h, void* stream);

/* Per-particle update selected by TSG_ADVECT_*; see the enum for the reference kernels. */
int tsg_advect(tsg_handle* h, int which, void* stream);

/* d_density_RK += m d_density, d_vel_RK += m d_vel, d_stress_RK += m d_stress for real
 * particles, m = 1 or 2.  Replaces update_RK (eng/solver_sph_base.py:153-160); with the
 * TSG_RK_* advect calls it lets a caller run substep_RK on a handle of any integrator. */
int tsg_rk_update(tsg_handle* h, int32_t m, void* stream);

/* substep(): SE / LF / RK4 sequence of one_step and advect calls
 * (eng/solver_sph_base.py:53-61, :89-91, :116-120, :172-180). */
int tsg_substep(tsg_handle* h, void* stream);

/* nsteps x SPHBase.step (eng/solver_sph_base.py:41-51).  The FP32-mixed WCSPH step
 * (symplectic Euler or leap-frog) computes the Shepard factors, and with leap-frog the
 * CSPM matrices, inside its first rates and boundary passes instead of a separate
 * correction pass; the factors equal tsg_kernel_corr's bit for bit, and the fields hold
 * them after the step as in the reference. */
int tsg_step(tsg_handle* h, int nsteps, void* stream);

/* Device view of a named particle field in the current (cell-sorted) order.  Replaces
 * attribute access on the reference's `pt` struct field (eng/particle_func.py:10-88).
 * FP32-mixed instances return views of a f64 staging copy refreshed by this call. */
int tsg_field(tsg_handle* h, const char* name, tsg_view* out, void* stream);

/* Number of particles (ParticleSystem.particle_num[None], eng/particle_system.py:39). */
int64_t tsg_particle_num(const tsg_handle* h);

/* Cell offsets after the last sort: out[c] = inclusive end offset of cell c for
 * c < grid_num_total, out[grid_num_total] = n (the trailing out-of-grid bin).  Mirrors
 * grid_particle_num after the prefix sum (eng/particle_system.py:118, :256).  Host copy;
 * synchronises the stream.  FP64 form only (the FP32-mixed form keeps its own cell tables
 * for its real and boundary particle blocks): TSG_E_UNSUPPORTED otherwise. */
int tsg_grid(tsg_handle* h, int32_t* out, void* stream);

/* Neighbour lists in the reference's traversal order (for_all_neighbors,
 * eng/particle_system.py:259-269): counts[i] per particle and the concatenated indices.
 * Host copies; synchronises.  *total receives the number of pairs; list may be NULL to
 * query it; returns TSG_E_CAPACITY when cap is too small. */
int tsg_neighbors(tsg_handle* h, int32_t* counts, int32_t* list, int64_t cap, int64_t* total, void* stream);

/* Shape matching of every dynamic rigid body: centre of mass, A = sum m_V rho (x - cm)
 * (x0 - rest cm)^T, its orthogonal polar factor R, x = cm + R (x0 - rest cm).  Replaces
 * solve_rigid_body / solve_constraints (eng/solver_sph_base.py:472-500); tsg_step calls it
 * after advect_something as SPHBase.step does.  The reference's ti.polar_decompose is
 * replaced by Higham's scaled Newton iteration (orthogonal polar factor, converged to 1e-14).
 * The reaction of the flow on dynamic rigid particles, which the reference scatters without
 * synchronisation (eng/solver_sph_wc.py:70-71), is gathered by each rigid particle in
 * ascending neighbour order inside tsg_one_step.  Dynamic rigid bodies take both forms for
 * WCSPH and the FP64 form for the granular solvers (tsg_upload returns TSG_E_UNSUPPORTED
 * for them in a granular FP32-mixed scene or a batched ensemble); a handle without dynamic
 * rigid bodies returns 0 at once. */
int tsg_solve_rigid_body(tsg_handle* h, void* stream);

/* Density summation: out[i] = sum over the neighbours j != i of particle i (support radius,
 * the reference's traversal) of mass_j W(x_i - x_j), for every particle, in the current
 * particle order (the order of tsg_field views).  out is a device array of n doubles.
 * Replaces WCSPHSolver.calc_density_task summed by for_all_neighbors
 * (eng/solver_sph_wc.py:30-31, eng/particle_system.py:259-269), which the reference
 * defines but never calls from a step; like it, the sum has no self term and dummy
 * particles carry zero mass.  FP64 form: bit-identical to the f64 reference order; FP32-mixed
 * form: compensated f32 sums.  Needs a sorted state (tsg_sort or a step). */
int tsg_density_sum(tsg_handle* h, double* out, void* stream);

/* FP64 diagnostics over flow particles: out[0] total mass, out[1..3] momentum,
 * out[4] kinetic energy, out[5] potential energy (-m g.x), out[6] max |v|,
 * out[7] max x of flow particles (front / runout).  No reference counterpart (the
 * reference prints no conservation figures); synchronises. */
int tsg_reduce_diag(tsg_handle* h, double out[8], void* stream);

/* Neighbour-list occupancy of the FP32-mixed form (TSG_E_UNSUPPORTED for FP64, which
 * traverses cells and keeps no lists): out[0] list entries stored for real particles
 * (pairs within the support plus the skin), out[1] the same for dummy / repulsive
 * particles, out[2] particles whose neighbours exceeded the list capacity (served by
 * direct traversal), out[3] list builds since upload, out[4] dummy / repulsive particles
 * with a non-empty list (the ones the per-step kernel correction and boundary
 * extrapolation visit; the others keep the values written at the list build).
 * No reference counterpart (the reference re-walks the cells in every loop); used for
 * byte accounting and to report the rebuild rate.  Synchronises. */
int tsg_list_stats(tsg_handle* h, int64_t out[5], void* stream);

/* Device error word accumulated since the last call (and cleared).  Synchronises. */
int tsg_last_error(tsg_handle* h, void* stream);

/* Copy one named field between a caller buffer and the device state, in the current
 * (cell-sorted) particle order.  The caller buffer is row-major (n, k) f64 for float fields
 * and int32 for integer fields; host buffers should be pinned for the copies to overlap.
 * Replaces the reference's from_numpy / to_numpy transfers (eng/particle_system.py:289-314,
 * :413-456).  tsg_write with a page-locked host source (FP32-mixed form): the conversion
 * kernel reads it in place, in stream order, so the caller keeps it unchanged until the
 * stream has passed the call (as for an asynchronous copy from pinned memory).
 * tsg_read's to_device: 0 host destination (synchronises the stream), 1 device
 * destination, 2 host destination without synchronising (several reads can then share one
 * synchronisation; the caller synchronises the stream before touching dst). */
int tsg_write(tsg_handle* h, const char* name, const void* src, int from_device, void* stream);
int tsg_read(tsg_handle* h, const char* name, void* dst, int to_device, void* stream);
/* tsg_read of several fields in one call (count <= 8): the FP32-mixed form converts them
 * in one pass over the particle state before the copies. */
int tsg_read_fields(tsg_handle* h, int count, const char* const* names, void* const* dsts, int to_device,
                    void* stream);

/* Number of kernel launches this library has issued since it was loaded (all handles).
 * No reference counterpart: instrumentation for launch accounting. */
int64_t tsg_launch_count(void);

/* Per-phase CUDA-event timing (no reference counterpart; measurement only).  While enabled,
 * every phase's kernels are bracketed by events on their launch stream.  tsg_profile_read
 * synchronises the device, returns the summed milliseconds and bracket counts per phase
 * (0 sort, 1 kernel correction, 2 init_tmp, 3 EOS / stress adaptation, 4 boundary
 * extrapolation, 5 rates, 6 integration, 7 advect_pos, 8 post-step, 9 other, 10 neighbour
 * lists) and clears. */
int tsg_profile(int enable);
int tsg_profile_read(double* ms, int64_t* counts, int nphase);

/* Allocation-free cell-list sort.  No counterpart in the reference: it serves callers
 * that cannot call cudaMalloc - code whose device memory is planned up front by a
 * fixed-budget pool or another framework's allocator, and stepping loops that must not
 * risk the device-wide synchronisation cudaMalloc / cudaFree can cause.  It performs the
 * same stable counting sort as tsg_sort on caller-owned buffers: x is a device array of
 * n positions, row-major (n, 3) f64; the grid comes from cfg (vdomain_start, grid_size,
 * grid_num, grid_num_total).  Outputs, both on the device: cell_start (grid_num_total + 2
 * ints; cell c holds new positions [cell_start[c], cell_start[c + 1]), the last bin holds
 * particles outside the grid) and perm (n ints; new position -> index into x).
 * It allocates nothing: its scratch lives in fixed file-scope device arrays (about 3 MB
 * per GPU, held until the process exits), so n must not exceed TSG_NOALLOC_MAX_PARTICLES
 * and grid_num_total + 1 must not exceed TSG_NOALLOC_MAX_CELLS (else TSG_E_CAPACITY).
 * Every call shares that scratch, so calls that overlap on the GPU race.  The first call
 * on a device looks up the scratch address (once per device, kept for the life of the
 * process, so do not call it again after a cudaDeviceReset); make it before any stream
 * capture begins.  Unlike tsg_sort it raises no status for particles outside the grid or
 * with non-finite positions: they land in the trailing bin in ascending index order, and
 * cell_start[grid_num_total + 1] - cell_start[grid_num_total] counts them. */
#define TSG_NOALLOC_MAX_PARTICLES 262144
#define TSG_NOALLOC_MAX_CELLS 262144
int tsg_sort_noalloc(const tsg_config* cfg, const double* x, int64_t n, int32_t* cell_start, int32_t* perm,
                     void* stream);

/* Launch configuration of the FP32-mixed form.  No reference counterpart (Taichi picks
 * its own launch shapes): threads_per_block of the neighbour-traversal kernels (64, 128,
 * 256); cells_per_cta of the neighbour-list build, one warp per cell (2, 4, 8; 0 = one
 * thread per particle); steps_per_graph, how many steps one captured CUDA graph replays
 * (1..64).  tsg_step runs FP32-mixed steps as graph replays (each step re-sorts inside the
 * graph only when the device-side displacement check asks for it); while tsg_profile is
 * on it runs them eagerly. */
typedef struct tsg_launch_cfg {
    int32_t threads_per_block;
    int32_t cells_per_cta;
    int32_t steps_per_graph;
} tsg_launch_cfg;
int tsg_set_launch(tsg_handle* h, const tsg_launch_cfg* cfg);
int tsg_get_launch(tsg_handle* h, tsg_launch_cfg* cfg);

/* Autotuner (no reference counterpart): times candidate launch configurations from the
 * current state - threads per block over trial_steps full steps, cells per CTA over the
 * re-sort + list build, steps per graph over full steps - keeps the fastest, writes it to
 * *best and the best milliseconds per step to *ms_per_step (either may be NULL), and puts
 * the particle state back as it was (re-sorted), so tuning does not advance the
 * simulation.  Synchronises.  TSG_E_STATE while tsg_profile is on. */
int tsg_autotune(tsg_handle* h, int32_t trial_steps, tsg_launch_cfg* best, double* ms_per_step, void* stream);

/* Batched ensemble: nscenes independent WCSPH scenes stepped together by the same
 * launches (no reference counterpart; the reference runs one scene per process).  Every
 * scene must share dim, kernel, correction, integrator, dummy boundary (2), the FP32-mixed
 * precision, the grid, spacing, dt, density0, exponent and gravity; stiffness and
 * viscosity may differ per scene, particle counts may differ freely.  The scenes are
 * placed side by side along x, scene q shifted by q * tsg_batch_pitch(h) (so fields read
 * through tsg_field / tsg_read carry that shift), with a gap wider than the support
 * radius plus the list skin, so no pair crosses scenes.  Particles are numbered scene by
 * scene in the order given (id0).  parts are host arrays.  The handle then takes every
 * ordinary entry point (tsg_step, tsg_field, tsg_autotune, ...).  At most 4096 scenes. */
int tsg_batch_create(const tsg_config* cfgs, const tsg_particles* parts, int32_t nscenes, void* stream,
                     tsg_handle** out);
/* Per-scene FP64 diagnostics: out[8 * q + k] with k as in tsg_reduce_diag, positions
 * relative to scene q's own origin.  Synchronises. */
int tsg_batch_diag(tsg_handle* h, double* out, int32_t nscenes, void* stream);
/* x shift between consecutive scenes of a batch (0 for an ordinary handle). */
double tsg_batch_pitch(const tsg_handle* h);

/* Granular material parameters of a created handle: friction angle (rad) and cohesion
 * (Pa), with the solver constructor's derived constants recomputed (mu = tan(friction) for
 * mu(I), eng/solver_sph_muI.py:20; alpha, k_c for Drucker-Prager,
 * eng/solver_sph_dp.py:20-27).  No reference counterpart: the reference fixes them at
 * construction; the differentiable rollout perturbs them. */
int tsg_set_soil(tsg_handle* h, double friction, double cohesion);

/* WCSPH fluid parameters of a created handle: Tait stiffness B (Pa) and kinematic
 * viscosity, with the viscosity factor 2 (dim + 2) viscosity recomputed
 * (eng/solver_sph_wc.py:12-28).  No reference counterpart (fixed at construction there);
 * the differentiable WCSPH rollout perturbs them.  Not for batched ensembles. */
int tsg_set_fluid(tsg_handle* h, double stiffness, double viscosity);

/* Bitwise snapshots of the FP32-mixed particle state (every per-particle array that
 * carries from one step to the next, in the current particle order) into / from a device
 * buffer of tsg_snapshot_bytes(h) bytes.  After a load the next step re-sorts first, so
 * stepping on from a loaded snapshot repeats the original steps bit for bit.  No
 * reference counterpart (checkpointing for the adjoint). */
int64_t tsg_snapshot_bytes(tsg_handle* h);
int tsg_snapshot_save(tsg_handle* h, void* dst, void* stream);
int tsg_snapshot_load(tsg_handle* h, const void* src, void* stream);

/* Hand-written adjoint of one FP32-mixed WCSPH or mu(I) step (2D, symplectic Euler, no
 * kernel correction, dummy boundary, no XSPH, not a batched ensemble; no reference
 * counterpart - the reference's Taichi kernels are not differentiated).  Call with the
 * state loaded from the snapshot taken before the step: it repeats the step's forward, then
 * reverses it.  The adjoint arrays are device f64 arrays in particle-id (id0) order,
 * row-major: adj_x, adj_v, adj_v_tmp (n, 3), adj_density (n,).  On entry they hold the
 * adjoint of the state after the step (x, v, density of the fluid / soil particles; for
 * mu(I) also v_tmp of the dummy particles, which the next step reads - WCSPH recomputes it
 * and returns zeros there), on return the adjoint of the state before it.  adj_params
 * (device, 2 doubles) accumulates, for WCSPH, d/d B (Tait stiffness) and d/d nu' (the
 * viscosity factor 2 (dim + 2) viscosity); for mu(I), d/d mu and d/d cohesion
 * (mu = tan(friction)).  TSG_E_CAPACITY if a neighbour list overflowed. */
int tsg_adjoint_step(tsg_handle* h, double* adj_x, double* adj_v, double* adj_density, double* adj_v_tmp,
                     double* adj_params, void* stream);

/* Headless visual buffer (replaces the GUI's inputs; no window or graphics API): per
 * particle the value chosen by color_title (the reference's colour titles: 1 id0,
 * 2 density, 21 d_density, 3 |v|, 31 v.x, 32 -v.y, 33 v.z, 34 |d_vel|, 35-37 d_vel
 * components, 4 |x|, 41-43 x components, 44 |x - x0| (FP64 form), 51-57 stress terms,
 * 61 strain_equ, 62 strain_equ_p, 7 pressure, 8 return-mapping flag, 102 CSPM_L[0][0],
 * 103 |v_tmp|; assign_value_color, eng/solver_sph_base.py:721-785), its range over the flow
 * particles with the given / fixed bounds (v_maxmin, eng/particle_system.py:389-398), the
 * jet colour of the normalised value (set_color, eng/particle_system.py:400-407,
 * eng/colormap.py:8-50) and the position times w2s_ratio (copy2vis,
 * eng/particle_system.py:380-386).  pos and color are device float arrays (n, 3) indexed
 * by particle id (id0); entries the selection leaves out are not written.  range_out (host,
 * may be NULL) receives (max, min).  TSG_E_ARG for an unknown title, TSG_E_UNSUPPORTED when
 * the form does not keep the field (x0 in the FP32-mixed form). */
typedef struct tsg_visual_cfg {
    int32_t color_title;
    int32_t color_group;   /* 0 flow, 1 real, 2 real + shown dummies */
    int32_t show_bdy;
    int32_t fix_max, fix_min;
    double w2s_ratio;
    double given_max, given_min;  /* -1: none */
} tsg_visual_cfg;
int tsg_visual(tsg_handle* h, const tsg_visual_cfg* cfg, float* pos, float* color, double* range_out, void* stream);

/* Human-readable text for a status code. */
const char* tsg_status_string(int status);

void tsg_destroy(tsg_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* TISPHI_GB300_H */
