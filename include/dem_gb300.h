/*
 * dem_gb300.h -- C ABI of the GB300 DEM step engine.
 *
 * The engine replaces the GPU hot path that the reference program reaches
 * through `class CudaDemSolver` (include/cuda_backend.h:40-72 in the
 * reference).  Every entry point below names the member function or free
 * function it stands in for.  All functions return DEM_OK (0) on success and
 * a nonzero dem_status otherwise; the message of the last failure on the
 * calling thread is returned by dem_last_error().  No entry point throws.
 *
 * Arrays are plain host pointers in the reference's own units and orders:
 * owners (particles) in input-file order, bodies and triangles in
 * CouplePolyFileName.csv order, vectors as consecutive xyz triples and
 * quaternions as (w, x, y, z).
 */
#ifndef DEM_GB300_H
#define DEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEM_GB300_ABI_VERSION 1

/* Capacity constants of the reference (src/cuda/cuda_contact_backend.cuh:11-16). */
#define DEM_PARTICLE_HISTORY_SLOTS 64
#define DEM_WALL_HISTORY_SLOTS 16
#define DEM_BODY_HISTORY_SLOTS 64
#define DEM_BODY_REGIME_COUNTERS 7
#define DEM_BODY_MICROSTATE_VALUES 22

typedef enum dem_status {
    DEM_OK = 0,
    DEM_ERR_INVALID = 1,   /* bad argument or scene */
    DEM_ERR_CUDA = 2,      /* CUDA runtime error */
    DEM_ERR_STATE = 3,     /* call out of order (not initialized, ...) */
    DEM_ERR_CAPACITY = 4,  /* history / grid capacity exceeded */
    DEM_ERR_IO = 5,        /* checkpoint file error */
    DEM_ERR_NO_DEVICE = 6  /* no CUDA device */
} dem_status;

typedef enum dem_precision {
    DEM_PRECISION_FP64 = 0,  /* the reference's all-FP64 method */
    DEM_PRECISION_MIXED = 1  /* FP32 per-contact law + FP32 history; FP64 state */
} dem_precision;

/* Contact material, one per contact class.  Mirrors the fields of the
 * reference's MECH that the GPU path reads (include/simulation.h:48-64,
 * routed at src/cuda_backend_cuda.cu:345-377). */
typedef struct dem_mech {
    double epsS, mu, epsN, cohesion, beta, muT, muR, kN;
} dem_mech;

/* One scene: the data the reference's initialize() takes from PARTICLE,
 * BODYSET, CONTROL, MECH x3 and ODE (src/cuda_backend_cuda.cu:302-381). */
typedef struct dem_scene {
    int n_owners;
    const int* owner_id;          /* stable particle id (Particles.bt col 1) */
    const int* owner_status;      /* -1 = fixed (Particles.bt col 2) */
    const double* owner_mass;
    const double* owner_radius;
    const double* owner_inertia;  /* [n][3] principal inertia */
    const double* owner_pos;      /* [n][3] */
    const double* owner_vel;      /* [n][3] */
    const double* owner_omega;    /* [n][3] body-frame angular velocity */
    const double* owner_quat;     /* [n][4] */

    /* Clump components; n_components == 0 means one sphere per owner. */
    int n_components;
    const int* comp_owner;        /* owner row */
    const int* comp_id;           /* stable component id */
    const double* comp_radius;
    const double* comp_offset;    /* [nc][3] body-frame offset */

    int n_walls;
    const double* wall_origin;    /* [nw][3] */
    const double* wall_normal;    /* [nw][3] points into the domain */

    int n_bodies;
    const double* body_mass;
    const double* body_center;    /* [nb][3] initial mass centre */
    const double* body_quat;      /* [nb][4] */
    const double* body_vel;       /* [nb][3] */
    const double* body_omega;     /* [nb][3] body-frame */
    const double* body_inertia;   /* [nb][9] row-major */
    const int* body_state;        /* 0 dynamic, 1 fixed, 2 prescribed */

    int n_triangles;
    const int* tri_body;          /* owning body row */
    const double* tri_local;      /* [nt][15]: v1, v2, v3, v4, normal (body frame) */

    dem_mech pp, pt, pw;          /* particle-particle, -triangle, -wall */
    double dt;
    double gravity[3];
    int gravity_enabled;
    int universal_gravity_enabled;
    int keep_body_particle;       /* allocate [nb][n][6] body->particle output */
    int keep_body_detail;         /* allocate [nb][n][19] contact detail output */
} dem_scene;

/* Engine options (no counterpart in the reference, which has fixed 256-thread
 * launches and meshSize = 2.5 r_max). */
typedef struct dem_options {
    int precision;           /* dem_precision */
    double cell_factor;      /* cell edge / r_max; >= 2.0; 2.5 = reference */
    int max_cells;           /* dense cell-table capacity, 0 = automatic */
    int block_size;          /* threads per block of the contact kernels, 0 = 128 */
    int pt_fp32;             /* mixed form only: particle-triangle law, area and
                                history in FP32 too (default 0: FP64, since
                                they alone make the body loads) */
} dem_options;

/* Per-step body state uploaded by compute_forces (the 13 doubles per body
 * of src/cuda_backend_cuda.cu:205-227). */
typedef struct dem_body_states {
    const double* center;  /* [nb][3] */
    const double* quat;    /* [nb][4] */
    const double* vel;     /* [nb][3] */
    const double* omega;   /* [nb][3] body-frame */
} dem_body_states;

/* Scalar part of CudaStepStats (include/cuda_backend.h:17-37). */
typedef struct dem_step_stats {
    int particle_contacts;
    int body_contacts;
    double body_max_depth;
    double body_contact_fz;
    int particle_history_overflows;
    int body_history_overflows;
    int particle_history_high_water;
    int body_history_high_water;
    int triangle_grid_overflows;
    int cell_table_overflows;      /* engine-only: dense cell table capacity */
    uint64_t body_regime_interval_native_steps;
    int body_candidate_items;      /* engine-only: (particle, cell) items that the
                                      FP32 particle-triangle probe passed */
    int wall_candidates;           /* engine-only: particle-wall pairs that the
                                      FP32 plane test passed */
} dem_step_stats;

typedef struct dem_engine dem_engine;

/* Version of this header the library was built from. */
int dem_abi_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* dem_last_error(void);

/* CudaBackendAvailable() (src/cuda_backend_cuda.cu:906-910). */
int dem_device_available(void);

/* CudaDeviceDescription() (src/cuda_backend_cuda.cu:912-927). */
const char* dem_device_description(void);

/* CudaDemSolver::CudaDemSolver / ~CudaDemSolver (include/cuda_backend.h:43-44). */
int dem_create(dem_engine** out);
int dem_destroy(dem_engine* engine);

/* Defaults: FP64, cell_factor 2.5, automatic capacities. */
void dem_default_options(dem_options* options);

/* CudaDemSolver::initialize (src/cuda_backend_cuda.cu:302-381).  `options`
 * may be NULL.  An engine (one scene or a whole batch) takes at most
 * 33,554,431 components, because the contact slots are indexed by int;
 * beyond that it returns DEM_ERR_CAPACITY. */
int dem_initialize(dem_engine* engine, const dem_scene* scene,
                   const dem_options* options);

/* Batched form: n_scenes independent scenes advance together.  Scenes never
 * interact; each keeps its own walls, bodies and materials.  Owners, bodies
 * and triangles are numbered by concatenation in scene order.  No
 * counterpart in the reference (which is one scene per process). */
int dem_initialize_batch(dem_engine* engine, const dem_scene* scenes,
                         int n_scenes, const dem_options* options);

/* CudaDemSolver::computeForces (src/cuda_backend_cuda.cu:383-524).
 * `bodies` may be NULL (pure DEM or unchanged bodies); `body_forces`, if not
 * NULL, receives [nb][6] contact loads plus m_b*g as in the reference.
 * With collect_diagnostics != 0 the counters are downloaded and capacity
 * overflows are reported as DEM_ERR_CAPACITY. */
int dem_compute_forces(dem_engine* engine, double time,
                       const dem_body_states* bodies, double* body_forces,
                       int collect_diagnostics);

/* CudaDemSolver::initializeParticleHalfStep (src/cuda_backend_cuda.cu:526-529). */
int dem_leapfrog_init(dem_engine* engine, double half_dt);
/* CudaDemSolver::advanceParticles (src/cuda_backend_cuda.cu:531-538). */
int dem_leapfrog_advance(dem_engine* engine, double dt);
/* CudaDemSolver::finishParticleStep (src/cuda_backend_cuda.cu:540-543). */
int dem_leapfrog_finish(dem_engine* engine, double dt, double half_dt);

/* Whole integration loop of the reference's IntegrateDem /
 * IntegrateDemMultiBody (src/cuda_simulation_integrator.cpp:245-446) for
 * `steps` steps, host MBD step included, with no output frames.  The first
 * call performs the step-0 force evaluation and the half-step start.  The
 * last step's half-step quaternion rate is computed by the next call: a
 * following dem_run_steps takes it into its first advance, and every other
 * call that reads, replaces or steps the particle state completes it first,
 * so every call sees the reference's state after the last step. */
int dem_run_steps(dem_engine* engine, int steps);

/* Body state kept by dem_run_steps (host MBD): [nb][3] / [nb][4] arrays,
 * any pointer may be NULL.  Loads are the last contact loads plus m_b*g. */
int dem_get_bodies(dem_engine* engine, double* center, double* quat,
                   double* vel, double* omega, double* loads);

/* CudaDemSolver::saveContactHistory / loadContactHistory /
 * hasRestoredParticleLeapfrogState (src/cuda_backend_cuda.cu:545-827),
 * DMHIST2 format. */
int dem_save_history(dem_engine* engine, const char* path);
int dem_load_history(dem_engine* engine, const char* path);
int dem_has_restored_leapfrog_state(dem_engine* engine, int* restored);

/* CudaDemSolver::downloadParticleState (src/cuda_backend_cuda.cu:829-846).
 * Any pointer may be NULL. */
int dem_download_state(dem_engine* engine, double* pos, double* vel,
                       double* omega, double* quat);

/* CudaDemSolver::downloadForceOutput (src/cuda_backend_cuda.cu:848-892):
 * [n][6] contact, field, wall, total; [nb][n][6] body_particle and
 * [nb][n][19] body_detail when kept.  Any pointer may be NULL. */
int dem_download_forces(dem_engine* engine, double* contact, double* field,
                        double* wall, double* total, double* body_particle,
                        double* body_detail);

/* CudaDemSolver::stepStats (src/cuda_backend_cuda.cu:894): counters of the
 * last compute_forces call that collected diagnostics. */
int dem_stats(dem_engine* engine, dem_step_stats* stats);

/* Per-body regime counters [nb][7] and microstate sums [nb][22]
 * (CudaStepStats::bodyRegime* / bodyMicrostate*).  Any pointer may be NULL. */
int dem_body_diagnostics(dem_engine* engine, uint64_t* regime_instant,
                         uint64_t* regime_interval, double* micro_instant,
                         double* micro_interval);

/* particleGridEntryCount / triangleGridEntryCount / deviceMemoryBytes
 * (src/cuda_backend_cuda.cu:895-904). */
int dem_grid_entry_counts(dem_engine* engine, size_t* particle_entries,
                          size_t* triangle_entries);
int dem_device_memory_bytes(dem_engine* engine, size_t* bytes);

/* Counts of the initialized scene. */
int dem_counts(dem_engine* engine, int* n_owners, int* n_components,
               int* n_bodies, int* n_triangles, int* n_walls);

/* Parity introspection.  The sorted cell keys and entity ids of the last
 * force evaluation, equal to the reference's GpuGridArrays after
 * gpuBuildComponentGrid (src/cuda/cuda_grid_backend.cu:121-145). */
int dem_download_grid(dem_engine* engine, uint64_t* sorted_key,
                      int* sorted_id);

/* Contact history in the reference's slot layout
 * (GpuContactHistory, src/cuda/cuda_contact_backend.cuh:41-52):
 * kind 0 particle [nc][64], 1 wall [nc][16], 2 body [nc][64];
 * keys, last-seen step and 9 values per slot.  Any pointer may be NULL. */
int dem_download_history(dem_engine* engine, int kind, uint64_t* keys,
                         int* last_seen, double* values);

/* Time the pipeline phases of one force evaluation with CUDA events
 * (milliseconds, any pointer NULL).  No counterpart in the reference. */
int dem_last_phase_times(dem_engine* engine, float* ms, int capacity,
                         int* count);

/* Limits of dem_cell_sort_static's built-in working memory. */
#define DEM_STATIC_SORT_MAX_COMPONENTS 262144
#define DEM_STATIC_SORT_MAX_CELLS 1048576

/* The cell sort without any device allocation.  No counterpart in the
 * reference: it serves callers that may not call cudaMalloc where they need
 * the sort (device memory owned by another pool or arena, allocation-free
 * real-time loops, an exhausted memory quota).  Same result as the engine's
 * grid build and the reference's sortedCellKey / sortedEntityId: cell keys
 * packCell(floor(p / mesh_size)) of the n positions, sorted stably over the
 * input order.  x, y, z, sorted_key[n] and sorted_id[n] are DEVICE buffers
 * owned by the caller; stream is a cudaStream_t (NULL = default stream).
 * The call waits for that stream to finish the work and reads its error
 * word back before it returns.  Inside a cell the members are ranked by
 * counting the members with a smaller index, so a cell of m members costs
 * O(m^2) work (every component in one cell: n^2 compares).
 * Working memory is one built-in device array of about 14 MB that every GPU
 * loading this library keeps until the process exits; n is limited to
 * DEM_STATIC_SORT_MAX_COMPONENTS and the occupied cell box to
 * DEM_STATIC_SORT_MAX_CELLS cells (DEM_ERR_CAPACITY beyond).  The first call
 * on a device looks up that array's device address and should come before
 * any stream capture on that device.  All calls share the array, so calls
 * that overlap on the GPU race: order them on one stream or synchronize. */
int dem_cell_sort_static(const double* x, const double* y, const double* z,
                         int n, double mesh_size, uint64_t* sorted_key,
                         int* sorted_id, void* stream);

/* ---- reverse mode (the shape a torch.autograd.Function wraps) ----------
 * No counterpart in the reference, which has no gradients.  A hand-written
 * adjoint of each step of the FP64 form: within a step the contact set is
 * the one the forward step found, and at the Coulomb / twisting / rolling
 * caps the derivative is that of the branch taken.  Covers spheres (any
 * principal inertia) with walls, particle contacts and rigid bodies (particle-triangle manifolds
 * and the host MBD step of dynamic bodies; prescribed and fixed bodies carry
 * no adjoint), one scene or a batch (dem_initialize_batch), precision
 * DEM_PRECISION_FP64; other engines return DEM_ERR_INVALID.
 *
 * dem_adjoint_forward runs the reference's step sequence from a freshly
 * initialized engine: the first evaluation (dt = 0), the leapfrog start and
 * `steps` steps, keeping a checkpoint every `checkpoint_every` steps.
 *
 * dem_adjoint_backward takes the adjoint of a scalar loss with respect to
 * the final positions and velocities ([n][3] each, owner order; either may
 * be NULL for zero) and returns its gradient with respect to the initial
 * positions, velocities and angular velocities ([n][3]; NULL to skip) and
 * to the materials (dl_dparams[scenes][3][6]: per scene of the engine,
 * particle-particle, particle-wall, then particle-triangle, each d/dkN,
 * d/dmu, d/depsN, d/depsS, d/dmuT, d/dmuR; scenes is 1 for dem_initialize).
 * It recomputes each segment from its checkpoint and leaves the engine at
 * the end of the forward run.
 *
 * dem_adjoint_backward_mbd adds the loss's adjoint with respect to the
 * dynamic bodies' final centres and velocities ([nb][3] each, the pose of
 * the last force evaluation; either may be NULL). */
int dem_adjoint_forward(dem_engine* e, int steps, int checkpoint_every);
int dem_adjoint_backward(dem_engine* e, const double* dl_dpos, const double* dl_dvel,
                         double* dl_dpos0, double* dl_dvel0, double* dl_domega0,
                         double* dl_dparams);
int dem_adjoint_backward_mbd(dem_engine* e, const double* dl_dpos, const double* dl_dvel,
                             const double* dl_dbody_center, const double* dl_dbody_vel,
                             double* dl_dpos0, double* dl_dvel0, double* dl_domega0,
                             double* dl_dparams);
/* The last backward run's gradient with respect to the rigid bodies'
 * initial state: centres and velocities [nb][3], orientations [nb][4]
 * (w, x, y, z; the component along q is the normalisation's null direction)
 * and body-frame spins [nb][3].  Dynamic bodies only; prescribed and fixed
 * bodies read zero.  Any pointer may be NULL.  DEM_ERR_STATE before a
 * backward run.  No counterpart in the reference. */
int dem_adjoint_body_gradients(dem_engine* e, double* dl_dbody_center0, double* dl_dbody_quat0,
                               double* dl_dbody_vel0, double* dl_dbody_omega0);

#ifdef __cplusplus
}
#endif

#endif /* DEM_GB300_H */
