/*
 * ziran_gb300.h — C ABI of the GB300-native explicit MPM substep.
 *
 * Drop-in boundary for Ziran's explicit MPM path (Lib/MPM over Lib/SPGrid, as driven by
 * Projects/anisofracture). Plain pointers and sizes only. Every call returns an int status
 * (ZR_OK = 0) and never throws; the message of the last failure is available per handle.
 * A handle is used by one host thread at a time; different handles may be driven concurrently
 * (each owns a CUDA stream). Host arrays are owned by the caller and copied; device state lives in
 * HBM for the lifetime of the handle (the reference's Particles own their DataArrays the same way,
 * Lib/Ziran/CS/DataStructure/DataManager.h:67-140).
 *
 * Conventions: positions in metres in the positive octant; 3x3 matrices row-major, 9 values per
 * particle; "first/count" are particle ranges in the order particles were added.
 */
#ifndef ZIRAN_GB300_H
#define ZIRAN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference throws: Debug.h:19-37, RestartException MpmSimulationBase.cpp:1498) ---- */
#define ZR_OK 0
#define ZR_ERR_ARG 1           /* invalid argument */
#define ZR_ERR_CUDA 2          /* CUDA runtime failure or no device */
#define ZR_ERR_CFL 3           /* a particle moved more than one cell; state is left at the start of that substep */
#define ZR_ERR_NONFINITE 4     /* NaN/Inf in the particle state; state is left at the start of that substep */
#define ZR_ERR_OUT_OF_DOMAIN 5 /* a base node left the scene domain; state is left at the start of that substep */
#define ZR_ERR_BUDGET 6        /* request does not fit the serving memory budget */
#define ZR_ERR_TIMEOUT 7       /* a bounded device wait gave up */
#define ZR_ERR_CAPACITY 8      /* active-block table could not grow */
#define ZR_ERR_STATE 9         /* call not valid in the handle's current state */

/* ---- precision of the device state ---- */
#define ZR_F32 4
#define ZR_F64 8

/* ---- constitutive models ---- */
#define ZR_COROTATED 0           /* Physics/ConstitutiveModel/CorotatedElasticity.cpp */
#define ZR_NEOHOOKEAN_BORDEN 1   /* Physics/ConstitutiveModel/NeoHookeanBorden.cpp */
#define ZR_QR_STABLE_NEOHOOKEAN 2 /* Physics/ConstitutiveModel/QRStableNeoHookean.h */

/* ---- collision object types (Math/Geometry/CollisionObject.h:47-50) ---- */
#define ZR_STICKY 1
#define ZR_SLIP 2
#define ZR_SEPARATE 3

/* ---- particle fields ---- */
#define ZR_FIELD_X 0       /* 3 values */
#define ZR_FIELD_V 1       /* 3 */
#define ZR_FIELD_C 2       /* 9, APIC affine matrix */
#define ZR_FIELD_F 3       /* 9, deformation gradient */
#define ZR_FIELD_D 4       /* 1, damage */
#define ZR_FIELD_M 5       /* 1, mass */
#define ZR_FIELD_V0 6      /* 1, initial volume (element measure) */
#define ZR_FIELD_SIGMA_C 7 /* 1, critical stress */
#define ZR_FIELD_DTILDE_MAX 8 /* 1, largest damage drive so far: the implicit damage solve's history
                               * (AnisoFractureSimulation.h:285-340, maxDTilde) */

typedef struct zr_scene zr_scene;
typedef struct zr_batch zr_batch;
typedef struct zr_server zr_server;

/* Simulation knobs: the public members of MpmSimulationBase<T,3> (MpmSimulationBase.h:47-76).
 * dt is the substep size (the reference's step.max_dt when the CFL bound does not bind).
 * domain_cells bounds base-node coordinates to [0, domain_cells) (0 = the full 4096^3 SPGrid). */
typedef struct zr_sim_params {
    double dx;
    double dt;
    double gravity[3];
    double apic_rpic_ratio; /* 1 = APIC, 0 = RPIC (MpmSimulationBase.cpp:39-40) */
    double cfl;             /* default 0.6 (MpmSimulationBase.cpp:46) */
    int32_t domain_cells;
    int32_t reserved;
} zr_sim_params;

/* ======================= scene: one MpmSimulationBase<T,3> / AnisoFractureSimulation ======================= */

/* MpmSimulationBase<T,3>::MpmSimulationBase() (MpmSimulationBase.cpp:36-67); precision ZR_F32 or ZR_F64. */
int zr_scene_create(int precision, zr_scene** out);
int zr_scene_destroy(zr_scene* s);
/* sim.dx / sim.step.max_dt / sim.gravity / sim.apic_rpic_ratio / sim.cfl (MpmSimulationBase.h:47-76). */
int zr_scene_set_params(zr_scene* s, const zr_sim_params* p);
/* MpmInitializationHelper samplers + MpmParticleHandleBase (MpmInitializationHelper.h:114-123,1344-1414,
 * MpmParticleHandleBase.cpp:72-79): adds n particles; v and F may be NULL (zero / identity).
 * *first receives the index of the first added particle. */
int zr_scene_add_particles(zr_scene* s, int64_t n, const double* x, const double* v, const double* m, const double* V0, const double* F,
    int64_t* first);
/* MpmParticleHandleBase::addFBasedMpmForce(CorotatedElasticity(E, nu)) (MpmParticleHandleBase.cpp:132-145). */
int zr_scene_add_corotated(zr_scene* s, int64_t first, int64_t count, double E, double nu);
/* MpmParticleHandleBase::addFBasedMpmForce(NeoHookeanBorden(E, nu)). */
int zr_scene_add_neohookean_borden(zr_scene* s, int64_t first, int64_t count, double E, double nu);
/* MpmParticleHandleBase::addFBasedMpmForce(QRStableNeoHookean(E, nu)) after setExtraFiberStiffness(0, fiber_x)
 * and setExtraFiberStiffness(1, fiber_y) (QRStableNeoHookean.h:98-107): fibre stiffness kx = fiber_x mu
 * along the material x axis (r00 of F = QR) and ky = fiber_y mu; 0 and 0 give the isotropic model. */
int zr_scene_add_qr_stable_neohookean(zr_scene* s, int64_t first, int64_t count, double E, double nu, double fiber_x, double fiber_y);
/* AnisoFractureSimulation's implicit damage (AnisoFractureSimulation.h:343-352 selects solveDamageSystem,
 * :437-626, when implicit is set): after the grid update the nodal phase field is solved with
 * Jacobi-preconditioned conjugate gradients (ConjugateGradient.h: tolerance 1e-6 on sqrt(r.z), at most 100
 * iterations, x0 = 0) and G2P adds the interpolated change to the damage, which never decreases. on = 0
 * restores the explicit update. Must be called before the first substep. */
int zr_scene_set_implicit_damage(zr_scene* s, int on);
/* Conjugate-gradient iterations of the last substep's implicit damage solve (0 without one). */
int zr_scene_cg_iterations(zr_scene* s, int* iterations);
/* MpmParticleHandleBase::addFBasedMpmForceWithAnisotropicPhaseField (MpmParticleHandleBase.cpp:175-222) for a
 * range that already has a Neo-Hookean (Borden) or QR-stable Neo-Hookean model: one structural director a0 = e1 with weight alpha
 * (fibre directions are encoded in the initial F, see zr_rotated_F), length scale l0, viscosity eta,
 * scale zeta, residual stiffness; sigma_crit holds one critical stress per particle of the range. */
int zr_scene_add_aniso_damage(zr_scene* s, int64_t first, int64_t count, double alpha, double l0, double eta, double zeta, double residual,
    const double* sigma_crit);
/* init_helper.addAnalyticCollisionObject(AnalyticCollisionObject(HalfSpace(origin, normal), type)) with a
 * translation b(t) = velocity * t (MpmInitializationHelper.h:1421-1424, CollisionObject.h:144-148). */
int zr_scene_add_halfspace(zr_scene* s, const double origin[3], const double normal[3], int type, double friction, const double velocity[3]);
/* nsteps calls of MpmSimulationBase::advanceOneTimeStep(dt) (MpmSimulationBase.cpp:262-357). On ZR_ERR_CFL,
 * ZR_ERR_NONFINITE or ZR_ERR_OUT_OF_DOMAIN the state is left at the start of the failing substep and
 * *done (may be NULL) tells how many substeps completed. */
int zr_scene_step(zr_scene* s, int nsteps, int* done);
/* Field read/write in the order particles were added; dtype ZR_F32 or ZR_F64 for the host buffer. */
int zr_scene_get_field(zr_scene* s, int field, void* out, int dtype);
int zr_scene_set_field(zr_scene* s, int field, const void* in, int dtype);
/* Whole dynamic state, 25 values per particle: x(3) v(3) C(9) F(9) d(1). */
int zr_scene_get_state(zr_scene* s, void* out, int dtype);
int zr_scene_set_state(zr_scene* s, const void* in, int dtype);
/* get_state into out, then set_state from in, in one call (the two buffers must not overlap). With both buffers
 * in pinned host memory one kernel moves the two directions over the host link at the same time, so a pipeline
 * that streams states through the GPU downloads one result while it uploads the next input. The reference has
 * no counterpart (its state never leaves host memory); it replaces a writeState/readState pair
 * (MpmSimulationBase.cpp:1060-1114) between two scenes that share one device. */
int zr_scene_exchange_state(zr_scene* s, const void* in, void* out, int dtype);
/* nsteps independent jobs through the scene: job i sets the state from in[i] (as zr_scene_set_state), advances one
 * substep and writes the result to out[i] (as zr_scene_get_state); all buffers hold count x 25 values of dtype.
 * out[i] may be in[i], but no output may overlap the input of a later job (ZR_ERR_ARG).
 * The host-to-device copies of the next inputs and the device-to-host copies of the last results run on the copy
 * engines while the GPU computes (pinned buffers give the overlap; the buffers stay in use until the call
 * returns). A job that fails (a substep that aborts, a position outside the domain) is run again as
 * zr_scene_set_state, zr_scene_step and zr_scene_get_state would run it, with the same retries; if it still fails,
 * the error code is returned, the results of the earlier jobs are written, the state is that of the failing job
 * and the later output buffers hold unspecified values. The reference has no counterpart (one scene per process, frames written to files); it serves a
 * pipeline that runs many independent states (ensembles, parameter sweeps, a host-side coupler) through one GPU. */
int zr_scene_step_stream(zr_scene* s, int nsteps, const void* const* in, void* const* out, int dtype);
/* Jobs of zr_scene_step_stream calls that ran again the safe way because a job aborted on the pipelined path
 * (cumulative over the scene's life; 0 while every job ran pipelined). No reference counterpart. */
int zr_scene_stream_reruns(zr_scene* s, int64_t* reruns);
/* FP64-accumulated reductions (MpmSimulationDataAnalysis.h:67-151): total mass, momentum x/y/z, kinetic
 * energy, max particle speed, grid mass of the last substep. */
int zr_scene_reductions(zr_scene* s, double out[7]);
int zr_scene_set_dt(zr_scene* s, double dt);
double zr_scene_time(zr_scene* s);
/* Snapshots (SimulationBase::write/read, SimulationBase.h:149-187, with MpmSimulationBase::writeState/readState,
 * MpmSimulationBase.cpp:1060-1114): a versioned binary image of the dynamic state (header, then x v C F d m V0
 * sigma_c and the damage drive history in the caller's particle order and the scene's precision, so a restore
 * is exact) with the clock and dt. Images of version 1 (without the history) still load, with a zero history. zr_scene_state_bytes gives the image size; load_state needs a scene with the same precision and particle
 * count (built the same way, as the reference re-runs its scene set-up before readState). */
int64_t zr_scene_state_bytes(zr_scene* s);
int zr_scene_save_state(zr_scene* s, void* buf, int64_t bytes);
int zr_scene_load_state(zr_scene* s, const void* buf, int64_t bytes);
int zr_scene_write_state_file(zr_scene* s, const char* path);
int zr_scene_read_state_file(zr_scene* s, const char* path);
/* Frame output for visualisation (writePartio, Lib/Ziran/Math/Geometry/PartioIO.h:166-210, called from
 * MpmSimulationBase::writeState, MpmSimulationBase.cpp:1067-1080; AnisoFractureSimulation::writeState,
 * Projects/anisofracture/AnisoFractureSimulation.h:73-100, through aniso_visualize_particles_vec,
 * AnisoVisualizer.h:36-64): a Houdini classic binary geometry file (.bgeo, format version 5, the layout partio
 * writes) with one point per particle in the caller's order, its position, and the attributes the flags select,
 * all as 32-bit floats of the vector type: ZR_BGEO_V "v" (3), ZR_BGEO_D "d" (1, damage), ZR_BGEO_A1 "a_1"
 * (3, the current fibre director R e1, R the rotation of F's polar decomposition; the fibre of F0 from
 * initializeRotatedFHelper is its first column). flags = 0 writes positions only, as writePartio does. The
 * reference's "laplacian" attribute is not written: the substep does not keep it. */
#define ZR_BGEO_V 1
#define ZR_BGEO_D 2
#define ZR_BGEO_A1 4
int zr_scene_write_bgeo(zr_scene* s, const char* path, int flags);
/* The file writer alone, for host arrays: n points at x (3n doubles), nattr attributes, attribute k named
 * names[k] with sizes[k] components per point at data[k] (sizes[k] * n doubles). Values are stored as floats. */
int zr_write_bgeo(const char* path, int64_t n, const double* x, int nattr, const char* const* names, const int32_t* sizes, const double* const* data);
/* Advance whole frames the way SimulationBase::simulate does (SimulationBase.h:275-354): substeps from
 * TimeStepping::nextDt (TimeStepping.h:45-59) between min_dt and the scene's dt (max_dt), hitting every frame
 * boundary exactly; with cfl_dt != 0 the wanted substep is cfl dx / max particle speed (calculateDt,
 * MpmSimulationBase.cpp:1128-1151). A substep that moves a particle more than a cell restarts the frame from
 * its start with max_dt halved (the autorestart of MpmSimulationBase.cpp:1480-1510); *restarts counts them.
 * max_dt stays shrunk for later calls, as step.max_dt does. ZR_ERR_CFL if max_dt is already at min_dt. */
int zr_scene_advance_frames(zr_scene* s, int frames, double frame_dt, double min_dt, int cfl_dt, int* restarts);
int64_t zr_scene_count(zr_scene* s);
const char* zr_scene_last_error(zr_scene* s);
/* device time (ms) of the substeps of the last zr_scene_step call: CUDA events on the scene's stream */
double zr_scene_last_step_ms(zr_scene* s);
/* largest number of particle groups (occupied SPGrid blocks) and active blocks seen in the last zr_scene_step */
int zr_scene_last_grid(zr_scene* s, int64_t* n_groups, int64_t* n_blocks);
/* Binning of the current positions (MpmSimulationBase::sortParticlesAndPolluteGrid,
 * MpmSimulationBase.cpp:1531-1573, MpmGrid::pollute MpmGrid.h:153-193): the sorted 64-bit keys in the
 * reference's layout (n), the sorted particle order (n), the first sorted index of every particle group
 * (*n_groups, at most n) and the active SPGrid pages in ascending order (*n_pages, at most 8n). */
int zr_scene_binning(zr_scene* s, uint64_t* sorted_keys, int32_t* order, int32_t* group_first, int64_t* n_groups, uint64_t* pages,
    int64_t* n_pages);
/* Per-phase device time (ms) of substeps run while timing is enabled: sort+groups, activate, p2g, grid,
 * g2p; and the number of timed substeps. Timing runs the substeps without CUDA graphs. */
int zr_scene_set_timing(zr_scene* s, int on);
int zr_scene_get_timing(zr_scene* s, double out5[5], int64_t* steps);
/* Launch schedule of the substep: the P2G form (fused: one kernel that evaluates the stress; split: a
 * stress kernel writing a per-particle payload that a scatter kernel streams into shared memory with bulk
 * asynchronous copies), the particles staged per P2G chunk and the staging buffers of the split form, the
 * P2G CTAs per SM and the G2P threads per CTA (particles per warp pass over a block). No reference
 * counterpart: Ziran's CPU loops are scheduled by TBB (MpmSimulationBase.cpp:669-855, 1269-1515).
 * mode 0 = a fixed default schedule, 1 = autotuned: measured with trial substeps on the scene's own state
 * when it first steps (the trials are rolled back) and cached per workload class in the process,
 * 2 = autotuned, re-measured per batch. Schedules differ only in the order of floating-point sums.
 * get: out7 = fused, chunk, buffers, CTAs per SM, G2P threads, G2P register cut, 1 if measured.
 * set: in6 = fused (0 split, 1 fused, 2 fused with registers cut for one more CTA per SM),
 * (chunk, buffers) one of (512, 1), (512, 2), (256, 2) in FP32 or (256, 1), (256, 2), (128, 2) in FP64
 * (ignored when fused), CTAs per SM, G2P threads (64, 128 or 256), G2P register cut (0 or 1: more
 * resident threads per SM); an explicit schedule disables the autotuner for the scene. */
int zr_scene_set_autotune(zr_scene* s, int mode);
int zr_scene_set_schedule(zr_scene* s, const int32_t in6[6]);
int zr_scene_get_schedule(zr_scene* s, int32_t out7[7]);
/* kernels launched per substep (CUDA-graph node count) and device bytes held by the scene. */
int zr_scene_stats(zr_scene* s, int64_t* launches_per_step, int64_t* device_bytes, int64_t* fallbacks);

/* ================================ scene recipes (seeded synthetic scenes) ================================ */
#define ZR_RECIPE_ELASTIC_BOX 0 /* falling corotated cube over a sticky ground plane */
#define ZR_RECIPE_ANISO_SLAB 1  /* Neo-Hookean slab with vMF fibres and anisotropic damage, ends pulled apart */

typedef struct zr_scene_recipe {
    int32_t kind;
    int32_t ppc_side;     /* particles per cell = ppc_side^3 (2 -> 8) */
    uint64_t seed;
    double dx, dt;
    double size[3];       /* extents in metres, snapped to whole cells */
    double center[3];
    double velocity[3];   /* initial velocity */
    double gravity[3];
    double E, nu, rho;
    double apic_rpic_ratio;
    double ground_y;      /* ELASTIC_BOX: sticky half-space y <= ground_y */
    double kappa_vmf;     /* ANISO_SLAB: von Mises-Fisher concentration of fibres about +x */
    double alpha, l0, eta, zeta, residual;
    double sigma_c_mean, sigma_c_std;
    double pull_speed;    /* ANISO_SLAB: the two x ends move apart at +-pull_speed */
    double grip_cells;    /* ANISO_SLAB: width of each sticky end plate in cells */
    int32_t domain_cells; /* 0 = round(1/dx) + 4 (the unit box) */
    int32_t model;        /* ANISO_SLAB: 0 or ZR_NEOHOOKEAN_BORDEN (default), or ZR_QR_STABLE_NEOHOOKEAN */
    double fiber_stiffness; /* ANISO_SLAB with ZR_QR_STABLE_NEOHOOKEAN: kx in units of mu (setExtraFiberStiffness(0, .)) */
    int32_t implicit_damage; /* ANISO_SLAB: 1 = implicit damage solve (zr_scene_set_implicit_damage) */
    int32_t reserved2;
} zr_scene_recipe;

/* Defaults: ELASTIC_BOX = unit box, dx 1/64, cube side 0.25 at (0.5,0.6,0.5), 8 ppc, corotated E=1e4
 * nu=0.3 rho=1000, v0=(0,-1,0), gravity -9.8, ground y=0.05, dt=1e-4, APIC. ANISO_SLAB = dx 1/128,
 * 0.5x0.1x0.5 slab at (0.5,0.5,0.5), 8 ppc, Neo-Hookean E=5e4 nu=0.25 rho=800, kappa=20, alpha=-1,
 * l0=0.5dx, eta=0.1, zeta=1, k=0.01, sigma_c ~ N(400,40), ends pulled at 0.5 m/s, dt=5e-5, RPIC. */
int zr_recipe_default(int kind, zr_scene_recipe* out);
/* number of particles the recipe generates */
int64_t zr_recipe_count(const zr_scene_recipe* r);
/* Generate the recipe's particles into caller arrays (any may be NULL): x(3n) v(3n) m(n) V0(n) F(9n) sigma_c(n). */
int zr_recipe_generate(const zr_scene_recipe* r, double* x, double* v, double* m, double* V0, double* F, double* sigma_c);
/* Build a whole scene (params, particles, materials, damage, collision objects) from a recipe. */
int zr_scene_from_recipe(zr_scene* s, const zr_scene_recipe* r);
/* MpmParticleHandleBase::initializeRotatedFHelper (MpmParticleHandleBase.cpp:224-268) for one unit director. */
void zr_rotated_F(const double a0[3], double F[9]);
/* NeoHookeanBorden::getSigmaCrit(percentage) (NeoHookeanBorden.cpp:38-44): psi at F = (1+p) I. */
double zr_nhb_sigma_crit(double E, double nu, double percentage);
/* QRStableNeoHookean::getSigmaCrit(percentage) (QRStableNeoHookean.h:68-84): psi at F = (1+p) I of the
 * undegraded isotropic model. */
double zr_qrnh_sigma_crit(double E, double nu, double percentage);

/* ================================ batch: many scenes, one launch per kernel ================================ */
int zr_batch_create(int precision, zr_batch** out);
int zr_batch_destroy(zr_batch* b);
/* Copies the scene's current description into the batch (the scene handle stays usable). *slot receives
 * its index in the batch. Scenes must be added before zr_batch_commit. */
int zr_batch_add_scene(zr_batch* b, zr_scene* s, int* slot);
int zr_batch_add_recipe(zr_batch* b, const zr_scene_recipe* r, int* slot);
int zr_batch_commit(zr_batch* b);
int zr_batch_step(zr_batch* b, int nsteps, int* done);
int zr_batch_get_field(zr_batch* b, int slot, int field, void* out, int dtype);
int zr_batch_reductions(zr_batch* b, int slot, double out[7]);
int64_t zr_batch_count(zr_batch* b, int slot);
int zr_batch_set_timing(zr_batch* b, int on);
int zr_batch_set_autotune(zr_batch* b, int mode);
int zr_batch_get_schedule(zr_batch* b, int32_t out7[7]);
int zr_batch_get_timing(zr_batch* b, double out5[5], int64_t* steps);
int zr_batch_stats(zr_batch* b, int64_t* launches_per_step, int64_t* device_bytes, int64_t* fallbacks);
const char* zr_batch_last_error(zr_batch* b);
double zr_batch_last_step_ms(zr_batch* b);

/* ================================ serving loop: continuous batching of requests ================================
 * A request is a scene (a recipe or a built scene description) and a number of substeps. zr_server_tick
 * admits queued requests in arrival order while the device-memory budget and max_scenes allow, re-forms
 * the batch (resident scenes keep their state on the device), advances every resident scene by
 * min(tick_substeps, fewest remaining substeps) in one batched substep sequence and retires finished
 * requests (their final x, v, C, F, d are copied to the host). No counterpart in the reference, whose
 * driver runs one scene per process (Projects/anisofracture/anisofracture.cpp:25-139). */
int zr_server_create(int precision, double budget_bytes, int tick_substeps, int max_scenes, zr_server** out);
int zr_server_destroy(zr_server* sv);
int zr_server_submit_recipe(zr_server* sv, const zr_scene_recipe* r, int substeps, int64_t* id);
/* takes the particles of a scene that has not stepped (the scene handle is left empty) */
int zr_server_submit_scene(zr_server* sv, zr_scene* s, int substeps, int64_t* id);
/* *running / *queued: requests resident / waiting after the tick; *finished: requests completed by it */
int zr_server_tick(zr_server* sv, int* running, int* queued, int* finished);
/* state: 0 queued, 1 running, 2 done, 3 failed; latency (s) is submit -> completion, -1 before completion */
int zr_server_request(zr_server* sv, int64_t id, int* state, double* latency_s, int64_t* particles, int* substeps);
/* final field of a finished request (x, v, C, F or d) in the request's particle order */
int zr_server_result(zr_server* sv, int64_t id, int field, void* out, int dtype);
int zr_server_release(zr_server* sv, int64_t id);
/* particle-substeps advanced, device time of the batched substeps (ms), device bytes held */
int zr_server_stats(zr_server* sv, double* particle_substeps, double* device_ms, int64_t* device_bytes);
const char* zr_server_last_error(zr_server* sv);

/* ============================== binning into caller memory, no device allocation ==============================
 * No counterpart in the reference: it is the binning of MpmSimulationBase::sortParticlesAndPolluteGrid
 * (MpmSimulationBase.cpp:1531-1573) offered to callers that may not allocate device memory while they
 * run (a host that reserves one arena at start-up and forbids cudaMalloc afterwards, a loop with a fixed
 * memory budget, a callback inside another runtime whose device memory is accounted by that runtime).
 * Inputs and outputs are device pointers owned by the caller: x holds n*3 coordinates of the precision's
 * type (xyz per particle); sorted_keys receives the n keys in the reference's layout in ascending order,
 * order the n original indices in that order, group_first the first sorted index of every SPGrid block
 * (capacity n); *n_groups (host) the number of blocks. All scratch lives in one static device array of
 * ZR_NOALLOC_SCRATCH_BYTES per GPU, held until the process exits; n above ZR_NOALLOC_MAX_PARTICLES is
 * rejected with ZR_ERR_ARG. The first call on a device resolves that array's address and sizes the
 * sort (no allocation): make it before any stream capture. The first call of each precision also loads
 * that precision's kernels (lazy module loading), so a caller that must see no device memory change during
 * its run makes one warm-up call per precision at start-up. Calls must use the device's primary context
 * (the runtime API's context). Calls share the array, so calls that overlap on the GPU (different streams
 * or threads) race; serialise them. Returns ZR_ERR_OUT_OF_DOMAIN when a base node lies outside
 * [0, domain_cells) (0 = the full SPGrid range). The call synchronises `stream` before it returns. */
#define ZR_NOALLOC_MAX_PARTICLES (1 << 20)
#define ZR_NOALLOC_SCRATCH_BYTES (16u << 20)
int zr_bin_device_noalloc(int precision, int64_t n, const void* x, double dx, int32_t domain_cells, uint64_t* sorted_keys, int32_t* order,
    int32_t* group_first, int64_t* n_groups, void* stream);

/* library version string */
const char* zr_version(void);

#ifdef __cplusplus
}
#endif
#endif
