// Host-side interface of the GB300 explicit-MPM engine. Plain C++ (no CUDA types), so the C-ABI layer
// and the serving loop can be compiled without nvcc.
//
// One Engine<T> owns the device state of a batch of independent scenes: a particle pool in HBM
// (structure of arrays, two copies that alternate every substep), the sort buffers, the active-block
// table and the sparse grid. A single scene is a batch of one.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace zr {

// host description of one scene (all arrays in the caller's particle order, float64)
struct SceneDesc {
    double dx = 1.0 / 64;
    double dt = 1e-4;
    double gravity[3] = { 0, 0, 0 };
    double apic_rpic_ratio = 1.0; // 1 = APIC, 0 = RPIC (MpmSimulationBase.cpp:39-40)
    double cfl = 0.6;
    double time = 0;
    int implicit_damage = 0; // solve the damage implicitly (AnisoFractureSimulation.h:437-626) instead of the explicit update
    int32_t domain_cells = 0; // base nodes must stay in [0, domain_cells); 0 = the full 4096^3 SPGrid range
    struct Mat {
        int model = 0; // 0 fixed corotated, 1 Neo-Hookean (Borden), 2 QR-stable Neo-Hookean
        double E = 1e4, nu = 0.3;
        double kx_scale = 0, ky_scale = 0; // QR-stable Neo-Hookean fibre stiffness, in units of mu
        int damage = 0;
        double alpha = 0, l0 = 0, eta = 1, zeta = 1, residual = 0;
    };
    struct Obj {
        double origin[3] = { 0, 0, 0 }, normal[3] = { 0, 1, 0 }, vel[3] = { 0, 0, 0 };
        double friction = 0;
        int type = 1; // 1 STICKY, 2 SLIP, 3 SEPARATE
    };
    std::vector<Mat> materials;
    std::vector<Obj> objects;
    int64_t n = 0;
    std::vector<double> x, v, C, F, m, V0, d, sigma_c; // C, F row-major 3x3 per particle
    std::vector<double> dtilde_max; // implicit damage: the damage drive history max D~ (empty = 0)
    std::vector<uint8_t> material; // per particle material index (empty = all 0)
};

enum Field : int {
    FIELD_X = 0, // 3
    FIELD_V = 1, // 3
    FIELD_C = 2, // 9
    FIELD_F = 3, // 9
    FIELD_D = 4, // 1 damage
    FIELD_M = 5, // 1 mass
    FIELD_V0 = 6, // 1 initial volume
    FIELD_SIGMA_C = 7, // 1 critical stress
    FIELD_DTILDE_MAX = 8, // 1 largest damage drive so far (the implicit damage solve's history)
};

struct StepReport {
    double device_ms = 0; // device time of the substeps, CUDA events on the engine's stream
    uint32_t flags = 0;
    int32_t steps_done = 0;
    uint32_t n_groups = 0, n_blocks = 0, fallback = 0;
};

// Launch schedule of the substep (what the autotuner picks). None of these changes the arithmetic beyond
// the order of floating-point sums.
struct Schedule {
    int fused = 0; // P2G: 1 = one kernel evaluating the stress itself, 2 = the same with registers cut for one more
                   // CTA per SM, 3 = the same split into producer warps (state loads, stress, payload) and consumer
                   // warps (accumulation) working on alternating shared-memory buffers; 0 = a stress kernel writing a
                   // payload that a scatter kernel streams into shared memory with bulk asynchronous copies
    int chunk = 0; // P2G: particles per chunk staged in shared memory by one bulk copy per payload field
    int buffers = 1; // P2G: staging buffers (2: the next chunk's copy overlaps the whole current chunk)
    int scatter_ctas_per_sm = 0; // P2G scatter: persistent CTAs per SM
    int g2p_threads = 0; // G2P: threads per CTA, i.e. particles per pass over a group
    int g2p_tight = 0; // G2P: +1 = registers cut for more resident threads per SM; +2 = the velocities of the group's
                       // 8 neighbouring blocks staged in shared memory by bulk asynchronous copies
    int tuned = 0; // 1 when chosen by the autotuner's measurements
};

struct KernelTimes {
    // milliseconds accumulated per phase while timing is enabled
    double sort = 0, blocks = 0, p2g = 0, grid = 0, g2p = 0;
    int64_t steps = 0;
};

class EngineBase {
public:
    virtual ~EngineBase() = default;
    virtual int precision() const = 0;
    // Build device state for the given scenes (replaces any previous batch).
    virtual int load(const std::vector<const SceneDesc*>& scenes) = 0;
    // Re-form the batch: keep the listed scene slots (device state, in that order) and append new scenes.
    // Slots are renumbered: kept scenes first, then the new ones.
    virtual int repack(const std::vector<int>& keep, const std::vector<const SceneDesc*>& add) = 0;
    // Advance every scene of the batch by nsteps substeps. Returns 0 or a ZR_ERR code; rep gets details.
    virtual int step(int nsteps, StepReport* rep) = 0;
    // Copy one field of one scene, in the caller's particle order, into out (float64 or float32).
    virtual int get_field(int scene, int field, void* out, int out_is_f32) = 0;
    // Overwrite one field of one scene from host memory (caller's particle order).
    virtual int set_field(int scene, int field, const void* in, int in_is_f32) = 0;
    // Dynamic state in one call: x,v,C,F,d interleaved per particle as 25 values (d = 0 without damage).
    virtual int get_state(int scene, void* out25, int out_is_f32) = 0;
    virtual int set_state(int scene, const void* in25, int in_is_f32) = 0;
    // get_state into out25, then set_state from in25 (disjoint buffers of one precision); with both in pinned host
    // memory one kernel moves the two directions over the host link at the same time.
    virtual int exchange_state(int scene, const void* in25, void* out25, int is_f32) = 0;
    // nsteps jobs, each: set_state(in25[i]), one substep, get_state(out25[i]); the host copies of the next inputs and
    // the last outputs run on copy engines while the GPU computes (the buffers stay in use until the call returns)
    virtual int stream_steps(int scene, int nsteps, const void* const* in25, void* const* out25, int is_f32) = 0;
    virtual int64_t stream_reruns() const = 0; // jobs stream_steps ran again the safe way (cumulative)
    // FP64-accumulated reductions: mass, momentum(3), kinetic energy, max speed, grid mass
    virtual int reductions(int scene, double* out7) = 0;
    virtual int set_dt(int scene, double dt) = 0;
    virtual double dt(int scene) const = 0;
    virtual double time(int scene) const = 0;
    virtual int set_time(int scene, double t) = 0;
    // Device-side checkpoint of the whole batch (particle state, ids, scene clocks and dt): save, then restore
    // to return to it (a re-formed batch invalidates it).
    virtual int checkpoint_save() = 0;
    virtual int checkpoint_restore() = 0;
    // iterations of the last substep's implicit damage solve for a scene (0 when it solves nothing)
    virtual int cg_iterations(int scene, int* out) = 0;
    virtual int64_t count(int scene) const = 0;
    virtual int n_scenes() const = 0;
    // Binning products of the current substep input (for parity tests): sorted keys (scene bits
    // removed), sorted original indices, group starts, active pages.
    virtual int binning(int scene, std::vector<uint64_t>& keys, std::vector<int32_t>& order, std::vector<int32_t>& group_first,
        std::vector<uint64_t>& pages) = 0;
    virtual void set_timing(bool on) = 0;
    virtual KernelTimes timing() const = 0;
    virtual void reset_timing() = 0;
    virtual int sync() = 0;
    virtual void* stream() const = 0;
    virtual int64_t device_bytes() const = 0;
    virtual int use_graph(bool on) = 0;
    virtual int kernel_launches_per_step() const = 0;
    // autotuner: 0 off (default schedule), 1 on with a process-wide cache, 2 on and re-measured per batch
    virtual int set_autotune(int mode) = 0;
    virtual Schedule schedule() const = 0;
    virtual int set_schedule(const Schedule& s) = 0;
    virtual std::string last_error() const = 0;
};

std::unique_ptr<EngineBase> make_engine_f32();
std::unique_ptr<EngineBase> make_engine_f64();

} // namespace zr
