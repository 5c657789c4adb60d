// ziran_gb300.hpp — header-only C++ shim over the C ABI (ziran_gb300.h) that keeps the names and shape of
// Ziran's explicit-MPM API, so code written against MpmSimulationBase / particle handles / constitutive
// models can switch to the GPU path with few edits.
//
//   Ziran (Lib/MPM, Projects/anisofracture)                     this shim
//   MpmSimulationBase<T,3> sim; sim.dx = ...; sim.gravity = ...   ziran_gb300::MpmSimulation<T> sim; same members
//   init_helper.sample...(...) -> MpmParticleHandleBase           sim.addParticles(x, m, V0, v, F) -> ParticleHandle
//   handle.addFBasedMpmForce(CorotatedElasticity<T,3>(E, nu))      handle.addFBasedMpmForce(CorotatedElasticity<T>(E, nu))
//   handle.addFBasedMpmForceWithAnisotropicPhaseField(...)        handle.addFBasedMpmForceWithAnisotropicPhaseField(...)
//   init_helper.addAnalyticCollisionObject(obj)                   sim.addCollisionObject(HalfSpace<T>{o, n}, STICKY, ...)
//   sim.advanceOneTimeStep(dt)                                     sim.advanceOneTimeStep() / sim.advance(n)
//   RestartException (MpmSimulationBase.cpp:1498)                  ziran_gb300::RestartException (dt left unchanged)
//
// Errors are thrown as std::runtime_error, as ZIRAN_ASSERT does (Debug.h:19-37).
#ifndef ZIRAN_GB300_HPP
#define ZIRAN_GB300_HPP

#include "ziran_gb300.h"

#include <array>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace ziran_gb300 {

struct RestartException : std::runtime_error {
    int substeps_done;
    RestartException(const std::string& m, int done) : std::runtime_error(m), substeps_done(done) {}
};

template <class T>
struct CorotatedElasticity {
    T E, nu;
    CorotatedElasticity(T E_, T nu_) : E(E_), nu(nu_) {}
};

template <class T>
struct NeoHookeanBorden {
    T E, nu;
    NeoHookeanBorden(T E_, T nu_) : E(E_), nu(nu_) {}
    // NeoHookeanBorden::getSigmaCrit (NeoHookeanBorden.cpp:38-44)
    T getSigmaCrit(T percentage) const { return (T)zr_nhb_sigma_crit(E, nu, percentage); }
};

// QRStableNeoHookean(E, nu) with setExtraFiberStiffness (QRStableNeoHookean.h:58-107)
template <class T>
struct QRStableNeoHookean {
    T E, nu;
    T kx_scale = 0, ky_scale = 0; // fibre stiffness in units of mu
    QRStableNeoHookean(T E_, T nu_) : E(E_), nu(nu_) {}
    void setExtraFiberStiffness(int component, T scale)
    {
        if (component == 0)
            kx_scale = scale;
        else if (component == 1)
            ky_scale = scale;
        else
            throw std::runtime_error("It is not allowed to put fiber at z direction");
    }
    // QRStableNeoHookean::getSigmaCrit (QRStableNeoHookean.h:68-84)
    T getSigmaCrit(T percentage) const { return (T)zr_qrnh_sigma_crit(E, nu, percentage); }
};

enum CollisionType { STICKY = ZR_STICKY, SLIP = ZR_SLIP, SEPARATE = ZR_SEPARATE };

template <class T>
struct HalfSpace {
    std::array<T, 3> origin, outward_normal;
};

template <class T>
class MpmSimulation;

template <class T>
class ParticleHandle {
public:
    int64_t first, count;

    // MpmParticleHandleBase::addFBasedMpmForce (MpmParticleHandleBase.cpp:132-145)
    void addFBasedMpmForce(const CorotatedElasticity<T>& m) { sim_->check(zr_scene_add_corotated(sim_->h_, first, count, m.E, m.nu)); }
    void addFBasedMpmForce(const NeoHookeanBorden<T>& m) { sim_->check(zr_scene_add_neohookean_borden(sim_->h_, first, count, m.E, m.nu)); }
    void addFBasedMpmForce(const QRStableNeoHookean<T>& m)
    {
        sim_->check(zr_scene_add_qr_stable_neohookean(sim_->h_, first, count, m.E, m.nu, m.kx_scale, m.ky_scale));
    }

    // MpmParticleHandleBase::addFBasedMpmForceWithAnisotropicPhaseField (MpmParticleHandleBase.cpp:175-222) with one
    // director a0 = e1 (fibre directions are carried by the initial F, see fibreRotatedF) and a critical stress per
    // particle (the reference sets one per handle from `percentage`; pass model.getSigmaCrit(percentage) to all).
    template <class Model> // NeoHookeanBorden<T> or QRStableNeoHookean<T>
    void addFBasedMpmForceWithAnisotropicPhaseField(T alpha, T l0, const Model& model, T eta, T zeta, T residual,
        const std::vector<T>& sigma_crit)
    {
        addFBasedMpmForce(model);
        std::vector<double> sc(sigma_crit.begin(), sigma_crit.end());
        if ((int64_t)sc.size() != count) throw std::runtime_error("sigma_crit needs one value per particle of the handle");
        sim_->check(zr_scene_add_aniso_damage(sim_->h_, first, count, alpha, l0, eta, zeta, residual, sc.data()));
    }

private:
    friend class MpmSimulation<T>;
    MpmSimulation<T>* sim_ = nullptr;
};

// MpmParticleHandleBase::initializeRotatedFHelper (MpmParticleHandleBase.cpp:224-268), row-major
inline std::array<double, 9> fibreRotatedF(const std::array<double, 3>& a0)
{
    std::array<double, 9> F;
    zr_rotated_F(a0.data(), F.data());
    return F;
}

template <class T>
class MpmSimulation {
public:
    // public knobs of MpmSimulationBase (MpmSimulationBase.h:47-76); read when the first substep runs
    T dx = (T)1;
    T dt = (T)1 / 24; // the substep (the reference's step.max_dt)
    std::array<T, 3> gravity{ 0, 0, 0 };
    T apic_rpic_ratio = (T)1;
    T cfl = (T).6;
    int domain_cells = 0;
    // AnisoFractureSimulation::implicit (AnisoFractureSimulation.h:59-70, the driver's --implicit_damage):
    // solve the phase field implicitly; read at the first substep
    bool implicit = false;

    MpmSimulation()
    {
        static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double");
        check(zr_scene_create(sizeof(T) == 4 ? ZR_F32 : ZR_F64, &h_));
    }
    ~MpmSimulation() { zr_scene_destroy(h_); }
    MpmSimulation(const MpmSimulation&) = delete;
    MpmSimulation& operator=(const MpmSimulation&) = delete;

    // x, v: 3 per particle; F: 9 per particle row-major (empty v / F = zero / identity)
    ParticleHandle<T> addParticles(const std::vector<double>& x, const std::vector<double>& m, const std::vector<double>& V0,
        const std::vector<double>& v = {}, const std::vector<double>& F = {})
    {
        push_params();
        int64_t n = (int64_t)m.size(), first = 0;
        check(zr_scene_add_particles(h_, n, x.data(), v.empty() ? nullptr : v.data(), m.data(), V0.data(), F.empty() ? nullptr : F.data(), &first));
        ParticleHandle<T> ph;
        ph.first = first;
        ph.count = n;
        ph.sim_ = this;
        return ph;
    }

    // AnalyticCollisionObject(HalfSpace, type) translated by velocity*t (CollisionObject.h:144-148)
    void addCollisionObject(const HalfSpace<T>& hs, CollisionType type, T friction = 0, std::array<T, 3> velocity = { 0, 0, 0 })
    {
        double o[3] = { hs.origin[0], hs.origin[1], hs.origin[2] }, n[3] = { hs.outward_normal[0], hs.outward_normal[1], hs.outward_normal[2] };
        double v[3] = { velocity[0], velocity[1], velocity[2] };
        check(zr_scene_add_halfspace(h_, o, n, (int)type, friction, v));
    }

    // MpmSimulationBase::advanceOneTimeStep (MpmSimulationBase.cpp:262-357)
    void advanceOneTimeStep() { advance(1); }
    void advance(int substeps)
    {
        push_params();
        int done = 0;
        int rc = zr_scene_step(h_, substeps, &done);
        if (rc == ZR_ERR_CFL) throw RestartException(zr_scene_last_error(h_), done);
        check(rc);
    }

    std::vector<double> field(int which) const
    {
        int nc = (which == ZR_FIELD_X || which == ZR_FIELD_V) ? 3 : (which == ZR_FIELD_C || which == ZR_FIELD_F) ? 9 : 1;
        std::vector<double> out((size_t)zr_scene_count(h_) * nc);
        check(zr_scene_get_field(h_, which, out.data(), ZR_F64));
        return out;
    }
    double time() const { return zr_scene_time(h_); }

    // SimulationBase::write / read (SimulationBase.h:149-187): the dynamic state to and from a file
    void writeState(const std::string& path) { check(zr_scene_write_state_file(h_, path.c_str())); }
    void readState(const std::string& path) { check(zr_scene_read_state_file(h_, path.c_str())); }

    // SimulationBase::simulate with autorestart (SimulationBase.h:275-354, MpmSimulationBase.cpp:1480-1510):
    // frames of frame_dt, substeps up to dt (shrunk by half and the frame redone after a CFL violation);
    // returns the number of restarts
    int simulate(int frames, double frame_dt, double min_dt = 1e-6, bool cfl_dt = false)
    {
        push_params();
        int restarts = 0;
        check(zr_scene_advance_frames(h_, frames, frame_dt, min_dt, cfl_dt ? 1 : 0, &restarts));
        return restarts;
    }
    int64_t particleCount() const { return zr_scene_count(h_); }
    // The dynamic state (x, v, C, F, d: 25 values per particle in T) in and out, and jobs of one substep each
    // (state in, substep, result out) pipelined with their host copies; buffers of particleCount() * 25 values
    void getState(T* out) { check(zr_scene_get_state(h_, out, sizeof(T) == 4 ? ZR_F32 : ZR_F64)); }
    void setState(const T* in) { check(zr_scene_set_state(h_, in, sizeof(T) == 4 ? ZR_F32 : ZR_F64)); }
    void stepJobs(const std::vector<const T*>& in, const std::vector<T*>& out)
    {
        if (in.size() != out.size()) throw std::invalid_argument("ziran_gb300: stepJobs needs one output per input");
        push_params();
        check(zr_scene_step_stream(h_, (int)in.size(), reinterpret_cast<const void* const*>(in.data()), reinterpret_cast<void* const*>(out.data()),
            sizeof(T) == 4 ? ZR_F32 : ZR_F64));
    }
    // jobs of stepJobs calls that ran again the safe way after an aborted job (cumulative)
    long long stepJobsRerun() const
    {
        int64_t n = 0;
        check(zr_scene_stream_reruns(h_, &n));
        return (long long)n;
    }
    // conjugate-gradient iterations of the last substep's implicit damage solve
    int cgIterations() const
    {
        int it = 0;
        check(zr_scene_cg_iterations(h_, &it));
        return it;
    }

private:
    friend class ParticleHandle<T>;
    zr_scene* h_ = nullptr;
    bool pushed_ = false;

    void check(int rc) const
    {
        if (rc) throw std::runtime_error(std::string("ziran_gb300: ") + zr_scene_last_error(h_));
    }
    void push_params()
    {
        if (zr_scene_time(h_) == 0 && !pushed_) {
            zr_sim_params p{};
            p.dx = dx;
            p.dt = dt;
            for (int a = 0; a < 3; a++) p.gravity[a] = gravity[a];
            p.apic_rpic_ratio = apic_rpic_ratio;
            p.cfl = cfl;
            p.domain_cells = domain_cells;
            if (zr_scene_set_params(h_, &p) == ZR_OK) {
                check(zr_scene_set_implicit_damage(h_, implicit ? 1 : 0));
                return;
            }
            pushed_ = true; // parameters froze at the first substep; later changes of dt go through set_dt
        }
        check(zr_scene_set_dt(h_, dt));
    }
};

} // namespace ziran_gb300

#endif
