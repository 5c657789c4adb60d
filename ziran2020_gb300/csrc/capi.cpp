// C ABI of the GB300 explicit-MPM engine (declared in include/ziran_gb300.h).
#include "../../include/ziran_gb300.h"
#include "engine.h"
#include "physics.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <vector>

using namespace zr;

struct zr_scene {
    // TimeStepping state of zr_scene_advance_frames (TimeStepping.h:17-31): max_dt shrinks on restarts
    double max_dt = -1, max_dt_original = -1;
    int autotune = -1; // -1: the engine's default
    bool has_schedule = false;
    zr::Schedule schedule;
    double last_ms = 0;
    int64_t last_groups = 0, last_blocks = 0;
    int precision = ZR_F32;
    SceneDesc desc;
    std::unique_ptr<EngineBase> eng;
    std::string err;
    bool committed = false;
    int64_t fallbacks = 0;
};

struct zr_batch {
    int autotune = -1;
    double last_ms = 0;
    int precision = ZR_F32;
    std::vector<std::unique_ptr<SceneDesc>> descs;
    std::unique_ptr<EngineBase> eng;
    std::string err;
    bool committed = false;
    int64_t fallbacks = 0;
};

namespace {

const char* kVersion = "ziran2020_gb300 0.1 (sm_103a)";

int set_err(std::string& e, int code, const std::string& m)
{
    e = m;
    return code;
}

std::unique_ptr<EngineBase> make_engine(int precision)
{
    return precision == ZR_F64 ? make_engine_f64() : make_engine_f32();
}

// assign a material to a particle range, creating a new material entry
int assign_material(SceneDesc& d, int64_t first, int64_t count, const SceneDesc::Mat& m, std::string& err)
{
    if (first < 0 || count < 0 || first + count > d.n) return set_err(err, ZR_ERR_ARG, "particle range out of bounds");
    if ((int)d.materials.size() >= 16) return set_err(err, ZR_ERR_ARG, "at most 16 materials per scene");
    if (d.material.empty() && !d.materials.empty()) d.material.assign(d.n, 0);
    if (d.material.size() < (size_t)d.n) d.material.resize(d.n, 0);
    d.materials.push_back(m);
    const uint8_t id = (uint8_t)(d.materials.size() - 1);
    for (int64_t i = first; i < first + count; i++) d.material[i] = id;
    return ZR_OK;
}

// ---------------------------------------------------------------------------------------------------
// seeded generators (identical on every host: raw mt19937_64 outputs, own uniform / normal / vMF)
// ---------------------------------------------------------------------------------------------------
struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    double uniform() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); } // [0,1)
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
    // von Mises-Fisher on the unit sphere about +x (Wood's method for three dimensions)
    void vmf(double kappa, double out[3])
    {
        double u = uniform();
        double w = 1.0 + std::log(u + (1.0 - u) * std::exp(-2.0 * kappa)) / kappa;
        if (w > 1) w = 1;
        if (w < -1) w = -1;
        double phi = 6.283185307179586 * uniform();
        double r = std::sqrt(std::max(0.0, 1.0 - w * w));
        out[0] = w;
        out[1] = r * std::cos(phi);
        out[2] = r * std::sin(phi);
    }
};

void recipe_cells(const zr_scene_recipe* r, int64_t nc[3], int64_t lo[3])
{
    for (int a = 0; a < 3; a++) {
        nc[a] = std::max<int64_t>(1, std::llround(r->size[a] / r->dx));
        lo[a] = std::llround((r->center[a] - 0.5 * (double)nc[a] * r->dx) / r->dx);
    }
}

} // namespace

extern "C" {

const char* zr_version(void) { return kVersion; }

// MpmParticleHandleBase::initializeRotatedFHelper, one director (MpmParticleHandleBase.cpp:224-268):
// columns a0, a0_perp = normalize(-a0y, a0x, 0) (e1 when a0 is along z), a0 x a0_perp
void zr_rotated_F(const double a0[3], double F[9])
{
    double c1[3];
    if (std::fabs(a0[0]) < 1e-6 && std::fabs(a0[1]) < 1e-6) {
        c1[0] = 1;
        c1[1] = 0;
        c1[2] = 0;
    }
    else {
        c1[0] = -a0[1];
        c1[1] = a0[0];
        c1[2] = 0;
        double nn = std::sqrt(c1[0] * c1[0] + c1[1] * c1[1]);
        c1[0] /= nn;
        c1[1] /= nn;
    }
    double c2[3] = { a0[1] * c1[2] - a0[2] * c1[1], a0[2] * c1[0] - a0[0] * c1[2], a0[0] * c1[1] - a0[1] * c1[0] };
    for (int r = 0; r < 3; r++) {
        F[3 * r + 0] = a0[r];
        F[3 * r + 1] = c1[r];
        F[3 * r + 2] = c2[r];
    }
}

// NeoHookeanBorden::getSigmaCrit: psi((1+p) I) with g = 1 (NeoHookeanBorden.cpp:38-68)
double zr_qrnh_sigma_crit(double E, double nu, double p)
{
    double lambda = E * nu / ((1 + nu) * (1 - 2 * nu));
    double mu = E / (2 * (1 + nu));
    double r = 1 + p, J = r * r * r;
    // R = (1+p) I: sum_{i<=j} r_ij^2 = 3 r^2
    return 0.5 * lambda * (J - 1) * (J - 1) + (mu / 2 * (3 * r * r - 3) - mu * (J - 1));
}

double zr_nhb_sigma_crit(double E, double nu, double p)
{
    double lambda = E * nu / ((1 + nu) * (1 - 2 * nu));
    double mu = E / (2 * (1 + nu));
    double kappa = 0.666666 * mu + lambda;
    double J = (1 + p) * (1 + p) * (1 + p);
    // the deviatoric part vanishes for an isotropic stretch; psi = psi_vol whether J >= 1 or not
    return kappa / 2 * ((J * J - 1) / 2 - std::log(J));
}

int zr_recipe_default(int kind, zr_scene_recipe* r)
{
    if (!r) return ZR_ERR_ARG;
    std::memset(r, 0, sizeof *r);
    r->kind = kind;
    r->ppc_side = 2;
    r->seed = 12345;
    if (kind == ZR_RECIPE_ELASTIC_BOX) {
        r->dx = 1.0 / 64;
        r->dt = 1e-4;
        r->size[0] = r->size[1] = r->size[2] = 0.25;
        r->center[0] = 0.5;
        r->center[1] = 0.6;
        r->center[2] = 0.5;
        r->velocity[1] = -1.0;
        r->gravity[1] = -9.8;
        r->E = 1e4;
        r->nu = 0.3;
        r->rho = 1000;
        r->apic_rpic_ratio = 1.0;
        r->ground_y = 0.05;
        return ZR_OK;
    }
    if (kind == ZR_RECIPE_ANISO_SLAB) {
        r->dx = 1.0 / 128;
        r->dt = 5e-5;
        r->size[0] = 0.5;
        r->size[1] = 0.1;
        r->size[2] = 0.5;
        r->center[0] = r->center[1] = r->center[2] = 0.5;
        r->E = 5e4;
        r->nu = 0.25;
        r->rho = 800;
        r->apic_rpic_ratio = 0.0; // the AnisoMPM demos run RPIC (examples/vonMisesTear.h:28)
        r->kappa_vmf = 20;
        r->alpha = -1;
        r->l0 = 0.5 * r->dx;
        r->eta = 0.1;
        r->zeta = 1;
        r->residual = 0.01;
        r->sigma_c_mean = 400;
        r->sigma_c_std = 40;
        r->pull_speed = 0.5;
        r->grip_cells = 2;
        return ZR_OK;
    }
    return ZR_ERR_ARG;
}

int64_t zr_recipe_count(const zr_scene_recipe* r)
{
    if (!r || r->dx <= 0 || r->ppc_side <= 0) return -1;
    int64_t nc[3], lo[3];
    recipe_cells(r, nc, lo);
    int64_t p = r->ppc_side;
    return nc[0] * nc[1] * nc[2] * p * p * p;
}

int zr_recipe_generate(const zr_scene_recipe* r, double* x, double* v, double* m, double* V0, double* F, double* sigma_c)
{
    if (!r || r->dx <= 0 || r->ppc_side <= 0) return ZR_ERR_ARG;
    int64_t nc[3], lo[3];
    recipe_cells(r, nc, lo);
    const int ps = r->ppc_side;
    const double sub = r->dx / ps;
    const double vol = r->dx * r->dx * r->dx / (double)(ps * ps * ps);
    Rng rng(r->seed);
    int64_t p = 0;
    for (int64_t i = 0; i < nc[0]; i++)
        for (int64_t j = 0; j < nc[1]; j++)
            for (int64_t k = 0; k < nc[2]; k++)
                for (int a = 0; a < ps; a++)
                    for (int b = 0; b < ps; b++)
                        for (int c = 0; c < ps; c++, p++) {
                            const int64_t cell[3] = { lo[0] + i, lo[1] + j, lo[2] + k };
                            const int s[3] = { a, b, c };
                            for (int d = 0; d < 3; d++) {
                                double u = rng.uniform();
                                if (x) x[3 * p + d] = (double)cell[d] * r->dx + ((double)s[d] + u) * sub;
                                if (v) v[3 * p + d] = r->velocity[d];
                            }
                            if (m) m[p] = r->rho * vol;
                            if (V0) V0[p] = vol;
                            if (r->kind == ZR_RECIPE_ANISO_SLAB) {
                                double a0[3];
                                rng.vmf(r->kappa_vmf, a0);
                                if (F) zr_rotated_F(a0, F + 9 * p);
                                double sc = r->sigma_c_mean + r->sigma_c_std * rng.normal();
                                if (sigma_c) sigma_c[p] = sc;
                            }
                            else {
                                if (F)
                                    for (int q = 0; q < 9; q++) F[9 * p + q] = (q % 4 == 0) ? 1.0 : 0.0;
                                if (sigma_c) sigma_c[p] = 1.0;
                            }
                        }
    return ZR_OK;
}

// ------------------------------------------------------------------------------------------- scene
int zr_scene_create(int precision, zr_scene** out)
{
    if (!out || (precision != ZR_F32 && precision != ZR_F64)) return ZR_ERR_ARG;
    zr_scene* s = new (std::nothrow) zr_scene();
    if (!s) return ZR_ERR_ARG;
    s->precision = precision;
    *out = s;
    return ZR_OK;
}

int zr_scene_destroy(zr_scene* s)
{
    delete s;
    return ZR_OK;
}

int zr_scene_set_params(zr_scene* s, const zr_sim_params* p)
{
    if (!s || !p) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "parameters are fixed once the scene has stepped; use zr_scene_set_dt");
    if (!(p->dx > 0) || !(p->dt > 0)) return set_err(s->err, ZR_ERR_ARG, "dx and dt must be positive");
    if (p->apic_rpic_ratio < 0 || p->apic_rpic_ratio > 1) return set_err(s->err, ZR_ERR_ARG, "apic_rpic_ratio must be in [0,1] (MpmSimulationBase.cpp:125)");
    s->desc.dx = p->dx;
    s->desc.dt = p->dt;
    for (int a = 0; a < 3; a++) s->desc.gravity[a] = p->gravity[a];
    s->desc.apic_rpic_ratio = p->apic_rpic_ratio;
    s->desc.cfl = p->cfl > 0 ? p->cfl : 0.6;
    s->desc.domain_cells = p->domain_cells;
    return ZR_OK;
}

int zr_scene_add_particles(zr_scene* s, int64_t n, const double* x, const double* v, const double* m, const double* V0, const double* F, int64_t* first)
{
    if (!s || n <= 0 || !x || !m || !V0) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "particles must be added before the first substep");
    SceneDesc& d = s->desc;
    const int64_t f0 = d.n;
    d.x.insert(d.x.end(), x, x + 3 * n);
    if (v)
        d.v.insert(d.v.end(), v, v + 3 * n);
    else
        d.v.insert(d.v.end(), 3 * n, 0.0);
    d.m.insert(d.m.end(), m, m + n);
    d.V0.insert(d.V0.end(), V0, V0 + n);
    if (F)
        d.F.insert(d.F.end(), F, F + 9 * n);
    else
        for (int64_t i = 0; i < n; i++)
            for (int q = 0; q < 9; q++) d.F.push_back((q % 4 == 0) ? 1.0 : 0.0);
    d.C.insert(d.C.end(), 9 * n, 0.0);
    d.d.insert(d.d.end(), n, 0.0);
    d.sigma_c.insert(d.sigma_c.end(), n, 1.0);
    if (!d.material.empty()) d.material.resize(f0 + n, 0);
    d.n = f0 + n;
    if (first) *first = f0;
    return ZR_OK;
}

static int add_model(zr_scene* s, int64_t first, int64_t count, int model, double E, double nu)
{
    if (!s) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "materials must be attached before the first substep");
    if (!(E > 0) || !(nu > -1 && nu < 0.5)) return set_err(s->err, ZR_ERR_ARG, "need E > 0 and -1 < nu < 0.5");
    SceneDesc::Mat m;
    m.model = model;
    m.E = E;
    m.nu = nu;
    return assign_material(s->desc, first, count, m, s->err);
}

int zr_scene_add_corotated(zr_scene* s, int64_t first, int64_t count, double E, double nu) { return add_model(s, first, count, ZR_COROTATED, E, nu); }
int zr_scene_add_qr_stable_neohookean(zr_scene* s, int64_t first, int64_t count, double E, double nu, double fiber_x, double fiber_y)
{
    if (!s) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "materials must be attached before the first substep");
    if (!(E > 0) || !(nu > -1 && nu < 0.5)) return set_err(s->err, ZR_ERR_ARG, "need E > 0 and -1 < nu < 0.5");
    if (!(fiber_x >= 0) || !(fiber_y >= 0)) return set_err(s->err, ZR_ERR_ARG, "fibre stiffness scales must be >= 0");
    SceneDesc::Mat m;
    m.model = ZR_QR_STABLE_NEOHOOKEAN;
    m.E = E;
    m.nu = nu;
    m.kx_scale = fiber_x;
    m.ky_scale = fiber_y;
    return assign_material(s->desc, first, count, m, s->err);
}
int zr_scene_add_neohookean_borden(zr_scene* s, int64_t first, int64_t count, double E, double nu)
{
    return add_model(s, first, count, ZR_NEOHOOKEAN_BORDEN, E, nu);
}

int zr_scene_add_aniso_damage(zr_scene* s, int64_t first, int64_t count, double alpha, double l0, double eta, double zeta, double residual,
    const double* sigma_crit)
{
    if (!s || !sigma_crit) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "damage must be attached before the first substep");
    SceneDesc& d = s->desc;
    if (first < 0 || count <= 0 || first + count > d.n) return set_err(s->err, ZR_ERR_ARG, "particle range out of bounds");
    if (d.material.empty() || d.materials.empty()) return set_err(s->err, ZR_ERR_ARG, "attach a Neo-Hookean (Borden) model to the range first");
    const uint8_t base = d.material[first];
    for (int64_t i = first; i < first + count; i++)
        if (d.material[i] != base) return set_err(s->err, ZR_ERR_ARG, "the range must carry a single model");
    if (d.materials[base].model != ZR_NEOHOOKEAN_BORDEN && d.materials[base].model != ZR_QR_STABLE_NEOHOOKEAN)
        return set_err(s->err, ZR_ERR_ARG, "anisotropic damage is defined for the Neo-Hookean (Borden) and QR-stable Neo-Hookean models");
    if (!(eta > 0)) return set_err(s->err, ZR_ERR_ARG, "eta must be positive");
    SceneDesc::Mat m = d.materials[base];
    m.damage = 1;
    m.alpha = alpha;
    m.l0 = l0;
    m.eta = eta;
    m.zeta = zeta;
    m.residual = residual;
    int rc = assign_material(d, first, count, m, s->err);
    if (rc) return rc;
    for (int64_t i = 0; i < count; i++) {
        if (!(sigma_crit[i] > 0)) return set_err(s->err, ZR_ERR_ARG, "sigma_crit must be positive");
        d.sigma_c[first + i] = sigma_crit[i];
    }
    return ZR_OK;
}

int zr_scene_add_halfspace(zr_scene* s, const double origin[3], const double normal[3], int type, double friction, const double velocity[3])
{
    if (!s || !origin || !normal) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "collision objects must be added before the first substep");
    if (type < ZR_STICKY || type > ZR_SEPARATE) return set_err(s->err, ZR_ERR_ARG, "type must be ZR_STICKY, ZR_SLIP or ZR_SEPARATE");
    if ((int)s->desc.objects.size() >= 8) return set_err(s->err, ZR_ERR_ARG, "at most 8 collision objects per scene");
    SceneDesc::Obj o;
    for (int a = 0; a < 3; a++) {
        o.origin[a] = origin[a];
        o.normal[a] = normal[a];
        o.vel[a] = velocity ? velocity[a] : 0.0;
    }
    o.friction = friction;
    o.type = type;
    s->desc.objects.push_back(o);
    return ZR_OK;
}

static int commit(zr_scene* s)
{
    if (s->committed) return ZR_OK;
    if (s->desc.n <= 0) return set_err(s->err, ZR_ERR_STATE, "no particles");
    if (s->desc.materials.empty()) return set_err(s->err, ZR_ERR_STATE, "no constitutive model attached");
    // particles without an explicit model take the first one
    s->eng = make_engine(s->precision);
    if (s->autotune >= 0) s->eng->set_autotune(s->autotune);
    if (s->has_schedule && s->eng->set_schedule(s->schedule)) {
        s->err = s->eng->last_error();
        s->eng.reset();
        return ZR_ERR_ARG;
    }
    std::vector<const SceneDesc*> v{ &s->desc };
    int rc = s->eng->load(v);
    if (rc) {
        s->err = s->eng->last_error();
        s->eng.reset();
        return rc;
    }
    s->committed = true;
    return ZR_OK;
}

int zr_scene_step(zr_scene* s, int nsteps, int* done)
{
    if (!s) return ZR_ERR_ARG;
    if (done) *done = 0;
    int rc = commit(s);
    if (rc) return rc;
    StepReport rep;
    rc = s->eng->step(nsteps, &rep);
    s->fallbacks += rep.fallback;
    s->last_ms = rep.device_ms;
    s->last_groups = rep.n_groups;
    s->last_blocks = rep.n_blocks;
    if (done) *done = rep.steps_done;
    if (rc) s->err = s->eng->last_error();
    return rc;
}

#define NEED_ENGINE(s)            \
    do {                          \
        if (!s) return ZR_ERR_ARG; \
        int rc_ = commit(s);      \
        if (rc_) return rc_;      \
    } while (0)

int zr_scene_get_field(zr_scene* s, int field, void* out, int dtype)
{
    NEED_ENGINE(s);
    if (!out || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->get_field(0, field, out, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_set_field(zr_scene* s, int field, const void* in, int dtype)
{
    NEED_ENGINE(s);
    if (!in || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->set_field(0, field, in, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_get_state(zr_scene* s, void* out, int dtype)
{
    NEED_ENGINE(s);
    if (!out || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->get_state(0, out, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_set_state(zr_scene* s, const void* in, int dtype)
{
    NEED_ENGINE(s);
    if (!in || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->set_state(0, in, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_step_stream(zr_scene* s, int nsteps, const void* const* in, void* const* out, int dtype)
{
    NEED_ENGINE(s);
    if (nsteps < 0 || (nsteps > 0 && (!in || !out)) || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->stream_steps(0, nsteps, in, out, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_stream_reruns(zr_scene* s, int64_t* reruns)
{
    NEED_ENGINE(s);
    if (!reruns) return ZR_ERR_ARG;
    *reruns = s->eng->stream_reruns();
    return ZR_OK;
}

int zr_scene_exchange_state(zr_scene* s, const void* in, void* out, int dtype)
{
    NEED_ENGINE(s);
    if (!in || !out || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = s->eng->exchange_state(0, in, out, dtype == ZR_F32);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_reductions(zr_scene* s, double out[7])
{
    NEED_ENGINE(s);
    if (!out) return ZR_ERR_ARG;
    int rc = s->eng->reductions(0, out);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_set_implicit_damage(zr_scene* s, int on)
{
    if (!s) return ZR_ERR_ARG;
    if (s->committed) return set_err(s->err, ZR_ERR_STATE, "the damage solve must be chosen before the first substep");
    s->desc.implicit_damage = on ? 1 : 0;
    return ZR_OK;
}

int zr_scene_cg_iterations(zr_scene* s, int* iterations)
{
    if (!s || !iterations) return ZR_ERR_ARG;
    *iterations = 0;
    if (!s->committed) return ZR_OK;
    int rc = s->eng->cg_iterations(0, iterations);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

int zr_scene_set_dt(zr_scene* s, double dt)
{
    if (!s || !(dt > 0)) return ZR_ERR_ARG;
    s->desc.dt = dt;
    if (!s->committed) return ZR_OK;
    int rc = s->eng->set_dt(0, dt);
    if (rc) s->err = s->eng->last_error();
    return rc;
}

double zr_scene_time(zr_scene* s)
{
    if (!s) return NAN;
    if (!s->committed) return s->desc.time;
    return s->eng->time(0);
}

int64_t zr_scene_count(zr_scene* s) { return s ? s->desc.n : -1; }

// ---------------------------------------------------------------------------------------------------
// snapshots: SimulationBase::write/read + MpmSimulationBase::writeState/readState (SimulationBase.h:149-187,
// MpmSimulationBase.cpp:1060-1114), as one versioned binary image of the dynamic state
// ---------------------------------------------------------------------------------------------------
namespace {
struct StateHeader {
    char magic[8]; // "ZRSTATE"
    uint32_t version;
    int32_t precision;
    int64_t n;
    double time, dt;
    uint32_t fields, reserved;
};
static_assert(sizeof(StateHeader) == 48, "state header layout");
const char kStateMagic[8] = { 'Z', 'R', 'S', 'T', 'A', 'T', 'E', 0 };
// stored fields, in order, with their component counts: x v C F d m V0 sigma_c, and (version 2) the damage drive
// history of the implicit damage solve
const uint32_t kStateVersion = 2;
const int kStateFields[9] = { ZR_FIELD_X, ZR_FIELD_V, ZR_FIELD_C, ZR_FIELD_F, ZR_FIELD_D, ZR_FIELD_M, ZR_FIELD_V0, ZR_FIELD_SIGMA_C, ZR_FIELD_DTILDE_MAX };
const int kStateComps[9] = { 3, 3, 9, 9, 1, 1, 1, 1, 1 };
int fields_of_version(uint32_t v) { return v == 1 ? 8 : (v == 2 ? 9 : -1); }
int64_t state_bytes(int precision, int64_t n, int fields)
{
    int64_t vals = 0;
    for (int f = 0; f < fields; f++) vals += kStateComps[f];
    return (int64_t)sizeof(StateHeader) + n * vals * (precision == ZR_F64 ? 8 : 4);
}
} // namespace

int64_t zr_scene_state_bytes(zr_scene* s)
{
    if (!s || s->desc.n <= 0) return -1;
    return state_bytes(s->precision, s->desc.n, fields_of_version(kStateVersion));
}

int zr_scene_save_state(zr_scene* s, void* buf, int64_t bytes)
{
    NEED_ENGINE(s);
    const int nf = fields_of_version(kStateVersion);
    const int64_t n = s->desc.n, need = state_bytes(s->precision, n, nf);
    if (!buf || bytes < need) return set_err(s->err, ZR_ERR_ARG, "state buffer smaller than zr_scene_state_bytes");
    StateHeader h;
    std::memcpy(h.magic, kStateMagic, 8);
    h.version = kStateVersion;
    h.precision = s->precision;
    h.n = n;
    h.time = s->eng->time(0);
    h.dt = s->eng->dt(0);
    h.fields = (uint32_t)nf;
    h.reserved = 0;
    std::memcpy(buf, &h, sizeof h);
    char* p = (char*)buf + sizeof h;
    const size_t es = s->precision == ZR_F64 ? 8 : 4;
    for (int f = 0; f < nf; f++) {
        // native precision: the image restores the state bit for bit
        int rc = s->eng->get_field(0, kStateFields[f], p, s->precision == ZR_F32);
        if (rc) {
            s->err = s->eng->last_error();
            return rc;
        }
        p += (size_t)n * kStateComps[f] * es;
    }
    return ZR_OK;
}

int zr_scene_load_state(zr_scene* s, const void* buf, int64_t bytes)
{
    NEED_ENGINE(s);
    if (!buf || bytes < (int64_t)sizeof(StateHeader)) return set_err(s->err, ZR_ERR_ARG, "state image too short");
    StateHeader h;
    std::memcpy(&h, buf, sizeof h);
    if (std::memcmp(h.magic, kStateMagic, 8) != 0) return set_err(s->err, ZR_ERR_ARG, "not a state image");
    const int nf = fields_of_version(h.version);
    if (nf < 0 || h.fields != (uint32_t)nf) return set_err(s->err, ZR_ERR_ARG, "state image of an unknown version");
    if (h.precision != s->precision) return set_err(s->err, ZR_ERR_ARG, "state image of the other precision");
    if (h.n != s->desc.n) return set_err(s->err, ZR_ERR_ARG, "state image of a scene with a different particle count");
    if (bytes < state_bytes(s->precision, h.n, nf) || !(h.dt > 0) || !(h.time >= 0)) return set_err(s->err, ZR_ERR_ARG, "state image truncated or corrupt");
    const char* p = (const char*)buf + sizeof h;
    const size_t es = s->precision == ZR_F64 ? 8 : 4;
    // the fields are written one at a time: a device checkpoint taken first is restored if any write fails, so
    // the scene keeps either its old state or the whole image, never a mix
    int rc = s->eng->checkpoint_save();
    if (rc) {
        s->err = s->eng->last_error();
        return rc;
    }
    auto fail = [&](int code) {
        s->err = s->eng->last_error();
        if (s->eng->checkpoint_restore() != ZR_OK) s->err += " (and restoring the previous state failed)";
        return code;
    };
    for (int f = 0; f < nf; f++) {
        rc = s->eng->set_field(0, kStateFields[f], p, s->precision == ZR_F32);
        if (rc) return fail(rc);
        p += (size_t)h.n * kStateComps[f] * es;
    }
    if (nf < 9) { // an image without the history: it restarts from zero
        std::vector<char> zeros((size_t)h.n * es, 0);
        rc = s->eng->set_field(0, ZR_FIELD_DTILDE_MAX, zeros.data(), s->precision == ZR_F32);
        if (rc) return fail(rc);
    }
    rc = s->eng->set_time(0, h.time);
    if (!rc) rc = s->eng->set_dt(0, h.dt);
    if (rc) return fail(rc);
    s->desc.dt = h.dt;
    return rc;
}

int zr_scene_write_state_file(zr_scene* s, const char* path)
{
    if (!s || !path) return ZR_ERR_ARG;
    const int64_t nb = zr_scene_state_bytes(s);
    if (nb < 0) return set_err(s->err, ZR_ERR_STATE, "no particles");
    std::vector<char> buf((size_t)nb);
    int rc = zr_scene_save_state(s, buf.data(), nb);
    if (rc) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_err(s->err, ZR_ERR_ARG, std::string("cannot open ") + path + " for writing");
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    const bool closed = std::fclose(f) == 0;
    return ok && closed ? ZR_OK : set_err(s->err, ZR_ERR_ARG, std::string("short write to ") + path);
}

int zr_scene_read_state_file(zr_scene* s, const char* path)
{
    if (!s || !path) return ZR_ERR_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_err(s->err, ZR_ERR_ARG, std::string("cannot open ") + path);
    std::vector<char> buf;
    char tmp[1 << 16];
    size_t got;
    while ((got = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
    std::fclose(f);
    return zr_scene_load_state(s, buf.data(), (int64_t)buf.size());
}

// ---------------------------------------------------------------------------------------------------
// .bgeo frame files. Houdini's classic binary geometry layout, version 5, as partio writes it (all numbers
// big-endian): the magic "Bgeo", the version character 'V' and int32 version 5; int32 counts of points,
// primitives, point groups, primitive groups, point attributes (besides the position), vertex attributes,
// primitive attributes and detail attributes; per point attribute its name (uint16 length, then the bytes), its
// component count (uint16), its type (int32: 5 = float vector) and one default value per component (float32);
// then per point x, y, z, w = 1 and each attribute's components (float32); then the end bytes 0x00 0xff.
// ---------------------------------------------------------------------------------------------------
namespace {

struct BigEndianFile {
    FILE* f = nullptr;
    bool ok = true;
    void bytes(const void* p, size_t n) { ok = ok && std::fwrite(p, 1, n, f) == n; }
    void u16(uint16_t v)
    {
        const unsigned char b[2] = { (unsigned char)(v >> 8), (unsigned char)v };
        bytes(b, 2);
    }
    void u32(uint32_t v)
    {
        const unsigned char b[4] = { (unsigned char)(v >> 24), (unsigned char)(v >> 16), (unsigned char)(v >> 8), (unsigned char)v };
        bytes(b, 4);
    }
    void f32(float v)
    {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        u32(u);
    }
};

} // namespace

extern "C" int zr_write_bgeo(const char* path, int64_t n, const double* x, int nattr, const char* const* names, const int32_t* sizes,
    const double* const* data)
{
    if (!path || n < 0 || n > 0x7fffffff || (n > 0 && !x) || nattr < 0 || (nattr > 0 && (!names || !sizes || !data))) return ZR_ERR_ARG;
    for (int k = 0; k < nattr; k++)
        if (!names[k] || sizes[k] < 1 || sizes[k] > 0xffff || std::strlen(names[k]) > 0xffff || (n > 0 && !data[k])) return ZR_ERR_ARG;
    BigEndianFile o;
    o.f = std::fopen(path, "wb");
    if (!o.f) return ZR_ERR_ARG;
    o.bytes("Bgeo", 4);
    o.bytes("V", 1);
    o.u32(5);
    const uint32_t counts[8] = { (uint32_t)n, 0, 0, 0, (uint32_t)nattr, 0, 0, 0 };
    for (uint32_t c : counts) o.u32(c);
    for (int k = 0; k < nattr; k++) {
        const size_t len = std::strlen(names[k]);
        o.u16((uint16_t)len);
        o.bytes(names[k], len);
        o.u16((uint16_t)sizes[k]);
        o.u32(5); // vector of floats (Partio::VECTOR, as the reference adds every attribute)
        for (int c = 0; c < sizes[k]; c++) o.f32(0.0f);
    }
    std::vector<unsigned char> row;
    for (int64_t p = 0; p < n && o.ok; p++) {
        for (int a = 0; a < 3; a++) o.f32((float)x[3 * p + a]);
        o.f32(1.0f);
        for (int k = 0; k < nattr; k++)
            for (int c = 0; c < sizes[k]; c++) o.f32((float)data[k][(size_t)sizes[k] * p + c]);
    }
    const unsigned char end[2] = { 0x00, 0xff };
    o.bytes(end, 2);
    const bool closed = std::fclose(o.f) == 0;
    return o.ok && closed ? ZR_OK : ZR_ERR_ARG;
}

extern "C" int zr_scene_write_bgeo(zr_scene* s, const char* path, int flags)
{
    NEED_ENGINE(s);
    if (!path || (flags & ~(ZR_BGEO_V | ZR_BGEO_D | ZR_BGEO_A1))) return set_err(s->err, ZR_ERR_ARG, "unknown .bgeo attribute flags");
    const int64_t n = s->desc.n;
    std::vector<double> x((size_t)(3 * n)), v, d, a1, F;
    std::vector<const char*> names;
    std::vector<int32_t> sizes;
    std::vector<const double*> data;
    auto field = [&](int f, std::vector<double>& out, int comps) {
        out.resize((size_t)(comps * n));
        int rc = s->eng->get_field(0, f, out.data(), 0);
        if (rc) s->err = s->eng->last_error();
        return rc;
    };
    int rc = field(ZR_FIELD_X, x, 3);
    if (!rc && (flags & ZR_BGEO_V)) {
        rc = field(ZR_FIELD_V, v, 3);
        names.push_back("v");
        sizes.push_back(3);
        data.push_back(v.data());
    }
    if (!rc && (flags & ZR_BGEO_A1)) {
        rc = field(ZR_FIELD_F, F, 9);
        if (!rc) { // the current director R e1 (AnisoFractureSimulation.h:90-97 takes R = U V^T of F's SVD)
            a1.resize((size_t)(3 * n));
            for (int64_t p = 0; p < n; p++) {
                double R[9];
                zr::polar_rotation(F.data() + 9 * p, R);
                for (int a = 0; a < 3; a++) a1[3 * p + a] = R[3 * a];
            }
            names.push_back("a_1");
            sizes.push_back(3);
            data.push_back(a1.data());
        }
    }
    if (!rc && (flags & ZR_BGEO_D)) {
        rc = field(ZR_FIELD_D, d, 1);
        names.push_back("d");
        sizes.push_back(1);
        data.push_back(d.data());
    }
    if (rc) return rc;
    rc = zr_write_bgeo(path, n, x.data(), (int)names.size(), names.data(), sizes.data(), data.data());
    if (rc) return set_err(s->err, rc, std::string("cannot write ") + path);
    return ZR_OK;
}

// ---------------------------------------------------------------------------------------------------
// frames with the reference driver's time stepping and restarts (SimulationBase::simulate/advanceOneFrame,
// SimulationBase.h:275-354; TimeStepping::nextDt, TimeStepping.h:45-59; calculateDt,
// MpmSimulationBase.cpp:1128-1151; the autorestart of MpmSimulationBase.cpp:1480-1510)
// ---------------------------------------------------------------------------------------------------
int zr_scene_advance_frames(zr_scene* s, int frames, double frame_dt, double min_dt, int cfl_dt, int* restarts)
{
    if (restarts) *restarts = 0;
    NEED_ENGINE(s);
    if (frames < 0 || !(frame_dt > 0) || !(min_dt > 0)) return set_err(s->err, ZR_ERR_ARG, "need frames >= 0, frame_dt > 0, min_dt > 0");
    if (s->max_dt_original <= 0) {
        s->max_dt_original = s->eng->dt(0); // the scene's dt is the largest substep (step.max_dt)
        s->max_dt = s->max_dt_original;
    }
    int nrestart = 0;
    for (int f = 0; f < frames; f++) {
        int rc = s->eng->checkpoint_save(); // the frame-start state a restart reads back
        if (rc) {
            s->err = s->eng->last_error();
            return rc;
        }
        double since = 0;
        bool restart = false;
        while (since < frame_dt && !restart) {
            double want = s->max_dt;
            if (cfl_dt) { // cfl dx / max particle speed
                double red[7];
                rc = s->eng->reductions(0, red);
                if (rc) {
                    s->err = s->eng->last_error();
                    return rc;
                }
                if (red[5] > 0) want = s->desc.cfl * s->desc.dx / red[5];
            }
            // TimeStepping::nextDt; without a CFL-derived dt, the equal substeps up to the frame's last two run as one launch
            const double maxd = std::min(s->max_dt, s->max_dt_original);
            double dt = want < min_dt ? min_dt : (want > maxd ? maxd : want);
            int k = 1;
            if (since + dt >= frame_dt)
                dt = frame_dt - since;
            else if (since + 2 * dt > frame_dt)
                dt = (frame_dt - since) / 2;
            else if (!cfl_dt) {
                double t = since;
                k = 0;
                while (t + 2 * dt <= frame_dt && t + dt < frame_dt) {
                    t += dt;
                    k++;
                }
                k = std::max(k, 1);
            }
            if (s->eng->dt(0) != dt) {
                rc = s->eng->set_dt(0, dt);
                if (rc) {
                    s->err = s->eng->last_error();
                    return rc;
                }
            }
            StepReport rep;
            rc = s->eng->step(k, &rep);
            s->last_ms = rep.device_ms;
            s->fallbacks += rep.fallback;
            if (rc == ZR_ERR_CFL) {
                // a particle moved more than a cell: halve max_dt and redo the frame from its start
                if (s->max_dt <= min_dt) return set_err(s->err, ZR_ERR_CFL, "unable to shrink dt further (max_dt at min_dt)");
                s->max_dt = std::max(s->max_dt / 2, min_dt);
                rc = s->eng->checkpoint_restore();
                if (rc) {
                    s->err = s->eng->last_error();
                    return rc;
                }
                nrestart++;
                restart = true;
                break;
            }
            if (rc) {
                s->err = s->eng->last_error();
                return rc;
            }
            for (int q = 0; q < k; q++) since += dt; // TimeStepping::advance, one substep at a time
        }
        if (restart) f--;
    }
    if (restarts) *restarts = nrestart;
    s->desc.dt = s->eng->dt(0);
    return ZR_OK;
}

const char* zr_scene_last_error(zr_scene* s) { return s ? s->err.c_str() : "null scene"; }

double zr_scene_last_step_ms(zr_scene* s) { return s ? s->last_ms : -1.0; }

int zr_scene_last_grid(zr_scene* s, int64_t* n_groups, int64_t* n_blocks)
{
    if (!s) return ZR_ERR_ARG;
    if (n_groups) *n_groups = s->last_groups;
    if (n_blocks) *n_blocks = s->last_blocks;
    return ZR_OK;
}
double zr_batch_last_step_ms(zr_batch* b) { return b ? b->last_ms : -1.0; }

int zr_scene_binning(zr_scene* s, uint64_t* sorted_keys, int32_t* order, int32_t* group_first, int64_t* n_groups, uint64_t* pages, int64_t* n_pages)
{
    NEED_ENGINE(s);
    std::vector<uint64_t> k, pg;
    std::vector<int32_t> o, gf;
    int rc = s->eng->binning(0, k, o, gf, pg);
    if (rc) {
        s->err = s->eng->last_error();
        return rc;
    }
    if (sorted_keys) std::memcpy(sorted_keys, k.data(), 8 * k.size());
    if (order) std::memcpy(order, o.data(), 4 * o.size());
    if (group_first) std::memcpy(group_first, gf.data(), 4 * gf.size());
    if (n_groups) *n_groups = (int64_t)gf.size();
    if (pages) std::memcpy(pages, pg.data(), 8 * pg.size());
    if (n_pages) *n_pages = (int64_t)pg.size();
    return ZR_OK;
}

int zr_scene_set_timing(zr_scene* s, int on)
{
    NEED_ENGINE(s);
    s->eng->set_timing(on != 0);
    s->eng->reset_timing();
    return ZR_OK;
}

int zr_scene_set_autotune(zr_scene* s, int mode)
{
    if (!s || mode < 0 || mode > 2) return ZR_ERR_ARG;
    s->autotune = mode;
    if (s->eng) s->eng->set_autotune(mode);
    return ZR_OK;
}

int zr_scene_set_schedule(zr_scene* s, const int32_t in6[6])
{
    if (!s || !in6) return ZR_ERR_ARG;
    zr::Schedule sc;
    sc.fused = in6[0];
    sc.chunk = in6[1];
    sc.buffers = in6[2];
    sc.scatter_ctas_per_sm = in6[3];
    sc.g2p_threads = in6[4];
    sc.g2p_tight = in6[5];
    if (s->eng) {
        int rc = s->eng->set_schedule(sc);
        if (rc) s->err = s->eng->last_error();
        return rc;
    }
    s->schedule = sc;
    s->has_schedule = true;
    return ZR_OK;
}

static void schedule_out(const zr::Schedule& sc, int32_t out7[7])
{
    out7[0] = sc.fused;
    out7[1] = sc.chunk;
    out7[2] = sc.buffers;
    out7[3] = sc.scatter_ctas_per_sm;
    out7[4] = sc.g2p_threads;
    out7[5] = sc.g2p_tight;
    out7[6] = sc.tuned;
}

int zr_scene_get_schedule(zr_scene* s, int32_t out7[7])
{
    NEED_ENGINE(s);
    if (!out7) return ZR_ERR_ARG;
    schedule_out(s->eng->schedule(), out7);
    return ZR_OK;
}

int zr_scene_get_timing(zr_scene* s, double out5[5], int64_t* steps)
{
    NEED_ENGINE(s);
    KernelTimes t = s->eng->timing();
    if (out5) {
        out5[0] = t.sort;
        out5[1] = t.blocks;
        out5[2] = t.p2g;
        out5[3] = t.grid;
        out5[4] = t.g2p;
    }
    if (steps) *steps = t.steps;
    return ZR_OK;
}

int zr_scene_stats(zr_scene* s, int64_t* launches, int64_t* bytes, int64_t* fallbacks)
{
    NEED_ENGINE(s);
    if (launches) *launches = s->eng->kernel_launches_per_step();
    if (bytes) *bytes = s->eng->device_bytes();
    if (fallbacks) *fallbacks = s->fallbacks;
    return ZR_OK;
}

static int desc_from_recipe(SceneDesc& d, const zr_scene_recipe* r, std::string& err)
{
    int64_t n = zr_recipe_count(r);
    if (n <= 0) return set_err(err, ZR_ERR_ARG, "bad recipe");
    d = SceneDesc();
    d.dx = r->dx;
    d.dt = r->dt;
    for (int a = 0; a < 3; a++) d.gravity[a] = r->gravity[a];
    d.apic_rpic_ratio = r->apic_rpic_ratio;
    d.cfl = 0.6;
    d.domain_cells = r->domain_cells > 0 ? r->domain_cells : (int32_t)std::lround(1.0 / r->dx) + 4;
    d.n = n;
    d.x.resize(3 * n);
    d.v.resize(3 * n);
    d.m.resize(n);
    d.V0.resize(n);
    d.F.resize(9 * n);
    d.C.assign(9 * n, 0.0);
    d.d.assign(n, 0.0);
    d.sigma_c.resize(n);
    int rc = zr_recipe_generate(r, d.x.data(), d.v.data(), d.m.data(), d.V0.data(), d.F.data(), d.sigma_c.data());
    if (rc) return set_err(err, rc, "recipe generation failed");
    SceneDesc::Mat m;
    m.E = r->E;
    m.nu = r->nu;
    if (r->kind == ZR_RECIPE_ELASTIC_BOX) {
        m.model = ZR_COROTATED;
        d.materials.push_back(m);
        SceneDesc::Obj g;
        g.origin[1] = r->ground_y;
        g.normal[0] = 0;
        g.normal[1] = 1;
        g.normal[2] = 0;
        g.type = ZR_STICKY;
        d.objects.push_back(g);
    }
    else if (r->kind == ZR_RECIPE_ANISO_SLAB) {
        if (r->model != 0 && r->model != ZR_NEOHOOKEAN_BORDEN && r->model != ZR_QR_STABLE_NEOHOOKEAN)
            return set_err(err, ZR_ERR_ARG, "recipe model must be Neo-Hookean (Borden) or QR-stable Neo-Hookean");
        m.model = r->model == ZR_QR_STABLE_NEOHOOKEAN ? ZR_QR_STABLE_NEOHOOKEAN : ZR_NEOHOOKEAN_BORDEN;
        if (m.model == ZR_QR_STABLE_NEOHOOKEAN) m.kx_scale = r->fiber_stiffness;
        m.damage = 1;
        m.alpha = r->alpha;
        m.l0 = r->l0;
        m.eta = r->eta;
        m.zeta = r->zeta;
        m.residual = r->residual;
        d.materials.push_back(m);
        d.implicit_damage = r->implicit_damage ? 1 : 0;
        int64_t nc[3], lo[3];
        recipe_cells(r, nc, lo);
        const double x_lo = (double)lo[0] * r->dx, x_hi = (double)(lo[0] + nc[0]) * r->dx;
        SceneDesc::Obj left, right;
        left.origin[0] = x_lo + r->grip_cells * r->dx; // nodes with x <= x_lo + grip follow the left plate
        left.normal[0] = 1;
        left.normal[1] = 0;
        left.vel[0] = -r->pull_speed;
        left.type = ZR_STICKY;
        right.origin[0] = x_hi - r->grip_cells * r->dx;
        right.normal[0] = -1;
        right.normal[1] = 0;
        right.vel[0] = r->pull_speed;
        right.type = ZR_STICKY;
        d.objects.push_back(left);
        d.objects.push_back(right);
    }
    else
        return set_err(err, ZR_ERR_ARG, "unknown recipe kind");
    return ZR_OK;
}

int zr_scene_from_recipe(zr_scene* s, const zr_scene_recipe* r)
{
    if (!s || !r) return ZR_ERR_ARG;
    if (s->committed || s->desc.n) return set_err(s->err, ZR_ERR_STATE, "zr_scene_from_recipe needs an empty scene");
    return desc_from_recipe(s->desc, r, s->err);
}

// ------------------------------------------------------------------------------------------- batch
int zr_batch_create(int precision, zr_batch** out)
{
    if (!out || (precision != ZR_F32 && precision != ZR_F64)) return ZR_ERR_ARG;
    zr_batch* b = new (std::nothrow) zr_batch();
    if (!b) return ZR_ERR_ARG;
    b->precision = precision;
    *out = b;
    return ZR_OK;
}

int zr_batch_destroy(zr_batch* b)
{
    delete b;
    return ZR_OK;
}

int zr_batch_add_scene(zr_batch* b, zr_scene* s, int* slot)
{
    if (!b || !s) return ZR_ERR_ARG;
    if (b->committed) return set_err(b->err, ZR_ERR_STATE, "scenes must be added before zr_batch_commit");
    if (s->desc.n <= 0 || s->desc.materials.empty()) return set_err(b->err, ZR_ERR_ARG, "scene has no particles or no model");
    b->descs.push_back(std::unique_ptr<SceneDesc>(new SceneDesc(s->desc)));
    if (slot) *slot = (int)b->descs.size() - 1;
    return ZR_OK;
}

int zr_batch_add_recipe(zr_batch* b, const zr_scene_recipe* r, int* slot)
{
    if (!b || !r) return ZR_ERR_ARG;
    if (b->committed) return set_err(b->err, ZR_ERR_STATE, "scenes must be added before zr_batch_commit");
    std::unique_ptr<SceneDesc> d(new SceneDesc());
    int rc = desc_from_recipe(*d, r, b->err);
    if (rc) return rc;
    b->descs.push_back(std::move(d));
    if (slot) *slot = (int)b->descs.size() - 1;
    return ZR_OK;
}

int zr_batch_commit(zr_batch* b)
{
    if (!b) return ZR_ERR_ARG;
    if (b->committed) return ZR_OK;
    if (b->descs.empty()) return set_err(b->err, ZR_ERR_STATE, "empty batch");
    b->eng = make_engine(b->precision);
    if (b->autotune >= 0) b->eng->set_autotune(b->autotune);
    std::vector<const SceneDesc*> v;
    for (auto& d : b->descs) v.push_back(d.get());
    int rc = b->eng->load(v);
    if (rc) {
        b->err = b->eng->last_error();
        b->eng.reset();
        return rc;
    }
    b->committed = true;
    // host copies are no longer needed once the device holds the state
    for (auto& d : b->descs) {
        d->x.clear();
        d->x.shrink_to_fit();
        d->v.clear();
        d->v.shrink_to_fit();
        d->C.clear();
        d->C.shrink_to_fit();
        d->F.clear();
        d->F.shrink_to_fit();
        d->m.clear();
        d->m.shrink_to_fit();
        d->V0.clear();
        d->V0.shrink_to_fit();
        d->d.clear();
        d->d.shrink_to_fit();
        d->sigma_c.clear();
        d->sigma_c.shrink_to_fit();
        d->material.clear();
        d->material.shrink_to_fit();
    }
    return ZR_OK;
}

#define NEED_BATCH(b)                 \
    do {                              \
        if (!b) return ZR_ERR_ARG;    \
        int rc_ = zr_batch_commit(b); \
        if (rc_) return rc_;          \
    } while (0)

int zr_batch_step(zr_batch* b, int nsteps, int* done)
{
    if (done) *done = 0;
    NEED_BATCH(b);
    StepReport rep;
    int rc = b->eng->step(nsteps, &rep);
    b->fallbacks += rep.fallback;
    b->last_ms = rep.device_ms;
    if (done) *done = rep.steps_done;
    if (rc) b->err = b->eng->last_error();
    return rc;
}

int zr_batch_get_field(zr_batch* b, int slot, int field, void* out, int dtype)
{
    NEED_BATCH(b);
    if (!out || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    int rc = b->eng->get_field(slot, field, out, dtype == ZR_F32);
    if (rc) b->err = b->eng->last_error();
    return rc;
}

int zr_batch_reductions(zr_batch* b, int slot, double out[7])
{
    NEED_BATCH(b);
    int rc = b->eng->reductions(slot, out);
    if (rc) b->err = b->eng->last_error();
    return rc;
}

int64_t zr_batch_count(zr_batch* b, int slot)
{
    if (!b || slot < 0 || slot >= (int)b->descs.size()) return -1;
    return b->descs[slot]->n;
}

int zr_batch_set_timing(zr_batch* b, int on)
{
    NEED_BATCH(b);
    b->eng->set_timing(on != 0);
    b->eng->reset_timing();
    return ZR_OK;
}

int zr_batch_set_autotune(zr_batch* b, int mode)
{
    if (!b || mode < 0 || mode > 2) return ZR_ERR_ARG;
    b->autotune = mode;
    if (b->eng) b->eng->set_autotune(mode);
    return ZR_OK;
}

int zr_batch_get_schedule(zr_batch* b, int32_t out7[7])
{
    NEED_BATCH(b);
    if (!out7) return ZR_ERR_ARG;
    schedule_out(b->eng->schedule(), out7);
    return ZR_OK;
}

int zr_batch_get_timing(zr_batch* b, double out5[5], int64_t* steps)
{
    NEED_BATCH(b);
    KernelTimes t = b->eng->timing();
    if (out5) {
        out5[0] = t.sort;
        out5[1] = t.blocks;
        out5[2] = t.p2g;
        out5[3] = t.grid;
        out5[4] = t.g2p;
    }
    if (steps) *steps = t.steps;
    return ZR_OK;
}

int zr_batch_stats(zr_batch* b, int64_t* launches, int64_t* bytes, int64_t* fallbacks)
{
    NEED_BATCH(b);
    if (launches) *launches = b->eng->kernel_launches_per_step();
    if (bytes) *bytes = b->eng->device_bytes();
    if (fallbacks) *fallbacks = b->fallbacks;
    return ZR_OK;
}

const char* zr_batch_last_error(zr_batch* b) { return b ? b->err.c_str() : "null batch"; }

} // extern "C"

// ------------------------------------------------------------------------------------------- serving loop
// Continuous batching: requests (a scene and a number of substeps) queue on submit; every tick admits
// queued requests in arrival order while the memory budget and the scene limit allow, re-forms the batch
// (resident scenes stay on the device), advances all resident scenes together by
// min(tick_substeps, fewest remaining) substeps and retires the scenes that are done, reading their final
// state to the host. Latency = completion time - submit time (steady clock).
struct zr_server {
    struct Req {
        SceneDesc desc;
        int substeps = 0, remaining = 0, state = 0; // 0 queued, 1 running, 2 done, 3 failed
        double t_submit = 0, t_admit = 0, t_done = 0, bytes = 0;
        std::vector<double> result; // 25 values per particle at completion
    };
    int precision = ZR_F32;
    double budget = 0;
    int tick_substeps = 10, max_scenes = 256;
    std::unique_ptr<EngineBase> eng;
    std::map<int64_t, Req> reqs;
    std::deque<int64_t> queue;
    std::vector<int64_t> resident; // requests on the device
    std::vector<int> slot; // engine slot of each resident request (slots of retired requests are dropped at the next repack)
    bool dirty = false; // resident set changed since the last repack
    double resident_bytes = 0, particle_substeps = 0, busy_ms = 0;
    int64_t next_id = 1;
    std::string err;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {
// device bytes a resident scene needs: two particle copies, sort buffers, and the grid blocks of about
// n / 256 occupied blocks plus their neighbours (8 per occupied block at most)
double scene_bytes(int precision, int64_t n)
{
    const double s = precision == ZR_F64 ? 8 : 4, nodes = precision == ZR_F64 ? 32 : 64;
    // two pool copies (30 fields and the id), keys (in, sorted), sort values, iota, group starts, the P2G payload
    // (27 fields at 9/8 density) and the incremental sort's six index and key lists
    const double per_particle = 2 * (30 * s + 4) + 8 + 8 + 4 + 4 + 4 + 27 * s * 9 / 8 + 6 * 4;
    const double groups = (double)n / (nodes * 4) + 64;
    return n * per_particle + 8 * groups * (10 * nodes * s + 64);
}
} // namespace

extern "C" {

int zr_server_create(int precision, double budget_bytes, int tick_substeps, int max_scenes, zr_server** out)
{
    if (!out || (precision != ZR_F32 && precision != ZR_F64) || !(budget_bytes > 0) || tick_substeps <= 0 || max_scenes <= 0 || max_scenes > 4096)
        return ZR_ERR_ARG;
    zr_server* sv = new (std::nothrow) zr_server();
    if (!sv) return ZR_ERR_ARG;
    sv->precision = precision;
    sv->budget = budget_bytes;
    sv->tick_substeps = tick_substeps;
    sv->max_scenes = max_scenes;
    *out = sv;
    return ZR_OK;
}

int zr_server_destroy(zr_server* sv)
{
    delete sv;
    return ZR_OK;
}

static int server_enqueue(zr_server* sv, SceneDesc&& d, int substeps, int64_t* id)
{
    if (substeps <= 0) return set_err(sv->err, ZR_ERR_ARG, "substeps must be positive");
    const double bytes = scene_bytes(sv->precision, d.n);
    if (bytes > sv->budget) return set_err(sv->err, ZR_ERR_BUDGET, "the request alone exceeds the memory budget");
    const int64_t rid = sv->next_id++;
    zr_server::Req& r = sv->reqs[rid];
    r.desc = std::move(d);
    r.substeps = r.remaining = substeps;
    r.t_submit = sv->now();
    r.bytes = bytes;
    sv->queue.push_back(rid);
    if (id) *id = rid;
    return ZR_OK;
}

int zr_server_submit_recipe(zr_server* sv, const zr_scene_recipe* rcp, int substeps, int64_t* id)
{
    if (!sv || !rcp) return ZR_ERR_ARG;
    SceneDesc d;
    int rc = desc_from_recipe(d, rcp, sv->err);
    if (rc) return rc;
    return server_enqueue(sv, std::move(d), substeps, id);
}

int zr_server_submit_scene(zr_server* sv, zr_scene* s, int substeps, int64_t* id)
{
    if (!sv || !s) return ZR_ERR_ARG;
    if (s->desc.n <= 0 || s->desc.materials.empty()) return set_err(sv->err, ZR_ERR_ARG, "scene has no particles or no model");
    if (s->committed) return set_err(sv->err, ZR_ERR_STATE, "submit a scene before it has stepped");
    SceneDesc d = std::move(s->desc); // the server takes the particles; the scene handle is left empty
    s->desc = SceneDesc();
    return server_enqueue(sv, std::move(d), substeps, id);
}

int zr_server_tick(zr_server* sv, int* running, int* queued, int* finished)
{
    if (!sv) return ZR_ERR_ARG;
    int done_now = 0;
    // admit in arrival order while the budget and the scene limit allow
    std::vector<int64_t> add_ids;
    double bytes = sv->resident_bytes;
    while (!sv->queue.empty() && (int)(sv->resident.size() + add_ids.size()) < sv->max_scenes) {
        zr_server::Req& r = sv->reqs[sv->queue.front()];
        if (bytes + r.bytes > sv->budget) break;
        bytes += r.bytes;
        add_ids.push_back(sv->queue.front());
        sv->queue.pop_front();
    }
    if (!add_ids.empty() || sv->dirty) {
        std::vector<int> keep = sv->slot; // the engine slots of the requests that are still resident
        std::vector<const SceneDesc*> add;
        for (int64_t rid : add_ids) add.push_back(&sv->reqs[rid].desc);
        if (keep.empty() && add.empty()) {
            sv->eng.reset();
        }
        else {
            if (!sv->eng) sv->eng = make_engine(sv->precision);
            int rc = keep.empty() ? sv->eng->load(add) : sv->eng->repack(keep, add);
            if (rc) {
                // the batch could not be formed: fail the requests involved and start from an empty device
                set_err(sv->err, rc, sv->eng->last_error());
                for (int64_t rid : add_ids) sv->reqs[rid].state = 3;
                for (int64_t rid : sv->resident) sv->reqs[rid].state = 3;
                sv->resident.clear();
                sv->slot.clear();
                sv->resident_bytes = 0;
                sv->dirty = false;
                sv->eng.reset();
                return rc;
            }
        }
        // the engine renumbered its slots: kept scenes first, in order, then the admitted ones
        for (size_t k = 0; k < sv->slot.size(); k++) sv->slot[k] = (int)k;
        const double t = sv->now();
        for (int64_t rid : add_ids) {
            zr_server::Req& r = sv->reqs[rid];
            r.state = 1;
            r.t_admit = t;
            sv->slot.push_back((int)sv->resident.size());
            sv->resident.push_back(rid);
            r.desc.x.clear(); // the device holds the state now
            r.desc.v.clear();
            r.desc.C.clear();
            r.desc.F.clear();
            r.desc.d.clear();
        }
        sv->resident_bytes = bytes;
        sv->dirty = false;
    }
    if (!sv->resident.empty()) {
        int k = sv->tick_substeps;
        for (int64_t rid : sv->resident) k = std::min(k, sv->reqs[rid].remaining);
        StepReport rep;
        int rc = sv->eng->step(k, &rep);
        sv->busy_ms += rep.device_ms;
        if (rc) {
            set_err(sv->err, rc, sv->eng->last_error());
            for (int64_t rid : sv->resident) sv->reqs[rid].state = 3;
            sv->resident.clear();
            sv->slot.clear();
            sv->resident_bytes = 0;
            sv->dirty = false;
            sv->eng.reset();
            return rc;
        }
        std::vector<int64_t> still;
        std::vector<int> still_slot;
        const double t = sv->now();
        for (size_t k2 = 0; k2 < sv->resident.size(); k2++) {
            const int64_t rid = sv->resident[k2];
            const int slot = sv->slot[k2];
            zr_server::Req& r = sv->reqs[rid];
            r.remaining -= k;
            sv->particle_substeps += (double)r.desc.n * k;
            if (r.remaining > 0) {
                still.push_back(rid);
                still_slot.push_back(slot);
                continue;
            }
            if (sv->eng->count(slot) != r.desc.n) return set_err(sv->err, ZR_ERR_STATE, "server slot bookkeeping does not match the engine");
            r.result.resize((size_t)r.desc.n * 25);
            int rc2 = sv->eng->get_state(slot, r.result.data(), 0);
            if (rc2) return set_err(sv->err, rc2, sv->eng->last_error());
            r.state = 2;
            r.t_done = t;
            sv->resident_bytes -= r.bytes;
            sv->dirty = true;
            done_now++;
        }
        sv->resident.swap(still);
        sv->slot.swap(still_slot);
    }
    if (running) *running = (int)sv->resident.size();
    if (queued) *queued = (int)sv->queue.size();
    if (finished) *finished = done_now;
    return ZR_OK;
}

int zr_server_request(zr_server* sv, int64_t id, int* state, double* latency_s, int64_t* particles, int* substeps)
{
    if (!sv) return ZR_ERR_ARG;
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return set_err(sv->err, ZR_ERR_ARG, "unknown request");
    const zr_server::Req& r = it->second;
    if (state) *state = r.state;
    if (latency_s) *latency_s = r.state == 2 ? r.t_done - r.t_submit : -1.0;
    if (particles) *particles = r.desc.n;
    if (substeps) *substeps = r.substeps;
    return ZR_OK;
}

int zr_server_result(zr_server* sv, int64_t id, int field, void* out, int dtype)
{
    if (!sv || !out || (dtype != ZR_F32 && dtype != ZR_F64)) return ZR_ERR_ARG;
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end() || it->second.state != 2) return set_err(sv->err, ZR_ERR_STATE, "request not finished");
    const zr_server::Req& r = it->second;
    int off, nc;
    switch (field) {
    case ZR_FIELD_X: off = 0; nc = 3; break;
    case ZR_FIELD_V: off = 3; nc = 3; break;
    case ZR_FIELD_C: off = 6; nc = 9; break;
    case ZR_FIELD_F: off = 15; nc = 9; break;
    case ZR_FIELD_D: off = 24; nc = 1; break;
    default: return set_err(sv->err, ZR_ERR_ARG, "results hold x, v, C, F and d");
    }
    for (int64_t p = 0; p < r.desc.n; p++)
        for (int c = 0; c < nc; c++) {
            const double v = r.result[(size_t)p * 25 + off + c];
            if (dtype == ZR_F64)
                ((double*)out)[p * nc + c] = v;
            else
                ((float*)out)[p * nc + c] = (float)v;
        }
    return ZR_OK;
}

int zr_server_release(zr_server* sv, int64_t id)
{
    if (!sv) return ZR_ERR_ARG;
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end() || (it->second.state != 2 && it->second.state != 3)) return set_err(sv->err, ZR_ERR_STATE, "request not finished");
    sv->reqs.erase(it);
    return ZR_OK;
}

int zr_server_stats(zr_server* sv, double* particle_substeps, double* device_ms, int64_t* device_bytes)
{
    if (!sv) return ZR_ERR_ARG;
    if (particle_substeps) *particle_substeps = sv->particle_substeps;
    if (device_ms) *device_ms = sv->busy_ms;
    if (device_bytes) *device_bytes = sv->eng ? sv->eng->device_bytes() : 0;
    return ZR_OK;
}

const char* zr_server_last_error(zr_server* sv) { return sv ? sv->err.c_str() : "null server"; }

} // extern "C"
