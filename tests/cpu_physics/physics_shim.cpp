// Test shim: exposes the GPU physics routines (ziran2020_gb300/csrc/physics.cuh, compiled here as host
// C++) to the CPU tests, which compare them with the oracle and with numpy.
#include "../../ziran2020_gb300/csrc/physics.cuh"

using namespace zr;

template <class T>
static Material<T> mat(int model, double E, double nu)
{
    Material<T> m{};
    m.model = model;
    T Et = (T)E, nut = (T)nu;
    m.lambda = Et * nut / (((T)1 + nut) * ((T)1 - (T)2 * nut));
    m.mu = Et / ((T)2 * ((T)1 + nut));
    m.kappa = (T).666666 * m.mu + m.lambda;
    return m;
}

extern "C" {
// returns 1 when the FP64 SVD path was taken
int shim_polar(int prec, const double* F, double* R)
{
    if (prec == 4) {
        float f[9], r[9];
        for (int i = 0; i < 9; i++) f[i] = (float)F[i];
        bool fb = polar_rotation(f, r);
        for (int i = 0; i < 9; i++) R[i] = r[i];
        return fb;
    }
    double r[9];
    bool fb = polar_rotation(F, r);
    for (int i = 0; i < 9; i++) R[i] = r[i];
    return fb;
}
void shim_svd_jacobi(const double* A, double* U, double* s, double* V) { svd3_jacobi(A, U, s, V); }
void shim_tension(int prec, const double* S, double* Sp)
{
    if (prec == 4) {
        float a[9], b[9];
        for (int i = 0; i < 9; i++) a[i] = (float)S[i];
        tension_part(a, b);
        for (int i = 0; i < 9; i++) Sp[i] = b[i];
        return;
    }
    tension_part(S, Sp);
}
void shim_tau(int model, double E, double nu, const double* F, double g, double* tau)
{
    Material<double> m = mat<double>(model, E, nu);
    if (model == MODEL_COROTATED)
        tau_corotated(m, F, tau);
    else
        tau_nhb(m, F, g, tau);
}
// any model with fibre stiffness (scales of mu) and the effective (undegraded, isotropic) form; returns J
double shim_tau2(int prec, int model, double E, double nu, double kx, double ky, const double* F, double g, int effective, double* tau)
{
    if (prec == 4) {
        Material<float> m = mat<float>(model, E, nu);
        m.kx = (float)kx * m.mu;
        m.ky = (float)ky * m.mu;
        float f[9], t[9];
        for (int i = 0; i < 9; i++) f[i] = (float)F[i];
        float J = model == MODEL_QR_STABLE_NEOHOOKEAN ? tau_qrnh(m, f, (float)g, t, effective != 0) : det3(f);
        if (model == MODEL_NEOHOOKEAN_BORDEN) tau_nhb(m, f, effective ? 1.f : (float)g, t);
        if (model == MODEL_COROTATED) tau_corotated(m, f, t);
        for (int i = 0; i < 9; i++) tau[i] = t[i];
        return J;
    }
    Material<double> m = mat<double>(model, E, nu);
    m.kx = kx * m.mu;
    m.ky = ky * m.mu;
    double J = model == MODEL_QR_STABLE_NEOHOOKEAN ? tau_qrnh(m, F, g, tau, effective != 0) : det3(F);
    if (model == MODEL_NEOHOOKEAN_BORDEN) tau_nhb(m, F, effective ? 1.0 : g, tau);
    if (model == MODEL_COROTATED) tau_corotated(m, F, tau);
    return J;
}
void shim_qr(const double* F, double* Q, double* R) { givens_qr3(F, Q, R); }
double shim_damage2(int model, double E, double nu, double alpha, double l0, double eta, double zeta, double k, const double* F, double d, double lap,
    double sc, double dt)
{
    Material<double> m = mat<double>(model, E, nu);
    m.damage = 1;
    m.alpha = alpha;
    m.l0 = l0;
    m.eta = eta;
    m.zeta = zeta;
    m.residual = k;
    bool fb = false;
    return damage_update(m, F, d, lap, sc, dt, fb);
}
double shim_damage(double E, double nu, double alpha, double l0, double eta, double zeta, double k, const double* F, double d, double lap, double sc,
    double dt)
{
    Material<double> m = mat<double>(MODEL_NEOHOOKEAN_BORDEN, E, nu);
    m.damage = 1;
    m.alpha = alpha;
    m.l0 = l0;
    m.eta = eta;
    m.zeta = zeta;
    m.residual = k;
    bool fb = false;
    return damage_update(m, F, d, lap, sc, dt, fb);
}
int shim_key(int prec, int i, int j, int k, unsigned id, unsigned long long* key)
{
    *key = prec == 4 ? SpLayout<6>::key(i, j, k, id) : SpLayout<7>::key(i, j, k, id);
    return 0;
}

// one grid node through the scene's collision objects (collide): objs as in the oracle's orc_collide,
// origin[3] normal[3] velocity[3] friction type per object (normal normalised as the engine does)
void shim_collide(int prec, int n_obj, const double* objs, double time, const double* x, double* v)
{
    auto run = [&](auto zero) {
        using T = decltype(zero);
        SceneParams<T> sp{};
        sp.n_objects = n_obj;
        for (int k = 0; k < n_obj; k++) {
            const double* o = objs + 11 * k;
            double nn = std::sqrt(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
            for (int a = 0; a < 3; a++) {
                sp.objects[k].origin[a] = (T)o[a];
                sp.objects[k].normal[a] = (T)(o[3 + a] / nn);
                sp.objects[k].vel[a] = (T)o[6 + a];
            }
            sp.objects[k].friction = (T)o[9];
            sp.objects[k].type = (int)o[10];
        }
        T xt[3] = { (T)x[0], (T)x[1], (T)x[2] }, vt[3] = { (T)v[0], (T)v[1], (T)v[2] };
        collide(sp, (T)time, xt, vt);
        for (int a = 0; a < 3; a++) v[a] = (double)vt[a];
    };
    if (prec == 4)
        run(0.0f);
    else
        run(0.0);
}

// the damage drive D~ = zeta <phi - 1> of one particle (damage_drive) for model 1 (Borden) or 2 (QR-stable, fibre
// stiffness kx = kx_scale mu)
double shim_drive(int prec, int model, double E, double nu, double kx_scale, double alpha, double zeta, double sigma_c, const double* F)
{
    auto run = [&](auto zero) -> double {
        using T = decltype(zero);
        Material<T> m = mat<T>(model, E, nu);
        m.kx = (T)kx_scale * m.mu;
        m.damage = 1;
        m.alpha = (T)alpha;
        m.zeta = (T)zeta;
        T f[9];
        for (int i = 0; i < 9; i++) f[i] = (T)F[i];
        bool fb = false;
        return (double)damage_drive(m, f, (T)sigma_c, fb);
    };
    return prec == 4 ? run(0.0f) : run(0.0);
}
}
