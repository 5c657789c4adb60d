// Per-particle and per-node physics of the explicit MPM substep, written for the GPU (also compiles as
// plain C++ so the same code can be exercised on the host). Matrices are row-major T[9].
#pragma once
#include "common.cuh"
#include <cmath>
#include <cfloat>
#include <limits>

namespace zr {

template <class T>
struct Eps;
template <>
struct Eps<float> {
    static constexpr float polar_tol = 3e-4f; // Newton stops once a step changes X by less (quadratic phase)
    static constexpr int polar_iters = 12;
    static constexpr float polar_kappa = 1e3f; // condition bound above which FP64 takes over
};
template <>
struct Eps<double> {
    static constexpr double polar_tol = 1e-8;
    static constexpr int polar_iters = 16;
    static constexpr double polar_kappa = 1e7;
};

// correctly rounded multiply / subtract with no contraction: the base node must match the
// reference's floor(x * (1/dx) - 0.5) bit for bit (BSplines.h:16-20, MpmSimulationBase.cpp:1544-1549)
ZR_HD float mul_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
ZR_HD double mul_rn(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}
ZR_HD float sub_rn(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
ZR_HD double sub_rn(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dsub_rn(a, b);
#else
    volatile double r = a - b;
    return r;
#endif
}

// int_floor: truncate, then step down when truncation rounded up (MathTools.h:15-25)
template <class T>
ZR_HD int int_floor(T x)
{
    int i = (int)x;
    return i - ((T)i > x);
}

// base node of a particle coordinate (in metres) along one axis
template <class T>
ZR_HD int base_node(T X, T inv_dx)
{
    return int_floor(sub_rn(mul_rn(X, inv_dx), (T)0.5));
}

// quadratic B-spline weights and derivatives of the three nodes base..base+2 (BSplines.h:73-100)
template <class T>
ZR_HD void bspline_w(T xs, int base, T w[3], T dw[3])
{
    T d0 = xs - (T)base;
    T z = (T)1.5 - d0;
    T d1 = d0 - (T)1;
    T zz = d0 - (T)0.5;
    w[0] = (T)0.5 * z * z;
    w[1] = (T)0.75 - d1 * d1;
    w[2] = (T)0.5 * zz * zz;
    dw[0] = -z;
    dw[1] = (T)-2 * d1;
    dw[2] = zz;
}

// ------------------------------------------------------------------------------------------------
// 3x3 helpers
// ------------------------------------------------------------------------------------------------
template <class T>
ZR_HD T det3(const T* F)
{
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}
// J F^{-T} (DenseExt.h:241-252)
template <class T>
ZR_HD void cofactor3(const T* F, T* A)
{
    A[0] = F[4] * F[8] - F[5] * F[7];
    A[1] = F[5] * F[6] - F[3] * F[8];
    A[2] = F[3] * F[7] - F[4] * F[6];
    A[3] = F[2] * F[7] - F[1] * F[8];
    A[4] = F[0] * F[8] - F[2] * F[6];
    A[5] = F[1] * F[6] - F[0] * F[7];
    A[6] = F[1] * F[5] - F[2] * F[4];
    A[7] = F[2] * F[3] - F[0] * F[5];
    A[8] = F[0] * F[4] - F[1] * F[3];
}
template <class T>
ZR_HD void mul3(const T* A, const T* B, T* R)
{
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) R[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
}
template <class T>
ZR_HD void mul3_bt(const T* A, const T* B, T* R) // A B^T
{
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) R[3 * r + c] = A[3 * r] * B[3 * c] + A[3 * r + 1] * B[3 * c + 1] + A[3 * r + 2] * B[3 * c + 2];
}

ZR_HD float rcbrt_(float x)
{
#if defined(__CUDA_ARCH__)
    return rcbrtf(x);
#else
    return 1.0f / std::cbrt(x);
#endif
}
ZR_HD double rcbrt_(double x)
{
#if defined(__CUDA_ARCH__)
    return rcbrt(x);
#else
    return 1.0 / std::cbrt(x);
#endif
}

// ------------------------------------------------------------------------------------------------
// Robust FP64 SVD by one-sided (Hestenes) Jacobi, with Ziran's sign convention: U and V proper
// rotations, |s0| >= |s1| >= |s2|, only s2 may be negative (ImplicitQRSVD.h:455-460 contract).
// Used when the FP32/FP64 Newton polar iteration is not applicable (inverted or ill-conditioned F).
// ------------------------------------------------------------------------------------------------
ZR_HD void svd3_jacobi(const double* A, double* U, double* s, double* V)
{
    double W[9], Vm[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 };
    for (int i = 0; i < 9; i++) W[i] = A[i];
    for (int sweep = 0; sweep < 30; sweep++) {
        double off = 0;
        for (int pq = 0; pq < 3; pq++) {
            int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            double a = 0, b = 0, g = 0;
            for (int r = 0; r < 3; r++) {
                a += W[3 * r + p] * W[3 * r + p];
                b += W[3 * r + q] * W[3 * r + q];
                g += W[3 * r + p] * W[3 * r + q];
            }
            double ab = sqrt(a * b);
            if (ab == 0 || fabs(g) <= 1e-17 * ab) continue;
            off = fmax(off, fabs(g) / ab);
            double zeta = (b - a) / (2 * g);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
            double c = 1 / sqrt(1 + t * t), sn = c * t;
            for (int r = 0; r < 3; r++) {
                double wp = W[3 * r + p], wq = W[3 * r + q];
                W[3 * r + p] = c * wp - sn * wq;
                W[3 * r + q] = sn * wp + c * wq;
                double vp = Vm[3 * r + p], vq = Vm[3 * r + q];
                Vm[3 * r + p] = c * vp - sn * vq;
                Vm[3 * r + q] = sn * vp + c * vq;
            }
        }
        if (off < 1e-15) break;
    }
    double sg[3];
    for (int c = 0; c < 3; c++) sg[c] = sqrt(W[c] * W[c] + W[3 + c] * W[3 + c] + W[6 + c] * W[6 + c]);
    // sort columns by decreasing singular value (swap in W and V together)
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2 - i; j++)
            if (sg[j] < sg[j + 1]) {
                double t = sg[j];
                sg[j] = sg[j + 1];
                sg[j + 1] = t;
                for (int r = 0; r < 3; r++) {
                    t = W[3 * r + j];
                    W[3 * r + j] = W[3 * r + j + 1];
                    W[3 * r + j + 1] = t;
                    t = Vm[3 * r + j];
                    Vm[3 * r + j] = Vm[3 * r + j + 1];
                    Vm[3 * r + j + 1] = t;
                }
            }
    if (det3(Vm) < 0) // keep V a proper rotation; negating a column of both W and V leaves A unchanged
        for (int r = 0; r < 3; r++) {
            Vm[3 * r + 2] = -Vm[3 * r + 2];
            W[3 * r + 2] = -W[3 * r + 2];
        }
    const double tiny = 1e-150;
    double Um[9];
    // first column
    if (sg[0] > tiny)
        for (int r = 0; r < 3; r++) Um[3 * r] = W[3 * r] / sg[0];
    else {
        Um[0] = 1;
        Um[3] = 0;
        Um[6] = 0;
    }
    // second column, orthogonal to the first
    if (sg[1] > tiny * fmax(1.0, sg[0]))
        for (int r = 0; r < 3; r++) Um[3 * r + 1] = W[3 * r + 1] / sg[1];
    else {
        double u0 = Um[0], u1 = Um[3], u2 = Um[6];
        double px, py, pz;
        if (fabs(u0) < 0.9) { px = 0; py = -u2; pz = u1; } // u x e0
        else { px = u2; py = 0; pz = -u0; } // u x e1
        double nn = sqrt(px * px + py * py + pz * pz);
        Um[1] = px / nn;
        Um[4] = py / nn;
        Um[7] = pz / nn;
    }
    // third column completes a right-handed frame; the sign of s2 follows from W
    double cx = Um[3] * Um[7] - Um[6] * Um[4];
    double cy = Um[6] * Um[1] - Um[0] * Um[7];
    double cz = Um[0] * Um[4] - Um[3] * Um[1];
    double proj = cx * W[2] + cy * W[5] + cz * W[8];
    Um[2] = cx;
    Um[5] = cy;
    Um[8] = cz;
    sg[2] = proj; // negative when det(A) < 0: the sign sits on the smallest singular value
    for (int i = 0; i < 9; i++) {
        U[i] = Um[i];
        V[i] = Vm[i];
    }
    s[0] = sg[0];
    s[1] = sg[1];
    s[2] = sg[2];
}

// Rotation of the polar decomposition F = R S (ImplicitQRSVD.h:546-558: R = U V^T of Ziran's SVD).
// Determinant-scaled Newton iteration X <- (g X + X^{-T}/g)/2 in T; it converges quadratically to R
// whenever det F > 0. Inverted, nearly singular or ill-conditioned F goes to the FP64 SVD.
// Returns true when the FP64 path was taken.
// One Newton step of the polar iteration on the 9 entries, X <- a X + b Cf, returning |step|^2, and the cofactor
// of the new X. On Blackwell the FP32 form runs two entries per instruction (__ffma2_rn, __fmul2_rn; each lane
// rounds as the scalar operation); FP64 and host builds keep scalar arithmetic.
template <class T>
ZR_HD T newton_step(T* X, T* Cf, T a, T b)
{
    T diff = 0;
    for (int i = 0; i < 9; i++) {
        const T xn = a * X[i] + b * Cf[i];
        const T dd = xn - X[i];
        diff += dd * dd;
        X[i] = xn;
    }
    cofactor3(X, Cf);
    return diff;
}
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <>
__device__ __forceinline__ float newton_step<float>(float* X, float* Cf, float a, float b)
{
    const float2 A = make_float2(a, a), Bv = make_float2(b, b);
    float2 d2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const float2 x = make_float2(X[i], X[i + 1]);
        const float2 xn = __ffma2_rn(A, x, __fmul2_rn(Bv, make_float2(Cf[i], Cf[i + 1])));
        const float2 dd = __fadd2_rn(xn, make_float2(-x.x, -x.y));
        d2 = __ffma2_rn(dd, dd, d2);
        X[i] = xn.x;
        X[i + 1] = xn.y;
    }
    const float x8 = a * X[8] + b * Cf[8], d8 = x8 - X[8];
    X[8] = x8;
    // cofactor pairs: (A0, A1) (A2, A3) (A4, A5) (A6, A7) as p q - r s per lane, A8 scalar
    const float2 c01 = __ffma2_rn(make_float2(X[4], X[5]), make_float2(X[8], X[6]), make_float2(-X[5] * X[7], -X[3] * X[8]));
    const float2 c23 = __ffma2_rn(make_float2(X[3], X[2]), make_float2(X[7], X[7]), make_float2(-X[4] * X[6], -X[1] * X[8]));
    const float2 c45 = __ffma2_rn(make_float2(X[0], X[1]), make_float2(X[8], X[6]), make_float2(-X[2] * X[6], -X[0] * X[7]));
    const float2 c67 = __ffma2_rn(make_float2(X[1], X[2]), make_float2(X[5], X[3]), make_float2(-X[2] * X[4], -X[0] * X[5]));
    Cf[0] = c01.x;
    Cf[1] = c01.y;
    Cf[2] = c23.x;
    Cf[3] = c23.y;
    Cf[4] = c45.x;
    Cf[5] = c45.y;
    Cf[6] = c67.x;
    Cf[7] = c67.y;
    Cf[8] = X[0] * X[4] - X[1] * X[3];
    return d2.x + d2.y + d8 * d8;
}
#endif

// The FP64 path of polar_rotation, kept out of line: it is rare, and inlining it into every kernel that
// decomposes F would crowd the instruction cache of the hot loops.
template <class T>
ZR_COLD void polar_rotation_fp64(const T* F, T* R)
{
    double A[9], U[9], s[3], V[9];
    for (int i = 0; i < 9; i++) A[i] = (double)F[i];
    svd3_jacobi(A, U, s, V);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) R[3 * r + c] = (T)(U[3 * r] * V[3 * c] + U[3 * r + 1] * V[3 * c + 1] + U[3 * r + 2] * V[3 * c + 2]);
}

template <class T>
ZR_HD bool polar_rotation(const T* F, T* R)
{
    T X[9], Cf[9];
    for (int i = 0; i < 9; i++) X[i] = F[i];
    bool ok = false;
    {
        cofactor3(X, Cf);
        T J = X[0] * Cf[0] + X[1] * Cf[1] + X[2] * Cf[2];
        T nf = 0, nc = 0;
        for (int i = 0; i < 9; i++) {
            nf += X[i] * X[i];
            nc += Cf[i] * Cf[i];
        }
        // Frobenius condition number ||F|| ||F^-1|| = sqrt(nf nc) / J
        if (J > 0 && nf * nc < (Eps<T>::polar_kappa * Eps<T>::polar_kappa) * (J * J)) {
            for (int it = 0; it < Eps<T>::polar_iters; it++) {
                T g = rcbrt_(J);
                T a = (T)0.5 * g, b = (T)0.5 / (g * J);
                const T diff = newton_step(X, Cf, a, b);
                if (diff < Eps<T>::polar_tol * Eps<T>::polar_tol) {
                    ok = true;
                    break;
                }
                J = X[0] * Cf[0] + X[1] * Cf[1] + X[2] * Cf[2];
                if (!(J > 0)) break;
            }
        }
    }
    if (ok) {
        for (int i = 0; i < 9; i++) R[i] = X[i];
        return false;
    }
    polar_rotation_fp64(F, R);
    return true;
}

// Tensile part sigma+ = sum_i <lambda_i>_+ q_i q_i^T of a symmetric 3x3 matrix (the quantity
// AnisoFractureSimulation.h:240-254 builds from an eigen-decomposition). Eigenvalues come from the
// trigonometric closed form; at most one eigenvector is needed: with one positive eigenvalue
// sigma+ = l1 q1 q1^T, with two sigma+ = S - l3 q3 q3^T, each eigenvector taken as the largest cross
// product of two rows of (S - l I). When that eigenvalue is close to another one, it is also close to
// zero (the other lies on the far side of zero), so the error of its eigenvector is scaled by a small
// eigenvalue: sigma+ stays accurate.
template <class T>
ZR_HD void eig_vec_of(const T* S, T l, T* q)
{
    const T r0[3] = { S[0] - l, S[1], S[2] }, r1[3] = { S[3], S[4] - l, S[5] }, r2[3] = { S[6], S[7], S[8] - l };
    // the three row cross products; keep the longest (selects, no dynamic indexing)
    const T a0 = r0[1] * r1[2] - r0[2] * r1[1], a1 = r0[2] * r1[0] - r0[0] * r1[2], a2 = r0[0] * r1[1] - r0[1] * r1[0];
    const T b0 = r0[1] * r2[2] - r0[2] * r2[1], b1 = r0[2] * r2[0] - r0[0] * r2[2], b2 = r0[0] * r2[1] - r0[1] * r2[0];
    const T e0 = r1[1] * r2[2] - r1[2] * r2[1], e1 = r1[2] * r2[0] - r1[0] * r2[2], e2 = r1[0] * r2[1] - r1[1] * r2[0];
    const T na = a0 * a0 + a1 * a1 + a2 * a2, nb = b0 * b0 + b1 * b1 + b2 * b2, ne = e0 * e0 + e1 * e1 + e2 * e2;
    T q0 = a0, q1 = a1, q2 = a2, nk = na;
    if (nb > nk) {
        q0 = b0;
        q1 = b1;
        q2 = b2;
        nk = nb;
    }
    if (ne > nk) {
        q0 = e0;
        q1 = e1;
        q2 = e2;
        nk = ne;
    }
    if (!(nk > (T)0)) {
        q[0] = (T)1;
        q[1] = q[2] = (T)0;
        return;
    }
    const T inv = (T)1 / sqrt(nk);
    q[0] = q0 * inv;
    q[1] = q1 * inv;
    q[2] = q2 * inv;
}

template <class T>
ZR_HD void tension_part(const T* S, T* Sp)
{
    const T s00 = S[0], s11 = S[4], s22 = S[8];
    const T s01 = (T)0.5 * (S[1] + S[3]), s02 = (T)0.5 * (S[2] + S[6]), s12 = (T)0.5 * (S[5] + S[7]);
    const T Ssym[9] = { s00, s01, s02, s01, s11, s12, s02, s12, s22 };
    const T q = (s00 + s11 + s22) * ((T)1 / (T)3);
    const T p1 = s01 * s01 + s02 * s02 + s12 * s12;
    const T a = s00 - q, b = s11 - q, c = s22 - q;
    const T p2 = a * a + b * b + c * c + (T)2 * p1;
    T l1, l2, l3;
    const T p = sqrt(p2 * ((T)1 / (T)6));
    if (!(p > std::numeric_limits<T>::epsilon() * (fabs(q) + std::numeric_limits<T>::min()))) {
        l1 = l2 = l3 = q; // a multiple of the identity
    }
    else {
        const T ip = (T)1 / p;
        const T B00 = a * ip, B11 = b * ip, B22 = c * ip, B01 = s01 * ip, B02 = s02 * ip, B12 = s12 * ip;
        T r = (T)0.5 * (B00 * (B11 * B22 - B12 * B12) - B01 * (B01 * B22 - B12 * B02) + B02 * (B01 * B12 - B11 * B02));
        r = r < (T)-1 ? (T)-1 : (r > (T)1 ? (T)1 : r);
        const T phi = acos(r) * ((T)1 / (T)3);
        l1 = q + (T)2 * p * cos(phi);
        l3 = q + (T)2 * p * cos(phi + (T)2.0943951023931954923);
        l2 = (T)3 * q - l1 - l3;
    }
    if (l3 >= (T)0) { // all tensile
        for (int i = 0; i < 9; i++) Sp[i] = Ssym[i];
        return;
    }
    if (l1 <= (T)0) { // all compressive
        for (int i = 0; i < 9; i++) Sp[i] = (T)0;
        return;
    }
    T v[3];
    if (l2 <= (T)0) { // one tensile direction
        eig_vec_of(Ssym, l1, v);
        for (int r0 = 0; r0 < 3; r0++)
            for (int c0 = 0; c0 < 3; c0++) Sp[3 * r0 + c0] = l1 * v[r0] * v[c0];
    }
    else { // two tensile directions: remove the compressive one
        eig_vec_of(Ssym, l3, v);
        for (int r0 = 0; r0 < 3; r0++)
            for (int c0 = 0; c0 < 3; c0++) Sp[3 * r0 + c0] = Ssym[3 * r0 + c0] - l3 * v[r0] * v[c0];
    }
}

// ------------------------------------------------------------------------------------------------
// Constitutive models. Both return the Kirchhoff stress tau; FBasedMpmForceHelper multiplies by V0
// (FBasedMpmForceHelper.cpp:43-63).
// ------------------------------------------------------------------------------------------------
// Fixed corotated: P = 2 mu (F - R) + lambda (J-1) J F^{-T}, tau = P F^T
// (CorotatedElasticity.cpp:56-76, HyperelasticConstitutiveModel.h:75-80)
template <class T>
ZR_HD bool tau_corotated(const Material<T>& mt, const T* F, T* tau)
{
    T R[9], Cf[9], P[9];
    bool fb = polar_rotation(F, R);
    cofactor3(F, Cf);
    T J = det3(F);
    T a = (T)2 * mt.mu, b = mt.lambda * (J - (T)1);
    for (int i = 0; i < 9; i++) P[i] = a * (F[i] - R[i]) + b * Cf[i];
    mul3_bt(P, F, tau);
    return fb;
}

// Neo-Hookean (Borden): tau = g (tau_dev + tau_vol) for J >= 1, g tau_dev + tau_vol otherwise
// (NeoHookeanBorden.cpp:71-94); kappa = 0.666666 mu + lambda (NeoHookeanBorden.cpp:20)
template <class T>
ZR_HD void tau_nhb(const Material<T>& mt, const T* F, T g, T* tau)
{
    T B[9];
    mul3_bt(F, F, B);
    T J = det3(F);
    T tr3 = (B[0] + B[4] + B[8]) * ((T)1 / (T)3);
    T rc = rcbrt_(J);
    T s = J > (T)0 ? mt.mu * (rc * rc) : (T)NAN; // mu J^{-2/3}; pow() of a negative J is NaN in the reference too
    T vol = J * (mt.kappa * (T)0.5 * (J - (T)1 / J));
    bool tension = J >= (T)1;
    T gd = g * s, gv = tension ? g * vol : vol;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) tau[3 * r + c] = gd * (B[3 * r + c] - (r == c ? tr3 : (T)0)) + (r == c ? gv : (T)0);
}

// Givens QR of a 3x3 matrix, F = Q R, with Ziran's rotation order (GivensQR.h: for each column j, rows
// i = 2 .. j+1 bottom-up, a rotation of rows (i-1, i) zeroing R(i, j), applied to R and accumulated into
// Q^T) and the sign convention of QRStableNeoHookean::updateScratch (QRStableNeoHookean.h:102-122): R(0,0)
// and R(1,1) made non-negative by flipping a column of Q with the matching row of R and, to keep Q a
// rotation, column 2 of Q with R(2,2).
template <class T>
ZR_HD void givens_qr3(const T* F, T* Q, T* R)
{
    T M[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 }; // Q^T
    for (int i = 0; i < 9; i++) R[i] = F[i];
    for (int j = 0; j < 3; j++)
        for (int i = 2; i > j; i--) {
            // rotation (c -s; s c) of rows (i-1, i) with (c -s; s c) (a; b) = (r; 0) (Givens.h GivensRotation)
            const T a = R[3 * (i - 1) + j], b = R[3 * i + j];
            const T d = a * a + b * b;
            T c = 1, sn = 0;
            if (d != (T)0) {
                const T t = (T)1 / sqrt(d);
                c = a * t;
                sn = -b * t;
            }
            for (int k = 0; k < 3; k++) {
                const T r1 = R[3 * (i - 1) + k], r2 = R[3 * i + k];
                R[3 * (i - 1) + k] = c * r1 - sn * r2;
                R[3 * i + k] = sn * r1 + c * r2;
                const T m1 = M[3 * (i - 1) + k], m2 = M[3 * i + k];
                M[3 * (i - 1) + k] = c * m1 - sn * m2;
                M[3 * i + k] = sn * m1 + c * m2;
            }
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Q[3 * r + c] = M[3 * c + r];
    if (R[0] < (T)0) {
        R[0] = -R[0];
        R[1] = -R[1];
        R[2] = -R[2];
        R[8] = -R[8];
        for (int r = 0; r < 3; r++) {
            Q[3 * r] = -Q[3 * r];
            Q[3 * r + 2] = -Q[3 * r + 2];
        }
    }
    if (R[4] < (T)0) {
        R[4] = -R[4];
        R[5] = -R[5];
        R[8] = -R[8];
        for (int r = 0; r < 3; r++) {
            Q[3 * r + 1] = -Q[3 * r + 1];
            Q[3 * r + 2] = -Q[3 * r + 2];
        }
    }
}

// QR-stable Neo-Hookean with fibre stiffness (QRStableNeoHookean.h:102-173, QrBasedHelper.h:30-40): with
// F = Q R, J = r00 r11 r22 and the energy
//   psi = [g] lambda/2 (J-1)^2 + g (mu/2 (sum_{i<=j} r_ij^2 - 3) - mu (J-1)) + kx/2 (r00-1)^2
//         + ky/2 (sqrt(r01^2 + r11^2) - 1)^2,
// where the volume term is degraded only when J >= 1 and the fibre terms never, D = dpsi/dR (upper
// triangular) and A = D R^T with its lower triangle mirrored from the upper, P = Q A R^{-T}. The Kirchhoff
// stress P F^T (HyperelasticConstitutiveModel.h:75-80) is then Q A Q^T, evaluated here in that form (no
// inverse of R). With effective = true the model is undegraded and isotropic (g = 1, kx = ky = 0), as
// evaluateEffectiveCauchyStress uses it (QRStableNeoHookean.h:86-96). Returns J.
template <class T>
ZR_HD T tau_qrnh(const Material<T>& mt, const T* F, T g, T* tau, bool effective = false)
{
    T Q[9], R[9];
    givens_qr3(F, Q, R);
    const T J = R[0] * R[4] * R[8];
    const T kx = effective ? (T)0 : mt.kx, ky = effective ? (T)0 : mt.ky;
    if (effective) g = (T)1;
    T D[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 };
    const T lam = (J >= (T)1 ? g : (T)1) * mt.lambda * (J - (T)1) * J;
    for (int i = 0; i < 3; i++) D[4 * i] += lam / R[4 * i];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) D[3 * i + j] += g * mt.mu * R[3 * i + j];
    for (int i = 0; i < 3; i++) D[4 * i] -= g * mt.mu * J / R[4 * i];
    D[0] += kx * (R[0] - (T)1);
    if (ky != (T)0) {
        const T ss = sqrt(R[1] * R[1] + R[4] * R[4]);
        D[1] += ky * (ss - (T)1) * R[1] / ss;
        D[4] += ky * (ss - (T)1) * R[4] / ss;
    }
    T A[9];
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) { // (D R^T)_ij = sum_k D_ik R_jk, D upper triangular
            T acc = 0;
            for (int k = j; k < 3; k++) acc += D[3 * i + k] * R[3 * j + k];
            A[3 * i + j] = acc;
            A[3 * j + i] = acc;
        }
    T QA[9];
    mul3(Q, A, QA);
    mul3_bt(QA, Q, tau);
    return J;
}

// degradation g(d) = (1-d)^2 (1-k) + k (AnisoFractureSimulation.h:279-280)
template <class T>
ZR_HD T degradation(T d, T k)
{
    return (((T)1 - d) * ((T)1 - d)) * ((T)1 - k) + k;
}

// The damage drive D~ = zeta <phi - 1> of one particle, phi = (A sigma+) : (sigma+ A) / sigma_c^2 with the
// undegraded Cauchy stress's tensile part sigma+ and the structural tensor A = I + alpha (R e1)(R e1)^T, R the
// rotation of F = R S (AnisoFractureSimulation.h:224-270, :365-391; updateDTildeHelper :292-333 for the implicit
// solve).
//
// For the Borden model the polar decomposition is not needed. Its stress is an isotropic function of B = F F^T, and
// B = R C R^T with C = F^T F = S^2, so sigma(F) = R sigma~ R^T where sigma~ is the same formula evaluated on C
// (tau_nhb of F^T), and sigma+ = R sigma~+ R^T. The contraction is invariant under that rotation, and
// R^T A R = I + alpha e1 e1^T = diag(w) with w = (1 + alpha, 1, 1). So phi sigma_c^2 = sum_ij w_i w_j (sigma~+_ij)^2.
// This is the same quantity with different rounding. The QR-stable model's fibre term makes its stress
// anisotropic, so it keeps the polar rotation.
template <class T>
ZR_HD T damage_drive(const Material<T>& mt, const T* F, T sigma_c, bool& fallback)
{
    T tau[9], invJ;
    const bool qr = mt.model == MODEL_QR_STABLE_NEOHOOKEAN;
    if (qr) {
        invJ = (T)1 / tau_qrnh(mt, F, (T)1, tau, true); // cauchy = P F^T / J with J from the QR (QRStableNeoHookean.h:86-96)
    }
    else {
        const T Ft[9] = { F[0], F[3], F[6], F[1], F[4], F[7], F[2], F[5], F[8] };
        tau_nhb(mt, Ft, (T)1, tau); // tau~ = R^T tau R: the formula on F^T F
        invJ = (T)1 / det3(F);
    }
    T S[9], sp[9], s2 = 0;
    for (int i = 0; i < 9; i++) {
        S[i] = tau[i] * invJ; // undegraded Cauchy stress (in the material frame for the Borden model)
        s2 += S[i] * S[i];
    }
    // phi sigma_c^2 = tr((A sigma+)^2) <= |A|_2^2 |sigma+|_F^2 <= max(1, (1 + alpha)^2) |sigma|_F^2 (A = I + alpha a a^T
    // with |a| = 1; sigma+ keeps a subset of sigma's eigenvalues). Below that bound, with a margin far above
    // rounding, the drive is exactly zero: skip the eigen split (and the polar decomposition).
    const T ap1 = (T)1 + mt.alpha, anorm2 = ap1 * ap1 > (T)1 ? ap1 * ap1 : (T)1;
    if (s2 * anorm2 <= (T)0.999 * sigma_c * sigma_c) {
        fallback = false;
        return (T)0;
    }
    tension_part(S, sp); // sum of Macaulay-bracketed principal stresses times their projectors
    T contraction = 0;
    if (qr) {
        T R[9];
        fallback = polar_rotation(F, R);
        T a[3] = { R[0], R[3], R[6] }; // R e1
        T M[9]; // A sigma+ with A = I + alpha a a^T
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                T as = a[0] * sp[c] + a[1] * sp[3 + c] + a[2] * sp[6 + c];
                M[3 * r + c] = sp[3 * r + c] + mt.alpha * a[r] * as;
            }
        // (A sigma+) : (sigma+ A) = sum_ij M_ij M_ji since sigma+ A = (A sigma+)^T
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) contraction += M[3 * r + c] * M[3 * c + r];
    }
    else {
        fallback = false;
        // sum_ij w_i w_j sp_ij^2, w = (1 + alpha, 1, 1): the first row and column carry 1 + alpha once each
        const T s00 = sp[0], s01 = sp[1], s02 = sp[2], s11 = sp[4], s12 = sp[5], s22 = sp[8];
        contraction = ap1 * ap1 * (s00 * s00) + (T)2 * ap1 * (s01 * s01 + s02 * s02) + (s11 * s11 + s22 * s22) + (T)2 * (s12 * s12);
    }
    T phi = contraction / (sigma_c * sigma_c);
    return mt.zeta * (phi > (T)1 ? phi - (T)1 : (T)0);
}

// Explicit AnisoMPM damage update of one particle (AnisoFractureSimulation.h:210-283, :365-391) with one
// structural director a0 = e1 rotated by the polar R of F. Returns the new damage.
template <class T>
ZR_HD T damage_update(const Material<T>& mt, const T* F, T d, T lap, T sigma_c, T dt, bool& fallback)
{
    // fully damaged: d + (dt/eta) <...> >= d >= 1 and the update is capped at 1, whatever the drive is
    if (d >= (T)1) {
        fallback = false;
        return (T)1;
    }
    T geo = d - mt.l0 * mt.l0 * lap;
    T dtilde = damage_drive(mt, F, sigma_c, fallback);
    T diff = ((T)1 - d) * dtilde - geo;
    T nd = d + (dt / mt.eta) * (diff > (T)0 ? diff : (T)0);
    return nd < (T)1 ? nd : (T)1;
}

// Analytic translating half-spaces at a grid node (AnalyticCollisionObject::multiObjectCollision and
// detectAndResolveCollision, CollisionObject.cpp:67-105, :342-406; HalfSpace, AnalyticLevelSet.cpp:318-334).
// Objects apply in order: a STICKY hit sets the object's velocity and ends the loop; a SLIP hit removes the
// normal part of the relative velocity, a SEPARATE hit only an approaching one, both with kinetic friction.
// Every SLIP or SEPARATE hit adds its normal to a basis, orthogonalised against the earlier ones (Gram-Schmidt,
// a parallel normal adds nothing); once the basis holds three normals the loop ends.
template <class T>
ZR_HD void collide(const SceneParams<T>& sp, T time, const T* x, T* v)
{
    T basis[3][3];
    int nslip = 0;
    for (int k = 0; k < sp.n_objects; k++) {
        const HalfSpaceObj<T>& h = sp.objects[k];
        T phi = h.normal[0] * (x[0] - h.vel[0] * time - h.origin[0]) + h.normal[1] * (x[1] - h.vel[1] * time - h.origin[1])
            + h.normal[2] * (x[2] - h.vel[2] * time - h.origin[2]);
        if (!(phi <= (T)0)) continue;
        T r[3] = { v[0] - h.vel[0], v[1] - h.vel[1], v[2] - h.vel[2] };
        if (h.type == OBJ_STICKY) {
            v[0] = h.vel[0];
            v[1] = h.vel[1];
            v[2] = h.vel[2];
            break;
        }
        T dot = r[0] * h.normal[0] + r[1] * h.normal[1] + r[2] * h.normal[2];
        if (h.type == OBJ_SLIP || dot < (T)0) {
            for (int a = 0; a < 3; a++) r[a] -= h.normal[a] * dot;
            if (h.friction != (T)0 && dot < (T)0) {
                T vn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                if (-dot * h.friction < vn) {
                    T sc = dot * h.friction / vn;
                    for (int a = 0; a < 3; a++) r[a] += r[a] * sc;
                }
                else
                    r[0] = r[1] = r[2] = (T)0;
            }
        }
        for (int a = 0; a < 3; a++) v[a] = r[a] + h.vel[a];
        T nv[3] = { h.normal[0], h.normal[1], h.normal[2] };
        for (int c = 0; c < nslip; c++) {
            const T d = basis[c][0] * nv[0] + basis[c][1] * nv[1] + basis[c][2] * nv[2];
            for (int a = 0; a < 3; a++) nv[a] -= d * basis[c][a];
        }
        const T len = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        if (len != (T)0) {
            for (int a = 0; a < 3; a++) basis[nslip][a] = nv[a] / len;
            if (++nslip == 3) break;
        }
    }
}

} // namespace zr
