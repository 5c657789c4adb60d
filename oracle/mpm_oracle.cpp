// =====================================================================================================
// TEST INFRASTRUCTURE — the CPU oracle. Not product code.
//
// A CPU restatement of Ziran's explicit MPM substep (Lib/MPM over Lib/SPGrid, driven by
// Projects/anisofracture), written from the reference's algorithm, not copied from it. Only the
// tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and only as the
// checker (or as the timed CPU baseline); the product path never calls it.
//
// Scope of the restatement (reference file:line in each block below):
//   * SPGrid bit-interleaved offsets and Packed_Add        Lib/SPGrid/Core/SPGrid_Mask.h:22-48,76-80,119-245
//   * particle binning / sort keys / groups / pollute      Lib/MPM/MpmSimulationBase.cpp:1531-1573, MpmGrid.h:153-193
//   * quadratic B-spline weights, int_floor                Ziran/Math/Splines/BSplines.h:16-20,73-100, MathTools.h:15-25
//   * stress  V0*tau(F)                                    Lib/MPM/Force/FBasedMpmForceHelper.cpp:43-63
//       - fixed corotated                                  Physics/ConstitutiveModel/CorotatedElasticity.cpp:16-21,56-76
//       - Neo-Hookean (Borden) with degradation g          Physics/ConstitutiveModel/NeoHookeanBorden.cpp:16-108
//       - 3x3 implicit-QR SVD (Wilkinson shift) + polar    Math/Linear/ImplicitQRSVD.h:219-558, Givens.h:33-270
//   * APIC P2G, 8-colour block schedule                    MpmSimulationBase.cpp:618-855
//   * grid velocity update + analytic half-space BCs       MpmSimulationBase.cpp:1179-1228,
//                                                          Math/Geometry/CollisionObject.cpp:67-105,342-406,
//                                                          Math/Geometry/AnalyticLevelSet.cpp:318-363
//   * G2P (APIC/RPIC blend), x update, CFL flags, F update MpmSimulationBase.cpp:1269-1515, FBasedMpmForceHelper.cpp:95-108
//   * explicit AnisoMPM damage                             Projects/anisofracture/AnisoFractureSimulation.h:129-283,365-391
//   * substep ordering                                     MpmSimulationBase.cpp:262-357
//   * FP64-accumulated reductions                          Lib/MPM/MpmSimulationDataAnalysis.h:67-151
//
// Determinism: every scatter runs in the reference's order (colour-major, then group, then sorted
// particle, then the 27 stencil nodes in i,j,k order). Groups of one colour never touch the same
// node, so running them on several threads gives the same bits as running them on one.
//
// Arithmetic order. For T=float the transfers follow the reference's SSE/FMA branch
// (MpmSimulationBase.cpp:680-790, :1326-1373) using std::fma; for T=double they follow the
// generic branch as written (left-to-right sums, no contraction: built with -ffp-contract=off).
// The reference binary's own rounding also depends on Eigen's vectorised reductions and GCC's
// contraction, which cannot be reproduced without building it; the oracle fixes one order.
//
// Eigen::EigenSolver (AnisoFractureSimulation.h:244) is replaced by a cyclic Jacobi solver for the
// symmetric Cauchy stress; on symmetric input both give the same sigma+ up to rounding.
// =====================================================================================================
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

namespace orc {

// ----------------------------------------------------------------------------------------------
// SPGrid layout (SPGrid_Mask.h:22-48 page masks, :76-80 element masks, :119-123 aggregate masks)
// GridState is 64 B for float and 128 B for double (MpmGrid.h:16-45), so log2_struct = 6 / 7.
// ----------------------------------------------------------------------------------------------
template <int LOG2_STRUCT>
struct Layout {
    static constexpr int data_bits = LOG2_STRUCT;
    static constexpr int block_bits = 12 - LOG2_STRUCT;
    static constexpr int zbits = block_bits / 3 + (block_bits % 3 > 0);
    static constexpr int ybits = block_bits / 3 + (block_bits % 3 > 1);
    static constexpr int xbits = block_bits / 3;
    static constexpr int page_shift = 3 - block_bits % 3;
    static constexpr uint64_t page_zmask = (0x9249249249249249ULL << page_shift) & ~0xfffULL;
    static constexpr uint64_t page_ymask = (0x2492492492492492ULL << page_shift) & ~0xfffULL;
    static constexpr uint64_t page_xmask = (0x4924924924924924ULL << page_shift) & ~0xfffULL;
    static constexpr uint64_t elem_zmask = ((1ULL << zbits) - 1) << data_bits;
    static constexpr uint64_t elem_ymask = ((1ULL << ybits) - 1) << (data_bits + zbits);
    static constexpr uint64_t elem_xmask = ((1ULL << xbits) - 1) << (data_bits + zbits + ybits);
    static constexpr uint64_t zmask = page_zmask | elem_zmask;
    static constexpr uint64_t ymask = page_ymask | elem_ymask;
    static constexpr uint64_t xmask = page_xmask | elem_xmask;
    static constexpr int index_bits = 32 - block_bits; // MpmSimulationBase.cpp:1535
    static constexpr int sx = 1 << xbits, sy = 1 << ybits, sz = 1 << zbits;
    static constexpr int nodes_per_block = 1 << block_bits;

    // Bit deposit: the low bits of v go, in order, to the set bits of mask (SPGrid_Utilities.h Bit_Spread).
    // A negative value is sign-extended, so all mask bits above its magnitude receive ones.
    struct Positions {
        int pos[64];
        int count;
    };
    static Positions positions(uint64_t mask)
    {
        Positions P{};
        for (int b = 0; b < 64; b++)
            if (mask & (1ULL << b)) P.pos[P.count++] = b;
        return P;
    }
    static uint64_t deposit(int64_t sv, uint64_t mask)
    {
        static const Positions PX = positions(xmask), PY = positions(ymask), PZ = positions(zmask);
        const Positions& P = mask == xmask ? PX : (mask == ymask ? PY : (mask == zmask ? PZ : positions(mask)));
        uint64_t v = (uint64_t)sv, r = 0;
        if (sv < 0) {
            for (int k = 0; k < P.count; k++)
                if (k >= 64 || ((v >> k) & 1)) r |= 1ULL << P.pos[k];
            return r;
        }
        for (int k = 0; v && k < P.count; k++, v >>= 1)
            if (v & 1) r |= 1ULL << P.pos[k];
        return r;
    }
    // Bit extract, the inverse of deposit (SPGrid Bit_Pack).
    static int64_t extract(uint64_t v, uint64_t mask)
    {
        uint64_t r = 0, out = 1;
        for (uint64_t bit = 1; bit; bit <<= 1)
            if (mask & bit) {
                if (v & bit) r |= out;
                out <<= 1;
            }
        return (int64_t)r;
    }
    static uint64_t linear_offset(int i, int j, int k)
    {
        return deposit(i, xmask) | deposit(j, ymask) | deposit(k, zmask);
    }
    static void coord(uint64_t off, int& i, int& j, int& k)
    {
        i = (int)extract(off, xmask);
        j = (int)extract(off, ymask);
        k = (int)extract(off, zmask);
    }
    // SPGrid_Mask.h:237-245
    static uint64_t packed_add(uint64_t a, uint64_t b)
    {
        const uint64_t wmask = xmask | ymask | zmask;
        uint64_t x = ((a | ~xmask) + (b & xmask)) & xmask;
        uint64_t y = ((a | ~ymask) + (b & ymask)) & ymask;
        uint64_t z = ((a | ~zmask) + (b & zmask)) & zmask;
        uint64_t w = ((a | wmask) + (b & ~wmask)) & ~wmask;
        return x | y | z | w;
    }
    // in-block node index = element bits of the offset (z fastest, then y, then x)
    static int element(int lx, int ly, int lz) { return (lx << (zbits + ybits)) | (ly << zbits) | lz; }
};

template <class T>
using LayoutOf = Layout<std::is_same<T, float>::value ? 6 : 7>;

// MathTools.h:15-25
template <class T>
inline int int_floor(T x)
{
    int i = (int)x;
    return i - (i > x);
}

// BSplines.h:73-100 (quadratic), base node BSplines.h:16-20
template <class T>
inline void bspline(T x, int& base, T w[3], T dw[3])
{
    base = int_floor(x - (T)0.5);
    T d0 = x - (T)base;
    T z = (T)1.5 - d0;
    T z2 = z * z;
    w[0] = (T)0.5 * z2;
    T d1 = d0 - (T)1;
    w[1] = (T)0.75 - d1 * d1;
    T d2 = (T)1 - d1;
    T zz = (T)1.5 - d2;
    T zz2 = zz * zz;
    w[2] = (T)0.5 * zz2;
    dw[0] = -z;
    dw[1] = -(T)2 * d1;
    dw[2] = zz;
}

// ----------------------------------------------------------------------------------------------
// 3x3 helpers, row-major M[3*r+c]
// ----------------------------------------------------------------------------------------------
template <class T>
struct M3 {
    T a[9];
    T& operator()(int r, int c) { return a[3 * r + c]; }
    const T& operator()(int r, int c) const { return a[3 * r + c]; }
    static M3 identity()
    {
        M3 m{};
        m(0, 0) = m(1, 1) = m(2, 2) = 1;
        return m;
    }
};
template <class T>
inline M3<T> mul(const M3<T>& A, const M3<T>& B)
{
    M3<T> R;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            R(r, c) = A(r, 0) * B(0, c) + A(r, 1) * B(1, c) + A(r, 2) * B(2, c);
    return R;
}
template <class T>
inline M3<T> mul_bt(const M3<T>& A, const M3<T>& B) // A * B^T
{
    M3<T> R;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            R(r, c) = A(r, 0) * B(c, 0) + A(r, 1) * B(c, 1) + A(r, 2) * B(c, 2);
    return R;
}
template <class T>
inline T det(const M3<T>& F)
{
    return F(0, 0) * (F(1, 1) * F(2, 2) - F(1, 2) * F(2, 1)) - F(0, 1) * (F(1, 0) * F(2, 2) - F(1, 2) * F(2, 0))
        + F(0, 2) * (F(1, 0) * F(2, 1) - F(1, 1) * F(2, 0));
}
// DenseExt.h:241-252 cofactor matrix J F^{-T}
template <class T>
inline M3<T> cofactor(const M3<T>& F)
{
    M3<T> A;
    A(0, 0) = F(1, 1) * F(2, 2) - F(1, 2) * F(2, 1);
    A(0, 1) = F(1, 2) * F(2, 0) - F(1, 0) * F(2, 2);
    A(0, 2) = F(1, 0) * F(2, 1) - F(1, 1) * F(2, 0);
    A(1, 0) = F(0, 2) * F(2, 1) - F(0, 1) * F(2, 2);
    A(1, 1) = F(0, 0) * F(2, 2) - F(0, 2) * F(2, 0);
    A(1, 2) = F(0, 1) * F(2, 0) - F(0, 0) * F(2, 1);
    A(2, 0) = F(0, 1) * F(1, 2) - F(0, 2) * F(1, 1);
    A(2, 1) = F(0, 2) * F(1, 0) - F(0, 0) * F(1, 2);
    A(2, 2) = F(0, 0) * F(1, 1) - F(0, 1) * F(1, 0);
    return A;
}

// ----------------------------------------------------------------------------------------------
// Givens rotations (Givens.h:33-185) and the implicit-QR 3x3 SVD of Gast et al.
// (ImplicitQRSVD.h:219-558): bidiagonalise with Givens, Wilkinson-shifted implicit QR sweeps until
// one super-diagonal or diagonal entry falls below tol, then a 2x2 SVD and the sign/sort rules that
// put sigma in decreasing magnitude with the only negative value last.
// ----------------------------------------------------------------------------------------------
template <class T>
struct Givens {
    int i, k;
    T c = 1, s = 0;
    Givens(int i_, int k_) : i(i_), k(k_) {}
    void compute(T a, T b) // ( c -s ; s c ) (a ; b) = (* ; 0)
    {
        T d = a * a + b * b;
        c = 1;
        s = 0;
        T sd = std::sqrt(d);
        if (sd != 0) {
            T t = 1 / sd;
            c = a * t;
            s = -b * t;
        }
    }
    void compute_unconventional(T a, T b) // ( c -s ; s c ) (a ; b) = (0 ; *)
    {
        T d = a * a + b * b;
        c = 0;
        s = 1;
        T sd = std::sqrt(d);
        if (sd != 0) {
            T t = 1 / sd;
            s = a * t;
            c = b * t;
        }
    }
    template <int R, int C>
    void rows(T (&A)[R][C]) const
    {
        for (int j = 0; j < C; j++) {
            T t1 = A[i][j], t2 = A[k][j];
            A[i][j] = c * t1 - s * t2;
            A[k][j] = s * t1 + c * t2;
        }
    }
    template <int R, int C>
    void cols(T (&A)[R][C]) const
    {
        for (int j = 0; j < R; j++) {
            T t1 = A[j][i], t2 = A[j][k];
            A[j][i] = c * t1 - s * t2;
            A[j][k] = s * t1 + c * t2;
        }
    }
    void compose(const Givens& o)
    {
        T nc = c * o.c - s * o.s;
        T ns = s * o.c + c * o.s;
        c = nc;
        s = ns;
    }
};

template <class T>
using A33 = T[3][3];

template <class T>
inline void zero_chase(A33<T>& H, A33<T>& U, A33<T>& V)
{
    Givens<T> r1(0, 1);
    r1.compute(H[0][0], H[1][0]);
    Givens<T> r2(1, 2);
    if (H[1][0] != 0)
        r2.compute(H[0][0] * H[0][1] + H[1][0] * H[1][1], H[0][0] * H[0][2] + H[1][0] * H[1][2]);
    else
        r2.compute(H[0][1], H[0][2]);
    r1.rows(H);
    r2.cols(H);
    r2.cols(V);
    Givens<T> r3(1, 2);
    r3.compute(H[1][1], H[2][1]);
    r3.rows(H);
    r1.cols(U);
    r3.cols(U);
}

template <class T>
inline void upper_bidiag(A33<T>& H, A33<T>& U, A33<T>& V)
{
    Givens<T> r(1, 2);
    r.compute(H[1][0], H[2][0]);
    r.rows(H);
    r.cols(U);
    zero_chase(H, U, V);
}

// 2x2 polar + SVD (ImplicitQRSVD.h:44-161)
template <class T>
inline void svd2(T a00, T a01, T a10, T a11, Givens<T>& U, T& s0, T& s1, Givens<T>& V)
{
    T x0 = a00 + a11, x1 = a10 - a01;
    T den = std::sqrt(x0 * x0 + x1 * x1);
    U.c = 1;
    U.s = 0;
    if (den != 0) {
        U.c = x0 / den;
        U.s = -x1 / den;
    }
    // S = U^T-rotation applied to rows of A
    T S00 = U.c * a00 - U.s * a10, S01 = U.c * a01 - U.s * a11;
    T S11 = U.s * a01 + U.c * a11;
    T x = S00, y = S01, z = S11, y2 = y * y, cs, sn;
    if (y2 == 0) {
        cs = 1;
        sn = 0;
        s0 = x;
        s1 = z;
    }
    else {
        T tau = (T)0.5 * (x - z);
        T w = std::sqrt(tau * tau + y2);
        T t = tau > 0 ? y / (tau + w) : y / (tau - w);
        cs = T(1) / std::sqrt(t * t + T(1));
        sn = -t * cs;
        T c2 = cs * cs, csy = 2 * cs * sn * y, s2 = sn * sn;
        s0 = c2 * x - csy + s2 * z;
        s1 = s2 * x + csy + c2 * z;
    }
    if (s0 < s1) {
        std::swap(s0, s1);
        V.c = -sn;
        V.s = cs;
    }
    else {
        V.c = cs;
        V.s = sn;
    }
    U.compose(V);
}

template <class T>
inline T wilkinson_shift(T a1, T b1, T a2)
{
    T d = (T)0.5 * (a1 - a2);
    T bs = b1 * b1;
    return a2 - std::copysign(bs / (std::fabs(d) + std::sqrt(d * d + bs)), d);
}

template <class T>
inline void swap_cols(A33<T>& M, int a, int b)
{
    for (int r = 0; r < 3; r++) std::swap(M[r][a], M[r][b]);
}
template <class T>
inline void negate_col(A33<T>& M, int a)
{
    for (int r = 0; r < 3; r++) M[r][a] = -M[r][a];
}
template <class T>
inline void flip_sign(int i, A33<T>& U, T* s)
{
    s[i] = -s[i];
    negate_col(U, i);
}

template <int t, class T>
inline void process_block(A33<T>& B, A33<T>& U, T* s, A33<T>& V)
{
    int other = (t == 1) ? 0 : 2;
    Givens<T> u(0, 1), v(0, 1);
    s[other] = B[other][other];
    svd2(B[t][t], B[t][t + 1], B[t + 1][t], B[t + 1][t + 1], u, s[t], s[t + 1], v);
    u.i += t;
    u.k += t;
    v.i += t;
    v.k += t;
    u.cols(U);
    v.cols(V);
}

template <class T>
inline void sort0(A33<T>& U, T* s, A33<T>& V)
{
    if (std::fabs(s[1]) >= std::fabs(s[2])) {
        if (s[1] < 0) {
            flip_sign(1, U, s);
            flip_sign(2, U, s);
        }
        return;
    }
    if (s[2] < 0) {
        flip_sign(1, U, s);
        flip_sign(2, U, s);
    }
    std::swap(s[1], s[2]);
    swap_cols(U, 1, 2);
    swap_cols(V, 1, 2);
    if (s[1] > s[0]) {
        std::swap(s[0], s[1]);
        swap_cols(U, 0, 1);
        swap_cols(V, 0, 1);
    }
    else {
        negate_col(U, 2);
        negate_col(V, 2);
    }
}

template <class T>
inline void sort1(A33<T>& U, T* s, A33<T>& V)
{
    if (std::fabs(s[0]) >= s[1]) {
        if (s[0] < 0) {
            flip_sign(0, U, s);
            flip_sign(2, U, s);
        }
        return;
    }
    std::swap(s[0], s[1]);
    swap_cols(U, 0, 1);
    swap_cols(V, 0, 1);
    if (std::fabs(s[1]) < std::fabs(s[2])) {
        std::swap(s[1], s[2]);
        swap_cols(U, 1, 2);
        swap_cols(V, 1, 2);
    }
    else {
        negate_col(U, 1);
        negate_col(V, 1);
    }
    if (s[1] < 0) {
        flip_sign(1, U, s);
        flip_sign(2, U, s);
    }
}

template <class T>
inline void svd3(const M3<T>& A, M3<T>& Uo, T sigma[3], M3<T>& Vo)
{
    T tol = std::is_same<T, float>::value ? (T)128 * std::numeric_limits<T>::epsilon() : (T)1024 * std::numeric_limits<T>::epsilon();
    A33<T> B, U, V;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            B[r][c] = A(r, c);
            U[r][c] = V[r][c] = (r == c);
        }
    upper_bidiag(B, U, V);
    Givens<T> r(0, 1);
    T a1 = B[0][0], b1 = B[0][1], a2 = B[1][1], a3 = B[2][2], b2 = B[1][2];
    T g1 = a1 * b1, g2 = a2 * b2;
    tol *= std::max((T)0.5 * std::sqrt(a1 * a1 + a2 * a2 + a3 * a3 + b1 * b1 + b2 * b2), (T)1);
    while (std::fabs(b2) > tol && std::fabs(b1) > tol && std::fabs(a1) > tol && std::fabs(a2) > tol && std::fabs(a3) > tol) {
        T mu = wilkinson_shift(a2 * a2 + b1 * b1, g2, a3 * a3 + b2 * b2);
        r.compute(a1 * a1 - mu, g1);
        r.cols(B);
        r.cols(V);
        zero_chase(B, U, V);
        a1 = B[0][0];
        b1 = B[0][1];
        a2 = B[1][1];
        a3 = B[2][2];
        b2 = B[1][2];
        g1 = a1 * b1;
        g2 = a2 * b2;
    }
    if (std::fabs(b2) <= tol) {
        process_block<0>(B, U, sigma, V);
        sort0(U, sigma, V);
    }
    else if (std::fabs(b1) <= tol) {
        process_block<1>(B, U, sigma, V);
        sort1(U, sigma, V);
    }
    else if (std::fabs(a2) <= tol) {
        Givens<T> r1(1, 2);
        r1.compute_unconventional(B[1][2], B[2][2]);
        r1.rows(B);
        r1.cols(U);
        process_block<0>(B, U, sigma, V);
        sort0(U, sigma, V);
    }
    else if (std::fabs(a3) <= tol) {
        Givens<T> r1(1, 2);
        r1.compute(B[1][1], B[1][2]);
        r1.cols(B);
        r1.cols(V);
        Givens<T> r2(0, 2);
        r2.compute(B[0][0], B[0][2]);
        r2.cols(B);
        r2.cols(V);
        process_block<0>(B, U, sigma, V);
        sort0(U, sigma, V);
    }
    else if (std::fabs(a1) <= tol) {
        Givens<T> r1(0, 1);
        r1.compute_unconventional(B[0][1], B[1][1]);
        r1.rows(B);
        r1.cols(U);
        Givens<T> r2(0, 2);
        r2.compute_unconventional(B[0][2], B[2][2]);
        r2.rows(B);
        r2.cols(U);
        process_block<1>(B, U, sigma, V);
        sort1(U, sigma, V);
    }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            Uo(a, b) = U[a][b];
            Vo(a, b) = V[a][b];
        }
}

// ImplicitQRSVD.h:546-558: R = U V^T
template <class T>
inline M3<T> polar_rotation(const M3<T>& F)
{
    M3<T> U, V;
    T s[3];
    svd3(F, U, s, V);
    return mul_bt(U, V);
}

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (stands in for Eigen::EigenSolver on the
// symmetric Cauchy stress, AnisoFractureSimulation.h:244-254). Always run in double.
inline void sym_eigen(const double S[3][3], double lam[3], double Q[3][3])
{
    double A[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            A[r][c] = S[r][c];
            Q[r][c] = (r == c);
        }
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (off <= 1e-30 * diag || off == 0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                double apq = A[p][q];
                if (apq == 0) continue;
                double theta = (A[q][q] - A[p][p]) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < 3; k++) { // A <- J^T A J with J rotating (p,q)
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    double qkp = Q[k][p], qkq = Q[k][q];
                    Q[k][p] = c * qkp - s * qkq;
                    Q[k][q] = s * qkp + c * qkq;
                }
            }
    }
    for (int i = 0; i < 3; i++) lam[i] = A[i][i];
}

// ----------------------------------------------------------------------------------------------
// Materials
// ----------------------------------------------------------------------------------------------
enum { MODEL_COROTATED = 0, MODEL_NHB = 1, MODEL_QRNH = 2 };

template <class T>
struct Material {
    int model = MODEL_COROTATED;
    T mu = 0, lambda = 0, kappa = 0;
    T kx = 0, ky = 0; // QRStableNeoHookean fibre stiffness (QRStableNeoHookean.h:98-107)
    bool damage = false;
    T alpha = 0, l0 = 0, eta = 1, zeta = 1, residual = 0;
};

// Corotated: CorotatedElasticity.cpp:16-21 (Lame), :56-76 (P), HyperelasticConstitutiveModel.h:75-80 (tau = P F^T)
template <class T>
inline M3<T> tau_corotated(const Material<T>& mat, const M3<T>& F)
{
    T J = det(F);
    M3<T> JFinvT = cofactor(F);
    M3<T> R = polar_rotation(F);
    M3<T> P;
    for (int a = 0; a < 9; a++) P.a[a] = (T)2 * mat.mu * (F.a[a] - R.a[a]) + mat.lambda * (J - 1) * JFinvT.a[a];
    return mul_bt(P, F);
}

// NeoHookeanBorden.cpp:71-94 kirchhoff(), g = degradation
template <class T>
inline M3<T> tau_nhb(const Material<T>& mat, const M3<T>& F, T g)
{
    T J = det(F);
    M3<T> B = mul_bt(F, F);
    T tr = B(0, 0) + B(1, 1) + B(2, 2);
    M3<T> tau;
    T s = mat.mu * std::pow(J, -(T)2 / (T)3);
    T prime = mat.kappa / 2 * (J - 1 / J);
    T vol = J * prime;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            T devB = B(r, c) - (r == c ? (T)1 / 3 * tr : (T)0);
            T td = s * devB;
            T tv = (r == c) ? vol : (T)0;
            tau(r, c) = (J >= 1) ? g * (td + tv) : g * td + tv;
        }
    return tau;
}

// Givens QR, GivensQR.h:10-48 (inplaceGivensQR: for each column j, rows i = m-1 .. j+1, a rotation of rows
// (i-1, i) built from (A(i-1,j), A(i,j)) applied to A and to M = I; Q = M^T), then the 3D sign convention of
// QRStableNeoHookean::updateScratch (QRStableNeoHookean.h:108-122)
template <class T>
inline void givens_qr(const M3<T>& F, M3<T>& Q, M3<T>& R)
{
    T A[3][3], M[3][3] = { { 1, 0, 0 }, { 0, 1, 0 }, { 0, 0, 1 } };
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) A[r][c] = F(r, c);
    for (int j = 0; j < 3; j++)
        for (int i = 2; i > j; i--) {
            Givens<T> g(i - 1, i);
            g.compute(A[i - 1][j], A[i][j]);
            g.rows(A);
            g.rows(M);
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            R(r, c) = A[r][c];
            Q(r, c) = M[c][r];
        }
    if (R(0, 0) < 0) {
        R(0, 0) *= -1;
        for (int r = 0; r < 3; r++) Q(r, 0) *= -1;
        R(0, 1) *= -1;
        R(0, 2) *= -1;
        R(2, 2) *= -1;
        for (int r = 0; r < 3; r++) Q(r, 2) *= -1;
    }
    if (R(1, 1) < 0) {
        R(1, 1) *= -1;
        for (int r = 0; r < 3; r++) Q(r, 1) *= -1;
        R(1, 2) *= -1;
        R(2, 2) *= -1;
        for (int r = 0; r < 3; r++) Q(r, 2) *= -1;
    }
}

// QRStableNeoHookean::updateScratch (QRStableNeoHookean.h:102-173) -> dPsiHat/dR; firstPiola through
// QrBasedHelper::evaluateP (QrBasedHelper.h:30-40): A = dPsiHatdR R^T with the lower triangle mirrored,
// P = Q A R^{-T}; kirchhoff = P F^T (HyperelasticConstitutiveModel.h:75-80). effective: g = 1, kx = ky = 0
// (evaluateEffectiveCauchyStress, QRStableNeoHookean.h:86-96). J (from R) is returned through Jout.
template <class T>
inline M3<T> tau_qrnh(const Material<T>& mat, const M3<T>& F, T g, bool effective, T* Jout = nullptr)
{
    M3<T> Q, R;
    givens_qr(F, Q, R);
    T kx = mat.kx, ky = mat.ky;
    if (effective) {
        g = 1;
        kx = 0;
        ky = 0;
    }
    T J = 1;
    for (int i = 0; i < 3; i++) J *= R(i, i);
    M3<T> D{};
    if (J >= 1)
        for (int i = 0; i < 3; i++) D(i, i) += g * mat.lambda * (J - 1) * J / R(i, i);
    else
        for (int i = 0; i < 3; i++) D(i, i) += mat.lambda * (J - 1) * J / R(i, i);
    for (int i = 0; i < 3; i++)
        for (int j = i; j < 3; j++) D(i, j) += g * mat.mu * R(i, j);
    for (int i = 0; i < 3; i++) D(i, i) -= g * mat.mu * J / R(i, i);
    D(0, 0) += kx * (R(0, 0) - 1);
    T ss = std::sqrt(R(0, 1) * R(0, 1) + R(1, 1) * R(1, 1));
    D(0, 1) += ky * (ss - 1) * R(0, 1) / ss;
    D(1, 1) += ky * (ss - 1) * R(1, 1) / ss;
    M3<T> A = mul_bt(D, R); // dPsiHatdR * R^T
    for (int i = 1; i < 3; i++)
        for (int j = 0; j < i; j++) A(i, j) = A(j, i);
    M3<T> RinvT = cofactor(R); // R^{-T} = cofactor(R) / det(R)
    T dR = det(R);
    for (int a = 0; a < 9; a++) RinvT.a[a] /= dR;
    M3<T> P = mul(mul(Q, A), RinvT);
    if (Jout) *Jout = J;
    return mul_bt(P, F);
}

template <class T>
inline T degradation(T d, T k) { return ((1 - d) * (1 - d) * (1 - k)) + k; } // AnisoFractureSimulation.h:279-280

enum { OBJ_STICKY = 1, OBJ_SLIP = 2, OBJ_SEPARATE = 3 };

template <class T>
struct HalfSpace {
    T o[3], n[3], vel[3];
    int type;
    T friction;
};

// CollisionObject.cpp:342-406 for a translating HalfSpace (R = I, s = 1, b(t) = vel*t), AnalyticLevelSet.cpp:318-334
template <class T>
inline bool resolve_halfspace(const HalfSpace<T>& h, T time, const T x[3], T v[3])
{
    T X[3];
    for (int d = 0; d < 3; d++) X[d] = x[d] - h.vel[d] * time;
    T phi = h.n[0] * (X[0] - h.o[0]) + h.n[1] * (X[1] - h.o[1]) + h.n[2] * (X[2] - h.o[2]);
    if (!(phi <= 0)) return false;
    for (int d = 0; d < 3; d++) v[d] -= h.vel[d];
    if (h.type == OBJ_STICKY) {
        v[0] = v[1] = v[2] = 0;
    }
    else {
        T dot = v[0] * h.n[0] + v[1] * h.n[1] + v[2] * h.n[2];
        bool project = (h.type == OBJ_SLIP) || (dot < 0);
        if (project) {
            for (int d = 0; d < 3; d++) v[d] -= h.n[d] * dot;
            if (h.friction != 0 && dot < 0) {
                T vn = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (-dot * h.friction < vn) {
                    for (int d = 0; d < 3; d++) v[d] += v[d] / vn * dot * h.friction;
                }
                else
                    v[0] = v[1] = v[2] = 0;
            }
        }
    }
    for (int d = 0; d < 3; d++) v[d] += h.vel[d];
    return true;
}

// CollisionObject.cpp:67-105: objects are applied in order; a STICKY hit ends the loop; the normal of every
// SLIP/SEPARATE hit is Gram-Schmidt orthogonalised against the earlier ones (:84-92) and, when it is not
// zero, normalised into the basis; the dim-th basis vector ends the loop (:93-98)
template <class T>
inline void multi_object_collision(const std::vector<HalfSpace<T>>& objs, T time, const T x[3], T v[3])
{
    T basis[3][3];
    int count = 0;
    for (auto& h : objs) {
        bool hit = resolve_halfspace(h, time, x, v);
        if (!hit) continue;
        if (h.type == OBJ_STICKY) break;
        T n[3] = { h.n[0], h.n[1], h.n[2] };
        for (int c = 0; c < count; c++) {
            T dot = basis[c][0] * n[0] + basis[c][1] * n[1] + basis[c][2] * n[2];
            for (int d = 0; d < 3; d++) n[d] -= dot * basis[c][d];
        }
        T length = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (length != 0) {
            for (int d = 0; d < 3; d++) basis[count][d] = n[d] / length;
            if (++count == 3) break;
        }
    }
}

// ----------------------------------------------------------------------------------------------
// Scene
// ----------------------------------------------------------------------------------------------
// Open-addressing page -> block-slot table (stands in for SPGrid_Page_Map's bitmap, SPGrid_Page_Map.h:61-95).
struct PageTable {
    std::vector<uint64_t> keys;
    std::vector<int> vals;
    uint64_t mask = 0;
    int count = 0;
    void reset(size_t expect)
    {
        size_t cap = 1024;
        while (cap < 2 * expect) cap <<= 1;
        keys.assign(cap, ~0ULL);
        vals.assign(cap, -1);
        mask = cap - 1;
        count = 0;
    }
    static uint64_t h(uint64_t k)
    {
        k ^= k >> 31;
        k *= 0x9e3779b97f4a7c15ULL;
        return k ^ (k >> 29);
    }
    // returns true when the page was not present (and inserts it with slot = count)
    bool insert(uint64_t page)
    {
        if (2 * (size_t)(count + 1) > keys.size()) grow();
        uint64_t i = h(page) & mask;
        while (keys[i] != ~0ULL) {
            if (keys[i] == page) return false;
            i = (i + 1) & mask;
        }
        keys[i] = page;
        vals[i] = count++;
        return true;
    }
    int at(uint64_t page) const
    {
        uint64_t i = h(page) & mask;
        while (keys[i] != ~0ULL) {
            if (keys[i] == page) return vals[i];
            i = (i + 1) & mask;
        }
        return -1;
    }
    void grow()
    {
        std::vector<uint64_t> ok = keys;
        std::vector<int> ov = vals;
        keys.assign(ok.size() * 2, ~0ULL);
        vals.assign(ok.size() * 2, -1);
        mask = keys.size() - 1;
        for (size_t q = 0; q < ok.size(); q++)
            if (ok[q] != ~0ULL) {
                uint64_t i = h(ok[q]) & mask;
                while (keys[i] != ~0ULL) i = (i + 1) & mask;
                keys[i] = ok[q];
                vals[i] = ov[q];
            }
    }
};

template <class T>
struct Node {
    T v[3];
    T m;
    T f[3]; // the reference's new_v, holding the force during P2G
    T pf, pfm; // phase field and its weight sum (GridState phase_field / phase_field_multiplier)
};

template <class T>
struct Scene {
    using L = LayoutOf<T>;
    T dx, dt, gravity[3], apic_ratio, cfl;
    double time = 0;
    std::vector<Material<T>> materials;
    std::vector<HalfSpace<T>> objects;
    bool damage = false;
    bool implicit = false; // AnisoFractureSimulation's implicit damage solve (--implicit_damage)
    int cg_iterations = 0; // of the last solve

    int64_t n = 0;
    std::vector<std::array<T, 3>> x, v;
    std::vector<M3<T>> C, F, vtau, gradV;
    std::vector<T> m, V0, d, sigc, lap, vol, maxdt;
    std::vector<int32_t> mat;

    // binning products (MpmSimulationBase.cpp:1531-1573)
    std::vector<uint64_t> sorter, base_offset, block_offset;
    std::vector<int32_t> order;
    std::vector<std::pair<int, int>> groups;
    std::vector<uint64_t> pages; // first-touch order (MpmGrid.h:157-183, SPGrid_Page_Map.h:61-70)
    PageTable page_slot;
    std::vector<Node<T>> grid; // pages.size() * nodes_per_block
    std::vector<std::array<int, 8>> group_nbr; // neighbour block slots of each group, index dx*4+dy*2+dz
    int cfl_flags = 0;
    size_t pages_hint = 1024;

    void bin()
    {
        constexpr int index_bits = L::index_bits;
        sorter.resize(n);
        base_offset.resize(n);
        order.resize(n);
        T one_over_dx = (T)1 / dx;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            int b[3];
            for (int a = 0; a < 3; a++) b[a] = int_floor(x[i][a] * one_over_dx - (T)0.5);
            uint64_t off = L::linear_offset(b[0], b[1], b[2]);
            base_offset[i] = off;
            sorter[i] = ((off >> L::data_bits) << index_bits) + (uint64_t)i;
        }
#ifdef _OPENMP
        __gnu_parallel::sort(sorter.begin(), sorter.end()); // tbb::parallel_sort in the reference (:1552)
#else
        std::sort(sorter.begin(), sorter.end());
#endif
        groups.clear();
        block_offset.clear();
        int last = 0;
        for (int64_t i = 0; i < n; i++) {
            if (i == n - 1 || (sorter[i] >> 32) != (sorter[i + 1] >> 32)) {
                groups.push_back({ last, (int)i });
                block_offset.push_back(sorter[i] >> 32);
                last = (int)i + 1;
            }
            order[i] = (int32_t)(sorter[i] & ((1ULL << index_bits) - 1));
        }
        // pollute: original particle order, consecutive dedup, page of base node + 7 neighbours
        pages.clear();
        page_slot.reset(pages_hint);
        auto set_page = [&](uint64_t off) {
            uint64_t p = off >> 12;
            if (page_slot.insert(p)) pages.push_back(p);
        };
        uint64_t nbr_disp[8];
        for (int a = 0; a < 8; a++) nbr_disp[a] = L::linear_offset(L::sx * (a >> 2), L::sy * ((a >> 1) & 1), L::sz * (a & 1));
        for (int64_t i = 0; i < n; i++) {
            uint64_t off = base_offset[i];
            if (i == 0 || off != base_offset[i - 1]) {
                set_page(off);
                for (int a = 0; a < 8; a++) set_page(L::packed_add(off, nbr_disp[a]));
            }
        }
        pages_hint = pages.size();
        grid.assign(pages.size() * L::nodes_per_block, Node<T>{});
        group_nbr.resize(groups.size());
        for (size_t g = 0; g < groups.size(); g++) {
            uint64_t off = block_offset[g] << 12;
            for (int a = 0; a < 8; a++) group_nbr[g][a] = page_slot.at(L::packed_add(off, nbr_disp[a]) >> 12);
        }
    }

    // Node of the stencil: base node coords b (absolute), stencil offset (i,j,k), group origin o.
    Node<T>& node_at(size_t g, const int o[3], const int b[3], int i, int j, int k)
    {
        int lx = b[0] + i - o[0], ly = b[1] + j - o[1], lz = b[2] + k - o[2];
        int ax = lx >= L::sx, ay = ly >= L::sy, az = lz >= L::sz;
        int slot = group_nbr[g][ax * 4 + ay * 2 + az];
        return grid[(size_t)slot * L::nodes_per_block + L::element(lx - ax * L::sx, ly - ay * L::sy, lz - az * L::sz)];
    }

    void group_origin(size_t g, int o[3]) const { L::coord(block_offset[g] << 12, o[0], o[1], o[2]); }

    void weights(int64_t p, int b[3], T w[3][3], T dw[3][3]) const
    {
        T one_over_dx = 1 / dx;
        for (int a = 0; a < 3; a++) bspline(one_over_dx * x[p][a], b[a], w[a], dw[a]);
    }

    void stress()
    {
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++) {
            const Material<T>& mt = materials[mat[p]];
            M3<T> tau;
            const T g = damage && mt.damage ? degradation(d[p], mt.residual) : (T)1;
            if (mt.model == MODEL_COROTATED)
                tau = tau_corotated(mt, F[p]); // no degradation member: never damaged (AnisoFractureSimulation.h:343-352)
            else if (mt.model == MODEL_QRNH)
                tau = tau_qrnh(mt, F[p], g, false);
            else
                tau = tau_nhb(mt, F[p], g);
            for (int a = 0; a < 9; a++) vtau[p].a[a] = tau.a[a] * V0[p]; // FBasedMpmForceHelper.cpp:58-62
        }
    }

    template <class Body>
    void colour_scatter(Body body)
    {
        for (uint64_t colour = 0; colour < 8; colour++) {
#pragma omp parallel for schedule(dynamic, 4)
            for (int64_t g = 0; g < (int64_t)groups.size(); g++) {
                if ((block_offset[g] & 7) != colour) continue;
                int o[3];
                group_origin(g, o);
                for (int idx = groups[g].first; idx <= groups[g].second; idx++) body(g, o, order[idx]);
            }
        }
    }

    // MpmSimulationBase.cpp:680-854
    void p2g()
    {
        T one_over_dx = 1 / dx;
        colour_scatter([&](size_t g, const int o[3], int p) {
            int b[3];
            T w[3][3], dw[3][3];
            weights(p, b, w, dw);
            T mass = m[p];
            T mom[3] = { mass * v[p][0], mass * v[p][1], mass * v[p][2] };
            M3<T> Cm;
            for (int a = 0; a < 9; a++) Cm.a[a] = mass * C[p].a[a];
            const M3<T>& S = vtau[p];
            const T* X = x[p].data();
            for (int i = 0; i < 3; i++) {
                T wi = w[0][i], dwidxi = one_over_dx * dw[0][i];
                for (int j = 0; j < 3; j++) {
                    T wj = w[1][j], wij = wi * wj, dwijdxi = dwidxi * wj, dwijdxj = wi * one_over_dx * dw[1][j];
                    for (int k = 0; k < 3; k++) {
                        T wk = w[2][k], wijk = wij * wk;
                        T gw[3] = { dwijdxi * wk, dwijdxj * wk, wij * one_over_dx * dw[2][k] };
                        Node<T>& nd = node_at(g, o, b, i, j, k);
                        int node[3] = { b[0] + i, b[1] + j, b[2] + k };
                        if constexpr (std::is_same<T, float>::value) {
                            T xm[3];
                            for (int a = 0; a < 3; a++) xm[a] = std::fma((T)node[a], dx, -X[a]);
                            for (int r = 0; r < 3; r++) {
                                T del = std::fma(S(r, 2), gw[2], std::fma(S(r, 1), gw[1], std::fma(S(r, 0), gw[0], (T)0 * wijk)));
                                T tmp = std::fma(Cm(r, 2), xm[2], std::fma(Cm(r, 1), xm[1], Cm(r, 0) * xm[0]));
                                nd.v[r] += wijk * (mom[r] + tmp);
                                nd.f[r] -= del;
                            }
                            nd.m += wijk * (mass + (T)0);
                        }
                        else {
                            T xm[3];
                            for (int a = 0; a < 3; a++) xm[a] = (T)node[a] * dx - X[a];
                            for (int r = 0; r < 3; r++) {
                                T fd = S(r, 0) * gw[0] + S(r, 1) * gw[1] + S(r, 2) * gw[2] + (T)0 * wijk;
                                T vd = (Cm(r, 0) * xm[0] + Cm(r, 1) * xm[1] + Cm(r, 2) * xm[2] + mom[r]) * wijk;
                                nd.v[r] += vd;
                                nd.f[r] -= fd;
                            }
                            nd.m += mass * wijk;
                        }
                    }
                }
            }
        });
        // getNumNodes + v /= m (MpmSimulationBase.cpp:655-666, MpmGrid.h:195-208)
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < (int64_t)grid.size(); q++) {
            Node<T>& nd = grid[q];
            if (nd.m != 0)
                for (int a = 0; a < 3; a++) nd.v[a] /= nd.m;
        }
    }

    // AnisoFractureSimulation.h:150-209
    void laplacians()
    {
        T one_over_dx = 1 / dx;
        colour_scatter([&](size_t g, const int o[3], int p) {
            int b[3];
            T w[3][3], dw[3][3];
            weights(p, b, w, dw);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) {
                        T wijk = w[0][i] * w[1][j] * w[2][k];
                        Node<T>& nd = node_at(g, o, b, i, j, k);
                        nd.pfm += wijk;
                        nd.pf += d[p] * wijk;
                    }
        });
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < (int64_t)grid.size(); q++)
            if (grid[q].m != 0) grid[q].pf /= grid[q].pfm;
        const T ddw[3] = { 1, -2, 1 };
#pragma omp parallel for schedule(dynamic, 4)
        for (int64_t g = 0; g < (int64_t)groups.size(); g++) {
            int o[3];
            group_origin(g, o);
            for (int idx = groups[g].first; idx <= groups[g].second; idx++) {
                int p = order[idx];
                int b[3];
                T w[3][3], dw[3][3];
                weights(p, b, w, dw);
                T lp = 0;
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++) {
                            T wi = w[0][i], wj = w[1][j], wk = w[2][k];
                            // MpmGrid.h:607-613 (all three terms use ddw(i): the reference's 3D form)
                            T t1 = one_over_dx * one_over_dx * ddw[i] * wj * wk;
                            T t2 = one_over_dx * one_over_dx * ddw[i] * wi * wk;
                            T t3 = one_over_dx * one_over_dx * ddw[i] * wi * wj;
                            T L = t1 + t2 + t3;
                            Node<T>& nd = node_at(g, o, b, i, j, k);
                            if (nd.m != 0) lp += nd.pf * L;
                        }
                lap[p] = lp;
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++) vol[p] = V0[p] * det(F[p]);
    }

    bool damageable(int64_t p) const
    {
        // the reference damages only particles that carry a phase field and one of its damageable models
        // (AnisoFractureSimulation.h:210-218,343-352)
        const Material<T>& mt = materials[mat[p]];
        return (mt.model == MODEL_NHB || mt.model == MODEL_QRNH) && mt.damage;
    }

    // AnisoFractureSimulation.h:210-283, :365-391 (one director a0 = e1, one weight alpha)
    void update_damage()
    {
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++) {
            if (!damageable(p)) continue;
            const Material<T>& mt = materials[mat[p]];
            T geo = d[p] - (mt.l0 * mt.l0 * lap[p]);
            T dtilde = dtilde_of(p);
            T diff = ((1 - d[p]) * dtilde) - geo;
            T newd = d[p] + ((dt / mt.eta) * ((diff + std::abs(diff)) / 2));
            d[p] = std::min(newd, (T)1);
        }
    }

    // D-tilde = zeta <phi - 1> of one particle (AnisoFractureSimulation.h:224-270, updateDTildeHelper :292-333)
    T dtilde_of(int64_t p) const
    {
        {
            const Material<T>& mt = materials[mat[p]];
            T J;
            M3<T> tau;
            if (mt.model == MODEL_QRNH)
                tau = tau_qrnh(mt, F[p], (T)1, true, &J); // cauchy = P F^T / J, J from the QR (QRStableNeoHookean.h:86-96)
            else {
                tau = tau_nhb(mt, F[p], (T)1);
                J = det(F[p]);
            }
            double S[3][3], lam[3], Q[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) S[r][c] = (double)(tau(r, c) / J);
            sym_eigen(S, lam, Q);
            M3<T> sp{};
            for (int e = 0; e < 3; e++) {
                T l = (T)lam[e];
                T mac = (l + std::abs(l)) / 2; // MathTools.h:276-281
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) sp(r, c) += mac * ((T)Q[r][e] * (T)Q[c][e]);
            }
            M3<T> R = polar_rotation(F[p]);
            T a1[3] = { R(0, 0), R(1, 0), R(2, 0) }; // R * e1
            M3<T> A = M3<T>::identity();
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) A(r, c) += mt.alpha * (a1[r] * a1[c]);
            M3<T> As = mul(A, sp), sA = mul(sp, A);
            T contraction = 0;
            for (int a = 0; a < 9; a++) contraction += As.a[a] * sA.a[a];
            T phi = ((T)1 / (sigc[p] * sigc[p])) * contraction;
            T pm1 = phi - 1;
            return mt.zeta * ((pm1 + std::abs(pm1)) / 2);
        }
    }

    // damageP2G (AnisoFractureSimulation.h:393-435): normalised nodal phase field and vol = V0 det F
    void damage_p2g()
    {
        colour_scatter([&](size_t g, const int o[3], int p) {
            int b[3];
            T w[3][3], dw[3][3];
            weights(p, b, w, dw);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) {
                        T wijk = w[0][i] * w[1][j] * w[2][k];
                        Node<T>& nd = node_at(g, o, b, i, j, k);
                        nd.pfm += wijk;
                        nd.pf += d[p] * wijk;
                    }
        });
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < (int64_t)grid.size(); q++)
            if (grid[q].m != 0) grid[q].pf /= grid[q].pfm;
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++) vol[p] = V0[p] * det(F[p]);
    }

    // solveDamageSystem (AnisoFractureSimulation.h:437-562) with ConjugateGradient::solve (ConjugateGradient.h,
    // tolerance 1e-6, relative tolerance 1, at most 100 iterations, x0 = 0) and damageG2P (:564-626). Only
    // particles of a damageable model take part, and the unknowns are the nodes they reach (the reference's
    // nodes with mass, MpmGrid::getNumNodes, when every particle carries a phase field, as it assumes).
    void solve_damage()
    {
        damage_p2g();
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++)
            if (damageable(p)) maxdt[p] = std::max(dtilde_of(p), maxdt[p]); // updateDTilde (:334-338)
        // the preconditioner's diagonal, sum_p vol (1 + dt/eta (D~ + 1)) w, per grid node; it selects the unknowns
        std::vector<T> gdiag(grid.size(), 0);
        colour_scatter([&](size_t g, const int o[3], int p) {
            if (!damageable(p)) return;
            const Material<T>& mt = materials[mat[p]];
            int b[3];
            T w[3][3], dw[3][3];
            weights(p, b, w, dw);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++)
                        gdiag[&node_at(g, o, b, i, j, k) - grid.data()] += vol[p] * (1 + ((dt / mt.eta) * (maxdt[p] + 1))) * (w[0][i] * w[1][j] * w[2][k]);
        });
        std::vector<int64_t> id(grid.size(), -1);
        int64_t nn = 0;
        for (size_t q = 0; q < grid.size(); q++)
            if (grid[q].m != 0 && gdiag[q] > 0) id[q] = nn++;
        auto nid = [&](Node<T>& nd) { return id[&nd - grid.data()]; };
        auto grad = [&](const T w[3][3], const T dw[3][3], int i, int j, int k, T gw[3]) {
            T odx = 1 / dx;
            gw[0] = odx * dw[0][i] * w[1][j] * w[2][k];
            gw[1] = w[0][i] * odx * dw[1][j] * w[2][k];
            gw[2] = w[0][i] * w[1][j] * odx * dw[2][k];
        };
        std::vector<T> xv(nn, 0), rhs(nn, 0), diag(nn, 0);
        colour_scatter([&](size_t g, const int o[3], int p) {
            if (!damageable(p)) return;
            const Material<T>& mt = materials[mat[p]];
            int b[3];
            T w[3][3], dw[3][3];
            weights(p, b, w, dw);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    for (int k = 0; k < 3; k++) {
                        Node<T>& nd = node_at(g, o, b, i, j, k);
                        int64_t q = nid(nd);
                        if (q < 0) continue;
                        T wijk = w[0][i] * w[1][j] * w[2][k];
                        rhs[q] += (((dt * maxdt[p]) / mt.eta) + nd.pf) * vol[p] * wijk;
                    }
        });
        for (size_t q = 0; q < grid.size(); q++)
            if (id[q] >= 0) diag[id[q]] = gdiag[q];
        std::vector<std::array<T, 3>> gradc(n);
        auto multiply = [&](const std::vector<T>& xx, std::vector<T>& bb) {
#pragma omp parallel for schedule(dynamic, 4)
            for (int64_t g = 0; g < (int64_t)groups.size(); g++) {
                int o[3];
                group_origin(g, o);
                for (int idx = groups[g].first; idx <= groups[g].second; idx++) {
                    int p = order[idx];
                    gradc[p] = { 0, 0, 0 };
                    if (!damageable(p)) continue;
                    const Material<T>& mt = materials[mat[p]];
                    int b[3];
                    T w[3][3], dw[3][3];
                    weights(p, b, w, dw);
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            for (int k = 0; k < 3; k++) {
                                int64_t q = nid(node_at(g, o, b, i, j, k));
                                if (q < 0) continue;
                                T gw[3];
                                grad(w, dw, i, j, k, gw);
                                for (int a = 0; a < 3; a++) gradc[p][a] += xx[q] * gw[a];
                            }
                    for (int a = 0; a < 3; a++) gradc[p][a] *= vol[p] * (dt / mt.eta) * mt.l0 * mt.l0;
                }
            }
            std::fill(bb.begin(), bb.end(), (T)0);
            colour_scatter([&](size_t g, const int o[3], int p) {
                if (!damageable(p)) return;
                const Material<T>& mt = materials[mat[p]];
                int b[3];
                T w[3][3], dw[3][3];
                weights(p, b, w, dw);
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++) {
                            int64_t q = nid(node_at(g, o, b, i, j, k));
                            if (q < 0) continue;
                            T wijk = w[0][i] * w[1][j] * w[2][k], gw[3];
                            grad(w, dw, i, j, k, gw);
                            bb[q] += vol[p] * (1 + ((dt / mt.eta) * (maxdt[p] + 1))) * wijk * xx[q];
                            bb[q] += gradc[p][0] * gw[0] + gradc[p][1] * gw[1] + gradc[p][2] * gw[2];
                        }
            });
        };
        auto dotp = [&](const std::vector<T>& a, const std::vector<T>& c) {
            T s = 0;
            for (int64_t q = 0; q < nn; q++) s += a[q] * c[q];
            return s;
        };
        std::vector<T> r(nn), qv(nn), pv(nn), tmp(nn);
        multiply(xv, tmp);
        for (int64_t q = 0; q < nn; q++) {
            r[q] = rhs[q] - tmp[q];
            qv[q] = r[q] / diag[q];
        }
        pv = qv;
        T zTrk = dotp(r, qv), zTrk_last;
        T res = std::sqrt(zTrk);
        const T local_tol = std::min((T)1 * res, (T)1e-6);
        int cnt = 0;
        for (; cnt < 100; ++cnt) {
            if (res <= local_tol) break;
            multiply(pv, tmp);
            T alpha = zTrk / dotp(tmp, pv);
            for (int64_t q = 0; q < nn; q++) {
                xv[q] += pv[q] * alpha;
                r[q] -= tmp[q] * alpha;
                qv[q] = r[q] / diag[q];
            }
            zTrk_last = zTrk;
            zTrk = dotp(qv, r);
            T beta = zTrk / zTrk_last;
            for (int64_t q = 0; q < nn; q++) pv[q] = qv[q] + beta * pv[q];
            res = std::sqrt(zTrk);
        }
        cg_iterations = cnt;
        for (size_t q = 0; q < grid.size(); q++)
            if (id[q] >= 0) grid[q].pf = xv[id[q]] - grid[q].pf; // the change of the nodal phase field
#pragma omp parallel for schedule(dynamic, 4)
        for (int64_t g = 0; g < (int64_t)groups.size(); g++) {
            int o[3];
            group_origin(g, o);
            for (int idx = groups[g].first; idx <= groups[g].second; idx++) {
                int p = order[idx];
                if (!damageable(p)) continue;
                int b[3];
                T w[3][3], dw[3][3];
                weights(p, b, w, dw);
                T pf = 0;
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < 3; k++) {
                            Node<T>& nd = node_at(g, o, b, i, j, k);
                            if (nid(nd) >= 0) pf += w[0][i] * w[1][j] * w[2][k] * nd.pf;
                        }
                T new_d = d[p] + pf;
                d[p] = std::min(std::max(d[p], new_d), (T)1);
            }
        }
    }

    // MpmSimulationBase.cpp:1179-1228
    void grid_update()
    {
        T dvg[3] = { gravity[0] * dt, gravity[1] * dt, gravity[2] * dt };
#pragma omp parallel for schedule(static)
        for (int64_t bslot = 0; bslot < (int64_t)pages.size(); bslot++) {
            int o[3];
            L::coord(pages[bslot] << 12, o[0], o[1], o[2]);
            for (int lx = 0; lx < L::sx; lx++)
                for (int ly = 0; ly < L::sy; ly++)
                    for (int lz = 0; lz < L::sz; lz++) {
                        Node<T>& nd = grid[(size_t)bslot * L::nodes_per_block + L::element(lx, ly, lz)];
                        if (nd.m == 0) continue;
                        T dt_over_mi = dt / nd.m;
                        T xi[3] = { (T)(o[0] + lx) * dx, (T)(o[1] + ly) * dx, (T)(o[2] + lz) * dx };
                        T vi[3];
                        for (int a = 0; a < 3; a++) vi[a] = nd.v[a] + dvg[a] + nd.f[a] * dt_over_mi;
                        multi_object_collision(objects, (T)time, xi, vi);
                        for (int a = 0; a < 3; a++) nd.f[a] = vi[a]; // new_v
                    }
        }
    }

    // MpmSimulationBase.cpp:1269-1515 and FBasedMpmForceHelper.cpp:95-108
    void g2p()
    {
        T one_over_dx = 1 / dx;
        T dx2 = dx * dx;
        T D_inverse = 4 / dx2; // MpmSimulationBase.cpp:118-122
        T ca = (apic_ratio + 1) * (T)0.5, cb = (apic_ratio - 1) * (T)0.5;
        int flags = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : flags)
        for (int64_t g = 0; g < (int64_t)groups.size(); g++) {
            int o[3];
            group_origin(g, o);
            for (int idx = groups[g].first; idx <= groups[g].second; idx++) {
                int p = order[idx];
                int b[3];
                T w[3][3], dw[3][3];
                weights(p, b, w, dw);
                const T* X = x[p].data();
                T pv[3] = { 0, 0, 0 };
                M3<T> Bm{}, G{};
                for (int i = 0; i < 3; i++) {
                    T wi = w[0][i], dwidxi = one_over_dx * dw[0][i];
                    for (int j = 0; j < 3; j++) {
                        T wj = w[1][j], wij = wi * wj, dwijdxi = dwidxi * wj, dwijdxj = wi * one_over_dx * dw[1][j];
                        for (int k = 0; k < 3; k++) {
                            T wk = w[2][k], wijk = wij * wk;
                            T gw[3] = { dwijdxi * wk, dwijdxj * wk, wij * one_over_dx * dw[2][k] };
                            Node<T>& nd = node_at(g, o, b, i, j, k);
                            int node[3] = { b[0] + i, b[1] + j, b[2] + k };
                            const T* nv = nd.f;
                            if constexpr (std::is_same<T, float>::value) {
                                T xm[3];
                                for (int a = 0; a < 3; a++) {
                                    xm[a] = std::fma((T)node[a], dx, -X[a]);
                                    pv[a] = std::fma(nv[a], wijk, pv[a]);
                                }
                                T xmw[3] = { xm[0] * wijk, xm[1] * wijk, xm[2] * wijk };
                                for (int r = 0; r < 3; r++)
                                    for (int c = 0; c < 3; c++) {
                                        Bm(r, c) = std::fma(nv[r], xmw[c], Bm(r, c));
                                        G(r, c) = std::fma(nv[r], gw[c], G(r, c));
                                    }
                            }
                            else {
                                T xm[3];
                                for (int a = 0; a < 3; a++) {
                                    pv[a] += wijk * nv[a];
                                    xm[a] = (T)node[a] * dx - X[a];
                                }
                                for (int r = 0; r < 3; r++)
                                    for (int c = 0; c < 3; c++) {
                                        Bm(r, c) += wijk * nv[r] * xm[c];
                                        G(r, c) += nv[r] * gw[c];
                                    }
                            }
                        }
                    }
                }
                for (int a = 0; a < 3; a++) v[p][a] = pv[a];
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        if constexpr (std::is_same<T, float>::value)
                            C[p](r, c) = (ca * Bm(r, c) + cb * Bm(c, r)) * D_inverse;
                        else
                            C[p](r, c) = ca * (Bm(r, c) * D_inverse) + cb * (Bm(c, r) * D_inverse);
                    }
                gradV[p] = G;
                T inc[3] = { dt * pv[0], dt * pv[1], dt * pv[2] };
                for (int a = 0; a < 3; a++) x[p][a] += inc[a];
                T inc2 = inc[0] * inc[0] + inc[1] * inc[1] + inc[2] * inc[2];
                if (inc2 > dx2) flags |= 1;
                if (inc2 > dx2 * (T)0.25 * (cfl * cfl)) flags |= 2;
            }
        }
        cfl_flags = flags;
        // evolveStrain: F <- (I + dt gradV) F
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < n; p++) {
            M3<T> A = M3<T>::identity();
            for (int a = 0; a < 9; a++) A.a[a] += dt * gradV[p].a[a];
            F[p] = mul(A, F[p]);
        }
    }

    // MpmSimulationBase.cpp:262-357 (symplectic branch) with the AnisoFractureSimulation override
    int step()
    {
        bin();
        stress();
        p2g();
        if (damage && implicit)
            solve_damage();
        else if (damage) {
            laplacians();
            update_damage();
        }
        grid_update();
        g2p();
        time += (double)dt;
        return cfl_flags;
    }

    void resize(int64_t nn)
    {
        n = nn;
        x.resize(n);
        v.resize(n);
        C.resize(n);
        F.resize(n);
        vtau.resize(n);
        gradV.resize(n);
        m.resize(n);
        V0.resize(n);
        d.resize(n);
        sigc.resize(n);
        lap.resize(n);
        vol.resize(n);
        maxdt.assign(n, (T)0);
        mat.resize(n);
    }
};

struct Handle {
    int precision;
    void* scene;
};

template <class T>
Scene<T>* S(Handle* h) { return static_cast<Scene<T>*>(h->scene); }

} // namespace orc

using namespace orc;

#define DISPATCH(h, ...)                       \
    do {                                       \
        if ((h)->precision == 4) {             \
            auto* sc = S<float>(h);            \
            __VA_ARGS__;                       \
        }                                      \
        else {                                 \
            auto* sc = S<double>(h);           \
            __VA_ARGS__;                       \
        }                                      \
    } while (0)

// ----------------------------------------------------------------------------------------------
// Seeded scene inputs, restated here so that the CPU baseline builds its inputs without the product
// library. The sampling is the reference's (MpmInitializationHelper.h:1344-1414 samples a jittered
// lattice; MpmParticleHandleBase.cpp:175-268 draws fibres and turns one director into F with
// initializeRotatedFHelper); the random stream is the library's recipe format: raw std::mt19937_64
// outputs (defined bit for bit by the C++ standard), uniforms from the top 53 bits, normals by
// Box-Muller, fibres from a von Mises-Fisher law about +x by Wood's method for the 2-sphere. Per
// particle, in lattice order (cell i, j, k; sub-cell a, b, c): three jitter uniforms; for the slab also
// a fibre (two uniforms) and sigma_c (two uniforms).
// ----------------------------------------------------------------------------------------------
struct SeedStream {
    std::mt19937_64 g;
    explicit SeedStream(uint64_t seed) : g(seed) {}
    double u01() { return (double)(g() >> 11) * 0x1.0p-53; }
    double gauss()
    {
        const double a = std::max(u01(), 1e-300), b = u01();
        return std::sqrt(-2.0 * std::log(a)) * std::cos(2.0 * M_PI * b);
    }
    void fibre(double kappa, double d[3])
    {
        const double u = u01();
        const double w = std::min(1.0, std::max(-1.0, 1.0 + std::log(u + (1.0 - u) * std::exp(-2.0 * kappa)) / kappa));
        const double ph = 2.0 * M_PI * u01(), r = std::sqrt(std::max(0.0, 1.0 - w * w));
        d[0] = w;
        d[1] = r * std::cos(ph);
        d[2] = r * std::sin(ph);
    }
};

// initializeRotatedFHelper for one director a (MpmParticleHandleBase.cpp:224-268): F's columns are a,
// a_perp = normalize(-a_y, a_x, 0) (e_x when a lies along z) and a x a_perp
inline void rotated_F(const double a[3], double F[9])
{
    double p[3] = { 1, 0, 0 };
    if (!(std::fabs(a[0]) < 1e-6 && std::fabs(a[1]) < 1e-6)) {
        const double len = std::sqrt(a[1] * a[1] + a[0] * a[0]);
        p[0] = -a[1] / len;
        p[1] = a[0] / len;
    }
    const double q[3] = { a[1] * p[2] - a[2] * p[1], a[2] * p[0] - a[0] * p[2], a[0] * p[1] - a[1] * p[0] };
    for (int r = 0; r < 3; r++) {
        F[3 * r] = a[r];
        F[3 * r + 1] = p[r];
        F[3 * r + 2] = q[r];
    }
}

extern "C" {

void* orc_create(int precision, double dx, double dt, const double* gravity, double apic_ratio, double cfl)
{
    Handle* h = new Handle{ precision, nullptr };
    auto init = [&](auto* sc) {
        sc->dx = dx;
        sc->dt = dt;
        for (int a = 0; a < 3; a++) sc->gravity[a] = gravity[a];
        sc->apic_ratio = apic_ratio;
        sc->cfl = cfl;
    };
    if (precision == 4) {
        auto* s = new Scene<float>();
        init(s);
        h->scene = s;
    }
    else {
        auto* s = new Scene<double>();
        init(s);
        h->scene = s;
    }
    return h;
}

void orc_destroy(void* hp)
{
    Handle* h = (Handle*)hp;
    if (!h) return;
    if (h->precision == 4)
        delete S<float>(h);
    else
        delete S<double>(h);
    delete h;
}

// model 0 = fixed corotated, 1 = Neo-Hookean (Borden), 2 = QR-stable Neo-Hookean with fibre stiffness
// kx = kx_scale mu, ky = ky_scale mu. Returns the material index.
int orc_add_material(void* hp, int model, double E, double nu, int damage, double alpha, double l0, double eta, double zeta, double residual,
    double kx_scale, double ky_scale)
{
    Handle* h = (Handle*)hp;
    int id = -1;
    DISPATCH(h, {
        using T = std::remove_reference_t<decltype(sc->dx)>;
        Material<T> mt;
        mt.model = model;
        T Et = (T)E, nut = (T)nu;
        // CorotatedElasticity.cpp:16-21 / NeoHookeanBorden.cpp:16-21
        T lambda = Et * nut / (((T)1 + nut) * ((T)1 - (T)2 * nut));
        mt.mu = Et / ((T)2 * ((T)1 + nut));
        mt.lambda = lambda;
        mt.kappa = (T).666666 * mt.mu + lambda;
        mt.kx = (T)kx_scale * mt.mu; // QRStableNeoHookean::setExtraFiberStiffness (QRStableNeoHookean.h:98-107)
        mt.ky = (T)ky_scale * mt.mu;
        mt.damage = damage != 0;
        mt.alpha = (T)alpha;
        mt.l0 = (T)l0;
        mt.eta = (T)eta;
        mt.zeta = (T)zeta;
        mt.residual = (T)residual;
        if (mt.damage) sc->damage = true;
        sc->materials.push_back(mt);
        id = (int)sc->materials.size() - 1;
    });
    return id;
}

int orc_add_halfspace(void* hp, const double* origin, const double* normal, int type, double friction, const double* vel)
{
    Handle* h = (Handle*)hp;
    DISPATCH(h, {
        using T = std::remove_reference_t<decltype(sc->dx)>;
        HalfSpace<T> hs;
        double nn = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
        for (int a = 0; a < 3; a++) {
            hs.o[a] = (T)origin[a];
            hs.n[a] = (T)(normal[a] / nn);
            hs.vel[a] = (T)vel[a];
        }
        hs.type = type;
        hs.friction = (T)friction;
        sc->objects.push_back(hs);
    });
    return 0;
}

// F and C are row-major n*9 (NULL: identity / zero). d, sigma_c may be NULL (0 / 1). material may be NULL (all 0).
int orc_set_particles(void* hp, int64_t n, const double* x, const double* v, const double* m, const double* V0, const double* F,
    const double* C, const double* d, const double* sigma_c, const int32_t* material)
{
    Handle* h = (Handle*)hp;
    DISPATCH(h, {
        using T = std::remove_reference_t<decltype(sc->dx)>;
        sc->resize(n);
        for (int64_t p = 0; p < n; p++) {
            for (int a = 0; a < 3; a++) {
                sc->x[p][a] = (T)x[3 * p + a];
                sc->v[p][a] = (T)v[3 * p + a];
            }
            for (int a = 0; a < 9; a++) {
                sc->F[p].a[a] = F ? (T)F[9 * p + a] : (T)((a % 4) == 0);
                sc->C[p].a[a] = C ? (T)C[9 * p + a] : (T)0;
            }
            sc->m[p] = (T)m[p];
            sc->V0[p] = (T)V0[p];
            sc->d[p] = d ? (T)d[p] : (T)0;
            sc->sigc[p] = sigma_c ? (T)sigma_c[p] : (T)1;
            sc->mat[p] = material ? material[p] : 0;
            sc->lap[p] = 0;
            sc->vol[p] = sc->V0[p];
        }
    });
    return 0;
}

// Runs nsteps substeps; returns the OR of the CFL flags (bit 0: a particle moved more than dx, the
// reference's RestartException trigger; bit 1: more than cfl*dx/2).
// damage by the implicit phase-field solve instead of the explicit update (AnisoFractureSimulation.h:129-141)
void orc_set_implicit(void* hp, int on)
{
    Handle* h = (Handle*)hp;
    DISPATCH(h, { sc->implicit = on != 0; });
}

// CG iterations of the last implicit damage solve
int orc_cg_iterations(void* hp)
{
    Handle* h = (Handle*)hp;
    int it = 0;
    DISPATCH(h, { it = sc->cg_iterations; });
    return it;
}

int orc_step(void* hp, int nsteps)
{
    Handle* h = (Handle*)hp;
    int flags = 0;
    DISPATCH(h, {
        for (int s = 0; s < nsteps; s++) flags |= sc->step();
    });
    return flags;
}

int orc_get_state(void* hp, double* x, double* v, double* C, double* F, double* d)
{
    Handle* h = (Handle*)hp;
    DISPATCH(h, {
        for (int64_t p = 0; p < sc->n; p++) {
            for (int a = 0; a < 3; a++) {
                if (x) x[3 * p + a] = sc->x[p][a];
                if (v) v[3 * p + a] = sc->v[p][a];
            }
            for (int a = 0; a < 9; a++) {
                if (C) C[9 * p + a] = sc->C[p].a[a];
                if (F) F[9 * p + a] = sc->F[p].a[a];
            }
            if (d) d[p] = sc->d[p];
        }
    });
    return 0;
}

double orc_time(void* hp)
{
    Handle* h = (Handle*)hp;
    double t = 0;
    DISPATCH(h, { t = sc->time; });
    return t;
}

// Binning of the current positions. Outputs (each may be NULL): sorter (n), order (n),
// groups as first/last sorted index and block_offset (n_groups), pages in first-touch order (n_pages).
// Returns n_groups; *n_pages receives the page count.
int64_t orc_bin(void* hp, uint64_t* sorter, int32_t* order, int32_t* group_first, int32_t* group_last, uint64_t* block_offset,
    uint64_t* pages, int64_t* n_pages)
{
    Handle* h = (Handle*)hp;
    int64_t ng = 0;
    DISPATCH(h, {
        sc->bin();
        for (int64_t p = 0; p < sc->n; p++) {
            if (sorter) sorter[p] = sc->sorter[p];
            if (order) order[p] = sc->order[p];
        }
        ng = (int64_t)sc->groups.size();
        for (int64_t g = 0; g < ng; g++) {
            if (group_first) group_first[g] = sc->groups[g].first;
            if (group_last) group_last[g] = sc->groups[g].second;
            if (block_offset) block_offset[g] = sc->block_offset[g];
        }
        if (pages)
            for (size_t q = 0; q < sc->pages.size(); q++) pages[q] = sc->pages[q];
        if (n_pages) *n_pages = (int64_t)sc->pages.size();
    });
    return ng;
}

// SPGrid KAT helpers (precision 4 -> float layout, 8 -> double layout)
uint64_t orc_linear_offset(int precision, int i, int j, int k)
{
    return precision == 4 ? Layout<6>::linear_offset(i, j, k) : Layout<7>::linear_offset(i, j, k);
}
uint64_t orc_packed_add(int precision, uint64_t a, uint64_t b)
{
    return precision == 4 ? Layout<6>::packed_add(a, b) : Layout<7>::packed_add(a, b);
}
void orc_masks(int precision, uint64_t* out6)
{
    if (precision == 4) {
        using L = Layout<6>;
        uint64_t v[6] = { L::xmask, L::ymask, L::zmask, (uint64_t)L::block_bits, (uint64_t)L::data_bits, (uint64_t)L::index_bits };
        std::memcpy(out6, v, sizeof v);
    }
    else {
        using L = Layout<7>;
        uint64_t v[6] = { L::xmask, L::ymask, L::zmask, (uint64_t)L::block_bits, (uint64_t)L::data_bits, (uint64_t)L::index_bits };
        std::memcpy(out6, v, sizeof v);
    }
}

// 3x3 SVD and polar on one matrix (row-major), for unit tests of the restatement.
void orc_svd3(int precision, const double* A, double* U, double* sigma, double* V)
{
    auto run = [&](auto zero) {
        using T = decltype(zero);
        M3<T> a, u, vv;
        T s[3];
        for (int i = 0; i < 9; i++) a.a[i] = (T)A[i];
        svd3(a, u, s, vv);
        for (int i = 0; i < 9; i++) {
            U[i] = u.a[i];
            V[i] = vv.a[i];
        }
        for (int i = 0; i < 3; i++) sigma[i] = s[i];
    };
    if (precision == 4)
        run(0.0f);
    else
        run(0.0);
}

// Kirchhoff stress of one model at one F (row-major), for unit tests: g = degradation, effective = the
// undegraded isotropic form the damage update uses. Returns J as the model defines it.
double orc_tau(int precision, int model, double E, double nu, double kx_scale, double ky_scale, double g, int effective, const double* F, double* tau)
{
    double J = 0;
    auto run = [&](auto zero) {
        using T = decltype(zero);
        Material<T> mt;
        mt.model = model;
        T Et = (T)E, nut = (T)nu;
        mt.lambda = Et * nut / (((T)1 + nut) * ((T)1 - (T)2 * nut));
        mt.mu = Et / ((T)2 * ((T)1 + nut));
        mt.kappa = (T).666666 * mt.mu + mt.lambda;
        mt.kx = (T)kx_scale * mt.mu;
        mt.ky = (T)ky_scale * mt.mu;
        M3<T> f, t;
        for (int i = 0; i < 9; i++) f.a[i] = (T)F[i];
        T Jm = det(f);
        if (model == MODEL_COROTATED)
            t = tau_corotated(mt, f);
        else if (model == MODEL_QRNH)
            t = tau_qrnh(mt, f, (T)g, effective != 0, &Jm);
        else
            t = tau_nhb(mt, f, effective ? (T)1 : (T)g);
        for (int i = 0; i < 9; i++) tau[i] = t.a[i];
        J = Jm;
    };
    if (precision == 4)
        run(0.0f);
    else
        run(0.0);
    return J;
}

// FP64-accumulated reductions (MpmSimulationDataAnalysis.h:67-151): out = {mass, px, py, pz, kinetic energy, max speed}
void orc_reductions(void* hp, double* out)
{
    Handle* h = (Handle*)hp;
    DISPATCH(h, {
        double M = 0, P[3] = { 0, 0, 0 }, KE = 0, vmax = 0;
        for (int64_t p = 0; p < sc->n; p++) {
            double mm = sc->m[p];
            M += mm;
            double s2 = 0;
            for (int a = 0; a < 3; a++) {
                P[a] += mm * (double)sc->v[p][a];
                s2 += (double)sc->v[p][a] * (double)sc->v[p][a];
            }
            KE += 0.5 * mm * s2;
            vmax = std::max(vmax, std::sqrt(s2));
        }
        out[0] = M;
        out[1] = P[0];
        out[2] = P[1];
        out[3] = P[2];
        out[4] = KE;
        out[5] = vmax;
    });
}

// Seeded inputs of a box or slab of size[3] metres centred at center[3], snapped to whole cells of dx, ppc_side^3
// particles per cell. kind 0: elastic box (F = I, sigma_c = 1); kind 1: fibre slab (F from a vMF(kappa) fibre
// about +x, sigma_c ~ N(sc_mean, sc_std)). Any output may be NULL. Returns the particle count; with x == NULL only
// the count is computed. lo_cell (3 ints, may be NULL) receives the first cell of the lattice.
int64_t orc_seeded_inputs(int kind, int ppc_side, uint64_t seed, double dx, const double* size, const double* center, const double* vel, double rho,
    double kappa, double sc_mean, double sc_std, double* x, double* v, double* m, double* V0, double* F, double* sigma_c, int64_t* lo_cell)
{
    if (!(dx > 0) || ppc_side <= 0) return -1;
    int64_t nc[3], lo[3];
    for (int a = 0; a < 3; a++) {
        nc[a] = std::max<int64_t>(1, std::llround(size[a] / dx));
        lo[a] = std::llround((center[a] - 0.5 * (double)nc[a] * dx) / dx);
        if (lo_cell) lo_cell[a] = lo[a];
    }
    const int64_t per = (int64_t)ppc_side * ppc_side * ppc_side, count = nc[0] * nc[1] * nc[2] * per;
    if (!x) return count;
    const double h = dx / ppc_side, vol = dx * dx * dx / (double)per;
    SeedStream rs(seed);
    int64_t p = 0;
    for (int64_t i = 0; i < nc[0]; i++)
        for (int64_t j = 0; j < nc[1]; j++)
            for (int64_t k = 0; k < nc[2]; k++)
                for (int64_t sub = 0; sub < per; sub++, p++) {
                    const int64_t cell[3] = { lo[0] + i, lo[1] + j, lo[2] + k };
                    const int64_t sl[3] = { sub / (ppc_side * ppc_side), (sub / ppc_side) % ppc_side, sub % ppc_side };
                    for (int a = 0; a < 3; a++) {
                        const double u = rs.u01();
                        const double base = (double)cell[a] * dx, off = ((double)sl[a] + u) * h;
                        x[3 * p + a] = base + off;
                        if (v) v[3 * p + a] = vel[a];
                    }
                    if (m) m[p] = rho * vol;
                    if (V0) V0[p] = vol;
                    double Fp[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 }, sc = 1.0;
                    if (kind == 1) {
                        double dir[3];
                        rs.fibre(kappa, dir);
                        rotated_F(dir, Fp);
                        sc = sc_mean + sc_std * rs.gauss();
                    }
                    if (F) std::memcpy(F + 9 * p, Fp, sizeof Fp);
                    if (sigma_c) sigma_c[p] = sc;
                }
    return count;
}

// One grid node through the collision objects (multiObjectCollision): objs holds per object origin[3],
// normal[3] (normalised here, as HalfSpace does), velocity[3], friction and type (11 doubles).
void orc_collide(int precision, int n_obj, const double* objs, double time, const double* x, double* v)
{
    auto run = [&](auto zero) {
        using T = decltype(zero);
        std::vector<HalfSpace<T>> hs(n_obj);
        for (int k = 0; k < n_obj; k++) {
            const double* o = objs + 11 * k;
            double nn = std::sqrt(o[3] * o[3] + o[4] * o[4] + o[5] * o[5]);
            for (int a = 0; a < 3; a++) {
                hs[k].o[a] = (T)o[a];
                hs[k].n[a] = (T)(o[3 + a] / nn);
                hs[k].vel[a] = (T)o[6 + a];
            }
            hs[k].friction = (T)o[9];
            hs[k].type = (int)o[10];
        }
        T xt[3] = { (T)x[0], (T)x[1], (T)x[2] }, vt[3] = { (T)v[0], (T)v[1], (T)v[2] };
        multi_object_collision(hs, (T)time, xt, vt);
        for (int a = 0; a < 3; a++) v[a] = (double)vt[a];
    };
    if (precision == 4)
        run(0.0f);
    else
        run(0.0);
}

// The damage drive D~ = zeta <phi - 1> of one particle (AnisoFractureSimulation.h:224-270) with a damaged model
// (1 Neo-Hookean Borden, 2 QR-stable with fibre stiffness kx_scale mu), for unit tests and fixtures.
double orc_damage_drive(int precision, int model, double E, double nu, double kx_scale, double alpha, double zeta, double sigma_c, const double* F)
{
    double out = 0;
    auto run = [&](auto zero) {
        using T = decltype(zero);
        Scene<T> sc;
        Material<T> mt{};
        mt.model = model;
        T Et = (T)E, nut = (T)nu;
        mt.lambda = Et * nut / (((T)1 + nut) * ((T)1 - (T)2 * nut));
        mt.mu = Et / ((T)2 * ((T)1 + nut));
        mt.kappa = (T).666666 * mt.mu + mt.lambda;
        mt.kx = (T)kx_scale * mt.mu;
        mt.damage = 1;
        mt.alpha = (T)alpha;
        mt.zeta = (T)zeta;
        sc.materials.push_back(mt);
        M3<T> f;
        for (int i = 0; i < 9; i++) f.a[i] = (T)F[i];
        sc.F.push_back(f);
        sc.sigc.push_back((T)sigma_c);
        sc.mat.push_back(0);
        sc.n = 1;
        out = (double)sc.dtilde_of(0);
    };
    if (precision == 4)
        run(0.0f);
    else
        run(0.0);
    return out;
}

int orc_num_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
