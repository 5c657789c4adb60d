// Kernels and host orchestration of the GB300 explicit-MPM substep (templated on the scalar type).
// Included by engine_f32.cu and engine_f64.cu, which instantiate one precision each.
//
// One substep (MpmSimulationBase::advanceOneTimeStep, MpmSimulationBase.cpp:262-357, with the
// AnisoFractureSimulation particlesToGrid override, AnisoFractureSimulation.h:129-141):
//   1. sort      CUB radix sort of the 64-bit particle keys written by the previous G2P (or k_keys)
//   2. groups    CUB select of the first sorted index of every (scene, SPGrid page)
//   3. activate  every group inserts its page and the 7 pages at +1 block into a hash table; new
//                entries get a grid slot (MpmGrid::pollute, MpmGrid.h:153-193)
//   4. p2g       one CTA per group: stress V0*tau(F, g(d)) + APIC scatter of m, m v + m C (x_i - x_p),
//                -V0 tau grad w and the phase-field pair (d w, w) into a shared node tile, then
//                vector atomics into the 8 neighbouring grid blocks (MpmSimulationBase.cpp:669-855,
//                FBasedMpmForceHelper.cpp:43-63, AnisoFractureSimulation.h:161-176)
//   5. grid      v = m v / m, v += g dt + f dt / m, half-space BCs, phase field normalised; clears the
//                accumulators and the hash table for the next substep (MpmSimulationBase.cpp:655-666,
//                1179-1228, AnisoFractureSimulation.h:177-179)
//   6. g2p       one CTA per group: gather v, C (APIC/RPIC blend), grad v and the damage Laplacian,
//                damage update with the old F, F <- (I + dt grad v) F, x += dt v, CFL / finiteness /
//                domain checks, next key; writes the particle to its sorted slot of the other buffer
//                (MpmSimulationBase.cpp:1269-1515, FBasedMpmForceHelper.cpp:95-108,
//                AnisoFractureSimulation.h:182-283)
//   7. end       time += dt per scene, substep counter
#pragma once
#include "common.cuh"
#include "engine.h"
#include "physics.cuh"

#include <cub/cub.cuh>
#include <cuda_runtime.h>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace zr {

constexpr int NACC = 6; // m, m v + dt f (3), d w, w
constexpr int NVEL = 4; // v_new (3), normalised phase field
constexpr uint64_t HASH_EMPTY = ~0ULL;
constexpr int HASH_PROBES = 64;

// particle pool: field k of storage slot i at f[k * stride + i]
enum { P_X = 0, P_V = 3, P_C = 6, P_F = 15, P_M = 24, P_V0 = 25, P_D = 26, P_SC = 27, P_NF = 28 };

template <class T>
struct Pool {
    T* f;
    uint32_t* pid; // original index (low index_bits) | material << index_bits
    int64_t stride;
};

struct KeyLayout {
    int ib; // bits of the original particle index
    int cp; // bits of (offset >> data_bits): page and in-block cell
    int sb; // bits of the scene slot
    int block_bits;
    __host__ __device__ int total() const { return sb + cp + ib; }
    __host__ __device__ uint32_t scene(uint64_t k) const { return (uint32_t)(k >> (cp + ib)); }
    __host__ __device__ uint64_t page(uint64_t k) const { return (k >> (ib + block_bits)) & ((1ULL << (cp - block_bits)) - 1); }
    __host__ __device__ uint64_t group(uint64_t k) const { return k >> (ib + block_bits); }
    __host__ __device__ uint32_t orig(uint64_t k) const { return (uint32_t)(k & ((1ULL << ib) - 1)); }
};

template <class T>
struct StepArgs {
    const uint64_t* keys_sorted;
    const uint32_t* vals_sorted;
    uint64_t* keys_next;
    Pool<T> pin, pout;
    const uint32_t* g_start;
    int32_t* g_nbr;
    uint64_t* b_key;
    T* acc;
    T* vel;
    uint64_t* h_keys;
    int32_t* h_vals;
    uint32_t h_mask;
    SceneParams<T>* scenes;
    double* grid_mass; // per scene, refreshed every substep
    DevStatus* st;
    uint32_t n_total;
    uint32_t b_cap;
    KeyLayout kl;
};

__host__ __device__ inline uint64_t hash64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

__device__ inline void raise_flag(DevStatus* st, uint32_t f)
{
    uint32_t old = atomicOr(&st->flags, f | ((f & ABORTING) ? FLAG_ABORT : 0u));
    if ((f & ABORTING) && !(old & FLAG_ABORT)) atomicExch(&st->abort_step, (int32_t)st->step);
}

__device__ inline bool aborted(const DevStatus* st) { return (*(volatile const uint32_t*)&st->flags & FLAG_ABORT) != 0; }

// the same decision for every thread of the CTA (kernels with barriers or full-warp shuffles must not
// let some threads leave early)
__device__ inline bool aborted_cta(const DevStatus* st)
{
    __shared__ int s_abort;
    if (threadIdx.x == 0) s_abort = aborted(st) ? 1 : 0;
    __syncthreads();
    bool r = s_abort != 0;
    __syncthreads();
    return r;
}

__device__ inline int hash_find(const uint64_t* hk, const int32_t* hv, uint32_t mask, uint64_t key)
{
    uint32_t h = (uint32_t)hash64(key) & mask;
    for (int p = 0; p < HASH_PROBES; p++) {
        uint64_t k = hk[h];
        if (k == key) return hv[h];
        if (k == HASH_EMPTY) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}

// ---------------------------------------------------------------------------------------------------
// keys of the current particle positions (used after a load or a host upload; afterwards G2P writes
// the keys of the next substep). Also checks that every base node lies in its scene's domain.
// ---------------------------------------------------------------------------------------------------
template <class T>
__global__ void k_keys(Pool<T> p, const SceneParams<T>* scenes, int n_scenes, uint64_t* keys, uint32_t n_total, KeyLayout kl, DevStatus* st)
{
    using L = typename LayoutOf<T>::type;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_total; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = n_scenes - 1; // scene owning storage slot i
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (scenes[mid].first <= (int64_t)i) lo = mid;
            else hi = mid - 1;
        }
        const SceneParams<T>& sp = scenes[lo];
        int b[3];
        bool ok = true;
        for (int a = 0; a < 3; a++) {
            T x = p.f[(P_X + a) * p.stride + i];
            b[a] = base_node(x, sp.inv_dx);
            ok = ok && (x == x) && b[a] >= 0 && b[a] < sp.domain_cells - 3;
        }
        if (!ok) {
            raise_flag(st, FLAG_OUT_OF_DOMAIN);
            b[0] = b[1] = b[2] = 0;
        }
        keys[i] = ((uint64_t)lo << (kl.cp + kl.ib)) | ((L::offset(b[0], b[1], b[2]) >> L::data_bits) << kl.ib);
    }
}

// The hot-path keys hold (scene, page, cell) only, so the radix sort needs 4 passes instead of 7; a
// stable sort of storage-ordered input leaves the particles of one cell in their previous order. This pass
// restores the reference's order inside each cell (ascending original index, the low bits of the
// reference key, MpmSimulationBase.cpp:1547-1552) with an insertion sort per run of equal keys; runs are
// short (~8) and nearly sorted (a cell keeps most of its particles from one substep to the next).
template <class T>
__global__ void k_cellfix(const uint64_t* ks, uint32_t* vals, const uint32_t* pid, uint32_t n)
{
    using L = typename LayoutOf<T>::type;
    const uint32_t mask = (1u << L::index_bits) - 1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = ks[i];
        if (i > 0 && ks[i - 1] == k) continue; // not the first of its run
        uint32_t e = i + 1;
        while (e < n && ks[e] == k) e++;
        for (uint32_t q = i + 1; q < e; q++) {
            const uint32_t v = vals[q], o = pid[v] & mask;
            uint32_t r = q;
            while (r > i) {
                const uint32_t u = vals[r - 1];
                if ((pid[u] & mask) <= o) break;
                vals[r] = u;
                r--;
            }
            vals[r] = v;
        }
    }
}

// group heads of the sorted keys: first index of every (scene, page)
struct GroupHead {
    const uint64_t* k;
    KeyLayout kl;
    __device__ bool operator()(uint32_t i) const { return i == 0 || kl.group(k[i]) != kl.group(k[i - 1]); }
};

template <class T>
__global__ void k_activate(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    if (aborted(a.st)) return;
    const uint32_t G = a.st->n_groups;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->max_groups_seen = max(a.st->max_groups_seen, G);
    if (G > a.b_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) raise_flag(a.st, FLAG_CAPACITY);
        return;
    }
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < G * 8; t += gridDim.x * blockDim.x) {
        uint32_t g = t >> 3, dl = t & 7;
        uint64_t key0 = a.keys_sorted[a.g_start[g]];
        uint64_t scene = a.kl.scene(key0);
        uint32_t bi, bj, bk;
        L::block_of_page(a.kl.page(key0), bi, bj, bk);
        uint64_t hk = (scene << 40) | L::page_of_block(bi + (dl >> 2), bj + ((dl >> 1) & 1), bk + (dl & 1));
        uint32_t h = (uint32_t)hash64(hk) & a.h_mask;
        bool done = false;
        for (int p = 0; p < HASH_PROBES && !done; p++) {
            unsigned long long prev = atomicCAS((unsigned long long*)&a.h_keys[h], (unsigned long long)HASH_EMPTY, (unsigned long long)hk);
            if (prev == HASH_EMPTY) {
                uint32_t slot = atomicAdd(&a.st->n_blocks, 1u);
                if (slot >= a.b_cap) {
                    raise_flag(a.st, FLAG_CAPACITY);
                    a.h_vals[h] = -1;
                }
                else {
                    a.h_vals[h] = (int32_t)slot;
                    a.b_key[slot] = hk;
                }
                done = true;
            }
            else if (prev == hk)
                done = true;
            else
                h = (h + 1) & a.h_mask;
        }
        if (!done) raise_flag(a.st, FLAG_CAPACITY);
    }
}

// ---------------------------------------------------------------------------------------------------
// P2G
// ---------------------------------------------------------------------------------------------------
template <class T>
__device__ inline void flush_column(T* dst, const T* src, int n)
{
    if constexpr (std::is_same<T, float>::value) {
        if (n == 4) {
            float4 v = make_float4(src[0], src[1], src[2], src[3]);
            if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd((float4*)dst, v);
        }
        else {
            float2 v = make_float2(src[0], src[1]);
            if (v.x != 0.f || v.y != 0.f) atomicAdd((float2*)dst, v);
        }
    }
    else {
        for (int q = 0; q < n; q++)
            if (src[q] != (T)0) atomicAdd(dst + q, src[q]);
    }
}

// P2G with no atomics in the hot loop. For every group (one occupied SPGrid block):
//   phase 1 (thread per particle): stress and a 26-value payload per particle, staged in shared memory
//   phase 2 (thread per cell and x-offset of the stencil): the particles of one cell all share the same
//           27 nodes, so each thread accumulates its 9 nodes x 6 fields in registers over the cell's
//           particles (deterministic order, no conflicts)
//   phase 3: one shared add per node and field (distinct nodes within a warp), then vector atomics of
//           the 6x6x6 node tile into the 8 neighbouring grid blocks
// Payload: fractional index-space position f = x/dx - base, m, A = m v - dx (m C) f,
// Bc = dx m C, K = -dt V0 tau / dx, d. With xm = (delta - f) dx for stencil offset delta:
//   m v + m C xm = A + Bc delta  and  dt f_i = K . (dw_i w_j w_k, w_i dw_j w_k, w_i w_j dw_k),
// so the node receives m w, w (A + Bc delta) + K grad-hat w, d w and w. The force enters the
// momentum directly (m v + dt f), which the grid update turns into v + f dt/m + g dt as the reference's
// gridVelocityExplicitUpdate does (MpmSimulationBase.cpp:1197-1226).
constexpr int NPAY = 26;
enum { Y_F = 0, Y_M = 3, Y_A = 4, Y_B = 7, Y_K = 16, Y_D = 25 };

template <class T>
struct P2GShape {
    using L = typename LayoutOf<T>::type;
    static constexpr int NT = 3 * L::nodes; // cells x stencil x-offsets
    static constexpr int CHUNK = std::is_same<T, float>::value ? 512 : 256;
    static constexpr int CPAD = CHUNK + CHUNK / 8;
    static constexpr size_t dyn_bytes = sizeof(T) * NPAY * CPAD;
};

__device__ __forceinline__ int pay_slot(int q) { return q + (q >> 3); } // bank swizzle: cells hold ~8 particles

// MODELS: bit 0 = fixed corotated present in the batch, bit 1 = Neo-Hookean (Borden) present; a batch
// with one model kind runs a kernel without the other model's code (fewer registers).
template <class T, int MODELS>
__global__ void __launch_bounds__(P2GShape<T>::NT, 2) k_p2g(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using S = P2GShape<T>;
    constexpr int NT = S::NT, CHUNK = S::CHUNK, CPAD = S::CPAD, NC = L::nodes;
    constexpr int TX = L::sx + 2, TY = L::sy + 2, TZ = L::sz + 2, TN = TX * TY * TZ;
    extern __shared__ __align__(16) unsigned char p2g_dyn[];
    T* pay = reinterpret_cast<T*>(p2g_dyn);
    __shared__ T tile[NACC * TN];
    __shared__ uint8_t cellof[CHUNK];
    __shared__ int16_t cfirst[NC], clast[NC];
    __shared__ int s_g, s_nbr[8], s_scene;
    __shared__ int s_org[3];
    if (aborted_cta(a.st)) return;
    const uint32_t G = a.st->n_groups;
    const int tid = threadIdx.x;
    // phase-2 role of this thread: cell c, stencil x-offset ii
    const int ii = tid / NC, c = tid % NC;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    for (;;) {
        if (tid == 0) s_g = (int)atomicAdd(&a.st->work_p2g, 1u);
        __syncthreads();
        const int g = s_g;
        if (g >= (int)G) break;
        const uint32_t start = a.g_start[g], end = (g + 1 < (int)G) ? a.g_start[g + 1] : a.n_total;
        if (tid < 8) {
            uint64_t key0 = a.keys_sorted[start];
            uint64_t scene = a.kl.scene(key0);
            uint32_t bi, bj, bk;
            L::block_of_page(a.kl.page(key0), bi, bj, bk);
            int dl = tid;
            uint64_t hk = (scene << 40) | L::page_of_block(bi + (dl >> 2), bj + ((dl >> 1) & 1), bk + (dl & 1));
            int slot = hash_find(a.h_keys, a.h_vals, a.h_mask, hk);
            if (slot < 0) raise_flag(a.st, FLAG_CAPACITY);
            s_nbr[dl] = slot;
            a.g_nbr[g * 8 + dl] = slot;
            if (dl == 0) {
                s_scene = (int)scene;
                s_org[0] = (int)(bi * L::sx);
                s_org[1] = (int)(bj * L::sy);
                s_org[2] = (int)(bk * L::sz);
            }
        }
        for (int q = tid; q < NACC * TN; q += NT) tile[q] = (T)0;
        __syncthreads();
        bool bad_slot = false;
        for (int d = 0; d < 8; d++) bad_slot |= s_nbr[d] < 0;
        const SceneParams<T>& sp = a.scenes[s_scene];
        const T dx = sp.dx, inv_dx = sp.inv_dx, dt = sp.dt;
        const bool damage = sp.damage != 0;
        const int nf = damage ? NACC : 4;
        for (uint32_t c0 = start; c0 < end && !bad_slot; c0 += CHUNK) {
            const int cnt = (int)min((uint32_t)CHUNK, end - c0);
            // ---- phase 1: per particle
            if (tid < NC) {
                cfirst[tid] = 0;
                clast[tid] = 0;
            }
            const Pool<T>& P = a.pin;
            for (int q = tid; q < cnt; q += NT) {
                const uint32_t j = a.vals_sorted[c0 + q];
                T x[3], v[3], Cm[9], F[9];
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    x[e] = P.f[(P_X + e) * P.stride + j];
                    v[e] = P.f[(P_V + e) * P.stride + j];
                }
#pragma unroll
                for (int e = 0; e < 9; e++) {
                    Cm[e] = P.f[(P_C + e) * P.stride + j];
                    F[e] = P.f[(P_F + e) * P.stride + j];
                }
                const T mass = P.f[P_M * P.stride + j], V0 = P.f[P_V0 * P.stride + j];
                const T dd = damage ? P.f[P_D * P.stride + j] : (T)0;
                const uint32_t mat = P.pid[j] >> L::index_bits;
                const Material<T>& mt = sp.materials[mat < (uint32_t)sp.n_materials ? mat : 0];
                T tau[9];
                if (MODELS == 1 || (MODELS == 3 && mt.model == MODEL_COROTATED)) {
                    if (tau_corotated(mt, F, tau)) atomicAdd(&a.st->fallback, 1u);
                }
                else
                    tau_nhb(mt, F, (damage && mt.damage) ? degradation(dd, mt.residual) : (T)1, tau);
                T fr[3];
                int l[3];
#pragma unroll
                for (int e = 0; e < 3; e++) {
                    const T xs = mul_rn(x[e], inv_dx);
                    const int b = int_floor(sub_rn(xs, (T)0.5));
                    fr[e] = xs - (T)b;
                    l[e] = b - s_org[e];
                }
                const bool inside = l[0] >= 0 && l[0] < L::sx && l[1] >= 0 && l[1] < L::sy && l[2] >= 0 && l[2] < L::sz;
                if (!inside) raise_flag(a.st, FLAG_CAPACITY); // keys and positions disagree: abort the substep
                cellof[q] = inside ? (uint8_t)L::element(l[0], l[1], l[2]) : (uint8_t)0xff;
                T* y = pay + pay_slot(q);
                const T kf = -dt * V0 * inv_dx;
#pragma unroll
                for (int e = 0; e < 3; e++) y[(Y_F + e) * CPAD] = fr[e];
                y[Y_M * CPAD] = mass;
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    const T m0 = mass * Cm[3 * r], m1 = mass * Cm[3 * r + 1], m2 = mass * Cm[3 * r + 2];
                    y[(Y_A + r) * CPAD] = mass * v[r] - dx * (m0 * fr[0] + m1 * fr[1] + m2 * fr[2]);
                    y[(Y_B + 3 * r) * CPAD] = dx * m0;
                    y[(Y_B + 3 * r + 1) * CPAD] = dx * m1;
                    y[(Y_B + 3 * r + 2) * CPAD] = dx * m2;
                    y[(Y_K + 3 * r) * CPAD] = kf * tau[3 * r];
                    y[(Y_K + 3 * r + 1) * CPAD] = kf * tau[3 * r + 1];
                    y[(Y_K + 3 * r + 2) * CPAD] = kf * tau[3 * r + 2];
                }
                y[Y_D * CPAD] = dd;
            }
            __syncthreads();
            // particles of one cell are contiguous (sorted by cell inside the block)
            for (int q = tid; q < cnt; q += NT) {
                const int e = cellof[q];
                if (e == 0xff) continue;
                if (q == 0 || cellof[q - 1] != e) cfirst[e] = (int16_t)q;
                if (q == cnt - 1 || cellof[q + 1] != e) clast[e] = (int16_t)(q + 1);
            }
            __syncthreads();
            // ---- phase 2: per (cell, stencil x-offset), register accumulators of the thread's 9 nodes
            if (ii < 3) {
                T acc[9][NACC];
#pragma unroll
                for (int n = 0; n < 9; n++)
#pragma unroll
                    for (int f = 0; f < NACC; f++) acc[n][f] = (T)0;
                const int q1 = clast[c];
                for (int q = cfirst[c]; q < q1; q++) {
                    const T* y = pay + pay_slot(q);
                    T w[3][3], dw[3][3];
#pragma unroll
                    for (int e = 0; e < 3; e++) {
                        const T d0 = y[(Y_F + e) * CPAD];
                        const T z = (T)1.5 - d0, d1 = d0 - (T)1, zz = d0 - (T)0.5;
                        w[e][0] = (T)0.5 * z * z;
                        w[e][1] = (T)0.75 - d1 * d1;
                        w[e][2] = (T)0.5 * zz * zz;
                        dw[e][0] = -z;
                        dw[e][1] = (T)-2 * d1;
                        dw[e][2] = zz;
                    }
                    const T wx = ii == 0 ? w[0][0] : (ii == 1 ? w[0][1] : w[0][2]);
                    const T dwx = ii == 0 ? dw[0][0] : (ii == 1 ? dw[0][1] : dw[0][2]);
                    const T mass = y[Y_M * CPAD];
                    const T dd = y[Y_D * CPAD];
                    T Ai[3], B1[3], B2[3], K0[3], K1[3], K2[3];
#pragma unroll
                    for (int r = 0; r < 3; r++) {
                        Ai[r] = y[(Y_A + r) * CPAD] + (T)ii * y[(Y_B + 3 * r) * CPAD];
                        B1[r] = y[(Y_B + 3 * r + 1) * CPAD];
                        B2[r] = y[(Y_B + 3 * r + 2) * CPAD];
                        K0[r] = y[(Y_K + 3 * r) * CPAD];
                        K1[r] = y[(Y_K + 3 * r + 1) * CPAD];
                        K2[r] = y[(Y_K + 3 * r + 2) * CPAD];
                    }
                    // node (ii, jj, kk) receives, per momentum component r,
                    //   wz_k al_r(j) + k wz_k be_r(j) + dwz_k ga_r(j)   with
                    //   al = wx wy (A + j B1) + K0 dwx wy + K1 wx dwy,  be = wx wy B2,  ga = wx wy K2
#pragma unroll
                    for (int jj = 0; jj < 3; jj++) {
                        const T c0 = wx * w[1][jj], gx = dwx * w[1][jj], gy = wx * dw[1][jj];
                        T al[3], be[3], ga[3];
#pragma unroll
                        for (int r = 0; r < 3; r++) {
                            al[r] = c0 * (jj ? Ai[r] + (T)jj * B1[r] : Ai[r]) + (K0[r] * gx + K1[r] * gy);
                            be[r] = c0 * B2[r];
                            ga[r] = c0 * K2[r];
                        }
                        const T mc = mass * c0, dc = dd * c0;
#pragma unroll
                        for (int kk = 0; kk < 3; kk++) {
                            const T wk = w[2][kk], dwk = dw[2][kk];
                            T* ac = acc[jj * 3 + kk];
                            ac[0] += mc * wk;
#pragma unroll
                            for (int r = 0; r < 3; r++) ac[1 + r] += wk * al[r] + (kk ? ((T)kk * wk) * be[r] : (T)0) + dwk * ga[r];
                            if (damage) {
                                ac[4] += dc * wk;
                                ac[5] += c0 * wk;
                            }
                        }
                    }
                }
                // ---- phase 3: registers -> shared tile (distinct nodes within a warp, so no contention)
                if (q1 > cfirst[c]) {
#pragma unroll
                    for (int jj = 0; jj < 3; jj++)
#pragma unroll
                        for (int kk = 0; kk < 3; kk++) {
                            T* t = tile + ((cx + ii) * TY + (cy + jj)) * TZ + (cz + kk);
                            const T* ac = acc[jj * 3 + kk];
                            for (int f = 0; f < nf; f++) atomicAdd(t + f * TN, ac[f]);
                        }
                }
            }
            __syncthreads();
        }
        if (!bad_slot) {
            // tile -> global: z columns split at the block boundary (4 + 2 nodes)
            for (int q = tid; q < nf * TX * TY * 2; q += NT) {
                const int half = q & 1, col = q >> 1;
                const int f = col / (TX * TY), ab = col % (TX * TY), ta = ab / TY, tb = ab % TY;
                const int ax = ta >= L::sx, ay = tb >= L::sy;
                const int slot = s_nbr[ax * 4 + ay * 2 + half];
                T* dst = a.acc + ((size_t)slot * NACC + f) * L::nodes + L::element(ta - ax * L::sx, tb - ay * L::sy, 0);
                const T* src = tile + f * TN + (ta * TY + tb) * TZ + half * L::sz;
                flush_column(dst, src, half ? TZ - L::sz : L::sz);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------------------
// grid update
// ---------------------------------------------------------------------------------------------------
template <class T>
__global__ void k_grid(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    if (aborted_cta(a.st)) return;
    const uint32_t B = min(a.st->n_blocks, a.b_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->max_blocks_seen = max(a.st->max_blocks_seen, B);
    const uint32_t total = B * L::nodes;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ((total + 31) & ~31u); t += gridDim.x * blockDim.x) {
        T gm = 0;
        int scene = -1;
        if (t < total) {
            const uint32_t b = t / L::nodes, e = t % L::nodes;
            const uint64_t hk = a.b_key[b];
            scene = (int)(hk >> 40);
            const SceneParams<T>& sp = a.scenes[scene];
            T* A = a.acc + (size_t)b * NACC * L::nodes + e;
            T m = A[0];
            T P[3] = { A[L::nodes], A[2 * L::nodes], A[3 * L::nodes] };
            T pf = A[4 * L::nodes], pfm = A[5 * L::nodes];
#pragma unroll
            for (int q = 0; q < NACC; q++) A[q * L::nodes] = (T)0;
            T* V = a.vel + (size_t)b * NVEL * L::nodes + e;
            gm = m;
            if (m != (T)0) {
                uint32_t bi, bj, bk;
                L::block_of_page(hk & ((1ULL << 40) - 1), bi, bj, bk);
                const int lx = e >> (L::zbits + L::ybits), ly = (e >> L::zbits) & (L::sy - 1), lz = e & (L::sz - 1);
                const T xi[3] = { (T)(bi * L::sx + lx) * sp.dx, (T)(bj * L::sy + ly) * sp.dx, (T)(bk * L::sz + lz) * sp.dx };
                const T dt = sp.dt;
                T vi[3];
                // P = m v + dt f: v + g dt + f dt / m (MpmSimulationBase.cpp:1204-1210)
#pragma unroll
                for (int c = 0; c < 3; c++) vi[c] = P[c] / m + sp.gravity[c] * dt;
                collide(sp, (T)sp.time, xi, vi);
                V[0] = vi[0];
                V[L::nodes] = vi[1];
                V[2 * L::nodes] = vi[2];
                V[3 * L::nodes] = pfm != (T)0 ? pf / pfm : (T)0;
            }
            else {
                V[0] = V[L::nodes] = V[2 * L::nodes] = V[3 * L::nodes] = (T)0;
            }
        }
        // grid mass per scene: nodes of one warp share a block (and so a scene) whenever L::nodes >= 32
        double s = (double)gm;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        int sc0 = __shfl_sync(0xffffffffu, scene, 0);
        if ((threadIdx.x & 31) == 0 && sc0 >= 0) atomicAdd(&a.grid_mass[sc0], s);
    }
    // the hash table is used only by activate and P2G: clear it for the next substep
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= a.h_mask; h += gridDim.x * blockDim.x) a.h_keys[h] = HASH_EMPTY;
}

// ---------------------------------------------------------------------------------------------------
// G2P
// ---------------------------------------------------------------------------------------------------
template <class T, int NT>
__global__ void __launch_bounds__(NT, 4) k_g2p(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    __shared__ __align__(16) T sv[8 * NVEL * L::nodes];
    __shared__ int s_g, s_nbr[8], s_scene, s_org[3];
    if (aborted_cta(a.st)) return;
    const uint32_t G = a.st->n_groups;
    const KeyLayout kl = a.kl;
    for (;;) {
        if (threadIdx.x == 0) s_g = (int)atomicAdd(&a.st->work_g2p, 1u);
        __syncthreads();
        const int g = s_g;
        if (g >= (int)G) break;
        const uint32_t start = a.g_start[g], end = (g + 1 < (int)G) ? a.g_start[g + 1] : a.n_total;
        if (threadIdx.x < 8) {
            s_nbr[threadIdx.x] = a.g_nbr[g * 8 + threadIdx.x];
            if (threadIdx.x == 0) {
                uint64_t key0 = a.keys_sorted[start];
                uint32_t bi, bj, bk;
                L::block_of_page(kl.page(key0), bi, bj, bk);
                s_scene = (int)kl.scene(key0);
                s_org[0] = (int)(bi * L::sx);
                s_org[1] = (int)(bj * L::sy);
                s_org[2] = (int)(bk * L::sz);
            }
        }
        __syncthreads();
        // stage the velocities of the 8 neighbouring blocks (1 KiB contiguous per block, 16-byte loads)
        {
            constexpr int V4 = NVEL * L::nodes * (int)sizeof(T) / 16; // 16-byte words per block
            uint4* dst = reinterpret_cast<uint4*>(sv);
            for (int q = threadIdx.x; q < 8 * V4; q += NT) {
                const int d = q / V4, r = q % V4;
                const int slot = s_nbr[d];
                dst[q] = slot >= 0 ? reinterpret_cast<const uint4*>(a.vel + (size_t)slot * NVEL * L::nodes)[r] : make_uint4(0, 0, 0, 0);
            }
        }
        __syncthreads();
        const SceneParams<T>& sp = a.scenes[s_scene];
        const T dx = sp.dx, inv_dx = sp.inv_dx, dt = sp.dt, D_inv = sp.D_inv;
        const T ca = sp.apic_a, cb = sp.apic_b;
        const bool damage = sp.damage != 0;
        const T dx2 = dx * dx, half_cfl2 = dx2 * (T)0.25 * (sp.cfl * sp.cfl);
        const Pool<T>& P = a.pin;
        const Pool<T>& Q = a.pout;
        uint32_t flags = 0;
        for (uint32_t i = start + threadIdx.x; i < end; i += NT) {
            const uint32_t j = a.vals_sorted[i];
            // every particle load is issued here, so one memory latency covers them all
            T x[3], F[9];
#pragma unroll
            for (int c = 0; c < 3; c++) x[c] = P.f[(P_X + c) * P.stride + j];
#pragma unroll
            for (int c = 0; c < 9; c++) F[c] = P.f[(P_F + c) * P.stride + j];
            const uint32_t pid = P.pid[j];
            const T pm = P.f[P_M * P.stride + j], pV0 = P.f[P_V0 * P.stride + j];
            T dd = damage ? P.f[P_D * P.stride + j] : (T)0;
            const T sc = damage ? P.f[P_SC * P.stride + j] : (T)0;
            int b[3], l[3];
            T w[3][3], dw[3][3], fr[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                T xs = mul_rn(x[c], inv_dx);
                b[c] = int_floor(sub_rn(xs, (T)0.5));
                bspline_w(xs, b[c], w[c], dw[c]);
                fr[c] = xs - (T)b[c];
                l[c] = b[c] - s_org[c];
            }
            if (l[0] < 0 || l[0] >= L::sx || l[1] < 0 || l[1] >= L::sy || l[2] < 0 || l[2] >= L::sz) {
                flags |= FLAG_CAPACITY; // a particle outside its group's block: keys and positions disagree
                continue;
            }
            // Separable gather: the stencil weight is wx_i wy_j wz_k, so sums over k, then j, then i give
            //   pv = sum w v,  M_rc = sum w v_r delta_c,  G_rc = sum v_r (grad w)_c dx,
            // and the APIC moment sum w v (x_i - x_p)^T = dx (M - pv fr^T) because x_i - x_p = (delta - fr) dx.
            T pv[3] = { 0, 0, 0 }, M[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 }, Gv[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 }, lap = 0;
#pragma unroll
            for (int ii = 0; ii < 3; ii++) {
                const int tx = l[0] + ii, ax = tx >= L::sx, ex = tx - ax * L::sx;
                T Si[3] = { 0, 0, 0 }, Ji[3] = { 0, 0, 0 }, Ki[3] = { 0, 0, 0 }, Ui[3] = { 0, 0, 0 }, Ti[3] = { 0, 0, 0 };
                T lA = 0, lB = 0, lC = 0;
#pragma unroll
                for (int jj = 0; jj < 3; jj++) {
                    const int ty = l[1] + jj, ay = ty >= L::sy, ey = ty - ay * L::sy;
                    T sj[3] = { 0, 0, 0 }, tj[3] = { 0, 0, 0 }, uj[3] = { 0, 0, 0 }, pz = 0, p1 = 0;
#pragma unroll
                    for (int kk = 0; kk < 3; kk++) {
                        const int tz = l[2] + kk, az = tz >= L::sz, ez = tz - az * L::sz;
                        const T* nv = sv + (ax * 4 + ay * 2 + az) * NVEL * L::nodes + L::element(ex, ey, ez);
                        const T wk = w[2][kk], dwk = dw[2][kk];
#pragma unroll
                        for (int r = 0; r < 3; r++) {
                            const T vr = nv[r * L::nodes];
                            sj[r] += wk * vr;
                            tj[r] += dwk * vr;
                            if (kk) uj[r] += ((T)kk * wk) * vr;
                        }
                        if (damage) {
                            const T pf = nv[3 * L::nodes];
                            pz += wk * pf;
                            p1 += pf;
                        }
                    }
                    const T wj = w[1][jj], dwj = dw[1][jj];
#pragma unroll
                    for (int r = 0; r < 3; r++) {
                        Si[r] += wj * sj[r];
                        Ui[r] += dwj * sj[r];
                        Ti[r] += wj * tj[r];
                        Ki[r] += wj * uj[r];
                        if (jj) Ji[r] += ((T)jj * wj) * sj[r];
                    }
                    if (damage) {
                        lA += wj * pz;
                        lB += pz;
                        lC += wj * p1;
                    }
                }
                const T wi = w[0][ii], dwi = dw[0][ii];
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    pv[r] += wi * Si[r];
                    if (ii) M[3 * r] += ((T)ii * wi) * Si[r];
                    M[3 * r + 1] += wi * Ji[r];
                    M[3 * r + 2] += wi * Ki[r];
                    Gv[3 * r] += dwi * Si[r];
                    Gv[3 * r + 1] += wi * Ui[r];
                    Gv[3 * r + 2] += wi * Ti[r];
                }
                // the reference's 3D Laplacian weights every term with d2w(i) = (1,-2,1)(i) (MpmGrid.h:607-613):
                // sum_jk pf * d2w_i (wy_j wz_k + wx_i wz_k + wx_i wy_j)
                if (damage) lap += (ii == 1 ? (T)-2 : (T)1) * (lA + wi * (lB + lC));
            }
            lap *= inv_dx * inv_dx;
            T Bm[9];
#pragma unroll
            for (int r = 0; r < 3; r++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    Bm[3 * r + c] = dx * (M[3 * r + c] - fr[c] * pv[r]);
                    Gv[3 * r + c] *= inv_dx;
                }
            // finish the transfer first so the gather accumulators die before the damage update
            {
                T Fn[9], A[9];
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const T cn = (ca * Bm[3 * r + c] + cb * Bm[3 * c + r]) * D_inv;
                        Q.f[(P_C + 3 * r + c) * Q.stride + i] = cn;
                        if (!isfinite(cn)) flags |= FLAG_NONFINITE;
                        A[3 * r + c] = (r == c ? (T)1 : (T)0) + dt * Gv[3 * r + c];
                    }
                mul3(A, F, Fn);
                bool finite = true;
#pragma unroll
                for (int c = 0; c < 9; c++) {
                    finite = finite && isfinite(Fn[c]);
                    Q.f[(P_F + c) * Q.stride + i] = Fn[c];
                }
                T xn[3], inc2 = 0;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    T inc = dt * pv[c];
                    inc2 += inc * inc;
                    xn[c] = x[c] + inc;
                    Q.f[(P_X + c) * Q.stride + i] = xn[c];
                    Q.f[(P_V + c) * Q.stride + i] = pv[c];
                }
                if (inc2 > dx2) flags |= FLAG_CFL;
                if (inc2 > half_cfl2) flags |= FLAG_CFL_HALF;
                if (!finite || !isfinite(inc2)) flags |= FLAG_NONFINITE;
                // key of the next substep
                int nb[3];
                bool in_dom = true;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    nb[c] = base_node(xn[c], inv_dx);
                    in_dom = in_dom && nb[c] >= 0 && nb[c] < sp.domain_cells - 3;
                }
                if (!in_dom) {
                    flags |= FLAG_OUT_OF_DOMAIN;
                    nb[0] = nb[1] = nb[2] = 0;
                }
                a.keys_next[i] = ((uint64_t)s_scene << (kl.cp + kl.ib)) | ((L::offset(nb[0], nb[1], nb[2]) >> L::data_bits) << kl.ib);
            }
            Q.f[P_M * Q.stride + i] = pm;
            Q.f[P_V0 * Q.stride + i] = pV0;
            Q.pid[i] = pid;
            if (damage) {
                // AnisoMPM damage with the F of the start of the substep (AnisoFractureSimulation.h:210-283)
                const uint32_t mat = pid >> L::index_bits;
                const Material<T>& mt = sp.materials[mat < (uint32_t)sp.n_materials ? mat : 0];
                if (mt.damage && mt.model == MODEL_NEOHOOKEAN_BORDEN) {
                    bool fb = false;
                    dd = damage_update(mt, F, dd, lap, sc, dt, fb);
                    if (fb) atomicAdd(&a.st->fallback, 1u);
                    if (!isfinite(dd)) flags |= FLAG_NONFINITE;
                }
                Q.f[P_D * Q.stride + i] = dd;
                Q.f[P_SC * Q.stride + i] = sc;
            }
        }
        if (flags) raise_flag(a.st, flags);
        __syncthreads();
    }
}

template <class T>
__global__ void k_step_end(SceneParams<T>* scenes, int n_scenes, DevStatus* st)
{
    if (aborted(st)) return;
    for (int s = threadIdx.x; s < n_scenes; s += blockDim.x) scenes[s].time += (double)scenes[s].dt;
    __syncthreads();
    if (threadIdx.x == 0) {
        st->step += 1;
        st->n_blocks = 0;
        st->work_p2g = 0;
        st->work_g2p = 0;
    }
}

template <class T>
__global__ void k_zero_grid_mass(double* gm, int n)
{
    for (int s = threadIdx.x; s < n; s += blockDim.x) gm[s] = 0;
}

// ---------------------------------------------------------------------------------------------------
// host <-> device field transfer (caller order <-> storage order via the original index)
// ---------------------------------------------------------------------------------------------------
template <class T, class O>
__global__ void k_export(Pool<T> p, int64_t first, int64_t n, int f0, int nc, O* out, int out_stride, int out_off)
{
    using L = typename LayoutOf<T>::type;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = first + i;
        const uint32_t orig = p.pid[s] & ((1u << L::index_bits) - 1);
        for (int c = 0; c < nc; c++) out[(int64_t)orig * out_stride + out_off + c] = (O)p.f[(f0 + c) * p.stride + s];
    }
}

template <class T, class I>
__global__ void k_import(Pool<T> p, int64_t first, int64_t n, int f0, int nc, const I* in, int in_stride, int in_off)
{
    using L = typename LayoutOf<T>::type;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = first + i;
        const uint32_t orig = p.pid[s] & ((1u << L::index_bits) - 1);
        for (int c = 0; c < nc; c++) p.f[(f0 + c) * p.stride + s] = (T)in[(int64_t)orig * in_stride + in_off + c];
    }
}

// FP64-accumulated particle reductions of one scene: mass, momentum (3), kinetic energy, max speed
template <class T>
__global__ void k_reduce(Pool<T> p, int64_t first, int64_t n, double* out)
{
    double M = 0, px = 0, py = 0, pz = 0, ke = 0, vmax = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = first + i;
        double m = p.f[P_M * p.stride + s];
        double vx = p.f[(P_V + 0) * p.stride + s], vy = p.f[(P_V + 1) * p.stride + s], vz = p.f[(P_V + 2) * p.stride + s];
        M += m;
        px += m * vx;
        py += m * vy;
        pz += m * vz;
        double s2 = vx * vx + vy * vy + vz * vz;
        ke += 0.5 * m * s2;
        vmax = fmax(vmax, sqrt(s2));
    }
    for (int o = 16; o > 0; o >>= 1) {
        M += __shfl_down_sync(0xffffffffu, M, o);
        px += __shfl_down_sync(0xffffffffu, px, o);
        py += __shfl_down_sync(0xffffffffu, py, o);
        pz += __shfl_down_sync(0xffffffffu, pz, o);
        ke += __shfl_down_sync(0xffffffffu, ke, o);
        vmax = fmax(vmax, __shfl_down_sync(0xffffffffu, vmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, M);
        atomicAdd(out + 1, px);
        atomicAdd(out + 2, py);
        atomicAdd(out + 3, pz);
        atomicAdd(out + 4, ke);
        // speeds are non-negative: their IEEE bit patterns order like unsigned integers
        atomicMax((unsigned long long*)(out + 5), (unsigned long long)__double_as_longlong(vmax));
    }
}

template <class T>
__global__ void k_iota_pid(uint32_t* pid, const uint8_t* mat, int64_t first, int64_t n)
{
    using L = typename LayoutOf<T>::type;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        pid[first + i] = (uint32_t)i | ((uint32_t)(mat ? mat[i] : 0) << L::index_bits);
}

template <class T>
__global__ void k_iota(uint32_t* v, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

} // namespace zr
