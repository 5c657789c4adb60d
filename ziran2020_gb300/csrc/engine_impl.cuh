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
#include "tma.cuh"

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
// P_MDT: the implicit damage solve's D~ history; P_DRV: the damage drive of the particle's current F (implicit
// scenes), kept by G2P and refilled after state writes
enum { P_X = 0, P_V = 3, P_C = 6, P_F = 15, P_M = 24, P_V0 = 25, P_D = 26, P_SC = 27, P_MDT = 28, P_DRV = 29, P_NF = 30 };

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
    int wide; // keys are stored as 64-bit words; 0: as 32-bit words (total() <= 32), a third less sort traffic
    __host__ __device__ int total() const { return sb + cp + ib; }
    __host__ __device__ uint64_t at(const uint64_t* k, uint32_t i) const { return wide ? k[i] : (uint64_t)reinterpret_cast<const uint32_t*>(k)[i]; }
    __host__ __device__ void put(uint64_t* k, uint32_t i, uint64_t v) const
    {
        if (wide)
            k[i] = v;
        else
            reinterpret_cast<uint32_t*>(k)[i] = (uint32_t)v;
    }
    __host__ __device__ uint32_t scene(uint64_t k) const { return (uint32_t)(k >> (cp + ib)); }
    __host__ __device__ uint64_t page(uint64_t k) const { return (k >> (ib + block_bits)) & ((1ULL << (cp - block_bits)) - 1); }
    __host__ __device__ uint64_t group(uint64_t k) const { return k >> (ib + block_bits); }
    __host__ __device__ uint32_t orig(uint64_t k) const { return (uint32_t)(k & ((1ULL << ib) - 1)); }
};

// per-scene state of the implicit damage solve's conjugate gradients (ConjugateGradient.h), kept on the device
struct CgScalars {
    double zr; // r . z
    double zr_new;
    double pAp; // p . A p
    double tol; // min(|r0|_z, 1e-6)
    int32_t iter, done;
    int32_t pad0, pad1;
};

template <class T>
struct StepArgs {
    const uint64_t* keys_sorted;
    const uint32_t* vals_sorted;
    uint64_t* keys_next;
    Pool<T> pin, pout;
    const uint32_t* g_start;
    int32_t* g_nbr;
    T* pay; // P2G payload, NPAY fields of pstride elements (also the implicit damage solve's particle scratch)
    int64_t pstride;
    T* cg; // implicit damage solve: CG_NF node vectors of b_cap * nodes
    CgScalars* cgs; // per scene
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
    int n_scenes;
    uint32_t opts; // OPT_* bits
    KeyLayout kl;
};
// OPT_PREFETCH: P2G prefetches the state of the groups ahead into L2
enum : uint32_t { OPT_PREFETCH = 1u };

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

// an internal consistency check failed: record the first check's code, count, abort the substep
__device__ inline void check_failed(DevStatus* st, uint32_t code)
{
    atomicCAS(&st->check_code, 0u, code);
    atomicAdd(&st->check_count, 1u);
    raise_flag(st, FLAG_CHECK);
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
        kl.put(keys, i, ((uint64_t)lo << (kl.cp + kl.ib)) | ((L::offset(b[0], b[1], b[2]) >> L::data_bits) << kl.ib));
    }
}

// The hot-path keys hold (scene, page, cell) only, so the radix sort needs 4 passes instead of 7; a
// stable sort of storage-ordered input leaves the particles of one cell in their previous order, which is
// deterministic and changes nothing in the substep but the order of floating-point sums. For the binning
// products (zr_scene_binning) this pass restores the reference's order inside each cell (ascending original
// index, the low bits of the reference key, MpmSimulationBase.cpp:1547-1552) with an insertion sort per run
// of equal keys; runs are short (~8) and nearly sorted.
template <class T>
__global__ void k_cellfix(const uint64_t* ks, uint32_t* vals, const uint32_t* pid, uint32_t n, KeyLayout kl)
{
    using L = typename LayoutOf<T>::type;
    const uint32_t mask = (1u << L::index_bits) - 1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = kl.at(ks, i);
        if (i > 0 && kl.at(ks, i - 1) == k) continue; // not the first of its run
        uint32_t e = i + 1;
        while (e < n && kl.at(ks, e) == k) e++;
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
    __device__ bool operator()(uint32_t i) const { return i == 0 || kl.group(kl.at(k, i)) != kl.group(kl.at(k, i - 1)); }
};

// ---------------------------------------------------------------------------------------------------
// Incremental sort (32-bit keys), hand-written. The storage order is the previous substep's sorted order, so the
// particles whose cell did not change ("stayers") are already sorted; only the particles that changed cell
// ("movers", ~2% per substep at the slab's speeds) need placing.
//
// Storage is cut into tiles of SORT_TILE indices. B[j] = the smallest stayer key in tiles >= j (non-decreasing;
// "no key" past the last stayer). Mover key k belongs to bucket b(k) = the largest j with B[j] <= k (0 when there is
// none): every element of bucket j (its movers) and tile j (its stayers) lies in [B[j], B[j+1]] and comes after
// every element of lower tiles and buckets, so tile j's merged output starts at
// (stayers in tiles < j) + (movers in buckets < j). Inside it, in the order (key, stayers first, storage index), a
// stayer goes to its rank among the tile's stayers plus the bucket's movers with a smaller key, a mover to its rank
// in the bucket plus the tile's stayers with a key not above its own. The order is fully determined by the keys
// and storage indices (no dependence on the order in which movers were found).
//
//   k_sort_tiles      per tile: stayer count, first and last stayer key; movers appended to a list (one atomic per
//                     tile)
//   k_sort_bucket     per mover: bucket (binary search over B, read from the tiles' first stayer keys), a ticket
//                     within it, the bucket's largest key, and (key, storage index) into the bucket's fixed slots
//   k_sort_merge      per tile: where its output starts and the key just before it (sums and maxima over the lower
//                     tiles and buckets, by the CTA itself), then the tile's stayers and its bucket's movers (sorted
//                     in shared memory) to their places; the group heads in the tile's output counted
//   k_heads_activate  per tile: the group heads of its output written to g_start after the lower tiles' heads, and
//                     their blocks and +1 neighbours activated in the grid hash
//
// More movers than the list holds, or a bucket larger than SORT_MAXM, raises FLAG_SORT: the host repeats the
// substep with a full radix sort (and grows the list).
// ---------------------------------------------------------------------------------------------------
constexpr int SORT_NT = 256, SORT_PER = 8, SORT_TILE = SORT_NT * SORT_PER, SORT_MAXM = 1024;
constexpr uint32_t SORT_NOKEY = 0xffffffffu; // keys of the incremental sort hold at most 31 bits

struct SortBufs {
    int64_t* cnt; // [0] movers found (zeroed per substep)
    uint32_t* b_cnt; // [tiles] movers per bucket (zeroed per substep)
    uint32_t* b_max; // [tiles] largest mover key per bucket (zeroed per substep)
    uint32_t* stay_bits; // [ceil(n / 32)] bit i % 32 of word i / 32: storage index i keeps its key
    uint32_t* t_stay; // [tiles] stayers per tile
    uint32_t* t_first; // [tiles] first stayer key per tile (SORT_NOKEY: none)
    uint32_t* t_last; // [tiles] last stayer key per tile (SORT_NOKEY: none)
    uint32_t* t_base; // [tiles] sorted position of the tile's first output (the merge writes it)
    uint32_t* t_heads; // [tiles] group heads in the tile's output (the merge counts them)
    uint32_t* m_idx; // [mcap] movers' storage indices (list order)
    uint32_t* b_key; // [tiles * SORT_MAXM] movers' keys: bucket j's at j * SORT_MAXM + ticket
    uint32_t* b_idx; // [tiles * SORT_MAXM] movers' storage indices, likewise
    int64_t mcap;
    int64_t n;
    int tiles;
};

static __global__ void __launch_bounds__(SORT_NT) k_sort_tiles(const uint32_t* knew, const uint32_t* kold, SortBufs sb, DevStatus* st)
{
    __shared__ uint32_t s_cnt[SORT_NT / 32], s_first[SORT_NT / 32], s_last[SORT_NT / 32], s_moff[SORT_NT / 32][SORT_PER];
    __shared__ uint64_t s_base;
    const int j = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)j * SORT_TILE;
    uint32_t nst = 0, first = SORT_NOKEY, last = SORT_NOKEY;
    unsigned moves = 0; // bit r: this thread's item of round r moved
    // items in storage order; a warp takes 256 consecutive ones, 32 at a time; every load issued first
    uint32_t kn[SORT_PER], ko[SORT_PER];
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const int64_t i = t0 + (int64_t)w * (32 * SORT_PER) + r * 32 + lane;
        kn[r] = i < sb.n ? knew[i] : 0u;
        ko[r] = i < sb.n ? kold[i] : 1u;
    }
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const int64_t i = t0 + (int64_t)w * (32 * SORT_PER) + r * 32 + lane;
        const bool valid = i < sb.n, stay = valid && kn[r] == ko[r], move = valid && !stay;
        const unsigned bs = __ballot_sync(0xffffffffu, stay), bm = __ballot_sync(0xffffffffu, move);
        if (lane == 0 && valid) sb.stay_bits[i >> 5] = bs; // the merge reads these: it overwrites the old keys
        if (bs) {
            if (first == SORT_NOKEY) first = __shfl_sync(0xffffffffu, kn[r], __ffs(bs) - 1);
            last = __shfl_sync(0xffffffffu, kn[r], 31 - __clz(bs));
        }
        nst += __popc(bs);
        if (move) moves |= 1u << r;
        if (lane == 0) s_moff[w][r] = __popc(bm);
    }
    if (lane == 0) {
        s_cnt[w] = nst;
        s_first[w] = first;
        s_last[w] = last;
    }
    __syncthreads();
    if (w == 0) {
        // the tile's movers in storage order (warp-major, then round): 64 counts, two per lane, one warp scan
        static_assert(SORT_PER * (SORT_NT / 32) == 64, "two counts per lane");
        uint32_t* mo = &s_moff[0][0];
        const uint32_t a0 = mo[2 * lane], a1 = mo[2 * lane + 1];
        uint32_t x = a0 + a1;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        mo[2 * lane] = x - a0 - a1;
        mo[2 * lane + 1] = x - a1;
        const uint32_t m = __shfl_sync(0xffffffffu, x, 31);
        if (lane == 0) {
            uint32_t c = 0, f = SORT_NOKEY, l = SORT_NOKEY;
            for (int q = 0; q < SORT_NT / 32; q++) {
                c += s_cnt[q];
                if (f == SORT_NOKEY) f = s_first[q];
                if (s_last[q] != SORT_NOKEY) l = s_last[q];
            }
            sb.t_stay[j] = c;
            sb.t_first[j] = f;
            sb.t_last[j] = l;
            s_base = m ? (uint64_t)atomicAdd((unsigned long long*)&sb.cnt[0], (unsigned long long)m) : 0ull; // one atomic per tile
        }
    }
    __syncthreads();
    const uint64_t base = s_base;
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const unsigned bm = __ballot_sync(0xffffffffu, (moves >> r) & 1u);
        if ((moves >> r) & 1u) {
            const uint64_t pos = base + s_moff[w][r] + __popc(bm & ((1u << lane) - 1u));
            if (pos < (uint64_t)sb.mcap) sb.m_idx[pos] = (uint32_t)(t0 + (int64_t)w * (32 * SORT_PER) + r * 32 + lane);
        }
    }
    (void)st;
}

static __global__ void __launch_bounds__(SORT_NT) k_sort_bucket(const uint32_t* knew, SortBufs sb, DevStatus* st)
{
    const int64_t Mall = sb.cnt[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicMax(&st->max_movers, (uint32_t)(Mall < 0xffffffffLL ? Mall : 0xffffffffLL));
        if (Mall > sb.mcap) raise_flag(st, FLAG_SORT);
    }
    const int64_t M = min(Mall, sb.mcap);
    const int T = sb.tiles;
    // B[q] = the first stayer key at or after tile q: a tile without a stayer takes the next tile's (emptying a tile
    // takes 2048 listed movers, so these walks are short); non-decreasing, as the stayers keep their order
    auto B = [&](int q) {
        uint32_t v = sb.t_first[q];
        while (v == SORT_NOKEY && ++q < T) v = sb.t_first[q];
        return v;
    };
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t i = sb.m_idx[m];
        const uint32_t k = i < (uint64_t)sb.n ? knew[i] : SORT_NOKEY;
        int lo = 0, hi = T; // first j with B[j] > k
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (B(mid) <= k) lo = mid + 1;
            else hi = mid;
        }
        const uint32_t b = lo > 0 ? (uint32_t)(lo - 1) : 0u;
        const uint32_t t = atomicAdd(&sb.b_cnt[b], 1u);
        atomicMax(&sb.b_max[b], k);
        if (t < (uint32_t)SORT_MAXM) { // a fuller bucket makes the merge raise FLAG_SORT
            sb.b_key[(size_t)b * SORT_MAXM + t] = k;
            sb.b_idx[(size_t)b * SORT_MAXM + t] = i;
        }
    }
}

static __global__ void __launch_bounds__(SORT_NT) k_sort_merge(const uint32_t* knew, SortBufs sb, uint32_t* out_keys, uint32_t* out_vals, KeyLayout kl,
    DevStatus* st)
{
    __shared__ uint32_t s_key[SORT_TILE], s_idx[SORT_TILE]; // the tile's stayers in storage (= key) order
    __shared__ uint32_t m_key[SORT_MAXM], m_idx[SORT_MAXM], m_key2[SORT_MAXM], m_idx2[SORT_MAXM];
    __shared__ uint32_t o_key[SORT_TILE + SORT_MAXM]; // the tile's output in order
    __shared__ uint32_t s_heads;
    __shared__ uint32_t s_wcnt[SORT_PER][SORT_NT / 32];
    __shared__ uint32_t s_red[2][SORT_NT / 32];
    __shared__ int s_ns;
    const int j = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int64_t M = sb.cnt[0];
    if (M > sb.mcap) return; // FLAG_SORT raised: the substep is repeated with a full sort
    const uint32_t bc = sb.b_cnt[j];
    if (bc > (uint32_t)SORT_MAXM) {
        if (tid == 0) raise_flag(st, FLAG_SORT);
        return;
    }
    const int nm = (int)bc;
    // the lower tiles and buckets: their element count (where this tile's output starts) and their largest key (the
    // key just before the output: stayer and bucket key ranges ascend with the tile). pk holds key + 1, 0 for none.
    uint32_t below = 0, pk = 0;
#pragma unroll 4
    for (int q = tid; q < j; q += SORT_NT) {
        const uint32_t c = sb.b_cnt[q], l = sb.t_last[q], mk = sb.b_max[q];
        below += sb.t_stay[q] + c;
        if (l != SORT_NOKEY) pk = max(pk, l + 1);
        if (c) pk = max(pk, mk + 1);
    }
    for (int o = 16; o > 0; o >>= 1) {
        below += __shfl_down_sync(0xffffffffu, below, o);
        pk = max(pk, __shfl_down_sync(0xffffffffu, pk, o));
    }
    if (lane == 0) {
        s_red[0][w] = below;
        s_red[1][w] = pk;
    }
    // the tile's stayers, compacted in storage order: item (r, w, lane) = t0 + r*256 + w*32 + lane
    const int64_t t0 = (int64_t)j * SORT_TILE;
    unsigned mine = 0; // bit r: this thread's item of round r stays
    uint32_t keys[SORT_PER];
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const int64_t i = t0 + r * SORT_NT + tid;
        keys[r] = 0;
        bool stay = false;
        if (i < sb.n) {
            keys[r] = knew[i];
            stay = (sb.stay_bits[i >> 5] >> lane) & 1u; // i % 32 == lane: rounds and warps start at multiples of 32
        }
        const unsigned b = __ballot_sync(0xffffffffu, stay);
        if (stay) mine |= 1u << r;
        if (lane == 0) s_wcnt[r][w] = __popc(b);
    }
    for (int q = tid; q < nm; q += SORT_NT) {
        m_key[q] = sb.b_key[(size_t)j * SORT_MAXM + q];
        m_idx[q] = sb.b_idx[(size_t)j * SORT_MAXM + q];
    }
    __syncthreads();
    if (w == 0) { // exclusive offsets of the 64 (round, warp) groups in storage order: two per lane, one warp scan
        static_assert(SORT_PER * (SORT_NT / 32) == 64, "two groups per lane");
        uint32_t* c = &s_wcnt[0][0];
        const uint32_t a0 = c[2 * lane], a1 = c[2 * lane + 1];
        uint32_t x = a0 + a1;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        const uint32_t ex = x - a0 - a1;
        c[2 * lane] = ex;
        c[2 * lane + 1] = ex + a0;
        if (lane == 31) s_ns = (int)x;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const unsigned b = __ballot_sync(0xffffffffu, (mine >> r) & 1u);
        if ((mine >> r) & 1u) {
            const uint32_t pos = s_wcnt[r][w] + __popc(b & ((1u << lane) - 1u));
            s_key[pos] = keys[r];
            s_idx[pos] = (uint32_t)(t0 + r * SORT_NT + tid);
        }
    }
    // the bucket's movers ranked by (key, storage index): distinct pairs, so the ranks are a permutation
    for (int q = tid; q < nm; q += SORT_NT) {
        const uint32_t k = m_key[q], i = m_idx[q];
        int rank = 0;
        for (int o = 0; o < nm; o++) rank += (m_key[o] < k || (m_key[o] == k && m_idx[o] < i)) ? 1 : 0;
        m_key2[rank] = k;
        m_idx2[rank] = i;
    }
    __syncthreads();
    const int ns = s_ns;
    uint32_t below_all = 0, pk_all = 0;
#pragma unroll
    for (int q = 0; q < SORT_NT / 32; q++) {
        below_all += s_red[0][q];
        pk_all = max(pk_all, s_red[1][q]);
    }
    const int64_t base = below_all; // elements of lower tiles and buckets
    if (tid == 0) sb.t_base[j] = below_all;
    for (int t = tid; t < ns; t += SORT_NT) { // stayer: its rank + the bucket's movers with a smaller key
        const uint32_t k = s_key[t];
        int lo = 0, hi = nm;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (m_key2[mid] < k) lo = mid + 1;
            else hi = mid;
        }
        const int64_t pos = base + t + lo;
        if (pos < 0 || pos >= sb.n) {
            check_failed(st, 8);
            continue;
        }
        out_keys[pos] = k;
        out_vals[pos] = s_idx[t];
        o_key[t + lo] = k;
    }
    for (int r = tid; r < nm; r += SORT_NT) { // mover: its rank + the tile's stayers with a key not above its own
        const uint32_t k = m_key2[r];
        int lo = 0, hi = ns;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (s_key[mid] <= k) lo = mid + 1;
            else hi = mid;
        }
        const int64_t pos = base + r + lo;
        if (pos < 0 || pos >= sb.n) {
            check_failed(st, 8);
            continue;
        }
        out_keys[pos] = k;
        out_vals[pos] = m_idx2[r];
        o_key[r + lo] = k;
    }
    // group heads in the tile's output (compared with the key before it): counted here, placed by k_heads_activate
    if (tid == 0) s_heads = 0;
    __syncthreads();
    const uint32_t pred = pk_all ? pk_all - 1 : SORT_NOKEY;
    uint32_t h = 0;
    for (int p = tid; p < ns + nm; p += SORT_NT) {
        const uint32_t k = o_key[p];
        const bool first = p == 0 ? pred == SORT_NOKEY : false;
        const uint32_t kp = p == 0 ? pred : o_key[p - 1];
        h += (first || kl.group(k) != kl.group(kp)) ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
    if (lane == 0 && h) atomicAdd(&s_heads, h);
    __syncthreads();
    if (tid == 0) sb.t_heads[j] = s_heads;
}

// ---------------------------------------------------------------------------------------------------
// group heads: the first sorted index of every (scene, SPGrid page), compacted in order into g_start, their number
// into n_groups. One pass over the sorted keys with a decoupled look-back: tiles are taken in order from a counter
// (a tile's predecessors have started, so they publish), each publishes its head count, then the running total
// once its predecessors' is known. Waits are bounded; a wait that runs out raises FLAG_TIMEOUT.
// ---------------------------------------------------------------------------------------------------
constexpr uint64_t LB_AGG = 1ull << 62, LB_PREFIX = 2ull << 62, LB_VALUE = (1ull << 62) - 1;

static __global__ void __launch_bounds__(SORT_NT) k_group_heads(const uint64_t* keys, int64_t n, KeyLayout kl, uint64_t* status, uint32_t* counter,
    uint32_t* g_start, uint32_t cap, DevStatus* st)
{
    __shared__ uint32_t s_w[SORT_PER][SORT_NT / 32];
    __shared__ int s_tile;
    __shared__ uint64_t s_prefix;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int j = s_tile;
    const int64_t t0 = (int64_t)j * SORT_TILE;
    unsigned mine = 0;
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const int64_t i = t0 + r * SORT_NT + tid;
        const bool head = i < n && (i == 0 || kl.group(kl.at(keys, (uint32_t)i)) != kl.group(kl.at(keys, (uint32_t)(i - 1))));
        const unsigned b = __ballot_sync(0xffffffffu, head);
        if (head) mine |= 1u << r;
        if (lane == 0) s_w[r][w] = __popc(b);
    }
    __syncthreads();
    if (tid == 0) {
        uint32_t run = 0;
        for (int r = 0; r < SORT_PER; r++)
            for (int q = 0; q < SORT_NT / 32; q++) {
                const uint32_t c = s_w[r][q];
                s_w[r][q] = run;
                run += c;
            }
        s_prefix = run; // the tile's head count until the look-back below replaces it by the prefix
        volatile uint64_t* vs = status;
        vs[j] = (j == 0 ? LB_PREFIX : LB_AGG) | run;
    }
    __syncthreads();
    if (w == 0) { // look-back by the first warp: 32 predecessors per step, back to the nearest published prefix
        const uint32_t run = s_prefix;
        uint64_t prefix = 0;
        if (j > 0) {
            volatile uint64_t* vs = status;
            int q = j - 1;
            uint32_t spins = 0;
            bool timed_out = false;
            while (q >= 0 && !timed_out) {
                const int idx = q - lane;
                uint64_t v = LB_PREFIX + 0; // before tile 0: a prefix of zero
                if (idx >= 0) v = vs[idx];
                while (__any_sync(0xffffffffu, (v & (LB_AGG | LB_PREFIX)) == 0)) {
                    if (++spins > (1u << 22)) { // a predecessor never published: give up (the substep is aborted)
                        timed_out = true;
                        break;
                    }
                    __nanosleep(64);
                    if ((v & (LB_AGG | LB_PREFIX)) == 0) v = vs[idx];
                }
                if (timed_out) break;
                const unsigned pm = __ballot_sync(0xffffffffu, (v & LB_PREFIX) != 0);
                const int stop = pm ? __ffs(pm) - 1 : 31; // lanes 0..stop count (lane 0 is the nearest predecessor)
                uint64_t c = lane <= stop ? (v & LB_VALUE) : 0ull;
                for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
                prefix += __shfl_sync(0xffffffffu, c, 0);
                if (pm) break;
                q -= 32;
            }
            if (timed_out && lane == 0) raise_flag(st, FLAG_TIMEOUT);
            if (lane == 0) {
                __threadfence();
                vs[j] = LB_PREFIX | (prefix + run);
            }
        }
        if (lane == 0) {
            s_prefix = prefix;
            if ((int64_t)(j + 1) * SORT_TILE >= n) st->n_groups = (uint32_t)(prefix + run); // the last tile
        }
    }
    __syncthreads();
    const uint64_t prefix = s_prefix;
#pragma unroll
    for (int r = 0; r < SORT_PER; r++) {
        const unsigned b = __ballot_sync(0xffffffffu, (mine >> r) & 1u);
        if ((mine >> r) & 1u) {
            const uint64_t pos = prefix + s_w[r][w] + __popc(b & ((1u << lane) - 1u));
            if (pos < cap) g_start[pos] = (uint32_t)(t0 + r * SORT_NT + tid);
            else check_failed(st, 9);
        }
    }
}

// Block dl (x*4 + y*2 + z, at +1 block) of the group whose first sorted key is key0, into the block hash; a block
// seen for the first time takes the next grid slot (one slot counter atomic per group of converged lanes).
template <class T>
__device__ __forceinline__ void activate_block(const StepArgs<T>& a, uint64_t key0, uint32_t dl, int32_t* hpos)
{
    using L = typename LayoutOf<T>::type;
    const uint64_t scene = a.kl.scene(key0);
    uint32_t bi, bj, bk;
    L::block_of_page(a.kl.page(key0), bi, bj, bk);
    const uint64_t hk = (scene << 40) | L::page_of_block(bi + (dl >> 2), bj + ((dl >> 1) & 1), bk + (dl & 1));
    uint32_t h = (uint32_t)hash64(hk) & a.h_mask;
    bool done = false, fresh = false;
    for (int p = 0; p < HASH_PROBES && !done; p++) {
        const unsigned long long prev = atomicCAS((unsigned long long*)&a.h_keys[h], (unsigned long long)HASH_EMPTY, (unsigned long long)hk);
        if (prev == HASH_EMPTY)
            done = fresh = true;
        else if (prev == hk)
            done = true;
        else
            h = (h + 1) & a.h_mask;
    }
    if (!done) raise_flag(a.st, FLAG_CAPACITY);
    // The group's neighbour entry gets the block's hash position, whether this thread inserted the block or found
    // it: the slot is written by the inserting thread below, so it is read (nbr_slot) only by a later kernel.
    *hpos = done ? (int32_t)h : -1;
    const unsigned am = __activemask();
    const unsigned nw = __ballot_sync(am, fresh);
    if (nw) {
        const int lane = threadIdx.x & 31, leader = __ffs(nw) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&a.st->n_blocks, (uint32_t)__popc(nw));
        base = __shfl_sync(am, base, leader);
        if (fresh) {
            const uint32_t slot = base + (uint32_t)__popc(nw & ((1u << lane) - 1u));
            if (slot >= a.b_cap) {
                raise_flag(a.st, FLAG_CAPACITY);
                a.h_vals[h] = -1;
            }
            else {
                a.h_vals[h] = (int32_t)slot;
                a.b_key[slot] = hk;
            }
        }
    }
}

// the blocks of every group (after a full sort and k_group_heads), 8 per group
template <class T>
__global__ void k_activate(StepArgs<T> a)
{
    if (blockIdx.x == 0) // the per-scene grid mass k_grid accumulates
        for (int s = threadIdx.x; s < a.n_scenes; s += blockDim.x) a.grid_mass[s] = 0;
    if (aborted(a.st)) return;
    const uint32_t G = a.st->n_groups;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->max_groups_seen = max(a.st->max_groups_seen, G);
    if (G > a.b_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) raise_flag(a.st, FLAG_CAPACITY);
        return;
    }
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < G * 8; t += gridDim.x * blockDim.x)
        activate_block(a, a.kl.at(a.keys_sorted, a.g_start[t >> 3]), t & 7, a.g_nbr + t);
}

// After the incremental sort's merge, per tile: the group heads of the tile's output (sorted positions
// [t_base of the tile, of the next tile), each compared with the sorted key before it) written in order into
// g_start after the heads of the lower tiles (summed by the CTA itself from the merge's counts), then the 8 blocks
// of each of these groups activated. The last tile stores the number of groups.
template <class T>
__global__ void __launch_bounds__(SORT_NT) k_heads_activate(StepArgs<T> a, SortBufs sb, uint32_t* g_start, uint32_t cap)
{
    constexpr int RMAX = (SORT_TILE + SORT_MAXM) / SORT_NT;
    __shared__ uint32_t s_c[RMAX][SORT_NT / 32], s_part[SORT_NT / 32];
    __shared__ uint32_t s_pos[RMAX * SORT_NT]; // sorted positions of the tile's heads, in order
    __shared__ uint32_t s_g0, s_nh;
    if (blockIdx.x == 0) // the per-scene grid mass k_grid accumulates
        for (int s = threadIdx.x; s < a.n_scenes; s += blockDim.x) a.grid_mass[s] = 0;
    if (aborted_cta(a.st)) return; // FLAG_SORT from the merge, or an earlier failure: the substep is repeated
    const int j = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t* keys = reinterpret_cast<const uint32_t*>(a.keys_sorted); // the incremental sort's keys are 32-bit
    const int64_t b0 = sb.t_base[j];
    const int64_t b1 = j + 1 < sb.tiles ? (int64_t)sb.t_base[j + 1] : sb.n;
    if (b1 < b0 || b1 > sb.n || b1 - b0 > (int64_t)RMAX * SORT_NT) { // the merge's outputs cannot give this range
        if (tid == 0) check_failed(a.st, 9);
        return;
    }
    // heads of the lower tiles
    uint32_t pre = 0;
    for (int q = tid; q < j; q += SORT_NT) pre += sb.t_heads[q];
    for (int o = 16; o > 0; o >>= 1) pre += __shfl_down_sync(0xffffffffu, pre, o);
    if (lane == 0) s_part[w] = pre;
    // the range's keys and head flags, items (r, w, lane) = b0 + r*256 + w*32 + lane, every load issued first
    const int R = (int)((b1 - b0 + SORT_NT - 1) / SORT_NT);
    uint32_t k[RMAX], kl0[RMAX]; // the item's key; for lane 0 also the key before it (another warp's item)
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        const int64_t p = b0 + r * SORT_NT + tid;
        const bool in = r < R && p < b1;
        k[r] = in ? keys[p] : 0u;
        kl0[r] = (in && lane == 0 && p > 0) ? keys[p - 1] : 0u;
    }
    unsigned mine = 0;
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r >= R) break;
        const int64_t p = b0 + r * SORT_NT + tid;
        uint32_t prev = __shfl_up_sync(0xffffffffu, k[r], 1);
        if (lane == 0) prev = kl0[r];
        const bool head = p < b1 && (p == 0 || a.kl.group(k[r]) != a.kl.group(prev));
        const unsigned b = __ballot_sync(0xffffffffu, head);
        if (head) mine |= 1u << r;
        if (lane == 0) s_c[r][w] = __popc(b);
    }
    __syncthreads();
    if (w == 0) { // exclusive offsets of the (row, warp) counts in order, after the lower tiles' heads
        uint32_t base = 0;
        for (int q = 0; q < SORT_NT / 32; q++) base += s_part[q];
        uint32_t carry = base;
        for (int r = 0; r < R; r++) {
            uint32_t c = lane < SORT_NT / 32 ? s_c[r][lane] : 0u, x = c;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane < SORT_NT / 32) s_c[r][lane] = carry + x - c;
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) {
            s_g0 = base;
            s_nh = carry - base;
            if (j + 1 == sb.tiles) {
                a.st->n_groups = carry;
                a.st->max_groups_seen = max(a.st->max_groups_seen, carry);
            }
        }
    }
    __syncthreads();
    const uint32_t g0 = s_g0;
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r >= R) break;
        const unsigned b = __ballot_sync(0xffffffffu, (mine >> r) & 1u);
        if ((mine >> r) & 1u) {
            const uint32_t pos = s_c[r][w] + __popc(b & ((1u << lane) - 1u)), p = (uint32_t)(b0 + r * SORT_NT + tid);
            s_pos[pos - g0] = p; // pos - g0 < the tile's item count <= RMAX * SORT_NT
            if (pos < cap) g_start[pos] = p;
            else check_failed(a.st, 9);
        }
    }
    __syncthreads();
    const uint32_t nh = s_nh;
    for (uint32_t t = tid; t < nh * 8; t += SORT_NT) {
        if (g0 + (t >> 3) >= a.b_cap) { // more groups than grid blocks: the host grows the grid and repeats the substep
            raise_flag(a.st, FLAG_CAPACITY);
            continue;
        }
        activate_block(a, (uint64_t)keys[s_pos[t >> 3]], t & 7, a.g_nbr + (size_t)g0 * 8 + t);
    }
}

// ---------------------------------------------------------------------------------------------------
// neighbour slots: the grid slots of every group's block and its 7 neighbours at +1 block (read by P2G and
// G2P). Activation leaves the hash position of each of these blocks in g_nbr; the slot behind it is final once
// activation has ended. The fused P2G translates its groups' entries itself while it sets them up (and writes
// the slots back for G2P); the other P2G forms read slots, so k_nbr translates every entry before them.
// ---------------------------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ int32_t nbr_slot(const StepArgs<T>& a, int32_t hpos)
{
    return (uint32_t)hpos <= a.h_mask ? a.h_vals[hpos] : -1; // -1: the probe failed and raised FLAG_CAPACITY
}

template <class T>
__global__ void k_nbr(StepArgs<T> a)
{
    if (aborted(a.st)) return;
    const uint32_t G = a.st->n_groups;
    if (G > a.b_cap) return; // activation already raised FLAG_CAPACITY
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < G * 8; t += gridDim.x * blockDim.x) {
        const int32_t slot = nbr_slot(a, a.g_nbr[t]);
        if (slot < 0) raise_flag(a.st, FLAG_CAPACITY);
        a.g_nbr[t] = slot;
    }
}

// ---------------------------------------------------------------------------------------------------
// P2G, in two kernels.
//
// k_stress (thread per sorted particle): stress V0 tau(F, g(d)) (FBasedMpmForceHelper.cpp:43-63) and a
// 27-value payload per particle, written in sorted order: fractional index-space position
// f = x/dx - base, m, A = m v - dx (m C) f, Bc = dx m C, K = -dt V0 tau / dx, d, and the particle's
// cell inside its block. With xm = (delta - f) dx for stencil offset delta,
//   m v + m C xm = A + Bc delta   and   dt f_i = K . (dw_i w_j w_k, w_i dw_j w_k, w_i w_j dw_k),
// so a node receives m w, w (A + Bc delta) + K grad-hat w, d w and w. The force enters the momentum
// directly (m v + dt f), which the grid update turns into v + f dt/m + g dt as the reference's
// gridVelocityExplicitUpdate does (MpmSimulationBase.cpp:1197-1226).
//
// k_scatter (CTA per group, persistent): a producer warp streams each chunk of a group's payload from
// HBM into shared memory with bulk asynchronous copies (double-buffered, mbarrier-synchronised); the
// consumer threads, one per (cell, stencil x-offset), accumulate the 9 nodes x 6 fields of their cell's
// particles in registers (all particles of a cell share the same 27 nodes), add them into a shared
// 6x6x6 node tile, and after the group's last chunk the tile goes to the 8 neighbouring grid blocks as
// vector atomics (MpmSimulationBase.cpp:669-855, AnisoFractureSimulation.h:161-176).
//
// Payload storage: field k of sorted particle q at pay[k * pstride + q + q/8]. The gap after every 8
// particles carries over into shared memory with the copy and staggers the shared-memory banks of the
// consumer lanes (one lane per cell, ~8 particles per cell).
// The Kirchhoff stress of every model here is symmetric (the energies are frame-indifferent), so K keeps its
// upper triangle, each off-diagonal entry the mean of the two that were computed: six fields instead of nine,
// three shared-memory loads fewer per particle and stencil x-offset in the accumulation.
// ---------------------------------------------------------------------------------------------------
constexpr int NPAY = 24;
enum { Y_F = 0, Y_M = 3, Y_A = 4, Y_B = 7, Y_K = 16, Y_D = 22, Y_CELL = 23 };
enum { K_00 = 0, K_01 = 1, K_02 = 2, K_11 = 3, K_12 = 4, K_22 = 5 }; // offsets of the K entries from Y_K

__host__ __device__ __forceinline__ uint64_t pay_pos(uint64_t q) { return q + (q >> 3); }

// Stress and payload of one particle (storage slot j of pool P): fields Y_F..Y_D at y[f * S]; b gets the
// base node. V0 tau(F) of the particle's model (FBasedMpmForceHelper.cpp:43-63) with the degradation g(d).
template <class T, int MODELS>
__device__ __forceinline__ void particle_payload(const Pool<T>& P, uint32_t j, const SceneParams<T>& sp, T* y, int64_t S, int (&b)[3],
    uint32_t& fallbacks)
{
    using L = typename LayoutOf<T>::type;
    // The corotated stress's polar decomposition needs many registers: with it, v and C are loaded after the
    // stress (a second memory latency) instead of being held through it (spills)
    constexpr bool LATE_VC = (MODELS & 1) != 0;
    T x[3], v[3], Cm[9], F[9];
    auto load_vc = [&]() {
#pragma unroll
        for (int e = 0; e < 3; e++) v[e] = P.f[(P_V + e) * P.stride + j];
#pragma unroll
        for (int e = 0; e < 9; e++) Cm[e] = P.f[(P_C + e) * P.stride + j];
    };
#pragma unroll
    for (int e = 0; e < 3; e++) x[e] = P.f[(P_X + e) * P.stride + j];
#pragma unroll
    for (int e = 0; e < 9; e++) F[e] = P.f[(P_F + e) * P.stride + j];
    if constexpr (!LATE_VC) load_vc();
    const T mass = P.f[P_M * P.stride + j], V0 = P.f[P_V0 * P.stride + j];
    const bool damage = sp.damage != 0;
    const T dd = damage ? P.f[P_D * P.stride + j] : (T)0;
    const uint32_t mat = P.pid[j] >> L::index_bits;
    const Material<T>& mt = sp.materials[mat < (uint32_t)sp.n_materials ? mat : 0];
    T tau[9];
    const T g = (damage && mt.damage) ? degradation(dd, mt.residual) : (T)1;
    if (MODELS == 1 || (MODELS == 7 && mt.model == MODEL_COROTATED)) { // the reference degrades no corotated model
        if (tau_corotated(mt, F, tau)) fallbacks++;
    }
    else if (MODELS == 4 || (MODELS == 7 && mt.model == MODEL_QR_STABLE_NEOHOOKEAN))
        tau_qrnh(mt, F, g, tau);
    else
        tau_nhb(mt, F, g, tau);
    if constexpr (LATE_VC) load_vc();
    const T dx = sp.dx, inv_dx = sp.inv_dx, dt = sp.dt;
    T fr[3];
#pragma unroll
    for (int e = 0; e < 3; e++) {
        const T xs = mul_rn(x[e], inv_dx);
        b[e] = int_floor(sub_rn(xs, (T)0.5));
        fr[e] = xs - (T)b[e];
    }
    const T kf = -dt * V0 * inv_dx;
#pragma unroll
    for (int e = 0; e < 3; e++) y[(Y_F + e) * S] = fr[e];
    y[Y_M * S] = mass;
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const T m0 = mass * Cm[3 * r], m1 = mass * Cm[3 * r + 1], m2 = mass * Cm[3 * r + 2];
        y[(Y_A + r) * S] = mass * v[r] - dx * (m0 * fr[0] + m1 * fr[1] + m2 * fr[2]);
        y[(Y_B + 3 * r) * S] = dx * m0;
        y[(Y_B + 3 * r + 1) * S] = dx * m1;
        y[(Y_B + 3 * r + 2) * S] = dx * m2;
    }
    const T hk = (T)0.5 * kf;
    y[(Y_K + K_00) * S] = kf * tau[0];
    y[(Y_K + K_01) * S] = hk * (tau[1] + tau[3]);
    y[(Y_K + K_02) * S] = hk * (tau[2] + tau[6]);
    y[(Y_K + K_11) * S] = kf * tau[4];
    y[(Y_K + K_12) * S] = hk * (tau[5] + tau[7]);
    y[(Y_K + K_22) * S] = kf * tau[8];
    y[Y_D * S] = dd;
}

template <class T, int MODELS>
__global__ void __launch_bounds__(256) k_stress(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    if (aborted(a.st)) return;
    const KeyLayout kl = a.kl;
    const uint64_t cmask = (1ULL << kl.cp) - 1;
    const int64_t S = a.pstride;
    uint32_t flags = 0, fallbacks = 0;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < a.n_total; q += gridDim.x * blockDim.x) {
        const uint64_t key = a.kl.at(a.keys_sorted, q);
        T* y = a.pay + pay_pos(q);
        int b[3];
        particle_payload<T, MODELS>(a.pin, a.vals_sorted[q], a.scenes[kl.scene(key)], y, S, b, fallbacks);
        // the key was computed from this position by the previous G2P (or k_keys): they must agree
        const uint64_t want = (key >> kl.ib) & cmask;
        const bool ok = b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && (L::offset(b[0], b[1], b[2]) >> L::data_bits) == want;
        if (!ok) flags |= FLAG_CAPACITY;
        y[Y_CELL * S] = ok ? (T)(int)(want & (L::nodes - 1)) : (T)255;
        if ((q & 7) == 7) { // the gap slot after every 8th particle: writing it keeps every 32-byte sector whole
#pragma unroll
            for (int f = 0; f < NPAY; f++) y[f * S + 1] = (T)0;
        }
    }
    if (flags) raise_flag(a.st, flags);
    if (fallbacks) atomicAdd(&a.st->fallback, fallbacks);
}

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

// Paired arithmetic: Blackwell issues two FP32 FMAs as one instruction on float2 operands (__ffma2_rn rounds each
// lane as fmaf does). The accumulators of a (cell, x-offset) thread are kept as pairs so that every update of
// two fields is one instruction; FP64 keeps scalar FMAs.
template <class T>
struct PairOf;
template <>
struct PairOf<float> {
    using type = float2;
};
template <>
struct PairOf<double> {
    using type = double2;
};
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// 16 bytes of consecutive values (4 FP32 or 2 FP64), moved with one access
template <class T>
struct alignas(16) Vec16 {
    T v[16 / sizeof(T)];
};
// four values of one grid node read with one shared-memory access (velocity x, y, z and the phase field)
template <class T>
struct alignas(4 * sizeof(T)) Quad {
    T x, y, z, w;
};
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) { return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y)); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
template <class P, class T>
__device__ __forceinline__ P pmake(T x, T y)
{
    P r;
    r.x = x;
    r.y = y;
    return r;
}

// The 9 nodes (jj, kk) x NACC fields of a (cell, stencil x-offset ii) thread, as pairs (p_x, p_y), (p_z, m), (d w, w)
template <class T>
struct NodeAcc {
    using P = typename PairOf<T>::type;
    P a[9][3];
    __device__ __forceinline__ void zero()
    {
#pragma unroll
        for (int n = 0; n < 9; n++)
#pragma unroll
            for (int k = 0; k < 3; k++) a[n][k] = pmake<P>((T)0, (T)0);
    }
    // field f of node n: 0 mass, 1-3 momentum, 4 d w, 5 w (the accumulator order of the grid)
    __device__ __forceinline__ T field(int n, int f) const
    {
        return f == 0 ? a[n][1].y : f == 1 ? a[n][0].x : f == 2 ? a[n][0].y : f == 3 ? a[n][1].x : f == 4 ? a[n][2].x : a[n][2].y;
    }
};

// One particle's contribution to the 9 nodes (ii, jj, kk) of a (cell, stencil x-offset ii) thread; y points
// at the particle's payload, fields STRIDE apart. Weights from the fractional position (BSplines.h:73-100).
// Node (ii, jj, kk) receives, per momentum component r,
//   wz_k al_r(j) + k wz_k be_r(j) + dwz_k ga_r(j)   with
//   al = wx wy (A + j B1) + K0 dwx wy + K1 wx dwy,  be = wx wy B2,  ga = wx wy K2
// Everything that does not depend on (jj, kk) is folded first, per particle and offset ii:
//   U = wx (A + ii B0) + dwx K0,  V = wx B1,  Wk = wx K1,  X = wx B2,  Y = wx K2
// so that al = wy_j U + j wy_j V + dwy_j Wk, be = wy_j X, ga = wy_j Y. All of it runs on pairs (two FP32 lanes
// per instruction): (x, y) and (z, m), the mass lane carrying wx m through U and zeros elsewhere, and (d w, w).
template <class T, int STRIDE, bool DAMAGE>
__device__ __forceinline__ void accumulate_particle(NodeAcc<T>& acc, const T* y, int ii)
{
    using P = typename NodeAcc<T>::P;
    T wy[3], dwy[3], wz[3], dwz[3];
    T wx, dwx;
    {
        const T d0 = y[Y_F * STRIDE];
        const T z = (T)1.5 - d0, d1 = d0 - (T)1, zz = d0 - (T)0.5;
        wx = ii == 0 ? (T)0.5 * z * z : (ii == 1 ? (T)0.75 - d1 * d1 : (T)0.5 * zz * zz);
        dwx = ii == 0 ? -z : (ii == 1 ? (T)-2 * d1 : zz);
    }
#pragma unroll
    for (int e = 1; e < 3; e++) {
        const T d0 = y[(Y_F + e) * STRIDE];
        const T z = (T)1.5 - d0, d1 = d0 - (T)1, zz = d0 - (T)0.5;
        T* w = e == 1 ? wy : wz;
        T* dw = e == 1 ? dwy : dwz;
        w[0] = (T)0.5 * z * z;
        w[1] = (T)0.75 - d1 * d1;
        w[2] = (T)0.5 * zz * zz;
        dw[0] = -z;
        dw[1] = (T)-2 * d1;
        dw[2] = zz;
    }
    const T mass = y[Y_M * STRIDE];
    const T dd = DAMAGE ? y[Y_D * STRIDE] : (T)0;
    const T fi = (T)ii;
    const P WX = pmake<P>(wx, wx), DWX = pmake<P>(dwx, dwx), FI = pmake<P>(fi, fi);
    // pairs of payload fields: (x, y) and (z, mass lane)
    auto pr = [&](int f0, int f1) { return pmake<P>(y[f0 * STRIDE], y[f1 * STRIDE]); };
    auto pz = [&](int f0) { return pmake<P>(y[f0 * STRIDE], (T)0); };
    const P A01 = pr(Y_A, Y_A + 1), A2 = pmake<P>(y[(Y_A + 2) * STRIDE], mass);
    // K is symmetric: column c of it is (K0c, K1c, K2c) read from the upper triangle
    const P U01 = pfma(DWX, pr(Y_K + K_00, Y_K + K_01), pmul(WX, pfma(FI, pr(Y_B, Y_B + 3), A01)));
    const P U2 = pfma(DWX, pz(Y_K + K_02), pmul(WX, pfma(FI, pz(Y_B + 6), A2)));
    const P V01 = pmul(WX, pr(Y_B + 1, Y_B + 4)), V2 = pmul(WX, pz(Y_B + 7));
    const P K01 = pmul(WX, pr(Y_K + K_01, Y_K + K_11)), K2 = pmul(WX, pz(Y_K + K_12));
    const P X01 = pmul(WX, pr(Y_B + 2, Y_B + 5)), X2 = pmul(WX, pz(Y_B + 8));
    const P Y01 = pmul(WX, pr(Y_K + K_02, Y_K + K_12)), Y2 = pmul(WX, pz(Y_K + K_22));
    const P D = pmake<P>(wx * dd, wx);
#pragma unroll
    for (int jj = 0; jj < 3; jj++) {
        const P WY = pmake<P>(wy[jj], wy[jj]), DWY = pmake<P>(dwy[jj], dwy[jj]);
        P AL0 = pfma(DWY, K01, pmul(WY, U01)), AL1 = pfma(DWY, K2, pmul(WY, U2));
        if (jj) {
            const T jw = (T)jj * wy[jj];
            const P JW = pmake<P>(jw, jw);
            AL0 = pfma(JW, V01, AL0);
            AL1 = pfma(JW, V2, AL1);
        }
        const P BE0 = pmul(WY, X01), BE1 = pmul(WY, X2);
        const P GA0 = pmul(WY, Y01), GA1 = pmul(WY, Y2);
        const P DW = pmul(WY, D);
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            const T wk = wz[kk], dwk = dwz[kk];
            const P W = pmake<P>(wk, wk), DWK = pmake<P>(dwk, dwk);
            P* ac = acc.a[jj * 3 + kk];
            ac[0] = pfma(W, AL0, ac[0]);
            ac[1] = pfma(W, AL1, ac[1]);
            if (kk) {
                const T kw = (T)kk * wk;
                const P KW = pmake<P>(kw, kw);
                ac[0] = pfma(KW, BE0, ac[0]);
                ac[1] = pfma(KW, BE1, ac[1]);
            }
            ac[0] = pfma(DWK, GA0, ac[0]);
            ac[1] = pfma(DWK, GA1, ac[1]);
            if (DAMAGE) ac[2] = pfma(W, DW, ac[2]);
        }
    }
}

// registers -> shared node tile of the block plus its +2 halo (distinct nodes within a warp: no contention)
template <class T, class L>
__device__ __forceinline__ void add_to_tile(const NodeAcc<T>& acc, T* tile, int cx, int cy, int cz, int ii, int nf)
{
    constexpr int TY = L::sy + 2, TZ = L::sz + 2, TN = (L::sx + 2) * TY * TZ;
#pragma unroll
    for (int jj = 0; jj < 3; jj++)
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            T* t = tile + ((cx + ii) * TY + (cy + jj)) * TZ + (cz + kk);
#pragma unroll
            for (int f = 0; f < NACC; f++)
                if (f < nf) atomicAdd(t + f * TN, acc.field(jj * 3 + kk, f));
        }
}

// tile -> the 8 neighbouring grid blocks: z columns split at the block boundary (4 + 2 nodes), vector atomics;
// the tile is cleared behind the flush. nbr: grid slots of the block and its +1 neighbours (x*4 + y*2 + z).
template <class T, class L>
__device__ __forceinline__ void flush_tile(const StepArgs<T>& a, T* tile, const int32_t* nbr, int nf, int tid, int nthreads)
{
    constexpr int TX = L::sx + 2, TY = L::sy + 2, TZ = L::sz + 2, TN = TX * TY * TZ;
    for (int q = tid; q < nf * TX * TY * 2; q += nthreads) {
        const int half = q & 1, col = q >> 1;
        const int f = col / (TX * TY), ab = col % (TX * TY), ta = ab / TY, tb = ab % TY;
        const int ax = ta >= L::sx, ay = tb >= L::sy;
        const int slot = nbr[ax * 4 + ay * 2 + half];
        if ((uint32_t)slot >= a.b_cap) {
            check_failed(a.st, 5);
            continue;
        }
        T* dst = a.acc + ((size_t)slot * NACC + f) * L::nodes + L::element(ta - ax * L::sx, tb - ay * L::sy, 0);
        T* src = tile + f * TN + (ta * TY + tb) * TZ + half * L::sz;
        const int n = half ? TZ - L::sz : L::sz;
        flush_column(dst, src, n);
        for (int z = 0; z < n; z++) src[z] = (T)0;
    }
}

// The fused P2G's node tiles, one per stencil x-offset ii: tile ii holds nodes x = cx + ii for cx in [0, sx), all
// y and z of the block plus its +2 halo. The warps of one offset cover disjoint cx, and within a warp the lanes'
// cells are distinct, so each of the 9 node steps below touches distinct nodes: a plain read-modify-write
// replaces the shared-memory float atomics (about twice their throughput). Lanes of one warp reach the same
// node in different steps, so the steps are separated by __syncwarp (it orders the lanes' shared accesses).
// Every lane of the warp must call it.
template <class L>
struct OffsetTiles {
    static constexpr int TY = L::sy + 2, TZ = L::sz + 2;
    static constexpr int TS = L::sx * TY * TZ; // nodes of one offset's tile (per field)
    static constexpr int ELEMS = 3 * NACC * TS;
};

template <class T, class L>
__device__ __forceinline__ void add_to_offset_tile(const NodeAcc<T>& acc, T* tiles, int cx, int cy, int cz, int ii, int nf)
{
    using OT = OffsetTiles<L>;
    T* base = tiles + ii * NACC * OT::TS + (cx * OT::TY + cy) * OT::TZ + cz;
#pragma unroll
    for (int jj = 0; jj < 3; jj++)
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            T* t = base + jj * OT::TZ + kk;
#pragma unroll
            for (int f = 0; f < NACC; f++)
                if (f < nf) t[f * OT::TS] += acc.field(jj * 3 + kk, f);
            __syncwarp();
        }
}

// node (X, Y, z-column) of the block's 6x6x6 tile = the sum over the offsets ii with X - ii in [0, sx); written to
// the 8 neighbouring grid blocks as flush_tile does, the offset tiles cleared behind the flush
template <class T, int N>
__device__ __forceinline__ void flush_offset_column(T* dst, T* tiles, int f, int X, int Y, int z0)
{
    using L = typename LayoutOf<T>::type;
    using OT = OffsetTiles<L>;
    T v[N];
#pragma unroll
    for (int z = 0; z < N; z++) v[z] = (T)0;
#pragma unroll
    for (int ii = 0; ii < 3; ii++) {
        const int xl = X - ii;
        if (xl < 0 || xl >= L::sx) continue;
        T* src = tiles + (ii * NACC + f) * OT::TS + (xl * OT::TY + Y) * OT::TZ + z0;
#pragma unroll
        for (int z = 0; z < N; z++) {
            v[z] += src[z];
            src[z] = (T)0;
        }
    }
    flush_column(dst, v, N);
}

template <class T, class L>
__device__ __forceinline__ void flush_offset_tiles(const StepArgs<T>& a, T* tiles, const int32_t* nbr, int nf, int tid, int nthreads)
{
    constexpr int TX = L::sx + 2, TY = L::sy + 2;
    static_assert(L::sz + 2 - L::sz == 2, "z columns split 4 + 2");
    for (int q = tid; q < nf * TX * TY * 2; q += nthreads) {
        const int half = q & 1, col = q >> 1;
        const int f = col / (TX * TY), ab = col % (TX * TY), ta = ab / TY, tb = ab % TY;
        const int ax = ta >= L::sx, ay = tb >= L::sy;
        const int slot = nbr[ax * 4 + ay * 2 + half];
        if ((uint32_t)slot >= a.b_cap) {
            check_failed(a.st, 5);
            continue;
        }
        T* dst = a.acc + ((size_t)slot * NACC + f) * L::nodes + L::element(ta - ax * L::sx, tb - ay * L::sy, 0);
        if (half)
            flush_offset_column<T, 2>(dst, tiles, f, ta, tb, L::sz);
        else
            flush_offset_column<T, L::sz>(dst, tiles, f, ta, tb, 0);
    }
}

// CHUNK: particles staged per copy (the tile of particles); the scatter CTA is the consumer threads
// (cell x stencil x-offset) plus one producer warp
// NBUF: staging buffers (1: the next chunk's copy overlaps the tile accumulation and flush of the current
// one; 2: it overlaps the whole chunk)
template <class T, int CHUNK, int NBUF>
struct ScatterShape {
    using L = typename LayoutOf<T>::type;
    static constexpr int NCONS = 3 * L::nodes;
    static constexpr int NT = NCONS + 32;
    static constexpr int VEC = 16 / (int)sizeof(T); // elements per 16 bytes: copy granularity
    static constexpr int WIN = CHUNK + CHUNK / 8 + 8; // payload window per field, >= the span of CHUNK particles
    static constexpr size_t buf_bytes = sizeof(T) * NPAY * WIN;
    static constexpr size_t dyn_bytes = NBUF * buf_bytes;
    static constexpr int MIN_CTAS = sizeof(T) == 4 ? 2 : 1;
    static_assert(CHUNK % 32 == 0 && (WIN * sizeof(T)) % 16 == 0 && (NBUF == 1 || NBUF == 2), "copy alignment, buffers");
};

enum : uint32_t { ITEM_LAST = 1, ITEM_DONE = 2, ITEM_BAD = 4 };

struct ScatterItem {
    uint32_t q0, q1; // sorted particle range of the chunk
    uint32_t base; // payload position of element 0 of the staged window
    uint32_t flags;
    int32_t nf; // accumulator fields in use (4 without damage)
    int32_t nbr[8]; // grid slots of the group's block and its +1 neighbours
};

constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull; // 2 s: far beyond any copy; only a broken pipeline waits this long

// the producer: claims groups, cuts them into chunks and issues one bulk copy per payload field and chunk
template <class T, int CHUNK, int NBUF>
__device__ void scatter_producer(const StepArgs<T>& a, unsigned char* dyn, uint64_t* full, uint64_t* empty, ScatterItem* item)
{
    using S = ScatterShape<T, CHUNK, NBUF>;
    constexpr int WIN = S::WIN, VEC = S::VEC;
    const uint32_t G = a.st->n_groups;
    uint32_t ph_empty = 3u; // parity bit per buffer; a fresh barrier counts as released
    uint32_t issues0 = 0, issues1 = 0;
    int b = 0;
    bool stop = false;
    while (!stop) {
        const uint32_t g = atomicAdd(&a.st->work_p2g, 1u);
        uint32_t qs = 0, qe = 0, flags = 0;
        int nf = 4;
        int32_t nbr[8];
        if (g < G) {
            qs = a.g_start[g];
            qe = (g + 1 < G) ? a.g_start[g + 1] : a.n_total;
            nf = a.scenes[a.kl.scene(a.kl.at(a.keys_sorted, qs))].damage ? NACC : 4;
#pragma unroll
            for (int d = 0; d < 8; d++) {
                nbr[d] = a.g_nbr[g * 8 + d];
                if (nbr[d] < 0) flags |= ITEM_BAD; // the lookup failed and raised FLAG_CAPACITY
                else if ((uint32_t)nbr[d] >= a.b_cap) {
                    check_failed(a.st, 4);
                    flags |= ITEM_BAD;
                }
            }
            if (qe <= qs || qe > a.n_total) {
                check_failed(a.st, 1);
                flags |= ITEM_BAD;
                qe = qs + 1 <= a.n_total ? qs + 1 : qs; // keep the pipeline moving with an in-bounds chunk
            }
        }
        else
            flags = ITEM_DONE;
        uint32_t q0 = qs;
        do {
            if (!mbar_wait(&empty[b], (ph_empty >> b) & 1u, WAIT_LIMIT_NS)) {
                raise_flag(a.st, FLAG_TIMEOUT);
                stop = true;
                break;
            }
            ph_empty ^= 1u << b;
            ScatterItem& it = item[b];
            if (b) issues1++;
            else issues0++;
            if (flags & ITEM_DONE) {
                it.flags = ITEM_DONE;
                mbar_arrive(&full[b]);
                stop = true;
                break;
            }
            const uint32_t q1 = min(q0 + (uint32_t)CHUNK, qe);
            const uint64_t p0 = pay_pos(q0) & ~(uint64_t)(VEC - 1);
            const uint64_t p1 = (pay_pos(q1 - 1) + VEC) & ~(uint64_t)(VEC - 1);
            uint32_t bytes = (uint32_t)(p1 - p0) * (uint32_t)sizeof(T);
            uint64_t src0 = p0;
            if (p1 > (uint64_t)a.pstride || bytes > (uint32_t)(WIN * sizeof(T))) { // never expected: record it, copy 16 in-bounds bytes
                check_failed(a.st, 2);
                flags |= ITEM_BAD;
                bytes = 16;
                src0 = 0;
            }
            it.q0 = q0;
            it.q1 = q1;
            it.base = (uint32_t)p0;
            it.flags = flags | (q1 == qe ? ITEM_LAST : 0u);
            it.nf = nf;
#pragma unroll
            for (int d = 0; d < 8; d++) it.nbr[d] = nbr[d];
            T* dst = reinterpret_cast<T*>(dyn + b * S::buf_bytes);
            fence_async_smem();
            mbar_arrive_expect_tx(&full[b], bytes * NPAY);
            for (int f = 0; f < NPAY; f++) bulk_load(dst + f * WIN, a.pay + f * a.pstride + src0, bytes, &full[b]);
            b = NBUF == 2 ? b ^ 1 : 0;
            q0 = q1;
        } while (q0 < qe);
    }
    // leave no copy in flight behind: wait (bounded) for the last phase issued on each buffer
    if (issues0) mbar_wait(&full[0], (issues0 - 1) & 1u, WAIT_LIMIT_NS);
    if (issues1) mbar_wait(&full[1], (issues1 - 1) & 1u, WAIT_LIMIT_NS);
}

template <class T, int CHUNK, int NBUF, int MIN_CTAS = ScatterShape<T, CHUNK, NBUF>::MIN_CTAS>
__global__ void __launch_bounds__(ScatterShape<T, CHUNK, NBUF>::NT, MIN_CTAS) k_scatter(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using S = ScatterShape<T, CHUNK, NBUF>;
    constexpr int NCONS = S::NCONS, WIN = S::WIN, NC = L::nodes;
    constexpr int TX = L::sx + 2, TY = L::sy + 2, TZ = L::sz + 2, TN = TX * TY * TZ;
    extern __shared__ __align__(128) unsigned char scat_dyn[];
    __shared__ T tile[NACC * TN];
    __shared__ __align__(8) uint64_t full[2], empty[2];
    __shared__ ScatterItem item[2];
    __shared__ int16_t cfirst[2][NC], clast[2][NC];
    __shared__ uint32_t ctag[2][NC];
    __shared__ int32_t s_nbr[8]; // the grid slots of the group being flushed (the item is released before the flush)
    __shared__ int s_stop;
    if (aborted_cta(a.st)) return;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&empty[0], NCONS / 32); // one arrival per consumer warp
        mbar_init(&empty[1], NCONS / 32);
        mbar_init_fence();
        s_stop = 0;
    }
    for (int q = tid; q < NACC * TN; q += S::NT) tile[q] = (T)0;
    for (int q = tid; q < 2 * NC; q += S::NT) (&ctag[0][0])[q] = 0xffffffffu;
    __syncthreads();
    if (tid >= NCONS) { // the producer warp (one lane works); no CTA-wide barrier follows this point
        if (tid == NCONS) scatter_producer<T, CHUNK, NBUF>(a, scat_dyn, full, empty, item);
        return;
    }
    // consumer role: cell c, stencil x-offset ii
    const int ii = tid / NC, c = tid % NC;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    uint32_t ph_full = 0; // parity bit per buffer
    int b = 0;
    for (uint32_t seq = 0;; seq++) {
        const bool ready = mbar_wait(&full[b], (ph_full >> b) & 1u, WAIT_LIMIT_NS);
        ph_full ^= 1u << b;
        const T* buf = reinterpret_cast<const T*>(scat_dyn + b * S::buf_bytes);
        const ScatterItem& it = item[b];
        uint32_t fl = ITEM_DONE;
        uint32_t q0 = 0, base = 0;
        if (!ready) {
            s_stop = 1;
            raise_flag(a.st, FLAG_TIMEOUT);
        }
        else {
            fl = it.flags;
            q0 = it.q0;
            base = it.base;
            if (!(fl & (ITEM_DONE | ITEM_BAD)) && (it.q1 <= q0 || it.q1 - q0 > (uint32_t)CHUNK || pay_pos(it.q1 - 1) - base >= (uint64_t)WIN)) {
                check_failed(a.st, 6); // an item that does not fit its window: skip it
                fl |= ITEM_BAD;
            }
            if (!(fl & (ITEM_DONE | ITEM_BAD))) {
                // runs of equal cells (particles are sorted by cell inside a block)
                const uint32_t q1 = it.q1;
                const T* cellv = buf + Y_CELL * WIN;
                for (uint32_t q = q0 + tid; q < q1; q += NCONS) {
                    const int e = (int)cellv[pay_pos(q) - base];
                    if ((unsigned)e >= (unsigned)NC) continue; // 255 marks a particle whose key disagreed
                    const int ep = q > q0 ? (int)cellv[pay_pos(q - 1) - base] : -1;
                    if (ep > e) check_failed(a.st, 3); // cells must ascend inside a block: the staged data is not what was written
                    if (q == q0 || ep != e) {
                        cfirst[b][e] = (int16_t)(q - q0);
                        ctag[b][e] = seq;
                    }
                    if (q + 1 == q1 || (int)cellv[pay_pos(q + 1) - base] != e) clast[b][e] = (int16_t)(q + 1 - q0);
                }
            }
        }
        bar_sync(1, NCONS);
        if (s_stop || (fl & ITEM_DONE)) break;
        const int nf = it.nf;
        const bool damage = nf == NACC;
        if ((fl & ITEM_LAST) && tid < 8) s_nbr[tid] = it.nbr[tid]; // read before this warp releases the item
        // per (cell, stencil x-offset): register accumulators of the thread's 9 nodes
        NodeAcc<T> acc;
        acc.zero();
        // decided once: after the release below, faster warps may already mark the next chunk
        const bool mine = !(fl & ITEM_BAD) && ctag[b][c] == seq;
        if (mine) {
            const uint32_t qa = q0 + cfirst[b][c], qb = q0 + clast[b][c];
            if (damage)
                for (uint32_t q = qa; q < qb; q++) accumulate_particle<T, WIN, true>(acc, buf + (pay_pos(q) - base), ii);
            else
                for (uint32_t q = qa; q < qb; q++) accumulate_particle<T, WIN, false>(acc, buf + (pay_pos(q) - base), ii);
        }
        // the chunk's payload is no longer needed: release the buffer (and the item) to the producer
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&empty[b]);
        if (mine) add_to_tile<T, L>(acc, tile, cx, cy, cz, ii, nf);
        if (fl & ITEM_LAST) {
            bar_sync(1, NCONS); // every chunk of the group is in the tile
            if (!(fl & ITEM_BAD)) flush_tile<T, L>(a, tile, s_nbr, nf, tid, NCONS);
        }
        b = NBUF == 2 ? b ^ 1 : 0;
    }
}

// The fused P2G: one kernel per substep with the same arithmetic, the stress evaluated in the kernel. Per
// group, phase 1 (thread per particle) loads the particle state through the sorted order and stages its
// payload in shared memory (bank-staggered at q + q/8); phases 2 and 3 are those of k_scatter. No payload
// round trip through HBM, at the price of the state loads' latency inside the kernel: the autotuner times
// both forms on the workload.
// CH: particles staged per chunk (a whole block at 8 per cell by default; half of it lets more CTAs fit)
template <class T, int CH = (sizeof(T) == 4 ? 512 : 256)>
struct FusedShape {
    using L = typename LayoutOf<T>::type;
    static constexpr int NT = 3 * L::nodes; // cells x stencil x-offsets
    static constexpr int CHUNK = CH;
    static constexpr int CPAD = CHUNK + CHUNK / 8;
    static constexpr size_t dyn_bytes = sizeof(T) * Y_CELL * CPAD; // fields Y_F..Y_D
};

// Elements [lo, hi] of one array, prefetched into L2 (widened to 16-byte boundaries, kept inside [base, end)).
template <class E>
__device__ __forceinline__ void prefetch_l2_range(const E* arr, int64_t lo, int64_t hi, const void* base, const void* end)
{
    uintptr_t b0 = (uintptr_t)(arr + lo) & ~(uintptr_t)15, b1 = ((uintptr_t)(arr + hi + 1) + 15) & ~(uintptr_t)15;
    const uintptr_t lo_lim = ((uintptr_t)base + 15) & ~(uintptr_t)15, hi_lim = (uintptr_t)end & ~(uintptr_t)15;
    b0 = b0 < lo_lim ? lo_lim : b0;
    b1 = b1 > hi_lim ? hi_lim : b1;
    if (b1 > b0) bulk_prefetch_l2((const void*)b0, (uint32_t)(b1 - b0));
}

// MINB: CTAs per SM the register budget is cut for (more CTAs hide more load latency; fewer registers may spill)
template <class T, int MODELS, int MINB, int CH = FusedShape<T>::CHUNK>
__global__ void __launch_bounds__(FusedShape<T, CH>::NT, MINB) k_p2g_fused(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using S = FusedShape<T, CH>;
    constexpr int NT = S::NT, CHUNK = S::CHUNK, CPAD = S::CPAD, NC = L::nodes;
    extern __shared__ __align__(16) unsigned char fused_dyn[];
    T* pay = reinterpret_cast<T*>(fused_dyn);
    __shared__ T tile[OffsetTiles<L>::ELEMS]; // one node tile per stencil x-offset
    __shared__ uint8_t cellof[CHUNK];
    // the set-up of the current group (buffer b) and of the next one (b ^ 1): group, scene, a bad neighbour slot,
    // the grid slots of the block and its +1 neighbours, the block origin, the sorted range
    __shared__ int s_g[2], s_scene[2], s_bad[2];
    __shared__ int32_t s_nbr[2][8];
    __shared__ int s_org[2][3];
    __shared__ uint32_t s_se[2][2];
    if (aborted_cta(a.st)) return;
    const uint32_t G = a.st->n_groups;
    const int tid = threadIdx.x;
    // Groups are claimed one ahead: warp 0 claims the next group at the start of a group; around the group's flush
    // lanes 0-7 load its range and neighbour slots (lane 0 also the key of its first particle) and write them into
    // the other buffer before the group's last barrier, so no barrier waits on a claim alone.
    auto claim = [&]() { // warp 0 only: the next group index, in every lane
        int v = 0;
        if (tid == 0) v = (int)atomicAdd(&a.st->work_p2g, 1u);
        return __shfl_sync(0xffffffffu, v, 0);
    };
    auto setup_store = [&](int bb, int gn, uint32_t st, uint32_t en, int32_t slot, uint64_t key0) { // lanes 0-7 of warp 0
        const unsigned badm = __ballot_sync(0xffu, slot < 0 || (uint32_t)slot >= a.b_cap); // a failed lookup raised FLAG_CAPACITY
        s_nbr[bb][tid] = slot;
        if (tid == 0) {
            uint32_t bi, bj, bk;
            L::block_of_page(a.kl.page(key0), bi, bj, bk);
            s_g[bb] = gn;
            s_bad[bb] = badm != 0;
            s_scene[bb] = (int)a.kl.scene(key0);
            s_org[bb][0] = (int)(bi * L::sx);
            s_org[bb][1] = (int)(bj * L::sy);
            s_org[bb][2] = (int)(bk * L::sz);
            s_se[bb][0] = st;
            s_se[bb][1] = en;
        }
    };
    // A group's neighbour entries hold hash positions (activation); the set-up translates them into grid slots and
    // writes the slots back for G2P.
    auto take_slot = [&](int gg, int32_t hpos) { // lanes 0-7 of warp 0
        const int32_t slot = nbr_slot(a, hpos);
        a.g_nbr[gg * 8 + tid] = slot;
        return slot;
    };
    const int ii = tid / NC, c = tid % NC;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    for (int q = tid; q < OffsetTiles<L>::ELEMS; q += NT) tile[q] = (T)0;
    uint32_t fallbacks = 0;
    if (tid < 32) { // the first group
        const int g0 = claim();
        if (g0 < (int)G) {
            if (tid < 8) {
                const uint32_t st = a.g_start[g0], en = g0 + 1 < (int)G ? a.g_start[g0 + 1] : a.n_total;
                setup_store(0, g0, st, en, take_slot(g0, a.g_nbr[g0 * 8 + tid]), tid == 0 ? a.kl.at(a.keys_sorted, st) : 0ull);
            }
        }
        else if (tid == 0)
            s_g[0] = g0;
    }
    __syncthreads();
    int bcur = 0;
    for (;;) {
        const int g = s_g[bcur];
        if (g >= (int)G) break;
        // the next group, claimed now (its set-up is loaded around this group's flush)
        const int gn = tid < 32 ? claim() : (int)G;
        const uint32_t start = s_se[bcur][0], end = s_se[bcur][1];
        const bool bad = s_bad[bcur] != 0;
        const SceneParams<T>& sp = a.scenes[s_scene[bcur]];
        const int nf = sp.damage ? NACC : 4;
        // The state of the group one round of claims ahead (whichever CTA takes it) is prefetched into L2 while this
        // group runs, so that its phase 1 reads L2: the lanes of warp 1 take one array each (state fields P_X .. P_D
        // and the particle ids). Its storage range is that of its first and last sorted particles (storage keeps the
        // previous substep's sorted order; a range that does not look like one group is skipped). The loads are
        // spread over the group so that none of them is waited for.
        constexpr int NPF = P_D + 2;
        const int gpf = g + (int)gridDim.x, pfl = tid - 32;
        const bool pf = (a.opts & OPT_PREFETCH) && pfl >= 0 && pfl < NPF && gpf < (int)G;
        uint32_t pf_a = 0, pf_b = 0, pf_j0 = 0, pf_j1 = 0;
        if (pf) {
            pf_a = a.g_start[gpf];
            pf_b = gpf + 1 < (int)G ? a.g_start[gpf + 1] : a.n_total;
        }
        for (uint32_t c0 = start; c0 < end && !bad; c0 += CHUNK) {
            const int cnt = (int)min((uint32_t)CHUNK, end - c0);
            // ---- phase 1: per particle
            // the storage slots of all the thread's particles first (one latency for all), then one particle at a time
            constexpr int PER = (CHUNK + NT - 1) / NT;
            uint32_t js[PER];
#pragma unroll
            for (int k = 0; k < PER; k++) js[k] = tid + k * NT < cnt ? a.vals_sorted[c0 + tid + k * NT] : 0u;
#pragma unroll
            for (int k = 0; k < PER; k++) {
                const int q = tid + k * NT;
                if (q >= cnt) break;
                int b[3];
                particle_payload<T, MODELS>(a.pin, js[k], sp, pay + (q + (q >> 3)), CPAD, b, fallbacks);
                const int l0 = b[0] - s_org[bcur][0], l1 = b[1] - s_org[bcur][1], l2 = b[2] - s_org[bcur][2];
                const bool inside = l0 >= 0 && l0 < L::sx && l1 >= 0 && l1 < L::sy && l2 >= 0 && l2 < L::sz;
                if (!inside) raise_flag(a.st, FLAG_CAPACITY); // keys and positions disagree: abort the substep
                cellof[q] = inside ? (uint8_t)L::element(l0, l1, l2) : (uint8_t)0xff;
            }
            __syncthreads();
            // ---- phases 2 and 3. Particles of one cell are contiguous and the cells ascend (sorted by cell inside
            // the block): the cell's range by two binary searches over the chunk's cells, no pass or barrier of its
            // own (a position that disagreed with its key has raised FLAG_CAPACITY; the searches stay in [0, cnt])
            auto cell_lower = [&](int v) {
                int lo = 0, hi = cnt;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cellof[mid] < v) lo = mid + 1;
                    else hi = mid;
                }
                return lo;
            };
            const int qa = cell_lower(c), qb = cell_lower(c + 1);
            NodeAcc<T> acc;
            acc.zero();
            if (nf == NACC)
                for (int q = qa; q < qb; q++) accumulate_particle<T, CPAD, true>(acc, pay + (q + (q >> 3)), ii);
            else
                for (int q = qa; q < qb; q++) accumulate_particle<T, CPAD, false>(acc, pay + (q + (q >> 3)), ii);
            add_to_offset_tile<T, L>(acc, tile, cx, cy, cz, ii, nf); // all lanes (an empty cell adds zeros)
            __syncthreads();
        }
        uint32_t n_st = 0, n_en = 0;
        int32_t n_hpos = -1;
        if (tid < 8 && gn < (int)G) {
            n_st = a.g_start[gn];
            n_en = gn + 1 < (int)G ? a.g_start[gn + 1] : a.n_total;
            n_hpos = a.g_nbr[gn * 8 + tid];
        }
        if (pf && pf_b > pf_a && pf_b <= a.n_total) {
            pf_j0 = a.vals_sorted[pf_a];
            pf_j1 = a.vals_sorted[pf_b - 1];
        }
        if (!bad) flush_offset_tiles<T, L>(a, tile, s_nbr[bcur], nf, tid, NT);
        if (pf && pf_j1 >= pf_j0 && pf_j1 - pf_j0 < 2 * (pf_b - pf_a) + 64) {
            const Pool<T>& P = a.pin;
            if (pfl < NPF - 1)
                prefetch_l2_range(P.f + (int64_t)pfl * P.stride, pf_j0, pf_j1, P.f, P.f + (int64_t)P_NF * P.stride);
            else
                prefetch_l2_range(P.pid, pf_j0, pf_j1, P.pid, P.pid + P.stride);
        }
        // the next group's set-up into the other buffer (the flush above read this one)
        if (tid < 8) {
            if (gn < (int)G)
                setup_store(bcur ^ 1, gn, n_st, n_en, take_slot(gn, n_hpos), tid == 0 ? a.kl.at(a.keys_sorted, n_st) : 0ull);
            else if (tid == 0)
                s_g[bcur ^ 1] = gn;
        }
        __syncthreads();
        bcur ^= 1;
    }
    if (fallbacks) atomicAdd(&a.st->fallback, fallbacks);
}

// ---------------------------------------------------------------------------------------------------
// Warp-specialised fused P2G (the same arithmetic as k_p2g_fused). Producer warps load each chunk's particle
// state, evaluate V0 tau and stage the payload in one of NSTAGE shared-memory buffers; consumer warps (thread per
// (cell, stencil x-offset)) accumulate the previous buffer meanwhile, so the state loads' latency and the
// accumulation overlap inside the CTA instead of alternating behind CTA-wide barriers. Hand-offs are mbarriers:
// full[s] completes when every producer thread has written buffer s, empty[s] when every consumer warp has read
// it. A group's node tiles are double-buffered: the consumer warps meet on one mbarrier before the flush of a
// group, while the next group's additions go to the other tile buffer. Every wait is bounded (2 s) and raises
// FLAG_TIMEOUT. Groups are dealt to CTAs round-robin (blockIdx, + gridDim, ...), so every producer thread knows
// the sequence of chunks without exchanging it.
// ---------------------------------------------------------------------------------------------------
template <class T>
struct WsShape {
    using L = typename LayoutOf<T>::type;
    static constexpr int NCONS = 3 * L::nodes; // consumers: cells x stencil x-offsets
    static constexpr int NPROD = sizeof(T) == 4 ? 128 : 64;
    static constexpr int NT = NCONS + NPROD;
    static constexpr int CHUNK = sizeof(T) == 4 ? 256 : 128;
    static constexpr int CPAD = CHUNK + CHUNK / 8;
    static constexpr int NSTAGE = 2;
    static constexpr size_t pay_bytes = sizeof(T) * Y_CELL * CPAD;
    static constexpr size_t stage_bytes = pay_bytes + CHUNK; // payload fields Y_F..Y_D, then the cells
    static constexpr size_t dyn_bytes = NSTAGE * stage_bytes;
    static_assert(pay_bytes % 16 == 0 && NCONS % 32 == 0 && NPROD % 32 == 0, "whole warps, aligned buffers");
};

struct WsItem {
    uint32_t c0; // first sorted particle of the chunk
    int32_t cnt, flags, scene, nf;
    int32_t nbr[8];
};

template <class T, int MODELS>
__global__ void __launch_bounds__(WsShape<T>::NT, 2) k_p2g_ws(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using S = WsShape<T>;
    using OT = OffsetTiles<L>;
    constexpr int NCONS = S::NCONS, NPROD = S::NPROD, CHUNK = S::CHUNK, CPAD = S::CPAD, NST = S::NSTAGE, NC = L::nodes;
    extern __shared__ __align__(16) unsigned char ws_dyn[];
    __shared__ T tiles[2][OT::ELEMS]; // one set of per-offset node tiles per group parity
    __shared__ __align__(8) uint64_t full[NST], empty[NST], flushed;
    __shared__ WsItem item[NST];
    __shared__ int32_t s_nbr[2][8];
    if (aborted_cta(a.st)) return;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < NST; s++) {
            mbar_init(&full[s], NPROD);
            mbar_init(&empty[s], NCONS / 32);
        }
        mbar_init(&flushed, NCONS / 32);
        mbar_init_fence();
    }
    for (int q = tid; q < 2 * OT::ELEMS; q += S::NT) (&tiles[0][0])[q] = (T)0;
    __syncthreads(); // the last CTA-wide barrier: the roles never meet again
    const uint32_t G = a.st->n_groups;
    if (tid >= NCONS) {
        // ---------------- producers
        const int pt = tid - NCONS;
        uint32_t fallbacks = 0, k = 0;
        bool stop = false;
        for (uint32_t g = blockIdx.x; g < G && !stop; g += gridDim.x) {
            const uint32_t start = a.g_start[g], end = (g + 1 < G) ? a.g_start[g + 1] : a.n_total;
            const uint64_t key0 = a.kl.at(a.keys_sorted, start);
            uint32_t bi, bj, bk;
            L::block_of_page(a.kl.page(key0), bi, bj, bk);
            const int scene = (int)a.kl.scene(key0);
            const int org0 = (int)(bi * L::sx), org1 = (int)(bj * L::sy), org2 = (int)(bk * L::sz);
            const SceneParams<T>& sp = a.scenes[scene];
            int bad = (end <= start || end > a.n_total) ? 1 : 0;
            if (bad) check_failed(a.st, 1);
            for (uint32_t c0 = start; c0 < end || (bad && c0 == start); c0 += CHUNK) {
                const int s = k % NST;
                if (!mbar_wait(&empty[s], ((k / NST) & 1u) ^ 1u, WAIT_LIMIT_NS)) {
                    raise_flag(a.st, FLAG_TIMEOUT);
                    stop = true;
                    break;
                }
                const int cnt = bad ? 0 : (int)min((uint32_t)CHUNK, end - c0);
                const bool last = bad || c0 + CHUNK >= end;
                WsItem& it = item[s];
                if (pt < 32) { // the first producer warp fills the item; a failed slot lookup raised FLAG_CAPACITY
                    int slot = 0;
                    if (pt < 8) {
                        slot = a.g_nbr[g * 8 + pt];
                        it.nbr[pt] = slot;
                    }
                    const bool nbad = __ballot_sync(0xffffffffu, pt < 8 && (slot < 0 || (uint32_t)slot >= a.b_cap)) != 0;
                    if (pt == 0) {
                        it.c0 = c0;
                        it.cnt = cnt;
                        it.scene = scene;
                        it.nf = sp.damage ? NACC : 4;
                        it.flags = (last ? ITEM_LAST : 0) | ((bad || nbad) ? ITEM_BAD : 0);
                    }
                }
                T* pay = reinterpret_cast<T*>(ws_dyn + s * S::stage_bytes);
                uint8_t* cellof = ws_dyn + s * S::stage_bytes + S::pay_bytes;
                constexpr int PER = (CHUNK + NPROD - 1) / NPROD;
                uint32_t js[PER];
#pragma unroll
                for (int r = 0; r < PER; r++) js[r] = pt + r * NPROD < cnt ? a.vals_sorted[c0 + pt + r * NPROD] : 0u;
#pragma unroll
                for (int r = 0; r < PER; r++) {
                    const int q = pt + r * NPROD;
                    if (q >= cnt) break;
                    int b[3];
                    particle_payload<T, MODELS>(a.pin, js[r], sp, pay + (q + (q >> 3)), CPAD, b, fallbacks);
                    const int l0 = b[0] - org0, l1 = b[1] - org1, l2 = b[2] - org2;
                    const bool inside = l0 >= 0 && l0 < L::sx && l1 >= 0 && l1 < L::sy && l2 >= 0 && l2 < L::sz;
                    if (!inside) raise_flag(a.st, FLAG_CAPACITY); // keys and positions disagree: abort the substep
                    cellof[q] = inside ? (uint8_t)L::element(l0, l1, l2) : (uint8_t)0xff;
                }
                mbar_arrive(&full[s]);
                k++;
                if (bad) break;
            }
        }
        if (!stop) { // the end marker
            const int s = k % NST;
            if (mbar_wait(&empty[s], ((k / NST) & 1u) ^ 1u, WAIT_LIMIT_NS)) {
                if (pt == 0) item[s].flags = ITEM_DONE;
                mbar_arrive(&full[s]);
            }
            else
                raise_flag(a.st, FLAG_TIMEOUT);
        }
        if (fallbacks) atomicAdd(&a.st->fallback, fallbacks);
        return;
    }
    // ---------------- consumers: cell c, stencil x-offset ii
    const int ii = tid / NC, c = tid % NC, lane = tid & 31;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    int tb = 0; // tile buffer of the current group
    uint32_t gseq = 0; // groups flushed (parity of the flush barrier)
    for (uint32_t k = 0;; k++) {
        const int s = k % NST;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[s], (k / NST) & 1u, WAIT_LIMIT_NS));
        if (!ok) {
            if (lane == 0) raise_flag(a.st, FLAG_TIMEOUT);
            break;
        }
        const WsItem& it = item[s];
        const int fl = it.flags;
        if (fl & ITEM_DONE) break;
        const int cnt = it.cnt, nf = it.nf;
        const T* pay = reinterpret_cast<const T*>(ws_dyn + s * S::stage_bytes);
        const uint8_t* cellof = ws_dyn + s * S::stage_bytes + S::pay_bytes;
        if ((fl & ITEM_LAST) && tid < 8) s_nbr[tb][tid] = it.nbr[tid]; // read before this warp releases the buffer
        NodeAcc<T> acc;
        acc.zero();
        const bool use = !(fl & ITEM_BAD);
        if (use) {
            auto cell_lower = [&](int v) {
                int lo = 0, hi = cnt;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cellof[mid] < v) lo = mid + 1;
                    else hi = mid;
                }
                return lo;
            };
            const int qa = cell_lower(c), qb = cell_lower(c + 1);
            if (nf == NACC)
                for (int q = qa; q < qb; q++) accumulate_particle<T, CPAD, true>(acc, pay + (q + (q >> 3)), ii);
            else
                for (int q = qa; q < qb; q++) accumulate_particle<T, CPAD, false>(acc, pay + (q + (q >> 3)), ii);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]); // the buffer is free for the producers
        if (use) add_to_offset_tile<T, L>(acc, tiles[tb], cx, cy, cz, ii, nf); // all lanes (an empty cell adds zeros)
        if (fl & ITEM_LAST) {
            // every consumer warp has added the group: flush its tiles (the next group fills the other tile buffer)
            __syncwarp();
            if (lane == 0) mbar_arrive(&flushed);
            const bool fok = __all_sync(0xffffffffu, mbar_wait(&flushed, gseq & 1u, WAIT_LIMIT_NS));
            gseq++;
            if (!fok) {
                if (lane == 0) raise_flag(a.st, FLAG_TIMEOUT);
                break;
            }
            if (use) flush_offset_tiles<T, L>(a, tiles[tb], s_nbr[tb], nf, tid, NCONS);
            else
                for (int q = tid; q < OT::ELEMS; q += NCONS) tiles[tb][q] = (T)0; // a bad group's partial sums are dropped
            tb ^= 1;
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// grid update
// ---------------------------------------------------------------------------------------------------
constexpr int GRID_NT = 256; // threads per CTA of the grid update

template <class T>
__global__ void __launch_bounds__(GRID_NT) k_grid(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    // GV consecutive nodes of one block per thread: every field moves as one 16-byte access; TPB threads cover
    // one block (16 in both precisions), so a warp spans 32 / TPB blocks, which may belong to different scenes
    constexpr int GV = (int)(16 / sizeof(T));
    constexpr int TPB = L::nodes / GV;
    static_assert(L::nodes % GV == 0, "a block holds whole vectors");
    static_assert(32 % TPB == 0 && GRID_NT % TPB == 0, "a warp holds whole blocks");
    __shared__ double s_mass[GRID_NT / TPB];
    __shared__ int s_msc[GRID_NT / TPB];
    if (aborted_cta(a.st)) return;
    const uint32_t B = min(a.st->n_blocks, a.b_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->max_blocks_seen = max(a.st->max_blocks_seen, B);
    const uint32_t total = B * (L::nodes / GV);
    // every thread of the CTA runs the same iterations (the loop holds barriers)
    for (uint32_t base = blockIdx.x * GRID_NT; base < total; base += gridDim.x * GRID_NT) {
        const uint32_t t = base + threadIdx.x;
        double gm = 0; // grid mass of the thread's nodes, accumulated in FP64 from the first add
        int scene = -1;
        if (t < total) {
            const uint32_t b = t / (L::nodes / GV), e0 = (t % (L::nodes / GV)) * GV;
            const uint64_t hk = a.b_key[b];
            scene = (int)(hk >> 40);
            const SceneParams<T>& sp = a.scenes[scene];
            Vec16<T>* A = reinterpret_cast<Vec16<T>*>(a.acc + (size_t)b * NACC * L::nodes + e0);
            constexpr int FS = L::nodes / GV; // field stride in vectors
            const Vec16<T> m = A[0], P0 = A[FS], P1 = A[2 * FS], P2 = A[3 * FS], pf = A[4 * FS], pfm = A[5 * FS];
            Vec16<T> zero;
#pragma unroll
            for (int k = 0; k < GV; k++) zero.v[k] = (T)0;
#pragma unroll
            for (int q = 0; q < NACC; q++) A[q * FS] = zero;
            Vec16<T> o0, o1, o2, o3;
            uint32_t bi, bj, bk;
            L::block_of_page(hk & ((1ULL << 40) - 1), bi, bj, bk);
            const T dt = sp.dt;
#pragma unroll
            for (int k = 0; k < GV; k++) {
                const T mk = m.v[k];
                gm += (double)mk;
                if (mk != (T)0) {
                    const int e = (int)e0 + k;
                    const int lx = e >> (L::zbits + L::ybits), ly = (e >> L::zbits) & (L::sy - 1), lz = e & (L::sz - 1);
                    const T xi[3] = { (T)(bi * L::sx + lx) * sp.dx, (T)(bj * L::sy + ly) * sp.dx, (T)(bk * L::sz + lz) * sp.dx };
                    // P = m v + dt f: v + g dt + f dt / m (MpmSimulationBase.cpp:1204-1210)
                    T vi[3] = { P0.v[k] / mk + sp.gravity[0] * dt, P1.v[k] / mk + sp.gravity[1] * dt, P2.v[k] / mk + sp.gravity[2] * dt };
                    collide(sp, (T)sp.time, xi, vi);
                    o0.v[k] = vi[0];
                    o1.v[k] = vi[1];
                    o2.v[k] = vi[2];
                    o3.v[k] = pfm.v[k] != (T)0 ? pf.v[k] / pfm.v[k] : (T)0;
                }
                else
                    o0.v[k] = o1.v[k] = o2.v[k] = o3.v[k] = (T)0;
            }
            Vec16<T>* V = reinterpret_cast<Vec16<T>*>(a.vel + (size_t)b * NVEL * L::nodes + e0);
            V[0] = o0;
            V[FS] = o1;
            V[2 * FS] = o2;
            V[3 * FS] = o3;
        }
        // grid mass per scene (MpmSimulationDataAnalysis.h:130-151, FP64): the TPB threads of one block (one scene)
        // sum in a segmented shuffle, then thread 0 combines the CTA's block sums, one atomic per run of blocks of
        // one scene (a single scene would otherwise send every block's atomic to the same address). Threads past
        // the last block form whole segments with scene -1 (total and base are multiples of TPB).
        double s = gm;
        for (int o = TPB / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPB);
        if (threadIdx.x % TPB == 0) {
            s_mass[threadIdx.x / TPB] = s;
            s_msc[threadIdx.x / TPB] = scene;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double run = 0;
            int rsc = -1;
            for (int w = 0; w < GRID_NT / TPB; w++) {
                if (s_msc[w] != rsc) {
                    if (rsc >= 0 && run != 0.0) atomicAdd(&a.grid_mass[rsc], run);
                    rsc = s_msc[w];
                    run = 0;
                }
                run += s_mass[w];
            }
            if (rsc >= 0 && run != 0.0) atomicAdd(&a.grid_mass[rsc], run);
        }
        __syncthreads();
    }
    // the hash table is used only by activate and P2G: clear it for the next substep
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h <= a.h_mask; h += gridDim.x * blockDim.x) a.h_keys[h] = HASH_EMPTY;
}

// ---------------------------------------------------------------------------------------------------
// G2P
// ---------------------------------------------------------------------------------------------------
// NT threads per CTA; RESIDENT: threads per SM the register budget is cut for
// G2P's staged particle state: x, F, m, V0, d, sigma_c (fields G2P_SF) and the pid, per thread and buffer
enum { GS_X = 0, GS_F = 3, GS_M = 12, GS_V0 = 13, GS_D = 14, GS_SC = 15, G2P_SF = 16 };
template <class T, int NT>
struct G2pStage {
    // double-buffered per-thread slots, field-major so a warp's accesses are consecutive words; off where the
    // buffers would not fit the 48 KB of static shared memory (FP64 at 256 threads)
    static constexpr bool ON = 2 * NT * (G2P_SF * sizeof(T) + 4) <= 40 * 1024;
    static constexpr int NS = ON ? 2 * G2P_SF * NT : 1, NP = ON ? 2 * NT : 1;
};

// BULK: the 8 neighbouring blocks' velocities reach shared memory by bulk asynchronous copies (one 4-field block of
// NVEL * nodes values per copy, completing on an mbarrier) and the node tile is built from there; otherwise each
// thread loads its tile nodes from global memory
template <class T, int NT, int RESIDENT, bool BULK = false>
__global__ void __launch_bounds__(NT, RESIDENT / NT) k_g2p(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using GS = G2pStage<T, NT>;
    constexpr int BLK = NVEL * L::nodes; // values of one block's velocity fields (1 KB in both precisions)
    __shared__ __align__(128) T s_halo[BULK ? 8 * BLK : 1];
    __shared__ __align__(8) uint64_t s_hbar;
    uint32_t hphase = 0;
    // the grid velocities around the group's block as one dense node tile (the block plus 2 nodes on the
    // + side of every axis, the reach of the quadratic stencil): every stencil read is a fixed offset
    constexpr int TY = L::sy + 2, TZ = L::sz + 2, TN = (L::sx + 2) * TY * TZ;
    static_assert(NVEL == 4, "one Quad per tile node");
    __shared__ Quad<T> tq[TN]; // node-major: the 4 fields of a node in one access
    __shared__ Material<T> s_mat[MAX_MATERIALS]; // the group's scene's materials
    __shared__ T s_st[GS::NS]; // staged state of the thread's current and next particle
    __shared__ uint32_t s_pid[GS::NP];
    __shared__ int s_g, s_nbr[8], s_scene, s_org[3];
    __shared__ uint16_t s_map[TN]; // tile node -> (neighbour block 0-7) << 8 | element in that block
    if (aborted_cta(a.st)) return;
    if (BULK && threadIdx.x == 0) {
        mbar_init(&s_hbar, 1);
        mbar_init_fence();
    }
    for (int node = threadIdx.x; node < TN; node += NT) {
        const int tx = node / (TY * TZ), ty = (node / TZ) % TY, tz = node % TZ;
        const int ax = tx >= L::sx, ay = ty >= L::sy, az = tz >= L::sz;
        s_map[node] = (uint16_t)(((ax * 4 + ay * 2 + az) << 8) | L::element(tx - ax * L::sx, ty - ay * L::sy, tz - az * L::sz));
    }
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
                uint64_t key0 = a.kl.at(a.keys_sorted, start);
                uint32_t bi, bj, bk;
                L::block_of_page(kl.page(key0), bi, bj, bk);
                s_scene = (int)kl.scene(key0);
                s_org[0] = (int)(bi * L::sx);
                s_org[1] = (int)(bj * L::sy);
                s_org[2] = (int)(bk * L::sz);
            }
        }
        __syncthreads();
        const SceneParams<T>& sp = a.scenes[s_scene];
        const bool damage = sp.damage != 0;
        const Pool<T>& P = a.pin;
        const Pool<T>& Q = a.pout;
        const uint32_t i0 = start + threadIdx.x;
        uint32_t j_cur = i0 < end ? a.vals_sorted[i0] : 0u; // storage slot of the thread's current particle
        // asynchronous copy of one particle's state into buffer bf of the thread's slots
        auto stage = [&](int bf, uint32_t j) {
            T* d = s_st + bf * G2P_SF * NT + threadIdx.x;
            const T* src = P.f + j;
            const int64_t ps = P.stride;
#pragma unroll
            for (int c = 0; c < 3; c++) cp_async<sizeof(T)>(d + (GS_X + c) * NT, src + (P_X + c) * ps);
#pragma unroll
            for (int c = 0; c < 9; c++) cp_async<sizeof(T)>(d + (GS_F + c) * NT, src + (P_F + c) * ps);
            cp_async<sizeof(T)>(d + GS_M * NT, src + P_M * ps);
            cp_async<sizeof(T)>(d + GS_V0 * NT, src + P_V0 * ps);
            if (damage) {
                cp_async<sizeof(T)>(d + GS_D * NT, src + P_D * ps);
                cp_async<sizeof(T)>(d + GS_SC * NT, src + P_SC * ps);
            }
            cp_async<4>(s_pid + bf * NT + threadIdx.x, P.pid + j);
        };
        // stage the tile from the 8 neighbouring blocks (s_map was built before the first barrier)
        if constexpr (BULK) {
            if (threadIdx.x == 0) { // every thread is past the previous group's reads of s_halo (the barrier above)
                uint32_t nvalid = 0;
                for (int b = 0; b < 8; b++) nvalid += (s_nbr[b] >= 0 && (uint32_t)s_nbr[b] < a.b_cap) ? 1u : 0u;
                fence_async_smem();
                mbar_arrive_expect_tx(&s_hbar, nvalid * (uint32_t)(BLK * sizeof(T)));
                for (int b = 0; b < 8; b++) {
                    const int slot = s_nbr[b];
                    if (slot >= 0 && (uint32_t)slot < a.b_cap) bulk_load(s_halo + b * BLK, a.vel + (size_t)slot * BLK, (uint32_t)(BLK * sizeof(T)), &s_hbar);
                }
            }
            if (!mbar_wait(&s_hbar, hphase, WAIT_LIMIT_NS)) raise_flag(a.st, FLAG_TIMEOUT);
            hphase ^= 1u;
            for (int node = threadIdx.x; node < TN; node += NT) {
                const int m = s_map[node], slot = s_nbr[m >> 8];
                const bool ok = slot >= 0 && (uint32_t)slot < a.b_cap;
                const T* src = s_halo + (m >> 8) * BLK + (m & 0xff);
                Quad<T> qv;
                qv.x = ok ? src[0] : (T)0;
                qv.y = ok ? src[L::nodes] : (T)0;
                qv.z = ok ? src[2 * L::nodes] : (T)0;
                qv.w = ok ? src[3 * L::nodes] : (T)0;
                tq[node] = qv;
            }
        }
        else
            for (int node = threadIdx.x; node < TN; node += NT) {
                const int m = s_map[node], slot = s_nbr[m >> 8];
                const bool ok = slot >= 0 && (uint32_t)slot < a.b_cap;
                const T* src = a.vel + (size_t)(ok ? slot : 0) * NVEL * L::nodes + (m & 0xff);
                Quad<T> qv;
                qv.x = ok ? src[0] : (T)0;
                qv.y = ok ? src[L::nodes] : (T)0;
                qv.z = ok ? src[2 * L::nodes] : (T)0;
                qv.w = ok ? src[3 * L::nodes] : (T)0;
                tq[node] = qv;
            }
        {
            constexpr int MW = (int)(sizeof(Material<T>) / 4);
            const uint32_t* ms = reinterpret_cast<const uint32_t*>(sp.materials);
            uint32_t* md = reinterpret_cast<uint32_t*>(s_mat);
            for (int k = threadIdx.x; k < MAX_MATERIALS * MW; k += NT) md[k] = ms[k];
        }
        if (GS::ON && i0 < end) stage(0, j_cur);
        __syncthreads();
        const T dx = sp.dx, inv_dx = sp.inv_dx, dt = sp.dt, D_inv = sp.D_inv;
        const T ca = sp.apic_a, cb = sp.apic_b;
        const T dx2 = dx * dx, half_cfl2 = dx2 * (T)0.25 * (sp.cfl * sp.cfl);
        // scene constants in registers: read through sp inside the loop they would be re-read after every store
        const int key_cells = sp.domain_cells - 3, n_mat = sp.n_materials;
        const bool implicit = sp.implicit != 0;
        uint32_t flags = 0;
        // storage slots run one particle ahead of the state: with staging the next particle's state is copied
        // while this one computes; without, its slot is known when its loads issue (one latency, not two)
        uint32_t j_nxt = i0 + (GS::ON ? NT : 0) < end ? a.vals_sorted[i0 + (GS::ON ? NT : 0)] : 0u;
        int bf = 0;
        for (uint32_t i = i0; i < end; i += NT, bf ^= 1) {
            T x[3], F[9], pm, pV0, dd = 0, sc = 0;
            uint32_t pid, j;
            // staged: x now, the rest of the state from shared memory where it is used (it stays valid for the
            // whole iteration), so it holds no registers through the gather
            const T* dsl = s_st + bf * G2P_SF * NT + threadIdx.x;
            if constexpr (GS::ON) {
                j = j_cur;
                cp_async_wait_all(); // this particle's state (the thread's own copies)
#pragma unroll
                for (int c = 0; c < 3; c++) x[c] = dsl[(GS_X + c) * NT];
                if (i + NT < end) stage(bf ^ 1, j_nxt); // the other buffer was read in the previous iteration
                j_cur = j_nxt;
                if (i + 2 * NT < end) j_nxt = a.vals_sorted[i + 2 * NT];
            }
            else {
                j = j_nxt;
                if (i + NT < end) j_nxt = a.vals_sorted[i + NT];
                // every particle load is issued here, so one memory latency covers them all
#pragma unroll
                for (int c = 0; c < 3; c++) x[c] = P.f[(P_X + c) * P.stride + j];
#pragma unroll
                for (int c = 0; c < 9; c++) F[c] = P.f[(P_F + c) * P.stride + j];
                pid = P.pid[j];
                pm = P.f[P_M * P.stride + j];
                pV0 = P.f[P_V0 * P.stride + j];
                if (damage) {
                    dd = P.f[P_D * P.stride + j];
                    sc = P.f[P_SC * P.stride + j];
                }
            }
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
            T pv[3] = { 0, 0, 0 }, M[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 }, Gv[9] = { 0, 0, 0, 0, 0, 0, 0, 0, 0 }, lap = 0, pw = 0;
            const Quad<T>* nq0 = tq + (l[0] * TY + l[1]) * TZ + l[2];
            // the z and y sums run on pairs (two fields per instruction): velocity lanes (x, y) and (z, phase field)
            using PT = typename PairOf<T>::type;
            const PT Z = pmake<PT>((T)0, (T)0);
#pragma unroll
            for (int ii = 0; ii < 3; ii++) {
                // (S_x, S_y) (S_z, lA) (U_x, U_y) (U_z, lB) (T_x, T_y) (T_z, lC) (K_x, K_y) (K_z, -) (J_x, J_y) (J_z, -)
                PT S01 = Z, S2A = Z, U01 = Z, U2B = Z, T01 = Z, T2C = Z, K01 = Z, K2 = Z, J01 = Z, J2 = Z;
#pragma unroll
                for (int jj = 0; jj < 3; jj++) {
                    // (s_x, s_y) (s_z, pz) (t_x, t_y) (t_z, p1) (u_x, u_y) (u_z, -)
                    PT s01 = Z, s2z = Z, t01 = Z, t2p = Z, u01 = Z, u2 = Z;
#pragma unroll
                    for (int kk = 0; kk < 3; kk++) {
                        const Quad<T> nv = nq0[(ii * TY + jj) * TZ + kk];
                        const T wk = w[2][kk], dwk = dw[2][kk];
                        const PT v01 = pmake<PT>(nv.x, nv.y), v2f = pmake<PT>(nv.z, damage ? nv.w : (T)0);
                        const PT W = pmake<PT>(wk, wk);
                        s01 = pfma(W, v01, s01);
                        s2z = pfma(W, v2f, s2z);
                        t01 = pfma(pmake<PT>(dwk, dwk), v01, t01);
                        t2p = pfma(pmake<PT>(dwk, (T)1), v2f, t2p);
                        if (kk) {
                            const T kw = (T)kk * wk;
                            const PT KW = pmake<PT>(kw, kw);
                            u01 = pfma(KW, v01, u01);
                            u2 = pfma(KW, v2f, u2);
                        }
                    }
                    const T wj = w[1][jj], dwj = dw[1][jj];
                    const PT WJ = pmake<PT>(wj, wj);
                    S01 = pfma(WJ, s01, S01);
                    S2A = pfma(WJ, s2z, S2A);
                    U01 = pfma(pmake<PT>(dwj, dwj), s01, U01);
                    U2B = pfma(pmake<PT>(dwj, (T)1), s2z, U2B);
                    T01 = pfma(WJ, t01, T01);
                    T2C = pfma(WJ, t2p, T2C);
                    K01 = pfma(WJ, u01, K01);
                    K2 = pfma(WJ, u2, K2);
                    if (jj) {
                        const T jw = (T)jj * wj;
                        const PT JW = pmake<PT>(jw, jw);
                        J01 = pfma(JW, s01, J01);
                        J2 = pfma(JW, s2z, J2);
                    }
                }
                const T Si[3] = { S01.x, S01.y, S2A.x }, Ui[3] = { U01.x, U01.y, U2B.x }, Ti[3] = { T01.x, T01.y, T2C.x };
                const T Ki[3] = { K01.x, K01.y, K2.x }, Ji[3] = { J01.x, J01.y, J2.x };
                const T lA = S2A.y, lB = U2B.y, lC = T2C.y;
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
                if (damage) {
                    lap += (ii == 1 ? (T)-2 : (T)1) * (lA + wi * (lB + lC));
                    pw += wi * lA; // sum w times the node field (the damage change of an implicit solve)
                }
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
                if constexpr (GS::ON) {
#pragma unroll
                    for (int c = 0; c < 9; c++) F[c] = dsl[(GS_F + c) * NT];
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
                    in_dom = in_dom && nb[c] >= 0 && nb[c] < key_cells;
                }
                if (!in_dom) {
                    flags |= FLAG_OUT_OF_DOMAIN;
                    nb[0] = nb[1] = nb[2] = 0;
                }
                // the engine's keys carry no particle index (ib = 0), so a particle that stays in its cell gets
                // exactly the key it was sorted by (k_keys and this kernel share base_node): the incremental
                // sort's stayer test compares the two
                kl.put(a.keys_next, i, ((uint64_t)s_scene << (kl.cp + kl.ib)) | ((L::offset(nb[0], nb[1], nb[2]) >> L::data_bits) << kl.ib));
            }
            if constexpr (GS::ON) {
                pm = dsl[GS_M * NT];
                pV0 = dsl[GS_V0 * NT];
                pid = s_pid[bf * NT + threadIdx.x];
                if (damage) {
                    dd = dsl[GS_D * NT];
                    sc = dsl[GS_SC * NT];
                }
            }
            Q.f[P_M * Q.stride + i] = pm;
            Q.f[P_V0 * Q.stride + i] = pV0;
            Q.pid[i] = pid;
            if (implicit) Q.f[P_MDT * Q.stride + i] = P.f[P_MDT * P.stride + j]; // the implicit damage solve's history travels with the particle
            if (damage) {
                // AnisoMPM damage with the F of the start of the substep (AnisoFractureSimulation.h:210-283)
                const uint32_t mat = pid >> L::index_bits;
                const Material<T>& mt = s_mat[mat < (uint32_t)n_mat ? mat : 0];
                if (mt.damage && (mt.model == MODEL_NEOHOOKEAN_BORDEN || mt.model == MODEL_QR_STABLE_NEOHOOKEAN)) {
                    if (implicit) {
                        // damageG2P (AnisoFractureSimulation.h:578-610): the grid holds the solve's change of the
                        // nodal phase field; damage never decreases and stays <= 1
                        const T nd = dd + pw;
                        dd = nd > dd ? nd : dd;
                        dd = dd < (T)1 ? dd : (T)1;
                        // the next substep's solve folds the drive of the new F into the history: computed here,
                        // where the explicit update would evaluate the drive of the old F
                        T Fn[9];
#pragma unroll
                        for (int c = 0; c < 9; c++) Fn[c] = Q.f[(P_F + c) * Q.stride + i];
                        bool fb = false;
                        Q.f[P_DRV * Q.stride + i] = damage_drive(mt, Fn, sc, fb);
                        if (fb) atomicAdd(&a.st->fallback, 1u);
                    }
                    else {
                        bool fb = false;
                        dd = damage_update(mt, F, dd, lap, sc, dt, fb);
                        if (fb) atomicAdd(&a.st->fallback, 1u);
                    }
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

// ---------------------------------------------------------------------------------------------------
// Implicit damage solve (AnisoFractureSimulation::solveDamageSystem, AnisoFractureSimulation.h:437-626), run
// between the grid update and G2P for scenes that ask for it. Unknowns: the nodal phase field x on the nodes
// that damageable particles reach. With per-particle vol = V0 det F, the damage drive history
// D~ = max(D~, zeta <phi - 1>) (updateDTilde, :285-340), c_p = vol (1 + dt/eta (D~ + 1)) and
// e_p = vol dt/eta l0^2:
//   rhs_i = sum_p (dt D~/eta + pf_i) vol w_ip          (pf: the normalised nodal damage of this substep)
//   (A x)_i = diag_i x_i + sum_p (e_p sum_j x_j grad w_jp) . grad w_ip,   diag_i = sum_p c_p w_ip
// solved by Jacobi-preconditioned conjugate gradients from x = 0 as ConjugateGradient::solve does (stop when
// sqrt(r.z) <= min(sqrt(r0.z0), 1e-6), at most 100 iterations). Dot products are per scene, so every scene of a
// batch runs the iterations it would run alone. G2P then adds sum_i w_ip (x_i - pf_i) to the damage.
// ---------------------------------------------------------------------------------------------------
enum { CG_SA = 0, CG_SV, CG_DIAG, CG_X, CG_R, CG_Z, CG_P, CG_AP, CG_NF }; // node vectors
enum { DS_F = 0, DS_A = 3, DS_VOL = 4, DS_C = 5, DS_E = 6 }; // particle scratch fields in the payload buffer
constexpr int CG_MAX_ITERATIONS = 100;

template <class T>
__device__ __forceinline__ T* cgv(const StepArgs<T>& a, int f, uint32_t slot) { return a.cg + ((size_t)f * a.b_cap + slot) * LayoutOf<T>::type::nodes; }

// The damage drive of every particle of the implicit scenes from its current F, in storage order (the scene from
// the particle's current key): fills the cache P_DRV after a state write made it stale; G2P keeps it afterwards.
template <class T>
__global__ void k_dmg_drive(StepArgs<T> a, const uint64_t* keys)
{
    using L = typename LayoutOf<T>::type;
    const Pool<T>& P = a.pin;
    uint32_t fallbacks = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n_total; i += gridDim.x * blockDim.x) {
        const SceneParams<T>& sp = a.scenes[a.kl.scene(a.kl.at(keys, i))];
        if (!sp.implicit) continue;
        const uint32_t mat = P.pid[i] >> L::index_bits;
        const Material<T>& mt = sp.materials[mat < (uint32_t)sp.n_materials ? mat : 0];
        T drive = 0;
        if (mt.damage && (mt.model == MODEL_NEOHOOKEAN_BORDEN || mt.model == MODEL_QR_STABLE_NEOHOOKEAN)) {
            T F[9];
#pragma unroll
            for (int e = 0; e < 9; e++) F[e] = P.f[(P_F + e) * P.stride + i];
            bool fb = false;
            drive = damage_drive(mt, F, P.f[P_SC * P.stride + i], fb);
            if (fb) fallbacks++;
        }
        P.f[P_DRV * P.stride + i] = drive;
    }
    if (fallbacks) atomicAdd(&a.st->fallback, fallbacks);
}

// Per sorted particle of an implicit scene (one thread each, no barriers): the D~ history folded with the drive
// of the particle's F (cached in P_DRV), and into the particle scratch the fractional position, vol D~ dt/eta,
// vol, c_p and e_p.
template <class T>
__global__ void k_dmg_prep(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    if (aborted(a.st)) return;
    const KeyLayout kl = a.kl;
    const int64_t S = a.pstride;
    const Pool<T>& P = a.pin;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < a.n_total; q += gridDim.x * blockDim.x) {
        const SceneParams<T>& sp = a.scenes[kl.scene(kl.at(a.keys_sorted, q))];
        const uint32_t j = a.vals_sorted[q];
        // every state load of the particle at once (one latency), ahead of the scene and material tests
        T x[3], F[9];
#pragma unroll
        for (int e = 0; e < 3; e++) x[e] = P.f[(P_X + e) * P.stride + j];
#pragma unroll
        for (int e = 0; e < 9; e++) F[e] = P.f[(P_F + e) * P.stride + j];
        const T V0 = P.f[P_V0 * P.stride + j], drive = P.f[P_DRV * P.stride + j];
        T hist = P.f[P_MDT * P.stride + j];
        const uint32_t pid = P.pid[j];
        if (!sp.implicit) continue;
        T* y = a.pay + pay_pos(q);
#pragma unroll
        for (int e = 0; e < 3; e++) {
            const T xs = mul_rn(x[e], sp.inv_dx);
            y[(DS_F + e) * S] = xs - (T)int_floor(sub_rn(xs, (T)0.5));
        }
        const uint32_t mat = pid >> L::index_bits;
        const Material<T>& mt = sp.materials[mat < (uint32_t)sp.n_materials ? mat : 0];
        T av = 0, vol = 0, c = 0, ev = 0;
        if (mt.damage && (mt.model == MODEL_NEOHOOKEAN_BORDEN || mt.model == MODEL_QR_STABLE_NEOHOOKEAN)) {
            vol = V0 * det3(F);
            hist = drive > hist ? drive : hist;
            P.f[P_MDT * P.stride + j] = hist;
            const T dt = sp.dt;
            av = ((dt * hist) / mt.eta) * vol;
            c = vol * ((T)1 + ((dt / mt.eta) * (hist + (T)1)));
            ev = vol * (dt / mt.eta) * mt.l0 * mt.l0;
        }
        y[DS_A * S] = av;
        y[DS_VOL * S] = vol;
        y[DS_C * S] = c;
        y[DS_E * S] = ev;
    }
}

// node tile of a group (its block plus 2 nodes on the + side): index of node (lx, ly, lz)
template <class L>
__device__ __forceinline__ int tile_index(int lx, int ly, int lz) { return (lx * (L::sy + 2) + ly) * (L::sz + 2) + lz; }

// The per-offset tiles of the fused P2G (OffsetTiles) for NF node vectors of the implicit solve: get(n, f) is
// field f of the thread's node n = 3 jj + kk. Every lane of the warp must call it.
template <class L, int NF, class T, class Get>
__device__ __forceinline__ void add_to_offset_tile_cg(T* tiles, int cx, int cy, int cz, int ii, Get get)
{
    using OT = OffsetTiles<L>;
    T* base = tiles + ii * NF * OT::TS + (cx * OT::TY + cy) * OT::TZ + cz;
#pragma unroll
    for (int jj = 0; jj < 3; jj++)
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            T* t = base + jj * OT::TZ + kk;
#pragma unroll
            for (int f = 0; f < NF; f++) t[f * OT::TS] += get(jj * 3 + kk, f);
            __syncwarp();
        }
}

// sum the offsets' tiles per node of the block + halo into node vectors f_of[f] of the 8 neighbouring blocks
// (scalar atomics, zeros skipped), clearing the tiles
template <class T, class L, int NF>
__device__ void flush_offset_tiles_cg(const StepArgs<T>& a, T* tiles, const int32_t* nbr, const int* f_of, int tid, int nthreads)
{
    using OT = OffsetTiles<L>;
    constexpr int TX = L::sx + 2, TY = OT::TY, TZ = OT::TZ, TN = TX * TY * TZ;
    for (int q = tid; q < NF * TN; q += nthreads) {
        const int f = q / TN, node = q % TN;
        const int tx = node / (TY * TZ), ty = (node / TZ) % TY, tz = node % TZ;
        T v = (T)0;
#pragma unroll
        for (int ii = 0; ii < 3; ii++) {
            const int xl = tx - ii;
            if (xl < 0 || xl >= L::sx) continue;
            T* src = tiles + (ii * NF + f) * OT::TS + (xl * TY + ty) * TZ + tz;
            v += *src;
            *src = (T)0;
        }
        if (v == (T)0) continue;
        const int ax = tx >= L::sx, ay = ty >= L::sy, az = tz >= L::sz;
        const int slot = nbr[ax * 4 + ay * 2 + az];
        if (slot < 0 || (uint32_t)slot >= a.b_cap) {
            check_failed(a.st, 7);
            continue;
        }
        atomicAdd(cgv(a, f_of[f], slot) + L::element(tx - ax * L::sx, ty - ay * L::sy, tz - az * L::sz), v);
    }
}

// Claim the next group of an implicit scene for a damage-solve kernel (thread 0 claims, all threads get the same
// answer): the group's particle range and neighbour blocks. Returns the scene, or -1 when the groups are exhausted.
template <class T>
__device__ int dmg_claim(const StepArgs<T>& a, uint32_t* counter, bool need_unfinished, uint32_t& start, uint32_t& end, int32_t* s_nbr, int* s_g,
    int* s_skip)
{
    const KeyLayout kl = a.kl;
    const uint32_t G = a.st->n_groups;
    for (;;) {
        if (threadIdx.x == 0) *s_g = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int g = *s_g;
        if (g >= (int)G) return -1;
        start = a.g_start[g];
        end = (g + 1 < (int)G) ? a.g_start[g + 1] : a.n_total;
        const uint32_t sc = kl.scene(kl.at(a.keys_sorted, start));
        if (threadIdx.x == 0) *s_skip = !a.scenes[sc].implicit || (need_unfinished && a.cgs[sc].done);
        if (threadIdx.x < 8) s_nbr[threadIdx.x] = a.g_nbr[g * 8 + threadIdx.x];
        __syncthreads();
        if (!*s_skip) return (int)sc;
        __syncthreads(); // every thread has read *s_skip before thread 0 claims again
    }
}

// threads and particle chunk of the damage solve's group kernels: one thread per (in-block cell, stencil x-offset);
// a chunk's per-particle values are staged in shared memory for the per-cell sums
template <class T>
struct DmgShape {
    using L = typename LayoutOf<T>::type;
    static constexpr int NT = 3 * L::nodes;
    static constexpr int CHUNK = 512;
    static constexpr int NS = 6; // staged values per particle
    static constexpr int MINB = 4; // CTAs per SM the registers are cut for: these kernels wait on memory
};

// cell ranges of a staged chunk: particles of one cell are contiguous (sorted by cell inside the block)
template <int NC>
__device__ __forceinline__ void chunk_cells(const uint8_t* cellof, int cnt, int16_t* cfirst, int16_t* clast, int tid, int nt)
{
    for (int q = tid; q < cnt; q += nt) {
        const int e = cellof[q];
        if (q == 0 || cellof[q - 1] != e) cfirst[e] = (int16_t)q;
        if (q == cnt - 1 || cellof[q + 1] != e) clast[e] = (int16_t)(q + 1);
    }
}

// Right-hand side parts and the preconditioner's diagonal. Per chunk: the particles' scratch values staged in
// shared memory (phase 1), then one thread per (in-block cell, x-offset) sums the 9 (y, z) nodes over its cell's
// particles in registers (phase 2) and adds them to the group's shared node tile; the tile goes to the node
// vectors CG_SA, CG_SV, CG_DIAG.
template <class T>
__global__ void __launch_bounds__(DmgShape<T>::NT, DmgShape<T>::MINB) k_dmg_rhs(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using D = DmgShape<T>;
    constexpr int NC = L::nodes, NT = D::NT, CHUNK = D::CHUNK, TY = L::sy + 2, TZ = L::sz + 2, TN = (L::sx + 2) * TY * TZ;
    constexpr int TE = 3 * 3 * OffsetTiles<L>::TS; // per-offset tiles of the 3 node vectors
    __shared__ T tile[TE];
    __shared__ T st[D::NS][CHUNK]; // fr x3, vol D~ dt/eta, vol, c
    __shared__ uint8_t cellof[CHUNK];
    __shared__ int16_t cfirst[NC], clast[NC];
    __shared__ int s_g, s_skip;
    __shared__ int32_t s_nbr[8];
    if (aborted_cta(a.st)) return;
    const KeyLayout kl = a.kl;
    const int64_t S = a.pstride;
    const int tid = threadIdx.x, ii = tid / NC, c = tid % NC;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    for (int q = tid; q < TE; q += NT) tile[q] = (T)0;
    const int f_of[3] = { CG_SA, CG_SV, CG_DIAG };
    for (;;) {
        uint32_t start, end;
        const int sc = dmg_claim<T>(a, &a.st->work_dmg, false, start, end, s_nbr, &s_g, &s_skip);
        if (sc < 0) break;
        bool any = false;
        for (uint32_t c0 = start; c0 < end; c0 += CHUNK) {
            const int cnt = (int)min((uint32_t)CHUNK, end - c0);
            if (tid < NC) {
                cfirst[tid] = 0;
                clast[tid] = 0;
            }
            for (int q = tid; q < cnt; q += NT) {
                const T* y = a.pay + pay_pos(c0 + q);
#pragma unroll
                for (int f = 0; f < D::NS; f++) st[f][q] = y[(DS_F + f) * S];
                cellof[q] = (uint8_t)((kl.at(a.keys_sorted, c0 + q) >> kl.ib) & (NC - 1));
            }
            __syncthreads();
            chunk_cells<NC>(cellof, cnt, cfirst, clast, tid, NT);
            __syncthreads();
            T acc[9][3];
#pragma unroll
            for (int n = 0; n < 9; n++) acc[n][0] = acc[n][1] = acc[n][2] = (T)0;
            const int qa = cfirst[c], qb = clast[c];
            for (int q = qa; q < qb; q++) {
                const T cc = st[5][q];
                if (cc == (T)0) continue; // not damageable
                const T av = st[3][q], vol = st[4][q];
                T w[3][3], dw[3][3];
#pragma unroll
                for (int e = 0; e < 3; e++) bspline_w(st[e][q], 0, w[e], dw[e]);
                const T wx = w[0][ii];
#pragma unroll
                for (int j = 0; j < 3; j++)
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const T wijk = wx * w[1][j] * w[2][k];
                        acc[j * 3 + k][0] += wijk * av;
                        acc[j * 3 + k][1] += wijk * vol;
                        acc[j * 3 + k][2] += wijk * cc;
                    }
            }
            add_to_offset_tile_cg<L, 3>(tile, cx, cy, cz, ii, [&](int n, int f) { return acc[n][f]; }); // all lanes
            any = true;
            __syncthreads();
        }
        if (any) flush_offset_tiles_cg<T, L, 3>(a, tile, s_nbr, f_of, tid, NT);
        __syncthreads();
    }
}

// The operator's particle part for the search direction p. Per chunk: per particle gc = e_p / dx^2 sum_j p_j
// grad w_jp (gradients per unit cell; phase 1, from p staged on the group's tile), staged with the fractional
// position; then per (cell, x-offset) thread the sums gc . grad w over its cell's particles for its 9 nodes
// (phase 2) into the tile, which goes to A p (CG_AP).
template <class T>
__global__ void __launch_bounds__(DmgShape<T>::NT, DmgShape<T>::MINB) k_dmg_apply(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    using D = DmgShape<T>;
    constexpr int NC = L::nodes, NT = D::NT, CHUNK = D::CHUNK, TY = L::sy + 2, TZ = L::sz + 2, TN = (L::sx + 2) * TY * TZ;
    constexpr int TE = 3 * OffsetTiles<L>::TS; // per-offset tiles of A p
    __shared__ T tile[TE];
    __shared__ T ptile[TN];
    __shared__ T st[D::NS][CHUNK]; // fr x3, gc x3
    __shared__ uint8_t cellof[CHUNK];
    __shared__ int16_t cfirst[NC], clast[NC];
    __shared__ int s_g, s_skip;
    __shared__ int32_t s_nbr[8];
    __shared__ uint16_t s_map[TN]; // tile node -> (neighbour block 0-7) << 8 | element in that block
    if (aborted_cta(a.st)) return;
    const KeyLayout kl = a.kl;
    const int64_t S = a.pstride;
    const int tid = threadIdx.x, ii = tid / NC, c = tid % NC;
    const int cx = c >> (L::zbits + L::ybits), cy = (c >> L::zbits) & (L::sy - 1), cz = c & (L::sz - 1);
    for (int q = tid; q < TE; q += NT) tile[q] = (T)0;
    for (int q = tid; q < TN; q += NT) {
        const int tx = q / (TY * TZ), ty = (q / TZ) % TY, tz = q % TZ;
        const int ax = tx >= L::sx, ay = ty >= L::sy, az = tz >= L::sz;
        s_map[q] = (uint16_t)(((ax * 4 + ay * 2 + az) << 8) | L::element(tx - ax * L::sx, ty - ay * L::sy, tz - az * L::sz));
    }
    const int f_of[1] = { CG_AP };
    for (;;) {
        uint32_t start, end;
        const int sc = dmg_claim<T>(a, &a.st->work_cg, true, start, end, s_nbr, &s_g, &s_skip);
        if (sc < 0) break;
        for (int q = tid; q < TN; q += NT) { // (s_map was built before the claim's first barrier)
            const int m = s_map[q], slot = s_nbr[m >> 8];
            ptile[q] = (slot >= 0 && (uint32_t)slot < a.b_cap) ? cgv(a, CG_P, slot)[m & 0xff] : (T)0;
        }
        __syncthreads();
        const T inv_dx = a.scenes[sc].inv_dx;
        for (uint32_t c0 = start; c0 < end; c0 += CHUNK) {
            const int cnt = (int)min((uint32_t)CHUNK, end - c0);
            if (tid < NC) {
                cfirst[tid] = 0;
                clast[tid] = 0;
            }
            for (int q = tid; q < cnt; q += NT) {
                const T* y = a.pay + pay_pos(c0 + q);
                const T ev = y[DS_E * S];
                const int e = (int)((kl.at(a.keys_sorted, c0 + q) >> kl.ib) & (NC - 1));
                cellof[q] = (uint8_t)e;
                T fr[3], w[3][3], dw[3][3];
#pragma unroll
                for (int f = 0; f < 3; f++) {
                    fr[f] = y[(DS_F + f) * S];
                    st[f][q] = fr[f];
                    bspline_w(fr[f], 0, w[f], dw[f]);
                }
                T g0 = 0, g1 = 0, g2 = 0;
                if (ev != (T)0) {
                    const int lx = e >> (L::zbits + L::ybits), ly = (e >> L::zbits) & (L::sy - 1), lz = e & (L::sz - 1);
                    const T* pt = ptile + tile_index<L>(lx, ly, lz);
                    // separable sums of p against the gradient weights: over z, then y, then x
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        T sA = 0, sB = 0, sC = 0;
#pragma unroll
                        for (int j = 0; j < 3; j++) {
                            T zA = 0, zD = 0;
#pragma unroll
                            for (int k = 0; k < 3; k++) {
                                const T pj = pt[(i * TY + j) * TZ + k];
                                zA += w[2][k] * pj;
                                zD += dw[2][k] * pj;
                            }
                            sA += w[1][j] * zA;
                            sB += dw[1][j] * zA;
                            sC += w[1][j] * zD;
                        }
                        g0 += dw[0][i] * sA;
                        g1 += w[0][i] * sB;
                        g2 += w[0][i] * sC;
                    }
                    const T sgc = ev * inv_dx * inv_dx; // both gradients carry 1/dx
                    g0 *= sgc;
                    g1 *= sgc;
                    g2 *= sgc;
                }
                st[3][q] = g0;
                st[4][q] = g1;
                st[5][q] = g2;
            }
            __syncthreads();
            chunk_cells<NC>(cellof, cnt, cfirst, clast, tid, NT);
            __syncthreads();
            T acc[9];
#pragma unroll
            for (int n = 0; n < 9; n++) acc[n] = (T)0;
            const int qa = cfirst[c], qb = clast[c];
            for (int q = qa; q < qb; q++) {
                const T g0 = st[3][q], g1 = st[4][q], g2 = st[5][q];
                if (g0 == (T)0 && g1 == (T)0 && g2 == (T)0) continue;
                T w[3][3], dw[3][3];
#pragma unroll
                for (int e = 0; e < 3; e++) bspline_w(st[e][q], 0, w[e], dw[e]);
                const T a0 = g0 * dw[0][ii], a1 = g1 * w[0][ii], a2 = g2 * w[0][ii];
#pragma unroll
                for (int j = 0; j < 3; j++)
#pragma unroll
                    for (int k = 0; k < 3; k++) acc[j * 3 + k] += (a0 * w[1][j] + a1 * dw[1][j]) * w[2][k] + a2 * (w[1][j] * dw[2][k]);
            }
            add_to_offset_tile_cg<L, 1>(tile, cx, cy, cz, ii, [&](int n, int) { return acc[n]; }); // all lanes
            __syncthreads();
        }
        flush_offset_tiles_cg<T, L, 1>(a, tile, s_nbr, f_of, tid, NT);
        __syncthreads();
    }
}

// per scene of a node, with the warp's nodes all of one block (and so of one scene)
template <class T>
__device__ __forceinline__ void scene_sum(double v, int scene, double* dst)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int s0 = __shfl_sync(0xffffffffu, scene, 0);
    if ((threadIdx.x & 31) == 0 && s0 >= 0 && v != 0.0) atomicAdd(dst + (size_t)s0 * (sizeof(CgScalars) / sizeof(double)), v);
}

// node kernels: STAGE 0 init (r = rhs, z = r/diag, p = z, r.z), 1 A p += diag p and p.Ap, 2 x, r, z update
// and r.z, 3 p = z + beta p and A p = 0, 4 finish (the grid's phase field becomes x - pf)
template <class T, int STAGE>
__global__ void k_cg_nodes(StepArgs<T> a)
{
    using L = typename LayoutOf<T>::type;
    if (aborted(a.st)) return;
    const uint32_t B = min(a.st->n_blocks, a.b_cap);
    const uint32_t total = B * L::nodes;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ((total + 31) & ~31u); t += gridDim.x * blockDim.x) {
        double acc = 0;
        int scene = -1;
        if (t < total) {
            const uint32_t b = t / L::nodes, e = t % L::nodes;
            const int sc = (int)(a.b_key[b] >> 40);
            const SceneParams<T>& sp = a.scenes[sc];
            CgScalars& cs = a.cgs[sc];
            if (sp.implicit && (STAGE == 0 || STAGE == 4 || !cs.done)) {
                scene = sc;
                T* dg = cgv(a, CG_DIAG, b) + e;
                const T diag = *dg;
                T* x = cgv(a, CG_X, b) + e;
                T* r = cgv(a, CG_R, b) + e;
                T* z = cgv(a, CG_Z, b) + e;
                T* p = cgv(a, CG_P, b) + e;
                T* Ap = cgv(a, CG_AP, b) + e;
                T* pf = a.vel + (size_t)b * NVEL * L::nodes + 3 * L::nodes + e;
                const bool on = diag > (T)0;
                if (STAGE == 0) {
                    const T rhs = on ? cgv(a, CG_SA, b)[e] + *pf * cgv(a, CG_SV, b)[e] : (T)0;
                    const T zz = on ? rhs / diag : (T)0;
                    *x = 0;
                    *r = rhs;
                    *z = zz;
                    *p = zz;
                    *Ap = 0;
                    acc = (double)rhs * (double)zz;
                }
                else if (STAGE == 1) {
                    const T ap = on ? *Ap + diag * *p : (T)0;
                    *Ap = ap;
                    acc = (double)ap * (double)*p;
                }
                else if (STAGE == 2) {
                    const T alpha = (T)(cs.zr / cs.pAp);
                    const T xn = *x + *p * alpha, rn = *r - *Ap * alpha, zn = on ? rn / diag : (T)0;
                    *x = xn;
                    *r = rn;
                    *z = zn;
                    acc = (double)zn * (double)rn;
                }
                else if (STAGE == 3) {
                    const T beta = (T)(cs.zr_new / cs.zr);
                    *p = *z + beta * *p;
                    *Ap = 0;
                }
                else {
                    *pf = on ? *x - *pf : (T)0;
                    // the solve's vectors start from zero next time
                    cgv(a, CG_SA, b)[e] = 0;
                    cgv(a, CG_SV, b)[e] = 0;
                    *dg = 0;
                    *Ap = 0;
                }
            }
        }
        if (STAGE == 0 || STAGE == 2) scene_sum<T>(acc, scene, STAGE == 0 ? &a.cgs[0].zr : &a.cgs[0].zr_new);
        if (STAGE == 1) scene_sum<T>(acc, scene, &a.cgs[0].pAp);
    }
}

// per-scene CG bookkeeping (one block): STAGE 0 after init, 1 after an iteration. STAGE 1 runs as the last
// kernel of the loop body and sets the loop's condition: some scene unfinished, and never more than
// CG_MAX_ITERATIONS + 1 passes (each scene stops itself at CG_MAX_ITERATIONS, so the loop always ends).
template <class T, int STAGE>
__global__ void k_cg_scalars(StepArgs<T> a, int n_scenes, cudaGraphConditionalHandle loop)
{
    __shared__ uint32_t s_active;
    if (threadIdx.x == 0) s_active = 0;
    __syncthreads();
    const bool ab = aborted(a.st);
    for (int s = threadIdx.x; s < n_scenes; s += blockDim.x) {
        CgScalars& cs = a.cgs[s];
        if (!a.scenes[s].implicit) {
            cs.done = 1;
            continue;
        }
        if (STAGE == 0) {
            const double res = sqrt(cs.zr);
            cs.tol = res < 1e-6 ? res : 1e-6;
            cs.iter = 0;
            cs.done = res <= cs.tol;
        }
        else if (!cs.done) {
            cs.zr = cs.zr_new;
            cs.iter++;
            cs.done = sqrt(cs.zr) <= cs.tol || cs.iter >= CG_MAX_ITERATIONS;
        }
        cs.pAp = 0;
        cs.zr_new = 0;
        if (ab) cs.done = 1;
        if (!cs.done) atomicAdd(&s_active, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a.st->work_cg = 0;
        if (STAGE == 0)
            a.st->cg_loops = 0;
        else {
            const uint32_t loops = ++a.st->cg_loops;
            cudaGraphSetConditional(loop, (s_active > 0 && loops <= (uint32_t)CG_MAX_ITERATIONS) ? 1u : 0u);
        }
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
        st->work_dmg = 0;
    }
}

// ---------------------------------------------------------------------------------------------------
// host <-> device field transfer (caller order <-> storage order via the original index)
// ---------------------------------------------------------------------------------------------------
// Storage slot of every particle of a scene in the caller's order (inv[orig] = slot), for the row transfers.
template <class T>
__global__ void k_inv(Pool<T> p, int64_t first, int64_t n, uint32_t* inv)
{
    using L = typename LayoutOf<T>::type;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t orig = p.pid[first + i] & ((1u << L::index_bits) - 1);
        if (orig < (uint64_t)n) inv[orig] = (uint32_t)(first + i);
    }
}

// Field groups of a row transfer: rows of W = sum nc values in the caller's order, fields f0[k] .. f0[k]+nc[k]-1.
struct RowFields {
    int f0[8], nc[8], count, W;
};
constexpr int IO_ROWS = 128; // rows per CTA (one per thread)

// Rows of a scene between the particle pool and row-major buffers (host memory mapped into the device, or a
// staging buffer). A CTA moves IO_ROWS consecutive rows: pool <-> shared memory per row (thread per row, slot from
// inv), shared memory <-> buffer as one contiguous run of IO_ROWS * W values (coalesced, whole lines over the
// host link). MODE: ROWS_IMPORT (in -> pool), ROWS_EXPORT (pool -> out), ROWS_EXCHANGE (pool -> out, then in ->
// pool, row by row: a CTA reads its rows out of the pool before it overwrites them, and CTAs own disjoint rows,
// so out receives the state from before the call; with many CTAs in flight both directions of the link are busy
// at once).
enum { ROWS_IMPORT = 0, ROWS_EXPORT = 1, ROWS_EXCHANGE = 2 };
template <class T, class O, int MODE>
__global__ void __launch_bounds__(IO_ROWS) k_rows(Pool<T> p, const uint32_t* inv, int64_t n, RowFields rf, const O* in, O* out)
{
    extern __shared__ __align__(16) unsigned char rows_dyn[];
    const int W = rf.W;
    O* sm_o = reinterpret_cast<O*>(rows_dyn); // rows leaving the pool
    O* sm_i = MODE == ROWS_EXCHANGE ? sm_o + IO_ROWS * W : sm_o; // rows entering it
    for (int64_t base = (int64_t)blockIdx.x * IO_ROWS; base < n; base += (int64_t)gridDim.x * IO_ROWS) {
        const int rows = (int)min((int64_t)IO_ROWS, n - base);
        const uint32_t slot = threadIdx.x < rows ? inv[base + threadIdx.x] : 0u;
        if (MODE != ROWS_IMPORT) {
            if (threadIdx.x < rows) {
                O* r = sm_o + threadIdx.x * W;
                int c0 = 0;
                for (int k = 0; k < rf.count; k++) {
                    for (int c = 0; c < rf.nc[k]; c++) r[c0 + c] = (O)p.f[(int64_t)(rf.f0[k] + c) * p.stride + slot];
                    c0 += rf.nc[k];
                }
            }
            __syncthreads();
        }
        {
            O* run_o = MODE != ROWS_IMPORT ? out + base * W : nullptr;
            const O* run_i = MODE != ROWS_EXPORT ? in + base * W : nullptr;
            for (int q = threadIdx.x; q < rows * W; q += IO_ROWS) {
                if (MODE != ROWS_IMPORT) run_o[q] = sm_o[q];
                if (MODE != ROWS_EXPORT) sm_i[q] = run_i[q];
            }
            __syncthreads();
        }
        if (MODE != ROWS_EXPORT) {
            if (threadIdx.x < rows) {
                const O* r = sm_i + threadIdx.x * W;
                int c0 = 0;
                for (int k = 0; k < rf.count; k++) {
                    for (int c = 0; c < rf.nc[k]; c++) p.f[(int64_t)(rf.f0[k] + c) * p.stride + slot] = (T)r[c0 + c];
                    c0 += rf.nc[k];
                }
            }
            __syncthreads();
        }
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
