// Shared definitions of the GB300 explicit-MPM engine: SPGrid layout arithmetic, per-scene parameter
// blocks, status flags. Includable from CUDA and plain C++ translation units.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define ZR_HD __host__ __device__ __forceinline__
#define ZR_D __device__ __forceinline__
#define ZR_COLD __host__ __device__ __noinline__
#else
#define ZR_HD inline
#define ZR_D inline
#define ZR_COLD inline
#endif

namespace zr {

// -------------------------------------------------------------------------------------------------
// SPGrid layout. Ziran stores grid nodes in SPGrid pages of 4 KiB holding 2^block_bits GridState
// records of 2^LOG2 bytes (64 B for float, 128 B for double: Lib/MPM/MpmGrid.h:16-45), so a block is
// 4x4x4 nodes for float and 2x4x4 (x,y,z) for double. A node's byte offset interleaves its
// coordinates: inside the page z is the fastest field, then y, then x; above bit 12 the remaining
// coordinate bits alternate one bit per axis (Lib/SPGrid/Core/SPGrid_Mask.h:22-48,76-123,150-166).
// Keys, groups and the 8-colour parity all derive from these offsets, so they are reproduced here
// bit for bit; the arithmetic is a Morton spread rather than SPGrid's bit-by-bit deposit.
// -------------------------------------------------------------------------------------------------
template <int LOG2>
struct SpLayout {
    static constexpr int data_bits = LOG2;
    static constexpr int block_bits = 12 - LOG2;
    static constexpr int zbits = block_bits / 3 + (block_bits % 3 > 0);
    static constexpr int ybits = block_bits / 3 + (block_bits % 3 > 1);
    static constexpr int xbits = block_bits / 3;
    static constexpr int sx = 1 << xbits, sy = 1 << ybits, sz = 1 << zbits;
    static constexpr int nodes = 1 << block_bits;
    static constexpr int index_bits = 32 - block_bits; // MpmSimulationBase.cpp:1535
    // element bit positions of each axis inside the page
    static constexpr int ez = data_bits, ey = data_bits + zbits, ex = data_bits + zbits + ybits;
    // lowest page-level bit of each axis: page masks are every third bit from bit 12, rotated by
    // 3 - block_bits % 3 (SPGrid_Mask.h:36-39)
    static constexpr int shift = 3 - block_bits % 3;
    static constexpr int pz = 12 + (shift + 0) % 3;
    static constexpr int py = 12 + (shift + 1) % 3;
    static constexpr int px = 12 + (shift + 2) % 3;

    // bit t of v -> bit 3t (v < 2^21)
    ZR_HD static uint64_t spread3(uint64_t v)
    {
        v &= 0x1fffffULL;
        v = (v | v << 32) & 0x1f00000000ffffULL;
        v = (v | v << 16) & 0x1f0000ff0000ffULL;
        v = (v | v << 8) & 0x100f00f00f00f00fULL;
        v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
        v = (v | v << 2) & 0x1249249249249249ULL;
        return v;
    }
    // inverse of spread3
    ZR_HD static uint32_t compact3(uint64_t v)
    {
        v &= 0x1249249249249249ULL;
        v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ULL;
        v = (v ^ (v >> 4)) & 0x100f00f00f00f00fULL;
        v = (v ^ (v >> 8)) & 0x1f0000ff0000ffULL;
        v = (v ^ (v >> 16)) & 0x1f00000000ffffULL;
        v = (v ^ (v >> 32)) & 0x1fffffULL;
        return (uint32_t)v;
    }
    // Linear_Offset of a node with non-negative coordinates
    ZR_HD static uint64_t offset(uint32_t i, uint32_t j, uint32_t k)
    {
        uint64_t e = ((uint64_t)(i & (sx - 1)) << ex) | ((uint64_t)(j & (sy - 1)) << ey) | ((uint64_t)(k & (sz - 1)) << ez);
        return e | (spread3(i >> xbits) << px) | (spread3(j >> ybits) << py) | (spread3(k >> zbits) << pz);
    }
    // page index (offset >> 12) of the block with block coordinates (bi,bj,bk)
    ZR_HD static uint64_t page_of_block(uint32_t bi, uint32_t bj, uint32_t bk)
    {
        return (spread3(bi) << (px - 12)) | (spread3(bj) << (py - 12)) | (spread3(bk) << (pz - 12));
    }
    ZR_HD static void block_of_page(uint64_t page, uint32_t& bi, uint32_t& bj, uint32_t& bk)
    {
        bi = compact3(page >> (px - 12));
        bj = compact3(page >> (py - 12));
        bk = compact3(page >> (pz - 12));
    }
    // node index inside a block, identical to the element bits of the offset (z fastest)
    ZR_HD static int element(int lx, int ly, int lz) { return (lx << (zbits + ybits)) | (ly << zbits) | lz; }
    // MpmSimulationBase.cpp:1547-1549: key = ((offset >> data_bits) << index_bits) + i
    ZR_HD static uint64_t key(uint32_t i, uint32_t j, uint32_t k, uint32_t id)
    {
        return ((offset(i, j, k) >> data_bits) << index_bits) | (uint64_t)id;
    }
};

template <class T>
struct LayoutOf;
template <>
struct LayoutOf<float> {
    using type = SpLayout<6>;
};
template <>
struct LayoutOf<double> {
    using type = SpLayout<7>;
};

// -------------------------------------------------------------------------------------------------
// status word (device), read by the host after a batch of substeps
// -------------------------------------------------------------------------------------------------
enum : uint32_t {
    FLAG_CFL = 1u << 0, // a particle moved more than dx in one substep (the reference's restart trigger)
    FLAG_CFL_HALF = 1u << 1, // a particle moved more than cfl*dx/2 (informational)
    FLAG_NONFINITE = 1u << 2, // NaN/Inf in the particle state
    FLAG_OUT_OF_DOMAIN = 1u << 3, // a base node left the scene's domain
    FLAG_CAPACITY = 1u << 4, // active-block table or grid storage full
    FLAG_TIMEOUT = 1u << 5, // a bounded wait on a copy barrier gave up
    FLAG_CHECK = 1u << 6, // an internal consistency check failed (status.check_code says which); the access was skipped
    FLAG_SORT = 1u << 7, // more particles changed cell than the incremental sort's mover buffer holds (the host grows it)
    FLAG_ABORT = 1u << 31, // processing stopped at status.abort_step; later substeps were no-ops
};
constexpr uint32_t ABORTING = FLAG_CFL | FLAG_NONFINITE | FLAG_OUT_OF_DOMAIN | FLAG_CAPACITY | FLAG_TIMEOUT | FLAG_CHECK | FLAG_SORT;

struct DevStatus {
    uint32_t flags;
    int32_t abort_step; // substep index (counted from the last reset) that raised an aborting flag
    uint32_t step; // substeps started since the last reset
    uint32_t n_groups; // groups (occupied SPGrid blocks) of the current substep
    uint32_t n_blocks; // active blocks (occupied + neighbours) of the current substep
    uint32_t work_p2g; // dynamic work counters of the persistent kernels
    uint32_t work_g2p;
    uint32_t fallback; // polar decompositions that took the FP64 SVD path (cumulative)
    uint32_t max_blocks_seen;
    uint32_t max_groups_seen;
    uint32_t check_code; // first failed internal check (0 = none)
    uint32_t check_count;
    uint32_t work_dmg; // work counters of the implicit damage solve's group kernels
    uint32_t work_cg;
    uint32_t cg_loops; // iterations of the damage solve's loop in this substep (any scene)
    uint32_t max_movers; // most particles that changed cell in one substep (incremental sort)
};

constexpr int MAX_OBJECTS = 8;
constexpr int MAX_MATERIALS = 16;

enum { MODEL_COROTATED = 0, MODEL_NEOHOOKEAN_BORDEN = 1, MODEL_QR_STABLE_NEOHOOKEAN = 2 };
enum { OBJ_STICKY = 1, OBJ_SLIP = 2, OBJ_SEPARATE = 3 };

template <class T>
struct Material {
    int model;
    int damage; // AnisoMPM phase-field damage attached
    T mu, lambda, kappa;
    T kx, ky; // QR-stable Neo-Hookean fibre stiffness (scale x mu, QRStableNeoHookean.h:75-86)
    T alpha, l0, eta, zeta, residual; // structural-tensor weight, length scale, viscosity, scale, residual stiffness
};

template <class T>
struct HalfSpaceObj {
    T origin[3], normal[3], vel[3]; // translating half-space: b(t) = vel * t, inside if n.(x - b - o) <= 0
    T friction;
    int type;
    int pad;
};

// Per-scene constants, indexed by the scene slot carried in the high bits of every key.
template <class T>
struct SceneParams {
    T dx, inv_dx, dt, D_inv; // D_inv = 4/dx^2 (MpmSimulationBase.cpp:118-122)
    T gravity[3];
    T apic_a, apic_b; // (r+1)/2, (r-1)/2 with r = apic_rpic_ratio
    T cfl;
    double time; // simulation time at the start of the current substep
    int64_t first; // first storage slot of the scene in the particle pool
    int64_t count;
    int32_t domain_cells; // base-node coordinates must stay in [0, domain_cells)
    int32_t n_objects;
    int32_t n_materials;
    int32_t damage;
    int32_t implicit; // damage by the implicit phase-field solve (AnisoFractureSimulation.h:129-141)
    int32_t pad_;
    Material<T> materials[MAX_MATERIALS];
    HalfSpaceObj<T> objects[MAX_OBJECTS];
};

} // namespace zr
