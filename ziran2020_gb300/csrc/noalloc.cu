// Binning of particles that already live in device memory, with no device allocation.
//
// Some callers cannot allocate device memory while they run: a host application that hands this
// library a slice of a pre-reserved arena and forbids cudaMalloc after start-up, a simulation loop
// whose memory budget was fixed when it was admitted, or a callback running inside another runtime
// (a renderer's or solver's step) where an allocation would synchronise the device or break that
// runtime's memory accounting. They still need the SPGrid binning of their particles
// (MpmSimulationBase::sortParticlesAndPolluteGrid, MpmSimulationBase.cpp:1531-1573): the reference's
// 64-bit keys sorted ascending, the sorted particle order and the first sorted index of each block.
//
// zr_bin_device_noalloc takes device inputs and device outputs from the caller and keeps all of its
// scratch (radix-sort temporary storage, the unsorted key buffer, the group counter) in one file-scope
// __device__ array of ZR_NOALLOC_SCRATCH_BYTES, sized for ZR_NOALLOC_MAX_PARTICLES particles. Every
// GPU that loads the library holds that array until the process exits.
#include "../../include/ziran_gb300.h"
#include "common.cuh"
#include "physics.cuh"

#include <cub/cub.cuh>
#include <cuda_runtime.h>
#include <thrust/iterator/counting_iterator.h>

#include <cstring>
#include <mutex>

namespace {

constexpr size_t kScratchBytes = ZR_NOALLOC_SCRATCH_BYTES;
constexpr int64_t kMaxN = ZR_NOALLOC_MAX_PARTICLES;

// the scratch itself: one array per device, shared by every call on that device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceScratch {
    bool ready = false; // set only by a set-up that succeeded
    unsigned char* base = nullptr; // device address of g_noalloc_scratch on this device
    size_t sort_bytes[2] = { 0, 0 }, sel_bytes[2] = { 0, 0 }; // CUB temporary storage at kMaxN (float, double keys)
};

constexpr int kMaxDevices = 64;
DeviceScratch g_dev[kMaxDevices];
std::mutex g_setup_mutex;

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

struct HeadOp {
    const uint64_t* k;
    __device__ bool operator()(uint32_t i) const { return i == 0 || (k[i] >> 32) != (k[i - 1] >> 32); }
};

// layout of the scratch array: [ sort temp | select temp | keys (8 kMaxN) | indices (4 kMaxN) | counters (256) ]
struct Layout {
    size_t sort_off, sel_off, keys_off, idx_off, cnt_off, end;
};

Layout layout(const DeviceScratch& d)
{
    Layout L;
    size_t sort = std::max(d.sort_bytes[0], d.sort_bytes[1]), sel = std::max(d.sel_bytes[0], d.sel_bytes[1]);
    L.sort_off = 0;
    L.sel_off = align256(sort);
    L.keys_off = L.sel_off + align256(sel);
    L.idx_off = L.keys_off + align256(sizeof(uint64_t) * (size_t)kMaxN);
    L.cnt_off = L.idx_off + align256(sizeof(uint32_t) * (size_t)kMaxN);
    L.end = L.cnt_off + 256;
    return L;
}

// Set-up, once per device, with that device current: resolve the array's device address and check that
// the radix sort and the selection fit next to the key buffer. Only a set-up that succeeded is kept: after a
// failure (for example a sticky error left by an unrelated earlier launch) the next call tries again. The
// address belongs to the device's primary context (the runtime API's context), which every call must use.
int setup(int dev)
{
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    DeviceScratch& d = g_dev[dev];
    if (d.ready) return ZR_OK;
    DeviceScratch fresh;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return ZR_ERR_CUDA;
    fresh.base = (unsigned char*)p;
    uint64_t* k = nullptr;
    uint32_t* v = nullptr;
    uint32_t* cnt = nullptr;
    for (int t = 0; t < 2; t++) {
        cub::DoubleBuffer<uint64_t> kb(k, k);
        cub::DoubleBuffer<uint32_t> vb(v, v);
        if (cub::DeviceRadixSort::SortPairs(nullptr, fresh.sort_bytes[t], kb, vb, (int64_t)kMaxN, 0, 64) != cudaSuccess
            || cub::DeviceSelect::If(nullptr, fresh.sel_bytes[t], thrust::counting_iterator<uint32_t>(0), v, cnt, (int64_t)kMaxN, HeadOp{ k })
                != cudaSuccess)
            return ZR_ERR_CUDA;
    }
    if (layout(fresh).end > kScratchBytes) return ZR_ERR_CAPACITY;
    fresh.ready = true;
    d = fresh;
    return ZR_OK;
}

template <class T>
__global__ void k_keys_ref(const T* x, int64_t n, T inv_dx, int domain_cells, uint64_t* keys, uint32_t* iota, uint32_t* flag)
{
    using L = typename zr::LayoutOf<T>::type;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int b[3];
        bool ok = true;
        for (int a = 0; a < 3; a++) {
            b[a] = zr::base_node(x[3 * i + a], inv_dx);
            ok = ok && b[a] >= 0 && b[a] < domain_cells;
        }
        if (!ok) {
            atomicOr(flag, 1u);
            b[0] = b[1] = b[2] = 0;
        }
        keys[i] = L::key(b[0], b[1], b[2], (uint32_t)i); // MpmSimulationBase.cpp:1547-1549
        iota[i] = (uint32_t)i;
    }
}

template <class T>
int run(int dev, int64_t n, const void* x, double dx, int domain_cells, uint64_t* sorted_keys, int32_t* order, int32_t* group_first, int64_t* n_groups,
    cudaStream_t st)
{
    using L = typename zr::LayoutOf<T>::type;
    const DeviceScratch& d = g_dev[dev];
    const Layout lay = layout(d);
    unsigned char* base = d.base;
    void* sort_tmp = base + lay.sort_off;
    void* sel_tmp = base + lay.sel_off;
    uint64_t* keys = (uint64_t*)(base + lay.keys_off);
    uint32_t* idx = (uint32_t*)(base + lay.idx_off);
    uint32_t* cnt = (uint32_t*)(base + lay.cnt_off); // [0] groups, [1] out-of-domain flag
    // the scratch keeps the previous call's contents: clear the counters that must start at zero
    if (cudaMemsetAsync(cnt, 0, 8, st) != cudaSuccess) return ZR_ERR_CUDA;
    const T inv_dx = (T)1 / (T)dx;
    k_keys_ref<T><<<256, 256, 0, st>>>((const T*)x, n, inv_dx, domain_cells, keys, idx, cnt + 1);
    const int t = std::is_same<T, float>::value ? 0 : 1;
    // highest key bit in use: coordinates below 2^cb, indices below 2^ib
    int cb = 0;
    while ((1 << cb) < domain_cells) cb++;
    const uint32_t maxc = (1u << cb) - 1;
    uint64_t top = L::key(maxc, maxc, maxc, (uint32_t)(n - 1));
    int end_bit = 0;
    while (end_bit < 64 && (top >> end_bit)) end_bit++;
    size_t sb = d.sort_bytes[t], se = d.sel_bytes[t];
    // ping-pong between the scratch buffers and the caller's outputs; copy back if the result ends in scratch
    cub::DoubleBuffer<uint64_t> kb(keys, sorted_keys);
    cub::DoubleBuffer<uint32_t> vb(idx, (uint32_t*)order);
    if (cub::DeviceRadixSort::SortPairs(sort_tmp, sb, kb, vb, n, 0, end_bit, st) != cudaSuccess) return ZR_ERR_CUDA;
    if (kb.Current() != sorted_keys && cudaMemcpyAsync(sorted_keys, kb.Current(), 8 * (size_t)n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return ZR_ERR_CUDA;
    if (vb.Current() != (uint32_t*)order && cudaMemcpyAsync(order, vb.Current(), 4 * (size_t)n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return ZR_ERR_CUDA;
    if (cub::DeviceSelect::If(sel_tmp, se, thrust::counting_iterator<uint32_t>(0), (uint32_t*)group_first, cnt, n, HeadOp{ sorted_keys }, st)
        != cudaSuccess)
        return ZR_ERR_CUDA;
    uint32_t host_cnt[2] = { 0, 0 };
    if (cudaMemcpyAsync(host_cnt, cnt, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
        return ZR_ERR_CUDA;
    if (n_groups) *n_groups = host_cnt[0];
    return host_cnt[1] ? ZR_ERR_OUT_OF_DOMAIN : ZR_OK;
}

} // namespace

extern "C" int zr_bin_device_noalloc(int precision, int64_t n, const void* x, double dx, int32_t domain_cells, uint64_t* sorted_keys, int32_t* order,
    int32_t* group_first, int64_t* n_groups, void* stream)
{
    if (precision != ZR_F32 && precision != ZR_F64) return ZR_ERR_ARG;
    if (n <= 0 || n > kMaxN) return ZR_ERR_ARG; // beyond the static scratch: the caller must split the call
    if (!x || !sorted_keys || !order || !group_first || !(dx > 0)) return ZR_ERR_ARG;
    if (domain_cells <= 0) domain_cells = 4096 - 8;
    if (domain_cells > 4096 - 8) return ZR_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ZR_ERR_CUDA;
    int rc = setup(dev);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    return precision == ZR_F32 ? run<float>(dev, n, x, dx, domain_cells, sorted_keys, order, group_first, n_groups, st)
                               : run<double>(dev, n, x, dx, domain_cells, sorted_keys, order, group_first, n_groups, st);
}
