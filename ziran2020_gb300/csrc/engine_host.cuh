// Host orchestration of Engine<T>: allocation, CUDA-graph capture of the substep, recovery after an
// aborted substep, transfers and timing. Included after engine_impl.cuh by engine_f32.cu / engine_f64.cu.
#pragma once
#include "engine_impl.cuh"

#include <cstdlib>
#include <map>
#include <mutex>

#define ZR_CUDA(call)                                                                                      \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) {                                                                           \
            err_ = std::string(#call) + ": " + cudaGetErrorString(e_);                                     \
            return ZR_ERR_CUDA_;                                                                           \
        }                                                                                                  \
    } while (0)

namespace zr {

enum { ZR_OK_ = 0, ZR_ERR_ARG_ = 1, ZR_ERR_CUDA_ = 2, ZR_ERR_CFL_ = 3, ZR_ERR_NONFINITE_ = 4, ZR_ERR_OUT_OF_DOMAIN_ = 5, ZR_ERR_BUDGET_ = 6,
    ZR_ERR_TIMEOUT_ = 7, ZR_ERR_CAPACITY_ = 8, ZR_ERR_STATE_ = 9 };

inline int bitlen(uint64_t v)
{
    int b = 0;
    while (v) {
        b++;
        v >>= 1;
    }
    return b;
}

template <class T>
class Engine final : public EngineBase {
    using L = typename LayoutOf<T>::type;
    static constexpr int GRAPH_K = 8; // substeps per multi-step graph (even: returns to the same buffer)
    // compiled schedule variants. P2G scatter: (particles per staged chunk, staging buffers); the large chunk
    // holds a whole occupied block of 8 particles per cell. G2P: threads per CTA.
    static constexpr int CH_BIG = sizeof(T) == 4 ? 512 : 256;
    static constexpr int VAR_CHUNK[3] = { CH_BIG, CH_BIG, CH_BIG / 2 };
    static constexpr int VAR_NBUF[3] = { 1, 2, 2 };
    static constexpr int G2P_NT[3] = { 64, 128, 256 };
    // G2P register budgets: threads per SM (FP32 448: a ~146-register cap, under which ptxas settles at 128 with
    // little spilling; 512: a 128 cap, more spills; FP64: ~255 or ~200)
    static constexpr int G2P_RES[2] = { sizeof(T) == 4 ? 448 : 256, sizeof(T) == 4 ? 512 : 320 };
    // fused P2G variants (schedule fused = 1, 2): register budgets cut for 2 or 3 CTAs per SM (FP32; 1 or 2 for FP64).
    // (Cut for 4 CTAs, with half-block chunks so that the staging buffers fit, it spilled and ran 60% slower.)
    static constexpr int FUSED_MINB[2] = { sizeof(T) == 4 ? 2 : 1, sizeof(T) == 4 ? 3 : 2 };
    static constexpr int FUSED_CH[2] = { FusedShape<T>::CHUNK, FusedShape<T>::CHUNK };
    static int fused_variant(int fused) { return fused - 1; }
    static int fused_code(int fv) { return fv + 1; }

public:
    Engine() { init_device(); }
    ~Engine() override { release(); }
    int precision() const override { return (int)sizeof(T); }
    std::string last_error() const override { return err_; }
    void* stream() const override { return (void*)stream_; }
    int n_scenes() const override { return (int)h_scenes_.size(); }
    int64_t count(int s) const override { return (s >= 0 && s < n_scenes()) ? h_scenes_[s].count : -1; }
    int64_t device_bytes() const override { return dev_bytes_; }

    int load(const std::vector<const SceneDesc*>& scenes) override
    {
        if (init_err_) return init_err_;
        release_batch();
        if (scenes.empty()) return arg("empty batch");
        return repack({}, scenes);
    }

    // Re-form the batch: keep the listed scenes (device state, in the given order) and append new ones.
    // Kept scenes move device-to-device into the other particle buffer (or into larger buffers when the
    // capacity grows); their time, materials and collision objects stay as they are on the device.
    int repack(const std::vector<int>& keep, const std::vector<const SceneDesc*>& add) override
    {
        if (init_err_) return init_err_;
        if (keep.empty() && add.empty()) return arg("empty batch");
        std::vector<SceneParams<T>> np;
        std::vector<int64_t> src_first;
        int64_t N = 0;
        if (!keep.empty()) {
            std::vector<SceneParams<T>> curp(h_scenes_.size());
            ZR_CUDA(cudaStreamSynchronize(stream_));
            ZR_CUDA(cudaMemcpy(curp.data(), d_scenes_, sizeof(SceneParams<T>) * curp.size(), cudaMemcpyDeviceToHost));
            for (int k : keep) {
                if (k < 0 || k >= (int)curp.size()) return arg("repack: kept scene out of range");
                SceneParams<T> sp = curp[k];
                src_first.push_back(sp.first);
                sp.first = N;
                N += sp.count;
                np.push_back(sp);
            }
        }
        int64_t max_add = 1;
        for (auto* sd : add) {
            if (!sd) return arg("null scene");
            SceneParams<T> sp;
            int rc = params_from_desc(*sd, sp);
            if (rc) return rc;
            sp.first = N;
            N += sd->n;
            max_add = std::max<int64_t>(max_add, sd->n);
            np.push_back(sp);
        }
        if (N >= (int64_t)0xffffffffLL) return arg("batch too large");
        // key layout of the new batch
        int max_domain = 0;
        for (auto& sp : np) max_domain = std::max(max_domain, sp.domain_cells);
        KeyLayout kl;
        const int cb = bitlen((uint64_t)(max_domain + 2 * std::max(L::sx, std::max(L::sy, L::sz)) - 1));
        const uint32_t maxc = (1u << cb) - 1;
        kl.ib = 0; // hot-path keys carry no particle index (binning() restores the reference's in-cell order)
        kl.cp = bitlen(L::offset(maxc, maxc, maxc)) - L::data_bits;
        kl.sb = bitlen((uint64_t)(np.size() - 1));
        kl.block_bits = L::block_bits;
        kl.wide = kl.total() > 32;
        if (kl.total() > 64) return arg("batch too large for 64-bit keys: reduce the number of scenes or their domain");
        drop_graphs();
        // particle buffers: the free half of the current pair, or a larger pair
        int dst;
        T* old_pool = pool_[cur_];
        uint32_t* old_pid = pid_[cur_];
        const int64_t old_cap = cap_;
        T* grown_pool[2] = { nullptr, nullptr };
        uint32_t* grown_pid[2] = { nullptr, nullptr };
        if ((uint64_t)N > cap_) {
            const int64_t cap = std::max<int64_t>(N, 2 * (int64_t)cap_);
            if (alloc((void**)&grown_pool[0], sizeof(T) * P_NF * cap) || alloc((void**)&grown_pool[1], sizeof(T) * P_NF * cap)
                || alloc((void**)&grown_pid[0], 4 * cap) || alloc((void**)&grown_pid[1], 4 * cap))
                return ZR_ERR_CUDA_;
            ZR_CUDA(cudaMemsetAsync(grown_pool[0], 0, sizeof(T) * P_NF * cap, stream_));
            ZR_CUDA(cudaMemsetAsync(grown_pool[1], 0, sizeof(T) * P_NF * cap, stream_));
            for (size_t q = 0; q < np.size() - add.size(); q++) {
                for (int f = 0; f < P_NF; f++)
                    ZR_CUDA(cudaMemcpyAsync(grown_pool[0] + (size_t)f * cap + np[q].first, old_pool + (size_t)f * old_cap + src_first[q],
                        sizeof(T) * np[q].count, cudaMemcpyDeviceToDevice, stream_));
                ZR_CUDA(cudaMemcpyAsync(grown_pid[0] + np[q].first, old_pid + src_first[q], 4 * np[q].count, cudaMemcpyDeviceToDevice, stream_));
            }
            ZR_CUDA(cudaStreamSynchronize(stream_));
            void* olds[] = { pool_[0], pool_[1], pid_[0], pid_[1], keys_in_, keys_sorted_, iota_, vals_sorted_, g_start_, sort_tmp_, pay_,
                sort_aux_, inc_move_, inc_bkey_, inc_bidx_ };
            for (void* p : olds)
                if (p) cudaFree(p);
            pool_[0] = grown_pool[0];
            pool_[1] = grown_pool[1];
            pid_[0] = grown_pid[0];
            pid_[1] = grown_pid[1];
            cap_ = (uint64_t)cap;
            pay_ = nullptr;
            sort_aux_ = nullptr;
            inc_move_ = inc_bkey_ = inc_bidx_ = nullptr;
            // P2G payload: NPAY fields of sorted particles at q + q/8, plus the copy granularity at the end
            pstride_ = (int64_t)((pay_pos((uint64_t)cap) + 64 + 63) & ~(uint64_t)63);
            if (alloc((void**)&keys_in_, 8 * cap) || alloc((void**)&keys_sorted_, 8 * cap) || alloc((void**)&iota_, 4 * cap)
                || alloc((void**)&vals_sorted_, 4 * cap) || alloc((void**)&g_start_, 4 * cap) || alloc((void**)&pay_, sizeof(T) * NPAY * (size_t)pstride_)
                || alloc((void**)&sort_aux_, sort_aux_bytes(cap)) || alloc((void**)&inc_move_, 4 * cap)
                || alloc((void**)&inc_bkey_, 4 * bucket_slots(cap)) || alloc((void**)&inc_bidx_, 4 * bucket_slots(cap)))
                return ZR_ERR_CUDA_;
            mcap_ = std::min<int64_t>(cap, std::max<int64_t>(MCAP_MIN, cap / 32));
            ZR_CUDA(cudaMemsetAsync(pay_, 0, sizeof(T) * NPAY * (size_t)pstride_, stream_));
            k_iota<T><<<nsm_ * 4, 256, 0, stream_>>>(iota_, (uint32_t)cap);
            size_t sb = 0, sb32 = 0;
            ZR_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sb, keys_in_, keys_sorted_, iota_, vals_sorted_, cap, 0, 64, stream_));
            ZR_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sb32, (uint32_t*)keys_in_, (uint32_t*)keys_sorted_, iota_, vals_sorted_, cap, 0, 32,
                stream_));
            sort_bytes_ = std::max(sb, sb32); // the key width follows the batch: room for either
            if (alloc(&sort_tmp_, sort_bytes_)) return ZR_ERR_CUDA_;
            dst = 0;
        }
        else {
            dst = cur_ ^ 1;
            for (size_t q = 0; q < np.size() - add.size(); q++) {
                for (int f = 0; f < P_NF; f++)
                    ZR_CUDA(cudaMemcpyAsync(pool_[dst] + (size_t)f * cap_ + np[q].first, pool_[cur_] + (size_t)f * cap_ + src_first[q],
                        sizeof(T) * np[q].count, cudaMemcpyDeviceToDevice, stream_));
                ZR_CUDA(cudaMemcpyAsync(pid_[dst] + np[q].first, pid_[cur_] + src_first[q], 4 * np[q].count, cudaMemcpyDeviceToDevice, stream_));
            }
        }
        // per-scene device arrays
        if (np.size() > scene_cap_) {
            void* p1 = d_scenes_;
            dfree(p1);
            void* p2 = grid_mass_;
            dfree(p2);
            void* p3 = cgs_;
            dfree(p3);
            d_scenes_ = nullptr;
            grid_mass_ = nullptr;
            cgs_ = nullptr;
            scene_cap_ = std::max<size_t>(np.size(), 2 * scene_cap_);
            if (alloc((void**)&d_scenes_, sizeof(SceneParams<T>) * scene_cap_) || alloc((void**)&grid_mass_, 8 * scene_cap_)
                || alloc((void**)&cgs_, sizeof(CgScalars) * scene_cap_))
                return ZR_ERR_CUDA_;
        }
        if (!st_ && alloc((void**)&st_, sizeof(DevStatus))) return ZR_ERR_CUDA_;
        h_scenes_ = np;
        N_ = (uint32_t)N;
        kl_ = kl;
        cur_ = dst;
        models_ = 0;
        any_damage_ = false;
        implicit_ = false;
        drive_stale_ = true;
        for (auto& sp : h_scenes_) {
            for (int k = 0; k < sp.n_materials; k++) models_ |= 1 << sp.materials[k].model;
            any_damage_ = any_damage_ || sp.damage;
            implicit_ = implicit_ || sp.implicit;
        }
        tuned_ = false;
        sorted_storage_ = false;
        sort_base_stale_ = true;
        ck_valid_ = false;
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        ZR_CUDA(cudaMemsetAsync(grid_mass_, 0, 8 * scene_cap_, stream_));
        ZR_CUDA(cudaMemcpyAsync(d_scenes_, h_scenes_.data(), sizeof(SceneParams<T>) * h_scenes_.size(), cudaMemcpyHostToDevice, stream_));
        // new scenes: host -> device
        const size_t first_new = np.size() - add.size();
        uint8_t* d_mat = nullptr;
        if (!add.empty() && alloc((void**)&d_mat, (size_t)max_add)) return ZR_ERR_CUDA_;
        std::vector<T> buf;
        for (size_t q = 0; q < add.size(); q++) {
            int rc = upload_scene(*add[q], h_scenes_[first_new + q].first, dst, d_mat, buf);
            if (rc) {
                cudaFree(d_mat);
                return rc;
            }
        }
        if (d_mat) {
            cudaFree(d_mat);
            dev_bytes_ -= (int64_t)max_add;
        }
        // keys, and a first binning pass that sizes the grid (every group activates at most 8 blocks)
        k_keys<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), d_scenes_, n_scenes(), keys_in_, N_, kl_, st_);
        ZR_CUDA(sort_keys((int64_t)N_));
        ZR_CUDA(group_heads((int64_t)N_));
        DevStatus hs;
        ZR_CUDA(cudaMemcpyAsync(&hs, st_, sizeof hs, cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        if (hs.flags & FLAG_OUT_OF_DOMAIN) return fail(ZR_ERR_OUT_OF_DOMAIN_, "a particle lies outside its scene's domain");
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        const uint32_t need = std::max<uint32_t>(4096, 8 * hs.n_groups + 1024);
        if (need > b_cap_) {
            int rc = alloc_grid(std::max(need, b_cap_ * 2));
            if (rc) return rc;
        }
        else {
            ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)b_cap_ * NACC * L::nodes, stream_));
            ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
            int rc = ensure_cg();
            if (rc) return rc;
        }
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    int step(int nsteps, StepReport* rep) override
    {
        if (init_err_) return init_err_;
        if (!N_) return fail(ZR_ERR_STATE_, "no scenes loaded");
        if (nsteps < 0) return arg("nsteps must be >= 0");
        int done = 0;
        StepReport r;
        int rc = 0;
        if (nsteps > 0 && !tuned_ && !fixed_schedule_ && !autotune_cached()) {
            // the trials must see the particles in sorted storage order, which one substep of G2P produces
            if (!sorted_storage_) rc = run_steps(1, r, done);
            if (!rc && done < nsteps) rc = autotune_trials();
        }
        if (!rc) rc = run_steps(nsteps - done, r, done);
        r.steps_done = done;
        if (rep) *rep = r;
        return rc;
    }

    // Advance nsteps substeps with the current schedule; r accumulates the report, done counts finished substeps.
    // An aborted substep is retried after growing the grid (capacity) or reported with the state left at its start.
    int run_steps(int nsteps, StepReport& r, int& done)
    {
        if (int rc = refresh_drive()) return rc;
        const int target = done + nsteps;
        int grow_rounds = 0;
        while (done < target) {
            ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
            const int cur0 = cur_;
            int todo = target - done;
            if (!timing_ && graphs_on_) {
                int rcg = prepare_graphs(todo - (sort_base_stale_ ? 1 : 0));
                if (rcg) return rcg;
            }
            ZR_CUDA(cudaEventRecord(t0_, stream_));
            int rc = launch_steps(todo);
            if (rc) return rc;
            ZR_CUDA(cudaEventRecord(t1_, stream_));
            ZR_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_));
            ZR_CUDA(cudaStreamSynchronize(stream_));
            float ms = 0;
            cudaEventElapsedTime(&ms, t0_, t1_);
            r.device_ms += ms;
            if (timing_) collect_timing(todo);
            r.fallback += hst_->fallback;
            r.n_groups = hst_->max_groups_seen;
            r.n_blocks = hst_->max_blocks_seen;
            r.flags |= hst_->flags;
            if (!(hst_->flags & FLAG_ABORT)) {
                cur_ = (cur0 + todo) & 1;
                done += todo;
                sorted_storage_ = true;
                sort_base_stale_ = false;
                // the mover buffer follows the movers seen: shrink to 3x the most seen when it is 8x too large
                // (graphs are re-captured); a substep with more movers than it holds is repeated after growing it
                const int64_t mm = (int64_t)hst_->max_movers;
                if (inc_sort_usable() && todo >= 8 && mm > 0 && 8 * mm < mcap_ && mcap_ > MCAP_MIN) {
                    mcap_ = std::min<int64_t>((int64_t)cap_, std::max<int64_t>(MCAP_MIN, 3 * mm));
                    drop_graphs();
                }
                break;
            }
            sort_base_stale_ = true; // the aborted substep's sort overwrote the base
            const int k = hst_->abort_step;
            done += k;
            cur_ = (cur0 + k) & 1;
            if (k > 0) sorted_storage_ = true;
            // the aborted substep may have left partial grid sums, hash entries or next keys behind
            ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)b_cap_ * NACC * L::nodes, stream_));
            ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
            if (cg_) ZR_CUDA(cudaMemsetAsync(cg_, 0, sizeof(T) * CG_NF * (size_t)b_cap_ * L::nodes, stream_));
            ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
            k_keys<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), d_scenes_, n_scenes(), keys_in_, N_, kl_, st_);
            ZR_CUDA(cudaStreamSynchronize(stream_));
            const uint32_t f = hst_->flags;
            if ((f & FLAG_SORT) && !(f & (FLAG_CFL | FLAG_NONFINITE | FLAG_OUT_OF_DOMAIN | FLAG_TIMEOUT | FLAG_CHECK | FLAG_CAPACITY))) {
                // more movers than the list holds (grow it), or a bucket beyond the merge's shared memory: the
                // substep is repeated with a full sort (it cannot raise FLAG_SORT, so every retry makes progress)
                const int64_t mm = (int64_t)hst_->max_movers;
                if (mm > mcap_ && mcap_ < (int64_t)cap_) {
                    mcap_ = std::min<int64_t>((int64_t)cap_, std::max<int64_t>(2 * mcap_, mm + mm / 2));
                    drop_graphs();
                }
                continue;
            }
            if ((f & FLAG_CAPACITY) && !(f & (FLAG_CFL | FLAG_NONFINITE | FLAG_OUT_OF_DOMAIN | FLAG_TIMEOUT | FLAG_CHECK)) && grow_rounds < 6) {
                grow_rounds++;
                int rc2 = alloc_grid(b_cap_ * 2);
                if (rc2) return rc2;
                continue; // retry the aborted substep with a larger grid
            }
            if (f & FLAG_NONFINITE) return fail(ZR_ERR_NONFINITE_, "non-finite particle state at substep " + std::to_string(done));
            if (f & FLAG_OUT_OF_DOMAIN) return fail(ZR_ERR_OUT_OF_DOMAIN_, "a particle left its scene's domain at substep " + std::to_string(done));
            if (f & FLAG_CFL) return fail(ZR_ERR_CFL_, "a particle moved more than one cell at substep " + std::to_string(done) + " (reduce dt)");
            if (f & FLAG_TIMEOUT) return fail(ZR_ERR_TIMEOUT_, "bounded wait expired at substep " + std::to_string(done));
            if (f & FLAG_CHECK)
                return fail(ZR_ERR_STATE_, "internal consistency check " + std::to_string(hst_->check_code) + " failed " + std::to_string(hst_->check_count) +
                        " times at substep " + std::to_string(done));
            return fail(ZR_ERR_CAPACITY_, "active-block capacity exhausted");
        }
        return 0;
    }

    // storage slot of every particle of scene s in the caller's order (inv_), for the row transfers
    int fill_inv(int s)
    {
        if (!inv_ || inv_cap_ < cap_) {
            void* old = inv_;
            dfree(old);
            inv_ = nullptr;
            inv_cap_ = 0;
            if (alloc((void**)&inv_, 4 * (size_t)cap_)) return ZR_ERR_CUDA_;
            inv_cap_ = cap_;
        }
        k_inv<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), h_scenes_[s].first, h_scenes_[s].count, inv_);
        ZR_CUDA(cudaGetLastError());
        return 0;
    }
    // the device address of a buffer in pinned host memory, or null for any other buffer
    static void* mapped(const void* host)
    {
        cudaPointerAttributes at;
        void* dev = nullptr;
        if (cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) dev = at.devicePointer;
        cudaGetLastError(); // an unknown pointer only means: not mapped
        return dev;
    }
    template <int MODE>
    int launch_rows(int s, const RowFields& rf, const void* in, void* out, int f32)
    {
        const int64_t n = h_scenes_[s].count;
        const int grid = (int)std::min<int64_t>((n + IO_ROWS - 1) / IO_ROWS, (int64_t)nsm_ * 16);
        const size_t sm = (size_t)IO_ROWS * rf.W * (f32 ? 4 : 8) * (MODE == ROWS_EXCHANGE ? 2 : 1);
        if (grid > 0) {
            if (f32) {
                if (sm > 48 * 1024) ZR_CUDA(cudaFuncSetAttribute(k_rows<T, float, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                k_rows<T, float, MODE><<<grid, IO_ROWS, sm, stream_>>>(pool(cur_), inv_, n, rf, (const float*)in, (float*)out);
            }
            else {
                if (sm > 48 * 1024) ZR_CUDA(cudaFuncSetAttribute(k_rows<T, double, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                k_rows<T, double, MODE><<<grid, IO_ROWS, sm, stream_>>>(pool(cur_), inv_, n, rf, (const double*)in, (double*)out);
            }
        }
        ZR_CUDA(cudaGetLastError());
        return 0;
    }

    // Rows of scene s between the pool and a caller's row-major buffer (rf: which fields). A buffer in pinned host
    // memory is read or written by the kernel itself over the host link; any other goes through the staging buffer
    // with one copy. Synchronises.
    int transfer_rows(int s, const RowFields& rf, void* host, int f32, bool exporting)
    {
        const size_t bytes = (size_t)h_scenes_[s].count * rf.W * (f32 ? 4 : 8);
        int rc = fill_inv(s);
        if (rc) return rc;
        void* dev = mapped(host);
        if (!dev) {
            rc = ensure_stage(bytes);
            if (rc) return rc;
            dev = stage_;
            if (!exporting) ZR_CUDA(cudaMemcpyAsync(stage_, host, bytes, cudaMemcpyHostToDevice, stream_));
        }
        rc = exporting ? launch_rows<ROWS_EXPORT>(s, rf, nullptr, dev, f32) : launch_rows<ROWS_IMPORT>(s, rf, dev, nullptr, f32);
        if (rc) return rc;
        if (exporting && dev == stage_) ZR_CUDA(cudaMemcpyAsync(host, stage_, bytes, cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }
    static RowFields state_fields()
    {
        RowFields rf{};
        const int f0s[5] = { P_X, P_V, P_C, P_F, P_D }, ncs[5] = { 3, 3, 9, 9, 1 };
        for (int q = 0; q < 5; q++) {
            rf.f0[q] = f0s[q];
            rf.nc[q] = ncs[q];
        }
        rf.count = 5;
        rf.W = 25;
        return rf;
    }

    int get_field(int s, int field, void* out, int f32) override
    {
        RowFields rf{};
        if (!field_range(field, rf.f0[0], rf.nc[0])) return arg("unknown field");
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        rf.count = 1;
        rf.W = rf.nc[0];
        return transfer_rows(s, rf, out, f32, true);
    }

    int set_field(int s, int field, const void* in, int f32) override
    {
        RowFields rf{};
        if (!field_range(field, rf.f0[0], rf.nc[0])) return arg("unknown field");
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        rf.count = 1;
        rf.W = rf.nc[0];
        int rc = transfer_rows(s, rf, const_cast<void*>(in), f32, false);
        if (rc) return rc;
        if (field == FIELD_F || field == FIELD_SIGMA_C) ZR_CUDA(forget_drive(s));
        if (field == FIELD_X) return rekey();
        return 0;
    }

    int get_state(int s, void* out, int f32) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        return transfer_rows(s, state_fields(), out, f32, true);
    }

    int set_state(int s, const void* in, int f32) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        int rc = transfer_rows(s, state_fields(), const_cast<void*>(in), f32, false);
        if (rc) return rc;
        ZR_CUDA(forget_drive(s));
        return rekey();
    }

    int exchange_state(int s, const void* in, void* out, int f32) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        const RowFields rf = state_fields();
        const size_t bytes = (size_t)h_scenes_[s].count * rf.W * (f32 ? 4 : 8);
        const char *i0 = (const char*)in, *o0 = (const char*)out;
        if (bytes && i0 < o0 + bytes && o0 < i0 + bytes) return arg("exchange_state: the input and output buffers overlap");
        void *din = mapped(in), *dout = mapped(out);
        if (!din || !dout) { // not both mapped: one direction after the other
            int rc = get_state(s, out, f32);
            return rc ? rc : set_state(s, in, f32);
        }
        int rc = fill_inv(s);
        if (rc) return rc;
        rc = launch_rows<ROWS_EXCHANGE>(s, rf, din, dout, f32);
        if (rc) return rc;
        ZR_CUDA(cudaStreamSynchronize(stream_));
        ZR_CUDA(forget_drive(s));
        return rekey();
    }

    // Pipelined jobs. Job 0 runs the safe way (set_state, step, get_state: it tunes the schedule, builds the one-substep
    // graphs and leaves a valid sort base). Jobs 1.. run without a host check between them: input i is copied host ->
    // device (copy engine, stream h2d_) into one of two device slots two jobs ahead, imported by a kernel, keyed, stepped
    // by the one-substep graph, exported into one of two output slots and copied device -> host (stream d2h_) while the
    // next jobs compute. The status is read once at the end; the status flags accumulate, so after the first aborted
    // job every later substep returns at once, and the jobs from the aborted one on are run again the safe way (its
    // retries and errors are those of step()). Events order slot reuse: 0-1 input copied, 2-3 input imported, 4-5
    // output exported, 6-7 output copied.
    int stream_steps(int s, int nsteps, const void* const* in, void* const* out, int f32) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        if (nsteps < 0 || (nsteps > 0 && (!in || !out))) return arg("stream_steps: bad step count or buffer lists");
        for (int i = 0; i < nsteps; i++)
            if (!in[i] || !out[i]) return arg("stream_steps: a null buffer");
        const RowFields rf = state_fields();
        const size_t bytes = (size_t)h_scenes_[s].count * rf.W * (f32 ? 4 : 8);
        // a later job's input is copied while earlier results are written: no output may overlap a later input
        for (int i = 0; i < nsteps; i++)
            for (int j = i + 1; j < nsteps; j++) {
                const char *o = (const char*)out[i], *q = (const char*)in[j];
                if (bytes && o < q + bytes && q < o + bytes) return arg("stream_steps: an output overlaps the input of a later job");
            }
        auto safe_job = [&](int i) -> int {
            int rc = set_state(s, in[i], f32);
            StepReport r;
            if (!rc) rc = step(1, &r);
            if (!rc) rc = get_state(s, out[i], f32);
            return rc;
        };
        if (nsteps <= 1 || timing_ || !graphs_on_) {
            for (int i = 0; i < nsteps; i++)
                if (int rc = safe_job(i)) return rc;
            return 0;
        }
        int rc = ensure_io(bytes);
        if (rc) return rc;
        auto issue_in = [&](int i) -> cudaError_t {
            const int b = i & 1;
            cudaError_t e = cudaStreamWaitEvent(h2d_, io_ev_[2 + b], 0); // the slot's previous input was imported
            if (e == cudaSuccess) e = cudaMemcpyAsync(io_in_[b], in[i], bytes, cudaMemcpyHostToDevice, h2d_);
            if (e == cudaSuccess) e = cudaEventRecord(io_ev_[b], h2d_);
            return e;
        };
        // the caller's buffers are in use until every copy has finished, also after a failure
        auto drain = [&]() -> cudaError_t {
            const cudaError_t e1 = cudaStreamSynchronize(h2d_), e2 = cudaStreamSynchronize(d2h_), e3 = cudaStreamSynchronize(stream_);
            return e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
        };
        cudaError_t e = issue_in(1);
        if (e != cudaSuccess) {
            drain();
            return cuda_fail(e);
        }
        rc = safe_job(0);
        if (!rc && nsteps > 2 && (e = issue_in(2)) != cudaSuccess) rc = cuda_fail(e);
        if (!rc) rc = prepare_graphs(1);
        if (rc) {
            drain();
            return rc;
        }
        const int cur1 = cur_; // the parity job 1 reads
        e = cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_);
        for (int i = 1; i < nsteps && e == cudaSuccess && !rc; i++) {
            const int b = i & 1;
            if ((e = cudaStreamWaitEvent(stream_, io_ev_[b], 0)) != cudaSuccess) break;
            if ((rc = fill_inv(s)) || (rc = launch_rows<ROWS_IMPORT>(s, rf, io_in_[b], nullptr, f32))) break;
            if ((e = cudaEventRecord(io_ev_[2 + b], stream_)) != cudaSuccess) break;
            k_keys<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), d_scenes_, n_scenes(), keys_in_, N_, kl_, st_); // raises FLAG_OUT_OF_DOMAIN
            forget_drive(s);
            if ((rc = refresh_drive())) break;
            if (i + 2 < nsteps && (e = issue_in(i + 2)) != cudaSuccess) break;
            if ((e = cudaGraphLaunch(g1_[cur_ & 1], stream_)) != cudaSuccess) break;
            cur_ ^= 1;
            if ((e = cudaStreamWaitEvent(stream_, io_ev_[6 + b], 0)) != cudaSuccess) break; // the slot's previous output was copied
            if ((rc = fill_inv(s)) || (rc = launch_rows<ROWS_EXPORT>(s, rf, nullptr, io_out_[b], f32))) break;
            if ((e = cudaEventRecord(io_ev_[4 + b], stream_)) != cudaSuccess || (e = cudaStreamWaitEvent(d2h_, io_ev_[4 + b], 0)) != cudaSuccess
                || (e = cudaMemcpyAsync(out[i], io_out_[b], bytes, cudaMemcpyDeviceToHost, d2h_)) != cudaSuccess
                || (e = cudaEventRecord(io_ev_[6 + b], d2h_)) != cudaSuccess)
                break;
        }
        const cudaError_t ed = drain();
        if (!rc && e != cudaSuccess) rc = cuda_fail(e);
        if (!rc && ed != cudaSuccess) rc = cuda_fail(ed);
        if (rc) return rc;
        ZR_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        sorted_storage_ = true;
        if (!(hst_->flags & FLAG_ABORT)) return 0;
        // job k aborted (substeps are counted from job 1): its input pool (parity) was intact when it started; the later
        // jobs' imports and the aborted substep may have left partial grid sums, hash entries and a broken sort base
        const int k = 1 + std::max(0, (int)hst_->abort_step);
        cur_ = (cur1 + k - 1) & 1;
        sort_base_stale_ = true;
        sorted_storage_ = false;
        ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)b_cap_ * NACC * L::nodes, stream_));
        ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
        if (cg_) ZR_CUDA(cudaMemsetAsync(cg_, 0, sizeof(T) * CG_NF * (size_t)b_cap_ * L::nodes, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        stream_reruns_ += nsteps - k;
        for (int i = k; i < nsteps; i++)
            if ((rc = safe_job(i))) return rc;
        return 0;
    }
    int64_t stream_reruns() const override { return stream_reruns_; }
    int ensure_io(size_t bytes)
    {
        if (!h2d_) {
            if (cudaStreamCreateWithFlags(&h2d_, cudaStreamNonBlocking) != cudaSuccess || cudaStreamCreateWithFlags(&d2h_, cudaStreamNonBlocking) != cudaSuccess)
                return fail(ZR_ERR_CUDA_, "copy stream creation failed");
            for (auto& ev : io_ev_)
                if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return fail(ZR_ERR_CUDA_, "event creation failed");
        }
        if (bytes <= io_bytes_) return 0;
        ZR_CUDA(cudaStreamSynchronize(h2d_));
        ZR_CUDA(cudaStreamSynchronize(d2h_));
        free_io();
        for (int b = 0; b < 2; b++)
            if (alloc(&io_in_[b], bytes) || alloc(&io_out_[b], bytes)) return ZR_ERR_CUDA_;
        io_bytes_ = bytes;
        return 0;
    }
    void free_io()
    {
        for (int b = 0; b < 2; b++) {
            dfree(io_in_[b]);
            dfree(io_out_[b]);
            io_in_[b] = io_out_[b] = nullptr;
        }
        io_bytes_ = 0;
    }

    int reductions(int s, double* out7) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        int rc = ensure_stage(64);
        if (rc) return rc;
        ZR_CUDA(cudaMemsetAsync(stage_, 0, 64, stream_));
        k_reduce<T><<<nsm_ * 2, 256, 0, stream_>>>(pool(cur_), h_scenes_[s].first, h_scenes_[s].count, (double*)stage_);
        ZR_CUDA(cudaMemcpyAsync(out7, stage_, 6 * 8, cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaMemcpyAsync(out7 + 6, grid_mass_ + s, 8, cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    int set_dt(int s, double dt) override
    {
        if (s < 0 || s >= n_scenes() || !(dt > 0)) return arg("bad scene or dt");
        h_scenes_[s].dt = (T)dt;
        ZR_CUDA(cudaMemcpyAsync((char*)(d_scenes_ + s) + offsetof(SceneParams<T>, dt), &h_scenes_[s].dt, sizeof(T), cudaMemcpyHostToDevice, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    double dt(int s) const override { return (s >= 0 && s < n_scenes()) ? (double)h_scenes_[s].dt : NAN; }

    int set_time(int s, double t) override
    {
        if (s < 0 || s >= n_scenes() || !(t >= 0)) return arg("bad scene or time");
        ZR_CUDA(cudaMemcpyAsync((char*)(d_scenes_ + s) + offsetof(SceneParams<T>, time), &t, 8, cudaMemcpyHostToDevice, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    int checkpoint_save() override
    {
        if (!N_) return fail(ZR_ERR_STATE_, "no scenes loaded");
        const size_t pool_b = sizeof(T) * P_NF * (size_t)cap_, pid_b = 4 * (size_t)cap_, sc_b = sizeof(SceneParams<T>) * h_scenes_.size();
        if (!ck_pool_ || ck_cap_ != cap_ || ck_scenes_n_ < h_scenes_.size()) {
            dfree(ck_pool_);
            dfree(ck_pid_);
            dfree(ck_scenes_);
            if (alloc(&ck_pool_, pool_b) || alloc(&ck_pid_, pid_b) || alloc(&ck_scenes_, sc_b)) return ZR_ERR_CUDA_;
            ck_cap_ = cap_;
            ck_scenes_n_ = h_scenes_.size();
        }
        ZR_CUDA(cudaMemcpyAsync(ck_pool_, pool_[cur_], pool_b, cudaMemcpyDeviceToDevice, stream_));
        ZR_CUDA(cudaMemcpyAsync(ck_pid_, pid_[cur_], pid_b, cudaMemcpyDeviceToDevice, stream_));
        ZR_CUDA(cudaMemcpyAsync(ck_scenes_, d_scenes_, sc_b, cudaMemcpyDeviceToDevice, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        ck_host_scenes_ = h_scenes_;
        ck_valid_ = true;
        return 0;
    }

    // the cached damage drive (P_DRV) no longer matches F: refilled before the next substep
    cudaError_t forget_drive(int)
    {
        drive_stale_ = true;
        return cudaSuccess;
    }
    int refresh_drive()
    {
        if (!implicit_ || !drive_stale_) return 0;
        k_dmg_drive<T><<<nsm_ * 8, 256, 0, stream_>>>(args(cur_), keys_in_);
        ZR_CUDA(cudaGetLastError());
        drive_stale_ = false;
        return 0;
    }

    int cg_iterations(int s, int* out) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        *out = 0;
        if (!h_scenes_[s].implicit || !cgs_) return 0;
        CgScalars c;
        ZR_CUDA(cudaMemcpyAsync(&c, cgs_ + s, sizeof c, cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        *out = c.iter;
        return 0;
    }

    int checkpoint_restore() override
    {
        if (!ck_valid_ || ck_cap_ != cap_ || ck_host_scenes_.size() != h_scenes_.size()) return fail(ZR_ERR_STATE_, "no checkpoint of this batch");
        const size_t pool_b = sizeof(T) * P_NF * (size_t)cap_, pid_b = 4 * (size_t)cap_, sc_b = sizeof(SceneParams<T>) * h_scenes_.size();
        ZR_CUDA(cudaMemcpyAsync(pool_[cur_], ck_pool_, pool_b, cudaMemcpyDeviceToDevice, stream_));
        ZR_CUDA(cudaMemcpyAsync(pid_[cur_], ck_pid_, pid_b, cudaMemcpyDeviceToDevice, stream_));
        ZR_CUDA(cudaMemcpyAsync(d_scenes_, ck_scenes_, sc_b, cudaMemcpyDeviceToDevice, stream_));
        h_scenes_ = ck_host_scenes_;
        // a clean grid and the keys of the restored positions
        ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)b_cap_ * NACC * L::nodes, stream_));
        ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
        return rekey();
    }

    double time(int s) const override
    {
        if (s < 0 || s >= n_scenes()) return NAN;
        double t = NAN;
        if (cudaMemcpy(&t, (const char*)(d_scenes_ + s) + offsetof(SceneParams<T>, time), 8, cudaMemcpyDeviceToHost) != cudaSuccess) return NAN;
        return t;
    }

    int binning(int s, std::vector<uint64_t>& keys, std::vector<int32_t>& order, std::vector<int32_t>& group_first, std::vector<uint64_t>& pages) override
    {
        if (s < 0 || s >= n_scenes()) return arg("scene index out of range");
        const int64_t n = N_;
        for (int attempt = 0;; attempt++) {
            ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
            ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
            StepArgs<T> a = args(cur_);
            ZR_CUDA(sort_keys(n));
            k_cellfix<T><<<nsm_ * 8, 256, 0, stream_>>>(keys_sorted_, vals_sorted_, pid_[cur_], N_, kl_);
            ZR_CUDA(group_heads(n));
            k_activate<T><<<nsm_ * 4, 256, 0, stream_>>>(a);
            ZR_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_));
            ZR_CUDA(cudaStreamSynchronize(stream_));
            if (!(hst_->flags & FLAG_CAPACITY) || attempt >= 6) break;
            int rcg = alloc_grid(b_cap_ * 2);
            if (rcg) return rcg;
        }
        StepArgs<T> a = args(cur_);
        (void)a;
        const uint32_t G = hst_->n_groups, B = std::min(hst_->n_blocks, b_cap_);
        std::vector<uint64_t> sk(n), bk(B);
        std::vector<uint32_t> gs(G), vs(n), pd(n);
        if (kl_.wide)
            ZR_CUDA(cudaMemcpy(sk.data(), keys_sorted_, 8 * n, cudaMemcpyDeviceToHost));
        else {
            std::vector<uint32_t> sk32(n);
            ZR_CUDA(cudaMemcpy(sk32.data(), keys_sorted_, 4 * n, cudaMemcpyDeviceToHost));
            for (int64_t i = 0; i < n; i++) sk[i] = sk32[i];
        }
        ZR_CUDA(cudaMemcpy(vs.data(), vals_sorted_, 4 * n, cudaMemcpyDeviceToHost));
        ZR_CUDA(cudaMemcpy(pd.data(), pid_[cur_], 4 * n, cudaMemcpyDeviceToHost));
        ZR_CUDA(cudaMemcpy(gs.data(), g_start_, 4 * (size_t)G, cudaMemcpyDeviceToHost));
        ZR_CUDA(cudaMemcpy(bk.data(), b_key_, 8 * (size_t)B, cudaMemcpyDeviceToHost));
        // restore a clean grid for the next substep
        ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        const int64_t first = h_scenes_[s].first, cnt = h_scenes_[s].count;
        keys.resize(cnt);
        order.resize(cnt);
        const uint64_t cpmask = (1ULL << kl_.cp) - 1;
        for (int64_t i = 0; i < cnt; i++) {
            uint64_t k = sk[first + i];
            uint32_t o = pd[vs[first + i]] & ((1u << L::index_bits) - 1); // original index from the particle id
            keys[i] = (((k >> kl_.ib) & cpmask) << L::index_bits) | o; // the reference's key layout
            order[i] = (int32_t)o;
        }
        group_first.clear();
        for (uint32_t g = 0; g < G; g++)
            if ((int64_t)gs[g] >= first && (int64_t)gs[g] < first + cnt) group_first.push_back((int32_t)(gs[g] - first));
        pages.clear();
        for (uint32_t b = 0; b < B; b++)
            if ((bk[b] >> 40) == (uint64_t)s) pages.push_back(bk[b] & ((1ULL << 40) - 1));
        std::sort(pages.begin(), pages.end());
        if (hst_->flags & FLAG_ABORT) return fail(ZR_ERR_CAPACITY_, "binning overflowed the active-block table");
        return 0;
    }

    void set_timing(bool on) override { timing_ = on; }
    KernelTimes timing() const override { return kt_; }
    void reset_timing() override { kt_ = KernelTimes(); }
    int sync() override
    {
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }
    int use_graph(bool on) override
    {
        graphs_on_ = on;
        return 0;
    }
    int kernel_launches_per_step() const override { return launches_per_step_; }

    // Schedule autotuner. The tunable launch shapes change no arithmetic beyond the order of floating-point
    // sums: P2G particles per staged chunk and P2G CTAs per SM, G2P threads per CTA (particles per warp
    // per pass over a group). Each candidate runs single trial substeps on the current state, timed with
    // CUDA events on the engine's stream; the state is rolled back after each trial (the trial writes only
    // the other particle buffer, the next-substep keys and the scene clocks, which are restored). The
    // choice is cached per (precision, models, damage, particle-count and scene-count magnitude).
    int set_autotune(int mode) override
    {
        autotune_mode_ = mode;
        fixed_schedule_ = false;
        tuned_ = false;
        return 0;
    }
    Schedule schedule() const override { return sched_; }
    int set_schedule(const Schedule& sc) override
    {
        if (sc.fused < 0 || sc.fused > 3 || (!sc.fused && variant_index(sc.chunk, sc.buffers) < 0) || g2p_index(sc.g2p_threads) < 0
            || sc.scatter_ctas_per_sm < 1 || sc.scatter_ctas_per_sm > 8 || sc.g2p_tight < 0 || sc.g2p_tight > 3)
            return arg("schedule: unknown P2G form, (chunk, buffers) pair or G2P width, or CTAs per SM outside [1, 8]");
        sched_ = sc;
        if (sc.fused) {
            sched_.chunk = sc.fused == 3 ? WsShape<T>::CHUNK : FUSED_CH[fused_variant(sc.fused)];
            sched_.buffers = sc.fused == 3 ? WsShape<T>::NSTAGE : 0;
        }
        sched_.tuned = 0;
        fixed_schedule_ = true; // explicit schedules are not overridden by the autotuner
        drop_graphs();
        return 0;
    }

private:
    int dev_ = 0, nsm_ = 0;
    cudaStream_t stream_ = nullptr;
    int init_err_ = 0;
    std::string err_;
    std::vector<SceneParams<T>> h_scenes_;
    SceneParams<T>* d_scenes_ = nullptr;
    uint32_t N_ = 0;
    uint64_t cap_ = 0; // particle capacity of the buffers (the pool's field stride)
    size_t scene_cap_ = 0;
    KeyLayout kl_{};
    T* pool_[2] = { nullptr, nullptr };
    uint32_t* pid_[2] = { nullptr, nullptr };
    int cur_ = 0;
    uint64_t *keys_in_ = nullptr, *keys_sorted_ = nullptr;
    uint32_t *iota_ = nullptr, *vals_sorted_ = nullptr, *g_start_ = nullptr;
    int32_t* g_nbr_ = nullptr;
    uint64_t* b_key_ = nullptr;
    T *acc_ = nullptr, *vel_ = nullptr;
    uint64_t* h_keys_ = nullptr;
    int32_t* h_vals_ = nullptr;
    uint32_t h_mask_ = 0, b_cap_ = 0;
    double* grid_mass_ = nullptr;
    DevStatus* st_ = nullptr;
    DevStatus* hst_ = nullptr;
    void *sort_tmp_ = nullptr, *stage_ = nullptr;
    size_t sort_bytes_ = 0, stage_bytes_ = 0;
    int occ_stress_[4] = { 1, 1, 1, 1 }, occ_scatter_[3] = { 1, 1, 1 }, occ_g2p_[4][3] = { { 1, 1, 1 }, { 1, 1, 1 }, { 1, 1, 1 }, { 1, 1, 1 } };
    int occ_fused_[2][4] = { { 1, 1, 1, 1 }, { 1, 1, 1, 1 } }; // [fused variant][model set]
    int occ_ws_[4] = { 1, 1, 1, 1 }; // warp-specialised P2G, per model set
    int occ_grid_ = 1; // grid update CTAs per SM
    int64_t stream_reruns_ = 0; // stream_steps jobs run again the safe way after an abort
    int models_ = 7; // bit m set: a material of model m (corotated, Neo-Hookean Borden, QR-stable Neo-Hookean) is present
    bool any_damage_ = false;
    bool implicit_ = false; // some scene solves its damage implicitly
    bool drive_stale_ = true; // P_DRV must be refilled from F before the next substep
    T* cg_ = nullptr; // the damage solve's node vectors (CG_NF x b_cap_ blocks), allocated when implicit_
    CgScalars* cgs_ = nullptr; // per scene (scene_cap_)
    cudaStream_t side_ = nullptr; // captures the damage solve's loop body
    // stream_steps: two device slots for inputs and two for outputs, the copy streams and their events
    void* io_in_[2] = { nullptr, nullptr };
    void* io_out_[2] = { nullptr, nullptr };
    size_t io_bytes_ = 0;
    cudaStream_t h2d_ = nullptr, d2h_ = nullptr;
    cudaEvent_t io_ev_[8] = {};
    cudaGraphExec_t cg_exec_ = nullptr; // the damage solve's loop alone, for substeps launched outside graphs
    int occ_dmg_[2] = { 1, 1 };
    uint32_t* inv_ = nullptr; // storage slot of each particle of a scene in the caller's order (row transfers)
    uint64_t inv_cap_ = 0;
    T* pay_ = nullptr;
    int64_t pstride_ = 0;
    Schedule sched_{ 0, VAR_CHUNK[0], VAR_NBUF[0], 2, 128, 0, 0 };
    int autotune_mode_ = 1; // 0 off (defaults), 1 on (cached), 2 always re-tune on a new batch
    bool tuned_ = false;
    bool fixed_schedule_ = false;
    bool sorted_storage_ = false; // particles sit in the sorted order of their last substep (after one G2P)
    // incremental sort: keys_sorted_ holds the keys the current storage order was sorted by (false after state
    // writes, aborts and autotuner trials: the next substep sorts in full)
    bool sort_base_stale_ = true;
    bool inc_sort_on_ = true; // ZR_SORT=full turns the incremental sort off
    bool prefetch_ = true; // P2G's L2 prefetch of the groups ahead (ZR_PREFETCH=0 turns it off)
    static constexpr int64_t MCAP_MIN = 4096;
    // the sort's tile arrays (stayer bits, per-tile counts and keys, bucket counts, group-head look-back words);
    // the movers' list, buckets and tickets, and their keys and storage indices grouped by bucket
    unsigned char* sort_aux_ = nullptr;
    uint32_t *inc_move_ = nullptr, *inc_bkey_ = nullptr, *inc_bidx_ = nullptr; // mover list; movers by bucket (fixed slots)
    int64_t mcap_ = 0; // movers the incremental sort takes per substep
    void *ck_pool_ = nullptr, *ck_pid_ = nullptr, *ck_scenes_ = nullptr; // device checkpoint
    uint64_t ck_cap_ = 0;
    size_t ck_scenes_n_ = 0;
    bool ck_valid_ = false;
    std::vector<SceneParams<T>> ck_host_scenes_;
    void* scenes_backup_ = nullptr;
    size_t scenes_backup_bytes_ = 0;
    bool graphs_on_ = true, timing_ = false;
    cudaGraphExec_t g1_[2] = { nullptr, nullptr }, gk_[2] = { nullptr, nullptr };
    int launches_per_step_ = 0;
    std::vector<cudaEvent_t> ev_;
    cudaEvent_t t0_ = nullptr, t1_ = nullptr;
    KernelTimes kt_;
    int64_t dev_bytes_ = 0;

    Pool<T> pool(int which) const { return Pool<T>{ pool_[which], pid_[which], (int64_t)cap_ }; }

    // radix sort of the n keys in keys_in_ (32- or 64-bit words, as the key layout says) with their storage
    // indices; stable, so particles of one cell keep their storage order
    cudaError_t sort_keys(int64_t n)
    {
        if (kl_.wide)
            return cub::DeviceRadixSort::SortPairs(sort_tmp_, sort_bytes_, keys_in_, keys_sorted_, iota_, vals_sorted_, n, 0, kl_.total(), stream_);
        return cub::DeviceRadixSort::SortPairs(sort_tmp_, sort_bytes_, (uint32_t*)keys_in_, (uint32_t*)keys_sorted_, iota_, vals_sorted_, n, 0,
            kl_.total(), stream_);
    }

    // tiles of the sort and of the group-head pass (SORT_TILE keys each) for up to cap particles
    static int64_t sort_tiles(int64_t n) { return std::max<int64_t>(1, (n + SORT_TILE - 1) / SORT_TILE); }
    // movers' fixed bucket slots: SORT_MAXM per tile
    static int64_t bucket_slots(int64_t cap) { return sort_tiles(cap) * SORT_MAXM; }
    // sort_aux_: [zeroed every substep: movers found (i64), unused (3 x i64), b_cnt, b_max (tiles u32 each)]
    // [stay bits: ceil(cap/32) u32][t_stay, t_first, t_last, t_base, t_heads: tiles u32 each][look-back: tiles + 1 u64]
    static size_t sort_zero_bytes(int64_t cap) { return 32 + 8 * (size_t)sort_tiles(cap); }
    static size_t sort_aux_words(int64_t cap) { return sort_zero_bytes(cap) / 4 + (size_t)((cap + 31) / 32) + 5 * (size_t)sort_tiles(cap) + 1; }
    static size_t sort_aux_bytes(int64_t cap) { return 4 * sort_aux_words(cap) + 8 * ((size_t)sort_tiles(cap) + 2); }
    uint64_t* lookback_words() const
    {
        const size_t off = (4 * sort_aux_words((int64_t)cap_) + 7) & ~(size_t)7;
        return reinterpret_cast<uint64_t*>(sort_aux_ + off);
    }
    bool inc_sort_usable() const { return inc_sort_on_ && !kl_.wide && kl_.total() <= 31 && inc_move_; }

    // The sorted keys and storage indices of keys_in_ from the previous substep's sorted keys (keys_sorted_), by
    // the hand-written kernels of the incremental sort (stayers in place, movers bucketed by stayer tile and merged),
    // then the group heads placed and their blocks activated (k_heads_activate).
    // ev_sorted (may be null) is recorded between the merge and the head placement.
    cudaError_t sort_and_activate_incremental(int64_t n, const StepArgs<T>& a, cudaEvent_t ev_sorted)
    {
        const uint32_t* nk = (const uint32_t*)keys_in_;
        const uint32_t* ok = (const uint32_t*)keys_sorted_;
        SortBufs sb;
        const int64_t tiles = sort_tiles(n), tcap = sort_tiles((int64_t)cap_);
        sb.cnt = reinterpret_cast<int64_t*>(sort_aux_);
        sb.b_cnt = reinterpret_cast<uint32_t*>(sort_aux_ + 32);
        sb.b_max = sb.b_cnt + tcap;
        sb.stay_bits = sb.b_max + tcap;
        sb.t_stay = sb.stay_bits + (cap_ + 31) / 32;
        sb.t_first = sb.t_stay + tcap;
        sb.t_last = sb.t_first + tcap;
        sb.t_base = sb.t_last + tcap;
        sb.t_heads = sb.t_base + tcap;
        sb.m_idx = inc_move_;
        sb.b_key = inc_bkey_;
        sb.b_idx = inc_bidx_;
        sb.mcap = mcap_;
        sb.n = n;
        sb.tiles = (int)tiles;
        cudaError_t e = cudaMemsetAsync(sort_aux_, 0, sort_zero_bytes((int64_t)cap_), stream_);
        if (e != cudaSuccess) return e;
        const int mgrid = (int)std::max<int64_t>(1, std::min<int64_t>(nsm_ * 4, (mcap_ + SORT_NT - 1) / SORT_NT));
        k_sort_tiles<<<(unsigned)tiles, SORT_NT, 0, stream_>>>(nk, ok, sb, st_);
        k_sort_bucket<<<mgrid, SORT_NT, 0, stream_>>>(nk, sb, st_);
        k_sort_merge<<<(unsigned)tiles, SORT_NT, 0, stream_>>>(nk, sb, (uint32_t*)keys_sorted_, vals_sorted_, kl_, st_);
        if (ev_sorted && (e = cudaEventRecord(ev_sorted, stream_)) != cudaSuccess) return e;
        k_heads_activate<T><<<(unsigned)tiles, SORT_NT, 0, stream_>>>(a, sb, g_start_, (uint32_t)cap_);
        return cudaGetLastError();
    }

    // first sorted index of every (scene, page) into g_start_, their number into st_->n_groups
    cudaError_t group_heads(int64_t n)
    {
        const int64_t tiles = sort_tiles(n);
        uint64_t* lb = lookback_words();
        cudaError_t e = cudaMemsetAsync(lb, 0, 8 * ((size_t)tiles + 1), stream_);
        if (e != cudaSuccess) return e;
        k_group_heads<<<(unsigned)tiles, SORT_NT, 0, stream_>>>(keys_sorted_, n, kl_, lb, reinterpret_cast<uint32_t*>(lb + tiles), g_start_,
            (uint32_t)cap_, st_);
        return cudaGetLastError();
    }

    int params_from_desc(const SceneDesc& sdr, SceneParams<T>& sp)
    {
        const SceneDesc* sd = &sdr;
        if (sd->n <= 0) return arg("scene without particles");
        if (sd->n >= (int64_t)(1u << L::index_bits)) return arg("too many particles in one scene for the SPGrid key (limit 2^" + std::to_string(L::index_bits) + ")");
        if ((int)sd->materials.size() > MAX_MATERIALS || sd->materials.empty()) return arg("a scene needs 1.." + std::to_string(MAX_MATERIALS) + " materials");
        if ((int)sd->objects.size() > MAX_OBJECTS) return arg("at most " + std::to_string(MAX_OBJECTS) + " collision objects per scene");
        if (!(sd->dx > 0) || !(sd->dt > 0)) return arg("dx and dt must be positive");
        int dc = sd->domain_cells > 0 ? sd->domain_cells : 4096 - 8;
        if (dc > 4096 - 8 || dc < 8) return arg("domain_cells must be in [8, 4088]");
        std::memset(&sp, 0, sizeof sp);
        sp.dx = (T)sd->dx;
        sp.inv_dx = (T)1 / sp.dx; // BSplineWeights one_over_dx(1 / dx) (MpmGrid.h:69)
        sp.dt = (T)sd->dt;
        T dx2 = sp.dx * sp.dx;
        sp.D_inv = (T)4 / dx2;
        for (int c = 0; c < 3; c++) sp.gravity[c] = (T)sd->gravity[c];
        T r = (T)sd->apic_rpic_ratio;
        sp.apic_a = (r + 1) * (T)0.5;
        sp.apic_b = (r - 1) * (T)0.5;
        sp.cfl = (T)sd->cfl;
        sp.time = sd->time;
        sp.count = sd->n;
        sp.domain_cells = dc;
        sp.n_objects = (int)sd->objects.size();
        sp.n_materials = (int)sd->materials.size();
        sp.damage = 0;
        for (int k = 0; k < sp.n_materials; k++) {
            const auto& m = sd->materials[k];
            Material<T>& mt = sp.materials[k];
            T E = (T)m.E, nu = (T)m.nu;
            mt.model = m.model;
            mt.damage = m.damage;
            mt.lambda = E * nu / (((T)1 + nu) * ((T)1 - (T)2 * nu)); // CorotatedElasticity.cpp:16-21
            mt.mu = E / ((T)2 * ((T)1 + nu));
            mt.kappa = (T).666666 * mt.mu + mt.lambda; // NeoHookeanBorden.cpp:20
            mt.kx = (T)m.kx_scale * mt.mu; // QRStableNeoHookean::setExtraFiberStiffness (QRStableNeoHookean.h:98-107)
            mt.ky = (T)m.ky_scale * mt.mu;
            mt.alpha = (T)m.alpha;
            mt.l0 = (T)m.l0;
            mt.eta = (T)m.eta;
            mt.zeta = (T)m.zeta;
            mt.residual = (T)m.residual;
            if (m.damage) sp.damage = 1;
        }
        // the implicit solve replaces the explicit damage update (AnisoFractureSimulation.h:343-352 picks one)
        sp.implicit = (sd->implicit_damage && sp.damage) ? 1 : 0;
        for (int k = 0; k < sp.n_objects; k++) {
            const auto& o = sd->objects[k];
            double nn = std::sqrt(o.normal[0] * o.normal[0] + o.normal[1] * o.normal[1] + o.normal[2] * o.normal[2]);
            if (!(nn > 0)) return arg("half-space normal must be non-zero");
            if (o.type < 1 || o.type > 3) return arg("collision type must be STICKY(1), SLIP(2) or SEPARATE(3)");
            HalfSpaceObj<T>& h = sp.objects[k];
            for (int c = 0; c < 3; c++) {
                h.origin[c] = (T)o.origin[c];
                h.normal[c] = (T)(o.normal[c] / nn); // AnalyticLevelSet.cpp:318-323 normalises
                h.vel[c] = (T)o.vel[c];
            }
            h.friction = (T)o.friction;
            h.type = o.type;
        }
        return 0;
    }

    // host arrays of one scene -> storage slots [first, first + n) of particle buffer `which`
    int upload_scene(const SceneDesc& sd, int64_t first, int which, uint8_t* d_mat, std::vector<T>& buf)
    {
        const int64_t cnt = sd.n, stride = (int64_t)cap_;
        if ((int64_t)sd.x.size() != 3 * cnt || (int64_t)sd.m.size() != cnt || (int64_t)sd.V0.size() != cnt) return arg("x, m, V0 are required");
        if (!sd.v.empty() && (int64_t)sd.v.size() != 3 * cnt) return arg("v must have 3n values");
        if (!sd.F.empty() && (int64_t)sd.F.size() != 9 * cnt) return arg("F must have 9n values");
        if (!sd.C.empty() && (int64_t)sd.C.size() != 9 * cnt) return arg("C must have 9n values");
        if (!sd.d.empty() && (int64_t)sd.d.size() != cnt) return arg("d must have n values");
        if (!sd.sigma_c.empty() && (int64_t)sd.sigma_c.size() != cnt) return arg("sigma_c must have n values");
        if (!sd.dtilde_max.empty() && (int64_t)sd.dtilde_max.size() != cnt) return arg("dtilde_max must have n values");
        auto put = [&](int f0, int nc, const std::vector<double>& src, double dflt_diag, double dflt) -> int {
            buf.resize(cnt);
            for (int c = 0; c < nc; c++) {
                for (int64_t i = 0; i < cnt; i++)
                    buf[i] = !src.empty() ? (T)src[(size_t)i * nc + c] : (T)((nc == 9 && (c % 4) == 0) ? dflt_diag : dflt);
                ZR_CUDA(cudaMemcpy(pool_[which] + (size_t)(f0 + c) * stride + first, buf.data(), sizeof(T) * cnt, cudaMemcpyHostToDevice));
            }
            return 0;
        };
        int rc;
        if ((rc = put(P_X, 3, sd.x, 0, 0)) || (rc = put(P_V, 3, sd.v, 0, 0)) || (rc = put(P_C, 9, sd.C, 0, 0)) || (rc = put(P_F, 9, sd.F, 1, 0))
            || (rc = put(P_M, 1, sd.m, 0, 0)) || (rc = put(P_V0, 1, sd.V0, 0, 0)) || (rc = put(P_D, 1, sd.d, 0, 0)) || (rc = put(P_SC, 1, sd.sigma_c, 1, 1))
            || (rc = put(P_MDT, 1, sd.dtilde_max, 0, 0)))
            return rc;
        const uint8_t* mp = nullptr;
        if (!sd.material.empty()) {
            if ((int64_t)sd.material.size() != cnt) return arg("material must have n values");
            for (auto mm : sd.material)
                if ((int)mm >= (int)sd.materials.size()) return arg("material index out of range");
            ZR_CUDA(cudaMemcpy(d_mat, sd.material.data(), cnt, cudaMemcpyHostToDevice));
            mp = d_mat;
        }
        k_iota_pid<T><<<nsm_ * 4, 256, 0, stream_>>>(pid_[which], mp, first, cnt);
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    int arg(const std::string& m) { return fail(ZR_ERR_ARG_, m); }
    int fail(int code, const std::string& m)
    {
        err_ = m;
        return code;
    }

    void init_device()
    {
        if (cudaGetDevice(&dev_) != cudaSuccess || cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_) != cudaSuccess) {
            init_err_ = fail(ZR_ERR_CUDA_, "no CUDA device");
            return;
        }
        if (cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking) != cudaSuccess || cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess
            || cudaMallocHost((void**)&hst_, sizeof(DevStatus)) != cudaSuccess
            || cudaEventCreate(&t0_) != cudaSuccess || cudaEventCreate(&t1_) != cudaSuccess) {
            init_err_ = fail(ZR_ERR_CUDA_, "stream/pinned allocation failed");
            return;
        }
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_dmg_[0], k_dmg_rhs<T>, DmgShape<T>::NT, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_dmg_[1], k_dmg_apply<T>, DmgShape<T>::NT, 0);
        occ_dmg_[0] = std::max(1, occ_dmg_[0]);
        occ_dmg_[1] = std::max(1, occ_dmg_[1]);
        scatter_setup<0>();
        scatter_setup<1>();
        scatter_setup<2>();
        fused_setup_all<0>();
        fused_setup_all<1>();
        ws_setup<1>(0);
        ws_setup<2>(1);
        ws_setup<4>(2);
        ws_setup<7>(3);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_stress_[0], k_stress<T, 1>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_stress_[1], k_stress<T, 2>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_stress_[2], k_stress<T, 4>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_stress_[3], k_stress<T, 7>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_grid_, k_grid<T>, GRID_NT, 0);
        occ_grid_ = std::max(1, occ_grid_);
        g2p_setup<0, 0>();
        g2p_setup<0, 1>();
        g2p_setup<0, 2>();
        g2p_setup<1, 0>();
        g2p_setup<1, 1>();
        g2p_setup<1, 2>();
        g2p_setup<2, 0>();
        g2p_setup<2, 1>();
        g2p_setup<2, 2>();
        g2p_setup<3, 0>();
        g2p_setup<3, 1>();
        g2p_setup<3, 2>();
        for (int& o : occ_scatter_) o = std::max(1, o);
        for (int& o : occ_stress_) o = std::max(1, o);
        for (auto& row : occ_g2p_)
            for (int& o : row) o = std::max(1, o);
        sched_.scatter_ctas_per_sm = occ_scatter_[0];
        sched_.tuned = 0;
        if (const char* e = std::getenv("ZR_AUTOTUNE")) autotune_mode_ = std::atoi(e);
        if (const char* e = std::getenv("ZR_SORT")) inc_sort_on_ = std::string(e) != "full";
        if (const char* e = std::getenv("ZR_PREFETCH")) prefetch_ = std::atoi(e) != 0;
    }

    int alloc(void** p, size_t bytes)
    {
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            *p = nullptr;
            err_ = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
            return ZR_ERR_CUDA_;
        }
        dev_bytes_ += (int64_t)bytes;
        return 0;
    }
    int cuda_fail(cudaError_t e)
    {
        err_ = std::string("CUDA error: ") + cudaGetErrorString(e);
        return ZR_ERR_CUDA_;
    }
    void dfree(void*& p)
    {
        if (p) cudaFree(p);
        p = nullptr;
    }

    int alloc_grid(uint32_t cap)
    {
        drop_graphs();
        void* p;
        p = g_nbr_;
        dfree(p);
        p = b_key_;
        dfree(p);
        p = acc_;
        dfree(p);
        p = vel_;
        dfree(p);
        p = h_keys_;
        dfree(p);
        p = h_vals_;
        dfree(p);
        p = cg_;
        dfree(p);
        cg_ = nullptr;
        g_nbr_ = nullptr;
        b_key_ = nullptr;
        acc_ = vel_ = nullptr;
        h_keys_ = nullptr;
        h_vals_ = nullptr;
        b_cap_ = cap;
        uint32_t hs = 1;
        while (hs < 4 * cap) hs <<= 1;
        h_mask_ = hs - 1;
        if (alloc((void**)&g_nbr_, 32 * (size_t)cap) || alloc((void**)&b_key_, 8 * (size_t)cap) || alloc((void**)&acc_, sizeof(T) * (size_t)cap * NACC * L::nodes)
            || alloc((void**)&vel_, sizeof(T) * (size_t)cap * NVEL * L::nodes) || alloc((void**)&h_keys_, 8 * (size_t)hs) || alloc((void**)&h_vals_, 4 * (size_t)hs))
            return ZR_ERR_CUDA_;
        ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)cap * NACC * L::nodes, stream_));
        ZR_CUDA(cudaMemsetAsync(vel_, 0, sizeof(T) * (size_t)cap * NVEL * L::nodes, stream_));
        ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)hs, stream_));
        return ensure_cg();
    }

    int ensure_stage(size_t bytes)
    {
        if (bytes <= stage_bytes_) return 0;
        dfree(stage_);
        if (alloc(&stage_, bytes)) return ZR_ERR_CUDA_;
        stage_bytes_ = bytes;
        return 0;
    }

    int rekey()
    {
        sorted_storage_ = false; // new positions: the storage order may no longer follow the cells
        // the sort base (keys_sorted_) stays a sorted array of the same keys' layout, which is all the incremental
        // sort needs to be correct: particles whose key matches it at their slot form a sorted subsequence
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        k_keys<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), d_scenes_, n_scenes(), keys_in_, N_, kl_, st_);
        ZR_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        if (hst_->flags & FLAG_OUT_OF_DOMAIN) return fail(ZR_ERR_OUT_OF_DOMAIN_, "a particle lies outside its scene's domain");
        return 0;
    }

    static bool field_range(int field, int& f0, int& nc)
    {
        switch (field) {
        case FIELD_X: f0 = P_X; nc = 3; return true;
        case FIELD_V: f0 = P_V; nc = 3; return true;
        case FIELD_C: f0 = P_C; nc = 9; return true;
        case FIELD_F: f0 = P_F; nc = 9; return true;
        case FIELD_D: f0 = P_D; nc = 1; return true;
        case FIELD_M: f0 = P_M; nc = 1; return true;
        case FIELD_V0: f0 = P_V0; nc = 1; return true;
        case FIELD_SIGMA_C: f0 = P_SC; nc = 1; return true;
        case FIELD_DTILDE_MAX: f0 = P_MDT; nc = 1; return true;
        }
        return false;
    }

    StepArgs<T> args(int parity) const
    {
        StepArgs<T> a;
        a.keys_sorted = keys_sorted_;
        a.vals_sorted = vals_sorted_;
        a.keys_next = keys_in_;
        a.pin = pool(parity);
        a.pout = pool(parity ^ 1);
        a.g_start = g_start_;
        a.g_nbr = g_nbr_;
        a.pay = pay_;
        a.pstride = pstride_;
        a.cg = cg_;
        a.cgs = cgs_;
        a.b_key = b_key_;
        a.acc = acc_;
        a.vel = vel_;
        a.h_keys = h_keys_;
        a.h_vals = h_vals_;
        a.h_mask = h_mask_;
        a.scenes = d_scenes_;
        a.grid_mass = grid_mass_;
        a.st = st_;
        a.n_total = N_;
        a.b_cap = b_cap_;
        a.n_scenes = n_scenes();
        a.opts = prefetch_ ? OPT_PREFETCH : 0u;
        a.kl = kl_;
        return a;
    }

    // Enqueue one substep reading buffer `parity`. With ev != nullptr, events are recorded between the
    // phases (sort | group heads, activate, neighbour slots | p2g | grid | g2p+end).
    int enqueue_step(int parity, cudaEvent_t* ev, bool full_sort = false)
    {
        StepArgs<T> a = args(parity);
        const int64_t n = N_;
        if (ev) ZR_CUDA(cudaEventRecord(ev[0], stream_));
        if (full_sort || !inc_sort_usable()) {
            ZR_CUDA(sort_keys(n));
            if (ev) ZR_CUDA(cudaEventRecord(ev[1], stream_));
            ZR_CUDA(group_heads(n));
            k_activate<T><<<nsm_ * 4, 256, 0, stream_>>>(a);
        }
        else // its last kernel places the group heads and activates their blocks (after ev[1]: the activate phase)
            ZR_CUDA(sort_and_activate_incremental(n, a, ev ? ev[1] : nullptr));
        if (sched_.fused == 0 || sched_.fused == 3) // these P2G forms read grid slots; the fused one translates its groups' entries
            k_nbr<T><<<nsm_ * 4, 256, 0, stream_>>>(a);
        if (ev) ZR_CUDA(cudaEventRecord(ev[2], stream_));
        if (sched_.fused == 3)
            launch_ws(a, nsm_ * std::min(sched_.scatter_ctas_per_sm, occ_ws_[models_slot()]));
        else if (sched_.fused) {
            const int fv = fused_variant(sched_.fused);
            const int fctas = nsm_ * std::min(sched_.scatter_ctas_per_sm, occ_fused_[fv][models_slot()]);
            if (fv == 0)
                launch_fused<0>(a, fctas);
            else
                launch_fused<1>(a, fctas);
        }
        else {
            const int ms = models_slot();
            if (ms == 0)
                k_stress<T, 1><<<nsm_ * occ_stress_[0], 256, 0, stream_>>>(a);
            else if (ms == 1)
                k_stress<T, 2><<<nsm_ * occ_stress_[1], 256, 0, stream_>>>(a);
            else if (ms == 2)
                k_stress<T, 4><<<nsm_ * occ_stress_[2], 256, 0, stream_>>>(a);
            else
                k_stress<T, 7><<<nsm_ * occ_stress_[3], 256, 0, stream_>>>(a);
            const int vi = std::max(0, variant_index(sched_.chunk, sched_.buffers));
            const int sctas = nsm_ * std::min(sched_.scatter_ctas_per_sm, occ_scatter_[vi]);
            if (vi == 0)
                launch_scatter<0>(a, sctas);
            else if (vi == 1)
                launch_scatter<1>(a, sctas);
            else
                launch_scatter<2>(a, sctas);
        }
        if (ev) ZR_CUDA(cudaEventRecord(ev[3], stream_));
        k_grid<T><<<nsm_ * occ_grid_, GRID_NT, 0, stream_>>>(a); // one resident wave, striding over the blocks
        if (implicit_) {
            int rc = enqueue_damage_solve(a);
            if (rc) return rc;
        }
        if (ev) ZR_CUDA(cudaEventRecord(ev[4], stream_));
        const int gi = std::max(0, g2p_index(sched_.g2p_threads));
        switch (sched_.g2p_tight) {
        case 1: launch_g2p<1>(a, gi); break;
        case 2: launch_g2p<2>(a, gi); break;
        case 3: launch_g2p<3>(a, gi); break;
        default: launch_g2p<0>(a, gi);
        }
        k_step_end<T><<<1, 256, 0, stream_>>>(d_scenes_, n_scenes(), st_);
        if (ev) ZR_CUDA(cudaEventRecord(ev[5], stream_));
        ZR_CUDA(cudaGetLastError());
        return 0;
    }

    // Implicit damage solve of the substep (AnisoFractureSimulation.h:437-626): D~ history and coefficients,
    // right-hand side and preconditioner sums, CG initialisation, the iterations, the nodal change for G2P.
    int enqueue_damage_solve(const StepArgs<T>& a)
    {
        ZR_CUDA(cudaMemsetAsync(cgs_, 0, sizeof(CgScalars) * h_scenes_.size(), stream_));
        k_dmg_prep<T><<<nsm_ * 8, 256, 0, stream_>>>(a);
        k_dmg_rhs<T><<<nsm_ * occ_dmg_[0], DmgShape<T>::NT, 0, stream_>>>(a);
        k_cg_nodes<T, 0><<<nsm_ * 8, 256, 0, stream_>>>(a);
        k_cg_scalars<T, 0><<<1, 256, 0, stream_>>>(a, n_scenes(), cudaGraphConditionalHandle{});
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        ZR_CUDA(cudaStreamIsCapturing(stream_, &cs));
        if (cs == cudaStreamCaptureStatusActive) {
            int rc = capture_cg_loop(a);
            if (rc) return rc;
        }
        else {
            if (!cg_exec_) {
                cudaGraph_t g;
                ZR_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                int rc = capture_cg_loop(a);
                cudaError_t e = cudaStreamEndCapture(stream_, &g);
                if (rc) return rc;
                if (e != cudaSuccess) return fail(ZR_ERR_CUDA_, std::string("damage solve capture: ") + cudaGetErrorString(e));
                e = cudaGraphInstantiate(&cg_exec_, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return fail(ZR_ERR_CUDA_, std::string("damage solve instantiate: ") + cudaGetErrorString(e));
            }
            ZR_CUDA(cudaGraphLaunch(cg_exec_, stream_));
        }
        k_cg_nodes<T, 4><<<nsm_ * 8, 256, 0, stream_>>>(a);
        return 0;
    }

    // Append the CG iterations to the capture under way on stream_: a conditional WHILE node whose body (one
    // iteration) is captured on the side stream; the body's last kernel sets the condition and ends the loop
    // after at most CG_MAX_ITERATIONS + 1 passes.
    int capture_cg_loop(const StepArgs<T>& a)
    {
        cudaStreamCaptureStatus cs;
        cudaGraph_t g;
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* edges = nullptr;
        size_t nd = 0;
        ZR_CUDA(cudaStreamGetCaptureInfo(stream_, &cs, nullptr, &g, &deps, &edges, &nd));
        cudaGraphConditionalHandle h;
        ZR_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {}; // reserved fields zero
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        ZR_CUDA(cudaGraphAddNode(&node, g, deps, edges, nd, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        ZR_CUDA(cudaStreamUpdateCaptureDependencies(stream_, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        ZR_CUDA(cudaStreamBeginCaptureToGraph(side_, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        k_dmg_apply<T><<<nsm_ * occ_dmg_[1], DmgShape<T>::NT, 0, side_>>>(a);
        k_cg_nodes<T, 1><<<nsm_ * 8, 256, 0, side_>>>(a);
        k_cg_nodes<T, 2><<<nsm_ * 8, 256, 0, side_>>>(a);
        k_cg_nodes<T, 3><<<nsm_ * 8, 256, 0, side_>>>(a);
        k_cg_scalars<T, 1><<<1, 256, 0, side_>>>(a, n_scenes(), h);
        cudaGraph_t out = nullptr;
        const cudaError_t le = cudaGetLastError();
        ZR_CUDA(cudaStreamEndCapture(side_, &out));
        ZR_CUDA(le);
        return 0;
    }

    // the damage solve's vectors and scalars (the vectors follow the grid's block capacity)
    int ensure_cg()
    {
        if (!implicit_ || cg_) return 0;
        const size_t bytes = sizeof(T) * CG_NF * (size_t)b_cap_ * L::nodes;
        if (alloc((void**)&cg_, bytes)) return ZR_ERR_CUDA_;
        ZR_CUDA(cudaMemsetAsync(cg_, 0, bytes, stream_));
        return 0;
    }

    int build_graph(int parity, int nsub, cudaGraphExec_t* out)
    {
        cudaGraph_t g;
        ZR_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        int rc = 0;
        for (int s = 0; s < nsub && !rc; s++) rc = enqueue_step(parity ^ (s & 1), nullptr);
        cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (rc) return rc;
        if (e != cudaSuccess) return fail(ZR_ERR_CUDA_, std::string("graph capture: ") + cudaGetErrorString(e));
        if (nsub == 1) {
            size_t nn = 0;
            cudaGraphGetNodes(g, nullptr, &nn);
            launches_per_step_ = 0;
            std::vector<cudaGraphNode_t> nodes(nn);
            cudaGraphGetNodes(g, nodes.data(), &nn);
            for (auto& nd : nodes) {
                cudaGraphNodeType t;
                cudaGraphNodeGetType(nd, &t);
                if (t == cudaGraphNodeTypeKernel) launches_per_step_++;
            }
        }
        e = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(ZR_ERR_CUDA_, std::string("graph instantiate: ") + cudaGetErrorString(e));
        return 0;
    }

    void drop_graphs()
    {
        if (cg_exec_) cudaGraphExecDestroy(cg_exec_);
        cg_exec_ = nullptr;
        for (int p = 0; p < 2; p++) {
            if (g1_[p]) cudaGraphExecDestroy(g1_[p]);
            if (gk_[p]) cudaGraphExecDestroy(gk_[p]);
            g1_[p] = gk_[p] = nullptr;
        }
    }

    // Substeps from buffer cur_. The first one sorts in full when the sort base is stale; the others (and the
    // captured graphs) sort incrementally.
    int launch_steps(int nsteps)
    {
        if (timing_ && (int)ev_.size() < 6 * nsteps) {
            size_t old = ev_.size();
            ev_.resize(6 * (size_t)nsteps);
            for (size_t i = old; i < ev_.size(); i++) ZR_CUDA(cudaEventCreate(&ev_[i]));
        }
        int s0 = 0;
        if (nsteps > 0 && sort_base_stale_) {
            int rc = enqueue_step(cur_ & 1, timing_ ? &ev_[0] : nullptr, true);
            if (rc) return rc;
            s0 = 1;
        }
        if (timing_ || !graphs_on_) {
            for (int s = s0; s < nsteps; s++) {
                int rc = enqueue_step((cur_ + s) & 1, timing_ ? &ev_[6 * (size_t)s] : nullptr);
                if (rc) return rc;
            }
            return 0;
        }
        int rc = prepare_graphs(nsteps - s0);
        if (rc) return rc;
        int par = (cur_ + s0) & 1;
        int s = s0;
        if (nsteps - s0 >= GRAPH_K)
            for (; s + GRAPH_K <= nsteps; s += GRAPH_K) ZR_CUDA(cudaGraphLaunch(gk_[par], stream_)); // GRAPH_K even: parity unchanged
        for (; s < nsteps; s++) {
            ZR_CUDA(cudaGraphLaunch(g1_[par], stream_));
            par ^= 1;
        }
        return 0;
    }

    // capture the 1-substep graphs (both buffer parities) and, for long runs, the GRAPH_K-substep graphs
    int prepare_graphs(int nsteps)
    {
        for (int p = 0; p < 2; p++)
            if (!g1_[p]) {
                int rc = build_graph(p, 1, &g1_[p]);
                if (rc) return rc;
            }
        if (nsteps >= GRAPH_K)
            for (int p = 0; p < 2; p++)
                if (!gk_[p]) {
                    int rc = build_graph(p, GRAPH_K, &gk_[p]);
                    if (rc) return rc;
                }
        return 0;
    }

    static int variant_index(int chunk, int buffers)
    {
        for (int v = 0; v < 3; v++)
            if (VAR_CHUNK[v] == chunk && VAR_NBUF[v] == buffers) return v;
        return -1;
    }
    template <int V>
    void scatter_setup()
    {
        using S = ScatterShape<T, VAR_CHUNK[V], VAR_NBUF[V]>;
        auto k = k_scatter<T, VAR_CHUNK[V], VAR_NBUF[V]>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::dyn_bytes);
        // the staging buffers are the point: ask for the largest shared-memory carveout
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_scatter_[V], k, S::NT, S::dyn_bytes);
    }
    // G2P variant R = g2p_tight: bit 0 the register budget (G2P_RES), bit 1 the halo staged by bulk copies
    template <int R, int N>
    void g2p_setup()
    {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_g2p_[R][N], k_g2p<T, G2P_NT[N], G2P_RES[R & 1], (R >> 1) != 0>, G2P_NT[N], 0);
    }
    template <int R>
    void launch_g2p(const StepArgs<T>& a, int gi)
    {
        constexpr int RES = G2P_RES[R & 1];
        constexpr bool BULK = (R >> 1) != 0;
        if (gi == 0)
            k_g2p<T, G2P_NT[0], RES, BULK><<<nsm_ * occ_g2p_[R][0], G2P_NT[0], 0, stream_>>>(a);
        else if (gi == 1)
            k_g2p<T, G2P_NT[1], RES, BULK><<<nsm_ * occ_g2p_[R][1], G2P_NT[1], 0, stream_>>>(a);
        else
            k_g2p<T, G2P_NT[2], RES, BULK><<<nsm_ * occ_g2p_[R][2], G2P_NT[2], 0, stream_>>>(a);
    }
    template <int M, int V>
    void fused_setup(int slot)
    {
        using FS = FusedShape<T, FUSED_CH[V]>;
        auto k = k_p2g_fused<T, M, FUSED_MINB[V], FUSED_CH[V]>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FS::dyn_bytes);
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_fused_[V][slot], k, FS::NT, FS::dyn_bytes);
        occ_fused_[V][slot] = std::max(1, occ_fused_[V][slot]);
    }
    template <int V>
    void fused_setup_all()
    {
        fused_setup<1, V>(0);
        fused_setup<2, V>(1);
        fused_setup<4, V>(2);
        fused_setup<7, V>(3);
    }
    template <int M>
    void ws_setup(int slot)
    {
        auto k = k_p2g_ws<T, M>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WsShape<T>::dyn_bytes);
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_ws_[slot], k, WsShape<T>::NT, WsShape<T>::dyn_bytes);
        occ_ws_[slot] = std::max(1, occ_ws_[slot]);
    }
    void launch_ws(const StepArgs<T>& a, int ctas)
    {
        const int ms = models_slot();
        if (ms == 0)
            k_p2g_ws<T, 1><<<ctas, WsShape<T>::NT, WsShape<T>::dyn_bytes, stream_>>>(a);
        else if (ms == 1)
            k_p2g_ws<T, 2><<<ctas, WsShape<T>::NT, WsShape<T>::dyn_bytes, stream_>>>(a);
        else if (ms == 2)
            k_p2g_ws<T, 4><<<ctas, WsShape<T>::NT, WsShape<T>::dyn_bytes, stream_>>>(a);
        else
            k_p2g_ws<T, 7><<<ctas, WsShape<T>::NT, WsShape<T>::dyn_bytes, stream_>>>(a);
    }
    template <int V>
    void launch_fused(const StepArgs<T>& a, int ctas)
    {
        using FS = FusedShape<T, FUSED_CH[V]>;
        constexpr int MB = FUSED_MINB[V], CH = FUSED_CH[V];
        const int ms = models_slot();
        if (ms == 0)
            k_p2g_fused<T, 1, MB, CH><<<ctas, FS::NT, FS::dyn_bytes, stream_>>>(a);
        else if (ms == 1)
            k_p2g_fused<T, 2, MB, CH><<<ctas, FS::NT, FS::dyn_bytes, stream_>>>(a);
        else if (ms == 2)
            k_p2g_fused<T, 4, MB, CH><<<ctas, FS::NT, FS::dyn_bytes, stream_>>>(a);
        else
            k_p2g_fused<T, 7, MB, CH><<<ctas, FS::NT, FS::dyn_bytes, stream_>>>(a);
    }
    int models_slot() const { return models_ == 1 ? 0 : (models_ == 2 ? 1 : (models_ == 4 ? 2 : 3)); }
    template <int V>
    void launch_scatter(const StepArgs<T>& a, int ctas)
    {
        using S = ScatterShape<T, VAR_CHUNK[V], VAR_NBUF[V]>;
        k_scatter<T, VAR_CHUNK[V], VAR_NBUF[V]><<<ctas, S::NT, S::dyn_bytes, stream_>>>(a);
    }
    static int g2p_index(int nt) { return nt == G2P_NT[0] ? 0 : (nt == G2P_NT[1] ? 1 : (nt == G2P_NT[2] ? 2 : -1)); }

    static std::map<uint64_t, Schedule>& tune_cache()
    {
        static std::map<uint64_t, Schedule> c;
        return c;
    }
    static std::mutex& tune_mutex()
    {
        static std::mutex m;
        return m;
    }
    uint64_t tune_key() const
    {
        return (uint64_t)sizeof(T) | ((uint64_t)models_ << 4) | ((uint64_t)any_damage_ << 6) | ((uint64_t)bitlen(N_) << 8)
            | ((uint64_t)bitlen((uint64_t)n_scenes()) << 16) | ((uint64_t)nsm_ << 24);
    }

    // one trial substep with schedule sc on the current state; p2g / g2p milliseconds; state rolled back
    int trial(const Schedule& sc, float& p2g_ms, float& g2p_ms, bool& aborted_out)
    {
        if (int rc = refresh_drive()) return rc;
        sched_ = sc;
        if ((int)ev_.size() < 6) {
            size_t old = ev_.size();
            ev_.resize(6);
            for (size_t i = old; i < ev_.size(); i++) ZR_CUDA(cudaEventCreate(&ev_[i]));
        }
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        int rc = enqueue_step(cur_, ev_.data(), sort_base_stale_);
        sort_base_stale_ = true; // the trial's sort overwrote the base
        if (rc) return rc;
        ZR_CUDA(cudaMemcpyAsync(hst_, st_, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        ZR_CUDA(cudaEventElapsedTime(&p2g_ms, ev_[2], ev_[3]));
        ZR_CUDA(cudaEventElapsedTime(&g2p_ms, ev_[4], ev_[5]));
        aborted_out = (hst_->flags & FLAG_ABORT) != 0;
        // roll back: scene clocks, a clean grid after an aborted trial, the keys of the current buffer
        ZR_CUDA(cudaMemcpyAsync(d_scenes_, scenes_backup_, sizeof(SceneParams<T>) * h_scenes_.size(), cudaMemcpyDeviceToDevice, stream_));
        if (aborted_out) {
            ZR_CUDA(cudaMemsetAsync(acc_, 0, sizeof(T) * (size_t)b_cap_ * NACC * L::nodes, stream_));
            ZR_CUDA(cudaMemsetAsync(h_keys_, 0xff, 8 * (size_t)(h_mask_ + 1), stream_));
            if (cg_) ZR_CUDA(cudaMemsetAsync(cg_, 0, sizeof(T) * CG_NF * (size_t)b_cap_ * L::nodes, stream_));
        }
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        k_keys<T><<<nsm_ * 4, 256, 0, stream_>>>(pool(cur_), d_scenes_, n_scenes(), keys_in_, N_, kl_, st_);
        ZR_CUDA(cudaMemsetAsync(st_, 0, sizeof(DevStatus), stream_));
        ZR_CUDA(cudaStreamSynchronize(stream_));
        return 0;
    }

    // A schedule without measuring: the fixed default (mode 0) or a cached choice (mode 1). False when trials are needed.
    bool autotune_cached()
    {
        if (autotune_mode_ == 0) {
            sched_ = default_schedule();
            tuned_ = true;
            drop_graphs();
            return true;
        }
        if (autotune_mode_ == 1) {
            std::lock_guard<std::mutex> lk(tune_mutex());
            auto it = tune_cache().find(tune_key());
            if (it != tune_cache().end()) {
                sched_ = it->second;
                tuned_ = true;
                drop_graphs();
                return true;
            }
        }
        return false;
    }

    Schedule default_schedule() const { return Schedule{ 0, VAR_CHUNK[0], VAR_NBUF[0], occ_scatter_[0], G2P_NT[1], 0, 0 }; }

    int autotune_trials()
    {
        tuned_ = true;
        const size_t sb = sizeof(SceneParams<T>) * h_scenes_.size();
        if (sb > scenes_backup_bytes_) {
            dfree(scenes_backup_);
            scenes_backup_bytes_ = 0;
            if (alloc(&scenes_backup_, sb)) return ZR_ERR_CUDA_;
            scenes_backup_bytes_ = sb;
        }
        ZR_CUDA(cudaMemcpyAsync(scenes_backup_, d_scenes_, sb, cudaMemcpyDeviceToDevice, stream_));
        // P2G candidates with the default G2P, then G2P candidates with the chosen P2G
        std::vector<Schedule> p2g_c;
        for (int vi = 0; vi < 3; vi++)
            for (int c = occ_scatter_[vi]; c >= std::max(1, occ_scatter_[vi] - 1); c--)
                p2g_c.push_back(Schedule{ 0, VAR_CHUNK[vi], VAR_NBUF[vi], c, G2P_NT[1], 0, 1 });
        for (int fv = 0; fv < 2; fv++) {
            const int of = occ_fused_[fv][models_slot()];
            for (int c = of; c >= std::max(1, of - 1); c--) p2g_c.push_back(Schedule{ fused_code(fv), FUSED_CH[fv], 0, c, G2P_NT[1], 0, 1 });
        }
        {
            const int ow = occ_ws_[models_slot()];
            for (int c = ow; c >= std::max(1, ow - 1); c--) p2g_c.push_back(Schedule{ 3, WsShape<T>::CHUNK, WsShape<T>::NSTAGE, c, G2P_NT[1], 0, 1 });
        }
        constexpr int REPS = 2; // the first run of a candidate warms caches and instruction memory
        Schedule best = p2g_c[0];
        float best_p2g = 1e30f, best_g2p = 1e30f;
        for (const Schedule& sc : p2g_c) {
            float mp = 1e30f;
            for (int r = 0; r < REPS; r++) {
                float p = 0, g = 0;
                bool ab = false;
                int rc = trial(sc, p, g, ab);
                if (rc) return rc;
                if (ab) { // the state cannot step (CFL, out of domain, capacity): keep defaults, the step reports it
                    sched_ = default_schedule();
                    drop_graphs();
                    return 0;
                }
                mp = std::min(mp, p);
            }
            if (mp < best_p2g) {
                best_p2g = mp;
                best = sc;
            }
        }
        // G2P: 3 thread counts x 2 register budgets. The variants with the halo staged by bulk copies (g2p_tight + 2)
        // stay selectable by set_schedule but are not tried: as fast as the others in the first substeps of a pull,
        // where the trials run, and 4% slower late in it (0.290 against 0.279 ms per substep on the 3.4 M slab)
        for (int gc = 0; gc < 6; gc++) {
            const int gi = gc % 3;
            Schedule sc = best;
            sc.g2p_threads = G2P_NT[gi];
            sc.g2p_tight = gc / 3;
            float mg = 1e30f;
            for (int r = 0; r < REPS; r++) {
                float p = 0, g = 0;
                bool ab = false;
                int rc = trial(sc, p, g, ab);
                if (rc) return rc;
                if (ab) {
                    sched_ = default_schedule();
                    drop_graphs();
                    return 0;
                }
                mg = std::min(mg, g);
            }
            if (mg < best_g2p) {
                best_g2p = mg;
                best.g2p_threads = sc.g2p_threads;
                best.g2p_tight = sc.g2p_tight;
            }
        }
        best.tuned = 1;
        sched_ = best;
        drop_graphs();
        std::lock_guard<std::mutex> lk(tune_mutex());
        tune_cache()[tune_key()] = best;
        return 0;
    }

    void collect_timing(int nsteps)
    {
        for (int s = 0; s < nsteps; s++) {
            float t[5];
            for (int q = 0; q < 5; q++) cudaEventElapsedTime(&t[q], ev_[6 * s + q], ev_[6 * s + q + 1]);
            kt_.sort += t[0];
            kt_.blocks += t[1];
            kt_.p2g += t[2];
            kt_.grid += t[3];
            kt_.g2p += t[4];
            kt_.steps++;
        }
    }

    void release_batch()
    {
        drop_graphs();
        if (h2d_) cudaStreamSynchronize(h2d_);
        if (d2h_) cudaStreamSynchronize(d2h_);
        free_io();
        void* ps[] = { pool_[0], pool_[1], pid_[0], pid_[1], keys_in_, keys_sorted_, iota_, vals_sorted_, g_start_, g_nbr_, b_key_, acc_, vel_, h_keys_, h_vals_,
            d_scenes_, grid_mass_, st_, sort_tmp_, stage_, pay_, scenes_backup_, ck_pool_, ck_pid_, ck_scenes_, cg_, cgs_,
            sort_aux_, inc_move_, inc_bkey_, inc_bidx_, inv_ };
        for (void* p : ps)
            if (p) cudaFree(p);
        pool_[0] = pool_[1] = nullptr;
        pid_[0] = pid_[1] = nullptr;
        keys_in_ = keys_sorted_ = nullptr;
        iota_ = vals_sorted_ = g_start_ = nullptr;
        g_nbr_ = nullptr;
        b_key_ = nullptr;
        acc_ = vel_ = nullptr;
        h_keys_ = nullptr;
        h_vals_ = nullptr;
        d_scenes_ = nullptr;
        grid_mass_ = nullptr;
        st_ = nullptr;
        sort_tmp_ = stage_ = nullptr;
        stage_bytes_ = 0;
        pay_ = nullptr;
        pstride_ = 0;
        cg_ = nullptr;
        cgs_ = nullptr;
        implicit_ = false;
        sort_aux_ = nullptr;
        inc_move_ = inc_bkey_ = inc_bidx_ = nullptr;
        mcap_ = 0;
        inv_ = nullptr;
        inv_cap_ = 0;
        sort_base_stale_ = true;
        scenes_backup_ = nullptr;
        scenes_backup_bytes_ = 0;
        ck_pool_ = ck_pid_ = ck_scenes_ = nullptr;
        ck_cap_ = 0;
        ck_scenes_n_ = 0;
        ck_valid_ = false;
        tuned_ = false;
        N_ = 0;
        cap_ = 0;
        scene_cap_ = 0;
        b_cap_ = 0;
        dev_bytes_ = 0;
        h_scenes_.clear();
    }

    void release()
    {
        release_batch();
        for (auto& e : ev_) cudaEventDestroy(e);
        ev_.clear();
        if (t0_) cudaEventDestroy(t0_);
        if (t1_) cudaEventDestroy(t1_);
        t0_ = t1_ = nullptr;
        if (hst_) cudaFreeHost(hst_);
        hst_ = nullptr;
        if (stream_) cudaStreamDestroy(stream_);
        stream_ = nullptr;
        if (side_) cudaStreamDestroy(side_);
        side_ = nullptr;
        for (auto& ev : io_ev_)
            if (ev) cudaEventDestroy(ev);
        for (auto& ev : io_ev_) ev = nullptr;
        if (h2d_) cudaStreamDestroy(h2d_);
        if (d2h_) cudaStreamDestroy(d2h_);
        h2d_ = d2h_ = nullptr;
    }
};

} // namespace zr
