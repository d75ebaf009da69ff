// sim_base.h -- the simulation object behind amr_sim (the reference's AMR_data plugin concept,
// AMR.h:296-334): octree, device mirror of its arrays, host generator, streams, staged transfers.
// The plugins derive from SimBase: sim.cu holds the reference's two, evolve_sim.cu the evolutions.
//
// A simulation owns an Octree (AMR<T>) whose node_ctor hook prolongates new domains, a device mirror of
// the octree arrays uploaded when the octree changed (AMR<T>::copy_to_gpu, AMR.h:268-275), and a
// host fast_prng that hands every kernel launch its global seed in the reference's order.
//
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "evolve_kernels.h"

namespace amr {

inline int32_t host_prng_next(int32_t& s) {                       // fast_prng::generate_int, tensors.h:281-285
    uint32_t v = (uint32_t)s + 1124781675u;
    v ^= (uint32_t)((int32_t)v >> 7);
    v *= 1246477263u;
    s = (int32_t)v;
    return s;
}

template <class T>
inline cudaError_t dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) { *p = nullptr; return e; }
    return cudaMemset(*p, 0, count * sizeof(T));
}

class SimBase : public NodeHooks {
public:
    SimBase(const amr_config& c, uint32_t slots, int mode)
        : cfg(c), dims(make_dims(c)), geo(make_geo(c)), mode(mode), tree(slots, this) {}
    virtual ~SimBase() {
        if (side_stream) cudaStreamSynchronize(side_stream);
        for (cudaStream_t t : {up_stream, down_stream}) if (t) cudaStreamSynchronize(t);
        if (stream) cudaStreamSynchronize(stream);
        if (side_stream) cudaStreamDestroy(side_stream);
        for (cudaStream_t t : {up_stream, down_stream}) if (t) cudaStreamDestroy(t);
        for (Staging* set : {&up[0][0], &down[0][0]})
            for (int i = 0; i < 36; i++) set[i].release();
        if (main_mark) cudaEventDestroy(main_mark);
        for (auto& row : side_done)
            for (auto& ev : row) if (ev) cudaEventDestroy(ev);
        cudaFree(d_positions); cudaFree(d_children); cudaFree(d_boundaries); cudaFree(d_items); cudaFree(ctor_items);
        cudaFree(ghost_stage);
        for (auto& ev : events) cudaEventDestroy(ev);
        for (auto& ev : user_events) if (ev) cudaEventDestroy(ev);
        if (own_stream) cudaStreamDestroy(own_stream);   // a caller's stream stays the caller's
    }

    virtual int init() {
        const uint32_t s = tree.max_slots();
        cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        own_stream = stream;
        if (e == cudaSuccess) e = dev_alloc(&d_positions, s);
        if (e == cudaSuccess) e = dev_alloc(&d_children, (size_t)s * 8u);
        if (e == cudaSuccess) e = dev_alloc(&d_boundaries, (size_t)s * 6u);
        if (e == cudaSuccess) e = dev_alloc(&d_items, (size_t)s << (kDepthLimit + 1));   // active and parent lists
        if (e == cudaSuccess) { err_flag = device_error_flag(); if (!err_flag) e = cudaErrorMemoryAllocation; }
        if (e == cudaSuccess && config_supported(&cfg)) {
            // set the kernels' shared-memory limits now, outside any later stream capture (the
            // evolutions, whose sizes these kernels need not support, set their own)
            StencilArgs none;
            std::memset(&none, 0, sizeof(none));
            for (int kind : {SK_GRAD, SK_GRAD_HESS, SK_MIXED, SK_BSSN}) {
                if (kind == SK_BSSN && !bssn_fused_supported(&cfg)) continue;
                e = launch_stencil(cfg, kind, none, 0, stream);
                if (e != cudaSuccess) break;
            }
            FieldSet nofields;
            std::memset(&nofields, 0, sizeof(nofields));
            if (e == cudaSuccess) e = launch_copy_boundaries(dims, nofields, nullptr, 0, 0, 0, 1, nullptr, stream);
        }
        return cuda_status(e);
    }

    // The plugin interface of the reference (AMR.h:296-334).
    virtual int copy_back() = 0;
    virtual int modify_nodes() = 0;
    virtual int predictor() = 0;
    virtual int copy_bounds() = 0;
    virtual int corrector() = 0;
    virtual int timestep() {
        in_timestep = true;
        int st = AMR_OK;
        do {
            if ((st = copy_back())) break;
            if ((st = modify_nodes())) break;
            if ((st = predictor())) break;
            if ((st = copy_bounds())) break;
            if ((st = corrector())) break;
            tree.increment_timer();
        } while (tree.timer() != 0u);
        in_timestep = false;
        return st;
    }
    // Set while timestep() runs its substeps: each copy_bounds then follows the substep's copy_back,
    // so every active domain has old == new outside the cells its children cover.
    bool in_timestep = false;
    virtual int buffer(int which, int comp, void** ptr, uint64_t* count) = 0;
    // Launch-shape autotuning (amr_sim_autotune): only the BSSN plugin has a tunable pass.
    virtual int autotune(uint32_t reps, uint32_t* n_tuned) {
        (void)reps;
        if (n_tuned) *n_tuned = 0;
        return AMR_ERR_INVALID;
    }

    void node_dtor(int32_t) override {}
    // Batched node_ctor: upload the deferred constructors once, then prolongate each group into
    // every buffer of `bufs` with one launch; errors are kept for take_ctor_status().
    // Copy a batch of deferred constructors to the device (ctor_items); false (and ctor_status set)
    // on failure.
    bool upload_ctor_items(const NodeCtor* items, size_t n) {
        if (!ctor_items || ctor_items_cap < n) {
            cudaError_t e = cudaStreamSynchronize(stream);   // a launch of the last batch may still read it
            cudaFree(ctor_items);
            ctor_items = nullptr;
            ctor_items_cap = 0;
            const size_t cap = std::max<size_t>(n, tree.max_slots());
            if (e == cudaSuccess) e = cudaMalloc(&ctor_items, sizeof(NodeCtor) * cap);
            if (e != cudaSuccess) { ctor_status = cuda_status(e); return false; }
            ctor_items_cap = cap;
        }
        cudaError_t e = cudaMemcpyAsync(ctor_items, items, sizeof(NodeCtor) * n, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);   // `items` is pageable and short-lived
        if (e != cudaSuccess) { ctor_status = cuda_status(e); return false; }
        return true;
    }
    void prolongate_groups(const NodeCtor* items, const uint32_t* group_end, uint32_t groups, float* const* bufs,
                           int nbuf) {
        const size_t n = groups ? group_end[groups - 1] : 0u;
        if (n == 0 || !upload_ctor_items(items, n)) return;
        cudaError_t e = cudaSuccess;
        for (uint32_t g = 0, b = 0; g < groups && e == cudaSuccess; b = group_end[g++]) {
            e = launch_copy_to_children(dims, bufs, nbuf, reinterpret_cast<const int32_t*>(ctor_items + b),
                                        group_end[g] - b, stream);
            launches++;
        }
        if (e != cudaSuccess) ctor_status = cuda_status(e);
    }
    int take_ctor_status() { const int st = ctor_status; ctor_status = AMR_OK; return st; }
    NodeCtor* ctor_items = nullptr;
    size_t ctor_items_cap = 0;
    int ctor_status = AMR_OK;

    // AMR<T>::copy_to_gpu (AMR.h:268-275): upload the octree arrays if they changed.
    int sync_octree() {
        if (!tree.dirty()) return AMR_OK;
        const uint32_t s = tree.max_slots();
        cudaError_t e = cudaMemcpyAsync(d_positions, tree.positions().data(), s * 4u, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_children, tree.children().data(), (size_t)s * 32u, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_boundaries, tree.boundaries().data(), (size_t)s * 48u, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);   // host vectors are pageable
        if (e != cudaSuccess) return cuda_status(e);
        tree.mark_clean();
        items_valid = false;
        graph_valid = false;
        return AMR_OK;
    }

    // Lists of the domains active at each substep of a timestep (batched launches use these).
    int build_items() {
        if (items_valid) return AMR_OK;
        const uint32_t md = (uint32_t)tree.read_max_depth(), used = tree.curr_used_slots();
        const uint32_t nsub = 1u << md;
        std::vector<uint32_t> all;
        item_offset.assign(nsub, 0);
        item_count.assign(nsub, 0);
        parent_offset.assign(nsub, 0);
        parent_count.assign(nsub, 0);
        for (uint32_t s = 0; s < nsub; s++) {
            item_offset[s] = (uint32_t)all.size();
            for (uint32_t i = 0; i < used; i++) {
                const int d = pos_depth_host(tree.positions()[i]);
                if (d != -1 && (s & ((1u << (md - (uint32_t)d)) - 1u)) == 0u) all.push_back(i);
            }
            item_count[s] = (uint32_t)all.size() - item_offset[s];
            parent_offset[s] = (uint32_t)all.size();   // the active domains that have children
            for (uint32_t k = item_offset[s]; k < item_offset[s] + item_count[s]; k++) {
                bool parent = false;
                for (int c = 0; c < 8; c++) parent |= tree.children()[(size_t)all[k] * 8u + c] != -1;
                if (parent) all.push_back(all[k]);
            }
            parent_count[s] = (uint32_t)all.size() - parent_offset[s];
        }
        cudaError_t e = cudaMemcpyAsync(d_items, all.data(), all.size() * 4u, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_status(e);
        items_valid = true;
        return AMR_OK;
    }

    int ensure_ghost_stage(int ncomp) {
        const size_t need = ghost_scratch_floats(dims, tree.max_slots(), ncomp);
        if (need <= ghost_stage_floats) return AMR_OK;
        cudaStreamSynchronize(stream);
        cudaFree(ghost_stage);
        ghost_stage_floats = 0;
        cudaError_t e = dev_alloc(&ghost_stage, need);
        if (e != cudaSuccess) return cuda_status(e);
        ghost_stage_floats = need;
        return AMR_OK;
    }

    int32_t next_seed() { return host_prng_next(rng); }
    int check(cudaError_t e) {
        if (e != cudaSuccess) return cuda_status(e);
        launches++;
        return AMR_OK;
    }
    // Optional CUDA-event timing of the dominant kernel.
    void time_begin() {
        if (!timing || capturing) return;
        if (ev_used + 2 > events.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a); cudaEventCreate(&b);
            events.push_back(a); events.push_back(b);
        }
        cudaEventRecord(events[ev_used], stream);
    }
    void time_end() {
        if (!timing || capturing) return;
        cudaEventRecord(events[ev_used + 1], stream);
        ev_used += 2;
    }
    int harvest_timing(double* ms, uint64_t* n) {
        cudaError_t e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_status(e);
        for (size_t i = 0; i + 1 < ev_used; i += 2) {
            float t = 0.f;
            cudaEventElapsedTime(&t, events[i], events[i + 1]);
            timed_ms += t;
            timed_launches++;
        }
        ev_used = 0;
        *ms = timed_ms;
        *n = timed_launches;
        timed_ms = 0.0;
        timed_launches = 0;
        return AMR_OK;
    }

    int kind_id = 0;              // AMR_SIM_* of this simulation
    amr_config cfg;
    Dims dims;
    Geo geo;
    int mode;
    Octree tree;
    cudaStream_t stream = nullptr;       // where the simulation's work goes: its own or a caller's
    cudaStream_t own_stream = nullptr;   // the stream the simulation created (destroyed with it)
    // Run the simulation's work on a caller's stream from now on (nullptr: its own again); the
    // work queued so far, on every stream of the simulation, completes first.
    int set_stream(cudaStream_t s) {
        if (capturing) return AMR_ERR_INVALID;
        int st = sync_transfer_streams();
        if (!st && side_stream && cudaStreamSynchronize(side_stream) != cudaSuccess) st = AMR_ERR_CUDA;
        if (!st) st = cuda_status(cudaStreamSynchronize(stream));
        if (st) return st;
        stream = s ? s : own_stream;
        return AMR_OK;
    }
    uint32_t* d_positions = nullptr;
    int32_t* d_children = nullptr;
    uint64_t* d_boundaries = nullptr;
    uint32_t* d_items = nullptr;
    std::vector<uint32_t> item_offset, item_count, parent_offset, parent_count;
    bool items_valid = false;
    bool graph_valid = false;
    bool capturing = false;
    int* err_flag = nullptr;
    float* ghost_stage = nullptr;
    size_t ghost_stage_floats = 0;
    int32_t rng = 12894712;      // fast_prng default seed, tensors.h:280
    uint64_t launches = 0;
    bool timing = false;
    std::vector<cudaEvent_t> events;
    size_t ev_used = 0;
    cudaEvent_t user_events[16] = {};
    // Side stream for reads of results that overlap later work on `stream` (amr_sim_copy_to_host_side):
    // side_done[which][comp] marks the last side copy of a buffer, side_pending that one is outstanding.
    cudaStream_t side_stream = nullptr;
    cudaEvent_t main_mark = nullptr;
    cudaEvent_t side_done[6][6] = {};
    bool side_pending[6][6] = {};

    // Make `stream` wait for outstanding side copies: of one buffer, or (which < 0) of all.
    int wait_side(int which, int comp) {
        for (int w = 0; w < 6; w++)
            for (int c = 0; c < 6; c++) {
                if (!side_pending[w][c] || (which >= 0 && (w != which || c != comp))) continue;
                cudaError_t e = cudaStreamWaitEvent(stream, side_done[w][c], 0);
                if (e != cudaSuccess) return cuda_status(e);
                side_pending[w][c] = false;
            }
        return AMR_OK;
    }
    // Staged transfers (amr_sim_stage_to_device, amr_sim_snapshot_to_host): per buffer a device
    // staging copy for uploads and one for downloads; host transfers run on their own streams
    // (one per direction) and overlap the simulation's work, which meets them only at the
    // device-to-device copies between a buffer and its staging copy.
    struct Staging {
        float* buf = nullptr;
        uint64_t cap = 0;               // floats
        cudaEvent_t copied = nullptr;   // stream: the device-to-device copy (into or out of buf) is done
        cudaEvent_t moved = nullptr;    // transfer stream: the host transfer (into or out of buf) is done
        bool pending = false;           // download: a host transfer from buf is outstanding
        int ensure(uint64_t floats) {
            if (!copied && cudaEventCreateWithFlags(&copied, cudaEventDisableTiming) != cudaSuccess) return AMR_ERR_CUDA;
            if (!moved && cudaEventCreateWithFlags(&moved, cudaEventDisableTiming) != cudaSuccess) return AMR_ERR_CUDA;
            if (cap >= floats) return AMR_OK;
            if (buf) { cudaEventSynchronize(copied); cudaEventSynchronize(moved); cudaFree(buf); buf = nullptr; cap = 0; }
            if (cudaMalloc(&buf, floats * sizeof(float)) != cudaSuccess) { buf = nullptr; return AMR_ERR_CUDA; }
            cap = floats;
            return AMR_OK;
        }
        void release() {
            cudaFree(buf);
            if (copied) cudaEventDestroy(copied);
            if (moved) cudaEventDestroy(moved);
        }
    };
    cudaStream_t up_stream = nullptr, down_stream = nullptr;
    Staging up[6][6], down[6][6];
    int ensure_transfer_streams() {
        if (!up_stream && cudaStreamCreateWithFlags(&up_stream, cudaStreamNonBlocking) != cudaSuccess) return AMR_ERR_CUDA;
        if (!down_stream && cudaStreamCreateWithFlags(&down_stream, cudaStreamNonBlocking) != cudaSuccess) return AMR_ERR_CUDA;
        return AMR_OK;
    }
    // Make `stream` wait for the outstanding downloads of snapshots (so that an event recorded next
    // follows them).
    int wait_snapshots() {
        for (auto& row : down)
            for (Staging& d : row) {
                if (!d.pending) continue;
                cudaError_t e = cudaStreamWaitEvent(stream, d.moved, 0);
                if (e != cudaSuccess) return cuda_status(e);
                d.pending = false;
            }
        return AMR_OK;
    }
    int sync_transfer_streams() {
        for (cudaStream_t t : {side_stream, up_stream, down_stream})
            if (t && cudaStreamSynchronize(t) != cudaSuccess) return AMR_ERR_CUDA;
        return AMR_OK;
    }
    double timed_ms = 0.0;
    uint64_t timed_launches = 0;

    // CTAs of the fused BSSN pass: fixed by amr_sim_set_stencil_ctas (0: automatic), else the
    // autotuned choice for this domain count, else the library's rule (stencil_grid).
    uint32_t stencil_ctas = 0;
    // failure-path test hooks of the fused pass (amr_sim_set_fault_injection; StencilArgs)
    uint32_t fault_spin_limit = 0, fault_withhold = 0;
    std::vector<std::pair<uint32_t, uint32_t>> tuned_ctas;   // (active domains, CTAs)
    uint32_t fused_grid(uint32_t n_items) const {
        if (stencil_ctas) return stencil_ctas;
        for (const auto& t : tuned_ctas)
            if (t.first == n_items) return t.second;
        return stencil_grid(cfg, SK_BSSN, n_items);
    }
};

// Simulations of the evolution kinds (AMR_SIM_BSSN_EVOLVE, AMR_SIM_WAVE_RK4; evolve_sim.cu).
SimBase* make_evolve_sim(const amr_config& c, int kind, uint32_t slots, int mode);
bool is_evolve_sim(const SimBase* s);

}  // namespace amr

struct amr_sim {
    amr::SimBase* impl;
};
