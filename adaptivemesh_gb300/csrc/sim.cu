// sim.cu -- the reference's plugins (AMR_data, AMR.h:296-334) on the GB300 kernels.
//
//   BssnSim  ~ BSSN_AMR_data  (BSSN.h:104-171)
//   WaveSim  ~ wave_AMR_data  (SimpleWave.h:191-279)
//
// Both derive from SimBase (sim_base.h).  Modes: PLAIN issues the reference's launch sequence (one
// launch per operator and component); BATCHED issues one launch per phase for all components over
// the list of domains active at the substep; GRAPH replays a captured CUDA graph of one whole BSSN
// timestep (all substeps).
#include <algorithm>

#include "sim_base.h"

namespace amr {

// ============================================================================ BSSN
class BssnSim : public SimBase {
public:
    using SimBase::SimBase;
    ~BssnSim() override {
        if (stream) cudaStreamSynchronize(stream);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        for (int k = 0; k < 6; k++) {
            cudaFree(old6[k]); cudaFree(new6[k]); cudaFree(ricci6[k]); cudaFree(dmet6[k]); cudaFree(chr6[k]);
        }
        for (int k = 0; k < 4; k++) cudaFree(hint[k]);
        cudaFree(d_seeds);
    }
    int init() override {
        int st = SimBase::init();
        if (st) return st;
        const size_t s = tree.max_slots();
        const size_t padded = s * dims.t * dims.t * dims.t, inner = s * dims.n * dims.n * dims.n;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 6 && e == cudaSuccess; k++) {
            e = dev_alloc(&old6[k], padded);
            if (e == cudaSuccess) e = dev_alloc(&new6[k], padded);
            if (e == cudaSuccess) e = dev_alloc(&ricci6[k], inner);
            if (e == cudaSuccess) e = dev_alloc(&dmet6[k], inner);
            if (e == cudaSuccess) e = dev_alloc(&chr6[k], inner);
        }
        for (int k = 0; k < 4 && e == cudaSuccess; k++) e = dev_alloc(&hint[k], inner);   // didjA / didjW
        if (e == cudaSuccess) e = dev_alloc(&d_seeds, (size_t)kSeedsPerSubstep << kDepthLimit);
        if (e != cudaSuccess) return cuda_status(e);
        return ensure_ghost_stage(6);
    }
    // BSSN_AMR_data::node_ctor (BSSN.h:131-137): prolongate old and new metric into the child.
    void node_ctor(int32_t node) override {
        const uint32_t off = (uint32_t)pos_final_offset(tree.positions()[node]);
        const int32_t parent = tree.parents()[node];
        for (int k = 0; k < 6; k++) check(launch_copy_to_child(dims, old6[k], off, node, parent, stream));
        for (int k = 0; k < 6; k++) check(launch_copy_to_child(dims, new6[k], off, node, parent, stream));
        graph_valid = false;
    }
    void node_ctor_groups(const NodeCtor* items, const uint32_t* group_end, uint32_t groups) override {
        float* bufs[12];
        for (int k = 0; k < 6; k++) { bufs[k] = old6[k]; bufs[6 + k] = new6[k]; }
        prolongate_groups(items, group_end, groups, bufs, 12);
        graph_valid = false;
    }

    // --- phases
    int copy_back() override {                                   // BSSN.h:126-130
        int st = sync_octree();
        if (st) return st;
        const uint32_t s = tree.timer(), md = (uint32_t)tree.read_max_depth(), used = tree.curr_used_slots();
        FieldSet f;
        std::memset(&f, 0, sizeof(f));
        if (mode == AMR_MODE_PLAIN) {
            f.ncomp = 1;
            for (int k = 0; k < 6; k++) {
                f.old_f[0] = old6[k]; f.new_f[0] = new6[k];
                if ((st = check(launch_copy_new_to_old(dims, f, d_positions, d_children, nullptr, used, s, md, stream)))) return st;
            }
            return AMR_OK;
        }
        if ((st = build_items())) return st;
        f.ncomp = 6;
        for (int k = 0; k < 6; k++) { f.old_f[k] = old6[k]; f.new_f[k] = new6[k]; }
        // Inside timestep(), with the fused predictor, leaves restrict themselves as the predictor
        // streams their planes (old <- new plane by plane); only the domains with children are
        // restricted here.  A phase called on its own restricts every active domain.
        const bool fused = in_timestep && bssn_fused_supported(&cfg);
        if ((fused ? parent_count[s] : item_count[s]) == 0u) return AMR_OK;   // nothing to launch
        return check(launch_copy_new_to_old(dims, f, d_positions, d_children,
                                            d_items + (fused ? parent_offset[s] : item_offset[s]),
                                            fused ? parent_count[s] : item_count[s], s, md, stream, fused));
    }
    int modify_nodes() override { return AMR_OK; }              // BSSN.h:139-142
    int predictor() override { return derivatives(old6, seed_slot(0), in_timestep); }
    int corrector() override { return derivatives(new6, seed_slot(1)); }
    int copy_bounds() override {                                 // BSSN.h:149-153
        int st = sync_octree();
        if (st) return st;
        const uint32_t s = tree.timer(), md = (uint32_t)tree.read_max_depth(), used = tree.curr_used_slots();
        FieldSet f;
        std::memset(&f, 0, sizeof(f));
        if (mode == AMR_MODE_PLAIN) {
            f.ncomp = 1;
            for (int k = 0; k < 6; k++) {
                f.old_f[0] = old6[k]; f.new_f[0] = new6[k];
                if ((st = check(launch_copy_boundaries(dims, f, d_boundaries, used, s, md, 1, ghost_stage, stream)))) return st;
                launches++;   // fill + commit
            }
            return AMR_OK;
        }
        f.ncomp = 6;
        for (int k = 0; k < 6; k++) { f.old_f[k] = old6[k]; f.new_f[k] = new6[k]; }
        // inside a timestep the fill writes in place, in one launch (launch_copy_boundaries)
        st = check(launch_copy_boundaries(dims, f, d_boundaries, used, s, md, 1, ghost_stage, stream, in_timestep));
        if (!st && !in_timestep) launches++;   // + the commit launch
        return st;
    }

    int timestep() override {
        if (mode != AMR_MODE_GRAPH) {
            seeds_from_device = false;
            return SimBase::timestep();
        }
        return graph_timestep();
    }

    int buffer(int which, int comp, void** ptr, uint64_t* count) override {
        if (comp < 0 || comp > 5) return AMR_ERR_INVALID;
        const uint64_t s = tree.max_slots();
        switch (which) {
            case 0: *ptr = old6[comp]; *count = s * dims.t * dims.t * dims.t; return AMR_OK;
            case 1: *ptr = new6[comp]; *count = s * dims.t * dims.t * dims.t; return AMR_OK;
            case 2: *ptr = ricci6[comp]; *count = s * dims.n * dims.n * dims.n; return AMR_OK;
            case 3: *ptr = dmet6[comp]; *count = s * dims.n * dims.n * dims.n; return AMR_OK;
            case 4: *ptr = chr6[comp]; *count = s * dims.n * dims.n * dims.n; return AMR_OK;
            default: return AMR_ERR_INVALID;
        }
    }

    // The fused pass's grid, tuned per active-domain count of this octree: every distinct count of
    // a timestep's substeps is timed at a set of candidate grids (CUDA events on the simulation's
    // stream, the predictor's form with the leaves' restriction) and the fastest is kept.  The
    // candidate launches read the metric and write only scratch buffers allocated here, so the
    // simulation's state and outputs are left as they were.  Results do not depend on the grid.
    int autotune(uint32_t reps, uint32_t* n_tuned) override {
        if (n_tuned) *n_tuned = 0;
        if (!bssn_fused_supported(&cfg) || capturing || reps == 0u || reps > 100u) return AMR_ERR_INVALID;
        int st = wait_side(-1, 0);
        if (!st) st = sync_octree();
        if (!st) st = build_items();
        if (st) return st;
        const uint32_t md = (uint32_t)tree.read_max_depth(), nsub = 1u << md, used = tree.curr_used_slots();
        const size_t padded = (size_t)used * dims.t * dims.t * dims.t, inner = (size_t)used * dims.n * dims.n * dims.n;
        float* scratch = nullptr;
        cudaError_t e = cudaMalloc(&scratch, sizeof(float) * (6u * padded + 18u * inner));
        if (e != cudaSuccess) return cuda_status(e);
        e = cudaMemsetAsync(scratch, 0, sizeof(float) * (6u * padded + 18u * inner), stream);
        cudaEvent_t ev[2] = {nullptr, nullptr};
        e = cudaEventCreate(&ev[0]);
        if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
        int sms = 0, dev = 0;
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        std::vector<std::pair<uint32_t, uint32_t>> tuned;
        for (uint32_t s = 0; s < nsub && e == cudaSuccess; s++) {
            const uint32_t n = item_count[s];
            bool seen = n == 0u;
            for (const auto& t : tuned) seen |= t.first == n;
            if (seen) continue;
            StencilArgs a;
            std::memset(&a, 0, sizeof(a));
            a.positions = d_positions;
            a.substep = s;
            a.max_depth = md;
            a.geo = geo;
            a.err = err_flag;
            a.christoffel_mode = AMR_CHRISTOFFEL_REFERENCE;
            for (int k = 0; k < 6; k++) { a.seed_d[k] = 1 + k; a.seed_m[k] = 7 + k; }
            a.seed_c = 13;
            a.items = d_items + item_offset[s];
            a.n_items = n;
            for (int k = 0; k < 6; k++) {
                a.field[k] = scratch + k * padded;   // read by domains with children, written for leaves
                a.leaf_src[k] = new6[k];
                a.grad[k] = reinterpret_cast<uint32_t*>(scratch + 6u * padded + k * inner);
                a.lap[k] = scratch + 6u * padded + (6u + k) * inner;
                a.chr[k] = reinterpret_cast<uint32_t*>(scratch + 6u * padded + (12u + k) * inner);
            }
            a.children = d_children;
            // candidates: the library's rule, one and two CTAs per SM, and ranges of 2 to 64 planes
            const uint32_t rule = stencil_grid(cfg, SK_BSSN, n), planes = n * dims.n;
            std::vector<uint32_t> cand = {rule, (uint32_t)sms, 2u * (uint32_t)sms, 3u * (uint32_t)sms, 4u * (uint32_t)sms};
            for (uint32_t r = 2; r <= 64; r *= 2) cand.push_back((planes + r - 1u) / r);
            std::sort(cand.begin(), cand.end());
            cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
            uint32_t best = rule;
            float best_ms = 0.f;
            for (uint32_t g : cand) {
                if (g == 0u || g > planes) continue;
                e = launch_stencil(cfg, SK_BSSN, a, g, stream);   // warm-up
                if (e == cudaSuccess) e = cudaEventRecord(ev[0], stream);
                for (uint32_t r = 0; r < reps && e == cudaSuccess; r++) e = launch_stencil(cfg, SK_BSSN, a, g, stream);
                if (e == cudaSuccess) e = cudaEventRecord(ev[1], stream);
                if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
                if (e != cudaSuccess) break;
                if (best_ms == 0.f || ms < best_ms) { best_ms = ms; best = g; }
            }
            tuned.emplace_back(n, best);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        cudaFree(scratch);
        if (e != cudaSuccess) return cuda_status(e);
        st = take_device_error(err_flag);   // a candidate whose waits gave up leaves the flag set
        if (st) return st;
        tuned_ctas = tuned;
        graph_valid = false;
        if (n_tuned) *n_tuned = (uint32_t)tuned.size();
        return AMR_OK;
    }

private:
    static constexpr int kSeedsPerSubstep = 26;   // 13 per predictor / corrector

    // Where this phase's 13 seeds come from: the host generator (plain/batched) or, inside a
    // captured graph, the device array filled before each replay.
    const int32_t* seed_slot(int phase) const {
        return seeds_from_device ? d_seeds + (size_t)tree.timer() * kSeedsPerSubstep + phase * 13 : nullptr;
    }

    // metric_derivatives_noncovariant + compute_raised_christoffel_symbols (BSSN.h:38-102)
    // restrict_leaves: the predictor's pass also performs the leaves' part of copy_back.
    int derivatives(float* const* g, const int32_t* dev_seeds, bool restrict_leaves = false) {
        int st = sync_octree();
        if (st) return st;
        const uint32_t s = tree.timer(), md = (uint32_t)tree.read_max_depth(), used = tree.curr_used_slots();
        StencilArgs a;
        std::memset(&a, 0, sizeof(a));
        a.positions = d_positions;
        a.substep = s;
        a.max_depth = md;
        a.geo = geo;
        a.err = err_flag;
        a.christoffel_mode = AMR_CHRISTOFFEL_REFERENCE;
        if (!dev_seeds) {
            for (int k = 0; k < 6; k++) { a.seed_d[k] = next_seed(); a.seed_m[k] = next_seed(); }
            a.seed_c = next_seed();
        }
        a.seed_ptr = dev_seeds;
        if (mode == AMR_MODE_PLAIN || !bssn_fused_supported(&cfg)) {
            a.items = nullptr;
            a.n_items = used;
            for (int k = 0; k < 6; k++) {
                // the reference alternates two intermediate Hessians between two streams
                uint32_t* hd = hint[(k & 1) * 2], *ho = hint[(k & 1) * 2 + 1];
                StencilArgs b = a;
                b.seed_ptr = nullptr;
                b.field[0] = g[k]; b.grad[0] = dmet6[k]; b.hdiag = hd; b.seed_d[0] = a.seed_d[k];
                time_begin();
                if ((st = check(launch_stencil(cfg, SK_GRAD_HESS, b, stencil_grid(cfg, SK_GRAD_HESS, used), stream)))) return st;
                time_end();
                b.hoff = ho; b.seed_m[0] = a.seed_m[k];
                if ((st = check(launch_stencil(cfg, SK_MIXED, b, stencil_grid(cfg, SK_MIXED, used), stream)))) return st;
                if ((st = check(launch_deriv_trace(dims, hd, ho, g, ricci6[k], d_positions, used, s, md, stream)))) return st;
            }
            return check(launch_christoffel(dims, g, dmet6, a.seed_c, chr6, d_positions, used, s, md,
                                            AMR_CHRISTOFFEL_REFERENCE, stream));
        }
        if ((st = build_items())) return st;
        a.items = d_items + item_offset[s];
        a.n_items = item_count[s];
        for (int k = 0; k < 6; k++) { a.field[k] = g[k]; a.grad[k] = dmet6[k]; a.lap[k] = ricci6[k]; a.chr[k] = chr6[k]; }
        if (restrict_leaves) {
            a.children = d_children;
            for (int k = 0; k < 6; k++) a.leaf_src[k] = new6[k];
        }
        a.spin_limit = fault_spin_limit;
        a.withhold = fault_withhold;
        time_begin();
        st = check(launch_stencil(cfg, SK_BSSN, a, fused_grid(a.n_items), stream));
        time_end();
        return st;
    }

    // One timestep from a captured graph: the host draws the seeds of every launch of the
    // timestep in the reference's order, uploads them, and replays the graph.
    int graph_timestep() {
        int st = sync_octree();
        if (st) return st;
        if ((st = build_items())) return st;
        if (tree.timer() != 0u) {   // a timestep always starts at counter 0 (AMR.h:324-333)
            seeds_from_device = false;
            return SimBase::timestep();
        }
        const uint32_t nsub = 1u << tree.read_max_depth();
        const bool capture = !graph_valid;   // capturing runs the host loop, counter and lifetimes included
        if (capture) {
            if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
            cudaGraph_t graph;
            cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_status(e);
            capturing = true;
            seeds_from_device = true;
            const uint64_t before = launches;
            st = SimBase::timestep();        // records every launch; the counter returns to 0
            capturing = false;
            seeds_from_device = false;
            e = cudaStreamEndCapture(stream, &graph);
            if (st) { if (e == cudaSuccess) cudaGraphDestroy(graph); return st; }
            if (e != cudaSuccess) return cuda_status(e);
            e = cudaGraphInstantiate(&graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(e);
            graph_launches = launches - before;
            launches = before;
            graph_valid = true;
        }
        // the seeds go to the device as launch parameters, not by a copy: a copy could queue behind
        // a bulk transfer on the copy engine (amr_sim_stage_to_device) and hold up the replay
        seed_words.resize((size_t)nsub * kSeedsPerSubstep);
        for (uint32_t s = 0; s < nsub; s++)
            for (int i = 0; i < kSeedsPerSubstep; i++) seed_words[(size_t)s * kSeedsPerSubstep + i] = next_seed();
        uint32_t seed_launches = 0;
        cudaError_t e = launch_store_words(d_seeds, seed_words.data(), (uint32_t)seed_words.size(), stream, &seed_launches);
        launches += seed_launches;
        if (e == cudaSuccess) e = cudaGraphLaunch(graph_exec, stream);
        if (e != cudaSuccess) return cuda_status(e);
        launches += graph_launches;
        // a replay does the device work only: advance the octree's counter and lifetimes as the
        // timestep loop would (AMR.h:180-188, once per substep; the counter returns to 0)
        if (!capture)
            for (uint32_t s = 0; s < nsub; s++) tree.increment_timer();
        return AMR_OK;
    }

    float* old6[6] = {};
    float* new6[6] = {};
    float* ricci6[6] = {};
    uint32_t* dmet6[6] = {};
    uint32_t* chr6[6] = {};
    uint32_t* hint[4] = {};
    int32_t* d_seeds = nullptr;
    std::vector<int32_t> seed_words;
    bool seeds_from_device = false;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_launches = 0;
};

// ============================================================================ SimpleWave
class WaveSim : public SimBase {
public:
    using SimBase::SimBase;
    ~WaveSim() override {
        if (stream) cudaStreamSynchronize(stream);
        cudaFree(old_f); cudaFree(new_f); cudaFree(derivs); cudaFree(hess); cudaFree(crit);
        if (crit_host) cudaFreeHost(crit_host);
    }
    int init() override {
        int st = SimBase::init();
        if (st) return st;
        const size_t s = tree.max_slots();
        const size_t padded = s * dims.t * dims.t * dims.t, inner = s * dims.n * dims.n * dims.n;
        cudaError_t e = dev_alloc(&old_f, padded);
        if (e == cudaSuccess) e = dev_alloc(&new_f, padded);
        if (e == cudaSuccess) e = dev_alloc(&derivs, inner);
        if (e == cudaSuccess) e = dev_alloc(&hess, inner);
        if (e == cudaSuccess) e = dev_alloc(&crit, s * dims.n * dims.n);
        if (e == cudaSuccess) e = cudaMallocHost(&crit_host, sizeof(float) * s * dims.n * dims.n);
        if (e != cudaSuccess) return cuda_status(e);
        return ensure_ghost_stage(1);
    }
    void node_ctor(int32_t node) override {                     // SimpleWave.h:219-225
        const uint32_t off = (uint32_t)pos_final_offset(tree.positions()[node]);
        const int32_t parent = tree.parents()[node];
        check(launch_copy_to_child(dims, old_f, off, node, parent, stream));
        check(launch_copy_to_child(dims, new_f, off, node, parent, stream));
    }
    void node_ctor_groups(const NodeCtor* items, const uint32_t* group_end, uint32_t groups) override {
        float* bufs[2] = {old_f, new_f};
        prolongate_groups(items, group_end, groups, bufs, 2);
    }
    int copy_back() override {                                   // SimpleWave.h:214-218
        int st = sync_octree();
        if (st) return st;
        FieldSet f;
        std::memset(&f, 0, sizeof(f));
        f.old_f[0] = old_f; f.new_f[0] = new_f; f.ncomp = 1;
        return check(launch_copy_new_to_old(dims, f, d_positions, d_children, nullptr, tree.curr_used_slots(), tree.timer(),
                                            (uint32_t)tree.read_max_depth(), stream));
    }
    // amr_criterion (SimpleWave.h:142-187) followed by the triage of modify_nodes (:228-248).
    int modify_nodes() override {
        int st = sync_octree();
        if (st) return st;
        const uint32_t used = tree.curr_used_slots(), n = dims.n;
        if ((st = check(launch_criterion(dims, geo, derivs, hess, crit, d_positions, used, tree.timer(),
                                         (uint32_t)tree.read_max_depth(), stream)))) return st;
        launches++;
        cudaError_t e = cudaMemcpyAsync(crit_host, crit, sizeof(float) * used * n * n, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_status(e);
        float* c = crit_host;
        float avg1 = 0.f, avg2 = 0.f;
        uint32_t active = 0;
        const uint32_t nn = n * n;
        for (uint32_t i = 0; i < used; i++) {
            const uint32_t b = i * nn, h = n >> 1, q4 = nn >> 2, q2 = nn >> 1;
            c[i * 8u] = c[b];
            c[i * 8u + 1u] = c[b + h];
            c[i * 8u + 2u] = c[b + q4];
            c[i * 8u + 3u] = c[b + h + q4];
            c[i * 8u + 4u] = c[b + q2];
            c[i * 8u + 5u] = c[b + h + q2];
            c[i * 8u + 6u] = c[b + q4 + q2];
            c[i * 8u + 7u] = c[b + h + q4 + q2];
            for (int j = 0; j < 8; j++)
                if (!std::isnan(c[i * 8u + j])) avg2 += fmaxf(0.f, fminf(c[i * 8u + j], 2.f));
        }
        for (uint32_t i = 0; i < used; i++) {
            float t = c[i * 8u];
            for (int j = 1; j < 8; j++) t = fmaxf(t, c[i * 8u + j]);
            c[i + used * 8u] = t;
            if (!std::isnan(t)) { avg1 += fmaxf(0.f, fminf(t, 2.f)); active++; }
        }
        float ax = avg1 / (float)active, ay = (avg2 * .125f) / (float)active;
        if (used == 1u) ax = ay = .15f;
        const float urgency = (float)(used - 1u) / (float)tree.max_slots();
        // one batch: each decision still sees the tree as the calls before it left it, but the
        // boundary refresh runs once and the new nodes are prolongated per depth level
        tree.begin_batch();
        for (uint32_t i = 1, s = used; i < s; i++) {               // root cannot be removed
            const float ratio = (float)pos_depth_host(tree.positions()[i]) / (float)tree.read_max_depth();
            if (ratio <= 0.f) continue;
            const float life = fmaxf(0.f, fminf((float)tree.lifetime()[i] * .1f - .2f, 1.f));
            const float weight = life * urgency * urgency * ax * std::sqrt(ratio);
            if (c[s * 8u + i] < weight) tree.remove_node((int32_t)i);
        }
        for (uint32_t i = 0, s = used * 8u; i < s; i++) {
            const float weight = ay * 3.f / (1.f - urgency);
            if (c[i] > weight && tree.children()[i] == -1) tree.add_node((int32_t)(i >> 3u), (int32_t)(i & 7u));
        }
        tree.end_batch();
        return take_ctor_status();
    }
    int predictor() override {                                   // SimpleWave.h:249-255
        int st = sync_octree();
        if (st) return st;
        if ((st = differentiate(old_f))) return st;
        return check(launch_wave_step(dims, geo, 0, old_f, derivs, hess, new_f, d_positions, tree.curr_used_slots(),
                                      tree.timer(), (uint32_t)tree.read_max_depth(), stream));
    }
    int copy_bounds() override {                                 // SimpleWave.h:256-260
        int st = sync_octree();
        if (st) return st;
        FieldSet f;
        std::memset(&f, 0, sizeof(f));
        f.old_f[0] = old_f; f.new_f[0] = new_f; f.ncomp = 1;
        st = check(launch_copy_boundaries(dims, f, d_boundaries, tree.curr_used_slots(), tree.timer(),
                                          (uint32_t)tree.read_max_depth(), 1, ghost_stage, stream));
        if (!st) launches++;
        return st;
    }
    int corrector() override {                                   // SimpleWave.h:261-267
        int st = sync_octree();
        if (st) return st;
        if ((st = differentiate(new_f))) return st;
        return check(launch_wave_step(dims, geo, 1, old_f, derivs, hess, new_f, d_positions, tree.curr_used_slots(),
                                      tree.timer(), (uint32_t)tree.read_max_depth(), stream));
    }
    int buffer(int which, int comp, void** ptr, uint64_t* count) override {
        if (comp != 0) return AMR_ERR_INVALID;
        const uint64_t s = tree.max_slots();
        switch (which) {
            case 0: *ptr = old_f; *count = s * dims.t * dims.t * dims.t; return AMR_OK;
            case 1: *ptr = new_f; *count = s * dims.t * dims.t * dims.t; return AMR_OK;
            case 3: *ptr = derivs; *count = s * dims.n * dims.n * dims.n; return AMR_OK;
            case 4: *ptr = hess; *count = s * dims.n * dims.n * dims.n; return AMR_OK;
            case 5: *ptr = crit; *count = s * dims.n * dims.n; return AMR_OK;
            default: return AMR_ERR_INVALID;
        }
    }

private:
    int differentiate(const float* field) {
        StencilArgs a;
        std::memset(&a, 0, sizeof(a));
        a.positions = d_positions;
        a.n_items = tree.curr_used_slots();
        a.substep = tree.timer();
        a.max_depth = (uint32_t)tree.read_max_depth();
        a.geo = geo;
        a.err = err_flag;
        a.field[0] = field;
        a.grad[0] = derivs;
        a.hdiag = hess;
        a.seed_d[0] = next_seed();
        time_begin();
        const int st = check(launch_stencil(cfg, SK_GRAD_HESS, a, stencil_grid(cfg, SK_GRAD_HESS, a.n_items), stream));
        time_end();
        return st;
    }
    float* old_f = nullptr;
    float* new_f = nullptr;
    uint32_t* derivs = nullptr;
    uint32_t* hess = nullptr;
    float* crit = nullptr;
    float* crit_host = nullptr;
};

}  // namespace amr

using namespace amr;

#define AMR_API extern "C" __attribute__((visibility("default")))

AMR_API int amr_sim_create(const amr_config* cfg, int kind, uint32_t node_slots, int mode, amr_sim** out) {
    if (!cfg || !out || node_slots < 1u || node_slots > (1u << 23)) return AMR_ERR_INVALID;
    if (mode < AMR_MODE_PLAIN || mode > AMR_MODE_GRAPH) return AMR_ERR_INVALID;
    const bool evolution = kind == AMR_SIM_BSSN_EVOLVE || kind == AMR_SIM_WAVE_RK4;
    if (evolution ? !(cfg->outer_size > 0.f) || !evo_config_supported(cfg->size_domain, cfg->padding_domain)
                  : !config_supported(cfg))
        return AMR_ERR_UNSUPPORTED;
    if (kind == AMR_SIM_WAVE && cfg->size_domain % 4u != 0u) return AMR_ERR_UNSUPPORTED;
    SimBase* s = nullptr;
    if (kind == AMR_SIM_BSSN) s = new (std::nothrow) BssnSim(*cfg, node_slots, mode);
    else if (kind == AMR_SIM_WAVE) s = new (std::nothrow) WaveSim(*cfg, node_slots, mode == AMR_MODE_GRAPH ? AMR_MODE_BATCHED : mode);
    else if (evolution) s = make_evolve_sim(*cfg, kind, node_slots, mode);
    else return AMR_ERR_INVALID;
    if (!s) return AMR_ERR_CAPACITY;
    if (!evolution) s->kind_id = kind;
    const int st = s->init();
    if (st) { delete s; return st; }
    *out = new (std::nothrow) amr_sim{s};
    if (!*out) { delete s; return AMR_ERR_CAPACITY; }
    return AMR_OK;
}
AMR_API int amr_sim_destroy(amr_sim* s) {
    if (!s) return AMR_ERR_INVALID;
    delete s->impl;
    delete s;
    return AMR_OK;
}
AMR_API int amr_sim_set_mode(amr_sim* s, int mode) {
    if (!s || mode < AMR_MODE_PLAIN || mode > AMR_MODE_GRAPH) return AMR_ERR_INVALID;
    if (dynamic_cast<WaveSim*>(s->impl) && mode == AMR_MODE_GRAPH) mode = AMR_MODE_BATCHED;
    if (mode == AMR_MODE_GRAPH && s->impl->timing) return AMR_ERR_INVALID;
    s->impl->mode = mode;
    s->impl->graph_valid = false;
    return AMR_OK;
}
AMR_API int amr_sim_add_node(amr_sim* s, int32_t parent, int32_t offset) {
    if (!s || parent < 0 || (uint32_t)parent >= s->impl->tree.max_slots() || offset < 0 || offset > 7) return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);   // node_ctor writes the new slot's fields
    if (st) return st;
    s->impl->tree.add_node(parent, offset);
    return AMR_OK;
}
AMR_API int amr_sim_remove_node(amr_sim* s, int32_t node) {
    if (!s || node < -1 || node >= (int32_t)s->impl->tree.max_slots()) return AMR_ERR_INVALID;
    s->impl->tree.remove_node(node);
    return AMR_OK;
}
AMR_API int amr_sim_add_nodes(amr_sim* s, const int32_t* parents, const int32_t* offsets, uint32_t n) {
    if (!s || (n && (!parents || !offsets))) return AMR_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++)
        if (parents[i] < 0 || (uint32_t)parents[i] >= s->impl->tree.max_slots() || offsets[i] < 0 || offsets[i] > 7)
            return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);   // node_ctor writes the new slots' fields
    if (st) return st;
    s->impl->tree.begin_batch();
    for (uint32_t i = 0; i < n; i++) s->impl->tree.add_node(parents[i], offsets[i]);
    s->impl->tree.end_batch();
    return s->impl->take_ctor_status();
}
AMR_API int amr_sim_remove_nodes(amr_sim* s, const int32_t* nodes, uint32_t n) {
    if (!s || (n && !nodes)) return AMR_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++)
        if (nodes[i] < -1 || nodes[i] >= (int32_t)s->impl->tree.max_slots()) return AMR_ERR_INVALID;
    s->impl->tree.begin_batch();
    for (uint32_t i = 0; i < n; i++) s->impl->tree.remove_node(nodes[i]);
    s->impl->tree.end_batch();
    return AMR_OK;
}
AMR_API int amr_sim_octree_state(const amr_sim* s, uint32_t* positions, int32_t* parent, int32_t* children,
                                 uint64_t* boundaries, uint32_t* lifetime, uint32_t* scalars) {
    if (!s) return AMR_ERR_INVALID;
    return octree_state_impl(s->impl->tree, positions, parent, children, boundaries, lifetime, scalars);
}
AMR_API int amr_sim_buffer(amr_sim* s, int which, int comp, void** ptr, uint64_t* count) {
    if (!s || !ptr || !count) return AMR_ERR_INVALID;
    return s->impl->buffer(which, comp, ptr, count);
}
static int sim_copy(amr_sim* s, int which, int comp, void* host, uint64_t count, bool to_device) {
    if (!s || !host) return AMR_ERR_INVALID;
    void* dev = nullptr;
    uint64_t n = 0;
    int st = s->impl->buffer(which, comp, &dev, &n);
    if (st) return st;
    if (count > n) return AMR_ERR_INVALID;
    if (count == 0) return AMR_OK;
    if (to_device && (st = s->impl->wait_side(which, comp))) return st;   // a side read of this buffer first
    return cuda_status(to_device ? cudaMemcpyAsync(dev, host, count * 4u, cudaMemcpyHostToDevice, s->impl->stream)
                                 : cudaMemcpyAsync(host, dev, count * 4u, cudaMemcpyDeviceToHost, s->impl->stream));
}
AMR_API int amr_sim_copy_to_host_side(amr_sim* s, int which, int comp, void* host, uint64_t count) {
    if (!s || !host || which < 0 || which >= 6 || comp < 0 || comp >= 6) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    void* dev = nullptr;
    uint64_t n = 0;
    int st = b->buffer(which, comp, &dev, &n);
    if (st) return st;
    if (count > n) return AMR_ERR_INVALID;
    if (count == 0) return AMR_OK;
    cudaError_t e = cudaSuccess;
    if (!b->side_stream) e = cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !b->main_mark) e = cudaEventCreateWithFlags(&b->main_mark, cudaEventDisableTiming);
    if (e == cudaSuccess && !b->side_done[which][comp])
        e = cudaEventCreateWithFlags(&b->side_done[which][comp], cudaEventDisableTiming);
    // after everything already enqueued on the simulation's stream ...
    if (e == cudaSuccess) e = cudaEventRecord(b->main_mark, b->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side_stream, b->main_mark, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, count * 4u, cudaMemcpyDeviceToHost, b->side_stream);
    // ... and before the next timestep or write of this buffer there
    if (e == cudaSuccess) e = cudaEventRecord(b->side_done[which][comp], b->side_stream);
    if (e != cudaSuccess) return cuda_status(e);
    b->side_pending[which][comp] = true;
    return AMR_OK;
}
AMR_API int amr_sim_stage_to_device(amr_sim* s, int which, int comp, const void* host, uint64_t count) {
    if (!s || !host || which < 0 || which >= 6 || comp < 0 || comp >= 6) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    void* dev = nullptr;
    uint64_t n = 0;
    int st = b->buffer(which, comp, &dev, &n);
    if (st) return st;
    if (count > n) return AMR_ERR_INVALID;
    if (count == 0) return AMR_OK;
    SimBase::Staging& u = b->up[which][comp];
    if ((st = b->ensure_transfer_streams()) || (st = u.ensure(n))) return st;
    // host -> staging on the upload stream, once the staging copy's previous contents are in place
    cudaError_t e = cudaStreamWaitEvent(b->up_stream, u.copied, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u.buf, host, count * 4u, cudaMemcpyHostToDevice, b->up_stream);
    if (e == cudaSuccess) e = cudaEventRecord(u.moved, b->up_stream);
    if (e != cudaSuccess) return cuda_status(e);
    // staging -> buffer on the simulation's stream, after everything enqueued there so far and a
    // side read of the buffer
    if ((st = b->wait_side(which, comp))) return st;
    e = cudaStreamWaitEvent(b->stream, u.moved, 0);
    if (e == cudaSuccess) e = launch_copy_words(dev, u.buf, count, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(u.copied, b->stream);
    b->launches++;
    return cuda_status(e);
}
AMR_API int amr_sim_snapshot_to_host(amr_sim* s, int which, int comp, void* host, uint64_t count) {
    if (!s || !host || which < 0 || which >= 6 || comp < 0 || comp >= 6) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    void* dev = nullptr;
    uint64_t n = 0;
    int st = b->buffer(which, comp, &dev, &n);
    if (st) return st;
    if (count > n) return AMR_ERR_INVALID;
    if (count == 0) return AMR_OK;
    SimBase::Staging& d = b->down[which][comp];
    if ((st = b->ensure_transfer_streams()) || (st = d.ensure(n))) return st;
    // buffer -> staging on the simulation's stream, once the previous snapshot has left it
    cudaError_t e = d.pending ? cudaStreamWaitEvent(b->stream, d.moved, 0) : cudaSuccess;
    if (e == cudaSuccess) e = launch_copy_words(d.buf, dev, count, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(d.copied, b->stream);
    b->launches++;
    // staging -> host on the download stream
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->down_stream, d.copied, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, d.buf, count * 4u, cudaMemcpyDeviceToHost, b->down_stream);
    if (e == cudaSuccess) e = cudaEventRecord(d.moved, b->down_stream);
    if (e != cudaSuccess) return cuda_status(e);
    d.pending = true;
    return AMR_OK;
}
// The batched forms: the same transfers for up to 36 distinct buffers, with one copy launch on the
// simulation's stream for all of them (host transfers stay one per buffer).
static int check_many(SimBase* b, uint32_t n, const int* which, const int* comp, const void* const* host,
                      const uint64_t* count, void** dev) {
    if (n > CopyList::kMax || (n && (!which || !comp || !host || !count))) return AMR_ERR_INVALID;
    for (uint32_t i = 0; i < n; i++) {
        if (which[i] < 0 || which[i] >= 6 || comp[i] < 0 || comp[i] >= 6 || !host[i]) return AMR_ERR_INVALID;
        for (uint32_t j = 0; j < i; j++)
            if (which[j] == which[i] && comp[j] == comp[i]) return AMR_ERR_INVALID;   // one staging copy each
        uint64_t cap = 0;
        const int st = b->buffer(which[i], comp[i], &dev[i], &cap);
        if (st) return st;
        if (count[i] > cap) return AMR_ERR_INVALID;
    }
    return b->ensure_transfer_streams();
}
AMR_API int amr_sim_stage_many(amr_sim* s, uint32_t n, const int* which, const int* comp, const void* const* host,
                               const uint64_t* count) {
    if (!s) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    void* dev[CopyList::kMax];
    int st = check_many(b, n, which, comp, host, count, dev);
    if (st) return st;
    // every staging allocation and every wait on a side read first: an error return then means
    // that nothing was queued
    for (uint32_t i = 0; i < n; i++) {
        if (count[i] == 0) continue;
        uint64_t cap = 0;
        void* unused = nullptr;
        if ((st = b->buffer(which[i], comp[i], &unused, &cap)) || (st = b->up[which[i]][comp[i]].ensure(cap)) ||
            (st = b->wait_side(which[i], comp[i])))
            return st;
    }
    CopyList list;
    SimBase::Staging* last = nullptr;
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++) {
        if (count[i] == 0) continue;
        SimBase::Staging& u = b->up[which[i]][comp[i]];
        e = cudaStreamWaitEvent(b->up_stream, u.copied, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(u.buf, host[i], count[i] * 4u, cudaMemcpyHostToDevice, b->up_stream);
        if (e == cudaSuccess) e = cudaEventRecord(u.moved, b->up_stream);
        list.item[list.n++] = {dev[i], u.buf, count[i]};
        last = &u;
    }
    if (e != cudaSuccess) return cuda_status(e);
    if (!last) return AMR_OK;
    // the upload stream runs in order: its last transfer done means all are
    e = cudaStreamWaitEvent(b->stream, last->moved, 0);
    if (e == cudaSuccess) e = launch_copy_many(list, b->stream);
    b->launches++;
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++)
        if (count[i]) e = cudaEventRecord(b->up[which[i]][comp[i]].copied, b->stream);
    return cuda_status(e);
}
AMR_API int amr_sim_snapshot_many(amr_sim* s, uint32_t n, const int* which, const int* comp, void* const* host,
                                  const uint64_t* count) {
    if (!s) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    void* dev[CopyList::kMax];
    int st = check_many(b, n, which, comp, const_cast<const void* const*>(host), count, dev);
    if (st) return st;
    for (uint32_t i = 0; i < n; i++) {   // staging allocations first: an error then queues nothing
        if (count[i] == 0) continue;
        uint64_t cap = 0;
        void* unused = nullptr;
        if ((st = b->buffer(which[i], comp[i], &unused, &cap)) || (st = b->down[which[i]][comp[i]].ensure(cap))) return st;
    }
    CopyList list;
    SimBase::Staging* first = nullptr;
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++) {
        if (count[i] == 0) continue;
        SimBase::Staging& d = b->down[which[i]][comp[i]];
        if (d.pending) e = cudaStreamWaitEvent(b->stream, d.moved, 0);   // the previous snapshot has left
        list.item[list.n++] = {d.buf, dev[i], count[i]};
        if (!first) first = &d;
    }
    if (e != cudaSuccess) return cuda_status(e);
    if (!first) return AMR_OK;
    e = launch_copy_many(list, b->stream);
    b->launches++;
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++)
        if (count[i]) e = cudaEventRecord(b->down[which[i]][comp[i]].copied, b->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->down_stream, first->copied, 0);
    for (uint32_t i = 0; i < n && e == cudaSuccess; i++) {
        if (count[i] == 0) continue;
        SimBase::Staging& d = b->down[which[i]][comp[i]];
        e = cudaMemcpyAsync(host[i], d.buf, count[i] * 4u, cudaMemcpyDeviceToHost, b->down_stream);
        if (e == cudaSuccess) e = cudaEventRecord(d.moved, b->down_stream);
        if (e == cudaSuccess) d.pending = true;
    }
    return cuda_status(e);
}
AMR_API int amr_sim_copy_to_device(amr_sim* s, int which, int comp, const void* host, uint64_t count) {
    return sim_copy(s, which, comp, const_cast<void*>(host), count, true);
}
AMR_API int amr_sim_copy_to_host(amr_sim* s, int which, int comp, void* host, uint64_t count) {
    return sim_copy(s, which, comp, host, count, false);
}
AMR_API int amr_sim_event_record(amr_sim* s, int slot) {
    if (!s || slot < 0 || slot >= 16) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    int st0 = b->wait_side(-1, 0);   // the event follows side copies and snapshot downloads too
    if (!st0) st0 = b->wait_snapshots();
    if (st0) return st0;
    if (!b->user_events[slot]) {
        const int st = cuda_status(cudaEventCreate(&b->user_events[slot]));
        if (st) return st;
    }
    return cuda_status(cudaEventRecord(b->user_events[slot], b->stream));
}
AMR_API int amr_sim_event_elapsed(amr_sim* s, int first, int second, float* ms) {
    if (!s || !ms || first < 0 || first >= 16 || second < 0 || second >= 16) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    if (!b->user_events[first] || !b->user_events[second]) return AMR_ERR_INVALID;
    const int st = cuda_status(cudaEventSynchronize(b->user_events[second]));
    if (st) return st;
    return cuda_status(cudaEventElapsedTime(ms, b->user_events[first], b->user_events[second]));
}
// ---------------------------------------------------------------- checkpoint
// Raw little-endian files, one per array, in the reference's io_helper.h:9-40 format (the buffer's
// bytes and nothing else), plus state.bin: kCheckpointWords uint32 words of identity and counters.
namespace {
constexpr uint32_t kCheckpointMagic = 0x54504B43u;   // "CKPT"
constexpr int kCheckpointWords = 16;

bool write_file(const std::string& path, const void* data, size_t bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}
bool read_file(const std::string& path, void* data, size_t bytes) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    bool ok = std::fread(data, 1, bytes, f) == bytes;
    ok = ok && std::fgetc(f) == EOF;   // exactly the expected size
    std::fclose(f);
    return ok;
}
int sim_kind(const SimBase* b) { return b->kind_id; }
}  // namespace

AMR_API int amr_sim_save(amr_sim* s, const char* dir) {
    if (!s || !dir) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    int st = b->sync_transfer_streams();
    if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
    if (st) return st;
    const std::string d(dir);
    const Octree& t = b->tree;
    const uint32_t slots = t.max_slots();
    uint32_t words[kCheckpointWords] = {};
    float outer = b->cfg.outer_size;
    words[0] = kCheckpointMagic; words[1] = 1u; words[2] = (uint32_t)sim_kind(b);
    words[3] = b->cfg.size_domain; words[4] = b->cfg.padding_domain; std::memcpy(&words[5], &outer, 4);
    words[6] = slots; words[7] = t.timer(); words[8] = (uint32_t)t.read_max_depth();
    words[9] = t.read_first_free_slot(); words[10] = t.final_used_slot(); words[11] = (uint32_t)b->rng;
    if (!write_file(d + "/state.bin", words, sizeof(words)) ||
        !write_file(d + "/positions.bin", t.positions().data(), slots * 4u) ||
        !write_file(d + "/parent.bin", t.parents().data(), slots * 4u) ||
        !write_file(d + "/children.bin", t.children().data(), (size_t)slots * 32u) ||
        !write_file(d + "/boundaries.bin", t.boundaries().data(), (size_t)slots * 48u) ||
        !write_file(d + "/lifetime.bin", t.lifetime().data(), slots * 4u))
        return AMR_ERR_INVALID;
    std::vector<uint8_t> host;
    for (int which = 0; which < 6; which++)
        for (int comp = 0; comp < kMaxFields; comp++) {
            void* ptr = nullptr;
            uint64_t count = 0;
            if (b->buffer(which, comp, &ptr, &count) != AMR_OK) continue;
            host.resize(count * 4u);
            if ((st = cuda_status(cudaMemcpy(host.data(), ptr, count * 4u, cudaMemcpyDeviceToHost)))) return st;
            if (!write_file(d + "/field_" + std::to_string(which) + "_" + std::to_string(comp) + ".bin", host.data(),
                            host.size()))
                return AMR_ERR_INVALID;
        }
    return AMR_OK;
}

// The device kernels index with these arrays and shift by (max_depth - depth): parents, children
// and boundary targets must name slots, the counter must lie in 0 .. 2^max_depth - 1, and every
// live node, and every boundary record of a live node, must be no deeper than max_depth (itself at
// most the depth limit).
static bool octree_state_valid(uint32_t slots, const uint32_t* pos, const int32_t* par, const int32_t* ch,
                               const uint64_t* bd, uint32_t timer, uint32_t max_depth, uint32_t first_free,
                               uint32_t used) {
    if (max_depth > kDepthLimit || timer >= (1u << max_depth) || first_free > slots || used == 0u || used > slots)
        return false;
    for (uint32_t i = 0; i < slots; i++) {
        const int d = pos_depth_host(pos[i]);
        if (d > (int)max_depth || par[i] < -1 || par[i] >= (int32_t)slots) return false;
    }
    for (size_t i = 0; i < (size_t)slots * 8u; i++)
        if (ch[i] < -1 || ch[i] >= (int32_t)slots) return false;
    for (size_t i = 0; i < (size_t)slots * 6u; i++) {
        const uint32_t nd = (uint32_t)bd[i];
        const int32_t target = (int32_t)((nd & 16777215u) | ((nd & (1u << 23)) ? 4278190080u : 0u));
        if (target < -1 || target >= (int32_t)slots) return false;
        // a record in use (a live node's, with a target) carries the node's depth in bits 28..31
        // and the depth difference to its target in bits 24..27
        if (target != -1 && pos_depth_host(pos[i / 6u]) != -1) {
            const uint32_t depth = nd >> 28, diff = (nd >> 24) & 15u;
            if (depth > max_depth || diff > depth) return false;
        }
    }
    return true;
}

AMR_API int amr_sim_set_octree(amr_sim* s, const uint32_t* positions, const int32_t* parent, const int32_t* children,
                               const uint64_t* boundaries, const uint32_t* lifetime, const uint32_t* scalars5) {
    if (!s || !positions || !parent || !children || !boundaries || !lifetime || !scalars5) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    const uint32_t slots = b->tree.max_slots();
    const uint32_t timer = scalars5[0], max_depth = scalars5[1], first_free = scalars5[2], used = scalars5[3];
    if (scalars5[4] != slots ||
        !octree_state_valid(slots, positions, parent, children, boundaries, timer, max_depth, first_free, used))
        return AMR_ERR_INVALID;
    int st = b->wait_side(-1, 0);   // side reads of the old tree's domains finish first
    if (st) return st;
    b->tree.restore(positions, parent, children, boundaries, lifetime, timer, (int)max_depth, first_free, used - 1u);
    b->graph_valid = false;
    return AMR_OK;
}

AMR_API int amr_sim_phase(amr_sim* s, int phase) {
    if (!s) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    if (phase < AMR_PHASE_COPY_BACK || phase > AMR_PHASE_INCREMENT_TIMER) return AMR_ERR_INVALID;
    const int st = b->wait_side(-1, 0);   // the phase may overwrite a buffer a side read still copies
    if (st) return st;
    switch (phase) {
        case AMR_PHASE_COPY_BACK: return b->copy_back();
        case AMR_PHASE_MODIFY_NODES: return b->modify_nodes();
        case AMR_PHASE_PREDICTOR: return b->predictor();
        case AMR_PHASE_COPY_BOUNDS: return b->copy_bounds();
        case AMR_PHASE_CORRECTOR: return b->corrector();
        default: b->tree.increment_timer(); return AMR_OK;
    }
}

AMR_API int amr_sim_load(amr_sim* s, const char* dir) {
    if (!s || !dir) return AMR_ERR_INVALID;
    SimBase* b = s->impl;
    int st = b->sync_transfer_streams();
    if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
    if (st) return st;
    const std::string d(dir);
    const uint32_t slots = b->tree.max_slots();
    uint32_t words[kCheckpointWords];
    float outer = b->cfg.outer_size;
    uint32_t outer_bits;
    std::memcpy(&outer_bits, &outer, 4);
    if (!read_file(d + "/state.bin", words, sizeof(words))) return AMR_ERR_INVALID;
    if (words[0] != kCheckpointMagic || words[1] != 1u || words[2] != (uint32_t)sim_kind(b) ||
        words[3] != b->cfg.size_domain || words[4] != b->cfg.padding_domain || words[5] != outer_bits ||
        words[6] != slots || words[8] > kDepthLimit || words[10] >= slots || words[9] > slots)
        return AMR_ERR_INVALID;
    std::vector<uint32_t> pos(slots), life(slots);
    std::vector<int32_t> par(slots), ch((size_t)slots * 8u);
    std::vector<uint64_t> bd((size_t)slots * 6u);
    if (!read_file(d + "/positions.bin", pos.data(), slots * 4u) || !read_file(d + "/parent.bin", par.data(), slots * 4u) ||
        !read_file(d + "/children.bin", ch.data(), (size_t)slots * 32u) ||
        !read_file(d + "/boundaries.bin", bd.data(), (size_t)slots * 48u) ||
        !read_file(d + "/lifetime.bin", life.data(), slots * 4u))
        return AMR_ERR_INVALID;
    if (!octree_state_valid(slots, pos.data(), par.data(), ch.data(), bd.data(), words[7], words[8], words[9],
                            words[10] + 1u))
        return AMR_ERR_INVALID;
    // every field file is read and size-checked before anything is uploaded, so that a missing or
    // truncated file leaves the simulation as it was
    std::vector<std::vector<uint8_t>> fields;
    std::vector<void*> targets;
    for (int which = 0; which < 6; which++)
        for (int comp = 0; comp < kMaxFields; comp++) {
            void* ptr = nullptr;
            uint64_t count = 0;
            if (b->buffer(which, comp, &ptr, &count) != AMR_OK) continue;
            fields.emplace_back(count * 4u);
            if (!read_file(d + "/field_" + std::to_string(which) + "_" + std::to_string(comp) + ".bin",
                           fields.back().data(), fields.back().size()))
                return AMR_ERR_INVALID;
            targets.push_back(ptr);
        }
    for (size_t i = 0; i < fields.size(); i++)
        if ((st = cuda_status(cudaMemcpy(targets[i], fields[i].data(), fields[i].size(), cudaMemcpyHostToDevice))))
            return st;
    b->tree.restore(pos.data(), par.data(), ch.data(), bd.data(), life.data(), words[7], (int)words[8], words[9],
                    words[10]);
    b->rng = (int32_t)words[11];
    b->graph_valid = false;
    return AMR_OK;
}

AMR_API int amr_sim_timestep(amr_sim* s) {
    if (!s) return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);
    return st ? st : s->impl->timestep();
}
AMR_API int amr_sim_copy_bounds(amr_sim* s) {
    if (!s) return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);
    return st ? st : s->impl->copy_bounds();
}
AMR_API int amr_sim_rng(const amr_sim* s, int32_t* seed) {
    if (!s || !seed) return AMR_ERR_INVALID;
    *seed = s->impl->rng;
    return AMR_OK;
}
AMR_API int amr_sim_set_rng(amr_sim* s, int32_t seed) {
    if (!s) return AMR_ERR_INVALID;
    s->impl->rng = seed;
    return AMR_OK;
}
AMR_API int amr_sim_stream(amr_sim* s, void** stream) {
    if (!s || !stream) return AMR_ERR_INVALID;
    *stream = s->impl->stream;
    return AMR_OK;
}
AMR_API int amr_sim_set_stream(amr_sim* s, void* stream) {
    if (!s) return AMR_ERR_INVALID;
    return s->impl->set_stream(static_cast<cudaStream_t>(stream));
}
AMR_API int amr_sim_synchronize(amr_sim* s) {
    if (!s) return AMR_ERR_INVALID;
    int st = s->impl->sync_transfer_streams();
    if (st) return st;
    st = cuda_status(cudaStreamSynchronize(s->impl->stream));
    if (st) return st;
    return take_device_error(s->impl->err_flag);
}
AMR_API int amr_sim_set_fault_injection(amr_sim* s, uint32_t spin_limit, uint32_t withhold_plane) {
    if (!s) return AMR_ERR_INVALID;
    s->impl->fault_spin_limit = spin_limit;
    s->impl->fault_withhold = withhold_plane;
    s->impl->graph_valid = false;
    return AMR_OK;
}
AMR_API uint64_t amr_sim_kernel_launches(const amr_sim* s) { return s ? s->impl->launches : 0u; }
AMR_API int amr_sim_autotune(amr_sim* s, uint32_t reps, uint32_t* n_tuned) {
    if (!s) return AMR_ERR_INVALID;
    return s->impl->autotune(reps, n_tuned);
}
AMR_API int amr_sim_tuned_shapes(const amr_sim* s, uint32_t capacity, uint32_t* domains, uint32_t* ctas,
                                 uint32_t* count) {
    if (!s || !count || (capacity && (!domains || !ctas))) return AMR_ERR_INVALID;
    const auto& t = s->impl->tuned_ctas;
    *count = (uint32_t)t.size();
    for (uint32_t i = 0; i < capacity && i < t.size(); i++) { domains[i] = t[i].first; ctas[i] = t[i].second; }
    return t.size() > capacity ? AMR_ERR_CAPACITY : AMR_OK;
}
AMR_API int amr_sim_set_stencil_ctas(amr_sim* s, uint32_t ctas) {
    if (!s || ctas > (1u << 20)) return AMR_ERR_INVALID;
    s->impl->stencil_ctas = ctas;
    s->impl->graph_valid = false;
    return AMR_OK;
}
AMR_API int amr_sim_enable_kernel_timing(amr_sim* s, int enable) {
    if (!s) return AMR_ERR_INVALID;
    if (enable && s->impl->mode == AMR_MODE_GRAPH) return AMR_ERR_INVALID;
    s->impl->timing = enable != 0;
    return AMR_OK;
}
AMR_API int amr_sim_kernel_timing(amr_sim* s, double* ms, uint64_t* n) {
    if (!s || !ms || !n) return AMR_ERR_INVALID;
    return s->impl->harvest_timing(ms, n);
}
