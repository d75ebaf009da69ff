// evolve_sim.cu -- simulations of the evolution kinds (AMR_SIM_BSSN_EVOLVE, AMR_SIM_WAVE_RK4) on the
// amr_sim object: the reference's timestep loop (AMR.h:324-333) with RK4 substeps (evolve.h).
//
// Phases of one substep (the plugin interface's names):
//   copy_back     restriction of every active domain: old <- new, child-covered cells <- the child's
//                 new field at the cell's centre, fourth order (the reference's copy_new_to_old,
//                 AMR.h:961-996, averages the 2x2x2 cells: second order)
//   modify_nodes  nothing (regridding is driven from outside between timesteps: amr_sim_regrid, or
//                 amr_sim_add_nodes / remove_nodes; new domains are interpolated tricubically)
//   predictor     the four RK4 stages over the active evolved domains, each a derivative pass and a
//                 pointwise update, with the ghost cells of stages 2-4 filled in between
//   copy_bounds   ghost fill of the final state (so that the next restriction copies valid ghosts)
//   corrector     nothing (RK4 has no separate corrector stage)
// Modes: PLAIN launches every kernel once per domain (the plain per-domain form), BATCHED once per
// phase over the substep's active domains, GRAPH replays a captured CUDA graph of a whole timestep.
// Buffers per field: old (state at the start of a step), new (final state; also the stage-3 input),
// stage (stages 2 and 4), all padded; the RK accumulator (inner layout).
#include <algorithm>

#include "evolve_kernels.h"
#include "sim_base.h"

namespace amr {

class EvolveSim : public SimBase {
public:
    EvolveSim(const amr_config& c, int kind, uint32_t slots, int mode) : SimBase(c, slots, mode), kind(kind) {
        nf = kind == AMR_SIM_BSSN_EVOLVE ? BSSN_NF : WAVE_NF;
        nd = kind == AMR_SIM_BSSN_EVOLVE ? BSSN_ND_CONSTRAINTS : WAVE_ND;
        kind_id = kind;
        prm.physics = kind == AMR_SIM_BSSN_EVOLVE ? 0 : 1;
        prm.slicing = AMR_SLICING_1PLUSLOG;
        prm.shift = 0;
        prm.eta = 2.f;
        prm.ko_sigma = .1f;
        prm.cfl = .25f;
        prm.chi_floor = 1e-6f;
        prm.outer_size = c.outer_size;
    }
    ~EvolveSim() override {
        if (stream) cudaStreamSynchronize(stream);
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        for (int f = 0; f < kMaxFields; f++) { cudaFree(old_f[f]); cudaFree(new_f[f]); cudaFree(stage_f[f]); cudaFree(acc[f]); }
        for (float* c : cons.c) cudaFree(c);
        cudaFree(deriv); cudaFree(d_evolved); cudaFree(d_lists); cudaFree(d_part); cudaFree(d_norms);
        cudaFree(d_feat); cudaFree(d_ind); cudaFree(d_pred);
    }
    int init() override {
        int st = SimBase::init();
        if (st) return st;
        const size_t s = tree.max_slots();
        const size_t padded = s * dims.t * dims.t * dims.t, inner = s * dims.n * dims.n * dims.n;
        cudaError_t e = cudaSuccess;
        for (int f = 0; f < nf && e == cudaSuccess; f++) {
            e = dev_alloc(&old_f[f], padded);
            if (e == cudaSuccess) e = dev_alloc(&new_f[f], padded);
            if (e == cudaSuccess) e = dev_alloc(&stage_f[f], padded);
            if (e == cudaSuccess) e = dev_alloc(&acc[f], inner);
        }
        if (e == cudaSuccess) e = dev_alloc(&deriv, inner * (size_t)nd);
        for (int k = 0; k < 4 && e == cudaSuccess && kind == AMR_SIM_BSSN_EVOLVE; k++) e = dev_alloc(&cons.c[k], inner);
        if (e == cudaSuccess) e = dev_alloc(&d_evolved, s);
        if (e == cudaSuccess) e = dev_alloc(&d_lists, s * 2u * ((size_t)1u << kDepthLimit) + 2u * s);
        if (e == cudaSuccess) e = dev_alloc(&d_part, s * 5u);
        if (e == cudaSuccess) e = dev_alloc(&d_norms, 8);
        if (e == cudaSuccess) {   // the derivative pass's shared-memory limit, outside any stream capture
            EvoArgs none;
            std::memset(&none, 0, sizeof(none));
            none.n = dims.n;
            e = launch_evo_derivs(none, stream);
        }
        return cuda_status(e);
    }

    // ---- node constructors: both state buffers of every field of a new domain by tricubic
    // interpolation of its parent's padded state (fourth order, in place of the reference's rule,
    // AMR.h:1053-1115, whose second-order error seeds O(1) constraint violations on refined cells;
    // chi and alpha through their fourth and square roots)
    void node_ctor(int32_t node) override {
        const NodeCtor c = {node, tree.parents()[node], (int32_t)pos_final_offset(tree.positions()[node])};
        const uint32_t end = 1;
        node_ctor_groups(&c, &end, 1);
    }
    void node_ctor_groups(const NodeCtor* items, const uint32_t* group_end, uint32_t groups) override {
        graph_valid = false;
        lists_valid = false;
        const size_t n = groups ? group_end[groups - 1] : 0u;
        if (n == 0 || !upload_ctor_items(items, n)) return;
        EvoProlongArgs g;
        std::memset(&g, 0, sizeof(g));
        for (int f = 0; f < nf; f++) { g.bufs[f] = old_f[f]; g.bufs[nf + f] = new_f[f]; }
        g.nbuf = 2u * (uint32_t)nf;
        g.n = dims.n; g.p = dims.p; g.t = dims.t;
        const bool bssn = kind == AMR_SIM_BSSN_EVOLVE;   // chi, stored less 1, kept at its floor
        g.floor_buf[0] = bssn ? F_CHI : -1;
        g.floor_buf[1] = bssn ? nf + F_CHI : -1;
        g.floor_val = prm.chi_floor - 1.f;
        if (bssn)
            for (int b = 0; b < 2; b++) { g.root[b * nf + F_CHI] = 4; g.root[b * nf + F_ALPHA] = 2; }
        cudaError_t e = cudaSuccess;
        for (uint32_t k = 0, b = 0; k < groups && e == cudaSuccess; b = group_end[k++]) {   // depth order
            g.items = reinterpret_cast<const int32_t*>(ctor_items + b);
            g.n_items = group_end[k] - b;
            e = launch_evo_prolong(g, stream);
            launches++;
        }
        if (e != cudaSuccess) ctor_status = cuda_status(e);
    }
    void node_dtor(int32_t) override { lists_valid = false; }

    int buffer(int which, int comp, void** ptr, uint64_t* count) override {
        const uint64_t s = tree.max_slots();
        const uint64_t padded = s * dims.t * dims.t * dims.t, inner = s * dims.n * dims.n * dims.n;
        if (comp < 0) return AMR_ERR_INVALID;
        switch (which) {
            case 0: if (comp >= nf) return AMR_ERR_INVALID; *ptr = old_f[comp]; *count = padded; return AMR_OK;
            case 1: if (comp >= nf) return AMR_ERR_INVALID; *ptr = new_f[comp]; *count = padded; return AMR_OK;
            case 2: if (comp >= nf) return AMR_ERR_INVALID; *ptr = stage_f[comp]; *count = padded; return AMR_OK;
            case 3: if (comp >= nf) return AMR_ERR_INVALID; *ptr = acc[comp]; *count = inner; return AMR_OK;
            case 4: if (comp >= 4 || !cons.c[comp]) return AMR_ERR_INVALID; *ptr = cons.c[comp]; *count = inner; return AMR_OK;
            case 5: if (comp >= nd) return AMR_ERR_INVALID; *ptr = deriv + (size_t)comp * inner; *count = inner; return AMR_OK;
            default: return AMR_ERR_INVALID;
        }
    }

    // ---- lists per substep: active domains (restriction) and active evolved domains
    int build_lists() {
        if (lists_valid) return AMR_OK;
        const uint32_t md = (uint32_t)tree.read_max_depth(), used = tree.curr_used_slots();
        const uint32_t nsub = 1u << md;
        std::vector<uint8_t> evolved(tree.max_slots(), 0);
        leaves.clear();
        // Every live domain is evolved, covered parents included: a leaf beside a covered parent of
        // its own depth takes its ghost values from it at every stage (and the parent's values are
        // replaced by its children's at each restriction).
        for (uint32_t i = 0; i < used; i++) {
            if (pos_depth_host(tree.positions()[i]) == -1) continue;
            int nchild = 0;
            for (int c = 0; c < 8; c++) nchild += tree.children()[(size_t)i * 8u + c] != -1;
            evolved[i] = 1;
            if (nchild == 0) leaves.push_back(i);
        }
        std::vector<uint8_t> is_leaf(tree.max_slots(), 0);
        for (uint32_t i : leaves) is_leaf[i] = 1;
        std::vector<uint32_t> all, sub;
        act_off.assign(nsub, 0); act_cnt.assign(nsub, 0); act_leaves.assign(nsub, 0);
        evo_off.assign(nsub, 0); evo_cnt.assign(nsub, 0);
        for (uint32_t s = 0; s < nsub; s++) {
            sub.clear();   // the substep's active domains in slot order
            for (uint32_t i = 0; i < used; i++) {
                const int d = pos_depth_host(tree.positions()[i]);
                if (d != -1 && (s & ((1u << (md - (uint32_t)d)) - 1u)) == 0u) sub.push_back(i);
            }
            // the restriction's list: the leaves (straight copies) first, then the domains with children
            act_off[s] = (uint32_t)all.size();
            for (uint32_t i : sub) if (is_leaf[i]) all.push_back(i);
            act_leaves[s] = (uint32_t)all.size() - act_off[s];
            for (uint32_t i : sub) if (!is_leaf[i]) all.push_back(i);
            act_cnt[s] = (uint32_t)all.size() - act_off[s];
            evo_off[s] = (uint32_t)all.size();
            for (uint32_t i : sub) if (evolved[i]) all.push_back(i);
            evo_cnt[s] = (uint32_t)all.size() - evo_off[s];
        }
        all_evolved_off = (uint32_t)all.size();
        for (uint32_t i = 0; i < used; i++)
            if (evolved[i]) all.push_back(i);
        all_evolved_cnt = (uint32_t)all.size() - all_evolved_off;
        leaves_off = (uint32_t)all.size();
        all.insert(all.end(), leaves.begin(), leaves.end());
        const size_t cap = (size_t)tree.max_slots() * 2u * ((size_t)1u << kDepthLimit) + 2u * tree.max_slots();
        if (all.size() > cap) return AMR_ERR_CAPACITY;
        cudaError_t e = cudaMemcpyAsync(d_lists, all.data(), all.size() * 4u, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_evolved, evolved.data(), evolved.size(), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_status(e);
        lists_valid = true;
        return AMR_OK;
    }
    int prepare() {
        int st = sync_octree();
        if (st) return st;
        if (!items_valid) { lists_valid = false; items_valid = true; }
        return build_lists();
    }

    // ---- phases
    int copy_back() override {
        int st = prepare();
        if (st) return st;
        const uint32_t s = tree.timer(), md = (uint32_t)tree.read_max_depth();
        if (act_cnt[s] == 0) return AMR_OK;
        EvoRestrictArgs g;
        std::memset(&g, 0, sizeof(g));
        for (int f = 0; f < nf; f++) { g.old_f[f] = old_f[f]; g.new_f[f] = new_f[f]; }
        g.children = d_children;
        g.items = d_lists + act_off[s];
        g.n_items = act_cnt[s];
        g.n = dims.n; g.p = dims.p; g.t = dims.t;
        g.nf = nf;
        g.fgroup = nf;
        (void)md;
        if (mode == AMR_MODE_PLAIN) {   // one launch per domain
            const uint32_t* base = g.items;
            for (uint32_t i = 0; i < act_cnt[s]; i++) {
                g.items = base + i;
                g.n_items = 1;
                if ((st = check(launch_evo_restrict(g, stream)))) return st;
            }
            return AMR_OK;
        }
        // the leaves with every field of a plane per CTA, then the domains with children with
        // kEvoRestrictGroup fields per CTA
        g.n_items = act_leaves[s];
        if (g.n_items && (st = check(launch_evo_restrict(g, stream)))) return st;
        g.items = d_lists + act_off[s] + act_leaves[s];
        g.n_items = act_cnt[s] - act_leaves[s];
        g.fgroup = kEvoRestrictGroup;
        if (g.n_items && (st = check(launch_evo_restrict(g, stream)))) return st;
        return AMR_OK;
    }
    int modify_nodes() override { return AMR_OK; }
    int predictor() override {
        int st = prepare();
        if (st) return st;
        const uint32_t s = tree.timer();
        if (evo_cnt[s] == 0) return AMR_OK;
        float* const* in[4] = {old_f, stage_f, new_f, stage_f};
        float* const* out[4] = {stage_f, new_f, stage_f, new_f};
        const float c_next[3] = {.5f, .5f, 1.f};
        for (int stage = 1; stage <= 4; stage++) {
            EvoArgs a = args(s, in[stage - 1], out[stage - 1], stage, 0);
            if (mode == AMR_MODE_PLAIN) {
                // the plain per-domain form: each domain's derivative pass and update launched alone
                const uint32_t* base = a.items;
                for (uint32_t i = 0; i < evo_cnt[s]; i++) {
                    a.items = base + i;
                    a.n_items = 1;
                    if ((st = check(launch_evo_derivs(a, stream))) || (st = check(launch_evo_rhs(a, stream)))) return st;
                }
            } else {
                if ((st = check(launch_evo_derivs(a, stream)))) return st;
                time_begin();
                if ((st = check(launch_evo_rhs(a, stream)))) return st;
                time_end();
            }
            if (stage < 4 && (st = fill(s, out[stage - 1], c_next[stage - 1]))) return st;
        }
        return AMR_OK;
    }
    int copy_bounds() override {
        int st = prepare();
        if (st) return st;
        return fill(tree.timer(), new_f, 1.f);
    }
    int corrector() override { return AMR_OK; }

    int timestep() override {
        if (mode != AMR_MODE_GRAPH) return SimBase::timestep();
        int st = prepare();
        if (st) return st;
        if (tree.timer() != 0u) return SimBase::timestep();
        const uint32_t nsub = 1u << tree.read_max_depth();
        if (!graph_valid) {
            if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
            cudaGraph_t graph;
            cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_status(e);
            capturing = true;
            const uint64_t before = launches;
            st = SimBase::timestep();
            capturing = false;
            e = cudaStreamEndCapture(stream, &graph);
            if (st) { if (e == cudaSuccess) cudaGraphDestroy(graph); return st; }
            if (e != cudaSuccess) return cuda_status(e);
            e = cudaGraphInstantiate(&graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(e);
            graph_launches = launches - before;
            launches = before;
            graph_valid = true;
            // the capture ran the host loop (counter and lifetimes) without device work: replay it
            const cudaError_t e2 = cudaGraphLaunch(graph_exec, stream);
            if (e2 != cudaSuccess) return cuda_status(e2);
            launches += graph_launches;
            return AMR_OK;
        }
        const cudaError_t e = cudaGraphLaunch(graph_exec, stream);
        if (e != cudaSuccess) return cuda_status(e);
        launches += graph_launches;
        for (uint32_t s = 0; s < nsub; s++) tree.increment_timer();
        return AMR_OK;
    }

    // ---- evolution interface
    int set_evolution(const amr_evolution& e) {
        if (!(e.cfl > 0.f) || e.cfl > 1.f || e.ko_sigma < 0.f || e.eta < 0.f) return AMR_ERR_INVALID;
        if (e.slicing != AMR_SLICING_1PLUSLOG && e.slicing != AMR_SLICING_HARMONIC) return AMR_ERR_INVALID;
        prm.slicing = e.slicing;
        prm.shift = e.shift ? 1 : 0;
        prm.eta = e.eta;
        prm.ko_sigma = e.ko_sigma;
        prm.cfl = e.cfl;
        tree.set_periodic(e.periodic != 0);
        graph_valid = false;
        return AMR_OK;
    }
    int initial_data(const amr_initial_data& d) {
        int st = sync_octree();
        if (st) return st;
        EvoInitArgs a;
        std::memset(&a, 0, sizeof(a));
        for (int f = 0; f < nf; f++) { a.out1[f] = old_f[f]; a.out2[f] = new_f[f]; a.out3[f] = stage_f[f]; }
        a.positions = d_positions;
        a.used = tree.curr_used_slots();
        a.n = dims.n;
        a.t = dims.t;
        a.nf = nf;
        a.physics = prm.physics;
        a.outer_size = cfg.outer_size;
        a.id.kind = d.kind;
        a.id.amplitude = d.amplitude;
        a.id.wavelength = d.wavelength;
        a.id.n_punctures = std::min(d.n_punctures, 4);
        for (int i = 0; i < 4; i++) {
            a.id.mass[i] = d.mass[i];
            for (int k = 0; k < 3; k++) a.id.pos[i][k] = d.position[i][k];
        }
        a.id.width = d.width;
        id_used = a.id;
        tree.set_timer(0u);
        return check(launch_evo_init(a, stream));
    }
    // Launch-shape tuning of the derivative pass (amr_sim_autotune): its slab depth (interior
    // z-planes per CTA) timed at every compiled depth over all evolved domains, reps launches each
    // with CUDA events; the fastest is kept.  The pass writes only its derivative scratch, which
    // every RK stage rewrites, so the state is unchanged.
    int autotune(uint32_t reps, uint32_t* n_tuned) override {
        if (n_tuned) *n_tuned = 0;
        if (capturing || reps == 0u || reps > 100u) return AMR_ERR_INVALID;
        int st = wait_side(-1, 0);
        if (!st) st = prepare();
        if (st) return st;
        if (all_evolved_cnt == 0u) return AMR_OK;
        uint32_t cand[4];
        const uint32_t nc = evo_deriv_zs_candidates(dims.n, cand);
        EvoArgs a = args(0, new_f, new_f, 1, 0);
        a.items = d_lists + all_evolved_off;
        a.n_items = all_evolved_cnt;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        cudaError_t e = cudaEventCreate(&ev[0]);
        if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
        uint32_t best = 0;
        float best_ms = 0.f;
        for (uint32_t i = 0; i < nc && e == cudaSuccess; i++) {
            a.deriv_zs = cand[i];
            e = launch_evo_derivs(a, stream);   // warm-up
            if (e == cudaSuccess) e = cudaEventRecord(ev[0], stream);
            for (uint32_t r = 0; r < reps && e == cudaSuccess; r++) e = launch_evo_derivs(a, stream);
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (e == cudaSuccess && (best == 0u || ms < best_ms)) { best = cand[i]; best_ms = ms; }
        }
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (e != cudaSuccess) return cuda_status(e);
        if ((st = take_device_error(err_flag))) return st;
        deriv_zs = best;
        tuned_ctas.assign(1, {all_evolved_cnt, best});
        graph_valid = false;
        if (n_tuned) *n_tuned = 1;
        return AMR_OK;
    }
    int constraint_norms(float excision, double* out) {
        if (kind != AMR_SIM_BSSN_EVOLVE) return AMR_ERR_INVALID;
        int st = prepare();
        if (st) return st;
        // derivatives of the current state (new) on every evolved domain, then the constraints
        EvoArgs a = args(0, new_f, new_f, 0, 1);
        a.items = d_lists + all_evolved_off;
        a.n_items = all_evolved_cnt;
        if ((st = check(launch_evo_derivs(a, stream)))) return st;
        if ((st = check(launch_evo_constraints(a, cons, stream)))) return st;
        EvoNormArgs g;
        std::memset(&g, 0, sizeof(g));
        g.cons = cons;
        g.items = a.items;
        g.n_items = a.n_items;
        g.n = dims.n;
        g.positions = d_positions;
        g.children = d_children;
        g.outer_size = cfg.outer_size;
        g.excision2 = excision * excision;
        g.n_punctures = excision > 0.f ? id_used.n_punctures : 0;
        for (int i = 0; i < 4; i++)
            for (int k = 0; k < 3; k++) g.pos[i][k] = id_used.pos[i][k];
        if ((st = check(launch_evo_norms(g, d_part, d_norms, stream)))) return st;
        cudaError_t e = cudaMemcpyAsync(out, d_norms, 5 * sizeof(double), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        return cuda_status(e);
    }

    // ---- refinement (the learned estimator with the plain criterion as fallback and judge)
    // Features and plain-criterion indicators of every leaf, in leaf order (device buffers kept).
    int tile_features(std::vector<uint32_t>& leaf_slots) {
        if (kind != AMR_SIM_BSSN_EVOLVE) return AMR_ERR_INVALID;
        int st = prepare();
        if (st) return st;
        leaf_slots = leaves;
        const size_t need = leaves.size();
        if (need > feat_cap) {
            cudaStreamSynchronize(stream);
            cudaFree(d_feat); cudaFree(d_ind); cudaFree(d_pred);
            d_feat = d_ind = d_pred = nullptr;
            feat_cap = 0;
            cudaError_t e = dev_alloc(&d_feat, need * 1536u);
            if (e == cudaSuccess) e = dev_alloc(&d_ind, need);
            if (e == cudaSuccess) e = dev_alloc(&d_pred, need);
            if (e != cudaSuccess) return cuda_status(e);
            feat_cap = need;
        }
        EvoFeatureArgs g;
        std::memset(&g, 0, sizeof(g));
        for (int f = 0; f < nf; f++) g.state[f] = new_f[f];
        g.positions = d_positions;
        g.items = d_lists + leaves_off;
        g.n_items = (uint32_t)leaves.size();
        g.n = dims.n; g.p = dims.p; g.t = dims.t;
        g.outer_size = cfg.outer_size;
        g.features = d_feat;
        g.indicator = d_ind;
        return check(launch_evo_features(g, stream));
    }
    int regrid(amr_estimator* est, const amr_regrid& r, uint32_t* stats) {
        std::vector<uint32_t> leaf;
        int st = tile_features(leaf);
        if (st) return st;
        const size_t nl = leaf.size();
        std::vector<float> ind(nl), pred(nl, 0.f);
        cudaError_t e = cudaMemcpyAsync(ind.data(), d_ind, nl * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return cuda_status(e);
        if (est) {
            if ((st = amr_estimator_forward(est, d_feat, (uint32_t)nl, d_pred))) return st;
            if ((e = cudaMemcpy(pred.data(), d_pred, nl * 4, cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_status(e);
        }
        // decisions per leaf: refine by the network (or the plain criterion without one); the
        // plain criterion overrides a network that declines a tile whose indicator exceeds
        // judge_factor times its own refinement threshold
        const auto& pos = tree.positions();
        const auto& ch = tree.children();
        uint32_t refined = 0, coarsened = 0, overridden = 0;
        std::vector<int32_t> add_p, add_o;
        std::vector<char> calm(tree.max_slots(), 0);   // leaf whose criterion allows coarsening
        for (size_t i = 0; i < nl; i++) {
            const uint32_t sl = leaf[i];
            const int d = pos_depth_host(pos[sl]);
            const bool plain_refine = ind[i] > r.refine_threshold;
            const bool judge = ind[i] > r.judge_factor * r.refine_threshold;
            bool refine = est ? pred[i] > r.learned_refine : plain_refine;
            if (est && !refine && judge) { refine = true; overridden++; }
            calm[sl] = !refine && (est ? (pred[i] < r.learned_coarsen && !plain_refine) : ind[i] < r.coarsen_threshold);
            if (refine && (uint32_t)d < r.max_depth) {
                for (int c = 0; c < 8; c++) { add_p.push_back((int32_t)sl); add_o.push_back(c); }
                refined++;
            }
        }
        // coarsen: parents whose eight children are all calm leaves, above the minimum depth
        std::vector<int32_t> rem;
        const uint32_t used = tree.curr_used_slots();
        for (uint32_t sl = 0; sl < used; sl++) {
            const int d = pos_depth_host(pos[sl]);
            if (d == -1 || (uint32_t)d < r.min_depth) continue;
            bool all = true;
            for (int c = 0; c < 8 && all; c++) {
                const int32_t k = ch[(size_t)sl * 8u + c];
                all = k != -1 && calm[k];
                if (all)
                    for (int cc = 0; cc < 8; cc++) all &= ch[(size_t)k * 8u + cc] == -1;
            }
            if (!all) continue;
            for (int c = 0; c < 8; c++) rem.push_back(ch[(size_t)sl * 8u + c]);
            coarsened++;
        }
        // Between root steps every domain holds its state at one time in `new`; `old` (the start of
        // each domain's last step) is rewritten by the next step's restriction.  Setting old = new
        // first makes every ghost fill below take the current state: the fill blends a coarser
        // neighbour's old and new states by the substep's time fraction.
        auto sync_old = [&]() -> int {
            const size_t bytes = (size_t)tree.max_slots() * dims.t * dims.t * dims.t * 4u;
            for (int f = 0; f < nf; f++) {
                const cudaError_t ce = cudaMemcpyAsync(old_f[f], new_f[f], bytes, cudaMemcpyDeviceToDevice, stream);
                if (ce != cudaSuccess) return cuda_status(ce);
            }
            return AMR_OK;
        };
        if (!rem.empty() || !add_p.empty()) {
            if ((st = sync_old())) return st;
        }
        if (!rem.empty()) {
            tree.begin_batch();
            for (int32_t k : rem) tree.remove_node(k);
            tree.end_batch();
        }
        if (!add_p.empty()) {
            // the parents' ghost layers feed the new domains' interpolation stencils at their faces
            if ((st = prepare()) || (st = fill(tree.timer(), new_f, 1.f))) return st;
            tree.begin_batch();
            for (size_t i = 0; i < add_p.size(); i++) tree.add_node(add_p[i], add_o[i]);
            tree.end_batch();
        }
        if ((st = take_ctor_status())) return st;
        lists_valid = false;
        graph_valid = false;
        if (!rem.empty() || !add_p.empty()) {
            // the ghost cells from the new neighbours, in both state buffers
            if ((st = prepare()) || (st = fill(tree.timer(), new_f, 1.f)) || (st = sync_old())) return st;
        }
        if (stats) {
            stats[0] = refined;
            stats[1] = coarsened;
            stats[2] = overridden;
            stats[3] = (uint32_t)(nl + 7u * refined - 7u * coarsened);
        }
        return AMR_OK;
    }
    float* features_ptr() const { return d_feat; }
    float* indicator_ptr() const { return d_ind; }

private:
    float* d_feat = nullptr;
    float* d_ind = nullptr;
    float* d_pred = nullptr;
    size_t feat_cap = 0;

    EvoArgs args(uint32_t s, float* const* in, float* const* out, int stage, int constraints) {
        EvoArgs a;
        std::memset(&a, 0, sizeof(a));
        for (int f = 0; f < nf; f++) {
            a.fields[f] = in[f];
            a.out[f] = out[f];
            a.old_f[f] = old_f[f];
            a.acc[f] = acc[f];
        }
        a.deriv = deriv;
        a.deriv_stride = (uint64_t)tree.max_slots() * dims.n * dims.n * dims.n;
        a.positions = d_positions;
        a.items = d_lists + (evo_off.empty() ? 0u : evo_off[s]);
        a.n_items = evo_cnt.empty() ? 0u : evo_cnt[s];
        a.n = dims.n;
        a.p = dims.p;
        a.t = dims.t;
        a.dt0 = prm.cfl * cfg.outer_size / (float)dims.n;
        a.stage = stage;
        a.constraints = constraints;
        a.deriv_zs = deriv_zs;
        a.prm = prm;
        a.err = err_flag;
        return a;
    }
    // ghost fill of `x` (the state at c_stage of the active domains' step), three axis passes
    int fill(uint32_t s, float* const* x, float c_stage) {
        if (evo_cnt[s] == 0) return AMR_OK;
        EvoGhostArgs g;
        std::memset(&g, 0, sizeof(g));
        for (int f = 0; f < nf; f++) { g.X[f] = x[f]; g.old_f[f] = old_f[f]; g.new_f[f] = new_f[f]; }
        g.boundaries = d_boundaries;
        g.evolved = d_evolved;
        g.items = d_lists + evo_off[s];
        g.n_items = evo_cnt[s];
        g.n = dims.n; g.p = dims.p; g.t = dims.t;
        g.substep = s;
        g.max_depth = (uint32_t)tree.read_max_depth();
        g.nf = nf;
        g.c_stage = c_stage;
        g.err = err_flag;
        for (int axis = 0; axis < 3; axis++) {   // every domain's pass along an axis before the next axis
            g.axis = axis;
            if (mode == AMR_MODE_PLAIN) {   // one launch per domain
                const uint32_t* base = d_lists + evo_off[s];
                for (uint32_t i = 0; i < evo_cnt[s]; i++) {
                    g.items = base + i;
                    g.n_items = 1;
                    const int st = check(launch_evo_ghost(g, stream));
                    if (st) return st;
                }
                continue;
            }
            const int st = check(launch_evo_ghost(g, stream));
            if (st) return st;
        }
        return AMR_OK;
    }

    int kind, nf, nd;
    EvoParams prm;
    InitData id_used = {};     // the last initial data (puncture positions for the excision)
    float* old_f[kMaxFields] = {};
    float* new_f[kMaxFields] = {};
    float* stage_f[kMaxFields] = {};
    float* acc[kMaxFields] = {};
    float* deriv = nullptr;
    ConsPtrs cons = {};
    uint8_t* d_evolved = nullptr;
    uint32_t* d_lists = nullptr;
    double* d_part = nullptr;
    double* d_norms = nullptr;
    bool lists_valid = false;
    std::vector<uint32_t> act_off, act_cnt, act_leaves, evo_off, evo_cnt, leaves;
    uint32_t all_evolved_off = 0, all_evolved_cnt = 0, leaves_off = 0;
    uint32_t deriv_zs = 0;   // the derivative pass's slab depth (0: the default; amr_sim_autotune)
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_launches = 0;
};

SimBase* make_evolve_sim(const amr_config& c, int kind, uint32_t slots, int mode) {
    return new (std::nothrow) EvolveSim(c, kind, slots, mode);
}
bool is_evolve_sim(const SimBase* s) { return dynamic_cast<const EvolveSim*>(s) != nullptr; }

}  // namespace amr

using namespace amr;

#define AMR_API extern "C" __attribute__((visibility("default")))

AMR_API int amr_sim_set_evolution(amr_sim* s, const amr_evolution* e) {
    if (!s || !e) return AMR_ERR_INVALID;
    EvolveSim* v = dynamic_cast<EvolveSim*>(s->impl);
    if (!v) return AMR_ERR_INVALID;
    return v->set_evolution(*e);
}
AMR_API int amr_sim_initial_data(amr_sim* s, const amr_initial_data* d) {
    if (!s || !d) return AMR_ERR_INVALID;
    EvolveSim* v = dynamic_cast<EvolveSim*>(s->impl);
    if (!v) return AMR_ERR_INVALID;
    if (d->kind < AMR_ID_FLAT || d->kind > AMR_ID_GAUSSIAN_PULSE || d->n_punctures < 0 || d->n_punctures > 4)
        return AMR_ERR_INVALID;
    if (d->kind == AMR_ID_GAUGE_WAVE && !(d->wavelength > 0.f)) return AMR_ERR_INVALID;
    if (d->kind == AMR_ID_GAUSSIAN_PULSE && !(d->width > 0.f)) return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);
    return st ? st : v->initial_data(*d);
}
AMR_API int amr_sim_tile_features(amr_sim* s, float* features, float* indicators, uint32_t* leaf_slots,
                                  uint32_t capacity, uint32_t* n_leaves) {
    if (!s || !n_leaves) return AMR_ERR_INVALID;
    EvolveSim* v = dynamic_cast<EvolveSim*>(s->impl);
    if (!v) return AMR_ERR_INVALID;
    int st = s->impl->wait_side(-1, 0);
    std::vector<uint32_t> leaf;
    if (!st) st = v->tile_features(leaf);
    if (st) return st;
    *n_leaves = (uint32_t)leaf.size();
    if (leaf.size() > capacity) return AMR_ERR_CAPACITY;
    cudaStream_t stream = s->impl->stream;
    cudaError_t e = cudaSuccess;
    if (features && !leaf.empty())
        e = cudaMemcpyAsync(features, v->features_ptr(), leaf.size() * 1536u * 4u, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess && indicators && !leaf.empty())
        e = cudaMemcpyAsync(indicators, v->indicator_ptr(), leaf.size() * 4u, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_status(e);
    if (leaf_slots) std::memcpy(leaf_slots, leaf.data(), leaf.size() * 4u);
    return AMR_OK;
}
AMR_API int amr_sim_regrid(amr_sim* s, amr_estimator* est, const amr_regrid* r, uint32_t* stats4) {
    if (!s || !r || r->max_depth > kDepthLimit || !(r->judge_factor >= 1.f)) return AMR_ERR_INVALID;
    EvolveSim* v = dynamic_cast<EvolveSim*>(s->impl);
    if (!v) return AMR_ERR_INVALID;
    if (s->impl->tree.timer() != 0u) return AMR_ERR_INVALID;   // between timesteps only
    const int st = s->impl->wait_side(-1, 0);
    return st ? st : v->regrid(est, *r, stats4);
}
AMR_API int amr_sim_constraint_norms(amr_sim* s, float excision_radius, double* out5) {
    if (!s || !out5 || !(excision_radius >= 0.f)) return AMR_ERR_INVALID;
    EvolveSim* v = dynamic_cast<EvolveSim*>(s->impl);
    if (!v) return AMR_ERR_INVALID;
    const int st = s->impl->wait_side(-1, 0);
    return st ? st : v->constraint_norms(excision_radius, out5);
}
