// partition.cpp -- domains over ranks, and the ghost-exchange plan between them.
//
// The hot path shards by domain: given its ghost cells, a domain's stencils need nothing else.
// Ranks own contiguous ranges of the domains in Morton (preorder) order of their octree positions
// (AMR.h:22-55), so neighbours mostly share an owner.  Before each ghost fill, a rank needs, for
// every active face of a domain it owns whose source domain another rank owns, the source box that
// the fill's interpolation reads (AMR.h:737-753): the range of the face's nearest source indices,
// widened by one cell for the 10-point stencil (AMR.h:672-699).  The box is computed with the
// device's arithmetic, so it is exactly the box the ghost kernel reads.  The reference has no
// multi-GPU path; this is the host half of one.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <set>
#include <vector>

#include "capi_internal.h"
#include "octree.h"

namespace amr {
namespace {

// Preorder key of a position: the path's octant digits from the root down (zeros below the node's
// depth), then the depth, so a parent sorts just before its first child.
uint64_t preorder_key(uint32_t pos) {
    const int d = pos_depth_host(pos);
    uint64_t key = 0;
    for (int i = 0; i < (int)kDepthLimit; i++) key = (key << 3) | (i < d ? (uint64_t)((pos >> (3 * i)) & 7u) : 0u);
    return (key << 4) | (uint64_t)d;
}

// compressed_float3 decode (tensors.h:335-348): m * 2^(E-22), sign applied last.
float cf3_component_host(uint32_t w, uint32_t mpos, uint32_t spos) {
    const float m = (float)((w >> mpos) & 255u);
    const float v = std::ldexp(m, (int)(w >> 27) - 22);
    return ((w >> spos) & 1u) ? -v : v;
}

// Nearest source index along one axis for written coordinate w: the ghost kernel's arithmetic
// (the same operations, rounded one by one).
uint32_t ghost_source_index(uint32_t w, uint32_t n, uint32_t p, float rel_scale, float relp, bool root) {
    const uint32_t t = n + 2u * p;
    const float inv_n = 1.f / (float)n;
    float rp = std::fma(((float)w - (float)p) + .5f, inv_n, -.5f);
    rp = std::fma(rp, rel_scale, relp);
    rp = std::fma(rp + .5f, (float)n, (float)p) - .5f;
    const uint32_t idx = root ? (uint32_t)(std::fmax(rp, 0.f) + .5f) : (uint32_t)(std::fmax(rp, (float)p) + .5f);
    return std::min(idx, root ? t - 2u : t - p - 2u);
}

}  // namespace
}  // namespace amr

using namespace amr;

extern "C" __attribute__((visibility("default")))
int amr_partition_morton(const uint32_t* positions, uint32_t used_slots, uint32_t ranks, int32_t* owner) {
    if (!positions || !owner || ranks == 0) return AMR_ERR_INVALID;
    std::vector<std::pair<uint64_t, uint32_t>> live;
    for (uint32_t s = 0; s < used_slots; s++) {
        owner[s] = -1;
        if (positions[s] != 0xFFFFFFFFu) live.emplace_back(preorder_key(positions[s]), s);
    }
    std::sort(live.begin(), live.end());
    const uint64_t n = live.size();
    for (uint64_t i = 0; i < n; i++) owner[live[i].second] = (int32_t)(i * ranks / n);   // balanced ranges
    return AMR_OK;
}

extern "C" __attribute__((visibility("default")))
int amr_ghost_exchange_plan(const amr_config* cfg, const uint64_t* boundaries, const int32_t* owner,
                            uint32_t used_slots, uint32_t substep, uint32_t max_depth, uint32_t rank,
                            uint32_t* boxes, uint32_t capacity, uint32_t* n_boxes) {
    if (!cfg) return AMR_ERR_INVALID;
    if (!config_supported(cfg)) return AMR_ERR_UNSUPPORTED;
    if (!boundaries || !owner || !n_boxes || (capacity && !boxes) || max_depth > kDepthLimit) return AMR_ERR_INVALID;
    const uint32_t n = cfg->size_domain, p = cfg->padding_domain, t = n + 2u * p;
    std::set<std::vector<uint32_t>> plan;
    for (uint32_t s = 0; s < used_slots; s++) {
        if (owner[s] != (int32_t)rank) continue;
        for (uint32_t face = 0; face < 6u; face++) {
            const uint64_t bd = boundaries[(size_t)s * 6u + face];
            const uint32_t nd = (uint32_t)bd;
            const int32_t target = (int32_t)((nd & 16777215u) | ((nd & (1u << 23)) ? 4278190080u : 0u));
            const int cd = (nd >> 28) == 15u ? -1 : (int)(nd >> 28);
            const uint32_t dd = (nd >> 24) & 15u;
            if (target == -1 || cd <= 0) continue;
            if (cd > (int)max_depth) return AMR_ERR_INVALID;   // a record deeper than the tree
            if ((substep & ((1u << (max_depth - (uint32_t)cd)) - 1u)) != 0u) continue;
            if ((uint32_t)target >= used_slots) return AMR_ERR_INVALID;
            const int32_t src_rank = owner[target];
            if (src_rank == (int32_t)rank) continue;
            if (src_rank < 0) return AMR_ERR_INVALID;
            const uint32_t rel = (uint32_t)(bd >> 32);
            const float relp[3] = {cf3_component_host(rel, 0u, 8u), cf3_component_host(rel, 9u, 17u),
                                   cf3_component_host(rel, 18u, 26u)};
            const float rel_scale = std::ldexp(1.f, -(int)dd);
            const bool root = target == 0;
            const uint32_t normal = face % 3u;
            std::vector<uint32_t> rec = {(uint32_t)target, (uint32_t)src_rank, 0, 0, 0, t, t, t};
            bool whole = false;
            uint32_t lo[3], ext[3];
            for (uint32_t a = 0; a < 3; a++) {
                const uint32_t wlo = a == normal ? (face < 3u ? p + n : 0u) : p;
                const uint32_t whi = a == normal ? wlo + p - 1u : p + n - 1u;
                const uint32_t r0 = ghost_source_index(wlo, n, p, rel_scale, relp[a], root);
                const uint32_t r1 = ghost_source_index(whi, n, p, rel_scale, relp[a], root);
                if (r0 == 0u) whole = true;   // the stencil would step out of the cube (a root source only)
                lo[a] = r0 - 1u;
                ext[a] = r1 - r0 + 3u;
            }
            if (!whole)
                for (uint32_t a = 0; a < 3; a++) { rec[2 + a] = lo[a]; rec[5 + a] = ext[a]; }
            plan.insert(rec);
        }
    }
    // drop boxes that another box of the same source slot contains (the records are distinct, so
    // containment is strict and never mutual)
    std::vector<std::vector<uint32_t>> recs(plan.begin(), plan.end()), kept;
    for (size_t i = 0; i < recs.size(); i++) {
        bool inside = false;
        for (size_t j = 0; j < recs.size() && !inside; j++) {
            if (i == j || recs[i][0] != recs[j][0]) continue;
            inside = true;
            for (int a = 0; a < 3; a++)
                inside &= recs[j][2 + a] <= recs[i][2 + a] &&
                          recs[i][2 + a] + recs[i][5 + a] <= recs[j][2 + a] + recs[j][5 + a];
        }
        if (!inside) kept.push_back(recs[i]);
    }
    *n_boxes = (uint32_t)kept.size();
    if (kept.size() > capacity) return AMR_ERR_CAPACITY;
    for (size_t i = 0; i < kept.size(); i++) std::memcpy(boxes + 8u * i, kept[i].data(), 8u * sizeof(uint32_t));
    return AMR_OK;
}

// The restriction (copy_new_to_old, AMR.h:961-996) of an active domain with children averages each
// child's new field over 2x2x2 cells, which covers the child's whole interior.  So before the
// restriction of `substep`, `rank` needs the interior of every child that another rank owns of every
// active domain that it owns; same records as the ghost plan.
extern "C" __attribute__((visibility("default")))
int amr_restriction_exchange_plan(const amr_config* cfg, const uint32_t* positions, const int32_t* children,
                                  const int32_t* owner, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                                  uint32_t rank, uint32_t* boxes, uint32_t capacity, uint32_t* n_boxes) {
    if (!cfg) return AMR_ERR_INVALID;
    if (!config_supported(cfg)) return AMR_ERR_UNSUPPORTED;
    if (!positions || !children || !owner || !n_boxes || (capacity && !boxes) || max_depth > kDepthLimit)
        return AMR_ERR_INVALID;
    const uint32_t n = cfg->size_domain, p = cfg->padding_domain;
    std::vector<uint32_t> out;
    for (uint32_t s = 0; s < used_slots; s++) {
        const int d = pos_depth_host(positions[s]);
        if (owner[s] != (int32_t)rank || d == -1 || d > (int)max_depth) continue;
        if ((substep & ((1u << (max_depth - (uint32_t)d)) - 1u)) != 0u) continue;   // not active
        for (uint32_t i = 0; i < 8u; i++) {
            const int32_t c = children[(size_t)s * 8u + i];
            if (c == -1) continue;
            if (c < 0 || (uint32_t)c >= used_slots || owner[c] < 0) return AMR_ERR_INVALID;
            if (owner[c] == (int32_t)rank) continue;
            const uint32_t rec[8] = {(uint32_t)c, (uint32_t)owner[c], p, p, p, n, n, n};
            out.insert(out.end(), rec, rec + 8);
        }
    }
    *n_boxes = (uint32_t)(out.size() / 8u);
    if (*n_boxes > capacity) return AMR_ERR_CAPACITY;
    if (!out.empty()) std::memcpy(boxes, out.data(), out.size() * sizeof(uint32_t));
    return AMR_OK;
}
