// octree.cpp -- host octree (see octree.h).  Compiled with -ffp-contract=off so the few float
// operations (boundary offsets) round identically on x86-64 and aarch64.
#include "octree.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "amr_types.h"

namespace amr {

uint32_t reverse_bits32(uint32_t a) {
    a = (a >> 16) | (a << 16);
    a = ((a & 0xFF00FF00u) >> 8) | ((a & 0x00FF00FFu) << 8);
    a = ((a & 0xF0F0F0F0u) >> 4) | ((a & 0x0F0F0F0Fu) << 4);
    a = ((a & 0xCCCCCCCCu) >> 2) | ((a & 0x33333333u) << 2);
    return ((a & 0xAAAAAAAAu) >> 1) | ((a & 0x55555555u) << 1);
}

// Each axis occupies every third bit of the 27-bit path.  Filling the other axes' bits with ones
// lets a carry ripple to the next bit of the same axis; a carry or borrow out of bit 24+axis lands
// in bit 27+axis and means the neighbour lies outside the root.
namespace {
constexpr uint32_t kLane = 0x1249249u;       // bits 0, 3, ..., 24
constexpr uint32_t kLaneOut = 0x9249249u;    // the same plus bit 27
}
uint32_t morton_sum(uint32_t a, uint32_t b, bool overflow) {
    uint32_t r = 0;
    for (uint32_t axis = 0; axis < 3; axis++) {
        const uint32_t gaps = (kPathMask & ~kLane) << axis;
        r |= ((a | gaps) + (b & (kLane << axis))) & (kLaneOut << axis);
    }
    return ((r & (7u << 27)) && overflow) ? ~0u : (r & kPathMask);
}
uint32_t morton_diff(uint32_t a, uint32_t b, bool overflow) {
    uint32_t r = 0;
    for (uint32_t axis = 0; axis < 3; axis++) {
        const uint32_t lane = kLane << axis;
        r |= ((a & lane) - (b & lane)) & (kLaneOut << axis);
    }
    return ((r & (7u << 27)) && overflow) ? ~0u : (r & kPathMask);
}

static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

uint32_t cf3_encode_host(float x, float y, float z) {
    const float v[3] = {x, y, z};
    uint32_t e = 0;
    for (int i = 0; i < 3; i++) e = std::max(e, (fbits(v[i]) >> 23) & 255u);
    const uint32_t E = std::min(std::max(e, 112u) - 112u, 31u);
    const float scale = 4194304.f / (float)(1u << E);      // 2^(22-E), exact
    uint32_t w = E << 27;
    const uint32_t mpos[3] = {0, 9, 18}, spos[3] = {8, 17, 26};
    for (int i = 0; i < 3; i++) {
        float s = v[i] * scale;
        s = fmaxf(-255.f, fminf(s, 255.f));
        w |= ((uint32_t)(fabsf(s) + .5f) << mpos[i]) | ((uint32_t)(s < 0.f) << spos[i]);
    }
    return w;
}

uint64_t make_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx) {
    return make_boundary(this_pos, other_pos, other_idx, 0, 0.f);
}
uint64_t make_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx, int axis, float shift) {
    const int td = pos_depth_host(this_pos), od = pos_depth_host(other_pos);
    const uint32_t node_data = ((uint32_t)other_idx & 16777215u) | (((uint32_t)(td - od) & 15u) << 24) |
                               (((uint32_t)td & 15u) << 28);
    // offset of this domain's centre from the other's, in units of the other's half-edge
    float r[3] = {0.f, 0.f, 0.f};
    const float mult = .25f * (float)(1u << od);
    uint32_t s = this_pos & kPathMask;
    for (int i = 0; i < td; i++, s >>= 3)
        for (int a = 0; a < 3; a++) r[a] += ((s & (1u << a)) ? mult : -mult) / (float)(1 << i);
    s = other_pos & kPathMask;
    for (int i = 0; i < od; i++, s >>= 3)
        for (int a = 0; a < 3; a++) r[a] -= ((s & (1u << a)) ? mult : -mult) / (float)(1 << i);
    r[axis] += shift;
    return (uint64_t)node_data | ((uint64_t)cf3_encode_host(r[0], r[1], r[2]) << 32);
}

Octree::Octree(uint32_t node_slots, NodeHooks* hooks)
    : hooks_(hooks), max_slots_(node_slots), positions_(node_slots, ~0u), parent_(node_slots, -1),
      children_((size_t)node_slots * 8u, -1), boundaries_((size_t)node_slots * 6u, kNoBoundary),
      lifetime_(node_slots, 0) {
    positions_[0] = 0u;   // the root
    depth_count_[0] = 1u;
}

void Octree::restore(const uint32_t* positions, const int32_t* parent, const int32_t* children,
                     const uint64_t* boundaries, const uint32_t* lifetime, uint32_t timer, int max_depth,
                     uint32_t first_free, uint32_t final_used) {
    positions_.assign(positions, positions + max_slots_);
    parent_.assign(parent, parent + max_slots_);
    children_.assign(children, children + (size_t)max_slots_ * 8u);
    boundaries_.assign(boundaries, boundaries + (size_t)max_slots_ * 6u);
    lifetime_.assign(lifetime, lifetime + max_slots_);
    timer_ = timer;
    max_depth_ = max_depth;
    first_free_slot_ = first_free;
    final_used_slot_ = final_used;
    dirty_ = true;
    for (uint32_t& c : depth_count_) c = 0u;
    for (uint32_t p : positions_)
        if (pos_depth_host(p) != -1) depth_count_[pos_depth_host(p)]++;
}

int Octree::counted_max_depth() const {
    for (int d = 31; d > 0; d--)
        if (depth_count_[d]) return d;
    return 0;
}
void Octree::note_change(int depth) {
    if (batching_) batch_min_depth_ = std::min(batch_min_depth_, depth);
    else refresh_boundaries(depth);
}
void Octree::begin_batch() {
    batching_ = true;
    batch_min_depth_ = 32;
    pending_ctor_.clear();
}
void Octree::end_batch() {
    batching_ = false;
    if (batch_min_depth_ < 32) refresh_boundaries(batch_min_depth_);
    batch_min_depth_ = 32;
    if (hooks_ && !pending_ctor_.empty()) run_pending_ctors();
    pending_ctor_.clear();
}
void Octree::run_pending_ctors() {
    const size_t n = pending_ctor_.size();
    // Depth order matches the calls' order if every slot is written once and each constructor
    // that reads a slot written in the batch comes after that write and deeper.
    bool by_depth = true;
    std::vector<int32_t> writer(max_slots_, -1);
    for (size_t i = 0; i < n && by_depth; i++) {
        int32_t& w = writer[(size_t)pending_ctor_[i].c.node];
        if (w != -1) by_depth = false;
        w = (int32_t)i;
    }
    for (size_t i = 0; i < n && by_depth; i++) {
        const int32_t j = writer[(size_t)pending_ctor_[i].c.parent];
        if (j != -1 && !((size_t)j < i && pending_ctor_[(size_t)j].depth < pending_ctor_[i].depth)) by_depth = false;
    }
    if (by_depth)
        std::stable_sort(pending_ctor_.begin(), pending_ctor_.end(),
                         [](const PendingCtor& a, const PendingCtor& b) { return a.depth < b.depth; });
    std::vector<NodeCtor> items(n);
    std::vector<uint32_t> ends;
    for (size_t i = 0; i < n; i++) {
        items[i] = pending_ctor_[i].c;
        if (i + 1 == n || !by_depth || pending_ctor_[i + 1].depth != pending_ctor_[i].depth) ends.push_back((uint32_t)i + 1u);
    }
    hooks_->node_ctor_groups(items.data(), ends.data(), (uint32_t)ends.size());
}
void Octree::refresh_node(uint32_t node) {
    for (uint32_t f = 0; f < 6; f++) boundaries_[(size_t)node * 6u + f] = yield_boundary((int32_t)node, f);
}
// Inside a batch, a node about to be removed gets the boundaries it would have had from the last
// call (since the batch began) that refreshed it: its value now, before the tree changes.
void Octree::refresh_subtree_before_removal(int32_t node) {
    if (node == -1) return;
    const int d = pos_depth_host(positions_[node]);
    if (d == -1) return;
    if (d >= batch_min_depth_) refresh_node((uint32_t)node);
    for (uint32_t i = 0; i < 8u; i++) refresh_subtree_before_removal(children_[(size_t)node * 8u + i]);
}
void Octree::increment_timer() {
    for (uint32_t i = 0; i <= final_used_slot_; i++) {
        const int depth = pos_depth_host(positions_[i]);
        if (depth == -1) continue;
        lifetime_[i] += ((timer_ & ((1u << (uint32_t)(max_depth_ - depth)) - 1u)) == 0u);
    }
    timer_ = (timer_ + 1u) & ((1u << (uint32_t)max_depth_) - 1u);
}

void Octree::add_node(int32_t parent, int32_t offset) {
    if (first_free_slot_ >= max_slots_ || children_[(size_t)parent * 8u + offset] != -1) return;
    if (pos_depth_host(positions_[parent]) >= (int)kDepthLimit) return;
    const uint32_t slot = first_free_slot_;
    lifetime_[slot] = 0u;
    parent_[slot] = parent;
    children_[(size_t)parent * 8u + offset] = (int32_t)slot;
    positions_[slot] = pos_child(positions_[parent], (uint32_t)offset);
    const int new_depth = pos_depth_host(positions_[slot]);
    depth_count_[new_depth]++;
    const int change = std::max(max_depth_, new_depth) - max_depth_;
    timer_ <<= change;
    max_depth_ += change;
    if (hooks_) {
        if (batching_) pending_ctor_.push_back({{(int32_t)slot, parent, pos_final_offset(positions_[slot])}, new_depth});
        else hooks_->node_ctor((int32_t)slot);
    }
    final_used_slot_ = std::max(final_used_slot_, slot);
    while (first_free_slot_ < max_slots_ && pos_depth_host(positions_[first_free_slot_]) != -1) first_free_slot_++;
    note_change(new_depth);
    dirty_ = true;
}

void Octree::remove_node_recursive(int32_t node) {
    if (node == -1 || pos_depth_host(positions_[node]) == -1) return;
    if (hooks_) hooks_->node_dtor(node);
    for (uint32_t i = 0; i < 8u; i++) remove_node_recursive(children_[(size_t)node * 8u + i]);
    children_[(size_t)parent_[node] * 8u + pos_final_offset(positions_[node])] = -1;
    parent_[node] = -1;
    depth_count_[pos_depth_host(positions_[node])]--;
    positions_[node] = ~0u;
    first_free_slot_ = std::min(first_free_slot_, (uint32_t)node);
}

void Octree::remove_node(int32_t node) {
    if (node == -1) return;
    const int curr_depth = pos_depth_host(positions_[node]);
    if (curr_depth == -1) return;
    if (batching_) refresh_subtree_before_removal(node);
    remove_node_recursive(node);
    const int old_max = max_depth_;
    max_depth_ = counted_max_depth();   // the deepest node left (AMR.h:243-246)
    timer_ >>= (old_max - max_depth_);
    while (pos_depth_host(positions_[final_used_slot_]) == -1 && final_used_slot_ > 0u) final_used_slot_--;
    note_change(curr_depth);
    dirty_ = true;
}

void Octree::refresh_boundaries(int from_depth) {
    for (uint32_t i = 0; i <= final_used_slot_; i++)
        if (pos_depth_host(positions_[i]) >= from_depth)
            for (uint32_t f = 0; f < 6; f++) boundaries_[(size_t)i * 6u + f] = yield_boundary((int32_t)i, f);
}

uint32_t Octree::find_node_idx(uint32_t packed, uint32_t max_depth) const {
    uint32_t curr = 0, depth = 0;
    while (true) {
        const int32_t c = children_[(size_t)curr * 8u + (packed & 7u)];
        if (c == -1 || depth >= max_depth) return curr;
        packed >>= 3u;
        curr = (uint32_t)c;
        depth++;
    }
}

uint64_t Octree::yield_boundary(int32_t node, uint32_t face) const {
    static const uint32_t kDirections[3] = {4u, 2u, 1u};   // x, y, z within a reversed level triple
    const int depth = pos_depth_host(positions_[node]);
    if (depth <= 0) return kNoBoundary;
    // Reverse the word so levels are most-significant-first (x in the high bit of each triple),
    // step one domain along the face normal at this depth, and reverse back.
    uint32_t p = reverse_bits32(positions_[node]) >> 5u;
    const uint32_t step = (kDirections[face % 3u] << ((9u - (uint32_t)depth) * 3u)) & kPathMask;
    const uint32_t q = face < 3 ? morton_sum(p, step, true) : morton_diff(p, step, true);
    if (q == ~0u && periodic_) {
        // across the root's boundary: the domain at the wrapped position, shifted by one root edge
        // (2^depth of the neighbour's edges) to lie beside this one
        const uint32_t w = face < 3 ? morton_sum(p, step, false) : morton_diff(p, step, false);
        const uint32_t neighbour = find_node_idx(reverse_bits32(w) >> 5u, (uint32_t)depth);
        const float root_edges = (float)(1u << (uint32_t)pos_depth_host(positions_[neighbour]));
        return make_boundary(positions_[node], positions_[neighbour], (int32_t)neighbour, (int)(face % 3u),
                             face < 3 ? -root_edges : root_edges);
    }
    uint32_t neighbour = find_node_idx(reverse_bits32(q) >> 5u, (uint32_t)depth);
    if (q == ~0u) neighbour = 0;   // outside the root: the root's ghost layer is the source
    return make_boundary(positions_[node], positions_[neighbour], (int32_t)neighbour);
}

void Octree::set_periodic(bool periodic) {
    if (periodic == periodic_) return;
    periodic_ = periodic;
    refresh_boundaries(1);
    dirty_ = true;
}

}  // namespace amr
