// octree.h -- host-side octree of fixed-size domains (the reference's AMR<T>, AMR.h:118-294).
//
// Node slots, Morton positions (octree_abs_pos, AMR.h:22-55), face boundary descriptors
// (domain_boundary, AMR.h:56-100) and the 0..2^max_depth-1 subcycling counter are kept
// bit-identical to the reference, so its arrays can be exchanged with this class as is.
#pragma once

#include <cstdint>
#include <vector>

namespace amr {

// A node constructor deferred by a batch: prolongate slot `parent`, as the batch had it when the
// node was added, into slot `node` as child `offset` (three int32 words, as device item lists).
struct NodeCtor {
    int32_t node, parent, offset;
};
static_assert(sizeof(NodeCtor) == 12, "NodeCtor is three int32 words");

// Receives the reference plugin's node_ctor / node_dtor callbacks (AMR.h:138, 221).
class NodeHooks {
public:
    virtual ~NodeHooks() = default;
    virtual void node_ctor(int32_t node) = 0;
    virtual void node_dtor(int32_t node) = 0;
    // The constructors a batch deferred, as groups to run in order: group g is
    // items[group_end[g-1] .. group_end[g]) (group_end[-1] = 0), and no item of a group reads a
    // slot that another item of the same group writes.
    virtual void node_ctor_groups(const NodeCtor* items, const uint32_t* group_end, uint32_t groups) = 0;
};

// octree_abs_pos helpers (AMR.h:22-55): depth in bits 27..31, Morton path (3 bits per level,
// level 1 in the lowest bits) below; 0xFFFFFFFF marks a free slot.
inline int pos_depth_host(uint32_t p) { return (~p) ? (int)(p >> 27) : -1; }
// The shift count is taken modulo 32, as the shifters do, for a (degenerate) depth-0 position.
inline int pos_final_offset(uint32_t p) { return (int)((p >> (((uint32_t)(pos_depth_host(p) - 1) * 3u) & 31u)) & 7u); }
// octree_abs_pos::set_child (AMR.h:50-54).  The shift count is taken modulo 32 as the x86-64 and
// Arm shifters do, which keeps a (degenerate) free parent well defined.
inline uint32_t pos_child(uint32_t parent, uint32_t offset) {
    return (parent + (1u << 27)) | (offset << (((uint32_t)pos_depth_host(parent) * 3u) & 31u));
}

uint32_t reverse_bits32(uint32_t a);
uint32_t morton_sum(uint32_t a, uint32_t b, bool overflow);        // yield_sum_coordinates, AMR.h:102-108
uint32_t morton_diff(uint32_t a, uint32_t b, bool overflow);       // yield_diff_coordinates, AMR.h:109-115
uint64_t make_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx);  // AMR.h:64-86
// The same with `shift` other-domain edges added to the offset along `axis` (a periodic
// neighbour across the root's boundary is described as if it lay next to this domain).
uint64_t make_boundary(uint32_t this_pos, uint32_t other_pos, int32_t other_idx, int axis, float shift);
constexpr uint64_t kNoBoundary = 0xFFFFFFFFull;                   // domain_boundary(), AMR.h:63
// Host deterministic compressed_float3 encoder (tensors.h:374-393), for boundary offsets.
uint32_t cf3_encode_host(float x, float y, float z);

class Octree {
public:
    explicit Octree(uint32_t node_slots, NodeHooks* hooks = nullptr);

    void set_hooks(NodeHooks* h) { hooks_ = h; }
    void add_node(int32_t parent, int32_t offset);           // AMR.h:208-232
    void remove_node(int32_t node);                          // AMR.h:233-254
    void increment_timer();                                  // AMR.h:180-188
    // Batches of add_node / remove_node calls (the regrid path) with the same final state as the
    // calls one by one, without their per-call costs: inside a batch the boundary refresh that
    // every call makes over all nodes at or below its depth is done once at end_batch (a node's
    // boundaries depend only on nodes no deeper than it, so the last call that would have
    // refreshed it sees what the end of the batch sees; a node removed inside the batch is
    // refreshed just before its removal if such a call came first).  Node constructors are
    // recorded with the parent and offset they would have read and run at end_batch through
    // NodeHooks::node_ctor_groups: one group per depth level, parents first, when that order
    // reads and writes every slot as the calls one by one would; otherwise (a slot written twice,
    // or read before a later constructor rewrites it) one group per constructor in call order.
    // The maximum depth comes from a count of nodes per depth.
    void begin_batch();
    void end_batch();
    uint32_t find_node_idx(uint32_t packed_pos, uint32_t max_depth = ~0u) const;   // AMR.h:255-263
    uint64_t yield_boundary(int32_t node, uint32_t face) const;                    // AMR.h:276-290
    // Periodic root (no counterpart in the reference, whose outside neighbour is the root's frozen
    // ghost layer): a face whose neighbour lies outside the root takes the domain on the opposite
    // side, found as the reference finds any neighbour, and every boundary is recomputed.
    void set_periodic(bool periodic);
    bool periodic() const { return periodic_; }

    uint32_t curr_used_slots() const { return final_used_slot_ + 1u; }
    uint32_t read_first_free_slot() const { return first_free_slot_; }
    int read_max_depth() const { return max_depth_; }
    uint32_t max_slots() const { return max_slots_; }
    uint32_t timer() const { return timer_; }
    void set_timer(uint32_t t) { timer_ = t; }

    // Replace the whole state (a checkpoint being resumed); arrays hold max_slots() entries
    // (children 8x, boundaries 6x).
    void restore(const uint32_t* positions, const int32_t* parent, const int32_t* children, const uint64_t* boundaries,
                 const uint32_t* lifetime, uint32_t timer, int max_depth, uint32_t first_free, uint32_t final_used);
    uint32_t final_used_slot() const { return final_used_slot_; }

    // True when the arrays changed since the last mark_clean() (the reference's `dirty`).
    bool dirty() const { return dirty_; }
    void mark_clean() { dirty_ = false; }

    const std::vector<uint32_t>& positions() const { return positions_; }
    const std::vector<int32_t>& parents() const { return parent_; }
    const std::vector<int32_t>& children() const { return children_; }
    const std::vector<uint64_t>& boundaries() const { return boundaries_; }
    const std::vector<uint32_t>& lifetime() const { return lifetime_; }

private:
    void remove_node_recursive(int32_t node);
    void refresh_boundaries(int from_depth);
    void refresh_node(uint32_t node);
    void refresh_subtree_before_removal(int32_t node);
    void note_change(int depth);   // a call that refreshes every node at or below `depth`
    void run_pending_ctors();
    int counted_max_depth() const;

    NodeHooks* hooks_;
    uint32_t max_slots_;
    std::vector<uint32_t> positions_;
    std::vector<int32_t> parent_;
    std::vector<int32_t> children_;
    std::vector<uint64_t> boundaries_;
    std::vector<uint32_t> lifetime_;
    int max_depth_ = 0;
    uint32_t first_free_slot_ = 1;
    uint32_t final_used_slot_ = 0;
    uint32_t timer_ = 0;
    bool dirty_ = true;
    bool periodic_ = false;
    uint32_t depth_count_[32] = {};   // live nodes per depth (any depth a position word can hold)
    bool batching_ = false;
    int batch_min_depth_ = 32;        // shallowest change inside the current batch (32: none)
    struct PendingCtor {
        NodeCtor c;
        int depth;
    };
    std::vector<PendingCtor> pending_ctor_;
};

}  // namespace amr
