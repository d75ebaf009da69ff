/* amr_gb300.h -- C ABI of the GB300 (sm_103a) implementation of AdaptiveMesh's per-timestep
 * hot path.
 *
 * Data layout (identical to the reference so its host octree can hand buffers over as is):
 *   padded field   float    slot * T^3 + (z*T + y)*T + x,  T = size_domain + 2*padding_domain
 *                           (AdaptiveMesh/AMR.h:1165-1166); one buffer per tensor component.
 *   inner field    float or compressed_float3 words (uint32)
 *                           slot * N^3 + (z*N + y)*N + x,  N = size_domain (AMR.h:1177-1178).
 *   positions      uint32 octree_abs_pos words, one per slot (AMR.h:22-55).
 *   children       int32, 8 per slot, -1 = none (AMR.h:123).
 *   boundaries     uint64 domain_boundary words, 6 per slot in face order +x,+y,+z,-x,-y,-z
 *                           (AMR.h:56-100, AMR.h:276-290).
 *
 * Conventions: every entry point returns AMR_OK (0) or an error code; device work is enqueued
 * on the caller's stream (a cudaStream_t passed as void*, NULL = legacy default stream) with no
 * implicit device synchronisation.  `used_slots` is the octree's curr_used_slots() (AMR.h:205).
 * Slots with octree_abs_pos == 0xFFFFFFFF, and slots whose depth is not active at `substep`
 * (AMR.h:640-644), are skipped, as in the reference.  Not thread-safe per simulation object.
 */
#ifndef AMR_GB300_H
#define AMR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMR_OK 0
#define AMR_ERR_INVALID 1           /* bad argument (null pointer, size out of range) */
#define AMR_ERR_UNSUPPORTED 2       /* (size_domain, padding_domain) not compiled in */
#define AMR_ERR_CUDA 3              /* a CUDA runtime call failed; see amr_last_cuda_error() */
#define AMR_ERR_NO_DEVICE 4         /* no CUDA device is visible */
#define AMR_ERR_CAPACITY 5          /* node slots exhausted or a fixed-size buffer is too small */
#define AMR_ERR_TIMEOUT 6           /* a kernel's bounded wait gave up; that work's results are invalid */

/* Domain configuration: the reference's compile-time constants (AMR.h:9-20) as run-time values. */
typedef struct amr_config {
    uint32_t size_domain;       /* interior cells per edge, N   (AMR.h:11) */
    uint32_t padding_domain;    /* ghost cells per side, p      (AMR.h:12); FD order = 2p (AMR.h:1171) */
    float outer_size;           /* edge length of the root      (AMR.h:10) */
} amr_config;

/* Christoffel modes for amr_christoffel: AMR_CHRISTOFFEL_REFERENCE multiplies the lowered
 * symbols by the metric as BSSN.h:82 does; AMR_CHRISTOFFEL_RAISED multiplies by its inverse. */
#define AMR_CHRISTOFFEL_REFERENCE 0
#define AMR_CHRISTOFFEL_RAISED 1

/* ---------------------------------------------------------------- library */
const char* amr_version(void);
/* 1 if (size_domain, padding_domain) has compiled kernels. */
int amr_config_supported(const amr_config* cfg);
/* The last CUDA error code seen by this thread (0 if none). */
int amr_last_cuda_error(void);
/* Human-readable text for a status code. */
const char* amr_status_string(int status);
/* Synchronise `stream`, then report whether a kernel of this library on the current device gave
 * up a bounded wait (a data copy that never arrived) since the last report: AMR_ERR_TIMEOUT once,
 * and the device's flag is cleared.  The operator entry points are asynchronous, so this is how
 * their callers learn of such a failure.  No counterpart in the reference, whose kernels do not
 * wait on one another. */
int amr_device_status(void* stream);

/* ---------------------------------------------------------------- compressed_float3 codec
 * 3 x (sign + 8-bit mantissa) with a 5-bit shared exponent, bit-exact with the reference's
 * device build (tensors.h:305-394).  seeds == NULL selects the deterministic encoder
 * (tensors.h:374-393); otherwise element i uses a fresh fast_prng(seeds[i]) (tensors.h:276-304). */
int amr_cf3_encode(const float* xyz, const int32_t* seeds, uint64_t n, uint32_t* out, void* stream);
int amr_cf3_decode(const uint32_t* words, uint64_t n, float* xyz, void* stream);

/* ---------------------------------------------------------------- operator kernels
 * One entry point per reference operator; the global seed is the value the reference draws
 * from its host fast_prng for that launch (rng.generate_int(), AMR.h:1277, 1289, 1301). */

/* Gradient (and, if d2if != NULL, the diagonal of the Hessian) by (2p+1)-point centred
 * differences, scaled by 2^depth / outer_dx.  Replaces differentiate(), AMR.h:1280-1302. */
int amr_differentiate(const amr_config* cfg, const float* field, uint32_t* dif, uint32_t* d2if,
                      const uint32_t* positions, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                      int32_t seed, void* stream);
/* Off-diagonal Hessian (xy, xz, yz) with the reference's edge rule.  Replaces mixed_partials(),
 * AMR.h:1268-1278. */
int amr_mixed_partials(const amr_config* cfg, const float* field, uint32_t* off_diag,
                       const uint32_t* positions, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                       int32_t seed, void* stream);
/* g^kl H_kl from a compressed Hessian (diag, off-diag) and the six padded metric components
 * (xx, xy, xz, yy, yz, zz; a host array of device pointers).  Replaces the third launch of
 * scalar_laplacian_noncovariant(), BSSN.h:24-36. */
int amr_deriv_trace(const amr_config* cfg, const uint32_t* hess_diag, const uint32_t* hess_off,
                    float* const* metric6, float* out, const uint32_t* positions, uint32_t used_slots,
                    uint32_t substep, uint32_t max_depth, void* stream);
/* Christoffel symbols from the six compressed metric gradients.  Replaces
 * compute_raised_christoffel_symbols(), BSSN.h:93-102.  mode: AMR_CHRISTOFFEL_*. */
int amr_christoffel(const amr_config* cfg, float* const* metric6, uint32_t* const* derivs6, int32_t seed,
                    uint32_t* const* out6, const uint32_t* positions, uint32_t used_slots, uint32_t substep,
                    uint32_t max_depth, int mode, void* stream);
/* Face ghost fill with space (10-point) and time interpolation from the coarser-or-equal
 * neighbour.  Replaces copy_boundaries(), AMR.h:880-900.  All reads see the fields as they
 * were before the call (the reference's single launch races where a domain reads a coarser
 * neighbour's innermost ghost layer); the values are staged in scratch memory that each call
 * takes from the device's stream-ordered pool (cudaMallocAsync) and returns after the fill. */
int amr_copy_boundaries(const amr_config* cfg, float* old_f, float* new_f, const uint64_t* boundaries,
                        uint32_t used_slots, uint32_t substep, uint32_t max_depth, int copy_only_new,
                        void* stream);
/* The same ghost fill as amr_copy_boundaries, for callers that cannot let the library allocate
 * device memory (an application that owns a fixed device-memory budget, or a time-critical loop
 * that must not block on cudaMalloc).  It has no counterpart in the reference.  Instead of an
 * allocated staging buffer it uses a fixed 8 MiB array compiled into the library (held by every
 * GPU that loads it, until exit), so it calls no allocator.  Limit: 2 * 3 * size_domain^2 floats
 * per slot must fit in 2^21 floats (1365 slots at 16/3, 445 at 28/2, 341 at 32/3); larger cases
 * return AMR_ERR_CAPACITY.  The first call on a device looks up the array's
 * address; make that first call before any stream capture.  All calls share the array, so calls
 * that overlap on the GPU race and must be ordered by the caller; nothing in it needs clearing. */
int amr_copy_boundaries_noalloc(const amr_config* cfg, float* old_f, float* new_f, const uint64_t* boundaries,
                                uint32_t used_slots, uint32_t substep, uint32_t max_depth, int copy_only_new,
                                void* stream);
/* Rasterise the z = z_slice plane of the unit cube ([-0.5, 0.5]^3, the root's extent) into a
 * width x height RGBA float image (16-byte aligned, row-major, y rows): per pixel, descend the
 * octree (children, used_slots) to the leaf containing the point and interpolate `field` (a padded
 * field) there; the grey value is the interpolated value + 0.5, alpha 1.  With bounding_boxes != 0,
 * pixels within 2^(depth+1) / width of a leaf's x or y border are red (1, 0, 0, 1), as the
 * reference's build draws them (DISPLAY_BOUNDING_BOXES, AMR.h:1312).  Replaces rasterise_to_image
 * (AMR.h:1313-1365), bit for bit; width, height <= 65536. */
int amr_rasterise(const amr_config* cfg, const float* field, const int32_t* children, uint32_t used_slots,
                  uint32_t width, uint32_t height, float z_slice, int bounding_boxes, float* raster_rgba,
                  void* stream);
/* ---- sharding by domain (no counterpart in the reference, which runs on one GPU) ----
 * Ranks own contiguous ranges of the live slots in the preorder (Morton) order of their positions
 * (octree_abs_pos, AMR.h:22-55), balanced by count; owner[s] = rank, or -1 for a free slot
 * (positions[s] == 0xFFFFFFFF).  Host only. */
int amr_partition_morton(const uint32_t* positions, uint32_t used_slots, uint32_t ranks, int32_t* owner);
/* The source boxes that `rank` must receive before the ghost fill of `substep`
 * (amr_copy_boundaries; AMR.h:701-762): for every active face of a slot it owns whose source slot
 * another rank owns, the cells that the fill's interpolation reads, computed with the device's
 * arithmetic.  Each box is 8 uint32: {source slot, source rank, lo x, lo y, lo z, extent x, extent y,
 * extent z} in padded-domain cells; duplicates are merged.  Writes at most `capacity` boxes and sets
 * *n_boxes to the number needed (AMR_ERR_CAPACITY if larger than capacity).  The sender of a box
 * calls this for each receiving rank.  Host only. */
int amr_ghost_exchange_plan(const amr_config* cfg, const uint64_t* boundaries, const int32_t* owner,
                            uint32_t used_slots, uint32_t substep, uint32_t max_depth, uint32_t rank,
                            uint32_t* boxes, uint32_t capacity, uint32_t* n_boxes);
/* The boxes that `rank` must receive before the restriction of `substep` (amr_copy_new_to_old;
 * AMR.h:961-996): the interior (new field) of every child, owned by another rank, of an active
 * domain that `rank` owns.  Same records, capacity and count rules as amr_ghost_exchange_plan;
 * positions / children are the host octree arrays.  Host only. */
int amr_restriction_exchange_plan(const amr_config* cfg, const uint32_t* positions, const int32_t* children,
                                  const int32_t* owner, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                                  uint32_t rank, uint32_t* boxes, uint32_t capacity, uint32_t* n_boxes);
/* Copy the boxes of one padded field (used_slots domains) into `out` (box b, x fastest, at float
 * offset offsets[b]), or back from `in`.  boxes / offsets are device arrays; a record outside the
 * slot range or its cube is skipped. */
int amr_pack_boxes(const amr_config* cfg, const float* field, uint32_t used_slots, const uint32_t* boxes,
                   const uint64_t* offsets, uint32_t n_boxes, float* out, void* stream);
int amr_unpack_boxes(const amr_config* cfg, float* field, uint32_t used_slots, const uint32_t* boxes,
                     const uint64_t* offsets, uint32_t n_boxes, const float* in, void* stream);
/* old <- new for active domains; cells covered by a child <- mean of the child's 2x2x2 cells.
 * Replaces copy_new_to_old(), AMR.h:998-1018. */
int amr_copy_new_to_old(const amr_config* cfg, float* old_f, const float* new_f, const uint32_t* positions,
                        const int32_t* children, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                        void* stream);
/* Prolongation of a parent's padded domain into a new child (all cells, ghosts included).
 * Replaces copy_to_child(), AMR.h:1075-1082. */
int amr_copy_to_child(const amr_config* cfg, float* field, uint32_t offset, int32_t child, int32_t parent,
                      void* stream);
/* SimpleWave Heun predictor / corrector.  Replace wave_equation_predictor() and
 * wave_equation_corrector(), SimpleWave.h:48-72. */
int amr_wave_predictor(const amr_config* cfg, const float* old_f, const uint32_t* derivs, const uint32_t* hess_diag,
                       float* new_f, const uint32_t* positions, uint32_t used_slots, uint32_t substep,
                       uint32_t max_depth, void* stream);
int amr_wave_corrector(const amr_config* cfg, const float* old_f, const uint32_t* derivs, const uint32_t* hess_diag,
                       float* new_f, const uint32_t* positions, uint32_t used_slots, uint32_t substep,
                       uint32_t max_depth, void* stream);
/* Device half of amr_criterion(): per-octant maxima of |grad u| dx and |diag H| dx^2, written
 * at the strided positions __amr_criterion_2 leaves them (SimpleWave.h:91-150).  crit holds
 * used_slots * N * N floats. */
int amr_criterion(const amr_config* cfg, const uint32_t* derivs, const uint32_t* hess_diag, float* crit,
                  const uint32_t* positions, uint32_t used_slots, uint32_t substep, uint32_t max_depth,
                  void* stream);

/* ---------------------------------------------------------------- host octree
 * The reference's AMR<T> (AMR.h:118-294) without device data: same slot allocation, Morton
 * positions, boundary descriptors and subcycling counter, bit for bit. */
typedef struct amr_octree amr_octree;
int amr_octree_create(uint32_t node_slots, amr_octree** out);
int amr_octree_destroy(amr_octree* o);
int amr_octree_add_node(amr_octree* o, int32_t parent, int32_t offset);        /* AMR.h:208-232 */
int amr_octree_remove_node(amr_octree* o, int32_t node);                       /* AMR.h:233-254 */
/* The same calls in order, as one batch: the final state equals n single calls, but the
 * boundary refresh each single call makes over all nodes at or below its depth (AMR.h:231,
 * 253) is done once, and the maximum depth after a removal is kept by counts per depth instead
 * of a scan of all slots (AMR.h:243-246).  A batch of removals must not contain a node added in
 * the same batch. */
int amr_octree_add_nodes(amr_octree* o, const int32_t* parents, const int32_t* offsets, uint32_t n);
int amr_octree_remove_nodes(amr_octree* o, const int32_t* nodes, uint32_t n);
int amr_octree_increment_timer(amr_octree* o);                                 /* AMR.h:180-188 */
/* Periodic root (no counterpart in the reference, whose neighbour outside the root is the root's
 * frozen ghost layer, AMR.h:276-290): a face leaving the root takes the domain on the opposite side,
 * found as any neighbour is, with its offset given as if it lay beside this domain. */
int amr_octree_set_periodic(amr_octree* o, int periodic);
uint32_t amr_octree_find_node_idx(const amr_octree* o, uint32_t packed_pos, uint32_t max_depth); /* AMR.h:255-263 */
/* scalars: timer_helper, max_depth, first_free_slot, curr_used_slots, max_slots.  Any output
 * pointer may be NULL; arrays hold node_slots (x8 children, x6 boundaries) entries. */
int amr_octree_state(const amr_octree* o, uint32_t* positions, int32_t* parent, int32_t* children,
                     uint64_t* boundaries, uint32_t* lifetime, uint32_t* scalars5);

/* ---------------------------------------------------------------- simulations (plugins)
 * A simulation owns an octree, the device fields of one reference plugin and its host
 * fast_prng (default seed 12894712, tensors.h:280), and runs the plugin's timestep loop
 * (AMR.h:324-333): copy_back, modify_nodes, predictor, copy_bounds, corrector, increment_timer,
 * until the counter wraps.  Kinds: */
#define AMR_SIM_BSSN 1      /* BSSN_AMR_data, BSSN.h:104-171 */
#define AMR_SIM_WAVE 2      /* wave_AMR_data, SimpleWave.h:191-279 */
/* Execution modes: */
#define AMR_MODE_PLAIN 0    /* one launch per operator and component, in the reference's order */
#define AMR_MODE_BATCHED 1  /* fused multi-component kernels over the active-domain list */
#define AMR_MODE_GRAPH 2    /* AMR_MODE_BATCHED, each timestep replayed from a captured CUDA graph */

typedef struct amr_sim amr_sim;
int amr_sim_create(const amr_config* cfg, int kind, uint32_t node_slots, int mode, amr_sim** out);
int amr_sim_destroy(amr_sim* s);
int amr_sim_set_mode(amr_sim* s, int mode);
int amr_sim_add_node(amr_sim* s, int32_t parent, int32_t offset);     /* runs node_ctor (prolongation) */
int amr_sim_remove_node(amr_sim* s, int32_t node);
/* Batches of the same (see amr_octree_add_nodes); the new nodes' node_ctor prolongations run at
 * the end of the batch, one launch per depth level, parents before children. */
int amr_sim_add_nodes(amr_sim* s, const int32_t* parents, const int32_t* offsets, uint32_t n);
int amr_sim_remove_nodes(amr_sim* s, const int32_t* nodes, uint32_t n);
int amr_sim_octree_state(const amr_sim* s, uint32_t* positions, int32_t* parent, int32_t* children,
                         uint64_t* boundaries, uint32_t* lifetime, uint32_t* scalars5);
/* Device address and element count of a simulation buffer.
 *   BSSN: which 0 cyij_old, 1 cyij_new (padded float), 2 cRij (inner float),
 *         3 cyij_k, 4 cGijk (inner compressed_float3); comp 0..5 = xx, xy, xz, yy, yz, zz.
 *   WAVE: which 0 old_field, 1 new_field (padded float), 3 first_derivs, 4 hessian_diag
 *         (inner compressed_float3), 5 criterion (used_slots * N * N float); comp 0. */
int amr_sim_buffer(amr_sim* s, int which, int comp, void** dev_ptr, uint64_t* count);
/* Asynchronous copies between host memory (page-locked for overlap) and a simulation buffer on
 * the simulation's stream, the counterparts of smart_gpu_cpu_buffer::copy_to_gpu / copy_to_cpu
 * (CUDA_memory.h:177-184).  `count` elements (4 bytes each) from the start of the buffer. */
int amr_sim_copy_to_device(amr_sim* s, int which, int comp, const void* host, uint64_t count);
int amr_sim_copy_to_host(amr_sim* s, int which, int comp, void* host, uint64_t count);
/* The same read, on the simulation's side stream: it runs after the work already enqueued on the
 * simulation's stream and may overlap what is enqueued afterwards (uploads of other buffers); the
 * next timestep, copy_bounds, add_node or upload into this buffer waits for it.  Completion:
 * amr_sim_synchronize. */
int amr_sim_copy_to_host_side(amr_sim* sim, int which, int comp, void* host, uint64_t count);
/* Transfers that overlap the simulation's work (no counterpart in the reference, whose copies
 * block).  Each buffer has a device staging copy per direction; host transfers run on an upload
 * and a download stream, and the simulation's stream meets them only at a device-to-device copy.
 *   amr_sim_stage_to_device: host -> staging starts at once (after the staging copy's previous
 *     contents were taken), and staging -> buffer is enqueued on the simulation's stream after the
 *     work already there.  Calling it right after amr_sim_timestep uploads the next step's input
 *     while this step computes.
 *   amr_sim_snapshot_to_host: buffer -> staging is enqueued on the simulation's stream (the next
 *     timestep may overwrite the buffer at once), staging -> host follows on the download stream,
 *     overlapping later work.
 * `host` must stay valid (and, for uploads, unchanged) until the transfer is complete:
 * amr_sim_synchronize, or an amr_sim_event_record (which follows the downloads) that has
 * completed. */
int amr_sim_stage_to_device(amr_sim* sim, int which, int comp, const void* host, uint64_t count);
int amr_sim_snapshot_to_host(amr_sim* sim, int which, int comp, void* host, uint64_t count);
/* The same transfers for n (at most 36) distinct buffers at once: arrays of (which, comp, host,
 * count).  The device-to-device copies of all of them are one launch on the simulation's stream;
 * the host transfers are one per buffer on the transfer stream.  Results equal n single calls. */
int amr_sim_stage_many(amr_sim* sim, uint32_t n, const int* which, const int* comp, const void* const* host,
                       const uint64_t* count);
int amr_sim_snapshot_many(amr_sim* sim, uint32_t n, const int* which, const int* comp, void* const* host,
                          const uint64_t* count);
/* Checkpoint of a simulation into the existing directory `dir`: the octree arrays
 * (positions.bin, parent.bin, children.bin, boundaries.bin, lifetime.bin), every field buffer
 * amr_sim_buffer names (field_<which>_<comp>.bin), each the raw little-endian bytes of the whole
 * array as the reference's write_to_file (io_helper.h:9-17) writes a buffer, and state.bin
 * (16 uint32: "CKPT", version 1, kind, size_domain, padding_domain, outer_size bits, node_slots,
 * timer, max depth, first free slot, final used slot, generator state, 0...).  amr_sim_load restores
 * them into a simulation of the same kind, configuration and node_slots (else AMR_ERR_INVALID);
 * a resumed timestep is bit-identical to an uninterrupted one.  Both synchronise the stream.  The
 * reference has no checkpoint of its own. */
int amr_sim_save(amr_sim* sim, const char* dir);
int amr_sim_load(amr_sim* sim, const char* dir);
/* Timing events on the simulation's stream: record event `slot` (0..15) after all work enqueued
 * so far (side-stream copies included), and read the milliseconds between two recorded events
 * (waits for the later one). */
int amr_sim_event_record(amr_sim* s, int slot);
int amr_sim_event_elapsed(amr_sim* s, int first, int second, float* ms);
int amr_sim_timestep(amr_sim* s);                                      /* the plugin's timestep() */
int amr_sim_copy_bounds(amr_sim* s);                                   /* the plugin's copy_bounds() */
/* One phase of the plugin interface (AMR.h:296-334), for a caller that runs the reference's loop
 *   do { copy_back; modify_nodes; predictor; copy_bounds; corrector; increment_timer } while (timer)
 * itself (AMR.h:324-333): each call issues that phase's work on the simulation's stream and draws
 * its seeds from the simulation's generator, so the loop of phases gives amr_sim_timestep's
 * results bit for bit.  A single phase is self-contained (the BSSN copy_back restricts every
 * active domain; inside amr_sim_timestep the leaves' restriction is fused into the predictor). */
#define AMR_PHASE_COPY_BACK 0
#define AMR_PHASE_MODIFY_NODES 1
#define AMR_PHASE_PREDICTOR 2
#define AMR_PHASE_COPY_BOUNDS 3
#define AMR_PHASE_CORRECTOR 4
#define AMR_PHASE_INCREMENT_TIMER 5   /* AMR<T>::increment_timer (AMR.h:180-188) */
int amr_sim_phase(amr_sim* s, int phase);
/* Replace the simulation's octree with arrays in the layout amr_sim_octree_state returns (the
 * reference's AMR<T> arrays, AMR.h:118-136, and scalars5 = timer, max depth, first free slot,
 * used slots, node_slots), as AMR<T>::copy_to_gpu uploads them (AMR.h:268-275), for a caller that
 * keeps its own octree.  Children, parents and boundary targets must name slots and positions be
 * free or at most 8 deep (AMR.h:9), else AMR_ERR_INVALID.  Fields are not touched (prolongate new nodes with
 * amr_copy_to_child on amr_sim_buffer's addresses). */
int amr_sim_set_octree(amr_sim* s, const uint32_t* positions, const int32_t* parent, const int32_t* children,
                       const uint64_t* boundaries, const uint32_t* lifetime, const uint32_t* scalars5);
int amr_sim_rng(const amr_sim* s, int32_t* seed);
int amr_sim_set_rng(amr_sim* s, int32_t seed);
int amr_sim_stream(amr_sim* s, void** stream);
/* Enqueue the simulation's work on a caller-supplied stream from now on (the reference passes its
 * cudaStream_t& to every operator, AMR.h:880-1310); nullptr returns to the simulation's own stream.
 * Everything queued so far completes first.  The stream must not be the legacy default stream
 * (AMR_MODE_GRAPH captures on it) and must outlive its use by the simulation (amr_sim_destroy
 * synchronises it but does not destroy it).  Not during a stream capture. */
int amr_sim_set_stream(amr_sim* s, void* stream);
/* Wait for the simulation's work; AMR_ERR_TIMEOUT (once) if a kernel gave up a bounded wait. */
int amr_sim_synchronize(amr_sim* s);
/* Kernel launches the library issued for this simulation since creation (graph replays count
 * the kernels in the graph). */
uint64_t amr_sim_kernel_launches(const amr_sim* s);
/* Test hook of the failure path (no counterpart in the reference): with spin_limit != 0 the fused
 * BSSN pass's data waits give up after that many polls, and with withhold_plane = q + 1 each CTA's
 * producer skips its q-th plane request, so the waits on it run out.  The pass then leaves with
 * invalid results and amr_sim_synchronize returns AMR_ERR_TIMEOUT (once).  (0, 0) turns it off. */
int amr_sim_set_fault_injection(amr_sim* s, uint32_t spin_limit, uint32_t withhold_plane);
/* Number of CTAs of the fused BSSN derivative pass (AMR_MODE_BATCHED / AMR_MODE_GRAPH), in place
 * of the library's choice; 0 restores it.  Results do not depend on it (every CTA takes an equal
 * contiguous range of the active domains' planes).  The reference sizes its launches from the
 * domain constants instead (AMR.h:1119-1142). */
int amr_sim_set_stencil_ctas(amr_sim* s, uint32_t ctas);
/* Launch-shape autotuner (no counterpart in the reference, whose launch shapes are fixed by the
 * domain constants, AMR.h:647-668, 1119-1142).  Times candidate shapes reps times each with CUDA
 * events on the simulation's stream and keeps the fastest; synchronises the stream; call it
 * between timesteps, after the octree changes.
 *   AMR_SIM_BSSN: the fused derivative pass's grid, for every distinct number of active domains
 *   among the octree's substeps (candidates: the library's rule, 1-4 CTAs per SM, ranges of 2-64
 *   planes per CTA), used by AMR_MODE_BATCHED / AMR_MODE_GRAPH for that count (a fixed
 *   amr_sim_set_stencil_ctas still wins).  The candidate launches write only scratch memory
 *   allocated for the call.
 *   AMR_SIM_BSSN_EVOLVE / AMR_SIM_WAVE_RK4: the derivative pass's slab depth (interior z-planes
 *   per CTA: 1, 2 or 4 at 16^3; 4 or 8 at 8^3; 1 at 32^3), timed over every evolved domain; the
 *   pass writes only its derivative scratch, which every RK stage rewrites.
 * The simulation's state is unchanged.  *n_tuned = shapes tuned.  AMR_SIM_WAVE: AMR_ERR_INVALID. */
int amr_sim_autotune(amr_sim* s, uint32_t reps, uint32_t* n_tuned);
/* The tuned pairs, up to capacity: (active domains, CTAs of the fused pass) for AMR_SIM_BSSN,
 * (evolved domains, z-planes per derivative slab) for the evolution kinds; *count = how many
 * there are (AMR_ERR_CAPACITY if more than capacity). */
int amr_sim_tuned_shapes(const amr_sim* s, uint32_t capacity, uint32_t* domains, uint32_t* ctas, uint32_t* count);
/* Optional timing of the dominant kernel (the derivative stencil) with CUDA events on the
 * simulation's stream.  amr_sim_kernel_timing returns the summed milliseconds and launch count
 * since the last reset. */
int amr_sim_enable_kernel_timing(amr_sim* s, int enable);
int amr_sim_kernel_timing(amr_sim* s, double* ms, uint64_t* launches);

/* ---------------------------------------------------------------- evolution
 * The physics the reference's BSSN plugin stops short of (it recomputes metric derivatives and
 * Christoffel symbols only, BSSN.h:143-159, and its one time integrator is SimpleWave's two-stage
 * update, SimpleWave.h:7-46): the full BSSN system in moving-puncture form and the scalar wave
 * u_tt = Δu, both with RK4 on the reference's octree, 2:1 subcycling driven by the same
 * 0..2^max_depth-1 counter (AMR.h:180-188, 634-644), ghost cells filled from coarser-or-equal
 * neighbours with space and time interpolation (AMR.h:701-762; edges and corners included here)
 * and restriction of children into parents (AMR.h:961-996).  Simulations of these kinds use the
 * amr_sim_* entry points above (create, add / remove nodes, timestep, buffers, save / load).
 * Compiled for padding_domain 3 and size_domain 8, 16 or 32.  No counterpart in the reference. */
#define AMR_SIM_BSSN_EVOLVE 3   /* 24 fields: chi, gt_ij (6), K, At_ij (6), Gt^i (3), alpha, beta^i (3), B^i (3) */
#define AMR_SIM_WAVE_RK4 4      /* 2 fields: u, v = u_t */
/* Buffers of these simulations (amr_sim_buffer, comp = field): which 0 the state at the start of
 * the current step (padded), 1 the latest state (padded), 2 the RK stage state (padded), 3 the RK
 * accumulator (inner layout), 4 the constraints H, M_x, M_y, M_z (inner layout, comp 0..3, written
 * by amr_sim_constraint_norms), 5 derivative scratch planes (inner layout).  The BSSN fields chi,
 * gt_xx, gt_yy, gt_zz and alpha are stored less 1 (their deviation from flat space), which keeps
 * single-precision rounding relative to the deviation. */
#define AMR_SLICING_1PLUSLOG 0  /* d_t alpha = beta.d alpha - 2 alpha K */
#define AMR_SLICING_HARMONIC 1  /* d_t alpha = beta.d alpha - alpha^2 K */
typedef struct amr_evolution {
    int slicing;        /* AMR_SLICING_* */
    int shift;          /* 0: shift frozen at its initial value (zero), 1: Gamma-driver */
    float eta;          /* Gamma-driver damping (e.g. 2) */
    float ko_sigma;     /* Kreiss-Oliger dissipation strength (e.g. 0.1; 0 turns it off) */
    float cfl;          /* dt = cfl * dx at every depth (e.g. 0.25) */
    int periodic;       /* 1: the root is periodic (opposite faces are neighbours) */
} amr_evolution;
#define AMR_ID_FLAT 0
#define AMR_ID_GAUGE_WAVE 1       /* alpha^2 = gamma_xx = 1 - A sin(2 pi x / d) (Alcubierre et al. 2004) */
#define AMR_ID_BRILL_LINDQUIST 2  /* psi = 1 + sum m_a / (2 r_a), chi = psi^-4, alpha = psi^-2 */
#define AMR_ID_GAUSSIAN_PULSE 3   /* wave: u = exp(-|x|^2 / width^2), u_t = 0 */
typedef struct amr_initial_data {
    int kind;                 /* AMR_ID_* */
    float amplitude;          /* gauge wave A */
    float wavelength;         /* gauge wave d */
    int n_punctures;          /* Brill-Lindquist: up to 4 */
    float mass[4];
    float position[4][3];     /* in the coordinates of the root, which spans [-outer_size/2, outer_size/2]^3 */
    float width;              /* Gaussian pulse */
} amr_initial_data;
/* Set the physics and gauge of an AMR_SIM_BSSN_EVOLVE / AMR_SIM_WAVE_RK4 simulation. */
int amr_sim_set_evolution(amr_sim* s, const amr_evolution* e);
/* Write analytic initial data into every cell (ghosts included) of both state buffers of every live
 * slot; the counter is reset to 0.  Build the octree first. */
int amr_sim_initial_data(amr_sim* s, const amr_initial_data* d);
/* Hamiltonian and momentum constraints of the current state over the composite grid (every interior
 * cell that no child covers), leaving out cells closer than excision_radius to a puncture of the
 * initial data (0: none), reduced in double precision with a fixed order:
 * out5 = {rms H, max |H|, rms |M|, max |M|, cells} (|M| the Euclidean norm of M_i).  The constraint
 * fields themselves are amr_sim_buffer(4, 0..3).  Synchronises the simulation's stream.  BSSN only. */
int amr_sim_constraint_norms(amr_sim* s, float excision_radius, double* out5);

/* ---------------------------------------------------------------- learned refinement estimator
 * No counterpart in the reference, whose refinement is a gradient / curvature threshold per octant
 * (SimpleWave.h:91-187, 228-248).  A small network predicts each tile's (domain's) log10 truncation
 * error from 3 x 8^3 features (conformal factor, lapse, |d gt| dx, averaged onto 8^3): conv 3->16
 * (3^3, ReLU), conv 16->16 (3^3, stride 2, ReLU), dense 1024->32 (ReLU), dense 32->1.  Forward and
 * backward run on the tcgen05 tensor cores (BF16 operands, FP32 accumulation in Tensor Memory); FP32 master weights and
 * Adam.  Buffers are device pointers; features are [tile][3][512] floats. */
typedef struct amr_estimator amr_estimator;
int amr_estimator_create(uint32_t max_batch, uint64_t seed, amr_estimator** out);
int amr_estimator_destroy(amr_estimator* e);
uint64_t amr_estimator_param_count(void);
/* The FP32 parameters as one flat host array: W1[96][16] (rows 81..95 zero), b1[16], W2[432][16],
 * b2[16], W3[1024][32], b3[32], W4[32], b4[1]; im2col row j = channel * 27 + dz * 9 + dy * 3 + dx. */
int amr_estimator_get_params(amr_estimator* e, float* host);
int amr_estimator_set_params(amr_estimator* e, const float* host);
/* Predictions for n tiles (any n; batches of max_batch), synchronous. */
int amr_estimator_forward(amr_estimator* e, const float* features, uint32_t n, float* out);
/* Gradients of the mean squared error against targets (n <= max_batch) into a host array laid out
 * as the parameters; *loss = the mean squared error.  One Adam step with amr_estimator_train_step. */
int amr_estimator_gradients(amr_estimator* e, const float* features, const float* targets, uint32_t n,
                            float* grads_host, float* loss);
int amr_estimator_train_step(amr_estimator* e, const float* features, const float* targets, uint32_t n, float lr,
                             float* loss);
/* Features (device [n][3][512]), plain-criterion indicators (device [n]: the largest undivided
 * gradient |d chi| + |d alpha| over the tile's cells) and slots (host [n]) of the leaves of a BSSN
 * evolution, from its latest state.  Per cell of an 8^3 grid over the tile: the mean conformal
 * factor, log10(max(|d chi| + |d alpha|) + 1e-10) / 5 + 1, log10(rms |d gt| + 1e-10) / 5 + 1.
 * *n_leaves is set even when capacity is too small (AMR_ERR_CAPACITY). */
int amr_sim_tile_features(amr_sim* s, float* features, float* indicators, uint32_t* leaf_slots, uint32_t capacity,
                          uint32_t* n_leaves);
typedef struct amr_regrid {
    float refine_threshold;   /* plain criterion: refine a leaf whose indicator exceeds this */
    float coarsen_threshold;  /* plain criterion: a leaf below this may merge with its siblings */
    float learned_refine;     /* network: refine a leaf whose predicted log10 error exceeds this */
    float learned_coarsen;    /* network: a leaf predicted below this may merge with its siblings */
    float judge_factor;       /* the plain criterion refines a leaf the network declines when its
                                 indicator exceeds judge_factor * refine_threshold (>= 1) */
    uint32_t max_depth;       /* no leaf is refined beyond this depth */
    uint32_t min_depth;       /* no parent shallower than this is coarsened */
} amr_regrid;
/* Refine / coarsen the leaves of a BSSN evolution between timesteps: with an estimator its
 * predictions decide and the plain criterion is the judge (overriding declined refinements it
 * finds strong, and vetoing coarsening where it would refine); with est == NULL the plain
 * criterion decides.  New domains are interpolated from their parents' padded cells (tricubic, as
 * for every domain added to an evolution; the parents' ghost layers are refilled first), removed
 * ones dropped, ghost cells refilled.  stats4 (optional) = {refined leaves, coarsened parents,
 * refinements the judge forced, leaves after}. */
int amr_sim_regrid(amr_sim* s, amr_estimator* est, const amr_regrid* r, uint32_t* stats4);

/* ---------------------------------------------------------------- scan and reductions
 * The reference's general-purpose device algorithms (AdaptiveMesh/parallel.h) on a device array
 * of `count` elements (count < 2^32), each `ncomp` (1-4) consecutive values of type `dtype` (the
 * reference's uint/int/float and their 2-4 component vector types).  The values computed and the
 * values left in the array are the reference's, float rounding included.  All three run on
 * `stream` (NULL: the default stream); the reductions return after writing `ncomp` values to
 * host memory at `result`. */
#define AMR_DTYPE_UINT32 0
#define AMR_DTYPE_INT32 1
#define AMR_DTYPE_FLOAT32 2
/* In place inclusive cumulative sum, apply_incl_cum_sum (parallel.h:62-82). */
int amr_inclusive_scan(int dtype, int ncomp, void* data, uint64_t count, void* stream);
/* Component-wise maximum, find_maximum_val (parallel.h:239-251); the array is used as scratch
 * as by the reference (elements k * 512^j end with partial results). */
int amr_reduce_max(int dtype, int ncomp, void* data, uint64_t count, void* result, void* stream);
/* Component-wise minimum, find_minimum_val (parallel.h:409-421).  As in the reference, a block
 * of 512 that runs past the end of the array counts its missing elements as 0 (parallel.h:389),
 * so the result is at most 0 unless every pass fills its blocks. */
int amr_reduce_min(int dtype, int ncomp, void* data, uint64_t count, void* result, void* stream);
/* Norms of a padded field (slot-major, the layout of cyij_old / old_field) over the interior cells
 * of the leaf domains (live slots with no children, from the device arrays positions[used] and
 * children[8 * used]), in double precision, for monitoring a field or a constraint residual:
 * out4 = {sum, sum of squares, largest magnitude (NaN if any cell is NaN), number of cells}.  The
 * reduction order is fixed, so a result repeats exactly.  Synchronises the stream.  No counterpart
 * in the reference, which has no FP64 reductions. */
int amr_field_norms(const amr_config* cfg, const float* field, const uint32_t* positions, const int32_t* children,
                    uint32_t used_slots, double* out4, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* AMR_GB300_H */
