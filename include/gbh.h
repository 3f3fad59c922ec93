/*
 * gbh.h — C ABI of the GB300-native Barnes–Hut step.
 *
 * This header is the drop-in boundary for the per-step pipeline of the
 * gkane1234/gravity simulator.  A Java host (Panama FFM or JNI), a Python host
 * (ctypes) or C/C++ code binds these entry points; nothing in the signatures is
 * a torch or CUDA-runtime type (streams are passed as opaque `void*`).
 *
 * Reference interface replaced (paths inside the reference project):
 *   - BarnesHut.init()/step()          src/main/java/com/grumbo/simulation/BarnesHut.java:99-173
 *   - GPU.initGPU()/uploadPlanetsData  src/main/java/com/grumbo/gpu/GPU.java:172-188, 1166-1196
 *   - the SSBO binding table           src/main/java/com/grumbo/gpu/SSBO.java:40-55,
 *                                      src/main/resources/shaders/common/common.glsl:80-120
 *   - uniforms of the step             common.glsl:126-158, GPU.java:402-498
 *
 * Layouts are byte-identical to the reference's std430 SSBO layouts so buffers
 * read back from this library can be handed to code written for the reference.
 *
 * Error convention: every entry point returns an int status (GBH_OK == 0,
 * negative == error class).  gbh_last_error(ctx) returns a human-readable
 * message for the last failing call on that context; gbh_last_error(NULL)
 * returns the message of the last failing gbh_create on this thread.  No C++
 * exception crosses this boundary.
 *
 * Threading: one context per host thread; calls on one context must be
 * serialised by the caller (the reference runs everything on its single GL
 * thread, GPUSimulation.java:379-384).  All device work of a context runs on
 * the context's own CUDA stream.
 */
#ifndef GBH_H
#define GBH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBH_ABI_VERSION 1

/* ---- status codes -------------------------------------------------------- */
#define GBH_OK 0
#define GBH_ERR_INVALID (-1)  /* bad argument (null pointer, size out of range, bad enum) */
#define GBH_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define GBH_ERR_OOM (-3)      /* device allocation failed */
#define GBH_ERR_DEVICE (-4)   /* a kernel raised the device error word (see gbh_stats.error_word) */
#define GBH_ERR_STATE (-5)    /* call out of order (e.g. step before init) */
#define GBH_ERR_UNSUPPORTED (-6)

/* ---- device error word bits (gbh_stats.error_word) ------------------------ */
#define GBH_DEVERR_SORT_LOOKBACK 0x1u   /* onesweep look-back spin gave up (bounded wait) */
#define GBH_DEVERR_FILL_SPIN 0x2u       /* bottom-up fill: frontier list overflow (cannot happen at its capacity N) */
#define GBH_DEVERR_WALK_STACK 0x4u      /* a tree walk needed more stack than GBH_WALK_STACK */
#define GBH_DEVERR_MERGE_OVERFLOW 0x8u  /* merge resolution did not finish (cannot happen: each round runs a task) */
#define GBH_DEVERR_TREE_HEIGHT 0x10u    /* tree height above 64 (the reference fills only 64 levels) */
#define GBH_DEVERR_MAC_FRONTIER 0x20u   /* learned walk frontier overflow */

/* ---- enums mirroring the reference uniforms ------------------------------ */
/* mergingCollisionOrNeither (common.glsl:133-140, defaultProperties.json order) */
#define GBH_MODE_NEITHER 0u
#define GBH_MODE_MERGE 1u
#define GBH_MODE_COLLISION 2u
/* staticOrDynamic (common.glsl:146-149) */
#define GBH_BOUNDS_STATIC 0u
#define GBH_BOUNDS_DYNAMIC 1u
/* acceptance criterion of the walk (new in this library) */
#define GBH_MAC_PLAIN 0u    /* reference rule: (longest AABB side / 2) * invDist < theta, per body */
#define GBH_MAC_LEARNED 1u  /* learned MLP criterion, one decision per (body group of up to 96, node) */
#define GBH_MAC_GROUP 2u    /* group theta rule used as the learned criterion's ablation */
/* precision form (new in this library) */
#define GBH_PRECISION_FP32 0u     /* reference arithmetic */
/* GBH_PRECISION_COMPENSATED: FP64 positions on the device (the drift
 * x += v dt runs in FP64; the body buffer holds their FP32 rounding), the
 * Morton quantisation from the FP64 positions, and walk coordinates relative
 * to the body (plain walk) or to the group centre (group walks) formed from
 * the FP32 position plus its FP32 residual, with Kahan-compensated sums of
 * the near field (leaf) terms.  Gravity only (merging_collision_or_neither 0).
 * The FP64 positions start from the body buffer at the first such step and
 * after every gbh_upload_bodies or FP32 step. */
#define GBH_PRECISION_COMPENSATED 1u

/* step flags */
#define GBH_FLAG_STORE_ACCEL 0x1u      /* keep each body's walk acceleration (gbh_read_accel) */
#define GBH_FLAG_STORE_POTENTIAL 0x2u  /* keep each body's walk potential (gbh_read_potential,
                                          the potential energy of gbh_diagnostics) */

/* ---- buffers, byte-identical to the reference std430 layouts -------------- */

/* struct Body, common.glsl:25-29 (32 bytes). Empty <=> pos_mass[3] == 0. */
typedef struct gbh_body {
    float pos_mass[4];    /* x, y, z, mass */
    float vel_density[4]; /* vx, vy, vz, density */
} gbh_body;

/* struct Node, common.glsl:40-58 (80 bytes).  Leaves are indexed by sorted
 * position; internal node ids are offset by initialNumBodies; a leaf has
 * child_a == 0xFFFFFFFF. */
typedef struct gbh_node {
    float com_mass[4];      /* @0  centre of mass xyz, mass */
    float aabb[6];          /* @16 min xyz, max xyz */
    uint32_t child_a;       /* @40 */
    uint32_t child_b;       /* @44 */
    uint32_t node_depth;    /* @48 height above the deepest leaf after the fill */
    uint32_t bodies_contained; /* @52 */
    uint32_t ready_children;   /* @56 0xFFFFFFFF once filled */
    uint32_t parent_id;        /* @60 0xFFFFFFFF for the root */
    float avg_color[4];        /* @64 mass-weighted star colour (rgb), w unused */
} gbh_node;

/* buffer SimulationValues, common.glsl:86-88, with std430 offsets (896 bytes
 * as allocated by GPU.java:1096-1143). */
typedef struct gbh_sim_values {
    uint32_t num_bodies;         /* @0 live bodies */
    uint32_t initial_num_bodies; /* @4 capacity */
    uint32_t just_died;          /* @8 */
    uint32_t merged;             /* @12 (never incremented by the reference) */
    uint32_t out_of_bounds;      /* @16 cumulative count of bodies killed out of bounds */
    uint32_t relative_to;        /* @20 */
    uint32_t pad1, pad2;         /* @24 */
    float bounds_min[3];         /* @32 */
    uint32_t pad_min;            /* @44 */
    float bounds_max[3];         /* @48 */
    uint32_t pad_max;            /* @60 */
    float unit_mass;             /* @64 */
    float unit_density;          /* @68 */
    float unit_len;              /* @72 */
    float unit_time;             /* @76 */
    float camera_scale;          /* @80 */
    float gravitational_constant;/* @84 */
    float body_length_constant;  /* @88 bodyLengthInSimulationLengthsConstant */
    uint32_t uint_debug[100];    /* @92 uint_debug[0] = internal nodes opened by the walk */
    float float_debug[100];      /* @492 */
    uint32_t tail_pad;           /* @892 */
} gbh_sim_values;

/* UnitSet (common.glsl:61-70, UnitSet.java:242-245).  G and the body length
 * constant are derived from these in FP32 like common.glsl:346-360 unless
 * gravitational_constant > 0, which then overrides the derived G. */
typedef struct gbh_units {
    float mass;
    float density;
    float len;
    float time;
    float camera_scale;
    float gravitational_constant; /* > 0: use this G directly */
} gbh_units;

/* The step's uniforms (common.glsl:126-158). */
typedef struct gbh_step_params {
    float dt;
    float theta;
    float softening;   /* added to r.r directly: this is eps^2 (bh_force.comp:27-32) */
    float elasticity;
    float restitution; /* the reference hard-codes 0.2 (GPU.java:442-446) */
    uint32_t merging_collision_or_neither; /* GBH_MODE_* */
    uint32_t static_or_dynamic;            /* GBH_BOUNDS_* */
    uint32_t wrap_around;                  /* static bounds: wrap instead of kill */
    gbh_units units;   /* units.mass == 0 keeps the current units (bh_update.comp:22-25) */
    uint32_t mac_mode;        /* GBH_MAC_* */
    uint32_t precision_mode;  /* GBH_PRECISION_* */
    float mac_tolerance;      /* learned MAC: accept when predicted log10 error < this */
    uint32_t flags;           /* GBH_FLAG_* */
} gbh_step_params;

/* Per-step counters (read with gbh_read_stats). */
typedef struct gbh_stats {
    uint64_t interactions;   /* body-node force evaluations (accepted nodes + leaves) */
    uint64_t nodes_opened;   /* body-node openings (equals sim.uint_debug[0] when it fits) */
    uint64_t mac_evaluations;/* learned/group walk: (group, node) criterion evaluations */
    uint32_t alive;          /* live bodies after compaction */
    uint32_t died;           /* bodies removed by this step's compaction */
    uint32_t merged;         /* merge tasks applied */
    uint32_t merge_tasks;    /* merge tasks emitted by the walk */
    uint32_t merge_conflicts;/* tasks that shared a body with another task */
    uint32_t out_of_bounds;  /* bodies killed out of bounds in this step */
    uint32_t tree_height;    /* height of the root */
    uint32_t max_stack;      /* deepest walk stack seen */
    uint32_t error_word;     /* GBH_DEVERR_* bits, sticky until gbh_clear_error */
    uint32_t frontier_saturated; /* group walks whose candidate stack filled up: nodes were
                                    accepted instead of opened (less accurate, still a valid sum) */
} gbh_stats;

/* Device pointers of the live buffers, for headless consumers that replace the
 * reference's render shaders reading the same SSBOs (nodeglow.vert, regions.vert,
 * impostor.vert).  Valid until the next gbh_step (body/index buffers swap) or
 * gbh_step_streamed (which rotates the body buffers through two more). */
typedef struct gbh_device_buffers {
    void* bodies_in;      /* gbh_body[initial_num_bodies] (current state) */
    void* bodies_out;
    void* leaf_nodes;     /* gbh_node[initial_num_bodies] */
    void* internal_nodes; /* gbh_node[initial_num_bodies - 1] */
    void* sim_values;     /* gbh_sim_values */
    void* morton_in;      /* uint64_t[initial_num_bodies] sorted keys */
    void* index_in;       /* uint32_t[initial_num_bodies] sorted body indices */
    void* merge_tasks;    /* uint32_t head, tail, then uint32_t[2] pairs */
} gbh_device_buffers;

typedef struct gbh_ctx gbh_ctx;

/* ---- lifecycle ----------------------------------------------------------- */

/* GPU.initGPU (GPU.java:172-358): allocate every buffer for `initial_num_bodies`
 * bodies on `device` and write SimulationValues like GPU.packValues
 * (GPU.java:1096-1143).  bounds = {minx, miny, minz, maxx, maxy, maxz}. */
int gbh_create(gbh_ctx** out, uint32_t initial_num_bodies, const float bounds[6],
               const gbh_units* units, int device);
int gbh_destroy(gbh_ctx* ctx);

/* GPU.uploadPlanetsData (GPU.java:1166-1196): copy `count` bodies into the
 * current body buffer starting at body `offset` (chunked uploads allowed). */
int gbh_upload_bodies(gbh_ctx* ctx, const gbh_body* host, uint32_t count, uint32_t offset);
/* Read bodies [offset, offset + count) of the current body buffer into
 * `host_out` and replace them with `host_in`, in one call: the range moves in
 * chunks, each chunk's upload waiting only for its own read-back, so the two
 * directions run at the same time on the GPU's two copy engines (with pinned
 * host memory).  For a host that streams states through the simulation: one
 * call per step returns the last step's bodies and installs the next input.
 * Returns when both copies have finished; the buffers must not overlap. */
int gbh_exchange_bodies(gbh_ctx* ctx, gbh_body* host_out, const gbh_body* host_in, uint32_t count, uint32_t offset);

/* Streamed steps, for a host that hands the simulation a new state every step
 * or keeps every step's state (the headless counterpart of the reference's
 * per-frame recording, src/main/java/com/grumbo/record/FrameRecorder.java,
 * which captures rendered frames), without stalling the GPU on the copies.
 * No single reference call is replaced; it combines BarnesHut.step with the
 * body upload (GPU.java:1166-1196) and read-back (SSBO.java:274-290).
 * One call:
 *   - runs one step (gbh_step) on the current state;
 *   - while it runs, copies `next_input` (initial_num_bodies bodies, host
 *     memory; pinned memory lets the copy overlap) to the device, and copies
 *     the result of the PREVIOUS call's step into `last_result`;
 *   - after the step, keeps its result for the next call and makes
 *     `next_input` the current state (the step after it starts from it).
 * `next_input` NULL: the step's result stays the current state (a plain
 * simulation whose every state is streamed back).  `last_result` NULL, or the
 * first call: no result is copied.  Returns when both copies have finished
 * (the host buffers may be reused); the step itself may still be running.
 * gbh_step_streamed_finish copies the last call's result and waits for the
 * context.  The first call allocates three body-sized device buffers: the
 * body buffers rotate through them, so no body buffer is copied on the device
 * (device pointers from gbh_device_ptrs change with every call). */
int gbh_step_streamed(gbh_ctx* ctx, const gbh_step_params* params, const gbh_body* next_input,
                      gbh_body* last_result);
int gbh_step_streamed_finish(gbh_ctx* ctx, gbh_body* last_result);

/* BarnesHut.init (BarnesHut.java:170-173, bh_init.comp:10-27): identity index,
 * derive G and the body length constant. */
int gbh_init(gbh_ctx* ctx);

/* BarnesHut.step (BarnesHut.java:99-164): one full step, launched as one CUDA
 * graph on the context stream.  Asynchronous; errors raised by kernels are
 * reported by the next synchronising call (read_* / gbh_synchronize). */
int gbh_step(gbh_ctx* ctx, const gbh_step_params* params);
/* `count` steps back to back with the same parameters. */
int gbh_step_n(gbh_ctx* ctx, const gbh_step_params* params, uint32_t count);

/* Wait for the context stream and return GBH_ERR_DEVICE if the device error
 * word is non-zero. */
int gbh_synchronize(gbh_ctx* ctx);
int gbh_clear_error(gbh_ctx* ctx);

/* ---- sharded step (one process per GPU; the exchange is the caller's) ------
 * One BarnesHut.step split over `world` ranks.  Every rank holds the whole
 * state and builds the whole tree (the stages before the walk are
 * deterministic, so all ranks build the same one); each walks only its share
 * of the live bodies, sorted slots [n r / W, n (r + 1) / W) (the group walks:
 * the groups whose first slot lies there).  The reference walks every body
 * independently of the others (bh_force.comp:40-142), so the split walk
 * equals the whole walk body for body.  Per step, on every rank:
 *   1. gbh_step_shard_walk: reset, compaction, sort, build, fill and this
 *      rank's walk; range = the sorted slots [lo, hi) it updated (the ranks'
 *      ranges tile [0, n) in rank order);
 *   2. gbh_shard_pack: its updated bodies, slot order, into a DEVICE buffer
 *      (with their acceleration magnitudes: 36 bytes per body);
 *   3. the caller all-gathers the ranges and packed bodies (NCCL, or any
 *      transport), and gbh_shard_unpack installs every other rank's range;
 *   4. gbh_read_merge_tasks_full / gbh_write_merge_tasks: the caller gathers
 *      every rank's merge tasks and writes the union (any order) on every rank;
 *   5. gbh_step_shard_finish: adds the other ranks' out-of-bounds kills to
 *      SimulationValues.outOfBounds, resolves the merges and swaps.
 * The state is then the same on every rank and equal, bit for bit, to one
 * gbh_step on one rank.  FP32 form only (GBH_ERR_UNSUPPORTED otherwise). */
int gbh_step_shard_walk(gbh_ctx* ctx, const gbh_step_params* params, uint32_t rank, uint32_t world,
                        uint32_t range[2]);
/* the packed form of `count` updated bodies: count gbh_body records, then
 * count floats |a| of their walk (the learned criterion reads them in the
 * next step): GBH_SHARD_BYTES_PER_BODY bytes per body */
#define GBH_SHARD_BYTES_PER_BODY 36u
int gbh_shard_pack(gbh_ctx* ctx, uint32_t lo, uint32_t count, void* device_out);
int gbh_shard_unpack(gbh_ctx* ctx, uint32_t lo, uint32_t count, const void* device_in);
/* the last walk's merge tasks: pairs (body, other), ordering keys (sorted slot
 * << 32 | sequence) and the sorted slot of each task's second body */
int gbh_read_merge_tasks_full(gbh_ctx* ctx, uint32_t* pairs, uint64_t* keys, uint32_t* slots, uint32_t capacity,
                              uint32_t* count);
int gbh_write_merge_tasks(gbh_ctx* ctx, const uint32_t* pairs, const uint64_t* keys, const uint32_t* slots,
                          uint32_t count);
int gbh_step_shard_finish(gbh_ctx* ctx, uint32_t out_of_bounds_other_ranks);

/* ---- read-back (synchronous; host buffers are caller-owned) --------------- */
#define GBH_BODIES_IN 0u
#define GBH_BODIES_OUT 1u
int gbh_read_bodies(gbh_ctx* ctx, uint32_t which, gbh_body* host, uint32_t count, uint32_t offset);
int gbh_read_leaf_nodes(gbh_ctx* ctx, gbh_node* host, uint32_t count, uint32_t offset);
int gbh_read_internal_nodes(gbh_ctx* ctx, gbh_node* host, uint32_t count, uint32_t offset);
int gbh_read_sim_values(gbh_ctx* ctx, gbh_sim_values* host);
int gbh_read_index(gbh_ctx* ctx, uint32_t* host, uint32_t count, uint32_t offset);
int gbh_read_morton(gbh_ctx* ctx, uint64_t* host, uint32_t count, uint32_t offset);
/* merge tasks emitted by the last walk: pairs (body, other); returns the count */
int gbh_read_merge_tasks(gbh_ctx* ctx, uint32_t* host_pairs, uint32_t capacity, uint32_t* count);
/* walk acceleration per body index (needs GBH_FLAG_STORE_ACCEL): float[4] per body */
int gbh_read_accel(gbh_ctx* ctx, float* host_xyzw, uint32_t count, uint32_t offset);
int gbh_read_stats(gbh_ctx* ctx, gbh_stats* host);
/* walk potential per body index (needs GBH_FLAG_STORE_POTENTIAL): float per body,
 * sum over accepted nodes and leaves of -G m / sqrt(r.r + softening) */
int gbh_read_potential(gbh_ctx* ctx, float* host, uint32_t count, uint32_t offset);
/* FP64 positions of the precision form per body index: double[4] (x, y, z, 0) per
 * body; GBH_ERR_STATE when they are not current */
int gbh_read_positions_fp64(gbh_ctx* ctx, double* host_xyz0, uint32_t count, uint32_t offset);
/* Set FP64 positions of the precision form (double[4] per body, the fourth
 * ignored) for bodies [offset, offset + count); their FP32 body positions
 * become the rounded values.  The other bodies keep their positions. */
int gbh_write_positions_fp64(gbh_ctx* ctx, const double* host_xyz0, uint32_t count, uint32_t offset);

/* Conserved quantities of the current state, summed in FP64 over the live
 * bodies (positions from the FP64 copy when it is current).  The potential
 * energy needs the potential of the last walk (GBH_FLAG_STORE_POTENTIAL);
 * potential_valid says whether it was taken from the current state. */
typedef struct gbh_diagnostics {
    double mass;
    double momentum[3];
    double centre_of_mass[3];
    double kinetic_energy;   /* sum 1/2 m v.v */
    double potential_energy; /* 1/2 sum m phi */
    double total_energy;
    double angular_momentum[3]; /* about the origin: sum m x cross v */
    uint32_t live_bodies;
    uint32_t potential_valid;
    uint32_t positions_fp64; /* 1 when the FP64 positions were used */
    uint32_t pad;
} gbh_diagnostics;
int gbh_read_diagnostics(gbh_ctx* ctx, gbh_diagnostics* out);
int gbh_device_ptrs(gbh_ctx* ctx, gbh_device_buffers* out);
/* opaque cudaStream_t of the context */
void* gbh_stream(gbh_ctx* ctx);

/* ---- write-back, for tests and checkpoint/resume -------------------------- */
int gbh_write_sim_values(gbh_ctx* ctx, const gbh_sim_values* host);
int gbh_write_index(gbh_ctx* ctx, const uint32_t* host, uint32_t count, uint32_t offset);
int gbh_write_morton(gbh_ctx* ctx, const uint64_t* host, uint32_t count, uint32_t offset);

/* ---- stage entry points (eager launches, for parity tests and profiling) ---
 * Together, in this order, they are exactly one gbh_step:
 *   reset -> prepare -> sort -> build -> fill -> walk -> merge -> swap.   */
/* bh_update.comp:10-28 (resetValues, BarnesHut.java:193-212) */
int gbh_stage_reset(gbh_ctx* ctx, const gbh_step_params* params);
/* partitionDeadBodies + swap + decrementDeadBodies + updateBounds +
 * generateMortonCodes (BarnesHut.java:114-131; bh_dead.comp, bh_update.comp:29-34,
 * bh_morton.comp), fused into one pass over the index */
int gbh_stage_prepare(gbh_ctx* ctx, const gbh_step_params* params);
/* radixSort (BarnesHut.java:358-448; bh_radix.comp) over the live keys */
int gbh_stage_sort(gbh_ctx* ctx);
/* buildBinaryRadixTree (BarnesHut.java:453-469; bh_tree.comp:43-133) */
int gbh_stage_build(gbh_ctx* ctx);
/* computeCOMAndLocation (BarnesHut.java:474-535; bh_tree.comp:140-259) */
int gbh_stage_fill(gbh_ctx* ctx);
/* computeForce (BarnesHut.java:540-558; bh_force.comp:40-142) */
int gbh_stage_walk(gbh_ctx* ctx, const gbh_step_params* params);
/* mergeBodies (BarnesHut.java:563-579; bh_merge.comp:30-71) */
int gbh_stage_merge(gbh_ctx* ctx, const gbh_step_params* params);
/* GPU.swapBodyBuffers (GPU.java:1060-1066) */
int gbh_stage_swap(gbh_ctx* ctx);

/* ---- profiling (the reference's debug-mode per-stage timers,
 *      BarnesHut.java:628-682, as CUDA events) ---------------------------- */
#define GBH_NUM_STAGES 8
/* Run one step as eager stage launches with CUDA events between stages and
 * return per-stage milliseconds in stage order (reset, prepare, sort, build,
 * fill, walk, merge, swap). */
int gbh_step_profiled(gbh_ctx* ctx, const gbh_step_params* params, float ms_out[GBH_NUM_STAGES]);

/* ---- accuracy reference -------------------------------------------------------
 * FP64 direct-sum accelerations for `count` sampled body indices against every
 * live body of the current state: FP64 terms and FP64 sums, reduced in a fixed
 * order.  Positions are the FP32 body positions widened to FP64, or, with
 * params->precision_mode == GBH_PRECISION_COMPENSATED and current FP64
 * positions, the FP64 positions.  out: double[3*count].  Uses G and softening
 * from `params`. */
int gbh_direct_sum(gbh_ctx* ctx, const gbh_step_params* params, const uint32_t* sample,
                   uint32_t count, double* out_accel);

/* ---- learned multipole-acceptance criterion -------------------------------- */
#define GBH_MAC_FEATURES 12
#define GBH_MAC_HIDDEN 32
/* number of floats in the parameter vector: W1[32x12], b1[32], W2[32x32], b2[32], w3[32], b3[1] */
#define GBH_MAC_NUM_PARAMS (32 * 12 + 32 + 32 * 32 + 32 + 32 + 1)
int gbh_mac_set_weights(gbh_ctx* ctx, const float* params, uint32_t count);
int gbh_mac_get_weights(gbh_ctx* ctx, float* params, uint32_t count);
/* The band the network decides, as two group-rule thetas (half side of the
 * node < theta x distance from its centre of mass to the group's bounding
 * sphere): nodes that pass the rule at theta_accept are accepted without the
 * network, nodes that fail it at theta_open are opened without it.  Defaults
 * 0.25 and 4.0.  Training pairs are recorded in the same band. */
int gbh_mac_set_band(gbh_ctx* ctx, float theta_accept, float theta_open);
int gbh_mac_get_band(gbh_ctx* ctx, float* theta_accept, float* theta_open);
/* Sample (body group, node) pairs from the current tree, compute their
 * features and labels (log10 of the relative error of accepting the node's
 * monopole against its exact subtree sum, max over the group) into device
 * buffers owned by the context.  Returns the number of pairs written. */
int gbh_mac_generate(gbh_ctx* ctx, const gbh_step_params* params, uint32_t max_pairs,
                     uint64_t seed, uint32_t* out_count);
int gbh_mac_read_pairs(gbh_ctx* ctx, float* features, float* labels, uint32_t count, uint32_t offset);
/* Group and node of each generated pair, uint32_t[3] per pair: the group's
 * first sorted slot, its body count, and the node's global id. */
int gbh_mac_read_pair_ids(gbh_ctx* ctx, uint32_t* slot_count_node, uint32_t count, uint32_t offset);
int gbh_mac_write_pairs(gbh_ctx* ctx, const float* features, const float* labels, uint32_t count);
/* Train the MLP on the stored pairs with Adam (hand-written forward, backward
 * and Adam kernels; BF16 tensor-core matmuls, FP32 master weights).
 * losses: per-epoch mean loss (may be NULL). */
int gbh_mac_train(gbh_ctx* ctx, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                  float* losses);
/* Forward + backward of one batch (no update) for gradient checks:
 * features[count*12], labels[count] in host memory; grad[GBH_MAC_NUM_PARAMS]. */
int gbh_mac_loss_grad(gbh_ctx* ctx, const float* features, const float* labels, uint32_t count,
                      float* loss, float* grad);
/* Inference on host features: out[count] predicted log10 error. */
int gbh_mac_predict(gbh_ctx* ctx, const float* features, uint32_t count, float* out);

/* ---- sorting without allocation ---------------------------------------------
 * No counterpart in the reference: this entry point is new in this library.
 * For callers that cannot call cudaMalloc — a host whose device memory belongs
 * to another allocator or engine, code running while another component owns
 * the memory pool, or a loop that must never take the allocator's locks.
 * Stable ascending sort of n (uint64 key, uint32 value) pairs by all 64 key
 * bits, on device memory the caller provides.  Each output buffer is either
 * identical to its input (sorted in place) or disjoint from it; partly
 * overlapping buffers return GBH_ERR_INVALID.  Disjoint inputs are left
 * untouched.  The same onesweep kernels as the step's sort.
 *   - n is at most 1,048,576 (GBH_SORT_NOALLOC_MAX_PAIRS); larger n returns
 *     GBH_ERR_INVALID.
 *   - Allocates nothing: its scratch (about 15 MB) is a static device array
 *     that every GPU loading this library holds until exit, shared by all
 *     calls.  Each call clears what must start at zero; calls that overlap on
 *     the GPU race on the scratch and must be serialised by the caller.
 *   - The first call on a device does its set-up (the scratch's device
 *     address, with that device current); make that first call before any
 *     stream capture.  The library must not be used again on a device after a
 *     cudaDeviceReset of it.
 *   - Runs on `stream` (a cudaStream_t, NULL = default stream) on the current
 *     device, reads the device error word and synchronises `stream` before
 *     it returns, so it cannot be captured in a CUDA graph.  GBH_ERR_DEVICE
 *     when a bounded wait of the sort gave up.
 *   - Clears the calling thread's pending CUDA launch error at entry, so that
 *     GBH_ERR_CUDA reports a failure of this call's own launches. */
#define GBH_SORT_NOALLOC_MAX_PAIRS (1u << 20)
int gbh_sort_pairs_noalloc(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                           uint32_t* vals_out, uint32_t n, void* stream);

/* ---- seeded initial conditions, generated on the device ----------------------
 * gbh_generate_bodies writes bodies [offset, offset + count) of the current
 * body buffer (like gbh_upload_bodies, without a host copy).  Every number is
 * drawn from a counter-based generator keyed by (seed, body index, draw), so
 * a range generated in chunks equals the same range generated at once, on any
 * GPU.  Kinds:
 *   GBH_IC_BOX       makeNewRandomBox (PlanetGenerator.java:310-321): x, y, z,
 *                    vx, vy, vz, mass, density each uniform in [lo[k], hi[k]].
 *   GBH_IC_DISK      makeNewRandomDisk (PlanetGenerator.java:418-489): count - 1
 *                    disk bodies and, last, the centre body.  Radius uniform in
 *                    [lo[0], hi[0]], mass in [lo[6], hi[6]], density in
 *                    [lo[7], hi[7]]; disk normal (0, sin phi, cos phi); the
 *                    deviation from the plane pi (1 - U^(1 - adherence)) above
 *                    or below it; orbital speed sqrt((centre_mass + approximate
 *                    enclosed mass) G / r) * orbital_factor when flags has
 *                    GBH_IC_ORBITAL, counter-clockwise with GBH_IC_CCW.
 *   GBH_IC_PLUMMER   Plummer sphere of scale radius `scale` and mass
 *                    `total_mass` in `count` equal bodies (the count of this
 *                    call; chunks keep positions and velocities) (Aarseth, Henon & Wielen 1974:
 *                    radius from the mass fraction, speed by rejection from
 *                    q^2 (1 - q^2)^(7/2), isotropic directions), density `density`.
 *   GBH_IC_CLUSTERS  `clusters` isotropic Gaussians: centres uniform in
 *                    [-scale, scale]^3, sigma log-uniform in [sigma_lo, sigma_hi],
 *                    each body in a uniformly chosen cluster; masses from the
 *                    power law dN/dm ~ m^-2 on [lo[6], hi[6]]; density `density`.
 * DISK and PLUMMER add `center` and `velocity` to every body. */
#define GBH_IC_BOX 0u
#define GBH_IC_DISK 1u
#define GBH_IC_PLUMMER 2u
#define GBH_IC_CLUSTERS 3u
#define GBH_IC_ORBITAL 0x1u
#define GBH_IC_CCW 0x2u
typedef struct gbh_ic_params {
    uint32_t kind;           /* GBH_IC_* */
    uint32_t flags;          /* DISK: GBH_IC_ORBITAL | GBH_IC_CCW */
    float lo[8];             /* ranges: x, y, z, vx, vy, vz, mass, density (see the kinds) */
    float hi[8];
    float center[3];
    float velocity[3];
    float scale;             /* PLUMMER: scale radius; CLUSTERS: half side of the centres' cube */
    float total_mass;        /* PLUMMER */
    float density;           /* PLUMMER, CLUSTERS */
    float G;                 /* PLUMMER, DISK: gravitational constant of the velocities */
    float phi;               /* DISK: tilt of the normal about x */
    float center_mass;       /* DISK */
    float center_density;    /* DISK (also the exponent of the enclosed-mass estimate, as the reference) */
    float adherence;         /* DISK: adherenceToPlane */
    float orbital_factor;    /* DISK */
    uint32_t clusters;       /* CLUSTERS */
    float sigma_lo, sigma_hi;/* CLUSTERS */
} gbh_ic_params; /* 144 bytes */
int gbh_generate_bodies(gbh_ctx* ctx, const gbh_ic_params* params, uint64_t seed, uint32_t count, uint32_t offset);

/* ---- headless consumers of the tree: level-of-detail node selection ---------
 * The reference's render shaders read the internal nodes directly: the
 * hierarchical node glow (nodeglow.vert:46-150) draws a soft splat at the
 * centre of mass of every node whose projected size falls inside a band, and
 * the region boxes (regions.vert:19-45) draw the AABB of every node inside a
 * depth range.  These entry points run the same per-node arithmetic as CUDA
 * kernels over the tree of the last step (the bodies of the current state for
 * `relative_to`) and append one record per selected node to a DEVICE buffer
 * the caller owns; nothing is drawn.  Records come in no particular order
 * (sort by `node` for a stable one).  `*count` receives the number of nodes
 * selected; when it exceeds `capacity`, only `capacity` records are written.
 * They return after the selection has finished.
 * Differences from the shaders, both reference defects: only the live internal
 * nodes [0, n - 1) are visited (the shaders visit every slot up to N - 1 or n,
 * including stale ones), and tan(fov_y / 2) is computed once on the host. */
typedef struct gbh_view {
    float model_view[16];     /* uModelView, column-major (GLSL mat4 memory order) */
    float proj[16];           /* uProj, column-major */
    float fov_y;              /* uFovY, radians */
    float aspect;             /* uAspect */
    float camera_scale;       /* cameraScale: camera units per length unit */
    uint32_t relative_to;     /* uRelativeTo: body index, 0xFFFFFFFF = absolute */
    float glow_theta_ndc;     /* uNodeGlowThetaNdc = 2 * nodeGlowThetaPx / framebuffer height */
    float glow_activate_dist; /* uNodeGlowActivateDist (view-space depth) */
    int32_t glow_max_depth;   /* uNodeGlowMaxDepth (node height above its furthest leaf) */
    float glow_intensity;     /* uNodeGlowIntensity */
    int32_t region_min_depth; /* uMinMaxDepth.x */
    int32_t region_max_depth; /* uMinMaxDepth.y */
    uint32_t pad[2];
} gbh_view; /* 176 bytes */

/* per selected node: the outputs of nodeglow.vert for its instance (the four
 * corner vertices add +-1.5 * ndc_scale * center_clip.w to center_clip.xy) */
typedef struct gbh_glow_splat {
    float center_clip[4];     /* uProj * uModelView * com */
    float center_view[3];     /* vCenterView */
    float intensity;          /* vIntensity (after the Reinhard map) */
    float color[3];           /* vColor: the node's avgColor.rgb */
    uint32_t node;            /* internal node index (global id N + node) */
    float ndc_scale[2];       /* vNdcScaleX, vNdcScaleY */
    uint32_t depth;           /* nodeDepth */
    uint32_t pad;
} gbh_glow_splat; /* 64 bytes */

/* per selected node: the box regions.vert scales its unit cube to (camera
 * units, relative to `relative_to`), and the depth it passes on */
typedef struct gbh_region {
    float center[3];
    float size[3];
    uint32_t node;            /* internal node index */
    uint32_t depth;           /* nodeDepth */
} gbh_region; /* 32 bytes */

int gbh_select_glow_nodes(gbh_ctx* ctx, const gbh_view* view, gbh_glow_splat* out_device, uint32_t capacity,
                          uint32_t* count);
int gbh_select_regions(gbh_ctx* ctx, const gbh_view* view, gbh_region* out_device, uint32_t capacity,
                       uint32_t* count);

/* ---- library info ---------------------------------------------------------- */
int gbh_abi_version(void);
const char* gbh_last_error(gbh_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* GBH_H */
