// gbh_common.cuh — device-side types and helpers shared by the step kernels.
//
// Arithmetic convention: the library is compiled with --fmad=false, so every
// FP32 expression below rounds once per operation in source order, matching
// the reference GLSL evaluated as IEEE FP32 (SH/compute/*, SH/common/common.glsl).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbh.h"

#define GBH_NONE 0xFFFFFFFFu
#define GBH_WARP 32
#define GBH_WALK_STACK 192     // per-warp walk stack entries (tree height + 1 needed)
#ifndef GBH_GROUP_MAX
#define GBH_GROUP_MAX 96       // bodies per group of the group walk (one warp, three per lane)
#endif
// words per group of the group walks' start lists: a count and up to 63 nodes
// (deeper groups start from the root)
#define GBH_PATH_WORDS 64
#define GBH_MAX_TREE_HEIGHT_REF 64  // the reference fills 64 levels (GPU.java:41)

// onesweep radix sort geometry (8-bit digits, 8 passes over the 63-bit key)
#define SORT_BITS 8
#define SORT_RADIX 256
#define SORT_PASSES 8
#define SORT_THREADS 256
#define SORT_ITEMS 16
#define SORT_TILE (SORT_THREADS * SORT_ITEMS)

// fused compaction / bounds / encode geometry
#define PREP_THREADS 256
#define PREP_ITEMS 8
#define PREP_TILE (PREP_THREADS * PREP_ITEMS)

// Compact node record read by the walk: 32 bytes = one DRAM sector.
struct __align__(16) WalkRec {
    float4 cm;        // centre of mass xyz, mass (a leaf: the body's posMass)
    float half_side;  // getLongestSide(node), bh_force.comp:14-20 (0 for a leaf)
    uint32_t id;      // global node id: < N leaf (sorted slot), >= N internal
    uint32_t count;   // bodies contained
    uint32_t pad;
};

// The records of both children of one internal node, written by the fill and
// read by the walk with one 64-byte load when the node is opened.
struct __align__(16) ChildPair {
    WalkRec a;  // childA
    WalkRec b;  // childB
};

// Device-resident state of one step (never read by the reference-facing
// buffers; these are the library's own counters and scratch scalars).
struct DevState {
    uint32_t n_old;        // live count entering the step
    uint32_t n_new;        // live count after compaction
    uint32_t just_died;
    uint32_t error_word;   // GBH_DEVERR_* (sticky)
    uint32_t merge_conflicts;
    uint32_t merged;
    uint32_t oob;
    uint32_t tree_height;
    uint32_t max_stack;
    uint32_t merge_tasks;
    uint32_t sort_tiles[SORT_PASSES];  // onesweep tile tickets
    uint32_t num_groups;               // body groups of the group walk
    uint32_t group_next;               // the next group a warp of the group walk takes (ticket)
    uint32_t frontier_saturated;       // group walks that accepted instead of opening (full stack)
    uint32_t fill_frontier;            // nodes handed from the tiled fill to the top-tree fill
    uint32_t sorted_valid;             // sorted_pm holds the current positions in index order
    uint32_t view_count;               // records of the last node selection (gbh_select_*)
    uint32_t shard_lo, shard_hi;       // sorted slots a sharded walk updated [lo, hi)
    unsigned long long interactions;
    unsigned long long opened;
    unsigned long long mac_evals;
};

// Merge queue with the reference layout (MergeTasks: head, tail, uvec2[]),
// common.glsl:117.
struct MergeQueue {
    uint32_t head;
    uint32_t tail;
    uint2 pairs[1];  // flexible
};

// Pointers handed to every kernel (by value).
struct StepBuffers {
    gbh_body* bodies_in;
    gbh_body* bodies_out;
    uint64_t* keys_in;    // MortonIn at step start
    uint32_t* idx_in;     // IndexIn at step start
    uint64_t* keys_out;   // the other buffer
    uint32_t* idx_out;
    gbh_node* leaf;
    gbh_node* internal;
    ChildPair* pairs;     // per internal node
    WalkRec* root_rec;    // record of the root (internal node 0)
    float4* leaf_pm;      // sorted-order copy of posMass (leaf comMass)
    float4* sorted_pm;    // posMass after the walk's update, by the walk's sorted slot: the next
                          // step's compaction and encode read it in order instead of gathering
    float* leaf_rad;      // sorted-order radius(body)
    gbh_sim_values* sim;
    DevState* st;
    const gbh_step_params* params;
    MergeQueue* mq;
    unsigned long long* mkeys;  // merge ordering keys (slot << 32 | seq)
    uint32_t* mslots;           // per merge task: the sorted slot of its second body
    uint32_t* locks;
    uint32_t* conflicts;
    float4* accel;
    float* accel_mag;     // |acceleration| of the last walk, by body id (learned MAC feature)
    uint32_t* node_lo;    // first sorted slot of each internal node's leaf range
    // compact topology written by the build and read by the fill, which then
    // writes whole 80-byte nodes (no partial-sector writes to the node arrays)
    uint2* topo_kids;      // (childA, childB) per internal node
    uint32_t* topo_cnt;    // bodiesContained per internal node
    uint32_t* fill_ready;  // arrival counters of the fill's climb across tiles
    uint32_t* parent_int;  // parentId per internal node
    uint32_t* parent_leaf; // parentId per leaf
    uint2* groups;        // (first slot, body count) of the group walk's body groups
    uint32_t* group_node; // per group: the node whose subtree it is (global id)
    // per group (below group_path_cap): where its walk starts, word 0 the
    // count (0: from the root), then the group's own node and the siblings of
    // its ancestors (k_group_paths)
    uint32_t* group_path;
    uint32_t group_path_cap;
    uint2* fill_frontier; // (node, bodies) handed from the tiled fill to the top-tree fill
    uint32_t fill_frontier_cap;
    // precision form (GBH_PRECISION_COMPENSATED); null until first used
    const double* pos64_in;  // [N][4] FP64 positions (x, y, z, 0) by body id, current state
    double* pos64_out;       // the next state's
    float4* leaf_lo;         // by sorted slot: FP32 residual x64 - (float)x64 of the leaf's body
    float* potential;        // walk potential by body id (GBH_FLAG_STORE_POTENTIAL)
    uint32_t prec;           // 1: this step runs the precision form
    uint32_t merge;          // 1: this step emits merge tasks (mode GBH_MODE_MERGE)
    // compaction scratch
    uint32_t* tile_dead;
    float* tile_aabb;
    // sort scratch
    uint32_t* hist;         // [SORT_PASSES][SORT_RADIX]
    uint32_t* bucket_base;  // [SORT_PASSES][SORT_RADIX]
    uint32_t* lookback;     // [SORT_PASSES][sort_tiles_cap][SORT_RADIX]
    uint32_t N;
    uint32_t sort_tiles_cap;
    uint32_t prep_tiles_cap;
    uint32_t num_sms;  // multiprocessors of the context's device (grid sizes of the persistent kernels)
    // sharded walk: this rank's share of the live bodies (world 1: all)
    uint32_t shard_rank, shard_world;
};

// The walk's share of rank r of W: sorted slots [n r / W, n (r + 1) / W).  The
// plain walk updates exactly these slots; the group walks walk the groups
// whose first slot lies in them.
__device__ __forceinline__ void shard_slots(const StepBuffers& b, uint32_t n, uint32_t& lo, uint32_t& hi) {
    lo = (uint32_t)((uint64_t)n * b.shard_rank / b.shard_world);
    hi = (uint32_t)((uint64_t)n * (b.shard_rank + 1) / b.shard_world);
}

// ---- GLSL built-in semantics (GLSL 4.30 §8.3) -------------------------------
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

__device__ __forceinline__ void set_error(DevState* st, uint32_t bit) { atomicOr(&st->error_word, bit); }

// expandBits21 / morton3D64, bh_morton.comp:6-21
__device__ __forceinline__ uint64_t expand_bits21(uint32_t v) {
    uint64_t x = (uint64_t)v & 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__device__ __forceinline__ bool finite3(float x, float y, float z) {
    return !(isnan(x) || isnan(y) || isnan(z) || isinf(x) || isinf(y) || isinf(z));
}

// mortonEncodeKernel body, bh_morton.comp:238-262
__device__ __forceinline__ uint64_t morton_encode(float px, float py, float pz, const float* mn, const float* mx) {
    float p[3] = {px, py, pz};
    uint32_t q[3];
    const bool empty = mn[0] > mx[0];
    const bool centre = !finite3(px, py, pz) || empty;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float pos = centre ? 0.5f * (mn[k] + mx[k]) : gclamp(p[k], mn[k], mx[k]);
        float ext = gmax(mx[k] - mn[k], 1e-9f);
        float nrm = (pos - mn[k]) / ext;
        float f = gclamp(floorf(nrm * 2097151.0f), 0.0f, 2097151.0f);
        q[k] = (uint32_t)floorf(f);
    }
    return (expand_bits21(q[0]) << 2) | (expand_bits21(q[1]) << 1) | expand_bits21(q[2]);
}

// The same quantisation from an FP64 position (the precision form): the
// normalisation (x - min) / extent runs in FP64 about the FP32 box.
__device__ __forceinline__ uint64_t morton_encode64(const double* p64, const float* mn, const float* mx) {
    uint32_t q[3];
    const bool empty = mn[0] > mx[0];
    const bool centre = empty || !(isfinite(p64[0]) && isfinite(p64[1]) && isfinite(p64[2]));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double lo = mn[k], hi = mx[k];
        const double pos = centre ? 0.5 * (lo + hi) : fmin(fmax(p64[k], lo), hi);
        const double ext = fmax(hi - lo, 1e-9);
        const double f = fmin(fmax(floor((pos - lo) / ext * 2097151.0), 0.0), 2097151.0);
        q[k] = (uint32_t)f;
    }
    return (expand_bits21(q[0]) << 2) | (expand_bits21(q[1]) << 1) | expand_bits21(q[2]);
}

// radius(Body), common.glsl:228-230
__device__ __forceinline__ float body_radius(float body_len_const, float m, float rho) {
    return body_len_const * powf(m / rho, 1.0f / 3.0f);
}

// Body access as two 16-byte vectors (bodies are 32 bytes, 16-byte aligned).
__device__ __forceinline__ float4 ld_pos_mass(const gbh_body* b, uint32_t i) {
    return reinterpret_cast<const float4*>(b)[2 * (size_t)i];
}
__device__ __forceinline__ float4 ld_vel_density(const gbh_body* b, uint32_t i) {
    return reinterpret_cast<const float4*>(b)[2 * (size_t)i + 1];
}
__device__ __forceinline__ void st_body(gbh_body* b, uint32_t i, float4 pm, float4 vd) {
    float4* p = reinterpret_cast<float4*>(b) + 2 * (size_t)i;
    p[0] = pm;
    p[1] = vd;
}

// device-scope acquire-release atomic add (orders this thread's earlier writes
// before the add and the sibling's released writes before later reads)
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Symplectic update and static bounds of one body after its walk
// (bh_force.comp:117-141); writes the output body buffer.
__device__ __forceinline__ void walk_update(const StepBuffers& b, const gbh_step_params* P, const gbh_sim_values* sim,
                                            uint32_t g, uint32_t bi, float4 pm, float4 vd, float ax, float ay,
                                            float az) {
    const float dt = P->dt;
    const float nvx = vd.x + ax * dt, nvy = vd.y + ay * dt, nvz = vd.z + az * dt;
    float npx = pm.x + nvx * dt, npy = pm.y + nvy * dt, npz = pm.z + nvz * dt;
    if (P->static_or_dynamic == GBH_BOUNDS_STATIC) {
        const float* mn = sim->bounds_min;
        const float* mx = sim->bounds_max;
        if (P->wrap_around) {
            float x, y;
            x = npx - mn[0]; y = mx[0] - mn[0]; npx = (x - y * floorf(x / y)) + mn[0];
            x = npy - mn[1]; y = mx[1] - mn[1]; npy = (x - y * floorf(x / y)) + mn[1];
            x = npz - mn[2]; y = mx[2] - mn[2]; npz = (x - y * floorf(x / y)) + mn[2];
        } else if (pm.x < mn[0] || pm.x > mx[0] || pm.y < mn[1] || pm.y > mx[1] || pm.z < mn[2] || pm.z > mx[2]) {
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            st_body(b.bodies_out, bi, z, z);
            b.sorted_pm[g] = z;
            atomicAdd(&b.sim->out_of_bounds, 1u);
            atomicAdd(&b.st->oob, 1u);
            return;
        }
    }
    st_body(b.bodies_out, bi, make_float4(npx, npy, npz, pm.w), make_float4(nvx, nvy, nvz, vd.w));
    b.sorted_pm[g] = make_float4(npx, npy, npz, pm.w);
}

// The update of the precision form: the kick in FP32 as above, the drift in
// FP64 from the FP64 position (pos64_in -> pos64_out); the body buffer gets
// the FP32 rounding of the new position.  Static bounds as walk_update, the
// wrap in FP64.
__device__ __forceinline__ void walk_update_fp64(const StepBuffers& b, const gbh_step_params* P,
                                                 const gbh_sim_values* sim, uint32_t g, uint32_t bi, float4 pm,
                                                 float4 vd, float ax, float ay, float az) {
    const float dt = P->dt;
    const float nvx = vd.x + ax * dt, nvy = vd.y + ay * dt, nvz = vd.z + az * dt;
    const double2 xy = reinterpret_cast<const double2*>(b.pos64_in)[2 * (size_t)bi];
    const double z0 = b.pos64_in[4 * (size_t)bi + 2];
    double px = xy.x + (double)nvx * (double)dt;
    double py = xy.y + (double)nvy * (double)dt;
    double pz = z0 + (double)nvz * (double)dt;
    if (P->static_or_dynamic == GBH_BOUNDS_STATIC) {
        const float* mn = sim->bounds_min;
        const float* mx = sim->bounds_max;
        if (P->wrap_around) {
            double x, y;
            x = px - mn[0]; y = (double)mx[0] - mn[0]; px = (x - y * floor(x / y)) + mn[0];
            x = py - mn[1]; y = (double)mx[1] - mn[1]; py = (x - y * floor(x / y)) + mn[1];
            x = pz - mn[2]; y = (double)mx[2] - mn[2]; pz = (x - y * floor(x / y)) + mn[2];
        } else if (pm.x < mn[0] || pm.x > mx[0] || pm.y < mn[1] || pm.y > mx[1] || pm.z < mn[2] || pm.z > mx[2]) {
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            st_body(b.bodies_out, bi, z, z);
            reinterpret_cast<double2*>(b.pos64_out)[2 * (size_t)bi] = make_double2(0.0, 0.0);
            reinterpret_cast<double2*>(b.pos64_out)[2 * (size_t)bi + 1] = make_double2(0.0, 0.0);
            b.sorted_pm[g] = z;
            atomicAdd(&b.sim->out_of_bounds, 1u);
            atomicAdd(&b.st->oob, 1u);
            return;
        }
    }
    reinterpret_cast<double2*>(b.pos64_out)[2 * (size_t)bi] = make_double2(px, py);
    reinterpret_cast<double2*>(b.pos64_out)[2 * (size_t)bi + 1] = make_double2(pz, 0.0);
    st_body(b.bodies_out, bi, make_float4((float)px, (float)py, (float)pz, pm.w), make_float4(nvx, nvy, nvz, vd.w));
    b.sorted_pm[g] = make_float4((float)px, (float)py, (float)pz, pm.w);
}

// Kahan-compensated accumulation (sum, c): sum + (x - c), c the lost low part
__device__ __forceinline__ void kahan_add(float& sum, float& c, float x) {
    const float y = x - c;
    const float t = sum + y;
    c = (t - sum) - y;
    sum = t;
}

// ---- launchers (host), one translation unit each -----------------------------
void launch_reset(const StepBuffers& b, cudaStream_t s);
void launch_prepare(const StepBuffers& b, cudaStream_t s);
void launch_sort(const StepBuffers& b, cudaStream_t s);
// histograms for launch_sort when the keys come from elsewhere than the encode
// pass (hist must be zero; also sets st->n_new = n)
void launch_sort_hist(const uint64_t* keys, uint32_t n, uint32_t* hist, DevState* st, uint32_t num_sms,
                      cudaStream_t s);
void launch_generate_bodies(gbh_body* bodies, uint32_t count, uint32_t offset, const gbh_ic_params& p, uint64_t seed,
                            cudaStream_t s);
void launch_build(const StepBuffers& b, cudaStream_t s);
void launch_group_paths(const StepBuffers& b, cudaStream_t s);
void launch_fill(const StepBuffers& b, cudaStream_t s);
void launch_build_nodes(const StepBuffers& b, cudaStream_t s);
void launch_walk_plain(const StepBuffers& b, cudaStream_t s);
void launch_init_pos64(const gbh_body* bodies, double* pos64, uint32_t N, cudaStream_t s);
void launch_round_pos64(gbh_body* bodies, const double* pos64, uint32_t offset, uint32_t count, cudaStream_t s);
void launch_direct_sum64(const double* pos64, const gbh_body* bodies, uint32_t nb, const uint32_t* sample,
                         uint32_t count, double G, double soft, double* partial, double* out, uint32_t chunks,
                         cudaStream_t s);
void launch_diagnostics(const gbh_body* bodies, uint32_t nb, const double* pos64, const float* potential,
                        double* partial, uint32_t blocks, double* out, cudaStream_t s);
void launch_merge(const StepBuffers& b, cudaStream_t s);
// sharded walk: the updated slot range into st->shard_lo/hi (after the walk),
// and the copies of updated bodies out of and into the output body buffer
void launch_shard_range(const StepBuffers& b, bool groups, cudaStream_t s);
void launch_shard_pack(const StepBuffers& b, uint32_t lo, uint32_t count, gbh_body* out, cudaStream_t s);
void launch_shard_unpack(const StepBuffers& b, uint32_t lo, uint32_t count, const gbh_body* in, cudaStream_t s);
void launch_shard_add_oob(const StepBuffers& b, uint32_t oob, cudaStream_t s);
void launch_init_index(uint32_t* idx, uint32_t N, gbh_sim_values* sim, const gbh_units* units_dev, cudaStream_t s);
