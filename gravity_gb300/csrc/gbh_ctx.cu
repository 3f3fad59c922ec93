// gbh_ctx.cu — host side of the C ABI (include/gbh.h): context, device arena,
// stage sequencing, CUDA-graph capture of the whole step, read-back.
//
// Replaces the reference's host orchestration: BarnesHut.step/init
// (src/main/java/com/grumbo/simulation/BarnesHut.java:99-173), the GPU object
// registry and buffer swaps (src/main/java/com/grumbo/gpu/GPU.java:172-358,
// 1060-1196).  Where the reference issues ~140 dispatches with a full memory
// barrier after each, one step here is one CUDA-graph launch of ~20 kernels.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gbh_common.cuh"
#include "gbh_ctx.h"

static thread_local std::string g_create_error;

// ---------------------------------------------------------------------------
// error helpers

static int fail(gbh_ctx* c, int code, const std::string& msg) {
    if (c)
        c->last_error = msg;
    else
        g_create_error = msg;
    return code;
}

#define CUDA_TRY(ctx, call)                                                                          \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return fail((ctx), GBH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
    } while (0)

// ---------------------------------------------------------------------------
// arena

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct ArenaPlan {
    size_t total = 0;
    size_t add(size_t bytes) {
        size_t off = total;
        total = align_up(total + bytes, 256);
        return off;
    }
};

StepBuffers ctx_buffers(const gbh_ctx* c) {
    StepBuffers b;
    b.bodies_in = c->bodies[c->bin];
    b.bodies_out = c->bodies[1 - c->bin];
    b.keys_in = c->keys[c->iin];
    b.idx_in = c->idx[c->iin];
    b.keys_out = c->keys[1 - c->iin];
    b.idx_out = c->idx[1 - c->iin];
    b.leaf = c->leaf;
    b.internal = c->internal;
    b.pairs = c->pairs;
    b.root_rec = c->root_rec;
    b.leaf_pm = c->leaf_pm;
    b.leaf_rad = c->leaf_rad;
    b.sorted_pm = c->sorted_pm;
    b.sim = c->sim;
    b.st = c->st;
    b.params = c->params_dev;
    b.mq = c->mq;
    b.mkeys = c->mkeys;
    b.mslots = c->mslots;
    b.locks = c->locks;
    b.conflicts = c->conflicts;
    b.accel = c->accel;
    b.accel_mag = c->accel_mag;
    b.node_lo = c->node_lo;
    b.topo_kids = c->topo_kids;
    b.topo_cnt = c->topo_cnt;
    b.fill_ready = c->fill_ready;
    b.parent_int = c->parent_int;
    b.parent_leaf = c->parent_leaf;
    b.groups = c->groups;
    b.group_node = c->group_node;
    b.group_path = c->group_path;
    b.group_path_cap = c->group_path_cap;
    // the fill's frontier lives in the sort's spare key buffer (free once the
    // sorted keys are back in keys_in, until the next step's encode)
    b.fill_frontier = reinterpret_cast<uint2*>(c->keys[1 - c->iin]);
    b.fill_frontier_cap = c->N;
    b.pos64_in = c->pos64[c->bin];
    b.pos64_out = c->pos64[1 - c->bin];
    b.leaf_lo = c->leaf_lo;
    b.potential = c->potential;
    b.prec = (c->params_valid && c->params_host.precision_mode == GBH_PRECISION_COMPENSATED && c->pos64[0]) ? 1u : 0u;
    b.merge = (c->params_valid && c->params_host.merging_collision_or_neither == GBH_MODE_MERGE) ? 1u : 0u;
    b.tile_dead = c->tile_dead;
    b.tile_aabb = c->tile_aabb;
    b.hist = c->hist;
    b.bucket_base = c->bucket_base;
    b.lookback = c->lookback;
    b.N = c->N;
    b.sort_tiles_cap = c->sort_tiles_cap;
    b.prep_tiles_cap = c->prep_tiles_cap;
    b.num_sms = c->num_sms;
    b.shard_rank = c->shard_rank;
    b.shard_world = c->shard_world;
    return b;
}

static int check_launch(gbh_ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, GBH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return GBH_OK;
}

// ---------------------------------------------------------------------------
// stage enqueue (shared by eager stage calls, profiling and graph capture)

int enqueue_reset(gbh_ctx* c) {
    launch_reset(ctx_buffers(c), c->stream);
    return check_launch(c, "reset");
}

int enqueue_prepare(gbh_ctx* c) {
    launch_prepare(ctx_buffers(c), c->stream);
    c->iin = 1 - c->iin;  // GPU.swapMortonAndIndexBuffers after the partition
    return check_launch(c, "prepare");
}

int enqueue_sort(gbh_ctx* c) {
    CUDA_TRY(c, cudaMemsetAsync(c->lookback, 0, c->lookback_bytes, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->st->sort_tiles, 0, sizeof(c->st->sort_tiles), c->stream));
    launch_sort(ctx_buffers(c), c->stream);
    return check_launch(c, "sort");
}

int enqueue_build(gbh_ctx* c) {
    launch_build(ctx_buffers(c), c->stream);
    // the group walks' start lists belong to the tree: built with it when a
    // group walk is selected (otherwise the group walk builds them itself)
    c->paths_current = c->mac_mode != GBH_MAC_PLAIN;
    if (c->paths_current) launch_group_paths(ctx_buffers(c), c->stream);
    return check_launch(c, "build");
}

int enqueue_fill(gbh_ctx* c) {
    launch_fill(ctx_buffers(c), c->stream);
    return check_launch(c, "fill");
}

int enqueue_walk(gbh_ctx* c) {
    if (c->mac_mode == GBH_MAC_PLAIN) {
        launch_walk_plain(ctx_buffers(c), c->stream);
    } else {
        int rc = enqueue_walk_learned(c);
        if (rc) return rc;
    }
    return check_launch(c, "walk");
}

int enqueue_merge(gbh_ctx* c) {
    launch_merge(ctx_buffers(c), c->stream);
    return check_launch(c, "merge");
}

int enqueue_swap(gbh_ctx* c) {
    c->bin = 1 - c->bin;  // GPU.swapBodyBuffers
    return GBH_OK;
}

typedef int (*stage_fn)(gbh_ctx*);
static const stage_fn k_stages[GBH_NUM_STAGES] = {enqueue_reset, enqueue_prepare, enqueue_sort, enqueue_build,
                                                  enqueue_fill,  enqueue_walk,    enqueue_merge, enqueue_swap};

static int enqueue_step(gbh_ctx* c) {
    for (int s = 0; s < GBH_NUM_STAGES; ++s) {
        int rc = k_stages[s](c);
        if (rc) return rc;
    }
    return GBH_OK;
}

// FP64 positions (two, following the body buffers), leaf residuals and the
// potential: 84 bytes per body, allocated when first needed.  Captured graphs
// hold the old (null) pointers, so they are dropped.
static int ensure_precision_buffers(gbh_ctx* c) {
    if (c->pos64[0]) return GBH_OK;
    const size_t n = c->N;
    CUDA_TRY(c, cudaMalloc(&c->pos64[0], n * 32));
    CUDA_TRY(c, cudaMalloc(&c->pos64[1], n * 32));
    CUDA_TRY(c, cudaMalloc(&c->leaf_lo, n * 16));
    CUDA_TRY(c, cudaMalloc(&c->potential, n * 4));
    CUDA_TRY(c, cudaMemsetAsync(c->potential, 0, n * 4, c->stream));
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    c->pos64_valid = false;
    return GBH_OK;
}

// The next compaction gathers the positions through the index instead of
// reading the last walk's in-order copy (after any eager stage call, upload or
// write that the step graph does not see).
static int invalidate_sorted(gbh_ctx* c) {
    CUDA_TRY(c, cudaMemsetAsync(&c->st->sorted_valid, 0, 4, c->stream));
    return GBH_OK;
}

// Before a precision-form step: FP64 positions from the body buffer when they
// are not current (first such step, after an upload or an FP32 step).
static int prepare_precision(gbh_ctx* c) {
    if (c->params_host.precision_mode != GBH_PRECISION_COMPENSATED || c->pos64_valid) return GBH_OK;
    launch_init_pos64(c->bodies[c->bin], c->pos64[c->bin], c->N, c->stream);
    c->pos64_valid = true;
    return check_launch(c, "init fp64 positions");
}

// After the state advanced (swap): the FP64 positions are current only after
// a precision-form walk.
static void after_swap(gbh_ctx* c, bool precision_walk) {
    c->pos64_valid = precision_walk && c->pos64[0] != nullptr;
    ++c->state_epoch;
}

static int upload_params(gbh_ctx* c, const gbh_step_params* p) {
    if (!p) return fail(c, GBH_ERR_INVALID, "null step params");
    if (p->merging_collision_or_neither > 2 || p->static_or_dynamic > 1 || p->mac_mode > 2 || p->precision_mode > 1)
        return fail(c, GBH_ERR_INVALID, "step params: enum out of range");
    if ((p->flags & GBH_FLAG_STORE_ACCEL) && !c->accel) return fail(c, GBH_ERR_INVALID, "accel buffer missing");
    if (p->mac_mode == GBH_MAC_LEARNED && !c->mac_ready)
        return fail(c, GBH_ERR_STATE, "learned MAC selected but no weights were set");
    if (p->mac_mode != GBH_MAC_PLAIN && p->merging_collision_or_neither == GBH_MODE_COLLISION)
        return fail(c, GBH_ERR_UNSUPPORTED, "group and learned acceptance criteria run gravity and merges (no collisions)");
    if (p->precision_mode == GBH_PRECISION_COMPENSATED && p->merging_collision_or_neither != GBH_MODE_NEITHER)
        return fail(c, GBH_ERR_UNSUPPORTED, "the precision form runs gravity only (no merges or collisions)");
    if (p->precision_mode == GBH_PRECISION_COMPENSATED || (p->flags & GBH_FLAG_STORE_POTENTIAL)) {
        int rc = ensure_precision_buffers(c);
        if (rc) return rc;
    }
    // pageable source: the copy is staged before cudaMemcpyAsync returns
    if (!c->params_valid || memcmp(&c->params_host, p, sizeof(*p)) != 0) {
        CUDA_TRY(c, cudaMemcpyAsync(c->params_dev, p, sizeof(*p), cudaMemcpyHostToDevice, c->stream));
        c->params_host = *p;
        c->params_valid = true;
    }
    c->mac_mode = p->mac_mode;
    return GBH_OK;
}

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

int gbh_abi_version(void) { return GBH_ABI_VERSION; }

const char* gbh_last_error(gbh_ctx* c) { return c ? c->last_error.c_str() : g_create_error.c_str(); }

int gbh_create(gbh_ctx** out, uint32_t n, const float bounds[6], const gbh_units* units, int device) {
    if (!out) return fail(nullptr, GBH_ERR_INVALID, "out is null");
    *out = nullptr;
    if (!bounds || !units) return fail(nullptr, GBH_ERR_INVALID, "bounds/units is null");
    if (n == 0 || n > (1u << 30)) return fail(nullptr, GBH_ERR_INVALID, "initial_num_bodies must be in [1, 2^30]");
    if (units->density == 0.0f || units->len == 0.0f)
        return fail(nullptr, GBH_ERR_INVALID, "units: density and len must be non-zero");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(nullptr, GBH_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(nullptr, GBH_ERR_INVALID, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, GBH_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));

    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess || sms <= 0)
        return fail(nullptr, GBH_ERR_CUDA, std::string("multiprocessor count: ") + cudaGetErrorString(e));

    gbh_ctx* c = new gbh_ctx();
    c->device = device;
    c->num_sms = (uint32_t)sms;
    c->N = n;
    c->prep_tiles_cap = (n + PREP_TILE - 1) / PREP_TILE;
    c->sort_tiles_cap = (n + SORT_TILE - 1) / SORT_TILE;
    const uint32_t ni = n > 1 ? n - 1 : 1;

    ArenaPlan A;
    size_t o_bodies0 = A.add((size_t)n * 32), o_bodies1 = A.add((size_t)n * 32);
    size_t o_keys0 = A.add((size_t)n * 8), o_keys1 = A.add((size_t)n * 8);
    size_t o_idx0 = A.add((size_t)n * 4), o_idx1 = A.add((size_t)n * 4);
    size_t o_leaf = A.add((size_t)n * 80), o_int = A.add((size_t)ni * 80);
    size_t o_pairs = A.add((size_t)ni * sizeof(ChildPair)), o_root = A.add(sizeof(WalkRec));
    size_t o_lpm = A.add((size_t)n * 16), o_lrad = A.add((size_t)n * 4), o_spm = A.add((size_t)n * 16);
    size_t o_sim = A.add(sizeof(gbh_sim_values)), o_st = A.add(sizeof(DevState));
    size_t o_par = A.add(sizeof(gbh_step_params));
    size_t o_mq = A.add(8 + (size_t)n * 8), o_mkeys = A.add((size_t)n * 8), o_mslots = A.add((size_t)n * 4);
    size_t o_locks = A.add((size_t)n * 4), o_conf = A.add((size_t)n * 4);
    size_t o_accel = A.add((size_t)n * 16), o_amag = A.add((size_t)n * 4);
    size_t o_nlo = A.add((size_t)ni * 4), o_groups = A.add((size_t)n * 8), o_gnode = A.add((size_t)n * 4);
    // start lists for one group per 16 bodies (groups hold up to 96, about 60
    // on average; the groups past the capacity start from the root)
    c->group_path_cap = n / 16 + 64;
    size_t o_gpath = A.add((size_t)c->group_path_cap * GBH_PATH_WORDS * 4);
    size_t o_tkids = A.add((size_t)ni * 8), o_tcnt = A.add((size_t)ni * 4), o_tready = A.add((size_t)ni * 4);
    size_t o_pint = A.add((size_t)ni * 4), o_pleaf = A.add((size_t)n * 4);
    size_t o_tdead = A.add((size_t)c->prep_tiles_cap * 4), o_taabb = A.add((size_t)c->prep_tiles_cap * 24);
    size_t o_hist = A.add(SORT_PASSES * SORT_RADIX * 4), o_bbase = A.add(SORT_PASSES * SORT_RADIX * 4);
    c->lookback_bytes = (size_t)SORT_PASSES * c->sort_tiles_cap * SORT_RADIX * 4;
    size_t o_lb = A.add(c->lookback_bytes);
    e = cudaMalloc(&c->arena, A.total);
    if (e != cudaSuccess) {
        delete c;
        return fail(nullptr, GBH_ERR_OOM, "cudaMalloc of " + std::to_string(A.total) + " bytes failed");
    }
    c->arena_bytes = A.total;
    char* base = (char*)c->arena;
    c->bodies[0] = (gbh_body*)(base + o_bodies0);
    c->bodies[1] = (gbh_body*)(base + o_bodies1);
    c->body_phys[0] = c->bodies[0];
    c->body_phys[1] = c->bodies[1];
    c->keys[0] = (uint64_t*)(base + o_keys0);
    c->keys[1] = (uint64_t*)(base + o_keys1);
    c->idx[0] = (uint32_t*)(base + o_idx0);
    c->idx[1] = (uint32_t*)(base + o_idx1);
    c->leaf = (gbh_node*)(base + o_leaf);
    c->internal = (gbh_node*)(base + o_int);
    c->pairs = (ChildPair*)(base + o_pairs);
    c->root_rec = (WalkRec*)(base + o_root);
    c->leaf_pm = (float4*)(base + o_lpm);
    c->leaf_rad = (float*)(base + o_lrad);
    c->sorted_pm = (float4*)(base + o_spm);
    c->sim = (gbh_sim_values*)(base + o_sim);
    c->st = (DevState*)(base + o_st);
    c->params_dev = (gbh_step_params*)(base + o_par);
    c->mq = (MergeQueue*)(base + o_mq);
    c->mkeys = (unsigned long long*)(base + o_mkeys);
    c->mslots = (uint32_t*)(base + o_mslots);
    c->locks = (uint32_t*)(base + o_locks);
    c->conflicts = (uint32_t*)(base + o_conf);
    c->accel = (float4*)(base + o_accel);
    c->accel_mag = (float*)(base + o_amag);
    c->topo_kids = (uint2*)(base + o_tkids);
    c->topo_cnt = (uint32_t*)(base + o_tcnt);
    c->fill_ready = (uint32_t*)(base + o_tready);
    c->parent_int = (uint32_t*)(base + o_pint);
    c->parent_leaf = (uint32_t*)(base + o_pleaf);
    c->node_lo = (uint32_t*)(base + o_nlo);
    c->groups = (uint2*)(base + o_groups);
    c->group_node = (uint32_t*)(base + o_gnode);
    c->group_path = (uint32_t*)(base + o_gpath);
    c->tile_dead = (uint32_t*)(base + o_tdead);
    c->tile_aabb = (float*)(base + o_taabb);
    c->hist = (uint32_t*)(base + o_hist);
    c->bucket_base = (uint32_t*)(base + o_bbase);
    c->lookback = (uint32_t*)(base + o_lb);

    sort_setup();
    group_walk_setup();
    fill_setup();
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    for (cudaEvent_t& ev : c->copy_events)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->arena, 0, A.total, c->stream);
    // SimulationValues as packed by GPU.packValues (GPU.java:1096-1143)
    gbh_sim_values sv;
    memset(&sv, 0, sizeof(sv));
    sv.num_bodies = n;
    sv.initial_num_bodies = n;
    for (int k = 0; k < 3; ++k) {
        sv.bounds_min[k] = bounds[k];
        sv.bounds_max[k] = bounds[3 + k];
    }
    sv.unit_mass = units->mass;
    sv.unit_density = units->density;
    sv.unit_len = units->len;
    sv.unit_time = units->time;
    sv.camera_scale = units->camera_scale;
    c->units = *units;
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->sim, &sv, sizeof(sv), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        std::string m = std::string("create: ") + cudaGetErrorString(e);
        gbh_destroy(c);
        return fail(nullptr, GBH_ERR_CUDA, m);
    }
    *out = c;
    return GBH_OK;
}

int gbh_destroy(gbh_ctx* c) {
    if (!c) return GBH_ERR_INVALID;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    mac_release(c);
    cudaFree(c->pos64[0]);
    cudaFree(c->pos64[1]);
    cudaFree(c->leaf_lo);
    cudaFree(c->potential);
    if (c->arena) cudaFree(c->arena);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        for (cudaEvent_t& e : c->copy_events)
            if (e) cudaEventDestroy(e);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->copy_stream2) {
        cudaStreamSynchronize(c->copy_stream2);
        cudaStreamDestroy(c->copy_stream2);
    }
    for (cudaEvent_t e : {c->ev_in_ready, c->ev_out_ready, c->ev_out_done})
        if (e) cudaEventDestroy(e);
    // the role pointers (state, output, stage_in, spare) may name any of the
    // four body buffers: free the allocations
    cudaFree(c->stage_alloc[0]);
    cudaFree(c->stage_alloc[1]);
    cudaFree(c->stage_out);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return GBH_OK;
}

int gbh_upload_bodies(gbh_ctx* c, const gbh_body* host, uint32_t count, uint32_t offset) {
    if (!c || !host) return fail(c, GBH_ERR_INVALID, "null argument");
    if ((uint64_t)offset + count > c->N) return fail(c, GBH_ERR_INVALID, "upload range exceeds initial_num_bodies");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(c->bodies[c->bin] + offset, host, (size_t)count * sizeof(gbh_body),
                                cudaMemcpyHostToDevice, c->stream));
    c->pos64_valid = false;
    ++c->state_epoch;
    int rc = invalidate_sorted(c);
    if (rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_exchange_bodies(gbh_ctx* c, gbh_body* host_out, const gbh_body* host_in, uint32_t count, uint32_t offset) {
    if (!c || !host_out || !host_in) return fail(c, GBH_ERR_INVALID, "null argument");
    if ((uint64_t)offset + count > c->N) return fail(c, GBH_ERR_INVALID, "exchange range exceeds initial_num_bodies");
    if (!count) return GBH_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    constexpr uint32_t CHUNKS = sizeof(c->copy_events) / sizeof(c->copy_events[0]);
    gbh_body* dev = c->bodies[c->bin] + offset;
    // the read-back starts once the work queued so far (the last step) is done
    CUDA_TRY(c, cudaEventRecord(c->copy_events[0], c->stream));
    CUDA_TRY(c, cudaStreamWaitEvent(c->copy_stream, c->copy_events[0], 0));
    const uint32_t per = (count + CHUNKS - 1) / CHUNKS;
    for (uint32_t k = 0, s = 0; s < count; ++k, s += per) {
        const size_t bytes = (size_t)min(per, count - s) * sizeof(gbh_body);
        // chunk k out on the copy stream, then in on the context stream:
        // the two directions overlap chunk by chunk
        CUDA_TRY(c, cudaMemcpyAsync(host_out + s, dev + s, bytes, cudaMemcpyDeviceToHost, c->copy_stream));
        CUDA_TRY(c, cudaEventRecord(c->copy_events[k], c->copy_stream));
        CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->copy_events[k], 0));
        CUDA_TRY(c, cudaMemcpyAsync(dev + s, host_in + s, bytes, cudaMemcpyHostToDevice, c->stream));
    }
    c->pos64_valid = false;
    ++c->state_epoch;
    int rc = invalidate_sorted(c);
    if (rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->copy_stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

// The two rotating body buffers, the result buffer of calls without a next
// input, the second copy stream and the events of the streamed steps,
// created on first use (three body buffers: 96 bytes per body).
static int ensure_stream_buffers(gbh_ctx* c) {
    if (c->stage_alloc[0]) return GBH_OK;
    const size_t bytes = (size_t)c->N * sizeof(gbh_body);
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->copy_stream2, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&c->ev_in_ready, &c->ev_out_ready, &c->ev_out_done})
        CUDA_TRY(c, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    CUDA_TRY(c, cudaMalloc(&c->stage_out, bytes));
    CUDA_TRY(c, cudaMalloc(&c->stage_alloc[0], bytes));
    CUDA_TRY(c, cudaMalloc(&c->stage_alloc[1], bytes));
    c->stage_in = c->body_phys[2] = c->stage_alloc[0];
    c->spare = c->body_phys[3] = c->stage_alloc[1];
    return GBH_OK;
}

int gbh_step_streamed(gbh_ctx* c, const gbh_step_params* p, const gbh_body* next_input, gbh_body* last_result) {
    if (!c) return GBH_ERR_INVALID;
    if (!c->inited) return fail(c, GBH_ERR_STATE, "gbh_step_streamed before gbh_init");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = ensure_stream_buffers(c);
    if (rc) return rc;
    const size_t bytes = (size_t)c->N * sizeof(gbh_body);
    // the last call's result, once it is there
    if (c->stream_have_result && last_result) {
        CUDA_TRY(c, cudaStreamWaitEvent(c->copy_stream2, c->ev_out_ready, 0));
        CUDA_TRY(c, cudaMemcpyAsync(last_result, c->result_buf, bytes, cudaMemcpyDeviceToHost, c->copy_stream2));
    }
    CUDA_TRY(c, cudaEventRecord(c->ev_out_done, c->copy_stream2));
    // the next input into stage_in: it held the result of the step before
    // last, whose read-back the last call finished (each call waits for its
    // copies), so only that step must have finished
    if (next_input) {
        CUDA_TRY(c, cudaStreamWaitEvent(c->copy_stream, c->ev_out_ready, 0));
        CUDA_TRY(c, cudaMemcpyAsync(c->stage_in, next_input, bytes, cudaMemcpyHostToDevice, c->copy_stream));
        CUDA_TRY(c, cudaEventRecord(c->ev_in_ready, c->copy_stream));
    }
    // this call's step on the current state (one graph launch)
    if ((rc = gbh_step_n(c, p, 1))) return rc;
    gbh_body* const result = c->bodies[c->bin];
    gbh_body* const consumed = c->bodies[1 - c->bin];
    if (next_input) {
        // rotate: the next input becomes the state, the consumed input the
        // next step's output, the result waits in the spare slot for the next
        // call's read-back, and the slot this call read back takes the next
        // input
        CUDA_TRY(c, cudaEventRecord(c->ev_out_ready, c->stream));
        CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_in_ready, 0));
        c->bodies[c->bin] = c->stage_in;
        c->bodies[1 - c->bin] = consumed;
        c->stage_in = c->spare;
        c->spare = result;
        c->result_buf = result;
        c->pos64_valid = false;
        ++c->state_epoch;
        if ((rc = invalidate_sorted(c))) return rc;
    } else {
        // the result stays the state, which the step after next overwrites:
        // the read-back takes a copy (once the last read-back has left it)
        CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_out_done, 0));
        CUDA_TRY(c, cudaMemcpyAsync(c->stage_out, result, bytes, cudaMemcpyDeviceToDevice, c->stream));
        CUDA_TRY(c, cudaEventRecord(c->ev_out_ready, c->stream));
        c->result_buf = c->stage_out;
    }
    c->stream_have_result = true;
    // the host buffers are free again; the step itself may still run
    CUDA_TRY(c, cudaStreamSynchronize(c->copy_stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->copy_stream2));
    return GBH_OK;
}

int gbh_step_streamed_finish(gbh_ctx* c, gbh_body* last_result) {
    if (!c) return GBH_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (!c->stream_have_result) return fail(c, GBH_ERR_STATE, "no streamed step has run since the last finish");
    if (last_result) {
        CUDA_TRY(c, cudaStreamWaitEvent(c->copy_stream2, c->ev_out_ready, 0));
        CUDA_TRY(c, cudaMemcpyAsync(last_result, c->result_buf, (size_t)c->N * sizeof(gbh_body),
                                    cudaMemcpyDeviceToHost, c->copy_stream2));
        CUDA_TRY(c, cudaStreamSynchronize(c->copy_stream2));
    }
    c->stream_have_result = false;
    return gbh_synchronize(c);
}

// ---- sharded step -------------------------------------------------------------

static int read_dev(gbh_ctx* c, void* host, const void* dev, size_t bytes);

int gbh_step_shard_walk(gbh_ctx* c, const gbh_step_params* p, uint32_t rank, uint32_t world, uint32_t range[2]) {
    if (!c || !p || !range) return fail(c, GBH_ERR_INVALID, "null argument");
    if (!c->inited) return fail(c, GBH_ERR_STATE, "gbh_step_shard_walk before gbh_init");
    if (c->shard_open) return fail(c, GBH_ERR_STATE, "a sharded step is already open");
    if (world == 0 || rank >= world) return fail(c, GBH_ERR_INVALID, "rank must be below world");
    if (p->precision_mode != GBH_PRECISION_FP32)
        return fail(c, GBH_ERR_UNSUPPORTED, "the sharded step runs the FP32 form");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = upload_params(c, p);
    if (rc) return rc;
    // the tree of the whole state, as every rank builds it
    if ((rc = enqueue_reset(c)) || (rc = enqueue_prepare(c)) || (rc = enqueue_sort(c)) || (rc = enqueue_build(c)) ||
        (rc = enqueue_fill(c)))
        return rc;
    // this rank's share of the walk and the slots it updated
    c->shard_rank = rank;
    c->shard_world = world;
    rc = enqueue_walk(c);
    if (!rc) {
        launch_shard_range(ctx_buffers(c), c->mac_mode != GBH_MAC_PLAIN, c->stream);
        rc = check_launch(c, "shard range");
    }
    c->shard_rank = 0;
    c->shard_world = 1;
    if (rc) return rc;
    c->shard_open = true;
    if ((rc = gbh_synchronize(c))) return rc;
    uint32_t r[2];
    CUDA_TRY(c, cudaMemcpy(r, &c->st->shard_lo, 8, cudaMemcpyDeviceToHost));
    range[0] = r[0];
    range[1] = r[1];
    return GBH_OK;
}

int gbh_shard_pack(gbh_ctx* c, uint32_t lo, uint32_t count, void* device_out) {
    if (!c || (!device_out && count)) return fail(c, GBH_ERR_INVALID, "null argument");
    if (!c->shard_open) return fail(c, GBH_ERR_STATE, "no sharded step is open");
    if ((uint64_t)lo + count > c->N) return fail(c, GBH_ERR_INVALID, "slot range exceeds initial_num_bodies");
    CUDA_TRY(c, cudaSetDevice(c->device));
    launch_shard_pack(ctx_buffers(c), lo, count, static_cast<gbh_body*>(device_out), c->stream);
    int rc = check_launch(c, "shard pack");
    if (rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_shard_unpack(gbh_ctx* c, uint32_t lo, uint32_t count, const void* device_in) {
    if (!c || (!device_in && count)) return fail(c, GBH_ERR_INVALID, "null argument");
    if (!c->shard_open) return fail(c, GBH_ERR_STATE, "no sharded step is open");
    if ((uint64_t)lo + count > c->N) return fail(c, GBH_ERR_INVALID, "slot range exceeds initial_num_bodies");
    CUDA_TRY(c, cudaSetDevice(c->device));
    launch_shard_unpack(ctx_buffers(c), lo, count, static_cast<const gbh_body*>(device_in), c->stream);
    int rc = check_launch(c, "shard unpack");
    if (rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_read_merge_tasks_full(gbh_ctx* c, uint32_t* pairs, uint64_t* keys, uint32_t* slots, uint32_t capacity,
                              uint32_t* count) {
    if (!c || !count) return GBH_ERR_INVALID;
    uint32_t ht[2];
    int rc = read_dev(c, ht, c->mq, 8);
    if (rc) return rc;
    const uint32_t m = ht[1] < c->N ? ht[1] : c->N;
    *count = m;
    const uint32_t k = m < capacity ? m : capacity;
    if (!k) return GBH_OK;
    if (pairs && (rc = read_dev(c, pairs, c->mq->pairs, (size_t)k * 8))) return rc;
    if (keys && (rc = read_dev(c, keys, c->mkeys, (size_t)k * 8))) return rc;
    if (slots && (rc = read_dev(c, slots, c->mslots, (size_t)k * 4))) return rc;
    return GBH_OK;
}

int gbh_write_merge_tasks(gbh_ctx* c, const uint32_t* pairs, const uint64_t* keys, const uint32_t* slots,
                          uint32_t count) {
    if (!c || (count && (!pairs || !keys || !slots))) return fail(c, GBH_ERR_INVALID, "null argument");
    if (count > c->N) return fail(c, GBH_ERR_INVALID, "more merge tasks than bodies");
    CUDA_TRY(c, cudaSetDevice(c->device));
    const uint32_t ht[2] = {0u, count};
    CUDA_TRY(c, cudaMemcpyAsync(c->mq, ht, 8, cudaMemcpyHostToDevice, c->stream));
    if (count) {
        CUDA_TRY(c, cudaMemcpyAsync(c->mq->pairs, pairs, (size_t)count * 8, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->mkeys, keys, (size_t)count * 8, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaMemcpyAsync(c->mslots, slots, (size_t)count * 4, cudaMemcpyHostToDevice, c->stream));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_step_shard_finish(gbh_ctx* c, uint32_t out_of_bounds_other_ranks) {
    if (!c) return GBH_ERR_INVALID;
    if (!c->shard_open) return fail(c, GBH_ERR_STATE, "no sharded step is open");
    CUDA_TRY(c, cudaSetDevice(c->device));
    launch_shard_add_oob(ctx_buffers(c), out_of_bounds_other_ranks, c->stream);
    int rc = check_launch(c, "shard out-of-bounds count");
    if (rc) return rc;
    if ((rc = enqueue_merge(c)) || (rc = enqueue_swap(c))) return rc;
    after_swap(c, false);
    c->shard_open = false;
    return gbh_synchronize(c);
}

int gbh_generate_bodies(gbh_ctx* c, const gbh_ic_params* p, uint64_t seed, uint32_t count, uint32_t offset) {
    if (!c || !p) return fail(c, GBH_ERR_INVALID, "null argument");
    if ((uint64_t)offset + count > c->N) return fail(c, GBH_ERR_INVALID, "generate range exceeds initial_num_bodies");
    if (p->kind > GBH_IC_CLUSTERS) return fail(c, GBH_ERR_INVALID, "unknown initial-condition kind");
    if (p->kind == GBH_IC_CLUSTERS && !(p->sigma_lo > 0.0f && p->sigma_hi > 0.0f && p->lo[6] > 0.0f && p->hi[6] > 0.0f))
        return fail(c, GBH_ERR_INVALID, "cluster sigmas and masses must be positive");
    if (p->kind == GBH_IC_PLUMMER && !(p->scale > 0.0f)) return fail(c, GBH_ERR_INVALID, "Plummer scale must be positive");
    CUDA_TRY(c, cudaSetDevice(c->device));
    launch_generate_bodies(c->bodies[c->bin], count, offset, *p, seed, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    // the same bookkeeping as an upload
    c->pos64_valid = false;
    ++c->state_epoch;
    int rc = invalidate_sorted(c);
    if (rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_init(gbh_ctx* c) {
    if (!c) return fail(c, GBH_ERR_INVALID, "null context");
    CUDA_TRY(c, cudaSetDevice(c->device));
    launch_init_index(c->idx[c->iin], c->N, c->sim, &c->units, c->stream);
    int rc = check_launch(c, "init");
    if (rc) return rc;
    if ((rc = invalidate_sorted(c))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->inited = true;
    return GBH_OK;
}

// which of the four body buffers a state pointer names (4: none)
static int body_slot(const gbh_ctx* c, const gbh_body* p) {
    for (int i = 0; i < 4; ++i)
        if (c->body_phys[i] && c->body_phys[i] == p) return i;
    return 4;
}

// A captured step names its buffers: the key holds the parities, the modes
// and which body buffers are the step's input and output (streamed steps
// rotate four).
static int graph_key(const gbh_ctx* c) {
    return (c->bin) | (c->iin << 1) | ((int)c->mac_mode << 2) |
           ((c->params_host.precision_mode == GBH_PRECISION_COMPENSATED) ? 16 : 0) |
           ((int)c->params_host.merging_collision_or_neither << 5) |
           ((body_slot(c, c->bodies[c->bin]) * 8 + body_slot(c, c->bodies[1 - c->bin])) << 7);
}

int gbh_step(gbh_ctx* c, const gbh_step_params* p) { return gbh_step_n(c, p, 1); }

int gbh_step_n(gbh_ctx* c, const gbh_step_params* p, uint32_t count) {
    if (!c) return fail(c, GBH_ERR_INVALID, "null context");
    if (!c->inited) return fail(c, GBH_ERR_STATE, "gbh_step before gbh_init");
    if (c->shard_open) return fail(c, GBH_ERR_STATE, "a sharded step is open: gbh_step_shard_finish first");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = upload_params(c, p);
    if (rc) return rc;
    const bool prec = c->params_host.precision_mode == GBH_PRECISION_COMPENSATED;
    for (uint32_t s = 0; s < count; ++s) {
        if ((rc = prepare_precision(c))) return rc;
        const int key = graph_key(c);
        auto it = c->graphs.find(key);
        if (it == c->graphs.end()) {
            const int bin0 = c->bin, iin0 = c->iin;
            cudaGraph_t g = nullptr;
            CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_step(c);
            cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            c->bin = bin0;
            c->iin = iin0;
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return fail(c, GBH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            cudaGraphExec_t ex = nullptr;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(c, GBH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            it = c->graphs.emplace(key, ex).first;
        }
        CUDA_TRY(c, cudaGraphLaunch(it->second, c->stream));
        // the graph's build stage ran for this mode (the key holds it): the
        // start lists are current exactly when a group walk is selected
        c->paths_current = c->mac_mode != GBH_MAC_PLAIN;
        // the step flips both the body buffers and the (morton, index) buffers
        c->bin = 1 - c->bin;
        c->iin = 1 - c->iin;
        after_swap(c, prec);
    }
    return GBH_OK;
}

int gbh_synchronize(gbh_ctx* c) {
    if (!c) return fail(c, GBH_ERR_INVALID, "null context");
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    uint32_t ew = 0;
    CUDA_TRY(c, cudaMemcpy(&ew, &c->st->error_word, 4, cudaMemcpyDeviceToHost));
    if (ew) {
        char buf[128];
        snprintf(buf, sizeof buf, "device error word 0x%x", ew);
        return fail(c, GBH_ERR_DEVICE, buf);
    }
    return GBH_OK;
}

int gbh_clear_error(gbh_ctx* c) {
    if (!c) return GBH_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemsetAsync(&c->st->error_word, 0, 4, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->last_error.clear();
    return GBH_OK;
}

// ---- read-back --------------------------------------------------------------

static int read_dev(gbh_ctx* c, void* host, const void* dev, size_t bytes) {
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

static int write_dev(gbh_ctx* c, void* dev, const void* host, size_t bytes) {
    CUDA_TRY(c, cudaSetDevice(c->device));
    CUDA_TRY(c, cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

#define RANGE_CHECK(c, host, count, offset, cap)                                                  \
    do {                                                                                          \
        if (!(c)) return GBH_ERR_INVALID;                                                         \
        if (!(host) && (count)) return fail((c), GBH_ERR_INVALID, "null host buffer");            \
        if ((uint64_t)(offset) + (count) > (cap)) return fail((c), GBH_ERR_INVALID, "range out of bounds"); \
    } while (0)

int gbh_read_bodies(gbh_ctx* c, uint32_t which, gbh_body* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    if (which > 1) return fail(c, GBH_ERR_INVALID, "which must be GBH_BODIES_IN or GBH_BODIES_OUT");
    const gbh_body* src = c->bodies[which == GBH_BODIES_IN ? c->bin : 1 - c->bin];
    return read_dev(c, host, src + offset, (size_t)count * sizeof(gbh_body));
}

int gbh_read_leaf_nodes(gbh_ctx* c, gbh_node* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    return read_dev(c, host, c->leaf + offset, (size_t)count * sizeof(gbh_node));
}

int gbh_read_internal_nodes(gbh_ctx* c, gbh_node* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N > 1 ? c->N - 1 : 1);
    return read_dev(c, host, c->internal + offset, (size_t)count * sizeof(gbh_node));
}

int gbh_read_sim_values(gbh_ctx* c, gbh_sim_values* host) {
    if (!c || !host) return GBH_ERR_INVALID;
    return read_dev(c, host, c->sim, sizeof(gbh_sim_values));
}

int gbh_read_index(gbh_ctx* c, uint32_t* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    return read_dev(c, host, c->idx[c->iin] + offset, (size_t)count * 4);
}

int gbh_read_morton(gbh_ctx* c, uint64_t* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    return read_dev(c, host, c->keys[c->iin] + offset, (size_t)count * 8);
}

int gbh_read_merge_tasks(gbh_ctx* c, uint32_t* host_pairs, uint32_t capacity, uint32_t* count) {
    if (!c || !count) return GBH_ERR_INVALID;
    uint32_t ht[2];
    int rc = read_dev(c, ht, c->mq, 8);
    if (rc) return rc;
    const uint32_t m = ht[1] < c->N ? ht[1] : c->N;
    *count = m;
    const uint32_t k = m < capacity ? m : capacity;
    if (k && host_pairs) return read_dev(c, host_pairs, c->mq->pairs, (size_t)k * 8);
    return GBH_OK;
}

int gbh_read_accel(gbh_ctx* c, float* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    return read_dev(c, host, c->accel + offset, (size_t)count * 16);
}

int gbh_read_potential(gbh_ctx* c, float* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    if (!c->potential) return fail(c, GBH_ERR_STATE, "no potential (step with GBH_FLAG_STORE_POTENTIAL first)");
    return read_dev(c, host, c->potential + offset, (size_t)count * 4);
}

int gbh_read_positions_fp64(gbh_ctx* c, double* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    if (!c->pos64[0] || !c->pos64_valid) return fail(c, GBH_ERR_STATE, "FP64 positions are not current");
    return read_dev(c, host, c->pos64[c->bin] + 4 * (size_t)offset, (size_t)count * 32);
}

int gbh_write_positions_fp64(gbh_ctx* c, const double* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    int rc = ensure_precision_buffers(c);
    if (rc) return rc;
    if (!c->pos64_valid) {
        launch_init_pos64(c->bodies[c->bin], c->pos64[c->bin], c->N, c->stream);
        if ((rc = check_launch(c, "init fp64 positions"))) return rc;
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->pos64[c->bin] + 4 * (size_t)offset, host, (size_t)count * 32,
                                cudaMemcpyHostToDevice, c->stream));
    launch_round_pos64(c->bodies[c->bin], c->pos64[c->bin], offset, count, c->stream);
    if ((rc = check_launch(c, "round fp64 positions"))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->pos64_valid = true;
    ++c->state_epoch;
    return invalidate_sorted(c);
}

int gbh_read_diagnostics(gbh_ctx* c, gbh_diagnostics* out) {
    if (!c || !out) return GBH_ERR_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const bool pot = c->potential && c->potential_epoch == c->state_epoch;
    const bool p64 = c->pos64[0] && c->pos64_valid;
    const uint32_t blocks = c->num_sms * 4;
    double* d = nullptr;
    CUDA_TRY(c, cudaMalloc(&d, (size_t)(blocks + 1) * 16 * 8));
    launch_diagnostics(c->bodies[c->bin], c->N, p64 ? c->pos64[c->bin] : nullptr, pot ? c->potential : nullptr,
                       d + 16, blocks, d, c->stream);
    double v[16] = {0};
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, d, 15 * 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(c, GBH_ERR_CUDA, std::string("diagnostics: ") + cudaGetErrorString(e));
    memset(out, 0, sizeof(*out));
    out->mass = v[0];
    for (int k = 0; k < 3; ++k) {
        out->momentum[k] = v[1 + k];
        out->centre_of_mass[k] = v[0] != 0.0 ? v[4 + k] / v[0] : 0.0;
        out->angular_momentum[k] = v[9 + k];
    }
    out->kinetic_energy = v[7];
    out->potential_energy = pot ? v[8] : 0.0;
    out->total_energy = out->kinetic_energy + out->potential_energy;
    out->live_bodies = (uint32_t)v[12];
    out->potential_valid = pot ? 1u : 0u;
    out->positions_fp64 = p64 ? 1u : 0u;
    return GBH_OK;
}

int gbh_read_stats(gbh_ctx* c, gbh_stats* s) {
    if (!c || !s) return GBH_ERR_INVALID;
    DevState st;
    int rc = read_dev(c, &st, c->st, sizeof(st));
    if (rc) return rc;
    memset(s, 0, sizeof(*s));
    s->interactions = st.interactions;
    s->nodes_opened = st.opened;
    s->mac_evaluations = st.mac_evals;
    s->alive = st.n_new;
    s->died = st.just_died;
    s->merged = st.merged;
    s->merge_tasks = st.merge_tasks;
    s->merge_conflicts = st.merge_conflicts;
    s->out_of_bounds = st.oob;
    s->tree_height = st.tree_height;
    s->max_stack = st.max_stack;
    s->error_word = st.error_word;
    s->frontier_saturated = st.frontier_saturated;
    return GBH_OK;
}

int gbh_device_ptrs(gbh_ctx* c, gbh_device_buffers* o) {
    if (!c || !o) return GBH_ERR_INVALID;
    o->bodies_in = c->bodies[c->bin];
    o->bodies_out = c->bodies[1 - c->bin];
    o->leaf_nodes = c->leaf;
    o->internal_nodes = c->internal;
    o->sim_values = c->sim;
    o->morton_in = c->keys[c->iin];
    o->index_in = c->idx[c->iin];
    o->merge_tasks = c->mq;
    return GBH_OK;
}

void* gbh_stream(gbh_ctx* c) { return c ? (void*)c->stream : nullptr; }

int gbh_write_sim_values(gbh_ctx* c, const gbh_sim_values* host) {
    if (!c || !host) return GBH_ERR_INVALID;
    int rc = write_dev(c, c->sim, host, sizeof(gbh_sim_values));
    if (rc) return rc;
    return invalidate_sorted(c);
}

int gbh_write_index(gbh_ctx* c, const uint32_t* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    int rc = write_dev(c, c->idx[c->iin] + offset, host, (size_t)count * 4);
    if (rc) return rc;
    return invalidate_sorted(c);
}

int gbh_write_morton(gbh_ctx* c, const uint64_t* host, uint32_t count, uint32_t offset) {
    RANGE_CHECK(c, host, count, offset, c->N);
    int rc = write_dev(c, c->keys[c->iin] + offset, host, (size_t)count * 8);
    if (rc) return rc;
    return invalidate_sorted(c);
}

// ---- stage entry points -------------------------------------------------------

static int stage_common(gbh_ctx* c, const gbh_step_params* p) {
    if (!c) return GBH_ERR_INVALID;
    if (!c->inited) return fail(c, GBH_ERR_STATE, "stage call before gbh_init");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if (p) return upload_params(c, p);
    if (!c->params_valid) return fail(c, GBH_ERR_STATE, "stage call before any step parameters were given");
    return GBH_OK;
}

// eager stages run outside the step graph: the next compaction gathers
#define STAGE_BODY(c, p, fn)                   \
    do {                                       \
        int rc_ = stage_common(c, p);          \
        if (rc_) return rc_;                   \
        rc_ = fn(c);                           \
        if (rc_) return rc_;                   \
        if ((rc_ = invalidate_sorted(c))) return rc_; \
        return gbh_synchronize(c);             \
    } while (0)

int gbh_stage_reset(gbh_ctx* c, const gbh_step_params* p) {
    int rc = stage_common(c, p);
    if (rc) return rc;
    if ((rc = prepare_precision(c))) return rc;
    if ((rc = enqueue_reset(c))) return rc;
    if ((rc = invalidate_sorted(c))) return rc;
    return gbh_synchronize(c);
}
int gbh_stage_prepare(gbh_ctx* c, const gbh_step_params* p) { STAGE_BODY(c, p, enqueue_prepare); }
int gbh_stage_sort(gbh_ctx* c) { STAGE_BODY(c, nullptr, enqueue_sort); }
int gbh_stage_build(gbh_ctx* c) {
    int rc = stage_common(c, nullptr);
    if (rc) return rc;
    if ((rc = enqueue_build(c))) return rc;
    // the stage boundary of the reference: its Node topology words as
    // buildBinaryRadixTree leaves them (the step itself goes straight to the
    // fill, which writes whole nodes)
    launch_build_nodes(ctx_buffers(c), c->stream);
    if ((rc = check_launch(c, "build nodes"))) return rc;
    if ((rc = invalidate_sorted(c))) return rc;
    return gbh_synchronize(c);
}
int gbh_stage_fill(gbh_ctx* c) { STAGE_BODY(c, nullptr, enqueue_fill); }
int gbh_stage_walk(gbh_ctx* c, const gbh_step_params* p) {
    int rc = stage_common(c, p);
    if (rc) return rc;
    if (c->params_host.precision_mode == GBH_PRECISION_COMPENSATED && !c->pos64_valid)
        return fail(c, GBH_ERR_STATE, "precision-form walk without current FP64 positions (run gbh_stage_reset first)");
    if ((rc = enqueue_walk(c))) return rc;
    if (c->params_host.flags & GBH_FLAG_STORE_POTENTIAL) c->potential_epoch = c->state_epoch;
    if ((rc = invalidate_sorted(c))) return rc;
    return gbh_synchronize(c);
}
int gbh_stage_merge(gbh_ctx* c, const gbh_step_params* p) { STAGE_BODY(c, p, enqueue_merge); }
int gbh_stage_swap(gbh_ctx* c) {
    if (!c) return GBH_ERR_INVALID;
    int rc = enqueue_swap(c);
    after_swap(c, c->params_valid && c->params_host.precision_mode == GBH_PRECISION_COMPENSATED);
    if (rc) return rc;
    return invalidate_sorted(c);
}

int gbh_step_profiled(gbh_ctx* c, const gbh_step_params* p, float ms_out[GBH_NUM_STAGES]) {
    int rc = stage_common(c, p);
    if (rc) return rc;
    if (!ms_out) return fail(c, GBH_ERR_INVALID, "ms_out is null");
    if ((rc = prepare_precision(c))) return rc;
    cudaEvent_t ev[GBH_NUM_STAGES + 1];
    for (int i = 0; i <= GBH_NUM_STAGES; ++i) CUDA_TRY(c, cudaEventCreate(&ev[i]));
    CUDA_TRY(c, cudaEventRecord(ev[0], c->stream));
    for (int s = 0; s < GBH_NUM_STAGES; ++s) {
        rc = k_stages[s](c);
        if (rc) break;
        CUDA_TRY(c, cudaEventRecord(ev[s + 1], c->stream));
    }
    if (!rc) {
        CUDA_TRY(c, cudaEventSynchronize(ev[GBH_NUM_STAGES]));
        for (int s = 0; s < GBH_NUM_STAGES; ++s) CUDA_TRY(c, cudaEventElapsedTime(&ms_out[s], ev[s], ev[s + 1]));
    }
    for (int i = 0; i <= GBH_NUM_STAGES; ++i) cudaEventDestroy(ev[i]);
    if (rc) return rc;
    // a whole step: the walk's in-order position copy stays current
    after_swap(c, c->params_host.precision_mode == GBH_PRECISION_COMPENSATED);
    return gbh_synchronize(c);
}

int gbh_direct_sum(gbh_ctx* c, const gbh_step_params* p, const uint32_t* sample, uint32_t count, double* out) {
    if (!c || !p || (!sample && count) || (!out && count)) return fail(c, GBH_ERR_INVALID, "null argument");
    if (count == 0) return GBH_OK;
    for (uint32_t i = 0; i < count; ++i)
        if (sample[i] >= c->N) return fail(c, GBH_ERR_INVALID, "sample index out of range");
    CUDA_TRY(c, cudaSetDevice(c->device));
    gbh_sim_values sv;
    int rc = read_dev(c, &sv, c->sim, sizeof(sv));
    if (rc) return rc;
    const uint32_t blocks = (count + 127) / 128;
    uint32_t chunks = (c->num_sms * 16 + blocks - 1) / blocks;
    if (chunks < 1) chunks = 1;
    if (chunks > c->N) chunks = c->N;
    uint32_t* d_sample = nullptr;
    double *d_partial = nullptr, *d_out = nullptr;
    CUDA_TRY(c, cudaMalloc(&d_sample, (size_t)count * 4));
    CUDA_TRY(c, cudaMalloc(&d_partial, (size_t)chunks * count * 3 * 8));
    CUDA_TRY(c, cudaMalloc(&d_out, (size_t)count * 3 * 8));
    cudaError_t e = cudaMemcpyAsync(d_sample, sample, (size_t)count * 4, cudaMemcpyHostToDevice, c->stream);
    // FP64 positions of the precision form when they hold the current state,
    // else the FP32 positions widened
    const bool pos64 = p->precision_mode == GBH_PRECISION_COMPENSATED && c->pos64_valid;
    if (e == cudaSuccess) {
        launch_direct_sum64(pos64 ? c->pos64[c->bin] : nullptr, c->bodies[c->bin], c->N, d_sample, count,
                            sv.gravitational_constant, p->softening, d_partial, d_out, chunks, c->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, (size_t)count * 3 * 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_sample);
    cudaFree(d_partial);
    cudaFree(d_out);
    if (e != cudaSuccess) return fail(c, GBH_ERR_CUDA, std::string("direct sum: ") + cudaGetErrorString(e));
    return GBH_OK;
}

}  // extern "C"
