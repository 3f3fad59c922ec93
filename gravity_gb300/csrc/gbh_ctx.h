// gbh_ctx.h — the context object behind the opaque gbh_ctx handle.
#pragma once

#include <map>
#include <string>

#include "gbh_common.cuh"

struct MacState;  // learned MAC buffers (k_mac.cu)

struct gbh_ctx {
    int device = 0;
    uint32_t num_sms = 1;  // cudaDevAttrMultiProcessorCount of `device`
    cudaStream_t stream = nullptr;
    uint32_t N = 0;
    uint32_t prep_tiles_cap = 0;
    uint32_t sort_tiles_cap = 0;
    gbh_units units{};
    bool inited = false;

    // one device arena holding every buffer below
    void* arena = nullptr;
    size_t arena_bytes = 0;
    gbh_body* bodies[2] = {nullptr, nullptr};
    int bin = 0;  // bodies[bin] is BodiesIn
    uint64_t* keys[2] = {nullptr, nullptr};
    uint32_t* idx[2] = {nullptr, nullptr};
    int iin = 0;  // keys[iin], idx[iin] are MortonIn / IndexIn
    gbh_node* leaf = nullptr;
    gbh_node* internal = nullptr;
    ChildPair* pairs = nullptr;
    WalkRec* root_rec = nullptr;
    float4* leaf_pm = nullptr;
    float4* sorted_pm = nullptr;
    float* leaf_rad = nullptr;
    gbh_sim_values* sim = nullptr;
    DevState* st = nullptr;
    gbh_step_params* params_dev = nullptr;
    MergeQueue* mq = nullptr;
    unsigned long long* mkeys = nullptr;
    uint32_t* mslots = nullptr;
    uint32_t* locks = nullptr;
    uint32_t* conflicts = nullptr;
    float4* accel = nullptr;
    float* accel_mag = nullptr;
    uint32_t* node_lo = nullptr;
    uint2* topo_kids = nullptr;
    uint32_t* topo_cnt = nullptr;
    uint32_t* fill_ready = nullptr;
    uint32_t* parent_int = nullptr;
    uint32_t* parent_leaf = nullptr;
    uint2* groups = nullptr;
    uint32_t* group_node = nullptr;
    uint32_t* group_path = nullptr;
    uint32_t group_path_cap = 0;
    bool paths_current = false;  // the start lists describe the current tree (enqueue_build)
    uint32_t* tile_dead = nullptr;
    float* tile_aabb = nullptr;
    uint32_t* hist = nullptr;
    uint32_t* bucket_base = nullptr;
    uint32_t* lookback = nullptr;
    size_t lookback_bytes = 0;

    // precision form and potential (allocated on first use, outside the arena)
    double* pos64[2] = {nullptr, nullptr};  // follow the body buffers' parity
    float4* leaf_lo = nullptr;
    float* potential = nullptr;
    bool pos64_valid = false;      // pos64[bin] holds the current state
    uint64_t state_epoch = 0;      // advances with every swap and upload
    uint64_t potential_epoch = ~0ull;  // state whose potential is in `potential`

    gbh_step_params params_host{};
    bool params_valid = false;
    uint32_t mac_mode = GBH_MAC_PLAIN;
    bool mac_ready = false;
    MacState* mac = nullptr;

    // gbh_exchange_bodies: a second stream for the device-to-host half and
    // one event per chunk (created with the context)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_events[16] = {};

    // gbh_step_streamed: two more body buffers (allocated on first use), one
    // taking the next input and one the result waiting for its read-back;
    // after the step the four rotate (the input becomes the state, the
    // consumed input the next output, the step's result waits for the next
    // call's read-back, and the buffer read back by this call takes the next
    // input), so no body buffer is copied on the device and the two copies
    // never wait for each other.  A call without a next input keeps the
    // result as the state and copies it to stage_out for the read-back.  The
    // read-back runs on a second copy stream; events order the copies with
    // the steps.
    gbh_body* stage_in = nullptr;       // takes the next input (rotates)
    gbh_body* spare = nullptr;          // the rotating result slot (rotates)
    gbh_body* stage_alloc[2] = {};      // the two extra buffers' allocations
    gbh_body* stage_out = nullptr;
    gbh_body* body_phys[4] = {};        // the four body buffers as allocated (graph keys name them)
    gbh_body* result_buf = nullptr;     // where the last streamed step's result waits
    cudaStream_t copy_stream2 = nullptr;
    cudaEvent_t ev_in_ready = nullptr, ev_out_ready = nullptr, ev_out_done = nullptr;
    bool stream_have_result = false;  // result_buf holds the result of the last streamed step

    // sharded step (gbh_step_shard_walk ... gbh_step_shard_finish)
    uint32_t shard_rank = 0, shard_world = 1;  // the walk's share while a shard walk is enqueued
    bool shard_open = false;                   // a shard walk ran; finish it before the next step

    std::map<int, cudaGraphExec_t> graphs;
    std::string last_error;
};

StepBuffers ctx_buffers(const gbh_ctx* c);
int enqueue_walk_learned(gbh_ctx* c);
void mac_release(gbh_ctx* c);
void sort_setup();
void group_walk_setup();
void fill_setup();
