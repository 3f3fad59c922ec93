// k_merge.cu — merge resolution.
//
// Replaces mergeBodiesKernel (SH/compute/merge/bh_merge.comp:30-71): every
// thread loops on an atomic queue head and try-locks both bodies, skipping a
// task when a lock is taken, so the outcome depends on scheduling.
//
// Here the outcome is deterministic and equals the reference run with a
// single thread in the walk's emission order (slot-major, then depth-first
// order inside a body's walk), a schedule under which no try-lock fails:
//   1. count how many tasks touch each body (the lock words double as counters);
//   2. a task whose two bodies appear in no other task commutes with every
//      other task and is applied at once, in parallel;
//   3. the remaining (conflicting) tasks are resolved in rounds by one block:
//      a task runs in a round when its emission key is the earliest pending
//      key of both its bodies, so every earlier task on those bodies has run
//      and the round's tasks touch disjoint bodies; each round runs at least
//      the globally earliest pending task, so the rounds end, and the result
//      is the one-thread schedule's for any number of conflicts;
//   4. the lock words are cleared again.
#include "gbh_common.cuh"

#define MERGE_SORT_THREADS 1024
#define MERGE_DONE 0x80000000u  // a conflict-list entry whose task has run (task ids < 2^30)

// mergeBodies, bh_merge.comp:5-22
__device__ __forceinline__ void merge_two(float4& p1, float4& v1, const float4 p2, const float4 v2) {
    const float m1 = p1.w, m2 = p2.w;
    const float M = m1 + m2;
    if (M == 0.0f) {
        p1 = make_float4(0.f, 0.f, 0.f, 0.f);
        v1 = p1;
        return;
    }
    if (m1 == 0.0f) {
        p1 = p2;
        v1 = v2;
        return;
    }
    if (m2 == 0.0f) return;
    float4 np, nv;
    np.x = (p1.x * m1 + p2.x * m2) / M;
    np.y = (p1.y * m1 + p2.y * m2) / M;
    np.z = (p1.z * m1 + p2.z * m2) / M;
    np.w = M;
    nv.x = (v1.x * m1 + v2.x * m2) / M;
    nv.y = (v1.y * m1 + v2.y * m2) / M;
    nv.z = (v1.z * m1 + v2.z * m2) / M;
    nv.w = (m1 + m2) / (m1 / v1.w + m2 / v2.w);
    p1 = np;
    v1 = nv;
}

// apply task t, bodies (a, c), on the output bodies, and keep the in-order
// copy of the positions (sorted slots of a and c) equal to them; returns true
// when merged
__device__ __forceinline__ bool apply_task(const StepBuffers& b, uint32_t t, uint32_t a, uint32_t c) {
    if (a == c) return false;
    gbh_body* dst = b.bodies_out;
    float4 p1 = ld_pos_mass(dst, a), v1 = ld_vel_density(dst, a);
    const float4 p2 = ld_pos_mass(dst, c), v2 = ld_vel_density(dst, c);
    if (p1.w == 0.0f || p2.w == 0.0f) return false;
    merge_two(p1, v1, p2, v2);
    st_body(dst, a, p1, v1);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    st_body(dst, c, z, z);
    b.sorted_pm[(uint32_t)(b.mkeys[t] >> 32)] = p1;
    b.sorted_pm[b.mslots[t]] = z;
    return true;
}

__global__ void k_merge_count(StepBuffers b) {
    const uint32_t M = min(b.mq->tail, b.N);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const uint2 pr = b.mq->pairs[t];
        atomicAdd(&b.locks[pr.x], 1u);
        atomicAdd(&b.locks[pr.y], 1u);
    }
}

__global__ void k_merge_apply(StepBuffers b) {
    const uint32_t M = min(b.mq->tail, b.N);
    uint32_t merged = 0;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const uint2 pr = b.mq->pairs[t];
        if (b.locks[pr.x] == 1u && b.locks[pr.y] == 1u) {
            merged += apply_task(b, t, pr.x, pr.y) ? 1u : 0u;
        } else {
            const uint32_t slot = atomicAdd(&b.st->merge_conflicts, 1u);
            b.conflicts[slot] = t;
        }
    }
    if (merged) atomicAdd(&b.st->merged, merged);
}

// Step 3.  The earliest pending key per body lives in the step's spare key
// buffer (keys_out, by body id), free from the end of the fill to the next
// step's encode.
__global__ __launch_bounds__(MERGE_SORT_THREADS) void k_merge_conflicts(StepBuffers b) {
    __shared__ uint32_t s_pending, s_merged;
    const uint32_t C = b.st->merge_conflicts;
    if (threadIdx.x == 0) b.st->merge_tasks = min(b.mq->tail, b.N);
    if (C == 0) return;
    unsigned long long* first = reinterpret_cast<unsigned long long*>(b.keys_out);
    uint32_t* list = b.conflicts;
    for (uint32_t k = threadIdx.x; k < C; k += blockDim.x) {
        const uint2 pr = b.mq->pairs[list[k]];
        first[pr.x] = ~0ull;
        first[pr.y] = ~0ull;
    }
    if (threadIdx.x == 0) s_merged = 0;
    __syncthreads();
    uint32_t pending = C;
    for (uint32_t round = 0; pending > 0 && round <= C; ++round) {
        // the earliest pending key of every body of a pending task
        for (uint32_t k = threadIdx.x; k < C; k += blockDim.x) {
            const uint32_t e = list[k];
            if (e & MERGE_DONE) continue;
            const uint2 pr = b.mq->pairs[e];
            const unsigned long long key = b.mkeys[e];
            atomicMin(&first[pr.x], key);
            atomicMin(&first[pr.y], key);
        }
        if (threadIdx.x == 0) s_pending = 0;
        __syncthreads();
        // the tasks first on both bodies run (disjoint bodies); the rest wait
        uint32_t merged = 0, left = 0;
        for (uint32_t k = threadIdx.x; k < C; k += blockDim.x) {
            const uint32_t e = list[k];
            if (e & MERGE_DONE) continue;
            const uint2 pr = b.mq->pairs[e];
            const unsigned long long key = b.mkeys[e];
            if (first[pr.x] == key && first[pr.y] == key) {
                merged += apply_task(b, e, pr.x, pr.y) ? 1u : 0u;
                list[k] = e | MERGE_DONE;
            } else {
                ++left;
            }
        }
        if (merged) atomicAdd(&s_merged, merged);
        if (left) atomicAdd(&s_pending, left);
        __syncthreads();
        pending = s_pending;
        // forget this round's minima
        for (uint32_t k = threadIdx.x; k < C; k += blockDim.x) {
            const uint2 pr = b.mq->pairs[list[k] & ~MERGE_DONE];
            first[pr.x] = ~0ull;
            first[pr.y] = ~0ull;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (pending) set_error(b.st, GBH_DEVERR_MERGE_OVERFLOW);  // cannot happen: a round always runs a task
        b.st->merged += s_merged;
    }
}

__global__ void k_merge_clear(StepBuffers b) {
    const uint32_t M = min(b.mq->tail, b.N);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < M; t += gridDim.x * blockDim.x) {
        const uint2 pr = b.mq->pairs[t];
        b.locks[pr.x] = 0u;
        b.locks[pr.y] = 0u;
    }
}

void launch_merge(const StepBuffers& b, cudaStream_t s) {
    const uint32_t blocks = b.num_sms * 4;
    k_merge_count<<<blocks, 256, 0, s>>>(b);
    k_merge_apply<<<blocks, 256, 0, s>>>(b);
    k_merge_conflicts<<<1, MERGE_SORT_THREADS, 0, s>>>(b);
    k_merge_clear<<<blocks, 256, 0, s>>>(b);
}
