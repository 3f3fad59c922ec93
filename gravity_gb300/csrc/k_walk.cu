// k_walk.cu — plain theta walk with leaf collisions, merge-task emission and
// the symplectic update.
//
// Replaces forceComputeKernel (SH/compute/force/bh_force.comp:6-142): one
// thread per body with a private 64-entry stack, a full 80-byte node gather per
// visit and a global atomic per opened node.
//
// Here a warp walks for 32 consecutive bodies of the Morton order (spatial
// neighbours) with ONE shared stack in shared memory.  Each stack entry
// carries the mask of lanes that opened its parent; a lane evaluates only the
// entries that carry its bit, so every lane visits exactly the nodes its own
// reference walk would visit, in the same depth-first order (childB popped
// before childA), and accumulates the same terms in the same order.  Node
// records are 32-byte WalkNodes (one sector) read warp-uniformly, so a visit
// is one broadcast load instead of 32 divergent 80-byte gathers.  The per-node
// debug atomic of the reference (bh_force.comp:72) becomes one add per warp.
#include "gbh_common.cuh"

#define WALK_THREADS 256
#define WALK_WARPS (WALK_THREADS / 32)

__global__ __launch_bounds__(WALK_THREADS) void k_walk_plain(StepBuffers b) {
    __shared__ uint32_t s_node[WALK_WARPS][GBH_WALK_STACK];
    __shared__ uint32_t s_mask[WALK_WARPS][GBH_WALK_STACK];
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t warp_global = blockIdx.x * WALK_WARPS + w;
    const uint32_t g = warp_global * 32 + lane;
    if (warp_global * 32 >= n) return;
    const bool active = g < n;
    const gbh_step_params* P = b.params;
    const gbh_sim_values* sim = b.sim;
    const float G = sim->gravitational_constant;
    const float soft = P->softening, theta = P->theta;
    const uint32_t mode = P->merging_collision_or_neither;
    const float4* __restrict__ leaf_pm = b.leaf_pm;
    const WalkNode* __restrict__ wn = b.wnode;

    const uint32_t bi = active ? b.idx_in[g] : 0u;
    float4 pm = active ? leaf_pm[g] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 vd = active ? ld_vel_density(b.bodies_in, bi) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float my_rad = (active && mode != GBH_MODE_NEITHER) ? b.leaf_rad[g] : 0.0f;
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    uint32_t inter = 0, seq = 0;
    uint32_t opened = 0;  // lane 0 only
    uint32_t max_sp = 0;
    bool overflow = false;

    int sp = 0;
    const uint32_t act_mask = __ballot_sync(0xffffffffu, active);
    if (n > 1) {
        if (lane == 0) {
            s_node[w][0] = N;  // root, bh_force.comp:53
            s_mask[w][0] = act_mask;
        }
        sp = 1;
    }
    __syncwarp();
    while (sp > 0) {
        --sp;
        const uint32_t node = s_node[w][sp];
        const uint32_t mask = s_mask[w][sp];
        __syncwarp();
        const bool me = (mask >> lane) & 1u;
        if (node >= N) {
            const WalkNode* p = wn + (node - N);
            const float4 cm = __ldg(&p->cm);
            const uint4 rest = __ldg(reinterpret_cast<const uint4*>(p) + 1);
            const float half = __uint_as_float(rest.x);
            const float rx = cm.x - pm.x, ry = cm.y - pm.y, rz = cm.z - pm.z;
            const float d2 = rx * rx + ry * ry + rz * rz + soft;
            const float inv = rsqrtf(d2);
            const bool accept = half * inv < theta;
            if (me && accept) {
                const float s = G * cm.w;
                ax = ax + s * rx * inv * inv * inv;
                ay = ay + s * ry * inv * inv * inv;
                az = az + s * rz * inv * inv * inv;
                ++inter;
            }
            const uint32_t om = __ballot_sync(0xffffffffu, me && !accept);
            if (om) {
                if (sp + 2 > GBH_WALK_STACK) {
                    overflow = true;
                    break;
                }
                if (lane == 0) {
                    s_node[w][sp] = rest.y;      // childA
                    s_mask[w][sp] = om;
                    s_node[w][sp + 1] = rest.z;  // childB, popped first
                    s_mask[w][sp + 1] = om;
                    opened += __popc(om);
                }
                sp += 2;
                max_sp = max(max_sp, (uint32_t)sp);
                __syncwarp();
            }
        } else {
            // leaf: sorted slot `node`; skip the body's own leaf (bh_force.comp:76-78)
            const float4 o = __ldg(leaf_pm + node);
            if (me && node != g) {
                const float rx = o.x - pm.x, ry = o.y - pm.y, rz = o.z - pm.z;
                const float rr = rx * rx + ry * ry + rz * rz;
                const float inv = rsqrtf(rr + soft);
                const float s = G * o.w;
                ax = ax + s * rx * inv * inv * inv;
                ay = ay + s * ry * inv * inv * inv;
                az = az + s * rz * inv * inv * inv;
                ++inter;
                if (mode != GBH_MODE_NEITHER) {
                    const uint32_t oi = b.idx_in[node];
                    const float orad = b.leaf_rad[node];
                    const float dist = sqrtf(rr);
                    const float pen = my_rad + orad - dist;
                    if (mode == GBH_MODE_COLLISION && pen > 0.0f) {
                        // bh_force.comp:93-107
                        const float4 ov = ld_vel_density(b.bodies_in, oi);
                        const float vx = ov.x - vd.x, vy = ov.y - vd.y, vz = ov.z - vd.z;
                        const float len = sqrtf(rr);
                        const float nx = rx / len, ny = ry / len, nz = rz / len;
                        const float vimp = vx * nx + vy * ny + vz * nz;
                        if (vimp < 0.0f) {
                            const float meff = 1.0f / (1.0f / pm.w + 1.0f / o.w);
                            const float imp = (1.0f + P->elasticity) * meff * vimp;
                            vd.x += nx * imp / pm.w;
                            vd.y += ny * imp / pm.w;
                            vd.z += nz * imp / pm.w;
                        }
                        const float sc = pen / (pm.w + o.w) * P->restitution;
                        pm.x -= sc * nx;
                        pm.y -= sc * ny;
                        pm.z -= sc * nz;
                    }
                    if (mode == GBH_MODE_MERGE && pen > 0.0f && bi < oi) {
                        // bh_force.comp:109-112, plus an ordering key for merge resolution
                        const uint32_t slot = atomicAdd(&b.mq->tail, 1u);
                        if (slot < N) {
                            b.mq->pairs[slot] = make_uint2(bi, oi);
                            b.mkeys[slot] = ((unsigned long long)g << 32) | seq;
                        }
                        ++seq;
                    }
                }
            }
        }
    }
    if (overflow && lane == 0) set_error(b.st, GBH_DEVERR_WALK_STACK);

    // counters: one atomic per warp
    uint32_t tot = inter;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) {
        atomicAdd(&b.st->interactions, (unsigned long long)tot);
        atomicAdd(&b.st->opened, (unsigned long long)opened);
        atomicAdd(&b.sim->uint_debug[0], opened);
        atomicMax(&b.st->max_stack, max_sp);
    }
    if (!active) return;
    if (b.accel && (P->flags & GBH_FLAG_STORE_ACCEL)) b.accel[bi] = make_float4(ax, ay, az, 0.0f);

    // symplectic update and static bounds, bh_force.comp:117-141
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
            atomicAdd(&b.sim->out_of_bounds, 1u);
            atomicAdd(&b.st->oob, 1u);
            return;
        }
    }
    st_body(b.bodies_out, bi, make_float4(npx, npy, npz, pm.w), make_float4(nvx, nvy, nvz, vd.w));
}

void launch_walk_plain(const StepBuffers& b, cudaStream_t s) {
    const uint32_t blocks = (b.N + WALK_THREADS - 1) / WALK_THREADS;
    k_walk_plain<<<blocks, WALK_THREADS, 0, s>>>(b);
}
