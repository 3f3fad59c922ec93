// k_walk.cu — plain theta walk with leaf collisions, merge-task emission and
// the symplectic update.
//
// Replaces forceComputeKernel (SH/compute/force/bh_force.comp:6-142): one
// thread per body with a private 64-entry stack, a full 80-byte node gather per
// visit and a global atomic per opened node.
//
// Here a warp walks for 32 consecutive bodies of the Morton order (spatial
// neighbours) with ONE shared stack.  Each stack entry carries the mask of
// lanes that opened its parent; a lane evaluates only the entries that carry
// its bit, so every lane visits exactly the nodes its own reference walk would
// visit, in the same depth-first order (childB evaluated before childA), and
// accumulates its terms in that order.
//
// Node data travel with the traversal: opening a node reads its ChildPair
// (the 32-byte records of both children, one 64-byte warp-uniform load);
// childB is evaluated next straight from registers and childA is pushed, with
// its record, on the warp's shared-memory stack.  A visit therefore costs no
// global load of its own, and one load serves two visits.  The per-node debug
// atomic of the reference (bh_force.comp:72) becomes one add per warp.
//
// Arithmetic: the MAC is the reference's (half side * invDist < theta, with
// invDist from the softened distance); the force sum uses fused multiply-adds
// (G m inv^3 r accumulated with FMA), which is within 1e-7 relative of the
// reference's operation order.
#include "gbh_common.cuh"

#define WALK_THREADS 256
#define WALK_WARPS (WALK_THREADS / 32)
#define WALK_STACK 128

struct __align__(16) StackEntry {
    float4 cm;
    float half;
    uint32_t id;
    uint32_t mask;
    uint32_t pad;
};

// PREC: the precision form.  Offsets are formed from the FP32 position and
// its FP32 residual (leaf_lo), r = (x_j - x_b) + (lo_j - lo_b) for a leaf and
// (com - x_b) - lo_b for a node, and the leaf terms are summed with Kahan
// compensation apart from the node terms.  Gravity only.
template <bool PREC>
__global__ __launch_bounds__(WALK_THREADS) void k_walk_plain(StepBuffers b) {
    __shared__ StackEntry s_stack[WALK_WARPS][WALK_STACK];
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t warp_global = blockIdx.x * WALK_WARPS + w;
    const uint32_t g = warp_global * 32 + lane;
    if (blockIdx.x == 0 && threadIdx.x == 0) b.st->sorted_valid = 1u;  // the update below fills sorted_pm
    if (warp_global * 32 >= n) return;
    uint32_t s_lo, s_hi;
    shard_slots(b, n, s_lo, s_hi);
    if (warp_global * 32 + 32 <= s_lo || warp_global * 32 >= s_hi) return;
    const bool active = g < n && g >= s_lo && g < s_hi;
    const gbh_step_params* P = b.params;
    const gbh_sim_values* sim = b.sim;
    const float G = sim->gravitational_constant;
    const float soft = P->softening, theta = P->theta;
    const uint32_t mode = P->merging_collision_or_neither;
    const ChildPair* __restrict__ pairs = b.pairs;
    StackEntry* stk = s_stack[w];

    const uint32_t bi = active ? b.idx_in[g] : 0u;
    float4 pm = active ? b.leaf_pm[g] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 vd = active ? ld_vel_density(b.bodies_in, bi) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float my_rad = (active && mode != GBH_MODE_NEITHER) ? b.leaf_rad[g] : 0.0f;
    const float4 lo_b = (PREC && active) ? b.leaf_lo[g] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool want_pot = (P->flags & GBH_FLAG_STORE_POTENTIAL) && b.potential;
    float ax = 0.0f, ay = 0.0f, az = 0.0f, pot = 0.0f;
    float nx_ = 0.0f, ny_ = 0.0f, nz_ = 0.0f, np_ = 0.0f;  // PREC: leaf terms (Kahan)
    float cx_ = 0.0f, cy_ = 0.0f, cz_ = 0.0f, cp_ = 0.0f;
    uint32_t inter = 0, seq = 0;
    uint32_t opened = 0;
    uint32_t sp = 0, max_sp = 0;
    bool overflow = false;

    // current entry (warp-uniform): starts at the root, bh_force.comp:53
    float4 cur_cm;
    float cur_half;
    uint32_t cur_id, cur_mask;
    {
        const WalkRec root = *b.root_rec;
        cur_cm = root.cm;
        cur_half = root.half_side;
        cur_id = N;
        cur_mask = __ballot_sync(0xffffffffu, active);
    }
    const bool walk = n > 1;
    while (walk) {
        const bool me = (cur_mask >> lane) & 1u;
        float rx = cur_cm.x - pm.x, ry = cur_cm.y - pm.y, rz = cur_cm.z - pm.z;
        if (PREC) {
            float4 lo_j = make_float4(0.f, 0.f, 0.f, 0.f);
            if (cur_id < N) lo_j = b.leaf_lo[cur_id];
            rx = rx + (lo_j.x - lo_b.x);
            ry = ry + (lo_j.y - lo_b.y);
            rz = rz + (lo_j.z - lo_b.z);
        }
        const float rr = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
        const float inv = rsqrtf(rr + soft);
        bool open = false, interact;
        if (cur_id >= N) {
            const bool accept = cur_half * inv < theta;
            interact = me && accept;
            open = me && !accept;
        } else {
            interact = me && cur_id != g;  // the body's own leaf, bh_force.comp:76-78
        }
        if (interact) {
            const float f = G * cur_cm.w * (inv * inv * inv);
            if (PREC && cur_id < N) {
                kahan_add(nx_, cx_, f * rx);
                kahan_add(ny_, cy_, f * ry);
                kahan_add(nz_, cz_, f * rz);
                if (want_pot) kahan_add(np_, cp_, -(G * cur_cm.w) * inv);
            } else {
                ax = __fmaf_rn(f, rx, ax);
                ay = __fmaf_rn(f, ry, ay);
                az = __fmaf_rn(f, rz, az);
                if (want_pot) pot = __fmaf_rn(-(G * cur_cm.w), inv, pot);
            }
            ++inter;
            if (!PREC && mode != GBH_MODE_NEITHER && cur_id < N) {
                const uint32_t oi = b.idx_in[cur_id];
                const float orad = b.leaf_rad[cur_id];
                const float dist = sqrtf(rx * rx + ry * ry + rz * rz);
                const float pen = my_rad + orad - dist;
                if (mode == GBH_MODE_COLLISION && pen > 0.0f) {
                    // bh_force.comp:93-107, in the reference's operation order
                    const float ow = cur_cm.w;
                    const float4 ov = ld_vel_density(b.bodies_in, oi);
                    const float vx = ov.x - vd.x, vy = ov.y - vd.y, vz = ov.z - vd.z;
                    const float nx = rx / dist, ny = ry / dist, nz = rz / dist;
                    const float vimp = vx * nx + vy * ny + vz * nz;
                    if (vimp < 0.0f) {
                        const float meff = 1.0f / (1.0f / pm.w + 1.0f / ow);
                        const float imp = (1.0f + P->elasticity) * meff * vimp;
                        vd.x += nx * imp / pm.w;
                        vd.y += ny * imp / pm.w;
                        vd.z += nz * imp / pm.w;
                    }
                    const float sc = pen / (pm.w + ow) * P->restitution;
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
                        b.mslots[slot] = cur_id;
                    }
                    ++seq;
                }
            }
        }
        const uint32_t om = __ballot_sync(0xffffffffu, open);
        if (om) {
            opened += __popc(om);
            const float4* q = reinterpret_cast<const float4*>(pairs + (cur_id - N));
            const float4 a_cm = __ldg(q + 0);
            const uint4 a_meta = __ldg(reinterpret_cast<const uint4*>(q + 1));
            const float4 b_cm = __ldg(q + 2);
            const uint4 b_meta = __ldg(reinterpret_cast<const uint4*>(q + 3));
            if (sp >= WALK_STACK) {
                overflow = true;
                break;
            }
            if (lane == 0) {
                stk[sp].cm = a_cm;
                *reinterpret_cast<uint4*>(&stk[sp].half) = make_uint4(a_meta.x, a_meta.y, om, 0u);
            }
            ++sp;
            max_sp = max(max_sp, sp);
            cur_cm = b_cm;
            cur_half = __uint_as_float(b_meta.x);
            cur_id = b_meta.y;
            cur_mask = om;
        } else {
            if (sp == 0) break;
            --sp;
            __syncwarp();
            const float4 e_cm = stk[sp].cm;
            const uint4 e_meta = *reinterpret_cast<const uint4*>(&stk[sp].half);
            __syncwarp();
            cur_cm = e_cm;
            cur_half = __uint_as_float(e_meta.x);
            cur_id = e_meta.y;
            cur_mask = e_meta.z;
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
        atomicMax(&b.st->max_stack, max_sp + 1);
    }
    if (!active) return;
    if (PREC) {
        ax = ax + (nx_ - cx_);
        ay = ay + (ny_ - cy_);
        az = az + (nz_ - cz_);
        pot = pot + (np_ - cp_);
    }
    if (b.accel && (P->flags & GBH_FLAG_STORE_ACCEL)) b.accel[bi] = make_float4(ax, ay, az, 0.0f);
    if (b.accel_mag) b.accel_mag[bi] = sqrtf(ax * ax + ay * ay + az * az);
    if (want_pot) b.potential[bi] = pot;
    if (PREC)
        walk_update_fp64(b, P, sim, g, bi, pm, vd, ax, ay, az);
    else
        walk_update(b, P, sim, g, bi, pm, vd, ax, ay, az);
}

void launch_walk_plain(const StepBuffers& b, cudaStream_t s) {
    const uint32_t blocks = (b.N + WALK_THREADS - 1) / WALK_THREADS;
    if (b.prec)
        k_walk_plain<true><<<blocks, WALK_THREADS, 0, s>>>(b);
    else
        k_walk_plain<false><<<blocks, WALK_THREADS, 0, s>>>(b);
}
