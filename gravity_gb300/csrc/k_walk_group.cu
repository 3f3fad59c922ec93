// k_walk_group.cu — group walk: one acceptance decision per (body group, node).
//
// The reference decides per body (bh_force.comp:57-115).  Here a warp takes
// one body group, a subtree of at most GBH_GROUP_MAX = 96 bodies (three per
// lane; the build lists the groups, k_tree.cu), and walks the tree once for
// all of its bodies:
//   * candidates come off a per-warp stack 32 at a time, one per lane; each
//     lane evaluates the acceptance criterion of the group against its node;
//   * accepted nodes and leaves are appended to an interaction list, opened
//     nodes push their two children;
//   * every 32 list entries, all lanes accumulate the forces of the whole
//     list on their own bodies (dense FMA loop, node data broadcast from
//     shared memory).
// Criteria (gbh_step_params.mac_mode):
//   GBH_MAC_GROUP    accept when the boxes are disjoint and half_side < theta *
//                    sqrt(d^2 + softening), d = max(|com - c_g| - R_g, 0), with
//                    c_g, R_g the centre and half diagonal of the group's box;
//   GBH_MAC_LEARNED  nodes that pass the group rule at the band's lower theta
//                    (default 0.25) are accepted, nodes that fail it at its
//                    upper theta (default 4) are opened (gbh_mac_set_band),
//                    and in between the MLP decides: accept when its predicted
//                    log10 relative error of the monopole, max over the group,
//                    is below mac_tolerance (mac_mlp.cuh: features and
//                    tensor-core inference).
// A third instance records (group, node) candidates and their features for
// the MLP's training data (gbh_mac_generate).
// The kernel is persistent: one grid of as many blocks as fit on the GPU at
// once, and each warp takes its next group from a ticket counter when it has
// finished the last, so warps that meet short walks are not left idle while
// the rest of their block finishes long ones.
// Only gravity (merging_collision_or_neither == 0) runs here.
#include <cstddef>
#include <type_traits>

#include "gbh_ctx.h"
#include "mac_mlp.cuh"

#define GW_STACK 768
#define GW_LIST 64
#define GW_QUEUE 64  // queued band candidates per warp: a full MLP batch + one pop
#define GW_BPL (GBH_GROUP_MAX / 32)  // bodies per lane
#ifndef GW_DECIDE_SP
#define GW_DECIDE_SP 64u  // learned walk: decide the queue early below this stack depth...
#endif
#ifndef GW_DECIDE_NP
#define GW_DECIDE_NP 16u  // ...when at least this many rows wait
#endif

enum GroupMode { GM_THETA = 0, GM_LEARNED = 1, GM_RECORD = 2 };

// Block shape per mode.  The learned walk runs 4-warp blocks, five per SM
// (96 registers, 44 KB of shared memory each): 20 warps per SM, where 8-warp
// blocks fit two (16 warps).  The others run 8-warp blocks.
template <int MODE>
struct GroupShape {
    static constexpr int warps = MODE == GM_LEARNED ? 4 : 8;
    static constexpr int threads = warps * 32;
};

// shared memory: the stacks and lists first, the network's tiles last (only
// the learned walk allocates them).  The learned walk's stacks are shorter so
// that more blocks fit on an SM.
template <int STACK, int GW_WARPS>
struct GroupSmem {
    uint32_t stack[GW_WARPS][STACK];
    float4 list_cm[GW_WARPS][GW_LIST];  // centre of mass, G x mass
    uint32_t list_id[GW_WARPS][GW_LIST];
    float list_rad[GW_WARPS][GW_LIST];  // merge form: the leaf entries' body radii
    // merge form: each group body's radius and task counter (slot q * 32 +
    // lane), the group's largest radius
    float body_rad[GW_WARPS][GBH_GROUP_MAX];
    uint32_t body_seq[GW_WARPS][GBH_GROUP_MAX];
    float grp_rad[GW_WARPS];
    // queued band candidates of the learned walk: centre of mass, box and
    // count, box and id, children
    float4 pend_cm[GW_WARPS][GW_QUEUE];
    float4 pend_b0[GW_WARPS][GW_QUEUE];
    float4 pend_b1[GW_WARPS][GW_QUEUE];
    uint2 pend_kids[GW_WARPS][GW_QUEUE];
    GroupGeom geom[GW_WARPS];  // the group's geometry and feature terms
    alignas(16) uint32_t frag[MAC_SMEM_FRAG_WORDS];
    __nv_bfloat16 x[GW_WARPS * 32 * 16];  // feature tile of the batch being decided
};
#ifndef GW_STACK_LEARNED
#define GW_STACK_LEARNED 640
#endif
template <int MODE>
struct GroupCfg {
    static constexpr int stack = MODE == GM_LEARNED ? GW_STACK_LEARNED : GW_STACK;
    using Smem = GroupSmem<stack, GroupShape<MODE>::warps>;
    static constexpr size_t smem = MODE == GM_LEARNED ? sizeof(Smem) : offsetof(Smem, pend_cm);
};

// PREC: the precision form.  The lanes' bodies and the list entries are kept
// relative to the group centre c_g: (x - c_g) + lo for a leaf (lo its FP32
// residual), com - c_g for a node; leaf terms are summed with Kahan
// compensation apart from the node terms.
// FORM: the arithmetic form and the step's extra work, fixed per instance so
// that the common case keeps its registers: FORM_FP32, FORM_PREC (precision
// form), FORM_MERGE (merge tasks from the leaf entries).
enum GroupForm { FORM_FP32 = 0, FORM_PREC = 1, FORM_MERGE = 2 };

// resident blocks per SM each instance is compiled for: the learned FP32 walk
// five 4-warp blocks, its precision and merge forms four (their registers
// need more than 96), the group-theta FP32 walk three 8-warp blocks, the rest
// two
template <int MODE, int FORM>
struct GroupMinBlocks {
    static constexpr int value = MODE == GM_LEARNED ? (FORM == FORM_FP32 ? 5 : 4)
                                 : (MODE == GM_THETA && FORM == FORM_FP32) ? 3 : 2;
};

template <int MODE, int FORM>
__global__ __launch_bounds__(GroupShape<MODE>::threads, GroupMinBlocks<MODE, FORM>::value) void k_walk_group(
    StepBuffers b, MacDeviceWeights mw) {
    constexpr bool PREC = FORM == FORM_PREC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Cfg = GroupCfg<MODE>;
    typename Cfg::Smem& S = *reinterpret_cast<typename Cfg::Smem*>(smem_raw);
    if (MODE == GM_LEARNED) mac_load_frag(mw, S.frag, S.x);
    // the updates below fill sorted_pm (the recording walk updates nothing the
    // step keeps)
    if (MODE != GM_RECORD && blockIdx.x == 0 && threadIdx.x == 0) b.st->sorted_valid = 1u;
    const float band_lo = (MODE != GM_THETA) ? mw.band[0] : 0.0f;
    const float band_hi = (MODE != GM_THETA) ? mw.band[1] : 0.0f;
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t num_groups = b.st->num_groups;
    // groups hold up to GBH_GROUP_MAX bodies, usually fewer: each warp takes
    // the next group's ticket; lane l holds bodies l, l + 32, l + 64 of it
    for (;;) {
    uint32_t gi = 0;
    if (lane == 0) gi = atomicAdd(&b.st->group_next, 1u);
    gi = __shfl_sync(0xffffffffu, gi, 0);
    if (gi >= num_groups) break;
    if (b.shard_world > 1) {  // a sharded walk: this rank's groups only
        uint32_t s_lo, s_hi;
        shard_slots(b, n, s_lo, s_hi);
        const uint32_t first = b.groups[gi].x;
        if (first < s_lo || first >= s_hi) continue;
    }
    const uint2 grp = b.groups[gi];
    uint32_t gq[GW_BPL];
    bool actq[GW_BPL];
#pragma unroll
    for (int q = 0; q < GW_BPL; ++q) {
        gq[q] = grp.x + lane + 32u * q;
        actq[q] = lane + 32u * q < grp.y;
    }
    const gbh_step_params* P = b.params;
    const gbh_sim_values* sim = b.sim;
    const float G = sim->gravitational_constant;
    const float soft = P->softening, theta = P->theta, tol = P->mac_tolerance;
    uint32_t* stk = S.stack[w];
    float4* lcm = S.list_cm[w];
    uint32_t* lid = S.list_id[w];
    float* lrad = S.list_rad[w];

    // group box (inactive slots repeat the first body)
    float4 pmq[GW_BPL];
#pragma unroll
    for (int q = 0; q < GW_BPL; ++q) pmq[q] = b.leaf_pm[actq[q] ? gq[q] : grp.x];
    float mnx = pmq[0].x, mny = pmq[0].y, mnz = pmq[0].z, mxx = pmq[0].x, mxy = pmq[0].y, mxz = pmq[0].z;
#pragma unroll
    for (int q = 1; q < GW_BPL; ++q) {
        mnx = fminf(mnx, pmq[q].x);
        mny = fminf(mny, pmq[q].y);
        mnz = fminf(mnz, pmq[q].z);
        mxx = fmaxf(mxx, pmq[q].x);
        mxy = fmaxf(mxy, pmq[q].y);
        mxz = fmaxf(mxz, pmq[q].z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o));
        mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
        mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
    }
    GroupGeom gg;
    gg.cx = 0.5f * (mnx + mxx);
    gg.cy = 0.5f * (mny + mxy);
    gg.cz = 0.5f * (mnz + mxz);
    const float hx = 0.5f * (mxx - mnx), hy = 0.5f * (mxy - mny), hz = 0.5f * (mxz - mnz);
    gg.R = sqrtf(hx * hx + hy * hy + hz * hz);
    gg.bmin = make_float3(mnx, mny, mnz);
    gg.bmax = make_float3(mxx, mxy, mxz);
    gg.a_ref = (MODE != GM_THETA) ? group_accel_ref(b, actq, gq) : 0.0f;
    gg.soft = soft;
    if (MODE != GM_THETA) group_feature_terms(gg, G, soft);
    if (MODE == GM_LEARNED) {
        // the features read the group's terms from shared memory
        __syncwarp();
        if (lane == 0) S.geom[w] = gg;
        __syncwarp();
    }

    // walk coordinates of this lane's bodies (absolute, or group-relative)
    float3 pw[GW_BPL];
#pragma unroll
    for (int q = 0; q < GW_BPL; ++q) {
        pw[q] = make_float3(pmq[q].x, pmq[q].y, pmq[q].z);
        if (PREC) {
            const float4 lo_b = b.leaf_lo[actq[q] ? gq[q] : grp.x];
            pw[q] = make_float3((pmq[q].x - gg.cx) + lo_b.x, (pmq[q].y - gg.cy) + lo_b.y, (pmq[q].z - gg.cz) + lo_b.z);
        }
    }
    const bool want_pot = (P->flags & GBH_FLAG_STORE_POTENTIAL) && b.potential;
    // merging (bh_force.comp:109-112): every leaf entry is tested for overlap
    constexpr bool merging = FORM == FORM_MERGE;
    // the merge state lives in shared memory: the tests are rare (screened)
    float* my_rad = S.body_rad[w];
    uint32_t* seq = S.body_seq[w];
    if (merging) {
        float gr = 0.0f;
#pragma unroll
        for (int q = 0; q < GW_BPL; ++q) {
            const float r = actq[q] ? b.leaf_rad[gq[q]] : 0.0f;
            my_rad[q * 32 + lane] = r;
            seq[q * 32 + lane] = 0;
            gr = fmaxf(gr, r);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gr = fmaxf(gr, __shfl_xor_sync(0xffffffffu, gr, o));
        __syncwarp();
        if (lane == 0) S.grp_rad[w] = gr;
        __syncwarp();
    }
    float ax[GW_BPL], ay[GW_BPL], az[GW_BPL], pot[GW_BPL];
    float nx_[GW_BPL], ny_[GW_BPL], nz_[GW_BPL], np_[GW_BPL];  // PREC: leaf terms (Kahan)
    float cx_[GW_BPL], cy_[GW_BPL], cz_[GW_BPL], cp_[GW_BPL];
#pragma unroll
    for (int q = 0; q < GW_BPL; ++q) {
        ax[q] = ay[q] = az[q] = pot[q] = 0.f;
        nx_[q] = ny_[q] = nz_[q] = np_[q] = 0.f;
        cx_[q] = cy_[q] = cz_[q] = cp_[q] = 0.f;
    }
    uint32_t inter = 0, evals = 0, opened = 0;
    uint32_t sp = 0, ln = 0, np = 0;
    bool saturated = false;
    if (n > 1) {
        // the group's start list when it has one (k_group_paths: its own
        // subtree, then the siblings of its ancestors), else the root.  The
        // group's own subtree enters as its leaves, sorted slots [first,
        // first + count): a walk opens every internal node of it (their boxes
        // hold group bodies) and lists every leaf.
        const uint32_t* path = b.group_path + (size_t)gi * GBH_PATH_WORDS;
        const uint32_t len = gi < b.group_path_cap ? path[0] : 0u;
        if (len == 0) {
            if (lane == 0) stk[0] = N;
            sp = 1;
        } else {
            for (uint32_t k = lane; k < len - 1; k += 32) stk[k] = path[2 + k];
            for (uint32_t k = lane; k < grp.y; k += 32) stk[len - 1 + k] = grp.x + k;
            sp = len - 1 + grp.y;
        }
    }
    __syncwarp();

    // forces of list entries [0, cnt) on every lane's own body.  With a
    // softening of at least 1e-20 a body's own entry adds exactly zero (its
    // offset is zero, its 1/r^3 finite), so only smaller softenings compare ids.
    const bool self_check = !(soft >= 1e-20f);
    // penetration of group body q with the leaf entry j (body id lj, radius
    // kept with the entry): a task when the distance is below the sum of the
    // radii and this body's index is the smaller (bh_force.comp:109-112)
    auto merge_test = [&](int q, uint32_t lj, float rx, float ry, float rz, float lr) {
        if (lj < N && actq[q] && lj != gq[q]) {
            const float rs = my_rad[q * 32 + lane] + lr;
            if (rx * rx + ry * ry + rz * rz < rs * rs) {
                const uint32_t bi = b.idx_in[gq[q]], oi = b.idx_in[lj];
                if (bi < oi) {
                    const uint32_t slot = atomicAdd(&b.mq->tail, 1u);
                    if (slot < N) {
                        b.mq->pairs[slot] = make_uint2(bi, oi);
                        b.mkeys[slot] = ((unsigned long long)gq[q] << 32) | seq[q * 32 + lane];
                        b.mslots[slot] = lj;
                    }
                    ++seq[q * 32 + lane];
                }
            }
        }
    };
    auto flush = [&](uint32_t cnt) {
        // body slots in use: slot q holds bodies 32 q .. 32 q + 31 of the
        // group, so slots at or above nq are empty in every lane
        const int nq = (int)((grp.y + 31u) >> 5);
        if (PREC || want_pot) {
            // the general loop: leaf terms apart (PREC), potential, self
            // check, merge tasks
#pragma unroll 2
            for (uint32_t j = 0; j < cnt; ++j) {
                const float4 c = lcm[j];
                const uint32_t lj = lid[j];
#pragma unroll
                for (int q = 0; q < GW_BPL; ++q) {
                    const float rx = c.x - pw[q].x, ry = c.y - pw[q].y, rz = c.z - pw[q].z;
                    if (merging) merge_test(q, lj, rx, ry, rz, lrad[j]);
                    const float rr = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmaf_rn(rx, rx, soft)));
                    const float inv = rsqrtf(rr);
                    const bool self = self_check && lj == gq[q];
                    const float f = self ? 0.0f : c.w * (inv * inv * inv);
                    const float ph = self ? 0.0f : -c.w * inv;
                    if (PREC && lj < N) {
                        kahan_add(nx_[q], cx_[q], f * rx);
                        kahan_add(ny_[q], cy_[q], f * ry);
                        kahan_add(nz_[q], cz_[q], f * rz);
                        if (want_pot) kahan_add(np_[q], cp_[q], ph);
                    } else {
                        ax[q] = __fmaf_rn(f, rx, ax[q]);
                        ay[q] = __fmaf_rn(f, ry, ay[q]);
                        az[q] = __fmaf_rn(f, rz, az[q]);
                        if (want_pot) pot[q] += ph;
                    }
                }
            }
        } else if (self_check) {
#pragma unroll 2
            for (uint32_t j = 0; j < cnt; ++j) {
                const float4 c = lcm[j];
                const uint32_t lj = lid[j];
#pragma unroll
                for (int q = 0; q < GW_BPL; ++q) {
                    const float rx = c.x - pw[q].x, ry = c.y - pw[q].y, rz = c.z - pw[q].z;
                    const float rr = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmaf_rn(rx, rx, soft)));
                    const float inv = rsqrtf(rr);
                    const float f = (lj == gq[q]) ? 0.0f : c.w * (inv * inv * inv);
                    ax[q] = __fmaf_rn(f, rx, ax[q]);
                    ay[q] = __fmaf_rn(f, ry, ay[q]);
                    az[q] = __fmaf_rn(f, rz, az[q]);
                }
            }
        } else {
            // one loop per number of slots in use (warp-uniform), unrolled
            // over a constant
            auto slots = [&](auto qn) {
                constexpr int Q = decltype(qn)::value;
#pragma unroll 2
                for (uint32_t j = 0; j < cnt; ++j) {
                    const float4 c = lcm[j];
#pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        const float rx = c.x - pw[q].x, ry = c.y - pw[q].y, rz = c.z - pw[q].z;
                        const float rr = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmaf_rn(rx, rx, soft)));
                        const float inv = rsqrtf(rr);
                        const float f = c.w * (inv * inv * inv);
                        ax[q] = __fmaf_rn(f, rx, ax[q]);
                        ay[q] = __fmaf_rn(f, ry, ay[q]);
                        az[q] = __fmaf_rn(f, rz, az[q]);
                    }
                }
            };
            if (nq >= GW_BPL)
                slots(std::integral_constant<int, GW_BPL>{});
            else if (GW_BPL > 3 && nq == 3)
                slots(std::integral_constant<int, (GW_BPL > 3 ? 3 : 1)>{});
            else if (nq == 2)
                slots(std::integral_constant<int, 2>{});
            else
                slots(std::integral_constant<int, 1>{});
        }
        if (merging && !(PREC || want_pot)) {
            // merge tests outside the force loop: lane j screens entry j with
            // the distance from the leaf to the group's box against its radius
            // plus the group's largest (with a margin for rounding); only the
            // leaves within reach get the per-body test, in list order
            const float3 bmn = MODE == GM_LEARNED ? S.geom[w].bmin : gg.bmin;
            const float3 bmx = MODE == GM_LEARNED ? S.geom[w].bmax : gg.bmax;
            for (uint32_t j0 = 0; j0 < cnt; j0 += 32) {
                bool near = false;
                if (j0 + lane < cnt && lid[j0 + lane] < N) {
                    const float4 c = lcm[j0 + lane];
                    const float dx = fmaxf(fmaxf(bmn.x - c.x, c.x - bmx.x), 0.0f);
                    const float dy = fmaxf(fmaxf(bmn.y - c.y, c.y - bmx.y), 0.0f);
                    const float dz = fmaxf(fmaxf(bmn.z - c.z, c.z - bmx.z), 0.0f);
                    const float reach = lrad[j0 + lane] + S.grp_rad[w];
                    near = dx * dx + dy * dy + dz * dz <= 1.001f * (reach * reach);
                }
                uint32_t m = __ballot_sync(0xffffffffu, near);
                while (m) {
                    const uint32_t j = j0 + __ffs(m) - 1;
                    m &= m - 1;
                    const float4 c = lcm[j];
                    const uint32_t lj = lid[j];
                    const float lr = lrad[j];
#pragma unroll
                    for (int q = 0; q < GW_BPL; ++q)
                        merge_test(q, lj, c.x - pw[q].x, c.y - pw[q].y, c.z - pw[q].z, lr);
                }
            }
        }
        inter += cnt;
    };
    // each lane's outcome: 1 list, 2 open (push children); warp-collective
    auto commit = [&](uint32_t kind, uint32_t id, float4 cm, uint32_t ca, uint32_t cb, float4 lo) {
        uint32_t bo = __ballot_sync(0xffffffffu, kind == 2);
        if (sp + 2 * __popc(bo) > (uint32_t)Cfg::stack) {
            // frontier full: accept instead of opening (less accurate, never wrong)
            saturated = true;
            if (kind == 2) kind = 1;
            bo = 0;
        }
        const uint32_t bl = __ballot_sync(0xffffffffu, kind == 1);
        if (kind == 1) {
            const uint32_t pos = ln + __popc(bl & lanemask_lt());
            if (PREC)
                lcm[pos] = make_float4((cm.x - gg.cx) + lo.x, (cm.y - gg.cy) + lo.y, (cm.z - gg.cz) + lo.z, G * cm.w);
            else
                lcm[pos] = make_float4(cm.x, cm.y, cm.z, G * cm.w);
            lid[pos] = id;
            if (merging) lrad[pos] = lo.x;  // the leaf's radius, read at the pop (0 for nodes)
        }
        ln += __popc(bl);
        if (kind == 2) {
            const uint32_t pos = sp + 2 * __popc(bo & lanemask_lt());
            stk[pos] = ca;
            stk[pos + 1] = cb;
        }
        sp += 2 * __popc(bo);
        opened += __popc(bo);
        __syncwarp();
        if (ln >= 32) {
            flush(32);
            ln -= 32;
            __syncwarp();
            if (lane < ln) {  // move the remaining entries to the front
                lcm[lane] = lcm[32 + lane];
                lid[lane] = lid[32 + lane];
                if (merging) lrad[lane] = lrad[32 + lane];
            }
            __syncwarp();
        }
    };

    // decide the first `cnt` (<= 32) queued band candidates with one MLP pass
    // and move the rest of the queue to the front
    auto decide_queue = [&](uint32_t cnt) {
        // features of queue rows [0, cnt), one per lane, then one MLP pass
        float feat[MAC_FEATURES];
#pragma unroll
        for (int q = 0; q < MAC_FEATURES; ++q) feat[q] = 0.0f;
        if (lane < cnt) {
            NodeGeom ng;
            ng.cm = S.pend_cm[w][lane];
            const float4 b0 = S.pend_b0[w][lane];
            const float4 b1 = S.pend_b1[w][lane];
            ng.bmin = make_float3(b0.x, b0.y, b0.z);
            ng.bmax = make_float3(b1.x, b1.y, b1.z);
            ng.count = __float_as_uint(b0.w);
            mac_features(S.geom[w], ng, feat);
        }
        mac_stage_features(mw, w, lane, feat);
        const float pred = mac_infer_warp(mw, w, lane);
        evals += cnt;
        // the row's node, read back after the network (fewer live registers)
        uint32_t kind = 0, id = 0, ca = 0, cb = 0;
        float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lane < cnt) {
            kind = pred < tol ? 1u : 2u;
            cm = S.pend_cm[w][lane];
            id = __float_as_uint(S.pend_b1[w][lane].w);
            const uint2 kids = S.pend_kids[w][lane];
            ca = kids.x;
            cb = kids.y;
        }
        const uint32_t rest = np - cnt;
        __syncwarp();
        if (lane < rest) {
            S.pend_cm[w][lane] = S.pend_cm[w][32 + lane];
            S.pend_b0[w][lane] = S.pend_b0[w][32 + lane];
            S.pend_b1[w][lane] = S.pend_b1[w][32 + lane];
            S.pend_kids[w][lane] = S.pend_kids[w][32 + lane];
        }
        np = rest;
        __syncwarp();
        commit(kind, id, cm, ca, cb, make_float4(0.f, 0.f, 0.f, 0.f));
    };

    while (sp > 0 || np > 0) {
        // the network decides the queue before a pop when the stack holds
        // fewer than GW_DECIDE_SP nodes and GW_DECIDE_NP or more rows wait:
        // its opened nodes refill the stack, so pops run fuller (a decision
        // does not depend on the batch)
        if (MODE == GM_LEARNED && (sp == 0 || (sp < GW_DECIDE_SP && np >= GW_DECIDE_NP))) {
            decide_queue(min(np, 32u));
            continue;
        }
        const uint32_t k = min(sp, 32u);
        sp -= k;
        const bool has = lane < k;
        const uint32_t id = has ? stk[sp + lane] : 0u;
        __syncwarp();
        uint32_t kind = 0;  // 0 nothing, 1 list, 2 open, 3 queued for the network
        float4 cm = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 qb0 = cm, qb1 = cm, lo = cm;
        uint32_t ca = 0, cb = 0, qcount = 0;
        if (has) {
            if (id < N) {
                cm = b.leaf_pm[id];
                if (PREC) lo = b.leaf_lo[id];
                if (merging) lo.x = b.leaf_rad[id];
                kind = 1;
            } else {
                const gbh_node* nd = &b.internal[id - N];
                const float4* q = reinterpret_cast<const float4*>(nd);
                cm = __ldg(q + 0);
                qb0 = __ldg(q + 1);
                qb1 = __ldg(q + 2);  // aabb4, aabb5, childA, childB
                ca = __float_as_uint(qb1.z);
                cb = __float_as_uint(qb1.w);
                qcount = __ldg(&nd->bodies_contained);
                NodeGeom ng;
                ng.cm = cm;
                ng.bmin = make_float3(qb0.x, qb0.y, qb0.z);
                ng.bmax = make_float3(qb0.w, qb1.x, qb1.y);
                ng.count = qcount;
                if (MODE == GM_LEARNED) {
                    // the network decides the band between a rule that is
                    // safe to accept (band_lo, default theta_g = 0.25) and one
                    // that must open (band_hi, default theta_g = 4): it never
                    // accepts a node the group reaches
                    const float rho = group_rho(S.geom[w], ng);  // shared copy: fewer live registers
                    kind = rho < band_lo ? 1u : rho < band_hi ? 3u : 2u;
                } else {
                    kind = group_theta_accept(gg, ng, theta) ? 1 : 2;
                    // training pairs: the band the network decides (see GM_LEARNED)
                    if (MODE == GM_RECORD && ng.count <= mw.rec_max_bodies &&
                        hash32(id ^ hash32(grp.x + mw.rec_seed)) <= mw.rec_keep &&
                        group_rho(gg, ng) < band_hi && !(group_rho(gg, ng) < band_lo)) {
                        const uint32_t slot = atomicAdd(mw.rec_count, 1u);
                        if (slot < mw.rec_cap) {
                            float f[MAC_FEATURES];
                            mac_features(gg, ng, f);
                            mw.rec_pairs[slot] = make_uint2(gi, id);
#pragma unroll
                            for (int q = 0; q < MAC_FEATURES; ++q) mw.rec_feats[(size_t)slot * MAC_FEATURES + q] = f[q];
                        }
                    }
                }
            }
        }
        if (MODE == GM_LEARNED) {
            // queue band candidates with their geometry; the network decides
            // them 32 at a time
            const uint32_t bq = __ballot_sync(0xffffffffu, kind == 3);
            if (kind == 3) {
                const uint32_t row = np + __popc(bq & lanemask_lt());
                S.pend_cm[w][row] = cm;
                S.pend_b0[w][row] = make_float4(qb0.x, qb0.y, qb0.z, __uint_as_float(qcount));
                S.pend_b1[w][row] = make_float4(qb0.w, qb1.x, qb1.y, __uint_as_float(id));
                S.pend_kids[w][row] = make_uint2(ca, cb);
                kind = 0;
            }
            np += __popc(bq);
            __syncwarp();
        } else {
            evals += __popc(__ballot_sync(0xffffffffu, has && id >= N));
        }
        commit(kind, id, cm, ca, cb, lo);
        if (MODE == GM_LEARNED && np >= 32) decide_queue(32);
    }
    if (ln) flush(ln);
    (void)saturated;

    // counters: interactions count the group's bodies for every list entry
    if (lane == 0) {
        atomicAdd(&b.st->interactions, (unsigned long long)inter * grp.y);
        atomicAdd(&b.st->mac_evals, (unsigned long long)evals);
        atomicAdd(&b.st->opened, (unsigned long long)opened);
    }
#pragma unroll
    for (int q = 0; q < GW_BPL; ++q) {
        if (!actq[q]) continue;
        // body index and position again (not kept live through the walk)
        const uint32_t bi = b.idx_in[gq[q]];
        const float4 pm = b.leaf_pm[gq[q]];
        float fx = ax[q], fy = ay[q], fz = az[q], fp = pot[q];
        if (PREC) {
            fx = fx + (nx_[q] - cx_[q]);
            fy = fy + (ny_[q] - cy_[q]);
            fz = fz + (nz_[q] - cz_[q]);
            fp = fp + (np_[q] - cp_[q]);
        }
        if (b.accel && (P->flags & GBH_FLAG_STORE_ACCEL)) b.accel[bi] = make_float4(fx, fy, fz, 0.0f);
        if (b.accel_mag) b.accel_mag[bi] = sqrtf(fx * fx + fy * fy + fz * fz);
        if (want_pot) b.potential[bi] = fp;
        const float4 vd = ld_vel_density(b.bodies_in, bi);
        if (PREC)
            walk_update_fp64(b, P, sim, gq[q], bi, pm, vd, fx, fy, fz);
        else
            walk_update(b, P, sim, gq[q], bi, pm, vd, fx, fy, fz);
    }
    __syncwarp();
    }  // groups
}

static size_t group_smem(int mode) {
    return mode == GM_LEARNED ? GroupCfg<GM_LEARNED>::smem : mode == GM_RECORD ? GroupCfg<GM_RECORD>::smem
                                                                              : GroupCfg<GM_THETA>::smem;
}

// resident blocks per SM of each instance (set up once per process)
static int g_blocks_per_sm[3][3];

template <int MODE, int FORM>
static void set_smem() {
    cudaFuncSetAttribute(k_walk_group<MODE, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)group_smem(MODE));
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_walk_group<MODE, FORM>, GroupShape<MODE>::threads,
                                                      group_smem(MODE)) !=
            cudaSuccess ||
        nb < 1)
        nb = 1;
    g_blocks_per_sm[MODE][FORM] = nb;
}

void group_walk_setup() {
    set_smem<GM_THETA, FORM_FP32>();
    set_smem<GM_THETA, FORM_PREC>();
    set_smem<GM_THETA, FORM_MERGE>();
    set_smem<GM_LEARNED, FORM_FP32>();
    set_smem<GM_LEARNED, FORM_PREC>();
    set_smem<GM_LEARNED, FORM_MERGE>();
    set_smem<GM_RECORD, FORM_FP32>();
}

template <int MODE, int FORM>
static void launch_mode(const StepBuffers& b, const MacDeviceWeights& mw, cudaStream_t s) {
    // the step's walks find the start lists built with the tree
    // (enqueue_build); the recording walk builds its own
    if (MODE == GM_RECORD) launch_group_paths(b, s);
    cudaMemsetAsync(&b.st->group_next, 0, 4, s);
    // persistent: the blocks that fit at once (no more than the groups need)
    constexpr uint32_t threads = GroupShape<MODE>::threads;
    const uint32_t need = (b.N + threads - 1) / threads + 1;
    uint32_t blocks = b.num_sms * (uint32_t)g_blocks_per_sm[MODE][FORM];
    if (blocks > need) blocks = need;
    k_walk_group<MODE, FORM><<<blocks, threads, group_smem(MODE), s>>>(b, mw);
}

template <int MODE>
static void launch_form(const StepBuffers& b, const MacDeviceWeights& mw, cudaStream_t s) {
    if (b.prec)
        launch_mode<MODE, FORM_PREC>(b, mw, s);
    else if (b.merge)
        launch_mode<MODE, FORM_MERGE>(b, mw, s);
    else
        launch_mode<MODE, FORM_FP32>(b, mw, s);
}

void launch_walk_group(const StepBuffers& b, const MacDeviceWeights& mw, bool learned, cudaStream_t s) {
    if (learned)
        launch_form<GM_LEARNED>(b, mw, s);
    else
        launch_form<GM_THETA>(b, mw, s);
}

// pairs name groups by their index in the build's group list
void launch_walk_group_record(const StepBuffers& b, const MacDeviceWeights& mw, cudaStream_t s) {
    launch_mode<GM_RECORD, FORM_FP32>(b, mw, s);
}
