// k_tree.cu — Karras LBVH build and single-pass bottom-up fill.
//
// Build: treeBuildBinaryRadixTreeKernel (SH/compute/tree/bh_tree.comp:43-133),
//   one thread per internal node, integer-exact.  It writes the topology into
//   compact arrays (children, counts, first slots, parents, arrival counters)
//   instead of the 80-byte nodes; the fill then writes every node whole, all
//   its words including the topology ones, so no sector of the node arrays is
//   written in part.  The stage entry point gbh_stage_build also writes the
//   reference's intermediate topology words into the nodes (k_build_nodes).
// Fill: treeInitLeafNodesKernel (bh_tree.comp:140-175) + 64 launches of
//   treePropagateNodesKernel (bh_tree.comp:183-259) become one kernel: each
//   leaf thread initialises its leaf and climbs; at every internal node an
//   atomic on readyChildren lets the second arriving child finish the node
//   (Karras 2012 / Apetrei 2014).  There is no pass limit, so trees taller
//   than 64 levels are filled completely, and the queue-reset race of the
//   reference (bh_tree.comp:188-193) does not exist.
#include "gbh_common.cuh"

// safeLCP, bh_tree.comp:20-37
__device__ __forceinline__ int safe_lcp(const uint64_t* __restrict__ keys, int n, int i, int j) {
    if (i < 0 || j < 0 || i >= n || j >= n) return -1;
    const uint64_t a = __ldg(keys + i), c = __ldg(keys + j);
    if (a == c) {
        const uint32_t x = (uint32_t)i ^ (uint32_t)j;
        return x == 0 ? 64 : 64 + __clz(x);
    }
    return __clzll(a ^ c);
}

// Body groups of the group walks: the subtrees of at most GBH_GROUP_MAX
// bodies whose parent holds more (every leaf lies in exactly one), as (first
// sorted slot, body count).  A group is a contiguous range of sorted slots,
// spatially compact because it is one tree node.  The build lists them: node
// i knows its children's ranges, so an internal node with more than
// GBH_GROUP_MAX bodies emits each child that holds at most that many; one
// counter update per warp.
__device__ __forceinline__ void emit_groups(const StepBuffers& b, uint32_t k, const uint2 (&mine)[2],
                                            const uint32_t (&node)[2]) {
    const uint32_t lane = lane_id();
    uint32_t incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(&b.st->num_groups, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    const uint32_t first = base + incl - k;
    for (uint32_t q = 0; q < k; ++q) {
        b.groups[first + q] = mine[q];
        b.group_node[first + q] = node[q];
    }
}

__global__ __launch_bounds__(256) void k_build(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t* keys = b.keys_in;
    if (n <= 1) {
        if (n == 1 && gid == 0) {
            // single body, bh_tree.comp:46-62: root with one child, bodiesContained 0,
            // readyChildren 1
            b.topo_kids[0] = make_uint2(0u, GBH_NONE);
            b.topo_cnt[0] = 0;
            b.node_lo[0] = 0;
            b.fill_ready[0] = 1;
            b.parent_int[0] = GBH_NONE;
            b.parent_leaf[0] = N;
            b.groups[0] = make_uint2(0u, 1u);
            b.group_node[0] = N;
            b.st->num_groups = 1;
        }
        return;
    }
    // every lane of a warp reaches the group list below
    uint2 mine[2];
    uint32_t mine_node[2] = {0u, 0u};
    uint32_t k = 0;
    if (gid < n - 1) {
    const int i = (int)gid, ni = (int)n;
    const int lcp_r = safe_lcp(keys, ni, i, i + 1);
    const int lcp_l = safe_lcp(keys, ni, i, i - 1);
    const int d = (lcp_l > lcp_r) ? -1 : 1;
    const int delta_min = safe_lcp(keys, ni, i, i - d);
    int lmax = 2;
    while (safe_lcp(keys, ni, i, i + d * lmax) > delta_min) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t > 0; t /= 2)
        if (safe_lcp(keys, ni, i, i + d * (l + t)) > delta_min) l += t;
    const int j = i + l * d;
    const int delta_node = safe_lcp(keys, ni, i, j);
    int s = 0;
    int t = l;
    while (t > 1) {
        t = (t + 1) / 2;
        if (safe_lcp(keys, ni, i, i + (s + t) * d) > delta_node) s += t;
    }
    const int gamma = i + s * d + min(d, 0);
    const int mn = min(i, j), mx = max(i, j);
    const uint32_t left = (mn == gamma) ? (uint32_t)gamma : (uint32_t)gamma + N;
    const uint32_t right = (mx == gamma + 1) ? (uint32_t)(gamma + 1) : (uint32_t)(gamma + 1) + N;
    b.topo_kids[i] = make_uint2(left, right);
    b.node_lo[i] = (uint32_t)mn;
    b.topo_cnt[i] = (uint32_t)(mx - mn + 1);
    b.fill_ready[i] = 0;
    const uint32_t self = (uint32_t)i + N;
    if (left < N) b.parent_leaf[left] = self; else b.parent_int[left - N] = self;
    if (right < N) b.parent_leaf[right] = self; else b.parent_int[right - N] = self;
    if (i == 0) b.parent_int[0] = GBH_NONE;
    const uint32_t cnt = (uint32_t)(mx - mn + 1);
    if (cnt > GBH_GROUP_MAX) {
        const uint32_t cl = (uint32_t)(gamma - mn + 1), cr = (uint32_t)(mx - gamma);
        if (cl <= GBH_GROUP_MAX) {
            mine_node[k] = left;
            mine[k++] = make_uint2((uint32_t)mn, cl);
        }
        if (cr <= GBH_GROUP_MAX) {
            mine_node[k] = right;
            mine[k++] = make_uint2((uint32_t)gamma + 1u, cr);
        }
    } else if (i == 0) {
        mine_node[k] = N;
        mine[k++] = make_uint2(0u, cnt);  // the whole tree is one group
    }
    }
    emit_groups(b, k, mine, mine_node);
}

// The reference's Node topology words after buildBinaryRadixTree (childA/B,
// nodeDepth = min(i, j), bodiesContained, readyChildren = 0, parentId; leaves:
// parentId), for the stage-level API.
__global__ void k_build_nodes(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (n == 0) return;
    const uint32_t ni = n > 1 ? n - 1 : 1;
    if (t < ni) {
        gbh_node* nd = &b.internal[t];
        const uint2 k = b.topo_kids[t];
        nd->child_a = k.x;
        nd->child_b = k.y;
        nd->node_depth = b.node_lo[t];
        nd->bodies_contained = b.topo_cnt[t];
        nd->ready_children = b.fill_ready[t];
        nd->parent_id = b.parent_int[t];
    }
    if (t < n) b.leaf[t].parent_id = b.parent_leaf[t];
}

void launch_build_nodes(const StepBuffers& b, cudaStream_t s) {
    k_build_nodes<<<(b.N + 255) / 256, 256, 0, s>>>(b);
}

// Where each group's walk starts: the group's own subtree and the sibling of
// every ancestor of it, which together hold every body once.  A walk from the
// root opens each ancestor of the group anyway (its box holds the group's
// bodies), one level per round of candidates; starting from this list gives
// the same accepted and listed nodes without those rounds.  One thread per
// group climbs the parent links; a group deeper than GBH_PATH_WORDS - 2
// levels, or past the list's capacity, starts from the root (count 0).
__global__ __launch_bounds__(256) void k_group_paths(StepBuffers b) {
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ng = min(b.st->num_groups, b.group_path_cap);
    if (gi >= ng) return;
    const uint32_t N = b.N, root = N;
    uint32_t* out = b.group_path + (size_t)gi * GBH_PATH_WORDS;
    uint32_t node = b.group_node[gi];
    uint32_t len = 0;
    out[1 + len++] = node;
    while (node != root && len < GBH_PATH_WORDS - 1) {
        const uint32_t p = node < N ? b.parent_leaf[node] : b.parent_int[node - N];
        if (p < N || p - N >= N) {  // not an internal node: leave the group to the root start
            len = 0;
            break;
        }
        const uint2 kids = b.topo_kids[p - N];
        out[1 + len++] = kids.x == node ? kids.y : kids.x;
        node = p;
    }
    if (node != root) len = 0;
    out[0] = len;
}

void launch_group_paths(const StepBuffers& b, cudaStream_t s) {
    // the groups of the step are counted on the device: enough threads for
    // the list's capacity, the surplus returns at once
    const uint32_t threads = min(b.N, b.group_path_cap);
    k_group_paths<<<(threads + 255) / 256, 256, 0, s>>>(b);
}

void launch_build(const StepBuffers& b, cudaStream_t s) {
    const uint32_t nodes = b.N > 1 ? b.N - 1 : 1;
    cudaMemsetAsync(&b.st->num_groups, 0, 4, s);
    k_build<<<(nodes + 255) / 256, 256, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// getStarColor, common.glsl:232-276
__device__ void star_color(float mass, float density, float rgb[3]) {
    const float e = 0.875f - 1.0f / 6.0f;
    float t = 5.95589e-19f * powf(mass, e);
    t = t * powf(density, 1.0f / 6.0f);
    const float temp = t / 100.0f;
    float r, g, bl;
    if (temp <= 66.0f) {
        r = 255.0f;
    } else {
        r = 329.698727446f * powf(temp - 60.0f, -0.1332047592f);
    }
    if (temp <= 66.0f) {
        g = 99.4708025861f * logf(gmax(temp, 1e-3f)) - 161.1195681661f;
    } else {
        g = 288.1221695283f * powf(temp, -0.0755148492f);
    }
    if (temp >= 66.0f) {
        bl = 255.0f;
    } else {
        bl = 138.5177312231f * logf(gmax(temp - 10.0f, 1e-3f)) - 305.0447927307f;
    }
    rgb[0] = gclamp(r, 0.0f, 255.0f) / 255.0f;
    rgb[1] = gclamp(g, 0.0f, 255.0f) / 255.0f;
    rgb[2] = gclamp(bl, 0.0f, 255.0f) / 255.0f;
}

struct NodeVals {
    float4 cm;
    float box[6];
    float4 col;
    uint32_t depth;
};

// L2-coherent read of the fields of a node written by another thread of this kernel
__device__ __forceinline__ NodeVals load_node_cg(const gbh_node* nd) {
    NodeVals v;
    const float4* p = reinterpret_cast<const float4*>(nd);
    v.cm = __ldcg(p + 0);
    const float4 a = __ldcg(p + 1);
    const float2 c = __ldcg(reinterpret_cast<const float2*>(p + 2));  // aabb4, aabb5
    v.depth = __ldcg(reinterpret_cast<const uint32_t*>(p + 3));
    v.col = __ldcg(p + 4);
    v.box[0] = a.x;
    v.box[1] = a.y;
    v.box[2] = a.z;
    v.box[3] = a.w;
    v.box[4] = c.x;
    v.box[5] = c.y;
    return v;
}

__device__ __forceinline__ float half_side(const float box[6]) {
    const float ex = box[3] - box[0], ey = box[4] - box[1], ez = box[5] - box[2];
    return gmax(ex, gmax(ey, ez)) / 2.0f;
}

__device__ __forceinline__ WalkRec make_rec(const NodeVals& v, uint32_t id, uint32_t count, bool leaf) {
    WalkRec r;
    r.cm = v.cm;
    r.half_side = leaf ? 0.0f : half_side(v.box);
    r.id = id;
    r.count = count;
    r.pad = 0;
    return r;
}

// One internal node from its two children (bh_tree.comp:223-246); L is
// childA's values, R childB's.
__device__ __forceinline__ NodeVals combine(const NodeVals& L, const NodeVals& R) {
    const float lw = L.cm.w, rw = R.cm.w;
    const float M = lw + rw;
    NodeVals out;
    if (M > 0.0f) {
        out.cm.x = (lw * L.cm.x + rw * R.cm.x) / M;
        out.cm.y = (lw * L.cm.y + rw * R.cm.y) / M;
        out.cm.z = (lw * L.cm.z + rw * R.cm.z) / M;
        // the colour (render-only, compared with a tolerance) by one reciprocal
        const float inv_m = 1.0f / M;
        out.col.x = (lw * L.col.x + rw * R.col.x) * inv_m;
        out.col.y = (lw * L.col.y + rw * R.col.y) * inv_m;
        out.col.z = (lw * L.col.z + rw * R.col.z) * inv_m;
    } else {
        out.cm.x = (L.cm.x + R.cm.x) * 0.5f;
        out.cm.y = (L.cm.y + R.cm.y) * 0.5f;
        out.cm.z = (L.cm.z + R.cm.z) * 0.5f;
        out.col.x = (L.col.x + R.col.x) * 0.5f;
        out.col.y = (L.col.y + R.col.y) * 0.5f;
        out.col.z = (L.col.z + R.col.z) * 0.5f;
    }
    out.cm.w = M;
    out.col.w = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        out.box[k] = gmin(L.box[k], R.box[k]);
        out.box[3 + k] = gmax(L.box[3 + k], R.box[3 + k]);
    }
    out.depth = 1u + max(L.depth, R.depth);
    return out;
}

// Write a finished internal node whole: its Node words (reference layout,
// common.glsl:40-58) including the topology ones, readyChildren claimed
// (0xFFFFFFFF, bh_tree.comp:200), and, for the plain walk, the walk records
// of its two children.
__device__ __forceinline__ void store_internal(const StepBuffers& b, uint32_t i, const NodeVals& out, const NodeVals& L,
                                               const NodeVals& R, uint32_t a_id, uint32_t b_id, uint32_t a_count,
                                               uint32_t b_count, uint32_t bodies, uint32_t parent) {
    float4* np = reinterpret_cast<float4*>(&b.internal[i]);
    __stcg(np + 0, out.cm);
    __stcg(np + 1, make_float4(out.box[0], out.box[1], out.box[2], out.box[3]));
    __stcg(reinterpret_cast<uint4*>(np + 2), make_uint4(__float_as_uint(out.box[4]), __float_as_uint(out.box[5]), a_id, b_id));
    __stcg(reinterpret_cast<uint4*>(np + 3), make_uint4(out.depth, bodies, GBH_NONE, parent));
    __stcg(np + 4, out.col);
    // the children's walk records feed the plain walk only
    if (b.params->mac_mode == GBH_MAC_PLAIN) {
        ChildPair pr;
        pr.a = make_rec(L, a_id, a_count, a_id < b.N);
        pr.b = make_rec(R, b_id, b_count, b_id < b.N);
        b.pairs[i] = pr;
    }
}

// Node values kept in shared memory by the tiled fill (64 bytes)
struct TileVals {
    float4 cm;
    float4 col;
    float4 box03;
    float box4, box5;
    uint32_t depth, pad;
};

__device__ __forceinline__ TileVals to_tile(const NodeVals& v) {
    TileVals t;
    t.cm = v.cm;
    t.col = v.col;
    t.box03 = make_float4(v.box[0], v.box[1], v.box[2], v.box[3]);
    t.box4 = v.box[4];
    t.box5 = v.box[5];
    t.depth = v.depth;
    t.pad = 0;
    return t;
}

__device__ __forceinline__ NodeVals from_tile(const TileVals& t) {
    NodeVals v;
    v.cm = t.cm;
    v.col = t.col;
    v.box[0] = t.box03.x;
    v.box[1] = t.box03.y;
    v.box[2] = t.box03.z;
    v.box[3] = t.box03.w;
    v.box[4] = t.box4;
    v.box[5] = t.box5;
    v.depth = t.depth;
    return v;
}

// block-scope release/acquire add on a shared-memory counter
__device__ __forceinline__ uint32_t atomic_add_acq_rel_cta(uint32_t* p, uint32_t v) {
    uint32_t old;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;" : "=r"(old) : "r"(a), "r"(v) : "memory");
    return old;
}

#ifndef FILL_TILE
#define FILL_TILE 512
#endif

// Tiled fill.  Block k owns the sorted slots [k T, k T + T) (T = FILL_TILE).
// Phase 1: every thread initialises its leaf and keeps its values in shared
// memory.  Phase 2: the leaf threads climb while the node's leaf range lies
// inside the tile; the second child to arrive (a shared-memory counter)
// combines the children from shared memory.  A thread whose next node crosses
// a tile boundary hands its node to k_fill_top through a frontier list and
// ends, so no block waits on a long climb.  The arithmetic of a node depends
// only on its two children, so the result is the same in any schedule.
__global__ __launch_bounds__(FILL_TILE) void k_fill(StepBuffers b) {
    extern __shared__ __align__(16) unsigned char fill_smem[];
    TileVals* s_leaf = reinterpret_cast<TileVals*>(fill_smem);  // [FILL_TILE]
    TileVals* s_node = s_leaf + FILL_TILE;                       // [FILL_TILE]
    uint4* s_topo = reinterpret_cast<uint4*>(s_node + FILL_TILE);  // childA, childB, first slot, bodies
    uint32_t* s_parent = reinterpret_cast<uint32_t*>(s_topo + FILL_TILE);
    uint32_t* s_ready = s_parent + FILL_TILE;  // arrival counters of the tile's internal nodes
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t base = blockIdx.x * FILL_TILE;
    const uint32_t t = threadIdx.x;
    const uint32_t g = base + t;
    if (base >= n) return;
    const gbh_sim_values* sim = b.sim;
    s_ready[t] = 0u;
    if (g + 1 < n) {
        // topology of internal node g (written by the build), read once
        const uint2 kids = b.topo_kids[g];
        s_topo[t] = make_uint4(kids.x, kids.y, b.node_lo[g], b.topo_cnt[g]);
        s_parent[t] = b.parent_int[g];
    }
    NodeVals own;
    uint32_t parent0 = GBH_NONE;
    if (g < n) {
        const uint32_t bi = b.idx_in[g];
        const float4 pm = ld_pos_mass(b.bodies_in, bi);
        const float4 vd = ld_vel_density(b.bodies_in, bi);
        // leaf init, bh_tree.comp:153-166
        gbh_node* lf = &b.leaf[g];
        float4* lp = reinterpret_cast<float4*>(lf);
        parent0 = b.parent_leaf[g];
        own.cm = pm;
        own.box[0] = own.box[3] = pm.x;
        own.box[1] = own.box[4] = pm.y;
        own.box[2] = own.box[5] = pm.z;
        own.col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        own.depth = 0;
        if (pm.w > 0.0f && vd.w > 0.0f) {
            float rgb[3];
            star_color(pm.w * sim->unit_mass, vd.w * sim->unit_density, rgb);
            own.col = make_float4(rgb[0], rgb[1], rgb[2], 0.0f);
        }
        lp[0] = pm;
        lp[1] = make_float4(pm.x, pm.y, pm.z, pm.x);
        reinterpret_cast<uint4*>(lp)[2] = make_uint4(__float_as_uint(pm.y), __float_as_uint(pm.z), GBH_NONE, GBH_NONE);
        reinterpret_cast<uint4*>(lp)[3] = make_uint4(0u, 0u, GBH_NONE, parent0);
        lp[4] = own.col;
        b.leaf_pm[g] = pm;
        if (b.params->merging_collision_or_neither != GBH_MODE_NEITHER)
            b.leaf_rad[g] = body_radius(sim->body_length_constant, pm.w, vd.w);
        if (b.prec) {
            // precision form: the FP32 residual of the FP64 position
            const double2 xy = reinterpret_cast<const double2*>(b.pos64_in)[2 * (size_t)bi];
            const double z = b.pos64_in[4 * (size_t)bi + 2];
            b.leaf_lo[g] = make_float4((float)(xy.x - (double)pm.x), (float)(xy.y - (double)pm.y),
                                       (float)(z - (double)pm.z), 0.0f);
        }
        s_leaf[t] = to_tile(own);
    }
    __syncthreads();
    if (g >= n) return;
    const uint32_t tile_end = min(base + FILL_TILE, n);

    uint32_t self = g;  // global id of the node whose values are in `own`
    uint32_t self_count = 1;
    uint32_t node = parent0;
    // phase 2: nodes inside the tile (never for a single-body tree, whose root
    // has one child)
    while (n > 1 && node != GBH_NONE) {
        const uint32_t i = node - N;
        if (i < base || i >= tile_end) break;
        const uint4 topo = s_topo[i - base];  // childA, childB, first slot, bodies
        if (topo.z < base || topo.z + topo.w > tile_end) break;
        if (atomic_add_acq_rel_cta(&s_ready[i - base], 1u) == 0u) return;
        const bool self_is_a = topo.x == self;
        const uint32_t sib = self_is_a ? topo.y : topo.x;
        // the sibling lies inside the tile too
        uint32_t sib_count = 1;
        NodeVals S;
        if (sib < N) {
            S = from_tile(s_leaf[sib - base]);
        } else {
            S = from_tile(s_node[sib - N - base]);
            sib_count = s_topo[sib - N - base].w;
        }
        const NodeVals& L = self_is_a ? own : S;
        const NodeVals& R = self_is_a ? S : own;
        const NodeVals out = combine(L, R);
        const uint32_t a_id = self_is_a ? self : sib, b_id = self_is_a ? sib : self;
        store_internal(b, i, out, L, R, a_id, b_id, self_is_a ? self_count : sib_count,
                       self_is_a ? sib_count : self_count, topo.w, s_parent[i - base]);
        s_node[i - base] = to_tile(out);
        self = node;
        self_count += sib_count;
        own = out;
        node = s_parent[i - base];
        if (node == GBH_NONE) {
            b.st->tree_height = out.depth;
            *b.root_rec = make_rec(out, self, self_count, false);
            return;
        }
    }
    // the next node crosses a tile boundary: hand over
    if (node != GBH_NONE) {
        const uint32_t slot = atomicAdd(&b.st->fill_frontier, 1u);
        if (slot < b.fill_frontier_cap)
            b.fill_frontier[slot] = make_uint2(self, self_count);
        else
            set_error(b.st, GBH_DEVERR_FILL_SPIN);
    }
}

// Climb from node `self` (values `own`, `self_count` bodies) through the
// global counters readyChildren (release/acquire at GPU scope): the second
// arriving child reads its sibling from L2 and finishes the node.
__device__ void climb_global(const StepBuffers& b, uint32_t self, uint32_t self_count, NodeVals own,
                             uint32_t node) {
    const uint32_t N = b.N;
    while (node != GBH_NONE) {
        const uint32_t i = node - N;
        // release: own node's writes before the count; acquire: the sibling's writes after it
        const uint32_t old = atomic_add_acq_rel(&b.fill_ready[i], 1u);
        if (old == 0u) return;
        const uint2 kids = b.topo_kids[i];
        const bool self_is_a = kids.x == self;
        const uint32_t sib = self_is_a ? kids.y : kids.x;
        NodeVals S;
        uint32_t sib_count = 1;
        if (sib == GBH_NONE) {  // single-body tree: the missing child contributes nothing
            S.cm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            S.col = S.cm;
            S.box[0] = S.box[1] = S.box[2] = 1e38f;
            S.box[3] = S.box[4] = S.box[5] = -1e38f;
            S.depth = 0;
            sib_count = 0;
        } else if (sib < N) {
            S = load_node_cg(&b.leaf[sib]);
        } else {
            S = load_node_cg(&b.internal[sib - N]);
            sib_count = b.topo_cnt[sib - N];
        }
        const NodeVals& L = self_is_a ? own : S;
        const NodeVals& R = self_is_a ? S : own;
        const NodeVals out = combine(L, R);
        const uint32_t a_id = self_is_a ? self : sib, b_id = self_is_a ? sib : self;
        const uint32_t parent = b.parent_int[i];
        store_internal(b, i, out, L, R, a_id, b_id, self_is_a ? self_count : sib_count,
                       self_is_a ? sib_count : self_count, b.topo_cnt[i], parent);
        self = node;
        self_count = self_count + sib_count;
        own = out;
        if (parent == GBH_NONE) {
            b.st->tree_height = out.depth;
            *b.root_rec = make_rec(out, node, self_count, false);
            return;
        }
        node = parent;
    }
}

// Top-tree fill: the nodes that cross tile boundaries (about 2 N / FILL_TILE),
// climbing from the frontier the tiled fill left.
__global__ __launch_bounds__(256) void k_fill_top(StepBuffers b) {
    const uint32_t count = min(b.st->fill_frontier, b.fill_frontier_cap);
    const uint32_t N = b.N;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
        const uint2 fr = b.fill_frontier[e];
        const gbh_node* nd = fr.x < N ? &b.leaf[fr.x] : &b.internal[fr.x - N];
        climb_global(b, fr.x, fr.y, load_node_cg(nd), fr.x < N ? b.parent_leaf[fr.x] : b.parent_int[fr.x - N]);
    }
}

#define FILL_SMEM (FILL_TILE * (2 * sizeof(TileVals) + sizeof(uint4) + 2 * sizeof(uint32_t)))

void fill_setup() {
    cudaFuncSetAttribute(k_fill, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FILL_SMEM);
}

void launch_fill(const StepBuffers& b, cudaStream_t s) {
    k_fill<<<(b.N + FILL_TILE - 1) / FILL_TILE, FILL_TILE, FILL_SMEM, s>>>(b);
    k_fill_top<<<b.num_sms * 4, 256, 0, s>>>(b);
}
