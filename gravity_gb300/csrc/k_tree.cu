// k_tree.cu — Karras LBVH build and single-pass bottom-up fill.
//
// Build: treeBuildBinaryRadixTreeKernel (SH/compute/tree/bh_tree.comp:43-133),
//   one thread per internal node, integer-exact.  Like the reference it writes
//   the topology words (childA/B, parentId, bodiesContained, nodeDepth =
//   min(i, j), readyChildren = 0); the COM/AABB/colour words it also zeroes are
//   rewritten by the fill before anything reads them, so they are not written.
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

__global__ __launch_bounds__(256) void k_build(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t* keys = b.keys_in;
    if (n <= 1) {
        if (n == 1 && gid == 0) {
            // single body, bh_tree.comp:46-62
            gbh_node* r = &b.internal[0];
            r->child_a = 0;
            r->child_b = GBH_NONE;
            r->ready_children = 1;
            r->node_depth = 0;
            r->bodies_contained = 0;
            r->parent_id = GBH_NONE;
            b.leaf[0].parent_id = N;
        }
        return;
    }
    if (gid >= n - 1) return;
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
    gbh_node* nd = &b.internal[i];
    // words @40..@59: childA, childB, nodeDepth, bodiesContained, readyChildren
    nd->child_a = left;
    nd->child_b = right;
    nd->node_depth = (uint32_t)mn;
    nd->bodies_contained = (uint32_t)(mx - mn + 1);
    nd->ready_children = 0;
    const uint32_t self = (uint32_t)i + N;
    if (left < N) b.leaf[left].parent_id = self; else b.internal[left - N].parent_id = self;
    if (right < N) b.leaf[right].parent_id = self; else b.internal[right - N].parent_id = self;
    if (i == 0) nd->parent_id = GBH_NONE;
}

void launch_build(const StepBuffers& b, cudaStream_t s) {
    const uint32_t nodes = b.N > 1 ? b.N - 1 : 1;
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

// L2-coherent read of a node written by another thread of this kernel
__device__ __forceinline__ NodeVals load_node_cg(const gbh_node* nd) {
    NodeVals v;
    const float4* p = reinterpret_cast<const float4*>(nd);
    v.cm = __ldcg(p + 0);
    const float4 a = __ldcg(p + 1);
    const float4 c = __ldcg(p + 2);  // aabb4, aabb5, childA, childB
    const uint4 e = __ldcg(reinterpret_cast<const uint4*>(p + 3));
    v.col = __ldcg(p + 4);
    v.box[0] = a.x;
    v.box[1] = a.y;
    v.box[2] = a.z;
    v.box[3] = a.w;
    v.box[4] = c.x;
    v.box[5] = c.y;
    v.depth = e.x;
    return v;
}

__global__ __launch_bounds__(256) void k_fill(StepBuffers b) {
    const uint32_t n = b.st->n_new;
    const uint32_t N = b.N;
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const gbh_sim_values* sim = b.sim;
    const uint32_t bi = b.idx_in[g];
    const float4 pm = ld_pos_mass(b.bodies_in, bi);
    const float4 vd = ld_vel_density(b.bodies_in, bi);
    // leaf init, bh_tree.comp:153-166
    gbh_node* lf = &b.leaf[g];
    float4* lp = reinterpret_cast<float4*>(lf);
    const uint32_t parent0 = lf->parent_id;
    lp[0] = pm;
    lp[1] = make_float4(pm.x, pm.y, pm.z, pm.x);
    reinterpret_cast<uint4*>(lp)[2] = make_uint4(__float_as_uint(pm.y), __float_as_uint(pm.z), GBH_NONE, GBH_NONE);
    reinterpret_cast<uint4*>(lp)[3] = make_uint4(0u, 0u, GBH_NONE, parent0);
    float4 col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (pm.w > 0.0f && vd.w > 0.0f) {
        float rgb[3];
        star_color(pm.w * sim->unit_mass, vd.w * sim->unit_density, rgb);
        col = make_float4(rgb[0], rgb[1], rgb[2], 0.0f);
    }
    lp[4] = col;
    b.leaf_pm[g] = pm;
    if (b.params->merging_collision_or_neither != GBH_MODE_NEITHER)
        b.leaf_rad[g] = body_radius(sim->body_length_constant, pm.w, vd.w);

    // climb
    uint32_t node = parent0;
    while (node != GBH_NONE) {
        const uint32_t i = node - N;
        gbh_node* nd = &b.internal[i];
        __threadfence();
        const uint32_t old = atomicAdd(&nd->ready_children, 1u);
        if (old == 0u) return;  // first child to arrive; the sibling finishes this node
        __threadfence();
        const uint32_t ca = nd->child_a, cb = nd->child_b;
        NodeVals L = load_node_cg(ca < N ? &b.leaf[ca] : &b.internal[ca - N]);
        NodeVals R;
        if (cb == GBH_NONE) {  // single-body tree: the missing child contributes nothing
            R.cm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            R.col = R.cm;
            R.box[0] = R.box[1] = R.box[2] = 1e38f;
            R.box[3] = R.box[4] = R.box[5] = -1e38f;
            R.depth = 0;
        } else {
            R = load_node_cg(cb < N ? &b.leaf[cb] : &b.internal[cb - N]);
        }
        // bh_tree.comp:223-246
        const float lw = L.cm.w, rw = R.cm.w;
        const float M = lw + rw;
        float c[3], a[3];
        const float lc[3] = {L.cm.x, L.cm.y, L.cm.z}, rc[3] = {R.cm.x, R.cm.y, R.cm.z};
        const float la[3] = {L.col.x, L.col.y, L.col.z}, ra[3] = {R.col.x, R.col.y, R.col.z};
        if (M > 0.0f) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                c[k] = (lw * lc[k] + rw * rc[k]) / M;
                a[k] = (lw * la[k] + rw * ra[k]) / M;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                c[k] = (lc[k] + rc[k]) * 0.5f;
                a[k] = (la[k] + ra[k]) * 0.5f;
            }
        }
        float box[6];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            box[k] = gmin(L.box[k], R.box[k]);
            box[3 + k] = gmax(L.box[3 + k], R.box[3 + k]);
        }
        const uint32_t depth = 1u + max(L.depth, R.depth);
        float4* np = reinterpret_cast<float4*>(nd);
        __stcg(np + 0, make_float4(c[0], c[1], c[2], M));
        __stcg(np + 1, make_float4(box[0], box[1], box[2], box[3]));
        __stcg(reinterpret_cast<float2*>(np + 2), make_float2(box[4], box[5]));
        nd->node_depth = depth;
        nd->ready_children = GBH_NONE;
        __stcg(np + 4, make_float4(a[0], a[1], a[2], 0.0f));
        // walk record, getLongestSide: bh_force.comp:14-20
        const float ex = box[3] - box[0], ey = box[4] - box[1], ez = box[5] - box[2];
        const float half = gmax(ex, gmax(ey, ez)) / 2.0f;
        WalkNode wn;
        wn.cm = make_float4(c[0], c[1], c[2], M);
        wn.half_side = half;
        wn.child_a = ca;
        wn.child_b = cb;
        wn.count = nd->bodies_contained;
        b.wnode[i] = wn;
        const uint32_t parent = nd->parent_id;
        if (parent == GBH_NONE) {
            b.st->tree_height = depth;
            return;
        }
        node = parent;
    }
}

void launch_fill(const StepBuffers& b, cudaStream_t s) { k_fill<<<(b.N + 255) / 256, 256, 0, s>>>(b); }
