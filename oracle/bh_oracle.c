/*
 * bh_oracle.c — CPU oracle of the gkane1234/gravity Barnes–Hut step.
 *
 * TEST INFRASTRUCTURE ONLY (see bh_oracle.h).  Every function cites the
 * reference GLSL / Java it restates; paths are inside the reference project,
 * SH = src/main/resources/shaders, J = src/main/java/com/grumbo.
 *
 * Compile with -ffp-contract=off: the restatement is defined as IEEE FP32 with
 * one rounding per GLSL operation, evaluated left to right.
 */
#include "bh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NONE_ID 0xFFFFFFFFu
#define MAX_VALUE_21 2097151.0f

struct orc_ctx {
    uint32_t N;
    gbh_sim_values sim;
    gbh_body* bodies[2];
    int bin; /* bodies[bin] is BodiesIn */
    uint64_t* morton[2];
    uint32_t* index[2];
    int iin; /* morton[iin]/index[iin] are MortonIn/IndexIn */
    gbh_node* leaf;
    gbh_node* internal;
    uint32_t mtail;
    uint32_t* mtasks;   /* pairs, emission order */
    uint64_t* mkeys;    /* (sorted slot << 32) | per-body sequence, for ordering */
    uint32_t mcap;
    float* accel;       /* float4 per body index */
    int store_accel;
    uint64_t opened;
    uint64_t interactions;
    uint32_t died;
    uint32_t oob_step;
    uint32_t merged;
    uint32_t tree_height;
    int inited;
};

static int g_threads = 0;

void orc_set_threads(int threads) {
    g_threads = threads;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- GLSL built-in semantics (GLSL 4.30 §8) ------------------------------ */
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
static inline float gdot3(const float a[3], const float b[3]) {
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}
static inline float ginversesqrt(float x) { return 1.0f / sqrtf(x); }
static inline int finite3(const float v[3]) {
    for (int k = 0; k < 3; ++k)
        if (isnan(v[k]) || isinf(v[k])) return 0;
    return 1;
}

/* ---- units: common.glsl:346-360 ------------------------------------------ */
static void update_units(orc_ctx* c, const gbh_units* u) {
    c->sim.unit_mass = u->mass;
    c->sim.unit_density = u->density;
    c->sim.unit_len = u->len;
    c->sim.unit_time = u->time;
    if (u->camera_scale != 0.0f) c->sim.camera_scale = u->camera_scale;
    if (u->gravitational_constant > 0.0f) {
        c->sim.gravitational_constant = u->gravitational_constant;
    } else {
        float g = 6.67430e-11f * powf(u->len, -3.0f);
        g = g * powf(u->time, 2.0f);
        g = g * powf(u->mass, 1.0f);
        c->sim.gravitational_constant = g;
    }
    c->sim.body_length_constant = 0.6203504909f * powf(u->mass / u->density, 1.0f / 3.0f) / u->len;
}

/* ---- star colour: common.glsl:232-276 ------------------------------------ */
static float star_temp(float mass, float density) {
    const float constant = 5.95589e-19f;
    float e = 0.875f - 1.0f / 6.0f;
    float t = constant * powf(mass, e);
    return t * powf(density, 1.0f / 6.0f);
}

void orc_star_color(float mass, float density, float rgb[3]) {
    float temp = star_temp(mass, density) / 100.0f;
    float r, g, b;
    if (temp <= 66.0f) {
        r = 255.0f;
    } else {
        r = temp - 60.0f;
        r = 329.698727446f * powf(r, -0.1332047592f);
    }
    if (temp <= 66.0f) {
        g = 99.4708025861f * logf(gmax(temp, 1e-3f)) - 161.1195681661f;
    } else {
        g = temp;
        g = 288.1221695283f * powf(g, -0.0755148492f);
    }
    if (temp >= 66.0f) {
        b = 255.0f;
    } else {
        b = temp - 10.0f;
        b = 138.5177312231f * logf(gmax(b, 1e-3f)) - 305.0447927307f;
    }
    rgb[0] = gclamp(r, 0.0f, 255.0f) / 255.0f;
    rgb[1] = gclamp(g, 0.0f, 255.0f) / 255.0f;
    rgb[2] = gclamp(b, 0.0f, 255.0f) / 255.0f;
}

/* radius(Body): common.glsl:228-230 */
static inline float body_radius(const orc_ctx* c, float m, float rho) {
    return c->sim.body_length_constant * powf(m / rho, 1.0f / 3.0f);
}

/* ---- Morton: SH/compute/morton/bh_morton.comp:6-34 ------------------------ */
uint64_t orc_expand_bits21(uint32_t v) {
    uint64_t x = (uint64_t)v & 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

uint64_t orc_morton3d64(uint32_t x, uint32_t y, uint32_t z) {
    return (orc_expand_bits21(x) << 2) | (orc_expand_bits21(y) << 1) | orc_expand_bits21(z);
}

static inline int aabb_empty(const float mn[3], const float mx[3]) { return mn[0] > mx[0]; }

/* mortonEncodeKernel body, bh_morton.comp:238-262 */
uint64_t orc_morton_encode(const float p_in[3], const float mn[3], const float mx[3]) {
    float pos[3], ext[3], q[3];
    uint32_t qi[3];
    if (!finite3(p_in) || aabb_empty(mn, mx)) {
        for (int k = 0; k < 3; ++k) pos[k] = 0.5f * (mn[k] + mx[k]);
    } else {
        for (int k = 0; k < 3; ++k) pos[k] = gclamp(p_in[k], mn[k], mx[k]);
    }
    for (int k = 0; k < 3; ++k) {
        ext[k] = gmax(mx[k] - mn[k], (float)1e-9);
        q[k] = (pos[k] - mn[k]) / ext[k];
        float f = gclamp(floorf(q[k] * MAX_VALUE_21), 0.0f, MAX_VALUE_21);
        qi[k] = (uint32_t)floorf(f);
    }
    return orc_morton3d64(qi[0], qi[1], qi[2]);
}

/* ---- LCP: SH/compute/tree/bh_tree.comp:6-37 ------------------------------- */
static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

int orc_safe_lcp(const uint64_t* keys, int n, int i, int j) {
    if (i < 0 || j < 0 || i >= n || j >= n) return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a == b) {
        uint32_t x = (uint32_t)i ^ (uint32_t)j;
        if (x == 0) return 64;
        return 64 + clz32(x);
    }
    return clz64(a ^ b);
}

/* ---- lifecycle ------------------------------------------------------------ */
orc_ctx* orc_create(uint32_t n, const float bounds[6], const gbh_units* units) {
    if (n == 0 || !bounds || !units) return NULL;
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    if (!c) return NULL;
    c->N = n;
    for (int k = 0; k < 2; ++k) {
        c->bodies[k] = (gbh_body*)calloc(n, sizeof(gbh_body));
        c->morton[k] = (uint64_t*)calloc(n, sizeof(uint64_t));
        c->index[k] = (uint32_t*)calloc(n, sizeof(uint32_t));
    }
    c->leaf = (gbh_node*)calloc(n, sizeof(gbh_node));
    c->internal = (gbh_node*)calloc(n > 1 ? n - 1 : 1, sizeof(gbh_node));
    c->mcap = n;
    c->mtasks = (uint32_t*)calloc(2 * (size_t)n, sizeof(uint32_t));
    c->mkeys = (uint64_t*)calloc(n, sizeof(uint64_t));
    c->accel = (float*)calloc(4 * (size_t)n, sizeof(float));
    if (!c->bodies[0] || !c->bodies[1] || !c->morton[0] || !c->morton[1] || !c->index[0] ||
        !c->index[1] || !c->leaf || !c->internal || !c->mtasks || !c->mkeys || !c->accel) {
        orc_destroy(c);
        return NULL;
    }
    /* GPU.packValues, GPU.java:1096-1143 */
    c->sim.num_bodies = n;
    c->sim.initial_num_bodies = n;
    for (int k = 0; k < 3; ++k) {
        c->sim.bounds_min[k] = bounds[k];
        c->sim.bounds_max[k] = bounds[3 + k];
    }
    c->sim.unit_mass = units->mass;
    c->sim.unit_density = units->density;
    c->sim.unit_len = units->len;
    c->sim.unit_time = units->time;
    c->sim.camera_scale = units->camera_scale;
    /* keep the override for init */
    c->sim.gravitational_constant = units->gravitational_constant;
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    for (int k = 0; k < 2; ++k) {
        free(c->bodies[k]);
        free(c->morton[k]);
        free(c->index[k]);
    }
    free(c->leaf);
    free(c->internal);
    free(c->mtasks);
    free(c->mkeys);
    free(c->accel);
    free(c);
}

int orc_upload_bodies(orc_ctx* c, const gbh_body* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(c->bodies[c->bin] + offset, host, (size_t)count * sizeof(gbh_body));
    return GBH_OK;
}

/* bh_init.comp:10-27 */
int orc_init(orc_ctx* c) {
    if (!c) return GBH_ERR_INVALID;
    gbh_units u = {c->sim.unit_mass, c->sim.unit_density, c->sim.unit_len, c->sim.unit_time,
                   c->sim.camera_scale, c->sim.gravitational_constant};
    update_units(c, &u);
    for (uint32_t g = 0; g < c->N; ++g) c->index[c->iin][g] = g;
    c->inited = 1;
    return GBH_OK;
}

/* ---- stages --------------------------------------------------------------- */

/* bh_update.comp:10-28 with resetValuesOrDecrementDeadBodies == 1 */
int orc_stage_reset(orc_ctx* c, const gbh_step_params* p) {
    c->mtail = 0;
    c->opened = 0;
    c->interactions = 0;
    c->died = 0;
    c->oob_step = 0;
    c->merged = 0;
    if (p->units.mass != 0.0f) {
        gbh_units u = p->units;
        if (u.camera_scale == 0.0f) u.camera_scale = c->sim.camera_scale;
        update_units(c, &u);
    }
    return GBH_OK;
}

/* bh_dead.comp:13-112 (count, exclusive scan, stable scatter) then
 * GPU.swapMortonAndIndexBuffers (GPU.java:1070-1078). */
int orc_stage_partition(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    const uint32_t* in = c->index[c->iin];
    uint32_t* out = c->index[1 - c->iin];
    gbh_body* src = c->bodies[c->bin];
    gbh_body* dst = c->bodies[1 - c->bin];
    uint32_t dead = 0;
    for (uint32_t g = 0; g < n; ++g) {
        uint32_t b = in[g];
        if (src[b].pos_mass[3] == 0.0f) {
            memset(&src[b], 0, sizeof(gbh_body));
            memset(&dst[b], 0, sizeof(gbh_body));
            ++dead;
        }
    }
    uint32_t a = 0, d = 0;
    for (uint32_t g = 0; g < n; ++g) {
        uint32_t b = in[g];
        if (src[b].pos_mass[3] == 0.0f)
            out[n - dead + d++] = b;
        else
            out[a++] = b;
    }
    c->sim.just_died = dead;
    c->died = dead;
    c->iin = 1 - c->iin;
    return GBH_OK;
}

/* bh_update.comp:29-34 with resetValuesOrDecrementDeadBodies == 0 */
int orc_stage_decrement(orc_ctx* c) {
    c->sim.num_bodies -= c->sim.just_died;
    c->sim.just_died = 0;
    c->sim.uint_debug[0] = 0;
    return GBH_OK;
}

/* mortonAABBRepopulateKernel + mortonAABBCollapseKernel, bh_morton.comp:36-231.
 * Min/max unions are order independent, so the workgroup tree reductions are
 * restated as one serial union over the live bodies. */
int orc_stage_bounds(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    const uint32_t* in = c->index[c->iin];
    const gbh_body* src = c->bodies[c->bin];
    float pmin[3], pmax[3], lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        pmin[k] = c->sim.bounds_min[k];
        pmax[k] = c->sim.bounds_max[k];
    }
    const int prev_empty = aabb_empty(pmin, pmax);
    /* mortonInlierWindow, bh_morton.comp:50-56 */
    for (int k = 0; k < 3; ++k) {
        float center = 0.5f * (pmin[k] + pmax[k]);
        float half = gmax(0.5f * (pmax[k] - pmin[k]) * 1.05f, (float)1e-9);
        lo[k] = center - half;
        hi[k] = center + half;
    }
    float amin[3] = {1e38f, 1e38f, 1e38f}, amax[3] = {-1e38f, -1e38f, -1e38f};
    for (uint32_t g = 0; g < n; ++g) {
        const gbh_body* b = &src[in[g]];
        if (b->pos_mass[3] == 0.0f) continue;
        const float* p = b->pos_mass;
        /* mortonContributorAABB, bh_morton.comp:60-74 */
        if (!finite3(p)) continue;
        if (!prev_empty) {
            int outlier = 0;
            for (int k = 0; k < 3; ++k)
                if (p[k] < lo[k] || p[k] > hi[k]) outlier = 1;
            if (outlier) continue;
        }
        for (int k = 0; k < 3; ++k) {
            amin[k] = gmin(amin[k], p[k]);
            amax[k] = gmax(amax[k], p[k]);
        }
    }
    if (aabb_empty(amin, amax)) {
        if (prev_empty) {
            for (int k = 0; k < 3; ++k) {
                c->sim.bounds_min[k] = amin[k];
                c->sim.bounds_max[k] = amax[k];
            }
        }
        return GBH_OK;
    }
    if (prev_empty) {
        for (int k = 0; k < 3; ++k) {
            c->sim.bounds_min[k] = amin[k];
            c->sim.bounds_max[k] = amax[k];
        }
        return GBH_OK;
    }
    /* clampAABBExtentGrowth, bh_morton.comp:77-88 */
    for (int k = 0; k < 3; ++k) {
        float prev_ext = gmax(pmax[k] - pmin[k], (float)1e-9);
        float max_ext = prev_ext * 1.1f;
        float center = 0.5f * (amin[k] + amax[k]);
        float half = 0.5f * (amax[k] - amin[k]);
        float max_half = 0.5f * max_ext;
        half = gmin(half, max_half);
        c->sim.bounds_min[k] = center - half;
        c->sim.bounds_max[k] = center + half;
    }
    return GBH_OK;
}

/* mortonEncodeKernel, bh_morton.comp:238-262 */
int orc_stage_encode(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    const uint32_t* in = c->index[c->iin];
    uint64_t* keys = c->morton[c->iin];
    const gbh_body* src = c->bodies[c->bin];
    const float* mn = c->sim.bounds_min;
    const float* mx = c->sim.bounds_max;
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)n; ++g) keys[g] = orc_morton_encode(src[in[g]].pos_mass, mn, mx);
    return GBH_OK;
}

/* radixSort, BarnesHut.java:358-448 with bh_radix.comp:12-166: a stable LSD
 * sort of (key, index) pairs.  Any stable sort yields the same permutation, so
 * this restatement uses 8-bit digits (8 passes) and ends with the result in
 * the *_IN buffers like the reference's 16 passes. */
int orc_stage_sort(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    uint64_t* ka = c->morton[c->iin];
    uint32_t* va = c->index[c->iin];
    uint64_t* kb = c->morton[1 - c->iin];
    uint32_t* vb = c->index[1 - c->iin];
    if (n <= 1) return GBH_OK;
    int nt = orc_get_threads();
    if (nt < 1) nt = 1;
    if (nt > 256) nt = 256;
    size_t* hist = (size_t*)malloc(sizeof(size_t) * 256 * (size_t)nt);
    if (!hist) return GBH_ERR_OOM;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 8 * pass;
        memset(hist, 0, sizeof(size_t) * 256 * (size_t)nt);
#pragma omp parallel num_threads(nt)
        {
#ifdef _OPENMP
            int t = omp_get_thread_num();
            int T = omp_get_num_threads();
#else
            int t = 0, T = 1;
#endif
            size_t lo = (size_t)n * t / T, hi = (size_t)n * (t + 1) / T;
            size_t* h = hist + 256 * (size_t)t;
            for (size_t i = lo; i < hi; ++i) h[(ka[i] >> shift) & 0xFF]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int d = 0; d < 256; ++d)
                    for (int tt = 0; tt < T; ++tt) {
                        size_t v = hist[256 * (size_t)tt + d];
                        hist[256 * (size_t)tt + d] = run;
                        run += v;
                    }
            }
            for (size_t i = lo; i < hi; ++i) {
                size_t pos = h[(ka[i] >> shift) & 0xFF]++;
                kb[pos] = ka[i];
                vb[pos] = va[i];
            }
        }
        uint64_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    free(hist);
    return GBH_OK;
}

/* treeBuildBinaryRadixTreeKernel, bh_tree.comp:43-133 (Karras 2012). */
int orc_stage_build(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    const uint32_t N = c->N;
    const uint64_t* keys = c->morton[c->iin];
    gbh_node* in_nodes = c->internal;
    gbh_node* leaves = c->leaf;
    if (n == 0) return GBH_OK;
    if (n == 1) {
        gbh_node* r = &in_nodes[0];
        r->parent_id = NONE_ID;
        r->child_a = 0;
        r->child_b = NONE_ID;
        r->ready_children = 1;
        memset(r->com_mass, 0, sizeof(r->com_mass));
        r->aabb[0] = r->aabb[1] = r->aabb[2] = 1e38f;
        r->aabb[3] = r->aabb[4] = r->aabb[5] = -1e38f;
        r->node_depth = 0;
        r->bodies_contained = 0;
        memset(r->avg_color, 0, sizeof(r->avg_color));
        leaves[0].parent_id = N;
        return GBH_OK;
    }
    const int ni = (int)n;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ni - 1; ++i) {
        int lcp_r = orc_safe_lcp(keys, ni, i, i + 1);
        int lcp_l = orc_safe_lcp(keys, ni, i, i - 1);
        int d = (lcp_l > lcp_r) ? -1 : 1;
        int delta_min = orc_safe_lcp(keys, ni, i, i - d);
        int lmax = 2;
        while (orc_safe_lcp(keys, ni, i, i + d * lmax) > delta_min) lmax *= 2;
        int l = 0;
        int t = lmax / 2;
        while (t > 0) {
            if (orc_safe_lcp(keys, ni, i, i + d * (l + t)) > delta_min) l = l + t;
            t /= 2;
        }
        int j = i + l * d;
        int delta_node = orc_safe_lcp(keys, ni, i, j);
        int s = 0;
        t = l;
        while (t > 1) {
            t = (t + 1) / 2;
            if (orc_safe_lcp(keys, ni, i, i + (s + t) * d) > delta_node) s += t;
        }
        int gamma = i + s * d + (d < 0 ? d : 0);
        int mn = i < j ? i : j, mx = i < j ? j : i;
        uint32_t left = (mn == gamma) ? (uint32_t)gamma : (uint32_t)gamma + N;
        uint32_t right = (mx == gamma + 1) ? (uint32_t)(gamma + 1) : (uint32_t)(gamma + 1) + N;
        gbh_node* nd = &in_nodes[i];
        nd->child_a = left;
        nd->child_b = right;
        nd->ready_children = 0;
        memset(nd->com_mass, 0, sizeof(nd->com_mass));
        nd->aabb[0] = nd->aabb[1] = nd->aabb[2] = 1e38f;
        nd->aabb[3] = nd->aabb[4] = nd->aabb[5] = -1e38f;
        memset(nd->avg_color, 0, sizeof(nd->avg_color));
        uint32_t gidx = (uint32_t)i + N;
        if (left < N) leaves[left].parent_id = gidx; else in_nodes[left - N].parent_id = gidx;
        if (right < N) leaves[right].parent_id = gidx; else in_nodes[right - N].parent_id = gidx;
        nd->node_depth = (uint32_t)mn;
        nd->bodies_contained = (uint32_t)(mx - mn + 1);
        if (i == 0) nd->parent_id = NONE_ID;
    }
    return GBH_OK;
}

/* combine two children into an internal node: bh_tree.comp:223-246 */
static void combine(gbh_node* dst, const gbh_node* L, const gbh_node* R) {
    float lw = L->com_mass[3], rw = R->com_mass[3];
    float M = lw + rw;
    if (M > 0.0f) {
        for (int k = 0; k < 3; ++k) {
            float a = lw * L->com_mass[k];
            float b = rw * R->com_mass[k];
            dst->com_mass[k] = (a + b) / M;
            float ca = lw * L->avg_color[k];
            float cb = rw * R->avg_color[k];
            dst->avg_color[k] = (ca + cb) / M;
        }
    } else {
        for (int k = 0; k < 3; ++k) {
            dst->com_mass[k] = (L->com_mass[k] + R->com_mass[k]) * 0.5f;
            dst->avg_color[k] = (L->avg_color[k] + R->avg_color[k]) * 0.5f;
        }
    }
    dst->com_mass[3] = M;
    dst->avg_color[3] = 0.0f;
    for (int k = 0; k < 3; ++k) {
        dst->aabb[k] = gmin(L->aabb[k], R->aabb[k]);
        dst->aabb[3 + k] = gmax(L->aabb[3 + k], R->aabb[3 + k]);
    }
    dst->ready_children = NONE_ID;
    uint32_t hd = L->node_depth > R->node_depth ? L->node_depth : R->node_depth;
    dst->node_depth = 1u + hd;
}

/* treeInitLeafNodesKernel (bh_tree.comp:140-175) and treePropagateNodesKernel
 * (bh_tree.comp:183-259).  The reference propagates with 64 queue passes; this
 * restatement fills every level (post-order), which equals the reference
 * whenever the tree height is at most 64 (tree_height reports it). */
int orc_stage_fill(orc_ctx* c) {
    const uint32_t n = c->sim.num_bodies;
    const uint32_t N = c->N;
    const uint32_t* in = c->index[c->iin];
    const gbh_body* src = c->bodies[c->bin];
    gbh_node* leaves = c->leaf;
    gbh_node* nodes = c->internal;
    c->tree_height = 0;
    if (n == 0) return GBH_OK;
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < (int64_t)n; ++g) {
        const gbh_body* b = &src[in[g]];
        gbh_node* lf = &leaves[g];
        for (int k = 0; k < 4; ++k) lf->com_mass[k] = b->pos_mass[k];
        for (int k = 0; k < 3; ++k) {
            lf->aabb[k] = b->pos_mass[k];
            lf->aabb[3 + k] = b->pos_mass[k];
        }
        lf->child_a = NONE_ID;
        lf->child_b = NONE_ID;
        lf->ready_children = NONE_ID;
        lf->node_depth = 0;
        if (b->pos_mass[3] > 0.0f && b->vel_density[3] > 0.0f) {
            float rgb[3];
            orc_star_color(b->pos_mass[3] * c->sim.unit_mass, b->vel_density[3] * c->sim.unit_density, rgb);
            lf->avg_color[0] = rgb[0];
            lf->avg_color[1] = rgb[1];
            lf->avg_color[2] = rgb[2];
            lf->avg_color[3] = 0.0f;
        } else {
            memset(lf->avg_color, 0, sizeof(lf->avg_color));
        }
    }
    if (n == 1) {
        /* single body: the root's second child does not exist; the root takes
         * the leaf's values (the reference reads past its buffer here) */
        gbh_node empty;
        memset(&empty, 0, sizeof(empty));
        empty.aabb[0] = empty.aabb[1] = empty.aabb[2] = 1e38f;
        empty.aabb[3] = empty.aabb[4] = empty.aabb[5] = -1e38f;
        combine(&nodes[0], &leaves[0], &empty);
        c->tree_height = nodes[0].node_depth;
        return GBH_OK;
    }
    /* iterative post-order over internal nodes from the root */
    uint32_t* stack = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)n + 16);
    uint8_t* state = (uint8_t*)calloc(n, 1);
    if (!stack || !state) {
        free(stack);
        free(state);
        return GBH_ERR_OOM;
    }
    size_t sp = 0;
    stack[sp++] = 0;
    while (sp) {
        uint32_t i = stack[sp - 1];
        gbh_node* nd = &nodes[i];
        if (!state[i]) {
            state[i] = 1;
            if (nd->child_b >= N) stack[sp++] = nd->child_b - N;
            if (nd->child_a >= N) stack[sp++] = nd->child_a - N;
            continue;
        }
        --sp;
        const gbh_node* L = nd->child_a < N ? &leaves[nd->child_a] : &nodes[nd->child_a - N];
        const gbh_node* R = nd->child_b < N ? &leaves[nd->child_b] : &nodes[nd->child_b - N];
        combine(nd, L, R);
    }
    c->tree_height = nodes[0].node_depth;
    free(stack);
    free(state);
    return GBH_OK;
}

/* ---- the walk: forceComputeKernel, bh_force.comp:6-142 -------------------- */
typedef struct {
    uint32_t* tasks; /* pairs */
    uint64_t* keys;
    uint32_t count, cap;
} task_buf;

static void task_push(task_buf* tb, uint32_t a, uint32_t b, uint64_t key) {
    if (tb->count == tb->cap) {
        uint32_t nc = tb->cap ? tb->cap * 2 : 64;
        tb->tasks = (uint32_t*)realloc(tb->tasks, sizeof(uint32_t) * 2 * nc);
        tb->keys = (uint64_t*)realloc(tb->keys, sizeof(uint64_t) * nc);
        tb->cap = nc;
    }
    tb->tasks[2 * tb->count] = a;
    tb->tasks[2 * tb->count + 1] = b;
    tb->keys[tb->count] = key;
    tb->count++;
}

typedef struct {
    uint64_t opened, interactions;
    uint32_t oob;
} walk_counts;

/* Walk one sorted slot g; returns 1 if the body was killed out of bounds.
 * When `dst` is NULL nothing is written (CPU-baseline samples). */
static void walk_body(orc_ctx* c, const gbh_step_params* p, uint32_t g, gbh_body* dst, task_buf* tb,
                      walk_counts* wc, uint32_t* stack, uint32_t stack_cap) {
    const uint32_t N = c->N;
    const uint32_t* in = c->index[c->iin];
    const gbh_body* src = c->bodies[c->bin];
    const gbh_node* leaves = c->leaf;
    const gbh_node* nodes = c->internal;
    const float G = c->sim.gravitational_constant;
    const float soft = p->softening, theta = p->theta;
    const uint32_t mode = p->merging_collision_or_neither;
    const uint32_t b_idx = in[g];
    gbh_body body = src[b_idx];
    float acc[3] = {0.0f, 0.0f, 0.0f};
    uint32_t seq = 0;
    uint32_t sp = 0;
    const int single = (c->sim.num_bodies == 1);
    if (!single) stack[sp++] = N;
    while (sp > 0) {
        uint32_t id = stack[--sp];
        const gbh_node* nd = id < N ? &leaves[id] : &nodes[id - N];
        float r[3];
        for (int k = 0; k < 3; ++k) r[k] = nd->com_mass[k] - body.pos_mass[k];
        float inv = ginversesqrt(gdot3(r, r) + soft);
        if (nd->child_a != NONE_ID) {
            float ex = nd->aabb[3] - nd->aabb[0];
            float ey = nd->aabb[4] - nd->aabb[1];
            float ez = nd->aabb[5] - nd->aabb[2];
            float longest = gmax(ex, gmax(ey, ez)) / 2.0f;
            if (longest * inv < theta) {
                float s = G * nd->com_mass[3];
                for (int k = 0; k < 3; ++k) {
                    float f = s * r[k];
                    f = f * inv;
                    f = f * inv;
                    f = f * inv;
                    acc[k] = acc[k] + f;
                }
                wc->interactions++;
            } else {
                if (sp + 2 > stack_cap) break; /* cannot happen with stack_cap >= 2n */
                stack[sp++] = nd->child_a;
                stack[sp++] = nd->child_b;
                wc->opened++;
            }
        } else {
            if (in[id] == b_idx) continue;
            float s = G * nd->com_mass[3];
            for (int k = 0; k < 3; ++k) {
                float f = s * r[k];
                f = f * inv;
                f = f * inv;
                f = f * inv;
                acc[k] = acc[k] + f;
            }
            wc->interactions++;
            if (mode == GBH_MODE_NEITHER) continue;
            const uint32_t o_idx = in[id];
            const gbh_body* other = &src[o_idx];
            float br = body_radius(c, body.pos_mass[3], body.vel_density[3]);
            float orad = body_radius(c, other->pos_mass[3], other->vel_density[3]);
            float dist = sqrtf(gdot3(r, r));
            float pen = br + orad - dist;
            if (mode == GBH_MODE_COLLISION && pen > 0.0f) {
                float vd[3], nrm[3];
                for (int k = 0; k < 3; ++k) vd[k] = other->vel_density[k] - body.vel_density[k];
                float len = sqrtf(gdot3(r, r));
                for (int k = 0; k < 3; ++k) nrm[k] = r[k] / len;
                float vimp = gdot3(vd, nrm);
                if (vimp < 0.0f) {
                    float meff = 1.0f / (1.0f / body.pos_mass[3] + 1.0f / other->pos_mass[3]);
                    float impulse = (1.0f + p->elasticity) * meff;
                    impulse = impulse * vimp;
                    for (int k = 0; k < 3; ++k) body.vel_density[k] += (nrm[k] * impulse) / body.pos_mass[3];
                }
                float sc = pen / (body.pos_mass[3] + other->pos_mass[3]);
                sc = sc * p->restitution;
                for (int k = 0; k < 3; ++k) body.pos_mass[k] -= sc * nrm[k];
            }
            if (mode == GBH_MODE_MERGE && pen > 0.0f && b_idx < o_idx && tb)
                task_push(tb, b_idx, o_idx, ((uint64_t)g << 32) | seq++);
        }
    }
    if (c->store_accel && dst) {
        float* a = &c->accel[4 * (size_t)b_idx];
        a[0] = acc[0];
        a[1] = acc[1];
        a[2] = acc[2];
        a[3] = 0.0f;
    }
    if (!dst) return;
    /* symplectic update and static-bounds handling, bh_force.comp:117-141 */
    float nv[3], np[3];
    for (int k = 0; k < 3; ++k) {
        nv[k] = body.vel_density[k] + acc[k] * p->dt;
        np[k] = body.pos_mass[k] + nv[k] * p->dt;
    }
    if (p->static_or_dynamic == GBH_BOUNDS_STATIC) {
        const float* mn = c->sim.bounds_min;
        const float* mx = c->sim.bounds_max;
        if (p->wrap_around) {
            for (int k = 0; k < 3; ++k) {
                float x = np[k] - mn[k];
                float y = mx[k] - mn[k];
                np[k] = (x - y * floorf(x / y)) + mn[k];
            }
        } else {
            const float* bp = body.pos_mass;
            if (bp[0] < mn[0] || bp[0] > mx[0] || bp[1] < mn[1] || bp[1] > mx[1] || bp[2] < mn[2] ||
                bp[2] > mx[2]) {
                memset(&dst[b_idx], 0, sizeof(gbh_body));
                wc->oob++;
                return;
            }
        }
    }
    gbh_body* o = &dst[b_idx];
    o->vel_density[0] = nv[0];
    o->vel_density[1] = nv[1];
    o->vel_density[2] = nv[2];
    o->vel_density[3] = body.vel_density[3];
    o->pos_mass[0] = np[0];
    o->pos_mass[1] = np[1];
    o->pos_mass[2] = np[2];
    o->pos_mass[3] = body.pos_mass[3];
}

static int cmp_u64_pair(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* the walk of sorted slots [lo, hi) */
static int walk_slots(orc_ctx* c, const gbh_step_params* p, uint32_t lo, uint32_t hi) {
    gbh_body* dst = c->bodies[1 - c->bin];
    c->store_accel = (p->flags & GBH_FLAG_STORE_ACCEL) != 0;
    uint64_t opened = 0, inter = 0;
    uint32_t oob = 0;
    const uint32_t stack_cap = 2 * (c->N + 8);
    int nt = orc_get_threads();
    task_buf* tbs = (task_buf*)calloc((size_t)nt, sizeof(task_buf));
#pragma omp parallel num_threads(nt) reduction(+ : opened, inter, oob)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        uint32_t* stack = (uint32_t*)malloc(sizeof(uint32_t) * stack_cap);
        walk_counts wc = {0, 0, 0};
#pragma omp for schedule(dynamic, 256)
        for (int64_t g = lo; g < (int64_t)hi; ++g) walk_body(c, p, (uint32_t)g, dst, &tbs[t], &wc, stack, stack_cap);
        opened += wc.opened;
        inter += wc.interactions;
        oob += wc.oob;
        free(stack);
    }
    /* gather merge tasks in emission order of a sequential walk */
    uint32_t total = 0;
    for (int t = 0; t < nt; ++t) total += tbs[t].count;
    uint64_t* order = (uint64_t*)malloc(sizeof(uint64_t) * 2 * (size_t)(total + 1));
    uint32_t k = 0;
    for (int t = 0; t < nt; ++t)
        for (uint32_t i = 0; i < tbs[t].count; ++i) {
            order[2 * k] = tbs[t].keys[i];
            order[2 * k + 1] = ((uint64_t)tbs[t].tasks[2 * i] << 32) | tbs[t].tasks[2 * i + 1];
            ++k;
        }
    qsort(order, total, 2 * sizeof(uint64_t), cmp_u64_pair);
    if (total > c->mcap) total = c->mcap;
    for (uint32_t i = 0; i < total; ++i) {
        c->mkeys[i] = order[2 * i];
        c->mtasks[2 * i] = (uint32_t)(order[2 * i + 1] >> 32);
        c->mtasks[2 * i + 1] = (uint32_t)order[2 * i + 1];
    }
    c->mtail = total;
    free(order);
    for (int t = 0; t < nt; ++t) {
        free(tbs[t].tasks);
        free(tbs[t].keys);
    }
    free(tbs);
    c->opened += opened;
    c->interactions += inter;
    c->oob_step += oob;
    c->sim.out_of_bounds += oob;
    c->sim.uint_debug[0] += (uint32_t)opened;
    return GBH_OK;
}

int orc_stage_walk(orc_ctx* c, const gbh_step_params* p) { return walk_slots(c, p, 0, c->sim.num_bodies); }

/* ---- the sharded step (the GPU's gbh_step_shard_* restated): rank r of W
 * walks sorted slots [n r / W, n (r + 1) / W); bh_force.comp:40-142 walks
 * every body independently, so the shares together equal the whole walk. */
int orc_step_shard_walk(orc_ctx* c, const gbh_step_params* p, uint32_t rank, uint32_t world, uint32_t range[2]) {
    if (!c || !p || !range || world == 0 || rank >= world) return GBH_ERR_INVALID;
    orc_stage_reset(c, p);
    orc_stage_partition(c);
    orc_stage_decrement(c);
    if (p->static_or_dynamic == GBH_BOUNDS_DYNAMIC) orc_stage_bounds(c);
    orc_stage_encode(c);
    int rc = orc_stage_sort(c);
    if (rc) return rc;
    orc_stage_build(c);
    if ((rc = orc_stage_fill(c))) return rc;
    const uint64_t n = c->sim.num_bodies;
    range[0] = (uint32_t)(n * rank / world);
    range[1] = (uint32_t)(n * (rank + 1) / world);
    return walk_slots(c, p, range[0], range[1]);
}

int orc_shard_pack(orc_ctx* c, uint32_t lo, uint32_t count, gbh_body* out) {
    if (!c || (!out && count) || (uint64_t)lo + count > c->N) return GBH_ERR_INVALID;
    const gbh_body* dst = c->bodies[1 - c->bin];
    const uint32_t* in = c->index[c->iin];
    for (uint32_t i = 0; i < count; ++i) out[i] = dst[in[lo + i]];
    return GBH_OK;
}

int orc_shard_unpack(orc_ctx* c, uint32_t lo, uint32_t count, const gbh_body* body) {
    if (!c || (!body && count) || (uint64_t)lo + count > c->N) return GBH_ERR_INVALID;
    gbh_body* dst = c->bodies[1 - c->bin];
    const uint32_t* in = c->index[c->iin];
    for (uint32_t i = 0; i < count; ++i) dst[in[lo + i]] = body[i];
    return GBH_OK;
}

int orc_read_merge_tasks_full(orc_ctx* c, uint32_t* pairs, uint64_t* keys, uint32_t capacity, uint32_t* count) {
    if (!c || !count) return GBH_ERR_INVALID;
    *count = c->mtail;
    const uint32_t k = c->mtail < capacity ? c->mtail : capacity;
    if (pairs) memcpy(pairs, c->mtasks, (size_t)k * 8);
    if (keys) memcpy(keys, c->mkeys, (size_t)k * 8);
    return GBH_OK;
}

/* tasks in ascending key order: the merge applies them in array order */
int orc_write_merge_tasks(orc_ctx* c, const uint32_t* pairs, const uint64_t* keys, uint32_t count) {
    if (!c || (count && (!pairs || !keys)) || count > c->mcap) return GBH_ERR_INVALID;
    memcpy(c->mtasks, pairs, (size_t)count * 8);
    memcpy(c->mkeys, keys, (size_t)count * 8);
    c->mtail = count;
    return GBH_OK;
}

int orc_step_shard_finish(orc_ctx* c, uint32_t oob_other_ranks) {
    if (!c) return GBH_ERR_INVALID;
    c->sim.out_of_bounds += oob_other_ranks;
    c->oob_step += oob_other_ranks;
    orc_stage_merge(c);
    orc_stage_swap(c);
    return GBH_OK;
}

int orc_stage_walk_sample(orc_ctx* c, const gbh_step_params* p, uint32_t stride, uint64_t* interactions) {
    const uint32_t n = c->sim.num_bodies;
    if (stride == 0) stride = 1;
    uint64_t inter = 0;
    const uint32_t stack_cap = 2 * (c->N + 8);
    const int64_t cnt = (n + stride - 1) / stride;
#pragma omp parallel reduction(+ : inter)
    {
        uint32_t* stack = (uint32_t*)malloc(sizeof(uint32_t) * stack_cap);
        walk_counts wc = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
        for (int64_t s = 0; s < cnt; ++s) walk_body(c, p, (uint32_t)(s * stride), NULL, NULL, &wc, stack, stack_cap);
        inter += wc.interactions;
        free(stack);
    }
    if (interactions) *interactions = inter;
    return GBH_OK;
}

/* mergeBodies, bh_merge.comp:5-22 */
static gbh_body merge_two(const gbh_body* b1, const gbh_body* b2) {
    gbh_body m;
    memset(&m, 0, sizeof(m));
    float m1 = b1->pos_mass[3], m2 = b2->pos_mass[3];
    float M = m1 + m2;
    if (M == 0.0f) return m;
    if (m1 == 0.0f) return *b2;
    if (m2 == 0.0f) return *b1;
    for (int k = 0; k < 3; ++k) {
        float a = b1->pos_mass[k] * m1;
        float b = b2->pos_mass[k] * m2;
        m.pos_mass[k] = (a + b) / M;
        float va = b1->vel_density[k] * m1;
        float vb = b2->vel_density[k] * m2;
        m.vel_density[k] = (va + vb) / M;
    }
    m.pos_mass[3] = M;
    float s = m1 + m2;
    float q = m1 / b1->vel_density[3];
    q = q + m2 / b2->vel_density[3];
    m.vel_density[3] = s / q;
    return m;
}

/* mergeBodiesKernel, bh_merge.comp:30-71, run as one thread in the walk's
 * emission order (a schedule of the reference under which no try-lock fails). */
int orc_stage_merge(orc_ctx* c) {
    gbh_body* dst = c->bodies[1 - c->bin];
    uint32_t merged = 0;
    for (uint32_t t = 0; t < c->mtail; ++t) {
        uint32_t a = c->mtasks[2 * t], b = c->mtasks[2 * t + 1];
        if (a == b) continue;
        gbh_body b1 = dst[a], b2 = dst[b];
        if (b1.pos_mass[3] != 0.0f && b2.pos_mass[3] != 0.0f) {
            dst[a] = merge_two(&b1, &b2);
            memset(&dst[b], 0, sizeof(gbh_body));
            ++merged;
        }
    }
    c->merged = merged;
    return GBH_OK;
}

int orc_stage_swap(orc_ctx* c) {
    c->bin = 1 - c->bin;
    return GBH_OK;
}

/* BarnesHut.step, BarnesHut.java:99-164 */
int orc_step(orc_ctx* c, const gbh_step_params* p) {
    if (!c || !p) return GBH_ERR_INVALID;
    if (!c->inited) return GBH_ERR_STATE;
    orc_stage_reset(c, p);
    orc_stage_partition(c);
    orc_stage_decrement(c);
    if (p->static_or_dynamic == GBH_BOUNDS_DYNAMIC) orc_stage_bounds(c);
    orc_stage_encode(c);
    int rc = orc_stage_sort(c);
    if (rc) return rc;
    orc_stage_build(c);
    rc = orc_stage_fill(c);
    if (rc) return rc;
    orc_stage_walk(c, p);
    orc_stage_merge(c);
    orc_stage_swap(c);
    return GBH_OK;
}

/* ---- read / write ----------------------------------------------------------- */
int orc_read_bodies(orc_ctx* c, uint32_t which, gbh_body* host, uint32_t count, uint32_t offset) {
    if (!c || !host || which > 1 || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(host, c->bodies[which == GBH_BODIES_IN ? c->bin : 1 - c->bin] + offset, (size_t)count * sizeof(gbh_body));
    return GBH_OK;
}
int orc_read_leaf_nodes(orc_ctx* c, gbh_node* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(host, c->leaf + offset, (size_t)count * sizeof(gbh_node));
    return GBH_OK;
}
int orc_read_internal_nodes(orc_ctx* c, gbh_node* host, uint32_t count, uint32_t offset) {
    uint32_t cap = c && c->N > 1 ? c->N - 1 : 1;
    if (!c || !host || (uint64_t)offset + count > cap) return GBH_ERR_INVALID;
    memcpy(host, c->internal + offset, (size_t)count * sizeof(gbh_node));
    return GBH_OK;
}
int orc_read_sim_values(orc_ctx* c, gbh_sim_values* host) {
    if (!c || !host) return GBH_ERR_INVALID;
    *host = c->sim;
    return GBH_OK;
}
int orc_read_index(orc_ctx* c, uint32_t* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(host, c->index[c->iin] + offset, (size_t)count * sizeof(uint32_t));
    return GBH_OK;
}
int orc_read_morton(orc_ctx* c, uint64_t* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(host, c->morton[c->iin] + offset, (size_t)count * sizeof(uint64_t));
    return GBH_OK;
}
int orc_read_merge_tasks(orc_ctx* c, uint32_t* host_pairs, uint32_t capacity, uint32_t* count) {
    if (!c || !count) return GBH_ERR_INVALID;
    *count = c->mtail;
    uint32_t k = c->mtail < capacity ? c->mtail : capacity;
    if (host_pairs && k) memcpy(host_pairs, c->mtasks, sizeof(uint32_t) * 2 * (size_t)k);
    return GBH_OK;
}
int orc_read_accel(orc_ctx* c, float* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(host, c->accel + 4 * (size_t)offset, sizeof(float) * 4 * (size_t)count);
    return GBH_OK;
}
int orc_read_stats(orc_ctx* c, gbh_stats* s) {
    if (!c || !s) return GBH_ERR_INVALID;
    memset(s, 0, sizeof(*s));
    s->interactions = c->interactions;
    s->nodes_opened = c->opened;
    s->alive = c->sim.num_bodies;
    s->died = c->died;
    s->merged = c->merged;
    s->merge_tasks = c->mtail;
    s->out_of_bounds = c->oob_step;
    s->tree_height = c->tree_height;
    return GBH_OK;
}
int orc_write_sim_values(orc_ctx* c, const gbh_sim_values* host) {
    if (!c || !host) return GBH_ERR_INVALID;
    c->sim = *host;
    return GBH_OK;
}
int orc_write_index(orc_ctx* c, const uint32_t* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(c->index[c->iin] + offset, host, (size_t)count * sizeof(uint32_t));
    return GBH_OK;
}
int orc_write_morton(orc_ctx* c, const uint64_t* host, uint32_t count, uint32_t offset) {
    if (!c || !host || (uint64_t)offset + count > c->N) return GBH_ERR_INVALID;
    memcpy(c->morton[c->iin] + offset, host, (size_t)count * sizeof(uint64_t));
    return GBH_OK;
}

/* ---- FP64 direct sum (the accuracy reference) ----------------------------------- */
int orc_direct_sum_fp64(const gbh_body* bodies, uint32_t n, const uint32_t* sample, uint32_t count, double G,
                        double soft, double* out) {
    if (!bodies || !sample || !out) return GBH_ERR_INVALID;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t s = 0; s < (int64_t)count; ++s) {
        uint32_t i = sample[s];
        double xi = bodies[i].pos_mass[0], yi = bodies[i].pos_mass[1], zi = bodies[i].pos_mass[2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (uint32_t j = 0; j < n; ++j) {
            if (j == i) continue;
            double m = bodies[j].pos_mass[3];
            if (m == 0.0) continue;
            double dx = bodies[j].pos_mass[0] - xi, dy = bodies[j].pos_mass[1] - yi, dz = bodies[j].pos_mass[2] - zi;
            double r2 = dx * dx + dy * dy + dz * dz + soft;
            double inv = 1.0 / sqrt(r2);
            double f = G * m * inv * inv * inv;
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        out[3 * s] = ax;
        out[3 * s + 1] = ay;
        out[3 * s + 2] = az;
    }
    return GBH_OK;
}

/* ------------------------------------------------------------------------
 * Render-side level-of-detail selection (nodeglow.vert:46-150,
 * regions.vert:19-45), restated in FP32 with one rounding per operation.
 * mat4 * vec4 follows GLSL's column-major layout, columns added in order.
 * ------------------------------------------------------------------------ */
static void view_rel(const float a[3], const gbh_view* v, const gbh_body* bodies, uint32_t cap, float out[3]) {
    /* relativeLocation, common.glsl:291-299 */
    if (v->relative_to == 0xFFFFFFFFu || v->relative_to >= cap) {
        out[0] = a[0];
        out[1] = a[1];
        out[2] = a[2];
        return;
    }
    const float* p = bodies[v->relative_to].pos_mass;
    out[0] = a[0] - p[0];
    out[1] = a[1] - p[1];
    out[2] = a[2] - p[2];
}

static void view_mat4(const float m[16], const float x[4], float r[4]) {
    for (int row = 0; row < 4; ++row)
        r[row] = m[row] * x[0] + m[4 + row] * x[1] + m[8 + row] * x[2] + m[12 + row] * x[3];
}

static float view_smoothstep(float e0, float e1, float x) {
    /* GLSL smoothstep: t = clamp((x - e0) / (e1 - e0), 0, 1), t^2 (3 - 2t) */
    float t = (x - e0) / (e1 - e0);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

/* the AABB corners relative to view->relative_to, times cameraScale */
static void view_box(const gbh_node* nd, const gbh_view* v, const gbh_body* bodies, uint32_t cap, float mn[3],
                     float mx[3]) {
    float a[3], b[3];
    view_rel(&nd->aabb[0], v, bodies, cap, a);
    view_rel(&nd->aabb[3], v, bodies, cap, b);
    for (int k = 0; k < 3; ++k) {
        mn[k] = a[k] * v->camera_scale;
        mx[k] = b[k] * v->camera_scale;
    }
}

uint32_t orc_select_glow_nodes(const gbh_node* internal, uint32_t count, const gbh_body* bodies,
                               uint32_t num_bodies_cap, const gbh_view* v, gbh_glow_splat* out, uint32_t capacity) {
    const float tan_half = tanf(0.5f * v->fov_y);
    uint32_t sel = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const gbh_node* nd = &internal[i];
        /* culls in the shader's order */
        if (nd->aabb[0] > nd->aabb[3] || nd->com_mass[3] <= 0.0f || nd->bodies_contained == 0u) continue;
        if (nd->node_depth < 1u || nd->node_depth > (uint32_t)v->glow_max_depth) continue;
        float mn[3], mx[3];
        view_box(nd, v, bodies, num_bodies_cap, mn, mx);
        const float sx = mx[0] - mn[0], sy = mx[1] - mn[1], sz = mx[2] - mn[2];
        const float longest = fmaxf(sx, fmaxf(sy, sz));
        const float half_extent = 0.5f * longest;
        float com[3];
        view_rel(nd->com_mass, v, bodies, num_bodies_cap, com);
        const float com4[4] = {com[0] * v->camera_scale, com[1] * v->camera_scale, com[2] * v->camera_scale, 1.0f};
        float cv[4];
        view_mat4(v->model_view, com4, cv);
        const float cam_dist = fmaxf(-cv[2], 1e-6f);
        if (cam_dist < v->glow_activate_dist) continue;
        const float projected = longest / (cam_dist * tan_half);
        const float theta_ndc = fmaxf(v->glow_theta_ndc, 1e-6f);
        const float min_ndc = theta_ndc * 0.04f;
        if (projected >= theta_ndc || projected < min_ndc) continue;
        float accept = 1.0f - view_smoothstep(theta_ndc * 0.75f, theta_ndc, projected);
        accept = accept * view_smoothstep(min_ndc, min_ndc * 2.5f, projected);
        const float area = fmaxf(projected * projected, 1e-8f);
        const float luminosity = nd->com_mass[3] * (1.0e6f / (cam_dist * cam_dist));
        const float surface = luminosity / area;
        const float raw = surface * 2.5e-4f * accept * v->glow_intensity;
        const float intensity = raw / (1.0f + raw);
        if (intensity < 1e-4f) continue;
        if (sel < capacity) {
            gbh_glow_splat* r = &out[sel];
            float clip[4];
            view_mat4(v->proj, cv, clip);
            const float glow_half = fmaxf(half_extent * 1.1f, min_ndc * 0.5f * cam_dist * tan_half);
            const float ndc_y = glow_half / (cam_dist * tan_half);
            memcpy(r->center_clip, clip, sizeof(clip));
            memcpy(r->center_view, cv, 3 * sizeof(float));
            r->intensity = intensity;
            memcpy(r->color, nd->avg_color, 3 * sizeof(float));
            r->node = i;
            r->ndc_scale[0] = ndc_y / fmaxf(v->aspect, 1e-6f);
            r->ndc_scale[1] = ndc_y;
            r->depth = nd->node_depth;
            r->pad = 0;
        }
        ++sel;
    }
    return sel;
}

uint32_t orc_select_regions(const gbh_node* internal, uint32_t count, const gbh_body* bodies,
                            uint32_t num_bodies_cap, const gbh_view* v, gbh_region* out, uint32_t capacity) {
    uint32_t sel = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const gbh_node* nd = &internal[i];
        if (nd->aabb[0] > nd->aabb[3]) continue;
        if (nd->node_depth < (uint32_t)v->region_min_depth || nd->node_depth > (uint32_t)v->region_max_depth) continue;
        if (sel < capacity) {
            float mn[3], mx[3];
            view_box(nd, v, bodies, num_bodies_cap, mn, mx);
            gbh_region* r = &out[sel];
            for (int k = 0; k < 3; ++k) {
                r->center[k] = (mn[k] + mx[k]) * 0.5f;
                r->size[k] = mx[k] - mn[k];
            }
            r->node = i;
            r->depth = nd->node_depth;
        }
        ++sel;
    }
    return sel;
}
