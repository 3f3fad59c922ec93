// ref_kernels.cpp — runs the reference's own GLSL compute kernels on the CPU.
//
// TEST INFRASTRUCTURE ONLY (see glsl_shim.hpp).  The kernel bodies below come
// from the reference sources, #included unmodified from
// src/main/resources/shaders/compute/ (include path set by the Makefile).  This
// file adds (1) the dispatcher: one workgroup of 256 invocations at a time,
// invocations of kernels that call barrier() run as cooperative ucontext
// coroutines that yield at each barrier; (2) the host driver, a restatement of
// BarnesHut.step (src/main/java/com/grumbo/simulation/BarnesHut.java:99-164)
// with the dispatch widths of GPU.java:504-832 and the buffer swaps of
// GPU.java:1060-1086.  Atomics and queues run in one valid sequential schedule.
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "glsl_shim.hpp"

namespace glsl {
uvec3 gl_GlobalInvocationID, gl_LocalInvocationID, gl_WorkGroupID, gl_NumWorkGroups, gl_WorkGroupSize;
Node* leafNodes;
Node* internalNodes;
SimulationValues sim;
BodyBuffer srcB, dstB;
uint64_t* mortonIn;
uint64_t* mortonOut;
uint* indexIn;
uint* indexOut;
WorkQueue* g_queue_in;
WorkQueue* g_queue_out;
uint* wgHist;
uint* wgScanned;
uint bucketTotals[NUM_BUCKETS];
uint globalBase[NUM_BUCKETS];
uint mergeTasksHead, mergeTasksTail;
uvec2* mergeTasks;
uint* bodyLocks;
uint resetValuesOrDecrementDeadBodies;
float softening, theta, dt;
uint mergingCollisionOrNeither;
float cameraScale, elasticity, restitution, bothCriterion;
bool wrapAround;
uint staticOrDynamic;
uint passShift;
uint numWorkGroups;
float mass, density, len, time;
float g_gravity_override;

// the reference kernels, in bh_main.comp:44-53 order
#include "compute/init/bh_init.comp"
#include "compute/morton/bh_morton.comp"
#include "compute/radix/bh_radix.comp"
#include "compute/tree/bh_tree.comp"
#include "compute/force/bh_force.comp"
#include "compute/merge/bh_merge.comp"
#include "compute/update/bh_update.comp"
#include "compute/dead/bh_dead.comp"
}  // namespace glsl

using namespace glsl;

// ---- dispatcher ------------------------------------------------------------
static ucontext_t g_sched;
static ucontext_t g_inv[WG_SIZE];
static std::vector<char> g_stack[WG_SIZE];
static bool g_done[WG_SIZE];
static int g_cur = -1;
static void (*g_fn)() = nullptr;
static const size_t STACK_BYTES = 256 * 1024;

void glsl::barrier() {
    if (g_cur < 0) {
        fprintf(stderr, "barrier() outside a cooperative dispatch\n");
        abort();
    }
    swapcontext(&g_inv[g_cur], &g_sched);
}

static void trampoline() {
    g_fn();
    g_done[g_cur] = true;
}

static void set_ids(uint wg, uint lid) {
    gl_LocalInvocationID = {lid, 0, 0};
    gl_WorkGroupID = {wg, 0, 0};
    gl_GlobalInvocationID = {wg * WG_SIZE + lid, 0, 0};
}

static void dispatch(void (*fn)(), uint groups, bool cooperative) {
    gl_NumWorkGroups = {groups, 1, 1};
    gl_WorkGroupSize = {WG_SIZE, 1, 1};
    g_fn = fn;
    for (uint wg = 0; wg < groups; ++wg) {
        if (!cooperative) {
            for (uint lid = 0; lid < WG_SIZE; ++lid) {
                set_ids(wg, lid);
                fn();
            }
            continue;
        }
        for (uint lid = 0; lid < WG_SIZE; ++lid) {
            if (g_stack[lid].empty()) g_stack[lid].resize(STACK_BYTES);
            getcontext(&g_inv[lid]);
            g_inv[lid].uc_stack.ss_sp = g_stack[lid].data();
            g_inv[lid].uc_stack.ss_size = STACK_BYTES;
            g_inv[lid].uc_link = &g_sched;
            makecontext(&g_inv[lid], trampoline, 0);
            g_done[lid] = false;
        }
        uint remaining = WG_SIZE;
        while (remaining) {
            for (uint lid = 0; lid < WG_SIZE; ++lid) {
                if (g_done[lid]) continue;
                set_ids(wg, lid);
                g_cur = (int)lid;
                swapcontext(&g_sched, &g_inv[lid]);
                g_cur = -1;
                if (g_done[lid]) --remaining;
            }
        }
    }
}

// ---- host driver: BarnesHut.step with GPU.java's buffers and widths ---------
struct RefState {
    uint N = 0, groups = 0;
    std::vector<Body> bodies[2];
    std::vector<uint64_t> morton[2];
    std::vector<uint> index[2];
    std::vector<Node> leaf, internal;
    WorkQueue queues[2];
    std::vector<uint> qitems[2];
    std::vector<uint> hist, scanned;
    std::vector<uvec2> tasks;
    std::vector<uint> locks;
    int bin = 0, iin = 0, qin = 0;
};
static RefState* S = nullptr;

static void bind() {
    srcB.bodies = S->bodies[S->bin].data();
    dstB.bodies = S->bodies[1 - S->bin].data();
    mortonIn = S->morton[S->iin].data();
    mortonOut = S->morton[1 - S->iin].data();
    indexIn = S->index[S->iin].data();
    indexOut = S->index[1 - S->iin].data();
    leafNodes = S->leaf.data();
    internalNodes = S->internal.data();
    g_queue_in = &S->queues[S->qin];
    g_queue_out = &S->queues[1 - S->qin];
    wgHist = S->hist.data();
    wgScanned = S->scanned.data();
    mergeTasks = S->tasks.data();
    bodyLocks = S->locks.data();
    numWorkGroups = S->groups;
}

static void run(void (*fn)(), uint groups, bool coop) {
    bind();
    dispatch(fn, groups, coop);
}

extern "C" {

typedef struct {
    float dt, theta, softening, elasticity, restitution;
    uint32_t mode, static_or_dynamic, wrap_around;
    float mass, density, len, time, camera_scale, G;
} ref_params;

int ref_create(uint32_t n, const float bounds[6], float umass, float udensity, float ulen, float utime,
               float camera_scale, float G) {
    delete S;
    S = new RefState();
    S->N = n;
    S->groups = (n + WG_SIZE - 1) / WG_SIZE;
    const size_t pad = (size_t)S->groups * WG_SIZE + WG_SIZE;
    for (int k = 0; k < 2; ++k) {
        S->bodies[k].assign(pad, make_empty_body());
        S->morton[k].assign(pad, 0);
        S->index[k].assign(pad, 0);
        S->qitems[k].assign(pad + 4, 0);
        S->queues[k].head = S->queues[k].tail = 0;
        S->queues[k].items = S->qitems[k].data();
    }
    Node zero;
    memset(&zero, 0, sizeof(zero));
    S->leaf.assign(pad, zero);
    S->internal.assign(pad, zero);
    S->hist.assign((size_t)S->groups * NUM_BUCKETS + 16, 0);
    S->scanned.assign((size_t)S->groups * NUM_BUCKETS + 16, 0);
    S->tasks.assign(pad, uvec2(0, 0));
    S->locks.assign(pad, 0);
    memset(&sim, 0, sizeof(sim));
    // GPU.packValues, GPU.java:1096-1143
    sim.numBodies = n;
    sim.initialNumBodies = n;
    sim.bounds = AABB(vec3(bounds[0], bounds[1], bounds[2]), vec3(bounds[3], bounds[4], bounds[5]));
    sim.units.mass = umass;
    sim.units.density = udensity;
    sim.units.len = ulen;
    sim.units.time = utime;
    sim.units.cameraScale = camera_scale;
    mass = umass;
    density = udensity;
    len = ulen;
    time = utime;
    cameraScale = camera_scale;
    g_gravity_override = G;
    mergeTasksHead = mergeTasksTail = 0;
    return 0;
}

int ref_upload_bodies(const void* host, uint32_t count, uint32_t offset) {
    memcpy(S->bodies[S->bin].data() + offset, host, (size_t)count * sizeof(Body));
    return 0;
}

// BarnesHut.init, BarnesHut.java:170-173
int ref_init() {
    run(initKernel, S->groups, false);
    return 0;
}

static void set_uniforms(const ref_params* p) {
    dt = p->dt;
    theta = p->theta;
    softening = p->softening;
    elasticity = p->elasticity;
    restitution = p->restitution;
    mergingCollisionOrNeither = p->mode;
    staticOrDynamic = p->static_or_dynamic;
    wrapAround = p->wrap_around != 0;
    // the unit uniforms come from Settings every dispatch (GPU.java:484-496)
    mass = p->mass;
    density = p->density;
    len = p->len;
    time = p->time;
    cameraScale = p->camera_scale;
}

int ref_stage_reset(const ref_params* p) {
    set_uniforms(p);
    resetValuesOrDecrementDeadBodies = 1u;
    run(updateKernel, 1, false);
    return 0;
}

// partitionDeadBodies + swap + decrementDeadBodies (BarnesHut.java:114-120)
int ref_stage_partition() {
    run(deadCountKernel, S->groups, true);
    run(deadExclusiveScanKernel, 1, false);
    run(deadScatterKernel, S->groups, true);
    S->iin = 1 - S->iin;
    resetValuesOrDecrementDeadBodies = 0u;
    run(updateKernel, 1, false);
    return 0;
}

int ref_stage_bounds() {
    run(mortonAABBRepopulateKernel, S->groups, true);
    run(mortonAABBCollapseKernel, 1, true);
    return 0;
}

int ref_stage_encode() {
    run(mortonEncodeKernel, S->groups, false);
    return 0;
}

// BarnesHut.radixSort, BarnesHut.java:358-448
int ref_stage_sort() {
    const int passes = 16;  // ceil(63 / RADIX_BITS)
    for (int pass = 0; pass < passes; ++pass) {
        passShift = 4u * (uint)pass;
        run(radixHistogramKernel, S->groups, true);
        run(radixBucketScanKernel, NUM_BUCKETS, true);
        run(radixGlobalScanKernel, NUM_BUCKETS, true);
        run(radixScatterKernel, S->groups, true);
        S->iin = 1 - S->iin;
    }
    return 0;
}

int ref_stage_build() {
    const uint groups = (S->N - 1 + WG_SIZE - 1) / WG_SIZE;
    run(treeBuildBinaryRadixTreeKernel, groups > 0 ? groups : 1, false);
    return 0;
}

// computeCOMAndLocation, BarnesHut.java:474-535 (64 propagate passes)
int ref_stage_fill() {
    run(treeInitLeafNodesKernel, S->groups, false);
    for (int pass = 0; pass < 64; ++pass) {
        long maxNodes = (long)((double)(S->N - 1) / std::pow(2.0, (double)pass));
        if (maxNodes < 4 * (long)WG_SIZE) maxNodes = 4 * WG_SIZE;
        const uint groups = (uint)((maxNodes + WG_SIZE - 1) / WG_SIZE);
        run(treePropagateNodesKernel, groups, false);
        S->qin = 1 - S->qin;
    }
    return 0;
}

int ref_stage_walk(const ref_params* p) {
    set_uniforms(p);
    run(forceComputeKernel, S->groups, false);
    return 0;
}

int ref_stage_merge() {
    run(mergeBodiesKernel, S->groups, false);
    return 0;
}

int ref_stage_swap() {
    S->bin = 1 - S->bin;
    return 0;
}

int ref_step(const ref_params* p) {
    ref_stage_reset(p);
    ref_stage_partition();
    if (p->static_or_dynamic == DYNAMIC) ref_stage_bounds();
    ref_stage_encode();
    ref_stage_sort();
    ref_stage_build();
    ref_stage_fill();
    ref_stage_walk(p);
    ref_stage_merge();
    ref_stage_swap();
    return 0;
}

int ref_read_bodies(uint32_t which, void* host, uint32_t count, uint32_t offset) {
    const std::vector<Body>& b = S->bodies[which == 0 ? S->bin : 1 - S->bin];
    memcpy(host, b.data() + offset, (size_t)count * sizeof(Body));
    return 0;
}
int ref_read_leaf_nodes(void* host, uint32_t count, uint32_t offset) {
    memcpy(host, S->leaf.data() + offset, (size_t)count * sizeof(Node));
    return 0;
}
int ref_read_internal_nodes(void* host, uint32_t count, uint32_t offset) {
    memcpy(host, S->internal.data() + offset, (size_t)count * sizeof(Node));
    return 0;
}
int ref_read_index(void* host, uint32_t count, uint32_t offset) {
    memcpy(host, S->index[S->iin].data() + offset, (size_t)count * 4);
    return 0;
}
int ref_read_morton(void* host, uint32_t count, uint32_t offset) {
    memcpy(host, S->morton[S->iin].data() + offset, (size_t)count * 8);
    return 0;
}
// SimulationValues in the std430 byte layout (896 bytes)
int ref_read_sim_values(void* host) {
    unsigned char* o = (unsigned char*)host;
    memset(o, 0, 896);
    memcpy(o, &sim, 32);
    memcpy(o + 32, &sim.bounds.minCorner, 12);
    memcpy(o + 48, &sim.bounds.maxCorner, 12);
    memcpy(o + 64, &sim.units, 28);
    memcpy(o + 92, sim.uintDebug, 400);
    memcpy(o + 492, sim.floatDebug, 400);
    return 0;
}
int ref_read_merge_tasks(void* host, uint32_t capacity, uint32_t* count) {
    *count = mergeTasksTail;
    uint32_t k = mergeTasksTail < capacity ? mergeTasksTail : capacity;
    if (host && k) memcpy(host, S->tasks.data(), (size_t)k * 8);
    return 0;
}
int ref_write_index(const void* host, uint32_t count, uint32_t offset) {
    memcpy(S->index[S->iin].data() + offset, host, (size_t)count * 4);
    return 0;
}
int ref_write_morton(const void* host, uint32_t count, uint32_t offset) {
    memcpy(S->morton[S->iin].data() + offset, host, (size_t)count * 8);
    return 0;
}
void ref_destroy() {
    delete S;
    S = nullptr;
}

}  // extern "C"
