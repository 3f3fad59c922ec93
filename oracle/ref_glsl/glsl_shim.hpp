// glsl_shim.hpp — lets the reference's GLSL compute kernels compile as C++.
//
// TEST INFRASTRUCTURE ONLY.  ref_kernels.cpp includes the reference's own
// kernel sources (src/main/resources/shaders/compute/*/bh_*.comp, unmodified)
// after this header.  The header restates, in C++, what those files take from
// GLSL and from the reference's common.glsl:
//   * GLSL types and built-ins (vec3/vec4 with the .xyz/.rgb/.w swizzles the
//     kernels use, min/max/clamp/floor/mod/dot/length/normalize/inversesqrt,
//     atomics, barrier) with GLSL semantics evaluated as IEEE FP32 (compile
//     with -ffp-contract=off; inversesqrt is 1.0f/sqrtf);
//   * the structs, SSBO bindings, uniforms, constants and helper functions of
//     SH/common/common.glsl:25-360 (restated; that file also holds render-only
//     and #version lines and cannot be included as C++);
//   * the compute built-in variables (gl_GlobalInvocationID, ...), set per
//     invocation by the dispatcher in ref_kernels.cpp.
// Workgroup `shared` variables become statics (one workgroup runs at a time).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

typedef unsigned int uint;
using std::uint64_t;

// ---- vectors -------------------------------------------------------------
struct bvec3 {
    bool x, y, z;
};

struct vec3 {
    float x, y, z;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator-=(const vec3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
};
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

struct alignas(16) vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        vec3 xyz;
        vec3 rgb;
    };
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
    vec4(vec3 v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
};

struct uvec2 {
    uint x, y;
    uvec2() = default;
    uvec2(uint a, uint b) : x(a), y(b) {}
};

struct uvec3 {
    uint x, y, z;
};

// ---- built-in functions (GLSL 4.30 chapter 8) ------------------------------
inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline int min(int x, int y) { return (y < x) ? y : x; }
inline int max(int x, int y) { return (x < y) ? y : x; }
inline uint min(uint x, uint y) { return (y < x) ? y : x; }
inline uint max(uint x, uint y) { return (x < y) ? y : x; }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 clamp(vec3 x, vec3 lo, vec3 hi) { return min(max(x, lo), hi); }
inline float floor(float x) { return std::floor(x); }
inline vec3 floor(vec3 v) { return vec3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline vec3 mod(vec3 x, vec3 y) { return x - y * floor(x / y); }
inline float dot(vec3 a, vec3 b) {
    float s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / length(v); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float log(float x) { return std::log(x); }
inline bool isnan(float x) { return std::isnan(x); }
inline bool isinf(float x) { return std::isinf(x); }
inline bvec3 isnan(vec3 v) { return bvec3{std::isnan(v.x), std::isnan(v.y), std::isnan(v.z)}; }
inline bvec3 isinf(vec3 v) { return bvec3{std::isinf(v.x), std::isinf(v.y), std::isinf(v.z)}; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }
inline bvec3 lessThan(vec3 a, vec3 b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec3 greaterThan(vec3 a, vec3 b) { return bvec3{a.x > b.x, a.y > b.y, a.z > b.z}; }
inline int findMSB(uint v) { return v ? 31 - __builtin_clz(v) : -1; }
// atomics: one invocation runs at a time in this harness
inline uint atomicAdd(uint& mem, uint v) { uint o = mem; mem = o + v; return o; }
inline uint atomicCompSwap(uint& mem, uint cmp, uint v) { uint o = mem; if (o == cmp) mem = v; return o; }
inline void memoryBarrierBuffer() {}
void barrier();  // yields to the workgroup scheduler (ref_kernels.cpp)

// ---- compute built-in variables -------------------------------------------
extern uvec3 gl_GlobalInvocationID, gl_LocalInvocationID, gl_WorkGroupID, gl_NumWorkGroups, gl_WorkGroupSize;

// ---- common.glsl:6-20 constants ---------------------------------------------
const uint WG_SIZE = 256u;
const uint RADIX_BITS = 4u;
const uint NUM_BUCKETS = 1u << RADIX_BITS;

// ---- common.glsl:25-70 structs ------------------------------------------------
struct Body {
    vec4 posMass;
    vec4 velDensity;
};

struct AABB {
    vec3 minCorner;
    float pad0;
    vec3 maxCorner;
    float pad1;
    AABB() = default;
    AABB(vec3 a, vec3 b) : minCorner(a), pad0(0), maxCorner(b), pad1(0) {}
};

struct F6 {
    float v[6];
    float& operator[](int i) { return v[i]; }
    const float& operator[](int i) const { return v[i]; }
};

struct Node {
    vec4 comMass;
    F6 aabb;
    uint childA;
    uint childB;
    uint nodeDepth;
    uint bodiesContained;
    uint readyChildren;
    uint parentId;
    vec4 avgColor;
};
static_assert(sizeof(Node) == 80, "Node is 80 bytes (std430)");

struct UnitSet {
    float mass, density, len, time, cameraScale, gravitationalConstant, bodyLengthInSimulationLengthsConstant;
};

// ---- common.glsl:80-120 SSBOs ------------------------------------------------
struct SimulationValues {
    uint numBodies, initialNumBodies, justDied, merged, outOfBounds, relativeTo, pad1, pad2;
    AABB bounds;
    UnitSet units;
    uint uintDebug[100];
    // floatDebug[100] in GLSL; the extra room absorbs the writes of
    // floatDebug[13 + wgId] past index 99 (bh_morton.comp:187)
    float floatDebug[100 + (1 << 20)];
};

struct BodyBuffer {
    Body* bodies;
};
struct WorkQueue {
    uint head, tail;
    uint* items;
};

extern Node* leafNodes;
extern Node* internalNodes;
extern SimulationValues sim;
extern BodyBuffer srcB, dstB;
extern uint64_t* mortonIn;
extern uint64_t* mortonOut;
extern uint* indexIn;
extern uint* indexOut;
extern WorkQueue* g_queue_in;
extern WorkQueue* g_queue_out;
#define headIn (::glsl::g_queue_in->head)
#define tailIn (::glsl::g_queue_in->tail)
#define itemsIn (::glsl::g_queue_in->items)
#define headOut (::glsl::g_queue_out->head)
#define tailOut (::glsl::g_queue_out->tail)
#define itemsOut (::glsl::g_queue_out->items)
extern uint* wgHist;
extern uint* wgScanned;
extern uint bucketTotals[NUM_BUCKETS];
extern uint globalBase[NUM_BUCKETS];
extern uint mergeTasksHead, mergeTasksTail;
extern uvec2* mergeTasks;
extern uint* bodyLocks;

// ---- common.glsl:126-158 uniforms (compute) ------------------------------------
extern uint resetValuesOrDecrementDeadBodies;
extern float softening, theta, dt;
extern uint mergingCollisionOrNeither;
extern float cameraScale, elasticity, restitution, bothCriterion;
extern bool wrapAround;
extern uint staticOrDynamic;
extern uint passShift;
extern uint numWorkGroups;
extern float mass, density, len, time;
extern float g_gravity_override;  // harness: > 0 replaces the derived G (stated deviation)

const uint NEITHER = 0u;
const uint MERGING = 1u;
const uint COLLISION = 2u;
const uint BOTH = 3u;
const uint STATIC = 0u;
const uint DYNAMIC = 1u;

// ---- common.glsl:187-198 constants ------------------------------------------------
inline Body make_empty_body() {
    Body b;
    b.posMass = vec4(0.0f);
    b.velDensity = vec4(0.0f);
    return b;
}
const Body EMPTY_BODY = make_empty_body();
const AABB DEFAULT_AABB = AABB(vec3(1e38f), vec3(-1e38f));
const float PI = 3.14159265358979323846f;
const float THREE_OVER_FOUR_PI_TO_THE_ONE_THIRD = 0.6203504909f;
const float GRAVITATIONAL_CONSTANT = 6.67430e-11f;

// ---- common.glsl:202-342 helpers ---------------------------------------------------
inline bool isEmpty(Body b) { return b.posMass.w == 0.0f; }
inline bool outOfBounds(Body b) {
    return b.posMass.x < sim.bounds.minCorner.x || b.posMass.x > sim.bounds.maxCorner.x ||
           b.posMass.y < sim.bounds.minCorner.y || b.posMass.y > sim.bounds.maxCorner.y ||
           b.posMass.z < sim.bounds.minCorner.z || b.posMass.z > sim.bounds.maxCorner.z;
}
inline float scaledDensity(Body b) { return b.velDensity.w * sim.units.density; }
inline float scaledMass(Body b) { return b.posMass.w * sim.units.mass; }
inline float scaledMass(Node n) { return n.comMass.w * sim.units.mass; }
inline float radius(Body b) {
    return sim.units.bodyLengthInSimulationLengthsConstant * pow(b.posMass.w / b.velDensity.w, 1.0f / 3.0f);
}
inline float starTemp(float m, float d) {
    float constant = 5.95589e-19f;
    return constant * pow(m, 0.875f - 1.0f / 6.0f) * pow(d, 1.0f / 6.0f);
}
inline vec3 tempToColor(float kelvin) {
    float temp = kelvin / 100.0f;
    float r, g, b;
    if (temp <= 66.0f) {
        r = 255.0f;
    } else {
        r = temp - 60.0f;
        r = 329.698727446f * pow(r, -0.1332047592f);
    }
    if (temp <= 66.0f) {
        g = 99.4708025861f * log(max(temp, 1e-3f)) - 161.1195681661f;
    } else {
        g = temp;
        g = 288.1221695283f * pow(g, -0.0755148492f);
    }
    if (temp >= 66.0f) {
        b = 255.0f;
    } else {
        b = temp - 10.0f;
        b = 138.5177312231f * log(max(b, 1e-3f)) - 305.0447927307f;
    }
    return vec3(clamp(r, 0.0f, 255.0f) / 255.0f, clamp(g, 0.0f, 255.0f) / 255.0f, clamp(b, 0.0f, 255.0f) / 255.0f);
}
inline vec3 getStarColor(float m, float d) { return tempToColor(starTemp(m, d)); }
inline AABB updateAABB(AABB a, AABB b) { return AABB(min(a.minCorner, b.minCorner), max(a.maxCorner, b.maxCorner)); }
inline AABB unpackAABB(F6 a) { return AABB(vec3(a[0], a[1], a[2]), vec3(a[3], a[4], a[5])); }
inline F6 packAABB(AABB a) {
    F6 r = {{a.minCorner.x, a.minCorner.y, a.minCorner.z, a.maxCorner.x, a.maxCorner.y, a.maxCorner.z}};
    return r;
}
inline bool emptyAABB(AABB a) { return a.minCorner.x > a.maxCorner.x; }
inline bool emptyAABB(F6 a) { return a[0] > a[3]; }
inline Node getNode(uint nodeIdx) {
    return nodeIdx < sim.initialNumBodies ? leafNodes[nodeIdx] : internalNodes[nodeIdx - sim.initialNumBodies];
}
inline bool isInternalNode(Node n) { return n.childA != 0xFFFFFFFFu; }
inline void setScaledGravitationalConstant(UnitSet) {
    if (g_gravity_override > 0.0f) {
        sim.units.gravitationalConstant = g_gravity_override;
        return;
    }
    sim.units.gravitationalConstant =
        GRAVITATIONAL_CONSTANT * pow(sim.units.len, -3.0f) * pow(sim.units.time, 2.0f) * pow(sim.units.mass, 1.0f);
}
inline void setScaledBodyLengthInSimulationLengthsConstant(UnitSet) {
    sim.units.bodyLengthInSimulationLengthsConstant =
        THREE_OVER_FOUR_PI_TO_THE_ONE_THIRD * pow((sim.units.mass / sim.units.density), 1.0f / 3.0f) / sim.units.len;
}
inline void updateUnits(float m, float d, float l, float t) {
    sim.units.mass = m;
    sim.units.density = d;
    sim.units.len = l;
    sim.units.time = t;
    setScaledGravitationalConstant(sim.units);
    setScaledBodyLengthInSimulationLengthsConstant(sim.units);
}

}  // namespace glsl

// ---- GLSL qualifiers used by the kernel files -------------------------------------
#define shared static
// `out` parameters (bh_morton.comp:50, mortonInlierWindow) are GLSL copy-out
// parameters.  The macros below turn that one declaration into reference
// parameters and leave the call site unchanged: the first macro argument of
// the declaration starts with GLSL_OUT_, the call's does not.
#define out GLSL_OUT_
#define GLSL_CAT(a, ...) GLSL_CAT_I(a, __VA_ARGS__)
#define GLSL_CAT_I(a, ...) a##__VA_ARGS__
#define GLSL_SECOND(a, b, ...) b
#define GLSL_CHECK(...) GLSL_SECOND(__VA_ARGS__, 0, )
#define GLSL_PROBE ~, 1,
#define GLSL_IS_OUT_GLSL_OUT_ GLSL_PROBE
#define mortonInlierWindow(a, b) GLSL_CAT(GLSL_MIW_, GLSL_CHECK(GLSL_CAT(GLSL_IS_OUT_, a)))(a, b)
#define GLSL_MIW_1(a, b) mortonInlierWindow_ref(vec3& lo, vec3& hi)
#define GLSL_MIW_0(a, b) mortonInlierWindow_ref(a, b)
