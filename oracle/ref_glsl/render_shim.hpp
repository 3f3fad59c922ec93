// render_shim.hpp — lets the reference's node-glow and region vertex shaders
// (src/main/resources/shaders/render/nodeglow/nodeglow.vert,
// render/regions/regions.vert) compile as C++.
//
// TEST INFRASTRUCTURE ONLY.  ref_render.cpp includes those two files,
// unmodified, after this header.  It restates what they take from GLSL and
// from the reference's common.glsl: the vector and matrix types with the
// swizzles the shaders use, min/max/clamp/smoothstep/tan with GLSL semantics
// in IEEE FP32 (the Makefile compiles with -ffp-contract=off and
// -fsingle-precision-constant, so literals are single precision as in GLSL),
// the Node and Body layouts (common.glsl:25-58), the render uniforms
// (common.glsl:160-182), relativeLocation and emptyAABB (common.glsl:291-334),
// and the vertex built-ins (gl_InstanceID, gl_VertexID, gl_Position).
// mat4 * vec4 adds the four column terms in column order.
#pragma once

#include <cmath>
#include <cstdint>

namespace glslr {

typedef unsigned int uint;

struct vec2 {
    float x, y;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
};
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }

struct vec3 {
    float x, y, z;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        vec3 xyz;
        vec3 rgb;
        vec2 xy;
    };
    vec4() = default;
    vec4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
    vec4(vec3 v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
    vec4(vec2 v, float c_, float d_) : x(v.x), y(v.y), z(c_), w(d_) {}
};

struct ivec2 {
    int x, y;
};

// column-major, m[column][row] (GLSL mat4 memory order)
struct mat4 {
    float m[4][4];
};
inline vec4 operator*(const mat4& M, vec4 v) {
    float o[4];
    for (int i = 0; i < 4; ++i) {
        float s = M.m[0][i] * v.x;
        s = s + M.m[1][i] * v.y;
        s = s + M.m[2][i] * v.z;
        s = s + M.m[3][i] * v.w;
        o[i] = s;
    }
    return vec4(o[0], o[1], o[2], o[3]);
}

inline float min(float x, float y) { return (y < x) ? y : x; }
inline float max(float x, float y) { return (x < y) ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
// GLSL 4.30 8.3: t = clamp((x - edge0) / (edge1 - edge0), 0, 1); t * t * (3 - 2 t)
inline float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float tan(float x) { return std::tan(x); }

struct F6 {
    float v[6];
    float& operator[](int i) { return v[i]; }
    const float& operator[](int i) const { return v[i]; }
};
struct Node {
    vec4 comMass;
    F6 aabb;
    uint childA, childB, nodeDepth, bodiesContained, readyChildren, parentId;
    vec4 avgColor;
};
static_assert(sizeof(Node) == 80, "Node is 80 bytes (std430)");
struct Body {
    vec4 posMass;
    vec4 velDensity;
};
struct SimulationValues {
    uint numBodies, initialNumBodies;
};
struct BodyBuffer {
    Body* bodies;
};

// buffers and uniforms, set by ref_render.cpp before each invocation
extern Node* internalNodes;
extern SimulationValues sim;
extern BodyBuffer srcB;
extern float cameraScale;
extern mat4 uMVP, uProj, uModelView;
extern float uFovY, uAspect;
extern ivec2 uMinMaxDepth;
extern uint uRelativeTo;
extern float uNodeGlowThetaNdc, uNodeGlowActivateDist, uNodeGlowIntensity;
extern int uNodeGlowMaxDepth;
extern int gl_InstanceID, gl_VertexID;
extern vec4 gl_Position;

// common.glsl:291-299
inline vec3 relativeLocation(vec3 a, uint relativeTo) {
    if (relativeTo == 0xFFFFFFFFu) return a;
    if (relativeTo >= sim.initialNumBodies) return a;
    const vec4 p = srcB.bodies[relativeTo].posMass;
    return a - p.xyz;
}
// common.glsl:332-334
inline bool emptyAABB(const F6& aabb) { return aabb[0] > aabb[3]; }

}  // namespace glslr
