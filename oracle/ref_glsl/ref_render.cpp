// ref_render.cpp — runs the reference's node-glow and region vertex shaders
// on the CPU, one vertex at a time.
//
// TEST INFRASTRUCTURE ONLY (see render_shim.hpp).  The shader bodies come from
// the reference sources, #included unmodified from
// src/main/resources/shaders/render/ (include path set by the Makefile, with
// render_include/ first so that their #include "common/common.glsl" lands on
// a stand-in).  Each shader sits in a namespace of its own (both define
// main()).  The GLSL storage qualifiers they use (layout, in, out, flat) are
// defined away while they are included.
#include <cstring>

#include "../../include/gbh.h"
#include "render_shim.hpp"

namespace glslr {
Node* internalNodes;
SimulationValues sim;
BodyBuffer srcB;
float cameraScale;
mat4 uMVP, uProj, uModelView;
float uFovY, uAspect;
ivec2 uMinMaxDepth;
uint uRelativeTo;
float uNodeGlowThetaNdc, uNodeGlowActivateDist, uNodeGlowIntensity;
int uNodeGlowMaxDepth;
int gl_InstanceID, gl_VertexID;
vec4 gl_Position;

#define layout(...)
#define in
#define out
#define flat
namespace glow {
#include "render/nodeglow/nodeglow.vert"
}
namespace regions {
#include "render/regions/regions.vert"
}
#undef layout
#undef in
#undef out
#undef flat
}  // namespace glslr

using namespace glslr;

static void set_mat(mat4& M, const float* m16) { memcpy(M.m, m16, 16 * sizeof(float)); }

extern "C" {

// The tree and bodies the shaders read, and the uniforms of a view (mvp: the
// uMVP of the region shader).  `internal` must hold num_bodies internal
// node slots (the region shader visits instances up to num_bodies - 1).
void ref_render_set(gbh_node* internal, gbh_body* bodies, uint32_t num_bodies, uint32_t initial_num_bodies,
                    const gbh_view* v, const float* mvp) {
    internalNodes = reinterpret_cast<Node*>(internal);
    srcB.bodies = reinterpret_cast<Body*>(bodies);
    sim.numBodies = num_bodies;
    sim.initialNumBodies = initial_num_bodies;
    cameraScale = v->camera_scale;
    set_mat(uModelView, v->model_view);
    set_mat(uProj, v->proj);
    set_mat(uMVP, mvp);
    uFovY = v->fov_y;
    uAspect = v->aspect;
    uRelativeTo = v->relative_to;
    uNodeGlowThetaNdc = v->glow_theta_ndc;
    uNodeGlowActivateDist = v->glow_activate_dist;
    uNodeGlowMaxDepth = v->glow_max_depth;
    uNodeGlowIntensity = v->glow_intensity;
    uMinMaxDepth.x = v->region_min_depth;
    uMinMaxDepth.y = v->region_max_depth;
}

// nodeglow.vert for (instance, vertex): out = gl_Position[4], vMapping[2],
// vIntensity, vColor[3], vCenterView[3], vNdcScaleX, vNdcScaleY (16 floats)
void ref_glow_vertex(int instance, int vertex, float* out) {
    gl_InstanceID = instance;
    gl_VertexID = vertex;
    glow::main();
    const float o[16] = {gl_Position.x, gl_Position.y, gl_Position.z, gl_Position.w, glow::vMapping.x,
                         glow::vMapping.y, glow::vIntensity, glow::vColor.x, glow::vColor.y, glow::vColor.z,
                         glow::vCenterView.x, glow::vCenterView.y, glow::vCenterView.z, glow::vNdcScaleX,
                         glow::vNdcScaleY, 0.0f};
    memcpy(out, o, sizeof(o));
}

// regions.vert for (instance, unit-cube corner aPos): out = gl_Position[4],
// uTreeDepth (as a float)
void ref_region_vertex(int instance, const float* apos, float* out) {
    gl_InstanceID = instance;
    regions::aPos = vec3(apos[0], apos[1], apos[2]);
    regions::main();
    out[0] = gl_Position.x;
    out[1] = gl_Position.y;
    out[2] = gl_Position.z;
    out[3] = gl_Position.w;
    out[4] = (float)regions::uTreeDepth;
}

// every instance [0, count) through the vertex shaders: glow out[count][4][16]
// (vertices 0-3), regions out[count][2][5] (unit-cube corners -0.5 and +0.5)
void ref_glow_instances(int count, float* out) {
    for (int i = 0; i < count; ++i)
        for (int vtx = 0; vtx < 4; ++vtx) ref_glow_vertex(i, vtx, out + ((size_t)i * 4 + vtx) * 16);
}
void ref_region_instances(int count, float* out) {
    const float corners[2][3] = {{-0.5f, -0.5f, -0.5f}, {0.5f, 0.5f, 0.5f}};
    for (int i = 0; i < count; ++i)
        for (int k = 0; k < 2; ++k) ref_region_vertex(i, corners[k], out + ((size_t)i * 2 + k) * 5);
}

}  // extern "C"
