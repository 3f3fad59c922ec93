// k_view.cu — headless level-of-detail selection over the tree's internal
// nodes: the per-node arithmetic of the reference's hierarchical node glow
// (src/main/resources/shaders/render/nodeglow/nodeglow.vert:46-150) and region
// boxes (shaders/render/regions/regions.vert:19-45), as kernels that append
// one record per selected node to a device buffer instead of drawing.
//
// One thread per live internal node; a warp reserves its records with one
// atomic.  Arithmetic: FP32, one rounding per operation in source order (this
// translation unit is compiled without multiply-add contraction), matrix times
// vector as column 0 + column 1 + column 2 + column 3, so a C restatement in
// the same operation order gives the same bits.
#include <cmath>
#include <string>

#include "gbh_ctx.h"

namespace {

struct ViewConsts {
    gbh_view v;
    float tan_half_fov;  // tan(fov_y / 2), once on the host
};

__device__ __forceinline__ bool empty_aabb(const float* aabb) { return aabb[0] > aabb[3]; }

// relativeLocation (common.glsl:291-299)
__device__ __forceinline__ float3 relative_location(float3 a, uint32_t rel, uint32_t N, const gbh_body* bodies) {
    if (rel == 0xFFFFFFFFu || rel >= N) return a;
    const float4 p = *reinterpret_cast<const float4*>(bodies[rel].pos_mass);
    return make_float3(a.x - p.x, a.y - p.y, a.z - p.z);
}

// column-major mat4 times vec4, columns summed in order
__device__ __forceinline__ float4 mat4_mul(const float* m, float4 v) {
    float4 r;
    r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
    r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
    r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
    r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
    return r;
}

__device__ __forceinline__ float smoothstep_f(float e0, float e1, float x) {
    float t = (x - e0) / (e1 - e0);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// warp-aggregated append: one atomic per warp, records past `cap` dropped
__device__ __forceinline__ uint32_t append_slot(bool take, uint32_t* counter) {
    const uint32_t m = __ballot_sync(0xffffffffu, take);
    if (!m) return 0xFFFFFFFFu;
    const uint32_t lane = lane_id(), leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return take ? base + __popc(m & lanemask_lt()) : 0xFFFFFFFFu;
}

// nodeglow.vert:46-150 for internal node i; true when it is drawn
__device__ bool glow_node(const gbh_node& nd, const ViewConsts& V, uint32_t N, const gbh_body* bodies,
                          gbh_glow_splat& out) {
    const gbh_view& v = V.v;
    if (empty_aabb(nd.aabb) || nd.com_mass[3] <= 0.0f || nd.bodies_contained == 0u) return false;
    const uint32_t depth = nd.node_depth;
    if (depth < 1u || depth > (uint32_t)v.glow_max_depth) return false;
    const float cs = v.camera_scale;
    const float3 mn = relative_location(make_float3(nd.aabb[0], nd.aabb[1], nd.aabb[2]), v.relative_to, N, bodies);
    const float3 mx = relative_location(make_float3(nd.aabb[3], nd.aabb[4], nd.aabb[5]), v.relative_to, N, bodies);
    const float3 minC = make_float3(mn.x * cs, mn.y * cs, mn.z * cs);
    const float3 maxC = make_float3(mx.x * cs, mx.y * cs, mx.z * cs);
    const float sx = maxC.x - minC.x, sy = maxC.y - minC.y, sz = maxC.z - minC.z;
    const float longest = fmaxf(sx, fmaxf(sy, sz));
    const float half_extent = 0.5f * longest;
    const float3 c = relative_location(make_float3(nd.com_mass[0], nd.com_mass[1], nd.com_mass[2]), v.relative_to, N,
                                       bodies);
    const float4 cv = mat4_mul(v.model_view, make_float4(c.x * cs, c.y * cs, c.z * cs, 1.0f));
    const float cam_dist = fmaxf(-cv.z, 1e-6f);
    if (cam_dist < v.glow_activate_dist) return false;
    const float th = V.tan_half_fov;
    const float projected = longest / (cam_dist * th);
    const float theta_ndc = fmaxf(v.glow_theta_ndc, 1e-6f);
    const float min_ndc = theta_ndc * 0.04f;
    if (projected >= theta_ndc || projected < min_ndc) return false;
    float accept = 1.0f - smoothstep_f(theta_ndc * 0.75f, theta_ndc, projected);
    accept = accept * smoothstep_f(min_ndc, min_ndc * 2.5f, projected);
    const float area = fmaxf(projected * projected, 1e-8f);
    const float luminosity = nd.com_mass[3] * (1.0e6f / (cam_dist * cam_dist));
    const float surface = luminosity / area;
    const float raw = surface * 2.5e-4f * accept * v.glow_intensity;
    const float intensity = raw / (1.0f + raw);
    if (intensity < 1e-4f) return false;
    const float4 clip = mat4_mul(v.proj, cv);
    const float glow_half = fmaxf(half_extent * 1.1f, min_ndc * 0.5f * cam_dist * th);
    const float ndc_y = glow_half / (cam_dist * th);
    const float ndc_x = ndc_y / fmaxf(v.aspect, 1e-6f);
    out.center_clip[0] = clip.x;
    out.center_clip[1] = clip.y;
    out.center_clip[2] = clip.z;
    out.center_clip[3] = clip.w;
    out.center_view[0] = cv.x;
    out.center_view[1] = cv.y;
    out.center_view[2] = cv.z;
    out.intensity = intensity;
    out.color[0] = nd.avg_color[0];
    out.color[1] = nd.avg_color[1];
    out.color[2] = nd.avg_color[2];
    out.ndc_scale[0] = ndc_x;
    out.ndc_scale[1] = ndc_y;
    out.depth = depth;
    out.pad = 0;
    return true;
}

__global__ void k_select_glow(const gbh_node* __restrict__ internal, const gbh_body* __restrict__ bodies,
                              const DevState* __restrict__ st, uint32_t N, ViewConsts V, gbh_glow_splat* out,
                              uint32_t cap, uint32_t* counter) {
    const uint32_t n = st->n_new;
    const uint32_t live = n > 1 ? n - 1 : 0;
    const uint32_t start = blockIdx.x * blockDim.x;
    if (start >= live) return;  // whole block past the live nodes
    const uint32_t i = start + threadIdx.x;
    gbh_glow_splat rec;
    bool take = false;
    if (i < live) {
        const gbh_node nd = internal[i];
        take = glow_node(nd, V, N, bodies, rec);
    }
    const uint32_t slot = append_slot(take, counter);
    if (take && slot < cap) {
        rec.node = i;
        out[slot] = rec;
    }
}

// regions.vert:19-45 for internal node i
__global__ void k_select_regions(const gbh_node* __restrict__ internal, const gbh_body* __restrict__ bodies,
                                 const DevState* __restrict__ st, uint32_t N, ViewConsts V, gbh_region* out,
                                 uint32_t cap, uint32_t* counter) {
    const uint32_t n = st->n_new;
    const uint32_t live = n > 1 ? n - 1 : 0;
    const uint32_t start = blockIdx.x * blockDim.x;
    if (start >= live) return;
    const uint32_t i = start + threadIdx.x;
    const gbh_view& v = V.v;
    gbh_region rec;
    bool take = false;
    if (i < live) {
        const gbh_node nd = internal[i];
        if (!empty_aabb(nd.aabb) && !(nd.node_depth < (uint32_t)v.region_min_depth) &&
            !(nd.node_depth > (uint32_t)v.region_max_depth)) {
            const float cs = v.camera_scale;
            const float3 mn =
                relative_location(make_float3(nd.aabb[0], nd.aabb[1], nd.aabb[2]), v.relative_to, N, bodies);
            const float3 mx =
                relative_location(make_float3(nd.aabb[3], nd.aabb[4], nd.aabb[5]), v.relative_to, N, bodies);
            const float3 minC = make_float3(mn.x * cs, mn.y * cs, mn.z * cs);
            const float3 maxC = make_float3(mx.x * cs, mx.y * cs, mx.z * cs);
            rec.center[0] = (minC.x + maxC.x) * 0.5f;
            rec.center[1] = (minC.y + maxC.y) * 0.5f;
            rec.center[2] = (minC.z + maxC.z) * 0.5f;
            rec.size[0] = maxC.x - minC.x;
            rec.size[1] = maxC.y - minC.y;
            rec.size[2] = maxC.z - minC.z;
            rec.node = i;
            rec.depth = nd.node_depth;
            take = true;
        }
    }
    const uint32_t slot = append_slot(take, counter);
    if (take && slot < cap) out[slot] = rec;
}

int view_fail(gbh_ctx* c, int code, const std::string& m) {
    c->last_error = m;
    return code;
}

}  // namespace

static int select_common(gbh_ctx* c, const gbh_view* view, void* out, uint32_t* count, bool glow,
                         uint32_t capacity) {
    if (!c || !view || !count || (!out && capacity)) return c ? view_fail(c, GBH_ERR_INVALID, "null argument") : GBH_ERR_INVALID;
    if (!c->inited) return view_fail(c, GBH_ERR_STATE, "selection before init");
    if (cudaSetDevice(c->device) != cudaSuccess) return view_fail(c, GBH_ERR_CUDA, "cudaSetDevice");
    ViewConsts V;
    V.v = *view;
    V.tan_half_fov = tanf(0.5f * view->fov_y);
    uint32_t* counter = &c->st->view_count;
    cudaError_t e = cudaMemsetAsync(counter, 0, 4, c->stream);
    const uint32_t nodes = c->N > 1 ? c->N - 1 : 1;
    const uint32_t threads = 256, blocks = (nodes + threads - 1) / threads;
    if (e == cudaSuccess) {
        const gbh_body* bodies = c->bodies[c->bin];
        if (glow)
            k_select_glow<<<blocks, threads, 0, c->stream>>>(c->internal, bodies, c->st, c->N, V,
                                                             static_cast<gbh_glow_splat*>(out), capacity, counter);
        else
            k_select_regions<<<blocks, threads, 0, c->stream>>>(c->internal, bodies, c->st, c->N, V,
                                                                static_cast<gbh_region*>(out), capacity, counter);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(count, counter, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return view_fail(c, GBH_ERR_CUDA, std::string("node selection: ") + cudaGetErrorString(e));
    return GBH_OK;
}

extern "C" {

int gbh_select_glow_nodes(gbh_ctx* c, const gbh_view* view, gbh_glow_splat* out_device, uint32_t capacity,
                          uint32_t* count) {
    return select_common(c, view, out_device, count, true, capacity);
}

int gbh_select_regions(gbh_ctx* c, const gbh_view* view, gbh_region* out_device, uint32_t capacity,
                       uint32_t* count) {
    return select_common(c, view, out_device, count, false, capacity);
}

}  // extern "C"
