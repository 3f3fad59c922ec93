// k_mac.cu — the learned multipole-acceptance criterion: weights, training
// data, training (hand-written forward, backward and Adam kernels) and the
// learned walk's launch.
//
// Training data (gbh_mac_generate):
//   1. the current state's tree is built and walked with the plain theta = 0.2
//      rule, which stores every body's acceleration (the normaliser a_i);
//   2. two group walks, with a conservative (theta_g = 0.25) and a loose
//      (theta_g = 0.6) group rule, record the (group, node) candidate pairs
//      they evaluate with their features, half of the budget each;
//   3. k_mac_label computes each pair's label: for every body i of the group,
//      the monopole of the node against the node's subtree sum, relative to
//      |a_i|; the label is log10 of the maximum over the group.  Subtrees of
//      at most 1024 bodies are summed exactly over their contiguous sorted
//      leaf range; larger ones by a strict walk of the subtree.
//   Which pairs are kept depends only on (group, node): the group is named by
//   its first sorted slot, and a pass that would overflow the budget is run
//   again with a smaller keep fraction.  The kept pairs are then sorted by
//   (group, node) with the step's radix sort, so that the pair list, and
//   with it every minibatch, is the same in every run.
// Training (gbh_mac_train): minibatches drawn with a counter-based hash; the
// forward pass is the inference code (BF16 mma.sync, FP32 accumulation), the
// backward pass runs in FP32 on the CUDA cores (straight-through for the BF16
// rounding), each warp writes its gradient sums, one kernel adds them in warp
// order (no float atomics: training is bit-reproducible), then Adam updates
// the FP32 master weights and rebuilds the BF16 fragment table.
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "gbh_ctx.h"
#include "mac_mlp.cuh"

void launch_walk_group(const StepBuffers& b, const MacDeviceWeights& mw, bool learned, cudaStream_t s);
void launch_walk_group_record(const StepBuffers& b, const MacDeviceWeights& mw, cudaStream_t s);
int enqueue_reset(gbh_ctx* c);
int enqueue_prepare(gbh_ctx* c);
int enqueue_sort(gbh_ctx* c);
int enqueue_build(gbh_ctx* c);
int enqueue_fill(gbh_ctx* c);

#define MAC_TRAIN_WARPS 4
#define MAC_LABEL_MAX_BODIES 1024
#define MAC_LABEL_STACK 160

struct MacState {
    float* params = nullptr;  // FP32 master weights
    float* grad = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    uint32_t* frag = nullptr;  // BF16/FP32 fragment table [MAC_FRAG_WORDS][32]
    float* loss = nullptr;     // device accumulators [2]
    float* feats = nullptr;    // training pairs [cap][12]
    float* labels = nullptr;   // [cap]
    uint2* pairs = nullptr;    // [cap] (group, node)
    uint32_t* count = nullptr; // device counter
    float* band = nullptr;     // device [2]: the learned walk's band (group-rule thetas)
    float band_host[2] = {MAC_BAND_LO, MAC_BAND_HI};
    uint32_t cap = 0;
    uint32_t num_pairs = 0;
    uint64_t adam_t = 0;
    // sorting the recorded pairs by (group, node): keys and row indices
    // (ping-pong), the sort's histograms, look-back words and counters, and
    // the gathered copies of the pairs and features
    uint64_t* skeys[2] = {nullptr, nullptr};
    uint32_t* svals[2] = {nullptr, nullptr};
    uint32_t* shist = nullptr;
    uint32_t* sbase = nullptr;
    uint32_t* slook = nullptr;
    DevState* sst = nullptr;
    uint32_t stiles = 0;
    float* feats_tmp = nullptr;
    uint2* pairs_tmp = nullptr;
    // per-warp gradient sums of one training step [warps][MAC_NPARAMS + 1]
    float* part = nullptr;
    uint32_t part_warps = 0;
};

#define MAC_PART_STRIDE (MAC_NPARAMS + 1)  // the parameters' gradients, then the loss

// ---------------------------------------------------------------------------
// fragment table from the FP32 parameters (layout in mac_mlp.cuh)
__global__ void k_mac_build_frag(const float* __restrict__ p, uint32_t* __restrict__ frag) {
    const uint32_t lane = threadIdx.x;
    const uint32_t gid = lane >> 2, tig = lane & 3;
    const float* W1 = p + MAC_OFF_W1;
    const float* W2 = p + MAC_OFF_W2;
    const float* w3 = p + MAC_OFF_W3;
    auto w1 = [&](uint32_t o, uint32_t k) { return k < MAC_FEATURES ? W1[o * MAC_FEATURES + k] : 0.0f; };
    for (int nt = 0; nt < 4; ++nt) {
        const uint32_t o = 8 * nt + gid;
        frag[(2 * nt) * 32 + lane] = pack_bf16x2(w1(o, 2 * tig), w1(o, 2 * tig + 1));
        frag[(2 * nt + 1) * 32 + lane] = pack_bf16x2(w1(o, 2 * tig + 8), w1(o, 2 * tig + 9));
        for (int ks = 0; ks < 2; ++ks) {
            const uint32_t k = 16 * ks + 2 * tig;
            frag[(MAC_FRAG_W1 + (nt * 2 + ks) * 2) * 32 + lane] = pack_bf16x2(W2[o * 32 + k], W2[o * 32 + k + 1]);
            frag[(MAC_FRAG_W1 + (nt * 2 + ks) * 2 + 1) * 32 + lane] =
                pack_bf16x2(W2[o * 32 + k + 8], W2[o * 32 + k + 9]);
        }
    }
    for (int ks = 0; ks < 2; ++ks) {
        const uint32_t k = 16 * ks + 2 * tig;
        const bool col0 = gid == 0;
        frag[(MAC_FRAG_W1 + MAC_FRAG_W2 + 2 * ks) * 32 + lane] = col0 ? pack_bf16x2(w3[k], w3[k + 1]) : 0u;
        frag[(MAC_FRAG_W1 + MAC_FRAG_W2 + 2 * ks + 1) * 32 + lane] = col0 ? pack_bf16x2(w3[k + 8], w3[k + 9]) : 0u;
    }
    const int b1o = MAC_FRAG_W1 + MAC_FRAG_W2 + MAC_FRAG_W3;
    const int b2o = b1o + MAC_FRAG_B1;
    for (int nt = 0; nt < 4; ++nt)
        for (int c = 0; c < 2; ++c) {
            frag[(b1o + 2 * nt + c) * 32 + lane] = __float_as_uint(p[MAC_OFF_B1 + 8 * nt + 2 * tig + c]);
            frag[(b2o + 2 * nt + c) * 32 + lane] = __float_as_uint(p[MAC_OFF_B2 + 8 * nt + 2 * tig + c]);
        }
    frag[(MAC_FRAG_WORDS - 1) * 32 + lane] = __float_as_uint(p[MAC_OFF_B3]);
}

// ---------------------------------------------------------------------------
// inference over stored features (one warp per 32 rows)
__global__ void k_mac_predict(const float* __restrict__ feats, uint32_t n, float* __restrict__ out,
                              MacDeviceWeights mw) {
    __shared__ __align__(16) uint32_t s_frag[MAC_SMEM_FRAG_WORDS];
    __shared__ __nv_bfloat16 s_x[MAC_TRAIN_WARPS * 32 * 16];
    mac_load_frag(mw, s_frag, s_x);
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t row = (blockIdx.x * MAC_TRAIN_WARPS + w) * 32 + lane;
    float f[MAC_FEATURES];
#pragma unroll
    for (int k = 0; k < MAC_FEATURES; ++k) f[k] = row < n ? feats[(size_t)row * MAC_FEATURES + k] : 0.0f;
    mac_stage_features(mw, w, lane, f);
    const float y = mac_infer_warp(mw, w, lane);
    if (row < n) out[row] = y;
}

// ---------------------------------------------------------------------------
// labels of recorded pairs: one warp per pair
// Relative error of the node's monopole against its exact subtree sum on the
// body in sorted slot g (accelerations of the last reference walk in b.accel).
__device__ float mac_label_body(const StepBuffers& b, uint32_t node, uint32_t g) {
    const uint32_t N = b.N;
    const float G = b.sim->gravitational_constant;
    const float soft = b.params->softening;
    const float4 pm = b.leaf_pm[g];
    const gbh_node* nd = &b.internal[node - N];
    const float4 cm = *reinterpret_cast<const float4*>(nd);
    const uint32_t cnt = nd->bodies_contained;
    float ex = 0.f, ey = 0.f, ez = 0.f;
    if (cnt <= MAC_LABEL_MAX_BODIES) {
        // exact: every body of the subtree (its contiguous sorted range, which
        // starts at the subtree's leftmost leaf)
        uint32_t id = node;
        while (id >= N) id = b.internal[id - N].child_a;
        const uint32_t lo = id;
        for (uint32_t j = lo; j < lo + cnt; ++j) {
            if (j == g) continue;
            const float4 o = b.leaf_pm[j];
            const float rx = o.x - pm.x, ry = o.y - pm.y, rz = o.z - pm.z;
            const float inv = rsqrtf(rx * rx + ry * ry + rz * rz + soft);
            const float f = G * o.w * inv * inv * inv;
            ex = fmaf(f, rx, ex);
            ey = fmaf(f, ry, ey);
            ez = fmaf(f, rz, ez);
        }
    } else {
        // large subtree: a strict per-body walk of the subtree (theta 0.05 on
        // the half side), accurate to ~1e-5 of the subtree's pull
        uint32_t stack[MAC_LABEL_STACK];
        uint32_t sp = 0;
        stack[sp++] = node;
        while (sp > 0) {
            const uint32_t id = stack[--sp];
            if (id < N) {
                if (id == g) continue;
                const float4 o = b.leaf_pm[id];
                const float rx = o.x - pm.x, ry = o.y - pm.y, rz = o.z - pm.z;
                const float inv = rsqrtf(rx * rx + ry * ry + rz * rz + soft);
                const float f = G * o.w * inv * inv * inv;
                ex = fmaf(f, rx, ex);
                ey = fmaf(f, ry, ey);
                ez = fmaf(f, rz, ez);
                continue;
            }
            const float4* q = reinterpret_cast<const float4*>(&b.internal[id - N]);
            const float4 c = q[0];
            const float4 a0 = q[1];
            const float4 a1 = q[2];
            const float half = 0.5f * fmaxf(a0.w - a0.x, fmaxf(a1.x - a0.y, a1.y - a0.z));
            const float rx = c.x - pm.x, ry = c.y - pm.y, rz = c.z - pm.z;
            const float rr = rx * rx + ry * ry + rz * rz;
            const bool inside = pm.x >= a0.x && pm.x <= a0.w && pm.y >= a0.y && pm.y <= a1.x && pm.z >= a0.z &&
                                pm.z <= a1.y;
            if (!inside && half * half < 0.0025f * rr) {
                const float inv = rsqrtf(rr + soft);
                const float f = G * c.w * inv * inv * inv;
                ex = fmaf(f, rx, ex);
                ey = fmaf(f, ry, ey);
                ez = fmaf(f, rz, ez);
            } else if (sp + 2 <= MAC_LABEL_STACK) {
                stack[sp++] = __float_as_uint(a1.z);
                stack[sp++] = __float_as_uint(a1.w);
            }
        }
    }
    const float rx = cm.x - pm.x, ry = cm.y - pm.y, rz = cm.z - pm.z;
    const float inv = rsqrtf(rx * rx + ry * ry + rz * rz + soft);
    const float f = G * cm.w * inv * inv * inv;
    const float dx = f * rx - ex, dy = f * ry - ey, dz = f * rz - ez;
    const float4 a = b.accel[b.idx_in[g]];
    const float amag = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return sqrtf(dx * dx + dy * dy + dz * dz) / fmaxf(amag, 1e-30f);
}

// One warp per pair: lane l takes the group's bodies l, l + 32, ...; the label
// is log10 of the largest error over the group.
__global__ void k_mac_label(StepBuffers b, const uint2* __restrict__ pairs, const uint32_t* __restrict__ count,
                            float* __restrict__ labels) {
    const uint32_t lane = lane_id();
    const uint32_t p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t np = *count;
    if (p >= np) return;
    const uint2 pr = pairs[p];
    const uint2 grp = b.groups[pr.x];
    float err = 0.0f;
    for (uint32_t k = lane; k < grp.y; k += 32) err = fmaxf(err, mac_label_body(b, pr.y, grp.x + k));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err = fmaxf(err, __shfl_xor_sync(0xffffffffu, err, o));
    if (lane == 0) labels[p] = log10f(fmaxf(err, 1e-12f));
}

// ---------------------------------------------------------------------------
// canonical order of the recorded pairs: key (group's first sorted slot, node)
__global__ void k_mac_pair_keys(const uint2* __restrict__ pairs, const uint2* __restrict__ groups, uint32_t n,
                                uint64_t* __restrict__ keys, uint32_t* __restrict__ rows) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint2 pr = pairs[p];
    keys[p] = ((uint64_t)groups[pr.x].x << 32) | pr.y;
    rows[p] = p;
}

__global__ void k_mac_gather_pairs(const uint32_t* __restrict__ rows, uint32_t n, const float* __restrict__ feats,
                                   const uint2* __restrict__ pairs, float* __restrict__ feats_out,
                                   uint2* __restrict__ pairs_out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint32_t src = rows[r];
#pragma unroll
    for (int k = 0; k < MAC_FEATURES; ++k) feats_out[(size_t)r * MAC_FEATURES + k] = feats[(size_t)src * MAC_FEATURES + k];
    pairs_out[r] = pairs[src];
}

// ---------------------------------------------------------------------------
// training: forward (tensor cores) + backward (FP32) of 32 samples per warp
struct TrainSmem {
    alignas(16) uint32_t frag[MAC_SMEM_FRAG_WORDS];
    __nv_bfloat16 x[MAC_TRAIN_WARPS * 32 * 16];
    float h1[MAC_TRAIN_WARPS][32][33];
    float h2[MAC_TRAIN_WARPS][32][33];
    float dz2[MAC_TRAIN_WARPS][32][33];
    float dz1[MAC_TRAIN_WARPS][32][33];
    float dy[MAC_TRAIN_WARPS][32];
};

__device__ __forceinline__ uint32_t sample_index(uint32_t seed, uint32_t step, uint32_t i, uint32_t n) {
    return hash32(hash32(seed * 0x9E3779B9u + step) ^ (i * 0x85EBCA6Bu)) % n;
}

// random = 1: sample indices with the hash; 0: rows [0, total) in order
__global__ __launch_bounds__(MAC_TRAIN_WARPS * 32) void k_mac_train_step(
    const float* __restrict__ feats, const float* __restrict__ labels, uint32_t n_pairs, uint32_t total,
    int random, uint32_t seed, uint32_t step, MacDeviceWeights mw, const float* __restrict__ params,
    float* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    mac_load_frag(mw, S.frag, S.x);
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t i = (blockIdx.x * MAC_TRAIN_WARPS + w) * 32 + lane;
    const bool valid = i < total;
    const uint32_t row = valid ? (random ? sample_index(seed, step, i, n_pairs) : i) : 0u;
    float f[MAC_FEATURES];
#pragma unroll
    for (int k = 0; k < MAC_FEATURES; ++k) f[k] = valid ? feats[(size_t)row * MAC_FEATURES + k] : 0.0f;
    const float y = valid ? labels[row] : 0.0f;
    mac_stage_features(mw, w, lane, f);
    MacActs acts;
    const float pred = mac_forward_warp<true>(mw, w, lane, &acts);
    // loss: mean squared error over `total` samples
    const float e = pred - y;
    float l = valid ? e * e : 0.0f;
    const float d = valid ? 2.0f * e / (float)total : 0.0f;
    // activations to shared memory, [sample][unit]
    const uint32_t gid = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const uint32_t rr = 16 * mt + gid + 8 * (r >> 1), cc = 8 * nt + 2 * tig + (r & 1);
                S.h1[w][rr][cc] = acts.h1[mt][nt][r];
                S.h2[w][rr][cc] = acts.h2[mt][nt][r];
            }
    S.dy[w][lane] = d;
    __syncwarp();
    // lane = sample: dz2 = d * w3 * relu'(z2); dz1 = (dz2 . W2) * relu'(z1)
    const float* W2 = params + MAC_OFF_W2;
    const float* w3 = params + MAC_OFF_W3;
    float dz2[32];
#pragma unroll
    for (int o = 0; o < 32; ++o) {
        dz2[o] = S.h2[w][lane][o] > 0.0f ? d * w3[o] : 0.0f;
        S.dz2[w][lane][o] = dz2[o];
    }
    for (int k = 0; k < 32; ++k) {
        float acc = 0.0f;
#pragma unroll
        for (int o = 0; o < 32; ++o) acc = fmaf(dz2[o], W2[o * 32 + k], acc);
        S.dz1[w][lane][k] = S.h1[w][lane][k] > 0.0f ? acc : 0.0f;
    }
    __syncwarp();
    // lane = output unit: weight gradients summed over the warp's samples
    const uint32_t o = lane;
    float g_w3 = 0.f, g_b2 = 0.f, g_b1 = 0.f, g_b3 = 0.f;
    float g_w2[32], g_w1[MAC_FEATURES];
#pragma unroll
    for (int k = 0; k < 32; ++k) g_w2[k] = 0.f;
#pragma unroll
    for (int k = 0; k < MAC_FEATURES; ++k) g_w1[k] = 0.f;
    const __nv_bfloat16* X = S.x + (size_t)w * 32 * 16;
    for (int s = 0; s < 32; ++s) {
        const float ds = S.dy[w][s];
        g_w3 = fmaf(ds, S.h2[w][s][o], g_w3);
        g_b3 += ds;
        const float z2 = S.dz2[w][s][o];
        g_b2 += z2;
#pragma unroll
        for (int k = 0; k < 32; ++k) g_w2[k] = fmaf(z2, S.h1[w][s][k], g_w2[k]);
        const float z1 = S.dz1[w][s][o];
        g_b1 += z1;
#pragma unroll
        for (int k = 0; k < MAC_FEATURES; ++k) g_w1[k] = fmaf(z1, __bfloat162float(X[s * 16 + k]), g_w1[k]);
    }
    // this warp's sums: every parameter once (lane o: the weights of unit o)
    float* gp = part + (size_t)(blockIdx.x * MAC_TRAIN_WARPS + w) * MAC_PART_STRIDE;
#pragma unroll
    for (int k = 0; k < MAC_FEATURES; ++k) gp[MAC_OFF_W1 + o * MAC_FEATURES + k] = g_w1[k];
    gp[MAC_OFF_B1 + o] = g_b1;
#pragma unroll
    for (int k = 0; k < 32; ++k) gp[MAC_OFF_W2 + o * 32 + k] = g_w2[k];
    gp[MAC_OFF_B2 + o] = g_b2;
    gp[MAC_OFF_W3 + o] = g_w3;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) l += __shfl_xor_sync(0xffffffffu, l, s);
    if (lane == 0) {
        gp[MAC_OFF_B3] = g_b3;
        gp[MAC_NPARAMS] = l;
    }
}

// The gradient of one step: the warps' sums added in warp order (the same
// bits in every run); the loss slot adds into the epoch's running loss.
__global__ void k_mac_reduce(const float* __restrict__ part, uint32_t warps, float* __restrict__ grad,
                             float* __restrict__ loss) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > MAC_NPARAMS) return;
    float sum = 0.0f;
    for (uint32_t w = 0; w < warps; ++w) sum += part[(size_t)w * MAC_PART_STRIDE + i];
    if (i < MAC_NPARAMS)
        grad[i] = sum;
    else
        loss[0] += sum;
}

__global__ void k_mac_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           float lr, float bc1, float bc2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MAC_NPARAMS) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
    g[i] = 0.0f;
}

// ---------------------------------------------------------------------------
// host

static int mac_fail(gbh_ctx* c, int code, const std::string& m) {
    c->last_error = m;
    return code;
}

#define MTRY(c, call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return mac_fail((c), GBH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static int mac_ensure(gbh_ctx* c) {
    if (c->mac) return GBH_OK;
    MacState* m = new MacState();
    c->mac = m;
    MTRY(c, cudaMalloc(&m->params, MAC_NPARAMS * 4));
    MTRY(c, cudaMalloc(&m->grad, MAC_NPARAMS * 4));
    MTRY(c, cudaMalloc(&m->adam_m, MAC_NPARAMS * 4));
    MTRY(c, cudaMalloc(&m->adam_v, MAC_NPARAMS * 4));
    MTRY(c, cudaMalloc(&m->frag, MAC_FRAG_WORDS * 32 * 4));
    MTRY(c, cudaMalloc(&m->loss, 16));
    MTRY(c, cudaMalloc(&m->count, 4));
    MTRY(c, cudaMalloc(&m->band, 8));
    MTRY(c, cudaMemcpyAsync(m->band, m->band_host, 8, cudaMemcpyHostToDevice, c->stream));
    MTRY(c, cudaMemsetAsync(m->grad, 0, MAC_NPARAMS * 4, c->stream));
    MTRY(c, cudaMemsetAsync(m->adam_m, 0, MAC_NPARAMS * 4, c->stream));
    MTRY(c, cudaMemsetAsync(m->adam_v, 0, MAC_NPARAMS * 4, c->stream));
    MTRY(c, cudaMemsetAsync(m->count, 0, 4, c->stream));
    return GBH_OK;
}

static void mac_free_pairs(MacState* m) {
    for (void* p : {(void*)m->feats, (void*)m->labels, (void*)m->pairs, (void*)m->skeys[0], (void*)m->skeys[1],
                    (void*)m->svals[0], (void*)m->svals[1], (void*)m->shist, (void*)m->sbase, (void*)m->slook,
                    (void*)m->sst, (void*)m->feats_tmp, (void*)m->pairs_tmp})
        cudaFree(p);
    m->feats = m->feats_tmp = nullptr;
    m->labels = nullptr;
    m->pairs = m->pairs_tmp = nullptr;
    m->skeys[0] = m->skeys[1] = nullptr;
    m->svals[0] = m->svals[1] = nullptr;
    m->shist = m->sbase = m->slook = nullptr;
    m->sst = nullptr;
    m->cap = 0;
}

// pair buffers for `cap` pairs, with the buffers of their canonical sort
static int mac_ensure_pairs(gbh_ctx* c, uint32_t cap) {
    MacState* m = c->mac;
    if (m->cap >= cap) return GBH_OK;
    mac_free_pairs(m);
    const uint32_t tiles = (cap + SORT_TILE - 1) / SORT_TILE;
    MTRY(c, cudaMalloc(&m->feats, (size_t)cap * MAC_FEATURES * 4));
    MTRY(c, cudaMalloc(&m->labels, (size_t)cap * 4));
    MTRY(c, cudaMalloc(&m->pairs, (size_t)cap * 8));
    MTRY(c, cudaMalloc(&m->feats_tmp, (size_t)cap * MAC_FEATURES * 4));
    MTRY(c, cudaMalloc(&m->pairs_tmp, (size_t)cap * 8));
    for (int k = 0; k < 2; ++k) {
        MTRY(c, cudaMalloc(&m->skeys[k], (size_t)cap * 8));
        MTRY(c, cudaMalloc(&m->svals[k], (size_t)cap * 4));
    }
    MTRY(c, cudaMalloc(&m->shist, SORT_PASSES * SORT_RADIX * 4));
    MTRY(c, cudaMalloc(&m->sbase, SORT_PASSES * SORT_RADIX * 4));
    MTRY(c, cudaMalloc(&m->slook, (size_t)SORT_PASSES * tiles * SORT_RADIX * 4));
    MTRY(c, cudaMalloc(&m->sst, sizeof(DevState)));
    m->stiles = tiles;
    m->cap = cap;
    return GBH_OK;
}

// Sort the n recorded pairs (and their features) by (group's first sorted
// slot, node): the step's onesweep radix sort on the 64-bit keys, then one
// gather.  Needs the groups of the recording walks in c->groups.
static int mac_sort_pairs(gbh_ctx* c, uint32_t n) {
    MacState* m = c->mac;
    if (n < 2) return GBH_OK;
    const uint32_t threads = 256, blocks = (n + threads - 1) / threads;
    k_mac_pair_keys<<<blocks, threads, 0, c->stream>>>(m->pairs, c->groups, n, m->skeys[0], m->svals[0]);
    MTRY(c, cudaGetLastError());
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    MTRY(c, cudaMemsetAsync(m->shist, 0, SORT_PASSES * SORT_RADIX * 4, c->stream));
    MTRY(c, cudaMemsetAsync(m->sst, 0, sizeof(DevState), c->stream));
    for (uint32_t p = 0; p < SORT_PASSES; ++p)
        MTRY(c, cudaMemsetAsync(m->slook + (size_t)p * m->stiles * SORT_RADIX, 0, (size_t)tiles * SORT_RADIX * 4,
                                c->stream));
    launch_sort_hist(m->skeys[0], n, m->shist, m->sst, c->num_sms, c->stream);
    StepBuffers sb;
    memset(&sb, 0, sizeof(sb));
    sb.keys_in = m->skeys[0];
    sb.idx_in = m->svals[0];
    sb.keys_out = m->skeys[1];
    sb.idx_out = m->svals[1];
    sb.st = m->sst;
    sb.hist = m->shist;
    sb.bucket_base = m->sbase;
    sb.lookback = m->slook;
    sb.N = n;
    sb.sort_tiles_cap = m->stiles;
    sb.num_sms = c->num_sms;
    launch_sort(sb, c->stream);  // eight passes: the result is back in skeys[0], svals[0]
    k_mac_gather_pairs<<<blocks, threads, 0, c->stream>>>(m->svals[0], n, m->feats, m->pairs, m->feats_tmp,
                                                           m->pairs_tmp);
    MTRY(c, cudaGetLastError());
    uint32_t err = 0;
    MTRY(c, cudaMemcpyAsync(&err, &m->sst->error_word, 4, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    if (err) return mac_fail(c, GBH_ERR_DEVICE, "sorting the training pairs: device error word set");
    std::swap(m->feats, m->feats_tmp);
    std::swap(m->pairs, m->pairs_tmp);
    return GBH_OK;
}

void mac_release(gbh_ctx* c) {
    MacState* m = c->mac;
    if (!m) return;
    cudaFree(m->params);
    cudaFree(m->grad);
    cudaFree(m->adam_m);
    cudaFree(m->adam_v);
    cudaFree(m->frag);
    cudaFree(m->loss);
    cudaFree(m->count);
    cudaFree(m->band);
    cudaFree(m->part);
    mac_free_pairs(m);
    delete m;
    c->mac = nullptr;
}

static MacDeviceWeights mac_weights(const gbh_ctx* c) {
    MacDeviceWeights mw;
    memset(&mw, 0, sizeof(mw));
    mw.frag = c->mac ? c->mac->frag : nullptr;
    mw.band = c->mac ? c->mac->band : nullptr;
    return mw;
}

int enqueue_walk_learned(gbh_ctx* c) {
    const bool learned = c->mac_mode == GBH_MAC_LEARNED;
    if (learned && (!c->mac || !c->mac_ready)) return mac_fail(c, GBH_ERR_STATE, "learned MAC without weights");
    if (!c->paths_current) {  // the tree was built for the plain walk
        launch_group_paths(ctx_buffers(c), c->stream);
        c->paths_current = true;
    }
    launch_walk_group(ctx_buffers(c), mac_weights(c), learned, c->stream);
    return GBH_OK;
}

static int upload_step_params(gbh_ctx* c, const gbh_step_params& p) {
    MTRY(c, cudaMemcpyAsync(c->params_dev, &p, sizeof(p), cudaMemcpyHostToDevice, c->stream));
    c->params_host = p;
    c->params_valid = true;
    c->mac_mode = p.mac_mode;
    return GBH_OK;
}

extern "C" {

int gbh_mac_set_weights(gbh_ctx* c, const float* params, uint32_t count) {
    if (!c || !params || count != MAC_NPARAMS) return c ? mac_fail(c, GBH_ERR_INVALID, "expected GBH_MAC_NUM_PARAMS floats") : GBH_ERR_INVALID;
    MTRY(c, cudaSetDevice(c->device));
    int rc = mac_ensure(c);
    if (rc) return rc;
    MTRY(c, cudaMemcpyAsync(c->mac->params, params, MAC_NPARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    k_mac_build_frag<<<1, 32, 0, c->stream>>>(c->mac->params, c->mac->frag);
    MTRY(c, cudaGetLastError());
    MTRY(c, cudaStreamSynchronize(c->stream));
    c->mac_ready = true;
    return GBH_OK;
}

int gbh_mac_set_band(gbh_ctx* c, float theta_accept, float theta_open) {
    if (!c) return GBH_ERR_INVALID;
    if (!(theta_accept > 0.0f) || !(theta_open >= theta_accept) || !(theta_open < 1e30f))
        return mac_fail(c, GBH_ERR_INVALID, "band needs 0 < theta_accept <= theta_open");
    MTRY(c, cudaSetDevice(c->device));
    int rc = mac_ensure(c);
    if (rc) return rc;
    c->mac->band_host[0] = theta_accept;
    c->mac->band_host[1] = theta_open;
    MTRY(c, cudaMemcpyAsync(c->mac->band, c->mac->band_host, 8, cudaMemcpyHostToDevice, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_mac_get_band(gbh_ctx* c, float* theta_accept, float* theta_open) {
    if (!c || !theta_accept || !theta_open) return GBH_ERR_INVALID;
    *theta_accept = c->mac ? c->mac->band_host[0] : MAC_BAND_LO;
    *theta_open = c->mac ? c->mac->band_host[1] : MAC_BAND_HI;
    return GBH_OK;
}

int gbh_mac_get_weights(gbh_ctx* c, float* params, uint32_t count) {
    if (!c || !params || count != MAC_NPARAMS) return GBH_ERR_INVALID;
    if (!c->mac) return mac_fail(c, GBH_ERR_STATE, "no weights");
    MTRY(c, cudaSetDevice(c->device));
    MTRY(c, cudaMemcpyAsync(params, c->mac->params, MAC_NPARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_mac_predict(gbh_ctx* c, const float* features, uint32_t count, float* out) {
    if (!c || (!features && count) || (!out && count)) return GBH_ERR_INVALID;
    if (!c->mac_ready) return mac_fail(c, GBH_ERR_STATE, "no weights");
    if (count == 0) return GBH_OK;
    MTRY(c, cudaSetDevice(c->device));
    float *df = nullptr, *dout = nullptr;
    MTRY(c, cudaMalloc(&df, (size_t)count * MAC_FEATURES * 4));
    MTRY(c, cudaMalloc(&dout, (size_t)count * 4));
    cudaError_t e = cudaMemcpyAsync(df, features, (size_t)count * MAC_FEATURES * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        const uint32_t rows = MAC_TRAIN_WARPS * 32;
        k_mac_predict<<<(count + rows - 1) / rows, rows, 0, c->stream>>>(df, count, dout, mac_weights(c));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)count * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(df);
    cudaFree(dout);
    if (e != cudaSuccess) return mac_fail(c, GBH_ERR_CUDA, std::string("mac predict: ") + cudaGetErrorString(e));
    return GBH_OK;
}

int gbh_mac_generate(gbh_ctx* c, const gbh_step_params* params, uint32_t max_pairs, uint64_t seed, uint32_t* out_count) {
    if (!c || !params || !out_count || max_pairs == 0) return GBH_ERR_INVALID;
    if (!c->inited) return mac_fail(c, GBH_ERR_STATE, "generate before init");
    if (params->merging_collision_or_neither != GBH_MODE_NEITHER)
        return mac_fail(c, GBH_ERR_UNSUPPORTED, "training pairs are generated for gravity only");
    MTRY(c, cudaSetDevice(c->device));
    int rc = mac_ensure(c);
    if (rc) return rc;
    rc = mac_ensure_pairs(c, max_pairs);
    if (rc) return rc;
    MacState* m = c->mac;
    // 1. tree of the current state and the plain theta = 0.2 walk (accelerations)
    gbh_step_params p = *params;
    p.mac_mode = GBH_MAC_PLAIN;
    p.precision_mode = GBH_PRECISION_FP32;
    p.theta = 0.2f;
    p.flags |= GBH_FLAG_STORE_ACCEL;
    rc = upload_step_params(c, p);
    if (rc) return rc;
    const int bin0 = c->bin;
    if ((rc = enqueue_reset(c)) || (rc = enqueue_prepare(c)) || (rc = enqueue_sort(c)) || (rc = enqueue_build(c)) ||
        (rc = enqueue_fill(c)))
        return rc;
    launch_walk_plain(ctx_buffers(c), c->stream);
    MTRY(c, cudaGetLastError());
    // 2. record candidate pairs from a conservative and an aggressive group
    //    walk (half of the budget each), so that the pairs cover what both
    //    strict and loose criteria meet.  A walk meets far more band
    //    candidates than the budget holds: a count pass first, then a hashed
    //    subset of (group, node) sized to about 95% of the budget, so the
    //    pairs come from every group rather than from the first ones to run.
    const float thetas[2] = {0.25f, 0.6f};  // the groups come from the build above
    uint32_t start = 0;
    for (int r = 0; r < 2; ++r) {
        p.mac_mode = GBH_MAC_GROUP;
        p.theta = thetas[r];
        p.flags &= ~GBH_FLAG_STORE_ACCEL;
        rc = upload_step_params(c, p);
        if (rc) return rc;
        MacDeviceWeights mw = mac_weights(c);
        mw.rec_count = m->count;
        mw.rec_pairs = m->pairs;
        mw.rec_feats = m->feats;
        mw.rec_max_bodies = 0xFFFFFFFFu;
        mw.rec_seed = (uint32_t)(seed ^ (seed >> 32)) + 0x51ED27u * r;
        const uint32_t cap = r == 0 ? max_pairs / 2 : max_pairs;
        const uint32_t budget = cap - start;
        // count pass over a 1/16 hashed subset (nothing stored; the 32-bit
        // counter stays far from wrapping); the group walk writes the output
        // bodies, which are discarded (no swap)
        uint32_t met = 0;
        MTRY(c, cudaMemsetAsync(m->count, 0, 4, c->stream));
        mw.rec_cap = 0;
        mw.rec_keep = 0x0FFFFFFFu;
        launch_walk_group_record(ctx_buffers(c), mw, c->stream);
        MTRY(c, cudaGetLastError());
        MTRY(c, cudaMemcpyAsync(&met, m->count, 4, cudaMemcpyDeviceToHost, c->stream));
        MTRY(c, cudaStreamSynchronize(c->stream));
        double frac = met ? 0.95 * (double)budget / (16.0 * (double)met) : 1.0;
        // record pass, appending after the pairs kept so far; a pass that
        // meets more kept pairs than the budget holds (the ones stored would
        // then depend on the order the warps ran in) runs again with a
        // smaller fraction
        uint32_t end = 0;
        for (int attempt = 0;; ++attempt) {
            mw.rec_keep = frac >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(frac * 4294967296.0);
            MTRY(c, cudaMemcpyAsync(m->count, &start, 4, cudaMemcpyHostToDevice, c->stream));
            mw.rec_cap = cap;
            launch_walk_group_record(ctx_buffers(c), mw, c->stream);
            MTRY(c, cudaGetLastError());
            MTRY(c, cudaMemcpyAsync(&end, m->count, 4, cudaMemcpyDeviceToHost, c->stream));
            MTRY(c, cudaStreamSynchronize(c->stream));
            if (end <= cap || attempt == 8) break;
            frac *= 0.95 * (double)budget / (double)(end - start);
        }
        start = end < cap ? end : cap;
        MTRY(c, cudaMemcpyAsync(m->count, &start, 4, cudaMemcpyHostToDevice, c->stream));
    }
    uint32_t recorded = 0;
    MTRY(c, cudaMemcpyAsync(&recorded, m->count, 4, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    recorded = recorded < max_pairs ? recorded : max_pairs;
    MTRY(c, cudaMemcpyAsync(m->count, &recorded, 4, cudaMemcpyHostToDevice, c->stream));
    // canonical order of the pairs (and so of every minibatch)
    if ((rc = mac_sort_pairs(c, recorded))) return rc;
    // 3. labels
    if (recorded) {
        const uint32_t threads = 256;
        k_mac_label<<<(recorded * 32 + threads - 1) / threads, threads, 0, c->stream>>>(ctx_buffers(c), m->pairs,
                                                                                        m->count, m->labels);
        MTRY(c, cudaGetLastError());
    }
    MTRY(c, cudaStreamSynchronize(c->stream));
    c->bin = bin0;
    m->num_pairs = recorded;
    *out_count = recorded;
    // the walks above wrote the in-order position copy for a state that did
    // not advance: the next compaction gathers
    MTRY(c, cudaMemsetAsync(&c->st->sorted_valid, 0, 4, c->stream));
    // leave the caller's step parameters in force again
    return upload_step_params(c, *params);
}

int gbh_mac_read_pairs(gbh_ctx* c, float* features, float* labels, uint32_t count, uint32_t offset) {
    if (!c || !c->mac) return GBH_ERR_INVALID;
    if ((uint64_t)offset + count > c->mac->num_pairs) return mac_fail(c, GBH_ERR_INVALID, "pair range");
    MTRY(c, cudaSetDevice(c->device));
    if (features)
        MTRY(c, cudaMemcpyAsync(features, c->mac->feats + (size_t)offset * MAC_FEATURES, (size_t)count * MAC_FEATURES * 4,
                                cudaMemcpyDeviceToHost, c->stream));
    if (labels)
        MTRY(c, cudaMemcpyAsync(labels, c->mac->labels + offset, (size_t)count * 4, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_mac_read_pair_ids(gbh_ctx* c, uint32_t* out, uint32_t count, uint32_t offset) {
    if (!c || !c->mac || (!out && count)) return GBH_ERR_INVALID;
    if ((uint64_t)offset + count > c->mac->num_pairs) return mac_fail(c, GBH_ERR_INVALID, "pair range");
    MTRY(c, cudaSetDevice(c->device));
    std::vector<uint2> pairs(count);
    uint32_t ng = 0;
    MTRY(c, cudaMemcpyAsync(pairs.data(), c->mac->pairs + offset, (size_t)count * 8, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaMemcpyAsync(&ng, &c->st->num_groups, 4, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    std::vector<uint2> groups(ng);
    if (ng) MTRY(c, cudaMemcpyAsync(groups.data(), c->groups, (size_t)ng * 8, cudaMemcpyDeviceToHost, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    for (uint32_t k = 0; k < count; ++k) {
        const uint2 g = pairs[k].x < ng ? groups[pairs[k].x] : make_uint2(0u, 0u);
        out[3 * k] = g.x;
        out[3 * k + 1] = g.y;
        out[3 * k + 2] = pairs[k].y;
    }
    return GBH_OK;
}

int gbh_mac_write_pairs(gbh_ctx* c, const float* features, const float* labels, uint32_t count) {
    if (!c || !features || !labels) return GBH_ERR_INVALID;
    MTRY(c, cudaSetDevice(c->device));
    int rc = mac_ensure(c);
    if (rc) return rc;
    rc = mac_ensure_pairs(c, count > 0 ? count : 1);
    if (rc) return rc;
    MTRY(c, cudaMemcpyAsync(c->mac->feats, features, (size_t)count * MAC_FEATURES * 4, cudaMemcpyHostToDevice, c->stream));
    MTRY(c, cudaMemcpyAsync(c->mac->labels, labels, (size_t)count * 4, cudaMemcpyHostToDevice, c->stream));
    MTRY(c, cudaStreamSynchronize(c->stream));
    c->mac->num_pairs = count;
    return GBH_OK;
}

static void init_params_host(std::vector<float>& p, uint64_t seed) {
    // He-uniform initialisation from a splitmix64 stream
    uint64_t s = seed + 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) / (double)(1ull << 53) * 2.0 - 1.0;
    };
    p.assign(MAC_NPARAMS, 0.0f);
    const double a1 = std::sqrt(6.0 / MAC_FEATURES), a2 = std::sqrt(6.0 / 32.0);
    for (int i = 0; i < 32 * MAC_FEATURES; ++i) p[MAC_OFF_W1 + i] = (float)(a1 * uni());
    for (int i = 0; i < 32 * 32; ++i) p[MAC_OFF_W2 + i] = (float)(a2 * uni());
    for (int i = 0; i < 32; ++i) p[MAC_OFF_W3 + i] = (float)(a2 * 0.5 * uni());
    p[MAC_OFF_B3] = -3.0f;
}

static size_t train_smem() { return sizeof(TrainSmem); }

int gbh_mac_train(gbh_ctx* c, uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* losses) {
    if (!c || batch == 0) return GBH_ERR_INVALID;
    if (!c->mac || c->mac->num_pairs == 0) return mac_fail(c, GBH_ERR_STATE, "no training pairs");
    MTRY(c, cudaSetDevice(c->device));
    MacState* m = c->mac;
    if (!c->mac_ready) {
        std::vector<float> p;
        init_params_host(p, seed);
        int rc = gbh_mac_set_weights(c, p.data(), MAC_NPARAMS);
        if (rc) return rc;
        MTRY(c, cudaMemsetAsync(m->adam_m, 0, MAC_NPARAMS * 4, c->stream));
        MTRY(c, cudaMemsetAsync(m->adam_v, 0, MAC_NPARAMS * 4, c->stream));
        m->adam_t = 0;
    }
    MTRY(c, cudaFuncSetAttribute(k_mac_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    const uint32_t rows = MAC_TRAIN_WARPS * 32;
    const uint32_t steps = (m->num_pairs + batch - 1) / batch;
    const uint32_t tblocks = (batch + rows - 1) / rows, warps = tblocks * MAC_TRAIN_WARPS;
    if (m->part_warps < warps) {
        cudaFree(m->part);
        m->part = nullptr;
        m->part_warps = 0;
        MTRY(c, cudaMalloc(&m->part, (size_t)warps * MAC_PART_STRIDE * 4));
        m->part_warps = warps;
    }
    for (uint32_t ep = 0; ep < epochs; ++ep) {
        MTRY(c, cudaMemsetAsync(m->loss, 0, 16, c->stream));
        for (uint32_t s = 0; s < steps; ++s) {
            const uint32_t st = ep * steps + s;
            k_mac_train_step<<<tblocks, rows, train_smem(), c->stream>>>(
                m->feats, m->labels, m->num_pairs, batch, 1, (uint32_t)seed, st, mac_weights(c), m->params, m->part);
            k_mac_reduce<<<(MAC_PART_STRIDE + 255) / 256, 256, 0, c->stream>>>(m->part, warps, m->grad, m->loss);
            ++m->adam_t;
            const float bc1 = 1.0f - std::pow(0.9f, (float)m->adam_t);
            const float bc2 = 1.0f - std::pow(0.999f, (float)m->adam_t);
            k_mac_adam<<<(MAC_NPARAMS + 255) / 256, 256, 0, c->stream>>>(m->params, m->grad, m->adam_m, m->adam_v, lr,
                                                                        bc1, bc2);
            k_mac_build_frag<<<1, 32, 0, c->stream>>>(m->params, m->frag);
        }
        MTRY(c, cudaGetLastError());
        if (losses) {
            float l = 0.0f;
            MTRY(c, cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, c->stream));
            MTRY(c, cudaStreamSynchronize(c->stream));
            losses[ep] = l / ((float)steps * (float)batch);
        }
    }
    MTRY(c, cudaStreamSynchronize(c->stream));
    return GBH_OK;
}

int gbh_mac_loss_grad(gbh_ctx* c, const float* features, const float* labels, uint32_t count, float* loss,
                      float* grad) {
    if (!c || !features || !labels || !loss || !grad || count == 0) return GBH_ERR_INVALID;
    if (!c->mac_ready) return mac_fail(c, GBH_ERR_STATE, "no weights");
    MTRY(c, cudaSetDevice(c->device));
    MacState* m = c->mac;
    float *df = nullptr, *dl = nullptr, *dp = nullptr;
    const uint32_t rows = MAC_TRAIN_WARPS * 32, tblocks = (count + rows - 1) / rows;
    const uint32_t warps = tblocks * MAC_TRAIN_WARPS;
    MTRY(c, cudaMalloc(&df, (size_t)count * MAC_FEATURES * 4));
    MTRY(c, cudaMalloc(&dl, (size_t)count * 4));
    MTRY(c, cudaMalloc(&dp, (size_t)warps * MAC_PART_STRIDE * 4));
    cudaError_t e = cudaMemcpyAsync(df, features, (size_t)count * MAC_FEATURES * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dl, labels, (size_t)count * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, MAC_NPARAMS * 4, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, 16, c->stream);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mac_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
    if (e == cudaSuccess) {
        k_mac_train_step<<<tblocks, rows, train_smem(), c->stream>>>(df, dl, count, count, 0, 0, 0, mac_weights(c),
                                                                      m->params, dp);
        k_mac_reduce<<<(MAC_PART_STRIDE + 255) / 256, 256, 0, c->stream>>>(dp, warps, m->grad, m->loss);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, m->grad, MAC_NPARAMS * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(loss, m->loss, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, MAC_NPARAMS * 4, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(df);
    cudaFree(dl);
    cudaFree(dp);
    if (e != cudaSuccess) return mac_fail(c, GBH_ERR_CUDA, std::string("mac loss_grad: ") + cudaGetErrorString(e));
    *loss = *loss / (float)count;
    return GBH_OK;
}

}  // extern "C"
