// mac_mlp.cuh — the learned multipole-acceptance criterion: features of a
// (32-body group, node) pair and the 12-32-32-1 MLP evaluated per warp on the
// tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation).
//
// The MLP predicts log10 of the relative error of replacing the node by its
// monopole, maximised over the bodies of the group: max_i |a_mono,i - a_exact,i|
// / |a_i|, with a_exact the exact sum over the node's subtree and a_i the
// body's total acceleration.  The walk accepts a node when the prediction is
// below gbh_step_params.mac_tolerance.
//
// Per-warp batch: the 32 lanes each hold one candidate; features are staged as
// a 32x16 BF16 tile in shared memory (12 features + 4 zero columns).  Layer 1
// is 2 (rows) x 4 (cols) mma, layer 2 2 x 4 x 2, layer 3 2 x 2 (one useful
// output column): 28 mma per 32 candidates.  The FP32 accumulator fragments
// of one layer are, repacked to BF16 pairs, exactly the A fragments of the
// next layer, so activations never leave registers.  Weights live in shared
// memory, pre-arranged per lane in fragment order (conflict-free loads).
#pragma once

#include <cuda_bf16.h>

#include "gbh_common.cuh"

#define MAC_FEATURES GBH_MAC_FEATURES
#define MAC_HIDDEN GBH_MAC_HIDDEN
#define MAC_NPARAMS GBH_MAC_NUM_PARAMS
// parameter vector layout (float32): W1[32][12], b1[32], W2[32][32], b2[32], w3[32], b3
#define MAC_OFF_W1 0
#define MAC_OFF_B1 (MAC_OFF_W1 + 32 * 12)
#define MAC_OFF_W2 (MAC_OFF_B1 + 32)
#define MAC_OFF_B2 (MAC_OFF_W2 + 32 * 32)
#define MAC_OFF_W3 (MAC_OFF_B2 + 32)
#define MAC_OFF_B3 (MAC_OFF_W3 + 32)
// fragment table: words per lane
#define MAC_FRAG_W1 8    // 4 n-tiles x 2 regs
#define MAC_FRAG_W2 16   // 4 n-tiles x 2 k-steps x 2 regs
#define MAC_FRAG_W3 4    // 2 k-steps x 2 regs
#define MAC_FRAG_B1 8    // 4 n-tiles x 2 columns
#define MAC_FRAG_B2 8
#define MAC_FRAG_WORDS (MAC_FRAG_W1 + MAC_FRAG_W2 + MAC_FRAG_W3 + MAC_FRAG_B1 + MAC_FRAG_B2 + 1)
#define MAC_WALK_WARPS 8
// the learned walk: below MAC_BAND_LO (group rule) accept, above MAC_BAND_HI open
#define MAC_BAND_LO 0.25f
#define MAC_BAND_HI 1.0f

struct MacDeviceWeights {
    const uint32_t* frag;  // [MAC_FRAG_WORDS][32]: per-lane fragment words (global)
    uint32_t* smem_frag;   // block copy in shared memory (set by the kernel)
    __nv_bfloat16* smem_x; // [warps][x_rows][16] feature tiles (set by the kernel)
    uint32_t x_rows;       // feature rows per warp (32, or more for a queue)
    // recording of training pairs (gbh_mac_generate); rec_count == nullptr: off
    uint32_t* rec_count;
    uint2* rec_pairs;      // (group = first sorted slot / 32, node id)
    float* rec_feats;      // [cap][MAC_FEATURES]
    uint32_t rec_cap;
    uint32_t rec_max_bodies;  // only nodes with at most this many bodies
    uint32_t rec_keep;        // keep a pair when hash % 1024 < rec_keep
    uint32_t rec_seed;
};

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

struct GroupGeom {
    float cx, cy, cz;  // centre of the group's bounding box
    float R;           // half diagonal of the group's bounding box
    float a_ref;       // smallest |acceleration| of the group's bodies in the previous step
    float3 bmin, bmax; // the group's bounding box
};

struct NodeGeom {
    float4 cm;
    float3 bmin, bmax;
    uint32_t count;
};

// Distance between the group's box and the node's box (0 when they overlap).
__device__ __forceinline__ float box_gap(const GroupGeom& g, const NodeGeom& n) {
    const float gx = fmaxf(0.0f, fmaxf(n.bmin.x - g.bmax.x, g.bmin.x - n.bmax.x));
    const float gy = fmaxf(0.0f, fmaxf(n.bmin.y - g.bmax.y, g.bmin.y - n.bmax.y));
    const float gz = fmaxf(0.0f, fmaxf(n.bmin.z - g.bmax.z, g.bmin.z - n.bmax.z));
    return sqrtf(gx * gx + gy * gy + gz * gz);
}

// Group theta rule (the learned criterion's ablation): accept when the boxes
// of the group and the node are disjoint and the node's half side is below
// theta times the distance from its centre of mass to the group's bounding
// sphere.
__device__ __forceinline__ bool group_theta_accept(const GroupGeom& g, const NodeGeom& n, float theta) {
    const float ex = n.bmax.x - n.bmin.x, ey = n.bmax.y - n.bmin.y, ez = n.bmax.z - n.bmin.z;
    const float half = 0.5f * fmaxf(ex, fmaxf(ey, ez));
    const float dx = n.cm.x - g.cx, dy = n.cm.y - g.cy, dz = n.cm.z - g.cz;
    const float d = sqrtf(dx * dx + dy * dy + dz * dz) - g.R;
    return d > 0.0f && half < theta * d && box_gap(g, n) > 0.0f;
}

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// The 12 features, all scale free.  h: half of the longest side; d: distance
// from the node's centre of mass to the group centre; R: group half diagonal.
__device__ __forceinline__ void mac_features(const GroupGeom& g, const NodeGeom& n, float G, float soft,
                                             float f[MAC_FEATURES]) {
    const float tiny = 1e-30f;
    const float ex = n.bmax.x - n.bmin.x, ey = n.bmax.y - n.bmin.y, ez = n.bmax.z - n.bmin.z;
    const float emax = fmaxf(ex, fmaxf(ey, ez));
    const float emin = fminf(ex, fminf(ey, ez));
    const float emid = ex + ey + ez - emax - emin;
    const float h = fmaxf(0.5f * emax, tiny);
    const float dx = n.cm.x - g.cx, dy = n.cm.y - g.cy, dz = n.cm.z - g.cz;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float d = fmaxf(sqrtf(d2), tiny);
    const float R = fmaxf(g.R, 1e-6f * d);
    const float q = clampf((d - R) / d, 1e-4f, 1.0f);
    const float ox = n.cm.x - 0.5f * (n.bmin.x + n.bmax.x);
    const float oy = n.cm.y - 0.5f * (n.bmin.y + n.bmax.y);
    const float oz = n.cm.z - 0.5f * (n.bmin.z + n.bmax.z);
    const float off = sqrtf(ox * ox + oy * oy + oz * oz);
    const float force = G * n.cm.w / (d2 + soft);
    f[0] = clampf(__log2f(h / d), -24.f, 8.f) * 0.125f;
    f[1] = clampf(__log2f(R / d), -24.f, 8.f) * 0.125f;
    f[2] = __log2f(q) * 0.125f;
    f[3] = clampf(off / h, 0.f, 2.f);
    f[4] = emax > 0.f ? emin / emax : 1.f;
    f[5] = emax > 0.f ? emid / emax : 1.f;
    f[6] = __log2f((float)min(n.count, 1u << 16)) * (1.0f / 16.0f);
    f[7] = off > tiny ? (ox * dx + oy * dy + oz * dz) / (off * d) : 0.f;
    f[8] = (g.a_ref > 0.f ? clampf(__log2f(force / g.a_ref), -32.f, 32.f) : 32.f) * (1.0f / 16.0f);
    f[9] = clampf(__log2f(soft / d2 + 1e-30f), -48.f, 8.f) * (1.0f / 16.0f);
    f[10] = clampf(__log2f(h / R), -16.f, 16.f) * 0.125f;
    f[11] = clampf(__log2f(box_gap(g, n) / h + 1e-6f), -20.f, 8.f) * 0.125f;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Stage this lane's features as row `lane` of the warp's BF16 tile.
__device__ __forceinline__ void mac_stage_features(const MacDeviceWeights& mw, uint32_t warp, uint32_t lane,
                                                   const float f[MAC_FEATURES]) {
    uint32_t* row = reinterpret_cast<uint32_t*>(mw.smem_x + ((size_t)warp * mw.x_rows + lane) * 16);
#pragma unroll
    for (int k = 0; k < 6; ++k) row[k] = pack_bf16x2(f[2 * k], f[2 * k + 1]);
    row[6] = 0u;
    row[7] = 0u;
}

// Activations of the two hidden layers, in accumulator-fragment order
// (layer x m-tile x n-tile x 4), for the backward pass of training.
struct MacActs {
    float h1[2][4][4];
    float h2[2][4][4];
};

// Forward pass of the warp's 32 staged rows; returns row `lane`'s output.
template <bool KEEP>
__device__ __forceinline__ float mac_forward_warp(const MacDeviceWeights& mw, uint32_t warp, uint32_t lane,
                                                  MacActs* acts) {
    __syncwarp();
    const uint32_t gid = lane >> 2, tig = lane & 3;
    const uint32_t* F = mw.smem_frag;
    const uint32_t* X = reinterpret_cast<const uint32_t*>(mw.smem_x + (size_t)warp * mw.x_rows * 16);
    uint32_t a2[2][2][4];  // layer-2 A fragments [m-tile][k-step]
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        uint32_t a[4];
        a[0] = X[(16 * mt + gid) * 8 + tig];
        a[1] = X[(16 * mt + gid + 8) * 8 + tig];
        a[2] = X[(16 * mt + gid) * 8 + tig + 4];
        a[3] = X[(16 * mt + gid + 8) * 8 + tig + 4];
        float c[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const float b0 = __uint_as_float(F[(MAC_FRAG_W1 + MAC_FRAG_W2 + MAC_FRAG_W3 + 2 * nt) * 32 + lane]);
            const float b1 = __uint_as_float(F[(MAC_FRAG_W1 + MAC_FRAG_W2 + MAC_FRAG_W3 + 2 * nt + 1) * 32 + lane]);
            c[nt][0] = b0;
            c[nt][1] = b1;
            c[nt][2] = b0;
            c[nt][3] = b1;
            mma_bf16(c[nt], a, F[(2 * nt) * 32 + lane], F[(2 * nt + 1) * 32 + lane]);
#pragma unroll
            for (int r = 0; r < 4; ++r) c[nt][r] = fmaxf(c[nt][r], 0.0f);
            if (KEEP)
#pragma unroll
                for (int r = 0; r < 4; ++r) acts->h1[mt][nt][r] = c[nt][r];
        }
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            a2[mt][ks][0] = pack_bf16x2(c[2 * ks][0], c[2 * ks][1]);
            a2[mt][ks][1] = pack_bf16x2(c[2 * ks][2], c[2 * ks][3]);
            a2[mt][ks][2] = pack_bf16x2(c[2 * ks + 1][0], c[2 * ks + 1][1]);
            a2[mt][ks][3] = pack_bf16x2(c[2 * ks + 1][2], c[2 * ks + 1][3]);
        }
    }
    float out[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        float c[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            const int bo = MAC_FRAG_W1 + MAC_FRAG_W2 + MAC_FRAG_W3 + MAC_FRAG_B1;
            const float b0 = __uint_as_float(F[(bo + 2 * nt) * 32 + lane]);
            const float b1 = __uint_as_float(F[(bo + 2 * nt + 1) * 32 + lane]);
            c[nt][0] = b0;
            c[nt][1] = b1;
            c[nt][2] = b0;
            c[nt][3] = b1;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks)
                mma_bf16(c[nt], a2[mt][ks], F[(MAC_FRAG_W1 + (nt * 2 + ks) * 2) * 32 + lane],
                         F[(MAC_FRAG_W1 + (nt * 2 + ks) * 2 + 1) * 32 + lane]);
#pragma unroll
            for (int r = 0; r < 4; ++r) c[nt][r] = fmaxf(c[nt][r], 0.0f);
            if (KEEP)
#pragma unroll
                for (int r = 0; r < 4; ++r) acts->h2[mt][nt][r] = c[nt][r];
        }
        uint32_t a3[2][4];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            a3[ks][0] = pack_bf16x2(c[2 * ks][0], c[2 * ks][1]);
            a3[ks][1] = pack_bf16x2(c[2 * ks][2], c[2 * ks][3]);
            a3[ks][2] = pack_bf16x2(c[2 * ks + 1][0], c[2 * ks + 1][1]);
            a3[ks][3] = pack_bf16x2(c[2 * ks + 1][2], c[2 * ks + 1][3]);
        }
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
            mma_bf16(o, a3[ks], F[(MAC_FRAG_W1 + MAC_FRAG_W2 + 2 * ks) * 32 + lane],
                     F[(MAC_FRAG_W1 + MAC_FRAG_W2 + 2 * ks + 1) * 32 + lane]);
        out[mt][0] = o[0];  // row 16 mt + gid, column 0 (valid in lanes with tig == 0)
        out[mt][1] = o[2];  // row 16 mt + gid + 8
    }
    // row `lane` lives in lane 4 * (lane & 7), in (m-tile lane >> 4, half (lane >> 3) & 1)
    const uint32_t src = 4 * (lane & 7);
    const float v00 = __shfl_sync(0xffffffffu, out[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, out[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, out[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, out[1][1], src);
    const uint32_t sel = lane >> 3;
    const float v = sel == 0 ? v00 : sel == 1 ? v01 : sel == 2 ? v10 : v11;
    const float b3 = __uint_as_float(F[(MAC_FRAG_WORDS - 1) * 32 + lane]);
    return v + b3;
}

__device__ __forceinline__ float mac_infer_warp(const MacDeviceWeights& mw, uint32_t warp, uint32_t lane) {
    return mac_forward_warp<false>(mw, warp, lane, nullptr);
}

// Copy the fragment table into the block's shared memory (all threads).
__device__ __forceinline__ void mac_load_frag(MacDeviceWeights& mw, uint32_t* smem_frag, __nv_bfloat16* smem_x,
                                              uint32_t x_rows = 32) {
    for (uint32_t i = threadIdx.x; i < MAC_FRAG_WORDS * 32; i += blockDim.x) smem_frag[i] = mw.frag[i];
    mw.smem_frag = smem_frag;
    mw.smem_x = smem_x;
    mw.x_rows = x_rows;
    __syncthreads();
}

// smallest |a| of the group's bodies in the previous step (feature 8)
__device__ __forceinline__ float group_accel_ref(const StepBuffers& b, bool active, uint32_t bi) {
    float a = (active && b.accel_mag) ? b.accel_mag[bi] : 3.0e38f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
    return a < 3.0e38f ? a : 0.0f;
}
