// mac_mlp.cuh — the learned multipole-acceptance criterion: features of a
// (body group, node) pair and the 12-32-32-1 MLP evaluated per warp on the
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
// In shared memory the table is stored in 16-byte chunks of four consecutive
// words per lane, [chunk][lane][4], so that a lane reads four words with one
// 128-bit load (the blocks above all start on multiples of four words):
//   chunk 0-1 W1 (n-tiles 0,1 | 2,3)   chunk 7-8  b1 (n-tiles 0,1 | 2,3)
//   chunk 2-5 W2 (n-tile 0..3)          chunk 9-10 b2 (n-tiles 0,1 | 2,3)
//   chunk 6   w3                        chunk 11   b3 (word 0)
#define MAC_FRAG_CHUNKS 12
#define MAC_SMEM_FRAG_WORDS (MAC_FRAG_CHUNKS * 4 * 32)
#define MAC_WALK_WARPS 8
// the learned walk's default band: nodes that pass the group rule at
// MAC_BAND_LO are accepted, nodes that fail it at MAC_BAND_HI opened
#define MAC_BAND_LO 0.25f
#define MAC_BAND_HI 4.0f

struct MacDeviceWeights {
    const uint32_t* frag;  // [MAC_FRAG_WORDS][32]: per-lane fragment words (global)
    const float* band;     // [2]: group-rule theta below which nodes are accepted, above which opened
    uint32_t* smem_frag;   // block copy in shared memory, chunked (set by the kernel)
    __nv_bfloat16* smem_x; // [warps][x_rows][16] feature tiles (set by the kernel)
    uint32_t x_rows;       // feature rows per warp (32, or more for a queue)
    // recording of training pairs (gbh_mac_generate); rec_count == nullptr: off
    uint32_t* rec_count;
    uint2* rec_pairs;      // (group = first sorted slot / 32, node id)
    float* rec_feats;      // [cap][MAC_FEATURES]
    uint32_t rec_cap;
    uint32_t rec_max_bodies;  // only nodes with at most this many bodies
    uint32_t rec_keep;        // keep a pair when its 32-bit hash <= rec_keep (0xFFFFFFFF: all)
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
    // per-group terms of the features (set by group_feature_terms)
    float soft;        // softening (length squared)
    float l_R;         // log2 R
    float l_soft;      // log2 softening
    float l_g_aref;    // log2 (G / a_ref); +inf when a_ref == 0
};

struct NodeGeom {
    float4 cm;
    float3 bmin, bmax;
    uint32_t count;
};

// Squared distance between the group's box and the node's box (0 when they
// overlap).
__device__ __forceinline__ float box_gap2(const GroupGeom& g, const NodeGeom& n) {
    const float gx = fmaxf(0.0f, fmaxf(n.bmin.x - g.bmax.x, g.bmin.x - n.bmax.x));
    const float gy = fmaxf(0.0f, fmaxf(n.bmin.y - g.bmax.y, g.bmin.y - n.bmax.y));
    const float gz = fmaxf(0.0f, fmaxf(n.bmin.z - g.bmax.z, g.bmin.z - n.bmax.z));
    return gx * gx + gy * gy + gz * gz;
}

// Group theta rule (the learned criterion's ablation), with the softened
// distance of the reference's rule (bh_force.comp:62-66 adds the softening to
// r.r): accept when the boxes of the group and the node are disjoint and the
// node's half side is below theta times sqrt(d^2 + softening), d the distance
// from its centre of mass to the group's bounding sphere (0 inside it).
__device__ __forceinline__ float group_soft_dist2(const GroupGeom& g, const NodeGeom& n) {
    const float dx = n.cm.x - g.cx, dy = n.cm.y - g.cy, dz = n.cm.z - g.cz;
    const float D2 = dx * dx + dy * dy + dz * dz;
    const float D = D2 > 0.0f ? D2 * rsqrtf(D2) : 0.0f;
    const float d = fmaxf(D - g.R, 0.0f);
    return d * d + g.soft;
}

__device__ __forceinline__ float node_half(const NodeGeom& n) {
    const float ex = n.bmax.x - n.bmin.x, ey = n.bmax.y - n.bmin.y, ez = n.bmax.z - n.bmin.z;
    return 0.5f * fmaxf(ex, fmaxf(ey, ez));
}

__device__ __forceinline__ bool group_theta_accept(const GroupGeom& g, const NodeGeom& n, float theta) {
    const float half = node_half(n);
    return theta > 0.0f && half * half < theta * theta * group_soft_dist2(g, n) && box_gap2(g, n) > 0.0f;
}

// The smallest theta at which the group rule accepts the node,
// rho = half / sqrt(d^2 + softening); +inf when the boxes overlap.  The
// learned walk and the recording of training pairs compare it against the
// band's two thetas.
__device__ __forceinline__ float group_rho(const GroupGeom& g, const NodeGeom& n) {
    const float den2 = group_soft_dist2(g, n);
    return (den2 > 0.0f && box_gap2(g, n) > 0.0f) ? node_half(n) * rsqrtf(den2) : __int_as_float(0x7f800000);
}

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

__device__ __forceinline__ void group_feature_terms(GroupGeom& g, float G, float soft) {
    g.soft = soft;
    g.l_R = __log2f(fmaxf(g.R, 1e-30f));
    g.l_soft = __log2f(soft);  // -inf for zero softening: feature 9 clamps
    g.l_g_aref = g.a_ref > 0.f ? __log2f(G) - __log2f(g.a_ref) : __int_as_float(0x7f800000);
}

// The 12 features, all scale free.  h: half of the longest side; d: distance
// from the node's centre of mass to the group centre; R: group half diagonal
// (at least 1e-6 d); off: offset of the centre of mass from the box centre.
//   f0  log2(h/d)/8            f6  log2(min(count, 2^16))/16
//   f1  log2(R/d)/8            f7  cos(offset, direction to the group)
//   f2  log2(1 - R/d)/8        f8  log2(G m / (d^2 + soft) / a_ref)/16
//   f3  off/h                  f9  log2(soft / d^2)/16
//   f4  shortest/longest side  f10 log2(h/R)/8
//   f5  middle/longest side    f11 log2(max(box gap, 1e-6 h)/h)/8
// They are inputs of a BF16 network (8 significant bits), so the fast
// hardware log2, reciprocal and reciprocal square root are accurate enough;
// the logarithms of group terms are computed once per group.
__device__ __forceinline__ void mac_features(const GroupGeom& g, const NodeGeom& n, float f[MAC_FEATURES]) {
    const float ex = n.bmax.x - n.bmin.x, ey = n.bmax.y - n.bmin.y, ez = n.bmax.z - n.bmin.z;
    const float emax = fmaxf(ex, fmaxf(ey, ez));
    const float emin = fminf(ex, fminf(ey, ez));
    const float emid = ex + ey + ez - emax - emin;
    const float h = fmaxf(0.5f * emax, 1e-30f);
    const float dx = n.cm.x - g.cx, dy = n.cm.y - g.cy, dz = n.cm.z - g.cz;
    const float d2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-36f);
    const float inv_d = rsqrtf(d2);
    const float l_d2 = __log2f(d2);
    const float l_d = 0.5f * l_d2;
    const float l_h = __log2f(h);
    const float l_R = fmaxf(g.l_R, l_d - 19.931568f);  // R >= 1e-6 d
    const float R = fmaxf(g.R, 1e-6f * d2 * inv_d);
    const float inv_h = __fdividef(1.0f, h);
    const float ox = n.cm.x - 0.5f * (n.bmin.x + n.bmax.x);
    const float oy = n.cm.y - 0.5f * (n.bmin.y + n.bmax.y);
    const float oz = n.cm.z - 0.5f * (n.bmin.z + n.bmax.z);
    const float off2 = ox * ox + oy * oy + oz * oz;
    const float inv_off = rsqrtf(fmaxf(off2, 1e-36f));
    const float inv_emax = emax > 0.f ? __fdividef(1.0f, emax) : 0.f;
    const float gap2 = box_gap2(g, n);
    f[0] = clampf(l_h - l_d, -24.f, 8.f) * 0.125f;
    f[1] = clampf(l_R - l_d, -24.f, 8.f) * 0.125f;
    f[2] = __log2f(clampf(1.0f - R * inv_d, 1e-4f, 1.0f)) * 0.125f;
    f[3] = clampf(off2 * inv_off * inv_h, 0.f, 2.f);
    f[4] = emax > 0.f ? emin * inv_emax : 1.f;
    f[5] = emax > 0.f ? emid * inv_emax : 1.f;
    f[6] = __log2f((float)min(max(n.count, 1u), 1u << 16)) * (1.0f / 16.0f);
    f[7] = off2 > 1e-36f ? clampf((ox * dx + oy * dy + oz * dz) * inv_off * inv_d, -1.f, 1.f) : 0.f;
    f[8] = clampf(g.l_g_aref + __log2f(n.cm.w) - __log2f(d2 + g.soft), -32.f, 32.f) * (1.0f / 16.0f);
    f[9] = clampf(g.l_soft - l_d2, -48.f, 8.f) * (1.0f / 16.0f);
    f[10] = clampf(l_h - l_R, -16.f, 16.f) * 0.125f;
    f[11] = clampf(0.5f * __log2f(fmaxf(gap2, 1e-12f * h * h)) - l_h, -20.f, 8.f) * 0.125f;
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// ReLU and BF16 rounding of two values in one instruction (the same result as
// rounding max(x, 0): rounding keeps the sign)
__device__ __forceinline__ uint32_t pack_bf16x2_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
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
// The two 16-row m-tiles go through all three layers one after the other,
// which keeps the live accumulators to one tile's.  KEEP also returns the
// FP32 activations (training); inference fuses ReLU into the BF16 packing.
template <bool KEEP>
__device__ __forceinline__ float mac_forward_warp(const MacDeviceWeights& mw, uint32_t warp, uint32_t lane,
                                                  MacActs* acts) {
    __syncwarp();
    const uint32_t gid = lane >> 2, tig = lane & 3;
    const uint4* F4 = reinterpret_cast<const uint4*>(mw.smem_frag) + lane;  // chunk c at F4[32 c]
    const uint32_t* X = reinterpret_cast<const uint32_t*>(mw.smem_x + (size_t)warp * mw.x_rows * 16);
    auto act = [&](float x0, float x1) { return KEEP ? pack_bf16x2(x0, x1) : pack_bf16x2_relu(x0, x1); };
    float out[2][2];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        uint32_t a[4];
        a[0] = X[(16 * mt + gid) * 8 + tig];
        a[1] = X[(16 * mt + gid + 8) * 8 + tig];
        a[2] = X[(16 * mt + gid) * 8 + tig + 4];
        a[3] = X[(16 * mt + gid + 8) * 8 + tig + 4];
        // layer 1: 16 x 12(16) by 12(16) x 32, ReLU; n-tiles 2 ks, 2 ks + 1
        uint32_t a2[2][4];  // layer-2 A fragments [k-step]
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const uint4 wv = F4[32 * ks];
            const uint4 bv = F4[32 * (7 + ks)];
            float c[2][4] = {{__uint_as_float(bv.x), __uint_as_float(bv.y), __uint_as_float(bv.x), __uint_as_float(bv.y)},
                             {__uint_as_float(bv.z), __uint_as_float(bv.w), __uint_as_float(bv.z), __uint_as_float(bv.w)}};
            mma_bf16(c[0], a, wv.x, wv.y);
            mma_bf16(c[1], a, wv.z, wv.w);
            if (KEEP) {
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        c[h][r] = fmaxf(c[h][r], 0.0f);
                        acts->h1[mt][2 * ks + h][r] = c[h][r];
                    }
            }
            a2[ks][0] = act(c[0][0], c[0][1]);
            a2[ks][1] = act(c[0][2], c[0][3]);
            a2[ks][2] = act(c[1][0], c[1][1]);
            a2[ks][3] = act(c[1][2], c[1][3]);
        }
        // layer 2: 16 x 32 by 32 x 32, ReLU; its output is layer 3's A
        uint32_t a3[2][4];
#pragma unroll
        for (int ks3 = 0; ks3 < 2; ++ks3) {
            const uint4 bv = F4[32 * (9 + ks3)];
            float c[2][4] = {{__uint_as_float(bv.x), __uint_as_float(bv.y), __uint_as_float(bv.x), __uint_as_float(bv.y)},
                             {__uint_as_float(bv.z), __uint_as_float(bv.w), __uint_as_float(bv.z), __uint_as_float(bv.w)}};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * ks3 + h;
                const uint4 wv = F4[32 * (2 + nt)];  // (k-step 0: b0 b1, k-step 1: b0 b1)
                mma_bf16(c[h], a2[0], wv.x, wv.y);
                mma_bf16(c[h], a2[1], wv.z, wv.w);
                if (KEEP)
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        c[h][r] = fmaxf(c[h][r], 0.0f);
                        acts->h2[mt][nt][r] = c[h][r];
                    }
            }
            a3[ks3][0] = act(c[0][0], c[0][1]);
            a3[ks3][1] = act(c[0][2], c[0][3]);
            a3[ks3][2] = act(c[1][0], c[1][1]);
            a3[ks3][3] = act(c[1][2], c[1][3]);
        }
        // layer 3: 16 x 32 by 32 x 1 (one useful column of an n8 tile)
        const uint4 w3 = F4[32 * 6];
        float o[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(o, a3[0], w3.x, w3.y);
        mma_bf16(o, a3[1], w3.z, w3.w);
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
    const float b3 = __uint_as_float(mw.smem_frag[(11 * 32 + lane) * 4]);
    return v + b3;
}

__device__ __forceinline__ float mac_infer_warp(const MacDeviceWeights& mw, uint32_t warp, uint32_t lane) {
    return mac_forward_warp<false>(mw, warp, lane, nullptr);
}

// Copy the fragment table into the block's shared memory (all threads);
// smem_frag holds MAC_SMEM_FRAG_WORDS words.
__device__ __forceinline__ void mac_load_frag(MacDeviceWeights& mw, uint32_t* smem_frag, __nv_bfloat16* smem_x,
                                              uint32_t x_rows = 32) {
    // [word][lane] in global memory -> [chunk][lane][4] here
    for (uint32_t i = threadIdx.x; i < MAC_FRAG_WORDS * 32; i += blockDim.x) {
        const uint32_t word = i >> 5, l = i & 31;
        smem_frag[((word >> 2) * 32 + l) * 4 + (word & 3)] = mw.frag[i];
    }
    mw.smem_frag = smem_frag;
    mw.smem_x = smem_x;
    mw.x_rows = x_rows;
    __syncthreads();
}

// smallest |a| of the group's bodies in the previous step (feature 8)
// (act[q], slot[q]: the lane's bodies, q < BPL)
template <int BPL>
__device__ __forceinline__ float group_accel_ref(const StepBuffers& b, const bool (&act)[BPL],
                                                 const uint32_t (&slot)[BPL]) {
    float a = 3.0e38f;
#pragma unroll
    for (int q = 0; q < BPL; ++q)
        if (act[q] && b.accel_mag) a = fminf(a, b.accel_mag[b.idx_in[slot[q]]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
    return a < 3.0e38f ? a : 0.0f;
}
