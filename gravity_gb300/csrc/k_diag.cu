// k_diag.cu — the accuracy judge: direct-sum accelerations of sampled bodies.
//
// The reference has no accuracy check.  The judge sums G m_j r / (r.r + eps^2)^1.5
// over every live body j != i for a sample of bodies i.  Each term is computed
// in FP32 (the positions are FP32, so r = x_j - x_i carries one rounding) and
// the sums are carried in double-float (TwoSum compensation), so the result
// matches an FP64 direct sum to ~1e-6 relative while running at FP32 rate
// (the GB300's FP64 rate is 1/64 of FP32).
//
// Grid: (sample blocks) x (source chunks).  Each block keeps 128 targets in
// registers and streams its chunk of sources through shared memory; partial
// sums per chunk are reduced in FP64 in a fixed order (deterministic).
#include "gbh_common.cuh"

#define DS_THREADS 128
#define DS_TILE 512

__device__ __forceinline__ void two_sum(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo = lo + err;
}

__global__ __launch_bounds__(DS_THREADS) void k_direct_sum(const gbh_body* __restrict__ bodies, uint32_t nb,
                                                           const uint32_t* __restrict__ sample, uint32_t count, float G,
                                                           float soft, uint32_t chunks, double* __restrict__ partial) {
    __shared__ float4 s_src[DS_TILE];
    const uint32_t t = blockIdx.x * DS_THREADS + threadIdx.x;
    const uint32_t chunk = blockIdx.y;
    const bool valid = t < count;
    const uint32_t i = valid ? sample[t] : 0u;
    const float4 me = valid ? ld_pos_mass(bodies, i) : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t per = (nb + chunks - 1) / chunks;
    const uint32_t j0 = chunk * per;
    const uint32_t j1 = min(nb, j0 + per);
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f, hz = 0.f, lz = 0.f;
    for (uint32_t base = j0; base < j1; base += DS_TILE) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < DS_TILE; k += DS_THREADS) {
            const uint32_t j = base + k;
            s_src[k] = j < j1 ? ld_pos_mass(bodies, j) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)DS_TILE, j1 - base);
        for (uint32_t k = 0; k < cnt; ++k) {
            const float4 s = s_src[k];
            if (s.w == 0.0f) continue;
            const float rx = s.x - me.x, ry = s.y - me.y, rz = s.z - me.z;
            const float rr = rx * rx + ry * ry + rz * rz;
            if (rr == 0.0f) continue;  // the body itself (a zero vector adds nothing)
            const float d2 = rr + soft;
            const float inv = 1.0f / sqrtf(d2);
            const float f = G * s.w * inv * inv * inv;
            two_sum(hx, lx, f * rx);
            two_sum(hy, ly, f * ry);
            two_sum(hz, lz, f * rz);
        }
    }
    if (valid) {
        double* o = partial + ((size_t)chunk * count + t) * 3;
        o[0] = (double)hx + (double)lx;
        o[1] = (double)hy + (double)ly;
        o[2] = (double)hz + (double)lz;
    }
}

__global__ void k_direct_sum_reduce(const double* __restrict__ partial, uint32_t count, uint32_t chunks,
                                    double* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * count) return;
    double s = 0.0;
    for (uint32_t c = 0; c < chunks; ++c) s += partial[(size_t)c * count * 3 + t];
    out[t] = s;
}

void launch_direct_sum(const gbh_body* bodies, uint32_t nb, const uint32_t* sample, uint32_t count, float G,
                       float soft, double* partial, double* out, uint32_t chunks, cudaStream_t s) {
    dim3 grid((count + DS_THREADS - 1) / DS_THREADS, chunks);
    k_direct_sum<<<grid, DS_THREADS, 0, s>>>(bodies, nb, sample, count, G, soft, chunks, partial);
    k_direct_sum_reduce<<<(3 * count + 255) / 256, 256, 0, s>>>(partial, count, chunks, out);
}
