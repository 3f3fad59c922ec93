// k_diag.cu — the accuracy reference (an FP64 direct sum of sampled bodies),
// the FP64 diagnostics of conserved quantities, and the FP64 positions of the
// precision form.
//
// The reference has no accuracy check.  The direct sum adds G m_j r / (r.r + eps^2)^1.5
// over every live body j != i for a sample of bodies i, with FP64 terms and
// FP64 sums: positions come from the precision form's FP64 copy when it is
// current, otherwise the FP32 body positions widened to FP64 (exactly).  This
// is the judge every acceleration-error distribution is measured against.
//
// Grid: (sample blocks) x (source chunks).  Each block keeps 128 targets in
// registers and streams its chunk of sources through shared memory; partial
// sums per chunk are reduced in FP64 in a fixed order (deterministic).
#include "gbh_common.cuh"

#define DS_THREADS 128
#define DS_TILE 512

__global__ void k_direct_sum_reduce(const double* __restrict__ partial, uint32_t count, uint32_t chunks,
                                    double* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * count) return;
    double s = 0.0;
    for (uint32_t c = 0; c < chunks; ++c) s += partial[(size_t)c * count * 3 + t];
    out[t] = s;
}

// ---------------------------------------------------------------------------
// FP64 direct sum: positions from the FP64 copy (pos64 != null) or the FP32
// body positions widened, terms and sums in FP64 (the GB300 runs FP64 at a
// fraction of the FP32 rate; the judge samples a few thousand bodies).
__global__ __launch_bounds__(DS_THREADS) void k_direct_sum64(const double* __restrict__ pos64,
                                                             const gbh_body* __restrict__ bodies, uint32_t nb,
                                                             const uint32_t* __restrict__ sample, uint32_t count,
                                                             double G, double soft, uint32_t chunks,
                                                             double* __restrict__ partial) {
    struct Src {
        double x, y, z, w;  // FP64 position and mass of a source body
    };
    __shared__ Src s_src[DS_TILE / 2];
    const uint32_t t = blockIdx.x * DS_THREADS + threadIdx.x;
    const uint32_t chunk = blockIdx.y;
    const bool valid = t < count;
    const uint32_t i = valid ? sample[t] : 0u;
    double mx = 0.0, my = 0.0, mz = 0.0;
    if (valid && pos64) {
        mx = pos64[4 * (size_t)i];
        my = pos64[4 * (size_t)i + 1];
        mz = pos64[4 * (size_t)i + 2];
    } else if (valid) {
        const float4 pm = ld_pos_mass(bodies, i);
        mx = pm.x;
        my = pm.y;
        mz = pm.z;
    }
    const uint32_t per = (nb + chunks - 1) / chunks;
    const uint32_t j0 = chunk * per;
    const uint32_t j1 = min(nb, j0 + per);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    const uint32_t tile = DS_TILE / 2;
    for (uint32_t base = j0; base < j1; base += tile) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < tile; k += DS_THREADS) {
            const uint32_t j = base + k;
            Src v = {0.0, 0.0, 0.0, 0.0};
            if (j < j1) {
                const float4 pm = ld_pos_mass(bodies, j);
                if (pos64) {
                    v.x = pos64[4 * (size_t)j];
                    v.y = pos64[4 * (size_t)j + 1];
                    v.z = pos64[4 * (size_t)j + 2];
                } else {
                    v.x = pm.x;
                    v.y = pm.y;
                    v.z = pm.z;
                }
                v.w = (double)pm.w;
            }
            s_src[k] = v;
        }
        __syncthreads();
        const uint32_t cnt = min(tile, j1 - base);
        for (uint32_t k = 0; k < cnt; ++k) {
            const Src s = s_src[k];
            if (s.w == 0.0) continue;
            const double rx = s.x - mx, ry = s.y - my, rz = s.z - mz;
            const double rr = rx * rx + ry * ry + rz * rz;
            if (rr == 0.0) continue;  // the body itself
            const double inv = 1.0 / sqrt(rr + soft);
            const double f = G * s.w * inv * inv * inv;
            sx += f * rx;
            sy += f * ry;
            sz += f * rz;
        }
    }
    if (valid) {
        double* o = partial + ((size_t)chunk * count + t) * 3;
        o[0] = sx;
        o[1] = sy;
        o[2] = sz;
    }
}

void launch_direct_sum64(const double* pos64, const gbh_body* bodies, uint32_t nb, const uint32_t* sample,
                         uint32_t count, double G, double soft, double* partial, double* out, uint32_t chunks,
                         cudaStream_t s) {
    dim3 grid((count + DS_THREADS - 1) / DS_THREADS, chunks);
    k_direct_sum64<<<grid, DS_THREADS, 0, s>>>(pos64, bodies, nb, sample, count, G, soft, chunks, partial);
    k_direct_sum_reduce<<<(3 * count + 255) / 256, 256, 0, s>>>(partial, count, chunks, out);
}

// ---------------------------------------------------------------------------
// Conserved quantities in FP64 over the non-empty bodies (mass != 0): per
// block partial sums in a fixed order, then one block sums the partials in
// block order (deterministic).
#define DG_THREADS 256
#define DG_VALUES 15  // mass, p[3], m x[3], K, W, L[3], count, pad, pad

__global__ __launch_bounds__(DG_THREADS) void k_diag_partial(const gbh_body* __restrict__ bodies, uint32_t nb,
                                                             const double* __restrict__ pos64,
                                                             const float* __restrict__ potential,
                                                             double* __restrict__ partial) {
    __shared__ double s_red[DG_THREADS / 32][DG_VALUES];
    double v[DG_VALUES];
#pragma unroll
    for (int k = 0; k < DG_VALUES; ++k) v[k] = 0.0;
    for (uint32_t i = blockIdx.x * DG_THREADS + threadIdx.x; i < nb; i += gridDim.x * DG_THREADS) {
        const float4 pm = ld_pos_mass(bodies, i);
        if (pm.w == 0.0f) continue;
        const float4 vd = ld_vel_density(bodies, i);
        const double m = pm.w;
        double x = pm.x, y = pm.y, z = pm.z;
        if (pos64) {
            x = pos64[4 * (size_t)i];
            y = pos64[4 * (size_t)i + 1];
            z = pos64[4 * (size_t)i + 2];
        }
        const double vx = vd.x, vy = vd.y, vz = vd.z;
        v[0] += m;
        v[1] += m * vx;
        v[2] += m * vy;
        v[3] += m * vz;
        v[4] += m * x;
        v[5] += m * y;
        v[6] += m * z;
        v[7] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        if (potential) v[8] += 0.5 * m * (double)potential[i];
        v[9] += m * (y * vz - z * vy);
        v[10] += m * (z * vx - x * vz);
        v[11] += m * (x * vy - y * vx);
        v[12] += 1.0;
    }
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < DG_VALUES; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) s_red[w][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < DG_VALUES) {
        double x = 0.0;
        for (int ww = 0; ww < DG_THREADS / 32; ++ww) x += s_red[ww][threadIdx.x];
        partial[(size_t)blockIdx.x * DG_VALUES + threadIdx.x] = x;
    }
}

__global__ void k_diag_final(const double* __restrict__ partial, uint32_t blocks, double* __restrict__ out) {
    const uint32_t k = threadIdx.x;
    if (k >= DG_VALUES) return;
    double x = 0.0;
    for (uint32_t bidx = 0; bidx < blocks; ++bidx) x += partial[(size_t)bidx * DG_VALUES + k];
    out[k] = x;
}

// out: DG_VALUES doubles (device); partial: blocks * DG_VALUES doubles (device)
void launch_diagnostics(const gbh_body* bodies, uint32_t nb, const double* pos64, const float* potential,
                        double* partial, uint32_t blocks, double* out, cudaStream_t s) {
    k_diag_partial<<<blocks, DG_THREADS, 0, s>>>(bodies, nb, pos64, potential, partial);
    k_diag_final<<<1, 32, 0, s>>>(partial, blocks, out);
}

// FP64 positions from the body buffer (start of the precision form)
__global__ void k_init_pos64(const gbh_body* __restrict__ bodies, double* __restrict__ pos64, uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 pm = ld_pos_mass(bodies, i);
    reinterpret_cast<double2*>(pos64)[2 * (size_t)i] = make_double2(pm.x, pm.y);
    reinterpret_cast<double2*>(pos64)[2 * (size_t)i + 1] = make_double2(pm.z, 0.0);
}

void launch_init_pos64(const gbh_body* bodies, double* pos64, uint32_t N, cudaStream_t s) {
    k_init_pos64<<<(N + 255) / 256, 256, 0, s>>>(bodies, pos64, N);
}

// FP32 body positions from FP64 ones, bodies [offset, offset + count)
__global__ void k_round_pos64(gbh_body* __restrict__ bodies, const double* __restrict__ pos64, uint32_t offset,
                              uint32_t count) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const uint32_t i = offset + t;
    float4* p = reinterpret_cast<float4*>(bodies) + 2 * (size_t)i;
    const float4 pm = *p;
    *p = make_float4((float)pos64[4 * (size_t)i], (float)pos64[4 * (size_t)i + 1], (float)pos64[4 * (size_t)i + 2], pm.w);
}

void launch_round_pos64(gbh_body* bodies, const double* pos64, uint32_t offset, uint32_t count, cudaStream_t s) {
    if (count) k_round_pos64<<<(count + 255) / 256, 256, 0, s>>>(bodies, pos64, offset, count);
}
