// k_ic.cu — seeded initial conditions written straight into the body buffer
// (gbh_generate_bodies).  One thread per body.  Every number comes from a
// counter-based generator: draw d of body i under seed s is the splitmix64
// finaliser of s * K0 + (i + 1) * K1 + (d + 1) * K2 (mod 2^64), whose top 24
// bits make a float in [0, 1); nothing depends on the launch shape, so chunked
// and one-shot generation agree.
//
// Kinds (gbh.h):
//   BOX       makeNewRandomBox, PlanetGenerator.java:310-321;
//   DISK      makeNewRandomDisk, PlanetGenerator.java:418-489 (the last body
//             of the range is the centre body);
//   PLUMMER   Aarseth, Henon & Wielen (1974);
//   CLUSTERS  Gaussian mixture with m^-2 masses.
#include "gbh_common.cuh"

namespace {

constexpr uint64_t K0 = 0x9E3779B97F4A7C15ull, K1 = 0xD1B54A32D192ED03ull, K2 = 0x8CB92BA72F3D8DD7ull;
constexpr uint64_t CLUSTER_SALT = 0x632BE59BD9B4E019ull;
constexpr float TWO_PI = 6.28318530717958647692f;
constexpr float PI_F = 3.14159265358979323846f;

__device__ __forceinline__ float ic_uniform(uint64_t seed, uint32_t index, uint32_t draw) {
    uint64_t z = seed * K0 + ((uint64_t)index + 1ull) * K1 + ((uint64_t)draw + 1ull) * K2;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(uint32_t)(z >> 40) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ float3 unit_vector(float uz, float uphi) {
    const float z = 2.0f * uz - 1.0f;
    const float phi = TWO_PI * uphi;
    const float s = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    return make_float3(s * cosf(phi), s * sinf(phi), z);
}

__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

__device__ __forceinline__ float3 normalize3(float3 a) {
    const float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return l > 0.0f ? make_float3(a.x / l, a.y / l, a.z / l) : a;
}

// polarToPlanarCoordinates (PlanetGenerator.java:341-347): r (cos t u + sin t v)
__device__ __forceinline__ float3 polar(float r, float t, float3 u, float3 v) {
    const float a = r * cosf(t), b = r * sinf(t);
    return make_float3(u.x * a + v.x * b, u.y * a + v.y * b, u.z * a + v.z * b);
}

__device__ __forceinline__ float range(const gbh_ic_params& p, int k, float u) { return u * (p.hi[k] - p.lo[k]) + p.lo[k]; }

__global__ void k_generate(gbh_body* __restrict__ out, uint32_t count, uint32_t offset, gbh_ic_params p, uint64_t seed) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const uint32_t i = offset + t;  // the body's index keys its draws
    float3 pos = make_float3(0.f, 0.f, 0.f), vel = pos;
    float mass = 0.f, density = 1.f;
    if (p.kind == GBH_IC_BOX) {
        pos = make_float3(range(p, 0, ic_uniform(seed, i, 0)), range(p, 1, ic_uniform(seed, i, 1)),
                          range(p, 2, ic_uniform(seed, i, 2)));
        vel = make_float3(range(p, 3, ic_uniform(seed, i, 3)), range(p, 4, ic_uniform(seed, i, 4)),
                          range(p, 5, ic_uniform(seed, i, 5)));
        mass = range(p, 6, ic_uniform(seed, i, 6));
        density = range(p, 7, ic_uniform(seed, i, 7));
    } else if (p.kind == GBH_IC_DISK) {
        if (t == count - 1) {
            // the centre body (PlanetGenerator.java:485-486)
            mass = p.center_mass;
            density = p.center_density;
        } else {
            const float3 n = make_float3(0.0f, sinf(p.phi), cosf(p.phi));
            const float3 a = fabsf(n.x) < 0.9f ? make_float3(1.f, 0.f, 0.f) : make_float3(0.f, 1.f, 0.f);
            const float3 u = normalize3(cross3(n, a));
            const float3 v = cross3(n, u);
            const float r = range(p, 0, ic_uniform(seed, i, 0));
            const float theta = ic_uniform(seed, i, 1) * TWO_PI;
            float dev = PI_F * (1.0f - powf(ic_uniform(seed, i, 2), 1.0f - p.adherence));
            if (!(ic_uniform(seed, i, 3) < 0.5f)) dev = -dev;
            const float3 planar = polar(1.0f, theta, u, v);
            const float3 dir = polar(1.0f, dev, planar, n);
            const float3 nn = polar(1.0f, dev, n, planar);
            const float num = (float)(count - 1);
            const float approx = (p.hi[6] + p.lo[6]) / 2.0f * num * powf(r / p.hi[0], p.center_density + 1.0f);
            pos = make_float3(dir.x * r, dir.y * r, dir.z * r);
            if (p.flags & GBH_IC_ORBITAL) {
                const float sgn = (p.flags & GBH_IC_CCW) ? 1.0f : -1.0f;
                const float speed = sqrtf((p.center_mass + approx) * p.G / r) * p.orbital_factor;
                const float3 td = normalize3(cross3(nn, dir));
                vel = make_float3(td.x * speed * sgn, td.y * speed * sgn, td.z * speed * sgn);
            }
            mass = range(p, 6, ic_uniform(seed, i, 4));
            density = range(p, 7, ic_uniform(seed, i, 5));
        }
        pos = make_float3(pos.x + p.center[0], pos.y + p.center[1], pos.z + p.center[2]);
        vel = make_float3(vel.x + p.velocity[0], vel.y + p.velocity[1], vel.z + p.velocity[2]);
    } else if (p.kind == GBH_IC_PLUMMER) {
        const float a = p.scale;
        const float x1 = fmaxf(ic_uniform(seed, i, 0) * 0.999f, 1e-12f);
        const float r = a / sqrtf(powf(x1, -2.0f / 3.0f) - 1.0f);
        const float3 d = unit_vector(ic_uniform(seed, i, 1), ic_uniform(seed, i, 2));
        // speed fraction from g(q) = q^2 (1 - q^2)^(7/2) (maximum below 0.1),
        // at most 64 rejection rounds (acceptance about 0.5 per round)
        float q = 0.0f;
        for (uint32_t k = 0; k < 64; ++k) {
            const float x4 = ic_uniform(seed, i, 3 + 2 * k);
            const float x5 = 0.1f * ic_uniform(seed, i, 4 + 2 * k);
            const float w = 1.0f - x4 * x4;
            if (x5 < x4 * x4 * w * w * w * sqrtf(w)) {
                q = x4;
                break;
            }
        }
        const float vesc = sqrtf(2.0f * p.G * p.total_mass / a) * powf(1.0f + (r / a) * (r / a), -0.25f);
        const float3 e = unit_vector(ic_uniform(seed, i, 200), ic_uniform(seed, i, 201));
        pos = make_float3(d.x * r + p.center[0], d.y * r + p.center[1], d.z * r + p.center[2]);
        const float s = q * vesc;
        vel = make_float3(e.x * s + p.velocity[0], e.y * s + p.velocity[1], e.z * s + p.velocity[2]);
        mass = p.total_mass / (float)count;
        density = p.density;
    } else {  // GBH_IC_CLUSTERS
        const uint32_t k = p.clusters ? p.clusters : 1u;
        const uint32_t c = min((uint32_t)(ic_uniform(seed, i, 0) * (float)k), k - 1u);
        const uint64_t cs = seed + CLUSTER_SALT;
        const float3 centre = make_float3((2.0f * ic_uniform(cs, c, 0) - 1.0f) * p.scale,
                                          (2.0f * ic_uniform(cs, c, 1) - 1.0f) * p.scale,
                                          (2.0f * ic_uniform(cs, c, 2) - 1.0f) * p.scale);
        const float lsig = logf(p.sigma_lo) + ic_uniform(cs, c, 3) * (logf(p.sigma_hi) - logf(p.sigma_lo));
        const float sig = expf(lsig);
        // Box-Muller normals
        float g[4];
        for (int h = 0; h < 2; ++h) {
            const float u1 = fmaxf(ic_uniform(seed, i, 1 + 2 * h), 1e-7f), u2 = ic_uniform(seed, i, 2 + 2 * h);
            const float rr = sqrtf(-2.0f * logf(u1));
            g[2 * h] = rr * cosf(TWO_PI * u2);
            g[2 * h + 1] = rr * sinf(TWO_PI * u2);
        }
        pos = make_float3(centre.x + g[0] * sig, centre.y + g[1] * sig, centre.z + g[2] * sig);
        vel = make_float3(p.velocity[0], p.velocity[1], p.velocity[2]);
        const float lo = p.lo[6], hi = p.hi[6], um = ic_uniform(seed, i, 5);
        mass = 1.0f / (1.0f / lo - um * (1.0f / lo - 1.0f / hi));
        density = p.density;
    }
    float4* b = reinterpret_cast<float4*>(&out[i]);
    b[0] = make_float4(pos.x, pos.y, pos.z, mass);
    b[1] = make_float4(vel.x, vel.y, vel.z, density);
}

}  // namespace

void launch_generate_bodies(gbh_body* bodies, uint32_t count, uint32_t offset, const gbh_ic_params& p, uint64_t seed,
                            cudaStream_t s) {
    if (!count) return;
    k_generate<<<(count + 255) / 256, 256, 0, s>>>(bodies, count, offset, p, seed);
}
