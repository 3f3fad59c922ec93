// k_prepare.cu — step reset, dead-body compaction, dynamic AABB and Morton
// encode, fused into three passes over the index.
//
// Reference stages replaced (SH = src/main/resources/shaders):
//   resetValues        SH/compute/update/bh_update.comp:10-28
//   partitionDead      SH/compute/dead/bh_dead.comp:13-112 (+ GPU.swapMortonAndIndexBuffers)
//   decrementDead      SH/compute/update/bh_update.comp:29-34
//   updateBounds       SH/compute/morton/bh_morton.comp:36-231
//   generateMorton     SH/compute/morton/bh_morton.comp:238-262
//
// Pass 1 (prep_count): per tile of PREP_TILE sorted slots, count the dead
//   bodies, zero them in both body buffers, and reduce the AABB of the finite
//   inliers (the alive set is the same set the reference's repopulate kernel
//   sees after compaction, and min/max unions are order independent).
// Pass 2 (prep_scan, one block): exclusive scan of the per-tile dead counts,
//   justDied, the new live count, and the bounds collapse with the 1.1x growth
//   cap.
// Pass 3 (prep_scatter): stable alive-first / dead-last scatter of the index,
//   the Morton key of every alive body written at its new slot, and the
//   histograms of all eight radix digits for the onesweep sort.
#include "gbh_common.cuh"

// ---------------------------------------------------------------------------
__global__ void k_reset(StepBuffers b) {
    const gbh_step_params* p = b.params;
    DevState* st = b.st;
    for (uint32_t i = threadIdx.x; i < SORT_PASSES * SORT_RADIX; i += blockDim.x) b.hist[i] = 0;
    if (threadIdx.x < SORT_PASSES) st->sort_tiles[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        b.mq->head = 0;
        b.mq->tail = 0;
        st->merge_conflicts = 0;
        st->merged = 0;
        st->oob = 0;
        st->tree_height = 0;
        st->max_stack = 0;
        st->merge_tasks = 0;
        st->interactions = 0;
        st->opened = 0;
        st->mac_evals = 0;
        st->frontier_saturated = 0;
        st->fill_frontier = 0;
        // units update, bh_update.comp:22-25 / common.glsl:346-360
        if (p->units.mass != 0.0f) {
            gbh_sim_values* sim = b.sim;
            const gbh_units u = p->units;
            sim->unit_mass = u.mass;
            sim->unit_density = u.density;
            sim->unit_len = u.len;
            sim->unit_time = u.time;
            if (u.camera_scale != 0.0f) sim->camera_scale = u.camera_scale;
            if (u.gravitational_constant > 0.0f) {
                sim->gravitational_constant = u.gravitational_constant;
            } else {
                float g = 6.67430e-11f * powf(u.len, -3.0f);
                g = g * powf(u.time, 2.0f);
                g = g * powf(u.mass, 1.0f);
                sim->gravitational_constant = g;
            }
            sim->body_length_constant = 0.6203504909f * powf(u.mass / u.density, 1.0f / 3.0f) / u.len;
        }
    }
}

void launch_reset(const StepBuffers& b, cudaStream_t s) { k_reset<<<1, 256, 0, s>>>(b); }

// ---------------------------------------------------------------------------
__device__ __forceinline__ void warp_minmax(float v[6]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            v[k] = gmin(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
            v[3 + k] = gmax(v[3 + k], __shfl_xor_sync(0xffffffffu, v[3 + k], o));
        }
    }
}

__global__ __launch_bounds__(PREP_THREADS) void k_prep_count(StepBuffers b) {
    const gbh_sim_values* sim = b.sim;
    const uint32_t n = sim->num_bodies;
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * PREP_TILE;
    if (base >= n) return;
    const bool dynamic = b.params->static_or_dynamic == GBH_BOUNDS_DYNAMIC;
    // positions in index order from the last walk when nothing changed them since
    const bool sorted = b.st->sorted_valid != 0u;
    float pmin[3], pmax[3], lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        pmin[k] = sim->bounds_min[k];
        pmax[k] = sim->bounds_max[k];
    }
    const bool prev_empty = pmin[0] > pmax[0];
    // mortonInlierWindow, bh_morton.comp:50-56
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float c = 0.5f * (pmin[k] + pmax[k]);
        float h = gmax(0.5f * (pmax[k] - pmin[k]) * 1.05f, 1e-9f);
        lo[k] = c - h;
        hi[k] = c + h;
    }
    float box[6] = {1e38f, 1e38f, 1e38f, -1e38f, -1e38f, -1e38f};
    uint32_t dead = 0;
#pragma unroll
    for (int it = 0; it < PREP_ITEMS; ++it) {
        const uint32_t g = base + it * PREP_THREADS + threadIdx.x;
        if (g < n) {
            const uint32_t bi = b.idx_in[g];
            const float4 pm = sorted ? b.sorted_pm[g] : ld_pos_mass(b.bodies_in, bi);
            if (pm.w == 0.0f) {
                ++dead;
                const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                st_body(b.bodies_in, bi, z, z);
                st_body(b.bodies_out, bi, z, z);
            } else if (dynamic && finite3(pm.x, pm.y, pm.z)) {
                // mortonContributorAABB, bh_morton.comp:60-74
                bool inlier = prev_empty || !(pm.x < lo[0] || pm.y < lo[1] || pm.z < lo[2] || pm.x > hi[0] ||
                                              pm.y > hi[1] || pm.z > hi[2]);
                if (inlier) {
                    box[0] = gmin(box[0], pm.x);
                    box[1] = gmin(box[1], pm.y);
                    box[2] = gmin(box[2], pm.z);
                    box[3] = gmax(box[3], pm.x);
                    box[4] = gmax(box[4], pm.y);
                    box[5] = gmax(box[5], pm.z);
                }
            }
        }
    }
    __shared__ float s_box[PREP_THREADS / 32][6];
    __shared__ uint32_t s_dead[PREP_THREADS / 32];
    warp_minmax(box);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dead += __shfl_xor_sync(0xffffffffu, dead, o);
    const uint32_t w = threadIdx.x >> 5;
    if (lane_id() == 0) {
        s_dead[w] = dead;
#pragma unroll
        for (int k = 0; k < 6; ++k) s_box[w][k] = box[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t d = 0;
        float r[6] = {1e38f, 1e38f, 1e38f, -1e38f, -1e38f, -1e38f};
        for (int i = 0; i < PREP_THREADS / 32; ++i) {
            d += s_dead[i];
            for (int k = 0; k < 3; ++k) {
                r[k] = gmin(r[k], s_box[i][k]);
                r[3 + k] = gmax(r[3 + k], s_box[i][3 + k]);
            }
        }
        b.tile_dead[tile] = d;
        for (int k = 0; k < 6; ++k) b.tile_aabb[6 * tile + k] = r[k];
    }
}

// ---------------------------------------------------------------------------
__global__ __launch_bounds__(1024) void k_prep_scan(StepBuffers b) {
    gbh_sim_values* sim = b.sim;
    DevState* st = b.st;
    const uint32_t n = sim->num_bodies;
    const uint32_t tiles = (n + PREP_TILE - 1) / PREP_TILE;
    const uint32_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const uint32_t t0 = threadIdx.x * per;
    const uint32_t t1 = min(t0 + per, tiles);
    uint32_t local = 0;
    float box[6] = {1e38f, 1e38f, 1e38f, -1e38f, -1e38f, -1e38f};
    for (uint32_t t = t0; t < t1; ++t) {
        local += b.tile_dead[t];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            box[k] = gmin(box[k], b.tile_aabb[6 * t + k]);
            box[3 + k] = gmax(box[3 + k], b.tile_aabb[6 * t + 3 + k]);
        }
    }
    // block exclusive scan of `local`
    __shared__ uint32_t s_w[32];
    __shared__ float s_box[32][6];
    uint32_t incl = local;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    warp_minmax(box);
    if (lane == 31) s_w[w] = incl;
    if (lane == 0)
        for (int k = 0; k < 6; ++k) s_box[w][k] = box[k];
    __syncthreads();
    if (w == 0) {
        uint32_t v = s_w[lane];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        s_w[lane] = x - v;  // exclusive warp offsets
    }
    __syncthreads();
    uint32_t run = s_w[w] + incl - local;
    for (uint32_t t = t0; t < t1; ++t) {
        uint32_t v = b.tile_dead[t];
        b.tile_dead[t] = run;  // exclusive prefix of dead bodies per tile
        run += v;
    }
    if (threadIdx.x == blockDim.x - 1) {
        const uint32_t died = run;
        st->n_old = n;
        st->just_died = died;
        st->n_new = n - died;
        // decrementDeadBodies, bh_update.comp:29-34
        sim->num_bodies = n - died;
        sim->just_died = 0;
        sim->uint_debug[0] = 0;
    }
    if (b.params->static_or_dynamic == GBH_BOUNDS_DYNAMIC && threadIdx.x == 0) {
        float r[6] = {1e38f, 1e38f, 1e38f, -1e38f, -1e38f, -1e38f};
        for (uint32_t i = 0; i < (blockDim.x + 31) / 32; ++i)
            for (int k = 0; k < 3; ++k) {
                r[k] = gmin(r[k], s_box[i][k]);
                r[3 + k] = gmax(r[3 + k], s_box[i][3 + k]);
            }
        float pmin[3], pmax[3];
        for (int k = 0; k < 3; ++k) {
            pmin[k] = sim->bounds_min[k];
            pmax[k] = sim->bounds_max[k];
        }
        const bool prev_empty = pmin[0] > pmax[0];
        const bool res_empty = r[0] > r[3];
        // mortonAABBCollapseKernel, bh_morton.comp:218-230
        if (res_empty) {
            if (prev_empty)
                for (int k = 0; k < 3; ++k) {
                    sim->bounds_min[k] = r[k];
                    sim->bounds_max[k] = r[3 + k];
                }
        } else if (prev_empty) {
            for (int k = 0; k < 3; ++k) {
                sim->bounds_min[k] = r[k];
                sim->bounds_max[k] = r[3 + k];
            }
        } else {
            // clampAABBExtentGrowth, bh_morton.comp:77-88
            for (int k = 0; k < 3; ++k) {
                float prev_ext = gmax(pmax[k] - pmin[k], 1e-9f);
                float max_ext = prev_ext * 1.1f;
                float c = 0.5f * (r[k] + r[3 + k]);
                float h = 0.5f * (r[3 + k] - r[k]);
                float mh = 0.5f * max_ext;
                h = gmin(h, mh);
                sim->bounds_min[k] = c - h;
                sim->bounds_max[k] = c + h;
            }
        }
    }
}

// ---------------------------------------------------------------------------
__global__ __launch_bounds__(PREP_THREADS) void k_prep_scatter(StepBuffers b) {
    const DevState* st = b.st;
    const uint32_t n_old = st->n_old;
    const uint32_t n_new = st->n_new;
    const uint32_t tile = blockIdx.x;
    const uint32_t base = tile * PREP_TILE;
    if (base >= n_old) return;
    const bool sorted = st->sorted_valid != 0u;
    __shared__ uint32_t s_hist[SORT_PASSES * SORT_RADIX];
    __shared__ uint32_t s_cnt[PREP_ITEMS][PREP_THREADS / 32];
    __shared__ float s_mn[3], s_mx[3];
    for (uint32_t i = threadIdx.x; i < SORT_PASSES * SORT_RADIX; i += PREP_THREADS) s_hist[i] = 0;
    if (threadIdx.x < 3) {
        s_mn[threadIdx.x] = b.sim->bounds_min[threadIdx.x];
        s_mx[threadIdx.x] = b.sim->bounds_max[threadIdx.x];
    }
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    uint32_t bidx[PREP_ITEMS];
    float4 pm[PREP_ITEMS];
    uint32_t wrank[PREP_ITEMS];
    bool alive[PREP_ITEMS];
#pragma unroll
    for (int it = 0; it < PREP_ITEMS; ++it) {
        const uint32_t g = base + it * PREP_THREADS + threadIdx.x;
        const bool in = g < n_old;
        bidx[it] = in ? b.idx_in[g] : 0u;
        pm[it] = in ? (sorted ? b.sorted_pm[g] : ld_pos_mass(b.bodies_in, bidx[it])) : make_float4(0, 0, 0, 0);
        alive[it] = in && pm[it].w != 0.0f;
        const uint32_t bal = __ballot_sync(0xffffffffu, alive[it]);
        wrank[it] = __popc(bal & lanemask_lt());
        if (lane == 0) s_cnt[it][w] = __popc(bal);
    }
    __syncthreads();
    // exclusive prefix over (row, warp) in slot order
    if (threadIdx.x < 32) {
        const int E = PREP_ITEMS * (PREP_THREADS / 32);  // 64 entries
        uint32_t v0 = 0, v1 = 0;
        uint32_t* flat = &s_cnt[0][0];
        if (lane < E / 2) {
            v0 = flat[2 * lane];
            v1 = flat[2 * lane + 1];
        }
        uint32_t s = v0 + v1, x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        const uint32_t ex = x - s;
        if (lane < E / 2) {
            flat[2 * lane] = ex;
            flat[2 * lane + 1] = ex + v0;
        }
    }
    __syncthreads();
    const uint32_t dead_before = b.tile_dead[tile];
    const uint32_t alive_before_tile = base - dead_before;
#pragma unroll
    for (int it = 0; it < PREP_ITEMS; ++it) {
        const uint32_t slot = it * PREP_THREADS + threadIdx.x;  // position inside the tile
        const uint32_t g = base + slot;
        if (g >= n_old) continue;
        const uint32_t arank = s_cnt[it][w] + wrank[it];
        if (alive[it]) {
            const uint32_t dst = alive_before_tile + arank;
            b.idx_out[dst] = bidx[it];
            const uint64_t key = b.prec ? morton_encode64(b.pos64_in + 4 * (size_t)bidx[it], s_mn, s_mx)
                                        : morton_encode(pm[it].x, pm[it].y, pm[it].z, s_mn, s_mx);
            b.keys_out[dst] = key;
#pragma unroll
            for (int p = 0; p < SORT_PASSES; ++p) atomicAdd(&s_hist[p * SORT_RADIX + ((key >> (8 * p)) & 0xFF)], 1u);
        } else {
            const uint32_t drank = slot - arank;
            b.idx_out[n_new + dead_before + drank] = bidx[it];
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < SORT_PASSES * SORT_RADIX; i += PREP_THREADS) {
        const uint32_t v = s_hist[i];
        if (v) atomicAdd(&b.hist[i], v);
    }
}

void launch_prepare(const StepBuffers& b, cudaStream_t s) {
    k_prep_count<<<b.prep_tiles_cap, PREP_THREADS, 0, s>>>(b);
    k_prep_scan<<<1, 1024, 0, s>>>(b);
    k_prep_scatter<<<b.prep_tiles_cap, PREP_THREADS, 0, s>>>(b);
}

// ---------------------------------------------------------------------------
// initKernel, bh_init.comp:10-27
__global__ void k_init_index(uint32_t* idx, uint32_t N, gbh_sim_values* sim, gbh_units u) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < N) idx[g] = g;
    if (g == 0) {
        sim->unit_mass = u.mass;
        sim->unit_density = u.density;
        sim->unit_len = u.len;
        sim->unit_time = u.time;
        if (u.gravitational_constant > 0.0f) {
            sim->gravitational_constant = u.gravitational_constant;
        } else {
            float gc = 6.67430e-11f * powf(u.len, -3.0f);
            gc = gc * powf(u.time, 2.0f);
            gc = gc * powf(u.mass, 1.0f);
            sim->gravitational_constant = gc;
        }
        sim->body_length_constant = 0.6203504909f * powf(u.mass / u.density, 1.0f / 3.0f) / u.len;
    }
}

void launch_init_index(uint32_t* idx, uint32_t N, gbh_sim_values* sim, const gbh_units* units, cudaStream_t s) {
    k_init_index<<<(N + 255) / 256, 256, 0, s>>>(idx, N, sim, *units);
}
