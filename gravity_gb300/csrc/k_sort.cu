// k_sort.cu — stable LSD radix sort of (63-bit Morton key, u32 body index).
//
// Replaces radixSort (src/main/java/com/grumbo/simulation/BarnesHut.java:358-448)
// and its four kernels (SH/compute/radix/bh_radix.comp:12-166): 16 passes of
// 4-bit digits, each pass histogram -> per-bucket scan -> global scan ->
// scatter with an O(256) serial rank loop.  Any stable LSD sort of the same
// keys yields the same permutation, so this is a onesweep sort (Adinets &
// Merrill 2022): 8 passes of 8-bit digits, one kernel per pass.
//   * The eight digit histograms are accumulated by the encode pass
//     (k_prep_scatter) and scanned here once (k_sort_scan).
//   * Each pass kernel takes a tile ticket, ranks its keys per warp (digit
//     peers from one ballot per digit bit, ranks reserved with shared-memory
//     atomics in item order), publishes the tile's digit counts, resolves its global digit
//     offsets with a decoupled look-back (bounded spin, error word on
//     timeout), stages keys digit-ordered in shared memory and writes them out
//     with coalesced runs.
#include "gbh_common.cuh"

#define LB_FLAG_AGG 0x40000000u
#define LB_FLAG_INC 0x80000000u
#define LB_COUNT_MASK 0x3FFFFFFFu
#define LB_SPIN_LIMIT (1u << 22)
#ifndef LB_WINDOW
#define LB_WINDOW 4
#endif

__global__ void k_sort_scan(StepBuffers b) {
    // one block per pass: exclusive scan of the 256 digit counts
    const uint32_t p = blockIdx.x;
    const uint32_t d = threadIdx.x;
    const uint32_t v = b.hist[p * SORT_RADIX + d];
    __shared__ uint32_t s_w[SORT_RADIX / 32];
    const uint32_t lane = lane_id(), w = d >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    uint32_t off = 0;
    for (uint32_t i = 0; i < w; ++i) off += s_w[i];
    b.bucket_base[p * SORT_RADIX + d] = off + x - v;
}

struct SortSmem {
    uint32_t warp_hist[SORT_THREADS / 32][SORT_RADIX + 1];  // +1: sentinel bucket of out-of-range items
#ifdef SORT_RANK_MATCH
    uint32_t match[SORT_THREADS / 32][SORT_RADIX + 1];       // per-warp digit masks of the ranking
#endif
    uint32_t block_excl[SORT_RADIX + 1];
    uint32_t delta[SORT_RADIX];
    uint32_t warp_tot[SORT_THREADS / 32];
    uint32_t tile;
    unsigned long long keys[SORT_TILE];
    uint32_t vals[SORT_TILE];
};

// Warp-level stable ranking of the items, item rounds in slot order: lanes
// with the same digit from one ballot per digit bit (BITS = 9 in a partial
// tile, whose out-of-range slots carry the sentinel digit 256); the digit's
// leader reserves the group's ranks with a shared-memory atomic.  A warp's
// shared memory atomics take effect in program order, so items stay in slot
// order.
template <uint32_t SHIFT, int BITS>
__device__ __forceinline__ void rank_items(const uint64_t (&key)[SORT_ITEMS], uint32_t (&rank)[SORT_ITEMS],
                                           uint32_t* warp_hist, uint32_t lane, uint32_t seg, uint32_t n) {
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        uint32_t dig = (uint32_t)(key[i] >> SHIFT) & 0xFFu;
        if (BITS > 8 && seg + i * 32 + lane >= n) dig = SORT_RADIX;
        uint32_t peers = 0xffffffffu;
#pragma unroll
        for (int bit = 0; bit < BITS; ++bit) {
            const bool on = (dig >> bit) & 1u;
            const uint32_t m = __ballot_sync(0xffffffffu, on);
            peers &= on ? m : ~m;
        }
        const uint32_t leader = __ffs(peers) - 1;
        const uint32_t before = __popc(peers & lanemask_lt());
        uint32_t prev = 0;
        if (lane == leader) prev = atomicAdd(&warp_hist[dig], (uint32_t)__popc(peers));
        rank[i] = __shfl_sync(0xffffffffu, prev, leader) + before;
    }
}

#ifdef SORT_RANK_MATCH
// The same stable ranking with the peers found in shared memory: each lane
// ORs its bit into its digit's word of a per-warp mask table, reads the word
// back (the lanes with its digit), and the digit's lowest lane reserves the
// group's ranks and clears the word.  One shared atomic per item instead of
// eight ballots.
template <uint32_t SHIFT, int BITS>
__device__ __forceinline__ void rank_items_match(const uint64_t (&key)[SORT_ITEMS], uint32_t (&rank)[SORT_ITEMS],
                                                 uint32_t* warp_hist, uint32_t* match, uint32_t lane, uint32_t seg,
                                                 uint32_t n) {
    const uint32_t bit = 1u << lane;
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        uint32_t dig = (uint32_t)(key[i] >> SHIFT) & 0xFFu;
        if (BITS > 8 && seg + i * 32 + lane >= n) dig = SORT_RADIX;
        atomicOr(&match[dig], bit);
        __syncwarp();
        const uint32_t peers = match[dig];
        const uint32_t leader = __ffs(peers) - 1;
        const uint32_t before = __popc(peers & (bit - 1u));
        uint32_t prev = 0;
        __syncwarp();
        if (lane == leader) {
            prev = atomicAdd(&warp_hist[dig], (uint32_t)__popc(peers));
            match[dig] = 0u;
        }
        rank[i] = __shfl_sync(0xffffffffu, prev, leader) + before;
    }
}
#endif

// One kernel instance per pass: the digit's bit offset is a constant.
template <uint32_t PASS>
__global__ __launch_bounds__(SORT_THREADS, 3) void k_sort_pass(StepBuffers b, const uint64_t* __restrict__ kin,
                                                               const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                                               uint32_t* __restrict__ vout) {
    constexpr uint32_t pass = PASS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem& S = *reinterpret_cast<SortSmem*>(smem_raw);
    const uint32_t n = b.st->n_new;
    constexpr uint32_t shift = SORT_BITS * PASS;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    if (threadIdx.x == 0) S.tile = atomicAdd(&b.st->sort_tiles[pass], 1u);
    for (uint32_t i = threadIdx.x; i < (SORT_THREADS / 32) * (SORT_RADIX + 1); i += SORT_THREADS) {
        (&S.warp_hist[0][0])[i] = 0;
#ifdef SORT_RANK_MATCH
        (&S.match[0][0])[i] = 0;
#endif
    }
    __syncthreads();
    const uint32_t tile = S.tile;
    const uint32_t base = tile * SORT_TILE;
    if (base >= n) return;
    uint32_t* lb = b.lookback + ((size_t)pass * b.sort_tiles_cap) * SORT_RADIX;

    // load: warp w owns slots [base + w*32*ITEMS, +32*ITEMS), item i of lane l at +i*32+l
    const uint32_t seg = base + w * 32 * SORT_ITEMS;
    const bool full = base + SORT_TILE <= n;  // uniform over the block
    uint64_t key[SORT_ITEMS];
    uint32_t val[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
    if (full) {
#pragma unroll
        for (int i = 0; i < SORT_ITEMS; ++i) {
            key[i] = kin[seg + i * 32 + lane];
            val[i] = vin[seg + i * 32 + lane];
        }
#ifdef SORT_RANK_MATCH
        rank_items_match<shift, 8>(key, rank, S.warp_hist[w], S.match[w], lane, seg, n);
#else
        rank_items<shift, 8>(key, rank, S.warp_hist[w], lane, seg, n);
#endif
    } else {
#pragma unroll
        for (int i = 0; i < SORT_ITEMS; ++i) {
            const uint32_t pos = seg + i * 32 + lane;
            if (pos < n) {
                key[i] = kin[pos];
                val[i] = vin[pos];
            } else {
                key[i] = ~0ull;
                val[i] = 0;
            }
        }
#ifdef SORT_RANK_MATCH
        rank_items_match<shift, 9>(key, rank, S.warp_hist[w], S.match[w], lane, seg, n);
#else
        rank_items<shift, 9>(key, rank, S.warp_hist[w], lane, seg, n);
#endif
    }
    __syncthreads();
    // thread d: exclusive prefix of digit d over warps, tile total
    const uint32_t d = threadIdx.x;
    uint32_t total = 0;
#pragma unroll
    for (int ww = 0; ww < SORT_THREADS / 32; ++ww) {
        const uint32_t c = S.warp_hist[ww][d];
        S.warp_hist[ww][d] = total;
        total += c;
    }
    // publish this tile's count for digit d (inclusive when it is the first tile)
    volatile uint32_t* my = lb + (size_t)tile * SORT_RADIX + d;
    if (tile == 0) {
        *my = LB_FLAG_INC | total;
    } else {
        *my = LB_FLAG_AGG | total;
    }
    // block exclusive scan of totals over digits -> block_excl
    {
        uint32_t x = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) S.warp_tot[w] = x;
        __syncthreads();
        uint32_t off = 0;
        for (uint32_t i = 0; i < w; ++i) off += S.warp_tot[i];
        S.block_excl[d] = off + x - total;
        if (d == 0) S.block_excl[SORT_RADIX] = 0;
    }
    __syncthreads();
    // stage digit-ordered in shared memory (tile-local offsets only), before
    // the look-back: the items leave the registers, and the predecessors
    // have longer to publish their inclusive counts
#pragma unroll
    for (int i = 0; i < SORT_ITEMS; ++i) {
        const uint32_t pos = seg + i * 32 + lane;
        if (pos < n) {
            const uint32_t dg = (uint32_t)(key[i] >> shift) & 0xFFu;
            const uint32_t local = S.block_excl[dg] + S.warp_hist[w][dg] + rank[i];
            S.keys[local] = key[i];
            S.vals[local] = val[i];
        }
    }
    // decoupled look-back for digit d, LB_WINDOW predecessors per round
    // trip; tile 0 always publishes an inclusive count, so the walk ends
    // there at the latest
    uint32_t prefix = 0;
    if (tile > 0) {
        int32_t j = (int32_t)tile - 1;
        uint32_t spins = 0;
        while (true) {
            uint32_t v[LB_WINDOW];
#pragma unroll
            for (int k = 0; k < LB_WINDOW; ++k)
                v[k] = (j - k >= 0) ? *(volatile uint32_t*)(lb + (size_t)(j - k) * SORT_RADIX + d) : LB_FLAG_INC;
            // aggregates add and continue, an inclusive count adds and ends
            // the walk, a word not yet published ends the round
            uint32_t add = 0, used = 0, state = 0;  // state 1: inclusive found, 2: not yet published
#pragma unroll
            for (int k = 0; k < LB_WINDOW; ++k) {
                if (state == 0) {
                    const uint32_t xv = v[k];
                    if (xv & LB_FLAG_INC) {
                        add += xv & LB_COUNT_MASK;
                        state = 1;
                    } else if (xv & LB_FLAG_AGG) {
                        add += xv & LB_COUNT_MASK;
                        ++used;
                    } else {
                        state = 2;
                    }
                }
            }
            prefix += add;
            if (state == 1) break;
            j -= (int32_t)used;
            if (used == 0) {
                if (++spins > LB_SPIN_LIMIT) {
                    set_error(b.st, GBH_DEVERR_SORT_LOOKBACK);
                    break;
                }
                __nanosleep(20);
            }
        }
        *my = LB_FLAG_INC | (prefix + total);
    }
    S.delta[d] = b.bucket_base[pass * SORT_RADIX + d] + prefix - S.block_excl[d];
    __syncthreads();
    const uint32_t valid = min((uint32_t)SORT_TILE, n - base);
    bool bad = false;
    for (uint32_t j = threadIdx.x; j < valid; j += SORT_THREADS) {
        const uint64_t k = S.keys[j];
        const uint32_t dst = S.delta[(uint32_t)(k >> shift) & 0xFFu] + j;
        if (dst < n) {  // holds whenever the digit histograms describe these keys
            kout[dst] = k;
            vout[dst] = S.vals[j];
        } else {
            bad = true;
        }
    }
    if (bad) set_error(b.st, GBH_DEVERR_SORT_LOOKBACK);
}

// The eight digit histograms of `n` keys (for a sort whose keys were not
// written by the step's encode pass) and the live count the passes read.
__global__ void k_sort_hist(const uint64_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                            DevState* __restrict__ st) {
    __shared__ uint32_t h[SORT_PASSES * SORT_RADIX];
    for (uint32_t i = threadIdx.x; i < SORT_PASSES * SORT_RADIX; i += blockDim.x) h[i] = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->n_new = n;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < SORT_PASSES; ++p) atomicAdd(&h[p * SORT_RADIX + ((k >> (8 * p)) & 0xFF)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < SORT_PASSES * SORT_RADIX; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

void launch_sort_hist(const uint64_t* keys, uint32_t n, uint32_t* hist, DevState* st, uint32_t num_sms,
                      cudaStream_t s) {
    const uint32_t blocks = min((n + 255) / 256, num_sms * 4u);
    k_sort_hist<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(keys, n, hist, st);
}

void sort_setup() {
    cudaFuncSetAttribute(k_sort_pass<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
    cudaFuncSetAttribute(k_sort_pass<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SortSmem));
}

void launch_sort(const StepBuffers& b, cudaStream_t s) {
    const size_t smem = sizeof(SortSmem);
    k_sort_scan<<<SORT_PASSES, SORT_RADIX, 0, s>>>(b);
    // keys/index of the live bodies are in the *_in buffers (the compaction
    // swap already happened); 8 ping-pong passes through *_out end there again
    const uint64_t* kin = b.keys_in;
    const uint32_t* vin = b.idx_in;
    uint64_t* kt = b.keys_out;
    uint32_t* vt = b.idx_out;
    static_assert(SORT_PASSES == 8, "one kernel instance per pass");
    void (*const kernels[SORT_PASSES])(StepBuffers, const uint64_t*, const uint32_t*, uint64_t*, uint32_t*) = {
        k_sort_pass<0>, k_sort_pass<1>, k_sort_pass<2>, k_sort_pass<3>,
        k_sort_pass<4>, k_sort_pass<5>, k_sort_pass<6>, k_sort_pass<7>};
    for (uint32_t p = 0; p < SORT_PASSES; ++p) {
        kernels[p]<<<b.sort_tiles_cap, SORT_THREADS, smem, s>>>(b, kin, vin, kt, vt);
        const uint64_t* nk = kt;
        const uint32_t* nv = vt;
        kt = const_cast<uint64_t*>(kin);
        vt = const_cast<uint32_t*>(vin);
        kin = nk;
        vin = nv;
    }
}
