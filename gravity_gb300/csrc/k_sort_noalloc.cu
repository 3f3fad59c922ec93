// k_sort_noalloc.cu — gbh_sort_pairs_noalloc: the step's radix sort for
// callers that must not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not wanted:
// a host whose device memory is owned by another allocator (a Java or game
// engine renderer that hands out only its own buffers), code that runs while
// another component holds the device's memory pool, or a hot loop that must
// never hit the allocator's locks.  It sorts (uint64 key, uint32 value) pairs
// that the caller already has on the device.
//
// Scratch: everything the onesweep sort needs beyond the caller's inputs and
// outputs (a ping-pong copy of the pairs, the digit histograms, the look-back
// words, the tile tickets and the error word) lives in one file-scope
// __device__ array below.  Every GPU that loads this library holds it, about
// 15 MB, until the process exits.  All calls share it: a call clears what must
// start at zero, and calls that overlap on the GPU (on different streams or
// threads) race on it; serialise them.
//
// Set-up, once per device, by the first call with that device current: the
// array's device address (cudaGetSymbolAddress), the sort kernels' shared
// memory limits and the multiprocessor count.  Make that first call before
// any stream capture.  Every call ends by reading the device error word and
// synchronising its stream, so no call can be captured in a CUDA graph.
// The cached address belongs to the device's current context: after a
// cudaDeviceReset of that device the library must not be used again in the
// same process.
#include <cstring>
#include <mutex>

#include "gbh_common.cuh"

void sort_setup();  // k_sort.cu

#define NOALLOC_MAX_PAIRS (1u << 20)
#define NOALLOC_TILES ((NOALLOC_MAX_PAIRS + SORT_TILE - 1) / SORT_TILE)
#define NOALLOC_MAX_DEVICES 64

struct NoAllocScratch {
    unsigned long long keys_tmp[NOALLOC_MAX_PAIRS];
    uint32_t vals_tmp[NOALLOC_MAX_PAIRS];
    uint32_t hist[SORT_PASSES * SORT_RADIX];
    uint32_t bucket_base[SORT_PASSES * SORT_RADIX];
    uint32_t lookback[SORT_PASSES * NOALLOC_TILES * SORT_RADIX];
    DevState st;
};

static __device__ __align__(256) NoAllocScratch g_sort_scratch;

struct NoAllocDevice {
    NoAllocScratch* scratch = nullptr;  // device address of g_sort_scratch
    uint32_t num_sms = 0;
};
static NoAllocDevice g_dev[NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;

// The set-up of the current device, done once: the scratch's device address,
// the sort kernels' attributes and the multiprocessor count.
static const NoAllocDevice* setup_current_device(int* status) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        *status = GBH_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    NoAllocDevice& d = g_dev[dev];
    if (!d.scratch) {
        void* p = nullptr;
        int sms = 0;
        if (cudaGetSymbolAddress(&p, g_sort_scratch) != cudaSuccess || !p ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            *status = GBH_ERR_CUDA;
            return nullptr;
        }
        sort_setup();
        d.num_sms = (uint32_t)sms;
        d.scratch = static_cast<NoAllocScratch*>(p);
    }
    *status = GBH_OK;
    return &d;
}

extern "C" int gbh_sort_pairs_noalloc(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                                      uint32_t* vals_out, uint32_t n, void* stream) {
    if (n > NOALLOC_MAX_PAIRS) return GBH_ERR_INVALID;
    if (n == 0) return GBH_OK;
    if (!keys_in || !vals_in || !keys_out || !vals_out) return GBH_ERR_INVALID;
    // outputs either are the inputs (sorted in place) or do not overlap them
    const char *ki = (const char*)keys_in, *ko = (const char*)keys_out;
    const char *vi = (const char*)vals_in, *vo = (const char*)vals_out;
    if ((ko != ki && ko < ki + (size_t)n * 8 && ki < ko + (size_t)n * 8) ||
        (vo != vi && vo < vi + (size_t)n * 4 && vi < vo + (size_t)n * 4))
        return GBH_ERR_INVALID;
    int status = GBH_OK;
    const NoAllocDevice* dv = setup_current_device(&status);
    if (!dv) return status;
    NoAllocScratch* s = dv->scratch;
    // a launch error pending from earlier work of this thread is cleared here,
    // so that the check after the launches below reports this call's own
    (void)cudaGetLastError();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the sort runs in place in the caller's output buffers
    if (keys_out != keys_in &&
        cudaMemcpyAsync(keys_out, keys_in, (size_t)n * 8, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GBH_ERR_CUDA;
    if (vals_out != vals_in &&
        cudaMemcpyAsync(vals_out, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return GBH_ERR_CUDA;
    // clear what the previous call left: histograms, tickets, error word, look-back words
    if (cudaMemsetAsync(s->hist, 0, sizeof(s->hist), st) != cudaSuccess) return GBH_ERR_CUDA;
    if (cudaMemsetAsync(&s->st, 0, sizeof(s->st), st) != cudaSuccess) return GBH_ERR_CUDA;
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    for (uint32_t p = 0; p < SORT_PASSES; ++p)
        if (cudaMemsetAsync(s->lookback + (size_t)p * NOALLOC_TILES * SORT_RADIX, 0, (size_t)tiles * SORT_RADIX * 4,
                            st) != cudaSuccess)
            return GBH_ERR_CUDA;
    launch_sort_hist(keys_out, n, s->hist, &s->st, dv->num_sms, st);
    StepBuffers b;
    memset(&b, 0, sizeof(b));
    b.keys_in = keys_out;
    b.idx_in = vals_out;
    b.keys_out = reinterpret_cast<uint64_t*>(s->keys_tmp);
    b.idx_out = s->vals_tmp;
    b.st = &s->st;
    b.hist = s->hist;
    b.bucket_base = s->bucket_base;
    b.lookback = s->lookback;
    b.N = n;
    b.sort_tiles_cap = NOALLOC_TILES;
    b.num_sms = dv->num_sms;
    launch_sort(b, st);
    if (cudaGetLastError() != cudaSuccess) return GBH_ERR_CUDA;
    // report errors raised on the device (bounded look-back waits)
    uint32_t err = 0;
    if (cudaMemcpyAsync(&err, &s->st.error_word, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return GBH_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return GBH_ERR_CUDA;
    return err ? GBH_ERR_DEVICE : GBH_OK;
}
