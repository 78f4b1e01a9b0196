// gvx_noalloc.cu -- a radix-sort entry point that allocates no device memory.
//
// gvx_radix_sort keeps its scratch (digit histograms, look-back words and the
// ping-pong copy of keys and values) in buffers the grid allocates on first
// use.  Callers that must not allocate -- a host that hands this library a
// fixed device-memory budget up front, a plugin whose host owns every device
// allocation, or code that already runs close to a hard memory limit -- can use
// gvx_radix_sort_noalloc instead: the same onesweep kernels (gvx_sort.cu), run
// on a scratch area that is a file-scope __device__ array of this library, so
// the call itself never calls cudaMalloc/cudaFree or any allocating routine.
//
// Limits and rules:
//  - at most GVX_NOALLOC_SORT_MAX_KEYS pairs per call (larger requests are
//    rejected with GVX_ERR_CAPACITY before anything is launched);
//  - the scratch array (about 2.4 MB) is part of the library image: every GPU
//    that loads the library holds it until the process exits;
//  - every call on a device shares the one array, so calls whose work overlaps
//    on the GPU (different streams, or different host threads without ordering)
//    race and give wrong results; order them on one stream;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <mutex>

#include "gvx_internal.cuh"

// the onesweep kernels of gvx_sort.cu
__global__ void k_sort_hist(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist);
__global__ void k_sort_bases(const uint32_t* hist, uint32_t* base);
__global__ void k_onesweep(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                           int shift, const uint32_t* base, uint32_t* lookback, uint32_t* counter, uint32_t* err);

namespace {
constexpr uint32_t kMaxKeys = GVX_NOALLOC_SORT_MAX_KEYS;
constexpr uint32_t kTile = 4096;  // keys per onesweep tile (gvx_sort.cu)
constexpr uint32_t kMaxTiles = (kMaxKeys + kTile - 1) / kTile;
constexpr size_t kHistOff = 0;                                       // 4 passes * 256 counts
constexpr size_t kBaseOff = kHistOff + 4 * 256 * 4;                  // 4 passes * 256 bases
constexpr size_t kCounterOff = kBaseOff + 4 * 256 * 4;               // 4 tile counters
constexpr size_t kErrOff = kCounterOff + 256;                        // device error word
constexpr size_t kLookbackOff = kErrOff + 256;                       // 4 passes * tiles * 256 words
constexpr size_t kKeysOff = kLookbackOff + (size_t)4 * kMaxTiles * 256 * 4;
constexpr size_t kValsOff = kKeysOff + (size_t)kMaxKeys * 4;
constexpr size_t kScratchBytes = kValsOff + (size_t)kMaxKeys * 4;
constexpr int kMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kScratchBytes];

static std::mutex s_mutex;
static unsigned char* s_scratch[kMaxDevices];

extern "C" gvx_status gvx_radix_sort_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                                             uint32_t* vals_out, uint32_t n, int bits, void* stream)
{
    if (n > kMaxKeys) {
        gvx_set_error("radix_sort_noalloc: %u pairs exceed the static scratch limit of %u", n, kMaxKeys);
        return GVX_ERR_CAPACITY;
    }
    if (bits < 1 || bits > 32) {
        gvx_set_error("radix_sort_noalloc: bits must be 1..32, got %d", bits);
        return GVX_ERR_INVALID_ARG;
    }
    if (n > 0 && (!keys_in || !vals_in || !keys_out || !vals_out)) {
        gvx_set_error("radix_sort_noalloc: null buffer");
        return GVX_ERR_INVALID_ARG;
    }
    if (n == 0) return GVX_OK;
    int dev = 0;
    GVX_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        gvx_set_error("radix_sort_noalloc: device %d", dev);
        return GVX_ERR_INVALID_ARG;
    }
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lock(s_mutex);
        if (!s_scratch[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
            if (e != cudaSuccess) return gvx_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_sort_scratch)");
            s_scratch[dev] = (unsigned char*)p;
        }
        base = s_scratch[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 1) {
        GVX_CK(cudaMemcpyAsync(keys_out, keys_in, 4, cudaMemcpyDeviceToDevice, st));
        GVX_CK(cudaMemcpyAsync(vals_out, vals_in, 4, cudaMemcpyDeviceToDevice, st));
        return GVX_OK;
    }
    const int passes = (bits + 7) / 8;
    const uint32_t tiles = (n + kTile - 1) / kTile;
    uint32_t* hist = (uint32_t*)(base + kHistOff);
    uint32_t* bases = (uint32_t*)(base + kBaseOff);
    uint32_t* counter = (uint32_t*)(base + kCounterOff);
    uint32_t* err = (uint32_t*)(base + kErrOff);
    uint32_t* lookback = (uint32_t*)(base + kLookbackOff);
    uint32_t* ktmp = (uint32_t*)(base + kKeysOff);
    uint32_t* vtmp = (uint32_t*)(base + kValsOff);

    // the previous call's contents stay in the array: clear what must start at zero
    GVX_CK(cudaMemsetAsync(hist, 0, 4 * 256 * 4, st));
    GVX_CK(cudaMemsetAsync(counter, 0, 4 * 4, st));
    GVX_CK(cudaMemsetAsync(err, 0, 4, st));
    GVX_CK(cudaMemsetAsync(lookback, 0, (size_t)passes * tiles * 256 * 4, st));
    k_sort_hist<<<tiles < 1024 ? tiles : 1024, 256, 0, st>>>(keys_in, n, passes, hist);
    k_sort_bases<<<passes, 256, 0, st>>>(hist, bases);
    // the last pass lands in the caller's output; earlier passes alternate with the scratch copy
    const uint32_t* ksrc = keys_in;
    const uint32_t* vsrc = vals_in;
    for (int p = 0; p < passes; p++) {
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        uint32_t* kdst = to_out ? keys_out : ktmp;
        uint32_t* vdst = to_out ? vals_out : vtmp;
        k_onesweep<<<tiles, 256, 0, st>>>(ksrc, vsrc, kdst, vdst, n, 8 * p, bases + p * 256,
                                          lookback + (size_t)p * tiles * 256, counter + p, err);
        ksrc = kdst;
        vsrc = vdst;
    }
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
