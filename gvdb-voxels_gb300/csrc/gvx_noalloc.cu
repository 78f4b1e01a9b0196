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
//  - the array's device address is looked up (cudaGetSymbolAddress) once per
//    device and CUDA context, by the first call made with that device current,
//    and again whenever the current context is a new one (cudaDeviceReset
//    replaces the primary context, and the array with it); make that first call
//    before any stream capture;
//  - sorting in place is allowed (keys_out may be keys_in, vals_out vals_in);
//    the two outputs must not overlap each other;
//  - a bounded look-back wait that gives up leaves a sticky flag in the array;
//    gvx_radix_sort_noalloc_status reads and clears it.
#include <cuda.h>

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
constexpr size_t kErrOff = kCounterOff + 256;                        // device error word (sticky)
constexpr size_t kLookbackOff = kErrOff + 256;                       // 4 passes * tiles * 256 words
constexpr size_t kKeysOff = kLookbackOff + (size_t)4 * kMaxTiles * 256 * 4;
constexpr size_t kValsOff = kKeysOff + (size_t)kMaxKeys * 4;
constexpr size_t kScratchBytes = kValsOff + (size_t)kMaxKeys * 4;
constexpr int kMaxDevices = 64;

typedef CUresult (*FnCtxGetCurrent)(CUcontext*);
typedef CUresult (*FnCtxGetId)(CUcontext, unsigned long long*);

struct Slot {
    unsigned char* ptr;
    unsigned long long ctx;  // id of the context the address belongs to
};
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_sort_scratch[kScratchBytes];

static std::mutex s_mutex;
static Slot s_slot[kMaxDevices];
static std::once_flag s_entry_once;
static FnCtxGetCurrent s_ctx_get_current;
static FnCtxGetId s_ctx_get_id;

// Id of the current CUDA context (0 when none is current).  libgvx links no
// libcuda, so the two driver calls are taken through the runtime's entry-point
// table; without them every call looks the address up again.
static unsigned long long current_context_id()
{
    std::call_once(s_entry_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            s_ctx_get_current = (FnCtxGetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            s_ctx_get_id = (FnCtxGetId)f;
        (void)cudaGetLastError();
    });
    if (!s_ctx_get_current || !s_ctx_get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (s_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (s_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device and context.
static gvx_status scratch_address(const char* who, unsigned char** out)
{
    int dev = 0;
    GVX_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        gvx_set_error("%s: device %d", who, dev);
        return GVX_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(s_mutex);
    unsigned long long ctx = current_context_id();
    if (s_slot[dev].ptr && ctx != 0 && s_slot[dev].ctx == ctx) {
        *out = s_slot[dev].ptr;
        return GVX_OK;
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_sort_scratch);
    if (e != cudaSuccess) return gvx_cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_sort_scratch)");
    // the lookup makes the device's primary context current when none was
    if (ctx == 0) ctx = current_context_id();
    s_slot[dev].ptr = (unsigned char*)p;
    s_slot[dev].ctx = ctx;
    *out = s_slot[dev].ptr;
    return GVX_OK;
}

static bool ranges_overlap(const void* a, const void* b, size_t bytes)
{
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return x < y + bytes && y < x + bytes;
}

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
    const size_t bytes = (size_t)n * 4;
    if (n > 0 && ranges_overlap(keys_out, vals_out, bytes)) {
        gvx_set_error("radix_sort_noalloc: keys_out and vals_out overlap");
        return GVX_ERR_INVALID_ARG;
    }
    if (n == 0) return GVX_OK;
    unsigned char* base = nullptr;
    gvx_status rc = scratch_address("radix_sort_noalloc", &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 1) {
        if (keys_out != keys_in) GVX_CK(cudaMemcpyAsync(keys_out, keys_in, 4, cudaMemcpyDeviceToDevice, st));
        if (vals_out != vals_in) GVX_CK(cudaMemcpyAsync(vals_out, vals_in, 4, cudaMemcpyDeviceToDevice, st));
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

    // the previous call's contents stay in the array: clear what must start at
    // zero (the error word is sticky until gvx_radix_sort_noalloc_status reads it)
    GVX_CK(cudaMemsetAsync(hist, 0, 4 * 256 * 4, st));
    GVX_CK(cudaMemsetAsync(counter, 0, 4 * 4, st));
    GVX_CK(cudaMemsetAsync(lookback, 0, (size_t)passes * tiles * 256 * 4, st));
    k_sort_hist<<<tiles < 1024 ? tiles : 1024, 256, 0, st>>>(keys_in, n, passes, hist);
    k_sort_bases<<<passes, 256, 0, st>>>(hist, bases);
    // the last pass lands in the caller's output; earlier passes alternate with
    // the scratch copy.  With an odd pass count the first pass writes the
    // output, so an input that overlaps an output is first copied to the
    // scratch copy: a pass's tiles must not overwrite keys other tiles still read.
    const uint32_t* ksrc = keys_in;
    const uint32_t* vsrc = vals_in;
    const bool in_place = ranges_overlap(keys_in, keys_out, bytes) || ranges_overlap(keys_in, vals_out, bytes) ||
                          ranges_overlap(vals_in, keys_out, bytes) || ranges_overlap(vals_in, vals_out, bytes);
    if (in_place && (passes & 1)) {
        GVX_CK(cudaMemcpyAsync(ktmp, keys_in, bytes, cudaMemcpyDeviceToDevice, st));
        GVX_CK(cudaMemcpyAsync(vtmp, vals_in, bytes, cudaMemcpyDeviceToDevice, st));
        ksrc = ktmp;
        vsrc = vtmp;
    }
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

extern "C" gvx_status gvx_radix_sort_noalloc_status(void* stream)
{
    unsigned char* base = nullptr;
    gvx_status rc = scratch_address("radix_sort_noalloc_status", &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* err = (uint32_t*)(base + kErrOff);
    uint32_t word = 0;
    GVX_CK(cudaMemcpyAsync(&word, err, 4, cudaMemcpyDeviceToHost, st));
    GVX_CK(cudaMemsetAsync(err, 0, 4, st));
    GVX_CK(cudaStreamSynchronize(st));
    if (word & GVX_DERR_TIMEOUT) {
        gvx_set_error("radix_sort_noalloc: a look-back wait gave up; the sorted output of that call is wrong");
        return GVX_ERR_TIMEOUT;
    }
    return GVX_OK;
}

// Test hook: one pass over the static scratch with the first tile withheld
// (the tile counter starts at 1 and tiles - 1 blocks run, so every block takes
// a tile in range), so the second tile's bounded look-back wait runs out and
// sets the sticky error word.  The partial prefix it publishes is a lower bound
// of the true one, so every scatter index stays below n.
extern "C" gvx_status gvx_test_sort_noalloc_withheld_tile(const uint32_t* keys_in, const uint32_t* vals_in,
                                                          uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                                                          void* stream)
{
    const uint32_t tiles = (n + kTile - 1) / kTile;
    if (n > kMaxKeys || tiles < 2 || !keys_in || !vals_in || !keys_out || !vals_out ||
        ranges_overlap(keys_in, keys_out, (size_t)n * 4) || ranges_overlap(vals_in, vals_out, (size_t)n * 4)) {
        gvx_set_error("test_sort_noalloc_withheld_tile: needs %u < n <= %u and separate buffers", kTile, kMaxKeys);
        return GVX_ERR_INVALID_ARG;
    }
    unsigned char* base = nullptr;
    gvx_status rc = scratch_address("test_sort_noalloc_withheld_tile", &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* hist = (uint32_t*)(base + kHistOff);
    uint32_t* bases = (uint32_t*)(base + kBaseOff);
    uint32_t* counter = (uint32_t*)(base + kCounterOff);
    uint32_t* err = (uint32_t*)(base + kErrOff);
    uint32_t* lookback = (uint32_t*)(base + kLookbackOff);
    static const uint32_t one = 1u;
    GVX_CK(cudaMemsetAsync(hist, 0, 4 * 256 * 4, st));
    GVX_CK(cudaMemsetAsync(lookback, 0, (size_t)tiles * 256 * 4, st));
    GVX_CK(cudaMemcpyAsync(counter, &one, 4, cudaMemcpyHostToDevice, st));
    k_sort_hist<<<tiles < 1024 ? tiles : 1024, 256, 0, st>>>(keys_in, n, 1, hist);
    k_sort_bases<<<1, 256, 0, st>>>(hist, bases);
    k_onesweep<<<tiles - 1, 256, 0, st>>>(keys_in, vals_in, keys_out, vals_out, n, 0, bases, lookback, counter, err);
    GVX_CK(cudaGetLastError());
    return GVX_OK;
}
