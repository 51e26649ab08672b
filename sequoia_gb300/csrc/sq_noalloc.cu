// sq_noalloc.cu -- a radix-sort entry point that allocates no memory.
//
// Who needs it: callers that must not call cudaMalloc / cudaFree themselves
// or through a library.  Examples are a host application whose memory
// pool has already reserved the GPU's memory (a framework's caching
// allocator, a game engine's arena), where a stray cudaMalloc can fail or
// fragment that pool, and latency-critical loops where cudaFree's implicit
// device synchronisation is not acceptable.  Such callers hand in their own
// input and output buffers; everything else the sort needs lives in the
// file-scope device array below.
//
// The scratch array is one fixed block of device memory (about 12.6 MB,
// sized for SQ_NOALLOC_MAX_KEYS keys).  Every GPU on which this library's
// code is loaded holds it until the process exits.  The first call on a
// device looks up the array's device address there (cudaGetSymbolAddress,
// with that device current); make that first call before any stream
// capture.  All calls share the array and it keeps the last call's
// contents, so each call clears the parts that must start at zero, and two
// calls that overlap on the GPU (on different streams, or from different
// host threads) race on it and must not be issued.
#include "sq_common.cuh"

#include <mutex>

namespace {

constexpr uint32_t kMaxKeys = SQ_NOALLOC_MAX_KEYS;
constexpr uint32_t kTileKeys = 4096;  // the smallest onesweep tile (sq_sort.cu): bounds the tile count
constexpr uint32_t kMaxTiles = (kMaxKeys + kTileKeys - 1) / kTileKeys;
// largest (passes x radix) over the supported digit widths for 32-bit keys:
// 6 bits: 6 x 64, 8 bits: 4 x 256, 10 bits: 4 x 1024
constexpr uint32_t kMaxPassRadix = 4 * 1024;
constexpr size_t kOffAltKeys = 0;
constexpr size_t kOffAltVals = kOffAltKeys + kMaxKeys;
constexpr size_t kOffHist = kOffAltVals + kMaxKeys;
constexpr size_t kOffCounters = kOffHist + kMaxPassRadix;
constexpr size_t kOffError = kOffCounters + 8;
constexpr size_t kOffLookback = kOffError + 8;
constexpr size_t kWords = kOffLookback + (size_t)kMaxTiles * kMaxPassRadix;

// The scratch.  Host code must never pass this name to a kernel: on the host
// it is only a stand-in; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t g_sort_scratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device (set up once per
// device); nullptr if the lookup fails.
uint32_t* scratch_on_current_device(int dev)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        uint32_t* ptr = nullptr;
        if (cudaGetSymbolAddress((void**)&ptr, g_sort_scratch) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_scratch_ptr[dev] = ptr;
    }
    return g_scratch_ptr[dev];
}

bool on_device(const void* p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

}  // namespace

extern "C" sq_status sq_radix_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* values_in, uint32_t n,
                                                 uint32_t key_bits, uint32_t digit_bits, uint32_t* keys_out,
                                                 uint32_t* values_out, void* stream)
{
    if (n > kMaxKeys) return SQ_ERR_TOO_LARGE;
    if (key_bits < 1 || key_bits > 32) return SQ_ERR_INVALID;
    if (digit_bits == 0) digit_bits = 8;
    if (digit_bits != 6 && digit_bits != 8 && digit_bits != 10) return SQ_ERR_INVALID;
    if (n == 0) return SQ_OK;
    if (!keys_in || !values_in || !keys_out || !values_out) return SQ_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return SQ_ERR_NO_DEVICE;
    }
    if (!on_device(keys_in, dev) || !on_device(values_in, dev) || !on_device(keys_out, dev) ||
        !on_device(values_out, dev))
        return SQ_ERR_INVALID;
    uint32_t* base = scratch_on_current_device(dev);
    if (!base) return SQ_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    const uint32_t passes = (key_bits + digit_bits - 1) / digit_bits;
    const size_t radix = (size_t)1 << digit_bits;
    const size_t tiles = (n + kTileKeys - 1) / kTileKeys;
    uint32_t* alt_k = base + kOffAltKeys;
    uint32_t* alt_v = base + kOffAltVals;
    uint32_t* hist = base + kOffHist;
    uint32_t* counters = base + kOffCounters;
    uint32_t* err = base + kOffError;
    uint32_t* lookback = base + kOffLookback;
    const size_t bytes = sizeof(uint32_t) * (size_t)n;

    // clear what must start at zero: histogram, tile counters, error word,
    // and the look-back words this call uses
    if (cudaMemsetAsync(hist, 0, sizeof(uint32_t) * (kOffLookback - kOffHist), s) != cudaSuccess ||
        cudaMemsetAsync(lookback, 0, sizeof(uint32_t) * passes * tiles * radix, s) != cudaSuccess) {
        cudaGetLastError();
        return SQ_ERR_CUDA;
    }
    // The passes alternate between two buffers and the last one lands in the
    // first buffer when the pass count is even, in the second when it is odd;
    // arrange for that to be the caller's output.
    uint32_t *ka, *va, *kb, *vb;
    if (passes % 2 == 0) {
        ka = keys_out; va = values_out; kb = alt_k; vb = alt_v;
    } else {
        ka = alt_k; va = alt_v; kb = keys_out; vb = values_out;
    }
    if (ka != keys_in && cudaMemcpyAsync(ka, keys_in, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        cudaGetLastError();
        return SQ_ERR_CUDA;
    }
    if (va != values_in && cudaMemcpyAsync(va, values_in, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        cudaGetLastError();
        return SQ_ERR_CUDA;
    }
    sqk::sort_histogram(ka, n, hist, digit_bits, passes, s);
    sqk::sort_passes(ka, va, kb, vb, n, hist, lookback, counters, digit_bits, passes, err, s);
    if (cudaGetLastError() != cudaSuccess) return SQ_ERR_CUDA;
    // wait for the sort so a device-side error (a look-back wait that ran
    // out) can be reported by this call
    uint32_t bits = 0;
    if (cudaMemcpyAsync(&bits, err, sizeof bits, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return SQ_ERR_CUDA;
    }
    return bits ? SQ_ERR_DEVICE : SQ_OK;
}
