// pt_static_table.cu - a bucket-table builder that allocates no device memory.
//
// Some callers cannot call cudaMalloc on their path: a host that hands this library
// device buffers from its own memory pool and forbids other allocations (the pool
// owns the whole budget), or a loop that keeps other streams busy, where cudaMalloc
// and cudaFree would synchronise the device and stall that unrelated work.  For
// them, pt_bucket_table_static builds the same table as the simulation's workplace
// and errand tables (person ids grouped by key, ascending within each key, with
// offsets) using only scratch space compiled into the library: the array below.
//
// The array is part of the library's device code.  With lazy module loading (the
// CUDA default) its memory is committed when the module first loads on a device: at
// the first call, or at the first kernel any entry point of the library launches
// there.  From then on that GPU holds it until the process exits.  A caller whose
// pool claims the whole device budget should make one call at initialisation,
// before carving the pool.  All calls share the array and it keeps the last call's
// contents, so two calls that overlap on the GPU (on different streams, or from
// different host threads) race and corrupt each other's tables: serialise them.
// The device address is looked up once per device and kept; the library must not be
// used across a cudaDeviceReset.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>

#include "pandemic_gb300.h"
#include "pt_kernels.h"

namespace {

constexpr int kMaxEntries = PT_STATIC_TABLE_MAX_ENTRIES;
constexpr int kMaxBuckets = PT_STATIC_TABLE_MAX_BUCKETS;
constexpr int kTile = 4096;                                      // radix and scan tile
static_assert(kTile == ptk::kRadixTileEntries && kTile == ptk::kScanTileEntries,
              "the scratch layout sizes the look-back words by the kernels' tile sizes");
constexpr int kRadixTiles = (kMaxEntries + kTile - 1) / kTile;
constexpr int kScanTiles = (kMaxBuckets + 1 + kTile - 1) / kTile + 4;

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Scratch layout (byte offsets into the static array)
constexpr size_t kOffCounts = 0;                                                  // int[kMaxBuckets], zero between calls
constexpr size_t kOffK0 = kOffCounts + align256((size_t)kMaxBuckets * 4);         // radix ping-pong buffers
constexpr size_t kOffV0 = kOffK0 + align256((size_t)kMaxEntries * 4);
constexpr size_t kOffK1 = kOffV0 + align256((size_t)kMaxEntries * 4);
constexpr size_t kOffV1 = kOffK1 + align256((size_t)kMaxEntries * 4);
constexpr size_t kOffStatus = kOffV1 + align256((size_t)kMaxEntries * 4);         // radix look-back words
constexpr size_t kOffScanTiles = kOffStatus + align256((size_t)kRadixTiles * 256 * 8);  // scan look-back words + control
constexpr size_t kOffRadixCtl = kOffScanTiles + align256((size_t)(kScanTiles + 4) * 8);
constexpr size_t kOffDigitHist = kOffRadixCtl + 256;
constexpr size_t kOffDigitBase = kOffDigitHist + align256(4 * 256 * 4);
constexpr size_t kOffError = kOffDigitBase + align256(4 * 256 * 4);
constexpr size_t kScratchBytes = kOffError + 256;

static __device__ __align__(256) unsigned char g_table_scratch[kScratchBytes];

// Device address of g_table_scratch for each device, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

// Counts keys with a bounds check: a key outside [0, buckets) sets the error word
// and is skipped, so a bad input cannot write outside the scratch counts.
__global__ void k_count_keys_checked(const int32_t *keys, int n, int buckets, int32_t *count, int *error)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int k = keys[i];
        if (k < 0 || k >= buckets) {
            atomicExch(error, 1);
            continue;
        }
        atomicAdd(&count[k], 1);
    }
}

}  // namespace

extern "C" pt_status pt_bucket_table_static(const int32_t *keys, int n, int buckets, int32_t *offsets,
                                            int32_t *table, void *cuda_stream)
{
    if (n < 0 || buckets < 1 || (n > 0 && (!keys || !table)) || !offsets) return PT_ERR_ARG;
    if (n > kMaxEntries || buckets > kMaxBuckets) return PT_ERR_ARG;  // beyond the compiled-in scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PT_ERR_CUDA;
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_ptr[dev]) {
            // The array's name is a host-side stand-in; the kernels need the device
            // address, which is fixed per device once the module is loaded.
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_table_scratch) != cudaSuccess || !p) return PT_ERR_CUDA;
            g_scratch_ptr[dev] = (unsigned char *)p;
        }
        base = g_scratch_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)cuda_stream;
    int32_t *counts = (int32_t *)(base + kOffCounts);
    unsigned long long *scan_tiles = (unsigned long long *)(base + kOffScanTiles);
    int *scan_ctl = (int *)(scan_tiles + kScanTiles);
    int *error = (int *)(base + kOffError);
    // what must start at zero: counts, look-back control words, digit histograms, error
    if (cudaMemsetAsync(counts, 0, (size_t)buckets * 4, s) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaMemsetAsync(scan_tiles, 0, (size_t)(kScanTiles + 4) * 8, s) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaMemsetAsync(base + kOffRadixCtl, 0, 256, s) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaMemsetAsync(base + kOffStatus, 0, (size_t)kRadixTiles * 256 * 8, s) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaMemsetAsync(base + kOffDigitHist, 0, 4 * 256 * 4, s) != cudaSuccess) return PT_ERR_CUDA;
    if (cudaMemsetAsync(error, 0, sizeof(int), s) != cudaSuccess) return PT_ERR_CUDA;
    int herr = 0;
    if (n > 0) {
        const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
        k_count_keys_checked<<<blocks, 256, 0, s>>>(keys, n, buckets, counts, error);
        if (cudaGetLastError() != cudaSuccess) return PT_ERR_CUDA;
        if (cudaMemcpyAsync(&herr, error, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return PT_ERR_CUDA;
        if (herr) return PT_ERR_ARG;  // a key outside [0, buckets)
    }
    ptk::RadixArgs r;
    r.keys = (const uint32_t *)keys;
    r.E = n;
    r.buckets = buckets;
    r.N = n;
    r.person_mode = 0;  // entry i is item i
    r.k0 = (uint32_t *)(base + kOffK0);
    r.v0 = (uint32_t *)(base + kOffV0);
    r.k1 = (uint32_t *)(base + kOffK1);
    r.v1 = (uint32_t *)(base + kOffV1);
    r.out = (uint32_t *)table;
    r.digit_base = (const int *)(base + kOffDigitBase);
    r.status = (unsigned long long *)(base + kOffStatus);
    r.ctl = (int *)(base + kOffRadixCtl);
    r.error = error;
    r.skip = nullptr;
    if (n == 0) {
        // an empty table: every offset is zero
        if (cudaMemsetAsync(offsets, 0, ((size_t)buckets + 1) * 4, s) != cudaSuccess) return PT_ERR_CUDA;
        return cudaStreamSynchronize(s) == cudaSuccess ? PT_OK : PT_ERR_CUDA;
    }
    if (ptk::launch_bucket_table(r, counts, false, offsets, scan_tiles, scan_ctl, (int *)(base + kOffDigitHist), s) !=
        cudaSuccess)
        return PT_ERR_CUDA;
    if (cudaMemcpyAsync(&herr, error, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PT_ERR_CUDA;
    return herr ? PT_ERR_TIMEOUT : PT_OK;
}
