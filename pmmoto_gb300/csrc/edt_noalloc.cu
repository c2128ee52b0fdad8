// EDT entry point that allocates no device memory.
//
// pmg_edt3d takes its ping-pong buffer from the device's stream-ordered
// memory pool.  Some callers cannot let a library allocate: a host framework
// that owns every byte of device memory through its own pool or budget (a
// plugin allocating behind its back breaks that accounting and can fail under
// the framework's memory cap), and latency-critical loops where a pool
// allocation may block, grow the pool or fail mid-run.  For them
// pmg_edt3d_noalloc uses a fixed scratch array reserved in this file instead
// of allocating; the caller still passes the input and output buffers.
//
// The arrays are file-scope __device__ variables: every GPU that loads this
// library holds them (64 MiB for the intermediate volume, 4 MiB for the
// per-line flags and the deferred voxels of the windowed envelope path) until
// the process exits.
// Host code may not use an array's name as a device address, so the first
// call on each device resolves both addresses with cudaGetSymbolAddress
// while that device is current and caches them.  The cache is not
// invalidated by cudaDeviceReset: calls after a reset of the device are not
// supported.
#include <mutex>

#include "edt_internal.cuh"

namespace pmg {

// 16 Mi float32 = 64 MiB: volumes of up to 16,777,216 voxels (e.g. 256^3).
constexpr long long kNoAllocMaxVoxels = 16LL * 1024 * 1024;

// 1 Mi int32 = 4 MiB: the first half per-line flags (an envelope pass with
// more lines runs in blocks of rows that fit; one row is at most PMG_MAX_LINE
// lines), the second half the voxels the line-pair kernels defer (about 262 K;
// beyond that a line takes the whole float envelope).
constexpr long long kNoAllocMaxFlagLines = 1LL << 20;
static_assert(kNoAllocMaxFlagLines / 2 >= PMG_MAX_LINE, "a row of lines must fit the flag half");

static __device__ __align__(256) float g_edt_noalloc_scratch[kNoAllocMaxVoxels];
static __device__ __align__(256) int g_edt_noalloc_flags[kNoAllocMaxFlagLines];

static std::mutex g_noalloc_mu;
static float *g_noalloc_ptr[64] = {nullptr};
static int *g_noalloc_flags[64] = {nullptr};

// Addresses of this device's scratch arrays (resolved once per device, with
// the device current).
static int noalloc_scratch(float **out, int **flags)
{
    int dev = 0;
    PMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("pmg_edt3d_noalloc: device index %d outside the supported range", dev);
        return PMG_ERANGE;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_edt_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("pmg_edt3d_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return PMG_ECUDA;
        }
        void *q = nullptr;
        const cudaError_t e2 = cudaGetSymbolAddress(&q, g_edt_noalloc_flags);
        if (e2 != cudaSuccess || !q) {
            set_error("pmg_edt3d_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e2));
            return PMG_ECUDA;
        }
        g_noalloc_ptr[dev] = (float *)p;
        g_noalloc_flags[dev] = (int *)q;
    }
    *out = g_noalloc_ptr[dev];
    *flags = g_noalloc_flags[dev];
    return PMG_OK;
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_edt3d_noalloc(const uint8_t *img, float *out, const int64_t shape[3],
                                 const float res[3], const pmg_axis_cfg cfg[3], int32_t num_hull,
                                 int32_t form, void *stream)
{
    if (!img || !out || !shape || !res || !cfg) {
        set_error("pmg_edt3d_noalloc: null argument");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; d++) {
        if (shape[d] <= 0) {
            set_error("pmg_edt3d_noalloc: shape[%d] = %lld must be positive", d, (long long)shape[d]);
            return PMG_EINVAL;
        }
        if (shape[d] > PMG_MAX_LINE) {
            set_error("pmg_edt3d_noalloc: shape[%d] = %lld exceeds the line limit %d", d,
                      (long long)shape[d], PMG_MAX_LINE);
            return PMG_ERANGE;
        }
    }
    const long long n = (long long)shape[0] * shape[1] * shape[2];
    if (n > kNoAllocMaxVoxels) {
        set_error("pmg_edt3d_noalloc: volume of %lld voxels exceeds the fixed scratch of %lld voxels "
                  "(64 MiB); use pmg_edt3d for larger volumes",
                  n, kNoAllocMaxVoxels);
        return PMG_ERANGE;
    }
    if (num_hull < 0 || num_hull + 1 > kMaxHull) {
        set_error("pmg_edt3d_noalloc: num_hull %d outside [0, %d]", num_hull, kMaxHull - 1);
        return PMG_ERANGE;
    }
    if (form != PMG_EDT_SQUARED && form != PMG_EDT_DIST) {
        set_error("pmg_edt3d_noalloc: form must be PMG_EDT_SQUARED or PMG_EDT_DIST");
        return PMG_EINVAL;
    }
    float *tmp = nullptr;
    int *flags = nullptr;
    PMG_TRY(noalloc_scratch(&tmp, &flags));
    // every scratch element read by the second envelope pass is written by the
    // first one, and the envelope clears the flags of each block of lines
    // before it uses them, so nothing left by an earlier call leaks through
    return edt3d_run(img, out, tmp, shape, res, cfg, num_hull, form, as_stream(stream), flags,
                     kNoAllocMaxFlagLines);
}
