// Runtime support: error strings, stream-ordered scratch memory, version.
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "pmg_common.cuh"

namespace pmg {

static thread_local char g_err[1024] = {0};

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

// The first scratch request on a device raises the release threshold of its
// default memory pool, so freed scratch stays mapped and later requests of
// the same size are served without new allocations.
static std::mutex g_pool_mu;
static bool g_pool_ready[64] = {false};

static int ensure_pool()
{
    int dev = 0;
    PMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
        return PMG_OK;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (g_pool_ready[dev])
        return PMG_OK;
    cudaMemPool_t pool;
    PMG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t thr = UINT64_MAX;
    PMG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    g_pool_ready[dev] = true;
    return PMG_OK;
}

int scratch_alloc(void **p, size_t bytes, cudaStream_t st)
{
    PMG_TRY(ensure_pool());
    if (bytes == 0)
        bytes = 256;
    PMG_CUDA(cudaMallocAsync(p, bytes, st));
    return PMG_OK;
}

int scratch_free(void *p, cudaStream_t st)
{
    if (p)
        PMG_CUDA(cudaFreeAsync(p, st));
    return PMG_OK;
}

} // namespace pmg

extern "C" int pmg_last_error(char *buf, size_t len)
{
    if (!buf || len == 0)
        return PMG_EINVAL;
    strncpy(buf, pmg::g_err, len - 1);
    buf[len - 1] = '\0';
    return PMG_OK;
}

extern "C" const char *pmg_version(void)
{
    return "pmmoto_gb300 0.1 (sm_103a)";
}
