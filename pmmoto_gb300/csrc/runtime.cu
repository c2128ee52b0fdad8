// Runtime support: error strings, stream-ordered scratch memory, version.
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

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

// Scratch comes from a memory pool the library creates on each device (the
// device's default pool, which other code in the process may use, is left
// as it is).  Its release threshold is unlimited, so freed scratch stays
// mapped and later requests of the same size are served without new
// allocations from the driver.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[64] = {nullptr};
static std::atomic<long long> g_scratch_allocs{0};

static int library_pool(cudaMemPool_t *out)
{
    int dev = 0;
    PMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("scratch: device index %d outside the supported range", dev);
        return PMG_ERANGE;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        PMG_CUDA(cudaMemPoolCreate(&pool, &props));
        uint64_t thr = UINT64_MAX;
        PMG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
        g_pool[dev] = pool;
    }
    *out = g_pool[dev];
    return PMG_OK;
}

int scratch_alloc(void **p, size_t bytes, cudaStream_t st)
{
    cudaMemPool_t pool = nullptr;
    PMG_TRY(library_pool(&pool));
    if (bytes == 0)
        bytes = 256;
    g_scratch_allocs.fetch_add(1);
    PMG_CUDA(cudaMallocFromPoolAsync(p, bytes, pool, st));
    return PMG_OK;
}

int scratch_free(void *p, cudaStream_t st)
{
    if (p)
        PMG_CUDA(cudaFreeAsync(p, st));
    return PMG_OK;
}

// ---- tunable launch parameters ------------------------------------------------
struct TuneSpec {
    const char *name;
    int def, lo, hi;
};
static const TuneSpec g_tune_spec[kTuneKnobs] = {
    {"edt.pair_seg", 256, 32, 8192},    // positions per thread of the strided line-pair pass
    {"edt.pair_ctas", 32, 1, 256},      // CTAs per SM of that pass (grid cap)
    {"edt.rows_ctas", 16, 1, 256},      // CTAs per SM of the contiguous line-pair pass
    {"cc.cross_fused", 0, 0, 1},        // block labelling: one fused cross-tile pass (1) or two (0)
    {"edt.path", 0, 0, 2},              // envelope passes: windowed (0), exact stream (1), float envelope (2)
    {"edt.fallback", 96, 0, 8193},      // probe samples (of 8192) from which a strided windowed pass goes to the envelope
    {"edt.fallback_rows", 2048, 0, 8193}, // the same for the contiguous (row) pass
    {"edt.narrow", 64, 0, 8193},        // probe samples (of 8192) below which a strided pass takes the +-8 window
    {"edt.narrow_rows", 32, 0, 8193},   // the same for the contiguous (row) pass
    {"cc.seam_batched", 1, 0, 1},       // periodic merge: all features' seams in one sort (1) or one by one (0)
    {"edt.wide", 1024, 0, 8193},        // probe samples (of 8192) below which a strided pass takes the +-24 window
};
static std::atomic<int> g_tune[kTuneKnobs] = {{256}, {32}, {16}, {0}, {0}, {96}, {2048}, {64}, {32}, {1}, {1024}};

int tune_value(int knob) { return knob >= 0 && knob < kTuneKnobs ? g_tune[knob].load() : 0; }

static int tune_index(const char *name)
{
    for (int i = 0; name && i < kTuneKnobs; i++)
        if (strcmp(name, g_tune_spec[i].name) == 0)
            return i;
    return -1;
}

static std::atomic<long long> g_launches{0};
static std::atomic<int> g_prof_on{0};
struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
    double bytes;
};
static std::mutex g_prof_mu;
static std::vector<ProfRec> g_prof;
struct ProfTot {
    double ms = 0, bytes = 0;
    long long n = 0;
};
static std::map<std::string, ProfTot> g_prof_tot;

// Units processed by kernels whose amount of work is decided on the device
// (a range computed by an earlier kernel): each launch adds its count to a
// device counter, and the profile converts the total to bytes.
__device__ unsigned long long g_units[kUnitSlots];
struct UnitInfo {
    const char *name = nullptr;
    double bytes_per_unit = 0.0;
};
static UnitInfo g_unit_info[kUnitSlots];

unsigned long long *prof_units(int id)
{
    unsigned long long *p = nullptr;
    if (id < 0 || id >= kUnitSlots || cudaGetSymbolAddress((void **)&p, g_units) != cudaSuccess)
        return nullptr;
    return p + id;
}

__global__ void k_set_int2(int *p, int a, int b)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        p[0] = a;
        p[1] = b;
    }
}

int prof_begin(const char *name, cudaStream_t st)
{
    g_launches.fetch_add(1);
    if (!g_prof_on.load())
        return -1;
    ProfRec r{name, nullptr, nullptr, 0.0};
    if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess)
        return -1;
    cudaEventRecord(r.a, st);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof.push_back(r);
    return (int)g_prof.size() - 1;
}

void prof_end(int slot, double bytes, cudaStream_t st)
{
    if (slot < 0)
        return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (slot >= (int)g_prof.size())
        return;
    g_prof[(size_t)slot].bytes = bytes;
    cudaEventRecord(g_prof[(size_t)slot].b, st);
}

void prof_end_units(int slot, int id, double bytes_per_unit, cudaStream_t st)
{
    if (slot < 0)
        return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (slot >= (int)g_prof.size())
        return;
    if (id >= 0 && id < kUnitSlots) {
        g_unit_info[id].name = g_prof[(size_t)slot].name;
        g_unit_info[id].bytes_per_unit = bytes_per_unit;
    }
    g_prof[(size_t)slot].bytes = 0.0;
    cudaEventRecord(g_prof[(size_t)slot].b, st);
}

static void prof_resolve()
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto &r : g_prof) {
        float ms = 0.0f;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            ProfTot &t = g_prof_tot[r.name];
            t.ms += ms;
            t.bytes += r.bytes;
            t.n += 1;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    g_prof.clear();
}

} // namespace pmg

extern "C" long long pmg_launch_count(void) { return pmg::g_launches.load(); }

extern "C" long long pmg_scratch_alloc_count(void) { return pmg::g_scratch_allocs.load(); }

extern "C" int pmg_prof_enable(int32_t on)
{
    pmg::prof_resolve();
    pmg::g_prof_on.store(on ? 1 : 0);
    return PMG_OK;
}

extern "C" int pmg_prof_reset(void)
{
    pmg::prof_resolve();
    std::lock_guard<std::mutex> lk(pmg::g_prof_mu);
    pmg::g_prof_tot.clear();
    unsigned long long *u = pmg::prof_units(0);
    if (u && cudaMemset(u, 0, sizeof(unsigned long long) * pmg::kUnitSlots) != cudaSuccess) {
        pmg::set_error("pmg_prof_reset: clearing the unit counters failed");
        return PMG_ECUDA;
    }
    return PMG_OK;
}

extern "C" int pmg_prof_read(char *names, size_t names_len, double *ms, double *bytes,
                             long long *launches, int32_t cap, int32_t *count)
{
    if (!names || !ms || !bytes || !launches || !count || cap < 0) {
        pmg::set_error("pmg_prof_read: null argument");
        return PMG_EINVAL;
    }
    pmg::prof_resolve();
    std::lock_guard<std::mutex> lk(pmg::g_prof_mu);
    {
        // bytes of the kernels that count their own units
        unsigned long long units[pmg::kUnitSlots] = {};
        unsigned long long *u = pmg::prof_units(0);
        if (u && cudaMemcpy(units, u, sizeof(units), cudaMemcpyDeviceToHost) == cudaSuccess)
            for (int i = 0; i < pmg::kUnitSlots; i++) {
                const pmg::UnitInfo &ui = pmg::g_unit_info[i];
                auto it = ui.name ? pmg::g_prof_tot.find(ui.name) : pmg::g_prof_tot.end();
                if (it != pmg::g_prof_tot.end())
                    it->second.bytes = (double)units[i] * ui.bytes_per_unit;
            }
    }
    std::string joined;
    int k = 0;
    for (auto &kv : pmg::g_prof_tot) {
        if (k >= cap)
            break;
        joined += kv.first;
        joined += "\n";
        ms[k] = kv.second.ms;
        bytes[k] = kv.second.bytes;
        launches[k] = kv.second.n;
        k++;
    }
    *count = k;
    strncpy(names, joined.c_str(), names_len - 1);
    names[names_len - 1] = '\0';
    return PMG_OK;
}

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

extern "C" int pmg_tune_set(const char *name, int32_t value)
{
    const int i = pmg::tune_index(name);
    if (i < 0) {
        pmg::set_error("pmg_tune_set: unknown parameter '%s'", name ? name : "(null)");
        return PMG_EINVAL;
    }
    const pmg::TuneSpec &t = pmg::g_tune_spec[i];
    if (value == 0 && t.lo > 0)
        value = t.def;
    if (value < 0)
        value = t.def;
    if (value < t.lo || value > t.hi) {
        pmg::set_error("pmg_tune_set: %s = %d outside [%d, %d]", name, value, t.lo, t.hi);
        return PMG_ERANGE;
    }
    pmg::g_tune[i].store(value);
    return PMG_OK;
}

extern "C" int pmg_tune_get(const char *name, int32_t *value)
{
    const int i = pmg::tune_index(name);
    if (i < 0 || !value) {
        pmg::set_error("pmg_tune_get: unknown parameter '%s'", name ? name : "(null)");
        return PMG_EINVAL;
    }
    *value = pmg::g_tune[i].load();
    return PMG_OK;
}
