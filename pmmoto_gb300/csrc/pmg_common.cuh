// Shared definitions for the pmmoto_gb300 CUDA library (sm_103a).
#pragma once

#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/pmmoto_gb300.h"

namespace pmg {

// ---------------------------------------------------------------------------
// error reporting: every C entry point returns a status; the message of the
// last failure on the calling host thread is kept for pmg_last_error().
// ---------------------------------------------------------------------------
void set_error(const char *fmt, ...);

#define PMG_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t e__ = (call);                                             \
        if (e__ != cudaSuccess) {                                             \
            ::pmg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,       \
                             cudaGetErrorString(e__));                        \
            return PMG_ECUDA;                                                 \
        }                                                                     \
    } while (0)

#define PMG_CHECK_LAUNCH() PMG_CUDA(cudaGetLastError())

#define PMG_TRY(expr)                                                         \
    do {                                                                      \
        int s__ = (expr);                                                     \
        if (s__ != PMG_OK)                                                    \
            return s__;                                                       \
    } while (0)

// Stream-ordered scratch from a memory pool the library owns on each device
// (unlimited release threshold, so it stays resident between calls).
int scratch_alloc(void **p, size_t bytes, cudaStream_t st);
int scratch_free(void *p, cudaStream_t st);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch accounting.  Every kernel launch is bracketed by prof_begin /
// prof_end: the launch counter always advances; when profiling is switched
// on (pmg_prof_enable) a CUDA event pair is recorded on the launching stream
// together with the launch's algorithmic bytes, and pmg_prof_read later
// resolves the events into per-kernel totals.
int prof_begin(const char *name, cudaStream_t st);
void prof_end(int slot, double bytes, cudaStream_t st);
// Kernels whose work is sized on the device add the units they process to
// prof_units(id) (one counter per kind of kernel); prof_end_units records the
// bytes per unit for the profile.
constexpr int kUnitSlots = 16;
constexpr int kUnitsCapRows = 0, kUnitsCapMid = 1, kUnitsCapLast = 2, kUnitsDrainUpdate = 3;
constexpr int kUnitsGrowUniteA = 4, kUnitsGrowUniteB = 5, kUnitsCrossUnite = 6, kUnitsGrowApply = 7;
constexpr int kUnitsGrowUnitePair = 8;
unsigned long long *prof_units(int id);
void prof_end_units(int slot, int id, double bytes_per_unit, cudaStream_t st);

// Launch parameters an autotuner may change at run time (pmg_tune_set):
// results never depend on them, only speed.  Read once per launch.
enum TuneKnob { kTuneEdtPairSeg = 0, kTuneEdtPairCtas, kTuneEdtRowsCtas, kTuneCcCrossFused, kTuneEdtPath, kTuneEdtFallback, kTuneEdtFallbackRows, kTuneEdtNarrow, kTuneEdtNarrowRows,
               kTuneCcSeamBatched, kTuneEdtWide, kTuneKnobs };
int tune_value(int knob);

// Validate a padded single-rank geometry: positive shape, boundary codes in
// range, non-negative pads that leave a non-empty own region on every axis.
inline int check_geometry(const int64_t *shape, const int32_t *bc, const int32_t *pad)
{
    if (!shape || !bc || !pad) {
        set_error("null geometry argument");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; d++) {
        if (shape[d] <= 0) {
            set_error("shape[%d] must be positive", d);
            return PMG_EINVAL;
        }
        for (int s = 0; s < 2; s++) {
            if (bc[2 * d + s] < PMG_BC_END || bc[2 * d + s] > PMG_BC_PERIODIC) {
                set_error("boundary code %d out of range", bc[2 * d + s]);
                return PMG_EINVAL;
            }
            if (pad[2 * d + s] < 0) {
                set_error("negative pad on axis %d", d);
                return PMG_EINVAL;
            }
        }
        if ((long long)pad[2 * d] + pad[2 * d + 1] >= shape[d]) {
            set_error("pads of axis %d leave no own voxels", d);
            return PMG_EINVAL;
        }
        if ((bc[2 * d] == PMG_BC_PERIODIC) != (bc[2 * d + 1] == PMG_BC_PERIODIC)) {
            set_error("axis %d is periodic on one face only", d);
            return PMG_EINVAL;
        }
    }
    return PMG_OK;
}

inline int check_box6(const int64_t *shape, const int64_t *box)
{
    for (int d = 0; d < 3; d++)
        if (box[2 * d] < 0 || box[2 * d + 1] > shape[d] || box[2 * d] > box[2 * d + 1]) {
            set_error("box outside the volume on axis %d", d);
            return PMG_EINVAL;
        }
    return PMG_OK;
}

inline unsigned grid_for(long long n, int block, long long cap = 152LL * 64)
{
    long long g = (n + block - 1) / block;
    if (g < 1)
        g = 1;
    if (g > cap)
        g = cap;
    return (unsigned)g;
}

// ---------------------------------------------------------------------------
// exact float32 arithmetic (round-to-nearest, no contraction), matching the
// reference's x86-64 build where no multiply-add is fused.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// Intersection abscissa of the parabolas a(x-r)^2+f_r and a(x-q)^2+f_q as
// the reference computes it (_distance.hpp:60-72): float numerator, then
// (float)((double)num / (2.0 * factor1)).  Both operands of that division
// are float32 values, and double has 53 >= 2*24+2 significand bits, so
// rounding the double quotient to float equals the correctly rounded float32
// quotient (double rounding is innocuous for division at these precisions;
// S. A. Figueroa, "When is double rounding innocuous?", SIGNUM 1995).  The
// float32 IEEE division __fdiv_rn therefore gives the same bits without the
// slow FP64 path.  2*factor1 is exact in float32 (a power-of-two scaling).
__device__ __forceinline__ float isect(float f_r, float r, float f_q, float q, float aniso)
{
    float factor1 = fmul(fsub(r, q), aniso);
    float factor2 = fadd(r, q);
    float num = fadd(fsub(f_r, f_q), fmul(factor1, factor2));
    return __fdiv_rn(num, fmul(2.0f, factor1));
}

// Two ints set on the device in stream order (a host-to-device copy from
// pageable memory would wait for the stream first).
__global__ void k_set_int2(int *p, int a, int b);

// x range of a set of 2x2x2 blocks kept in device memory as two ints, both
// raised with atomicMax from zero: [0] = 1 + the largest block plane,
// [1] = kRangeBig - the smallest (so a zeroed pair is the empty range).
constexpr int kRangeBig = 1 << 30;

} // namespace pmg
