// Internal interface between the EDT kernels and their users (morphology).
#pragma once

#include <climits>
#include <cmath>

#include "pmg_common.cuh"

namespace pmg {

// Imported boundary hulls per side the envelope kernels hold (the reference
// keeps at most num_hull + 1 = 5); entry points accept num_hull + 1 <= kMaxHull.
constexpr int kMaxHull = 8;

// Lines of a pass: all lines along axis `ax` whose coordinates on the other
// two axes (d1 < d2) lie in [b1lo, b1lo + nb1) x [b2lo, b2lo + nb2).
struct Lines {
    long long s0, s1, s2;
    int ax;
    int b1lo, nb1, b2lo, nb2;
    __host__ __device__ long long count() const { return (long long)nb1 * nb2; }
};

struct LineGeo {
    long long base, stride;
    int n;
    int a, b; // coordinates of the line along the two other axes (d1 < d2)
};

__device__ __forceinline__ LineGeo line_addr(const Lines &L, long long li)
{
    LineGeo g;
    const int a = L.b1lo + (int)(li / L.nb2);
    const int b = L.b2lo + (int)(li - (li / L.nb2) * L.nb2);
    g.a = a;
    g.b = b;
    if (L.ax == 0) { // lines over (j, k)
        g.base = (long long)a * L.s2 + b;
        g.stride = L.s1 * L.s2;
        g.n = (int)L.s0;
    } else if (L.ax == 1) { // lines over (i, k)
        g.base = (long long)a * L.s1 * L.s2 + b;
        g.stride = L.s2;
        g.n = (int)L.s1;
    } else { // lines over (i, j)
        g.base = ((long long)a * L.s1 + b) * L.s2;
        g.stride = 1;
        g.n = (int)L.s2;
    }
    return g;
}

__host__ inline Lines all_lines(const int64_t *shape, int ax)
{
    Lines L;
    L.s0 = shape[0];
    L.s1 = shape[1];
    L.s2 = shape[2];
    L.ax = ax;
    const int d1 = ax == 0 ? 1 : 0, d2 = ax == 2 ? 1 : 2;
    L.b1lo = 0;
    L.nb1 = (int)shape[d1];
    L.b2lo = 0;
    L.nb2 = (int)shape[d2];
    return L;
}

// Fused morphology epilogue of the last envelope pass (addition/subtraction,
// src/pmmoto/filters/morphological_operators.py:103-228): the distance is
// square-rooted as np.sqrt does, compared with the radius in the precision
// numpy would use, the extension halo is cut off (utils.unpad) and wall
// planes are forced to 0 (set_wall_bcs).
struct MorphEpi {
    uint8_t *out;         // unextended volume (o0, o1, o2)
    long long o0, o1, o2; // unextended shape
    int e0, e1, e2;       // low-side extension per axis
    int wall[6];          // wall planes: axis0 lo/hi, axis1 lo/hi, axis2 lo/hi
    float r32;            // radius rounded to float32
    double r64;           // radius as float64
    int cmp64;            // 1: compare in float64 (numpy float64 radius)
    int dilate;           // 1: addition (1 where d <= r), 0: subtraction
    double thr_sq;        // >= 0: compare the squared unit-resolution distance
                          // with this integer bound instead (FFT-ball modes)
};

// Store of the fused morphology epilogue: "distance within the radius" at
// position i of line g (extended coordinates) -> 0/1 of the unextended volume.
__device__ __forceinline__ void morph_put(const MorphEpi &me, const LineGeo &g, int i, bool within)
{
    const long long io = g.a - me.e0, jo = g.b - me.e1;
    const int ko = i - me.e2;
    if (ko < 0 || ko >= me.o2)
        return;
    uint8_t v = me.dilate ? (uint8_t)within : (uint8_t)!within;
    if ((me.wall[0] && io == 0) || (me.wall[1] && io == me.o0 - 1) || (me.wall[2] && jo == 0) ||
        (me.wall[3] && jo == me.o1 - 1) || (me.wall[4] && ko == 0) || (me.wall[5] && ko == me.o2 - 1))
        v = 0;
    me.out[(io * me.o1 + jo) * me.o2 + ko] = v;
}

// The threshold of the epilogue on a squared distance `val`.
__host__ __device__ __forceinline__ bool morph_within(const MorphEpi &me, float val)
{
    if (me.thr_sq >= 0.0)
        return (double)val <= me.thr_sq;
#ifdef __CUDA_ARCH__
    const float dist = __fsqrt_rn(val);
#else
    const float dist = sqrtf(val); // IEEE correctly rounded, as __fsqrt_rn
#endif
    return me.cmp64 ? ((double)dist <= me.r64) : (dist <= me.r32);
}

__device__ __forceinline__ void morph_store(const MorphEpi &me, const LineGeo &g, int i, float val)
{
    morph_put(me, g, i, morph_within(me, val));
}

// Lines the exact streaming kernel hands back to the general one carry a
// marker in their first output: NaN (float forms) or 255 (morphology).
__device__ __forceinline__ bool line_marked(const float *fout, const MorphEpi &me, const LineGeo &g, int form)
{
    if (form == PMG_EDT_MORPH) {
        const long long io = g.a - me.e0, jo = g.b - me.e1;
        return me.out[(io * me.o1 + jo) * me.o2] == 255;
    }
    const float v = fout[g.base];
    return v != v;
}

// cap: heights above cap * res^2 are treated as absent and outputs above it
// are written as FLT_MAX (INT_MAX: no cap).
int launch_envelope_exact(const float *fin, float *fout, const Lines &Ls, float res, int form,
                          const MorphEpi &me, cudaStream_t st, int cap);
bool exact_path_ok(float res, const pmg_axis_cfg &cfg, int n);
// Largest integer T < lim with morph_within(T * a) (the threshold is monotone
// in the squared distance), -1 when not even 0 is within, lim when T >= lim.
int morph_threshold(const MorphEpi &me, float a, int lim);
// Last morphology pass on exact integer heights: within iff E(x) <= T.
int launch_env_thresh(const float *fin, const Lines &Ls, float res, int T, const MorphEpi &me,
                      cudaStream_t st);

// Capped integer morphology (morph_cap.cu): isotropic power-of-two voxels,
// binary image, threshold T <= kCapMaxT; KA, KB: uint16 scratch of the
// extended volume.
constexpr int kCapMaxT = 1023;
bool cap_path_ok(const float *res, const int64_t *X, int T);
// raw_dilate: E is the unextended image of a dilation without periodic axes
// (no k_extend copy); gate: a device count of the seeds (null: not known to
// be empty), zero making the result all zeros without the envelope passes;
// xr: a device x range of the seed blocks (kRangeBig encoding) -- the
// result is then written only on the x range orange receives ([lo, hi] in
// whole blocks, lo > hi for none) and is undefined elsewhere; blk (with
// raw_dilate): the seeds as one mask per 2x2x2 block (bit (x * 2 + y) * 2 +
// z, blocks in C order over the ceil-halved shape) instead of E
int morph_cap_run(const uint8_t *E, uint16_t *KA, uint16_t *KB, const int64_t *X, int T, const MorphEpi &me,
                  cudaStream_t st, int raw_dilate = 0, const unsigned long long *gate = nullptr,
                  const int *xr = nullptr, int *orange = nullptr, const uint8_t *blk = nullptr);
int edt_cap_run(const uint8_t *E, uint16_t *KA, uint16_t *KB, uint16_t *KC, const int64_t *X, int T,
                cudaStream_t st);

int launch_pass0(const uint8_t *img, float *out, const Lines &Ls, float res,
                 const pmg_axis_cfg &cfg, cudaStream_t st);
// flag_buf (optional): per-line flags of the windowed path, flag_cap lines
// long; without it the flags come from the stream-ordered scratch pool.
int launch_envelope(const float *fin, float *fout, const Lines &Ls, float res,
                    const pmg_axis_cfg &cfg, int num_hull, int form, const MorphEpi &me,
                    cudaStream_t st, int cap = INT_MAX, int *flag_buf = nullptr, long long flag_cap = 0);
int edt3d_run(const uint8_t *img, float *out, float *tmp, const int64_t *shape, const float *res,
              const pmg_axis_cfg *cfg, int num_hull, int form, cudaStream_t st, int *flag_buf = nullptr,
              long long flag_cap = 0);

} // namespace pmg
