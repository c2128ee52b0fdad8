// Internal interface between the EDT kernels and their users (morphology).
#pragma once

#include "pmg_common.cuh"

namespace pmg {

// Lines of a pass: all lines along axis `ax` whose coordinates on the other
// two axes (d1 < d2) lie in [b1lo, b1lo + nb1) x [b2lo, b2lo + nb2).
struct Lines {
    long long s0, s1, s2;
    int ax;
    int b1lo, nb1, b2lo, nb2;
    __host__ __device__ long long count() const { return (long long)nb1 * nb2; }
};

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

int launch_pass0(const uint8_t *img, float *out, const Lines &Ls, float res,
                 const pmg_axis_cfg &cfg, cudaStream_t st);
int launch_envelope(const float *fin, float *fout, const Lines &Ls, float res,
                    const pmg_axis_cfg &cfg, int num_hull, int form, const MorphEpi &me,
                    cudaStream_t st);
int edt3d_run(const uint8_t *img, float *out, float *tmp, const int64_t *shape, const float *res,
              const pmg_axis_cfg *cfg, int num_hull, int form, cudaStream_t st);

} // namespace pmg
