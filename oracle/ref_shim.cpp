/*
 * ORACLE -- test infrastructure only.
 *
 * C-ABI wrappers around PMMoTo's own C++ kernels, compiled straight from the
 * reference source tree by oracle/build.py into oracle/_ref/libpmref.so.  The
 * reference headers are included from where they lie (the include path is
 * given on the compiler command line); nothing of them is copied here.  The
 * tests use this library to pin the C restatement in pmg_oracle.c to the
 * reference arithmetic line by line, on random inputs.
 */
#include <cstdint>
#include <cstring>
#include <vector>

#include "_distance.hpp"      /* src/pmmoto/filters/distance */
#include "_voxels.hpp"        /* src/pmmoto/core */
#include "spheres.hpp"        /* src/pmmoto/particles */

extern "C" {

void ref_squared_edt_1d(const uint8_t *img, float *d, int n, long stride,
                        float res, float lc, float uc)
{
    squared_edt_1d<uint8_t>(const_cast<uint8_t *>(img), d, n, stride, res, lc,
                            uc);
}

void ref_parabolic_1d(float *img, int n, float res, long stride,
                      const Hull *lower, int nl, const Hull *upper, int nu)
{
    std::vector<Hull> lo(lower, lower + nl), up(upper, upper + nu);
    squared_edt_1d_parabolic(img, n, res, stride, lo, up);
}

int ref_boundary_hull(float *img, int n, float res, long stride, int num_hull,
                      int index_corrector, int forward, Hull *out)
{
    std::vector<Hull> h = return_boundary_hull(img, n, res, stride, num_hull,
                                               index_corrector, forward != 0);
    for (size_t i = 0; i < h.size(); i++)
        out[i] = h[i];
    return (int)h.size();
}

int64_t ref_nearest_index(uint8_t *img, uint8_t label, int n, long stride,
                          int index_corrector, int forward)
{
    return _get_nearest_boundary_index(img, label, n, stride, index_corrector,
                                       forward != 0);
}

int64_t ref_unique_pairs(unsigned long *data, int64_t nrows, uint64_t *out)
{
    auto r = unique_pairs(data, (size_t)nrows);
    for (size_t i = 0; i < r.size(); i++) {
        out[2 * i] = r[i].first;
        out[2 * i + 1] = r[i].second;
    }
    return (int64_t)r.size();
}

/* Sphere::contains for every (voxel centre, sphere) of a grid. */
void ref_spheres(const double *sph, long nsph, const double *cx,
                 const double *cy, const double *cz, uint8_t *img, long n0,
                 long n1, long n2)
{
    std::vector<Sphere> s;
    s.reserve((size_t)nsph);
    for (long i = 0; i < nsph; i++)
        s.emplace_back(sph[4 * i], sph[4 * i + 1], sph[4 * i + 2], sph[4 * i + 3]);
    std::vector<double> v(3);
    for (long i = 0; i < n0; i++)
        for (long j = 0; j < n1; j++)
            for (long k = 0; k < n2; k++) {
                v[0] = cx[i];
                v[1] = cy[j];
                v[2] = cz[k];
                uint8_t o = 1;
                for (auto &sp : s)
                    if (sp.contains(v)) {
                        o = 0;
                        break;
                    }
                img[(i * n1 + j) * n2 + k] = o;
            }
}

} // extern "C"
