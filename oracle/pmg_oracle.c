/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C restatement of PMMoTo's voxel-morphology arithmetic, used by the
 * test suite, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py as the checker for the CUDA path.  Nothing in the shipped package
 * links, imports or executes this file.
 *
 * Every function states which reference routine it restates (paths relative
 * to the PMMoTo source tree, v1.0.7).  The arithmetic is kept in the same
 * precision and the same operation order as the reference so that results
 * are bit-identical; build with -ffp-contract=off so that no multiply-add is
 * fused (the x86-64 reference build has no FMA contraction).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Number of OpenMP threads the 3-D drivers use (1 without OpenMP). */
#ifdef _OPENMP
#include <omp.h>
int or_num_threads(void) { return omp_get_max_threads(); }
void or_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
#else
int or_num_threads(void) { return 1; }
void or_set_threads(int n) { (void)n; }
#endif

typedef struct {
    int32_t vertex;
    float height;
    float range;
} or_hull; /* layout of `Hull`, src/pmmoto/filters/distance/_distance.hpp:15-20 */

/* intersect_parabolas, _distance.hpp:60-72: float numerator, double divide. */
static float or_intersect(float f_r, float r, float f_q, float q, float aniso)
{
    float factor1 = (r - q) * aniso;
    float factor2 = r + q;
    float num = f_r - f_q + factor1 * factor2;
    return (float)((double)num / (2.0 * (double)factor1));
}

/* update_hull, _distance.hpp:89-112. */
static void or_update_hull(int *k, long i, float ff, int32_t *hv, float *hh,
                           float *ranges, float aniso)
{
    int kk = *k;
    float s = or_intersect(ff, (float)i, hh[kk], (float)hv[kk], aniso);
    while (kk > 0 && s <= ranges[kk]) {
        kk--;
        s = or_intersect(ff, (float)i, hh[kk], (float)hv[kk], aniso);
    }
    kk++;
    hv[kk] = (int32_t)i;
    hh[kk] = ff;
    ranges[kk] = s;
    ranges[kk + 1] = INFINITY;
    *k = kk;
}

/*
 * squared_edt_1d<uint8_t>, _distance.hpp:135-182.  Linear two-sweep distance
 * along one line with multi-label resets and optional correctors.
 */
void or_edt_pass0_line(const uint8_t *img, float *d, int n, long stride,
                       float res, float lower_corrector, float upper_corrector)
{
    if (n <= 0)
        return;
    uint8_t seg = img[0];
    d[0] = seg == 0 ? 0.0f : lower_corrector * res;
    for (long i = 1; i < n; i++) {
        uint8_t v = img[i * stride];
        if (v == 0) {
            d[i * stride] = 0.0f;
        } else if (v == seg) {
            d[i * stride] = d[(i - 1) * stride] + res;
        } else {
            d[i * stride] = res;
            d[(i - 1) * stride] = (float)(img[(i - 1) * stride] != 0) * res;
            seg = v;
        }
    }
    if (d[(long)(n - 1) * stride] > upper_corrector * res)
        d[(long)(n - 1) * stride] = upper_corrector * res;
    for (long i = n - 2; i >= 0; i--) {
        float a = d[i * stride];
        float b = d[(i + 1) * stride] + res;
        d[i * stride] = fminf(a, b);
    }
    for (long i = 0; i < n; i++)
        d[i * stride] *= d[i * stride];
}

/* Scratch for one line of the lower-envelope routines. */
typedef struct {
    float *ff, *hh, *ranges;
    int32_t *hv;
    long cap;
} or_scratch;

static int or_scratch_reserve(or_scratch *s, long n)
{
    if (n <= s->cap)
        return 0;
    free(s->ff);
    free(s->hh);
    free(s->ranges);
    free(s->hv);
    s->ff = (float *)malloc(sizeof(float) * (size_t)(n + 1));
    s->hh = (float *)malloc(sizeof(float) * (size_t)(n + 1));
    s->ranges = (float *)malloc(sizeof(float) * (size_t)(n + 2));
    s->hv = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    s->cap = n;
    return (s->ff && s->hh && s->ranges && s->hv) ? 0 : -1;
}

static void or_scratch_free(or_scratch *s)
{
    free(s->ff);
    free(s->hh);
    free(s->ranges);
    free(s->hv);
    memset(s, 0, sizeof(*s));
}

/*
 * squared_edt_1d_parabolic, _distance.hpp:184-272.  Lower envelope of the
 * parabolas res^2 (i - v)^2 + f(v) with imported boundary hulls.
 */
static void or_parabolic_line_s(float *img, int n, float res, long stride,
                                const or_hull *lower, int nl,
                                const or_hull *upper, int nu, or_scratch *s)
{
    if (n <= 0)
        return;
    const float aniso = res * res;
    long cap = (long)n + nl + nu;
    or_scratch_reserve(s, cap + 1);
    float *ff = s->ff, *hh = s->hh, *ranges = s->ranges;
    int32_t *hv = s->hv;
    for (long i = 0; i < cap; i++) {
        hh[i] = 0.0f;
        hv[i] = 0;
        ranges[i] = 0.0f;
    }
    ranges[cap] = 0.0f;
    for (long i = 0; i < n; i++)
        ff[i] = img[i * stride];

    long loop_start = 1;
    ranges[0] = -INFINITY;
    ranges[1] = INFINITY;
    int k = 0;
    if (nl > 0) {
        loop_start = 0;
        for (int j = nl - 1; j >= 0; j--) {
            hv[k] = lower[j].vertex;
            hh[k] = lower[j].height;
            ranges[k] = lower[j].range;
            ranges[k + 1] = INFINITY;
            k++;
        }
        k--;
    } else {
        hv[0] = 0;
        hh[0] = ff[0];
    }
    for (long i = loop_start; i < n; i++)
        or_update_hull(&k, i, ff[i], hv, hh, ranges, aniso);
    for (int j = 0; j < nu; j++)
        or_update_hull(&k, (long)upper[j].vertex + n, upper[j].height, hv, hh,
                       ranges, aniso);
    k = 0;
    for (long i = 0; i < n; i++) {
        while (ranges[k + 1] < (float)i)
            k++;
        float dx = (float)(i - hv[k]);
        img[i * stride] = aniso * (dx * dx) + hh[k];
    }
}

void or_parabolic_line(float *img, int n, float res, long stride,
                       const or_hull *lower, int nl, const or_hull *upper,
                       int nu)
{
    or_scratch s = {0};
    or_parabolic_line_s(img, n, res, stride, lower, nl, upper, nu, &s);
    or_scratch_free(&s);
}

/*
 * return_boundary_hull, _distance.hpp:296-356.  Envelope of one line segment,
 * of which up to num_hull+1 finite parabolas are kept from the chosen end.
 * The reference's to_finite(img, n) call ignores the stride; no value on this
 * path can be +inf (pass 0 maps inf to FLT_MAX, and a parabola evaluation
 * cannot overflow at these sizes), so the call is a no-op and is restated
 * here on the line itself.  When n == 1 and the value is not finite the
 * reference reads one slot past its vectors (the "phantom" parabola at k=1);
 * that slot is taken here as vertex 0, height 0.
 * Returns the number of hulls written to `out` (capacity num_hull+1).
 */
static int or_boundary_hull_s(float *img, int n, float res, long stride,
                              int num_hull, int index_corrector, int forward,
                              or_hull *out, or_scratch *s)
{
    for (long i = 0; i < n; i++)
        if (img[i * stride] == INFINITY)
            img[i * stride] = FLT_MAX;
    int cnt = 0;
    if (n <= 0)
        return 0;
    if (n == 1 && img[0] < FLT_MAX) {
        out[0].vertex = index_corrector;
        out[0].height = img[0];
        out[0].range = INFINITY;
        return 1;
    }
    const float aniso = res * res;
    long cap = n > 2 ? n : 2;
    or_scratch_reserve(s, cap + 1);
    float *ff = s->ff, *hh = s->hh, *ranges = s->ranges;
    int32_t *hv = s->hv;
    for (long i = 0; i < cap; i++) {
        ff[i] = 0.0f;
        hh[i] = 0.0f;
        hv[i] = 0;
        ranges[i] = 0.0f;
    }
    ranges[cap] = 0.0f;
    for (long i = 0; i < n; i++)
        ff[i] = img[i * stride];
    hh[0] = ff[0];
    ranges[0] = -INFINITY;
    ranges[1] = INFINITY;
    int k = 1;
    for (long i = 1; i < n; i++)
        or_update_hull(&k, i, ff[i], hv, hh, ranges, aniso);

    if (num_hull > k)
        num_hull = k;
    int kk = forward ? 0 : k;
    int step = forward ? 1 : -1;
    while (cnt <= num_hull && kk >= 0 && kk <= k) {
        if (hh[kk] < FLT_MAX) {
            out[cnt].vertex = hv[kk] + index_corrector;
            out[cnt].height = hh[kk];
            out[cnt].range = ranges[kk] + (float)index_corrector;
            cnt++;
            if (hh[kk] == 0.9f)
                break;
        }
        kk += step;
    }
    return cnt;
}

int or_boundary_hull(float *img, int n, float res, long stride, int num_hull,
                     int index_corrector, int forward, or_hull *out)
{
    or_scratch s = {0};
    int c = or_boundary_hull_s(img, n, res, stride, num_hull, index_corrector,
                               forward, out, &s);
    or_scratch_free(&s);
    return c;
}

/*
 * _get_nearest_boundary_index, src/pmmoto/core/_voxels.hpp:60-79 with the
 * skip handling of determine_index_nearest_boundary, _voxels.pyx:118-153.
 * Returns the absolute index of the first (forward) or last (backward) voxel
 * equal to `label` within [lower_skip, n - upper_skip), or -1.
 */
long or_nearest_index(const uint8_t *line, long n, long stride, uint8_t label,
                      int forward, long lower_skip, long upper_skip)
{
    long m = n - lower_skip - upper_skip;
    if (m <= 0)
        return -1;
    if (forward) {
        for (long c = 0; c < m; c++)
            if (line[(lower_skip + c) * stride] == label)
                return c + lower_skip;
    } else {
        for (long c = 0; c < m; c++) {
            long idx = m - 1 - c;
            if (line[(lower_skip + idx) * stride] == label)
                return idx + lower_skip;
        }
    }
    return -1;
}

/*
 * Per-axis boundary configuration for the 3-D drivers.
 *   periodic  : the axis imports correctors (axis 0) or hulls (axes 1, 2)
 *   Axis 0 (correctors, euclidean_distance_transform.py:395-447 and
 *   _distance.pyx:240-279):
 *     F = first zero in [f_lo, n), L = last zero in [l_lo, n - l_hi)
 *     upper corrector = F + a_u, lower corrector = n - L + a_l (inf if none)
 *   Axes 1, 2 (hulls, euclidean_distance_transform.py:270-291, :450-528):
 *     forward hull segment search skips hf_lo at the low end,
 *     backward hull segment search skips hb_hi at the high end.
 * edt3d uses f_lo = l_lo = l_hi = 0, a_u = 1, a_l = 0, hf_lo = hb_hi = 0.
 * corrected_edt on a padded image with pads (plo, phi) uses
 *   f_lo = l_lo = 2 plo, l_hi = 2 phi, a_u = -plo, a_l = -phi - 1,
 *   hf_lo = 2 plo, hb_hi = 2 phi.
 */
typedef struct {
    int32_t periodic, f_lo, l_lo, l_hi, a_u, a_l, hf_lo, hb_hi;
} or_axis_cfg;

static void axis_dims(int axis, const int64_t *shape, int *d1, int *d2)
{
    (void)shape;
    if (axis == 0) {
        *d1 = 1;
        *d2 = 2;
    } else if (axis == 1) {
        *d1 = 0;
        *d2 = 2;
    } else {
        *d1 = 0;
        *d2 = 1;
    }
}

/* get_initial_envelope, _distance.pyx:308-353 (+ to_finite over the image).
   Lines are independent; they are spread over OpenMP threads. */
static void or_pass0_3d(const uint8_t *img, float *out, const int64_t *shape,
                        const float *res, int axis, const or_axis_cfg *cfg)
{
    long st[3] = {shape[1] * shape[2], shape[2], 1};
    int d1, d2;
    axis_dims(axis, shape, &d1, &d2);
    long n = shape[axis];
    long s1 = shape[d1], s2 = shape[d2];
#pragma omp parallel for schedule(static)
    for (long li = 0; li < s1 * s2; li++) {
        long a = li / s2, b = li % s2;
        long base = a * st[d1] + b * st[d2];
        float lc = INFINITY, uc = INFINITY;
        if (cfg->periodic) {
            long F = or_nearest_index(img + base, n, st[axis], 0, 1, cfg->f_lo, 0);
            long L = or_nearest_index(img + base, n, st[axis], 0, 0, cfg->l_lo,
                                      cfg->l_hi);
            if (F != -1)
                uc = (float)(F + cfg->a_u);
            if (L != -1)
                lc = (float)(n - L + cfg->a_l);
        }
        or_edt_pass0_line(img + base, out + base, (int)n, st[axis], res[axis], lc,
                          uc);
    }
    long total = shape[0] * shape[1] * shape[2];
#pragma omp parallel for schedule(static)
    for (long i = 0; i < total; i++)
        if (out[i] == INFINITY)
            out[i] = FLT_MAX;
}

/*
 * get_boundary_hull (_distance.pyx:544-618) for both ends of one line, then
 * get_parabolic_envelope (_distance.pyx:86-127) on that line.  The far-end
 * hull (backward) becomes the lower import and the near-end hull (forward)
 * the upper import (euclidean_distance_transform.py:288-290, :514-526).
 */
static void or_parabolic_3d(const uint8_t *og, float *out,
                            const int64_t *shape, const float *res, int axis,
                            const or_axis_cfg *cfg, int num_hull)
{
    long st[3] = {shape[1] * shape[2], shape[2], 1};
    int d1, d2;
    axis_dims(axis, shape, &d1, &d2);
    long n = shape[axis];
    long s1 = shape[d1], s2 = shape[d2];
    or_hull *lo = NULL, *up = NULL;
    int *nlo = NULL, *nup = NULL;
    int hcap = num_hull + 2;
    if (cfg->periodic) {
        lo = (or_hull *)malloc(sizeof(or_hull) * (size_t)(s1 * s2 * hcap));
        up = (or_hull *)malloc(sizeof(or_hull) * (size_t)(s1 * s2 * hcap));
        nlo = (int *)calloc((size_t)(s1 * s2), sizeof(int));
        nup = (int *)calloc((size_t)(s1 * s2), sizeof(int));
#pragma omp parallel
        {
            or_scratch s = {0};
#pragma omp for schedule(static)
            for (long li = 0; li < s1 * s2; li++) {
                long a = li / s2, b = li % s2;
                long base = a * st[d1] + b * st[d2];
                for (int fwd = 1; fwd >= 0; fwd--) {
                    long lsk = fwd ? cfg->hf_lo : 0;
                    long usk = fwd ? 0 : cfg->hb_hi;
                    long bound = or_nearest_index(og + base, n, st[axis], 0, fwd,
                                                  lsk, usk);
                    long start, nv;
                    int corr;
                    if (bound == -1) {
                        start = lsk;
                        nv = n - usk - lsk;
                        corr = fwd ? 0 : (int)(-nv);
                    } else if (fwd) {
                        start = lsk;
                        nv = bound - lsk + 1;
                        corr = 0;
                    } else {
                        start = bound;
                        nv = n - bound - usk;
                        corr = (int)(-nv);
                    }
                    or_hull *dst = fwd ? up + li * hcap : lo + li * hcap;
                    int c = or_boundary_hull_s(out + base + start * st[axis],
                                               (int)nv, res[axis], st[axis],
                                               num_hull, corr, fwd, dst, &s);
                    if (fwd)
                        nup[li] = c;
                    else
                        nlo[li] = c;
                }
            }
            or_scratch_free(&s);
        }
    }
#pragma omp parallel
    {
        or_scratch s = {0};
#pragma omp for schedule(static)
        for (long li = 0; li < s1 * s2; li++) {
            long a = li / s2, b = li % s2;
            long base = a * st[d1] + b * st[d2];
            if (cfg->periodic)
                or_parabolic_line_s(out + base, (int)n, res[axis], st[axis],
                                    lo + li * hcap, nlo[li], up + li * hcap,
                                    nup[li], &s);
            else
                or_parabolic_line_s(out + base, (int)n, res[axis], st[axis],
                                    NULL, 0, NULL, 0, &s);
        }
        or_scratch_free(&s);
    }
    free(lo);
    free(up);
    free(nlo);
    free(nup);
}

/*
 * Squared EDT of a 3-D uint8 image, C order.  With the edt3d configuration
 * this restates edt3d (euclidean_distance_transform.py:208-303) without the
 * final square root; with the corrected configuration it restates
 * corrected_edt (:56-101) on a single rank.  `cfg` holds three axis entries.
 */
int or_edt3d_sq(const uint8_t *img, float *out, const int64_t *shape,
                const float *res, const or_axis_cfg *cfg, int num_hull)
{
    if (shape[0] <= 0 || shape[1] <= 0 || shape[2] <= 0)
        return 0;
    or_pass0_3d(img, out, shape, res, 0, &cfg[0]);
    or_parabolic_3d(img, out, shape, res, 1, &cfg[1], num_hull);
    or_parabolic_3d(img, out, shape, res, 2, &cfg[2], num_hull);
    return 0;
}

/*
 * edt2d (euclidean_distance_transform.py:104-205): linear pass along axis 1,
 * then the envelope along axis 0.  The periodic correctors of axis 1 follow
 * :126-140 and the hulls of axis 0 follow :154-195.
 */
int or_edt2d_sq(const uint8_t *img, float *out, const int64_t *shape2,
                const float *res, const int32_t *periodic, int num_hull)
{
    long n0 = shape2[0], n1 = shape2[1];
    if (n0 <= 0 || n1 <= 0)
        return 0;
    for (long x = 0; x < n0; x++) {
        float lc = INFINITY, uc = INFINITY;
        const uint8_t *line = img + x * n1;
        if (periodic[1]) {
            long F = or_nearest_index(line, n1, 1, 0, 1, 0, 0);
            long L = or_nearest_index(line, n1, 1, 0, 0, 0, 0);
            if (F != -1)
                uc = (float)(F + 1);
            if (L != -1)
                lc = (float)(n1 - L);
        }
        or_edt_pass0_line(line, out + x * n1, (int)n1, 1, res[1], lc, uc);
    }
    for (long i = 0; i < n0 * n1; i++)
        if (out[i] == INFINITY)
            out[i] = FLT_MAX;
    int64_t shape3[3] = {1, n0, n1};
    or_axis_cfg c = {periodic[0], 0, 0, 0, 1, 0, 0, 0};
    float res3[3] = {1.0f, res[0], res[1]};
    /* the 2-D envelope along axis 0 is the 3-D envelope along axis 1 of a
       (1, n0, n1) view: same lines, same stride, same hull rules */
    or_parabolic_3d(img, out, shape3, res3, 1, &c, num_hull);
    return 0;
}

/*
 * Sphere voxelisation: gen_sphere_img_brute_force + Sphere::contains
 * (src/pmmoto/domain_generation/domain_generation.hpp:38-58,91-127,
 * src/pmmoto/particles/spheres.hpp:41-48).  img is set to 1, then 0 where a
 * voxel centre lies in any sphere: (dx*dx + dy*dy + dz*dz) <= r*r in double,
 * dx = centre - voxel.  Spheres are (n, 4) rows of x, y, z, r.  The Verlet
 * culling of the reference only skips spheres that cannot contain a voxel
 * centre of the cell, so testing every sphere gives the same image.
 */
int or_spheres(const double *sph, long nsph, const double *cx, const double *cy,
               const double *cz, uint8_t *img, const int64_t *shape)
{
    long n0 = shape[0], n1 = shape[1], n2 = shape[2];
    double *r2 = (double *)malloc(sizeof(double) * (size_t)(nsph > 0 ? nsph : 1));
    for (long s = 0; s < nsph; s++)
        r2[s] = sph[s * 4 + 3] * sph[s * 4 + 3];
#pragma omp parallel for schedule(dynamic, 1)
    for (long i = 0; i < n0; i++)
        for (long j = 0; j < n1; j++)
            for (long k = 0; k < n2; k++) {
                uint8_t v = 1;
                for (long s = 0; s < nsph; s++) {
                    double dx = sph[s * 4 + 0] - cx[i];
                    double dy = sph[s * 4 + 1] - cy[j];
                    double dz = sph[s * 4 + 2] - cz[k];
                    if ((dx * dx + dy * dy + dz * dz) <= r2[s]) {
                        v = 0;
                        break;
                    }
                }
                img[(i * n1 + j) * n2 + k] = v;
            }
    free(r2);
    return 0;
}
