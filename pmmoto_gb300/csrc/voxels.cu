// Sphere voxelisation, halo update and small reductions (sm_103a).
//
//  * pmg_spheres  -- gen_sphere_img_brute_force / Sphere::contains
//    (src/pmmoto/domain_generation/domain_generation.hpp:38-127,
//    src/pmmoto/particles/spheres.hpp:41-48): img = 1, then 0 where a voxel
//    centre satisfies (dx*dx + dy*dy + dz*dz) <= r*r in float64 with
//    dx = centre - voxel, evaluated left to right without fused multiply-add.
//    One thread block per sphere walks a bounding box of voxel indices (two
//    voxels of margin around the analytic box, so no candidate is missed) and
//    stores 0 where the exact test holds; the stores are idempotent so sphere
//    order and overlaps do not matter.
//  * pmg_update_buffer -- communication.update_buffer on one rank
//    (core/communication.py:101-118, 160-228): halo voxels of periodic axes
//    take the value of the own voxel they copy, wall planes become 0.
//  * pmg_count_eq / pmg_max_f32 -- the scalar reductions behind porosity,
//    saturation, phase_exists and PorousMedia.max_distance.
#include <cfloat>
#include <cstring>

#include "pmg_common.cuh"

namespace pmg {

struct Grid1 {
    const double *c; // voxel-centre coordinates (linspace)
    long long n;
    double c0, h;    // first centre and spacing used only for the index box
};

__device__ __forceinline__ void index_box(const Grid1 &g, double x, double r, long long &lo, long long &hi)
{
    const double a = (x - r - g.c0) / g.h, b = (x + r - g.c0) / g.h;
    double la = floor(a) - 2.0, hb = ceil(b) + 2.0;
    const double n = (double)g.n;
    if (!(la == la) || !(hb == hb)) { // NaN radius or centre: test the whole axis
        la = 0.0;
        hb = n;
    }
    // clamp before converting so that no coordinate can leave [0, n]
    la = fmin(fmax(la, 0.0), n);
    hb = fmin(fmax(hb, 0.0), n);
    lo = (long long)la;
    hi = (long long)hb;
    if (hi < lo)
        hi = lo;
}

__global__ void k_spheres(const double *__restrict__ sph, long long nsph, Grid1 gx, Grid1 gy, Grid1 gz,
                          uint8_t *__restrict__ img)
{
    for (long long s = blockIdx.x; s < nsph; s += gridDim.x) {
        const double x = sph[4 * s], y = sph[4 * s + 1], z = sph[4 * s + 2], r = sph[4 * s + 3];
        const double r2 = __dmul_rn(r, r);
        long long i0, i1, j0, j1, k0, k1;
        index_box(gx, x, r, i0, i1);
        index_box(gy, y, r, j0, j1);
        index_box(gz, z, r, k0, k1);
        const long long ni = i1 - i0, nj = j1 - j0, nk = k1 - k0;
        const long long tot = ni * nj * nk;
        for (long long q = threadIdx.x; q < tot; q += blockDim.x) {
            const long long k = k0 + q % nk;
            const long long j = j0 + (q / nk) % nj;
            const long long i = i0 + q / (nk * nj);
            const double dx = __dsub_rn(x, gx.c[i]);
            const double dy = __dsub_rn(y, gy.c[j]);
            const double dz = __dsub_rn(z, gz.c[k]);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (d2 <= r2)
                img[(i * gy.n + j) * gz.n + k] = 0;
        }
    }
}

struct Halo {
    long long s[3];
    int periodic[3];
    int own_lo[3], own_len[3];
    int wall_lo[3], wall_hi[3];
};

template <typename T>
__global__ void k_update_buffer(T *img, Halo H)
{
    const long long n = H.s[0] * H.s[1] * H.s[2];
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        long long c[3];
        c[2] = idx % H.s[2];
        const long long r = idx / H.s[2];
        c[1] = r % H.s[1];
        c[0] = r / H.s[1];
        bool wall = false, halo = false, ok = true;
        long long t[3];
        for (int d = 0; d < 3; d++) {
            t[d] = c[d];
            if ((H.wall_lo[d] && c[d] == 0) || (H.wall_hi[d] && c[d] == H.s[d] - 1))
                wall = true;
            const bool out = c[d] < H.own_lo[d] || c[d] >= H.own_lo[d] + H.own_len[d];
            if (out) {
                if (H.periodic[d] && H.own_len[d] > 0) {
                    long long q = (c[d] - H.own_lo[d]) % H.own_len[d];
                    if (q < 0)
                        q += H.own_len[d];
                    t[d] = q + H.own_lo[d];
                    halo = true;
                } else {
                    ok = false; // reservoir or end/wall halo: no neighbour copy
                }
            }
        }
        if (wall) {
            img[idx] = (T)0;
        } else if (halo && ok) {
            img[idx] = img[(t[0] * H.s[1] + t[1]) * H.s[2] + t[2]];
        }
    }
}

// One warp per row of the box; lanes walk the row's contiguous bytes.
__global__ void k_count_eq(const uint8_t *__restrict__ img, long long s1, long long s2, long long lo0,
                           long long n0, long long lo1, long long n1, long long lo2, long long n2,
                           uint8_t value, unsigned long long *cnt)
{
    const long long rows = n0 * n1;
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned int c = 0;
    for (long long r = warp; r < rows; r += nwarps) {
        const long long i = r / n1, j = r - (r / n1) * n1;
        const uint8_t *row = img + ((lo0 + i) * s1 + lo1 + j) * s2 + lo2;
        for (long long k = lane; k < n2; k += 32)
            c += row[k] == value;
    }
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c)
        atomicAdd(cnt, (unsigned long long)c);
}

__global__ void k_max_f32(const float *__restrict__ x, long long s1, long long s2, long long lo0, long long n0,
                          long long lo1, long long n1, long long lo2, long long n2, unsigned int *best)
{
    const long long tot = n0 * n1 * n2;
    float m = -FLT_MAX;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < tot;
         q += (long long)gridDim.x * blockDim.x) {
        const long long k = q % n2, j = (q / n2) % n1, i = q / (n2 * n1);
        m = fmaxf(m, x[((lo0 + i) * s1 + lo1 + j) * s2 + lo2 + k]);
    }
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) {
        // order-preserving map of float to unsigned for atomicMax
        unsigned int u = __float_as_uint(m);
        u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        atomicMax(best, u);
    }
}

Halo make_halo(const int64_t *shape, const int32_t *bc, const int32_t *pad)
{
    Halo H;
    for (int d = 0; d < 3; d++) {
        H.s[d] = shape[d];
        H.periodic[d] = bc[2 * d] == PMG_BC_PERIODIC;
        H.own_lo[d] = pad[2 * d];
        H.own_len[d] = (int)(shape[d] - pad[2 * d] - pad[2 * d + 1]);
        H.wall_lo[d] = bc[2 * d] == PMG_BC_WALL;
        H.wall_hi[d] = bc[2 * d + 1] == PMG_BC_WALL;
    }
    return H;
}

int update_buffer_run(void *img, int elem_bytes, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, cudaStream_t st)
{
    const Halo H = make_halo(shape, bc, pad);
    const long long n = shape[0] * shape[1] * shape[2];
    const unsigned g = grid_for(n, 256, 152LL * 16);
    if (elem_bytes == 1)
        {
            const int ps__ = prof_begin("k_update_buffer", st);
            k_update_buffer<uint8_t><<<g, 256, 0, st>>>((uint8_t *)img, H);
            prof_end(ps__, 0.0, st);
        }
    else if (elem_bytes == 4)
        {
            const int ps__ = prof_begin("k_update_buffer", st);
            k_update_buffer<float><<<g, 256, 0, st>>>((float *)img, H);
            prof_end(ps__, 0.0, st);
        }
    else if (elem_bytes == 8)
        {
            const int ps__ = prof_begin("k_update_buffer", st);
            k_update_buffer<uint64_t><<<g, 256, 0, st>>>((uint64_t *)img, H);
            prof_end(ps__, 0.0, st);
        }
    else {
        set_error("update_buffer: element size %d not supported", elem_bytes);
        return PMG_EINVAL;
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

// Count voxels equal to `value` inside box (device counter, not synchronized).
int count_eq_async(const uint8_t *img, const int64_t *shape, const int64_t *box, uint8_t value,
                   unsigned long long *d_cnt, cudaStream_t st)
{
    const long long n0 = box[1] - box[0], n1 = box[3] - box[2], n2 = box[5] - box[4];
    if (n0 <= 0 || n1 <= 0 || n2 <= 0)
        return PMG_OK;
    {
        const int ps__ = prof_begin("k_count_eq", st);
        k_count_eq<<<grid_for(n0 * n1 * 32, 256, 152LL * 64), 256, 0, st>>>(img, shape[1], shape[2], box[0], n0, box[2],
                                                                      n1, box[4], n2, value, d_cnt);
        prof_end(ps__, (double)(n0 * n1 * n2), st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

static int check_box(const int64_t *shape, const int64_t *box)
{
    for (int d = 0; d < 3; d++)
        if (box[2 * d] < 0 || box[2 * d + 1] > shape[d] || box[2 * d] > box[2 * d + 1]) {
            set_error("box outside the volume on axis %d", d);
            return PMG_EINVAL;
        }
    return PMG_OK;
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_spheres(const double *spheres, int64_t nsph, const double *cx, const double *cy,
                           const double *cz, const double grid_c0[3], const double grid_h[3],
                           uint8_t *img, const int64_t shape[3], void *stream)
{
    if (!img || !shape || !cx || !cy || !cz || !grid_c0 || !grid_h || (nsph > 0 && !spheres)) {
        set_error("pmg_spheres: null argument");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; d++)
        if (shape[d] <= 0 || !(grid_h[d] > 0.0)) {
            set_error("pmg_spheres: bad grid on axis %d", d);
            return PMG_EINVAL;
        }
    cudaStream_t st = as_stream(stream);
    const long long n = shape[0] * shape[1] * shape[2];
    PMG_CUDA(cudaMemsetAsync(img, 1, (size_t)n, st));
    if (nsph > 0) {
        Grid1 gx{cx, shape[0], grid_c0[0], grid_h[0]}, gy{cy, shape[1], grid_c0[1], grid_h[1]},
            gz{cz, shape[2], grid_c0[2], grid_h[2]};
        const long long blocks = nsph < (1LL << 20) ? nsph : (1LL << 20);
        {
            const int ps__ = prof_begin("k_spheres", st);
            k_spheres<<<(unsigned)blocks, 256, 0, st>>>(spheres, nsph, gx, gy, gz, img);
            prof_end(ps__, 0.0, st);
        }
        PMG_CHECK_LAUNCH();
    }
    return PMG_OK;
}

extern "C" int pmg_update_buffer(void *img, int32_t elem_bytes, const int64_t shape[3], const int32_t bc[6],
                                 const int32_t pad[6], void *stream)
{
    if (!img || !shape || !bc || !pad) {
        set_error("pmg_update_buffer: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geometry(shape, bc, pad));
    return update_buffer_run(img, elem_bytes, shape, bc, pad, as_stream(stream));
}

extern "C" int pmg_count_eq(const uint8_t *img, const int64_t shape[3], const int64_t box[6], int32_t value,
                            int64_t *count, void *stream)
{
    if (!img || !shape || !box || !count) {
        set_error("pmg_count_eq: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_box(shape, box));
    cudaStream_t st = as_stream(stream);
    unsigned long long *d = nullptr, h = 0;
    PMG_TRY(scratch_alloc((void **)&d, sizeof(unsigned long long), st));
    PMG_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), st));
    int s = count_eq_async(img, shape, box, (uint8_t)value, d, st);
    if (s == PMG_OK) {
        PMG_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaStreamSynchronize(st));
        *count = (int64_t)h;
    }
    PMG_TRY(scratch_free(d, st));
    return s;
}

extern "C" int pmg_max_f32(const float *x, const int64_t shape[3], const int64_t box[6], float *out,
                           void *stream)
{
    if (!x || !shape || !box || !out) {
        set_error("pmg_max_f32: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_box(shape, box));
    cudaStream_t st = as_stream(stream);
    unsigned int *d = nullptr, h = 0;
    PMG_TRY(scratch_alloc((void **)&d, sizeof(unsigned int), st));
    PMG_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned int), st));
    const long long n0 = box[1] - box[0], n1 = box[3] - box[2], n2 = box[5] - box[4];
    if (n0 > 0 && n1 > 0 && n2 > 0) {
        {
            const int ps__ = prof_begin("k_max_f32", st);
            k_max_f32<<<grid_for(n0 * n1 * n2, 256, 152LL * 8), 256, 0, st>>>(x, shape[1], shape[2], box[0], n0,
                                                                         box[2], n1, box[4], n2, d);
            prof_end(ps__, (double)(n0 * n1 * n2) * 4, st);
        }
        PMG_CHECK_LAUNCH();
    }
    PMG_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    PMG_TRY(scratch_free(d, st));
    const unsigned int u = (h & 0x80000000u) ? (h & 0x7fffffffu) : ~h;
    float f;
    memcpy(&f, &u, sizeof(f));
    *out = f;
    return PMG_OK;
}
