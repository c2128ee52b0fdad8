// Porosimetry and morphological drainage driven from native code.
//
// porosimetry (src/pmmoto/filters/porosimetry.py:84-160, mode="distance"):
//   erode -> [inlet-connected] -> if phase 1 exists: [multiphase constraint:
//   inlet-connected phase 1 of the multiphase image] -> dilate.
// drainage, standard method (src/pmmoto/filters/equilibrium_distribution.py:
//   25-179): per capillary pressure, porosimetry with the inlet and multiphase
//   constraints, outlet-connected wetting phase, update, reservoir refill,
//   wetting-phase count in the own region (the saturation numerator).
// All images stay on the device between steps; the host reads back only the
// two phase-existence counts porosimetry branches on and, at the end, the
// per-pressure counts.
#include <vector>

#include "edt_internal.cuh"
#include "pmg_internal.cuh"

namespace pmg {

// Bytes equal to 1 in both words -> 1, else 0 (four voxels per 32-bit word).
__device__ __forceinline__ uint32_t both_one(uint32_t a, uint32_t b)
{
    const uint32_t z = (a ^ 0x01010101u) | (b ^ 0x01010101u);
    const uint32_t t = ((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z; // high bit set where the byte is nonzero
    return (~t & 0x80808080u) >> 7;
}

// res = (res == 1 && nconn == 1) ? 1 : 0, i.e. where((res != 1) | (nconn != 1), 0, res)
__global__ void k_constrain(uint8_t *res, const uint8_t *__restrict__ nconn, long long n)
{
    const long long nw = n >> 4; // 16-byte vectors (both buffers are 256-byte aligned)
    uint4 *r4 = (uint4 *)res;
    const uint4 *c4 = (const uint4 *)nconn;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nw;
         q += (long long)gridDim.x * blockDim.x) {
        uint4 a = r4[q];
        const uint4 b = c4[q];
        a.x = both_one(a.x, b.x);
        a.y = both_one(a.y, b.y);
        a.z = both_one(a.z, b.z);
        a.w = both_one(a.w, b.w);
        r4[q] = a;
    }
    for (long long i = (nw << 4) + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        res[i] = (res[i] == 1 && nconn[i] == 1) ? 1 : 0;
}

// Erosion by thresholding a precomputed squared EDT (subtraction's
// np.where(d <= r, 0, 1), unpad being the identity without extension), wall
// planes forced to 0 (set_wall_bcs).  One warp per (i, j) row.
struct ErodeThr {
    float r32;
    double r64;
    int cmp64;
    double thr_sq; // >= 0: FFT-ball mode, compare the voxel-unit squared distance
    int wall[6];
};

__global__ void k_erode_from_edt(const float *__restrict__ D, uint8_t *__restrict__ out, long long s0,
                                 long long s1, long long s2, ErodeThr T)
{
    const long long rows = s0 * s1;
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = warp; r < rows; r += nwarps) {
        const long long i = r / s1, j = r - (r / s1) * s1;
        const bool wrow = (T.wall[0] && i == 0) || (T.wall[1] && i == s0 - 1) || (T.wall[2] && j == 0) ||
                          (T.wall[3] && j == s1 - 1);
        const long long base = r * s2;
        for (long long k = lane; k < s2; k += 32) {
            const float v = D[base + k];
            bool within;
            if (T.thr_sq >= 0.0) {
                within = (double)v <= T.thr_sq;
            } else {
                const float dist = __fsqrt_rn(v);
                within = T.cmp64 ? ((double)dist <= T.r64) : (dist <= T.r32);
            }
            uint8_t o = within ? 0 : 1;
            if (wrow || (T.wall[4] && k == 0) || (T.wall[5] && k == s2 - 1))
                o = 0;
            out[base + k] = o;
        }
    }
}

struct Work {
    uint8_t *t1, *t2, *t3; // uint8 volumes
    uint8_t *E;            // morphology scratch
    float *A, *B;
    int *P;
    uint8_t *M, *mark; // per-block masks and marks of the binary selection
    int *err;
    unsigned long long *cnt; // scalar counter
    void *base;
};

static int work_alloc(Work &w, const int64_t *shape, size_t morph_bytes, cudaStream_t st)
{
    const size_t n = (size_t)shape[0] * shape[1] * shape[2];
    const size_t a = (n + 255) & ~(size_t)255;
    const size_t nb = (size_t)((shape[0] + 1) / 2) * ((shape[1] + 1) / 2) * ((shape[2] + 1) / 2);
    const size_t bb = (nb + 255) & ~(size_t)255;
    const size_t total = 3 * a + ((morph_bytes + 255) & ~(size_t)255) + a * 4 + 2 * bb + 512;
    PMG_TRY(scratch_alloc(&w.base, total, st));
    char *p = (char *)w.base;
    w.t1 = (uint8_t *)p;
    p += a;
    w.t2 = (uint8_t *)p;
    p += a;
    w.t3 = (uint8_t *)p;
    p += a;
    w.E = (uint8_t *)p;
    p += (morph_bytes + 255) & ~(size_t)255;
    w.P = (int *)p;
    p += a * 4;
    w.M = (uint8_t *)p;
    p += bb;
    w.mark = (uint8_t *)p;
    p += bb;
    w.err = (int *)p;
    w.cnt = (unsigned long long *)(p + 256);
    return PMG_OK;
}

// Step of every voxel in a growing eroded space: the first radius index whose
// threshold its capped squared distance exceeds (the thresholds never rise),
// read from a table over the capped values; wall planes never enter (255).
// One warp per (i, j) row.
__global__ void k_step_volume(const uint16_t *__restrict__ KC, uint8_t *__restrict__ S,
                              const uint8_t *__restrict__ tab, int tmax, long long s0, long long s1, long long s2,
                              unsigned walls)
{
    __shared__ uint8_t s_tab[kCapMaxT + 2];
    for (int v = threadIdx.x; v <= tmax; v += blockDim.x)
        s_tab[v] = tab[v];
    __syncthreads();
    const long long rows = s0 * s1;
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = warp; r < rows; r += nwarps) {
        const long long i = r / s1, j = r - (r / s1) * s1;
        const bool wrow = ((walls & 1u) && i == 0) || ((walls & 2u) && i == s0 - 1) || ((walls & 4u) && j == 0) ||
                          ((walls & 8u) && j == s1 - 1);
        const long long base = r * s2;
        for (long long k = lane; k < s2; k += 32) {
            const int v = min((int)KC[base + k], tmax);
            const bool wall = wrow || ((walls & 16u) && k == 0) || ((walls & 32u) && k == s2 - 1);
            S[base + k] = wall ? (uint8_t)255 : s_tab[v];
        }
    }
}

static void morph_split(Work &w, const int64_t *shape, const int32_t *bc, const int32_t *ext,
                        uint8_t *&E, float *&A, float *&B)
{
    long long nv = 1;
    for (int d = 0; d < 3; d++)
        nv *= shape[d] + (bc[2 * d] == PMG_BC_PERIODIC ? ext[2 * d] + ext[2 * d + 1] : 0);
    E = w.E;
    A = (float *)(w.E + (((size_t)nv + 255) & ~(size_t)255));
    B = A + nv;
}

static int count_sync(const uint8_t *img, const int64_t *shape, const int64_t *box, uint8_t value, Work &w,
                      cudaStream_t st, long long &out)
{
    PMG_CUDA(cudaMemsetAsync(w.cnt, 0, sizeof(unsigned long long), st));
    PMG_TRY(count_eq_async(img, shape, box, value, w.cnt, st));
    unsigned long long h = 0;
    PMG_CUDA(cudaMemcpyAsync(&h, w.cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    out = (long long)h;
    return PMG_OK;
}

// porosimetry.py:84-160 (mode="distance") into `out`.
static int porosimetry_run(const uint8_t *pm, uint8_t *out, const int64_t *shape, const int32_t *bc,
                           const int32_t *pad, const int32_t *ext_e, const int32_t *ext_d, const float *res,
                           double r_e, int cmp_e, double r_d, int cmp_d, int inlet, const uint8_t *mp,
                           const Boxes &Bx, Work &w, cudaStream_t st, double ball_e, double ball_d,
                           const float *De = nullptr, const uint16_t *KC = nullptr, int Te = -1,
                           bool m1_counted = false, GrowSel *g_er = nullptr, GrowSel *g_nw = nullptr,
                           const uint8_t *Sv = nullptr, int step = -1, int *orange = nullptr)
{
    // m1_counted: w.cnt[1] already holds count(mp == 1) (the drainage update
    // counts it); the inlet selection counts its kept voxels into w.cnt[0], and
    // both come back with one copy
    const long long n = shape[0] * shape[1] * shape[2];
    const int64_t all[6] = {0, shape[0], 0, shape[1], 0, shape[2]};
    uint8_t *E;
    float *A, *B;
    morph_split(w, shape, bc, ext_e, E, A, B);
    uint8_t *cur = w.t1;
    PMG_CUDA(cudaMemsetAsync(w.cnt, 0, sizeof(unsigned long long), st));
    if (g_er && g_nw && (KC || Sv) && inlet && mp && m1_counted) {
        // both selections grow along the curve: one pass writes the eroded
        // inlet-connected space constrained by the inlet-connected
        // non-wetting phase (when that phase exists, counted in w.cnt[1])
        PMG_TRY(grow_marks_pair(*g_er, Sv, step, KC, Te, *g_nw, mp, 1, shape, bc, pad, Bx.inlet, w.err, st));
        // the selection's x range (w.cnt[4]) limits the dilation to the planes
        // it can reach; the dilation's result range goes to orange
        int *xr = orange ? (int *)(w.cnt + 4) : nullptr;
        // the selection is written as per-block masks (w.M): the dilation's
        // row pass reads them directly (w.t2 receives bytes on other paths)
        PMG_TRY(grow_pair_select(*g_er, *g_nw, w.cnt + 1, w.M, shape, w.err, st, w.cnt, xr, true));
        // the dilation reads the kept count (w.cnt[0]) on the device: no
        // dilation of an empty selection, and no host round trip per radius
        morph_split(w, shape, bc, ext_d, E, A, B);
        return morph_run(w.t2, out, shape, bc, pad, ext_d, res, r_d, cmp_d, 1, E, A, B, st, ball_d, w.cnt, xr,
                         orange, w.M);
    }
    if (orange) {
        // the paths below write the whole result
        k_set_int2<<<1, 32, 0, st>>>(orange, 0, (int)shape[0] - 1);
        PMG_CHECK_LAUNCH();
    }
    if (KC && inlet) {
        if (g_er)
            PMG_TRY(select_grow_erode(*g_er, KC, Te, w.t2, shape, bc, pad, Bx.inlet, nullptr, PMG_SEL_INLET, w.err,
                                      st, w.cnt));
        else
            PMG_TRY(select_run_erode(KC, Te, w.t2, shape, bc, pad, Bx.inlet, nullptr, PMG_SEL_INLET, w.P, w.M,
                                     w.mark, w.err, st, w.cnt));
        cur = w.t2;
    } else if (De) {
        ErodeThr T;
        T.r32 = (float)r_e;
        T.r64 = r_e;
        T.cmp64 = cmp_e;
        T.thr_sq = ball_e;
        for (int q = 0; q < 6; q++)
            T.wall[q] = bc[q] == PMG_BC_WALL;
        const int ps__ = prof_begin("k_erode_from_edt", st);
        k_erode_from_edt<<<grid_for(shape[0] * shape[1] * 32, 256, 152LL * 64), 256, 0, st>>>(
            De, w.t1, shape[0], shape[1], shape[2], T);
        prof_end(ps__, (double)n * 5, st);
        PMG_CHECK_LAUNCH();
    } else {
        PMG_TRY(morph_run(pm, w.t1, shape, bc, pad, ext_e, res, r_e, cmp_e, 0, E, A, B, st, ball_e));
    }
    if (inlet && cur == w.t1) {
        // the eroded image holds only 0 and 1
        PMG_TRY(select_run_binary(w.t1, w.t2, 1, shape, bc, pad, Bx.inlet, nullptr, PMG_SEL_INLET, -1, w.P, w.M,
                                  w.mark, w.err, st, w.cnt));
        cur = w.t2;
    }
    long long c1 = 0, m1 = -1;
    if (inlet) {
        unsigned long long h[2] = {0, 0};
        PMG_CUDA(cudaMemcpyAsync(h, w.cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaStreamSynchronize(st));
        c1 = (long long)h[0];
        if (m1_counted)
            m1 = (long long)h[1];
    } else {
        PMG_TRY(count_sync(cur, shape, all, 1, w, st, c1));
    }
    if (c1 > 0) {
        if (mp) {
            if (m1 < 0)
                PMG_TRY(count_sync(mp, shape, all, 1, w, st, m1));
            if (m1 > 0) {
                if (g_nw)
                    PMG_TRY(select_grow_binary(*g_nw, mp, 1, w.t3, shape, bc, pad, Bx.inlet, nullptr,
                                               PMG_SEL_INLET, w.err, st));
                else
                    PMG_TRY(select_run_binary(mp, w.t3, 1, shape, bc, pad, Bx.inlet, nullptr, PMG_SEL_INLET, 1,
                                              w.P, w.M, w.mark, w.err, st));
                {
                    const int ps__ = prof_begin("k_constrain", st);
                    k_constrain<<<grid_for(n / 16 + 1, 256, 152LL * 32), 256, 0, st>>>(cur, w.t3, n);
                    prof_end(ps__, (double)n * 3, st);
                }
                PMG_CHECK_LAUNCH();
            }
        }
        morph_split(w, shape, bc, ext_d, E, A, B);
        PMG_TRY(morph_run(cur, out, shape, bc, pad, ext_d, res, r_d, cmp_d, 1, E, A, B, st, ball_d));
    } else if (cur != out) {
        PMG_CUDA(cudaMemcpyAsync(out, cur, (size_t)n, cudaMemcpyDeviceToDevice, st));
    }
    return PMG_OK;
}

static int ext_of(const int32_t *bc, const int32_t *pad, const int32_t *ratio, int32_t *ext)
{
    for (int d = 0; d < 3; d++)
        for (int s = 0; s < 2; s++) {
            const int b = bc[2 * d + s];
            ext[2 * d + s] = (b == PMG_BC_END || (b == PMG_BC_WALL && pad[2 * d + s] == 1)) ? 0 : ratio[d];
        }
    return PMG_OK;
}

static size_t max_morph_bytes(const int64_t *shape, const int32_t *bc, const int32_t *ext_a, const int32_t *ext_b)
{
    const size_t a = morph_scratch_bytes(shape, bc, ext_a), b = morph_scratch_bytes(shape, bc, ext_b);
    return a > b ? a : b;
}

static int check_common(const int64_t *shape, const int32_t *bc, const int32_t *pad)
{
    PMG_TRY(check_geometry(shape, bc, pad));
    return check_volume(shape);
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_porosimetry(const uint8_t *pm_img, const uint8_t *mp_img, uint8_t *out,
                               const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                               const int64_t inlet_box[6], const float res[3], double r_erode,
                               int32_t cmp_erode, const int32_t ratio_erode[3], double r_dilate,
                               int32_t cmp_dilate, const int32_t ratio_dilate[3], int32_t inlet,
                               double ball_erode, double ball_dilate, void *stream)
{
    PMG_TRY(check_common(shape, bc, pad));
    if (!pm_img || !out || !res || !ratio_erode || !ratio_dilate) {
        set_error("pmg_porosimetry: null argument");
        return PMG_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    int32_t ext_e[6], ext_d[6];
    ext_of(bc, pad, ratio_erode, ext_e);
    ext_of(bc, pad, ratio_dilate, ext_d);
    Boxes Bx{};
    for (int q = 0; q < 6; q++) {
        Bx.inlet[q] = inlet_box ? inlet_box[q] : -1;
        Bx.outlet[q] = -1;
    }
    Work w{};
    PMG_TRY(work_alloc(w, shape, max_morph_bytes(shape, bc, ext_e, ext_d), st));
    PMG_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), st));
    int s = porosimetry_run(pm_img, out, shape, bc, pad, ext_e, ext_d, res, r_erode, cmp_erode, r_dilate,
                            cmp_dilate, inlet, mp_img, Bx, w, st, ball_erode, ball_dilate);
    if (s == PMG_OK)
        s = check_err(w.err, st);
    int s2 = scratch_free(w.base, st);
    return s != PMG_OK ? s : s2;
}

extern "C" int pmg_drainage_ext(const uint8_t *pm_img, uint8_t *mp_img, const int64_t shape[3],
                                const int32_t bc[6], const int32_t pad[6], const int32_t rpad[6],
                                const int64_t own_box[6], const int64_t inlet_box[6],
                                const int64_t outlet_box[6], const float res[3], int32_t n_radii,
                                const double *radii, const int32_t *active, const int32_t *ratios,
                                const double *ball_erode, const double *ball_dilate, int64_t *counts,
                                const double *radii_dilate, const int32_t *ratios_dilate, void *stream)
{
    if (!radii_dilate)
        radii_dilate = radii;
    if (!ratios_dilate)
        ratios_dilate = ratios;
    PMG_TRY(check_common(shape, bc, pad));
    if (!pm_img || !mp_img || !rpad || !own_box || !res || !counts || n_radii < 0 ||
        (n_radii > 0 && (!radii || !active || !ratios))) {
        set_error("pmg_drainage: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_box6(shape, own_box));
    for (int q = 0; q < 6; q++)
        if (rpad[q] < 0) {
            set_error("pmg_drainage: negative reservoir pad");
            return PMG_EINVAL;
        }
    cudaStream_t st = as_stream(stream);
    const long long n = shape[0] * shape[1] * shape[2];
    Boxes Bx{};
    for (int q = 0; q < 6; q++) {
        Bx.own[q] = own_box[q];
        Bx.inlet[q] = inlet_box ? inlet_box[q] : -1;
        Bx.outlet[q] = outlet_box ? outlet_box[q] : -1;
        Bx.rpad[q] = rpad[q];
    }
    size_t mb = 0;
    for (int k = 0; k < n_radii; k++) {
        int32_t ext[6];
        ext_of(bc, pad, ratios + 3 * k, ext);
        size_t b = morph_scratch_bytes(shape, bc, ext);
        if (b > mb)
            mb = b;
        ext_of(bc, pad, ratios_dilate + 3 * k, ext);
        b = morph_scratch_bytes(shape, bc, ext);
        if (b > mb)
            mb = b;
    }
    Work w{};
    PMG_TRY(work_alloc(w, shape, mb, st));
    PMG_CUDA(cudaMemsetAsync(w.err, 0, sizeof(int), st));
    uint8_t *morph = nullptr;
    unsigned long long *d_counts = nullptr;
    // Without periodic axes the erosion's extended image is the same for every
    // radius (no wrap extension), so its EDT is computed once and thresholded
    // per radius -- the same values the per-radius EDT would produce.
    const bool reuse_erosion = bc[0] != PMG_BC_PERIODIC && bc[2] != PMG_BC_PERIODIC && bc[4] != PMG_BC_PERIODIC;
    float *De = nullptr;
    int unit_res = -1;
    for (int k = 0; k < n_radii; k++)
        if (active[k]) {
            unit_res = (ball_erode && ball_erode[k] >= 0.0) ? 1 : 0;
            break;
        }
    int s = PMG_OK;
    // Isotropic power-of-two voxels: the erosion EDT is kept as a capped
    // integer volume (uint16, values above the largest erosion bound clamp)
    // and each radius's erosion "E > T" is read off it inside the inlet
    // selection -- no eroded image is written.
    uint16_t *KC = nullptr;
    int Tcap = 0;
    std::vector<int> Te((size_t)n_radii, -1);
    if (reuse_erosion && unit_res >= 0) {
        const float unit[3] = {1.0f, 1.0f, 1.0f};
        const float *r = unit_res ? unit : res;
        const pmg_axis_cfg plain = {0, 0, 0, 0, 1, 0, 0, 0};
        bool ok = r[0] == r[1] && r[1] == r[2];
        for (int d = 0; d < 3 && ok; d++)
            ok = exact_path_ok(r[d], plain, (int)shape[d]);
        Tcap = 0;
        for (int k = 0; k < n_radii && ok; k++) {
            if (!active[k])
                continue;
            MorphEpi me{};
            me.r32 = (float)radii[k];
            me.r64 = radii[k];
            me.cmp64 = 1;
            me.thr_sq = ball_erode ? ball_erode[k] : -1.0;
            Te[(size_t)k] = morph_threshold(me, r[0] * r[0], kCapMaxT + 1);
            ok = Te[(size_t)k] >= 0 && Te[(size_t)k] <= kCapMaxT;
            Tcap = Te[(size_t)k] > Tcap ? Te[(size_t)k] : Tcap;
        }
        if (ok) {
            s = scratch_alloc((void **)&KC, (size_t)n * sizeof(uint16_t), st);
            int nonbinary = 0;
            if (s == PMG_OK) {
                uint8_t *E;
                float *A, *B;
                const int32_t zero_ext[6] = {0, 0, 0, 0, 0, 0};
                morph_split(w, shape, bc, zero_ext, E, A, B);
                s = erosion_cap_run(pm_img, KC, shape, bc, pad, Tcap, E, (uint16_t *)A, (uint16_t *)B,
                                    (int *)((char *)w.err + 128), &nonbinary, st);
            }
            if (s == PMG_OK && nonbinary) {
                s = scratch_free(KC, st);
                KC = nullptr;
            }
        }
    }
    if (s == PMG_OK && !KC && reuse_erosion && unit_res >= 0) {
        s = scratch_alloc((void **)&De, (size_t)n * sizeof(float), st);
        if (s == PMG_OK) {
            uint8_t *E;
            float *A, *B;
            const int32_t zero_ext[6] = {0, 0, 0, 0, 0, 0};
            morph_split(w, shape, bc, zero_ext, E, A, B);
            s = erosion_edt_run(pm_img, De, shape, bc, pad, res, unit_res, E, A, st);
        }
    }
    // The non-wetting phase only grows along the curve, and so does the eroded
    // pore space when the thresholds of the active radii never rise: both
    // selections keep their block union-find from one radius to the next.
    GrowSel g_er, g_nw;
    bool grow_er = KC != nullptr;
    {
        int last = INT_MAX;
        for (int k = 0; k < n_radii && grow_er; k++)
            if (active[k]) {
                grow_er = Te[(size_t)k] <= last;
                last = Te[(size_t)k];
            }
    }
    // the growing eroded space as one byte per voxel: the radius index at
    // which the voxel enters (the capped distances are not needed after it)
    uint8_t *Sv = nullptr;
    if (s == PMG_OK && grow_er && n_radii <= 254) {
        std::vector<uint8_t> tab((size_t)Tcap + 2, 255);
        for (int v = 0; v <= Tcap + 1; v++)
            for (int k = 0; k < n_radii; k++)
                if (active[k] && Te[(size_t)k] < v) {
                    tab[(size_t)v] = (uint8_t)k;
                    break;
                }
        uint8_t *dtab = nullptr;
        s = scratch_alloc((void **)&Sv, (size_t)n + 256 + tab.size(), st);
        if (s == PMG_OK) {
            dtab = Sv + (((size_t)n + 255) & ~(size_t)255);
            s = cudaMemcpyAsync(dtab, tab.data(), tab.size(), cudaMemcpyHostToDevice, st) == cudaSuccess
                    ? PMG_OK
                    : PMG_ECUDA;
        }
        if (s == PMG_OK) {
            unsigned walls = 0;
            for (int q = 0; q < 6; q++)
                walls |= (bc[q] == PMG_BC_WALL ? 1u : 0u) << q;
            const int ps__ = prof_begin("k_step_volume", st);
            k_step_volume<<<grid_for(shape[0] * shape[1] * 32, 256, 152LL * 64), 256, 0, st>>>(
                KC, Sv, dtab, Tcap + 1, shape[0], shape[1], shape[2], walls);
            prof_end(ps__, (double)n * 3, st);
            // (a copy from pageable memory has read the table when it returns)
            s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
        }
        if (s == PMG_OK) {
            s = scratch_free(KC, st);
            KC = nullptr;
        }
    }
    void *grow_mem = nullptr;
    const size_t gb = grow_sel_bytes(shape), sb = shrink_sel_bytes(shape);
    if (s == PMG_OK)
        s = scratch_alloc(&grow_mem, gb * (grow_er ? 2 : 1) + sb, st);
    ShrinkSel g_w;
    if (s == PMG_OK)
        shrink_sel_init(g_w, (char *)grow_mem + gb * (grow_er ? 2 : 1), shape);
    if (s == PMG_OK) {
        grow_sel_init(g_nw, grow_mem, shape);
        g_nw.unite_label = "k_grow_unite[nonwetting]";
        g_nw.unite_units = kUnitsGrowUniteB;
        if (grow_er) {
            grow_sel_init(g_er, (char *)grow_mem + gb, shape);
            g_er.unite_label = "k_grow_unite[eroded]";
            g_er.unite_units = kUnitsGrowUniteA;
        }
    }
    // the blocks of the eroded space that grow at each radius, listed once
    void *lists_mem = nullptr;
    if (s == PMG_OK && Sv)
        s = step_lists_build(g_er, Sv, shape, n_radii, &lists_mem, st);
    if (s == PMG_OK)
        s = scratch_alloc((void **)&morph, (size_t)n, st);
    if (s == PMG_OK)
        s = scratch_alloc((void **)&d_counts, sizeof(unsigned long long) * (size_t)(n_radii + 1), st);
    if (s == PMG_OK)
        s = cudaMemsetAsync(d_counts, 0, sizeof(unsigned long long) * (size_t)(n_radii + 1), st) == cudaSuccess
                ? PMG_OK
                : PMG_ECUDA;
    // count(mp == 1) for the first radius; the update kernel keeps it current
    const int64_t whole[6] = {0, shape[0], 0, shape[1], 0, shape[2]};
    if (s == PMG_OK)
        s = cudaMemsetAsync(w.cnt + 1, 0, sizeof(unsigned long long), st) == cudaSuccess ? PMG_OK : PMG_ECUDA;
    if (s == PMG_OK)
        s = count_eq_async(mp_img, shape, whole, 1, w.cnt + 1, st);
    // After the first update (which refills the reservoir slabs), a radius can
    // change only voxels within the dilation's x range: the update visits that
    // range alone and keeps the saturation counts as running totals
    // (w.cnt[10], w.cnt[11]) from the changes it counts (w.cnt[8], w.cnt[9]).
    int *orange = (int *)(w.cnt + 5);
    bool full_done = false;
    for (int k = 0; k < n_radii && s == PMG_OK; k++) {
        if (!active[k] && full_done) {
            // no dilation: nothing changes, the totals stand
            PMG_CUDA(cudaMemsetAsync(w.cnt + 8, 0, 2 * sizeof(unsigned long long), st));
            s = drain_totals(true, w.cnt + 8, w.cnt + 9, w.cnt + 10, d_counts + k, w.cnt + 1, st);
            continue;
        }
        if (active[k]) {
            int32_t ext[6], ext_d[6];
            ext_of(bc, pad, ratios + 3 * k, ext);
            ext_of(bc, pad, ratios_dilate + 3 * k, ext_d);
            // the probe radii are numpy float64: compare in float64
            s = porosimetry_run(pm_img, morph, shape, bc, pad, ext, ext_d, res, radii[k], 1, radii_dilate[k], 1, 1,
                                mp_img,
                                Bx, w, st, ball_erode ? ball_erode[k] : -1.0, ball_dilate ? ball_dilate[k] : -1.0,
                                De, KC, Te[(size_t)k], true, grow_er ? &g_er : nullptr, &g_nw, Sv, k, orange);
        } else {
            s = cudaMemsetAsync(morph, 0, (size_t)n, st) == cudaSuccess ? PMG_OK : PMG_ECUDA;
        }
        if (s != PMG_OK)
            break;
        // wetting phase connected to the outlet (its union-find and marks
        // only; tiles the last update left alone keep their tile-local
        // parents), then the
        // update on blocks, which also brings the non-wetting phase's growing
        // selection and the wetting phase's masks and tile flags up to date
        s = shrink_marks_binary(g_w, mp_img, 2, shape, bc, pad, nullptr, Bx.outlet, w.err, st);
        if (s != PMG_OK)
            break;
        GrowSel *gn = nullptr;
        if (g_nw.built) {
            if (g_nw.pending) {
                // the last update's list was never consumed: rebuild instead
                g_nw.built = false;
                g_nw.pending = false;
            } else {
                PMG_CUDA(cudaMemsetAsync(g_nw.count, 0, sizeof(int), st));
                gn = &g_nw;
            }
        }
        PMG_CUDA(cudaMemsetAsync(w.cnt + 8, 0, 2 * sizeof(unsigned long long), st));
        s = drain_update_blocks(mp_img, morph, shape, g_w.P, g_w.M, g_w.mark, Bx, gn, w.cnt + 8, w.cnt + 9, w.err,
                                st, g_w.dirty, active[k] ? orange : nullptr, full_done);
        if (s == PMG_OK)
            s = drain_totals(full_done, w.cnt + 8, w.cnt + 9, w.cnt + 10, d_counts + k, w.cnt + 1, st);
        if (s != PMG_OK)
            break;
        full_done = true;
        if (gn)
            g_nw.pending = true;
    }
    // union-find iteration caps are checked once per curve: the status word
    // is only ever set, never cleared, during the sweep
    if (s == PMG_OK)
        s = check_err(w.err, st);
    if (s == PMG_OK && n_radii > 0) {
        std::vector<unsigned long long> h((size_t)n_radii);
        PMG_CUDA(cudaMemcpyAsync(h.data(), d_counts, sizeof(unsigned long long) * (size_t)n_radii,
                                 cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaStreamSynchronize(st));
        for (int k = 0; k < n_radii; k++)
            counts[k] = (int64_t)h[(size_t)k];
    }
    scratch_free(lists_mem, st);
    scratch_free(grow_mem, st);
    scratch_free(Sv, st);
    scratch_free(De, st);
    scratch_free(KC, st);
    scratch_free(morph, st);
    scratch_free(d_counts, st);
    int s2 = scratch_free(w.base, st);
    return s != PMG_OK ? s : s2;
}

extern "C" int pmg_drainage(const uint8_t *pm_img, uint8_t *mp_img, const int64_t shape[3],
                            const int32_t bc[6], const int32_t pad[6], const int32_t rpad[6],
                            const int64_t own_box[6], const int64_t inlet_box[6],
                            const int64_t outlet_box[6], const float res[3], int32_t n_radii,
                            const double *radii, const int32_t *active, const int32_t *ratios,
                            const double *ball_erode, const double *ball_dilate, int64_t *counts,
                            void *stream)
{
    return pmg_drainage_ext(pm_img, mp_img, shape, bc, pad, rpad, own_box, inlet_box, outlet_box, res, n_radii,
                            radii, active, ratios, ball_erode, ball_dilate, counts, nullptr, nullptr, stream);
}
