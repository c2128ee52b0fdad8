// Morphological addition / subtraction on the GPU (EDT path).
//
// The reference (src/pmmoto/filters/morphological_operators.py:103-228)
// wrap-pads the padded subdomain by ceil(r/res) voxels on periodic faces
// (communication.update_extended_buffer, core/communication.py:121-157),
// zeroes wall planes, runs a non-periodic EDT of the extended image (or of its
// logical_not for addition), thresholds d <= r, removes the extension and
// zeroes wall planes again.  Here the extended image is produced by one
// gather kernel whose periodic axes read the own region modulo its length --
// the halo exchange becomes index arithmetic -- and the threshold, unpadding
// and wall rule are fused into the last envelope pass, which writes the
// uint8 result directly.
#include "edt_internal.cuh"

namespace pmg {

struct ExtAxis {
    int periodic;
    int own_lo, own_len; // own region of the padded axis
    int ext_lo;          // low-side extension
    int wall_lo, wall_hi;
    long long S, X;      // padded and extended lengths
};

struct ExtGeo {
    ExtAxis ax[3];
};

__device__ __forceinline__ long long src_index(const ExtAxis &a, long long x, bool &zero)
{
    const long long p = x - a.ext_lo; // coordinate in the padded image
    if (a.periodic) {
        long long q = (x - (a.own_lo + a.ext_lo)) % a.own_len;
        if (q < 0)
            q += a.own_len;
        return q + a.own_lo;
    }
    if ((a.wall_lo && p == 0) || (a.wall_hi && p == a.S - 1))
        zero = true;
    return p;
}

// E[x] = img[wrap(x)] (0 on wall planes); logical_not for addition.  One warp
// per (x0, x1) row of the extended volume: the row's source row and wall state
// are resolved once, lanes walk x2.
__global__ void k_extend(const uint8_t *__restrict__ img, uint8_t *__restrict__ ext, ExtGeo G,
                         int logical_not, int *nonbinary)
{
    const long long X1 = G.ax[1].X, X2 = G.ax[2].X;
    const long long rows = G.ax[0].X * X1;
    const long long S1 = G.ax[1].S, S2 = G.ax[2].S;
    const ExtAxis &a2 = G.ax[2];
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long q0 = a2.own_lo + a2.ext_lo; // x2 of the first own voxel
    for (long long r = warp; r < rows; r += nwarps) {
        const long long x0 = r / X1, x1 = r - (r / X1) * X1;
        bool zero_row = false;
        const long long s0 = src_index(G.ax[0], x0, zero_row);
        const long long s1 = src_index(G.ax[1], x1, zero_row);
        const uint8_t *src = img + (s0 * S1 + s1) * S2;
        uint8_t *dst = ext + r * X2;
        for (long long x2 = lane; x2 < X2; x2 += 32) {
            long long s2;
            bool zero = zero_row;
            if (a2.periodic) {
                // the extension never exceeds the own length, so one wrap suffices
                s2 = x2 - q0;
                if (s2 < 0)
                    s2 += a2.own_len;
                else if (s2 >= a2.own_len)
                    s2 -= a2.own_len;
                if (s2 < 0 || s2 >= a2.own_len) // extensions beyond one period
                    s2 = src_index(a2, x2, zero);
                else
                    s2 += a2.own_lo;
            } else {
                s2 = x2;
                if ((a2.wall_lo && x2 == 0) || (a2.wall_hi && x2 == S2 - 1))
                    zero = true;
            }
            uint8_t v = zero ? (uint8_t)0 : src[s2];
            if (logical_not)
                v = v == 0 ? 1 : 0;
            else if (v > 1 && nonbinary)
                *nonbinary = 1;
            dst[x2] = v;
        }
    }
}

// One byte per voxel from per-block masks (bit (x * 2 + y) * 2 + z of the
// block over the ceil-halved shape), one thread per block.
__global__ void k_blocks_to_bytes(const uint8_t *__restrict__ blk, uint8_t *__restrict__ out, long long s0,
                                  long long s1, long long s2)
{
    const long long b1 = (s1 + 1) / 2, b2 = (s2 + 1) / 2, nb = (s0 + 1) / 2 * b1 * b2;
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nb;
         b += (long long)gridDim.x * blockDim.x) {
        const long long r = b / b2, c2 = b - r * b2, c0 = r / b1, c1 = r - c0 * b1;
        const unsigned m = blk[b];
        for (int x = 0; x < 2; x++)
            for (int y = 0; y < 2; y++) {
                const long long i = 2 * c0 + x, j = 2 * c1 + y;
                if (i >= s0 || j >= s1)
                    continue;
                uint8_t *row = out + (i * s1 + j) * s2;
                for (int z = 0; z < 2; z++)
                    if (2 * c2 + z < s2)
                        row[2 * c2 + z] = (uint8_t)((m >> ((x * 2 + y) * 2 + z)) & 1);
            }
    }
}

int morph_run(const uint8_t *img, uint8_t *out, const int64_t *shape, const int32_t *bc,
              const int32_t *pad, const int32_t *ext, const float *res, double radius, int cmp64,
              int dilate, uint8_t *E, float *A, float *B, cudaStream_t st, double thr_sq,
              const unsigned long long *gate, const int *xr, int *orange, const uint8_t *blk)
{
    // orange: on the paths below that ignore xr the whole result is written
    if (orange) {
        k_set_int2<<<1, 32, 0, st>>>(orange, 0, (int)shape[0] - 1);
        PMG_CHECK_LAUNCH();
    }
    ExtGeo G;
    int64_t X[3];
    for (int d = 0; d < 3; d++) {
        ExtAxis &a = G.ax[d];
        a.periodic = bc[2 * d] == PMG_BC_PERIODIC;
        a.own_lo = pad[2 * d];
        a.own_len = (int)(shape[d] - pad[2 * d] - pad[2 * d + 1]);
        a.ext_lo = a.periodic ? ext[2 * d] : 0;
        a.wall_lo = bc[2 * d] == PMG_BC_WALL;
        a.wall_hi = bc[2 * d + 1] == PMG_BC_WALL;
        a.S = shape[d];
        a.X = shape[d] + (a.periodic ? ext[2 * d] + ext[2 * d + 1] : 0);
        X[d] = a.X;
        if (a.periodic && a.own_len <= 0) {
            set_error("morph: empty own region on periodic axis %d", d);
            return PMG_EINVAL;
        }
    }
    const long long total = (long long)X[0] * X[1] * X[2];

    pmg_axis_cfg plain = {0, 0, 0, 0, 1, 0, 0, 0};
    MorphEpi me{};
    me.out = out;
    me.o0 = shape[0];
    me.o1 = shape[1];
    me.o2 = shape[2];
    me.e0 = G.ax[0].ext_lo;
    me.e1 = G.ax[1].ext_lo;
    me.e2 = G.ax[2].ext_lo;
    for (int d = 0; d < 3; d++) {
        me.wall[2 * d] = G.ax[d].wall_lo;
        me.wall[2 * d + 1] = G.ax[d].wall_hi;
    }
    me.r32 = (float)radius;
    me.r64 = radius;
    me.cmp64 = cmp64;
    me.dilate = dilate;
    me.thr_sq = thr_sq;
    // the ball of the FFT modes is measured in voxels: unit resolution keeps
    // every squared distance an exact integer in float32
    const float unit[3] = {1.0f, 1.0f, 1.0f};
    if (thr_sq >= 0.0)
        res = unit;

    // Isotropic power-of-two voxels make every squared distance an exact
    // integer multiple of res^2, and the reference's threshold becomes
    // "E <= T" for one integer T: the middle pass then only needs heights up
    // to T and the last pass is a union of intervals.
    int T = INT_MIN;
    if (res[0] == res[1] && res[1] == res[2] && exact_path_ok(res[1], plain, (int)X[1]) &&
        exact_path_ok(res[2], plain, (int)X[2])) {
        const int nm = (int)(X[1] > X[2] ? X[1] : X[2]);
        const int lim = (1 << 24) - nm * nm - 1;
        const int t = morph_threshold(me, res[2] * res[2], lim);
        if (t < lim)
            T = t;
    }

    const bool cap = T != INT_MIN && cap_path_ok(res, X, T);
    const bool any_per = G.ax[0].periodic || G.ax[1].periodic || G.ax[2].periodic;
    if (cap && dilate && !any_per) // the row pass reads the image (or its block masks) itself
        return morph_cap_run(img, (uint16_t *)A, (uint16_t *)B, X, T, me, st, 1, gate, xr, orange, blk);
    if (blk) {
        // the paths below read one byte per voxel: img is the caller's scratch
        const long long nb = (shape[0] + 1) / 2 * ((shape[1] + 1) / 2) * ((shape[2] + 1) / 2);
        const int ps__ = prof_begin("k_blocks_to_bytes", st);
        k_blocks_to_bytes<<<grid_for(nb, 256, 152LL * 32), 256, 0, st>>>(blk, const_cast<uint8_t *>(img), shape[0],
                                                                          shape[1], shape[2]);
        prof_end(ps__, (double)nb * 9, st);
        PMG_CHECK_LAUNCH();
    }
    if (gate) {
        // the other paths read the seed count on the host: an empty dilation
        // source gives zeros
        unsigned long long h = 0;
        PMG_CUDA(cudaMemcpyAsync(&h, gate, sizeof(h), cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaStreamSynchronize(st));
        if (h == 0) {
            PMG_CUDA(cudaMemsetAsync(out, 0, (size_t)shape[0] * shape[1] * shape[2], st));
            return PMG_OK;
        }
    }

    // last int of B: "the image holds a value above 1" (erosion only; the
    // capped pipeline needs a binary image)
    int *flag = dilate ? nullptr : (int *)(B + total) - 1;
    if (flag)
        PMG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    {
        const int ps__ = prof_begin("k_extend", st);
        k_extend<<<grid_for(X[0] * X[1] * 32, 256, 152LL * 64), 256, 0, st>>>(img, E, G, dilate, flag);
        prof_end(ps__, (double)total * 2, st);
    }
    PMG_CHECK_LAUNCH();

    if (cap) {
        int nonbin = 0;
        if (flag) {
            PMG_CUDA(cudaMemcpyAsync(&nonbin, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
            PMG_CUDA(cudaStreamSynchronize(st));
        }
        if (!nonbin)
            return morph_cap_run(E, (uint16_t *)A, (uint16_t *)B, X, T, me, st);
    }

    PMG_TRY(launch_pass0(E, A, all_lines(X, 0), res[0], plain, st));
    Lines L1 = all_lines(X, 1); // lines over (i, k): keep i inside the unextended range
    L1.b1lo = me.e0;
    L1.nb1 = (int)shape[0];
    PMG_TRY(launch_envelope(A, B, L1, res[1], plain, 4, PMG_EDT_SQUARED, me, st, T == INT_MIN ? INT_MAX : T));
    Lines L2 = all_lines(X, 2); // lines over (i, j): both inside the unextended range
    L2.b1lo = me.e0;
    L2.nb1 = (int)shape[0];
    L2.b2lo = me.e1;
    L2.nb2 = (int)shape[1];
    if (T != INT_MIN)
        return launch_env_thresh(B, L2, res[2], T, me, st);
    PMG_TRY(launch_envelope(B, nullptr, L2, res[2], plain, 4, PMG_EDT_MORPH, me, st));
    return PMG_OK;
}

// Squared EDT of the unextended erosion image (wall planes zeroed), for
// subdomains without periodic axes, where every radius sees this same image:
// E is uint8 scratch of the volume, A float scratch, D receives the result.
// unit_res selects the voxel-unit distances of the FFT-ball modes.
int erosion_edt_run(const uint8_t *img, float *D, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, const float *res, int unit_res, uint8_t *E, float *A,
                    cudaStream_t st)
{
    ExtGeo G;
    for (int d = 0; d < 3; d++) {
        ExtAxis &a = G.ax[d];
        if (bc[2 * d] == PMG_BC_PERIODIC) {
            set_error("erosion EDT reuse needs a subdomain without periodic axes");
            return PMG_EINVAL;
        }
        a.periodic = 0;
        a.own_lo = pad[2 * d];
        a.own_len = (int)(shape[d] - pad[2 * d] - pad[2 * d + 1]);
        a.ext_lo = 0;
        a.wall_lo = bc[2 * d] == PMG_BC_WALL;
        a.wall_hi = bc[2 * d + 1] == PMG_BC_WALL;
        a.S = shape[d];
        a.X = shape[d];
    }
    {
        const int ps__ = prof_begin("k_extend", st);
        k_extend<<<grid_for(shape[0] * shape[1] * 32, 256, 152LL * 64), 256, 0, st>>>(img, E, G, 0, nullptr);
        prof_end(ps__, (double)shape[0] * shape[1] * shape[2] * 2, st);
    }
    PMG_CHECK_LAUNCH();
    const float unit[3] = {1.0f, 1.0f, 1.0f};
    const float *r = unit_res ? unit : res;
    pmg_axis_cfg plain[3] = {{0, 0, 0, 0, 1, 0, 0, 0}, {0, 0, 0, 0, 1, 0, 0, 0}, {0, 0, 0, 0, 1, 0, 0, 0}};
    return edt3d_run(E, D, A, shape, r, plain, 4, PMG_EDT_SQUARED, st);
}

// Capped integer squared EDT of the same erosion image (isotropic power-of-two
// voxels, no periodic axes): KC = min(E, Tcap + 1) in units of res^2, uint16.
// The pipeline needs a binary image; *nonbinary reports an image with values
// above 1 (KC is then not written and the caller takes the float path).
int erosion_cap_run(const uint8_t *img, uint16_t *KC, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, int Tcap, uint8_t *E, uint16_t *KA, uint16_t *KB, int *flag,
                    int *nonbinary, cudaStream_t st)
{
    ExtGeo G;
    for (int d = 0; d < 3; d++) {
        ExtAxis &a = G.ax[d];
        if (bc[2 * d] == PMG_BC_PERIODIC) {
            set_error("erosion EDT reuse needs a subdomain without periodic axes");
            return PMG_EINVAL;
        }
        a.periodic = 0;
        a.own_lo = pad[2 * d];
        a.own_len = (int)(shape[d] - pad[2 * d] - pad[2 * d + 1]);
        a.ext_lo = 0;
        a.wall_lo = bc[2 * d] == PMG_BC_WALL;
        a.wall_hi = bc[2 * d + 1] == PMG_BC_WALL;
        a.S = shape[d];
        a.X = shape[d];
    }
    PMG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    {
        const int ps__ = prof_begin("k_extend", st);
        k_extend<<<grid_for(shape[0] * shape[1] * 32, 256, 152LL * 64), 256, 0, st>>>(img, E, G, 0, flag);
        prof_end(ps__, (double)shape[0] * shape[1] * shape[2] * 2, st);
    }
    PMG_CHECK_LAUNCH();
    int h = 0;
    PMG_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    *nonbinary = h;
    if (h)
        return PMG_OK;
    return edt_cap_run(E, KA, KB, KC, shape, Tcap, st);
}

size_t morph_scratch_bytes(const int64_t *shape, const int32_t *bc, const int32_t *ext)
{
    long long n = 1;
    for (int d = 0; d < 3; d++)
        n *= shape[d] + (bc[2 * d] == PMG_BC_PERIODIC ? ext[2 * d] + ext[2 * d + 1] : 0);
    // uint8 extended image (256-byte aligned) + two float32 buffers
    return (((size_t)n + 255) & ~(size_t)255) + 2 * (size_t)n * sizeof(float);
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_morph(const uint8_t *img, uint8_t *out, const int64_t shape[3],
                         const int32_t bc[6], const int32_t pad[6], const int32_t ext[6],
                         const float res[3], double radius, int32_t cmp64, int32_t dilate,
                         double ball_sq, void *stream)
{
    if (!img || !out || !shape || !bc || !pad || !ext || !res) {
        set_error("pmg_morph: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geometry(shape, bc, pad));
    for (int d = 0; d < 3; d++) {
        if (shape[d] <= 0) {
            set_error("pmg_morph: shape[%d] must be positive", d);
            return PMG_EINVAL;
        }
        const long long X = shape[d] + (bc[2 * d] == PMG_BC_PERIODIC ? ext[2 * d] + ext[2 * d + 1] : 0);
        if (X > PMG_MAX_LINE) {
            set_error("pmg_morph: extended axis %d length %lld exceeds %d", d, X, PMG_MAX_LINE);
            return PMG_ERANGE;
        }
        if (ext[2 * d] < 0 || ext[2 * d + 1] < 0) {
            set_error("pmg_morph: negative extension");
            return PMG_EINVAL;
        }
    }
    cudaStream_t st = as_stream(stream);
    const size_t bytes = morph_scratch_bytes(shape, bc, ext);
    void *buf = nullptr;
    PMG_TRY(scratch_alloc(&buf, bytes, st));
    long long nvox = 1;
    for (int d = 0; d < 3; d++)
        nvox *= shape[d] + (bc[2 * d] == PMG_BC_PERIODIC ? ext[2 * d] + ext[2 * d + 1] : 0);
    uint8_t *E = (uint8_t *)buf;
    float *A = (float *)((char *)buf + (((size_t)nvox + 255) & ~(size_t)255));
    float *B = A + nvox;
    int s = morph_run(img, out, shape, bc, pad, ext, res, radius, cmp64, dilate, E, A, B, st, ball_sq, nullptr,
                      nullptr, nullptr, nullptr);
    int s2 = scratch_free(buf, st);
    return s != PMG_OK ? s : s2;
}
