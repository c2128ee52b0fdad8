// Learned radius schedule: the small 3-D CNN that predicts a drainage
// curve from a downsampled distance field.  No counterpart in the
// reference (its drainage loop, equilibrium_distribution.py:93-128, sweeps
// every radius); the network only proposes which radii the exact loop
// evaluates.
//
// Convolutions (3x3x3, stride 2, padding 1, channels-last bf16 activations)
// are implicit GEMMs on the 5th-generation tensor cores:
//
//   forward   D[pos_out, c_out] = sum_{tap, c_in} X[pos_in(pos_out, tap), c_in] W[c_out, tap, c_in]
//   dgrad     D[pos_in, c_in]   = sum_{tap, c_out} dZ[pos_out(pos_in, tap), c_out] W[c_out, tap, c_in]
//   wgrad     D[(tap, c_in), c_out] = sum_{pos_out} X[pos_in(pos_out, tap), c_in] dZ[pos_out, c_out]
//
// One CTA of 128 threads computes a 128 x N tile (N = 16, 32 or 64 output
// columns) with the fp32 accumulator in tensor memory.  The K loop runs in
// chunks of 64 bf16 (one 128-byte row per tile row): all threads gather the
// chunk's operands from global memory (the im2col gather, zero outside the
// volume) into shared memory in the 128-byte-swizzled K-major layout, one
// elected thread issues four tcgen05.mma (K = 16 each) and commits them to
// the stage's mbarrier, and the next chunk is gathered into another of
// three stages meanwhile.  The epilogue reads the accumulator with
// tcgen05.ld (thread t owns row t) and applies bias + ReLU (forward), the
// ReLU mask of the layer below (dgrad) or an fp32 atomic add into the
// weight gradient (wgrad, split over K across CTAs).
//
// Every mbarrier wait has a time limit (about 1 s of %globaltimer); a wait
// that runs out records an error code, the CTA waits (again bounded) for its
// own MMAs, frees its tensor memory and returns.
#include <algorithm>
#include <cmath>

#include <cuda_bf16.h>

#include "pmg_common.cuh"

namespace pmg {
namespace cnn {

constexpr int kBM = 128;    // tile rows = TMEM lanes
constexpr int kBK = 64;     // K elements per chunk (128 bytes of bf16)
constexpr int kStages = 3;  // shared-memory pipeline depth
constexpr int kThreads = 128;
constexpr unsigned long long kWaitNs = 1000000000ull; // 1 s

// ---- PTX wrappers -----------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long gtime()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *b, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(b)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity)
{
    if (mbar_try(b, parity))
        return true;
    const unsigned long long t0 = gtime();
    while (!mbar_try(b, parity))
        if (gtime() - t0 > kWaitNs)
            return false;
    return true;
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, int ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, int ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D(tmem) (+)= A(smem) * B(smem)^T, bf16 inputs, fp32 accumulate.
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                 "l"(a), "l"(b), "r"(idesc), "r"(acc)
                 : "memory");
}

// Arrive on the mbarrier once all tcgen05 operations this thread issued
// before have completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

// ---- layouts and descriptors ------------------------------------------------

// Byte offset of the 16-byte chunk j (of 8) of row r in a tile stored K-major
// with the 128-byte swizzle: rows of 128 bytes, groups of 8 rows 1024 bytes
// apart, chunk index XORed with the row's position in its group.
__device__ __forceinline__ uint32_t sw128(int r, int j)
{
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((j ^ (r & 7)) << 4));
}

// Shared-memory matrix descriptor of a K-major, 128-byte-swizzled tile
// starting at byte address addr (tile base 1024-aligned; addr may be offset
// by 32-byte K steps inside the first row): start address >> 4, leading
// byte offset 16 (unused by this layout), stride byte offset 1024 (8-row
// groups), descriptor version 1, swizzle mode 2 (128 bytes).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | (64ull << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void st_shared16(uint8_t *base, uint32_t off, uint4 v)
{
    *reinterpret_cast<uint4 *>(base + off) = v;
}

// ---- convolution geometry -----------------------------------------------------

// Cubic volumes: input side di, output side do_ = (di + 1) / 2, channels-last.
struct Geo {
    int batch, di, dout, cin, cout;
    __device__ __forceinline__ long long npos_in() const { return (long long)batch * di * di * di; }
    __device__ __forceinline__ long long npos_out() const { return (long long)batch * dout * dout * dout; }
};

// Zero-filled 8 x bf16.
__device__ __forceinline__ uint4 zero4() { return make_uint4(0u, 0u, 0u, 0u); }

// ---- the three convolution operators as GEMM operand gatherers ---------------------

// forward: rows = output positions, K = 27 * cin (tap-major), N = cout.
// B operand: Wk [cout][kp] bf16, k = tap * cin + c, zero-padded to kp.
struct OpFwd {
    Geo g;
    const __nv_bfloat16 *x;  // [npos_in][cin]
    const __nv_bfloat16 *wk; // [cout][kp]
    const float *bias;       // [cout]
    __nv_bfloat16 *y;        // [npos_out][cout]
    int kp;
    __device__ __forceinline__ long long rows() const { return g.npos_out(); }
    __device__ __forceinline__ int kchunks() const { return kp / kBK; }

    __device__ __forceinline__ void load_a(uint8_t *sa, long long m0, int kc, int tid) const
    {
        const long long m = m0 + tid;
        const bool live = m < rows();
        int n = 0, z = 0, yy = 0, xx = 0;
        if (live) {
            long long q = m;
            xx = (int)(q % g.dout);
            q /= g.dout;
            yy = (int)(q % g.dout);
            q /= g.dout;
            z = (int)(q % g.dout);
            n = (int)(q / g.dout);
        }
        const int d = g.di;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int k0 = kc * kBK + j * 8;
            uint4 v = zero4();
            if (live) {
                if (g.cin >= 8) {
                    const int t = k0 / g.cin, c0 = k0 - t * g.cin;
                    if (t < 27) {
                        const int iz = 2 * z + t / 9 - 1, iy = 2 * yy + (t / 3) % 3 - 1, ix = 2 * xx + t % 3 - 1;
                        if (iz >= 0 && iz < d && iy >= 0 && iy < d && ix >= 0 && ix < d)
                            v = *reinterpret_cast<const uint4 *>(
                                x + ((((long long)n * d + iz) * d + iy) * d + ix) * g.cin + c0);
                    }
                } else { // cin == 1: eight taps
                    __nv_bfloat16 e[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const int t = k0 + u;
                        e[u] = __float2bfloat16(0.0f);
                        if (t < 27) {
                            const int iz = 2 * z + t / 9 - 1, iy = 2 * yy + (t / 3) % 3 - 1, ix = 2 * xx + t % 3 - 1;
                            if (iz >= 0 && iz < d && iy >= 0 && iy < d && ix >= 0 && ix < d)
                                e[u] = x[(((long long)n * d + iz) * d + iy) * d + ix];
                        }
                    }
                    v = *reinterpret_cast<const uint4 *>(e);
                }
            }
            st_shared16(sa, sw128(tid, j), v);
        }
    }

    __device__ __forceinline__ void load_b(uint8_t *sb, int kc, int tid, int bn) const
    {
        for (int it = tid; it < bn * 8; it += kThreads) {
            const int r = it >> 3, j = it & 7;
            const uint4 v = *reinterpret_cast<const uint4 *>(wk + (long long)r * kp + kc * kBK + j * 8);
            st_shared16(sb, sw128(r, j), v);
        }
    }

    __device__ __forceinline__ void store(long long m, int c0, const float *v, int) const
    {
        if (m >= rows())
            return;
        __align__(16) __nv_bfloat16 o[16];
#pragma unroll
        for (int i = 0; i < 16; i++)
            o[i] = __float2bfloat16(fmaxf(v[i] + bias[c0 + i], 0.0f));
        uint4 *dst = reinterpret_cast<uint4 *>(y + m * g.cout + c0);
        dst[0] = reinterpret_cast<const uint4 *>(o)[0];
        dst[1] = reinterpret_cast<const uint4 *>(o)[1];
    }
};

// dgrad: rows = input positions, K = 27 * cout (tap-major), N = cin.
// B operand: WkT [cin][kp] bf16, k = tap * cout + o.  The result is masked by
// ReLU' of the layer below (its output xact > 0) -- the gradient of that
// layer's pre-activation.
struct OpDgrad {
    Geo g;
    const __nv_bfloat16 *dz;   // [npos_out][cout]
    const __nv_bfloat16 *wkt;  // [cin][kp]
    const __nv_bfloat16 *xact; // [npos_in][cin]
    __nv_bfloat16 *dx;         // [npos_in][cin]
    int kp;
    __device__ __forceinline__ long long rows() const { return g.npos_in(); }
    __device__ __forceinline__ int kchunks() const { return kp / kBK; }

    __device__ __forceinline__ void load_a(uint8_t *sa, long long m0, int kc, int tid) const
    {
        const long long m = m0 + tid;
        const bool live = m < rows();
        int n = 0, iz = 0, iy = 0, ix = 0;
        if (live) {
            long long q = m;
            ix = (int)(q % g.di);
            q /= g.di;
            iy = (int)(q % g.di);
            q /= g.di;
            iz = (int)(q % g.di);
            n = (int)(q / g.di);
        }
        const int d = g.dout;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int k0 = kc * kBK + j * 8;
            uint4 v = zero4();
            const int t = k0 / g.cout, o0 = k0 - t * g.cout;
            if (live && t < 27) {
                // input iz takes tap kz from output oz when iz = 2 oz + kz - 1
                const int sz = iz + 1 - t / 9, sy = iy + 1 - (t / 3) % 3, sx = ix + 1 - t % 3;
                if (sz >= 0 && sy >= 0 && sx >= 0 && !(sz & 1) && !(sy & 1) && !(sx & 1)) {
                    const int oz = sz >> 1, oy = sy >> 1, ox = sx >> 1;
                    if (oz < d && oy < d && ox < d)
                        v = *reinterpret_cast<const uint4 *>(
                            dz + ((((long long)n * d + oz) * d + oy) * d + ox) * g.cout + o0);
                }
            }
            st_shared16(sa, sw128(tid, j), v);
        }
    }

    __device__ __forceinline__ void load_b(uint8_t *sb, int kc, int tid, int bn) const
    {
        for (int it = tid; it < bn * 8; it += kThreads) {
            const int r = it >> 3, j = it & 7;
            const uint4 v = *reinterpret_cast<const uint4 *>(wkt + (long long)r * kp + kc * kBK + j * 8);
            st_shared16(sb, sw128(r, j), v);
        }
    }

    __device__ __forceinline__ void store(long long m, int c0, const float *v, int) const
    {
        if (m >= rows())
            return;
        const __nv_bfloat16 *xa = xact + m * g.cin + c0;
        __align__(16) __nv_bfloat16 o[16];
#pragma unroll
        for (int i = 0; i < 16; i++)
            o[i] = __float2bfloat16(__bfloat162float(xa[i]) > 0.0f ? v[i] : 0.0f);
        uint4 *dst = reinterpret_cast<uint4 *>(dx + m * g.cin + c0);
        dst[0] = reinterpret_cast<const uint4 *>(o)[0];
        dst[1] = reinterpret_cast<const uint4 *>(o)[1];
    }
};

// wgrad: rows = (tap, c_in) pairs (27 * cin, tile rows beyond are zero),
// K = output positions (split over CTAs), N = cout.  Both operands are
// gathered transposed (positions along K).  The result is added into dw
// [27 * cin][cout] fp32 with atomics.
struct OpWgrad {
    Geo g;
    const __nv_bfloat16 *x;  // [npos_in][cin]
    const __nv_bfloat16 *dz; // [npos_out][cout]
    float *dw;               // [27 * cin][cout]
    int kchunks_total;       // ceil(npos_out / 64)
    __device__ __forceinline__ long long rows() const { return 27LL * g.cin; }
    __device__ __forceinline__ int kchunks() const { return kchunks_total; }

    // element (row r, K column j) of a tile: byte offset in the swizzled layout
    static __device__ __forceinline__ uint32_t el(int r, int j) { return sw128(r, j >> 3) + ((j & 7) << 1); }

    __device__ __forceinline__ void load_a(uint8_t *sa, long long m0, int kc, int tid) const
    {
        // zero the tile, then scatter the live (position, tap, channel) values
        for (int it = tid; it < kBM * 8; it += kThreads)
            st_shared16(sa, sw128(it >> 3, it & 7), zero4());
        __syncthreads();
        const long long p0 = (long long)kc * kBK;
        const long long np = g.npos_out();
        const int d = g.di, dd = g.dout;
        if (g.cin >= 8) {
            const int groups = kBM / 8; // 8 channels per group
            for (int it = tid; it < kBK * groups; it += kThreads) {
                const int j = it % kBK, gr = it / kBK;
                const long long r0 = m0 + (long long)gr * 8;
                const long long p = p0 + j;
                if (r0 >= rows() || p >= np)
                    continue;
                const int t = (int)(r0 / g.cin), c0 = (int)(r0 - (long long)t * g.cin);
                long long q = p;
                const int ox = (int)(q % dd);
                q /= dd;
                const int oy = (int)(q % dd);
                q /= dd;
                const int oz = (int)(q % dd);
                const int n = (int)(q / dd);
                const int iz = 2 * oz + t / 9 - 1, iy = 2 * oy + (t / 3) % 3 - 1, ix = 2 * ox + t % 3 - 1;
                if (iz < 0 || iz >= d || iy < 0 || iy >= d || ix < 0 || ix >= d)
                    continue;
                const uint4 v = *reinterpret_cast<const uint4 *>(
                    x + ((((long long)n * d + iz) * d + iy) * d + ix) * g.cin + c0);
                const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
                const int rl = gr * 8;
#pragma unroll
                for (int u = 0; u < 8; u++)
                    *reinterpret_cast<__nv_bfloat16 *>(sa + el(rl + u, j)) = e[u];
            }
        } else { // cin == 1: rows are the 27 taps
            for (int it = tid; it < kBK * 27; it += kThreads) {
                const int j = it % kBK, t = it / kBK;
                const long long p = p0 + j;
                if (m0 != 0 || p >= np)
                    continue;
                long long q = p;
                const int ox = (int)(q % dd);
                q /= dd;
                const int oy = (int)(q % dd);
                q /= dd;
                const int oz = (int)(q % dd);
                const int n = (int)(q / dd);
                const int iz = 2 * oz + t / 9 - 1, iy = 2 * oy + (t / 3) % 3 - 1, ix = 2 * ox + t % 3 - 1;
                if (iz < 0 || iz >= d || iy < 0 || iy >= d || ix < 0 || ix >= d)
                    continue;
                *reinterpret_cast<__nv_bfloat16 *>(sa + el(t, j)) = x[(((long long)n * d + iz) * d + iy) * d + ix];
            }
        }
    }

    __device__ __forceinline__ void load_b(uint8_t *sb, int kc, int tid, int bn) const
    {
        for (int it = tid; it < bn * 8; it += kThreads)
            st_shared16(sb, sw128(it >> 3, it & 7), zero4());
        __syncthreads();
        const long long p0 = (long long)kc * kBK;
        const long long np = g.npos_out();
        const int groups = bn / 8;
        for (int it = tid; it < kBK * groups; it += kThreads) {
            const int j = it % kBK, gr = it / kBK;
            const long long p = p0 + j;
            if (p >= np)
                continue;
            const uint4 v = *reinterpret_cast<const uint4 *>(dz + p * g.cout + gr * 8);
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int u = 0; u < 8; u++)
                *reinterpret_cast<__nv_bfloat16 *>(sb + el(gr * 8 + u, j)) = e[u];
        }
    }

    __device__ __forceinline__ void store(long long m, int c0, const float *v, int bn) const
    {
        if (m >= rows())
            return;
        float *dst = dw + m * g.cout + c0;
#pragma unroll
        for (int i = 0; i < 16; i++)
            if (v[i] != 0.0f)
                atomicAdd(dst + i, v[i]);
        (void)bn;
    }
};

// ---- the tile kernel ----------------------------------------------------------------

template <int BN>
struct TileSmem {
    static constexpr int kA = kBM * 128; // 16 KB per A stage
    static constexpr int kB = BN * 128;  // B stage
    static constexpr int kStage = kA + kB;
    static constexpr int kBytes = kStages * kStage + 1024; // + alignment slack
};

// Error codes written to *err: 1 = an mbarrier wait ran out of time.
template <class Op, int BN>
__global__ void __launch_bounds__(kThreads) k_umma_conv(Op op, int ksplit, int *err)
{
    static_assert(BN == 16 || BN == 32 || BN == 64, "tile width");
    constexpr int kCols = BN < 32 ? 32 : BN; // TMEM allocation: a power of two >= 32
    constexpr uint32_t kIdesc = idesc_bf16(BN);
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar[kStages];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base;

    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;

    if (warp == 0) {
        tmem_alloc(&tmem_base, kCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; s++)
            mbar_init(&bar[s], 1);
        mbar_init(&done_bar, 1);
        fence_barrier_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    const long long m0 = (long long)blockIdx.x * kBM;
    const int nk_all = op.kchunks();
    const int per = (nk_all + ksplit - 1) / ksplit;
    const int kc0 = blockIdx.y * per;
    const int kc1 = min(nk_all, kc0 + per);
    bool ok = true;
    int issued = 0;
    for (int kc = kc0; kc < kc1; kc++) {
        const int i = kc - kc0;
        const int s = i % kStages;
        uint8_t *sa = smem + s * TileSmem<BN>::kStage;
        uint8_t *sb = sa + TileSmem<BN>::kA;
        if (i >= kStages) // the MMAs that read this stage (chunk i - kStages) are done
            ok = mbar_wait(&bar[s], (unsigned)((i / kStages) - 1) & 1u);
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        op.load_a(sa, m0, kc, tid);
        op.load_b(sb, kc, tid, BN);
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; kk++)
                umma_bf16(tmem, sdesc_sw128(a0 + kk * 32), sdesc_sw128(b0 + kk * 32), kIdesc,
                          (i > 0 || kk > 0) ? 1u : 0u);
            umma_commit(&bar[s]);
        }
        issued++;
    }
    // all MMAs of this CTA done (or none issued)
    if (tid == 0)
        umma_commit(&done_bar);
    const bool done = mbar_wait(&done_bar, 0);
    tc_fence_after();
    // one decision for the whole CTA: tcgen05.ld below is warp-collective
    const bool good = __syncthreads_and(done && ok) != 0;
    if (!good) {
        if (tid == 0)
            atomicExch(err, 1);
    } else if (issued > 0) {
        const long long m = m0 + tid;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tmem_ld16(lane_addr + (uint32_t)c0, v);
            op.store(m, c0, v, BN);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, kCols);
}

template <class Op, int BN>
static int launch_tiles(const Op &op, long long rows, int ksplit, int *err, cudaStream_t st, const char *name,
                        double flops)
{
    const int smem = TileSmem<BN>::kBytes;
    PMG_CUDA(cudaFuncSetAttribute(k_umma_conv<Op, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const dim3 grid((unsigned)((rows + kBM - 1) / kBM), (unsigned)ksplit);
    const int ps__ = prof_begin(name, st);
    k_umma_conv<Op, BN><<<grid, kThreads, smem, st>>>(op, ksplit, err);
    prof_end(ps__, flops, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

template <class Op>
static int launch_bn(const Op &op, int bn, long long rows, int ksplit, int *err, cudaStream_t st, const char *name,
                     double flops)
{
    switch (bn) {
    case 16:
        return launch_tiles<Op, 16>(op, rows, ksplit, err, st, name, flops);
    case 32:
        return launch_tiles<Op, 32>(op, rows, ksplit, err, st, name, flops);
    case 64:
        return launch_tiles<Op, 64>(op, rows, ksplit, err, st, name, flops);
    default:
        set_error("cnn: output channels %d not in {16, 32, 64}", bn);
        return PMG_EINVAL;
    }
}

static int check_geo(int batch, int di, int cin, int cout)
{
    if (batch <= 0 || di <= 1 || di > 1024) {
        set_error("cnn: batch %d / side %d out of range", batch, di);
        return PMG_EINVAL;
    }
    if (!(cin == 1 || cin == 16 || cin == 32 || cin == 64) || !(cout == 16 || cout == 32 || cout == 64)) {
        set_error("cnn: channels %d -> %d not supported (cin in {1,16,32,64}, cout in {16,32,64})", cin, cout);
        return PMG_EINVAL;
    }
    return PMG_OK;
}

static int kpad(int k) { return (k + kBK - 1) / kBK * kBK; }

// ---- weight packing (fp32 master [cout][cin][27] -> bf16 GEMM operands) -------------

__global__ void k_pack_w(const float *__restrict__ w, int cin, int cout, int kp, __nv_bfloat16 *__restrict__ wk,
                         int kpt, __nv_bfloat16 *__restrict__ wkt)
{
    const int n1 = cout * kp, n2 = wkt ? cin * kpt : 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1 + n2; i += gridDim.x * blockDim.x) {
        if (i < n1) {
            const int o = i / kp, k = i - o * kp;
            const int t = k / cin, c = k - t * cin;
            wk[i] = __float2bfloat16(t < 27 ? w[((long long)o * cin + c) * 27 + t] : 0.0f);
        } else {
            const int i2 = i - n1;
            const int c = i2 / kpt, k = i2 - c * kpt;
            const int t = k / cout, o = k - t * cout;
            wkt[i2] = __float2bfloat16(t < 27 ? w[((long long)o * cin + c) * 27 + t] : 0.0f);
        }
    }
}

// dw [27 * cin][cout] (tap-major rows) -> grad [cout][cin][27]
__global__ void k_unpack_dw(const float *__restrict__ dw, int cin, int cout, float *__restrict__ grad)
{
    const int n = cout * cin * 27;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = i % 27, c = (i / 27) % cin, o = i / (27 * cin);
        grad[i] = dw[((long long)t * cin + c) * cout + o];
    }
}

// bias gradient: db[o] = sum over positions of dz[p][o]
__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ dz, long long np, int cout, float *__restrict__ db)
{
    __shared__ float acc[64];
    if (threadIdx.x < 64)
        acc[threadIdx.x] = 0.0f;
    __syncthreads();
    const int o = threadIdx.x % cout;
    const int lanes = blockDim.x / cout;
    float s = 0.0f;
    for (long long p = (long long)blockIdx.x * lanes + threadIdx.x / cout; p < np; p += (long long)gridDim.x * lanes)
        s += __bfloat162float(dz[p * cout + o]);
    atomicAdd(&acc[o], s);
    __syncthreads();
    if (threadIdx.x < cout)
        atomicAdd(db + threadIdx.x, acc[threadIdx.x]);
}

// ---- head: global average pool, MLP 64-64-64, sigmoid, MSE loss and its backward ----
// One CTA of 64 threads per sample.  y4: [batch][64 positions][64 channels]
// bf16 (the last convolution's ReLU output, 4^3 positions); parameters fp32:
// w5 [64][64] b5 [64] (hidden, ReLU), w6 [64][64] b6 [64] (outputs, sigmoid).
// With target != null the loss mean((s - t)^2) / batch is accumulated into
// *loss and the gradients are added into the g* buffers (atomics across
// samples) and written to dy4 (masked by the last ReLU).
constexpr int kHead = 64;

__global__ void k_head(const __nv_bfloat16 *__restrict__ y4, const float *__restrict__ w5,
                       const float *__restrict__ b5, const float *__restrict__ w6, const float *__restrict__ b6,
                       const float *__restrict__ target, float *__restrict__ pred, float *__restrict__ loss,
                       float *__restrict__ gw5, float *__restrict__ gb5, float *__restrict__ gw6,
                       float *__restrict__ gb6, __nv_bfloat16 *__restrict__ dy4, float inv_batch)
{
    __shared__ float h0[kHead], h1[kHead], dout[kHead], dh1[kHead];
    const int n = blockIdx.x, t = threadIdx.x;
    const __nv_bfloat16 *y = y4 + (long long)n * 64 * kHead;
    float a = 0.0f;
    for (int p = 0; p < 64; p++)
        a += __bfloat162float(y[p * kHead + t]);
    h0[t] = a * (1.0f / 64.0f);
    __syncthreads();
    float z = b5[t];
    for (int c = 0; c < kHead; c++)
        z += w5[t * kHead + c] * h0[c];
    h1[t] = fmaxf(z, 0.0f);
    __syncthreads();
    float o = b6[t];
    for (int j = 0; j < kHead; j++)
        o += w6[t * kHead + j] * h1[j];
    const float s = 1.0f / (1.0f + __expf(-o));
    pred[(long long)n * kHead + t] = s;
    if (!target)
        return;
    const float e = s - target[(long long)n * kHead + t];
    atomicAdd(loss, e * e * (inv_batch / kHead));
    dout[t] = 2.0f * e * (inv_batch / kHead) * s * (1.0f - s);
    __syncthreads();
    for (int j = 0; j < kHead; j++)
        atomicAdd(gw6 + t * kHead + j, dout[t] * h1[j]);
    atomicAdd(gb6 + t, dout[t]);
    float d1 = 0.0f;
    for (int k = 0; k < kHead; k++)
        d1 += w6[k * kHead + t] * dout[k];
    dh1[t] = h1[t] > 0.0f ? d1 : 0.0f;
    __syncthreads();
    for (int c = 0; c < kHead; c++)
        atomicAdd(gw5 + t * kHead + c, dh1[t] * h0[c]);
    atomicAdd(gb5 + t, dh1[t]);
    float d0 = 0.0f;
    for (int j = 0; j < kHead; j++)
        d0 += w5[j * kHead + t] * dh1[j];
    d0 *= 1.0f / 64.0f;
    __nv_bfloat16 *dy = dy4 + (long long)n * 64 * kHead;
    for (int p = 0; p < 64; p++)
        dy[p * kHead + t] = __float2bfloat16(__bfloat162float(y[p * kHead + t]) > 0.0f ? d0 : 0.0f);
}

// Adam (Kingma and Ba) over a flat fp32 parameter vector, bias-corrected.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, float wd)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * w[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Network input: the distance field of the own region, averaged over 64^3
// cells (cell a of an axis of length L covers [a L / 64, (a + 1) L / 64)),
// divided by `scale` (the medium's largest distance), as bf16.
__global__ void k_downsample(const float *__restrict__ d, long long s1, long long s2, int lo0, int lo1, int lo2,
                             int l0, int l1, int l2, float inv_scale, __nv_bfloat16 *__restrict__ out)
{
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= 64 * 64 * 64)
        return;
    const int a = cell >> 12, b = (cell >> 6) & 63, c = cell & 63;
    const int i0 = a * l0 / 64, i1 = (a + 1) * l0 / 64;
    const int j0 = b * l1 / 64, j1 = (b + 1) * l1 / 64;
    const int k0 = c * l2 / 64, k1 = (c + 1) * l2 / 64;
    float acc = 0.0f;
    int cnt = 0;
    for (int i = i0; i < i1; i++)
        for (int j = j0; j < j1; j++)
            for (int k = k0; k < k1; k++) {
                acc += d[((long long)(lo0 + i) * s1 + (lo1 + j)) * s2 + (lo2 + k)];
                cnt++;
            }
    out[cell] = __float2bfloat16(cnt ? acc / cnt * inv_scale : 0.0f);
}

} // namespace cnn
} // namespace pmg

using namespace pmg;
using namespace pmg::cnn;

namespace {
int cnn_err_check(int *err, cudaStream_t st)
{
    int h = 0;
    PMG_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    if (h) {
        set_error("cnn: a tensor-core pipeline wait ran out of time (code %d)", h);
        return PMG_EITER;
    }
    return PMG_OK;
}
} // namespace

extern "C" int pmg_cnn_pack_weights(const float *w, int32_t cin, int32_t cout, void *wk, void *wkt, void *stream)
{
    if (!w || !wk) {
        set_error("pmg_cnn_pack_weights: null argument");
        return PMG_EINVAL;
    }
    const int kp = kpad(27 * cin), kpt = kpad(27 * cout);
    cudaStream_t st = as_stream(stream);
    const int ps__ = prof_begin("k_pack_w", st);
    k_pack_w<<<64, 256, 0, st>>>(w, cin, cout, kp, (__nv_bfloat16 *)wk, kpt, (__nv_bfloat16 *)wkt);
    prof_end(ps__, 0.0, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

extern "C" int pmg_cnn_conv_fwd(const void *x, const void *wk, const float *bias, void *y, int32_t batch,
                                int32_t di, int32_t cin, int32_t cout, int32_t *err, void *stream)
{
    if (!x || !wk || !bias || !y || !err) {
        set_error("pmg_cnn_conv_fwd: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geo(batch, di, cin, cout));
    OpFwd op;
    op.g = Geo{batch, di, (di + 1) / 2, cin, cout};
    op.x = (const __nv_bfloat16 *)x;
    op.wk = (const __nv_bfloat16 *)wk;
    op.bias = bias;
    op.y = (__nv_bfloat16 *)y;
    op.kp = kpad(27 * cin);
    const long long rows = (long long)batch * op.g.dout * op.g.dout * op.g.dout;
    return launch_bn(op, cout, rows, 1, err, as_stream(stream), "k_umma_conv_fwd",
                     2.0 * rows * cout * 27.0 * cin);
}

extern "C" int pmg_cnn_conv_dgrad(const void *dz, const void *wkt, const void *xact, void *dx, int32_t batch,
                                  int32_t di, int32_t cin, int32_t cout, int32_t *err, void *stream)
{
    if (!dz || !wkt || !xact || !dx || !err) {
        set_error("pmg_cnn_conv_dgrad: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geo(batch, di, cin, cout));
    if (cin < 16) {
        set_error("pmg_cnn_conv_dgrad: the input gradient of a %d-channel layer is not needed", cin);
        return PMG_EINVAL;
    }
    OpDgrad op;
    op.g = Geo{batch, di, (di + 1) / 2, cin, cout};
    op.dz = (const __nv_bfloat16 *)dz;
    op.wkt = (const __nv_bfloat16 *)wkt;
    op.xact = (const __nv_bfloat16 *)xact;
    op.dx = (__nv_bfloat16 *)dx;
    op.kp = kpad(27 * cout);
    const long long rows = (long long)batch * di * di * di;
    return launch_bn(op, cin, rows, 1, err, as_stream(stream), "k_umma_conv_dgrad",
                     2.0 * rows * cin * 27.0 * cout / 8.0);
}

extern "C" int pmg_cnn_conv_wgrad(const void *x, const void *dz, float *dw, float *grad, float *dbias,
                                  int32_t batch, int32_t di, int32_t cin, int32_t cout, int32_t *err,
                                  void *stream)
{
    if (!x || !dz || !dw || !grad || !dbias || !err) {
        set_error("pmg_cnn_conv_wgrad: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geo(batch, di, cin, cout));
    cudaStream_t st = as_stream(stream);
    OpWgrad op;
    op.g = Geo{batch, di, (di + 1) / 2, cin, cout};
    op.x = (const __nv_bfloat16 *)x;
    op.dz = (const __nv_bfloat16 *)dz;
    op.dw = dw;
    const long long np = (long long)batch * op.g.dout * op.g.dout * op.g.dout;
    op.kchunks_total = (int)((np + kBK - 1) / kBK);
    const long long rows = 27LL * cin;
    const int mt = (int)((rows + kBM - 1) / kBM);
    // split K so that about four CTAs run per SM
    int ksplit = (4 * 152 + mt - 1) / mt;
    ksplit = std::max(1, std::min(ksplit, op.kchunks_total));
    PMG_CUDA(cudaMemsetAsync(dw, 0, sizeof(float) * (size_t)rows * cout, st));
    PMG_CUDA(cudaMemsetAsync(dbias, 0, sizeof(float) * (size_t)cout, st));
    PMG_TRY(launch_bn(op, cout, rows, ksplit, err, st, "k_umma_conv_wgrad", 2.0 * np * cout * 27.0 * cin));
    {
        const int ps__ = prof_begin("k_unpack_dw", st);
        k_unpack_dw<<<64, 256, 0, st>>>(dw, cin, cout, grad);
        prof_end(ps__, 0.0, st);
    }
    {
        const int ps__ = prof_begin("k_bias_grad", st);
        k_bias_grad<<<152, 256, 0, st>>>((const __nv_bfloat16 *)dz, np, cout, dbias);
        prof_end(ps__, 0.0, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

extern "C" int pmg_cnn_check(int32_t *err, void *stream) { return cnn_err_check(err, as_stream(stream)); }

extern "C" int pmg_cnn_head(const void *y4, const float *params, int32_t batch, const float *target, float *pred,
                            float *loss, float *grads, void *dy4, void *stream)
{
    if (!y4 || !params || !pred || batch <= 0 || (target && (!loss || !grads || !dy4))) {
        set_error("pmg_cnn_head: bad argument");
        return PMG_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    const float *w5 = params, *b5 = w5 + kHead * kHead, *w6 = b5 + kHead, *b6 = w6 + kHead * kHead;
    float *gw5 = grads, *gb5 = grads ? gw5 + kHead * kHead : nullptr, *gw6 = grads ? gb5 + kHead : nullptr,
          *gb6 = grads ? gw6 + kHead * kHead : nullptr;
    const int ps__ = prof_begin("k_head", st);
    k_head<<<batch, kHead, 0, st>>>((const __nv_bfloat16 *)y4, w5, b5, w6, b6, target, pred, loss, gw5, gb5, gw6,
                                    gb6, (__nv_bfloat16 *)dy4, 1.0f / (float)batch);
    prof_end(ps__, 0.0, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

extern "C" int pmg_cnn_adam(float *w, const float *g, float *m, float *v, int64_t n, double lr, double b1,
                            double b2, double eps, int64_t step, double weight_decay, void *stream)
{
    if (!w || !g || !m || !v || n <= 0 || step <= 0) {
        set_error("pmg_cnn_adam: bad argument");
        return PMG_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    const float c1 = (float)(1.0 - std::pow(b1, (double)step)), c2 = (float)(1.0 - std::pow(b2, (double)step));
    const int ps__ = prof_begin("k_adam", st);
    k_adam<<<152, 256, 0, st>>>(w, g, m, v, n, (float)lr, (float)b1, (float)b2, (float)eps, c1, c2,
                                (float)weight_decay);
    prof_end(ps__, 0.0, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

extern "C" int pmg_cnn_downsample(const float *dist, const int64_t shape[3], const int64_t box[6], double scale,
                                  void *out, void *stream)
{
    if (!dist || !shape || !box || !out || !(scale > 0.0)) {
        set_error("pmg_cnn_downsample: bad argument");
        return PMG_EINVAL;
    }
    const int l0 = (int)(box[1] - box[0]), l1 = (int)(box[3] - box[2]), l2 = (int)(box[5] - box[4]);
    if (l0 < 64 || l1 < 64 || l2 < 64 || box[0] < 0 || box[2] < 0 || box[4] < 0 || box[1] > shape[0] ||
        box[3] > shape[1] || box[5] > shape[2]) {
        set_error("pmg_cnn_downsample: box must lie in the volume and span at least 64 voxels per axis");
        return PMG_EINVAL;
    }
    cudaStream_t st = as_stream(stream);
    const int ps__ = prof_begin("k_downsample", st);
    k_downsample<<<64 * 64 * 64 / 256, 256, 0, st>>>(dist, shape[1], shape[2], (int)box[0], (int)box[2],
                                                     (int)box[4], l0, l1, l2, (float)(1.0 / scale),
                                                     (__nv_bfloat16 *)out);
    prof_end(ps__, (double)l0 * l1 * l2 * 4, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}
