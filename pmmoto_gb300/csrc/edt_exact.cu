// Exact streaming lower envelope for power-of-two resolutions (sm_103a).
//
// With a power-of-two voxel size every height the EDT passes carry is an
// exact integer multiple K of res^2, and the reference's float32
// Felzenszwalb envelope (src/pmmoto/filters/distance/_distance.hpp:184-272)
// returns exactly min_v res^2 * (K_v + (x - v)^2) at every integer x when no
// periodic hull is imported (its rounding can only reorder ties).  That
// minimum is what this kernel computes, in integers:
//
//  * intersections of parabolas are compared by cross-multiplication
//    (no division), popping on ties as the reference does;
//  * an output x is emitted as soon as it is final -- once the current
//    envelope value E(x) <= (i + 1 - x)^2, no later parabola (height >= 0) can
//    lower it -- so the line is streamed once, reading each height once;
//  * the stack lives in a per-line ring of kRing entries in shared memory; the
//    bottom entry is dropped once the entry above it can provably never be
//    popped again (its value at its left boundary is below what any later
//    parabola can reach there);
//  * heights at FLT_MAX (no solid on the earlier passes' lines) never win
//    against a finite one and are skipped; a line without finite heights
//    yields FLT_MAX everywhere.
//
// A line whose live stack would exceed the ring, or whose heights are not
// exact integer multiples of res^2, is marked (NaN / 255 in its first output)
// and redone by the general kernel, which reproduces the reference's float
// arithmetic step by step.
#include <cfloat>
#include <climits>

#include "edt_internal.cuh"

namespace pmg {

constexpr int kRing = 32; // live stack entries per line (power of two)

struct Ring {
    int *k;      // heights, slot s of this thread at k[s * nthr]
    short *v;    // vertices
    int nthr;
    __device__ __forceinline__ int K(int c) const { return k[(c & (kRing - 1)) * nthr]; }
    __device__ __forceinline__ int V(int c) const { return v[(c & (kRing - 1)) * nthr]; }
    __device__ __forceinline__ void put(int c, int vv, int kk)
    {
        k[(c & (kRing - 1)) * nthr] = kk;
        v[(c & (kRing - 1)) * nthr] = (short)vv;
    }
};

__device__ __forceinline__ long long pval(long long K, long long v, long long x)
{
    const long long d = x - v;
    return K + d * d;
}

// true when the intersection of (i, Ki) with (t, Kt) lies at or left of the
// intersection of (t, Kt) with (b, Kb): the reference's "s <= ranges[k]"
__device__ __forceinline__ bool pops(long long i, long long Ki, long long t, long long Kt, long long b,
                                     long long Kb)
{
    const long long n1 = Ki - Kt + (i - t) * (i + t), d1 = 2 * (i - t);
    const long long n2 = Kt - Kb + (t - b) * (t + b), d2 = 2 * (t - b);
    return n1 * d2 <= n2 * d1;
}

// entry (u, Ku) above (w, Kw) can never be popped by a parabola at >= i1
__device__ __forceinline__ bool unpoppable(long long u, long long Ku, long long w, long long Kw, long long i1)
{
    const long long N = Ku - Kw + (u - w) * (u + w), D = 2 * (u - w); // left boundary N / D
    if (N >= i1 * D)
        return false;
    const long long a = N - u * D, c = i1 * D - N;
    return Ku * D * D + a * a < c * c;
}

__device__ __forceinline__ void store_out(float *fout, const LineGeo &g, const MorphEpi &me, int form, int x,
                                          long long E, bool inf, float a)
{
    const float val = inf ? FLT_MAX : fmul((float)E, a);
    if (form == PMG_EDT_MORPH) {
        morph_store(me, g, x, val);
        return;
    }
    fout[g.base + (long long)x * g.stride] = form == PMG_EDT_DIST ? __fsqrt_rn(val) : val;
}

__device__ __forceinline__ void mark_line(float *fout, const LineGeo &g, const MorphEpi &me, int form)
{
    if (form == PMG_EDT_MORPH) {
        const long long io = g.a - me.e0, jo = g.b - me.e1;
        me.out[(io * me.o1 + jo) * me.o2] = 255;
    } else {
        fout[g.base] = __int_as_float(0x7fc00000); // NaN
    }
}

__global__ void __launch_bounds__(128) k_env_exact(const float *__restrict__ fin, float *__restrict__ fout,
                                                   Lines Ls, float a, float inv_a, int form, MorphEpi me,
                                                   int cap)
{
    extern __shared__ int smem_ring[];
    Ring R;
    R.nthr = blockDim.x;
    R.k = smem_ring + threadIdx.x;
    R.v = (short *)(smem_ring + kRing * blockDim.x) + threadIdx.x;
    const long long nlines = Ls.count();
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < nlines;
         li += (long long)gridDim.x * blockDim.x) {
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        const long long st = g.stride;
        const int n = g.n;
        // heights up to 2^24 - n^2 keep every float32 sum of the reference's
        // intersection and evaluation formulas an exact integer
        const float kmax = 16777216.0f - (float)n * (float)n;
        // heights above the cap never matter to the caller: skipped like FLT_MAX
        const float fcap = cap == INT_MAX ? __int_as_float(0x7f7ffffe) : fmul((float)cap, a);
        int bot = 0, top = -1, e = 0, x = 0;
        bool bad = false;
        const long long capl = cap;
        for (int i = 0; i < n; i++) {
            const float f = line[i * st];
            if (f <= fcap) {
                const float kf = fmul(f, inv_a);
                const int Ki = (int)kf;
                if ((float)Ki != kf || fmul((float)Ki, a) != f || kf >= kmax) {
                    bad = true; // not an exact integer height
                    break;
                }
                while (top > bot && pops(i, Ki, R.V(top), R.K(top), R.V(top - 1), R.K(top - 1))) {
                    if (e == top)
                        e--;
                    top--;
                }
                if (top - bot + 1 >= kRing) {
                    bad = true;
                    break;
                }
                top++;
                R.put(top, i, Ki);
                if (top == bot)
                    e = bot;
            }
            // emit every output that no later parabola can change: its value is
            // at most (i + 1 - x)^2, or that bound already exceeds the cap
            while (x <= i) {
                const long long dd = (long long)(i + 1 - x);
                if (top < bot) {
                    if (dd * dd <= capl)
                        break;
                    store_out(fout, g, me, form, x, 0, true, a);
                    x++;
                    continue;
                }
                while (e < top && pval(R.K(e + 1), R.V(e + 1), x) <= pval(R.K(e), R.V(e), x))
                    e++;
                const long long E = pval(R.K(e), R.V(e), x);
                if (E > dd * dd && dd * dd <= capl)
                    break;
                store_out(fout, g, me, form, x, E, E > capl, a);
                x++;
            }
            // drop bottom entries the stack can never pop back to
            while (bot < e && unpoppable(R.V(bot + 1), R.K(bot + 1), R.V(bot), R.K(bot), i + 1))
                bot++;
        }
        if (bad) {
            mark_line(fout, g, me, form);
            continue;
        }
        for (; x < n; x++) {
            if (top < bot) {
                store_out(fout, g, me, form, x, 0, true, a);
                continue;
            }
            while (e < top && pval(R.K(e + 1), R.V(e + 1), x) <= pval(R.K(e), R.V(e), x))
                e++;
            const long long E = pval(R.K(e), R.V(e), x);
            store_out(fout, g, me, form, x, E, E > capl, a);
        }
    }
}

// The exact path needs a power-of-two voxel size (so res^2 scales integers
// exactly) and no periodic hull import.  Lines are limited to 2048 voxels: the
// reference rounds each intersection N / D (D <= 2(n - 1)) once to float32,
// and below 2048 that error (< 2^-13) is smaller than the distance 1 / D of a
// non-integer intersection to the nearest integer, so the reference's float
// envelope can differ from the exact one only where two parabolas tie at an
// integer point -- the same value either way.
bool exact_path_ok(float res, const pmg_axis_cfg &cfg, int n)
{
    if (cfg.periodic || n > 2048 || !(res > 0.0f))
        return false;
    int ex = 0;
    const float m = frexpf(res, &ex);
    return m == 0.5f && ex > -40 && ex < 40;
}

int launch_envelope_exact(const float *fin, float *fout, const Lines &Ls, float res, int form,
                          const MorphEpi &me, cudaStream_t st, int cap)
{
    const float a = res * res;
    const float inv_a = 1.0f / a;
    const int block = 128;
    const size_t smem = (size_t)kRing * block * (sizeof(int) + sizeof(short));
    const int n = (int)(Ls.ax == 0 ? Ls.s0 : Ls.ax == 1 ? Ls.s1 : Ls.s2);
    {
        const int ps__ = prof_begin("k_env_exact", st);
        k_env_exact<<<grid_for(Ls.count(), block, 1LL << 30), block, smem, st>>>(fin, fout, Ls, a, inv_a,
                                                                                  form, me, cap);
        prof_end(ps__,
                 (double)Ls.count() * n * 4 +
                     (form == PMG_EDT_MORPH ? (double)Ls.count() * me.o2 : (double)Ls.count() * n * 4),
                 st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

// ---------------------------------------------------------------------------
// Last morphology pass as a union of intervals.  With exact integer heights K_v
// (units of res^2) the squared distance is E(x) = min_v K_v + (x - v)^2, and
// the epilogue's test "within" is E(x) <= T for the integer T found by
// morph_threshold.  A height K_v <= T therefore covers exactly the positions
// |x - v| <= w_v = floor(sqrt(T - K_v)), and x is within iff some interval
// covers it: a forward max-scan of v + w_v and a backward min-scan of
// v - w_v decide every position without a stack.  One warp per line, lanes
// on 32 consecutive positions; n <= 2048 keeps one coverage bit per chunk in
// a 64-bit mask.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int isqrt_floor(int m)
{
    int r = (int)__fsqrt_rn((float)m); // m < 2^24: exact operand, result off by at most 1
    if (r * r > m)
        r--;
    else if ((r + 1) * (r + 1) <= m)
        r++;
    return r;
}

__global__ void __launch_bounds__(256) k_env_thresh(const float *__restrict__ fin, Lines Ls, float inv_a,
                                                    float fT, int T, MorphEpi me)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long nlines = Ls.count();
    for (long long li = warp; li < nlines; li += nwarps) {
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        const long long st = g.stride;
        const int n = g.n;
        const int nc = (n + 31) >> 5;
        uint64_t fwd = 0;
        int carry = INT_MIN;
        for (int c = 0; c < nc; c++) {
            const int x = (c << 5) + lane;
            int r = INT_MIN;
            if (x < n) {
                const float f = line[x * st];
                if (f <= fT)
                    r = x + isqrt_floor(T - (int)fmul(f, inv_a));
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(FULL, r, off);
                if (lane >= off)
                    r = max(r, t);
            }
            r = max(r, carry);
            carry = __shfl_sync(FULL, r, 31);
            if (r >= x)
                fwd |= 1ull << c;
        }
        carry = INT_MAX;
        for (int c = nc - 1; c >= 0; c--) {
            const int x = (c << 5) + lane;
            int l = INT_MAX;
            if (x < n) {
                const float f = line[x * st];
                if (f <= fT)
                    l = x - isqrt_floor(T - (int)fmul(f, inv_a));
            }
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_down_sync(FULL, l, off);
                if (lane + off < 32)
                    l = min(l, t);
            }
            l = min(l, carry);
            carry = __shfl_sync(FULL, l, 0);
            if (x < n)
                morph_put(me, g, x, ((fwd >> c) & 1ull) || l <= x);
        }
    }
}

int morph_threshold(const MorphEpi &me, float a, int lim)
{
    if (!morph_within(me, 0.0f))
        return -1;
    if (morph_within(me, (float)lim * a))
        return lim;
    int lo = 0, hi = lim; // within(lo), not within(hi)
    while (hi - lo > 1) {
        const int mid = lo + (hi - lo) / 2;
        if (morph_within(me, (float)mid * a))
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

int launch_env_thresh(const float *fin, const Lines &Ls, float res, int T, const MorphEpi &me,
                      cudaStream_t st)
{
    const float a = res * res;
    const float inv_a = 1.0f / a;
    const float fT = T >= 0 ? (float)T * a : -1.0f;
    const int n = (int)(Ls.ax == 0 ? Ls.s0 : Ls.ax == 1 ? Ls.s1 : Ls.s2);
    if (n > 2048) {
        set_error("threshold pass: line length %d above 2048", n);
        return PMG_ERANGE;
    }
    const int block = 256;
    {
        const int ps__ = prof_begin("k_env_thresh", st);
        k_env_thresh<<<grid_for(Ls.count() * 32, block, 152LL * 16), block, 0, st>>>(fin, Ls, inv_a, fT, T,
                                                                                      me);
        prof_end(ps__, (double)Ls.count() * n * 4 + (double)Ls.count() * me.o2, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

} // namespace pmg
