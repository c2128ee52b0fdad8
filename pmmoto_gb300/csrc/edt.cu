// Exact Euclidean distance transform on GB300 (sm_103a).
//
// Three kernels, one thread per 1-D line, lanes of a warp on neighbouring
// lines so that the strided axes are read and written coalesced:
//
//  * k_pass0     -- the linear two-sweep pass of squared_edt_1d
//                   (src/pmmoto/filters/distance/_distance.hpp:135-182) with
//                   the periodic correctors of _distance.pyx:240-279 /
//                   euclidean_distance_transform.py:395-447 found in-kernel.
//  * k_envelope  -- the lower envelope of parabolas of
//                   squared_edt_1d_parabolic (_distance.hpp:184-272) with the
//                   periodic boundary hulls of return_boundary_hull
//                   (_distance.hpp:296-356) computed in-kernel from the same
//                   line, so the MPI feature exchange of the reference becomes
//                   index arithmetic.
//
// The envelope stack is kept as a bitmask of surviving vertices in shared
// memory (one bit per voxel of the line, words interleaved across the block so
// every access is bank-conflict free).  A vertex's height is re-read from the
// input line and a segment's range is recomputed from the two neighbouring
// vertices with the same float expression the reference used when it pushed
// the segment, so the result is bit-identical while the per-line state is
// n/8 bytes instead of 16 n bytes.
//
// All floating-point steps use round-to-nearest intrinsics with no
// multiply-add contraction, in the reference's operation order.
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <cooperative_groups.h>

#include "edt_internal.cuh"

namespace pmg {


// ---------------------------------------------------------------------------
// pass 0: squared_edt_1d along axis `ax`
// ---------------------------------------------------------------------------
__global__ void k_pass0(const uint8_t *__restrict__ img, float *__restrict__ out, Lines Ls,
                        float res, pmg_axis_cfg cfg)
{
    const long long nlines = Ls.count();
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < nlines;
         li += (long long)gridDim.x * blockDim.x) {
        const LineGeo g = line_addr(Ls, li);
        const uint8_t *in = img + g.base;
        float *d = out + g.base;
        const long long st = g.stride;
        const int n = g.n;
        float lc = INFINITY, uc = INFINITY;
        if (cfg.periodic) {
            int F = -1, L = -1;
            for (int i = cfg.f_lo; i < n; i++)
                if (in[i * st] == 0) {
                    F = i;
                    break;
                }
            for (int i = n - cfg.l_hi - 1; i >= cfg.l_lo; i--)
                if (in[i * st] == 0) {
                    L = i;
                    break;
                }
            if (F != -1)
                uc = (float)(F + cfg.a_u);
            if (L != -1)
                lc = (float)(n - L + cfg.a_l);
        }
        // forward sweep (reset at zeros, restart at a change of nonzero value)
        uint8_t seg = in[0];
        float prev = seg == 0 ? 0.0f : fmul(lc, res);
        d[0] = prev;
        uint8_t prev_v = seg;
        for (int i = 1; i < n; i++) {
            const uint8_t v = in[i * st];
            float cur;
            if (v == 0) {
                cur = 0.0f;
            } else if (v == seg) {
                cur = fadd(prev, res);
            } else {
                cur = res;
                d[(i - 1) * st] = prev_v != 0 ? res : 0.0f;
                seg = v;
            }
            d[i * st] = cur;
            prev = cur;
            prev_v = v;
        }
        // clamp the last voxel, backward sweep, square, inf -> FLT_MAX
        float b = d[(n - 1) * st];
        const float ucr = fmul(uc, res);
        if (b > ucr)
            b = ucr;
        {
            float q = fmul(b, b);
            d[(n - 1) * st] = q == INFINITY ? FLT_MAX : q;
        }
        for (int i = n - 2; i >= 0; i--) {
            const float a = d[i * st];
            b = fminf(a, fadd(b, res));
            const float q = fmul(b, b);
            d[i * st] = q == INFINITY ? FLT_MAX : q;
        }
    }
}

// k_pass0 on four adjacent strided lines per thread (their voxels are
// adjacent along the contiguous axis): uchar4 loads of the image and float4
// loads and stores of the distances, each of the four lines with the same
// state and the same float operations as k_pass0.
__global__ void __launch_bounds__(256) k_pass0_x4(const uint8_t *__restrict__ img, float *__restrict__ out, Lines Ls,
                                                  float res, pmg_axis_cfg cfg)
{
    const long long nquads = Ls.count() >> 2;
    for (long long qi = blockIdx.x * (long long)blockDim.x + threadIdx.x; qi < nquads;
         qi += (long long)gridDim.x * blockDim.x) {
        const LineGeo g = line_addr(Ls, qi * 4);
        const uint8_t *in = img + g.base;
        float *d = out + g.base;
        const long long st = g.stride;
        const int n = g.n;
        float lc[4] = {INFINITY, INFINITY, INFINITY, INFINITY}, uc[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
        if (cfg.periodic) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                int F = -1, L = -1;
                for (int i = cfg.f_lo; i < n; i++)
                    if (in[i * st + q] == 0) {
                        F = i;
                        break;
                    }
                for (int i = n - cfg.l_hi - 1; i >= cfg.l_lo; i--)
                    if (in[i * st + q] == 0) {
                        L = i;
                        break;
                    }
                if (F != -1)
                    uc[q] = (float)(F + cfg.a_u);
                if (L != -1)
                    lc[q] = (float)(n - L + cfg.a_l);
            }
        }
        // forward sweep (reset at zeros, restart at a change of nonzero value)
        const uchar4 v0 = *reinterpret_cast<const uchar4 *>(in);
        uint8_t seg[4] = {v0.x, v0.y, v0.z, v0.w};
        uint8_t prev_v[4] = {v0.x, v0.y, v0.z, v0.w};
        float prev[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
            prev[q] = seg[q] == 0 ? 0.0f : fmul(lc[q], res);
        *reinterpret_cast<float4 *>(d) = make_float4(prev[0], prev[1], prev[2], prev[3]);
#pragma unroll 4
        for (int i = 1; i < n; i++) {
            const uchar4 vv = *reinterpret_cast<const uchar4 *>(in + i * st);
            const uint8_t v[4] = {vv.x, vv.y, vv.z, vv.w};
            float cur[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (v[q] == 0) {
                    cur[q] = 0.0f;
                } else if (v[q] == seg[q]) {
                    cur[q] = fadd(prev[q], res);
                } else {
                    cur[q] = res;
                    d[(i - 1) * st + q] = prev_v[q] != 0 ? res : 0.0f;
                    seg[q] = v[q];
                }
                prev[q] = cur[q];
                prev_v[q] = v[q];
            }
            *reinterpret_cast<float4 *>(d + i * st) = make_float4(cur[0], cur[1], cur[2], cur[3]);
        }
        // clamp the last voxel, backward sweep, square, inf -> FLT_MAX
        float b[4];
        {
            const float4 t = *reinterpret_cast<const float4 *>(d + (n - 1) * st);
            const float tv[4] = {t.x, t.y, t.z, t.w};
            float q4[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                b[q] = tv[q];
                const float ucr = fmul(uc[q], res);
                if (b[q] > ucr)
                    b[q] = ucr;
                const float sq = fmul(b[q], b[q]);
                q4[q] = sq == INFINITY ? FLT_MAX : sq;
            }
            *reinterpret_cast<float4 *>(d + (n - 1) * st) = make_float4(q4[0], q4[1], q4[2], q4[3]);
        }
#pragma unroll 4
        for (int i = n - 2; i >= 0; i--) {
            const float4 t = *reinterpret_cast<const float4 *>(d + i * st);
            const float tv[4] = {t.x, t.y, t.z, t.w};
            float q4[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                b[q] = fminf(tv[q], fadd(b[q], res));
                const float sq = fmul(b[q], b[q]);
                q4[q] = sq == INFINITY ? FLT_MAX : sq;
            }
            *reinterpret_cast<float4 *>(d + i * st) = make_float4(q4[0], q4[1], q4[2], q4[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// envelope stack kept as a bitmask in shared memory
// ---------------------------------------------------------------------------
struct Entry {
    int v;
    float h;
};

struct Stack {
    uint32_t *bm; // word w of this thread at bm[w * nthr]
    int nthr;
    // imported lower hulls, bottom -> top (given ranges)
    int lv[kMaxHull];
    float lh[kMaxHull], lr[kMaxHull];
    int nl;
    // imported upper hulls pushed after the native vertices
    int uv[kMaxHull];
    float uh[kMaxHull], ur[kMaxHull];
    int nu;
    // native vertices (bits); ntv = topmost native vertex or -1
    int nn, ntv;
    // cached top of the whole stack
    int tv;
    float th, tr;

    __device__ __forceinline__ uint32_t &word(int w) { return bm[(long long)w * nthr]; }
    __device__ __forceinline__ void setbit(int v) { word(v >> 5) |= (1u << (v & 31)); }
    __device__ __forceinline__ void clrbit(int v) { word(v >> 5) &= ~(1u << (v & 31)); }
    // highest set bit strictly below v (callers guarantee one exists; the
    // search still stops at word 0 so a broken invariant cannot leave the
    // thread's shared-memory words)
    __device__ __forceinline__ int prev_bit(int v)
    {
        int w = v >> 5;
        uint32_t m = word(w) & ((1u << (v & 31)) - 1u);
        while (m == 0) {
            if (w == 0)
                return 0;
            --w;
            m = word(w);
        }
        return (w << 5) + 31 - __clz(m);
    }
    // lowest set bit strictly above v, or -1 if none below `lim` bits
    __device__ __forceinline__ int next_bit(int v, int nwords)
    {
        int w = (v + 1) >> 5;
        if (w >= nwords)
            return -1;
        uint32_t m = (v + 1) & 31 ? word(w) & ~((1u << ((v + 1) & 31)) - 1u) : word(w);
        while (m == 0) {
            if (++w >= nwords)
                return -1;
            m = word(w);
        }
        return (w << 5) + __ffs(m) - 1;
    }
    __device__ __forceinline__ void clear(int nwords)
    {
        for (int w = 0; w < nwords; w++)
            word(w) = 0u;
    }
};

// Height of a native vertex (re-read from the input line).
__device__ __forceinline__ float vh(const float *line, long long st, int v) { return line[v * st]; }

// Range of the native vertex `v` = intersection with the entry below it.
__device__ __forceinline__ float native_range(Stack &S, const float *line, long long st, int v,
                                              float h, float aniso, int below_native_count)
{
    if (below_native_count > 0) {
        int pv = S.prev_bit(v);
        return isect(h, (float)v, vh(line, st, pv), (float)pv, aniso);
    }
    if (S.nl > 0)
        return isect(h, (float)v, S.lh[S.nl - 1], (float)S.lv[S.nl - 1], aniso);
    return -INFINITY;
}

// Pop the top entry and reload the cache with the new top.
__device__ __forceinline__ void pop_top(Stack &S, const float *line, long long st, float aniso)
{
    if (S.nu > 0) {
        --S.nu;
        if (S.nu > 0) {
            S.tv = S.uv[S.nu - 1];
            S.th = S.uh[S.nu - 1];
            S.tr = S.ur[S.nu - 1];
            return;
        }
    } else if (S.nn > 0) {
        S.clrbit(S.ntv);
        --S.nn;
        S.ntv = S.nn > 0 ? S.prev_bit(S.ntv) : -1;
    } else {
        --S.nl;
    }
    if (S.nn > 0) {
        S.tv = S.ntv;
        S.th = vh(line, st, S.ntv);
        S.tr = native_range(S, line, st, S.ntv, S.th, aniso, S.nn - 1);
    } else {
        S.tv = S.lv[S.nl - 1];
        S.th = S.lh[S.nl - 1];
        S.tr = S.lr[S.nl - 1];
    }
}

// update_hull (_distance.hpp:89-112) for vertex i with height f; `kind`
// 0 = native vertex (a bit), 1 = imported upper hull.
__device__ __forceinline__ void insert(Stack &S, const float *line, long long st, int i, float f,
                                       float aniso, int kind)
{
    float s = isect(f, (float)i, S.th, (float)S.tv, aniso);
    while (S.nl + S.nn + S.nu > 1 && s <= S.tr) {
        pop_top(S, line, st, aniso);
        s = isect(f, (float)i, S.th, (float)S.tv, aniso);
    }
    if (kind == 0) {
        S.setbit(i);
        ++S.nn;
        S.ntv = i;
    } else {
        S.uv[S.nu] = i;
        S.uh[S.nu] = f;
        S.ur[S.nu] = s;
        ++S.nu;
    }
    S.tv = i;
    S.th = f;
    S.tr = s;
}

// Build the envelope of a line segment [0, n) of `line` with no imports:
// entry (0, f(0)) at the bottom, then vertices 1..n-1.
__device__ __forceinline__ void build_plain(Stack &S, const float *line, long long st, int n,
                                            float aniso)
{
    S.nl = 0;
    S.nu = 0;
    S.setbit(0);
    S.nn = 1;
    S.ntv = 0;
    S.tv = 0;
    S.th = vh(line, st, 0);
    S.tr = -INFINITY;
    for (int i = 1; i < n; i++)
        insert(S, line, st, i, vh(line, st, i), aniso, 0);
}

// Iterator over the final stack, bottom to top.
struct Iter {
    int phase; // 0 lower, 1 native, 2 upper, 3 done
    int idx;   // lower/upper index or native vertex
};

__device__ __forceinline__ bool iter_next(Stack &S, Iter &it, const float *line, long long st,
                                          int nwords, Entry &e, int &is_lower, float &given_r)
{
    for (;;) {
        if (it.phase == 0) {
            if (it.idx < S.nl) {
                e.v = S.lv[it.idx];
                e.h = S.lh[it.idx];
                given_r = S.lr[it.idx];
                is_lower = 1;
                ++it.idx;
                return true;
            }
            it.phase = 1;
            it.idx = -1;
        }
        if (it.phase == 1) {
            int nb = S.nn > 0 ? S.next_bit(it.idx, nwords) : -1;
            if (nb >= 0) {
                it.idx = nb;
                e.v = nb;
                e.h = vh(line, st, nb);
                is_lower = 0;
                return true;
            }
            it.phase = 2;
            it.idx = 0;
        }
        if (it.phase == 2) {
            if (it.idx < S.nu) {
                e.v = S.uv[it.idx];
                e.h = S.uh[it.idx];
                is_lower = 0;
                ++it.idx;
                return true;
            }
            it.phase = 3;
        }
        return false;
    }
}

// return_boundary_hull (_distance.hpp:296-356) on segment [start, start+nv)
// of the line: keep up to num_hull+1 finite parabolas from the chosen end,
// vertices and ranges shifted by `corr`.  Returns the count; the bitmask is
// left cleared.
__device__ int boundary_hull(Stack &S, const float *line, long long st, int start, int nv,
                             float aniso, int num_hull, int corr, bool forward, int *ov,
                             float *oh, float *orr)
{
    const float *seg = line + (long long)start * st;
    if (nv <= 0)
        return 0;
    if (nv == 1) {
        const float f0 = seg[0];
        if (f0 < FLT_MAX) {
            ov[0] = corr;
            oh[0] = f0;
            orr[0] = INFINITY;
            return 1;
        }
        // the reference reads its "phantom" second slot here: vertex 0, height 0
        ov[0] = corr;
        oh[0] = 0.0f;
        orr[0] = INFINITY;
        return 1;
    }
    const int nwords = (nv + 31) >> 5;
    build_plain(S, seg, st, nv, aniso);
    const int top = S.nn - 1; // stack index of the top entry
    const int keep = num_hull < top ? num_hull : top;
    int cnt = 0;
    if (forward) {
        int v = -1;
        float prev_h = 0.0f;
        int prev_v = 0;
        for (int k = 0; k <= top && cnt <= keep; k++) {
            v = S.next_bit(v, nwords);
            const float h = vh(seg, st, v);
            const float r = k == 0 ? -INFINITY : isect(h, (float)v, prev_h, (float)prev_v, aniso);
            if (h < FLT_MAX) {
                ov[cnt] = v + corr;
                oh[cnt] = h;
                orr[cnt] = fadd(r, (float)corr);
                ++cnt;
                if (h == 0.9f)
                    break;
            }
            prev_h = h;
            prev_v = v;
        }
    } else {
        int v = S.ntv;
        float h = vh(seg, st, v);
        for (int k = top; k >= 0 && cnt <= keep; k--) {
            int pv = 0;
            float ph = 0.0f, r;
            if (k > 0) {
                pv = S.prev_bit(v);
                ph = vh(seg, st, pv);
                r = isect(h, (float)v, ph, (float)pv, aniso);
            } else {
                r = -INFINITY;
            }
            if (h < FLT_MAX) {
                ov[cnt] = v + corr;
                oh[cnt] = h;
                orr[cnt] = fadd(r, (float)corr);
                ++cnt;
                if (h == 0.9f)
                    break;
            }
            v = pv;
            h = ph;
        }
    }
    S.clear(nwords);
    return cnt;
}

// ---------------------------------------------------------------------------
// envelope pass along axis `ax`: fin -> fout (out of place)
// ---------------------------------------------------------------------------

// The imported boundary hulls of a periodic line (return_boundary_hull on the
// segment before the first zero and after the last zero, the far end's hull
// becoming the lower imports): lower imports into S, upper ones into up_*.
__device__ __forceinline__ void load_imports(Stack &S, const float *line, long long st, int n, float aniso,
                                             const pmg_axis_cfg &cfg, int num_hull, int *up_v, float *up_h,
                                             float *up_r, int &n_up)
{
    // first / last zero (a zero height is exactly a zero voxel of the
    // original image: pass 0 gives 0 only there and every later pass keeps
    // it, all other values being >= res^2 > 0)
    int bf = -1, bb = -1;
    for (int i = cfg.hf_lo; i < n; i++)
        if (line[i * st] == 0.0f) {
            bf = i;
            break;
        }
    for (int i = n - cfg.hb_hi - 1; i >= 0; i--)
        if (line[i * st] == 0.0f) {
            bb = i;
            break;
        }
    // near end (forward) -> upper imports
    int start, nv, corr;
    if (bf == -1) {
        start = cfg.hf_lo;
        nv = n - cfg.hf_lo;
    } else {
        start = cfg.hf_lo;
        nv = bf - cfg.hf_lo + 1;
    }
    corr = 0;
    n_up = boundary_hull(S, line, st, start, nv, aniso, num_hull, corr, true, up_v, up_h, up_r);
    // far end (backward) -> lower imports, given in top-down order
    int lo_v[kMaxHull];
    float lo_h[kMaxHull], lo_r[kMaxHull];
    if (bb == -1) {
        start = 0;
        nv = n - cfg.hb_hi;
    } else {
        start = bb;
        nv = n - bb - cfg.hb_hi;
    }
    corr = -nv;
    const int n_lo = boundary_hull(S, line, st, start, nv, aniso, num_hull, corr, false, lo_v, lo_h, lo_r);
    // the reference pushes the lower list in reverse (rbegin..rend)
    for (int j = 0; j < n_lo; j++) {
        S.lv[j] = lo_v[n_lo - 1 - j];
        S.lh[j] = lo_h[n_lo - 1 - j];
        S.lr[j] = lo_r[n_lo - 1 - j];
    }
    S.nl = n_lo;
}

// Evaluation sweep over the final stack (bottom to top), written for
// positions [i_lo, i_hi) of the line.
__device__ __forceinline__ void evaluate(Stack &S, const float *line, long long st, int nwords, float aniso,
                                         int form, const MorphEpi &me, const LineGeo &g, float *o, int i_lo,
                                         int i_hi)
{
    Iter it{0, 0};
    Entry cur, nxt;
    int is_lower;
    float given_r;
    iter_next(S, it, line, st, nwords, cur, is_lower, given_r);
    bool has_next = iter_next(S, it, line, st, nwords, nxt, is_lower, given_r);
    float nr = has_next ? (is_lower ? given_r : isect(nxt.h, (float)nxt.v, cur.h, (float)cur.v, aniso)) : INFINITY;
    for (int i = i_lo; i < i_hi; i++) {
        const float fi = (float)i;
        while (nr < fi) {
            cur = nxt;
            has_next = iter_next(S, it, line, st, nwords, nxt, is_lower, given_r);
            nr = has_next ? (is_lower ? given_r : isect(nxt.h, (float)nxt.v, cur.h, (float)cur.v, aniso))
                          : INFINITY;
        }
        const float dx = (float)(i - cur.v);
        float val = fadd(fmul(aniso, fmul(dx, dx)), cur.h);
        if (form == PMG_EDT_MORPH) {
            morph_store(me, g, i, val);
            continue;
        }
        if (form == PMG_EDT_DIST)
            val = __fsqrt_rn(val);
        o[i * st] = val;
    }
}

// The choice a windowed pass makes from its probe (k_env_probe, below):
// count[0] and count[1] are the samples the +-8 and the +-12 windows do not
// finish.  Choice 0 runs the +-8 line-pair kernels, 1 the +-12 ones, 2 the
// float envelope on every line; the kernels of the other choices return at
// once.  Without a probe the +-12 window runs.
// count[2] counts those the +-24 window does not finish: below thr24 (the
// strided passes only) the +-24 kernel takes a pass the +-12 one would
// leave to the envelope (choice 3).
struct Probe {
    const int *count;
    int thr8, thr12, thr24;
    __device__ __forceinline__ int choice() const
    {
        if (!count)
            return 1;
        if (count[0] < thr8)
            return 0;
        if (count[1] < thr12)
            return 1;
        return count[2] < thr24 ? 3 : 2;
    }
};

template <int W>
__host__ __device__ constexpr int window_choice()
{
    static_assert(W == 8 || W == 12 || W == 24, "windows of +-8, +-12 and +-24");
    return W == 8 ? 0 : W == 12 ? 1 : 3;
}

__global__ void k_envelope(const float *__restrict__ fin, float *__restrict__ fout, Lines Ls, float res,
                           pmg_axis_cfg cfg, int num_hull, int form, MorphEpi me, int redo, Probe probe)
{
    // behind the windowed kernels: every line, when the probe chose the envelope
    if (probe.count && probe.choice() != 2)
        return;
    const long long nlines = Ls.count();
    extern __shared__ uint32_t smem_bm[];
    const float aniso = fmul(res, res);
    Stack S;
    S.bm = smem_bm + threadIdx.x;
    S.nthr = blockDim.x;
    for (long long li = blockIdx.x * (long long)blockDim.x + threadIdx.x; li < nlines;
         li += (long long)gridDim.x * blockDim.x) {
        const LineGeo g = line_addr(Ls, li);
        // second chance for lines the exact streaming kernel handed back
        if (redo && !line_marked(fout, me, g, form))
            continue;
        const float *line = fin + g.base;
        const long long st = g.stride;
        const int n = g.n;
        const int nwords = (n + 31) >> 5;
        S.clear(nwords);
        S.nl = 0;
        S.nu = 0;
        int up_v[kMaxHull];
        float up_h[kMaxHull], up_r[kMaxHull];
        int n_up = 0;
        if (cfg.periodic)
            load_imports(S, line, st, n, aniso, cfg, num_hull, up_v, up_h, up_r, n_up);
        // main build
        int loop_start;
        if (S.nl > 0) {
            loop_start = 0;
            S.nn = 0;
            S.ntv = -1;
            S.tv = S.lv[S.nl - 1];
            S.th = S.lh[S.nl - 1];
            S.tr = S.lr[S.nl - 1];
        } else {
            loop_start = 1;
            S.setbit(0);
            S.nn = 1;
            S.ntv = 0;
            S.tv = 0;
            S.th = vh(line, st, 0);
            S.tr = -INFINITY;
        }
        for (int i = loop_start; i < n; i++)
            insert(S, line, st, i, vh(line, st, i), aniso, 0);
        for (int j = 0; j < n_up; j++)
            insert(S, line, st, up_v[j] + n, up_h[j], aniso, 1);
        evaluate(S, line, st, nwords, aniso, form, me, g, fout + g.base, 0, n);
    }
}

// ---------------------------------------------------------------------------
// periodic lines with power-of-two voxels: windowed exact minimum + end
// segments
// ---------------------------------------------------------------------------
// Every height is an exact integer multiple K * res^2, and a zero height (a
// solid voxel) shields everything beyond it: at x, a parabola beyond the
// nearest zero on either side is above that zero's value.  So the result at x
// is the exact minimum of K_v + (x - v)^2 over the voxels v that the scan
// outward from x reaches before (x - v)^2 exceeds the best value, and the
// reference's float32 envelope returns exactly that minimum there (the
// rounding argument of edt_exact.cu) -- unless the scan runs off the end of
// a periodic line, where the imported boundary hulls (a truncated set) come
// into play.  k_env_window computes every voxel whose scan stays inside the
// line and flags the lines with one that does not; k_envelope_ends then
// replays the reference's float envelope on those lines' end segments only:
// the lower imports with the voxels up to the first zero, and the voxels from
// the last zero with the upper imports.  No parabola can pop a zero off the
// stack, so these partial stacks and sweeps make the same float decisions as
// the whole line's.  A line without a zero, with a height that is not an
// exact integer, or with a scan longer than kWinMax is flagged for the whole
// float envelope.

constexpr int kWinMax = 64;

// One voxel: the exact windowed minimum (returns true and the value), or
// false with the flag bits its line needs (2: the whole float envelope, 1: its
// end segments).  Heights are exact multiples of res^2 here (the passes
// before only ever produce such values, or FLT_MAX for a line without a
// solid voxel), so K = f / res^2 and every sum below are exact in float32.
__device__ __forceinline__ bool window_voxel(const float *line, long long st, int n, int x, float inv_a, float kmax,
                                             int periodic, float &best, int &need)
{
    const float f = line[x * st];
    if (f == 0.0f) {
        best = 0.0f;
        return true;
    }
    best = fmul(f, inv_a);
    if (best >= kmax) {
        need = 2;
        return false;
    }
    bool ldone = false, rdone = false;
    for (int t = 1; (float)(t * t) < best; t++) {
        if (t > kWinMax) {
            need = 2;
            return false;
        }
        const float tt = (float)(t * t);
        if (!ldone) {
            const int v = x - t;
            if (v < 0) {
                if (periodic) {
                    need = 1;
                    return false;
                }
                ldone = true;
            } else {
                const float kv = fmul(line[v * st], inv_a);
                if (kv >= kmax) {
                    need = 2;
                    return false;
                }
                best = fminf(best, fadd(kv, tt));
                ldone = kv == 0.0f;
            }
        }
        if (!rdone) {
            const int v = x + t;
            if (v >= n) {
                if (periodic) {
                    need = 1;
                    return false;
                }
                rdone = true;
            } else {
                const float kv = fmul(line[v * st], inv_a);
                if (kv >= kmax) {
                    need = 2;
                    return false;
                }
                best = fminf(best, fadd(kv, tt));
                rdone = kv == 0.0f;
            }
        }
        if (ldone && rdone)
            break;
    }
    return true;
}

// Strided lines: one thread per chunk of kWinChunk voxels of a line,
// neighbouring lines in neighbouring lanes; contiguous lines: one warp per
// line, lanes 32 voxels apart.
constexpr int kWinChunk = 64;

__global__ void k_env_window(const float *__restrict__ fin, float *__restrict__ fout, Lines Ls, float a,
                             float inv_a, int periodic, int form, int *__restrict__ flag,
                             Probe probe)
{
    if (probe.choice() == 2)
        return;
    const long long nlines = Ls.count();
    const LineGeo g0 = line_addr(Ls, 0);
    const int n = g0.n;
    const bool contiguous = g0.stride == 1;
    const int nchunk = contiguous ? 1 : (n + kWinChunk - 1) / kWinChunk;
    const float kmax = 16777216.0f - (float)(3 * n) * (float)(3 * n);
    const int lane = threadIdx.x & 31;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long items = nlines * nchunk;
    const long long first = contiguous ? tid >> 5 : tid, step = contiguous ? nthreads >> 5 : nthreads;
    for (long long it = first; it < items; it += step) {
        const int chunk = (int)(it / nlines);
        const long long li = it - (long long)chunk * nlines;
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        float *o = fout + g.base;
        const long long st = g.stride;
        int need = 0;
        const int x0 = contiguous ? lane : chunk * kWinChunk, dx = contiguous ? 32 : 1;
        const int x1 = contiguous ? n : min(n, x0 + kWinChunk);
        for (int x = x0; x < x1; x += dx) {
            float best = 0.0f;
            int nd = 0;
            if (!window_voxel(line, st, n, x, inv_a, kmax, periodic, best, nd)) {
                need |= nd;
                continue;
            }
            float val = fmul(best, a);
            if (form == PMG_EDT_DIST)
                val = __fsqrt_rn(val);
            o[x * st] = val;
        }
        // bit 1: the whole line needs the float envelope; bit 0: its ends
        if (need)
            atomicOr(flag + li, need);
    }
}

// The line-pair kernels' slow path, out of line: window_voxel from the start
// (t0 = 1), or continued past a window of +-W = t0 - 1 whose exact minimum m0
// (units of res^2, every height in the window an exact integer) is above
// (W + 1)^2.  In the second case no solid voxel lies within the window (one
// would give at most W^2), so the scan from the start would cover the whole
// window: it runs off a periodic line end there (flag 1), or closes the side
// of a non-periodic end there, and otherwise continues at distance W + 1 with
// the best value m0.  Either way the result and the flags are those of
// window_voxel.  Four distances are loaded per side at a time so that the
// loads overlap.
__device__ __forceinline__ bool window_voxel_from(const float *line, long long st, int n, int x, float inv_a,
                                               float kmax, int periodic, int t0, float m0, float *best_out,
                                               int *need)
{
    float best;
    bool ldone, rdone;
    if (t0 <= 1) {
        const float f = line[x * st];
        if (f == 0.0f) {
            *best_out = 0.0f;
            return true;
        }
        best = fmul(f, inv_a);
        if (best >= kmax) {
            *need = 2;
            return false;
        }
        t0 = 1;
        ldone = rdone = false;
    } else {
        const int W = t0 - 1;
        if (periodic && (x + 1 <= W || n - x <= W)) {
            *need = 1;
            return false;
        }
        best = m0;
        ldone = !periodic && x + 1 <= W;
        rdone = !periodic && n - x <= W;
    }
    for (int t = t0; (float)(t * t) < best && !(ldone && rdone); t += 4) {
        float kl[4], kr[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int vl = x - t - q, vr = x + t + q;
            kl[q] = (!ldone && vl >= 0) ? __ldg(line + vl * st) : 0.0f;
            kr[q] = (!rdone && vr < n) ? __ldg(line + vr * st) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int tq = t + q;
            const float tt = (float)(tq * tq);
            if (tt >= best)
                break;
            if (tq > kWinMax) {
                *need = 2;
                return false;
            }
            if (!ldone) {
                if (x - tq < 0) {
                    if (periodic) {
                        *need = 1;
                        return false;
                    }
                    ldone = true;
                } else {
                    const float kv = fmul(kl[q], inv_a);
                    if (kv >= kmax) {
                        *need = 2;
                        return false;
                    }
                    best = fminf(best, fadd(kv, tt));
                    ldone = kv == 0.0f;
                }
            }
            if (!rdone) {
                if (x + tq >= n) {
                    if (periodic) {
                        *need = 1;
                        return false;
                    }
                    rdone = true;
                } else {
                    const float kv = fmul(kr[q], inv_a);
                    if (kv >= kmax) {
                        *need = 2;
                        return false;
                    }
                    best = fminf(best, fadd(kv, tt));
                    rdone = kv == 0.0f;
                }
            }
            if (ldone && rdone)
                break;
        }
    }
    *best_out = best;
    return true;
}

// Voxels the line-pair kernels do not finish in their window are deferred to
// k_env_slow: one 64-bit entry each, the line index (<< 32), the position
// (<< 17), whether the scan continues past the window (<< 16) and the window
// minimum (low 16 bits).  Appends are aggregated over the lanes that defer at
// the same step; when the list is full the line is flagged for the whole float
// envelope instead (a correct, slower result).
__device__ __forceinline__ unsigned long long slow_entry(long long li, int x, bool resume, unsigned m)
{
    return ((unsigned long long)li << 32) | ((unsigned long long)(unsigned)x << 17) |
           ((unsigned long long)(resume ? 1u : 0u) << 16) | (unsigned long long)(resume ? (m & 0xFFFFu) : 0u);
}

__device__ __forceinline__ bool slow_push(unsigned long long *list, int *count, int cap, unsigned long long e)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0)
        base = atomicAdd(count, (int)g.size());
    base = g.shfl(base, 0);
    const int pos = base + (int)g.thread_rank();
    if (pos >= cap)
        return false;
    list[pos] = e;
    return true;
}

// The deferred voxels, one thread each: window_voxel_from, then the output or
// the line's flags (before the flagged lines are listed and replayed).
__global__ void __launch_bounds__(256) k_env_slow(const float *__restrict__ fin, float *__restrict__ fout, Lines Ls,
                                                  float a, float inv_a, int periodic, int form,
                                                  int *__restrict__ flag, const unsigned long long *__restrict__ list,
                                                  const int *__restrict__ count, int cap, Probe probe)
{
    // the window of the kernel that deferred the voxels
    const int ch = probe.choice();
    const int W = ch == 0 ? 8 : ch == 3 ? 24 : 12;
    const int cnt = min(*count, cap);
    const int n = line_addr(Ls, 0).n;
    const float kmax = 16777216.0f - (float)(3 * n) * (float)(3 * n);
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < cnt; it += gridDim.x * blockDim.x) {
        const unsigned long long e = list[it];
        const long long li = (long long)(e >> 32);
        const int x = (int)((e >> 17) & 0x7FFFu);
        const bool resume = (e >> 16) & 1u;
        const LineGeo g = line_addr(Ls, li);
        float best = 0.0f;
        int nd = 0;
        if (!window_voxel_from(fin + g.base, g.stride, n, x, inv_a, kmax, periodic, resume ? W + 1 : 1,
                               (float)(unsigned)(e & 0xFFFFu), &best, &nd)) {
            atomicOr(flag + li, nd);
            continue;
        }
        float val = fmul(best, a);
        if (form == PMG_EDT_DIST)
            val = __fsqrt_rn(val);
        fout[g.base + (long long)x * g.stride] = val;
    }
}

// How often the windowed passes would fall back, sampled before a pass:
// kProbe (line, position) samples spread over the lines; a sample counts for a
// window of +-W when its minimum there is above (W + 1)^2 (not final: the
// per-voxel scan would take it) or the window holds a height that is not an
// integer below 2^16, for W = 8 and W = 12.  Media with wide pores (sphere packs) fall back at most voxels,
// and the per-voxel scans cost several times the float envelope's sweep; so
// when the count reaches the threshold the windowed kernels return at once
// and the float envelope takes every line of the pass.  The choice is made on
// the device (no host round trip) and changes no output: both give the
// reference's values.
constexpr int kProbe = 8192;

__global__ void __launch_bounds__(256) k_env_probe(const float *__restrict__ fin, Lines Ls, float inv_a,
                                                   int *__restrict__ count)
{
    const long long nl = Ls.count();
    if (nl <= 0)
        return;
    const int n = line_addr(Ls, 0).n;
    int c8 = 0, c12 = 0, c24 = 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < kProbe; s += gridDim.x * blockDim.x) {
        const long long li = (long long)(((unsigned long long)s * (unsigned long long)nl) / kProbe);
        const int x = (int)(((unsigned)s * 2654435761u) % (unsigned)n);
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        const long long st = g.stride;
        float best = fmul(line[x * st], inv_a);
        bool bad = !(best < 65000.0f && best == truncf(best));
#pragma unroll
        for (int d = 1; d <= 24; d++) {
            const float dd = (float)(d * d);
            if (x - d >= 0) {
                const float k = fmul(line[(x - d) * st], inv_a);
                bad |= !(k < 65000.0f && k == truncf(k));
                best = fminf(best, fadd(k, dd));
            }
            if (x + d < n) {
                const float k = fmul(line[(x + d) * st], inv_a);
                bad |= !(k < 65000.0f && k == truncf(k));
                best = fminf(best, fadd(k, dd));
            }
            if (d == 8)
                c8 += (bad || best > 81.0f) ? 1 : 0;
            if (d == 12)
                c12 += (bad || best > 169.0f) ? 1 : 0;
        }
        c24 += (bad || best > 625.0f) ? 1 : 0;
    }
    c8 = __reduce_add_sync(0xffffffffu, c8);
    c12 = __reduce_add_sync(0xffffffffu, c12);
    c24 = __reduce_add_sync(0xffffffffu, c24);
    if ((threadIdx.x & 31) == 0) {
        if (c8)
            atomicAdd(count, c8);
        if (c12)
            atomicAdd(count + 1, c12);
        if (c24)
            atomicAdd(count + 2, c24);
    }
}

// Strided lines, two at a time (adjacent along the contiguous axis, packed
// as the halves of 32-bit words of integer heights K = f / res^2): the exact
// minimum of K(x + d) + d^2 over |d| <= W by packed add-min, walking each
// line segment with a register ring of 2W + 1 words.  A minimum m <= (W+1)^2
// is final (every position beyond the window adds at least (W+1)^2); a
// larger one, a window holding a height that is not an integer below 2^16
// (clamped, so no sum wraps) or a periodic line end within reach ((x+1)^2 or
// (n-x)^2 <= m: the per-voxel scan would run off the line there) falls back
// to window_voxel for that voxel, which sets the same line flags as
// k_env_window.  Outputs are those of k_env_window, with far fewer
// divergent loops.
template <int W, int A>
__global__ void __launch_bounds__(256) k_env_pair(const float *__restrict__ fin, float *__restrict__ fout, Lines Ls,
                                                  float a, float inv_a, int periodic, int form, int *__restrict__ flag,
                                                  int seglen, Probe probe,
                                                  unsigned long long *__restrict__ slow, int *__restrict__ slow_count,
                                                  int slow_cap)
{
    if (probe.choice() != window_choice<W>())
        return;
    constexpr int R = 2 * W + 1; // the window of packed heights
    constexpr unsigned kClamp = 65535u - (unsigned)(W * W) - 1u;
    constexpr unsigned kFinal = (unsigned)((W + 1) * (W + 1));
    const long long nlines = Ls.count();
    const long long npairs = nlines >> 1;
    const LineGeo g0 = line_addr(Ls, 0);
    const int n = g0.n;
    const long long st = g0.stride;
    const int nseg = (n + seglen - 1) / seglen;
    const uint32_t big = kClamp * 0x10001u;
    const float2 kOut = make_float2(-1.0f, -1.0f); // marks a position outside the line
    for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < npairs * nseg;
         it += (long long)gridDim.x * blockDim.x) {
        const int seg = (int)(it / npairs);
        const long long li = (it - (long long)seg * npairs) * 2;
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        float *o = fout + g.base;
        const int x0 = seg * seglen, x1 = min(n, x0 + seglen);
        // big_until*: the last output position whose window holds a height
        // that is not an integer below 2^16 (clamped); those outputs take the scan
        int big_until0 = -1, big_until1 = -1;
        auto raw = [&](int y) -> float2 {
            return (y < 0 || y >= n) ? kOut : __ldg(reinterpret_cast<const float2 *>(line + y * st));
        };
        // packing happens when a position enters the window, A positions
        // after its load was issued, so the warp does not wait on the load
        auto pack = [&](float2 f, int y) -> uint32_t {
            if (f.x < 0.0f)
                return big;
            // heights are integers K res^2 when every axis has the same
            // power-of-two voxel size; any other height takes the scan
            const float k0 = fmul(f.x, inv_a), k1 = fmul(f.y, inv_a);
            unsigned u0 = kClamp, u1 = kClamp;
            if (k0 < (float)kClamp && k0 == truncf(k0))
                u0 = (unsigned)k0;
            else
                big_until0 = y + W;
            if (k1 < (float)kClamp && k1 == truncf(k1))
                u1 = (unsigned)k1;
            else
                big_until1 = y + W;
            return u0 | (u1 << 16);
        };
        // win[s] holds position x - W + s; ahead[q] the raw load of position
        // x + W + 1 + q.  The loop is rolled and the window shifts by register
        // moves, so the loop body stays small enough for the instruction cache.
        uint32_t win[R];
        float2 ahead[A];
#pragma unroll
        for (int s2 = 0; s2 < R; s2++)
            win[s2] = pack(raw(x0 - W + s2), x0 - W + s2);
#pragma unroll
        for (int q = 0; q < A; q++)
            ahead[q] = raw(x0 + W + 1 + q);
        int need0 = 0, need1 = 0;
#pragma unroll 1
        for (int x = x0; x < x1; x++) {
            uint32_t m = win[W];
#pragma unroll
            for (int d = 1; d <= W; d++) {
                const uint32_t dd = (uint32_t)(d * d) * 0x10001u;
                m = __viaddmin_u16x2(win[W - d], dd, m);
                m = __viaddmin_u16x2(win[W + d], dd, m);
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const unsigned mh = h ? (m >> 16) : (m & 0xFFFFu);
                // clean: every height in the window is an exact integer below the clamp
                const bool clean = x > (h ? big_until1 : big_until0);
                bool fin_ok = mh <= kFinal && clean;
                const bool resume = mh > kFinal && clean;
                if (fin_ok && periodic) {
                    const unsigned el = (unsigned)((x + 1) * (x + 1)), er = (unsigned)((n - x) * (n - x));
                    if (el < mh || er < mh) {
                        // no solid voxel between x and that line end (it would
                        // bound the minimum below): the scan runs off the line
                        if (h)
                            need1 |= 1;
                        else
                            need0 |= 1;
                        continue;
                    }
                    if (el == mh || er == mh)
                        fin_ok = false;
                }
                if (!fin_ok) {
                    // deferred to k_env_slow
                    if (!slow_push(slow, slow_count, slow_cap, slow_entry(li + h, x, resume, mh))) {
                        if (h)
                            need1 |= 2;
                        else
                            need0 |= 2;
                    }
                    continue;
                }
                float val = fmul((float)mh, a);
                if (form == PMG_EDT_DIST)
                    val = __fsqrt_rn(val);
                o[x * st + h] = val;
            }
#pragma unroll
            for (int s2 = 0; s2 < R - 1; s2++)
                win[s2] = win[s2 + 1];
            win[R - 1] = pack(ahead[0], x + W + 1);
#pragma unroll
            for (int q = 0; q < A - 1; q++)
                ahead[q] = ahead[q + 1];
            ahead[A - 1] = raw(x + W + 1 + A);
        }
        if (need0)
            atomicOr(flag + li, need0);
        if (need1)
            atomicOr(flag + li + 1, need1);
    }
}

// Contiguous lines (the last axis), 64 rows at a time: the rows' heights over
// kRowsTX columns plus a W halo on each side are staged in shared memory as
// packed 16-bit pairs (rows 2p, 2p + 1 in one word; a padded row stride keeps
// the column walk free of bank conflicts), each thread walks 16 columns of
// one row pair with the same register ring as k_env_pair, results go through
// a shared tile to coalesced stores.  A row with a clamped height anywhere in
// its staged span, an inconclusive minimum or a periodic end within reach
// takes window_voxel on the row in global memory, as k_env_window does.
constexpr int kRowsTX = 128;

template <int W>
constexpr size_t rows_smem_bytes()
{
    return sizeof(uint32_t) * 32 * (kRowsTX + 2 * W + 1) + sizeof(float) * 64 * (kRowsTX + 1) + sizeof(int) * 64;
}

template <int W>
__global__ void __launch_bounds__(256) k_env_pair_rows(const float *__restrict__ fin, float *__restrict__ fout,
                                                       Lines Ls, float a, float inv_a, int periodic, int form,
                                                       int *__restrict__ flag, Probe probe,
                                                       unsigned long long *__restrict__ slow,
                                                       int *__restrict__ slow_count, int slow_cap)
{
    if (probe.choice() != window_choice<W>())
        return;
    constexpr int R = 2 * W + 1;
    constexpr int SPAN = kRowsTX + 2 * W;
    constexpr int SROW = SPAN + 1; // padded word stride of a pair row
    constexpr unsigned kClamp = 65535u - (unsigned)(W * W) - 1u;
    constexpr unsigned kFinal = (unsigned)((W + 1) * (W + 1));
    constexpr float kSkip = -1.0f; // "left to k_env_slow or the end-segment replay"
    extern __shared__ uint32_t rows_smem[];
    uint32_t *sin = rows_smem;                                // [32][SROW]
    float *sout = reinterpret_cast<float *>(sin + 32 * SROW); // [64][kRowsTX + 1]
    int *sbig = reinterpret_cast<int *>(sout + 64 * (kRowsTX + 1));
    __shared__ long long sbase[64]; // first element of each staged row
    const long long nlines = Ls.count();
    const int n = (int)Ls.s2;
    const int ntx = (n + kRowsTX - 1) / kRowsTX;
    const long long ntiles = ((nlines + 63) / 64) * ntx;
    const uint32_t big = kClamp * 0x10001u;
    const int tid = threadIdx.x;
    // rows start on 16-byte boundaries when the row length is a multiple of 4
    // (and the volume starts on one)
    const bool vec4 = !(n & 3) && !(reinterpret_cast<uintptr_t>(fin) & 15);
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long li0 = (tile / ntx) * 64;
        const int c0 = (int)(tile % ntx) * kRowsTX;
        const int rows = (int)min(64LL, nlines - li0);
        if (tid < 64) {
            sbig[tid] = 0;
            sbase[tid] = tid < rows ? line_addr(Ls, li0 + tid).base : 0;
        }
        __syncthreads();
        // stage: (pair, 4-column group) items, columns fastest (coalesced
        // rows); 16-byte loads where the rows allow them
        auto pack = [&](int pr, float f0, float f1) -> uint32_t {
            const float k0 = fmul(f0, inv_a), k1 = fmul(f1, inv_a);
            unsigned u0 = kClamp, u1 = kClamp;
            if (k0 < (float)kClamp && k0 == truncf(k0))
                u0 = (unsigned)k0;
            else
                sbig[2 * pr] = 1;
            if (k1 < (float)kClamp && k1 == truncf(k1))
                u1 = (unsigned)k1;
            else
                sbig[2 * pr + 1] = 1;
            return u0 | (u1 << 16);
        };
        static_assert(SPAN % 4 == 0 && W % 4 == 0, "4-column groups");
        for (int it = tid; it < 32 * (SPAN / 4); it += blockDim.x) {
            const int pr = it / (SPAN / 4), cc = (it - pr * (SPAN / 4)) * 4;
            const int c = c0 - W + cc;
            uint32_t wv[4] = {big, big, big, big};
            if (2 * pr < rows) {
                const long long b0 = sbase[2 * pr];
                if (vec4 && c >= 0 && c + 3 < n) {
                    const float4 f0 = __ldg(reinterpret_cast<const float4 *>(fin + b0 + c));
                    const float4 f1 = __ldg(reinterpret_cast<const float4 *>(fin + b0 + (long long)n + c));
                    wv[0] = pack(pr, f0.x, f1.x);
                    wv[1] = pack(pr, f0.y, f1.y);
                    wv[2] = pack(pr, f0.z, f1.z);
                    wv[3] = pack(pr, f0.w, f1.w);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (c + q >= 0 && c + q < n)
                            wv[q] = pack(pr, fin[b0 + c + q], fin[b0 + (long long)n + c + q]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                sin[pr * SROW + cc + q] = wv[q];
        }
        __syncthreads();
        {
            const int pr = tid & 31, seg = tid >> 5; // 8 segments of 16 columns
            const uint32_t *row = sin + pr * SROW;
            const int xs = c0 + seg * 16, xe = min(n, xs + 16);
            int need0 = 0, need1 = 0;
            const long long lia = li0 + 2 * pr;
            if (2 * pr < rows && xs < xe) {
                uint32_t win[R];
#pragma unroll
                for (int s2 = 0; s2 < R; s2++)
                    win[s2] = row[seg * 16 + s2];
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const int x = xs + u;
                    if (x < xe) {
                        uint32_t m = win[(u + W) % R];
#pragma unroll
                        for (int d = 1; d <= W; d++) {
                            const uint32_t dd = (uint32_t)(d * d) * 0x10001u;
                            m = __viaddmin_u16x2(win[(u + W - d) % R], dd, m);
                            m = __viaddmin_u16x2(win[(u + W + d) % R], dd, m);
                        }
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const unsigned mh = h ? (m >> 16) : (m & 0xFFFFu);
                            const bool clean = !sbig[2 * pr + h];
                            bool fin_ok = mh <= kFinal && clean;
                            const bool resume = mh > kFinal && clean;
                            if (fin_ok && periodic) {
                                const unsigned el = (unsigned)((x + 1) * (x + 1)),
                                               er = (unsigned)((n - x) * (n - x));
                                if (el < mh || er < mh) {
                                    // the scan would run off the line: flag it directly
                                    if (h)
                                        need1 |= 1;
                                    else
                                        need0 |= 1;
                                    sout[(2 * pr + h) * (kRowsTX + 1) + (x - c0)] = kSkip;
                                    continue;
                                }
                                if (el == mh || er == mh)
                                    fin_ok = false;
                            }
                            if (!fin_ok) {
                                // deferred to k_env_slow
                                if (!slow_push(slow, slow_count, slow_cap, slow_entry(lia + h, x, resume, mh))) {
                                    if (h)
                                        need1 |= 2;
                                    else
                                        need0 |= 2;
                                }
                                sout[(2 * pr + h) * (kRowsTX + 1) + (x - c0)] = kSkip;
                                continue;
                            }
                            float val = fmul((float)mh, a);
                            if (form == PMG_EDT_DIST)
                                val = __fsqrt_rn(val);
                            sout[(2 * pr + h) * (kRowsTX + 1) + (x - c0)] = val;
                        }
                    }
                    win[u % R] = row[seg * 16 + u + R < SPAN ? seg * 16 + u + R : SPAN - 1];
                }
            }
            if (need0)
                atomicOr(flag + lia, need0);
            if (need1)
                atomicOr(flag + lia + 1, need1);
        }
        __syncthreads();
        // coalesced stores of the tile
        const int tw = min(kRowsTX, n - c0);
        for (int it = tid; it < rows * kRowsTX; it += blockDim.x) {
            const int r = it / kRowsTX, c = it - r * kRowsTX;
            if (c >= tw)
                continue;
            const float v = sout[r * (kRowsTX + 1) + c];
            if (v != kSkip)
                fout[sbase[r] + c0 + c] = v;
        }
        __syncthreads();
    }
}

// Flagged lines, compacted: list[0 .. *count) gets the indices of the lines
// whose flag is set (in no particular order), so the replay's warps only hold
// lines with work.
__global__ void k_flag_list(const int *__restrict__ flag, long long nlines, int *__restrict__ list,
                            int *__restrict__ count)
{
    const int lane = threadIdx.x & 31;
    for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane; base < nlines;
         base += (long long)gridDim.x * blockDim.x) {
        const long long li = base + lane;
        const bool f = li < nlines && flag[li] != 0;
        const unsigned bal = __ballot_sync(0xffffffffu, f);
        if (!bal)
            continue;
        int pos = 0;
        if (lane == 0)
            pos = atomicAdd(count, __popc(bal));
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (f)
            list[pos + __popc(bal & ((1u << lane) - 1u))] = (int)li;
    }
}

// list (optional): the flagged lines' indices and their number (*count);
// without it every line is visited and unflagged ones are skipped.
__global__ void k_envelope_ends(const float *__restrict__ fin, float *__restrict__ fout, Lines Ls, float res,
                                pmg_axis_cfg cfg, int num_hull, int form, const int *__restrict__ flag,
                                const int *__restrict__ list, const int *__restrict__ count)
{
    const long long nlines = list ? (long long)*count : Ls.count();
    extern __shared__ uint32_t smem_bm[];
    const float aniso = fmul(res, res);
    const MorphEpi none{};
    Stack S;
    S.bm = smem_bm + threadIdx.x;
    S.nthr = blockDim.x;
    for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < nlines;
         it += (long long)gridDim.x * blockDim.x) {
        const long long li = list ? (long long)list[it] : it;
        const int fl = flag[li];
        if (!fl)
            continue;
        const LineGeo g = line_addr(Ls, li);
        const float *line = fin + g.base;
        const long long st = g.stride;
        const int n = g.n;
        const int nwords = (n + 31) >> 5;
        int z1 = -1, z2 = -1;
        for (int i = 0; i < n; i++)
            if (line[i * st] == 0.0f) {
                z1 = i;
                break;
            }
        for (int i = n - 1; i >= 0; i--)
            if (line[i * st] == 0.0f) {
                z2 = i;
                break;
            }
        S.clear(nwords);
        S.nl = 0;
        S.nu = 0;
        int up_v[kMaxHull];
        float up_h[kMaxHull], up_r[kMaxHull];
        int n_up = 0;
        if (cfg.periodic)
            load_imports(S, line, st, n, aniso, cfg, num_hull, up_v, up_h, up_r, n_up);
        const bool whole = (fl & 2) || z1 < 0;
        const int lo_end = whole ? n - 1 : z1; // last native of the lower stack
        // lower part: the imports below, natives up to lo_end
        if (whole || z1 > 0) {
            int loop_start;
            if (S.nl > 0) {
                loop_start = 0;
                S.nn = 0;
                S.ntv = -1;
                S.tv = S.lv[S.nl - 1];
                S.th = S.lh[S.nl - 1];
                S.tr = S.lr[S.nl - 1];
            } else {
                loop_start = 1;
                S.setbit(0);
                S.nn = 1;
                S.ntv = 0;
                S.tv = 0;
                S.th = vh(line, st, 0);
                S.tr = -INFINITY;
            }
            for (int i = loop_start; i <= lo_end; i++)
                insert(S, line, st, i, vh(line, st, i), aniso, 0);
            if (whole) {
                for (int j = 0; j < n_up; j++)
                    insert(S, line, st, up_v[j] + n, up_h[j], aniso, 1);
                evaluate(S, line, st, nwords, aniso, form, none, g, fout + g.base, 0, n);
                S.clear(nwords);
                continue;
            }
            evaluate(S, line, st, nwords, aniso, form, none, g, fout + g.base, 0, z1);
            S.clear(nwords);
        }
        // upper part: the zero at z2 at the bottom, natives above it, the
        // upper imports on top
        if (z2 < n - 1) {
            S.nl = 0;
            S.nu = 0;
            S.setbit(z2);
            S.nn = 1;
            S.ntv = z2;
            S.tv = z2;
            S.th = 0.0f;
            S.tr = -INFINITY;
            for (int i = z2 + 1; i < n; i++)
                insert(S, line, st, i, vh(line, st, i), aniso, 0);
            for (int j = 0; j < n_up; j++)
                insert(S, line, st, up_v[j] + n, up_h[j], aniso, 1);
            evaluate(S, line, st, nwords, aniso, form, none, g, fout + g.base, z2 + 1, n);
            S.clear(nwords);
        }
    }
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
int launch_pass0(const uint8_t *img, float *out, const Lines &Ls, float res,
                 const pmg_axis_cfg &cfg, cudaStream_t st)
{
    const int block = 256;
    {
        const int ps__ = prof_begin("k_pass0", st);
        // four adjacent strided lines per thread where the quads align to 16
        // bytes (float4) and 4 bytes (uchar4)
        const bool quads = Ls.ax != 2 && !(Ls.nb2 & 3) && !(Ls.b2lo & 3) && !(Ls.s2 & 3) &&
                           !(reinterpret_cast<uintptr_t>(out) & 15) && !(reinterpret_cast<uintptr_t>(img) & 3);
        if (quads)
            k_pass0_x4<<<grid_for(Ls.count() >> 2, block, 1LL << 30), block, 0, st>>>(img, out, Ls, res, cfg);
        else
            k_pass0<<<grid_for(Ls.count(), block, 1LL << 30), block, 0, st>>>(img, out, Ls, res, cfg);
        prof_end(ps__, (double)Ls.count() * (Ls.ax == 0 ? Ls.s0 : Ls.ax == 1 ? Ls.s1 : Ls.s2) * 5, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

static int envelope_block(int n)
{
    // shared bitmask: ceil(n/32) words per thread; keep <= 48 KB per block
    int words = (n + 31) / 32;
    int block = 256;
    while (block > 32 && (size_t)words * block * 4 > 48 * 1024)
        block >>= 1;
    return block;
}

// power-of-two voxel size and lines of at most 1024 voxels (imported hull
// vertices then stay within the exact float range of the reference's
// intersection arithmetic)
static bool window_path_ok(float res, int n)
{
    if (n > 1024 || !(res > 0.0f))
        return false;
    int ex = 0;
    const float m = frexpf(res, &ex);
    return m == 0.5f && ex > -40 && ex < 40;
}

int launch_envelope(const float *fin, float *fout, const Lines &Ls, float res,
                    const pmg_axis_cfg &cfg, int num_hull, int form, const MorphEpi &me,
                    cudaStream_t st, int cap, int *flag_buf, long long flag_cap)
{
    const int n = (int)(Ls.ax == 0 ? Ls.s0 : Ls.ax == 1 ? Ls.s1 : Ls.s2);
    int block = envelope_block(n);
    size_t smem = (size_t)((n + 31) / 32) * block * 4;
    if (smem > 48 * 1024)
        PMG_CUDA(cudaFuncSetAttribute(k_envelope, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    const int path = tune_value(kTuneEdtPath);
    if (form != PMG_EDT_MORPH && window_path_ok(res, n) && path == 0) {
        // windowed exact minimum everywhere, the float envelope on the end
        // segments of periodic lines (or whole lines) the window kernel flags
        const long long nl = Ls.count();
        // The library's own buffer (ints): flags [0, nl) | the flagged-line
        // list [nl, 2nl) | its count | the probe's count | the deferred count |
        // the deferred voxels (8-byte entries).  A caller's buffer of flag_cap
        // ints: flags in its first half (one block of rows at a time), then
        // the two counts and the deferred voxels; no flagged-line list.
        int *flag = flag_buf, *probe = nullptr, *slow_cnt = nullptr;
        unsigned long long *slow = nullptr;
        long long fcap = nl, slow_cap = 0;
        if (!flag_buf) {
            slow_cap = std::min<long long>(nl * n / 16 + 1024, 1LL << 27);
            const size_t head = ((sizeof(int) * (size_t)(2 * nl + 5)) + 15) & ~(size_t)15;
            void *mem = nullptr;
            PMG_TRY(scratch_alloc(&mem, head + sizeof(unsigned long long) * (size_t)slow_cap, st));
            flag = (int *)mem;
            probe = flag + 2 * nl + 1;
            slow = (unsigned long long *)((char *)mem + head);
        } else {
            fcap = flag_cap / 2;
            probe = flag_buf + fcap;
            const uintptr_t lo = ((uintptr_t)(probe + 4) + 15) & ~(uintptr_t)15, hi = (uintptr_t)(flag_buf + flag_cap);
            slow = (unsigned long long *)lo;
            slow_cap = hi > lo ? (long long)((hi - lo) / sizeof(unsigned long long)) : 0;
        }
        slow_cnt = probe + 3;
        const bool rows_pass = Ls.ax == 2;
        // the +-24 window only for strided passes of many lines (on small
        // volumes its 106-register grid runs too few warps and the envelope
        // is faster), unless its threshold is 8193 (always)
        const int wide = tune_value(kTuneEdtWide);
        const Probe pr{probe, tune_value(rows_pass ? kTuneEdtNarrowRows : kTuneEdtNarrow),
                       tune_value(rows_pass ? kTuneEdtFallbackRows : kTuneEdtFallback),
                       rows_pass || (nl < (1LL << 17) && wide < 8193) ? 0 : wide};
        // a caller-supplied flag buffer smaller than the line count is used
        // for one block of rows (lines along the first other axis) at a time
        const int rows = flag_buf ? (int)std::min<long long>(Ls.nb1, std::max<long long>(1, fcap / Ls.nb2))
                                  : Ls.nb1;
        int s = PMG_OK;
        if (flag_buf && (long long)Ls.nb2 > fcap) {
            set_error("envelope: flag buffer of %lld lines holds less than one row of %d lines", fcap, Ls.nb2);
            s = PMG_EINVAL;
        }
        for (int r0 = 0; s == PMG_OK && r0 < Ls.nb1; r0 += rows) {
            Lines C = Ls;
            C.b1lo = Ls.b1lo + r0;
            C.nb1 = std::min(rows, Ls.nb1 - r0);
            const long long nc = C.count();
            s = cudaMemsetAsync(flag, 0, sizeof(int) * (size_t)nc, st) == cudaSuccess ? PMG_OK : PMG_ECUDA;
            if (s == PMG_OK) // the probe's three counts and the deferred count
                s = cudaMemsetAsync(probe, 0, 4 * sizeof(int), st) == cudaSuccess ? PMG_OK : PMG_ECUDA;
            if (s == PMG_OK) {
                const int ps__ = prof_begin("k_env_probe", st);
                k_env_probe<<<kProbe / 256, 256, 0, st>>>(fin, C, 1.0f / (res * res), probe);
                prof_end(ps__, 0.0, st);
            }
            if (s == PMG_OK) {
                const float a = res * res;
                const bool contiguous = C.ax == 2;
                constexpr int kAhead = 5;
                if (!contiguous && !(C.nb2 & 1) && !(C.b2lo & 1)) {
                    // line pairs along the contiguous axis (float2 aligned);
                    // the +-8 and +-12 kernels both launch, the probe runs one
                    const int seg = tune_value(kTuneEdtPairSeg);
                    const long long work = (nc >> 1) * ((n + seg - 1) / seg);
                    const unsigned grid = (unsigned)grid_for(work, 256, 152LL * tune_value(kTuneEdtPairCtas));
                    const int ps__ = prof_begin("k_env_pair", st);
                    k_env_pair<8, kAhead><<<grid, 256, 0, st>>>(fin, fout, C, a, 1.0f / a, cfg.periodic ? 1 : 0, form,
                                                                flag, seg, pr, slow, slow_cnt, (int)slow_cap);
                    k_env_pair<12, kAhead><<<grid, 256, 0, st>>>(fin, fout, C, a, 1.0f / a, cfg.periodic ? 1 : 0,
                                                                 form, flag, seg, pr, slow, slow_cnt, (int)slow_cap);
                    if (pr.thr24 > 0)
                        k_env_pair<24, kAhead><<<grid, 256, 0, st>>>(fin, fout, C, a, 1.0f / a,
                                                                     cfg.periodic ? 1 : 0, form, flag, seg, pr, slow,
                                                                     slow_cnt, (int)slow_cap);
                    prof_end(ps__, (double)nc * n * 8, st);
                } else if (contiguous && !(C.nb2 & 1) && !(C.b2lo & 1)) {
                    // row pairs through shared-memory tiles
                    const long long tiles = ((nc + 63) / 64) * ((n + kRowsTX - 1) / kRowsTX);
                    const unsigned grid = (unsigned)std::min<long long>(tiles, 152LL * tune_value(kTuneEdtRowsCtas));
                    const size_t sm8 = rows_smem_bytes<8>(), sm12 = rows_smem_bytes<12>();
                    s = cudaFuncSetAttribute(k_env_pair_rows<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sm8) == cudaSuccess &&
                                cudaFuncSetAttribute(k_env_pair_rows<12>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sm12) == cudaSuccess
                            ? PMG_OK
                            : PMG_ECUDA;
                    const int ps__ = prof_begin("k_env_pair_rows", st);
                    if (s == PMG_OK) {
                        k_env_pair_rows<8><<<grid, 256, sm8, st>>>(fin, fout, C, a, 1.0f / a, cfg.periodic ? 1 : 0,
                                                                  form, flag, pr, slow, slow_cnt, (int)slow_cap);
                        k_env_pair_rows<12><<<grid, 256, sm12, st>>>(fin, fout, C, a, 1.0f / a,
                                                                    cfg.periodic ? 1 : 0, form, flag, pr, slow,
                                                                    slow_cnt, (int)slow_cap);
                    }
                    prof_end(ps__, (double)nc * n * 8, st);
                } else {
                    const int ps__ = prof_begin("k_env_window", st);
                    k_env_window<<<grid_for(contiguous ? nc * 32 : nc * ((n + 63) / 64), 256, 152LL * 32), 256, 0,
                                   st>>>(fin, fout, C, a, 1.0f / a, cfg.periodic ? 1 : 0, form, flag, pr);
                    prof_end(ps__, (double)nc * n * 8, st);
                }
                if (s == PMG_OK)
                    s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
                if (s == PMG_OK && !(C.nb2 & 1) && !(C.b2lo & 1)) {
                    // the voxels the line-pair kernels deferred
                    const int ps__ = prof_begin("k_env_slow", st);
                    k_env_slow<<<152 * 8, 256, 0, st>>>(fin, fout, C, a, 1.0f / a, cfg.periodic ? 1 : 0, form, flag,
                                                        slow, slow_cnt, (int)slow_cap, pr);
                    prof_end(ps__, 0.0, st);
                    s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
                }
            }
            if (s == PMG_OK) {
                // the library's own flag buffer has room for the compacted list
                // of flagged lines after the flags; a caller's buffer is used
                // as it is (every line visited)
                int *list = flag_buf ? nullptr : flag + nl, *cnt = flag_buf ? nullptr : flag + 2 * nl;
                if (list) {
                    s = cudaMemsetAsync(cnt, 0, sizeof(int), st) == cudaSuccess ? PMG_OK : PMG_ECUDA;
                    const int ps__ = prof_begin("k_flag_list", st);
                    if (s == PMG_OK)
                        k_flag_list<<<grid_for(nc, 256, 152LL * 16), 256, 0, st>>>(flag, nc, list, cnt);
                    prof_end(ps__, (double)nc * 4, st);
                }
                const int ps__ = prof_begin("k_envelope_ends", st);
                if (s == PMG_OK)
                    k_envelope_ends<<<grid_for(nc, block, 1LL << 30), block, smem, st>>>(
                        fin, fout, C, res, cfg, num_hull, form, flag, list, cnt);
                prof_end(ps__, 0.0, st);
                if (s == PMG_OK)
                    s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
            }
            if (s == PMG_OK) {
                // the whole pass on the float envelope when the probe chose it
                const int ps__ = prof_begin("k_envelope[probed]", st);
                k_envelope<<<grid_for(nc, block, 1LL << 30), block, smem, st>>>(
                    fin, fout, C, res, cfg, num_hull, form, MorphEpi{}, 0, pr);
                prof_end(ps__, 0.0, st);
                s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
            }
        }
        const int s2 = flag_buf ? PMG_OK : scratch_free(flag, st);
        return s != PMG_OK ? s : s2;
    }
    int redo = 0;
    if (path != 2 && exact_path_ok(res, cfg, n)) {
        // exact integer streaming pass; lines it cannot finish are redone below
        PMG_TRY(launch_envelope_exact(fin, fout, Ls, res, form, me, st, cap));
        redo = 1;
    }
    {
        const int ps__ = prof_begin(redo ? "k_envelope_redo" : "k_envelope", st);
        k_envelope<<<grid_for(Ls.count(), block, redo ? 152LL * 8 : 1LL << 30), block, smem, st>>>(
            fin, fout, Ls, res, cfg, num_hull, form, me, redo, Probe{nullptr, 0, 0, 0});
        prof_end(ps__, redo ? 0.0 : (double)Ls.count() * n * 4 + (form == PMG_EDT_MORPH ? (double)Ls.count() * me.o2 : (double)Ls.count() * n * 4), st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

static int check_shape(const int64_t *shape, int nd)
{
    for (int d = 0; d < nd; d++) {
        if (shape[d] <= 0) {
            set_error("shape[%d] = %lld must be positive", d, (long long)shape[d]);
            return PMG_EINVAL;
        }
        if (shape[d] > PMG_MAX_LINE) {
            set_error("shape[%d] = %lld exceeds the line limit %d", d, (long long)shape[d],
                      PMG_MAX_LINE);
            return PMG_ERANGE;
        }
    }
    return PMG_OK;
}

// EDT with one ping-pong buffer: pass 0 -> out, envelope 1: out -> tmp,
// envelope 2: tmp -> out.
int edt3d_run(const uint8_t *img, float *out, float *tmp, const int64_t *shape, const float *res,
              const pmg_axis_cfg *cfg, int num_hull, int form, cudaStream_t st, int *flag_buf,
              long long flag_cap)
{
    MorphEpi none{};
    PMG_TRY(launch_pass0(img, out, all_lines(shape, 0), res[0], cfg[0], st));
    PMG_TRY(launch_envelope(out, tmp, all_lines(shape, 1), res[1], cfg[1], num_hull,
                            PMG_EDT_SQUARED, none, st, INT_MAX, flag_buf, flag_cap));
    PMG_TRY(launch_envelope(tmp, out, all_lines(shape, 2), res[2], cfg[2], num_hull, form, none,
                            st, INT_MAX, flag_buf, flag_cap));
    return PMG_OK;
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_edt3d(const uint8_t *img, float *out, const int64_t shape[3], const float res[3],
                         const pmg_axis_cfg cfg[3], int32_t num_hull, int32_t form, void *stream)
{
    if (!img || !out || !shape || !res || !cfg) {
        set_error("pmg_edt3d: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_shape(shape, 3));
    if (num_hull < 0 || num_hull + 1 > kMaxHull) {
        set_error("pmg_edt3d: num_hull %d outside [0, %d]", num_hull, kMaxHull - 1);
        return PMG_ERANGE;
    }
    cudaStream_t st = as_stream(stream);
    size_t bytes = (size_t)shape[0] * shape[1] * shape[2] * sizeof(float);
    void *tmp = nullptr;
    PMG_TRY(scratch_alloc(&tmp, bytes, st));
    int s = edt3d_run(img, out, (float *)tmp, shape, res, cfg, num_hull, form, st);
    int s2 = scratch_free(tmp, st);
    return s != PMG_OK ? s : s2;
}

extern "C" int pmg_edt2d(const uint8_t *img, float *out, const int64_t shape2[2], const float res[2],
                         const int32_t periodic[2], int32_t num_hull, int32_t form, void *stream)
{
    if (!img || !out || !shape2 || !res || !periodic) {
        set_error("pmg_edt2d: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_shape(shape2, 2));
    if (num_hull < 0 || num_hull + 1 > kMaxHull) {
        set_error("pmg_edt2d: num_hull %d outside [0, %d]", num_hull, kMaxHull - 1);
        return PMG_ERANGE;
    }
    cudaStream_t st = as_stream(stream);
    const int64_t shape[3] = {1, shape2[0], shape2[1]};
    pmg_axis_cfg c_lin = {periodic[1], 0, 0, 0, 1, 0, 0, 0};
    pmg_axis_cfg c_env = {periodic[0], 0, 0, 0, 1, 0, 0, 0};
    size_t bytes = (size_t)shape2[0] * shape2[1] * sizeof(float);
    void *tmp = nullptr;
    PMG_TRY(scratch_alloc(&tmp, bytes, st));
    MorphEpi none{};
    int s = launch_pass0(img, (float *)tmp, all_lines(shape, 2), res[1], c_lin, st);
    if (s == PMG_OK)
        s = launch_envelope((float *)tmp, out, all_lines(shape, 1), res[0], c_env, num_hull, form,
                            none, st);
    int s2 = scratch_free(tmp, st);
    return s != PMG_OK ? s : s2;
}
