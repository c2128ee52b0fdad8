// Capped integer morphology for isotropic power-of-two voxels (sm_103a).
//
// With a voxel size res = 2^k on every axis the reference's float32 squared
// distances are exact integer multiples of res^2 (src/pmmoto/filters/distance/
// _distance.hpp:135-272 performs only exact float operations on them, see
// edt_exact.cu), so the reference's test "sqrt(d2) <= r" (morphological_
// operators.py:103-228) is "E <= T" for the integer squared distance E and one
// integer bound T (morph_threshold).  Only values up to T matter, which gives
// a different, cheaper pipeline with the same result:
//
//   pass A (rows, the contiguous axis): E_A = min(d^2, T + 1), d the distance
//     to the nearest zero of the row -- one warp per row, ballots per chunk of
//     32 voxels, uint16 output;
//   pass B (axis 1, strided): E_B = min(E_A envelope, T + 1) -- one thread
//     per line, lanes on adjacent lines (coalesced), lower envelope of the
//     parabolas with E_A <= T, each output written a fixed W = floor(sqrt T)
//     positions behind the input (no later parabola can lower a value to <= T
//     after that), so all lanes store the same position; live parabolas lie
//     in [i - 2W, i] and fit a 64-entry ring when T <= 1023;
//   pass C (axis 0, strided): a height E_B <= T covers |x - v| <= floor(sqrt(
//     T - E_B)); x is within iff some interval covers it -- one thread per
//     line, a 64-bit window of pending positions, the result fused with the
//     unpadding and the wall rule.
//
// The exact squared EDT is separable in any axis order, so doing the linear
// pass on the contiguous axis leaves both envelope passes on strided axes,
// where a warp reads and writes 32 adjacent voxels at a time.  The reference's
// linear pass restarts at changes between nonzero values (multi-label
// images), which depends on the axis: this pipeline serves binary images only.
#include <type_traits>

#include "edt_internal.cuh"

namespace pmg {

constexpr int kCapRing = 64;

struct CapGeo {
    int X0, X1, X2;       // extended shape
    int j0, nj, k0, nk;   // unextended ranges of axes 1 and 2
};

// ---- x range of the seeds -------------------------------------------------------
// An optional block-plane range of the seeds (kRangeBig encoding, device
// memory): planes outside [hlo, hhi] hold no seed, so the row and envelope
// passes skip them, and the last pass produces only the outputs within W of
// the seeds, [olo, ohi] widened to whole 2x2x2 blocks.
struct SeedRange {
    int hlo, hhi, olo, ohi; // hlo > hhi: no seeds
    __device__ __forceinline__ void load(const int *xr, int n, int W)
    {
        const int a = xr[0], b = xr[1];
        if (a == 0) {
            hlo = olo = 2;
            hhi = ohi = -1;
            return;
        }
        hlo = 2 * (kRangeBig - b);
        hhi = min(2 * (a - 1) + 1, n - 1);
        olo = max(0, hlo - W) & ~1;
        ohi = min(n - 1, (hhi + W) | 1);
    }
};

// ---- pass A: rows -------------------------------------------------------------
// raw == 0: E is the (extended) image whose zeros are the seeds.  raw == 1:
// E is the unextended image of a dilation without periodic axes, read
// directly -- the seeds are its nonzero voxels off the wall planes (the
// logical_not of k_extend's image), so no extended copy is written.
// With blk (raw only), the seeds come from per-block masks over the
// ceil-halved shape (b1, b2 blocks along axes 1 and 2).
struct RowSrc {
    int raw;
    int X1;
    int wall[6];
    const uint8_t *blk;
    int b1, b2;
};

// Only distances d <= W = floor(sqrt T) <= 31 give values below T + 1, so a
// voxel needs the seeds within 31 positions on either side: the row's seeds
// are first gathered as bit words (one ballot per 32 voxels, kept in shared
// memory with an empty word on either side), then every lane finds its
// voxel's nearest seed in the three words around it with one count of
// leading / trailing zeros each way.
__global__ void __launch_bounds__(256) k_cap_rows(const uint8_t *__restrict__ E, uint16_t *__restrict__ KA,
                                                  long long rows, int X2, int T, int W, RowSrc rs,
                                                  const unsigned long long *__restrict__ gate,
                                                  const int *__restrict__ xr, unsigned long long *units)
{
    if (gate && *gate == 0)
        return; // empty seed set: the last pass writes the result alone
    SeedRange sr{0, 0x7fffffff, 0, 0};
    if (xr)
        sr.load(xr, (int)(rows / rs.X1), W);
    extern __shared__ uint32_t s_zw[];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nw = (X2 + 31) >> 5;
    uint32_t *zw = s_zw + (threadIdx.x >> 5) * (nw + 2) + 1; // zw[-1] and zw[nw] stay 0
    if (lane == 0) {
        zw[-1] = 0u;
        zw[nw] = 0u;
    }
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int big = T + 1;
    // with a seed range, only the rows of its planes
    const long long r0 = xr ? (long long)max(sr.hlo, 0) * rs.X1 : 0;
    const long long r1 = xr ? min(rows, (long long)(sr.hhi + 1) * rs.X1) : rows;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && r1 > r0)
        atomicAdd(units, (unsigned long long)((r1 - r0) * X2));
    for (long long r = r0 + warp; r < r1; r += nwarps) {
        const uint8_t *src = E + r * X2;
        bool wrow = false;
        const long long i = r / rs.X1, j = r - (r / rs.X1) * rs.X1;
        if (rs.raw)
            wrow = (rs.wall[0] && i == 0) || (rs.wall[1] && i == rows / rs.X1 - 1) || (rs.wall[2] && j == 0) ||
                   (rs.wall[3] && j == rs.X1 - 1);
        if (wrow) {
            // a wall row holds no seeds
            for (int c = lane; c < nw; c += 32)
                zw[c] = 0u;
        } else if (rs.blk) {
            // the row's bits of its block row: two per block, lanes 2q and
            // 2q + 1 on block q of the chunk
            const uint8_t *brow = rs.blk + ((i >> 1) * rs.b1 + (j >> 1)) * (long long)rs.b2;
            const int bsh = (int)(((i & 1) * 2 + (j & 1)) * 2) + (lane & 1);
#pragma unroll 4
            for (int c = 0; c < nw; c++) {
                const int x = (c << 5) + lane;
                const bool seed = x < X2 && ((brow[x >> 1] >> bsh) & 1);
                const unsigned zm = __ballot_sync(FULL, seed);
                if (lane == 0)
                    zw[c] = zm;
            }
        } else {
            const uint8_t want = rs.raw ? 0 : 1; // a seed is a voxel != want (raw) or == 0
#pragma unroll 4
            for (int c = 0; c < nw; c++) {
                const int x = (c << 5) + lane;
                const bool seed = x < X2 && ((src[x] == 0) != (want == 0));
                const unsigned zm = __ballot_sync(FULL, seed);
                if (lane == 0)
                    zw[c] = zm;
            }
        }
        if (!wrow && rs.raw && lane == 0) {
            // wall planes at the row ends hold no seeds (lane 0 wrote every word)
            if (rs.wall[4])
                zw[0] &= ~1u;
            if (rs.wall[5])
                zw[(X2 - 1) >> 5] &= ~(1u << ((X2 - 1) & 31));
        }
        __syncwarp();
        uint16_t *dst = KA + r * X2;
        uint32_t wp = 0u, wc = zw[0];
        for (int c = 0; c < nw; c++) {
            const uint32_t wn = zw[c + 1];
            const int x = (c << 5) + lane;
            // bit t of R: position x + t; bit 31 - t of L: position x - t
            const uint32_t R = __funnelshift_r(wc, wn, lane);
            const uint32_t L = __funnelshift_l(wp, wc, 31 - lane);
            const int d = min(__clz(L), __clz(__brev(R)));
            if (x < X2)
                dst[x] = (uint16_t)(d <= W ? d * d : big);
            wp = wc;
            wc = wn;
        }
        __syncwarp();
    }
}

// ---- pass B: capped envelope along axis 1 --------------------------------------
// Ring entries pack a height (<= T <= 1023) and a vertex (< 2048): K << 11 | v.
__device__ __forceinline__ int cap_val(int ent, int x)
{
    const int d = x - (ent & 2047);
    return (ent >> 11) + d * d;
}

// Per-line state of the capped envelope; RING (a power of two) >= 2W + 2.
template <int RING>
struct CapLine {
    int *R; // ring slot s of this thread at R[s * 128]
    int bot, top, e;
    __device__ __forceinline__ int &at(int c) const { return R[(c & (RING - 1)) * 128]; }

    // consume height K at position i (K > T: absent), then return the value
    // at x = i - W (big when above T); x < 0 returns nothing meaningful
    __device__ __forceinline__ int step(int i, int K, int T, int W, int big)
    {
        if (K <= T) {
            while (top > bot) {
                const int t = at(top), u = at(top - 1);
                const int Kt = t >> 11, Vt = t & 2047, Ku = u >> 11, Vu = u & 2047;
                const int n1 = K - Kt + (i - Vt) * (i + Vt), d1 = 2 * (i - Vt);
                const int n2 = Kt - Ku + (Vt - Vu) * (Vt + Vu), d2 = 2 * (Vt - Vu);
                if (n1 * d2 > n2 * d1)
                    break;
                if (e == top)
                    e--;
                top--;
            }
            top++;
            at(top) = (K << 11) | i;
            if (top == bot)
                e = bot;
        }
        const int x = i - W;
        if (x < 0)
            return big;
        // parabolas with v + W < x exceed T at every later position
        while (bot <= top && (at(bot) & 2047) + W < x)
            bot++;
        if (e < bot)
            e = bot;
        if (top < bot)
            return big;
        int ce = at(e);
        while (e < top) {
            const int cn = at(e + 1);
            if (cap_val(cn, x) > cap_val(ce, x))
                break;
            ce = cn;
            e++;
        }
        const int Ev = cap_val(ce, x);
        return Ev <= T ? Ev : big;
    }
};

constexpr int kCapChunk = 8; // heights loaded ahead per line (memory-level parallelism)

// AX = 1: lines over (x0 in [0, X0), x2 in [k0, k0 + nk)) along axis 1;
// AX = 0: lines over (x1 in [j0, j0 + nj), x2 in [k0, k0 + nk)) along axis 0.
// One thread per line; each loop trip loads the next kCapChunk heights before
// it processes the current ones, so a thread keeps several loads in flight.
// Lines are cut into nseg segments: an output at x depends only on the
// heights within W of it, so a segment [a, b) is exact when its sweep starts
// at a - W (2W extra steps per segment buy nseg times the threads).
template <int AX, int RING>
__global__ void __launch_bounds__(128) k_cap_mid(const uint16_t *__restrict__ KA, uint16_t *__restrict__ KB,
                                                 CapGeo G, int T, int W, const unsigned long long *__restrict__ gate,
                                                 const int *__restrict__ xr, int nseg, unsigned long long *units)
{
    if (gate && *gate == 0)
        return;
    SeedRange sr{0, 0x7fffffff, 0, 0};
    if (xr)
        sr.load(xr, G.X0, W);
    __shared__ int ring[RING * 128];
    const long long nlines = (long long)(AX == 1 ? G.X0 : G.nj) * G.nk;
    const long long st = AX == 1 ? (long long)G.X2 : (long long)G.X1 * G.X2;
    const int n = AX == 1 ? G.X1 : G.X0;
    const int seglen = (n + nseg - 1) / nseg;
    const int big = T + 1;
    // with a seed range (axis-1 lines), only the lines of its planes
    const long long l0 = AX == 1 && xr ? (long long)max(sr.hlo, 0) * G.nk : 0;
    const long long l1 = AX == 1 && xr ? min(nlines, (long long)(sr.hhi + 1) * G.nk) : nlines;
    const long long span = l1 > l0 ? l1 - l0 : 0;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && span)
        atomicAdd(units, (unsigned long long)(span * n));
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < span * nseg;
         g += (long long)gridDim.x * blockDim.x) {
        const int seg = (int)(g / span);
        const long long li = l0 + (g - (long long)seg * span);
        const long long q = li / G.nk;
        const int a = seg * seglen, b = min(n, a + seglen);
        if (a >= b)
            continue;
        const int x2 = G.k0 + (int)(li - q * G.nk);
        const long long base = AX == 1 ? q * G.X1 * G.X2 + x2 : (G.j0 + q) * G.X2 + x2;
        const uint16_t *in = KA + base;
        uint16_t *out = KB + base;
        CapLine<RING> L{ring + threadIdx.x, 0, -1, 0};
        const int i_first = max(0, a - W), i_last = b - 1 + W; // steps; step i emits x = i - W
        int cur[kCapChunk];
        const uint16_t *pin = in + (long long)i_first * st; // next height to prefetch
#pragma unroll
        for (int u = 0; u < kCapChunk; u++) {
            cur[u] = i_first + u < n ? (int)*pin : big;
            pin += st;
        }
        uint16_t *po = out + (long long)a * st; // output position x = i - W
        for (int i0 = i_first; i0 <= i_last; i0 += kCapChunk) {
            int nxt[kCapChunk];
#pragma unroll
            for (int u = 0; u < kCapChunk; u++) {
                nxt[u] = i0 + kCapChunk + u < n ? (int)*pin : big;
                pin += st;
            }
#pragma unroll
            for (int u = 0; u < kCapChunk; u++) {
                const int i = i0 + u;
                const int v = L.step(i, cur[u], T, W, big);
                const int x = i - W;
                if (x >= a && x < b) {
                    *po = (uint16_t)v;
                    po += st;
                }
            }
#pragma unroll
            for (int u = 0; u < kCapChunk; u++)
                cur[u] = nxt[u];
        }
    }
}

// ---- pass B for small W: direct minima on line pairs ----------------------------
// E_B(y) = min over |d| <= W of E_A(y + d) + d^2: heights above T are stored
// as T + 1 and every term with |d| > W exceeds T, so the capped envelope is
// this minimum over 2W + 1 terms.  Two adjacent lines (x2 and x2 + 1) share a
// thread, packed in the halves of a 32-bit word, and each pair of terms costs
// two packed add-min instructions (values stay below 2^11: no carries between
// the halves).  The heights of a segment live in a register ring of
// R = 2W + 1 + pair_ahead(W) words whose slots are fixed at compile time: at
// step u of a group of R outputs starting at y0, slot s holds position
// y0 - W + s (s >= u) or y0 - W + s + R (s < u), so the term at y + d sits in
// slot (u + W + d) mod R, and the slot of y - W, dead after output y, takes
// position y + W + 1 + pair_ahead(W) (loaded that many steps before its use).
constexpr int kPairMaxW = 20;
// heights loaded ahead: fewer for the wide windows, whose rings hold more
__host__ __device__ constexpr int pair_ahead(int W) { return W <= 12 ? 8 : 4; }

// Lines of a pass on pairs: AX = 1, pairs over (x0 in [0, X0), x2 / 2 in
// [k0 / 2, (k0 + nk) / 2)) along axis 1; AX = 0, pairs over (x1 in [j0, j0 +
// nj), x2 / 2 ...) along axis 0.  Word offset of line pair li and its stride.
template <int AX>
__device__ __forceinline__ long long pair_base(const CapGeo &G, long long li, int np)
{
    const long long q = li / np;
    const long long kp = li - q * np;
    const long long v = AX == 1 ? q * G.X1 * G.X2 + G.k0 : (G.j0 + q) * G.X2 + G.k0;
    return (v >> 1) + kp;
}

template <int AX, int W>
__global__ void __launch_bounds__(256) k_cap_mid_pair(const uint16_t *__restrict__ KA, uint16_t *__restrict__ KB,
                                                      CapGeo G, int T, const unsigned long long *__restrict__ gate,
                                                      const int *__restrict__ xr, int seglen,
                                                      unsigned long long *units)
{
    constexpr int R = 2 * W + 1 + pair_ahead(W);
    if (gate && *gate == 0)
        return;
    SeedRange sr{0, 0x7fffffff, 0, 0};
    if (xr)
        sr.load(xr, G.X0, W);
    const int np = G.nk >> 1;
    const long long nlines = (long long)(AX == 1 ? G.X0 : G.nj) * np;
    const long long st = AX == 1 ? (long long)(G.X2 >> 1) : (long long)G.X1 * (G.X2 >> 1);
    const int n = AX == 1 ? G.X1 : G.X0;
    const int nseg = (n + seglen - 1) / seglen;
    const long long l0 = AX == 1 && xr ? (long long)max(sr.hlo, 0) * np : 0;
    const long long l1 = AX == 1 && xr ? min(nlines, (long long)(sr.hhi + 1) * np) : nlines;
    const long long span = l1 > l0 ? l1 - l0 : 0;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && span)
        atomicAdd(units, (unsigned long long)(span * 2 * n));
    const uint32_t bigp = (uint32_t)(T + 1) * 0x10001u;
    const uint32_t *in0 = (const uint32_t *)KA;
    uint32_t *out0 = (uint32_t *)KB;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < span * nseg;
         g += (long long)gridDim.x * blockDim.x) {
        const int seg = (int)(g / span);
        const long long base = pair_base<AX>(G, l0 + (g - (long long)seg * span), np);
        const uint32_t *in = in0 + base;
        uint32_t *out = out0 + base;
        const int a = seg * seglen, b = min(n, a + seglen);
        uint32_t win[R];
#pragma unroll
        for (int s = 0; s < R; s++) {
            const int y = a - W + s;
            win[s] = y >= 0 && y < n ? __ldg(in + y * st) : bigp;
        }
        for (int y0 = a; y0 < b; y0 += R) {
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int y = y0 + u;
                uint32_t m = win[(u + W) % R];
#pragma unroll
                for (int d = 1; d <= W; d++) {
                    const uint32_t dd = (uint32_t)(d * d) * 0x10001u;
                    m = __viaddmin_u16x2(win[(u + W - d) % R], dd, m);
                    m = __viaddmin_u16x2(win[(u + W + d) % R], dd, m);
                }
                if (y < b)
                    out[y * st] = m;
                const int yn = y + W + 1 + pair_ahead(W);
                win[u] = y < b && yn < n ? __ldg(in + yn * st) : bigp;
            }
        }
    }
}

// ---- pass C: intervals along axis 0, fused epilogue ----------------------------
__device__ __forceinline__ int isqrt_small(int m)
{
    int r = (int)__fsqrt_rn((float)m);
    if (r * r > m)
        r--;
    else if ((r + 1) * (r + 1) <= m)
        r++;
    return r;
}

// gate: a count of the seeds held in device memory (null: always seeds); when
// it is zero the dilation is empty and only zeros are written.
// Lines are cut into nseg segments of outputs, each swept from W positions
// before its first output (heights farther away cannot reach it).
__global__ void __launch_bounds__(128) k_cap_last(const uint16_t *__restrict__ KB, CapGeo G, int T, int W,
                                                  MorphEpi me, const unsigned long long *__restrict__ gate,
                                                  const int *__restrict__ xr, int *__restrict__ orange, int nseg,
                                                  unsigned long long *units)
{
    SeedRange sr{0, G.X0 - 1, 0, G.X0 - 1};
    if (xr)
        sr.load(xr, G.X0, W);
    if (gate && *gate == 0) {
        sr.olo = 2;
        sr.ohi = -1;
    }
    if (orange && blockIdx.x == 0 && threadIdx.x == 0) {
        orange[0] = sr.olo;
        orange[1] = sr.ohi;
    }
    if (xr && sr.olo > sr.ohi)
        return; // nothing within reach of a seed: the caller reads no output
    if (gate && *gate == 0) {
        const long long nl = (long long)me.o1 * me.o2, no = me.o0 * nl;
        for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < no;
             q += (long long)gridDim.x * blockDim.x)
            me.out[q] = 0;
        return;
    }
    // half-width of the interval of every height K <= T: floor(sqrt(T - K))
    __shared__ uint8_t s_w[kCapMaxT + 1];
    for (int q = threadIdx.x; q <= T; q += blockDim.x)
        s_w[q] = (uint8_t)isqrt_small(T - q);
    __syncthreads();
    const long long nlines = (long long)G.nj * G.nk;
    const long long st = (long long)G.X1 * G.X2;
    const int n = G.X0;
    // positions x of the line that lie in the unextended volume (and in the
    // output range of the seeds)
    const int xlo = max(max(0, me.e0), sr.olo), xhi = min(min(n, me.e0 + (int)me.o0), sr.ohi + 1);
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && xhi > xlo)
        atomicAdd(units, (unsigned long long)(nlines * (xhi - xlo)));
    const int seglen = (n + nseg - 1) / nseg;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nlines * nseg;
         g += (long long)gridDim.x * blockDim.x) {
        const int seg = (int)(g / nlines);
        const long long li = g - (long long)seg * nlines;
        // this segment's outputs [ax, bx); heights exist on [sr.hlo, sr.hhi]
        // only, and the sweep starts W steps before the first output
        const int ax = max(xlo, seg * seglen), bx = min(xhi, (seg + 1) * seglen);
        if (ax >= bx)
            continue;
        const int istart = max(0, ax - W), iend = bx - 1 + W;
        const int x1 = G.j0 + (int)(li / G.nk);
        const int x2 = G.k0 + (int)(li - (li / G.nk) * G.nk);
        const uint16_t *in = KB + (long long)x1 * G.X2 + x2;
        const long long jo = x1 - me.e1, ko = x2 - me.e2;
        const bool wall_jk = (me.wall[2] && jo == 0) || (me.wall[3] && jo == me.o1 - 1) ||
                             (me.wall[4] && ko == 0) || (me.wall[5] && ko == me.o2 - 1);
        const long long ost = me.o1 * me.o2;
        uint8_t *dst = me.out + jo * me.o2 + ko + (long long)(ax - me.e0) * ost; // output of x = ax
        // wall planes of axis 0 (unextended coordinates 0 and o0 - 1)
        const int xw0 = me.wall[0] ? me.e0 : -1, xw1 = me.wall[1] ? me.e0 + (int)me.o0 - 1 : -1;
        const uint8_t in_v = me.dilate ? 1 : 0, out_v = me.dilate ? 0 : 1;
        uint64_t pend = 0; // bit b: position i - b is covered
        int reach = -1;
        const int big = T + 1;
        const int hend = min(n, sr.hhi + 1); // heights are read on [hlo, hend)
        int cur[kCapChunk];
        const uint16_t *pin = in + (long long)istart * st;
#pragma unroll
        for (int u = 0; u < kCapChunk; u++) {
            const int i = istart + u;
            cur[u] = i >= sr.hlo && i < hend ? (int)*pin : big;
            pin += st;
        }
        for (int i0 = istart; i0 <= iend; i0 += kCapChunk) {
            int nxt[kCapChunk];
#pragma unroll
            for (int u = 0; u < kCapChunk; u++) {
                const int i = i0 + kCapChunk + u;
                nxt[u] = i >= sr.hlo && i < hend ? (int)*pin : big;
                pin += st;
            }
#pragma unroll
            for (int u = 0; u < kCapChunk; u++) {
                const int i = i0 + u;
                pend <<= 1;
                const int K = cur[u]; // big past the end of the line
                if (K <= T) {
                    const int w = s_w[K];
                    pend |= (2ull << w) - 1ull;
                    reach = max(reach, i + w);
                }
                if (reach >= i && i < n)
                    pend |= 1ull;
                const int x = i - W;
                if (x < ax || x >= bx)
                    continue;
                uint8_t v = ((pend >> W) & 1ull) ? in_v : out_v;
                if (wall_jk || x == xw0 || x == xw1)
                    v = 0;
                *dst = v;
                dst += ost;
            }
#pragma unroll
            for (int u = 0; u < kCapChunk; u++)
                cur[u] = nxt[u];
        }
    }
}

// Pass C for small W on line pairs (pairs over (x1 in [j0, j0 + nj), x2 / 2)
// along axis 0): x is within iff min over |d| <= W of E_B(x + d) + d^2 <= T,
// the same test as the intervals of k_cap_last, then the same epilogue; the
// two outputs of a pair are stored as one 16-bit word (o2 and x2 - e2 even).
template <int W>
__global__ void __launch_bounds__(256) k_cap_last_pair(const uint16_t *__restrict__ KB, CapGeo G, int T, MorphEpi me,
                                                       const unsigned long long *__restrict__ gate,
                                                       const int *__restrict__ xr, int *__restrict__ orange,
                                                       int seglen, unsigned long long *units)
{
    constexpr int R = 2 * W + 1 + pair_ahead(W);
    SeedRange sr{0, G.X0 - 1, 0, G.X0 - 1};
    if (xr)
        sr.load(xr, G.X0, W);
    if (gate && *gate == 0) {
        sr.olo = 2;
        sr.ohi = -1;
    }
    if (orange && blockIdx.x == 0 && threadIdx.x == 0) {
        orange[0] = sr.olo;
        orange[1] = sr.ohi;
    }
    if (xr && sr.olo > sr.ohi)
        return; // nothing within reach of a seed: the caller reads no output
    if (gate && *gate == 0) {
        const long long nl = (long long)me.o1 * me.o2, no = me.o0 * nl;
        for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < no;
             q += (long long)gridDim.x * blockDim.x)
            me.out[q] = 0;
        return;
    }
    const int np = G.nk >> 1;
    const long long nlines = (long long)G.nj * np;
    const long long st = (long long)G.X1 * (G.X2 >> 1);
    const int n = G.X0;
    const int xlo = max(max(0, me.e0), sr.olo), xhi = min(min(n, me.e0 + (int)me.o0), sr.ohi + 1);
    if (xhi <= xlo)
        return;
    if (units && blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(units, (unsigned long long)(nlines * 2 * (xhi - xlo)));
    const int nseg = (xhi - xlo + seglen - 1) / seglen;
    const int hlo = sr.hlo, hend = min(n, sr.hhi + 1); // heights are read on [hlo, hend)
    const uint32_t bigp = (uint32_t)(T + 1) * 0x10001u, tp = (uint32_t)T * 0x10001u;
    const long long ost = me.o1 * me.o2;
    const int xw0 = me.wall[0] ? me.e0 : -1, xw1 = me.wall[1] ? me.e0 + (int)me.o0 - 1 : -1;
    const uint32_t *in0 = (const uint32_t *)KB;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nlines * nseg;
         g += (long long)gridDim.x * blockDim.x) {
        const int seg = (int)(g / nlines);
        const long long li = g - (long long)seg * nlines;
        const int a = xlo + seg * seglen, b = min(xhi, a + seglen);
        const long long q = li / np;
        const int x1 = G.j0 + (int)q;
        const int x2 = G.k0 + 2 * (int)(li - q * np);
        const uint32_t *in = in0 + pair_base<0>(G, li, np);
        const long long jo = x1 - me.e1, ko = x2 - me.e2;
        const bool wall_j = (me.wall[2] && jo == 0) || (me.wall[3] && jo == me.o1 - 1);
        // bytes of the pair kept off the wall lines
        const uint32_t keep = (wall_j || (me.wall[4] && ko == 0) ? 0u : 0x00ffu) |
                              (wall_j || (me.wall[5] && ko + 1 == me.o2 - 1) ? 0u : 0xff00u);
        uint16_t *dst = (uint16_t *)(me.out + jo * me.o2 + ko + (long long)(a - me.e0) * ost);
        const long long ostw = ost >> 1;
        uint32_t win[R];
#pragma unroll
        for (int s = 0; s < R; s++) {
            const int y = a - W + s;
            win[s] = y >= hlo && y < hend ? __ldg(in + y * st) : bigp;
        }
        for (int y0 = a; y0 < b; y0 += R) {
#pragma unroll
            for (int u = 0; u < R; u++) {
                const int y = y0 + u;
                uint32_t m = win[(u + W) % R];
#pragma unroll
                for (int d = 1; d <= W; d++) {
                    const uint32_t dd = (uint32_t)(d * d) * 0x10001u;
                    m = __viaddmin_u16x2(win[(u + W - d) % R], dd, m);
                    m = __viaddmin_u16x2(win[(u + W + d) % R], dd, m);
                }
                if (y < b) {
                    uint32_t sel = __vcmpleu2(m, tp); // 0xffff in each half within reach
                    if (!me.dilate)
                        sel = ~sel;
                    uint32_t v = ((sel & 1u) | ((sel >> 8) & 0x100u)) & keep;
                    if (y == xw0 || y == xw1)
                        v = 0u;
                    *dst = (uint16_t)v;
                    dst += ostw;
                }
                const int yn = y + W + 1 + pair_ahead(W);
                win[u] = y < b && yn >= hlo && yn < hend ? __ldg(in + yn * st) : bigp;
            }
        }
    }
}

// Segment length of the pair kernels: whole groups of the register ring,
// about four per segment.
static int pair_seglen(int W) { return 4 * (2 * W + 1 + pair_ahead(W)); }

// Calls f with std::integral_constant<int, w> for 0 <= w <= kPairMaxW.
template <int W, class F>
static void with_w(int w, F &&f)
{
    if constexpr (W < kPairMaxW) {
        if (w > W) {
            with_w<W + 1>(w, f);
            return;
        }
    }
    f(std::integral_constant<int, W>{});
}

template <int AX, int W>
static void launch_mid_pair_w(const uint16_t *in, uint16_t *out, const CapGeo &G, int T, cudaStream_t st,
                              const unsigned long long *gate, const int *xr, unsigned long long *units)
{
    const int n = AX == 1 ? G.X1 : G.X0;
    const int seglen = pair_seglen(W);
    const long long lines = (long long)(AX == 1 ? G.X0 : G.nj) * (G.nk >> 1);
    const long long work = lines * ((n + seglen - 1) / seglen);
    k_cap_mid_pair<AX, W><<<grid_for(work, 256, 1LL << 30), 256, 0, st>>>(in, out, G, T, gate, xr, seglen, units);
}

template <int AX>
static void launch_mid_pair(const uint16_t *in, uint16_t *out, const CapGeo &G, int T, int W, cudaStream_t st,
                            const unsigned long long *gate, const int *xr, unsigned long long *units)
{
    with_w<0>(W, [&](auto c) { launch_mid_pair_w<AX, decltype(c)::value>(in, out, G, T, st, gate, xr, units); });
}

template <int W>
static void launch_last_pair_w(const uint16_t *KB, const CapGeo &G, int T, const MorphEpi &me, cudaStream_t st,
                               const unsigned long long *gate, const int *xr, int *orange, unsigned long long *units)
{
    const int seglen = pair_seglen(W);
    const long long lines = (long long)G.nj * (G.nk >> 1);
    const long long work = lines * ((G.X0 + seglen - 1) / seglen);
    k_cap_last_pair<W><<<grid_for(work, 256, 1LL << 30), 256, 0, st>>>(KB, G, T, me, gate, xr, orange, seglen, units);
}

static void launch_last_pair(const uint16_t *KB, const CapGeo &G, int T, int W, const MorphEpi &me, cudaStream_t st,
                             const unsigned long long *gate, const int *xr, int *orange, unsigned long long *units)
{
    with_w<0>(W, [&](auto c) { launch_last_pair_w<decltype(c)::value>(KB, G, T, me, st, gate, xr, orange, units); });
}

// Line pairs need even x2 extents and starts (32-bit words of two heights,
// 16-bit output words).
static bool pair_ok(const CapGeo &G, int W) { return W <= kPairMaxW && !((G.X2 | G.k0 | G.nk) & 1); }

// the ring holds the live parabolas, at most 2W + 2
template <int AX>
static int launch_cap_mid(const uint16_t *in, uint16_t *out, const CapGeo &G, int T, int W, long long lines,
                          cudaStream_t st, const unsigned long long *gate = nullptr, const int *xr = nullptr)
{
    // segments of at least 4 W + 32 positions, at most 4 per line
    const int n = AX == 1 ? G.X1 : G.X0;
    int nseg = n / (4 * W + 32);
    nseg = nseg < 1 ? 1 : nseg > 4 ? 4 : nseg;
    const unsigned grid = grid_for(lines * nseg, 128, 1LL << 30);
    // axis-1 passes count their voxels (k_cap_mid); the axis-0 pass of the
    // erosion EDT (k_cap_mid0) is booked from the host
    unsigned long long *units = AX == 1 ? prof_units(kUnitsCapMid) : nullptr;
    if (pair_ok(G, W)) {
        launch_mid_pair<AX>(in, out, G, T, W, st, gate, xr, units);
        return PMG_OK;
    }
    if (2 * W + 2 <= 16)
        k_cap_mid<AX, 16><<<grid, 128, 0, st>>>(in, out, G, T, W, gate, xr, nseg, units);
    else if (2 * W + 2 <= 32)
        k_cap_mid<AX, 32><<<grid, 128, 0, st>>>(in, out, G, T, W, gate, xr, nseg, units);
    else
        k_cap_mid<AX, 64><<<grid, 128, 0, st>>>(in, out, G, T, W, gate, xr, nseg, units);
    return PMG_OK;
}

bool cap_path_ok(const float *res, const int64_t *X, int T)
{
    if (!(res[0] == res[1] && res[1] == res[2]) || T < 0 || T > kCapMaxT)
        return false;
    const pmg_axis_cfg plain = {0, 0, 0, 0, 1, 0, 0, 0};
    for (int d = 0; d < 3; d++)
        if (!exact_path_ok(res[d], plain, (int)X[d]))
            return false;
    return true;
}

int morph_cap_run(const uint8_t *E, uint16_t *KA, uint16_t *KB, const int64_t *X, int T, const MorphEpi &me,
                  cudaStream_t st, int raw_dilate, const unsigned long long *gate, const int *xr, int *orange,
                  const uint8_t *blk)
{
    RowSrc rs{};
    rs.raw = raw_dilate;
    rs.X1 = (int)X[1];
    rs.blk = raw_dilate ? blk : nullptr;
    rs.b1 = (int)((X[1] + 1) / 2);
    rs.b2 = (int)((X[2] + 1) / 2);
    for (int q = 0; q < 6; q++)
        rs.wall[q] = me.wall[q];
    int W = 0;
    while ((W + 1) * (W + 1) <= T)
        W++;
    CapGeo G;
    G.X0 = (int)X[0];
    G.X1 = (int)X[1];
    G.X2 = (int)X[2];
    G.j0 = me.e1;
    G.nj = (int)me.o1;
    G.k0 = me.e2;
    G.nk = (int)me.o2;
    const long long rows = (long long)G.X0 * G.X1;
    {
        const int block = 256;
        const size_t smem = (size_t)(block / 32) * ((G.X2 + 31) / 32 + 2) * sizeof(uint32_t);
        const int ps__ = prof_begin("k_cap_rows", st);
        k_cap_rows<<<grid_for(rows * 32, block, 152LL * 16), block, smem, st>>>(
            E, KA, rows, G.X2, T, W, rs, gate, xr, prof_units(kUnitsCapRows));
        // 1 B read (1/8 B from block masks) + 2 B written per voxel
        prof_end_units(ps__, kUnitsCapRows, rs.blk ? 2.125 : 3.0, st);
    }
    PMG_CHECK_LAUNCH();
    {
        const long long lines = (long long)G.X0 * G.nk;
        const int ps__ = prof_begin("k_cap_mid", st);
        PMG_TRY(launch_cap_mid<1>(KA, KB, G, T, W, lines, st, gate, xr));
        prof_end_units(ps__, kUnitsCapMid, 4.0, st); // 2 B read + 2 B written per voxel
    }
    PMG_CHECK_LAUNCH();
    {
        const long long lines = (long long)G.nj * G.nk;
        const int ps__ = prof_begin("k_cap_last", st);
        // one segment per line: this pass is short per voxel, the extra sweep
        // of a cut costs more than the threads it adds
        const int nseg = 1;
        if (pair_ok(G, W))
            launch_last_pair(KB, G, T, W, me, st, gate, xr, orange, prof_units(kUnitsCapLast));
        else
            k_cap_last<<<grid_for(lines * nseg, 128, 1LL << 30), 128, 0, st>>>(KB, G, T, W, me, gate, xr, orange,
                                                                               nseg, prof_units(kUnitsCapLast));
        prof_end_units(ps__, kUnitsCapLast, 3.0, st); // 2 B read + 1 B written per output
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

// Capped squared EDT of a binary image without extension: E = min(exact d^2
// in units of res^2, T + 1) as uint16, all three passes on the same volume.
int edt_cap_run(const uint8_t *E, uint16_t *KA, uint16_t *KB, uint16_t *KC, const int64_t *X, int T,
                cudaStream_t st)
{
    int W = 0;
    while ((W + 1) * (W + 1) <= T)
        W++;
    CapGeo G;
    G.X0 = (int)X[0];
    G.X1 = (int)X[1];
    G.X2 = (int)X[2];
    G.j0 = 0;
    G.nj = G.X1;
    G.k0 = 0;
    G.nk = G.X2;
    const long long rows = (long long)G.X0 * G.X1;
    const long long vox = rows * G.X2;
    {
        const int block = 256;
        const size_t smem = (size_t)(block / 32) * ((G.X2 + 31) / 32 + 2) * sizeof(uint32_t);
        const int ps__ = prof_begin("k_cap_rows", st);
        k_cap_rows<<<grid_for(rows * 32, block, 152LL * 16), block, smem, st>>>(E, KA, rows, G.X2, T, W,
                                                                                RowSrc{}, nullptr, nullptr,
                                                                                prof_units(kUnitsCapRows));
        prof_end_units(ps__, kUnitsCapRows, 3.0, st);
    }
    PMG_CHECK_LAUNCH();
    {
        const long long lines = (long long)G.X0 * G.nk;
        const int ps__ = prof_begin("k_cap_mid", st);
        PMG_TRY(launch_cap_mid<1>(KA, KB, G, T, W, lines, st));
        prof_end_units(ps__, kUnitsCapMid, 4.0, st);
    }
    PMG_CHECK_LAUNCH();
    {
        const long long lines = (long long)G.nj * G.nk;
        const int ps__ = prof_begin("k_cap_mid0", st);
        PMG_TRY(launch_cap_mid<0>(KB, KC, G, T, W, lines, st));
        prof_end(ps__, (double)vox * 4, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

} // namespace pmg
