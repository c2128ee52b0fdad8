// Connected components on GB300 (sm_103a).
//
// Reference: pmmoto.filters.connected_components (src/pmmoto/filters/
// connected_components.py:32-392) -- labelling by the third-party cc3d
// (26-connectivity, each nonzero value separately, background 0), periodic
// seam merge (connect_subdomain_boundaries :65-101 with core/voxels.py:
// 167-397 and core/_voxels.pyx:335-383, 548-579), inlet/outlet selection
// (:144-392, voxels.py:400-454).
//
// Device algorithm: lock-free union-find over voxel indices where a union
// always links the larger root under the smaller, so a component's final root
// is its smallest voxel index -- its first voxel in C-order raster scan.
// Numbering components by the rank of their root therefore numbers them in
// order of first appearance, the order cc3d issues labels.  Each voxel unites
// with one representative of every 26-connected group of equal-valued
// already-scanned neighbours (13 candidates), which removes most redundant
// unions.  Periodic seams are united voxel-with-twin (the voxel its halo
// copies), which is what the reference's pair matching does.
//
// Every data-dependent loop carries an iteration cap; hitting it sets a
// device status word and the entry point returns PMG_EITER.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <type_traits>
#include <array>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "pmg_common.cuh"
#include "pmg_internal.cuh"
#include "uf.cuh"

namespace pmg {

struct Vol3 {
    long long s0, s1, s2;
};

// The 13 already-scanned neighbours (C order) and their mutual 26-adjacency.
__constant__ int c_nb[13][3];
__constant__ unsigned short c_adj[13];

static void host_tables(int nb[13][3], unsigned short adj[13])
{
    int n = 0;
    for (int di = -1; di <= 0; di++)
        for (int dj = -1; dj <= 1; dj++)
            for (int dk = -1; dk <= 1; dk++) {
                if (di == 0 && (dj > 0 || (dj == 0 && dk >= 0)))
                    continue;
                nb[n][0] = di;
                nb[n][1] = dj;
                nb[n][2] = dk;
                n++;
            }
    for (int a = 0; a < 13; a++) {
        adj[a] = 0;
        for (int b = 0; b < 13; b++) {
            if (a == b)
                continue;
            if (abs(nb[a][0] - nb[b][0]) <= 1 && abs(nb[a][1] - nb[b][1]) <= 1 &&
                abs(nb[a][2] - nb[b][2]) <= 1)
                adj[a] |= (unsigned short)(1u << b);
        }
    }
}

// ---- tiled labelling ------------------------------------------------------
// Tiles of 4 x 8 x 32 voxels (C order, the last axis contiguous), one thread
// per voxel.  Phase 1 unites equal neighbours inside the tile with a shared-
// memory union-find whose roots are the smallest local index -- which is also
// the smallest global index of that part of the component, because C order
// inside a box follows the global C order.  Phase 2 unites neighbours that lie
// in other tiles through the global parents.  Both phases use one
// representative per 26-connected group of equal earlier neighbours.
constexpr int kT0 = 4, kT1 = 8, kT2 = 32, kTile = kT0 * kT1 * kT2;

__device__ __forceinline__ int sfind(const int *L, int x)
{
    int p = L[x];
    int it = 0;
    while (p != x && it++ < kTile) {
        x = p;
        p = L[x];
    }
    return x;
}

// root search with path halving (same argument as find_root_halve)
__device__ __forceinline__ int sfind_halve(int *L, int x)
{
    int p = L[x];
    int it = 0;
    while (p != x && it++ < kTile) {
        const int g = L[p];
        if (g == p)
            return p;
        L[x] = g;
        x = g;
        p = L[x];
    }
    return x;
}

__device__ __forceinline__ void sunite(int *L, int a, int b)
{
    for (int it = 0; it < 4 * kTile; it++) {
        a = sfind_halve(L, a);
        b = sfind_halve(L, b);
        if (a == b)
            return;
        if (a < b) {
            const int old = atomicMin(L + b, a);
            if (old == b)
                return;
            b = old;
        } else {
            const int old = atomicMin(L + a, b);
            if (old == a)
                return;
            a = old;
        }
    }
}

// adj: shared-memory copy of c_adj (lanes index it with different values,
// which constant memory would serialise)
__device__ __forceinline__ unsigned cover_group(unsigned q_mask, unsigned same, const unsigned short *adj)
{
    unsigned grp = q_mask, prev = 0;
    while (grp != prev) {
        prev = grp;
        unsigned g = grp;
        while (g) {
            const int w = __ffs(g) - 1;
            g &= g - 1;
            grp |= adj[w] & same;
        }
    }
    return grp;
}

__device__ __forceinline__ void load_adj(unsigned short *s_adj)
{
    if (threadIdx.x < 13)
        s_adj[threadIdx.x] = c_adj[threadIdx.x];
}

template <typename T>
__global__ void __launch_bounds__(kTile) k_cc_tile(const T *__restrict__ img, int *__restrict__ P, Vol3 V)
{
    __shared__ T sv[kTile];
    __shared__ int L[kTile];
    __shared__ unsigned short s_adj[13];
    load_adj(s_adj);
    const int nt1 = (int)((V.s1 + kT1 - 1) / kT1), nt2 = (int)((V.s2 + kT2 - 1) / kT2);
    const long long tile = blockIdx.x;
    const long long ti = tile / ((long long)nt1 * nt2);
    const int tj = (int)((tile / nt2) % nt1), tk = (int)(tile % nt2);
    const int t = threadIdx.x;
    const int a = t / (kT1 * kT2), b = (t / kT2) % kT1, c = t % kT2;
    const long long i = ti * kT0 + a, j = (long long)tj * kT1 + b, k = (long long)tk * kT2 + c;
    const bool inside = i < V.s0 && j < V.s1 && k < V.s2;
    const long long g = (i * V.s1 + j) * V.s2 + k;
    const T v = inside ? img[g] : (T)0;
    sv[t] = v;
    L[t] = v != 0 ? t : -1;
    __syncthreads();
    if (v != 0) {
        unsigned same = 0;
#pragma unroll
        for (int q = 0; q < 13; q++) {
            const int aa = a + c_nb[q][0], bb = b + c_nb[q][1], cc = c + c_nb[q][2];
            if (aa < 0 || bb < 0 || bb >= kT1 || cc < 0 || cc >= kT2)
                continue;
            if (sv[(aa * kT1 + bb) * kT2 + cc] == v)
                same |= 1u << q;
        }
        unsigned covered = 0;
        while (same & ~covered) {
            const int q = __ffs(same & ~covered) - 1;
            sunite(L, t, ((a + c_nb[q][0]) * kT1 + b + c_nb[q][1]) * kT2 + c + c_nb[q][2]);
            covered |= cover_group(1u << q, same, s_adj);
        }
    }
    __syncthreads();
    if (v != 0)
        L[t] = sfind(L, t);
    __syncthreads();
    if (inside) {
        int out = -1;
        if (v != 0) {
            const int r = L[t];
            const int ra = r / (kT1 * kT2), rb = (r / kT2) % kT1, rc = r % kT2;
            out = (int)(((ti * kT0 + ra) * V.s1 + (long long)tj * kT1 + rb) * V.s2 + (long long)tk * kT2 + rc);
        }
        P[g] = out;
    }
}

// Phase 2: unions with equal earlier neighbours in other tiles.  Neighbours in
// the voxel's own tile (and everything 26-connected to them among the equal
// neighbours) are already united by phase 1.
template <typename T>
__global__ void k_cc_cross(const T *__restrict__ img, int *P, Vol3 V, int *err)
{
    __shared__ unsigned short s_adj[13];
    load_adj(s_adj);
    __syncthreads();
    // volumes are below 2^31 voxels, so 32-bit index arithmetic suffices
    const int n = (int)(V.s0 * V.s1 * V.s2);
    const int S1 = (int)V.s1, S2 = (int)V.s2;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int r = idx / S2;
        const int k = idx - r * S2;
        const int i = r / S1;
        const int j = r - i * S1;
        const int a = i & (kT0 - 1), b = j & (kT1 - 1), c = k & (kT2 - 1);
        if (a > 0 && b > 0 && b < kT1 - 1 && c > 0 && c < kT2 - 1)
            continue; // every earlier neighbour is inside the tile
        const T v = img[idx];
        if (v == 0)
            continue;
        unsigned same = 0, local = 0;
#pragma unroll
        for (int q = 0; q < 13; q++) {
            const int ai = i + c_nb[q][0], bj = j + c_nb[q][1], ck = k + c_nb[q][2];
            if (ai < 0 || bj < 0 || ck < 0 || bj >= S1 || ck >= S2)
                continue;
            if (img[(ai * S1 + bj) * S2 + ck] != v)
                continue;
            same |= 1u << q;
            const int aa = a + c_nb[q][0], bb = b + c_nb[q][1], cc = c + c_nb[q][2];
            if (aa >= 0 && bb >= 0 && bb < kT1 && cc >= 0 && cc < kT2)
                local |= 1u << q;
        }
        unsigned covered = 0;
        unsigned lm = local;
        while (lm) { // groups reached through in-tile neighbours are done
            const int q = __ffs(lm) - 1;
            const unsigned grp = cover_group(1u << q, same, s_adj);
            covered |= grp;
            lm &= ~grp;
        }
        while (same & ~covered) {
            const int q = __ffs(same & ~covered) - 1;
            const int ai = i + c_nb[q][0], bj = j + c_nb[q][1], ck = k + c_nb[q][2];
            unite(P, idx, (ai * S1 + bj) * S2 + ck, err);
            covered |= cover_group(1u << q, same, s_adj);
        }
    }
}

// Seam twins of the voxel labelling (see Twins).
template <typename T>
__global__ void k_cc_twins(const T *__restrict__ img, int *P, Twins W, int *err)
{
    const long long n = W.s0 * W.s1 * W.s2;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        long long c[3];
        c[2] = idx % W.s2;
        long long r = idx / W.s2;
        c[1] = r % W.s1;
        c[0] = r / W.s1;
        bool halo = false;
        long long t[3];
        bool ok = true;
        for (int d = 0; d < 3; d++) {
            t[d] = c[d];
            const long long S = d == 0 ? W.s0 : d == 1 ? W.s1 : W.s2;
            const bool in_halo = c[d] < W.own_lo[d] || c[d] >= W.own_lo[d] + W.own_len[d];
            if (in_halo) {
                if (!W.periodic[d] || W.own_len[d] <= 0 || c[d] < 0 || c[d] >= S) {
                    ok = false;
                } else {
                    long long q = (c[d] - W.own_lo[d]) % W.own_len[d];
                    if (q < 0)
                        q += W.own_len[d];
                    t[d] = q + W.own_lo[d];
                    halo = true;
                }
            }
        }
        if (!halo || !ok || img[idx] == 0)
            continue;
        const long long tw = (t[0] * W.s1 + t[1]) * W.s2 + t[2];
        if (img[tw] != 0)
            unite(P, (int)idx, (int)tw, err);
    }
}

__global__ void k_cc_flatten(int *P, long long n, int *err)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int)n; i += gridDim.x * blockDim.x) {
        const int p = P[i];
        if (p >= 0 && p != i)
            P[i] = find_root(P, p, err);
    }
}

// ---- numbering by root order -------------------------------------------
constexpr int kNumBlock = 512;
constexpr int kNumItems = 4; // voxels per thread in the numbering kernels
constexpr long long kNumTile = (long long)kNumBlock * kNumItems;

__global__ void k_root_count(const int *__restrict__ P, long long n, int *__restrict__ counts)
{
    typedef cub::BlockReduce<int, kNumBlock> BR;
    __shared__ typename BR::TempStorage tmp;
    const long long base = blockIdx.x * kNumTile;
    int c = 0;
#pragma unroll
    for (int q = 0; q < kNumItems; q++) {
        const long long i = base + (long long)threadIdx.x * kNumItems + q;
        if (i < n && P[i] == (int)i)
            c++;
    }
    const int tot = BR(tmp).Sum(c);
    if (threadIdx.x == 0)
        counts[blockIdx.x] = tot;
}

// R[i] = rank of root i among all roots (0-based); P is left unchanged.
__global__ void k_root_rank(const int *__restrict__ P, long long n, const int *__restrict__ offs,
                            int *__restrict__ R)
{
    typedef cub::BlockScan<int, kNumBlock> BS;
    __shared__ typename BS::TempStorage tmp;
    const long long base = blockIdx.x * kNumTile;
    int f[kNumItems];
#pragma unroll
    for (int q = 0; q < kNumItems; q++) {
        const long long i = base + (long long)threadIdx.x * kNumItems + q;
        f[q] = (i < n && P[i] == (int)i) ? 1 : 0;
    }
    int x[kNumItems];
    BS(tmp).ExclusiveSum(f, x);
#pragma unroll
    for (int q = 0; q < kNumItems; q++) {
        const long long i = base + (long long)threadIdx.x * kNumItems + q;
        if (f[q])
            R[i] = offs[blockIdx.x] + x[q];
    }
}

__global__ void k_label_out(const int *__restrict__ P, const int *__restrict__ R, long long n,
                            uint64_t *__restrict__ L)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int p = P[i];
        L[i] = p < 0 ? 0ull : (uint64_t)R[p] + 1ull;
    }
}

// ---- seam pairs for the reference's periodic numbering --------------------

// keys[r] = label(own/neighbour voxel r) << 32 | label(twin), rows in the
// reference's order: own slab then neighbour slab of the feature, each
// flattened in C order, paired with the opposite feature's neighbour then own.
// Labels read from a label volume ...
struct LabImg {
    const uint64_t *L;
    Vol3 V;
    __device__ __forceinline__ uint64_t at(long long i, long long j, long long k) const
    {
        return L[(i * V.s1 + j) * V.s2 + k];
    }
};

// keys[row0 + r] = fkey | label << lbits | twin label (fkey = 0, lbits = 32
// for one feature alone), idx[row0 + r] = row0 + r.
template <class Src>
__global__ void k_seam_pairs(Src src, Box a0, Box a1, Box b0, Box b1, uint64_t fkey, int lbits, long long row0,
                             uint64_t *__restrict__ keys, uint32_t *__restrict__ idx)
{
    keys += row0;
    idx += row0;
    const long long n0 = a0.size(), n = n0 + a1.size();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
         r += (long long)gridDim.x * blockDim.x) {
        const Box &A = r < n0 ? a0 : a1;
        const Box &B = r < n0 ? b0 : b1;
        const long long q = r < n0 ? r : r - n0;
        const long long wa = A.hi[2] - A.lo[2], ha = A.hi[1] - A.lo[1];
        const long long wb = B.hi[2] - B.lo[2], hb = B.hi[1] - B.lo[1];
        const long long ak = q % wa, aj = (q / wa) % ha, ai = q / (wa * ha);
        const long long bk = q % wb, bj = (q / wb) % hb, bi = q / (wb * hb);
        const uint64_t la = src.at(A.lo[0] + ai, A.lo[1] + aj, A.lo[2] + ak);
        const uint64_t lb = src.at(B.lo[0] + bi, B.lo[1] + bj, B.lo[2] + bk);
        keys[r] = fkey | (la << lbits) | lb;
        idx[r] = (uint32_t)(row0 + r);
    }
}

__global__ void k_head_flags(const uint64_t *__restrict__ k, long long n, uint8_t *__restrict__ f)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        f[i] = (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
}

__global__ void k_apply_lut(uint64_t *L, long long n, const uint64_t *__restrict__ lut)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        L[i] = lut[L[i]];
}

__global__ void k_lut_flags(const uint64_t *__restrict__ bl, const uint64_t *__restrict__ bg, long long nbnd,
                            uint8_t *__restrict__ flag, uint64_t *__restrict__ lut)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nbnd;
         i += (long long)gridDim.x * blockDim.x) {
        flag[bl[i]] = 1;
        lut[bl[i]] = bg[i];
    }
}

__global__ void k_lut_nonflag(const uint8_t *__restrict__ flag, long long m, int *__restrict__ nf)
{
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < m;
         l += (long long)gridDim.x * blockDim.x)
        nf[l] = (l > 0 && !flag[l]) ? 1 : 0;
}

__global__ void k_lut_fill(const uint8_t *__restrict__ flag, const int *__restrict__ rank, long long m,
                           uint64_t start, uint64_t *__restrict__ lut)
{
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < m;
         l += (long long)gridDim.x * blockDim.x) {
        if (l == 0)
            lut[0] = 0;
        else if (!flag[l])
            lut[l] = start + (uint64_t)rank[l];
    }
}

// ---- inlet / outlet selection ---------------------------------------------
__global__ void k_mark_face(const int *__restrict__ P, Vol3 V, Box b, uint8_t *__restrict__ mark,
                            uint8_t bit)
{
    const long long n = b.size();
    const long long w = b.hi[2] - b.lo[2], h = b.hi[1] - b.lo[1];
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const long long k = q % w, j = (q / w) % h, i = q / (w * h);
        const long long idx = ((b.lo[0] + i) * V.s1 + b.lo[1] + j) * V.s2 + b.lo[2] + k;
        const int p = P[idx];
        if (p >= 0 && !(mark[p] & bit))
            atomicOr((unsigned int *)(mark + (p & ~3ll)), (unsigned int)bit << (8 * (p & 3)));
    }
}

template <typename TO>
__global__ void k_select(const uint8_t *__restrict__ img, const int *__restrict__ P,
                         const uint8_t *__restrict__ mark, long long n, int mode, int phase,
                         TO *__restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint8_t v = img[i];
        const int p = P[i];
        TO o = 0;
        if (v != 0 && p >= 0 && (phase < 0 || v == phase)) {
            const uint8_t m = mark[p];
            const bool in = m & 1, ou = m & 2;
            bool keep;
            if (mode == PMG_SEL_INLET)
                keep = in;
            else if (mode == PMG_SEL_OUTLET)
                keep = ou;
            else if (mode == PMG_SEL_BOTH)
                keep = in && ou;
            else
                keep = !(in || ou);
            if (keep)
                o = (TO)v;
        }
        out[i] = o;
    }
}

// ---------------------------------------------------------------------------
static bool g_tables_ready[64] = {false};

static int ensure_tables()
{
    int dev = 0;
    PMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_tables_ready[dev])
        return PMG_OK;
    int nb[13][3];
    unsigned short adj[13];
    host_tables(nb, adj);
    PMG_CUDA(cudaMemcpyToSymbol(c_nb, nb, sizeof(nb)));
    PMG_CUDA(cudaMemcpyToSymbol(c_adj, adj, sizeof(adj)));
    if (dev >= 0 && dev < 64)
        g_tables_ready[dev] = true;
    return PMG_OK;
}

// Union-find of a volume into P (roots = smallest index); twins optional.
template <typename T>
static int uf_build(const T *img, int *P, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, bool twins, int *err, cudaStream_t st)
{
    PMG_TRY(ensure_tables());
    const long long n = shape[0] * shape[1] * shape[2];
    Vol3 V{shape[0], shape[1], shape[2]};
    const int block = 256;
    const long long tiles = ((shape[0] + kT0 - 1) / kT0) * ((shape[1] + kT1 - 1) / kT1) *
                            ((shape[2] + kT2 - 1) / kT2);
    {
        const int ps__ = prof_begin("k_cc_tile", st);
        k_cc_tile<T><<<(unsigned)tiles, kTile, 0, st>>>(img, P, V);
        prof_end(ps__, (double)n * (sizeof(T) + 4), st);
    }
    PMG_CHECK_LAUNCH();
    {
        const int ps__ = prof_begin("k_cc_cross", st);
        k_cc_cross<T><<<grid_for(n, block, 152LL * 32), block, 0, st>>>(img, P, V, err);
        prof_end(ps__, 0.0, st);
    }
    PMG_CHECK_LAUNCH();
    if (twins && any_periodic(bc)) {
        {
            const int ps__ = prof_begin("k_cc_twins", st);
            k_cc_twins<T><<<grid_for(n, block, 152LL * 32), block, 0, st>>>(img, P,
                                                                         make_twins(shape, bc, pad), err);
            prof_end(ps__, 0.0, st);
        }
        PMG_CHECK_LAUNCH();
    }
    {
        const int ps__ = prof_begin("k_cc_flatten", st);
        k_cc_flatten<<<grid_for(n, block, 152LL * 32), block, 0, st>>>(P, n, err);
        prof_end(ps__, (double)n * 8, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

static int read_err(int *err, cudaStream_t st)
{
    int h = 0;
    PMG_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    if (h == 3) {
        set_error("connected components: a growing-set selection lost voxels between steps");
        return PMG_EINVAL;
    }
    if (h != 0) {
        set_error("connected components: union-find iteration cap reached (code %d)", h);
        return PMG_EITER;
    }
    return PMG_OK;
}

// Feature slabs (src/pmmoto/core/features.py:76-139) of a single-rank
// padded subdomain; `kind` is the feature's boundary kind (boundary_order).
static void feature_slabs(const int f[3], int kind, const int64_t *shape, const int32_t *pad,
                          Box &own, Box &nb)
{
    bool padded = false;
    for (int d = 0; d < 6; d++)
        padded |= pad[d] != 0;
    for (int d = 0; d < 3; d++) {
        const long long L = shape[d], pb = pad[2 * d], pa = pad[2 * d + 1];
        if (f[d] == -1) {
            if (pb && kind != PMG_BC_WALL) {
                own.lo[d] = pb;
                own.hi[d] = 2 * pb;
            } else if (pb) {
                own.lo[d] = 1;
                own.hi[d] = 2;
            } else {
                own.lo[d] = 0;
                own.hi[d] = 1;
            }
            nb.lo[d] = 0;
            nb.hi[d] = padded ? (kind == PMG_BC_WALL ? 1 : pb) : 0;
        } else if (f[d] == 1) {
            if (pa && kind != PMG_BC_WALL) {
                own.lo[d] = L - 2 * pa;
                own.hi[d] = L - pa;
            } else if (pa) {
                own.lo[d] = L - 2;
                own.hi[d] = L - 1;
            } else {
                own.lo[d] = L - 1;
                own.hi[d] = L;
            }
            nb.lo[d] = padded ? (kind == PMG_BC_WALL ? L - 1 : L - pa) : 0;
            nb.hi[d] = padded ? L : 0;
        } else {
            own.lo[d] = pb;
            own.hi[d] = L - pa;
            nb.lo[d] = padded ? pb : 0;
            nb.hi[d] = padded ? L - pa : 0;
        }
    }
}

// Features in the reference's iteration order (faces, edges, corners;
// core/orientation.py:40-183).
static std::vector<std::array<int, 3>> feature_order()
{
    std::vector<std::array<int, 3>> faces, edges, corners;
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++)
            for (int c = -1; c <= 1; c++) {
                const int s = abs(a) + abs(b) + abs(c);
                if (s == 1)
                    faces.push_back({a, b, c});
                else if (s == 2)
                    edges.push_back({a, b, c});
            }
    for (int a : {-1, 1})
        for (int b : {-1, 1})
            for (int c : {-1, 1})
                corners.push_back({a, b, c});
    std::vector<std::array<int, 3>> all = faces;
    all.insert(all.end(), edges.begin(), edges.end());
    all.insert(all.end(), corners.begin(), corners.end());
    return all;
}

// One periodic feature's seam: its own and neighbour slabs and the opposite
// feature's neighbour and own slabs they pair with, row by row.
struct SeamFeature {
    Box own, nb, oown, onb;
    long long rows;
};

// Every feature's distinct seam keys (label << 32 | twin label) in order of
// first row, one feature at a time: keys in row order, stable radix sort,
// first row of every distinct key.  Two host round trips per feature.
template <class Src>
static int seam_keys_each(const Src &src, const std::vector<SeamFeature> &fs,
                          std::vector<std::vector<uint64_t>> &out, cudaStream_t st)
{
    out.assign(fs.size(), {});
    for (size_t fi = 0; fi < fs.size(); fi++) {
        const SeamFeature &f = fs[fi];
        const long long rows = f.rows;
        uint64_t *d_k = nullptr, *d_k2 = nullptr, *d_k3 = nullptr;
        uint32_t *d_i = nullptr, *d_i2 = nullptr;
        uint8_t *d_f = nullptr;
        int *d_nsel = nullptr;
        PMG_TRY(scratch_alloc((void **)&d_k, rows * 8, st));
        PMG_TRY(scratch_alloc((void **)&d_k2, rows * 8, st));
        PMG_TRY(scratch_alloc((void **)&d_k3, rows * 8, st));
        PMG_TRY(scratch_alloc((void **)&d_i, rows * 4, st));
        PMG_TRY(scratch_alloc((void **)&d_i2, rows * 4, st));
        PMG_TRY(scratch_alloc((void **)&d_f, rows, st));
        PMG_TRY(scratch_alloc((void **)&d_nsel, 2 * sizeof(int), st));
        {
            const int ps__ = prof_begin("k_seam_pairs", st);
            k_seam_pairs<Src><<<grid_for(rows, 256, 1LL << 30), 256, 0, st>>>(src, f.own, f.nb, f.onb, f.oown, 0ull,
                                                                            32, 0, d_k, d_i);
            prof_end(ps__, (double)rows * 28, st);
        }
        PMG_CHECK_LAUNCH();
        size_t tb = 0, tb2 = 0, tb3 = 0;
        PMG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, d_k, d_k2, d_i, d_i2, (int)rows, 0, 64, st));
        PMG_CUDA(cub::DeviceSelect::Flagged(nullptr, tb2, d_i2, d_f, d_i, d_nsel, (int)rows, st));
        PMG_CUDA(cub::DeviceSelect::Flagged(nullptr, tb3, d_k2, d_f, d_k3, d_nsel + 1, (int)rows, st));
        size_t tbs = std::max(tb, std::max(tb2, tb3));
        void *d_t = nullptr;
        PMG_TRY(scratch_alloc(&d_t, tbs, st));
        PMG_CUDA(cub::DeviceRadixSort::SortPairs(d_t, tbs, d_k, d_k2, d_i, d_i2, (int)rows, 0, 64, st));
        {
            const int ps__ = prof_begin("k_head_flags", st);
            k_head_flags<<<grid_for(rows, 256, 1LL << 30), 256, 0, st>>>(d_k2, rows, d_f);
            prof_end(ps__, (double)rows * 9, st);
        }
        PMG_CHECK_LAUNCH();
        PMG_CUDA(cub::DeviceSelect::Flagged(d_t, tbs, d_i2, d_f, d_i, d_nsel, (int)rows, st));
        PMG_CUDA(cub::DeviceSelect::Flagged(d_t, tbs, d_k2, d_f, d_k3, d_nsel + 1, (int)rows, st));
        int nsel = 0;
        PMG_CUDA(cudaMemcpyAsync(&nsel, d_nsel, sizeof(int), cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaStreamSynchronize(st));
        std::vector<uint32_t> first((size_t)nsel);
        std::vector<uint64_t> dkeys((size_t)nsel);
        if (nsel > 0) {
            PMG_CUDA(cudaMemcpyAsync(first.data(), d_i, (size_t)nsel * 4, cudaMemcpyDeviceToHost, st));
            PMG_CUDA(cudaMemcpyAsync(dkeys.data(), d_k3, (size_t)nsel * 8, cudaMemcpyDeviceToHost, st));
        }
        PMG_CUDA(cudaStreamSynchronize(st));
        for (void *q : {(void *)d_t, (void *)d_k, (void *)d_k2, (void *)d_k3, (void *)d_i, (void *)d_i2, (void *)d_f,
                        (void *)d_nsel})
            PMG_TRY(scratch_free(q, st));
        std::vector<size_t> order((size_t)nsel);
        for (size_t q = 0; q < order.size(); q++)
            order[q] = q;
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return first[x] < first[y]; });
        for (size_t q : order)
            out[fi].push_back(dkeys[q]);
    }
    return PMG_OK;
}

// The same for all features at once, when labels fit `lbits` bits with
// 2 lbits + 5 <= 64: keys (feature << 2 lbits | label << lbits | twin label)
// of every feature in one array, one stable radix sort over those bits, the
// first row of every distinct key; two host round trips in all.  Rows of a
// feature are consecutive and in its row order, so the first row of a key is
// its first occurrence in that feature, as above.
template <class Src>
static int seam_keys_batched(const Src &src, const std::vector<SeamFeature> &fs, int lbits,
                             std::vector<std::vector<uint64_t>> &out, cudaStream_t st)
{
    out.assign(fs.size(), {});
    long long T = 0;
    for (auto &f : fs)
        T += f.rows;
    if (T == 0)
        return PMG_OK;
    if (T >= (1LL << 31)) {
        set_error("periodic merge: %lld seam rows", T);
        return PMG_ERANGE;
    }
    uint64_t *d_k = nullptr, *d_k2 = nullptr, *d_k3 = nullptr;
    uint32_t *d_i = nullptr, *d_i2 = nullptr;
    uint8_t *d_f = nullptr;
    int *d_nsel = nullptr;
    PMG_TRY(scratch_alloc((void **)&d_k, T * 8, st));
    PMG_TRY(scratch_alloc((void **)&d_k2, T * 8, st));
    PMG_TRY(scratch_alloc((void **)&d_k3, T * 8, st));
    PMG_TRY(scratch_alloc((void **)&d_i, T * 4, st));
    PMG_TRY(scratch_alloc((void **)&d_i2, T * 4, st));
    PMG_TRY(scratch_alloc((void **)&d_f, T, st));
    PMG_TRY(scratch_alloc((void **)&d_nsel, 2 * sizeof(int), st));
    {
        const int ps__ = prof_begin("k_seam_pairs", st);
        long long row0 = 0;
        for (size_t fi = 0; fi < fs.size(); fi++) {
            const SeamFeature &f = fs[fi];
            k_seam_pairs<Src><<<grid_for(f.rows, 256, 1LL << 30), 256, 0, st>>>(
                src, f.own, f.nb, f.onb, f.oown, (uint64_t)fi << (2 * lbits), lbits, row0, d_k, d_i);
            row0 += f.rows;
        }
        prof_end(ps__, (double)T * 28, st);
    }
    PMG_CHECK_LAUNCH();
    const int nbits = 2 * lbits + 5;
    size_t tb = 0, tb2 = 0, tb3 = 0;
    PMG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, d_k, d_k2, d_i, d_i2, (int)T, 0, nbits, st));
    PMG_CUDA(cub::DeviceSelect::Flagged(nullptr, tb2, d_i2, d_f, d_i, d_nsel, (int)T, st));
    PMG_CUDA(cub::DeviceSelect::Flagged(nullptr, tb3, d_k2, d_f, d_k3, d_nsel + 1, (int)T, st));
    size_t tbs = std::max(tb, std::max(tb2, tb3));
    void *d_t = nullptr;
    PMG_TRY(scratch_alloc(&d_t, tbs, st));
    PMG_CUDA(cub::DeviceRadixSort::SortPairs(d_t, tbs, d_k, d_k2, d_i, d_i2, (int)T, 0, nbits, st));
    {
        const int ps__ = prof_begin("k_head_flags", st);
        k_head_flags<<<grid_for(T, 256, 1LL << 30), 256, 0, st>>>(d_k2, T, d_f);
        prof_end(ps__, (double)T * 9, st);
    }
    PMG_CHECK_LAUNCH();
    PMG_CUDA(cub::DeviceSelect::Flagged(d_t, tbs, d_i2, d_f, d_i, d_nsel, (int)T, st));
    PMG_CUDA(cub::DeviceSelect::Flagged(d_t, tbs, d_k2, d_f, d_k3, d_nsel + 1, (int)T, st));
    int nsel = 0;
    PMG_CUDA(cudaMemcpyAsync(&nsel, d_nsel, sizeof(int), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> first((size_t)nsel);
    std::vector<uint64_t> dkeys((size_t)nsel);
    if (nsel > 0) {
        PMG_CUDA(cudaMemcpyAsync(first.data(), d_i, (size_t)nsel * 4, cudaMemcpyDeviceToHost, st));
        PMG_CUDA(cudaMemcpyAsync(dkeys.data(), d_k3, (size_t)nsel * 8, cudaMemcpyDeviceToHost, st));
    }
    PMG_CUDA(cudaStreamSynchronize(st));
    for (void *q : {(void *)d_t, (void *)d_k, (void *)d_k2, (void *)d_k3, (void *)d_i, (void *)d_i2, (void *)d_f,
                    (void *)d_nsel})
        PMG_TRY(scratch_free(q, st));
    // entries come sorted by feature: split, then first-row order per feature
    const uint64_t mask = (1ull << lbits) - 1ull;
    size_t q0 = 0;
    while (q0 < (size_t)nsel) {
        const size_t fi = (size_t)(dkeys[q0] >> (2 * lbits));
        size_t q1 = q0;
        while (q1 < (size_t)nsel && (size_t)(dkeys[q1] >> (2 * lbits)) == fi)
            q1++;
        if (fi >= fs.size()) {
            set_error("periodic merge: bad seam key");
            return PMG_EINVAL;
        }
        std::vector<size_t> order;
        for (size_t q = q0; q < q1; q++)
            order.push_back(q);
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return first[x] < first[y]; });
        for (size_t q : order)
            out[fi].push_back((((dkeys[q] >> lbits) & mask) << 32) | (dkeys[q] & mask));
        q0 = q1;
    }
    return PMG_OK;
}

// Periodic renumbering of the reference (connect_subdomain_boundaries on one
// rank): boundary pairs of every periodic feature, deduplicated on the device
// in first-occurrence order, replayed through the same hash-set container the
// reference uses so its iteration order is reproduced, then the dict / stack
// merge of merge_matched_voxels and local_to_global_labeling on the host
// (boundary data only), and one relabel pass on the device.
// The labels come from src; with lut_out the relabelling table (indexed by
// the local label) is handed back instead of being applied to L.
template <class Src>
static int periodic_renumber(const Src &src, uint64_t *L, const int64_t *shape, const int32_t *bc,
                             const int32_t *pad, int64_t count, int64_t *out_count, cudaStream_t st,
                             uint64_t **lut_out = nullptr)
{
    const long long n = shape[0] * shape[1] * shape[2];
    auto feats = feature_order();
    std::vector<SeamFeature> fs;
    for (auto &f : feats) {
        int fid[3] = {f[0], f[1], f[2]};
        bool has_nb = true;
        int kind = PMG_BC_PERIODIC;
        for (int d = 0; d < 3; d++) {
            if (fid[d] == 0)
                continue;
            const int b = bc[2 * d + (fid[d] > 0 ? 1 : 0)];
            if (b != PMG_BC_PERIODIC)
                has_nb = false;
            if (b == PMG_BC_END)
                kind = PMG_BC_END;
            else if (b == PMG_BC_WALL && kind != PMG_BC_END)
                kind = PMG_BC_WALL;
        }
        if (!has_nb)
            continue;
        int opp[3] = {-fid[0], -fid[1], -fid[2]};
        SeamFeature sf;
        feature_slabs(fid, kind, shape, pad, sf.own, sf.nb);
        feature_slabs(opp, kind, shape, pad, sf.oown, sf.onb);
        sf.rows = sf.own.size() + sf.nb.size();
        if (sf.rows == 0)
            continue;
        if (sf.own.size() != sf.onb.size() || sf.nb.size() != sf.oown.size()) {
            set_error("periodic merge: mismatched feature slabs");
            return PMG_EINVAL;
        }
        fs.push_back(sf);
    }
    // labels (0 .. count) in lbits bits
    int lbits = 1;
    while (lbits < 40 && ((uint64_t)count >> lbits) != 0)
        lbits++;
    std::vector<std::vector<uint64_t>> seam;
    if (2 * lbits + 5 <= 64 && fs.size() <= 32 && tune_value(kTuneCcSeamBatched))
        PMG_TRY(seam_keys_batched(src, fs, lbits, seam, st));
    else
        PMG_TRY(seam_keys_each(src, fs, seam, st));
    // insertion-ordered map (key label -> neighbour list), as a Python dict
    std::vector<uint64_t> keys_order;
    std::vector<std::vector<uint64_t>> nbrs;
    std::unordered_map<uint64_t, long long> key_pos;
    for (auto &keys : seam) {
        // unique_pairs (_voxels.hpp:106-125): the same container fed the same
        // sequence of first insertions iterates in the same order (repeated
        // keys are no-ops)
        std::unordered_set<unsigned long> uset;
        for (uint64_t k : keys)
            uset.insert((unsigned long)k);
        for (unsigned long e : uset) {
            const uint64_t a = e >> 32, b = e & 0xFFFFFFFFul;
            if (a == 0 || b == 0)
                continue;
            // process_matches_by_feature (_voxels.pyx:548-579)
            auto it = key_pos.find(a);
            if (it == key_pos.end()) {
                key_pos.emplace(a, (long long)keys_order.size());
                keys_order.push_back(a);
                nbrs.push_back({b});
            } else {
                auto &lst = nbrs[(size_t)it->second];
                if (std::find(lst.begin(), lst.end(), b) == lst.end())
                    lst.push_back(b);
            }
        }
    }
    // merge_matched_voxels (_voxels.pyx:335-383): stack walk in key order
    std::vector<uint64_t> bl, bg;
    std::vector<char> visited(keys_order.size(), 0);
    uint64_t global_id = 1;
    for (size_t s = 0; s < keys_order.size(); s++) {
        if (visited[s])
            continue;
        std::vector<uint64_t> stack{keys_order[s]};
        std::vector<uint64_t> conns;
        while (!stack.empty()) {
            const uint64_t cur = stack.back();
            stack.pop_back();
            auto it = key_pos.find(cur);
            if (it == key_pos.end()) {
                set_error("periodic merge: neighbour label without a key");
                return PMG_EINVAL;
            }
            if (visited[(size_t)it->second])
                continue;
            visited[(size_t)it->second] = 1;
            conns.push_back(cur);
            for (uint64_t nbl : nbrs[(size_t)it->second]) {
                auto jt = key_pos.find(nbl);
                if (jt == key_pos.end()) {
                    set_error("periodic merge: neighbour label without a key");
                    return PMG_EINVAL;
                }
                if (!visited[(size_t)jt->second])
                    stack.push_back(nbl);
            }
        }
        for (uint64_t c : conns) {
            if (c > (uint64_t)count) {
                set_error("periodic merge: label out of range");
                return PMG_EINVAL;
            }
            bl.push_back(c);
            bg.push_back(global_id);
        }
        global_id += conns.empty() ? 0 : 1;
    }
    // local_to_global_labeling (core/voxels.py:344-397) on the device:
    // boundary labels take their merged id, the others global_id, +1, ...
    // in increasing label order
    const long long m = count + 1;
    const long long nbnd = (long long)bl.size();
    uint64_t *d_lut = nullptr, *d_bl = nullptr, *d_bg = nullptr;
    uint8_t *d_flag = nullptr;
    int *d_nf = nullptr, *d_rank = nullptr;
    PMG_TRY(scratch_alloc((void **)&d_lut, (size_t)m * 8, st));
    PMG_TRY(scratch_alloc((void **)&d_flag, (size_t)m, st));
    PMG_TRY(scratch_alloc((void **)&d_nf, (size_t)m * 4, st));
    PMG_TRY(scratch_alloc((void **)&d_rank, (size_t)m * 4, st));
    PMG_TRY(scratch_alloc((void **)&d_bl, (size_t)(nbnd + 1) * 8, st));
    PMG_TRY(scratch_alloc((void **)&d_bg, (size_t)(nbnd + 1) * 8, st));
    PMG_CUDA(cudaMemsetAsync(d_flag, 0, (size_t)m, st));
    if (nbnd > 0) {
        PMG_CUDA(cudaMemcpyAsync(d_bl, bl.data(), (size_t)nbnd * 8, cudaMemcpyHostToDevice, st));
        PMG_CUDA(cudaMemcpyAsync(d_bg, bg.data(), (size_t)nbnd * 8, cudaMemcpyHostToDevice, st));
        {
            const int ps__ = prof_begin("k_lut_flags", st);
            k_lut_flags<<<grid_for(nbnd, 256, 1LL << 30), 256, 0, st>>>(d_bl, d_bg, nbnd, d_flag, d_lut);
            prof_end(ps__, (double)nbnd * 25, st);
        }
        PMG_CHECK_LAUNCH();
    }
    {
        const int ps__ = prof_begin("k_lut_nonflag", st);
        k_lut_nonflag<<<grid_for(m, 256, 1LL << 30), 256, 0, st>>>(d_flag, m, d_nf);
        prof_end(ps__, (double)m * 5, st);
    }
    PMG_CHECK_LAUNCH();
    size_t tb = 0;
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, d_nf, d_rank, (int)m, st));
    void *d_t = nullptr;
    PMG_TRY(scratch_alloc(&d_t, tb, st));
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(d_t, tb, d_nf, d_rank, (int)m, st));
    {
        const int ps__ = prof_begin("k_lut_fill", st);
        k_lut_fill<<<grid_for(m, 256, 1LL << 30), 256, 0, st>>>(d_flag, d_rank, m, global_id, d_lut);
        prof_end(ps__, (double)m * 13, st);
    }
    PMG_CHECK_LAUNCH();
    if (!lut_out) {
        const int ps__ = prof_begin("k_apply_lut", st);
        k_apply_lut<<<grid_for(n, 256, 1LL << 30), 256, 0, st>>>(L, n, d_lut);
        prof_end(ps__, (double)n * 16, st);
        PMG_CHECK_LAUNCH();
    }
    const long long nloc = (long long)count - nbnd;
    int64_t max_label = (int64_t)(nloc + (long long)global_id);
    if (max_label < 1)
        max_label = (int64_t)global_id;
    PMG_TRY(scratch_free(d_t, st));
    if (lut_out)
        *lut_out = d_lut;
    else
        PMG_TRY(scratch_free(d_lut, st));
    PMG_TRY(scratch_free(d_flag, st));
    PMG_TRY(scratch_free(d_nf, st));
    PMG_TRY(scratch_free(d_rank, st));
    PMG_TRY(scratch_free(d_bl, st));
    PMG_TRY(scratch_free(d_bg, st));
    *out_count = max_label;
    return PMG_OK;
}

template <typename T>
static int cc_label_t(const T *img, uint64_t *labels, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, int64_t *count, cudaStream_t st)
{
    const long long n = shape[0] * shape[1] * shape[2];
    int *P = nullptr, *R = nullptr, *err = nullptr, *cnt = nullptr, *offs = nullptr;
    const long long nb = (n + kNumTile - 1) / kNumTile;
    PMG_TRY(scratch_alloc((void **)&P, (size_t)n * 4, st));
    PMG_TRY(scratch_alloc((void **)&R, (size_t)n * 4, st));
    PMG_TRY(scratch_alloc((void **)&err, sizeof(int), st));
    PMG_TRY(scratch_alloc((void **)&cnt, (size_t)nb * 4 + 4, st));
    PMG_TRY(scratch_alloc((void **)&offs, (size_t)nb * 4 + 4, st));
    PMG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    PMG_TRY(uf_build<T>(img, P, shape, bc, pad, false, err, st));
    {
        const int ps__ = prof_begin("k_root_count", st);
        k_root_count<<<(unsigned)nb, kNumBlock, 0, st>>>(P, n, cnt);
        prof_end(ps__, (double)n * 4, st);
    }
    PMG_CHECK_LAUNCH();
    size_t tb = 0;
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, offs, (int)nb + 1, st));
    void *tmp = nullptr;
    PMG_TRY(scratch_alloc(&tmp, tb, st));
    PMG_CUDA(cudaMemsetAsync(cnt + nb, 0, 4, st));
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, offs, (int)nb + 1, st));
    {
        const int ps__ = prof_begin("k_root_rank", st);
        k_root_rank<<<(unsigned)nb, kNumBlock, 0, st>>>(P, n, offs, R);
        prof_end(ps__, (double)n * 4, st);
    }
    PMG_CHECK_LAUNCH();
    {
        const int ps__ = prof_begin("k_label_out", st);
        k_label_out<<<grid_for(n, 256, 1LL << 30), 256, 0, st>>>(P, R, n, labels);
        prof_end(ps__, (double)n * 12, st);
    }
    PMG_CHECK_LAUNCH();
    int total = 0;
    PMG_CUDA(cudaMemcpyAsync(&total, offs + nb, sizeof(int), cudaMemcpyDeviceToHost, st));
    int s = read_err(err, st);
    PMG_TRY(scratch_free(tmp, st));
    PMG_TRY(scratch_free(P, st));
    PMG_TRY(scratch_free(R, st));
    PMG_TRY(scratch_free(err, st));
    PMG_TRY(scratch_free(cnt, st));
    PMG_TRY(scratch_free(offs, st));
    if (s != PMG_OK)
        return s;
    *count = total;
    if (any_periodic(bc))
        return periodic_renumber(LabImg{labels, Vol3{shape[0], shape[1], shape[2]}}, labels, shape, bc, pad, total,
                                 count, st);
    return PMG_OK;
}

static int check_vol(const int64_t *shape)
{
    for (int d = 0; d < 3; d++)
        if (shape[d] <= 0) {
            set_error("shape[%d] must be positive", d);
            return PMG_EINVAL;
        }
    const long long n = shape[0] * shape[1] * shape[2];
    if (n >= (1LL << 31) - 1) {
        set_error("volume of %lld voxels exceeds the 2^31-1 voxel limit of the int32 union-find", n);
        return PMG_ERANGE;
    }
    return PMG_OK;
}

int cc_label_u8(const uint8_t *img, uint64_t *labels, const int64_t *shape, const int32_t *bc, const int32_t *pad,
                int64_t *count, cudaStream_t st);

} // namespace pmg

using namespace pmg;

extern "C" int pmg_cc_label(const void *img, int32_t elem_bytes, uint64_t *labels,
                            const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                            int64_t *count, void *stream)
{
    if (!img || !labels || !shape || !bc || !pad || !count) {
        set_error("pmg_cc_label: null argument");
        return PMG_EINVAL;
    }
    PMG_TRY(check_geometry(shape, bc, pad));
    PMG_TRY(check_vol(shape));
    cudaStream_t st = as_stream(stream);
    switch (elem_bytes) {
    case 1:
        return cc_label_u8((const uint8_t *)img, labels, shape, bc, pad, count, st);
    case 2:
        return cc_label_t((const uint16_t *)img, labels, shape, bc, pad, count, st);
    case 4:
        return cc_label_t((const uint32_t *)img, labels, shape, bc, pad, count, st);
    case 8:
        return cc_label_t((const uint64_t *)img, labels, shape, bc, pad, count, st);
    default:
        set_error("pmg_cc_label: element size %d not supported", elem_bytes);
        return PMG_EINVAL;
    }
}

namespace pmg {

// ---- binary selection on 2x2x2 blocks -----------------------------------------
// When the foreground is a single value (a phase filter, or an image known to
// hold only 0 and 1), all foreground voxels of a 2x2x2 block are mutually
// 26-adjacent and hence in one component, so the union-find runs on blocks:
// eight times fewer elements (the parents of a 512^3 volume fit in L2).  Two
// neighbouring blocks are connected exactly when each has a foreground voxel in
// the part of the block that touches the other (a face, an edge or a corner):
// every voxel of one touching part is 26-adjacent to every voxel of the other.
// floor(n / d) of a 32-bit n by one multiplication (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994: the
// round-up multiplier m = floor(2^32 (2^l - d) / d) + 1, l = ceil(log2 d),
// with the add-and-halve fix-up), exact for every n and d >= 1
struct FastDiv {
    unsigned m;
    int s1, s2;
};

static inline FastDiv fastdiv_of(unsigned d)
{
    int l = 0;
    while (l < 32 && (1ull << l) < d)
        l++;
    FastDiv f;
    f.m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1ull);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}

__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv &f)
{
    const unsigned t = __umulhi(f.m, n);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

struct BGrid {
    int s0, s1, s2;    // voxel shape
    int b0, b1, b2;    // block shape
    FastDiv q2, q1;    // division by b2 and by b1
    // block index -> (c0, c1, c2)
    __device__ __forceinline__ void coords(int b, int &c0, int &c1, int &c2) const
    {
        const int r = (int)fdiv((unsigned)b, q2);
        c2 = b - r * b2;
        c0 = (int)fdiv((unsigned)r, q1);
        c1 = r - c0 * b1;
    }
};

__device__ __forceinline__ bool fg_of(uint8_t v, int fgval) { return fgval >= 0 ? v == fgval : v != 0; }

// touching voxels of a block for neighbour offset (d0, d1, d2): bit (x*2+y)*2+z
__host__ __device__ inline unsigned touch_mask(int d0, int d1, int d2)
{
    unsigned m = 0;
    for (int x = 0; x < 2; x++)
        for (int y = 0; y < 2; y++)
            for (int z = 0; z < 2; z++) {
                if ((d0 == -1 && x != 0) || (d0 == 1 && x != 1))
                    continue;
                if ((d1 == -1 && y != 0) || (d1 == 1 && y != 1))
                    continue;
                if ((d2 == -1 && z != 0) || (d2 == 1 && z != 1))
                    continue;
                m |= 1u << ((x * 2 + y) * 2 + z);
            }
    return m;
}

// Touch masks of the 13 earlier neighbours: voxels of a block that touch
// neighbour q, voxels of neighbour q that touch the block, and voxels of
// neighbour r that touch neighbour q (0 when r and q are not adjacent).
__constant__ uint8_t c_bt_self[13];
__constant__ uint8_t c_bt_nb[13];
__constant__ uint8_t c_bt_pair[13][13];
// all 26 neighbours: offsets, voxels of a block touching neighbour q, voxels of
// neighbour q touching the block
__constant__ signed char c_g_d[26][3];
__constant__ uint8_t c_g_self[26];
__constant__ uint8_t c_g_nb[26];

__device__ __forceinline__ unsigned bmask_of(int q, uint64_t mlo, uint64_t mhi)
{
    return (unsigned)((q < 8 ? mlo >> (8 * q) : mhi >> (8 * (q - 8))) & 0xffu);
}

struct BTabs {
    unsigned short adj[13];
    uint8_t pair[13][13];
};

__device__ __forceinline__ void load_btabs(BTabs &tb)
{
    if (threadIdx.x < 13)
        tb.adj[threadIdx.x] = c_adj[threadIdx.x];
    for (int q = threadIdx.x; q < 169; q += blockDim.x)
        tb.pair[q / 13][q % 13] = c_bt_pair[q / 13][q % 13];
}

// Neighbours in `conn` that touch neighbour w (one step), w included: a union
// with w links them too, because the union of each touching pair is done by
// the later block of the pair.
__device__ __forceinline__ unsigned bcover1(int w, unsigned conn, uint64_t mlo, uint64_t mhi, const BTabs &tb)
{
    unsigned grp = 1u << w;
    const unsigned mw = bmask_of(w, mlo, mhi);
    unsigned cand = tb.adj[w] & conn;
    while (cand) {
        const int u = __ffs(cand) - 1;
        cand &= cand - 1;
        if ((mw & tb.pair[w][u]) && (bmask_of(u, mlo, mhi) & tb.pair[u][w]))
            grp |= 1u << u;
    }
    return grp;
}

// Everything in `conn` connected to neighbour w through chains of touching
// neighbours (the closure of bcover1): worth its cost where a union is a
// global-memory atomic.
__device__ __forceinline__ unsigned bcover(int w, unsigned conn, uint64_t mlo, uint64_t mhi, const BTabs &tb)
{
    unsigned grp = 1u << w, frontier = 1u << w;
    while (frontier) {
        const int v = __ffs(frontier) - 1;
        frontier &= frontier - 1;
        const unsigned add = bcover1(v, conn & ~grp, mlo, mhi, tb) & ~grp;
        grp |= add;
        frontier |= add;
    }
    return grp;
}

// Neighbour (-1, 0, 0) (index 4 in c_nb order) is 26-adjacent to all twelve
// other earlier neighbours, so it is taken first: in a dense region one union
// with it covers every other one.
constexpr int kCentre = 4;

__device__ __forceinline__ int next_cover(unsigned rest)
{
    return ((rest >> kCentre) & 1u) ? kCentre : __ffs(rest) - 1;
}

// Foreground of the block selection: the voxels of one value (or nonzero)
// of a uint8 image ...
struct SrcImg {
    const uint8_t *img;
    int fgval;
    __device__ __forceinline__ bool fg(long long idx, int, int, int) const { return fg_of(img[idx], fgval); }
    // voxels idx and idx + 1 (idx even) with one 16-bit load: bit 0, bit 1
    __device__ __forceinline__ unsigned fg2(long long idx, int, int, int) const
    {
        const unsigned v = *(const uint16_t *)(img + idx);
        return (unsigned)fg_of((uint8_t)v, fgval) | ((unsigned)fg_of((uint8_t)(v >> 8), fgval) << 1);
    }
};

// ... or an erosion read off a capped squared EDT: voxels with E > T stay,
// wall planes are cleared (subtraction + set_wall_bcs,
// morphological_operators.py:171-228).
struct SrcErode {
    const uint16_t *E;
    int T;
    int s0, s1, s2;
    unsigned walls; // bit q: face q (axis q / 2, low / high) is a wall
    __device__ __forceinline__ bool fg(long long idx, int i, int j, int k) const
    {
        const unsigned on = (i == 0) | ((i == s0 - 1) << 1) | ((j == 0) << 2) | ((j == s1 - 1) << 3) |
                            ((k == 0) << 4) | ((k == s2 - 1) << 5);
        return !(on & walls) && (int)E[idx] > T;
    }
    // voxels idx and idx + 1 (idx even, k + 1 < s2) with one 32-bit load
    __device__ __forceinline__ unsigned fg2(long long idx, int i, int j, int k) const
    {
        const unsigned v = *(const uint32_t *)(E + idx);
        const unsigned row = (i == 0) | ((i == s0 - 1) << 1) | ((j == 0) << 2) | ((j == s1 - 1) << 3);
        const unsigned on0 = row | ((k == 0) << 4) | ((k == s2 - 1) << 5);
        const unsigned on1 = row | ((k + 1 == s2 - 1) << 5);
        return (unsigned)(!(on0 & walls) && (int)(v & 0xffffu) > T) |
               ((unsigned)(!(on1 & walls) && (int)(v >> 16) > T) << 1);
    }
};

// ... or the voxels whose step (the first step at which they belong to a
// growing set, 255 for never) is at most k.
struct SrcStep {
    const uint8_t *S;
    int k;
    __device__ __forceinline__ bool fg(long long idx, int, int, int) const { return (int)S[idx] <= k; }
    __device__ __forceinline__ unsigned fg2(long long idx, int, int, int) const
    {
        const unsigned v = *(const uint16_t *)(S + idx);
        return (unsigned)((int)(v & 0xffu) <= k) | ((unsigned)((int)(v >> 8) <= k) << 1);
    }
};

// ... or the block masks themselves, kept current by the producer of the set
// (the drainage update keeps the wetting phase's).
struct SrcMask {
    const uint8_t *M;
};

// Mask of block (c0, c1, c2): bit (x * 2 + y) * 2 + z for a foreground voxel
// (2 c0 + x, 2 c1 + y, 2 c2 + z) inside the volume.
template <class Src>
__device__ __forceinline__ unsigned block_mask(const Src &src, const BGrid &G, int c0, int c1, int c2)
{
    unsigned m = 0;
    const long long sy = G.s2, sx = (long long)G.s1 * G.s2;
    const long long base = (2LL * c0 * G.s1 + 2 * c1) * sy + 2 * c2;
    const bool whole = 2 * c0 + 1 < G.s0 && 2 * c1 + 1 < G.s1 && 2 * c2 + 1 < G.s2;
    if (whole && !(G.s2 & 1)) {
        // even rows: every voxel pair (z = 0, 1) starts on an even index
#pragma unroll
        for (int x = 0; x < 2; x++)
#pragma unroll
            for (int y = 0; y < 2; y++)
                m |= src.fg2(base + x * sx + y * sy, 2 * c0 + x, 2 * c1 + y, 2 * c2) << ((x * 2 + y) * 2);
    } else {
#pragma unroll
        for (int x = 0; x < 2; x++)
#pragma unroll
            for (int y = 0; y < 2; y++)
#pragma unroll
                for (int z = 0; z < 2; z++) {
                    const int i = 2 * c0 + x, j = 2 * c1 + y, k = 2 * c2 + z;
                    if ((whole || (i < G.s0 && j < G.s1 && k < G.s2)) &&
                        src.fg(base + x * sx + y * sy + z, i, j, k))
                        m |= 1u << ((x * 2 + y) * 2 + z);
                }
    }
    return m;
}

__device__ __forceinline__ unsigned block_mask(const SrcMask &src, const BGrid &G, int c0, int c1, int c2)
{
    return src.M[((long long)c0 * G.b1 + c1) * G.b2 + c2];
}

// The 13 earlier neighbours in the order of c_nb, as arithmetic of the index
// (constants once a loop over q is unrolled): (-1, q / 3 - 1, q % 3 - 1) for
// q < 9, (0, -1, q - 10) for q < 12, (0, 0, -1) for q = 12.
__device__ __forceinline__ int nb_d0(int q) { return q < 9 ? -1 : 0; }
__device__ __forceinline__ int nb_d1(int q) { return q < 9 ? q / 3 - 1 : (q < 12 ? -1 : 0); }
__device__ __forceinline__ int nb_d2(int q) { return q < 9 ? q % 3 - 1 : (q < 12 ? q - 10 : -1); }

// Voxels of a block that touch its neighbour at offset (d0, d1, d2): bit
// (x * 2 + y) * 2 + z, x on the d0 side and so on.
__device__ __forceinline__ unsigned touch_bits(int d0, int d1, int d2)
{
    const unsigned X = d0 < 0 ? 0x0Fu : d0 > 0 ? 0xF0u : 0xFFu;
    const unsigned Y = d1 < 0 ? 0x33u : d1 > 0 ? 0xCCu : 0xFFu;
    const unsigned Z = d2 < 0 ? 0x55u : d2 > 0 ? 0xAAu : 0xFFu;
    return X & Y & Z;
}

// Phase 1 on tiles of 4 x 8 x 32 blocks (8 x 16 x 64 voxels), one thread per
// block: block masks from the source, then a shared-memory union-find of the
// tile whose roots are the smallest block index of each tile-local part.
// Every later step reads the block masks M, never the source again.
//
// With Pl, the tile-local parents are also kept in Pl; with dirty (per tile),
// a tile whose flag is clear has not changed since Pl was written and only
// copies Pl to P, and every recomputed tile clears its flag.
template <class Src>
__global__ void __launch_bounds__(kTile, 2) k_bcc_tile(Src src, int *__restrict__ P, uint8_t *__restrict__ M,
                                                   BGrid G, int *__restrict__ Pl, int *__restrict__ dirty)
{
    __shared__ uint8_t sm[kTile];
    __shared__ int L[kTile];
    __shared__ BTabs tb;
    const int nt1 = (G.b1 + kT1 - 1) / kT1, nt2 = (G.b2 + kT2 - 1) / kT2;
    const int tile = blockIdx.x;
    const int ti = tile / (nt1 * nt2), tj = (tile / nt2) % nt1, tk = tile % nt2;
    const int t = threadIdx.x;
    const int a = t / (kT1 * kT2), b = (t / kT2) % kT1, c = t % kT2;
    const int c0 = ti * kT0 + a, c1 = tj * kT1 + b, c2 = tk * kT2 + c;
    const bool inside = c0 < G.b0 && c1 < G.b1 && c2 < G.b2;
    if (dirty && !dirty[tile]) {
        if (inside) {
            const int bidx = (c0 * G.b1 + c1) * G.b2 + c2;
            P[bidx] = Pl[bidx];
        }
        return;
    }
    load_btabs(tb);
    const unsigned m = inside ? block_mask(src, G, c0, c1, c2) : 0u;
    sm[t] = (uint8_t)m;
    L[t] = m ? t : -1;
    __syncthreads();
    if (m) {
        unsigned conn = 0;
        uint64_t mlo = 0, mhi = 0;
        bool full = m == 0xffu; // this block and every connected neighbour full
#pragma unroll
        for (int q = 0; q < 13; q++) {
            const int aa = a + nb_d0(q), bb = b + nb_d1(q), cc = c + nb_d2(q);
            if (aa < 0 || bb < 0 || bb >= kT1 || cc < 0 || cc >= kT2)
                continue;
            if (!(m & touch_bits(nb_d0(q), nb_d1(q), nb_d2(q))))
                continue;
            const unsigned mn = sm[(aa * kT1 + bb) * kT2 + cc];
            if (mn & touch_bits(-nb_d0(q), -nb_d1(q), -nb_d2(q))) {
                conn |= 1u << q;
                full = full && mn == 0xffu;
                if (q < 8)
                    mlo |= (uint64_t)mn << (8 * q);
                else
                    mhi |= (uint64_t)mn << (8 * (q - 8));
            }
        }
        // dense fast path: full blocks touch whenever they are 26-adjacent, and
        // the centre neighbour is adjacent to every other one
        unsigned covered = (full && ((conn >> kCentre) & 1u)) ? conn & ~(1u << kCentre) : 0u;
        while (conn & ~covered) {
            const unsigned rest = conn & ~covered;
            const int q = next_cover(rest);
            sunite(L, t, ((a + nb_d0(q)) * kT1 + b + nb_d1(q)) * kT2 + c + nb_d2(q));
            covered |= bcover1(q, rest, mlo, mhi, tb);
        }
    }
    __syncthreads();
    if (m)
        L[t] = sfind(L, t);
    __syncthreads();
    if (inside) {
        const int bidx = (c0 * G.b1 + c1) * G.b2 + c2;
        if constexpr (!std::is_same<Src, SrcMask>::value)
            M[bidx] = (uint8_t)m;
        int out = -1;
        if (m) {
            const int r = L[t];
            const int ra = r / (kT1 * kT2), rb = (r / kT2) % kT1, rc = r % kT2;
            out = ((ti * kT0 + ra) * G.b1 + tj * kT1 + rb) * G.b2 + tk * kT2 + rc;
        }
        P[bidx] = out;
        if (Pl)
            Pl[bidx] = out;
    }
    if (dirty && t == 0)
        dirty[tile] = 0;
}

// Phase 2: blocks on a tile border unite with touching earlier neighbours in
// other tiles; neighbours reached through an in-tile neighbour are skipped.
// Border blocks of a tile (the only ones with earlier neighbours in other
// tiles), numbered densely so that every lane of a warp has one: the a = 0
// plane (kT1 x kT2), then the b = 0 and b = kT1 - 1 rows of the other planes,
// then the c = 0 and c = kT2 - 1 ends of the remaining rows.
constexpr int kBorderPlane = kT1 * kT2;
constexpr int kBorderRows = (kT0 - 1) * 2 * kT2;
constexpr int kBorderEnds = (kT0 - 1) * (kT1 - 2) * 2;
constexpr int kBorder = kBorderPlane + kBorderRows + kBorderEnds;
static_assert(kBorder <= 512, "a tile's border items fit one 512-thread block");

__device__ __forceinline__ void border_block(int q, int &a, int &b, int &c)
{
    if (q < kBorderPlane) {
        a = 0;
        b = q / kT2;
        c = q % kT2;
    } else if (q < kBorderPlane + kBorderRows) {
        const int r = q - kBorderPlane;
        a = 1 + r / (2 * kT2);
        b = ((r / kT2) & 1) ? kT1 - 1 : 0;
        c = r % kT2;
    } else {
        const int r = q - kBorderPlane - kBorderRows;
        a = 1 + r / (2 * (kT1 - 2));
        b = 1 + (r % (2 * (kT1 - 2))) / 2;
        c = (r & 1) ? kT2 - 1 : 0;
    }
}

// Touching earlier neighbours of border block (c0, c1, c2) at tile offset
// (a, b, c): conn, those inside the tile (local), the dense flag and their
// masks (mlo: neighbours 0-7, mhi: 8-12).
// Touching earlier neighbours of border block bi = (c0, c1, c2) at tile
// offset (a, b, c): conn, those inside the tile (local), the dense flag and
// their masks (MASKS: mlo for neighbours 0-7, mhi for 8-12).  INTERIOR: all
// 13 neighbours lie inside the volume (no bounds checks).  LAZY: in-tile
// neighbours are read only when the block is full (their only use in the
// cross-tile test is the dense rule).
template <bool INTERIOR, bool LAZY, bool MASKS>
__device__ __forceinline__ void border_conn(const uint8_t *__restrict__ M, const BGrid &G, int bi, int c0, int c1,
                                            int c2, int a, int b, int c, unsigned m, unsigned &conn,
                                            unsigned &local, bool &full, uint64_t &mlo, uint64_t &mhi)
{
    conn = 0;
    local = 0;
    mlo = 0;
    mhi = 0;
    full = m == 0xffu;
    const int plane = G.b1 * G.b2;
#pragma unroll
    for (int q = 0; q < 13; q++) {
        const int d0 = nb_d0(q), d1 = nb_d1(q), d2 = nb_d2(q);
        if (!INTERIOR) {
            const int a0 = c0 + d0, a1 = c1 + d1, a2 = c2 + d2;
            if (a0 < 0 || a1 < 0 || a2 < 0 || a1 >= G.b1 || a2 >= G.b2)
                continue;
        }
        if (!(m & touch_bits(d0, d1, d2)))
            continue;
        const bool in_tile = a + d0 >= 0 && b + d1 >= 0 && b + d1 < kT1 && c + d2 >= 0 && c + d2 < kT2;
        if (LAZY && in_tile && m != 0xffu)
            continue;
        const unsigned mn = M[bi + d0 * plane + d1 * G.b2 + d2];
        if (!(mn & touch_bits(-d0, -d1, -d2)))
            continue;
        conn |= 1u << q;
        full = full && mn == 0xffu;
        if (MASKS) {
            if (q < 8)
                mlo |= (uint64_t)mn << (8 * q);
            else
                mhi |= (uint64_t)mn << (8 * (q - 8));
        }
        if (in_tile)
            local |= 1u << q;
    }
}

// All 13 earlier neighbours of block (c0, c1, c2) inside the volume.
__device__ __forceinline__ bool nb_interior(const BGrid &G, int c0, int c1, int c2)
{
    return c0 >= 1 && c1 >= 1 && c1 + 1 < G.b1 && c2 >= 1 && c2 + 1 < G.b2;
}

// Phase 2a: border blocks whose cross-tile links need no union (empty, no
// touching neighbour outside the tile, or dense with an in-tile neighbour
// that links them all) stop here; the others are listed for phase 2b (as
// block indices), so that its warps run full.  One thread block per tile,
// border item t on thread t.  The in-tile neighbours matter only for the
// dense rule, so only full blocks read their masks.
__global__ void __launch_bounds__(512) k_bcc_cross(const uint8_t *__restrict__ M, BGrid G, int *hard, int *nhard)
{
    const int nt1 = (G.b1 + kT1 - 1) / kT1, nt2 = (G.b2 + kT2 - 1) / kT2;
    const int tile = blockIdx.x;
    const int ti = tile / (nt1 * nt2), tj = (tile / nt2) % nt1, tk = tile % nt2;
    const int t = threadIdx.x;
    bool need = false;
    int bi = -1;
    if (t < kBorder) {
        int a, b, c;
        border_block(t, a, b, c);
        const int c0 = ti * kT0 + a, c1 = tj * kT1 + b, c2 = tk * kT2 + c;
        const unsigned m = c0 < G.b0 && c1 < G.b1 && c2 < G.b2 ? M[(c0 * G.b1 + c1) * G.b2 + c2] : 0u;
        bi = (c0 * G.b1 + c1) * G.b2 + c2;
        if (m) {
            unsigned conn, local;
            bool full;
            uint64_t mlo, mhi;
            if (nb_interior(G, c0, c1, c2))
                border_conn<true, true, false>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            else
                border_conn<false, true, false>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            // in-tile neighbours were united in phase 1, and so was
            // everything touching them
            need = (conn & ~local) != 0 && !(full && ((conn >> kCentre) & 1u) && local);
        }
    }
    if (t >= (kBorder + 31) / 32 * 32)
        return; // warps without border items
    const int lane = t & 31;
    const unsigned bal = __ballot_sync(0xffffffffu, need);
    if (bal) {
        int pos = 0;
        if (lane == 0)
            pos = atomicAdd(nhard, __popc(bal));
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (need)
            hard[pos + __popc(bal & ((1u << lane) - 1u))] = bi;
    }
}

// Phase 2b: the listed border blocks unite with touching earlier neighbours in
// other tiles; neighbours reached through an in-tile neighbour are skipped.
// Each lane first collects its block's union targets, then the warp issues
// them in rounds: lanes whose (block parent, neighbour parent) pairs are
// equal would unite the same two components, so one lane per distinct pair
// unites (parents only ever move towards roots, so equal parents read at
// any time mean equal roots).  Consecutive listed blocks mostly come from one
// tile and reach the same neighbouring components.
__global__ void k_bcc_cross_unite(int *P, const uint8_t *__restrict__ M, BGrid G, int *err, const int *hard,
                                  const int *nhard, unsigned long long *units)
{
    __shared__ BTabs tb;
    load_btabs(tb);
    __syncthreads();
    const int cnt = *nhard;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && cnt > 0)
        atomicAdd(units, (unsigned long long)cnt);
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int h0 = warp * 32; h0 < cnt; h0 += nwarps * 32) {
        // listed border blocks (block indices) and their offsets in their tile
        const int h = h0 + lane;
        unsigned todo = 0;
        int bi = 0, pb = 0;
        if (h < cnt) {
            bi = hard[h];
            int c2, c0, c1;
            G.coords(bi, c0, c1, c2);
            const int a = c0 % kT0, b = c1 % kT1, c = c2 % kT2;
            const unsigned m = M[bi];
            unsigned conn, local;
            bool full;
            uint64_t mlo, mhi;
            if (nb_interior(G, c0, c1, c2))
                border_conn<true, false, true>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            else
                border_conn<false, false, true>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            unsigned covered = 0;
            if (full && ((conn >> kCentre) & 1u))
                covered = conn & ~(1u << kCentre); // the centre links all of them
            while (local & ~covered) {
                const int q = next_cover(local & ~covered);
                covered |= bcover(q, conn & ~covered, mlo, mhi, tb);
            }
            while (conn & ~covered) {
                const unsigned rest = conn & ~covered;
                const int q = next_cover(rest);
                todo |= 1u << q;
                covered |= bcover(q, rest, mlo, mhi, tb);
            }
            pb = ld(P + bi);
        }
        while (__any_sync(0xffffffffu, todo != 0)) {
            int o = -1;
            unsigned long long key = ~0ull - (unsigned)lane; // unique for lanes without a target
            if (todo) {
                const int q = __ffs(todo) - 1;
                todo &= todo - 1;
                o = bi + nb_d0(q) * G.b1 * G.b2 + nb_d1(q) * G.b2 + nb_d2(q);
                key = ((unsigned long long)(unsigned)pb << 32) | (unsigned)ld(P + o);
            }
            const unsigned same = __match_any_sync(0xffffffffu, key);
            if (o >= 0 && (__ffs(same) - 1) == lane)
                unite(P, bi, o, err);
        }
    }
}

// Phases 2a and 2b in one pass: one thread block per tile, border item t on
// thread t; a border block that needs cross-tile unions collects its targets
// (as k_bcc_cross_unite does) and its warp unites in rounds, one lane per
// distinct (block parent, neighbour parent) pair.  Each border block and its
// neighbours' masks are read once, and no list is written.
__global__ void __launch_bounds__(512) k_bcc_cross_fused(int *P, const uint8_t *__restrict__ M, BGrid G, int *err,
                                                         unsigned long long *units)
{
    __shared__ BTabs tb;
    load_btabs(tb);
    __syncthreads();
    const int nt1 = (G.b1 + kT1 - 1) / kT1, nt2 = (G.b2 + kT2 - 1) / kT2;
    const int tile = blockIdx.x;
    const int ti = tile / (nt1 * nt2), tj = (tile / nt2) % nt1, tk = tile % nt2;
    const int t = threadIdx.x;
    if (t >= (kBorder + 31) / 32 * 32)
        return; // warps without border items
    const int lane = t & 31;
    unsigned todo = 0;
    int bi = 0, pb = 0;
    if (t < kBorder) {
        int a, b, c;
        border_block(t, a, b, c);
        const int c0 = ti * kT0 + a, c1 = tj * kT1 + b, c2 = tk * kT2 + c;
        const unsigned m = c0 < G.b0 && c1 < G.b1 && c2 < G.b2 ? M[(c0 * G.b1 + c1) * G.b2 + c2] : 0u;
        bi = (c0 * G.b1 + c1) * G.b2 + c2;
        if (m) {
            unsigned conn, local;
            bool full;
            uint64_t mlo, mhi;
            if (nb_interior(G, c0, c1, c2))
                border_conn<true, false, true>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            else
                border_conn<false, false, true>(M, G, bi, c0, c1, c2, a, b, c, m, conn, local, full, mlo, mhi);
            // in-tile neighbours were united in phase 1, and so was
            // everything touching them
            if ((conn & ~local) != 0 && !(full && ((conn >> kCentre) & 1u) && local)) {
                unsigned covered = 0;
                if (full && ((conn >> kCentre) & 1u))
                    covered = conn & ~(1u << kCentre); // the centre links all of them
                while (local & ~covered) {
                    const int q = next_cover(local & ~covered);
                    covered |= bcover(q, conn & ~covered, mlo, mhi, tb);
                }
                while (conn & ~covered) {
                    const unsigned rest = conn & ~covered;
                    const int q = next_cover(rest);
                    todo |= 1u << q;
                    covered |= bcover(q, rest, mlo, mhi, tb);
                }
                pb = ld(P + bi);
            }
        }
    }
    if (units && todo)
        atomicAdd(units, 1ull);
    while (__any_sync(0xffffffffu, todo != 0)) {
        int o = -1;
        unsigned long long key = ~0ull - (unsigned)lane; // unique for lanes without a target
        if (todo) {
            const int q = __ffs(todo) - 1;
            todo &= todo - 1;
            o = bi + nb_d0(q) * G.b1 * G.b2 + nb_d1(q) * G.b2 + nb_d2(q);
            key = ((unsigned long long)(unsigned)pb << 32) | (unsigned)ld(P + o);
        }
        const unsigned same = __match_any_sync(0xffffffffu, key);
        if (o >= 0 && (__ffs(same) - 1) == lane)
            unite(P, bi, o, err);
    }
}

static bool g_btables_ready[64] = {false};

static int ensure_block_tables()
{
    int dev = 0;
    PMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_btables_ready[dev])
        return PMG_OK;
    int nb[13][3];
    unsigned short adj[13];
    host_tables(nb, adj);
    uint8_t self[13], other[13], pair[13][13];
    for (int q = 0; q < 13; q++) {
        self[q] = (uint8_t)touch_mask(nb[q][0], nb[q][1], nb[q][2]);
        other[q] = (uint8_t)touch_mask(-nb[q][0], -nb[q][1], -nb[q][2]);
        for (int r = 0; r < 13; r++)
            pair[r][q] = (adj[r] >> q) & 1
                             ? (uint8_t)touch_mask(nb[q][0] - nb[r][0], nb[q][1] - nb[r][1], nb[q][2] - nb[r][2])
                             : (uint8_t)0;
    }
    PMG_CUDA(cudaMemcpyToSymbol(c_bt_self, self, sizeof(self)));
    PMG_CUDA(cudaMemcpyToSymbol(c_bt_nb, other, sizeof(other)));
    PMG_CUDA(cudaMemcpyToSymbol(c_bt_pair, pair, sizeof(pair)));
    signed char gd[26][3];
    uint8_t gself[26], gnb[26];
    int q26 = 0;
    for (int d0 = -1; d0 <= 1; d0++)
        for (int d1 = -1; d1 <= 1; d1++)
            for (int d2 = -1; d2 <= 1; d2++) {
                if (!d0 && !d1 && !d2)
                    continue;
                gd[q26][0] = (signed char)d0;
                gd[q26][1] = (signed char)d1;
                gd[q26][2] = (signed char)d2;
                gself[q26] = (uint8_t)touch_mask(d0, d1, d2);
                gnb[q26] = (uint8_t)touch_mask(-d0, -d1, -d2);
                q26++;
            }
    PMG_CUDA(cudaMemcpyToSymbol(c_g_d, gd, sizeof(gd)));
    PMG_CUDA(cudaMemcpyToSymbol(c_g_self, gself, sizeof(gself)));
    PMG_CUDA(cudaMemcpyToSymbol(c_g_nb, gnb, sizeof(gnb)));
    if (dev >= 0 && dev < 64)
        g_btables_ready[dev] = true;
    return PMG_OK;
}

// periodic seams at block level: a foreground halo voxel joins the block of the
// own voxel it copies when that voxel is foreground too
__device__ __forceinline__ bool mfg(const uint8_t *__restrict__ M, const BGrid &G, long long i, long long j,
                                    long long k)
{
    const int b = (int)(((i >> 1) * G.b1 + (j >> 1)) * G.b2 + (k >> 1));
    return (M[b] >> ((((int)i & 1) * 2 + ((int)j & 1)) * 2 + ((int)k & 1))) & 1;
}

__global__ void k_bcc_twins(const uint8_t *__restrict__ M, int *P, BGrid G, Twins W, int *err)
{
    const long long n = W.s0 * W.s1 * W.s2;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        long long c[3];
        c[2] = idx % W.s2;
        const long long r = idx / W.s2;
        c[1] = r % W.s1;
        c[0] = r / W.s1;
        bool halo = false, ok = true;
        long long t[3];
        for (int d = 0; d < 3; d++) {
            t[d] = c[d];
            const long long S = d == 0 ? W.s0 : d == 1 ? W.s1 : W.s2;
            if (c[d] < W.own_lo[d] || c[d] >= W.own_lo[d] + W.own_len[d]) {
                if (!W.periodic[d] || W.own_len[d] <= 0 || c[d] >= S) {
                    ok = false;
                } else {
                    long long q = (c[d] - W.own_lo[d]) % W.own_len[d];
                    if (q < 0)
                        q += W.own_len[d];
                    t[d] = q + W.own_lo[d];
                    halo = true;
                }
            }
        }
        if (!halo || !ok || !mfg(M, G, c[0], c[1], c[2]) || !mfg(M, G, t[0], t[1], t[2]))
            continue;
        const int ba = (int)(((c[0] >> 1) * G.b1 + (c[1] >> 1)) * G.b2 + (c[2] >> 1));
        const int bb = (int)(((t[0] >> 1) * G.b1 + (t[1] >> 1)) * G.b2 + (t[2] >> 1));
        unite(P, ba, bb, err);
    }
}

__global__ void k_bcc_flatten(int *P, int nb, int *err)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const int p = P[b];
        if (p >= 0 && p != b)
            P[b] = find_root(P, p, err);
    }
}

// two consecutive coordinates v0, v0 + 1 inside [lo, hi): bits 0, 1
__device__ __forceinline__ unsigned in2(int v0, long long lo, long long hi)
{
    return (unsigned)(v0 >= lo && v0 < hi) | ((unsigned)(v0 + 1 >= lo && v0 + 1 < hi) << 1);
}

// per-axis 2-bit masks spread over the block's bit layout (x * 2 + y) * 2 + z
__device__ __forceinline__ unsigned spread_x(unsigned a) { return (a & 1 ? 0x0Fu : 0u) | (a & 2 ? 0xF0u : 0u); }
__device__ __forceinline__ unsigned spread_y(unsigned a) { return (a & 1 ? 0x33u : 0u) | (a & 2 ? 0xCCu : 0u); }
__device__ __forceinline__ unsigned spread_z(unsigned a) { return (a & 1 ? 0x55u : 0u) | (a & 2 ? 0xAAu : 0u); }

// bytes 0 and 1 of a 16-bit pair equal to v: bits 0, 1
__device__ __forceinline__ unsigned eq2(unsigned pair, unsigned v)
{
    return (unsigned)((pair & 0xffu) == v) | ((unsigned)((pair >> 8) == v) << 1);
}

// Marks of the roots of the blocks with a foreground voxel inside the box:
// one thread per block that meets the box.
__global__ void k_bcc_mark(const uint8_t *__restrict__ M, const int *__restrict__ P, BGrid G, Box bx,
                           uint8_t *mark, uint8_t bit, int *err)
{
    long long lo[3], nbk[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = bx.lo[d] >> 1;
        nbk[d] = ((bx.hi[d] + 1) >> 1) - lo[d];
    }
    const long long n = nbk[0] * nbk[1] * nbk[2];
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c2 = (int)(lo[2] + q % nbk[2]), c1 = (int)(lo[1] + (q / nbk[2]) % nbk[1]),
                  c0 = (int)(lo[0] + q / (nbk[2] * nbk[1]));
        const int b = (c0 * G.b1 + c1) * G.b2 + c2;
        const unsigned inbox = spread_x(in2(2 * c0, bx.lo[0], bx.hi[0])) & spread_y(in2(2 * c1, bx.lo[1], bx.hi[1])) &
                               spread_z(in2(2 * c2, bx.lo[2], bx.hi[2]));
        if (!(M[b] & inbox))
            continue;
        int p = ld(P + b);
        if (p >= 0)
            p = find_root(P, p, err);
        if (p >= 0 && !(mark[p] & bit))
            atomicOr((unsigned int *)(mark + (p & ~3)), (unsigned int)bit << (8 * (p & 3)));
    }
}

// k_bcc_mark for two block union-finds of the same grid at once
// (blockIdx.y picks the set), marking the same face box.
__global__ void k_bcc_mark2(const uint8_t *__restrict__ Ma, const int *__restrict__ Pa, uint8_t *mark_a,
                            const uint8_t *__restrict__ Mb, const int *__restrict__ Pb, uint8_t *mark_b, BGrid G,
                            Box bx, uint8_t bit, int *err)
{
    const uint8_t *M = blockIdx.y ? Mb : Ma;
    const int *P = blockIdx.y ? Pb : Pa;
    uint8_t *mark = blockIdx.y ? mark_b : mark_a;
    long long lo[3], nbk[3];
    for (int d = 0; d < 3; d++) {
        lo[d] = bx.lo[d] >> 1;
        nbk[d] = ((bx.hi[d] + 1) >> 1) - lo[d];
    }
    const long long n = nbk[0] * nbk[1] * nbk[2];
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int c2 = (int)(lo[2] + q % nbk[2]), c1 = (int)(lo[1] + (q / nbk[2]) % nbk[1]),
                  c0 = (int)(lo[0] + q / (nbk[2] * nbk[1]));
        const int b = (c0 * G.b1 + c1) * G.b2 + c2;
        const unsigned inbox = spread_x(in2(2 * c0, bx.lo[0], bx.hi[0])) & spread_y(in2(2 * c1, bx.lo[1], bx.hi[1])) &
                               spread_z(in2(2 * c2, bx.lo[2], bx.hi[2]));
        if (!(M[b] & inbox))
            continue;
        int p = ld(P + b);
        if (p >= 0)
            p = find_root(P, p, err);
        if (p >= 0 && !(mark[p] & bit))
            atomicOr((unsigned int *)(mark + (p & ~3)), (unsigned int)bit << (8 * (p & 3)));
    }
}

// One thread per block: the block's root and marks decide all its voxels at
// once; kept foreground voxels receive `val`, everything else 0.  A warp
// covers 32 consecutive blocks, i.e. 64 contiguous voxels of each of the
// block's four rows.
template <typename TO>
__global__ void k_bcc_select(const uint8_t *__restrict__ M, int *P, const uint8_t *__restrict__ mark, BGrid G,
                             int mode, TO val, TO *__restrict__ out, unsigned long long *kept, int *err)
{
    const int nb = G.b0 * G.b1 * G.b2;
    unsigned int cnt = 0; // kept voxels (mask bits exist only for voxels inside the volume)
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int c0, c1, c2;
        G.coords(b, c0, c1, c2);
        unsigned m = M[b];
        if (m) {
            // the root, and the parent flattened to it
            int p = ld(P + b);
            if (p >= 0 && p != b) {
                const int q = find_root(P, p, err);
                if (q != p)
                    P[b] = q;
                p = q;
            }
            const uint8_t mk = p >= 0 ? mark[p] : 0;
            const bool in = mk & 1, ou = mk & 2;
            bool keep;
            if (mode == PMG_SEL_INLET)
                keep = in;
            else if (mode == PMG_SEL_OUTLET)
                keep = ou;
            else if (mode == PMG_SEL_BOTH)
                keep = in && ou;
            else
                keep = !(in || ou);
            if (!keep)
                m = 0;
        }
        cnt += __popc(m);
#pragma unroll
        for (int x = 0; x < 2; x++)
#pragma unroll
            for (int y = 0; y < 2; y++) {
                const int i = 2 * c0 + x, j = 2 * c1 + y;
                if (i >= G.s0 || j >= G.s1)
                    continue;
                TO *row = out + ((long long)i * G.s1 + j) * G.s2;
#pragma unroll
                for (int z = 0; z < 2; z++) {
                    const int k = 2 * c2 + z;
                    if (k < G.s2)
                        row[k] = ((m >> ((x * 2 + y) * 2 + z)) & 1) ? val : (TO)0;
                }
            }
    }
    if (kept) {
        for (int o = 16; o > 0; o >>= 1)
            cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        if ((threadIdx.x & 31) == 0 && cnt)
            atomicAdd(kept, (unsigned long long)cnt);
    }
}

__host__ __device__ inline const uint8_t *src_elem(const SrcImg &s) { return s.img; }
__host__ __device__ inline const uint16_t *src_elem(const SrcErode &s) { return s.E; }
__host__ __device__ inline const uint8_t *src_elem(const SrcStep &s) { return s.S; }
// bytes a tile pass reads from its source: one element per voxel, or one mask per block
template <class Src>
static double src_bytes(const Src &src, long long n, long long nb)
{
    return std::is_same<Src, SrcMask>::value ? (double)nb : (double)n * sizeof(*src_elem(src));
}
__host__ __device__ inline const uint8_t *src_elem(const SrcMask &s) { return s.M; }

static BGrid bgrid_of(const int64_t *shape)
{
    BGrid G;
    G.s0 = (int)shape[0];
    G.s1 = (int)shape[1];
    G.s2 = (int)shape[2];
    G.b0 = (G.s0 + 1) / 2;
    G.b1 = (G.s1 + 1) / 2;
    G.b2 = (G.s2 + 1) / 2;
    G.q2 = fastdiv_of((unsigned)G.b2);
    G.q1 = fastdiv_of((unsigned)G.b1);
    return G;
}

// Block union-find of the source: tiles, cross-tile unions, periodic seams
// (twins), flattening.  P[b] = root block (the smallest block index of the
// component), -1 for empty blocks; M[b] = block mask.
template <class Src>
static int bcc_build(const Src &src, const int64_t *shape, const int32_t *bc, const int32_t *pad, bool twins,
                     int *P, uint8_t *M, int *err, cudaStream_t st, bool flatten = true, int *Pl = nullptr,
                     int *dirty = nullptr, int *hard_buf = nullptr)
{
    PMG_TRY(ensure_tables());
    PMG_TRY(ensure_block_tables());
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    {
        const int nt = ((G.b0 + kT0 - 1) / kT0) * ((G.b1 + kT1 - 1) / kT1) * ((G.b2 + kT2 - 1) / kT2);
        const int ps__ = prof_begin("k_bcc_tile", st);
        k_bcc_tile<Src><<<nt, kTile, 0, st>>>(src, P, M, G, Pl, dirty);
        prof_end(ps__, src_bytes(src, n, nb) + (double)nb * 5, st);
    }
    PMG_CHECK_LAUNCH();
    if (tune_value(kTuneCcCrossFused)) {
        const int nt = ((G.b0 + kT0 - 1) / kT0) * ((G.b1 + kT1 - 1) / kT1) * ((G.b2 + kT2 - 1) / kT2);
        const int ps__ = prof_begin("k_bcc_cross_fused", st);
        k_bcc_cross_fused<<<nt, 512, 0, st>>>(P, M, G, err, prof_units(kUnitsCrossUnite));
        // per border block: its mask and the masks of its 13 earlier
        // neighbours; two parents per union
        prof_end(ps__, (double)nt * kBorder * 14, st);
        PMG_CHECK_LAUNCH();
    } else {
        const long long border = (long long)((G.b0 + kT0 - 1) / kT0) * ((G.b1 + kT1 - 1) / kT1) *
                                 ((G.b2 + kT2 - 1) / kT2) * kBorder;
        // list of the border blocks that need unions, and its length (in the
        // caller's buffer of border + 64 ints, if given)
        int *hard = hard_buf;
        if (!hard)
            PMG_TRY(scratch_alloc((void **)&hard, sizeof(int) * (size_t)(border + 64), st));
        int *nhard = hard + border + 32;
        PMG_CUDA(cudaMemsetAsync(nhard, 0, sizeof(int), st));
        {
            const int ps__ = prof_begin("k_bcc_cross", st);
            const int nt = (int)(border / kBorder);
            k_bcc_cross<<<nt, 512, 0, st>>>(M, G, hard, nhard);
            // per border block: its mask, the mask facing it across the tile
            // border
            prof_end(ps__, (double)border * 2, st);
        }
        PMG_CHECK_LAUNCH();
        {
            const int ps__ = prof_begin("k_bcc_cross_unite", st);
            k_bcc_cross_unite<<<152 * 16, 256, 0, st>>>(P, M, G, err, hard, nhard, prof_units(kUnitsCrossUnite));
            // per listed border block: its entry and mask, the masks of its 13
            // earlier neighbours, two parents per union
            prof_end_units(ps__, kUnitsCrossUnite, 4 + 1 + 13 + 8, st);
        }
        PMG_CHECK_LAUNCH();
        if (!hard_buf)
            PMG_TRY(scratch_free(hard, st));
    }
    if (twins && any_periodic(bc)) {
        const int ps__ = prof_begin("k_bcc_twins", st);
        k_bcc_twins<<<grid_for(n, 256, 152LL * 32), 256, 0, st>>>(M, P, G, make_twins(shape, bc, pad), err);
        prof_end(ps__, 0.0, st);
        PMG_CHECK_LAUNCH();
    }
    if (flatten) {
        const int ps__ = prof_begin("k_bcc_flatten", st);
        k_bcc_flatten<<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(P, nb, err);
        prof_end(ps__, (double)nb * 8, st);
        PMG_CHECK_LAUNCH();
    }
    return PMG_OK;
}

// Inlet / outlet boxes (lo0, hi0, lo1, hi1, lo2, hi2; null or lo0 < 0 for
// none) must lie inside the volume.
static int check_boxes(const int64_t *shape, const int64_t *inlet_box, const int64_t *outlet_box)
{
    const int64_t *boxes[2] = {inlet_box, outlet_box};
    for (int w = 0; w < 2; w++) {
        const int64_t *bxp = boxes[w];
        if (!bxp || bxp[0] < 0)
            continue;
        for (int d = 0; d < 3; d++)
            if (bxp[2 * d] < 0 || bxp[2 * d + 1] > shape[d] || bxp[2 * d] > bxp[2 * d + 1]) {
                set_error("connected-image selection: face box outside the volume");
                return PMG_EINVAL;
            }
    }
    return PMG_OK;
}

// Marks of the roots of blocks with foreground in the inlet (bit 0) and
// outlet (bit 1) boxes; parents need not be flat.
static int bcc_marks(const int64_t *shape, const int64_t *inlet_box, const int64_t *outlet_box, const int *P,
                     const uint8_t *M, uint8_t *mark, int *err, cudaStream_t st)
{
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    PMG_CUDA(cudaMemsetAsync(mark, 0, ((size_t)nb + 3) & ~(size_t)3, st));
    const int64_t *boxes[2] = {inlet_box, outlet_box};
    for (int w = 0; w < 2; w++) {
        const int64_t *bxp = boxes[w];
        if (!bxp || bxp[0] < 0)
            continue;
        Box b;
        for (int d = 0; d < 3; d++) {
            b.lo[d] = bxp[2 * d];
            b.hi[d] = bxp[2 * d + 1];
        }
        if (b.size() > 0) {
            long long nbk = 1;
            for (int d = 0; d < 3; d++)
                nbk *= ((b.hi[d] + 1) >> 1) - (b.lo[d] >> 1);
            const int ps__ = prof_begin("k_bcc_mark", st);
            k_bcc_mark<<<grid_for(nbk, 256, 1LL << 30), 256, 0, st>>>(M, P, G, b, mark, (uint8_t)(1 << w), err);
            // per block meeting the box: mask, parent, root parent
            prof_end(ps__, (double)nbk * 9, st);
            PMG_CHECK_LAUNCH();
        }
    }
    return PMG_OK;
}

// The selection from parents P (flattened on the way), masks M and marks.
static int bcc_select_out(void *out, int out_bytes, const int64_t *shape, int mode, int val, int *P,
                          const uint8_t *M, const uint8_t *mark, int *err, cudaStream_t st,
                          unsigned long long *kept)
{
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    const int ps__ = prof_begin("k_bcc_select", st);
    if (out_bytes == 1)
        k_bcc_select<uint8_t><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(M, P, mark, G, mode, (uint8_t)val,
                                                                           (uint8_t *)out, kept, err);
    else
        k_bcc_select<uint64_t><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(M, P, mark, G, mode, (uint64_t)val,
                                                                            (uint64_t *)out, kept, err);
    prof_end(ps__, (double)n * out_bytes + (double)nb * 5, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

static int bcc_mark_select(void *out, int out_bytes, const int64_t *shape, const int64_t *inlet_box,
                           const int64_t *outlet_box, int mode, int val, int *P, const uint8_t *M, uint8_t *mark,
                           int *err, cudaStream_t st, unsigned long long *kept)
{
    PMG_TRY(bcc_marks(shape, inlet_box, outlet_box, P, M, mark, err, st));
    return bcc_select_out(out, out_bytes, shape, mode, val, P, M, mark, err, st, kept);
}

template <class Src>
static int bcc_select_core(const Src &src, void *out, int out_bytes, const int64_t *shape, const int32_t *bc,
                           const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode,
                           int val, int *P, uint8_t *M, uint8_t *mark, int *err, cudaStream_t st,
                           unsigned long long *kept)
{
    PMG_TRY(check_boxes(shape, inlet_box, outlet_box));
    PMG_TRY(bcc_build(src, shape, bc, pad, true, P, M, err, st, false));
    return bcc_mark_select(out, out_bytes, shape, inlet_box, outlet_box, mode, val, P, M, mark, err, st, kept);
}

// Binary selection: P and mark need one int / one byte per 2x2x2 block.  Kept
// voxels receive `fgval`, or 1 for fgval < 0 (an image of 0s and 1s).
int select_run_binary(const uint8_t *img, void *out, int out_bytes, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode,
                      int fgval, int *P, uint8_t *M, uint8_t *mark, int *err, cudaStream_t st,
                      unsigned long long *kept)
{
    SrcImg src{img, fgval};
    return bcc_select_core(src, out, out_bytes, shape, bc, pad, inlet_box, outlet_box, mode, fgval >= 0 ? fgval : 1,
                           P, M, mark, err, st, kept);
}

// Erosion fused into the selection: the foreground is E > T off the wall
// planes, with E a capped squared EDT (uint16, units of res^2) of the
// unextended image; kept voxels receive 1.
int select_run_erode(const uint16_t *E, int T, void *out, const int64_t *shape, const int32_t *bc,
                     const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode, int *P,
                     uint8_t *M, uint8_t *mark, int *err, cudaStream_t st, unsigned long long *kept)
{
    SrcErode src;
    src.E = E;
    src.T = T;
    src.s0 = (int)shape[0];
    src.s1 = (int)shape[1];
    src.s2 = (int)shape[2];
    src.walls = 0;
    for (int q = 0; q < 6; q++)
        src.walls |= (bc[q] == PMG_BC_WALL ? 1u : 0u) << q;
    return bcc_select_core(src, out, 1, shape, bc, pad, inlet_box, outlet_box, mode, 1, P, M, mark, err, st, kept);
}

// ---- selection of a growing set -----------------------------------------------
// Along a drainage curve two selected sets only ever grow: the eroded pore
// space (its threshold falls with the radius) and the non-wetting phase (the
// update turns wetting voxels non-wetting, never back).  Components of a
// growing set only merge, so after one full block union-find a step re-reads
// the block masks, lists the blocks whose mask grew, and unites each of them
// with every touching neighbour; a pair of blocks that starts to touch always
// has a grown member, and every other block keeps its parent.  The parents
// keep pointing to smaller indices, so roots stay the smallest block of each
// component and the flattened parents, marks and selection are those of a
// full union-find of the same set.

// New masks; a block whose mask changed is listed (warp-aggregated append)
// and, if it was empty, becomes its own root.  A mask that lost voxels is an
// error (code 3): the set did not grow.
template <class Src>
__global__ void k_grow_masks(Src src, uint8_t *__restrict__ M, int *__restrict__ P, BGrid G, int *list,
                             int *count, int *err)
{
    const int nb = G.b0 * G.b1 * G.b2;
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < nb; base += gridDim.x * blockDim.x) {
        const int b = base + threadIdx.x;
        bool changed = false;
        if (b < nb) {
            // the old mask and the source are loaded independently
            int c2, c0, c1;
            G.coords(b, c0, c1, c2);
            const unsigned old = M[b];
            const unsigned m = block_mask(src, G, c0, c1, c2);
            if (m != old) {
                if (old & ~m)
                    atomicExch(err, 3);
                M[b] = (uint8_t)m;
                if (!old)
                    P[b] = b;
                changed = true;
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, changed);
        if (bal) {
            int pos = 0;
            if (lane == 0)
                pos = atomicAdd(count, __popc(bal));
            pos = __shfl_sync(0xffffffffu, pos, 0);
            if (changed)
                list[pos + __popc(bal & ((1u << lane) - 1u))] = b;
        }
    }
}


// One warp per listed block, one lane per neighbour (lanes 0-25): every lane
// loads its neighbour's mask and parent at once.  The parents were flattened
// after the previous step, so a touching neighbour whose parent equals the
// block's starting parent is already in its component; of the others, one
// lane per distinct parent unites (neighbours with one parent are in one
// component already).
// One listed block b of a growing set: its lane's neighbour (q, d) and, once
// per distinct neighbour parent, the union.
__device__ __forceinline__ void grow_unite_block(int *P, const uint8_t *__restrict__ M, const BGrid &G, int b,
                                                 int lane, int d0, int d1, int d2, unsigned tself, unsigned tnb,
                                                 int *err)
{
    int c2, c0, c1;
    G.coords(b, c0, c1, c2);
    const unsigned m = M[b];
    const int pb = ld(P + b);
    const int a0 = c0 + d0, a1 = c1 + d1, a2 = c2 + d2;
    const bool valid = (m & tself) && a0 >= 0 && a1 >= 0 && a2 >= 0 && a0 < G.b0 && a1 < G.b1 && a2 < G.b2;
    const int o = (a0 * G.b1 + a1) * G.b2 + a2;
    unsigned mo = 0;
    int po = -1;
    if (valid) {
        mo = M[o];
        po = ld(P + o);
    }
    const bool need = (mo & tnb) && po != pb;
    const unsigned needs = __ballot_sync(0xffffffffu, need);
    if (!needs)
        return;
    const unsigned same = __match_any_sync(0xffffffffu, need ? po : -2 - lane);
    if (need && (__ffs(same & needs) - 1) == lane)
        unite(P, b, o, err);
}

// A set's listed blocks: step k's precomputed list (off) or the list a mask
// pass (or the drainage update) filled (count).
struct UniteList {
    int *P;
    const uint8_t *M;
    const int *list, *count, *off;
    __device__ __forceinline__ int size(const int *&l) const
    {
        if (off) {
            l = list + off[0];
            return off[1] - off[0];
        }
        l = list;
        return *count;
    }
};

// One warp per listed block of set A, then of set B (two growing sets of the
// same grid in one launch: their dependent loads overlap), one lane per
// neighbour (lanes 0-25): every lane loads its neighbour's mask and parent
// at once.  The parents were flattened after the previous step, so a
// touching neighbour whose parent equals the block's starting parent is
// already in its component; of the others, one lane per distinct parent
// unites (neighbours with one parent are in one component already).
__global__ void k_grow_unite2(UniteList A, UniteList B, BGrid G, int *err, unsigned long long *units)
{
    const int *la = nullptr, *lb = nullptr;
    const int ca = A.P ? A.size(la) : 0, cb = B.P ? B.size(lb) : 0;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && ca + cb > 0)
        atomicAdd(units, (unsigned long long)(ca + cb));
    const int lane = threadIdx.x & 31;
    const int q = lane < 13 ? lane : lane + 1; // offset code (d0 + 1) * 9 + (d1 + 1) * 3 + d2 + 1, 13 skipped
    const int d0 = q / 9 - 1, d1 = (q / 3) % 3 - 1, d2 = q % 3 - 1;
    const unsigned tself = lane < 26 ? touch_bits(d0, d1, d2) : 0u, tnb = touch_bits(-d0, -d1, -d2);
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = warp; it < (long long)ca + cb; it += nwarps) {
        if (it < ca)
            grow_unite_block(A.P, A.M, G, la[it], lane, d0, d1, d2, tself, tnb, err);
        else
            grow_unite_block(B.P, B.M, G, lb[it - ca], lane, d0, d1, d2, tself, tnb, err);
    }
}

// A single set: set B empty.
__global__ void k_grow_unite(int *P, const uint8_t *__restrict__ M, BGrid G, const int *__restrict__ list,
                             const int *__restrict__ count, const int *__restrict__ off, int *err,
                             unsigned long long *units)
{
    UniteList A{P, M, list, count, off};
    const int *la = nullptr;
    const int ca = A.size(la);
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && ca > 0)
        atomicAdd(units, (unsigned long long)ca);
    const int lane = threadIdx.x & 31;
    const int q = lane < 13 ? lane : lane + 1;
    const int d0 = q / 9 - 1, d1 = (q / 3) % 3 - 1, d2 = q % 3 - 1;
    const unsigned tself = lane < 26 ? touch_bits(d0, d1, d2) : 0u, tnb = touch_bits(-d0, -d1, -d2);
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = warp; it < ca; it += nwarps)
        grow_unite_block(P, M, G, la[it], lane, d0, d1, d2, tself, tnb, err);
}

size_t grow_sel_bytes(const int64_t *shape)
{
    const BGrid G = bgrid_of(shape);
    const size_t nb = (size_t)G.b0 * G.b1 * G.b2;
    const size_t a = (nb + 255) & ~(size_t)255;
    return a * 4 + a + a + a * 4 + 256;
}

void grow_sel_init(GrowSel &g, void *mem, const int64_t *shape)
{
    const BGrid G = bgrid_of(shape);
    const size_t nb = (size_t)G.b0 * G.b1 * G.b2;
    const size_t a = (nb + 255) & ~(size_t)255;
    char *p = (char *)mem;
    g.P = (int *)p;
    p += a * 4;
    g.M = (uint8_t *)p;
    p += a;
    g.mark = (uint8_t *)p;
    p += a;
    g.list = (int *)p;
    p += a * 4;
    g.count = (int *)p;
    g.built = false;
}

// One step of a growing selection up to the marks: the full block union-find
// the first time, afterwards the grown blocks only.
// Listed blocks take their masks from the source (steps known in advance).
template <class Src>
__global__ void k_grow_apply(Src src, uint8_t *__restrict__ M, int *__restrict__ P, BGrid G,
                             const int *__restrict__ list, const int *__restrict__ off, int *err,
                             unsigned long long *units)
{
    const int a = off[0], cnt = off[1] - a;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && cnt > 0)
        atomicAdd(units, (unsigned long long)cnt);
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < cnt; it += gridDim.x * blockDim.x) {
        const int b = list[a + it];
        int c2, c0, c1;
        G.coords(b, c0, c1, c2);
        const unsigned old = M[b];
        const unsigned m = block_mask(src, G, c0, c1, c2);
        if (old & ~m)
            atomicExch(err, 3);
        M[b] = (uint8_t)m;
        if (!old)
            P[b] = b;
    }
}

template <class Src>
static int grow_step(GrowSel &g, const Src &src, const int64_t *shape, const int32_t *bc, const int32_t *pad,
                     const int64_t *inlet_box, const int64_t *outlet_box, int *err, cudaStream_t st,
                     const int *off = nullptr)
{
    PMG_TRY(check_boxes(shape, inlet_box, outlet_box));
    if (!g.built) {
        PMG_TRY(bcc_build(src, shape, bc, pad, true, g.P, g.M, err, st, false));
        g.built = true;
        return bcc_marks(shape, inlet_box, outlet_box, g.P, g.M, g.mark, err, st);
    }
    PMG_TRY(ensure_tables());
    PMG_TRY(ensure_block_tables());
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    if (off) {
        const int ps__ = prof_begin("k_grow_apply", st);
        k_grow_apply<Src><<<152 * 8, 256, 0, st>>>(src, g.M, g.P, G, g.ev, off, err, prof_units(kUnitsGrowApply));
        // per listed block: its list entry, eight source elements, mask read
        // and written, parent written
        prof_end_units(ps__, kUnitsGrowApply, 4 + 8 * sizeof(*src_elem(src)) + 2 + 4, st);
        PMG_CHECK_LAUNCH();
    } else if (g.pending) {
        g.pending = false;
    } else {
        PMG_CUDA(cudaMemsetAsync(g.count, 0, sizeof(int), st));
        const int ps__ = prof_begin("k_grow_masks", st);
        k_grow_masks<Src><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(src, g.M, g.P, G, g.list, g.count, err);
        prof_end(ps__, (double)n * sizeof(*src_elem(src)) + (double)nb, st);
        PMG_CHECK_LAUNCH();
    }
    {
        const int ps__ = prof_begin(g.unite_label, st);
        k_grow_unite<<<152 * 32, 256, 0, st>>>(g.P, g.M, G, off ? g.ev : g.list, g.count, off, err,
                                               prof_units(g.unite_units));
        // per listed block: its list entry, mask and parent, and the masks and
        // parents of its 26 neighbours
        if (g.unite_units >= 0)
            prof_end_units(ps__, g.unite_units, 4 + 5 + 26 * 5, st);
        else
            prof_end(ps__, 0.0, st);
    }
    PMG_CHECK_LAUNCH();
    if (any_periodic(bc)) {
        const int ps__ = prof_begin("k_bcc_twins", st);
        k_bcc_twins<<<grid_for(n, 256, 152LL * 32), 256, 0, st>>>(g.M, g.P, G, make_twins(shape, bc, pad), err);
        prof_end(ps__, 0.0, st);
        PMG_CHECK_LAUNCH();
    }
    return bcc_marks(shape, inlet_box, outlet_box, g.P, g.M, g.mark, err, st);
}

template <class Src>
static int grow_select_core(GrowSel &g, const Src &src, void *out, const int64_t *shape, const int32_t *bc,
                            const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode,
                            int val, int *err, cudaStream_t st, unsigned long long *kept)
{
    PMG_TRY(grow_step(g, src, shape, bc, pad, inlet_box, outlet_box, err, st));
    return bcc_select_out(out, 1, shape, mode, val, g.P, g.M, g.mark, err, st, kept);
}

static SrcErode erode_src(const uint16_t *E, int T, const int64_t *shape, const int32_t *bc)
{
    SrcErode src;
    src.E = E;
    src.T = T;
    src.s0 = (int)shape[0];
    src.s1 = (int)shape[1];
    src.s2 = (int)shape[2];
    src.walls = 0;
    for (int q = 0; q < 6; q++)
        src.walls |= (bc[q] == PMG_BC_WALL ? 1u : 0u) << q;
    return src;
}

constexpr int kPairBatch = 4;

// Inlet selections of two growing sets A and B in one pass: out = 1 where A
// is inlet-connected and, when *b_count > 0, B is inlet-connected too
// (porosimetry.py:130-148: img_results kept where n_connected == 1 once the
// phase exists); kept counts A's inlet-connected voxels before the
// constraint.  Both parent arrays are flattened on the way.
// BLK: out holds one mask per 2x2x2 block (bit (x * 2 + y) * 2 + z), else
// one byte per voxel.
template <bool BLK>
__global__ void k_grow_pair_select(const uint8_t *__restrict__ MA, int *PA, const uint8_t *__restrict__ markA,
                                   const uint8_t *__restrict__ MB, int *PB, const uint8_t *__restrict__ markB,
                                   const unsigned long long *__restrict__ b_count, BGrid G,
                                   uint8_t *__restrict__ out, unsigned long long *kept, int *err, int *xr)
{
    const int nb = G.b0 * G.b1 * G.b2;
    const bool constrain = *b_count > 0;
    unsigned int cnt = 0;
    int xmax = 0, xmin = 0; // block-plane range of the output's voxels, encoded as in XRange
    // kPairBatch blocks per thread, each level of the root lookups (masks,
    // parents, their parents, marks) loaded for all of them before any is
    // used: the lookups are chains of dependent loads
    constexpr int NB = kPairBatch;
    for (int base = blockIdx.x * blockDim.x * NB + threadIdx.x; base < nb; base += gridDim.x * blockDim.x * NB) {
        int bb[NB], pa[NB], pb[NB], ga[NB], gb[NB];
        unsigned m[NB], mb[NB], ka[NB], kb[NB];
#pragma unroll
        for (int q = 0; q < NB; q++) {
            bb[q] = base + q * blockDim.x;
            const bool in = bb[q] < nb;
            m[q] = in ? MA[bb[q]] : 0u;
            mb[q] = in ? MB[bb[q]] : 0u;
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            pa[q] = m[q] ? ld(PA + bb[q]) : -1;
            pb[q] = mb[q] ? ld(PB + bb[q]) : -1;
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            ga[q] = pa[q] >= 0 && pa[q] != bb[q] ? ld(PA + pa[q]) : pa[q];
            gb[q] = pb[q] >= 0 && pb[q] != bb[q] ? ld(PB + pb[q]) : pb[q];
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            // the root: the parent when it is its own parent, else further up
            // (rare once the parents were flattened); parents flattened to it
            int ra = pa[q], rb = pb[q];
            if (ra >= 0 && ra != bb[q] && ga[q] != ra)
                ra = find_root(PA, ga[q], err);
            if (rb >= 0 && rb != bb[q] && gb[q] != rb)
                rb = find_root(PB, gb[q], err);
            if (ra != pa[q])
                PA[bb[q]] = ra;
            if (rb != pb[q])
                PB[bb[q]] = rb;
            pa[q] = ra;
            pb[q] = rb;
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            ka[q] = pa[q] >= 0 ? markA[pa[q]] : 0u;
            kb[q] = pb[q] >= 0 ? markB[pb[q]] : 0u;
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            const int b = bb[q];
            if (b >= nb)
                continue;
            int c0, c1, c2;
            G.coords(b, c0, c1, c2);
            unsigned mm = ka[q] & 1u ? m[q] : 0u;
            const unsigned keepB = kb[q] & 1u ? mb[q] : 0u;
            cnt += __popc(mm);
            if (constrain)
                mm &= keepB;
            if (mm) {
                xmax = max(xmax, c0 + 1);
                xmin = max(xmin, kRangeBig - c0);
            }
            if constexpr (BLK) {
                out[b] = (uint8_t)mm;
            } else {
#pragma unroll
                for (int x = 0; x < 2; x++)
#pragma unroll
                    for (int y = 0; y < 2; y++) {
                        const int i = 2 * c0 + x, j = 2 * c1 + y;
                        if (i >= G.s0 || j >= G.s1)
                            continue;
                        uint8_t *row = out + ((long long)i * G.s1 + j) * G.s2;
#pragma unroll
                        for (int z = 0; z < 2; z++) {
                            const int k = 2 * c2 + z;
                            if (k < G.s2)
                                row[k] = (uint8_t)((mm >> ((x * 2 + y) * 2 + z)) & 1);
                        }
                    }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        xmax = max(xmax, __shfl_down_sync(0xffffffffu, xmax, o));
        xmin = max(xmin, __shfl_down_sync(0xffffffffu, xmin, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (cnt)
            atomicAdd(kept, (unsigned long long)cnt);
        if (xr && xmax) {
            atomicMax(xr, xmax);
            atomicMax(xr + 1, xmin);
        }
    }
}

int grow_marks_erode(GrowSel &g, const uint16_t *E, int T, const int64_t *shape, const int32_t *bc,
                     const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st)
{
    return grow_step(g, erode_src(E, T, shape, bc), shape, bc, pad, inlet_box, nullptr, err, st);
}

int grow_marks_step(GrowSel &g, const uint8_t *S, int k, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st)
{
    SrcStep src{S, k};
    return grow_step(g, src, shape, bc, pad, inlet_box, nullptr, err, st, g.ev ? g.off + k : nullptr);
}

// Step values (255 outside the volume) of the eight voxels of a block, byte
// (x * 2 + y) * 2 + z of the result.
__device__ __forceinline__ unsigned long long block_steps(const uint8_t *S, const BGrid &G, int c0, int c1, int c2)
{
    unsigned long long v = ~0ull;
#pragma unroll
    for (int x = 0; x < 2; x++)
#pragma unroll
        for (int y = 0; y < 2; y++) {
            const int i = 2 * c0 + x, j = 2 * c1 + y, k = 2 * c2;
            if (i >= G.s0 || j >= G.s1)
                continue;
            const long long a = ((long long)i * G.s1 + j) * G.s2 + k;
            unsigned pair;
            if (!(G.s2 & 1))
                pair = *(const uint16_t *)(S + a);
            else
                pair = S[a] | (k + 1 < G.s2 ? (unsigned)S[a + 1] << 8 : 0xff00u);
            const int sh = 8 * ((x * 2 + y) * 2);
            v = (v & ~(0xffffull << sh)) | ((unsigned long long)pair << sh);
        }
    return v;
}

// Distinct steps < nsteps among a block's eight voxels, packed in the low
// bytes of the result; their number in nd.
__device__ __forceinline__ unsigned long long distinct_steps(unsigned long long v, int nsteps, int &nd)
{
    unsigned long long d = 0;
    nd = 0;
#pragma unroll
    for (int e = 0; e < 8; e++) {
        const int x = (int)((v >> (8 * e)) & 0xffu);
        bool fresh = x < nsteps;
#pragma unroll
        for (int f = 0; f < e; f++)
            fresh = fresh && x != (int)((v >> (8 * f)) & 0xffu);
        if (fresh) {
            d |= (unsigned long long)x << (8 * nd);
            nd++;
        }
    }
    return d;
}

// Per-step counters live 32 ints apart (separate cache lines, separate L2
// slices).
constexpr int kStepStride = 32;

// Events (block, step) for every distinct step of a block: counted per step
// in shared memory, then added to the global counters once per CTA.
__global__ void k_step_count(const uint8_t *__restrict__ S, BGrid G, int nsteps, int *cnt)
{
    __shared__ int hist[256];
    for (int v = threadIdx.x; v < 256; v += blockDim.x)
        hist[v] = 0;
    __syncthreads();
    const int nb = G.b0 * G.b1 * G.b2;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int c0, c1, c2, nd;
        G.coords(b, c0, c1, c2);
        const unsigned long long d = distinct_steps(block_steps(S, G, c0, c1, c2), nsteps, nd);
        for (int e = 0; e < nd; e++)
            atomicAdd(&hist[(d >> (8 * e)) & 0xffu], 1);
    }
    __syncthreads();
    for (int v = threadIdx.x; v < nsteps; v += blockDim.x)
        if (hist[v])
            atomicAdd(cnt + v * kStepStride, hist[v]);
}

// The events written at per-step cursors: each round of blockDim.x blocks
// counts its events per step in shared memory, reserves one range per step
// with a single global atomic, then writes them.
__global__ void k_step_scatter(const uint8_t *__restrict__ S, BGrid G, int nsteps, int *cursor, int *__restrict__ ev)
{
    __shared__ int hist[256];
    __shared__ int sbase[256];
    for (int v = threadIdx.x; v < 256; v += blockDim.x)
        hist[v] = 0;
    __syncthreads();
    const int nb = G.b0 * G.b1 * G.b2;
    for (int base = blockIdx.x * blockDim.x; base < nb; base += gridDim.x * blockDim.x) {
        const int b = base + threadIdx.x;
        int nd = 0;
        unsigned long long d = 0;
        int loc[8];
        if (b < nb) {
            int c0, c1, c2;
            G.coords(b, c0, c1, c2);
            d = distinct_steps(block_steps(S, G, c0, c1, c2), nsteps, nd);
        }
#pragma unroll
        for (int e = 0; e < 8; e++)
            loc[e] = e < nd ? atomicAdd(&hist[(d >> (8 * e)) & 0xffu], 1) : 0;
        __syncthreads();
        for (int v = threadIdx.x; v < nsteps; v += blockDim.x) {
            sbase[v] = hist[v] ? atomicAdd(cursor + v * kStepStride, hist[v]) : 0;
            hist[v] = 0;
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < 8; e++)
            if (e < nd)
                ev[sbase[(d >> (8 * e)) & 0xffu] + loc[e]] = b;
    }
}

// Exclusive prefix of the per-step counts into the offsets (off[nsteps] =
// total), the cursors reset to the offsets; one thread block.
__global__ void k_step_offsets(int *cnt_cursor, int nsteps, int *off)
{
    if (threadIdx.x == 0) {
        int total = 0;
        for (int k = 0; k < nsteps; k++) {
            const int c = cnt_cursor[k * kStepStride];
            off[k] = total;
            cnt_cursor[k * kStepStride] = total;
            total += c;
        }
        off[nsteps] = total;
    }
}

int step_lists_build(GrowSel &g, const uint8_t *S, const int64_t *shape, int nsteps, void **mem, cudaStream_t st)
{
    *mem = nullptr;
    if (nsteps <= 0 || nsteps > 255) {
        set_error("step lists: %d steps outside [1, 255]", nsteps);
        return PMG_EINVAL;
    }
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    // a block has at most min(8, nsteps) distinct steps: the list is sized for
    // that, so nothing has to be read back before the scatter
    const size_t cap = (size_t)nb * (size_t)(nsteps < 8 ? nsteps : 8);
    const size_t tmpb = sizeof(int) * (size_t)kStepStride * 256;
    const size_t offb = ((size_t)(nsteps + 1) * sizeof(int) + 255) & ~(size_t)255;
    char *m = nullptr;
    PMG_TRY(scratch_alloc((void **)&m, tmpb + offb + sizeof(int) * cap, st));
    int *tmp = (int *)m;
    g.off = (int *)(m + tmpb);
    g.ev = (int *)(m + tmpb + offb);
    *mem = m;
    PMG_CUDA(cudaMemsetAsync(tmp, 0, tmpb, st));
    {
        const int ps__ = prof_begin("k_step_count", st);
        k_step_count<<<grid_for(nb, 256, 152LL * 8), 256, 0, st>>>(S, G, nsteps, tmp);
        prof_end(ps__, (double)nb * 8, st);
    }
    PMG_CHECK_LAUNCH();
    k_step_offsets<<<1, 32, 0, st>>>(tmp, nsteps, g.off);
    PMG_CHECK_LAUNCH();
    {
        const int ps__ = prof_begin("k_step_scatter", st);
        k_step_scatter<<<grid_for(nb, 256, 152LL * 8), 256, 0, st>>>(S, G, nsteps, tmp, g.ev);
        prof_end(ps__, (double)nb * 8, st);
    }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

int grow_marks_binary(GrowSel &g, const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st)
{
    SrcImg src{img, fgval};
    return grow_step(g, src, shape, bc, pad, inlet_box, nullptr, err, st);
}

// The two growing selections of a drainage radius, up to their inlet marks,
// in one union launch and one marks launch: the eroded space A (its step k
// from the precomputed lists when S is given, else from the capped EDT E > T)
// and the non-wetting phase B (fgval in img, or the list the last drainage
// update left).  Taken once both are past their first full build and no axis
// is periodic (no seam twins); otherwise the two steps run one after the
// other.  Same parents and marks either way: each set's unions only involve
// its own parents.
int grow_marks_pair(GrowSel &a, const uint8_t *S, int k, const uint16_t *E, int T, GrowSel &b, const uint8_t *img,
                    int fgval, const int64_t *shape, const int32_t *bc, const int32_t *pad, const int64_t *inlet_box,
                    int *err, cudaStream_t st)
{
    const bool step_lists = S && a.ev;
    if (!a.built || !b.built || any_periodic(bc) || (!S && !E)) {
        if (S)
            PMG_TRY(grow_marks_step(a, S, k, shape, bc, pad, inlet_box, err, st));
        else
            PMG_TRY(grow_marks_erode(a, E, T, shape, bc, pad, inlet_box, err, st));
        return grow_marks_binary(b, img, fgval, shape, bc, pad, inlet_box, err, st);
    }
    PMG_TRY(check_boxes(shape, inlet_box, nullptr));
    PMG_TRY(ensure_tables());
    PMG_TRY(ensure_block_tables());
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    const int *a_off = step_lists ? a.off + k : nullptr;
    // A's grown blocks
    if (step_lists) {
        const SrcStep src{S, k};
        const int ps__ = prof_begin("k_grow_apply", st);
        k_grow_apply<SrcStep><<<152 * 8, 256, 0, st>>>(src, a.M, a.P, G, a.ev, a_off, err,
                                                       prof_units(kUnitsGrowApply));
        prof_end_units(ps__, kUnitsGrowApply, 4 + 8 * sizeof(*src_elem(src)) + 2 + 4, st);
        PMG_CHECK_LAUNCH();
    } else if (S) {
        const SrcStep src{S, k};
        PMG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
        const int ps__ = prof_begin("k_grow_masks", st);
        k_grow_masks<SrcStep><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(src, a.M, a.P, G, a.list, a.count, err);
        prof_end(ps__, (double)n + (double)nb, st);
        PMG_CHECK_LAUNCH();
    } else {
        const SrcErode src = erode_src(E, T, shape, bc);
        PMG_CUDA(cudaMemsetAsync(a.count, 0, sizeof(int), st));
        const int ps__ = prof_begin("k_grow_masks", st);
        k_grow_masks<SrcErode><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(src, a.M, a.P, G, a.list, a.count,
                                                                            err);
        prof_end(ps__, (double)n * 2 + (double)nb, st);
        PMG_CHECK_LAUNCH();
    }
    // B's grown blocks: listed by the last update, or from its new masks
    if (b.pending) {
        b.pending = false;
    } else {
        const SrcImg src{img, fgval};
        PMG_CUDA(cudaMemsetAsync(b.count, 0, sizeof(int), st));
        const int ps__ = prof_begin("k_grow_masks", st);
        k_grow_masks<SrcImg><<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(src, b.M, b.P, G, b.list, b.count, err);
        prof_end(ps__, (double)n + (double)nb, st);
        PMG_CHECK_LAUNCH();
    }
    {
        const int ps__ = prof_begin("k_grow_unite[pair]", st);
        k_grow_unite2<<<152 * 32, 256, 0, st>>>(UniteList{a.P, a.M, step_lists ? a.ev : a.list, a.count, a_off},
                                                UniteList{b.P, b.M, b.list, b.count, nullptr}, G, err,
                                                prof_units(kUnitsGrowUnitePair));
        // per listed block: its list entry, mask and parent, and the masks and
        // parents of its 26 neighbours
        prof_end_units(ps__, kUnitsGrowUnitePair, 4 + 5 + 26 * 5, st);
        PMG_CHECK_LAUNCH();
    }
    // inlet marks of both
    PMG_CUDA(cudaMemsetAsync(a.mark, 0, ((size_t)nb + 3) & ~(size_t)3, st));
    PMG_CUDA(cudaMemsetAsync(b.mark, 0, ((size_t)nb + 3) & ~(size_t)3, st));
    if (inlet_box && inlet_box[0] >= 0) {
        Box bx;
        for (int d = 0; d < 3; d++) {
            bx.lo[d] = inlet_box[2 * d];
            bx.hi[d] = inlet_box[2 * d + 1];
        }
        if (bx.size() > 0) {
            long long nbk = 1;
            for (int d = 0; d < 3; d++)
                nbk *= ((bx.hi[d] + 1) >> 1) - (bx.lo[d] >> 1);
            const int ps__ = prof_begin("k_bcc_mark", st);
            k_bcc_mark2<<<dim3((unsigned)grid_for(nbk, 256, 1LL << 30), 2), 256, 0, st>>>(
                a.M, a.P, a.mark, b.M, b.P, b.mark, G, bx, (uint8_t)1, err);
            prof_end(ps__, (double)nbk * 18, st);
            PMG_CHECK_LAUNCH();
        }
    }
    return PMG_OK;
}

int grow_pair_select(GrowSel &a, GrowSel &b, const unsigned long long *b_count, uint8_t *out,
                     const int64_t *shape, int *err, cudaStream_t st, unsigned long long *kept, int *xr,
                     bool blocks)
{
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    const int ps__ = prof_begin("k_grow_pair_select", st);
    if (xr)
        PMG_CUDA(cudaMemsetAsync(xr, 0, 2 * sizeof(int), st));
    const unsigned grid = grid_for((nb + kPairBatch - 1) / kPairBatch, 256, 152LL * 64);
    if (blocks)
        k_grow_pair_select<true><<<grid, 256, 0, st>>>(a.M, a.P, a.mark, b.M, b.P, b.mark, b_count, G, out, kept,
                                                        err, xr);
    else
        k_grow_pair_select<false><<<grid, 256, 0, st>>>(a.M, a.P, a.mark, b.M, b.P, b.mark, b_count, G, out, kept,
                                                         err, xr);
    // masks 2 B, parents and marks of the nonempty blocks about 8 B per block
    prof_end(ps__, (blocks ? 0.0 : (double)n) + (double)nb * (blocks ? 11 : 10), st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

int select_grow_binary(GrowSel &g, const uint8_t *img, int fgval, void *out, const int64_t *shape,
                       const int32_t *bc, const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box,
                       int mode, int *err, cudaStream_t st, unsigned long long *kept)
{
    SrcImg src{img, fgval};
    return grow_select_core(g, src, out, shape, bc, pad, inlet_box, outlet_box, mode, fgval >= 0 ? fgval : 1, err,
                            st, kept);
}

int select_grow_erode(GrowSel &g, const uint16_t *E, int T, void *out, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode, int *err,
                      cudaStream_t st, unsigned long long *kept)
{
    return grow_select_core(g, erode_src(E, T, shape, bc), out, shape, bc, pad, inlet_box, outlet_box, mode, 1, err,
                            st, kept);
}

int bcc_marks_binary(const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc, const int32_t *pad,
                     const int64_t *inlet_box, const int64_t *outlet_box, int *P, uint8_t *M, uint8_t *mark,
                     int *err, cudaStream_t st)
{
    PMG_TRY(check_boxes(shape, inlet_box, outlet_box));
    SrcImg src{img, fgval};
    PMG_TRY(bcc_build(src, shape, bc, pad, true, P, M, err, st, false));
    return bcc_marks(shape, inlet_box, outlet_box, P, M, mark, err, st);
}

// ---- selection of a shrinking set, tile by tile ---------------------------------
// The wetting phase of a drainage curve only loses voxels; components can
// split, so its union-find is rebuilt every step, but the tile phase is local:
// a tile none of whose voxels changed gives the same tile-local parents as
// before, kept in Pl.  The producer of the changes (the drainage update)
// flags the tiles it touched and writes their new block masks.

size_t shrink_sel_bytes(const int64_t *shape)
{
    const BGrid G = bgrid_of(shape);
    const size_t nb = (size_t)G.b0 * G.b1 * G.b2;
    const size_t a = (nb + 255) & ~(size_t)255;
    const size_t nt = (size_t)((G.b0 + kT0 - 1) / kT0) * ((G.b1 + kT1 - 1) / kT1) * ((G.b2 + kT2 - 1) / kT2);
    // P, Pl, M, mark, per-tile flags, the cross-tile list (kBorder per tile + 64)
    return a * 4 * 2 + a * 2 + ((nt * 4 + 255) & ~(size_t)255) + (((nt * kBorder + 64) * 4 + 255) & ~(size_t)255) +
           256;
}

void shrink_sel_init(ShrinkSel &g, void *mem, const int64_t *shape)
{
    const BGrid G = bgrid_of(shape);
    const size_t nb = (size_t)G.b0 * G.b1 * G.b2;
    const size_t a = (nb + 255) & ~(size_t)255;
    const size_t nt = (size_t)((G.b0 + kT0 - 1) / kT0) * ((G.b1 + kT1 - 1) / kT1) * ((G.b2 + kT2 - 1) / kT2);
    char *p = (char *)mem;
    g.P = (int *)p;
    p += a * 4;
    g.Pl = (int *)p;
    p += a * 4;
    g.M = (uint8_t *)p;
    p += a;
    g.mark = (uint8_t *)p;
    p += a;
    g.dirty = (int *)p;
    p += (nt * 4 + 255) & ~(size_t)255;
    g.hard = (int *)p;
    g.ntiles = (int)nt;
    g.built = false;
}

int shrink_marks_binary(ShrinkSel &g, const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc,
                        const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int *err,
                        cudaStream_t st)
{
    PMG_TRY(check_boxes(shape, inlet_box, outlet_box));
    if (!g.built)
        PMG_CUDA(cudaMemsetAsync(g.dirty, 0, sizeof(int) * (size_t)g.ntiles, st));
    if (g.built) {
        // the producer of the changes kept the block masks current
        PMG_TRY(bcc_build(SrcMask{g.M}, shape, bc, pad, true, g.P, g.M, err, st, false, g.Pl, g.dirty, g.hard));
    } else {
        SrcImg src{img, fgval};
        PMG_TRY(bcc_build(src, shape, bc, pad, true, g.P, g.M, err, st, false, g.Pl, nullptr, g.hard));
    }
    g.built = true;
    return bcc_marks(shape, inlet_box, outlet_box, g.P, g.M, g.mark, err, st);
}

// ---- drainage update on blocks -------------------------------------------------
// mp = 1 where morph == 1 on a wetting voxel (2) connected to the outlet,
// reservoir slabs -> 1 (equilibrium_distribution.py:133-179,
// subdomain_padded.py:285-307), fused with the saturation counts (value 2
// inside the own box, multiphase.py:56-96; value 1 anywhere).  One thread per
// 2x2x2 block: the wetting phase's outlet connection comes from its block
// union-find (outlet mark bit 1), so no selected image is written.  With Mn,
// the block masks of the non-wetting phase (value 1) are brought up to date
// and grown blocks are listed for its next growing-selection step.

constexpr int kUpdateBatch = 2;

__global__ void __launch_bounds__(256, 5) k_drain_update_blocks(uint8_t *__restrict__ mp, const uint8_t *__restrict__ morph, int *Pw,
                                      uint8_t *__restrict__ Mw, const uint8_t *__restrict__ markw, BGrid G,
                                      Boxes B, uint8_t *__restrict__ Mn, int *__restrict__ Pn,
                                      int *__restrict__ list, int *count, unsigned long long *cnt2,
                                      unsigned long long *cnt1, int *err, int *__restrict__ wdirty,
                                      const int *__restrict__ orange, int ranged, unsigned long long *units)
{
    // orange: the x range [olo, ohi] (whole blocks) where the dilation result
    // is defined; outside it the dilation is empty.  ranged: only blocks that
    // can change are visited (the dilation range: the reservoir slabs were
    // refilled by an earlier update), and cnt2 / cnt1 receive the changes
    // (voxels leaving value 2 inside the own box, voxels newly 1) instead of
    // the totals.
    const int bxlo = orange ? orange[0] >> 1 : 0, bxhi = orange ? orange[1] >> 1 : G.b0 - 1;
    // a ranged update walks the dilation's block planes only
    const int plane = G.b1 * G.b2;
    const int bstart = ranged ? max(0, bxlo) * plane : 0;
    const int nb = G.b0 * G.b1 * G.b2;
    const int bend = ranged ? min(nb, max(0, bxhi + 1) * plane) : nb;
    if (units && blockIdx.x == 0 && threadIdx.x == 0 && bend > bstart)
        atomicAdd(units, (unsigned long long)(bend - bstart) * 8ull);
    const int lane = threadIdx.x & 31;
    unsigned int c2 = 0, c1 = 0;
    const bool pairs = !(G.s2 & 1);
    const long long sx = (long long)G.s1 * G.s2, sy = G.s2;
    // kUpdateBatch blocks per thread: every load of all of them is issued
    // before any of them is updated
    constexpr int NB = kUpdateBatch;
    for (int base = bstart + blockIdx.x * blockDim.x * NB; base < bend; base += gridDim.x * blockDim.x * NB) {
        int bq[NB];
        bool act[NB], ind[NB];
        unsigned vol[NB], wold[NB], oldn[NB], pv[NB][4], mv[NB][4];
        long long base0[NB];
#pragma unroll
        for (int q = 0; q < NB; q++) {
            const int b = base + q * blockDim.x + threadIdx.x;
            bq[q] = b;
            int c0, c1b, c2b;
            G.coords(b, c0, c1b, c2b);
            ind[q] = c0 >= bxlo && c0 <= bxhi;
            act[q] = b < bend && (ind[q] || !ranged);
            const int i0 = 2 * c0, j0 = 2 * c1b, k0 = 2 * c2b;
            vol[q] = act[q] ? spread_x(in2(i0, 0, G.s0)) & spread_y(in2(j0, 0, G.s1)) & spread_z(in2(k0, 0, G.s2)) : 0u;
            base0[q] = (long long)i0 * sx + (long long)j0 * sy + k0;
            wold[q] = act[q] ? Mw[b] : 0u;
            oldn[q] = act[q] && Mn ? Mn[b] : 0u;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                pv[q][t] = 0;
                mv[q][t] = 0;
                if ((vol[q] >> (2 * t)) & 3u) {
                    const long long a = base0[q] + (t >> 1) * sx + (t & 1) * sy;
                    if (pairs) {
                        pv[q][t] = *(const uint16_t *)(mp + a);
                        if (ind[q])
                            mv[q][t] = *(const uint16_t *)(morph + a);
                    } else {
                        pv[q][t] = mp[a];
                        if (ind[q])
                            mv[q][t] = morph[a];
                        if ((vol[q] >> (2 * t)) & 2u) {
                            pv[q][t] |= (unsigned)mp[a + 1] << 8;
                            if (ind[q])
                                mv[q][t] |= (unsigned)morph[a + 1] << 8;
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < NB; q++) {
            const int b = bq[q];
            bool changed = false;
            if (act[q]) {
                int c2b, c0, c1b;
                G.coords(b, c0, c1b, c2b);
                const int i0 = 2 * c0, j0 = 2 * c1b, k0 = 2 * c2b;
                // voxels inside the own box and the reservoir slabs
                const unsigned v = vol[q];
                const unsigned own = spread_x(in2(i0, B.own[0], B.own[1])) & spread_y(in2(j0, B.own[2], B.own[3])) &
                                     spread_z(in2(k0, B.own[4], B.own[5]));
                const unsigned res = (spread_x(~in2(i0, B.rpad[0], (long long)G.s0 - B.rpad[1]) & 3u) |
                                      spread_y(~in2(j0, B.rpad[2], (long long)G.s1 - B.rpad[3]) & 3u) |
                                      spread_z(~in2(k0, B.rpad[4], (long long)G.s2 - B.rpad[5]) & 3u)) &
                                     v;
                unsigned wet = wold[q];
                unsigned m1 = 0, is1 = 0, is2o = 0;
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    m1 |= eq2(mv[q][t], 1) << (2 * t);
                    is1 |= eq2(pv[q][t], 1) << (2 * t);
                    is2o |= eq2(pv[q][t], 2) << (2 * t);
                }
                // the wetting phase's outlet connection matters only where the
                // dilation meets it
                if (m1 & wet) {
                    const int rw = find_root(Pw, ld(Pw + b), err);
                    if (rw < 0 || !(markw[rw] & 2))
                        wet = 0;
                }
                // voxels set to 1: invaded wetting voxels and reservoir slabs
                const unsigned set1 = ((m1 & wet) | res) & v;
                unsigned is2 = 0;
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const unsigned bits = (set1 >> (2 * t)) & 3u;
                    unsigned p = pv[q][t];
                    if (bits) {
                        const unsigned bm = (bits & 1u ? 0x00ffu : 0u) | (bits & 2u ? 0xff00u : 0u);
                        p = (p & ~bm) | (0x0101u & bm);
                        const long long a = base0[q] + (t >> 1) * sx + (t & 1) * sy;
                        if (pairs) {
                            *(uint16_t *)(mp + a) = (uint16_t)p;
                        } else {
                            if (bits & 1u)
                                mp[a] = 1;
                            if (bits & 2u)
                                mp[a + 1] = 1;
                        }
                    }
                    is2 |= eq2(p, 2) << (2 * t);
                }
                const unsigned nwm = (is1 | set1) & v;
                if (wdirty && (is2 & v) != wold[q]) {
                    // the wetting phase changed here: its tile is recomputed next step
                    Mw[b] = (uint8_t)(is2 & v);
                    const int nt1 = (G.b1 + kT1 - 1) / kT1, nt2 = (G.b2 + kT2 - 1) / kT2;
                    const int tl = ((c0 / kT0) * nt1 + c1b / kT1) * nt2 + c2b / kT2;
                    if (!wdirty[tl])
                        wdirty[tl] = 1;
                }
                if (ranged) {
                    c2 += __popc(set1 & is2o & own & v);
                    c1 += __popc(set1 & ~is1 & v);
                } else {
                    c2 += __popc(is2 & own & v);
                    c1 += __popc(nwm);
                }
                if (Mn && nwm != oldn[q]) {
                    if (oldn[q] & ~nwm)
                        atomicExch(err, 3);
                    Mn[b] = (uint8_t)nwm;
                    if (!oldn[q])
                        Pn[b] = b;
                    changed = true;
                }
            }
            if (Mn) {
                const unsigned bal = __ballot_sync(0xffffffffu, changed);
                if (bal) {
                    int pos = 0;
                    if (lane == 0)
                        pos = atomicAdd(count, __popc(bal));
                    pos = __shfl_sync(0xffffffffu, pos, 0);
                    if (changed)
                        list[pos + __popc(bal & ((1u << lane) - 1u))] = b;
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        c2 += __shfl_down_sync(0xffffffffu, c2, o);
        c1 += __shfl_down_sync(0xffffffffu, c1, o);
    }
    if (lane == 0 && c2)
        atomicAdd(cnt2, (unsigned long long)c2);
    if (lane == 0 && c1)
        atomicAdd(cnt1, (unsigned long long)c1);
}

// Running totals (count(own == 2), count(== 1)) from the update's full counts
// or changes; the saturation numerator and the phase-1 count out.
__global__ void k_drain_totals(int ranged, const unsigned long long *cnt2, const unsigned long long *cnt1,
                               unsigned long long *tot, unsigned long long *sat_out, unsigned long long *ones_out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (ranged) {
            tot[0] -= *cnt2;
            tot[1] += *cnt1;
        } else {
            tot[0] = *cnt2;
            tot[1] = *cnt1;
        }
        *sat_out = tot[0];
        *ones_out = tot[1];
    }
}

int drain_totals(bool ranged, const unsigned long long *cnt2, const unsigned long long *cnt1, unsigned long long *tot,
                 unsigned long long *sat_out, unsigned long long *ones_out, cudaStream_t st)
{
    k_drain_totals<<<1, 32, 0, st>>>(ranged ? 1 : 0, cnt2, cnt1, tot, sat_out, ones_out);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

int drain_update_blocks(uint8_t *mp, const uint8_t *morph, const int64_t *shape, int *P, uint8_t *M,
                        const uint8_t *mark, const Boxes &B, GrowSel *g_nw, unsigned long long *cnt2_own,
                        unsigned long long *cnt1, int *err, cudaStream_t st, int *wdirty, const int *orange,
                        bool ranged)
{
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    const int ps__ = prof_begin("k_drain_update_blocks", st);
    k_drain_update_blocks<<<grid_for((nb + kUpdateBatch - 1) / kUpdateBatch, 256, 152LL * 64), 256, 0, st>>>(
        mp, morph, P, M, mark, G, B, g_nw ? g_nw->M : nullptr, g_nw ? g_nw->P : nullptr,
        g_nw ? g_nw->list : nullptr, g_nw ? g_nw->count : nullptr, cnt2_own, cnt1, err, wdirty, orange,
        ranged ? 1 : 0, prof_units(kUnitsDrainUpdate));
    // per voxel visited: multiphase read and written, dilation read
    prof_end_units(ps__, kUnitsDrainUpdate, 3.0, st);
    (void)n;
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

// ---- binary labelling on blocks -----------------------------------------------
// connect_components (connected_components.py:32-62; cc3d numbers components
// 1..N in the order of their first voxel in C order) for an image with a
// single nonzero value: the block union-find gives the components, and the
// first voxel of each one is found and ranked without a per-voxel parent
// array.  The first voxel of a block is its lowest set mask bit (bit order
// x, y, z follows C order); the first voxel of a component lies in the
// component's first block plane (the plane of its root, the smallest block
// index), so only blocks of that plane compete for it.

// smallest and largest nonzero value: 16 bytes per load where the image is
// 16-byte aligned (per-byte SIMD minima with zeros mapped to 255), bytes
// otherwise and for the tail
__global__ void k_nz_range(const uint8_t *__restrict__ img, long long n, unsigned *lohi)
{
    unsigned lo = 255, hi = 0;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x, nth = (long long)gridDim.x * blockDim.x;
    long long head = 0;
    if (!(reinterpret_cast<uintptr_t>(img) & 15)) {
        const long long nv = n >> 4;
        const uint4 *v4 = reinterpret_cast<const uint4 *>(img);
        unsigned lo4 = 0xFFFFFFFFu, hi4 = 0u;
        for (long long i = tid; i < nv; i += nth) {
            const uint4 w = __ldg(v4 + i);
            const unsigned ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                hi4 = __vmaxu4(hi4, ws[q]);
                lo4 = __vminu4(lo4, ws[q] | __vcmpeq4(ws[q], 0u));
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            lo = min(lo, (lo4 >> (8 * q)) & 0xFFu);
            hi = max(hi, (hi4 >> (8 * q)) & 0xFFu);
        }
        head = nv << 4;
    }
    for (long long i = head + tid; i < n; i += nth) {
        const unsigned v = img[i];
        if (v) {
            lo = min(lo, v);
            hi = max(hi, v);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_down_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(lohi, lo);
        atomicMax(lohi + 1, hi);
    }
}

__global__ void k_fill_i32(int *a, long long n, int v)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        a[i] = v;
}

__device__ __forceinline__ int block_first_voxel(const BGrid &G, int b, unsigned m)
{
    int c0, c1, c2;
    G.coords(b, c0, c1, c2);
    const int bit = __ffs(m) - 1;
    const int x = bit >> 2, y = (bit >> 1) & 1, z = bit & 1;
    return ((2 * c0 + x) * G.s1 + 2 * c1 + y) * G.s2 + 2 * c2 + z;
}

// F[root] = first voxel of the component
__global__ void k_blk_first(const int *__restrict__ P, const uint8_t *__restrict__ M, BGrid G, int *F)
{
    const int nb = G.b0 * G.b1 * G.b2;
    const int plane = G.b1 * G.b2;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        const unsigned m = M[b];
        if (!m)
            continue;
        const int r = P[b];
        if (r < 0 || b / plane != r / plane)
            continue;
        const int f = block_first_voxel(G, b, m);
        if (f < F[r])
            atomicMin(F + r, f);
    }
}

// bit f of `bits` set for every component's first voxel f
__global__ void k_blk_first_bits(const int *__restrict__ P, const uint8_t *__restrict__ M, const int *__restrict__ F,
                                 int nb, unsigned *bits)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        if (M[b] && P[b] == b) {
            const int f = F[b];
            atomicOr(bits + (f >> 5), 1u << (f & 31));
        }
}

// set bits per tile of 32 words (1024 voxels)
__global__ void k_bits_count(const unsigned *__restrict__ bits, long long nwords, int *cnt)
{
    const long long ntiles = (nwords + 31) / 32;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntiles;
         t += (long long)gridDim.x * blockDim.x) {
        int c = 0;
        const long long w1 = min(nwords, 32 * t + 32);
        for (long long w = 32 * t; w < w1; w++)
            c += __popc(bits[w]);
        cnt[t] = c;
    }
}

// root blocks: F[root] <- 1 + rank of its first voxel among all first voxels
__global__ void k_root_label(const int *__restrict__ P, const uint8_t *__restrict__ M, int *F, int nb,
                             const unsigned *__restrict__ bits, const int *__restrict__ offs)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        if (!M[b] || P[b] != b)
            continue;
        const int f = F[b];
        const int w = f >> 5;
        int r = offs[f >> 10] + __popc(bits[w] & ((1u << (f & 31)) - 1u));
        for (int u = (f >> 10) * 32; u < w; u++)
            r += __popc(bits[u]);
        F[b] = r + 1;
    }
}

// labels of every voxel: a block's label on its foreground voxels, 0 elsewhere
__global__ void k_blk_label_out(const int *__restrict__ P, const uint8_t *__restrict__ M, const int *__restrict__ F,
                                BGrid G, uint64_t *__restrict__ labels, const uint64_t *__restrict__ lut)
{
    const int nb = G.b0 * G.b1 * G.b2;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int c0, c1, c2;
        G.coords(b, c0, c1, c2);
        const unsigned m = M[b];
        uint64_t lab = m ? (uint64_t)F[P[b]] : 0;
        if (lut && lab)
            lab = lut[lab];
#pragma unroll
        for (int x = 0; x < 2; x++)
#pragma unroll
            for (int y = 0; y < 2; y++) {
                const int i = 2 * c0 + x, j = 2 * c1 + y;
                if (i >= G.s0 || j >= G.s1)
                    continue;
                uint64_t *row = labels + ((long long)i * G.s1 + j) * G.s2;
#pragma unroll
                for (int z = 0; z < 2; z++) {
                    const int k = 2 * c2 + z;
                    if (k < G.s2)
                        row[k] = ((m >> ((x * 2 + y) * 2 + z)) & 1u) ? lab : 0;
                }
            }
    }
}

// 1: the image holds one nonzero value (or none), so blocks can label it
static int single_value(const uint8_t *img, long long n, int *yes, cudaStream_t st)
{
    unsigned *lohi = nullptr;
    PMG_TRY(scratch_alloc((void **)&lohi, 2 * sizeof(unsigned), st));
    const unsigned init[2] = {255u, 0u};
    PMG_CUDA(cudaMemcpyAsync(lohi, init, sizeof(init), cudaMemcpyHostToDevice, st));
    {
        const int ps__ = prof_begin("k_nz_range", st);
        k_nz_range<<<grid_for(n, 256, 152LL * 16), 256, 0, st>>>(img, n, lohi);
        prof_end(ps__, (double)n, st);
    }
    PMG_CHECK_LAUNCH();
    unsigned h[2] = {0, 0};
    PMG_CUDA(cudaMemcpyAsync(h, lohi, sizeof(h), cudaMemcpyDeviceToHost, st));
    PMG_CUDA(cudaStreamSynchronize(st));
    PMG_TRY(scratch_free(lohi, st));
    *yes = h[1] == 0 || h[0] == h[1];
    return PMG_OK;
}

// ... or computed from the block union-find: a voxel's label is its block's
// root's number when the voxel is foreground.
struct LabBlk {
    const int *P;
    const uint8_t *M;
    const int *F;
    BGrid G;
    __device__ __forceinline__ uint64_t at(long long i, long long j, long long k) const
    {
        const int b = (int)(((i >> 1) * G.b1 + (j >> 1)) * G.b2 + (k >> 1));
        const int bit = (int)(((i & 1) * 2 + (j & 1)) * 2 + (k & 1));
        return ((M[b] >> bit) & 1u) ? (uint64_t)F[P[b]] : 0;
    }
};

int cc_label_blocks(const uint8_t *img, uint64_t *labels, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, int64_t *count, cudaStream_t st)
{
    const BGrid G = bgrid_of(shape);
    const int nb = G.b0 * G.b1 * G.b2;
    const long long n = shape[0] * shape[1] * shape[2];
    const long long nwords = (n + 31) / 32, ntiles = (nwords + 31) / 32;
    int *P = nullptr, *F = nullptr, *err = nullptr, *cnt = nullptr, *offs = nullptr;
    uint8_t *M = nullptr;
    unsigned *bits = nullptr;
    PMG_TRY(scratch_alloc((void **)&P, (size_t)nb * 4, st));
    PMG_TRY(scratch_alloc((void **)&F, (size_t)nb * 4, st));
    PMG_TRY(scratch_alloc((void **)&M, (size_t)nb, st));
    PMG_TRY(scratch_alloc((void **)&err, sizeof(int), st));
    PMG_TRY(scratch_alloc((void **)&bits, (size_t)nwords * 4, st));
    PMG_TRY(scratch_alloc((void **)&cnt, (size_t)ntiles * 4 + 4, st));
    PMG_TRY(scratch_alloc((void **)&offs, (size_t)ntiles * 4 + 4, st));
    PMG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    PMG_CUDA(cudaMemsetAsync(bits, 0, (size_t)nwords * 4, st));
    SrcImg src{img, -1};
    PMG_TRY(bcc_build(src, shape, bc, pad, false, P, M, err, st));
    {
        const int ps__ = prof_begin("k_blk_first", st);
        k_fill_i32<<<grid_for(nb, 256, 152LL * 32), 256, 0, st>>>(F, nb, INT_MAX);
        k_blk_first<<<grid_for(nb, 256, 152LL * 32), 256, 0, st>>>(P, M, G, F);
        k_blk_first_bits<<<grid_for(nb, 256, 152LL * 32), 256, 0, st>>>(P, M, F, nb, bits);
        k_bits_count<<<grid_for(ntiles, 256, 152LL * 32), 256, 0, st>>>(bits, nwords, cnt);
        prof_end(ps__, (double)nb * 13, st);
    }
    PMG_CHECK_LAUNCH();
    size_t tb = 0;
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt, offs, (int)ntiles + 1, st));
    void *tmp = nullptr;
    PMG_TRY(scratch_alloc(&tmp, tb, st));
    PMG_CUDA(cudaMemsetAsync(cnt + ntiles, 0, 4, st));
    PMG_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, cnt, offs, (int)ntiles + 1, st));
    k_root_label<<<grid_for(nb, 256, 152LL * 32), 256, 0, st>>>(P, M, F, nb, bits, offs);
    PMG_CHECK_LAUNCH();
    int total = 0;
    PMG_CUDA(cudaMemcpyAsync(&total, offs + ntiles, sizeof(int), cudaMemcpyDeviceToHost, st));
    int s = read_err(err, st);
    // periodic seams: the relabelling table is built from the blocks' labels
    // on the seam slabs and folded into the one pass that writes the labels
    uint64_t *lut = nullptr;
    int64_t merged = total;
    if (s == PMG_OK && any_periodic(bc))
        s = periodic_renumber(LabBlk{P, M, F, G}, labels, shape, bc, pad, total, &merged, st, &lut);
    if (s == PMG_OK) {
        const int ps__ = prof_begin("k_blk_label_out", st);
        k_blk_label_out<<<grid_for(nb, 256, 152LL * 64), 256, 0, st>>>(P, M, F, G, labels, lut);
        prof_end(ps__, (double)n * 8 + (double)nb * 9, st);
        s = cudaGetLastError() == cudaSuccess ? PMG_OK : PMG_ECUDA;
    }
    if (lut)
        PMG_TRY(scratch_free(lut, st));
    PMG_TRY(scratch_free(tmp, st));
    PMG_TRY(scratch_free(P, st));
    PMG_TRY(scratch_free(F, st));
    PMG_TRY(scratch_free(M, st));
    PMG_TRY(scratch_free(err, st));
    PMG_TRY(scratch_free(bits, st));
    PMG_TRY(scratch_free(cnt, st));
    PMG_TRY(scratch_free(offs, st));
    if (s != PMG_OK)
        return s;
    *count = merged;
    return PMG_OK;
}

int cc_label_u8(const uint8_t *img, uint64_t *labels, const int64_t *shape, const int32_t *bc, const int32_t *pad,
                int64_t *count, cudaStream_t st)
{
    const long long n = shape[0] * shape[1] * shape[2];
    int yes = 0;
    PMG_TRY(single_value(img, n, &yes, st));
    if (yes)
        return cc_label_blocks(img, labels, shape, bc, pad, count, st);
    return cc_label_t(img, labels, shape, bc, pad, count, st);
}

// Selection with caller-provided scratch: P (n int32), mark (n bytes rounded
// up to 4), err (one int, zeroed by the caller).  Does not synchronize.
int select_run(const uint8_t *img, void *out, int out_bytes, const int64_t *shape,
               const int32_t *bc, const int32_t *pad, const int64_t *inlet_box,
               const int64_t *outlet_box, int mode, int phase, int *P, uint8_t *mark, int *err,
               cudaStream_t st)
{
    const long long n = shape[0] * shape[1] * shape[2];
    PMG_CUDA(cudaMemsetAsync(mark, 0, ((size_t)n + 3) & ~(size_t)3, st));
    PMG_TRY(uf_build<uint8_t>(img, P, shape, bc, pad, true, err, st));
    Vol3 V{shape[0], shape[1], shape[2]};
    const int64_t *boxes[2] = {inlet_box, outlet_box};
    for (int w = 0; w < 2; w++) {
        const int64_t *bx = boxes[w];
        if (!bx || bx[0] < 0)
            continue;
        Box b;
        for (int d = 0; d < 3; d++) {
            b.lo[d] = bx[2 * d];
            b.hi[d] = bx[2 * d + 1];
            if (b.lo[d] < 0 || b.hi[d] > shape[d] || b.lo[d] > b.hi[d]) {
                set_error("connected-image selection: face box outside the volume");
                return PMG_EINVAL;
            }
        }
        if (b.size() > 0) {
            {
                const int ps__ = prof_begin("k_mark_face", st);
                k_mark_face<<<grid_for(b.size(), 256, 1LL << 30), 256, 0, st>>>(P, V, b, mark,
                                                                              (uint8_t)(1 << w));
                prof_end(ps__, (double)b.size() * 4, st);
            }
            PMG_CHECK_LAUNCH();
        }
    }
    if (out_bytes == 1)
        {
            const int ps__ = prof_begin("k_select", st);
            k_select<uint8_t><<<grid_for(n, 256, 1LL << 30), 256, 0, st>>>(img, P, mark, n, mode, phase,
                                                                        (uint8_t *)out);
            prof_end(ps__, (double)n * (5 + out_bytes), st);
        }
    else
        {
            const int ps__ = prof_begin("k_select", st);
            k_select<uint64_t><<<grid_for(n, 256, 1LL << 30), 256, 0, st>>>(img, P, mark, n, mode, phase,
                                                                         (uint64_t *)out);
            prof_end(ps__, (double)n * (5 + out_bytes), st);
        }
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}

int check_err(int *err, cudaStream_t st) { return read_err(err, st); }

int check_volume(const int64_t *shape) { return check_vol(shape); }

} // namespace pmg

extern "C" int pmg_cc_select(const uint8_t *img, void *out, int32_t out_bytes,
                             const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                             const int64_t inlet_box[6], const int64_t outlet_box[6], int32_t mode,
                             int32_t phase, void *stream)
{
    if (!img || !out || !shape || !bc || !pad) {
        set_error("pmg_cc_select: null argument");
        return PMG_EINVAL;
    }
    if (out_bytes != 1 && out_bytes != 8) {
        set_error("pmg_cc_select: output element size must be 1 or 8");
        return PMG_EINVAL;
    }
    const bool binary = (mode & PMG_SEL_BINARY) != 0;
    mode &= ~PMG_SEL_BINARY;
    if (mode < PMG_SEL_INLET || mode > PMG_SEL_ISOLATED) {
        set_error("pmg_cc_select: unknown mode %d", mode);
        return PMG_EINVAL;
    }
    PMG_TRY(check_geometry(shape, bc, pad));
    PMG_TRY(check_vol(shape));
    cudaStream_t st = as_stream(stream);
    const long long n = shape[0] * shape[1] * shape[2];
    int *P = nullptr, *err = nullptr;
    uint8_t *mark = nullptr;
    int s;
    if (phase >= 0 || binary) {
        const long long nb = ((shape[0] + 1) / 2) * ((shape[1] + 1) / 2) * ((shape[2] + 1) / 2);
        const size_t mb = ((size_t)nb + 255) & ~(size_t)255;
        PMG_TRY(scratch_alloc((void **)&P, (size_t)nb * 4, st));
        PMG_TRY(scratch_alloc((void **)&mark, 2 * mb, st));
        PMG_TRY(scratch_alloc((void **)&err, sizeof(int), st));
        PMG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        s = select_run_binary(img, out, out_bytes, shape, bc, pad, inlet_box, outlet_box, mode, phase >= 0 ? phase : -1,
                              P, mark, mark + mb, err, st, nullptr);
    } else {
        PMG_TRY(scratch_alloc((void **)&P, (size_t)n * 4, st));
        PMG_TRY(scratch_alloc((void **)&mark, ((size_t)n + 3) & ~(size_t)3, st));
        PMG_TRY(scratch_alloc((void **)&err, sizeof(int), st));
        PMG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        s = select_run(img, out, out_bytes, shape, bc, pad, inlet_box, outlet_box, mode, phase, P, mark, err, st);
    }
    if (s == PMG_OK)
        s = read_err(err, st);
    PMG_TRY(scratch_free(P, st));
    PMG_TRY(scratch_free(mark, st));
    PMG_TRY(scratch_free(err, st));
    return s;
}

// Testing aid: lower every union-find iteration cap (c_uf_cap) to `cap`
// (<= 0 restores the default bounds).
extern "C" int pmg_set_iteration_cap(int32_t cap)
{
    const int v = cap > 0 ? cap : INT_MAX;
    PMG_CUDA(cudaMemcpyToSymbol(c_uf_cap, &v, sizeof(int)));
    return PMG_OK;
}
