// Lock-free union-find shared by the labelling and selection kernels.
//
// Parents live in an int32 array; a root points to itself; unions link the
// larger root under the smaller with atomicMin (Playne and Hawick's
// lock-free scheme), so every component's root is its smallest index.  All
// searches and unions stop after a bounded number of steps and record an
// error code instead of spinning.
#pragma once

#include <climits>

#include "pmg_common.cuh"

namespace pmg {

// Iteration caps.  Parents always point to smaller indices, so a root
// search from x legitimately takes at most x steps, and every retry of a
// union lowers the larger of its two roots, so a union retries at most
// max(a, b) + 1 times: the caps below are those bounds (a loop that exceeds
// one has met a corrupted parent array, e.g. a cycle).  A loop also gives up
// as soon as another thread has recorded an error (checked every
// kErrPoll steps).  c_uf_cap (constant memory, default INT_MAX) lowers every
// cap further -- a testing aid (pmg_set_iteration_cap) that makes the caps
// run out on ordinary inputs.
// (Defined here: only cc.cu includes this header, so there is one copy.)
static __constant__ int c_uf_cap = INT_MAX;
constexpr int kErrPoll = 256;

__device__ __forceinline__ int ld(const int *p) { return __ldcg(p); }

__device__ __forceinline__ bool uf_gave_up(int it, const int *err)
{
    return (it & (kErrPoll - 1)) == 0 && *(volatile const int *)err != 0;
}

__device__ __forceinline__ int find_root(const int *P, int x, int *err)
{
    const int cap = min(x + 1, c_uf_cap);
    int p = ld(P + x);
    int it = 0;
    while (p != x) {
        x = p;
        p = ld(P + x);
        if (++it > cap) {
            atomicExch(err, 1);
            break;
        }
        if (uf_gave_up(it, err))
            break;
    }
    return x;
}

// Root search with path halving: each visited element is re-pointed to its
// grandparent.  Parents only ever point to smaller indices and an element's
// ancestors stay its ancestors, so a plain store of an ancestor never breaks a
// link; a store that overwrites a concurrent atomicMin on a former root is
// harmless because that union retries with the value the atomic returned.
__device__ __forceinline__ int find_root_halve(int *P, int x, int *err)
{
    const int cap = min(x + 1, c_uf_cap);
    int p = ld(P + x);
    int it = 0;
    while (p != x) {
        const int g = ld(P + p);
        if (g == p)
            return p;
        P[x] = g;
        x = g;
        p = ld(P + x);
        if (++it > cap) {
            atomicExch(err, 1);
            break;
        }
        if (uf_gave_up(it, err))
            break;
    }
    return x;
}

// Playne-Hawick union (atomicMin links the larger root under the smaller).
__device__ __forceinline__ void unite(int *P, int a, int b, int *err)
{
    const int cap = min(max(a, b) + 1, c_uf_cap);
    for (int it = 0; it < cap; it++) {
        a = find_root_halve(P, a, err);
        b = find_root_halve(P, b, err);
        if (a == b)
            return;
        if (a < b) {
            int old = atomicMin(P + b, a);
            if (old == b)
                return;
            b = old;
        } else {
            int old = atomicMin(P + a, b);
            if (old == a)
                return;
            a = old;
        }
    }
    atomicExch(err, 2);
}

// Seam twins: every halo voxel of a periodic feature is united with the own
// voxel it copies, when both are foreground (the reference pairs labels
// without comparing values, skipping zeros).
struct Twins {
    long long s0, s1, s2;
    int periodic[3];
    int own_lo[3], own_len[3];
};

struct Box {
    long long lo[3], hi[3];
    __host__ __device__ long long size() const
    {
        return (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    }
};

inline Twins make_twins(const int64_t *shape, const int32_t *bc, const int32_t *pad)
{
    Twins W;
    W.s0 = shape[0];
    W.s1 = shape[1];
    W.s2 = shape[2];
    for (int d = 0; d < 3; d++) {
        W.periodic[d] = bc[2 * d] == PMG_BC_PERIODIC;
        W.own_lo[d] = pad[2 * d];
        W.own_len[d] = (int)(shape[d] - pad[2 * d] - pad[2 * d + 1]);
    }
    return W;
}

inline bool any_periodic(const int32_t *bc)
{
    return bc[0] == PMG_BC_PERIODIC || bc[2] == PMG_BC_PERIODIC || bc[4] == PMG_BC_PERIODIC;
}

} // namespace pmg
