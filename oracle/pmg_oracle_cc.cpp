/*
 * ORACLE -- test infrastructure only (connected components).
 *
 * PMMoTo labels with the third-party package connected_components_3d
 * ("cc3d", pyproject.toml:24, >=3.12.4), called at
 * src/pmmoto/filters/connected_components.py:52-54 with its defaults:
 * 26-connectivity, every nonzero value labelled separately, background 0,
 * uint64 output.  cc3d is not vendored with PMMoTo and is not installed
 * here.  This file restates its published behaviour: components are the
 * 26-connected sets of equal nonzero values, numbered 1..N in the order in
 * which their first voxel appears in a C-order raster scan (cc3d's
 * provisional labels are issued in scan order and then renumbered
 * consecutively).  The numbering is therefore an assumption ("parity
 * unpinned" for label numbers); partitions and counts are pinned by the
 * reference's own tests.
 *
 * or_unique_pairs restates unique_pairs (src/pmmoto/core/_voxels.hpp:106-125)
 * with the same container, so that its iteration order is the one the
 * reference sees on the same C++ standard library.
 */
#include <cstdint>
#include <cstring>
#include <unordered_set>
#include <vector>

namespace {

struct dsu {
    std::vector<int64_t> p;
    explicit dsu(int64_t n) : p((size_t)n)
    {
        for (int64_t i = 0; i < n; i++)
            p[(size_t)i] = i;
    }
    int64_t find(int64_t x)
    {
        while (p[(size_t)x] != x) {
            p[(size_t)x] = p[(size_t)p[(size_t)x]];
            x = p[(size_t)x];
        }
        return x;
    }
    void unite(int64_t a, int64_t b)
    {
        a = find(a);
        b = find(b);
        if (a == b)
            return;
        if (a < b)
            p[(size_t)b] = a;
        else
            p[(size_t)a] = b;
    }
};

template <typename T>
int64_t label_impl(const T *img, uint64_t *labels, const int64_t *shape)
{
    const int64_t n0 = shape[0], n1 = shape[1], n2 = shape[2];
    const int64_t total = n0 * n1 * n2;
    dsu d(total);
    for (int64_t i = 0; i < n0; i++)
        for (int64_t j = 0; j < n1; j++)
            for (int64_t k = 0; k < n2; k++) {
                int64_t idx = (i * n1 + j) * n2 + k;
                T v = img[idx];
                if (v == 0)
                    continue;
                for (int di = -1; di <= 0; di++)
                    for (int dj = -1; dj <= 1; dj++)
                        for (int dk = -1; dk <= 1; dk++) {
                            if (di == 0 && (dj > 0 || (dj == 0 && dk >= 0)))
                                continue;
                            int64_t a = i + di, b = j + dj, c = k + dk;
                            if (a < 0 || b < 0 || c < 0 || b >= n1 || c >= n2)
                                continue;
                            int64_t nidx = (a * n1 + b) * n2 + c;
                            if (img[nidx] == v)
                                d.unite(idx, nidx);
                        }
            }
    std::vector<uint64_t> id((size_t)total, 0);
    int64_t next = 0;
    for (int64_t idx = 0; idx < total; idx++) {
        if (img[idx] == 0) {
            labels[idx] = 0;
            continue;
        }
        int64_t r = d.find(idx);
        if (id[(size_t)r] == 0)
            id[(size_t)r] = (uint64_t)(++next);
        labels[idx] = id[(size_t)r];
    }
    return next;
}

} // namespace

extern "C" {

/* dtype: 1 = uint8, 4 = int32/uint32, 8 = int64/uint64 (value equality only) */
int64_t or_cc_label(const void *img, int dtype_bytes, uint64_t *labels,
                    const int64_t *shape)
{
    switch (dtype_bytes) {
    case 1:
        return label_impl((const uint8_t *)img, labels, shape);
    case 2:
        return label_impl((const uint16_t *)img, labels, shape);
    case 4:
        return label_impl((const uint32_t *)img, labels, shape);
    case 8:
        return label_impl((const uint64_t *)img, labels, shape);
    default:
        return -1;
    }
}

/* unique_pairs, _voxels.hpp:106-125.  out must hold 2*nrows values;
   returns the number of unique pairs written, in container iteration order. */
int64_t or_unique_pairs(const uint64_t *data, int64_t nrows, uint64_t *out)
{
    std::unordered_set<unsigned long> unique_set;
    for (int64_t i = 0; i < nrows; ++i) {
        unsigned long encoded =
            ((unsigned long)data[2 * i] << 32) | (unsigned long)data[2 * i + 1];
        unique_set.insert(encoded);
    }
    int64_t m = 0;
    for (unsigned long encoded : unique_set) {
        out[2 * m] = encoded >> 32;
        out[2 * m + 1] = encoded & 0xFFFFFFFFul;
        m++;
    }
    return m;
}

} // extern "C"
