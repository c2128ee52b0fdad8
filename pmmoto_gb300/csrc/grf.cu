// Periodic binomial smoothing of Gaussian-random-field media (a workload
// generator with no counterpart in the reference: the large EDT + CC
// configuration and the schedule network's training media).  One pass
// convolves every line along one axis with the (order + 1)-tap binomial
// kernel w_k = C(order, k) / 2^order, periodic, as
//     acc = w_0 x[i - h];  acc = acc + w_k x[i + k - h]  (k = 1..order)
// with every product and sum rounded once (__dmul_rn / __dadd_rn), the same
// operations in the same order as the host generator and the tensor
// formulation, so all three give the same bytes.
#include "pmg_common.cuh"

namespace pmg {

constexpr int kGrfMaxOrder = 256;

struct GrfTaps {
    double w[kGrfMaxOrder + 1];
};

__global__ void k_grf_smooth(const double *__restrict__ in, double *__restrict__ out, long long total, long long n0,
                             long long n1, long long n2, int axis, GrfTaps taps, int order)
{
    const int h = order / 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long k2 = e % n2;
        const long long r = e / n2;
        const long long k1 = r % n1;
        const long long r2 = r / n1;
        const long long k0 = r2 % n0;
        long long n, stride, pos;
        if (axis == 2) {
            n = n2, stride = 1, pos = k2;
        } else if (axis == 1) {
            n = n1, stride = n2, pos = k1;
        } else {
            n = n0, stride = n1 * n2, pos = k0;
        }
        const double *line = in + (e - pos * stride);
        long long j = pos - h;
        j %= n;
        if (j < 0)
            j += n;
        double acc = __dmul_rn(taps.w[0], line[j * stride]);
        for (int k = 1; k <= order; k++) {
            if (++j == n)
                j = 0;
            acc = __dadd_rn(acc, __dmul_rn(taps.w[k], line[j * stride]));
        }
        out[e] = acc;
    }
}

} // namespace pmg

using namespace pmg;

extern "C" int pmg_grf_smooth(const double *in, double *out, int64_t batch, const int64_t shape[3], int32_t axis,
                              const double *weights, int32_t order, void *stream)
{
    if (!in || !out || !shape || !weights || batch <= 0 || axis < 0 || axis > 2 || order < 0 ||
        order > kGrfMaxOrder || in == out) {
        set_error("pmg_grf_smooth: bad argument");
        return PMG_EINVAL;
    }
    for (int d = 0; d < 3; d++)
        if (shape[d] <= 0) {
            set_error("pmg_grf_smooth: shape[%d] must be positive", d);
            return PMG_EINVAL;
        }
    GrfTaps taps;
    for (int k = 0; k <= order; k++)
        taps.w[k] = weights[k];
    const long long total = batch * shape[0] * shape[1] * shape[2];
    cudaStream_t st = as_stream(stream);
    const int ps__ = prof_begin("k_grf_smooth", st);
    k_grf_smooth<<<grid_for(total, 256, 152LL * 16), 256, 0, st>>>(in, out, total, shape[0], shape[1], shape[2], axis,
                                                                    taps, order);
    prof_end(ps__, (double)total * 16, st);
    PMG_CHECK_LAUNCH();
    return PMG_OK;
}
