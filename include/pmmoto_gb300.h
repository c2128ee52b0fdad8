/*
 * pmmoto_gb300 -- C ABI of the GB300 voxel-morphology library.
 *
 * Conventions
 *   - Arrays are C-ordered 3-D volumes (shape[0], shape[1], shape[2]);
 *     2-D images use shape {1, n0, n1}.
 *   - Array arguments are CUDA device pointers owned by the caller unless a
 *     parameter is documented as a host pointer.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Work is
 *     enqueued on it; functions that return host scalars synchronize it.
 *   - Every function returns PMG_OK (0), a positive input error, or a
 *     negative device error; pmg_last_error() describes the last failure on
 *     the calling thread.  No exception crosses the ABI.
 *
 * Each entry point names the reference routine (PMMoTo v1.0.7, paths
 * relative to its source tree) whose result it reproduces bit for bit.
 */
#ifndef PMMOTO_GB300_H
#define PMMOTO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PMG_OK 0
#define PMG_EINVAL 1   /* bad shape, pointer or parameter */
#define PMG_ERANGE 2   /* size beyond a documented limit */
#define PMG_ECUDA (-1) /* CUDA runtime error */
#define PMG_EITER (-2) /* a bounded device loop hit its iteration cap */

/* Boundary kinds of one face (core/boundary_types.py:11-17). */
#define PMG_BC_END 0
#define PMG_BC_WALL 1
#define PMG_BC_PERIODIC 2

/* Largest line length the envelope kernels accept. */
#define PMG_MAX_LINE 8192

/*
 * Per-axis rules for importing periodic information into one EDT pass.
 *   periodic      the axis wraps
 *   Axis of the linear pass (correctors):
 *     F = first zero voxel in [f_lo, n), L = last zero voxel in
 *     [l_lo, n - l_hi); upper corrector = F + a_u, lower corrector =
 *     n - L + a_l (infinite when no zero exists).
 *   Axes of the envelope passes (boundary hulls):
 *     the near-end hull segment search skips hf_lo voxels at the low end,
 *     the far-end search skips hb_hi voxels at the high end.
 * edt3d / edt2d use {p, 0, 0, 0, 1, 0, 0, 0}; the padded-subdomain EDT with
 * pads (lo, hi) uses {p, 2lo, 2lo, 2hi, -lo, -hi-1, 2lo, 2hi}
 * (filters/distance/euclidean_distance_transform.py:56-101, 306-528).
 */
typedef struct pmg_axis_cfg {
    int32_t periodic, f_lo, l_lo, l_hi, a_u, a_l, hf_lo, hb_hi;
} pmg_axis_cfg;

/* Output forms of the EDT entry points. */
#define PMG_EDT_SQUARED 0 /* float32 squared distance */
#define PMG_EDT_DIST 1    /* float32 sqrt of it (np.sqrt on float32) */
#define PMG_EDT_MORPH 2   /* internal: fused threshold of the morphology ops */

/*
 * Squared/plain Euclidean distance transform of a uint8 volume: zeros are
 * the "solid" voxels, distinct nonzero values restart the linear pass.
 * Pass order and arithmetic follow edt3d (euclidean_distance_transform.py:
 * 208-303) with `cfg` as above; replaces the Python/Cython driver loops
 * _distance.pyx:86-127, 308-353, 544-618 and the kernels
 * squared_edt_1d / squared_edt_1d_parabolic / return_boundary_hull
 * (_distance.hpp:135-356).  num_hull is the reference's hull count (4).
 */
int pmg_edt3d(const uint8_t *img, float *out, const int64_t shape[3],
              const float res[3], const pmg_axis_cfg cfg[3], int32_t num_hull,
              int32_t form, void *stream);

/*
 * pmg_edt3d without any device allocation.  No counterpart in the reference:
 * it is an addition for callers that cannot let a library allocate device
 * memory -- a host framework that owns all device memory through its own
 * pool or budget, or a latency-critical loop where a pool allocation could
 * block or fail mid-run.  Same arguments and results as pmg_edt3d; the
 * intermediate volume lives in a fixed 64 MiB array and the per-line flags
 * and deferred voxels of the envelope passes in a fixed 4 MiB array (a line
 * whose deferred voxels find the array full takes the float envelope
 * instead: same results, slower), both reserved by the
 * library on every device that loads it (held until the process exits), so
 * volumes are limited to 16,777,216 voxels (256^3); larger ones return
 * PMG_ERANGE with a message.  The first call on a device looks up that
 * device's array addresses, so make the first call before any stream
 * capture; calls after a cudaDeviceReset of that device are not supported.
 * All calls share the arrays: calls that overlap on the GPU (concurrent
 * streams, threads) race and must be serialized by the caller.
 */
int pmg_edt3d_noalloc(const uint8_t *img, float *out, const int64_t shape[3],
                      const float res[3], const pmg_axis_cfg cfg[3], int32_t num_hull,
                      int32_t form, void *stream);

/*
 * edt2d (euclidean_distance_transform.py:104-205): linear pass along axis 1,
 * envelope along axis 0.  img/out hold shape2[0]*shape2[1] values.
 */
int pmg_edt2d(const uint8_t *img, float *out, const int64_t shape2[2],
              const float res[2], const int32_t periodic[2], int32_t num_hull,
              int32_t form, void *stream);

/*
 * Morphological addition (dilate != 0) or subtraction of a padded
 * single-rank subdomain image by the EDT path: addition / subtraction
 * (filters/morphological_operators.py:103-228) with the halo extension of
 * update_extended_buffer (core/communication.py:121-157).
 *   bc[2d], bc[2d+1]   boundary kind of the low / high face of axis d
 *   pad[2d], pad[2d+1] padding of the subdomain on those faces
 *   ext[2d], ext[2d+1] extension of those faces (ceil(r/res) on periodic
 *                      faces; ignored elsewhere)
 *   res                voxel size, float32 as the reference passes it
 *   radius, cmp64      compare sqrt(d2) <= radius in float64 when cmp64 is
 *                      1 (a numpy float64 radius) or in float32 when 0 (a
 *                      Python float radius, numpy's weak-scalar rule)
 *   ball_sq            < 0 for the EDT path above.  >= 0 selects the FFT
 *                      path of the reference (fft=True): scipy fftconvolve
 *                      with the structuring element {i^2+j^2+k^2 <= R2},
 *                      R2 = (radius/res)^2 in float64 (gen_struct_element,
 *                      :66-100), thresholded; that equals comparing the
 *                      integer squared voxel-unit distance with
 *                      ball_sq = floor(R2), which is what is done.
 * img and out have the padded shape; out gets 0/1 with wall planes 0.
 */
int pmg_morph(const uint8_t *img, uint8_t *out, const int64_t shape[3],
              const int32_t bc[6], const int32_t pad[6], const int32_t ext[6],
              const float res[3], double radius, int32_t cmp64, int32_t dilate,
              double ball_sq, void *stream);

/*
 * Connected components of a padded single-rank subdomain image (elements of
 * elem_bytes = 1, 2, 4 or 8 bytes, compared by value): 26-connectivity, every
 * nonzero value labelled separately, background 0 -- the call of
 * connect_components (filters/connected_components.py:32-62) to the
 * third-party cc3d, numbered 1..N in order of first voxel in C-order scan --
 * followed, when an axis is periodic, by the reference's seam merge and
 * renumbering (connect_subdomain_boundaries :65-101, core/voxels.py:167-397,
 * core/_voxels.pyx:335-383, 548-579).  labels: uint64, padded shape.
 * *count (host) receives the label count the reference returns.
 */
int pmg_cc_label(const void *img, int32_t elem_bytes, uint64_t *labels,
                 const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                 int64_t *count, void *stream);

/* Selection modes of pmg_cc_select. */
#define PMG_SEL_INLET 1    /* inlet_connected_img  (connected_components.py:254-296) */
#define PMG_SEL_OUTLET 2   /* outlet_connected_img (:299-341) */
#define PMG_SEL_BOTH 3     /* inlet_outlet_connected_img (:203-251) */
#define PMG_SEL_ISOLATED 4 /* isolated_img (:344-392) */
#define PMG_SEL_BINARY 16  /* flag: the image holds only 0 and 1 (phase < 0 case) */

/*
 * Keep the voxels of `img` (uint8, padded shape) whose component (periodic
 * seams merged) touches the inlet and/or outlet face slab, as `mode` says;
 * phase >= 0 keeps only voxels of that value.  out receives the kept value
 * or 0, as uint8 (out_bytes 1) or uint64 (8).  inlet_box / outlet_box are
 * {lo0, hi0, lo1, hi1, lo2, hi2} own-slab boxes of the face flagged inlet /
 * outlet (the last such face in face order, core/voxels.py:400-454), or NULL
 * / lo0 < 0 when the subdomain has none.  With phase >= 0, or with
 * PMG_SEL_BINARY or-ed into mode for an image of 0s and 1s, the selection
 * runs on 2x2x2 blocks (one value is in play, and all its voxels in a block
 * are mutually 26-adjacent); results are the same.
 */
int pmg_cc_select(const uint8_t *img, void *out, int32_t out_bytes,
                  const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                  const int64_t inlet_box[6], const int64_t outlet_box[6],
                  int32_t mode, int32_t phase, void *stream);

/*
 * Sphere voxelisation of a padded grid (gen_sphere_img_brute_force,
 * domain_generation/domain_generation.hpp:91-127, with Sphere::contains,
 * particles/spheres.hpp:41-48): img = 1, then 0 where a voxel centre lies in
 * any sphere, tested in float64 as (dx*dx + dy*dy + dz*dz) <= r*r.
 * spheres: nsph rows of (x, y, z, r) float64 (device); cx/cy/cz: voxel-centre
 * coordinates of the three axes (device, the subdomain's linspace coords);
 * grid_c0 / grid_h (host): first centre and spacing per axis, used only to
 * bound the voxels each sphere can reach.
 */
int pmg_spheres(const double *spheres, int64_t nsph, const double *cx,
                const double *cy, const double *cz, const double grid_c0[3],
                const double grid_h[3], uint8_t *img, const int64_t shape[3],
                void *stream);

/*
 * update_buffer on one rank (core/communication.py:101-118): halo voxels of
 * periodic axes take the value of the own voxel they copy; wall planes are
 * set to 0.  elem_bytes 1 (uint8), 4 (float32) or 8 (uint64), in place.
 */
int pmg_update_buffer(void *img, int32_t elem_bytes, const int64_t shape[3],
                      const int32_t bc[6], const int32_t pad[6], void *stream);

/* Number of uint8 voxels equal to `value` in box {lo0,hi0,lo1,hi1,lo2,hi2}
   (np.count_nonzero(img == value) of that region); *count is a host pointer. */
int pmg_count_eq(const uint8_t *img, const int64_t shape[3], const int64_t box[6],
                 int32_t value, int64_t *count, void *stream);

/* Maximum of a float32 volume over a box (np.amax); *out is a host pointer. */
int pmg_max_f32(const float *x, const int64_t shape[3], const int64_t box[6],
                float *out, void *stream);

/*
 * porosimetry (filters/porosimetry.py:84-160) with mode="distance": erode
 * pm_img by r_erode, keep the inlet-connected part when `inlet`, and if any
 * voxel is left, constrain by the inlet-connected phase 1 of mp_img (when
 * mp_img is not NULL and holds phase 1) and dilate by r_dilate.  ratio_* are
 * ceil(radius/res) per axis (gen_struct_ratio); cmp_* and ball_* as in
 * pmg_morph (ball_* >= 0 selects the reference's FFT erosion / dilation:
 * mode "morph" uses both, mode "hybrid" only ball_dilate).
 */
int pmg_porosimetry(const uint8_t *pm_img, const uint8_t *mp_img, uint8_t *out,
                    const int64_t shape[3], const int32_t bc[6], const int32_t pad[6],
                    const int64_t inlet_box[6], const float res[3], double r_erode,
                    int32_t cmp_erode, const int32_t ratio_erode[3], double r_dilate,
                    int32_t cmp_dilate, const int32_t ratio_dilate[3], int32_t inlet,
                    double ball_erode, double ball_dilate, void *stream);

/*
 * drainage, standard method (filters/equilibrium_distribution.py:25-179)
 * with mode="distance", on the device.  For each of n_radii probe radii
 * (float64, host array, in capillary-pressure order): when active[k] the
 * porosimetry step above with the inlet and multiphase constraints, else an
 * empty morph; then the outlet-connected phase 2 of mp_img, the update
 * mp = (morph == 1 && connected == 2) ? 1 : mp, the reservoir refill
 * (rpad slabs set to 1) and counts[k] (host) = number of own voxels (own_box)
 * equal to 2 -- the numerator of Multiphase.get_saturation.  mp_img (device)
 * is updated in place; ratios holds ceil(r/res) per axis per radius;
 * ball_erode / ball_dilate (host arrays or NULL) select the FFT-mode ball per
 * radius as in pmg_porosimetry.
 */
int pmg_drainage(const uint8_t *pm_img, uint8_t *mp_img, const int64_t shape[3],
                 const int32_t bc[6], const int32_t pad[6], const int32_t rpad[6],
                 const int64_t own_box[6], const int64_t inlet_box[6],
                 const int64_t outlet_box[6], const float res[3], int32_t n_radii,
                 const double *radii, const int32_t *active, const int32_t *ratios,
                 const double *ball_erode, const double *ball_dilate, int64_t *counts,
                 void *stream);

/*
 * pmg_drainage with dilation radii that differ from the erosion radii: the
 * extended contact-angle method (equilibrium_distribution.py:230-289,
 * dilation radius = erosion radius * |cos(theta)|).  radii_dilate (host,
 * float64) and ratios_dilate (ceil(r/res) per axis per radius) may be NULL,
 * which gives pmg_drainage.  The contact_angle method (:182-228) is
 * pmg_drainage with its own probe radii.
 */
int pmg_drainage_ext(const uint8_t *pm_img, uint8_t *mp_img, const int64_t shape[3],
                     const int32_t bc[6], const int32_t pad[6], const int32_t rpad[6],
                     const int64_t own_box[6], const int64_t inlet_box[6],
                     const int64_t outlet_box[6], const float res[3], int32_t n_radii,
                     const double *radii, const int32_t *active, const int32_t *ratios,
                     const double *ball_erode, const double *ball_dilate, int64_t *counts,
                     const double *radii_dilate, const int32_t *ratios_dilate, void *stream);

/*
 * Learned radius schedule: kernels of the 3-D CNN that predicts a drainage
 * curve (no counterpart in the reference, whose drainage loop,
 * filters/equilibrium_distribution.py:93-128, evaluates every radius).
 * Activations are bf16, channels last ([batch][z][y][x][c]); convolutions
 * are 3x3x3 with stride 2 and padding 1 from a cubic side di to
 * (di + 1) / 2, computed on the tensor cores (tcgen05, fp32 accumulate);
 * c_in is 1, 16, 32 or 64 and c_out 16, 32 or 64.  Weights are fp32
 * [c_out][c_in][27] (tap = (kz * 3 + ky) * 3 + kx); pmg_cnn_pack_weights
 * writes their bf16 operands: wk [c_out][kp], kp = 27 c_in rounded up to 64,
 * and (c_in >= 16) wkt [c_in][kpt], kpt = 27 c_out rounded up to 64.
 * err: a device int that a pipeline wait which runs out of time sets (read
 * by pmg_cnn_check, which returns PMG_EITER then).
 */
int pmg_cnn_pack_weights(const float *w, int32_t cin, int32_t cout, void *wk, void *wkt, void *stream);
/* y = ReLU(conv(x, w) + bias), bf16. */
int pmg_cnn_conv_fwd(const void *x, const void *wk, const float *bias, void *y, int32_t batch, int32_t di,
                     int32_t cin, int32_t cout, int32_t *err, void *stream);
/* dx = conv_transpose(dz, w) masked where xact (the layer input, a ReLU
   output) is 0: the gradient of the lower layer's pre-activation, bf16. */
int pmg_cnn_conv_dgrad(const void *dz, const void *wkt, const void *xact, void *dx, int32_t batch, int32_t di,
                       int32_t cin, int32_t cout, int32_t *err, void *stream);
/* grad [c_out][c_in][27] and dbias [c_out] (fp32) of the loss given dz;
   dw is fp32 scratch of 27 c_in c_out values. */
int pmg_cnn_conv_wgrad(const void *x, const void *dz, float *dw, float *grad, float *dbias, int32_t batch,
                       int32_t di, int32_t cin, int32_t cout, int32_t *err, void *stream);
/* Head on y4 [batch][64][64]: average pool, MLP 64-64 (ReLU) -64, sigmoid ->
   pred [batch][64].  params: w5 [64][64], b5, w6 [64][64], b6 (fp32).  With a
   target: *loss += mean squared error, grads (same layout) += gradients,
   dy4 = gradient of y4's pre-activation. */
int pmg_cnn_head(const void *y4, const float *params, int32_t batch, const float *target, float *pred,
                 float *loss, float *grads, void *dy4, void *stream);
/* One bias-corrected Adam step (step >= 1) over n fp32 parameters. */
int pmg_cnn_adam(float *w, const float *g, float *m, float *v, int64_t n, double lr, double b1, double b2,
                 double eps, int64_t step, double weight_decay, void *stream);
/* Network input: the float32 distance field's box {lo0,hi0,lo1,hi1,lo2,hi2}
   (at least 64 voxels per axis) averaged over 64^3 cells, divided by scale,
   as bf16 [64][64][64]. */
int pmg_cnn_downsample(const float *dist, const int64_t shape[3], const int64_t box[6], double scale, void *out,
                       void *stream);
/* PMG_EITER (and a message) if a kernel above recorded a timed-out wait. */
int pmg_cnn_check(int32_t *err, void *stream);

/*
 * Workload generator (no counterpart in the reference): one periodic
 * smoothing pass along `axis` of `batch` float64 volumes of `shape`
 * (in != out) with the (order + 1) weights w (host array, order <= 256):
 * out[i] = w_0 in[i - order/2] + ... + w_order in[i + order/2], summed in
 * that order with each product and sum rounded once.  The Gaussian random
 * field media of the large EDT + CC configuration and of the schedule
 * network's training set apply it with the binomial weights C(order, k) / 2^order.
 */
int pmg_grf_smooth(const double *in, double *out, int64_t batch, const int64_t shape[3], int32_t axis,
                   const double *weights, int32_t order, void *stream);

/* Number of kernels this library has launched in the process. */
long long pmg_launch_count(void);

/*
 * Number of scratch allocations this library has requested in the process
 * (stream-ordered, from a memory pool the library owns on each device; the
 * device's default pool is not touched).  A diagnostic with no counterpart
 * in the reference: it lets a caller check that an entry point allocated
 * nothing.
 */
long long pmg_scratch_alloc_count(void);

/*
 * Per-kernel timing: when enabled, every launch records a CUDA event pair on
 * its stream with the launch's algorithmic bytes.  pmg_prof_read resolves
 * them (synchronizing on the events) into per-kernel totals: `names` gets
 * newline-separated kernel names, ms / bytes / launches the totals, *count
 * the number of kernels (at most cap).  pmg_prof_reset clears the totals.
 */
int pmg_prof_enable(int32_t on);
int pmg_prof_reset(void);
int pmg_prof_read(char *names, size_t names_len, double *ms, double *bytes,
                  long long *launches, int32_t cap, int32_t *count);

/*
 * Testing aid with no counterpart in the reference: every data-dependent
 * device loop of the union-find (root searches, union retries) is bounded by
 * the longest chain a valid parent array allows and returns PMG_EITER, with
 * the CUDA context intact, when a loop runs past it.  This call lowers all
 * those bounds to `cap` iterations (cap <= 0 restores the defaults) on the
 * current device, so that a test can make a bound run out on an ordinary
 * input.  Not for production use: results of calls that return PMG_EITER
 * are undefined.
 */
int pmg_set_iteration_cap(int32_t cap);

/*
 * Tunable launch parameters (no counterpart in the reference): results never
 * depend on them, only speed.  Names: "edt.pair_seg" (positions per thread
 * of the strided line-pair envelope pass, default 256), "edt.pair_ctas" and
 * "edt.rows_ctas" (CTAs per SM of the strided and contiguous line-pair
 * passes, defaults 32 and 16), "cc.cross_fused" (block labelling's
 * cross-tile phase as one fused pass, 1, or as a classification pass and a
 * union pass, 0; default 0), "edt.path" (envelope passes with power-of-two
 * voxels: windowed with the probed fallback, 0, the exact integer stream, 1,
 * or the float envelope, 2; default 0), "edt.fallback" and
 * "edt.fallback_rows" (probe samples, of 8192, that the +-12 window does not
 * finish, from which a strided or a contiguous windowed pass hands the whole
 * pass to the float envelope; 0 always, 8193 never; defaults 96 and 2048),
 * "edt.narrow" and "edt.narrow_rows" (probe samples the +-8 window does not
 * finish, below which the pass runs the +-8 window instead of the +-12 one;
 * 0 never; defaults 64 and 32), "edt.wide" (probe samples the +-24 window
 * does not finish, below which a strided pass of at least 131,072 lines that
 * the +-12 window would hand to the float envelope runs the +-24 window;
 * 0 never, 8193 always and for any line count; default 1024),
 * "cc.seam_batched" (periodic merge: the
 * seams of all periodic features deduplicated in one sort, 1, or one
 * feature at a time, 0; default 1; one at a time is also taken when labels
 * need more than 29 bits).  A negative value restores the default, and so
 * does 0 for the knobs whose smallest value is 1; values are process-wide
 * and apply to launches that follow.  pmmoto_gb300.tune sets them from its
 * cached measurements.
 */
int pmg_tune_set(const char *name, int32_t value);
int pmg_tune_get(const char *name, int32_t *value);

/* Message of the last failure on this host thread (empty if none). */
int pmg_last_error(char *buf, size_t len);

/* Library version and build information. */
const char *pmg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PMMOTO_GB300_H */
