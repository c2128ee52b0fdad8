// Internal entry points shared between translation units (not part of the C ABI).
#pragma once

#include "pmg_common.cuh"

namespace pmg {

// blk (dilation): the seeds as per-block masks (bit (x * 2 + y) * 2 + z over
// the ceil-halved shape); img is then scratch of one byte per voxel, written
// only on the paths that need the seeds as bytes.
int morph_run(const uint8_t *img, uint8_t *out, const int64_t *shape, const int32_t *bc,
              const int32_t *pad, const int32_t *ext, const float *res, double radius, int cmp64,
              int dilate, uint8_t *E, float *A, float *B, cudaStream_t st, double thr_sq = -1.0,
              const unsigned long long *gate = nullptr, const int *xr = nullptr, int *orange = nullptr,
              const uint8_t *blk = nullptr);
size_t morph_scratch_bytes(const int64_t *shape, const int32_t *bc, const int32_t *ext);
int erosion_edt_run(const uint8_t *img, float *D, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, const float *res, int unit_res, uint8_t *E, float *A,
                    cudaStream_t st);
int erosion_cap_run(const uint8_t *img, uint16_t *KC, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, int Tcap, uint8_t *E, uint16_t *KA, uint16_t *KB, int *flag,
                    int *nonbinary, cudaStream_t st);

int select_run(const uint8_t *img, void *out, int out_bytes, const int64_t *shape,
               const int32_t *bc, const int32_t *pad, const int64_t *inlet_box,
               const int64_t *outlet_box, int mode, int phase, int *P, uint8_t *mark, int *err,
               cudaStream_t st);
int select_run_binary(const uint8_t *img, void *out, int out_bytes, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode,
                      int fgval, int *P, uint8_t *M, uint8_t *mark, int *err, cudaStream_t st,
                      unsigned long long *kept = nullptr);
int select_run_erode(const uint16_t *E, int T, void *out, const int64_t *shape, const int32_t *bc,
                     const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode, int *P,
                     uint8_t *M, uint8_t *mark, int *err, cudaStream_t st, unsigned long long *kept = nullptr);

// Boxes of a drainage run: own voxels, inlet / outlet faces (lo0, hi0, lo1,
// hi1, lo2, hi2; lo0 < 0 for none), reservoir widths per face.
struct Boxes {
    int64_t own[6];
    int64_t inlet[6], outlet[6];
    int32_t rpad[6];
};

// Selection of a set that only grows from one call to the next (same shape,
// boundaries and boxes): the block union-find is kept and only blocks whose
// mask grew are united again.  Scratch of grow_sel_bytes(shape) bytes.
struct GrowSel {
    int *P = nullptr;
    uint8_t *M = nullptr;
    uint8_t *mark = nullptr;
    int *list = nullptr;
    int *count = nullptr;
    bool built = false;
    // masks already brought up to date and grown blocks listed by the producer
    // of the set (the drainage update); the next step skips its mask pass
    bool pending = false;
    // blocks that grow at each step, known in advance (step_lists_build):
    // step k's blocks are ev[off[k] .. off[k + 1])
    int *ev = nullptr;
    int *off = nullptr;
    // profiler label of the union step, and its unit counter (-1: none)
    const char *unite_label = "k_grow_unite";
    int unite_units = -1;
};
// Per-step lists of the blocks of a step volume S (steps < nsteps; 255:
// never) that grow at that step, in one allocation *mem (freed by the caller).
int step_lists_build(GrowSel &g, const uint8_t *S, const int64_t *shape, int nsteps, void **mem, cudaStream_t st);
size_t grow_sel_bytes(const int64_t *shape);
void grow_sel_init(GrowSel &g, void *mem, const int64_t *shape);
int select_grow_binary(GrowSel &g, const uint8_t *img, int fgval, void *out, const int64_t *shape,
                       const int32_t *bc, const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box,
                       int mode, int *err, cudaStream_t st, unsigned long long *kept = nullptr);
int select_grow_erode(GrowSel &g, const uint16_t *E, int T, void *out, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int mode, int *err,
                      cudaStream_t st, unsigned long long *kept = nullptr);
// The step of a growing selection up to the inlet marks (no output) ...
int grow_marks_erode(GrowSel &g, const uint16_t *E, int T, const int64_t *shape, const int32_t *bc,
                     const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st);
int grow_marks_binary(GrowSel &g, const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st);
// (the set: voxels with step S <= k)
int grow_marks_step(GrowSel &g, const uint8_t *S, int k, const int64_t *shape, const int32_t *bc,
                    const int32_t *pad, const int64_t *inlet_box, int *err, cudaStream_t st);
// Both growing selections of a drainage radius up to their inlet marks (the
// eroded space a: step k of S when S is given, else E > T; the non-wetting
// phase b: fgval in img) in one union launch and one marks launch, once both
// are built and no axis is periodic; the two steps above otherwise.
int grow_marks_pair(GrowSel &a, const uint8_t *S, int k, const uint16_t *E, int T, GrowSel &b, const uint8_t *img,
                    int fgval, const int64_t *shape, const int32_t *bc, const int32_t *pad, const int64_t *inlet_box,
                    int *err, cudaStream_t st);
// ... and the inlet selection of a constrained by b (when *b_count > 0) in one
// pass; kept counts a's inlet-connected voxels.
// xr (optional): the x range of the output's set (kRangeBig encoding);
// blocks: out holds one mask per 2x2x2 block (bit (x * 2 + y) * 2 + z)
int grow_pair_select(GrowSel &a, GrowSel &b, const unsigned long long *b_count, uint8_t *out,
                     const int64_t *shape, int *err, cudaStream_t st, unsigned long long *kept, int *xr = nullptr,
                     bool blocks = false);
// Selection of a set that only shrinks (the drainage's wetting phase): full
// block union-find every step, but tiles the producer did not flag reuse
// their tile-local parents Pl.  Scratch of shrink_sel_bytes(shape) bytes.
struct ShrinkSel {
    int *P = nullptr;
    int *Pl = nullptr;
    uint8_t *M = nullptr;
    uint8_t *mark = nullptr;
    int *dirty = nullptr; // per tile: changed since the last step
    int *hard = nullptr;  // the cross-tile union list (kBorder per tile + 64 ints)
    int ntiles = 0;
    bool built = false;
};
size_t shrink_sel_bytes(const int64_t *shape);
void shrink_sel_init(ShrinkSel &g, void *mem, const int64_t *shape);
int shrink_marks_binary(ShrinkSel &g, const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc,
                        const int32_t *pad, const int64_t *inlet_box, const int64_t *outlet_box, int *err,
                        cudaStream_t st);
// Block union-find of the voxels equal to fgval with inlet / outlet marks,
// without a selected image (parents left unflattened).
int bcc_marks_binary(const uint8_t *img, int fgval, const int64_t *shape, const int32_t *bc, const int32_t *pad,
                     const int64_t *inlet_box, const int64_t *outlet_box, int *P, uint8_t *M, uint8_t *mark,
                     int *err, cudaStream_t st);
// The drainage update on blocks, reading the wetting phase's outlet
// connection from its block union-find (P, M, mark from bcc_marks_binary with
// the outlet box); maintains g_nw's masks when given.
// With wdirty, M (the wetting phase's masks) is brought up to date and the
// tiles whose masks changed are flagged.  orange (device, voxel x range
// [lo, hi] in whole blocks, null: everything): the only blocks that can
// change; ranged: the counts are changes since the last update rather than
// totals (drain_totals keeps the running totals).
int drain_update_blocks(uint8_t *mp, const uint8_t *morph, const int64_t *shape, int *P, uint8_t *M,
                        const uint8_t *mark, const Boxes &B, GrowSel *g_nw, unsigned long long *cnt2_own,
                        unsigned long long *cnt1, int *err, cudaStream_t st, int *wdirty = nullptr,
                        const int *orange = nullptr, bool ranged = false);
int drain_totals(bool ranged, const unsigned long long *cnt2, const unsigned long long *cnt1, unsigned long long *tot,
                 unsigned long long *sat_out, unsigned long long *ones_out, cudaStream_t st);
int check_err(int *err, cudaStream_t st);
int check_volume(const int64_t *shape);

int update_buffer_run(void *img, int elem_bytes, const int64_t *shape, const int32_t *bc,
                      const int32_t *pad, cudaStream_t st);
int count_eq_async(const uint8_t *img, const int64_t *shape, const int64_t *box, uint8_t value,
                   unsigned long long *d_cnt, cudaStream_t st);

} // namespace pmg
