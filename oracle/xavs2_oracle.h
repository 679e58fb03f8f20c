/*
 * xavs2_oracle.h -- CPU restatement of the xavs2 encoder hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GPU library is
 * checked against: a plain-C restatement of the reference algorithms (SAD,
 * SATD, SA8D, SSD, block ops, AVS2 luma/chroma interpolation, integer DCT
 * with the 64-point wavelet, secondary transforms, quant/dequant, and the
 * full-search + sub-pel motion search), written from the reference's
 * behaviour with one citation per function.  Only tests/, the smoke check
 * and bench.py's CPU-baseline leg may call it; the product path never does.
 *
 * Parity pin: oracle/_ref (the reference's own C primitives compiled from
 * their source files by oracle/Makefile) is compared with this restatement on
 * seeded and adversarial inputs, and the golden fixtures under tests/golden/
 * were produced by that reference build.
 *
 * All pixel types follow the reference (8-bit build): pel = uint8_t,
 * coeff = int16_t, dist = int32_t.
 */
#ifndef XAVS2_ORACLE_H
#define XAVS2_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* LumaPU shape index order (pixel.h:50-65). */
int  xo_num_parts(void);
int  xo_part_width(int part);
int  xo_part_height(int part);
int  xo_part_index(int w, int h);          /* -1 if (w,h) is not a PU shape */

/* ---- block cost / block ops (pixel.c) --------------------------------- */
int32_t xo_sad (int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);
int32_t xo_satd(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);
int32_t xo_sa8d(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);
int32_t xo_ssd (int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);
void xo_sad_x3(int part, const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,
               const uint8_t *r2, intptr_t i_ref, int32_t res[3]);
void xo_sad_x4(int part, const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,
               const uint8_t *r2, const uint8_t *r3, intptr_t i_ref, int32_t res[4]);
void xo_avg(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *a, intptr_t i_a,
            const uint8_t *b, intptr_t i_b);
void xo_sub_ps(int part, int16_t *dst, intptr_t i_dst, const uint8_t *a, const uint8_t *b,
               intptr_t i_a, intptr_t i_b);
void xo_add_ps(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *a, const int16_t *b,
               intptr_t i_a, intptr_t i_b);
void xo_copy_pp(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *src, intptr_t i_src);
void xo_copy_ps(int part, int16_t *dst, intptr_t i_dst, const uint8_t *src, intptr_t i_src);
void xo_copy_sp(int part, uint8_t *dst, intptr_t i_dst, const int16_t *src, intptr_t i_src);
void xo_copy_ss(int part, int16_t *dst, intptr_t i_dst, const int16_t *src, intptr_t i_src);
int32_t xo_ssd_block(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2, int w, int h);
void xo_average(uint8_t *dst, int i_dst, const uint8_t *a, int i_a, const uint8_t *b, int i_b,
                int w, int h);
int  xo_mad(const uint8_t *src, int i_src, int cu_size);

/* ---- interpolation (mc.c) --------------------------------------------- */
const int8_t *xo_luma_filter(int frac);    /* frac 0..3 */
const int8_t *xo_chroma_filter(int frac);  /* frac 0..7 */
void xo_intpl_luma_hor(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, const uint8_t *src,
                       int i_src, int w, int h, const int8_t *coef);
void xo_intpl_luma_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w, int h,
                       const int8_t *coef);
void xo_intpl_luma_ext(uint8_t *dst, int i_dst, const int16_t *tmp, int i_tmp, int w, int h,
                       const int8_t *coef);
void xo_intpl_luma_block_hor(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef);
void xo_intpl_luma_block_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef);
void xo_intpl_luma_block_ext(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef_x, const int8_t *coef_y);
void xo_intpl_chroma_block_hor(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef);
void xo_intpl_chroma_block_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef);
void xo_intpl_chroma_block_ext(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef_x, const int8_t *coef_y);
/* Frame-level sub-pel planes.  `planes[k]` (k = 4*dy + dx, 1..15) point at
 * pixel (0,0) of padded planes with stride `stride` and `pad` valid pixels
 * on every side; `src` likewise (its padding must already hold the clamped
 * border).  mode 1 fills planes 2, 8, 10 only (half-pel ME), mode 2 all 15.
 * Planes not filled may be NULL. */
void xo_interpolate_frame(uint8_t *const planes[16], const uint8_t *src, int stride,
                          int width, int height, int pad, int mode);
/* Replicate-border padding of a plane in place (frame.c plane_expand_border
 * with both bands on). */
void xo_expand_border(uint8_t *pix, int stride, int width, int height, int pad);

/* ---- transform / quant (transform.c, quant.c) ------------------------- */
/* `tu` is a LumaPU index of one of the 11 TU shapes. */
int  xo_is_tu_shape(int part);
void xo_dct (int part, const int16_t *src, int16_t *dst, int i_src);
void xo_idct(int part, const int16_t *src, int16_t *dst, int i_dst);
void xo_dct_half(int part, const int16_t *src, int16_t *dst, int i_src);
void xo_transform_4x4_2nd(int16_t *coef, int i_coef);
void xo_inv_transform_4x4_2nd(int16_t *coef, int i_coef);
void xo_transform_2nd(int16_t *coef, int i_coef, int i_mode, int b_top, int b_left);
void xo_inv_transform_2nd(int16_t *coef, int i_coef, int i_mode, int b_top, int b_left);
int  xo_quant(int16_t *coef, int n, int scale, int shift, int add);
int  xo_wquant(int16_t *coef, int n, int scale, int shift, int add, const int *levelscale);
void xo_dequant(int16_t *coef, int n, int scale, int shift);
void xo_abs_coeff(int16_t *dst, const int16_t *src, int n);
int  xo_add_sign(int16_t *dst, const int16_t *abs_val, int n);
int  xo_q_scale(int qp);                   /* tab_Q_TAB[qp] */
int  xo_iq_scale(int qp);                  /* tab_IQ_TAB[qp] */
int  xo_iq_shift(int qp);                  /* tab_IQ_SHIFT[qp] */
int  xo_quant_fwd_add(int shift, int b_intra);
/* One TU through dct -> quant -> (dequant -> idct when nnz > 0), the way
 * rdo.c:1333-1370 chains them.  `blk` holds the residual (w x h, stride w)
 * on entry; `coef_out` gets the quantised levels (w_tr x h_tr) and `blk` the
 * reconstructed residual.  Returns nnz. */
int  xo_tq_chain(int part, int16_t *blk, int16_t *coef_out, int qp, int b_intra, int use_2nd);

/* Batch descriptor (same layout as the GPU library's xavs2gpu_tq_block_t). */
typedef struct xo_tq_block {
    int64_t offset, coef_offset;
    int32_t part, qp, flags, pad_;
} xo_tq_block_t;
void xo_tq_batch(const xo_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef, int16_t *recon,
                 int32_t *nnz, int threads);

/* ---- motion search (me.c) --------------------------------------------- */
typedef struct xo_me_params {
    int32_t search_range;     /* full search over [-R, R) in both axes   */
    int32_t lambda_factor;    /* i_lambda_factor (16.16 sqrt(lambda))    */
    int32_t use_hadamard;     /* fpel_cmp: 1 = SATD, 0 = SAD             */
    int32_t fractional_me;    /* 0 none, 1 half-pel, 2 half + quarter    */
    int32_t fast_sub_me;      /* Spiral2 pattern with step 2             */
    int32_t enable_pmvr;
} xo_me_params_t;

typedef struct xo_pu {
    int16_t x, y;             /* luma position of the PU                 */
    uint8_t part, ref;        /* LumaPU index, reference index           */
    int16_t mvp_x, mvp_y;     /* predictor, quarter-pel                  */
    int16_t min_x, min_y;     /* integer-pel search limits (inclusive)   */
    int16_t max_x, max_y;
} xo_pu_t;

typedef struct xo_me_result {
    int16_t bmv_x, bmv_y;     /* final MV, quarter-pel                   */
    int32_t bcost;            /* final cost                              */
    int32_t mvcost;           /* MV cost of bmv                          */
    int16_t imv_x, imv_y;     /* integer-pel best MV                     */
    int32_t icost;            /* integer-pel best cost                   */
} xo_me_result_t;

int  xo_mvbits(int d);
/* Search one PU against one reference.  `fenc` points at the PU's top-left
 * pixel; `fref[k]` are the 16 sub-pel planes of the reference (k = 0 the
 * full-pel plane) all pointing at pixel (0,0) with stride `i_fref`. */
int32_t xo_me_search(const xo_me_params_t *prm, const xo_pu_t *pu, const uint8_t *fenc,
                     intptr_t i_fenc, const uint8_t *const fref[16], intptr_t i_fref,
                     xo_me_result_t *out);
/* Searches every PU of a list (threads > 1 uses OpenMP when available). */
void xo_me_search_list(const xo_me_params_t *prm, const xo_pu_t *pus, int n_pus,
                       const uint8_t *fenc, intptr_t i_fenc,
                       const uint8_t *const *frefs /* [n_refs][16] */, intptr_t i_fref,
                       xo_me_result_t *out, int threads);
/* MV search limits from md_inter.c:910-926 (m = 6 margin, 64-pixel pad). */
void xo_pu_set_limits(xo_pu_t *pu, int width, int height, int vmin_qpel, int vmax_qpel);

#ifdef __cplusplus
}
#endif


/* ---- intra prediction (intra.c) and rough mode decision (md_intra.c) ---- */
/* Prediction of a bsx x bsy block in mode 0..32 from the edge samples
 * around ep (ep[0] top-left, ep[1..] top / top-right, ep[-1..] left /
 * left-down); dc_avail = (top available << 8) | left available. */
void xo_intra_pred(int mode, const uint8_t *ep, uint8_t *dst, int i_dst, int dc_avail, int bsx, int bsy);
/* The edge samples of a bsx x bsy block at (x0, y0) of a picture, as
 * fill_reference_samples builds them (intra.c:1580-1860) when its neighbour
 * samples are the picture's: avail bits 0 left, 1 top, 2 left-down, 3
 * top-right, 4 top-left (MD_I_*); ep is the top-left edge sample. */
void xo_intra_fill_edge(const uint8_t *pic, int stride, int x0, int y0, int bsx, int bsy, int avail, uint8_t *ep);
/* A batch of xo_intra_fill_edge over one picture (job layout of
 * xavs2gpu_intra_edge_job_t): the window -(h + 11w/4 + 6) .. w + 11h/4 + 6
 * around each edge_offset, beyond the reference's padding repeating the
 * run's last sample; sides outside the picture count as missing; jobs with
 * an invalid shape or window outside [0, edges_size) are skipped. */
typedef struct {
    int64_t edge_offset;
    int32_t x, y;
    int16_t width, height;
    int32_t avail;
} xo_intra_edge_job_t;
void xo_intra_fill_edges(const xo_intra_edge_job_t *jobs, int n, const uint8_t *pic, int stride, int width, int height,
                         uint8_t *edges, int64_t edges_size);
/* lambda * mode bits + SATD (hadamard) or SAD of every mode's prediction. */
void xo_intra_mode_costs(const uint8_t *ep, const uint8_t *fenc, int i_fenc, int bsx, int bsy, int dc_avail,
                         const int mpm[2], double lambda, int hadamard, double cost[33]);
/* The candidate list (9 entries) and the number of modes for RDO the
 * encoder derives from those costs: all modes (rough = 0,
 * rdo_get_pred_intra_luma) or the rough three-phase search (rough = 1,
 * rdo_get_pred_intra_luma_rmd) with dist2 / dist1 neighbours. */
int xo_intra_candidates(const double cost[33], int rough, int dist2, int dist1, int num_for_rdo, const int mpm[2],
                        int *modes, double *costs);

/* Batched form of the two above with the GPU entry's block / result
 * layouts (xavs2gpu_intra_block_t / _result_t): edges + edge_offset is a
 * block's top-left edge sample, the source block is fenc + fenc_offset. */
typedef struct xo_intra_block {
    int64_t edge_offset, fenc_offset;
    int16_t width, height, dc_avail;
    int8_t mpm[2];
    int32_t num_for_rdo, pad_;
} xo_intra_block_t;
typedef struct xo_intra_result {
    double cost[33];
    double cand_cost[9];
    int32_t cand_mode[9];
    int32_t num_for_rdo;
} xo_intra_result_t;
void xo_intra_rmd_batch(const xo_intra_block_t *blocks, int n, const uint8_t *edges, const uint8_t *fenc,
                        int fenc_stride, double lambda, int hadamard, int rough, int dist2, int dist1,
                        xo_intra_result_t *out, int threads);

/* ---- in-loop filters (filter_deblock.c, filter_sao.c) ------------------ */
/* One deblocking edge: dir 0 = vertical edge (lines run down, samples across
 * are horizontal neighbours), 1 = horizontal edge; 8 lines for luma, 4 per
 * chroma plane; flt_flag[0] / [1] enable the first / second half. */
void xo_deblock_luma(int dir, uint8_t *src, int stride, int alpha, int beta, const uint8_t *flt_flag);
void xo_deblock_chroma(int dir, uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                       const uint8_t *flt_flag);
/* Per-8x8-block edge parameters of a picture (the values lf_scu_deblock
 * derives from the CU data, filter_deblock.c:434-486): per direction the edge
 * type (0 none, 1 luma only, 2 luma and chroma), the two half-edge filter
 * flags, and alpha / beta for luma and for chroma. */
typedef struct xo_deblock_scu {
    uint8_t type[2];
    uint8_t flag[2][2];
    uint8_t alpha[2], beta[2];
    uint8_t alpha_c[2], beta_c[2];
    uint8_t pad_[2];
} xo_deblock_scu_t;
/* Deblocks a 4:2:0 picture in place (width, height multiples of 8), in the
 * reference's LCU order (lcu_order = 1, xavs2_lcu_deblock per LCU) or as two
 * picture-wide passes (all vertical edges, then all horizontal edges; in a
 * picture one LCU wide the horizontal edges of the last 8x8 column are left
 * unfiltered, as the LCU loop leaves them). */
void xo_deblock_picture(uint8_t *y, int stride, uint8_t *u, uint8_t *v, int stride_c, int width, int height,
                        const xo_deblock_scu_t *scus, int lcu_level, int lcu_order);

/* SAOBlkParam (basic_types.h:88-94) */
typedef struct xo_sao_param {
    int merge_idx, type_idc, start_band, delta_band;
    int offset[32];
} xo_sao_param_t;
/* sao_block: dst = clip(src + offset[class]) over the block's filtered
 * range; avail[8] = top, down, left, right, top-left, top-right, down-left,
 * down-right (lcu_neighbor_e, filter.h). */
void xo_sao_block(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w, int h, const int *avail,
                  const xo_sao_param_t *prm);
/* Per-LCU SAO parameters of a picture: type per component (-1 off, EO_0,
 * EO_90, EO_135, EO_45, BO), offsets per component, and the availability of
 * the top / down / left / right LCUs (bits 0..3; the diagonals are their
 * conjunctions, sao.c:898-929). */
typedef struct xo_sao_lcu {
    int8_t type[3];
    uint8_t avail;
    int8_t offset[3][32];
} xo_sao_lcu_t;
/* SAO of a 4:2:0 picture: every LCU's region (the LCU moved 4 samples up
 * and left inside the picture, sao.c:898-975) filtered from src into dst. */
void xo_sao_picture(uint8_t *const dst[3], const uint8_t *const src[3], int stride, int stride_c, int width,
                    int height, int lcu_level, const xo_sao_lcu_t *lcus);

/* ---- lookahead analysis (mc.c:838-855, pixel.c:1620-1649, rdo.c:3286-3297) */
/* lowres_filter: dst[y][x] = avg(avg(s[2y][2x], s[2y+1][2x]), avg(s[2y][2x+1],
 * s[2y+1][2x+1])), each avg rounding up; width, height = output size. */
void xo_lowres_filter(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height);
/* The half-resolution picture (width/2 x height/2) and the MAD of every
 * aligned 16x16, 32x32, 64x64 block fully inside the picture (raster order
 * per size over ceil(width/N) x ceil(height/N) positions; -1 where a block
 * leaves the picture). */
void xo_lookahead_picture(const uint8_t *src, int stride, int width, int height, uint8_t *lowres, int lowres_stride,
                          int32_t *mad16, int32_t *mad32, int32_t *mad64);

/* ---- skip / direct rough cost (rdo.c:2366-2480) ------------------------ */
typedef struct xo_skip_cand {
    int16_t x, y;
    uint8_t size_log2, n_pu;
    int16_t pad_;
    int32_t cu, rate;
    int8_t ref[4][2];
    int16_t mv[4][2][2];
} xo_skip_cand_t;
/* Per candidate: the luma prediction from the reference planes (planes[16 r
 * + k] at pixel (0,0), margin 80, stride `stride`; one list or the rounded
 * average of two), its SA8D against cur, cost = dist + lambda * rate; per CU
 * the first candidate with the strictly smallest cost.  Candidates whose
 * motion repeats an earlier one of their CU, or that are malformed, get
 * dist -1 and cost MAX_COST. */
void xo_skip_costs(const uint8_t *cur, int cur_stride, const uint8_t *const *planes, int stride, int width,
                   int height, int nrefs, const xo_skip_cand_t *cands, int n, double lambda, int n_cus,
                   int32_t *dist, double *cost, int32_t *best);

#endif
