/*
 * ref_harness.c -- drives the reference's own C primitives (compiled from the
 * xavs2 source files by oracle/Makefile into oracle/_ref/libxavs2ref.so).
 *
 * TEST INFRASTRUCTURE ONLY.  It exists to pin the oracle restatement: tests
 * compare xo_* (xavs2_oracle.c) with the xr_* entry points below on seeded and
 * adversarial inputs, and tests/golden/make_golden.py records xr_* outputs as
 * fixtures.  The primitive table is filled with the pure-C functions
 * (cpuid = 0), which is the reference's correctness baseline.
 */
#include "common.h"
#include "primitives.h"
#include "mc.h"
#include "me.h"
#include "filter.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The table the reference code dispatches through (primitives.c:51). */
intrinsic_func_t g_funcs;

/* Minimal stand-ins for the reference's logging/allocation helpers
 * (common.c), which the compiled primitives link against. */
void xavs2_log(void *p, int i_log_level, const char *psz_fmt, ...)
{
    (void)p; (void)i_log_level; (void)psz_fmt;
}
void *xavs2_malloc(size_t i_size) { return calloc(1, i_size); }
/* Placeholder for the chroma QP table (avs2tab.h:68) that the picture-level
 * deblocking loop (xavs2_lcu_deblock, never called here) references; the
 * per-edge filters driven below do not read it. */
const uint8_t tab_qp_scale_chroma[64] = {0};
void xavs2_free(void *ptr) { free(ptr); }

static int g_inited = 0;

void xr_init(void)
{
    if (g_inited) return;
    memset(&g_funcs, 0, sizeof(g_funcs));
    g_funcs.cpuid = 0;
    xavs2_mem_oper_init(0, &g_funcs);
    xavs2_pixel_init(0, &g_funcs.pixf);
    xavs2_mc_init(0, &g_funcs);
    xavs2_dct_init(0, &g_funcs.dctf);
    xavs2_quant_init(0, &g_funcs.dctf);
    xavs2_mad_init(0, g_funcs.pixf.madf);
    xavs2_intra_pred_init(0, &g_funcs);
    xavs2_deblock_init(0, &g_funcs);
    xavs2_sao_init(0, &g_funcs);
    g_inited = 1;
}

/* ---- pixel ------------------------------------------------------------- */
int32_t xr_cmp(int kind, int part, const pel_t *p1, intptr_t s1, const pel_t *p2, intptr_t s2)
{
    xr_init();
    switch (kind) {
    case 0: return g_funcs.pixf.sad[part](p1, s1, p2, s2);
    case 1: return g_funcs.pixf.satd[part](p1, s1, p2, s2);
    case 2: return g_funcs.pixf.sa8d[part](p1, s1, p2, s2);
    default: return g_funcs.pixf.ssd[part](p1, s1, p2, s2);
    }
}

void xr_sad_x3(int part, const pel_t *fenc, const pel_t *r0, const pel_t *r1, const pel_t *r2,
               intptr_t stride, int *res)
{
    xr_init();
    g_funcs.pixf.sad_x3[part](fenc, r0, r1, r2, stride, res);
}

void xr_sad_x4(int part, const pel_t *fenc, const pel_t *r0, const pel_t *r1, const pel_t *r2,
               const pel_t *r3, intptr_t stride, int *res)
{
    xr_init();
    g_funcs.pixf.sad_x4[part](fenc, r0, r1, r2, r3, stride, res);
}

void xr_avg(int part, pel_t *dst, intptr_t ds, const pel_t *a, intptr_t sa, const pel_t *b,
            intptr_t sb)
{
    xr_init();
    g_funcs.pixf.avg[part](dst, ds, a, sa, b, sb, 32);
}

void xr_sub_ps(int part, coeff_t *dst, intptr_t ds, const pel_t *a, const pel_t *b, intptr_t sa,
               intptr_t sb)
{
    xr_init();
    g_funcs.pixf.sub_ps[part](dst, ds, a, b, sa, sb);
}

void xr_add_ps(int part, pel_t *dst, intptr_t ds, const pel_t *a, const coeff_t *b, intptr_t sa,
               intptr_t sb)
{
    xr_init();
    g_funcs.pixf.add_ps[part](dst, ds, a, b, sa, sb);
}

void xr_copy(int kind, int part, void *dst, intptr_t ds, const void *src, intptr_t ss)
{
    xr_init();
    switch (kind) {
    case 0: g_funcs.pixf.copy_pp[part]((pel_t *)dst, ds, (const pel_t *)src, ss); break;
    case 1: g_funcs.pixf.copy_ps[part]((coeff_t *)dst, ds, (const pel_t *)src, ss); break;
    case 2: g_funcs.pixf.copy_sp[part]((pel_t *)dst, ds, (const coeff_t *)src, ss); break;
    default: g_funcs.pixf.copy_ss[part]((coeff_t *)dst, ds, (const coeff_t *)src, ss); break;
    }
}

int32_t xr_ssd_block(const pel_t *p1, intptr_t s1, const pel_t *p2, intptr_t s2, int w, int h)
{
    xr_init();
    return g_funcs.pixf.ssd_block(p1, s1, p2, s2, w, h);
}

void xr_average(pel_t *dst, int ds, pel_t *a, int sa, pel_t *b, int sb, int w, int h)
{
    xr_init();
    g_funcs.pixf.average(dst, ds, a, sa, b, sb, w, h);
}

int xr_mad(pel_t *src, int stride, int cu_size)
{
    int lvl = cu_size == 16 ? 1 : (cu_size == 32 ? 2 : 3);
    xr_init();
    return g_funcs.pixf.madf[lvl](src, stride, cu_size);
}

/* ---- interpolation ----------------------------------------------------- */
void xr_intpl_luma_hor(pel_t *dst, int ds, mct_t *tmp, int ts, pel_t *src, int ss, int w, int h,
                       const int8_t *c)
{
    xr_init();
    g_funcs.intpl_luma_hor(dst, ds, tmp, ts, src, ss, w, h, c);
}
void xr_intpl_luma_ver(pel_t *dst, int ds, pel_t *src, int ss, int w, int h, const int8_t *c)
{
    xr_init();
    g_funcs.intpl_luma_ver(dst, ds, src, ss, w, h, c);
}
void xr_intpl_luma_ext(pel_t *dst, int ds, mct_t *tmp, int ts, int w, int h, const int8_t *c)
{
    xr_init();
    g_funcs.intpl_luma_ext(dst, ds, tmp, ts, w, h, c);
}
void xr_intpl_block(int kind, pel_t *dst, int ds, pel_t *src, int ss, int w, int h,
                    const int8_t *cx, const int8_t *cy)
{
    xr_init();
    switch (kind) {
    case 0: g_funcs.intpl_luma_block_hor(dst, ds, src, ss, w, h, cx); break;
    case 1: g_funcs.intpl_luma_block_ver(dst, ds, src, ss, w, h, cy); break;
    case 2: g_funcs.intpl_luma_block_ext(dst, ds, src, ss, w, h, cx, cy); break;
    case 3: g_funcs.intpl_chroma_block_hor(dst, ds, src, ss, w, h, cx); break;
    case 4: g_funcs.intpl_chroma_block_ver(dst, ds, src, ss, w, h, cy); break;
    default: g_funcs.intpl_chroma_block_ext(dst, ds, src, ss, w, h, cx, cy); break;
    }
}

/* Runs the reference's per-LCU-row interpolation (mc.c:748-785) over a whole
 * frame.  `planes[k]` point at pixel (0,0) of buffers with `stride` and an
 * 80-pixel margin; planes[0] is the padded full-pel picture. */
void xr_interpolate_frame(pel_t **planes, int stride, int width, int height, int lcu_level,
                          int mode)
{
    xavs2_t *h = (xavs2_t *)calloc(1, sizeof(xavs2_t));
    xavs2_param_t *param = (xavs2_param_t *)calloc(1, sizeof(xavs2_param_t));
    xavs2_frame_t *frm = (xavs2_frame_t *)calloc(1, sizeof(xavs2_frame_t));
    int i_tmp = width + 2 * XAVS2_PAD;
    int rows = (height + (1 << lcu_level) - 1) >> lcu_level;
    int k, r;
    xr_init();
    param->slice_num = 1;
    h->param = param;
    h->use_fractional_me = mode;
    h->i_lcu_level = lcu_level;
    h->i_height_in_lcu = rows;
    h->i_height = height;
    h->i_width = width;
    for (k = 0; k < 3; k++) h->img4Y_tmp[k] = (mct_t *)calloc((size_t)i_tmp * (height + 2 * XAVS2_PAD), sizeof(mct_t));
    frm->i_stride[0] = stride;
    frm->i_width[0] = width;
    frm->i_lines[0] = height;
    frm->planes[0] = planes[0];
    for (k = 0; k < 16; k++) frm->filtered[k] = planes[k];
    for (r = 0; r < rows; r++) interpolate_lcu_row(h, frm, r);
    for (k = 0; k < 3; k++) free(h->img4Y_tmp[k]);
    free(frm);
    free(param);
    free(h);
}

/* ---- transform / quant ------------------------------------------------- */
void xr_dct(int kind, int part, const coeff_t *src, coeff_t *dst, int stride)
{
    xr_init();
    switch (kind) {
    case 0: g_funcs.dctf.dct[part](src, dst, stride); break;
    case 1: g_funcs.dctf.idct[part](src, dst, stride); break;
    default: g_funcs.dctf.dct_half[part](src, dst, stride); break;
    }
}

void xr_2nd(int kind, coeff_t *coef, int stride, int mode, int b_top, int b_left)
{
    xr_init();
    switch (kind) {
    case 0: g_funcs.dctf.transform_4x4_2nd(coef, stride); break;
    case 1: g_funcs.dctf.inv_transform_4x4_2nd(coef, stride); break;
    case 2: g_funcs.dctf.transform_2nd(coef, stride, mode, b_top, b_left); break;
    default: g_funcs.dctf.inv_transform_2nd(coef, stride, mode, b_top, b_left); break;
    }
}

int xr_quant(coeff_t *coef, int n, int scale, int shift, int add)
{
    xr_init();
    return g_funcs.dctf.quant(coef, n, scale, shift, add);
}

int xr_wquant(coeff_t *coef, int n, int scale, int shift, int add, int *levelscale)
{
    xr_init();
    return g_funcs.dctf.wquant(coef, n, scale, shift, add, levelscale);
}

void xr_dequant(coeff_t *coef, int n, int scale, int shift)
{
    xr_init();
    g_funcs.dctf.dequant(coef, n, scale, shift);
}

void xr_abs_coeff(coeff_t *dst, const coeff_t *src, int n)
{
    xr_init();
    g_funcs.dctf.abs_coeff(dst, src, n);
}

int xr_add_sign(coeff_t *dst, const coeff_t *abs_val, int n)
{
    xr_init();
    return g_funcs.dctf.add_sign(dst, abs_val, n);
}

extern const uint16_t tab_Q_TAB[80];
extern const uint16_t tab_IQ_TAB[80];
extern const uint8_t tab_IQ_SHIFT[80];
int xr_q_scale(int qp) { return tab_Q_TAB[qp]; }
int xr_iq_scale(int qp) { return tab_IQ_TAB[qp]; }
int xr_iq_shift(int qp) { return tab_IQ_SHIFT[qp]; }

/* ---- motion search ----------------------------------------------------- */
typedef struct xr_me_params {
    int32_t search_range, lambda_factor, use_hadamard, fractional_me, fast_sub_me, enable_pmvr;
} xr_me_params_t;

typedef struct xr_pu {
    int16_t x, y;
    uint8_t part, ref;
    int16_t mvp_x, mvp_y;
    int16_t min_x, min_y, max_x, max_y;
} xr_pu_t;

typedef struct xr_me_result {
    int16_t bmv_x, bmv_y;
    int32_t bcost, mvcost;
    int16_t imv_x, imv_y;
    int32_t icost;
} xr_me_result_t;

/* Calls the reference's xavs2_me_search (me.c:879) in full-search mode for
 * one PU.  The encode block is copied into a FENC_STRIDE buffer as the
 * encoder's LCU buffer would hold it; candidates are built the way
 * pred_inter_search_single does (md_inter.c:840-865, 957-959). */
int32_t xr_me_search(const xr_me_params_t *prm, const xr_pu_t *pu, const pel_t *fenc,
                     intptr_t i_fenc, pel_t *const fref[16], int i_fref, xr_me_result_t *out)
{
    static __thread xavs2_t *h = NULL;
    static __thread xavs2_param_t *param = NULL;
    static __thread uint8_t *mvbuf = NULL;
    xavs2_me_t me;
    xavs2_frame_t frm;
    ALIGN32(pel_t blk[FENC_STRIDE * MAX_CU_SIZE]);
    int16_t mvc[8][2];
    int i_mvc = 0, c, y;
    dist_t cost;
    xr_init();
    if (h == NULL) {
        uint8_t *mb;
        h = (xavs2_t *)calloc(1, sizeof(xavs2_t));
        param = (xavs2_param_t *)calloc(1, sizeof(xavs2_param_t));
        h->param = param;
        param->search_range = 64;
        mvbuf = (uint8_t *)calloc(1, (size_t)xavs2_me_get_buf_size(param) + 64);
        mb = mvbuf;
        xavs2_me_init(h, &mb);
    }
    param->me_method = XAVS2_ME_FS;
    param->search_range = prm->search_range;
    param->enable_hadamard = prm->use_hadamard;
    param->enable_pmvr = prm->enable_pmvr;
    h->i_lambda_factor = prm->lambda_factor;
    h->use_fractional_me = prm->fractional_me;
    h->use_fast_sub_me = prm->fast_sub_me;
    h->UMH_big_hex_level = 2;
    g_funcs.pixf.fpel_cmp = prm->use_hadamard ? g_funcs.pixf.satd : g_funcs.pixf.sad;

    {
        int bw = 0, bh = 0, k;
        static const uint8_t pw[25] = {4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32,
                                       16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16};
        static const uint8_t ph[25] = {4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64,
                                       12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64};
        bw = pw[pu->part]; bh = ph[pu->part];
        for (y = 0; y < bh; y++) memcpy(blk + y * FENC_STRIDE, fenc + y * i_fenc, (size_t)bw);
        memset(&me, 0, sizeof(me));
        memset(&frm, 0, sizeof(frm));
        frm.i_stride[0] = i_fref;
        frm.planes[0] = fref[0];
        for (k = 0; k < 16; k++) frm.filtered[k] = fref[k];
        me.p_fenc = blk;
        me.i_pixel = pu->part;
        me.i_pix_x = pu->x; me.i_pix_y = pu->y;
        me.i_block_w = bw; me.i_block_h = bh;
        me.i_bias = pu->y * i_fref + pu->x;
        me.p_fref_1st = &frm;
        me.mvp.x = pu->mvp_x; me.mvp.y = pu->mvp_y;
        me.mv_min_fpel[0] = pu->min_x; me.mv_min_fpel[1] = pu->min_y;
        me.mv_max_fpel[0] = pu->max_x; me.mv_max_fpel[1] = pu->max_y;
    }
    {
        int xs[2] = {(pu->mvp_x + 2) >> 2, 0}, ys[2] = {(pu->mvp_y + 2) >> 2, 0};
        for (c = 0; c < 2; c++) {
            int x = XAVS2_CLIP3(me.mv_min_fpel[0], me.mv_max_fpel[0], xs[c]);
            int yy = XAVS2_CLIP3(me.mv_min_fpel[1], me.mv_max_fpel[1], ys[c]);
            int i;
            for (i = 0; i < i_mvc; i++)
                if (mvc[i][0] == x && mvc[i][1] == yy) break;
            if (i == i_mvc) { mvc[i_mvc][0] = (int16_t)x; mvc[i_mvc][1] = (int16_t)yy; i_mvc++; }
        }
    }
    cost = xavs2_me_search(h, &me, mvc, i_mvc);
    out->bmv_x = me.bmv.x; out->bmv_y = me.bmv.y;
    out->bcost = cost;
    out->mvcost = me.mvcost[PDIR_FWD];
    out->imv_x = me.bmv2.x; out->imv_y = me.bmv2.y;
    out->icost = (cost == MAX_DISTORTION) ? cost : me.bcost2;
    return cost;
}

/* xr_me_search over a PU list (frefs: 16 planes per reference), on
 * `threads` OpenMP threads, in the same loop form as the oracle's
 * xo_me_search_list, so that the two can be timed side by side.  xr_init
 * runs first on this thread: it fills the shared table once. */
void xr_me_search_list(const xr_me_params_t *prm, const xr_pu_t *pus, int n, const pel_t *fenc, intptr_t i_fenc,
                       pel_t *const *frefs, int i_fref, xr_me_result_t *out, int threads)
{
    int i;
    xr_init();
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads > 0 ? threads : 1)
#endif
    for (i = 0; i < n; i++) {
        const xr_pu_t *pu = &pus[i];
        xr_me_search(prm, pu, fenc + pu->y * i_fenc + pu->x, i_fenc, frefs + 16 * pu->ref, i_fref, &out[i]);
    }
    (void)threads;
}

int xr_mvbits(int d)
{
    static xavs2_t *h = NULL;
    if (h == NULL) {
        xavs2_param_t *param = (xavs2_param_t *)calloc(1, sizeof(xavs2_param_t));
        uint8_t *mb;
        h = (xavs2_t *)calloc(1, sizeof(xavs2_t));
        param->search_range = 64;
        h->param = param;
        mb = (uint8_t *)calloc(1, (size_t)xavs2_me_get_buf_size(param) + 64);
        xavs2_me_init(h, &mb);
    }
    return h->mvbits[d];
}

/* ---- intra prediction (intra.c) ---------------------------------------- */
/* One table entry: `ep` is the top-left edge sample (intra.c's src), the
 * block is written to dst with stride i_dst; dir_mode as the encoder passes
 * it (the availability word for DC, md_intra.c:170-185). */
void xr_intra_pred(int mode, pel_t *ep, pel_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    xr_init();
    g_funcs.intraf[mode](ep, dst, i_dst, dir_mode, bsx, bsy);
}

/* fill_edge_f[xy] (intra.c:1580-1840): builds the edge samples of a block
 * whose top-left neighbour is pTL (stride i_TL), with the top border line
 * pLcuEP for blocks on the CTU's top edge. */
void xr_intra_fill_edge(int xy, const pel_t *pTL, int i_TL, const pel_t *pLcuEP, pel_t *EP, uint32_t avail, int bsx,
                        int bsy)
{
    xr_init();
    g_funcs.fill_edge_f[xy](pTL, i_TL, pLcuEP, EP, avail, bsx, bsy);
}

/* ---- in-loop filters (filter_deblock.c, filter_sao.c) -------------------- */
/* deblock_luma[dir] / deblock_chroma[dir] (filter_deblock.c:400-431): one
 * 8-sample edge (4 per chroma plane), dir 0 = vertical edge, 1 = horizontal. */
void xr_deblock_luma(int dir, pel_t *src, int stride, int alpha, int beta, uint8_t *flt_flag)
{
    xr_init();
    g_funcs.deblock_luma[dir](src, stride, alpha, beta, flt_flag);
}
void xr_deblock_chroma(int dir, pel_t *src_u, pel_t *src_v, int stride, int alpha, int beta, uint8_t *flt_flag)
{
    xr_init();
    g_funcs.deblock_chroma[dir](src_u, src_v, stride, alpha, beta, flt_flag);
}
/* sao_block (filter_sao.c:50-226) */
void xr_sao_block(pel_t *p_dst, int i_dst, pel_t *p_src, int i_src, int w, int h, int *avail, SAOBlkParam *prm)
{
    xr_init();
    g_funcs.sao_block(p_dst, i_dst, p_src, i_src, w, h, avail, prm);
}

/* lowres_filter (mc.c:838-855, table member primitives.h:140) */
void xr_lowres_filter(pel_t *src, int i_src, pel_t *dst, int i_dst, int width, int height)
{
    xr_init();
    g_funcs.lowres_filter(src, i_src, dst, i_dst, width, height);
}
