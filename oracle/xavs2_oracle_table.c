/*
 * xavs2_oracle_table.c -- the oracle's restatements behind the reference's
 * primitive-table signatures.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference's table entries carry no shape argument: the shape is the
 * array index (pixf.sad[PART], dctf.dct[PART], intraf[MODE],
 * deblock_luma[DIR]).  These adapters bind the index, so that the oracle can
 * be installed in a real encoder's table (the bitstream check) and replayed
 * on recorded calls exactly like the GPU drop-ins.  xo_tab_entry() maps
 * (kind, slot) of oracle/enc_calls.h to an adapter.
 */
#include <stddef.h>
#include <stdint.h>

#include "enc_calls.h"
#include "xavs2_oracle.h"

#define FOR25(X) X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) \
                 X(16) X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24)
#define FOR33(X) FOR25(X) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)
#define LIST25(P) {P##0, P##1, P##2, P##3, P##4, P##5, P##6, P##7, P##8, P##9, P##10, P##11, P##12, P##13, \
                   P##14, P##15, P##16, P##17, P##18, P##19, P##20, P##21, P##22, P##23, P##24}
#define LIST33(P) {P##0, P##1, P##2, P##3, P##4, P##5, P##6, P##7, P##8, P##9, P##10, P##11, P##12, P##13, \
                   P##14, P##15, P##16, P##17, P##18, P##19, P##20, P##21, P##22, P##23, P##24, P##25,     \
                   P##26, P##27, P##28, P##29, P##30, P##31, P##32}

/* pixel_funcs_t members (pixel.h:124-137 signatures) */
#define CMP(k)                                                                                          \
    static int32_t sad_##k(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)               \
    { return xo_sad(k, a, sa, b, sb); }                                                                 \
    static int32_t satd_##k(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)              \
    { return xo_satd(k, a, sa, b, sb); }                                                                \
    static int32_t sa8d_##k(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)              \
    { return xo_sa8d(k, a, sa, b, sb); }                                                                \
    static int32_t ssd_##k(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)               \
    { return xo_ssd(k, a, sa, b, sb); }                                                                 \
    static void sadx3_##k(const uint8_t *f, const uint8_t *r0, const uint8_t *r1, const uint8_t *r2,    \
                          intptr_t s, int res[3])                                                       \
    { xo_sad_x3(k, f, r0, r1, r2, s, res); }                                                            \
    static void sadx4_##k(const uint8_t *f, const uint8_t *r0, const uint8_t *r1, const uint8_t *r2,    \
                          const uint8_t *r3, intptr_t s, int res[4])                                    \
    { xo_sad_x4(k, f, r0, r1, r2, r3, s, res); }                                                        \
    static void subps_##k(int16_t *d, intptr_t sd, const uint8_t *a, const uint8_t *b, intptr_t sa,     \
                          intptr_t sb)                                                                  \
    { xo_sub_ps(k, d, sd, a, b, sa, sb); }                                                              \
    static void addps_##k(uint8_t *d, intptr_t sd, const uint8_t *a, const int16_t *b, intptr_t sa,     \
                          intptr_t sb)                                                                  \
    { xo_add_ps(k, d, sd, a, b, sa, sb); }                                                              \
    static void cpsp_##k(uint8_t *d, intptr_t sd, const int16_t *s, intptr_t ss) { xo_copy_sp(k, d, sd, s, ss); } \
    static void cpps_##k(int16_t *d, intptr_t sd, const uint8_t *s, intptr_t ss) { xo_copy_ps(k, d, sd, s, ss); } \
    static void cpss_##k(int16_t *d, intptr_t sd, const int16_t *s, intptr_t ss) { xo_copy_ss(k, d, sd, s, ss); } \
    static void cppp_##k(uint8_t *d, intptr_t sd, const uint8_t *s, intptr_t ss) { xo_copy_pp(k, d, sd, s, ss); } \
    static void avg_##k(uint8_t *d, intptr_t sd, const uint8_t *a, intptr_t sa, const uint8_t *b,       \
                        intptr_t sb, int weight)                                                        \
    { (void)weight; xo_avg(k, d, sd, a, sa, b, sb); }                                                   \
    static void dct_##k(const int16_t *s, int16_t *d, int i) { xo_dct(k, s, d, i); }                    \
    static void idct_##k(const int16_t *s, int16_t *d, int i) { xo_idct(k, s, d, i); }                  \
    static void dcth_##k(const int16_t *s, int16_t *d, int i) { xo_dct_half(k, s, d, i); }
FOR25(CMP)

static void *const t_sad[25] = LIST25(sad_), *const t_satd[25] = LIST25(satd_), *const t_sa8d[25] = LIST25(sa8d_),
                   *const t_ssd[25] = LIST25(ssd_), *const t_sadx3[25] = LIST25(sadx3_),
                   *const t_sadx4[25] = LIST25(sadx4_), *const t_subps[25] = LIST25(subps_),
                   *const t_addps[25] = LIST25(addps_), *const t_cpsp[25] = LIST25(cpsp_),
                   *const t_cpps[25] = LIST25(cpps_), *const t_cpss[25] = LIST25(cpss_),
                   *const t_cppp[25] = LIST25(cppp_), *const t_avg[25] = LIST25(avg_),
                   *const t_dct[25] = LIST25(dct_), *const t_idct[25] = LIST25(idct_),
                   *const t_dcth[25] = LIST25(dcth_);

static int mad_fn(uint8_t *src, int i_src, int cu_size) { return xo_mad(src, i_src, cu_size); }
static int32_t ssd_block_fn(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb, int w, int h)
{
    return xo_ssd_block(a, sa, b, sb, w, h);
}
static void average_fn(uint8_t *d, int sd, uint8_t *a, int sa, uint8_t *b, int sb, int w, int h)
{
    xo_average(d, sd, a, sa, b, sb, w, h);
}

/* interpolation (primitives.h:62-70 signatures) */
static void luma_hor(uint8_t *d, int sd, int16_t *t, int st, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_luma_hor(d, sd, t, st, s, ss, w, h, c);
}
static void luma_ver(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_luma_ver(d, sd, s, ss, w, h, c);
}
static void luma_ext(uint8_t *d, int sd, int16_t *t, int st, int w, int h, const int8_t *c)
{
    xo_intpl_luma_ext(d, sd, t, st, w, h, c);
}
static void luma_ver_x3(uint8_t *const d[3], int sd, uint8_t *s, int ss, int w, int h, const int8_t **c)
{
    for (int k = 0; k < 3; k++) xo_intpl_luma_ver(d[k], sd, s, ss, w, h, c[k]);
}
static void luma_hor_x3(uint8_t *const d[3], int sd, int16_t *const t[3], int st, uint8_t *s, int ss, int w,
                        int h, const int8_t **c)
{
    for (int k = 0; k < 3; k++) xo_intpl_luma_hor(d[k], sd, t[k], st, s, ss, w, h, c[k]);
}
static void luma_ext_x3(uint8_t *const d[3], int sd, int16_t *t, int st, int w, int h, const int8_t **c)
{
    for (int k = 0; k < 3; k++) xo_intpl_luma_ext(d[k], sd, t, st, w, h, c[k]);
}
static void luma_blk_hor(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_luma_block_hor(d, sd, s, ss, w, h, c);
}
static void luma_blk_ver(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_luma_block_ver(d, sd, s, ss, w, h, c);
}
static void luma_blk_ext(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *cx, const int8_t *cy)
{
    xo_intpl_luma_block_ext(d, sd, s, ss, w, h, cx, cy);
}
static void chroma_blk_hor(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_chroma_block_hor(d, sd, s, ss, w, h, c);
}
static void chroma_blk_ver(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *c)
{
    xo_intpl_chroma_block_ver(d, sd, s, ss, w, h, c);
}
static void chroma_blk_ext(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, const int8_t *cx,
                           const int8_t *cy)
{
    xo_intpl_chroma_block_ext(d, sd, s, ss, w, h, cx, cy);
}

/* intra_pred_t (primitives.h:76): the table index is the mode; for DC the
 * fourth argument carries the availability (md_intra.c:176-185). */
#define INTRA(k)                                                                                        \
    static void intra_##k(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)       \
    { xo_intra_pred(k, src, dst, i_dst, k == 0 ? dir_mode : 0, bsx, bsy); }
FOR33(INTRA)
static void *const t_intra[33] = LIST33(intra_);

/* transforms and quantisation (dct_funcs_t) */
static void t4_2nd(int16_t *c, int i) { xo_transform_4x4_2nd(c, i); }
static void inv_t4_2nd(int16_t *c, int i) { xo_inv_transform_4x4_2nd(c, i); }
static void t_2nd(int16_t *c, int i, int m, int t, int l) { xo_transform_2nd(c, i, m, t, l); }
static void inv_t_2nd(int16_t *c, int i, int m, int t, int l) { xo_inv_transform_2nd(c, i, m, t, l); }
static void abs_coeff(int16_t *d, const int16_t *s, const int n) { xo_abs_coeff(d, s, n); }
static int add_sign(int16_t *d, const int16_t *a, const int n) { return xo_add_sign(d, a, n); }
static int quant(int16_t *c, const int n, const int sc, const int sh, const int add) { return xo_quant(c, n, sc, sh, add); }
static void dequant(int16_t *c, const int n, const int sc, const int sh) { xo_dequant(c, n, sc, sh); }
static int wquant(int16_t *c, const int n, const int sc, const int sh, const int add, int *ls)
{
    return xo_wquant(c, n, sc, sh, add, ls);
}

/* in-loop filters (primitives.h:202-208) */
static void dbk_luma_0(uint8_t *s, int st, int a, int b, uint8_t *f) { xo_deblock_luma(0, s, st, a, b, f); }
static void dbk_luma_1(uint8_t *s, int st, int a, int b, uint8_t *f) { xo_deblock_luma(1, s, st, a, b, f); }
static void dbk_chroma_0(uint8_t *u, uint8_t *v, int st, int a, int b, uint8_t *f)
{
    xo_deblock_chroma(0, u, v, st, a, b, f);
}
static void dbk_chroma_1(uint8_t *u, uint8_t *v, int st, int a, int b, uint8_t *f)
{
    xo_deblock_chroma(1, u, v, st, a, b, f);
}
static void sao_fn(uint8_t *d, int sd, uint8_t *s, int ss, int w, int h, int *avail, void *prm)
{
    xo_sao_block(d, sd, s, ss, w, h, avail, (const xo_sao_param_t *)prm);
}
static void lowres_fn(uint8_t *s, int ss, uint8_t *d, int sd, int w, int h) { xo_lowres_filter(s, ss, d, sd, w, h); }

void *xo_tab_entry(int kind, int slot)
{
    if (slot < 0 || slot >= EC_MAX_SLOTS) return NULL;
    const int s25 = slot < 25;
    switch (kind) {
    case EC_SAD: return s25 ? t_sad[slot] : NULL;
    case EC_SATD: return s25 ? t_satd[slot] : NULL;
    case EC_SA8D: return s25 ? t_sa8d[slot] : NULL;
    case EC_SSD: return s25 ? t_ssd[slot] : NULL;
    case EC_SAD_X3: return s25 ? t_sadx3[slot] : NULL;
    case EC_SAD_X4: return s25 ? t_sadx4[slot] : NULL;
    case EC_SUB_PS: return s25 ? t_subps[slot] : NULL;
    case EC_ADD_PS: return s25 ? t_addps[slot] : NULL;
    case EC_COPY_SP: return s25 ? t_cpsp[slot] : NULL;
    case EC_COPY_PS: return s25 ? t_cpps[slot] : NULL;
    case EC_COPY_SS: return s25 ? t_cpss[slot] : NULL;
    case EC_COPY_PP: return s25 ? t_cppp[slot] : NULL;
    case EC_AVG: return s25 ? t_avg[slot] : NULL;
    case EC_MAD: return slot < 4 ? (void *)mad_fn : NULL;
    case EC_SSD_BLOCK: return slot == 0 ? (void *)ssd_block_fn : NULL;
    case EC_AVERAGE: return slot == 0 ? (void *)average_fn : NULL;
    case EC_LUMA_HOR: return slot == 0 ? (void *)luma_hor : NULL;
    case EC_LUMA_VER: return slot == 0 ? (void *)luma_ver : NULL;
    case EC_LUMA_EXT: return slot == 0 ? (void *)luma_ext : NULL;
    case EC_LUMA_VER_X3: return slot == 0 ? (void *)luma_ver_x3 : NULL;
    case EC_LUMA_HOR_X3: return slot == 0 ? (void *)luma_hor_x3 : NULL;
    case EC_LUMA_EXT_X3: return slot == 0 ? (void *)luma_ext_x3 : NULL;
    case EC_LUMA_BLOCK_HOR: return slot == 0 ? (void *)luma_blk_hor : NULL;
    case EC_LUMA_BLOCK_VER: return slot == 0 ? (void *)luma_blk_ver : NULL;
    case EC_LUMA_BLOCK_EXT: return slot == 0 ? (void *)luma_blk_ext : NULL;
    case EC_CHROMA_BLOCK_HOR: return slot == 0 ? (void *)chroma_blk_hor : NULL;
    case EC_CHROMA_BLOCK_VER: return slot == 0 ? (void *)chroma_blk_ver : NULL;
    case EC_CHROMA_BLOCK_EXT: return slot == 0 ? (void *)chroma_blk_ext : NULL;
    case EC_INTRA: return t_intra[slot];
    case EC_DCT: return s25 && xo_is_tu_shape(slot) ? t_dct[slot] : NULL;
    case EC_IDCT: return s25 && xo_is_tu_shape(slot) ? t_idct[slot] : NULL;
    case EC_DCT_HALF: return (slot == 3 || slot == 4) ? t_dcth[slot] : NULL;
    case EC_T4_2ND: return slot == 0 ? (void *)t4_2nd : NULL;
    case EC_INV_T4_2ND: return slot == 0 ? (void *)inv_t4_2nd : NULL;
    case EC_T_2ND: return slot == 0 ? (void *)t_2nd : NULL;
    case EC_INV_T_2ND: return slot == 0 ? (void *)inv_t_2nd : NULL;
    case EC_ABS_COEFF: return slot == 0 ? (void *)abs_coeff : NULL;
    case EC_ADD_SIGN: return slot == 0 ? (void *)add_sign : NULL;
    case EC_QUANT: return slot == 0 ? (void *)quant : NULL;
    case EC_DEQUANT: return slot == 0 ? (void *)dequant : NULL;
    case EC_WQUANT: return slot == 0 ? (void *)wquant : NULL;
    case EC_DEBLOCK_LUMA: return slot == 0 ? (void *)dbk_luma_0 : slot == 1 ? (void *)dbk_luma_1 : NULL;
    case EC_DEBLOCK_CHROMA: return slot == 0 ? (void *)dbk_chroma_0 : slot == 1 ? (void *)dbk_chroma_1 : NULL;
    case EC_SAO: return slot == 0 ? (void *)sao_fn : NULL;
    case EC_LOWRES: return slot == 0 ? (void *)lowres_fn : NULL;
    default: return NULL;
    }
}
