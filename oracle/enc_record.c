/*
 * enc_record.c -- drives the reference encoder (built from its own source
 * files by oracle/Makefile) and records or replaces its primitive-table
 * calls.  TEST INFRASTRUCTURE ONLY: it makes the config-0 oracle (every
 * primitive call of a real encode, with the strides, aliasing and flag bits
 * the encoder really uses) and checks that a table of drop-ins leaves the
 * encoder's output unchanged.
 *
 *   xavs2_record MODE RECORDS -- <xavs2 arguments, e.g. -f encoder_ra.cfg
 *                                 -p preset=0 -p input=a.yuv ...>
 *   MODE plain   the stock table
 *        record  the stock table, with a sample of every entry's calls
 *                written to RECORDS (format: oracle/enc_calls.h), followed
 *                by the number of calls of every entry
 *        oracle  every entry the oracle restates replaced by
 *                xo_tab_entry() (oracle/xavs2_oracle_table.c); RECORDS gets
 *                the list of replaced entries
 *
 * The table is patched after encoder_create, i.e. after
 * xavs2_init_all_primitives (encoder/xavs2.c:274-278); the encoder's later
 * intra_cmp / fpel_cmp aliasing (encoder.c:1837-1847) points at the patched
 * sad / satd arrays.  The frame loop follows the reference's test driver
 * (test/test.c:125-199).
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "xavs2.h"
#include "enc_calls.h"

/* LumaPU shapes (pixel.h:50-65) */
static const int k_pw[25] = {4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32, 16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16};
static const int k_ph[25] = {4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64, 12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64};

static intrinsic_func_t g_stock;            /* the table as the encoder set it up */
static FILE *g_rec;
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static uint64_t g_calls[EC_NUM_KINDS][EC_MAX_SLOTS];
static uint64_t g_next[EC_NUM_KINDS][EC_MAX_SLOTS];
static int g_taken[EC_NUM_KINDS][EC_MAX_SLOTS];

/* ---- the recorder ------------------------------------------------------ */
typedef struct {
    char type;
    int64_t v;
    const uint8_t *p;
    int esize, alias;
    int64_t stride;
    int in[4], out[4];
    uint8_t *snap_in, *snap_out;
} rarg_t;

typedef struct {
    int on, kind, slot, n;
    uint32_t idx;
    rarg_t a[24];
} rec_t;

/* entries whose calls carry whole picture rows get fewer samples */
static int is_plane_kind(int kind)
{
    return kind == EC_LUMA_HOR || kind == EC_LUMA_VER || kind == EC_LUMA_EXT || kind == EC_LUMA_VER_X3 ||
           kind == EC_LUMA_HOR_X3 || kind == EC_LUMA_EXT_X3 || kind == EC_LOWRES;
}

/* Sampling: the first calls of every entry, then calls whose index grows
 * geometrically (x1.5), so that a sample reaches every picture of the
 * sequence; at most 24 records per entry (2 for plane-level entries). */
static void rec_begin(rec_t *r, int kind, int slot)
{
    memset(r, 0, sizeof(*r));
    r->kind = kind;
    r->slot = slot;
    pthread_mutex_lock(&g_mu);
    uint64_t c = g_calls[kind][slot]++;
    const int first = is_plane_kind(kind) ? 1 : 6, cap = is_plane_kind(kind) ? 2 : 24;
    if (g_rec && g_taken[kind][slot] < cap && (c < (uint64_t)first || c == g_next[kind][slot])) {
        r->on = 1;
        r->idx = (uint32_t)c;
        g_taken[kind][slot]++;
        if (c >= (uint64_t)first || g_next[kind][slot] == 0)
            g_next[kind][slot] = (c < (uint64_t)first ? (uint64_t)first : c) * 3 / 2 + 1;
    }
    pthread_mutex_unlock(&g_mu);
}

static void rec_int(rec_t *r, char type, int64_t v)
{
    if (!r->on) return;
    rarg_t *a = &r->a[r->n++];
    a->type = type;
    a->v = v;
}

static void rec_arr(rec_t *r, int count) { rec_int(r, 'a', count); }

static uint8_t *snap(const uint8_t *p, int esize, int64_t stride, const int reg[4])
{
    const int rows = reg[1] - reg[0], cols = reg[3] - reg[2];
    if (rows <= 0 || cols <= 0) return NULL;
    uint8_t *s = (uint8_t *)malloc((size_t)rows * cols * esize);
    for (int y = 0; y < rows; y++)
        memcpy(s + (size_t)y * cols * esize, p + ((int64_t)(reg[0] + y) * stride + reg[2]) * esize, (size_t)cols * esize);
    return s;
}

/* A buffer argument: input region rows [ir0, ir1) x cols [ic0, ic1) and
 * output region likewise, in elements relative to p (empty = none). */
static void rec_buf(rec_t *r, const void *p, int esize, int64_t stride, int ir0, int ir1, int ic0, int ic1, int or0,
                    int or1, int oc0, int oc1)
{
    if (!r->on) return;
    rarg_t *a = &r->a[r->n++];
    a->type = 'b';
    a->p = (const uint8_t *)p;
    a->esize = esize;
    a->stride = stride;
    a->alias = -1;
    for (int k = 0; k < r->n - 1; k++)
        if (r->a[k].type == 'b' && r->a[k].p == a->p) { a->alias = k; break; }
    a->in[0] = ir0; a->in[1] = ir1; a->in[2] = ic0; a->in[3] = ic1;
    a->out[0] = or0; a->out[1] = or1; a->out[2] = oc0; a->out[3] = oc1;
    a->snap_in = snap(a->p, esize, stride, a->in);
}

static void w8(uint8_t v) { fwrite(&v, 1, 1, g_rec); }
static void w16(int16_t v) { fwrite(&v, 2, 1, g_rec); }
static void w32(int32_t v) { fwrite(&v, 4, 1, g_rec); }
static void w64(int64_t v) { fwrite(&v, 8, 1, g_rec); }

static void rec_end(rec_t *r, int64_t ret)
{
    if (!r->on) return;
    for (int k = 0; k < r->n; k++)
        if (r->a[k].type == 'b') r->a[k].snap_out = snap(r->a[k].p, r->a[k].esize, r->a[k].stride, r->a[k].out);
    pthread_mutex_lock(&g_mu);
    w32((int32_t)EC_MAGIC);
    w16((int16_t)r->kind);
    w16((int16_t)r->slot);
    w32((int32_t)r->idx);
    w16((int16_t)r->n);
    w16(0);
    w64(ret);
    for (int k = 0; k < r->n; k++) {
        rarg_t *a = &r->a[k];
        w8((uint8_t)a->type);
        if (a->type != 'b') {
            w64(a->v);
            continue;
        }
        w8((uint8_t)a->esize);
        w8((uint8_t)((a->snap_in ? 1 : 0) | (a->snap_out ? 2 : 0)));
        w16((int16_t)a->alias);
        w64(a->stride);
        for (int j = 0; j < 4; j++) w32(a->in[j]);
        for (int j = 0; j < 4; j++) w32(a->out[j]);
        if (a->snap_in)
            fwrite(a->snap_in, 1, (size_t)(a->in[1] - a->in[0]) * (a->in[3] - a->in[2]) * a->esize, g_rec);
        if (a->snap_out)
            fwrite(a->snap_out, 1, (size_t)(a->out[1] - a->out[0]) * (a->out[3] - a->out[2]) * a->esize, g_rec);
        free(a->snap_in);
        free(a->snap_out);
    }
    pthread_mutex_unlock(&g_mu);
}

/* ---- wrappers, one per entry kind (argument regions follow what the
 * reference's C functions read and write: pixel.c, mc.c, intra.c,
 * transform.c, quant.c, filter_deblock.c, filter_sao.c) --------------------- */
#define NONE 0, 0, 0, 0

static cmp_dist_t w_cmp(int kind, int k, const pel_t *p1, intptr_t i1, const pel_t *p2, intptr_t i2)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, kind, k);
    rec_buf(&r, p1, 1, i1, 0, h, 0, w, NONE);
    rec_int(&r, 'p', i1);
    rec_buf(&r, p2, 1, i2, 0, h, 0, w, NONE);
    rec_int(&r, 'p', i2);
    cmp_dist_t v = kind == EC_SAD ? g_stock.pixf.sad[k](p1, i1, p2, i2)
                 : kind == EC_SATD ? g_stock.pixf.satd[k](p1, i1, p2, i2)
                 : kind == EC_SA8D ? g_stock.pixf.sa8d[k](p1, i1, p2, i2)
                 : (cmp_dist_t)g_stock.pixf.ssd[k](p1, i1, p2, i2);
    rec_end(&r, v);
    return v;
}

static void w_sad_x3(int k, const pel_t *f, const pel_t *a, const pel_t *b, const pel_t *c, intptr_t s, int res[3])
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_SAD_X3, k);
    rec_buf(&r, f, 1, FENC_STRIDE, 0, h, 0, w, NONE);
    rec_buf(&r, a, 1, s, 0, h, 0, w, NONE);
    rec_buf(&r, b, 1, s, 0, h, 0, w, NONE);
    rec_buf(&r, c, 1, s, 0, h, 0, w, NONE);
    rec_int(&r, 'p', s);
    rec_buf(&r, res, 4, 0, NONE, 0, 1, 0, 3);
    g_stock.pixf.sad_x3[k](f, a, b, c, s, res);
    rec_end(&r, 0);
}

static void w_sad_x4(int k, const pel_t *f, const pel_t *a, const pel_t *b, const pel_t *c, const pel_t *d,
                     intptr_t s, int res[4])
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_SAD_X4, k);
    rec_buf(&r, f, 1, FENC_STRIDE, 0, h, 0, w, NONE);
    rec_buf(&r, a, 1, s, 0, h, 0, w, NONE);
    rec_buf(&r, b, 1, s, 0, h, 0, w, NONE);
    rec_buf(&r, c, 1, s, 0, h, 0, w, NONE);
    rec_buf(&r, d, 1, s, 0, h, 0, w, NONE);
    rec_int(&r, 'p', s);
    rec_buf(&r, res, 4, 0, NONE, 0, 1, 0, 4);
    g_stock.pixf.sad_x4[k](f, a, b, c, d, s, res);
    rec_end(&r, 0);
}

static void w_sub_ps(int k, coeff_t *d, intptr_t sd, const pel_t *a, const pel_t *b, intptr_t sa, intptr_t sb)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_SUB_PS, k);
    rec_buf(&r, d, 2, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'p', sd);
    rec_buf(&r, a, 1, sa, 0, h, 0, w, NONE);
    rec_buf(&r, b, 1, sb, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sa);
    rec_int(&r, 'p', sb);
    g_stock.pixf.sub_ps[k](d, sd, a, b, sa, sb);
    rec_end(&r, 0);
}

static void w_add_ps(int k, pel_t *d, intptr_t sd, const pel_t *a, const coeff_t *b, intptr_t sa, intptr_t sb)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_ADD_PS, k);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'p', sd);
    rec_buf(&r, a, 1, sa, 0, h, 0, w, NONE);
    rec_buf(&r, b, 2, sb, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sa);
    rec_int(&r, 'p', sb);
    g_stock.pixf.add_ps[k](d, sd, a, b, sa, sb);
    rec_end(&r, 0);
}

#define W_COPY(NAME, KIND, DT, DS, ST, SS)                                                     \
    static void w_##NAME(int k, DT *d, intptr_t sd, const ST *s, intptr_t ss)                 \
    {                                                                                          \
        rec_t r;                                                                               \
        const int w = k_pw[k], h = k_ph[k];                                                    \
        rec_begin(&r, KIND, k);                                                                \
        rec_buf(&r, d, DS, sd, NONE, 0, h, 0, w);                                              \
        rec_int(&r, 'p', sd);                                                                  \
        rec_buf(&r, s, SS, ss, 0, h, 0, w, NONE);                                              \
        rec_int(&r, 'p', ss);                                                                  \
        g_stock.pixf.NAME[k](d, sd, s, ss);                                                    \
        rec_end(&r, 0);                                                                        \
    }
W_COPY(copy_sp, EC_COPY_SP, pel_t, 1, coeff_t, 2)
W_COPY(copy_ps, EC_COPY_PS, coeff_t, 2, pel_t, 1)
W_COPY(copy_ss, EC_COPY_SS, coeff_t, 2, coeff_t, 2)
W_COPY(copy_pp, EC_COPY_PP, pel_t, 1, pel_t, 1)

static void w_avg(int k, pel_t *d, intptr_t sd, const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb, int wt)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_AVG, k);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'p', sd);
    rec_buf(&r, a, 1, sa, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sa);
    rec_buf(&r, b, 1, sb, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sb);
    rec_int(&r, 'i', wt);
    g_stock.pixf.avg[k](d, sd, a, sa, b, sb, wt);
    rec_end(&r, 0);
}

static int w_mad(int k, pel_t *s, int is, int cs)
{
    rec_t r;
    rec_begin(&r, EC_MAD, k);
    rec_buf(&r, s, 1, is, 0, cs, 0, cs, NONE);
    rec_int(&r, 'i', is);
    rec_int(&r, 'i', cs);
    int v = g_stock.pixf.madf[k](s, is, cs);
    rec_end(&r, v);
    return v;
}

static dist_t w_ssd_block(const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb, int w, int h)
{
    rec_t r;
    rec_begin(&r, EC_SSD_BLOCK, 0);
    rec_buf(&r, a, 1, sa, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sa);
    rec_buf(&r, b, 1, sb, 0, h, 0, w, NONE);
    rec_int(&r, 'p', sb);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    dist_t v = g_stock.pixf.ssd_block(a, sa, b, sb, w, h);
    rec_end(&r, v);
    return v;
}

static void w_average(pel_t *d, int sd, pel_t *a, int sa, pel_t *b, int sb, int w, int h)
{
    rec_t r;
    rec_begin(&r, EC_AVERAGE, 0);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, a, 1, sa, 0, h, 0, w, NONE);
    rec_int(&r, 'i', sa);
    rec_buf(&r, b, 1, sb, 0, h, 0, w, NONE);
    rec_int(&r, 'i', sb);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    g_stock.pixf.average(d, sd, a, sa, b, sb, w, h);
    rec_end(&r, 0);
}

/* interpolation: 8-tap luma reads x-3..x+4, 4-tap chroma x-1..x+2 (mc.c:73-91) */
static void w_luma_hor(pel_t *d, int sd, mct_t *t, int st, pel_t *s, int ss, int w, int h, const int8_t *c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_HOR, 0);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, t, 2, st, NONE, 0, h, 0, w);
    rec_int(&r, 'i', st);
    rec_buf(&r, s, 1, ss, 0, h, -3, w + 4, NONE);
    rec_int(&r, 'i', ss);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_buf(&r, c, 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_hor(d, sd, t, st, s, ss, w, h, c);
    rec_end(&r, 0);
}

static void w_luma_ver(pel_t *d, int sd, pel_t *s, int ss, int w, int h, int8_t const *c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_VER, 0);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, s, 1, ss, -3, h + 4, 0, w, NONE);
    rec_int(&r, 'i', ss);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_buf(&r, c, 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_ver(d, sd, s, ss, w, h, c);
    rec_end(&r, 0);
}

static void w_luma_ext(pel_t *d, int sd, mct_t *t, int st, int w, int h, const int8_t *c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_EXT, 0);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, t, 2, st, -3, h + 4, 0, w, NONE);
    rec_int(&r, 'i', st);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_buf(&r, c, 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_ext(d, sd, t, st, w, h, c);
    rec_end(&r, 0);
}

static void w_luma_ver_x3(pel_t *const d[3], int sd, pel_t *s, int ss, int w, int h, int8_t const **c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_VER_X3, 0);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, d[k], 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, s, 1, ss, -3, h + 4, 0, w, NONE);
    rec_int(&r, 'i', ss);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, c[k], 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_ver_x3(d, sd, s, ss, w, h, c);
    rec_end(&r, 0);
}

static void w_luma_hor_x3(pel_t *const d[3], int sd, mct_t *const t[3], int st, pel_t *s, int ss, int w, int h,
                          const int8_t **c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_HOR_X3, 0);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, d[k], 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, t[k], 2, st, NONE, 0, h, 0, w);
    rec_int(&r, 'i', st);
    rec_buf(&r, s, 1, ss, 0, h, -3, w + 4, NONE);
    rec_int(&r, 'i', ss);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, c[k], 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_hor_x3(d, sd, t, st, s, ss, w, h, c);
    rec_end(&r, 0);
}

static void w_luma_ext_x3(pel_t *const d[3], int sd, mct_t *t, int st, int w, int h, const int8_t **c)
{
    rec_t r;
    rec_begin(&r, EC_LUMA_EXT_X3, 0);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, d[k], 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, t, 2, st, -3, h + 4, 0, w, NONE);
    rec_int(&r, 'i', st);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_arr(&r, 3);
    for (int k = 0; k < 3; k++) rec_buf(&r, c[k], 1, 0, 0, 1, 0, 8, NONE);
    g_stock.intpl_luma_ext_x3(d, sd, t, st, w, h, c);
    rec_end(&r, 0);
}

#define W_BLOCK(NAME, KIND, R0, R1, C0, C1, NT)                                                \
    static void w_##NAME(pel_t *d, int sd, pel_t *s, int ss, int w, int h, const int8_t *c)    \
    {                                                                                          \
        rec_t r;                                                                               \
        rec_begin(&r, KIND, 0);                                                                \
        rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);                                               \
        rec_int(&r, 'i', sd);                                                                  \
        rec_buf(&r, s, 1, ss, R0, R1, C0, C1, NONE);                                           \
        rec_int(&r, 'i', ss);                                                                  \
        rec_int(&r, 'i', w);                                                                   \
        rec_int(&r, 'i', h);                                                                   \
        rec_buf(&r, c, 1, 0, 0, 1, 0, NT, NONE);                                               \
        g_stock.NAME(d, sd, s, ss, w, h, c);                                                   \
        rec_end(&r, 0);                                                                        \
    }
W_BLOCK(intpl_luma_block_hor, EC_LUMA_BLOCK_HOR, 0, h, -3, w + 4, 8)
W_BLOCK(intpl_luma_block_ver, EC_LUMA_BLOCK_VER, -3, h + 4, 0, w, 8)
W_BLOCK(intpl_chroma_block_hor, EC_CHROMA_BLOCK_HOR, 0, h, -1, w + 2, 4)
W_BLOCK(intpl_chroma_block_ver, EC_CHROMA_BLOCK_VER, -1, h + 2, 0, w, 4)

#define W_BLOCK_EXT(NAME, KIND, M0, M1, NT)                                                    \
    static void w_##NAME(pel_t *d, int sd, pel_t *s, int ss, int w, int h, const int8_t *cx,   \
                         const int8_t *cy)                                                     \
    {                                                                                          \
        rec_t r;                                                                               \
        rec_begin(&r, KIND, 0);                                                                \
        rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);                                               \
        rec_int(&r, 'i', sd);                                                                  \
        rec_buf(&r, s, 1, ss, -(M0), h + (M1), -(M0), w + (M1), NONE);                         \
        rec_int(&r, 'i', ss);                                                                  \
        rec_int(&r, 'i', w);                                                                   \
        rec_int(&r, 'i', h);                                                                   \
        rec_buf(&r, cx, 1, 0, 0, 1, 0, NT, NONE);                                              \
        rec_buf(&r, cy, 1, 0, 0, 1, 0, NT, NONE);                                              \
        g_stock.NAME(d, sd, s, ss, w, h, cx, cy);                                              \
        rec_end(&r, 0);                                                                        \
    }
W_BLOCK_EXT(intpl_luma_block_ext, EC_LUMA_BLOCK_EXT, 3, 4, 8)
W_BLOCK_EXT(intpl_chroma_block_ext, EC_CHROMA_BLOCK_EXT, 1, 2, 4)

/* intra: the edge window around src the predictors may read (see the
 * header of the GPU library); dst is recorded before and after because mode
 * 31 on 16x64 leaves columns 4..15 as they were (intra.c). */
static void w_intra(int k, pel_t *src, pel_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    rec_t r;
    rec_begin(&r, EC_INTRA, k);
    rec_buf(&r, src, 1, 0, 0, 1, -(bsy + 11 * bsx / 4 + 6), bsx + 11 * bsy / 4 + 7, NONE);
    rec_buf(&r, dst, 1, i_dst, 0, bsy, 0, bsx, 0, bsy, 0, bsx);
    rec_int(&r, 'i', i_dst);
    rec_int(&r, 'i', dir_mode);
    rec_int(&r, 'i', bsx);
    rec_int(&r, 'i', bsy);
    g_stock.intraf[k](src, dst, i_dst, dir_mode, bsx, bsy);
    rec_end(&r, 0);
}

/* transforms: the 64-point shapes read a contiguous block and write
 * (w/2)x(h/2) coefficients (the rest of dst holds wavelet intermediates no
 * caller reads, transform.c:1505-1587); the other shapes use the stride
 * without its lowest bit (the wavelet flag). */
static int is64(int k) { return k == 4 || k == 23 || k == 24; }

static void w_dct(int kind, int k, const coeff_t *s, coeff_t *d, int is)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, kind, k);
    if (is64(k)) {
        rec_buf(&r, s, 2, w, 0, h, 0, w, NONE);
        rec_buf(&r, d, 2, 0, NONE, 0, 1, 0, w * h / 4);
    } else {
        rec_buf(&r, s, 2, is & ~1, 0, h, 0, w, NONE);
        rec_buf(&r, d, 2, 0, NONE, 0, 1, 0, w * h);
    }
    rec_int(&r, 'i', is);
    if (kind == EC_DCT) g_stock.dctf.dct[k](s, d, is);
    else g_stock.dctf.dct_half[k](s, d, is);
    rec_end(&r, 0);
}

static void w_idct(int k, const coeff_t *s, coeff_t *d, int id)
{
    rec_t r;
    const int w = k_pw[k], h = k_ph[k];
    rec_begin(&r, EC_IDCT, k);
    if (is64(k)) {
        rec_buf(&r, s, 2, 0, 0, 1, 0, w * h / 4, NONE);
        rec_buf(&r, d, 2, w, NONE, 0, h, 0, w);
    } else {
        rec_buf(&r, s, 2, 0, 0, 1, 0, w * h, NONE);
        rec_buf(&r, d, 2, id & ~1, NONE, 0, h, 0, w);
    }
    rec_int(&r, 'i', id);
    g_stock.dctf.idct[k](s, d, id);
    rec_end(&r, 0);
}

static void w_t4_2nd(int inv, coeff_t *c, int ic)
{
    rec_t r;
    rec_begin(&r, inv ? EC_INV_T4_2ND : EC_T4_2ND, 0);
    rec_buf(&r, c, 2, ic, 0, 4, 0, 4, 0, 4, 0, 4);
    rec_int(&r, 'i', ic);
    if (inv) g_stock.dctf.inv_transform_4x4_2nd(c, ic);
    else g_stock.dctf.transform_4x4_2nd(c, ic);
    rec_end(&r, 0);
}

static void w_t_2nd(int inv, coeff_t *c, int ic, int m, int t, int l)
{
    rec_t r;
    rec_begin(&r, inv ? EC_INV_T_2ND : EC_T_2ND, 0);
    rec_buf(&r, c, 2, ic, 0, 4, 0, 4, 0, 4, 0, 4);
    rec_int(&r, 'i', ic);
    rec_int(&r, 'i', m);
    rec_int(&r, 'i', t);
    rec_int(&r, 'i', l);
    if (inv) g_stock.dctf.inv_transform_2nd(c, ic, m, t, l);
    else g_stock.dctf.transform_2nd(c, ic, m, t, l);
    rec_end(&r, 0);
}

static void w_abs_coeff(coeff_t *d, const coeff_t *s, const int n)
{
    rec_t r;
    rec_begin(&r, EC_ABS_COEFF, 0);
    rec_buf(&r, d, 2, 0, NONE, 0, 1, 0, n);
    rec_buf(&r, s, 2, 0, 0, 1, 0, n, NONE);
    rec_int(&r, 'i', n);
    g_stock.dctf.abs_coeff(d, s, n);
    rec_end(&r, 0);
}

static int w_add_sign(coeff_t *d, const coeff_t *a, const int n)
{
    rec_t r;
    rec_begin(&r, EC_ADD_SIGN, 0);
    rec_buf(&r, d, 2, 0, 0, 1, 0, n, 0, 1, 0, n);
    rec_buf(&r, a, 2, 0, 0, 1, 0, n, NONE);
    rec_int(&r, 'i', n);
    int v = g_stock.dctf.add_sign(d, a, n);
    rec_end(&r, v);
    return v;
}

static int w_quant(coeff_t *c, const int n, const int sc, const int sh, const int add)
{
    rec_t r;
    rec_begin(&r, EC_QUANT, 0);
    rec_buf(&r, c, 2, 0, 0, 1, 0, n, 0, 1, 0, n);
    rec_int(&r, 'i', n);
    rec_int(&r, 'i', sc);
    rec_int(&r, 'i', sh);
    rec_int(&r, 'i', add);
    int v = g_stock.dctf.quant(c, n, sc, sh, add);
    rec_end(&r, v);
    return v;
}

static void w_dequant(coeff_t *c, const int n, const int sc, const int sh)
{
    rec_t r;
    rec_begin(&r, EC_DEQUANT, 0);
    rec_buf(&r, c, 2, 0, 0, 1, 0, n, 0, 1, 0, n);
    rec_int(&r, 'i', n);
    rec_int(&r, 'i', sc);
    rec_int(&r, 'i', sh);
    g_stock.dctf.dequant(c, n, sc, sh);
    rec_end(&r, 0);
}

static int w_wquant(coeff_t *c, const int n, const int sc, const int sh, const int add, int *ls)
{
    rec_t r;
    rec_begin(&r, EC_WQUANT, 0);
    rec_buf(&r, c, 2, 0, 0, 1, 0, n, 0, 1, 0, n);
    rec_int(&r, 'i', n);
    rec_int(&r, 'i', sc);
    rec_int(&r, 'i', sh);
    rec_int(&r, 'i', add);
    rec_buf(&r, ls, 4, 0, 0, 1, 0, n, NONE);
    int v = g_stock.dctf.wquant(c, n, sc, sh, add, ls);
    rec_end(&r, v);
    return v;
}

/* deblocking: 8 lines, 3 samples read on each side (lf_edge_core,
 * filter_deblock.c:292-380); [0] vertical edge, [1] horizontal edge */
static void w_dbk_luma(int dir, pel_t *s, int st, int a, int b, uint8_t *f)
{
    rec_t r;
    rec_begin(&r, EC_DEBLOCK_LUMA, dir);
    if (dir == 0) rec_buf(&r, s, 1, st, 0, 8, -3, 3, 0, 8, -3, 3);
    else rec_buf(&r, s, 1, st, -3, 3, 0, 8, -3, 3, 0, 8);
    rec_int(&r, 'i', st);
    rec_int(&r, 'i', a);
    rec_int(&r, 'i', b);
    rec_buf(&r, f, 1, 0, 0, 1, 0, 2, NONE);
    g_stock.deblock_luma[dir](s, st, a, b, f);
    rec_end(&r, 0);
}

static void w_dbk_chroma(int dir, pel_t *u, pel_t *v, int st, int a, int b, uint8_t *f)
{
    rec_t r;
    rec_begin(&r, EC_DEBLOCK_CHROMA, dir);
    if (dir == 0) {
        rec_buf(&r, u, 1, st, 0, 8, -3, 3, 0, 8, -3, 3);
        rec_buf(&r, v, 1, st, 0, 8, -3, 3, 0, 8, -3, 3);
    } else {
        rec_buf(&r, u, 1, st, -3, 3, 0, 8, -3, 3, 0, 8);
        rec_buf(&r, v, 1, st, -3, 3, 0, 8, -3, 3, 0, 8);
    }
    rec_int(&r, 'i', st);
    rec_int(&r, 'i', a);
    rec_int(&r, 'i', b);
    rec_buf(&r, f, 1, 0, 0, 1, 0, 2, NONE);
    g_stock.deblock_chroma[dir](u, v, st, a, b, f);
    rec_end(&r, 0);
}

/* SAO reads one sample around the block and writes inside it */
static void w_sao(pel_t *d, int sd, pel_t *s, int ss, int w, int h, int *avail, SAOBlkParam *prm)
{
    rec_t r;
    rec_begin(&r, EC_SAO, 0);
    rec_buf(&r, d, 1, sd, 0, h, 0, w, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_buf(&r, s, 1, ss, -1, h + 1, -1, w + 1, NONE);
    rec_int(&r, 'i', ss);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    rec_buf(&r, avail, 4, 0, 0, 1, 0, 8, NONE);
    rec_buf(&r, prm, 4, 0, 0, 1, 0, (int)(sizeof(SAOBlkParam) / 4), NONE);
    g_stock.sao_block(d, sd, s, ss, w, h, avail, prm);
    rec_end(&r, 0);
}

static void w_lowres(pel_t *s, int ss, pel_t *d, int sd, int w, int h)
{
    rec_t r;
    rec_begin(&r, EC_LOWRES, 0);
    rec_buf(&r, s, 1, ss, 0, 2 * h, 0, 2 * w, NONE);
    rec_int(&r, 'i', ss);
    rec_buf(&r, d, 1, sd, NONE, 0, h, 0, w);
    rec_int(&r, 'i', sd);
    rec_int(&r, 'i', w);
    rec_int(&r, 'i', h);
    g_stock.lowres_filter(s, ss, d, sd, w, h);
    rec_end(&r, 0);
}

/* ---- per-slot trampolines ---------------------------------------------- */
#define FOR25(X) X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) \
                 X(16) X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24)
#define FOR33(X) FOR25(X) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)
#define LIST25(P) {(void *)P##0, (void *)P##1, (void *)P##2, (void *)P##3, (void *)P##4, (void *)P##5,       \
                   (void *)P##6, (void *)P##7, (void *)P##8, (void *)P##9, (void *)P##10, (void *)P##11,    \
                   (void *)P##12, (void *)P##13, (void *)P##14, (void *)P##15, (void *)P##16,              \
                   (void *)P##17, (void *)P##18, (void *)P##19, (void *)P##20, (void *)P##21,              \
                   (void *)P##22, (void *)P##23, (void *)P##24}
#define LIST33(P) {(void *)P##0, (void *)P##1, (void *)P##2, (void *)P##3, (void *)P##4, (void *)P##5,       \
                   (void *)P##6, (void *)P##7, (void *)P##8, (void *)P##9, (void *)P##10, (void *)P##11,    \
                   (void *)P##12, (void *)P##13, (void *)P##14, (void *)P##15, (void *)P##16,              \
                   (void *)P##17, (void *)P##18, (void *)P##19, (void *)P##20, (void *)P##21,              \
                   (void *)P##22, (void *)P##23, (void *)P##24, (void *)P##25, (void *)P##26,              \
                   (void *)P##27, (void *)P##28, (void *)P##29, (void *)P##30, (void *)P##31, (void *)P##32}

#define TRAMP(k)                                                                                              \
    static cmp_dist_t t_sad_##k(const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb)                   \
    { return w_cmp(EC_SAD, k, a, sa, b, sb); }                                                               \
    static cmp_dist_t t_satd_##k(const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb)                  \
    { return w_cmp(EC_SATD, k, a, sa, b, sb); }                                                              \
    static cmp_dist_t t_sa8d_##k(const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb)                  \
    { return w_cmp(EC_SA8D, k, a, sa, b, sb); }                                                              \
    static dist_t t_ssd_##k(const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb)                       \
    { return w_cmp(EC_SSD, k, a, sa, b, sb); }                                                               \
    static void t_sadx3_##k(const pel_t *f, const pel_t *a, const pel_t *b, const pel_t *c, intptr_t s,     \
                            int res[3])                                                                      \
    { w_sad_x3(k, f, a, b, c, s, res); }                                                                     \
    static void t_sadx4_##k(const pel_t *f, const pel_t *a, const pel_t *b, const pel_t *c,                 \
                            const pel_t *d, intptr_t s, int res[4])                                          \
    { w_sad_x4(k, f, a, b, c, d, s, res); }                                                                  \
    static void t_subps_##k(coeff_t *d, intptr_t sd, const pel_t *a, const pel_t *b, intptr_t sa,           \
                            intptr_t sb)                                                                     \
    { w_sub_ps(k, d, sd, a, b, sa, sb); }                                                                    \
    static void t_addps_##k(pel_t *d, intptr_t sd, const pel_t *a, const coeff_t *b, intptr_t sa,           \
                            intptr_t sb)                                                                     \
    { w_add_ps(k, d, sd, a, b, sa, sb); }                                                                    \
    static void t_cpsp_##k(pel_t *d, intptr_t sd, const coeff_t *s, intptr_t ss) { w_copy_sp(k, d, sd, s, ss); } \
    static void t_cpps_##k(coeff_t *d, intptr_t sd, const pel_t *s, intptr_t ss) { w_copy_ps(k, d, sd, s, ss); } \
    static void t_cpss_##k(coeff_t *d, intptr_t sd, const coeff_t *s, intptr_t ss) { w_copy_ss(k, d, sd, s, ss); } \
    static void t_cppp_##k(pel_t *d, intptr_t sd, const pel_t *s, intptr_t ss) { w_copy_pp(k, d, sd, s, ss); }   \
    static void t_avg_##k(pel_t *d, intptr_t sd, const pel_t *a, intptr_t sa, const pel_t *b, intptr_t sb,  \
                          int wt)                                                                            \
    { w_avg(k, d, sd, a, sa, b, sb, wt); }                                                                   \
    static void t_dct_##k(const coeff_t *s, coeff_t *d, int i) { w_dct(EC_DCT, k, s, d, i); }                \
    static void t_idct_##k(const coeff_t *s, coeff_t *d, int i) { w_idct(k, s, d, i); }                      \
    static void t_dcth_##k(const coeff_t *s, coeff_t *d, int i) { w_dct(EC_DCT_HALF, k, s, d, i); }
FOR25(TRAMP)

#define TRAMP_INTRA(k)                                                                                        \
    static void t_intra_##k(pel_t *s, pel_t *d, int id, int m, int bx, int by) { w_intra(k, s, d, id, m, bx, by); }
FOR33(TRAMP_INTRA)

static int t_mad_0(pel_t *s, int is, int cs) { return w_mad(0, s, is, cs); }
static int t_mad_1(pel_t *s, int is, int cs) { return w_mad(1, s, is, cs); }
static int t_mad_2(pel_t *s, int is, int cs) { return w_mad(2, s, is, cs); }
static int t_mad_3(pel_t *s, int is, int cs) { return w_mad(3, s, is, cs); }
static void t_t4(coeff_t *c, int i) { w_t4_2nd(0, c, i); }
static void t_it4(coeff_t *c, int i) { w_t4_2nd(1, c, i); }
static void t_t2(coeff_t *c, int i, int m, int t, int l) { w_t_2nd(0, c, i, m, t, l); }
static void t_it2(coeff_t *c, int i, int m, int t, int l) { w_t_2nd(1, c, i, m, t, l); }
static void t_dbk_luma_0(pel_t *s, int st, int a, int b, uint8_t *f) { w_dbk_luma(0, s, st, a, b, f); }
static void t_dbk_luma_1(pel_t *s, int st, int a, int b, uint8_t *f) { w_dbk_luma(1, s, st, a, b, f); }
static void t_dbk_chroma_0(pel_t *u, pel_t *v, int st, int a, int b, uint8_t *f) { w_dbk_chroma(0, u, v, st, a, b, f); }
static void t_dbk_chroma_1(pel_t *u, pel_t *v, int st, int a, int b, uint8_t *f) { w_dbk_chroma(1, u, v, st, a, b, f); }

static void *const k_sad[25] = LIST25(t_sad_), *const k_satd[25] = LIST25(t_satd_), *const k_sa8d[25] = LIST25(t_sa8d_),
                   *const k_ssd[25] = LIST25(t_ssd_), *const k_sadx3[25] = LIST25(t_sadx3_),
                   *const k_sadx4[25] = LIST25(t_sadx4_), *const k_subps[25] = LIST25(t_subps_),
                   *const k_addps[25] = LIST25(t_addps_), *const k_cpsp[25] = LIST25(t_cpsp_),
                   *const k_cpps[25] = LIST25(t_cpps_), *const k_cpss[25] = LIST25(t_cpss_),
                   *const k_cppp[25] = LIST25(t_cppp_), *const k_avg[25] = LIST25(t_avg_),
                   *const k_dct[25] = LIST25(t_dct_), *const k_idct[25] = LIST25(t_idct_),
                   *const k_dcth[25] = LIST25(t_dcth_);
static void *const k_intra[33] = LIST33(t_intra_);
static void *const k_mad[4] = {(void *)t_mad_0, (void *)t_mad_1, (void *)t_mad_2, (void *)t_mad_3};

/* Address of the table member for (kind, slot); NULL if there is none. */
static void **member(intrinsic_func_t *t, int kind, int slot)
{
    const int s25 = slot >= 0 && slot < NUM_PU_SIZES;
    switch (kind) {
    case EC_SAD: return s25 ? (void **)&t->pixf.sad[slot] : NULL;
    case EC_SATD: return s25 ? (void **)&t->pixf.satd[slot] : NULL;
    case EC_SA8D: return s25 ? (void **)&t->pixf.sa8d[slot] : NULL;
    case EC_SSD: return s25 ? (void **)&t->pixf.ssd[slot] : NULL;
    case EC_SAD_X3: return s25 ? (void **)&t->pixf.sad_x3[slot] : NULL;
    case EC_SAD_X4: return s25 ? (void **)&t->pixf.sad_x4[slot] : NULL;
    case EC_SUB_PS: return s25 ? (void **)&t->pixf.sub_ps[slot] : NULL;
    case EC_ADD_PS: return s25 ? (void **)&t->pixf.add_ps[slot] : NULL;
    case EC_COPY_SP: return s25 ? (void **)&t->pixf.copy_sp[slot] : NULL;
    case EC_COPY_PS: return s25 ? (void **)&t->pixf.copy_ps[slot] : NULL;
    case EC_COPY_SS: return s25 ? (void **)&t->pixf.copy_ss[slot] : NULL;
    case EC_COPY_PP: return s25 ? (void **)&t->pixf.copy_pp[slot] : NULL;
    case EC_AVG: return s25 ? (void **)&t->pixf.avg[slot] : NULL;
    case EC_MAD: return slot >= 0 && slot < 4 ? (void **)&t->pixf.madf[slot] : NULL;
    case EC_SSD_BLOCK: return slot == 0 ? (void **)&t->pixf.ssd_block : NULL;
    case EC_AVERAGE: return slot == 0 ? (void **)&t->pixf.average : NULL;
    case EC_LUMA_HOR: return slot == 0 ? (void **)&t->intpl_luma_hor : NULL;
    case EC_LUMA_VER: return slot == 0 ? (void **)&t->intpl_luma_ver : NULL;
    case EC_LUMA_EXT: return slot == 0 ? (void **)&t->intpl_luma_ext : NULL;
    case EC_LUMA_VER_X3: return slot == 0 ? (void **)&t->intpl_luma_ver_x3 : NULL;
    case EC_LUMA_HOR_X3: return slot == 0 ? (void **)&t->intpl_luma_hor_x3 : NULL;
    case EC_LUMA_EXT_X3: return slot == 0 ? (void **)&t->intpl_luma_ext_x3 : NULL;
    case EC_LUMA_BLOCK_HOR: return slot == 0 ? (void **)&t->intpl_luma_block_hor : NULL;
    case EC_LUMA_BLOCK_VER: return slot == 0 ? (void **)&t->intpl_luma_block_ver : NULL;
    case EC_LUMA_BLOCK_EXT: return slot == 0 ? (void **)&t->intpl_luma_block_ext : NULL;
    case EC_CHROMA_BLOCK_HOR: return slot == 0 ? (void **)&t->intpl_chroma_block_hor : NULL;
    case EC_CHROMA_BLOCK_VER: return slot == 0 ? (void **)&t->intpl_chroma_block_ver : NULL;
    case EC_CHROMA_BLOCK_EXT: return slot == 0 ? (void **)&t->intpl_chroma_block_ext : NULL;
    case EC_INTRA: return slot >= 0 && slot < NUM_INTRA_MODE ? (void **)&t->intraf[slot] : NULL;
    case EC_DCT: return s25 ? (void **)&t->dctf.dct[slot] : NULL;
    case EC_IDCT: return s25 ? (void **)&t->dctf.idct[slot] : NULL;
    case EC_DCT_HALF: return s25 ? (void **)&t->dctf.dct_half[slot] : NULL;
    case EC_T4_2ND: return slot == 0 ? (void **)&t->dctf.transform_4x4_2nd : NULL;
    case EC_INV_T4_2ND: return slot == 0 ? (void **)&t->dctf.inv_transform_4x4_2nd : NULL;
    case EC_T_2ND: return slot == 0 ? (void **)&t->dctf.transform_2nd : NULL;
    case EC_INV_T_2ND: return slot == 0 ? (void **)&t->dctf.inv_transform_2nd : NULL;
    case EC_ABS_COEFF: return slot == 0 ? (void **)&t->dctf.abs_coeff : NULL;
    case EC_ADD_SIGN: return slot == 0 ? (void **)&t->dctf.add_sign : NULL;
    case EC_QUANT: return slot == 0 ? (void **)&t->dctf.quant : NULL;
    case EC_DEQUANT: return slot == 0 ? (void **)&t->dctf.dequant : NULL;
    case EC_WQUANT: return slot == 0 ? (void **)&t->dctf.wquant : NULL;
    case EC_DEBLOCK_LUMA: return slot == 0 || slot == 1 ? (void **)&t->deblock_luma[slot] : NULL;
    case EC_DEBLOCK_CHROMA: return slot == 0 || slot == 1 ? (void **)&t->deblock_chroma[slot] : NULL;
    case EC_SAO: return slot == 0 ? (void **)&t->sao_block : NULL;
    case EC_LOWRES: return slot == 0 ? (void **)&t->lowres_filter : NULL;
    default: return NULL;
    }
}

static void *recorder(int kind, int slot)
{
    switch (kind) {
    case EC_SAD: return k_sad[slot];
    case EC_SATD: return k_satd[slot];
    case EC_SA8D: return k_sa8d[slot];
    case EC_SSD: return k_ssd[slot];
    case EC_SAD_X3: return k_sadx3[slot];
    case EC_SAD_X4: return k_sadx4[slot];
    case EC_SUB_PS: return k_subps[slot];
    case EC_ADD_PS: return k_addps[slot];
    case EC_COPY_SP: return k_cpsp[slot];
    case EC_COPY_PS: return k_cpps[slot];
    case EC_COPY_SS: return k_cpss[slot];
    case EC_COPY_PP: return k_cppp[slot];
    case EC_AVG: return k_avg[slot];
    case EC_MAD: return k_mad[slot];
    case EC_SSD_BLOCK: return (void *)w_ssd_block;
    case EC_AVERAGE: return (void *)w_average;
    case EC_LUMA_HOR: return (void *)w_luma_hor;
    case EC_LUMA_VER: return (void *)w_luma_ver;
    case EC_LUMA_EXT: return (void *)w_luma_ext;
    case EC_LUMA_VER_X3: return (void *)w_luma_ver_x3;
    case EC_LUMA_HOR_X3: return (void *)w_luma_hor_x3;
    case EC_LUMA_EXT_X3: return (void *)w_luma_ext_x3;
    case EC_LUMA_BLOCK_HOR: return (void *)w_intpl_luma_block_hor;
    case EC_LUMA_BLOCK_VER: return (void *)w_intpl_luma_block_ver;
    case EC_LUMA_BLOCK_EXT: return (void *)w_intpl_luma_block_ext;
    case EC_CHROMA_BLOCK_HOR: return (void *)w_intpl_chroma_block_hor;
    case EC_CHROMA_BLOCK_VER: return (void *)w_intpl_chroma_block_ver;
    case EC_CHROMA_BLOCK_EXT: return (void *)w_intpl_chroma_block_ext;
    case EC_INTRA: return k_intra[slot];
    case EC_DCT: return k_dct[slot];
    case EC_IDCT: return k_idct[slot];
    case EC_DCT_HALF: return k_dcth[slot];
    case EC_T4_2ND: return (void *)t_t4;
    case EC_INV_T4_2ND: return (void *)t_it4;
    case EC_T_2ND: return (void *)t_t2;
    case EC_INV_T_2ND: return (void *)t_it2;
    case EC_ABS_COEFF: return (void *)w_abs_coeff;
    case EC_ADD_SIGN: return (void *)w_add_sign;
    case EC_QUANT: return (void *)w_quant;
    case EC_DEQUANT: return (void *)w_dequant;
    case EC_WQUANT: return (void *)w_wquant;
    case EC_DEBLOCK_LUMA: return slot ? (void *)t_dbk_luma_1 : (void *)t_dbk_luma_0;
    case EC_DEBLOCK_CHROMA: return slot ? (void *)t_dbk_chroma_1 : (void *)t_dbk_chroma_0;
    case EC_SAO: return (void *)w_sao;
    case EC_LOWRES: return (void *)w_lowres;
    default: return NULL;
    }
}

/* ---- the encode loop (test/test.c:125-199) ------------------------------ */
static int read_frame(FILE *f, xavs2_image_t *img)
{
    for (int k = 0; k < img->i_plane; k++)
        for (int j = 0; j < img->i_lines[k]; j++)
            if (fread(img->img_planes[k] + (size_t)img->i_stride[k] * j, (size_t)img->i_width[k], 1, f) != 1)
                return -1;
    return 0;
}

static void write_packet(const xavs2_api_t *api, void *enc, xavs2_outpacket_t *pkt, FILE *out)
{
    if (pkt->state == XAVS2_STATE_ENCODED || pkt->state == XAVS2_STATE_FLUSH_END) fwrite(pkt->stream, pkt->len, 1, out);
    api->encoder_packet_unref(enc, pkt);
}

int main(int argc, char **argv)
{
    if (argc < 4 || strcmp(argv[3], "--") != 0) {
        fprintf(stderr, "usage: %s plain|record|oracle RECORDS -- <xavs2 arguments>\n", argv[0]);
        return 2;
    }
    const char *mode = argv[1];
    const xavs2_api_t *api = xavs2_api_get(8);
    xavs2_param_t *param = api->opt_alloc();
    /* opt_set parses argv[1..]: hand it "prog <xavs2 arguments>" */
    argv[3] = argv[0];
    if (api->opt_set(param, argc - 3, argv + 3) < 0) {
        fprintf(stderr, "bad xavs2 arguments\n");
        return 2;
    }
    const char *in_file = api->opt_get(param, "input");
    const char *bs_file = api->opt_get(param, "output");
    int num_frames = atoi(api->opt_get(param, "frames"));
    FILE *in = fopen(in_file, "rb"), *out = fopen(bs_file, "wb");
    if (!in || !out) {
        fprintf(stderr, "cannot open %s or %s\n", in_file, bs_file);
        return 1;
    }
    void *enc = api->encoder_create(param);
    if (!enc) {
        fprintf(stderr, "encoder_create failed\n");
        return 1;
    }
    /* the table as the encoder set it up, then the requested replacement */
    memcpy(&g_stock, &g_funcs, sizeof(g_funcs));
    FILE *side = fopen(argv[2], "wb");
    if (!side) {
        fprintf(stderr, "cannot open %s\n", argv[2]);
        return 1;
    }
    if (!strcmp(mode, "record")) g_rec = side;
    int replaced = 0;
    for (int kind = 0; kind < EC_NUM_KINDS; kind++)
        for (int slot = 0; slot < EC_MAX_SLOTS; slot++) {
            void **m = member(&g_funcs, kind, slot);
            if (!m || !*m) continue;
            void *f = !strcmp(mode, "record") ? recorder(kind, slot) : !strcmp(mode, "oracle") ? xo_tab_entry(kind, slot)
                                                                                            : NULL;
            if (!f) continue;
            *m = f;
            replaced++;
            if (!strcmp(mode, "oracle")) fprintf(side, "%d %d\n", kind, slot);
        }
    fprintf(stderr, "%s: %d table entries replaced\n", mode, replaced);

    xavs2_picture_t pic;
    xavs2_outpacket_t pkt;
    memset(&pkt, 0, sizeof(pkt));
    for (int k = 0; k < num_frames; k++) {
        if (api->encoder_get_buffer(enc, &pic) < 0) break;
        if (read_frame(in, &pic.img) < 0) {
            pic.i_state = XAVS2_STATE_NO_DATA;
            api->encoder_encode(enc, &pic, &pkt);
            write_packet(api, enc, &pkt, out);
            break;
        }
        pic.i_state = 0;
        pic.i_type = XAVS2_TYPE_AUTO;
        pic.i_pts = k;
        api->encoder_encode(enc, &pic, &pkt);
        write_packet(api, enc, &pkt, out);
    }
    while (pkt.state != XAVS2_STATE_FLUSH_END) {
        api->encoder_encode(enc, NULL, &pkt);
        write_packet(api, enc, &pkt, out);
    }
    api->encoder_destroy(enc);
    fclose(in);
    fclose(out);
    if (g_rec) {
        /* trailer: the number of calls of every entry */
        w32(0x544e4358);   /* "XCNT" */
        w32(EC_NUM_KINDS);
        w32(EC_MAX_SLOTS);
        for (int kind = 0; kind < EC_NUM_KINDS; kind++)
            for (int slot = 0; slot < EC_MAX_SLOTS; slot++) w64((int64_t)g_calls[kind][slot]);
    }
    fclose(side);
    api->opt_destroy(param);
    return 0;
}
