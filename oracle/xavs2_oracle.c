/*
 * xavs2_oracle.c -- CPU restatement of the xavs2 encoder hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see xavs2_oracle.h).  Every function restates the
 * arithmetic of one reference routine; the citation in front of each one is
 * the reference file:line it follows (paths relative to the xavs2 source
 * tree).  The formulation is deliberately plain: SATD is computed as a sum
 * of absolute Hadamard coefficients over the reference's rounding units
 * instead of its SWAR packing, and the DCTs are direct matrix products built
 * from one cosine-magnitude table instead of partial butterflies; both are
 * exact integer identities for 8-bit input (checked against the reference
 * build in tests/test_oracle_vs_reference.py).
 */
#include "xavs2_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------
 * PU shapes, in LumaPU order (pixel.h:50-65)
 * ---------------------------------------------------------------------- */
static const uint8_t k_pu_w[25] = {4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32,
                                   16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16};
static const uint8_t k_pu_h[25] = {4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64,
                                   12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64};

int xo_num_parts(void) { return 25; }
int xo_part_width(int part) { return (part >= 0 && part < 25) ? k_pu_w[part] : 0; }
int xo_part_height(int part) { return (part >= 0 && part < 25) ? k_pu_h[part] : 0; }

/* PART_INDEX (pixel.h:178, table pixel.c:60-78) */
int xo_part_index(int w, int h)
{
    int i;
    for (i = 0; i < 25; i++) {
        if (k_pu_w[i] == w && k_pu_h[i] == h) return i;
    }
    return -1;
}

static inline int iabs(int v) { return v < 0 ? -v : v; }
static inline int clip3(int lo, int hi, int v) { return v < lo ? lo : (v > hi ? hi : v); }
static inline uint8_t clip_pel(int v) { return (uint8_t)clip3(0, 255, v); }

/* ------------------------------------------------------------------------
 * SAD / SSD (pixel.c:93-135, 537-592)
 * ---------------------------------------------------------------------- */
static int32_t sad_wh(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb, int w, int h)
{
    int32_t s = 0;
    int x, y;
    for (y = 0; y < h; y++, a += sa, b += sb)
        for (x = 0; x < w; x++) s += iabs(a[x] - b[x]);
    return s;
}

/* One SAD function per shape with the block size a compile-time constant,
 * as the reference instantiates them (PIXEL_SAD_C, pixel.c:93-135), so that
 * the compiler unrolls and vectorises the rows: the CPU baseline times this
 * port on hosts where the reference build is absent, and it must run at the
 * reference C's speed. */
#define SAD_FIXED(W, H)                                                                          \
    static int32_t sad_##W##x##H(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)   \
    {                                                                                            \
        int32_t s = 0;                                                                           \
        for (int y = 0; y < H; y++, a += sa, b += sb)                                            \
            for (int x = 0; x < W; x += 4) {                                                     \
                s += abs(a[x] - b[x]);                                                           \
                s += abs(a[x + 1] - b[x + 1]);                                                   \
                s += abs(a[x + 2] - b[x + 2]);                                                   \
                s += abs(a[x + 3] - b[x + 3]);                                                   \
            }                                                                                    \
        return s;                                                                                \
    }
SAD_FIXED(4, 4) SAD_FIXED(8, 8) SAD_FIXED(16, 16) SAD_FIXED(32, 32) SAD_FIXED(64, 64)
SAD_FIXED(8, 4) SAD_FIXED(4, 8) SAD_FIXED(16, 8) SAD_FIXED(8, 16) SAD_FIXED(32, 16) SAD_FIXED(16, 32)
SAD_FIXED(64, 32) SAD_FIXED(32, 64) SAD_FIXED(16, 12) SAD_FIXED(12, 16) SAD_FIXED(16, 4) SAD_FIXED(4, 16)
SAD_FIXED(32, 24) SAD_FIXED(24, 32) SAD_FIXED(32, 8) SAD_FIXED(8, 32) SAD_FIXED(64, 48) SAD_FIXED(48, 64)
SAD_FIXED(64, 16) SAD_FIXED(16, 64)
typedef int32_t (*sad_fn_t)(const uint8_t *, intptr_t, const uint8_t *, intptr_t);
static const sad_fn_t k_sad_fn[25] = {
    sad_4x4, sad_8x8, sad_16x16, sad_32x32, sad_64x64, sad_8x4, sad_4x8, sad_16x8, sad_8x16,
    sad_32x16, sad_16x32, sad_64x32, sad_32x64, sad_16x12, sad_12x16, sad_16x4, sad_4x16,
    sad_32x24, sad_24x32, sad_32x8, sad_8x32, sad_64x48, sad_48x64, sad_64x16, sad_16x64};

int32_t xo_sad(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    return k_sad_fn[part](p1, s1, p2, s2);
}

/* sad_x3 / sad_x4: the encode block always has stride FENC_STRIDE = 64
 * (pixel.c:143-243, common.h:1350). */
void xo_sad_x3(int part, const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,
               const uint8_t *r2, intptr_t i_ref, int32_t res[3])
{
    int w = k_pu_w[part], h = k_pu_h[part];
    res[0] = sad_wh(fenc, 64, r0, i_ref, w, h);
    res[1] = sad_wh(fenc, 64, r1, i_ref, w, h);
    res[2] = sad_wh(fenc, 64, r2, i_ref, w, h);
}

void xo_sad_x4(int part, const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,
               const uint8_t *r2, const uint8_t *r3, intptr_t i_ref, int32_t res[4])
{
    int w = k_pu_w[part], h = k_pu_h[part];
    res[0] = sad_wh(fenc, 64, r0, i_ref, w, h);
    res[1] = sad_wh(fenc, 64, r1, i_ref, w, h);
    res[2] = sad_wh(fenc, 64, r2, i_ref, w, h);
    res[3] = sad_wh(fenc, 64, r3, i_ref, w, h);
}

int32_t xo_ssd_block(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2, int w, int h)
{
    int32_t s = 0;
    int x, y;
    for (y = 0; y < h; y++, p1 += s1, p2 += s2)
        for (x = 0; x < w; x++) {
            int d = p1[x] - p2[x];
            s += d * d;
        }
    return s;
}

int32_t xo_ssd(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    return xo_ssd_block(p1, s1, p2, s2, k_pu_w[part], k_pu_h[part]);
}

/* ------------------------------------------------------------------------
 * Hadamard costs (pixel.c:297-530)
 *
 * hsum4/hsum8 return the unnormalised sum of |H D H^T| over one 4x4 or 8x8
 * difference block, H the +-1 Hadamard matrix.  The reference packs two
 * 16-bit lanes per word; for 8-bit samples no lane can overflow (the largest
 * lane sum is bounded by Parseval), so the plain sum is identical.
 * ---------------------------------------------------------------------- */
static void fwht4(int *v)
{
    int a = v[0] + v[1], b = v[0] - v[1], c = v[2] + v[3], d = v[2] - v[3];
    v[0] = a + c; v[1] = b + d; v[2] = a - c; v[3] = b - d;
}

static void fwht8(int *v)
{
    int t[8], i;
    for (i = 0; i < 4; i++) { t[i] = v[i] + v[i + 4]; t[i + 4] = v[i] - v[i + 4]; }
    fwht4(t); fwht4(t + 4);
    for (i = 0; i < 8; i++) v[i] = t[i];
}

static int hsum4(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)
{
    int d[4][4], col[4], s = 0, x, y;
    for (y = 0; y < 4; y++) {
        for (x = 0; x < 4; x++) d[y][x] = a[y * sa + x] - b[y * sb + x];
        fwht4(d[y]);
    }
    for (x = 0; x < 4; x++) {
        for (y = 0; y < 4; y++) col[y] = d[y][x];
        fwht4(col);
        for (y = 0; y < 4; y++) s += iabs(col[y]);
    }
    return s;
}

static int hsum8(const uint8_t *a, intptr_t sa, const uint8_t *b, intptr_t sb)
{
    int d[8][8], col[8], s = 0, x, y;
    for (y = 0; y < 8; y++) {
        for (x = 0; x < 8; x++) d[y][x] = a[y * sa + x] - b[y * sb + x];
        fwht8(d[y]);
    }
    for (x = 0; x < 8; x++) {
        for (y = 0; y < 8; y++) col[y] = d[y][x];
        fwht8(col);
        for (y = 0; y < 8; y++) s += iabs(col[y]);
    }
    return s;
}

/* SATD rounding units: shapes 4x4, 4x8, 4x16 and 12x16 tile in 4x4 units
 * rounded once each (pixel.c:297-322, 354-366, 404-407); every other shape
 * tiles in 8x4 units whose two 4x4 halves are summed before one rounding
 * (pixel.c:327-348, 371-403). */
static int satd_unit4(int w, int h) { return w == 4 || (w == 12 && h == 16); }

int32_t xo_satd(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    int32_t s = 0;
    if (satd_unit4(w, h)) {
        for (y = 0; y < h; y += 4)
            for (x = 0; x < w; x += 4)
                s += hsum4(p1 + y * s1 + x, s1, p2 + y * s2 + x, s2) >> 1;
    } else {
        for (y = 0; y < h; y += 4)
            for (x = 0; x < w; x += 8)
                s += (hsum4(p1 + y * s1 + x, s1, p2 + y * s2 + x, s2) +
                      hsum4(p1 + y * s1 + x + 4, s1, p2 + y * s2 + x + 4, s2)) >> 1;
    }
    return s;
}

/* SA8D: shapes with a 4-sample side alias SATD (pixel.c:508-514); 8x8-unit
 * shapes round each 8x8 with (s+2)>>2 (pixel.c:454-457, 477-489); the rest
 * round once per 16x16 (pixel.c:461-472, 494-506). */
int32_t xo_sa8d(int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    int32_t s = 0;
    int unit16;
    if (w == 4 || h == 4 || w == 12 || h == 12) return xo_satd(part, p1, s1, p2, s2);
    /* 8x16, 8x32, 16x8, 32x8, 32x24, 24x32 and 8x8 use 8x8 units */
    unit16 = !(w == 8 || h == 8 || (w == 32 && h == 24) || (w == 24 && h == 32));
    if (!unit16) {
        for (y = 0; y < h; y += 8)
            for (x = 0; x < w; x += 8)
                s += (hsum8(p1 + y * s1 + x, s1, p2 + y * s2 + x, s2) + 2) >> 2;
    } else {
        for (y = 0; y < h; y += 16)
            for (x = 0; x < w; x += 16) {
                int t = hsum8(p1 + y * s1 + x, s1, p2 + y * s2 + x, s2) +
                        hsum8(p1 + y * s1 + x + 8, s1, p2 + y * s2 + x + 8, s2) +
                        hsum8(p1 + (y + 8) * s1 + x, s1, p2 + (y + 8) * s2 + x, s2) +
                        hsum8(p1 + (y + 8) * s1 + x + 8, s1, p2 + (y + 8) * s2 + x + 8, s2);
                s += (t + 2) >> 2;
            }
    }
    return s;
}

/* ------------------------------------------------------------------------
 * block ops (pixel.c:680-856)
 * ---------------------------------------------------------------------- */
void xo_avg(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *a, intptr_t i_a,
            const uint8_t *b, intptr_t i_b)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    for (y = 0; y < h; y++, dst += i_dst, a += i_a, b += i_b)
        for (x = 0; x < w; x++) dst[x] = (uint8_t)((a[x] + b[x] + 1) >> 1);
}

void xo_average(uint8_t *dst, int i_dst, const uint8_t *a, int i_a, const uint8_t *b, int i_b,
                int w, int h)
{
    int x, y;
    for (y = 0; y < h; y++, dst += i_dst, a += i_a, b += i_b)
        for (x = 0; x < w; x++) dst[x] = (uint8_t)((a[x] + b[x] + 1) >> 1);
}

void xo_sub_ps(int part, int16_t *dst, intptr_t i_dst, const uint8_t *a, const uint8_t *b,
               intptr_t i_a, intptr_t i_b)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    for (y = 0; y < h; y++, dst += i_dst, a += i_a, b += i_b)
        for (x = 0; x < w; x++) dst[x] = (int16_t)(a[x] - b[x]);
}

void xo_add_ps(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *a, const int16_t *b,
               intptr_t i_a, intptr_t i_b)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    for (y = 0; y < h; y++, dst += i_dst, a += i_a, b += i_b)
        for (x = 0; x < w; x++) dst[x] = clip_pel(a[x] + b[x]);
}

void xo_copy_pp(int part, uint8_t *dst, intptr_t i_dst, const uint8_t *src, intptr_t i_src)
{
    int w = k_pu_w[part], h = k_pu_h[part], y;
    for (y = 0; y < h; y++) memcpy(dst + y * i_dst, src + y * i_src, (size_t)w);
}

void xo_copy_ps(int part, int16_t *dst, intptr_t i_dst, const uint8_t *src, intptr_t i_src)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++) dst[y * i_dst + x] = (int16_t)src[y * i_src + x];
}

void xo_copy_sp(int part, uint8_t *dst, intptr_t i_dst, const int16_t *src, intptr_t i_src)
{
    int w = k_pu_w[part], h = k_pu_h[part], x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++) dst[y * i_dst + x] = (uint8_t)src[y * i_src + x];
}

void xo_copy_ss(int part, int16_t *dst, intptr_t i_dst, const int16_t *src, intptr_t i_src)
{
    int w = k_pu_w[part], h = k_pu_h[part], y;
    for (y = 0; y < h; y++) memcpy(dst + y * i_dst, src + y * i_src, (size_t)w * 2);
}

/* mad_NxN_c (pixel.c:1620-1649): rounded mean, then sum of |p - mean| */
int xo_mad(const uint8_t *src, int i_src, int cu_size)
{
    int n = cu_size * cu_size, sum = 0, mean, mad = 0, x, y;
    for (y = 0; y < cu_size; y++)
        for (x = 0; x < cu_size; x++) sum += src[y * i_src + x];
    mean = (sum + (n >> 1)) / n;
    for (y = 0; y < cu_size; y++)
        for (x = 0; x < cu_size; x++) mad += iabs(src[y * i_src + x] - mean);
    return mad;
}

/* ------------------------------------------------------------------------
 * interpolation (mc.c:73-91 taps, 275-547 filters, 593-744 frame planes)
 * ---------------------------------------------------------------------- */
/* AVS2 luma 8-tap (quarter-pel) and chroma 4-tap (eighth-pel) filters, as
 * fixed by the standard. */
static const int8_t k_luma_taps[4][8] = {
    {0, 0, 0, 64, 0, 0, 0, 0},
    {-1, 4, -10, 57, 19, -7, 3, -1},
    {-1, 4, -11, 40, 40, -11, 4, -1},
    {-1, 3, -7, 19, 57, -10, 4, -1},
};
static const int8_t k_chroma_taps[8][4] = {
    {0, 64, 0, 0},   {-4, 62, 6, 0},   {-6, 56, 15, -1}, {-5, 47, 25, -3},
    {-4, 36, 36, -4}, {-3, 25, 47, -5}, {-1, 15, 56, -6}, {0, 6, 62, -4},
};

const int8_t *xo_luma_filter(int frac) { return k_luma_taps[frac & 3]; }
const int8_t *xo_chroma_filter(int frac) { return k_chroma_taps[frac & 7]; }

/* 8 taps over p[-3*step .. +4*step] */
static inline int tap8(const uint8_t *p, intptr_t step, const int8_t *c)
{
    int k, s = 0;
    for (k = 0; k < 8; k++) s += c[k] * p[(k - 3) * step];
    return s;
}
static inline int tap8s(const int16_t *p, intptr_t step, const int8_t *c)
{
    int k, s = 0;
    for (k = 0; k < 8; k++) s += c[k] * p[(k - 3) * step];
    return s;
}
static inline int tap4(const uint8_t *p, intptr_t step, const int8_t *c)
{
    int k, s = 0;
    for (k = 0; k < 4; k++) s += c[k] * p[(k - 1) * step];
    return s;
}

/* intpl_luma_hor_c (mc.c:403-417): raw sum to tmp, rounded sample to dst */
void xo_intpl_luma_hor(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, const uint8_t *src,
                       int i_src, int w, int h, const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++) {
            int v = tap8(src + y * i_src + x, 1, coef);
            tmp[y * i_tmp + x] = (int16_t)v;
            dst[y * i_dst + x] = clip_pel((v + 32) >> 6);
        }
}

/* intpl_luma_ver_c (mc.c:422-435); also the block vertical filter (358) */
void xo_intpl_luma_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w, int h,
                       const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap8(src + y * i_src + x, i_src, coef) + 32) >> 6);
}

/* intpl_luma_ext_c (mc.c:501-516): vertical pass over the int16 raw sums */
void xo_intpl_luma_ext(uint8_t *dst, int i_dst, const int16_t *tmp, int i_tmp, int w, int h,
                       const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap8s(tmp + y * i_tmp + x, i_tmp, coef) + 2048) >> 12);
}

/* intpl_luma_block_hor_c (mc.c:342-354) */
void xo_intpl_luma_block_hor(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap8(src + y * i_src + x, 1, coef) + 32) >> 6);
}

void xo_intpl_luma_block_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef)
{
    xo_intpl_luma_ver(dst, i_dst, src, i_src, w, h, coef);
}

/* intpl_luma_block_ext_c (mc.c:362-398): int16 raw horizontal sums over
 * rows -3..h+3, then a vertical pass with +2048 >> 12 */
void xo_intpl_luma_block_ext(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                             int h, const int8_t *coef_x, const int8_t *coef_y)
{
    int16_t tmp[(64 + 7) * 64];
    int x, y;
    for (y = -3; y < h + 4; y++)
        for (x = 0; x < w; x++) tmp[(y + 3) * 64 + x] = (int16_t)tap8(src + y * i_src + x, 1, coef_x);
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap8s(tmp + (y + 3) * 64 + x, 64, coef_y) + 2048) >> 12);
}

/* intpl_chroma_block_{hor,ver,ext}_c (mc.c:274-337) */
void xo_intpl_chroma_block_hor(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap4(src + y * i_src + x, 1, coef) + 32) >> 6);
}

void xo_intpl_chroma_block_ver(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef)
{
    int x, y;
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++)
            dst[y * i_dst + x] = clip_pel((tap4(src + y * i_src + x, i_src, coef) + 32) >> 6);
}

void xo_intpl_chroma_block_ext(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w,
                               int h, const int8_t *coef_x, const int8_t *coef_y)
{
    int32_t tmp[(32 + 3) * 32];
    int x, y, k;
    for (y = -1; y < h + 2; y++)
        for (x = 0; x < w; x++) tmp[(y + 1) * 32 + x] = tap4(src + y * i_src + x, 1, coef_x);
    for (y = 0; y < h; y++)
        for (x = 0; x < w; x++) {
            int s = 0;
            for (k = 0; k < 4; k++) s += coef_y[k] * tmp[(y + k) * 32 + x];
            dst[y * i_dst + x] = clip_pel((s + 2048) >> 12);
        }
}

/* Frame sub-pel planes (mc.c:593-744, frame.c:471-507).  The reference
 * filters rows [-4, H+4) x cols [-4, W+4) of each plane and then replicates
 * that region's edge outwards; every filtered sample is therefore the filter
 * evaluated at the position clamped into that region, with full-pel reads
 * clamped into the picture (the padding of the source plane).  This routine
 * states exactly that: value(x, y) = F(clamp(x,-4,W+3), clamp(y,-4,H+3)). */
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static int hraw(const uint8_t *src, int stride, int w, int h, int x, int y, int fx)
{
    const int8_t *c = k_luma_taps[fx];
    int k, s = 0, yy = clampi(y, 0, h - 1);
    for (k = 0; k < 8; k++) s += c[k] * src[yy * stride + clampi(x + k - 3, 0, w - 1)];
    return (int16_t)s;
}

static uint8_t subpel_sample(const uint8_t *src, int stride, int w, int h, int x, int y, int fx, int fy)
{
    int k, s = 0;
    if (fy == 0) return clip_pel((hraw(src, stride, w, h, x, y, fx) + 32) >> 6);
    if (fx == 0) {
        const int8_t *c = k_luma_taps[fy];
        int xx = clampi(x, 0, w - 1);
        for (k = 0; k < 8; k++) s += c[k] * src[clampi(y + k - 3, 0, h - 1) * stride + xx];
        return clip_pel((s + 32) >> 6);
    }
    for (k = 0; k < 8; k++) s += k_luma_taps[fy][k] * hraw(src, stride, w, h, x, y + k - 3, fx);
    return clip_pel((s + 2048) >> 12);
}

void xo_interpolate_frame(uint8_t *const planes[16], const uint8_t *src, int stride,
                          int width, int height, int pad, int mode)
{
    int k, x, y;
    for (k = 1; k < 16; k++) {
        int fx = k & 3, fy = k >> 2;
        uint8_t *dst = planes[k];
        if (mode < 2 && !(k == 2 || k == 8 || k == 10)) continue;
        if (dst == NULL) continue;
        /* interior of the filtered region, then replicate outwards */
        for (y = -4; y < height + 4; y++)
            for (x = -4; x < width + 4; x++)
                dst[y * stride + x] = subpel_sample(src, stride, width, height, x, y, fx, fy);
        for (y = -pad; y < height + pad; y++) {
            int yy = clampi(y, -4, height + 3);
            for (x = -pad; x < width + pad; x++) {
                int xx = clampi(x, -4, width + 3);
                if (xx != x || yy != y) dst[y * stride + x] = dst[yy * stride + xx];
            }
        }
    }
}

void xo_expand_border(uint8_t *pix, int stride, int width, int height, int pad)
{
    int x, y;
    for (y = -pad; y < height + pad; y++) {
        int yy = clampi(y, 0, height - 1);
        for (x = -pad; x < width + pad; x++) {
            int xx = clampi(x, 0, width - 1);
            if (xx != x || yy != y) pix[y * stride + x] = pix[yy * stride + xx];
        }
    }
}

/* ------------------------------------------------------------------------
 * integer DCT (transform.c:59-135 basis, 167-582 passes, 1123-1587 sizes)
 *
 * Every AVS2 DCT basis entry is +-c[a] for the reduced angle
 * a = k(2n+1) mod 128 (units of pi/64); the N-point matrices are the rows
 * k*32/N of the 32-point one.  A pass is the exact integer product
 * sum_n T[k][n] x[n] followed by the pass's rounding shift, which is what the
 * partial butterflies compute.
 * ---------------------------------------------------------------------- */
static const int8_t k_avs2_cos[32] = {32, 45, 45, 45, 44, 44, 43, 43, 42, 41, 40,
                                      39, 38, 36, 35, 34, 32, 30, 29, 27, 25, 23,
                                      21, 19, 17, 15, 13, 11, 9,  7,  4,  2};

static int basis32(int k, int n)
{
    int a = (k * (2 * n + 1)) % 128, s = 1;
    if (k == 0) return 32;
    if (a > 64) a = 128 - a;
    if (a > 32) { a = 64 - a; s = -1; }
    return s * k_avs2_cos[a];
}

/* T_N[k][n] */
static inline int basis(int N, int k, int n) { return basis32(k * (32 / N), n); }

/* forward pass over `lines` vectors of length N (stride `in_stride` between
 * vectors, unit stride inside), writing coefficient k of vector j to
 * out[k * lines + j] with int16 wrap */
static void fwd_pass(const int16_t *in, int in_stride, int16_t *out, int N, int lines, int shift)
{
    int j, k, n;
    int add = (1 << shift) >> 1;
    for (j = 0; j < lines; j++)
        for (k = 0; k < N; k++) {
            int s = 0;
            for (n = 0; n < N; n++) s += basis(N, k, n) * in[j * in_stride + n];
            out[k * lines + j] = (int16_t)((s + add) >> shift);
        }
}

/* inverse pass: vector j's coefficients are in[k * lines + j]; sample n goes
 * to out[j * N + n], clipped to a signed `bits`-bit range */
static void inv_pass(const int16_t *in, int16_t *out, int N, int lines, int shift, int bits)
{
    int j, k, n;
    int add = (1 << shift) >> 1;
    int hi = (1 << (bits - 1)) - 1, lo = -hi - 1;
    for (j = 0; j < lines; j++)
        for (n = 0; n < N; n++) {
            int s = 0;
            for (k = 0; k < N; k++) s += basis(N, k, n) * in[k * lines + j];
            out[j * N + n] = (int16_t)clip3(lo, hi, (s + add) >> shift);
        }
}

/* 2-D forward DCT of a w x h block: rows first (length w), then columns. */
static void dct2d(const int16_t *src, int i_src, int16_t *dst, int w, int h, int s1, int s2)
{
    int16_t blk[64 * 64], mid[64 * 64];
    int y;
    for (y = 0; y < h; y++) memcpy(blk + y * w, src + y * i_src, (size_t)w * 2);
    fwd_pass(blk, w, mid, w, h, s1);  /* mid[k][j]: row j, horizontal freq k */
    fwd_pass(mid, h, dst, h, w, s2);  /* dst[m][k] */
}

/* 2-D inverse DCT: columns first (length h), then rows (length w). */
static void idct2d(const int16_t *src, int16_t *dst, int i_dst, int w, int h, int s2, int bits2)
{
    int16_t mid[64 * 64], blk[64 * 64];
    int y;
    inv_pass(src, mid, h, w, 5, 16);    /* mid[j][n]: column j, row n */
    inv_pass(mid, blk, w, h, s2, bits2);
    for (y = 0; y < h; y++) memcpy(dst + y * i_dst, blk + y * w, (size_t)w * 2);
}

/* 5/3 lifting wavelet that halves a w x h block to its low band
 * (transform.c:586-783).  The reference stores every lifted sample as
 * coeff_t, hence the int16 casts. */
static void lift_fwd(int16_t *v, int n, int vertical)
{
    int16_t e[64 + 4], *p = e + 2;
    int i;
    memcpy(p, v, (size_t)n * 2);
    p[-1] = p[1]; p[-2] = p[2]; p[n] = p[n - 2]; p[n + 1] = p[n - 3];
    for (i = -1; i < n; i += 2) p[i] = (int16_t)(p[i] - ((p[i - 1] + p[i + 1]) >> 1));
    for (i = 0; i < n; i += 2) {
        if (vertical)
            p[i] = (int16_t)((p[i] << 1) + ((p[i - 1] + p[i + 1] + 1) >> 1));
        else
            p[i] = (int16_t)(p[i] + ((p[i - 1] + p[i + 1] + 2) >> 2));
    }
    for (i = 0; i < n / 2; i++) v[i] = p[2 * i];
}

static void wavelet_fwd(const int16_t *src, int16_t *ll, int w, int h)
{
    int16_t rows[64 * 64], col[64];
    int x, y;
    for (y = 0; y < h; y++) {
        int16_t r[64];
        memcpy(r, src + y * w, (size_t)w * 2);
        lift_fwd(r, w, 0);
        memcpy(rows + y * (w / 2), r, (size_t)(w / 2) * 2);
    }
    for (x = 0; x < w / 2; x++) {
        for (y = 0; y < h; y++) col[y] = rows[y * (w / 2) + x];
        lift_fwd(col, h, 1);
        for (y = 0; y < h / 2; y++) ll[y * (w / 2) + x] = col[y];
    }
}

/* inverse wavelet (transform.c:787-951): vertical upsampling halves the
 * low-band samples and averages between them; horizontal upsampling only
 * averages.  The last odd sample mirrors the last even one. */
static void lift_inv(const int16_t *in, int16_t *out, int n, int halve)
{
    int16_t p[64 + 2];
    int i;
    for (i = 0; i < n / 2; i++) p[2 * i] = in[i];
    p[n] = p[n - 2];
    if (halve)
        for (i = 0; i <= n; i += 2) p[i] = (int16_t)(p[i] >> 1);
    for (i = 1; i < n; i += 2) p[i] = (int16_t)((p[i - 1] + p[i + 1]) >> 1);
    memcpy(out, p, (size_t)n * 2);
}

static void wavelet_inv(const int16_t *ll, int16_t *dst, int w, int h)
{
    int16_t cols[64 * 64], in[64], out[64];
    int x, y;
    for (x = 0; x < w / 2; x++) {
        for (y = 0; y < h / 2; y++) in[y] = ll[y * (w / 2) + x];
        lift_inv(in, out, h, 1);
        for (y = 0; y < h; y++) cols[y * (w / 2) + x] = out[y];
    }
    for (y = 0; y < h; y++) lift_inv(cols + y * (w / 2), dst + y * w, w, 0);
}

int xo_is_tu_shape(int part)
{
    switch (part) {
    case 0: case 1: case 2: case 3: case 4:   /* squares */
    case 15: case 16: case 19: case 20:       /* 16x4 4x16 32x8 8x32 */
    case 23: case 24:                         /* 64x16 16x64 */
        return 1;
    default:
        return 0;
    }
}

/* Forward shifts per size for 8-bit input: shift1 = log2(N_row)+5+9-16 with
 * the asymmetric -2 adjustments and the wavelet flag (low bit of the stride)
 * of dct_32x32/32x8/8x32 (transform.c:1123-1587). */
void xo_dct(int part, const int16_t *src, int16_t *dst, int i_src)
{
    int flag = i_src & 1;
    int16_t ll[32 * 32];
    switch (part) {
    case 0: dct2d(src, i_src, dst, 4, 4, 0, 7); break;
    case 1: dct2d(src, i_src, dst, 8, 8, 1, 8); break;
    case 2: dct2d(src, i_src, dst, 16, 16, 2, 9); break;
    case 3: dct2d(src, i_src & 0xFE, dst, 32, 32, 3 + flag, 10); break;
    case 15: dct2d(src, i_src, dst, 16, 4, 2, 7); break;      /* 16x4 */
    case 16: dct2d(src, i_src, dst, 4, 16, 0, 9); break;      /* 4x16 */
    case 19: dct2d(src, i_src & 0xFE, dst, 32, 8, 3, 8 - flag); break;   /* 32x8 */
    case 20: dct2d(src, i_src & 0xFE, dst, 8, 32, 1 + flag, 10); break;  /* 8x32 */
    case 4:  /* 64x64: wavelet to 32x32 (input contiguous, stride 64) */
        wavelet_fwd(src, ll, 64, 64);
        dct2d(ll, 32, dst, 32, 32, 4, 10);
        break;
    case 23: /* 64x16 -> 32x8 */
        wavelet_fwd(src, ll, 64, 16);
        dct2d(ll, 32, dst, 32, 8, 3, 7);
        break;
    case 24: /* 16x64 -> 8x32 */
        wavelet_fwd(src, ll, 16, 64);
        dct2d(ll, 8, dst, 8, 32, 2, 10);
        break;
    default: break;
    }
}

/* dct_32x32_half_c (transform.c:1276-1286): keep the top-left 16x16 */
void xo_dct_half(int part, const int16_t *src, int16_t *dst, int i_src)
{
    int y;
    if (part != 3 && part != 4) return;   /* only 32x32 and 64x64 have one */
    xo_dct(part, src, dst, part == 4 ? 64 : i_src);
    for (y = 0; y < 32; y++) {
        if (y < 16) memset(dst + y * 32 + 16, 0, 16 * 2);
        else memset(dst + y * 32, 0, 32 * 2);
    }
}

/* Inverse: shift 5 with a 16-bit clip, then shift 12 with a 9-bit clip, one
 * less shift and one more clip bit under the wavelet flag. */
void xo_idct(int part, const int16_t *src, int16_t *dst, int i_dst)
{
    int flag = i_dst & 1;
    int16_t ll[32 * 32];
    switch (part) {
    case 0: idct2d(src, dst, i_dst, 4, 4, 12, 9); break;
    case 1: idct2d(src, dst, i_dst, 8, 8, 12, 9); break;
    case 2: idct2d(src, dst, i_dst, 16, 16, 12, 9); break;
    case 3: idct2d(src, dst, i_dst & 0xFE, 32, 32, 12 - flag, 9 + flag); break;
    case 15: idct2d(src, dst, i_dst, 16, 4, 12, 9); break;
    case 16: idct2d(src, dst, i_dst, 4, 16, 12, 9); break;
    case 19: idct2d(src, dst, i_dst & 0xFE, 32, 8, 12 - flag, 9 + flag); break;
    case 20: idct2d(src, dst, i_dst & 0xFE, 8, 32, 12 - flag, 9 + flag); break;
    case 4:
        idct2d(src, ll, 32, 32, 32, 11, 10);
        wavelet_inv(ll, dst, 64, 64);
        break;
    case 23:
        idct2d(src, ll, 32, 32, 8, 11, 10);
        wavelet_inv(ll, dst, 64, 16);
        break;
    case 24:
        idct2d(src, ll, 8, 8, 32, 11, 10);
        wavelet_inv(ll, dst, 16, 64);
        break;
    default: break;
    }
}

/* ------------------------------------------------------------------------
 * secondary transforms (transform.c:140-155 matrices, 962-1119)
 * ---------------------------------------------------------------------- */
static const int16_t k_sec_mode[16] = {123, -35, -8, -3, -32, -120, 30, 10,
                                       14, 25, 123, -22, 8, 13, 19, 126};
static const int16_t k_sec_4x4[16] = {34, 58, 72, 81, 77, 69, -7, -75,
                                      79, -33, -75, 58, 55, -84, 73, -28};

/* Y = M X (M^T when transposed), on the 4x4 corner of a strided block;
 * `rows` selects whether the transform runs along rows (X M^T) or columns. */
static void sec_apply(int16_t *c, int stride, const int16_t *m, int transposed, int along_rows,
                      int shift, int bits)
{
    int x[4][4], i, j, k;
    int add = (1 << shift) >> 1;
    int hi = (1 << (bits - 1)) - 1, lo = -hi - 1;
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++) x[i][j] = c[i * stride + j];
    for (i = 0; i < 4; i++)
        for (j = 0; j < 4; j++) {
            int s = add;
            for (k = 0; k < 4; k++) {
                int mk = transposed ? m[k * 4 + i] : m[i * 4 + k];
                s += mk * (along_rows ? x[j][k] : x[k][j]);
            }
            if (along_rows) c[j * stride + i] = (int16_t)clip3(lo, hi, s >> shift);
            else c[i * stride + j] = (int16_t)clip3(lo, hi, s >> shift);
        }
}

void xo_transform_4x4_2nd(int16_t *coef, int i_coef)
{
    sec_apply(coef, i_coef, k_sec_4x4, 0, 1, 1, 16);
    sec_apply(coef, i_coef, k_sec_4x4, 0, 0, 8, 16);
}

void xo_inv_transform_4x4_2nd(int16_t *coef, int i_coef)
{
    sec_apply(coef, i_coef, k_sec_4x4, 1, 0, 5, 16);
    sec_apply(coef, i_coef, k_sec_4x4, 1, 1, 14, 9);
}

static void sec_dirs(int i_mode, int *vt, int *ht)
{
    *vt = (i_mode >= 0 && i_mode <= 23);
    *ht = (i_mode >= 13 && i_mode <= 32) || (i_mode >= 0 && i_mode <= 2);
}

void xo_transform_2nd(int16_t *coef, int i_coef, int i_mode, int b_top, int b_left)
{
    int vt, ht;
    sec_dirs(i_mode, &vt, &ht);
    if (vt && b_top) sec_apply(coef, i_coef, k_sec_mode, 0, 0, 7, 16);
    if (ht && b_left) sec_apply(coef, i_coef, k_sec_mode, 0, 1, 7, 16);
}

void xo_inv_transform_2nd(int16_t *coef, int i_coef, int i_mode, int b_top, int b_left)
{
    int vt, ht;
    sec_dirs(i_mode, &vt, &ht);
    if (ht && b_left) sec_apply(coef, i_coef, k_sec_mode, 1, 1, 7, 16);
    if (vt && b_top) sec_apply(coef, i_coef, k_sec_mode, 1, 0, 7, 16);
}

/* ------------------------------------------------------------------------
 * quantisation (quant.c:55-184; rdo.c:659-759 for the parameters)
 * ---------------------------------------------------------------------- */
static const uint16_t k_q_scale[80] = {
    32768, 29775, 27554, 25268, 23170, 21247, 19369, 17770, 16302, 15024, 13777, 12634,
    11626, 10624, 9742,  8958,  8192,  7512,  6889,  6305,  5793,  5303,  4878,  4467,
    4091,  3756,  3444,  3161,  2894,  2654,  2435,  2235,  2048,  1878,  1722,  1579,
    1449,  1329,  1218,  1117,  1024,  939,   861,   790,   724,   664,   609,   558,
    512,   470,   430,   395,   362,   332,   304,   279,   256,   235,   215,   197,
    181,   166,   152,   140,   128,   116,   108,   99,    91,    83,    76,    69,
    64,    59,    54,    49,    45,    41,    38,    35};
static const uint16_t k_iq_scale[80] = {
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495,
    46177, 50535, 55109, 59933, 65535, 35734, 38968, 42577, 46341, 50617, 55027, 60097,
    32809, 35734, 38968, 42454, 46382, 50576, 55109, 60056, 65535, 35734, 38968, 42495,
    46320, 50515, 55109, 60076, 65535, 35744, 38968, 42495, 46341, 50535, 55099, 60087,
    65535, 35734, 38973, 42500, 46341, 50535, 55109, 60097, 32771, 35734, 38965, 42497,
    46341, 50535, 55109, 60099, 32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424,
    32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933};
/* IQ shift: 15 for qp 0-7, then one less every 8 qp, except that qp 16, 32,
 * 40 and 48 keep the previous group's shift (quant.c:85-96) */
static int iq_shift_of(int qp)
{
    int s = 15 - (qp >> 3);
    if (qp == 16 || qp == 32 || qp == 40 || qp == 48) s += 1;
    return s;
}

int xo_q_scale(int qp) { return k_q_scale[qp]; }
int xo_iq_scale(int qp) { return k_iq_scale[qp]; }
int xo_iq_shift(int qp) { return iq_shift_of(qp); }

/* tab_quant_fwd_add (rdo.c:661-666): floor(2^x * 5 / 31) */
int xo_quant_fwd_add(int shift, int b_intra)
{
    int x = shift + b_intra;
    return (int)(((int64_t)1 << x) * 5 / 31);
}

/* quant_c (quant.c:108-120); the sign of zero counts as positive */
int xo_quant(int16_t *coef, int n, int scale, int shift, int add)
{
    int i, nz = 0;
    for (i = 0; i < n; i++) {
        int c = coef[i];
        int q = (iabs(c) * scale + add) >> shift;
        coef[i] = (int16_t)(c < 0 ? -q : q);
        nz += coef[i] != 0;
    }
    return nz;
}

/* quant_weighted_c (quant.c:158-169) */
int xo_wquant(int16_t *coef, int n, int scale, int shift, int add, const int *levelscale)
{
    int i, nz = 0;
    for (i = 0; i < n; i++) {
        int c = coef[i];
        int a = (iabs(c) * levelscale[i] + (1 << 18)) >> 19;
        int q = (a * scale + add) >> shift;
        coef[i] = (int16_t)(c < 0 ? -q : q);
        nz += coef[i] != 0;
    }
    return nz;
}

/* dequant_c (quant.c:173-184): zeros stay zero */
void xo_dequant(int16_t *coef, int n, int scale, int shift)
{
    int i;
    int add = 1 << (shift - 1);
    for (i = 0; i < n; i++)
        if (coef[i]) coef[i] = (int16_t)clip3(-32768, 32767, (coef[i] * scale + add) >> shift);
}

void xo_abs_coeff(int16_t *dst, const int16_t *src, int n)
{
    int i;
    for (i = 0; i < n; i++) dst[i] = (int16_t)iabs(src[i]);
}

int xo_add_sign(int16_t *dst, const int16_t *abs_val, int n)
{
    int i, nz = 0;
    for (i = 0; i < n; i++) {
        dst[i] = (int16_t)(dst[i] > 0 ? abs_val[i] : -abs_val[i]);
        nz += abs_val[i] != 0;
    }
    return nz;
}

static int ilog2i(int v) { int l = 0; while ((1 << (l + 1)) <= v) l++; return l; }

int xo_tq_chain(int part, int16_t *blk, int16_t *coef_out, int qp, int b_intra, int use_2nd)
{
    int w = k_pu_w[part], h = k_pu_h[part];
    int wavelet = (w == 64 || h == 64);
    int w_tr = wavelet ? w / 2 : w, h_tr = wavelet ? h / 2 : h;
    /* i_level of the TU: log2 of the side for squares (64 -> 6), one less
     * than the parent CU level for the split shapes (rdo.c:1440-1463) */
    int level = (ilog2i(w) + ilog2i(h)) >> 1;
    int n = w_tr * h_tr, nz, qshift, dqshift;
    int16_t buf[64 * 64];
    memcpy(buf, blk, (size_t)w * h * 2);
    if (part == 0 && use_2nd) xo_transform_4x4_2nd(buf, 4);
    else xo_dct(part, buf, buf, wavelet ? 64 : w_tr);
    qshift = 15 + 16 - 9 - level;
    nz = xo_quant(buf, n, k_q_scale[qp], qshift, xo_quant_fwd_add(qshift, b_intra));
    memcpy(coef_out, buf, (size_t)n * 2);
    if (nz == 0) {
        memset(blk, 0, (size_t)w * h * 2);
        return 0;
    }
    dqshift = iq_shift_of(qp) + 9 + level - 16;
    xo_dequant(buf, n, k_iq_scale[qp], dqshift);
    if (part == 0 && use_2nd) {
        xo_inv_transform_4x4_2nd(buf, 4);
        memcpy(blk, buf, 32);
    } else {
        int16_t out[64 * 64];
        xo_idct(part, buf, out, wavelet ? 64 : w_tr);
        memcpy(blk, out, (size_t)w * h * 2);
    }
    return nz;
}

/* Batch form of xo_tq_chain over the GPU batch descriptor layout
 * (xavs2gpu_tq_block_t: offset, coef_offset, part, qp, flags): residual and
 * recon at offset, levels at coef_offset, nnz per block (-1 for an invalid
 * descriptor).  OpenMP over blocks when threads > 1. */
static int tq_one(const xo_tq_block_t *b, const int16_t *residual, int16_t *coef, int16_t *recon)
{
    int16_t blk[64 * 64], cf[64 * 64];
    int w, h, n, nz;
    if (b->part < 0 || b->part >= 25 || b->qp < 0 || b->qp > 79) return -1;
    w = k_pu_w[b->part];
    h = k_pu_h[b->part];
    if (!(w * h == 16 || (w == h && w >= 8) || (w == 16 && h == 4) || (w == 4 && h == 16) ||
          (w == 32 && h == 8) || (w == 8 && h == 32) || (w == 64 && h == 16) || (w == 16 && h == 64)))
        return -1;
    n = (w == 64 || h == 64) ? (w / 2) * (h / 2) : w * h;
    memcpy(blk, residual + b->offset, (size_t)w * h * 2);
    nz = xo_tq_chain(b->part, blk, cf, b->qp, b->flags & 1, (b->flags >> 1) & 1);
    memcpy(coef + b->coef_offset, cf, (size_t)n * 2);
    memcpy(recon + b->offset, blk, (size_t)w * h * 2);
    return nz;
}

void xo_tq_batch(const xo_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef, int16_t *recon,
                 int32_t *nnz, int threads)
{
    int i;
#ifdef _OPENMP
    if (threads > 1) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
        for (i = 0; i < n; i++) nnz[i] = tq_one(&blocks[i], residual, coef, recon);
        return;
    }
#endif
    (void)threads;
    for (i = 0; i < n; i++) nnz[i] = tq_one(&blocks[i], residual, coef, recon);
}

/* ------------------------------------------------------------------------
 * motion search (me.c:479-579, 614-641, 879-1183; md_inter.c:840-926)
 * ---------------------------------------------------------------------- */
/* mvbits (me.c:614-641): 1 bit for 0, else the exp-Golomb length
 * 2*bitlen(|d|) + 1 */
int xo_mvbits(int d)
{
    const unsigned a = (unsigned)iabs(d);
    return a ? 2 * (32 - __builtin_clz(a)) + 1 : 1;   /* 2 * bit length + 1 */
}

static inline int32_t mv_cost(int lambda, int mvx, int mvy, int pmx, int pmy)
{
    return (int32_t)(((int64_t)lambda * (xo_mvbits(mvx - pmx) + xo_mvbits(mvy - pmy))) >> 16);
}

void xo_pu_set_limits(xo_pu_t *pu, int width, int height, int vmin_qpel, int vmax_qpel)
{
    int w = k_pu_w[pu->part], h = k_pu_h[pu->part];
    int mn, mx;
    mn = clip3(-8192, 8191, (-64 - pu->x) * 4);
    mx = clip3(-8192, 8191, (width + 64 - pu->x - w) * 4);
    pu->min_x = (int16_t)((mn >> 2) + 6);
    pu->max_x = (int16_t)((mx >> 2) - 6);
    mn = clip3(vmin_qpel, vmax_qpel, (-64 - pu->y) * 4);
    mx = clip3(vmin_qpel, vmax_qpel, (height + 64 - pu->y - h) * 4);
    pu->min_y = (int16_t)((mn >> 2) + 6);
    pu->max_y = (int16_t)((mx >> 2) - 6);
}

/* the two spiral orders of me.c:129-139 */
static const int8_t k_spiral[9][2] = {{0, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1},
                                      {-1, 0}, {1, 0}, {-1, 1}, {1, 1}};
static const int8_t k_spiral2[9][2] = {{0, 0}, {0, -1}, {-1, -1}, {-1, 0}, {-1, 1},
                                       {0, 1}, {1, 1}, {1, 0}, {1, -1}};

static inline int in_box(const xo_pu_t *pu, int mx, int my)
{
    return mx >= pu->min_x && mx <= pu->max_x && my >= pu->min_y && my <= pu->max_y;
}

static inline int floor4(int v) { return v >> 2; }   /* arithmetic shift */

int32_t xo_me_search(const xo_me_params_t *prm, const xo_pu_t *pu, const uint8_t *fenc,
                     intptr_t i_fenc, const uint8_t *const fref[16], intptr_t i_fref,
                     xo_me_result_t *out)
{
    const int part = pu->part, lam = prm->lambda_factor;
    const int pmx = pu->mvp_x, pmy = pu->mvp_y;
    const uint8_t *ref0 = fref[0] + pu->y * i_fref + pu->x;
    int cand[2][2], ncand = 0, i, j, c;
    int32_t bcost = 1 << 30;
    int bmx = 0, bmy = 0, omx, omy;

    /* candidates: rounded and clipped MVP, then (0,0) (md_inter.c:840-865,
     * 957-959); duplicates dropped */
    {
        int xs[2] = {(pmx + 2) >> 2, 0}, ys[2] = {(pmy + 2) >> 2, 0};
        for (c = 0; c < 2; c++) {
            int x = clip3(pu->min_x, pu->max_x, xs[c]);
            int y = clip3(pu->min_y, pu->max_y, ys[c]);
            if (ncand == 1 && cand[0][0] == x && cand[0][1] == y) continue;
            cand[ncand][0] = x; cand[ncand][1] = y; ncand++;
        }
    }
    for (c = 0; c < ncand; c++) {
        int mx = cand[c][0], my = cand[c][1];
        if (in_box(pu, mx, my)) {
            int32_t cost = xo_sad(part, fenc, i_fenc, ref0 + my * i_fref + mx, i_fref) +
                           mv_cost(lam, mx * 4, my * 4, pmx, pmy);
            if (cost < bcost) { bcost = cost; bmx = mx; bmy = my; }
        }
    }
    if (bcost == (1 << 30)) {
        out->bmv_x = out->bmv_y = out->imv_x = out->imv_y = 0;
        out->bcost = out->icost = bcost;
        out->mvcost = 0;
        return bcost;
    }
    /* full search, j outer, i inner, first strictly smaller cost wins
     * (me.c:1156-1164) */
    omx = bmx; omy = bmy;
    {
        /* the window clipped to the limits (the positions outside are
         * skipped in the reference's loop), the vertical MV bits hoisted */
        const sad_fn_t sad = k_sad_fn[part];
        const int R = prm->search_range;
        const int j0 = pu->min_y - omy > -R ? pu->min_y - omy : -R, j1 = pu->max_y - omy < R - 1 ? pu->max_y - omy : R - 1;
        const int i0 = pu->min_x - omx > -R ? pu->min_x - omx : -R, i1 = pu->max_x - omx < R - 1 ? pu->max_x - omx : R - 1;
        for (j = j0; j <= j1; j++) {
            const int my = omy + j, by = xo_mvbits(my * 4 - pmy);
            const uint8_t *row = ref0 + my * i_fref;
            for (i = i0; i <= i1; i++) {
                const int mx = omx + i;
                const int32_t cost = sad(fenc, i_fenc, row + mx, i_fref) +
                                     (int32_t)(((int64_t)lam * (xo_mvbits(mx * 4 - pmx) + by)) >> 16);
                if (cost < bcost) { bcost = cost; bmx = mx; bmy = my; }
            }
        }
    }
    out->imv_x = (int16_t)bmx; out->imv_y = (int16_t)bmy;
    out->icost = bcost;
    out->bmv_x = (int16_t)(bmx * 4); out->bmv_y = (int16_t)(bmy * 4);
    out->bcost = bcost;
    out->mvcost = mv_cost(lam, bmx * 4, bmy * 4, pmx, pmy);

    /* sub-pel refinement (me.c:479-579) */
    if (prm->fractional_me) {
        const int8_t (*pat)[2] = prm->fast_sub_me ? k_spiral2 : k_spiral;
        const int step = prm->fast_sub_me ? 2 : 1;
        int cx = bmx * 4, cy = bmy * 4, bx = cx, by = cy, pos;
        int ctr_x = (pmx >> 1) << 1, ctr_y = (pmy >> 1) << 1;
        int32_t best;
#define QCOST(mx_, my_)                                                                        \
    ((prm->use_hadamard ? xo_satd : xo_sad)(                                                  \
         part, fenc, i_fenc,                                                                   \
         fref[((my_) & 3) * 4 + ((mx_) & 3)] + (pu->y + floor4(my_)) * i_fref + pu->x +       \
             floor4(mx_),                                                                      \
         i_fref) +                                                                             \
     mv_cost(lam, (mx_), (my_), pmx, pmy))
        best = prm->use_hadamard ? QCOST(cx, cy) : bcost;
        for (pos = 1; pos < 9; pos += step) {
            int mx = cx + 2 * pat[pos][0], my = cy + 2 * pat[pos][1];
            int32_t cost = QCOST(mx, my);
            if (cost < best) { best = cost; bx = mx; by = my; }
        }
        if (prm->fractional_me > 1) {
            cx = bx; cy = by;
            for (pos = 1; pos < 9; pos += step) {
                int mx, my;
                if (prm->enable_pmvr) {
                    /* pmvr_adapt_mv (me.c:412-424), TH_PMVR = 2 */
                    if (iabs(cx - ctr_x) > 2 || iabs(cy - ctr_y) > 2) {
                        mx = cx + 2 * pat[pos][0]; my = cy + 2 * pat[pos][1];
                        if (iabs(mx - ctr_x) <= 2 && iabs(my - ctr_y) <= 2) continue;
                    } else {
                        mx = cx + pat[pos][0]; my = cy + pat[pos][1];
                        if (iabs(mx - ctr_x) > 2 || iabs(my - ctr_y) > 2) continue;
                    }
                } else {
                    mx = cx + pat[pos][0]; my = cy + pat[pos][1];
                }
                {
                    int32_t cost = QCOST(mx, my);
                    if (cost < best) { best = cost; bx = mx; by = my; }
                }
            }
        }
#undef QCOST
        out->bmv_x = (int16_t)bx; out->bmv_y = (int16_t)by;
        out->bcost = best;
        out->mvcost = mv_cost(lam, bx, by, pmx, pmy);
    }
    return out->bcost;
}

void xo_me_search_list(const xo_me_params_t *prm, const xo_pu_t *pus, int n_pus,
                       const uint8_t *fenc, intptr_t i_fenc,
                       const uint8_t *const *frefs, intptr_t i_fref,
                       xo_me_result_t *out, int threads)
{
    int i;
#ifdef _OPENMP
    if (threads > 1) {
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
        for (i = 0; i < n_pus; i++) {
            const xo_pu_t *pu = &pus[i];
            xo_me_search(prm, pu, fenc + pu->y * i_fenc + pu->x, i_fenc, frefs + 16 * pu->ref,
                         i_fref, &out[i]);
        }
        return;
    }
#endif
    (void)threads;
    for (i = 0; i < n_pus; i++) {
        const xo_pu_t *pu = &pus[i];
        xo_me_search(prm, pu, fenc + pu->y * i_fenc + pu->x, i_fenc, frefs + 16 * pu->ref, i_fref,
                     &out[i]);
    }
}

/* ==========================================================================
 * Intra prediction (common/intra.c) and the rough mode decision
 * (encoder/md_intra.c).  `ep` points at the top-left edge sample: ep[1..]
 * is the top row continuing into the top-right, ep[-1..] the left column
 * continuing downwards (intra.c:1590-1594).
 * ======================================================================== */

/* Angle steps of the angular modes as (multiplier, shift) pairs, for the
 * step along x per row (index 0) and along y per column (index 1)
 * (intra.c:98-120, normative AVS2 geometry). */
static const int8_t k_ang_ms[2][33][2] = {
    {{0, 0}, {0, 0}, {0, 0},
     {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}, {93, 8}, {1, 2}, {1, 3},
     {0, 0},
     {1, 3}, {1, 2}, {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}, {11, 2}, {4, 0}, {8, 0},
     {0, 0},
     {8, 0}, {4, 0}, {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}},
    {{0, 0}, {0, 0}, {0, 0},
     {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}, {11, 2}, {4, 0}, {8, 0},
     {0, 0},
     {8, 0}, {4, 0}, {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}, {93, 8}, {1, 2}, {1, 3},
     {0, 0},
     {1, 3}, {1, 2}, {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}}};

/* integer step and 1/32 fraction of displacement d (intra.c:295-306) */
static int ang_step(int mode, int axis, int d, int *frac)
{
    const int t = d * k_ang_ms[axis][mode][0], sh = k_ang_ms[axis][mode][1];
    const int n = t >> sh;
    *frac = ((t << 5) >> sh) - (n << 5);
    return n;
}

static int ilog2_pos(int v) { int r = 0; while (v > 1) { v >>= 1; r++; } return r; }

/* The reference's table entry for mode 5 on the narrow 4x16 and 8x32 shapes
 * (intra_pred_ang_x_5_c, intra.c:455-605): the first 4 (8) rows follow the
 * angular formula, the rest of the block is one edge sample (ep[8], ep[16])
 * except a few samples just below those rows. */
static void mode5_narrow(const uint8_t *ep, uint8_t *dst, int i_dst, int bsx, int bsy)
{
    int x, y;
    const int rows = bsx == 4 ? 4 : 8;
    for (y = 0; y < rows; y++) {
        int f, ix = ang_step(5, 0, y + 1, &f);
        for (x = 0; x < bsx; x++, ix++)
            dst[y * i_dst + x] = (uint8_t)((ep[ix] * (32 - f) + ep[ix + 1] * (64 - f) + ep[ix + 2] * (32 + f) +
                                            ep[ix + 3] * f + 64) >> 7);
    }
    const uint8_t pad = ep[2 * rows];
    for (y = rows; y < bsy; y++)
        for (x = 0; x < bsx; x++) dst[y * i_dst + x] = pad;
    if (bsx == 4) {
        const uint8_t *s = ep + 8;
        dst[4 * i_dst + 0] = (uint8_t)((s[-2] + 9 * s[-1] + 15 * s[0] + 7 * s[1] + 16) >> 5);
        dst[4 * i_dst + 1] = (uint8_t)((s[-1] + 9 * s[0] + 15 * s[1] + 7 * s[2] + 16) >> 5);
    } else {
        const uint8_t *s = ep + 12;
        for (x = 0; x < 4; x++)
            dst[8 * i_dst + x] = (uint8_t)((5 * s[x] + 13 * s[x + 1] + 11 * s[x + 2] + 3 * s[x + 3] + 16) >> 5);
        for (x = 0; x < 3; x++)
            dst[9 * i_dst + x] = (uint8_t)((s[x + 1] + 5 * s[x + 2] + 7 * s[x + 3] + 3 * s[x + 4] + 8) >> 4);
        dst[10 * i_dst] = (uint8_t)((7 * s[3] + 15 * s[4] + 9 * s[5] + s[6] + 16) >> 5);
    }
}

static void pred_ang_left(int mode, const uint8_t *ep, uint8_t *dst, int i_dst, int bsx, int bsy)
{
    int x, y;
    for (x = 0; x < bsx; x++) {
        int f, s = ang_step(mode, 1, x + 1, &f);
        for (y = 0; y < bsy; y++) {
            const int iy = y + s;
            dst[y * i_dst + x] = (uint8_t)((ep[-iy] * (32 - f) + ep[-iy - 1] * (64 - f) + ep[-iy - 2] * (32 + f) +
                                            ep[-iy - 3] * f + 64) >> 7);
        }
    }
}

void xo_intra_pred(int mode, const uint8_t *ep, uint8_t *dst, int i_dst, int dc_avail, int bsx, int bsy)
{
    int x, y;
    if (mode == 5 && ((bsx == 4 && bsy == 16) || (bsx == 8 && bsy == 32))) {
        mode5_narrow(ep, dst, i_dst, bsx, bsy);
        return;
    }
    if (mode == 31 && ((bsx == 16 && bsy == 4) || (bsx == 32 && bsy == 8))) {
        /* intra_pred_ang_y_31_c (intra.c:1147-1161): mode 5 on the
         * transposed edge and block */
        uint8_t et[2 * 64 + 8], tb[64 * 64];
        const int n = bsy + bsx * 11 / 8 + 3;
        for (x = 0; x < n; x++) et[x] = ep[-x];
        mode5_narrow(et, tb, bsy, bsy, bsx);
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) dst[y * i_dst + x] = tb[x * bsy + y];
        return;
    }
    if (mode == 31 && bsx == 16 && bsy == 64) {
        /* the reference writes columns 0-3 only (intra.c:1176-1183) and
         * leaves the rest of the block as it was */
        for (x = 0; x < 4; x++) {
            int f, sy = ang_step(31, 1, x + 1, &f);
            for (y = 0; y < bsy; y++) {
                const int iy = y + sy;
                dst[y * i_dst + x] = (uint8_t)((ep[-iy] * (32 - f) + ep[-iy - 1] * (64 - f) +
                                                ep[-iy - 2] * (32 + f) + ep[-iy - 3] * f + 64) >> 7);
            }
        }
        return;
    }
    if (mode == 0) {                                           /* DC, intra.c:153-190 */
        const int top = dc_avail >> 8, left = dc_avail & 0xFF;
        int sl = 0, sa = 0, v;
        for (y = 0; y < bsy; y++) sl += ep[-1 - y];
        for (x = 0; x < bsx; x++) sa += ep[1 + x];
        if (top && left) v = ((sl + sa + ((bsx + bsy) >> 1)) * (512 / (bsx + bsy))) >> 9;
        else if (left) v = (sl + (bsy >> 1)) >> ilog2_pos(bsy);
        else if (top) v = (sa + (bsx >> 1)) >> ilog2_pos(bsx);
        else v = 128;
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) dst[y * i_dst + x] = (uint8_t)v;
    } else if (mode == 1) {                                    /* plane, intra.c:192-236 */
        static const int mult[7] = {0, 0, 13, 17, 5, 11, 23}, shf[7] = {0, 0, 7, 10, 11, 15, 19};
        const int lx = ilog2_pos(bsx), ly = ilog2_pos(bsy), w2 = bsx >> 1, h2 = bsy >> 1;
        int H = 0, V = 0, a, b, c;
        for (x = 1; x <= w2; x++) H += x * (ep[w2 + x] - ep[w2 - x]);
        for (y = 1; y <= h2; y++) V += y * (ep[-h2 - y] - ep[-h2 + y]);
        a = (ep[-bsy] + ep[bsx]) << 4;
        b = ((H << 5) * mult[lx] + (1 << (shf[lx] - 1))) >> shf[lx];
        c = ((V << 5) * mult[ly] + (1 << (shf[ly] - 1))) >> shf[ly];
        a += 16 - b * (w2 - 1) - c * (h2 - 1);
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) {
                const int v = (a + b * x + c * y) >> 5;
                dst[y * i_dst + x] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
            }
    } else if (mode == 2) {                                    /* bilinear, intra.c:238-293 */
        const int lx = ilog2_pos(bsx), ly = ilog2_pos(bsy), sh = lx < ly ? lx : ly, shxy = lx + ly + 1;
        const int a = ep[bsx], b = ep[-bsy];
        const int c = bsx == bsy ? (a + b + 1) >> 1 : (((a << lx) + (b << ly)) * 13 + (1 << (sh + 5))) >> (sh + 6);
        const int t = 2 * c - a - b;
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) {
                /* the reference accumulates these terms row by row and
                 * column by column; the closed forms are equal */
                const int top = ep[1 + x], left = ep[-1 - y];
                const int predx = (left << lx) + (x + 1) * (a - left);
                const int predy = (top << ly) + (y + 1) * (b - top);
                const int wxy = x * y * t;
                int v = ((predx << ly) + (predy << lx) + wxy + (1 << (lx + ly))) >> shxy;
                dst[y * i_dst + x] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
            }
    } else if (mode == 12) {                                   /* vertical */
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) dst[y * i_dst + x] = ep[1 + x];
    } else if (mode == 24) {                                   /* horizontal */
        for (y = 0; y < bsy; y++)
            for (x = 0; x < bsx; x++) dst[y * i_dst + x] = ep[-1 - y];
    } else if (mode < 12) {                                    /* angular, from the top row (intra.c:310-331) */
        for (y = 0; y < bsy; y++) {
            int f, ix = ang_step(mode, 0, y + 1, &f);
            for (x = 0; x < bsx; x++, ix++)
                dst[y * i_dst + x] = (uint8_t)((ep[ix] * (32 - f) + ep[ix + 1] * (64 - f) + ep[ix + 2] * (32 + f) +
                                                ep[ix + 3] * f + 64) >> 7);
        }
    } else if (mode > 24) {                                    /* angular, from the left column (intra.c:336-358) */
        pred_ang_left(mode, ep, dst, i_dst, bsx, bsy);
    } else {                                                   /* angular, both edges (intra.c:363-397) */
        for (y = 0; y < bsy; y++) {
            int fx, ixx = -ang_step(mode, 0, y + 1, &fx);
            for (x = 0; x < bsx; x++, ixx++) {
                int fy, sy = ang_step(mode, 1, x + 1, &fy);
                const int iyy = y - sy;
                int v;
                if (iyy <= -1)
                    v = ep[ixx + 2] * (32 - fx) + ep[ixx + 1] * (64 - fx) + ep[ixx] * (32 + fx) + ep[ixx - 1] * fx;
                else
                    v = ep[-iyy - 2] * (32 - fy) + ep[-iyy - 1] * (64 - fy) + ep[-iyy] * (32 + fy) + ep[-iyy + 1] * fy;
                dst[y * i_dst + x] = (uint8_t)((v + 64) >> 7);
            }
        }
    }
}

/* Cost of every mode for a block (md_intra.c:216-226): lambda * mode bits
 * (2 for the two most probable modes, else 6) + SATD (or SAD) of the
 * prediction against the source block, as rdcost_t (double). */
void xo_intra_mode_costs(const uint8_t *ep, const uint8_t *fenc, int i_fenc, int bsx, int bsy, int dc_avail,
                         const int mpm[2], double lambda, int hadamard, double cost[33])
{
    uint8_t pred[64 * 64];
    int m, part = -1;
    for (m = 0; m < 25; m++)
        if (k_pu_w[m] == bsx && k_pu_h[m] == bsy) part = m;
    for (m = 0; m < 33; m++) {
        const int bits = (mpm[0] == m || mpm[1] == m) ? 2 : 6;
        int32_t d;
        if (m == 31 && bsx == 16 && bsy == 64)
            pred_ang_left(m, ep, pred, bsx, bsx, bsy);   /* every column predicted (the table entry writes 4) */
        else
            xo_intra_pred(m, ep, pred, bsx, m == 0 ? dc_avail : m, bsx, bsy);
        d = hadamard ? xo_satd(part, fenc, i_fenc, pred, bsx) : xo_sad(part, fenc, i_fenc, pred, bsx);
        cost[m] = lambda * bits + (double)d;
    }
}

/* update_candidate_list (md_intra.c:195-210): insertion into a list kept
 * sorted by cost, a new entry going after equal costs */
static void cand_insert(int mode, double cost, int n, int *modes, double *costs)
{
    int i = n - 1;
    if (!(cost < costs[i])) return;
    while (i > 0 && cost < costs[i - 1]) {
        modes[i] = modes[i - 1];
        costs[i] = costs[i - 1];
        i--;
    }
    modes[i] = mode;
    costs[i] = cost;
}

int xo_intra_candidates(const double cost[33], int rough, int dist2, int dist1, int num_for_rdo, const int mpm[2],
                        int *modes, double *costs)
{
    const int N = 9;   /* INTRA_MODE_NUM_FOR_RDO (defines.h:290) */
    int visited[33] = {0}, i, j, m, num_angle;
    for (i = 0; i < N; i++) {
        modes[i] = 0;
        costs[i] = (double)(1LL << 50);   /* MAX_COST (defines.h:299) */
    }
#define XO_VISIT(k) do { cand_insert((k), cost[(k)], N, modes, costs); visited[(k)] = 1; } while (0)
    if (!rough) {                                              /* md_intra.c:231-256 */
        for (m = 0; m < 33; m++) XO_VISIT(m);
        return num_for_rdo;
    }
    /* md_intra.c:258-380 */
    for (m = 0; m < 3; m++) XO_VISIT(m);
    for (m = 4; m < 33; m += 4) XO_VISIT(m);
    for (i = 0; i < dist2; i++) {
        m = modes[i];
        if (m <= 2) continue;
        if (m > 3 && !visited[m - 2]) XO_VISIT(m - 2);
        if (m < 31 && !visited[m + 2]) XO_VISIT(m + 2);
    }
    for (i = 0, num_angle = 0; num_angle < dist1 && i < N; i++) {
        m = modes[i];
        if (m <= 2) continue;
        if (m > 3 && !visited[m - 1]) { XO_VISIT(m - 1); num_angle++; }
        if (m < 32 && !visited[m + 1]) { XO_VISIT(m + 1); num_angle++; }
    }
    if (!visited[mpm[0]]) XO_VISIT(mpm[0]);
    if (!visited[mpm[1]]) XO_VISIT(mpm[1]);
#undef XO_VISIT
    if (modes[0] == mpm[0] || modes[0] == mpm[1] || modes[1] == mpm[0] || modes[1] == mpm[1])
        return num_for_rdo < 3 ? num_for_rdo : 3;
    visited[modes[0]] = 2;
    visited[modes[1]] = 2;
    for (i = 2, j = 2; i < N && j < num_for_rdo; i++) {
        m = modes[i];
        if (!visited[m]) continue;
        if (m <= 2) {
            modes[j++] = m;
            visited[m] = 2;
        } else if (m == 3) {
            if (visited[4] == 1) { modes[j++] = 3; visited[3] = 2; }
        } else if (m == 32) {
            if (visited[31] == 1) { modes[j++] = 32; visited[32] = 2; }
        } else if (visited[m - 1] == 1 && visited[m + 1] == 1) {
            modes[j++] = m;
            visited[m] = 2;
        }
        if (visited[0] == 2 && visited[1] == 2 && visited[2] == 2) break;
    }
    return num_for_rdo < j ? num_for_rdo : j;
}

static void rmd_one(const xo_intra_block_t *b, const uint8_t *edges, const uint8_t *fenc, int fenc_stride,
                    double lambda, int hadamard, int rough, int dist2, int dist1, xo_intra_result_t *r)
{
    const int mpm[2] = {b->mpm[0], b->mpm[1]};
    xo_intra_mode_costs(edges + b->edge_offset, fenc + b->fenc_offset, fenc_stride, b->width, b->height,
                        b->dc_avail, mpm, lambda, hadamard, r->cost);
    r->num_for_rdo = xo_intra_candidates(r->cost, rough, dist2, dist1, b->num_for_rdo, mpm, r->cand_mode,
                                         r->cand_cost);
}

void xo_intra_rmd_batch(const xo_intra_block_t *blocks, int n, const uint8_t *edges, const uint8_t *fenc,
                        int fenc_stride, double lambda, int hadamard, int rough, int dist2, int dist1,
                        xo_intra_result_t *out, int threads)
{
    int i;
#ifdef _OPENMP
    if (threads > 1) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
        for (i = 0; i < n; i++)
            rmd_one(&blocks[i], edges, fenc, fenc_stride, lambda, hadamard, rough, dist2, dist1, &out[i]);
        return;
    }
#endif
    (void)threads;
    for (i = 0; i < n; i++)
        rmd_one(&blocks[i], edges, fenc, fenc_stride, lambda, hadamard, rough, dist2, dist1, &out[i]);
}

/* ------------------------------------------------------------------------
 * in-loop filters (filter_deblock.c, filter_sao.c, encoder/sao.c)
 * ---------------------------------------------------------------------- */
/* One line across an edge (lf_edge_core, filter_deblock.c:254-360): s points
 * at the first sample of the Q side, `a` steps across the edge.  The filter
 * strength fs comes from the flatness of both sides; the formulas are the
 * reference's written as weighted sums. */
static void deblock_line(uint8_t *s, int a, int alpha, int beta, int chroma)
{
    const int L0 = s[-a], L1 = s[-2 * a], L2 = s[-3 * a];
    const int R0 = s[0], R1 = s[a], R2 = s[2 * a];
    const int d = iabs(R0 - L0);
    int fl, fr, fs;
    if (d >= alpha || d <= 1) return;
    fl = (iabs(L1 - L0) < beta ? 2 : 0) + (iabs(L2 - L0) < beta ? 1 : 0);
    fr = (iabs(R0 - R1) < beta ? 2 : 0) + (iabs(R0 - R2) < beta ? 1 : 0);
    switch (fl + fr) {
    case 6: fs = (R1 == R0 && L0 == L1) ? 4 : 3; break;
    case 5: fs = (R1 == R0 && L0 == L1) ? 3 : 2; break;
    case 4: fs = fl == 2 ? 2 : 1; break;
    case 3: fs = iabs(L1 - R1) < beta ? 1 : 0; break;
    default: fs = 0; break;
    }
    if (chroma && fs > 0) fs--;
    if (fs == 4) {
        s[-a] = (uint8_t)((9 * L0 + 9 * L2 + 8 * R0 + 6 * R2 + 16) >> 5);
        s[-2 * a] = (uint8_t)((7 * L0 + 6 * L2 + 3 * R0 + 8) >> 4);
        s[-3 * a] = (uint8_t)((4 * L0 + 3 * L2 + R0 + 4) >> 3);
        s[0] = (uint8_t)((9 * R0 + 9 * R2 + 8 * L0 + 6 * L2 + 16) >> 5);
        s[a] = (uint8_t)((7 * R0 + 6 * R2 + 3 * L0 + 8) >> 4);
        s[2 * a] = (uint8_t)((4 * R0 + 3 * R2 + L0 + 4) >> 3);
    } else if (fs == 3) {
        s[-a] = (uint8_t)((L2 + 4 * L1 + 6 * L0 + 4 * R0 + R1 + 8) >> 4);
        s[0] = (uint8_t)((L1 + 4 * L0 + 6 * R0 + 4 * R1 + R2 + 8) >> 4);
        s[-2 * a] = (uint8_t)((3 * L2 + 8 * L1 + 4 * L0 + R0 + 8) >> 4);
        s[a] = (uint8_t)((3 * R2 + 8 * R1 + 4 * R0 + L0 + 8) >> 4);
    } else if (fs == 2) {
        s[-a] = (uint8_t)((3 * L1 + 10 * L0 + 3 * R0 + 8) >> 4);
        s[0] = (uint8_t)((3 * L0 + 10 * R0 + 3 * R1 + 8) >> 4);
    } else if (fs == 1) {
        s[-a] = (uint8_t)((3 * L0 + R0 + 2) >> 2);
        s[0] = (uint8_t)((3 * R0 + L0 + 2) >> 2);
    }
}

/* n lines of an edge, `along` apart; the first half uses flt_flag[0] */
static void deblock_edge(uint8_t *src, int n, int along, int across, int alpha, int beta, int chroma,
                         const uint8_t *flt_flag)
{
    int k;
    for (k = 0; k < n; k++)
        if (flt_flag[k >= n / 2]) deblock_line(src + k * along, across, alpha, beta, chroma);
}

void xo_deblock_luma(int dir, uint8_t *src, int stride, int alpha, int beta, const uint8_t *flt_flag)
{
    if (dir == 0) deblock_edge(src, 8, stride, 1, alpha, beta, 0, flt_flag);
    else deblock_edge(src, 8, 1, stride, alpha, beta, 0, flt_flag);
}

void xo_deblock_chroma(int dir, uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                       const uint8_t *flt_flag)
{
    if (dir == 0) {
        deblock_edge(src_u, 4, stride, 1, alpha, beta, 1, flt_flag);
        deblock_edge(src_v, 4, stride, 1, alpha, beta, 1, flt_flag);
    } else {
        deblock_edge(src_u, 4, 1, stride, alpha, beta, 1, flt_flag);
        deblock_edge(src_v, 4, 1, stride, alpha, beta, 1, flt_flag);
    }
}

/* the edge of one 8x8 block in one direction (lf_scu_deblock,
 * filter_deblock.c:434-486); no edge on the picture border */
static void deblock_scu(uint8_t *y, int stride, uint8_t *u, uint8_t *v, int stride_c, int sx, int sy, int w_scu,
                        const xo_deblock_scu_t *scus, int dir)
{
    const xo_deblock_scu_t *e = &scus[sy * w_scu + sx];
    if (!e->type[dir] || (dir == 0 && sx == 0) || (dir == 1 && sy == 0)) return;
    if (!e->flag[dir][0] && !e->flag[dir][1]) return;
    xo_deblock_luma(dir, y + (sy * 8) * stride + sx * 8, stride, e->alpha[dir], e->beta[dir], e->flag[dir]);
    if (e->type[dir] == 2 && ((dir == 1 && !(sy & 1)) || (dir == 0 && !(sx & 1)))) {
        const int o = (sy * 4) * stride_c + sx * 4;
        xo_deblock_chroma(dir, u + o, v + o, stride_c, e->alpha_c[dir], e->beta_c[dir], e->flag[dir]);
    }
}

void xo_deblock_picture(uint8_t *y, int stride, uint8_t *u, uint8_t *v, int stride_c, int width, int height,
                        const xo_deblock_scu_t *scus, int lcu_level, int lcu_order)
{
    const int w_scu = width / 8, h_scu = height / 8;
    int i, j;
    if (!lcu_order) {
        /* a picture one LCU wide: the LCU loop leaves the horizontal edges
         * of its last 8x8 column for a next LCU that does not exist */
        const int n_hor = w_scu <= (1 << (lcu_level - 3)) ? w_scu - 1 : w_scu;
        for (j = 0; j < h_scu; j++)
            for (i = 0; i < w_scu; i++) deblock_scu(y, stride, u, v, stride_c, i, j, w_scu, scus, 0);
        for (j = 0; j < h_scu; j++)
            for (i = 0; i < n_hor; i++) deblock_scu(y, stride, u, v, stride_c, i, j, w_scu, scus, 1);
        return;
    } else {
        /* xavs2_lcu_deblock (filter_deblock.c:497-546) for each LCU in raster
         * order: its vertical edges, then its horizontal edges one 8x8 column
         * to the left (the last column waits for the next LCU's vertical
         * edges, except in the last LCU of a row) */
        const int lcu_scu = 1 << (lcu_level - 3);
        int lx, ly;
        for (ly = 0; ly < h_scu; ly += lcu_scu)
            for (lx = 0; lx < w_scu; lx += lcu_scu) {
                const int nh = lcu_scu < w_scu - lx ? lcu_scu : w_scu - lx;
                const int nv = lcu_scu < h_scu - ly ? lcu_scu : h_scu - ly;
                int x0 = lx, n = nh;
                for (j = 0; j < nv; j++)
                    for (i = 0; i < nh; i++) deblock_scu(y, stride, u, v, stride_c, lx + i, ly + j, w_scu, scus, 0);
                if (lx == 0) {
                    n--;
                } else {
                    if (lx + nh == w_scu) n++;
                    x0--;
                }
                for (j = 0; j < nv; j++)
                    for (i = 0; i < n; i++) deblock_scu(y, stride, u, v, stride_c, x0 + i, ly + j, w_scu, scus, 1);
            }
    }
}

static int sign3(int v) { return (v > 0) - (v < 0); }

/* sao_block_c (filter_sao.c:50-226) in closed form: a sample's edge class
 * is sign(s - n1) + sign(s - n2) + 2 over its two neighbours along the EO
 * direction, its band (BO) the top 5 bits.  The filtered range of each row
 * follows the reference's availability rules; samples outside it keep dst.
 * (When a diagonal neighbour is available but an adjacent side is not --
 * never the case in the encoder, whose diagonals are conjunctions of the
 * sides -- the reference reads a line-buffer entry it has not set; this
 * restatement uses the true neighbour there.) */
void xo_sao_block(uint8_t *dst, int i_dst, const uint8_t *src, int i_src, int w, int h, const int *avail,
                  const xo_sao_param_t *prm)
{
    const int T = avail[0], D = avail[1], L = avail[2], R = avail[3];
    const int TL = avail[4], TR = avail[5], DL = avail[6], DR = avail[7];
    static const int nb[4][4] = {{-1, 0, 1, 0}, {0, -1, 0, 1}, {-1, -1, 1, 1}, {1, -1, -1, 1}};
    const int type = prm->type_idc;
    const int sx = L ? 0 : 1, ex = R ? w : w - 1;
    int x, y;
    if (type == 4) {                                           /* BO */
        for (y = 0; y < h; y++)
            for (x = 0; x < w; x++) {
                const int s = src[y * i_src + x];
                dst[y * i_dst + x] = clip_pel(s + prm->offset[s >> 3]);
            }
        return;
    }
    if (type < 0 || type > 3) return;
    for (y = 0; y < h; y++) {
        int x0 = sx, x1 = ex;
        if (type == 1) {                                       /* EO_90: rows limited, all columns */
            if ((y == 0 && !T) || (y == h - 1 && !D)) continue;
            x0 = 0;
            x1 = w;
        } else if (type == 2 && y == 0) {                      /* EO_135 first / last row */
            x0 = TL ? 0 : 1;
            x1 = T ? (R ? w : w - 1) : 1;
        } else if (type == 2 && y == h - 1) {
            x0 = D ? (L ? 0 : 1) : w - 1;
            x1 = DR ? w : w - 1;
        } else if (type == 3 && y == 0) {                      /* EO_45 first / last row */
            x0 = T ? (L ? 0 : 1) : w - 1;
            x1 = TR ? w : w - 1;
        } else if (type == 3 && y == h - 1) {
            x0 = DL ? 0 : 1;
            x1 = D ? (R ? w : w - 1) : 1;
        }
        for (x = x0; x < x1; x++) {
            const uint8_t *p = src + y * i_src + x;
            const int s = p[0];
            const int c = sign3(s - p[nb[type][1] * i_src + nb[type][0]]) +
                          sign3(s - p[nb[type][3] * i_src + nb[type][2]]) + 2;
            dst[y * i_dst + x] = clip_pel(s + prm->offset[c]);
        }
    }
}

/* the filtered region of an LCU (sao_get_neighbor_avail, sao.c:898-975):
 * comp 0 luma, 1/2 chroma; returns 0 when empty */
static int sao_region(int lx, int ly, int lcu_level, int width, int height, int avail, int comp, int *px, int *py,
                      int *pw, int *ph)
{
    const int T = avail & 1, D = (avail >> 1) & 1, L = (avail >> 2) & 1, R = (avail >> 3) & 1;
    const int S = 1 << lcu_level, c = comp > 0;
    int x = lx * S, y = ly * S;
    int w = (S < width - x ? S : width - x), h = (S < height - y ? S : height - y);
    const int W = c ? width >> 1 : width, H = c ? height >> 1 : height;
    if (c) {
        x >>= 1; y >>= 1; w >>= 1; h >>= 1;
    }
    if (!R) w += 4;
    if (!D) h += 4;
    if (L) x -= 4; else w -= 4;
    if (T) y -= 4; else h -= 4;
    if (w > W - x) w = W - x;
    if (h > H - y) h = H - y;
    *px = x; *py = y; *pw = w; *ph = h;
    return w > 0 && h > 0;
}

void xo_sao_picture(uint8_t *const dst[3], const uint8_t *const src[3], int stride, int stride_c, int width,
                    int height, int lcu_level, const xo_sao_lcu_t *lcus)
{
    const int S = 1 << lcu_level;
    const int wl = (width + S - 1) / S, hl = (height + S - 1) / S;
    int lx, ly, comp, k;
    for (ly = 0; ly < hl; ly++)
        for (lx = 0; lx < wl; lx++) {
            const xo_sao_lcu_t *p = &lcus[ly * wl + lx];
            const int a = p->avail;
            const int av[8] = {a & 1, (a >> 1) & 1, (a >> 2) & 1, (a >> 3) & 1, (a & 1) && ((a >> 2) & 1),
                               (a & 1) && ((a >> 3) & 1), ((a >> 1) & 1) && ((a >> 2) & 1),
                               ((a >> 1) & 1) && ((a >> 3) & 1)};
            for (comp = 0; comp < 3; comp++) {
                xo_sao_param_t prm;
                int x, y, w, h;
                const int st = comp ? stride_c : stride;
                if (p->type[comp] < 0 || !sao_region(lx, ly, lcu_level, width, height, a, comp, &x, &y, &w, &h))
                    continue;
                memset(&prm, 0, sizeof(prm));
                prm.type_idc = p->type[comp];
                for (k = 0; k < 32; k++) prm.offset[k] = p->offset[comp][k];
                xo_sao_block(dst[comp] + y * st + x, st, src[comp] + y * st + x, st, w, h, av, &prm);
            }
        }
}

/* ------------------------------------------------------------------------
 * lookahead analysis
 * ---------------------------------------------------------------------- */
/* lowres_filter_core_c (mc.c:838-855) */
void xo_lowres_filter(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height)
{
    int x, y;
    for (y = 0; y < height; y++) {
        const uint8_t *a = src + 2 * y * i_src, *b = a + i_src;
        for (x = 0; x < width; x++) {
            const int l = (a[2 * x] + b[2 * x] + 1) >> 1, r = (a[2 * x + 1] + b[2 * x + 1] + 1) >> 1;
            dst[y * i_dst + x] = (uint8_t)((l + r + 1) >> 1);
        }
    }
}

void xo_lookahead_picture(const uint8_t *src, int stride, int width, int height, uint8_t *lowres, int lowres_stride,
                          int32_t *mad16, int32_t *mad32, int32_t *mad64)
{
    int32_t *out[3] = {mad16, mad32, mad64};
    int k, x, y;
    xo_lowres_filter(src, stride, lowres, lowres_stride, width / 2, height / 2);
    for (k = 0; k < 3; k++) {
        const int n = 16 << k, nx = (width + n - 1) / n, ny = (height + n - 1) / n;
        for (y = 0; y < ny; y++)
            for (x = 0; x < nx; x++)
                out[k][y * nx + x] = ((x + 1) * n <= width && (y + 1) * n <= height)
                                         ? xo_mad(src + (size_t)y * n * stride + x * n, stride, n) : -1;
    }
}

/* ------------------------------------------------------------------------
 * skip / direct rough cost (cu_check_skip_direct_rough2, rdo.c:2395-2480)
 * ---------------------------------------------------------------------- */
static int skip_same_motion(const xo_skip_cand_t *a, const xo_skip_cand_t *b)
{
    int q, l;
    if (a->n_pu != b->n_pu) return 0;
    for (q = 0; q < a->n_pu; q++)
        for (l = 0; l < 2; l++) {
            if (a->ref[q][l] != b->ref[q][l]) return 0;
            if (a->ref[q][l] >= 0 && (a->mv[q][l][0] != b->mv[q][l][0] || a->mv[q][l][1] != b->mv[q][l][1]))
                return 0;
        }
    return 1;
}

void xo_skip_costs(const uint8_t *cur, int cur_stride, const uint8_t *const *planes, int stride, int width,
                   int height, int nrefs, const xo_skip_cand_t *cands, int n, double lambda, int n_cus,
                   int32_t *dist, double *cost, int32_t *best)
{
    static uint8_t pred[64 * 64];
    const double max_cost = (double)(1LL << 50);   /* MAX_COST (defines.h:299) */
    int i, j, q, l, x, y;
    for (i = 0; i < n; i++) {
        const xo_skip_cand_t *k = &cands[i];
        const int S = 1 << k->size_log2;
        int ok = k->size_log2 >= 3 && k->size_log2 <= 6 && (k->n_pu == 1 || k->n_pu == 4) && k->x >= 0 &&
                 k->y >= 0 && k->x + S <= width && k->y + S <= height;
        /* update_skip_mv_list (rdo.c:2366-2389): repeated motion is skipped */
        for (j = i - 1; ok && j >= 0 && cands[j].cu == k->cu; j--)
            if (skip_same_motion(&cands[j], k)) ok = 0;
        if (ok) {
            const int hp = k->n_pu == 4 ? S / 2 : S;
            for (q = 0; q < k->n_pu; q++) {
                if (k->ref[q][0] < 0 && k->ref[q][1] < 0) ok = 0;
                for (l = 0; l < 2; l++) {
                    const int r = k->ref[q][l];
                    int px, py;
                    if (r < 0) continue;
                    px = k->x + (q & 1) * hp + (k->mv[q][l][0] >> 2);
                    py = k->y + (q >> 1) * hp + (k->mv[q][l][1] >> 2);
                    if (r >= nrefs || px < -80 || py < -80 || px + hp > width + 80 || py + hp > height + 80) ok = 0;
                }
            }
        }
        if (!ok) {
            dist[i] = -1;
            cost[i] = max_cost;
            continue;
        }
        for (y = 0; y < S; y++)
            for (x = 0; x < S; x++) {
                const int qq = k->n_pu == 4 ? (x >= S / 2) + 2 * (y >= S / 2) : 0;
                int v[2], nv = 0;
                for (l = 0; l < 2; l++) {
                    const int r = k->ref[qq][l];
                    const int mx = k->mv[qq][l][0], my = k->mv[qq][l][1];
                    const uint8_t *pl;
                    if (r < 0) continue;
                    /* frame sub-pel plane of the fractional position (mc.c:570-574) */
                    pl = planes[16 * r + ((my & 3) << 2) + (mx & 3)];
                    v[nv++] = pl[(intptr_t)(k->y + y + (my >> 2)) * stride + k->x + x + (mx >> 2)];
                }
                /* bi-prediction: pixel_avg (pixel.c:680-719) */
                pred[y * 64 + x] = (uint8_t)(nv == 2 ? (v[0] + v[1] + 1) >> 1 : v[0]);
            }
        dist[i] = xo_sa8d(k->size_log2 - 2, cur + (intptr_t)k->y * cur_stride + k->x, cur_stride, pred, 64);
        cost[i] = (double)dist[i] + lambda * (double)k->rate;
    }
    for (i = 0; i < n_cus; i++) best[i] = -1;
    for (i = 0; i < n; i++) {
        const int cu = cands[i].cu;
        double m = max_cost;
        if (cu < 0 || cu >= n_cus || (i > 0 && cands[i - 1].cu == cu)) continue;
        for (j = i; j < n && cands[j].cu == cu; j++)
            if (cost[j] < m) {
                m = cost[j];
                best[cu] = j;
            }
    }
}

/* fill_reference_samples_{0,x,y,xy}_c (intra.c:1580-1860) with the neighbour
 * samples taken from one picture (the four variants differ only in whether
 * the top row / left column come from the CTU's border buffers or from the
 * CTU's reconstruction) */
void xo_intra_fill_edge(const uint8_t *pic, int stride, int x0, int y0, int bsx, int bsy, int avail, uint8_t *ep)
{
    const int L = avail & 1, T = (avail >> 1) & 1, LD = (avail >> 2) & 1, TR = (avail >> 3) & 1, TL = (avail >> 4) & 1;
    const uint8_t *top = pic + (intptr_t)(y0 - 1) * stride + x0 - 1;   /* top[k] = edge sample k > 0 */
    int k, npad;
    for (k = -2 * bsy; k <= 2 * bsx; k++) ep[k] = 128;               /* g_dc_value, 8-bit */
    if (T)
        for (k = 1; k <= bsx; k++) ep[k] = top[k];
    for (k = bsx + 1; k <= 2 * bsx; k++) ep[k] = TR ? top[k] : ep[bsx];
    npad = bsy * 11 / 4 - bsx + 4;
    for (k = 1; k <= npad; k++) ep[2 * bsx + k] = ep[2 * bsx];
    if (L)
        for (k = 1; k <= bsy; k++) ep[-k] = pic[(intptr_t)(y0 + k - 1) * stride + x0 - 1];
    for (k = bsy + 1; k <= 2 * bsy; k++) ep[-k] = LD ? pic[(intptr_t)(y0 + k - 1) * stride + x0 - 1] : ep[-bsy];
    if (TL) ep[0] = top[0];
    else if (T) ep[0] = top[1];
    else if (L) ep[0] = pic[(intptr_t)y0 * stride + x0 - 1];
    npad = bsx * 11 / 4 - bsy + 4;
    for (k = 1; k <= npad; k++) ep[-2 * bsy - k] = ep[-2 * bsy];
}

static int xo_side_log(int v)
{
    int l;
    for (l = 2; l <= 6; l++)
        if (v == (1 << l)) return l;
    return -1;
}

/* the picture-bounds part of is_block_available (md_intra.c:44-56) applied
 * to each side's samples */
static int xo_usable_sides(int avail, int x, int y, int bsx, int bsy, int width, int height)
{
    const int l = x >= 1 && y >= 0 && y + bsy <= height, t = y >= 1 && x >= 0 && x + bsx <= width;
    int ok = (l ? 1 : 0) | (t ? 2 : 0);
    if (l && y + 2 * bsy <= height) ok |= 4;
    if (t && x + 2 * bsx <= width) ok |= 8;
    if (l && t) ok |= 16;
    return avail & ok;
}

void xo_intra_fill_edges(const xo_intra_edge_job_t *jobs, int n, const uint8_t *pic, int stride, int width, int height,
                         uint8_t *edges, int64_t edges_size)
{
    int i, k;
    uint8_t buf[1024];
    for (i = 0; i < n; i++) {
        const xo_intra_edge_job_t *j = &jobs[i];
        const int bsx = j->width, bsy = j->height, a = xo_side_log(bsx), c = xo_side_log(bsy);
        int lo, hi, lo_ref, hi_ref;
        if (a < 0 || c < 0 || a - c > 2 || c - a > 2) continue;
        lo = bsy + 11 * bsx / 4 + 6;
        hi = bsx + 11 * bsy / 4 + 6;
        if (j->edge_offset < lo || j->edge_offset > edges_size - 1 - hi) continue;
        xo_intra_fill_edge(pic, stride, j->x, j->y, bsx, bsy,
                           xo_usable_sides(j->avail, j->x, j->y, bsx, bsy, width, height), buf + 512);
        /* last sample the reference writes on each side */
        hi_ref = 2 * bsx + (bsy * 11 / 4 - bsx + 4 > 0 ? bsy * 11 / 4 - bsx + 4 : 0);
        lo_ref = 2 * bsy + (bsx * 11 / 4 - bsy + 4 > 0 ? bsx * 11 / 4 - bsy + 4 : 0);
        for (k = hi_ref + 1; k <= hi; k++) buf[512 + k] = buf[512 + hi_ref];
        for (k = lo_ref + 1; k <= lo; k++) buf[512 - k] = buf[512 - lo_ref];
        memcpy(edges + j->edge_offset - lo, buf + 512 - lo, (size_t)(lo + hi + 1));
    }
}
