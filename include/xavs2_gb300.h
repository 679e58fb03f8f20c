/*
 * xavs2_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the xavs2
 * encoder hot path: block costs, interpolation, integer DCT + quantisation and
 * full-search/sub-pel motion search.
 *
 * Two kinds of entry points:
 *
 *  1. Drop-ins.  One function per entry of the reference's primitive tables
 *     (`pixel_funcs_t`, `dct_funcs_t` and the interpolation members of
 *     `intrinsic_func_t`, source/common/primitives.h:101-221 and
 *     source/common/pixel.h:124-166), with the same signature, argument
 *     meaning and in-place behaviour.  Buffers are caller-owned host memory,
 *     exactly as for the reference's C functions; each call stages its
 *     operands to the GPU, runs one kernel and copies the result back on a
 *     per-thread CUDA stream, so the functions may be called from the
 *     encoder's frame and row threads concurrently.  xavs2gpu_pixel_init /
 *     xavs2gpu_dct_init / xavs2gpu_quant_init fill tables laid out like the
 *     reference's so that an encoder can install them wholesale.
 *
 *  2. Batched forms (no counterpart in the reference): whole-frame sub-pel
 *     interpolation, batched block costs, batched transform+quant chains and
 *     a batched full-search + sub-pel motion search over every PU of a frame.
 *
 * Errors: the reference's signatures have no error channel, so failures are
 * recorded in a process-wide status (xavs2gpu_get_status/get_error).  By
 * default a failure also prints the message and aborts the process; there is
 * no CPU fallback and no silently wrong result.
 *
 * Types follow the reference's 8-bit build (source/common/basic_types.h:
 * 50-62): pel = uint8_t, coeff = int16_t, dist = cmp_dist = int32_t,
 * mct = int16_t.
 */
#ifndef XAVS2_GB300_H
#define XAVS2_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XAVS2GPU_API __attribute__((visibility("default")))

typedef uint8_t xavs2gpu_pel_t;
typedef int16_t xavs2gpu_coeff_t;
typedef int32_t xavs2gpu_dist_t;

/* ===========================================================================
 * status and device selection
 * ======================================================================== */
enum {
    XAVS2GPU_OK = 0,
    XAVS2GPU_ERR_CUDA = 1,      /* a CUDA call failed                        */
    XAVS2GPU_ERR_ARG = 2,       /* invalid argument (shape, size, pointer)   */
    XAVS2GPU_ERR_NO_DEVICE = 3, /* no usable GPU                             */
    XAVS2GPU_ERR_TIMEOUT = 4,   /* a bounded device wait gave up             */
    XAVS2GPU_ERR_CAPACITY = 5   /* request larger than the session capacity  */
};

/* Select the CUDA device used by this thread's calls (default 0). */
XAVS2GPU_API int xavs2gpu_init(int device);
XAVS2GPU_API int xavs2gpu_get_status(void);
XAVS2GPU_API const char *xavs2gpu_get_error(void);
XAVS2GPU_API void xavs2gpu_clear_error(void);
/* 1 (default): print and abort on any failure.  0: record and return. */
XAVS2GPU_API void xavs2gpu_set_abort_on_error(int enable);
/* Per-call block costs (the SAD / SATD / SA8D / SSD and sad_x3 / sad_x4
 * table entries).  1 (default): where the device reads pageable host memory
 * coherently (cudaDevAttrPageableMemoryAccess, e.g. a Grace host over
 * NVLink-C2C) the kernel reads the caller's blocks in place -- one launch
 * and one synchronisation per call; elsewhere, and with 0, the blocks are
 * packed into a pinned buffer and copied to the device and back. */
XAVS2GPU_API void xavs2gpu_set_percall_mode(int in_place);
/* 1 when this thread's per-call block costs run in place (mode 1 and a
 * device that reads pageable host memory coherently). */
XAVS2GPU_API int xavs2gpu_percall_in_place(void);
/* Number of kernels this library has launched in the process. */
XAVS2GPU_API uint64_t xavs2gpu_kernel_launches(void);
XAVS2GPU_API const char *xavs2gpu_version(void);
/* Synchronous copies between host and device memory (helpers for bindings
 * that hold raw device pointers); return the status. */
XAVS2GPU_API int xavs2gpu_copy_d2h(void *dst, const void *src, size_t bytes);
XAVS2GPU_API int xavs2gpu_copy_h2d(void *dst, const void *src, size_t bytes);

/* ===========================================================================
 * 1. drop-in primitives
 * ======================================================================== */

/* LumaPU indices, same order as enum LumaPU (source/common/pixel.h:50-65). */
enum {
    XAVS2GPU_LUMA_4x4, XAVS2GPU_LUMA_8x8, XAVS2GPU_LUMA_16x16, XAVS2GPU_LUMA_32x32,
    XAVS2GPU_LUMA_64x64, XAVS2GPU_LUMA_8x4, XAVS2GPU_LUMA_4x8, XAVS2GPU_LUMA_16x8,
    XAVS2GPU_LUMA_8x16, XAVS2GPU_LUMA_32x16, XAVS2GPU_LUMA_16x32, XAVS2GPU_LUMA_64x32,
    XAVS2GPU_LUMA_32x64, XAVS2GPU_LUMA_16x12, XAVS2GPU_LUMA_12x16, XAVS2GPU_LUMA_16x4,
    XAVS2GPU_LUMA_4x16, XAVS2GPU_LUMA_32x24, XAVS2GPU_LUMA_24x32, XAVS2GPU_LUMA_32x8,
    XAVS2GPU_LUMA_8x32, XAVS2GPU_LUMA_64x48, XAVS2GPU_LUMA_48x64, XAVS2GPU_LUMA_64x16,
    XAVS2GPU_LUMA_16x64, XAVS2GPU_NUM_PU_SIZES
};

/* Function pointer types of the reference tables (pixel.h:124-139,
 * primitives.h:62-118). */
typedef int32_t (*xavs2gpu_pixel_cmp_t)(const uint8_t *pix1, intptr_t i_pix1, const uint8_t *pix2, intptr_t i_pix2);
typedef int32_t (*xavs2gpu_pixel_ssd_t)(const uint8_t *pix1, intptr_t i_pix1, const uint8_t *pix2, intptr_t i_pix2);
typedef int32_t (*xavs2gpu_pixel_ssd2_t)(const uint8_t *pix1, intptr_t i_pix1, const uint8_t *pix2, intptr_t i_pix2, int width, int height);
typedef void (*xavs2gpu_pixel_cmp_x3_t)(const uint8_t *fenc, const uint8_t *pix0, const uint8_t *pix1, const uint8_t *pix2, intptr_t i_stride, int scores[3]);
typedef void (*xavs2gpu_pixel_cmp_x4_t)(const uint8_t *fenc, const uint8_t *pix0, const uint8_t *pix1, const uint8_t *pix2, const uint8_t *pix3, intptr_t i_stride, int scores[4]);
typedef void (*xavs2gpu_copy_pp_t)(uint8_t *dst, intptr_t dstStride, const uint8_t *src, intptr_t srcStride);
typedef void (*xavs2gpu_copy_sp_t)(uint8_t *dst, intptr_t dstStride, const int16_t *src, intptr_t srcStride);
typedef void (*xavs2gpu_copy_ps_t)(int16_t *dst, intptr_t dstStride, const uint8_t *src, intptr_t srcStride);
typedef void (*xavs2gpu_copy_ss_t)(int16_t *dst, intptr_t dstStride, const int16_t *src, intptr_t srcStride);
typedef void (*xavs2gpu_pixel_sub_ps_t)(int16_t *dst, intptr_t dstride, const uint8_t *src0, const uint8_t *src1, intptr_t sstride0, intptr_t sstride1);
typedef void (*xavs2gpu_pixel_add_ps_t)(uint8_t *a, intptr_t dstride, const uint8_t *b0, const int16_t *b1, intptr_t sstride0, intptr_t sstride1);
typedef void (*xavs2gpu_pixel_avg_pp_t)(uint8_t *dst, intptr_t dstride, const uint8_t *src0, intptr_t sstride0, const uint8_t *src1, intptr_t sstride1, int weight);
typedef int (*xavs2gpu_mad_funcs_t)(uint8_t *p_src, int i_src, int cu_size);
typedef void (*xavs2gpu_average_t)(uint8_t *dst, int i_dst, uint8_t *src1, int i_src1, uint8_t *src2, int i_src2, int width, int height);

/* Same member order and types as pixel_funcs_t (pixel.h:141-166). */
typedef struct xavs2gpu_pixel_funcs_t {
    xavs2gpu_pixel_cmp_t    sad    [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_cmp_t    satd   [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_cmp_t    sa8d   [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_ssd_t    ssd    [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_cmp_x3_t sad_x3 [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_cmp_x4_t sad_x4 [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_sub_ps_t sub_ps [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_add_ps_t add_ps [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_copy_sp_t      copy_sp[XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_copy_ps_t      copy_ps[XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_copy_ss_t      copy_ss[XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_copy_pp_t      copy_pp[XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_avg_pp_t avg    [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_pixel_cmp_t   *intra_cmp;
    xavs2gpu_pixel_cmp_t   *fpel_cmp;
    xavs2gpu_mad_funcs_t    madf[4];
    xavs2gpu_pixel_ssd2_t   ssd_block;
    xavs2gpu_average_t      average;
} xavs2gpu_pixel_funcs_t;

/* Replaces xavs2_pixel_init (pixel.c:1050): fills every member with the GPU
 * functions below.  intra_cmp/fpel_cmp are left as they are; the encoder
 * points them at the satd or sad array afterwards (encoder.c:1837-1847). */
XAVS2GPU_API void xavs2gpu_pixel_init(uint32_t cpuid, xavs2gpu_pixel_funcs_t *pixf);
/* Replaces xavs2_mad_init (pixel.c:1654). */
XAVS2GPU_API void xavs2gpu_mad_init(uint32_t cpuid, xavs2gpu_mad_funcs_t *madf);

/* Per-shape drop-ins.  Names follow the reference's per-shape C functions
 * (pixel.c:93-840): xavs2gpu_pixel_sad_WxH replaces xavs2_pixel_sad_WxH, etc. */
#define XAVS2GPU_DECLARE_PIXEL(w, h)                                                                                  \
    XAVS2GPU_API int32_t xavs2gpu_pixel_sad_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);  \
    XAVS2GPU_API int32_t xavs2gpu_pixel_satd_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2); \
    XAVS2GPU_API int32_t xavs2gpu_pixel_sa8d_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2); \
    XAVS2GPU_API int32_t xavs2gpu_pixel_ssd_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2);  \
    XAVS2GPU_API void xavs2gpu_pixel_sad_x3_##w##x##h(const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,       \
                                                      const uint8_t *r2, intptr_t i_ref, int scores[3]);               \
    XAVS2GPU_API void xavs2gpu_pixel_sad_x4_##w##x##h(const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,       \
                                                      const uint8_t *r2, const uint8_t *r3, intptr_t i_ref,            \
                                                      int scores[4]);                                                  \
    XAVS2GPU_API void xavs2gpu_pixel_avg_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *a, intptr_t sa,           \
                                                   const uint8_t *b, intptr_t sb, int weight);                        \
    XAVS2GPU_API void xavs2gpu_pixel_sub_ps_##w##x##h(int16_t *dst, intptr_t ds, const uint8_t *a, const uint8_t *b,   \
                                                      intptr_t sa, intptr_t sb);                                       \
    XAVS2GPU_API void xavs2gpu_pixel_add_ps_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *a, const int16_t *b,   \
                                                      intptr_t sa, intptr_t sb);                                       \
    XAVS2GPU_API void xavs2gpu_blockcopy_pp_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *src, intptr_t ss);     \
    XAVS2GPU_API void xavs2gpu_blockcopy_ps_##w##x##h(int16_t *dst, intptr_t ds, const uint8_t *src, intptr_t ss);     \
    XAVS2GPU_API void xavs2gpu_blockcopy_sp_##w##x##h(uint8_t *dst, intptr_t ds, const int16_t *src, intptr_t ss);     \
    XAVS2GPU_API void xavs2gpu_blockcopy_ss_##w##x##h(int16_t *dst, intptr_t ds, const int16_t *src, intptr_t ss);

#define XAVS2GPU_FOR_EACH_PU(X)                                                                 \
    X(4, 4) X(8, 8) X(16, 16) X(32, 32) X(64, 64) X(8, 4) X(4, 8) X(16, 8) X(8, 16) X(32, 16)  \
    X(16, 32) X(64, 32) X(32, 64) X(16, 12) X(12, 16) X(16, 4) X(4, 16) X(32, 24) X(24, 32)    \
    X(32, 8) X(8, 32) X(64, 48) X(48, 64) X(64, 16) X(16, 64)

XAVS2GPU_FOR_EACH_PU(XAVS2GPU_DECLARE_PIXEL)

/* xavs2_get_block_ssd_c (pixel.c:537), xavs2_pixel_average (pixel.c:844),
 * mad_NxN_c (pixel.c:1620) */
XAVS2GPU_API int32_t xavs2gpu_get_block_ssd(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2, int w, int h);
XAVS2GPU_API void xavs2gpu_pixel_average(uint8_t *dst, int i_dst, uint8_t *a, int i_a, uint8_t *b, int i_b, int w, int h);
XAVS2GPU_API int xavs2gpu_mad_NxN(uint8_t *src, int i_src, int cu_size);

/* ---- interpolation: members of intrinsic_func_t (primitives.h:157-171),
 * C versions in mc.c:274-547.  `coeff` points at the filter taps (8 for
 * luma, 4 for chroma) exactly as in the reference. */
XAVS2GPU_API void xavs2gpu_intpl_luma_hor(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_ext(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_ver_x3(uint8_t *const dst[3], int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t **coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_hor_x3(uint8_t *const dst[3], int i_dst, int16_t *const tmp[3], int i_tmp, uint8_t *src, int i_src, int width, int height, const int8_t **coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_ext_x3(uint8_t *const dst[3], int i_dst, int16_t *tmp, int i_tmp, int width, int height, const int8_t **coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_luma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff_x, const int8_t *coeff_y);
XAVS2GPU_API void xavs2gpu_intpl_chroma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_chroma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff);
XAVS2GPU_API void xavs2gpu_intpl_chroma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height, const int8_t *coeff_x, const int8_t *coeff_y);

/* ---- transform and quantisation (dct_funcs_t, primitives.h:101-119) ---- */
typedef void (*xavs2gpu_dct_t)(const int16_t *src, int16_t *dst, int i_src);

/* Same member order and types as dct_funcs_t. */
typedef struct xavs2gpu_dct_funcs_t {
    xavs2gpu_dct_t dct     [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_dct_t idct    [XAVS2GPU_NUM_PU_SIZES];
    xavs2gpu_dct_t dct_half[XAVS2GPU_NUM_PU_SIZES];
    void (*transform_4x4_2nd)    (int16_t *coeff, int i_coeff);
    void (*inv_transform_4x4_2nd)(int16_t *coeff, int i_coeff);
    void (*transform_2nd)        (int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left);
    void (*inv_transform_2nd)    (int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left);
    void (*abs_coeff)(int16_t *coef, const int16_t *src, const int i_coef);
    int  (*add_sign) (int16_t *coef, const int16_t *abs_val, const int i_coef);
    int  (*quant)    (int16_t *coef, const int i_coef, const int scale, const int shift, const int add);
    void (*dequant)  (int16_t *coef, const int i_coef, const int scale, const int shift);
    int  (*wquant)   (int16_t *coef, const int i_coef, const int scale, const int shift, const int add, int *levelscale);
} xavs2gpu_dct_funcs_t;

/* Replace xavs2_dct_init (transform.c:1599) and xavs2_quant_init (quant.c:212). */
XAVS2GPU_API void xavs2gpu_dct_init(uint32_t cpuid, xavs2gpu_dct_funcs_t *dctf);
XAVS2GPU_API void xavs2gpu_quant_init(uint32_t cpuid, xavs2gpu_dct_funcs_t *dctf);

/* Per-shape transforms (transform.c:1123-1587).  For the 32-point shapes the
 * lowest bit of the stride is the reference's wavelet flag; the 64-point
 * shapes read a contiguous block (stride 64 or 16) and write the
 * (w/2)x(h/2) coefficients contiguously. */
#define XAVS2GPU_DECLARE_DCT(w, h)                                                               \
    XAVS2GPU_API void xavs2gpu_dct_##w##x##h(const int16_t *src, int16_t *dst, int i_src);        \
    XAVS2GPU_API void xavs2gpu_idct_##w##x##h(const int16_t *src, int16_t *dst, int i_dst);
#define XAVS2GPU_FOR_EACH_TU(X) \
    X(4, 4) X(8, 8) X(16, 16) X(32, 32) X(64, 64) X(16, 4) X(4, 16) X(32, 8) X(8, 32) X(64, 16) X(16, 64)
XAVS2GPU_FOR_EACH_TU(XAVS2GPU_DECLARE_DCT)
XAVS2GPU_API void xavs2gpu_dct_32x32_half(const int16_t *src, int16_t *dst, int i_src);
XAVS2GPU_API void xavs2gpu_dct_64x64_half(const int16_t *src, int16_t *dst, int i_src);
XAVS2GPU_API void xavs2gpu_transform_4x4_2nd(int16_t *coeff, int i_coeff);
XAVS2GPU_API void xavs2gpu_inv_transform_4x4_2nd(int16_t *coeff, int i_coeff);
XAVS2GPU_API void xavs2gpu_transform_2nd(int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left);
XAVS2GPU_API void xavs2gpu_inv_transform_2nd(int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left);
/* quant_c, dequant_c, quant_weighted_c, abs_coeff_c, add_sign_c (quant.c:108-184) */
XAVS2GPU_API int  xavs2gpu_quant(int16_t *coef, const int i_coef, const int scale, const int shift, const int add);
XAVS2GPU_API void xavs2gpu_dequant(int16_t *coef, const int i_coef, const int scale, const int shift);
XAVS2GPU_API int  xavs2gpu_quant_weighted(int16_t *coef, const int i_coef, const int scale, const int shift, const int add, int *levelscale);
XAVS2GPU_API void xavs2gpu_abs_coeff(int16_t *dst, const int16_t *src, const int i_coef);
XAVS2GPU_API int  xavs2gpu_add_sign(int16_t *dst, const int16_t *abs_val, const int i_coef);

/* ===========================================================================
 * 2. batched forms (device pointers unless a name ends in _host)
 * ======================================================================== */

/* ---- block costs over a job list --------------------------------------
 * out[i] = cost `kind` (0 SAD, 1 SATD, 2 SA8D, 3 SSD) of shape jobs[i].part
 * between base1 + off1 (stride s1) and base2 + off2 (stride s2); the
 * per-block results equal the drop-ins'.  Kernels run on `stream`
 * (a cudaStream_t, 0 = default). */
typedef struct xavs2gpu_cost_job {
    int64_t off1, off2;
    int32_t s1, s2;
    int32_t part;
    int32_t pad_;
} xavs2gpu_cost_job_t;
XAVS2GPU_API int xavs2gpu_cost_batch(int kind, const xavs2gpu_cost_job_t *jobs, int n, const uint8_t *base1,
                                     const uint8_t *base2, int32_t *out, void *stream);

/* ---- whole-frame sub-pel planes ----------------------------------------
 * The reference's interpolate_lcu_row (mc.c:748-785) over every LCU row of a
 * frame: planes[k] (k = 4*dy + dx) of the 15 quarter-pel positions, each with
 * the same stride and `pad` pixels of replicated border as `src`, which must
 * already hold its own replicated border of at least 8 pixels.  mode 1
 * computes planes 2, 8, 10 (half-pel ME), mode 2 all 15.  Device pointers. */
XAVS2GPU_API int xavs2gpu_interpolate_frame(const uint8_t *src, int stride, int width, int height, int pad,
                                            uint8_t *const planes[16], int mode, void *stream);
/* Replicates the border of a device plane outwards by `pad` pixels
 * (plane_expand_border, frame.c:471-507, both bands). */
XAVS2GPU_API int xavs2gpu_expand_border(uint8_t *pix, int stride, int width, int height, int pad, void *stream);

/* ---- intra prediction (primitives.h:84, 186-188; intra.c) ----------------
 * intra_pred_t: src = the top-left edge sample (src[1..] top / top-right,
 * src[-1..] left / left-down), dst a bsx x bsy block with stride i_dst;
 * dir_mode is the mode (3..32 for the angular entry) or, for DC, the
 * availability (top << 8) | left (md_intra.c:170-185).  The predictors read
 * src[-(bsy + 11*bsx/4 + 6) .. bsx + 11*bsy/4 + 6].  Like the reference,
 * mode 31 on 16x64 writes columns 0-3 only. */
typedef void (*xavs2gpu_intra_pred_t)(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_dc(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_plane(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_bilinear(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_ver(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_hor(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
XAVS2GPU_API void xavs2gpu_intra_pred_ang(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy);
/* Fills intraf[0..32] (the layout of intrinsic_func_t.intraf). */
XAVS2GPU_API void xavs2gpu_intra_pred_init(uint32_t cpuid, xavs2gpu_intra_pred_t intraf[33]);

/* Batched rough mode decision (no single counterpart: the encoder's
 * rdo_get_pred_intra_luma / _rmd per block, md_intra.c:216-380).  For every
 * block: each mode's prediction, cost = lambda * (2 for an MPM, else 6) +
 * SATD (use_hadamard) or SAD against the source block (rdcost_t, double,
 * rounded as the reference's  lambda * bits + cost), and the 9-entry
 * candidate list with the number of modes for RDO the encoder derives from
 * them -- all 33 modes (rough = 0) or the rough three-phase search
 * (rough = 1, dist2 / dist1 = num_intra_rmd_dist2 / _dist1).  Mode 31 on
 * 16x64 is predicted in all 16 columns (the reference leaves 12 of them as
 * they were in its buffer).  Device pointers; edges + edge_offset is the
 * block's top-left edge sample and samples -(height + 11*width/4 + 6) ..
 * width + 11*height/4 + 6 around it are read.
 * A block whose sides are not powers of two in 4..64 with an aspect ratio of
 * at most 4, or whose MPMs are not modes, reports num_for_rdo = -1 (and no
 * costs).  Blocks are processed sorted by shape; the order of the batch is
 * free. */
typedef struct xavs2gpu_intra_block {
    int64_t edge_offset;
    int64_t fenc_offset;     /* source block: fenc + fenc_offset, stride fenc_stride */
    int16_t width, height;
    int16_t dc_avail;        /* (top available << 8) | left available */
    int8_t mpm[2];
    int32_t num_for_rdo;     /* tab_num_intra_rdo entry of the block's level */
    int32_t pad_;
} xavs2gpu_intra_block_t;
typedef struct xavs2gpu_intra_params {
    double lambda;           /* h->f_lambda_mode */
    int32_t use_hadamard;
    int32_t rough;
    int32_t dist2, dist1;
} xavs2gpu_intra_params_t;
typedef struct xavs2gpu_intra_result {
    double cost[33];
    double cand_cost[9];
    int32_t cand_mode[9];
    int32_t num_for_rdo;
} xavs2gpu_intra_result_t;
XAVS2GPU_API int xavs2gpu_intra_rmd_batch(const xavs2gpu_intra_block_t *blocks, int n, const uint8_t *edges,
                                          const uint8_t *fenc, int fenc_stride, const xavs2gpu_intra_params_t *prm,
                                          xavs2gpu_intra_result_t *out, void *stream);

/* Edge samples of a batch of blocks from one reconstructed picture, as
 * fill_reference_samples builds them (intra.c:1580-1860; the encoder's call
 * fill_ref_samples_luma, md_intra.c:137-160) when every neighbour sample is
 * the picture's: for each job, edges + edge_offset receives the block's
 * edge, samples -(height + 11*width/4 + 6) .. width + 11*height/4 + 6 around
 * it (the window xavs2gpu_intra_rmd_batch reads; beyond the reference's
 * padding the run's last sample repeats).  avail holds the MD_I_* bits of
 * get_intra_neighbors (md_intra.c:60-83): bit 0 left, 1 top, 2 left-down,
 * 3 top-right, 4 top-left; a side whose samples are not inside the
 * width x height picture is treated as missing.  Jobs with an invalid shape
 * (as for the RMD batch) or a window outside [0, edges_size) are skipped.
 * Device pointers; the jobs are independent and run in parallel, so windows
 * must not overlap. */
typedef struct xavs2gpu_intra_edge_job {
    int64_t edge_offset;     /* the block's top-left edge sample in edges */
    int32_t x, y;            /* the block's top-left sample in the picture */
    int16_t width, height;
    int32_t avail;           /* MD_I_* availability bits */
} xavs2gpu_intra_edge_job_t;
XAVS2GPU_API int xavs2gpu_intra_fill_edges(const xavs2gpu_intra_edge_job_t *jobs, int n, const uint8_t *pic,
                                           int stride, int width, int height, uint8_t *edges, int64_t edges_size,
                                           void *stream);

/* ---- in-loop filters (primitives.h:202-208; filter_deblock.c, filter_sao.c)
 * Deblocking of one edge: src is the first sample on the Q side (right of a
 * vertical edge, below a horizontal one); 8 lines for luma, 4 per chroma
 * plane; flt_flag[0] / [1] enable the first / second half of the lines.
 * Members in the layout of intrinsic_func_t.deblock_luma[2] /
 * deblock_chroma[2] ([0] vertical edge, [1] horizontal edge). */
typedef struct xavs2gpu_deblock_funcs {
    void (*deblock_luma[2])(uint8_t *src, int stride, int alpha, int beta, uint8_t *flt_flag);
    void (*deblock_chroma[2])(uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta, uint8_t *flt_flag);
} xavs2gpu_deblock_funcs_t;
XAVS2GPU_API void xavs2gpu_deblock_luma_ver(uint8_t *src, int stride, int alpha, int beta, uint8_t *flt_flag);
XAVS2GPU_API void xavs2gpu_deblock_luma_hor(uint8_t *src, int stride, int alpha, int beta, uint8_t *flt_flag);
XAVS2GPU_API void xavs2gpu_deblock_chroma_ver(uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                                              uint8_t *flt_flag);
XAVS2GPU_API void xavs2gpu_deblock_chroma_hor(uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                                              uint8_t *flt_flag);
XAVS2GPU_API void xavs2gpu_deblock_init(uint32_t cpuid, xavs2gpu_deblock_funcs_t *f);

/* SAOBlkParam (basic_types.h:88-94): type_idc -1 off, 0 EO_0, 1 EO_90,
 * 2 EO_135, 3 EO_45, 4 BO; offset[] by edge class (EO) or band (BO). */
typedef struct xavs2gpu_sao_param {
    int merge_idx, type_idc, start_band, delta_band;
    int offset[32];
} xavs2gpu_sao_param_t;
/* sao_flt_t (primitives.h:123-125): filters a w x h block of p_src into
 * p_dst; lcu_avail[8] = top, down, left, right, top-left, top-right,
 * down-left, down-right; samples outside the filtered range keep p_dst.
 * One sample around the source block is read (the reference's frames have
 * a margin). */
typedef void (*xavs2gpu_sao_flt_t)(uint8_t *p_dst, int i_dst, uint8_t *p_src, int i_src, int i_block_w,
                                   int i_block_h, int *lcu_avail, xavs2gpu_sao_param_t *sao_param);
XAVS2GPU_API void xavs2gpu_sao_block(uint8_t *p_dst, int i_dst, uint8_t *p_src, int i_src, int i_block_w,
                                     int i_block_h, int *lcu_avail, xavs2gpu_sao_param_t *sao_param);
XAVS2GPU_API void xavs2gpu_sao_init(uint32_t cpuid, xavs2gpu_sao_flt_t *f);

/* Picture-level deblocking (no single counterpart: xavs2_lcu_deblock,
 * filter_deblock.c:497-546, over every LCU).  Per 8x8 block (raster order,
 * width/8 per row) and direction (0 its left edge, 1 its top edge): the edge
 * type (0 none, 1 luma only, 2 luma and chroma; edges on the picture border
 * are never filtered), the half-edge flags (lf_skip_filter), and alpha /
 * beta for luma and chroma (tab_deblock_alpha / _beta at the edge's QP,
 * lf_scu_deblock).  4:2:0, in place, device pointers; width and height
 * multiples of 8, planes and strides 4-byte aligned, lcu_level 3..6.
 * Result = the reference's LCU-order result (including, in a picture one
 * LCU wide, the horizontal edges of the last 8x8 column left unfiltered). */
typedef struct xavs2gpu_deblock_scu {
    uint8_t type[2];
    uint8_t flag[2][2];
    uint8_t alpha[2], beta[2];
    uint8_t alpha_c[2], beta_c[2];
    uint8_t pad_[2];
} xavs2gpu_deblock_scu_t;
XAVS2GPU_API int xavs2gpu_deblock_picture(uint8_t *y, int stride, uint8_t *u, uint8_t *v, int stride_c, int width,
                                          int height, int lcu_level, const xavs2gpu_deblock_scu_t *scus,
                                          void *stream);
/* Picture-level SAO (sao_filter_lcu, sao.c:1170-1200, over every LCU): per
 * LCU (raster order) the type per component (-1 off), the offsets per
 * component and the availability of the top / down / left / right LCUs
 * (bits 0..3; diagonals are their conjunctions).  Each LCU's region is the
 * LCU moved 4 samples up and left inside the picture (sao.c:898-975); src
 * (the deblocked picture) and dst must not overlap; dst samples outside the
 * filtered ranges keep their values, or, with XAVS2GPU_SAO_COPY_UNFILTERED
 * in flags, get src's (dst is then written whole: the encoder's result
 * without its copy of the picture; this mode requires availabilities
 * consistent between neighbours -- a side is available exactly when the
 * neighbour there sees this LCU as available, none on the picture border --
 * as the encoder derives them).  Without the flag any availabilities are
 * accepted and overlapping regions resolve as in the reference's LCU loop.
 * 4:2:0, device pointers, LCU 16..64. */
#define XAVS2GPU_SAO_COPY_UNFILTERED 1
typedef struct xavs2gpu_sao_lcu {
    int8_t type[3];
    uint8_t avail;
    int8_t offset[3][32];
} xavs2gpu_sao_lcu_t;
XAVS2GPU_API int xavs2gpu_sao_picture(uint8_t *dst_y, uint8_t *dst_u, uint8_t *dst_v, const uint8_t *src_y,
                                      const uint8_t *src_u, const uint8_t *src_v, int stride, int stride_c,
                                      int width, int height, int lcu_level, const xavs2gpu_sao_lcu_t *lcus,
                                      int flags, void *stream);

/* Deblocking and SAO of a picture in one pass (both loops of the encoder,
 * xavs2_lcu_deblock and sao_filter_lcu, over every LCU): dst = SAO of the
 * deblocked src, written whole; src is left unchanged and must not overlap
 * dst.  The same per-8x8 edge parameters and per-LCU SAO parameters as
 * xavs2gpu_deblock_picture / xavs2gpu_sao_picture, one LCU size for both;
 * the availabilities must be consistent between neighbours (as the
 * encoder derives them), so that the SAO regions tile the picture.  4:2:0,
 * device pointers, width and height multiples of 8, LCU 16..64, planes and
 * strides 4-byte aligned. */
XAVS2GPU_API int xavs2gpu_loopfilter_picture(const uint8_t *src_y, const uint8_t *src_u, const uint8_t *src_v,
                                             uint8_t *dst_y, uint8_t *dst_u, uint8_t *dst_v, int stride,
                                             int stride_c, int width, int height, int lcu_level,
                                             const xavs2gpu_deblock_scu_t *scus, const xavs2gpu_sao_lcu_t *lcus,
                                             void *stream);

/* ---- lookahead analysis (mc.c:838-855, pixel.c:1620-1649, rdo.c:3286-3297)
 * lowres_filter (intrinsic_func_t.lowres_filter, primitives.h:140): the
 * width x height output from 2*width x 2*height source samples, each output
 * the rounded average of the rounded vertical averages of a 2x2 quad. */
XAVS2GPU_API void xavs2gpu_lowres_filter(uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height);
/* The same over device buffers, stream-ordered. */
XAVS2GPU_API int xavs2gpu_lowres_picture(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width,
                                         int height, void *stream);
/* One pass over a luma picture (device pointers): the width/2 x height/2
 * low-resolution picture and the MAD (mad_NxN_c) of every aligned 16x16,
 * 32x32 and 64x64 block, raster order over ceil(width/N) x ceil(height/N)
 * positions per size, -1 for blocks not fully inside the picture.  The
 * encoder's CU-depth prediction splits a CU when its MAD reaches 512 (16x16),
 * 2048 (32x32) or 12288 (64x64) (ctu_intra_depth_pred_mad). */
XAVS2GPU_API int xavs2gpu_lookahead_picture(const uint8_t *src, int stride, int width, int height, uint8_t *lowres,
                                            int lowres_stride, int32_t *mad16, int32_t *mad32, int32_t *mad64,
                                            void *stream);

/* ---- batched transform + quant chain -----------------------------------
 * For every block: dct (or, for a 4x4 block with flag bit 1, the 4x4
 * secondary transform) -> quant -> when any level is non-zero, dequant ->
 * inverse transform; the order of the reference's TU reconstruction
 * (rdo.c:1333-1370, 876-947).  The residual of a block is w x h contiguous
 * int16 at residual + offset and the reconstructed residual goes to the
 * same offset of `recon` (all zero when nnz = 0); the quantised levels
 * ((w/2)x(h/2) for the 64-point shapes) go to coef + coef_offset.
 * Quant parameters follow tu_quant_forward/inverse (rdo.c:659-759) with
 * i_level = log2 of the TU side (64 -> 6; the mean of the two side logs for
 * the split shapes).  nnz[i] = number of non-zero levels, -1 for an invalid
 * descriptor.  Device pointers. */
typedef struct xavs2gpu_tq_block {
    int64_t offset;        /* residual / recon offset (elements)            */
    int64_t coef_offset;   /* quantised levels offset (elements)            */
    int32_t part;          /* TU shape as a LumaPU index                    */
    int32_t qp;            /* 0..79                                         */
    int32_t flags;         /* bit 0: b_intra, bit 1: 4x4 secondary transform */
    int32_t pad_;
} xavs2gpu_tq_block_t;
XAVS2GPU_API int xavs2gpu_tq_batch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                                   int16_t *recon, int32_t *nnz, void *stream);
/* The same chain on host buffers (descriptors, residual, levels, recon,
 * nnz in host memory, same layout); returns when the outputs are on the
 * host.  The batch is cut into `chunks` runs of consecutive descriptors
 * (1..256): while one run is transformed, the next one's inputs are copied
 * in and the previous one's outputs copied out.  The overlap needs
 * page-locked buffers (cudaHostAlloc / cudaHostRegister); with pageable ones
 * the batch runs as one chunk.  chunks = 0 (page-locked arrays only): the
 * chain reads and writes the host arrays in place over the host link, no
 * copies (on a coherent CPU-GPU link this is the faster form).  Elements of the level and recon arrays that
 * no valid descriptor owns may be overwritten.  Device buffers are kept per
 * host thread and grow to the largest batch. */
XAVS2GPU_API int xavs2gpu_tq_batch_host(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual,
                                        int16_t *coef, int16_t *recon, int32_t *nnz, int chunks);

/* ---- batched motion search -----------------------------------------------
 * Full search + sub-pel refinement of many PUs against device-resident
 * reference planes.  Per PU and reference the result equals the
 * reference's xavs2_me_search (me.c:879-1183) with me_method = full search,
 * candidates {rounded MVP, (0,0)} built as pred_inter_search_single does
 * (md_inter.c:840-865, 957-959), and me_subpel_refine (me.c:479-579). */
typedef struct xavs2gpu_me_params {
    int32_t search_range;     /* full search over [-R, R) on both axes, R <= 128 */
    int32_t lambda_factor;    /* h->i_lambda_factor = round(65536*sqrt(lambda))  */
    int32_t use_hadamard;     /* fpel_cmp: 1 = SATD, 0 = SAD                     */
    int32_t fractional_me;    /* 0 none, 1 half-pel, 2 half + quarter-pel         */
    int32_t fast_sub_me;      /* spiral-2 pattern with step 2                     */
    int32_t enable_pmvr;      /* PMVR restriction of the quarter-pel step         */
} xavs2gpu_me_params_t;

typedef struct xavs2gpu_pu {
    int16_t x, y;             /* luma position of the PU                          */
    uint8_t part, ref;        /* LumaPU index, reference slot                     */
    int16_t mvp_x, mvp_y;     /* predictor, quarter-pel                           */
    int16_t min_x, min_y;     /* integer-pel search limits, inclusive             */
    int16_t max_x, max_y;     /*   (xavs2_me_t mv_min_fpel / mv_max_fpel)         */
} xavs2gpu_pu_t;

typedef struct xavs2gpu_me_result {
    int16_t bmv_x, bmv_y;     /* best MV after refinement, quarter-pel (bmv)      */
    int32_t bcost;            /* its cost (bcost; 1<<30 when no candidate fits)   */
    int32_t mvcost;           /* MV cost of bmv (mvcost[PDIR_FWD])                */
    int16_t imv_x, imv_y;     /* integer-pel best MV (bmv2)                       */
    int32_t icost;            /* integer-pel best cost (bcost2)                   */
} xavs2gpu_me_result_t;

/* Search limits of a PU the way pred_inter_search_single derives them
 * (md_inter.c:910-926): a 64-pixel margin minus 6, the vertical range
 * clipped to [vmin_qpel, vmax_qpel] (encoder.c:852-870). */
XAVS2GPU_API void xavs2gpu_pu_set_limits(xavs2gpu_pu_t *pu, int width, int height, int vmin_qpel, int vmax_qpel);

typedef struct xavs2gpu_me_session xavs2gpu_me_session_t;

/* A session owns device-resident planes for one current picture and
 * `num_refs` reference pictures of width x height (each reference with its
 * 15 quarter-pel planes), a PU list of up to `max_pus` entries, the results
 * and one CUDA stream.  Returns NULL on failure. */
XAVS2GPU_API xavs2gpu_me_session_t *xavs2gpu_me_create(int width, int height, int num_refs, int max_pus);
XAVS2GPU_API void xavs2gpu_me_destroy(xavs2gpu_me_session_t *s);
/* Load a picture: slot -1 = the current picture, 0..num_refs-1 = references
 * (their borders are replicated and their sub-pel planes computed on the
 * device).  _host copies from host memory, _device from device memory.  A
 * page-locked host picture is copied asynchronously on the session stream
 * (keep it unchanged until the stream has passed it, e.g. until the next
 * get_results / sync); pageable memory is copied before the call returns. */
XAVS2GPU_API int xavs2gpu_me_set_picture_host(xavs2gpu_me_session_t *s, int slot, const uint8_t *luma, intptr_t stride);
XAVS2GPU_API int xavs2gpu_me_set_picture_device(xavs2gpu_me_session_t *s, int slot, const uint8_t *luma, intptr_t stride);
/* Set the PU list (host memory).  The list is uploaded and planned once;
 * runs reuse it until the next call. */
XAVS2GPU_API int xavs2gpu_me_set_pus(xavs2gpu_me_session_t *s, const xavs2gpu_pu_t *pus, int n);
/* Run the search for every PU on the session's stream (asynchronous). */
XAVS2GPU_API int xavs2gpu_me_run(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm);
/* Copy the results (one per PU, in list order) to host memory; waits. */
XAVS2GPU_API int xavs2gpu_me_get_results(xavs2gpu_me_session_t *s, xavs2gpu_me_result_t *out);
XAVS2GPU_API int xavs2gpu_me_sync(xavs2gpu_me_session_t *s);
/* Device views for tests and chaining. */
XAVS2GPU_API const xavs2gpu_me_result_t *xavs2gpu_me_results_device(xavs2gpu_me_session_t *s);
XAVS2GPU_API uint8_t *xavs2gpu_me_plane_device(xavs2gpu_me_session_t *s, int slot, int k);
XAVS2GPU_API int xavs2gpu_me_plane_stride(xavs2gpu_me_session_t *s);
/* Copies plane k of a slot, margin included ((W+160) x (H+160) bytes), to
 * host memory with row stride `stride`; waits. */
XAVS2GPU_API int xavs2gpu_me_get_plane(xavs2gpu_me_session_t *s, int slot, int k, uint8_t *out, intptr_t stride);
XAVS2GPU_API int xavs2gpu_me_plane_pad(xavs2gpu_me_session_t *s);
/* 1 when the session's CTU search copies its reference windows with the
 * tensor memory accelerator (a tensor map over the session's planes was
 * encoded), 0 when it uses 16-byte loads.  Results are the same either way. */
XAVS2GPU_API int xavs2gpu_me_window_tma(xavs2gpu_me_session_t *s);
XAVS2GPU_API void *xavs2gpu_me_stream(xavs2gpu_me_session_t *s);
/* Geometry and PU list of a session (host copies). */
XAVS2GPU_API void xavs2gpu_me_session_info(const xavs2gpu_me_session_t *s, int *width, int *height, int *num_refs,
                                           int *n_pus);
XAVS2GPU_API int xavs2gpu_me_session_pus(const xavs2gpu_me_session_t *s, xavs2gpu_pu_t *out);
/* How the last xavs2gpu_me_set_pus split the list: PUs searched by the
 * shared-window CTU kernel and by the per-PU kernel. */
XAVS2GPU_API void xavs2gpu_me_plan_stats(xavs2gpu_me_session_t *s, int *n_ctu_pus, int *n_generic_pus, int *n_ctu_jobs);
/* Phase timing: when enabled, xavs2gpu_me_run records CUDA events on the
 * session stream around its phases; xavs2gpu_me_phase_ms waits and returns
 * the last run's durations in ms: [0] candidates, [1] shared-window CTU
 * search, [2] per-PU search, [3] sub-pel refinement. */
XAVS2GPU_API void xavs2gpu_me_set_profiling(xavs2gpu_me_session_t *s, int enable);
XAVS2GPU_API int xavs2gpu_me_phase_ms(xavs2gpu_me_session_t *s, float ms[4]);
/* Launch shapes of the sub-pel refinement (no counterpart in the reference;
 * results never depend on them): searches of at most refine_split_px
 * pixels refine one per thread, larger ones one per warp; refine_block
 * threads per CTA (32, 64 or 128); cu_groups = 1 refines the partitions of
 * each 16x16..64x64 CU together, sharing the unit costs of partitions with
 * a common centre (faster when partitions agree on their motion, the
 * default), 0 refines every search on its own. */
typedef struct xavs2gpu_me_tuning {
    int32_t refine_split_px;
    int32_t refine_block;
    int32_t cu_groups;
    int32_t pad_;
} xavs2gpu_me_tuning_t;
XAVS2GPU_API int xavs2gpu_me_set_tuning(xavs2gpu_me_session_t *s, const xavs2gpu_me_tuning_t *t);
XAVS2GPU_API int xavs2gpu_me_get_tuning(const xavs2gpu_me_session_t *s, xavs2gpu_me_tuning_t *t);
/* Builds the search plan for prm->search_range now (host work and one
 * stream synchronisation) so that the next xavs2gpu_me_run only enqueues
 * device work -- required before capturing a run into a CUDA graph. */
XAVS2GPU_API int xavs2gpu_me_prepare(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm);
/* Autotuner (no counterpart in the reference): runs the search `reps` times
 * for every candidate refinement split (0..4096 px) and CTA size (64, 128),
 * keeps the fastest and returns its time per run in ms.  The results of a
 * run never depend on the choice. */
XAVS2GPU_API int xavs2gpu_me_autotune(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm, int reps,
                                      float *best_ms);

/* ---- skip / direct rough cost (rdo.c:2366-2480) ---------------------------
 * One candidate of a CU (skip or direct mode, motion derived by the host):
 * the CU (size_log2 3..6, inside the picture), one PU or four quadrant PUs
 * (z-order), per PU the reference slot of list 0 / 1 (-1 unused; both: the
 * average of the two predictions) and quarter-pel vectors, and the mode's
 * header bits.  A CU's candidates are contiguous, in evaluation order. */
typedef struct xavs2gpu_skip_cand {
    int16_t x, y;
    uint8_t size_log2, n_pu;
    int16_t pad_;
    int32_t cu;
    int32_t rate;
    int8_t ref[4][2];
    int16_t mv[4][2][2];
} xavs2gpu_skip_cand_t;
/* Against the current picture and reference planes of a motion-search
 * session: dist[i] = luma SA8D of candidate i's prediction (-1: not
 * evaluated -- same motion as an earlier candidate of its CU, or a bad
 * candidate), cost[i] = dist + lambda * rate (rdcost_t rounding),
 * best[cu] = the first candidate with the strictly smallest cost (-1:
 * none).  Device arrays; stream NULL = the session's stream. */
XAVS2GPU_API int xavs2gpu_skip_costs(xavs2gpu_me_session_t *s, const xavs2gpu_skip_cand_t *cands, int n,
                                     double lambda, int n_cus, int32_t *dist, double *cost, int32_t *best,
                                     void *stream);

/* ---- several pictures per launch -------------------------------------------
 * No counterpart in the reference (its search runs one PU at a time).  The
 * session's work (CTU jobs, per-PU searches, refinements) of up to 256
 * sessions -- pictures of any sizes, each with its own resident references
 * -- is concatenated and searched by one launch of each kernel on `stream`.
 * Results land in each session's own result array, identical to
 * xavs2gpu_me_run on that session alone.  The sessions' pictures must be
 * loaded on `stream` (xavs2gpu_me_set_stream) or before the call. */
typedef struct xavs2gpu_me_batch xavs2gpu_me_batch_t;
XAVS2GPU_API xavs2gpu_me_batch_t *xavs2gpu_me_batch_create(void);
XAVS2GPU_API void xavs2gpu_me_batch_destroy(xavs2gpu_me_batch_t *b);
XAVS2GPU_API int xavs2gpu_me_batch_run(xavs2gpu_me_batch_t *b, xavs2gpu_me_session_t *const *sessions, int n,
                                       const xavs2gpu_me_params_t *prm, void *stream);
/* Make the session enqueue on `stream` (NULL: back to its own stream).  No
 * synchronisation: work already enqueued on the previous stream must be
 * ordered before the next by the caller, and a session must be switched
 * back (or destroyed) before its external stream is destroyed. */
XAVS2GPU_API int xavs2gpu_me_set_stream(xavs2gpu_me_session_t *s, void *stream);
/* Device table of the reference planes in the current slot order: entry
 * 16 r + k = plane k of reference r (updated in place, stream-ordered, by
 * xavs2gpu_me_rotate_refs). */
XAVS2GPU_API const uint8_t *const *xavs2gpu_me_plane_table_device(xavs2gpu_me_session_t *s);
/* Reference r+1 takes over reference r's planes and reference 0 gets the
 * oldest buffer (to be overwritten by the next xavs2gpu_me_set_picture_*
 * of slot 0) -- the reference list update of a P-picture sequence without
 * moving pixels. */
XAVS2GPU_API int xavs2gpu_me_rotate_refs(xavs2gpu_me_session_t *s);

/* ---- full-picture chain ---------------------------------------------------
 * No single counterpart in the reference: the device-side sequence of one
 * P picture over its leaf CUs -- sub-pel planes of every reference
 * (interpolate_lcu_row), the current picture, the batched motion search
 * (xavs2_me_search per PU and reference), and every inter candidate of
 * every leaf CU through the TU chain: each partition mode (2Nx2N, 2NxN,
 * Nx2N, 2NxnU, 2NxnD, nLx2N, nRx2N; 8x8 CUs the first three) predicted PU by
 * PU from the reference with the smallest search cost (mc_luma on the
 * frame's sub-pel planes, mc.c:559-589), its residual (pixel_sub_ps), and
 * dct -> quant -> dequant -> idct both as one CU-sized TU and as the mode's
 * four split TUs (tu_recon_inter_luma, rdo.c:1333-1370; NSQT strips for the
 * asymmetric modes of CUs above 8x8, quarters otherwise, rdo.c:103-192),
 * with the SSD of each reconstruction -- enqueued on the session stream,
 * eagerly or as one captured CUDA graph.  The encoder's RDO (rates from the
 * entropy coder) stays on the host; so that the chain reconstructs a
 * picture, each CU takes the mode with the smallest sum of its PUs' search
 * costs and then the TU variant with the smaller SSD (the first on ties).
 * A CU whose partition PUs are not in the PU list (see below) has the 2Nx2N
 * candidate only. */
typedef struct xavs2gpu_cu {
    int16_t x, y;              /* luma position of the CU (multiples of 8)         */
    int16_t size;              /* 8, 16, 32 or 64                                  */
    int16_t pad_;
    int32_t pu[4];             /* index of the CU's 2Nx2N PU in the session's PU
                                  list for reference 0..3 (-1: not searched); the
                                  mode's other PUs follow it: 2NxN top, bottom,
                                  Nx2N left, right, 2NxnU, 2NxnD, nLx2N, nRx2N
                                  (two each; 8x8 CUs: 2NxN and Nx2N)               */
    int64_t offset;            /* unused by the chain and the server (kept for the
                                  caller's own residual layout)                    */
    int64_t coef_offset;       /* unused likewise                                   */
} xavs2gpu_cu_t;

typedef struct xavs2gpu_chain xavs2gpu_chain_t;
/* `s` must already hold the PU list the CUs index.  flags bit 0 (feedback):
 * after each picture the reference sources shift by one (ref r+1 <- ref r)
 * and the reconstructed picture becomes reference 0, as in an encoder's
 * P-picture loop.  Returns NULL on failure. */
XAVS2GPU_API xavs2gpu_chain_t *xavs2gpu_chain_create(xavs2gpu_me_session_t *s, const xavs2gpu_cu_t *cus, int n_cus,
                                                     int qp, int flags);
XAVS2GPU_API void xavs2gpu_chain_destroy(xavs2gpu_chain_t *c);
/* Device source picture (width x height, stride = width): idx 0 = the
 * current picture, 1 + r = reference r. */
XAVS2GPU_API uint8_t *xavs2gpu_chain_source(xavs2gpu_chain_t *c, int idx);
/* Enqueue one picture eagerly / capture it into a CUDA graph (after one
 * eager run with the same parameters) / launch the captured graph. */
XAVS2GPU_API int xavs2gpu_chain_run(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm);
XAVS2GPU_API int xavs2gpu_chain_capture(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm);
XAVS2GPU_API int xavs2gpu_chain_launch(xavs2gpu_chain_t *c);
/* Device outputs of the last picture.  Candidates are numbered CU by CU,
 * modes in the order above; candidate i owns TU descriptors (and nnz)
 * 5 i (one TU) and 5 i + 1 .. 5 i + 4 (split TUs, in TU order), SSDs 2 i (one
 * TU) and 2 i + 1 (split), and the residual / reconstructed-residual / level
 * regions of its table entry.  The reconstructed picture is width x height,
 * stride = width. */
typedef struct xavs2gpu_cand {
    int32_t cu;                /* CU index                                          */
    int8_t mode;               /* 0 2Nx2N, 1 2NxN, 2 Nx2N, 3 2NxnU, 4 2NxnD, 5 nLx2N, 6 nRx2N */
    int8_t split_type;         /* split TUs: 1 quarters, 2 horizontal strips S x S/4,
                                  3 vertical strips S/4 x S                         */
    int16_t pad_;
    int64_t res_offset;        /* residual and reconstructed residual: S*S elements
                                  of the one TU (row-major), then the four split TUs
                                  (each contiguous, stride = TU width)              */
    int64_t coef_offset;       /* levels, without gaps: the one TU's (S*S; 64: 32*32),
                                  then the split TUs' (each w*h; 64-point: w*h/4)   */
} xavs2gpu_cand_t;
typedef struct xavs2gpu_cu_choice {
    int32_t cand;              /* chosen candidate (index into the candidate table) */
    int16_t mode;              /* its partition mode                                */
    int16_t split;             /* 0 one TU, 1 split TUs                             */
} xavs2gpu_cu_choice_t;
typedef struct xavs2gpu_chain_outputs {
    int16_t *coef;
    int16_t *recon_residual;
    int32_t *nnz;
    xavs2gpu_tq_block_t *blocks;
    uint8_t *recon;
    xavs2gpu_cu_choice_t *choice;
    int64_t n_residual, n_coef;
    const xavs2gpu_cand_t *cands;      /* candidate table (device)                 */
    int32_t *cand_cost;                /* per candidate: sum of its PUs' search costs */
    int32_t *dist;                     /* per candidate: SSD one TU, SSD split TUs  */
    int64_t n_cands;                   /* candidates (TU descriptors: 5 n_cands)    */
} xavs2gpu_chain_outputs_t;
XAVS2GPU_API int xavs2gpu_chain_get_outputs(xavs2gpu_chain_t *c, xavs2gpu_chain_outputs_t *o);
/* Autotuner: times the chain eagerly for every candidate launch shape
 * (refinement split and CTA size, TU-chain warps per CTA), keeps the fastest
 * and returns its mean time per picture in ms (*best_ms).  Results do not
 * depend on the choice.  Invalidates a captured graph. */
typedef struct xavs2gpu_chain_tuning {
    xavs2gpu_me_tuning_t me;
    int32_t tq_warps;          /* warps per CTA of the TU chain: 4 or 8 */
    int32_t pad_;
} xavs2gpu_chain_tuning_t;
XAVS2GPU_API int xavs2gpu_chain_autotune(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm, int reps,
                                         float *best_ms);
XAVS2GPU_API int xavs2gpu_chain_get_tuning(const xavs2gpu_chain_t *c, xavs2gpu_chain_tuning_t *t);
XAVS2GPU_API int xavs2gpu_chain_set_tuning(xavs2gpu_chain_t *c, const xavs2gpu_chain_tuning_t *t);
/* Kernel nodes of the captured graph (what one xavs2gpu_chain_launch runs). */
XAVS2GPU_API int xavs2gpu_chain_graph_kernels(const xavs2gpu_chain_t *c);

/* ---- serving ------------------------------------------------------------------
 * No counterpart in the reference.  Many concurrent streams of different
 * resolutions submit pictures; a scheduler thread batches the arrived
 * pictures (at most one per stream, up to max_batch_frames and
 * max_batch_pixels per batch) and runs every batch with one launch per
 * kernel: reference update and sub-pel planes per picture, the motion search
 * of all pictures (xavs2gpu_me_batch_run), each CU's motion-compensated
 * residual from its best reference, one TU chain over all CUs, the
 * reconstruction and a per-picture checksum.  Each stream keeps its two
 * references and their planes resident; a stream is admitted when its
 * resident memory fits both hbm_budget_bytes (if set) and the device's free
 * memory at that moment (cudaMemGetInfo) less hbm_reserve_bytes and less
 * what streams admitted but not yet allocated will take.  The first two
 * pictures of a stream only fill its
 * references (ref_only results); every later picture is searched against
 * the two before it. */
typedef struct xavs2gpu_server_config {
    int64_t hbm_budget_bytes;    /* device memory the server may hold (0: unlimited) */
    int64_t max_batch_pixels;    /* luma pixels per batch (sizes two batch buffer sets) */
    int32_t max_batch_frames;    /* pictures per batch, 1..256 */
    int32_t qp;                  /* quantiser of every TU */
    xavs2gpu_me_params_t me;     /* search parameters */
    int64_t hbm_reserve_bytes;   /* device memory admission leaves free (0: 1/32 of the device, at least 1 GiB) */
    int64_t batch_pixels_target; /* luma pixels a batch takes while the backlog is short (0: max_batch_pixels);
                                    while more than twice this waits, batches grow up to max_batch_pixels */
} xavs2gpu_server_config_t;

typedef struct xavs2gpu_server_result {
    int32_t stream, frame;       /* stream id, picture number within the stream */
    int64_t tag;                 /* the submitter's tag */
    int64_t t_submit_ns;         /* steady clock at submission */
    int64_t t_done_ns;           /* steady clock when the batch completed */
    uint64_t hash;               /* sum over the 32-bit words w_i of [reconstruction | levels |
                                    search results] of (w_i + 1) * (2 i + 1) mod 2^64; 0 when ref_only */
    int32_t batch_frames;        /* pictures in the batch that carried it */
    int32_t ref_only;
} xavs2gpu_server_result_t;

typedef struct xavs2gpu_server xavs2gpu_server_t;
XAVS2GPU_API xavs2gpu_server_t *xavs2gpu_server_create(const xavs2gpu_server_config_t *cfg);
XAVS2GPU_API void xavs2gpu_server_destroy(xavs2gpu_server_t *s);
/* A stream of width x height pictures with its leaf-CU PU list (2
 * references) and CU list (as for xavs2gpu_chain_create) and `ring` pinned
 * picture slots.  Returns the stream id, or minus an error code
 * (-XAVS2GPU_ERR_CAPACITY when the stream does not fit the budget or the
 * free device memory). */
XAVS2GPU_API int xavs2gpu_server_open_stream(xavs2gpu_server_t *s, int width, int height, const xavs2gpu_pu_t *pus,
                                             int n_pus, const xavs2gpu_cu_t *cus, int n_cus, int ring);
/* Copies the picture into a free slot of the stream and queues it;
 * XAVS2GPU_ERR_CAPACITY when all of the stream's slots are in use. */
XAVS2GPU_API int xavs2gpu_server_submit(xavs2gpu_server_t *s, int stream, const uint8_t *luma, intptr_t stride,
                                        int64_t tag);
/* Completed pictures (waits up to timeout_ms for the first). */
XAVS2GPU_API int xavs2gpu_server_poll(xavs2gpu_server_t *s, xavs2gpu_server_result_t *out, int max, int timeout_ms);
XAVS2GPU_API void xavs2gpu_server_stats(xavs2gpu_server_t *s, int64_t *hbm_used, int64_t *batches, int64_t *frames,
                                        int64_t *pending);
/* Sum over completed batches of their device time (first to last command)
 * and of the scheduler's time to enqueue them, in ms. */
XAVS2GPU_API void xavs2gpu_server_timing(xavs2gpu_server_t *s, double *gpu_ms, double *host_ms);

/* ---- allocation-free motion search ---------------------------------------
 * No counterpart in the reference.  The same search as xavs2gpu_me_run
 * (identical results), for callers that cannot allocate device memory while
 * they run -- e.g. an encoder embedded in a host whose GPU memory comes from
 * the host's own pool, or a latency-critical thread that must not trigger the
 * device-wide synchronisation of cudaMalloc/cudaFree.  The caller passes
 * everything in device memory: `cur` and the 16*num_refs planes of
 * `ref_planes` (a host array; plane 16*r + k is sub-pel position k of
 * reference r, k = 0 the full-pel plane) point at pixel (0,0) of width x
 * height pictures that share `stride` and have an 80-pixel replicated margin
 * (as xavs2gpu_me_plane_device provides); `pus` and `out` hold n entries.
 * Nothing is allocated: the scratch is one fixed device array of about
 * 2.7 MB per GPU, kept until the process exits, limiting a call to 65536
 * PUs and 16 references (larger requests are rejected with
 * XAVS2GPU_ERR_CAPACITY).  The first call on a device looks the array's
 * address up (cudaGetSymbolAddress), so make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU (other streams or
 * threads) race and must be serialised by the caller.  PUs outside the
 * picture or with limits beyond the margin report bcost = 1 << 30.  Kernels
 * run on `stream` (a cudaStream_t, 0 = default); the call does not wait. */
XAVS2GPU_API int xavs2gpu_me_search_noalloc(const uint8_t *cur, int stride, int width, int height,
                                            const uint8_t *const *ref_planes, int num_refs,
                                            const xavs2gpu_pu_t *pus, int n, const xavs2gpu_me_params_t *prm,
                                            xavs2gpu_me_result_t *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* XAVS2_GB300_H */
