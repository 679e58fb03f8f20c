/*
 * enc_calls.h -- the primitive-table entries a recording of the reference
 * encoder covers, and the record format.  TEST INFRASTRUCTURE ONLY.
 *
 * An entry is (kind, slot): kinds follow the member order of xavs2's
 * primitive table (intrinsic_func_t, source/common/primitives.h:131-223;
 * pixel_funcs_t, pixel.h:141-166; dct_funcs_t, primitives.h:101-119), the
 * slot is the array index (LumaPU shape, intra mode, edge direction) or 0.
 *
 * Record format (little endian), one record per sampled call:
 *   u32 magic 'XREC', u16 kind, u16 slot, u32 call_index (per entry),
 *   u16 n_args, u16 reserved, i64 return value (0 for void entries),
 *   then n_args arguments in the callee's parameter order:
 *     u8 type:
 *       'i' int32 scalar  -> i64 value
 *       'p' intptr scalar -> i64 value
 *       'a' pointer array -> i64 count; the next `count` arguments are the
 *           buffers whose pointers form the array (pel_t *const dst[3] ...)
 *       'b' buffer        -> u8 elem_size, u8 flags (1 input snapshot,
 *           2 output snapshot), i16 alias (index of an earlier buffer
 *           argument with the same address, -1 none), i64 stride (elements),
 *           i32 in_r0, in_r1, in_c0, in_c1, i32 out_r0, out_r1, out_c0,
 *           out_c1 (row / column ranges in elements relative to the
 *           pointer), then the input bytes (rows x cols x elem_size, row
 *           major) and the output bytes taken after the call.
 */
#ifndef XAVS2_ENC_CALLS_H
#define XAVS2_ENC_CALLS_H

enum {
    EC_SAD, EC_SATD, EC_SA8D, EC_SSD, EC_SAD_X3, EC_SAD_X4, EC_SUB_PS, EC_ADD_PS,
    EC_COPY_SP, EC_COPY_PS, EC_COPY_SS, EC_COPY_PP, EC_AVG,            /* [25] each */
    EC_MAD, EC_SSD_BLOCK, EC_AVERAGE,                                 /* madf[4], single */
    EC_LUMA_HOR, EC_LUMA_VER, EC_LUMA_EXT, EC_LUMA_VER_X3, EC_LUMA_HOR_X3, EC_LUMA_EXT_X3,
    EC_LUMA_BLOCK_HOR, EC_LUMA_BLOCK_VER, EC_LUMA_BLOCK_EXT,
    EC_CHROMA_BLOCK_HOR, EC_CHROMA_BLOCK_VER, EC_CHROMA_BLOCK_EXT,
    EC_INTRA,                                                         /* [33] */
    EC_DCT, EC_IDCT, EC_DCT_HALF,                                     /* [25] each */
    EC_T4_2ND, EC_INV_T4_2ND, EC_T_2ND, EC_INV_T_2ND, EC_ABS_COEFF, EC_ADD_SIGN, EC_QUANT,
    EC_DEQUANT, EC_WQUANT,
    EC_DEBLOCK_LUMA, EC_DEBLOCK_CHROMA,                               /* [2]: vertical, horizontal edge */
    EC_SAO, EC_LOWRES,
    EC_NUM_KINDS
};

#define EC_MAX_SLOTS 33
#define EC_MAGIC 0x43455258u   /* "XREC" */

/* Address of the oracle's function with the reference entry's signature for
 * (kind, slot), or NULL where the oracle has none (liboracle). */
void *xo_tab_entry(int kind, int slot);

#endif
