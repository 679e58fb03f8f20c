// cand.cuh -- the inter candidates of leaf CUs through the transform chain,
// shared by the full-picture chain (chain.cu) and the server (serve.cu).
//
// A candidate is one partition mode of a CU (2Nx2N, 2NxN, Nx2N, 2NxnU, 2NxnD,
// nLx2N, nRx2N; 8x8 CUs have the first three): every PU of the mode is
// predicted from the reference whose search returned its smallest cost
// (lowest index on ties) at that search's MV (mc_luma on the frame's sub-pel
// planes, mc.c:559-589), the CU's residual is formed (pixel_sub_ps), and the
// residual goes through dct -> quant -> dequant -> idct both as one CU-sized
// TU and as the four TUs of the mode's TU split (tu_recon_inter_luma,
// rdo.c:1333-1370; split type cu_set_tu_split_type, rdo.c:183-192 with
// TU_SPLIT_TYPE, rdo.c:103-116, NSQT on: horizontal strips for the 2NxN-type
// modes and vertical strips for the Nx2N-type modes of CUs above 8x8,
// quarters otherwise; i_level one below the CU's, rdo.c:1440-1463).  For
// every candidate and TU variant the kernels report the levels, nnz, the
// reconstructed residual and the SSD of the reconstruction.  The encoder's
// RDO (rates from the entropy coder) is out of scope; so that the chain has a
// reconstruction to feed back, each CU takes the mode with the smallest sum
// of its PUs' search costs and then the TU variant with the smaller SSD (the
// first on ties).
#pragma once

#include "xavs2gpu_common.cuh"

#include <vector>

namespace xg {

// The picture a group of candidates belongs to.  The chain has one; a
// serving batch has one per picture, found from the batch-wide indices.
struct PicView {
    const uint8_t *cur;                 // current picture (stride `stride`)
    const uint8_t *const *planes;       // reference planes, 16 r + k (stride `stride`)
    const xavs2gpu_me_result_t *res;    // search results of the picture's PU list
    const xavs2gpu_cu_t *cus;           // leaf CUs
    const xavs2gpu_cand_t *cands;       // candidate table (picture-local offsets)
    const int32_t *cu_cand;             // per CU: first candidate; [n_cus] = number of candidates
    const int32_t *cand_units;          // work units over candidates: candidate << 2 | chunk
    const int32_t *cu_units;            // work units over CUs: CU << 2 | chunk
    uint8_t *recon;                     // reconstructed picture (stride `width`)
    unsigned long long *hash;           // serving checksum
    int64_t res_off, coef_off;          // base of the picture in the batch residual / level buffers
    int64_t cu_start;                   // first batch-wide CU index of the picture
    int64_t cand_start;                 // first batch-wide candidate index of the picture
    int64_t cand_unit_start, cu_unit_start;   // first batch-wide work units of the picture
    int64_t n_coef;                     // levels of the picture
    int n_cus, n_cands, stride, width, height, nrefs, n_pus;
};

// view holding batch-wide index i of a field with the given start member
template <int64_t PicView::*START>
__device__ __forceinline__ int find_view(const PicView *v, int nviews, int64_t i)
{
    int lo = 0, hi = nviews - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (v[mid].*START <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// PU k of a mode (0 or 1) covers pixel (xx, yy) of the S x S CU
__device__ __forceinline__ int mode_pu_of(int mode, int S, int xx, int yy)
{
    switch (mode) {
    case 1: return yy >= S / 2;
    case 2: return xx >= S / 2;
    case 3: return yy >= S / 4;
    case 4: return yy >= 3 * S / 4;
    case 5: return xx >= S / 4;
    case 6: return xx >= 3 * S / 4;
    default: return 0;
    }
}

// position of partition PU `k` of `mode` after the CU's 2Nx2N PU in the PU
// list (2Nx2N; 2NxN top, bottom; Nx2N left, right; then the AMP pairs)
__device__ __forceinline__ int mode_pu_index(int mode, int k) { return mode == 0 ? 0 : 2 * mode - 1 + k; }

// element offset of CU pixel (xx, yy) inside the four split TUs (each TU
// contiguous, in TU order)
__device__ __forceinline__ int split_offset(int split_type, int S, int xx, int yy)
{
    const int lq = 29 - __clz(S);                    // log2(S / 4)
    if (split_type == 2)                             // horizontal strips S x S/4
        return ((yy >> lq) << (2 * lq + 2)) + ((yy & ((1 << lq) - 1)) << (lq + 2)) + xx;
    if (split_type == 3)                             // vertical strips S/4 x S
        return ((xx >> lq) << (2 * lq + 2)) + (yy << lq) + (xx & ((1 << lq) - 1));
    const int lh = lq + 1, h = S >> 1;               // quarters
    return (((yy >> lh) * 2 + (xx >> lh)) << (2 * lh)) + ((yy & (h - 1)) << lh) + (xx & (h - 1));
}

__device__ __forceinline__ int luma_part(int w, int h)
{
    // LumaPU index of the TU shapes (pixel.h:50-65)
    if (w == h) return w == 4 ? 0 : w == 8 ? 1 : w == 16 ? 2 : w == 32 ? 3 : 4;
    if (w == 16 && h == 4) return 15;
    if (w == 4 && h == 16) return 16;
    if (w == 32 && h == 8) return 19;
    if (w == 8 && h == 32) return 20;
    if (w == 64 && h == 16) return 23;
    return 24;                                       // 16x64
}

// Best reference of partition PU k of a CU: the CU record holds its 2Nx2N
// PU per reference and the mode's PUs follow it.  (The record is read from
// global memory: a local copy indexed by the reference would live on the
// stack.)
struct PuPick { int ref, mvx, mvy, cost; };
__device__ __forceinline__ PuPick best_ref(const PicView &v, const xavs2gpu_cu_t *cp, int k)
{
    PuPick p{0, 0, 0, 0};
    for (int r = 0; r < v.nrefs; r++) {
        const xavs2gpu_me_result_t q = v.res[cp->pu[r] + k];
        if (r == 0 || q.bcost < p.cost) p = PuPick{r, q.bmv_x, q.bmv_y, q.bcost};
    }
    return p;
}

__device__ __forceinline__ const uint8_t *pred_ptr(const PicView &v, int cx, int cy, const PuPick &p)
{
    return v.planes[p.ref * 16 + ((p.mvy & 3) << 2) + (p.mvx & 3)] + (ptrdiff_t)(cy + (p.mvy >> 2)) * v.stride + cx +
           (p.mvx >> 2);
}

// Four-pixel groups.  CU sizes and TU sides are powers of two, PU and TU
// boundaries inside a CU fall on multiples of 4 columns (the 8x8 CUs have no
// AMP modes and split into 4x4 quarters), so the 4 pixels of a group share
// their PU and their TU row: one 32-bit source word, one unaligned
// prediction word and one 8-byte residual word per group.

// 4 bytes at any address (two aligned words and a byte permute)
__device__ __forceinline__ uint32_t load4u(const uint8_t *p)
{
    const uintptr_t a = (uintptr_t)p;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    return __byte_perm(w[0], w[1], 0x3210u + 0x1111u * (uint32_t)(a & 3));
}

// bytes 0,1 / 2,3 of a word as two zero-extended halfwords
__device__ __forceinline__ uint32_t lo_pairs(uint32_t b) { return __byte_perm(b, 0, 0x7170); }
__device__ __forceinline__ uint32_t hi_pairs(uint32_t b) { return __byte_perm(b, 0, 0x7372); }

// src - pred of 4 pixels as 4 int16 (pixel_sub_ps)
__device__ __forceinline__ uint2 sub4_s16(uint32_t s4, uint32_t p4)
{
    return make_uint2(__vsub2(lo_pairs(s4), lo_pairs(p4)), __vsub2(hi_pairs(s4), hi_pairs(p4)));
}

// clip(pred + residual) of 4 pixels as bytes: pred + residual saturates at
// the int16 limits, which the clip to [0, 255] then removes exactly
__device__ __forceinline__ uint32_t recon4(uint32_t p4, uint2 r)
{
    const uint32_t lo = __vmins2(__vmaxs2(__vaddss2(lo_pairs(p4), r.x), 0u), 0x00ff00ffu);
    const uint32_t hi = __vmins2(__vmaxs2(__vaddss2(hi_pairs(p4), r.y), 0u), 0x00ff00ffu);
    return __byte_perm(lo, hi, 0x6420);
}

// acc + sum of squared differences of 4 byte pairs
__device__ __forceinline__ unsigned ssd4(uint32_t a, uint32_t b, unsigned acc)
{
    const unsigned d = __vabsdiffu4(a, b);
    return __dp4a(d, d, acc);
}

// Work units: a warp takes at most kUnitPx pixels of a candidate (residual,
// SSD) or of a CU (reconstruction); the 64x64 CUs split into 4 units, so no
// warp runs four times longer than the rest of the launch.
constexpr int kUnitPx = 1024;
static inline void build_units(const xavs2gpu_cu_t *cus, int n_cus, const xavs2gpu_cand_t *cands, int n_cands,
                               std::vector<int32_t> &units, int &n_cand_units, int &n_cu_units)
{
    units.clear();
    for (int i = 0; i < n_cands; i++) {
        const int S = cus[cands[i].cu].size, nu = S * S > kUnitPx ? S * S / kUnitPx : 1;
        for (int k = 0; k < nu; k++) units.push_back(i << 2 | k);
    }
    n_cand_units = (int)units.size();
    for (int c = 0; c < n_cus; c++) {
        const int S = cus[c].size, nu = S * S > kUnitPx ? S * S / kUnitPx : 1;
        for (int k = 0; k < nu; k++) units.push_back(c << 2 | k);
    }
    n_cu_units = (int)units.size() - n_cand_units;
}

// Warp per candidate unit: prediction and residual in both TU layouts; the
// first unit of a candidate also writes its five TU descriptors, the sum of
// the mode's search costs and zeroes its two SSDs.
static __global__ void __launch_bounds__(128) cand_residual_kernel(const PicView *__restrict__ views, int nviews, int64_t n,
                                                            int qp, int16_t *__restrict__ residual,
                                                            xavs2gpu_tq_block_t *__restrict__ blocks,
                                                            int32_t *__restrict__ cand_cost, int32_t *__restrict__ dist)
{
    const int lane = threadIdx.x & 31;
    const int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (u >= n) return;
    const PicView &v = views[find_view<&PicView::cand_unit_start>(views, nviews, u)];
    const int32_t ue = v.cand_units[u - v.cand_unit_start];
    const int chunk = ue & 3;
    const int64_t i = v.cand_start + (ue >> 2);
    const xavs2gpu_cand_t cd = v.cands[ue >> 2];
    const xavs2gpu_cu_t *cp = v.cus + cd.cu;
    const int cx = cp->x, cy = cp->y, S = cp->size, lg = 31 - __clz(S), mode = cd.mode;
    const PuPick p0 = best_ref(v, cp, mode_pu_index(mode, 0));
    const PuPick p1 = mode ? best_ref(v, cp, mode_pu_index(mode, 1)) : p0;
    const uint8_t *pr0 = pred_ptr(v, cx, cy, p0), *pr1 = pred_ptr(v, cx, cy, p1);
    const uint8_t *src = v.cur + (ptrdiff_t)cy * v.stride + cx;
    int16_t *whole = residual + v.res_off + cd.res_offset, *split = whole + S * S;
    const int e1 = min(S * S, (chunk + 1) * kUnitPx);
    for (int e = chunk * kUnitPx + 4 * lane; e < e1; e += 128) {
        const int yy = e >> lg, xx = e & (S - 1);
        const ptrdiff_t o = (ptrdiff_t)yy * v.stride + xx;
        const uint8_t *pr = mode_pu_of(mode, S, xx, yy) ? pr1 : pr0;
        const uint2 r = sub4_s16(*reinterpret_cast<const uint32_t *>(src + o), load4u(pr + o));
        *reinterpret_cast<uint2 *>(whole + e) = r;
        *reinterpret_cast<uint2 *>(split + split_offset(cd.split_type, S, xx, yy)) = r;
    }
    if (chunk) return;
    if (lane < 5) {
        xavs2gpu_tq_block_t b;
        b.qp = qp;
        b.flags = 0;
        b.pad_ = 0;
        if (lane == 0) {
            b.offset = v.res_off + cd.res_offset;
            b.coef_offset = v.coef_off + cd.coef_offset;
            b.part = luma_part(S, S);
        } else {
            const int t = lane - 1;
            const int tw = cd.split_type == 3 ? S >> 2 : cd.split_type == 2 ? S : S >> 1;
            const int th = cd.split_type == 2 ? S >> 2 : cd.split_type == 3 ? S : S >> 1;
            const int wav = (tw == 64 || th == 64) ? 2 : 0;   // 64-point shapes keep a quarter of the levels
            b.offset = v.res_off + cd.res_offset + S * S + (int64_t)t * tw * th;
            b.coef_offset = v.coef_off + cd.coef_offset + (S == 64 ? 1024 : S * S) + (int64_t)t * ((tw * th) >> wav);
            b.part = luma_part(tw, th);
        }
        blocks[5 * i + lane] = b;
    }
    if (lane == 0) cand_cost[i] = p0.cost + (mode ? p1.cost : 0);
    if (lane < 2) dist[2 * i + lane] = 0;
}

// Warp per candidate unit: SSD of clip(pred + reconstructed residual) against
// the current picture for both TU variants, added into dist[2 i] (one TU) and
// dist[2 i + 1] (split).
static __global__ void __launch_bounds__(128) cand_eval_kernel(const PicView *__restrict__ views, int nviews, int64_t n,
                                                        const int16_t *__restrict__ rres, int32_t *__restrict__ dist)
{
    const int lane = threadIdx.x & 31;
    const int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (u >= n) return;
    const PicView &v = views[find_view<&PicView::cand_unit_start>(views, nviews, u)];
    const int32_t ue = v.cand_units[u - v.cand_unit_start];
    const int chunk = ue & 3;
    const int64_t i = v.cand_start + (ue >> 2);
    const xavs2gpu_cand_t cd = v.cands[ue >> 2];
    const xavs2gpu_cu_t *cp = v.cus + cd.cu;
    const int cx = cp->x, cy = cp->y, S = cp->size, lg = 31 - __clz(S), mode = cd.mode;
    const PuPick p0 = best_ref(v, cp, mode_pu_index(mode, 0));
    const PuPick p1 = mode ? best_ref(v, cp, mode_pu_index(mode, 1)) : p0;
    const uint8_t *pr0 = pred_ptr(v, cx, cy, p0), *pr1 = pred_ptr(v, cx, cy, p1);
    const uint8_t *src = v.cur + (ptrdiff_t)cy * v.stride + cx;
    const int16_t *whole = rres + v.res_off + cd.res_offset, *split = whole + S * S;
    unsigned d0 = 0, d1 = 0;
    const int e1 = min(S * S, (chunk + 1) * kUnitPx);
    for (int e = chunk * kUnitPx + 4 * lane; e < e1; e += 128) {
        const int yy = e >> lg, xx = e & (S - 1);
        const ptrdiff_t o = (ptrdiff_t)yy * v.stride + xx;
        const uint32_t p4 = load4u((mode_pu_of(mode, S, xx, yy) ? pr1 : pr0) + o);
        const uint32_t s4 = *reinterpret_cast<const uint32_t *>(src + o);
        d0 = ssd4(s4, recon4(p4, *reinterpret_cast<const uint2 *>(whole + e)), d0);
        d1 = ssd4(s4, recon4(p4, *reinterpret_cast<const uint2 *>(split + split_offset(cd.split_type, S, xx, yy))), d1);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        d0 += __shfl_xor_sync(0xffffffffu, d0, o);
        d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    }
    if (lane == 0) {
        atomicAdd(&dist[2 * i], (int32_t)d0);
        atomicAdd(&dist[2 * i + 1], (int32_t)d1);
    }
}

// Warp per CU unit: the mode with the smallest search cost, then the TU
// variant with the smaller SSD; its reconstruction into the picture (the
// unit's pixels); the first unit records the choice.
static __global__ void __launch_bounds__(128) cand_choose_kernel(const PicView *__restrict__ views, int nviews, int64_t n,
                                                          const int32_t *__restrict__ cand_cost,
                                                          const int32_t *__restrict__ dist,
                                                          const int16_t *__restrict__ rres,
                                                          xavs2gpu_cu_choice_t *__restrict__ choice)
{
    const int lane = threadIdx.x & 31;
    const int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (u >= n) return;
    const PicView &v = views[find_view<&PicView::cu_unit_start>(views, nviews, u)];
    const int32_t ue = v.cu_units[u - v.cu_unit_start];
    const int chunk = ue & 3, ci = ue >> 2;
    const int64_t i = v.cu_start + ci;
    const int64_t first = v.cand_start + v.cu_cand[ci], last = v.cand_start + v.cu_cand[ci + 1];
    int64_t best = first;
    for (int64_t k = first + 1; k < last; k++)
        if (cand_cost[k] < cand_cost[best]) best = k;
    const int split = dist[2 * best + 1] < dist[2 * best];
    const xavs2gpu_cand_t cd = v.cands[best - v.cand_start];
    const xavs2gpu_cu_t *cp = v.cus + ci;
    const int cx = cp->x, cy = cp->y, S = cp->size, lg = 31 - __clz(S), mode = cd.mode;
    const PuPick p0 = best_ref(v, cp, mode_pu_index(mode, 0));
    const PuPick p1 = mode ? best_ref(v, cp, mode_pu_index(mode, 1)) : p0;
    const uint8_t *pr0 = pred_ptr(v, cx, cy, p0), *pr1 = pred_ptr(v, cx, cy, p1);
    const int16_t *r = rres + v.res_off + cd.res_offset + (split ? S * S : 0);
    uint8_t *o = v.recon + (ptrdiff_t)cy * v.width + cx;
    const bool aligned = (v.width & 3) == 0;     // word stores into the reconstruction
    const int e1 = min(S * S, (chunk + 1) * kUnitPx);
    for (int e = chunk * kUnitPx + 4 * lane; e < e1; e += 128) {
        const int yy = e >> lg, xx = e & (S - 1);
        const uint32_t p4 = load4u((mode_pu_of(mode, S, xx, yy) ? pr1 : pr0) + (ptrdiff_t)yy * v.stride + xx);
        const uint32_t q = recon4(p4, *reinterpret_cast<const uint2 *>(r + (split ? split_offset(cd.split_type, S, xx, yy) : e)));
        uint8_t *d = o + (ptrdiff_t)yy * v.width + xx;
        if (aligned) {
            *reinterpret_cast<uint32_t *>(d) = q;
        } else {
            d[0] = (uint8_t)q; d[1] = (uint8_t)(q >> 8); d[2] = (uint8_t)(q >> 16); d[3] = (uint8_t)(q >> 24);
        }
    }
    if (lane == 0 && chunk == 0) {
        xavs2gpu_cu_choice_t ch;
        ch.cand = (int32_t)(best - v.cand_start);
        ch.mode = (int16_t)mode;
        ch.split = (int16_t)split;
        choice[i] = ch;
    }
}

}  // namespace xg
