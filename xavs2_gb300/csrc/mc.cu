// mc.cu -- AVS2 luma 8-tap / chroma 4-tap interpolation for sm_103a: the
// per-call drop-ins of the intpl_* members of intrinsic_func_t
// (source/common/primitives.h:157-171, C versions mc.c:274-547) and the
// whole-frame quarter-pel plane generation that replaces the reference's
// per-LCU-row interpolate_lcu_row (mc.c:593-785) + plane_expand_border
// (frame.c:471-507).
#include "xavs2gpu_common.cuh"

#include <cstring>

namespace xg {

struct Taps8 { int8_t c[8]; };
struct Taps4 { int8_t c[4]; };

static Taps8 taps8(const int8_t *p) { Taps8 t; memcpy(t.c, p, 8); return t; }
static Taps4 taps4(const int8_t *p) { Taps4 t; memcpy(t.c, p, 4); return t; }

// ---- plane-level filters on packed operands --------------------------------
// All per-call kernels index their operands as (x, y) relative to the block
// origin with explicit strides; the host packs each footprint so the origin
// sits at a fixed offset inside the staging buffer.

// intpl_luma_hor_c (mc.c:403-417): raw 8-tap sum to tmp (int16) and the
// rounded, clipped sample to dst.
__global__ void hor8_kernel(uint8_t *dst, int ds, int16_t *tmp, int ts, const uint8_t *src, int ss, int w, int h,
                            Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[k - 3];
        if (tmp) tmp[y * ts + x] = (int16_t)v;
        if (dst) dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
    }
}

// intpl_luma_ver_c (mc.c:422-435), also the block vertical filter
__global__ void ver8_kernel(uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[(k - 3) * ss];
        dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
    }
}

// intpl_luma_ext_c (mc.c:501-516): vertical 8-tap over int16 raw sums
__global__ void ext8_kernel(uint8_t *dst, int ds, const int16_t *tmp, int ts, int w, int h, Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const int16_t *p = tmp + y * ts + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[(k - 3) * ts];
        dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
    }
}

// intpl_luma_block_ext_c (mc.c:362-398): int16 raw horizontal sums of rows
// -3..h+3 then the vertical pass with +2048 >> 12.
__global__ void block_ext8_kernel(uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps8 tx, Taps8 ty)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint8_t *p = src + (y + k - 3) * ss + x;
            int r = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) r += tx.c[j] * p[j - 3];
            v += ty.c[k] * (int)(int16_t)r;
        }
        dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
    }
}

// intpl_chroma_block_{hor,ver,ext}_c (mc.c:274-337); ext keeps int32 sums
__global__ void chroma4_kernel(int mode, uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps4 tx,
                               Taps4 ty)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
        if (mode == 0) {
#pragma unroll
            for (int k = 0; k < 4; k++) v += tx.c[k] * p[k - 1];
            dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
        } else if (mode == 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) v += ty.c[k] * p[(k - 1) * ss];
            dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint8_t *q = p + (k - 1) * ss;
                int r = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) r += tx.c[j] * q[j - 1];
                v += ty.c[k] * r;
            }
            dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
        }
    }
}

static inline int nblocks(int n, int t = 256) { int b = (n + t - 1) / t; return b < 1 ? 1 : (b > 4096 ? 4096 : b); }

// ---- whole-frame quarter-pel planes ------------------------------------------
// Every sample of plane k = 4*fy + fx at (x, y) equals the AVS2 filter
// evaluated at (clamp(x, -4, W+3), clamp(y, -4, H+3)) with full-pel reads
// clamped into the picture: the reference filters rows [-4, H+4) x columns
// [-4, W+4) and replicates that region outwards.  One kernel writes the
// whole padded plane directly, so the replication costs no extra pass.
__constant__ int8_t c_luma_taps[4][8] = {
    {0, 0, 0, 64, 0, 0, 0, 0},
    {-1, 4, -10, 57, 19, -7, 3, -1},
    {-1, 4, -11, 40, 40, -11, 4, -1},
    {-1, 3, -7, 19, 57, -10, 4, -1},
};

// The three sub-pel phases of one axis from the 8 samples v[0..7] around a
// position.  The AVS2 taps are symmetric (half-pel) and mirror images of
// each other (quarter-pels: t3[k] = t1[7-k]), so with a_k = v[k] + v[7-k] and
// d_k = v[k] - v[7-k]:
//   p2      = -a0 + 4 a1 - 11 a2 + 40 a3
//   2 p1    = S + D,  2 p3 = S - D,
//   S = -2 a0 + 7 a1 - 17 a2 + 76 a3,  D = d1 - 3 d2 + 38 d3
// (exactly the 8-tap sums; 11 multiply-adds for the three phases instead
// of 24).  Returned: p2 and the doubled quarter-pel sums 2 p1, 2 p3.
__device__ __forceinline__ void phases3(const int (&v)[8], int &p2, int &p1x2, int &p3x2)
{
    const int a0 = v[0] + v[7], a1 = v[1] + v[6], a2 = v[2] + v[5], a3 = v[3] + v[4];
    const int d1 = v[1] - v[6], d2 = v[2] - v[5], d3 = v[3] - v[4];
    p2 = -a0 + 4 * a1 - 11 * a2 + 40 * a3;
    const int S = -2 * a0 + 7 * a1 - 17 * a2 + 76 * a3, D = d1 - 3 * d2 + 38 * d3;
    p1x2 = S + D;
    p3x2 = S - D;
}

constexpr int PT_W = 128, PT_H = 16;            // output tile of a padded plane
constexpr int PS_R = PT_H + 7, PS_C = PT_W + 16; // source window (rows, pitch)

struct PlaneSet { uint8_t *p[16]; };

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// Stores the 4 bytes of `v` at p[0..3], only those with column < `end_col`
// when the group straddles the right edge of the padded plane.
template <bool VEC>
__device__ __forceinline__ void store_group(uint8_t *p, uint32_t v, int x, int end_col)
{
    if (VEC && x + 3 < end_col) {
        *reinterpret_cast<uint32_t *>(p) = v;
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (x + i < end_col) p[i] = (uint8_t)(v >> (8 * i));
}

// Phase 3 of frame_planes_kernel for one horizontal phase FX: the 4-column
// group g of output rows [y0 + 8*half, y0 + 8*half + 8).
template <int FX, bool VEC>
__device__ __forceinline__ void planes_rows(const uint8_t (*s_src)[PS_C], const int16_t (*s_hor)[PS_R][PT_W],
                                            const PlaneSet &planes, int stride, int W, int H, int pad, int x0,
                                            int y0, int cx0, int cy0, int g, int half, int mode)
{
    const int xg = x0 + 4 * g;
    const int end_col = W + pad;
    if (xg >= end_col) return;
    int lc[4];
    bool contiguous = true;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        lc[c] = clampi(xg + c, -4, W + 3) - cx0;
        contiguous &= lc[c] == 4 * g + c;
    }
    // window element (row j, column c): the source byte at column lc+3 for
    // FX == 0, else the raw horizontal sum of phase FX
    auto fetch = [&](int row, int (&dst)[4]) {
        if (FX == 0) {
#pragma unroll
            for (int c = 0; c < 4; c++) dst[c] = s_src[row][lc[c] + 3];
        } else if (contiguous) {
            const uint2 pk = *reinterpret_cast<const uint2 *>(&s_hor[FX - 1][row][4 * g]);
            dst[0] = (int16_t)(pk.x & 0xFFFF); dst[1] = (int16_t)(pk.x >> 16);
            dst[2] = (int16_t)(pk.y & 0xFFFF); dst[3] = (int16_t)(pk.y >> 16);
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++) dst[c] = s_hor[FX - 1][row][lc[c]];
        }
    };
    const int ys = y0 + 8 * half;
    int cur = clampi(ys, -4, H + 3) - cy0;
    int win[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) fetch(cur + j, win[j]);
    uint32_t out[4] = {0, 0, 0, 0};
    bool have = false;
    // rolled: the body is the whole per-row filter, and the four phases' code
    // must stay small enough for the instruction cache
#pragma unroll 1
    for (int t = 0; t < 8; t++) {
        const int y = ys + t;
        if (y >= H + pad) break;
        const int l = clampi(y, -4, H + 3) - cy0;
        if (l != cur) {
#pragma unroll
            for (int j = 0; j < 7; j++)
#pragma unroll
                for (int c = 0; c < 4; c++) win[j][c] = win[j + 1][c];
            fetch(l + 7, win[7]);
            cur = l;
            have = false;
        }
        if (!have) {
            // rounding: fx = 0 (bytes) (s + 32) >> 6, else (s + 2048) >> 12;
            // the quarter-pel sums come doubled, one more shift
            constexpr int SH = FX == 0 ? 6 : 12;
            uint32_t pk[4] = {0, 0, 0, 0};
#pragma unroll
            for (int c = 0; c < 4; c++) {
                int v[8];
#pragma unroll
                for (int j = 0; j < 8; j++) v[j] = win[j][c];
                int p2, p1x2, p3x2;
                phases3(v, p2, p1x2, p3x2);
                const int q0 = (win[3][c] + 32) >> 6;
                const int q1 = (p1x2 + (1 << SH)) >> (SH + 1);
                const int q2 = (p2 + (1 << (SH - 1))) >> SH;
                const int q3 = (p3x2 + (1 << SH)) >> (SH + 1);
                pk[0] |= (uint32_t)clip_pel_d(q0) << (8 * c);
                pk[1] |= (uint32_t)clip_pel_d(q1) << (8 * c);
                pk[2] |= (uint32_t)clip_pel_d(q2) << (8 * c);
                pk[3] |= (uint32_t)clip_pel_d(q3) << (8 * c);
            }
#pragma unroll
            for (int fy = 0; fy < 4; fy++) out[fy] = pk[fy];
            have = true;
        }
        const ptrdiff_t ro = (ptrdiff_t)y * stride + xg;
#pragma unroll
        for (int fy = 0; fy < 4; fy++) {
            if (FX == 0 && fy == 0) continue;
            if (mode < 2 && fy != 0 && fy != 2) continue;
            store_group<VEC>(planes.p[4 * fy + FX] + ro, out[fy], xg, end_col);
        }
    }
}

// One CTA writes a 128 x 16 tile of every requested sub-pel plane over the
// whole padded area [-pad, W+pad) x [-pad, H+pad).  The sample at (x, y) is
// the filter output at (cx, cy) = (clamp(x, -4, W+3), clamp(y, -4, H+3)), so
// the tile only needs the clamped columns [cx(x0), cx(x0+127)] and rows
// [cy(y0), cy(y0+15)] (at most 128 x 16 distinct values).
//   phase 1: source window (clamped reads) -> shared memory;
//   phase 2: raw horizontal 8-tap sums for fx = 1..3, 4 columns per item;
//   phase 3: thread = (row half, fx, 4-column group): slides an 8-row window
//            down its 8 output rows and emits planes 4*fy + fx for fy = 0..3
//            as 32-bit stores (a warp writes 128 contiguous bytes of a row).
// resident 256-thread CTAs per SM the register budget is sized for
#ifndef XG_PLANES_MINB
#define XG_PLANES_MINB 3
#endif

template <bool VEC>
__global__ void __launch_bounds__(256, XG_PLANES_MINB) frame_planes_kernel(const uint8_t *__restrict__ src, int stride, int W, int H,
                                                           int pad, PlaneSet planes, int mode)
{
    __shared__ __align__(16) uint8_t s_src[PS_R][PS_C];
    __shared__ __align__(16) int16_t s_hor[3][PS_R][PT_W];
    const int x0 = -pad + blockIdx.x * PT_W, y0 = -pad + blockIdx.y * PT_H;
    const int cx0 = clampi(x0, -4, W + 3), cy0 = clampi(y0, -4, H + 3);
    const int tid = threadIdx.x;
    for (int i = tid; i < PS_R * (PT_W + 8); i += 256) {
        const int r = i / (PT_W + 8), m = i - r * (PT_W + 8);
        const int sy = clampi(cy0 - 3 + r, 0, H - 1), sx = clampi(cx0 - 3 + m, 0, W - 1);
        s_src[r][m] = src[(ptrdiff_t)sy * stride + sx];
    }
    __syncthreads();
    for (int i = tid; i < PS_R * (PT_W / 4); i += 256) {
        const int r = i / (PT_W / 4), g = i - r * (PT_W / 4);
        const uint32_t *w = reinterpret_cast<const uint32_t *>(&s_src[r][4 * g]);
        int b[12];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const uint32_t v = w[q];
#pragma unroll
            for (int e = 0; e < 4; e++) b[4 * q + e] = (v >> (8 * e)) & 0xFF;
        }
        int o[3][4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            int v[8];
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = b[c + k];
            int p2, p1x2, p3x2;
            phases3(v, p2, p1x2, p3x2);
            o[0][c] = p1x2 >> 1;
            o[1][c] = p2;
            o[2][c] = p3x2 >> 1;
        }
#pragma unroll
        for (int f = 0; f < 3; f++) {
            if (mode < 2 && f != 1) continue;
            uint2 pk;
            pk.x = (uint32_t)(o[f][0] & 0xFFFF) | ((uint32_t)o[f][1] << 16);
            pk.y = (uint32_t)(o[f][2] & 0xFFFF) | ((uint32_t)o[f][3] << 16);
            *reinterpret_cast<uint2 *>(&s_hor[f][r][4 * g]) = pk;
        }
    }
    __syncthreads();
    const int g = tid & 31, fx = (tid >> 5) & 3, half = tid >> 7;
    switch (fx) {
    case 0: planes_rows<0, VEC>(s_src, s_hor, planes, stride, W, H, pad, x0, y0, cx0, cy0, g, half, mode); break;
    case 1: if (mode == 2) planes_rows<1, VEC>(s_src, s_hor, planes, stride, W, H, pad, x0, y0, cx0, cy0, g, half, mode); break;
    case 2: planes_rows<2, VEC>(s_src, s_hor, planes, stride, W, H, pad, x0, y0, cx0, cy0, g, half, mode); break;
    default: if (mode == 2) planes_rows<3, VEC>(s_src, s_hor, planes, stride, W, H, pad, x0, y0, cx0, cy0, g, half, mode); break;
    }
}

// Writes the padding of a full-pel plane: (x, y) outside [0, W) x [0, H)
// takes the sample at (clamp(x, 0, W-1), clamp(y, 0, H-1)) (plane_expand_border,
// frame.c:471-507).  One grid row per picture row; 4 columns per thread.
template <bool VEC>
__global__ void expand_plane_kernel(uint8_t *pix, int stride, int W, int H, int pad)
{
    const int groups = (W + 2 * pad + 3) / 4, end_col = W + pad;
    const int y = -pad + (int)blockIdx.y;
    const bool inner_row = y >= 0 && y < H;
    const uint8_t *srow = pix + (ptrdiff_t)clampi(y, 0, H - 1) * stride;
    uint8_t *drow = pix + (ptrdiff_t)y * stride;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < groups; gi += gridDim.x * blockDim.x) {
        const int x = -pad + 4 * gi;
        if (inner_row && x >= 0 && x + 3 < W) continue;
        uint32_t v = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) v |= (uint32_t)srow[clampi(x + c, 0, W - 1)] << (8 * c);
        if (!inner_row) {
            store_group<VEC>(drow + x, v, x, end_col);
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++)
                if ((x + c < 0 || x + c >= W) && x + c < end_col) drow[x + c] = (uint8_t)(v >> (8 * c));
        }
    }
}

}  // namespace xg

using namespace xg;

// ---- per-call drop-ins --------------------------------------------------------
// Footprints: hor reads columns [-3, w+4], ver rows [-3, h+4], ext reads tmp
// rows [-3, h+4]; the luma block ext reads rows [-3, h+3] x columns [-3,
// w+4]; chroma reads [-1, +2] around the block.

namespace {

struct Stage {
    CallCtx &c;
    size_t used = 0;
    explicit Stage(size_t need) : c(call_ctx(need)) {}
    size_t take(size_t bytes) { size_t o = used; used += align_up(bytes); return o; }
    uint8_t *h(size_t o) { return c.h_stage + o; }
    uint8_t *d(size_t o) { return c.d_stage + o; }
};

// Bytes needed for a footprint of `cols` x `rows` elements of `es` bytes.
inline size_t fp(int cols, int rows, int es) { return align_up((size_t)cols * rows * es); }

}  // namespace

extern "C" void xavs2gpu_intpl_luma_hor(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, uint8_t *src, int i_src,
                                        int width, int height, const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7;
    Stage s(fp(fw, height, 1) + fp(width, height, 1) + fp(width, height, 2) + 1024);
    size_t oi = s.take((size_t)fw * height), od = s.take((size_t)width * height), ot = s.take((size_t)width * height * 2);
    pack_rows(s.h(oi), src - 3, i_src, fw, height);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * height, cudaMemcpyHostToDevice, s.c.stream));
    hor8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>((uint8_t *)s.d(od), width, (int16_t *)s.d(ot), width,
                                                                 s.d(oi) + 3, fw, width, height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), s.used - od, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
    unpack_rows(tmp, (intptr_t)i_tmp * 2, s.h(ot), width * 2, height);
}

extern "C" void xavs2gpu_intpl_luma_hor_x3(uint8_t *const dst[3], int i_dst, int16_t *const tmp[3], int i_tmp,
                                           uint8_t *src, int i_src, int width, int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_hor(dst[k], i_dst, tmp[k], i_tmp, src, i_src, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                        const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fh = height + 7;
    Stage s(fp(width, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)width * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3 * (intptr_t)i_src, i_src, width, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)width * fh, cudaMemcpyHostToDevice, s.c.stream));
    ver8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, s.d(oi) + 3 * width, width, width,
                                                                 height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_ver_x3(uint8_t *const dst[3], int i_dst, uint8_t *src, int i_src, int width,
                                           int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_ver(dst[k], i_dst, src, i_src, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_ext(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, int width, int height,
                                        const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fh = height + 7;
    Stage s(fp(width, fh, 2) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)width * fh * 2), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), tmp - 3 * (intptr_t)i_tmp, (intptr_t)i_tmp * 2, width * 2, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)width * fh * 2, cudaMemcpyHostToDevice, s.c.stream));
    ext8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, (const int16_t *)s.d(oi) + 3 * width,
                                                                 width, width, height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_ext_x3(uint8_t *const dst[3], int i_dst, int16_t *tmp, int i_tmp, int width,
                                           int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_ext(dst[k], i_dst, tmp, i_tmp, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7;
    Stage s(fp(fw, height, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * height), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3, i_src, fw, height);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * height, cudaMemcpyHostToDevice, s.c.stream));
    hor8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, nullptr, 0, s.d(oi) + 3, fw, width,
                                                                 height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff)
{
    xavs2gpu_intpl_luma_ver(dst, i_dst, src, i_src, width, height, coeff);
}

extern "C" void xavs2gpu_intpl_luma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff_x, const int8_t *coeff_y)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7, fh = height + 7;
    Stage s(fp(fw, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3 * (intptr_t)i_src - 3, i_src, fw, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * fh, cudaMemcpyHostToDevice, s.c.stream));
    block_ext8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, s.d(oi) + 3 * fw + 3, fw, width,
                                                                       height, taps8(coeff_x), taps8(coeff_y));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

static void chroma_call(int mode, uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                        const int8_t *cx, const int8_t *cy)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 3, fh = height + 3;
    Stage s(fp(fw, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - (intptr_t)i_src - 1, i_src, fw, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * fh, cudaMemcpyHostToDevice, s.c.stream));
    Taps4 tx = taps4(cx ? cx : cy), ty = taps4(cy ? cy : cx);
    chroma4_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(mode, s.d(od), width, s.d(oi) + fw + 1, fw, width,
                                                                    height, tx, ty);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_chroma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff)
{
    chroma_call(0, dst, i_dst, src, i_src, width, height, coeff, nullptr);
}

extern "C" void xavs2gpu_intpl_chroma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff)
{
    chroma_call(1, dst, i_dst, src, i_src, width, height, nullptr, coeff);
}

extern "C" void xavs2gpu_intpl_chroma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff_x, const int8_t *coeff_y)
{
    chroma_call(2, dst, i_dst, src, i_src, width, height, coeff_x, coeff_y);
}

// ---- whole-frame planes (device pointers) ---------------------------------------
extern "C" int xavs2gpu_interpolate_frame(const uint8_t *src, int stride, int width, int height, int pad,
                                          uint8_t *const planes[16], int mode, void *stream)
{
    if (width <= 0 || height <= 0 || pad < 4 || stride < width + 2 * pad || (mode != 1 && mode != 2)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_interpolate_frame", "bad geometry or mode");
        return XAVS2GPU_ERR_ARG;
    }
    PlaneSet ps;
    int mask = 0;
    for (int k = 0; k < 16; k++) {
        ps.p[k] = planes[k];
        bool want = k > 0 && (mode == 2 || k == 2 || k == 8 || k == 10);
        if (want) {
            if (!planes[k]) {
                fail(XAVS2GPU_ERR_ARG, "xavs2gpu_interpolate_frame", "missing output plane");
                return XAVS2GPU_ERR_ARG;
            }
            mask |= 1 << k;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    bool vec = stride % 4 == 0;
    for (int k = 1; k < 16; k++)
        if ((mask >> k) & 1) vec &= ((uintptr_t)planes[k] - (uintptr_t)pad) % 4 == 0;
    dim3 grid((width + 2 * pad + PT_W - 1) / PT_W, (height + 2 * pad + PT_H - 1) / PT_H);
    if (vec)
        frame_planes_kernel<true><<<grid, 256, 0, st>>>(src, stride, width, height, pad, ps, mode);
    else
        frame_planes_kernel<false><<<grid, 256, 0, st>>>(src, stride, width, height, pad, ps, mode);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_expand_border(uint8_t *pix, int stride, int width, int height, int pad, void *stream)
{
    if (width <= 0 || height <= 0 || pad < 0 || stride < width + 2 * pad) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_expand_border", "bad geometry");
        return XAVS2GPU_ERR_ARG;
    }
    const bool vec = stride % 4 == 0 && ((uintptr_t)pix - (uintptr_t)pad) % 4 == 0;
    const int groups = (width + 2 * pad + 3) / 4;
    dim3 grid((groups + 255) / 256, height + 2 * pad);
    if (vec)
        expand_plane_kernel<true><<<grid, 256, 0, (cudaStream_t)stream>>>(pix, stride, width, height, pad);
    else
        expand_plane_kernel<false><<<grid, 256, 0, (cudaStream_t)stream>>>(pix, stride, width, height, pad);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
