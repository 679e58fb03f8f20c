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
// [-4, W+4) and replicates that region outwards.  Pass 1 computes that
// region tile by tile; pass 2 replicates it into the padding.
__constant__ int8_t c_luma_taps[4][8] = {
    {0, 0, 0, 64, 0, 0, 0, 0},
    {-1, 4, -10, 57, 19, -7, 3, -1},
    {-1, 4, -11, 40, 40, -11, 4, -1},
    {-1, 3, -7, 19, 57, -10, 4, -1},
};

constexpr int TW = 32, TH = 16;   // output tile

struct PlaneSet { uint8_t *p[16]; };

// 256 threads: each computes 2 vertically adjacent outputs of the tile for
// every requested plane.
__global__ void __launch_bounds__(256) frame_subpel_kernel(const uint8_t *__restrict__ src, int stride, int W, int H,
                                                           PlaneSet planes, int mode)
{
    __shared__ uint8_t s_src[TH + 7][TW + 8];       // rows y0-3 .. y0+TH+3, cols x0-3 .. x0+TW+4
    __shared__ int16_t s_hor[3][TH + 7][TW];        // raw horizontal sums for fx = 1..3
    const int x0 = -4 + blockIdx.x * TW, y0 = -4 + blockIdx.y * TH;
    const int tid = threadIdx.x;
    for (int i = tid; i < (TH + 7) * (TW + 8); i += 256) {
        int r = i / (TW + 8), c = i - r * (TW + 8);
        int sy = min(max(y0 - 3 + r, 0), H - 1);
        int sx = min(max(x0 - 3 + c, 0), W - 1);
        s_src[r][c] = src[(size_t)sy * stride + sx];
    }
    __syncthreads();
    for (int i = tid; i < 3 * (TH + 7) * TW; i += 256) {
        int f = i / ((TH + 7) * TW), rem = i - f * (TH + 7) * TW;
        int r = rem / TW, c = rem - r * TW;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += c_luma_taps[f + 1][k] * s_src[r][c + k];
        s_hor[f][r][c] = (int16_t)v;
    }
    __syncthreads();
    const int tx = tid & (TW - 1), ty = (tid >> 5) * 2;
    const int X = x0 + tx;
    if (X >= W + 4) return;
#pragma unroll
    for (int dy = 0; dy < 2; dy++) {
        const int r = ty + dy, Y = y0 + r;
        if (Y >= H + 4) break;
        const size_t o = (ptrdiff_t)Y * stride + X;
#pragma unroll
        for (int k = 1; k < 16; k++) {
            if (mode < 2 && !(k == 2 || k == 8 || k == 10)) continue;
            const int fx = k & 3, fy = k >> 2;
            int v = 0;
            uint8_t out;
            if (fy == 0) {
                out = clip_pel_d((s_hor[fx - 1][r + 3][tx] + 32) >> 6);
            } else if (fx == 0) {
#pragma unroll
                for (int j = 0; j < 8; j++) v += c_luma_taps[fy][j] * s_src[r + j][tx + 3];
                out = clip_pel_d((v + 32) >> 6);
            } else {
#pragma unroll
                for (int j = 0; j < 8; j++) v += c_luma_taps[fy][j] * s_hor[fx - 1][r + j][tx];
                out = clip_pel_d((v + 2048) >> 12);
            }
            planes.p[k][o] = out;
        }
    }
}

// Pass 2: replicate the computed region [-4, W+4) x [-4, H+4) of each
// requested plane into [-pad, W+pad) x [-pad, H+pad).  `lo`/`hi` give the
// region that is already valid (lo = -4, hi = W+4 / H+4 for sub-pel planes,
// 0 / W / H for a full-pel plane).
__global__ void expand_kernel(PlaneSet planes, int nplanes_mask, int stride, int W, int H, int pad, int lox, int hix,
                              int loy, int hiy)
{
    const int PW = W + 2 * pad, PH = H + 2 * pad;
    const int64_t total = (int64_t)PW * PH;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int y = (int)(i / PW) - pad, x = (int)(i % PW) - pad;
        int cx = min(max(x, lox), hix - 1), cy = min(max(y, loy), hiy - 1);
        if (cx == x && cy == y) continue;
        for (int k = 0; k < 16; k++) {
            if (!((nplanes_mask >> k) & 1)) continue;
            uint8_t *p = planes.p[k];
            p[(ptrdiff_t)y * stride + x] = p[(ptrdiff_t)cy * stride + cx];
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
    dim3 grid((width + 8 + TW - 1) / TW, (height + 8 + TH - 1) / TH);
    frame_subpel_kernel<<<grid, 256, 0, st>>>(src, stride, width, height, ps, mode);
    count_launch();
    int64_t total = (int64_t)(width + 2 * pad) * (height + 2 * pad);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    expand_kernel<<<blocks, 256, 0, st>>>(ps, mask, stride, width, height, pad, -4, width + 4, -4, height + 4);
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
    PlaneSet ps;
    memset(&ps, 0, sizeof(ps));
    ps.p[0] = pix;
    int64_t total = (int64_t)(width + 2 * pad) * (height + 2 * pad);
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    expand_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(ps, 1, stride, width, height, pad, 0, width, 0, height);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
