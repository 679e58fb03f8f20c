// analysis.cu -- lookahead picture analysis for sm_103a: the half-resolution
// picture (lowres_filter, mc.c:838-855; table member primitives.h:140) and
// the MAD of every aligned 16x16 / 32x32 / 64x64 block (mad_NxN_c,
// pixel.c:1620-1649), which the encoder's CU-depth prediction compares with
// its thresholds (ctu_intra_depth_pred_mad, rdo.c:3286-3297).  One CTA per
// 64x64 tile reads the tile once and produces the tile's 32x32 low-resolution
// samples and its 16 + 4 + 1 MADs.
#include "xavs2gpu_common.cuh"

namespace xg {
namespace la {

__device__ __forceinline__ int avg2(int a, int b) { return (a + b + 1) >> 1; }

// per-call: one row of output per thread
__global__ void lowres_kernel(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= width || y >= height) return;
    const uint8_t *a = src + (long long)(2 * y) * i_src + 2 * x, *b = a + i_src;
    dst[(long long)y * i_dst + x] = (uint8_t)avg2(avg2(a[0], b[0]), avg2(a[1], b[1]));
}

// bytewise (a + b + 1) >> 1
__device__ __forceinline__ uint32_t avg_bytes(uint32_t a, uint32_t b)
{
    return (a | b) - (((a ^ b) >> 1) & 0x7F7F7F7Fu);
}
__device__ __forceinline__ int sum_bytes(uint32_t w, int acc) { return (int)__dp4a(w, 0x01010101u, (unsigned)acc); }
__device__ __forceinline__ int mad_bytes(uint32_t w, int avg, int acc)
{
    return sum_bytes(__vabsdiffu4(w, (uint32_t)avg * 0x01010101u), acc);
}

// One CTA of 64 threads per 64x64 tile; a thread owns a 16x4 strip (four
// 16-byte rows when AL == 2, four words a row when AL == 1, samples with
// bounds otherwise; 0 outside the picture).  Lanes: qx = t & 3 the strip
// column, qy = t >> 2 the strip row, so the 4 strips of a 16x16 block differ
// in lane bits 2-3 and the 16 strips of a 32x32 block in bits 0 and 2-4: the
// block sums and MADs are warp butterflies, the 64x64 ones add the two warps.
template <int AL>
__global__ void __launch_bounds__(64) lookahead_kernel(const uint8_t *__restrict__ src, int stride, int width,
                                                       int height, uint8_t *__restrict__ lowres, int lowres_stride,
                                                       int32_t *__restrict__ mad16, int32_t *__restrict__ mad32,
                                                       int32_t *__restrict__ mad64)
{
    __shared__ int part[2][2];
    const int t = threadIdx.x, qx = t & 3, qy = t >> 2, warp = t >> 5;
    const int tx = blockIdx.x, ty = blockIdx.y;
    const int x0 = tx * 64 + 16 * qx, y0 = ty * 64 + 4 * qy;
    uint32_t w[4][4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int y = y0 + r;
        const uint8_t *row = src + (long long)y * stride + x0;
        if (AL == 2 && y < height && x0 + 15 < width) {
            const uint4 q = *reinterpret_cast<const uint4 *>(row);
            w[r][0] = q.x; w[r][1] = q.y; w[r][2] = q.z; w[r][3] = q.w;
            continue;
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if (AL >= 1 && y < height && x0 + 4 * c + 3 < width) {
                w[r][c] = *reinterpret_cast<const uint32_t *>(row + 4 * c);
            } else {
                uint32_t v = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int x = x0 + 4 * c + k;
                    if (x < width && y < height) v |= (uint32_t)row[4 * c + k] << (8 * k);
                }
                w[r][c] = v;
            }
        }
    }
    // the strip's 8x2 low-resolution samples
    const int lw = width >> 1, lh = height >> 1, ox = x0 >> 1;
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const int oy = (y0 >> 1) + j;
        uint32_t o[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint32_t a = avg_bytes(w[2 * j][2 * h], w[2 * j + 1][2 * h]);
            const uint32_t b = avg_bytes(w[2 * j][2 * h + 1], w[2 * j + 1][2 * h + 1]);
            o[h] = avg_bytes(__byte_perm(a, b, 0x6420), __byte_perm(a, b, 0x7531));
        }
        if (oy >= lh) continue;
        uint8_t *d = lowres + (long long)oy * lowres_stride + ox;
        if (ox + 7 < lw && ((reinterpret_cast<uintptr_t>(d) & 7) == 0)) {
            *reinterpret_cast<uint2 *>(d) = make_uint2(o[0], o[1]);
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (ox + k < lw) d[k] = (uint8_t)(o[k >> 2] >> (8 * (k & 3)));
        }
    }
    // block sums
    int s = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) s = sum_bytes(w[r][c], s);
    int s16 = s + __shfl_xor_sync(0xFFFFFFFFu, s, 4);
    s16 += __shfl_xor_sync(0xFFFFFFFFu, s16, 8);
    int s32 = s16 + __shfl_xor_sync(0xFFFFFFFFu, s16, 1);
    s32 += __shfl_xor_sync(0xFFFFFFFFu, s32, 16);
    const int sw = s32 + __shfl_xor_sync(0xFFFFFFFFu, s32, 2);
    if ((t & 31) == 0) part[0][warp] = sw;
    __syncthreads();
    const int s64 = part[0][0] + part[0][1];
    // block averages (sum + n/2) / n, n a power of two, and the MADs
    const int a16 = (s16 + 128) >> 8, a32 = (s32 + 512) >> 10, a64 = (s64 + 2048) >> 12;
    int d16 = 0, d32 = 0, d64 = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            d16 = mad_bytes(w[r][c], a16, d16);
            d32 = mad_bytes(w[r][c], a32, d32);
            d64 = mad_bytes(w[r][c], a64, d64);
        }
    d16 += __shfl_xor_sync(0xFFFFFFFFu, d16, 4);
    d16 += __shfl_xor_sync(0xFFFFFFFFu, d16, 8);
    d32 += __shfl_xor_sync(0xFFFFFFFFu, d32, 4);
    d32 += __shfl_xor_sync(0xFFFFFFFFu, d32, 8);
    d32 += __shfl_xor_sync(0xFFFFFFFFu, d32, 1);
    d32 += __shfl_xor_sync(0xFFFFFFFFu, d32, 16);
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) d64 += __shfl_xor_sync(0xFFFFFFFFu, d64, m);
    if ((t & 31) == 0) part[1][warp] = d64;
    // outputs: blocks fully inside the picture, else -1
    const int n16x = (width + 15) >> 4, n32x = (width + 31) >> 5, n64x = (width + 63) >> 6;
    const int n16y = (height + 15) >> 4, n32y = (height + 31) >> 5;
    if ((qy & 3) == 0) {
        const int bx = tx * 4 + qx, by = ty * 4 + (qy >> 2);
        if (bx < n16x && by < n16y)
            mad16[by * n16x + bx] = ((bx + 1) * 16 <= width && (by + 1) * 16 <= height) ? d16 : -1;
    }
    if ((qx & 1) == 0 && (qy & 7) == 0) {
        const int bx = tx * 2 + (qx >> 1), by = ty * 2 + (qy >> 3);
        if (bx < n32x && by < n32y)
            mad32[by * n32x + bx] = ((bx + 1) * 32 <= width && (by + 1) * 32 <= height) ? d32 : -1;
    }
    __syncthreads();
    if (t == 0)
        mad64[ty * n64x + tx] = ((tx + 1) * 64 <= width && (ty + 1) * 64 <= height) ? part[1][0] + part[1][1] : -1;
}

}  // namespace la
}  // namespace xg

using namespace xg;

extern "C" void xavs2gpu_lowres_filter(uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height)
{
    if (width <= 0 || height <= 0) return;
    const int sw = 2 * width, sh = 2 * height;
    const size_t o_dst = align_up((size_t)sw * sh);
    CallCtx &c = call_ctx(o_dst + (size_t)width * height);
    pack_rows(c.h_stage, src, i_src, sw, sh);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, (size_t)sw * sh, cudaMemcpyHostToDevice, c.stream));
    la::lowres_kernel<<<dim3((width + 127) / 128, height), 128, 0, c.stream>>>(c.d_stage, sw, c.d_stage + o_dst,
                                                                              width, width, height);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_dst, c.d_stage + o_dst, (size_t)width * height, cudaMemcpyDeviceToHost,
                            c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    unpack_rows(dst, i_dst, c.h_stage + o_dst, width, height);
}

extern "C" int xavs2gpu_lowres_picture(const uint8_t *src, int i_src, uint8_t *dst, int i_dst, int width, int height,
                                       void *stream)
{
    if (width < 0 || height < 0 || !src || !dst) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_lowres_picture", "bad size or pointer");
        return XAVS2GPU_ERR_ARG;
    }
    if (width == 0 || height == 0) return XAVS2GPU_OK;
    la::lowres_kernel<<<dim3((width + 127) / 128, height), 128, 0, (cudaStream_t)stream>>>(src, i_src, dst, i_dst,
                                                                                          width, height);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_lookahead_picture(const uint8_t *src, int stride, int width, int height, uint8_t *lowres,
                                          int lowres_stride, int32_t *mad16, int32_t *mad32, int32_t *mad64,
                                          void *stream)
{
    if (width < 2 || height < 2 || stride < width || lowres_stride < width / 2 || !src || !lowres || !mad16 ||
        !mad32 || !mad64) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_lookahead_picture", "bad size or pointer");
        return XAVS2GPU_ERR_ARG;
    }
    const dim3 grid((width + 63) / 64, (height + 63) / 64);
    const int al = ((((uintptr_t)src) | (uintptr_t)stride) & 15) == 0 ? 2
                   : ((((uintptr_t)src) | (uintptr_t)stride) & 3) == 0 ? 1 : 0;
    auto launch = [&](auto kernel) {
        kernel<<<grid, 64, 0, (cudaStream_t)stream>>>(src, stride, width, height, lowres, lowres_stride, mad16, mad32,
                                                      mad64);
    };
    if (al == 2)
        launch(la::lookahead_kernel<2>);
    else if (al == 1)
        launch(la::lookahead_kernel<1>);
    else
        launch(la::lookahead_kernel<0>);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
