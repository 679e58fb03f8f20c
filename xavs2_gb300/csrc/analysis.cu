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

// A thread owns a 4x4 quad of the tile: 16 samples in registers, 2x2 output
// samples, and its share of the block sums and MADs (shared-memory atomics).
template <bool AL>
__global__ void __launch_bounds__(256) lookahead_kernel(const uint8_t *__restrict__ src, int stride, int width,
                                                        int height, uint8_t *__restrict__ lowres, int lowres_stride,
                                                        int32_t *__restrict__ mad16, int32_t *__restrict__ mad32,
                                                        int32_t *__restrict__ mad64)
{
    __shared__ int s16[16], s32[4], s64;
    __shared__ int m16[16], m32[4], m64;
    const int t = threadIdx.x, qx = t & 15, qy = t >> 4;
    const int tx = blockIdx.x, ty = blockIdx.y;
    const int x0 = tx * 64 + 4 * qx, y0 = ty * 64 + 4 * qy;
    if (t < 16) {
        s16[t] = 0;
        m16[t] = 0;
    }
    if (t < 4) {
        s32[t] = 0;
        m32[t] = 0;
    }
    if (t == 0) {
        s64 = 0;
        m64 = 0;
    }
    int v[4][4];
    int sum = 0;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int y = y0 + r;
        if (AL && y < height && x0 + 3 < width) {
            // the quad's row as one word (source and stride 4-byte aligned)
            const uint32_t w = *reinterpret_cast<const uint32_t *>(src + (long long)y * stride + x0);
#pragma unroll
            for (int c = 0; c < 4; c++) v[r][c] = (int)((w >> (8 * c)) & 0xFFu);
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int x = x0 + c;
                v[r][c] = (x < width && y < height) ? src[(long long)y * stride + x] : 0;
            }
        }
#pragma unroll
        for (int c = 0; c < 4; c++) sum += v[r][c];
    }
    // the tile's 32x32 low-resolution samples
    const int lw = width >> 1, lh = height >> 1;
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int ox = (x0 >> 1) + i, oy = (y0 >> 1) + j;
            if (ox < lw && oy < lh)
                lowres[(long long)oy * lowres_stride + ox] =
                    (uint8_t)avg2(avg2(v[2 * j][2 * i], v[2 * j + 1][2 * i]), avg2(v[2 * j][2 * i + 1], v[2 * j + 1][2 * i + 1]));
        }
    __syncthreads();
    const int b16 = (qy >> 2) * 4 + (qx >> 2), b32 = (qy >> 3) * 2 + (qx >> 3);
    atomicAdd(&s16[b16], sum);
    __syncthreads();
    if (t < 4) atomicAdd(&s32[t], s16[(t >> 1) * 8 + (t & 1) * 2] + s16[(t >> 1) * 8 + (t & 1) * 2 + 1] +
                                      s16[(t >> 1) * 8 + (t & 1) * 2 + 4] + s16[(t >> 1) * 8 + (t & 1) * 2 + 5]);
    __syncthreads();
    if (t == 0) s64 = s32[0] + s32[1] + s32[2] + s32[3];
    __syncthreads();
    // block averages (sum + n/2) / n, n a power of two
    const int a16 = (s16[b16] + 128) >> 8, a32 = (s32[b32] + 512) >> 10, a64 = (s64 + 2048) >> 12;
    int d16 = 0, d32 = 0, d64 = 0;
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) {
            d16 += abs(v[r][c] - a16);
            d32 += abs(v[r][c] - a32);
            d64 += abs(v[r][c] - a64);
        }
    atomicAdd(&m16[b16], d16);
    atomicAdd(&m32[b32], d32);
    atomicAdd(&m64, d64);
    __syncthreads();
    // outputs: blocks fully inside the picture, else -1
    const int n16x = (width + 15) >> 4, n32x = (width + 31) >> 5, n64x = (width + 63) >> 6;
    const int n16y = (height + 15) >> 4, n32y = (height + 31) >> 5;
    if (t < 16) {
        const int bx = tx * 4 + (t & 3), by = ty * 4 + (t >> 2);
        if (bx < n16x && by < n16y)
            mad16[by * n16x + bx] = ((bx + 1) * 16 <= width && (by + 1) * 16 <= height) ? m16[t] : -1;
    } else if (t < 20) {
        const int k = t - 16, bx = tx * 2 + (k & 1), by = ty * 2 + (k >> 1);
        if (bx < n32x && by < n32y)
            mad32[by * n32x + bx] = ((bx + 1) * 32 <= width && (by + 1) * 32 <= height) ? m32[k] : -1;
    } else if (t == 20) {
        mad64[ty * n64x + tx] = ((tx + 1) * 64 <= width && (ty + 1) * 64 <= height) ? m64 : -1;
    }
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
    if ((((uintptr_t)src) & 3) == 0 && (stride & 3) == 0)
        la::lookahead_kernel<true><<<grid, 256, 0, (cudaStream_t)stream>>>(src, stride, width, height, lowres,
                                                                           lowres_stride, mad16, mad32, mad64);
    else
        la::lookahead_kernel<false><<<grid, 256, 0, (cudaStream_t)stream>>>(src, stride, width, height, lowres,
                                                                            lowres_stride, mad16, mad32, mad64);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
