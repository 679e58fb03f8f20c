// xavs2gpu_common.cuh -- shared definitions of the GB300 (sm_103a) hot-path
// library: PU shape tables, the error channel, per-thread call contexts and
// device helpers used by several kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/xavs2_gb300.h"

namespace xg {

// LumaPU order (pixel.h:50-65 of the reference)
constexpr int kNumParts = 25;
// (one copy per translation unit: the library is built without relocatable
// device code)
static __constant__ uint8_t c_pu_w[kNumParts] = {4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32,
                                                 16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16};
static __constant__ uint8_t c_pu_h[kNumParts] = {4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64,
                                                 12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64};
static const uint8_t h_pu_w[kNumParts] = {4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32,
                                          16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16};
static const uint8_t h_pu_h[kNumParts] = {4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64,
                                          12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64};

// ---- error channel ---------------------------------------------------------
// The reference's primitive signatures have no error return.  Failures are
// recorded here (status + message); unless the caller switched it off with
// xavs2gpu_set_abort_on_error(0), a failure prints the message and aborts, so
// a wrong cost is never returned silently.
void fail(int status, const char *where, const char *msg);
void count_launch(int n = 1);   // kernel launch counter (xavs2gpu_kernel_launches)
void check_cuda(cudaError_t e, const char *where);
#define XG_CUDA(call) ::xg::check_cuda((call), #call)

// ---- per-thread call context ------------------------------------------------
// Every host thread that calls a per-call entry point gets its own stream and
// its own pinned host / device staging buffers, so the entry points are
// re-entrant from the encoder's frame and row threads.
struct CallCtx {
    int device = -1;
    cudaStream_t stream = nullptr;
    uint8_t *h_stage = nullptr;   // pinned host staging
    uint8_t *d_stage = nullptr;   // device staging
    size_t cap = 0;
};
CallCtx &call_ctx(size_t need_bytes);
// 1: per-call block costs read host blocks in place where the device allows
int percall_mode();
int current_device();
// Number of SMs of the current device (queried once per device).
int sm_count();
// A reference picture (W x H, any stride, no border needed) into its 16
// planes: the full-pel plane with `pad` replicated border and the 15
// quarter-pel planes, one kernel (mc.cu).
int reference_planes_from(const uint8_t *src, int src_stride, int width, int height, int pad, uint8_t *const planes[16],
                          int stride, cudaStream_t st);

// Byte offset rounded up to 256 for staging sub-buffers.
static inline size_t align_up(size_t v, size_t a = 256) { return (v + a - 1) / a * a; }

// Packs `rows` rows of `row_bytes` from a strided host buffer into `dst`.
void pack_rows(uint8_t *dst, const void *src, intptr_t src_stride_bytes, int row_bytes, int rows);
void unpack_rows(void *dst, intptr_t dst_stride_bytes, const uint8_t *src, int row_bytes, int rows);

// ---- device helpers ---------------------------------------------------------
__device__ __forceinline__ int iabs_d(int v) { return v < 0 ? -v : v; }
// c + sum over the four bytes of |a - b|
__device__ __forceinline__ uint32_t sad4_acc(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t d;
    asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
__device__ __forceinline__ int clip3_d(int lo, int hi, int v) { return min(max(v, lo), hi); }
__device__ __forceinline__ uint8_t clip_pel_d(int v) { return (uint8_t)min(max(v, 0), 255); }

// 4-point Walsh-Hadamard butterfly (unnormalised)
__device__ __forceinline__ void fwht4_d(int &a, int &b, int &c, int &d)
{
    int s0 = a + b, d0 = a - b, s1 = c + d, d1 = c - d;
    a = s0 + s1; b = d0 + d1; c = s0 - s1; d = d0 - d1;
}

// sum of |H D H^T| over the 4x4 difference block at (p1, p2)
__device__ __forceinline__ int hsum4_d(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    int m[4][4];
#pragma unroll
    for (int y = 0; y < 4; y++) {
        int a = p1[y * s1 + 0] - p2[y * s2 + 0], b = p1[y * s1 + 1] - p2[y * s2 + 1];
        int c = p1[y * s1 + 2] - p2[y * s2 + 2], d = p1[y * s1 + 3] - p2[y * s2 + 3];
        fwht4_d(a, b, c, d);
        m[y][0] = a; m[y][1] = b; m[y][2] = c; m[y][3] = d;
    }
    int s = 0;
#pragma unroll
    for (int x = 0; x < 4; x++) {
        int a = m[0][x], b = m[1][x], c = m[2][x], d = m[3][x];
        fwht4_d(a, b, c, d);
        s += iabs_d(a) + iabs_d(b) + iabs_d(c) + iabs_d(d);
    }
    return s;
}

// sum of |H8 D H8^T| over one 8x8 difference block
__device__ __forceinline__ int hsum8_d(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    int m[8][8];
#pragma unroll
    for (int y = 0; y < 8; y++) {
        int v[8];
#pragma unroll
        for (int x = 0; x < 8; x++) v[x] = p1[y * s1 + x] - p2[y * s2 + x];
        int t[8];
#pragma unroll
        for (int i = 0; i < 4; i++) { t[i] = v[i] + v[i + 4]; t[i + 4] = v[i] - v[i + 4]; }
        fwht4_d(t[0], t[1], t[2], t[3]);
        fwht4_d(t[4], t[5], t[6], t[7]);
#pragma unroll
        for (int x = 0; x < 8; x++) m[y][x] = t[x];
    }
    int s = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
        int t[8];
#pragma unroll
        for (int i = 0; i < 4; i++) { t[i] = m[i][x] + m[i + 4][x]; t[i + 4] = m[i][x] - m[i + 4][x]; }
        fwht4_d(t[0], t[1], t[2], t[3]);
        fwht4_d(t[4], t[5], t[6], t[7]);
#pragma unroll
        for (int i = 0; i < 8; i++) s += iabs_d(t[i]);
    }
    return s;
}

// SATD rounding units (pixel.c:354-407): 4x4 units for widths 4 and for
// 12x16, otherwise 8x4 units whose two halves share one rounding.
__host__ __device__ __forceinline__ bool satd_unit4(int w, int h) { return w == 4 || (w == 12 && h == 16); }

// Cost of one SATD unit whose top-left corner is (x, y) inside the block.
__device__ __forceinline__ int satd_unit_d(bool u4, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    if (u4) return hsum4_d(p1, s1, p2, s2) >> 1;
    return (hsum4_d(p1, s1, p2, s2) + hsum4_d(p1 + 4, s1, p2 + 4, s2)) >> 1;
}

// SA8D unit kind for a shape: 0 = alias of SATD, 1 = 8x8 units, 2 = 16x16 units
__host__ __device__ __forceinline__ int sa8d_kind(int w, int h)
{
    if (w == 4 || h == 4 || w == 12 || h == 12) return 0;
    if (w == 8 || h == 8 || (w == 32 && h == 24) || (w == 24 && h == 32)) return 1;
    return 2;
}

// mvbits (me.c:614-641): 1 for 0, else 2*bitlen(|d|)+1
__host__ __device__ __forceinline__ int mvbits_hd(int d)
{
    unsigned a = (unsigned)(d < 0 ? -d : d);
#ifdef __CUDA_ARCH__
    return a ? 2 * (32 - __clz((int)a)) + 1 : 1;
#else
    int bl = 0;
    while (a) { bl++; a >>= 1; }
    return d ? 2 * bl + 1 : 1;
#endif
}

__host__ __device__ __forceinline__ int mv_cost_hd(int lambda, int mvx, int mvy, int pmx, int pmy)
{
    return (int)(((int64_t)lambda * (mvbits_hd(mvx - pmx) + mvbits_hd(mvy - pmy))) >> 16);
}

}  // namespace xg
