// pixel.cu -- block costs (SAD, SATD, SA8D, SSD, SAD x3/x4) and block
// operations (avg, sub_ps, add_ps, copies, MAD) for sm_103a, plus the
// per-shape drop-in entry points of the reference's pixel_funcs_t
// (source/common/pixel.h:141-166, C versions in pixel.c:93-856).
#include "xavs2gpu_common.cuh"

#include <cstring>

namespace xg {

// Device-side description of one block-cost evaluation.
struct CostJob {
    const uint8_t *p1;
    const uint8_t *p2;
    int32_t s1, s2;
    int32_t part, pad_;
};

// Cost contribution of lane `lane` of a warp to the job's cost.  SAD and SSD
// stride over pixels; SATD/SA8D stride over their rounding units (4x4, 8x4,
// 8x8 or 16x16), each rounded exactly as the reference's unit functions.
template <int KIND>
__device__ __forceinline__ int job_cost_lane(const CostJob &j, int lane)
{
    const int w = c_pu_w[j.part], h = c_pu_h[j.part];
    int s = 0;
    if (KIND == 0 || KIND == 3) {
        for (int i = lane; i < w * h; i += 32) {
            int y = i / w, x = i - y * w;
            int d = (int)j.p1[y * j.s1 + x] - (int)j.p2[y * j.s2 + x];
            s += KIND == 0 ? iabs_d(d) : d * d;
        }
        return s;
    }
    int kind = KIND == 1 ? 0 : sa8d_kind(w, h);
    if (kind == 0) {
        const bool u4 = satd_unit4(w, h);
        const int uw = u4 ? 4 : 8, nux = w / uw, nu = nux * (h >> 2);
        for (int u = lane; u < nu; u += 32) {
            int uy = u / nux, ux = u - uy * nux;
            s += satd_unit_d(u4, j.p1 + uy * 4 * j.s1 + ux * uw, j.s1, j.p2 + uy * 4 * j.s2 + ux * uw, j.s2);
        }
    } else if (kind == 1) {
        const int nux = w >> 3, nu = nux * (h >> 3);
        for (int u = lane; u < nu; u += 32) {
            int uy = u / nux, ux = u - uy * nux;
            s += (hsum8_d(j.p1 + uy * 8 * j.s1 + ux * 8, j.s1, j.p2 + uy * 8 * j.s2 + ux * 8, j.s2) + 2) >> 2;
        }
    } else {
        // 16x16 units: the four 8x8 sums are rounded together
        const int nux = w >> 4, nu = nux * (h >> 4);
        for (int u = lane; u < nu; u += 32) {
            int uy = u / nux, ux = u - uy * nux;
            const uint8_t *a = j.p1 + uy * 16 * j.s1 + ux * 16, *b = j.p2 + uy * 16 * j.s2 + ux * 16;
            int t = hsum8_d(a, j.s1, b, j.s2) + hsum8_d(a + 8, j.s1, b + 8, j.s2) +
                    hsum8_d(a + 8 * j.s1, j.s1, b + 8 * j.s2, j.s2) +
                    hsum8_d(a + 8 * j.s1 + 8, j.s1, b + 8 * j.s2 + 8, j.s2);
            s += (t + 2) >> 2;
        }
    }
    return s;
}

__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One warp per job.
template <int KIND>
__global__ void __launch_bounds__(128) cost_kernel(const CostJob *__restrict__ jobs, int n, int32_t *__restrict__ out)
{
    int job = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (job >= n) return;
    CostJob j = jobs[job];
    int s = warp_sum(job_cost_lane<KIND>(j, lane));
    if (lane == 0) out[job] = s;
}

// Same, with jobs addressed as offsets from two base pointers (batched API).
template <int KIND>
__global__ void __launch_bounds__(128) cost_batch_kernel(const xavs2gpu_cost_job_t *__restrict__ jobs, int n,
                                                         const uint8_t *__restrict__ b1, const uint8_t *__restrict__ b2,
                                                         int32_t *__restrict__ out)
{
    int job = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (job >= n) return;
    xavs2gpu_cost_job_t q = jobs[job];
    if ((unsigned)q.part >= (unsigned)kNumParts) {   // invalid shape: flagged, never read
        if (lane == 0) out[job] = -1;
        return;
    }
    CostJob j{b1 + q.off1, b2 + q.off2, q.s1, q.s2, q.part, 0};
    int s = warp_sum(job_cost_lane<KIND>(j, lane));
    if (lane == 0) out[job] = s;
}

void launch_cost(int kind, const CostJob *d_jobs, int n, int32_t *d_out, cudaStream_t st)
{
    int blocks = (n * 32 + 127) / 128;
    switch (kind) {
    case 0: cost_kernel<0><<<blocks, 128, 0, st>>>(d_jobs, n, d_out); break;
    case 1: cost_kernel<1><<<blocks, 128, 0, st>>>(d_jobs, n, d_out); break;
    case 2: cost_kernel<2><<<blocks, 128, 0, st>>>(d_jobs, n, d_out); break;
    default: cost_kernel<3><<<blocks, 128, 0, st>>>(d_jobs, n, d_out); break;
    }
    count_launch();
}

// Element-wise block operations on w x h blocks (strides in elements).
enum BlockOp { OP_AVG, OP_SUB_PS, OP_ADD_PS, OP_COPY_PP, OP_COPY_PS, OP_COPY_SP, OP_COPY_SS };

__global__ void blockop_kernel(int op, int w, int h, void *dst, int ds, const void *a, int sa, const void *b, int sb)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        switch (op) {
        case OP_AVG: {
            int v = ((const uint8_t *)a)[y * sa + x] + ((const uint8_t *)b)[y * sb + x] + 1;
            ((uint8_t *)dst)[y * ds + x] = (uint8_t)(v >> 1);
        } break;
        case OP_SUB_PS:
            ((int16_t *)dst)[y * ds + x] =
                (int16_t)(((const uint8_t *)a)[y * sa + x] - ((const uint8_t *)b)[y * sb + x]);
            break;
        case OP_ADD_PS:
            ((uint8_t *)dst)[y * ds + x] =
                clip_pel_d(((const uint8_t *)a)[y * sa + x] + ((const int16_t *)b)[y * sb + x]);
            break;
        case OP_COPY_PP: ((uint8_t *)dst)[y * ds + x] = ((const uint8_t *)a)[y * sa + x]; break;
        case OP_COPY_PS: ((int16_t *)dst)[y * ds + x] = (int16_t)((const uint8_t *)a)[y * sa + x]; break;
        case OP_COPY_SP: ((uint8_t *)dst)[y * ds + x] = (uint8_t)((const int16_t *)a)[y * sa + x]; break;
        default: ((int16_t *)dst)[y * ds + x] = ((const int16_t *)a)[y * sa + x]; break;
        }
    }
}

// mad_NxN_c (pixel.c:1620-1649): one CTA; rounded mean then sum |p - mean|
__global__ void mad_kernel(const uint8_t *src, int n_side, int32_t *out)
{
    __shared__ int red[32];
    int tid = threadIdx.x, n = n_side * n_side;
    int s = 0;
    for (int i = tid; i < n; i += blockDim.x) s += src[i];
    s = warp_sum(s);
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid < 32) {
        int v = tid < (int)(blockDim.x >> 5) ? red[tid] : 0;
        v = warp_sum(v);
        if (tid == 0) red[0] = v;
    }
    __syncthreads();
    int mean = (red[0] + (n >> 1)) / n;
    __syncthreads();
    int m = 0;
    for (int i = tid; i < n; i += blockDim.x) m += iabs_d(src[i] - mean);
    m = warp_sum(m);
    if ((tid & 31) == 0) red[tid >> 5] = m;
    __syncthreads();
    if (tid < 32) {
        int v = tid < (int)(blockDim.x >> 5) ? red[tid] : 0;
        v = warp_sum(v);
        if (tid == 0) out[0] = v;
    }
}

// ---- per-call staging helpers ---------------------------------------------
// Layout of one call in the staging buffers: [jobs][inputs...][outputs].
//
// In place: when the device reads pageable host memory coherently
// (cudaDevAttrPageableMemoryAccess: a Grace host's page tables over
// NVLink-C2C), the block costs read the caller's blocks where they lie, the
// job descriptors and the results sit in the pinned staging buffer, and a
// call is one launch and one synchronisation, with no copies.
// xavs2gpu_set_percall_mode(0) keeps the staged path.
static bool percall_in_place(int dev)
{
    static int cache[64] = {0};   // 0 unknown, 1 no, 2 yes
    if (!percall_mode() || dev < 0 || dev >= 64) return false;
    if (!cache[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) v = 0;
        cache[dev] = v ? 2 : 1;
    }
    return cache[dev] == 2;
}

}  // namespace xg
extern "C" int xavs2gpu_percall_in_place(void) { return xg::percall_in_place(xg::current_device()) ? 1 : 0; }
namespace xg {

static int32_t percall_cost(int kind, int part, const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)
{
    const int w = h_pu_w[part], h = h_pu_h[part];
    if (percall_in_place(current_device())) {
        CallCtx &c = call_ctx(512);
        CostJob *job = reinterpret_cast<CostJob *>(c.h_stage);
        int32_t *out = reinterpret_cast<int32_t *>(c.h_stage + 256);
        *job = CostJob{p1, p2, (int32_t)s1, (int32_t)s2, part, 0};
        launch_cost(kind, job, 1, out, c.stream);
        XG_CUDA(cudaStreamSynchronize(c.stream));
        return *out;
    }
    const size_t o_job = 0, o_a = 256, o_b = o_a + align_up((size_t)w * h), o_out = o_b + align_up((size_t)w * h);
    CallCtx &c = call_ctx(o_out + 256);
    pack_rows(c.h_stage + o_a, p1, s1, w, h);
    pack_rows(c.h_stage + o_b, p2, s2, w, h);
    CostJob j{c.d_stage + o_a, c.d_stage + o_b, w, w, part, 0};
    memcpy(c.h_stage + o_job, &j, sizeof(j));
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_out, cudaMemcpyHostToDevice, c.stream));
    launch_cost(kind, (const CostJob *)(c.d_stage + o_job), 1, (int32_t *)(c.d_stage + o_out), c.stream);
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_out, c.d_stage + o_out, 4, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    return *(int32_t *)(c.h_stage + o_out);
}

// sad_x3 / sad_x4: the encode block has the fixed stride FENC_STRIDE = 64
// (pixel.c:156, 211); the references share `i_ref`.
static void percall_sad_xn(int part, int nref, const uint8_t *fenc, const uint8_t *const *refs, intptr_t i_ref, int *scores)
{
    const int w = h_pu_w[part], h = h_pu_h[part];
    if (percall_in_place(current_device())) {
        CallCtx &c = call_ctx(512);
        CostJob *jobs = reinterpret_cast<CostJob *>(c.h_stage);
        int32_t *out = reinterpret_cast<int32_t *>(c.h_stage + 256);
        for (int r = 0; r < nref; r++) jobs[r] = CostJob{fenc, refs[r], 64, (int32_t)i_ref, part, 0};
        launch_cost(0, jobs, nref, out, c.stream);
        XG_CUDA(cudaStreamSynchronize(c.stream));
        memcpy(scores, out, 4 * nref);
        return;
    }
    const size_t blk = align_up((size_t)w * h);
    const size_t o_job = 0, o_in = 256, o_out = o_in + blk * (1 + nref);
    CallCtx &c = call_ctx(o_out + 256);
    pack_rows(c.h_stage + o_in, fenc, 64, w, h);
    CostJob jobs[4];
    for (int r = 0; r < nref; r++) {
        pack_rows(c.h_stage + o_in + blk * (1 + r), refs[r], i_ref, w, h);
        jobs[r] = CostJob{c.d_stage + o_in, c.d_stage + o_in + blk * (1 + r), w, w, part, 0};
    }
    memcpy(c.h_stage + o_job, jobs, sizeof(CostJob) * nref);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_out, cudaMemcpyHostToDevice, c.stream));
    launch_cost(0, (const CostJob *)(c.d_stage + o_job), nref, (int32_t *)(c.d_stage + o_out), c.stream);
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_out, c.d_stage + o_out, 4 * nref, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    memcpy(scores, c.h_stage + o_out, 4 * nref);
}

// Element sizes of the operands of each block op: (dst, a, b).
static void op_sizes(int op, int &ed, int &ea, int &eb)
{
    switch (op) {
    case OP_AVG: ed = 1; ea = 1; eb = 1; break;
    case OP_SUB_PS: ed = 2; ea = 1; eb = 1; break;
    case OP_ADD_PS: ed = 1; ea = 1; eb = 2; break;
    case OP_COPY_PP: ed = 1; ea = 1; eb = 0; break;
    case OP_COPY_PS: ed = 2; ea = 1; eb = 0; break;
    case OP_COPY_SP: ed = 1; ea = 2; eb = 0; break;
    default: ed = 2; ea = 2; eb = 0; break;
    }
}

// Strides are in elements of the respective operand, as in the reference.
static void percall_blockop(int op, int w, int h, void *dst, intptr_t ds, const void *a, intptr_t sa,
                            const void *b, intptr_t sb)
{
    int ed, ea, eb;
    op_sizes(op, ed, ea, eb);
    const size_t o_a = 0, o_b = align_up((size_t)w * h * ea), o_d = o_b + align_up((size_t)w * h * (eb ? eb : 1));
    const size_t total = o_d + align_up((size_t)w * h * ed);
    CallCtx &c = call_ctx(total);
    pack_rows(c.h_stage + o_a, a, sa * ea, w * ea, h);
    if (eb) pack_rows(c.h_stage + o_b, b, sb * eb, w * eb, h);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_d, cudaMemcpyHostToDevice, c.stream));
    int threads = 256, blocks = (w * h + threads - 1) / threads;
    blockop_kernel<<<blocks, threads, 0, c.stream>>>(op, w, h, c.d_stage + o_d, w, c.d_stage + o_a, w,
                                                     c.d_stage + o_b, w);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_d, c.d_stage + o_d, (size_t)w * h * ed, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    unpack_rows(dst, ds * ed, c.h_stage + o_d, w * ed, h);
}

__global__ void flat_ssd_kernel(const uint8_t *a, const uint8_t *b, int n, int32_t *out)
{
    __shared__ int red[32];
    int s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int d = (int)a[i] - (int)b[i];
        s += d * d;
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
        v = warp_sum(v);
        if (threadIdx.x == 0) out[0] = v;
    }
}

void launch_flat_ssd(const uint8_t *a, const uint8_t *b, int n, int32_t *out, cudaStream_t st)
{
    flat_ssd_kernel<<<1, 256, 0, st>>>(a, b, n, out);
    count_launch();
}

static int32_t percall_ssd_wh(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2, int w, int h)
{
    if (w <= 0 || h <= 0) return 0;
    // arbitrary sizes (the ALF caller passes any w x h): one CTA reduction
    // over the packed block
    const size_t o_a = 0, o_b = align_up((size_t)w * h), o_out = o_b + align_up((size_t)w * h);
    CallCtx &c = call_ctx(o_out + 256);
    pack_rows(c.h_stage + o_a, p1, s1, w, h);
    pack_rows(c.h_stage + o_b, p2, s2, w, h);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_out, cudaMemcpyHostToDevice, c.stream));
    launch_flat_ssd(c.d_stage + o_a, c.d_stage + o_b, w * h, (int32_t *)(c.d_stage + o_out), c.stream);
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_out, c.d_stage + o_out, 4, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    return *(int32_t *)(c.h_stage + o_out);
}

static int percall_mad(const uint8_t *src, int i_src, int cu_size)
{
    const size_t o_a = 0, o_out = align_up((size_t)cu_size * cu_size);
    CallCtx &c = call_ctx(o_out + 256);
    pack_rows(c.h_stage + o_a, src, i_src, cu_size, cu_size);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_out, cudaMemcpyHostToDevice, c.stream));
    mad_kernel<<<1, 256, 0, c.stream>>>(c.d_stage + o_a, cu_size, (int32_t *)(c.d_stage + o_out));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_out, c.d_stage + o_out, 4, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    return *(int32_t *)(c.h_stage + o_out);
}

}  // namespace xg

// ---- C ABI -----------------------------------------------------------------
using namespace xg;

#define XG_PART(w, h) (XAVS2GPU_LUMA_##w##x##h)

#define XG_DEFINE_PIXEL(w, h)                                                                                          \
    extern "C" int32_t xavs2gpu_pixel_sad_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)    \
    {                                                                                                                  \
        return percall_cost(0, XG_PART(w, h), p1, s1, p2, s2);                                                         \
    }                                                                                                                  \
    extern "C" int32_t xavs2gpu_pixel_satd_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)   \
    {                                                                                                                  \
        return percall_cost(1, XG_PART(w, h), p1, s1, p2, s2);                                                         \
    }                                                                                                                  \
    extern "C" int32_t xavs2gpu_pixel_sa8d_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)   \
    {                                                                                                                  \
        return percall_cost(2, XG_PART(w, h), p1, s1, p2, s2);                                                         \
    }                                                                                                                  \
    extern "C" int32_t xavs2gpu_pixel_ssd_##w##x##h(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2)    \
    {                                                                                                                  \
        return percall_cost(3, XG_PART(w, h), p1, s1, p2, s2);                                                         \
    }                                                                                                                  \
    extern "C" void xavs2gpu_pixel_sad_x3_##w##x##h(const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,         \
                                                    const uint8_t *r2, intptr_t i_ref, int scores[3])                  \
    {                                                                                                                  \
        const uint8_t *refs[3] = {r0, r1, r2};                                                                         \
        percall_sad_xn(XG_PART(w, h), 3, fenc, refs, i_ref, scores);                                                   \
    }                                                                                                                  \
    extern "C" void xavs2gpu_pixel_sad_x4_##w##x##h(const uint8_t *fenc, const uint8_t *r0, const uint8_t *r1,         \
                                                    const uint8_t *r2, const uint8_t *r3, intptr_t i_ref,              \
                                                    int scores[4])                                                     \
    {                                                                                                                  \
        const uint8_t *refs[4] = {r0, r1, r2, r3};                                                                     \
        percall_sad_xn(XG_PART(w, h), 4, fenc, refs, i_ref, scores);                                                   \
    }                                                                                                                  \
    extern "C" void xavs2gpu_pixel_avg_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *a, intptr_t sa,             \
                                                 const uint8_t *b, intptr_t sb, int weight)                           \
    {                                                                                                                  \
        (void)weight; /* unused by the reference too (pixel.c:684) */                                                 \
        percall_blockop(OP_AVG, w, h, dst, ds, a, sa, b, sb);                                                          \
    }                                                                                                                  \
    extern "C" void xavs2gpu_pixel_sub_ps_##w##x##h(int16_t *dst, intptr_t ds, const uint8_t *a, const uint8_t *b,     \
                                                    intptr_t sa, intptr_t sb)                                          \
    {                                                                                                                  \
        percall_blockop(OP_SUB_PS, w, h, dst, ds, a, sa, b, sb);                                                       \
    }                                                                                                                  \
    extern "C" void xavs2gpu_pixel_add_ps_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *a, const int16_t *b,     \
                                                    intptr_t sa, intptr_t sb)                                          \
    {                                                                                                                  \
        percall_blockop(OP_ADD_PS, w, h, dst, ds, a, sa, b, sb);                                                       \
    }                                                                                                                  \
    extern "C" void xavs2gpu_blockcopy_pp_##w##x##h(uint8_t *dst, intptr_t ds, const uint8_t *src, intptr_t ss)        \
    {                                                                                                                  \
        percall_blockop(OP_COPY_PP, w, h, dst, ds, src, ss, nullptr, 0);                                               \
    }                                                                                                                  \
    extern "C" void xavs2gpu_blockcopy_ps_##w##x##h(int16_t *dst, intptr_t ds, const uint8_t *src, intptr_t ss)        \
    {                                                                                                                  \
        percall_blockop(OP_COPY_PS, w, h, dst, ds, src, ss, nullptr, 0);                                               \
    }                                                                                                                  \
    extern "C" void xavs2gpu_blockcopy_sp_##w##x##h(uint8_t *dst, intptr_t ds, const int16_t *src, intptr_t ss)        \
    {                                                                                                                  \
        percall_blockop(OP_COPY_SP, w, h, dst, ds, src, ss, nullptr, 0);                                               \
    }                                                                                                                  \
    extern "C" void xavs2gpu_blockcopy_ss_##w##x##h(int16_t *dst, intptr_t ds, const int16_t *src, intptr_t ss)        \
    {                                                                                                                  \
        percall_blockop(OP_COPY_SS, w, h, dst, ds, src, ss, nullptr, 0);                                               \
    }

XAVS2GPU_FOR_EACH_PU(XG_DEFINE_PIXEL)

extern "C" int32_t xavs2gpu_get_block_ssd(const uint8_t *p1, intptr_t s1, const uint8_t *p2, intptr_t s2, int w, int h)
{
    return percall_ssd_wh(p1, s1, p2, s2, w, h);
}

extern "C" void xavs2gpu_pixel_average(uint8_t *dst, int i_dst, uint8_t *a, int i_a, uint8_t *b, int i_b, int w, int h)
{
    if (w <= 0 || h <= 0) return;
    percall_blockop(OP_AVG, w, h, dst, i_dst, a, i_a, b, i_b);
}

extern "C" int xavs2gpu_mad_NxN(uint8_t *src, int i_src, int cu_size)
{
    if (cu_size <= 0 || cu_size > 64) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_mad_NxN", "cu_size must be in (0, 64]");
        return 0;
    }
    return percall_mad(src, i_src, cu_size);
}

#define XG_TABLE_ROW(name, fn)                                              \
    do {                                                                    \
        pixf->name[XAVS2GPU_LUMA_4x4] = fn##_4x4;                           \
        pixf->name[XAVS2GPU_LUMA_8x8] = fn##_8x8;                           \
        pixf->name[XAVS2GPU_LUMA_16x16] = fn##_16x16;                       \
        pixf->name[XAVS2GPU_LUMA_32x32] = fn##_32x32;                       \
        pixf->name[XAVS2GPU_LUMA_64x64] = fn##_64x64;                       \
        pixf->name[XAVS2GPU_LUMA_8x4] = fn##_8x4;                           \
        pixf->name[XAVS2GPU_LUMA_4x8] = fn##_4x8;                           \
        pixf->name[XAVS2GPU_LUMA_16x8] = fn##_16x8;                         \
        pixf->name[XAVS2GPU_LUMA_8x16] = fn##_8x16;                         \
        pixf->name[XAVS2GPU_LUMA_32x16] = fn##_32x16;                       \
        pixf->name[XAVS2GPU_LUMA_16x32] = fn##_16x32;                       \
        pixf->name[XAVS2GPU_LUMA_64x32] = fn##_64x32;                       \
        pixf->name[XAVS2GPU_LUMA_32x64] = fn##_32x64;                       \
        pixf->name[XAVS2GPU_LUMA_16x12] = fn##_16x12;                       \
        pixf->name[XAVS2GPU_LUMA_12x16] = fn##_12x16;                       \
        pixf->name[XAVS2GPU_LUMA_16x4] = fn##_16x4;                         \
        pixf->name[XAVS2GPU_LUMA_4x16] = fn##_4x16;                         \
        pixf->name[XAVS2GPU_LUMA_32x24] = fn##_32x24;                       \
        pixf->name[XAVS2GPU_LUMA_24x32] = fn##_24x32;                       \
        pixf->name[XAVS2GPU_LUMA_32x8] = fn##_32x8;                         \
        pixf->name[XAVS2GPU_LUMA_8x32] = fn##_8x32;                         \
        pixf->name[XAVS2GPU_LUMA_64x48] = fn##_64x48;                       \
        pixf->name[XAVS2GPU_LUMA_48x64] = fn##_48x64;                       \
        pixf->name[XAVS2GPU_LUMA_64x16] = fn##_64x16;                       \
        pixf->name[XAVS2GPU_LUMA_16x64] = fn##_16x64;                       \
    } while (0)

extern "C" void xavs2gpu_pixel_init(uint32_t cpuid, xavs2gpu_pixel_funcs_t *pixf)
{
    (void)cpuid;
    XG_TABLE_ROW(sad, xavs2gpu_pixel_sad);
    XG_TABLE_ROW(satd, xavs2gpu_pixel_satd);
    XG_TABLE_ROW(sa8d, xavs2gpu_pixel_sa8d);
    XG_TABLE_ROW(ssd, xavs2gpu_pixel_ssd);
    XG_TABLE_ROW(sad_x3, xavs2gpu_pixel_sad_x3);
    XG_TABLE_ROW(sad_x4, xavs2gpu_pixel_sad_x4);
    XG_TABLE_ROW(sub_ps, xavs2gpu_pixel_sub_ps);
    XG_TABLE_ROW(add_ps, xavs2gpu_pixel_add_ps);
    XG_TABLE_ROW(copy_sp, xavs2gpu_blockcopy_sp);
    XG_TABLE_ROW(copy_ps, xavs2gpu_blockcopy_ps);
    XG_TABLE_ROW(copy_ss, xavs2gpu_blockcopy_ss);
    XG_TABLE_ROW(copy_pp, xavs2gpu_blockcopy_pp);
    XG_TABLE_ROW(avg, xavs2gpu_pixel_avg);
    pixf->ssd_block = xavs2gpu_get_block_ssd;
    pixf->average = xavs2gpu_pixel_average;
}

extern "C" void xavs2gpu_mad_init(uint32_t cpuid, xavs2gpu_mad_funcs_t *madf)
{
    (void)cpuid;
    madf[1] = madf[2] = madf[3] = xavs2gpu_mad_NxN;   // 16x16, 32x32, 64x64 (pixel.c:1654-1658)
}

extern "C" int xavs2gpu_cost_batch(int kind, const xavs2gpu_cost_job_t *jobs, int n, const uint8_t *base1,
                                   const uint8_t *base2, int32_t *out, void *stream)
{
    if (n < 0 || kind < 0 || kind > 3) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_cost_batch", "bad kind or count");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int blocks = (int)(((int64_t)n * 32 + 127) / 128);
    switch (kind) {
    case 0: cost_batch_kernel<0><<<blocks, 128, 0, st>>>(jobs, n, base1, base2, out); break;
    case 1: cost_batch_kernel<1><<<blocks, 128, 0, st>>>(jobs, n, base1, base2, out); break;
    case 2: cost_batch_kernel<2><<<blocks, 128, 0, st>>>(jobs, n, base1, base2, out); break;
    default: cost_batch_kernel<3><<<blocks, 128, 0, st>>>(jobs, n, base1, base2, out); break;
    }
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
