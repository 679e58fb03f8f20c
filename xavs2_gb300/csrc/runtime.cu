// runtime.cu -- error channel, device selection and the per-thread call
// contexts (stream + pinned/device staging) behind the drop-in entry points.
#include "xavs2gpu_common.cuh"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace xg {

static std::atomic<int> g_status{XAVS2GPU_OK};
static std::atomic<int> g_abort{1};
static std::atomic<uint64_t> g_launches{0};
static std::atomic<int> g_percall_mode{1};
static std::mutex g_msg_mu;
static char g_msg[512] = "";
static thread_local int t_device = 0;

void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

int percall_mode() { return g_percall_mode.load(std::memory_order_relaxed); }

void fail(int status, const char *where, const char *msg)
{
    {
        std::lock_guard<std::mutex> lk(g_msg_mu);
        snprintf(g_msg, sizeof(g_msg), "xavs2gpu: %s: %s", where, msg);
    }
    g_status.store(status);
    if (g_abort.load()) {
        fprintf(stderr, "%s\n", g_msg);
        fflush(stderr);
        abort();
    }
}

void check_cuda(cudaError_t e, const char *where)
{
    if (e != cudaSuccess) fail(XAVS2GPU_ERR_CUDA, where, cudaGetErrorString(e));
}

int current_device() { return t_device; }

int sm_count()
{
    static int sms[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!sms[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
        sms[dev] = n;
    }
    return sms[dev];
}

// One context per (thread, device).  Buffers grow on demand and live until
// thread exit.
struct CtxHolder {
    CallCtx ctx[8];
    ~CtxHolder()
    {
        for (auto &c : ctx) {
            if (c.device < 0) continue;
            cudaSetDevice(c.device);
            if (c.h_stage) cudaFreeHost(c.h_stage);
            if (c.d_stage) cudaFree(c.d_stage);
            if (c.stream) cudaStreamDestroy(c.stream);
        }
    }
};
static thread_local CtxHolder t_ctx;

CallCtx &call_ctx(size_t need)
{
    int dev = t_device;
    if (dev < 0 || dev >= 8) { fail(XAVS2GPU_ERR_ARG, "call_ctx", "device index out of range"); }
    CallCtx &c = t_ctx.ctx[dev];
    XG_CUDA(cudaSetDevice(dev));
    if (c.device < 0) {
        c.device = dev;
        XG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    }
    if (need > c.cap) {
        size_t cap = align_up(need > (1u << 20) ? need : (1u << 20), 1u << 16);
        if (c.h_stage) XG_CUDA(cudaFreeHost(c.h_stage));
        if (c.d_stage) XG_CUDA(cudaFree(c.d_stage));
        XG_CUDA(cudaMallocHost((void **)&c.h_stage, cap));
        XG_CUDA(cudaMalloc((void **)&c.d_stage, cap));
        c.cap = cap;
    }
    return c;
}

void pack_rows(uint8_t *dst, const void *src, intptr_t src_stride_bytes, int row_bytes, int rows)
{
    const uint8_t *s = (const uint8_t *)src;
    for (int y = 0; y < rows; y++) memcpy(dst + (size_t)y * row_bytes, s + y * src_stride_bytes, (size_t)row_bytes);
}

void unpack_rows(void *dst, intptr_t dst_stride_bytes, const uint8_t *src, int row_bytes, int rows)
{
    uint8_t *d = (uint8_t *)dst;
    for (int y = 0; y < rows; y++) memcpy(d + y * dst_stride_bytes, src + (size_t)y * row_bytes, (size_t)row_bytes);
}

}  // namespace xg

extern "C" {

int xavs2gpu_init(int device)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        xg::fail(XAVS2GPU_ERR_NO_DEVICE, "xavs2gpu_init", e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
        return XAVS2GPU_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n || device >= 8) {
        xg::fail(XAVS2GPU_ERR_ARG, "xavs2gpu_init", "device index out of range");
        return XAVS2GPU_ERR_ARG;
    }
    xg::t_device = device;
    xg::call_ctx(0);
    return XAVS2GPU_OK;
}

int xavs2gpu_get_status(void) { return xg::g_status.load(); }

const char *xavs2gpu_get_error(void) { return xg::g_msg; }

void xavs2gpu_clear_error(void)
{
    std::lock_guard<std::mutex> lk(xg::g_msg_mu);
    xg::g_msg[0] = 0;
    xg::g_status.store(XAVS2GPU_OK);
}

void xavs2gpu_set_abort_on_error(int enable) { xg::g_abort.store(enable ? 1 : 0); }

void xavs2gpu_set_percall_mode(int in_place) { xg::g_percall_mode.store(in_place ? 1 : 0); }

uint64_t xavs2gpu_kernel_launches(void) { return xg::g_launches.load(); }

const char *xavs2gpu_version(void) { return "xavs2-gb300 0.1 (sm_103a)"; }

int xavs2gpu_copy_d2h(void *dst, const void *src, size_t bytes)
{
    XG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return xavs2gpu_get_status();
}

int xavs2gpu_copy_h2d(void *dst, const void *src, size_t bytes)
{
    XG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return xavs2gpu_get_status();
}

}  // extern "C"
