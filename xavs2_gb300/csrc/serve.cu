// serve.cu -- the serving form of the hot path: many concurrent video
// streams of different resolutions submit P pictures; a scheduler thread
// batches the pictures that have arrived (continuous batching) and runs each
// batch with one launch per kernel:
//   per picture: upload, reference list update (the previous picture becomes
//   reference 0, xavs2gpu_me_rotate_refs), sub-pel planes of the new
//   reference, current picture;
//   then for the whole batch: the motion search of every picture's leaf-CU
//   PUs (xavs2gpu_me_batch_run), every inter candidate of every CU through
//   the TU chain as the full-picture chain runs it (cand.cuh: predictions,
//   residuals, one TU and the split TUs, SSDs), each CU's chosen
//   reconstruction, and a per-picture checksum of levels, reconstruction and
//   MVs.
// Each stream's references and sub-pel planes stay resident in its own
// motion-search session.  Streams are admitted against the device's free
// memory and an optional budget, pictures against the pixel capacity of the
// batch buffers; two
// batch buffer sets on two CUDA streams let the next batch be prepared and
// enqueued while the current one runs.  A picture of a stream is only
// batched once the stream's previous picture has completed, so every
// result is independent of what else shares its batch.
#include "cand.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

// batch buffer sets (each with its own CUDA stream): while one batch runs,
// the next ones are formed and enqueued
// backlog (in batch targets) beyond which batches take the full size
#ifndef XG_SERVE_BACKLOG
#define XG_SERVE_BACKLOG 2
#endif
#ifndef XG_SERVE_SETS
#define XG_SERVE_SETS 2
#endif

namespace xg {

int tq_batch_launch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                    int16_t *recon, int32_t *nnz, int warps, cudaStream_t stream);
bool build_candidates(const xavs2gpu_cu_t *cus, int n_cus, const xavs2gpu_pu_t *pus, int n_pus, int W, int H,
                      int nrefs, std::vector<xavs2gpu_cand_t> &cands, std::vector<int32_t> &cu_cand, int64_t &n_res,
                      int64_t &n_coef);

namespace srv {

using JobView = PicView;   // one picture of a batch as the kernels see it

// Checksum of a picture's outputs: sum over the 32-bit words w_i of
// [reconstruction (width*height bytes) | levels (int16 pairs) | search
// results (5 words each)] of (w_i + 1) * (2 i + 1), modulo 2^64.
__device__ __forceinline__ unsigned long long mixw(uint32_t w, uint64_t i)
{
    return (unsigned long long)((uint64_t)w + 1) * (unsigned long long)(2 * i + 1);
}

// The checksum of a picture: sum over its words i (reconstruction, then
// levels, then search results) of (w_i + 1)(2i + 1) mod 2^64.  The grid is
// sized for the largest picture of the batch; each region is walked by its
// own grid-stride loop.
__global__ void hash_kernel(const JobView *__restrict__ views, const int16_t *__restrict__ coef)
{
    const JobView &v = views[blockIdx.y];
    const uint64_t nrec = (uint64_t)v.width * v.height / 4;
    const uint64_t ncw = (uint64_t)v.n_coef / 2;
    const uint64_t nres = (uint64_t)v.n_pus * 5;
    const uint32_t *rec = reinterpret_cast<const uint32_t *>(v.recon);
    const uint32_t *cw = reinterpret_cast<const uint32_t *>(coef + v.coef_off);
    const uint32_t *rw = reinterpret_cast<const uint32_t *>(v.res);
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, step = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long h = 0;
    for (uint64_t i = t0; i < nrec; i += step) h += mixw(rec[i], i);
    for (uint64_t i = t0; i < ncw; i += step) h += mixw(cw[i], nrec + i);
    for (uint64_t i = t0; i < nres; i += step) h += mixw(rw[i], nrec + ncw + i);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    // one atomic per CTA (thousands of CTAs add into one word per picture)
    __shared__ unsigned long long part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = h;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) h += part[w];
        atomicAdd(v.hash, h);
    }
}

using Clock = std::chrono::steady_clock;
static int64_t now_ns() { return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now().time_since_epoch()).count(); }

struct Stream {
    int id = 0, W = 0, H = 0, nrefs = 2;
    xavs2gpu_me_session_t *sess = nullptr;
    xavs2gpu_cu_t *d_cus = nullptr;
    xavs2gpu_cand_t *d_cands = nullptr;
    int32_t *d_cu_cand = nullptr;
    int32_t *d_units = nullptr;                   // candidate units, then CU units
    int n_cus = 0, n_pus = 0, n_cands = 0, n_cand_units = 0, n_cu_units = 0;
    int64_t n_res = 0, n_coef = 0;
    uint8_t *d_in = nullptr, *d_prev = nullptr;   // upload buffer, previous picture (next reference)
    uint8_t *h_ring = nullptr;                    // pinned picture slots
    int ring = 0, ring_head = 0, ring_used = 0;
    int frames = 0;                               // pictures submitted
    int loaded = 0;                               // pictures that reached the device
    bool in_flight = false;
    int64_t bytes = 0;
};

struct Job {
    int stream = 0, frame = 0, slot = 0;
    int64_t tag = 0, t_submit = 0;
};

struct BatchSet {
    cudaStream_t st = nullptr;
    cudaEvent_t start = nullptr, done = nullptr;
    int16_t *d_res = nullptr, *d_rres = nullptr, *d_coef = nullptr;
    uint8_t *d_recon = nullptr;
    int32_t *d_nnz = nullptr, *d_cost = nullptr, *d_dist = nullptr;
    xavs2gpu_tq_block_t *d_blocks = nullptr;
    xavs2gpu_cu_choice_t *d_choice = nullptr;
    JobView *d_views = nullptr;
    unsigned long long *d_hash = nullptr, *h_hash = nullptr;
    JobView *h_views = nullptr;
    xavs2gpu_me_batch_t *me = nullptr;
    std::vector<Job> jobs;
    std::vector<int> searched;     // indices into jobs of the searched pictures
    bool busy = false;
};

}  // namespace srv
}  // namespace xg

using namespace xg;
using namespace xg::srv;

struct xavs2gpu_server {
    xavs2gpu_server_config_t cfg{};
    int device = 0;
    int64_t hbm_used = 0;
    int64_t hbm_pending = 0;                  // admitted streams whose memory is not allocated yet
    int64_t max_cus = 0, max_cands = 0;
    std::vector<Stream *> streams;
    BatchSet sets[XG_SERVE_SETS];
    int next_set = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job> pending;
    std::deque<int> inflight;                 // set indices in launch order
    std::deque<xavs2gpu_server_result_t> done;
    std::condition_variable cv_done;
    bool stop = false;
    std::thread sched, comp;
    int64_t batches = 0, frames_batched = 0;
    double gpu_ms = 0.0, host_ms = 0.0;       // batch start->done on the device; scheduler enqueue time
};

namespace {

int64_t frame_cap_cus(int64_t pixels) { return pixels / 64 + 64; }

void enqueue_batch(xavs2gpu_server_t *s, BatchSet &b)
{
    // per picture: upload, reference update, planes (all on the set's stream)
    std::vector<xavs2gpu_me_session_t *> sess;
    b.searched.clear();
    XG_CUDA(cudaEventRecord(b.start, b.st));
    int64_t res_off = 0, coef_off = 0, cu_start = 0, cand_start = 0, rec_off = 0, cand_unit_start = 0,
            cu_unit_start = 0;
    int nv = 0;
    for (size_t k = 0; k < b.jobs.size(); k++) {
        Job &j = b.jobs[k];
        Stream &S = *s->streams[j.stream];
        const size_t pic = (size_t)S.W * S.H;
        XG_CUDA(cudaMemcpyAsync(S.d_in, S.h_ring + (size_t)j.slot * pic, pic, cudaMemcpyHostToDevice, b.st));
        xavs2gpu_me_set_stream(S.sess, b.st);
        if (S.loaded >= 1) {
            xavs2gpu_me_rotate_refs(S.sess);
            xavs2gpu_me_set_picture_device(S.sess, 0, S.d_prev, S.W);
        }
        if (S.loaded >= S.nrefs) {
            xavs2gpu_me_set_picture_device(S.sess, -1, S.d_in, S.W);
            sess.push_back(S.sess);
            b.searched.push_back((int)k);
            JobView &v = b.h_views[nv++];
            v.cur = xavs2gpu_me_plane_device(S.sess, -1, 0);
            v.planes = xavs2gpu_me_plane_table_device(S.sess);
            v.res = xavs2gpu_me_results_device(S.sess);
            v.cus = S.d_cus;
            v.cands = S.d_cands;
            v.cu_cand = S.d_cu_cand;
            v.cand_units = S.d_units;
            v.cu_units = S.d_units + S.n_cand_units;
            v.cand_unit_start = cand_unit_start;
            v.cu_unit_start = cu_unit_start;
            v.recon = b.d_recon + rec_off;
            v.hash = b.d_hash + (nv - 1);
            v.res_off = res_off;
            v.coef_off = coef_off;
            v.cu_start = cu_start;
            v.cand_start = cand_start;
            v.n_cus = S.n_cus;
            v.n_cands = S.n_cands;
            v.n_coef = S.n_coef;
            v.stride = xavs2gpu_me_plane_stride(S.sess);
            v.width = S.W;
            v.height = S.H;
            v.nrefs = S.nrefs;
            v.n_pus = S.n_pus;
            res_off += S.n_res;
            coef_off += S.n_coef;
            cu_start += S.n_cus;
            cand_start += S.n_cands;
            cand_unit_start += S.n_cand_units;
            cu_unit_start += S.n_cu_units;
            rec_off += (int64_t)pic;
        }
        std::swap(S.d_in, S.d_prev);
        S.loaded++;
    }
    if (nv) {
        xavs2gpu_me_batch_run(b.me, sess.data(), (int)sess.size(), &s->cfg.me, b.st);
        XG_CUDA(cudaMemcpyAsync(b.d_views, b.h_views, sizeof(JobView) * nv, cudaMemcpyHostToDevice, b.st));
        XG_CUDA(cudaMemsetAsync(b.d_hash, 0, sizeof(unsigned long long) * nv, b.st));
        const int64_t nc = cand_start, ncu = cu_unit_start, ncand_u = cand_unit_start;
        const unsigned cblocks = (unsigned)((ncand_u * 32 + 127) / 128);
        cand_residual_kernel<<<cblocks, 128, 0, b.st>>>(b.d_views, nv, ncand_u, s->cfg.qp, b.d_res, b.d_blocks, b.d_cost,
                                                        b.d_dist);
        tq_batch_launch(b.d_blocks, (int)(5 * nc), b.d_res, b.d_coef, b.d_rres, b.d_nnz, 4, b.st);
        cand_eval_kernel<<<cblocks, 128, 0, b.st>>>(b.d_views, nv, ncand_u, b.d_rres, b.d_dist);
        cand_choose_kernel<<<(unsigned)((ncu * 32 + 127) / 128), 128, 0, b.st>>>(b.d_views, nv, ncu, b.d_cost,
                                                                                 b.d_dist, b.d_rres, b.d_choice);
        int64_t max_words = 0;
        for (int k = 0; k < nv; k++) {
            const JobView &v = b.h_views[k];
            max_words = std::max<int64_t>(max_words, (int64_t)v.width * v.height / 4 + v.n_coef / 2 + 5LL * v.n_pus);
        }
        // about 8 words of the largest picture per thread
        const unsigned hx = (unsigned)std::min<int64_t>(std::max<int64_t>((max_words + 2047) / 2048, 1), 4096);
        hash_kernel<<<dim3(hx, nv), 256, 0, b.st>>>(b.d_views, b.d_coef);
        count_launch(4);
        XG_CUDA(cudaMemcpyAsync(b.h_hash, b.d_hash, sizeof(unsigned long long) * nv, cudaMemcpyDeviceToHost, b.st));
    }
    XG_CUDA(cudaEventRecord(b.done, b.st));
}

void scheduler(xavs2gpu_server_t *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        BatchSet *free_set = nullptr;
        for (int t = 0; t < XG_SERVE_SETS && !free_set; t++) {
            BatchSet &c = s->sets[(s->next_set + t) % XG_SERVE_SETS];
            if (!c.busy) free_set = &c;
        }
        // take the arrived pictures whose stream is idle, oldest first
        std::vector<Job> take;
        if (free_set) {
            int64_t pix = 0;
            std::vector<char> used(s->streams.size(), 0);
            // the batch size: the target while the backlog (one picture per
            // idle stream) is short, the buffers' full size while more than
            // two target-sized batches wait
            const int64_t tgt = s->cfg.batch_pixels_target;
            int64_t cap = s->cfg.max_batch_pixels;
            if (tgt > 0 && tgt < cap) {
                int64_t backlog = 0;
                for (const Job &j : s->pending) {
                    Stream &S = *s->streams[j.stream];
                    if (S.in_flight || used[j.stream]) continue;
                    used[j.stream] = 1;
                    backlog += (int64_t)S.W * S.H;
                }
                std::fill(used.begin(), used.end(), 0);
                if (backlog <= XG_SERVE_BACKLOG * tgt) cap = tgt;
            }
            for (auto it = s->pending.begin(); it != s->pending.end() && (int)take.size() < s->cfg.max_batch_frames;) {
                Stream &S = *s->streams[it->stream];
                const int64_t p = (int64_t)S.W * S.H;
                // a batch's first picture may take the full size (a picture
                // larger than the target never waits for a backlog)
                if (S.in_flight || used[it->stream] || pix + p > (take.empty() ? s->cfg.max_batch_pixels : cap)) {
                    ++it;
                    continue;
                }
                used[it->stream] = 1;
                pix += p;
                take.push_back(*it);
                it = s->pending.erase(it);
            }
        }
        if (take.empty()) {
            s->cv.wait_for(lk, std::chrono::microseconds(200));
            continue;
        }
        BatchSet &b = *free_set;
        b.busy = true;
        b.jobs = take;
        for (auto &j : take) s->streams[j.stream]->in_flight = true;
        s->next_set = ((int)(&b - s->sets) + 1) % XG_SERVE_SETS;
        lk.unlock();
        const int64_t t0 = now_ns();
        enqueue_batch(s, b);
        const int64_t t1 = now_ns();
        lk.lock();
        s->host_ms += (t1 - t0) / 1e6;
        s->inflight.push_back((int)(&b - s->sets));
        s->batches++;
        s->frames_batched += (int64_t)take.size();
        s->cv.notify_all();
    }
}

void completer(xavs2gpu_server_t *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv.wait(lk, [&] { return s->stop || !s->inflight.empty(); });
        if (s->inflight.empty() && s->stop) break;
        const int si = s->inflight.front();
        BatchSet &b = s->sets[si];
        lk.unlock();
        cudaEventSynchronize(b.done);
        const int64_t t = now_ns();
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b.start, b.done);
        lk.lock();
        s->gpu_ms += ms;
        s->inflight.pop_front();
        std::vector<int> hidx(b.jobs.size(), -1);
        for (size_t q = 0; q < b.searched.size(); q++) hidx[b.searched[q]] = (int)q;
        for (size_t k = 0; k < b.jobs.size(); k++) {
            const Job &j = b.jobs[k];
            Stream &S = *s->streams[j.stream];
            S.in_flight = false;
            S.ring_used--;
            xavs2gpu_server_result_t r{};
            r.stream = j.stream;
            r.frame = j.frame;
            r.tag = j.tag;
            r.t_submit_ns = j.t_submit;
            r.t_done_ns = t;
            r.hash = hidx[k] >= 0 ? b.h_hash[hidx[k]] : 0;
            r.batch_frames = (int32_t)b.jobs.size();
            r.ref_only = hidx[k] < 0;
            s->done.push_back(r);
        }
        b.busy = false;
        s->cv.notify_all();
        s->cv_done.notify_all();
    }
}

void free_set(BatchSet &b)
{
    cudaFree(b.d_res); cudaFree(b.d_rres); cudaFree(b.d_coef); cudaFree(b.d_recon); cudaFree(b.d_nnz);
    cudaFree(b.d_blocks); cudaFree(b.d_choice); cudaFree(b.d_views); cudaFree(b.d_hash);
    cudaFree(b.d_cost); cudaFree(b.d_dist);
    cudaFreeHost(b.h_hash); cudaFreeHost(b.h_views);
    if (b.me) xavs2gpu_me_batch_destroy(b.me);
    if (b.done) cudaEventDestroy(b.done);
    if (b.start) cudaEventDestroy(b.start);
    if (b.st) cudaStreamDestroy(b.st);
}

}  // namespace

extern "C" xavs2gpu_server_t *xavs2gpu_server_create(const xavs2gpu_server_config_t *cfg)
{
    if (!cfg || cfg->max_batch_frames < 1 || cfg->max_batch_frames > 256 || cfg->max_batch_pixels < 64 * 64 ||
        cfg->batch_pixels_target < 0 ||
        cfg->qp < 0 || cfg->qp > 79 || cfg->me.search_range < 1 || cfg->me.search_range > 128) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_server_create", "bad configuration");
        return nullptr;
    }
    auto *s = new xavs2gpu_server();
    s->cfg = *cfg;
    s->device = current_device();
    const int64_t px = cfg->max_batch_pixels;
    s->max_cus = frame_cap_cus(px);
    s->max_cands = 7 * s->max_cus;
    // candidate residual / level regions: 2 S^2 per mode, at most 7 modes per
    // CU, so at most 14 elements per luma pixel of a batch
    const int64_t nres = 14 * px;
    for (auto &b : s->sets) {
        XG_CUDA(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
        XG_CUDA(cudaEventCreate(&b.start));
        XG_CUDA(cudaEventCreate(&b.done));
        XG_CUDA(cudaMalloc((void **)&b.d_res, sizeof(int16_t) * nres));
        XG_CUDA(cudaMalloc((void **)&b.d_rres, sizeof(int16_t) * nres));
        XG_CUDA(cudaMalloc((void **)&b.d_coef, sizeof(int16_t) * nres));
        XG_CUDA(cudaMemset(b.d_coef, 0, sizeof(int16_t) * nres));
        XG_CUDA(cudaMalloc((void **)&b.d_recon, px));
        XG_CUDA(cudaMalloc((void **)&b.d_nnz, sizeof(int32_t) * 5 * s->max_cands));
        XG_CUDA(cudaMalloc((void **)&b.d_blocks, sizeof(xavs2gpu_tq_block_t) * 5 * s->max_cands));
        XG_CUDA(cudaMalloc((void **)&b.d_cost, sizeof(int32_t) * s->max_cands));
        XG_CUDA(cudaMalloc((void **)&b.d_dist, sizeof(int32_t) * 2 * s->max_cands));
        XG_CUDA(cudaMalloc((void **)&b.d_choice, sizeof(xavs2gpu_cu_choice_t) * s->max_cus));
        XG_CUDA(cudaMalloc((void **)&b.d_views, sizeof(JobView) * 256));
        XG_CUDA(cudaMalloc((void **)&b.d_hash, sizeof(unsigned long long) * 256));
        XG_CUDA(cudaMallocHost((void **)&b.h_hash, sizeof(unsigned long long) * 256));
        XG_CUDA(cudaMallocHost((void **)&b.h_views, sizeof(JobView) * 256));
        b.me = xavs2gpu_me_batch_create();
        s->hbm_used += px + 3 * 2 * nres + s->max_cands * (5 * (32 + 4) + 12) + s->max_cus * 8;
    }
    if (cfg->hbm_budget_bytes > 0 && s->hbm_used > cfg->hbm_budget_bytes) {
        for (auto &b : s->sets) free_set(b);
        delete s;
        fail(XAVS2GPU_ERR_CAPACITY, "xavs2gpu_server_create", "batch buffers exceed the device-memory budget");
        return nullptr;
    }
    s->sched = std::thread(scheduler, s);
    s->comp = std::thread(completer, s);
    return s;
}

extern "C" void xavs2gpu_server_destroy(xavs2gpu_server_t *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    s->sched.join();
    s->comp.join();
    cudaSetDevice(s->device);
    for (auto &b : s->sets) cudaStreamSynchronize(b.st);
    // sessions first: they may still point at the batch streams
    for (Stream *S : s->streams) {
        if (!S) continue;
        xavs2gpu_me_set_stream(S->sess, nullptr);
        xavs2gpu_me_destroy(S->sess);
        cudaFree(S->d_cus); cudaFree(S->d_in); cudaFree(S->d_prev); cudaFreeHost(S->h_ring);
        cudaFree(S->d_cands); cudaFree(S->d_cu_cand); cudaFree(S->d_units);
        delete S;
    }
    for (auto &b : s->sets) free_set(b);
    delete s;
}

extern "C" int xavs2gpu_server_open_stream(xavs2gpu_server_t *s, int width, int height, const xavs2gpu_pu_t *pus,
                                           int n_pus, const xavs2gpu_cu_t *cus, int n_cus, int ring)
{
    if (!s || !pus || !cus || n_pus < 1 || n_cus < 1 || ring < 1 || ring > 64) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_server_open_stream", "bad arguments");
        return -XAVS2GPU_ERR_ARG;
    }
    if ((int64_t)width * height > s->cfg.max_batch_pixels || (width & 3)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_server_open_stream", "picture larger than a batch, or width not a multiple of 4");
        return -XAVS2GPU_ERR_ARG;
    }
    // the stream's candidates (validates the CU list against its PUs); the
    // leaf CUs tile the picture, so the batch buffers sized per luma pixel hold them
    std::vector<xavs2gpu_cand_t> cands;
    std::vector<int32_t> cu_cand;
    int64_t n_res = 0, n_coef = 0;
    if (!build_candidates(cus, n_cus, pus, n_pus, width, height, 2, cands, cu_cand, n_res, n_coef) ||
        (int64_t)n_cus > (int64_t)width * height / 64 || n_res > 14 * (int64_t)width * height) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_server_open_stream", "CU list does not tile the picture over its 2Nx2N PUs");
        return -XAVS2GPU_ERR_ARG;
    }
    // resident device memory of the stream: 33 padded planes, PU arrays, CUs,
    // candidates, two pictures
    const int64_t plane = (int64_t)((width + 160 + 63) / 64 * 64) * (height + 160);
    const int64_t need = 33 * plane + (int64_t)n_pus * (18 + 20 + 8 + 12 + 16) + (int64_t)n_cus * 44 +
                         (int64_t)cands.size() * 24 + 2 * (int64_t)width * height + (int64_t)n_cus * 849 * 4 / 16 +
                         (int64_t)cands.size() * 16 + (int64_t)n_cus * 16;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->cfg.hbm_budget_bytes > 0 && s->hbm_used + need > s->cfg.hbm_budget_bytes) {
        fail(XAVS2GPU_ERR_CAPACITY, "xavs2gpu_server_open_stream", "device-memory budget exhausted");
        return -XAVS2GPU_ERR_CAPACITY;
    }
    // admission by the device's free memory now, less the reserve and what
    // streams admitted before us still have to allocate
    {
        size_t free_b = 0, total_b = 0;
        XG_CUDA(cudaSetDevice(s->device));
        XG_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const int64_t reserve = s->cfg.hbm_reserve_bytes > 0 ? s->cfg.hbm_reserve_bytes
                                                            : std::max<int64_t>((int64_t)total_b / 32, (int64_t)1 << 30);
        if (need + s->hbm_pending > (int64_t)free_b - reserve) {
            fail(XAVS2GPU_ERR_CAPACITY, "xavs2gpu_server_open_stream", "not enough free device memory");
            return -XAVS2GPU_ERR_CAPACITY;
        }
    }
    s->hbm_used += need;
    s->hbm_pending += need;
    lk.unlock();
    auto *S = new Stream();
    S->W = width;
    S->H = height;
    S->n_cus = n_cus;
    S->n_pus = n_pus;
    S->sess = xavs2gpu_me_create(width, height, 2, n_pus);
    if (!S->sess || xavs2gpu_me_set_pus(S->sess, pus, n_pus) != XAVS2GPU_OK ||
        xavs2gpu_me_prepare(S->sess, &s->cfg.me) != XAVS2GPU_OK) {
        if (S->sess) xavs2gpu_me_destroy(S->sess);
        delete S;
        lk.lock();
        s->hbm_used -= need;
        s->hbm_pending -= need;
        return -XAVS2GPU_ERR_ARG;
    }
    S->n_res = n_res;
    S->n_coef = n_coef;
    S->n_cands = (int)cands.size();
    S->bytes = need;
    S->ring = ring;
    XG_CUDA(cudaMalloc((void **)&S->d_cus, sizeof(xavs2gpu_cu_t) * n_cus));
    XG_CUDA(cudaMemcpy(S->d_cus, cus, sizeof(xavs2gpu_cu_t) * n_cus, cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&S->d_cands, sizeof(xavs2gpu_cand_t) * cands.size()));
    XG_CUDA(cudaMemcpy(S->d_cands, cands.data(), sizeof(xavs2gpu_cand_t) * cands.size(), cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&S->d_cu_cand, sizeof(int32_t) * cu_cand.size()));
    XG_CUDA(cudaMemcpy(S->d_cu_cand, cu_cand.data(), sizeof(int32_t) * cu_cand.size(), cudaMemcpyHostToDevice));
    std::vector<int32_t> units;
    build_units(cus, n_cus, cands.data(), (int)cands.size(), units, S->n_cand_units, S->n_cu_units);
    XG_CUDA(cudaMalloc((void **)&S->d_units, sizeof(int32_t) * units.size()));
    XG_CUDA(cudaMemcpy(S->d_units, units.data(), sizeof(int32_t) * units.size(), cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&S->d_in, (size_t)width * height));
    XG_CUDA(cudaMalloc((void **)&S->d_prev, (size_t)width * height));
    XG_CUDA(cudaMallocHost((void **)&S->h_ring, (size_t)width * height * ring));
    lk.lock();
    s->hbm_pending -= need;
    S->id = (int)s->streams.size();
    s->streams.push_back(S);
    return S->id;
}

extern "C" int xavs2gpu_server_submit(xavs2gpu_server_t *s, int stream, const uint8_t *luma, intptr_t stride,
                                     int64_t tag)
{
    if (!s || !luma) return XAVS2GPU_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (stream < 0 || stream >= (int)s->streams.size()) return XAVS2GPU_ERR_ARG;
    Stream &S = *s->streams[stream];
    if (stride < S.W) return XAVS2GPU_ERR_ARG;
    if (S.ring_used >= S.ring) return XAVS2GPU_ERR_CAPACITY;   // the stream's picture slots are full
    Job j;
    j.stream = stream;
    j.frame = S.frames++;
    j.slot = S.ring_head;
    j.tag = tag;
    S.ring_head = (S.ring_head + 1) % S.ring;
    S.ring_used++;
    uint8_t *dst = S.h_ring + (size_t)j.slot * S.W * S.H;
    lk.unlock();
    for (int y = 0; y < S.H; y++) memcpy(dst + (size_t)y * S.W, luma + (size_t)y * stride, S.W);
    j.t_submit = now_ns();
    lk.lock();
    s->pending.push_back(j);
    s->cv.notify_all();
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_server_poll(xavs2gpu_server_t *s, xavs2gpu_server_result_t *out, int max, int timeout_ms)
{
    if (!s || !out || max < 1) return -XAVS2GPU_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && timeout_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !s->done.empty(); });
    int k = 0;
    while (k < max && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    return k;
}

extern "C" void xavs2gpu_server_stats(xavs2gpu_server_t *s, int64_t *hbm_used, int64_t *batches, int64_t *frames,
                                      int64_t *pending)
{
    if (!s) return;
    std::lock_guard<std::mutex> lk(s->mu);
    if (hbm_used) *hbm_used = s->hbm_used;
    if (batches) *batches = s->batches;
    if (frames) *frames = s->frames_batched;
    if (pending) *pending = (int64_t)s->pending.size();
}

extern "C" void xavs2gpu_server_timing(xavs2gpu_server_t *s, double *gpu_ms, double *host_ms)
{
    if (!s) return;
    std::lock_guard<std::mutex> lk(s->mu);
    if (gpu_ms) *gpu_ms = s->gpu_ms;
    if (host_ms) *host_ms = s->host_ms;
}
