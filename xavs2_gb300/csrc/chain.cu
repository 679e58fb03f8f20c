// chain.cu -- one P picture of the encoder hot path on the device, over the
// leaf CUs of its quadtree: sub-pel planes of every reference and the
// current picture (interpolate_lcu_row, mc.c:593-785), the batched motion
// search (xavs2_me_search, me.c:879-1183), each CU's motion-compensated
// 2Nx2N prediction from its best reference (mc_luma on the frame's sub-pel
// planes, mc.c:559-589) and residual (pixel_sub_ps, pixel.c:780-792), one
// CU-sized TU per CU through dct -> quant -> dequant -> idct (tq.cu), and
// the reconstruction clip(pred + residual) (pixel_add_ps, pixel.c:794-806).
// The sequence is enqueued on the motion-search session's stream, eagerly
// or as one captured CUDA graph; an autotuner picks launch shapes that do
// not change any result.
#include "xavs2gpu_common.cuh"

#include <vector>

namespace xg {

int tq_batch_launch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                    int16_t *recon, int32_t *nnz, int warps, cudaStream_t stream);

using CuChoice = xavs2gpu_cu_choice_t;

__device__ __forceinline__ int square_part(int s) { return s == 8 ? 1 : s == 16 ? 2 : s == 32 ? 3 : 4; }

// Warp per CU: the best reference is the one whose 2Nx2N search returned the
// smallest cost (the lowest index on ties); the prediction is the sub-pel
// plane (my&3)*4 + (mx&3) of that reference at the integer part of the MV.
__global__ void __launch_bounds__(128) mc_residual_kernel(const xavs2gpu_cu_t *__restrict__ cus, int n, int nrefs,
                                                          const xavs2gpu_me_result_t *__restrict__ res,
                                                          const uint8_t *__restrict__ cur,
                                                          const uint8_t *const *__restrict__ planes, int stride, int qp,
                                                          int16_t *__restrict__ residual,
                                                          xavs2gpu_tq_block_t *__restrict__ blocks,
                                                          CuChoice *__restrict__ choice)
{
    const int lane = threadIdx.x & 31;
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (i >= n) return;
    const xavs2gpu_cu_t c = cus[i];
    int best = 0, bcost = 0, mvx = 0, mvy = 0;
    for (int r = 0; r < nrefs; r++) {
        const xavs2gpu_me_result_t q = res[c.pu[r]];
        if (r == 0 || q.bcost < bcost) {
            best = r;
            bcost = q.bcost;
            mvx = q.bmv_x;
            mvy = q.bmv_y;
        }
    }
    const int S = c.size, lg = 31 - __clz(S);
    const uint8_t *pred = planes[best * 16 + ((mvy & 3) << 2) + (mvx & 3)] +
                          (ptrdiff_t)(c.y + (mvy >> 2)) * stride + c.x + (mvx >> 2);
    const uint8_t *src = cur + (ptrdiff_t)c.y * stride + c.x;
    int16_t *dst = residual + c.offset;
    for (int e = lane; e < S * S; e += 32) {
        const int yy = e >> lg, xx = e & (S - 1);
        dst[e] = (int16_t)((int)src[(ptrdiff_t)yy * stride + xx] - (int)pred[(ptrdiff_t)yy * stride + xx]);
    }
    if (lane == 0) {
        xavs2gpu_tq_block_t b;
        b.offset = c.offset;
        b.coef_offset = c.coef_offset;
        b.part = square_part(S);
        b.qp = qp;
        b.flags = 0;
        b.pad_ = 0;
        blocks[i] = b;
        CuChoice ch;
        ch.ref = best;
        ch.mv_x = (int16_t)mvx;
        ch.mv_y = (int16_t)mvy;
        choice[i] = ch;
    }
}

// Warp per CU: recon = clip(pred + reconstructed residual) into a
// width-strided picture.
__global__ void __launch_bounds__(128) reconstruct_kernel(const xavs2gpu_cu_t *__restrict__ cus, int n,
                                                          const CuChoice *__restrict__ choice,
                                                          const uint8_t *const *__restrict__ planes, int stride,
                                                          const int16_t *__restrict__ rres, uint8_t *__restrict__ out,
                                                          int out_stride)
{
    const int lane = threadIdx.x & 31;
    const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (i >= n) return;
    const xavs2gpu_cu_t c = cus[i];
    const CuChoice ch = choice[i];
    const int S = c.size, lg = 31 - __clz(S);
    const uint8_t *pred = planes[ch.ref * 16 + ((ch.mv_y & 3) << 2) + (ch.mv_x & 3)] +
                          (ptrdiff_t)(c.y + (ch.mv_y >> 2)) * stride + c.x + (ch.mv_x >> 2);
    const int16_t *r = rres + c.offset;
    uint8_t *o = out + (ptrdiff_t)c.y * out_stride + c.x;
    for (int e = lane; e < S * S; e += 32) {
        const int yy = e >> lg, xx = e & (S - 1);
        o[(ptrdiff_t)yy * out_stride + xx] = clip_pel_d((int)pred[(ptrdiff_t)yy * stride + xx] + r[e]);
    }
}

}  // namespace xg

using namespace xg;

struct xavs2gpu_chain {
    xavs2gpu_me_session_t *s = nullptr;
    int W = 0, H = 0, nrefs = 0, stride = 0, qp = 0, flags = 0, n_cus = 0, device = 0;
    cudaStream_t st = nullptr;
    xavs2gpu_cu_t *d_cus = nullptr;
    int16_t *d_res = nullptr, *d_rres = nullptr, *d_coef = nullptr;
    int32_t *d_nnz = nullptr;
    CuChoice *d_choice = nullptr;
    xavs2gpu_tq_block_t *d_blocks = nullptr;
    uint8_t *d_src = nullptr, *d_recon = nullptr;
    const uint8_t **d_planes = nullptr;
    int64_t n_res = 0, n_coef = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_kernels = 0;
    int tq_warps = 8;

    uint8_t *src(int idx) { return d_src + (size_t)idx * W * H; }
};

namespace {

int chain_enqueue(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm)
{
    int rc;
    for (int r = 0; r < c->nrefs; r++)
        if ((rc = xavs2gpu_me_set_picture_device(c->s, r, c->src(1 + r), c->W)) != XAVS2GPU_OK) return rc;
    if ((rc = xavs2gpu_me_set_picture_device(c->s, -1, c->src(0), c->W)) != XAVS2GPU_OK) return rc;
    if ((rc = xavs2gpu_me_run(c->s, prm)) != XAVS2GPU_OK) return rc;
    const int blocks = (c->n_cus * 32 + 127) / 128;
    mc_residual_kernel<<<blocks, 128, 0, c->st>>>(c->d_cus, c->n_cus, c->nrefs, xavs2gpu_me_results_device(c->s),
                                                 xavs2gpu_me_plane_device(c->s, -1, 0), c->d_planes, c->stride,
                                                 c->qp, c->d_res, c->d_blocks, c->d_choice);
    count_launch();
    if ((rc = tq_batch_launch(c->d_blocks, c->n_cus, c->d_res, c->d_coef, c->d_rres, c->d_nnz, c->tq_warps, c->st)) !=
        XAVS2GPU_OK)
        return rc;
    reconstruct_kernel<<<blocks, 128, 0, c->st>>>(c->d_cus, c->n_cus, c->d_choice, c->d_planes, c->stride, c->d_rres,
                                                 c->d_recon, c->W);
    count_launch();
    if (c->flags & 1) {
        const size_t pic = (size_t)c->W * c->H;
        for (int r = c->nrefs - 1; r >= 1; r--)
            XG_CUDA(cudaMemcpyAsync(c->src(1 + r), c->src(r), pic, cudaMemcpyDeviceToDevice, c->st));
        XG_CUDA(cudaMemcpyAsync(c->src(1), c->d_recon, pic, cudaMemcpyDeviceToDevice, c->st));
    }
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

void drop_graph(xavs2gpu_chain_t *c)
{
    if (c->exec) cudaGraphExecDestroy(c->exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->exec = nullptr;
    c->graph = nullptr;
    c->graph_kernels = 0;
}

}  // namespace

extern "C" xavs2gpu_chain_t *xavs2gpu_chain_create(xavs2gpu_me_session_t *s, const xavs2gpu_cu_t *cus, int n_cus,
                                                   int qp, int flags)
{
    if (!s || !cus || n_cus < 1 || qp < 0 || qp > 79) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_create", "bad session, CU list or QP");
        return nullptr;
    }
    // the session's geometry and PU list, to validate every CU
    int W = 0, H = 0, nrefs = 0, n = 0;
    xavs2gpu_me_session_info(s, &W, &H, &nrefs, &n);
    if (nrefs > 4) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_create", "at most 4 references");
        return nullptr;
    }
    std::vector<xavs2gpu_pu_t> pus(n);
    if (n) xavs2gpu_me_session_pus(s, pus.data());
    int64_t n_res = 0, n_coef = 0;
    for (int i = 0; i < n_cus; i++) {
        const xavs2gpu_cu_t &c = cus[i];
        const int S = c.size;
        bool ok = (S == 8 || S == 16 || S == 32 || S == 64) && c.x >= 0 && c.y >= 0 && c.x + S <= W &&
                  c.y + S <= H && c.offset >= 0 && c.coef_offset >= 0;
        const int part = S == 8 ? 1 : S == 16 ? 2 : S == 32 ? 3 : 4;
        for (int r = 0; ok && r < nrefs; r++) {
            const int k = c.pu[r];
            ok = k >= 0 && k < n && pus[k].x == c.x && pus[k].y == c.y && pus[k].part == part && pus[k].ref == r;
        }
        if (!ok) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_create",
                 "CU outside the picture, bad size or offsets, or pu[r] is not its 2Nx2N PU for reference r");
            return nullptr;
        }
        const int64_t nc = S == 64 ? 1024 : (int64_t)S * S;
        if (c.offset + (int64_t)S * S > n_res) n_res = c.offset + (int64_t)S * S;
        if (c.coef_offset + nc > n_coef) n_coef = c.coef_offset + nc;
    }
    auto *c = new xavs2gpu_chain();
    c->s = s;
    c->W = W; c->H = H; c->nrefs = nrefs; c->qp = qp; c->flags = flags; c->n_cus = n_cus;
    c->stride = xavs2gpu_me_plane_stride(s);
    c->st = (cudaStream_t)xavs2gpu_me_stream(s);
    c->device = current_device();
    c->n_res = n_res;
    c->n_coef = n_coef;
    XG_CUDA(cudaMalloc((void **)&c->d_cus, sizeof(xavs2gpu_cu_t) * n_cus));
    XG_CUDA(cudaMemcpy(c->d_cus, cus, sizeof(xavs2gpu_cu_t) * n_cus, cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&c->d_res, sizeof(int16_t) * n_res));
    XG_CUDA(cudaMalloc((void **)&c->d_rres, sizeof(int16_t) * n_res));
    XG_CUDA(cudaMalloc((void **)&c->d_coef, sizeof(int16_t) * n_coef));
    XG_CUDA(cudaMalloc((void **)&c->d_nnz, sizeof(int32_t) * n_cus));
    XG_CUDA(cudaMalloc((void **)&c->d_choice, sizeof(CuChoice) * n_cus));
    XG_CUDA(cudaMalloc((void **)&c->d_blocks, sizeof(xavs2gpu_tq_block_t) * n_cus));
    XG_CUDA(cudaMalloc((void **)&c->d_src, (size_t)W * H * (1 + nrefs)));
    XG_CUDA(cudaMemset(c->d_src, 0, (size_t)W * H * (1 + nrefs)));
    XG_CUDA(cudaMalloc((void **)&c->d_recon, (size_t)W * H));
    std::vector<const uint8_t *> planes(16 * nrefs);
    for (int r = 0; r < nrefs; r++)
        for (int k = 0; k < 16; k++) planes[16 * r + k] = xavs2gpu_me_plane_device(s, r, k);
    XG_CUDA(cudaMalloc((void **)&c->d_planes, sizeof(uint8_t *) * planes.size()));
    XG_CUDA(cudaMemcpy(c->d_planes, planes.data(), sizeof(uint8_t *) * planes.size(), cudaMemcpyHostToDevice));
    return c;
}

extern "C" void xavs2gpu_chain_destroy(xavs2gpu_chain_t *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    drop_graph(c);
    cudaFree(c->d_cus); cudaFree(c->d_res); cudaFree(c->d_rres); cudaFree(c->d_coef); cudaFree(c->d_nnz);
    cudaFree(c->d_choice); cudaFree(c->d_blocks); cudaFree(c->d_src); cudaFree(c->d_recon);
    cudaFree((void *)c->d_planes);
    delete c;
}

extern "C" uint8_t *xavs2gpu_chain_source(xavs2gpu_chain_t *c, int idx)
{
    if (!c || idx < 0 || idx > c->nrefs) return nullptr;
    return c->src(idx);
}

extern "C" int xavs2gpu_chain_run(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm)
{
    if (!c || !prm) return XAVS2GPU_ERR_ARG;
    XG_CUDA(cudaSetDevice(c->device));
    return chain_enqueue(c, prm);
}

extern "C" int xavs2gpu_chain_capture(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm)
{
    if (!c || !prm) return XAVS2GPU_ERR_ARG;
    XG_CUDA(cudaSetDevice(c->device));
    drop_graph(c);
    int rc = xavs2gpu_me_prepare(c->s, prm);
    if (rc != XAVS2GPU_OK) return rc;
    XG_CUDA(cudaStreamSynchronize(c->st));
    const uint64_t before = xavs2gpu_kernel_launches();
    XG_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
    rc = chain_enqueue(c, prm);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->st, &g);
    count_launch(-(int)(xavs2gpu_kernel_launches() - before));   // captured, not launched
    if (rc != XAVS2GPU_OK || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        fail(XAVS2GPU_ERR_CUDA, "xavs2gpu_chain_capture", e != cudaSuccess ? cudaGetErrorString(e) : "enqueue failed");
        return XAVS2GPU_ERR_CUDA;
    }
    c->graph = g;
    XG_CUDA(cudaGraphInstantiate(&c->exec, g, 0));
    size_t nn = 0;
    XG_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) XG_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
    int k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
    }
    c->graph_kernels = k;
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_chain_launch(xavs2gpu_chain_t *c)
{
    if (!c || !c->exec) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_launch", "no captured graph");
        return XAVS2GPU_ERR_ARG;
    }
    XG_CUDA(cudaSetDevice(c->device));
    XG_CUDA(cudaGraphLaunch(c->exec, c->st));
    count_launch(c->graph_kernels);
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_chain_graph_kernels(const xavs2gpu_chain_t *c) { return c ? c->graph_kernels : 0; }

extern "C" int xavs2gpu_chain_get_outputs(xavs2gpu_chain_t *c, xavs2gpu_chain_outputs_t *o)
{
    if (!c || !o) return XAVS2GPU_ERR_ARG;
    o->coef = c->d_coef;
    o->recon_residual = c->d_rres;
    o->nnz = c->d_nnz;
    o->blocks = c->d_blocks;
    o->recon = c->d_recon;
    o->choice = c->d_choice;
    o->n_residual = c->n_res;
    o->n_coef = c->n_coef;
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_chain_get_tuning(const xavs2gpu_chain_t *c, xavs2gpu_chain_tuning_t *t)
{
    if (!c || !t) return XAVS2GPU_ERR_ARG;
    xavs2gpu_me_get_tuning(c->s, &t->me);
    t->tq_warps = c->tq_warps;
    t->pad_ = 0;
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_chain_set_tuning(xavs2gpu_chain_t *c, const xavs2gpu_chain_tuning_t *t)
{
    if (!c || !t || (t->tq_warps != 4 && t->tq_warps != 8)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_set_tuning", "tq_warps must be 4 or 8");
        return XAVS2GPU_ERR_ARG;
    }
    const int rc = xavs2gpu_me_set_tuning(c->s, &t->me);
    if (rc != XAVS2GPU_OK) return rc;
    c->tq_warps = t->tq_warps;
    drop_graph(c);
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_chain_autotune(xavs2gpu_chain_t *c, const xavs2gpu_me_params_t *prm, int reps, float *best_ms)
{
    if (!c || !prm || reps < 1) return XAVS2GPU_ERR_ARG;
    XG_CUDA(cudaSetDevice(c->device));
    drop_graph(c);
    cudaEvent_t e0, e1;
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    auto time_cfg = [&](const xavs2gpu_chain_tuning_t &t, float &ms) -> int {
        int rc = xavs2gpu_chain_set_tuning(c, &t);
        if (rc != XAVS2GPU_OK) return rc;
        if ((rc = xavs2gpu_me_prepare(c->s, prm)) != XAVS2GPU_OK) return rc;
        if ((rc = chain_enqueue(c, prm)) != XAVS2GPU_OK) return rc;   // warm-up
        XG_CUDA(cudaEventRecord(e0, c->st));
        for (int i = 0; i < reps; i++)
            if ((rc = chain_enqueue(c, prm)) != XAVS2GPU_OK) return rc;
        XG_CUDA(cudaEventRecord(e1, c->st));
        XG_CUDA(cudaEventSynchronize(e1));
        XG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= reps;
        return XAVS2GPU_OK;
    };
    // coordinate search: the TU chain's CTA size, then the refinement split
    // and CTA size (the two stages are independent kernels)
    xavs2gpu_chain_tuning_t best;
    xavs2gpu_chain_get_tuning(c, &best);
    float best_t = 1e30f, t = 0.f;
    int rc = XAVS2GPU_OK;
    for (int w : {8, 4}) {
        xavs2gpu_chain_tuning_t cand = best;
        cand.tq_warps = w;
        if ((rc = time_cfg(cand, t)) != XAVS2GPU_OK) break;
        if (t < best_t) { best_t = t; best = cand; }
    }
    for (int split : {64, 128, 256, 512}) {
        if (rc != XAVS2GPU_OK) break;
        for (int cfg = 0; cfg < 4; cfg++) {
            xavs2gpu_chain_tuning_t cand = best;
            cand.me.refine_split_px = split;
            cand.me.refine_block = cfg & 1 ? 128 : 64;
            cand.me.cu_groups = cfg >> 1;
            if ((rc = time_cfg(cand, t)) != XAVS2GPU_OK) break;
            if (t < best_t) { best_t = t; best = cand; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != XAVS2GPU_OK) return rc;
    rc = xavs2gpu_chain_set_tuning(c, &best);
    if (rc == XAVS2GPU_OK) rc = xavs2gpu_me_prepare(c->s, prm);
    if (best_ms) *best_ms = best_t;
    return rc;
}
