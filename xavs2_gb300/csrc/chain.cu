// chain.cu -- one P picture of the encoder hot path on the device, over the
// leaf CUs of its quadtree: sub-pel planes of every reference and the
// current picture (interpolate_lcu_row, mc.c:593-785), the batched motion
// search (xavs2_me_search, me.c:879-1183), and every inter candidate of every
// CU through the TU chain (cand.cuh: predictions from the sub-pel planes,
// residuals, dct -> quant -> dequant -> idct as one TU and as the mode's TU
// split, SSDs, the reconstruction of each CU's chosen candidate).  The
// sequence is enqueued on the motion-search session's stream, eagerly or as
// one captured CUDA graph; an autotuner picks launch shapes that do not
// change any result.
#include "cand.cuh"

#include <vector>

namespace xg {

int tq_batch_launch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                    int16_t *recon, int32_t *nnz, int warps, cudaStream_t stream);

// Partition PUs of a CU relative to its 2Nx2N PU: (dx, dy, w, h) in units of
// S/4, in the order the CU record documents.
static const int8_t k_modes_big[13][4] = {{0, 0, 4, 4}, {0, 0, 4, 2}, {0, 2, 4, 2}, {0, 0, 2, 4}, {2, 0, 2, 4},
                                          {0, 0, 4, 1}, {0, 1, 4, 3}, {0, 0, 4, 3}, {0, 3, 4, 1},
                                          {0, 0, 1, 4}, {1, 0, 3, 4}, {0, 0, 3, 4}, {3, 0, 1, 4}};

static int part_of(int w, int h)
{
    for (int k = 0; k < kNumParts; k++)
        if (h_pu_w[k] == w && h_pu_h[k] == h) return k;
    return -1;
}

// The candidate table of a CU list over a PU list: every partition mode
// whose PUs follow the CU's 2Nx2N PU for every reference, else the 2Nx2N
// mode alone.  Returns false if a CU or its 2Nx2N PUs are invalid.
bool build_candidates(const xavs2gpu_cu_t *cus, int n_cus, const xavs2gpu_pu_t *pus, int n_pus, int W, int H,
                      int nrefs, std::vector<xavs2gpu_cand_t> &cands, std::vector<int32_t> &cu_cand, int64_t &n_res,
                      int64_t &n_coef)
{
    cands.clear();
    cu_cand.assign(n_cus + 1, 0);
    n_res = n_coef = 0;
    for (int i = 0; i < n_cus; i++) {
        const xavs2gpu_cu_t &c = cus[i];
        const int S = c.size;
        // CUs sit on the 8x8 grid (the candidate kernels read 4-pixel groups
        // as words)
        if (!(S == 8 || S == 16 || S == 32 || S == 64) || c.x < 0 || c.y < 0 || c.x + S > W || c.y + S > H ||
            ((c.x | c.y) & 7))
            return false;
        const int nk = S == 8 ? 5 : 13;
        bool all = true;
        for (int r = 0; r < nrefs; r++) {
            const int k0 = c.pu[r];
            if (k0 < 0 || k0 >= n_pus || pus[k0].x != c.x || pus[k0].y != c.y || pus[k0].part != part_of(S, S) ||
                pus[k0].ref != r)
                return false;
            for (int k = 1; k < nk && all; k++) {
                const int q = S / 4;
                const int8_t *m = k_modes_big[k];
                const int dx = m[0] * q, dy = m[1] * q, w = m[2] * q, h = m[3] * q;
                all = k0 + k < n_pus && pus[k0 + k].x == c.x + dx && pus[k0 + k].y == c.y + dy &&
                      pus[k0 + k].part == part_of(w, h) && pus[k0 + k].ref == r;
            }
        }
        const int nmodes = all ? (S == 8 ? 3 : 7) : 1;
        cu_cand[i] = (int32_t)cands.size();
        for (int m = 0; m < nmodes; m++) {
            xavs2gpu_cand_t cd;
            cd.cu = i;
            cd.mode = (int8_t)m;
            const bool nsqt = S > 8;
            cd.split_type = (int8_t)(!nsqt || m == 0 ? 1 : (m == 1 || m == 3 || m == 4) ? 2 : 3);
            cd.pad_ = 0;
            cd.res_offset = n_res;
            cd.coef_offset = n_coef;
            n_res += 2 * (int64_t)S * S;
            // levels packed without gaps: the one TU's, then the split TUs'
            // (64-point shapes keep a quarter)
            n_coef += (S == 64 ? 1024 : (int64_t)S * S) + (S == 64 && cd.split_type != 1 ? 1024 : (int64_t)S * S);
            cands.push_back(cd);
        }
    }
    cu_cand[n_cus] = (int32_t)cands.size();
    return true;
}

}  // namespace xg

using namespace xg;

struct xavs2gpu_chain {
    xavs2gpu_me_session_t *s = nullptr;
    int W = 0, H = 0, nrefs = 0, stride = 0, qp = 0, flags = 0, n_cus = 0, device = 0;
    int64_t n_cands = 0;
    cudaStream_t st = nullptr;
    xavs2gpu_cu_t *d_cus = nullptr;
    xavs2gpu_cand_t *d_cands = nullptr;
    int32_t *d_cu_cand = nullptr, *d_cost = nullptr, *d_dist = nullptr;
    int32_t *d_units = nullptr;                  // candidate units, then CU units
    int n_cand_units = 0, n_cu_units = 0;
    int16_t *d_res = nullptr, *d_rres = nullptr, *d_coef = nullptr;
    int32_t *d_nnz = nullptr;
    xavs2gpu_cu_choice_t *d_choice = nullptr;
    xavs2gpu_tq_block_t *d_blocks = nullptr;
    uint8_t *d_src = nullptr, *d_recon = nullptr;
    const uint8_t **d_planes = nullptr;
    PicView *d_view = nullptr;
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
    const unsigned cand_blocks = (unsigned)(((int64_t)c->n_cand_units * 32 + 127) / 128);
    cand_residual_kernel<<<cand_blocks, 128, 0, c->st>>>(c->d_view, 1, c->n_cand_units, c->qp, c->d_res, c->d_blocks,
                                                         c->d_cost, c->d_dist);
    count_launch();
    if ((rc = tq_batch_launch(c->d_blocks, (int)(5 * c->n_cands), c->d_res, c->d_coef, c->d_rres, c->d_nnz,
                              c->tq_warps, c->st)) != XAVS2GPU_OK)
        return rc;
    cand_eval_kernel<<<cand_blocks, 128, 0, c->st>>>(c->d_view, 1, c->n_cand_units, c->d_rres, c->d_dist);
    count_launch();
    cand_choose_kernel<<<(unsigned)(((int64_t)c->n_cu_units * 32 + 127) / 128), 128, 0, c->st>>>(
        c->d_view, 1, c->n_cu_units, c->d_cost, c->d_dist, c->d_rres, c->d_choice);
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
    std::vector<xavs2gpu_cand_t> cands;
    std::vector<int32_t> cu_cand;
    int64_t n_res = 0, n_coef = 0;
    if (!build_candidates(cus, n_cus, pus.data(), n, W, H, nrefs, cands, cu_cand, n_res, n_coef)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_create",
             "CU outside the picture or off the 8x8 grid, bad size, or pu[r] is not its 2Nx2N PU for reference r");
        return nullptr;
    }
    if (5 * (int64_t)cands.size() > INT32_MAX) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_chain_create", "too many candidates");
        return nullptr;
    }
    auto *c = new xavs2gpu_chain();
    c->s = s;
    c->W = W; c->H = H; c->nrefs = nrefs; c->qp = qp; c->flags = flags; c->n_cus = n_cus;
    c->n_cands = (int64_t)cands.size();
    c->stride = xavs2gpu_me_plane_stride(s);
    c->st = (cudaStream_t)xavs2gpu_me_stream(s);
    c->device = current_device();
    c->n_res = n_res;
    c->n_coef = n_coef;
    XG_CUDA(cudaMalloc((void **)&c->d_cus, sizeof(xavs2gpu_cu_t) * n_cus));
    XG_CUDA(cudaMemcpy(c->d_cus, cus, sizeof(xavs2gpu_cu_t) * n_cus, cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&c->d_cands, sizeof(xavs2gpu_cand_t) * cands.size()));
    XG_CUDA(cudaMemcpy(c->d_cands, cands.data(), sizeof(xavs2gpu_cand_t) * cands.size(), cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&c->d_cu_cand, sizeof(int32_t) * cu_cand.size()));
    XG_CUDA(cudaMemcpy(c->d_cu_cand, cu_cand.data(), sizeof(int32_t) * cu_cand.size(), cudaMemcpyHostToDevice));
    std::vector<int32_t> units;
    build_units(cus, n_cus, cands.data(), (int)cands.size(), units, c->n_cand_units, c->n_cu_units);
    XG_CUDA(cudaMalloc((void **)&c->d_units, sizeof(int32_t) * units.size()));
    XG_CUDA(cudaMemcpy(c->d_units, units.data(), sizeof(int32_t) * units.size(), cudaMemcpyHostToDevice));
    XG_CUDA(cudaMalloc((void **)&c->d_cost, sizeof(int32_t) * c->n_cands));
    XG_CUDA(cudaMalloc((void **)&c->d_dist, sizeof(int32_t) * 2 * c->n_cands));
    XG_CUDA(cudaMalloc((void **)&c->d_res, sizeof(int16_t) * n_res));
    XG_CUDA(cudaMalloc((void **)&c->d_rres, sizeof(int16_t) * n_res));
    XG_CUDA(cudaMalloc((void **)&c->d_coef, sizeof(int16_t) * n_coef));
    XG_CUDA(cudaMemset(c->d_coef, 0, sizeof(int16_t) * n_coef));
    XG_CUDA(cudaMalloc((void **)&c->d_nnz, sizeof(int32_t) * 5 * c->n_cands));
    XG_CUDA(cudaMalloc((void **)&c->d_choice, sizeof(xavs2gpu_cu_choice_t) * n_cus));
    XG_CUDA(cudaMalloc((void **)&c->d_blocks, sizeof(xavs2gpu_tq_block_t) * 5 * c->n_cands));
    XG_CUDA(cudaMalloc((void **)&c->d_src, (size_t)W * H * (1 + nrefs)));
    XG_CUDA(cudaMemset(c->d_src, 0, (size_t)W * H * (1 + nrefs)));
    XG_CUDA(cudaMalloc((void **)&c->d_recon, (size_t)W * H));
    std::vector<const uint8_t *> planes(16 * nrefs);
    for (int r = 0; r < nrefs; r++)
        for (int k = 0; k < 16; k++) planes[16 * r + k] = xavs2gpu_me_plane_device(s, r, k);
    XG_CUDA(cudaMalloc((void **)&c->d_planes, sizeof(uint8_t *) * planes.size()));
    XG_CUDA(cudaMemcpy(c->d_planes, planes.data(), sizeof(uint8_t *) * planes.size(), cudaMemcpyHostToDevice));
    PicView v{};
    v.cur = xavs2gpu_me_plane_device(s, -1, 0);
    v.planes = c->d_planes;
    v.res = xavs2gpu_me_results_device(s);
    v.cus = c->d_cus;
    v.cands = c->d_cands;
    v.cu_cand = c->d_cu_cand;
    v.cand_units = c->d_units;
    v.cu_units = c->d_units + c->n_cand_units;
    v.cand_unit_start = v.cu_unit_start = 0;
    v.recon = c->d_recon;
    v.hash = nullptr;
    v.res_off = v.coef_off = v.cu_start = v.cand_start = 0;
    v.n_coef = n_coef;
    v.n_cus = n_cus;
    v.n_cands = (int)c->n_cands;
    v.stride = c->stride;
    v.width = W;
    v.height = H;
    v.nrefs = nrefs;
    v.n_pus = n;
    XG_CUDA(cudaMalloc((void **)&c->d_view, sizeof(PicView)));
    XG_CUDA(cudaMemcpy(c->d_view, &v, sizeof(PicView), cudaMemcpyHostToDevice));
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
    cudaFree((void *)c->d_planes); cudaFree(c->d_cands); cudaFree(c->d_cu_cand); cudaFree(c->d_cost);
    cudaFree(c->d_dist); cudaFree(c->d_view); cudaFree(c->d_units);
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
    o->cands = c->d_cands;
    o->cand_cost = c->d_cost;
    o->dist = c->d_dist;
    o->n_cands = c->n_cands;
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
