// intra.cu -- AVS2 intra prediction for sm_103a: the per-call drop-ins of
// the reference's intraf[] table (source/common/primitives.h:186-188, C
// versions intra.c:127-1897) and the batched rough mode decision of the
// encoder (encoder/md_intra.c:195-380): every mode's prediction of a block,
// its SATD (or SAD) against the source plus lambda * mode bits, and the
// candidate list the encoder hands to RDO.
//
// `ep` is the top-left edge sample: ep[1..] the top row continuing into the
// top-right, ep[-1..] the left column continuing downwards (intra.c:1590).
// Every prediction sample is computed independently from the edge (the
// angular, DC, plane and bilinear formulas in closed form), so a warp
// predicts a block into shared memory and scores it in the same pass.
#include "xavs2gpu_common.cuh"

#include <cstring>

namespace xg {
namespace intra {

// Angle steps (multiplier, shift) along x per row (0) and along y per
// column (1) of every mode (intra.c:98-120, normative AVS2 geometry).
__constant__ int8_t c_ang[2][33][2] = {
    {{0, 0}, {0, 0}, {0, 0},
     {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}, {93, 8}, {1, 2}, {1, 3},
     {0, 0},
     {1, 3}, {1, 2}, {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}, {11, 2}, {4, 0}, {8, 0},
     {0, 0},
     {8, 0}, {4, 0}, {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}},
    {{0, 0}, {0, 0}, {0, 0},
     {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}, {11, 2}, {4, 0}, {8, 0},
     {0, 0},
     {8, 0}, {4, 0}, {11, 2}, {2, 0}, {11, 3}, {1, 0}, {93, 7}, {1, 1}, {93, 8}, {1, 2}, {1, 3},
     {0, 0},
     {1, 3}, {1, 2}, {93, 8}, {1, 1}, {93, 7}, {1, 0}, {11, 3}, {2, 0}}};

__device__ __forceinline__ int ang_step(int mode, int axis, int d, int &frac)
{
    const int t = d * c_ang[axis][mode][0], sh = c_ang[axis][mode][1];
    const int n = t >> sh;
    frac = ((t << 5) >> sh) - (n << 5);
    return n;
}

__device__ __forceinline__ int ilog2d(int v) { return 31 - __clz(v); }

// The edge samples the predictors of a bsx x bsy block read: from
// ep[-edge_below] (left-down padding) to ep[edge_above] (top-right padding),
// two beyond what fill_reference_samples writes (intra.c:1606-1640).
__host__ __device__ __forceinline__ int edge_below(int bsx, int bsy) { return bsy + (11 * bsx) / 4 + 6; }
__host__ __device__ __forceinline__ int edge_above(int bsx, int bsy) { return bsx + (11 * bsy) / 4 + 6; }

// Per-(block, mode) constants of the non-angular modes.
struct ModeConst {
    int dc;                  // DC value
    int pa, pb, pc;          // plane: a (with the 16 rounding and offsets folded in), b, c
    int ba, bb, bt, lx, ly;  // bilinear: top-right, bottom-left, corner term, log2 sizes
};

// angular sample from the top row
__device__ __forceinline__ int ang_top(int mode, const uint8_t *ep, int x, int y)
{
    int f;
    const int ix = ang_step(mode, 0, y + 1, f) + x;
    return (ep[ix] * (32 - f) + ep[ix + 1] * (64 - f) + ep[ix + 2] * (32 + f) + ep[ix + 3] * f + 64) >> 7;
}

// angular sample from the left column
__device__ __forceinline__ int ang_left(int mode, const uint8_t *ep, int x, int y)
{
    int f;
    const int iy = y + ang_step(mode, 1, x + 1, f);
    return (ep[-iy] * (32 - f) + ep[-iy - 1] * (64 - f) + ep[-iy - 2] * (32 + f) + ep[-iy - 3] * f + 64) >> 7;
}

// The reference's mode-5 entry on 4x16 / 8x32 (intra_pred_ang_x_5_c,
// intra.c:455-605): the first 4 / 8 rows angular, the rest one edge sample
// (ep[8] / ep[16]) except a few samples just below.  `ep(k)` reads edge k.
template <typename Edge>
__device__ __forceinline__ int mode5_narrow(Edge ep, int x, int y, int bsx)
{
    const int rows = bsx == 4 ? 4 : 8;
    if (y < rows) {
        int f;
        const int ix = ang_step(5, 0, y + 1, f) + x;
        return (ep(ix) * (32 - f) + ep(ix + 1) * (64 - f) + ep(ix + 2) * (32 + f) + ep(ix + 3) * f + 64) >> 7;
    }
    if (bsx == 4) {
        if (y == 4 && x < 2) return (ep(6 + x) + 9 * ep(7 + x) + 15 * ep(8 + x) + 7 * ep(9 + x) + 16) >> 5;
        return ep(8);
    }
    if (y == 8 && x < 4) return (5 * ep(12 + x) + 13 * ep(13 + x) + 11 * ep(14 + x) + 3 * ep(15 + x) + 16) >> 5;
    if (y == 9 && x < 3) return (ep(13 + x) + 5 * ep(14 + x) + 7 * ep(15 + x) + 3 * ep(16 + x) + 8) >> 4;
    if (y == 10 && x == 0) return (7 * ep(15) + 15 * ep(16) + 9 * ep(17) + ep(18) + 16) >> 5;
    return ep(16);
}

// Prediction sample (x, y) of a bsx x bsy block in `mode`.  Mode 31 on 16x64
// is the angular formula in every column (the reference writes columns 0-3
// only, intra.c:1176-1183).
__device__ __forceinline__ int pred_sample(int mode, const uint8_t *ep, int x, int y, int bsx, int bsy,
                                           const ModeConst &k)
{
    if (mode == 0) return k.dc;
    if (mode == 1) return min(max((k.pa + k.pb * x + k.pc * y) >> 5, 0), 255);
    if (mode == 2) {
        const int top = ep[1 + x], left = ep[-1 - y];
        const int predx = (left << k.lx) + (x + 1) * (k.ba - left);
        const int predy = (top << k.ly) + (y + 1) * (k.bb - top);
        const int v = ((predx << k.ly) + (predy << k.lx) + x * y * k.bt + (1 << (k.lx + k.ly))) >> (k.lx + k.ly + 1);
        return min(max(v, 0), 255);
    }
    if (mode == 12) return ep[1 + x];
    if (mode == 24) return ep[-1 - y];
    if (mode == 5 && ((bsx == 4 && bsy == 16) || (bsx == 8 && bsy == 32)))
        return mode5_narrow([ep](int i) { return (int)ep[i]; }, x, y, bsx);
    if (mode == 31 && ((bsx == 16 && bsy == 4) || (bsx == 32 && bsy == 8)))
        return mode5_narrow([ep](int i) { return (int)ep[-i]; }, y, x, bsy);   // on the transposed edge and block
    if (mode < 12) return ang_top(mode, ep, x, y);
    if (mode > 24) return ang_left(mode, ep, x, y);
    // both edges (intra.c:363-397)
    int fx, fy;
    const int ixx = -ang_step(mode, 0, y + 1, fx) + x;
    const int iyy = y - ang_step(mode, 1, x + 1, fy);
    int v;
    if (iyy <= -1)
        v = ep[ixx + 2] * (32 - fx) + ep[ixx + 1] * (64 - fx) + ep[ixx] * (32 + fx) + ep[ixx - 1] * fx;
    else
        v = ep[-iyy - 2] * (32 - fy) + ep[-iyy - 1] * (64 - fy) + ep[-iyy] * (32 + fy) + ep[-iyy + 1] * fy;
    return (v + 64) >> 7;
}

__device__ __forceinline__ int warp_sum(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Constants of the DC / plane / bilinear modes, computed by a whole warp.
__device__ ModeConst mode_const(int mode, const uint8_t *ep, int dc_avail, int bsx, int bsy, int lane)
{
    ModeConst k{};
    if (mode == 0) {          // intra.c:153-190
        int sl = 0, sa = 0;
        for (int i = lane; i < bsy; i += 32) sl += ep[-1 - i];
        for (int i = lane; i < bsx; i += 32) sa += ep[1 + i];
        sl = warp_sum(sl);
        sa = warp_sum(sa);
        const int top = dc_avail >> 8, left = dc_avail & 0xFF;
        if (top && left) k.dc = ((sl + sa + ((bsx + bsy) >> 1)) * (512 / (bsx + bsy))) >> 9;
        else if (left) k.dc = (sl + (bsy >> 1)) >> ilog2d(bsy);
        else if (top) k.dc = (sa + (bsx >> 1)) >> ilog2d(bsx);
        else k.dc = 128;
    } else if (mode == 1) {   // intra.c:192-236
        const int mult[7] = {0, 0, 13, 17, 5, 11, 23}, shf[7] = {0, 0, 7, 10, 11, 15, 19};
        const int lx = ilog2d(bsx), ly = ilog2d(bsy), w2 = bsx >> 1, h2 = bsy >> 1;
        int H = 0, V = 0;
        for (int i = lane + 1; i <= w2; i += 32) H += i * (ep[w2 + i] - ep[w2 - i]);
        for (int i = lane + 1; i <= h2; i += 32) V += i * (ep[-h2 - i] - ep[-h2 + i]);
        H = warp_sum(H);
        V = warp_sum(V);
        k.pb = ((H << 5) * mult[lx] + (1 << (shf[lx] - 1))) >> shf[lx];
        k.pc = ((V << 5) * mult[ly] + (1 << (shf[ly] - 1))) >> shf[ly];
        k.pa = ((ep[-bsy] + ep[bsx]) << 4) + 16 - k.pb * (w2 - 1) - k.pc * (h2 - 1);
    } else if (mode == 2) {   // intra.c:238-293
        const int lx = ilog2d(bsx), ly = ilog2d(bsy), sh = min(lx, ly);
        const int a = ep[bsx], b = ep[-bsy];
        const int c = bsx == bsy ? (a + b + 1) >> 1 : (((a << lx) + (b << ly)) * 13 + (1 << (sh + 5))) >> (sh + 6);
        k.ba = a;
        k.bb = b;
        k.bt = 2 * c - a - b;
        k.lx = lx;
        k.ly = ly;
    }
    return k;
}

// ---- per-call kernel: one block into dst (an untouched sample of mode 31
// on 16x64 keeps dst's value) -------------------------------------------------
__global__ void __launch_bounds__(256) pred_block_kernel(int mode, const uint8_t *ep, uint8_t *dst, int i_dst,
                                                         int dc_avail, int bsx, int bsy)
{
    __shared__ ModeConst k;
    if (threadIdx.x < 32) {
        const ModeConst v = mode_const(mode, ep, dc_avail, bsx, bsy, threadIdx.x);
        if (threadIdx.x == 0) k = v;
    }
    __syncthreads();
    const bool cols4 = mode == 31 && bsx == 16 && bsy == 64;
    for (int i = threadIdx.x; i < bsx * bsy; i += blockDim.x) {
        const int y = i / bsx, x = i - y * bsx;
        if (cols4 && x >= 4) continue;
        dst[y * i_dst + x] = (uint8_t)pred_sample(mode, ep, x, y, bsx, bsy, k);
    }
}

// ---- batched rough mode decision -----------------------------------------------
constexpr int kWarps = 8;
constexpr int kEdge = 256;        // staged edge: ep at edge[256], windows up to 246 below / 198 above
constexpr int kN = 9;             // INTRA_MODE_NUM_FOR_RDO (defines.h:290)

struct Smem {
    uint8_t edge[2 * kEdge];
    uint8_t fenc[64 * 64];
    uint8_t pred[kWarps][64 * 64];
    double cost[33];
};

// update_candidate_list (md_intra.c:195-210): insertion into the list kept
// sorted by cost, after equal costs
__device__ void cand_insert(int mode, double cost, int *modes, double *costs)
{
    int i = kN - 1;
    if (!(cost < costs[i])) return;
    while (i > 0 && cost < costs[i - 1]) {
        modes[i] = modes[i - 1];
        costs[i] = costs[i - 1];
        i--;
    }
    modes[i] = mode;
    costs[i] = cost;
}

// The candidate list of rdo_get_pred_intra_luma (all modes) or of the rough
// three-phase search rdo_get_pred_intra_luma_rmd (md_intra.c:258-380),
// replayed on the per-mode costs; returns the number of modes for RDO.
__device__ int candidates(const double *cost, int rough, int dist2, int dist1, int num_for_rdo, const int *mpm,
                          int *modes, double *costs)
{
    int visited[33];
    for (int m = 0; m < 33; m++) visited[m] = 0;
    for (int i = 0; i < kN; i++) {
        modes[i] = 0;
        costs[i] = (double)(1LL << 50);   // MAX_COST (defines.h:299)
    }
    auto visit = [&](int m) {
        cand_insert(m, cost[m], modes, costs);
        visited[m] = 1;
    };
    if (!rough) {
        for (int m = 0; m < 33; m++) visit(m);
        return num_for_rdo;
    }
    for (int m = 0; m < 3; m++) visit(m);
    for (int m = 4; m < 33; m += 4) visit(m);
    for (int i = 0; i < dist2; i++) {
        const int m = modes[i];
        if (m <= 2) continue;
        if (m > 3 && !visited[m - 2]) visit(m - 2);
        if (m < 31 && !visited[m + 2]) visit(m + 2);
    }
    for (int i = 0, na = 0; na < dist1 && i < kN; i++) {
        const int m = modes[i];
        if (m <= 2) continue;
        if (m > 3 && !visited[m - 1]) { visit(m - 1); na++; }
        if (m < 32 && !visited[m + 1]) { visit(m + 1); na++; }
    }
    if (!visited[mpm[0]]) visit(mpm[0]);
    if (!visited[mpm[1]]) visit(mpm[1]);
    if (modes[0] == mpm[0] || modes[0] == mpm[1] || modes[1] == mpm[0] || modes[1] == mpm[1])
        return num_for_rdo < 3 ? num_for_rdo : 3;
    visited[modes[0]] = 2;
    visited[modes[1]] = 2;
    int j = 2;
    for (int i = 2; i < kN && j < num_for_rdo; i++) {
        const int m = modes[i];
        if (!visited[m]) continue;
        if (m <= 2) {
            modes[j++] = m;
            visited[m] = 2;
        } else if (m == 3) {
            if (visited[4] == 1) { modes[j++] = 3; visited[3] = 2; }
        } else if (m == 32) {
            if (visited[31] == 1) { modes[j++] = 32; visited[32] = 2; }
        } else if (visited[m - 1] == 1 && visited[m + 1] == 1) {
            modes[j++] = m;
            visited[m] = 2;
        }
        if (visited[0] == 2 && visited[1] == 2 && visited[2] == 2) break;
    }
    return num_for_rdo < j ? num_for_rdo : j;
}

__global__ void __launch_bounds__(kWarps * 32) rmd_kernel(const xavs2gpu_intra_block_t *__restrict__ blocks, int n,
                                                          const uint8_t *__restrict__ edges,
                                                          const uint8_t *__restrict__ fenc, int fenc_stride,
                                                          xavs2gpu_intra_params_t prm,
                                                          xavs2gpu_intra_result_t *__restrict__ out)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    Smem &s = *reinterpret_cast<Smem *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int bi = blockIdx.x; bi < n; bi += gridDim.x) {
        const xavs2gpu_intra_block_t b = blocks[bi];
        const int bsx = b.width, bsy = b.height;
        const auto ok_side = [](int v) { return v == 4 || v == 8 || v == 16 || v == 32 || v == 64; };
        if (!ok_side(bsx) || !ok_side(bsy) || b.mpm[0] < 0 || b.mpm[0] > 32 || b.mpm[1] < 0 || b.mpm[1] > 32) {
            if (threadIdx.x == 0) out[bi].num_for_rdo = -1;   // not a block the encoder predicts
            continue;
        }
        const uint8_t *ep_g = edges + b.edge_offset;
        const int lo = edge_below(bsx, bsy), hi = edge_above(bsx, bsy);
        for (int i = threadIdx.x - lo; i <= hi; i += blockDim.x) s.edge[kEdge + i] = ep_g[i];
        const uint8_t *src = fenc + b.fenc_offset;
        for (int i = threadIdx.x; i < bsx * bsy; i += blockDim.x) s.fenc[i] = src[(i / bsx) * fenc_stride + i % bsx];
        __syncthreads();
        const uint8_t *ep = s.edge + kEdge;
        uint8_t *pred = s.pred[warp];
        const bool u4 = prm.use_hadamard ? satd_unit4(bsx, bsy) : (bsx == 4);
        const int uw = u4 ? 4 : 8, nux = bsx / uw, nu = nux * (bsy >> 2);
        for (int mode = warp; mode < 33; mode += kWarps) {
            const ModeConst k = mode_const(mode, ep, b.dc_avail, bsx, bsy, lane);
            for (int i = lane; i < bsx * bsy; i += 32) {
                const int y = i / bsx, x = i - y * bsx;
                pred[i] = (uint8_t)pred_sample(mode, ep, x, y, bsx, bsy, k);
            }
            __syncwarp();
            int d = 0;
            for (int u = lane; u < nu; u += 32) {
                const int uy = u / nux, ux = u - uy * nux;
                const int off = uy * 4 * bsx + ux * uw;
                if (prm.use_hadamard) {
                    d += satd_unit_d(u4, s.fenc + off, bsx, pred + off, bsx);
                } else {
                    for (int r = 0; r < 4; r++)
                        for (int c = 0; c < uw; c++) d += iabs_d((int)s.fenc[off + r * bsx + c] - (int)pred[off + r * bsx + c]);
                }
            }
            d = warp_sum(d);
            if (lane == 0) {
                const int bits = (b.mpm[0] == mode || b.mpm[1] == mode) ? 2 : 6;
                s.cost[mode] = __dadd_rn(__dmul_rn(prm.lambda, (double)bits), (double)d);
            }
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            xavs2gpu_intra_result_t &r = out[bi];
            const int mpm[2] = {b.mpm[0], b.mpm[1]};
            int modes[kN];
            double costs[kN];
            r.num_for_rdo = candidates(s.cost, prm.rough, prm.dist2, prm.dist1, b.num_for_rdo, mpm, modes, costs);
            for (int i = 0; i < kN; i++) {
                r.cand_mode[i] = modes[i];
                r.cand_cost[i] = costs[i];
            }
        }
        for (int m = threadIdx.x; m < 33; m += blockDim.x) out[bi].cost[m] = s.cost[m];
        __syncthreads();
    }
}

}  // namespace intra
}  // namespace xg

using namespace xg;

// ---- per-call drop-ins (intra_pred_t, primitives.h:84) -----------------------------
static void intra_call(int mode, uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    const int lo = intra::edge_below(bsx, bsy), hi = intra::edge_above(bsx, bsy);
    const int ne = lo + hi + 1;
    const size_t o_edge = 0, o_blk = align_up((size_t)ne);
    CallCtx &c = call_ctx(o_blk + (size_t)bsx * bsy);
    memcpy(c.h_stage + o_edge, src - lo, ne);
    pack_rows(c.h_stage + o_blk, dst, i_dst, bsx, bsy);   // samples a mode leaves alone keep their value
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_blk + (size_t)bsx * bsy, cudaMemcpyHostToDevice, c.stream));
    intra::pred_block_kernel<<<1, 256, 0, c.stream>>>(mode, c.d_stage + o_edge + lo, c.d_stage + o_blk, bsx, dir_mode,
                                                     bsx, bsy);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_blk, c.d_stage + o_blk, (size_t)bsx * bsy, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    unpack_rows(dst, i_dst, c.h_stage + o_blk, bsx, bsy);
}

extern "C" void xavs2gpu_intra_pred_dc(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    intra_call(0, src, dst, i_dst, dir_mode, bsx, bsy);
}
extern "C" void xavs2gpu_intra_pred_plane(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    (void)dir_mode;
    intra_call(1, src, dst, i_dst, 1, bsx, bsy);
}
extern "C" void xavs2gpu_intra_pred_bilinear(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    (void)dir_mode;
    intra_call(2, src, dst, i_dst, 2, bsx, bsy);
}
extern "C" void xavs2gpu_intra_pred_ver(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    (void)dir_mode;
    intra_call(12, src, dst, i_dst, 12, bsx, bsy);
}
extern "C" void xavs2gpu_intra_pred_hor(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    (void)dir_mode;
    intra_call(24, src, dst, i_dst, 24, bsx, bsy);
}
extern "C" void xavs2gpu_intra_pred_ang(uint8_t *src, uint8_t *dst, int i_dst, int dir_mode, int bsx, int bsy)
{
    if (dir_mode < 3 || dir_mode > 32 || dir_mode == 12 || dir_mode == 24) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_intra_pred_ang", "not an angular mode");
        return;
    }
    intra_call(dir_mode, src, dst, i_dst, dir_mode, bsx, bsy);
}

extern "C" void xavs2gpu_intra_pred_init(uint32_t cpuid, xavs2gpu_intra_pred_t intraf[33])
{
    (void)cpuid;
    intraf[0] = xavs2gpu_intra_pred_dc;
    intraf[1] = xavs2gpu_intra_pred_plane;
    intraf[2] = xavs2gpu_intra_pred_bilinear;
    for (int m = 3; m < 33; m++) intraf[m] = xavs2gpu_intra_pred_ang;
    intraf[12] = xavs2gpu_intra_pred_ver;
    intraf[24] = xavs2gpu_intra_pred_hor;
}

extern "C" int xavs2gpu_intra_rmd_batch(const xavs2gpu_intra_block_t *blocks, int n, const uint8_t *edges,
                                        const uint8_t *fenc, int fenc_stride, const xavs2gpu_intra_params_t *prm,
                                        xavs2gpu_intra_result_t *out, void *stream)
{
    if (n < 0 || !prm || prm->dist1 < 0 || prm->dist2 < 0) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_intra_rmd_batch", "bad count or parameters");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    static bool attr[64] = {false};
    const int dev = current_device();
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        XG_CUDA(cudaFuncSetAttribute(intra::rmd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(intra::Smem)));
        attr[dev] = true;
    }
    const int grid = n < 152 * 8 ? n : 152 * 8;
    intra::rmd_kernel<<<grid, intra::kWarps * 32, sizeof(intra::Smem), (cudaStream_t)stream>>>(
        blocks, n, edges, fenc, fenc_stride, *prm, out);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
