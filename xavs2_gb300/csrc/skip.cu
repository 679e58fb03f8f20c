// skip.cu -- rough cost of skip / direct candidates for sm_103a
// (cu_check_skip_direct_rough2, encoder/rdo.c:2395-2480): for every
// candidate of a CU its prediction from the resident sub-pel planes of a
// motion-search session (one list or the average of two, pixel_avg,
// pixel.c:680-719), the SA8D of the luma prediction against the source
// (pixf.sa8d, pixel.c:416-530) and rdcost = distortion + lambda * rate
// (rdcost_t, double); per CU the first candidate with the strictly smallest
// rdcost.  A candidate whose motion equals an earlier candidate's of the
// same CU is not evaluated (update_skip_mv_list, rdo.c:2366-2389).
#include "xavs2gpu_common.cuh"

namespace xg {
namespace skp {

constexpr int kPad = 80;   // plane margin of a session (XAVS2_PAD, defines.h:298)

struct Ctx {
    const uint8_t *cur;
    const uint8_t *const *planes;   // 16 r + k
    int stride, W, H, nrefs;
    const xavs2gpu_skip_cand_t *cands;
    int n;
    double lambda;
    int32_t *dist;
    double *cost;
};

// motion of two candidates equal (the n_pu PUs' references and vectors)
__device__ __forceinline__ bool same_motion(const xavs2gpu_skip_cand_t &a, const xavs2gpu_skip_cand_t &b)
{
    if (a.n_pu != b.n_pu) return false;
    for (int q = 0; q < a.n_pu; q++)
        for (int l = 0; l < 2; l++) {
            if (a.ref[q][l] != b.ref[q][l]) return false;
            if (a.ref[q][l] >= 0 && (a.mv[q][l][0] != b.mv[q][l][0] || a.mv[q][l][1] != b.mv[q][l][1])) return false;
        }
    return true;
}

// a PU's prediction stays inside the planes' margin
__device__ __forceinline__ bool pu_inside(const Ctx &c, int x, int y, int w, int h, int ref, int mvx, int mvy)
{
    if (ref < 0) return true;
    if (ref >= c.nrefs) return false;
    const int px = x + (mvx >> 2), py = y + (mvy >> 2);
    return px >= -kPad && py >= -kPad && px + w <= c.W + kPad && py + h <= c.H + kPad;
}

// Validity of a candidate (shape, inside the picture, every PU with a list,
// references inside the session and their blocks inside the planes'
// margin) and the encoder's repeated-motion check against the earlier
// candidates of the same CU.
__device__ bool cand_ok(const Ctx &c, int i, const xavs2gpu_skip_cand_t &k)
{
    const int S = 1 << k.size_log2;
    if (k.size_log2 < 3 || k.size_log2 > 6 || (k.n_pu != 1 && k.n_pu != 4) || k.x < 0 || k.y < 0 ||
        k.x + S > c.W || k.y + S > c.H)
        return false;
    const int hp = k.n_pu == 4 ? S >> 1 : S;
    for (int q = 0; q < k.n_pu; q++) {
        if (k.ref[q][0] < 0 && k.ref[q][1] < 0) return false;
        for (int l = 0; l < 2; l++)
            if (!pu_inside(c, k.x + (q & 1) * hp, k.y + (q >> 1) * hp, hp, hp, k.ref[q][l], k.mv[q][l][0],
                           k.mv[q][l][1]))
                return false;
    }
    for (int j = i - 1; j >= 0; j--) {
        const xavs2gpu_skip_cand_t &e = c.cands[j];
        if (e.cu != k.cu) break;
        if (same_motion(e, k)) return false;
    }
    return true;
}

// Prediction source of one PU: per list the address of the PU's top-left
// prediction sample in the sub-pel plane of its fractional vector.
struct PuSrc {
    const uint8_t *p[2];
    int n;
};
__device__ __forceinline__ PuSrc pu_src(const Ctx &c, const xavs2gpu_skip_cand_t &k, int q, int X, int Y)
{
    PuSrc s{{nullptr, nullptr}, 0};
    for (int l = 0; l < 2; l++) {
        const int r = k.ref[q][l];
        if (r < 0) continue;
        const int mx = k.mv[q][l][0], my = k.mv[q][l][1];
        s.p[s.n++] = c.planes[16 * r + ((my & 3) << 2) + (mx & 3)] + (long long)(Y + (my >> 2)) * c.stride + X +
                     (mx >> 2);
    }
    if (s.n == 1) s.p[1] = s.p[0];
    return s;
}

// 4 samples at any byte address, from the two aligned words holding them
// (the word after the last sample is read too: planes and pictures have an
// 80-sample margin, so it is inside the allocation)
__device__ __forceinline__ uint32_t ld4u(const uint8_t *p)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    return __funnelshift_r(w[0], w[1], (unsigned)(a & 3) * 8u);
}

// bytewise (a + b + 1) >> 1 of four packed samples (pixel_avg, pixel.c:680-700)
__device__ __forceinline__ uint32_t avg4(uint32_t a, uint32_t b) { return (a | b) - (((a ^ b) >> 1) & 0x7F7F7F7Fu); }

// |H8 (src - pred) H8^T| of the 8x8 block at (X, Y); the prediction of
// sample (x, y) comes from src4[(y >= 4) * 2 + (x >= 4)] (four 4x4 PUs of an
// 8x8 CU) or from src4[0] everywhere, relative to each PU's own corner.
// Rows are read as words: the current block's aligned, the prediction's at
// any alignment.
template <bool QUAD>
__device__ int hsum8_pred(const Ctx &c, int X, int Y, const PuSrc *src4)
{
    int m[8][8];
#pragma unroll
    for (int y = 0; y < 8; y++) {
        // the current picture is the session's plane: stride a multiple of
        // 64, origin 16-byte aligned, X a multiple of 8
        const uint2 cw = *reinterpret_cast<const uint2 *>(c.cur + (long long)(Y + y) * c.stride + X);
        const uint32_t c0 = cw.x, c1 = cw.y;
        uint32_t pw[2];
        if (QUAD) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const PuSrc &ps = src4[(y >= 4) * 2 + h];
                const long long o = (long long)(y & 3) * c.stride;
                const uint32_t a = ld4u(ps.p[0] + o);
                pw[h] = ps.n == 2 ? avg4(a, ld4u(ps.p[1] + o)) : a;   // one list: the plane's samples
            }
        } else {
            // the row's 8 prediction samples from the 3 aligned words holding them
            auto ld8u = [&](const uint8_t *q, uint32_t &lo, uint32_t &hi) {
                const uintptr_t a = reinterpret_cast<uintptr_t>(q);
                const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
                const unsigned sh = (unsigned)(a & 3) * 8u;
                const uint32_t w0 = w[0], w1 = w[1], w2 = w[2];
                lo = __funnelshift_r(w0, w1, sh);
                hi = __funnelshift_r(w1, w2, sh);
            };
            const long long o = (long long)y * c.stride;
            ld8u(src4[0].p[0] + o, pw[0], pw[1]);
            if (src4[0].n == 2) {
                uint32_t b0, b1;
                ld8u(src4[0].p[1] + o, b0, b1);
                pw[0] = avg4(pw[0], b0);
                pw[1] = avg4(pw[1], b1);
            }
        }
        int t[8];
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const uint32_t cv = x < 4 ? c0 : c1, pv = pw[x >> 2];
            t[x] = (int)((cv >> (8 * (x & 3))) & 0xFFu) - (int)((pv >> (8 * (x & 3))) & 0xFFu);
        }
        int u[8];
#pragma unroll
        for (int i = 0; i < 4; i++) { u[i] = t[i] + t[i + 4]; u[i + 4] = t[i] - t[i + 4]; }
        fwht4_d(u[0], u[1], u[2], u[3]);
        fwht4_d(u[4], u[5], u[6], u[7]);
#pragma unroll
        for (int x = 0; x < 8; x++) m[y][x] = u[x];
    }
    int s = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
        int u[8];
#pragma unroll
        for (int i = 0; i < 4; i++) { u[i] = m[i][x] + m[i + 4][x]; u[i + 4] = m[i][x] - m[i + 4][x]; }
        fwht4_d(u[0], u[1], u[2], u[3]);
        fwht4_d(u[4], u[5], u[6], u[7]);
#pragma unroll
        for (int i = 0; i < 8; i++) s += iabs_d(u[i]);
    }
    return s;
}

// 1. per-size counts (warp-aggregated); malformed candidates are reported here
__global__ void skip_count_kernel(Ctx c, int *__restrict__ counts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int cl = -1;
    if (i < c.n) {
        const int sl = c.cands[i].size_log2;
        cl = (sl >= 3 && sl <= 6) ? sl - 3 : -1;
        if (cl < 0) {
            c.dist[i] = -1;
            c.cost[i] = (double)(1LL << 50);
        }
    }
    const unsigned valid = __ballot_sync(0xffffffffu, cl >= 0);
    if (cl >= 0) {
        const unsigned same = __match_any_sync(valid, cl);
        if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&counts[cl], __popc(same));
    }
}

// 2. scatter into size order
__global__ void skip_scatter_kernel(Ctx c, const int *__restrict__ counts, int *__restrict__ cursor,
                                    int *__restrict__ sorted)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    int cl = -1;
    if (i < c.n) {
        const int sl = c.cands[i].size_log2;
        cl = (sl >= 3 && sl <= 6) ? sl - 3 : -1;
    }
    const unsigned valid = __ballot_sync(0xffffffffu, cl >= 0);
    if (cl < 0) return;
    const unsigned same = __match_any_sync(valid, cl);
    const int leader = __ffs(same) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&cursor[cl], __popc(same));
    base = __shfl_sync(same, base, leader);
    int start = 0;
    for (int k = 0; k < cl; k++) start += counts[k];
    sorted[start + base + __popc(same & ((1u << lane) - 1))] = i;
}

// 3. costs: a warp takes 32 / L candidates of one size, L = min(32, number
// of 8x8 blocks) lanes each; lane s of a candidate takes 8x8 blocks s and
// s + 32 in z-order, so the four blocks of a 16x16 SA8D unit sit in four
// consecutive lanes (their sums are rounded together, pixel.c:470-500).
// resident 128-thread CTAs per SM the register budget is sized for (4: 128
// registers; the kernel waits on plane gathers, and 4 CTAs measured faster
// than 3 (the compiler's own 134 registers), 5 and 6)
#ifndef XG_SKIP_MINB
#define XG_SKIP_MINB 4
#endif
__global__ void __launch_bounds__(128, XG_SKIP_MINB) skip_cost_kernel(Ctx c, const int *__restrict__ counts,
                                                                      const int *__restrict__ sorted)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    int start = 0, first = 0, cl = -1;
    for (int k = 0; k < 4; k++) {
        const int L = min(32, 1 << (2 * k)), groups = (counts[k] * L + 31) / 32;
        if (cl < 0 && warp < first + groups) {
            cl = k;
            start += (warp - first) * (32 / L);
            break;
        }
        first += groups;
        start += counts[k];
    }
    if (cl < 0) return;
    const int L = min(32, 1 << (2 * cl)), nsub = 1 << (2 * cl);
    const int slot = lane / L, sub = lane - slot * L;
    const int end = [&]() { int e = 0; for (int k = 0; k <= cl; k++) e += counts[k]; return e; }();
    const int pos = start + slot;
    const bool live = pos < end;
    const int i = live ? sorted[pos] : -1;
    xavs2gpu_skip_cand_t k{};
    bool ok = false;
    if (live) {
        k = c.cands[i];
        if (sub == 0) ok = cand_ok(c, i, k);
    }
    ok = __shfl_sync(0xffffffffu, ok, lane - sub) && live;
    int acc = 0;
    const int S = ok ? 1 << k.size_log2 : 8, hp = k.n_pu == 4 ? S >> 1 : S;
    const bool quad = ok && k.n_pu == 4 && S == 8;
    for (int s0 = 0; s0 < nsub; s0 += 32) {   // the same trip count for every lane of the warp
        const int s = s0 + sub;
        int h = 0;
        if (ok && s < nsub) {
            // z-order position of 8x8 block s
            int bx = 0, by = 0;
#pragma unroll
            for (int b = 0; b < 3; b++) {
                bx |= ((s >> (2 * b)) & 1) << b;
                by |= ((s >> (2 * b + 1)) & 1) << b;
            }
            const int X = k.x + 8 * bx, Y = k.y + 8 * by;
            PuSrc src4[4];
            if (quad) {
#pragma unroll
                for (int q = 0; q < 4; q++) src4[q] = pu_src(c, k, q, k.x + (q & 1) * 4, k.y + (q >> 1) * 4);
            } else {
                const int q = k.n_pu == 4 ? (8 * bx >= hp) + 2 * (8 * by >= hp) : 0;
                src4[0] = pu_src(c, k, q, X, Y);
            }
            h = quad ? hsum8_pred<true>(c, X, Y, src4) : hsum8_pred<false>(c, X, Y, src4);
        }
        if (cl == 0) {
            acc += (h + 2) >> 2;                          // one 8x8 SA8D unit
        } else {
            h += __shfl_xor_sync(0xffffffffu, h, 1);      // the 16x16 unit of 4 lanes
            h += __shfl_xor_sync(0xffffffffu, h, 2);
            if ((sub & 3) == 0) acc += (h + 2) >> 2;
        }
    }
    for (int o = L >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (live && sub == 0) {
        c.dist[i] = ok ? acc : -1;
        c.cost[i] = ok ? __dadd_rn((double)acc, __dmul_rn(c.lambda, (double)k.rate)) : (double)(1LL << 50);
    }
}

// per CU: the first candidate with the strictly smallest rdcost
__global__ void skip_best_kernel(const xavs2gpu_skip_cand_t *__restrict__ cands, int n, const double *__restrict__ cost,
                                 int n_cus, int32_t *__restrict__ best)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cu = cands[i].cu;
    if (cu < 0 || cu >= n_cus || (i > 0 && cands[i - 1].cu == cu)) return;
    int b = -1;
    double m = (double)(1LL << 50);
    for (int j = i; j < n && cands[j].cu == cu; j++)
        if (cost[j] < m) {
            m = cost[j];
            b = j;
        }
    best[cu] = b;
}

}  // namespace skp
}  // namespace xg

using namespace xg;

extern "C" int xavs2gpu_skip_costs(xavs2gpu_me_session_t *s, const xavs2gpu_skip_cand_t *cands, int n, double lambda,
                                   int n_cus, int32_t *dist, double *cost, int32_t *best, void *stream)
{
    if (!s || n < 0 || n_cus < 0 || (n > 0 && (!cands || !dist || !cost)) || (n_cus > 0 && !best)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_skip_costs", "bad session, count or pointer");
        return XAVS2GPU_ERR_ARG;
    }
    int W = 0, H = 0, nrefs = 0, npus = 0;
    xavs2gpu_me_session_info(s, &W, &H, &nrefs, &npus);
    const cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)xavs2gpu_me_stream(s);
    if (n_cus > 0) XG_CUDA(cudaMemsetAsync(best, 0xFF, sizeof(int32_t) * (size_t)n_cus, st));
    if (n == 0) return XAVS2GPU_OK;
    skp::Ctx c{xavs2gpu_me_plane_device(s, -1, 0), xavs2gpu_me_plane_table_device(s), xavs2gpu_me_plane_stride(s), W, H,
               nrefs, cands, n, lambda, dist, cost};
    // scratch: size counts and cursors, then the size-ordered list
    int *scratch = nullptr;
    XG_CUDA(cudaMallocAsync((void **)&scratch, sizeof(int) * (16 + (size_t)n), st));
    if (!scratch) return XAVS2GPU_ERR_CUDA;
    int *counts = scratch, *cursor = scratch + 8, *sorted = scratch + 16;
    XG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int) * 16, st));
    const int nb = (n + 255) / 256;
    skp::skip_count_kernel<<<nb, 256, 0, st>>>(c, counts);
    skp::skip_scatter_kernel<<<nb, 256, 0, st>>>(c, counts, cursor, sorted);
    // warps: at most one per candidate (sizes with fewer lanes share warps)
    skp::skip_cost_kernel<<<(unsigned)(((long long)n * 32 + 127) / 128), 128, 0, st>>>(c, counts, sorted);
    count_launch(3);
    XG_CUDA(cudaFreeAsync(scratch, st));
    if (n_cus > 0) {
        skp::skip_best_kernel<<<(n + 127) / 128, 128, 0, st>>>(cands, n, cost, n_cus, best);
        count_launch();
    }
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
