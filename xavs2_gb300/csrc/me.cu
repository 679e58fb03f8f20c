// me.cu -- batched full-search + sub-pel motion estimation for sm_103a.
//
// Per PU and reference the result equals the reference's xavs2_me_search
// (source/encoder/me.c:879-1183) in full-search mode with me_subpel_refine
// (me.c:479-579):
//   1. candidates {clip(IPEL(mvp)), clip(0,0)} (md_inter.c:840-865), first
//      strictly smaller cost wins; the best one is the search centre;
//   2. SAD + lambda*mvbits over the (2R)^2 window around the centre, raster
//      order j (rows) outer, i inner, first strictly smaller cost wins;
//   3. half-pel then quarter-pel refinement on the frame sub-pel planes with
//      SATD (or SAD) + lambda*mvbits.
// "First strictly smaller in visit order" is evaluated as the minimum of the
// 64-bit key (cost << 32 | visit order), which lets any number of threads
// search parts of a window in any order and merge with atomicMin.
//
// Kernels: me_init_kernel (candidates), fs_ctu_kernel (shared-window search
// of all PUs of a 64x64 CTU; fs_ctu.cuh), fs_generic_kernel (one PU per CTA)
// and refine_kernel.
#include "xavs2gpu_common.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

namespace xg {

constexpr int kPad = 80;                 // plane margin, as XAVS2_PAD (defines.h:298)
constexpr unsigned long long kNoKey = ~0ull;

struct PuState {
    int16_t cand[2][2];
    int16_t ncand;
    int16_t valid;     // 1 when a candidate was inside the limits
    int16_t cx, cy;    // search centre (best candidate)
};

struct Geometry {
    int W, H, stride;
};

// What the kernels read of one motion-search session.  A launch may cover
// several sessions (pictures of different sizes): work-list entries carry
// the session's index in their top 8 bits and the PU index below.
struct SessView {
    const uint8_t *cur;             // current picture, pixel (0,0)
    const uint8_t *const *ref0;     // [nrefs] full-pel reference planes
    const uint8_t *const *planes;   // [nrefs * 16] sub-pel planes (16 r + k)
    const xavs2gpu_pu_t *pus;
    PuState *state;
    unsigned long long *keys;
    xavs2gpu_me_result_t *res;
    const int32_t *slots;           // CTU slot map
    Geometry g;
    int n;                          // PUs
    // plane pool (every plane of the session, plane_bytes apart) and a
    // tensor map over it (3-D: column, row, plane), or null
    const void *tmap;
    const uint8_t *pool;
    size_t plane_bytes;
    unsigned *wait_flag;            // set by a kernel that gave up a bounded wait
};
constexpr int kSessShift = 24;
constexpr uint32_t kIdxMask = (1u << kSessShift) - 1;

__device__ __forceinline__ int sad_block_lane(const uint8_t *a, int sa, const uint8_t *b, int sb, int w, int h, int lane)
{
    int s = 0;
    for (int i = lane; i < w * h; i += 32) {
        int y = i / w, x = i - y * w;
        s += iabs_d((int)a[y * sa + x] - (int)b[y * sb + x]);
    }
    return s;
}

__device__ __forceinline__ int warp_sum_i(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ bool in_box(const xavs2gpu_pu_t &p, int mx, int my)
{
    return mx >= p.min_x && mx <= p.max_x && my >= p.min_y && my <= p.max_y;
}

// ---- 1. candidates ----------------------------------------------------------------
// One warp per PU.  keys[i] starts as the best candidate's (cost, order 0/1).
__device__ __forceinline__ void init_one(int i, int lane, const xavs2gpu_pu_t *__restrict__ pus,
                                         const uint8_t *__restrict__ cur, const uint8_t *const *refs,
                                         const Geometry &g, int lambda, PuState *__restrict__ state,
                                         unsigned long long *__restrict__ keys)
{
    const xavs2gpu_pu_t p = pus[i];
    const int w = c_pu_w[p.part], h = c_pu_h[p.part];
    const uint8_t *ref = refs[p.ref];
    PuState st;
    st.ncand = 0;
    const int xs[2] = {(p.mvp_x + 2) >> 2, 0}, ys[2] = {(p.mvp_y + 2) >> 2, 0};
    for (int c = 0; c < 2; c++) {
        int x = min(max(xs[c], (int)p.min_x), (int)p.max_x);
        int y = min(max(ys[c], (int)p.min_y), (int)p.max_y);
        if (st.ncand == 1 && st.cand[0][0] == x && st.cand[0][1] == y) continue;
        st.cand[st.ncand][0] = (int16_t)x;
        st.cand[st.ncand][1] = (int16_t)y;
        st.ncand++;
    }
    unsigned long long best = kNoKey;
    const uint8_t *o = cur + (ptrdiff_t)p.y * g.stride + p.x;
    for (int c = 0; c < st.ncand; c++) {
        int mx = st.cand[c][0], my = st.cand[c][1];
        if (!in_box(p, mx, my)) continue;
        const uint8_t *r = ref + (ptrdiff_t)(p.y + my) * g.stride + p.x + mx;
        int cost = warp_sum_i(sad_block_lane(o, g.stride, r, g.stride, w, h, lane)) +
                   mv_cost_hd(lambda, mx * 4, my * 4, p.mvp_x, p.mvp_y);
        unsigned long long k = ((unsigned long long)(unsigned)cost << 32) | (unsigned)c;
        if (k < best) best = k;
    }
    st.valid = best != kNoKey;
    int bc = st.valid ? (int)(best & 0xffffffffu) : 0;
    st.cx = st.valid ? st.cand[bc][0] : 0;
    st.cy = st.valid ? st.cand[bc][1] : 0;
    if (lane == 0) {
        state[i] = st;
        keys[i] = best;
    }
}

__global__ void __launch_bounds__(128) me_init_kernel(const xavs2gpu_pu_t *__restrict__ pus, int n,
                                                      const uint8_t *__restrict__ cur, const uint8_t *const *refs,
                                                      Geometry g, int lambda, PuState *__restrict__ state,
                                                      unsigned long long *__restrict__ keys)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    init_one(i, lane, pus, cur, refs, g, lambda, state, keys);
}

// Same over a session-tagged list (the PUs outside the CTU plan).
__global__ void __launch_bounds__(128) me_init_list_kernel(const uint32_t *__restrict__ list, int n,
                                                           const SessView *__restrict__ views, int lambda)
{
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= n) return;
    const uint32_t e = list[t];
    const SessView &v = views[e >> kSessShift];
    init_one((int)(e & kIdxMask), lane, v.pus, v.cur, v.ref0, v.g, lambda, v.state, v.keys);
}

// keys := no key, for every PU of every session of the launch
__global__ void reset_keys_kernel(const SessView *__restrict__ views, int nviews)
{
    for (int s = 0; s < nviews; s++) {
        const SessView &v = views[s];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.n; i += gridDim.x * blockDim.x) v.keys[i] = kNoKey;
    }
}

// ---- 2b. per-PU full search (one CTA per PU) --------------------------------------
// For PUs outside the CTU plan (their own search centre and predictor).  The
// CTA stages the PU's block and its (2R + w - 1) x (2R + h - 1) reference
// window in shared memory (a warp per window row, aligned word loads and a
// funnel shift when the window lies inside the padded plane); a thread takes
// groups of 4 horizontally adjacent displacements: per block row and 4-pixel
// word it reads the block word (the same for the whole warp) and one new
// window word, aligns the window at the 4 byte offsets with byte permutes and
// accumulates 4 SADs with vabsdiff4.  A thread owns one column group and
// kPuRows consecutive displacement rows at a time: each window word it loads
// and aligns serves the block rows of all kPuRows displacement rows, so the
// loads and permutes are shared by kPuRows x 4 displacements.  Only the rows
// and column groups inside the PU's limits are visited.  lambda x MV bits per
// column / row of the window come from shared tables (me.c:614-641): the
// cost of (i, j) is SAD + (lx[i] + ly[j]) >> 16.  Visit order of window
// position (i, j) is 2 + (j+R)*2R + (i+R); a thread's column group is fixed
// and its row blocks ascend, so it visits its positions in increasing order
// and a strictly smaller 32-bit cost keeps the first minimum; the CTA's
// (cost, order) keys are reduced and merged with atomicMin.
constexpr int kPuThreads = 256;
#ifndef XG_PU_ROWS
#define XG_PU_ROWS 4
#endif
constexpr int kPuRows = XG_PU_ROWS;   // displacement rows per thread and pass

// dynamic shared memory the per-PU search needs for range R
__host__ __device__ __forceinline__ int fs_pu_smem(int R)
{
    const int pitch = ((2 * R + 64 + 8 + 15) / 16) * 16;          // window bytes per row (max block 64)
    return 64 * 64 + 2 * (2 * R) * 8 + (2 * R + 64 + kPuRows) * pitch + 8 * 8;
}

// lambda x bits with lambda < 2^24 and bits < 128 fits 31 bits; larger
// lambdas take 64-bit table entries
template <bool WIDE> struct LamT { using T = int; };
template <> struct LamT<true> { using T = long long; };

template <bool WIDE>
__device__ __forceinline__ void fs_pu_search(const xavs2gpu_pu_t &p, const PuState &st, const SessView &v, int R,
                                             int lambda, uint8_t *smem_pu, unsigned long long *__restrict__ keys,
                                             int i)
{
    using L = typename LamT<WIDE>::T;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t *s_cur = reinterpret_cast<uint32_t *>(smem_pu);                 // [h][w/4] words
    L *s_lx = reinterpret_cast<L *>(smem_pu + 64 * 64);                      // [2R] lambda x MV bits per column
    L *s_ly = s_lx + 2 * R;                                                  // [2R] per row
    uint8_t *s_win = smem_pu + 64 * 64 + 2 * (2 * R) * 8;                    // [2R + h - 1][pitch]
    const int pitch = ((2 * R + 64 + 8 + 15) / 16) * 16;
    unsigned long long *s_red = reinterpret_cast<unsigned long long *>(s_win + (2 * R + 64 + kPuRows) * pitch);
    const Geometry g = v.g;
    const int w = c_pu_w[p.part], h = c_pu_h[p.part], wq = w >> 2;
    const int wx0 = p.x + st.cx - R, wy0 = p.y + st.cy - R;   // window origin (displacement -R, -R)
    // bytes read per row: the last group of 4 displacements starts at most
    // at 2R - 2 (odd R) and its words reach 6 bytes past the block width
    // rows: the last row block of kPuRows may reach kPuRows - 1 rows past the
    // window (their sums are dropped)
    const int wcols = 2 * R + w + 6, wrows = 2 * R + h - 1 + kPuRows - 1, nwords = (wcols + 3) >> 2;
    const uint8_t *ref = v.ref0[p.ref];
    // block words
    const uint8_t *o = v.cur + (ptrdiff_t)p.y * g.stride + p.x;
    const bool oal = (((uintptr_t)o | (uintptr_t)g.stride) & 3) == 0;
    for (int k = tid; k < h * wq; k += kPuThreads) {
        const int y = k / wq, c = k - y * wq;
        const uint8_t *q = o + (ptrdiff_t)y * g.stride + 4 * c;
        s_cur[k] = oal ? *reinterpret_cast<const uint32_t *>(q)
                       : (uint32_t)q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16 | (uint32_t)q[3] << 24;
    }
    // lambda x MV bits of the window's columns and rows (me.c:614-641)
    for (int k = tid; k < 2 * R; k += kPuThreads) {
        s_lx[k] = (L)lambda * mvbits_hd(4 * (st.cx + k - R) - p.mvp_x);
        s_ly[k] = (L)lambda * mvbits_hd(4 * (st.cy + k - R) - p.mvp_y);
    }
    // window bytes: inside the padded plane a warp copies a row as aligned
    // words (the 4 bytes past the row's last word included); elsewhere bytes
    // clamped into the padded plane (clamped bytes only feed displacements
    // outside the limits)
    if (wx0 >= -kPad && wx0 + 4 * nwords + 4 <= g.W + kPad && wy0 >= -kPad) {
        for (int r = warp; r < wrows; r += kPuThreads / 32) {
            const int y = min(wy0 + r, g.H + kPad - 1);
            const uintptr_t a = (uintptr_t)(ref + (ptrdiff_t)y * g.stride + wx0);
            const uint32_t *aw = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
            const int sh = 8 * (int)(a & 3);
            uint32_t *dst = reinterpret_cast<uint32_t *>(s_win + r * pitch);
            for (int c = lane; c < nwords; c += 32) dst[c] = __funnelshift_r(__ldg(aw + c), __ldg(aw + c + 1), sh);
        }
    } else {
        for (int r = warp; r < wrows; r += kPuThreads / 32) {
            const int y = min(max(wy0 + r, -kPad), g.H + kPad - 1);
            const uint8_t *row = ref + (ptrdiff_t)y * g.stride;
            for (int c = lane; c < wcols; c += 32)
                s_win[r * pitch + c] = row[min(max(wx0 + c, -kPad), g.W + kPad - 1)];
        }
    }
    __syncthreads();
    // window positions inside the limits
    const int ilo = max(0, p.min_x - (st.cx - R)), ihi = min(2 * R - 1, p.max_x - (st.cx - R));
    const int jlo = max(0, p.min_y - (st.cy - R)), jhi = min(2 * R - 1, p.max_y - (st.cy - R));
    uint32_t bestc = 0xffffffffu, besto = 0;
    const int g0 = ilo >> 2, ng = (ihi >> 2) - g0 + 1;
    const int tpg = ng > 0 ? kPuThreads / ng : 0;           // threads per column group
    if (ilo <= ihi && jlo <= jhi && tid < tpg * ng) {
        const int gx = g0 + tid % ng, trow = tid / ng;
        L lx[4];
#pragma unroll
        for (int t = 0; t < 4; t++) lx[t] = s_lx[min(4 * gx + t, 2 * R - 1)];
        for (int jr0 = jlo + kPuRows * trow; jr0 <= jhi; jr0 += kPuRows * tpg) {
            uint32_t acc[kPuRows][4];
#pragma unroll
            for (int i = 0; i < kPuRows; i++)
#pragma unroll
                for (int t = 0; t < 4; t++) acc[i][t] = 0;
            for (int r = 0; r < h + kPuRows - 1; r++) {
                // window row jr0 + r meets block row y = r - i of displacement row jr0 + i
                bool live[kPuRows];
#pragma unroll
                for (int i = 0; i < kPuRows; i++) live[i] = r - i >= 0 && r - i < h;
                const uint32_t *wr = reinterpret_cast<const uint32_t *>(s_win + (jr0 + r) * pitch) + gx;
                const uint32_t *cr = s_cur + r * wq;
                uint32_t lo = wr[0];
                for (int c = 0; c < wq; c++) {
                    const uint32_t hi = wr[c + 1];
                    const uint32_t b1 = __byte_perm(lo, hi, 0x4321), b2 = __byte_perm(lo, hi, 0x5432),
                                   b3 = __byte_perm(lo, hi, 0x6543);
#pragma unroll
                    for (int i = 0; i < kPuRows; i++) {
                        if (!live[i]) continue;
                        const uint32_t cw = cr[c - i * wq];
                        acc[i][0] = sad4_acc(cw, lo, acc[i][0]);
                        acc[i][1] = sad4_acc(cw, b1, acc[i][1]);
                        acc[i][2] = sad4_acc(cw, b2, acc[i][2]);
                        acc[i][3] = sad4_acc(cw, b3, acc[i][3]);
                    }
                    lo = hi;
                }
            }
#pragma unroll
            for (int i = 0; i < kPuRows; i++) {
                const int jr = jr0 + i;
                if (jr > jhi) break;
                const L ly = s_ly[jr];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int ir = 4 * gx + t;
                    const uint32_t cost = acc[i][t] + (uint32_t)((lx[t] + ly) >> 16);
                    if (ir >= ilo && ir <= ihi && cost < bestc) {
                        bestc = cost;
                        besto = (uint32_t)(jr * 2 * R + ir);
                    }
                }
            }
        }
    }
    unsigned long long best = bestc == 0xffffffffu ? kNoKey : ((unsigned long long)bestc << 32) | (2u + besto);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, off);
        best = other < best ? other : best;
    }
    if (lane == 0) s_red[warp] = best;
    __syncthreads();
    if (tid == 0) {
        for (int k = 1; k < kPuThreads / 32; k++) best = s_red[k] < best ? s_red[k] : best;
        if (best != kNoKey) atomicMin(&keys[i], best);
    }
}

template <bool WIDE>
__global__ void __launch_bounds__(kPuThreads) fs_generic_kernel(const uint32_t *__restrict__ list, int n,
                                                                const SessView *__restrict__ views, int R, int lambda)
{
    extern __shared__ __align__(16) uint8_t smem_pu[];
    for (int li = blockIdx.x; li < n; li += gridDim.x) {
        const uint32_t e = list[li];
        const SessView &v = views[e >> kSessShift];
        const int i = (int)(e & kIdxMask);
        const PuState st = v.state[i];
        if (!st.valid) continue;       // uniform over the CTA
        __syncthreads();               // the previous PU's readers are done
        fs_pu_search<WIDE>(v.pus[i], st, v, R, lambda, smem_pu, v.keys, i);
    }
}

// Launch of the per-PU search with the dynamic shared memory of range R (the
// attribute is raised once per device and size).
static int fs_generic_launch(const uint32_t *list, int n, const SessView *views, int R, int lambda, cudaStream_t st)
{
    static int attr_bytes[64] = {0};
    const int dev = current_device();
    const int bytes = fs_pu_smem(R);
    if (dev < 0 || dev >= 64) return XAVS2GPU_ERR_ARG;
    if (attr_bytes[dev] < bytes) {
        XG_CUDA(cudaFuncSetAttribute(fs_generic_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        XG_CUDA(cudaFuncSetAttribute(fs_generic_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        attr_bytes[dev] = bytes;
    }
    const int cap = sm_count() * 8, grid = n < cap ? n : cap;
    if (lambda < (1 << 24))
        fs_generic_kernel<false><<<grid, kPuThreads, bytes, st>>>(list, n, views, R, lambda);
    else
        fs_generic_kernel<true><<<grid, kPuThreads, bytes, st>>>(list, n, views, R, lambda);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

// ---- 3. sub-pel refinement ------------------------------------------------------------
// One warp per PU: the candidate costs of one refinement step are evaluated in
// parallel, then the first strictly smaller one (spiral order, centre first)
// is taken, as the reference's sequential loop does.
__constant__ int8_t c_spiral[2][9][2] = {
    {{0, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {1, 1}},
    {{0, 0}, {0, -1}, {-1, -1}, {-1, 0}, {-1, 1}, {0, 1}, {1, 1}, {1, 0}, {1, -1}}};

// cost (SATD or SAD) of the PU against plane[(my&3)*4 + (mx&3)] at quarter-pel (mx, my)
__device__ int qpel_cost_warp(const xavs2gpu_pu_t &p, int w, int h, bool hadamard, const uint8_t *o,
                              const uint8_t *const *planes, const Geometry &g, int mx, int my, int lane)
{
    const uint8_t *r = planes[((my & 3) << 2) + (mx & 3)] + (ptrdiff_t)(p.y + (my >> 2)) * g.stride + p.x + (mx >> 2);
    int s = 0;
    if (!hadamard) {
        s = sad_block_lane(o, g.stride, r, g.stride, w, h, lane);
    } else {
        const bool u4 = satd_unit4(w, h);
        const int uw = u4 ? 4 : 8, nux = w / uw, nu = nux * (h >> 2);
        for (int u = lane; u < nu; u += 32) {
            int uy = u / nux, ux = u - uy * nux;
            s += satd_unit_d(u4, o + (ptrdiff_t)uy * 4 * g.stride + ux * uw, g.stride,
                             r + (ptrdiff_t)uy * 4 * g.stride + ux * uw, g.stride);
        }
    }
    return warp_sum_i(s);
}

__global__ void __launch_bounds__(128) refine_kernel(const xavs2gpu_pu_t *__restrict__ pus, int n,
                                                     const PuState *__restrict__ state,
                                                     const unsigned long long *__restrict__ keys,
                                                     const uint8_t *__restrict__ cur,
                                                     const uint8_t *const *ref_planes,   // [ref*16 + k]
                                                     Geometry g, int R, xavs2gpu_me_params_t prm,
                                                     xavs2gpu_me_result_t *__restrict__ out)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    const xavs2gpu_pu_t p = pus[i];
    const PuState st = state[i];
    const unsigned long long key = keys[i];
    xavs2gpu_me_result_t res;
    if (!st.valid || key == kNoKey) {
        res.bmv_x = res.bmv_y = res.imv_x = res.imv_y = 0;
        res.bcost = res.icost = 1 << 30;
        res.mvcost = 0;
        if (lane == 0) out[i] = res;
        return;
    }
    const int icost = (int)(key >> 32);
    const unsigned order = (unsigned)(key & 0xffffffffu);
    int bmx, bmy;
    if (order < 2) {
        bmx = st.cand[order][0];
        bmy = st.cand[order][1];
    } else {
        const int q = (int)order - 2;
        bmx = st.cx + q % (2 * R) - R;
        bmy = st.cy + q / (2 * R) - R;
    }
    const int lam = prm.lambda_factor, pmx = p.mvp_x, pmy = p.mvp_y;
    res.imv_x = (int16_t)bmx;
    res.imv_y = (int16_t)bmy;
    res.icost = icost;
    int bx = bmx * 4, by = bmy * 4, best = icost;
    if (prm.fractional_me) {
        const int w = c_pu_w[p.part], h = c_pu_h[p.part];
        const bool had = prm.use_hadamard != 0;
        const uint8_t *o = cur + (ptrdiff_t)p.y * g.stride + p.x;
        const uint8_t *const *planes = ref_planes + 16 * p.ref;
        const int pat = prm.fast_sub_me ? 1 : 0, step = prm.fast_sub_me ? 2 : 1;
        int cx = bx, cy = by;
        if (had) best = qpel_cost_warp(p, w, h, true, o, planes, g, cx, cy, lane) + mv_cost_hd(lam, cx, cy, pmx, pmy);
        for (int pos = 1; pos < 9; pos += step) {
            int mx = cx + 2 * c_spiral[pat][pos][0], my = cy + 2 * c_spiral[pat][pos][1];
            int c = qpel_cost_warp(p, w, h, had, o, planes, g, mx, my, lane) + mv_cost_hd(lam, mx, my, pmx, pmy);
            if (c < best) { best = c; bx = mx; by = my; }
        }
        if (prm.fractional_me > 1) {
            cx = bx; cy = by;
            const int ctr_x = (pmx >> 1) << 1, ctr_y = (pmy >> 1) << 1;
            for (int pos = 1; pos < 9; pos += step) {
                int sx = c_spiral[pat][pos][0], sy = c_spiral[pat][pos][1], mx, my;
                if (prm.enable_pmvr) {
                    // pmvr_adapt_mv (me.c:412-424), TH_PMVR = 2
                    if (abs(cx - ctr_x) > 2 || abs(cy - ctr_y) > 2) {
                        mx = cx + 2 * sx; my = cy + 2 * sy;
                        if (abs(mx - ctr_x) <= 2 && abs(my - ctr_y) <= 2) continue;
                    } else {
                        mx = cx + sx; my = cy + sy;
                        if (abs(mx - ctr_x) > 2 || abs(my - ctr_y) > 2) continue;
                    }
                } else {
                    mx = cx + sx; my = cy + sy;
                }
                int c = qpel_cost_warp(p, w, h, had, o, planes, g, mx, my, lane) + mv_cost_hd(lam, mx, my, pmx, pmy);
                if (c < best) { best = c; bx = mx; by = my; }
            }
        }
    }
    res.bmv_x = (int16_t)bx;
    res.bmv_y = (int16_t)by;
    res.bcost = best;
    res.mvcost = mv_cost_hd(lam, bx, by, pmx, pmy);
    if (lane == 0) out[i] = res;
}

// ---- refinement v3: one thread per search (PUs up to 256 pixels) ---------------
// The thread runs the reference's sequential loop itself: the positions of a
// step are fixed by the centre, so their costs are accumulated unit by unit
// (the current block's unit is loaded once and compared with every
// position), then the first strictly smaller cost wins in spiral order.
// The refinement's unit costs (SATD with one rounding per 4x4 or 8x4 unit,
// pixel.c:321, 347, or SAD) on packed 16-bit pairs: a pair holds column k of
// the unit's left 4x4 block and column k of its right one (zero for a 4x4
// unit), so each vadd2 / vsub2 takes one butterfly of both blocks.  The
// differences (|d| <= 255) grow to at most 16 x 255 = 4080 through the two
// 4-point passes, well inside 16 bits, so every value equals the 32-bit
// form's; the absolute values are summed by dp2a.  Build option
// XG_REFINE_PACKED=0 keeps the 32-bit form.
#ifndef XG_REFINE_PACKED
#define XG_REFINE_PACKED 1
#endif

// 8 bytes of a row at any alignment as two words (aligned loads; the words
// after the row are read too: every plane has an 80-pixel margin and the
// planes' allocation 256 bytes of slack, so they are in bounds)
__device__ __forceinline__ void load8u(const uint8_t *p, uint32_t &lo, uint32_t &hi)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    const uint32_t w0 = w[0], w1 = w[1], w2 = w[2];
    lo = __funnelshift_r(w0, w1, sh);
    hi = __funnelshift_r(w1, w2, sh);
}

// (byte k, byte 4 + k) of the 8-byte row (lo, hi) as zero-extended halves
__device__ __forceinline__ void row_pairs(uint32_t lo, uint32_t hi, uint32_t (&q)[4])
{
    const uint32_t t = __byte_perm(lo, hi, 0x5140), u = __byte_perm(lo, hi, 0x7362);   // b0 b4 b1 b5 | b2 b6 b3 b7
    q[0] = __byte_perm(t, 0, 0x7170);
    q[1] = __byte_perm(t, 0, 0x7372);
    q[2] = __byte_perm(u, 0, 0x7170);
    q[3] = __byte_perm(u, 0, 0x7372);
}

// The current block's unit: raw row words (SAD) and column pairs (SATD).
struct UnitCur {
    uint32_t w[4][2];
    uint32_t q[4][4];
};

template <bool U4>
__device__ __forceinline__ void load_unit(const uint8_t *o, int stride, UnitCur &c)
{
#pragma unroll
    for (int y = 0; y < 4; y++) {
        uint32_t lo, hi;
        load8u(o + y * stride, lo, hi);
        c.w[y][0] = lo;
        c.w[y][1] = U4 ? 0u : hi;
        row_pairs(lo, c.w[y][1], c.q[y]);
    }
}

// |x| summed over the two halves of v, plus acc
__device__ __forceinline__ int abs_pair_acc(uint32_t v, int acc)
{
    return __dp2a_lo((int)__vabsss2(v), 0x0101, acc);
}

template <bool U4>
__device__ __forceinline__ int unit_cost_pre(bool had, const UnitCur &c, const uint8_t *r, int stride)
{
    if (!had) {
        uint32_t s = 0;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            uint32_t lo, hi;
            load8u(r + y * stride, lo, hi);
            s = sad4_acc(c.w[y][0], lo, s);
            if (!U4) s = sad4_acc(c.w[y][1], hi, s);
        }
        return (int)s;
    }
    uint32_t d[4][4];
#pragma unroll
    for (int y = 0; y < 4; y++) {
        uint32_t lo, hi, q[4];
        load8u(r + y * stride, lo, hi);
        row_pairs(lo, U4 ? 0u : hi, q);
        // differences, then the 4-point transform of the row in both blocks
        const uint32_t d0 = __vsub2(c.q[y][0], q[0]), d1 = __vsub2(c.q[y][1], q[1]);
        const uint32_t d2 = __vsub2(c.q[y][2], q[2]), d3 = __vsub2(c.q[y][3], q[3]);
        const uint32_t s0 = __vadd2(d0, d1), e0 = __vsub2(d0, d1), s1 = __vadd2(d2, d3), e1 = __vsub2(d2, d3);
        d[y][0] = __vadd2(s0, s1);
        d[y][1] = __vadd2(e0, e1);
        d[y][2] = __vsub2(s0, s1);
        d[y][3] = __vsub2(e0, e1);
    }
    int s = 0;
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const uint32_t s0 = __vadd2(d[0][x], d[1][x]), e0 = __vsub2(d[0][x], d[1][x]);
        const uint32_t s1 = __vadd2(d[2][x], d[3][x]), e1 = __vsub2(d[2][x], d[3][x]);
        s = abs_pair_acc(__vadd2(s0, s1), s);
        s = abs_pair_acc(__vadd2(e0, e1), s);
        s = abs_pair_acc(__vsub2(s0, s1), s);
        s = abs_pair_acc(__vsub2(e0, e1), s);
    }
    return s >> 1;
}

#if XG_REFINE_PACKED
using UnitC = UnitCur;
#else
using UnitC = int[4][8];
#endif

#if !XG_REFINE_PACKED
// Bytes p[0..n) (n = 4 or 8) of an arbitrarily aligned row as ints, from
// aligned 32-bit loads (the word after the row is read too; every plane has
// an 80-pixel margin, so it is in bounds).
template <int N>
__device__ __forceinline__ void load_row(const uint8_t *p, int (&v)[8])
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
    const uint32_t w0 = w[0], w1 = w[1];
    const uint32_t lo = __funnelshift_r(w0, w1, sh);
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = (int)__byte_perm(lo, 0, 0x4440 + k);
    if (N == 8) {
        const uint32_t hi = __funnelshift_r(w1, w[2], sh);
#pragma unroll
        for (int k = 0; k < 4; k++) v[4 + k] = (int)__byte_perm(hi, 0, 0x4440 + k);
    }
}

// SATD (one rounding per unit, pixel.c:321, 347) or SAD of one 4x4 (U4) or
// 8x4 unit; `c` holds the current block's unit.
template <bool U4>
__device__ __forceinline__ int unit_cost_pre(bool had, const int (&c)[4][8], const uint8_t *r, int stride)
{
    constexpr int UW = U4 ? 4 : 8;
    int d[4][8];
#pragma unroll
    for (int y = 0; y < 4; y++) {
        int v[8];
        load_row<UW>(r + y * stride, v);
#pragma unroll
        for (int x = 0; x < UW; x++) d[y][x] = c[y][x] - v[x];
    }
    int s = 0;
    if (!had) {
#pragma unroll
        for (int y = 0; y < 4; y++)
#pragma unroll
            for (int x = 0; x < UW; x++) s += iabs_d(d[y][x]);
        return s;
    }
#pragma unroll
    for (int y = 0; y < 4; y++) {
        fwht4_d(d[y][0], d[y][1], d[y][2], d[y][3]);
        if (!U4) fwht4_d(d[y][4], d[y][5], d[y][6], d[y][7]);
    }
#pragma unroll
    for (int x = 0; x < UW; x++) {
        int a = d[0][x], b = d[1][x], e = d[2][x], f = d[3][x];
        fwht4_d(a, b, e, f);
        s += iabs_d(a) + iabs_d(b) + iabs_d(e) + iabs_d(f);
    }
    return s >> 1;
}

template <bool U4>
__device__ __forceinline__ void load_unit(const uint8_t *o, int stride, int (&c)[4][8])
{
#pragma unroll
    for (int y = 0; y < 4; y++) {
        int v[8];
        load_row<U4 ? 4 : 8>(o + y * stride, v);
#pragma unroll
        for (int x = 0; x < 8; x++) c[y][x] = v[x];
    }
}

#endif

#if XG_REFINE_PACKED
// The unit loads and costs with the unit width a run-time flag (one copy of
// the code for 4x4 and 8x4 units: the per-thread refinement is bound by its
// instruction cache).
__device__ __forceinline__ void load_unit_rt(const uint8_t *o, int stride, UnitCur &c, bool u4)
{
#pragma unroll
    for (int y = 0; y < 4; y++) {
        uint32_t lo, hi;
        load8u(o + y * stride, lo, hi);
        c.w[y][0] = lo;
        c.w[y][1] = u4 ? 0u : hi;
        row_pairs(lo, c.w[y][1], c.q[y]);
    }
}

__device__ __forceinline__ int unit_cost_pre_rt(bool had, bool u4, const UnitCur &c, const uint8_t *r, int stride)
{
    if (!had) {
        uint32_t s = 0;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            uint32_t lo, hi;
            load8u(r + y * stride, lo, hi);
            s = sad4_acc(c.w[y][0], lo, s);
            s = sad4_acc(c.w[y][1], u4 ? 0u : hi, s);
        }
        return (int)s;
    }
    uint32_t d[4][4];
#pragma unroll
    for (int y = 0; y < 4; y++) {
        uint32_t lo, hi, q[4];
        load8u(r + y * stride, lo, hi);
        row_pairs(lo, u4 ? 0u : hi, q);
        const uint32_t d0 = __vsub2(c.q[y][0], q[0]), d1 = __vsub2(c.q[y][1], q[1]);
        const uint32_t d2 = __vsub2(c.q[y][2], q[2]), d3 = __vsub2(c.q[y][3], q[3]);
        const uint32_t s0 = __vadd2(d0, d1), e0 = __vsub2(d0, d1), s1 = __vadd2(d2, d3), e1 = __vsub2(d2, d3);
        d[y][0] = __vadd2(s0, s1);
        d[y][1] = __vadd2(e0, e1);
        d[y][2] = __vsub2(s0, s1);
        d[y][3] = __vsub2(e0, e1);
    }
    int s = 0;
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const uint32_t s0 = __vadd2(d[0][x], d[1][x]), e0 = __vsub2(d[0][x], d[1][x]);
        const uint32_t s1 = __vadd2(d[2][x], d[3][x]), e1 = __vsub2(d[2][x], d[3][x]);
        s = abs_pair_acc(__vadd2(s0, s1), s);
        s = abs_pair_acc(__vadd2(e0, e1), s);
        s = abs_pair_acc(__vsub2(s0, s1), s);
        s = abs_pair_acc(__vsub2(e0, e1), s);
    }
    return s >> 1;
}
#endif

// Accumulates the costs of up to 9 positions over all units of the PU.
__device__ __forceinline__ void refine_stage_thread(bool had, bool u4, int nux, int nu, const uint8_t *o,
                                                    const uint8_t *const *planes, int stride, int px, int py,
                                                    const int (&mxs)[9], const int (&mys)[9], int npos,
                                                    int (&acc)[9])
{
    const int uw = u4 ? 4 : 8;
#pragma unroll
    for (int k = 0; k < 9; k++) acc[k] = 0;
    for (int u = 0; u < nu; u++) {
        const int uy = u / nux, ux = u - uy * nux;
        UnitC c;
        const uint8_t *ou = o + (ptrdiff_t)uy * 4 * stride + ux * uw;
#if XG_REFINE_PACKED
        load_unit_rt(ou, stride, c, u4);
#else
        if (u4) load_unit<true>(ou, stride, c);
        else load_unit<false>(ou, stride, c);
#endif
#pragma unroll
        for (int k = 0; k < 9; k++) {
            if (k < npos) {
                const int mx = mxs[k], my = mys[k];
                const uint8_t *r = planes[((my & 3) << 2) + (mx & 3)] +
                                   (ptrdiff_t)(py + uy * 4 + (my >> 2)) * stride + px + ux * uw + (mx >> 2);
#if XG_REFINE_PACKED
                acc[k] += unit_cost_pre_rt(had, u4, c, r, stride);
#else
                acc[k] += u4 ? unit_cost_pre<true>(had, c, r, stride) : unit_cost_pre<false>(had, c, r, stride);
#endif
            }
        }
    }
}

// resident CTAs per SM the register budget of the per-thread refinement is
// sized for (4: 128 registers, measured slightly faster than the
// compiler's 168-register choice)
#ifndef XG_REFINE_MINB
#define XG_REFINE_MINB 4
#endif

// HAD: SATD (1) or SAD (0) unit costs, fixed per launch so that each
// instance holds the code of one (the kernel waits on its instruction cache
// otherwise)
template <bool HAD>
__global__ void __launch_bounds__(128, XG_REFINE_MINB) refine_thread_kernel(const uint32_t *__restrict__ list, int n,
                                                            const SessView *__restrict__ views, int R,
                                                            xavs2gpu_me_params_t prm)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t e = list[t];
    const SessView &v = views[e >> kSessShift];
    const int i = (int)(e & kIdxMask);
    const xavs2gpu_pu_t *__restrict__ pus = v.pus;
    const PuState *__restrict__ state = v.state;
    const unsigned long long *__restrict__ keys = v.keys;
    const uint8_t *__restrict__ cur = v.cur;
    const uint8_t *const *ref_planes = v.planes;
    const Geometry g = v.g;
    xavs2gpu_me_result_t *__restrict__ out = v.res;
    const xavs2gpu_pu_t p = pus[i];
    const PuState st = state[i];
    const unsigned long long key = keys[i];
    xavs2gpu_me_result_t res;
    if (!st.valid || key == kNoKey) {
        res.bmv_x = res.bmv_y = res.imv_x = res.imv_y = 0;
        res.bcost = res.icost = 1 << 30;
        res.mvcost = 0;
        out[i] = res;
        return;
    }
    const int icost = (int)(key >> 32);
    const unsigned order_ = (unsigned)(key & 0xffffffffu);
    int bmx, bmy;
    if (order_ < 2) { bmx = st.cand[order_][0]; bmy = st.cand[order_][1]; }
    else {
        const int q = (int)order_ - 2;
        bmx = st.cx + q % (2 * R) - R;
        bmy = st.cy + q / (2 * R) - R;
    }
    res.imv_x = (int16_t)bmx; res.imv_y = (int16_t)bmy; res.icost = icost;
    const int lam = prm.lambda_factor, pmx = p.mvp_x, pmy = p.mvp_y;
    int bx = bmx * 4, by = bmy * 4, best = icost;
    if (prm.fractional_me) {
        const int w = c_pu_w[p.part], h = c_pu_h[p.part];
        const bool had = HAD;
        const bool u4 = had ? satd_unit4(w, h) : (w == 4 || w == 12);
        const int nux = w / (u4 ? 4 : 8), nu = nux * (h >> 2);
        const uint8_t *o = cur + (ptrdiff_t)p.y * g.stride + p.x;
        const uint8_t *const *planes = ref_planes + 16 * p.ref;
        const int pat = prm.fast_sub_me ? 1 : 0, step = prm.fast_sub_me ? 2 : 1;
        const int ctr_x = (pmx >> 1) << 1, ctr_y = (pmy >> 1) << 1;
        for (int stage = 0; stage < (prm.fractional_me > 1 ? 2 : 1); stage++) {
            const int cx = bx, cy = by;
            int mxs[9], mys[9], npos = 0;
#pragma unroll
            for (int k = 0; k < 9; k++) { mxs[k] = cx; mys[k] = cy; }
            if (stage == 0 && had) npos = 1;
#pragma unroll
            for (int pos = 1; pos < 9; pos++) {
                if ((pos - 1) % step) continue;
                const int sx = c_spiral[pat][pos][0], sy = c_spiral[pat][pos][1];
                int mx, my;
                if (stage == 0) {
                    mx = cx + 2 * sx; my = cy + 2 * sy;
                } else if (prm.enable_pmvr) {
                    // pmvr_adapt_mv (me.c:412-424), TH_PMVR = 2
                    if (abs(cx - ctr_x) > 2 || abs(cy - ctr_y) > 2) {
                        mx = cx + 2 * sx; my = cy + 2 * sy;
                        if (abs(mx - ctr_x) <= 2 && abs(my - ctr_y) <= 2) continue;
                    } else {
                        mx = cx + sx; my = cy + sy;
                        if (abs(mx - ctr_x) > 2 || abs(my - ctr_y) > 2) continue;
                    }
                } else {
                    mx = cx + sx; my = cy + sy;
                }
#pragma unroll
                for (int k = 0; k < 9; k++)
                    if (k == npos) { mxs[k] = mx; mys[k] = my; }
                npos++;
            }
            int acc[9];
            refine_stage_thread(had, u4, nux, nu, o, planes, g.stride, p.x, p.y, mxs, mys, npos, acc);
            const int k0 = (stage == 0 && had) ? 1 : 0;
            if (k0) best = acc[0] + mv_cost_hd(lam, cx, cy, pmx, pmy);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                if (k < k0 || k >= npos) continue;
                const int c = acc[k] + mv_cost_hd(lam, mxs[k], mys[k], pmx, pmy);
                if (c < best) { best = c; bx = mxs[k]; by = mys[k]; }
            }
        }
    }
    res.bmv_x = (int16_t)bx; res.bmv_y = (int16_t)by;
    res.bcost = best;
    res.mvcost = mv_cost_hd(lam, bx, by, pmx, pmy);
    out[i] = res;
}

// Warp-cooperative cost of the PU at quarter-pel (mx, my): lanes take the
// PU's rounding units (4x4 or 8x4; the same tiling sums the SAD) in turn,
// rows read as aligned words.
__device__ int qpel_cost_warp_vec(const xavs2gpu_pu_t &p, int w, int h, bool had, const uint8_t *o,
                                  const uint8_t *const *planes, int stride, int mx, int my, int lane)
{
    const bool u4 = had ? satd_unit4(w, h) : (w == 4 || w == 12);
    const int uw = u4 ? 4 : 8, nux = w / uw, nu = nux * (h >> 2);
    const uint8_t *r = planes[((my & 3) << 2) + (mx & 3)] + (ptrdiff_t)(p.y + (my >> 2)) * stride + p.x + (mx >> 2);
    int s = 0;
    for (int u = lane; u < nu; u += 32) {
        const int uy = u / nux, ux = u - uy * nux;
        const ptrdiff_t off = (ptrdiff_t)uy * 4 * stride + ux * uw;
        UnitC c;
        if (u4) {
            load_unit<true>(o + off, stride, c);
            s += unit_cost_pre<true>(had, c, r + off, stride);
        } else {
            load_unit<false>(o + off, stride, c);
            s += unit_cost_pre<false>(had, c, r + off, stride);
        }
    }
    return warp_sum_i(s);
}

// One warp per search for the larger PUs, over a list.
__global__ void __launch_bounds__(128) refine_warp_list_kernel(const uint32_t *__restrict__ list, int n,
                                                               const SessView *__restrict__ views, int R,
                                                               xavs2gpu_me_params_t prm)
{
    const int wt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wt >= n) return;
    const uint32_t e = list[wt];
    const SessView &v = views[e >> kSessShift];
    const int i = (int)(e & kIdxMask);
    const xavs2gpu_pu_t *__restrict__ pus = v.pus;
    const PuState *__restrict__ state = v.state;
    const unsigned long long *__restrict__ keys = v.keys;
    const uint8_t *__restrict__ cur = v.cur;
    const uint8_t *const *ref_planes = v.planes;
    const Geometry g = v.g;
    xavs2gpu_me_result_t *__restrict__ out = v.res;
    const xavs2gpu_pu_t p = pus[i];
    const PuState st = state[i];
    const unsigned long long key = keys[i];
    xavs2gpu_me_result_t res;
    if (!st.valid || key == kNoKey) {
        res.bmv_x = res.bmv_y = res.imv_x = res.imv_y = 0;
        res.bcost = res.icost = 1 << 30;
        res.mvcost = 0;
        if (lane == 0) out[i] = res;
        return;
    }
    const int icost = (int)(key >> 32);
    const unsigned order_ = (unsigned)(key & 0xffffffffu);
    int bmx, bmy;
    if (order_ < 2) { bmx = st.cand[order_][0]; bmy = st.cand[order_][1]; }
    else {
        const int q = (int)order_ - 2;
        bmx = st.cx + q % (2 * R) - R;
        bmy = st.cy + q / (2 * R) - R;
    }
    const int lam = prm.lambda_factor, pmx = p.mvp_x, pmy = p.mvp_y;
    res.imv_x = (int16_t)bmx; res.imv_y = (int16_t)bmy; res.icost = icost;
    int bx = bmx * 4, by = bmy * 4, best = icost;
    if (prm.fractional_me) {
        const int w = c_pu_w[p.part], h = c_pu_h[p.part];
        const bool had = prm.use_hadamard != 0;
        const uint8_t *o = cur + (ptrdiff_t)p.y * g.stride + p.x;
        const uint8_t *const *planes = ref_planes + 16 * p.ref;
        const int pat = prm.fast_sub_me ? 1 : 0, step = prm.fast_sub_me ? 2 : 1;
        int cx = bx, cy = by;
        if (had) best = qpel_cost_warp_vec(p, w, h, true, o, planes, g.stride, cx, cy, lane) + mv_cost_hd(lam, cx, cy, pmx, pmy);
        for (int pos = 1; pos < 9; pos += step) {
            int mx = cx + 2 * c_spiral[pat][pos][0], my = cy + 2 * c_spiral[pat][pos][1];
            int c = qpel_cost_warp_vec(p, w, h, had, o, planes, g.stride, mx, my, lane) + mv_cost_hd(lam, mx, my, pmx, pmy);
            if (c < best) { best = c; bx = mx; by = my; }
        }
        if (prm.fractional_me > 1) {
            cx = bx; cy = by;
            const int ctr_x = (pmx >> 1) << 1, ctr_y = (pmy >> 1) << 1;
            for (int pos = 1; pos < 9; pos += step) {
                int sx = c_spiral[pat][pos][0], sy = c_spiral[pat][pos][1], mx, my;
                if (prm.enable_pmvr) {
                    if (abs(cx - ctr_x) > 2 || abs(cy - ctr_y) > 2) {
                        mx = cx + 2 * sx; my = cy + 2 * sy;
                        if (abs(mx - ctr_x) <= 2 && abs(my - ctr_y) <= 2) continue;
                    } else {
                        mx = cx + sx; my = cy + sy;
                        if (abs(mx - ctr_x) > 2 || abs(my - ctr_y) > 2) continue;
                    }
                } else {
                    mx = cx + sx; my = cy + sy;
                }
                int c = qpel_cost_warp_vec(p, w, h, had, o, planes, g.stride, mx, my, lane) + mv_cost_hd(lam, mx, my, pmx, pmy);
                if (c < best) { best = c; bx = mx; by = my; }
            }
        }
    }
    res.bmv_x = (int16_t)bx; res.bmv_y = (int16_t)by;
    res.bcost = best;
    res.mvcost = mv_cost_hd(lam, bx, by, pmx, pmy);
    if (lane == 0) out[i] = res;
}

// ---- refinement v4: the partitions of one CU together -----------------------------
// The searches of the canonical partitions of one aligned CU (16x16 and up:
// 2Nx2N, 2NxN, Nx2N and the four AMP modes) against one reference usually
// share their integer motion vector and often the half-pel winner.  Their
// SATD / SAD sums over the same units at the same positions are then the
// same numbers, so a warp takes all partitions of a CU: per refinement stage
// it groups the members by their current centre, computes the cost of every
// unit of the CU that a member of the group covers at each of the stage's
// positions once (a table in shared memory), sums each member's units, and
// lets each member pick its winner in the reference's order (the first
// strictly smaller cost in spiral order).  Unit tilings are the ones the
// per-PU kernels use: 8x4 units (4x4 for 4-wide and 12x16 PUs with SATD,
// 4- and 12-wide with SAD), aligned to the CU, since every partition of a
// CU starts at a multiple of its unit width.
struct RefineGroup {
    uint32_t first;     // first member in the member list
    int16_t cx, cy;     // CU origin
    uint8_t count;      // members, 1..32
    uint8_t lg;         // log2 of the CU size, 4..6
    uint8_t ref;
    uint8_t pad_;
};
constexpr int kGrpWarps = 4;
constexpr int kGrpMaxPos = 9;
constexpr int kGrpU8 = 128;   // 8x4 units of a 64x64 CU
constexpr int kGrpU4 = 16;    // 4x4 units of a 16x16 CU (the only size with 4- or 12-wide partitions)

struct GroupSmem {
    int t8[kGrpU8][kGrpMaxPos];
    int t4[kGrpU4][kGrpMaxPos];
    int16_t rx[32], ry[32], rw[32], rh[32];
    int8_t ru4[32];
    int offx[kGrpMaxPos], offy[kGrpMaxPos];   // the stage's positions relative to the centre
};

// floor(q / d) for q < 4096, d <= 16, with m = ceil(65536 / d)
__device__ __forceinline__ int div_small(int q, int m) { return (q * m) >> 16; }

// is unit (x, y, type u4) of the CU inside a member of `grp`?
__device__ __forceinline__ bool unit_covered(const GroupSmem &S, unsigned grp, int x, int y, int u4)
{
    while (grp) {
        const int m = __ffs(grp) - 1;
        grp &= grp - 1;
        if (S.ru4[m] == u4 && x >= S.rx[m] && x < S.rx[m] + S.rw[m] && y >= S.ry[m] && y < S.ry[m] + S.rh[m])
            return true;
    }
    return false;
}

// Costs of the covered units of one type at the P positions (qpel, absolute)
// ccx + offx[k], ccy + offy[k].
template <bool U4>
__device__ __forceinline__ void group_table(GroupSmem &S, unsigned grp, bool had, int cs, const uint8_t *o,
                                            const uint8_t *const *planes, int stride, int px, int py, int ccx,
                                            int ccy, int P, int lane)
{
    constexpr int UW = U4 ? 4 : 8;
    const int *offx = S.offx, *offy = S.offy;
    const int cols = cs / UW, nu = cols * (cs >> 2);
    const int mcols = (65536 + cols - 1) / cols;
    int(*T)[kGrpMaxPos] = U4 ? S.t4 : S.t8;
    if (nu >= 32) {
        // a lane per unit, its current block loaded once for all positions
        for (int u = lane; u < nu; u += 32) {
            const int uy = div_small(u, mcols), ux = u - uy * cols;
            if (!unit_covered(S, grp, ux * UW, uy * 4, U4)) continue;
            UnitC c;
            const ptrdiff_t off = (ptrdiff_t)uy * 4 * stride + ux * UW;
            load_unit<U4>(o + off, stride, c);
            // one copy of the unit's cost code (the kernel stays small in
            // the instruction cache)
#pragma unroll 1
            for (int k = 0; k < P; k++) {
                const int mx = ccx + offx[k], my = ccy + offy[k];
                const uint8_t *r = planes[((my & 3) << 2) + (mx & 3)] + (ptrdiff_t)(py + (my >> 2)) * stride + px +
                                   (mx >> 2) + off;
                T[u][k] = unit_cost_pre<U4>(had, c, r, stride);
            }
        }
    } else {
        // a lane per (unit, position)
        const int mp = (65536 + P - 1) / P;
        for (int e = lane; e < nu * P; e += 32) {
            const int u = div_small(e, mp), k = e - u * P;
            const int uy = div_small(u, mcols), ux = u - uy * cols;
            if (!unit_covered(S, grp, ux * UW, uy * 4, U4)) continue;
            UnitC c;
            const ptrdiff_t off = (ptrdiff_t)uy * 4 * stride + ux * UW;
            load_unit<U4>(o + off, stride, c);
            const int mx = ccx + offx[k], my = ccy + offy[k];
            const uint8_t *r = planes[((my & 3) << 2) + (mx & 3)] + (ptrdiff_t)(py + (my >> 2)) * stride + px +
                               (mx >> 2) + off;
            T[u][k] = unit_cost_pre<U4>(had, c, r, stride);
        }
    }
}

// resident CTAs per SM the register budget is sized for (5: 96 registers;
// measured faster on serving batches than 4 (126) and than the compiler's
// own choice of 168)
#ifndef XG_GROUP_MINB
#define XG_GROUP_MINB 5
#endif
__global__ void __launch_bounds__(32 * kGrpWarps, XG_GROUP_MINB) refine_group_kernel(const RefineGroup *__restrict__ groups,
                                                                      int ngroups,
                                                                      const uint32_t *__restrict__ members,
                                                                      const SessView *__restrict__ views, int R,
                                                                      xavs2gpu_me_params_t prm)
{
    __shared__ GroupSmem smem[kGrpWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kGrpWarps + warp;
    if (gi >= ngroups) return;   // the whole warp
    GroupSmem &S = smem[warp];
    const RefineGroup G = groups[gi];
    const uint32_t e0 = members[G.first];
    const SessView &v = views[e0 >> kSessShift];
    const Geometry g = v.g;
    const int M = G.count, cs = 1 << G.lg;
    const bool had = prm.use_hadamard != 0;
    const int lam = prm.lambda_factor;
    const bool mem = lane < M;
    int i = 0, pmx = 0, pmy = 0, bx = 0, by = 0, best = 0;
    bool valid = false;
    xavs2gpu_me_result_t res;
    if (mem) {
        i = (int)(members[G.first + lane] & kIdxMask);
        const xavs2gpu_pu_t p = v.pus[i];
        const PuState st = v.state[i];
        const unsigned long long key = v.keys[i];
        valid = st.valid && key != kNoKey;
        const int w = c_pu_w[p.part], h = c_pu_h[p.part];
        S.rx[lane] = (int16_t)(p.x - G.cx);
        S.ry[lane] = (int16_t)(p.y - G.cy);
        S.rw[lane] = (int16_t)w;
        S.rh[lane] = (int16_t)h;
        S.ru4[lane] = (int8_t)(had ? satd_unit4(w, h) : (w == 4 || w == 12));
        pmx = p.mvp_x;
        pmy = p.mvp_y;
        if (!valid) {
            res.bmv_x = res.bmv_y = res.imv_x = res.imv_y = 0;
            res.bcost = res.icost = 1 << 30;
            res.mvcost = 0;
            v.res[i] = res;
        } else {
            const int icost = (int)(key >> 32);
            const unsigned order_ = (unsigned)(key & 0xffffffffu);
            int bmx, bmy;
            if (order_ < 2) { bmx = st.cand[order_][0]; bmy = st.cand[order_][1]; }
            else {
                const int q = (int)order_ - 2;
                bmx = st.cx + q % (2 * R) - R;
                bmy = st.cy + q / (2 * R) - R;
            }
            res.imv_x = (int16_t)bmx; res.imv_y = (int16_t)bmy; res.icost = icost;
            bx = bmx * 4; by = bmy * 4; best = icost;
        }
    }
    __syncwarp();
    const uint8_t *o = v.cur + (ptrdiff_t)G.cy * g.stride + G.cx;
    const uint8_t *const *planes = v.planes + 16 * G.ref;
    if (prm.fractional_me) {
        const int pat = prm.fast_sub_me ? 1 : 0, step = prm.fast_sub_me ? 2 : 1;
        for (int stage = 0; stage < (prm.fractional_me > 1 ? 2 : 1); stage++) {
            // the stage's positions relative to the centre, in the reference's order
            int offx[kGrpMaxPos], offy[kGrpMaxPos], P = 0;
            const int k0 = (stage == 0 && had) ? 1 : 0;
#pragma unroll
            for (int k = 0; k < kGrpMaxPos; k++) { offx[k] = 0; offy[k] = 0; }
            P = k0;
#pragma unroll
            for (int pos = 1; pos < 9; pos++) {
                if ((pos - 1) % step) continue;
                const int mult = stage == 0 ? 2 : 1;
#pragma unroll
                for (int k = 0; k < kGrpMaxPos; k++)
                    if (k == P) { offx[k] = mult * c_spiral[pat][pos][0]; offy[k] = mult * c_spiral[pat][pos][1]; }
                P++;
            }
            if (lane == 0) {
#pragma unroll
                for (int k = 0; k < kGrpMaxPos; k++) { S.offx[k] = offx[k]; S.offy[k] = offy[k]; }
            }
            __syncwarp();
            unsigned pending = __ballot_sync(0xffffffffu, mem && valid);
            while (pending) {
                const int leader = __ffs(pending) - 1;
                const int ccx = __shfl_sync(0xffffffffu, bx, leader), ccy = __shfl_sync(0xffffffffu, by, leader);
                const unsigned grp = __ballot_sync(0xffffffffu, mem && valid && bx == ccx && by == ccy) & pending;
                pending &= ~grp;
                const bool need8 = __any_sync(0xffffffffu, ((grp >> lane) & 1) && !S.ru4[lane]);
                const bool need4 = __any_sync(0xffffffffu, ((grp >> lane) & 1) && S.ru4[lane]);
                if (need8)
                    group_table<false>(S, grp, had, cs, o, planes, g.stride, G.cx, G.cy, ccx, ccy, P, lane);
                // 4x4 units occur only in 16x16 CUs (4- and 12-wide partitions);
                // the 4x4 table holds one 16x16 CU
                if (need4 && cs == 16)
                    group_table<true>(S, grp, had, cs, o, planes, g.stride, G.cx, G.cy, ccx, ccy, P, lane);
                __syncwarp();
                // each member's sums over its units
                int acc[kGrpMaxPos];
#pragma unroll
                for (int k = 0; k < kGrpMaxPos; k++) acc[k] = 0;
                for (unsigned left = grp; left;) {
                    const int m = __ffs(left) - 1;
                    left &= left - 1;
                    const int u4 = S.ru4[m], uw = u4 ? 4 : 8;
                    const int nux = S.rw[m] / uw, n = nux * (S.rh[m] >> 2);
                    const int mnux = (65536 + nux - 1) / nux, cols = cs / uw;
                    const int base = (S.ry[m] >> 2) * cols + S.rx[m] / uw;
                    int part[kGrpMaxPos];
#pragma unroll
                    for (int k = 0; k < kGrpMaxPos; k++) part[k] = 0;
                    for (int q = lane; q < n; q += 32) {
                        const int qy = div_small(q, mnux), qx = q - qy * nux;
                        const int u = base + qy * cols + qx;
                        const int *row = u4 ? S.t4[u] : S.t8[u];
#pragma unroll
                        for (int k = 0; k < kGrpMaxPos; k++)
                            if (k < P) part[k] += row[k];
                    }
#pragma unroll
                    for (int k = 0; k < kGrpMaxPos; k++) {
                        if (k < P) {
                            const int t = __reduce_add_sync(0xffffffffu, part[k]);
                            if (lane == m) acc[k] = t;
                        }
                    }
                }
                __syncwarp();   // the tables are rebuilt for the next centre
                if ((grp >> lane) & 1) {
                    int nbx = bx, nby = by;
                    if (k0) best = acc[0] + mv_cost_hd(lam, ccx, ccy, pmx, pmy);
#pragma unroll
                    for (int k = 0; k < kGrpMaxPos; k++) {
                        if (k < k0 || k >= P) continue;
                        const int mx = ccx + offx[k], my = ccy + offy[k];
                        const int c = acc[k] + mv_cost_hd(lam, mx, my, pmx, pmy);
                        if (c < best) { best = c; nbx = mx; nby = my; }
                    }
                    bx = nbx;
                    by = nby;
                }
            }
        }
    }
    if (mem && valid) {
        res.bmv_x = (int16_t)bx; res.bmv_y = (int16_t)by;
        res.bcost = best;
        res.mvcost = mv_cost_hd(lam, bx, by, pmx, pmy);
        v.res[i] = res;
    }
}

// The CU-grouped refinement: a warp per group.
static void launch_groups(const RefineGroup *groups, int n, const uint32_t *members, const SessView *views, int R,
                          const xavs2gpu_me_params_t &prm, cudaStream_t st)
{
    if (n) {
        refine_group_kernel<<<(n + kGrpWarps - 1) / kGrpWarps, 32 * kGrpWarps, 0, st>>>(groups, n, members, views, R,
                                                                                      prm);
        count_launch();
    }
}

}  // namespace xg

#include "fs_ctu.cuh"

namespace xg {

// The refinement's per-warp list on the CTU search's side stream when the
// per-thread list runs too: the lists are disjoint, and each launch's last
// wave then overlaps the other's work.  fork returns the stream to launch on.
static cudaStream_t refine_fork(cudaStream_t st, bool both, CtuSide *&side)
{
    side = XG_CTU_FORK && both ? ctu_side(current_device()) : nullptr;
    if (!side) return st;
    XG_CUDA(cudaEventRecord(side->fork, st));
    XG_CUDA(cudaStreamWaitEvent(side->st, side->fork, 0));
    return side->st;
}
static void refine_join(cudaStream_t st, CtuSide *side)
{
    if (!side) return;
    XG_CUDA(cudaEventRecord(side->join, side->st));
    XG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
}

// The per-PU search beside the CTU search (their PUs are disjoint) on a
// second side stream, when both have work and phases are not being timed.
static cudaStream_t search_fork(cudaStream_t st, bool both, CtuSide *&side)
{
    side = XG_CTU_FORK && both ? ctu_side(current_device(), 1) : nullptr;
    if (!side) return st;
    XG_CUDA(cudaEventRecord(side->fork, st));
    XG_CUDA(cudaStreamWaitEvent(side->st, side->fork, 0));
    return side->st;
}

// ---- session ---------------------------------------------------------------------
// CU-grouped refinement on (1) or per-PU kernels only (0); the results are
// the same either way
#ifndef XG_REFINE_GROUPS
#define XG_REFINE_GROUPS 1
#endif
static constexpr bool use_groups() { return XG_REFINE_GROUPS != 0; }


#ifndef XG_REFINE_LPT
#define XG_REFINE_LPT 1
#endif

// default refinement split (pixels): searches of PUs up to this size refine
// one per thread, larger ones one per warp (xavs2gpu_me_set_tuning changes it)
#ifndef XG_REFINE_SPLIT
#define XG_REFINE_SPLIT 256
#endif

struct MeSessionImpl {
    int W = 0, H = 0, nrefs = 0, max_pus = 0;
    int stride = 0, rows = 0;
    size_t plane_bytes = 0;
    int device = 0;
    cudaStream_t st = nullptr;
    uint8_t *d_planes = nullptr;          // plane 0: current picture; 1 + r*16 + k: reference r, sub-pel k
    void *d_tmap = nullptr;               // tensor map over d_planes (window copies), or null
    uint8_t **d_plane_ptrs = nullptr;     // [1 + nrefs*16] pointers at pixel (0,0)
    const uint8_t **d_ref0 = nullptr;     // [nrefs] full-pel plane of each reference
    uint8_t *h_stage = nullptr;           // pinned staging for pictures
    size_t h_stage_cap = 0;
    uint8_t *d_upload = nullptr;          // device copy of an uploaded picture
    // PU list and plan
    int n = 0;
    xavs2gpu_pu_t *d_pus = nullptr;
    xavs2gpu_me_result_t *d_res = nullptr;
    xavs2gpu_me_result_t *h_res = nullptr;   // pinned
    unsigned long long *d_keys = nullptr;
    PuState *d_state = nullptr;
    int *d_generic = nullptr;
    int n_generic = 0;
    CtuPlan plan;
    int plan_R = -1;               // search range the plan was built for (-1: stale)
    bool plan_ctu = true;          // whether the plan could use the CTU search
    int n_ctu_pus = 0;
    std::vector<xavs2gpu_pu_t> h_pus;
    int *d_small = nullptr, *d_large = nullptr;   // refinement lists: thread / warp per search
    int n_small = 0, n_large = 0;
    bool profiling = false;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // launch shapes (results do not depend on them): searches of at most
    // tune_split pixels refine one per thread, larger ones one per warp;
    // tune_block threads per refinement CTA
    int tune_split = XG_REFINE_SPLIT, tune_block = 128;
    int cu_groups = 1;   // CU-grouped refinement (when PMVR is off)
    // reference slot r lives in plane buffer set slot_buf[r] (rotated by
    // xavs2gpu_me_rotate_refs without moving pixels)
    int slot_buf[16] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15};
    cudaStream_t own_st = nullptr;   // the stream the session created
    SessView h_view{};
    SessView *d_view = nullptr;      // this session as the kernels see it
    std::vector<uint32_t> h_generic, h_small, h_large;
    // CU-grouped refinement: the groups, their members, and the thread /
    // warp lists of the searches no group covers
    RefineGroup *d_groups = nullptr;
    uint32_t *d_members = nullptr;
    int *d_small_g = nullptr, *d_large_g = nullptr;
    int n_groups = 0, n_heavy = 0, n_small_g = 0, n_large_g = 0;   // groups [0, n_heavy): 32x32 and 64x64 CUs
    std::vector<RefineGroup> h_groups;
    std::vector<uint32_t> h_members, h_small_g, h_large_g;

    uint8_t *plane(int idx) { return d_planes + (size_t)idx * plane_bytes + (size_t)kPad * stride + kPad; }
    uint8_t *ref_plane(int slot, int k) { return plane(1 + 16 * slot_buf[slot] + k); }
};

// A mapped pinned word that kernels set when they give up a bounded wait
// (the window copy of the CTU search); the host reads it after a
// synchronisation.  Null when mapped memory is unavailable.
static unsigned *wait_flag_word()
{
    static unsigned *word = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = nullptr;
        if (cudaHostAlloc(&h, sizeof(unsigned), cudaHostAllocMapped | cudaHostAllocPortable) == cudaSuccess) {
            *static_cast<volatile unsigned *>(h) = 0;
            word = static_cast<unsigned *>(h);
        } else {
            cudaGetLastError();
        }
    });
    return word;
}

// Reports (once) a bounded wait a kernel gave up since the last check.
static int check_wait_flag(const char *where)
{
    unsigned *w = wait_flag_word();
    if (w && *static_cast<volatile unsigned *>(w)) {
        *static_cast<volatile unsigned *>(w) = 0;
        fail(XAVS2GPU_ERR_CUDA, where, "a search window copy did not complete within its wait limit");
        return XAVS2GPU_ERR_CUDA;
    }
    return XAVS2GPU_OK;
}

// Tensor map over a session's plane pool for the CTU search's window copies:
// 3-D u8 (column < stride, row < rows, plane < nplanes), rows stride bytes
// and planes plane_bytes apart, box kTmaBoxCols x kTmaBoxRows x 1, zero fill
// outside.  Returns a device copy (64-byte aligned), or null when the driver
// entry point or the encoding is unavailable (the search then fills its
// window with 16-byte loads).
static void *plane_pool_tmap(const uint8_t *pool, int stride, int rows, size_t plane_bytes, int nplanes)
{
#if XG_CTU_TMA
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    });
    if (!encode || ((uintptr_t)pool & 255) || (stride & 15) || (plane_bytes & 15)) return nullptr;
    CUtensorMap tm;
    const cuuint64_t dims[3] = {(cuuint64_t)stride, (cuuint64_t)rows, (cuuint64_t)nplanes};
    const cuuint64_t strides[2] = {(cuuint64_t)stride, (cuuint64_t)plane_bytes};
    const cuuint32_t box[3] = {(cuuint32_t)kTmaBoxCols, (cuuint32_t)kTmaBoxRows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (encode(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<uint8_t *>(pool), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return nullptr;
    void *d = nullptr;
    XG_CUDA(cudaMalloc(&d, sizeof(CUtensorMap)));
    XG_CUDA(cudaMemcpy(d, &tm, sizeof(CUtensorMap), cudaMemcpyHostToDevice));
    return d;
#else
    (void)pool; (void)stride; (void)rows; (void)plane_bytes; (void)nplanes;
    return nullptr;
#endif
}

static void refresh_view(MeSessionImpl &m)
{
    SessView v;
    v.cur = m.plane(0);
    v.ref0 = m.d_ref0;
    v.planes = (const uint8_t *const *)(m.d_plane_ptrs + 1);
    v.pus = m.d_pus;
    v.state = m.d_state;
    v.keys = m.d_keys;
    v.res = m.d_res;
    v.slots = m.plan.d_slots;
    v.g = Geometry{m.W, m.H, m.stride};
    v.n = m.n;
    v.tmap = m.d_tmap;
    v.pool = m.d_planes;
    v.plane_bytes = m.plane_bytes;
    v.wait_flag = wait_flag_word();
    m.h_view = v;
    XG_CUDA(cudaMemcpyAsync(m.d_view, &m.h_view, sizeof(SessView), cudaMemcpyHostToDevice, m.st));
}

}  // namespace xg

using namespace xg;

struct xavs2gpu_me_session {
    MeSessionImpl impl;
};

extern "C" void xavs2gpu_pu_set_limits(xavs2gpu_pu_t *pu, int width, int height, int vmin_qpel, int vmax_qpel)
{
    const int w = h_pu_w[pu->part], h = h_pu_h[pu->part];
    auto clip = [](int lo, int hi, int v) { return v < lo ? lo : (v > hi ? hi : v); };
    int mn = clip(-8192, 8191, (-64 - pu->x) * 4), mx = clip(-8192, 8191, (width + 64 - pu->x - w) * 4);
    pu->min_x = (int16_t)((mn >> 2) + 6);
    pu->max_x = (int16_t)((mx >> 2) - 6);
    mn = clip(vmin_qpel, vmax_qpel, (-64 - pu->y) * 4);
    mx = clip(vmin_qpel, vmax_qpel, (height + 64 - pu->y - h) * 4);
    pu->min_y = (int16_t)((mn >> 2) + 6);
    pu->max_y = (int16_t)((mx >> 2) - 6);
}

extern "C" xavs2gpu_me_session_t *xavs2gpu_me_create(int width, int height, int num_refs, int max_pus)
{
    if (width < 8 || height < 8 || width > 8192 || height > 8192 || num_refs < 1 || num_refs > 16 || max_pus < 1 ||
        max_pus > (int)kIdxMask) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_create", "bad size, reference count or PU capacity");
        return nullptr;
    }
    auto *s = new xavs2gpu_me_session();
    MeSessionImpl &m = s->impl;
    m.device = current_device();
    XG_CUDA(cudaSetDevice(m.device));
    m.W = width; m.H = height; m.nrefs = num_refs; m.max_pus = max_pus;
    m.stride = (int)align_up((size_t)width + 2 * kPad, 64);
    m.rows = height + 2 * kPad;
    m.plane_bytes = align_up((size_t)m.stride * m.rows, 256);
    const int nplanes = 1 + 16 * num_refs;
    XG_CUDA(cudaStreamCreateWithFlags(&m.own_st, cudaStreamNonBlocking));
    m.st = m.own_st;
    // 256 bytes of slack after the last plane: word-wise row readers (the skip
    // costs' 3-word prediction rows) may touch the aligned word after a row
    // that ends at the right edge of the margin, which lies past the last
    // plane when its size is already a multiple of 256.
    XG_CUDA(cudaMalloc((void **)&m.d_planes, m.plane_bytes * nplanes + 256));
    XG_CUDA(cudaMemsetAsync(m.d_planes, 0, m.plane_bytes * nplanes + 256, m.st));
    std::vector<uint8_t *> ptrs(nplanes);
    for (int k = 0; k < nplanes; k++) ptrs[k] = m.plane(k);
    XG_CUDA(cudaMalloc((void **)&m.d_plane_ptrs, sizeof(uint8_t *) * nplanes));
    XG_CUDA(cudaMemcpy(m.d_plane_ptrs, ptrs.data(), sizeof(uint8_t *) * nplanes, cudaMemcpyHostToDevice));
    m.d_tmap = plane_pool_tmap(m.d_planes, m.stride, m.rows, m.plane_bytes, nplanes);
    std::vector<const uint8_t *> r0(num_refs);
    for (int r = 0; r < num_refs; r++) r0[r] = m.plane(1 + 16 * r);
    XG_CUDA(cudaMalloc((void **)&m.d_ref0, sizeof(uint8_t *) * num_refs));
    XG_CUDA(cudaMemcpy(m.d_ref0, r0.data(), sizeof(uint8_t *) * num_refs, cudaMemcpyHostToDevice));
    m.h_stage_cap = (size_t)width * height;
    XG_CUDA(cudaMallocHost((void **)&m.h_stage, m.h_stage_cap));
    XG_CUDA(cudaMalloc((void **)&m.d_upload, m.h_stage_cap));
    XG_CUDA(cudaMalloc((void **)&m.d_pus, sizeof(xavs2gpu_pu_t) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_res, sizeof(xavs2gpu_me_result_t) * max_pus));
    XG_CUDA(cudaMallocHost((void **)&m.h_res, sizeof(xavs2gpu_me_result_t) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_keys, sizeof(unsigned long long) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_state, sizeof(PuState) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_generic, sizeof(int) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_small, sizeof(int) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_large, sizeof(int) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_groups, sizeof(RefineGroup) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_members, sizeof(uint32_t) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_small_g, sizeof(int) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_large_g, sizeof(int) * max_pus));
    XG_CUDA(cudaMalloc((void **)&m.d_view, sizeof(SessView)));
    refresh_view(m);
    XG_CUDA(cudaStreamSynchronize(m.st));
    return s;
}

extern "C" void xavs2gpu_me_destroy(xavs2gpu_me_session_t *s)
{
    if (!s) return;
    MeSessionImpl &m = s->impl;
    cudaSetDevice(m.device);
    if (m.st) cudaStreamSynchronize(m.st);
    cudaFree(m.d_view);
    ctu_plan_free(m.plan);
    cudaFree(m.d_planes); cudaFree(m.d_plane_ptrs); cudaFree(m.d_ref0);
    if (m.d_tmap) cudaFree(m.d_tmap);
    cudaFreeHost(m.h_stage); cudaFree(m.d_upload);
    cudaFree(m.d_pus); cudaFree(m.d_res); cudaFreeHost(m.h_res); cudaFree(m.d_keys);
    cudaFree(m.d_state); cudaFree(m.d_generic); 
    cudaFree(m.d_small); cudaFree(m.d_large);
    cudaFree(m.d_groups); cudaFree(m.d_members); cudaFree(m.d_small_g); cudaFree(m.d_large_g);
    for (auto &e : m.ev)
        if (e) cudaEventDestroy(e);
    if (m.own_st) cudaStreamDestroy(m.own_st);
    delete s;
}

// replicates the border of the picture just copied into the slot's plane;
// for references also computes the 15 sub-pel planes
static int finish_picture(MeSessionImpl &m, int slot)
{
    const int idx = slot < 0 ? 0 : 1 + 16 * m.slot_buf[slot];
    if (xavs2gpu_expand_border(m.plane(idx), m.stride, m.W, m.H, kPad, m.st) != XAVS2GPU_OK) return XAVS2GPU_ERR_CUDA;
    if (slot >= 0) {
        uint8_t *planes[16];
        for (int k = 0; k < 16; k++) planes[k] = m.plane(idx + k);
        return xavs2gpu_interpolate_frame(m.plane(idx), m.stride, m.W, m.H, kPad, planes, 2, m.st);
    }
    return XAVS2GPU_OK;
}

// a W x H picture in device memory (`stride`) into the slot: the current
// picture is copied into its plane and its border replicated; a reference's
// 16 planes (full-pel with border, 15 sub-pel) come from one kernel reading
// the source directly
static int load_picture(MeSessionImpl &m, int slot, const uint8_t *dsrc, intptr_t stride)
{
    const int idx = slot < 0 ? 0 : 1 + 16 * m.slot_buf[slot];
    if (slot >= 0 && stride <= INT32_MAX) {
        uint8_t *planes[16];
        for (int k = 0; k < 16; k++) planes[k] = m.plane(idx + k);
        return reference_planes_from(dsrc, (int)stride, m.W, m.H, kPad, planes, m.stride, m.st);
    }
    XG_CUDA(cudaMemcpy2DAsync(m.plane(idx), m.stride, dsrc, stride, m.W, m.H, cudaMemcpyDeviceToDevice, m.st));
    return finish_picture(m, slot);
}

extern "C" int xavs2gpu_me_set_picture_device(xavs2gpu_me_session_t *s, int slot, const uint8_t *luma, intptr_t stride)
{
    if (!s || slot < -1 || slot >= s->impl.nrefs || stride < s->impl.W) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_set_picture_device", "bad slot or stride");
        return XAVS2GPU_ERR_ARG;
    }
    XG_CUDA(cudaSetDevice(s->impl.device));
    return load_picture(s->impl, slot, luma, stride);
}

extern "C" int xavs2gpu_me_set_picture_host(xavs2gpu_me_session_t *s, int slot, const uint8_t *luma, intptr_t stride)
{
    if (!s || slot < -1 || slot >= s->impl.nrefs || stride < s->impl.W) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_set_picture_host", "bad slot or stride");
        return XAVS2GPU_ERR_ARG;
    }
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, luma) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
        // page-locked: one asynchronous 2-D copy into the plane, no staging
        const int idx = slot < 0 ? 0 : 1 + 16 * m.slot_buf[slot];
        XG_CUDA(cudaMemcpy2DAsync(m.plane(idx), m.stride, luma, stride, m.W, m.H, cudaMemcpyHostToDevice, m.st));
        return finish_picture(m, slot);
    }
    cudaGetLastError();   // pageable memory is reported as an error by some drivers
    // the staging buffer may still feed an earlier upload on the stream
    XG_CUDA(cudaStreamSynchronize(m.st));
    pack_rows(m.h_stage, luma, stride, m.W, m.H);
    XG_CUDA(cudaMemcpyAsync(m.d_upload, m.h_stage, (size_t)m.W * m.H, cudaMemcpyHostToDevice, m.st));
    return load_picture(m, slot, m.d_upload, m.W);
}

extern "C" int xavs2gpu_me_set_pus(xavs2gpu_me_session_t *s, const xavs2gpu_pu_t *pus, int n)
{
    if (!s || n < 0 || n > s->impl.max_pus) {
        fail(XAVS2GPU_ERR_CAPACITY, "xavs2gpu_me_set_pus", "PU count exceeds the session capacity");
        return XAVS2GPU_ERR_CAPACITY;
    }
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    for (int i = 0; i < n; i++) {
        const xavs2gpu_pu_t &p = pus[i];
        const int w = p.part < kNumParts ? h_pu_w[p.part] : 0, h = p.part < kNumParts ? h_pu_h[p.part] : 0;
        if (p.part >= kNumParts || p.ref >= m.nrefs || p.x < 0 || p.y < 0 || p.x + w > m.W || p.y + h > m.H) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_set_pus", "PU outside the picture or bad shape/reference");
            return XAVS2GPU_ERR_ARG;
        }
        // every reference read (window, sub-pel taps) must stay inside the margin
        if (p.min_x < -kPad + 8 - p.x || p.max_x > m.W + kPad - 8 - p.x - w || p.min_y < -kPad + 8 - p.y ||
            p.max_y > m.H + kPad - 8 - p.y - h) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_set_pus", "search limits reach beyond the 80-pixel margin");
            return XAVS2GPU_ERR_ARG;
        }
    }
    m.n = n;
    m.h_pus.assign(pus, pus + n);
    XG_CUDA(cudaStreamSynchronize(m.st));
    if (n) XG_CUDA(cudaMemcpyAsync(m.d_pus, pus, sizeof(xavs2gpu_pu_t) * n, cudaMemcpyHostToDevice, m.st));
    refresh_view(m);
    XG_CUDA(cudaStreamSynchronize(m.st));
    m.plan_R = -1;
    return XAVS2GPU_OK;
}

// Groups the searches that are canonical partitions of an aligned CU of
// 16x16 or larger by (reference, CU); larger CUs first.  The searches left
// over keep the thread / warp lists.
static void build_groups(MeSessionImpl &m, const std::vector<int> &small, const std::vector<int> &large)
{
    std::unordered_map<uint64_t, int> open;   // key -> group index (the one still filling)
    std::vector<std::vector<int>> gm;
    std::vector<RefineGroup> gd;
    std::vector<char> grouped(m.n, 0);
    for (int i = 0; i < m.n; i++) {
        const xavs2gpu_pu_t &p = m.h_pus[i];
        const int w = h_pu_w[p.part], h = h_pu_h[p.part], S = w > h ? w : h;
        const int lg = S == 16 ? 4 : S == 32 ? 5 : S == 64 ? 6 : 0;
        if (!lg) continue;
        const int cx = p.x & ~(S - 1), cy = p.y & ~(S - 1);
        bool canon = false;
        for (int mo = 0; mo < 13 && !canon; mo++) {
            const SlotGeom g = cu_mode_geom(S, cx, cy, mo);
            canon = g.part == p.part && g.ox == p.x && g.oy == p.y;
        }
        if (!canon) continue;
        const uint64_t key = ((uint64_t)p.ref << 40) | ((uint64_t)lg << 32) | ((uint64_t)(uint16_t)cx << 16) |
                             (uint64_t)(uint16_t)cy;
        auto it = open.find(key);
        int gi;
        if (it == open.end() || gm[it->second].size() >= 32) {
            gi = (int)gm.size();
            gm.emplace_back();
            RefineGroup d{};
            d.cx = (int16_t)cx;
            d.cy = (int16_t)cy;
            d.lg = (uint8_t)lg;
            d.ref = p.ref;
            gd.push_back(d);
            open[key] = gi;
        } else {
            gi = it->second;
        }
        gm[gi].push_back(i);
        grouped[i] = 1;
    }
    std::vector<int> ord(gd.size());
    for (size_t k = 0; k < ord.size(); k++) ord[k] = (int)k;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return gd[a].lg > gd[b].lg; });
    m.h_groups.clear();
    m.h_members.clear();
    for (int k : ord) {
        RefineGroup d = gd[k];
        d.first = (uint32_t)m.h_members.size();
        d.count = (uint8_t)gm[k].size();
        for (int i : gm[k]) m.h_members.push_back((uint32_t)i);
        m.h_groups.push_back(d);
    }
    m.h_small_g.clear();
    m.h_large_g.clear();
    for (int i : small)
        if (!grouped[i]) m.h_small_g.push_back((uint32_t)i);
    for (int i : large)
        if (!grouped[i]) m.h_large_g.push_back((uint32_t)i);
    m.n_groups = (int)m.h_groups.size();
    m.n_heavy = 0;
    while (m.n_heavy < m.n_groups && m.h_groups[m.n_heavy].lg >= 5) m.n_heavy++;
    m.n_small_g = (int)m.h_small_g.size();
    m.n_large_g = (int)m.h_large_g.size();
    if (m.n_groups) {
        XG_CUDA(cudaMemcpyAsync(m.d_groups, m.h_groups.data(), sizeof(RefineGroup) * m.n_groups,
                                cudaMemcpyHostToDevice, m.st));
        XG_CUDA(cudaMemcpyAsync(m.d_members, m.h_members.data(), sizeof(uint32_t) * m.h_members.size(),
                                cudaMemcpyHostToDevice, m.st));
    }
    if (m.n_small_g)
        XG_CUDA(cudaMemcpyAsync(m.d_small_g, m.h_small_g.data(), sizeof(int) * m.n_small_g, cudaMemcpyHostToDevice,
                                m.st));
    if (m.n_large_g)
        XG_CUDA(cudaMemcpyAsync(m.d_large_g, m.h_large_g.data(), sizeof(int) * m.n_large_g, cudaMemcpyHostToDevice,
                                m.st));
}

// (Re)builds the split into CTU jobs and per-PU searches for window size R.
// The CTU search keeps (cost << 11 | order) keys in 32 bits, which holds the
// MV costs of every lambda below 2^26 (the reference's QP range needs below
// 2^23); larger lambdas plan every PU for the per-PU search.
constexpr int kCtuMaxLambda = 1 << 26;

static void ensure_plan(MeSessionImpl &m, int R, int lambda)
{
    const bool ctu = lambda < kCtuMaxLambda;
    if (m.plan_R == R && m.plan_ctu == ctu) return;
    std::vector<int> generic;
    ctu_plan_build(m.plan, m.h_pus, m.W, m.H, m.nrefs, R, ctu, generic, m.st);
    m.n_generic = (int)generic.size();
    m.n_ctu_pus = m.n - m.n_generic;
    m.h_generic.assign(generic.begin(), generic.end());
    if (m.n_generic)
        XG_CUDA(cudaMemcpyAsync(m.d_generic, generic.data(), sizeof(int) * m.n_generic, cudaMemcpyHostToDevice, m.st));
    // PUs of the CTU plan have the single candidate (0,0), which is also the
    // search centre; their state is fixed by the plan (the CTU kernel
    // evaluates the candidate itself)
    {
        std::vector<PuState> st(m.n);
        std::vector<char> is_generic(m.n, 0);
        for (int i : generic) is_generic[i] = 1;
        for (int i = 0; i < m.n; i++) {
            PuState &x = st[i];
            memset(&x, 0, sizeof(x));
            x.ncand = 1;
            x.valid = is_generic[i] ? 0 : 1;
        }
        if (m.n) XG_CUDA(cudaMemcpyAsync(m.d_state, st.data(), sizeof(PuState) * m.n, cudaMemcpyHostToDevice, m.st));
        XG_CUDA(cudaStreamSynchronize(m.st));
    }
    // refinement order: PU searches grouped by shape
    std::vector<int> order(m.n), start(kNumParts + 1, 0);
    for (const auto &p : m.h_pus) start[p.part + 1]++;
    for (int k = 0; k < kNumParts; k++) start[k + 1] += start[k];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < m.n; i++) order[fill[m.h_pus[i].part]++] = i;
    std::vector<int> small, large;
    for (int k = 0; k < m.n; k++) {
        const int i = order[k];
        (h_pu_w[m.h_pus[i].part] * h_pu_h[m.h_pus[i].part] <= m.tune_split ? small : large).push_back(i);
    }
#if XG_REFINE_LPT
    // largest searches first (shape groups kept together): the long ones
    // start early instead of forming the launch's tail
    auto area = [&](int i) { return h_pu_w[m.h_pus[i].part] * h_pu_h[m.h_pus[i].part]; };
    std::stable_sort(small.begin(), small.end(), [&](int a, int b) { return area(a) > area(b); });
    std::stable_sort(large.begin(), large.end(), [&](int a, int b) { return area(a) > area(b); });
#endif
    m.n_small = (int)small.size();
    m.n_large = (int)large.size();
    m.h_small.assign(small.begin(), small.end());
    m.h_large.assign(large.begin(), large.end());
    if (m.n_small) XG_CUDA(cudaMemcpyAsync(m.d_small, small.data(), sizeof(int) * m.n_small, cudaMemcpyHostToDevice, m.st));
    if (m.n_large) XG_CUDA(cudaMemcpyAsync(m.d_large, large.data(), sizeof(int) * m.n_large, cudaMemcpyHostToDevice, m.st));
    build_groups(m, small, large);
    refresh_view(m);
    XG_CUDA(cudaStreamSynchronize(m.st));
    m.plan_R = R;
    m.plan_ctu = ctu;
}

extern "C" int xavs2gpu_me_run(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm)
{
    if (!s || !prm || prm->search_range < 1 || prm->search_range > 128 || prm->fractional_me < 0 ||
        prm->fractional_me > 2 || prm->lambda_factor < 0) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_run", "bad parameters");
        return XAVS2GPU_ERR_ARG;
    }
    MeSessionImpl &m = s->impl;
    if (m.n == 0) return XAVS2GPU_OK;
    XG_CUDA(cudaSetDevice(m.device));
    const int R = prm->search_range, lam = prm->lambda_factor;
    ensure_plan(m, R, lam);
    if (m.profiling) XG_CUDA(cudaEventRecord(m.ev[0], m.st));
    XG_CUDA(cudaMemsetAsync(m.d_keys, 0xff, sizeof(unsigned long long) * m.n, m.st));
    const uint32_t *gen = reinterpret_cast<const uint32_t *>(m.d_generic);
    if (m.n_generic) {
        me_init_list_kernel<<<(m.n_generic * 32 + 127) / 128, 128, 0, m.st>>>(gen, m.n_generic, m.d_view, lam);
        count_launch();
    }
    if (m.profiling) XG_CUDA(cudaEventRecord(m.ev[1], m.st));
    CtuSide *gside = nullptr;
    const cudaStream_t gst = search_fork(m.st, !m.profiling && m.n_generic && m.plan.n_jobs, gside);
    if (gside && m.n_generic) {
        const int rc = fs_generic_launch(gen, m.n_generic, m.d_view, R, lam, gst);
        if (rc != XAVS2GPU_OK) {
            refine_join(m.st, gside);
            return rc;
        }
    }
    ctu_jobs_run(m.plan.d_jobs, m.plan.n_jobs, m.plan.n_border, m.d_view, *prm, m.st);
    if (m.profiling) XG_CUDA(cudaEventRecord(m.ev[2], m.st));
    if (!gside && m.n_generic) {
        const int rc = fs_generic_launch(gen, m.n_generic, m.d_view, R, lam, m.st);
        if (rc != XAVS2GPU_OK) return rc;
    }
    refine_join(m.st, gside);
    if (m.profiling) XG_CUDA(cudaEventRecord(m.ev[3], m.st));
    // the CU-grouped refinement follows the reference's per-PU order, which
    // with PMVR depends on each PU's predictor; PMVR keeps the per-PU kernels
    const bool grouped = !prm->enable_pmvr && m.cu_groups && m.n_groups > 0 && use_groups();
    const int ns = grouped ? m.n_small_g : m.n_small, nl = grouped ? m.n_large_g : m.n_large;
    const int *lst_s = grouped ? m.d_small_g : m.d_small, *lst_l = grouped ? m.d_large_g : m.d_large;
    if (grouped) launch_groups(m.d_groups, m.n_groups, m.d_members, m.d_view, R, *prm, m.st);
    CtuSide *side = nullptr;
    const cudaStream_t wst = refine_fork(m.st, ns && nl, side);
    if (ns) {
        const unsigned g = (ns + m.tune_block - 1) / m.tune_block;
        if (prm->use_hadamard)
            refine_thread_kernel<true><<<g, m.tune_block, 0, m.st>>>(reinterpret_cast<const uint32_t *>(lst_s), ns,
                                                                     m.d_view, R, *prm);
        else
            refine_thread_kernel<false><<<g, m.tune_block, 0, m.st>>>(reinterpret_cast<const uint32_t *>(lst_s), ns,
                                                                      m.d_view, R, *prm);
        count_launch();
    }
    if (nl) {
        refine_warp_list_kernel<<<(nl * 32 + m.tune_block - 1) / m.tune_block, m.tune_block, 0, wst>>>(
            reinterpret_cast<const uint32_t *>(lst_l), nl, m.d_view, R, *prm);
        count_launch();
    }
    refine_join(m.st, side);
    if (m.profiling) XG_CUDA(cudaEventRecord(m.ev[4], m.st));
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

extern "C" void xavs2gpu_me_session_info(const xavs2gpu_me_session_t *s, int *width, int *height, int *num_refs,
                                         int *n_pus)
{
    if (!s) return;
    if (width) *width = s->impl.W;
    if (height) *height = s->impl.H;
    if (num_refs) *num_refs = s->impl.nrefs;
    if (n_pus) *n_pus = s->impl.n;
}

extern "C" int xavs2gpu_me_session_pus(const xavs2gpu_me_session_t *s, xavs2gpu_pu_t *out)
{
    if (!s || !out) return XAVS2GPU_ERR_ARG;
    for (int i = 0; i < s->impl.n; i++) out[i] = s->impl.h_pus[i];
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_me_set_tuning(xavs2gpu_me_session_t *s, const xavs2gpu_me_tuning_t *t)
{
    if (!s || !t || t->refine_split_px < 0 || t->refine_split_px > 4096 ||
        (t->refine_block != 32 && t->refine_block != 64 && t->refine_block != 128) ||
        (t->cu_groups != 0 && t->cu_groups != 1)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_set_tuning",
             "refine_split_px must be 0..4096, refine_block 32/64/128, cu_groups 0/1");
        return XAVS2GPU_ERR_ARG;
    }
    MeSessionImpl &m = s->impl;
    if (t->refine_split_px != m.tune_split) m.plan_R = -1;   // the refinement lists change
    m.tune_split = t->refine_split_px;
    m.tune_block = t->refine_block;
    m.cu_groups = t->cu_groups;
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_me_get_tuning(const xavs2gpu_me_session_t *s, xavs2gpu_me_tuning_t *t)
{
    if (!s || !t) return XAVS2GPU_ERR_ARG;
    t->refine_split_px = s->impl.tune_split;
    t->refine_block = s->impl.tune_block;
    t->cu_groups = s->impl.cu_groups;
    t->pad_ = 0;
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_me_autotune(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm, int reps,
                                    float *best_ms)
{
    if (!s || !prm || reps < 1) return XAVS2GPU_ERR_ARG;
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    cudaEvent_t e0, e1;
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    xavs2gpu_me_tuning_t best{m.tune_split, m.tune_block, m.cu_groups, 0}, cand{};
    float best_t = 1e30f;
    int rc = XAVS2GPU_OK;
    for (int split : {0, 64, 128, 256, 512, 1024, 4096}) {
        for (int cfg = 0; cfg < 4; cfg++) {
            cand.refine_split_px = split;
            cand.refine_block = cfg & 1 ? 128 : 64;
            cand.cu_groups = cfg >> 1;
            if ((rc = xavs2gpu_me_set_tuning(s, &cand)) != XAVS2GPU_OK) break;
            ensure_plan(m, prm->search_range, prm->lambda_factor);
            if ((rc = xavs2gpu_me_run(s, prm)) != XAVS2GPU_OK) break;   // warm-up
            XG_CUDA(cudaEventRecord(e0, m.st));
            for (int i = 0; i < reps; i++)
                if ((rc = xavs2gpu_me_run(s, prm)) != XAVS2GPU_OK) break;
            XG_CUDA(cudaEventRecord(e1, m.st));
            XG_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            XG_CUDA(cudaEventElapsedTime(&t, e0, e1));
            t /= reps;
            if (t < best_t) {
                best_t = t;
                best = cand;
            }
        }
        if (rc != XAVS2GPU_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != XAVS2GPU_OK) return rc;
    rc = xavs2gpu_me_set_tuning(s, &best);
    if (rc == XAVS2GPU_OK) ensure_plan(m, prm->search_range, prm->lambda_factor);
    if (best_ms) *best_ms = best_t;
    return rc;
}

extern "C" int xavs2gpu_me_prepare(xavs2gpu_me_session_t *s, const xavs2gpu_me_params_t *prm)
{
    if (!s || !prm || prm->search_range < 1 || prm->search_range > 128) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_prepare", "bad parameters");
        return XAVS2GPU_ERR_ARG;
    }
    XG_CUDA(cudaSetDevice(s->impl.device));
    ensure_plan(s->impl, prm->search_range, prm->lambda_factor);
    ctu_prime(prm->search_range);   // nothing created inside a capture that follows
    return XAVS2GPU_OK;
}

extern "C" void xavs2gpu_me_set_profiling(xavs2gpu_me_session_t *s, int enable)
{
    if (!s) return;
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    if (enable && !m.ev[0])
        for (auto &e : m.ev) XG_CUDA(cudaEventCreate(&e));
    m.profiling = enable != 0;
}

extern "C" int xavs2gpu_me_phase_ms(xavs2gpu_me_session_t *s, float ms[4])
{
    if (!s || !s->impl.profiling) return XAVS2GPU_ERR_ARG;
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaEventSynchronize(m.ev[4]));
    for (int i = 0; i < 4; i++) XG_CUDA(cudaEventElapsedTime(&ms[i], m.ev[i], m.ev[i + 1]));
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_me_get_results(xavs2gpu_me_session_t *s, xavs2gpu_me_result_t *out)
{
    if (!s || !out) return XAVS2GPU_ERR_ARG;
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    if (m.n) {
        // straight into the caller's buffer (one DMA when it is pinned; the
        // driver stages pageable memory itself)
        XG_CUDA(cudaMemcpyAsync(out, m.d_res, sizeof(xavs2gpu_me_result_t) * m.n, cudaMemcpyDeviceToHost, m.st));
        XG_CUDA(cudaStreamSynchronize(m.st));
    }
    return check_wait_flag("xavs2gpu_me_get_results");
}

extern "C" int xavs2gpu_me_sync(xavs2gpu_me_session_t *s)
{
    if (!s) return XAVS2GPU_ERR_ARG;
    XG_CUDA(cudaStreamSynchronize(s->impl.st));
    return check_wait_flag("xavs2gpu_me_sync");
}

extern "C" const xavs2gpu_me_result_t *xavs2gpu_me_results_device(xavs2gpu_me_session_t *s)
{
    return s ? s->impl.d_res : nullptr;
}

extern "C" uint8_t *xavs2gpu_me_plane_device(xavs2gpu_me_session_t *s, int slot, int k)
{
    if (!s || slot < -1 || slot >= s->impl.nrefs || k < 0 || k > 15 || (slot < 0 && k != 0)) return nullptr;
    return slot < 0 ? s->impl.plane(0) : s->impl.ref_plane(slot, k);
}

extern "C" int xavs2gpu_me_plane_stride(xavs2gpu_me_session_t *s) { return s ? s->impl.stride : 0; }

extern "C" int xavs2gpu_me_get_plane(xavs2gpu_me_session_t *s, int slot, int k, uint8_t *out, intptr_t stride)
{
    uint8_t *p = xavs2gpu_me_plane_device(s, slot, k);
    if (!p || !out || stride < s->impl.W + 2 * kPad) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_get_plane", "bad slot, plane or stride");
        return XAVS2GPU_ERR_ARG;
    }
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    XG_CUDA(cudaMemcpy2DAsync(out, stride, p - (size_t)kPad * m.stride - kPad, m.stride, m.W + 2 * kPad,
                              m.H + 2 * kPad, cudaMemcpyDeviceToHost, m.st));
    XG_CUDA(cudaStreamSynchronize(m.st));
    return XAVS2GPU_OK;
}
extern "C" int xavs2gpu_me_plane_pad(xavs2gpu_me_session_t *) { return kPad; }
extern "C" int xavs2gpu_me_window_tma(xavs2gpu_me_session_t *s) { return s && s->impl.d_tmap ? 1 : 0; }
extern "C" void *xavs2gpu_me_stream(xavs2gpu_me_session_t *s) { return s ? (void *)s->impl.st : nullptr; }

extern "C" void xavs2gpu_me_plan_stats(xavs2gpu_me_session_t *s, int *n_ctu_pus, int *n_generic_pus, int *n_ctu_jobs)
{
    if (!s) return;
    if (n_ctu_pus) *n_ctu_pus = s->impl.n_ctu_pus;
    if (n_generic_pus) *n_generic_pus = s->impl.n_generic;
    if (n_ctu_jobs) *n_ctu_jobs = s->impl.plan.n_jobs;
}

// ---- several sessions per launch ------------------------------------------------
extern "C" int xavs2gpu_me_set_stream(xavs2gpu_me_session_t *s, void *stream)
{
    if (!s) return XAVS2GPU_ERR_ARG;
    MeSessionImpl &m = s->impl;
    m.st = stream ? (cudaStream_t)stream : m.own_st;
    return XAVS2GPU_OK;
}

extern "C" const uint8_t *const *xavs2gpu_me_plane_table_device(xavs2gpu_me_session_t *s)
{
    return s ? (const uint8_t *const *)(s->impl.d_plane_ptrs + 1) : nullptr;
}

// Rotates the reference tables on the device (stream-ordered, no host
// staging): reference r takes reference r-1's planes, reference 0 the last's.
__global__ void rotate_tables_kernel(uint8_t **plane_ptrs, const uint8_t **ref0, int nrefs)
{
    const int k = threadIdx.x;   // one thread per sub-pel position, 16 threads
    uint8_t *last = plane_ptrs[1 + 16 * (nrefs - 1) + k];
    for (int r = nrefs - 1; r > 0; r--) plane_ptrs[1 + 16 * r + k] = plane_ptrs[1 + 16 * (r - 1) + k];
    plane_ptrs[1 + k] = last;
    __syncthreads();
    if (k == 0)
        for (int r = 0; r < nrefs; r++) ref0[r] = plane_ptrs[1 + 16 * r];
}

extern "C" int xavs2gpu_me_rotate_refs(xavs2gpu_me_session_t *s)
{
    if (!s) return XAVS2GPU_ERR_ARG;
    MeSessionImpl &m = s->impl;
    XG_CUDA(cudaSetDevice(m.device));
    const int last = m.slot_buf[m.nrefs - 1];
    for (int r = m.nrefs - 1; r > 0; r--) m.slot_buf[r] = m.slot_buf[r - 1];
    m.slot_buf[0] = last;
    rotate_tables_kernel<<<1, 16, 0, m.st>>>(m.d_plane_ptrs, m.d_ref0, m.nrefs);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

struct BatchBuf {
    CtuJob *d_jobs = nullptr;
    uint32_t *d_lists = nullptr;    // generic | small | large | group members
    SessView *d_views = nullptr;
    RefineGroup *d_groups = nullptr;
    size_t cap_jobs = 0, cap_lists = 0, cap_views = 0, cap_groups = 0;
    uint8_t *h_stage = nullptr;     // pinned: jobs | lists | views (uploads without a stream wait)
    size_t cap_stage = 0;
    cudaEvent_t done = nullptr;
    bool used = false;
};

struct xavs2gpu_me_batch {
    int device = 0;
    BatchBuf buf[2];
    int next = 0;
};

extern "C" xavs2gpu_me_batch_t *xavs2gpu_me_batch_create(void)
{
    auto *b = new xavs2gpu_me_batch();
    b->device = current_device();
    for (auto &x : b->buf) XG_CUDA(cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming));
    // the batch buffers grow with stream-ordered allocations: keep freed
    // blocks in the device's pool
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, b->device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return b;
}

extern "C" void xavs2gpu_me_batch_destroy(xavs2gpu_me_batch_t *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    for (auto &x : b->buf) {
        if (x.used) cudaEventSynchronize(x.done);
        cudaEventDestroy(x.done);
        cudaFree(x.d_jobs); cudaFree(x.d_lists); cudaFree(x.d_views); cudaFree(x.d_groups); cudaFreeHost(x.h_stage);
    }
    delete b;
}

// Stream-ordered growth of a batch buffer: no device-wide synchronisation
// (the buffer's previous launch has completed: its done event was waited
// for), freed blocks stay in the device's pool.
template <typename T>
static void grow(T *&p, size_t &cap, size_t need, cudaStream_t st)
{
    if (need <= cap) return;
    if (p) XG_CUDA(cudaFreeAsync(p, st));
    cap = need + need / 2 + 64;
    XG_CUDA(cudaMallocAsync((void **)&p, sizeof(T) * cap, st));
}

extern "C" int xavs2gpu_me_batch_run(xavs2gpu_me_batch_t *b, xavs2gpu_me_session_t *const *sessions, int n,
                                     const xavs2gpu_me_params_t *prm, void *stream)
{
    if (!b || !sessions || n < 0 || n > 256 || !prm || prm->search_range < 1 || prm->search_range > 128 ||
        prm->fractional_me < 0 || prm->fractional_me > 2 || prm->lambda_factor < 0) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_batch_run", "bad parameters or more than 256 sessions");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    XG_CUDA(cudaSetDevice(b->device));
    const int R = prm->search_range, lam = prm->lambda_factor;
    cudaStream_t st = (cudaStream_t)stream;
    // pass 1: plans and sizes
    const bool grouped = !prm->enable_pmvr && use_groups();
    size_t nj = 0, ng = 0, ns = 0, nl = 0, nm = 0, nheavy = 0, ngr = 0;
    int nborder = 0;
    int block = 128;
    for (int k = 0; k < n; k++) {
        MeSessionImpl &m = sessions[k]->impl;
        if (m.device != b->device) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_batch_run", "sessions on different devices");
            return XAVS2GPU_ERR_ARG;
        }
        ensure_plan(m, R, prm->lambda_factor);
        const bool g = grouped && m.cu_groups;
        nj += m.plan.h_jobs.size();
        nborder += m.plan.n_border;
        ng += m.h_generic.size();
        ns += g ? m.h_small_g.size() : m.h_small.size();
        nl += g ? m.h_large_g.size() : m.h_large.size();
        if (g) {
            nm += m.h_members.size();
            nheavy += (size_t)m.n_heavy;
            ngr += (size_t)m.n_groups;
        }
        if (k == 0) block = m.tune_block;
    }
    BatchBuf &bb = b->buf[b->next];
    b->next ^= 1;
    if (bb.used) XG_CUDA(cudaEventSynchronize(bb.done));   // its staging and lists may still be read
    const size_t nlist = ng + ns + nl + nm;
    grow(bb.d_jobs, bb.cap_jobs, nj, st);
    grow(bb.d_lists, bb.cap_lists, nlist, st);
    grow(bb.d_views, bb.cap_views, (size_t)n, st);
    grow(bb.d_groups, bb.cap_groups, ngr, st);
    const size_t bj = sizeof(CtuJob) * nj, bl = sizeof(uint32_t) * nlist;
    const size_t bv = sizeof(SessView) * n, bg = sizeof(RefineGroup) * ngr;
    const size_t oj = 0, ol = align_up(bj), ov = ol + align_up(bl), og = ov + align_up(bv), need = og + align_up(bg);
    if (need > bb.cap_stage) {
        cudaFreeHost(bb.h_stage);
        bb.cap_stage = need + need / 2 + 4096;
        XG_CUDA(cudaMallocHost((void **)&bb.h_stage, bb.cap_stage));
    }
    // pass 2: written straight into the pinned staging buffer, list entries
    // tagged with their session's index in this launch; groups of 32x32 and
    // 64x64 CUs first (longest work first)
    CtuJob *J = reinterpret_cast<CtuJob *>(bb.h_stage + oj);
    uint32_t *Lg = reinterpret_cast<uint32_t *>(bb.h_stage + ol), *Ls = Lg + ng, *Ll = Ls + ns, *Lm = Ll + nl;
    SessView *V = reinterpret_cast<SessView *>(bb.h_stage + ov);
    RefineGroup *Gh = reinterpret_cast<RefineGroup *>(bb.h_stage + og), *Gl = Gh + nheavy;
    uint32_t mbase = 0;
    auto put = [](uint32_t *&dst, const std::vector<uint32_t> &src, uint32_t tag) {
        const uint32_t *p = src.data();
        const size_t c = src.size();
        for (size_t i = 0; i < c; i++) dst[i] = tag | p[i];
        dst += c;
    };
    for (int k = 0; k < n; k++) {
        MeSessionImpl &m = sessions[k]->impl;
        const bool g = grouped && m.cu_groups;
        const uint32_t tag = (uint32_t)k << kSessShift;
        V[k] = m.h_view;
        for (const CtuJob &j0 : m.plan.h_jobs) {
            *J = j0;
            J->sess = (uint8_t)k;
            J++;
        }
        put(Lg, m.h_generic, tag);
        put(Ls, g ? m.h_small_g : m.h_small, tag);
        put(Ll, g ? m.h_large_g : m.h_large, tag);
        if (g) {
            for (int q = 0; q < m.n_groups; q++) {
                RefineGroup d = m.h_groups[q];
                d.first += mbase;
                *(q < m.n_heavy ? Gh++ : Gl++) = d;
            }
            put(Lm, m.h_members, tag);
            mbase += (uint32_t)m.h_members.size();
        }
    }
    if (bj) XG_CUDA(cudaMemcpyAsync(bb.d_jobs, bb.h_stage + oj, bj, cudaMemcpyHostToDevice, st));
    if (bl) XG_CUDA(cudaMemcpyAsync(bb.d_lists, bb.h_stage + ol, bl, cudaMemcpyHostToDevice, st));
    XG_CUDA(cudaMemcpyAsync(bb.d_views, bb.h_stage + ov, bv, cudaMemcpyHostToDevice, st));
    if (bg) XG_CUDA(cudaMemcpyAsync(bb.d_groups, bb.h_stage + og, bg, cudaMemcpyHostToDevice, st));
    const uint32_t *d_gen = bb.d_lists, *d_small = bb.d_lists + ng, *d_large = bb.d_lists + ng + ns;
    const uint32_t *d_members = bb.d_lists + ng + ns + nl;
    reset_keys_kernel<<<sm_count() * 4, 256, 0, st>>>(bb.d_views, n);
    count_launch();
    if (ng) {
        me_init_list_kernel<<<(unsigned)((ng * 32 + 127) / 128), 128, 0, st>>>(d_gen, (int)ng, bb.d_views, lam);
        count_launch();
    }
    CtuSide *gside = nullptr;
    const cudaStream_t gst = search_fork(st, ng && nj, gside);
    if (gside) {
        const int rc = fs_generic_launch(d_gen, (int)ng, bb.d_views, R, lam, gst);
        if (rc != XAVS2GPU_OK) {
            refine_join(st, gside);
            return rc;
        }
    }
    ctu_jobs_run(bb.d_jobs, (int)nj, nborder, bb.d_views, *prm, st);
    if (!gside && ng) {
        const int rc = fs_generic_launch(d_gen, (int)ng, bb.d_views, R, lam, st);
        if (rc != XAVS2GPU_OK) return rc;
    }
    refine_join(st, gside);
    if (ngr) launch_groups(bb.d_groups, (int)ngr, d_members, bb.d_views, R, *prm, st);
    CtuSide *side = nullptr;
    const cudaStream_t wst = refine_fork(st, ns && nl, side);
    if (ns) {
        const unsigned g = (unsigned)((ns + block - 1) / block);
        if (prm->use_hadamard)
            refine_thread_kernel<true><<<g, block, 0, st>>>(d_small, (int)ns, bb.d_views, R, *prm);
        else
            refine_thread_kernel<false><<<g, block, 0, st>>>(d_small, (int)ns, bb.d_views, R, *prm);
        count_launch();
    }
    if (nl) {
        refine_warp_list_kernel<<<(unsigned)((nl * 32 + block - 1) / block), block, 0, wst>>>(d_large, (int)nl,
                                                                                           bb.d_views, R, *prm);
        count_launch();
    }
    refine_join(st, side);
    XG_CUDA(cudaEventRecord(bb.done, st));
    bb.used = true;
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

// ---- allocation-free search ------------------------------------------------------
// For callers that cannot allocate device memory while they run: an encoder
// embedded in a host process whose GPU memory is handed out by the host's
// own pool, or a latency-critical encoder thread that must not trigger the
// device-wide synchronisation cudaMalloc/cudaFree imply.  The search's
// scratch (per-PU keys and state, a sanitised copy of the PU list, the plane
// pointer table) lives in one file-scope device array instead of session
// buffers.  Every call shares it, so calls that overlap on the GPU race; the
// array keeps the last call's contents, and every byte a call reads is
// written by that call first, so nothing needs clearing.
namespace xg {

constexpr int kNoAllocMaxPus = 65536;
constexpr int kNoAllocMaxRefs = 16;

struct NoAllocScratch {
    unsigned long long keys[kNoAllocMaxPus];
    PuState state[kNoAllocMaxPus];
    xavs2gpu_pu_t pus[kNoAllocMaxPus];
    int list[kNoAllocMaxPus];
    const uint8_t *planes[16 * kNoAllocMaxRefs];
    const uint8_t *ref0[kNoAllocMaxRefs];
    SessView view;            // the call as the list kernels see it
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

struct PlaneTable { const uint8_t *p[16 * kNoAllocMaxRefs]; };

// Copies the PU list into the scratch; a PU outside the picture, with a bad
// shape or reference, or with limits reaching beyond the 80-pixel margin is
// replaced by one that has no admissible candidate, so it is never searched
// and reports bcost = 1 << 30.  Also writes the plane tables and the index list.
__global__ void noalloc_prepare_kernel(const xavs2gpu_pu_t *__restrict__ in, int n, NoAllocScratch *s, PlaneTable t,
                                       int nrefs, int W, int H, const uint8_t *cur, int stride,
                                       xavs2gpu_me_result_t *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        for (int k = 0; k < 16 * nrefs; k++) s->planes[k] = t.p[k];
        for (int r = 0; r < nrefs; r++) s->ref0[r] = t.p[16 * r];
        SessView v;
        v.cur = cur;
        v.ref0 = s->ref0;
        v.planes = s->planes;
        v.pus = s->pus;
        v.state = s->state;
        v.keys = s->keys;
        v.res = out;
        v.slots = nullptr;
        v.g = Geometry{W, H, stride};
        v.n = n;
        v.tmap = nullptr;
        v.pool = nullptr;
        v.plane_bytes = 0;
        v.wait_flag = nullptr;
        s->view = v;
    }
    if (i >= n) return;
    xavs2gpu_pu_t p = in[i];
    bool ok = (unsigned)p.part < (unsigned)kNumParts && (unsigned)p.ref < (unsigned)nrefs;
    if (ok) {
        const int w = c_pu_w[p.part], h = c_pu_h[p.part];
        ok = p.x >= 0 && p.y >= 0 && p.x + w <= W && p.y + h <= H && p.min_x >= -kPad + 8 - p.x &&
             p.max_x <= W + kPad - 8 - p.x - w && p.min_y >= -kPad + 8 - p.y && p.max_y <= H + kPad - 8 - p.y - h;
    }
    if (!ok) {
        p.x = p.y = 0;
        p.part = 0;
        p.ref = 0;
        p.mvp_x = p.mvp_y = 0;
        p.min_x = p.min_y = 1;   // min > max: no candidate is admissible
        p.max_x = p.max_y = 0;
    }
    s->pus[i] = p;
    s->list[i] = i;
}

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static NoAllocScratch *g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch array on `dev` (the current device), looked
// up once per device.  The cached address stays valid until the device is
// reset (cudaDeviceReset); the library is not meant to outlive a reset.
static NoAllocScratch *noalloc_scratch(int dev)
{
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_search_noalloc", "device ordinal beyond the 64 the scratch table covers");
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            fail(XAVS2GPU_ERR_CUDA, "xavs2gpu_me_search_noalloc: cudaGetSymbolAddress", cudaGetErrorString(e));
            return nullptr;
        }
        g_noalloc_addr[dev] = static_cast<NoAllocScratch *>(ptr);
    }
    return g_noalloc_addr[dev];
}

}  // namespace xg

extern "C" int xavs2gpu_me_search_noalloc(const uint8_t *cur, int stride, int width, int height,
                                          const uint8_t *const *ref_planes, int num_refs,
                                          const xavs2gpu_pu_t *pus, int n, const xavs2gpu_me_params_t *prm,
                                          xavs2gpu_me_result_t *out, void *stream)
{
    if (n < 0 || n > kNoAllocMaxPus || num_refs < 1 || num_refs > kNoAllocMaxRefs) {
        fail(XAVS2GPU_ERR_CAPACITY, "xavs2gpu_me_search_noalloc",
             "at most 65536 PUs and 16 references per call (the fixed scratch size)");
        return XAVS2GPU_ERR_CAPACITY;
    }
    if (!cur || !ref_planes || !prm || (n > 0 && (!pus || !out)) || width < 8 || height < 8 ||
        stride < width + 2 * kPad || prm->search_range < 1 || prm->search_range > 128 || prm->fractional_me < 0 ||
        prm->fractional_me > 2 || prm->lambda_factor < 0) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_search_noalloc", "bad picture geometry, pointers or parameters");
        return XAVS2GPU_ERR_ARG;
    }
    PlaneTable t;
    memset(&t, 0, sizeof(t));
    for (int k = 0; k < 16 * num_refs; k++) {
        if (!ref_planes[k]) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_me_search_noalloc", "missing reference plane");
            return XAVS2GPU_ERR_ARG;
        }
        t.p[k] = ref_planes[k];
    }
    if (n == 0) return XAVS2GPU_OK;
    int dev = 0;
    XG_CUDA(cudaGetDevice(&dev));
    NoAllocScratch *s = noalloc_scratch(dev);
    if (!s) return xavs2gpu_get_status();
    cudaStream_t st = (cudaStream_t)stream;
    const Geometry g{width, height, stride};
    const int R = prm->search_range, lam = prm->lambda_factor;
    noalloc_prepare_kernel<<<(n + 255) / 256, 256, 0, st>>>(pus, n, s, t, num_refs, width, height, cur, stride, out);
    me_init_kernel<<<(n * 32 + 127) / 128, 128, 0, st>>>(s->pus, n, cur, s->ref0, g, lam, s->state, s->keys);
    const int rc = fs_generic_launch(reinterpret_cast<const uint32_t *>(s->list), n, &s->view, R, lam, st);
    if (rc != XAVS2GPU_OK) return rc;
    refine_kernel<<<(n * 32 + 127) / 128, 128, 0, st>>>(s->pus, n, s->state, s->keys, cur, s->planes, g, R, *prm,
                                                        out);
    count_launch(3);
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
