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

// Plane-mode multiplier and shift per log2 block side 2..6 (intra.c:194-195)
__device__ __forceinline__ int plane_mult(int l) { return (int)((0x170B05110DULL >> (8 * (l - 2))) & 0xFF); }
__device__ __forceinline__ int plane_shift(int l) { return (int)((0x130F0B0A07ULL >> (8 * (l - 2))) & 0xFF); }

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
        const int lx = ilog2d(bsx), ly = ilog2d(bsy), w2 = bsx >> 1, h2 = bsy >> 1;
        int H = 0, V = 0;
        for (int i = lane + 1; i <= w2; i += 32) H += i * (ep[w2 + i] - ep[w2 - i]);
        for (int i = lane + 1; i <= h2; i += 32) V += i * (ep[-h2 - i] - ep[-h2 + i]);
        H = warp_sum(H);
        V = warp_sum(V);
        k.pb = ((H << 5) * plane_mult(lx) + (1 << (plane_shift(lx) - 1))) >> plane_shift(lx);
        k.pc = ((V << 5) * plane_mult(ly) + (1 << (plane_shift(ly) - 1))) >> plane_shift(ly);
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

// ---- batched rough mode decision ---------------------------------------------
// Blocks are sorted by shape class ((log2 w - 2) * 5 + log2 h - 2); a CTA
// takes a tile of G blocks of one class and all 33 modes.  A warp handles
// one mode at a time for the whole tile, so its branches are uniform: a lane
// owns one SATD unit (8x4, or 4x4 for width-4 blocks) of one block, predicts
// it in registers straight from the edge samples and scores it; the lanes of
// a block then sum their units with shuffles.  Every prediction tap is a
// 4-sample window of the edge array (in ascending address order for all
// directions) taken with a funnel shift and weighted with one dp4a.
constexpr int kN = 9;             // INTRA_MODE_NUM_FOR_RDO (defines.h:290)
constexpr int kTW = 11;           // warps per CTA: 3 modes each
constexpr int kTT = kTW * 32;
constexpr int kCls = 25;
// max over classes of G * (align4(edge window) + 4: the window's offset in
// its first word), plus word-read slack
constexpr int kEdgeArea = 2112;

struct Geo {
    int w, h, uw, nux, lanes, iters, G, lo, hi, R;
};
__host__ __device__ __forceinline__ int side_log(int v)
{
    return v == 4 ? 0 : v == 8 ? 1 : v == 16 ? 2 : v == 32 ? 3 : v == 64 ? 4 : -1;
}
__host__ __device__ __forceinline__ Geo geo_of(int c)
{
    Geo g;
    g.w = 4 << (c / 5);
    g.h = 4 << (c % 5);
    g.uw = g.w == 4 ? 4 : 8;   // satd_unit4 (pixel.c:354-407)
    g.nux = g.w / g.uw;
    const int units = g.nux * (g.h >> 2);
    g.lanes = units < 32 ? units : 32;
    g.iters = units / g.lanes;
    g.G = 32 / g.lanes;
    g.lo = edge_below(g.w, g.h);
    g.hi = edge_above(g.w, g.h);
    g.R = (g.lo + g.hi + 1 + 3) & ~3;
    return g;
}

// Two tile buffers: the next tile is copied in (cp.async) while the warps
// score the current one.
struct TileBuf {
    uint8_t edge[kEdgeArea];          // block b: the words holding edge samples -lo..hi at b * (R + 4)
    uint8_t fenc[4096 + 64];          // block b: w x h source samples at b * (w * h + 4)
    int64_t eoff[32], foff[32];
    int idx[32], dc_avail[32], mpm[32][2];
    int emis[32];                     // byte offset of sample -lo in its first word
};
struct TileSmem {
    TileBuf buf[2];
    int satd[32][33];
    int next_mode;
    int tile_base[kCls + 1], order[kCls], start[kCls], count[kCls];
};

__device__ __forceinline__ void cp_async4(void *dst_smem, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Modes in the order warps take them: the per-sample two-edge modes first,
// then the one-edge angles, then the cheap ones (longest work first).
__constant__ int8_t c_mode_order[33] = {13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 3, 4, 5, 6, 7, 8,
                                        9,  10, 11, 25, 26, 27, 28, 29, 30, 31, 32, 2, 1, 0, 12, 24};

// Per-lane constants of the non-angular modes for the lane's block
struct LaneConst {
    int dc, pa, pb, pc, bt;
};

// 4 edge samples p[0..3] as one word (any byte alignment)
__device__ __forceinline__ uint32_t win4(const uint8_t *p)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
    return __funnelshift_r(w[0], w[1], (unsigned)(a & 3) * 8u);
}
__device__ __forceinline__ uint32_t wts(int b0, int b1, int b2, int b3)
{
    return (uint32_t)b0 | ((uint32_t)b1 << 8) | ((uint32_t)b2 << 16) | ((uint32_t)b3 << 24);
}
__device__ __forceinline__ int tap(const uint8_t *ep, int s, uint32_t w)
{
    return (int)(__dp4a(win4(ep + s), w, 64u) >> 7);
}

// Hadamard sum of a 4x4 difference block held in registers
__device__ __forceinline__ int hsum4_reg(int (&d)[4][4])
{
#pragma unroll
    for (int r = 0; r < 4; r++) fwht4_d(d[r][0], d[r][1], d[r][2], d[r][3]);
    int s = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        fwht4_d(d[0][c], d[1][c], d[2][c], d[3][c]);
        s += iabs_d(d[0][c]) + iabs_d(d[1][c]) + iabs_d(d[2][c]) + iabs_d(d[3][c]);
    }
    return s;
}

// |H (src - pred) H^T| of the 4x4 sub-block at (x0, y0) of a block in `mode`
__device__ __forceinline__ int sub4_hsum(int mode, const uint8_t *ep, const uint8_t *fb, int fstride, const Geo &g,
                                         int x0, int y0, const LaneConst &kc, bool narrow5, bool narrow31)
{
    int p[4][4];
    if (mode == 0) {
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) p[r][c] = kc.dc;
    } else if (mode == 1) {
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) p[r][c] = min(max((kc.pa + kc.pb * (x0 + c) + kc.pc * (y0 + r)) >> 5, 0), 255);
    } else if (mode == 2) {
        const int lx = ilog2d(g.w), ly = ilog2d(g.h), a = ep[g.w], b = ep[-g.h];
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int x = x0 + c, y = y0 + r, top = ep[1 + x], left = ep[-1 - y];
                const int predx = (left << lx) + (x + 1) * (a - left);
                const int predy = (top << ly) + (y + 1) * (b - top);
                const int v = ((predx << ly) + (predy << lx) + x * y * kc.bt + (1 << (lx + ly))) >> (lx + ly + 1);
                p[r][c] = min(max(v, 0), 255);
            }
    } else if (mode == 12) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int v = ep[1 + x0 + c];
#pragma unroll
            for (int r = 0; r < 4; r++) p[r][c] = v;
        }
    } else if (mode == 24) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int v = ep[-1 - y0 - r];
#pragma unroll
            for (int c = 0; c < 4; c++) p[r][c] = v;
        }
    } else if (narrow5 || narrow31) {
        // the reference's tabulated mode-5 / mode-31 variants (intra.c:455-605, 1147-1161)
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++)
                p[r][c] = narrow5 ? mode5_narrow([ep](int i) { return (int)ep[i]; }, x0 + c, y0 + r, g.w)
                                  : mode5_narrow([ep](int i) { return (int)ep[-i]; }, y0 + r, x0 + c, g.h);
    } else if (mode < 12) {
        // from the top row: row y reads ep[ix .. ix + 3], ix = step + x
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int f;
            const int ix = ang_step(mode, 0, y0 + r + 1, f) + x0;
            const uint32_t w = wts(32 - f, 64 - f, 32 + f, f);
#pragma unroll
            for (int c = 0; c < 4; c++) p[r][c] = tap(ep, ix + c, w);
        }
    } else if (mode > 24) {
        // from the left column: column x reads ep[-iy - 3 .. -iy], iy = y + step
#pragma unroll
        for (int c = 0; c < 4; c++) {
            int f;
            const int iy = ang_step(mode, 1, x0 + c + 1, f) + y0;
            const uint32_t w = wts(f, 32 + f, 64 - f, 32 - f);
#pragma unroll
            for (int r = 0; r < 4; r++) p[r][c] = tap(ep, -iy - r - 3, w);
        }
    } else {
        // both edges (intra.c:363-397)
        int sx[4], sy[4];
        uint32_t wx[4], wy[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int f;
            sx[r] = ang_step(mode, 0, y0 + r + 1, f);
            wx[r] = wts(f, 32 + f, 64 - f, 32 - f);
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
            int f;
            sy[c] = ang_step(mode, 1, x0 + c + 1, f);
            wy[c] = wts(32 - f, 64 - f, 32 + f, f);
        }
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int x = x0 + c, y = y0 + r, iyy = y - sy[c];
                p[r][c] = iyy <= -1 ? tap(ep, x - sx[r] - 1, wx[r]) : tap(ep, -iyy - 2, wy[c]);
            }
    }
    int d[4][4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const uint32_t f = *reinterpret_cast<const uint32_t *>(fb + (y0 + r) * fstride + x0);
#pragma unroll
        for (int c = 0; c < 4; c++) d[r][c] = (int)((f >> (8 * c)) & 0xFFu) - p[r][c];
    }
    return hsum4_reg(d);
}

// SAD of the same sub-block (use_hadamard = 0)
__device__ __forceinline__ int sub4_sad(int mode, const uint8_t *ep, const uint8_t *fb, const Geo &g, int x0, int y0,
                                        const ModeConst &k)
{
    int s = 0;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            s += iabs_d((int)fb[(y0 + r) * g.w + x0 + c] - pred_sample(mode, ep, x0 + c, y0 + r, g.w, g.h, k));
    return s;
}

// update_candidate_list (md_intra.c:195-210): insertion into the 9-entry
// list kept sorted by cost, after equal costs; a cost not below the last
// entry is dropped.  Costs are non-negative doubles, so their bit patterns
// order like the values.  Unrolled over the positions: the list stays in
// registers.
struct CandList {
    long long k[kN];
    int m[kN];
};
__device__ __forceinline__ void cand_insert(CandList &L, int mode, long long key)
{
#pragma unroll
    for (int i = kN - 1; i >= 0; i--) {
        const bool lt_prev = i > 0 && key < L.k[i > 0 ? i - 1 : 0];
        if (lt_prev) {
            L.k[i] = L.k[i - 1];
            L.m[i] = L.m[i - 1];
        } else if (key < L.k[i]) {
            L.k[i] = key;
            L.m[i] = mode;
        }
    }
}

// The candidate list of rdo_get_pred_intra_luma (all modes) or of the rough
// three-phase search rdo_get_pred_intra_luma_rmd (md_intra.c:258-380),
// replayed on the per-mode costs; returns the number of modes for RDO.
// `vis` / `fin` are the reference's visited[] states 1 / 2 as bit masks.
__device__ __forceinline__ int candidates(const long long *key, int rough, int dist2, int dist1, int num_for_rdo,
                                          int mpm0, int mpm1, CandList &L)
{
    const long long kMax = __double_as_longlong((double)(1LL << 50));   // MAX_COST (defines.h:299)
#pragma unroll
    for (int i = 0; i < kN; i++) {
        L.m[i] = 0;
        L.k[i] = kMax;
    }
    if (!rough) {
        for (int m = 0; m < 33; m++) cand_insert(L, m, key[m]);
        return num_for_rdo;
    }
    uint64_t vis = 0, fin = 0;
    auto visit = [&](int m) {
        cand_insert(L, m, key[m]);
        vis |= 1ull << m;
    };
    auto seen = [&](int m) { return (vis >> m) & 1ull; };
    for (int m = 0; m < 3; m++) visit(m);
    for (int m = 4; m < 33; m += 4) visit(m);
#pragma unroll
    for (int i = 0; i < kN; i++) {
        if (i >= dist2) break;
        const int m = L.m[i];
        if (m <= 2) continue;
        if (m > 3 && !seen(m - 2)) visit(m - 2);
        if (m < 31 && !seen(m + 2)) visit(m + 2);
    }
    int na = 0;
#pragma unroll
    for (int i = 0; i < kN; i++) {
        if (na >= dist1) break;
        const int m = L.m[i];
        if (m <= 2) continue;
        if (m > 3 && !seen(m - 1)) { visit(m - 1); na++; }
        if (m < 32 && !seen(m + 1)) { visit(m + 1); na++; }
    }
    if (!seen(mpm0)) visit(mpm0);
    if (!seen(mpm1)) visit(mpm1);
    if (L.m[0] == mpm0 || L.m[0] == mpm1 || L.m[1] == mpm0 || L.m[1] == mpm1)
        return num_for_rdo < 3 ? num_for_rdo : 3;
    fin |= (1ull << L.m[0]) | (1ull << L.m[1]);
    auto one = [&](int m) { return ((vis >> m) & 1ull) && !((fin >> m) & 1ull); };   // visited == 1
    int j = 2;
#pragma unroll
    for (int i = 2; i < kN; i++) {
        if (j >= num_for_rdo) break;
        const int m = L.m[i];
        if (!seen(m)) continue;
        bool take;
        if (m <= 2) take = true;
        else if (m == 3) take = one(4);
        else if (m == 32) take = one(31);
        else take = one(m - 1) && one(m + 1);
        if (take) {
#pragma unroll
            for (int p = 2; p < kN; p++)
                if (p == j) L.m[p] = m;
            j++;
            fin |= 1ull << m;
        }
        if (((fin & 7ull) == 7ull)) break;
    }
    return num_for_rdo < j ? num_for_rdo : j;
}

__device__ __forceinline__ int block_class(const xavs2gpu_intra_block_t &b)
{
    const int a = side_log(b.width), c = side_log(b.height);
    if (a < 0 || c < 0 || a - c > 2 || c - a > 2) return -1;   // sides 4..64, aspect ratio at most 4
    if (b.mpm[0] < 0 || b.mpm[0] > 32 || b.mpm[1] < 0 || b.mpm[1] > 32) return -1;
    return a * 5 + c;
}

// 1. per-class counts (warp-aggregated atomics); other blocks are reported
__global__ void rmd_count_kernel(const xavs2gpu_intra_block_t *__restrict__ blocks, int n, int *__restrict__ counts,
                                 xavs2gpu_intra_result_t *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1;
    if (i < n) {
        c = block_class(blocks[i]);
        if (c < 0) out[i].num_for_rdo = -1;   // not a block the encoder predicts
    }
    const unsigned valid = __ballot_sync(0xffffffffu, c >= 0);
    if (c >= 0) {
        const unsigned same = __match_any_sync(valid, c);
        if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&counts[c], __popc(same));
    }
}

// 2. scatter into the class-ordered list
__global__ void rmd_scatter_kernel(const xavs2gpu_intra_block_t *__restrict__ blocks, int n,
                                   const int *__restrict__ counts, int *__restrict__ cursor, int *__restrict__ sorted)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int c = i < n ? block_class(blocks[i]) : -1;
    const unsigned valid = __ballot_sync(0xffffffffu, c >= 0);
    if (c < 0) return;
    const unsigned same = __match_any_sync(valid, c);
    const int leader = __ffs(same) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&cursor[c], __popc(same));
    base = __shfl_sync(same, base, leader);
    int start = 0;
    for (int k = 0; k < c; k++) start += counts[k];
    sorted[start + base + __popc(same & ((1u << lane) - 1))] = i;
}

// 3. the tiles, persistent; classes with the most work per tile first
#ifndef XG_RMD_MINB
#define XG_RMD_MINB 3
#endif
__global__ void __launch_bounds__(kTT, XG_RMD_MINB) rmd_tile_kernel(const xavs2gpu_intra_block_t *__restrict__ blocks,
                                                        const int *__restrict__ counts, const int *__restrict__ sorted,
                                                        const uint8_t *__restrict__ edges,
                                                        const uint8_t *__restrict__ fenc, int fenc_stride,
                                                        xavs2gpu_intra_params_t prm,
                                                        xavs2gpu_intra_result_t *__restrict__ out)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    TileSmem &s = *reinterpret_cast<TileSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    (void)warp;
    if (tid == 0) {
        int acc = 0;
        for (int c = 0; c < kCls; c++) {
            s.count[c] = counts[c];
            s.start[c] = acc;
            acc += s.count[c];
        }
        // order: tile work (G * w * h) descending, ties by class
        for (int c = 0; c < kCls; c++) s.order[c] = c;
        for (int i = 1; i < kCls; i++) {
            const int c = s.order[i];
            const Geo gc = geo_of(c);
            const int wc = gc.G * gc.w * gc.h;
            int j = i;
            while (j > 0) {
                const Geo gp = geo_of(s.order[j - 1]);
                if (gp.G * gp.w * gp.h >= wc) break;
                s.order[j] = s.order[j - 1];
                j--;
            }
            s.order[j] = c;
        }
        s.tile_base[0] = 0;
        for (int k = 0; k < kCls; k++) {
            const Geo g = geo_of(s.order[k]);
            s.tile_base[k + 1] = s.tile_base[k] + (s.count[s.order[k]] + g.G - 1) / g.G;
        }
    }
    __syncthreads();
    const int total = s.tile_base[kCls];
    // tile t's class, its first block and its block count
    auto tile_of = [&](int t, int &k, Geo &g, int &first, int &nb) {
        k = 0;
        while (t >= s.tile_base[k + 1]) k++;
        const int c = s.order[k];
        g = geo_of(c);
        first = s.start[c] + (t - s.tile_base[k]) * g.G;
        const int rem = s.start[c] + s.count[c] - first;
        nb = rem < g.G ? rem : g.G;
    };
    // descriptors of tile t into buffer p (threads < nb)
    auto stage_desc = [&](int p, int first, int nb) {
        TileBuf &B = s.buf[p];
        if (tid < nb) {
            const int bi = sorted[first + tid];
            const xavs2gpu_intra_block_t b = blocks[bi];
            B.idx[tid] = bi;
            B.eoff[tid] = b.edge_offset;
            B.foff[tid] = b.fenc_offset;
            B.dc_avail[tid] = b.dc_avail;
            B.mpm[tid][0] = b.mpm[0];
            B.mpm[tid][1] = b.mpm[1];
            B.emis[tid] = (int)((uintptr_t)(edges + b.edge_offset - edge_below(b.width, b.height)) & 3);
        }
    };
    // samples of tile t into buffer p: the edge windows as the aligned words
    // holding them, the source rows as words when they are 4-byte aligned
    // (else bytes); asynchronous copies (cp.async) where possible
    auto stage_data = [&](int p, const Geo &g, int nb) {
        TileBuf &B = s.buf[p];
        const int ew = g.lo + g.hi + 1, RB = g.R + 4;
        const int nw = (ew + 3 + 3) >> 2;   // words covering the window at any offset
        for (int e = tid; e < nb * nw; e += kTT) {
            const int b = e / nw, q = e - b * nw;
            const uint8_t *src = edges + B.eoff[b] - g.lo;
            const uint8_t *w0 = reinterpret_cast<const uint8_t *>((uintptr_t)src & ~(uintptr_t)3);
            cp_async4(B.edge + b * RB + 4 * q, w0 + 4 * q);
        }
        const int area = g.w * g.h, fpitch = area + 4;
        const int lw = ilog2d(g.w);
        bool al = (fenc_stride & 3) == 0;
        for (int b = 0; b < nb; b++) al = al && ((uintptr_t)(fenc + B.foff[b]) & 3) == 0;
        if (al) {
            const int wpr = g.w >> 2, lwr = ilog2d(wpr);
            for (int e = tid; e < nb * (area >> 2); e += kTT) {
                const int b = e / (area >> 2), r = e - b * (area >> 2), y = r >> lwr, x = (r & (wpr - 1)) << 2;
                cp_async4(B.fenc + b * fpitch + (y << lw) + x, fenc + B.foff[b] + (int64_t)y * fenc_stride + x);
            }
        } else {
            for (int e = tid; e < nb * area; e += kTT) {
                const int b = e / area, r = e - b * area, y = r >> lw, x = r & (g.w - 1);
                B.fenc[b * fpitch + r] = fenc[B.foff[b] + (int64_t)y * fenc_stride + x];
            }
        }
    };
    int t = blockIdx.x, p = 0;
    if (t < total) {
        int k, first, nb;
        Geo g;
        tile_of(t, k, g, first, nb);
        stage_desc(0, first, nb);
        __syncthreads();
        stage_data(0, g, nb);
        cp_async_wait_all();
        __syncthreads();
    }
    for (; t < total; t += gridDim.x, p ^= 1) {
        int k, first, nb;
        Geo g;
        tile_of(t, k, g, first, nb);
        TileBuf &B = s.buf[p];
        // the next tile's descriptors, then its samples in flight while this one is scored
        const int tn = t + gridDim.x;
        int kn = 0, firstn = 0, nbn = 0;
        Geo gn;
        if (tn < total) {
            tile_of(tn, kn, gn, firstn, nbn);
            stage_desc(p ^ 1, firstn, nbn);
        }
        if (tid == 0) s.next_mode = 0;
        __syncthreads();
        if (tn < total) stage_data(p ^ 1, gn, nbn);
        const int area = g.w * g.h, fpitch = area + 4;
        // modes, taken by the warps in c_mode_order; a lane per SATD unit
        {
            const int b = lane / g.lanes, u0 = lane - b * g.lanes;
            const bool live = b < nb;
            const int bb = live ? b : 0;
            const uint8_t *ep = B.edge + bb * (g.R + 4) + B.emis[bb] + g.lo;
            const uint8_t *fb = B.fenc + bb * fpitch;
            const int lx = ilog2d(g.w), ly = ilog2d(g.h);
            int mi = 0;
            if (lane == 0) mi = atomicAdd(&s.next_mode, 1);
            mi = __shfl_sync(0xffffffffu, mi, 0);
            while (mi < 33) {
                const int mode = c_mode_order[mi];
                LaneConst kc{0, 0, 0, 0, 0};
                if (mode == 0) {                       // DC (intra.c:153-190)
                    int sl = 0, sa = 0;
                    for (int i = u0; i < g.h; i += g.lanes) sl += ep[-1 - i];
                    for (int i = u0; i < g.w; i += g.lanes) sa += ep[1 + i];
                    for (int o = g.lanes >> 1; o > 0; o >>= 1) {
                        sl += __shfl_xor_sync(0xffffffffu, sl, o);
                        sa += __shfl_xor_sync(0xffffffffu, sa, o);
                    }
                    const int top = B.dc_avail[bb] >> 8, left = B.dc_avail[bb] & 0xFF;
                    if (top && left) kc.dc = ((sl + sa + ((g.w + g.h) >> 1)) * (512 / (g.w + g.h))) >> 9;
                    else if (left) kc.dc = (sl + (g.h >> 1)) >> ly;
                    else if (top) kc.dc = (sa + (g.w >> 1)) >> lx;
                    else kc.dc = 128;
                } else if (mode == 1) {                // plane (intra.c:192-236)
                    const int w2 = g.w >> 1, h2 = g.h >> 1;
                    int H = 0, V = 0;
                    for (int i = u0 + 1; i <= w2; i += g.lanes) H += i * (ep[w2 + i] - ep[w2 - i]);
                    for (int i = u0 + 1; i <= h2; i += g.lanes) V += i * (ep[-h2 - i] - ep[-h2 + i]);
                    for (int o = g.lanes >> 1; o > 0; o >>= 1) {
                        H += __shfl_xor_sync(0xffffffffu, H, o);
                        V += __shfl_xor_sync(0xffffffffu, V, o);
                    }
                    kc.pb = ((H << 5) * plane_mult(lx) + (1 << (plane_shift(lx) - 1))) >> plane_shift(lx);
                    kc.pc = ((V << 5) * plane_mult(ly) + (1 << (plane_shift(ly) - 1))) >> plane_shift(ly);
                    kc.pa = ((ep[-g.h] + ep[g.w]) << 4) + 16 - kc.pb * (w2 - 1) - kc.pc * (h2 - 1);
                } else if (mode == 2) {                // bilinear (intra.c:238-293)
                    const int a = ep[g.w], bl = ep[-g.h], sh = min(lx, ly);
                    const int cc = g.w == g.h ? (a + bl + 1) >> 1
                                              : (((a << lx) + (bl << ly)) * 13 + (1 << (sh + 5))) >> (sh + 6);
                    kc.bt = 2 * cc - a - bl;
                }
                const bool n5 = mode == 5 && ((g.w == 4 && g.h == 16) || (g.w == 8 && g.h == 32));
                const bool n31 = mode == 31 && ((g.w == 16 && g.h == 4) || (g.w == 32 && g.h == 8));
                int acc = 0;
                if (live) {
                    for (int it = 0; it < g.iters; it++) {
                        const int u = u0 + it * g.lanes, uq = u / g.nux;
                        const int uy = uq * 4, ux = (u - uq * g.nux) * g.uw;
                        int hs = 0;
                        if (prm.use_hadamard) {
#pragma unroll 1
                            for (int x0 = ux; x0 < ux + g.uw; x0 += 4)
                                hs += sub4_hsum(mode, ep, fb, g.w, g, x0, uy, kc, n5, n31);
                            acc += hs >> 1;
                        } else {
                            ModeConst k{};
                            k.dc = kc.dc; k.pa = kc.pa; k.pb = kc.pb; k.pc = kc.pc; k.bt = kc.bt;
                            k.ba = ep[g.w]; k.bb = ep[-g.h]; k.lx = lx; k.ly = ly;
                            for (int r = 0; r < 4; r++)
                                for (int x = ux; x < ux + g.uw; x++)
                                    acc += iabs_d((int)fb[(uy + r) * g.w + x] - pred_sample(mode, ep, x, uy + r, g.w, g.h, k));
                        }
                    }
                }
                for (int o = g.lanes >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (live && u0 == 0) s.satd[b][mode] = acc;
                if (lane == 0) mi = atomicAdd(&s.next_mode, 1);
                mi = __shfl_sync(0xffffffffu, mi, 0);
            }
        }
        cp_async_wait_all();   // the next tile's samples have landed
        __syncthreads();
        // costs: lambda * mode bits + distortion as rdcost_t (md_intra.c:216-226)
        for (int e = tid; e < nb * 33; e += kTT) {
            const int b = e / 33, m = e - b * 33;
            const int bits = (B.mpm[b][0] == m || B.mpm[b][1] == m) ? 2 : 6;
            out[B.idx[b]].cost[m] = __dadd_rn(__dmul_rn(prm.lambda, (double)bits), (double)s.satd[b][m]);
        }
        __syncthreads();   // this buffer is refilled two tiles on
    }
}

// 4. the candidate lists, a thread per block
__global__ void __launch_bounds__(128) rmd_cand_kernel(const xavs2gpu_intra_block_t *__restrict__ blocks, int n,
                                                        xavs2gpu_intra_params_t prm,
                                                        xavs2gpu_intra_result_t *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const xavs2gpu_intra_block_t b = blocks[i];
    if (block_class(b) < 0) return;
    xavs2gpu_intra_result_t &r = out[i];
    long long key[33];
#pragma unroll
    for (int m = 0; m < 33; m++) key[m] = __double_as_longlong(r.cost[m]);
    CandList L;
    const int nr = candidates(key, prm.rough, prm.dist2, prm.dist1, b.num_for_rdo, b.mpm[0], b.mpm[1], L);
    r.num_for_rdo = nr;
#pragma unroll
    for (int k = 0; k < kN; k++) {
        r.cand_mode[k] = L.m[k];
        r.cand_cost[k] = __longlong_as_double(L.k[k]);
    }
}

// ---- edge samples of a batch of blocks from one reconstructed picture ---------------
// fill_reference_samples_{0,x,y,xy} (intra.c:1580-1860) as the encoder calls
// them (fill_ref_samples_luma, md_intra.c:137-160) with every neighbour sample
// in the picture.  The sides a block may use are the availability bits that
// lie inside the picture (the picture-bounds half of is_block_available,
// md_intra.c:44-56); a side claimed outside it is treated as missing.
__device__ __forceinline__ int usable_sides(int avail, int x, int y, int bsx, int bsy, int width, int height)
{
    const bool l = x >= 1 && y >= 0 && y + bsy <= height, t = y >= 1 && x >= 0 && x + bsx <= width;
    int ok = 0;
    if (l) ok |= 1 << 0;
    if (t) ok |= 1 << 1;
    if (l && y + 2 * bsy <= height) ok |= 1 << 2;   // left-down
    if (t && x + 2 * bsx <= width) ok |= 1 << 3;    // top-right
    if (l && t) ok |= 1 << 4;                       // top-left
    return avail & ok;
}

// A warp per block writes ep[-edge_below .. edge_above]: the top row and
// top-right run (the last top sample repeated when the top-right is
// missing), the left column and left-down run likewise, 128 for a missing
// side, the corner from the top-left, else the first top, else the first
// left sample, and the padding beyond 2 * bsx / 2 * bsy repeating the run's
// last sample.
__global__ void __launch_bounds__(256) fill_edges_kernel(const xavs2gpu_intra_edge_job_t *__restrict__ jobs, int n,
                                                         const uint8_t *__restrict__ pic, int stride, int width,
                                                         int height, uint8_t *__restrict__ edges, long long edges_size)
{
    const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= n) return;
    const xavs2gpu_intra_edge_job_t j = jobs[w];
    const int bsx = j.width, bsy = j.height, a = side_log(bsx), c = side_log(bsy);
    if (a < 0 || c < 0 || a - c > 2 || c - a > 2) return;
    const int lo = edge_below(bsx, bsy), hi = edge_above(bsx, bsy);
    if (j.edge_offset < lo || j.edge_offset > edges_size - 1 - hi) return;
    const int av = usable_sides(j.avail, j.x, j.y, bsx, bsy, width, height);
    const bool L = av & 1, T = av & 2, LD = av & 4, TR = av & 8, TL = av & 16;
    const long long row = (long long)(j.y - 1) * stride + j.x - 1;   // the corner's position
    uint8_t *ep = edges + j.edge_offset;
    for (int k = -lo + lane; k <= hi; k += 32) {
        int v = 128;
        if (k > 0) {
            const int kk = min(k, 2 * bsx);
            if (kk <= bsx) {
                if (T) v = pic[row + kk];
            } else if (TR) {
                v = pic[row + kk];
            } else if (T) {
                v = pic[row + bsx];
            }
        } else if (k < 0) {
            const int jj = min(-k, 2 * bsy);
            if (jj <= bsy) {
                if (L) v = pic[row + (long long)jj * stride];
            } else if (LD) {
                v = pic[row + (long long)jj * stride];
            } else if (L) {
                v = pic[row + (long long)bsy * stride];
            }
        } else {
            v = TL ? pic[row] : T ? pic[row + 1] : L ? pic[row + stride] : 128;
        }
        ep[k] = (uint8_t)v;
    }
}

}  // namespace intra
}  // namespace xg

using namespace xg;

extern "C" int xavs2gpu_intra_fill_edges(const xavs2gpu_intra_edge_job_t *jobs, int n, const uint8_t *pic, int stride,
                                         int width, int height, uint8_t *edges, int64_t edges_size, void *stream)
{
    if (n < 0 || width < 1 || height < 1 || stride < width || edges_size < 0 || (n > 0 && (!jobs || !pic || !edges))) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_intra_fill_edges", "bad count, size or pointer");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    intra::fill_edges_kernel<<<(unsigned)((n + 7) / 8), 256, 0, (cudaStream_t)stream>>>(jobs, n, pic, stride, width,
                                                                                         height, edges, edges_size);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

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
                                        xavs2gpu_intra_result_t *out, void *stream_)
{
    if (n < 0 || !prm || prm->dist1 < 0 || prm->dist2 < 0 || prm->dist2 > 9) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_intra_rmd_batch", "bad count or parameters");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    const cudaStream_t stream = (cudaStream_t)stream_;
    constexpr int smem = (int)sizeof(intra::TileSmem);
    static bool attr_set[64] = {false};
    static int ctas_per_sm[64] = {0}, sms[64] = {0};
    const int dev = current_device();
    if (dev < 0 || dev >= 64) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_intra_rmd_batch", "device index out of range");
        return XAVS2GPU_ERR_ARG;
    }
    if (!attr_set[dev]) {
        XG_CUDA(cudaFuncSetAttribute(intra::rmd_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas_per_sm[dev], intra::rmd_tile_kernel, intra::kTT,
                                                              smem));
        XG_CUDA(cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev));
        if (ctas_per_sm[dev] < 1) ctas_per_sm[dev] = 1;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        attr_set[dev] = true;
    }
    // scratch: class counts and cursors (32 ints each), then the ordered list
    int *scratch = nullptr;
    XG_CUDA(cudaMallocAsync((void **)&scratch, sizeof(int) * (64 + (size_t)n), stream));
    if (!scratch) return XAVS2GPU_ERR_CUDA;
    int *counts = scratch, *cursor = scratch + 32, *sorted = scratch + 64;
    XG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int) * 64, stream));
    const int nb = (n + 255) / 256;
    intra::rmd_count_kernel<<<nb, 256, 0, stream>>>(blocks, n, counts, out);
    intra::rmd_scatter_kernel<<<nb, 256, 0, stream>>>(blocks, n, counts, cursor, sorted);
    long long grid = (long long)sms[dev] * ctas_per_sm[dev];
    if (grid > n) grid = n;
    intra::rmd_tile_kernel<<<(int)grid, intra::kTT, smem, stream>>>(blocks, counts, sorted, edges, fenc, fenc_stride,
                                                                     *prm, out);
    intra::rmd_cand_kernel<<<(n + 127) / 128, 128, 0, stream>>>(blocks, n, *prm, out);
    count_launch(4);
    XG_CUDA(cudaFreeAsync(scratch, stream));
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
