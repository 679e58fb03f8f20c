// fs_ctu.cuh -- shared-window full search over every PU of a 64x64 CTU.
//
// The PU set of a CTU is the one an AVS2 encoder's mode decision searches:
// for CU sizes 64, 32 and 16 at every quadtree position the 13 PUs of the
// partitions 2Nx2N, 2NxN, Nx2N, 2NxnU, 2NxnD, nLx2N and nRx2N, and for every
// 8x8 CU its 8x8, 8x4 and 4x8 PUs plus the four 4x4 blocks -- 849 "slots",
// covering all 25 LumaPU shapes.  For PUs that share the search centre (0,0)
// and the MV predictor, the SAD of every PU at a displacement is a sum of the
// SADs of its 4x4 blocks at that displacement, so one warp computes the 256
// block SADs of the CTU once per displacement and derives all 849 PU costs
// from them (sums in registers, warp shuffles across regions).
//
// Warp layout: lane = ry*8 + rx*2 + half.  (rx, ry) is one of the 16 16x16
// regions of the CTU, half selects its top or bottom 8 rows.  A lane owns the
// 8 4x4 SADs of its half-region, the 18 PUs of its two 8x8 CUs and 6-7 PUs of
// its 16x16 CU; the 52 PUs of the 32x32 CUs and the 13 of the 64x64 CU are
// spread over the lanes (2 + 1 per lane at most).
//
// A CTA of 4 warps handles one (CTU, reference) and a chunk of 32 search rows
// (8 per warp) over the whole horizontal range; its reference window lives in
// shared memory.  Each warp keeps, per PU, the minimum of a 32-bit key
// (cost << 11 | row-in-warp << 8 | dx+R) for PUs up to 16x16 and per-row keys
// for the larger ones (the same form in interior jobs, cost << 8 | dx+R in
// border jobs, whose poisoned sums need the room), and merges them into the
// global 64-bit (cost, visit order) keys with atomicMin.  For ranges of 32
// and up a warp takes two search rows per pass over the window.
//
// Search limits: a PU is valid at a displacement iff the referenced block
// lies within [-58, W+58) x [-58, H+58) -- the limits pred_inter_search_single
// derives (md_inter.c:910-926) whenever they bind inside the search window.
// CTUs near the picture edge run a variant that replaces the SAD of every
// 4x4 block whose reference falls outside that region by a large value; the
// PUs containing such a block then never win and are not merged.
#pragma once

namespace xg {

constexpr int kSlots = 849;
constexpr int kDyChunk = 32;            // search rows per CTA
constexpr int kDyWarp = 8;              // search rows per warp
constexpr int kCtuThreads = 128;
constexpr uint32_t kPoisonSmall = 126976u;     // > any valid cost of a PU up to 16x16
constexpr uint32_t kPoisonLarge = 1u << 22;    // replaces a 4x4 SAD outside the limits
constexpr uint32_t kCapLarge = 2000000u;       // > any valid cost of a 64x64 PU
constexpr int kLimitMargin = 58;               // 64-pixel margin minus 6 (md_inter.c:913-926)

struct CtuJob {
    int16_t x0, y0;       // CTU origin
    uint8_t ref;
    uint8_t levels;       // CU sizes with a PU in the job: 1 8x8, 2 16x16, 4 32x32, 8 64x64
    int16_t mvp_x, mvp_y;
    uint8_t border;       // 1: limits may bind inside the window
    uint8_t sess;         // index into the session views of the launch
    int32_t slot_base;    // index of this job's row in its session's slot map
};

struct CtuPlan {
    int n_jobs = 0, cap_jobs = 0;
    int n_border = 0;             // jobs whose search limits may bind (border variant)
    CtuJob *d_jobs = nullptr;
    int32_t *d_slots = nullptr;   // [n_jobs][kSlots]: PU index or -1
    std::vector<CtuJob> h_jobs;   // host copy (sess = 0), for multi-session launches
};

// ---- slot geometry (host) --------------------------------------------------------
struct SlotGeom { int ox, oy, part; };

static inline int part_of(int w, int h)
{
    for (int i = 0; i < kNumParts; i++)
        if (h_pu_w[i] == w && h_pu_h[i] == h) return i;
    return -1;
}

// mode m of an N x N CU at (cx, cy): 0 2Nx2N, 1-2 2NxN, 3-4 Nx2N, 5-6 2NxnU,
// 7-8 2NxnD, 9-10 nLx2N, 11-12 nRx2N
static inline SlotGeom cu_mode_geom(int N, int cx, int cy, int m)
{
    const int h2 = N / 2, q = N / 4, q3 = 3 * N / 4;
    switch (m) {
    case 0: return {cx, cy, part_of(N, N)};
    case 1: return {cx, cy, part_of(N, h2)};
    case 2: return {cx, cy + h2, part_of(N, h2)};
    case 3: return {cx, cy, part_of(h2, N)};
    case 4: return {cx + h2, cy, part_of(h2, N)};
    case 5: return {cx, cy, part_of(N, q)};
    case 6: return {cx, cy + q, part_of(N, q3)};
    case 7: return {cx, cy, part_of(N, q3)};
    case 8: return {cx, cy + q3, part_of(N, q)};
    case 9: return {cx, cy, part_of(q, N)};
    case 10: return {cx + q, cy, part_of(q3, N)};
    case 11: return {cx, cy, part_of(q3, N)};
    default: return {cx + q3, cy, part_of(q, N)};
    }
}

static SlotGeom slot_geom(int s)
{
    if (s < 576) {
        int cu = s / 9, m = s % 9, cx = (cu % 8) * 8, cy = (cu / 8) * 8;
        switch (m) {
        case 0: return {cx, cy, part_of(8, 8)};
        case 1: return {cx, cy, part_of(8, 4)};
        case 2: return {cx, cy + 4, part_of(8, 4)};
        case 3: return {cx, cy, part_of(4, 8)};
        case 4: return {cx + 4, cy, part_of(4, 8)};
        case 5: return {cx, cy, 0};
        case 6: return {cx + 4, cy, 0};
        case 7: return {cx, cy + 4, 0};
        default: return {cx + 4, cy + 4, 0};
        }
    }
    if (s < 784) {
        int cu = (s - 576) / 13, m = (s - 576) % 13;
        return cu_mode_geom(16, (cu % 4) * 16, (cu / 4) * 16, m);
    }
    if (s < 836) {
        int cu = (s - 784) / 13, m = (s - 784) % 13;
        return cu_mode_geom(32, (cu % 2) * 32, (cu / 2) * 32, m);
    }
    return cu_mode_geom(64, 0, 0, s - 836);
}

// (part, ox/4, oy/4) -> slot, -1 if none
struct SlotTable {
    int16_t t[kNumParts][16][16];
    SlotTable()
    {
        memset(t, 0xff, sizeof(t));
        for (int s = 0; s < kSlots; s++) {
            SlotGeom g = slot_geom(s);
            t[g.part][g.oy >> 2][g.ox >> 2] = (int16_t)s;
        }
    }
};

// ---- device helpers ------------------------------------------------------------------

// bytes o..o+3 of the 8-byte little-endian pair (lo, hi), o = 1..3
#ifndef XG_CTU_PRMT
#define XG_CTU_PRMT 1
#endif
__device__ __forceinline__ uint32_t align_bytes(uint32_t lo, uint32_t hi, int o)
{
#if XG_CTU_PRMT
    return __byte_perm(lo, hi, o == 1 ? 0x4321 : o == 2 ? 0x5432 : 0x6543);
#else
    return __funnelshift_r(lo, hi, 8 * o);
#endif
}

__device__ __forceinline__ uint32_t addmin(uint32_t a, uint32_t b, uint32_t c)
{
    return __viaddmin_u32(a, b, c);   // min(a + b, c)
}

// Window row layout: rows are ww bytes apart (ww a multiple of 128, i.e. each
// row starts on bank 0) and row i is shifted right by swz(i) words.  In one
// shared load the 32 lanes read rows 8q + t (q = 2*ry + half, t common) at
// word 4*rx + k + t'; swz maps the eight q to {0,1,2,3,16,17,18,19}, so with
// the 4*rx offsets the lanes hit 32 distinct banks.
__host__ __device__ __forceinline__ int swz(int row) { return ((row >> 3) & 3) + 16 * ((row >> 5) & 1); }
constexpr int kSwzMax = 19;   // words

// slot of small key k (0..24) of a lane
__device__ __forceinline__ int small_slot(int rx, int ry, int half, int k)
{
    if (k < 18) {
        const int side = k / 9, m = k % 9;
        const int gx = 2 * rx + side, gy = 2 * ry + half;
        return (gy * 8 + gx) * 9 + m;
    }
    // 16-CU keys 18..24 -> modes (half 0 / half 1)
    const int i = k - 18;
    const int m0[7] = {0, 1, 3, 5, 6, 9, 10};
    const int m1[7] = {4, 2, 2, 8, 7, 12, 11};
    return 576 + (ry * 4 + rx) * 13 + (half ? m1[i] : m0[i]);
}

// 32-CU key modes per (half, qx, qy) (-1: none); keys A and B
__constant__ int8_t c_m32[2][2][2][2] = {
    // half 0: [qx][qy] -> {A, B}
    {{{1, 0}, {2, 8}}, {{5, 6}, {7, -1}}},
    // half 1
    {{{3, 9}, {10, 11}}, {{4, 12}, {-1, -1}}}};
// coefficients over (X1, X2, X3, X4) for the modes above
__constant__ int8_t c_c32[2][2][2][2][4] = {
    {{{{1, 0, 0, 0}, {1, 0, 1, 0}}, {{1, 0, 0, 0}, {1, -1, 0, 0}}},
     {{{0, 1, 0, 0}, {1, -1, 1, 0}}, {{0, 1, 1, 0}, {0, 0, 0, 0}}}},
    {{{{1, 0, 0, 0}, {0, 1, 0, 0}}, {{1, -1, 1, 0}, {1, 0, 0, 1}}},
     {{{1, 0, 0, 0}, {1, -1, 0, 0}}, {{0, 0, 0, 0}, {0, 0, 0, 0}}}}};
// 64-CU key per lane (lane = ry*8 + rx*2 + half): mode (-1 none) and
// coefficients over (TOT, P, RS) -- half-0 lanes hold row quantities (RS =
// sum of a row of regions, P = pair of rows), half-1 lanes the column ones.
__constant__ int8_t c_m64[32] = {0, 3, 1, -1, 5, 4, 6, 11, -1, 9, -1, -1, -1, -1, -1, 12,
                                 2, 10, -1, -1, -1, -1, -1, -1, 7, -1, 8, -1, -1, -1, -1, -1};
__constant__ int8_t c_c64[32][3] = {
    {1, 0, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {1, 0, -1}, {1, 0, -1},
    {0, 0, 0}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 1},
    {0, 1, 0}, {1, 0, -1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0},
    {1, 0, -1}, {0, 0, 0}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};

// Per-lane constants of the warp layout.
struct LaneRole {
    int half, rx, ry;
    int pr1, pr2, pr3, pr4, pr5;    // shuffle partners (see below)
    int c32a[4], c32b[4], c64[3];   // coefficient sets of the 32-CU / 64-CU keys
    int bx0, by0;                   // picture position of the half-region
};

// Folds the costs of one displacement into the lane's keys.  `raw` are the
// lane's eight 4x4 SADs; `mks` = (mvc << 11) | (row << 8) | dx+R for the
// small keys, `mkl` = (mvc << 8) | dx+R for the large ones.
// LV (a compile-time set of CU sizes, as CtuJob::levels) drops the key
// updates of the CU sizes a job has no PU of.  BORDER poisons the blocks
// outside the limits; BJ marks a border job, whose large keys are
// (cost << 8) | dx+R (poisoned sums need the room).  An interior job keeps its
// large keys in the small-key form (cost << 11 | row << 8 | dx+R: a 64x64
// cost plus its MV cost stays below 2^21), with no shifts.
template <bool BORDER, int LV, bool BJ = BORDER>
__device__ __forceinline__ void fold_displacement(const LaneRole &LR, uint32_t (&raw)[2][4], uint32_t mks,
                                                  uint32_t mkl, int dx, bool brow0, bool brow1, const Geometry &g,
                                                  uint32_t (&ks)[25], uint32_t (&rowl)[3])
{
    const int half = LR.half;
    if (BORDER) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int xb = LR.bx0 + 4 * c + dx;
            const bool colok = xb >= -kLimitMargin && xb + 4 <= g.W + kLimitMargin;
            if (!(colok && brow0)) raw[0][c] = kPoisonLarge;
            if (!(colok && brow1)) raw[1][c] = kPoisonLarge;
        }
    }
    // small-key domain: SAD << 11 (poison clamped for the small PUs)
    uint32_t t[2][4];
#pragma unroll
    for (int br = 0; br < 2; br++)
#pragma unroll
        for (int c = 0; c < 4; c++) t[br][c] = (BORDER ? min(raw[br][c], kPoisonSmall) : raw[br][c]) << 11;
    // 8x8 CUs of this half: left (cols 0,1) and right (cols 2,3)
    uint32_t qv[2], at[2], ab[2], vl[2], vr[2];
#pragma unroll
    for (int sd = 0; sd < 2; sd++) {
        const int c0 = 2 * sd;
        at[sd] = t[0][c0] + t[0][c0 + 1];
        ab[sd] = t[1][c0] + t[1][c0 + 1];
        vl[sd] = t[0][c0] + t[1][c0];
        vr[sd] = t[0][c0 + 1] + t[1][c0 + 1];
        qv[sd] = at[sd] + ab[sd];
        if (!(LV & 1)) continue;
        const int kb = 9 * sd;
        ks[kb + 0] = addmin(qv[sd], mks, ks[kb + 0]);
        ks[kb + 1] = addmin(at[sd], mks, ks[kb + 1]);
        ks[kb + 2] = addmin(ab[sd], mks, ks[kb + 2]);
        ks[kb + 3] = addmin(vl[sd], mks, ks[kb + 3]);
        ks[kb + 4] = addmin(vr[sd], mks, ks[kb + 4]);
        ks[kb + 5] = addmin(t[0][c0], mks, ks[kb + 5]);
        ks[kb + 6] = addmin(t[0][c0 + 1], mks, ks[kb + 6]);
        ks[kb + 7] = addmin(t[1][c0], mks, ks[kb + 7]);
        ks[kb + 8] = addmin(t[1][c0 + 1], mks, ks[kb + 8]);
    }
    // 16x16 CU: own half (Fh, Lh, strips) + partner half
    const uint32_t Fh = qv[0] + qv[1];
    const uint32_t Lh = qv[0];
    const uint32_t rr_ = half ? ab[0] + ab[1] : at[0] + at[1];   // own outer 16x4 strip
    const uint32_t c0h = vl[0], c3h = vr[1];
    const uint32_t Fh_o = __shfl_xor_sync(0xffffffffu, Fh, 1);
    const uint32_t Lh_o = __shfl_xor_sync(0xffffffffu, Lh, 1);
    const uint32_t xs = half ? c0h : c3h;
    const uint32_t xs_o = __shfl_xor_sync(0xffffffffu, xs, 1);
    const uint32_t F = Fh + Fh_o, L = Lh + Lh_o;
    const uint32_t cc = (half ? c3h : c0h) + xs_o;          // col 3 (half 1) / col 0 (half 0)
    if (LV & 2) {
        ks[18] = addmin(F - (half ? L : 0u), mks, ks[18]);     // 16x16 | 8x16 right
        ks[19] = addmin(Fh, mks, ks[19]);                      // 16x8 top | bottom
        ks[20] = addmin(half ? Fh : L, mks, ks[20]);           // 8x16 left | (dup)
        ks[21] = addmin(rr_, mks, ks[21]);                     // 16x4 y0 | y12
        ks[22] = addmin(F - rr_, mks, ks[22]);                 // 16x12 y4 | y0
        ks[23] = addmin(cc, mks, ks[23]);                      // 4x16 x0 | x12
        ks[24] = addmin(F - cc, mks, ks[24]);                  // 12x16 x4 | x0
    }
    // large PUs in the raw domain
    uint32_t Fr, Tr, Lr;
    if (BORDER) {
        uint32_t fh = 0, lh = 0;
#pragma unroll
        for (int br = 0; br < 2; br++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                fh += raw[br][c];
                if (c < 2) lh += raw[br][c];
            }
        const uint32_t fh_o = __shfl_xor_sync(0xffffffffu, fh, 1);
        const uint32_t lh_o = __shfl_xor_sync(0xffffffffu, lh, 1);
        Fr = fh + fh_o;
        Tr = half ? fh_o : fh;
        Lr = lh + lh_o;
    } else if (BJ) {
        Fr = F >> 11;
        Tr = (half ? Fh_o : Fh) >> 11;
        Lr = L >> 11;
    } else {
        Fr = F;
        Tr = half ? Fh_o : Fh;
        Lr = L;
    }
    // 32x32 CUs
    const uint32_t a1 = half ? Lr : Tr;
    const uint32_t F_p = __shfl_xor_sync(0xffffffffu, Fr, LR.pr1);
    const uint32_t a_p = __shfl_xor_sync(0xffffffffu, a1, LR.pr1);
    const uint32_t X1 = Fr + F_p, X2 = a1 + a_p;           // FH, TH  |  FV, LV
    const uint32_t X3 = __shfl_xor_sync(0xffffffffu, X1, LR.pr2);
    const uint32_t X4 = __shfl_xor_sync(0xffffffffu, X2, LR.pr2);
    const int va = LR.c32a[0] * (int)X1 + LR.c32a[1] * (int)X2 + LR.c32a[2] * (int)X3 + LR.c32a[3] * (int)X4;
    const int vb = LR.c32b[0] * (int)X1 + LR.c32b[1] * (int)X2 + LR.c32b[2] * (int)X3 + LR.c32b[3] * (int)X4;
    // 64x64 CU
    const uint32_t RS = X1 + __shfl_xor_sync(0xffffffffu, X1, LR.pr3);     // row | column sums
    const uint32_t P = RS + __shfl_xor_sync(0xffffffffu, RS, LR.pr4);      // row | column pairs
    const uint32_t TOT = P + __shfl_xor_sync(0xffffffffu, P, LR.pr5);
    const int v64 = LR.c64[0] * (int)TOT + LR.c64[1] * (int)P + LR.c64[2] * (int)RS;
    // without poisoned blocks a 64x64 cost stays below kCapLarge (1,044,480 <
    // 2,000,000) and a lane without a key has all-zero coefficients
    if (!BJ) {
        if (LV & 4) {
            rowl[0] = addmin((uint32_t)va, mks, rowl[0]);
            rowl[1] = addmin((uint32_t)vb, mks, rowl[1]);
        }
        if (LV & 8) rowl[2] = addmin((uint32_t)v64, mks, rowl[2]);
        return;
    }
    if (LV & 4) {
        rowl[0] = addmin((BORDER ? min((uint32_t)va, kCapLarge) : (uint32_t)va) << 8, mkl, rowl[0]);
        rowl[1] = addmin((BORDER ? min((uint32_t)vb, kCapLarge) : (uint32_t)vb) << 8, mkl, rowl[1]);
    }
    if (LV & 8) rowl[2] = addmin((BORDER ? min((uint32_t)v64, kCapLarge) : (uint32_t)v64) << 8, mkl, rowl[2]);
}

// 4x4 SADs of the lane's half-region against window rows wrow0.. at byte
// offset j (any alignment).
__device__ __forceinline__ void sad_at(const uint8_t *win, int ww, int wrow0, int rx, int j, const uint32_t (&cw)[8][4],
                                       uint32_t (&raw)[2][4])
{
    const int j0 = j & ~3, o = j & 3;
#pragma unroll
    for (int br = 0; br < 2; br++)
#pragma unroll
        for (int c = 0; c < 4; c++) raw[br][c] = 0;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int wr = wrow0 + r;
        const uint32_t *wp = reinterpret_cast<const uint32_t *>(win + wr * ww + 4 * swz(wr) + 16 * rx + j0);
#pragma unroll
        for (int c = 0; c < 4; c++) raw[r >> 2][c] = sad4_acc(cw[r][c], __funnelshift_r(wp[c], wp[c + 1], 8 * o), raw[r >> 2][c]);
    }
}

// border jobs: the interior fold for displacements that need no limit
#ifndef XG_CTU_SAFE_SPLIT
#define XG_CTU_SAFE_SPLIT 1
#endif

// window fill with 16-byte loads when the window lies inside the padded plane
#ifndef XG_CTU_VEC_FILL
#define XG_CTU_VEC_FILL 1
#endif

// Window fill by the tensor memory accelerator: where the session has a
// tensor map over its plane pool (3-D: column, row, plane; box 64 columns x
// 95 rows) and the window qualifies for the 16-byte fill, one thread issues
// the window as 64-column boxes into a dense staging area before the CTA
// computes its MV-cost keys, so the copy overlaps that work.  The search's
// row layout shifts rows by 1-3 words (the bank spread above), which no
// 16-byte-aligned TMA destination can hold, so a shared-to-shared pass then
// places the rows.
#ifndef XG_CTU_TMA
#define XG_CTU_TMA 1
#endif
constexpr int kTmaBoxCols = 64;
constexpr int kTmaBoxRows = 64 + kDyChunk - 1;
constexpr int kTmaPieceBytes = (kTmaBoxCols * kTmaBoxRows + 127) / 128 * 128;   // 6144
constexpr int kWaitLimit = 1 << 20;   // mbarrier polls before a CTA gives up its window

__host__ __device__ constexpr int tma_pieces(int R) { return (64 + 2 * R + 8 + kTmaBoxCols - 1) / kTmaBoxCols; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
    for (int i = 0; i < kWaitLimit; i++) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// Thread 0 only: the window rows [y, y + 95) of plane z, columns x .. x + 64*np
// (x a multiple of 16), as np boxes into stage (128-byte aligned), counted
// on the barrier at bar.
__device__ __forceinline__ void tma_window_issue(const void *tmap, uint32_t stage, uint32_t bar, int x, int y, int z,
                                                 int np)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                 "r"((uint32_t)(np * kTmaBoxCols * kTmaBoxRows))
                 : "memory");
    for (int p = 0; p < np; p++)
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                     " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(stage + (uint32_t)(p * kTmaPieceBytes)),
                     "l"(tmap), "r"(x + p * kTmaBoxCols), "r"(y), "r"(z), "r"(bar)
                     : "memory");
}

// resident CTAs per SM the register budget is sized for (3: up to 168
// registers; measured faster than 4 CTAs of 128 registers and than 2)
#ifndef XG_CTU_MINB
#define XG_CTU_MINB 3
#endif
// the same for the two-row form (2: up to 255 registers)
#ifndef XG_CTU_PAIR_MINB
#define XG_CTU_PAIR_MINB 2
#endif

// Ranges from which the search takes two displacement rows per window pass
// (see ctu_search): the pair form needs about 240 registers (2 CTAs per SM
// instead of 3) and measured 8 % faster at R = 64 (3.39 against 3.68 ms per
// 1080p picture), 9 % slower at R = 16 (0.269 against 0.247 ms), where the
// per-CTA setup of the 32-row chunk weighs more.
#ifndef XG_CTU_PAIR_MIN_R
#define XG_CTU_PAIR_MIN_R 32
#endif

// Folds the 4 displacements j0 .. j0 + 3 of one search row (SADs s[o]) into
// the lane's keys.
template <bool BORDER, int LV>
__device__ __forceinline__ void fold_four(const LaneRole &L, uint32_t (&s)[4][2][4], const uint32_t *mrow, int nd, int j0,
                                          int R, bool brow0, bool brow1, bool row_safe, const CtuJob &job,
                                          const Geometry &g, uint32_t (&ks)[25], uint32_t (&rowl)[3])
{
#if XG_CTU_SAFE_SPLIT
    // in a border job, displacements whose every block stays inside the
    // limits take the interior fold (same keys: nothing to poison)
    const bool safe = !BORDER || (row_safe && job.x0 + j0 - R >= -kLimitMargin &&
                                  job.x0 + 64 + j0 + 3 - R <= g.W + kLimitMargin);
    if (BORDER && !safe) {
#pragma unroll
        for (int o = 0; o < 4; o++) {
            const int dxr = j0 + o;
            const uint32_t mks = mrow[dxr], mkl = mrow[nd * kDyChunk + dxr];
            fold_displacement<true, LV, true>(L, s[o], mks, mkl, dxr - R, brow0, brow1, g, ks, rowl);
        }
    } else {
#pragma unroll
        for (int o = 0; o < 4; o++) {
            const int dxr = j0 + o;
            const uint32_t mks = mrow[dxr], mkl = mrow[nd * kDyChunk + dxr];
            fold_displacement<false, LV, BORDER>(L, s[o], mks, mkl, dxr - R, brow0, brow1, g, ks, rowl);
        }
    }
#else
    (void)row_safe;
    (void)job;
#pragma unroll
    for (int o = 0; o < 4; o++) {
        const int dxr = j0 + o;
        const uint32_t mks = mrow[dxr], mkl = mrow[nd * kDyChunk + dxr];
        fold_displacement<BORDER, LV>(L, s[o], mks, mkl, dxr - R, brow0, brow1, g, ks, rowl);
    }
#endif
}

// a search row's large-PU minima into the 64-bit (cost, order) keys (cost
// above the low 8 bits in a border job, above the low 11 in an interior job)
template <bool BJ>
__device__ __forceinline__ void merge_rowl(const uint32_t (&rowl)[3], int dy, int R, int nd,
                                           unsigned long long (&kl)[3])
{
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint32_t cost = rowl[k] >> (BJ ? 8 : 11), dxr = rowl[k] & 0xffu;
        if (cost >= kCapLarge) continue;
        const unsigned long long key = ((unsigned long long)cost << 32) | (unsigned)(2 + (dy + R) * nd + (int)dxr);
        kl[k] = key < kl[k] ? key : kl[k];
    }
}

template <bool BORDER, int LV, bool PAIR>
__device__ __forceinline__ void ctu_search(const CtuJob &job, int chunk, const SessView *__restrict__ views, int R,
                                           int lambda, int ww, uint8_t *smem)
{
    const SessView &view = views[job.sess];
    const int32_t *__restrict__ slots = view.slots;
    const uint8_t *__restrict__ cur = view.cur;
    const uint8_t *const *refs = view.ref0;
    const Geometry g = view.g;
    unsigned long long *__restrict__ keys = view.keys;
    const int dy0 = -R + chunk * kDyChunk;
    const int wrows = 64 + kDyChunk - 1;
    const int nd = 2 * R;
    // MV-cost keys: small-PU form [kDyChunk][nd], then the large-PU form
    uint32_t *mvk = reinterpret_cast<uint32_t *>(smem);                 // [2][kDyChunk][nd]
    uint8_t *win = smem + 2 * sizeof(uint32_t) * kDyChunk * nd;          // [wrows][ww]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // reference window: rows y0+dy0 .., columns x0-R .., clamped into the plane
    const uint8_t *ref = refs[job.ref];
    const int wx0 = job.x0 - R, wy0 = job.y0 + dy0;
    const int rowlen = ww - 4 * kSwzMax - 4;   // bytes of a row that are filled (a multiple of 16)
    const bool vec_ok = wx0 >= -kPad && wx0 + rowlen <= g.W + kPad && wy0 >= -kPad && wy0 + wrows <= g.H + kPad &&
                        (g.stride & 15) == 0 &&
                        ((uintptr_t)(ref + (ptrdiff_t)wy0 * g.stride + wx0) & 15) == 0;
#if XG_CTU_TMA
    // staging area after the window (128-byte aligned when the dynamic shared
    // memory base is), the barrier after it
    uint8_t *stage = win + (size_t)wrows * ww;
    const int np = tma_pieces(R);
    const uint32_t stage_s = smem_u32(stage), bar_s = stage_s + (uint32_t)(np * kTmaPieceBytes);
    int tx = 0, ty = 0, tz = 0;
    bool use_tma = false;
    // the launch gave the CTA the staging area (it does not where that would
    // cost a CTA per SM)
    uint32_t dyn_smem;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_smem));
    const bool staged = (uint32_t)(stage - smem) + (uint32_t)(np * kTmaPieceBytes) + 16u <= dyn_smem;
    if (view.tmap != nullptr && staged && vec_ok && (stage_s & 127) == 0) {
        const ptrdiff_t off = (ref + (ptrdiff_t)wy0 * g.stride + wx0) - view.pool;
        tz = (int)(off / (ptrdiff_t)view.plane_bytes);
        const ptrdiff_t rem = off - (ptrdiff_t)tz * view.plane_bytes;
        ty = (int)(rem / g.stride);
        tx = (int)(rem - (ptrdiff_t)ty * g.stride);
        use_tma = off >= 0 && (tx & 15) == 0;
    }
    if (use_tma && tid == 0) tma_window_issue(view.tmap, stage_s, bar_s, tx, ty, tz, np);
    __syncthreads();   // the barrier's initialisation, before any thread polls it
#endif

    // MV cost keys of this chunk's displacements (uniform over the CTU)
    for (int e = tid; e < kDyChunk * nd; e += kCtuThreads) {
        const int row = e / nd, dxr = e - row * nd;
        const int dy = dy0 + row, dx = dxr - R;
        const uint32_t mvc = (uint32_t)mv_cost_hd(lambda, dx * 4, dy * 4, job.mvp_x, job.mvp_y);
        mvk[e] = (mvc << 11) | ((uint32_t)(row & (kDyWarp - 1)) << 8) | (uint32_t)dxr;
        mvk[kDyChunk * nd + e] = (mvc << 8) | (uint32_t)dxr;
    }
#if XG_CTU_TMA
    if (use_tma) {
        const bool ok = mbar_wait_bounded(bar_s, 0);
        if (__syncthreads_or(!ok)) {
            // the copy did not land: record it, give the copies in flight
            // one more bounded wait, and leave this chunk unsearched
            if (tid == 0 && view.wait_flag) atomicOr(view.wait_flag, 1u);
            mbar_wait_bounded(bar_s, 0);
            return;
        }
        // staged rows [95][64] per box -> the swizzled window rows; only the
        // bytes the row layout holds (a multiple of 16, at least 64 + 2R + 8)
        const int cols = min(np * kTmaBoxCols, rowlen) >> 4;
        for (int e = tid; e < wrows * cols; e += kCtuThreads) {
            const int r = e / cols, c = (e - r * cols) << 4;
            const uint4 v = *reinterpret_cast<const uint4 *>(stage + (c >> 6) * kTmaPieceBytes + r * kTmaBoxCols +
                                                             (c & (kTmaBoxCols - 1)));
            uint32_t *d = reinterpret_cast<uint32_t *>(win + r * ww + 4 * swz(r) + c);
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
        }
    } else
#endif
#if XG_CTU_VEC_FILL
    if (vec_ok) {
        // the window lies inside the padded plane and its rows start on
        // 16-byte boundaries: 16-byte loads, word stores into the swizzled rows
        const int q = rowlen >> 4;
        for (int e = tid; e < wrows * q; e += kCtuThreads) {
            const int r = e / q, c = (e - r * q) << 4;
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(ref + (ptrdiff_t)(wy0 + r) * g.stride + wx0 + c));
            uint32_t *d = reinterpret_cast<uint32_t *>(win + r * ww + 4 * swz(r) + c);
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
        }
    } else
#endif
    {
        for (int e = tid; e < wrows * rowlen; e += kCtuThreads) {
            const int r = e / rowlen, c = e - r * rowlen;
            const int y = min(max(wy0 + r, -kPad), g.H + kPad - 1);
            const int x = min(max(wx0 + c, -kPad), g.W + kPad - 1);
            win[r * ww + 4 * swz(r) + c] = ref[(ptrdiff_t)y * g.stride + x];
        }
    }
    __syncthreads();

    LaneRole L;
    L.half = lane & 1;
    L.rx = (lane >> 1) & 3;
    L.ry = lane >> 3;
    const int half = L.half, rx = L.rx, ry = L.ry;
    const int qx = rx & 1, qy = ry & 1;
    // current block: 8 rows x 16 pixels of this half-region
    uint32_t cw[8][4];
    {
        const uint8_t *o = cur + (ptrdiff_t)(job.y0 + 16 * ry + 8 * half) * g.stride + job.x0 + 16 * rx;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const uint4 v = *reinterpret_cast<const uint4 *>(o + (ptrdiff_t)r * g.stride);
            cw[r][0] = v.x; cw[r][1] = v.y; cw[r][2] = v.z; cw[r][3] = v.w;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        L.c32a[k] = c_c32[half][qx][qy][0][k];
        L.c32b[k] = c_c32[half][qx][qy][1][k];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) L.c64[k] = c_c64[lane][k];
    const int m32a = c_m32[half][qx][qy][0], m32b = c_m32[half][qx][qy][1], m64 = c_m64[lane];
    // shuffle partners: region pairs along the axis this half works on
    L.pr1 = half ? 8 : 2;     // 32-CU pair (vertical for half 1, horizontal for half 0)
    L.pr2 = half ? 2 : 8;     // the other 32-CU row/column
    L.pr3 = half ? 16 : 4;    // 64-CU row / column sums
    L.pr4 = half ? 2 : 8;     // 64-CU pairs
    L.pr5 = half ? 4 : 16;    // 64-CU total
    L.bx0 = job.x0 + 16 * rx;
    L.by0 = job.y0 + 16 * ry + 8 * half;
    const int32_t *smap = slots + (size_t)job.slot_base;
    const int cu32 = (ry >> 1) * 2 + (rx >> 1);
    const int lm[3] = {m32a, m32b, m64};

    // The search candidate (0,0) is visited before the window (me.c:913-917):
    // its cost enters with visit order 0, so it wins every tie.  The CTA whose
    // rows contain dy = 0 evaluates it (warp 0).
    if (warp == 0 && dy0 <= 0 && 0 < dy0 + kDyChunk) {
        uint32_t ks0[25], rowl0[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
#pragma unroll
        for (int k = 0; k < 25; k++) ks0[k] = 0xffffffffu;
        uint32_t raw[2][4];
        sad_at(win, ww, 16 * ry + 8 * half - dy0, rx, R, cw, raw);
        const uint32_t mvc0 = (uint32_t)mv_cost_hd(lambda, 0, 0, job.mvp_x, job.mvp_y);
        bool b0 = true, b1 = true;
        if (BORDER) {
            b0 = L.by0 >= -kLimitMargin && L.by0 + 4 <= g.H + kLimitMargin;
            b1 = L.by0 + 4 >= -kLimitMargin && L.by0 + 8 <= g.H + kLimitMargin;
        }
        fold_displacement<BORDER, LV>(L, raw, mvc0 << 11, mvc0 << 8, 0, b0, b1, g, ks0, rowl0);
#pragma unroll
        for (int k = 0; k < 25; k++) {
            const uint32_t cost = ks0[k] >> 11;
            if (cost >= kPoisonSmall) continue;
            const int pu = smap[small_slot(rx, ry, half, k)];
            if (pu >= 0) atomicMin(&keys[pu], (unsigned long long)cost << 32);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint32_t cost = rowl0[k] >> (BORDER ? 8 : 11);
            if (lm[k] < 0 || cost >= kCapLarge) continue;
            const int pu = smap[k < 2 ? 784 + cu32 * 13 + lm[k] : 836 + lm[k]];
            if (pu >= 0) atomicMin(&keys[pu], (unsigned long long)cost << 32);
        }
    }

    uint32_t ks[25];
    unsigned long long kl[3] = {~0ull, ~0ull, ~0ull};
#pragma unroll
    for (int k = 0; k < 25; k++) ks[k] = 0xffffffffu;

    if constexpr (PAIR) {
    // two displacement rows per pass: window rows wrow0 .. wrow0 + 8 are
    // loaded and aligned once; row r serves block row r of the first
    // displacement row and block row r - 1 of the second
    for (int rr = 0; rr < kDyWarp; rr += 2) {
        const int row = warp * kDyWarp + rr;
        const int dy = dy0 + row;
        if (dy >= R) break;     // 2R and kDyWarp are even: a pair is all in or all out
        const int wrow0 = 16 * ry + 8 * half + row;
        const uint32_t *mrowA = mvk + row * nd, *mrowB = mrowA + nd;
        uint32_t rowlA[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, rowlB[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
        bool bA0 = true, bA1 = true, bB0 = true, bB1 = true;
        if (BORDER) {
            const int yb = L.by0 + dy;
            bA0 = yb >= -kLimitMargin && yb + 4 <= g.H + kLimitMargin;
            bA1 = yb + 4 >= -kLimitMargin && yb + 8 <= g.H + kLimitMargin;
            bB0 = yb + 1 >= -kLimitMargin && yb + 5 <= g.H + kLimitMargin;
            bB1 = yb + 5 >= -kLimitMargin && yb + 9 <= g.H + kLimitMargin;
        }
        const bool safeA = job.y0 + dy >= -kLimitMargin && job.y0 + 64 + dy <= g.H + kLimitMargin;
        const bool safeB = job.y0 + dy + 1 >= -kLimitMargin && job.y0 + 65 + dy <= g.H + kLimitMargin;
        for (int j0 = 0; j0 < nd; j0 += 4) {
            uint32_t sA[4][2][4], sB[4][2][4];
#pragma unroll
            for (int o = 0; o < 4; o++)
#pragma unroll
                for (int br = 0; br < 2; br++)
#pragma unroll
                    for (int c = 0; c < 4; c++) sA[o][br][c] = sB[o][br][c] = 0;
#pragma unroll
            for (int r = 0; r < 9; r++) {
                const int wr = wrow0 + r;
                const uint32_t *wp = reinterpret_cast<const uint32_t *>(win + wr * ww + 4 * swz(wr) + 16 * rx + j0);
                uint32_t w5[5];
#pragma unroll
                for (int k = 0; k < 5; k++) w5[k] = wp[k];
#pragma unroll
                for (int o = 0; o < 4; o++) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        const uint32_t a = o ? align_bytes(w5[c], w5[c + 1], o) : w5[c];
                        if (r < 8) sA[o][r >> 2][c] = sad4_acc(cw[r][c], a, sA[o][r >> 2][c]);
                        if (r >= 1) sB[o][(r - 1) >> 2][c] = sad4_acc(cw[r - 1][c], a, sB[o][(r - 1) >> 2][c]);
                    }
                }
            }
            fold_four<BORDER, LV>(L, sA, mrowA, nd, j0, R, bA0, bA1, safeA, job, g, ks, rowlA);
            fold_four<BORDER, LV>(L, sB, mrowB, nd, j0, R, bB0, bB1, safeB, job, g, ks, rowlB);
        }
        merge_rowl<BORDER>(rowlA, dy, R, nd, kl);
        merge_rowl<BORDER>(rowlB, dy + 1, R, nd, kl);
    }
    } else {
    for (int rr = 0; rr < kDyWarp; rr++) {
        const int row = warp * kDyWarp + rr;
        const int dy = dy0 + row;
        if (dy >= R) break;
        const int wrow0 = 16 * ry + 8 * half + row;
        const uint32_t *mrow = mvk + row * nd;
        uint32_t rowl[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu};
        bool brow0 = true, brow1 = true;
        if (BORDER) {
            const int yb = L.by0 + dy;
            brow0 = yb >= -kLimitMargin && yb + 4 <= g.H + kLimitMargin;
            brow1 = yb + 4 >= -kLimitMargin && yb + 8 <= g.H + kLimitMargin;
        }
        // every block of the CTU inside the vertical limits at this dy
        const bool row_safe = job.y0 + dy >= -kLimitMargin && job.y0 + 64 + dy <= g.H + kLimitMargin;
        for (int j0 = 0; j0 < nd; j0 += 4) {
            uint32_t s[4][2][4];
#pragma unroll
            for (int o = 0; o < 4; o++)
#pragma unroll
                for (int br = 0; br < 2; br++)
#pragma unroll
                    for (int c = 0; c < 4; c++) s[o][br][c] = 0;
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const int wr = wrow0 + r;
                const uint32_t *wp = reinterpret_cast<const uint32_t *>(win + wr * ww + 4 * swz(wr) + 16 * rx + j0);
                uint32_t w5[5];
#pragma unroll
                for (int k = 0; k < 5; k++) w5[k] = wp[k];
#pragma unroll
                for (int o = 0; o < 4; o++) {
#pragma unroll
                    for (int c = 0; c < 4; c++) {
                        // the 4 bytes at byte offset o: a byte permute with a
                        // constant selector (4321, 5432, 6543)
                        const uint32_t a = o ? align_bytes(w5[c], w5[c + 1], o) : w5[c];
                        s[o][r >> 2][c] = sad4_acc(cw[r][c], a, s[o][r >> 2][c]);
                    }
                }
            }
            fold_four<BORDER, LV>(L, s, mrow, nd, j0, R, brow0, brow1, row_safe, job, g, ks, rowl);
        }
        merge_rowl<BORDER>(rowl, dy, R, nd, kl);
    }
    }
    // merge into the global keys
    const int dyw = dy0 + warp * kDyWarp;
#pragma unroll
    for (int k = 0; k < 25; k++) {
        const uint32_t key = ks[k];
        const uint32_t cost = key >> 11;
        if (cost >= kPoisonSmall) continue;
        const int pu = smap[small_slot(rx, ry, half, k)];
        if (pu < 0) continue;
        const int dy = dyw + (int)((key >> 8) & 7), dxr = (int)(key & 0xffu);
        atomicMin(&keys[pu], ((unsigned long long)cost << 32) | (unsigned)(2 + (dy + R) * nd + dxr));
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (lm[k] < 0 || kl[k] == ~0ull) continue;
        const int slot = k < 2 ? 784 + cu32 * 13 + lm[k] : 836 + lm[k];
        const int pu = smap[slot];
        if (pu >= 0) atomicMin(&keys[pu], kl[k]);
    }
}

// CU sizes with separate compiled folds (serving's leaf CUs often have no
// 8x8 / 16x16 CU in a CTU): 1 on, 0 every job with the full fold
#ifndef XG_CTU_LEVELS
#define XG_CTU_LEVELS 1
#endif

template <bool BORDER, bool PAIR>
__global__ void __launch_bounds__(kCtuThreads, PAIR ? XG_CTU_PAIR_MINB : XG_CTU_MINB)
    fs_ctu_kernel(const CtuJob *__restrict__ jobs, int nchunks, const SessView *__restrict__ views, int R, int lambda,
                  int ww)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int job_idx = blockIdx.x / nchunks, chunk = blockIdx.x % nchunks;
    const CtuJob job = jobs[job_idx];
    if (BORDER != (job.border != 0)) return;
#if XG_CTU_LEVELS
    if (job.levels & 1) ctu_search<BORDER, 15, PAIR>(job, chunk, views, R, lambda, ww, smem);
    else if (job.levels & 2) ctu_search<BORDER, 14, PAIR>(job, chunk, views, R, lambda, ww, smem);
    else ctu_search<BORDER, 12, PAIR>(job, chunk, views, R, lambda, ww, smem);
#else
    ctu_search<BORDER, 15, PAIR>(job, chunk, views, R, lambda, ww, smem);
#endif
}

// ---- host planning -----------------------------------------------------------------
static inline void ctu_plan_free(CtuPlan &p)
{
    if (p.d_jobs) cudaFree(p.d_jobs);
    if (p.d_slots) cudaFree(p.d_slots);
    p = CtuPlan();
}

// Splits a PU list into CTU jobs and the rest (`generic`).  A PU joins its
// CTU's job when it sits on one of the CTU's slots, its MVP rounds to (0,0)
// (so the search centre is (0,0)), all PUs of the job share that MVP, and
// inside the (2R)^2 window its limits allow exactly the displacements the
// edge rule allows.
static inline bool same_range_in_window(int lo, int hi, int rule_lo, int rule_hi, int R)
{
    return max(lo, -R) == max(rule_lo, -R) && min(hi, R - 1) == min(rule_hi, R - 1);
}

static void ctu_plan_build(CtuPlan &p, const std::vector<xavs2gpu_pu_t> &pus, int W, int H, int nrefs, int R,
                           bool allow, std::vector<int> &generic, cudaStream_t st)
{
    static const SlotTable table;
    const int cw = (W + 63) / 64, ch = (H + 63) / 64;
    const int ngroups = cw * ch * nrefs;
    std::vector<int> group_job(ngroups, -1);
    std::vector<CtuJob> jobs;
    std::vector<int32_t> slots;
    generic.clear();
    // the CTU kernel walks a search row in steps of 4 displacements, so it
    // takes ranges whose 2R is a multiple of 4 (odd R: every PU per-PU)
    const bool range_ok = allow && (2 * R) % 4 == 0;
    for (int i = 0; i < (int)pus.size(); i++) {
        const xavs2gpu_pu_t &u = pus[i];
        const int w = h_pu_w[u.part], h = h_pu_h[u.part];
        bool ok = range_ok && ((u.mvp_x + 2) >> 2) == 0 && ((u.mvp_y + 2) >> 2) == 0 && !(u.x & 3) && !(u.y & 3);
        // (0,0) must be inside the limits for it to be the centre
        ok = ok && u.min_x <= 0 && u.max_x >= 0 && u.min_y <= 0 && u.max_y >= 0;
        ok = ok && same_range_in_window(u.min_x, u.max_x, -kLimitMargin - u.x, W + kLimitMargin - u.x - w, R) &&
             same_range_in_window(u.min_y, u.max_y, -kLimitMargin - u.y, H + kLimitMargin - u.y - h, R);
        const int s = ok ? table.t[u.part][(u.y & 63) >> 2][(u.x & 63) >> 2] : -1;
        if (s < 0) { generic.push_back(i); continue; }
        const int gidx = ((u.y >> 6) * cw + (u.x >> 6)) * nrefs + u.ref;
        int j = group_job[gidx];
        if (j < 0) {
            j = (int)jobs.size();
            group_job[gidx] = j;
            CtuJob cj;
            cj.x0 = (int16_t)(u.x & ~63); cj.y0 = (int16_t)(u.y & ~63); cj.ref = u.ref;
            cj.levels = 0;
            cj.mvp_x = u.mvp_x; cj.mvp_y = u.mvp_y;
            // can the edge rule bind for any block of this CTU inside the window?
            cj.border = (cj.x0 - R < -kLimitMargin || cj.x0 + 64 + R > W + kLimitMargin ||
                         cj.y0 - R < -kLimitMargin || cj.y0 + 64 + R > H + kLimitMargin) ? 1 : 0;
            cj.sess = 0;
            cj.slot_base = j * kSlots;
            jobs.push_back(cj);
            slots.resize(slots.size() + kSlots, -1);
        }
        CtuJob &cj = jobs[j];
        int32_t &slot = slots[(size_t)cj.slot_base + s];
        if (cj.mvp_x != u.mvp_x || cj.mvp_y != u.mvp_y || slot >= 0) { generic.push_back(i); continue; }
        slot = i;
        cj.levels |= (uint8_t)(s < 576 ? 1 : s < 784 ? 2 : s < 836 ? 4 : 8);
    }
    if ((int)jobs.size() > p.cap_jobs) {
        if (p.d_jobs) cudaFree(p.d_jobs);
        if (p.d_slots) cudaFree(p.d_slots);
        p.cap_jobs = (int)jobs.size() + 16;
        XG_CUDA(cudaMalloc((void **)&p.d_jobs, sizeof(CtuJob) * p.cap_jobs));
        XG_CUDA(cudaMalloc((void **)&p.d_slots, sizeof(int32_t) * kSlots * p.cap_jobs));
    }
    p.n_jobs = (int)jobs.size();
    p.n_border = 0;
    for (const CtuJob &j : jobs) p.n_border += j.border ? 1 : 0;
    p.h_jobs = jobs;
    if (p.n_jobs) {
        XG_CUDA(cudaMemcpyAsync(p.d_jobs, jobs.data(), sizeof(CtuJob) * p.n_jobs, cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaMemcpyAsync(p.d_slots, slots.data(), sizeof(int32_t) * slots.size(), cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaStreamSynchronize(st));
    }
}

// ww: row pitch of the window (bytes), a multiple of 128 that holds the
// 64 + 2R + 8 bytes a row needs after its swizzle shift.
static inline size_t ctu_smem_bytes(int R, int &ww, bool staging)
{
    ww = (int)align_up((size_t)64 + 2 * R + 8 + 4 * kSwzMax + 4, 128);
    const size_t keys_win = 2 * sizeof(uint32_t) * kDyChunk * 2 * R + (size_t)(64 + kDyChunk - 1) * ww;
    // the TMA staging boxes and their barrier
    return staging ? keys_win + (size_t)tma_pieces(R) * kTmaPieceBytes + 16 : keys_win;
}

// The kernels' dynamic shared-memory limit (the largest range's need), once
// per device; launches and occupancy queries come after it.
static void ctu_attrs(int dev)
{
    static std::atomic<bool> done[64];
    if (dev < 0 || dev >= 64 || done[dev].load(std::memory_order_acquire)) return;
    int ww_max;
    const int maxb = (int)ctu_smem_bytes(128, ww_max, XG_CTU_TMA != 0);
    XG_CUDA(cudaFuncSetAttribute(fs_ctu_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxb));
    XG_CUDA(cudaFuncSetAttribute(fs_ctu_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxb));
    XG_CUDA(cudaFuncSetAttribute(fs_ctu_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxb));
    XG_CUDA(cudaFuncSetAttribute(fs_ctu_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxb));
    done[dev].store(true, std::memory_order_release);
}

// Dynamic shared memory of a launch of variant (border, pair) at range R:
// with the TMA staging area where it costs no CTA per SM (it would from
// R = 96 on in the two-row form), else without (the CTAs then fill their
// windows with 16-byte loads).  Cached per device, variant and range.
template <bool BORDER, bool PAIR>
static size_t ctu_launch_smem(int dev, int R, int &ww)
{
    static std::atomic<int> choice[64][129];   // 0 unknown, 1 without, 2 with (threads agree)
    const size_t base = ctu_smem_bytes(R, ww, false);
#if XG_CTU_TMA
    if (dev < 0 || dev >= 64 || R < 1 || R > 128) return base;
    std::atomic<int> &slot = choice[dev][R];
    int c = slot.load(std::memory_order_relaxed);
    if (c == 0) {
        ctu_attrs(dev);
        int wwt, nb = 0, nt = 0;
        const size_t with = ctu_smem_bytes(R, wwt, true);
        const bool ok = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fs_ctu_kernel<BORDER, PAIR>, kCtuThreads,
                                                                      base) == cudaSuccess &&
                        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nt, fs_ctu_kernel<BORDER, PAIR>, kCtuThreads,
                                                                      with) == cudaSuccess;
        if (!ok) cudaGetLastError();
        c = ok && nb > 0 && nt >= nb ? 2 : 1;
        slot.store(c, std::memory_order_relaxed);
    }
    return c == 2 ? ctu_smem_bytes(R, ww, true) : base;
#else
    (void)dev;
    return base;
#endif
}

// Run the border variant on a side stream forked from the caller's, so its
// CTAs fill the SMs the interior launch's last wave leaves idle (and the
// reverse); joined back before the call returns.
#ifndef XG_CTU_FORK
#define XG_CTU_FORK 1
#endif

// A side stream and its fork / join events, per host thread and device
// (a thread's launches are sequenced, so they may share them; the fork and
// the join happen within one call, so stream capture sees a complete
// fork-join).
struct CtuSide {
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~CtuSide()   // at thread exit (a pool's threads do not keep theirs)
    {
        if (join) cudaEventDestroy(join);
        if (fork) cudaEventDestroy(fork);
        if (st) cudaStreamDestroy(st);
    }
};
static CtuSide *ctu_side(int dev, int k = 0)   // k: 0 the search's own, 1 the per-PU search's
{
    thread_local CtuSide side[2][64];
    if (dev < 0 || dev >= 64 || k < 0 || k > 1) return nullptr;
    CtuSide &s = side[k][dev];
    if (!s.st) {
        if (cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;   // the launches then stay on the caller's stream
        }
    }
    return &s;
}

// Creates what a search at range R launches with on this thread -- the side
// stream and the shared-memory choices -- ahead of a stream capture.
static void ctu_prime(int R)
{
    const int dev = current_device();
    int ww;
    if (XG_CTU_FORK) {
        ctu_side(dev, 0);
        ctu_side(dev, 1);
    }
    if (R < 1 || R > 128) return;
    if (R >= XG_CTU_PAIR_MIN_R) {
        ctu_launch_smem<false, true>(dev, R, ww);
        ctu_launch_smem<true, true>(dev, R, ww);
    } else {
        ctu_launch_smem<false, false>(dev, R, ww);
        ctu_launch_smem<true, false>(dev, R, ww);
    }
}

// One launch of each variant over `n_jobs` jobs (sessions per job.sess).
// n_border of the jobs need the border variant; a variant with no job of
// its kind is not launched.
static void ctu_jobs_run(const CtuJob *d_jobs, int n_jobs, int n_border, const SessView *d_views,
                         const xavs2gpu_me_params_t &prm, cudaStream_t st)
{
    if (n_jobs == 0) return;
    const int R = prm.search_range;
    int ww;
    const int dev = current_device();
    ctu_attrs(dev);
    const int nchunks = (2 * R + kDyChunk - 1) / kDyChunk;
    const int grid = n_jobs * nchunks;
    const bool pair = R >= XG_CTU_PAIR_MIN_R;
    const int lam = prm.lambda_factor;
    // the border launch on the side stream when both variants run
    CtuSide *side = XG_CTU_FORK && n_border > 0 && n_border < n_jobs ? ctu_side(dev) : nullptr;
    cudaStream_t bst = st;
    if (side) {
        XG_CUDA(cudaEventRecord(side->fork, st));
        XG_CUDA(cudaStreamWaitEvent(side->st, side->fork, 0));
        bst = side->st;
    }
    if (n_border < n_jobs) {
        if (pair) {
            const size_t smem = ctu_launch_smem<false, true>(dev, R, ww);
            fs_ctu_kernel<false, true><<<grid, kCtuThreads, smem, st>>>(d_jobs, nchunks, d_views, R, lam, ww);
        } else {
            const size_t smem = ctu_launch_smem<false, false>(dev, R, ww);
            fs_ctu_kernel<false, false><<<grid, kCtuThreads, smem, st>>>(d_jobs, nchunks, d_views, R, lam, ww);
        }
        count_launch();
    }
    if (n_border > 0) {
        if (pair) {
            const size_t smem = ctu_launch_smem<true, true>(dev, R, ww);
            fs_ctu_kernel<true, true><<<grid, kCtuThreads, smem, bst>>>(d_jobs, nchunks, d_views, R, lam, ww);
        } else {
            const size_t smem = ctu_launch_smem<true, false>(dev, R, ww);
            fs_ctu_kernel<true, false><<<grid, kCtuThreads, smem, bst>>>(d_jobs, nchunks, d_views, R, lam, ww);
        }
        count_launch();
    }
    if (side) {
        XG_CUDA(cudaEventRecord(side->join, side->st));
        XG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
    }
}

}  // namespace xg
