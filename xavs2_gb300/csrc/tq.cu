// tq.cu -- the batched TU reconstruction chain for sm_103a:
// dct (or the 4x4 secondary transform) -> quant -> [dequant -> idct when a
// level is non-zero] for every block of a batch, the order of the
// reference's TU reconstruction (rdo.c:1333-1370, 876-947) with the
// transforms of transform.c:1123-1587 and the quantiser of quant.c:108-184.
//
// Three launches per batch:
//   1. count the blocks of every TU shape (invalid descriptors get nnz = -1);
//   2. scatter the block indices into one list grouped by shape, largest
//      shapes first, so that at any moment the warps of the persistent
//      kernel run the code of one shape (a mixed order thrashes the
//      instruction cache);
//   3. the persistent chain kernel: a warp takes G = 32 / L TUs of one shape
//      at a time (L lanes per TU: one lane per line of the larger side).
// Every 1-D pass runs with one line per lane: the line's 16-bit values are
// packed in pairs and each output is a dot product with a byte-packed basis
// row, two products per dp2a instruction.  All pass inputs are 16-bit (the
// residual, the forward first pass's int16 output, the clipped dequantised
// levels, the inverse first pass's 16-bit clip), so the 32-bit sums are
// exactly the reference's sums before its rounding shifts.  Passes hand over
// through shared memory (transposes).  The 64-point shapes run the 5/3
// wavelet around the 32-point core (wavelet_fwd_d / wavelet_inv_d in
// transform.cu; transform.c:586-951).
#include "transform_tables.cuh"

#include <algorithm>
#include <vector>

namespace xg {
namespace tqw {

// The forward transforms' even/odd fold on packed 16-bit pairs.
#ifndef XG_TQ_PACKED_FOLD
#define XG_TQ_PACKED_FOLD 1
#endif

// ---- byte-packed basis rows --------------------------------------------------
// Forward table of an N-point transform: row k holds T_N[k][0..N) as N/4
// words (byte j of word w = T_N[k][4w + j]).  Inverse table: row n holds
// T_N[0..N)[n].  N = 4, 8, 16, 32 at word offsets 0, 4, 20, 84; then the 4x4
// secondary transform M (rows of M, resp. of M^T) at 340; then, for the
// even/odd split of N = 8, 16, 32 (at 344, 348, 364), the odd rows on half a
// line: forward row k < N/2 holds T_N[2k+1][0..N/2), inverse row n < N/2
// holds T_N[2k+1][n] over k < N/2.
constexpr int kTabWords = 428;
struct PackedTab { uint32_t w[kTabWords]; };

__host__ __device__ constexpr int tab_off(int N) { return N == 4 ? 0 : N == 8 ? 4 : N == 16 ? 20 : 84; }
__host__ __device__ constexpr int odd_off(int N) { return N == 8 ? 344 : N == 16 ? 348 : 364; }
constexpr int kSec = 340;

constexpr int sec4c(int i, int k)
{
    constexpr int8_t m[16] = {34, 58, 72, 81, 77, 69, -7, -75, 79, -33, -75, 58, 55, -84, 73, -28};
    return m[i * 4 + k];
}

constexpr PackedTab make_tab(bool inverse)
{
    PackedTab t{};
    for (int N = 4; N <= 32; N *= 2)
        for (int r = 0; r < N; r++)
            for (int j = 0; j < N; j++) {
                const int v = inverse ? basis32(j * (32 / N), r) : basis32(r * (32 / N), j);
                const int word = tab_off(N) + r * (N / 4) + j / 4;
                t.w[word] |= (uint32_t)(uint8_t)(int8_t)v << (8 * (j % 4));
            }
    for (int r = 0; r < 4; r++)
        for (int j = 0; j < 4; j++) {
            const int v = inverse ? sec4c(j, r) : sec4c(r, j);
            t.w[kSec + r] |= (uint32_t)(uint8_t)(int8_t)v << (8 * j);
        }
    for (int N = 8; N <= 32; N *= 2)
        for (int r = 0; r < N / 2; r++)
            for (int j = 0; j < N / 2; j++) {
                const int v = inverse ? basis32((2 * j + 1) * (32 / N), r) : basis32((2 * r + 1) * (32 / N), j);
                const int word = odd_off(N) + r * (N / 8) + j / 4;
                t.w[word] |= (uint32_t)(uint8_t)(int8_t)v << (8 * (j % 4));
            }
    return t;
}

static __constant__ PackedTab c_fwd = make_tab(false);
static __constant__ PackedTab c_inv = make_tab(true);

__device__ __forceinline__ uint32_t pack16(int a, int b) { return (uint32_t)(a & 0xFFFF) | ((uint32_t)b << 16); }
__device__ __forceinline__ int clipb(int v, int bits)
{
    const int hi = (1 << (bits - 1)) - 1;
    return min(max(v, -hi - 1), hi);
}

// sum_j row[j] * x[j] for the N values packed in pairs in xp; row = N/4 words
template <int N>
__device__ __forceinline__ int dot_row(const uint32_t (&xp)[N / 2], const uint32_t *row)
{
    int s = 0;
#pragma unroll
    for (int w = 0; w < N / 4; w++) {
        const uint32_t b = row[w];
        s = __dp2a_lo((int)xp[2 * w], (int)b, s);
        s = __dp2a_hi((int)xp[2 * w + 1], (int)b, s);
    }
    return s;
}

// pairs of a shared-memory line of N int16 (4-byte aligned)
template <int N>
__device__ __forceinline__ void load_pairs(const int16_t *p, uint32_t (&xp)[N / 2])
{
    const uint32_t *w = reinterpret_cast<const uint32_t *>(p);
#pragma unroll
    for (int i = 0; i < N / 2; i++) xp[i] = w[i];
}

// pairs of a global line of N int16 (16-byte aligned when `al` and N >= 8,
// 8-byte aligned when `al` and N == 4)
template <int N>
__device__ __forceinline__ void load_pairs_global(const int16_t *p, bool al, uint32_t (&xp)[N / 2])
{
    if constexpr (N >= 8) {
        if (al) {
#pragma unroll
            for (int q = 0; q < N / 8; q++) {
                const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p) + q);
                xp[4 * q] = v.x; xp[4 * q + 1] = v.y; xp[4 * q + 2] = v.z; xp[4 * q + 3] = v.w;
            }
            return;
        }
    } else {
        if (al) {
            const uint2 v = __ldg(reinterpret_cast<const uint2 *>(p));
            xp[0] = v.x; xp[1] = v.y;
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < N / 2; i++) xp[i] = pack16(p[2 * i], p[2 * i + 1]);
}

// Forward N-point transform (N >= 8) of one line by a single even/odd split:
// y[2k] = T_{N/2} (x[n] + x[N-1-n]), y[2k+1] = odd rows . (x[n] - x[N-1-n]),
// both as dp2a dot products over the folded values packed in pairs.  The
// folded values must fit 16 bits; `bad` reports a line where they do not
// (the caller then takes the full-matrix product).  out(k, y[k]).
template <int N>
__device__ __forceinline__ void fold_line(const uint32_t (&xp)[N / 2], uint32_t (&ep)[N / 4], uint32_t (&op)[N / 4],
                                          bool &bad)
{
#if XG_TQ_PACKED_FOLD
    // on the packed pairs: (x[2m], x[2m+1]) +- (x[N-1-2m], x[N-2-2m]), the
    // second the half-swapped pair N/2-1-m; a 16-bit sum is exact iff the
    // wrapping and the saturating forms agree (the wrapped value of an
    // overflowing sum of two int16 is never the saturation bound)
    uint32_t ov = 0;
#pragma unroll
    for (int m = 0; m < N / 4; m++) {
        const uint32_t a = xp[m], b = __byte_perm(xp[N / 2 - 1 - m], 0, 0x1032);
        const uint32_t e = __vadd2(a, b), o = __vsub2(a, b);
        ov |= (e ^ __vaddss2(a, b)) | (o ^ __vsubss2(a, b));
        ep[m] = e;
        op[m] = o;
    }
    bad |= ov != 0;
#else
    int x[N];
#pragma unroll
    for (int i = 0; i < N / 2; i++) {
        x[2 * i] = (int)(int16_t)(xp[i] & 0xFFFFu);
        x[2 * i + 1] = ((int)xp[i]) >> 16;
    }
#pragma unroll
    for (int m = 0; m < N / 4; m++) {
        const int e0 = x[2 * m] + x[N - 1 - 2 * m], e1 = x[2 * m + 1] + x[N - 2 - 2 * m];
        const int o0 = x[2 * m] - x[N - 1 - 2 * m], o1 = x[2 * m + 1] - x[N - 2 - 2 * m];
        bad |= (unsigned)(e0 + 32768) > 65535u || (unsigned)(e1 + 32768) > 65535u ||
               (unsigned)(o0 + 32768) > 65535u || (unsigned)(o1 + 32768) > 65535u;
        ep[m] = pack16(e0, e1);
        op[m] = pack16(o0, o1);
    }
#endif
}

template <int N, typename Out>
__device__ __forceinline__ void fwd_folded(const uint32_t (&ep)[N / 4], const uint32_t (&op)[N / 4], Out out)
{
    const uint32_t *fe = &c_fwd.w[tab_off(N / 2)], *fo = &c_fwd.w[odd_off(N)];
#pragma unroll 2
    for (int k = 0; k < N / 2; k++) {
        out(2 * k, dot_row<N / 2>(ep, fe + k * (N / 8)));
        out(2 * k + 1, dot_row<N / 2>(op, fo + k * (N / 8)));
    }
}

// Inverse N-point transform (N >= 8) of one line of 16-bit coefficients
// (always exact): x[n] = E[n] + O[n], x[N-1-n] = E[n] - O[n] with E the
// N/2-point inverse of the even coefficients and O the odd rows.
template <int N, typename Out>
__device__ __forceinline__ void inv_split(const uint32_t (&cp)[N / 2], Out out)
{
    uint32_t ce[N / 4], co[N / 4];
#pragma unroll
    for (int m = 0; m < N / 4; m++) {
        ce[m] = __byte_perm(cp[2 * m], cp[2 * m + 1], 0x5410);
        co[m] = __byte_perm(cp[2 * m], cp[2 * m + 1], 0x7632);
    }
    const uint32_t *ie = &c_inv.w[tab_off(N / 2)], *io = &c_inv.w[odd_off(N)];
#pragma unroll 2
    for (int n = 0; n < N / 2; n++) {
        const int e = dot_row<N / 2>(ce, ie + n * (N / 8));
        const int o = dot_row<N / 2>(co, io + n * (N / 8));
        out(n, e + o);
        out(N - 1 - n, e - o);
    }
}

// The wavelet's forward lifting on 32-bit words (two samples each), a chunk
// of each row loaded before the in-place stores, instead of one 16-bit
// sample per step.
#ifndef XG_TQ_LIFT_WORDS
#define XG_TQ_LIFT_WORDS 1
#endif
// The inverse upsampling reads the low band 4 rows ahead of its stores.
#ifndef XG_TQ_UPS_CHUNK
#define XG_TQ_UPS_CHUNK 1
#endif

// ---- shapes ------------------------------------------------------------------
template <int PART> struct Shape;
#define XG_TQ_SHAPE(P, IW_, IH_, TW_, TH_, S1_, S2_)                                                               \
    template <> struct Shape<P> {                                                                                  \
        static constexpr int IW = IW_, IH = IH_, TW = TW_, TH = TH_, S1 = S1_, S2 = S2_;                           \
        static constexpr bool WAV = IW_ != TW_ || IH_ != TH_;                                                      \
        static constexpr int L = WAV ? 32 : (TW_ > TH_ ? TW_ : TH_);                                               \
        static constexpr int G = 32 / L;                                                                           \
    };
XG_TQ_SHAPE(0, 4, 4, 4, 4, 0, 7)
XG_TQ_SHAPE(1, 8, 8, 8, 8, 1, 8)
XG_TQ_SHAPE(2, 16, 16, 16, 16, 2, 9)
XG_TQ_SHAPE(3, 32, 32, 32, 32, 3, 10)
XG_TQ_SHAPE(15, 16, 4, 16, 4, 2, 7)
XG_TQ_SHAPE(16, 4, 16, 4, 16, 0, 9)
XG_TQ_SHAPE(19, 32, 8, 32, 8, 3, 8)
XG_TQ_SHAPE(20, 8, 32, 8, 32, 1, 10)
XG_TQ_SHAPE(4, 64, 64, 32, 32, 4, 10)
XG_TQ_SHAPE(23, 64, 16, 32, 8, 3, 7)
XG_TQ_SHAPE(24, 16, 64, 8, 32, 2, 10)
#undef XG_TQ_SHAPE

// processing order: largest shapes first; TUs per warp of each class
constexpr int kNumClasses = 11;
__constant__ int c_class_part[kNumClasses] = {4, 23, 24, 3, 19, 20, 2, 15, 16, 1, 0};
__host__ __device__ constexpr int class_g(int c) { return c < 6 ? 1 : c < 9 ? 2 : c == 9 ? 4 : 8; }

__device__ __forceinline__ int class_of(int part)
{
    switch (part) {
    case 4: return 0; case 23: return 1; case 24: return 2; case 3: return 3; case 19: return 4; case 20: return 5;
    case 2: return 6; case 15: return 7; case 16: return 8; case 1: return 9; case 0: return 10;
    default: return -1;
    }
}

__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v / 2); }

// Per-warp shared memory: region A holds the wavelet input (64 rows, pitch
// 66 int16; the horizontal lifting leaves each row's low band in its first
// half) or the transposes and the output staging of the warp's G TUs;
// region B the wavelet's LL band (up to 32 rows, pitch 34 int16) and later
// the inverse transform's output for the upsampling.
constexpr int kRegionA = 64 * 66 * 2, kRegionB = 32 * 34 * 2;

struct Ctx {
    const xavs2gpu_tq_block_t *blocks;
    const int16_t *residual;
    int16_t *coef, *recon;
    int32_t *nnz;
};

// One group of up to G TUs of shape PART; `idx` = the block index of this
// lane's sub-warp (-1: no TU).
template <int PART, int RA = kRegionA>
__device__ __noinline__ void tu_group(const Ctx &cx, int idx, int lane, uint8_t *smem)
{
    using S = Shape<PART>;
    constexpr int IW = S::IW, IH = S::IH, TW = S::TW, TH = S::TH, L = S::L;
    constexpr int P1 = TH + 2, P2 = TW + 2;       // transpose pitches (int16, even)
    constexpr int F = S::WAV ? 1 : 0;
    constexpr int LEVEL = (ilog2c(IW) + ilog2c(IH)) >> 1;
    const int sub = lane / L, l = lane % L;
    const bool act = idx >= 0;
    xavs2gpu_tq_block_t b{};
    if (act) b = cx.blocks[idx];
    const bool sec = PART == 0 && (b.flags & 2);
    static_assert(S::WAV ? RA == kRegionA : RA / 2 / S::G >= 2 * TW * (TH + 2) + TW * TH,
                  "region A holds the transposes and the staging of every TU of the group");
    int16_t *tA = reinterpret_cast<int16_t *>(smem) + sub * (RA / 2 / S::G);
    int16_t *tB = reinterpret_cast<int16_t *>(smem + kRegionA);
    const int16_t *src = cx.residual + b.offset;
    const bool al_in = (reinterpret_cast<uintptr_t>(src) & 15) == 0;

    // ---- forward rows -> T1[k][j] (pitch P1) in region A
    uint32_t xp[TW / 2];
    if constexpr (S::WAV) {
        constexpr int PX = 66, PL = TW + 2;
        if (act) {
            if (al_in) {
                // the lane's 16-byte loads in batches of 8 (a batch is one
                // memory round trip), then the word stores into the padded rows
                constexpr int NV = IW * IH / 8 / 32, NB = NV < 8 ? NV : 8;
#pragma unroll 1
                for (int k0 = 0; k0 < NV; k0 += NB) {
                    uint4 v[NB];
#pragma unroll
                    for (int k = 0; k < NB; k++) v[k] = __ldg(reinterpret_cast<const uint4 *>(src) + lane + 32 * (k0 + k));
#pragma unroll
                    for (int k = 0; k < NB; k++) {
                        const int e = lane + 32 * (k0 + k);
                        uint32_t *d = reinterpret_cast<uint32_t *>(tA + ((e * 8) / IW) * PX + (e * 8) % IW);
                        d[0] = v[k].x; d[1] = v[k].y; d[2] = v[k].z; d[3] = v[k].w;
                    }
                }
            } else {
                for (int e = lane; e < IW * IH; e += 32) tA[(e / IW) * PX + e % IW] = src[e];
            }
        }
        __syncwarp();
        // horizontal lifting, one row per lane: odd[m] = p[2m+1] - (p[2m] +
        // p[2m+2]) >> 1, H[m] = p[2m] + (odd[m-1] + odd[m] + 2) >> 2, int16
        // after each step, mirrored ends (p[IW] = p[IW-2], odd[-1] = odd[0]);
        // H[m] goes to sample m of the same row (the samples still to be
        // read, 2m+1 on, lie beyond it)
        if (act) {
#if XG_TQ_LIFT_WORDS
            // the row as words (samples 2m, 2m+1), 8 words per chunk loaded
            // before any store; H[c..c+8) stored as 4 words behind the reads
            constexpr int NW = IW / 2;
            static_assert(NW % 8 == 0 && PX % 2 == 0, "word-wise lifting: rows of 16k samples, even pitch");
            for (int r = lane; r < IH; r += 32) {
                uint32_t *pw = reinterpret_cast<uint32_t *>(tA + r * PX);
                int prev_odd = 0, pe = (int)(int16_t)(pw[0] & 0xFFFFu);
#pragma unroll 1
                for (int c = 0; c < NW; c += 8) {
                    uint32_t w[9];
#pragma unroll
                    for (int k = 0; k < 8; k++) w[k] = pw[c + k];
                    w[8] = c + 8 < NW ? pw[c + 8] : w[7];   // last row: p[IW] mirrors to p[IW-2]
                    uint32_t hw[4];
                    int hl = 0;
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        const int po = (int)w[k] >> 16, pn = (int)(int16_t)(w[k + 1] & 0xFFFFu);
                        const int odd = (int16_t)(po - ((pe + pn) >> 1));
                        if (c + k == 0) prev_odd = odd;
                        const int h = (int16_t)(pe + ((prev_odd + odd + 2) >> 2));
                        prev_odd = odd;
                        pe = pn;
                        if (k & 1) hw[k >> 1] = pack16(hl, h);
                        else hl = h;
                    }
#pragma unroll
                    for (int k = 0; k < 4; k++) pw[c / 2 + k] = hw[k];
                }
            }
#else
            for (int r = lane; r < IH; r += 32) {
                int16_t *p = tA + r * PX;
                int prev_odd = 0, pe = p[0];
                for (int m = 0; m < IW / 2; m++) {
                    const int po = p[2 * m + 1], pn = m + 1 < IW / 2 ? p[2 * m + 2] : p[IW - 2];
                    const int odd = (int16_t)(po - ((pe + pn) >> 1));
                    if (m == 0) prev_odd = odd;
                    p[m] = (int16_t)(pe + ((prev_odd + odd + 2) >> 2));
                    prev_odd = odd;
                    pe = pn;
                }
            }
#endif
        }
        __syncwarp();
        // vertical lifting, one LL row per lane (j < TH), into region B:
        // odd'[m] = q[2m+1] - (q[2m] + q[2m+2]) >> 1,
        // LL[m] = 2 q[2m] + (odd'[m-1] + odd'[m] + 1) >> 1
        if (act && lane < TH) {
            const int j = lane;
            const int rm2 = j == 0 ? 2 : 2 * j - 2, rm1 = j == 0 ? 1 : 2 * j - 1;
            const int rp1 = 2 * j + 1, rp2 = j == TH - 1 ? 2 * j : 2 * j + 2;
#if XG_TQ_LIFT_WORDS
            // two columns per word, 4 words of each of the 5 rows per chunk
            static_assert(TW % 8 == 0 && PL % 2 == 0, "word-wise vertical lifting");
            const uint32_t *qa = reinterpret_cast<const uint32_t *>(tA + rm2 * PX);
            const uint32_t *qb = reinterpret_cast<const uint32_t *>(tA + rm1 * PX);
            const uint32_t *qc = reinterpret_cast<const uint32_t *>(tA + 2 * j * PX);
            const uint32_t *qd = reinterpret_cast<const uint32_t *>(tA + rp1 * PX);
            const uint32_t *qe = reinterpret_cast<const uint32_t *>(tA + rp2 * PX);
            uint32_t *ow = reinterpret_cast<uint32_t *>(tB + j * PL);
            auto ll = [](int a, int b, int c, int d, int e) {
                const int oa = (int16_t)(b - ((a + c) >> 1));
                const int ob = (int16_t)(d - ((c + e) >> 1));
                return (int16_t)((c << 1) + ((oa + ob + 1) >> 1));
            };
            auto lo = [](uint32_t v) { return (int)(int16_t)(v & 0xFFFFu); };
            auto hi = [](uint32_t v) { return (int)v >> 16; };
#pragma unroll 1
            for (int i0 = 0; i0 < TW / 2; i0 += 4) {
                uint32_t a[4], b[4], c[4], d[4], e[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    a[k] = qa[i0 + k]; b[k] = qb[i0 + k]; c[k] = qc[i0 + k]; d[k] = qd[i0 + k]; e[k] = qe[i0 + k];
                }
#pragma unroll
                for (int k = 0; k < 4; k++)
                    ow[i0 + k] = pack16(ll(lo(a[k]), lo(b[k]), lo(c[k]), lo(d[k]), lo(e[k])),
                                        ll(hi(a[k]), hi(b[k]), hi(c[k]), hi(d[k]), hi(e[k])));
            }
#else
            for (int i = 0; i < TW; i++) {
                const int qa = tA[rm2 * PX + i], qb = tA[rm1 * PX + i], qc = tA[2 * j * PX + i];
                const int qd = tA[rp1 * PX + i], qe = tA[rp2 * PX + i];
                const int oa = (int16_t)(qb - ((qa + qc) >> 1));
                const int ob = (int16_t)(qd - ((qc + qe) >> 1));
                tB[j * PL + i] = (int16_t)((qc << 1) + ((oa + ob + 1) >> 1));
            }
#endif
        }
        __syncwarp();
        if (act && lane < TH) load_pairs<TW>(tB + lane * PL, xp);
        __syncwarp();
    } else {
        if (act && l < TH) load_pairs_global<TW>(src + l * TW, al_in, xp);
    }
    if (act && l < TH) {
        bool done = false;
        if constexpr (PART == 0) {
            if (sec) {
                for (int k = 0; k < 4; k++)
                    tA[k * P1 + l] = (int16_t)clipb((dot_row<4>(xp, &c_fwd.w[kSec + k]) + 1) >> 1, 16);
                done = true;
            }
        }
        if (!done) {
            auto put = [&](int k, int v) { tA[k * P1 + l] = (int16_t)((v + ((1 << S::S1) >> 1)) >> S::S1); };
            bool full = TW < 8;
            if constexpr (TW >= 8) {
                uint32_t ep[TW / 4], op[TW / 4];
                bool bad = false;
                fold_line<TW>(xp, ep, op, bad);
                full = __any_sync(__activemask(), bad);
                if (!full) fwd_folded<TW>(ep, op, put);
            }
            if (full) {
                const uint32_t *rows = &c_fwd.w[tab_off(TW)];
#pragma unroll 2
                for (int k = 0; k < TW; k++) put(k, dot_row<TW>(xp, rows + k * (TW / 4)));
            }
        }
    }
    __syncwarp();

    // ---- forward columns + quant (lane l < TW holds column l): levels to
    // global, dequantised levels back into T1 row l
    const int qshift = 22 - LEVEL;
    const int qadd = (int)(((int64_t)1 << (qshift + (b.flags & 1))) * 5 / 31);
    const int qscale = c_q_scale[b.qp & 127];
    const int dqshift = iq_shift_of(b.qp) + 9 + LEVEL - 16;
    const int dqscale = c_iq_scale[b.qp & 127];
    int nz = 0;
    if (act && l < TW) {
        uint32_t cp[TH / 2];
        load_pairs<TH>(tA + l * P1, cp);
        int16_t *co = cx.coef + b.coef_offset + l;
        auto put = [&](int m, int s) {
            const int y = sec ? clipb((s + 128) >> 8, 16) : (int)(int16_t)((s + ((1 << S::S2) >> 1)) >> S::S2);
            const int a = (y < 0 ? -y : y) * qscale + qadd;
            const int q = y < 0 ? -(a >> qshift) : (a >> qshift);
            co[m * TW] = (int16_t)q;
            nz += q != 0;
            tA[l * P1 + m] = (int16_t)clipb((q * dqscale + (1 << (dqshift - 1))) >> dqshift, 16);
        };
        bool full = TH < 8;
        if constexpr (TH >= 8) {
            uint32_t ep[TH / 4], op[TH / 4];
            bool bad = false;
            fold_line<TH>(cp, ep, op, bad);
            full = __any_sync(__activemask(), bad);
            if (!full) fwd_folded<TH>(ep, op, put);
        }
        if (full) {
            const uint32_t *rows = sec ? &c_fwd.w[kSec] : &c_fwd.w[tab_off(TH)];
#pragma unroll 2
            for (int m = 0; m < TH; m++) put(m, dot_row<TH>(cp, rows + m * (TH / 4)));
        }
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) nz += __shfl_xor_sync(0xffffffffu, nz, o);
    if (act && l == 0) cx.nnz[idx] = nz;
    int16_t *dst = cx.recon + b.offset;
    const bool al_out = (reinterpret_cast<uintptr_t>(dst) & 15) == 0;
    if (act && nz == 0) {
        if (al_out)
            for (int i = l; i < IW * IH / 8; i += L) reinterpret_cast<uint4 *>(dst)[i] = make_uint4(0, 0, 0, 0);
        else
            for (int i = l; i < IW * IH; i += L) dst[i] = 0;
    }
    const bool inv = act && nz != 0;
    __syncwarp();

    // ---- inverse columns: lane l < TW -> T2[n][l] (pitch P2) after T1
    int16_t *t2 = tA + TW * P1;
    if (inv && l < TW) {
        uint32_t cp[TH / 2];
        load_pairs<TH>(tA + l * P1, cp);
        auto put = [&](int n, int v) { t2[n * P2 + l] = (int16_t)clipb((v + 16) >> 5, 16); };
        if constexpr (TH >= 8) {
            inv_split<TH>(cp, put);
        } else {
            const uint32_t *rows = sec ? &c_inv.w[kSec] : &c_inv.w[tab_off(TH)];
#pragma unroll 2
            for (int n = 0; n < TH; n++) put(n, dot_row<TH>(cp, rows + n * (TH / 4)));
        }
    }
    __syncwarp();

    // ---- inverse rows: lane l < TH; rows staged after T2 (or, for the
    // wavelet shapes, into region B for the upsampling)
    int16_t *stage = S::WAV ? tB : t2 + TH * P2;
    constexpr int PS = S::WAV ? TW + 2 : TW;
    if (inv && l < TH) {
        uint32_t vp[TW / 2];
        load_pairs<TW>(t2 + l * P2, vp);
        const uint32_t *rows = sec ? &c_inv.w[kSec] : &c_inv.w[tab_off(TW)];
        const int sh = sec ? 14 : 12 - F, bits = sec ? 9 : 9 + F;
        int16_t *o = stage + l * PS;
        auto put = [&](int x, int v) { o[x] = (int16_t)clipb((v + (1 << (sh - 1))) >> sh, bits); };
        if constexpr (TW >= 8) {
            inv_split<TW>(vp, put);
        } else {
#pragma unroll 2
            for (int x = 0; x < TW; x++) put(x, dot_row<TW>(vp, rows + x * (TW / 4)));
        }
    }
    __syncwarp();
    if constexpr (!S::WAV) {
        if (inv) {
            if (al_out) {
                for (int i = l; i < TW * TH / 8; i += L) {
                    const uint32_t *w = reinterpret_cast<const uint32_t *>(stage + 8 * i);
                    reinterpret_cast<uint4 *>(dst)[i] = make_uint4(w[0], w[1], w[2], w[3]);
                }
            } else {
                for (int i = l; i < TW * TH; i += L) dst[i] = stage[i];
            }
        }
    } else {
        // upsampling of the TW x TH low band in region B (pitch TW+2):
        // V[2y] = h[y], V[2y+1] = (h[y] + h[y+1]) >> 1 with h = LL >> 1 and
        // h[TH] = h[TH-1]; D[2i] = V[i], D[2i+1] = (V[i] + V[i+1]) >> 1 with
        // V[TW] = V[TW-1].  Lane i walks low-band column i down the rows and
        // writes output word i (samples 2i, 2i+1) of rows 2y and 2y+1: a
        // warp stores whole rows.
        if (inv && lane < TW) {
            const int i = lane, in1 = i + 1 < TW ? i + 1 : i;
            uint32_t *dw = reinterpret_cast<uint32_t *>(dst);
            int h0 = stage[i] >> 1, h1 = stage[in1] >> 1;
#if XG_TQ_UPS_CHUNK
            // low-band rows in chunks of 4: their reads before the stores
            static_assert(TH % 4 == 0, "upsampling by chunks of 4 rows");
#pragma unroll 1
            for (int y0 = 0; y0 < TH; y0 += 4) {
                int n0[4], n1[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int yn = y0 + k + 1 < TH ? y0 + k + 1 : TH - 1;
                    n0[k] = stage[yn * PS + i] >> 1;
                    n1[k] = stage[yn * PS + in1] >> 1;
                }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int v0 = (h0 + n0[k]) >> 1, v1 = (h1 + n1[k]) >> 1;
                    const uint32_t we = pack16(h0, (h0 + h1) >> 1), wo = pack16(v0, (v0 + v1) >> 1);
                    const int e = 2 * (y0 + k) * TW + i;
                    if (al_out) {
                        dw[e] = we;
                        dw[e + TW] = wo;
                    } else {
                        dst[2 * e] = (int16_t)(we & 0xFFFF);
                        dst[2 * e + 1] = (int16_t)(we >> 16);
                        dst[2 * (e + TW)] = (int16_t)(wo & 0xFFFF);
                        dst[2 * (e + TW) + 1] = (int16_t)(wo >> 16);
                    }
                    h0 = n0[k];
                    h1 = n1[k];
                }
            }
#else
            for (int y = 0; y < TH; y++) {
                const int yn = y + 1 < TH ? y + 1 : y;
                const int n0 = stage[yn * PS + i] >> 1, n1 = stage[yn * PS + in1] >> 1;
                const int v0 = (h0 + n0) >> 1, v1 = (h1 + n1) >> 1;
                const uint32_t we = pack16(h0, (h0 + h1) >> 1), wo = pack16(v0, (v0 + v1) >> 1);
                const int e = 2 * y * TW + i;
                if (al_out) {
                    dw[e] = we;
                    dw[e + TW] = wo;
                } else {
                    dst[2 * e] = (int16_t)(we & 0xFFFF);
                    dst[2 * e + 1] = (int16_t)(we >> 16);
                    dst[2 * (e + TW)] = (int16_t)(wo & 0xFFFF);
                    dst[2 * (e + TW) + 1] = (int16_t)(wo >> 16);
                }
                h0 = n0;
                h1 = n1;
            }
#endif
        }
    }
    __syncwarp();
}

// 1. per-class counts (warp-aggregated atomics)
__global__ void tq_count_kernel(const xavs2gpu_tq_block_t *__restrict__ blocks, int n, int *__restrict__ counts,
                                int32_t *__restrict__ nnz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = -1;
    if (i < n) {
        const xavs2gpu_tq_block_t b = blocks[i];
        c = (b.qp >= 0 && b.qp <= 79) ? class_of(b.part) : -1;
        if (c < 0) nnz[i] = -1;
    }
    const unsigned valid = __ballot_sync(0xffffffffu, c >= 0);
    if (c >= 0) {
        const unsigned same = __match_any_sync(valid, c);
        if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&counts[c], __popc(same));
    }
}

// 2. scatter into the class-ordered list (the order inside a class does not
//    matter: every TU writes only its own outputs)
__global__ void tq_scatter_kernel(const xavs2gpu_tq_block_t *__restrict__ blocks, int n, const int *__restrict__ counts,
                                  int *__restrict__ cursor, int *__restrict__ sorted)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int c = -1;
    if (i < n) {
        const xavs2gpu_tq_block_t b = blocks[i];
        c = (b.qp >= 0 && b.qp <= 79) ? class_of(b.part) : -1;
    }
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

// 3. the chain, persistent: warp-strided over the groups of the classes
//    [C0, C1), RA bytes of region A per warp (region B too when the range
//    holds the wavelet classes 0..2)
template <int WARPS, int C0, int C1, int RA, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) tq_chain_kernel(Ctx cx, const int *__restrict__ counts,
                                                                     const int *__restrict__ sorted)
{
    constexpr int kWarpBytes = C0 == 0 ? RA + kRegionB : RA;
    extern __shared__ __align__(16) uint8_t smem_raw[];
    uint8_t *smem = smem_raw + (threadIdx.x >> 5) * kWarpBytes;
    const int lane = threadIdx.x & 31;
    int cnt[kNumClasses], gstart[kNumClasses + 1], istart[kNumClasses];
    int acc = 0;
#pragma unroll
    for (int c = 0; c < kNumClasses; c++) {
        cnt[c] = counts[c];
        istart[c] = acc;
        acc += cnt[c];
    }
    gstart[C0] = 0;
#pragma unroll
    for (int c = C0; c < C1; c++) gstart[c + 1] = gstart[c] + (cnt[c] + class_g(c) - 1) / class_g(c);
    const int total = gstart[C1];
    const int nw = gridDim.x * WARPS;
    for (int item = blockIdx.x * WARPS + (threadIdx.x >> 5); item < total; item += nw) {
        int c = C0, gs = 0, is = istart[C0], cn = cnt[C0], G = class_g(C0);
#pragma unroll
        for (int k = C0 + 1; k < C1; k++)
            if (item >= gstart[k]) {
                c = k; gs = gstart[k]; is = istart[k]; cn = cnt[k]; G = class_g(k);
            }
        const int pos = (item - gs) * G + lane / (32 / G);
        const int idx = pos < cn ? sorted[is + pos] : -1;
        if constexpr (C0 == 0) {
            if (c < 3) {
                switch (c_class_part[c]) {
                case 4: tu_group<4>(cx, idx, lane, smem); break;
                case 23: tu_group<23>(cx, idx, lane, smem); break;
                default: tu_group<24>(cx, idx, lane, smem); break;
                }
                continue;
            }
        }
        if constexpr (C1 > 3) {
            switch (c_class_part[c]) {
            case 3: tu_group<3, RA>(cx, idx, lane, smem); break;
            case 19: tu_group<19, RA>(cx, idx, lane, smem); break;
            case 20: tu_group<20, RA>(cx, idx, lane, smem); break;
            case 2: tu_group<2, RA>(cx, idx, lane, smem); break;
            case 15: tu_group<15, RA>(cx, idx, lane, smem); break;
            case 16: tu_group<16, RA>(cx, idx, lane, smem); break;
            case 1: tu_group<1, RA>(cx, idx, lane, smem); break;
            default: tu_group<0, RA>(cx, idx, lane, smem); break;
            }
        }
    }
}

}  // namespace tqw

// Region A of the non-wavelet classes: the 32x32 TU's two transposes and its
// staging (2 x 32 x 34 + 32 x 32 int16).
constexpr int kRegionSmall = 6400;

// Build option: 1 runs the wavelet classes and the others as two launches,
// the latter with 6.4 KB of shared memory per warp and a register budget for
// more CTAs per SM; 0 one launch over all classes.
#ifndef XG_TQ_SPLIT
#define XG_TQ_SPLIT 1
#endif
#ifndef XG_TQ_SMALL_MINB
#define XG_TQ_SMALL_MINB 6
#endif
// resident CTAs of 4 warps per SM the register budgets are sized for: the
// wavelet classes at 5 (96 registers; 10.4 KB of shared memory per warp),
// the rest at 6 (85 registers; 6.25 KB)
#ifndef XG_TQ_BIG_MINB
#define XG_TQ_BIG_MINB 5
#endif

// One persistent launch of the chain over the classes [C0, C1): the shared-
// memory attribute and the occupancy are taken once per device and kernel
// instance (the statics belong to the instantiation).
template <int WARPS, int C0, int C1, int RA, int MINB>
static void tq_run(const tqw::Ctx &cx, const int *counts, const int *sorted, long long ctas_needed, int dev,
                   cudaStream_t st)
{
    constexpr int smem = WARPS * (C0 == 0 ? RA + tqw::kRegionB : RA);
    static bool attr_set[64] = {false};
    static int ctas_per_sm[64] = {0};
    if (!attr_set[dev]) {
        XG_CUDA(cudaFuncSetAttribute(tqw::tq_chain_kernel<WARPS, C0, C1, RA, MINB>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        XG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas_per_sm[dev], tqw::tq_chain_kernel<WARPS, C0, C1, RA, MINB>,
                                                              WARPS * 32, smem));
        if (ctas_per_sm[dev] < 1) ctas_per_sm[dev] = 1;
        attr_set[dev] = true;
    }
    long long grid = (long long)sm_count() * ctas_per_sm[dev];
    if (grid > ctas_needed) grid = ctas_needed;
    tqw::tq_chain_kernel<WARPS, C0, C1, RA, MINB><<<(int)grid, WARPS * 32, smem, st>>>(cx, counts, sorted);
}

template <int WARPS>
static int tq_launch_w(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                       int16_t *recon, int32_t *nnz, cudaStream_t stream)
{
    static bool pool_set[64] = {false};
    const int dev = current_device();
    if (dev < 0 || dev >= 64) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_tq_batch", "device index out of range");
        return XAVS2GPU_ERR_ARG;
    }
    if (!pool_set[dev]) {
        // keep freed stream-ordered scratch in the pool between batches
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool_set[dev] = true;
    }
    // scratch: class counts and cursors (32 ints each), then the ordered list
    int *scratch = nullptr;
    XG_CUDA(cudaMallocAsync((void **)&scratch, sizeof(int) * (64 + (size_t)n), stream));
    if (!scratch) return XAVS2GPU_ERR_CUDA;
    int *counts = scratch, *cursor = scratch + 32, *sorted = scratch + 64;
    XG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int) * 64, stream));
    const int nb = (n + 255) / 256;
    tqw::tq_count_kernel<<<nb, 256, 0, stream>>>(blocks, n, counts, nnz);
    tqw::tq_scatter_kernel<<<nb, 256, 0, stream>>>(blocks, n, counts, cursor, sorted);
    tqw::Ctx cx{blocks, residual, coef, recon, nnz};
    const long long ctas_needed = ((long long)n + WARPS - 1) / WARPS;
#if XG_TQ_SPLIT
    tq_run<WARPS, 0, 3, tqw::kRegionA, XG_TQ_BIG_MINB * 4 / WARPS>(cx, counts, sorted, ctas_needed, dev, stream);
    tq_run<WARPS, 3, tqw::kNumClasses, kRegionSmall, XG_TQ_SMALL_MINB * 4 / WARPS>(cx, counts, sorted, ctas_needed, dev,
                                                                                   stream);
    count_launch(4);
#else
    // 16 warps per SM (128 registers)
    tq_run<WARPS, 0, tqw::kNumClasses, tqw::kRegionA, 16 / WARPS>(cx, counts, sorted, ctas_needed, dev, stream);
    count_launch(3);
#endif
    XG_CUDA(cudaFreeAsync(scratch, stream));
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

// The batched TU chain with `warps` (4 or 8) warps per CTA.
int tq_batch_launch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                    int16_t *recon, int32_t *nnz, int warps, cudaStream_t stream)
{
    if (n < 0) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_tq_batch", "negative count");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    if (warps == 8) return tq_launch_w<8>(blocks, n, residual, coef, recon, nnz, stream);
    return tq_launch_w<4>(blocks, n, residual, coef, recon, nnz, stream);
}

}  // namespace xg

using namespace xg;

extern "C" int xavs2gpu_tq_batch(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual, int16_t *coef,
                                 int16_t *recon, int32_t *nnz, void *stream)
{
    return tq_batch_launch(blocks, n, residual, coef, recon, nnz, 4, (cudaStream_t)stream);
}

// ---- host-buffer form: copies and the chain overlapped by chunks ------------------
namespace {

struct HostTqCtx {
    int device = -1;
    cudaStream_t st[3] = {nullptr, nullptr, nullptr};   // copy in, chain, copy out
    std::vector<cudaEvent_t> ev_in, ev_done;
    xavs2gpu_tq_block_t *d_blocks = nullptr;
    int16_t *d_res = nullptr, *d_coef = nullptr, *d_rec = nullptr;
    int32_t *d_nnz = nullptr;
    size_t cap_blocks = 0, cap_nnz = 0, cap_res = 0, cap_rec = 0, cap_coef = 0;
    ~HostTqCtx()
    {
        if (device < 0) return;
        cudaSetDevice(device);
        for (auto s : st)
            if (s) cudaStreamDestroy(s);
        for (auto e : ev_in) cudaEventDestroy(e);
        for (auto e : ev_done) cudaEventDestroy(e);
        cudaFree(d_blocks); cudaFree(d_res); cudaFree(d_coef); cudaFree(d_rec); cudaFree(d_nnz);
    }
};
thread_local HostTqCtx t_host_tq;

template <typename T>
int grow(T *&p, size_t &cap, size_t need)
{
    if (need <= cap) return XAVS2GPU_OK;
    if (p) XG_CUDA(cudaFree(p));
    p = nullptr;
    XG_CUDA(cudaMalloc((void **)&p, sizeof(T) * need));
    cap = need;
    return XAVS2GPU_OK;
}

bool is_pinned(const void *p)
{
    cudaPointerAttributes a;
    return p && cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost;
}

}  // namespace

// Device address of page-locked host memory (nullptr if `p` is not).
static void *mapped(const void *p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess || a.type != cudaMemoryTypeHost) return nullptr;
    return a.devicePointer;
}

extern "C" int xavs2gpu_tq_batch_host(const xavs2gpu_tq_block_t *blocks, int n, const int16_t *residual,
                                      int16_t *coef, int16_t *recon, int32_t *nnz, int chunks)
{
    if (chunks == 0 && n > 0) {
        // the chain reads and writes the page-locked host arrays in place
        // over the host link (no copies, no device buffers)
        void *b = mapped(blocks), *r = mapped(residual), *c = mapped(coef), *q = mapped(recon), *z = mapped(nnz);
        if (!b || !r || !c || !q || !z) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_tq_batch_host", "chunks = 0 needs page-locked arrays");
            return XAVS2GPU_ERR_ARG;
        }
        HostTqCtx &hc = t_host_tq;
        const int dev = current_device();
        XG_CUDA(cudaSetDevice(dev));
        if (hc.device < 0) {
            hc.device = dev;
            for (auto &st : hc.st) XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        }
        int rc = tq_batch_launch(static_cast<const xavs2gpu_tq_block_t *>(b), n, static_cast<const int16_t *>(r),
                                 static_cast<int16_t *>(c), static_cast<int16_t *>(q), static_cast<int32_t *>(z), 4,
                                 hc.st[1]);
        if (rc != XAVS2GPU_OK) return rc;
        XG_CUDA(cudaStreamSynchronize(hc.st[1]));
        return XAVS2GPU_OK;
    }
    if (n < 0 || (n > 0 && (!blocks || !residual || !coef || !recon || !nnz)) || chunks < 1 || chunks > 256) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_tq_batch_host", "bad arguments");
        return XAVS2GPU_ERR_ARG;
    }
    if (n == 0) return XAVS2GPU_OK;
    HostTqCtx &c = t_host_tq;
    const int dev = current_device();
    XG_CUDA(cudaSetDevice(dev));
    if (c.device != dev) {
        if (c.device >= 0) {
            fail(XAVS2GPU_ERR_ARG, "xavs2gpu_tq_batch_host", "one device per host thread");
            return XAVS2GPU_ERR_ARG;
        }
        c.device = dev;
        for (auto &s : c.st) XG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    }
    // chunk extents over the residual / recon and level arrays (a chunk is a
    // run of consecutive descriptors; invalid descriptors touch nothing)
    chunks = std::min(chunks, n);
    std::vector<int64_t> r0(chunks, INT64_MAX), r1(chunks, 0), c0(chunks, INT64_MAX), c1(chunks, 0);
    int64_t res_len = 0, coef_len = 0;
    for (int i = 0; i < n; i++) {
        const xavs2gpu_tq_block_t &b = blocks[i];
        if (b.part < 0 || b.part >= kNumParts || b.offset < 0 || b.coef_offset < 0) continue;
        const int w = h_pu_w[b.part], h = h_pu_h[b.part];
        const int64_t sz = (int64_t)w * h, nc = (w == 64 || h == 64) ? sz / 4 : sz;
        const int k = (int)((int64_t)i * chunks / n);
        r0[k] = std::min(r0[k], b.offset);
        r1[k] = std::max(r1[k], b.offset + sz);
        c0[k] = std::min(c0[k], b.coef_offset);
        c1[k] = std::max(c1[k], b.coef_offset + nc);
        res_len = std::max(res_len, b.offset + sz);
        coef_len = std::max(coef_len, b.coef_offset + nc);
    }
    int rc;
    const size_t nres = (size_t)std::max<int64_t>(res_len, 1), ncoef = (size_t)std::max<int64_t>(coef_len, 1);
    if ((rc = grow(c.d_blocks, c.cap_blocks, (size_t)n)) != XAVS2GPU_OK ||
        (rc = grow(c.d_nnz, c.cap_nnz, (size_t)n)) != XAVS2GPU_OK ||
        (rc = grow(c.d_res, c.cap_res, nres)) != XAVS2GPU_OK || (rc = grow(c.d_rec, c.cap_rec, nres)) != XAVS2GPU_OK ||
        (rc = grow(c.d_coef, c.cap_coef, ncoef)) != XAVS2GPU_OK)
        return rc;
    while ((int)c.ev_in.size() < chunks) {
        cudaEvent_t a, b;
        XG_CUDA(cudaEventCreateWithFlags(&a, cudaEventDisableTiming));
        XG_CUDA(cudaEventCreateWithFlags(&b, cudaEventDisableTiming));
        c.ev_in.push_back(a);
        c.ev_done.push_back(b);
    }
    const bool pinned = is_pinned(blocks) && is_pinned(residual) && is_pinned(coef) && is_pinned(recon) &&
                        is_pinned(nnz);
    if (!pinned) chunks = 1;   // pageable memory: the copies cannot overlap anyway
    for (int k = 0; k < chunks; k++) {
        const int b0 = pinned ? (int)(((int64_t)k * n + chunks - 1) / chunks) : 0;
        const int b1 = pinned ? (int)(((int64_t)(k + 1) * n + chunks - 1) / chunks) : n;
        if (b1 <= b0) continue;
        XG_CUDA(cudaMemcpyAsync(c.d_blocks + b0, blocks + b0, sizeof(xavs2gpu_tq_block_t) * (b1 - b0),
                                cudaMemcpyHostToDevice, c.st[0]));
        const int64_t a = pinned ? r0[k] : 0, z = pinned ? r1[k] : res_len;
        if (z > a)
            XG_CUDA(cudaMemcpyAsync(c.d_res + a, residual + a, sizeof(int16_t) * (z - a), cudaMemcpyHostToDevice,
                                    c.st[0]));
        XG_CUDA(cudaEventRecord(c.ev_in[k], c.st[0]));
        XG_CUDA(cudaStreamWaitEvent(c.st[1], c.ev_in[k], 0));
        if ((rc = tq_batch_launch(c.d_blocks + b0, b1 - b0, c.d_res, c.d_coef, c.d_rec, c.d_nnz + b0, 4, c.st[1])) !=
            XAVS2GPU_OK)
            return rc;
        XG_CUDA(cudaEventRecord(c.ev_done[k], c.st[1]));
        XG_CUDA(cudaStreamWaitEvent(c.st[2], c.ev_done[k], 0));
        const int64_t ca = pinned ? c0[k] : 0, cz = pinned ? c1[k] : coef_len;
        if (z > a)
            XG_CUDA(cudaMemcpyAsync(recon + a, c.d_rec + a, sizeof(int16_t) * (z - a), cudaMemcpyDeviceToHost,
                                    c.st[2]));
        if (cz > ca)
            XG_CUDA(cudaMemcpyAsync(coef + ca, c.d_coef + ca, sizeof(int16_t) * (cz - ca), cudaMemcpyDeviceToHost,
                                    c.st[2]));
        XG_CUDA(cudaMemcpyAsync(nnz + b0, c.d_nnz + b0, sizeof(int32_t) * (b1 - b0), cudaMemcpyDeviceToHost, c.st[2]));
    }
    XG_CUDA(cudaStreamSynchronize(c.st[2]));
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
