// loopfilter.cu -- AVS2 in-loop filters for sm_103a: deblocking
// (filter_deblock.c) and sample adaptive offset (filter_sao.c, encoder/sao.c).
//
// Drop-ins for the reference's table entries (deblock_luma[2],
// deblock_chroma[2], sao_block; primitives.h:202-208) and picture-level
// batched forms.  Deblocking edges lie 8 samples apart and a filter reads 3
// and writes at most 3 samples on either side, so all vertical edges of a
// picture are independent of each other, and so are all horizontal edges; the
// reference's LCU-by-LCU order (xavs2_lcu_deblock) filters every sample's
// vertical edge before its horizontal edge, so the picture is done in two
// passes: every vertical edge, then every horizontal edge.  SAO reads the
// deblocked picture and writes another buffer, so every sample is
// independent.
#include "xavs2gpu_common.cuh"

#include <cstring>

namespace xg {
namespace lf {

// ---- one line across an edge (lf_edge_core, filter_deblock.c:254-360) ------
// p[0..5] = L2 L1 L0 R0 R1 R2; returns true when a sample changed.
__device__ __forceinline__ bool filter_line(int (&p)[6], int alpha, int beta, bool chroma)
{
    const int L2 = p[0], L1 = p[1], L0 = p[2], R0 = p[3], R1 = p[4], R2 = p[5];
    const int d = abs(R0 - L0);
    if (d >= alpha || d <= 1) return false;
    const int fl = (abs(L1 - L0) < beta ? 2 : 0) + (abs(L2 - L0) < beta ? 1 : 0);
    const int fr = (abs(R0 - R1) < beta ? 2 : 0) + (abs(R0 - R2) < beta ? 1 : 0);
    int fs;
    switch (fl + fr) {
    case 6: fs = (R1 == R0 && L0 == L1) ? 4 : 3; break;
    case 5: fs = (R1 == R0 && L0 == L1) ? 3 : 2; break;
    case 4: fs = fl == 2 ? 2 : 1; break;
    case 3: fs = abs(L1 - R1) < beta ? 1 : 0; break;
    default: fs = 0; break;
    }
    if (chroma && fs > 0) fs--;
    switch (fs) {
    case 4:
        p[2] = (9 * L0 + 9 * L2 + 8 * R0 + 6 * R2 + 16) >> 5;
        p[1] = (7 * L0 + 6 * L2 + 3 * R0 + 8) >> 4;
        p[0] = (4 * L0 + 3 * L2 + R0 + 4) >> 3;
        p[3] = (9 * R0 + 9 * R2 + 8 * L0 + 6 * L2 + 16) >> 5;
        p[4] = (7 * R0 + 6 * R2 + 3 * L0 + 8) >> 4;
        p[5] = (4 * R0 + 3 * R2 + L0 + 4) >> 3;
        return true;
    case 3:
        p[2] = (L2 + 4 * L1 + 6 * L0 + 4 * R0 + R1 + 8) >> 4;
        p[3] = (L1 + 4 * L0 + 6 * R0 + 4 * R1 + R2 + 8) >> 4;
        p[1] = (3 * L2 + 8 * L1 + 4 * L0 + R0 + 8) >> 4;
        p[4] = (3 * R2 + 8 * R1 + 4 * R0 + L0 + 8) >> 4;
        return true;
    case 2:
        p[2] = (3 * L1 + 10 * L0 + 3 * R0 + 8) >> 4;
        p[3] = (3 * L0 + 10 * R0 + 3 * R1 + 8) >> 4;
        return true;
    case 1:
        p[2] = (3 * L0 + R0 + 2) >> 2;
        p[3] = (3 * R0 + L0 + 2) >> 2;
        return true;
    default:
        return false;
    }
}

__device__ __forceinline__ int byte_of(uint32_t w, int k) { return (int)((w >> (8 * k)) & 0xFFu); }
__device__ __forceinline__ uint32_t set_byte(uint32_t w, int k, int v)
{
    return (w & ~(0xFFu << (8 * k))) | ((uint32_t)v << (8 * k));
}

// ---- per-call kernel: n lines of one edge ------------------------------------
// `src` points at the Q-side sample of line 0; lines `along` apart, samples
// across `across` apart; line k uses flag[k >= n / 2].
__global__ void edge_kernel(uint8_t *src, int n, int along, int across, int alpha, int beta, int chroma, int f0,
                            int f1)
{
    const int k = threadIdx.x;
    if (k >= n || !(k >= n / 2 ? f1 : f0)) return;
    uint8_t *s = src + k * along;
    int p[6];
    for (int i = 0; i < 6; i++) p[i] = s[(i - 3) * across];
    if (filter_line(p, alpha, beta, chroma != 0))
        for (int i = 0; i < 6; i++) s[(i - 3) * across] = (uint8_t)p[i];
}

// ---- four samples per word (SWAR, Hacker's Delight ch. 2) ---------------------
// bit 7 of each byte: a >= b, bytewise unsigned.  The low 7 bits are compared
// through (a | 0x80) - (b & 0x7F), which cannot borrow across bytes.
__device__ __forceinline__ uint32_t ge_bytes(uint32_t a, uint32_t b)
{
    const uint32_t t = (a | 0x80808080u) - (b & 0x7F7F7F7Fu);
    return ((a & ~b) | (~(a ^ b) & t)) & 0x80808080u;
}
// bytewise min(a + b, 255): the sum without carries between bytes, the
// carry out of each byte, and a byte of ones where it is set
__device__ __forceinline__ uint32_t addus_bytes(uint32_t a, uint32_t b)
{
    const uint32_t s = ((a & 0x7F7F7F7Fu) + (b & 0x7F7F7F7Fu)) ^ ((a ^ b) & 0x80808080u);
    const uint32_t cy = ((a & b) | ((a | b) & ~s)) & 0x80808080u;
    return s | cy | (cy - (cy >> 7));
}
// bytewise max(a - b, 0) = 255 - min(255 - a + b, 255)
__device__ __forceinline__ uint32_t subus_bytes(uint32_t a, uint32_t b) { return ~addus_bytes(~a, b); }

// SAO edge class per byte: sign(s - n1) + sign(s - n2) + 2, each term
// sign(s - n) + 1 = [s >= n] + (1 - [n >= s]); the sum is at most 4
__device__ __forceinline__ uint32_t eo_class(uint32_t s, uint32_t n1, uint32_t n2)
{
    const uint32_t H = 0x80808080u;
    return ((ge_bytes(s, n1) >> 7) + (ge_bytes(s, n2) >> 7)) +
           (((ge_bytes(n1, s) ^ H) >> 7) + ((ge_bytes(n2, s) ^ H) >> 7));
}
// the edge-offset table of eo_apply: the offsets of classes 0-4 clipped to
// [0, 255] (words 0-1) and their negations clipped likewise (words 2-3)
__device__ __forceinline__ void eo_table(const int8_t *offset, uint32_t *tab)
{
    uint32_t ad[2] = {0, 0}, sb[2] = {0, 0};
    for (int k = 0; k < 5; k++) {
        const int o = offset[k];
        ad[k >> 2] |= (uint32_t)min(max(o, 0), 255) << (8 * (k & 3));
        sb[k >> 2] |= (uint32_t)min(max(-o, 0), 255) << (8 * (k & 3));
    }
    tab[0] = ad[0]; tab[1] = ad[1]; tab[2] = sb[0]; tab[3] = sb[1];
}
// clip(s + offset[class], 0, 255) per byte: the classes (0..4) packed into
// the 4 selector nibbles of a byte permute over the offsets' positive and
// negative parts (each clipped to 255, which leaves the clipped sum exact)
__device__ __forceinline__ uint32_t eo_apply(uint32_t s, uint32_t cls, const uint32_t *tab)
{
    const uint32_t sel = __byte_perm(cls | (cls >> 4), 0, 0x0020);
    return subus_bytes(addus_bytes(s, __byte_perm(tab[0], tab[1], sel)), __byte_perm(tab[2], tab[3], sel));
}

// Four lines across one edge at once, a line per byte lane: w[0..5] hold
// L2 L1 L0 R0 R1 R2 of the four lines, `lanes` has bit 7 of each byte set for
// the lines the edge filters.  The filter-strength decision of filter_line
// becomes byte masks (no divergence between lines) and its sums are formed in
// 16-bit halves, the even and the odd lanes.  Returns false when no line
// changes.
__device__ __forceinline__ uint32_t lt_bytes(uint32_t a, uint32_t b) { return ge_bytes(a, b) ^ 0x80808080u; }
__device__ __forceinline__ uint32_t byte_mask(uint32_t m7) { return (m7 >> 7) * 0xFFu; }
__device__ __forceinline__ uint32_t pick(uint32_t a, uint32_t b, uint32_t m) { return (a & ~m) | (b & m); }

template <bool CHROMA>
__device__ __forceinline__ bool filter_lines4(uint32_t (&w)[6], uint32_t ew, uint32_t lanes)
{
    const uint32_t alpha = ((ew >> 8) & 0xFFu) * 0x01010101u, beta = ((ew >> 16) & 0xFFu) * 0x01010101u;
    const uint32_t L2 = w[0], L1 = w[1], L0 = w[2], R0 = w[3], R1 = w[4], R2 = w[5];
    const uint32_t d = __vabsdiffu4(R0, L0);
    const uint32_t on = lt_bytes(d, alpha) & ge_bytes(d, 0x02020202u) & lanes;
    if (!on) return false;
    const uint32_t dl1 = __vabsdiffu4(L1, L0), dr1 = __vabsdiffu4(R0, R1);
    const uint32_t a1 = lt_bytes(dl1, beta), a2 = lt_bytes(__vabsdiffu4(L2, L0), beta);
    const uint32_t b1 = lt_bytes(dr1, beta), b2 = lt_bytes(__vabsdiffu4(R0, R2), beta);
    const uint32_t eq = lt_bytes(dl1 | dr1, 0x01010101u);              // L1 == L0 and R1 == R0
    const uint32_t c3 = lt_bytes(__vabsdiffu4(L1, R1), beta);
    // fl = 2 a1 + a2, fr = 2 b1 + b2; strength by fl + fr
    const uint32_t s6 = a1 & a2 & b1 & b2;
    const uint32_t s5 = a1 & b1 & (a2 ^ b2);
    const uint32_t s4_2 = a1 & b1 & ~(a2 | b2);                            // fl = fr = 2
    const uint32_t s4_1 = a2 & b2 & (a1 ^ b1);                             // (3, 1), (1, 3)
    const uint32_t s3 = (a1 & a2 & ~(b1 | b2)) | (b1 & b2 & ~(a1 | a2)) | (a1 & b2 & ~(a2 | b1)) |
                        (a2 & b1 & ~(a1 | b2));
    const uint32_t f4 = s6 & eq, f3 = (s6 & ~eq) | (s5 & eq), f2 = (s5 & ~eq) | s4_2, f1 = s4_1 | (s3 & c3);
    // chroma filters one step weaker
    const uint32_t m4 = CHROMA ? 0u : byte_mask(f4 & on), m3 = byte_mask((CHROMA ? f4 : f3) & on),
                   m2 = byte_mask((CHROMA ? f3 : f2) & on), m1 = byte_mask((CHROMA ? f2 : f1) & on);
    if (!(m4 | m3 | m2 | m1)) return false;
    // the six words split into even / odd lanes (16 bits each); a sum's
    // result byte is bits 0-7 of each lane after the shift
    uint32_t e[6], o[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        e[k] = w[k] & 0x00FF00FFu;
        o[k] = __byte_perm(w[k], 0, 0x4341);
    }
    auto join = [](uint32_t ev, uint32_t od) { return __byte_perm(ev, od, 0x6240); };
    const uint32_t K2 = 0x00020002u, K4 = 0x00040004u, K8 = 0x00080008u, K16 = 0x00100010u;
    uint32_t nL2 = L2, nL1 = L1, nL0 = L0, nR0 = R0, nR1 = R1, nR2 = R2;
    if (m1) {
        auto l0 = [&](const uint32_t *v) { return (3 * v[2] + v[3] + K2) >> 2; };
        auto r0 = [&](const uint32_t *v) { return (3 * v[3] + v[2] + K2) >> 2; };
        nL0 = pick(nL0, join(l0(e), l0(o)), m1);
        nR0 = pick(nR0, join(r0(e), r0(o)), m1);
    }
    if (m2) {
        auto l0 = [&](const uint32_t *v) { return (3 * v[1] + 10 * v[2] + 3 * v[3] + K8) >> 4; };
        auto r0 = [&](const uint32_t *v) { return (3 * v[2] + 10 * v[3] + 3 * v[4] + K8) >> 4; };
        nL0 = pick(nL0, join(l0(e), l0(o)), m2);
        nR0 = pick(nR0, join(r0(e), r0(o)), m2);
    }
    if (m3) {
        auto l0 = [&](const uint32_t *v) { return (v[0] + 4 * v[1] + 6 * v[2] + 4 * v[3] + v[4] + K8) >> 4; };
        auto r0 = [&](const uint32_t *v) { return (v[1] + 4 * v[2] + 6 * v[3] + 4 * v[4] + v[5] + K8) >> 4; };
        auto l1 = [&](const uint32_t *v) { return (3 * v[0] + 8 * v[1] + 4 * v[2] + v[3] + K8) >> 4; };
        auto r1 = [&](const uint32_t *v) { return (3 * v[5] + 8 * v[4] + 4 * v[3] + v[2] + K8) >> 4; };
        nL0 = pick(nL0, join(l0(e), l0(o)), m3);
        nR0 = pick(nR0, join(r0(e), r0(o)), m3);
        nL1 = pick(nL1, join(l1(e), l1(o)), m3);
        nR1 = pick(nR1, join(r1(e), r1(o)), m3);
    }
    if (!CHROMA && m4) {
        auto l0 = [&](const uint32_t *v) { return (9 * v[2] + 9 * v[0] + 8 * v[3] + 6 * v[5] + K16) >> 5; };
        auto l1 = [&](const uint32_t *v) { return (7 * v[2] + 6 * v[0] + 3 * v[3] + K8) >> 4; };
        auto l2 = [&](const uint32_t *v) { return (4 * v[2] + 3 * v[0] + v[3] + K4) >> 3; };
        auto r0 = [&](const uint32_t *v) { return (9 * v[3] + 9 * v[5] + 8 * v[2] + 6 * v[0] + K16) >> 5; };
        auto r1 = [&](const uint32_t *v) { return (7 * v[3] + 6 * v[5] + 3 * v[2] + K8) >> 4; };
        auto r2 = [&](const uint32_t *v) { return (4 * v[3] + 3 * v[5] + v[2] + K4) >> 3; };
        nL0 = pick(nL0, join(l0(e), l0(o)), m4);
        nL1 = pick(nL1, join(l1(e), l1(o)), m4);
        nL2 = pick(nL2, join(l2(e), l2(o)), m4);
        nR0 = pick(nR0, join(r0(e), r0(o)), m4);
        nR1 = pick(nR1, join(r1(e), r1(o)), m4);
        nR2 = pick(nR2, join(r2(e), r2(o)), m4);
    }
    w[0] = nL2; w[1] = nL1; w[2] = nL0; w[3] = nR0; w[4] = nR1; w[5] = nR2;
    return true;
}

// 4x4 byte transpose: rows a..d (byte k = column k) to columns
__device__ __forceinline__ void transpose4(uint32_t &a, uint32_t &b, uint32_t &c, uint32_t &d)
{
    const uint32_t x = __byte_perm(a, b, 0x5140), y = __byte_perm(a, b, 0x7362);
    const uint32_t z = __byte_perm(c, d, 0x5140), v = __byte_perm(c, d, 0x7362);
    a = __byte_perm(x, z, 0x5410);
    b = __byte_perm(x, z, 0x7632);
    c = __byte_perm(y, v, 0x5410);
    d = __byte_perm(y, v, 0x7632);
}

// The bit-7 lane mask of four lines of one 8x8 block's edge: luma lines
// share the half's flag; chroma lines 0-1 are the first half, 2-3 the second.
__device__ __forceinline__ uint32_t edge_lanes(uint32_t ew, bool chroma, int half)
{
    if (chroma) return ((ew & 1u) ? 0x00008080u : 0u) | ((ew & 2u) ? 0x80800000u : 0u);
    return ((ew >> half) & 1u) ? 0x80808080u : 0u;
}

// ROWS (2 or 4) rows of one vertical edge: p = the samples at (row 0,
// edge - 4), rows `pitch` apart
template <bool CHROMA, int ROWS = 4>
__device__ __forceinline__ void filter_ver4(uint8_t *p, long long pitch, uint32_t ew, uint32_t lanes)
{
    uint32_t A[4] = {0, 0, 0, 0}, B[4] = {0, 0, 0, 0};
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        A[r] = *reinterpret_cast<const uint32_t *>(p + r * pitch);
        B[r] = *reinterpret_cast<const uint32_t *>(p + r * pitch + 4);
    }
    transpose4(A[0], A[1], A[2], A[3]);   // A[k] = column edge - 4 + k
    transpose4(B[0], B[1], B[2], B[3]);   // B[k] = column edge + k
    uint32_t w[6] = {A[1], A[2], A[3], B[0], B[1], B[2]};
    if (!filter_lines4<CHROMA>(w, ew, lanes)) return;
    A[1] = w[0]; A[2] = w[1]; A[3] = w[2]; B[0] = w[3]; B[1] = w[4]; B[2] = w[5];
    transpose4(A[0], A[1], A[2], A[3]);
    transpose4(B[0], B[1], B[2], B[3]);
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        *reinterpret_cast<uint32_t *>(p + r * pitch) = A[r];
        *reinterpret_cast<uint32_t *>(p + r * pitch + 4) = B[r];
    }
}

// Four columns of one horizontal edge: p = the samples at (edge - 3,
// column 0), rows `pitch` apart
template <bool CHROMA>
__device__ __forceinline__ void filter_hor4(uint8_t *p, long long pitch, uint32_t ew, uint32_t lanes)
{
    uint32_t w[6];
#pragma unroll
    for (int r = 0; r < 6; r++) w[r] = *reinterpret_cast<const uint32_t *>(p + r * pitch);
    if (!filter_lines4<CHROMA>(w, ew, lanes)) return;
#pragma unroll
    for (int r = 0; r < 6; r++) *reinterpret_cast<uint32_t *>(p + r * pitch) = w[r];
}

// ---- picture deblocking --------------------------------------------------------
struct Pic {
    uint8_t *y, *u, *v;
    int stride, stride_c, width, height, w_scu, h_scu;
    int n_hor;   // 8x8 columns whose horizontal edges are filtered
    const xavs2gpu_deblock_scu_t *scus;
};

// Pass 1: every vertical edge.  A thread filters one half of one edge (the
// 4 luma / 2 chroma lines sharing a filter flag): per line the 8 samples
// [x-4, x+4) as two words.  Consecutive threads take consecutive edges of
// the same lines, so a warp reads 256 contiguous bytes per line.
__global__ void __launch_bounds__(256) deblock_ver_kernel(Pic pc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int ne = pc.w_scu - 1;                         // luma edges per row (x = 8 .. width - 8)
    const int nec = (pc.w_scu - 1) >> 1;                 // chroma edges per row (x_c = 8, 16, ..)
    const long long n_luma = (long long)(pc.height >> 2) * ne;
    const long long n_chroma = (long long)(pc.height >> 2) * nec;   // 2-line groups of height / 2 rows
    uint8_t *row;
    int e, x, sx, sy, half, stride;
    bool chroma;
    if (i < n_luma) {
        const int g = (int)(i / ne);                     // 4-line group
        e = 1 + (int)(i - (long long)g * ne);
        x = 8 * e;
        sx = e;
        sy = g >> 1;
        half = g & 1;
        stride = pc.stride;
        row = pc.y + (long long)(4 * g) * stride;
        chroma = false;
    } else if (i < n_luma + 2 * n_chroma) {
        const long long j = i - n_luma;
        const int plane = j >= n_chroma;
        const long long jj = j - (plane ? n_chroma : 0);
        const int g = (int)(jj / nec);                   // 2-line group
        e = 1 + (int)(jj - (long long)g * nec);
        x = 8 * e;
        sx = 2 * e;
        sy = g >> 1;
        half = g & 1;
        stride = pc.stride_c;
        row = (plane ? pc.v : pc.u) + (long long)(2 * g) * stride;
        chroma = true;
    } else {
        return;
    }
    const xavs2gpu_deblock_scu_t q = pc.scus[sy * pc.w_scu + sx];
    if (q.type[0] == 0 || (chroma && q.type[0] != 2) || !q.flag[0][half]) return;
    const uint32_t ew = ((uint32_t)(chroma ? q.alpha_c[0] : q.alpha[0]) << 8) |
                        ((uint32_t)(chroma ? q.beta_c[0] : q.beta[0]) << 16);
    // the lines (4 luma, 2 chroma) as byte lanes of transposed words
    if (chroma)
        filter_ver4<true, 2>(row + x - 4, stride, ew, 0x00008080u);
    else
        filter_ver4<false, 4>(row + x - 4, stride, ew, 0x80808080u);
}

// filters the four columns of one word of a horizontal edge (rows y-3 ..
// y+2); the first two and the last two columns take flags f_lo and f_hi
__device__ __forceinline__ void hor_word(uint8_t *col, int stride, int alpha, int beta, bool chroma, bool f_lo,
                                         bool f_hi)
{
    const uint32_t ew = ((uint32_t)alpha << 8) | ((uint32_t)beta << 16);
    const uint32_t lanes = (f_lo ? 0x00008080u : 0u) | (f_hi ? 0x80800000u : 0u);
    if (!lanes) return;
    if (chroma)
        filter_hor4<true>(col - 3LL * stride, stride, ew, lanes);
    else
        filter_hor4<false>(col - 3LL * stride, stride, ew, lanes);
}

// Pass 2: every horizontal edge.  A thread filters one 8x8 block's edge: 8
// luma columns (two words of rows y-3 .. y+2, one per half) or the 4 chroma
// columns (one word; columns 0-1 and 2-3 are the halves).
__global__ void __launch_bounds__(256) deblock_hor_kernel(Pic pc)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int ne = pc.h_scu - 1;                         // luma edges (y = 8 .. height - 8)
    const int nec = (pc.h_scu - 1) >> 1;                 // chroma edges (y_c = 8, 16, ..)
    const long long n_luma = (long long)ne * pc.w_scu;
    const long long n_chroma = (long long)nec * pc.w_scu;
    int sx, sy;
    if (i < n_luma) {
        const int j = (int)(i / pc.w_scu);
        sx = (int)(i - (long long)j * pc.w_scu);
        sy = j + 1;
        if (sx >= pc.n_hor) return;
        const xavs2gpu_deblock_scu_t q = pc.scus[sy * pc.w_scu + sx];
        if (q.type[1] == 0) return;
        uint8_t *col = pc.y + (long long)(8 * sy) * pc.stride + 8 * sx;
        if (q.flag[1][0]) hor_word(col, pc.stride, q.alpha[1], q.beta[1], false, true, true);
        if (q.flag[1][1]) hor_word(col + 4, pc.stride, q.alpha[1], q.beta[1], false, true, true);
    } else if (i < n_luma + 2 * n_chroma) {
        const long long t = i - n_luma;
        const int plane = t >= n_chroma;
        const long long tt = t - (plane ? n_chroma : 0);
        const int j = (int)(tt / pc.w_scu);
        sx = (int)(tt - (long long)j * pc.w_scu);
        sy = 2 * (j + 1);
        if (sx >= pc.n_hor) return;
        const xavs2gpu_deblock_scu_t q = pc.scus[sy * pc.w_scu + sx];
        if (q.type[1] != 2 || (!q.flag[1][0] && !q.flag[1][1])) return;
        uint8_t *col = (plane ? pc.v : pc.u) + (long long)(8 * (j + 1)) * pc.stride_c + 4 * sx;
        hor_word(col, pc.stride_c, q.alpha_c[1], q.beta_c[1], true, q.flag[1][0] != 0, q.flag[1][1] != 0);
    }
}

// ---- SAO -------------------------------------------------------------------------
__device__ __forceinline__ int sign3(int v) { return (v > 0) - (v < 0); }

// The filtered column range [x0, x1) of row y of a w x h SAO block
// (filter_sao.c:50-226) for type t; avail bits: 0 T, 1 D, 2 L, 3 R, 4 TL,
// 5 TR, 6 DL, 7 DR.  Returns false for rows not filtered.
__host__ __device__ __forceinline__ bool sao_row_range(int t, int av, int y, int w, int h, int &x0, int &x1)
{
    const bool T = av & 1, D = av & 2, L = av & 4, R = av & 8, TL = av & 16, TR = av & 32, DL = av & 64,
               DR = av & 128;
    x0 = L ? 0 : 1;
    x1 = R ? w : w - 1;
    if (t == 4) {
        x0 = 0;
        x1 = w;
    } else if (t == 1) {
        if ((y == 0 && !T) || (y == h - 1 && !D)) return false;
        x0 = 0;
        x1 = w;
    } else if (t == 2 && y == 0) {
        x0 = TL ? 0 : 1;
        x1 = T ? (R ? w : w - 1) : 1;
    } else if (t == 2 && y == h - 1) {
        x0 = D ? (L ? 0 : 1) : w - 1;
        x1 = DR ? w : w - 1;
    } else if (t == 3 && y == 0) {
        x0 = T ? (L ? 0 : 1) : w - 1;
        x1 = TR ? w : w - 1;
    } else if (t == 3 && y == h - 1) {
        x0 = DL ? 0 : 1;
        x1 = D ? (R ? w : w - 1) : 1;
    }
    return x1 > x0;
}

// neighbour offsets (dx1, dy1, dx2, dy2) of the EO types
__constant__ int8_t c_eo_nb[4][4] = {{-1, 0, 1, 0}, {0, -1, 0, 1}, {-1, -1, 1, 1}, {1, -1, -1, 1}};

// per-call: one block, dst pre-filled with the caller's samples
__global__ void __launch_bounds__(256) sao_block_kernel(uint8_t *dst, int i_dst, const uint8_t *src, int i_src,
                                                        int w, int h, int av, xavs2gpu_sao_param_t prm)
{
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        const int y = i / w, x = i - y * w;
        int x0, x1;
        if (!sao_row_range(prm.type_idc, av, y, w, h, x0, x1) || x < x0 || x >= x1) continue;
        const uint8_t *p = src + y * i_src + x;
        const int s = p[0];
        int c;
        if (prm.type_idc == 4) {
            c = s >> 3;
        } else {
            const int8_t *nb = c_eo_nb[prm.type_idc];
            c = sign3(s - p[nb[1] * i_src + nb[0]]) + sign3(s - p[nb[3] * i_src + nb[2]]) + 2;
        }
        dst[y * i_dst + x] = (uint8_t)min(max(s + prm.offset[c], 0), 255);
    }
}

// The region of an LCU (sao_get_neighbor_avail, sao.c:898-975) for
// component c: the LCU moved 4 samples up / left where that side is
// available, grown by 4 where the right / lower side is not, kept inside the
// picture.
__host__ __device__ __forceinline__ bool sao_region(int lx, int ly, int lcu_level, int width, int height, int av,
                                                    int c, int &x, int &y, int &w, int &h)
{
    const int S = 1 << lcu_level;
    x = lx * S;
    y = ly * S;
    w = S < width - x ? S : width - x;
    h = S < height - y ? S : height - y;
    const int W = c ? width >> 1 : width, H = c ? height >> 1 : height;
    if (c) {
        x >>= 1; y >>= 1; w >>= 1; h >>= 1;
    }
    if (!(av & 8)) w += 4;
    if (!(av & 2)) h += 4;
    if (av & 4) x -= 4; else w -= 4;
    if (av & 1) y -= 4; else h -= 4;
    if (w > W - x) w = W - x;
    if (h > H - y) h = H - y;
    return w > 0 && h > 0;
}

struct SaoPic {
    uint8_t *dst[3];
    const uint8_t *src[3];
    int stride, stride_c, width, height, lcu_level, wl, hl, copy_rest;
    const xavs2gpu_sao_lcu_t *lcus;
};

__device__ __forceinline__ int full_avail(int a)
{
    const int T = a & 1, D = (a >> 1) & 1, L = (a >> 2) & 1, R = (a >> 3) & 1;
    return a & 15 | ((T & L) << 4) | ((T & R) << 5) | ((D & L) << 6) | ((D & R) << 7);
}

// A CTA filters one LCU's region of one component; a thread takes 4
// horizontally adjacent samples (one word) at a time.  Region boundaries are
// multiples of 4, so a word never straddles two regions.  Where regions
// overlap (availabilities inconsistent between neighbours, which the
// encoder's derivation never produces) the result is the reference's LCU
// loop's: a sample keeps the value of the last LCU in raster order that
// filters it, so a CTA leaves alone the samples that one of its later
// neighbours filters.
constexpr int kSaoThreads = 128;

__global__ void __launch_bounds__(kSaoThreads, 8) sao_lcu_kernel(SaoPic sp)
{
    const int l = blockIdx.x, c = blockIdx.y;
    const int lx = l % sp.wl, ly = l / sp.wl;
    const xavs2gpu_sao_lcu_t &q = sp.lcus[l];
    int rx, ry, rw, rh;
    if (!sao_region(lx, ly, sp.lcu_level, sp.width, sp.height, q.avail, c, rx, ry, rw, rh)) return;
    // neighbours whose regions overlap this one: x, y, w, h, type,
    // availability, later in raster order
    __shared__ int off[32];
    __shared__ int nb[8][7];
    __shared__ int n_nb;
    __shared__ uint32_t eo_tab[4];
    if (threadIdx.x < 32) off[threadIdx.x] = q.offset[c][threadIdx.x];
    if (threadIdx.x == 32) eo_table(q.offset[c], eo_tab);
    if (threadIdx.x == 0) {
        int no = 0;
        for (int my = ly - 1; my <= ly + 1; my++)
            for (int mx = lx - 1; mx <= lx + 1; mx++) {
                if (mx < 0 || mx >= sp.wl || my < 0 || my >= sp.hl || (mx == lx && my == ly)) continue;
                int x, y, w, h;
                const xavs2gpu_sao_lcu_t &m = sp.lcus[my * sp.wl + mx];
                if (!sao_region(mx, my, sp.lcu_level, sp.width, sp.height, m.avail, c, x, y, w, h)) continue;
                if (x >= rx + rw || x + w <= rx || y >= ry + rh || y + h <= ry) continue;
                nb[no][0] = x; nb[no][1] = y; nb[no][2] = w; nb[no][3] = h;
                nb[no][4] = m.type[c];
                nb[no][5] = full_avail(m.avail);
                nb[no][6] = my * sp.wl + mx > l;
                no++;
            }
        n_nb = no;
    }
    __syncthreads();
    const int no = n_nb;
    const int t = q.type[c];
    const int av = full_avail(q.avail);
    const int W = c ? sp.width >> 1 : sp.width, H = c ? sp.height >> 1 : sp.height;
    const int st = c ? sp.stride_c : sp.stride;
    const uint8_t *s = c == 0 ? sp.src[0] : c == 1 ? sp.src[1] : sp.src[2];
    uint8_t *dp = c == 0 ? sp.dst[0] : c == 1 ? sp.dst[1] : sp.dst[2];
    const int nwords = rw >> 2;
    for (int i = threadIdx.x; i < nwords * rh; i += kSaoThreads) {
        const int yy = i / nwords, x = rx + 4 * (i - yy * nwords), y = ry + yy;
        // samples of this word that a later neighbour filters (copy mode:
        // every sample a later neighbour's region holds); a word that
        // another region also holds is written byte by byte
        unsigned later = 0;
        bool shared = false;
        for (int k = 0; k < no; k++) {
            const int *o = nb[k];
            if (x < o[0] || x >= o[0] + o[2] || y < o[1] || y >= o[1] + o[3]) continue;
            shared = true;
            if (!o[6]) continue;
            int a0, a1;
            if (sp.copy_rest) {
                later = 15u;
            } else if (o[4] >= 0 && o[4] <= 4 && sao_row_range(o[4], o[5], y - o[1], o[2], o[3], a0, a1)) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (x + j >= o[0] + a0 && x + j < o[0] + a1) later |= 1u << j;
            }
        }
        if (later == 15u) continue;
        uint8_t *d = dp + (long long)y * st + x;
        int x0 = 0, x1 = 0;
        const bool filt = t >= 0 && t <= 4 && sao_row_range(t, av, yy, rw, rh, x0, x1) && x + 4 > rx + x0 &&
                          x < rx + x1;
        if (!filt) {
            // samples SAO leaves alone: the source value, or untouched
            if (sp.copy_rest && !shared)
                *reinterpret_cast<uint32_t *>(d) = *reinterpret_cast<const uint32_t *>(s + (long long)y * st + x);
            continue;
        }
        x0 += rx;
        x1 += rx;
        // source words: rows y-1, y, y+1 at x-4, x, x+4 (0 outside the
        // picture: the availability rules keep filtered samples' neighbours
        // inside)
        uint32_t win[3][3];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const int yr = y + r - 1;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const int xx = x + 4 * (k - 1);
                win[r][k] = (yr >= 0 && yr < H && xx >= 0 && xx < W)
                                ? *reinterpret_cast<const uint32_t *>(s + (long long)yr * st + xx) : 0u;
            }
        }
        const uint32_t old = sp.copy_rest ? win[1][1] : shared ? 0u : *reinterpret_cast<const uint32_t *>(d);
        // the samples written: inside [x0, x1) and not filtered by a later
        // neighbour; all four computed at once
        unsigned wrote = 0;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (x + k >= x0 && x + k < x1 && !((later >> k) & 1u)) wrote |= 1u << k;
        const uint32_t cur = win[1][1];
        uint32_t res;
        if (t == 4) {
            res = cur;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int sv = byte_of(cur, k);
                res = set_byte(res, k, min(max(sv + off[sv >> 3], 0), 255));
            }
        } else {
            // samples x-1 .. x+2 and x+1 .. x+4 of source row r
            auto lft = [&](int r) { return __byte_perm(win[r][0], win[r][1], 0x6543); };
            auto rgt = [&](int r) { return __byte_perm(win[r][1], win[r][2], 0x4321); };
            uint32_t n1, n2;
            switch (t) {
            case 0: n1 = lft(1); n2 = rgt(1); break;
            case 1: n1 = win[0][1]; n2 = win[2][1]; break;
            case 2: n1 = lft(0); n2 = rgt(2); break;
            default: n1 = rgt(0); n2 = lft(2); break;
            }
            res = eo_apply(cur, eo_class(cur, n1, n2), eo_tab);
        }
        const uint32_t m = ((wrote * 0x00204081u) & 0x01010101u) * 0xFFu;   // bit k -> byte k
        const uint32_t out = (res & m) | (old & ~m);
        if (shared) {
#pragma unroll
            for (int k = 0; k < 4; k++)
                if ((wrote >> k) & 1u) d[k] = (uint8_t)byte_of(out, k);
        } else if (sp.copy_rest || out != old) {
            *reinterpret_cast<uint32_t *>(d) = out;
        }
    }
}

// ---- fused deblocking + SAO --------------------------------------------------
// A CTA takes the SAO region of one LCU for one component and produces its
// final samples in one pass: the part of the region plus an 8-sample margin
// (clamped to the picture) that the filters read is loaded into shared
// memory, the vertical edges and then the horizontal edges that change a
// sample SAO reads are filtered there, four lines per thread, and SAO writes
// the region, four samples per thread.  A deblocked sample depends on source
// samples at most 5 away in each direction and SAO reads 1 around the region,
// so the margin holds everything the region needs and the result equals the
// picture-wide two-pass deblocking followed by SAO.  With most of the
// deblocking branch-free, 128 threads a CTA keep more CTAs in flight than
// 256 (0.043 against 0.055 ms for a 3840x2160 picture).
constexpr int kLfPitch = 96, kLfRows = 88;   // tile: region (<= 68) + 2 x 8
constexpr int kLfScus = 256;                  // 8x8 blocks the tile touches (<= 15 x 15)
#ifndef XG_LF_THREADS
#define XG_LF_THREADS 128
#endif

struct FusedPic {
    const uint8_t *src[3];
    uint8_t *dst[3];
    int stride, stride_c, width, height, lcu_level, wl, hl, w_scu, n_hor;
    const xavs2gpu_deblock_scu_t *scus;
    const xavs2gpu_sao_lcu_t *lcus;
};

// Per 8x8 block and direction, the edge as one word for the component:
// bit 0 filter the first half, bit 1 the second half (type and flag
// combined), alpha in bits 8-15, beta in bits 16-23.
__device__ __forceinline__ uint32_t edge_word(const xavs2gpu_deblock_scu_t &e, int dir, bool chroma)
{
    const bool on = chroma ? e.type[dir] == 2 : e.type[dir] != 0;
    if (!on) return 0;
    return (e.flag[dir][0] ? 1u : 0u) | (e.flag[dir][1] ? 2u : 0u) |
           ((uint32_t)(chroma ? e.alpha_c[dir] : e.alpha[dir]) << 8) |
           ((uint32_t)(chroma ? e.beta_c[dir] : e.beta[dir]) << 16);
}

// The deblocking of the tile: vertical edges on the rows [vy0, vy1) in
// 4-row groups, then horizontal edges on the word columns holding
// [cx0, cx1).  Rows and columns outside those ranges that a group or word
// also covers get filtered too; nothing after reads them.
template <bool CHROMA>
__device__ __forceinline__ void deblock_tile(uint8_t (*t)[kLfPitch], const uint32_t *ev, const uint32_t *eh,
                                             int tx0, int ty0, int sx0, int sy0, int nsx, int ex0, int nex, int ey0,
                                             int ney, int vy0, int vy1, int cx0, int cx1)
{
    const int sh = CHROMA ? 2 : 3, tid = threadIdx.x, nt = blockDim.x;
    const int gy0 = vy0 & ~3, ng = (vy1 - gy0 + 3) >> 2;
    for (int i = tid; i < nex * ng; i += nt) {
        const int g = i / nex, ex = ex0 + 8 * (i - g * nex), y = gy0 + 4 * g;
        const uint32_t ew = ev[((y >> sh) - sy0) * nsx + (ex >> sh) - sx0];
        const uint32_t lanes = edge_lanes(ew, CHROMA, (y & 7) >= 4);
        if (lanes) filter_ver4<CHROMA>(&t[y - ty0][ex - tx0 - 4], kLfPitch, ew, lanes);
    }
    __syncthreads();
    const int wx0 = cx0 & ~3, nwc = (((cx1 + 3) & ~3) - wx0) >> 2;
    for (int i = tid; i < nwc * ney; i += nt) {
        const int j = i / nwc, x = wx0 + 4 * (i - j * nwc), ey = ey0 + 8 * j;
        const uint32_t ew = eh[((ey >> sh) - sy0) * nsx + (x >> sh) - sx0];
        const uint32_t lanes = edge_lanes(ew, CHROMA, (x & 7) >= 4);
        if (lanes) filter_hor4<CHROMA>(&t[ey - ty0 - 3][x - tx0], kLfPitch, ew, lanes);
    }
}

#ifndef XG_LF_MINB
// resident CTAs per SM the register budget is sized for (0: the compiler's
// choice, 48 registers and 10 CTAs; 16 CTAs at 32 registers, a few spilled
// words, measured 0.041 against 0.044 ms per 2160p picture, 12 CTAs 0.044)
#define XG_LF_MINB 16
#endif
__global__ void
#if XG_LF_MINB > 0
__launch_bounds__(XG_LF_THREADS, XG_LF_MINB)
#else
__launch_bounds__(XG_LF_THREADS)
#endif
loopfilter_lcu_kernel(FusedPic fp)
{
    __shared__ __align__(16) uint8_t t[kLfRows][kLfPitch];
    __shared__ uint32_t ev[kLfScus], eh[kLfScus];   // edge words, vertical / horizontal
    __shared__ int off[32];
    __shared__ uint32_t eo_tab[4];   // edge-offset classes 0-4: added bytes (words 0-1), subtracted (2-3)
    const int l = blockIdx.x, c = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
    const bool chroma = c != 0;
    const int lx = l % fp.wl, ly = l / fp.wl;
    const xavs2gpu_sao_lcu_t &q = fp.lcus[l];
    int rx, ry, rw, rh;
    if (!sao_region(lx, ly, fp.lcu_level, fp.width, fp.height, q.avail, c, rx, ry, rw, rh)) return;
    const int W = chroma ? fp.width >> 1 : fp.width, H = chroma ? fp.height >> 1 : fp.height;
    const int st = chroma ? fp.stride_c : fp.stride;
    const uint8_t *src = c == 0 ? fp.src[0] : c == 1 ? fp.src[1] : fp.src[2];
    uint8_t *dst = c == 0 ? fp.dst[0] : c == 1 ? fp.dst[1] : fp.dst[2];
    const int tx0 = max(rx - 8, 0), tx1 = min(rx + rw + 8, W), ty0 = max(ry - 8, 0), ty1 = min(ry + rh + 8, H);
    if (tid < 32) off[tid] = q.offset[c][tid];
    if (tid == 32) eo_table(q.offset[c], eo_tab);
    // edge words of the 8x8 blocks the tile touches
    const int sh = chroma ? 2 : 3;
    const int sx0 = tx0 >> sh, sy0 = ty0 >> sh, nsx = ((tx1 - 1) >> sh) - sx0 + 1, nsy = ((ty1 - 1) >> sh) - sy0 + 1;
    for (int i = tid; i < nsx * nsy; i += nt) {
        const int r = i / nsx, sx = sx0 + i - r * nsx;
        const xavs2gpu_deblock_scu_t e = fp.scus[(sy0 + r) * fp.w_scu + sx];
        ev[i] = edge_word(e, 0, chroma);
        eh[i] = sx < fp.n_hor ? edge_word(e, 1, chroma) : 0u;
    }
    // The samples SAO reads are the region and one around it; only the edges
    // that change one of them are filtered (a filter changes at most 3
    // samples on either side of its edge), and only on the rows and columns
    // that SAO and the horizontal edges read.
    const int cx0 = max(rx - 1, tx0), cx1 = min(rx + rw + 1, tx1), cy0 = max(ry - 1, ty0),
              cy1 = min(ry + rh + 1, ty1);
    const int ex0 = (max(max(8, tx0 + 3), cx0 - 2) + 7) & ~7, ex1 = min(tx1 - 3, cx1 + 2);
    const int nex = ex1 >= ex0 ? (ex1 - ex0) / 8 + 1 : 0;
    const int ey0 = (max(max(8, ty0 + 3), cy0 - 2) + 7) & ~7, ey1 = min(ty1 - 3, cy1 + 2);
    const int ney = ey1 >= ey0 ? (ey1 - ey0) / 8 + 1 : 0;
    const int vy0 = ney ? min(cy0, ey0 - 3) : cy0, vy1 = ney ? max(cy1, ey0 + 8 * (ney - 1) + 3) : cy1;
    const int lx0 = (nex ? min(cx0, ex0 - 3) : cx0) & ~3,
              lx1 = min(((nex ? max(cx1, ex0 + 8 * (nex - 1) + 3) : cx1) + 3) & ~3, tx1);
    // the tile rows [vy0, vy1), columns [lx0, lx1): a thread keeps one word
    // column and walks the rows
    {
        const int nw = (lx1 - lx0) >> 2, w = tid % nw, r0 = tid / nw, rs = nt / nw;
        if (r0 < rs)
            for (int y = vy0 + r0; y < vy1; y += rs)
                *reinterpret_cast<uint32_t *>(&t[y - ty0][lx0 - tx0 + 4 * w]) =
                    *reinterpret_cast<const uint32_t *>(src + (long long)y * st + lx0 + 4 * w);
    }
    __syncthreads();
    if (chroma)
        deblock_tile<true>(t, ev, eh, tx0, ty0, sx0, sy0, nsx, ex0, nex, ey0, ney, vy0, vy1, cx0, cx1);
    else
        deblock_tile<false>(t, ev, eh, tx0, ty0, sx0, sy0, nsx, ex0, nex, ey0, ney, vy0, vy1, cx0, cx1);
    __syncthreads();
    // SAO of the region from the deblocked tile, a word (4 samples) at a
    // time; dst written whole; a thread keeps one word column and walks the
    // rows
    const int ty = q.type[c], av = full_avail(q.avail), rwords = rw >> 2;
    const int wi = tid % rwords, r0 = tid / rwords, rs = nt / rwords;
    if (r0 >= rs) return;
    const int x = rx + 4 * wi;
    const bool has_left = x - tx0 >= 4;
    for (int yy = r0; yy < rh; yy += rs) {
        const int y = ry + yy;
        const uint8_t *d = &t[y - ty0][x - tx0];
        const uint32_t cur = *reinterpret_cast<const uint32_t *>(d);
        uint32_t out = cur;
        int x0 = 0, x1 = 0;
        if (ty >= 0 && ty <= 4 && sao_row_range(ty, av, yy, rw, rh, x0, x1)) {
            const int lo = max(x0 - 4 * wi, 0), hi = min(x1 - 4 * wi, 4);
            if (lo < hi) {
                uint32_t res;
                if (ty == 4) {
                    res = cur;
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const int sv = byte_of(cur, k);
                        res = set_byte(res, k, min(max(sv + off[sv >> 3], 0), 255));
                    }
                } else {
                    // neighbour words of row y + dy: samples x-1 .. x+2 and x+1 .. x+4
                    auto lft = [&](int dy) {
                        const uint32_t *r = reinterpret_cast<const uint32_t *>(d + dy * kLfPitch);
                        return __byte_perm(has_left ? r[-1] : 0u, r[0], 0x6543);
                    };
                    auto rgt = [&](int dy) {
                        const uint32_t *r = reinterpret_cast<const uint32_t *>(d + dy * kLfPitch);
                        return __byte_perm(r[0], r[1], 0x4321);
                    };
                    uint32_t n1, n2;
                    switch (ty) {
                    case 0: n1 = lft(0); n2 = rgt(0); break;
                    case 1:
                        n1 = *reinterpret_cast<const uint32_t *>(d - kLfPitch);
                        n2 = *reinterpret_cast<const uint32_t *>(d + kLfPitch);
                        break;
                    case 2: n1 = lft(-1); n2 = rgt(1); break;
                    default: n1 = rgt(-1); n2 = lft(1); break;
                    }
                    res = eo_apply(cur, eo_class(cur, n1, n2), eo_tab);
                }
                const uint32_t m = (0xFFFFFFFFu << (8 * lo)) & (0xFFFFFFFFu >> (8 * (4 - hi)));
                out = (res & m) | (cur & ~m);
            }
        }
        *reinterpret_cast<uint32_t *>(dst + (long long)y * st + x) = out;
    }
}

}  // namespace lf
}  // namespace xg

using namespace xg;

// ---- per-call drop-ins ----------------------------------------------------------
// One edge through the per-thread staging area: the samples the filter can
// read (3 on the P side, 3 on the Q side) of each line are packed, filtered
// and unpacked.
static void deblock_call(uint8_t *const planes[2], int nplanes, int dir, int stride, int alpha, int beta,
                         const uint8_t *flt_flag, bool chroma)
{
    const int n = chroma ? 4 : 8;
    // a rectangle of `rows` x `cols` samples starting 3 before the edge
    const int rows = dir == 0 ? n : 6, cols = dir == 0 ? 6 : n;
    const size_t bytes = (size_t)rows * cols;
    CallCtx &c = call_ctx(align_up(bytes) * nplanes);
    for (int p = 0; p < nplanes; p++) {
        const uint8_t *o = dir == 0 ? planes[p] - 3 : planes[p] - 3 * (intptr_t)stride;
        pack_rows(c.h_stage + align_up(bytes) * p, o, stride, cols, rows);
    }
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, align_up(bytes) * nplanes, cudaMemcpyHostToDevice, c.stream));
    for (int p = 0; p < nplanes; p++) {
        uint8_t *base = c.d_stage + align_up(bytes) * p;
        uint8_t *q = dir == 0 ? base + 3 : base + 3 * cols;
        lf::edge_kernel<<<1, 32, 0, c.stream>>>(q, n, dir == 0 ? cols : 1, dir == 0 ? 1 : cols, alpha, beta,
                                               chroma ? 1 : 0, flt_flag[0], flt_flag[1]);
        count_launch();
    }
    XG_CUDA(cudaMemcpyAsync(c.h_stage, c.d_stage, align_up(bytes) * nplanes, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    for (int p = 0; p < nplanes; p++) {
        uint8_t *o = dir == 0 ? planes[p] - 3 : planes[p] - 3 * (intptr_t)stride;
        unpack_rows(o, stride, c.h_stage + align_up(bytes) * p, cols, rows);
    }
}

extern "C" void xavs2gpu_deblock_luma_ver(uint8_t *src, int stride, int alpha, int beta, uint8_t *flt_flag)
{
    uint8_t *p[2] = {src, nullptr};
    deblock_call(p, 1, 0, stride, alpha, beta, flt_flag, false);
}
extern "C" void xavs2gpu_deblock_luma_hor(uint8_t *src, int stride, int alpha, int beta, uint8_t *flt_flag)
{
    uint8_t *p[2] = {src, nullptr};
    deblock_call(p, 1, 1, stride, alpha, beta, flt_flag, false);
}
extern "C" void xavs2gpu_deblock_chroma_ver(uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                                            uint8_t *flt_flag)
{
    uint8_t *p[2] = {src_u, src_v};
    deblock_call(p, 2, 0, stride, alpha, beta, flt_flag, true);
}
extern "C" void xavs2gpu_deblock_chroma_hor(uint8_t *src_u, uint8_t *src_v, int stride, int alpha, int beta,
                                            uint8_t *flt_flag)
{
    uint8_t *p[2] = {src_u, src_v};
    deblock_call(p, 2, 1, stride, alpha, beta, flt_flag, true);
}

extern "C" void xavs2gpu_deblock_init(uint32_t cpuid, xavs2gpu_deblock_funcs_t *f)
{
    (void)cpuid;
    f->deblock_luma[0] = xavs2gpu_deblock_luma_ver;
    f->deblock_luma[1] = xavs2gpu_deblock_luma_hor;
    f->deblock_chroma[0] = xavs2gpu_deblock_chroma_ver;
    f->deblock_chroma[1] = xavs2gpu_deblock_chroma_hor;
}

extern "C" void xavs2gpu_sao_block(uint8_t *p_dst, int i_dst, uint8_t *p_src, int i_src, int i_block_w,
                                   int i_block_h, int *lcu_avail, xavs2gpu_sao_param_t *sao_param)
{
    if (sao_param->type_idc < 0 || sao_param->type_idc > 4 || i_block_w < 1 || i_block_h < 1) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_sao_block", "not a supported SAO type or empty block");
        return;
    }
    int av = 0;
    for (int k = 0; k < 8; k++) av |= (lcu_avail[k] ? 1 : 0) << k;
    // source with a one-sample ring (neighbours), destination block
    const int sw = i_block_w + 2, sh = i_block_h + 2;
    const size_t o_dst = align_up((size_t)sw * sh);
    CallCtx &c = call_ctx(o_dst + (size_t)i_block_w * i_block_h);
    pack_rows(c.h_stage, p_src - i_src - 1, i_src, sw, sh);
    pack_rows(c.h_stage + o_dst, p_dst, i_dst, i_block_w, i_block_h);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_dst + (size_t)i_block_w * i_block_h, cudaMemcpyHostToDevice,
                            c.stream));
    lf::sao_block_kernel<<<1, 256, 0, c.stream>>>(c.d_stage + o_dst, i_block_w, c.d_stage + sw + 1, sw, i_block_w,
                                                 i_block_h, av, *sao_param);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_dst, c.d_stage + o_dst, (size_t)i_block_w * i_block_h,
                            cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    unpack_rows(p_dst, i_dst, c.h_stage + o_dst, i_block_w, i_block_h);
}

extern "C" void xavs2gpu_sao_init(uint32_t cpuid, xavs2gpu_sao_flt_t *f)
{
    (void)cpuid;
    *f = xavs2gpu_sao_block;
}

// ---- picture-level forms ---------------------------------------------------------
static bool aligned4(const void *p) { return ((uintptr_t)p & 3) == 0; }

extern "C" int xavs2gpu_deblock_picture(uint8_t *y, int stride, uint8_t *u, uint8_t *v, int stride_c, int width,
                                        int height, int lcu_level, const xavs2gpu_deblock_scu_t *scus, void *stream)
{
    if (width < 8 || height < 8 || (width & 7) || (height & 7) || stride < width || stride_c < width / 2 ||
        (stride & 3) || (stride_c & 3) || !aligned4(y) || !aligned4(u) || !aligned4(v) || !scus ||
        lcu_level < 3 || lcu_level > 6) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_deblock_picture",
             "sizes must be multiples of 8, LCU 8..64, planes and strides 4-byte aligned");
        return XAVS2GPU_ERR_ARG;
    }
    // a picture one LCU wide: xavs2_lcu_deblock leaves the horizontal edges
    // of the last 8x8 column for a next LCU in the row, which does not exist
    const int w_scu = width / 8;
    const int n_hor = w_scu <= (1 << (lcu_level - 3)) ? w_scu - 1 : w_scu;
    lf::Pic pc{y, u, v, stride, stride_c, width, height, w_scu, height / 8, n_hor, scus};
    const cudaStream_t st = (cudaStream_t)stream;
    const long long nv = (long long)(height / 4) * (pc.w_scu - 1) + 2LL * (height / 4) * ((pc.w_scu - 1) >> 1);
    const long long nh = (long long)(pc.h_scu - 1) * pc.w_scu + 2LL * ((pc.h_scu - 1) >> 1) * pc.w_scu;
    if (nv > 0) {
        lf::deblock_ver_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, st>>>(pc);
        count_launch();
    }
    if (nh > 0) {
        lf::deblock_hor_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(pc);
        count_launch();
    }
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_sao_picture(uint8_t *dst_y, uint8_t *dst_u, uint8_t *dst_v, const uint8_t *src_y,
                                    const uint8_t *src_u, const uint8_t *src_v, int stride, int stride_c, int width,
                                    int height, int lcu_level, const xavs2gpu_sao_lcu_t *lcus, int flags,
                                    void *stream)
{
    const void *ptrs[6] = {dst_y, dst_u, dst_v, src_y, src_u, src_v};
    bool ok = width >= 8 && height >= 8 && !(width & 7) && !(height & 7) && stride >= width &&
              stride_c >= width / 2 && !(stride & 3) && !(stride_c & 3) && lcu_level >= 4 && lcu_level <= 6 && lcus;
    for (int k = 0; k < 6; k++) ok = ok && ptrs[k] && aligned4(ptrs[k]);
    if (!ok) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_sao_picture",
             "sizes must be multiples of 8, LCU 16..64, planes and strides 4-byte aligned");
        return XAVS2GPU_ERR_ARG;
    }
    const int S = 1 << lcu_level;
    lf::SaoPic sp{{dst_y, dst_u, dst_v}, {src_y, src_u, src_v}, stride, stride_c, width, height, lcu_level,
                  (width + S - 1) / S, (height + S - 1) / S, (flags & XAVS2GPU_SAO_COPY_UNFILTERED) ? 1 : 0, lcus};
    lf::sao_lcu_kernel<<<dim3((unsigned)(sp.wl * sp.hl), 3), lf::kSaoThreads, 0, (cudaStream_t)stream>>>(sp);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

extern "C" int xavs2gpu_loopfilter_picture(const uint8_t *src_y, const uint8_t *src_u, const uint8_t *src_v,
                                           uint8_t *dst_y, uint8_t *dst_u, uint8_t *dst_v, int stride, int stride_c,
                                           int width, int height, int lcu_level, const xavs2gpu_deblock_scu_t *scus,
                                           const xavs2gpu_sao_lcu_t *lcus, void *stream)
{
    const void *ptrs[6] = {src_y, src_u, src_v, dst_y, dst_u, dst_v};
    bool ok = width >= 8 && height >= 8 && !(width & 7) && !(height & 7) && stride >= width &&
              stride_c >= width / 2 && !(stride & 3) && !(stride_c & 3) && lcu_level >= 4 && lcu_level <= 6 && scus &&
              lcus;
    for (int k = 0; k < 6; k++) ok = ok && ptrs[k] && aligned4(ptrs[k]);
    if (!ok) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_loopfilter_picture",
             "sizes must be multiples of 8, LCU 16..64, planes and strides 4-byte aligned");
        return XAVS2GPU_ERR_ARG;
    }
    const int S = 1 << lcu_level, w_scu = width / 8;
    const int n_hor = w_scu <= (1 << (lcu_level - 3)) ? w_scu - 1 : w_scu;
    lf::FusedPic fp{{src_y, src_u, src_v}, {dst_y, dst_u, dst_v}, stride, stride_c, width, height, lcu_level,
                    (width + S - 1) / S, (height + S - 1) / S, w_scu, n_hor, scus, lcus};
    lf::loopfilter_lcu_kernel<<<dim3((unsigned)(fp.wl * fp.hl), 3), XG_LF_THREADS, 0, (cudaStream_t)stream>>>(fp);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
