// mc.cu -- AVS2 luma 8-tap / chroma 4-tap interpolation for sm_103a: the
// per-call drop-ins of the intpl_* members of intrinsic_func_t
// (source/common/primitives.h:157-171, C versions mc.c:274-547) and the
// whole-frame quarter-pel plane generation that replaces the reference's
// per-LCU-row interpolate_lcu_row (mc.c:593-785) + plane_expand_border
// (frame.c:471-507).
#include "xavs2gpu_common.cuh"

#include <cstring>

namespace xg {

struct Taps8 { int8_t c[8]; };
struct Taps4 { int8_t c[4]; };

static Taps8 taps8(const int8_t *p) { Taps8 t; memcpy(t.c, p, 8); return t; }
static Taps4 taps4(const int8_t *p) { Taps4 t; memcpy(t.c, p, 4); return t; }

// ---- plane-level filters on packed operands --------------------------------
// All per-call kernels index their operands as (x, y) relative to the block
// origin with explicit strides; the host packs each footprint so the origin
// sits at a fixed offset inside the staging buffer.

// intpl_luma_hor_c (mc.c:403-417): raw 8-tap sum to tmp (int16) and the
// rounded, clipped sample to dst.
__global__ void hor8_kernel(uint8_t *dst, int ds, int16_t *tmp, int ts, const uint8_t *src, int ss, int w, int h,
                            Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[k - 3];
        if (tmp) tmp[y * ts + x] = (int16_t)v;
        if (dst) dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
    }
}

// intpl_luma_ver_c (mc.c:422-435), also the block vertical filter
__global__ void ver8_kernel(uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[(k - 3) * ss];
        dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
    }
}

// intpl_luma_ext_c (mc.c:501-516): vertical 8-tap over int16 raw sums
__global__ void ext8_kernel(uint8_t *dst, int ds, const int16_t *tmp, int ts, int w, int h, Taps8 t)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const int16_t *p = tmp + y * ts + x;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) v += t.c[k] * p[(k - 3) * ts];
        dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
    }
}

// intpl_luma_block_ext_c (mc.c:362-398): int16 raw horizontal sums of rows
// -3..h+3 then the vertical pass with +2048 >> 12.
__global__ void block_ext8_kernel(uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps8 tx, Taps8 ty)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        int v = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint8_t *p = src + (y + k - 3) * ss + x;
            int r = 0;
#pragma unroll
            for (int j = 0; j < 8; j++) r += tx.c[j] * p[j - 3];
            v += ty.c[k] * (int)(int16_t)r;
        }
        dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
    }
}

// intpl_chroma_block_{hor,ver,ext}_c (mc.c:274-337); ext keeps int32 sums
__global__ void chroma4_kernel(int mode, uint8_t *dst, int ds, const uint8_t *src, int ss, int w, int h, Taps4 tx,
                               Taps4 ty)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        int y = i / w, x = i - y * w;
        const uint8_t *p = src + y * ss + x;
        int v = 0;
        if (mode == 0) {
#pragma unroll
            for (int k = 0; k < 4; k++) v += tx.c[k] * p[k - 1];
            dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
        } else if (mode == 1) {
#pragma unroll
            for (int k = 0; k < 4; k++) v += ty.c[k] * p[(k - 1) * ss];
            dst[y * ds + x] = clip_pel_d((v + 32) >> 6);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint8_t *q = p + (k - 1) * ss;
                int r = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) r += tx.c[j] * q[j - 1];
                v += ty.c[k] * r;
            }
            dst[y * ds + x] = clip_pel_d((v + 2048) >> 12);
        }
    }
}

static inline int nblocks(int n, int t = 256) { int b = (n + t - 1) / t; return b < 1 ? 1 : (b > 4096 ? 4096 : b); }

// ---- whole-frame quarter-pel planes ------------------------------------------
// Every sample of plane k = 4*fy + fx at (x, y) equals the AVS2 filter
// evaluated at (clamp(x, -4, W+3), clamp(y, -4, H+3)) with full-pel reads
// clamped into the picture: the reference filters rows [-4, H+4) x columns
// [-4, W+4) and replicates that region outwards.  One kernel writes the
// whole padded plane directly, so the replication costs no extra pass.
constexpr int PT_W = 128, PT_H = 16;            // output tile of a padded plane
constexpr int PS_R = PT_H + 7;                  // source rows a tile reads (23)
constexpr int PS_C = PT_W + 16;                 // source bytes per row, padded (144)
constexpr int PP_R = PT_H + 6;                  // row pairs of the vertical pass (22)

struct PlaneSet { uint8_t *p[16]; };

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// Stores the 4 bytes of `v` at p[0..3], only those with column < `end_col`
// when the group straddles the right edge of the padded plane.
template <bool VEC>
__device__ __forceinline__ void store_group(uint8_t *p, uint32_t v, int x, int end_col)
{
    if (VEC && x + 3 < end_col) {
        *reinterpret_cast<uint32_t *>(p) = v;
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (x + i < end_col) p[i] = (uint8_t)(v >> (8 * i));
}

// Four unsigned bytes of a times four signed bytes of b, plus c.
__device__ __forceinline__ int dp4a_us(uint32_t a, uint32_t b, int c)
{
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// The two signed 16-bit halves of a times signed bytes 0, 1 (lo) or 2, 3 (hi)
// of b, plus c.
__device__ __forceinline__ int dp2a_lo(uint32_t a, uint32_t b, int c)
{
    int d;
    asm("dp2a.lo.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
__device__ __forceinline__ int dp2a_hi(uint32_t a, uint32_t b, int c)
{
    int d;
    asm("dp2a.hi.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// x0..x3 clipped to [0, 255] and packed, x0 in the lowest byte.
__device__ __forceinline__ uint32_t pack_sat_u8(int x0, int x1, int x2, int x3)
{
    uint32_t t, d;
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, 0;" : "=r"(t) : "r"(x3), "r"(x2));
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(x1), "r"(x0), "r"(t));
    return d;
}

// The AVS2 luma taps (mc.c:73-78) as packed signed bytes: half 0 holds
// taps 0..3, half 1 taps 4..7.  Phase 0 is the full-pel position (only
// tap 3 = 64).
__host__ __device__ constexpr uint32_t pk4(int a, int b, int c, int d)
{
    return (uint32_t)(a & 255) | (uint32_t)(b & 255) << 8 | (uint32_t)(c & 255) << 16 | (uint32_t)(d & 255) << 24;
}
__host__ __device__ constexpr uint32_t tap_word(int phase, int half)
{
    return phase == 0 ? (half ? pk4(0, 0, 0, 0) : pk4(0, 0, 0, 64))
         : phase == 1 ? (half ? pk4(19, -7, 3, -1) : pk4(-1, 4, -10, 57))
         : phase == 2 ? (half ? pk4(40, -11, 4, -1) : pk4(-1, 4, -11, 40))
                      : (half ? pk4(57, -10, 4, -1) : pk4(-1, 3, -7, 19));
}

// Vertical 8-tap sum at one column from the four row pairs (h[l], h[l+1]),
// (h[l+2], h[l+3]), (h[l+4], h[l+5]), (h[l+6], h[l+7]) packed as int16 halves.
__device__ __forceinline__ int vsum(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t t03, uint32_t t47,
                                    int init)
{
    return dp2a_hi(d, t47, dp2a_lo(c, t47, dp2a_hi(b, t03, dp2a_lo(a, t03, init))));
}

// The four columns of one row pair (x..w) from shared memory: one 16-byte load
// when the columns are contiguous and aligned, else one load per column.
__device__ __forceinline__ uint4 load_pairs(const uint32_t *row, const int (&lc)[4], bool vec)
{
    if (vec) return *reinterpret_cast<const uint4 *>(row + lc[0]);
    return make_uint4(row[lc[0]], row[lc[1]], row[lc[2]], row[lc[3]]);
}

// One CTA writes a 128 x 16 tile of every requested plane over the whole
// padded area [-pad, W+pad) x [-pad, H+pad).  The sample at (x, y) is the
// filter output at (cx, cy) = (clamp(x, -4, W+3), clamp(y, -4, H+3)) (the
// reference filters [-4, W+4) x [-4, H+4) and replicates that region
// outwards), so a tile needs the filter at the clamped columns cx0 + [0, 128)
// and rows cy0 + [0, nL), nL <= 16 distinct clamped rows.  Source reads are
// clamped into the picture, so the source needs no border.
//   1: the source window, 23 rows x 135 bytes, into shared memory (word loads
//      away from the picture edge, clamped byte loads near it);
//   2: the raw horizontal 8-tap sums of the three sub-pel phases (two byte
//      dot products each) and the source bytes themselves, stored as row
//      pairs (h[s], h[s+1]) of int16 for s = 0..21: a warp per 2 pairs;
//   3: thread = (horizontal phase fx, 4 columns, 4 rows): every vertical
//      phase of a row is four 16-bit pair dot products on the pairs (one for
//      the full-pel phase), the rounding (+32 >> 6 on bytes, +2048 >> 12 on
//      raw sums) is one shift, and four samples are clipped and packed by two
//      saturating packs; the row is stored to every output row that clamps
//      to it (the top and bottom margins repeat rows -4 and H+3) as 32-bit
//      stores, a warp writing 128 contiguous bytes of a plane row.
// 512 threads per CTA: the 1,326 tiles of a 1080p plane set then make
// 4.4 waves of 2 CTAs per SM rather than 2.2 waves of 4 smaller CTAs (the
// partly filled last wave is the smaller share of the run).
// mode: 1 planes 2, 8, 10 (half-pel), 2 all 15 sub-pel planes; | 4: also
// plane 0 (the full-pel picture with its replicated border).
constexpr int kPlaneThreads = 512;
#ifndef XG_PLANES_MINB
#define XG_PLANES_MINB 2
#endif

template <bool VEC>
__global__ void __launch_bounds__(kPlaneThreads, XG_PLANES_MINB)
    frame_planes_kernel(const uint8_t *__restrict__ src, int src_stride, int stride, int W, int H, int pad,
                        PlaneSet planes, int mode, int src_words)
{
    __shared__ __align__(16) uint8_t s_src[PS_R][PS_C];
    __shared__ __align__(16) uint32_t s_pair[4][PP_R][PT_W];
    const int x0 = -pad + blockIdx.x * PT_W, y0 = -pad + blockIdx.y * PT_H;
    const int cx0 = clampi(x0, -4, W + 3), cy0 = clampi(y0, -4, H + 3);
    const int nL = clampi(y0 + PT_H - 1, -4, H + 3) - cy0 + 1;
    const int tid = threadIdx.x;
    // ---- 1: source window: s_src[r][m] = src(cy0 - 3 + r, cx0 - 3 + m) for
    // m < 136 (words 0..33; the filters read bytes 0..134).  Word loads (src
    // and its stride 4-byte aligned) only where every byte they touch, up to
    // column cx0 + 136, lies inside the picture.
    constexpr int kWords = (PT_W + 8) / 4;
    const bool inner = src_words && cx0 - 6 >= 0 && cx0 + PT_W + 12 <= W && cy0 - 3 >= 0 && cy0 + PT_H + 4 <= H;
    if (inner) {
        const int xa = cx0 - 3, sh = 8 * (xa & 3);
        for (int i = tid; i < PS_R * kWords; i += kPlaneThreads) {
            const int r = i / kWords, q = i - r * kWords;
            const uint32_t *p =
                reinterpret_cast<const uint32_t *>(src + (ptrdiff_t)(cy0 - 3 + r) * src_stride + ((xa + 4 * q) & ~3));
            const uint32_t lo = __ldg(p), hi = sh ? __ldg(p + 1) : 0u;
            *reinterpret_cast<uint32_t *>(&s_src[r][4 * q]) = __funnelshift_r(lo, hi, sh);
        }
    } else {
        for (int i = tid; i < PS_R * PS_C; i += kPlaneThreads) {
            const int r = i / PS_C, m = i - r * PS_C;
            const int sy = clampi(cy0 - 3 + r, 0, H - 1), sx = clampi(cx0 - 3 + m, 0, W - 1);
            s_src[r][m] = src[(ptrdiff_t)sy * src_stride + sx];
        }
    }
    __syncthreads();
    // ---- 2: horizontal phases as row pairs: warp `seg` < 11 makes pairs
    // 2 seg and 2 seg + 1 from rows 2 seg .. 2 seg + 2
    if ((tid >> 5) < PP_R / 2) {
        const int g = tid & 31, seg = tid >> 5;
        const int r0 = 2 * seg;
        uint32_t prev[4][4] = {};
#pragma unroll
        for (int dr = 0; dr < 3; dr++) {
            const int r = r0 + dr;
            const uint32_t *w = reinterpret_cast<const uint32_t *>(&s_src[r][0]);
            const uint32_t w0 = w[g], w1 = w[g + 1], w2 = w[g + 2];
            uint32_t cur[4][4];
            const uint32_t ctr = __byte_perm(w0, w1, 0x6543);   // the centre bytes (tap 3) of the 4 columns
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t sel = j == 0 ? 0x3210 : j == 1 ? 0x4321 : j == 2 ? 0x5432 : 0x6543;
                const uint32_t lo = __byte_perm(w0, w1, sel), hi = __byte_perm(w1, w2, sel);
#pragma unroll
                for (int f = 1; f < 4; f++) cur[f][j] = (uint32_t)dp4a_us(hi, tap_word(f, 1), dp4a_us(lo, tap_word(f, 0), 0));
                cur[0][j] = (ctr >> (8 * j)) & 0xFFu;
            }
            if (dr > 0) {
                const int s = r - 1;
#pragma unroll
                for (int f = 0; f < 4; f++) {
                    uint4 v;
                    v.x = __byte_perm(prev[f][0], cur[f][0], 0x5410);
                    v.y = __byte_perm(prev[f][1], cur[f][1], 0x5410);
                    v.z = __byte_perm(prev[f][2], cur[f][2], 0x5410);
                    v.w = __byte_perm(prev[f][3], cur[f][3], 0x5410);
                    *reinterpret_cast<uint4 *>(&s_pair[f][s][4 * g]) = v;
                }
            }
#pragma unroll
            for (int f = 0; f < 4; f++)
#pragma unroll
                for (int j = 0; j < 4; j++) prev[f][j] = cur[f][j];
        }
    }
    __syncthreads();
    // ---- 3: vertical phases, 4 columns x 4 rows per thread
    const int g = tid & 31, fx = (tid >> 5) & 3, qtr = tid >> 7;
    const int l0 = 4 * qtr;
    const int xg = x0 + 4 * g, end_col = W + pad;
    if (l0 >= nL || xg >= end_col) return;
    // planes this thread writes: fy = 0..3 of column phase fx (plane 0, the
    // full-pel picture, only with mode bit 2; mode 1 keeps planes 2, 8, 10)
    int want = 0;
#pragma unroll
    for (int fy = 0; fy < 4; fy++) {
        const int k = 4 * fy + fx;
        if (k == 0 ? (mode & 4) != 0 : ((mode & 3) == 2 || k == 2 || k == 8 || k == 10)) want |= 1 << fy;
    }
    if (!want) return;
    int lc[4];
    bool vec = true;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        lc[c] = clampi(xg + c, -4, W + 3) - cx0;
        vec &= lc[c] == lc[0] + c;
    }
    vec &= (lc[0] & 3) == 0;
    // a tile inside [-4, W+3] x [-4, H+3] whose columns map one to one: every
    // computed row goes to exactly one output row, every group of 4 columns
    // is a whole aligned word
    const bool direct = VEC && vec && y0 >= -4 && y0 + PT_H - 1 <= H + 3 && xg + 3 <= W + 3;
    const uint32_t *rows = &s_pair[fx][0][0];
    const int init = fx ? 2048 : 32, rsh = fx ? 12 : 6;
    uint8_t *base[4];
#pragma unroll
    for (int fy = 0; fy < 4; fy++)   // static parameter indices (a dynamic one copies the table to the stack)
        base[fy] = (fx == 0 ? planes.p[4 * fy] : fx == 1 ? planes.p[4 * fy + 1] : fx == 2 ? planes.p[4 * fy + 2]
                                                                                 : planes.p[4 * fy + 3]) + xg;
    // rows in the order l0, l0 + 2, l0 + 1, l0 + 3: row l uses the pairs of
    // rows l, l + 2, l + 4, l + 6, so two rows of one parity share three of
    // their four pair words and only five are live at a time
#pragma unroll
    for (int par = 0; par < 2; par++) {
        uint4 P[5];   // P[i] = pairs of row l0 + par + 2 i
#pragma unroll
        for (int i = 0; i < 4; i++) P[i] = load_pairs(rows + (l0 + par + 2 * i) * PT_W, lc, vec);
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int t = par + 2 * u, l = l0 + t;
            if (l >= nL) continue;
            if (u == 1) P[4] = load_pairs(rows + (l0 + par + 8) * PT_W, lc, vec);
            const uint4 A = P[u], B = P[u + 1], C = P[u + 2], D = P[u + 3];
            uint32_t out[4];
            // fy = 0 is the horizontal phase alone: 64 h[l + 3] = the upper half
            // of pair (h[l + 2], h[l + 3]) times 64 (for fx = 0 the picture itself)
            if (want & 1) {
                constexpr uint32_t t64 = 0x40000000u;
                out[0] = pack_sat_u8(dp2a_hi(B.x, t64, init) >> rsh, dp2a_hi(B.y, t64, init) >> rsh,
                                     dp2a_hi(B.z, t64, init) >> rsh, dp2a_hi(B.w, t64, init) >> rsh);
            } else {
                out[0] = 0;
            }
#pragma unroll
            for (int fy = 1; fy < 4; fy++) {
                const uint32_t t03 = tap_word(fy, 0), t47 = tap_word(fy, 1);
                const int vx = vsum(A.x, B.x, C.x, D.x, t03, t47, init) >> rsh;
                const int vy = vsum(A.y, B.y, C.y, D.y, t03, t47, init) >> rsh;
                const int vz = vsum(A.z, B.z, C.z, D.z, t03, t47, init) >> rsh;
                const int vw = vsum(A.w, B.w, C.w, D.w, t03, t47, init) >> rsh;
                out[fy] = pack_sat_u8(vx, vy, vz, vw);
            }
            if (direct) {
                const ptrdiff_t ro = (ptrdiff_t)(y0 + l) * stride;
#pragma unroll
                for (int fy = 0; fy < 4; fy++)
                    if ((want >> fy) & 1) *reinterpret_cast<uint32_t *>(base[fy] + ro) = out[fy];
                continue;
            }
            // output rows clamping to this row: one inside the picture's band,
            // the whole margin run at rows -4 and H + 3
            const int cyl = cy0 + l;
            const int ya = max(cyl == -4 ? y0 : cyl, y0);
            const int yb = min(min(cyl == H + 3 ? y0 + PT_H - 1 : cyl, y0 + PT_H - 1), H + pad - 1);
            for (int y = ya; y <= yb; y++) {
                const ptrdiff_t ro = (ptrdiff_t)y * stride;
#pragma unroll
                for (int fy = 0; fy < 4; fy++)
                    if ((want >> fy) & 1) store_group<VEC>(base[fy] + ro, out[fy], xg, end_col);
            }
        }
    }
}

// Writes the padding of a full-pel plane: (x, y) outside [0, W) x [0, H)
// takes the sample at (clamp(x, 0, W-1), clamp(y, 0, H-1)) (plane_expand_border,
// frame.c:471-507).  One grid row per picture row; 4 columns per thread.
template <bool VEC>
__global__ void expand_plane_kernel(uint8_t *pix, int stride, int W, int H, int pad)
{
    const int groups = (W + 2 * pad + 3) / 4, end_col = W + pad;
    const int y = -pad + (int)blockIdx.y;
    const bool inner_row = y >= 0 && y < H;
    const uint8_t *srow = pix + (ptrdiff_t)clampi(y, 0, H - 1) * stride;
    uint8_t *drow = pix + (ptrdiff_t)y * stride;
    for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < groups; gi += gridDim.x * blockDim.x) {
        const int x = -pad + 4 * gi;
        if (inner_row && x >= 0 && x + 3 < W) continue;
        uint32_t v = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) v |= (uint32_t)srow[clampi(x + c, 0, W - 1)] << (8 * c);
        if (!inner_row) {
            store_group<VEC>(drow + x, v, x, end_col);
        } else {
#pragma unroll
            for (int c = 0; c < 4; c++)
                if ((x + c < 0 || x + c >= W) && x + c < end_col) drow[x + c] = (uint8_t)(v >> (8 * c));
        }
    }
}

}  // namespace xg

using namespace xg;

// ---- per-call drop-ins --------------------------------------------------------
// Footprints: hor reads columns [-3, w+4], ver rows [-3, h+4], ext reads tmp
// rows [-3, h+4]; the luma block ext reads rows [-3, h+3] x columns [-3,
// w+4]; chroma reads [-1, +2] around the block.

namespace {

struct Stage {
    CallCtx &c;
    size_t used = 0;
    explicit Stage(size_t need) : c(call_ctx(need)) {}
    size_t take(size_t bytes) { size_t o = used; used += align_up(bytes); return o; }
    uint8_t *h(size_t o) { return c.h_stage + o; }
    uint8_t *d(size_t o) { return c.d_stage + o; }
};

// Bytes needed for a footprint of `cols` x `rows` elements of `es` bytes.
inline size_t fp(int cols, int rows, int es) { return align_up((size_t)cols * rows * es); }

}  // namespace

extern "C" void xavs2gpu_intpl_luma_hor(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, uint8_t *src, int i_src,
                                        int width, int height, const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7;
    Stage s(fp(fw, height, 1) + fp(width, height, 1) + fp(width, height, 2) + 1024);
    size_t oi = s.take((size_t)fw * height), od = s.take((size_t)width * height), ot = s.take((size_t)width * height * 2);
    pack_rows(s.h(oi), src - 3, i_src, fw, height);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * height, cudaMemcpyHostToDevice, s.c.stream));
    hor8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>((uint8_t *)s.d(od), width, (int16_t *)s.d(ot), width,
                                                                 s.d(oi) + 3, fw, width, height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), s.used - od, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
    unpack_rows(tmp, (intptr_t)i_tmp * 2, s.h(ot), width * 2, height);
}

extern "C" void xavs2gpu_intpl_luma_hor_x3(uint8_t *const dst[3], int i_dst, int16_t *const tmp[3], int i_tmp,
                                           uint8_t *src, int i_src, int width, int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_hor(dst[k], i_dst, tmp[k], i_tmp, src, i_src, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                        const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fh = height + 7;
    Stage s(fp(width, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)width * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3 * (intptr_t)i_src, i_src, width, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)width * fh, cudaMemcpyHostToDevice, s.c.stream));
    ver8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, s.d(oi) + 3 * width, width, width,
                                                                 height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_ver_x3(uint8_t *const dst[3], int i_dst, uint8_t *src, int i_src, int width,
                                           int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_ver(dst[k], i_dst, src, i_src, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_ext(uint8_t *dst, int i_dst, int16_t *tmp, int i_tmp, int width, int height,
                                        const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fh = height + 7;
    Stage s(fp(width, fh, 2) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)width * fh * 2), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), tmp - 3 * (intptr_t)i_tmp, (intptr_t)i_tmp * 2, width * 2, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)width * fh * 2, cudaMemcpyHostToDevice, s.c.stream));
    ext8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, (const int16_t *)s.d(oi) + 3 * width,
                                                                 width, width, height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_ext_x3(uint8_t *const dst[3], int i_dst, int16_t *tmp, int i_tmp, int width,
                                           int height, const int8_t **coeff)
{
    for (int k = 0; k < 3; k++) xavs2gpu_intpl_luma_ext(dst[k], i_dst, tmp, i_tmp, width, height, coeff[k]);
}

extern "C" void xavs2gpu_intpl_luma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7;
    Stage s(fp(fw, height, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * height), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3, i_src, fw, height);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * height, cudaMemcpyHostToDevice, s.c.stream));
    hor8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, nullptr, 0, s.d(oi) + 3, fw, width,
                                                                 height, taps8(coeff));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_luma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff)
{
    xavs2gpu_intpl_luma_ver(dst, i_dst, src, i_src, width, height, coeff);
}

extern "C" void xavs2gpu_intpl_luma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                                              const int8_t *coeff_x, const int8_t *coeff_y)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 7, fh = height + 7;
    Stage s(fp(fw, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - 3 * (intptr_t)i_src - 3, i_src, fw, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * fh, cudaMemcpyHostToDevice, s.c.stream));
    block_ext8_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(s.d(od), width, s.d(oi) + 3 * fw + 3, fw, width,
                                                                       height, taps8(coeff_x), taps8(coeff_y));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

static void chroma_call(int mode, uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width, int height,
                        const int8_t *cx, const int8_t *cy)
{
    if (width <= 0 || height <= 0) return;
    const int fw = width + 3, fh = height + 3;
    Stage s(fp(fw, fh, 1) + fp(width, height, 1) + 512);
    size_t oi = s.take((size_t)fw * fh), od = s.take((size_t)width * height);
    pack_rows(s.h(oi), src - (intptr_t)i_src - 1, i_src, fw, fh);
    XG_CUDA(cudaMemcpyAsync(s.d(oi), s.h(oi), (size_t)fw * fh, cudaMemcpyHostToDevice, s.c.stream));
    Taps4 tx = taps4(cx ? cx : cy), ty = taps4(cy ? cy : cx);
    chroma4_kernel<<<nblocks(width * height), 256, 0, s.c.stream>>>(mode, s.d(od), width, s.d(oi) + fw + 1, fw, width,
                                                                    height, tx, ty);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(s.h(od), s.d(od), (size_t)width * height, cudaMemcpyDeviceToHost, s.c.stream));
    XG_CUDA(cudaStreamSynchronize(s.c.stream));
    unpack_rows(dst, i_dst, s.h(od), width, height);
}

extern "C" void xavs2gpu_intpl_chroma_block_hor(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff)
{
    chroma_call(0, dst, i_dst, src, i_src, width, height, coeff, nullptr);
}

extern "C" void xavs2gpu_intpl_chroma_block_ver(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff)
{
    chroma_call(1, dst, i_dst, src, i_src, width, height, nullptr, coeff);
}

extern "C" void xavs2gpu_intpl_chroma_block_ext(uint8_t *dst, int i_dst, uint8_t *src, int i_src, int width,
                                                int height, const int8_t *coeff_x, const int8_t *coeff_y)
{
    chroma_call(2, dst, i_dst, src, i_src, width, height, coeff_x, coeff_y);
}

// ---- whole-frame planes (device pointers) ---------------------------------------
namespace xg {

// Launches the planes kernel; `mask` has bit k for every plane written.
static int planes_launch(const uint8_t *src, int src_stride, int stride, int width, int height, int pad,
                         const PlaneSet &ps, int mask, int mode, cudaStream_t st)
{
    bool vec = stride % 4 == 0;
    for (int k = 0; k < 16; k++)
        if ((mask >> k) & 1) vec &= ((uintptr_t)ps.p[k] - (uintptr_t)pad) % 4 == 0;
    const int src_words = src_stride % 4 == 0 && (uintptr_t)src % 4 == 0;
    dim3 grid((width + 2 * pad + PT_W - 1) / PT_W, (height + 2 * pad + PT_H - 1) / PT_H);
    if (vec)
        frame_planes_kernel<true><<<grid, kPlaneThreads, 0, st>>>(src, src_stride, stride, width, height, pad, ps,
                                                                   mode, src_words);
    else
        frame_planes_kernel<false><<<grid, kPlaneThreads, 0, st>>>(src, src_stride, stride, width, height, pad, ps,
                                                                    mode, src_words);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}

// A reference picture straight from a W x H source (any stride, no border)
// into its 16 planes: the full-pel plane with its replicated border and the
// 15 sub-pel planes, one launch (replaces the copy, border expansion and
// planes of the reference's frame setup).
int reference_planes_from(const uint8_t *src, int src_stride, int width, int height, int pad, uint8_t *const planes[16],
                          int stride, cudaStream_t st)
{
    PlaneSet ps;
    for (int k = 0; k < 16; k++) ps.p[k] = planes[k];
    return planes_launch(src, src_stride, stride, width, height, pad, ps, 0xFFFF, 2 | 4, st);
}

}  // namespace xg

extern "C" int xavs2gpu_interpolate_frame(const uint8_t *src, int stride, int width, int height, int pad,
                                          uint8_t *const planes[16], int mode, void *stream)
{
    if (width <= 0 || height <= 0 || pad < 4 || stride < width + 2 * pad || (mode != 1 && mode != 2)) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_interpolate_frame", "bad geometry or mode");
        return XAVS2GPU_ERR_ARG;
    }
    PlaneSet ps;
    int mask = 0;
    for (int k = 0; k < 16; k++) {
        ps.p[k] = planes[k];
        bool want = k > 0 && (mode == 2 || k == 2 || k == 8 || k == 10);
        if (want) {
            if (!planes[k]) {
                fail(XAVS2GPU_ERR_ARG, "xavs2gpu_interpolate_frame", "missing output plane");
                return XAVS2GPU_ERR_ARG;
            }
            mask |= 1 << k;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    return planes_launch(src, stride, stride, width, height, pad, ps, mask, mode, st);
}

extern "C" int xavs2gpu_expand_border(uint8_t *pix, int stride, int width, int height, int pad, void *stream)
{
    if (width <= 0 || height <= 0 || pad < 0 || stride < width + 2 * pad) {
        fail(XAVS2GPU_ERR_ARG, "xavs2gpu_expand_border", "bad geometry");
        return XAVS2GPU_ERR_ARG;
    }
    const bool vec = stride % 4 == 0 && ((uintptr_t)pix - (uintptr_t)pad) % 4 == 0;
    const int groups = (width + 2 * pad + 3) / 4;
    dim3 grid((groups + 255) / 256, height + 2 * pad);
    if (vec)
        expand_plane_kernel<true><<<grid, 256, 0, (cudaStream_t)stream>>>(pix, stride, width, height, pad);
    else
        expand_plane_kernel<false><<<grid, 256, 0, (cudaStream_t)stream>>>(pix, stride, width, height, pad);
    count_launch();
    XG_CUDA(cudaGetLastError());
    return XAVS2GPU_OK;
}
