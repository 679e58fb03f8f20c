// transform.cu -- AVS2 integer DCT/IDCT (4..32 points, asymmetric shapes and
// the 64-point 5/3-wavelet path), the 4x4 and mode-dependent secondary
// transforms, and quant/dequant for sm_103a: per-call drop-ins of the
// reference's dct_funcs_t (source/common/primitives.h:101-119; C versions
// transform.c:1123-1757 and quant.c:108-247).  The batched
// dct -> quant -> dequant -> idct chain is in tq.cu.
#include "transform_tables.cuh"

#include <cstring>

namespace xg {

// ---- TU geometry -------------------------------------------------------------
// Shift parameters of one TU shape for 8-bit input (transform.c:1123-1587).
struct TuGeom {
    int w, h;          // transform size (after the wavelet for 64-point shapes)
    int s1, s2;        // forward shifts
    int wavelet;       // 1: 64-point shape through the 5/3 wavelet
    int iw, ih;        // input block size
};

__host__ __device__ inline bool tu_geom(int part, int flag, TuGeom &g)
{
    switch (part) {
    case 0: g = {4, 4, 0, 7, 0, 4, 4}; return true;
    case 1: g = {8, 8, 1, 8, 0, 8, 8}; return true;
    case 2: g = {16, 16, 2, 9, 0, 16, 16}; return true;
    case 3: g = {32, 32, 3 + flag, 10, 0, 32, 32}; return true;
    case 15: g = {16, 4, 2, 7, 0, 16, 4}; return true;
    case 16: g = {4, 16, 0, 9, 0, 4, 16}; return true;
    case 19: g = {32, 8, 3, 8 - flag, 0, 32, 8}; return true;
    case 20: g = {8, 32, 1 + flag, 10, 0, 8, 32}; return true;
    case 4: g = {32, 32, 4, 10, 1, 64, 64}; return true;
    case 23: g = {32, 8, 3, 7, 1, 64, 16}; return true;
    case 24: g = {8, 32, 2, 10, 1, 16, 64}; return true;
    default: return false;
    }
}

// ---- block-cooperative passes (all threads of the CTA take part) -------------
__device__ __forceinline__ int basis_d(const int8_t (*B)[32], int N, int k, int n) { return B[k * (32 / N)][n]; }

// out[k*lines + j] = wrap16((sum_n T_N[k][n] in[j*in_stride + n] + add) >> shift)
__device__ void fwd_pass_d(const int8_t (*B)[32], const int16_t *in, int in_stride, int16_t *out, int N, int lines,
                           int shift)
{
    const int add = (1 << shift) >> 1;
    for (int i = threadIdx.x; i < N * lines; i += blockDim.x) {
        int k = i / lines, j = i - k * lines;
        const int16_t *v = in + j * in_stride;
        int s = 0;
        for (int n = 0; n < N; n++) s += basis_d(B, N, k, n) * v[n];
        out[i] = (int16_t)((s + add) >> shift);
    }
}

// out[j*N + n] = clip_bits((sum_k T_N[k][n] in[k*lines + j] + add) >> shift)
__device__ void inv_pass_d(const int8_t (*B)[32], const int16_t *in, int16_t *out, int N, int lines, int shift, int bits)
{
    const int add = (1 << shift) >> 1, hi = (1 << (bits - 1)) - 1, lo = -hi - 1;
    for (int i = threadIdx.x; i < N * lines; i += blockDim.x) {
        int j = i / N, n = i - j * N;
        int s = 0;
        for (int k = 0; k < N; k++) s += basis_d(B, N, k, n) * in[k * lines + j];
        out[i] = (int16_t)clip3_d(lo, hi, (s + add) >> shift);
    }
}

// 5/3 lifting of one vector of length n (stride `st`), in place, keeping the
// reference's int16 storage of every lifted sample (transform.c:586-783).
// Output: low band in the first n/2 entries (stride st).
__device__ void lift_fwd_d(int16_t *v, int st, int n, bool vertical)
{
    int16_t e[64 + 4];
    int16_t *p = e + 2;
    for (int i = 0; i < n; i++) p[i] = v[i * st];
    p[-1] = p[1]; p[-2] = p[2]; p[n] = p[n - 2]; p[n + 1] = p[n - 3];
    for (int i = -1; i < n; i += 2) p[i] = (int16_t)(p[i] - ((p[i - 1] + p[i + 1]) >> 1));
    for (int i = 0; i < n; i += 2)
        p[i] = vertical ? (int16_t)((p[i] << 1) + ((p[i - 1] + p[i + 1] + 1) >> 1))
                        : (int16_t)(p[i] + ((p[i - 1] + p[i + 1] + 2) >> 2));
    for (int i = 0; i < n / 2; i++) v[i * st] = p[2 * i];
}

// Forward wavelet: src (iw x ih, stride iw) -> ll ((iw/2) x (ih/2), stride iw/2).
// `tmp` holds ih x (iw/2).
__device__ void wavelet_fwd_d(const int16_t *src, int16_t *tmp, int16_t *ll, int iw, int ih)
{
    const int hw = iw / 2;
    for (int y = threadIdx.x; y < ih; y += blockDim.x) {
        int16_t row[64];
        for (int x = 0; x < iw; x++) row[x] = src[y * iw + x];
        lift_fwd_d(row, 1, iw, false);
        for (int x = 0; x < hw; x++) tmp[y * hw + x] = row[x];
    }
    __syncthreads();
    for (int x = threadIdx.x; x < hw; x += blockDim.x) {
        int16_t col[64];
        for (int y = 0; y < ih; y++) col[y] = tmp[y * hw + x];
        lift_fwd_d(col, 1, ih, true);
        for (int y = 0; y < ih / 2; y++) ll[y * hw + x] = col[y];
    }
}

// Inverse wavelet (transform.c:787-951): vertical upsampling halves the low
// band and averages between samples; horizontal upsampling only averages.
__device__ void lift_inv_d(const int16_t *in, int ist, int16_t *out, int ost, int n, bool halve)
{
    int16_t p[64 + 2];
    for (int i = 0; i < n / 2; i++) p[2 * i] = in[i * ist];
    p[n] = p[n - 2];
    if (halve)
        for (int i = 0; i <= n; i += 2) p[i] = (int16_t)(p[i] >> 1);
    for (int i = 1; i < n; i += 2) p[i] = (int16_t)((p[i - 1] + p[i + 1]) >> 1);
    for (int i = 0; i < n; i++) out[i * ost] = p[i];
}

__device__ void wavelet_inv_d(const int16_t *ll, int16_t *tmp, int16_t *dst, int ow, int oh)
{
    const int hw = ow / 2;
    for (int x = threadIdx.x; x < hw; x += blockDim.x) lift_inv_d(ll + x, hw, tmp + x, hw, oh, true);
    __syncthreads();
    for (int y = threadIdx.x; y < oh; y += blockDim.x) lift_inv_d(tmp + y * hw, 1, dst + y * ow, 1, ow, false);
}

// Secondary transform on a 4x4 corner (stride st) in place: Y = M X or X M^T
// (M^T when `transposed`), rounding `shift`, clipped to `bits`.  Single
// thread; the caller selects it.
__device__ void sec_apply_d(int16_t *c, int st, const int16_t *m, bool transposed, bool along_rows, int shift, int bits)
{
    int x[4][4];
    const int add = (1 << shift) >> 1, hi = (1 << (bits - 1)) - 1, lo = -hi - 1;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) x[i][j] = c[i * st + j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            int s = add;
            for (int k = 0; k < 4; k++) {
                int mk = transposed ? m[k * 4 + i] : m[i * 4 + k];
                s += mk * (along_rows ? x[j][k] : x[k][j]);
            }
            int v = clip3_d(lo, hi, s >> shift);
            if (along_rows) c[j * st + i] = (int16_t)v;
            else c[i * st + j] = (int16_t)v;
        }
}

__device__ void sec_4x4_fwd_d(int16_t *c, int st)
{
    sec_apply_d(c, st, c_sec_4x4, false, true, 1, 16);
    sec_apply_d(c, st, c_sec_4x4, false, false, 8, 16);
}

__device__ void sec_4x4_inv_d(int16_t *c, int st)
{
    sec_apply_d(c, st, c_sec_4x4, true, false, 5, 16);
    sec_apply_d(c, st, c_sec_4x4, true, true, 14, 9);
}

__device__ __forceinline__ void sec_dirs_d(int mode, bool &vt, bool &ht)
{
    vt = mode >= 0 && mode <= 23;
    ht = (mode >= 13 && mode <= 32) || (mode >= 0 && mode <= 2);
}

// Shared-memory workspace of one TU (largest case: 64x64 input).
struct TuSmem {
    int8_t basis[32][32];
    int16_t a[64 * 64];
    int16_t b[64 * 64];
    int red[32];
};

__device__ void load_basis(TuSmem &s)
{
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) (&s.basis[0][0])[i] = (&c_basis.v[0][0])[i];
}

// Forward transform of the block in s.a (iw x ih, stride iw).  Result:
// w*h coefficients in s.a.
__device__ void tu_forward_d(TuSmem &s, const TuGeom &g)
{
    const int16_t *in = s.a;
    if (g.wavelet) {
        wavelet_fwd_d(s.a, s.b, s.a, g.iw, g.ih);   // ll written into s.a (stride w)
        __syncthreads();
    }
    fwd_pass_d(s.basis, in, g.w, s.b, g.w, g.h, g.s1);    // s.b[k][j]
    __syncthreads();
    fwd_pass_d(s.basis, s.b, g.h, s.a, g.h, g.w, g.s2);   // s.a[m][k]
    __syncthreads();
}

// Inverse transform of the w*h coefficients in s.a; result (iw x ih, stride iw)
// in s.a.  `flag` is the reference's wavelet flag for the 32-point shapes.
__device__ void tu_inverse_d(TuSmem &s, const TuGeom &g, int flag)
{
    const int f = g.wavelet ? 1 : flag;
    inv_pass_d(s.basis, s.a, s.b, g.h, g.w, 5, 16);             // s.b[j][n]
    __syncthreads();
    inv_pass_d(s.basis, s.b, s.a, g.w, g.h, 12 - f, 9 + f);     // s.a[n][x]
    __syncthreads();
    if (g.wavelet) {
        // ll (w x h) in s.a -> copy to s.b, upsample into s.a
        for (int i = threadIdx.x; i < g.w * g.h; i += blockDim.x) s.b[i] = s.a[i];
        __syncthreads();
        wavelet_inv_d(s.b, s.b + 2048, s.a, g.iw, g.ih);
        __syncthreads();
    }
}

__device__ int block_sum(int v, int *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    __syncthreads();
    return t;
}

// quant_c (quant.c:108-120): sign of zero counts as positive
__device__ __forceinline__ int16_t quant1(int c, int scale, int shift, int add)
{
    int q = (iabs_d(c) * scale + add) >> shift;
    return (int16_t)(c < 0 ? -q : q);
}

// dequant_c (quant.c:173-184): zeros stay zero
__device__ __forceinline__ int16_t dequant1(int c, int scale, int shift)
{
    if (!c) return 0;
    return (int16_t)clip3_d(-32768, 32767, (c * scale + (1 << (shift - 1))) >> shift);
}

// ---- per-call kernels -----------------------------------------------------------
// op 0: dct, 1: idct, 2: dct_half.  `stride` is the reference's i_src/i_dst
// (the low bit is the wavelet flag of the 32-point shapes).
__global__ void __launch_bounds__(256) tu_percall_kernel(int op, int part, int flag, const int16_t *in, int16_t *out)
{
    extern __shared__ __align__(16) uint8_t smem_raw[];
    TuSmem &s = *reinterpret_cast<TuSmem *>(smem_raw);
    TuGeom g;
    tu_geom(part, flag, g);
    load_basis(s);
    const int n_in = op == 1 ? g.w * g.h : g.iw * g.ih;
    for (int i = threadIdx.x; i < n_in; i += blockDim.x) s.a[i] = in[i];
    __syncthreads();
    if (op == 1) {
        tu_inverse_d(s, g, flag);
        for (int i = threadIdx.x; i < g.iw * g.ih; i += blockDim.x) out[i] = s.a[i];
    } else {
        tu_forward_d(s, g);
        for (int i = threadIdx.x; i < g.w * g.h; i += blockDim.x) {
            int16_t v = s.a[i];
            if (op == 2) {   // dct_half: keep the top-left 16x16 of the 32x32 output
                int y = i >> 5, x = i & 31;
                if (y >= 16 || x >= 16) v = 0;
            }
            out[i] = v;
        }
    }
}

// op 0: 4x4 fwd, 1: 4x4 inv, 2: mode fwd, 3: mode inv
__global__ void sec_percall_kernel(int op, int16_t *c, int mode, int b_top, int b_left)
{
    if (threadIdx.x != 0) return;
    bool vt, ht;
    sec_dirs_d(mode, vt, ht);
    switch (op) {
    case 0: sec_4x4_fwd_d(c, 4); break;
    case 1: sec_4x4_inv_d(c, 4); break;
    case 2:
        if (vt && b_top) sec_apply_d(c, 4, c_sec_mode, false, false, 7, 16);
        if (ht && b_left) sec_apply_d(c, 4, c_sec_mode, false, true, 7, 16);
        break;
    default:
        if (ht && b_left) sec_apply_d(c, 4, c_sec_mode, true, true, 7, 16);
        if (vt && b_top) sec_apply_d(c, 4, c_sec_mode, true, false, 7, 16);
        break;
    }
}

// op 0 quant, 1 dequant, 2 wquant, 3 abs, 4 add_sign; result[0] = count
__global__ void __launch_bounds__(256) quant_percall_kernel(int op, int16_t *c, const int16_t *aux, const int *ls,
                                                            int n, int scale, int shift, int add, int *result)
{
    __shared__ int red[32];
    int nz = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        int v = c[i];
        switch (op) {
        case 0: c[i] = quant1(v, scale, shift, add); nz += c[i] != 0; break;
        case 1: c[i] = dequant1(v, scale, shift); break;
        case 2: {
            int a = (iabs_d(v) * ls[i] + (1 << 18)) >> 19;
            int q = (a * scale + add) >> shift;
            c[i] = (int16_t)(v < 0 ? -q : q);
            nz += c[i] != 0;
        } break;
        case 3: c[i] = (int16_t)iabs_d(aux[i]); break;
        default:
            c[i] = (int16_t)(v > 0 ? aux[i] : -aux[i]);
            nz += aux[i] != 0;
            break;
        }
    }
    nz = block_sum(nz, red);
    if (threadIdx.x == 0) result[0] = nz;
}

}  // namespace xg

using namespace xg;

// ---- per-call entry points -------------------------------------------------------
static void tu_call(int op, int part, const int16_t *src, int16_t *dst, int stride)
{
    const int flag = (part == 3 || part == 19 || part == 20) ? (stride & 1) : 0;
    TuGeom g;
    tu_geom(part, flag, g);
    // Input/output strides in elements.  The 32-point shapes drop the flag
    // bit and keep only 8 bits of the stride (transform.c:1262, 1304, ...);
    // the 64-point shapes read/write contiguously.
    int st = stride;
    if (part == 3 || part == 19 || part == 20) st &= 0xFE;
    if (g.wavelet) st = g.iw;
    const int in_w = op == 1 ? g.w : g.iw, in_h = op == 1 ? g.h : g.ih;
    const int out_w = op == 1 ? g.iw : g.w, out_h = op == 1 ? g.ih : g.h;
    const size_t o_in = 0, o_out = align_up((size_t)in_w * in_h * 2);
    CallCtx &c = call_ctx(o_out + align_up((size_t)out_w * out_h * 2));
    if (op == 1) memcpy(c.h_stage + o_in, src, (size_t)in_w * in_h * 2);     // coefficients are contiguous
    else pack_rows(c.h_stage + o_in, src, (intptr_t)st * 2, in_w * 2, in_h);
    XG_CUDA(cudaMemcpyAsync(c.d_stage + o_in, c.h_stage + o_in, (size_t)in_w * in_h * 2, cudaMemcpyHostToDevice, c.stream));
    tu_percall_kernel<<<1, 256, sizeof(TuSmem), c.stream>>>(op, part, flag, (const int16_t *)(c.d_stage + o_in),
                                                           (int16_t *)(c.d_stage + o_out));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage + o_out, c.d_stage + o_out, (size_t)out_w * out_h * 2, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    if (op == 1) unpack_rows(dst, (intptr_t)st * 2, c.h_stage + o_out, out_w * 2, out_h);
    else memcpy(dst, c.h_stage + o_out, (size_t)out_w * out_h * 2);
}

#define XG_DEFINE_DCT(w, h)                                                                   \
    extern "C" void xavs2gpu_dct_##w##x##h(const int16_t *src, int16_t *dst, int i_src)        \
    {                                                                                         \
        tu_call(0, XAVS2GPU_LUMA_##w##x##h, src, dst, i_src);                                 \
    }                                                                                         \
    extern "C" void xavs2gpu_idct_##w##x##h(const int16_t *src, int16_t *dst, int i_dst)       \
    {                                                                                         \
        tu_call(1, XAVS2GPU_LUMA_##w##x##h, src, dst, i_dst);                                 \
    }
XAVS2GPU_FOR_EACH_TU(XG_DEFINE_DCT)

extern "C" void xavs2gpu_dct_32x32_half(const int16_t *src, int16_t *dst, int i_src)
{
    tu_call(2, XAVS2GPU_LUMA_32x32, src, dst, i_src);
}

extern "C" void xavs2gpu_dct_64x64_half(const int16_t *src, int16_t *dst, int i_src)
{
    tu_call(2, XAVS2GPU_LUMA_64x64, src, dst, i_src);
}

static void sec_call(int op, int16_t *coeff, int i_coeff, int mode, int b_top, int b_left)
{
    CallCtx &c = call_ctx(256);
    pack_rows(c.h_stage, coeff, (intptr_t)i_coeff * 2, 8, 4);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, 32, cudaMemcpyHostToDevice, c.stream));
    sec_percall_kernel<<<1, 32, 0, c.stream>>>(op, (int16_t *)c.d_stage, mode, b_top, b_left);
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage, c.d_stage, 32, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    unpack_rows(coeff, (intptr_t)i_coeff * 2, c.h_stage, 8, 4);
}

extern "C" void xavs2gpu_transform_4x4_2nd(int16_t *coeff, int i_coeff) { sec_call(0, coeff, i_coeff, 0, 0, 0); }
extern "C" void xavs2gpu_inv_transform_4x4_2nd(int16_t *coeff, int i_coeff) { sec_call(1, coeff, i_coeff, 0, 0, 0); }
extern "C" void xavs2gpu_transform_2nd(int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left)
{
    sec_call(2, coeff, i_coeff, i_mode, b_top, b_left);
}
extern "C" void xavs2gpu_inv_transform_2nd(int16_t *coeff, int i_coeff, int i_mode, int b_top, int b_left)
{
    sec_call(3, coeff, i_coeff, i_mode, b_top, b_left);
}

static int quant_call(int op, int16_t *coef, const int16_t *aux, const int *ls, int n, int scale, int shift, int add)
{
    if (n <= 0) return 0;
    const size_t o_c = 0, o_aux = align_up((size_t)n * 2), o_ls = o_aux + align_up((size_t)n * 2);
    const size_t o_res = o_ls + align_up((size_t)n * 4);
    CallCtx &c = call_ctx(o_res + 256);
    memcpy(c.h_stage + o_c, coef, (size_t)n * 2);
    if (aux) memcpy(c.h_stage + o_aux, aux, (size_t)n * 2);
    if (ls) memcpy(c.h_stage + o_ls, ls, (size_t)n * 4);
    XG_CUDA(cudaMemcpyAsync(c.d_stage, c.h_stage, o_res, cudaMemcpyHostToDevice, c.stream));
    quant_percall_kernel<<<1, 256, 0, c.stream>>>(op, (int16_t *)(c.d_stage + o_c), (const int16_t *)(c.d_stage + o_aux),
                                                 (const int *)(c.d_stage + o_ls), n, scale, shift, add,
                                                 (int *)(c.d_stage + o_res));
    count_launch();
    XG_CUDA(cudaMemcpyAsync(c.h_stage, c.d_stage, o_res + 4, cudaMemcpyDeviceToHost, c.stream));
    XG_CUDA(cudaStreamSynchronize(c.stream));
    memcpy(coef, c.h_stage + o_c, (size_t)n * 2);
    return *(int *)(c.h_stage + o_res);
}

extern "C" int xavs2gpu_quant(int16_t *coef, const int i_coef, const int scale, const int shift, const int add)
{
    return quant_call(0, coef, nullptr, nullptr, i_coef, scale, shift, add);
}
extern "C" void xavs2gpu_dequant(int16_t *coef, const int i_coef, const int scale, const int shift)
{
    quant_call(1, coef, nullptr, nullptr, i_coef, scale, shift, 0);
}
extern "C" int xavs2gpu_quant_weighted(int16_t *coef, const int i_coef, const int scale, const int shift, const int add,
                                       int *levelscale)
{
    return quant_call(2, coef, nullptr, levelscale, i_coef, scale, shift, add);
}
extern "C" void xavs2gpu_abs_coeff(int16_t *dst, const int16_t *src, const int i_coef)
{
    quant_call(3, dst, src, nullptr, i_coef, 0, 0, 0);
}
extern "C" int xavs2gpu_add_sign(int16_t *dst, const int16_t *abs_val, const int i_coef)
{
    return quant_call(4, dst, abs_val, nullptr, i_coef, 0, 0, 0);
}

extern "C" void xavs2gpu_dct_init(uint32_t cpuid, xavs2gpu_dct_funcs_t *dctf)
{
    (void)cpuid;
#define XG_SET(w, h)                                                  \
    dctf->dct[XAVS2GPU_LUMA_##w##x##h] = xavs2gpu_dct_##w##x##h;       \
    dctf->idct[XAVS2GPU_LUMA_##w##x##h] = xavs2gpu_idct_##w##x##h;
    XAVS2GPU_FOR_EACH_TU(XG_SET)
#undef XG_SET
    dctf->dct_half[XAVS2GPU_LUMA_32x32] = xavs2gpu_dct_32x32_half;
    dctf->dct_half[XAVS2GPU_LUMA_64x64] = xavs2gpu_dct_64x64_half;
    dctf->transform_4x4_2nd = xavs2gpu_transform_4x4_2nd;
    dctf->inv_transform_4x4_2nd = xavs2gpu_inv_transform_4x4_2nd;
    dctf->transform_2nd = xavs2gpu_transform_2nd;
    dctf->inv_transform_2nd = xavs2gpu_inv_transform_2nd;
}

extern "C" void xavs2gpu_quant_init(uint32_t cpuid, xavs2gpu_dct_funcs_t *dctf)
{
    (void)cpuid;
    dctf->quant = xavs2gpu_quant;
    dctf->dequant = xavs2gpu_dequant;
    dctf->wquant = xavs2gpu_quant_weighted;
    dctf->abs_coeff = xavs2gpu_abs_coeff;
    dctf->add_sign = xavs2gpu_add_sign;
}
