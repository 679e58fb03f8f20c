// transform_tables.cuh -- AVS2 transform and quantiser constants shared by
// the per-call transform kernels (transform.cu) and the batched TU chain
// (tq.cu).  Each translation unit gets its own constant-bank copy.
#pragma once
#include "xavs2gpu_common.cuh"

namespace xg {

// ---- DCT basis ------------------------------------------------------------
// Every AVS2 basis entry is +-c[a] for the reduced angle a = k(2n+1) mod 128
// (units of pi/64); the N-point matrix is rows k*32/N of the 32-point one.
struct Basis32 { int8_t v[32][32]; };

static constexpr int8_t kCos[32] = {32, 45, 45, 45, 44, 44, 43, 43, 42, 41, 40, 39, 38, 36, 35, 34,
                                    32, 30, 29, 27, 25, 23, 21, 19, 17, 15, 13, 11, 9,  7,  4,  2};

static constexpr Basis32 make_basis()
{
    Basis32 b{};
    for (int k = 0; k < 32; k++)
        for (int n = 0; n < 32; n++) {
            int a = (k * (2 * n + 1)) % 128, s = 1;
            if (a > 64) a = 128 - a;
            if (a > 32) { a = 64 - a; s = -1; }
            b.v[k][n] = (int8_t)(k == 0 ? 32 : s * kCos[a]);
        }
    return b;
}

static __constant__ Basis32 c_basis = make_basis();

// Secondary transform matrices (transform.c:140-155), fixed by the standard.
static __constant__ int16_t c_sec_mode[16] = {123, -35, -8, -3, -32, -120, 30, 10, 14, 25, 123, -22, 8, 13, 19, 126};
static __constant__ int16_t c_sec_4x4[16] = {34, 58, 72, 81, 77, 69, -7, -75, 79, -33, -75, 58, 55, -84, 73, -28};

// Quant tables (quant.c:55-81).  IQ shift: 15 - qp/8, except that qp 16,
// 32, 40 and 48 keep the previous group's shift (quant.c:85-96).
static __constant__ uint16_t c_q_scale[80] = {
    32768, 29775, 27554, 25268, 23170, 21247, 19369, 17770, 16302, 15024, 13777, 12634, 11626, 10624, 9742, 8958,
    8192,  7512,  6889,  6305,  5793,  5303,  4878,  4467,  4091,  3756,  3444,  3161,  2894,  2654,  2435, 2235,
    2048,  1878,  1722,  1579,  1449,  1329,  1218,  1117,  1024,  939,   861,   790,   724,   664,   609,  558,
    512,   470,   430,   395,   362,   332,   304,   279,   256,   235,   215,   197,   181,   166,   152,  140,
    128,   116,   108,   99,    91,    83,    76,    69,    64,    59,    54,    49,    45,    41,    38,   35};
static __constant__ uint16_t c_iq_scale[80] = {
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933,
    65535, 35734, 38968, 42577, 46341, 50617, 55027, 60097, 32809, 35734, 38968, 42454, 46382, 50576, 55109, 60056,
    65535, 35734, 38968, 42495, 46320, 50515, 55109, 60076, 65535, 35744, 38968, 42495, 46341, 50535, 55099, 60087,
    65535, 35734, 38973, 42500, 46341, 50535, 55109, 60097, 32771, 35734, 38965, 42497, 46341, 50535, 55109, 60099,
    32768, 36061, 38968, 42495, 46341, 50535, 55437, 60424, 32932, 35734, 38968, 42495, 46177, 50535, 55109, 59933};

__host__ __device__ inline int iq_shift_of(int qp)
{
    int s = 15 - (qp >> 3);
    if (qp == 16 || qp == 32 || qp == 40 || qp == 48) s += 1;
    return s;
}

// T32[k][n] as a constant expression (folded when k and n are known at
// compile time): the same reduced-angle rule as make_basis.
__host__ __device__ constexpr int basis32(int k, int n)
{
    constexpr int8_t c[32] = {32, 45, 45, 45, 44, 44, 43, 43, 42, 41, 40, 39, 38, 36, 35, 34,
                              32, 30, 29, 27, 25, 23, 21, 19, 17, 15, 13, 11, 9,  7,  4,  2};
    int a = (k * (2 * n + 1)) % 128, s = 1;
    if (a > 64) a = 128 - a;
    if (a > 32) { a = 64 - a; s = -1; }
    return k == 0 ? 32 : s * c[a];
}

}  // namespace xg
