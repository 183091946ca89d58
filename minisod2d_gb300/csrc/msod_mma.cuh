// msod_mma.cuh -- helpers of the mixed-precision (tensor-core) kernels:
// hi + lo half splits, ldmatrix / mma.sync wrappers, the swizzled layout of
// one field's half plane, float -> double on the integer pipe.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace msod {

// L2 prefetch of each element's He and gpvol spans an element ahead in the
// mixed-precision kernels (1; 0 = none).  Off: measured slower, FP16
// convection / diffusion 6.16 / 4.36 ms against 4.82 / 4.14 ms on 51^3
// porder-5 hexes, 2.05 / 2.09 against 2.05 / 2.05 ms on 32^3 porder 7 (the
// plain kernels gain 1-3 % from the same prefetch).
#ifndef MIXED_PREFETCH
#define MIXED_PREFETCH 0
#endif

constexpr int kRowB = 16;  // bytes per half-plane row: 8 halves along i

// One field half of an element: 8 rows per k-plane of the element, 8 Q rows.
// The transposed (zeta) reads of input points beyond Q, which meet zero
// coefficients, and the discarded tiles of low orders reach up to row 63:
// past the last plane they land in a zero guard of (64 - 8 Q) rows.
// Measured against 8 x 8-row planes for every order (48^3 hexes): porder-5
// convection 5.24 -> 4.04 ms and porder-4 diffusion 2.78 -> 2.27 ms (more
// blocks per SM), the other kernels unchanged (0 selects the full planes).
#ifndef MIXED_TRIM_PLANES
#define MIXED_TRIM_PLANES 1
#endif
template <int Q>
constexpr int plane_bytes()
{
    return (MIXED_TRIM_PLANES ? 8 * Q : 64) * kRowB;
}
template <int Q>
constexpr int plane_guard_bytes()
{
    return (MIXED_TRIM_PLANES ? 64 - 8 * Q : 0) * kRowB;
}

// Row (k, j) of a half plane sits at position 8k + (j xor k): the eight rows
// of every ldmatrix phase fall on distinct banks for xi, eta and zeta lines.
__device__ __forceinline__ int row_pos(int k, int j) { return 8 * k + (j ^ k); }

template <bool BF16>
__device__ __forceinline__ unsigned pack2(float a, float b)
{
    if (BF16) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const unsigned *>(&h);
    }
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const unsigned *>(&h);
}

// Split of a pair of derivative-matrix entries into hi and lo halves.
template <bool BF16>
__device__ __forceinline__ void split_pair(float a, float b, unsigned &hi, unsigned &lo)
{
    hi = pack2<BF16>(a, b);
    float2 f;
    if (BF16)
        f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&hi));
    else
        f = __half22float2(*reinterpret_cast<const __half2 *>(&hi));
    lo = pack2<BF16>(a - f.x, b - f.y);
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void *row)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void *row)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// d = A B + d (m16n8k16, FP32 accumulate).
template <bool BF16>
__device__ __forceinline__ void mma_acc(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    if (BF16)
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                     "{%8,%9}, {%0,%1,%2,%3};"
                     : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    else
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                     "{%8,%9}, {%0,%1,%2,%3};"
                     : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// float -> double by re-biasing the IEEE exponent on the integer pipe (FP64
// arithmetic is scarce on this GPU); zeros, subnormals, infinities and NaNs
// take the FP64 conversion.
__device__ __forceinline__ double f2d(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned ex = (b >> 23) & 0xFFu;
    if (ex == 0u || ex == 0xFFu) return (double)x;
    const unsigned long long bits = ((unsigned long long)(b >> 31) << 63) |
                                    ((unsigned long long)(ex + (1023u - 127u)) << 52) |
                                    ((unsigned long long)(b & 0x7FFFFFu) << 29);
    return __longlong_as_double((long long)bits);
}

// A scaled pair -> packed hi halves (rint: exact small integers) and lo halves
// (the remainders, |lo| <= 1/2).
template <bool BF16>
__device__ __forceinline__ void split_scaled(float a, float b, unsigned &hi, unsigned &lo)
{
    const float M = 12582912.0f;  // 1.5 * 2^23: adding and subtracting it rounds to an integer
    const float ha = __fsub_rn(__fadd_rn(a, M), M), hb = __fsub_rn(__fadd_rn(b, M), M);
    hi = pack2<BF16>(ha, hb);
    lo = pack2<BF16>(__fsub_rn(a, ha), __fsub_rn(b, hb));
}

// Power-of-two scale s = 2^(bits-1-ex) of a field whose maximum magnitude
// (bit pattern of a non-negative float) lies in [2^ex, 2^(ex+1)), and 1/s;
// ex is clamped so both stay normal.
__device__ __forceinline__ void scale_from_max(unsigned maxbits, int bits, float &s, float &inv)
{
    int ex = (int)((maxbits >> 23) & 0xFFu) - 127;
    ex = min(max(ex, -100), 127);
    s = __int_as_float((127 + bits - 1 - ex) << 23);
    inv = __int_as_float((127 + ex - (bits - 1)) << 23);
}

}  // namespace msod
