// msod_device.cuh -- device-side building blocks shared by the msod kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "msod.h"

namespace msod {

// Fire-and-forget global reductions (no return value): the element-to-node
// scatter of the residuals (the reference's "!$acc atomic update",
// elem_convec.f90:412-426, elem_diffu.f90:182-192).
__device__ __forceinline__ void red_add(float *addr, float v)
{
    asm volatile("red.global.add.f32 [%0], %1;" ::"l"(addr), "f"(v) : "memory");
}
__device__ __forceinline__ void red_add(double *addr, double v)
{
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(v) : "memory");
}

// Read-only global loads through the non-coherent path.
template <typename T>
__device__ __forceinline__ T ldg(const T *p)
{
    return __ldg(p);
}

// Per-porder launch geometry of the line-parallel element kernels.
//   Q  = points per line, L = lines per direction, N = points per element.
//   QP = padded row pitch in shared memory (odd, so that line loads along x
//        hit distinct banks), ES = shared-memory words per element plane.
//   S  = threads per line (each owns R consecutive points of the line),
//   NE = elements per block, NT = threads per block.
template <typename real, int P>
struct LineGeom {
    static constexpr int Q = P + 1;
    static constexpr int L = Q * Q;
    static constexpr int N = Q * Q * Q;
    static constexpr int QP = (Q % 2 == 0) ? Q + 1 : Q;
    static constexpr int ES = Q * Q * QP;
    static constexpr int S = sizeof(real) == 8 ? Q : (P <= 5 ? 1 : (P <= 7 ? 2 : 3));
    static constexpr int R = (Q + S - 1) / S;
    static constexpr int TPE = L * S;  // threads per element
    static constexpr int CAP = sizeof(real) == 8 ? (TPE <= 128 ? 128 : ((TPE + 31) / 32) * 32)
                                                 : (TPE <= 32 ? 128 : 256);
    static constexpr int NE = CAP / TPE > 0 ? CAP / TPE : 1;
    static constexpr int NT = ((NE * TPE + 31) / 32) * 32;
};

// Per-call element tables in shared memory, read from the caller's
// reference-layout arrays:
//   perm[l]   lattice point l = (K*Q+J)*Q+I (SOD 1-D indices, 0-based) -> gmsh
//             local node a (invAtoIJK - 1)
//   lat[a]    gmsh local node a -> padded lattice offset (K*Q+J)*QP+I
//             (from gmshAtoI/J/K)
//   D[d][r][c] = dlxigp_ip(g, d, c) for a point g whose 1-D index in
//             direction d is r: the 1-D derivative matrix the reference
//             replicates per point (elem_hex.f90:43-44).
// Indices are clamped into range, so malformed tables give wrong numbers
// (caught by msod_check_element_tables), never out-of-bounds accesses.
template <typename real, int P>
__device__ __forceinline__ void load_element_tables(const int *__restrict__ invAtoIJK,
                                                    const int *__restrict__ AtoI,
                                                    const int *__restrict__ AtoJ,
                                                    const int *__restrict__ AtoK,
                                                    const real *__restrict__ dlxigp_ip, int *perm,
                                                    int *lat, real *D, int tid, int nthreads)
{
    using G = LineGeom<real, P>;
    constexpr int Q = G::Q, N = G::N;
    for (int i = tid; i < N; i += nthreads) {
        int a = ldg(invAtoIJK + i) - 1;
        perm[i] = min(max(a, 0), N - 1);
        int I = min(max(ldg(AtoI + i) - 1, 0), Q - 1);
        int J = min(max(ldg(AtoJ + i) - 1, 0), Q - 1);
        int K = min(max(ldg(AtoK + i) - 1, 0), Q - 1);
        lat[i] = (K * Q + J) * G::QP + I;
    }
    __syncthreads();
    for (int i = tid; i < 3 * Q * Q; i += nthreads) {
        const int d = i / (Q * Q), r = (i / Q) % Q, c = i % Q;
        const int l = d == 0 ? r : (d == 1 ? r * Q : r * Q * Q);
        const int g = perm[l];
        D[i] = ldg(dlxigp_ip + (size_t)(c * 3 + d) * N + g);
    }
}

}  // namespace msod
