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
//   S  = threads per line (each owns R consecutive points of the line; S_ > 0
//        overrides the default),
//   NE = elements per block (at most NECAP), NT = threads per block.
template <typename real_t, int P_, int NECAP = 64, int S_ = 0>
struct LineGeom {
    using real = real_t;
    static constexpr int P = P_;
    static constexpr int Q = P + 1;
    static constexpr int L = Q * Q;
    static constexpr int N = Q * Q * Q;
    static constexpr int QP = (Q % 2 == 0) ? Q + 1 : Q;
    static constexpr int ES = Q * Q * QP;
    static constexpr int S = S_ > 0 ? S_ : (sizeof(real) == 8 ? Q : (P <= 5 ? 1 : (P <= 7 ? 2 : 3)));
    static constexpr int R = (Q + S - 1) / S;
    static constexpr int TPE = L * S;  // threads per element
    static constexpr int CAP = sizeof(real) == 8 ? (TPE <= 128 ? 128 : ((TPE + 31) / 32) * 32)
                                                 : (TPE <= 32 ? 128 : 256);
    static constexpr int NE0 = CAP / TPE > 0 ? CAP / TPE : 1;
    static constexpr int NE = NE0 < NECAP ? NE0 : (NECAP > 0 ? NECAP : 1);
    static constexpr int NT = ((NE * TPE + 31) / 32) * 32;
    static constexpr int NPL = NE * ES;  // words per shared-memory plane
};

// Largest element count per block whose `planes` shared-memory planes of
// `bytes` bytes per word fit in `budget` bytes.
constexpr int necap_for(int planes, int es, int bytes, int budget) { return budget / (planes * es * bytes); }

// Thread -> (element, line, segment) of the line-parallel passes.
template <class G>
struct LineThread {
    int el, la, lb, r0;
    bool active;
    __device__ __forceinline__ LineThread(int tid)
    {
        active = tid < G::NE * G::TPE;
        const int t = active ? tid : 0;
        el = t / G::TPE;
        const int rem = t - el * G::TPE;
        const int line = G::S == 1 ? rem : rem / G::S;
        const int seg = G::S == 1 ? 0 : rem - line * G::S;
        la = line % G::Q;
        lb = line / G::Q;
        r0 = seg * G::R;
    }
    __device__ __forceinline__ bool owns(int rr) const { return (G::R * G::S == G::Q) || r0 + rr < G::Q; }
    __device__ __forceinline__ int rc(int rr) const { return owns(rr) ? r0 + rr : 0; }
};

// Offset of point r of the line (la, lb) running in direction DIR, in the
// padded lattice of one element, and its unpadded lattice index.
template <int DIR, int Q, int QP>
__device__ __forceinline__ int line_off(int la, int lb, int r)
{
    return DIR == 0 ? (lb * Q + la) * QP + r : (DIR == 1 ? (lb * Q + r) * QP + la : (r * Q + lb) * QP + la);
}
template <int DIR, int Q>
__device__ __forceinline__ int line_lat(int la, int lb, int r)
{
    return DIR == 0 ? (lb * Q + la) * Q + r : (DIR == 1 ? (lb * Q + r) * Q + la : (r * Q + lb) * Q + la);
}

// Order-preserving map of a float onto a signed int (for integer atomics).
__device__ __forceinline__ int f2key(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float key2f(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }

// Asynchronous 4/8-byte global->shared copies (cp.async); an invalid element is
// zero-filled without reading global memory.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst_smem, const T *src, bool valid)
{
    const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst_smem);
    const int nbytes = valid ? (int)sizeof(T) : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(saddr), "l"(src), "n"(sizeof(T)), "r"(nbytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Grid of a persistent kernel: resident blocks per SM x SMs, capped by the work.
template <typename Kernel>
inline int persistent_grid(Kernel kern, int threads, size_t smem, int ngroups)
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem) != cudaSuccess) return 0;
    if (per < 1) per = 1;
    const long long g = (long long)sms * per;
    return (int)(g < ngroups ? g : ngroups);
}

}  // namespace msod
