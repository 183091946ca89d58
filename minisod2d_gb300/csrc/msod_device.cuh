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
    // The line of a bank-aware map entry (LineMap), one thread per line.
    __device__ __forceinline__ LineThread(unsigned code, bool)
    {
        active = code != 0xFFFFu;
        el = active ? (int)(code >> 8) : 0;
        lb = active ? (int)((code >> 4) & 15u) : 0;
        la = active ? (int)(code & 15u) : 0;
        r0 = 0;
    }
    __device__ __forceinline__ bool owns(int rr) const { return (G::R * G::S == G::Q) || r0 + rr < G::Q; }
    __device__ __forceinline__ int rc(int rr) const { return owns(rr) ? r0 + rr : 0; }
};

// Offset of point r of the line (la, lb) running in direction DIR, in the
// padded lattice of one element, and its unpadded lattice index.
template <int DIR, int Q, int QP>
__host__ __device__ constexpr int line_off(int la, int lb, int r)
{
    return DIR == 0 ? (lb * Q + la) * QP + r : (DIR == 1 ? (lb * Q + r) * QP + la : (r * Q + lb) * QP + la);
}

// Bank-aware assignment of threads to the block's GLL lines, one per
// direction (one thread per line).  Shared-memory accesses of a line pass
// address point r of every line at (line base + r * stride), so a warp's
// lanes conflict exactly when their lines' bases fall in the same bank (mod
// 32).  Warps are filled one after the other with lines of distinct banks,
// taking from the banks with the most lines left first, so that the lines a
// bank has beyond one per warp end up together in the last warps.  At porder 4
// (5 elements per 128-thread block) this turns the 2-way conflicts of every
// eta and zeta access of the natural order (lines of consecutive elements
// side by side) into one extra wavefront on one or two of the four warps
// (counted from the index arithmetic: 100 -> 75 wavefronts per point step of
// the three directions, 60 without conflicts).
// code = (el << 8) | (lb << 4) | la; 0xFFFF marks an idle thread.
template <class G>
struct LineMap {
    unsigned short code[3][G::NT];
};
template <class G, int DIR>
constexpr int line_bank(int l)
{
    return (l / G::L * G::ES + line_off<DIR, G::Q, G::QP>(l % G::L % G::Q, l % G::L / G::Q, 0)) % 32;
}
template <class G, int DIR>
constexpr void fill_line_map(LineMap<G> &m)
{
    constexpr int NL = G::NE * G::L, NW = G::NT / 32;
    int start[33] = {}, left_b[32] = {}, order[NL] = {};
    for (int l = 0; l < NL; ++l) ++start[line_bank<G, DIR>(l) + 1];
    for (int b = 0; b < 32; ++b) {
        left_b[b] = start[b + 1];
        start[b + 1] += start[b];
    }
    {
        int fill[32] = {};
        for (int b = 0; b < 32; ++b) fill[b] = start[b];
        for (int l = 0; l < NL; ++l) order[fill[line_bank<G, DIR>(l)]++] = l;
    }
    for (int t = 0; t < G::NT; ++t) m.code[DIR][t] = 0xFFFF;
    int left = NL;
    for (int w = 0; w < NW; ++w) {
        const int want = left < 32 ? left : 32;
        int taken = 0;
        while (taken < want) {
            // One pass over distinct banks, most lines left first (ties: lower bank).
            bool used[32] = {};
            bool progress = false;
            while (taken < want) {
                int best = -1;
                for (int b = 0; b < 32; ++b)
                    if (!used[b] && left_b[b] > 0 && (best < 0 || left_b[b] > left_b[best])) best = b;
                if (best < 0) break;
                used[best] = true;
                const int l = order[start[best]++];
                --left_b[best];
                const int el = l / G::L, line = l % G::L;
                m.code[DIR][32 * w + taken] = (unsigned short)((el << 8) | ((line / G::Q) << 4) | (line % G::Q));
                ++taken;
                progress = true;
            }
            if (!progress) break;
        }
        left -= taken;
    }
}
template <class G>
constexpr LineMap<G> make_line_map()
{
    static_assert(G::S == 1 && G::NE < 256 && G::Q <= 16, "one thread per line");
    LineMap<G> m{};
    fill_line_map<G, 0>(m);
    fill_line_map<G, 1>(m);
    fill_line_map<G, 2>(m);
    return m;
}
template <class G>
__device__ const LineMap<G> kLineMap = make_line_map<G>();
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

// ---------------------------------------------------------------------------
// 1-D bulk copies (cp.async.bulk, the TMA engine's untiled form) completing on
// a shared-memory mbarrier.  Used to stage the contiguous per-group spans of
// He and gpvol: one elected thread issues the copy, no other thread spends an
// instruction or a register on it, and the data land in shared memory without
// passing through the L1 sector path.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One arrival that also expects `bytes` of asynchronous copies on this phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// Orders this thread's earlier generic-proxy accesses of shared memory (and,
// after a barrier, the block's) before later async-proxy writes (bulk copies).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// dst (shared) <- src (global), `bytes` bytes; both addresses 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase of the given parity to complete, for at most about
// 2^20 polls (~0.1 s with the back-off; a healthy copy of a group's span
// completes in microseconds).  Returns false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    for (int it = 0; it < (1 << 20); ++it) {
        if (mbar_test(bar, parity)) return true;
        if (it >= 32) __nanosleep(64);
    }
    return false;
}

// A contiguous global span [src, src + bytes) staged in shared memory at
// dst_base + (src mod 16): the 16-byte-aligned interior by one bulk copy, the
// unaligned head and tail (at most 12 bytes each; spans are 4-byte aligned) by
// threads 0..5 with plain loads.  Returns the bulk bytes the caller's
// mbar_arrive_expect_tx must announce.  Thread `issuer` issues the copy;
// dst_base is 16-byte aligned and holds bytes + 32.
// L2 prefetch of the 16-byte-aligned interior of [p, p + nbytes) by the bulk
// copy unit (one thread; a hint with nothing to wait for; no byte outside the
// span is touched).  No memory clobber: the prefetch writes nothing, and a
// clobber would keep the compiler from moving loads across it.
__device__ __forceinline__ void prefetch_span_l2(const void *p, size_t nbytes)
{
    const size_t a = reinterpret_cast<size_t>(p);
    const size_t a16 = (a + 15) & ~(size_t)15, e16 = (a + nbytes) & ~(size_t)15;
    if (a16 < e16)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a16), "r"((unsigned)(e16 - a16)));
}

// He(3,3,ngaus,e) and gpvol(ngaus,e) of element e into L2 (one thread).
__device__ __forceinline__ void prefetch_element_l2(const float *He, const float *gpvol, int e, int ngaus)
{
    prefetch_span_l2(He + (size_t)e * ngaus * 9, (size_t)ngaus * 9 * sizeof(float));
    prefetch_span_l2(gpvol + (size_t)e * ngaus, (size_t)ngaus * sizeof(float));
}

// L2 prefetch of the sector at p (a hint).
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

struct SpanPlan {
    const char *src;
    unsigned bytes, head, bulk, tail, shift;
    __device__ __forceinline__ SpanPlan(const void *p, size_t nbytes)
    {
        src = static_cast<const char *>(p);
        const size_t a = reinterpret_cast<size_t>(src);
        shift = (unsigned)(a & 15);
        bytes = (unsigned)nbytes;
        const size_t a16 = (a + 15) & ~(size_t)15, e = a + nbytes, e16 = e & ~(size_t)15;
        if (a16 < e16) {
            head = (unsigned)(a16 - a);
            bulk = (unsigned)(e16 - a16);
            tail = (unsigned)(e - e16);
        } else {
            head = (unsigned)nbytes;
            bulk = 0;
            tail = 0;
        }
    }
    // The bulk part (one thread).
    __device__ __forceinline__ void issue(char *dst_base, unsigned long long *bar) const
    {
        if (bulk) bulk_g2s(dst_base + shift + head, src + head, bulk, bar);
    }
    // Head and tail words: word w < 3 of the head, 3 <= w < 6 of the tail (threads 0..5);
    // all of the span when it is too short for a bulk part.
    __device__ __forceinline__ void plain(char *dst_base, int w) const
    {
        if (bulk == 0) {
            for (unsigned o = 4u * (unsigned)w; o < bytes; o += 24u)
                *reinterpret_cast<float *>(dst_base + shift + o) = __ldg(reinterpret_cast<const float *>(src + o));
            return;
        }
        if (w < 3) {
            const unsigned o = 4u * (unsigned)w;
            if (o < head)
                *reinterpret_cast<float *>(dst_base + shift + o) = __ldg(reinterpret_cast<const float *>(src + o));
        } else if (w < 6) {
            const unsigned o = head + bulk + 4u * (unsigned)(w - 3);
            if (o < bytes)
                *reinterpret_cast<float *>(dst_base + shift + o) = __ldg(reinterpret_cast<const float *>(src + o));
        }
    }
};

// Appends e to list[*count ..] for every lane whose f is set, with one atomic
// per warp; every lane of the warp calls it (the list order is unspecified).
__device__ __forceinline__ void warp_append(bool f, int e, int *list, int *count)
{
    const unsigned m = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (m && lane == __ffs(m) - 1) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, m ? __ffs(m) - 1 : 0);
    if (f) list[base + __popc(m & ((1u << lane) - 1u))] = e;
}

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
