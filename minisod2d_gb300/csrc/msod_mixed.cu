// msod_mixed.cu -- mixed-precision hex GLL convection residual on the tensor cores.
//
// Same residuals as full_convec_ijk (elem_convec.f90:198-431, Rener per
// :674-832; formulas in msod_convec.cu) from FP32 fields, with:
//   * the 1-D derivative contractions of the 31 differentiated nodal products
//     on the tensor cores as FP16 (or BF16) hi + lo split products with FP32
//     accumulation;
//   * the nodal scatter-add and the final energy-flux assembly in FP64 (the
//     outputs are FP64 arrays).
//
// Splitting.  Each field f of an element is shifted by its value at the
// element's lattice node (0,0,0) -- the derivative operator annihilates
// constants, so derivatives are unchanged while the split only has to carry
// the field's variation over the element -- and scaled by a power of two s_f
// chosen per element and field so that max |s_f (f - f_ref)| lies in
// [2^(B-1), 2^B) with B = 11 (FP16) or 8 (BF16).  hi = rint(v) is then an
// integer of at most B bits (exact in the half format) and lo = v - hi lies
// in [-1/2, 1/2].  The derivative matrix is split by plain rounding,
// D = D_hi + D_lo.  Products, shifts and scalings use explicit roundings, so
// a field that is constant over the element splits into exact zeros.
//
// Contraction.  Per (field, direction, 16 lines) two accumulating
// mma.sync.m16n8k16:
//   A (16x16) = [f_hi | f_lo]          rows: line, cols: input point (hi | lo)
//   B1 (16x8) = [D_hi^T ; D_hi^T]      rows: input point (hi | lo), cols: output point
//   B2 (16x8) = [D_lo^T ; 0]
// C = f_hi D_hi^T + f_lo D_hi^T + f_hi D_lo^T (the dropped f_lo D_lo^T is
// below 2^-21 of the product).  Lines shorter than 8 points are zero padded.
//
// Shared-memory layout of one field half: 64 rows of 16 bytes (8 halves along
// i), row (k, j) stored at position 8k + (j xor k).  ldmatrix reads the A
// operand of xi lines directly (rows = lines) and of eta / zeta lines
// transposed (rows = input points); the xor swizzle keeps the eight rows of
// every ldmatrix phase on distinct banks in all three directions.
//
// Accumulation.  As in the FP32 kernel, each direction pass adds the
// contribution of its iso-parametric derivatives, through the He column of
// that direction and the point's own nodal values, to seven per-point
// accumulators in shared memory; the last pass assembles the energy residual
// in FP64 and scatter-adds all residuals with red.global.add.f64.
// porder 1..7; persistent blocks of four warps, one element at a time.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"
#include "msod_mma.cuh"

namespace msod {
namespace {

constexpr int kNF = 31;       // differentiated products
constexpr int kThreads = 128;

enum { B_RHO = 0, B_P, B_E, B_U0, B_U1, B_U2, B_Q0, B_Q1, B_Q2, NBASE };
enum { A_M = 0, A_MOM0, A_MOM1, A_MOM2, A_E, A_DIVU, A_DIVQ, NACC };

// Field numbering: 0 rho, 1 p, 2-4 u_i, 5-7 q_i, 8-16 q_i u_j (i major),
// 17-22 u_i u_j (i <= j: 00 01 02 11 12 22), 23 H, 24 rho H, 25-27 rho H u_i,
// 28-30 H u_i, with H = E + |u|^2 / 2.
struct Nodal {
    float r, p, u[3], q[3], H, rH;
};

__device__ __forceinline__ Nodal nodal_from(const float *sBase, int N, int l)
{
    Nodal n;
    n.r = sBase[B_RHO * N + l];
    n.p = sBase[B_P * N + l];
    const float E = sBase[B_E * N + l];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        n.u[c] = sBase[(B_U0 + c) * N + l];
        n.q[c] = sBase[(B_Q0 + c) * N + l];
    }
    const float k2 = __fmaf_rn(n.u[0], n.u[0], __fmaf_rn(n.u[1], n.u[1], __fmul_rn(n.u[2], n.u[2])));
    n.H = __fmaf_rn(0.5f, k2, E);
    n.rH = __fmul_rn(n.r, n.H);
    return n;
}

__host__ __device__ constexpr int sym_i(int m) { return m < 3 ? 0 : (m < 5 ? 1 : 2); }
__host__ __device__ constexpr int sym_j(int m) { return m < 3 ? m : (m < 5 ? m - 2 : 2); }

__device__ __forceinline__ float field(int f, const Nodal &n)
{
    if (f == 0) return n.r;
    if (f == 1) return n.p;
    if (f < 5) return n.u[f - 2];
    if (f < 8) return n.q[f - 5];
    if (f < 17) return __fmul_rn(n.q[(f - 8) / 3], n.u[(f - 8) % 3]);
    if (f < 23) return __fmul_rn(n.u[sym_i(f - 17)], n.u[sym_j(f - 17)]);
    if (f == 23) return n.H;
    if (f == 24) return n.rH;
    if (f < 28) return __fmul_rn(n.rH, n.u[f - 25]);
    return __fmul_rn(n.H, n.u[f - 28]);
}

// Lattice point of slot s (s = 0, 1: line g of tile o1; 2, 3: line g of tile
// o2; output point 2t + (s & 1) along direction d); -1 when padded.
template <int Q>
__device__ __forceinline__ int pass_point(int d, int s, int g, int tq, int o1, int o2, bool has1, bool has2)
{
    const int o = s < 2 ? o1 : o2;
    const int pt = 2 * tq + (s & 1);
    const int I = d == 0 ? pt : g;
    const int J = d == 0 ? g : (d == 1 ? pt : o);
    const int K = d == 2 ? pt : o;
    const bool live = (s < 2 ? has1 : has2) && g < Q && pt < Q;
    return live ? (K * Q + J) * Q + I : -1;
}

// Per-point coefficients of one direction pass.
struct PointCoef {
    float rho, H, u[3], h[3], cu, cq;
};

// Adds field f's iso-derivative dv (this pass's direction) to the point's
// accumulators: the rules of the FP32 kernel, field by field.
__device__ __forceinline__ void apply_field(int f, float dv, const PointCoef &c, float (&acc)[NACC])
{
    const float h4 = 0.25f;
    if (f == 0) {
        const float t = c.cu * dv;
        acc[A_M] = fmaf(0.5f, t, acc[A_M]);
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[A_MOM0 + i] = fmaf(h4 * c.u[i], t, acc[A_MOM0 + i]);
        acc[A_E] = fmaf(h4 * c.H, t, acc[A_E]);
    } else if (f == 1) {
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[A_MOM0 + i] = fmaf(c.h[i], dv, acc[A_MOM0 + i]);
    } else if (f < 5) {
        acc[A_DIVU] = fmaf(c.h[f - 2], dv, acc[A_DIVU]);
        acc[A_MOM0 + f - 2] = fmaf(h4 * c.cq, dv, acc[A_MOM0 + f - 2]);
    } else if (f < 8) {
        acc[A_DIVQ] = fmaf(c.h[f - 5], dv, acc[A_DIVQ]);
        acc[A_MOM0 + f - 5] = fmaf(h4 * c.cu, dv, acc[A_MOM0 + f - 5]);
    } else if (f < 17) {
        const int i = (f - 8) / 3, j = (f - 8) % 3;
        acc[A_MOM0 + i] = fmaf(h4 * c.h[j], dv, acc[A_MOM0 + i]);
    } else if (f < 23) {
        const int i = sym_i(f - 17), j = sym_j(f - 17);
        const float rd = h4 * c.rho * dv;
        acc[A_MOM0 + i] = fmaf(c.h[j], rd, acc[A_MOM0 + i]);
        if (i != j) acc[A_MOM0 + j] = fmaf(c.h[i], rd, acc[A_MOM0 + j]);
    } else if (f == 23) {
        acc[A_E] = fmaf(h4 * c.cq, dv, acc[A_E]);
    } else if (f == 24) {
        acc[A_E] = fmaf(h4 * c.cu, dv, acc[A_E]);
    } else if (f < 28) {
        acc[A_E] = fmaf(h4 * c.h[f - 25], dv, acc[A_E]);
    } else {
        acc[A_E] = fmaf(h4 * c.rho * c.h[f - 28], dv, acc[A_E]);
    }
}

template <int P, bool BF16>
struct MixedGeom {
    static constexpr int Q = P + 1, N = Q * Q * Q, W = (Q + 1) / 2;
    static constexpr int NTASK = Q * Q * W;  // task: points (2w, 2w+1) of one i-row
    static constexpr int TPT = (NTASK + kThreads - 1) / kThreads;
    static constexpr int BITS = BF16 ? 8 : 11;
    static constexpr int PB = plane_bytes<Q>();  // bytes of one field half
    static constexpr size_t half_bytes = (size_t)2 * kNF * PB + plane_guard_bytes<Q>();
    static constexpr size_t smem = half_bytes + (size_t)(NBASE + NACC) * N * sizeof(float) +
                                   (size_t)2 * N * sizeof(int) + 2 * 32 * sizeof(float);
};

template <int P, bool BF16>
__global__ void __launch_bounds__(kThreads)
    convec_mixed_kernel(int nelem, int npoin, const int *__restrict__ connec, const float *__restrict__ He,
                        const float *__restrict__ gpvol, const TableScratch *__restrict__ tabs,
                        const float *__restrict__ u, const float *__restrict__ q, const float *__restrict__ rho,
                        const float *__restrict__ pr, const float *__restrict__ E, double *__restrict__ Rmass,
                        double *__restrict__ Rmom, double *__restrict__ Rener)
{
    using G = MixedGeom<P, BF16>;
    constexpr int Q = G::Q, N = G::N, W = G::W, NTASK = G::NTASK, TPT = G::TPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *sHalf = smem_raw;                                  // [2*kNF][G::PB]: hi, lo of each field
    float *sBase = reinterpret_cast<float *>(sHalf + G::half_bytes);  // [NBASE][N], lattice (K*Q+J)*Q+I
    float *sAcc = sBase + NBASE * N;                                   // [NACC][N]
    int *sNode = reinterpret_cast<int *>(sAcc + NACC * N);             // [N]
    int *sPerm = sNode + N;                                            // lattice -> gmsh node
    float *sScale = reinterpret_cast<float *>(sPerm + N);             // [32] s_f
    float *sInv = sScale + 32;                                         // [32] 1 / s_f (max bits first)
    unsigned *sMax = reinterpret_cast<unsigned *>(sInv);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Once per block: tables, the zero padding of the half planes (rows and
    // points beyond Q are never written), the B fragments.
    for (int i = tid; i < N; i += kThreads) sPerm[i] = tabs->perm[i];
    if (Q < 8) {
        uint4 *z = reinterpret_cast<uint4 *>(sHalf);
        for (int i = tid; i < (int)(G::half_bytes / 16); i += kThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    // B fragments per direction: col lane/4 (output point), rows 2t, 2t+1 (input point).
    unsigned Bh[3], Bl[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int r = lane >> 2, c0 = 2 * (lane & 3), c1 = c0 + 1;
        const float d0 = (r < Q && c0 < Q) ? tabs->Df[(d * Q + r) * Q + c0] : 0.0f;
        const float d1 = (r < Q && c1 < Q) ? tabs->Df[(d * Q + r) * Q + c1] : 0.0f;
        split_pair<BF16>(d0, d1, Bh[d], Bl[d]);
    }
    const size_t np = (size_t)npoin;
#pragma unroll 1
    for (int e = blockIdx.x; e < nelem; e += gridDim.x) {
    if (MIXED_PREFETCH != 0 && tid == 0) {  // He and gpvol spans into L2, an element ahead
        if (e == (int)blockIdx.x) prefetch_element_l2(He, gpvol, e, N);
        if (e + (int)gridDim.x < nelem) prefetch_element_l2(He, gpvol, e + gridDim.x, N);
    }
    __syncthreads();  // the previous element's passes are done with every shared array
    if (tid < 32) sMax[tid] = 0u;
    for (int l = tid; l < N; l += kThreads) {
        const int a = sPerm[l];
        const int v = ldg(connec + (size_t)a * nelem + e) - 1;
        const bool ok = (unsigned)v < (unsigned)npoin;
        const int p = ok ? v : 0;
        sNode[l] = ok ? v : -1;
        // asynchronous copies (a missing node reads as zeros)
        cp_async_elem(sBase + B_RHO * N + l, rho + p, ok);
        cp_async_elem(sBase + B_P * N + l, pr + p, ok);
        cp_async_elem(sBase + B_E * N + l, E + p, ok);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cp_async_elem(sBase + (B_U0 + c) * N + l, u + c * np + p, ok);
            cp_async_elem(sBase + (B_Q0 + c) * N + l, q + c * np + p, ok);
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();

    // He columns of the first direction pass, in flight during the split.
    const int g = lane >> 2, tq = lane & 3;
    const int o1 = warp, o2 = warp + 4 < Q ? warp + 4 : warp;
    const bool has1 = o1 < Q, has2 = warp + 4 < Q;
    float hcur[4][3];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int l = pass_point<Q>(0, s, g, tq, o1, o2, has1, has2);
        const float *hp = He + ((size_t)e * N + sPerm[l < 0 ? 0 : l]) * 9;
#pragma unroll
        for (int c = 0; c < 3; ++c) hcur[s][c] = ldg(hp + c);
    }

    // Shifted products of the thread's tasks (two points each) in registers,
    // their per-field maxima over the element (non-negative floats order like
    // their bit patterns), then the split into the half planes.
    const Nodal nref = nodal_from(sBase, N, 0);
    float v[TPT][kNF][2];
    {
        float mx[kNF];
#pragma unroll
        for (int f = 0; f < kNF; ++f) mx[f] = 0.0f;
#pragma unroll
        for (int tk = 0; tk < TPT; ++tk) {
            const int t = tid + tk * kThreads;
            const bool valid = t < NTASK;
            const int row = valid ? t / W : 0, w = valid ? t - row * W : 0;
            const int l0 = row * Q + 2 * w;
            const bool two = valid && 2 * w + 1 < Q;
            const Nodal n0 = nodal_from(sBase, N, l0);
            const Nodal n1 = nodal_from(sBase, N, two ? l0 + 1 : l0);
#pragma unroll
            for (int f = 0; f < kNF; ++f) {
                const float fr = field(f, nref);
                const float a = valid ? __fsub_rn(field(f, n0), fr) : 0.0f;
                const float b = two ? __fsub_rn(field(f, n1), fr) : 0.0f;
                v[tk][f][0] = a;
                v[tk][f][1] = b;
                mx[f] = fmaxf(mx[f], fmaxf(fabsf(a), fabsf(b)));
            }
        }
#pragma unroll
        for (int f = 0; f < kNF; ++f) {
            const unsigned mb = __reduce_max_sync(0xffffffffu, __float_as_uint(mx[f]));
            if (lane == 0) atomicMax(&sMax[f], mb);
        }
    }
    __syncthreads();
    if (tid < kNF) {
        // s_f = 2^(B-1-ex) for a maximum in [2^ex, 2^(ex+1)); ex clamped so s_f and 1/s_f are normal.
        int ex = (int)((sMax[tid] >> 23) & 0xFF) - 127;
        ex = min(max(ex, -100), 127);
        sScale[tid] = __int_as_float((127 + G::BITS - 1 - ex) << 23);
        sInv[tid] = __int_as_float((127 + ex - (G::BITS - 1)) << 23);
    }
    __syncthreads();
#pragma unroll
    for (int tk = 0; tk < TPT; ++tk) {
        const int t = tid + tk * kThreads;
        if (t >= NTASK) break;
        const int row = t / W, w = t - row * W;
        const int rk = row / Q, rj = row - rk * Q;
        const int off = row_pos(rk, rj) * kRowB + 4 * w;
#pragma unroll
        for (int f = 0; f < kNF; ++f) {
            const float s = sScale[f];
            const float a = __fmul_rn(v[tk][f][0], s), b = __fmul_rn(v[tk][f][1], s);
            const float M = 12582912.0f;  // 1.5 * 2^23: adding and subtracting it rounds to an integer
            const float ha = __fsub_rn(__fadd_rn(a, M), M), hb = __fsub_rn(__fadd_rn(b, M), M);
            *reinterpret_cast<unsigned *>(sHalf + (2 * f) * G::PB + off) = pack2<BF16>(ha, hb);
            *reinterpret_cast<unsigned *>(sHalf + (2 * f + 1) * G::PB + off) =
                pack2<BF16>(__fsub_rn(a, ha), __fsub_rn(b, hb));
        }
    }
    __syncthreads();

    // Warp w takes the 16 lines of tiles o1 = w and o2 = w + 4 (k-planes for
    // xi / eta lines, j-planes for zeta lines); ldmatrix matrix m of the A
    // operand is (hi o1, hi o2, lo o1, lo o2), row r8.
    const int m = lane >> 3, r8 = lane & 7;
    const int om = (m & 1) ? o2 : o1;
    const int plane_off = (m >> 1) * G::PB;
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        const unsigned bh = d == 0 ? Bh[0] : (d == 1 ? Bh[1] : Bh[2]);
        const unsigned bl = d == 0 ? Bl[0] : (d == 1 ? Bl[1] : Bl[2]);
        // The thread's points: s = 0, 1 line g of tile o1, s = 2, 3 line g of
        // tile o2; output points 2t and 2t+1 along the direction.
        int lat[4];
        bool live[4];
        PointCoef cf[4];
        float acc[4][NACC], gp[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const int lp = pass_point<Q>(d, s, g, tq, o1, o2, has1, has2);
            live[s] = lp >= 0;
            const int l = live[s] ? lp : 0;
            lat[s] = l;
            const Nodal n = nodal_from(sBase, N, l);
            cf[s].rho = n.r;
            cf[s].H = n.H;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                cf[s].u[c] = n.u[c];
                cf[s].h[c] = hcur[s][c];
            }
            cf[s].cu = n.u[0] * cf[s].h[0] + n.u[1] * cf[s].h[1] + n.u[2] * cf[s].h[2];
            cf[s].cq = n.q[0] * cf[s].h[0] + n.q[1] * cf[s].h[1] + n.q[2] * cf[s].h[2];
#pragma unroll
            for (int k = 0; k < NACC; ++k) acc[s][k] = (d == 0 || !live[s]) ? 0.0f : sAcc[k * N + l];
        }
        // Loads in flight during the contractions: the next pass's He columns,
        // or gpvol for the last pass's scatter.
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            if (d < 2) {
                const int l = pass_point<Q>(d + 1, s, g, tq, o1, o2, has1, has2);
                const float *hp = He + ((size_t)e * N + sPerm[l < 0 ? 0 : l]) * 9 + (d + 1) * 3;
#pragma unroll
                for (int c = 0; c < 3; ++c) hcur[s][c] = ldg(hp + c);
                gp[s] = 0.0f;
            } else {
                gp[s] = ldg(gpvol + (size_t)e * N + sPerm[lat[s]]);
            }
        }
        const unsigned char *rowp =
            sHalf + plane_off + (d == 2 ? row_pos(r8, om) : row_pos(om, r8)) * kRowB;
#pragma unroll
        for (int f = 0; f < kNF; ++f) {
            unsigned a[4];
            if (d == 0)
                ldsm_x4(a, rowp + 2 * f * G::PB);
            else
                ldsm_x4_t(a, rowp + 2 * f * G::PB);
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma_acc<BF16>(c, a, bh, bh);
            mma_acc<BF16>(c, a, bl, 0u);
            const float inv = sInv[f];
#pragma unroll
            for (int s = 0; s < 4; ++s) apply_field(f, c[s] * inv, cf[s], acc[s]);
        }
        if (d < 2) {
#pragma unroll
            for (int s = 0; s < 4; ++s)
                if (live[s])
#pragma unroll
                    for (int k = 0; k < NACC; ++k) sAcc[k * N + lat[s]] = acc[s][k];
            __syncthreads();
        } else {
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                if (!live[s]) continue;
                const int node = sNode[lat[s]];
                if (node < 0) continue;
                const Nodal n = nodal_from(sBase, N, lat[s]);
                const float divU = acc[s][A_DIVU], divQ = acc[s][A_DIVQ];
                const float rm = acc[s][A_M] + 0.5f * (divQ + n.r * divU);
                red_add(Rmass + node, f2d(gp[s] * rm));
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const float rmom = acc[s][A_MOM0 + i] + 0.25f * (n.u[i] * divQ + n.q[i] * divU);
                    red_add(Rmom + (size_t)i * npoin + node, f2d(gp[s] * rmom));
                }
                // energy-flux assembly in FP64
                const double t = fma(f2d(n.H), f2d(divQ), f2d(n.rH) * f2d(divU));
                red_add(Rener + node, f2d(gp[s]) * fma(0.25, t, f2d(acc[s][A_E])));
            }
        }
    }
    }  // elements
}

template <int P, bool BF16>
cudaError_t launch_mixed_pb(const MixedConvecArgs &a, const TableScratch *tabs, cudaStream_t st)
{
    using G = MixedGeom<P, BF16>;
    static_assert(G::smem <= 227 * 1024, "shared memory budget");
    auto kern = convec_mixed_kernel<P, BF16>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::smem);
    if (err != cudaSuccess) return err;
    if (a.nelem == 0) return cudaSuccess;
    const int grid = persistent_grid(kern, kThreads, G::smem, a.nelem);
    if (grid < 1) return cudaErrorInvalidConfiguration;
    kern<<<grid, kThreads, G::smem, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, tabs, a.u, a.q, a.rho,
                                             a.pr, a.E, a.Rmass, a.Rmom, a.Rener);
    return cudaGetLastError();
}

template <int P>
cudaError_t launch_mixed_p(const MixedConvecArgs &a, int precision, const TableScratch *tabs, cudaStream_t st)
{
    return precision == MSOD_PREC_BF16 ? launch_mixed_pb<P, true>(a, tabs, st) : launch_mixed_pb<P, false>(a, tabs, st);
}

}  // namespace

cudaError_t launch_convec_mixed(int porder, int precision, const MixedConvecArgs &a, const TableScratch *tabs,
                                cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_mixed_p<1>(a, precision, tabs, st);
    case 2: return launch_mixed_p<2>(a, precision, tabs, st);
    case 3: return launch_mixed_p<3>(a, precision, tabs, st);
    case 4: return launch_mixed_p<4>(a, precision, tabs, st);
    case 5: return launch_mixed_p<5>(a, precision, tabs, st);
    case 6: return launch_mixed_p<6>(a, precision, tabs, st);
    case 7: return launch_mixed_p<7>(a, precision, tabs, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace msod
