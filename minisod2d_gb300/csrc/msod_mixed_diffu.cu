// msod_mixed_diffu.cu -- mixed-precision hex GLL diffusion residual on the tensor cores.
//
// Same residuals as full_diffusion_ijk (elem_diffu.f90:10-197; formulas in
// msod_diffu.cu) from FP32 fields, with the 1-D contractions on the tensor
// cores as FP16 (or BF16) hi + lo split products (FP32 accumulation) and the
// energy-flux assembly and the nodal scatter-add in FP64 (FP64 outputs).
//
// Per element (one block of four warps, persistent over elements):
//   1. gather rho, T, u, mu_fluid, mu_e, mu_sgs into a lattice in shared memory;
//   2. gradient stage: rho, T, u_1..3 are shifted by their value at lattice
//      node (0,0,0) (the derivative annihilates constants), scaled by a power
//      of two per element and field, split into hi + lo half planes; per
//      direction, two accumulating mma.sync.m16n8k16 per field and 16 lines
//      (A = [f_hi | f_lo], B = [D_hi^T ; D_hi^T] then [D_lo^T ; 0]) give the
//      15 iso-parametric derivatives per point;
//   3. point pass: physical gradients, stress tau, tau.u and the contravariant
//      fluxes gpvol He(:,d)^T X of X = grad rho, tau.u, grad T, tau rows
//      (18 per point), plus nu_e and kappa_e per output node
//      (elem_diffu.f90:143-146); each flux is shifted by its value X_ref at
//      lattice node (0,0,0), scaled per element and flux, and split into half
//      planes;
//   4. weak divergence: per direction, the transposed 1-D operator
//      (B = [D_hi ; D_hi] then [D_lo ; 0], indexed (input, output)) on the six
//      shifted fluxes of that direction, plus X_ref times the operator's
//      column sum (evaluated in FP64 once per block); six sums per point
//      accumulated over the directions in shared memory;
//   5. Rmass += nu_e sum(grad rho), Rmom_m += sum(tau_m), and in FP64
//      Rener += sum(tau.u) + kappa_e sum(grad T); red.global.add.f64.
// Shared-memory half planes use the swizzled layout of msod_mma.cuh.
// porder 1..7.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"
#include "msod_mma.cuh"

namespace msod {
namespace {

constexpr int kThreads = 128;
constexpr int kNG = 5;   // differentiated node fields: rho, T, u_1..3
constexpr int kNX = 6;   // flux vectors: grad rho, tau.u, grad T, tau rows 1..3
constexpr int kNFX = 3 * kNX;

enum { S_RHO = 0, S_T, S_U0, S_U1, S_U2, S_MUF, S_MUE, S_MUS, NSB };  // gathered planes
enum { X_GRHO = 0, X_TAUU, X_GT, X_TAU0, X_TAU1, X_TAU2 };

template <int P, bool BF16>
struct MixedDiffuGeom {
    static constexpr int Q = P + 1, N = Q * Q * Q, W = (Q + 1) / 2;
    static constexpr int NTASK = Q * Q * W;  // task: points (2w, 2w+1) of one i-row
    static constexpr int TPT = (NTASK + kThreads - 1) / kThreads;
    static constexpr int BITS = BF16 ? 8 : 11;
    static constexpr int PB = plane_bytes<Q>();  // bytes of one field half
    static constexpr size_t half_bytes = (size_t)2 * kNFX * PB + plane_guard_bytes<Q>();
    static constexpr size_t smem = half_bytes + (size_t)(NSB + 3 * kNG + 2) * N * sizeof(float) +
                                   (size_t)2 * N * sizeof(int) + 3 * 32 * sizeof(float);
};

// Lattice point of slot s of a pass (see msod_mixed.cu); -1 when padded.
template <int Q>
__device__ __forceinline__ int dpass_point(int d, int s, int g, int tq, int o1, int o2, bool has1, bool has2)
{
    const int o = s < 2 ? o1 : o2;
    const int pt = 2 * tq + (s & 1);
    const int I = d == 0 ? pt : g;
    const int J = d == 0 ? g : (d == 1 ? pt : o);
    const int K = d == 2 ? pt : o;
    const bool live = (s < 2 ? has1 : has2) && g < Q && pt < Q;
    return live ? (K * Q + J) * Q + I : -1;
}

template <int P, bool BF16, bool NUE>
__global__ void __launch_bounds__(kThreads)
    diffu_mixed_kernel(int nelem, int npoin, const int *__restrict__ connec, const float *__restrict__ He,
                       const float *__restrict__ gpvol, const TableScratch *__restrict__ tabs, float Cp, float Pr,
                       const float *__restrict__ rho, const float *__restrict__ u, const float *__restrict__ Tem,
                       const float *__restrict__ mu_fluid, const float *__restrict__ mu_e,
                       const float *__restrict__ mu_sgs, const float *__restrict__ nu_elem,
                       double *__restrict__ Rmass, double *__restrict__ Rmom, double *__restrict__ Rener)
{
    using G = MixedDiffuGeom<P, BF16>;
    constexpr int Q = G::Q, N = G::N, W = G::W, NTASK = G::NTASK, TPT = G::TPT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char *sHalf = smem_raw;                                  // [2*kNFX][G::PB]
    float *sB = reinterpret_cast<float *>(sHalf + G::half_bytes);     // [NSB][N] lattice (K*Q+J)*Q+I
    float *sG = sB + NSB * N;                                          // [15][N] iso-derivatives; then [6][N] sums
    float *sNK = sG + 3 * kNG * N;                                     // [2][N] nu_e, kappa_e
    int *sNode = reinterpret_cast<int *>(sNK + 2 * N);                 // [N]
    int *sPerm = sNode + N;                                            // lattice -> gmsh node
    float *sScale = reinterpret_cast<float *>(sPerm + N);             // [32]: 0..4 gradient fields, 5..22 fluxes
    float *sInv = sScale + 32;
    unsigned *sMax = reinterpret_cast<unsigned *>(sInv);
    float *sRef = sInv + 32;  // [kNFX] flux values at lattice node (0,0,0)

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, tq = lane & 3;
    for (int i = tid; i < N; i += kThreads) sPerm[i] = tabs->perm[i];
    if (Q < 8) {  // rows and points beyond Q are never written and stay zero
        uint4 *z = reinterpret_cast<uint4 *>(sHalf);
        for (int i = tid; i < (int)(G::half_bytes / 16); i += kThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    // B fragments per direction.  Gradient: B[k][n] = D[n][k]; divergence:
    // B[k][n] = D[k][n] (k input point, n output point); hi and lo halves.
    unsigned Bgh[3], Bgl[3], Bdh[3], Bdl[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int c0 = 2 * tq, c1 = c0 + 1;
        const float *D = tabs->Df + d * Q * Q;
        split_pair<BF16>((g < Q && c0 < Q) ? D[g * Q + c0] : 0.0f, (g < Q && c1 < Q) ? D[g * Q + c1] : 0.0f,
                         Bgh[d], Bgl[d]);
        split_pair<BF16>((g < Q && c0 < Q) ? D[c0 * Q + g] : 0.0f, (g < Q && c1 < Q) ? D[c1 * Q + g] : 0.0f,
                         Bdh[d], Bdl[d]);
    }
    // Column sums of the divergence operator at the thread's output points 2t, 2t+1.
    float colsum[3][2];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int a = 2 * tq + h;
            double cs = 0.0;
            if (a < Q)
                for (int c = 0; c < Q; ++c) cs += (double)tabs->Df[(d * Q + c) * Q + a];
            colsum[d][h] = (float)cs;
        }
    const int o1 = warp, o2 = warp + 4 < Q ? warp + 4 : warp;
    const bool has1 = o1 < Q, has2 = warp + 4 < Q;
    const int m = lane >> 3, r8 = lane & 7;
    const int om = (m & 1) ? o2 : o1;
    const int plane_off = (m >> 1) * G::PB;
    const size_t np = (size_t)npoin;
    const float twoThirds = 2.0f / 3.0f;

#pragma unroll 1
    for (int e = blockIdx.x; e < nelem; e += gridDim.x) {
        if (MIXED_PREFETCH != 0 && tid == 0) {  // He and gpvol spans into L2, an element ahead
            if (e == (int)blockIdx.x) prefetch_element_l2(He, gpvol, e, N);
            if (e + (int)gridDim.x < nelem) prefetch_element_l2(He, gpvol, e + gridDim.x, N);
        }
        __syncthreads();  // the previous element is done with every shared array
        if (tid < 32) sMax[tid] = 0u;
        const float nue = NUE ? ldg(nu_elem + e) : 0.0f;
        for (int l = tid; l < N; l += kThreads) {
            const int a = sPerm[l];
            const int v = ldg(connec + (size_t)a * nelem + e) - 1;
            const bool ok = (unsigned)v < (unsigned)npoin;
            const int p = ok ? v : 0;
            sNode[l] = ok ? v : -1;
            const float r = ok ? ldg(rho + p) : 1.0f;  // 1 at a missing node keeps nu_e = mu_e / rho finite
            sB[S_RHO * N + l] = r;
            // the other fields by asynchronous copies (a missing node reads as zeros)
            cp_async_elem(sB + S_T * N + l, Tem + p, ok);
#pragma unroll
            for (int c = 0; c < 3; ++c) cp_async_elem(sB + (S_U0 + c) * N + l, u + c * np + p, ok);
            cp_async_elem(sB + S_MUF * N + l, mu_fluid + p, ok);
            if (NUE)
                sB[S_MUE * N + l] = r * nue;
            else
                cp_async_elem(sB + S_MUE * N + l, mu_e + (size_t)a * nelem + e, true);
            cp_async_elem(sB + S_MUS * N + l, mu_sgs + (size_t)a * nelem + e, true);
        }
        cp_async_commit();
        // He and gpvol of the point-pass points, in flight during the gradient stage.
        float hv[TPT][2][9], gv[TPT][2];
#pragma unroll
        for (int tk = 0; tk < TPT; ++tk) {
            const int t = tid + tk * kThreads;
            const int row = t < NTASK ? t / W : 0, w = t < NTASK ? t - row * W : 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int l = (t < NTASK && 2 * w + h < Q) ? row * Q + 2 * w + h : 0;
                const size_t base = (size_t)e * N + sPerm[l];
#pragma unroll
                for (int j = 0; j < 9; ++j) hv[tk][h][j] = ldg(He + base * 9 + j);
                gv[tk][h] = ldg(gpvol + base);
            }
        }
        cp_async_wait_all();
        __syncthreads();

        // ---- gradient stage: split rho, T, u_1..3 (shifted by node (0,0,0)) ----
        {
            float ref[kNG];
#pragma unroll
            for (int f = 0; f < kNG; ++f) ref[f] = sB[f * N];  // planes S_RHO..S_U2 are fields 0..4
            float v[TPT][kNG][2], mx[kNG];
#pragma unroll
            for (int f = 0; f < kNG; ++f) mx[f] = 0.0f;
#pragma unroll
            for (int tk = 0; tk < TPT; ++tk) {
                const int t = tid + tk * kThreads;
                const bool valid = t < NTASK;
                const int row = valid ? t / W : 0, w = valid ? t - row * W : 0;
                const int l0 = row * Q + 2 * w;
                const bool two = valid && 2 * w + 1 < Q;
#pragma unroll
                for (int f = 0; f < kNG; ++f) {
                    const float a = valid ? __fsub_rn(sB[f * N + l0], ref[f]) : 0.0f;
                    const float b = two ? __fsub_rn(sB[f * N + l0 + 1], ref[f]) : 0.0f;
                    v[tk][f][0] = a;
                    v[tk][f][1] = b;
                    mx[f] = fmaxf(mx[f], fmaxf(fabsf(a), fabsf(b)));
                }
            }
#pragma unroll
            for (int f = 0; f < kNG; ++f) {
                const unsigned mb = __reduce_max_sync(0xffffffffu, __float_as_uint(mx[f]));
                if (lane == 0) atomicMax(&sMax[f], mb);
            }
            __syncthreads();
            if (tid < kNG) scale_from_max(sMax[tid], G::BITS, sScale[tid], sInv[tid]);
            __syncthreads();
#pragma unroll
            for (int tk = 0; tk < TPT; ++tk) {
                const int t = tid + tk * kThreads;
                if (t >= NTASK) break;
                const int row = t / W, w = t - row * W;
                const int rk = row / Q, rj = row - rk * Q;
                const int off = row_pos(rk, rj) * kRowB + 4 * w;
#pragma unroll
                for (int f = 0; f < kNG; ++f) {
                    const float s = sScale[f];
                    unsigned hi, lo;
                    split_scaled<BF16>(__fmul_rn(v[tk][f][0], s), __fmul_rn(v[tk][f][1], s), hi, lo);
                    *reinterpret_cast<unsigned *>(sHalf + (2 * f) * G::PB + off) = hi;
                    *reinterpret_cast<unsigned *>(sHalf + (2 * f + 1) * G::PB + off) = lo;
                }
            }
        }
        __syncthreads();
#pragma unroll 1
        for (int d = 0; d < 3; ++d) {
            const unsigned bh = d == 0 ? Bgh[0] : (d == 1 ? Bgh[1] : Bgh[2]);
            const unsigned bl = d == 0 ? Bgl[0] : (d == 1 ? Bgl[1] : Bgl[2]);
            const unsigned char *rowp = sHalf + plane_off + (d == 2 ? row_pos(r8, om) : row_pos(om, r8)) * kRowB;
            int lat[4];
#pragma unroll
            for (int s = 0; s < 4; ++s) lat[s] = dpass_point<Q>(d, s, g, tq, o1, o2, has1, has2);
#pragma unroll
            for (int f = 0; f < kNG; ++f) {
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
                for (int s = 0; s < 4; ++s)
                    if (lat[s] >= 0) sG[(d * kNG + f) * N + lat[s]] = c[s] * inv;
            }
        }
        __syncthreads();

        // ---- point pass: stress, fluxes, nu_e, kappa_e; flux maxima ----
        {
            float fl[TPT][2][kNFX];
            float mx[kNFX];
#pragma unroll
            for (int x = 0; x < kNFX; ++x) mx[x] = 0.0f;
#pragma unroll
            for (int tk = 0; tk < TPT; ++tk) {
                const int t = tid + tk * kThreads;
                const int row = t < NTASK ? t / W : 0, w = t < NTASK ? t - row * W : 0;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const bool live = t < NTASK && 2 * w + h < Q;
                    const int l = live ? row * Q + 2 * w + h : 0;
                    float gi[3][kNG];
#pragma unroll
                    for (int d = 0; d < 3; ++d)
#pragma unroll
                        for (int f = 0; f < kNG; ++f) gi[d][f] = sG[(d * kNG + f) * N + l];
                    const float r = sB[S_RHO * N + l];
                    const float uu[3] = {sB[S_U0 * N + l], sB[S_U1 * N + l], sB[S_U2 * N + l]};
                    const float muf = sB[S_MUF * N + l], me = sB[S_MUE * N + l], ms = sB[S_MUS * N + l];
                    const float(&Hm)[9] = hv[tk][h];  // Hm[j*3+i] = He(i, j)
                    float gR[3], gT[3], gU[3][3];
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        gR[i] = Hm[i] * gi[0][0] + Hm[3 + i] * gi[1][0] + Hm[6 + i] * gi[2][0];
                        gT[i] = Hm[i] * gi[0][1] + Hm[3 + i] * gi[1][1] + Hm[6 + i] * gi[2][1];
#pragma unroll
                        for (int j = 0; j < 3; ++j)
                            gU[i][j] = Hm[j] * gi[0][2 + i] + Hm[3 + j] * gi[1][2 + i] + Hm[6 + j] * gi[2][2 + i];
                    }
                    const float mu_fgp = muf + r * ms;
                    const float mu_tot = mu_fgp + me;
                    const float divU = gU[0][0] + gU[1][1] + gU[2][2];
                    float tau[3][3], tauU[3];
#pragma unroll
                    for (int i = 0; i < 3; ++i)
#pragma unroll
                        for (int j = 0; j < 3; ++j) tau[i][j] = mu_tot * (gU[i][j] + gU[j][i]);
#pragma unroll
                    for (int i = 0; i < 3; ++i) tau[i][i] -= mu_fgp * twoThirds * divU;
#pragma unroll
                    for (int i = 0; i < 3; ++i) tauU[i] = tau[i][0] * uu[0] + tau[i][1] * uu[1] + tau[i][2] * uu[2];
                    const float *Xv[kNX] = {gR, tauU, gT, tau[0], tau[1], tau[2]};
#pragma unroll
                    for (int d = 0; d < 3; ++d)
#pragma unroll
                        for (int x = 0; x < kNX; ++x) {
                            const float val =
                                live ? gv[tk][h] * (Hm[d * 3] * Xv[x][0] + Hm[d * 3 + 1] * Xv[x][1] +
                                                    Hm[d * 3 + 2] * Xv[x][2])
                                     : 0.0f;
                            fl[tk][h][d * kNX + x] = val;
                        }
                    if (live) {
                        sNK[l] = me / r;
                        sNK[N + l] = muf * Cp / Pr + me * Cp / Pr + Cp * r * ms / 0.9f;
                    }
                }
            }
            if (tid == 0)  // task 0, first point: lattice node (0,0,0)
#pragma unroll
                for (int x = 0; x < kNFX; ++x) sRef[x] = fl[0][0][x];
            __syncthreads();
#pragma unroll
            for (int tk = 0; tk < TPT; ++tk) {
                const int t = tid + tk * kThreads;
                const int w = t < NTASK ? t % W : 0;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const bool live = t < NTASK && 2 * w + h < Q;
#pragma unroll
                    for (int x = 0; x < kNFX; ++x) {
                        fl[tk][h][x] = live ? __fsub_rn(fl[tk][h][x], sRef[x]) : 0.0f;
                        mx[x] = fmaxf(mx[x], fabsf(fl[tk][h][x]));
                    }
                }
            }
#pragma unroll
            for (int x = 0; x < kNFX; ++x) {
                const unsigned mb = __reduce_max_sync(0xffffffffu, __float_as_uint(mx[x]));
                if (lane == 0) atomicMax(&sMax[kNG + x], mb);
            }
            __syncthreads();
            if (tid >= kNG && tid < kNG + kNFX) scale_from_max(sMax[tid], G::BITS, sScale[tid], sInv[tid]);
            __syncthreads();
#pragma unroll
            for (int tk = 0; tk < TPT; ++tk) {
                const int t = tid + tk * kThreads;
                if (t >= NTASK) break;
                const int row = t / W, w = t - row * W;
                const int rk = row / Q, rj = row - rk * Q;
                const int off = row_pos(rk, rj) * kRowB + 4 * w;
#pragma unroll
                for (int x = 0; x < kNFX; ++x) {
                    const float s = sScale[kNG + x];
                    unsigned hi, lo;
                    split_scaled<BF16>(__fmul_rn(fl[tk][0][x], s), __fmul_rn(fl[tk][1][x], s), hi, lo);
                    *reinterpret_cast<unsigned *>(sHalf + (2 * x) * G::PB + off) = hi;
                    *reinterpret_cast<unsigned *>(sHalf + (2 * x + 1) * G::PB + off) = lo;
                }
            }
        }
        __syncthreads();

        // ---- weak divergence: six sums per point over the three directions ----
        float *sAcc = sG;  // the iso-derivatives are consumed
#pragma unroll 1
        for (int d = 0; d < 3; ++d) {
            const unsigned bh = d == 0 ? Bdh[0] : (d == 1 ? Bdh[1] : Bdh[2]);
            const unsigned bl = d == 0 ? Bdl[0] : (d == 1 ? Bdl[1] : Bdl[2]);
            const unsigned char *rowp = sHalf + plane_off + (d == 2 ? row_pos(r8, om) : row_pos(om, r8)) * kRowB;
            int lat[4];
            float acc[4][kNX];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                lat[s] = dpass_point<Q>(d, s, g, tq, o1, o2, has1, has2);
#pragma unroll
                for (int x = 0; x < kNX; ++x) acc[s][x] = (d == 0 || lat[s] < 0) ? 0.0f : sAcc[x * N + lat[s]];
            }
#pragma unroll
            for (int x = 0; x < kNX; ++x) {
                const int fx = d * kNX + x;
                unsigned a[4];
                if (d == 0)
                    ldsm_x4(a, rowp + 2 * fx * G::PB);
                else
                    ldsm_x4_t(a, rowp + 2 * fx * G::PB);
                float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                mma_acc<BF16>(c, a, bh, bh);
                mma_acc<BF16>(c, a, bl, 0u);
                const float inv = sInv[kNG + fx], ref = sRef[fx];
                const float cs0 = d == 0 ? colsum[0][0] : (d == 1 ? colsum[1][0] : colsum[2][0]);
                const float cs1 = d == 0 ? colsum[0][1] : (d == 1 ? colsum[1][1] : colsum[2][1]);
#pragma unroll
                for (int s = 0; s < 4; ++s) acc[s][x] = fmaf(c[s], inv, fmaf(ref, (s & 1) ? cs1 : cs0, acc[s][x]));
            }
            if (d < 2) {
#pragma unroll
                for (int s = 0; s < 4; ++s)
                    if (lat[s] >= 0)
#pragma unroll
                        for (int x = 0; x < kNX; ++x) sAcc[x * N + lat[s]] = acc[s][x];
                __syncthreads();
            } else {
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    if (lat[s] < 0) continue;
                    const int node = sNode[lat[s]];
                    if (node < 0) continue;
                    red_add(Rmass + node, f2d(sNK[lat[s]] * acc[s][X_GRHO]));
#pragma unroll
                    for (int i = 0; i < 3; ++i) red_add(Rmom + (size_t)i * npoin + node, f2d(acc[s][X_TAU0 + i]));
                    // energy-flux assembly in FP64
                    red_add(Rener + node, fma(f2d(sNK[N + lat[s]]), f2d(acc[s][X_GT]), f2d(acc[s][X_TAUU])));
                }
            }
        }
    }  // elements
}

template <int P, bool BF16, bool NUE>
cudaError_t launch_pbn(const MixedDiffuArgs &a, const TableScratch *tabs, cudaStream_t st)
{
    using G = MixedDiffuGeom<P, BF16>;
    static_assert(G::smem <= 227 * 1024, "shared memory budget");
    auto kern = diffu_mixed_kernel<P, BF16, NUE>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::smem);
    if (err != cudaSuccess) return err;
    if (a.nelem == 0) return cudaSuccess;
    const int grid = persistent_grid(kern, kThreads, G::smem, a.nelem);
    if (grid < 1) return cudaErrorInvalidConfiguration;
    kern<<<grid, kThreads, G::smem, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, tabs, a.Cp, a.Pr, a.rho, a.u,
                                          a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs, a.nu_elem, a.Rmass, a.Rmom, a.Rener);
    return cudaGetLastError();
}

template <int P>
cudaError_t launch_p(const MixedDiffuArgs &a, int precision, const TableScratch *tabs, cudaStream_t st)
{
    const bool bf = precision == MSOD_PREC_BF16, nue = a.nu_elem != nullptr;
    if (bf) return nue ? launch_pbn<P, true, true>(a, tabs, st) : launch_pbn<P, true, false>(a, tabs, st);
    return nue ? launch_pbn<P, false, true>(a, tabs, st) : launch_pbn<P, false, false>(a, tabs, st);
}

}  // namespace

cudaError_t launch_diffu_mixed(int porder, int precision, const MixedDiffuArgs &a, const TableScratch *tabs,
                               cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_p<1>(a, precision, tabs, st);
    case 2: return launch_p<2>(a, precision, tabs, st);
    case 3: return launch_p<3>(a, precision, tabs, st);
    case 4: return launch_p<4>(a, precision, tabs, st);
    case 5: return launch_p<5>(a, precision, tabs, st);
    case 6: return launch_p<6>(a, precision, tabs, st);
    case 7: return launch_p<7>(a, precision, tabs, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace msod
