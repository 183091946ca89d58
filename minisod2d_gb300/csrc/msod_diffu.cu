// msod_diffu.cu -- plain (FP32 / FP64) hex GLL diffusion residual.
//
// Computes what full_diffusion_ijk computes (elem_diffu.f90:10-197):
//   pass 1 (per point b): grad rho, grad T, grad u; mu_f = mu_fluid + rho mu_sgs;
//     tau = (mu_f + mu_e)(grad u + grad u^T) - 2/3 mu_f div u I;  tauU = tau u
//   pass 2 (per output node a):
//     Rmass += nu_e(a)   sum_{d,b} w_d(a,b) . grad rho(b)
//     Rener +=           sum_{d,b} w_d(a,b) . (tauU(b) + kappa_e(a) grad T(b))
//     Rmom_m +=          sum_{d,b} w_d(a,b) . tau_m(b)
//   with w_d(a,b)_i = He(i,d,b) gpvol(b) dlxigp_ip(b,d,iso_d(a)) over the
//   points b of a's d-line, nu_e(a) = mu_e/rho and
//   kappa_e(a) = mu_fluid Cp/Pr + mu_e Cp/Pr + Cp rho mu_sgs / 0.9 evaluated at
//   the output node (elem_diffu.f90:143-146).
//
// Design (one group of NE elements per block, one thread per GLL line):
//   1. gather rho, T, u, mu_fluid (nodes) and mu_e, mu_sgs (element layout)
//      into a shared-memory lattice;
//   2. three line passes store the 15 iso-parametric derivatives per point;
//   3. a point pass turns them into physical gradients and stress and stores,
//      per direction d, the contravariant fluxes gpvol * He(:,d)^T X for the
//      six vectors X = grad rho, tauU, grad T, tau rows 1..3 (18 per point),
//      plus nu_e and kappa_e per output node;
//   4. three line passes apply the transposed 1-D derivative matrix along the
//      lines (the weak divergence), accumulating five sums per node through
//      shared memory; the last pass scatter-adds with red.global.add.
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

namespace msod {
namespace {

enum { D_RHO = 0, D_T, D_U0, D_U1, D_U2, D_MUF, D_MUE, D_MUS, NDF };  // gathered planes
enum { X_GRHO = 0, X_TAUU, X_GT, X_TAU0, X_TAU1, X_TAU2, NX };        // flux vectors
// After the point pass the gathered planes hold: 0 nu_e, 1 kappa_e, 2..6 partial sums.
enum { P_NUE = 0, P_KAP = 1, P_DR = 2, P_DE = 3, P_DM0 = 4 };

template <int DIR, int Q, int QP>
__device__ __forceinline__ int line_off(int la, int lb, int r)
{
    return DIR == 0 ? (lb * Q + la) * QP + r : (DIR == 1 ? (lb * Q + r) * QP + la : (r * Q + lb) * QP + la);
}

// Pass 1, direction DIR: iso-parametric derivatives of rho, T, u0..2 at the
// thread's points, stored to planes sX[DIR*5 + f].
template <typename real, int P, int DIR>
__device__ __forceinline__ void diffu_grad_pass(const real *__restrict__ sF, real *__restrict__ sX,
                                                const real *__restrict__ sD)
{
    using G = LineGeom<real, P>;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, NE = G::NE, S = G::S, R = G::R, TPE = G::TPE;
    constexpr int NPL = NE * ES;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int tid = threadIdx.x;
    if (tid >= NE * TPE) return;
    const int el = tid / TPE, rem = tid - el * TPE;
    const int line = S == 1 ? rem : rem / S;
    const int seg = S == 1 ? 0 : rem - line * S;
    const int la = line % Q, lb = line / Q;
    const int base = el * ES + line_off<DIR, Q, QP>(la, lb, 0);
    const int r0 = seg * R;
    real Dm[R][Q];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int rc = ((R * S == Q) || r0 + rr < Q) ? r0 + rr : 0;
#pragma unroll
        for (int c = 0; c < Q; ++c) Dm[rr][c] = sD[(DIR * Q + rc) * Q + c];
    }
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        real v[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) v[c] = sF[f * NPL + base + c * OST];
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            const int r = r0 + rr;
            if (!((R * S == Q) || r < Q)) continue;
            real s = (real)0;
#pragma unroll
            for (int c = 0; c < Q; ++c) s = fma(Dm[rr][c], v[c], s);
            sX[(DIR * 5 + f) * NPL + base + r * OST] = s;
        }
    }
}

// Pass 2, direction DIR: weak divergence along the lines with the transposed
// derivative matrix; partial sums through planes P_DR..P_DM0+2 of sF.
template <typename real, int P, int DIR>
__device__ __forceinline__ void diffu_div_pass(real *__restrict__ sF, const real *__restrict__ sX,
                                               const real *__restrict__ sD, const int *__restrict__ sNode,
                                               int e0, int nelem, int npoin, real *__restrict__ Rmass,
                                               real *__restrict__ Rmom, real *__restrict__ Rener)
{
    using G = LineGeom<real, P>;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, NE = G::NE, S = G::S, R = G::R, TPE = G::TPE;
    constexpr int NPL = NE * ES;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int tid = threadIdx.x;
    if (tid >= NE * TPE) return;
    const int el = tid / TPE, rem = tid - el * TPE;
    const int line = S == 1 ? rem : rem / S;
    const int seg = S == 1 ? 0 : rem - line * S;
    const int la = line % Q, lb = line / Q;
    const int base = el * ES + line_off<DIR, Q, QP>(la, lb, 0);
    const int r0 = seg * R;
    const int e = e0 + el;
    real Dt[R][Q], acc[R][5], kap[R];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int rc = ((R * S == Q) || r0 + rr < Q) ? r0 + rr : 0;
#pragma unroll
        for (int c = 0; c < Q; ++c) Dt[rr][c] = sD[(DIR * Q + c) * Q + rc];
        const int o = base + rc * OST;
        kap[rr] = sF[P_KAP * NPL + o];
#pragma unroll
        for (int k = 0; k < 5; ++k) acc[rr][k] = DIR == 0 ? (real)0 : sF[(P_DR + k) * NPL + o];
    }
#pragma unroll
    for (int x = 0; x < NX; ++x) {
        real v[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) v[c] = sX[(DIR * NX + x) * NPL + base + c * OST];
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            real s = (real)0;
#pragma unroll
            for (int c = 0; c < Q; ++c) s = fma(Dt[rr][c], v[c], s);
            if (x == X_GRHO) acc[rr][0] += s;
            else if (x == X_TAUU) acc[rr][1] += s;
            else if (x == X_GT) acc[rr][1] = fma(kap[rr], s, acc[rr][1]);
            else acc[rr][2 + (x - X_TAU0)] += s;
        }
    }
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int r = r0 + rr;
        if (!((R * S == Q) || r < Q)) continue;
        const int o = base + r * OST;
        if (DIR < 2) {
#pragma unroll
            for (int k = 0; k < 5; ++k) sF[(P_DR + k) * NPL + o] = acc[rr][k];
        } else {
            const int node = sNode[o];
            if (node < 0 || e >= nelem) continue;
            red_add(Rmass + node, sF[P_NUE * NPL + o] * acc[rr][0]);
            red_add(Rener + node, acc[rr][1]);
#pragma unroll
            for (int m = 0; m < 3; ++m) red_add(Rmom + (size_t)m * npoin + node, acc[rr][2 + m]);
        }
    }
}

template <typename real, int P>
__global__ void __launch_bounds__(LineGeom<real, P>::NT)
    diffu_kernel(int nelem, int npoin, const int *__restrict__ connec, const real *__restrict__ He,
                 const real *__restrict__ gpvol, const real *__restrict__ dlxigp_ip,
                 const int *__restrict__ invAtoIJK, const int *__restrict__ AtoI, const int *__restrict__ AtoJ,
                 const int *__restrict__ AtoK, real Cp, real Pr, const real *__restrict__ rho,
                 const real *__restrict__ u, const real *__restrict__ Tem, const real *__restrict__ mu_fluid,
                 const real *__restrict__ mu_e, const real *__restrict__ mu_sgs, real *__restrict__ Rmass,
                 real *__restrict__ Rmom, real *__restrict__ Rener)
{
    using G = LineGeom<real, P>;
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT;
    constexpr int NPL = NE * ES;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real *sF = reinterpret_cast<real *>(smem_raw);  // NDF planes (+1 spare)
    real *sX = sF + (NDF + 1) * NPL;               // 3*NX planes
    real *sD = sX + 3 * NX * NPL;
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);
    int *sPerm = sNode + NPL;
    int *sLat = sPerm + N;

    const int tid = threadIdx.x;
    const int e0 = blockIdx.x * NE;
    load_element_tables<real, P>(invAtoIJK, AtoI, AtoJ, AtoK, dlxigp_ip, sPerm, sLat, sD, tid, NT);

    // Node ids and the element-layout viscosities (element-fastest, coalesced).
    for (int i = tid; i < NE * N; i += NT) {
        const int el = i % NE, a = i / NE, e = e0 + el;
        const int o = el * ES + sLat[a];
        int node = -1;
        real me = (real)0, ms = (real)0;
        if (e < nelem) {
            const int v = ldg(connec + (size_t)a * nelem + e) - 1;
            node = (v >= 0 && v < npoin) ? v : -1;
            me = ldg(mu_e + (size_t)a * nelem + e);
            ms = ldg(mu_sgs + (size_t)a * nelem + e);
        }
        sNode[o] = node;
        sF[D_MUE * NPL + o] = me;
        sF[D_MUS * NPL + o] = ms;
    }
    __syncthreads();
    const size_t np = (size_t)npoin;
    for (int i = tid; i < NE * N; i += NT) {
        const int el = i / N, l = i - el * N;
        const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
        const int o = el * ES + (K * Q + J) * QP + I;
        const int p = sNode[o];
        real v[6] = {(real)1, (real)0, (real)0, (real)0, (real)0, (real)0};
        if (p >= 0) {
            v[0] = ldg(rho + p);
            v[1] = ldg(Tem + p);
#pragma unroll
            for (int c = 0; c < 3; ++c) v[2 + c] = ldg(u + c * np + p);
            v[5] = ldg(mu_fluid + p);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) sF[c * NPL + o] = v[c];
    }
    __syncthreads();
    diffu_grad_pass<real, P, 0>(sF, sX, sD);
    diffu_grad_pass<real, P, 1>(sF, sX, sD);
    diffu_grad_pass<real, P, 2>(sF, sX, sD);
    __syncthreads();

    // Point pass: physical gradients, stress and contravariant fluxes.
    const real twoThirds = (real)2 / (real)3;
    for (int i = tid; i < NE * N; i += NT) {
        const int el = i / N, a = i - el * N, e = e0 + el;
        const int o = el * ES + sLat[a];
        real gi[3][5];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int f = 0; f < 5; ++f) gi[d][f] = sX[(d * 5 + f) * NPL + o];
        const real r = sF[D_RHO * NPL + o];
        const real uu[3] = {sF[D_U0 * NPL + o], sF[D_U1 * NPL + o], sF[D_U2 * NPL + o]};
        const real muf = sF[D_MUF * NPL + o], me = sF[D_MUE * NPL + o], ms = sF[D_MUS * NPL + o];
        real Hm[3][3];  // Hm[i][j] = He(i,j)
        real gp = (real)0;
        if (e < nelem) {
            const real *hp = He + ((size_t)e * N + a) * 9;
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int ii = 0; ii < 3; ++ii) Hm[ii][j] = ldg(hp + j * 3 + ii);
            gp = ldg(gpvol + (size_t)e * N + a);
        } else {
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int ii = 0; ii < 3; ++ii) Hm[ii][j] = (real)0;
        }
        real gR[3], gT[3], gU[3][3];
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
            gR[ii] = Hm[ii][0] * gi[0][D_RHO] + Hm[ii][1] * gi[1][D_RHO] + Hm[ii][2] * gi[2][D_RHO];
            gT[ii] = Hm[ii][0] * gi[0][D_T] + Hm[ii][1] * gi[1][D_T] + Hm[ii][2] * gi[2][D_T];
#pragma unroll
            for (int j = 0; j < 3; ++j)
                gU[ii][j] = Hm[j][0] * gi[0][D_U0 + ii] + Hm[j][1] * gi[1][D_U0 + ii] + Hm[j][2] * gi[2][D_U0 + ii];
        }
        const real mu_fgp = muf + r * ms;
        const real mu_tot = mu_fgp + me;
        const real divU = gU[0][0] + gU[1][1] + gU[2][2];
        real tau[3][3], tauU[3];
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int j = 0; j < 3; ++j) tau[ii][j] = mu_tot * (gU[ii][j] + gU[j][ii]);
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) tau[ii][ii] -= mu_fgp * twoThirds * divU;
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) tauU[ii] = tau[ii][0] * uu[0] + tau[ii][1] * uu[1] + tau[ii][2] * uu[2];
        const real *Xv[NX] = {gR, tauU, gT, tau[0], tau[1], tau[2]};
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int x = 0; x < NX; ++x)
                sX[(d * NX + x) * NPL + o] = gp * (Hm[0][d] * Xv[x][0] + Hm[1][d] * Xv[x][1] + Hm[2][d] * Xv[x][2]);
        sF[P_NUE * NPL + o] = me / r;
        sF[P_KAP * NPL + o] = muf * Cp / Pr + me * Cp / Pr + Cp * r * ms / (real)0.9;
    }
    __syncthreads();
    diffu_div_pass<real, P, 0>(sF, sX, sD, sNode, e0, nelem, npoin, Rmass, Rmom, Rener);
    __syncthreads();
    diffu_div_pass<real, P, 1>(sF, sX, sD, sNode, e0, nelem, npoin, Rmass, Rmom, Rener);
    __syncthreads();
    diffu_div_pass<real, P, 2>(sF, sX, sD, sNode, e0, nelem, npoin, Rmass, Rmom, Rener);
}

template <typename real, int P>
constexpr size_t diffu_smem()
{
    using G = LineGeom<real, P>;
    return (size_t)(NDF + 1 + 3 * NX) * G::NE * G::ES * sizeof(real) + 3 * G::Q * G::Q * sizeof(real) +
           (size_t)(G::NE * G::ES + 2 * G::N) * sizeof(int);
}

template <typename real, int P>
cudaError_t launch_diffu_p(const DiffuArgs<real> &a, cudaStream_t st)
{
    using G = LineGeom<real, P>;
    constexpr size_t smem = diffu_smem<real, P>();
    static_assert(smem <= 227 * 1024, "shared memory budget");
    cudaError_t err = cudaFuncSetAttribute(diffu_kernel<real, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    const unsigned grid = (unsigned)((a.nelem + G::NE - 1) / G::NE);
    diffu_kernel<real, P><<<grid, G::NT, smem, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.dlxigp_ip,
                                                     a.invAtoIJK, a.AtoI, a.AtoJ, a.AtoK, a.Cp, a.Pr, a.rho, a.u,
                                                     a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs, a.Rmass, a.Rmom, a.Rener);
    return cudaGetLastError();
}

}  // namespace

template <typename real>
cudaError_t launch_diffu_plain(int porder, const DiffuArgs<real> &a, cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_diffu_p<real, 1>(a, st);
    case 2: return launch_diffu_p<real, 2>(a, st);
    case 3: return launch_diffu_p<real, 3>(a, st);
    case 4: return launch_diffu_p<real, 4>(a, st);
    case 5: return launch_diffu_p<real, 5>(a, st);
    case 6: return launch_diffu_p<real, 6>(a, st);
    case 7: return launch_diffu_p<real, 7>(a, st);
    case 8: return launch_diffu_p<real, 8>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_diffu_plain<float>(int, const DiffuArgs<float> &, cudaStream_t);
template cudaError_t launch_diffu_plain<double>(int, const DiffuArgs<double> &, cudaStream_t);

}  // namespace msod
