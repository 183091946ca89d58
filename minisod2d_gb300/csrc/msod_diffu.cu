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
// Design (persistent blocks, groups of NE elements, one thread per GLL line):
//   0. the node ids of the next group are loaded into registers while the
//      current group is computed; after it, the next group's node fields
//      (rho, T, u, mu_fluid) and element-layout mu_e, mu_sgs are gathered with
//      cp.async into the shared-memory lattice (single-buffered: measured 6 %
//      faster than a double-buffered lattice, whose shared memory held the
//      kernel to two blocks per SM instead of three; DIFFU_NBUF = 2 selects
//      it); the He and gpvol values of the point pass are loaded into
//      registers before pass 1;
//   1. three line passes store the 15 iso-parametric derivatives per point;
//   2. a point pass turns them into physical gradients and stress and stores,
//      per direction d, the contravariant fluxes gpvol * He(:,d)^T X for the
//      six vectors X = grad rho, tauU, grad T, tau rows 1..3 (18 per point),
//      plus nu_e and kappa_e per output node;
//   3. three line passes apply the transposed 1-D derivative matrix along the
//      lines (the weak divergence), accumulating five sums per node through
//      shared memory; the last pass scatter-adds with red.global.add.
// With one thread per line from porder 3 up, the zeta derivative pass, the
// point pass and the zeta divergence pass run as one pass over each zeta line
// (the zeta derivatives and fluxes never reach shared memory, the He rows are
// loaded there one point ahead), and the flux region shrinks from 18 planes to
// 12: porder 4 then takes 53.8 KB of shared memory per block instead of 68.8 KB,
// three blocks leave ~88 KB of L1 instead of ~28 KB for the He and node-field
// loads, and the kernel runs 1.50 ms instead of 1.82 ms on 64^3 hexes (the same
// fusion with the 18-plane region: 1.79 ms; four blocks per SM at 128
// registers, which fill the shared memory again: 1.90 ms).
// The 1-D derivative matrices are constant-bank operands.
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

// Zeta stage (one thread per line only): 1 = the zeta derivatives, the point
// pass and the zeta divergence run as one pass over each zeta line, with the
// zeta derivatives and fluxes in registers; 0 = three line passes, a point
// pass over all points, three divergence passes.
#ifndef DIFFU_FUSEZ
#define DIFFU_FUSEZ 1
#endif

// Lattices of gathered node fields: 2 = double-buffered (the next group's
// fields are gathered with cp.async while the current group is computed),
// 1 = single (less shared memory, more blocks per SM).
#ifndef DIFFU_NBUF
#define DIFFU_NBUF 1
#endif

// Threads take their lines from the bank-aware map (LineMap) with one thread
// per line, up to this porder (0: never); other porders keep the lines of
// consecutive elements side by side.  Measured: plain_64 1.483 against
// 1.503 ms; porder 5 on 64^3 hexes 2.99 against 2.96 ms (off there).
#ifndef DIFFU_LINEMAP
#define DIFFU_LINEMAP 4
#endif
// Where the map applies: 0 = never, 1 = always, 2 = on meshes whose elements
// share nodes (npoin < nelem * nodes per element), not on disconnected ones.
// Measured through the driver, porder 4 (on / off): disconnected meshes of
// 192,000 and 262,144 hexes 1.043 / 1.018 and 1.404 / 1.373 ms; structured
// 64^3 and 48^3 meshes 1.323 / 1.373 and 0.585 / 0.604 ms.
#ifndef DIFFU_LINEMAP_MODE
#define DIFFU_LINEMAP_MODE 2
#endif
// Gather of the node fields: 0 = 4-byte cp.async copies, 1 = loads into
// registers, then 32-lane shared-memory stores.  Measured: plain_64 1.466
// against 1.483 ms (at three blocks per SM, DIFFU_MINB4=3), porder 5 on 64^3
// hexes 3.82 against 2.99 ms (registers); off.
#ifndef DIFFU_GATHER_LDG
#define DIFFU_GATHER_LDG 0
#endif

namespace msod {
namespace {

// The thread's line in direction dir (linemap: the launch's choice of map).
template <class G>
__device__ __forceinline__ LineThread<G> diffu_line(int tid, int dir, int linemap)
{
    if constexpr (G::P <= DIFFU_LINEMAP && G::S == 1)
        if (linemap) return LineThread<G>(kLineMap<G>.code[dir][tid], true);
    return LineThread<G>(tid);
}

__constant__ float c_Df[MSOD_MAX_PORDER + 1][kTableDMax];
__constant__ double c_Dd[MSOD_MAX_PORDER + 1][kTableDMax];

template <typename real>
__device__ __forceinline__ real cD(int P, int i);
template <>
__device__ __forceinline__ float cD<float>(int P, int i)
{
    return c_Df[P][i];
}
template <>
__device__ __forceinline__ double cD<double>(int P, int i)
{
    return c_Dd[P][i];
}

enum { D_RHO = 0, D_T, D_U0, D_U1, D_U2, D_MUF, D_MUE, D_MUS, NDF };  // gathered planes
enum { X_GRHO = 0, X_TAUU, X_GT, X_TAU0, X_TAU1, X_TAU2, NX };        // flux vectors
// After the point pass a stage's gathered planes hold: 0 nu_e, 1 kappa_e, 2..6 partial sums.
enum { P_NUE = 0, P_KAP = 1, P_DR = 2 };

// Pass 1, direction DIR: iso-parametric derivatives of rho, T, u0..2 at the
// thread's points, stored to planes sX[DIR*5 + f].
template <class G, int DIR>
__device__ __forceinline__ void grad_pass(const LineThread<G> &lt, const typename G::real *__restrict__ sF,
                                          typename G::real *__restrict__ sX, const typename G::real *__restrict__ sD)
{
    using real = typename G::real;
    constexpr int P = G::P, Q = G::Q, QP = G::QP, R = G::R, NPL = G::NPL;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int base = lt.el * G::ES + line_off<DIR, Q, QP>(lt.la, lt.lb, 0);
    // Several threads per line: the thread's rows of the matrix, in registers
    // for the pass (a per-lane index into the constant bank would serialise).
    real Dr[G::S > 1 ? R : 1][Q];
    if (G::S > 1)
#pragma unroll
        for (int rr = 0; rr < R; ++rr)
#pragma unroll
            for (int c = 0; c < Q; ++c) Dr[rr][c] = sD[(DIR * Q + lt.rc(rr)) * Q + c];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        real v[Q];
#pragma unroll
        for (int c = 0; c < Q; ++c) v[c] = sF[f * NPL + base + c * OST];
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            if (!lt.owns(rr)) continue;
            real s = (real)0;
#pragma unroll
            for (int c = 0; c < Q; ++c)
                s = fma(G::S == 1 ? cD<real>(P, (DIR * Q + rr) * Q + c) : Dr[G::S == 1 ? 0 : rr][c], v[c], s);
            sX[(DIR * 5 + f) * NPL + base + (lt.r0 + rr) * OST] = s;
        }
    }
}

// Pass 2, direction DIR: weak divergence along the lines with the transposed
// derivative matrix; partial sums through planes P_DR.. of the stage.
template <class G, int DIR, bool FIRST, bool LAST>
__device__ __forceinline__ void div_pass(const LineThread<G> &lt, typename G::real *__restrict__ sF,
                                         const typename G::real *__restrict__ sX, const typename G::real *__restrict__ sD,
                                         const int *__restrict__ sNode, int npoin,
                                         typename G::real *__restrict__ Rmass, typename G::real *__restrict__ Rmom,
                                         typename G::real *__restrict__ Rener)
{
    using real = typename G::real;
    constexpr int P = G::P, Q = G::Q, QP = G::QP, R = G::R, NPL = G::NPL;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int base = lt.el * G::ES + line_off<DIR, Q, QP>(lt.la, lt.lb, 0);
    real Dc[G::S > 1 ? R : 1][Q];  // several threads per line: the thread's columns
    if (G::S > 1)
#pragma unroll
        for (int rr = 0; rr < R; ++rr)
#pragma unroll
            for (int c = 0; c < Q; ++c) Dc[rr][c] = sD[(DIR * Q + c) * Q + lt.rc(rr)];
    real acc[R][5], kap[R];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int o = base + lt.rc(rr) * OST;
        kap[rr] = sF[P_KAP * NPL + o];
#pragma unroll
        for (int k = 0; k < 5; ++k) acc[rr][k] = FIRST ? (real)0 : sF[(P_DR + k) * NPL + o];
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
            for (int c = 0; c < Q; ++c)
                s = fma(G::S == 1 ? cD<real>(P, (DIR * Q + c) * Q + rr) : Dc[G::S == 1 ? 0 : rr][c], v[c], s);
            if (x == X_GRHO) acc[rr][0] += s;
            else if (x == X_TAUU) acc[rr][1] += s;
            else if (x == X_GT) acc[rr][1] = fma(kap[rr], s, acc[rr][1]);
            else acc[rr][2 + (x - X_TAU0)] += s;
        }
    }
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        if (!lt.owns(rr)) continue;
        const int o = base + (lt.r0 + rr) * OST;
        if (!LAST) {
#pragma unroll
            for (int k = 0; k < 5; ++k) sF[(P_DR + k) * NPL + o] = acc[rr][k];
        } else {
            const int node = sNode[o];
            if ((unsigned)node >= (unsigned)npoin) continue;
            red_add(Rmass + node, sF[P_NUE * NPL + o] * acc[rr][0]);
            red_add(Rener + node, acc[rr][1]);
#pragma unroll
            for (int m = 0; m < 3; ++m) red_add(Rmom + (size_t)m * npoin + node, acc[rr][2 + m]);
        }
    }
}

// Point pass at one point: physical gradients of rho, T, u from the
// iso-parametric ones gi[d][f] (He(ii, j) = H[j*3 + ii]), the stress and
// tau u, and the contravariant fluxes F[d][x] = gpvol He(:,d)^T X_x.
template <typename real>
__device__ __forceinline__ void point_flux(const real (&gi)[3][5], real r, const real (&uu)[3], real muf, real ms,
                                           real me, const real (&H)[9], real gv, real (&F)[3][NX])
{
    const real twoThirds = (real)2 / (real)3;
    real gR[3], gT[3], gU[3][3];
#pragma unroll
    for (int ii = 0; ii < 3; ++ii) {
        gR[ii] = H[ii] * gi[0][D_RHO] + H[3 + ii] * gi[1][D_RHO] + H[6 + ii] * gi[2][D_RHO];
        gT[ii] = H[ii] * gi[0][D_T] + H[3 + ii] * gi[1][D_T] + H[6 + ii] * gi[2][D_T];
#pragma unroll
        for (int j = 0; j < 3; ++j)
            gU[ii][j] = H[j] * gi[0][D_U0 + ii] + H[3 + j] * gi[1][D_U0 + ii] + H[6 + j] * gi[2][D_U0 + ii];
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
            F[d][x] = gv * (H[d * 3] * Xv[x][0] + H[d * 3 + 1] * Xv[x][1] + H[d * 3 + 2] * Xv[x][2]);
}

// The fused zeta stage runs where one thread owns a line, from porder 3 up
// (porder 2 on 120^3 hexes: 1.98 ms unfused, 2.03 ms fused).
template <class G>
constexpr bool diffu_fusez()
{
    return DIFFU_FUSEZ != 0 && G::S == 1 && G::P >= 3;
}
// Flux planes: three directions, or two with the fused zeta stage (the zeta
// derivatives and fluxes stay in registers).
template <class G>
constexpr int diffu_xplanes()
{
    return (diffu_fusez<G>() ? 2 : 3) * NX;
}

// He rows of the fused zeta stage: 0 = the line's rows in registers from the
// start of the group (across the gradient passes), 1 = each point's row loaded
// in the stage one point ahead (fewer registers).
#ifndef DIFFU_HE_LATE
#define DIFFU_HE_LATE 1
#endif
// Minimum blocks per SM in the launch bounds. The kernels with the fused zeta
// stage take 1, which lets the compiler spend registers (porder 4: 137 / 153 /
// 153 for the three viscosity sources, porder 5: 159-163); this holds them to
// three blocks per SM and keeps the L1 that the larger carveout of a fourth
// block would take (DIFFU_MINB4 = 4, 128 registers: 1.90 ms against 1.50 ms,
// porder 4 on 64^3). The other kernels take 0, the block-size-only heuristic
// (a 1 there raised porder 6 from 115 to 154 registers: one block per SM
// instead of two).
#ifndef DIFFU_MINB4
#define DIFFU_MINB4 1
#endif
template <class G>
constexpr int diffu_minb()
{
    return diffu_fusez<G>() ? ((sizeof(typename G::real) == 4 && G::P == 4) ? DIFFU_MINB4 : 1) : 0;
}

// kappa_e at a node (elem_diffu.f90:143-146).
template <typename real>
__device__ __forceinline__ real kappa_e(real muf, real me, real ms, real r, real Cp, real Pr)
{
    return muf * Cp / Pr + me * Cp / Pr + Cp * r * ms / (real)0.9;
}

// He and gpvol of a group staged in shared memory by bulk copies (the group's
// spans of He(3,3,ngaus,nelem) and gpvol(ngaus,nelem) are contiguous), issued
// one group ahead: 1 = the fused zeta stage's FP32 kernels, 0 = per-point
// loads from global memory.  Measured slower and off: the 25 KB per block
// leave two blocks per SM instead of three (plain_64 1.76 against 1.48 ms;
// porder 5 on 64^3 hexes 3.63 against 2.99 ms).
#ifndef DIFFU_HE_BULK
#define DIFFU_HE_BULK 0
#endif
template <class G>
constexpr bool diffu_staged()
{
    return DIFFU_HE_BULK != 0 && diffu_fusez<G>() && DIFFU_HE_LATE != 0 && sizeof(typename G::real) == 4;
}
template <class G>
constexpr size_t diffu_he_bytes()
{
    return ((size_t)G::NE * G::N * 9 * sizeof(typename G::real) + 31) / 16 * 16;
}
template <class G>
constexpr size_t diffu_gp_bytes()
{
    return ((size_t)G::NE * G::N * sizeof(typename G::real) + 31) / 16 * 16;
}
template <class G>
constexpr size_t diffu_stage_bytes()
{
    return diffu_staged<G>() ? diffu_he_bytes<G>() + diffu_gp_bytes<G>() + 16 : 0;
}

template <class G>
constexpr size_t diffu_smem_bytes()
{
    return diffu_stage_bytes<G>() +
           (size_t)(DIFFU_NBUF * NDF + diffu_xplanes<G>()) * G::NPL * sizeof(typename G::real) +
           (size_t)3 * G::Q * G::Q * sizeof(typename G::real) +
           (size_t)(DIFFU_NBUF * G::NPL + 2 * G::N) * sizeof(int);
}

// Threads per line of the FP32 diffusion (0: the line-geometry default: one
// up to porder 5, two at 6-7, three at 8; one is the only form with the fused
// zeta stage).  Measured on 64^3 hexes: porder 4
// is fastest with one (1.84 ms; 2.08-2.27 ms with 2, 3 or 5: more warps, but
// the line loads are repeated per thread).  Porder 5 with one and the fused
// zeta stage, three elements per 128-thread block: 2.97 ms, against 3.78 ms
// with two threads per line (three elements per 224-thread block, unfused) and
// 3.19 ms with one at two elements per block.  Porder 7 on 32^3 hexes with one
// and the fused zeta stage, two elements per 128-thread block (161 registers):
// 1.183 ms, against 1.266 ms with two (unfused, 256 threads), 1.345 ms with one
// element and 1.255 ms with three per block.  Porder 6 on 32^3 hexes with one,
// three elements per 160-thread block: 0.685 ms, against 0.787 ms with two
// (0.687 ms at two elements).  Porder 8 on 32^3 hexes keeps three: 1.907 ms,
// against 2.20 / 2.13 ms with one at one / two elements per block.
#ifndef DIFFU_S4
#define DIFFU_S4 0
#endif
#ifndef DIFFU_S5
#define DIFFU_S5 1
#endif
#ifndef DIFFU_S6
#define DIFFU_S6 1
#endif
#ifndef DIFFU_S7
#define DIFFU_S7 1
#endif
#ifndef DIFFU_S8
#define DIFFU_S8 0
#endif
template <typename real, int P>
constexpr int diffu_s()
{
    return sizeof(real) != 4 ? 0
           : P == 4          ? DIFFU_S4
           : P == 5          ? DIFFU_S5
           : P == 6          ? DIFFU_S6
           : P == 7          ? DIFFU_S7
           : P == 8          ? DIFFU_S8
                             : 0;
}

// Elements per block of the FP32 diffusion at porders 4-8 (0: the
// line-geometry default).
#ifndef DIFFU_NE4
#define DIFFU_NE4 0
#endif
#ifndef DIFFU_NE5
#define DIFFU_NE5 3
#endif
#ifndef DIFFU_NE6
#define DIFFU_NE6 3
#endif
#ifndef DIFFU_NE7
#define DIFFU_NE7 2
#endif
#ifndef DIFFU_NE8
#define DIFFU_NE8 0
#endif
template <typename real, int P>
constexpr int diffu_necap()
{
    constexpr int ne = sizeof(real) != 4 ? 0
                       : P == 4          ? DIFFU_NE4
                       : P == 5          ? DIFFU_NE5
                       : P == 6          ? DIFFU_NE6
                       : P == 7          ? DIFFU_NE7
                       : P == 8          ? DIFFU_NE8
                                         : 0;
    return ne > 0 ? ne : necap_for(2 * NDF + 3 * NX, LineGeom<real, P>::ES, (int)sizeof(real), 200 * 1024);
}

template <typename real, int P>
using DiffuGeom = LineGeom<real, P, diffu_necap<real, P>(), diffu_s<real, P>()>;

// Viscosity source of the diffusion kernel: the mu_e array, or one value per
// element (mu_e(e, a) = rho(a) nu_elem(e)).
enum { VISC_MU_E = 0, VISC_NU_ELEM = 1 };

template <class G, int VISC>
__global__ void __launch_bounds__(G::NT, diffu_minb<G>())
    diffu_kernel(int nelem, int npoin, int ngroups, const int *__restrict__ connec,
                 const typename G::real *__restrict__ He, const typename G::real *__restrict__ gpvol,
                 const TableScratch *__restrict__ tabs, typename G::real Cp, typename G::real Pr,
                 const typename G::real *__restrict__ rho, const typename G::real *__restrict__ u,
                 const typename G::real *__restrict__ Tem, const typename G::real *__restrict__ mu_fluid,
                 const typename G::real *__restrict__ mu_e, const typename G::real *__restrict__ mu_sgs,
                 const typename G::real *__restrict__ nu_elem, typename G::real *__restrict__ Rmass,
                 typename G::real *__restrict__ Rmom, typename G::real *__restrict__ Rener, int linemap)
{
    using real = typename G::real;
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT, NPL = G::NPL;
    constexpr int IPT = (NE * N + NT - 1) / NT;  // items (node ids, points) per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NBUF = DIFFU_NBUF;
    constexpr bool STAGED = diffu_staged<G>();
    char *sHeB = reinterpret_cast<char *>(smem_raw);  // staged He / gpvol spans, then the mbarrier
    char *sGpB = sHeB + diffu_he_bytes<G>();
    unsigned long long *sBar = reinterpret_cast<unsigned long long *>(sGpB + diffu_gp_bytes<G>());
    real *sF = reinterpret_cast<real *>(smem_raw + diffu_stage_bytes<G>());  // [NBUF][NDF][NPL]
    real *sX = sF + NBUF * NDF * NPL;                // [2 or 3 NX][NPL]
    real *sD = sX + diffu_xplanes<G>() * NPL;        // [3][Q][Q] (several threads per line)
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);  // [NBUF][NPL]
    int *sPerm = sNode + NBUF * NPL;
    int *sLat = sPerm + N;

    const int tid = threadIdx.x;
    const LineThread<G> lt0 = diffu_line<G>(tid, 0, linemap), lt1 = diffu_line<G>(tid, 1, linemap),
                        lt2 = diffu_line<G>(tid, 2, linemap);
    constexpr bool FUSEZ = diffu_fusez<G>();
    constexpr bool LATE = FUSEZ && DIFFU_HE_LATE != 0;
    constexpr int MP = LATE ? 1 : (FUSEZ ? Q : IPT);  // points whose He and gpvol a thread holds
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    if (G::S > 1)
        for (int i = tid; i < 3 * Q * Q; i += NT) sD[i] = table_D<real>(tabs)[i];
    auto load_ids = [&](int g, int (&ids)[IPT]) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            const int el = i % NE, a = i / NE, e = g * NE + el;
            ids[k] = (i < NE * N && e < nelem) ? ldg(connec + (size_t)a * nelem + e) : 0;
        }
    };
    auto store_ids = [&](const int (&ids)[IPT], int *dst) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            if (i < NE * N) {
                const int v = ids[k] - 1;
                dst[(i % NE) * ES + sLat[i / NE]] = (v >= 0 && v < npoin) ? v : -1;
            }
        }
    };
    // Node fields in lattice order; mu_e / mu_sgs along elements (coalesced).
    auto gather = [&](int g, const int *ids_s, real *dst) {
        if constexpr (DIFFU_GATHER_LDG != 0) {
            // Loads of all of a thread's items first, then the stores.
            real v[IPT][6], w[IPT][2];
            int ov[IPT], ow[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT;
                const bool in = i < NE * N;
                const int el = in ? i / N : 0, l = in ? i - el * N : 0;
                const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
                const int o = el * ES + (K * Q + J) * QP + I;
                ov[k] = in ? o : -1;
                const int p = in ? ids_s[o] : -1;
                const bool ok = (unsigned)p < (unsigned)npoin;
                const size_t pp = ok ? (size_t)p : 0, np = (size_t)npoin;
                v[k][0] = ok ? ldg(rho + pp) : (real)0;
                v[k][1] = ok ? ldg(Tem + pp) : (real)0;
#pragma unroll
                for (int c = 0; c < 3; ++c) v[k][2 + c] = ok ? ldg(u + c * np + pp) : (real)0;
                v[k][5] = ok ? ldg(mu_fluid + pp) : (real)0;
                const int el2 = i % NE, a = i / NE, e = g * NE + el2;
                ow[k] = in ? el2 * ES + sLat[in ? a : 0] : -1;
                const bool ok2 = in && e < nelem;
                const size_t idx = ok2 ? (size_t)a * nelem + e : 0;
                w[k][0] = (VISC == VISC_MU_E && ok2) ? ldg(mu_e + idx) : (real)0;
                w[k][1] = ok2 ? ldg(mu_sgs + idx) : (real)0;
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if (ov[k] < 0) continue;
                dst[D_RHO * NPL + ov[k]] = v[k][0];
                dst[D_T * NPL + ov[k]] = v[k][1];
#pragma unroll
                for (int c = 0; c < 3; ++c) dst[(D_U0 + c) * NPL + ov[k]] = v[k][2 + c];
                dst[D_MUF * NPL + ov[k]] = v[k][5];
                if (VISC == VISC_MU_E) dst[D_MUE * NPL + ow[k]] = w[k][0];
                dst[D_MUS * NPL + ow[k]] = w[k][1];
            }
            return;
        }
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i / N, l = i - el * N;
            const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
            const int o = el * ES + (K * Q + J) * QP + I;
            const int p = ids_s[o];
            const bool ok = (unsigned)p < (unsigned)npoin;
            const size_t pp = ok ? (size_t)p : 0, np = (size_t)npoin;
            cp_async_elem(dst + D_RHO * NPL + o, rho + pp, ok);
            cp_async_elem(dst + D_T * NPL + o, Tem + pp, ok);
#pragma unroll
            for (int c = 0; c < 3; ++c) cp_async_elem(dst + (D_U0 + c) * NPL + o, u + c * np + pp, ok);
            cp_async_elem(dst + D_MUF * NPL + o, mu_fluid + pp, ok);
        }
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i % NE, a = i / NE, e = g * NE + el;
            const int o = el * ES + sLat[a];
            const bool ok = e < nelem;
            const size_t idx = ok ? (size_t)a * nelem + e : 0;
            if (VISC == VISC_MU_E) cp_async_elem(dst + D_MUE * NPL + o, mu_e + idx, ok);
            cp_async_elem(dst + D_MUS * NPL + o, mu_sgs + idx, ok);
        }
        cp_async_commit();
    };
    // He(:,:) and gpvol of the thread's point-pass points: items tid + k NT
    // (lattice order), or the points of its zeta line in the zeta stage.
    auto load_metric = [&](int g, real (&Hm)[MP][9], real (&gv)[MP]) {
#pragma unroll
        for (int k = 0; k < MP; ++k) {
            const int i = tid + k * NT;
            const int el = FUSEZ ? lt2.el : i / N;
            const int l = FUSEZ ? line_lat<2, Q>(lt2.la, lt2.lb, k) : i - el * N, e = g * NE + el;
            const bool ok = (FUSEZ ? lt2.active : i < NE * N) && e < nelem;
            const int a = ok ? sPerm[l] : 0;
            const real *hp = He + (ok ? ((size_t)e * N + a) * 9 : 0);
#pragma unroll
            for (int j = 0; j < 9; ++j) Hm[k][j] = ok ? ldg(hp + j) : (real)0;
            gv[k] = ok ? ldg(gpvol + (size_t)e * N + a) : (real)0;
        }
    };

    // mu_e at a point of element el of group g (lattice offset o, density r).
    auto point_mu_e = [&](int g, int el, int o, real r, const real *sFs) -> real {
        const int ee = g * NE + el;
        return VISC == VISC_NU_ELEM ? (ee < nelem ? r * ldg(nu_elem + ee) : (real)0) : sFs[D_MUE * NPL + o];
    };

    // Staged He / gpvol: bulk copies of group g's spans (thread 0), the
    // unaligned ends by plain loads (threads 32..37, 64..69).  Offsets of the
    // spans' first words in the staging area.
    int he_off = 0, gp_off = 0;
    auto stage = [&](int g) {
        if constexpr (STAGED) {
            const int e0 = g * NE, e1 = min(e0 + NE, nelem);
            const SpanPlan ph(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
            const SpanPlan pg(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
            if (tid == 0) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(sBar, ph.bulk + pg.bulk);
                ph.issue(sHeB, sBar);
                pg.issue(sGpB, sBar);
            } else if (tid >= 32 && tid < 38) {
                ph.plain(sHeB, tid - 32);
            } else if (tid >= 64 && tid < 70) {
                pg.plain(sGpB, tid - 64);
            }
            he_off = (int)(ph.shift / sizeof(real));
            gp_off = (int)(pg.shift / sizeof(real));
        }
    };
    unsigned phase = 0;

    int g = blockIdx.x;
    const int stride = gridDim.x;
    if constexpr (STAGED) {
        if (tid == 0) mbar_init(sBar, 1);
        __syncthreads();
        stage(g);
    }
    int ids[IPT];
    load_ids(g, ids);
    __syncthreads();  // sLat ready
    store_ids(ids, sNode);
    __syncthreads();
    gather(g, sNode, sF);
    int gn = g + stride;
    if (gn < ngroups) load_ids(gn, ids);

    int s = 0;
    for (; g < ngroups; g = gn, gn += stride, s = NBUF == 2 ? s ^ 1 : 0) {
        real *sFs = sF + s * NDF * NPL;
        int *sNs = sNode + s * NPL;
        real Hm[MP][9], gv[MP];
        if (!LATE) load_metric(g, Hm, gv);
        if (NBUF == 2 && gn < ngroups) store_ids(ids, sNode + (s ^ 1) * NPL);
        cp_async_wait_all();
        __syncthreads();
        if (NBUF == 2 && gn < ngroups) {
            gather(gn, sNode + (s ^ 1) * NPL, sF + (s ^ 1) * NDF * NPL);
            if (gn + stride < ngroups) load_ids(gn + stride, ids);
        }
        if constexpr (FUSEZ) {
            if (lt0.active) grad_pass<G, 0>(lt0, sFs, sX, sD);
            if (lt1.active) grad_pass<G, 1>(lt1, sFs, sX, sD);
            if constexpr (STAGED) {
                // Bounded wait for group g's spans; every thread learns the outcome.
                const bool ok = mbar_wait(sBar, phase);
                phase ^= 1u;
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) report_wait_fault(tabs);
                    return;
                }
            } else {
                __syncthreads();
            }
            // Zeta stage, one thread per zeta line: the zeta derivatives at the
            // line's points (from its nodal values in registers), the point
            // pass there (the xi and eta fluxes are stored for their
            // divergence passes) and the zeta divergence of the zeta fluxes,
            // which stay in registers; the partial sums start the divergence.
            if (lt2.active) {
                const LineThread<G> &lt = lt2;
                constexpr int OST = Q * QP;
                const int base = lt.el * ES + line_off<2, Q, QP>(lt.la, lt.lb, 0);
                real v[5][Q];
#pragma unroll
                for (int f = 0; f < 5; ++f)
#pragma unroll
                    for (int c = 0; c < Q; ++c) v[f][c] = sFs[f * NPL + base + c * OST];
                real acc[Q][5], accT[Q], kap[Q];
#pragma unroll
                for (int rr = 0; rr < Q; ++rr) {
                    accT[rr] = (real)0;
#pragma unroll
                    for (int k = 0; k < 5; ++k) acc[rr][k] = (real)0;
                }
                const int ee = g * NE + lt.el;
                const bool eok = ee < nelem;
                // Late He rows: point c's row and gpvol, issued one point ahead.
                auto he_row = [&](int c, real (&h)[9], real &gp) {
                    const int a = sPerm[line_lat<2, Q>(lt.la, lt.lb, c)];
                    if constexpr (STAGED) {
                        const real *hp = reinterpret_cast<const real *>(sHeB) + he_off + (lt.el * N + a) * 9;
#pragma unroll
                        for (int j = 0; j < 9; ++j) h[j] = hp[j];
                        gp = reinterpret_cast<const real *>(sGpB)[gp_off + lt.el * N + a];
                    } else {
                        const real *hp = He + (eok ? ((size_t)ee * N + a) * 9 : 0);
#pragma unroll
                        for (int j = 0; j < 9; ++j) h[j] = eok ? ldg(hp + j) : (real)0;
                        gp = eok ? ldg(gpvol + (size_t)ee * N + a) : (real)0;
                    }
                };
                real Hn[9], gpn;
                if constexpr (LATE) he_row(0, Hn, gpn);
#pragma unroll
                for (int c = 0; c < Q; ++c) {
                    const int o = base + c * OST;
                    real Hc[9], gc;
                    if constexpr (LATE) {
#pragma unroll
                        for (int j = 0; j < 9; ++j) Hc[j] = Hn[j];
                        gc = gpn;
                        if (c + 1 < Q) he_row(c + 1, Hn, gpn);
                    } else {
#pragma unroll
                        for (int j = 0; j < 9; ++j) Hc[j] = Hm[c][j];
                        gc = gv[c];
                    }
                    real gi[3][5];
#pragma unroll
                    for (int d = 0; d < 2; ++d)
#pragma unroll
                        for (int f = 0; f < 5; ++f) gi[d][f] = sX[(d * 5 + f) * NPL + o];
#pragma unroll
                    for (int f = 0; f < 5; ++f) {
                        real t = (real)0;
#pragma unroll
                        for (int j = 0; j < Q; ++j) t = fma(cD<real>(G::P, (2 * Q + c) * Q + j), v[f][j], t);
                        gi[2][f] = t;
                    }
                    const real r = v[D_RHO][c];
                    const real uu[3] = {v[D_U0][c], v[D_U1][c], v[D_U2][c]};
                    const real muf = sFs[D_MUF * NPL + o], ms = sFs[D_MUS * NPL + o];
                    const real me = point_mu_e(g, lt.el, o, r, sFs);
                    real F[3][NX];
                    point_flux(gi, r, uu, muf, ms, me, Hc, gc, F);
#pragma unroll
                    for (int d = 0; d < 2; ++d)
#pragma unroll
                        for (int x = 0; x < NX; ++x) sX[(d * NX + x) * NPL + o] = F[d][x];
#pragma unroll
                    for (int rr = 0; rr < Q; ++rr) {
                        const real w = cD<real>(G::P, (2 * Q + c) * Q + rr);
                        acc[rr][0] = fma(w, F[2][X_GRHO], acc[rr][0]);
                        acc[rr][1] = fma(w, F[2][X_TAUU], acc[rr][1]);
                        accT[rr] = fma(w, F[2][X_GT], accT[rr]);
#pragma unroll
                        for (int m = 0; m < 3; ++m) acc[rr][2 + m] = fma(w, F[2][X_TAU0 + m], acc[rr][2 + m]);
                    }
                    // rho and T of this point are in registers or no longer
                    // needed: their planes take nu_e and kappa_e.
                    kap[c] = kappa_e(muf, me, ms, r, Cp, Pr);
                    sFs[P_NUE * NPL + o] = me / r;
                    sFs[P_KAP * NPL + o] = kap[c];
                }
#pragma unroll
                for (int rr = 0; rr < Q; ++rr) {
                    const int o = base + rr * OST;
                    acc[rr][1] = fma(kap[rr], accT[rr], acc[rr][1]);
#pragma unroll
                    for (int k = 0; k < 5; ++k) sFs[(P_DR + k) * NPL + o] = acc[rr][k];
                }
            }
            __syncthreads();
            if constexpr (STAGED) {
                if (gn < ngroups) stage(gn);  // the spans of the next group, during the divergence
            }
            if (lt0.active) div_pass<G, 0, false, false>(lt0, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            if (lt1.active) div_pass<G, 1, false, true>(lt1, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
        } else {
            if (lt0.active) grad_pass<G, 0>(lt0, sFs, sX, sD);
            if (lt1.active) grad_pass<G, 1>(lt1, sFs, sX, sD);
            if (lt2.active) grad_pass<G, 2>(lt2, sFs, sX, sD);
            __syncthreads();
            // Point pass: physical gradients, stress and contravariant fluxes.
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT;
                if (i >= NE * N) break;
                const int el = i / N, l = i - el * N;
                const int o = el * ES + (l / (Q * Q) * Q + (l / Q) % Q) * QP + l % Q;
                real gi[3][5];
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int f = 0; f < 5; ++f) gi[d][f] = sX[(d * 5 + f) * NPL + o];
                const real r = sFs[D_RHO * NPL + o];
                const real uu[3] = {sFs[D_U0 * NPL + o], sFs[D_U1 * NPL + o], sFs[D_U2 * NPL + o]};
                const real muf = sFs[D_MUF * NPL + o], ms = sFs[D_MUS * NPL + o];
                const real me = point_mu_e(g, el, o, r, sFs);
                real F[3][NX];
                point_flux(gi, r, uu, muf, ms, me, Hm[k], gv[k], F);
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int x = 0; x < NX; ++x) sX[(d * NX + x) * NPL + o] = F[d][x];
                sFs[P_NUE * NPL + o] = me / r;
                sFs[P_KAP * NPL + o] = kappa_e(muf, me, ms, r, Cp, Pr);
            }
            __syncthreads();
            if (lt0.active) div_pass<G, 0, true, false>(lt0, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            if (lt1.active) div_pass<G, 1, false, false>(lt1, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            if (lt2.active) div_pass<G, 2, false, true>(lt2, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
        }
        __syncthreads();
        if (NBUF == 1 && gn < ngroups) {  // the next group's node ids, then its fields
            store_ids(ids, sNode);
            __syncthreads();
            gather(gn, sNode, sF);
            if (gn + stride < ngroups) load_ids(gn + stride, ids);
        }
    }
}

template <typename real, int P, int VISC>
cudaError_t launch_diffu_pn(const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    using G = DiffuGeom<real, P>;
    constexpr size_t smem = diffu_smem_bytes<G>();
    static_assert(smem <= 227 * 1024, "shared memory budget");
    static_assert(G::NE >= 1, "element group");
    auto kern = diffu_kernel<G, VISC>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    if (sizeof(real) == 4)
        err = cudaMemcpyToSymbolAsync(c_Df, table_D<float>(tabs), sizeof(float) * 3 * G::Q * G::Q,
                                      sizeof(float) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
    else
        err = cudaMemcpyToSymbolAsync(c_Dd, table_D<double>(tabs), sizeof(double) * 3 * G::Q * G::Q,
                                      sizeof(double) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return err;
    const int ngroups = (a.nelem + G::NE - 1) / G::NE;
    const int grid = persistent_grid(kern, G::NT, smem, ngroups);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    const int linemap = DIFFU_LINEMAP_MODE == 2 ? (a.npoin < (long long)a.nelem * G::N ? 1 : 0) : DIFFU_LINEMAP_MODE;
    kern<<<grid, G::NT, smem, st>>>(a.nelem, a.npoin, ngroups, a.connec, a.He, a.gpvol, tabs, a.Cp, a.Pr, a.rho, a.u,
                                    a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs, a.nu_elem, a.Rmass, a.Rmom, a.Rener,
                                    linemap);
    return cudaGetLastError();
}

template <typename real, int P>
cudaError_t launch_diffu_p(const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    if (a.nu_elem) return launch_diffu_pn<real, P, VISC_NU_ELEM>(a, tabs, st);
    return launch_diffu_pn<real, P, VISC_MU_E>(a, tabs, st);
}

}  // namespace

template <typename real>
cudaError_t launch_diffu_plain(int porder, const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_diffu_p<real, 1>(a, tabs, st);
    case 2: return launch_diffu_p<real, 2>(a, tabs, st);
    case 3: return launch_diffu_p<real, 3>(a, tabs, st);
    case 4: return launch_diffu_p<real, 4>(a, tabs, st);
    case 5: return launch_diffu_p<real, 5>(a, tabs, st);
    case 6: return launch_diffu_p<real, 6>(a, tabs, st);
    case 7: return launch_diffu_p<real, 7>(a, tabs, st);
    case 8: return launch_diffu_p<real, 8>(a, tabs, st);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_diffu_plain<float>(int, const DiffuArgs<float> &, const TableScratch *, cudaStream_t);
template cudaError_t launch_diffu_plain<double>(int, const DiffuArgs<double> &, const TableScratch *, cudaStream_t);

}  // namespace msod
