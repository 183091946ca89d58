// msod_diffu.cuh -- device code of the plain hex diffusion: the line
// passes, the point pass, their tables in the constant bank and the launch
// configuration per porder.  Included by the diffusion kernel
// (msod_diffu.cu) and the fused convection + diffusion kernel
// (msod_fused.cu); each translation unit holds its own copy of the
// constant-bank tables and fills it before its launches.
#pragma once

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

// No FP64 copy under MSOD_FP32_ONLY (see msod_convec.cuh).
__constant__ float c_Df[MSOD_MAX_PORDER + 1][kTableDMax];
#ifndef MSOD_FP32_ONLY
__constant__ double c_Dd[MSOD_MAX_PORDER + 1][kTableDMax];
#endif

template <typename real>
__device__ __forceinline__ real cD(int P, int i);
template <>
__device__ __forceinline__ float cD<float>(int P, int i)
{
    return c_Df[P][i];
}
#ifndef MSOD_FP32_ONLY
template <>
__device__ __forceinline__ double cD<double>(int P, int i)
{
    return c_Dd[P][i];
}
#endif

enum { D_RHO = 0, D_T, D_U0, D_U1, D_U2, D_MUF, D_MUE, D_MUS, NDF };  // gathered planes
enum { X_GRHO = 0, X_TAUU, X_GT, X_TAU0, X_TAU1, X_TAU2, NX };        // flux vectors
// After the point pass a stage's gathered planes hold: 0 nu_e, 1 kappa_e, 2..6 partial sums.
enum { P_NUE = 0, P_KAP = 1, P_DR = 2 };

// Even-odd form of the call's 1-D derivative matrix D (TableScratch::EO and
// EOp, valid when eo_ok), per porder, for the xi and eta passes with one thread
// per line: with e_j, o_j the sums and differences of mirror-node values,
// (D v)[L_i] = S_i + T_i and (D v)[s'(L_i)] = S_i - T_i.  D^T, which the
// divergence passes apply, is centro-antisymmetric as well; its A and B are D's
// B and A transposed, and its centre row and column are D's centre column and
// row, so the same tables serve both.
__constant__ float c_DEO[MSOD_MAX_PORDER + 1][kTableEOMax];
__constant__ float2 c_DEOp[MSOD_MAX_PORDER + 1][kTableEOMax / 2];
// Bit P set: the even-odd xi / eta passes at porder P.  Measured (16.8 M-node
// meshes, even-odd / full matrix): porder 4 1.443 / 1.438 ms, porder 5 1.452 /
// 1.462 ms, porder 6 1.543 / 1.550 ms (not set), porder 7 1.809 / 1.852 ms.  The two forms round differently, and
// the diffusion's cancellation magnifies it: 1.1e-3 apart on plain_64's energy
// residual, each within the FP32 floor of the FP64 answer.
#ifndef DIFFU_EO
#define DIFFU_EO ((1 << 5) | (1 << 7))
#endif

// d = D v (TR = false) or D^T v (TR = true) along one line, FP32, even-odd
// form; the odd and even sums of a row advance together by packed FMAs.
template <int P, bool TR>
__device__ __forceinline__ void eo_line(const float (&v)[P + 1], float (&d)[P + 1])
{
    constexpr int Q = P + 1, M = Q / 2, MC = sod_centre(Q);
    constexpr bool ODD = (Q % 2) == 1;
    float ev[M > 0 ? M : 1], od[M > 0 ? M : 1];
#pragma unroll
    for (int j = 0; j < M; ++j) {
        ev[j] = v[sod_left(j)] + v[sod_mirror(Q, sod_left(j))];
        od[j] = v[sod_left(j)] - v[sod_mirror(Q, sod_left(j))];
    }
#pragma unroll
    for (int i = 0; i < M; ++i) {
        // (odd sum S_i, even sum T_i); D: A[i][j] o_j, B[i][j] e_j; D^T: B[j][i] o_j, A[j][i] e_j.
        const float mid = ODD ? c_DEO[P][2 * M * M + (TR ? M : 0) + i] * v[MC] : 0.0f;
        float sO, sE;
        if constexpr (!TR) {
            float2 s = make_float2(0.0f, mid);
#pragma unroll
            for (int j = 0; j < M; ++j) s = __ffma2_rn(c_DEOp[P][i * M + j], make_float2(od[j], ev[j]), s);
            sO = s.x;
            sE = s.y;
        } else {
            float2 s = make_float2(mid, 0.0f);  // (T_i, S_i)
#pragma unroll
            for (int j = 0; j < M; ++j) s = __ffma2_rn(c_DEOp[P][j * M + i], make_float2(ev[j], od[j]), s);
            sE = s.x;
            sO = s.y;
        }
        d[sod_left(i)] = sO + sE;
        d[sod_mirror(Q, sod_left(i))] = sO - sE;
    }
    if constexpr (ODD) {
        float sm = 0.0f;
#pragma unroll
        for (int j = 0; j < M; ++j) sm = fmaf(c_DEO[P][2 * M * M + (TR ? 0 : M) + j], od[j], sm);
        d[MC] = sm;
    }
}

// Pass 1, direction DIR: iso-parametric derivatives of rho, T, u0..2 at the
// thread's points, stored to planes sX[DIR*5 + f].
template <class G, int DIR, bool EO = false>
__device__ __forceinline__ void grad_pass(const LineThread<G> &lt, const typename G::real *__restrict__ sF,
                                          typename G::real *__restrict__ sX, const typename G::real *__restrict__ sD)
{
    using real = typename G::real;
    constexpr int P = G::P, Q = G::Q, QP = G::QP, R = G::R, NPL = G::NPL;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int base = lt.el * G::ES + line_off<DIR, Q, QP>(lt.la, lt.lb, 0);
    if constexpr (EO) {
        static_assert(G::S == 1 && sizeof(real) == 4, "even-odd passes: FP32, one thread per line");
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            float v[Q], d[Q];
#pragma unroll
            for (int c = 0; c < Q; ++c) v[c] = sF[f * NPL + base + c * OST];
            eo_line<P, false>(v, d);
#pragma unroll
            for (int r = 0; r < Q; ++r) sX[(DIR * 5 + f) * NPL + base + r * OST] = d[r];
        }
        return;
    }
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
template <class G, int DIR, bool FIRST, bool LAST, bool EO = false>
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
        real v[Q], dT[EO ? Q : 1];
#pragma unroll
        for (int c = 0; c < Q; ++c) v[c] = sX[(DIR * NX + x) * NPL + base + c * OST];
        if constexpr (EO) {
            static_assert(G::S == 1 && sizeof(real) == 4, "even-odd passes: FP32, one thread per line");
            eo_line<P, true>(v, dT);
        }
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            real s = (real)0;
            if constexpr (EO)
                s = dT[rr];
            else
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
// Bit P set: the gathers' group-invariant index arithmetic (lattice offsets,
// element-layout row offsets) computed once per thread, not per group, at
// three blocks per SM.  Porder 4 on 64^3 hexes: 1.391 against 1.439 ms;
// porder 5 on 51^3 1.455 against 1.446 ms (not set); porder 7 spills.
#ifndef DIFFU_GOFF
#define DIFFU_GOFF (1 << 4)
#endif
// Minimum blocks per SM in the launch bounds. The kernels with the fused zeta
// stage take 1, which lets the compiler spend registers (porder 4 without the
// gather offsets: 137 / 153 / 153 for the three viscosity sources; porder 5:
// 159-163); shared memory holds them to three blocks per SM and keeps the L1
// that the larger carveout of a fourth block would take (DIFFU_MINB4 = 4, 128
// registers: 1.90 ms against 1.50 ms, porder 4 on 64^3).  With the gather
// offsets (DIFFU_GOFF) they take 3: left free, the compiler would spend ~195
// registers (two blocks per SM).  The other kernels take 0, the
// block-size-only heuristic (a 1 there raised porder 6 from 115 to 154
// registers: one block per SM instead of two).
#ifndef DIFFU_MINB4
#define DIFFU_MINB4 1
#endif
template <class G>
constexpr int diffu_minb()
{
    return diffu_fusez<G>() ? ((sizeof(typename G::real) == 4 && ((DIFFU_GOFF >> G::P) & 1) != 0)
                                   ? 3
                                   : ((sizeof(typename G::real) == 4 && G::P == 4) ? DIFFU_MINB4 : 1))
                            : 0;
}

// kappa_e at a node (elem_diffu.f90:143-146).
template <typename real>
__device__ __forceinline__ real kappa_e(real muf, real me, real ms, real r, real Cp, real Pr)
{
    return muf * Cp / Pr + me * Cp / Pr + Cp * r * ms / (real)0.9;
}

// Zeta-stage He rows in flight two points ahead instead of one at the porders
// whose bit is set: porder 5 on 51^3 hexes 1.440 against 1.451 ms, porder 7 on
// 37^3 1.788 against 1.810 ms (32^3: 1.100 against 1.116 ms); porder 4 the
// same either way (1.438 / 1.437 ms), the one-call kernel slower (2.853
// against 2.844 ms), porder 6 within 0.4 % (1.544 against 1.550 ms; not set).
#ifndef DIFFU_HE_AHEAD2
#define DIFFU_HE_AHEAD2 ((1 << 5) | (1 << 7))
#endif
// Zeta stage of the fused form, one thread per zeta line (lt): the zeta
// derivatives at the line's points (from its nodal values in registers), the
// point pass there (the xi and eta fluxes go to sX for their divergence
// passes) and the zeta divergence of the zeta fluxes, which stay in registers;
// the partial sums start the divergence (planes P_DR.. of sFs).  he_row(c, h,
// gp) gives point c's He row and gpvol and is called one point ahead;
// mu_at(o, r) gives mu_e at lattice offset o of density r.
template <class G, class HeRow, class MuAt>
__device__ __forceinline__ void zeta_stage(const LineThread<G> &lt, typename G::real *__restrict__ sFs,
                                           typename G::real *__restrict__ sX, HeRow &&he_row, MuAt &&mu_at,
                                           typename G::real Cp, typename G::real Pr)
{
    using real = typename G::real;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, NPL = G::NPL;
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
    // Rows in flight one point ahead, or two (AHEAD2).
    constexpr bool AHEAD2 = ((DIFFU_HE_AHEAD2 >> G::P) & 1) != 0;
    real Hn[9], gpn, Hn2[9], gpn2;
    he_row(0, Hn, gpn);
    if (AHEAD2 && Q > 1) he_row(1, Hn2, gpn2);
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const int o = base + c * OST;
        real Hc[9], gc;
#pragma unroll
        for (int j = 0; j < 9; ++j) Hc[j] = Hn[j];
        gc = gpn;
        if constexpr (AHEAD2) {
#pragma unroll
            for (int j = 0; j < 9; ++j) Hn[j] = Hn2[j];
            gpn = gpn2;
            if (c + 2 < Q) he_row(c + 2, Hn2, gpn2);
        } else if (c + 1 < Q) {
            he_row(c + 1, Hn, gpn);
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
        const real me = mu_at(o, r);
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
        // rho and T of this point are in registers or no longer needed: their
        // planes take nu_e and kappa_e.
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

// L2 prefetches a group ahead, while a group is computed: 1 = the next
// group's He and gpvol spans (one bulk prefetch per span, by one thread);
// 2 = also its mu_e, mu_sgs rows (N rows of NE values, one prefetch per row
// each); 3 = also the node fields of its element points (its node ids are in
// registers by then); 0 = none.  Measured on 64^3 porder-4 hexes: 1.481 ms
// with none, 1.440 ms with the spans, 1.472 ms with the rows, 1.607 ms with
// the node fields as well (six scattered prefetches per element point cost
// more issue slots than the gather latency they hide); porder 5 on 51^3:
// 1.514 / 1.465 ms, porder 7 on 37^3: 1.922 / 1.838 ms (none / spans).
#ifndef DIFFU_PREFETCH
#define DIFFU_PREFETCH 1
#endif

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

}  // namespace
}  // namespace msod
