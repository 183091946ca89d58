// msod_convec.cuh -- device code of the plain hex convection: the line
// passes, their tables in the constant bank and the launch configuration
// per porder.  Included by the convection kernel (msod_convec.cu) and the
// fused convection + diffusion kernel (msod_fused.cu); each translation unit
// holds its own copy of the constant-bank tables and fills it before its
// launches.
#pragma once

#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

#ifndef CONVEC_MINB
#define CONVEC_MINB 4
#endif
#ifndef CONVEC_MINB5
#define CONVEC_MINB5 3
#endif

namespace msod {
namespace {

// 1-D derivative matrices of the current call, per porder (copied from the
// per-call table area before the launch): with one thread per line, the
// contraction FMAs take their coefficients as constant-bank operands.
// A translation unit that defines MSOD_FP32_ONLY (the one-call kernel) holds
// no FP64 copy: the constant bank of a unit is 64 KB.
__constant__ float c_CDf[MSOD_MAX_PORDER + 1][kTableDMax];
#ifndef MSOD_FP32_ONLY
__constant__ double c_CDd[MSOD_MAX_PORDER + 1][kTableDMax];
#endif

template <typename real>
__device__ __forceinline__ real cCD(int P, int i);
template <>
__device__ __forceinline__ float cCD<float>(int P, int i)
{
    return c_CDf[P][i];
}
#ifndef MSOD_FP32_ONLY
template <>
__device__ __forceinline__ double cCD<double>(int P, int i)
{
    return c_CDd[P][i];
}
#endif

// Elements per block at porder 5 in FP32 (36 threads per element): 3 fill a
// 128-thread block (with the packed passes at three blocks per SM: 3.05 ms
// against 3.62 ms for seven elements in a 256-thread block at one block per
// SM, 64^3 hexes).
#ifndef CONVEC_NE5
#define CONVEC_NE5 3
#endif
// Threads per line of the FP32 convection at porders 6 and 7 (0: the
// line-geometry default, two) and elements per block there (0: the default).
// One thread per line lets porder 6 take the compact even-odd pass and
// porder 7 the packed row-pair passes.  Measured on 32^3 hexes (A/B/A): porder
// 6 0.823 ms against 1.255 ms with two threads per line (three elements per
// block: 1.007 ms); porder 7 1.206 ms against 1.390 ms (one element per block:
// 1.229 ms).
#ifndef CONVEC_S6
#define CONVEC_S6 1
#endif
#ifndef CONVEC_S7
#define CONVEC_S7 1
#endif
#ifndef CONVEC_NE6
#define CONVEC_NE6 2
#endif
#ifndef CONVEC_NE7
#define CONVEC_NE7 2
#endif
#ifndef CONVEC_S8
#define CONVEC_S8 0
#endif
#ifndef CONVEC_NE8
#define CONVEC_NE8 0
#endif
template <typename real, int P>
constexpr int convec_necap()
{
    return sizeof(real) != 4                ? 64
           : P == 5                         ? CONVEC_NE5
           : (P == 6 && CONVEC_NE6 > 0)     ? CONVEC_NE6
           : (P == 7 && CONVEC_NE7 > 0)     ? CONVEC_NE7
           : (P == 8 && CONVEC_NE8 > 0)     ? CONVEC_NE8
                                            : 64;
}
template <typename real, int P>
constexpr int convec_s()
{
    return sizeof(real) != 4 ? 0 : P == 6 ? CONVEC_S6 : P == 7 ? CONVEC_S7 : P == 8 ? CONVEC_S8 : 0;
}
template <typename real, int P>
using ConvecGeom = LineGeom<real, P, convec_necap<real, P>(), convec_s<real, P>()>;

// Row pairs of the FP32 matrices (packed contractions), per porder:
// c_CDp[P][(d*Q + c)*H + m] = (D[d][2m][c], D[d][2m+1][c]), H = (Q+1)/2.
__constant__ float2 c_CDp[MSOD_MAX_PORDER + 1][kTableDPairMax / 2];

// Packed (f32x2) line passes: 0 never; 1 at odd porders >= 3, where the Q
// rows pair with no padded row (porder 3: 1.27 -> 1.23 ms on 80^3 hexes,
// porder 5: 3.62 -> 3.05 ms on 64^3; the padded pair makes porders 2 and 4
// slower: 1.83 -> 2.59 and 1.64 -> 2.37 ms); 2 whenever FP32 runs one thread
// per line.
#ifndef CONVEC_X2
#define CONVEC_X2 1
#endif

// Threads take their lines from the bank-aware map (LineMap) with one thread
// per line, up to this porder (0: never); other porders keep the lines of
// consecutive elements side by side.  Measured with the three full-matrix
// passes: plain_64 1.611 against 1.640 ms; porder 5 on 64^3 hexes 3.01
// either way.
#ifndef CONVEC_LINEMAP
#define CONVEC_LINEMAP 4
#endif

// The thread's line in direction dir.
template <class G>
__device__ __forceinline__ LineThread<G> convec_line(int tid, int dir)
{
    if constexpr (G::P <= CONVEC_LINEMAP && G::S == 1)
        return LineThread<G>(kLineMap<G>.code[dir][tid], true);
    else
        return LineThread<G>(tid);
}

template <int Q, typename real>
__device__ __forceinline__ real pick(const real (&a)[Q], int i)
{
    real v = a[0];
#pragma unroll
    for (int c = 1; c < Q; ++c) v = (i == c) ? a[c] : v;
    return v;
}

enum { F_RHO = 0, F_P, F_E, F_U0, F_U1, F_U2, F_Q0, F_Q1, F_Q2, NFIELD };
enum { A_M = 0, A_MOM0, A_MOM1, A_MOM2, A_E, A_DIVU, A_DIVQ, NACC };

// Planes of the node fields in the shared-memory lattice: the convection
// kernel's own order, or any other a kernel that shares the lattice lays out
// (u and q take three consecutive planes each).
struct ConvPlanes {
    static constexpr int RHO = F_RHO, PR = F_P, EN = F_E, U0 = F_U0, Q0 = F_Q0;
};

template <typename real, int P, int DIR, bool STAGED, class L = ConvPlanes>
__device__ __forceinline__ void convec_pass(const real *__restrict__ sF, real *__restrict__ sA,
                                            const real *__restrict__ sD, const int *__restrict__ sNode,
                                            const int *__restrict__ sPerm, const real *__restrict__ He,
                                            const real *__restrict__ gpvol, int e0, int nelem, int npoin,
                                            real *__restrict__ Rmass, real *__restrict__ Rmom,
                                            real *__restrict__ Rener)
{
    using G = ConvecGeom<real, P>;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, NE = G::NE, S = G::S, R = G::R, TPE = G::TPE, N = G::N;
    constexpr int NPL = NE * ES;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);

    const LineThread<G> lt = convec_line<G>(threadIdx.x, DIR);
    if (!lt.active) return;
    const int el = lt.el, la = lt.la, lb = lt.lb;
    const int e = e0 + el;
    const int base = el * ES + line_off<DIR, Q, QP>(la, lb, 0);

    // Nodal values along the line.
    real rho_[Q], p_[Q], H_[Q], rH_[Q], u_[3][Q], q_[3][Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const int o = base + c * OST;
        rho_[c] = sF[L::RHO * NPL + o];
        p_[c] = sF[L::PR * NPL + o];
        const real Ev = sF[L::EN * NPL + o];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            u_[i][c] = sF[(L::U0 + i) * NPL + o];
            q_[i][c] = sF[(L::Q0 + i) * NPL + o];
        }
        const real k = (real)0.5 * (u_[0][c] * u_[0][c] + u_[1][c] * u_[1][c] + u_[2][c] * u_[2][c]);
        H_[c] = Ev + k;
        rH_[c] = rho_[c] * H_[c];
    }

    // Per owned point: derivative-matrix row, He column DIR, coefficients.
    const int r0 = lt.r0;
    real Dm[R][Q], h[R][3], own_rho[R], own_H[R], own_rH[R], own_u[R][3], own_q[R][3], cu[R], cq[R];
    real acc[R][NACC];
    int gidx[R];
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int r = r0 + rr;
        const bool ok = (R * S == Q) || r < Q;
        const int rc = ok ? r : 0;
        if (S > 1)
#pragma unroll
            for (int c = 0; c < Q; ++c) Dm[rr][c] = sD[(DIR * Q + rc) * Q + c];
        const int a = sPerm[line_lat<DIR, Q>(la, lb, rc)];
        gidx[rr] = a;
        const real *hp = STAGED ? He + (el * N + a) * 9 + DIR * 3 : He + ((size_t)(e < nelem ? e : 0) * N + a) * 9 + DIR * 3;
#pragma unroll
        for (int i = 0; i < 3; ++i) h[rr][i] = STAGED ? hp[i] : ldg(hp + i);
        own_rho[rr] = pick<Q>(rho_, rc);
        own_H[rr] = pick<Q>(H_, rc);
        own_rH[rr] = pick<Q>(rH_, rc);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            own_u[rr][i] = pick<Q>(u_[i], rc);
            own_q[rr][i] = pick<Q>(q_[i], rc);
        }
        cu[rr] = own_u[rr][0] * h[rr][0] + own_u[rr][1] * h[rr][1] + own_u[rr][2] * h[rr][2];
        cq[rr] = own_q[rr][0] * h[rr][0] + own_q[rr][1] * h[rr][1] + own_q[rr][2] * h[rr][2];
        if (DIR == 0) {
#pragma unroll
            for (int k = 0; k < NACC; ++k) acc[rr][k] = (real)0;
        } else {
            const int o = base + rc * OST;
#pragma unroll
            for (int k = 0; k < NACC; ++k) acc[rr][k] = sA[k * NPL + o];
        }
    }

    real d[R], f[Q];
    auto deriv = [&](const real(&v)[Q]) {
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            real s = (real)0;
#pragma unroll
            for (int c = 0; c < Q; ++c) s = fma(S == 1 ? cCD<real>(P, (DIR * Q + rr) * Q + c) : Dm[rr][c], v[c], s);
            d[rr] = s;
        }
    };
    const real h4 = (real)0.25, h2 = (real)0.5;

    // rho: mass 1/2 u.grad rho, momentum 1/4 u_i u.grad rho, energy 1/4 H u.grad rho
    deriv(rho_);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const real t = cu[rr] * d[rr];
        acc[rr][A_M] = fma(h2, t, acc[rr][A_M]);
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[rr][A_MOM0 + i] = fma(h4 * own_u[rr][i], t, acc[rr][A_MOM0 + i]);
        acc[rr][A_E] = fma(h4 * own_H[rr], t, acc[rr][A_E]);
    }
    // p: grad p
    deriv(p_);
#pragma unroll
    for (int rr = 0; rr < R; ++rr)
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[rr][A_MOM0 + i] = fma(h[rr][i], d[rr], acc[rr][A_MOM0 + i]);
    // u_i: div u, 1/4 q.grad u_i ; q_i: div q, 1/4 u.grad q_i
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        deriv(u_[i]);
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            acc[rr][A_DIVU] = fma(h[rr][i], d[rr], acc[rr][A_DIVU]);
            acc[rr][A_MOM0 + i] = fma(h4 * cq[rr], d[rr], acc[rr][A_MOM0 + i]);
        }
        deriv(q_[i]);
#pragma unroll
        for (int rr = 0; rr < R; ++rr) {
            acc[rr][A_DIVQ] = fma(h[rr][i], d[rr], acc[rr][A_DIVQ]);
            acc[rr][A_MOM0 + i] = fma(h4 * cu[rr], d[rr], acc[rr][A_MOM0 + i]);
        }
    }
    // F_ij = q_i u_j: 1/4 div F_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = q_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int rr = 0; rr < R; ++rr) acc[rr][A_MOM0 + i] = fma(h4 * h[rr][j], d[rr], acc[rr][A_MOM0 + i]);
        }
    // Fuu_ij = u_i u_j (symmetric): 1/4 rho div Fuu_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = u_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int rr = 0; rr < R; ++rr) {
                const real rd = h4 * own_rho[rr] * d[rr];
                acc[rr][A_MOM0 + i] = fma(h[rr][j], rd, acc[rr][A_MOM0 + i]);
                if (i != j) acc[rr][A_MOM0 + j] = fma(h[rr][i], rd, acc[rr][A_MOM0 + j]);
            }
        }
    // H: 1/4 q.grad H ; rho H: 1/4 u.grad(rho H)
    deriv(H_);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) acc[rr][A_E] = fma(h4 * cq[rr], d[rr], acc[rr][A_E]);
    deriv(rH_);
#pragma unroll
    for (int rr = 0; rr < R; ++rr) acc[rr][A_E] = fma(h4 * cu[rr], d[rr], acc[rr][A_E]);
    // rho H u_i: 1/4 div(rho H u) ; H u_i: 1/4 rho div(H u)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = rH_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int rr = 0; rr < R; ++rr) acc[rr][A_E] = fma(h4 * h[rr][i], d[rr], acc[rr][A_E]);
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = H_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int rr = 0; rr < R; ++rr) acc[rr][A_E] = fma(h4 * own_rho[rr] * h[rr][i], d[rr], acc[rr][A_E]);
    }

#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        const int r = r0 + rr;
        if (!((R * S == Q) || r < Q)) continue;
        const int o = base + r * OST;
        if (DIR < 2) {
#pragma unroll
            for (int k = 0; k < NACC; ++k) sA[k * NPL + o] = acc[rr][k];
        } else {
            const int node = sNode[o];
            if (node < 0 || e >= nelem) continue;
            const real divU = acc[rr][A_DIVU], divQ = acc[rr][A_DIVQ];
            const real gp = STAGED ? gpvol[el * N + gidx[rr]] : ldg(gpvol + (size_t)e * N + gidx[rr]);
            const real rm = acc[rr][A_M] + h2 * (divQ + own_rho[rr] * divU);
            const real re = acc[rr][A_E] + h4 * (own_H[rr] * divQ + own_rH[rr] * divU);
            red_add(Rmass + node, gp * rm);
            red_add(Rener + node, gp * re);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const real rmom = acc[rr][A_MOM0 + i] + h4 * (own_u[rr][i] * divQ + own_q[rr][i] * divU);
                red_add(Rmom + (size_t)i * npoin + node, gp * rmom);
            }
        }
    }
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// The pass above for FP32 with one thread per line, two points of the line
// per instruction: rows (2m, 2m+1) are the two halves of fma.rn.f32x2 /
// mul.rn.f32x2 operands, operation for operation the scalar pass (a line of
// odd length pads its last pair with a zero row that is never stored).
template <int P, int DIR, bool STAGED, class L = ConvPlanes>
__device__ __forceinline__ void convec_pass_x2(const float *__restrict__ sF, float *__restrict__ sA,
                                               const int *__restrict__ sNode, const int *__restrict__ sPerm,
                                               const float *__restrict__ He, const float *__restrict__ gpvol, int e0,
                                               int nelem, int npoin, float *__restrict__ Rmass,
                                               float *__restrict__ Rmom, float *__restrict__ Rener)
{
    using G = ConvecGeom<float, P>;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, NE = G::NE, TPE = G::TPE, N = G::N;
    constexpr int H = (Q + 1) / 2;
    constexpr int NPL = NE * ES;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    static_assert(G::S == 1, "one thread per line");

    const LineThread<G> lt = convec_line<G>(threadIdx.x, DIR);
    if (!lt.active) return;
    const int el = lt.el, la = lt.la, lb = lt.lb;
    const int e = e0 + el;
    const int base = el * ES + line_off<DIR, Q, QP>(la, lb, 0);

    float rho_[Q], p_[Q], H_[Q], rH_[Q], u_[3][Q], q_[3][Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const int o = base + c * OST;
        rho_[c] = sF[L::RHO * NPL + o];
        p_[c] = sF[L::PR * NPL + o];
        const float Ev = sF[L::EN * NPL + o];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            u_[i][c] = sF[(L::U0 + i) * NPL + o];
            q_[i][c] = sF[(L::Q0 + i) * NPL + o];
        }
        const float k = 0.5f * (u_[0][c] * u_[0][c] + u_[1][c] * u_[1][c] + u_[2][c] * u_[2][c]);
        H_[c] = Ev + k;
        rH_[c] = rho_[c] * H_[c];
    }
    auto pr2 = [&](const float(&a)[Q], int m) { return make_float2(a[2 * m], 2 * m + 1 < Q ? a[2 * m + 1] : 0.0f); };

    // Per point pair: He column DIR, u.h and q.h, accumulators.
    float2 h[H][3], cu[H], cq[H], acc[H][NACC];
    int gidx[2 * H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
        float hv[2][3];
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int r = 2 * m + t;
            if (r < Q) {
                const int a = sPerm[line_lat<DIR, Q>(la, lb, r)];
                gidx[r] = a;
                const float *hp = STAGED ? He + (el * N + a) * 9 + DIR * 3
                                         : He + ((size_t)(e < nelem ? e : 0) * N + a) * 9 + DIR * 3;
#pragma unroll
                for (int i = 0; i < 3; ++i) hv[t][i] = STAGED ? hp[i] : ldg(hp + i);
            } else {
                gidx[r] = 0;
#pragma unroll
                for (int i = 0; i < 3; ++i) hv[t][i] = 0.0f;
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) h[m][i] = make_float2(hv[0][i], hv[1][i]);
        const float2 u0 = pr2(u_[0], m), u1 = pr2(u_[1], m), u2 = pr2(u_[2], m);
        const float2 q0 = pr2(q_[0], m), q1 = pr2(q_[1], m), q2 = pr2(q_[2], m);
        cu[m] = fma2(u2, h[m][2], fma2(u1, h[m][1], mul2(u0, h[m][0])));
        cq[m] = fma2(q2, h[m][2], fma2(q1, h[m][1], mul2(q0, h[m][0])));
#pragma unroll
        for (int k = 0; k < NACC; ++k) {
            if (DIR == 0) {
                acc[m][k] = f2(0.0f);
            } else {
                const int r1 = 2 * m + 1 < Q ? 2 * m + 1 : 2 * m;
                acc[m][k] = make_float2(sA[k * NPL + base + 2 * m * OST], sA[k * NPL + base + r1 * OST]);
            }
        }
    }

    float2 d[H];
    float f[Q];
    auto deriv = [&](const float(&v)[Q]) {
#pragma unroll
        for (int m = 0; m < H; ++m) d[m] = f2(0.0f);
#pragma unroll
        for (int c = 0; c < Q; ++c) {
            const float2 vv = f2(v[c]);
#pragma unroll
            for (int m = 0; m < H; ++m) d[m] = fma2(c_CDp[P][(DIR * Q + c) * H + m], vv, d[m]);
        }
    };
    const float2 h4 = f2(0.25f), h2 = f2(0.5f);

    // rho: mass 1/2 u.grad rho, momentum 1/4 u_i u.grad rho, energy 1/4 H u.grad rho
    deriv(rho_);
#pragma unroll
    for (int m = 0; m < H; ++m) {
        const float2 t = mul2(cu[m], d[m]);
        acc[m][A_M] = fma2(h2, t, acc[m][A_M]);
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[m][A_MOM0 + i] = fma2(mul2(h4, pr2(u_[i], m)), t, acc[m][A_MOM0 + i]);
        acc[m][A_E] = fma2(mul2(h4, pr2(H_, m)), t, acc[m][A_E]);
    }
    // p: grad p
    deriv(p_);
#pragma unroll
    for (int m = 0; m < H; ++m)
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[m][A_MOM0 + i] = fma2(h[m][i], d[m], acc[m][A_MOM0 + i]);
    // u_i: div u, 1/4 q.grad u_i ; q_i: div q, 1/4 u.grad q_i
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        deriv(u_[i]);
#pragma unroll
        for (int m = 0; m < H; ++m) {
            acc[m][A_DIVU] = fma2(h[m][i], d[m], acc[m][A_DIVU]);
            acc[m][A_MOM0 + i] = fma2(mul2(h4, cq[m]), d[m], acc[m][A_MOM0 + i]);
        }
        deriv(q_[i]);
#pragma unroll
        for (int m = 0; m < H; ++m) {
            acc[m][A_DIVQ] = fma2(h[m][i], d[m], acc[m][A_DIVQ]);
            acc[m][A_MOM0 + i] = fma2(mul2(h4, cu[m]), d[m], acc[m][A_MOM0 + i]);
        }
    }
    // F_ij = q_i u_j: 1/4 div F_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = q_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int m = 0; m < H; ++m) acc[m][A_MOM0 + i] = fma2(mul2(h4, h[m][j]), d[m], acc[m][A_MOM0 + i]);
        }
    // Fuu_ij = u_i u_j (symmetric): 1/4 rho div Fuu_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = u_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int m = 0; m < H; ++m) {
                const float2 rd = mul2(mul2(h4, pr2(rho_, m)), d[m]);
                acc[m][A_MOM0 + i] = fma2(h[m][j], rd, acc[m][A_MOM0 + i]);
                if (i != j) acc[m][A_MOM0 + j] = fma2(h[m][i], rd, acc[m][A_MOM0 + j]);
            }
        }
    // H: 1/4 q.grad H ; rho H: 1/4 u.grad(rho H)
    deriv(H_);
#pragma unroll
    for (int m = 0; m < H; ++m) acc[m][A_E] = fma2(mul2(h4, cq[m]), d[m], acc[m][A_E]);
    deriv(rH_);
#pragma unroll
    for (int m = 0; m < H; ++m) acc[m][A_E] = fma2(mul2(h4, cu[m]), d[m], acc[m][A_E]);
    // rho H u_i: 1/4 div(rho H u) ; H u_i: 1/4 rho div(H u)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = rH_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int m = 0; m < H; ++m) acc[m][A_E] = fma2(mul2(h4, h[m][i]), d[m], acc[m][A_E]);
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = H_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int m = 0; m < H; ++m) acc[m][A_E] = fma2(mul2(mul2(h4, pr2(rho_, m)), h[m][i]), d[m], acc[m][A_E]);
    }

#pragma unroll
    for (int r = 0; r < Q; ++r) {
        const int m = r >> 1;
        float a[NACC];
#pragma unroll
        for (int k = 0; k < NACC; ++k) a[k] = (r & 1) ? acc[m][k].y : acc[m][k].x;
        const int o = base + r * OST;
        if (DIR < 2) {
#pragma unroll
            for (int k = 0; k < NACC; ++k) sA[k * NPL + o] = a[k];
        } else {
            const int node = sNode[o];
            if (node < 0 || e >= nelem) continue;
            const float divU = a[A_DIVU], divQ = a[A_DIVQ];
            const float gp = STAGED ? gpvol[el * N + gidx[r]] : ldg(gpvol + (size_t)e * N + gidx[r]);
            const float rm = a[A_M] + 0.5f * (divQ + rho_[r] * divU);
            const float re = a[A_E] + 0.25f * (H_[r] * divQ + rH_[r] * divU);
            red_add(Rmass + node, gp * rm);
            red_add(Rener + node, gp * re);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float rmom = a[A_MOM0 + i] + 0.25f * (u_[i][r] * divQ + q_[i][r] * divU);
                red_add(Rmom + (size_t)i * npoin + node, gp * rmom);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The compact pass (FP32, one thread per line, scalar porders): one copy of
// the pass code serves the three directions (the direction is a run-time
// value), and the contraction takes the even-odd form of the derivative
// matrix.  Both need what the reference's tables provide: one 1-D matrix for
// the three directions, centro-antisymmetric (table_prep_kernel checks it per
// call, TableScratch::eo_ok); other tables take the three unrolled passes.
// ---------------------------------------------------------------------------
// 1 = even-odd contraction (porder 4: 20 instead of 25 FP32 operations per
// line and field), 0 = the full matrix of direction 0.  Measured on plain_64
// (unrolled passes, four blocks per SM): 1.48 ms against 1.62 ms for the
// three full-matrix passes; porder 2 on 120^3 hexes 1.71 against 1.79 ms.
// The contraction packed over pairs of fields (fma.rn.f32x2 on the even-odd
// coefficients, no padding) measured slower, 1.51 ms at three blocks per SM
// and 1.87 ms at four (its pairs of derivatives spill at 128 registers).
#ifndef CONVEC_EO
#define CONVEC_EO 1
#endif
// The even-odd contraction's odd and even sums of a row advanced together by
// packed FMAs (fma.rn.f32x2 with the (A, B) coefficient pair from the constant
// bank): the same operations in the same order per lane, so the same results
// as the scalar form, in fewer instructions.  Bit P set: packed at porder P.
// Measured (16.8 M-node meshes, packed / scalar): porder 2 2.041 / 2.135 ms,
// porder 4 1.451 / 1.462 ms, porder 6 (persistent, 255 registers) 1.846 /
// 1.718 ms.
#ifndef CONVEC_EO2
#define CONVEC_EO2 ((1 << 2) | (1 << 4))
#endif
// 1 = the direction loop is not unrolled (one copy of the pass code: a third
// of the instruction footprint), 0 = unrolled.  Measured on plain_64: the
// run-time direction loses (1.80 ms at four blocks per SM, 1.60 ms at three)
// against the unrolled passes (1.48 ms): the kernel is not bound by
// instruction fetch.
#ifndef CONVEC_RTDIR
#define CONVEC_RTDIR 0
#endif
// 1 = the compact pass runs when the call's tables allow it, 0 = never.
#ifndef CONVEC_COMPACT
#define CONVEC_COMPACT 1
#endif

__constant__ float c_CEO[MSOD_MAX_PORDER + 1][kTableEOMax];
// The (A, B) pairs of the even-odd form (TableScratch::EOp), per porder.
__constant__ float2 c_CEOp[MSOD_MAX_PORDER + 1][kTableEOMax / 2];

template <int Q, int QP>
__device__ __forceinline__ int line_off_rt(int dir, int la, int lb, int r)
{
    return dir == 0 ? (lb * Q + la) * QP + r : (dir == 1 ? (lb * Q + r) * QP + la : (r * Q + lb) * QP + la);
}
template <int Q>
__device__ __forceinline__ int line_lat_rt(int dir, int la, int lb, int r)
{
    return line_off_rt<Q, Q>(dir, la, lb, r);
}

template <int P, class L = ConvPlanes>
__device__ __forceinline__ void convec_pass_compact(int dir, const float *__restrict__ sF, float *__restrict__ sA,
                                                    const int *__restrict__ sNode, const int *__restrict__ sPerm,
                                                    const float *__restrict__ He, const float *__restrict__ gpvol,
                                                    int e0, int nelem, int npoin, float *__restrict__ Rmass,
                                                    float *__restrict__ Rmom, float *__restrict__ Rener)
{
    using G = ConvecGeom<float, P>;
    constexpr int Q = G::Q, QP = G::QP, ES = G::ES, N = G::N, NPL = G::NE * G::ES;
    constexpr int M = Q / 2, MC = sod_centre(Q);
    constexpr bool ODD = (Q % 2) == 1;
    static_assert(G::S == 1, "one thread per line");
    const LineThread<G> lt = convec_line<G>(threadIdx.x, dir);
    if (!lt.active) return;
    const int el = lt.el, la = lt.la, lb = lt.lb;
    const int e = e0 + el;
    const int ost = dir == 0 ? 1 : (dir == 1 ? QP : Q * QP);
    const int base = el * ES + line_off_rt<Q, QP>(dir, la, lb, 0);

    float rho_[Q], p_[Q], H_[Q], rH_[Q], u_[3][Q], q_[3][Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const int o = base + c * ost;
        rho_[c] = sF[L::RHO * NPL + o];
        p_[c] = sF[L::PR * NPL + o];
        const float Ev = sF[L::EN * NPL + o];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            u_[i][c] = sF[(L::U0 + i) * NPL + o];
            q_[i][c] = sF[(L::Q0 + i) * NPL + o];
        }
        const float k = 0.5f * (u_[0][c] * u_[0][c] + u_[1][c] * u_[1][c] + u_[2][c] * u_[2][c]);
        H_[c] = Ev + k;
        rH_[c] = rho_[c] * H_[c];
    }

    float h[Q][3], cu[Q], cq[Q], acc[Q][NACC];
    int gidx[Q];
#pragma unroll
    for (int r = 0; r < Q; ++r) {
        const int a = sPerm[line_lat_rt<Q>(dir, la, lb, r)];
        gidx[r] = a;
        const float *hp = He + ((size_t)(e < nelem ? e : 0) * N + a) * 9 + dir * 3;
#pragma unroll
        for (int i = 0; i < 3; ++i) h[r][i] = ldg(hp + i);
        cu[r] = u_[0][r] * h[r][0] + u_[1][r] * h[r][1] + u_[2][r] * h[r][2];
        cq[r] = q_[0][r] * h[r][0] + q_[1][r] * h[r][1] + q_[2][r] * h[r][2];
        const int o = base + r * ost;
#pragma unroll
        for (int k = 0; k < NACC; ++k) acc[r][k] = dir == 0 ? 0.0f : sA[k * NPL + o];
    }

    float d[Q], f[Q];
    auto deriv = [&](const float(&v)[Q]) {
        if constexpr (CONVEC_EO != 0) {
            float ev[M > 0 ? M : 1], od[M > 0 ? M : 1];
#pragma unroll
            for (int j = 0; j < M; ++j) {
                ev[j] = v[sod_left(j)] + v[sod_mirror(Q, sod_left(j))];
                od[j] = v[sod_left(j)] - v[sod_mirror(Q, sod_left(j))];
            }
#pragma unroll
            for (int i = 0; i < M; ++i) {
                float sO = 0.0f, sE = ODD ? c_CEO[P][2 * M * M + i] * v[MC] : 0.0f;
                if constexpr (((CONVEC_EO2 >> P) & 1) != 0) {
                    float2 s = make_float2(sO, sE);
#pragma unroll
                    for (int j = 0; j < M; ++j) s = __ffma2_rn(c_CEOp[P][i * M + j], make_float2(od[j], ev[j]), s);
                    sO = s.x;
                    sE = s.y;
                } else {
#pragma unroll
                    for (int j = 0; j < M; ++j) {
                        sO = fmaf(c_CEO[P][i * M + j], od[j], sO);
                        sE = fmaf(c_CEO[P][M * M + i * M + j], ev[j], sE);
                    }
                }
                d[sod_left(i)] = sO + sE;
                d[sod_mirror(Q, sod_left(i))] = sO - sE;
            }
            if constexpr (ODD) {
                float sm = 0.0f;
#pragma unroll
                for (int j = 0; j < M; ++j) sm = fmaf(c_CEO[P][2 * M * M + M + j], od[j], sm);
                d[MC] = sm;
            }
        } else {
#pragma unroll
            for (int r = 0; r < Q; ++r) {
                float sd = 0.0f;
#pragma unroll
                for (int c = 0; c < Q; ++c) sd = fmaf(cCD<float>(P, r * Q + c), v[c], sd);
                d[r] = sd;
            }
        }
    };

    // rho: mass 1/2 u.grad rho, momentum 1/4 u_i u.grad rho, energy 1/4 H u.grad rho
    deriv(rho_);
#pragma unroll
    for (int r = 0; r < Q; ++r) {
        const float t4 = 0.25f * (cu[r] * d[r]);
        acc[r][A_M] = fmaf(2.0f, t4, acc[r][A_M]);
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[r][A_MOM0 + i] = fmaf(u_[i][r], t4, acc[r][A_MOM0 + i]);
        acc[r][A_E] = fmaf(H_[r], t4, acc[r][A_E]);
    }
    // p: grad p
    deriv(p_);
#pragma unroll
    for (int r = 0; r < Q; ++r)
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[r][A_MOM0 + i] = fmaf(h[r][i], d[r], acc[r][A_MOM0 + i]);
    // u_i: div u, 1/4 q.grad u_i ; q_i: div q, 1/4 u.grad q_i
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        deriv(u_[i]);
#pragma unroll
        for (int r = 0; r < Q; ++r) {
            acc[r][A_DIVU] = fmaf(h[r][i], d[r], acc[r][A_DIVU]);
            acc[r][A_MOM0 + i] = fmaf(0.25f * cq[r], d[r], acc[r][A_MOM0 + i]);
        }
        deriv(q_[i]);
#pragma unroll
        for (int r = 0; r < Q; ++r) {
            acc[r][A_DIVQ] = fmaf(h[r][i], d[r], acc[r][A_DIVQ]);
            acc[r][A_MOM0 + i] = fmaf(0.25f * cu[r], d[r], acc[r][A_MOM0 + i]);
        }
    }
    // F_ij = q_i u_j: 1/4 div F_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = q_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int r = 0; r < Q; ++r) acc[r][A_MOM0 + i] = fmaf(0.25f * h[r][j], d[r], acc[r][A_MOM0 + i]);
        }
    // Fuu_ij = u_i u_j (symmetric): 1/4 rho div Fuu_i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
#pragma unroll
            for (int c = 0; c < Q; ++c) f[c] = u_[i][c] * u_[j][c];
            deriv(f);
#pragma unroll
            for (int r = 0; r < Q; ++r) {
                const float rd = (0.25f * rho_[r]) * d[r];
                acc[r][A_MOM0 + i] = fmaf(h[r][j], rd, acc[r][A_MOM0 + i]);
                if (i != j) acc[r][A_MOM0 + j] = fmaf(h[r][i], rd, acc[r][A_MOM0 + j]);
            }
        }
    // H: 1/4 q.grad H ; rho H: 1/4 u.grad(rho H)
    deriv(H_);
#pragma unroll
    for (int r = 0; r < Q; ++r) acc[r][A_E] = fmaf(0.25f * cq[r], d[r], acc[r][A_E]);
    deriv(rH_);
#pragma unroll
    for (int r = 0; r < Q; ++r) acc[r][A_E] = fmaf(0.25f * cu[r], d[r], acc[r][A_E]);
    // rho H u_i: 1/4 div(rho H u) ; H u_i: 1/4 rho div(H u)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = rH_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int r = 0; r < Q; ++r) acc[r][A_E] = fmaf(0.25f * h[r][i], d[r], acc[r][A_E]);
#pragma unroll
        for (int c = 0; c < Q; ++c) f[c] = H_[c] * u_[i][c];
        deriv(f);
#pragma unroll
        for (int r = 0; r < Q; ++r) acc[r][A_E] = fmaf((0.25f * rho_[r]) * h[r][i], d[r], acc[r][A_E]);
    }

#pragma unroll
    for (int r = 0; r < Q; ++r) {
        const int o = base + r * ost;
        if (dir < 2) {
#pragma unroll
            for (int k = 0; k < NACC; ++k) sA[k * NPL + o] = acc[r][k];
        } else {
            const int node = sNode[o];
            if (node < 0 || e >= nelem) continue;
            const float divU = acc[r][A_DIVU], divQ = acc[r][A_DIVQ];
            const float gp = ldg(gpvol + (size_t)e * N + gidx[r]);
            const float rm = acc[r][A_M] + 0.5f * (divQ + rho_[r] * divU);
            const float re = acc[r][A_E] + 0.25f * (H_[r] * divQ + rH_[r] * divU);
            red_add(Rmass + node, gp * rm);
            red_add(Rener + node, gp * re);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float rmom = acc[r][A_MOM0 + i] + 0.25f * (u_[i][r] * divQ + q_[i][r] * divU);
                red_add(Rmom + (size_t)i * npoin + node, gp * rmom);
            }
        }
    }
}

template <typename real, int P>
constexpr bool convec_packed()
{
    return (CONVEC_X2 == 2 || (CONVEC_X2 == 1 && P % 2 == 1 && P >= 3)) && sizeof(real) == 4 &&
           ConvecGeom<real, P>::S == 1;
}

template <typename real, int P, int DIR, bool STAGED, class L = ConvPlanes>
__device__ __forceinline__ void convec_dir(const real *sF, real *sA, const real *sD, const int *sNode,
                                           const int *sPerm, const real *He, const real *gpvol, int e0, int nelem,
                                           int npoin, real *Rmass, real *Rmom, real *Rener)
{
    if constexpr (convec_packed<real, P>())
        convec_pass_x2<P, DIR, STAGED, L>(sF, sA, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom, Rener);
    else
        convec_pass<real, P, DIR, STAGED, L>(sF, sA, sD, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom,
                                          Rener);
}

// He and gpvol of a block's elements prefetched into L2 at the block's start
// (one bulk prefetch per span, by one thread; 0 = no prefetch).  64^3
// porder-4 hexes: 1.468 ms against 1.480 ms; porder 5 on 51^3: 1.532
// against 1.545 ms.
#ifndef CONVEC_PREFETCH
#define CONVEC_PREFETCH 1
#endif
// He and gpvol of a block's elements staged in shared memory by bulk copies
// (the group's spans of He(3,3,ngaus,nelem) and gpvol(ngaus,nelem) are
// contiguous): 1 = FP32 kernels, 0 = per-point loads from global memory.
// Measured slower and off: plain_64 1.95 ms against 1.61 ms (three blocks per
// SM by shared memory instead of four, and the gmsh-ordered He records read
// from shared memory by line threads conflict on banks); porder 5 on 64^3
// hexes 3.10 against 3.01 ms.
#ifndef CONVEC_HE_BULK
#define CONVEC_HE_BULK 0
#endif
template <typename real>
constexpr bool convec_staged()
{
    return CONVEC_HE_BULK != 0 && sizeof(real) == 4;
}
// Porders whose kernels carry the compact pass (FP32, scalar line passes).
template <typename real, int P>
constexpr bool convec_compact_capable()
{
    return CONVEC_COMPACT != 0 && sizeof(real) == 4 && ConvecGeom<real, P>::S == 1 && !convec_packed<real, P>() &&
           !convec_staged<real>();
}
// Bytes of the staging area: He span, gpvol span (each with 16-byte slack for
// the unaligned start, rounded to 16) and the mbarrier.
template <typename real, int P>
constexpr size_t convec_stage_bytes()
{
    using G = ConvecGeom<real, P>;
    return convec_staged<real>() ? ((size_t)G::NE * G::N * 9 * sizeof(real) + 31) / 16 * 16 +
                                       ((size_t)G::NE * G::N * sizeof(real) + 31) / 16 * 16 + 16
                                 : 0;
}

// Blocks per SM the register budget is sized for: four 128-thread blocks (128
// registers) when the derivative matrices are constant-bank operands; three
// at porder 4 (168 registers, no spill): with the group's He prefetched into
// L2 the fourth block's latency hiding is worth less than the 88-byte spill
// of a 128-register budget (64^3 hexes: 1.460 against 1.470 ms; 1.508
// against 1.479 ms before the prefetch); three when He and gpvol are staged
// (their 25 KB per block leave room for three blocks).
#ifndef CONVEC_MINB4_STAGED
#define CONVEC_MINB4_STAGED 3
#endif
#ifndef CONVEC_MINB67
#define CONVEC_MINB67 1
#endif
#ifndef CONVEC_MINB4
#define CONVEC_MINB4 3
#endif
template <typename real, int P>
constexpr int convec_minb()
{
    using G = ConvecGeom<real, P>;
    return (sizeof(real) == 4 && G::S == 1 && G::NT <= 128 && P >= 3)
               ? (P == 5 ? CONVEC_MINB5
                         : (P == 4 ? (convec_staged<real>() ? CONVEC_MINB4_STAGED : CONVEC_MINB4)
                                   : (P >= 6 ? CONVEC_MINB67 : CONVEC_MINB)))
               : 1;
}

}  // namespace
}  // namespace msod
