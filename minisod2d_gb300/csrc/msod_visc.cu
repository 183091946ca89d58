// msod_visc.cu -- plain entropy-viscosity estimator for mu_e and the element
// features of the learned estimator.
//
// The reference consumes mu_e (elem_diffu.f90:19, mu_e(nelem,ngaus)) but
// contains no estimator; its numerical parameters name one
// (mod_numerical_params.f90:22-28: ce = 0.1, cmax = 0.5, cglob = 1,
// flag_normalise_entropy = 1).  This file writes the entropy-viscosity method
// of Guermond, Pasquetti & Popov (J. Comput. Phys. 230 (2011) 4248-4267) for
// one snapshot of the fields:
//   entropy      eta = rho/(gamma-1) * log(p / rho^gamma)
//   residual     R = div(eta u) - eta div u - u . grad eta      (per GLL point)
//                (the entropy equation's residual with the time derivative
//                replaced by its steady balance -eta div u - u.grad eta; R
//                vanishes where the discrete entropy flux is resolved and grows
//                across under-resolved fronts)
//   normalise    n_eta = || eta - mean(eta) ||_inf over the mesh (cglob = 1)
//   per element  h = (sum_g gpvol)^(1/3) / porder,
//                nu_max = cmax h max_e(|u| + c),  c = sqrt(gamma p / rho),
//                nu_E   = ce h^2 max_e |R| / n_eta,
//                nu     = min(nu_max, nu_E)
//   output       mu_e(e, a) = rho(a) nu(e)   in the reference's mu_e layout.
// The derivatives are one convection-type pass: the same line-parallel sum
// factorisation as the convection kernel, over eta, eta u and u.
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

// L2 prefetch of a group's He and gpvol spans at its start (0 = none; not in
// the list mode, whose groups are scattered elements).  64^3 porder-4 hexes:
// 0.924 ms against 0.964 ms; porder 5 on 51^3: 0.905 against 0.958 ms.
#ifndef VISC_PREFETCH
#define VISC_PREFETCH 1
#endif

namespace msod {

namespace {

// ---------------------------------------------------------------------------
// Entropy statistics over the nodes: sum, min and max of eta.
// ---------------------------------------------------------------------------
__global__ void entropy_stats_init(EntropyStats *st)
{
    st->sum = 0.0;
    st->kmin = f2key(3.0e38f);
    st->kmax = f2key(-3.0e38f);
}

// p is given directly (pr) or as rho * Rgas * T (Tem with Rgas > 0).
__global__ void entropy_stats_kernel(int npoin, const float *__restrict__ rho, const float *__restrict__ p_or_T,
                                     float Rgas, float gamma, EntropyStats *st)
{
    float s = 0.0f, mn = 3.0e38f, mx = -3.0e38f;
    auto add = [&](float r, float q) {
        const float p = Rgas > 0.0f ? r * Rgas * q : q;
        const float eta = r / (gamma - 1.0f) * (logf(p) - gamma * logf(r));
        s += eta;
        mn = fminf(mn, eta);
        mx = fmaxf(mx, eta);
    };
    // Four grid strides per trip, every load issued before the arithmetic
    // (eight loads in flight per thread instead of two).
    const int G = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i < npoin - 3 * G; i += 4 * G) {
        float r[4], q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = ldg(rho + i + k * G);
            q[k] = ldg(p_or_T + i + k * G);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) add(r[k], q[k]);
    }
    for (; i < npoin; i += G) add(ldg(rho + i), ldg(p_or_T + i));
    // Warp, then block reduction: one set of global atomics per block (the
    // atomics on these three words serialise in L2).
    double sd = (double)s;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sd += __shfl_xor_sync(0xffffffffu, sd, o);
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    __shared__ double bs[32];
    __shared__ float bmn[32], bmx[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        bs[warp] = sd;
        bmn[warp] = mn;
        bmx[warp] = mx;
    }
    __syncthreads();
    if (warp == 0) {
        sd = lane < nw ? bs[lane] : 0.0;
        mn = lane < nw ? bmn[lane] : 3.0e38f;
        mx = lane < nw ? bmx[lane] : -3.0e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sd += __shfl_xor_sync(0xffffffffu, sd, o);
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) {
            atomicAdd(&st->sum, sd);
            atomicMin(&st->kmin, f2key(mn));
            atomicMax(&st->kmax, f2key(mx));
        }
    }
}

// ---------------------------------------------------------------------------
// Plain estimator: one group of NE elements per block, one thread per line.
// ---------------------------------------------------------------------------
// 1-D derivative matrices of the current call, per porder (copied from the
// call's table area before the launch): constant-bank operands of the line
// passes when one thread owns a line.
__constant__ float c_VD[MSOD_MAX_PORDER + 1][kTableDMax];

enum { V_RHO = 0, V_P, V_U0, V_U1, V_U2, NVF };
constexpr int V_ETA = V_P;  // after the per-point preparation the pressure plane holds eta

template <class G, int DIR>
__device__ __forceinline__ void residual_pass(const LineThread<G> &lt, const float *__restrict__ sF,
                                              float *__restrict__ sR, const int *__restrict__ sPerm,
                                              const float *__restrict__ sD, const float *__restrict__ He, int e,
                                              float gamma)
{
    constexpr int Q = G::Q, QP = G::QP, R = G::R, NPL = G::NPL;
    constexpr int OST = DIR == 0 ? 1 : (DIR == 1 ? QP : Q * QP);
    const int base = lt.el * G::ES + line_off<DIR, Q, QP>(lt.la, lt.lb, 0);
    float eta[Q], u_[3][Q], eu[3][Q];
#pragma unroll
    for (int c = 0; c < Q; ++c) {
        const int o = base + c * OST;
        eta[c] = sF[V_ETA * NPL + o];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            u_[i][c] = sF[(V_U0 + i) * NPL + o];
            eu[i][c] = eta[c] * u_[i][c];
        }
    }
#pragma unroll
    for (int rr = 0; rr < R; ++rr) {
        if (!lt.owns(rr)) continue;
        const int r = lt.r0 + rr;
        const int a = sPerm[line_lat<DIR, Q>(lt.la, lt.lb, r)];
        const float *hp = He + ((size_t)e * G::N + a) * 9 + DIR * 3;
        const float h0 = ldg(hp), h1 = ldg(hp + 1), h2 = ldg(hp + 2);
        const float hh[3] = {h0, h1, h2};
        float deta = 0.0f, ddiv = 0.0f, dveta = 0.0f;  // D.eta, sum_i h_i D.(eta u_i), sum_i h_i D.u_i
        float dv[3] = {0.0f, 0.0f, 0.0f}, deu[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int c = 0; c < Q; ++c) {
            const float d = G::S == 1 ? c_VD[G::P][(DIR * Q + rr) * Q + c] : sD[(DIR * Q + r) * Q + c];
            deta = fmaf(d, eta[c], deta);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                deu[i] = fmaf(d, eu[i][c], deu[i]);
                dv[i] = fmaf(d, u_[i][c], dv[i]);
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) ddiv = fmaf(hh[i], deu[i], ddiv);
        float own_eta = eta[0], own_u[3] = {u_[0][0], u_[1][0], u_[2][0]};
#pragma unroll
        for (int c = 1; c < Q; ++c)
            if (c == r) {
                own_eta = eta[c];
#pragma unroll
                for (int i = 0; i < 3; ++i) own_u[i] = u_[i][c];
            }
#pragma unroll
        for (int i = 0; i < 3; ++i) dveta = fmaf(hh[i], dv[i], dveta);
        const float su = own_u[0] * h0 + own_u[1] * h1 + own_u[2] * h2;
        const float contrib = ddiv - own_eta * dveta - su * deta;
        const int o = base + r * OST;
        sR[o] = DIR == 0 ? contrib : sR[o] + contrib;
    }
}

// Elements per block at porders 4 and 5 (0: the line-geometry default, five
// and seven) and minimum resident blocks per SM (0: the block-size bound).
// Measured (plain estimator, CUDA events): porder 4 on 48^3 hexes 0.398 ms at
// three elements per 96-thread block against 0.413 ms at five (ten: 0.412 ms);
// porder 5 on 96^3 hexes 5.78 ms at seven against 5.91 / 6.19 ms at five /
// three; a minimum of two blocks per SM (more registers) 0.578 / 7.65 ms.
#ifndef VISC_NE4
#define VISC_NE4 3
#endif
#ifndef VISC_NE5
#define VISC_NE5 0
#endif
#ifndef VISC_MINB
#define VISC_MINB 0
#endif

template <class G>
__global__ void __launch_bounds__(G::NT, VISC_MINB)
    entropy_visc_kernel(int nelem, int npoin, const int *__restrict__ connec, const float *__restrict__ He,
                        const float *__restrict__ gpvol, const float *__restrict__ rho, const float *__restrict__ u,
                        const float *__restrict__ p_or_T, float Rgas, float gamma, float ce, float cmax,
                        int normalise, const EntropyStats *__restrict__ st, const int *__restrict__ list,
                        const int *__restrict__ count, float *__restrict__ mu_e, float *__restrict__ nu_out,
                        float *__restrict__ numax_out, const TableScratch *__restrict__ tabs)
{
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT, NPL = G::NPL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sF = reinterpret_cast<float *>(smem_raw);  // [NVF][NPL]
    float *sR = sF + NVF * NPL;                        // [NPL]
    float *sD = sR + NPL;                              // [3][Q][Q]
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);
    int *sPerm = sNode + NPL;
    int *sLat = sPerm + N;
    __shared__ int s_kS[NE], s_eid[NE];
    __shared__ float s_vol[NE], s_nu[NE];

    const int tid = threadIdx.x;
    // The block's elements: e0 .. e0+NE-1 (one group per block), or in list
    // mode (the per-element fallback) the entries e0 .. of the compacted list,
    // the blocks striding over the list's groups; -1 beyond the end.
    const int nwork = list ? ldg(count) : nelem;
    for (int gb = blockIdx.x; gb * NE < nwork; gb += gridDim.x) {
    const int e0 = gb * NE;
    if (VISC_PREFETCH != 0 && !list && tid == 0) {
        // The group's He and gpvol spans into L2 while its node fields are gathered.
        const int e1 = min(e0 + NE, nelem);
        prefetch_span_l2(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(float));
        prefetch_span_l2(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(float));
    }
    __syncthreads();  // the previous group's shared-memory reads are complete
    if (tid < NE) s_eid[tid] = e0 + tid < nwork ? (list ? ldg(list + e0 + tid) : e0 + tid) : -1;
    __syncthreads();
    // Node ids of the group (connec is element-fastest) into registers while
    // the call's tables are copied into shared memory.
    constexpr int IPT = (NE * N + NT - 1) / NT;
    int ids[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = tid + k * NT;
        const int el = i % NE, a = i / NE, e = s_eid[el];
        ids[k] = (i < NE * N && e >= 0) ? ldg(connec + (size_t)a * nelem + e) - 1 : -1;
    }
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    if (G::S > 1)
        for (int i = tid; i < 3 * Q * Q; i += NT) sD[i] = tabs->Df[i];
    if (tid < NE) {
        s_kS[tid] = 0;
        s_vol[tid] = 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = tid + k * NT;
        if (i < NE * N) {
            const int v = ids[k];
            sNode[(i % NE) * ES + sLat[i / NE]] = (v >= 0 && v < npoin) ? v : -1;
        }
    }
    __syncthreads();
    const size_t np = (size_t)npoin;
    for (int i = tid; i < NE * N; i += NT) {
        const int el = i / N, l = i - el * N;
        const int o = el * ES + (l / (Q * Q) * Q + (l / Q) % Q) * QP + l % Q;
        const int p = sNode[o];
        float v[NVF] = {1.0f, 1.0f, 0.0f, 0.0f, 0.0f};
        if (p >= 0) {
            v[V_RHO] = ldg(rho + p);
            v[V_P] = Rgas > 0.0f ? v[V_RHO] * Rgas * ldg(p_or_T + p) : ldg(p_or_T + p);
#pragma unroll
            for (int c = 0; c < 3; ++c) v[V_U0 + c] = ldg(u + c * np + p);
        }
        // Per point once: the entropy (replacing the pressure), the element
        // maxima of |u| + c and the element volume.
        const float spd = sqrtf(v[V_U0] * v[V_U0] + v[V_U1] * v[V_U1] + v[V_U2] * v[V_U2]) +
                          sqrtf(gamma * v[V_P] / v[V_RHO]);
        v[V_ETA] = v[V_RHO] / (gamma - 1.0f) * (logf(v[V_P]) - gamma * logf(v[V_RHO]));
#pragma unroll
        for (int c = 0; c < NVF; ++c) sF[c * NPL + o] = v[c];
        sR[o] = spd;  // the residual plane is free until the first pass
    }
    __syncthreads();
    // One warp per element: max |u| + c and the volume (warp reductions, no
    // shared-memory atomics on one address per element).
    {
        const int lane = tid & 31, warp = tid >> 5;
        for (int el = warp; el < NE; el += NT / 32) {
            const int ee = s_eid[el];
            unsigned mx = 0u;
            float vol = 0.0f;
            if (ee >= 0)
                for (int l = lane; l < N; l += 32) {
                    const int o = el * ES + (l / (Q * Q) * Q + (l / Q) % Q) * QP + l % Q;
                    mx = max(mx, __float_as_uint(sR[o]));  // non-negative floats order like their bits
                    vol += ldg(gpvol + (size_t)ee * N + sPerm[l]);
                }
            mx = __reduce_max_sync(0xffffffffu, mx);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) vol += __shfl_xor_sync(0xffffffffu, vol, off);
            if (lane == 0) {
                s_kS[el] = (int)mx;
                s_vol[el] = vol;
            }
        }
    }
    __syncthreads();
    const LineThread<G> lt(tid);
    const int e = s_eid[lt.el];
    const bool live = lt.active && e >= 0;
    if (live) residual_pass<G, 0>(lt, sF, sR, sPerm, sD, He, e, gamma);
    __syncthreads();
    if (live) residual_pass<G, 1>(lt, sF, sR, sPerm, sD, He, e, gamma);
    __syncthreads();
    if (live) residual_pass<G, 2>(lt, sF, sR, sPerm, sD, He, e, gamma);
    __syncthreads();
    float neta = 1.0f;
    if (normalise) {
        const double mean = st->sum / (double)npoin;
        const double lo = (double)key2f(st->kmin), hi = (double)key2f(st->kmax);
        neta = (float)fmax(hi - mean, mean - lo);
        if (!(neta > 0.0f)) neta = 1.0f;
    }
    // Element maxima of |R| and the element viscosity (one warp per element).
    {
        const int lane = tid & 31, warp = tid >> 5;
        for (int el = warp; el < NE; el += NT / 32) {
            const int ee = s_eid[el];
            unsigned mx = 0u;
            if (ee >= 0)
                for (int l = lane; l < N; l += 32) {
                    const int o = el * ES + (l / (Q * Q) * Q + (l / Q) % Q) * QP + l % Q;
                    mx = max(mx, __float_as_uint(fabsf(sR[o])));
                }
            mx = __reduce_max_sync(0xffffffffu, mx);
            if (lane == 0) {
                const float h = cbrtf(s_vol[el]) / (float)(Q - 1);
                const float numax = cmax * h * __int_as_float(s_kS[el]);
                const float nuE = ce * h * h * __uint_as_float(mx) / neta;
                const float nu = fminf(numax, nuE);
                s_nu[el] = nu;
                if (ee >= 0) {
                    if (nu_out) nu_out[ee] = nu;
                    if (numax_out && !list) numax_out[ee] = numax;
                }
            }
        }
    }
    if (list) continue;
    if (mu_e) {
        __syncthreads();
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i % NE, a = i / NE, ee = s_eid[el];
            if (ee < 0) continue;
            mu_e[(size_t)a * nelem + ee] = sF[V_RHO * NPL + el * ES + sLat[a]] * s_nu[el];
        }
    }
    break;  // one group per block outside list mode
    }
}

template <int P>
using ViscGeom = LineGeom<float, P, (P == 4 && VISC_NE4 > 0) ? VISC_NE4 : ((P == 5 && VISC_NE5 > 0) ? VISC_NE5 : 64)>;

// Preferred shared-memory carveout of the porder-5 estimator, percent of the
// maximum (-1: none). Its 51.5 KB blocks fill a 228 KB carveout four to an SM
// and leave ~28 KB of L1; at 58 % (132 KB: two blocks, ~124 KB of L1) it runs
// 1.80 ms instead of 2.36 ms on 64^3 hexes (72 %, three blocks: 1.86 ms).
// Porder 4 measures the same with or without (0.89 ms).
#ifndef VISC_CARVE5
#define VISC_CARVE5 58
#endif

template <int P>
cudaError_t visc_p(const ViscArgs &a, cudaStream_t st)
{
    using G = ViscGeom<P>;
    constexpr size_t smem = (size_t)(NVF + 1) * G::NPL * sizeof(float) + 3 * G::Q * G::Q * sizeof(float) +
                            (size_t)(G::NPL + 2 * G::N) * sizeof(int);
    static_assert(smem <= 227 * 1024, "shared memory budget");
    auto kern = entropy_visc_kernel<G>;
    if (!a.tabs) return cudaErrorInvalidValue;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    if (P == 5 && VISC_CARVE5 >= 0) {
        err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, VISC_CARVE5);
        if (err != cudaSuccess) return err;
    }
    if (G::S == 1) {
        err = cudaMemcpyToSymbolAsync(c_VD, a.tabs->Df, sizeof(float) * 3 * G::Q * G::Q, sizeof(float) * kTableDMax * P,
                                      cudaMemcpyDeviceToDevice, st);
        if (err != cudaSuccess) return err;
    }
    // List mode: resident blocks stride over the list (its length is known on
    // the device only); otherwise one group per block.
    const int ngroups = (a.nelem + G::NE - 1) / G::NE;
    const unsigned grid = (unsigned)(a.list ? persistent_grid(kern, G::NT, smem, ngroups) : ngroups);
    if (grid == 0) return cudaErrorInvalidConfiguration;
    kern<<<grid, G::NT, smem, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.rho, a.u, a.p_or_T, a.Rgas, a.gamma,
                                    a.ce, a.cmax, a.normalise,
                                    a.stats, a.list, a.count, a.mu_e, a.nu, a.numax, a.tabs);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_entropy_stats(int npoin, const float *rho, const float *p_or_T, float Rgas, float gamma,
                                 EntropyStats *st, cudaStream_t s)
{
    entropy_stats_init<<<1, 1, 0, s>>>(st);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int blocks = (npoin + 255) / 256;
    if (blocks > 8 * sms) blocks = 8 * sms;
    entropy_stats_kernel<<<blocks, 256, 0, s>>>(npoin, rho, p_or_T, Rgas, gamma, st);
    return cudaGetLastError();
}

cudaError_t launch_entropy_visc(int porder, const ViscArgs &a, cudaStream_t st)
{
    switch (porder) {
    case 1: return visc_p<1>(a, st);
    case 2: return visc_p<2>(a, st);
    case 3: return visc_p<3>(a, st);
    case 4: return visc_p<4>(a, st);
    case 5: return visc_p<5>(a, st);
    case 6: return visc_p<6>(a, st);
    case 7: return visc_p<7>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace msod
