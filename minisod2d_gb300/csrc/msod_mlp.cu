// msod_mlp.cu -- learned per-element artificial viscosity.
//
// A small per-element network stands in for the entropy-viscosity estimator
// of msod_visc.cu.  It maps 12 element-local features to y = nu / nu_max in
// (0, 1]; the learned viscosity is mu_e(e, a) = rho(a) * nu_max(e) * y(e).
// The plain estimator's y spans many decades (entropy viscosity far below
// the first-order bound away from under-resolved fronts), so the network
// works in decades: its softplus output s >= 0 gives y = 10^-s, and the
// heavy-tailed features enter as logarithms.
//   network   12 -> 32 -> 32 -> 1, SiLU hidden units, softplus output,
//             FP16 weights (FP32 master copy while training), FP32 accumulation
//   training  mean-squared error of s against -log10 of the plain estimator's
//             y (clamped to [1e-12, 1]) on feature -> y pairs, optionally
//             weighted per sample (the caller's weights), Adam (beta
//             0.9 / 0.999, eps 1e-8); the forward pass uses the FP16-rounded
//             weights it will be deployed with
//   fallback  an element whose features leave the training range [min, max]
//             (per feature) is flagged; the caller then takes its viscosity
//             from the plain estimator.
// Features of element e (nodal values gathered through connec; c = sound
// speed, s = log(p / rho^gamma) / (gamma - 1), eta = rho s, theta/omega/S =
// divergence, vorticity and strain-rate norms at the element centre, h =
// (sum gpvol)^(1/3) / porder, "centre lines" = the three GLL lines through
// the centre node, n_eta = ||eta - mean eta||_inf over the mesh; every
// feature except 3, 4 and 5 is stored as log(max(v, 0) + 1e-12)):
//   0 (rho_max - rho_min) / rho_mean      1 (p_max - p_min) / p_mean
//   2 s_max - s_min                       3 mean |u| / mean c
//   4 max |u| / c                         5 theta h / mean c
//   6 |omega| h / mean c                  7 |S| h / mean c
//   8 max over centre lines |rho(0) - 2 rho(mid) + rho(P)| / rho_mean
//   9 max over centre lines |eta(0) - 2 eta(mid) + eta(P)| / n_eta
//  10 (eta_max - eta_min) / n_eta
//  11 max over centre lines of the product-rule defect of eta u_d,
//     |(eta u)(P) - (eta u)(0) - eta(mid)(u(P) - u(0)) - u(mid)(eta(P) - eta(0))|
//     / (n_eta (mean |u| + mean c))
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"
#include "msod_mlp.cuh"

namespace msod {

namespace {

// ---------------------------------------------------------------------------
// Features: one warp per element.
// ---------------------------------------------------------------------------
template <int P>
constexpr int feat_warps()
{
    return 12288 / (5 * (P + 1) * (P + 1) * (P + 1)) < 8 ? 12288 / (5 * (P + 1) * (P + 1) * (P + 1)) : 8;
}

// Minimum resident blocks per SM of the features kernel (-1: per porder as
// measured, the block-size bound alone at the other porders; 0: that bound
// everywhere).  The kernel waits on its gathers, so residency
// pays: porder 4 at six 256-thread blocks per SM (40 registers, a 16-byte
// spill) 0.261 ms for the learned viscosity on 48^3 hexes, against 0.283 ms at
// five and 0.313 ms at four (the block-size bound, 56-64 registers); porder 5
// at five (48 registers) 2.69 ms on 96^3 hexes, against 2.87 ms at six and
// 2.84 ms at four.
#ifndef FEAT_MINB
#define FEAT_MINB -1
#endif
template <int P>
constexpr int feat_minb()
{
    return FEAT_MINB >= 0 ? FEAT_MINB : (P == 4 ? 6 : (P == 5 ? 5 : 0));
}

template <int P>
__global__ void __launch_bounds__(32 * feat_warps<P>(), feat_minb<P>())
    features_kernel(int nelem, int npoin, const int *__restrict__ connec, const float *__restrict__ He,
                    const float *__restrict__ gpvol, const TableScratch *__restrict__ tabs,
                    const float *__restrict__ rho, const float *__restrict__ u, const float *__restrict__ p_or_T,
                    float Rgas, float gamma, float cmax, const EntropyStats *__restrict__ st,
                    float *__restrict__ feat, float *__restrict__ numax_out)
{
    constexpr int Q = P + 1, N = Q * Q * Q, kFeatWarps = feat_warps<P>();
    constexpr int NPL = (N + 31) / 32;  // nodes per lane
    // rho, p, u0, u1, u2 by lattice point l = (K*Q+J)*Q+I (SOD 1-D indices);
    // plane 0 first holds the element's node ids by gmsh node.
    __shared__ float sv[kFeatWarps][5][N];
    __shared__ int sPerm[N];         // lattice -> gmsh node
    __shared__ float sD[3 * Q * Q];  // 1-D derivative matrices
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e0 = blockIdx.x * kFeatWarps, e = e0 + w;
    const TableScratch *t = tabs;
    for (int i = threadIdx.x; i < N; i += 32 * kFeatWarps) sPerm[i] = t->perm[i];
    for (int i = threadIdx.x; i < 3 * Q * Q; i += 32 * kFeatWarps) sD[i] = t->Df[i];
    // The block's node ids, element-fastest as connec stores them (the block's
    // elements share each 32-byte sector).
    for (int i = threadIdx.x; i < kFeatWarps * N; i += 32 * kFeatWarps) {
        const int el = i % kFeatWarps, a = i / kFeatWarps;
        const int id = e0 + el < nelem ? ldg(connec + (size_t)a * nelem + e0 + el) - 1 : 0;
        reinterpret_cast<int *>(sv[el][0])[a] = min(max(id, 0), npoin - 1);
    }
    __syncthreads();
    if (e >= nelem) return;
    // Entropy normalisation (read early: its latency hides behind the gathers).
    const double esum = st->sum;
    const int ekmin = st->kmin, ekmax = st->kmax;
    float rmin = 3e38f, rmax = -3e38f, rsum = 0.f, pmin = 3e38f, pmax = -3e38f, psum = 0.f;
    float smin = 3e38f, smax = -3e38f, emin = 3e38f, emax = -3e38f, machmax = 0.f, usum = 0.f, csum = 0.f;
    float spdmax = 0.f, vol = 0.f;
    const size_t np = (size_t)npoin;
    const float s_scale = 0.69314718f / (gamma - 1.0f);  // ln 2 / (gamma - 1): s from base-2 logarithms
    // All of the lane's node ids first, then every field load of the lane, then
    // the arithmetic: the loads overlap (15-17 % faster than loads interleaved
    // with the per-node statistics).  Lanes take the lattice points in order,
    // so a warp's loads follow the mesh lines (x-neighbours share sectors).
    int pn[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
        const int l = lane + 32 * k;
        pn[k] = l < N ? reinterpret_cast<const int *>(sv[w][0])[sPerm[l]] : 0;
    }
    __syncwarp();  // every id read before plane 0 takes the density
    float fr[NPL], fp[NPL], fx[NPL], fy[NPL], fz[NPL];
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
        const int l = lane + 32 * k;
        const int p = pn[k];
        const bool ok = l < N;
        fr[k] = ok ? ldg(rho + p) : 1.0f;
        fp[k] = ok ? ldg(p_or_T + p) : 1.0f;
        fx[k] = ok ? ldg(u + p) : 0.0f;
        fy[k] = ok ? ldg(u + np + p) : 0.0f;
        fz[k] = ok ? ldg(u + 2 * np + p) : 0.0f;
        vol += ok ? ldg(gpvol + (size_t)e * N + l) : 0.0f;  // the sum over all of the element's points
    }
#pragma unroll
    for (int k = 0; k < NPL; ++k) {
        const int a = lane + 32 * k;  // lattice point
        if (a >= N) break;
        const float r = fr[k];
        const float pr = Rgas > 0.0f ? r * Rgas * fp[k] : fp[k];
        const float ux = fx[k], uy = fy[k], uz = fz[k];
        sv[w][0][a] = r;
        sv[w][1][a] = pr;
        sv[w][2][a] = ux;
        sv[w][3][a] = uy;
        sv[w][4][a] = uz;
        // Per-node statistics with the hardware approximations (the element
        // reductions below are what the features keep).
        const float c = sqrt_approx(__fdividef(gamma * pr, r)), um = sqrt_approx(ux * ux + uy * uy + uz * uz);
        const float s = (log2_approx(pr) - gamma * log2_approx(r)) * s_scale;
        rmin = fminf(rmin, r); rmax = fmaxf(rmax, r); rsum += r;
        pmin = fminf(pmin, pr); pmax = fmaxf(pmax, pr); psum += pr;
        smin = fminf(smin, s); smax = fmaxf(smax, s);
        emin = fminf(emin, r * s); emax = fmaxf(emax, r * s);
        machmax = fmaxf(machmax, __fdividef(um, c));
        usum += um; csum += c;
        spdmax = fmaxf(spdmax, um + c);
    }
    // Warp minima / maxima as one reduction each on order-preserving integer
    // keys (the two non-negative ones on their bits); sums by butterfly, which
    // leaves the same value on every lane.
    auto wmin = [](float v) { return key2f(__reduce_min_sync(~0u, f2key(v))); };
    auto wmax = [](float v) { return key2f(__reduce_max_sync(~0u, f2key(v))); };
    rmin = wmin(rmin); rmax = wmax(rmax);
    pmin = wmin(pmin); pmax = wmax(pmax);
    smin = wmin(smin); smax = wmax(smax);
    emin = wmin(emin); emax = wmax(emax);
    machmax = __uint_as_float(__reduce_max_sync(~0u, __float_as_uint(machmax)));
    spdmax = __uint_as_float(__reduce_max_sync(~0u, __float_as_uint(spdmax)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rsum += __shfl_xor_sync(~0u, rsum, o); psum += __shfl_xor_sync(~0u, psum, o);
        usum += __shfl_xor_sync(~0u, usum, o); csum += __shfl_xor_sync(~0u, csum, o);
        vol += __shfl_xor_sync(~0u, vol, o);
    }
    __syncwarp();
    // Centre node and the natural -> SOD 1-D index map (0 -> 0, P -> 1, k -> k+1).
    const int mnat = P / 2;
    const int ms = mnat == 0 ? 0 : (mnat == P ? 1 : mnat + 1);
    auto node = [&](int I, int J, int K) { return (K * Q + J) * Q + I; };  // lattice point (planes of sv)
    const int nat[3] = {0, ms, 1};  // SOD positions of natural 0, mid, P
    // Lanes 0-8: iso derivative gi[i][d] of u_i along d at the centre (lane 3i + d);
    // lanes 9-11: second differences and product-rule defect along d = lane - 9;
    // lanes 12-20: He at the centre node.
    float gval = 0.f, d2r_l = 0.f, d2e_l = 0.f, def_l = 0.f, hval = 0.f;
    if (lane < 9) {
        const int i = lane / 3, d = lane % 3;
        float sacc = 0.f;
        for (int c = 0; c < Q; ++c) {
            const int I = d == 0 ? c : ms, J = d == 1 ? c : ms, K = d == 2 ? c : ms;
            sacc = fmaf(sD[(d * Q + ms) * Q + c], sv[w][2 + i][node(I, J, K)], sacc);
        }
        gval = sacc;
    } else if (lane < 12) {
        const int d = lane - 9;
        float rv[3], ev[3], uv[3];
        for (int k = 0; k < 3; ++k) {
            const int I = d == 0 ? nat[k] : ms, J = d == 1 ? nat[k] : ms, K = d == 2 ? nat[k] : ms;
            const int a = node(I, J, K);
            const float r = sv[w][0][a], pr = sv[w][1][a];
            rv[k] = r;
            ev[k] = r * ((log2_approx(pr) - gamma * log2_approx(r)) * s_scale);
            uv[k] = sv[w][2 + d][a];
        }
        d2r_l = fabsf(rv[0] - 2.f * rv[1] + rv[2]);
        d2e_l = fabsf(ev[0] - 2.f * ev[1] + ev[2]);
        const float A = ev[2] * uv[2] - ev[0] * uv[0];
        const float B = ev[1] * (uv[2] - uv[0]) + uv[1] * (ev[2] - ev[0]);
        def_l = fabsf(A - B);
    } else if (lane < 21) {
        hval = ldg(He + ((size_t)e * N + sPerm[node(ms, ms, ms)]) * 9 + (lane - 12));
    }
    float gi[3][3], Hc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        gi[k / 3][k % 3] = __shfl_sync(~0u, gval, k);
        Hc[k] = __shfl_sync(~0u, hval, 12 + k);
    }
    float d2r = 0.f, d2e = 0.f, defect = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        d2r = fmaxf(d2r, __shfl_sync(~0u, d2r_l, 9 + d));
        d2e = fmaxf(d2e, __shfl_sync(~0u, d2e_l, 9 + d));
        defect = fmaxf(defect, __shfl_sync(~0u, def_l, 9 + d));
    }
    // Every lane holds the element's reductions; lane k < 12 forms feature k
    // (one division and at most one logarithm per lane) and the twelve lanes
    // store the element's features together.
    const double mean = esum / (double)npoin;
    const double lo = (double)key2f(ekmin), hi = (double)key2f(ekmax);
    float neta = (float)fmax(hi - mean, mean - lo);
    if (!(neta > 0.0f)) neta = 1.0f;
    constexpr float invN = 1.0f / (float)N;
    const float rmean = rsum * invN, pmean = psum * invN, umean = usum * invN, cmean = csum * invN;
    const float h = cbrtf(vol) / (float)P;
    float G[3][3];  // G[i][j] = d u_i / d x_j = sum_k He(j,k) gi[i][k]
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G[i][j] = Hc[0 * 3 + j] * gi[i][0] + Hc[3 + j] * gi[i][1] + Hc[6 + j] * gi[i][2];
    const float theta = G[0][0] + G[1][1] + G[2][2];
    const float w0 = G[2][1] - G[1][2], w1 = G[0][2] - G[2][0], w2 = G[1][0] - G[0][1];
    float s2 = 0.f;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const float sij = 0.5f * (G[i][j] + G[j][i]);
            s2 += sij * sij;
        }
    // Feature k = num / den, through flog except features 3, 4 and 5.
    float num = rmax - rmin, den = rmean;                              // 0
    if (lane == 1) { num = pmax - pmin; den = pmean; }
    if (lane == 2) { num = smax - smin; den = 1.0f; }
    if (lane == 3) { num = umean; den = cmean; }
    if (lane == 4) { num = machmax; den = 1.0f; }
    if (lane == 5) { num = theta * h; den = cmean; }
    if (lane == 6) { num = sqrtf(w0 * w0 + w1 * w1 + w2 * w2) * h; den = cmean; }
    if (lane == 7) { num = sqrtf(s2) * h; den = cmean; }
    if (lane == 8) { num = d2r; den = rmean; }
    if (lane == 9) { num = d2e; den = neta; }
    if (lane == 10) { num = emax - emin; den = neta; }
    if (lane == 11) { num = defect; den = neta * (umean + cmean); }
    const float v = num / den;
    if (lane < kMlpIn) feat[(size_t)e * kMlpIn + lane] = (lane >= 3 && lane <= 5) ? v : flog(v);
    if (lane != 0) return;
    if (numax_out) numax_out[e] = cmax * h * spdmax;
}

template <int P>
cudaError_t features_p(const FeatureArgs &a, cudaStream_t st)
{
    constexpr int kFeatWarps = feat_warps<P>();
    const unsigned grid = (unsigned)((a.nelem + kFeatWarps - 1) / kFeatWarps);
    features_kernel<P><<<grid, 32 * kFeatWarps, 0, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.tabs, a.rho,
                                                         a.u, a.p_or_T, a.Rgas, a.gamma, a.cmax, a.stats, a.feat,
                                                         a.numax);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Network
// ---------------------------------------------------------------------------
struct Act {
    float x[kMlpIn], a1[kMlpH], h1[kMlpH], a2[kMlpH], h2[kMlpH], z, y;
};

// Forward pass with weights w (FP16-rounded values in FP32 registers).
__device__ __forceinline__ void mlp_forward(const float *__restrict__ w, const MlpNorm &nm, const float *x_raw,
                                            Act &s)
{
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) s.x[k] = (x_raw[k] - nm.mean[k]) * nm.inv_std[k];
    for (int j = 0; j < kMlpH; ++j) {
        float acc = w[kOffB1 + j];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) acc = fmaf(w[kOffW1 + j * kMlpIn + k], s.x[k], acc);
        s.a1[j] = acc;
        s.h1[j] = silu(acc);
    }
    for (int j = 0; j < kMlpH; ++j) {
        float acc = w[kOffB2 + j];
        for (int k = 0; k < kMlpH; ++k) acc = fmaf(w[kOffW2 + j * kMlpH + k], s.h1[k], acc);
        s.a2[j] = acc;
        s.h2[j] = silu(acc);
    }
    float z = w[kOffB3];
    for (int j = 0; j < kMlpH; ++j) z = fmaf(w[kOffW3 + j], s.h2[j], z);
    s.z = z;
    s.y = softplus(z);
}

// Inference: y = 10^-s in (0, 1] and the out-of-range flag per element.
__global__ void mlp_predict_kernel(int nelem, const float *__restrict__ feat, const __half *__restrict__ wh,
                                   const MlpNorm *__restrict__ nm, const float *__restrict__ numax,
                                   float *__restrict__ y, float *__restrict__ nu, int *__restrict__ flag,
                                   int *__restrict__ list, int *count)
{
    __shared__ float w[kMlpParams];
    __shared__ MlpNorm snm;
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = __half2float(wh[i]);
    if (threadIdx.x == 0) snm = *nm;
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    int out = 0;
    if (e < nelem) {
        float x[kMlpIn];
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) {
            x[k] = feat[(size_t)e * kMlpIn + k];
            if (!(x[k] >= snm.fmin[k] && x[k] <= snm.fmax[k])) out = 1;
        }
        const float yy = y_from_s(mlp_infer(w, snm, x));
        if (y) y[e] = yy;
        if (nu) nu[e] = yy * numax[e];
        if (flag) flag[e] = out;
    }
    if (list) warp_append(out != 0, e, list, count);  // every lane of the warp (the block is whole warps)
}

// Per-feature mean, 1/std, min, max over the training samples (one block per feature).
__global__ void mlp_norm_kernel(int n, const float *__restrict__ feat, MlpNorm *nm)
{
    const int k = blockIdx.x;
    double s = 0.0, s2 = 0.0;
    float mn = 3e38f, mx = -3e38f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float v = feat[(size_t)i * kMlpIn + k];
        s += v;
        s2 += (double)v * v;
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    __shared__ double ss[256], ss2[256];
    __shared__ float smn[256], smx[256];
    ss[threadIdx.x] = s; ss2[threadIdx.x] = s2; smn[threadIdx.x] = mn; smx[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            ss2[threadIdx.x] += ss2[threadIdx.x + o];
            smn[threadIdx.x] = fminf(smn[threadIdx.x], smn[threadIdx.x + o]);
            smx[threadIdx.x] = fmaxf(smx[threadIdx.x], smx[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mean = ss[0] / n;
        const double var = ss2[0] / n - mean * mean;
        nm->mean[k] = (float)mean;
        nm->inv_std[k] = (float)(1.0 / sqrt(var > 1e-24 ? var : 1e-24));
        nm->fmin[k] = smn[0];
        nm->fmax[k] = smx[0];
    }
}

__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    return v;
}

// One batch: loss gradient accumulated into grad (sum over the batch of
// dL/dparam with L = the weighted mean squared error, weight[sample] or 1).
// Sample i of the batch is idx ? idx[i] : hash(seed, step, i) mod n.
__global__ void __launch_bounds__(256) mlp_grad_kernel(int n, const float *__restrict__ feat,
                                                       const float *__restrict__ target,
                                                       const float *__restrict__ weight, const int *__restrict__ idx,
                                                       int batch, uint32_t seed, int step,
                                                       const float *__restrict__ master, const MlpNorm *__restrict__ nm,
                                                       float *__restrict__ grad, float *__restrict__ loss)
{
    __shared__ float w[kMlpParams];
    __shared__ float g[kMlpParams];
    __shared__ MlpNorm snm;
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
        w[i] = __half2float(__float2half_rn(master[i]));  // deployed FP16 weights
        g[i] = 0.0f;
    }
    if (threadIdx.x == 0) snm = *nm;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < batch;
    int sidx = 0;
    if (live) sidx = idx ? idx[i] : (int)(hash32(seed * 0x9E3779B9u ^ hash32((uint32_t)step * 0x85ebca6bu + i)) % (uint32_t)n);
    float x[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) x[k] = live ? feat[(size_t)sidx * kMlpIn + k] : 0.0f;
    Act s;
    mlp_forward(w, snm, x, s);
    const float t = live ? s_from_y(target[sidx]) : 0.0f;
    const float wt = live ? (weight ? weight[sidx] : 1.0f) : 0.0f;
    const float dy = live ? 2.0f * wt * (s.y - t) / (float)batch : 0.0f;
    if (loss) {
        const float l = warp_sum(live ? wt * (s.y - t) * (s.y - t) / (float)batch : 0.0f);
        if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
    }
    const float dz = dy * sigmoidf_(s.z);
    const int lane = threadIdx.x & 31;
    auto acc = [&](int off, float v) {
        v = warp_sum(v);
        if (lane == 0) atomicAdd(&g[off], v);
    };
    acc(kOffB3, dz);
    float da2[kMlpH];
    for (int j = 0; j < kMlpH; ++j) {
        acc(kOffW3 + j, dz * s.h2[j]);
        const float sg = sigmoidf_(s.a2[j]);
        da2[j] = dz * w[kOffW3 + j] * sg * (1.0f + s.a2[j] * (1.0f - sg));
        acc(kOffB2 + j, da2[j]);
    }
    for (int j = 0; j < kMlpH; ++j)
        for (int k = 0; k < kMlpH; ++k) acc(kOffW2 + j * kMlpH + k, da2[j] * s.h1[k]);
    for (int k = 0; k < kMlpH; ++k) {
        float dh1 = 0.0f;
        for (int j = 0; j < kMlpH; ++j) dh1 = fmaf(w[kOffW2 + j * kMlpH + k], da2[j], dh1);
        const float sg = sigmoidf_(s.a1[k]);
        const float da1 = dh1 * sg * (1.0f + s.a1[k] * (1.0f - sg));
        acc(kOffB1 + k, da1);
#pragma unroll
        for (int m = 0; m < kMlpIn; ++m) acc(kOffW1 + k * kMlpIn + m, da1 * s.x[m]);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < kMlpParams; p += blockDim.x) atomicAdd(&grad[p], g[p]);
}

// Adam step t (1-based) on the FP32 master weights; clears the gradient and
// refreshes the FP16 copy.
__global__ void mlp_adam_kernel(float *__restrict__ master, float *__restrict__ m, float *__restrict__ v,
                                float *__restrict__ grad, __half *__restrict__ wh, float lr, int t)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gr = grad[p];
    const float mm = b1 * m[p] + (1.0f - b1) * gr;
    const float vv = b2 * v[p] + (1.0f - b2) * gr * gr;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.0f - powf(b1, (float)t)), vh = vv / (1.0f - powf(b2, (float)t));
    const float w = master[p] - lr * mh / (sqrtf(vh) + eps);
    master[p] = w;
    wh[p] = __float2half_rn(w);
    grad[p] = 0.0f;
}

__global__ void mlp_to_half_kernel(const float *__restrict__ master, __half *__restrict__ wh)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < kMlpParams) wh[p] = __float2half_rn(master[p]);
}

}  // namespace

cudaError_t launch_features(int porder, const FeatureArgs &a, cudaStream_t st)
{
    switch (porder) {
    case 1: return features_p<1>(a, st);
    case 2: return features_p<2>(a, st);
    case 3: return features_p<3>(a, st);
    case 4: return features_p<4>(a, st);
    case 5: return features_p<5>(a, st);
    case 6: return features_p<6>(a, st);
    case 7: return features_p<7>(a, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mlp_predict(int nelem, const float *feat, const __half *wh, const MlpNorm *nm, const float *numax,
                               float *y, float *nu, int *flag, int *list, int *count, cudaStream_t st)
{
    if (list) {
        const cudaError_t err = cudaMemsetAsync(count, 0, sizeof(int), st);
        if (err != cudaSuccess) return err;
    }
    mlp_predict_kernel<<<(nelem + 127) / 128, 128, 0, st>>>(nelem, feat, wh, nm, numax, y, nu, flag, list, count);
    return cudaGetLastError();
}

cudaError_t launch_mlp_norm(int n, const float *feat, MlpNorm *nm, cudaStream_t st)
{
    mlp_norm_kernel<<<kMlpIn, 256, 0, st>>>(n, feat, nm);
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(int n, const float *feat, const float *target, const float *weight, const int *idx,
                            int batch, uint32_t seed,
                            int step, const float *master, const MlpNorm *nm, float *grad, float *loss, cudaStream_t st)
{
    mlp_grad_kernel<<<(batch + 255) / 256, 256, 0, st>>>(n, feat, target, weight, idx, batch, seed, step, master, nm, grad,
                                                         loss);
    return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float *master, float *m, float *v, float *grad, __half *wh, float lr, int t,
                            cudaStream_t st)
{
    mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, m, v, grad, wh, lr, t);
    return cudaGetLastError();
}

cudaError_t launch_mlp_to_half(const float *master, __half *wh, cudaStream_t st)
{
    mlp_to_half_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, wh);
    return cudaGetLastError();
}

}  // namespace msod
