// msod_tet.cu -- linear-tetrahedron convection and diffusion residuals.
//
// Computes what fem_convec (elem_convec.f90:839-948) and fem_diffu
// (elem_diffu.f90:199-317) compute: 4 nodes and 4 Gauss points per element,
// Cartesian shape derivatives gpcar(a,:) = He(:,:,g) . dNgp(:,a,g) at every
// point, point gradients from the element's nodal values, and the residual
// of each node accumulated over the points, then assembled into the nodes.
//
// Design (one thread per element; the work is a few hundred bytes and ~1.5
// kFLOP per element, so the kernels are bound by memory traffic and the
// nodal scatter, not by arithmetic):
//   * Ngp(4,4) and dNgp(3,4,4) are constant-bank operands, copied from the
//     caller's device tables before the launch;
//   * an element's metric is contiguous (He: 36 values, gpvol: 4), read whole
//     with 16-byte vector loads when the arrays are 16-byte aligned;
//   * node fields are gathered through connec (element-fastest, coalesced),
//     one 16-byte load per field for an element whose nodes are 4k..4k+3;
//   * assembly by fire-and-forget reductions; an element whose nodes are
//     4k..4k+3 (the reference driver's tet mesh, mod_mesh.f90:86-101) adds each
//     residual with one red.global.add.v4.f32 when the output arrays allow it.
// A connec entry outside 1..npoin reads node 1's values and is not assembled
// (wrong numbers for a malformed mesh, never an out-of-bounds access).
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

// Blocks per SM the register budgets are sized for.  Measured on 4.24 M
// tetrahedra: the convection 0.476 / 0.445 / 0.431 ms at 3 / 4 / 5 blocks (167,
// 128 and 96 registers, the last with a 140-byte spill), the diffusion 0.405 /
// 0.364 / 0.395 ms.
#ifndef TET_CONVEC_MINB
#define TET_CONVEC_MINB 5
#endif
#ifndef TET_DIFFU_MINB
#define TET_DIFFU_MINB 4
#endif
// L2 prefetch of a block's contiguous element data at its start (one
// thread), bits: 1 = the convection's He and gpvol spans (4.24 M tets: 0.409
// against 0.430 ms), 2 = the diffusion's, 4 = the diffusion's mu_e, mu_sgs
// rows as well (with 2: 0.381 against 0.363 ms, slower).
#ifndef TET_PREFETCH
#define TET_PREFETCH 1
#endif

namespace msod {
namespace {

__constant__ float c_TNf[16], c_TdNf[48];
__constant__ double c_TNd[16], c_TdNd[48];

template <typename real>
__device__ __forceinline__ real tN(int i);
template <>
__device__ __forceinline__ float tN<float>(int i)
{
    return c_TNf[i];
}
template <>
__device__ __forceinline__ double tN<double>(int i)
{
    return c_TNd[i];
}
template <typename real>
__device__ __forceinline__ real tdN(int i);
template <>
__device__ __forceinline__ float tdN<float>(int i)
{
    return c_TdNf[i];
}
template <>
__device__ __forceinline__ double tdN<double>(int i)
{
    return c_TdNd[i];
}

// 16-byte vectors of real.
template <typename real>
struct Vec16;
template <>
struct Vec16<float> {
    using T = float4;
    static constexpr int W = 4;
    __device__ static void put(const T &v, float *d) { d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w; }
};
template <>
struct Vec16<double> {
    using T = double2;
    static constexpr int W = 2;
    __device__ static void put(const T &v, double *d) { d[0] = v.x; d[1] = v.y; }
};

// NV consecutive values of the element's block (16-byte aligned when VEC).
template <bool VEC, typename real, int NV>
__device__ __forceinline__ void load_block(const real *__restrict__ src, real (&dst)[NV])
{
    if (VEC) {
        using V = Vec16<real>;
        const typename V::T *s = reinterpret_cast<const typename V::T *>(src);
#pragma unroll
        for (int k = 0; k < NV / V::W; ++k) V::put(ldg(s + k), dst + k * V::W);
    } else {
#pragma unroll
        for (int i = 0; i < NV; ++i) dst[i] = ldg(src + i);
    }
}

__device__ __forceinline__ void red_add_v4(float *addr, float a, float b, float c, float d)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Assembly of one residual over the element's nodes.
template <typename real>
__device__ __forceinline__ void assemble(real *__restrict__ dst, const int (&ip)[4], const bool (&ok)[4],
                                         const real (&v)[4], bool v4)
{
    if constexpr (sizeof(real) == 4) {
        if (v4) {
            red_add_v4(dst + ip[0], v[0], v[1], v[2], v[3]);
            return;
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (ok[a]) red_add(dst + ip[a], v[a]);
}

// Node ids of element e; returns whether they are 4k..4k+3 (all valid).
__device__ __forceinline__ bool element_nodes(const int *__restrict__ connec, int nelem, int npoin, int e,
                                              int (&ip)[4], bool (&ok)[4])
{
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int v = ldg(connec + (size_t)a * nelem + e) - 1;
        ok[a] = (unsigned)v < (unsigned)npoin;
        ip[a] = ok[a] ? v : 0;
    }
    return ok[0] && ok[1] && ok[2] && ok[3] && (ip[0] & 3) == 0 && ip[1] == ip[0] + 1 && ip[2] == ip[0] + 2 &&
           ip[3] == ip[0] + 3;
}

// Values of a node field at the element's nodes: one 16-byte load when the
// nodes are 4k..4k+3 and the field array allows it, else one load per node.
template <typename real>
__device__ __forceinline__ void node_values(const real *__restrict__ f, const int (&ip)[4], bool vec, real (&v)[4])
{
    if constexpr (sizeof(real) == 4) {
        if (vec) {
            const float4 x = ldg(reinterpret_cast<const float4 *>(f + ip[0]));
            v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
            return;
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) v[a] = ldg(f + ip[a]);
}

// The block's elements' He(3,3,4) and gpvol(4) spans, and the block's part of
// the four rows of mu(4, nelem) (mu_e, mu_sgs; may be null), into L2.
template <typename real>
__device__ __forceinline__ void prefetch_block_l2(const real *He, const real *gpvol, const real *mu_e,
                                                  const real *mu_sgs, int nelem)
{
    const int e0 = blockIdx.x * blockDim.x, e1 = min(e0 + (int)blockDim.x, nelem);
    if (e0 >= e1) return;
    const size_t ne = (size_t)(e1 - e0);
    prefetch_span_l2(He + (size_t)e0 * 36, ne * 36 * sizeof(real));
    prefetch_span_l2(gpvol + (size_t)e0 * 4, ne * 4 * sizeof(real));
    for (int a = 0; a < 4 && mu_e; ++a) {
        prefetch_span_l2(mu_e + (size_t)a * nelem + e0, ne * sizeof(real));
        prefetch_span_l2(mu_sgs + (size_t)a * nelem + e0, ne * sizeof(real));
    }
}

// gpcar(a, id) = sum_j He(id, j, g) dNgp(j, a, g)   (H = He(:,:,g), He(i,j) at H[j*3+i])
template <typename real>
__device__ __forceinline__ void shape_derivatives(const real *H, int g, real (&gpcar)[4][3])
{
#pragma unroll
    for (int id = 0; id < 3; ++id)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            real dot = (real)0;
#pragma unroll
            for (int j = 0; j < 3; ++j) dot = dot + H[j * 3 + id] * tdN<real>((g * 4 + a) * 3 + j);
            gpcar[a][id] = dot;
        }
}

template <typename real, bool VEC>
__global__ void __launch_bounds__(128, TET_CONVEC_MINB)
    fem_convec_kernel(int nelem, int npoin, const int *__restrict__ connec, const real *__restrict__ He,
                      const real *__restrict__ gpvol, const real *__restrict__ u, const real *__restrict__ q,
                      const real *__restrict__ rho, const real *__restrict__ pr, const real *__restrict__ E,
                      real *__restrict__ Rmass, real *__restrict__ Rmom, real *__restrict__ Rener, int vec_io)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if ((TET_PREFETCH & 1) && threadIdx.x == 0) prefetch_block_l2<real>(He, gpvol, nullptr, nullptr, nelem);
    if (e >= nelem) return;
    const size_t np = (size_t)npoin;
    int ip[4];
    bool ok[4];
    const bool quad = element_nodes(connec, nelem, npoin, e, ip, ok);
    const bool v4 = quad && (vec_io & 1), vin = quad && (vec_io & 2);
    real r[4], p[4], Ep[4], uu[4][3], qq[4][3], t[4];
    node_values(rho, ip, vin, r);
    node_values(pr, ip, vin, p);
    node_values(E, ip, vin, t);
#pragma unroll
    for (int a = 0; a < 4; ++a) Ep[a] = t[a] + p[a];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        node_values(u + c * np, ip, vin, t);
#pragma unroll
        for (int a = 0; a < 4; ++a) uu[a][c] = t[a];
        node_values(q + c * np, ip, vin, t);
#pragma unroll
        for (int a = 0; a < 4; ++a) qq[a][c] = t[a];
    }
    real gv[4], Hb[36];
    load_block<VEC>(gpvol + (size_t)e * 4, gv);
    load_block<VEC>(He + (size_t)e * 36, Hb);
    real Rm[4] = {0, 0, 0, 0}, Re[4] = {0, 0, 0, 0}, Rq[4][3] = {{0}};
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        real gpcar[4][3];
        shape_derivatives(Hb + g * 9, g, gpcar);
        real divQ = 0, divFe = 0, gR[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gP[3] = {0, 0, 0};
        real gU[3][3] = {{0}}, divF[3] = {0, 0, 0};
#pragma unroll
        for (int id = 0; id < 3; ++id)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const real c = gpcar[j][id];
                divQ = divQ + c * qq[j][id];
                divFe = divFe + c * Ep[j] * uu[j][id];
                gR[id] = gR[id] + c * r[j];
                gE[id] = gE[id] + c * Ep[j];
                gP[id] = gP[id] + c * p[j];
#pragma unroll
                for (int jd = 0; jd < 3; ++jd) {
                    gU[id][jd] = gU[id][jd] + gpcar[j][jd] * uu[j][id];
                    divF[id] = divF[id] + gpcar[j][jd] * qq[j][id] * uu[j][jd];
                }
            }
        const real divU = gU[0][0] + gU[1][1] + gU[2][2];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            real aux1 = 0, aux2 = 0;
#pragma unroll
            for (int id = 0; id < 3; ++id) {
                aux1 = aux1 + gR[id] * uu[a][id];
                aux2 = aux2 + gE[id] * uu[a][id];
            }
            const real w = gv[g] * tN<real>(a * 4 + g) * (real)0.5;  // Ngp(igaus, inode)
            Rm[a] = Rm[a] + w * (divQ + r[a] * divU + aux1);
            Re[a] = Re[a] + w * (divFe + Ep[a] * divU + aux2);
#pragma unroll
            for (int id = 0; id < 3; ++id) {
                real aux3 = 0, aux4 = 0;
#pragma unroll
                for (int jd = 0; jd < 3; ++jd) {
                    aux3 = aux3 + gU[id][jd] * qq[a][jd];
                    aux4 = aux4 + uu[a][id] * uu[a][jd] * gR[jd];
                }
                Rq[a][id] = Rq[a][id] + w * (divF[id] + qq[a][id] * divU + aux3 + aux4 + gP[id]);
            }
        }
    }
    assemble(Rmass, ip, ok, Rm, v4);
    assemble(Rener, ip, ok, Re, v4);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const real v[4] = {Rq[0][c], Rq[1][c], Rq[2][c], Rq[3][c]};
        assemble(Rmom + c * np, ip, ok, v, v4);
    }
}

template <typename real, bool VEC>
__global__ void __launch_bounds__(128, TET_DIFFU_MINB)
    fem_diffu_kernel(int nelem, int npoin, const int *__restrict__ connec, const real *__restrict__ He,
                     const real *__restrict__ gpvol, real Cp, real Pr, const real *__restrict__ rho,
                     const real *__restrict__ u, const real *__restrict__ Tem, const real *__restrict__ mu_fluid,
                     const real *__restrict__ mu_e, const real *__restrict__ mu_sgs, real *__restrict__ Rmass,
                     real *__restrict__ Rmom, real *__restrict__ Rener, int vec_io)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if ((TET_PREFETCH & 2) && threadIdx.x == 0)
        prefetch_block_l2<real>(He, gpvol, (TET_PREFETCH & 4) ? mu_e : nullptr, mu_sgs, nelem);
    if (e >= nelem) return;
    const size_t np = (size_t)npoin;
    int ip[4];
    bool ok[4];
    const bool quad = element_nodes(connec, nelem, npoin, e, ip, ok);
    const bool v4 = quad && (vec_io & 1), vin = quad && (vec_io & 2);
    real r[4], T[4], mf[4], me[4], ms[4], uu[4][3], t[4];
    node_values(rho, ip, vin, r);
    node_values(Tem, ip, vin, T);
    node_values(mu_fluid, ip, vin, mf);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        me[a] = ldg(mu_e + (size_t)a * nelem + e);
        ms[a] = ldg(mu_sgs + (size_t)a * nelem + e);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        node_values(u + c * np, ip, vin, t);
#pragma unroll
        for (int a = 0; a < 4; ++a) uu[a][c] = t[a];
    }
    real gv[4], Hb[36];
    load_block<VEC>(gpvol + (size_t)e * 4, gv);
    load_block<VEC>(He + (size_t)e * 36, Hb);
    const real c_rho = (real)1, c_ener = (real)1, CpPr = Cp / Pr;
    real Rm[4] = {0, 0, 0, 0}, Re[4] = {0, 0, 0, 0}, Rq[4][3] = {{0}};
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        // Ngp(inode, igaus): fem_diffu reads the table transposed (elem_diffu.f90:232-239).
        real auxRho = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) auxRho = auxRho + tN<real>(g * 4 + a) * r[a];
        const real rinv = c_rho / auxRho;
        real auxNu = 0, auxMu = 0, auxKappa = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const real N = tN<real>(g * 4 + a);
            auxNu = auxNu + N * me[a] * rinv;
            auxMu = auxMu + N * (mf[a] + auxRho * ms[a] + me[a]);
            auxKappa = auxKappa + N * (mf[a] * CpPr + c_ener * me[a] / (real)0.4 + auxRho * ms[a] / (real)0.9);
        }
        real gpcar[4][3];
        shape_derivatives(Hb + g * 9, g, gpcar);
        real gR[3] = {0, 0, 0}, gT[3] = {0, 0, 0}, gU[3][3] = {{0}};
#pragma unroll
        for (int id = 0; id < 3; ++id)
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                gR[id] = gR[id] + gpcar[a][id] * r[a];
                gT[id] = gT[id] + gpcar[a][id] * T[a];
#pragma unroll
                for (int jd = 0; jd < 3; ++jd) gU[id][jd] = gU[id][jd] + gpcar[a][id] * uu[a][jd];
            }
        const real divU = gU[0][0] + gU[1][1] + gU[2][2];
        real tau[3][3], tauU[3] = {0, 0, 0};
#pragma unroll
        for (int id = 0; id < 3; ++id)
#pragma unroll
            for (int jd = 0; jd < 3; ++jd)
                tau[id][jd] = (id == jd ? -((real)2 / (real)3 * divU) : (real)0) + gU[id][jd] + gU[jd][id];
#pragma unroll
        for (int jd = 0; jd < 3; ++jd) {
            real auxU = 0;
#pragma unroll
            for (int a = 0; a < 4; ++a) auxU = auxU + tN<real>(g * 4 + a) * uu[a][jd];
#pragma unroll
            for (int id = 0; id < 3; ++id) tauU[id] = tauU[id] + tau[id][jd] * auxU;
        }
#pragma unroll
        for (int id = 0; id < 3; ++id)
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                Rm[a] = Rm[a] + gv[g] * auxNu * gpcar[a][id] * gR[id];
                Re[a] = Re[a] + gv[g] * gpcar[a][id] * (auxMu * tauU[id] + auxKappa * gT[id]);
#pragma unroll
                for (int jd = 0; jd < 3; ++jd) Rq[a][id] = Rq[a][id] + gv[g] * gpcar[a][jd] * auxMu * tau[id][jd];
            }
    }
    assemble(Rmass, ip, ok, Rm, v4);
    assemble(Rener, ip, ok, Re, v4);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const real v[4] = {Rq[0][c], Rq[1][c], Rq[2][c], Rq[3][c]};
        assemble(Rmom + c * np, ip, ok, v, v4);
    }
}

__global__ void check_connec_kernel(long long count, int npoin, const int *__restrict__ connec, int *flags)
{
    int bad = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const int v = ldg(connec + i);
        if (v < 1 || v > npoin) bad = 1;
    }
    if (bad) atomicOr(flags, 8);
}

template <typename real>
cudaError_t copy_tables(const real *Ngp, const real *dNgp, cudaStream_t st)
{
    cudaError_t err;
    if (sizeof(real) == 4) {
        err = cudaMemcpyToSymbolAsync(c_TNf, Ngp, 16 * sizeof(float), 0, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess)
            err = cudaMemcpyToSymbolAsync(c_TdNf, dNgp, 48 * sizeof(float), 0, cudaMemcpyDeviceToDevice, st);
    } else {
        err = cudaMemcpyToSymbolAsync(c_TNd, Ngp, 16 * sizeof(double), 0, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess)
            err = cudaMemcpyToSymbolAsync(c_TdNd, dNgp, 48 * sizeof(double), 0, cudaMemcpyDeviceToDevice, st);
    }
    return err;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

template <typename real>
cudaError_t launch_fem_convec(const TetConvecArgs<real> &a, cudaStream_t st)
{
    cudaError_t err = copy_tables(a.Ngp, a.dNgp, st);
    if (err != cudaSuccess) return err;
    const bool vec = aligned16(a.gpvol) && aligned16(a.He);
    const bool np4 = (a.npoin % 4) == 0;
    const int vec_io = (np4 && aligned16(a.Rmass) && aligned16(a.Rmom) && aligned16(a.Rener) ? 1 : 0) |
                       (np4 && aligned16(a.rho) && aligned16(a.pr) && aligned16(a.E) && aligned16(a.u) &&
                                aligned16(a.q) ? 2 : 0);
    const unsigned grid = (unsigned)((a.nelem + 127) / 128);
    if (vec)
        fem_convec_kernel<real, true><<<grid, 128, 0, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.u, a.q,
                                                            a.rho, a.pr, a.E, a.Rmass, a.Rmom, a.Rener, vec_io);
    else
        fem_convec_kernel<real, false><<<grid, 128, 0, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.u, a.q,
                                                             a.rho, a.pr, a.E, a.Rmass, a.Rmom, a.Rener, vec_io);
    return cudaGetLastError();
}

template <typename real>
cudaError_t launch_fem_diffu(const TetDiffuArgs<real> &a, cudaStream_t st)
{
    cudaError_t err = copy_tables(a.Ngp, a.dNgp, st);
    if (err != cudaSuccess) return err;
    const bool vec = aligned16(a.gpvol) && aligned16(a.He);
    const bool np4 = (a.npoin % 4) == 0;
    const int vec_io = (np4 && aligned16(a.Rmass) && aligned16(a.Rmom) && aligned16(a.Rener) ? 1 : 0) |
                       (np4 && aligned16(a.rho) && aligned16(a.Tem) && aligned16(a.mu_fluid) && aligned16(a.u)
                            ? 2 : 0);
    const unsigned grid = (unsigned)((a.nelem + 127) / 128);
    if (vec)
        fem_diffu_kernel<real, true><<<grid, 128, 0, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.Cp, a.Pr,
                                                           a.rho, a.u, a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs, a.Rmass,
                                                           a.Rmom, a.Rener, vec_io);
    else
        fem_diffu_kernel<real, false><<<grid, 128, 0, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.Cp, a.Pr,
                                                            a.rho, a.u, a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs,
                                                            a.Rmass, a.Rmom, a.Rener, vec_io);
    return cudaGetLastError();
}

cudaError_t launch_check_connec(long long count, int npoin, const int *connec, int *flags, cudaStream_t st)
{
    long long blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    check_connec_kernel<<<(unsigned)blocks, 256, 0, st>>>(count, npoin, connec, flags);
    return cudaGetLastError();
}

template cudaError_t launch_fem_convec<float>(const TetConvecArgs<float> &, cudaStream_t);
template cudaError_t launch_fem_convec<double>(const TetConvecArgs<double> &, cudaStream_t);
template cudaError_t launch_fem_diffu<float>(const TetDiffuArgs<float> &, cudaStream_t);
template cudaError_t launch_fem_diffu<double>(const TetDiffuArgs<double> &, cudaStream_t);

}  // namespace msod
