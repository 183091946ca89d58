// msod_setup.cu -- device-side element setup and table validation.
//
// elem_jacobian (jacobian_oper.f90:7-136) runs on the device as in the
// reference (an OpenACC gang loop there): one block per element, one thread
// per GLL point.  The element's node coordinates are gathered once into
// shared memory; every product and sum is explicitly rounded (no fused
// multiply-add) in the reference's order, so the result matches a
// -ffp-contract=off CPU build bit for bit.
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

namespace msod {
namespace {

__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

template <typename real>
__global__ void elem_jacobian_kernel(int n, int nelem, int npoin, const int *__restrict__ connec,
                                     const real *__restrict__ coord, const real *__restrict__ dNgp,
                                     const real *__restrict__ wgp, real *__restrict__ gpvol, real *__restrict__ He)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real *sx = reinterpret_cast<real *>(smem_raw);  // [3][n]
    const int e = blockIdx.x;
    for (int a = threadIdx.x; a < n; a += blockDim.x) {
        int p = ldg(connec + (size_t)a * nelem + e) - 1;
        p = min(max(p, 0), npoin - 1);
#pragma unroll
        for (int d = 0; d < 3; ++d) sx[d * n + a] = ldg(coord + (size_t)d * npoin + p);
    }
    __syncthreads();
    for (int g = threadIdx.x; g < n; g += blockDim.x) {
        real J[3][3];
        const real *dn = dNgp + (size_t)g * n * 3;
        for (int id = 0; id < 3; ++id)
            for (int jd = 0; jd < 3; ++jd) {
                real dot = (real)0;
                for (int a = 0; a < n; ++a) dot = radd(dot, rmul(ldg(dn + a * 3 + id), sx[jd * n + a]));
                J[id][jd] = radd((real)0, dot);
            }
        // det = J11 J22 J33 + J12 J23 J31 + J13 J21 J32 - J31 J22 J13 - J32 J23 J11 - J33 J21 J12
        real det = rmul(rmul(J[0][0], J[1][1]), J[2][2]);
        det = radd(det, rmul(rmul(J[0][1], J[1][2]), J[2][0]));
        det = radd(det, rmul(rmul(J[0][2], J[1][0]), J[2][1]));
        det = rsub(det, rmul(rmul(J[2][0], J[1][1]), J[0][2]));
        det = rsub(det, rmul(rmul(J[2][1], J[1][2]), J[0][0]));
        det = rsub(det, rmul(rmul(J[2][2], J[1][0]), J[0][1]));
        real a[9];
        a[0] = rsub(rmul(J[1][1], J[2][2]), rmul(J[2][1], J[1][2]));
        a[1] = rsub(rmul(J[1][0], J[2][2]), rmul(J[2][0], J[1][2]));
        a[2] = rsub(rmul(J[1][0], J[2][1]), rmul(J[2][0], J[1][1]));
        a[3] = rsub(rmul(J[0][1], J[2][2]), rmul(J[2][1], J[0][2]));
        a[4] = rsub(rmul(J[0][0], J[2][2]), rmul(J[2][0], J[0][2]));
        a[5] = rsub(rmul(J[0][0], J[2][1]), rmul(J[2][0], J[0][1]));
        a[6] = rsub(rmul(J[0][1], J[1][2]), rmul(J[1][1], J[0][2]));
        a[7] = rsub(rmul(J[0][0], J[1][2]), rmul(J[1][0], J[0][2]));
        a[8] = rsub(rmul(J[0][0], J[1][1]), rmul(J[1][0], J[0][1]));
        a[1] = -a[1]; a[3] = -a[3]; a[5] = -a[5]; a[7] = -a[7];
        // b = transpose of the cofactors (row-major b[i*3+j] = He(i,j)), then / det.
        const int tr[9] = {0, 3, 6, 1, 4, 7, 2, 5, 8};
        const real rdet = rdiv((real)1, det);
        real *H = He + ((size_t)e * n + g) * 9;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) H[j * 3 + i] = rmul(rdet, a[tr[i * 3 + j]]);
        gpvol[(size_t)e * n + g] = rmul(ldg(wgp + g), det);
    }
}

// Validation of one element's tables (block 0) plus a grid-stride range check
// of connec.  Failure bits: 1 invAtoIJK not a permutation, 2 invAtoIJK and
// gmshAtoI/J/K disagree, 4 dlxigp_ip lacks the per-direction 1-D structure,
// 8 a connec entry outside 1..npoin.
__global__ void check_tables_kernel(int P, int nelem, int npoin, const int *__restrict__ connec,
                                    const float *__restrict__ dlxigp_ip, const int *__restrict__ inv,
                                    const int *__restrict__ AtoI, const int *__restrict__ AtoJ,
                                    const int *__restrict__ AtoK, int *flags)
{
    const int Q = P + 1, n = Q * Q * Q;
    int bits = 0;
    if (blockIdx.x == 0) {
        for (int l = threadIdx.x; l < n; l += blockDim.x) {
            const int a = inv[l];
            if (a < 1 || a > n) { bits |= 1; continue; }
            int cnt = 0;
            for (int m = 0; m < n; ++m) cnt += (inv[m] == a);
            if (cnt != 1) bits |= 1;
            const int I = l % Q + 1, J = (l / Q) % Q + 1, K = l / (Q * Q) + 1;
            if (AtoI[a - 1] != I || AtoJ[a - 1] != J || AtoK[a - 1] != K) bits |= 2;
        }
        __syncthreads();
        if (!bits) {
            // dlxigp_ip(g,d,c) must equal dlxigp_ip(g',d,c) whenever g and g' share
            // the 1-D index in direction d.
            for (int i = threadIdx.x; i < n * 3 * Q; i += blockDim.x) {
                const int g = i % n, d = (i / n) % 3, c = i / (3 * n);
                int I = AtoI[g] - 1, J = AtoJ[g] - 1, K = AtoK[g] - 1;
                if (I < 0 || J < 0 || K < 0 || I >= Q || J >= Q || K >= Q) { bits |= 2; continue; }
                const int r = d == 0 ? I : (d == 1 ? J : K);
                const int l0 = d == 0 ? r : (d == 1 ? r * Q : r * Q * Q);
                const int g0 = inv[l0] - 1;
                if (g0 < 0 || g0 >= n) { bits |= 1; continue; }
                const float v = dlxigp_ip[(size_t)(c * 3 + d) * n + g];
                const float v0 = dlxigp_ip[(size_t)(c * 3 + d) * n + g0];
                if (__float_as_int(v) != __float_as_int(v0)) bits |= 4;
            }
        }
    }
    const size_t total = (size_t)nelem * n;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int v = connec[i];
        if (v < 1 || v > npoin) bits |= 8;
    }
    if (bits) atomicOr(flags, bits);
}

}  // namespace

template <typename real>
cudaError_t launch_jacobian_nodes(int n, int nelem, int npoin, const int *connec, const real *coord,
                                  const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st)
{
    const int threads = n <= 32 ? 32 : (n <= 128 ? 128 : (n <= 256 ? 256 : (n <= 512 ? 512 : 768)));
    const size_t smem = 3 * (size_t)n * sizeof(real);
    elem_jacobian_kernel<real><<<nelem, threads, smem, st>>>(n, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He);
    return cudaGetLastError();
}

template <typename real>
cudaError_t launch_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const real *coord,
                                 const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st)
{
    const int n = (porder + 1) * (porder + 1) * (porder + 1);
    return launch_jacobian_nodes<real>(n, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, st);
}

template cudaError_t launch_jacobian_nodes<float>(int, int, int, const int *, const float *, const float *,
                                                  const float *, float *, float *, cudaStream_t);
template cudaError_t launch_jacobian_nodes<double>(int, int, int, const int *, const double *, const double *,
                                                   const double *, double *, double *, cudaStream_t);

template cudaError_t launch_elem_jacobian<float>(int, int, int, const int *, const float *, const float *,
                                                 const float *, float *, float *, cudaStream_t);
template cudaError_t launch_elem_jacobian<double>(int, int, int, const int *, const double *, const double *,
                                                  const double *, double *, double *, cudaStream_t);

cudaError_t launch_check_tables(int porder, int nelem, int npoin, const int *connec, const float *dlxigp_ip,
                                const int *invAtoIJK, const int *AtoI, const int *AtoJ, const int *AtoK, int *flags,
                                cudaStream_t st)
{
    const size_t total = (size_t)nelem * (porder + 1) * (porder + 1) * (porder + 1);
    size_t blocks = (total + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 4096) blocks = 4096;
    check_tables_kernel<<<(unsigned)blocks, 256, 0, st>>>(porder, nelem, npoin, connec, dlxigp_ip, invAtoIJK, AtoI,
                                                          AtoJ, AtoK, flags);
    return cudaGetLastError();
}

}  // namespace msod
