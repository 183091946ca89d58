// msod_tables.cu -- per-call element tables for the line-parallel kernels.
//
// Every kernel call first runs table_prep_kernel, one block that reads the
// caller's dlxigp_ip / invAtoIJK / gmshAtoI/J/K (device arrays in the
// reference's layouts) and writes, into a small library-owned device area:
//   perm[l]  lattice point l = (K*Q+J)*Q+I (SOD 1-D indices) -> gmsh node a
//   lat[a]   gmsh node a -> padded shared-memory lattice offset (K*Q+J)*QP+I
//   D[d][r][c] = dlxigp_ip(g, d, c) for a point g whose 1-D index in
//            direction d is r: the 1-D derivative matrix the reference
//            replicates per point (elem_hex.f90:43-44, mod_maths.f90:274-281).
// The kernels copy D into their constant bank (so the contractions take
// their coefficients as constant operands) and perm/lat into shared memory.
// Indices are clamped, so malformed tables give wrong numbers (reported by
// msod_check_element_tables), never out-of-bounds accesses.
#include <cuda_runtime.h>

#include "msod_device.cuh"
#include "msod_kernels.h"

namespace msod {
namespace {

template <typename real, int P>
__global__ void table_prep_kernel(const int *__restrict__ invAtoIJK, const int *__restrict__ AtoI,
                                  const int *__restrict__ AtoJ, const int *__restrict__ AtoK,
                                  const real *__restrict__ dlxigp_ip, TableScratch *out)
{
    using G = LineGeom<real, P>;
    constexpr int Q = G::Q, N = G::N;
    __shared__ int sperm[N];
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const int a = min(max(invAtoIJK[i] - 1, 0), N - 1);
        sperm[i] = a;
        out->perm[i] = a;
        const int I = min(max(AtoI[i] - 1, 0), Q - 1);
        const int J = min(max(AtoJ[i] - 1, 0), Q - 1);
        const int K = min(max(AtoK[i] - 1, 0), Q - 1);
        out->lat[i] = (K * Q + J) * G::QP + I;
    }
    __syncthreads();
    real *D = table_D<real>(out);
    for (int i = threadIdx.x; i < 3 * Q * Q; i += blockDim.x) {
        const int d = i / (Q * Q), r = (i / Q) % Q, c = i % Q;
        const int l = d == 0 ? r : (d == 1 ? r * Q : r * Q * Q);
        D[i] = dlxigp_ip[(size_t)(c * 3 + d) * N + sperm[l]];
    }
    if (sizeof(real) == 4) {
        __syncthreads();  // D complete
        // Even-odd form and its validity: the directions' matrices equal, the
        // matrix centro-antisymmetric to within 1e-6 of its largest entry.
        constexpr int M = Q / 2, mc = sod_centre(Q);
        const float *Dv = out->Df;
        for (int i = threadIdx.x; i < M * M; i += blockDim.x) {
            const int r = sod_left(i / M), c = sod_left(i % M), cm = sod_mirror(Q, c);
            out->EO[i] = 0.5f * (Dv[r * Q + c] - Dv[r * Q + cm]);
            out->EO[M * M + i] = 0.5f * (Dv[r * Q + c] + Dv[r * Q + cm]);
            out->EOp[2 * i] = out->EO[i];
            out->EOp[2 * i + 1] = out->EO[M * M + i];
        }
        if (Q % 2 == 1)
            for (int i = threadIdx.x; i < M; i += blockDim.x) {
                out->EO[2 * M * M + i] = Dv[sod_left(i) * Q + mc];
                out->EO[2 * M * M + M + i] = Dv[mc * Q + sod_left(i)];
            }
        if (threadIdx.x == 0) {
            float big = 0.0f;
            for (int i = 0; i < Q * Q; ++i) big = fmaxf(big, fabsf(Dv[i]));
            const float tol = 1e-6f * big;
            bool ok = true;
            for (int i = 0; i < Q * Q; ++i) {
                const int r = i / Q, c = i % Q;
                ok = ok && Dv[Q * Q + i] == Dv[i] && Dv[2 * Q * Q + i] == Dv[i];
                ok = ok && fabsf(Dv[sod_mirror(Q, r) * Q + sod_mirror(Q, c)] + Dv[i]) <= tol;
            }
            out->eo_ok = ok ? 1 : 0;
        }
        constexpr int H = (Q + 1) / 2;
        for (int i = threadIdx.x; i < 3 * Q * H * 2; i += blockDim.x) {
            const int t = i & 1, m = (i >> 1) % H, c = (i >> 1) / H % Q, d = (i >> 1) / (H * Q);
            const int r = 2 * m + t;
            float v = 0.0f;
            if (r < Q) {
                const int l = d == 0 ? r : (d == 1 ? r * Q : r * Q * Q);
                v = (float)dlxigp_ip[(size_t)(c * 3 + d) * N + sperm[l]];
            }
            out->Dp[i] = v;
        }
    }
}

template <typename real, int P>
cudaError_t prep_p(const ElementArgs<real> &a, TableScratch *scratch, cudaStream_t st)
{
    table_prep_kernel<real, P><<<1, 256, 0, st>>>(a.invAtoIJK, a.AtoI, a.AtoJ, a.AtoK, a.dlxigp_ip, scratch);
    return cudaGetLastError();
}

}  // namespace

template <typename real>
cudaError_t launch_table_prep(int porder, const ElementArgs<real> &a, TableScratch *scratch, cudaStream_t st)
{
    switch (porder) {
    case 1: return prep_p<real, 1>(a, scratch, st);
    case 2: return prep_p<real, 2>(a, scratch, st);
    case 3: return prep_p<real, 3>(a, scratch, st);
    case 4: return prep_p<real, 4>(a, scratch, st);
    case 5: return prep_p<real, 5>(a, scratch, st);
    case 6: return prep_p<real, 6>(a, scratch, st);
    case 7: return prep_p<real, 7>(a, scratch, st);
    case 8: return prep_p<real, 8>(a, scratch, st);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_table_prep<float>(int, const ElementArgs<float> &, TableScratch *, cudaStream_t);
template cudaError_t launch_table_prep<double>(int, const ElementArgs<double> &, TableScratch *, cudaStream_t);

}  // namespace msod
