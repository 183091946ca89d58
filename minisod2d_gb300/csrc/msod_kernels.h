// msod_kernels.h -- launcher interfaces between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

#include "msod.h"

namespace msod {

// Per-call element tables written by table_prep_kernel (msod_tables.cu) into a
// library-owned device area: the 1-D derivative matrices D[d][r][c] (FP32 and
// FP64 copies), lattice -> gmsh node (perm) and gmsh node -> padded lattice
// offset (lat).
constexpr int kTableDMax = 3 * (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1);
constexpr int kTableNMax = (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1);
struct TableScratch {
    float Df[kTableDMax];
    double Dd[kTableDMax];
    int perm[kTableNMax];
    int lat[kTableNMax];
};
template <typename real>
__host__ __device__ inline real *table_D(TableScratch *t);
template <>
__host__ __device__ inline float *table_D<float>(TableScratch *t)
{
    return t->Df;
}
template <>
__host__ __device__ inline double *table_D<double>(TableScratch *t)
{
    return t->Dd;
}
template <typename real>
__host__ __device__ inline const real *table_D(const TableScratch *t)
{
    return table_D<real>(const_cast<TableScratch *>(t));
}

template <typename real>
struct ElementArgs {
    int nelem, npoin;
    const int *connec;
    const real *He, *gpvol, *dlxigp_ip;
    const int *invAtoIJK, *AtoI, *AtoJ, *AtoK;
};

template <typename real>
struct ConvecArgs : ElementArgs<real> {
    const real *u, *q, *rho, *pr, *E;
    real *Rmass, *Rmom, *Rener;
};

template <typename real>
struct DiffuArgs : ElementArgs<real> {
    real Cp, Pr;
    const real *rho, *u, *Tem, *mu_fluid, *mu_e, *mu_sgs;
    real *Rmass, *Rmom, *Rener;
};

// Tables of one call (one block, stream-ordered before the kernels).
template <typename real>
cudaError_t launch_table_prep(int porder, const ElementArgs<real> &a, TableScratch *scratch, cudaStream_t st);

// Plain kernels (outputs must be zeroed by the caller; tables prepared).
template <typename real>
cudaError_t launch_convec_plain(int porder, const ConvecArgs<real> &a, const TableScratch *tabs, cudaStream_t st);
template <typename real>
cudaError_t launch_diffu_plain(int porder, const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st);

// Setup kernels.
template <typename real>
cudaError_t launch_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const real *coord,
                                 const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st);

// Validation: accumulates failure bits into *flags (device int).
cudaError_t launch_check_tables(int porder, int nelem, int npoin, const int *connec, const float *dlxigp_ip,
                                const int *invAtoIJK, const int *AtoI, const int *AtoJ, const int *AtoK,
                                int *flags, cudaStream_t st);

}  // namespace msod
