// msod_kernels.h -- launcher interfaces between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

namespace msod {

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

// Plain kernels (outputs must be zeroed by the caller).
template <typename real>
cudaError_t launch_convec_plain(int porder, const ConvecArgs<real> &a, cudaStream_t st);
template <typename real>
cudaError_t launch_diffu_plain(int porder, const DiffuArgs<real> &a, cudaStream_t st);

// Setup kernels.
template <typename real>
cudaError_t launch_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const real *coord,
                                 const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st);

// Validation: accumulates failure bits into *flags (device int).
cudaError_t launch_check_tables(int porder, int nelem, int npoin, const int *connec, const float *dlxigp_ip,
                                const int *invAtoIJK, const int *AtoI, const int *AtoJ, const int *AtoK,
                                int *flags, cudaStream_t st);

}  // namespace msod
