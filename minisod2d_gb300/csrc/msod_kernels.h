// msod_kernels.h -- launcher interfaces between the C-ABI layer and the kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "msod.h"

namespace msod {

// Per-call element tables written by table_prep_kernel (msod_tables.cu) into a
// library-owned device area: the 1-D derivative matrices D[d][r][c] (FP32 and
// FP64 copies), lattice -> gmsh node (perm) and gmsh node -> padded lattice
// offset (lat).
constexpr int kTableDMax = 3 * (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1);
constexpr int kTableNMax = (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 1);
// Row pairs of the FP32 matrices for packed (f32x2) contractions:
// Dp[((d*Q + c)*H + m)*2 + t] = D[d][2m+t][c] (zero for 2m+t = Q), H = (Q+1)/2.
constexpr int kTableDPairMax = 3 * (MSOD_MAX_PORDER + 1) * (MSOD_MAX_PORDER + 2);
// Even-odd form of the FP32 matrix (one direction), valid when the three
// directions' matrices are equal and centro-antisymmetric, as the GLL
// derivative matrix is: D[s'(r)][s'(c)] = -D[r][c] where s' mirrors a node
// through the element centre.  Lines are stored in the reference's SOD 1-D
// order (the two ends first, then the interior: natural indices 0, P, 1, ...,
// P-1), where the mirror is sod_mirror.  With M = Q/2 mirror pairs (L_i,
// s'(L_i)), L_i = sod_left(i), and for odd Q the centre node m:
//   EO[i*M + j]           A = (D[L_i][L_j] - D[L_i][s'(L_j)]) / 2
//   EO[M*M + i*M + j]     B = (D[L_i][L_j] + D[L_i][s'(L_j)]) / 2
//   EO[2*M*M + i]         D[L_i][m]                         (odd Q)
//   EO[2*M*M + M + j]     D[m][L_j]                         (odd Q)
// so that, with e_j = v[L_j] + v[s'(L_j)] and o_j = v[L_j] - v[s'(L_j)],
// d[L_i] = S_i + T_i and d[s'(L_i)] = S_i - T_i for S_i = sum_j A o_j and
// T_i = sum_j B e_j (+ D[L_i][m] v[m]), and d[m] = sum_j D[m][L_j] o_j.
__host__ __device__ constexpr int sod_mirror(int Q, int s) { return s == 0 ? 1 : (s == 1 ? 0 : Q + 1 - s); }
__host__ __device__ constexpr int sod_left(int i) { return i == 0 ? 0 : i + 1; }
__host__ __device__ constexpr int sod_centre(int Q) { return (Q + 1) / 2; }
constexpr int kTableEOMax = 2 * (MSOD_MAX_PORDER / 2 + 1) * (MSOD_MAX_PORDER / 2 + 1) + 2 * (MSOD_MAX_PORDER / 2 + 1);
struct TableScratch {
    float Df[kTableDMax];
    float EO[kTableEOMax];
    int eo_ok;  // 1 when EO represents all three directions' matrices
    // The even-odd A and B entries side by side, for packed (f32x2)
    // contractions: EOp[2*(i*M + j)] = A[i][j], EOp[2*(i*M + j) + 1] = B[i][j].
    alignas(8) float EOp[kTableEOMax];
    double Dd[kTableDMax];
    alignas(8) float Dp[kTableDPairMax];
    int perm[kTableNMax];
    int lat[kTableNMax];
    // Set (sticky, zero at allocation) by a kernel whose bounded wait for a
    // bulk copy into shared memory ran out; the kernel then skipped its work.
    // Checked mode reads and clears it after each call.
    int wait_fault;
};

// Records a bounded wait that ran out (see TableScratch::wait_fault).
__device__ __forceinline__ void report_wait_fault(const TableScratch *t)
{
    atomicOr(const_cast<int *>(&t->wait_fault), 1);
}
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

struct MlpNorm;

template <typename real>
struct DiffuArgs : ElementArgs<real> {
    real Cp, Pr;
    const real *rho, *u, *Tem, *mu_fluid, *mu_e, *mu_sgs;
    const real *nu_elem;  // if set: mu_e(e, a) = rho(a) * nu_elem[e] and mu_e is not read
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
// Both plain FP32 kernels on the same inputs (outputs zeroed by the caller;
// tables prepared): one kernel where fused_porder(porder), else the two
// kernels in turn.  The convection and diffusion outputs must not overlap.
bool fused_porder(int porder);
cudaError_t launch_fused(int porder, const ConvecArgs<float> &c, const DiffuArgs<float> &d, const TableScratch *tabs,
                         cudaStream_t st);

// Mixed-precision convection: FP32 fields, FP64 residuals (zeroed by the
// caller; tables prepared).  precision: MSOD_PREC_FP16 or MSOD_PREC_BF16.
struct MixedConvecArgs {
    int nelem, npoin;
    const int *connec;
    const float *He, *gpvol;
    const float *u, *q, *rho, *pr, *E;
    double *Rmass, *Rmom, *Rener;
};
cudaError_t launch_convec_mixed(int porder, int precision, const MixedConvecArgs &a,
                                const TableScratch *tabs, cudaStream_t st);

// Mixed-precision diffusion: FP32 fields, FP64 residuals (zeroed by the
// caller; tables prepared).  nu_elem set: mu_e(e, a) = rho(a) nu_elem[e] and
// mu_e is not read.
struct MixedDiffuArgs {
    int nelem, npoin;
    const int *connec;
    const float *He, *gpvol;
    float Cp, Pr;
    const float *rho, *u, *Tem, *mu_fluid, *mu_e, *mu_sgs, *nu_elem;
    double *Rmass, *Rmom, *Rener;
};
cudaError_t launch_diffu_mixed(int porder, int precision, const MixedDiffuArgs &a, const TableScratch *tabs,
                               cudaStream_t st);

// ---------------------------------------------------------------------------
// Entropy viscosity and the learned estimator
// ---------------------------------------------------------------------------
struct EntropyStats {
    double sum;  // sum of eta over the nodes
    int kmin;    // order-preserving int keys of min / max eta
    int kmax;
};

constexpr int kMlpIn = 12, kMlpH = 32;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH;
constexpr int kMlpParams = kOffB3 + 1;  // 1505
static_assert(kMlpParams == MSOD_MLP_NPARAMS, "parameter count");

struct MlpNorm {
    float mean[kMlpIn], inv_std[kMlpIn], fmin[kMlpIn], fmax[kMlpIn];
};

// Linear tetrahedra (fem_convec, fem_diffu): 4 nodes, 4 Gauss points; tables
// Ngp(4,4), dNgp(3,4,4) are device arrays in the reference's layouts.
template <typename real>
struct TetConvecArgs {
    int nelem, npoin;
    const int *connec;
    const real *Ngp, *dNgp, *He, *gpvol;
    const real *u, *q, *rho, *pr, *E;
    real *Rmass, *Rmom, *Rener;
};
template <typename real>
struct TetDiffuArgs {
    int nelem, npoin;
    const int *connec;
    const real *Ngp, *dNgp, *He, *gpvol;
    real Cp, Pr;
    const real *rho, *u, *Tem, *mu_fluid, *mu_e, *mu_sgs;
    real *Rmass, *Rmom, *Rener;
};
template <typename real>
cudaError_t launch_fem_convec(const TetConvecArgs<real> &a, cudaStream_t st);
template <typename real>
cudaError_t launch_fem_diffu(const TetDiffuArgs<real> &a, cudaStream_t st);
// Range check of count connec entries against 1..npoin (sets bit 8 of flags).
cudaError_t launch_check_connec(long long count, int npoin, const int *connec, int *flags, cudaStream_t st);
// Jacobian of elements with n nodes = n points (elem_jacobian / tet_jacobian).
template <typename real>
cudaError_t launch_jacobian_nodes(int n, int nelem, int npoin, const int *connec, const real *coord,
                                  const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st);

struct ViscArgs {
    int nelem, npoin;
    const int *connec;
    const float *He, *gpvol, *dlxigp_ip;
    const int *invAtoIJK, *AtoI, *AtoJ, *AtoK;
    const float *rho, *u, *p_or_T;
    float Rgas, gamma, ce, cmax;
    int normalise;
    const EntropyStats *stats;
    // If set: process only the elements list[0 .. *count) (the compacted list
    // of flagged elements written by launch_mlp_predict), write nu only.
    const int *list, *count;
    float *mu_e, *nu, *numax;
    const TableScratch *tabs;  // the call's element tables (table_prep_kernel)
};

struct FeatureArgs {
    int nelem, npoin;
    const int *connec;
    const float *He, *gpvol;
    const TableScratch *tabs;
    const float *rho, *u, *p_or_T;
    float Rgas, gamma, cmax;
    const EntropyStats *stats;
    float *feat, *numax;
};

cudaError_t launch_entropy_stats(int npoin, const float *rho, const float *p_or_T, float Rgas, float gamma,
                                 EntropyStats *st, cudaStream_t s);
cudaError_t launch_entropy_visc(int porder, const ViscArgs &a, cudaStream_t st);
cudaError_t launch_features(int porder, const FeatureArgs &a, cudaStream_t st);
// y = 10^-s, nu = y numax (if nu), flag = 1 outside the training range (if
// flag); with list: list[0 .. *count) = the flagged elements (any order).
cudaError_t launch_mlp_predict(int nelem, const float *feat, const __half *wh, const MlpNorm *nm, const float *numax,
                               float *y, float *nu, int *flag, int *list, int *count, cudaStream_t st);
cudaError_t launch_mlp_norm(int n, const float *feat, MlpNorm *nm, cudaStream_t st);
cudaError_t launch_mlp_grad(int n, const float *feat, const float *target, const float *weight, const int *idx,
                            int batch, uint32_t seed,
                            int step, const float *master, const MlpNorm *nm, float *grad, float *loss, cudaStream_t st);
cudaError_t launch_mlp_adam(float *master, float *m, float *v, float *grad, __half *wh, float lr, int t,
                            cudaStream_t st);
cudaError_t launch_mlp_to_half(const float *master, __half *wh, cudaStream_t st);

// Setup kernels.
template <typename real>
cudaError_t launch_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const real *coord,
                                 const real *dNgp, const real *wgp, real *gpvol, real *He, cudaStream_t st);

// Validation: accumulates failure bits into *flags (device int).
cudaError_t launch_check_tables(int porder, int nelem, int npoin, const int *connec, const float *dlxigp_ip,
                                const int *invAtoIJK, const int *AtoI, const int *AtoJ, const int *AtoK,
                                int *flags, cudaStream_t st);

}  // namespace msod
