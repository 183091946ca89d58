// msod_convec.cu -- plain (FP32 / FP64) hex GLL convection residual.
//
// Computes what full_convec_ijk computes (elem_convec.f90:198-431; Rener as
// defined by full_convec_ijk_split, elem_convec.f90:674-832):
//
//   Rmass  += gpvol [ 1/2 (div q + rho div u) + 1/2 u.grad rho ]
//   Rmom_i += gpvol [ 1/4 (div F_i + u_i div q + q_i div u + rho div Fuu_i) + d_i p
//                     + 1/4 sum_j (u_i u_j d_j rho + q_j d_j u_i + u_j d_j q_i) ]
//   Rener  += gpvol [ 1/4 (div(rho H u) + H div q + rho H div u + rho div(H u))
//                     + 1/4 sum_i (q_i d_i H + u_i d_i(rho H) + H u_i d_i rho) ]
//
// with F = q (x) u, Fuu = u (x) u, k = |u|^2/2 and H = E + k.  The energy
// residual uses the sums E+k, rho E + rho k, rho E u + rho k u and E u + k u
// of the reference's separate E and k terms (elem_convec.f90:810-817): the
// derivatives are linear, so the sums are differentiated once.
//
// Design (one group of NE elements per block at porders 2-5; a persistent
// form that loops over groups, below, at porders 1, 6, 7 and 8 in FP32):
//   * the block copies the node permutations of the call's tables (prepared
//     once per call from the caller's invAtoIJK / gmshAtoI/J/K, msod_tables.cu)
//     into shared memory while its connec entries load; the 1-D derivative
//     matrices are constant-bank operands (shared memory when S > 1);
//   * connec is read coalesced along elements (it is element-fastest), node
//     fields are gathered into a per-element (I,J,K) lattice in shared memory;
//   * each thread owns one GLL line (S threads share a line at high order).
//     Three passes (xi, eta, zeta) load the line's nodal values into
//     registers once, form every differentiated product on the fly and apply
//     the 1-D derivative matrix held in registers (sum factorisation).  The
//     residual is linear in the iso-parametric derivatives, so each pass adds
//     its direction's contribution -- through the He column of that direction
//     and the point's own nodal values -- to seven per-point accumulators kept
//     in shared memory;
//   * the last pass multiplies by gpvol and scatter-adds with red.global.add.
#include "msod_convec.cuh"

namespace msod {
namespace {

template <typename real, int P>
__global__ void __launch_bounds__(ConvecGeom<real, P>::NT, convec_minb<real, P>())
    convec_kernel(int nelem, int npoin, const int *__restrict__ connec, const real *__restrict__ He,
                  const real *__restrict__ gpvol, const real *__restrict__ dlxigp_ip,
                  const int *__restrict__ invAtoIJK, const int *__restrict__ AtoI,
                  const int *__restrict__ AtoJ, const int *__restrict__ AtoK, const real *__restrict__ u,
                  const real *__restrict__ q, const real *__restrict__ rho, const real *__restrict__ pr,
                  const real *__restrict__ E, const TableScratch *__restrict__ tabs, real *__restrict__ Rmass,
                  real *__restrict__ Rmom, real *__restrict__ Rener)
{
    using G = ConvecGeom<real, P>;
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT;
    constexpr int NPL = NE * ES;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr bool STAGED = convec_staged<real>();
    constexpr size_t HEB = ((size_t)NE * N * 9 * sizeof(real) + 31) / 16 * 16;
    constexpr size_t GPB = ((size_t)NE * N * sizeof(real) + 31) / 16 * 16;
    char *sHeB = reinterpret_cast<char *>(smem_raw);
    char *sGpB = sHeB + HEB;
    unsigned long long *sBar = reinterpret_cast<unsigned long long *>(sGpB + GPB);
    real *sF = reinterpret_cast<real *>(smem_raw + convec_stage_bytes<real, P>());
    real *sA = sF + NFIELD * NPL;
    real *sD = sA + NACC * NPL;
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);
    int *sPerm = sNode + NPL;
    int *sLat = sPerm + N;

    const int tid = threadIdx.x;
    const int e0 = blockIdx.x * NE;
    // The compact pass when the call's tables allow it (uniform over the grid).
    bool compact = false;
    if constexpr (convec_compact_capable<real, P>()) compact = ldg(&tabs->eo_ok) != 0;
    // The group's He and gpvol spans: bulk copies issued first, so that they
    // land while the node fields are gathered.
    const real *Hs = He, *Gs = gpvol;
    if constexpr (STAGED) {
        const int e1 = min(e0 + NE, nelem);
        const SpanPlan ph(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
        const SpanPlan pg(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
        if (tid == 0) {
            mbar_init(sBar, 1);
            mbar_arrive_expect_tx(sBar, ph.bulk + pg.bulk);
            ph.issue(sHeB, sBar);
            pg.issue(sGpB, sBar);
        } else if (tid >= 32 && tid < 38) {
            ph.plain(sHeB, tid - 32);
        } else if (tid >= 64 && tid < 70) {
            pg.plain(sGpB, tid - 64);
        }
        Hs = reinterpret_cast<const real *>(sHeB + ph.shift);
        Gs = reinterpret_cast<const real *>(sGpB + pg.shift);
    } else if (CONVEC_PREFETCH != 0 && tid == 0) {
        // The group's He and gpvol spans into L2 while the node fields are
        // gathered: the passes' first He loads then hit L2.  (Also
        // prefetching the spans of the block a wave later -- the grid's
        // resident blocks on -- measured slower: 1.489 against 1.468 ms.)
        const int e1 = min(e0 + NE, nelem);
        prefetch_span_l2(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
        prefetch_span_l2(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
    }
    // Node ids of the group's elements (connec is element-fastest), loaded
    // while the per-call tables are copied into shared memory.
    constexpr int IPT = (NE * N + NT - 1) / NT;
    int ids[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = tid + k * NT;
        const int el = i % NE, a = i / NE, e = e0 + el;
        ids[k] = (i < NE * N && e < nelem) ? ldg(connec + (size_t)a * nelem + e) - 1 : -1;
    }
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    if (G::S > 1)
        for (int i = tid; i < 3 * Q * Q; i += NT) sD[i] = table_D<real>(tabs)[i];
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
    // Gather node fields into the lattice: asynchronous copies, all of a
    // thread's in flight at once (a missing node reads as zeros).
    const size_t np = (size_t)npoin;
    for (int i = tid; i < NE * N; i += NT) {
        const int el = i / N, l = i - el * N;
        const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
        const int o = el * ES + (K * Q + J) * QP + I;
        const int p = sNode[o];
        const bool ok = p >= 0;
        const size_t pp = ok ? (size_t)p : 0;
        cp_async_elem(sF + F_RHO * NPL + o, rho + pp, ok);
        cp_async_elem(sF + F_P * NPL + o, pr + pp, ok);
        cp_async_elem(sF + F_E * NPL + o, E + pp, ok);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cp_async_elem(sF + (F_U0 + c) * NPL + o, u + c * np + pp, ok);
            cp_async_elem(sF + (F_Q0 + c) * NPL + o, q + c * np + pp, ok);
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    if constexpr (STAGED) {
        // Bounded wait for the bulk copies; every thread learns the outcome.
        const bool ok = mbar_wait(sBar, 0);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) report_wait_fault(tabs);
            return;
        }
    } else {
        __syncthreads();
    }
    if constexpr (convec_compact_capable<real, P>()) {
        if (compact) {
#if CONVEC_RTDIR
#pragma unroll 1
#else
#pragma unroll
#endif
            for (int dir = 0; dir < 3; ++dir) {
                if (dir > 0) __syncthreads();
                convec_pass_compact<P>(dir, sF, sA, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom, Rener);
            }
            return;
        }
    }
    convec_dir<real, P, 0, STAGED>(sF, sA, sD, sNode, sPerm, Hs, Gs, e0, nelem, npoin, Rmass, Rmom, Rener);
    __syncthreads();
    convec_dir<real, P, 1, STAGED>(sF, sA, sD, sNode, sPerm, Hs, Gs, e0, nelem, npoin, Rmass, Rmom, Rener);
    __syncthreads();
    convec_dir<real, P, 2, STAGED>(sF, sA, sD, sNode, sPerm, Hs, Gs, e0, nelem, npoin, Rmass, Rmom, Rener);
}

// Persistent form: blocks loop over element groups, the block's tables are
// copied once and a group's He and gpvol spans are prefetched into L2 a group
// ahead.  FP32 at the porders whose bit is set in CONVEC_PERSIST_PORDERS.
// Measured (16.8 M-node meshes, CUDA events, persistent against one-shot):
// porder 1 4.68 / 4.96 ms, 6 1.73 / 1.77, 7 1.53 / 1.72, 8 2.33 / 2.48 (few
// elements per block, or very many blocks, and the one-shot blocks' prologue
// and first He loads weigh on little work each); porder 2 2.40 / 2.13, 3
// 1.65 / 1.52, 4 1.78 / 1.47 (a 264-byte spill at 128 registers; 1.54 ms at
// 168 registers, three blocks per SM), 5 1.73 / 1.53.
// CONVEC_PERSIST: 1 = the next group's node ids load after the passes, 2 =
// during them (porder 7: 1.58 ms).
#ifndef CONVEC_PERSIST_PORDERS
#define CONVEC_PERSIST_PORDERS ((1 << 1) | (1 << 6) | (1 << 7) | (1 << 8))
#endif
#ifndef CONVEC_PERSIST
#define CONVEC_PERSIST 1
#endif
template <typename real, int P>
constexpr bool convec_persist()
{
    return sizeof(real) == 4 && ((CONVEC_PERSIST_PORDERS >> P) & 1) != 0 && !convec_staged<real>();
}
template <typename real, int P>
__global__ void __launch_bounds__(ConvecGeom<real, P>::NT, convec_minb<real, P>())
    convec_kernel_persist(int nelem, int npoin, int ngroups, const int *__restrict__ connec,
                          const real *__restrict__ He, const real *__restrict__ gpvol, const real *__restrict__ u,
                          const real *__restrict__ q, const real *__restrict__ rho, const real *__restrict__ pr,
                          const real *__restrict__ E, const TableScratch *__restrict__ tabs, real *__restrict__ Rmass,
                          real *__restrict__ Rmom, real *__restrict__ Rener)
{
    using G = ConvecGeom<real, P>;
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT;
    constexpr int NPL = NE * ES;
    constexpr int IPT = (NE * N + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real *sF = reinterpret_cast<real *>(smem_raw);
    real *sA = sF + NFIELD * NPL;
    real *sD = sA + NACC * NPL;
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);
    int *sPerm = sNode + NPL;
    int *sLat = sPerm + N;
    const int tid = threadIdx.x;
    bool compact = false;
    if constexpr (convec_compact_capable<real, P>()) compact = ldg(&tabs->eo_ok) != 0;
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    if (G::S > 1)
        for (int i = tid; i < 3 * Q * Q; i += NT) sD[i] = table_D<real>(tabs)[i];
    auto load_ids = [&](int g, int(&ids)[IPT]) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            const int el = i % NE, a = i / NE, e = g * NE + el;
            ids[k] = (i < NE * N && e < nelem) ? ldg(connec + (size_t)a * nelem + e) - 1 : -1;
        }
    };
    auto prefetch_group = [&](int g) {
        if (CONVEC_PREFETCH != 0 && tid == 0 && g < ngroups) {
            const int e0 = g * NE, e1 = min(e0 + NE, nelem);
            prefetch_span_l2(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
            prefetch_span_l2(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
        }
    };
    int g = blockIdx.x;
    const int stride = gridDim.x;
    prefetch_group(g);
    int ids[IPT];
    load_ids(g, ids);
    __syncthreads();  // sLat ready
    const size_t np = (size_t)npoin;
    for (;;) {
        const int e0 = g * NE;
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            if (i < NE * N) {
                const int v = ids[k];
                sNode[(i % NE) * ES + sLat[i / NE]] = (v >= 0 && v < npoin) ? v : -1;
            }
        }
        __syncthreads();
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i / N, l = i - el * N;
            const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
            const int o = el * ES + (K * Q + J) * QP + I;
            const int p = sNode[o];
            const bool ok = p >= 0;
            const size_t pp = ok ? (size_t)p : 0;
            cp_async_elem(sF + F_RHO * NPL + o, rho + pp, ok);
            cp_async_elem(sF + F_P * NPL + o, pr + pp, ok);
            cp_async_elem(sF + F_E * NPL + o, E + pp, ok);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                cp_async_elem(sF + (F_U0 + c) * NPL + o, u + c * np + pp, ok);
                cp_async_elem(sF + (F_Q0 + c) * NPL + o, q + c * np + pp, ok);
            }
        }
        cp_async_commit();
        const int gn = g + stride;
        prefetch_group(gn);
        if (CONVEC_PERSIST == 2 && gn < ngroups) load_ids(gn, ids);
        cp_async_wait_all();
        __syncthreads();
        bool done = false;
        if constexpr (convec_compact_capable<real, P>()) {
            if (compact) {
#pragma unroll
                for (int dir = 0; dir < 3; ++dir) {
                    if (dir > 0) __syncthreads();
                    convec_pass_compact<P>(dir, sF, sA, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom,
                                           Rener);
                }
                done = true;
            }
        }
        if (!done) {
            convec_dir<real, P, 0, false>(sF, sA, sD, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            convec_dir<real, P, 1, false>(sF, sA, sD, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            convec_dir<real, P, 2, false>(sF, sA, sD, sNode, sPerm, He, gpvol, e0, nelem, npoin, Rmass, Rmom, Rener);
        }
        if (gn >= ngroups) break;
        if (CONVEC_PERSIST != 2) load_ids(gn, ids);
        g = gn;
        __syncthreads();  // the passes are done with sNode and the lattice
    }
}

template <typename real, int P>
constexpr size_t convec_smem()
{
    using G = ConvecGeom<real, P>;
    return convec_stage_bytes<real, P>() + (size_t)(NFIELD + NACC) * G::NE * G::ES * sizeof(real) +
           3 * G::Q * G::Q * sizeof(real) + (size_t)(G::NE * G::ES + 2 * G::N) * sizeof(int);
}

template <typename real, int P>
cudaError_t launch_convec_p(const ConvecArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    using G = ConvecGeom<real, P>;
    constexpr size_t smem = convec_smem<real, P>();
    static_assert(smem <= 227 * 1024, "shared memory budget");
    cudaError_t err = cudaFuncSetAttribute(convec_kernel<real, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    if (!tabs) return cudaErrorInvalidValue;
    if (G::S == 1) {
        if (sizeof(real) == 4)
            err = cudaMemcpyToSymbolAsync(c_CDf, table_D<float>(tabs), sizeof(float) * 3 * G::Q * G::Q,
                                          sizeof(float) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
        else
            err = cudaMemcpyToSymbolAsync(c_CDd, table_D<double>(tabs), sizeof(double) * 3 * G::Q * G::Q,
                                          sizeof(double) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
        if (err != cudaSuccess) return err;
        if (convec_compact_capable<real, P>()) {
            err = cudaMemcpyToSymbolAsync(c_CEO, tabs->EO, sizeof(float) * kTableEOMax, sizeof(float) * kTableEOMax * P,
                                          cudaMemcpyDeviceToDevice, st);
            if (err == cudaSuccess)
                err = cudaMemcpyToSymbolAsync(c_CEOp, tabs->EOp, sizeof(float) * kTableEOMax,
                                              sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
            if (err != cudaSuccess) return err;
        }
        if (convec_packed<real, P>()) {
            constexpr int H = (G::Q + 1) / 2;
            err = cudaMemcpyToSymbolAsync(c_CDp, tabs->Dp, sizeof(float2) * 3 * G::Q * H,
                                          sizeof(float2) * (kTableDPairMax / 2) * P, cudaMemcpyDeviceToDevice, st);
            if (err != cudaSuccess) return err;
        }
    }
    if constexpr (convec_persist<real, P>()) {
        auto kern = convec_kernel_persist<real, P>;
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        const int ngroups = (a.nelem + G::NE - 1) / G::NE;
        const int pgrid = persistent_grid(kern, G::NT, smem, ngroups);
        if (pgrid <= 0) return cudaErrorInvalidConfiguration;
        kern<<<pgrid, G::NT, smem, st>>>(a.nelem, a.npoin, ngroups, a.connec, a.He, a.gpvol, a.u, a.q, a.rho, a.pr,
                                         a.E, tabs, a.Rmass, a.Rmom, a.Rener);
        return cudaGetLastError();
    }
    const unsigned grid = (unsigned)((a.nelem + G::NE - 1) / G::NE);
    convec_kernel<real, P><<<grid, G::NT, smem, st>>>(a.nelem, a.npoin, a.connec, a.He, a.gpvol, a.dlxigp_ip,
                                                      a.invAtoIJK, a.AtoI, a.AtoJ, a.AtoK, a.u, a.q, a.rho,
                                                      a.pr, a.E, tabs, a.Rmass, a.Rmom, a.Rener);
    return cudaGetLastError();
}

}  // namespace

template <typename real>
cudaError_t launch_convec_plain(int porder, const ConvecArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_convec_p<real, 1>(a, tabs, st);
    case 2: return launch_convec_p<real, 2>(a, tabs, st);
    case 3: return launch_convec_p<real, 3>(a, tabs, st);
    case 4: return launch_convec_p<real, 4>(a, tabs, st);
    case 5: return launch_convec_p<real, 5>(a, tabs, st);
    case 6: return launch_convec_p<real, 6>(a, tabs, st);
    case 7: return launch_convec_p<real, 7>(a, tabs, st);
    case 8: return launch_convec_p<real, 8>(a, tabs, st);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_convec_plain<float>(int, const ConvecArgs<float> &, const TableScratch *, cudaStream_t);
template cudaError_t launch_convec_plain<double>(int, const ConvecArgs<double> &, const TableScratch *, cudaStream_t);

}  // namespace msod
