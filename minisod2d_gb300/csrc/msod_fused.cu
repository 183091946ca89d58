// msod_fused.cu -- the convection and the diffusion residuals of the same
// inputs in one kernel (msod_convec_diffusion_ijk).
//
// The reference makes two calls per step on the same mesh and state,
// full_convec_ijk (elem_convec.f90:198-431; Rener as full_convec_ijk_split
// defines it, :674-832) and full_diffusion_ijk (elem_diffu.f90:10-197), and
// both gather connec, He, gpvol, rho and u at every element point
// (elem_convec.f90:228-252, elem_diffu.f90:44-59).  Here persistent blocks
// take groups of NE elements; per group the node ids are stored once and the
// two calls' node fields (rho, u, T, mu_fluid, p, E, q) and element-layout
// mu_e, mu_sgs are gathered once, with cp.async, into one shared-memory
// lattice of 20 planes:
//     0 rho, 1 T, 2-4 u, 5 mu_fluid, 6 mu_e, 7 mu_sgs   (the diffusion's planes)
//     8 p, 9 E, 10-12 q                                (convection only)
//    13-19 the convection's seven per-point accumulators
// The convection kernel's line passes (msod_convec.cuh), pointed at these
// planes, scatter the convection residuals.  Then the diffusion's gradient
// passes, its fused zeta stage and its divergence passes (msod_diffu.cuh) run
// on the same lattice, with their flux planes over planes 8-19, and scatter
// the diffusion residuals.  The group's He, gpvol and connec, which the
// convection has just read, come to the diffusion from L1 / L2.  The next
// group's node ids load during the convection passes, and its He and gpvol
// spans are prefetched into L2.
//
// The kernel serves porder 4 in FP32 (64^3 hexes: 2.85 ms against 2.90 ms
// for the two kernels, 35 % fewer DRAM reads).  Porders 5 and 7 also take
// the same element groups in both kernels (one thread per line, NE elements
// in NT threads), but there the kernel measured slower than the two kernels
// (FUSED_ALL below); they and the other porders run the two kernels one after
// the other on the call's one set of tables.
// FP32 only: the unit's constant bank holds both kernels' FP32 tables.
#define MSOD_FP32_ONLY 1
// Scalar even-odd contractions here (packed: 2.866 against 2.857 ms on 64^3
// porder-4 hexes).
#define CONVEC_EO2 0
#include "msod_convec.cuh"
#include "msod_diffu.cuh"

namespace msod {
namespace {

// Node-field planes of the convection passes in the shared lattice.
struct FusedPlanes {
    static constexpr int RHO = D_RHO, U0 = D_U0, PR = NDF, EN = NDF + 1, Q0 = NDF + 2;
};
constexpr int kFusedAcc = NDF + 5;    // first of the convection's accumulator planes
constexpr int kFusedPlanes = kFusedAcc + NACC;
static_assert(D_RHO == 0 && D_T == 1 && D_U0 == 2 && D_MUF == 5 && D_MUE == 6 && D_MUS == 7 && NDF == 8,
              "the diffusion's gathered planes");

template <int P>
using FusedConvGeom = ConvecGeom<float, P>;
template <int P>
using FusedDiffuGeom = DiffuGeom<float, P>;

// Porders 5 and 7 fused as well (1), for measuring: on meshes of about 16.8 M
// nodes (51^3 / 37^3 hexes) one kernel took 3.30 / 4.51 ms against 3.06 /
// 3.69 ms for the two kernels (porder 4, 64^3: 2.90 against 2.97 ms).  At
// porder 5 the 20-plane lattice leaves three blocks per SM little L1 for the
// He loads; at porder 7 the convection passes, which already take 255
// registers alone, spill 324 bytes beside the diffusion's state.
#ifndef FUSED_ALL
#define FUSED_ALL 0
#endif

template <int P>
constexpr bool fusable()
{
    using GC = FusedConvGeom<P>;
    using GD = FusedDiffuGeom<P>;
    return (P == 4 || FUSED_ALL != 0) && GC::S == 1 && GD::S == 1 && GC::NE == GD::NE && GC::NT == GD::NT &&
           GC::ES == GD::ES &&
           diffu_fusez<GD>() && !convec_staged<float>() && !diffu_staged<GD>() && DIFFU_NBUF == 1 &&
           diffu_xplanes<GD>() <= kFusedPlanes - NDF;
}

// Blocks per SM the register budget is sized for.  Porders 4 and 5: three
// (168 registers; the 20-plane lattice allows three or four blocks).  Porder
// 7: one, which lets the convection passes take 255 registers; the lattice
// holds the kernel to two blocks per SM, as the register file does.
#ifndef FUSED_MINB4
#define FUSED_MINB4 3
#endif
#ifndef FUSED_MINB5
#define FUSED_MINB5 3
#endif
// L2 prefetches a group ahead: 1 = the next group's He and gpvol spans; 2 =
// also its mu_e, mu_sgs rows; 3 = also the node fields of its element points;
// 0 = none.  Measured on 64^3 hexes: 2.876 / 2.857 / 2.898 / 3.17 ms (none /
// spans / spans and rows / all three).
#ifndef FUSED_PREFETCH
#define FUSED_PREFETCH 1
#endif
template <int P>
constexpr int fused_minb()
{
    return P == 4 ? FUSED_MINB4 : (P == 5 ? FUSED_MINB5 : 1);
}

template <int P>
constexpr size_t fused_smem()
{
    using GD = FusedDiffuGeom<P>;
    return (size_t)kFusedPlanes * GD::NPL * sizeof(float) + (size_t)(GD::NPL + 2 * GD::N) * sizeof(int);
}

template <int P>
__global__ void __launch_bounds__(FusedDiffuGeom<P>::NT, fused_minb<P>())
    fused_kernel(int nelem, int npoin, int ngroups, const int *__restrict__ connec, const float *__restrict__ He,
                 const float *__restrict__ gpvol, const TableScratch *__restrict__ tabs, float Cp, float Pr,
                 const float *__restrict__ u, const float *__restrict__ q, const float *__restrict__ rho,
                 const float *__restrict__ pr, const float *__restrict__ E, const float *__restrict__ Tem,
                 const float *__restrict__ mu_fluid, const float *__restrict__ mu_e,
                 const float *__restrict__ mu_sgs, float *__restrict__ Rmass_c, float *__restrict__ Rmom_c,
                 float *__restrict__ Rener_c, float *__restrict__ Rmass_d, float *__restrict__ Rmom_d,
                 float *__restrict__ Rener_d, int linemap)
{
    using GD = FusedDiffuGeom<P>;
    constexpr int Q = GD::Q, N = GD::N, QP = GD::QP, ES = GD::ES, NE = GD::NE, NT = GD::NT, NPL = GD::NPL;
    constexpr int IPT = (NE * N + NT - 1) / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sP = reinterpret_cast<float *>(smem_raw);  // [kFusedPlanes][NPL]
    float *sX = sP + NDF * NPL;                       // the diffusion's flux planes
    float *sA = sP + kFusedAcc * NPL;                 // the convection's accumulators
    int *sNode = reinterpret_cast<int *>(sP + kFusedPlanes * NPL);
    int *sPerm = sNode + NPL;
    int *sLat = sPerm + N;

    const int tid = threadIdx.x;
    bool compact = false;
    if constexpr (convec_compact_capable<float, P>()) compact = ldg(&tabs->eo_ok) != 0;
    // The diffusion's xi and eta passes in even-odd form, as in the diffusion
    // kernel, when the call's tables allow it.
    constexpr bool EOK = ((DIFFU_EO >> P) & 1) != 0;
    bool eo = false;
    if constexpr (EOK) eo = ldg(&tabs->eo_ok) != 0;
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    auto load_ids = [&](int g, int(&ids)[IPT]) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            const int el = i % NE, a = i / NE, e = g * NE + el;
            ids[k] = (i < NE * N && e < nelem) ? ldg(connec + (size_t)a * nelem + e) : 0;
        }
    };
    auto store_ids = [&](const int(&ids)[IPT]) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            if (i < NE * N) {
                const int v = ids[k] - 1;
                sNode[(i % NE) * ES + sLat[i / NE]] = (v >= 0 && v < npoin) ? v : -1;
            }
        }
    };
    // Both calls' node fields in lattice order (a missing node reads as
    // zeros); mu_e and mu_sgs along elements (coalesced).
    auto gather = [&](int g) {
        const size_t np = (size_t)npoin;
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i / N, l = i - el * N;
            const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
            const int o = el * ES + (K * Q + J) * QP + I;
            const int p = sNode[o];
            const bool ok = (unsigned)p < (unsigned)npoin;
            const size_t pp = ok ? (size_t)p : 0;
            cp_async_elem(sP + D_RHO * NPL + o, rho + pp, ok);
            cp_async_elem(sP + D_T * NPL + o, Tem + pp, ok);
            cp_async_elem(sP + D_MUF * NPL + o, mu_fluid + pp, ok);
            cp_async_elem(sP + FusedPlanes::PR * NPL + o, pr + pp, ok);
            cp_async_elem(sP + FusedPlanes::EN * NPL + o, E + pp, ok);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                cp_async_elem(sP + (D_U0 + c) * NPL + o, u + c * np + pp, ok);
                cp_async_elem(sP + (FusedPlanes::Q0 + c) * NPL + o, q + c * np + pp, ok);
            }
        }
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i % NE, a = i / NE, e = g * NE + el;
            const int o = el * ES + sLat[a];
            const bool ok = e < nelem;
            const size_t idx = ok ? (size_t)a * nelem + e : 0;
            cp_async_elem(sP + D_MUE * NPL + o, mu_e + idx, ok);
            cp_async_elem(sP + D_MUS * NPL + o, mu_sgs + idx, ok);
        }
        cp_async_commit();
    };

    // Group gg's He and gpvol spans into L2 (one thread), a group ahead of
    // their loads in the passes.
    auto prefetch_group = [&](int gg) {
        if (FUSED_PREFETCH != 0 && tid == 0 && gg < ngroups) {
            const int e0 = gg * NE, e1 = min(e0 + NE, nelem);
            prefetch_span_l2(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(float));
            prefetch_span_l2(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(float));
        }
    };
    int ids[IPT];
    // The next group's gathered inputs into L2 (ids holds its node ids), during
    // the diffusion stages: its node fields and its mu_e, mu_sgs rows.
    auto prefetch_nodes = [&](int gg) {
        if (FUSED_PREFETCH >= 3) {
            const size_t np = (size_t)npoin;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT, v = ids[k] - 1;
                if (i < NE * N && (unsigned)v < (unsigned)npoin) {
                    prefetch_l2(rho + v);
                    prefetch_l2(Tem + v);
                    prefetch_l2(mu_fluid + v);
                    prefetch_l2(pr + v);
                    prefetch_l2(E + v);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        prefetch_l2(u + c * np + v);
                        prefetch_l2(q + c * np + v);
                    }
                }
            }
        }
        if (FUSED_PREFETCH >= 2 && tid < N) {
            const size_t row = (size_t)tid * nelem + (size_t)gg * NE;
            prefetch_l2(mu_e + row);
            prefetch_l2(mu_sgs + row);
        }
    };
    int g = blockIdx.x;
    const int stride = gridDim.x;
    prefetch_group(g);
    load_ids(g, ids);
    __syncthreads();  // sLat ready
    store_ids(ids);
    __syncthreads();
    gather(g);

    for (int gn = g + stride; g < ngroups; g = gn, gn += stride) {
        prefetch_group(gn);
        cp_async_wait_all();
        __syncthreads();
        if (gn < ngroups) load_ids(gn, ids);
        const int e0 = g * NE;
        // Convection: three line passes, the last one scatters.
        if constexpr (convec_compact_capable<float, P>()) {
            if (compact) {
#pragma unroll
                for (int dir = 0; dir < 3; ++dir) {
                    if (dir > 0) __syncthreads();
                    convec_pass_compact<P, FusedPlanes>(dir, sP, sA, sNode, sPerm, He, gpvol, e0, nelem, npoin,
                                                        Rmass_c, Rmom_c, Rener_c);
                }
            }
        }
        if (!compact) {
            convec_dir<float, P, 0, false, FusedPlanes>(sP, sA, nullptr, sNode, sPerm, He, gpvol, e0, nelem, npoin,
                                                        Rmass_c, Rmom_c, Rener_c);
            __syncthreads();
            convec_dir<float, P, 1, false, FusedPlanes>(sP, sA, nullptr, sNode, sPerm, He, gpvol, e0, nelem, npoin,
                                                        Rmass_c, Rmom_c, Rener_c);
            __syncthreads();
            convec_dir<float, P, 2, false, FusedPlanes>(sP, sA, nullptr, sNode, sPerm, He, gpvol, e0, nelem, npoin,
                                                        Rmass_c, Rmom_c, Rener_c);
        }
        __syncthreads();
        if (gn < ngroups) prefetch_nodes(gn);
        // Diffusion: xi and eta derivatives, the zeta stage (zeta derivatives,
        // point pass, zeta divergence), the xi and eta divergence passes.
        const LineThread<GD> lt0 = diffu_line<GD>(tid, 0, linemap), lt1 = diffu_line<GD>(tid, 1, linemap),
                             lt2 = diffu_line<GD>(tid, 2, linemap);
        if (eo) {
            if (lt0.active) grad_pass<GD, 0, EOK>(lt0, sP, sX, nullptr);
            if (lt1.active) grad_pass<GD, 1, EOK>(lt1, sP, sX, nullptr);
        } else {
            if (lt0.active) grad_pass<GD, 0>(lt0, sP, sX, nullptr);
            if (lt1.active) grad_pass<GD, 1>(lt1, sP, sX, nullptr);
        }
        __syncthreads();
        if (lt2.active) {
            const int ee = e0 + lt2.el;
            const bool eok = ee < nelem;
            auto he_row = [&](int c, float(&h)[9], float &gp) {
                const int a = sPerm[line_lat<2, Q>(lt2.la, lt2.lb, c)];
                const float *hp = He + (eok ? ((size_t)ee * N + a) * 9 : 0);
#pragma unroll
                for (int j = 0; j < 9; ++j) h[j] = eok ? ldg(hp + j) : 0.0f;
                gp = eok ? ldg(gpvol + (size_t)ee * N + a) : 0.0f;
            };
            auto mu_at = [&](int o, float) -> float { return sP[D_MUE * NPL + o]; };
            zeta_stage<GD>(lt2, sP, sX, he_row, mu_at, Cp, Pr);
        }
        __syncthreads();
        if (eo) {
            if (lt0.active)
                div_pass<GD, 0, false, false, EOK>(lt0, sP, sX, nullptr, sNode, npoin, Rmass_d, Rmom_d, Rener_d);
            __syncthreads();
            if (lt1.active)
                div_pass<GD, 1, false, true, EOK>(lt1, sP, sX, nullptr, sNode, npoin, Rmass_d, Rmom_d, Rener_d);
        } else {
            if (lt0.active) div_pass<GD, 0, false, false>(lt0, sP, sX, nullptr, sNode, npoin, Rmass_d, Rmom_d, Rener_d);
            __syncthreads();
            if (lt1.active) div_pass<GD, 1, false, true>(lt1, sP, sX, nullptr, sNode, npoin, Rmass_d, Rmom_d, Rener_d);
        }
        __syncthreads();
        if (gn < ngroups) {  // the next group's node ids, then its fields
            store_ids(ids);
            __syncthreads();
            gather(gn);
        }
    }
}

template <int P>
cudaError_t launch_fused_p(const ConvecArgs<float> &c, const DiffuArgs<float> &d, const TableScratch *tabs,
                           cudaStream_t st)
{
    if constexpr (!fusable<P>()) {
        cudaError_t err = launch_convec_plain<float>(P, c, tabs, st);
        if (err != cudaSuccess) return err;
        return launch_diffu_plain<float>(P, d, tabs, st);
    } else {
        using GC = FusedConvGeom<P>;
        using GD = FusedDiffuGeom<P>;
        constexpr size_t smem = fused_smem<P>();
        static_assert(smem <= 227 * 1024, "shared memory budget");
        auto kern = fused_kernel<P>;
        cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        // This translation unit's constant-bank tables: the convection's
        // matrices (and their even-odd form or row pairs) and the diffusion's.
        const size_t dbytes = sizeof(float) * 3 * GC::Q * GC::Q;
        err = cudaMemcpyToSymbolAsync(c_CDf, table_D<float>(tabs), dbytes, sizeof(float) * kTableDMax * P,
                                      cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess)
            err = cudaMemcpyToSymbolAsync(c_Df, table_D<float>(tabs), dbytes, sizeof(float) * kTableDMax * P,
                                          cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && convec_compact_capable<float, P>())
            err = cudaMemcpyToSymbolAsync(c_CEO, tabs->EO, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && convec_compact_capable<float, P>())
            err = cudaMemcpyToSymbolAsync(c_CEOp, tabs->EOp, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && ((DIFFU_EO >> P) & 1) != 0)
            err = cudaMemcpyToSymbolAsync(c_DEO, tabs->EO, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && ((DIFFU_EO >> P) & 1) != 0)
            err = cudaMemcpyToSymbolAsync(c_DEOp, tabs->EOp, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && convec_packed<float, P>()) {
            constexpr int H = (GC::Q + 1) / 2;
            err = cudaMemcpyToSymbolAsync(c_CDp, tabs->Dp, sizeof(float2) * 3 * GC::Q * H,
                                          sizeof(float2) * (kTableDPairMax / 2) * P, cudaMemcpyDeviceToDevice, st);
        }
        if (err != cudaSuccess) return err;
        const int ngroups = (c.nelem + GD::NE - 1) / GD::NE;
        const int grid = persistent_grid(kern, GD::NT, smem, ngroups);
        if (grid <= 0) return cudaErrorInvalidConfiguration;
        const int linemap =
            DIFFU_LINEMAP_MODE == 2 ? (c.npoin < (long long)c.nelem * GD::N ? 1 : 0) : DIFFU_LINEMAP_MODE;
        kern<<<grid, GD::NT, smem, st>>>(c.nelem, c.npoin, ngroups, c.connec, c.He, c.gpvol, tabs, d.Cp, d.Pr, c.u,
                                         c.q, c.rho, c.pr, c.E, d.Tem, d.mu_fluid, d.mu_e, d.mu_sgs, c.Rmass, c.Rmom,
                                         c.Rener, d.Rmass, d.Rmom, d.Rener, linemap);
        return cudaGetLastError();
    }
}

}  // namespace

bool fused_porder(int porder)
{
    switch (porder) {
    case 4: return fusable<4>();
    case 5: return fusable<5>();
    case 7: return fusable<7>();
    default: return false;
    }
}

cudaError_t launch_fused(int porder, const ConvecArgs<float> &c, const DiffuArgs<float> &d, const TableScratch *tabs,
                         cudaStream_t st)
{
    switch (porder) {
    case 4: return launch_fused_p<4>(c, d, tabs, st);
    case 5: return launch_fused_p<5>(c, d, tabs, st);
    case 7: return launch_fused_p<7>(c, d, tabs, st);
    default: {
        cudaError_t err = launch_convec_plain<float>(porder, c, tabs, st);
        if (err != cudaSuccess) return err;
        return launch_diffu_plain<float>(porder, d, tabs, st);
    }
    }
}

}  // namespace msod
