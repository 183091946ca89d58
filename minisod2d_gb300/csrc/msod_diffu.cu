// msod_diffu.cu -- plain (FP32 / FP64) hex GLL diffusion residual.
//
// Computes what full_diffusion_ijk computes (elem_diffu.f90:10-197):
//   pass 1 (per point b): grad rho, grad T, grad u; mu_f = mu_fluid + rho mu_sgs;
//     tau = (mu_f + mu_e)(grad u + grad u^T) - 2/3 mu_f div u I;  tauU = tau u
//   pass 2 (per output node a):
//     Rmass += nu_e(a)   sum_{d,b} w_d(a,b) . grad rho(b)
//     Rener +=           sum_{d,b} w_d(a,b) . (tauU(b) + kappa_e(a) grad T(b))
//     Rmom_m +=          sum_{d,b} w_d(a,b) . tau_m(b)
//   with w_d(a,b)_i = He(i,d,b) gpvol(b) dlxigp_ip(b,d,iso_d(a)) over the
//   points b of a's d-line, nu_e(a) = mu_e/rho and
//   kappa_e(a) = mu_fluid Cp/Pr + mu_e Cp/Pr + Cp rho mu_sgs / 0.9 evaluated at
//   the output node (elem_diffu.f90:143-146).
//
// Design (persistent blocks, groups of NE elements, one thread per GLL line):
//   0. the node ids of the next group are loaded into registers while the
//      current group is computed; after it, the next group's node fields
//      (rho, T, u, mu_fluid) and element-layout mu_e, mu_sgs are gathered with
//      cp.async into the shared-memory lattice (single-buffered: measured 6 %
//      faster than a double-buffered lattice, whose shared memory held the
//      kernel to two blocks per SM instead of three; DIFFU_NBUF = 2 selects
//      it); the He and gpvol values of the point pass are loaded into
//      registers before pass 1;
//   1. three line passes store the 15 iso-parametric derivatives per point;
//   2. a point pass turns them into physical gradients and stress and stores,
//      per direction d, the contravariant fluxes gpvol * He(:,d)^T X for the
//      six vectors X = grad rho, tauU, grad T, tau rows 1..3 (18 per point),
//      plus nu_e and kappa_e per output node;
//   3. three line passes apply the transposed 1-D derivative matrix along the
//      lines (the weak divergence), accumulating five sums per node through
//      shared memory; the last pass scatter-adds with red.global.add.
// With one thread per line from porder 3 up, the zeta derivative pass, the
// point pass and the zeta divergence pass run as one pass over each zeta line
// (the zeta derivatives and fluxes never reach shared memory, the He rows are
// loaded there one point ahead), and the flux region shrinks from 18 planes to
// 12: porder 4 then takes 53.8 KB of shared memory per block instead of 68.8 KB,
// three blocks leave ~88 KB of L1 instead of ~28 KB for the He and node-field
// loads, and the kernel runs 1.50 ms instead of 1.82 ms on 64^3 hexes (the same
// fusion with the 18-plane region: 1.79 ms; four blocks per SM at 128
// registers, which fill the shared memory again: 1.90 ms).
// The 1-D derivative matrices are constant-bank operands.
#include "msod_diffu.cuh"

namespace msod {
namespace {

template <class G, int VISC>
__global__ void __launch_bounds__(G::NT, diffu_minb<G>())
    diffu_kernel(int nelem, int npoin, int ngroups, const int *__restrict__ connec,
                 const typename G::real *__restrict__ He, const typename G::real *__restrict__ gpvol,
                 const TableScratch *__restrict__ tabs, typename G::real Cp, typename G::real Pr,
                 const typename G::real *__restrict__ rho, const typename G::real *__restrict__ u,
                 const typename G::real *__restrict__ Tem, const typename G::real *__restrict__ mu_fluid,
                 const typename G::real *__restrict__ mu_e, const typename G::real *__restrict__ mu_sgs,
                 const typename G::real *__restrict__ nu_elem, typename G::real *__restrict__ Rmass,
                 typename G::real *__restrict__ Rmom, typename G::real *__restrict__ Rener, int linemap)
{
    using real = typename G::real;
    constexpr int Q = G::Q, N = G::N, QP = G::QP, ES = G::ES, NE = G::NE, NT = G::NT, NPL = G::NPL;
    constexpr int IPT = (NE * N + NT - 1) / NT;  // items (node ids, points) per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NBUF = DIFFU_NBUF;
    constexpr bool STAGED = diffu_staged<G>();
    char *sHeB = reinterpret_cast<char *>(smem_raw);  // staged He / gpvol spans, then the mbarrier
    char *sGpB = sHeB + diffu_he_bytes<G>();
    unsigned long long *sBar = reinterpret_cast<unsigned long long *>(sGpB + diffu_gp_bytes<G>());
    real *sF = reinterpret_cast<real *>(smem_raw + diffu_stage_bytes<G>());  // [NBUF][NDF][NPL]
    real *sX = sF + NBUF * NDF * NPL;                // [2 or 3 NX][NPL]
    real *sD = sX + diffu_xplanes<G>() * NPL;        // [3][Q][Q] (several threads per line)
    int *sNode = reinterpret_cast<int *>(sD + 3 * Q * Q);  // [NBUF][NPL]
    int *sPerm = sNode + NBUF * NPL;
    int *sLat = sPerm + N;

    const int tid = threadIdx.x;
    const LineThread<G> lt0 = diffu_line<G>(tid, 0, linemap), lt1 = diffu_line<G>(tid, 1, linemap),
                        lt2 = diffu_line<G>(tid, 2, linemap);
    constexpr bool FUSEZ = diffu_fusez<G>();
    constexpr bool LATE = FUSEZ && DIFFU_HE_LATE != 0;
    // The xi and eta passes in even-odd form when the call's tables allow it
    // (uniform over the grid).
    constexpr bool EOK = ((DIFFU_EO >> G::P) & 1) != 0 && FUSEZ && sizeof(real) == 4;
    bool eo = false;
    if constexpr (EOK) eo = ldg(&tabs->eo_ok) != 0;
    constexpr int MP = LATE ? 1 : (FUSEZ ? Q : IPT);  // points whose He and gpvol a thread holds
    for (int i = tid; i < N; i += NT) {
        sPerm[i] = tabs->perm[i];
        sLat[i] = tabs->lat[i];
    }
    if (G::S > 1)
        for (int i = tid; i < 3 * Q * Q; i += NT) sD[i] = table_D<real>(tabs)[i];
    // Group-invariant parts of the gathers (GOFF), per item k of the thread: the
    // lattice offset of its point in the node-field gather (go), and for the
    // element-layout loads (node ids, mu_e, mu_sgs) the row offset a nelem + el
    // (mr) and the element el in bits 20.. of mo, whose low bits take the
    // lattice offset el ES + lat(a) once sLat is in shared memory; -1 for no item.
    constexpr bool GOFF = ((DIFFU_GOFF >> G::P) & 1) != 0 && NBUF == 1 && DIFFU_GATHER_LDG == 0;
    constexpr int KG = GOFF ? IPT : 1;
    int go[KG], mr[KG], mo[KG];
    if constexpr (GOFF) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int i = tid + k * NT;
            const bool in = i < NE * N;
            const int el = i / N, l = i - el * N;
            const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
            go[k] = in ? el * ES + (K * Q + J) * QP + I : -1;
            const int el2 = i % NE, a = i / NE;
            mr[k] = in ? a * nelem + el2 : 0;
            mo[k] = in ? (el2 << 20) : -1;
        }
    }
    auto load_ids = [&](int g, int (&ids)[IPT]) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            if constexpr (GOFF) {
                const bool ok = mo[k] >= 0 && g * NE + (mo[k] >> 20) < nelem;
                ids[k] = ok ? ldg(connec + (size_t)(mr[k] + g * NE)) : 0;
            } else {
                const int i = tid + k * NT;
                const int el = i % NE, a = i / NE, e = g * NE + el;
                ids[k] = (i < NE * N && e < nelem) ? ldg(connec + (size_t)a * nelem + e) : 0;
            }
        }
    };
    auto store_ids = [&](const int (&ids)[IPT], int *dst) {
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const int v = ids[k] - 1;
            if constexpr (GOFF) {
                if (mo[k] >= 0) dst[mo[k] & 0xFFFFF] = (v >= 0 && v < npoin) ? v : -1;
            } else {
                const int i = tid + k * NT;
                if (i < NE * N) dst[(i % NE) * ES + sLat[i / NE]] = (v >= 0 && v < npoin) ? v : -1;
            }
        }
    };
    // Node fields in lattice order; mu_e / mu_sgs along elements (coalesced).
    auto gather = [&](int g, const int *ids_s, real *dst) {
        if constexpr (DIFFU_GATHER_LDG != 0) {
            // Loads of all of a thread's items first, then the stores.
            real v[IPT][6], w[IPT][2];
            int ov[IPT], ow[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT;
                const bool in = i < NE * N;
                const int el = in ? i / N : 0, l = in ? i - el * N : 0;
                const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
                const int o = el * ES + (K * Q + J) * QP + I;
                ov[k] = in ? o : -1;
                const int p = in ? ids_s[o] : -1;
                const bool ok = (unsigned)p < (unsigned)npoin;
                const size_t pp = ok ? (size_t)p : 0, np = (size_t)npoin;
                v[k][0] = ok ? ldg(rho + pp) : (real)0;
                v[k][1] = ok ? ldg(Tem + pp) : (real)0;
#pragma unroll
                for (int c = 0; c < 3; ++c) v[k][2 + c] = ok ? ldg(u + c * np + pp) : (real)0;
                v[k][5] = ok ? ldg(mu_fluid + pp) : (real)0;
                const int el2 = i % NE, a = i / NE, e = g * NE + el2;
                ow[k] = in ? el2 * ES + sLat[in ? a : 0] : -1;
                const bool ok2 = in && e < nelem;
                const size_t idx = ok2 ? (size_t)a * nelem + e : 0;
                w[k][0] = (VISC == VISC_MU_E && ok2) ? ldg(mu_e + idx) : (real)0;
                w[k][1] = ok2 ? ldg(mu_sgs + idx) : (real)0;
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if (ov[k] < 0) continue;
                dst[D_RHO * NPL + ov[k]] = v[k][0];
                dst[D_T * NPL + ov[k]] = v[k][1];
#pragma unroll
                for (int c = 0; c < 3; ++c) dst[(D_U0 + c) * NPL + ov[k]] = v[k][2 + c];
                dst[D_MUF * NPL + ov[k]] = v[k][5];
                if (VISC == VISC_MU_E) dst[D_MUE * NPL + ow[k]] = w[k][0];
                dst[D_MUS * NPL + ow[k]] = w[k][1];
            }
            return;
        }
        if constexpr (GOFF) {
            const size_t np = (size_t)npoin;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int o = go[k];
                if (o >= 0) {
                    const int p = ids_s[o];
                    const bool ok = (unsigned)p < (unsigned)npoin;
                    const size_t pp = ok ? (size_t)p : 0;
                    cp_async_elem(dst + D_RHO * NPL + o, rho + pp, ok);
                    cp_async_elem(dst + D_T * NPL + o, Tem + pp, ok);
#pragma unroll
                    for (int c = 0; c < 3; ++c) cp_async_elem(dst + (D_U0 + c) * NPL + o, u + c * np + pp, ok);
                    cp_async_elem(dst + D_MUF * NPL + o, mu_fluid + pp, ok);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if (mo[k] >= 0) {
                    const bool ok = g * NE + (mo[k] >> 20) < nelem;
                    const size_t idx = ok ? (size_t)(mr[k] + g * NE) : 0;
                    const int o = mo[k] & 0xFFFFF;
                    if (VISC == VISC_MU_E) cp_async_elem(dst + D_MUE * NPL + o, mu_e + idx, ok);
                    cp_async_elem(dst + D_MUS * NPL + o, mu_sgs + idx, ok);
                }
            }
            cp_async_commit();
            return;
        }
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i / N, l = i - el * N;
            const int I = l % Q, J = (l / Q) % Q, K = l / (Q * Q);
            const int o = el * ES + (K * Q + J) * QP + I;
            const int p = ids_s[o];
            const bool ok = (unsigned)p < (unsigned)npoin;
            const size_t pp = ok ? (size_t)p : 0, np = (size_t)npoin;
            cp_async_elem(dst + D_RHO * NPL + o, rho + pp, ok);
            cp_async_elem(dst + D_T * NPL + o, Tem + pp, ok);
#pragma unroll
            for (int c = 0; c < 3; ++c) cp_async_elem(dst + (D_U0 + c) * NPL + o, u + c * np + pp, ok);
            cp_async_elem(dst + D_MUF * NPL + o, mu_fluid + pp, ok);
        }
        for (int i = tid; i < NE * N; i += NT) {
            const int el = i % NE, a = i / NE, e = g * NE + el;
            const int o = el * ES + sLat[a];
            const bool ok = e < nelem;
            const size_t idx = ok ? (size_t)a * nelem + e : 0;
            if (VISC == VISC_MU_E) cp_async_elem(dst + D_MUE * NPL + o, mu_e + idx, ok);
            cp_async_elem(dst + D_MUS * NPL + o, mu_sgs + idx, ok);
        }
        cp_async_commit();
    };
    // He(:,:) and gpvol of the thread's point-pass points: items tid + k NT
    // (lattice order), or the points of its zeta line in the zeta stage.
    auto load_metric = [&](int g, real (&Hm)[MP][9], real (&gv)[MP]) {
#pragma unroll
        for (int k = 0; k < MP; ++k) {
            const int i = tid + k * NT;
            const int el = FUSEZ ? lt2.el : i / N;
            const int l = FUSEZ ? line_lat<2, Q>(lt2.la, lt2.lb, k) : i - el * N, e = g * NE + el;
            const bool ok = (FUSEZ ? lt2.active : i < NE * N) && e < nelem;
            const int a = ok ? sPerm[l] : 0;
            const real *hp = He + (ok ? ((size_t)e * N + a) * 9 : 0);
#pragma unroll
            for (int j = 0; j < 9; ++j) Hm[k][j] = ok ? ldg(hp + j) : (real)0;
            gv[k] = ok ? ldg(gpvol + (size_t)e * N + a) : (real)0;
        }
    };

    // mu_e at a point of element el of group g (lattice offset o, density r).
    auto point_mu_e = [&](int g, int el, int o, real r, const real *sFs) -> real {
        const int ee = g * NE + el;
        return VISC == VISC_NU_ELEM ? (ee < nelem ? r * ldg(nu_elem + ee) : (real)0) : sFs[D_MUE * NPL + o];
    };

    // Staged He / gpvol: bulk copies of group g's spans (thread 0), the
    // unaligned ends by plain loads (threads 32..37, 64..69).  Offsets of the
    // spans' first words in the staging area.
    int he_off = 0, gp_off = 0;
    auto stage = [&](int g) {
        if constexpr (STAGED) {
            const int e0 = g * NE, e1 = min(e0 + NE, nelem);
            const SpanPlan ph(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
            const SpanPlan pg(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
            if (tid == 0) {
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(sBar, ph.bulk + pg.bulk);
                ph.issue(sHeB, sBar);
                pg.issue(sGpB, sBar);
            } else if (tid >= 32 && tid < 38) {
                ph.plain(sHeB, tid - 32);
            } else if (tid >= 64 && tid < 70) {
                pg.plain(sGpB, tid - 64);
            }
            he_off = (int)(ph.shift / sizeof(real));
            gp_off = (int)(pg.shift / sizeof(real));
        }
    };
    unsigned phase = 0;

    int g = blockIdx.x;
    const int stride = gridDim.x;
    if constexpr (STAGED) {
        if (tid == 0) mbar_init(sBar, 1);
        __syncthreads();
        stage(g);
    }
    // Group g's He and gpvol spans into L2 (one thread), a group ahead of
    // their loads in the zeta stage.
    auto prefetch_group = [&](int gg) {
        if constexpr (DIFFU_PREFETCH != 0 && !STAGED) {
            if (tid == 0 && gg < ngroups) {
                const int e0 = gg * NE, e1 = min(e0 + NE, nelem);
                prefetch_span_l2(He + (size_t)e0 * N * 9, (size_t)(e1 - e0) * N * 9 * sizeof(real));
                prefetch_span_l2(gpvol + (size_t)e0 * N, (size_t)(e1 - e0) * N * sizeof(real));
            }
        }
    };
    // Group gg's gathered inputs into L2 (ids: its node ids), a group ahead of
    // the gather: the node fields of its element points and its mu_e, mu_sgs
    // rows (N rows of NE consecutive values).
    auto prefetch_nodes = [&](int gg, const int(&ids_g)[IPT]) {
        if constexpr (DIFFU_PREFETCH >= 3 && NBUF == 1) {
            const size_t np = (size_t)npoin;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT, v = ids_g[k] - 1;
                if (i < NE * N && (unsigned)v < (unsigned)npoin) {
                    prefetch_l2(rho + v);
                    prefetch_l2(Tem + v);
                    prefetch_l2(mu_fluid + v);
#pragma unroll
                    for (int c = 0; c < 3; ++c) prefetch_l2(u + c * np + v);
                }
            }
        }
        if constexpr (DIFFU_PREFETCH >= 2 && NBUF == 1) {
            if (tid < N) {
                const size_t row = (size_t)tid * nelem + (size_t)gg * NE;
                if (VISC == VISC_MU_E) prefetch_l2(mu_e + row);
                prefetch_l2(mu_sgs + row);
            }
        }
    };
    prefetch_group(g);
    int ids[IPT];
    load_ids(g, ids);
    __syncthreads();  // sLat ready
    if constexpr (GOFF) {
#pragma unroll
        for (int k = 0; k < IPT; ++k)
            if (mo[k] >= 0) mo[k] |= (mo[k] >> 20) * ES + sLat[(tid + k * NT) / NE];
    }
    store_ids(ids, sNode);
    __syncthreads();
    gather(g, sNode, sF);
    int gn = g + stride;
    if (gn < ngroups) load_ids(gn, ids);

    int s = 0;
    for (; g < ngroups; g = gn, gn += stride, s = NBUF == 2 ? s ^ 1 : 0) {
        prefetch_group(gn);
        real *sFs = sF + s * NDF * NPL;
        int *sNs = sNode + s * NPL;
        real Hm[MP][9], gv[MP];
        if (!LATE) load_metric(g, Hm, gv);
        if (NBUF == 2 && gn < ngroups) store_ids(ids, sNode + (s ^ 1) * NPL);
        cp_async_wait_all();
        __syncthreads();
        if (gn < ngroups) prefetch_nodes(gn, ids);
        if (NBUF == 2 && gn < ngroups) {
            gather(gn, sNode + (s ^ 1) * NPL, sF + (s ^ 1) * NDF * NPL);
            if (gn + stride < ngroups) load_ids(gn + stride, ids);
        }
        if constexpr (FUSEZ) {
            if (eo) {
                if (lt0.active) grad_pass<G, 0, EOK>(lt0, sFs, sX, sD);
                if (lt1.active) grad_pass<G, 1, EOK>(lt1, sFs, sX, sD);
            } else {
                if (lt0.active) grad_pass<G, 0>(lt0, sFs, sX, sD);
                if (lt1.active) grad_pass<G, 1>(lt1, sFs, sX, sD);
            }
            if constexpr (STAGED) {
                // Bounded wait for group g's spans; every thread learns the outcome.
                const bool ok = mbar_wait(sBar, phase);
                phase ^= 1u;
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) report_wait_fault(tabs);
                    return;
                }
            } else {
                __syncthreads();
            }
            if (lt2.active) {
                const int ee = g * NE + lt2.el;
                const bool eok = ee < nelem;
                // Point c's He row and gpvol: staged, in registers from the
                // start of the group, or loaded here (one point ahead).
                auto he_row = [&](int c, real(&h)[9], real &gp) {
                    const int a = sPerm[line_lat<2, Q>(lt2.la, lt2.lb, c)];
                    if constexpr (!LATE) {
#pragma unroll
                        for (int j = 0; j < 9; ++j) h[j] = Hm[c < MP ? c : 0][j];
                        gp = gv[c < MP ? c : 0];
                    } else if constexpr (STAGED) {
                        const real *hp = reinterpret_cast<const real *>(sHeB) + he_off + (lt2.el * N + a) * 9;
#pragma unroll
                        for (int j = 0; j < 9; ++j) h[j] = hp[j];
                        gp = reinterpret_cast<const real *>(sGpB)[gp_off + lt2.el * N + a];
                    } else {
                        const real *hp = He + (eok ? ((size_t)ee * N + a) * 9 : 0);
#pragma unroll
                        for (int j = 0; j < 9; ++j) h[j] = eok ? ldg(hp + j) : (real)0;
                        gp = eok ? ldg(gpvol + (size_t)ee * N + a) : (real)0;
                    }
                };
                auto mu_at = [&](int o, real r) -> real { return point_mu_e(g, lt2.el, o, r, sFs); };
                zeta_stage<G>(lt2, sFs, sX, he_row, mu_at, Cp, Pr);
            }
            __syncthreads();
            if constexpr (STAGED) {
                if (gn < ngroups) stage(gn);  // the spans of the next group, during the divergence
            }
            if (eo) {
                if (lt0.active) div_pass<G, 0, false, false, EOK>(lt0, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
                __syncthreads();
                if (lt1.active) div_pass<G, 1, false, true, EOK>(lt1, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            } else {
                if (lt0.active) div_pass<G, 0, false, false>(lt0, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
                __syncthreads();
                if (lt1.active) div_pass<G, 1, false, true>(lt1, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            }
        } else {
            if (lt0.active) grad_pass<G, 0>(lt0, sFs, sX, sD);
            if (lt1.active) grad_pass<G, 1>(lt1, sFs, sX, sD);
            if (lt2.active) grad_pass<G, 2>(lt2, sFs, sX, sD);
            __syncthreads();
            // Point pass: physical gradients, stress and contravariant fluxes.
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int i = tid + k * NT;
                if (i >= NE * N) break;
                const int el = i / N, l = i - el * N;
                const int o = el * ES + (l / (Q * Q) * Q + (l / Q) % Q) * QP + l % Q;
                real gi[3][5];
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int f = 0; f < 5; ++f) gi[d][f] = sX[(d * 5 + f) * NPL + o];
                const real r = sFs[D_RHO * NPL + o];
                const real uu[3] = {sFs[D_U0 * NPL + o], sFs[D_U1 * NPL + o], sFs[D_U2 * NPL + o]};
                const real muf = sFs[D_MUF * NPL + o], ms = sFs[D_MUS * NPL + o];
                const real me = point_mu_e(g, el, o, r, sFs);
                real F[3][NX];
                point_flux(gi, r, uu, muf, ms, me, Hm[k], gv[k], F);
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int x = 0; x < NX; ++x) sX[(d * NX + x) * NPL + o] = F[d][x];
                sFs[P_NUE * NPL + o] = me / r;
                sFs[P_KAP * NPL + o] = kappa_e(muf, me, ms, r, Cp, Pr);
            }
            __syncthreads();
            if (lt0.active) div_pass<G, 0, true, false>(lt0, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            if (lt1.active) div_pass<G, 1, false, false>(lt1, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
            __syncthreads();
            if (lt2.active) div_pass<G, 2, false, true>(lt2, sFs, sX, sD, sNs, npoin, Rmass, Rmom, Rener);
        }
        __syncthreads();
        if (NBUF == 1 && gn < ngroups) {  // the next group's node ids, then its fields
            store_ids(ids, sNode);
            __syncthreads();
            gather(gn, sNode, sF);
            if (gn + stride < ngroups) load_ids(gn + stride, ids);
        }
    }
}

template <typename real, int P, int VISC>
cudaError_t launch_diffu_pn(const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    using G = DiffuGeom<real, P>;
    constexpr size_t smem = diffu_smem_bytes<G>();
    static_assert(smem <= 227 * 1024, "shared memory budget");
    static_assert(G::NE >= 1, "element group");
    auto kern = diffu_kernel<G, VISC>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    if (sizeof(real) == 4) {
        err = cudaMemcpyToSymbolAsync(c_Df, table_D<float>(tabs), sizeof(float) * 3 * G::Q * G::Q,
                                      sizeof(float) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
        constexpr bool eo = ((DIFFU_EO >> P) & 1) != 0 && diffu_fusez<G>();
        if (err == cudaSuccess && eo)
            err = cudaMemcpyToSymbolAsync(c_DEO, tabs->EO, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
        if (err == cudaSuccess && eo)
            err = cudaMemcpyToSymbolAsync(c_DEOp, tabs->EOp, sizeof(float) * kTableEOMax,
                                          sizeof(float) * kTableEOMax * P, cudaMemcpyDeviceToDevice, st);
    }
    else
        err = cudaMemcpyToSymbolAsync(c_Dd, table_D<double>(tabs), sizeof(double) * 3 * G::Q * G::Q,
                                      sizeof(double) * kTableDMax * P, cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return err;
    const int ngroups = (a.nelem + G::NE - 1) / G::NE;
    const int grid = persistent_grid(kern, G::NT, smem, ngroups);
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    const int linemap = DIFFU_LINEMAP_MODE == 2 ? (a.npoin < (long long)a.nelem * G::N ? 1 : 0) : DIFFU_LINEMAP_MODE;
    kern<<<grid, G::NT, smem, st>>>(a.nelem, a.npoin, ngroups, a.connec, a.He, a.gpvol, tabs, a.Cp, a.Pr, a.rho, a.u,
                                    a.Tem, a.mu_fluid, a.mu_e, a.mu_sgs, a.nu_elem, a.Rmass, a.Rmom, a.Rener,
                                    linemap);
    return cudaGetLastError();
}

template <typename real, int P>
cudaError_t launch_diffu_p(const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    if (a.nu_elem) return launch_diffu_pn<real, P, VISC_NU_ELEM>(a, tabs, st);
    return launch_diffu_pn<real, P, VISC_MU_E>(a, tabs, st);
}

}  // namespace

template <typename real>
cudaError_t launch_diffu_plain(int porder, const DiffuArgs<real> &a, const TableScratch *tabs, cudaStream_t st)
{
    switch (porder) {
    case 1: return launch_diffu_p<real, 1>(a, tabs, st);
    case 2: return launch_diffu_p<real, 2>(a, tabs, st);
    case 3: return launch_diffu_p<real, 3>(a, tabs, st);
    case 4: return launch_diffu_p<real, 4>(a, tabs, st);
    case 5: return launch_diffu_p<real, 5>(a, tabs, st);
    case 6: return launch_diffu_p<real, 6>(a, tabs, st);
    case 7: return launch_diffu_p<real, 7>(a, tabs, st);
    case 8: return launch_diffu_p<real, 8>(a, tabs, st);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_diffu_plain<float>(int, const DiffuArgs<float> &, const TableScratch *, cudaStream_t);
template cudaError_t launch_diffu_plain<double>(int, const DiffuArgs<double> &, const TableScratch *, cudaStream_t);

}  // namespace msod
