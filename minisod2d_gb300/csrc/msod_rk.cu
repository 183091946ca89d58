// msod_rk.cu -- lumped mass and the explicit RK4 update around the two residual
// calls.
//
// The reference's parameters name the time integrator its kernels serve --
// flag_rk_order = 4 and flag_solver_type = 1, a lumped mass matrix
// (mod_numerical_params.f90:8,20) -- but it contains neither.  This file
// provides both on the library's residuals:
//   Ml(p)  = sum of gpvol(e, g) over the element points g at node p (GLL
//            quadrature at the nodes: the lumped mass matrix is diagonal);
//   dU/dt  = -Ml^-1 (R_conv(U) + R_diff(U)),  U = (rho, q = rho u, rhoE);
//   k_1 = F(U0), k_2 = F(U0 + dt/2 k_1), k_3 = F(U0 + dt/2 k_2),
//   k_4 = F(U0 + dt k_3), U1 = U0 + dt/6 (k_1 + 2 k_2 + 2 k_3 + k_4),
// with the primitive fields each residual call takes derived at every stage:
//   u = q / rho, E = rhoE / rho (the specific energy the convection takes),
//   pr = (gamma - 1) (rhoE - rho |u|^2 / 2), Tem = pr / (rho Rgas).
// Both residuals are the weak forms their kernels assemble (test functions on
// the left), so each enters the update with a minus sign.  Each stage calls
// msod_convec_diffusion_ijk: one kernel for both residuals at porder 4 in the
// default form, the two drop-in calls msod_convec_ijk and msod_diffusion_ijk
// otherwise, so the form msod_set_mode selects (precision, artificial
// viscosity) applies to every stage.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "msod.h"
#include "msod_internal.h"

namespace msod {
namespace {

// Ml(connec(e, a)) += gpvol(e, a): one thread per element point, element-
// fastest as connec stores them; atomics assemble the shared nodes.
__global__ void lumped_mass_kernel(int nelem, int n, int npoin, const int *__restrict__ connec,
                                   const float *__restrict__ gpvol, float *__restrict__ Ml)
{
    const long long total = (long long)nelem * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(i / nelem), e = (int)(i - (long long)a * nelem);
        const int p = __ldg(connec + i) - 1;
        if (p >= 0 && p < npoin) atomicAdd(Ml + p, __ldg(gpvol + (size_t)e * n + a));
    }
}

// Primitive fields u, E, pr, Tem of node p's state (rho, q0..2, rhoE).
__device__ __forceinline__ void rk_primitives(size_t np, int p, float r, float q0, float q1, float q2, float re,
                                              float gamma, float Rgas, float *__restrict__ u, float *__restrict__ E,
                                              float *__restrict__ pr, float *__restrict__ Tem)
{
    const float inv = 1.0f / r;
    const float u0 = q0 * inv, u1 = q1 * inv, u2 = q2 * inv;
    u[p] = u0;
    u[np + p] = u1;
    u[2 * np + p] = u2;
    E[p] = re * inv;
    const float pp = (gamma - 1.0f) * (re - 0.5f * r * (u0 * u0 + u1 * u1 + u2 * u2));
    pr[p] = pp;
    Tem[p] = pp * inv / Rgas;
}

// Primitive fields of the state for the first stage's residual calls.
__global__ void rk_derive_kernel(int npoin, const float *__restrict__ rho, const float *__restrict__ q,
                                 const float *__restrict__ rhoE, float gamma, float Rgas, float *__restrict__ u,
                                 float *__restrict__ E, float *__restrict__ pr, float *__restrict__ Tem)
{
    const size_t np = (size_t)npoin;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npoin; p += gridDim.x * blockDim.x)
        rk_primitives(np, p, rho[p], q[p], q[np + p], q[2 * np + p], rhoE[p], gamma, Rgas, u, E, pr, Tem);
}

// One stage: k = -(Rc + Rd) / Ml per component (rho, q0..2, rhoE); S = k
// (first stage) or S + w k; the state becomes U0 + cnext dt k, with the next
// stage's primitive fields written beside it, or at the last stage
// U0 + dt/6 (S + k).
__global__ void rk_stage_kernel(int npoin, const float *__restrict__ Ml, const float *__restrict__ Rc_m,
                                const float *__restrict__ Rc_q, const float *__restrict__ Rc_e,
                                const float *__restrict__ Rd_m, const float *__restrict__ Rd_q,
                                const float *__restrict__ Rd_e, const float *__restrict__ U0, float *__restrict__ S,
                                float *__restrict__ rho, float *__restrict__ q, float *__restrict__ rhoE, float dt,
                                int stage, float gamma, float Rgas, float *__restrict__ u, float *__restrict__ E,
                                float *__restrict__ pr, float *__restrict__ Tem)
{
    const size_t np = (size_t)npoin;
    const float w = (stage == 1 || stage == 2) ? 2.0f : 1.0f;
    const float cnext = stage < 2 ? 0.5f : 1.0f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npoin; p += gridDim.x * blockDim.x) {
        const float inv = 1.0f / Ml[p];
        float k[5];
        k[0] = -(Rc_m[p] + Rd_m[p]) * inv;
#pragma unroll
        for (int c = 0; c < 3; ++c) k[1 + c] = -(Rc_q[c * np + p] + Rd_q[c * np + p]) * inv;
        k[4] = -(Rc_e[p] + Rd_e[p]) * inv;
        float *out[5] = {rho + p, q + p, q + np + p, q + 2 * np + p, rhoE + p};
        float un[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const float u0 = U0[c * np + p];
            const float s = stage == 0 ? k[c] : fmaf(w, k[c], S[c * np + p]);
            if (stage < 3) {
                S[c * np + p] = s;
                un[c] = fmaf(cnext * dt, k[c], u0);
            } else {
                un[c] = fmaf(dt / 6.0f, s, u0);
            }
            *out[c] = un[c];
        }
        if (stage < 3) rk_primitives(np, p, un[0], un[1], un[2], un[3], un[4], gamma, Rgas, u, E, pr, Tem);
    }
}

int cuda_status(const char *what)
{
    const cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) return MSOD_OK;
    return set_error(MSOD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

int grid_for(long long n)
{
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = (n + 255) / 256;
    return (int)(blocks < 8LL * sms ? (blocks > 0 ? blocks : 1) : 8LL * sms);
}

// Workspace: U0 (5), primitive u (3), E, pr, Tem (3), Rc (5), Rd (5), S (5) npoin floats.
constexpr int kRkPlanes = 5 + 3 + 3 + 5 + 5 + 5;

}  // namespace
}  // namespace msod

using namespace msod;

extern "C" {

int msod_lumped_mass(int porder, int nelem, int npoin, const int *connec, const float *gpvol, float *Ml, void *stream)
{
    clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER) return set_error(MSOD_ERR_PORDER, "porder %d", porder);
    if (nelem < 1 || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    const long long n = (long long)(porder + 1) * (porder + 1) * (porder + 1);
    if ((long long)nelem * n >= (1LL << 31)) return set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode exceeds int32");
    if (!connec || !gpvol || !Ml) return set_error(MSOD_ERR_INVALID_ARG, "NULL connec, gpvol or Ml");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(Ml, 0, sizeof(float) * (size_t)npoin, st) != cudaSuccess) return cuda_status("Ml zeroing");
    lumped_mass_kernel<<<grid_for((long long)nelem * n), 256, 0, st>>>(nelem, (int)n, npoin, connec, gpvol, Ml);
    return cuda_status("lumped mass launch");
}

int msod_rk4_workspace_bytes(int npoin, size_t *bytes)
{
    clear_error();
    if (npoin < 1 || !bytes) return set_error(MSOD_ERR_INVALID_ARG, "npoin must be positive and bytes non-NULL");
    *bytes = sizeof(float) * (size_t)kRkPlanes * (size_t)npoin;
    return MSOD_OK;
}

int msod_rk4_step(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                  const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                  const int *gmshAtoK, float Cp, float Pr, float gamma, float Rgas, const float *Ml,
                  const float *mu_fluid, const float *mu_e, const float *mu_sgs, float dt, float *rho, float *q,
                  float *rhoE, void *workspace, size_t workspace_bytes, void *stream)
{
    clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER) return set_error(MSOD_ERR_PORDER, "porder %d", porder);
    if (nelem < 1 || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    const long long nn = (long long)(porder + 1) * (porder + 1) * (porder + 1);
    if ((long long)nelem * nn >= (1LL << 31)) return set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode exceeds int32");
    if (!Ml || !rho || !q || !rhoE || !workspace)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL mass, state or workspace");
    if (!(gamma > 1.0f) || !(Rgas > 0.0f) || !std::isfinite(dt))
        return set_error(MSOD_ERR_INVALID_ARG, "gamma must exceed 1, Rgas be positive and dt finite");
    const size_t np = (size_t)npoin;
    if (reinterpret_cast<uintptr_t>(workspace) % alignof(float) != 0)
        return set_error(MSOD_ERR_INVALID_ARG, "workspace is not %zu-byte aligned", alignof(float));
    if (workspace_bytes < sizeof(float) * (size_t)kRkPlanes * np)
        return set_error(MSOD_ERR_INVALID_ARG, "workspace of %zu bytes, %zu needed", workspace_bytes,
                         sizeof(float) * (size_t)kRkPlanes * np);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *w = static_cast<float *>(workspace);
    float *U0 = w, *u = U0 + 5 * np, *E = u + 3 * np, *pr = E + np, *Tem = pr + np;
    float *Rc = Tem + np, *Rd = Rc + 5 * np, *S = Rd + 5 * np;
    // U0: the state at the start of the step, components rho, q0..2, rhoE.
    if (cudaMemcpyAsync(U0, rho, sizeof(float) * np, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(U0 + np, q, sizeof(float) * 3 * np, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(U0 + 4 * np, rhoE, sizeof(float) * np, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return cuda_status("state copy");
    const int grid = grid_for(npoin);
    rk_derive_kernel<<<grid, 256, 0, st>>>(npoin, rho, q, rhoE, gamma, Rgas, u, E, pr, Tem);
    if (cuda_status("primitive-field launch")) return MSOD_ERR_CUDA;
    for (int stage = 0; stage < 4; ++stage) {
        int rc = msod_convec_diffusion_ijk(porder, nelem, npoin, connec, nullptr, nullptr, He, gpvol, dlxigp_ip,
                                           nullptr, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, u, q, rho, pr,
                                           E, Tem, mu_fluid, mu_e, mu_sgs, Rc, Rc + np, Rc + 4 * np, Rd, Rd + np,
                                           Rd + 4 * np, stream);
        if (rc) return rc;
        rk_stage_kernel<<<grid, 256, 0, st>>>(npoin, Ml, Rc, Rc + np, Rc + 4 * np, Rd, Rd + np, Rd + 4 * np, U0, S,
                                              rho, q, rhoE, dt, stage, gamma, Rgas, u, E, pr, Tem);
        rc = cuda_status("stage launch");
        if (rc) return rc;
    }
    return MSOD_OK;
}

}  // extern "C"
