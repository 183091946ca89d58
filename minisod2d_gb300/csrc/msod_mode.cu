// msod_mode.cu -- the process-wide form of the drop-in calls (msod_set_mode).
//
// The reference fixes its form at compile time (rp, mod_constants.f90:5) and
// reads mu_e from its caller (elem_diffu.f90:19).  msod_set_mode lets a
// driver that keeps its two calls -- full_convec_ijk and full_diffusion_ijk
// through msod_convec_ijk / msod_diffusion_ijk -- switch what they compute:
//   precision  MSOD_PREC_FP32 (the plain kernels, default) or MSOD_PREC_FP16 /
//              MSOD_PREC_BF16: the tensor-core kernels write FP64 residuals
//              into library buffers, and a conversion pass writes them into
//              the caller's FP32 arrays;
//   mu_e       MSOD_MU_E_GIVEN (the caller's mu_e, default), MSOD_MU_E_PLAIN
//              (the entropy-viscosity estimator) or MSOD_MU_E_LEARNED (the
//              network, with the estimator as per-element fallback); both
//              ignore the mu_e argument and take p = rho Rgas Tem with the
//              driver's gas constants (main.f90:52: gamma = 1.4, Rgas = 287)
//              and the estimator constants ce = 0.1, cmax = 0.5
//              (mod_numerical_params.f90:23-24).
// The library buffers (FP64 residuals, per-element viscosity, pressure) are
// per device, grow on demand with cudaMalloc and are shared by all calls on
// that device: calls that overlap on the GPU race on them.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "msod.h"
#include "msod_internal.h"

namespace msod {

namespace {

std::atomic<int> g_prec{MSOD_PREC_FP32};
std::atomic<int> g_mue{MSOD_MU_E_GIVEN};
std::atomic<const msod_mlp *> g_mlp{nullptr};

constexpr float kGamma = 1.4f, kRgas = 287.0f, kCe = 0.1f, kCmax = 0.5f;

enum { BUF_R64 = 0, BUF_NU, BUF_P, NBUF };
std::mutex g_buf_mu;
void *g_buf[64][NBUF] = {};
size_t g_buf_size[64][NBUF] = {};

void *mode_buffer(int slot, size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_buf_mu);
    if (g_buf_size[dev][slot] < bytes) {
        if (g_buf[dev][slot]) cudaFree(g_buf[dev][slot]);
        g_buf[dev][slot] = nullptr;
        g_buf_size[dev][slot] = 0;
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        g_buf[dev][slot] = p;
        g_buf_size[dev][slot] = bytes;
    }
    return g_buf[dev][slot];
}

__global__ void to_float_kernel(const double *__restrict__ src, float *__restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

__global__ void pressure_kernel(const float *__restrict__ rho, const float *__restrict__ Tem, float Rgas,
                                float *__restrict__ p, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = rho[i] * Rgas * Tem[i];
}

int launch_status(const char *what)
{
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MSOD_OK : set_error(MSOD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// FP64 residual buffers (Rmass, Rmom(3), Rener) and their conversion into the caller's arrays.
struct R64 {
    double *mass, *mom, *ener;
};

int r64_buffers(int npoin, R64 &r)
{
    double *b = static_cast<double *>(mode_buffer(BUF_R64, sizeof(double) * 5 * (size_t)npoin));
    if (!b) return set_error(MSOD_ERR_CUDA, "could not allocate the FP64 residual buffers");
    r.mass = b;
    r.mom = b + npoin;
    r.ener = b + 4 * (size_t)npoin;
    return MSOD_OK;
}

int r64_to_float(const R64 &r, int npoin, float *Rmass, float *Rmom, float *Rener, cudaStream_t st)
{
    const int grid = 4 * 152, block = 256;
    to_float_kernel<<<grid, block, 0, st>>>(r.mass, Rmass, (size_t)npoin);
    to_float_kernel<<<grid, block, 0, st>>>(r.mom, Rmom, 3 * (size_t)npoin);
    to_float_kernel<<<grid, block, 0, st>>>(r.ener, Rener, (size_t)npoin);
    return launch_status("residual conversion launch");
}

}  // namespace

bool mode_is_default_convec() { return g_prec.load() == MSOD_PREC_FP32; }
bool mode_is_default_diffusion() { return g_prec.load() == MSOD_PREC_FP32 && g_mue.load() == MSOD_MU_E_GIVEN; }

void mode_release()
{
    std::lock_guard<std::mutex> lk(g_buf_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (int d = 0; d < 64; ++d)
        for (int s = 0; s < NBUF; ++s)
            if (g_buf[d][s]) {
                cudaSetDevice(d);
                cudaFree(g_buf[d][s]);
                g_buf[d][s] = nullptr;
                g_buf_size[d][s] = 0;
            }
    cudaSetDevice(cur);
}

int mode_convec(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                const int *gmshAtoK, const float *u, const float *q, const float *rho, const float *pr,
                const float *E, float *Rmass, float *Rmom, float *Rener, void *stream)
{
    if (!Rmass || !Rmom || !Rener || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "NULL residual array");
    R64 r{};
    int rc = r64_buffers(npoin, r);
    if (rc) return rc;
    rc = msod_convec_ijk_mixed(g_prec.load(), porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK,
                               gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, r.mass, r.mom, r.ener, stream);
    if (rc) return rc;
    return r64_to_float(r, npoin, Rmass, Rmom, Rener, static_cast<cudaStream_t>(stream));
}

int mode_diffusion(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                   const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                   const int *gmshAtoK, float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                   const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass, float *Rmom,
                   float *Rener, void *stream)
{
    const int prec = g_prec.load(), mue = g_mue.load();
    const msod_mlp *mlp = g_mlp.load();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (nelem < 1 || npoin < 1 || !rho || !Tem) return set_error(MSOD_ERR_INVALID_ARG, "bad sizes or NULL field");
    // FP32 with the network: the one-call learned diffusion.
    if (mue == MSOD_MU_E_LEARNED && prec == MSOD_PREC_FP32)
        return msod_diffusion_ijk_learned(mlp, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK,
                                          gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_sgs, Tem,
                                          kRgas, kGamma, kCe, kCmax, Rmass, Rmom, Rener, nullptr, nullptr, stream);
    // Otherwise the per-element viscosity first (estimator or network + fallback).
    float *nu = nullptr;
    int rc = MSOD_OK;
    if (mue != MSOD_MU_E_GIVEN) {
        nu = static_cast<float *>(mode_buffer(BUF_NU, sizeof(float) * (size_t)nelem));
        if (!nu) return set_error(MSOD_ERR_CUDA, "could not allocate the per-element viscosity");
        if (mue == MSOD_MU_E_LEARNED) {
            rc = msod_learned_viscosity(mlp, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI,
                                        gmshAtoJ, gmshAtoK, rho, u, Tem, kRgas, kGamma, kCe, kCmax, nu, nullptr,
                                        stream);
        } else {
            float *p = static_cast<float *>(mode_buffer(BUF_P, sizeof(float) * (size_t)npoin));
            if (!p) return set_error(MSOD_ERR_CUDA, "could not allocate the pressure buffer");
            pressure_kernel<<<4 * 152, 256, 0, st>>>(rho, Tem, kRgas, p, npoin);
            rc = launch_status("pressure launch");
            if (!rc)
                rc = msod_entropy_viscosity(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI,
                                            gmshAtoJ, gmshAtoK, rho, u, p, kGamma, kCe, kCmax, 1, nullptr, nu,
                                            nullptr, stream);
        }
        if (rc) return rc;
    }
    if (prec == MSOD_PREC_FP32)
        return msod_diffusion_ijk_nu(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI,
                                     gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, nu, mu_sgs, Rmass, Rmom,
                                     Rener, stream);
    if (!Rmass || !Rmom || !Rener) return set_error(MSOD_ERR_INVALID_ARG, "NULL residual array");
    R64 r{};
    rc = r64_buffers(npoin, r);
    if (rc) return rc;
    rc = nu ? msod_diffusion_ijk_mixed_nu(prec, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK,
                                          gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, nu, mu_sgs,
                                          r.mass, r.mom, r.ener, stream)
            : msod_diffusion_ijk_mixed(prec, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK,
                                       gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs,
                                       r.mass, r.mom, r.ener, stream);
    if (rc) return rc;
    return r64_to_float(r, npoin, Rmass, Rmom, Rener, st);
}

}  // namespace msod

using namespace msod;

extern "C" {

int msod_set_mode(int precision, int mu_e_mode, const msod_mlp *mlp)
{
    clear_error();
    if (precision != MSOD_PREC_FP32 && precision != MSOD_PREC_FP16 && precision != MSOD_PREC_BF16)
        return set_error(MSOD_ERR_INVALID_ARG, "precision %d is not MSOD_PREC_FP32/FP16/BF16", precision);
    if (mu_e_mode != MSOD_MU_E_GIVEN && mu_e_mode != MSOD_MU_E_PLAIN && mu_e_mode != MSOD_MU_E_LEARNED)
        return set_error(MSOD_ERR_INVALID_ARG, "mu_e mode %d is not MSOD_MU_E_GIVEN/PLAIN/LEARNED", mu_e_mode);
    if (mu_e_mode == MSOD_MU_E_LEARNED && !mlp)
        return set_error(MSOD_ERR_INVALID_ARG, "MSOD_MU_E_LEARNED needs a network");
    g_mlp.store(mu_e_mode == MSOD_MU_E_LEARNED ? mlp : nullptr);
    g_mue.store(mu_e_mode);
    g_prec.store(precision);
    return MSOD_OK;
}

int msod_get_mode(int *precision, int *mu_e_mode)
{
    clear_error();
    if (precision) *precision = g_prec.load();
    if (mu_e_mode) *mu_e_mode = g_mue.load();
    return MSOD_OK;
}

}  // extern "C"
