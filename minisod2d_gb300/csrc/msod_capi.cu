// msod_capi.cu -- extern "C" entry points of libmsod (declared in include/msod.h).
//
// The kernel entry points mirror the reference's two hot-path subroutines
// argument for argument (elem_convec.f90:198, :433; elem_diffu.f90:10), with
// porder passed at run time (a compile-time parameter in the reference,
// mod_constants.f90:16) and a CUDA stream appended.  Arguments are validated
// on the host; errors are returned as MSOD_ERR_* codes with a message for
// msod_last_error_string().
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "msod.h"
#include "msod_internal.h"
#include "msod_kernels.h"

namespace msod {

namespace {
thread_local char g_err[512] = "";
std::atomic<int> g_checked{0};

// Per-device library-owned device memory: the 4-byte flag word of
// msod_check_element_tables and the per-call element tables of the kernels,
// one table area per porder (calls of different porders on different streams
// do not share one).
std::mutex g_mu;
int *g_flags[64] = {nullptr};
TableScratch *g_tables[64] = {nullptr};

TableScratch *device_tables(int porder)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (porder < 0 || porder > MSOD_MAX_PORDER) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_tables[dev]) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(TableScratch) * (MSOD_MAX_PORDER + 1)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(TableScratch) * (MSOD_MAX_PORDER + 1)) != cudaSuccess) {
            cudaFree(p);
            return nullptr;
        }
        g_tables[dev] = static_cast<TableScratch *>(p);
    }
    return g_tables[dev] + porder;
}

int *device_flags()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_flags[dev]) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        g_flags[dev] = static_cast<int *>(p);
    }
    return g_flags[dev];
}
}  // namespace

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_err[0] = '\0'; }

bool checked_mode() { return g_checked.load(std::memory_order_relaxed) != 0; }

static int cuda_status(cudaError_t err, const char *what)
{
    if (err == cudaSuccess) return MSOD_OK;
    return set_error(MSOD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

static int check_geometry(int porder, int nelem, int npoin, const void *connec, const void *He,
                          const void *gpvol, const void *dlx, const void *inv, const void *ai, const void *aj,
                          const void *ak)
{
    if (porder < 1 || porder > MSOD_MAX_PORDER)
        return set_error(MSOD_ERR_PORDER, "porder %d has no instantiation (1..%d)", porder, MSOD_MAX_PORDER);
    if (nelem < 1 || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    const long long n = (long long)(porder + 1) * (porder + 1) * (porder + 1);
    if ((long long)nelem * n >= (1LL << 31))
        return set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode exceeds the int32 range of connec");
    if (!connec || !He || !gpvol || !dlx || !inv || !ai || !aj || !ak)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL element or geometry array");
    return MSOD_OK;
}

static int run_check(int porder, int nelem, int npoin, const int *connec, const float *dlx, const int *inv,
                     const int *ai, const int *aj, const int *ak, cudaStream_t st)
{
    int *flags = device_flags();
    if (!flags) return set_error(MSOD_ERR_CUDA, "could not allocate the validation flag");
    int rc = cuda_status(cudaMemsetAsync(flags, 0, sizeof(int), st), "cudaMemsetAsync");
    if (rc) return rc;
    rc = cuda_status(launch_check_tables(porder, nelem, npoin, connec, dlx, inv, ai, aj, ak, flags, st),
                     "check_tables launch");
    if (rc) return rc;
    int h = 0;
    rc = cuda_status(cudaMemcpyAsync(&h, flags, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    if (rc) return rc;
    rc = cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (rc) return rc;
    if (h)
        return set_error(MSOD_ERR_BAD_TABLES,
                         "element tables failed validation (bits 0x%x: 1 invAtoIJK not a permutation, 2 "
                         "invAtoIJK/gmshAtoIJK disagree, 4 dlxigp_ip not 1-D structured, 8 connec out of range)",
                         h);
    return MSOD_OK;
}

// Checked mode, after a kernel: synchronise, then report (and clear) a bounded
// wait of the kernel that ran out.
static int check_wait_fault(TableScratch *tabs, cudaStream_t st, const char *what)
{
    int rc = cuda_status(cudaStreamSynchronize(st), what);
    if (rc) return rc;
    int h = 0;
    rc = cuda_status(cudaMemcpy(&h, &tabs->wait_fault, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (rc) return rc;
    if (h) {
        cudaMemset(&tabs->wait_fault, 0, sizeof(int));
        return set_error(MSOD_ERR_CUDA, "%s: a bulk copy into shared memory did not complete in time; "
                                        "the residuals are incomplete", what);
    }
    return MSOD_OK;
}

template <typename real>
static int zero_outputs(real *Rmass, real *Rmom, real *Rener, int npoin, cudaStream_t st)
{
    const size_t b = sizeof(real) * (size_t)npoin;
    int rc = cuda_status(cudaMemsetAsync(Rmass, 0, b, st), "cudaMemsetAsync(Rmass)");
    if (!rc) rc = cuda_status(cudaMemsetAsync(Rmom, 0, 3 * b, st), "cudaMemsetAsync(Rmom)");
    if (!rc) rc = cuda_status(cudaMemsetAsync(Rener, 0, b, st), "cudaMemsetAsync(Rener)");
    return rc;
}

template <typename real>
static int convec_impl(int porder, int nelem, int npoin, const int *connec, const real *He, const real *gpvol,
                       const real *dlx, const int *inv, const int *ai, const int *aj, const int *ak, const real *u,
                       const real *q, const real *rho, const real *pr, const real *E, real *Rmass, real *Rmom,
                       real *Rener, void *stream)
{
    clear_error();
    int rc = check_geometry(porder, nelem, npoin, connec, He, gpvol, dlx, inv, ai, aj, ak);
    if (rc) return rc;
    if (!u || !q || !rho || !pr || !E || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode() && sizeof(real) == 4) {
        rc = run_check(porder, nelem, npoin, connec, (const float *)dlx, inv, ai, aj, ak, st);
        if (rc) return rc;
    }
    TableScratch *tabs = device_tables(porder);
    if (!tabs) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    ConvecArgs<real> a;
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol; a.dlxigp_ip = dlx;
    a.invAtoIJK = inv; a.AtoI = ai; a.AtoJ = aj; a.AtoK = ak;
    a.u = u; a.q = q; a.rho = rho; a.pr = pr; a.E = E; a.Rmass = Rmass; a.Rmom = Rmom; a.Rener = Rener;
    rc = cuda_status(launch_table_prep<real>(porder, a, tabs, st), "table preparation launch");
    if (!rc) rc = cuda_status(launch_convec_plain<real>(porder, a, tabs, st), "convection kernel launch");
    if (!rc && checked_mode()) rc = check_wait_fault(tabs, st, "convection kernel");
    return rc;
}

template <typename real>
static int diffu_impl(int porder, int nelem, int npoin, const int *connec, const real *He, const real *gpvol,
                      const real *dlx, const int *inv, const int *ai, const int *aj, const int *ak, real Cp, real Pr,
                      const real *rho, const real *u, const real *Tem, const real *mu_fluid, const real *mu_e,
                      const real *mu_sgs, real *Rmass, real *Rmom, real *Rener, void *stream,
                      const real *nu_elem = nullptr)
{
    clear_error();
    int rc = check_geometry(porder, nelem, npoin, connec, He, gpvol, dlx, inv, ai, aj, ak);
    if (rc) return rc;
    if (!rho || !u || !Tem || !mu_fluid || !(mu_e || nu_elem) || !mu_sgs || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    if (!(Pr != (real)0)) return set_error(MSOD_ERR_INVALID_ARG, "Pr must be non-zero");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode() && sizeof(real) == 4) {
        rc = run_check(porder, nelem, npoin, connec, (const float *)dlx, inv, ai, aj, ak, st);
        if (rc) return rc;
    }
    TableScratch *tabs = device_tables(porder);
    if (!tabs) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    DiffuArgs<real> a;
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol; a.dlxigp_ip = dlx;
    a.invAtoIJK = inv; a.AtoI = ai; a.AtoJ = aj; a.AtoK = ak; a.Cp = Cp; a.Pr = Pr;
    a.rho = rho; a.u = u; a.Tem = Tem; a.mu_fluid = mu_fluid; a.mu_e = mu_e; a.mu_sgs = mu_sgs; a.nu_elem = nu_elem;
    a.Rmass = Rmass; a.Rmom = Rmom; a.Rener = Rener;
    rc = cuda_status(launch_table_prep<real>(porder, a, tabs, st), "table preparation launch");
    if (!rc) rc = cuda_status(launch_diffu_plain<real>(porder, a, tabs, st), "diffusion kernel launch");
    if (!rc && checked_mode()) rc = check_wait_fault(tabs, st, "diffusion kernel");
    return rc;
}

static int fused_impl(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                      const float *dlx, const int *inv, const int *ai, const int *aj, const int *ak, float Cp,
                      float Pr, const float *u, const float *q, const float *rho, const float *pr, const float *E,
                      const float *Tem, const float *mu_fluid, const float *mu_e, const float *mu_sgs,
                      float *Rmass_c, float *Rmom_c, float *Rener_c, float *Rmass_d, float *Rmom_d,
                      float *Rener_d, void *stream)
{
    clear_error();
    int rc = check_geometry(porder, nelem, npoin, connec, He, gpvol, dlx, inv, ai, aj, ak);
    if (rc) return rc;
    if (!u || !q || !rho || !pr || !E || !Tem || !mu_fluid || !mu_e || !mu_sgs)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field array");
    float *outs[6] = {Rmass_c, Rmom_c, Rener_c, Rmass_d, Rmom_d, Rener_d};
    for (int i = 0; i < 6; ++i) {
        if (!outs[i]) return set_error(MSOD_ERR_INVALID_ARG, "NULL residual array");
        for (int j = 0; j < i; ++j)
            if (outs[i] == outs[j]) return set_error(MSOD_ERR_INVALID_ARG, "the six residual arrays must be distinct");
    }
    if (!(Pr != 0.0f)) return set_error(MSOD_ERR_INVALID_ARG, "Pr must be non-zero");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode()) {
        rc = run_check(porder, nelem, npoin, connec, dlx, inv, ai, aj, ak, st);
        if (rc) return rc;
    }
    TableScratch *tabs = device_tables(porder);
    if (!tabs) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    rc = zero_outputs(Rmass_c, Rmom_c, Rener_c, npoin, st);
    if (!rc) rc = zero_outputs(Rmass_d, Rmom_d, Rener_d, npoin, st);
    if (rc) return rc;
    ConvecArgs<float> c;
    c.nelem = nelem; c.npoin = npoin; c.connec = connec; c.He = He; c.gpvol = gpvol; c.dlxigp_ip = dlx;
    c.invAtoIJK = inv; c.AtoI = ai; c.AtoJ = aj; c.AtoK = ak;
    c.u = u; c.q = q; c.rho = rho; c.pr = pr; c.E = E; c.Rmass = Rmass_c; c.Rmom = Rmom_c; c.Rener = Rener_c;
    DiffuArgs<float> d;
    static_cast<ElementArgs<float> &>(d) = c;
    d.Cp = Cp; d.Pr = Pr; d.rho = rho; d.u = u; d.Tem = Tem; d.mu_fluid = mu_fluid; d.mu_e = mu_e;
    d.mu_sgs = mu_sgs; d.nu_elem = nullptr; d.Rmass = Rmass_d; d.Rmom = Rmom_d; d.Rener = Rener_d;
    rc = cuda_status(launch_table_prep<float>(porder, c, tabs, st), "table preparation launch");
    if (!rc) rc = cuda_status(launch_fused(porder, c, d, tabs, st), "convection + diffusion kernel launch");
    if (!rc && checked_mode()) rc = check_wait_fault(tabs, st, "convection + diffusion kernel");
    return rc;
}

}  // namespace msod

using namespace msod;

extern "C" {

int msod_version(void) { return MSOD_VERSION; }

const char *msod_last_error_string(void) { return g_err; }

int msod_set_checked(int enabled)
{
    g_checked.store(enabled ? 1 : 0);
    return MSOD_OK;
}

int msod_init(int device)
{
    clear_error();
    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess || count < 1)
        return set_error(MSOD_ERR_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(err));
    if (device < 0 || device >= count) return set_error(MSOD_ERR_INVALID_ARG, "device %d of %d", device, count);
    return cuda_status(cudaSetDevice(device), "cudaSetDevice");
}

int msod_finalize(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (int d = 0; d < 64; ++d)
        if (g_flags[d] || g_tables[d]) {
            cudaSetDevice(d);
            if (g_flags[d]) cudaFree(g_flags[d]);
            if (g_tables[d]) cudaFree(g_tables[d]);
            g_flags[d] = nullptr;
            g_tables[d] = nullptr;
        }
    cudaSetDevice(cur);
    mode_release();
    return MSOD_OK;
}

int msod_malloc(void **ptr, size_t bytes)
{
    clear_error();
    if (!ptr) return set_error(MSOD_ERR_INVALID_ARG, "NULL output pointer");
    *ptr = nullptr;
    return cuda_status(cudaMalloc(ptr, bytes ? bytes : 1), "cudaMalloc");
}

int msod_free(void *ptr) { return cuda_status(cudaFree(ptr), "cudaFree"); }

int msod_h2d(void *dst, const void *src, size_t bytes, void *stream)
{
    return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, static_cast<cudaStream_t>(stream)),
                       "cudaMemcpyAsync(H2D)");
}

int msod_d2h(void *dst, const void *src, size_t bytes, void *stream)
{
    return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)),
                       "cudaMemcpyAsync(D2H)");
}

int msod_memset(void *dst, int value, size_t bytes, void *stream)
{
    return cuda_status(cudaMemsetAsync(dst, value, bytes, static_cast<cudaStream_t>(stream)), "cudaMemsetAsync");
}

int msod_stream_synchronize(void *stream)
{
    return cuda_status(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
}

int msod_convec_ijk(int porder, int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp,
                    const float *He, const float *gpvol, const float *dlxigp_ip, const float *xgp,
                    const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                    const float *u, const float *q, const float *rho, const float *pr, const float *E, float *Rmass,
                    float *Rmom, float *Rener, void *stream)
{
    (void)Ngp; (void)dNgp; (void)xgp;
    if (!mode_is_default_convec())
        return mode_convec(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                           gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream);
    return convec_impl<float>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                              gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream);
}

int msod_convec_ijk_split(int porder, int nelem, int npoin, const int *connec, const float *Ngp,
                          const float *dNgp, const float *He, const float *gpvol, const float *dlxigp_ip,
                          const float *xgp, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                          const int *gmshAtoK, const float *u, const float *q, const float *rho, const float *pr,
                          const float *E, float *Rmass, float *Rmom, float *Rener, void *stream)
{
    (void)Ngp; (void)dNgp; (void)xgp;
    if (!mode_is_default_convec())
        return mode_convec(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                           gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream);
    return convec_impl<float>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                              gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream);
}

int msod_diffusion_ijk(int porder, int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp,
                       const float *He, const float *gpvol, const float *dlxigp_ip, const float *xgp,
                       const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                       float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                       const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass, float *Rmom,
                       float *Rener, void *stream)
{
    (void)Ngp; (void)dNgp; (void)xgp;
    if (!mode_is_default_diffusion())
        return mode_diffusion(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                              gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream);
    return diffu_impl<float>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                             gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream);
}

int msod_convec_diffusion_ijk(int porder, int nelem, int npoin, const int *connec, const float *Ngp,
                              const float *dNgp, const float *He, const float *gpvol, const float *dlxigp_ip,
                              const float *xgp, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                              const int *gmshAtoK, float Cp, float Pr, const float *u, const float *q,
                              const float *rho, const float *pr, const float *E, const float *Tem,
                              const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass_c,
                              float *Rmom_c, float *Rener_c, float *Rmass_d, float *Rmom_d, float *Rener_d,
                              void *stream)
{
    if (!mode_is_default_convec() || !mode_is_default_diffusion()) {
        int rc = msod_convec_ijk(porder, nelem, npoin, connec, Ngp, dNgp, He, gpvol, dlxigp_ip, xgp, invAtoIJK,
                                 gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, Rmass_c, Rmom_c, Rener_c, stream);
        if (rc) return rc;
        return msod_diffusion_ijk(porder, nelem, npoin, connec, Ngp, dNgp, He, gpvol, dlxigp_ip, xgp, invAtoIJK,
                                  gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs,
                                  Rmass_d, Rmom_d, Rener_d, stream);
    }
    (void)Ngp; (void)dNgp; (void)xgp;
    return fused_impl(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                      Cp, Pr, u, q, rho, pr, E, Tem, mu_fluid, mu_e, mu_sgs, Rmass_c, Rmom_c, Rener_c, Rmass_d,
                      Rmom_d, Rener_d, stream);
}

int msod_diffusion_ijk_nu(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                          const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                          const int *gmshAtoK, float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                          const float *mu_fluid, const float *nu_elem, const float *mu_sgs, float *Rmass, float *Rmom,
                          float *Rener, void *stream)
{
    if (!nu_elem) {
        clear_error();
        return set_error(MSOD_ERR_INVALID_ARG, "NULL nu_elem");
    }
    return diffu_impl<float>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                             gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, nullptr, mu_sgs, Rmass, Rmom, Rener, stream,
                             nu_elem);
}

int msod_convec_ijk_f64(int porder, int nelem, int npoin, const int *connec, const double *He, const double *gpvol,
                        const double *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                        const int *gmshAtoK, const double *u, const double *q, const double *rho, const double *pr,
                        const double *E, double *Rmass, double *Rmom, double *Rener, void *stream)
{
    return convec_impl<double>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                               gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, Rener, stream);
}

int msod_convec_ijk_mixed(int precision, int porder, int nelem, int npoin, const int *connec, const float *He,
                          const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                          const int *gmshAtoJ, const int *gmshAtoK, const float *u, const float *q, const float *rho,
                          const float *pr, const float *E, double *Rmass, double *Rmom, double *Rener, void *stream)
{
    clear_error();
    const int prec = precision;
    if (prec != MSOD_PREC_FP16 && prec != MSOD_PREC_BF16)
        return set_error(MSOD_ERR_INVALID_ARG, "precision %d is neither MSOD_PREC_FP16 nor MSOD_PREC_BF16", precision);
    int rc = check_geometry(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                            gmshAtoK);
    if (rc) return rc;
    if (porder > 7) return set_error(MSOD_ERR_PORDER, "the mixed-precision kernel serves porder 1..7");
    if (!u || !q || !rho || !pr || !E || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode()) {
        rc = run_check(porder, nelem, npoin, connec, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, st);
        if (rc) return rc;
    }
    TableScratch *tabs = device_tables(porder);
    if (!tabs) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    ElementArgs<float> ea;
    ea.nelem = nelem; ea.npoin = npoin; ea.connec = connec; ea.He = He; ea.gpvol = gpvol; ea.dlxigp_ip = dlxigp_ip;
    ea.invAtoIJK = invAtoIJK; ea.AtoI = gmshAtoI; ea.AtoJ = gmshAtoJ; ea.AtoK = gmshAtoK;
    MixedConvecArgs a;
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol;
    a.u = u; a.q = q; a.rho = rho; a.pr = pr; a.E = E; a.Rmass = Rmass; a.Rmom = Rmom; a.Rener = Rener;
    rc = cuda_status(launch_table_prep<float>(porder, ea, tabs, st), "table preparation launch");
    if (!rc) rc = cuda_status(launch_convec_mixed(porder, prec, a, tabs, st), "mixed convection launch");
    if (!rc && checked_mode()) rc = cuda_status(cudaStreamSynchronize(st), "mixed convection kernel");
    return rc;
}

static int diffu_mixed_impl(int precision, int porder, int nelem, int npoin, const int *connec, const float *He,
                            const float *gpvol, const float *dlx, const int *inv, const int *ai, const int *aj,
                            const int *ak, float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                            const float *mu_fluid, const float *mu_e, const float *nu_elem, const float *mu_sgs,
                            double *Rmass, double *Rmom, double *Rener, void *stream)
{
    clear_error();
    if (precision != MSOD_PREC_FP16 && precision != MSOD_PREC_BF16)
        return set_error(MSOD_ERR_INVALID_ARG, "precision %d is neither MSOD_PREC_FP16 nor MSOD_PREC_BF16", precision);
    int rc = check_geometry(porder, nelem, npoin, connec, He, gpvol, dlx, inv, ai, aj, ak);
    if (rc) return rc;
    if (porder > 7) return set_error(MSOD_ERR_PORDER, "the mixed-precision kernels serve porder 1..7");
    if (!rho || !u || !Tem || !mu_fluid || !(mu_e || nu_elem) || !mu_sgs || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    if (!(Pr != 0.0f)) return set_error(MSOD_ERR_INVALID_ARG, "Pr must be non-zero");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode()) {
        rc = run_check(porder, nelem, npoin, connec, dlx, inv, ai, aj, ak, st);
        if (rc) return rc;
    }
    TableScratch *tabs = device_tables(porder);
    if (!tabs) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    ElementArgs<float> ea;
    ea.nelem = nelem; ea.npoin = npoin; ea.connec = connec; ea.He = He; ea.gpvol = gpvol; ea.dlxigp_ip = dlx;
    ea.invAtoIJK = inv; ea.AtoI = ai; ea.AtoJ = aj; ea.AtoK = ak;
    MixedDiffuArgs a;
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol; a.Cp = Cp; a.Pr = Pr;
    a.rho = rho; a.u = u; a.Tem = Tem; a.mu_fluid = mu_fluid; a.mu_e = mu_e; a.mu_sgs = mu_sgs; a.nu_elem = nu_elem;
    a.Rmass = Rmass; a.Rmom = Rmom; a.Rener = Rener;
    rc = cuda_status(launch_table_prep<float>(porder, ea, tabs, st), "table preparation launch");
    if (!rc) rc = cuda_status(launch_diffu_mixed(porder, precision, a, tabs, st), "mixed diffusion launch");
    if (!rc && checked_mode()) rc = cuda_status(cudaStreamSynchronize(st), "mixed diffusion kernel");
    return rc;
}

int msod_diffusion_ijk_mixed(int precision, int porder, int nelem, int npoin, const int *connec, const float *He,
                             const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                             const int *gmshAtoJ, const int *gmshAtoK, float Cp, float Pr, const float *rho,
                             const float *u, const float *Tem, const float *mu_fluid, const float *mu_e,
                             const float *mu_sgs, double *Rmass, double *Rmom, double *Rener, void *stream)
{
    if (!mu_e) {
        clear_error();
        return set_error(MSOD_ERR_INVALID_ARG, "NULL mu_e");
    }
    return diffu_mixed_impl(precision, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI,
                            gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, nullptr, mu_sgs, Rmass, Rmom,
                            Rener, stream);
}

int msod_diffusion_ijk_mixed_nu(int precision, int porder, int nelem, int npoin, const int *connec, const float *He,
                                const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                                const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK, float Cp, float Pr,
                                const float *rho, const float *u, const float *Tem, const float *mu_fluid,
                                const float *nu_elem, const float *mu_sgs, double *Rmass, double *Rmom, double *Rener,
                                void *stream)
{
    if (!nu_elem) {
        clear_error();
        return set_error(MSOD_ERR_INVALID_ARG, "NULL nu_elem");
    }
    return diffu_mixed_impl(precision, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI,
                            gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, nullptr, nu_elem, mu_sgs, Rmass, Rmom,
                            Rener, stream);
}

int msod_diffusion_ijk_f64(int porder, int nelem, int npoin, const int *connec, const double *He,
                           const double *gpvol, const double *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                           const int *gmshAtoJ, const int *gmshAtoK, double Cp, double Pr, const double *rho,
                           const double *u, const double *Tem, const double *mu_fluid, const double *mu_e,
                           const double *mu_sgs, double *Rmass, double *Rmom, double *Rener, void *stream)
{
    return diffu_impl<double>(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                              gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream);
}

int msod_check_element_tables(int porder, int nelem, int npoin, const int *connec, const float *dlxigp_ip,
                              const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                              void *stream)
{
    clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER) return set_error(MSOD_ERR_PORDER, "porder %d", porder);
    if (nelem < 1 || npoin < 1 || !connec || !dlxigp_ip || !invAtoIJK || !gmshAtoI || !gmshAtoJ || !gmshAtoK)
        return set_error(MSOD_ERR_INVALID_ARG, "bad sizes or NULL table");
    return run_check(porder, nelem, npoin, connec, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                     static_cast<cudaStream_t>(stream));
}

int msod_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const float *coord, const float *dNgp,
                       const float *wgp, float *gpvol, float *He, void *stream)
{
    clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER) return set_error(MSOD_ERR_PORDER, "porder %d", porder);
    if (nelem < 1 || npoin < 1 || !connec || !coord || !dNgp || !wgp || !gpvol || !He)
        return set_error(MSOD_ERR_INVALID_ARG, "bad sizes or NULL array");
    return cuda_status(launch_elem_jacobian<float>(porder, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He,
                                                   static_cast<cudaStream_t>(stream)),
                       "elem_jacobian launch");
}

int msod_elem_jacobian_f64(int porder, int nelem, int npoin, const int *connec, const double *coord,
                           const double *dNgp, const double *wgp, double *gpvol, double *He, void *stream)
{
    clear_error();
    if (porder < 1 || porder > MSOD_MAX_PORDER) return set_error(MSOD_ERR_PORDER, "porder %d", porder);
    if (nelem < 1 || npoin < 1 || !connec || !coord || !dNgp || !wgp || !gpvol || !He)
        return set_error(MSOD_ERR_INVALID_ARG, "bad sizes or NULL array");
    return cuda_status(launch_elem_jacobian<double>(porder, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He,
                                                    static_cast<cudaStream_t>(stream)),
                       "elem_jacobian launch");
}

// ---------------------------------------------------------------------------
// Linear tetrahedra: fem_convec (elem_convec.f90:839), fem_diffu (elem_diffu.f90:199)
// ---------------------------------------------------------------------------

extern "C++" {
static int tet_ok(int nelem, int npoin, const void *connec, const void *Ngp, const void *dNgp, const void *He,
                  const void *gpvol)
{
    if (nelem < 1 || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    if ((long long)nelem * 4 >= (1LL << 31)) return set_error(MSOD_ERR_INVALID_ARG, "nelem*4 exceeds int32");
    if (!connec || !Ngp || !dNgp || !He || !gpvol) return set_error(MSOD_ERR_INVALID_ARG, "NULL element array");
    return MSOD_OK;
}

static int tet_check(int nelem, int npoin, const int *connec, cudaStream_t st)
{
    int *flags = device_flags();
    if (!flags) return set_error(MSOD_ERR_CUDA, "could not allocate the validation flag");
    int rc = cuda_status(cudaMemsetAsync(flags, 0, sizeof(int), st), "cudaMemsetAsync");
    if (!rc) rc = cuda_status(launch_check_connec(4LL * nelem, npoin, connec, flags, st), "connec check launch");
    int h = 0;
    if (!rc) rc = cuda_status(cudaMemcpyAsync(&h, flags, sizeof(int), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (!rc && h) return set_error(MSOD_ERR_BAD_TABLES, "connec has entries outside 1..npoin");
    return rc;
}

template <typename real>
static int fem_convec_impl(int nelem, int npoin, const int *connec, const real *Ngp, const real *dNgp,
                           const real *He, const real *gpvol, const real *u, const real *q, const real *rho,
                           const real *pr, const real *E, real *Rmass, real *Rmom, real *Rener, void *stream)
{
    clear_error();
    int rc = tet_ok(nelem, npoin, connec, Ngp, dNgp, He, gpvol);
    if (rc) return rc;
    if (!u || !q || !rho || !pr || !E || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode() && (rc = tet_check(nelem, npoin, connec, st))) return rc;
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    TetConvecArgs<real> a{nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E, Rmass, Rmom, Rener};
    return cuda_status(launch_fem_convec<real>(a, st), "fem_convec launch");
}

template <typename real>
static int fem_diffu_impl(int nelem, int npoin, const int *connec, const real *Ngp, const real *dNgp,
                          const real *He, const real *gpvol, real Cp, real Pr, const real *rho, const real *u,
                          const real *Tem, const real *mu_fluid, const real *mu_e, const real *mu_sgs, real *Rmass,
                          real *Rmom, real *Rener, void *stream)
{
    clear_error();
    int rc = tet_ok(nelem, npoin, connec, Ngp, dNgp, He, gpvol);
    if (rc) return rc;
    if (!rho || !u || !Tem || !mu_fluid || !mu_e || !mu_sgs || !Rmass || !Rmom || !Rener)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field or residual array");
    if (Pr == (real)0) return set_error(MSOD_ERR_INVALID_ARG, "Pr must be nonzero");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (checked_mode() && (rc = tet_check(nelem, npoin, connec, st))) return rc;
    rc = zero_outputs(Rmass, Rmom, Rener, npoin, st);
    if (rc) return rc;
    TetDiffuArgs<real> a{nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr,
                         rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener};
    return cuda_status(launch_fem_diffu<real>(a, st), "fem_diffu launch");
}

template <typename real>
static int tet_jacobian_impl(int nelem, int npoin, const int *connec, const real *coord, const real *dNgp,
                             const real *wgp, real *gpvol, real *He, void *stream)
{
    clear_error();
    if (nelem < 1 || npoin < 1 || !connec || !coord || !dNgp || !wgp || !gpvol || !He)
        return set_error(MSOD_ERR_INVALID_ARG, "bad sizes or NULL array");
    return cuda_status(launch_jacobian_nodes<real>(4, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He,
                                                   static_cast<cudaStream_t>(stream)),
                       "tet_jacobian launch");
}

}  // extern "C++"

int msod_fem_convec(int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp, const float *He,
                    const float *gpvol, const float *u, const float *q, const float *rho, const float *pr,
                    const float *E, float *Rmass, float *Rmom, float *Rener, void *stream)
{
    return fem_convec_impl<float>(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E, Rmass, Rmom, Rener,
                                  stream);
}

int msod_fem_convec_f64(int nelem, int npoin, const int *connec, const double *Ngp, const double *dNgp,
                        const double *He, const double *gpvol, const double *u, const double *q, const double *rho,
                        const double *pr, const double *E, double *Rmass, double *Rmom, double *Rener,
                        void *stream)
{
    return fem_convec_impl<double>(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E, Rmass, Rmom,
                                   Rener, stream);
}

int msod_fem_diffu(int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp, const float *He,
                   const float *gpvol, float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                   const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass, float *Rmom,
                   float *Rener, void *stream)
{
    return fem_diffu_impl<float>(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, rho, u, Tem, mu_fluid, mu_e,
                                 mu_sgs, Rmass, Rmom, Rener, stream);
}

int msod_fem_diffu_f64(int nelem, int npoin, const int *connec, const double *Ngp, const double *dNgp,
                       const double *He, const double *gpvol, double Cp, double Pr, const double *rho,
                       const double *u, const double *Tem, const double *mu_fluid, const double *mu_e,
                       const double *mu_sgs, double *Rmass, double *Rmom, double *Rener, void *stream)
{
    return fem_diffu_impl<double>(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, rho, u, Tem, mu_fluid, mu_e,
                                  mu_sgs, Rmass, Rmom, Rener, stream);
}

int msod_tet_jacobian(int nelem, int npoin, const int *connec, const float *coord, const float *dNgp,
                      const float *wgp, float *gpvol, float *He, void *stream)
{
    return tet_jacobian_impl<float>(nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, stream);
}

int msod_tet_jacobian_f64(int nelem, int npoin, const int *connec, const double *coord, const double *dNgp,
                          const double *wgp, double *gpvol, double *He, void *stream)
{
    return tet_jacobian_impl<double>(nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, stream);
}

}  // extern "C"
