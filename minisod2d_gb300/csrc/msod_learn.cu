// msod_learn.cu -- C ABI of the entropy-viscosity estimator and of the learned
// per-element estimator (network training, inference, weight files) and the
// diffusion residual driven by a per-element viscosity.
//
// None of these has a counterpart in the reference, which consumes mu_e
// (elem_diffu.f90:19) without computing it; the knob defaults follow
// mod_numerical_params.f90:22-28 (ce = 0.1, cmax = 0.5, normalised entropy).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "msod.h"
#include "msod_internal.h"
#include "msod_kernels.h"

struct msod_mlp {
    int device;
    void *block;
    float *master, *m, *v, *grad;
    __half *wh;
    msod::MlpNorm *norm;
    int has_norm;
};

namespace msod {
namespace {

int cuda_rc(cudaError_t err, const char *what)
{
    if (err == cudaSuccess) return MSOD_OK;
    return set_error(MSOD_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

// Library-owned per-device scratch, grown on demand (slot-indexed).
std::mutex g_mu;
struct Slot {
    void *p = nullptr;
    size_t n = 0;
};
Slot g_slots[64][8];

void *scratch(int slot, size_t bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    Slot &s = g_slots[dev][slot];
    if (s.n < bytes) {
        if (s.p) cudaFree(s.p);
        s.p = nullptr;
        s.n = 0;
        if (cudaMalloc(&s.p, bytes) != cudaSuccess) return nullptr;
        s.n = bytes;
    }
    return s.p;
}
enum { SLOT_STATS = 0, SLOT_TABLES, SLOT_FEAT, SLOT_NUMAX, SLOT_NU, SLOT_LIST, SLOT_COUNT };

int geometry_ok(int porder, int nelem, int npoin, const void *connec, const void *He, const void *gpvol,
                const void *dlx, const void *inv, const void *ai, const void *aj, const void *ak)
{
    if (porder < 1 || porder > 7)
        return set_error(MSOD_ERR_PORDER, "porder %d outside 1..7 for the viscosity estimators", porder);
    if (nelem < 1 || npoin < 1) return set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    const long long n = (long long)(porder + 1) * (porder + 1) * (porder + 1);
    if ((long long)nelem * n >= (1LL << 31)) return set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode exceeds int32");
    if (!connec || !He || !gpvol || !dlx || !inv || !ai || !aj || !ak)
        return set_error(MSOD_ERR_INVALID_ARG, "NULL element or geometry array");
    return MSOD_OK;
}

int run_stats(int npoin, const float *rho, const float *p_or_T, float Rgas, float gamma, EntropyStats **out,
              cudaStream_t st)
{
    auto *s = static_cast<EntropyStats *>(scratch(SLOT_STATS, sizeof(EntropyStats)));
    if (!s) return set_error(MSOD_ERR_CUDA, "could not allocate the entropy statistics");
    *out = s;
    return cuda_rc(launch_entropy_stats(npoin, rho, p_or_T, Rgas, gamma, s, st), "entropy statistics launch");
}

// The call's element tables (perm, lat, derivative matrices) in the
// library-owned table area, prepared on the call's stream.
int prep_tables(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                const float *dlxigp_ip, const int *invAtoIJK, const int *AtoI, const int *AtoJ, const int *AtoK,
                TableScratch **out, cudaStream_t st)
{
    auto *area = static_cast<TableScratch *>(scratch(SLOT_TABLES, sizeof(TableScratch) * (MSOD_MAX_PORDER + 1)));
    if (!area) return set_error(MSOD_ERR_CUDA, "could not allocate the element-table area");
    TableScratch *tabs = area + porder;  // one table area per porder
    *out = tabs;
    ElementArgs<float> ea{};
    ea.nelem = nelem; ea.npoin = npoin; ea.connec = connec; ea.He = He; ea.gpvol = gpvol; ea.dlxigp_ip = dlxigp_ip;
    ea.invAtoIJK = invAtoIJK; ea.AtoI = AtoI; ea.AtoJ = AtoJ; ea.AtoK = AtoK;
    return cuda_rc(launch_table_prep<float>(porder, ea, tabs, st), "table preparation launch");
}

// The tables prepared by the last prep_tables call of this porder on this device.
const TableScratch *prepared_tables(int porder)
{
    return static_cast<TableScratch *>(scratch(SLOT_TABLES, sizeof(TableScratch) * (MSOD_MAX_PORDER + 1))) +
           porder;
}

uint32_t crc32(const unsigned char *p, size_t n)
{
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) {
        c ^= p[i];
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return ~c;
}

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace
}  // namespace msod

using namespace msod;

extern "C" {

int msod_entropy_viscosity(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                           const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                           const int *gmshAtoK, const float *rho, const float *u, const float *pr, float gamma,
                           float ce, float cmax, int normalise, float *mu_e, float *nu_elem, float *numax_elem,
                           void *stream)
{
    clear_error();
    int rc = geometry_ok(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK);
    if (rc) return rc;
    if (!rho || !u || !pr || !(mu_e || nu_elem))
        return set_error(MSOD_ERR_INVALID_ARG, "NULL field, or neither mu_e nor nu_elem");
    if (!(gamma > 1.0f)) return set_error(MSOD_ERR_INVALID_ARG, "gamma must exceed 1");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    EntropyStats *stats = nullptr;
    rc = run_stats(npoin, rho, pr, 0.0f, gamma, &stats, st);
    if (rc) return rc;
    TableScratch *tabs = nullptr;
    rc = prep_tables(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                     &tabs, st);
    if (rc) return rc;
    ViscArgs a{};
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol; a.dlxigp_ip = dlxigp_ip;
    a.invAtoIJK = invAtoIJK; a.AtoI = gmshAtoI; a.AtoJ = gmshAtoJ; a.AtoK = gmshAtoK;
    a.rho = rho; a.u = u; a.p_or_T = pr; a.Rgas = 0.0f; a.gamma = gamma; a.ce = ce; a.cmax = cmax;
    a.normalise = normalise; a.stats = stats; a.list = nullptr; a.count = nullptr; a.mu_e = mu_e; a.nu = nu_elem; a.numax = numax_elem;
    a.tabs = tabs;
    return cuda_rc(launch_entropy_visc(porder, a, st), "entropy viscosity launch");
}

// Features (and, with norm, the out-of-range flags of a trained network).
static int features_impl(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                         const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                         const int *gmshAtoK, const float *rho, const float *u, const float *p_or_T, float Rgas,
                         float gamma, float cmax, float *feat, float *numax_elem, void *stream);

int msod_mlp_features(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                      const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                      const int *gmshAtoK, const float *rho, const float *u, const float *p_or_T, float Rgas,
                      float gamma, float cmax, float *feat, float *numax_elem, void *stream)
{
    clear_error();
    return features_impl(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                         rho, u, p_or_T, Rgas, gamma, cmax, feat, numax_elem, stream);
}

static int features_impl(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                         const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                         const int *gmshAtoK, const float *rho, const float *u, const float *p_or_T, float Rgas,
                         float gamma, float cmax, float *feat, float *numax_elem, void *stream)
{
    int rc = geometry_ok(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK);
    if (rc) return rc;
    if (!rho || !u || !p_or_T || !feat) return set_error(MSOD_ERR_INVALID_ARG, "NULL field or feature array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    EntropyStats *stats = nullptr;
    rc = run_stats(npoin, rho, p_or_T, Rgas, gamma, &stats, st);
    if (rc) return rc;
    TableScratch *tabs = nullptr;
    rc = prep_tables(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                     &tabs, st);
    if (rc) return rc;
    FeatureArgs fa{};
    fa.nelem = nelem; fa.npoin = npoin; fa.connec = connec; fa.He = He; fa.gpvol = gpvol; fa.tabs = tabs;
    fa.rho = rho; fa.u = u; fa.p_or_T = p_or_T; fa.Rgas = Rgas; fa.gamma = gamma; fa.cmax = cmax; fa.stats = stats;
    fa.feat = feat; fa.numax = numax_elem;
    return cuda_rc(launch_features(porder, fa, st), "feature launch");
}

int msod_mlp_create(msod_mlp **out, uint64_t seed)
{
    clear_error();
    if (!out) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle pointer");
    *out = nullptr;
    auto *m = new msod_mlp();
    cudaGetDevice(&m->device);
    const size_t nf = (size_t)kMlpParams;
    const size_t bytes = 4 * nf * sizeof(float) + nf * sizeof(__half) + sizeof(MlpNorm) + 64;
    if (cudaMalloc(&m->block, bytes) != cudaSuccess) {
        delete m;
        return set_error(MSOD_ERR_CUDA, "could not allocate the network");
    }
    char *b = static_cast<char *>(m->block);
    m->norm = reinterpret_cast<MlpNorm *>(b);
    m->master = reinterpret_cast<float *>(b + sizeof(MlpNorm));
    m->m = m->master + nf;
    m->v = m->m + nf;
    m->grad = m->v + nf;
    m->wh = reinterpret_cast<__half *>(m->grad + nf);
    // Xavier-uniform weights, zero biases, output bias -2 (softplus(-2) = 0.13).
    std::vector<float> w(nf, 0.0f);
    Rng rng{seed ^ 0x3C6EF372FE94F82Bull};
    auto fill = [&](int off, int fan_out, int fan_in) {
        const double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int i = 0; i < fan_out * fan_in; ++i) w[off + i] = (float)((2.0 * rng.uniform() - 1.0) * a);
    };
    fill(kOffW1, kMlpH, kMlpIn);
    fill(kOffW2, kMlpH, kMlpH);
    fill(kOffW3, 1, kMlpH);
    w[kOffB3] = 5.0f;  // s = 5 decades: y = 1e-5 before training
    MlpNorm nm;
    for (int k = 0; k < kMlpIn; ++k) { nm.mean[k] = 0.f; nm.inv_std[k] = 1.f; nm.fmin[k] = -3e38f; nm.fmax[k] = 3e38f; }
    int rc = cuda_rc(cudaMemcpy(m->master, w.data(), nf * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!rc) rc = cuda_rc(cudaMemcpy(m->norm, &nm, sizeof nm, cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!rc) rc = cuda_rc(cudaMemset(m->m, 0, 3 * nf * sizeof(float)), "cudaMemset");
    if (!rc) rc = cuda_rc(launch_mlp_to_half(m->master, m->wh, 0), "to-half launch");
    if (!rc) rc = cuda_rc(cudaDeviceSynchronize(), "network initialisation");
    if (rc) {
        cudaFree(m->block);
        delete m;
        return rc;
    }
    *out = m;
    return MSOD_OK;
}

int msod_mlp_destroy(msod_mlp *m)
{
    if (!m) return MSOD_OK;
    cudaFree(m->block);
    delete m;
    return MSOD_OK;
}

int msod_mlp_train(msod_mlp *m, const float *feat, const float *target, const float *weight, int nsamples, int steps,
                   int batch, float lr, uint64_t seed, float *loss_host, void *stream)
{
    clear_error();
    if (!m || !feat || !target) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle or training data");
    if (nsamples < 2 || steps < 1 || batch < 1 || !(lr > 0.0f))
        return set_error(MSOD_ERR_INVALID_ARG, "bad training sizes");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *loss = nullptr;
    if (cudaMalloc(&loss, sizeof(float) * steps) != cudaSuccess)
        return set_error(MSOD_ERR_CUDA, "could not allocate the loss history");
    int rc = cuda_rc(cudaMemsetAsync(loss, 0, sizeof(float) * steps, st), "cudaMemsetAsync");
    if (!rc) rc = cuda_rc(cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, st), "cudaMemsetAsync");
    if (!rc) rc = cuda_rc(launch_mlp_norm(nsamples, feat, m->norm, st), "normalisation launch");
    for (int t = 1; t <= steps && !rc; ++t) {
        rc = cuda_rc(launch_mlp_grad(nsamples, feat, target, weight, nullptr, batch, (uint32_t)seed, t, m->master, m->norm,
                                     m->grad, loss + (t - 1), st),
                     "gradient launch");
        if (!rc) rc = cuda_rc(launch_mlp_adam(m->master, m->m, m->v, m->grad, m->wh, lr, t, st), "Adam launch");
    }
    if (!rc && loss_host)
        rc = cuda_rc(cudaMemcpyAsync(loss_host, loss, sizeof(float) * steps, cudaMemcpyDeviceToHost, st), "loss copy");
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(st), "training");
    cudaFree(loss);
    if (!rc) m->has_norm = 1;
    return rc;
}

int msod_mlp_gradient(msod_mlp *m, const float *feat, const float *target, const float *weight, const int *idx,
                      int batch, float *grad_host, void *stream)
{
    clear_error();
    if (!m || !feat || !target || !idx || !grad_host || batch < 1)
        return set_error(MSOD_ERR_INVALID_ARG, "bad gradient arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = cuda_rc(cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, st), "cudaMemsetAsync");
    if (!rc)
        rc = cuda_rc(launch_mlp_grad(1, feat, target, weight, idx, batch, 0u, 0, m->master, m->norm, m->grad, nullptr,
                                     st),
                     "gradient launch");
    if (!rc)
        rc = cuda_rc(cudaMemcpyAsync(grad_host, m->grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st),
                     "gradient copy");
    if (!rc) rc = cuda_rc(cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, st), "cudaMemsetAsync");
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(st), "gradient");
    return rc;
}

int msod_mlp_get_params(const msod_mlp *m, float *params, float *norm)
{
    clear_error();
    if (!m) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle");
    int rc = MSOD_OK;
    if (params) rc = cuda_rc(cudaMemcpy(params, m->master, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost), "copy");
    if (!rc && norm) rc = cuda_rc(cudaMemcpy(norm, m->norm, sizeof(MlpNorm), cudaMemcpyDeviceToHost), "copy");
    return rc;
}

int msod_mlp_set_params(msod_mlp *m, const float *params, const float *norm)
{
    clear_error();
    if (!m) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle");
    int rc = MSOD_OK;
    if (params) {
        rc = cuda_rc(cudaMemcpy(m->master, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice), "copy");
        if (!rc) rc = cuda_rc(launch_mlp_to_half(m->master, m->wh, 0), "to-half launch");
        if (!rc) rc = cuda_rc(cudaDeviceSynchronize(), "set params");
    }
    if (!rc && norm) {
        rc = cuda_rc(cudaMemcpy(m->norm, norm, sizeof(MlpNorm), cudaMemcpyHostToDevice), "copy");
        m->has_norm = 1;
    }
    return rc;
}

int msod_mlp_predict(const msod_mlp *m, const float *feat, const float *numax_elem, int nelem, float *y,
                     float *nu_elem, int *flag, void *stream)
{
    clear_error();
    if (!m || !feat || nelem < 1 || !y) return set_error(MSOD_ERR_INVALID_ARG, "bad prediction arguments");
    if (nu_elem && !numax_elem) return set_error(MSOD_ERR_INVALID_ARG, "nu needs numax");
    return cuda_rc(launch_mlp_predict(nelem, feat, m->wh, m->norm, numax_elem, y, nu_elem, flag, nullptr, nullptr,
                                      static_cast<cudaStream_t>(stream)),
                   "prediction launch");
}

// Weight file: "MSODMLP1", int32 version, n_in, n_hidden, n_params, the 48
// normalisation floats (mean, 1/std, min, max), the FP16 weights, CRC-32 of
// everything before it.
int msod_mlp_save(const msod_mlp *m, const char *path)
{
    clear_error();
    if (!m || !path) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle or path");
    std::vector<unsigned char> buf;
    auto put = [&](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        buf.insert(buf.end(), c, c + n);
    };
    put("MSODMLP1", 8);
    const int32_t hdr[4] = {1, kMlpIn, kMlpH, kMlpParams};
    put(hdr, sizeof hdr);
    MlpNorm nm;
    std::vector<__half> wh(kMlpParams);
    int rc = cuda_rc(cudaMemcpy(&nm, m->norm, sizeof nm, cudaMemcpyDeviceToHost), "copy");
    if (!rc) rc = cuda_rc(cudaMemcpy(wh.data(), m->wh, sizeof(__half) * kMlpParams, cudaMemcpyDeviceToHost), "copy");
    if (rc) return rc;
    put(&nm, sizeof nm);
    put(wh.data(), sizeof(__half) * kMlpParams);
    const uint32_t c = crc32(buf.data(), buf.size());
    put(&c, sizeof c);
    FILE *f = fopen(path, "wb");
    if (!f) return set_error(MSOD_ERR_INVALID_ARG, "cannot open %s for writing", path);
    const size_t nw = fwrite(buf.data(), 1, buf.size(), f);
    fclose(f);
    if (nw != buf.size()) return set_error(MSOD_ERR_INVALID_ARG, "short write to %s", path);
    return MSOD_OK;
}

int msod_mlp_load(msod_mlp *m, const char *path)
{
    clear_error();
    if (!m || !path) return set_error(MSOD_ERR_INVALID_ARG, "NULL handle or path");
    FILE *f = fopen(path, "rb");
    if (!f) return set_error(MSOD_ERR_INVALID_ARG, "cannot open %s", path);
    std::vector<unsigned char> buf;
    unsigned char tmp[4096];
    size_t n;
    while ((n = fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + n);
    fclose(f);
    const size_t want = 8 + 16 + sizeof(MlpNorm) + sizeof(__half) * kMlpParams + 4;
    if (buf.size() != want || memcmp(buf.data(), "MSODMLP1", 8) != 0)
        return set_error(MSOD_ERR_BAD_MODEL, "%s is not a weight file of this network", path);
    int32_t hdr[4];
    memcpy(hdr, buf.data() + 8, sizeof hdr);
    if (hdr[0] != 1 || hdr[1] != kMlpIn || hdr[2] != kMlpH || hdr[3] != kMlpParams)
        return set_error(MSOD_ERR_BAD_MODEL, "%s has another network shape", path);
    uint32_t c;
    memcpy(&c, buf.data() + want - 4, 4);
    if (c != crc32(buf.data(), want - 4)) return set_error(MSOD_ERR_BAD_MODEL, "%s fails its CRC check", path);
    MlpNorm nm;
    memcpy(&nm, buf.data() + 24, sizeof nm);
    std::vector<__half> wh(kMlpParams);
    memcpy(wh.data(), buf.data() + 24 + sizeof nm, sizeof(__half) * kMlpParams);
    std::vector<float> w(kMlpParams);
    for (int i = 0; i < kMlpParams; ++i) w[i] = __half2float(wh[i]);
    int rc = cuda_rc(cudaMemcpy(m->norm, &nm, sizeof nm, cudaMemcpyHostToDevice), "copy");
    if (!rc) rc = cuda_rc(cudaMemcpy(m->master, w.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice), "copy");
    if (!rc) rc = cuda_rc(cudaMemcpy(m->wh, wh.data(), sizeof(__half) * kMlpParams, cudaMemcpyHostToDevice), "copy");
    if (!rc) m->has_norm = 1;
    return rc;
}

// The learned viscosity into nu (nelem): the features kernel, then the
// prediction kernel (nu = 10^-s nu_max, the trusted-range flags, and the
// flagged elements as a compacted list), then the plain estimator over that
// list only, overwriting nu there -- its work follows the number of flagged
// elements (a shock band spread over many element groups would otherwise cost
// most of a full estimator pass).
static int learned_nu(const msod_mlp *m, int porder, int nelem, int npoin, const int *connec, const float *He,
                      const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                      const int *gmshAtoJ, const int *gmshAtoK, const float *rho, const float *u, const float *p_or_T,
                      float Rgas, float gamma, float ce, float cmax, float *nu, int *flag, void *stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *feat = static_cast<float *>(scratch(SLOT_FEAT, sizeof(float) * kMlpIn * (size_t)nelem));
    float *numax = static_cast<float *>(scratch(SLOT_NUMAX, sizeof(float) * (size_t)nelem));
    int *list = static_cast<int *>(scratch(SLOT_LIST, sizeof(int) * (size_t)nelem));
    int *count = static_cast<int *>(scratch(SLOT_COUNT, sizeof(int)));
    if (!feat || !numax || !list || !count) return set_error(MSOD_ERR_CUDA, "could not allocate per-element scratch");
    int rc = features_impl(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                           gmshAtoK, rho, u, p_or_T, Rgas, gamma, cmax, feat, numax, stream);
    if (rc) return rc;
    rc = cuda_rc(launch_mlp_predict(nelem, feat, m->wh, m->norm, numax, nullptr, nu, flag, list, count, st),
                 "prediction launch");
    if (rc) return rc;
    EntropyStats *stats = static_cast<EntropyStats *>(scratch(SLOT_STATS, sizeof(EntropyStats)));
    ViscArgs a{};
    a.nelem = nelem; a.npoin = npoin; a.connec = connec; a.He = He; a.gpvol = gpvol; a.dlxigp_ip = dlxigp_ip;
    a.invAtoIJK = invAtoIJK; a.AtoI = gmshAtoI; a.AtoJ = gmshAtoJ; a.AtoK = gmshAtoK;
    a.rho = rho; a.u = u; a.p_or_T = p_or_T; a.Rgas = Rgas; a.gamma = gamma; a.ce = ce; a.cmax = cmax;
    a.normalise = 1; a.stats = stats; a.list = list; a.count = count; a.mu_e = nullptr; a.nu = nu; a.numax = nullptr;
    a.tabs = prepared_tables(porder);  // prepared by the feature call above
    return cuda_rc(launch_entropy_visc(porder, a, st), "fallback estimator launch");
}

int msod_learned_viscosity(const msod_mlp *m, int porder, int nelem, int npoin, const int *connec, const float *He,
                           const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                           const int *gmshAtoJ, const int *gmshAtoK, const float *rho, const float *u,
                           const float *p_or_T, float Rgas, float gamma, float ce, float cmax, float *nu_elem,
                           int *flag, void *stream)
{
    clear_error();
    if (!m) return set_error(MSOD_ERR_INVALID_ARG, "NULL network");
    int rc = geometry_ok(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK);
    if (rc) return rc;
    if (!rho || !u || !p_or_T || !nu_elem) return set_error(MSOD_ERR_INVALID_ARG, "NULL field or nu");
    return learned_nu(m, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK,
                      rho, u, p_or_T, Rgas, gamma, ce, cmax, nu_elem, flag, stream);
}

int msod_diffusion_ijk_learned(const msod_mlp *m, int porder, int nelem, int npoin, const int *connec,
                               const float *He, const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                               const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK, float Cp, float Pr,
                               const float *rho, const float *u, const float *Tem, const float *mu_fluid,
                               const float *mu_sgs, const float *p_or_T, float Rgas, float gamma, float ce,
                               float cmax, float *Rmass, float *Rmom, float *Rener, float *nu_elem, int *flag,
                               void *stream)
{
    clear_error();
    if (!m) return set_error(MSOD_ERR_INVALID_ARG, "NULL network");
    if (!m->has_norm) return set_error(MSOD_ERR_BAD_MODEL, "the network has no training ranges (train or load it)");
    int rc = geometry_ok(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK);
    if (rc) return rc;
    if (!rho || !u || !Tem || !p_or_T) return set_error(MSOD_ERR_INVALID_ARG, "NULL field");
    float *nu = nu_elem ? nu_elem : static_cast<float *>(scratch(SLOT_NU, sizeof(float) * (size_t)nelem));
    if (!nu) return set_error(MSOD_ERR_CUDA, "could not allocate the per-element viscosity");
    rc = learned_nu(m, porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, rho,
                    u, p_or_T, Rgas, gamma, ce, cmax, nu, flag, stream);
    if (rc) return rc;
    return msod_diffusion_ijk_nu(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ,
                                 gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, nu, mu_sgs, Rmass, Rmom, Rener, stream);
}

}  // extern "C"
