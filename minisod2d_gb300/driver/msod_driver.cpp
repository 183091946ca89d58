// msod_driver.cpp -- the miniSOD2D benchmark driver (src/app/sources/main.f90)
// on libmsod's C ABI.
//
// What main.f90 does, in order: element tables (main.f90:110-255), mesh
// (create_mesh, :131-196), metric on the device (elem_jacobian, :275-290),
// initial condition (:320-361), the TET04 data (:365-407), then nruns timed
// calls of the five kernels it times -- full_convec_ijk, full_convec_ijk_split,
// fem_convec, full_diffusion_ijk, fem_diffu (:444-496) -- with one line per
// run in timers.dat, the timing summary and the "Basic results" extrema on
// stdout (:501-583) and, with --debug, results_convec.dat / results_diffu.dat
// (:586-599).  Every call is timed as the reference times its synchronous
// OpenACC regions: wall clock around the call and a stream synchronisation;
// CUDA events recorded on the stream around the same call time it on the
// device (timers_events.dat, same columns and format).  A JSON summary
// (results.json) adds both averages and the throughput of the hex pair.
//
//   msod_driver [--porder 4] [--nelem 192000] [--nruns 100]
//               [--mesh disconnected|structured --nx N --jitter J]
//               [--fields reference|smooth|shock --seed S] [--device D]
//               [--precision fp32|fp16|bf16] [--mu-e given|plain|learned]
//               [--weights FILE] [--fp64-check]
//               [--out DIR] [--debug] [--format-check]
//
// --precision and --mu-e choose the form of the two hex calls through
// msod_set_mode: the FP32 kernels or the FP16 / BF16 tensor-core kernels, and
// the caller's mu_e, the plain entropy-viscosity estimator or the learned one
// (the network in --weights, with the estimator as per-element fallback).
// --fp64-check then runs the FP64 build of the hex calls on the same inputs
// promoted to FP64 (with the plain estimator's mu_e when the viscosity is
// estimated) and prints and records the relative L2 distance of every
// residual.
//
// Defaults are the reference's compile-time parameters (mod_constants.f90:16,
// main.f90:21-22).  The tet kernels use npoin_t = 4 floor(npoin/4) nodes (the
// reference requires npoin divisible by 4 and stops otherwise, main.f90:367-372).
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "msod.h"

namespace {

struct Options {
    int porder = 4, nelem = 4 * 48000, nruns = 100, nx = 16, device = 0;
    double jitter = 0.0;
    uint64_t seed = 0;
    std::string mesh = "disconnected", fields = "reference", out = ".";
    std::string precision = "fp32", mu_e = "given", weights;
    bool debug = false, format_check = false, fp64_check = false;
};

[[noreturn]] void die(const char *what, int rc)
{
    std::fprintf(stderr, "msod_driver: %s failed (%d): %s\n", what, rc, msod_last_error_string());
    std::exit(1);
}

void check(int rc, const char *what)
{
    if (rc != MSOD_OK) die(what, rc);
}

// Fortran E editing with a three-digit exponent, as gfortran's list-directed
// output prints REAL(8) values: mantissa d.dddd, exponent E+ddd.
std::string fortran_e(double v, int digits)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*E", digits, v);
    std::string s(buf);
    const size_t e = s.find('E');
    if (e == std::string::npos) return s;  // inf / nan
    const int ex = std::atoi(s.c_str() + e + 1);
    char tail[16];
    std::snprintf(tail, sizeof tail, "E%c%03d", ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    return s.substr(0, e) + tail;
}

// One timers.dat line: format (i3,1x,4(f16.8,1x)) of main.f90:499-500.
std::string timers_line(int i, const double (&t)[4])
{
    char buf[128];
    int n = i >= 0 && i <= 999 ? std::snprintf(buf, sizeof buf, "%3d ", i) : std::snprintf(buf, sizeof buf, "*** ");
    for (int k = 0; k < 4; ++k) {
        char f[32];
        std::snprintf(f, sizeof f, "%16.8f", t[k]);
        if (std::strlen(f) > 16) std::snprintf(f, sizeof f, "****************");
        n += std::snprintf(buf + n, sizeof buf - n, "%s ", f);
    }
    return std::string(buf, n);
}

// One results_*.dat line (list-directed: ipoin, R1..R5): the integer in 12
// columns, each value in 17 (one blank, a sign column, 1PE editing with 8
// fractional digits).
std::string results_line(long long ipoin, const float (&v)[5])
{
    std::string s;
    char buf[64];
    std::snprintf(buf, sizeof buf, "%12lld", ipoin);
    s += buf;
    for (int k = 0; k < 5; ++k) {
        std::snprintf(buf, sizeof buf, "%17.8E", (double)v[k]);
        s += buf;
    }
    return s;
}

Options parse(int argc, char **argv)
{
    Options o;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto val = [&](const char *name) -> const char * {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "msod_driver: %s needs a value\n", name);
                std::exit(2);
            }
            return argv[++i];
        };
        if (a == "--porder") o.porder = std::atoi(val("--porder"));
        else if (a == "--nelem") o.nelem = std::atoi(val("--nelem"));
        else if (a == "--nruns") o.nruns = std::atoi(val("--nruns"));
        else if (a == "--mesh") o.mesh = val("--mesh");
        else if (a == "--nx") o.nx = std::atoi(val("--nx"));
        else if (a == "--jitter") o.jitter = std::atof(val("--jitter"));
        else if (a == "--fields") o.fields = val("--fields");
        else if (a == "--seed") o.seed = std::strtoull(val("--seed"), nullptr, 10);
        else if (a == "--device") o.device = std::atoi(val("--device"));
        else if (a == "--out") o.out = val("--out");
        else if (a == "--precision") o.precision = val("--precision");
        else if (a == "--mu-e") o.mu_e = val("--mu-e");
        else if (a == "--weights") o.weights = val("--weights");
        else if (a == "--fp64-check") o.fp64_check = true;
        else if (a == "--debug") o.debug = true;
        else if (a == "--format-check") o.format_check = true;
        else {
            std::fprintf(stderr, "msod_driver: unknown option %s\n", a.c_str());
            std::exit(2);
        }
    }
    if (o.porder < 1 || o.porder > MSOD_MAX_PORDER || o.nruns < 1 || o.nelem < 1 || o.nx < 1 ||
        (o.mesh != "disconnected" && o.mesh != "structured") ||
        (o.fields != "reference" && o.fields != "smooth" && o.fields != "shock") ||
        (o.precision != "fp32" && o.precision != "fp16" && o.precision != "bf16") ||
        (o.mu_e != "given" && o.mu_e != "plain" && o.mu_e != "learned") || (o.mu_e == "learned" && o.weights.empty())) {
        std::fprintf(stderr, "msod_driver: bad option value\n");
        std::exit(2);
    }
    return o;
}

void cuda_check(cudaError_t err, const char *what)
{
    if (err != cudaSuccess) {
        std::fprintf(stderr, "msod_driver: %s failed: %s\n", what, cudaGetErrorString(err));
        std::exit(1);
    }
}

// Relative L2 distance of an FP32 result from its FP64 reference.
double rel_l2(const std::vector<float> &a, const std::vector<double> &b)
{
    double num = 0.0, den = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const double d = (double)a[i] - b[i];
        num += d * d;
        den += b[i] * b[i];
    }
    return den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
}

template <typename T>
std::vector<double> widen(const std::vector<T> &v)
{
    return std::vector<double>(v.begin(), v.end());
}

// Device copy of a host array.
template <typename T>
T *upload(const std::vector<T> &h)
{
    void *d = nullptr;
    check(msod_malloc(&d, h.size() * sizeof(T)), "msod_malloc");
    check(msod_h2d(d, h.data(), h.size() * sizeof(T), nullptr), "msod_h2d");
    return static_cast<T *>(d);
}

template <typename T>
T *device_array(size_t n)
{
    void *d = nullptr;
    check(msod_malloc(&d, n * sizeof(T)), "msod_malloc");
    return static_cast<T *>(d);
}

template <typename T = float>
std::vector<T> download(const T *d, size_t n)
{
    std::vector<T> h(n);
    check(msod_d2h(h.data(), d, n * sizeof(T), nullptr), "msod_d2h");
    check(msod_stream_synchronize(nullptr), "msod_stream_synchronize");
    return h;
}

struct Stats {
    double sum = 0.0, mx = 0.0, mn = 1.0e6;  // main.f90:428-442
    void add(double t)
    {
        sum += t;
        mx = std::max(mx, t);
        mn = std::min(mn, t);
    }
};

void extrema(const char *label, const std::vector<float> &v, size_t off, size_t n)
{
    float mx = -INFINITY, mn = INFINITY;
    for (size_t i = 0; i < n; ++i) {
        mx = std::max(mx, v[off + i]);
        mn = std::min(mn, v[off + i]);
    }
    std::printf(" Max %-9s = %s Min %-9s = %s\n", label, fortran_e(mx, 8).c_str(), label, fortran_e(mn, 8).c_str());
}

void print_results(const char *title, const char *M, const char *E, const std::vector<float> &m,
                   const std::vector<float> &mom, const std::vector<float> &e, size_t np)
{
    std::printf(" %s\n", title);
    char lab[32];
    extrema(M, m, 0, np);
    for (int c = 0; c < 3; ++c) {
        std::snprintf(lab, sizeof lab, "%s(:,%d)", M[0] == 'R' ? "Rmom" : "Dmom", c + 1);
        extrema(lab, mom, c * np, np);
    }
    extrema(E, e, 0, np);
    std::printf(" ----------------------------------------\n");
}

}  // namespace

int main(int argc, char **argv)
{
    const Options o = parse(argc, argv);
    if (o.format_check) {  // the file formats, without a GPU
        const double t[4] = {1.0689999999999999e-4, 12.5, 0.0, 123456.78901234};
        std::printf("%s\n%s\n%s\n", timers_line(7, t).c_str(), timers_line(1000, t).c_str(),
                    fortran_e(1.0689999999999999e-4, 16).c_str());
        const float v[5] = {1.0f, -2.5e-3f, 0.0f, 3.0e7f, -1.0f};
        std::printf("%s\n", results_line(42, v).c_str());
        return 0;
    }
    check(msod_init(o.device), "msod_init");
    const int P = o.porder, Q = P + 1, n = Q * Q * Q;

    // Element tables (main.f90:110-255).
    std::vector<int> inv(n), atoijk(n), AI(n), AJ(n), AK(n);
    std::vector<float> xgp(3 * n), wgp(n), Ngp((size_t)n * n), dNgp(3 * (size_t)n * n), dlx(3 * (size_t)n * Q);
    check(msod_fem_element_tables(P, inv.data(), atoijk.data(), AI.data(), AJ.data(), AK.data(), xgp.data(),
                                  wgp.data(), Ngp.data(), dNgp.data(), dlx.data()),
          "msod_fem_element_tables");

    // Mesh.
    int nelem = o.nelem;
    int64_t npoin64;
    std::vector<int> connec;
    std::vector<float> coord;
    if (o.mesh == "disconnected") {
        npoin64 = (int64_t)nelem * n;
        connec.resize((size_t)nelem * n);
        coord.resize(3 * (size_t)npoin64);
        check(msod_mesh_disconnected(P, nelem, xgp.data(), connec.data(), coord.data()), "msod_mesh_disconnected");
    } else {
        nelem = o.nx * o.nx * o.nx;
        const int64_t m = (int64_t)o.nx * P + 1;
        npoin64 = m * m * m;
        connec.resize((size_t)nelem * n);
        coord.resize(3 * (size_t)npoin64);
        check(msod_mesh_structured(P, o.nx, o.nx, o.nx, AI.data(), AJ.data(), AK.data(), o.jitter, o.seed,
                                   connec.data(), coord.data()),
              "msod_mesh_structured");
    }
    if (npoin64 >= ((int64_t)1 << 31)) {
        std::fprintf(stderr, "msod_driver: npoin exceeds int32\n");
        return 1;
    }
    const int npoin = (int)npoin64;
    const size_t np = (size_t)npoin, ne = (size_t)nelem * n;

    // Fields (main.f90:320-361, or a seeded recipe), mu_e = mu_sgs = 1.
    std::vector<float> u(3 * np), q(3 * np), rho(np), pr(np), E(np), Tem(np), muf(np), mue(ne, 1.0f), mus(ne, 1.0f);
    if (o.fields == "reference")
        check(msod_reference_ic(P, nelem, npoin, connec.data(), u.data(), q.data(), rho.data(), pr.data(), E.data(),
                                Tem.data(), muf.data(), mue.data(), mus.data()),
              "msod_reference_ic");
    else
        check(msod_fields_recipe(o.fields == "smooth" ? MSOD_FIELDS_SMOOTH : MSOD_FIELDS_SHOCK, 8, o.seed, npoin,
                                 coord.data(), rho.data(), u.data(), q.data(), pr.data(), E.data(), Tem.data(),
                                 muf.data()),
              "msod_fields_recipe");

    // Device arrays and the metric (elem_jacobian on the device).
    int *d_connec = upload(connec), *d_inv = upload(inv), *d_AI = upload(AI), *d_AJ = upload(AJ), *d_AK = upload(AK);
    float *d_coord = upload(coord), *d_dNgp = upload(dNgp), *d_wgp = upload(wgp), *d_dlx = upload(dlx);
    float *d_He = device_array<float>(9 * ne), *d_gpvol = device_array<float>(ne);
    check(msod_elem_jacobian(P, nelem, npoin, d_connec, d_coord, d_dNgp, d_wgp, d_gpvol, d_He, nullptr),
          "msod_elem_jacobian");
    msod_free(d_coord);
    float *d_u = upload(u), *d_q = upload(q), *d_rho = upload(rho), *d_pr = upload(pr), *d_E = upload(E);
    float *d_Tem = upload(Tem), *d_muf = upload(muf), *d_mue = upload(mue), *d_mus = upload(mus);

    // TET04 data (main.f90:365-407): the driver's disconnected unit tets over the same nodes.
    const int npoin_t = (npoin / 4) * 4, nelem_t = npoin_t / 4;
    std::vector<float> tN(16), tdN(48), txgp(12), twgp(4);
    check(msod_tet_element_tables(tN.data(), tdN.data(), txgp.data(), twgp.data()), "msod_tet_element_tables");
    const float xyzTET[12] = {0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // xyzTET(4,3), main.f90:390-393
    std::vector<int> connec_t(4 * (size_t)nelem_t);
    std::vector<float> coord_t(3 * (size_t)npoin_t);
    check(msod_tet_mesh_disconnected(nelem_t, xyzTET, connec_t.data(), coord_t.data()), "msod_tet_mesh_disconnected");
    int *d_connec_t = upload(connec_t);
    float *d_coord_t = upload(coord_t), *d_tN = upload(tN), *d_tdN = upload(tdN), *d_twgp = upload(twgp);
    float *d_He_t = device_array<float>(36 * (size_t)nelem_t), *d_gpvol_t = device_array<float>(4 * (size_t)nelem_t);
    check(msod_tet_jacobian(nelem_t, npoin_t, d_connec_t, d_coord_t, d_tdN, d_twgp, d_gpvol_t, d_He_t, nullptr),
          "msod_tet_jacobian");
    msod_free(d_coord_t);
    const std::vector<float> ones_t(4 * (size_t)nelem_t, 1.0f);
    float *d_mue_t = upload(ones_t), *d_mus_t = upload(ones_t);

    // The form of the two hex calls (msod_set_mode).
    const int prec = o.precision == "fp16" ? MSOD_PREC_FP16 : (o.precision == "bf16" ? MSOD_PREC_BF16 : MSOD_PREC_FP32);
    const int mue_mode = o.mu_e == "plain" ? MSOD_MU_E_PLAIN : (o.mu_e == "learned" ? MSOD_MU_E_LEARNED : MSOD_MU_E_GIVEN);
    msod_mlp *mlp = nullptr;
    if (mue_mode == MSOD_MU_E_LEARNED) {
        check(msod_mlp_create(&mlp, 0), "msod_mlp_create");
        check(msod_mlp_load(mlp, o.weights.c_str()), "msod_mlp_load");
    }
    check(msod_set_mode(prec, mue_mode, mlp), "msod_set_mode");

    // Residual arrays.
    auto res = [&](size_t m) { return device_array<float>(m); };
    float *Rm = res(np), *Rq = res(3 * np), *Re = res(np), *Rms = res(np), *Rqs = res(3 * np), *Res = res(np);
    float *Rmt = res(npoin_t), *Rqt = res(3 * (size_t)npoin_t), *Ret = res(npoin_t);
    float *Dm = res(np), *Dq = res(3 * np), *De = res(np);
    float *Dmt = res(npoin_t), *Dqt = res(3 * (size_t)npoin_t), *Det = res(npoin_t);
    const float Cp = 1.0f, Pra = 1.0f;  // main.f90:412-413

    // Wall clock around the call and a stream synchronisation (the reference's
    // MPI_Wtime pair around a synchronous region), and CUDA events recorded on
    // the stream around the same call (device time, seconds, in *ev).
    cudaEvent_t ev0, ev1;
    cuda_check(cudaEventCreate(&ev0), "cudaEventCreate");
    cuda_check(cudaEventCreate(&ev1), "cudaEventCreate");
    auto timed = [&](double *ev, auto &&call) {
        const auto t0 = std::chrono::steady_clock::now();
        cuda_check(cudaEventRecord(ev0, nullptr), "cudaEventRecord");
        call();
        cuda_check(cudaEventRecord(ev1, nullptr), "cudaEventRecord");
        check(msod_stream_synchronize(nullptr), "msod_stream_synchronize");
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        float ms = 0.0f;
        cuda_check(cudaEventElapsedTime(&ms, ev0, ev1), "cudaEventElapsedTime");
        *ev = 1e-3 * (double)ms;
        return wall;
    };

    const std::string timers_path = o.out + "/timers.dat";
    FILE *tf = std::fopen(timers_path.c_str(), "w");
    if (!tf) {
        std::fprintf(stderr, "msod_driver: cannot open %s: %s\n", timers_path.c_str(), std::strerror(errno));
        return 1;
    }
    const std::string events_path = o.out + "/timers_events.dat";
    FILE *ef = std::fopen(events_path.c_str(), "w");
    if (!ef) {
        std::fprintf(stderr, "msod_driver: cannot open %s: %s\n", events_path.c_str(), std::strerror(errno));
        return 1;
    }
    Stats sc, ss, st, sd, sdt, ec, es, et, ed, edt;
    for (int i = 1; i <= o.nruns; ++i) {
        double xc, xs, xt, xd, xdt;
        const double tc = timed(&xc, [&] {
            check(msod_convec_ijk(P, nelem, npoin, d_connec, nullptr, nullptr, d_He, d_gpvol, d_dlx, nullptr, d_inv,
                                  d_AI, d_AJ, d_AK, d_u, d_q, d_rho, d_pr, d_E, Rm, Rq, Re, nullptr),
                  "msod_convec_ijk");
        });
        const double ts = timed(&xs, [&] {
            check(msod_convec_ijk_split(P, nelem, npoin, d_connec, nullptr, nullptr, d_He, d_gpvol, d_dlx, nullptr,
                                        d_inv, d_AI, d_AJ, d_AK, d_u, d_q, d_rho, d_pr, d_E, Rms, Rqs, Res, nullptr),
                  "msod_convec_ijk_split");
        });
        const double tt = timed(&xt, [&] {
            check(msod_fem_convec(nelem_t, npoin_t, d_connec_t, d_tN, d_tdN, d_He_t, d_gpvol_t, d_u, d_q, d_rho,
                                  d_pr, d_E, Rmt, Rqt, Ret, nullptr),
                  "msod_fem_convec");
        });
        const double td = timed(&xd, [&] {
            check(msod_diffusion_ijk(P, nelem, npoin, d_connec, nullptr, nullptr, d_He, d_gpvol, d_dlx, nullptr,
                                     d_inv, d_AI, d_AJ, d_AK, Cp, Pra, d_rho, d_u, d_Tem, d_muf, d_mue, d_mus, Dm,
                                     Dq, De, nullptr),
                  "msod_diffusion_ijk");
        });
        const double tdt = timed(&xdt, [&] {
            check(msod_fem_diffu(nelem_t, npoin_t, d_connec_t, d_tN, d_tdN, d_He_t, d_gpvol_t, Cp, Pra, d_rho, d_u,
                                 d_Tem, d_muf, d_mue_t, d_mus_t, Dmt, Dqt, Det, nullptr),
                  "msod_fem_diffu");
        });
        sc.add(tc);
        ss.add(ts);
        st.add(tt);
        sd.add(td);
        sdt.add(tdt);
        ec.add(xc);
        es.add(xs);
        et.add(xt);
        ed.add(xd);
        edt.add(xdt);
        const double row[4] = {tc, tt, td, tdt};
        std::fprintf(tf, "%s\n", timers_line(i, row).c_str());
        const double erow[4] = {xc, xt, xd, xdt};
        std::fprintf(ef, "%s\n", timers_line(i, erow).c_str());
    }
    std::fclose(tf);
    std::fclose(ef);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);

    // Timing summary (main.f90:501-537).
    const double nr = (double)o.nruns;
    const double ac = sc.sum / nr, as = ss.sum / nr, at = st.sum / nr, ad = sd.sum / nr, adt = sdt.sum / nr;
    auto line = [](const char *label, double v) { std::printf(" %s%s\n", label, fortran_e(v, 16).c_str()); };
    std::printf("\n Timings:\n ----------------------------------------\n");
    line("Avg. convective time     = ", ac);
    line("Avg. split convective time = ", as);
    line("Avg. TET convective time = ", at);
    line("Avg. diffusive time      = ", ad);
    line("Avg. TET diffusive time  = ", adt);
    line("Max. convective time     = ", sc.mx);
    line("Max. split convective time = ", ss.mx);
    line("Max. TET convective time = ", st.mx);
    line("Max. diffusive time      = ", sd.mx);
    line("Max. TET diffusive time  = ", sdt.mx);
    line("Min. convective time     = ", sc.mn);
    line("Min. split convective time     = ", ss.mn);
    line("Min. TET convective time = ", st.mn);
    line("Min. diffusive time      = ", sd.mn);
    line("Min. TET diffusive time  = ", sdt.mn);
    std::printf(" ----------------------------------------\n");
    line("Variation convec.        = ", (sc.mx - sc.mn) / ac);
    line("Variation split convec.  = ", (ss.mx - ss.mn) / as);
    line("Variation TET convec.    = ", (st.mx - st.mn) / at);
    line("Variation diffu.         = ", (sd.mx - sd.mn) / ad);
    line("Variation TET diffu.     = ", (sdt.mx - sdt.mn) / adt);
    std::printf(" ----------------------------------------\n");

    // Basic results (main.f90:539-583).
    const auto hRm = download(Rm, np), hRq = download(Rq, 3 * np), hRe = download(Re, np);
    const auto hRms = download(Rms, np), hRqs = download(Rqs, 3 * np), hRes = download(Res, np);
    const auto hDm = download(Dm, np), hDq = download(Dq, 3 * np), hDe = download(De, np);
    const size_t npt = (size_t)npoin_t;
    const auto hRmt = download(Rmt, npt), hRqt = download(Rqt, 3 * npt), hRet = download(Ret, npt);
    const auto hDmt = download(Dmt, npt), hDqt = download(Dqt, 3 * npt), hDet = download(Det, npt);
    std::printf("\n Basic results:\n ----------------------------------------\n");
    print_results("--| Convec", "Rmass", "Rener", hRm, hRq, hRe, np);
    print_results("--| Convec_split", "Rmass", "Rener", hRms, hRqs, hRes, np);
    print_results("--| Diffu", "Dmass", "Dener", hDm, hDq, hDe, np);
    std::printf(" Basic TET results:\n ----------------------------------------\n");
    print_results("--| Convec", "Rmass", "Rener", hRmt, hRqt, hRet, npt);
    print_results("--| Diffu", "Dmass", "Dener", hDmt, hDqt, hDet, npt);

    // Results files (main.f90:586-599, written there under __DEBUG__).
    if (o.debug) {
        const char *names[2] = {"results_convec.dat", "results_diffu.dat"};
        const std::vector<float> *sets[2][3] = {{&hRm, &hRq, &hRe}, {&hDm, &hDq, &hDe}};
        for (int k = 0; k < 2; ++k) {
            const std::string path = o.out + "/" + names[k];
            FILE *f = std::fopen(path.c_str(), "w");
            if (!f) {
                std::fprintf(stderr, "msod_driver: cannot open %s\n", path.c_str());
                return 1;
            }
            for (size_t p = 0; p < np; ++p) {
                const float v[5] = {(*sets[k][0])[p], (*sets[k][1])[p], (*sets[k][1])[np + p],
                                    (*sets[k][1])[2 * np + p], (*sets[k][2])[p]};
                std::fprintf(f, "%s\n", results_line((long long)p + 1, v).c_str());
            }
            std::fclose(f);
        }
    }

    // FP64 check: the FP64 build of the hex calls, with the element tables in
    // FP64 (as the reference's FP64 build computes them) and the same fields,
    // He and gpvol promoted to FP64 (mu_e: the caller's, or the plain
    // estimator's when it is estimated).
    double fe[6] = {0, 0, 0, 0, 0, 0};
    if (o.fp64_check) {
        auto up64 = [&](const std::vector<double> &h) { return upload(h); };
        const std::vector<double> He64 = widen(download(d_He, 9 * ne)), gp64 = widen(download(d_gpvol, ne));
        std::vector<int> i64(n), a64(n), b64(n), c64(n), k64(n);
        std::vector<double> x64(3 * n), w64(n), N64((size_t)n * n), dN64(3 * (size_t)n * n), dlx64(3 * (size_t)n * Q);
        check(msod_fem_element_tables_f64(P, i64.data(), k64.data(), a64.data(), b64.data(), c64.data(), x64.data(),
                                          w64.data(), N64.data(), dN64.data(), dlx64.data()),
              "msod_fem_element_tables_f64");
        double *e_He = up64(He64), *e_gp = up64(gp64), *e_dlx = up64(dlx64);
        double *e_u = up64(widen(u)), *e_q = up64(widen(q)), *e_rho = up64(widen(rho)), *e_pr = up64(widen(pr));
        double *e_E = up64(widen(E)), *e_Tem = up64(widen(Tem)), *e_muf = up64(widen(muf)), *e_mus = up64(widen(mus));
        std::vector<double> mue64;
        if (mue_mode == MSOD_MU_E_GIVEN) {
            mue64 = widen(mue);
        } else {
            // The plain estimator on the pressure the estimated modes use, p = rho Rgas Tem
            // (main.f90:52: Rgas = 287, gamma = 1.4; ce = 0.1, cmax = 0.5).
            std::vector<float> ph(np);
            for (size_t i = 0; i < np; ++i) ph[i] = rho[i] * 287.0f * Tem[i];
            float *d_p = upload(ph), *mu_p = device_array<float>(ne);
            check(msod_entropy_viscosity(P, nelem, npoin, d_connec, d_He, d_gpvol, d_dlx, d_inv, d_AI, d_AJ, d_AK, d_rho,
                                         d_u, d_p, 1.4f, 0.1f, 0.5f, 1, mu_p, nullptr, nullptr, nullptr),
                  "msod_entropy_viscosity");
            mue64 = widen(download(mu_p, ne));
            msod_free(mu_p);
            msod_free(d_p);
        }
        double *e_mue = up64(mue64);
        double *c_m = device_array<double>(np), *c_q = device_array<double>(3 * np), *c_e = device_array<double>(np);
        double *f_m = device_array<double>(np), *f_q = device_array<double>(3 * np), *f_e = device_array<double>(np);
        check(msod_convec_ijk_f64(P, nelem, npoin, d_connec, e_He, e_gp, e_dlx, d_inv, d_AI, d_AJ, d_AK, e_u, e_q,
                                  e_rho, e_pr, e_E, c_m, c_q, c_e, nullptr),
              "msod_convec_ijk_f64");
        check(msod_diffusion_ijk_f64(P, nelem, npoin, d_connec, e_He, e_gp, e_dlx, d_inv, d_AI, d_AJ, d_AK, 1.0, 1.0,
                                     e_rho, e_u, e_Tem, e_muf, e_mue, e_mus, f_m, f_q, f_e, nullptr),
              "msod_diffusion_ijk_f64");
        fe[0] = rel_l2(hRm, download(c_m, np));
        fe[1] = rel_l2(hRq, download(c_q, 3 * np));
        fe[2] = rel_l2(hRe, download(c_e, np));
        fe[3] = rel_l2(hDm, download(f_m, np));
        fe[4] = rel_l2(hDq, download(f_q, 3 * np));
        fe[5] = rel_l2(hDe, download(f_e, np));
        for (void *ptr : {(void *)e_He, (void *)e_gp, (void *)e_dlx, (void *)e_u, (void *)e_q, (void *)e_rho,
                          (void *)e_pr, (void *)e_E, (void *)e_Tem, (void *)e_muf, (void *)e_mus, (void *)e_mue,
                          (void *)c_m, (void *)c_q, (void *)c_e, (void *)f_m, (void *)f_q, (void *)f_e})
            msod_free(ptr);
        std::printf(" FP64 check (%s, mu_e %s; relative L2 against the FP64 build on the same inputs):\n",
                    o.precision.c_str(), o.mu_e.c_str());
        std::printf(" Convec Rmass %s Rmom %s Rener %s\n", fortran_e(fe[0], 4).c_str(), fortran_e(fe[1], 4).c_str(),
                    fortran_e(fe[2], 4).c_str());
        std::printf(" Diffu  Dmass %s Dmom %s Dener %s\n", fortran_e(fe[3], 4).c_str(), fortran_e(fe[4], 4).c_str(),
                    fortran_e(fe[5], 4).c_str());
        std::printf(" ----------------------------------------\n");
    }

    // JSON summary.
    const std::string jpath = o.out + "/results.json";
    if (FILE *j = std::fopen(jpath.c_str(), "w")) {
        std::fprintf(j,
                     "{\"porder\": %d, \"nelem\": %d, \"npoin\": %d, \"nelem_tet\": %d, \"npoin_tet\": %d, "
                     "\"mesh\": \"%s\", \"fields\": \"%s\", \"nruns\": %d, "
                     "\"avg_s\": {\"convec\": %.9e, \"convec_split\": %.9e, \"convec_tet\": %.9e, "
                     "\"diffu\": %.9e, \"diffu_tet\": %.9e}, "
                     "\"avg_event_s\": {\"convec\": %.9e, \"convec_split\": %.9e, \"convec_tet\": %.9e, "
                     "\"diffu\": %.9e, \"diffu_tet\": %.9e}, "
                     "\"hex_gdofs\": %.6f, \"hex_gdofs_event\": %.6f, \"precision\": \"%s\", \"mu_e\": \"%s\", "
                     "\"fp64_check\": %s, "
                     "\"timing\": \"avg_s: wall clock around each call and a stream synchronisation; avg_event_s: CUDA "
                     "events on the stream around the same call\"}\n",
                     P, nelem, npoin, nelem_t, npoin_t, o.mesh.c_str(), o.fields.c_str(), o.nruns, ac, as, at, ad, adt,
                     ec.sum / nr, es.sum / nr, et.sum / nr, ed.sum / nr, edt.sum / nr, 5.0 * npoin / (ac + ad) / 1e9,
                     5.0 * npoin / ((ec.sum + ed.sum) / nr) / 1e9, o.precision.c_str(), o.mu_e.c_str(),
                     o.fp64_check ? "true" : "false");
        std::fclose(j);
    }
    if (o.fp64_check) {
        const std::string fpath = o.out + "/fp64_check.json";
        if (FILE *j = std::fopen(fpath.c_str(), "w")) {
            std::fprintf(j,
                         "{\"precision\": \"%s\", \"mu_e\": \"%s\", \"Rmass\": %.6e, \"Rmom\": %.6e, "
                         "\"Rener\": %.6e, \"Dmass\": %.6e, \"Dmom\": %.6e, \"Dener\": %.6e}\n",
                         o.precision.c_str(), o.mu_e.c_str(), fe[0], fe[1], fe[2], fe[3], fe[4], fe[5]);
            std::fclose(j);
        }
    }
    msod_set_mode(MSOD_PREC_FP32, MSOD_MU_E_GIVEN, nullptr);
    if (mlp) msod_mlp_destroy(mlp);
    msod_finalize();
    return 0;
}
