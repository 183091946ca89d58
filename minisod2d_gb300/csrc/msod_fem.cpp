// msod_fem.cpp -- host-side element setup, structured mesh and field recipes.
//
// Element tables restate the reference's setup chain (main.f90:110-255):
//   GLL nodes/weights        mod_maths.f90:31-152 (ZELEGL/WELEGL/VALEPO, FP64)
//   SOD-order Lagrange basis mod_maths.f90:177-297 (computed in rp)
//   gmsh node ordering       mod_gmsh_indices.f90:11-108, elem_hex.f90:14-21, elem_qua.f90:12-17
//   gmsh->SOD relabel, maps  main.f90:131-206
//   hex quadrature           quadrature_rules.f90:50-82
// The arithmetic of every floating-point table follows the reference
// operation for operation, so an FP32 build gives the bits a Fortran caller
// passes.  The gmsh ordering is generated iteratively here (a work list of
// nested sub-cubes) instead of by recursion.
//
// The structured shared-node mesh and the seeded field recipes replace the
// reference's disconnected test mesh (mod_mesh.f90:11-65) and initial
// condition (main.f90:320-361) for the scaled workloads; mesh generation stays
// on the host.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "msod.h"
#include "msod_internal.h"

namespace {

constexpr int kMaxQ = MSOD_MAX_PORDER + 1;

// Legendre polynomial L_N and its first two derivatives (VALEPO).
void legendre(int N, double x, double &y, double &dy, double &d2y)
{
    y = 1.0; dy = 0.0; d2y = 0.0;
    if (N == 0) return;
    y = x; dy = 1.0; d2y = 0.0;
    if (N == 1) return;
    double yp = 1.0, dyp = 0.0, d2yp = 0.0;
    for (int i = 2; i <= N; ++i) {
        const double c1 = (double)i, c2 = 2.0 * c1 - 1.0, c4 = c1 - 1.0;
        const double ym = y;
        y = (c2 * x * y - c4 * yp) / c1;
        yp = ym;
        const double dym = dy;
        dy = (c2 * x * dy - c4 * dyp + c2 * yp) / c1;
        dyp = dym;
        const double d2ym = d2y;
        d2y = (c2 * x * d2y - c4 * d2yp + 2.0 * c2 * dyp) / c1;
        d2yp = d2ym;
    }
}

// GLL nodes (ascending) and weights in FP64 (ZELEGL + WELEGL).  pi_rp is the
// reference's v_pi, a real(rp) constant, used for the Newton start values.
void gll_fp64(int N, double pi_rp, double *x, double *w)
{
    double vn[kMaxQ];
    x[0] = -1.0; x[N] = 1.0;
    const int n2 = (N - 1) / 2;
    const double sn = (double)(2 * N - 4 * n2 - 3);
    vn[0] = sn; vn[N] = 1.0;
    if (N >= 2) {
        double y, dy, d2y;
        x[n2 + 1] = 0.0;
        legendre(N, 0.0, y, dy, d2y);
        vn[n2 + 1] = y;
        const double c = pi_rp / (double)N;
        for (int i = 1; i <= n2; ++i) {
            double t = std::cos(c * (double)i);
            for (int it = 0; it < 8; ++it) {
                legendre(N, t, y, dy, d2y);
                t = t - dy / d2y;
            }
            x[i] = -t; x[N - i] = t;
            vn[i] = y * sn; vn[N - i] = y;
        }
    }
    const double cw = 2.0 / ((double)N * ((double)N + 1.0));
    for (int i = 0; i <= n2; ++i) {
        const double wt = cw / (vn[i] * vn[i]);
        w[i] = wt; w[N - i] = wt;
    }
    if (N - 1 != 2 * n2) w[n2 + 1] = cw / (vn[n2 + 1] * vn[n2 + 1]);
}

// SOD 1-D order: position s (0-based) holds the natural node lorder[s].
inline int sod_to_nat(int P, int s) { return s == 0 ? 0 : (s == 1 ? P : s - 1); }

template <typename real>
void lagrange_sod(int P, const real *xi, real xp, real *l)
{
    for (int i = 0; i <= P; ++i) {
        const int li = sod_to_nat(P, i);
        l[i] = (real)1.0;
        for (int j = 0; j <= P; ++j)
            if (j != li) l[i] = l[i] * ((xp - xi[j]) / (xi[li] - xi[j]));
    }
}

template <typename real>
void lagrange_sod_deriv(int P, const real *xi, real xp, real *dl)
{
    for (int i = 0; i <= P; ++i) {
        const int li = sod_to_nat(P, i);
        dl[i] = (real)0.0;
        for (int j = 0; j <= P; ++j) {
            if (j == li) continue;
            real aux = (real)1.0;
            for (int m = 0; m <= P; ++m)
                if (m != j && m != li) aux = aux * (xp - xi[m]) / (xi[li] - xi[m]);
            dl[i] = dl[i] + ((real)1.0 / (xi[li] - xi[j])) * aux;
        }
    }
}

// gmsh high-order hex ordering (I,J,K in 0..p), generated with an explicit
// work list: each entry is a sub-cube (order q, offset o) whose corners,
// edge interiors and face interiors are emitted, after which its interior
// cube (order q-2, offset o+1) is processed next.  Face interiors are quads
// ordered the same way.
const int kHexEdges[12][2] = {{0, 1}, {0, 3}, {0, 4}, {1, 2}, {1, 5}, {2, 3},
                              {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};
const int kHexFaces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3},
                             {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
const int kQuadEdges[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};

void quad_order(int p, std::vector<int> &out /* pairs */)
{
    out.clear();
    int off = 0;
    for (int q = p; q >= 0; q -= 2, ++off) {
        const int c[4][2] = {{0, 0}, {q, 0}, {q, q}, {0, q}};
        const int ncorner = q > 0 ? 4 : 1;
        for (int a = 0; a < ncorner; ++a) { out.push_back(c[a][0] + off); out.push_back(c[a][1] + off); }
        if (q <= 1) break;
        for (int e = 0; e < 4; ++e) {
            const int *a0 = c[kQuadEdges[e][0]], *a1 = c[kQuadEdges[e][1]];
            for (int i = 1; i < q; ++i)
                for (int d = 0; d < 2; ++d) out.push_back(a0[d] + i * (a1[d] - a0[d]) / q + off);
        }
    }
}

void hex_order(int p, std::vector<int> &out /* triples */)
{
    out.clear();
    std::vector<int> face;
    int off = 0;
    for (int q = p; q >= 0; q -= 2, ++off) {
        int c[8][3];
        for (int a = 0; a < 8; ++a) {
            static const int u[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                        {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
            for (int d = 0; d < 3; ++d) c[a][d] = u[a][d] * q;
        }
        const int ncorner = q > 0 ? 8 : 1;
        for (int a = 0; a < ncorner; ++a)
            for (int d = 0; d < 3; ++d) out.push_back(c[a][d] + off);
        if (q <= 1) break;
        for (int e = 0; e < 12; ++e) {
            const int *a0 = c[kHexEdges[e][0]], *a1 = c[kHexEdges[e][1]];
            for (int i = 1; i < q; ++i)
                for (int d = 0; d < 3; ++d) out.push_back(a0[d] + i * ((a1[d] - a0[d]) / q) + off);
        }
        quad_order(q - 2, face);
        for (int f = 0; f < 6; ++f) {
            const int *a0 = c[kHexFaces[f][0]], *a1 = c[kHexFaces[f][1]], *a3 = c[kHexFaces[f][3]];
            for (size_t i = 0; i < face.size(); i += 2) {
                const int s = face[i] + 1, t = face[i + 1] + 1;
                for (int d = 0; d < 3; ++d)
                    out.push_back(a0[d] + ((a1[d] - a0[d]) / q) * s + ((a3[d] - a0[d]) / q) * t + off);
            }
        }
    }
}

template <typename real>
int element_tables(int P, int *inv, int *atoijk, int *ai, int *aj, int *ak, real *xgp, real *wgp,
                   real *Ngp, real *dNgp, real *dlx)
{
    if (P < 1 || P > MSOD_MAX_PORDER) return msod::set_error(MSOD_ERR_PORDER, "porder %d outside 1..%d", P, MSOD_MAX_PORDER);
    const int Q = P + 1, n = Q * Q * Q;
    std::vector<int> g;
    hex_order(P, g);
    if ((int)g.size() != 3 * n) return msod::set_error(MSOD_ERR_INTERNAL, "gmsh ordering size mismatch");
    // gmsh 1-D index -> SOD 1-D index: 0 -> 1, P -> 2, k -> k+2 (main.f90:133-157).
    for (int &v : g) v = (v == 0) ? 1 : (v == P ? 2 : v + 2);
    std::vector<int> lut(n, 0);
    for (int a = 0; a < n; ++a) {
        const int I = g[3 * a], J = g[3 * a + 1], K = g[3 * a + 2];
        lut[((K - 1) * Q + (J - 1)) * Q + (I - 1)] = a + 1;
        ai[a] = I; aj[a] = J; ak[a] = K;
    }
    int c = 0;
    for (int k = 0; k < Q; ++k)
        for (int i = 0; i < Q; ++i)
            for (int j = 0; j < Q; ++j) atoijk[c++] = lut[(k * Q + j) * Q + i];
    std::memcpy(inv, lut.data(), sizeof(int) * n);
    for (int a = 0; a < n; ++a)
        if (inv[a] == 0) return msod::set_error(MSOD_ERR_INTERNAL, "incomplete invAtoIJK");

    // 1-D GLL rule in rp (getGaussLobattoLegendre_weights_and_roots).
    const real pi_rp = (real)2.0 * (real)std::asin((real)1.0);
    double x64[kMaxQ], w64[kMaxQ];
    gll_fp64(P, (double)pi_rp, x64, w64);
    real xi[kMaxQ], w1[kMaxQ];
    for (int i = 0; i < Q; ++i) { xi[i] = (real)x64[i]; w1[i] = (real)w64[i]; }

    // Hex quadrature (GaussLobattoLegendre_hex): loop k, i, j over SOD positions.
    c = 0;
    for (int k = 0; k < Q; ++k)
        for (int i = 0; i < Q; ++i)
            for (int j = 0; j < Q; ++j) {
                const int a = atoijk[c++] - 1;
                xgp[0 * n + a] = xi[sod_to_nat(P, i)];
                xgp[1 * n + a] = xi[sod_to_nat(P, j)];
                xgp[2 * n + a] = xi[sod_to_nat(P, k)];
                wgp[a] = w1[sod_to_nat(P, i)] * w1[sod_to_nat(P, j)] * w1[sod_to_nat(P, k)];
            }

    // GLL-basis values and derivatives at every point (hex_highorder's second
    // TripleTensorProduct call; the equispaced copies are not part of the path).
    for (int gp = 0; gp < n; ++gp) {
        real l[3][kMaxQ], dl[3][kMaxQ];
        for (int d = 0; d < 3; ++d) {
            lagrange_sod<real>(P, xi, xgp[d * n + gp], l[d]);
            lagrange_sod_deriv<real>(P, xi, xgp[d * n + gp], dl[d]);
        }
        for (int d = 0; d < 3; ++d)
            for (int ii = 0; ii < Q; ++ii) dlx[(ii * 3 + d) * n + gp] = dl[d][ii];
        c = 0;
        for (int k = 0; k < Q; ++k)
            for (int i = 0; i < Q; ++i)
                for (int j = 0; j < Q; ++j) {
                    const int a = atoijk[c++] - 1;
                    Ngp[a * n + gp] = l[0][i] * l[1][j] * l[2][k];
                    dNgp[(gp * n + a) * 3 + 0] = dl[0][i] * l[1][j] * l[2][k];
                    dNgp[(gp * n + a) * 3 + 1] = l[0][i] * dl[1][j] * l[2][k];
                    dNgp[(gp * n + a) * 3 + 2] = l[0][i] * l[1][j] * dl[2][k];
                }
    }
    return MSOD_OK;
}

// ---------------------------------------------------------------------------
// Seeded random numbers: splitmix64 -> uniform doubles -> Box-Muller normals.
// ---------------------------------------------------------------------------
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

struct Mode {
    double k[3], phase, amp[3];
};

// nmodes Fourier modes with integer wavevectors in [-kmax, kmax]^3 (not all
// zero), uniform phases and per-component N(0, amp_sigma) amplitudes.
std::vector<Mode> make_modes(Rng &rng, int nmodes, int kmax, double amp_sigma)
{
    std::vector<Mode> m(nmodes);
    for (auto &md : m) {
        do {
            for (int d = 0; d < 3; ++d) md.k[d] = (double)((int)(rng.uniform() * (2 * kmax + 1)) - kmax);
        } while (md.k[0] == 0 && md.k[1] == 0 && md.k[2] == 0);
        md.phase = 2.0 * M_PI * rng.uniform();
        for (int d = 0; d < 3; ++d) md.amp[d] = amp_sigma * rng.normal();
    }
    return m;
}

// tet_4points (quadrature_rules.f90:84-99) and tet_04 (elem_tet.f90:9-36) at
// each point, filled as the driver fills its tet tables (main.f90:377-383):
// Ngp(igaus,inode) = N_inode(x_igaus) at Ngp[inode*4+igaus], dNgp(:,inode,igaus)
// at dNgp[(igaus*4+inode)*3+d], xgp(igaus,d) at xgp[d*4+igaus].  The two point
// coordinates round to the same FP32 value from the decimal literal directly
// or through FP64.
template <typename real>
void tet_tables(real *Ngp, real *dNgp, real *xgp, real *wgp)
{
    const real a = (real)0.5854101966249680, b = (real)0.1381966011250110;
    const real X[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
    static const int dN[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int g = 0; g < 4; ++g) {
        for (int d = 0; d < 3; ++d) xgp[d * 4 + g] = X[g][d];
        wgp[g] = (real)0.25;
        const real xi = X[g][0], eta = X[g][1], zeta = X[g][2];
        const real N[4] = {(real)1 - xi - eta - zeta, xi, eta, zeta};
        for (int k = 0; k < 4; ++k) {
            Ngp[k * 4 + g] = N[k];
            for (int d = 0; d < 3; ++d) dNgp[(g * 4 + k) * 3 + d] = (real)dN[k][d];
        }
    }
}

// gen_tet_mesh (mod_mesh.f90:71-126): connec(e,a) = (e-1)*4 + a, element e a
// copy of xyzBase (xyzBase[d*4+a]) shifted by 3.0 per element along every axis.
template <typename real>
void tet_mesh(int nelem, const real *xyzBase, int *connec, real *coord)
{
    const int64_t npoin = 4 * (int64_t)nelem;
    for (int64_t e = 0; e < nelem; ++e)
        for (int a = 0; a < 4; ++a) connec[(int64_t)a * nelem + e] = (int)(e * 4 + a + 1);
    if (!coord) return;
    real xyz0 = (real)0;
    for (int64_t e = 0; e < nelem; ++e) {
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) coord[(int64_t)d * npoin + e * 4 + a] = xyzBase[d * 4 + a] + xyz0;
        xyz0 = xyz0 + (real)3;
    }
}

}  // namespace


extern "C" {

int msod_fem_element_tables(int porder, int *invAtoIJK, int *AtoIJK, int *AtoI, int *AtoJ, int *AtoK,
                            float *xgp, float *wgp, float *Ngp, float *dNgp, float *dlxigp_ip)
{
    return element_tables<float>(porder, invAtoIJK, AtoIJK, AtoI, AtoJ, AtoK, xgp, wgp, Ngp, dNgp, dlxigp_ip);
}

int msod_fem_element_tables_f64(int porder, int *invAtoIJK, int *AtoIJK, int *AtoI, int *AtoJ, int *AtoK,
                                double *xgp, double *wgp, double *Ngp, double *dNgp, double *dlxigp_ip)
{
    return element_tables<double>(porder, invAtoIJK, AtoIJK, AtoI, AtoJ, AtoK, xgp, wgp, Ngp, dNgp, dlxigp_ip);
}

int msod_mesh_structured(int porder, int nx, int ny, int nz, const int *AtoI, const int *AtoJ, const int *AtoK,
                         double jitter, uint64_t seed, int *connec, float *coord)
{
    const int P = porder;
    if (P < 1 || P > MSOD_MAX_PORDER) return msod::set_error(MSOD_ERR_PORDER, "porder %d outside 1..%d", P, MSOD_MAX_PORDER);
    if (nx < 1 || ny < 1 || nz < 1) return msod::set_error(MSOD_ERR_INVALID_ARG, "mesh dimensions must be positive");
    if (jitter < 0.0 || jitter >= 0.25) return msod::set_error(MSOD_ERR_INVALID_ARG, "jitter must be in [0, 0.25)");
    const int Q = P + 1, n = Q * Q * Q;
    const int64_t NX = (int64_t)nx * P + 1, NY = (int64_t)ny * P + 1, NZ = (int64_t)nz * P + 1;
    const int64_t nelem = (int64_t)nx * ny * nz, npoin = NX * NY * NZ;
    if (nelem * n >= ((int64_t)1 << 31) || npoin >= ((int64_t)1 << 31))
        return msod::set_error(MSOD_ERR_INVALID_ARG, "mesh too large for int32 connectivity");
    for (int a = 0; a < n; ++a)
        if (AtoI[a] < 1 || AtoI[a] > Q || AtoJ[a] < 1 || AtoJ[a] > Q || AtoK[a] < 1 || AtoK[a] > Q)
            return msod::set_error(MSOD_ERR_INVALID_ARG, "AtoI/AtoJ/AtoK entry outside 1..porder+1");

    // Connectivity: element (ex,ey,ez) lexicographic, node (I,J,K) lexicographic.
    std::vector<int> ni(n), nj(n), nk(n);
    for (int a = 0; a < n; ++a) {
        ni[a] = sod_to_nat(P, AtoI[a] - 1);
        nj[a] = sod_to_nat(P, AtoJ[a] - 1);
        nk[a] = sod_to_nat(P, AtoK[a] - 1);
    }
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
        for (int a = 0; a < n; ++a) {
            const int64_t I = ex * P + ni[a], J = ey * P + nj[a], K = ez * P + nk[a];
            connec[(int64_t)a * nelem + e] = (int)((K * NY + J) * NX + I + 1);
        }
    }
    if (!coord) return MSOD_OK;

    // Vertex grid of the unit cube; interior vertices jittered by up to
    // +-jitter*h per component (boundary vertices stay on the cube faces).
    const int64_t VX = nx + 1, VY = ny + 1, VZ = nz + 1;
    std::vector<double> vx(VX * VY * VZ * 3);
    Rng rng(seed ^ 0x6A09E667F3BCC908ull);
    const double h[3] = {1.0 / nx, 1.0 / ny, 1.0 / nz};
    for (int64_t k = 0; k < VZ; ++k)
        for (int64_t j = 0; j < VY; ++j)
            for (int64_t i = 0; i < VX; ++i) {
                const int64_t v = (k * VY + j) * VX + i;
                const int64_t idx[3] = {i, j, k}, lim[3] = {nx, ny, nz};
                for (int d = 0; d < 3; ++d) {
                    double x = (double)idx[d] * h[d];
                    const double r = 2.0 * rng.uniform() - 1.0;  // drawn for every vertex: seed-stable
                    if (idx[d] > 0 && idx[d] < lim[d]) x += jitter * h[d] * r;
                    vx[v * 3 + d] = x;
                }
            }
    const float pi_f = 2.0f * (float)std::asin(1.0);
    double xg[kMaxQ], wg[kMaxQ];
    gll_fp64(P, (double)pi_f, xg, wg);
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < NZ; ++K) {
        for (int64_t J = 0; J < NY; ++J)
            for (int64_t I = 0; I < NX; ++I) {
                const int64_t ex = I / P < nx ? I / P : nx - 1, ey = J / P < ny ? J / P : ny - 1,
                              ez = K / P < nz ? K / P : nz - 1;
                const double s[3] = {xg[I - ex * P], xg[J - ey * P], xg[K - ez * P]};
                double x[3] = {0, 0, 0};
                for (int c = 0; c < 8; ++c) {
                    const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
                    const double wgt = 0.125 * (1 + (cx ? s[0] : -s[0])) * (1 + (cy ? s[1] : -s[1])) *
                                       (1 + (cz ? s[2] : -s[2]));
                    const int64_t v = ((ez + cz) * VY + (ey + cy)) * VX + (ex + cx);
                    for (int d = 0; d < 3; ++d) x[d] += wgt * vx[v * 3 + d];
                }
                const int64_t p = (K * NY + J) * NX + I;
                for (int d = 0; d < 3; ++d) coord[d * npoin + p] = (float)x[d];
            }
    }
    return MSOD_OK;
}

int msod_fields_recipe(int kind, int nmodes, uint64_t seed, int64_t npoin, const float *coord, float *rho,
                       float *u, float *q, float *pr, float *E, float *Tem, float *mu_fluid)
{
    if (kind != MSOD_FIELDS_SMOOTH && kind != MSOD_FIELDS_SHOCK)
        return msod::set_error(MSOD_ERR_INVALID_ARG, "unknown field recipe %d", kind);
    if (npoin < 1 || nmodes < 1 || nmodes > 64) return msod::set_error(MSOD_ERR_INVALID_ARG, "bad npoin or nmodes");
    const double gamma = 1.4, Rgas = 287.0, tpi = 2.0 * M_PI;
    const double uamp = kind == MSOD_FIELDS_SMOOTH ? 0.1 : 0.3;
    Rng rng(seed);
    std::vector<Mode> um[3];
    for (int c = 0; c < 3; ++c) um[c] = make_modes(rng, nmodes, 2, uamp);
    std::vector<Mode> noise = make_modes(rng, nmodes, 3, 1.0);
    double noise_norm = 0.0;
    for (auto &m : noise) noise_norm += std::fabs(m.amp[0]);
    if (noise_norm <= 0.0) noise_norm = 1.0;
    // Shock recipe: uniform pressure for a Mach number of 0.8 at the velocity
    // scale sqrt(3 * nmodes / 2) * uamp (the rms of the Fourier sum).
    const double urms = std::sqrt(3.0 * nmodes * 0.5) * uamp;
    const double p_shock = urms * urms / (gamma * 0.8 * 0.8);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npoin; ++p) {
        const double x = coord[p], y = coord[npoin + p], z = coord[2 * npoin + p];
        double uu[3];
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (const Mode &m : um[c]) s += m.amp[0] * std::sin(tpi * (m.k[0] * x + m.k[1] * y + m.k[2] * z) + m.phase);
            uu[c] = s;
        }
        double r, pp;
        if (kind == MSOD_FIELDS_SMOOTH) {
            r = 1.0 + 0.1 * std::sin(tpi * x) * std::sin(tpi * y) * std::sin(tpi * z);
            pp = 1.0 + 0.05 * std::cos(tpi * x);
        } else {
            double nz = 0.0;
            for (const Mode &m : noise) nz += m.amp[0] * std::sin(tpi * (m.k[0] * x + m.k[1] * y + m.k[2] * z) + m.phase);
            r = 1.0 + 0.5 * std::tanh((x - 0.5) / 0.02) + 0.05 * nz / noise_norm;
            pp = p_shock;
        }
        const float rf = (float)r, pf = (float)pp;
        float uf[3] = {(float)uu[0], (float)uu[1], (float)uu[2]};
        rho[p] = rf;
        pr[p] = pf;
        for (int c = 0; c < 3; ++c) { u[c * npoin + p] = uf[c]; q[c * npoin + p] = rf * uf[c]; }
        const float ke = 0.5f * (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]);
        E[p] = pf / (float)(gamma - 1.0) / rf + ke;
        Tem[p] = pf / (rf * (float)Rgas);
        mu_fluid[p] = 1.8e-5f;
    }
    return MSOD_OK;
}


int msod_tet_element_tables(float *Ngp, float *dNgp, float *xgp, float *wgp)
{
    if (!Ngp || !dNgp || !xgp || !wgp) return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL table");
    tet_tables<float>(Ngp, dNgp, xgp, wgp);
    return MSOD_OK;
}

int msod_tet_element_tables_f64(double *Ngp, double *dNgp, double *xgp, double *wgp)
{
    if (!Ngp || !dNgp || !xgp || !wgp) return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL table");
    tet_tables<double>(Ngp, dNgp, xgp, wgp);
    return MSOD_OK;
}

int msod_tet_mesh_disconnected(int nelem, const float *xyzBase, int *connec, float *coord)
{
    if (nelem < 1 || (int64_t)nelem * 4 >= ((int64_t)1 << 31))
        return msod::set_error(MSOD_ERR_INVALID_ARG, "nelem must be in 1..2^29-1");
    if (!connec || (coord && !xyzBase)) return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL array");
    tet_mesh<float>(nelem, xyzBase, connec, coord);
    return MSOD_OK;
}


int msod_mesh_disconnected(int porder, int nelem, const float *xyzBase, int *connec, float *coord)
{
    // create_mesh (mod_mesh.f90:11-65): connec(e,a) = (e-1) n + a; element e is
    // xyzBase(nnode,3) (xyzBase[d*n+a], the driver passes xgp) shifted by
    // 3 (e-1) along every axis.
    const int P = porder;
    if (P < 1 || P > MSOD_MAX_PORDER) return msod::set_error(MSOD_ERR_PORDER, "porder %d", P);
    const int n = (P + 1) * (P + 1) * (P + 1);
    if (nelem < 1 || (int64_t)nelem * n >= ((int64_t)1 << 31))
        return msod::set_error(MSOD_ERR_INVALID_ARG, "nelem*nnode must be in 1..2^31-1");
    if (!connec || (coord && !xyzBase)) return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL array");
    const int64_t npoin = (int64_t)nelem * n;
    for (int64_t e = 0; e < nelem; ++e)
        for (int a = 0; a < n; ++a) connec[(int64_t)a * nelem + e] = (int)(e * n + a + 1);
    if (!coord) return MSOD_OK;
    float shift = 0.0f;
    for (int64_t e = 0; e < nelem; ++e) {
        for (int a = 0; a < n; ++a)
            for (int d = 0; d < 3; ++d) coord[(int64_t)d * npoin + e * n + a] = xyzBase[d * n + a] + shift;
        shift = shift + 3.0f;
    }
    return MSOD_OK;
}

int msod_reference_ic(int porder, int nelem, int64_t npoin, const int *connec, float *u, float *q, float *rho,
                      float *pr, float *E, float *Tem, float *mu_fluid, float *mu_e, float *mu_sgs)
{
    // The driver's initial condition (main.f90:320-361): every field 1; nodes 1
    // and 4 of every element get u = 10 / 20, rho = 10 / 20, pr = 100 / 200;
    // then q = rho u, E = rho pr / ((gamma-1) rho) + q.u / 2, T = pr / (rho Rgas)
    // with gamma = 1.4, Rgas = 287 (main.f90:52), in the driver's operation order.
    const int P = porder;
    if (P < 1 || P > MSOD_MAX_PORDER) return msod::set_error(MSOD_ERR_PORDER, "porder %d", P);
    const int n = (P + 1) * (P + 1) * (P + 1);
    if (nelem < 1 || npoin < 1) return msod::set_error(MSOD_ERR_INVALID_ARG, "nelem and npoin must be positive");
    if (!connec || !u || !q || !rho || !pr || !E || !Tem || !mu_fluid || !mu_e || !mu_sgs)
        return msod::set_error(MSOD_ERR_INVALID_ARG, "NULL array");
    const float gamma = 1.4f, Rgas = 287.0f;
    for (int64_t p = 0; p < npoin; ++p) {
        for (int d = 0; d < 3; ++d) u[d * npoin + p] = 1.0f;
        rho[p] = pr[p] = E[p] = Tem[p] = mu_fluid[p] = 1.0f;
    }
    for (int64_t i = 0; i < (int64_t)nelem * n; ++i) mu_e[i] = mu_sgs[i] = 1.0f;
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t a = connec[e] - 1, b = connec[3 * (int64_t)nelem + e] - 1;  // nodes 1 and 4
        if (a < 0 || a >= npoin || b < 0 || b >= npoin)
            return msod::set_error(MSOD_ERR_INVALID_ARG, "connec entry outside 1..npoin");
        for (int d = 0; d < 3; ++d) {
            u[d * npoin + a] = 10.0f;
            u[d * npoin + b] = 20.0f;
        }
        rho[a] = 10.0f;
        rho[b] = 20.0f;
        pr[a] = 100.0f;
        pr[b] = 200.0f;
    }
    for (int64_t p = 0; p < npoin; ++p) {
        float fmag = 0.0f;
        for (int d = 0; d < 3; ++d) {
            q[d * npoin + p] = rho[p] * u[d * npoin + p];
            fmag = fmag + q[d * npoin + p] * u[d * npoin + p];
        }
        const float eint = pr[p] / ((gamma - 1.0f) * rho[p]);
        E[p] = rho[p] * eint + 0.5f * fmag;
        Tem[p] = pr[p] / (rho[p] * Rgas);
    }
    return MSOD_OK;
}

}  // extern "C"
