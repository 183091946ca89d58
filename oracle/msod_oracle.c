/*
 * msod_oracle.c -- CPU restatement of miniSOD2D's hex spectral-element hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load
 * it, and only as the checker or as the timed CPU baseline.  The product
 * library (minisod2d_gb300/csrc) never links or calls it.
 *
 * Parity status: the reference is Fortran 90 + OpenACC and no Fortran
 * compiler exists on either machine this project runs on, so the oracle is
 * NOT pinned against outputs of the reference binary.  It is pinned by
 * analytical known-answer tests (GLL nodes/weights, derivative-matrix
 * identities, index-map structure, Jacobian of affine maps, exact residuals
 * of polynomial fields on affine meshes) and cross-checked against a second,
 * independently structured numpy restatement (tests/test_oracle_*.py).
 *
 * Every routine follows the reference loop for loop, with Fortran's
 * left-to-right evaluation of products and sums.  Build with
 * -ffp-contract=off so that no fused multiply-add changes the rounding
 * (the same bits on x86-64 and aarch64).  The file is compiled twice:
 * -DORC_REAL=float -DORC_SFX=_f32 (rp=4, mod_constants.f90:5) and
 * -DORC_REAL=double -DORC_SFX=_f64 (rp=8).
 *
 * Array layouts are the reference's Fortran column-major layouts restated as
 * 0-based C index formulas (E = nelem, n = (P+1)^3, Q = P+1):
 *   connec(nelem,nnode)           connec[a*E+e]            (1-based values)
 *   He(ndime,ndime,ngaus,nelem)   He[((e*n+g)*3+j)*3+i]
 *   gpvol(1,ngaus,nelem)          gpvol[e*n+g]
 *   dlxigp_ip(ngaus,ndime,Q)      dlxigp_ip[(ii*3+d)*n+g]
 *   invAtoIJK(Q,Q,Q)              invAtoIJK[(k*Q+j)*Q+i]    (1-based values)
 *   AtoI/AtoJ/AtoK(nnode)         AtoI[a]                   (1-based values)
 *   u(npoin,ndime)                u[c*npoin+p]
 *   mu_e(nelem,ngaus)             mu_e[g*E+e]
 *   Ngp(ngaus,nnode)              Ngp[a*n+g]
 *   dNgp(ndime,nnode,ngaus)       dNgp[(g*n+a)*3+d]
 *   xgp(ngaus,ndime)              xgp[d*n+g]
 *   coord(npoin,ndime)            coord[d*npoin+p]
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORC_REAL
#define ORC_REAL float
#define ORC_SFX _f32
#endif

typedef ORC_REAL real;

#ifndef ORC_IS_FLOAT
#define ORC_IS_FLOAT 0
#endif

#define ORC_CAT2(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define F(name) ORC_CAT(name, ORC_SFX)

#define ORC_MAXP 8
#define ORC_MAXQ (ORC_MAXP + 1)
#define ORC_MAXN (ORC_MAXQ * ORC_MAXQ * ORC_MAXQ)

/* ------------------------------------------------------------------------- */
/* Quadrature: mod_maths.f90:46-152, quadrature_rules.f90:50-82              */
/* ------------------------------------------------------------------------- */

/* VALEPO, mod_maths.f90:113-152: Legendre polynomial of degree N and its
 * first two derivatives at X by the three-term recurrence (FP64). */
static void valepo(int N, double X, double *Y, double *DY, double *D2Y)
{
    *Y = 1.0; *DY = 0.0; *D2Y = 0.0;
    if (N == 0) return;
    *Y = X; *DY = 1.0; *D2Y = 0.0;
    if (N == 1) return;
    double YP = 1.0, DYP = 0.0, D2YP = 0.0;
    for (int I = 2; I <= N; ++I) {
        double C1 = (double)I;
        double C2 = 2.0 * C1 - 1.0;
        double C4 = C1 - 1.0;
        double YM = *Y;
        *Y = (C2 * X * (*Y) - C4 * YP) / C1;
        YP = YM;
        double DYM = *DY;
        *DY = (C2 * X * (*DY) - C4 * DYP + C2 * YP) / C1;
        DYP = DYM;
        double D2YM = *D2Y;
        *D2Y = (C2 * X * (*D2Y) - C4 * D2YP + 2.0 * C2 * DYP) / C1;
        D2YP = D2YM;
    }
}

/* ZELEGL, mod_maths.f90:46-82: GLL nodes ET(0:N) by 8 fixed Newton steps on
 * L_N' starting from cos(pi*I/N); VN = L_N at the nodes.  v_pi is a real(rp)
 * constant (mod_constants.f90:24), so its precision follows rp. */
void F(orc_zelegl)(int N, double *ET, double *VN)
{
    if (N == 0) return;
    int N2 = (N - 1) / 2;
    double SN = (double)(2 * N - 4 * N2 - 3);
    ET[0] = -1.0; ET[N] = 1.0;
    VN[0] = SN;  VN[N] = 1.0;
    if (N == 1) return;
    ET[N2 + 1] = 0.0;
    double Y, DY, D2Y;
    valepo(N, 0.0, &Y, &DY, &D2Y);
    VN[N2 + 1] = Y;
    if (N == 2) return;
    real v_pi = (real)2.0 * (real)asin((real)1.0);
    double C = (double)v_pi / (double)N;
    for (int I = 1; I <= N2; ++I) {
        double ETX = cos(C * (double)I);
        for (int IT = 1; IT <= 8; ++IT) {
            valepo(N, ETX, &Y, &DY, &D2Y);
            ETX = ETX - DY / D2Y;
        }
        ET[I] = -ETX;
        ET[N - I] = ETX;
        VN[I] = Y * SN;
        VN[N - I] = Y;
    }
}

/* WELEGL, mod_maths.f90:84-111: GLL weights 2/(N(N+1) L_N(x_i)^2). */
void F(orc_welegl)(int N, const double *ET, const double *VN, double *WT)
{
    (void)ET;
    if (N == 0) return;
    int N2 = (N - 1) / 2;
    double DN = (double)N;
    double C = 2.0 / (DN * (DN + 1.0));
    for (int I = 0; I <= N2; ++I) {
        double Y = VN[I];
        double WTX = C / (Y * Y);
        WT[I] = WTX;
        WT[N - I] = WTX;
    }
    if (N - 1 == 2 * N2) return;
    double Y = VN[N2 + 1];
    WT[N2 + 1] = C / (Y * Y);
}

/* getGaussLobattoLegendre_weights_and_roots, mod_maths.f90:31-42. */
void F(orc_gll_weights_and_roots)(int P, real *weights, real *roots)
{
    double r[ORC_MAXQ], v[ORC_MAXQ], w[ORC_MAXQ];
    F(orc_zelegl)(P, r, v);
    F(orc_welegl)(P, r, v, w);
    for (int i = 0; i <= P; ++i) { roots[i] = (real)r[i]; weights[i] = (real)w[i]; }
}

/* getGaussLobattoLegendre_roots, mod_maths.f90:18-27. */
static void gll_roots(int P, real *roots)
{
    double r[ORC_MAXQ], v[ORC_MAXQ];
    F(orc_zelegl)(P, r, v);
    for (int i = 0; i <= P; ++i) roots[i] = (real)r[i];
}

/* getEquispaced_roots, mod_maths.f90:154-175 (the grid of hex_highorder's
 * equispaced basis, elem_hex.f90:39-42; kept for the basis tests). */
void F(orc_equispaced_roots)(int P, real *xi)
{
    for (int i = 1; i <= P + 1; ++i)
        xi[i - 1] = (real)-1.0 + ((real)2.0 * (real)(i - 1) / (real)P);
}

/* "SOD 1-D order" of the Lagrange nodes: lorder = [1, P+1, 2, ..., P]
 * (mod_maths.f90:199-203, quadrature_rules.f90:65-69). 1-based. */
static void sod_lorder(int P, int *lorder)
{
    lorder[0] = 1;
    lorder[1] = P + 1;
    for (int i = 3; i <= P + 1; ++i) lorder[i - 1] = i - 1;
}

/* eval_lagrangePoly, mod_maths.f90:177-213 (computed in rp). */
void F(orc_eval_lagrange_poly)(int P, const real *xi, real xp, real *l_ip)
{
    int lorder[ORC_MAXQ];
    sod_lorder(P, lorder);
    for (int i = 0; i <= P; ++i) {
        l_ip[i] = (real)1.0;
        for (int j = 0; j <= P; ++j) {
            if (j != lorder[i] - 1)
                l_ip[i] = l_ip[i] * ((xp - xi[j]) / (xi[lorder[i] - 1] - xi[j]));
        }
    }
}

/* eval_lagrangePolyDeriv, mod_maths.f90:215-257 (computed in rp). */
void F(orc_eval_lagrange_poly_deriv)(int P, const real *xi, real xp, real *dl_ip)
{
    int lorder[ORC_MAXQ];
    sod_lorder(P, lorder);
    for (int i = 0; i <= P; ++i) {
        dl_ip[i] = (real)0.0;
        for (int j = 0; j <= P; ++j) {
            real aux = (real)1.0;
            if (j != lorder[i] - 1) {
                for (int m = 0; m <= P; ++m) {
                    if (m != j && m != lorder[i] - 1)
                        aux = aux * (xp - xi[m]) / (xi[lorder[i] - 1] - xi[m]);
                }
                dl_ip[i] = dl_ip[i] + ((real)1.0 / (xi[lorder[i] - 1] - xi[j])) * aux;
            }
        }
    }
}

/* TripleTensorProduct, mod_maths.f90:259-297.  N[n], dN[a*3+d] (= dN(d,a)),
 * dlx[d*Q+ii] (= dlxigp_ip(d,ii) of the caller's igaus slice) or NULL. */
static void triple_tensor_product(int P, int n, const real *xi_grid, real s, real t, real z,
                                  const int *atoIJK, real *N, real *dN, real *dlx)
{
    real lxi[ORC_MAXQ], leta[ORC_MAXQ], lzeta[ORC_MAXQ];
    real dlxi[ORC_MAXQ], dleta[ORC_MAXQ], dlzeta[ORC_MAXQ];
    int Q = P + 1;
    (void)n;
    F(orc_eval_lagrange_poly)(P, xi_grid, s, lxi);
    F(orc_eval_lagrange_poly)(P, xi_grid, t, leta);
    F(orc_eval_lagrange_poly)(P, xi_grid, z, lzeta);
    F(orc_eval_lagrange_poly_deriv)(P, xi_grid, s, dlxi);
    F(orc_eval_lagrange_poly_deriv)(P, xi_grid, t, dleta);
    F(orc_eval_lagrange_poly_deriv)(P, xi_grid, z, dlzeta);
    if (dlx) {
        for (int ii = 0; ii < Q; ++ii) {
            dlx[0 * Q + ii] = dlxi[ii];
            dlx[1 * Q + ii] = dleta[ii];
            dlx[2 * Q + ii] = dlzeta[ii];
        }
    }
    int c = 0;
    for (int k = 0; k < Q; ++k)
        for (int i = 0; i < Q; ++i)
            for (int j = 0; j < Q; ++j) {
                int a = atoIJK[c] - 1;
                ++c;
                N[a] = lxi[i] * leta[j] * lzeta[k];
                dN[a * 3 + 0] = dlxi[i] * leta[j] * lzeta[k];
                dN[a * 3 + 1] = lxi[i] * dleta[j] * lzeta[k];
                dN[a * 3 + 2] = lxi[i] * leta[j] * dlzeta[k];
            }
}

/* ------------------------------------------------------------------------- */
/* Element index tables: mod_gmsh_indices.f90:11-108, elem_hex.f90:14-21,    */
/* elem_qua.f90:12-17, main.f90:131-206                                      */
/* ------------------------------------------------------------------------- */

static const int hex_order_edges[12][2] = {
    {1, 2}, {1, 4}, {1, 5}, {2, 3}, {2, 6}, {3, 4}, {3, 7}, {4, 8}, {5, 6}, {5, 8}, {6, 7}, {7, 8}};
static const int hex_order_faces[6][4] = {
    {1, 4, 3, 2}, {1, 2, 6, 5}, {1, 5, 8, 4}, {2, 3, 7, 6}, {3, 4, 8, 7}, {5, 6, 7, 8}};
static const int quad_order_edges[4][2] = {{1, 2}, {2, 3}, {3, 4}, {4, 1}};

/* genHighOrderQuad, mod_gmsh_indices.f90:66-94.  table[(node)*2 + c]. */
static void gen_high_order_quad(int p, int *table)
{
    table[0] = 0; table[1] = 0;
    if (p <= 0) return;
    table[2] = p; table[3] = 0;
    table[4] = p; table[5] = p;
    table[6] = 0; table[7] = p;
    if (p <= 1) return;
    int inode = 5;
    for (int iedge = 0; iedge < 4; ++iedge) {
        int i0 = quad_order_edges[iedge][0] - 1, i1 = quad_order_edges[iedge][1] - 1;
        int u[2];
        for (int c = 0; c < 2; ++c) u[c] = (table[i1 * 2 + c] - table[i0 * 2 + c]) / p;
        for (int i = 1; i <= p - 1; ++i) {
            for (int c = 0; c < 2; ++c) table[(inode - 1) * 2 + c] = table[i0 * 2 + c] + i * u[c];
            ++inode;
        }
    }
    int nf = (p - 1) * (p - 1);
    int *face = (int *)malloc(sizeof(int) * 2 * (nf > 0 ? nf : 1));
    gen_high_order_quad(p - 2, face);
    for (int i = 0; i < nf; ++i)
        for (int c = 0; c < 2; ++c) table[(inode - 1 + i) * 2 + c] = face[i * 2 + c] + 1;
    free(face);
}

/* genHighOrderHex, mod_gmsh_indices.f90:11-64.  table[(node)*3 + c] = I,J,K
 * in gmsh's 0..p numbering. */
void F(orc_gen_high_order_hex)(int p, int *table)
{
    table[0] = 0; table[1] = 0; table[2] = 0;
    if (p <= 0) return;
    static const int corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    for (int a = 1; a < 8; ++a)
        for (int c = 0; c < 3; ++c) table[a * 3 + c] = corner[a][c] * p;
    if (p <= 1) return;
    int inode = 9;
    for (int iedge = 0; iedge < 12; ++iedge) {
        int i0 = hex_order_edges[iedge][0] - 1, i1 = hex_order_edges[iedge][1] - 1;
        int u[3];
        for (int c = 0; c < 3; ++c) u[c] = (table[i1 * 3 + c] - table[i0 * 3 + c]) / p;
        for (int i = 1; i <= p - 1; ++i) {
            for (int c = 0; c < 3; ++c) table[(inode - 1) * 3 + c] = table[i0 * 3 + c] + i * u[c];
            ++inode;
        }
    }
    int nf = (p - 1) * (p - 1);
    int *face = (int *)malloc(sizeof(int) * 2 * nf);
    gen_high_order_quad(p - 2, face);
    for (int i = 0; i < nf * 2; ++i) face[i] += 1;
    for (int iface = 0; iface < 6; ++iface) {
        int i0 = hex_order_faces[iface][0] - 1, i1 = hex_order_faces[iface][1] - 1;
        int i3 = hex_order_faces[iface][3] - 1;
        int u[3], v[3];
        for (int c = 0; c < 3; ++c) {
            u[c] = (table[i1 * 3 + c] - table[i0 * 3 + c]) / p;
            v[c] = (table[i3 * 3 + c] - table[i0 * 3 + c]) / p;
        }
        for (int i = 0; i < nf; ++i) {
            for (int c = 0; c < 3; ++c)
                table[(inode - 1) * 3 + c] = table[i0 * 3 + c] + u[c] * face[i * 2 + 0] + v[c] * face[i * 2 + 1];
            ++inode;
        }
    }
    free(face);
    int nv = (p - 1) * (p - 1) * (p - 1);
    int *vol = (int *)malloc(sizeof(int) * 3 * nv);
    F(orc_gen_high_order_hex)(p - 2, vol);
    for (int i = 0; i < nv; ++i)
        for (int c = 0; c < 3; ++c) table[(inode - 1 + i) * 3 + c] = vol[i * 3 + c] + 1;
    free(vol);
}

/* main.f90:131-206: relabel gmsh 1-D indices to SOD order (0->1, p->2,
 * k->k+1), then build invAtoIJK (loop k,i,j), AtoIJK and AtoI/J/K.
 * Returns 0 on success, -1 if some (i,j,k) has no node. */
int F(orc_element_maps)(int P, int *invAtoIJK, int *AtoIJK, int *AtoI, int *AtoJ, int *AtoK)
{
    int Q = P + 1, n = Q * Q * Q;
    int *g = (int *)malloc(sizeof(int) * 3 * n);
    F(orc_gen_high_order_hex)(P, g);
    int g2s[ORC_MAXQ][2];
    g2s[0][0] = 0; g2s[0][1] = 1;
    g2s[1][0] = P; g2s[1][1] = 2;
    for (int inode = 3; inode <= P + 1; ++inode) { g2s[inode - 1][0] = inode - 2; g2s[inode - 1][1] = inode; }
    for (int a = 0; a < n; ++a)
        for (int c = 0; c < 3; ++c)
            for (int io = 0; io < Q; ++io)
                if (g[a * 3 + c] == g2s[io][0]) { g[a * 3 + c] = g2s[io][1]; break; }
    int jnode = 0, rc = 0;
    for (int k = 1; k <= Q; ++k)
        for (int i = 1; i <= Q; ++i)
            for (int j = 1; j <= Q; ++j) {
                int found = 0;
                for (int a = 0; a < n; ++a)
                    if (g[a * 3 + 0] == i && g[a * 3 + 1] == j && g[a * 3 + 2] == k) { found = a + 1; break; }
                if (!found) rc = -1;
                invAtoIJK[((k - 1) * Q + (j - 1)) * Q + (i - 1)] = found;
                AtoIJK[jnode++] = found;
            }
    for (int a = 0; a < n; ++a) { AtoI[a] = g[a * 3 + 0]; AtoJ[a] = g[a * 3 + 1]; AtoK[a] = g[a * 3 + 2]; }
    free(g);
    return rc;
}

/* GaussLobattoLegendre_hex, quadrature_rules.f90:50-82. */
void F(orc_gll_hex)(int P, const int *AtoIJK, real *xgp, real *wgp)
{
    int Q = P + 1, n = Q * Q * Q;
    real xi[ORC_MAXQ], w1d[ORC_MAXQ];
    int lorder[ORC_MAXQ];
    F(orc_gll_weights_and_roots)(P, w1d, xi);
    sod_lorder(P, lorder);
    int inode = 0;
    for (int k = 0; k < Q; ++k)
        for (int i = 0; i < Q; ++i)
            for (int j = 0; j < Q; ++j) {
                int a = AtoIJK[inode++] - 1;
                xgp[0 * n + a] = xi[lorder[i] - 1];
                xgp[1 * n + a] = xi[lorder[j] - 1];
                xgp[2 * n + a] = xi[lorder[k] - 1];
                wgp[a] = w1d[lorder[i] - 1] * w1d[lorder[j] - 1] * w1d[lorder[k] - 1];
            }
}

/* main.f90:237-241 -> hex_highorder (elem_hex.f90:23-45): for every point
 * igaus the GLL-basis N, dN and the per-point derivative table dlxigp_ip.
 * Ngp_l/dNgp_l (equispaced basis) are not needed by the hot path. */
void F(orc_element_basis)(int P, const int *AtoIJK, const real *xgp,
                          real *Ngp, real *dNgp, real *dlxigp_ip)
{
    int Q = P + 1, n = Q * Q * Q;
    real grid[ORC_MAXQ];
    real *N = (real *)malloc(sizeof(real) * n);
    real *dN = (real *)malloc(sizeof(real) * 3 * n);
    real dlx[3 * ORC_MAXQ];
    gll_roots(P, grid);
    for (int g = 0; g < n; ++g) {
        triple_tensor_product(P, n, grid, xgp[0 * n + g], xgp[1 * n + g], xgp[2 * n + g], AtoIJK, N, dN, dlx);
        for (int a = 0; a < n; ++a) {
            Ngp[a * n + g] = N[a];
            for (int d = 0; d < 3; ++d) dNgp[(g * n + a) * 3 + d] = dN[a * 3 + d];
        }
        for (int d = 0; d < 3; ++d)
            for (int ii = 0; ii < Q; ++ii) dlxigp_ip[(ii * 3 + d) * n + g] = dlx[d * Q + ii];
    }
    free(N);
    free(dN);
}

/* elem_jacobian, jacobian_oper.f90:7-136 (3-D branch), and tet_jacobian,
 * jacobian_oper.f90:138-267 (the same steps for n = 4): Je = dNgp . x,
 * cofactor inverse He = Je^-1, gpvol = wgp * det(Je); n nodes = n points. */
static void jacobian_n(int n, int nelem, int npoin, const int *connec, const real *coord, const real *dNgp,
                       const real *wgp, real *gpvol, real *He)
{
    for (int64_t e = 0; e < nelem; ++e) {
        for (int g = 0; g < n; ++g) {
            real Je[3][3];
            for (int id = 0; id < 3; ++id)
                for (int jd = 0; jd < 3; ++jd) {
                    real dot = (real)0.0;
                    for (int a = 0; a < n; ++a) {
                        int64_t p = connec[(int64_t)a * nelem + e] - 1;
                        dot = dot + dNgp[((int64_t)g * n + a) * 3 + id] * coord[(int64_t)jd * npoin + p];
                    }
                    Je[id][jd] = (real)0.0 + dot;
                }
            real det = (Je[0][0] * Je[1][1] * Je[2][2] + Je[0][1] * Je[1][2] * Je[2][0] +
                        Je[0][2] * Je[1][0] * Je[2][1] - Je[2][0] * Je[1][1] * Je[0][2] -
                        Je[2][1] * Je[1][2] * Je[0][0] - Je[2][2] * Je[1][0] * Je[0][1]);
            real a[9], b[9];
            a[0] = Je[1][1] * Je[2][2] - Je[2][1] * Je[1][2];
            a[1] = Je[1][0] * Je[2][2] - Je[2][0] * Je[1][2];
            a[2] = Je[1][0] * Je[2][1] - Je[2][0] * Je[1][1];
            a[3] = Je[0][1] * Je[2][2] - Je[2][1] * Je[0][2];
            a[4] = Je[0][0] * Je[2][2] - Je[2][0] * Je[0][2];
            a[5] = Je[0][0] * Je[2][1] - Je[2][0] * Je[0][1];
            a[6] = Je[0][1] * Je[1][2] - Je[1][1] * Je[0][2];
            a[7] = Je[0][0] * Je[1][2] - Je[1][0] * Je[0][2];
            a[8] = Je[0][0] * Je[1][1] - Je[1][0] * Je[0][1];
            a[1] = -a[1]; a[3] = -a[3]; a[5] = -a[5]; a[7] = -a[7];
            for (int k = 0; k < 9; ++k) b[k] = a[k];
            b[1] = a[3]; b[2] = a[6]; b[3] = a[1]; b[5] = a[7]; b[6] = a[2]; b[7] = a[5];
            for (int k = 0; k < 9; ++k) b[k] = ((real)1.0 / det) * b[k];
            real *H = He + ((int64_t)e * n + g) * 9;
            /* He(i,j) at H[j*3+i]; b is row-major over (i,j). */
            H[0 + 0] = b[0]; H[3 + 0] = b[1]; H[6 + 0] = b[2];
            H[0 + 1] = b[3]; H[3 + 1] = b[4]; H[6 + 1] = b[5];
            H[0 + 2] = b[6]; H[3 + 2] = b[7]; H[6 + 2] = b[8];
            gpvol[(int64_t)e * n + g] = wgp[g] * det;
        }
    }
}

void F(orc_elem_jacobian)(int P, int nelem, int npoin, const int *connec, const real *coord,
                          const real *dNgp, const real *wgp, real *gpvol, real *He)
{
    int Q = P + 1;
    jacobian_n(Q * Q * Q, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He);
}

/* create_mesh, mod_mesh.f90:11-65: disconnected mesh, connec = (e-1)*n+a,
 * every element a copy of xyzBase shifted by 3.0 per element. */
void F(orc_create_mesh_disconnected)(int P, int nelem, const real *xyzBase, int *connec, real *coord)
{
    int Q = P + 1, n = Q * Q * Q;
    int64_t npoin = (int64_t)nelem * n;
    real xyz0 = (real)0.0;
    for (int64_t e = 0; e < nelem; ++e)
        for (int a = 0; a < n; ++a) connec[(int64_t)a * nelem + e] = (int)(e * n + a + 1);
    for (int64_t e = 0; e < nelem; ++e) {
        for (int a = 0; a < n; ++a) {
            int64_t p = connec[(int64_t)a * nelem + e] - 1;
            for (int d = 0; d < 3; ++d) coord[d * npoin + p] = xyzBase[d * n + a] + xyz0;
        }
        xyz0 = xyz0 + (real)3.0;
    }
}

/* main.f90:326-361: the reference driver's initial condition (all ones;
 * nodes 1 and 4 of every element set to 10/20 for u and rho, 100/200 for pr;
 * q = rho u, eint = pr/((gamma-1) rho), E = rho eint + q.u/2, T = pr/(rho Rgas)).
 * mu_fluid = mu_e = mu_sgs = 1. */
void F(orc_reference_ic)(int P, int nelem, int npoin, const int *connec, real *u, real *q,
                         real *rho, real *pr, real *E, real *Tem, real *mu_fluid,
                         real *mu_e, real *mu_sgs)
{
    int Q = P + 1, n = Q * Q * Q;
    const real gamma_ = (real)1.4, Rgas = (real)287.0;
    for (int64_t p = 0; p < npoin; ++p) {
        for (int d = 0; d < 3; ++d) u[d * (int64_t)npoin + p] = (real)1.0;
        rho[p] = pr[p] = E[p] = Tem[p] = mu_fluid[p] = (real)1.0;
    }
    for (int64_t i = 0; i < (int64_t)nelem * n; ++i) { mu_e[i] = (real)1.0; mu_sgs[i] = (real)1.0; }
    for (int64_t e = 0; e < nelem; ++e) {
        int64_t p1 = connec[0 * (int64_t)nelem + e] - 1, p4 = connec[3 * (int64_t)nelem + e] - 1;
        for (int d = 0; d < 3; ++d) { u[d * (int64_t)npoin + p1] = (real)10.0; u[d * (int64_t)npoin + p4] = (real)20.0; }
        rho[p1] = (real)10.0; rho[p4] = (real)20.0;
        pr[p1] = (real)100.0; pr[p4] = (real)200.0;
    }
    for (int64_t p = 0; p < npoin; ++p) {
        real fmag = (real)0.0;
        for (int d = 0; d < 3; ++d) {
            q[d * (int64_t)npoin + p] = rho[p] * u[d * (int64_t)npoin + p];
            fmag = fmag + q[d * (int64_t)npoin + p] * u[d * (int64_t)npoin + p];
        }
        real eint = pr[p] / ((gamma_ - (real)1.0) * rho[p]);
        E[p] = rho[p] * eint + (real)0.5 * fmag;
        Tem[p] = pr[p] / (rho[p] * Rgas);
    }
}

/* ------------------------------------------------------------------------- */
/* Convection: elem_convec.f90:198-431 (fused) and :433-836 (split)          */
/* ------------------------------------------------------------------------- */

typedef struct {
    int P, Q, n;
    const int *inv;          /* invAtoIJK */
    const int *AI, *AJ, *AK; /* gmshAtoI/J/K */
} elem_t;

/* Per-thread element work arrays (the reference's gang-private arrays). */
typedef struct {
    real ul[ORC_MAXN][3], ql[ORC_MAXN][3], rhol[ORC_MAXN], prl[ORC_MAXN], El[ORC_MAXN], REl[ORC_MAXN];
    real kl[ORC_MAXN], Rkl[ORC_MAXN], fel[ORC_MAXN][3], fuel[ORC_MAXN][3], fkl[ORC_MAXN][3], fukl[ORC_MAXN][3];
    real fl[ORC_MAXN][3][3], fuul[ORC_MAXN][3][3];
} scratch_t;

#define INV(el, i, j, k) ((el)->inv[(((k) - 1) * (el)->Q + ((j) - 1)) * (el)->Q + ((i) - 1)] - 1)
#define HE(e, g, i, j) He[(((int64_t)(e) * n + (g)) * 3 + (j)) * 3 + (i)]

/* One element of the fused kernel's mass and momentum residuals
 * (elem_convec.f90:229-405): the nodal products are re-evaluated inside the
 * ii loop exactly as written there. */
static void convec_fused_elem(scratch_t *s, const elem_t *el, int64_t e, int nelem, int64_t npoin, const int *connec,
                              const real *He, const real *gpvol, const real *dlxigp_ip,
                              const real *u, const real *q, const real *rho, const real *pr,
                              real *Re_mass, real *Re_mom /* [n*3] */, int64_t *ipoin)
{
    const int n = el->n, Q = el->Q;
    real (*ul)[3] = s->ul, (*ql)[3] = s->ql, *rhol = s->rhol, *prl = s->prl;
    for (int a = 0; a < n; ++a) {
        ipoin[a] = connec[(int64_t)a * nelem + e] - 1;
        rhol[a] = rho[ipoin[a]];
        prl[a] = pr[ipoin[a]];
        for (int d = 0; d < 3; ++d) {
            ul[a][d] = u[d * npoin + ipoin[a]];
            ql[a][d] = q[d * npoin + ipoin[a]];
        }
    }
    for (int g = 0; g < n; ++g) {
        int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
        real dlxi[ORC_MAXQ], dleta[ORC_MAXQ], dlzeta[ORC_MAXQ];
        for (int ii = 0; ii < Q; ++ii) {
            dlxi[ii] = dlxigp_ip[(ii * 3 + 0) * n + g];
            dleta[ii] = dlxigp_ip[(ii * 3 + 1) * n + g];
            dlzeta[ii] = dlxigp_ip[(ii * 3 + 2) * n + g];
        }
        real gRho[3] = {0, 0, 0}, gP[3] = {0, 0, 0}, gU[3][3], gQ[3][3], gF[3][3][3], gFuu[3][3][3];
        memset(gU, 0, sizeof gU); memset(gQ, 0, sizeof gQ);
        memset(gF, 0, sizeof gF); memset(gFuu, 0, sizeof gFuu);
        for (int ii = 1; ii <= Q; ++ii) {
            int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
            real d1 = dlxi[ii - 1], d2 = dleta[ii - 1], d3 = dlzeta[ii - 1];
            gRho[0] = gRho[0] + d1 * rhol[b1];
            gRho[1] = gRho[1] + d2 * rhol[b2];
            gRho[2] = gRho[2] + d3 * rhol[b3];
            gP[0] = gP[0] + d1 * prl[b1];
            gP[1] = gP[1] + d2 * prl[b2];
            gP[2] = gP[2] + d3 * prl[b3];
            for (int id = 0; id < 3; ++id) {
                gU[id][0] = gU[id][0] + d1 * ul[b1][id];
                gU[id][1] = gU[id][1] + d2 * ul[b2][id];
                gU[id][2] = gU[id][2] + d3 * ul[b3][id];
                gQ[id][0] = gQ[id][0] + d1 * ql[b1][id];
                gQ[id][1] = gQ[id][1] + d2 * ql[b2][id];
                gQ[id][2] = gQ[id][2] + d3 * ql[b3][id];
                for (int jd = 0; jd < 3; ++jd) {
                    gF[id][jd][0] = gF[id][jd][0] + d1 * ql[b1][id] * ul[b1][jd];
                    gF[id][jd][1] = gF[id][jd][1] + d2 * ql[b2][id] * ul[b2][jd];
                    gF[id][jd][2] = gF[id][jd][2] + d3 * ql[b3][id] * ul[b3][jd];
                    gFuu[id][jd][0] = gFuu[id][jd][0] + d1 * ul[b1][id] * ul[b1][jd];
                    gFuu[id][jd][1] = gFuu[id][jd][1] + d2 * ul[b2][id] * ul[b2][jd];
                    gFuu[id][jd][2] = gFuu[id][jd][2] + d3 * ul[b3][id] * ul[b3][jd];
                }
            }
        }
        real gradRho[3] = {0, 0, 0}, gradP[3] = {0, 0, 0}, gradU[3][3], gradQ[3][3];
        real divF[3] = {0, 0, 0}, divFuu[3] = {0, 0, 0};
        memset(gradU, 0, sizeof gradU); memset(gradQ, 0, sizeof gradQ);
        for (int id = 0; id < 3; ++id)
            for (int jd = 0; jd < 3; ++jd) {
                gradRho[id] = gradRho[id] + HE(e, g, id, jd) * gRho[jd];
                gradP[id] = gradP[id] + HE(e, g, id, jd) * gP[jd];
                for (int kd = 0; kd < 3; ++kd) {
                    gradU[id][jd] = gradU[id][jd] + HE(e, g, jd, kd) * gU[id][kd];
                    gradQ[id][jd] = gradQ[id][jd] + HE(e, g, jd, kd) * gQ[id][kd];
                    divF[id] = divF[id] + HE(e, g, jd, kd) * gF[id][jd][kd];
                    divFuu[id] = divFuu[id] + HE(e, g, jd, kd) * gFuu[id][jd][kd];
                }
            }
        real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
        real divQ = gradQ[0][0] + gradQ[1][1] + gradQ[2][2];
        real rm = (real)0.5 * (divQ + rhol[g] * divU);
        for (int id = 0; id < 3; ++id) {
            real rmom = (real)0.25 * (divF[id] + ul[g][id] * divQ + ql[g][id] * divU + rhol[g] * divFuu[id]) + gradP[id];
            rm = rm + (real)0.5 * (ul[g][id] * gradRho[id]);
            for (int jd = 0; jd < 3; ++jd) {
                real aux = ul[g][id] * ul[g][jd];
                rmom = rmom + (real)0.25 * (aux * gradRho[jd] + ql[g][jd] * gradU[id][jd] + ul[g][jd] * gradQ[id][jd]);
            }
            Re_mom[g * 3 + id] = gpvol[(int64_t)e * n + g] * rmom;
        }
        Re_mass[g] = gpvol[(int64_t)e * n + g] * rm;
    }
}

/* One element of the split kernel's mass residual (elem_convec.f90:466-538). */
static void convec_split_mass_elem(scratch_t *s, const elem_t *el, int64_t e, int nelem, int64_t npoin, const int *connec,
                                   const real *He, const real *gpvol, const real *dlxigp_ip,
                                   const real *u, const real *q, const real *rho, real *Re_mass, int64_t *ipoin)
{
    const int n = el->n, Q = el->Q;
    real (*ul)[3] = s->ul, (*ql)[3] = s->ql, *rhol = s->rhol;
    for (int a = 0; a < n; ++a) {
        ipoin[a] = connec[(int64_t)a * nelem + e] - 1;
        rhol[a] = rho[ipoin[a]];
        for (int d = 0; d < 3; ++d) { ul[a][d] = u[d * npoin + ipoin[a]]; ql[a][d] = q[d * npoin + ipoin[a]]; }
    }
    for (int g = 0; g < n; ++g) {
        int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
        real gRho[3] = {0, 0, 0}, gU[3][3], gQ[3][3];
        memset(gU, 0, sizeof gU); memset(gQ, 0, sizeof gQ);
        for (int ii = 1; ii <= Q; ++ii) {
            int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
            real d1 = dlxigp_ip[((ii - 1) * 3 + 0) * n + g];
            real d2 = dlxigp_ip[((ii - 1) * 3 + 1) * n + g];
            real d3 = dlxigp_ip[((ii - 1) * 3 + 2) * n + g];
            gRho[0] = gRho[0] + d1 * rhol[b1];
            gRho[1] = gRho[1] + d2 * rhol[b2];
            gRho[2] = gRho[2] + d3 * rhol[b3];
            for (int id = 0; id < 3; ++id) {
                gU[id][0] = gU[id][0] + d1 * ul[b1][id];
                gU[id][1] = gU[id][1] + d2 * ul[b2][id];
                gU[id][2] = gU[id][2] + d3 * ul[b3][id];
                gQ[id][0] = gQ[id][0] + d1 * ql[b1][id];
                gQ[id][1] = gQ[id][1] + d2 * ql[b2][id];
                gQ[id][2] = gQ[id][2] + d3 * ql[b3][id];
            }
        }
        real gradRho[3] = {0, 0, 0}, gradU[3][3], gradQ[3][3];
        memset(gradU, 0, sizeof gradU); memset(gradQ, 0, sizeof gradQ);
        for (int id = 0; id < 3; ++id)
            for (int jd = 0; jd < 3; ++jd) {
                gradRho[id] = gradRho[id] + HE(e, g, id, jd) * gRho[jd];
                for (int kd = 0; kd < 3; ++kd) {
                    gradU[id][jd] = gradU[id][jd] + HE(e, g, jd, kd) * gU[id][kd];
                    gradQ[id][jd] = gradQ[id][jd] + HE(e, g, jd, kd) * gQ[id][kd];
                }
            }
        real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
        real divQ = gradQ[0][0] + gradQ[1][1] + gradQ[2][2];
        real rm = (real)0.5 * (divQ + rhol[g] * divU);
        for (int id = 0; id < 3; ++id) rm = rm + (real)0.5 * (ul[g][id] * gradRho[id]);
        Re_mass[g] = gpvol[(int64_t)e * n + g] * rm;
    }
}

/* One element of the split kernel's momentum residual (elem_convec.f90:555-657):
 * the nodal products fl = q(x)u and fuul = u(x)u are formed once per node. */
static void convec_split_mom_elem(scratch_t *s, const elem_t *el, int64_t e, int nelem, int64_t npoin, const int *connec,
                                  const real *He, const real *gpvol, const real *dlxigp_ip,
                                  const real *u, const real *q, const real *rho, const real *pr,
                                  real *Re_mom, int64_t *ipoin)
{
    const int n = el->n, Q = el->Q;
    real (*ul)[3] = s->ul, (*ql)[3] = s->ql, *rhol = s->rhol, *prl = s->prl;
    real (*fl)[3][3] = s->fl, (*fuul)[3][3] = s->fuul;
    for (int a = 0; a < n; ++a) {
        ipoin[a] = connec[(int64_t)a * nelem + e] - 1;
        int64_t p = ipoin[a];
        rhol[a] = rho[p];
        prl[a] = pr[p];
        for (int id = 0; id < 3; ++id) {
            ul[a][id] = u[id * npoin + p];
            ql[a][id] = q[id * npoin + p];
            for (int jd = 0; jd < 3; ++jd) {
                fl[a][id][jd] = q[id * npoin + p] * u[jd * npoin + p];
                fuul[a][id][jd] = u[id * npoin + p] * u[jd * npoin + p];
            }
        }
    }
    for (int g = 0; g < n; ++g) {
        int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
        real gRho[3] = {0, 0, 0}, gP[3] = {0, 0, 0}, gU[3][3], gQ[3][3], gF[3][3][3], gFuu[3][3][3];
        memset(gU, 0, sizeof gU); memset(gQ, 0, sizeof gQ);
        memset(gF, 0, sizeof gF); memset(gFuu, 0, sizeof gFuu);
        for (int ii = 1; ii <= Q; ++ii) {
            int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
            real d1 = dlxigp_ip[((ii - 1) * 3 + 0) * n + g];
            real d2 = dlxigp_ip[((ii - 1) * 3 + 1) * n + g];
            real d3 = dlxigp_ip[((ii - 1) * 3 + 2) * n + g];
            gRho[0] = gRho[0] + d1 * rhol[b1];
            gRho[1] = gRho[1] + d2 * rhol[b2];
            gRho[2] = gRho[2] + d3 * rhol[b3];
            gP[0] = gP[0] + d1 * prl[b1];
            gP[1] = gP[1] + d2 * prl[b2];
            gP[2] = gP[2] + d3 * prl[b3];
            for (int id = 0; id < 3; ++id) {
                gU[id][0] = gU[id][0] + d1 * ul[b1][id];
                gU[id][1] = gU[id][1] + d2 * ul[b2][id];
                gU[id][2] = gU[id][2] + d3 * ul[b3][id];
                gQ[id][0] = gQ[id][0] + d1 * ql[b1][id];
                gQ[id][1] = gQ[id][1] + d2 * ql[b2][id];
                gQ[id][2] = gQ[id][2] + d3 * ql[b3][id];
                for (int jd = 0; jd < 3; ++jd) {
                    gF[id][jd][0] = gF[id][jd][0] + d1 * fl[b1][id][jd];
                    gF[id][jd][1] = gF[id][jd][1] + d2 * fl[b2][id][jd];
                    gF[id][jd][2] = gF[id][jd][2] + d3 * fl[b3][id][jd];
                    gFuu[id][jd][0] = gFuu[id][jd][0] + d1 * fuul[b1][id][jd];
                    gFuu[id][jd][1] = gFuu[id][jd][1] + d2 * fuul[b2][id][jd];
                    gFuu[id][jd][2] = gFuu[id][jd][2] + d3 * fuul[b3][id][jd];
                }
            }
        }
        real gradRho[3] = {0, 0, 0}, gradP[3] = {0, 0, 0}, gradU[3][3], gradQ[3][3];
        real divF[3] = {0, 0, 0}, divFuu[3] = {0, 0, 0};
        memset(gradU, 0, sizeof gradU); memset(gradQ, 0, sizeof gradQ);
        for (int id = 0; id < 3; ++id)
            for (int jd = 0; jd < 3; ++jd) {
                gradRho[id] = gradRho[id] + HE(e, g, id, jd) * gRho[jd];
                gradP[id] = gradP[id] + HE(e, g, id, jd) * gP[jd];
                for (int kd = 0; kd < 3; ++kd) {
                    gradU[id][jd] = gradU[id][jd] + HE(e, g, jd, kd) * gU[id][kd];
                    gradQ[id][jd] = gradQ[id][jd] + HE(e, g, jd, kd) * gQ[id][kd];
                    divF[id] = divF[id] + HE(e, g, jd, kd) * gF[id][jd][kd];
                    divFuu[id] = divFuu[id] + HE(e, g, jd, kd) * gFuu[id][jd][kd];
                }
            }
        real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
        real divQ = gradQ[0][0] + gradQ[1][1] + gradQ[2][2];
        for (int id = 0; id < 3; ++id) {
            real rmom = (real)0.25 * (divF[id] + ul[g][id] * divQ + ql[g][id] * divU + rhol[g] * divFuu[id]) + gradP[id];
            for (int jd = 0; jd < 3; ++jd)
                rmom = rmom + (real)0.25 * (fuul[g][id][jd] * gradRho[jd] + ql[g][jd] * gradU[id][jd] + ul[g][jd] * gradQ[id][jd]);
            Re_mom[g * 3 + id] = gpvol[(int64_t)e * n + g] * rmom;
        }
    }
}

/* One element of the split kernel's energy residual (elem_convec.f90:677-820).
 * This is the only complete definition of Rener in the reference: the fused
 * kernel reads fuel/fukl without assigning them (elem_convec.f90:247-250,
 * 394-396), so both oracle entry points take Rener from here. */
static void convec_split_ener_elem(scratch_t *s, const elem_t *el, int64_t e, int nelem, int64_t npoin, const int *connec,
                                   const real *He, const real *gpvol, const real *dlxigp_ip,
                                   const real *u, const real *q, const real *rho, const real *Earr,
                                   real *Re_ener, int64_t *ipoin)
{
    const int n = el->n, Q = el->Q;
    real (*ul)[3] = s->ul, (*ql)[3] = s->ql, *rhol = s->rhol, *El = s->El, *REl = s->REl;
    real *kl = s->kl, *Rkl = s->Rkl, (*fel)[3] = s->fel, (*fuel)[3] = s->fuel, (*fkl)[3] = s->fkl, (*fukl)[3] = s->fukl;
    for (int a = 0; a < n; ++a) {
        ipoin[a] = connec[(int64_t)a * nelem + e] - 1;
        int64_t p = ipoin[a];
        kl[a] = (real)0.0;
        for (int id = 0; id < 3; ++id) kl[a] = kl[a] + u[id * npoin + p] * u[id * npoin + p] * (real)0.5;
        rhol[a] = rho[p];
        El[a] = Earr[p];
        REl[a] = rho[p] * Earr[p];
        Rkl[a] = rho[p] * kl[a];
        for (int id = 0; id < 3; ++id) {
            ul[a][id] = u[id * npoin + p];
            ql[a][id] = q[id * npoin + p];
            fel[a][id] = rho[p] * Earr[p] * u[id * npoin + p];
            fuel[a][id] = Earr[p] * u[id * npoin + p];
            fkl[a][id] = rho[p] * kl[a] * u[id * npoin + p];
            fukl[a][id] = kl[a] * u[id * npoin + p];
        }
    }
    for (int g = 0; g < n; ++g) {
        int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
        real gRho[3] = {0, 0, 0}, gE[3] = {0, 0, 0}, gRE[3] = {0, 0, 0}, gk[3] = {0, 0, 0}, gRk[3] = {0, 0, 0};
        real gU[3][3], gQ[3][3], gFe[3][3], gFue[3][3], gFk[3][3], gFuk[3][3];
        memset(gU, 0, sizeof gU); memset(gQ, 0, sizeof gQ); memset(gFe, 0, sizeof gFe);
        memset(gFue, 0, sizeof gFue); memset(gFk, 0, sizeof gFk); memset(gFuk, 0, sizeof gFuk);
        for (int ii = 1; ii <= Q; ++ii) {
            int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
            real d1 = dlxigp_ip[((ii - 1) * 3 + 0) * n + g];
            real d2 = dlxigp_ip[((ii - 1) * 3 + 1) * n + g];
            real d3 = dlxigp_ip[((ii - 1) * 3 + 2) * n + g];
            gRho[0] = gRho[0] + d1 * rhol[b1]; gRho[1] = gRho[1] + d2 * rhol[b2]; gRho[2] = gRho[2] + d3 * rhol[b3];
            gE[0] = gE[0] + d1 * (El[b1]); gE[1] = gE[1] + d2 * (El[b2]); gE[2] = gE[2] + d3 * (El[b3]);
            gRE[0] = gRE[0] + d1 * (REl[b1]); gRE[1] = gRE[1] + d2 * (REl[b2]); gRE[2] = gRE[2] + d3 * (REl[b3]);
            gk[0] = gk[0] + d1 * (kl[b1]); gk[1] = gk[1] + d2 * (kl[b2]); gk[2] = gk[2] + d3 * (kl[b3]);
            gRk[0] = gRk[0] + d1 * (Rkl[b1]); gRk[1] = gRk[1] + d2 * (Rkl[b2]); gRk[2] = gRk[2] + d3 * (Rkl[b3]);
            for (int id = 0; id < 3; ++id) {
                gU[id][0] = gU[id][0] + d1 * ul[b1][id];
                gU[id][1] = gU[id][1] + d2 * ul[b2][id];
                gU[id][2] = gU[id][2] + d3 * ul[b3][id];
                gQ[id][0] = gQ[id][0] + d1 * ql[b1][id];
                gQ[id][1] = gQ[id][1] + d2 * ql[b2][id];
                gQ[id][2] = gQ[id][2] + d3 * ql[b3][id];
                gFe[id][0] = gFe[id][0] + d1 * fel[b1][id];
                gFe[id][1] = gFe[id][1] + d2 * fel[b2][id];
                gFe[id][2] = gFe[id][2] + d3 * fel[b3][id];
                gFue[id][0] = gFue[id][0] + d1 * fuel[b1][id];
                gFue[id][1] = gFue[id][1] + d2 * fuel[b2][id];
                gFue[id][2] = gFue[id][2] + d3 * fuel[b3][id];
                gFk[id][0] = gFk[id][0] + d1 * fkl[b1][id];
                gFk[id][1] = gFk[id][1] + d2 * fkl[b2][id];
                gFk[id][2] = gFk[id][2] + d3 * fkl[b3][id];
                gFuk[id][0] = gFuk[id][0] + d1 * fukl[b1][id];
                gFuk[id][1] = gFuk[id][1] + d2 * fukl[b2][id];
                gFuk[id][2] = gFuk[id][2] + d3 * fukl[b3][id];
            }
        }
        real gradRho[3] = {0, 0, 0}, gradE[3] = {0, 0, 0}, gradRE[3] = {0, 0, 0}, gradk[3] = {0, 0, 0}, gradRk[3] = {0, 0, 0};
        real gradU[3][3], gradQ[3][3];
        real divFe = 0, divFue = 0, divFk = 0, divFuk = 0;
        memset(gradU, 0, sizeof gradU); memset(gradQ, 0, sizeof gradQ);
        for (int id = 0; id < 3; ++id)
            for (int jd = 0; jd < 3; ++jd) {
                real h = HE(e, g, id, jd);
                gradRho[id] = gradRho[id] + h * gRho[jd];
                gradE[id] = gradE[id] + h * gE[jd];
                gradRE[id] = gradRE[id] + h * gRE[jd];
                divFe = divFe + h * gFe[id][jd];
                divFue = divFue + h * gFue[id][jd];
                gradk[id] = gradk[id] + h * gk[jd];
                gradRk[id] = gradRk[id] + h * gRk[jd];
                divFk = divFk + h * gFk[id][jd];
                divFuk = divFuk + h * gFuk[id][jd];
                for (int kd = 0; kd < 3; ++kd) {
                    gradU[id][jd] = gradU[id][jd] + HE(e, g, jd, kd) * gU[id][kd];
                    gradQ[id][jd] = gradQ[id][jd] + HE(e, g, jd, kd) * gQ[id][kd];
                }
            }
        real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
        real divQ = gradQ[0][0] + gradQ[1][1] + gradQ[2][2];
        real re = (real)0.25 * (divFe + El[g] * divQ + REl[g] * divU + rhol[g] * divFue) +
                  (real)0.25 * (divFk + kl[g] * divQ + Rkl[g] * divU + rhol[g] * divFuk);
        for (int id = 0; id < 3; ++id)
            re = re + (real)0.25 * (ql[g][id] * gradE[id] + ul[g][id] * gradRE[id] + fuel[g][id] * gradRho[id]) +
                 (real)0.25 * (ql[g][id] * gradk[id] + ul[g][id] * gradRk[id] + fukl[g][id] * gradRho[id]);
        Re_ener[g] = gpvol[(int64_t)e * n + g] * re;
    }
}

static int elem_setup(elem_t *el, int P, const int *inv, const int *AI, const int *AJ, const int *AK)
{
    if (P < 1 || P > ORC_MAXP) return -1;
    el->P = P; el->Q = P + 1; el->n = el->Q * el->Q * el->Q;
    el->inv = inv; el->AI = AI; el->AJ = AJ; el->AK = AK;
    return 0;
}

/* Scatter-add of element residuals to nodes (elem_convec.f90:412-426).  With
 * nthreads > 1 the element loop is shared by OpenMP threads and the adds are
 * atomic, like the OpenACC build's "atomic update". */
#define SCATTER(dst, idx, val, atomic)                 \
    do {                                               \
        if (atomic) {                                  \
            _Pragma("omp atomic") (dst)[idx] += (val); \
        } else {                                       \
            (dst)[idx] = (dst)[idx] + (val);           \
        }                                              \
    } while (0)

/* full_convec_ijk (elem_convec.f90:198-431): Rmass and Rmom as the fused
 * kernel evaluates them, Rener from the split kernel's definition (see
 * convec_split_ener_elem).  Returns 0, or -1 for an unsupported porder. */
int F(orc_full_convec_ijk)(int P, int nelem, int npoin, const int *connec, const real *He,
                           const real *gpvol, const real *dlxigp_ip, const int *invAtoIJK,
                           const int *AtoI, const int *AtoJ, const int *AtoK, const real *u,
                           const real *q, const real *rho, const real *pr, const real *E,
                           real *Rmass, real *Rmom, real *Rener, int nthreads)
{
    elem_t el;
    if (elem_setup(&el, P, invAtoIJK, AtoI, AtoJ, AtoK)) return -1;
    const int n = el.n;
    const int64_t np = npoin;
    memset(Rmass, 0, sizeof(real) * np);
    memset(Rmom, 0, sizeof(real) * 3 * np);
    memset(Rener, 0, sizeof(real) * np);
    const int atomic = nthreads > 1;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) if (atomic)
    {
        scratch_t *s = (scratch_t *)malloc(sizeof(scratch_t));
        real *Re_mass = (real *)malloc(sizeof(real) * n), *Re_ener = (real *)malloc(sizeof(real) * n);
        real *Re_mom = (real *)malloc(sizeof(real) * 3 * n);
        int64_t *ipoin = (int64_t *)malloc(sizeof(int64_t) * n);
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = 0; e < nelem; ++e) {
            convec_fused_elem(s, &el, e, nelem, np, connec, He, gpvol, dlxigp_ip, u, q, rho, pr, Re_mass, Re_mom, ipoin);
            convec_split_ener_elem(s, &el, e, nelem, np, connec, He, gpvol, dlxigp_ip, u, q, rho, E, Re_ener, ipoin);
            for (int a = 0; a < n; ++a) {
                SCATTER(Rmass, ipoin[a], Re_mass[a], atomic);
                SCATTER(Rener, ipoin[a], Re_ener[a], atomic);
                for (int d = 0; d < 3; ++d) SCATTER(Rmom, d * np + ipoin[a], Re_mom[a * 3 + d], atomic);
            }
        }
        free(Re_mass); free(Re_ener); free(Re_mom); free(ipoin); free(s);
    }
    return 0;
}

/* full_convec_ijk_split (elem_convec.f90:433-836): three element loops (mass,
 * momentum, energy), each with its own gather and scatter. */
int F(orc_full_convec_ijk_split)(int P, int nelem, int npoin, const int *connec, const real *He,
                                 const real *gpvol, const real *dlxigp_ip, const int *invAtoIJK,
                                 const int *AtoI, const int *AtoJ, const int *AtoK, const real *u,
                                 const real *q, const real *rho, const real *pr, const real *E,
                                 real *Rmass, real *Rmom, real *Rener, int nthreads)
{
    elem_t el;
    if (elem_setup(&el, P, invAtoIJK, AtoI, AtoJ, AtoK)) return -1;
    const int n = el.n;
    const int64_t np = npoin;
    memset(Rmass, 0, sizeof(real) * np);
    memset(Rmom, 0, sizeof(real) * 3 * np);
    memset(Rener, 0, sizeof(real) * np);
    const int atomic = nthreads > 1;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) if (atomic)
    {
        scratch_t *s = (scratch_t *)malloc(sizeof(scratch_t));
        real *Re = (real *)malloc(sizeof(real) * 3 * n);
        int64_t *ipoin = (int64_t *)malloc(sizeof(int64_t) * n);
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = 0; e < nelem; ++e) {
            convec_split_mass_elem(s, &el, e, nelem, np, connec, He, gpvol, dlxigp_ip, u, q, rho, Re, ipoin);
            for (int a = 0; a < n; ++a) SCATTER(Rmass, ipoin[a], Re[a], atomic);
        }
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = 0; e < nelem; ++e) {
            convec_split_mom_elem(s, &el, e, nelem, np, connec, He, gpvol, dlxigp_ip, u, q, rho, pr, Re, ipoin);
            for (int a = 0; a < n; ++a)
                for (int d = 0; d < 3; ++d) SCATTER(Rmom, d * np + ipoin[a], Re[a * 3 + d], atomic);
        }
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = 0; e < nelem; ++e) {
            convec_split_ener_elem(s, &el, e, nelem, np, connec, He, gpvol, dlxigp_ip, u, q, rho, E, Re, ipoin);
            for (int a = 0; a < n; ++a) SCATTER(Rener, ipoin[a], Re[a], atomic);
        }
        free(Re); free(ipoin); free(s);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Diffusion: elem_diffu.f90:10-197                                          */
/* ------------------------------------------------------------------------- */

/* full_diffusion_ijk.  Pass 1 (:67-139) forms per point tau, tau.u, grad T and
 * grad rho; pass 2 (:141-193) applies the weak divergence with nu_e and
 * kappa_e taken at the output node (:143-146).  c_rho = c_ener = 1
 * (mod_numerical_params.f90:26-27).  The kappa_e of :72 is dead code. */
int F(orc_full_diffusion_ijk)(int P, int nelem, int npoin, const int *connec, const real *He,
                              const real *gpvol, const real *dlxigp_ip, const int *invAtoIJK,
                              const int *AtoI, const int *AtoJ, const int *AtoK, real Cp, real Pr,
                              const real *rho, const real *u, const real *Tem, const real *mu_fluid,
                              const real *mu_e, const real *mu_sgs, real *Rmass, real *Rmom, real *Rener,
                              int nthreads)
{
    elem_t elx;
    if (elem_setup(&elx, P, invAtoIJK, AtoI, AtoJ, AtoK)) return -1;
    const elem_t *el = &elx;
    const int n = el->n, Q = el->Q;
    const int64_t np = npoin;
    const real c_rho = (real)1.0, c_ener = (real)1.0;
    const real twoThirds = (real)2.0 / (real)3.0;
    memset(Rmass, 0, sizeof(real) * np);
    memset(Rmom, 0, sizeof(real) * 3 * np);
    memset(Rener, 0, sizeof(real) * np);
    const int atomic = nthreads > 1;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1) if (atomic)
    {
        real (*ul)[3] = malloc(sizeof(real) * 3 * n);
        real *rhol = malloc(sizeof(real) * n), *Teml = malloc(sizeof(real) * n), *mufl = malloc(sizeof(real) * n);
        real (*tauXl)[3] = malloc(sizeof(real) * 3 * n), (*tauYl)[3] = malloc(sizeof(real) * 3 * n);
        real (*tauZl)[3] = malloc(sizeof(real) * 3 * n), (*gradTl)[3] = malloc(sizeof(real) * 3 * n);
        real (*gradRhol)[3] = malloc(sizeof(real) * 3 * n), (*tauUl)[3] = malloc(sizeof(real) * 3 * n);
        int64_t *ipoin = malloc(sizeof(int64_t) * n);
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = 0; e < nelem; ++e) {
            for (int a = 0; a < n; ++a) ipoin[a] = connec[(int64_t)a * nelem + e] - 1;
            for (int a = 0; a < n; ++a) {
                rhol[a] = rho[ipoin[a]];
                Teml[a] = Tem[ipoin[a]];
                mufl[a] = mu_fluid[ipoin[a]];
            }
            for (int a = 0; a < n; ++a)
                for (int d = 0; d < 3; ++d) ul[a][d] = u[d * np + ipoin[a]];
            for (int g = 0; g < n; ++g) {
                real mse = mu_sgs[(int64_t)g * nelem + e], me = mu_e[(int64_t)g * nelem + e];
                real mu_fgp = mufl[g] + rhol[g] * mse;
                real mu_egp = me;
                int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
                real gRho[3] = {0, 0, 0}, gT[3] = {0, 0, 0}, gU[3][3];
                memset(gU, 0, sizeof gU);
                for (int ii = 1; ii <= Q; ++ii) {
                    int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
                    real d1 = dlxigp_ip[((ii - 1) * 3 + 0) * n + g];
                    real d2 = dlxigp_ip[((ii - 1) * 3 + 1) * n + g];
                    real d3 = dlxigp_ip[((ii - 1) * 3 + 2) * n + g];
                    gRho[0] = gRho[0] + d1 * rhol[b1]; gRho[1] = gRho[1] + d2 * rhol[b2]; gRho[2] = gRho[2] + d3 * rhol[b3];
                    gT[0] = gT[0] + d1 * Teml[b1]; gT[1] = gT[1] + d2 * Teml[b2]; gT[2] = gT[2] + d3 * Teml[b3];
                    for (int id = 0; id < 3; ++id) {
                        gU[id][0] = gU[id][0] + d1 * ul[b1][id];
                        gU[id][1] = gU[id][1] + d2 * ul[b2][id];
                        gU[id][2] = gU[id][2] + d3 * ul[b3][id];
                    }
                }
                real gradRho[3] = {0, 0, 0}, gradT[3] = {0, 0, 0}, gradU[3][3];
                memset(gradU, 0, sizeof gradU);
                for (int id = 0; id < 3; ++id)
                    for (int jd = 0; jd < 3; ++jd) {
                        gradRho[id] = gradRho[id] + HE(e, g, id, jd) * gRho[jd];
                        gradT[id] = gradT[id] + HE(e, g, id, jd) * gT[jd];
                        for (int kd = 0; kd < 3; ++kd) gradU[id][jd] = gradU[id][jd] + HE(e, g, jd, kd) * gU[id][kd];
                    }
                real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
                real tauU[3] = {0, 0, 0}, tau[3][3];
                for (int id = 0; id < 3; ++id) {
                    for (int jd = 0; jd < 3; ++jd) {
                        tauU[id] = tauU[id] + (mu_fgp + mu_egp) * (gradU[id][jd] + gradU[jd][id]) * ul[g][jd];
                        tau[id][jd] = (mu_fgp + mu_egp) * (gradU[id][jd] + gradU[jd][id]);
                    }
                    tauU[id] = tauU[id] - (mu_fgp) * twoThirds * divU * ul[g][id];
                    tau[id][id] = tau[id][id] - (mu_fgp) * twoThirds * divU;
                }
                for (int id = 0; id < 3; ++id) {
                    tauXl[g][id] = tau[0][id];
                    tauYl[g][id] = tau[1][id];
                    tauZl[g][id] = tau[2][id];
                    gradTl[g][id] = gradT[id];
                    gradRhol[g][id] = gradRho[id];
                    tauUl[g][id] = tauU[id];
                }
            }
            for (int g = 0; g < n; ++g) {
                real me = mu_e[(int64_t)g * nelem + e], mse = mu_sgs[(int64_t)g * nelem + e];
                real nu_e = c_rho * me / rhol[g];
                real kappa_e = mufl[g] * Cp / Pr + c_ener * me * Cp / Pr + Cp * rhol[g] * mse / (real)0.9;
                int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
                real divDe = 0, divDr = 0, divDm[3] = {0, 0, 0};
                for (int ii = 1; ii <= Q; ++ii) {
                    int b1 = INV(el, ii, J, K), b2 = INV(el, I, ii, K), b3 = INV(el, I, J, ii);
                    real w1g = gpvol[(int64_t)e * n + b1], w2g = gpvol[(int64_t)e * n + b2], w3g = gpvol[(int64_t)e * n + b3];
                    real dl1 = dlxigp_ip[((I - 1) * 3 + 0) * n + b1];
                    real dl2 = dlxigp_ip[((J - 1) * 3 + 1) * n + b2];
                    real dl3 = dlxigp_ip[((K - 1) * 3 + 2) * n + b3];
                    for (int id = 0; id < 3; ++id) {
                        real c1 = HE(e, b1, id, 0) * w1g * dl1;
                        real c2 = HE(e, b2, id, 1) * w2g * dl2;
                        real c3 = HE(e, b3, id, 2) * w3g * dl3;
                        divDr = divDr + c1 * gradRhol[b1][id];
                        divDr = divDr + c2 * gradRhol[b2][id];
                        divDr = divDr + c3 * gradRhol[b3][id];
                        divDe = divDe + c1 * (tauUl[b1][id] + kappa_e * gradTl[b1][id]);
                        divDe = divDe + c2 * (tauUl[b2][id] + kappa_e * gradTl[b2][id]);
                        divDe = divDe + c3 * (tauUl[b3][id] + kappa_e * gradTl[b3][id]);
                        divDm[0] = divDm[0] + c1 * tauXl[b1][id];
                        divDm[0] = divDm[0] + c2 * tauXl[b2][id];
                        divDm[0] = divDm[0] + c3 * tauXl[b3][id];
                        divDm[1] = divDm[1] + c1 * tauYl[b1][id];
                        divDm[1] = divDm[1] + c2 * tauYl[b2][id];
                        divDm[1] = divDm[1] + c3 * tauYl[b3][id];
                        divDm[2] = divDm[2] + c1 * tauZl[b1][id];
                        divDm[2] = divDm[2] + c2 * tauZl[b2][id];
                        divDm[2] = divDm[2] + c3 * tauZl[b3][id];
                    }
                }
                SCATTER(Rmass, ipoin[g], nu_e * divDr, atomic);
                SCATTER(Rener, ipoin[g], divDe, atomic);
                for (int d = 0; d < 3; ++d) SCATTER(Rmom, d * np + ipoin[g], divDm[d], atomic);
            }
        }
        free(ul); free(rhol); free(Teml); free(mufl); free(tauXl); free(tauYl); free(tauZl);
        free(gradTl); free(gradRhol); free(tauUl); free(ipoin);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Entropy viscosity (no reference code: the reference consumes mu_e,        */
/* elem_diffu.f90:19; knobs mod_numerical_params.f90:22-28)                  */
/* ------------------------------------------------------------------------- */

/* Entropy-viscosity estimator of the library, restated point by point:
 * eta = rho/(gamma-1) log(p/rho^gamma); R(g) = div(eta u) - eta div u - u.grad eta
 * with the reference's per-point derivative table; per element
 * h = (sum gpvol)^(1/3)/P, nu_max = cmax h max(|u|+c), nu_E = ce h^2 max|R| / n_eta,
 * nu = min(nu_max, nu_E); mu_e(e,a) = rho(a) nu.  n_eta = max|eta - mean eta|
 * over the nodes (1 when normalise == 0).  nu/numax may be NULL. */
int F(orc_entropy_viscosity)(int P, int nelem, int npoin, const int *connec, const real *He, const real *gpvol,
                             const real *dlxigp_ip, const int *invAtoIJK, const int *AtoI, const int *AtoJ,
                             const int *AtoK, const real *rho, const real *u, const real *pr, real gamma, real ce,
                             real cmax, int normalise, real *mu_e, real *nu_out, real *numax_out)
{
    elem_t elx;
    if (elem_setup(&elx, P, invAtoIJK, AtoI, AtoJ, AtoK)) return -1;
    const elem_t *el = &elx;
    const int n = el->n, Q = el->Q;
    const int64_t np = npoin;
    double sum = 0.0, mn = 1e300, mx = -1e300;
    for (int64_t p = 0; p < np; ++p) {
        const double eta = (double)(rho[p] / (gamma - (real)1.0) * (log(pr[p]) - gamma * log(rho[p])));
        sum += eta;
        if (eta < mn) mn = eta;
        if (eta > mx) mx = eta;
    }
    real neta = (real)1.0;
    if (normalise) {
        const double mean = sum / (double)np;
        neta = (real)fmax(mx - mean, mean - mn);
        if (!(neta > 0)) neta = (real)1.0;
    }
    real *eta = (real *)malloc(sizeof(real) * n), (*ul)[3] = malloc(sizeof(real) * 3 * n), *rl = malloc(sizeof(real) * n);
    for (int64_t e = 0; e < nelem; ++e) {
        real vol = 0, rmax = 0, smax = 0;
        for (int a = 0; a < n; ++a) {
            const int64_t p = connec[(int64_t)a * nelem + e] - 1;
            rl[a] = rho[p];
            for (int d = 0; d < 3; ++d) ul[a][d] = u[d * np + p];
            eta[a] = rho[p] / (gamma - (real)1.0) * (log(pr[p]) - gamma * log(rho[p]));
            const real um = sqrt(ul[a][0] * ul[a][0] + ul[a][1] * ul[a][1] + ul[a][2] * ul[a][2]);
            const real spd = um + sqrt(gamma * pr[p] / rho[p]);
            if (spd > smax) smax = spd;
            vol += gpvol[e * n + a];
        }
        for (int g = 0; g < n; ++g) {
            int I = el->AI[g], J = el->AJ[g], K = el->AK[g];
            real ge[3] = {0, 0, 0}, gu[3][3], gf[3][3];
            memset(gu, 0, sizeof gu); memset(gf, 0, sizeof gf);
            for (int ii = 1; ii <= Q; ++ii) {
                const int b[3] = {INV(el, ii, J, K), INV(el, I, ii, K), INV(el, I, J, ii)};
                for (int d = 0; d < 3; ++d) {
                    const real dl = dlxigp_ip[((ii - 1) * 3 + d) * n + g];
                    ge[d] = ge[d] + dl * eta[b[d]];
                    for (int i = 0; i < 3; ++i) {
                        gu[i][d] = gu[i][d] + dl * ul[b[d]][i];
                        gf[i][d] = gf[i][d] + dl * (eta[b[d]] * ul[b[d]][i]);
                    }
                }
            }
            real divf = 0, divu = 0, ugrad = 0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    divf = divf + HE(e, g, i, j) * gf[i][j];
                    divu = divu + HE(e, g, i, j) * gu[i][j];
                    ugrad = ugrad + ul[g][i] * HE(e, g, i, j) * ge[j];
                }
            const real R = fabs(divf - eta[g] * divu - ugrad);
            if (R > rmax) rmax = R;
        }
        const real h = cbrt(vol) / (real)P;
        const real numax = cmax * h * smax;
        const real nuE = ce * h * h * rmax / neta;
        const real nu = numax < nuE ? numax : nuE;
        for (int a = 0; a < n; ++a) mu_e[(int64_t)a * nelem + e] = rl[a] * nu;
        if (nu_out) nu_out[e] = nu;
        if (numax_out) numax_out[e] = numax;
    }
    free(eta); free(ul); free(rl);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Linear tetrahedra: elem_tet.f90, quadrature_rules.f90:84-99,              */
/* mod_mesh.f90:71-126, jacobian_oper.f90:138-267, elem_convec.f90:839-948,  */
/* elem_diffu.f90:199-317.  Layouts (E = nelem):                             */
/*   connec(nelem,4) connec[a*E+e]; He(3,3,4,nelem) He[((e*4+g)*3+j)*3+i];   */
/*   gpvol(1,4,nelem) gpvol[e*4+g]; Ngp(4,4) Ngp[c*4+r] for Ngp(r,c);       */
/*   dNgp(3,4,4) dNgp[(g*4+a)*3+d]; mu_e(nelem,4) mu_e[a*E+e].               */
/* ------------------------------------------------------------------------- */

/* tet_4points (quadrature_rules.f90:84-99) and tet_04 (elem_tet.f90:9-36) at
 * each point, as the driver fills its tables (main.f90:377-383):
 * Ngp(igaus,inode) = N_inode(x_igaus), dNgp(:,inode,igaus) = dN_inode. */
void F(orc_tet_element_tables)(real *Ngp, real *dNgp, real *xgp, real *wgp)
{
    const real a = (real)0.5854101966249680, b = (real)0.1381966011250110;
    const real X[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
    for (int g = 0; g < 4; ++g) {
        for (int d = 0; d < 3; ++d) xgp[d * 4 + g] = X[g][d];
        wgp[g] = (real)0.25;
    }
    for (int g = 0; g < 4; ++g) {
        const real xi = xgp[0 * 4 + g], eta = xgp[1 * 4 + g], zeta = xgp[2 * 4 + g];
        const real N[4] = {(real)1.0 - xi - eta - zeta, xi, eta, zeta};
        const real dN[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int i = 0; i < 4; ++i) {
            Ngp[i * 4 + g] = N[i];
            for (int d = 0; d < 3; ++d) dNgp[(g * 4 + i) * 3 + d] = dN[i][d];
        }
    }
}

/* gen_tet_mesh (mod_mesh.f90:71-126): connec(e,a) = (e-1)*4 + a, every
 * element a copy of xyzBase(4,3) (xyzBase[d*4+a]) shifted by 3.0 per element. */
void F(orc_gen_tet_mesh)(int nelem, int npoin, const real *xyzBase, int *connec, real *coord)
{
    for (int64_t e = 0; e < nelem; ++e)
        for (int a = 0; a < 4; ++a) connec[(int64_t)a * nelem + e] = (int)(e * 4 + a + 1);
    real xyz0 = (real)0.0;
    for (int64_t e = 0; e < nelem; ++e) {
        for (int a = 0; a < 4; ++a) {
            int64_t p = connec[(int64_t)a * nelem + e] - 1;
            for (int d = 0; d < 3; ++d) coord[(int64_t)d * npoin + p] = xyzBase[d * 4 + a] + xyz0;
        }
        xyz0 = xyz0 + (real)3.0;
    }
}

void F(orc_tet_jacobian)(int nelem, int npoin, const int *connec, const real *coord, const real *dNgp,
                         const real *wgp, real *gpvol, real *He)
{
    jacobian_n(4, nelem, npoin, connec, coord, dNgp, wgp, gpvol, He);
}

/* gpcar(inode,idime) = DOT_PRODUCT(He(idime,:,igaus,ielem), dNgp(:,inode,igaus)). */
static void tet_gpcar(const real *He, const real *dNgp, int64_t e, int g, real gpcar[4][3])
{
    const real *H = He + ((int64_t)e * 4 + g) * 9;
    for (int id = 0; id < 3; ++id)
        for (int a = 0; a < 4; ++a) {
            real dot = (real)0.0;
            for (int j = 0; j < 3; ++j) dot = dot + H[j * 3 + id] * dNgp[(g * 4 + a) * 3 + j];
            gpcar[a][id] = dot;
        }
}

/* fem_convec, elem_convec.f90:839-948. */
int F(orc_fem_convec)(int nelem, int npoin, const int *connec, const real *Ngp, const real *dNgp, const real *He,
                      const real *gpvol, const real *u, const real *q, const real *rho, const real *pr,
                      const real *E, real *Rmass, real *Rmom, real *Rener, int nthreads)
{
    const int64_t np = npoin;
    memset(Rmass, 0, sizeof(real) * np);
    memset(Rmom, 0, sizeof(real) * 3 * np);
    memset(Rener, 0, sizeof(real) * np);
    const int atomic = nthreads > 1;
    const real half = (real)0.5;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) if (atomic) schedule(static, 1024)
    for (int64_t e = 0; e < nelem; ++e) {
        int64_t ip[4];
        for (int a = 0; a < 4; ++a) ip[a] = connec[(int64_t)a * nelem + e] - 1;
        real Re_mass[4] = {0, 0, 0, 0}, Re_ener[4] = {0, 0, 0, 0}, Re_mom[4][3] = {{0}};
        for (int g = 0; g < 4; ++g) {
            real divQ = 0, divFe = 0, gradRho[3] = {0, 0, 0}, gradE[3] = {0, 0, 0}, gradP[3] = {0, 0, 0};
            real gradU[3][3] = {{0}}, divF[3] = {0, 0, 0};
            real gpcar[4][3];
            tet_gpcar(He, dNgp, e, g, gpcar);
            for (int id = 0; id < 3; ++id)
                for (int j = 0; j < 4; ++j) {
                    const int64_t p = ip[j];
                    const real Ep = E[p] + pr[p];
                    divQ = divQ + gpcar[j][id] * q[id * np + p];
                    divFe = divFe + gpcar[j][id] * Ep * u[id * np + p];
                    gradRho[id] = gradRho[id] + gpcar[j][id] * rho[p];
                    gradE[id] = gradE[id] + gpcar[j][id] * Ep;
                    gradP[id] = gradP[id] + gpcar[j][id] * pr[p];
                    for (int jd = 0; jd < 3; ++jd) {
                        gradU[id][jd] = gradU[id][jd] + gpcar[j][jd] * u[id * np + p];
                        divF[id] = divF[id] + gpcar[j][jd] * q[id * np + p] * u[jd * np + p];
                    }
                }
            const real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
            for (int a = 0; a < 4; ++a) {
                const int64_t p = ip[a];
                real aux1 = 0, aux2 = 0;
                for (int id = 0; id < 3; ++id) {
                    aux1 = aux1 + gradRho[id] * u[id * np + p];
                    aux2 = aux2 + gradE[id] * u[id * np + p];
                }
                const real w = gpvol[e * 4 + g] * Ngp[a * 4 + g] * half;
                Re_mass[a] = Re_mass[a] + w * (divQ + rho[p] * divU + aux1);
                Re_ener[a] = Re_ener[a] + w * (divFe + (E[p] + pr[p]) * divU + aux2);
                for (int id = 0; id < 3; ++id) {
                    real aux3 = 0, aux4 = 0;
                    for (int jd = 0; jd < 3; ++jd) {
                        aux3 = aux3 + gradU[id][jd] * q[jd * np + p];
                        aux4 = aux4 + u[id * np + p] * u[jd * np + p] * gradRho[jd];
                    }
                    Re_mom[a][id] = Re_mom[a][id] + w * (divF[id] + q[id * np + p] * divU + aux3 + aux4 + gradP[id]);
                }
            }
        }
        for (int a = 0; a < 4; ++a) {
            SCATTER(Rmass, ip[a], Re_mass[a], atomic);
            SCATTER(Rener, ip[a], Re_ener[a], atomic);
            for (int d = 0; d < 3; ++d) SCATTER(Rmom, d * np + ip[a], Re_mom[a][d], atomic);
        }
    }
    return 0;
}

/* fem_diffu, elem_diffu.f90:199-317.  It reads Ngp(inode,igaus) -- the
 * transpose of fem_convec's Ngp(igaus,inode) -- and kappa with c_ener mu_e /
 * 0.4; c_rho = c_ener = 1 (mod_numerical_params.f90:26-27).  Its assembly has
 * no atomics (:306-312); the threaded oracle adds atomically. */
int F(orc_fem_diffu)(int nelem, int npoin, const int *connec, const real *Ngp, const real *dNgp, const real *He,
                     const real *gpvol, real Cp, real Pr, const real *rho, const real *u, const real *Tem,
                     const real *mu_fluid, const real *mu_e, const real *mu_sgs, real *Rmass, real *Rmom,
                     real *Rener, int nthreads)
{
    const int64_t np = npoin;
    memset(Rmass, 0, sizeof(real) * np);
    memset(Rmom, 0, sizeof(real) * 3 * np);
    memset(Rener, 0, sizeof(real) * np);
    const int atomic = nthreads > 1;
    const real c_rho = (real)1.0, c_ener = (real)1.0;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) if (atomic) schedule(static, 1024)
    for (int64_t e = 0; e < nelem; ++e) {
        int64_t ip[4];
        for (int a = 0; a < 4; ++a) ip[a] = connec[(int64_t)a * nelem + e] - 1;
        real Re_mass[4] = {0, 0, 0, 0}, Re_ener[4] = {0, 0, 0, 0}, Re_mom[4][3] = {{0}};
        for (int g = 0; g < 4; ++g) {
            real auxRho = 0, auxNu = 0, auxMu = 0, auxKappa = 0;
            for (int a = 0; a < 4; ++a) auxRho = auxRho + Ngp[g * 4 + a] * rho[ip[a]];
            for (int a = 0; a < 4; ++a) {
                const real me = mu_e[(int64_t)a * nelem + e], ms = mu_sgs[(int64_t)a * nelem + e];
                const real mf = mu_fluid[ip[a]];
                auxNu = auxNu + Ngp[g * 4 + a] * me * (c_rho / auxRho);
                auxMu = auxMu + Ngp[g * 4 + a] * (mf + auxRho * ms + me);
                auxKappa = auxKappa + Ngp[g * 4 + a] * (mf * (Cp / Pr) + c_ener * me / (real)0.4 + auxRho * ms / (real)0.9);
            }
            real gpcar[4][3];
            tet_gpcar(He, dNgp, e, g, gpcar);
            real gradRho[3] = {0, 0, 0}, gradT[3] = {0, 0, 0}, gradU[3][3] = {{0}};
            for (int id = 0; id < 3; ++id)
                for (int a = 0; a < 4; ++a) {
                    const int64_t p = ip[a];
                    gradRho[id] = gradRho[id] + gpcar[a][id] * rho[p];
                    gradT[id] = gradT[id] + gpcar[a][id] * Tem[p];
                    for (int jd = 0; jd < 3; ++jd) gradU[id][jd] = gradU[id][jd] + gpcar[a][id] * u[jd * np + p];
                }
            const real divU = gradU[0][0] + gradU[1][1] + gradU[2][2];
            real tau[3][3] = {{0}}, tauU[3] = {0, 0, 0};
            for (int id = 0; id < 3; ++id) {
                tau[id][id] = -((real)2.0 / (real)3.0 * divU);
                for (int jd = 0; jd < 3; ++jd) tau[id][jd] = tau[id][jd] + gradU[id][jd] + gradU[jd][id];
            }
            for (int jd = 0; jd < 3; ++jd) {
                real auxU = 0;
                for (int a = 0; a < 4; ++a) auxU = auxU + Ngp[g * 4 + a] * u[jd * np + ip[a]];
                for (int id = 0; id < 3; ++id) tauU[id] = tauU[id] + tau[id][jd] * auxU;
            }
            const real gv = gpvol[e * 4 + g];
            for (int id = 0; id < 3; ++id)
                for (int a = 0; a < 4; ++a) {
                    Re_mass[a] = Re_mass[a] + gv * auxNu * gpcar[a][id] * gradRho[id];
                    Re_ener[a] = Re_ener[a] + gv * gpcar[a][id] * (auxMu * tauU[id] + auxKappa * gradT[id]);
                    for (int jd = 0; jd < 3; ++jd)
                        Re_mom[a][id] = Re_mom[a][id] + gv * gpcar[a][jd] * auxMu * tau[id][jd];
                }
        }
        for (int a = 0; a < 4; ++a) {
            SCATTER(Rmass, ip[a], Re_mass[a], atomic);
            SCATTER(Rener, ip[a], Re_ener[a], atomic);
            for (int d = 0; d < 3; ++d) SCATTER(Rmom, d * np + ip[a], Re_mom[a][d], atomic);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Workload recipes: the structured shared-node mesh and the seeded node      */
/* fields of the benchmark configurations (no reference counterpart: the     */
/* reference meshes disconnected copies of one element, mod_mesh.f90:11-65,  */
/* and sets its own initial condition, main.f90:320-361).  Restated here so   */
/* that the CPU legs of the benchmark build their inputs without the product */
/* library; tests/test_oracle_kat.py checks them bit for bit against it.     */
/* FP32 build only (coordinates and fields are FP32).                        */
/* ------------------------------------------------------------------------- */
#if ORC_IS_FLOAT
/* splitmix64 -> uniform doubles in [0,1) -> Box-Muller normals. */
typedef struct { uint64_t s; } orc_rng;
static uint64_t rng_next(orc_rng *r)
{
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double rng_uniform(orc_rng *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static double rng_normal(orc_rng *r)
{
    double u1 = rng_uniform(r), u2 = rng_uniform(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
typedef struct { double k[3], phase, amp[3]; } orc_mode;
/* nmodes Fourier modes: integer wavevectors in [-kmax,kmax]^3 (not all zero),
 * uniform phases, per-component N(0, amp_sigma) amplitudes. */
static void make_modes(orc_rng *r, int nmodes, int kmax, double amp_sigma, orc_mode *m)
{
    for (int i = 0; i < nmodes; ++i) {
        do {
            for (int d = 0; d < 3; ++d) m[i].k[d] = (double)((int)(rng_uniform(r) * (2 * kmax + 1)) - kmax);
        } while (m[i].k[0] == 0 && m[i].k[1] == 0 && m[i].k[2] == 0);
        m[i].phase = 2.0 * M_PI * rng_uniform(r);
        for (int d = 0; d < 3; ++d) m[i].amp[d] = amp_sigma * rng_normal(r);
    }
}
static int sod_to_nat(int P, int s) { return s == 0 ? 0 : (s == 1 ? P : s - 1); }

/* nx*ny*nz hexes of the unit cube, lexicographic elements and nodes
 * ((nx P + 1)(ny P + 1)(nz P + 1) shared nodes); interior vertices of the
 * (n+1)^3 grid jittered by up to +-jitter*h per component (a draw per vertex
 * and component, seed-stable), high-order nodes placed at the GLL points of
 * the trilinear map of the element's vertices.  Returns 0 on success. */
int F(orc_mesh_structured)(int P, int nx, int ny, int nz, const int *AtoI, const int *AtoJ, const int *AtoK,
                           double jitter, uint64_t seed, int *connec, real *coord)
{
    const int Q = P + 1, n = Q * Q * Q;
    const int64_t NX = (int64_t)nx * P + 1, NY = (int64_t)ny * P + 1, NZ = (int64_t)nz * P + 1;
    const int64_t nelem = (int64_t)nx * ny * nz, npoin = NX * NY * NZ;
    int ni[ORC_MAXN], nj[ORC_MAXN], nk[ORC_MAXN];
    if (P < 1 || P > ORC_MAXP) return 1;
    for (int a = 0; a < n; ++a) {
        ni[a] = sod_to_nat(P, AtoI[a] - 1);
        nj[a] = sod_to_nat(P, AtoJ[a] - 1);
        nk[a] = sod_to_nat(P, AtoK[a] - 1);
    }
    for (int64_t e = 0; e < nelem; ++e) {
        const int64_t ex = e % nx, ey = (e / nx) % ny, ez = e / ((int64_t)nx * ny);
        for (int a = 0; a < n; ++a) {
            const int64_t I = ex * P + ni[a], J = ey * P + nj[a], K = ez * P + nk[a];
            connec[(int64_t)a * nelem + e] = (int)((K * NY + J) * NX + I + 1);
        }
    }
    if (!coord) return 0;
    const int64_t VX = nx + 1, VY = ny + 1, VZ = nz + 1;
    double *vx = (double *)malloc(sizeof(double) * (size_t)(VX * VY * VZ * 3));
    if (!vx) return 2;
    orc_rng rng = {seed ^ 0x6A09E667F3BCC908ull};
    const double h[3] = {1.0 / nx, 1.0 / ny, 1.0 / nz};
    for (int64_t k = 0; k < VZ; ++k)
        for (int64_t j = 0; j < VY; ++j)
            for (int64_t i = 0; i < VX; ++i) {
                const int64_t v = (k * VY + j) * VX + i;
                const int64_t idx[3] = {i, j, k}, lim[3] = {nx, ny, nz};
                for (int d = 0; d < 3; ++d) {
                    double x = (double)idx[d] * h[d];
                    const double r = 2.0 * rng_uniform(&rng) - 1.0;
                    if (idx[d] > 0 && idx[d] < lim[d]) x += jitter * h[d] * r;
                    vx[v * 3 + d] = x;
                }
            }
    double xg[ORC_MAXQ], vn[ORC_MAXQ];
    F(orc_zelegl)(P, xg, vn); /* FP32 build: Newton starts from the FP32 pi, as the tables */
    for (int64_t K = 0; K < NZ; ++K)
        for (int64_t J = 0; J < NY; ++J)
            for (int64_t I = 0; I < NX; ++I) {
                const int64_t ex = I / P < nx ? I / P : nx - 1, ey = J / P < ny ? J / P : ny - 1,
                              ez = K / P < nz ? K / P : nz - 1;
                const double sv[3] = {xg[I - ex * P], xg[J - ey * P], xg[K - ez * P]};
                double x[3] = {0, 0, 0};
                for (int c = 0; c < 8; ++c) {
                    const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
                    const double wgt = 0.125 * (1 + (cx ? sv[0] : -sv[0])) * (1 + (cy ? sv[1] : -sv[1])) *
                                       (1 + (cz ? sv[2] : -sv[2]));
                    const int64_t v = ((ez + cz) * VY + (ey + cy)) * VX + (ex + cx);
                    for (int d = 0; d < 3; ++d) x[d] += wgt * vx[v * 3 + d];
                }
                const int64_t p = (K * NY + J) * NX + I;
                for (int d = 0; d < 3; ++d) coord[d * npoin + p] = (real)x[d];
            }
    free(vx);
    return 0;
}

/* Seeded node fields: kind 0 (smooth) rho = 1 + 0.1 sin sin sin, pr = 1 +
 * 0.05 cos(2 pi x); kind 1 (shock-like) rho = 1 + 0.5 tanh((x-1/2)/0.02) + 5 %
 * Fourier noise, uniform pressure for Mach 0.8 at the velocity scale; u a sum of
 * nmodes Fourier modes per component (sigma 0.1 / 0.3); q = rho u; E =
 * pr/(gamma-1)/rho + |u|^2/2; Tem = pr/(rho Rgas); mu_fluid = 1.8e-5. */
int F(orc_fields_recipe)(int kind, int nmodes, uint64_t seed, int64_t npoin, const real *coord, real *rho, real *u,
                         real *q, real *pr, real *E, real *Tem, real *mu_fluid)
{
    const double gamma = 1.4, Rgas = 287.0, tpi = 2.0 * M_PI;
    const double uamp = kind == 0 ? 0.1 : 0.3;
    orc_mode um[3][64], noise[64];
    if ((kind != 0 && kind != 1) || nmodes < 1 || nmodes > 64) return 1;
    orc_rng rng = {seed};
    for (int c = 0; c < 3; ++c) make_modes(&rng, nmodes, 2, uamp, um[c]);
    make_modes(&rng, nmodes, 3, 1.0, noise);
    double noise_norm = 0.0;
    for (int i = 0; i < nmodes; ++i) noise_norm += fabs(noise[i].amp[0]);
    if (noise_norm <= 0.0) noise_norm = 1.0;
    const double urms = sqrt(3.0 * nmodes * 0.5) * uamp;
    const double p_shock = urms * urms / (gamma * 0.8 * 0.8);
    for (int64_t p = 0; p < npoin; ++p) {
        const double x = coord[p], y = coord[npoin + p], z = coord[2 * npoin + p];
        double uu[3];
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int i = 0; i < nmodes; ++i) {
                const orc_mode *m = &um[c][i];
                s += m->amp[0] * sin(tpi * (m->k[0] * x + m->k[1] * y + m->k[2] * z) + m->phase);
            }
            uu[c] = s;
        }
        double r, pp;
        if (kind == 0) {
            r = 1.0 + 0.1 * sin(tpi * x) * sin(tpi * y) * sin(tpi * z);
            pp = 1.0 + 0.05 * cos(tpi * x);
        } else {
            double nzv = 0.0;
            for (int i = 0; i < nmodes; ++i) {
                const orc_mode *m = &noise[i];
                nzv += m->amp[0] * sin(tpi * (m->k[0] * x + m->k[1] * y + m->k[2] * z) + m->phase);
            }
            r = 1.0 + 0.5 * tanh((x - 0.5) / 0.02) + 0.05 * nzv / noise_norm;
            pp = p_shock;
        }
        const float rf = (float)r, pf = (float)pp;
        const float uf[3] = {(float)uu[0], (float)uu[1], (float)uu[2]};
        rho[p] = rf;
        pr[p] = pf;
        for (int c = 0; c < 3; ++c) {
            u[c * npoin + p] = uf[c];
            q[c * npoin + p] = rf * uf[c];
        }
        const float ke = 0.5f * (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]);
        E[p] = pf / (float)(gamma - 1.0) / rf + ke;
        Tem[p] = pf / (rf * (float)Rgas);
        mu_fluid[p] = 1.8e-5f;
    }
    return 0;
}
#endif /* ORC_IS_FLOAT */
