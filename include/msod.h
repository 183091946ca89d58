/*
 * msod.h -- C ABI of the GB300-native miniSOD2D hex convection/diffusion path.
 *
 * Drop-in boundary for the two matrix-free spectral-element kernels of
 * miniSOD2D (src/kernels/sources/elem_convec.f90, elem_diffu.f90).  Every
 * entry point is plain C (extern "C", pointers, sizes, no C++ or torch types),
 * callable from Fortran through ISO_C_BINDING interfaces with scalars passed
 * by value.
 *
 * Conventions shared by all kernel entry points
 *  - Array arguments are DEVICE pointers (cudaMalloc'd, or msod_malloc'd)
 *    in the reference's Fortran column-major layouts (E = nelem, n = nnode =
 *    ngaus = (porder+1)^3, Q = porder+1, 0-based C index formulas):
 *        connec(nelem,nnode)          connec[a*E+e]            int32, 1-based node ids
 *        He(3,3,ngaus,nelem)          He[((e*n+g)*3+j)*3+i]    = He(i,j,g,e)
 *        gpvol(1,ngaus,nelem)         gpvol[e*n+g]
 *        dlxigp_ip(ngaus,3,Q)         dlxigp_ip[(ii*3+d)*n+g]
 *        invAtoIJK(Q,Q,Q)             invAtoIJK[(k*Q+j)*Q+i]   int32, 1-based
 *        gmshAtoI/J/K(nnode)          AtoI[a]                  int32, 1-based
 *        u,q(npoin,3), Rmom(npoin,3)  u[c*npoin+p]
 *        mu_e,mu_sgs(nelem,ngaus)     mu_e[g*E+e]
 *  - Outputs are intent(out): zeroed and then assembled inside the call.
 *  - Ngp, dNgp and xgp are accepted and ignored, as in the reference, whose
 *    hex kernels never read them (elem_convec.f90:198-205, elem_diffu.f90:10-16).
 *    They may be NULL.
 *  - dlxigp_ip must have the structure hex_highorder gives it
 *    (elem_hex.f90:23-45): dlxigp_ip(g,d,ii) depends on g only through node
 *    g's 1-D index in direction d.  The kernels read the 1-D derivative
 *    matrices from it at every call; msod_check_element_tables verifies the
 *    structure.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).  Kernel
 *    calls are asynchronous and stream-ordered; the host returns once the
 *    work is queued.
 *  - Concurrency: the library keeps per-device state (the element tables of
 *    the last call of each porder, the constant-bank derivative matrices of
 *    each porder, the work buffers of the estimators and the learned
 *    viscosity).  Kernel calls may overlap on different streams when calls of
 *    the same porder pass the same element tables (dlxigp_ip, invAtoIJK,
 *    gmshAtoI/J/K); calls of the viscosity estimators and the learned path must
 *    not overlap one another.
 *  - Return value: MSOD_OK (0) or one of the MSOD_ERR_* codes below.  No
 *    entry point exits or traps; msod_last_error_string() describes the last
 *    failure of the calling thread.
 */
#ifndef MSOD_H
#define MSOD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSOD_VERSION 100

#define MSOD_MAX_PORDER 8

#define MSOD_OK 0
#define MSOD_ERR_INVALID_ARG 1  /* a size, pointer or value outside its contract     */
#define MSOD_ERR_PORDER 2       /* porder has no compiled instantiation               */
#define MSOD_ERR_CUDA 3         /* a CUDA runtime call or kernel launch failed        */
#define MSOD_ERR_BAD_TABLES 4   /* element tables or connectivity failed validation   */
#define MSOD_ERR_NO_DEVICE 5    /* no usable CUDA device                              */
#define MSOD_ERR_INTERNAL 6
#define MSOD_ERR_UNSUPPORTED 7  /* a mode or option the library was not compiled with */
#define MSOD_ERR_BAD_MODEL 8    /* a network weight file is malformed or fails its CRC */

/* Per-element learned viscosity: 12 features -> 32 -> 32 -> 1 parameters. */
#define MSOD_MLP_NFEATURES 12
#define MSOD_MLP_NPARAMS 1505

/* Field recipes of msod_fields_recipe. */
#define MSOD_FIELDS_SMOOTH 0 /* rho = 1+0.1 sin sin sin, Fourier u (sigma 0.1), pr = 1+0.05 cos */
#define MSOD_FIELDS_SHOCK 1  /* tanh density jump + 5% noise, Fourier u (sigma 0.3), Mach 0.8   */

/* ---------------------------------------------------------------------------
 * Library state and errors
 * ------------------------------------------------------------------------- */

/* Select the CUDA device used by later calls of this host thread.  Replaces
 * the reference's implicit OpenACC device initialisation (main.f90:84-94
 * initialises MPI and the device on first use). */
int msod_init(int device);
/* Release library-owned device resources.  Safe to call more than once. */
int msod_finalize(void);
/* Text of the last error of the calling thread ("" if none). */
const char *msod_last_error_string(void);
int msod_version(void);
/* Checked mode (default off): every kernel call also validates its element
 * tables and connectivity on the device and synchronises the stream to report
 * MSOD_ERR_BAD_TABLES.  Meant for tests and debugging, not timing. */
int msod_set_checked(int enabled);

/* ---------------------------------------------------------------------------
 * Device memory (stand-ins for the reference's "!$acc enter data" regions,
 * main.f90:197-423, for hosts that hold device buffers as type(c_ptr))
 * ------------------------------------------------------------------------- */
int msod_malloc(void **ptr, size_t bytes);
int msod_free(void *ptr);
int msod_h2d(void *dst_device, const void *src_host, size_t bytes, void *stream);
int msod_d2h(void *dst_host, const void *src_device, size_t bytes, void *stream);
int msod_memset(void *dst_device, int value, size_t bytes, void *stream);
int msod_stream_synchronize(void *stream);

/* ---------------------------------------------------------------------------
 * Hot path: hex GLL convection and diffusion residuals
 * ------------------------------------------------------------------------- */

/* full_convec_ijk (elem_convec.f90:198-431).  Rmass, Rmom(npoin,3), Rener
 * receive the skew-symmetric split-form convection residual.  Rener follows
 * the complete definition of the split kernel (elem_convec.f90:674-832): the
 * fused reference kernel reads its energy-flux products without assigning
 * them (elem_convec.f90:247-250). */
int msod_convec_ijk(int porder, int nelem, int npoin, const int *connec, const float *Ngp,
                    const float *dNgp, const float *He, const float *gpvol, const float *dlxigp_ip,
                    const float *xgp, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                    const int *gmshAtoK, const float *u, const float *q, const float *rho,
                    const float *pr, const float *E, float *Rmass, float *Rmom, float *Rener,
                    void *stream);

/* full_convec_ijk_split (elem_convec.f90:433-836): same arguments and the same
 * residuals; served by the same fused single-pass kernel. */
int msod_convec_ijk_split(int porder, int nelem, int npoin, const int *connec, const float *Ngp,
                          const float *dNgp, const float *He, const float *gpvol,
                          const float *dlxigp_ip, const float *xgp, const int *invAtoIJK,
                          const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                          const float *u, const float *q, const float *rho, const float *pr,
                          const float *E, float *Rmass, float *Rmom, float *Rener, void *stream);

/* full_diffusion_ijk (elem_diffu.f90:10-197).  Viscous stress, heat flux and
 * artificial mass diffusion; nu_e and kappa_e are taken at the output node
 * (elem_diffu.f90:143-146); c_rho = c_ener = 1 (mod_numerical_params.f90:26-27). */
int msod_diffusion_ijk(int porder, int nelem, int npoin, const int *connec, const float *Ngp,
                       const float *dNgp, const float *He, const float *gpvol,
                       const float *dlxigp_ip, const float *xgp, const int *invAtoIJK,
                       const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK, float Cp,
                       float Pr, const float *rho, const float *u, const float *Tem,
                       const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass,
                       float *Rmom, float *Rener, void *stream);

/* Both calls of a step in one: what msod_convec_ijk followed by
 * msod_diffusion_ijk on the same geometry and state return (the reference
 * makes the two calls back to back on one mesh and state, main.f90:447,477).
 * The fields are the convection's (u, q, rho, press = its pr, E) and the diffusion's
 * (rho, u shared; Tem, mu_fluid, mu_e, mu_sgs); the residuals go to Rmass_c,
 * Rmom_c, Rener_c (convection) and Rmass_d, Rmom_d, Rener_d (diffusion),
 * which must be six distinct arrays.  At porder 4 one kernel computes both
 * from one gather per element group; other porders run the two kernels on
 * one set of tables.  While msod_set_mode selects another
 * form, the call makes the two drop-in calls in turn. */
int msod_convec_diffusion_ijk(int porder, int nelem, int npoin, const int *connec,
                              const float *Ngp, const float *dNgp, const float *He,
                              const float *gpvol, const float *dlxigp_ip, const float *xgp,
                              const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                              const int *gmshAtoK, float Cp, float Pr, const float *u,
                              const float *q, const float *rho, const float *press, const float *E,
                              const float *Tem, const float *mu_fluid, const float *mu_e,
                              const float *mu_sgs, float *Rmass_c, float *Rmom_c, float *Rener_c,
                              float *Rmass_d, float *Rmom_d, float *Rener_d, void *stream);

/* FP64 builds of the same kernels (the reference compiled with rp=8,
 * mod_constants.f90:5): the GPU-side FP64 oracle run. */
int msod_convec_ijk_f64(int porder, int nelem, int npoin, const int *connec, const double *He,
                        const double *gpvol, const double *dlxigp_ip, const int *invAtoIJK,
                        const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                        const double *u, const double *q, const double *rho, const double *pr,
                        const double *E, double *Rmass, double *Rmom, double *Rener, void *stream);
int msod_diffusion_ijk_f64(int porder, int nelem, int npoin, const int *connec, const double *He,
                           const double *gpvol, const double *dlxigp_ip, const int *invAtoIJK,
                           const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                           double Cp, double Pr, const double *rho, const double *u,
                           const double *Tem, const double *mu_fluid, const double *mu_e,
                           const double *mu_sgs, double *Rmass, double *Rmom, double *Rener,
                           void *stream);

/* No counterpart in the reference: mixed-precision form of full_convec_ijk.
 * FP32 fields and geometry as msod_convec_ijk; the 1-D derivative
 * contractions run on the tensor cores as hi + lo split FP16 (or BF16)
 * products with FP32 accumulation, after shifting each differentiated
 * product by its value at one node of the element and scaling it by a power
 * of two per element and product; the energy-flux assembly and the nodal
 * scatter-add run in FP64 and the residuals Rmass, Rmom(npoin,3), Rener are
 * FP64 arrays.  precision: MSOD_PREC_FP16 or MSOD_PREC_BF16.  porder 1..7. */
#define MSOD_PREC_FP16 0
#define MSOD_PREC_BF16 1
int msod_convec_ijk_mixed(int precision, int porder, int nelem, int npoin, const int *connec,
                          const float *He, const float *gpvol, const float *dlxigp_ip,
                          const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                          const int *gmshAtoK, const float *u, const float *q, const float *rho,
                          const float *pr, const float *E, double *Rmass, double *Rmom,
                          double *Rener, void *stream);

/* No counterpart in the reference: mixed-precision form of full_diffusion_ijk.
 * FP32 fields and geometry as msod_diffusion_ijk; the gradient and weak-
 * divergence contractions run on the tensor cores as hi + lo split FP16 (or
 * BF16) products with FP32 accumulation (gradient inputs shifted by their
 * value at one node of the element, every split field scaled by a power of
 * two per element); the energy-flux assembly (tau.u + kappa_e grad T) and the
 * nodal scatter-add run in FP64 and the residuals are FP64 arrays.  The _nu
 * form takes mu_e(e,a) = rho(a) nu_elem(e) as msod_diffusion_ijk_nu does.
 * precision: MSOD_PREC_FP16 or MSOD_PREC_BF16.  porder 1..7. */
int msod_diffusion_ijk_mixed(int precision, int porder, int nelem, int npoin, const int *connec,
                             const float *He, const float *gpvol, const float *dlxigp_ip,
                             const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                             const int *gmshAtoK, float Cp, float Pr, const float *rho,
                             const float *u, const float *Tem, const float *mu_fluid,
                             const float *mu_e, const float *mu_sgs, double *Rmass, double *Rmom,
                             double *Rener, void *stream);
int msod_diffusion_ijk_mixed_nu(int precision, int porder, int nelem, int npoin, const int *connec,
                                const float *He, const float *gpvol, const float *dlxigp_ip,
                                const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                                const int *gmshAtoK, float Cp, float Pr, const float *rho,
                                const float *u, const float *Tem, const float *mu_fluid,
                                const float *nu_elem, const float *mu_sgs, double *Rmass,
                                double *Rmom, double *Rener, void *stream);

/* Validate element tables and connectivity on the device (synchronous):
 * invAtoIJK is a permutation of 1..n consistent with gmshAtoI/J/K,
 * dlxigp_ip has the per-direction 1-D structure, every connec entry lies in
 * 1..npoin.  Returns MSOD_OK or MSOD_ERR_BAD_TABLES. */
int msod_check_element_tables(int porder, int nelem, int npoin, const int *connec,
                              const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI,
                              const int *gmshAtoJ, const int *gmshAtoK, void *stream);

/* No counterpart in the reference.  The same validation as
 * msod_check_element_tables, for callers that cannot let a library allocate
 * device memory (a Fortran host whose device memory belongs to the OpenACC
 * runtime's pool, a process under a capped or pre-reserved allocator, code
 * that finishes all allocations before capturing a CUDA graph): it calls no
 * cudaMalloc, cudaFree or allocating routine.  Its scratch is one 32-bit
 * status word in a static device array that stays resident on every GPU that
 * loads the library.  Limits are those of the kernel calls (porder <=
 * MSOD_MAX_PORDER, nelem*nnode < 2^31); larger sizes are rejected with
 * MSOD_ERR_PORDER / MSOD_ERR_INVALID_ARG.  Every call is synchronous: it
 * reads the verdict back to the host and synchronises the stream, so it must
 * not be made on a capturing stream or while a global-mode capture is under
 * way (its first call on a device also looks up the word's device address).
 * Calls share the word: calls that overlap on the GPU race and must be
 * serialised by the caller. */
int msod_check_element_tables_noalloc(int porder, int nelem, int npoin, const int *connec,
                                      const float *dlxigp_ip, const int *invAtoIJK,
                                      const int *gmshAtoI, const int *gmshAtoJ,
                                      const int *gmshAtoK, void *stream);

/* ---------------------------------------------------------------------------
 * Element setup (src/fem): metric on the device, tables and mesh on the host
 * ------------------------------------------------------------------------- */

/* elem_jacobian (jacobian_oper.f90:7-136) on the device: He = Je^-1 by
 * cofactors and gpvol = wgp*det(Je), Je = dNgp . coord.  Device pointers;
 * coord(npoin,3) is coord[d*npoin+p]; dNgp(3,nnode,ngaus) is
 * dNgp[(g*n+a)*3+d].  Rounding follows the reference: no fused
 * multiply-adds, sums in the reference's order. */
int msod_elem_jacobian(int porder, int nelem, int npoin, const int *connec, const float *coord,
                       const float *dNgp, const float *wgp, float *gpvol, float *He, void *stream);
int msod_elem_jacobian_f64(int porder, int nelem, int npoin, const int *connec,
                           const double *coord, const double *dNgp, const double *wgp,
                           double *gpvol, double *He, void *stream);

/* Host: per-element tables of main.f90:110-255 (invAtoIJK, AtoIJK, gmshAtoI/J/K,
 * xgp(ngaus,3), wgp, Ngp(ngaus,nnode), dNgp(3,nnode,ngaus),
 * dlxigp_ip(ngaus,3,porder+1)), all host arrays sized by porder. */
int msod_fem_element_tables(int porder, int *invAtoIJK, int *AtoIJK, int *AtoI, int *AtoJ,
                            int *AtoK, float *xgp, float *wgp, float *Ngp, float *dNgp,
                            float *dlxigp_ip);
int msod_fem_element_tables_f64(int porder, int *invAtoIJK, int *AtoIJK, int *AtoI, int *AtoJ,
                                int *AtoK, double *xgp, double *wgp, double *Ngp, double *dNgp,
                                double *dlxigp_ip);

/* Host: structured nx*ny*nz hex mesh of the unit cube with shared nodes,
 * lexicographic node and element numbering, GLL-spaced high-order nodes placed
 * by the trilinear map of the element's corner vertices; interior vertices
 * jittered by up to +-jitter*h per component (seeded).  connec(nelem,nnode)
 * host array (1-based); coord(npoin,3) host array or NULL.  npoin =
 * (nx*porder+1)(ny*porder+1)(nz*porder+1).  Replaces create_mesh
 * (mod_mesh.f90:11-65) for the scaled workloads. */
int msod_mesh_structured(int porder, int nx, int ny, int nz, const int *AtoI, const int *AtoJ,
                         const int *AtoK, double jitter, uint64_t seed, int *connec,
                         float *coord);

/* Host: the reference driver's own case.  create_mesh (mod_mesh.f90:11-65):
 * disconnected elements, connec(e,a) = (e-1)*nnode + a, element e = xyzBase
 * (xyzBase[d*nnode+a]; the driver passes xgp) shifted by 3(e-1) along every
 * axis; npoin = nelem*nnode; coord may be NULL.  msod_reference_ic: the driver's
 * initial condition (main.f90:320-361), FP32, mu_e = mu_sgs = mu_fluid = 1. */
int msod_mesh_disconnected(int porder, int nelem, const float *xyzBase, int *connec, float *coord);
int msod_reference_ic(int porder, int nelem, int64_t npoin, const int *connec, float *u, float *q,
                      float *rho, float *pr, float *E, float *Tem, float *mu_fluid, float *mu_e,
                      float *mu_sgs);

/* Host: seeded node fields (FP32) for recipe `kind` with `nmodes` Fourier
 * modes per velocity component: rho, u(npoin,3), q = rho u, pr,
 * E = pr/(gamma-1)/rho + |u|^2/2, Tem = pr/(rho Rgas), mu_fluid = 1.8e-5
 * (gamma = 1.4, Rgas = 287, as main.f90:52).  Replaces the reference's
 * initial condition (main.f90:320-361). */
int msod_fields_recipe(int kind, int nmodes, uint64_t seed, int64_t npoin, const float *coord,
                       float *rho, float *u, float *q, float *pr, float *E, float *Tem,
                       float *mu_fluid);

/* ---------------------------------------------------------------------------
 * Linear tetrahedra (TET04): the reference driver's other timed kernels
 * (main.f90:465-500).  4 nodes = 4 Gauss points per element; device arrays
 * (E = nelem):
 *     connec(nelem,4)     connec[a*E+e]           int32, 1-based
 *     Ngp(4,4)            Ngp[c*4+r] = Ngp(r,c)   (the driver's Ngp(igaus,inode))
 *     dNgp(3,4,4)         dNgp[(g*4+a)*3+d]
 *     He(3,3,4,nelem)     He[((e*4+g)*3+j)*3+i]
 *     gpvol(1,4,nelem)    gpvol[e*4+g]
 *     mu_e,mu_sgs(nelem,4) mu_e[a*E+e]
 * Outputs are intent(out).  Elements whose nodes are 4k..4k+3 (the driver's
 * tet mesh) are assembled with 16-byte vector reductions when the residual
 * arrays are 16-byte aligned and npoin is a multiple of 4.
 * ------------------------------------------------------------------------- */

/* fem_convec (elem_convec.f90:839-948): split-form convection on TET04
 * elements, Ngp read as Ngp(igaus,inode). */
int msod_fem_convec(int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp,
                    const float *He, const float *gpvol, const float *u, const float *q, const float *rho,
                    const float *pr, const float *E, float *Rmass, float *Rmom, float *Rener, void *stream);
int msod_fem_convec_f64(int nelem, int npoin, const int *connec, const double *Ngp, const double *dNgp,
                        const double *He, const double *gpvol, const double *u, const double *q,
                        const double *rho, const double *pr, const double *E, double *Rmass, double *Rmom,
                        double *Rener, void *stream);

/* fem_diffu (elem_diffu.f90:199-317): viscous, heat and artificial mass
 * diffusion on TET04 elements.  As in the reference it reads Ngp(inode,igaus)
 * (the transpose of fem_convec's reading), interpolates mu and kappa to the
 * Gauss points with kappa = mu_fluid Cp/Pr + mu_e/0.4 + rho mu_sgs/0.9, and
 * applies mu to the whole stress including its -2/3 div u part. */
int msod_fem_diffu(int nelem, int npoin, const int *connec, const float *Ngp, const float *dNgp,
                   const float *He, const float *gpvol, float Cp, float Pr, const float *rho, const float *u,
                   const float *Tem, const float *mu_fluid, const float *mu_e, const float *mu_sgs,
                   float *Rmass, float *Rmom, float *Rener, void *stream);
int msod_fem_diffu_f64(int nelem, int npoin, const int *connec, const double *Ngp, const double *dNgp,
                       const double *He, const double *gpvol, double Cp, double Pr, const double *rho,
                       const double *u, const double *Tem, const double *mu_fluid, const double *mu_e,
                       const double *mu_sgs, double *Rmass, double *Rmom, double *Rener, void *stream);

/* tet_jacobian (jacobian_oper.f90:138-267) on the device, rounded like
 * msod_elem_jacobian. */
int msod_tet_jacobian(int nelem, int npoin, const int *connec, const float *coord, const float *dNgp,
                      const float *wgp, float *gpvol, float *He, void *stream);
int msod_tet_jacobian_f64(int nelem, int npoin, const int *connec, const double *coord,
                          const double *dNgp, const double *wgp, double *gpvol, double *He, void *stream);

/* Host: tet_4points + tet_04 tables as the driver fills them (main.f90:377-383):
 * Ngp[16], dNgp[48], xgp[12] (xgp[d*4+g]), wgp[4]. */
int msod_tet_element_tables(float *Ngp, float *dNgp, float *xgp, float *wgp);
int msod_tet_element_tables_f64(double *Ngp, double *dNgp, double *xgp, double *wgp);

/* Host: the driver's disconnected tet mesh (gen_tet_mesh, mod_mesh.f90:71-126):
 * npoin = 4 nelem, connec(e,a) = 4(e-1)+a, element e = xyzBase(4,3)
 * (xyzBase[d*4+a]) shifted by 3(e-1) along every axis.  coord(npoin,3) may be
 * NULL. */
int msod_tet_mesh_disconnected(int nelem, const float *xyzBase, int *connec, float *coord);

/* ---------------------------------------------------------------------------
 * Artificial viscosity mu_e: plain entropy-viscosity estimator and the
 * learned per-element estimator.  No counterpart in the reference, which
 * consumes mu_e(nelem,ngaus) (elem_diffu.f90:19) without computing it; the
 * knobs follow mod_numerical_params.f90:22-28 (ce = 0.1, cmax = 0.5,
 * normalised entropy).
 * ------------------------------------------------------------------------- */

/* Entropy-viscosity estimator (Guermond, Pasquetti & Popov, JCP 230 (2011)):
 * eta = rho/(gamma-1) log(p/rho^gamma), R = div(eta u) - eta div u - u.grad eta,
 * per element nu = min(cmax h max(|u|+c), ce h^2 max|R| / ||eta - mean eta||_inf)
 * with h = (sum gpvol)^(1/3)/porder; mu_e(e,a) = rho(a) nu(e) in the reference's
 * mu_e(nelem,ngaus) layout.  nu_elem / numax_elem (nelem each) may be NULL,
 * and mu_e may be NULL when nu_elem is given.
 * porder 1..7. */
int msod_entropy_viscosity(int porder, int nelem, int npoin, const int *connec, const float *He,
                           const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                           const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                           const float *rho, const float *u, const float *pr, float gamma, float ce,
                           float cmax, int normalise, float *mu_e, float *nu_elem,
                           float *numax_elem, void *stream);

/* The 12 element features of the learned estimator (feat[e*12+k]) and the
 * element's first-order viscosity nu_max.  p_or_T is the pressure (Rgas = 0)
 * or the temperature with p = rho Rgas T. */
int msod_mlp_features(int porder, int nelem, int npoin, const int *connec, const float *He,
                      const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                      const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK,
                      const float *rho, const float *u, const float *p_or_T, float Rgas, float gamma,
                      float cmax, float *feat, float *numax_elem, void *stream);

/* Network handle: device weights (FP32 master, FP16 deployed copy), Adam
 * state and the feature normalisation (mean, 1/std, training min, max). */
typedef struct msod_mlp msod_mlp;
int msod_mlp_create(msod_mlp **out, uint64_t seed);
int msod_mlp_destroy(msod_mlp *m);
/* Adam over nsamples device pairs (feat[nsamples*12], target[nsamples] =
 * y = nu/nu_max of the plain estimator).  The network's output s is a number
 * of decades (y = 10^-s); the loss is the mean-squared error of s against
 * -log10(max(target, 1e-12)), each sample weighted by weight[i] (a device
 * array; NULL: all 1).  Batch samples are drawn per step from `seed`; the
 * feature normalisation and training ranges are set from the training data.
 * loss_host (steps floats) may be NULL.  Synchronous. */
int msod_mlp_train(msod_mlp *m, const float *feat, const float *target, const float *weight, int nsamples,
                   int steps, int batch, float lr, uint64_t seed, float *loss_host, void *stream);
/* Batch gradient of the (weighted) loss at the current weights (for gradient checks). */
int msod_mlp_gradient(msod_mlp *m, const float *feat, const float *target, const float *weight,
                      const int *idx, int batch, float *grad_host, void *stream);
int msod_mlp_get_params(const msod_mlp *m, float *params_host, float *norm_host);
int msod_mlp_set_params(msod_mlp *m, const float *params_host, const float *norm_host);
/* y = 10^-s in (0, 1] from the network output s >= 0, nu = y*numax (if numax
 * given), flag = 1 where a feature lies outside the training range. */
int msod_mlp_predict(const msod_mlp *m, const float *feat, const float *numax_elem, int nelem, float *y,
                     float *nu_elem, int *flag, void *stream);
/* Weight file with a CRC-32; a failed check returns MSOD_ERR_BAD_MODEL. */
int msod_mlp_save(const msod_mlp *m, const char *path);
int msod_mlp_load(msod_mlp *m, const char *path);
/* nu per element from the network (evaluated inside the features kernel,
 * one warp per element, with the bits of msod_mlp_predict); elements flagged
 * out of range take the plain estimator's value (computed for those
 * elements only). */
int msod_learned_viscosity(const msod_mlp *m, int porder, int nelem, int npoin, const int *connec,
                           const float *He, const float *gpvol, const float *dlxigp_ip,
                           const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                           const int *gmshAtoK, const float *rho, const float *u, const float *p_or_T,
                           float Rgas, float gamma, float ce, float cmax, float *nu_elem, int *flag,
                           void *stream);
/* No counterpart in the reference: full_diffusion_ijk with the artificial
 * viscosity from the network -- msod_learned_viscosity followed by
 * msod_diffusion_ijk_nu on the same stream.  The features take the pressure
 * p_or_T (Rgas = 0) or p = rho Rgas T from the temperature p_or_T (Rgas > 0).
 * Elements whose features leave the network's training range take the plain
 * estimator's value (computed for those elements only).  nu_elem and flag
 * (nelem each, optional) receive the viscosity used and the fallback flags. */
int msod_diffusion_ijk_learned(const msod_mlp *m, int porder, int nelem, int npoin, const int *connec,
                               const float *He, const float *gpvol, const float *dlxigp_ip,
                               const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                               const int *gmshAtoK, float Cp, float Pr, const float *rho,
                               const float *u, const float *Tem, const float *mu_fluid,
                               const float *mu_sgs, const float *p_or_T, float Rgas, float gamma,
                               float ce, float cmax, float *Rmass, float *Rmom, float *Rener,
                               float *nu_elem, int *flag, void *stream);
/* full_diffusion_ijk with mu_e(e,a) = rho(a) nu_elem(e): one viscosity value
 * per element instead of the mu_e(nelem,ngaus) array. */
int msod_diffusion_ijk_nu(int porder, int nelem, int npoin, const int *connec, const float *He,
                          const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                          const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK, float Cp,
                          float Pr, const float *rho, const float *u, const float *Tem,
                          const float *mu_fluid, const float *nu_elem, const float *mu_sgs,
                          float *Rmass, float *Rmom, float *Rener, void *stream);

/* No counterpart in the reference, whose form is fixed at compile time: the
 * form that every later msod_convec_ijk / msod_convec_ijk_split /
 * msod_diffusion_ijk call of the process computes, so that a driver keeps its
 * two calls and switches precision and artificial viscosity at run time.
 *   precision  MSOD_PREC_FP32: the plain kernels (default); MSOD_PREC_FP16 /
 *              MSOD_PREC_BF16: the tensor-core kernels (porder <= 7) write
 *              FP64 residuals into library buffers, converted into the
 *              caller's FP32 arrays.
 *   mu_e_mode  MSOD_MU_E_GIVEN: the caller's mu_e (default); MSOD_MU_E_PLAIN:
 *              the entropy-viscosity estimator; MSOD_MU_E_LEARNED: the
 *              network `mlp` (msod_learned_viscosity) with the estimator
 *              as per-element fallback.  Both ignore the mu_e
 *              argument and use p = rho Rgas Tem, gamma = 1.4, Rgas = 287
 *              (main.f90:52), ce = 0.1, cmax = 0.5 (mod_numerical_params.f90:23-24).
 * The network is kept by reference and must outlive its use.  The library
 * buffers are per device and grow with cudaMalloc; calls that overlap on the
 * GPU race on them. */
#define MSOD_PREC_FP32 2
#define MSOD_MU_E_GIVEN 0
#define MSOD_MU_E_PLAIN 1
#define MSOD_MU_E_LEARNED 2
int msod_set_mode(int precision, int mu_e_mode, const msod_mlp *mlp);
int msod_get_mode(int *precision, int *mu_e_mode);

/* ---------------------------------------------------------------------------
 * Time integration around the two residual calls.  The reference names it
 * (flag_rk_order = 4, flag_solver_type = 1 lumped mass,
 * mod_numerical_params.f90:8,20) but contains none of it.
 * ------------------------------------------------------------------------- */

/* Lumped (diagonal) mass matrix of the GLL quadrature: Ml(p) = sum of
 * gpvol(e, g) over the element points g at node p.  Ml (npoin) is written
 * (intent(out)).  Device pointers. */
int msod_lumped_mass(int porder, int nelem, int npoin, const int *connec, const float *gpvol,
                     float *Ml, void *stream);
/* Bytes of device workspace msod_rk4_step needs for npoin nodes (26 floats
 * per node). */
int msod_rk4_workspace_bytes(int npoin, size_t *bytes);
/* One classical four-stage Runge-Kutta step of
 *   dU/dt = -Ml^-1 (R_conv(U) + R_diff(U)),  U = (rho, q = rho u, rhoE),
 * updating rho (npoin), q (3*npoin, q[c*npoin+p]) and rhoE (npoin) in place.
 * Each stage derives u = q/rho, E = rhoE/rho (the specific energy the
 * convection takes), pr = (gamma-1)(rhoE - rho|u|^2/2) and
 * Tem = pr/(rho Rgas), and calls msod_convec_diffusion_ijk (in the form
 * msod_set_mode selects) with mu_fluid (npoin), mu_e and mu_sgs
 * (nelem*ngaus) as given.  Ml from msod_lumped_mass; workspace: device memory
 * of at least msod_rk4_workspace_bytes, 4-byte aligned.  Asynchronous on the
 * stream. */
int msod_rk4_step(int porder, int nelem, int npoin, const int *connec, const float *He,
                  const float *gpvol, const float *dlxigp_ip, const int *invAtoIJK,
                  const int *gmshAtoI, const int *gmshAtoJ, const int *gmshAtoK, float Cp, float Pr,
                  float gamma, float Rgas, const float *Ml, const float *mu_fluid,
                  const float *mu_e, const float *mu_sgs, float dt, float *rho, float *q,
                  float *rhoE, void *workspace, size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MSOD_H */
