/*
 * fcgpu.h -- C ABI of libfcgpu.so, the GB300 (sm_103a) implementation of
 * freeCappuccino's pressure-correction path.
 *
 * The reference exposes this path as Fortran subroutines working on module-global
 * arrays (modules `geometry`, `sparse_matrix`, `variables`).  This library keeps the
 * same arrays, index conventions and call sequence, but passes every array
 * explicitly:
 *   - index values are 1-based int32 exactly as the Fortran arrays hold them
 *     (owner, neighbour, ioffset, ja, diag, slot maps);
 *   - reals are IEEE binary64 (`real(dp)`); cell gradients are dPhidxi(3,numCells),
 *     component fastest;
 *   - a field of "numTotal" length holds the numCells cell values followed by one
 *     value per boundary face, grouped by boundary type in the order inlet, outlet,
 *     symmetry, wall, pressure outlet (mesh_geometry_and_topology.f90:593-605).
 * Every pointer argument may point to host memory (pageable or pinned) or to device
 * memory on the context's GPU; the library tells them apart and copies host arrays
 * in and out inside the call.  Device arrays are used in place.
 *
 * Every function returns FCG_OK (0) or a negative status; fcg_last_error() gives a
 * one-line description.  A context is not thread-safe (the reference is serial).
 * The library has no CPU fallback: without a usable sm_103a device every compute
 * entry point returns FCG_ERR_CUDA.
 */
#ifndef FCGPU_H
#define FCGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define FCG_ABI_VERSION 2  /* 2: fcg_mesh_desc gained the O-C pair fields */

/* Status codes. */
#define FCG_OK 0
#define FCG_ERR_ARG (-1)         /* bad argument: NULL pointer, size out of range */
#define FCG_ERR_STATE (-2)       /* call order: e.g. a solve before fcg_bind_mesh */
#define FCG_ERR_CUDA (-3)        /* CUDA runtime error or no usable device */
#define FCG_ERR_INDEX (-4)       /* owner/neighbour/boundary index out of range or duplicate face */
#define FCG_ERR_PIVOT (-5)       /* zero or non-finite pivot in a DIC/DILU factor */
#define FCG_ERR_STALL (-6)       /* a preconditioned iteration stalled (learned FCG) */
#define FCG_ERR_TIMEOUT (-7)     /* a bounded device-side wait gave up */
#define FCG_ERR_UNSUPPORTED (-8) /* an entry point that does not take O-C grid cuts */
#define FCG_ERR_NOMEM (-9)       /* device allocation failed */
#define FCG_ERR_NONFINITE (-10)  /* NaN/Inf reached a reduction */

typedef struct fcg_context fcg_context;

int fcg_abi_version(void);
const char *fcg_status_string(int status);
const char *fcg_last_error(const fcg_context *ctx);

/* Creates a context on CUDA device `device` (the module-global state of the
 * reference becomes per-context state). */
int fcg_create(fcg_context **ctx, int device);
int fcg_destroy(fcg_context *ctx);
/* All later work of the context is queued on this stream (cudaStream_t; NULL = the
 * context's own stream), ordered after the work already queued on the previous one.
 * Device arrays passed to the library must be ready on this stream: the library does
 * not wait for other streams. */
int fcg_set_stream(fcg_context *ctx, void *cuda_stream);
int fcg_synchronize(fcg_context *ctx);

/* ---------------------------------------------------------------------------
 * Mesh (module `geometry`, src/mesh_geometry_and_topology.f90:12-98).
 * ------------------------------------------------------------------------- */
typedef struct fcg_mesh_desc {
  int numCells, numFaces, numInnerFaces;
  /* Boundary faces per type and the 0-based start of each type's face range as the
   * boundary file gives it (face index iface = start + i, i = 1..count). */
  int ninl, nout, nsym, nwal, npru;
  int iInletFacesStart, iOutletFacesStart, iSymmetryFacesStart, iWallFacesStart,
      iPressOutletFacesStart;
  /* O-C grid cut and cyclic face pairs after `noc = noc + ncyc`
   * (mesh_geometry_and_topology.f90:1163); 0 for none.  See the fields at the end. */
  int noc;
  const int *owner;                             /* [numFaces], 1-based */
  const int *neighbour;                         /* [numInnerFaces], 1-based */
  const double *arx, *ary, *arz, *xf, *yf, *zf; /* [numFaces] */
  const double *xc, *yc, *zc, *vol;             /* [numCells] */
  const double *facint;                         /* [numInnerFaces] */
  /* The O-C pairs ('domain' and 'cyclic' patches, mesh_geometry_and_topology.f90:
   * 453-462, 800-845), read when noc > 0: pair i couples the owner of boundary face
   * ijlFace[i] (ijl) to the owner of its friend face ijrFace[i] (ijr), both 1-based;
   * the last ncyc pairs are cyclic (interpolation factor 1/2, :1149).  The O-C loops
   * take the area of pair i from face iOCFacesStart + i (0-based start, i 1-based;
   * fvm_laplacian.f90:70): the start of the first 'domain' patch, 0 without one.  With noc > 0 a matrix `a` holds nnz + 2 noc values: the
   * CSR values, then ar(1..noc), then al(1..noc) (module sparse_matrix's al, ar), and
   * a mass-flux array flmass holds numInnerFaces + noc values: the inner faces', then
   * the pairs' fmoc(1..noc) (module variables' fmoc).  The SIMPLE and PISO pressure-
   * correction paths take the pairs: fcg_laplacian, fcg_facefluxmass, fcg_fluxmc,
   * fcg_flux_correct, fcg_continuity_errors, fcg_correct_fields, fcg_correct_bc_velocity,
   * fcg_facefluxmass_piso, fcg_piso_hbya, fcg_adjust_mass_flow,
   * fcg_set_reference_pressure, fcg_correct_velocity_piso, the momentum assembly
   * fcg_calcuvw, fcg_grad, fcg_grad_lsq_matrix, fcg_bpres, fcg_dpcg, fcg_iccg,
   * fcg_bicgstab and fcg_spmv; the mixed, multi-RHS, batched and learned solvers (no
   * reference counterpart) return FCG_ERR_UNSUPPORTED on such a mesh. */
  int ncyc;
  int iOCFacesStart;
  const int *ijlFace, *ijrFace; /* [noc] */
} fcg_mesh_desc;

/* Uploads the mesh and builds, once, everything the kernels need: the CSR pattern
 * of create_CSR_matrix_from_mesh_data (src/sparse_matrix.f90:42-172), the sliced
 * ELL copy used by the solvers, the cell->face incidence lists that keep the
 * reference's face-loop summation order, and the level schedules of the
 * triangular sweeps.  Replaces: mesh_geometry (mesh_geometry_and_topology.f90:310)
 * as a consumer of its arrays, and create_CSR_matrix_from_mesh_data. */
int fcg_bind_mesh(fcg_context *ctx, const fcg_mesh_desc *mesh);
int fcg_mesh_sizes(const fcg_context *ctx, int *numCells, int *numFaces, int *numInnerFaces,
                   long long *nnz, int *numTotal);

/* CSR arrays of create_CSR_matrix_from_mesh_data (sparse_matrix.f90:42-172),
 * bit-exact, 1-based: ioffset[numCells+1], ja[nnz], diag[numCells], and the face
 * slot maps icell_jcell_csr_value_index / jcell_icell_csr_value_index
 * [numInnerFaces] (sparse_matrix.f90:153-167).  Any pointer may be NULL. */
int fcg_create_csr(fcg_context *ctx, int *ioffset, int *ja, int *diag, int *slot_pn,
                   int *slot_np);

/* A 64-bit FNV-1a digest over every topology array fcg_bind_mesh bound to the device
 * (CSR, slot maps, transpose positions, incidence lists, sliced ELL copy, level
 * schedules).  Two contexts on the same mesh agree exactly when their topologies do:
 * the GPU construction (the default) against FCG_TOPOLOGY=host. */
int fcg_topology_digest(fcg_context *ctx, unsigned long long *digest);

/* Host-only form of the same construction (no context, no GPU): the CSR arrays of
 * create_CSR_matrix_from_mesh_data for an owner/neighbour list (sparse_matrix.f90:
 * 42-172), 1-based, with nnz = numCells + 2*numInnerFaces. */
int fcg_csr_build(int numCells, int numInnerFaces, const int *owner, const int *neighbour,
                  int *ioffset, int *ja, int *diag, int *slot_pn, int *slot_np);

/* The same construction by kernels on ctx's device and stream (the context need not be
 * bound to a mesh); arrays host or device, results identical to fcg_csr_build.  Bad
 * indices and two faces on one cell pair give FCG_ERR_INDEX. */
int fcg_csr_build_gpu(fcg_context *ctx, int numCells, int numInnerFaces, const int *owner,
                      const int *neighbour, int *ioffset, int *ja, int *diag, int *slot_pn,
                      int *slot_np);

/* The geometry pass of mesh_geometry (mesh_geometry_and_topology.f90:859-1079) by kernels
 * on ctx's device: face area vectors by triangle fans from the first node, arithmetic-mean
 * face centres, divergence-theorem volumes, Nurnberg centroids and the interpolation
 * factor through the plane of the first three face nodes, bit-identical to the host form
 * fcg_mesh_geometry (fcgpu_meshgen.h).  x, y, z [numNodes]; face_ptr[numFaces+1]
 * (0-based offsets); face_nodes (1-based); owner[numFaces], neighbour[numInnerFaces]
 * 1-based; outputs arx..zf [numFaces], xc, yc, zc, vol [numCells], facint
 * [numInnerFaces].  Arrays host or device. */
int fcg_mesh_geometry_gpu(fcg_context *ctx, int numNodes, const double *x, const double *y,
                          const double *z, int numCells, int numFaces, int numInnerFaces,
                          const int *face_ptr, const int *face_nodes, const int *owner,
                          const int *neighbour, double *arx, double *ary, double *arz,
                          double *xf, double *yf, double *zf, double *xc, double *yc,
                          double *zc, double *vol, double *facint);

/* ---------------------------------------------------------------------------
 * Assembly (face loops into the CSR values a[nnz]).
 * ------------------------------------------------------------------------- */

/* laplacian(mu,phi), src/fvm_laplacian.f90:1-163: a = 0, then inner-face
 * coefficients (mu[numCells], linear interpolation by facint), then wall faces,
 * which also add a(diag)*phi(ijb) to su.  phi[numTotal] (only wall slots read),
 * a[nnz] out, su[numCells] in/out. */
int fcg_laplacian(fcg_context *ctx, const double *mu, const double *phi, double *a, double *su);

/* Flow fields read by facefluxmass (module `variables`). */
typedef struct fcg_flow_fields {
  const double *u, *v, *w, *p;                 /* [numTotal] */
  const double *dUdxi, *dVdxi, *dWdxi, *dPdxi; /* [3*numCells] */
  const double *apu, *apv, *apw;               /* [numCells] */
  const double *den;                           /* [numTotal] */
} fcg_flow_fields;

/* Pressure-correction assembly of calcp (calcp-multiple_correction_SIMPLE.f90:34-77)
 * with facefluxmass (facefluxmass.f90:34-199): a = 0, su = 0, then per inner face
 * the p' coefficients, the Rhie-Chow mass flux flmass[numInnerFaces] and its
 * divergence into su. */
int fcg_facefluxmass(fcg_context *ctx, const fcg_flow_fields *f, double *a, double *su,
                     double *flmass);

/* Non-orthogonal corrector source of calcp (calcp-multiple_correction_SIMPLE.f90:
 * 193-206) with fluxmc (facefluxmass.f90:520-607): su = 0, then per inner face
 * flmass += fmcor, su(P) -= fmcor, su(N) += fmcor. */
int fcg_fluxmc(fcg_context *ctx, const double *dPdxi, const double *apu, const double *den,
               double *su, double *flmass);

/* Mass-flux correction by the pressure correction, calcp-multiple_correction_SIMPLE.f90:
 * 159-171: flmass(f) += a(icell_jcell_csr_value_index(f)) * (pp(N) - pp(P)) over the
 * inner faces.  a[nnz], pp[numTotal], flmass[numInnerFaces] in/out. */
int fcg_flux_correct(fcg_context *ctx, const double *a, const double *pp, double *flmass);

/* Velocity and pressure correction, calcp-multiple_correction_SIMPLE.f90:147,184-189:
 * ppref = pp(pRefCell) (1-based); u -= dPdxi(1,:)*vol*apu, v -= dPdxi(2,:)*vol*apv,
 * w -= dPdxi(3,:)*vol*apw, p += urf*(pp - ppref) over the cells.  u, v, w, p, pp of
 * numTotal length (only the cell part is written), dPdxi(3,numCells), ap*[numCells]. */
int fcg_correct_fields(fcg_context *ctx, const double *dPdxi, const double *apu,
                       const double *apv, const double *apw, const double *pp, double urf,
                       int pRefCell, double *u, double *v, double *w, double *p);

/* correctBoundaryConditionsVelocity.f90:1-80: outlet slots of u, v, w take their cell's
 * value, fmo(i) = den(ijp) (u,v,w)(ijb).S, the outflow is scaled to flomas
 * (fac = flomas/(sum fmo + small), fmo and the outlet velocities times fac), symmetry
 * slots take the cell velocity minus ((u,v,w)(ijp).S) S with S the area vector (as the
 * reference does).  u, v, w, den [numTotal]; fmo[nout] out (may be NULL without outlets). */
int fcg_correct_bc_velocity(fcg_context *ctx, const double *den, double flomas, double *u,
                            double *v, double *w, double *fmo);

/* continuityErrors.h:1-52: res(numCells) = the divergence of the mass fluxes -- per inner
 * face res(ijp) -= flmass(ijp), res(ijn) += flmass(ijp), with flmass indexed by the owner
 * cell as the reference does (so numCells <= numInnerFaces is required, FCG_ERR_INDEX
 * otherwise) -- minus fmi over inlet and fmo over outlet faces; *sum_local = sum|res|,
 * *global = sum res (deterministic order; res may be NULL). */
int fcg_continuity_errors(fcg_context *ctx, const double *flmass, const double *fmi,
                          const double *fmo, double *res, double *sum_local, double *global);

/* ---------------------------------------------------------------------------
 * Momentum assembly (calcuvw.f90:48-438): the producer of the u, v, w systems.
 * ------------------------------------------------------------------------- */

/* Face-value schemes of face_value (interpolation.f90:20-60), in the order of its flags
 * lcds, lcdsc, lcds_flnt, l2nd_flnt, lmuscl_flnt, flux_limiter; MUSCL is also its default. */
#define FCG_CONV_CDS 0
#define FCG_CONV_CDS_CORRECTED 1
#define FCG_CONV_CENTRAL 2
#define FCG_CONV_SECOND_UPWIND 3
#define FCG_CONV_MUSCL 4
#define FCG_CONV_FLUX_LIMITER 5
/* Limiters of face_value_2nd_upwind_flux_limiter (interpolation.f90:364-389); UDS is its
 * psi = 1 branch. */
#define FCG_LIM_SMART 0
#define FCG_LIM_AVL 1
#define FCG_LIM_MUSCL 2
#define FCG_LIM_UMIST 3
#define FCG_LIM_KOREN 4
#define FCG_LIM_CHARM 5
#define FCG_LIM_OSPRE 6
#define FCG_LIM_UDS 7

/* Parameters calcuvw reads (modules_allocatable.f90:40-135).  urfr = 1/urf and urfm =
 * 1 - urf per component (u, v, w) as the reference stores them; gds = gds(iu). */
typedef struct fcg_uvw_params {
  int scheme, limiter;
  double gds, viscos;
  double urfr[3], urfm[3];
  int bdf, cn;
  double timestep, btime;
  int const_mflux;
  double gradPcmf;
  int buoyancy, boussinesq;
  double beta, densit, tref, gravx, gravy, gravz;
} fcg_uvw_params;

/* Fields calcuvw reads.  u, v, w, p, vis [numTotal]; den, t, uo..woo [numCells] (t, uo..woo
 * may be NULL where the parameters do not read them); dUdxi..dPdxi (3,numCells);
 * flmass[numInnerFaces]; fmi[ninl], fmo[nout]. */
typedef struct fcg_uvw_fields {
  const double *u, *v, *w, *p, *vis, *den, *t;
  const double *uo, *vo, *wo, *uoo, *voo, *woo;
  const double *dUdxi, *dVdxi, *dWdxi, *dPdxi;
  const double *flmass, *fmi, *fmo;
} fcg_uvw_fields;

/* calcuvw.f90:48-438 without its solves: the sources of calcPressDiv
 * (fieldManipulation.f90:89-160), the volume sources (:76-139), facefluxuvw on the inner
 * faces (faceflux_velocity.f90:35-184, sngrad gradients.f90:547-721 with nrelax 0 and the
 * skewness approach), the inlet, outlet, symmetry and wall terms (:223-378),
 * Crank-Nicolson (:381-412 and its v, w twins), the under-relaxed diagonals and ap*.
 * a[nnz] in/out: its incoming diagonal is read (the reference subtracts it from the
 * row sum) and the result holds the off-diagonals and the u system's diagonal.  Out:
 * diag_vw[2*numCells] the v and w diagonals (the reference writes them into a(diag)
 * before bicgstab(v) and bicgstab(w)), rhs[3*numCells] the right-hand side of each
 * solve, ap[3*numCells] = apu, apv, apw.  Turbulence stresses (lturb) are not part of
 * the path. */
int fcg_calcuvw(fcg_context *ctx, const fcg_uvw_params *prm, const fcg_uvw_fields *f,
                double *a, double *diag_vw, double *rhs, double *ap);

/* ---------------------------------------------------------------------------
 * PISO pressure path (PISO_multiple_correction.f90:83-307).
 * ------------------------------------------------------------------------- */

/* Parameters read by get_rAU_x_UEqnH (module parameters, modules_allocatable.f90:40-106).
 * buoyancy = lcal(ien) .and. lbuoy. */
typedef struct fcg_hbya_params {
  double timestep, btime;
  int bdf, cn, buoyancy, boussinesq;
  double beta, densit, tref, gravx, gravy, gravz;
} fcg_hbya_params;

/* Fields read by get_rAU_x_UEqnH; only the cell part [numCells] of each is read.  uo/vo/wo
 * are needed with bdf or cn, uoo/voo/woo with bdf and btime > 0.99, t with buoyancy and
 * boussinesq; the others may be NULL. */
typedef struct fcg_hbya_fields {
  const double *den, *t;
  const double *uo, *vo, *wo, *uoo, *voo, *woo;
  const double *apu, *apv, *apw;
} fcg_hbya_fields;

/* get_rAU_x_UEqnH.f90:3-208: su/sv/sw = the volume sources (buoyancy :37-56, BDF
 * :62-83), the Crank-Nicolson terms of the old time level (:90-110), and
 * H(U) = -sum_nb h(k) U_nb over the inner faces (:112-123), all summed in the
 * reference's order; then u = apu*su, v = apv*sv, w = apw*sw on the cells (:204-206).
 * h[nnz] is the momentum matrix saved before the corrector loop (PISO :84).  u, v, w
 * [numTotal] in/out (only the cell part is read and written); su, sv, sw [numCells] out
 * (each may be NULL). */
int fcg_piso_hbya(fcg_context *ctx, const fcg_hbya_params *prm, const fcg_hbya_fields *f,
                  const double *h, double *u, double *v, double *w, double *su, double *sv,
                  double *sw);

/* Pressure assembly of the PISO corrector (PISO_multiple_correction.f90:108-148) with
 * facefluxmass_piso (facefluxmass.f90:294-358): a = 0, su = 0, per inner face
 * cap = can = -dene (fxp vol_P apu_P + fxn vol_N apu_N) |S| / |d_PN|, the mass flux of the
 * centrally interpolated velocity flmass = dene (u_f.S) (no Rhie-Chow term), the diagonal
 * and su = -div(flmass) in face order.  Fields as fcg_facefluxmass (p, dPdxi, apv and
 * apw are not read and may be NULL). */
int fcg_facefluxmass_piso(fcg_context *ctx, const fcg_flow_fields *f, double *a, double *su,
                          double *flmass);

/* adjustMassFlow.f90:1-71: su(owner) -= fmi(i) over the inlet faces; the outlet slots of
 * u, v, w take their cell's velocity, fmo(i) = den(ijp) (u,v,w)(ijb).S, the outflow is
 * scaled to flomas (fac = flomas/(sum fmo + small)) and su(owner) -= fmo(i).  den, u, v, w
 * [numTotal]; fmi[ninl] in, fmo[nout] out; su[numCells] in/out. */
int fcg_adjust_mass_flow(fcg_context *ctx, const double *den, double flomas, const double *fmi,
                         double *u, double *v, double *w, double *fmo, double *su);

/* Reference pressure of the PISO pressure equation (PISO_multiple_correction.f90:188-192):
 * row pRefCell (1-based) of a is zeroed, its diagonal set to 1 and su(pRefCell) =
 * p(pRefCell).  a[nnz], su[numCells] in/out; p[numCells or numTotal]. */
int fcg_set_reference_pressure(fcg_context *ctx, int pRefCell, const double *p, double *a,
                               double *su);

/* PISO velocity correction (PISO_multiple_correction.f90:300-304): u -= apu*dPdxi(1,:)*vol,
 * v -= apv*dPdxi(2,:)*vol, w -= apw*dPdxi(3,:)*vol over the cells (the product in the
 * reference's order, which differs from calcp's).  u, v, w [numTotal] in/out. */
int fcg_correct_velocity_piso(fcg_context *ctx, const double *dPdxi, const double *apu,
                              const double *apv, const double *apw, double *u, double *v,
                              double *w);

/* ---------------------------------------------------------------------------
 * Gradients and boundary values.
 * ------------------------------------------------------------------------- */
#define FCG_GRAD_GAUSS 1           /* grad_gauss.f90, nigrad passes */
#define FCG_GRAD_GAUSS_CORRECTED 2 /* grad_gauss_corrected.f90, old gradient = dPhidxi on entry */
#define FCG_GRAD_LSQ 3             /* grad_lsq.f90 stage 2 (needs fcg_grad_lsq_matrix first) */

/* grad(phi,dPhidxi[,option]) (gradients.f90:95-151, :197-259) without limiter:
 * phi[numTotal] in, dPhidxi[3*numCells] out (in/out for GAUSS_CORRECTED). */
int fcg_grad(fcg_context *ctx, const double *phi, double *dPhidxi, int method, int nigrad);

/* grad_lsq stage 1 (grad_lsq.f90:50-165): builds the per-cell inverse normal
 * matrices on the device; dmat[9*numCells] may be NULL or receives a copy. */
int fcg_grad_lsq_matrix(fcg_context *ctx, double *dmat);

/* bpres(p,istage) (bpres.f90:3-152): istage 1 copies owner values into every
 * boundary slot, istage >= 2 extrapolates wall and pressure-outlet slots with
 * dPdxi[3*numCells].  p[numTotal] in/out. */
int fcg_bpres(fcg_context *ctx, double *p, const double *dPdxi, int istage);

/* ---------------------------------------------------------------------------
 * Krylov solvers on the CSR matrix (a[nnz], su[numCells]).
 * ------------------------------------------------------------------------- */
typedef struct fcg_solve_report {
  double res0;   /* initial L1 residual sum|su - A fi| */
  double resl;   /* final L1 residual */
  int iters;     /* sweeps done (itr_used) */
  int converged; /* resl/(res0+small) < sor reached */
  double l2_rel; /* FP64-recomputed ||su - A fi||_2 / ||su||_2 after the solve */
  double seconds;
} fcg_solve_report;

/* dpcg(fi,ifi) (src/dpcg.f90:3-154): Jacobi-preconditioned CG, L1-relative stop
 * resl/(res0+small) < sor, at most nsw sweeps, early return when res0 < 1e-13.
 * fi[numCells] in/out (the reference's fi(numTotal); only cells are touched);
 * res[numCells] (may be NULL) receives the final residual; *resor is set to res0
 * when at least one sweep ran (dpcg.f90:139), as the reference's resor(ifi). */
int fcg_dpcg(fcg_context *ctx, const double *a, const double *su, double *fi, double *res,
             double sor, int nsw, double *resor, fcg_solve_report *rep);

/* iccg(fi,ifi) (src/iccg.f90:3-177): CG preconditioned by the diagonal incomplete
 * Cholesky M = (D+L) D^-1 (D+U); triangular sweeps run level by level. */
int fcg_iccg(fcg_context *ctx, const double *a, const double *su, double *fi, double *res,
             double sor, int nsw, double *resor, fcg_solve_report *rep);

/* bicgstab(fi,ifi) (src/bicgstab.f90:1-231): right-preconditioned BiCGStab with the
 * diagonal ILU factor. */
int fcg_bicgstab(fcg_context *ctx, const double *a, const double *su, double *fi,
                 double *res, double sor, int nsw, double *resor, fcg_solve_report *rep);

/* dpcg with FP32 inner sweeps under FP64 reliable updates (no reference counterpart;
 * same arguments and stop test as fcg_dpcg).  The sweeps run CG on D^-1/2 A D^-1/2 in
 * FP32 (the Jacobi preconditioner of dpcg.f90 folded into a symmetric scaling); FP64 is
 * kept for the true residual su - A x, which replaces the FP32 one whenever the FP32
 * residual has fallen 10x since the last replacement or predicts convergence, for the
 * global sums that form alpha and beta, and for the solution.  The stop test
 * resl/(res0+small) < sor is evaluated on the true FP64 residual only.  rep->iters
 * counts FP32 sweeps; the trace holds one (resl, rsm) pair per FP64 replacement. */
int fcg_dpcg_mixed(fcg_context *ctx, const double *a, const double *su, double *fi,
                   double *res, double sor, int nsw, double *resor, fcg_solve_report *rep);

/* Several systems on the bound pattern solved together (no single reference call; it
 * replaces the three bicgstab(u/v/w) calls of calcuvw.f90:441,498,556, which share one
 * set of off-diagonals, and the bicgstab calls of the k and epsilon equations, e.g.
 * k_epsilon_std.f90:528).  a[nsys*nnz], su[nsys*n], fi[nsys*n] (system k at offset
 * k*nnz or k*n), 1 <= nsys <= 8.  DILU-BiCGStab sweeps (bicgstab.f90) in FP32 under an
 * FP64 defect-correction loop: the FP64 residual su - A x decides convergence with the
 * reference's test resl/(res0+small) < sor per system; the FP32 solve of each
 * correction runs until its L1 residual has dropped 1e4-fold.  resor[nsys] and
 * rep[nsys] (iters = FP32 sweeps of all systems together) may be NULL. */
int fcg_bicgstab_multi(fcg_context *ctx, int nsys, const double *a, const double *su, double *fi,
                       double sor, int nsw, double *resor, fcg_solve_report *rep);

/* Constants of the solvers: small (parameters::small, modules_allocatable.f90:27;
 * default the REAL literal 1e-20) and whether a solve returns at once when
 * res0 < 1e-13 (dpcg.f90:66-70; default 1).  The copies of the solvers in
 * tests/test_sparse_solvers.f90 use small = 1e-30 and never return early. */
int fcg_set_solver_options(fcg_context *ctx, double small, int early_exit);

/* Diagnostics for the timeout path of the DIC/DILU sweeps, which run in one launch with
 * each row waiting on the rows it reads: every wait gives up after `polls` polls (<= 0:
 * the default, about 0.4 s), and row absent_row (1-based; 0: none) never announces its
 * result in forward sweeps, so the waits of the rows that read it run out and the solve
 * returns FCG_ERR_TIMEOUT with the device still usable.  (0, 0) restores normal runs. */
int fcg_set_sweep_wait_test(fcg_context *ctx, int polls, int absent_row);

/* Diagnostics for the timeout path of the GPU build of the learned FCG's coarse
 * hierarchy, whose matching decides every row in one launch with each row waiting on the
 * decisions it reads: every wait gives up after `polls` polls (<= 0: the default), and
 * row absent_row (1-based; 0: none) of the first matching pass never announces its
 * decision, so the waits that read it run out, the GPU build gives up and the hierarchy
 * is built on the host (fcg_lp_hierarchy_built_on then reports 0).  Read when a
 * hierarchy is built; (0, 0) restores normal runs. */
int fcg_set_aggregation_wait_test(fcg_context *ctx, int polls, int absent_row);

/* Per-sweep (resl, rsm) pairs of the last solve -- what the reference prints per
 * sweep when ltest is set (dpcg.f90:141); for fcg_dpcg_mixed one pair per FP64 residual
 * replacement (the true residual).  *count receives the number available; at most
 * max_count pairs are copied to resl_rsm (which may be NULL). */
int fcg_get_solver_trace(fcg_context *ctx, double *resl_rsm, int max_count, int *count);

/* No counterpart in the reference.  dpcg for callers that cannot allocate device
 * memory -- a host code whose GPU memory is all reserved by its own pool, or a loop
 * whose rules forbid allocation after start-up.  It needs no context and allocates
 * nothing: every array is the caller's DEVICE array (the reference's 1-based CSR
 * ioffset[numCells+1], ja[nnz], diag[numCells], values a[nnz], su[numCells], fi
 * in/out, res out), and the work vectors sit in one file-scope device array sized for
 * at most FCG_NOALLOC_MAX_CELLS cells (about 6.4 MB, held until exit by every GPU it has
 * been used on).  Larger systems, host arrays and arrays of another GPU return
 * FCG_ERR_ARG.  All calls share that array: calls that overlap on the GPU race.  The
 * first call on a device looks up the array's address (cudaGetSymbolAddress) with that
 * device current; make it before any stream capture.  Under CUDA's default lazy module
 * loading that first call also loads this code and the array onto the device (about
 * 6.4 MB plus the code, once): a caller whose pool reserves the whole device must make
 * it before the pool takes its memory, or set CUDA_MODULE_LOADING=EAGER.  Later calls
 * allocate nothing.  Work runs on cuda_stream (NULL = legacy stream); the call returns
 * when the solve is done. */
#define FCG_NOALLOC_MAX_CELLS 262144
int fcg_dpcg_noalloc(int numCells, const int *ioffset, const int *ja, const int *diag,
                     const double *a, const double *su, double *fi, double *res, double sor,
                     int nsw, double *resor, fcg_solve_report *rep, void *cuda_stream);

/* Diagnostics (no reference counterpart; the reference times whole outer iterations
 * with cpu_time, main.f90:127-148).  Runs `reps` more sweeps of the last solve's method
 * kernel by kernel, outside the CUDA graph, with CUDA events around every kernel (a
 * triangular sweep counts as one unit), and writes the mean milliseconds of each unit
 * to ms[0..*units-1].  It continues the last solve's iteration and so changes its
 * state: solve again before using results.  fcg_profile_unit_name names unit i. */
int fcg_profile_sweeps(fcg_context *ctx, int reps, double *ms, int max_units, int *units);
const char *fcg_profile_unit_name(const fcg_context *ctx, int unit);

/* y = A x (the matvec of dpcg.f90:105-110) with CSR values a[nnz]; a == NULL reuses
 * the matrix of the previous solve or spmv call. */
int fcg_spmv(fcg_context *ctx, const double *a, const double *x, double *y);

/* ---------------------------------------------------------------------------------
 * Batched DPCG (no single reference call: it replaces a sequence of dpcg(fi,ifi) calls,
 * dpcg.f90:3-154, on independent pressure systems).  Each system lives on its own bound
 * context (its own mesh); all contexts must be on one device and distinct.  One
 * persistent cooperative kernel, captured in a CUDA graph, runs every system's DPCG
 * (the recurrence, constants and L1 stop test of dpcg.f90, per system) in lockstep
 * phases separated by grid-wide barriers whose waits are bounded (FCG_ERR_TIMEOUT when
 * one gives up).  Work items are runs of `slices_per_item` 32-row slices;
 * fcg_batch_autotune times the candidates on the caller's systems and keeps the
 * fastest (item size and CTAs per SM).  The batch runs on the first context's stream.
 * --------------------------------------------------------------------------------- */
typedef struct fcg_batch fcg_batch;
int fcg_batch_create(fcg_context *const *ctxs, int nsys, fcg_batch **out);
int fcg_batch_destroy(fcg_batch *batch);
const char *fcg_batch_last_error(const fcg_batch *batch);
int fcg_batch_set_params(fcg_batch *batch, int slices_per_item, int blocks_per_sm);
int fcg_batch_get_params(const fcg_batch *batch, int *slices_per_item, int *blocks_per_sm,
                         int *max_blocks_per_sm);
/* a[k] (nnz of system k; a == NULL or a[k] == NULL reuses the matrix loaded last),
 * su[k], fi[k] (in/out) of numCells of system k, host or device.  resor[nsys] and
 * rep[nsys] may be NULL; rep[k].seconds is the time of the whole batch. */
int fcg_batch_dpcg(fcg_batch *batch, const double *const *a, const double *const *su,
                   double *const *fi, double sor, int nsw, double *resor, fcg_solve_report *rep);
/* Diagnostics for the timeout path of the grid barriers: every barrier wait gives up
 * after `polls` polls (<= 0: the default, over 0.25 s), and CTA absent_block (>= 0)
 * leaves before the first barrier, so the other CTAs' waits run out and fcg_batch_dpcg
 * returns FCG_ERR_TIMEOUT with the device still usable.  (0, -1) restores normal runs. */
int fcg_batch_set_wait_test(fcg_batch *batch, long long polls, int absent_block);
/* Times `sweeps` fixed sweeps of every candidate (x = 0) and keeps the fastest. */
int fcg_batch_autotune(fcg_batch *batch, const double *const *a, const double *const *su,
                       int sweeps, double *best_ms);

/* ---------------------------------------------------------------------------------
 * Learned preconditioner (no reference counterpart; it is used in place of the
 * Jacobi preconditioner of dpcg.f90:85-100 inside flexible CG, with dpcg as fallback).
 *
 * A message-passing network of FCG_LP_LAYERS layers of width FCG_LP_WIDTH maps the
 * residual of the scaled system Ahat = D^-1/2 A D^-1/2 (D = diag(A)) to an
 * approximation of its error Ahat^-1 r.  Per-cell inputs (FCG_LP_FEATURES): the
 * residual divided by its rms, log(a_PP / vol^1/3) - log 6, log(vol / mean vol) and
 * the three face-area sums sum|S_x,y,z| / (2 vol^2/3) - 1.  Layer l:
 * h_l = h_{l-1} + relu(W_l [h_{l-1}; Ahat h_{l-1}] + b_l), BF16 activations, tensor
 * cores with FP32 accumulation.  Output: N(r) = r + rms(r) (w_out . h_L + b_out) -- the
 * Jacobi preconditioner plus a learned correction (zero output weights at creation).  Weights are
 * FP32 (FCG_LP_PARAMS values in the order W_in[32][6], b_in[32], then per layer
 * W_l[32][64] (row = output channel, columns h then Ahat h), b_l[32], then w_out[32],
 * b_out).  A handle holds weights and Adam state on one device and can serve several
 * contexts on that device; its calls are ordered on the stream of the context they
 * are given.  Vectors r, z, e are FP32 of numCells values in the scaled system
 * (r = D^-1/2 (su - A x), e = D^1/2 (x* - x)), host or device memory.  Errors of the
 * fcg_lp_* calls are described by fcg_lp_last_error. */
#define FCG_LP_WIDTH 32
#define FCG_LP_LAYERS 6
#define FCG_LP_FEATURES 6
#define FCG_LP_PARAMS 12737
typedef struct fcg_learned fcg_learned;
int fcg_lp_create(int device, unsigned long long seed, fcg_learned **out);
int fcg_lp_destroy(fcg_learned *lp);
const char *fcg_lp_last_error(const fcg_learned *lp);
/* FP32 weights out / in (count must be FCG_LP_PARAMS); set clears the Adam state. */
int fcg_lp_get_weights(fcg_learned *lp, float *out, int count);
int fcg_lp_set_weights(fcg_learned *lp, const float *w, int count);
/* Checkpoint of weights and Adam state: magic "FCGLP001", int32 width, layers,
 * features, parameter count, int64 step, then weights, Adam m, Adam v (FP32). */
int fcg_lp_save(fcg_learned *lp, const char *path);
int fcg_lp_load(fcg_learned *lp, const char *path);
/* Loads CSR values a[nnz] into the context, builds Ahat in FP32 and the features. */
int fcg_lp_set_matrix(fcg_learned *lp, fcg_context *ctx, const double *a);
/* Features of the last fcg_lp_set_matrix, feature-major: out[FCG_LP_FEATURES][numCells]
 * (feature 0 is the residual input of the last forward pass). */
int fcg_lp_features(fcg_learned *lp, fcg_context *ctx, float *out);
/* z = N(r). */
int fcg_lp_apply(fcg_learned *lp, fcg_context *ctx, const float *r, float *z);
/* The loss chosen by fcg_lp_set_loss (default: residual norm, |Ahat N(r) - r|^2 / |r|^2)
 * and d loss / d weights (grad[FCG_LP_PARAMS], may be NULL); BF16 roundings are treated
 * as identities in the gradient. */
int fcg_lp_loss_grad(fcg_learned *lp, fcg_context *ctx, const float *r, const float *e,
                     float *loss, float *grad);
/* Loss of fcg_lp_loss_grad and fcg_lp_train_step: FCG_LP_LOSS_RESIDUAL (default),
 * |Ahat N(r) - r|^2 / |r|^2, or FCG_LP_LOSS_ENERGY, (N(r) - e).Ahat (N(r) - e) / e.Ahat e
 * (the same error measured in the energy norm), or FCG_LP_LOSS_CYCLE, the energy norm of
 * the error of the whole preconditioner M (the network followed by the coarse-grid
 * correction below), (M(r) - e).Ahat (M(r) - e) / e.Ahat e (the correction must be on;
 * its hierarchy for the context is built on first use).  In every form r stands for
 * Ahat e. */
#define FCG_LP_LOSS_ENERGY 0
#define FCG_LP_LOSS_RESIDUAL 1
#define FCG_LP_LOSS_CYCLE 2
int fcg_lp_set_loss(fcg_learned *lp, int kind);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the pair (r, e) with rate lr;
 * *loss (may be NULL) receives the loss before the step. */
int fcg_lp_train_step(fcg_learned *lp, fcg_context *ctx, const float *r, const float *e,
                      float lr, float *loss);
/* Flexible-CG controls: the number of previous directions each new one is made
 * A-orthogonal to (1..8, default 8); FP64 residual replacement at least every ru_every
 * iterations (default 50); the FCG is declared stalled when the true L1 residual has not
 * fallen below stall_factor (default 0.5) times its value at the last such drop within
 * stall_window iterations (default 400). */
int fcg_lp_set_fcg_options(fcg_learned *lp, int directions, int ru_every, int stall_window,
                           double stall_factor);

/* FCG iterations and FP64 residual replacements of the last fcg_fcg_learned call. */
int fcg_lp_last_solve_stats(const fcg_learned *lp, int *iters, int *updates);
/* Diagnostics: mean milliseconds of each kernel of one forward pass on r, over `reps`
 * passes timed with CUDA events per launch: unit 0 rms, 1 embedding, 2..7 the six
 * message-passing layers, 8 output (*units receives 9). */
int fcg_lp_profile(fcg_learned *lp, fcg_context *ctx, const float *r, int reps, double *ms,
                   int max_units, int *units);
/* Which form of the message-passing layer inference runs for ctx's mesh (no reference
 * counterpart; valid after fcg_lp_set_matrix): *form = FCG_LP_LAYER_GATHER (the sliced
 * gather over the CSR pattern, any mesh) or FCG_LP_LAYER_PLANES (the cells form a
 * lexicographic nx x ny x nz hex block: planes staged by TMA copies; the same bits).
 * dims (may be NULL) receives nx, ny, nz for the plane form.  The environment variable
 * FCG_LP_LAYER=gather keeps the gather form on every mesh. */
#define FCG_LP_LAYER_GATHER 0
#define FCG_LP_LAYER_PLANES 1
int fcg_lp_layer_form(fcg_learned *lp, fcg_context *ctx, int *form, int *dims);

/* Coarse-grid correction of the flexible CG (on by default).  The preconditioner is
 *   M(r) = z + alpha P V(P^T (r - Ahat z)),  z = N(r),
 * where P is the piecewise-constant prolongation from an aggregation of the cells and
 * V a V-cycle below it: `sweeps` damped Jacobi sweeps (omega) before and after each
 * level's own correction (also scaled by alpha) and a dense inverse at the coarsest
 * level when it has at most dense_max rows.  A level aggregates the level above by
 * three passes of pairwise matching: each row, in ascending order, pairs with its
 * unmatched neighbour of most negative coupling in Ahat (ties: lowest column).  The
 * aggregation is built on the host once per mesh, from the first matrix solved (or set)
 * on it; the level matrices P^T Ahat P are recomputed on the device at every call.
 * smoother FCG_LP_SMOOTH_JACOBI replaces N by `sweeps` Jacobi sweeps before and after
 * the correction (the same cycle without the network).  With `smoothed` (default) the
 * first level uses the smoothed prolongation P = (I - omega D^-1 Ahat) P_tent of the
 * piecewise-constant P_tent, its level matrix is P^T Ahat P, and its correction is not
 * scaled by alpha (smoothed aggregation).  FP32 throughout. */
#define FCG_LP_SMOOTH_NETWORK 0
#define FCG_LP_SMOOTH_JACOBI 1
#define FCG_LP_MAX_LEVELS 16
typedef struct fcg_lp_multilevel {
  int enabled;    /* 1 (default) or 0: M(r) = N(r) */
  int smoother;   /* FCG_LP_SMOOTH_NETWORK (default) or FCG_LP_SMOOTH_JACOBI */
  int sweeps;     /* 1..8, default 2 */
  int max_levels; /* 2..FCG_LP_MAX_LEVELS levels counting the fine one, default 10 */
  int dense_max;  /* 1..160, default 128 */
  double alpha;   /* (0, 4), default 1.8: scaling of every unsmoothed prolongation */
  double omega;   /* (0, 2), default 0.67 */
  int smoothed;   /* 1 (default) or 0: the first level's prolongation P_tent */
} fcg_lp_multilevel;
int fcg_lp_set_multilevel(fcg_learned *lp, const fcg_lp_multilevel *opt);
int fcg_lp_get_multilevel(const fcg_learned *lp, fcg_lp_multilevel *opt);
/* The hierarchy for ctx's mesh and the matrix last set (built if needed): *levels
 * counting the fine one, cells[l] and entries[l] of every level (arrays of
 * FCG_LP_MAX_LEVELS, may be NULL), and the seconds its construction took. */
int fcg_lp_hierarchy_info(fcg_learned *lp, fcg_context *ctx, int *levels, int *cells,
                          long long *entries, double *setup_seconds);
/* Where that hierarchy was built: *on_device = 1 on the GPU (the default), 0 on the host
 * (FCG_AGG=host in the environment, or after the GPU build gave up: a matching wait that
 * ran out or a coarse row too wide for its accumulation table).  Both give the same
 * arrays element for element. */
int fcg_lp_hierarchy_built_on(fcg_learned *lp, fcg_context *ctx, int *on_device);
/* Arrays of coarse level `level` (1..levels-1), 0-based, each may be NULL: agg[n_above]
 * (row of the level above -> row of this level), mptr[n+1] and mem[n_above] (rows above
 * of every row, ascending), ptr[n+1] and col[entries] (pattern, columns ascending) and
 * val[entries] (P^T Ahat P, summed in FP32 from the FP32 Ahat in a fixed order: member
 * rows ascending, each row's entries in column order). */
int fcg_lp_hierarchy_level(fcg_learned *lp, fcg_context *ctx, int level, int *agg, int *mptr,
                           int *mem, int *ptr, int *col, float *val);
/* z = M(r), the preconditioner fcg_fcg_learned applies, for the matrix last set. */
int fcg_lp_precondition(fcg_learned *lp, fcg_context *ctx, const float *r, float *z);
/* out = z + alpha P V(P^T (r - Ahat z)), the coarse-grid correction alone. */
int fcg_lp_coarse_correct(fcg_learned *lp, fcg_context *ctx, const float *r, const float *z,
                          float *out);
/* Host utility (no device): the aggregation of one level as above, on a 0-based CSR
 * (ptr[n+1], col and val[ptr[n]], columns strictly ascending in each row) -- `passes`
 * matching passes, stopping once at most dense_max aggregates remain.  agg[n] receives
 * the aggregate of every row and *nc their number (agg[i] = i, *nc = n when the matrix
 * does not coarsen by 10%).  FCG_ERR_INDEX for a malformed CSR. */
int fcg_aggregate(int n, const int *ptr, const int *col, const double *val, int passes,
                  int dense_max, int *agg, int *nc);
/* Host utility (no device): P^T A P for the smoothed prolongation P = (I - omega D^-1 A)
 * P_tent of the aggregation agg[n] (nc aggregates, as fcg_aggregate returns it) of a
 * 0-based CSR with strictly ascending columns, in FP64 and in the order the hierarchy's
 * host construction uses.  With cptr NULL only *nnz is set; otherwise cptr[nc+1],
 * ccol[*nnz] and cval[*nnz] receive the matrix (*nnz in: their capacity, out: the count). */
int fcg_smoothed_level(int n, const int *ptr, const int *col, const double *val,
                       const int *agg, int nc, double omega, long long *nnz, int *cptr,
                       int *ccol, double *cval);

/* Truncated flexible CG (Notay, SIAM J. Sci. Comput. 22 (2000) 1444) preconditioned by
 * M (the network and the coarse-grid correction above), on
 * the arguments of fcg_dpcg and with its stop test resl/(res0+small) < sor on the
 * FP64 L1 residual.  The iteration runs in FP32 on Ahat with reliable updates: the
 * true residual su - A x is recomputed in FP64 when the FP32 residual has fallen 10x,
 * predicts convergence, or ru_every iterations have passed.  When the FCG stalls or a
 * value turns non-finite, fcg_dpcg continues from the current solution with the
 * remaining sweeps (rep->iters counts both; *fcg_iters the FCG iterations and
 * *fallback 1 when fcg_dpcg ran; both may be NULL). */
int fcg_fcg_learned(fcg_context *ctx, fcg_learned *lp, const double *a, const double *su,
                    double *fi, double *res, double sor, int nsw, double *resor,
                    fcg_solve_report *rep, int *fcg_iters, int *fallback);

#ifdef __cplusplus
}
#endif
#endif /* FCGPU_H */
