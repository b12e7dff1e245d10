/*
 * fcg_oracle.h -- CPU restatement of freeCappuccino's pressure-correction path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA library
 * (libfcgpu.so). Only the test-suite, the smoke check and the CPU-baseline leg of
 * the benchmark may load it. The product never links or calls it.
 *
 * Every routine restates one reference subroutine, loop for loop, in the
 * reference's evaluation order (Fortran left-to-right, no fused multiply-add:
 * the library is compiled with -O2 -ffp-contract=off).  Index VALUES stay 1-based
 * exactly as the Fortran arrays hold them (owner, neighbour, ioffset, ja, diag,
 * slot maps); the C arrays themselves are 0-based, so ref(i) is c[i-1].
 *
 * Parity pin: the three Krylov solvers reproduce the reference's own golden
 * traces (tests/test_sparse_solvers.f90 + tests/output.txt).  Geometry, assembly
 * and gradient routines have no stored reference outputs; they are pinned only by
 * this restatement.
 */
#ifndef FCG_ORACLE_H
#define FCG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Mesh description (module `geometry`, src/mesh_geometry_and_topology.f90:12-98). */
typedef struct orc_mesh {
  int numCells, numFaces, numInnerFaces;
  int ninl, nout, nsym, nwal, npru;
  /* 0-based starts as read from the boundary file (face iface = start + i, i 1-based). */
  int iInletFacesStart, iOutletFacesStart, iSymmetryFacesStart, iWallFacesStart,
      iPressOutletFacesStart;
  const int *owner;     /* [numFaces]      1-based */
  const int *neighbour; /* [numInnerFaces] 1-based */
  const double *arx, *ary, *arz, *xf, *yf, *zf; /* [numFaces] */
  const double *xc, *yc, *zc, *vol;             /* [numCells] */
  const double *facint;                         /* [numInnerFaces] */
  /* O-C grid cuts and cyclic faces (mesh_geometry_and_topology.f90:453-462, 800-845):
   * noc face pairs after `noc = noc + ncyc` (:1163), the last ncyc of them cyclic.
   * Pair i joins the owner of face ijlFace(i) (ijl) to the owner of its friend
   * ijrFace(i) (ijr); the O-C loops take the pair's area from face iOCFacesStart + i
   * (fvm_laplacian.f90:70). */
  int noc, ncyc, iOCFacesStart;
  const int *ijlFace, *ijrFace; /* [noc] 1-based face indices */
} orc_mesh;

/* ijl, ijr (1-based cells), foc and srdoc of the noc pairs
 * (mesh_geometry_and_topology.f90:814-845, 1083-1152; cyclic pairs take foc = 1/2). */
int orc_oc_geometry(const orc_mesh *m, int *ijl, int *ijr, double *foc, double *srdoc);

/* Float-literal constants of the reference: default-REAL literals promoted to real(dp). */
double orc_const_small_src(void);  /* parameters::small = 1e-20 (modules_allocatable.f90:27) */
double orc_const_small_test(void); /* small = 1e-30 (tests/test_sparse_solvers.f90:36) */
double orc_const_tol(void);        /* tol = 1e-13 (dpcg.f90:37) */

/* --- geometry: mesh_geometry_and_topology.f90:859-1079 (triangle fans from node 1) --- */
int orc_geometry(int numNodes, const double *x, const double *y, const double *z,
                 int numCells, int numFaces, int numInnerFaces,
                 const int *face_ptr,   /* [numFaces+1] 0-based offsets into face_nodes */
                 const int *face_nodes, /* 1-based node ids */
                 const int *owner, const int *neighbour,
                 double *arx, double *ary, double *arz, double *xf, double *yf, double *zf,
                 double *xc, double *yc, double *zc, double *vol, double *facint);

/* --- a1: sparse_matrix.f90:42-172 --- */
int orc_create_csr(int numCells, int numInnerFaces, const int *owner, const int *neighbour,
                   int *ioffset /*[n+1]*/, int *ja /*[nnz]*/, int *diag /*[n]*/,
                   int *slot_pn /*[nin]*/, int *slot_np /*[nin]*/);

/* --- a2: fvm_laplacian.f90:1-163 (+ facefluxlaplacian :171-221) --- */
/* fvm_laplacian.f90:1-163.  With m->noc > 0, a holds nnz + 2 noc values: the CSR
 * values, then ar(1..noc), then al(1..noc) of the O-C faces (:67-86). */
int orc_laplacian(const orc_mesh *m, const int *ioffset, const int *diag,
                  const int *slot_pn, const int *slot_np,
                  const double *mu /*[n]*/, const double *phi /*[numTotal]*/,
                  double *a /*[nnz] out*/, double *su /*[n] in/out*/);

/* --- a3: calcp-multiple_correction_SIMPLE.f90:34-77 + facefluxmass.f90:34-199 --- */
int orc_facefluxmass(const orc_mesh *m, const int *diag, const int *slot_pn, const int *slot_np,
                     const double *u, const double *v, const double *w, const double *p,
                     const double *dUdxi, const double *dVdxi, const double *dWdxi,
                     const double *dPdxi, /* (3,n) component fastest */
                     const double *apu, const double *apv, const double *apw, /* [n] */
                     const double *den, /* [numTotal] */
                     int nnz, double *a, double *su, double *flmass);

/* --- a4: calcp-multiple_correction_SIMPLE.f90:193-206 + facefluxmass.f90:520-607 --- */
int orc_fluxmc(const orc_mesh *m, const double *dPdxi, const double *apu, const double *den,
               double *su, double *flmass);

/* --- a5/a6: grad_gauss.f90:1-211, grad_gauss_corrected.f90:1-112 ---
 * Writes dPhidxi(3,n) the way gradients.f90:95-151 / :197-259 do (zeroed first).
 * corrected != 0 selects grad_gauss_corrected (one pass, old gradient = incoming). */
int orc_grad_gauss(const orc_mesh *m, const double *phi, int nigrad, int corrected,
                   double *dPhidxi);

/* --- a7: grad_lsq.f90 stage 1 (:50-165) and stage 2 (:168-306) --- */
int orc_grad_lsq_matrix(const orc_mesh *m, double *dmat /*(9,n)*/);
int orc_grad_lsq(const orc_mesh *m, const double *phi, const double *dmat, double *dPhidxi);

/* --- a8: bpres.f90:3-152 --- */
int orc_bpres(const orc_mesh *m, double *p /*[numTotal]*/, const double *dPdxi, int istage);

/* --- calcp corrections: calcp-multiple_correction_SIMPLE.f90:159-171 and :184-189 --- */
int orc_flux_correct(const orc_mesh *m, const int *slot_pn, const double *a, const double *pp,
                     double *flmass);
int orc_correct_bc_velocity(const orc_mesh *m, const double *den, double flomas, double *u,
                            double *v, double *w, double *fmo);
int orc_continuity_errors(const orc_mesh *m, const double *flmass, const double *fmi,
                          const double *fmo, double *res, double *sum_local, double *global);
int orc_correct_fields(const orc_mesh *m, const double *dPdxi, const double *apu,
                       const double *apv, const double *apw, const double *pp, double urf,
                       int pRefCell, double *u, double *v, double *w, double *p);

/* --- momentum assembly: calcuvw.f90:48-438 with facefluxuvw, sngrad, face_value and
 *     calcPressDiv --- */
typedef struct orc_uvw_params {
  int scheme, limiter; /* FCG_CONV_* / FCG_LIM_* numbering of include/fcgpu.h */
  double gds, viscos;
  double urfr[3], urfm[3];
  int bdf, cn;
  double timestep, btime;
  int const_mflux;
  double gradPcmf;
  int buoyancy, boussinesq;
  double beta, densit, tref, gravx, gravy, gravz;
} orc_uvw_params;
/* u, v, w, p, vis [numTotal]; den, t, uo..woo [numCells]; gradients (3,numCells);
 * a[nnz] in/out (diagonal read; out: off-diagonals and the u diagonal); diag_vw[2n],
 * rhs[3n], ap[3n] out. */
int orc_calcuvw(const orc_mesh *m, const int *ioffset, const int *diag, const int *slot_pn,
                const int *slot_np, const orc_uvw_params *prm, const double *u, const double *v,
                const double *w, const double *p, const double *vis, const double *den,
                const double *t, const double *uo, const double *vo, const double *wo,
                const double *uoo, const double *voo, const double *woo, const double *dUdxi,
                const double *dVdxi, const double *dWdxi, const double *dPdxi,
                const double *flmass, const double *fmi, const double *fmo, double *a,
                double *diag_vw, double *rhs, double *ap);

/* --- PISO pressure path: PISO_multiple_correction.f90, get_rAU_x_UEqnH.f90,
 *     facefluxmass_piso (facefluxmass.f90:294-358), adjustMassFlow.f90 --- */
typedef struct orc_hbya_params {
  double timestep, btime;
  int bdf, cn, buoyancy, boussinesq;
  double beta, densit, tref, gravx, gravy, gravz;
} orc_hbya_params;
/* Cell arrays [numCells]; uo..woo, t may be NULL where the parameters do not read them.
 * h[nnz]; u, v, w in/out [numCells+] (the cells are overwritten); su, sv, sw out. */
int orc_piso_hbya(const orc_mesh *m, const int *ioffset, const int *diag, const int *slot_pn,
                  const int *slot_np, const orc_hbya_params *prm, const double *h,
                  const double *den, const double *t, const double *uo, const double *vo,
                  const double *wo, const double *uoo, const double *voo, const double *woo,
                  const double *apu, const double *apv, const double *apw, double *u, double *v,
                  double *w, double *su, double *sv, double *sw);
int orc_facefluxmass_piso(const orc_mesh *m, const int *diag, const int *slot_pn,
                          const int *slot_np, const double *u, const double *v, const double *w,
                          const double *dUdxi, const double *dVdxi, const double *dWdxi,
                          const double *apu, const double *den, int nnz, double *a, double *su,
                          double *flmass);
int orc_adjust_mass_flow(const orc_mesh *m, const double *den, double flomas, const double *fmi,
                         double *u, double *v, double *w, double *fmo, double *su);
int orc_set_reference_pressure(const int *ioffset, const int *diag, int pRefCell,
                               const double *p, double *a, double *su);
int orc_correct_velocity_piso(const orc_mesh *m, const double *dPdxi, const double *apu,
                              const double *apv, const double *apw, double *u, double *v,
                              double *w);

/* --- a9-a11: dpcg.f90, iccg.f90, bicgstab.f90 --- */
typedef struct orc_solver_opts {
  double resmax;   /* sor(ifi) */
  int nsw;         /* nsw(ifi) */
  double small;    /* parameters::small (1e-20) or the test copies' 1e-30 */
  int early_exit;  /* 1: src/ variant returns when res0 < tol; 0: test copies never do */
  double *trace;   /* optional [2*nsw]: per sweep (resl, rsm) */
  /* O-C couplings (module sparse_matrix's al, ar): row ijl(i) couples to ijr(i) with
   * ar(i), row ijr(i) to ijl(i) with al(i); noc = 0 for none.  dpcg and iccg apply them
   * in the initial residual and in every A p (dpcg.f90:58-61,113-116; iccg.f90:59-62,
   * 137-140); bicgstab in the initial residual only (bicgstab.f90:49-52). */
  int noc;
  const int *ijl, *ijr; /* [noc] 1-based cells */
  const double *ar, *al; /* [noc] */
} orc_solver_opts;

typedef struct orc_solver_out {
  double res0, resl, resor; /* resor is written only when at least one sweep ran */
  int iters;
  int resor_written;
} orc_solver_out;

int orc_dpcg(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
             const double *su, double *fi, double *res, const orc_solver_opts *o,
             orc_solver_out *out);
int orc_iccg(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
             const double *su, double *fi, double *res, const orc_solver_opts *o,
             orc_solver_out *out);
int orc_bicgstab(int n, const int *ioffset, const int *ja, const int *diag, const double *a,
                 const double *su, double *fi, double *res, const orc_solver_opts *o,
                 orc_solver_out *out);

/* Plain CSR matrix-vector product y = A x (the loop of dpcg.f90:105-110). */
int orc_spmv(int n, const int *ioffset, const int *ja, const double *a, const double *x,
             double *y);

#ifdef __cplusplus
}
#endif
#endif
