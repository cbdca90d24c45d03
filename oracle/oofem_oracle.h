/*
 * CPU oracle for the OOFEM structural hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm, used by the test suite,
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, as the reference
 * the GPU results are compared with.
 * The product (liboofem_gb300.so) never links, loads or calls anything here.
 *
 * Parity pin: this restatement is checked against golden vectors produced by
 * the reference executable itself (tests/golden/, generated by
 * tests/golden/make_golden.py through oracle/ref_harness.C) and against the
 * golden values embedded in the reference's own decks (tests/sm/patch*.in).
 *
 * Conventions (all arrays row-major, C order):
 *   element types: 1 = LSpace (hex8), 2 = PlaneStress2d (quad4), 3 = LTRSpace (tet4)
 *   eq[node*ndofpn + d]: +k (1-based free equation) or -k (1-based prescribed)
 *   loc[e*nloc + a*ndofpn + d]: 1-based free equation or 0 (prescribed)
 *   CSR: rowptr (int64, neq+1), colind (int32, 0-based, sorted per row)
 *   Voigt order xx,yy,zz,yz,zx,xy (3D), xx,yy,xy (plane stress), engineering shear.
 *   materials: rows of 8 doubles  {kind, E, nu, sig0, H, e0, gf, 0}
 *              kind 1 = isole, 2 = misesmat (htype 0), 3 = idm1 (Mazars, exp. cohesive)
 */
#ifndef OOFEM_ORACLE_H
#define OOFEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int  oro_threads(void);
int  oro_nnpe(int etype);
int  oro_ndofpn(int etype);
int  oro_ngp(int etype);
int  oro_nstress(int etype);

int  oro_number_equations(int nnodes, int ndofpn, const uint8_t *bc_mask, int *eq, int *npeq);
void oro_location_arrays(int nelem, int nnpe, const int *conn, int ndofpn, const int *eq, int *loc);
void oro_prescribed_location_arrays(int nelem, int nnpe, const int *conn, int ndofpn, const int *eq, int *ploc);
int64_t oro_build_pattern(int neq, int nelem, int nloc, const int *loc, int64_t *rowptr, int *colind);

void oro_isole_d3d(double E, double nu, double *D36);
void oro_isole_dps(double E, double nu, double *D9);

int  oro_gp_gradients(int etype, const double *xe, int gp, double thickness,
                      double *dndx, double *dndx_shear, double *dV);
void oro_elem_stiffness(int etype, const double *xe, const double *Dgp, int d_per_gp,
                        double thickness, int symmetric, double *Ke);
void oro_elem_strains(int etype, const double *xe, const double *ue, double *eps);
void oro_elem_internal_force(int etype, const double *xe, const double *sig, double thickness,
                             double *fe);

void oro_gather_element(int etype, int ndim, const double *coords, const int *conn, int e, double *xe);

void oro_assemble_linear(int etype, int ndim, int nnodes, const double *coords, int nelem,
                         const int *conn, const int *elem_mat, const double *mats, double thickness,
                         int nloc, const int *loc, int neq, const int64_t *rowptr, const int *colind,
                         double *val);

void oro_spmv(int neq, const int64_t *rowptr, const int *colind, const double *val,
              const double *x, double *y);
int  oro_pcg(int neq, const int64_t *rowptr, const int *colind, const double *val,
             const double *b, double *x, double rtol, int maxit, int *iters, double *achieved);

/* Material state per Gauss point, 24 doubles (committed + temp):
 *  [0..5]   committed plastic strain (misesmat) / [0] kappa,[1] omega,[2] Le (idm1)
 *  [6]      committed kappa (misesmat)
 *  [7]      committed omega (misesmat, unused: no damage)
 *  [8..13]  temp plastic strain / idm1: [8] temp kappa, [9] temp omega
 *  [14]     temp kappa (misesmat)
 *  [15..20] trial deviatoric stress (misesmat)
 *  [21]     trial volumetric stress (misesmat)
 *  [22..23] spare
 */
#define ORO_NSTATE 24

void oro_material_stress(int etype, const double *mat, const double *eps, double *state,
                         double le_hint, const double *xe, double *sig);
void oro_material_tangent(int etype, const double *mat, const double *state, double *D);
void oro_commit_state(int etype, const double *mat, double *state);

/* Internal forces of the whole mesh for the total displacement field u_node
 * (nnodes*ndofpn, prescribed values included). Updates the temp material
 * state (nelem*ngp*ORO_NSTATE) and writes GP stresses (nelem*ngp*nstress). */
void oro_internal_forces(int etype, int ndim, int nnodes, const double *coords, int nelem,
                         const int *conn, const int *elem_mat, const double *mats,
                         double thickness, const double *u_node, double *state,
                         double *f_node, double *gp_stress, double *gp_strain, double *enorm);

void oro_assemble_tangent(int etype, int ndim, int nnodes, const double *coords, int nelem,
                          const int *conn, const int *elem_mat, const double *mats,
                          double thickness, const double *state, int nloc, const int *loc,
                          int neq, const int64_t *rowptr, const int *colind, double *val);

#ifdef __cplusplus
}
#endif
#endif
