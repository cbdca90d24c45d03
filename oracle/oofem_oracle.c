/*
 * CPU oracle for the OOFEM structural hot path -- TEST INFRASTRUCTURE ONLY.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * and only as the reference results are compared with / the timed CPU
 * baseline; the product never calls it.
 *
 * Each function restates one piece of the reference algorithm and cites the
 * reference file:line it follows (paths relative to the OOFEM source tree).
 * Parity is pinned against golden vectors written by the reference executable
 * (the .npz files under tests/golden, see tests/golden/make_golden.py).
 */
#include "oofem_oracle.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORO_PI 3.14159265358979323846

/* 2-point Gauss abscissa exactly as the reference writes it
 * (src/core/gaussintegrationrule.C:1436-1452): a 15-digit literal, not 1/sqrt(3). */
static const double GP2 = 0.577350269189626;

int oro_nnpe(int etype) { return etype == 1 ? 8 : 4; }
int oro_ndofpn(int etype) { return etype == 2 ? 2 : 3; }
int oro_ngp(int etype) { return etype == 1 ? 8 : (etype == 2 ? 4 : 1); }
int oro_nstress(int etype) { return etype == 2 ? 3 : 6; }

/* ------------------------------------------------------------------------ */
/* a1: equation numbering. EngngModel::forceEquationNumbering
 * (src/core/engngm.C:469-530) visits DOF managers in domain order and asks each
 * DOF (node DOF order D_u,D_v[,D_w]) for a number; MasterDof::askNewEquationNumber
 * (src/core/masterdof.C:105-120) gives free DOFs ++neq and prescribed -(++npeq). */
int oro_number_equations(int nnodes, int ndofpn, const uint8_t *bc_mask, int *eq, int *npeq)
{
    int neq = 0, np = 0;
    for (int n = 0; n < nnodes; ++n)
        for (int d = 0; d < ndofpn; ++d) {
            int k = n * ndofpn + d;
            eq[k] = bc_mask[k] ? -(++np) : ++neq;
        }
    if (npeq) *npeq = np;
    return neq;
}

/* a2: Element::giveLocationArray (src/core/element.C:429-454): node order x
 * DOF mask; with the default numbering scheme prescribed DOFs give 0. */
void oro_location_arrays(int nelem, int nnpe, const int *conn, int ndofpn, const int *eq, int *loc)
{
    int nloc = nnpe * ndofpn;
    for (int e = 0; e < nelem; ++e)
        for (int a = 0; a < nnpe; ++a)
            for (int d = 0; d < ndofpn; ++d) {
                int q = eq[conn[e * nnpe + a] * ndofpn + d];
                loc[e * nloc + a * ndofpn + d] = q > 0 ? q : 0;
            }
}

/* Same with the prescribed numbering (EModelDefaultPrescribedEquationNumbering):
 * prescribed DOFs give their positive prescribed number, free DOFs 0. */
void oro_prescribed_location_arrays(int nelem, int nnpe, const int *conn, int ndofpn, const int *eq, int *ploc)
{
    int nloc = nnpe * ndofpn;
    for (int e = 0; e < nelem; ++e)
        for (int a = 0; a < nnpe; ++a)
            for (int d = 0; d < ndofpn; ++d) {
                int q = eq[conn[e * nnpe + a] * ndofpn + d];
                ploc[e * nloc + a * ndofpn + d] = q < 0 ? -q : 0;
            }
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* a3: CompCol::buildInternalStructure (src/core/compcol.C:174-272): the union of
 * all element location-array pairs, one std::set per column, written out sorted
 * and 0-based. The full pattern is symmetric, so colptr/rowind of CompCol equal
 * rowptr/colind of the CSR built here. With colind == NULL only counts. */
int64_t oro_build_pattern(int neq, int nelem, int nloc, const int *loc, int64_t *rowptr, int *colind)
{
    int64_t *cnt = (int64_t *)calloc((size_t)neq + 1, sizeof(int64_t));
    for (int e = 0; e < nelem; ++e) {
        const int *l = loc + (size_t)e * nloc;
        int nz = 0;
        for (int j = 0; j < nloc; ++j) nz += l[j] > 0;
        for (int i = 0; i < nloc; ++i)
            if (l[i] > 0) cnt[l[i] - 1] += nz;
    }
    int64_t *start = (int64_t *)malloc(((size_t)neq + 1) * sizeof(int64_t));
    start[0] = 0;
    for (int r = 0; r < neq; ++r) start[r + 1] = start[r] + cnt[r];
    int *raw = (int *)malloc((size_t)(start[neq] > 0 ? start[neq] : 1) * sizeof(int));
    int64_t *fill = (int64_t *)calloc((size_t)neq + 1, sizeof(int64_t));
    for (int e = 0; e < nelem; ++e) {
        const int *l = loc + (size_t)e * nloc;
        for (int i = 0; i < nloc; ++i) {
            if (l[i] <= 0) continue;
            int r = l[i] - 1;
            for (int j = 0; j < nloc; ++j)
                if (l[j] > 0) raw[start[r] + fill[r]++] = l[j] - 1;
        }
    }
    int64_t nnz = 0;
    for (int r = 0; r < neq; ++r) {
        int *seg = raw + start[r];
        int64_t n = fill[r];
        qsort(seg, (size_t)n, sizeof(int), cmp_int);
        if (rowptr) rowptr[r] = nnz;
        int last = -1;
        for (int64_t k = 0; k < n; ++k) {
            if (seg[k] != last) {
                if (colind) colind[nnz] = seg[k];
                ++nnz;
                last = seg[k];
            }
        }
    }
    if (rowptr) rowptr[neq] = nnz;
    free(cnt); free(start); free(raw); free(fill);
    return nnz;
}

/* ------------------------------------------------------------------------ */
/* a11: IsotropicLinearElasticMaterial::initTangents
 * (src/sm/Materials/isolinearelasticmaterial.C:80-88): D = 2G I_dev6 + K I6(x)I6,
 * G = E/(2(1+nu)) (:73), K = E/(3(1-2nu)); I_dev6, I6_I6 as in
 * src/core/floatmatrixf.h:954-972. */
void oro_isole_d3d(double E, double nu, double *D)
{
    double G = E / (2.0 * (1. + nu));
    double K = E / (3.0 * (1. - 2. * nu));
    static const double Idev[36] = {
        2. / 3., -1. / 3., -1. / 3., 0, 0, 0,
        -1. / 3., 2. / 3., -1. / 3., 0, 0, 0,
        -1. / 3., -1. / 3., 2. / 3., 0, 0, 0,
        0, 0, 0, 0.5, 0, 0,
        0, 0, 0, 0, 0.5, 0,
        0, 0, 0, 0, 0, 0.5};
    for (int i = 0; i < 36; ++i) {
        int r = i / 6, c = i % 6;
        D[i] = 2 * G * Idev[i] + K * ((r < 3 && c < 3) ? 1.0 : 0.0);
    }
}

/* General square inverse by Gauss-Jordan with partial pivoting (n <= 6). */
static void inv_n(int n, const double *A, double *Ai)
{
    double M[6][12];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * n; ++j)
            M[i][j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
        if (p != c)
            for (int j = 0; j < 2 * n; ++j) { double t = M[c][j]; M[c][j] = M[p][j]; M[p][j] = t; }
        double piv = M[c][c];
        for (int j = 0; j < 2 * n; ++j) M[c][j] /= piv;
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = M[r][c];
            if (f != 0.0)
                for (int j = 0; j < 2 * n; ++j) M[r][j] -= f * M[c][j];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) Ai[i * n + j] = M[i][j + n];
}

/* LinearElasticMaterial::computesSubTangents (src/sm/Materials/linearelasticmaterial.C:62-79):
 * plane-stress stiffness = inverse of the (xx,yy,xy) block of the 3-D compliance. */
void oro_isole_dps(double E, double nu, double *D9)
{
    double D[36], C[36], R[9];
    oro_isole_d3d(E, nu, D);
    inv_n(6, D, C);
    static const int idx[3] = {0, 1, 5};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i * 3 + j] = C[idx[i] * 6 + idx[j]];
    inv_n(3, R, D9);
}

/* ------------------------------------------------------------------------ */
/* a4/a5/a7: Gauss point coordinates, shape-function gradients and dV.
 *  hex:  GaussIntegrationRule::SetUpPointsOnCube (gaussintegrationrule.C:190-213),
 *        i-j-k loop order, weight 1; FEI3dHexaLin::evaldNdxi/evaldNdx
 *        (src/core/fei3dhexalin.C:126-205): J = X * dN/dxi, dNdx = dN/dxi * J^-1;
 *        dV = |detJ| * w (structural3delement.C:330-342).
 *  quad: SetUpPointsOnSquare (gaussintegrationrule.C:102-121); FEI2dQuadLin
 *        (fei2dquadlin.C:80-104, 345-363); dV = |detJ| * thickness * w
 *        (structural2delement.C:118-129). PlaneStress2d evaluates the shear row of B
 *        at the element centre (planstrss.h:51, planstrss.C:98-105), returned
 *        through dndx_shear.
 *  tet:  one point (1/4,1/4,1/4), w = 1/6 (gaussintegrationrule.C:269-282, 492-507);
 *        FEI3dTetLin::evaldNdx closed form (fei3dtetlin.C:115-164).
 * dndx is nnpe x 3 (or x 2), row-major. Returns 0 on success, -1 on detJ <= 0 for tets. */
static void quad_dndx(const double *xe, double ksi, double eta, double *dndx, double *detJ)
{
    double dn[2][4] = {
        {0.25 * (1. + eta), -0.25 * (1. + eta), -0.25 * (1. - eta), 0.25 * (1. - eta)},
        {0.25 * (1. + ksi), 0.25 * (1. - ksi), -0.25 * (1. - ksi), -0.25 * (1. + ksi)}};
    double j00 = 0, j01 = 0, j10 = 0, j11 = 0;   /* jacT as in fei2dquadlin.C:80-96 */
    for (int i = 0; i < 4; ++i) {
        double x = xe[i * 2 + 0], y = xe[i * 2 + 1];
        j00 += dn[0][i] * x; j01 += dn[0][i] * y;
        j10 += dn[1][i] * x; j11 += dn[1][i] * y;
    }
    double det = j00 * j11 - j01 * j10;
    double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
    for (int i = 0; i < 4; ++i) {
        dndx[i * 2 + 0] = i00 * dn[0][i] + i01 * dn[1][i];
        dndx[i * 2 + 1] = i10 * dn[0][i] + i11 * dn[1][i];
    }
    *detJ = det;
}

int oro_gp_gradients(int etype, const double *xe, int gp, double thickness,
                     double *dndx, double *dndx_shear, double *dV)
{
    if (etype == 1) {
        double c[2] = {-GP2, GP2};
        double u = c[gp / 4], v = c[(gp / 2) % 2], w = c[gp % 2];
        double dN[8][3] = {
            {-0.125 * (1. - v) * (1. + w), -0.125 * (1. - u) * (1. + w), 0.125 * (1. - u) * (1. - v)},
            {-0.125 * (1. + v) * (1. + w), 0.125 * (1. - u) * (1. + w), 0.125 * (1. - u) * (1. + v)},
            {0.125 * (1. + v) * (1. + w), 0.125 * (1. + u) * (1. + w), 0.125 * (1. + u) * (1. + v)},
            {0.125 * (1. - v) * (1. + w), -0.125 * (1. + u) * (1. + w), 0.125 * (1. + u) * (1. - v)},
            {-0.125 * (1. - v) * (1. - w), -0.125 * (1. - u) * (1. - w), -0.125 * (1. - u) * (1. - v)},
            {-0.125 * (1. + v) * (1. - w), 0.125 * (1. - u) * (1. - w), -0.125 * (1. - u) * (1. + v)},
            {0.125 * (1. + v) * (1. - w), 0.125 * (1. + u) * (1. - w), -0.125 * (1. + u) * (1. + v)},
            {0.125 * (1. - v) * (1. - w), -0.125 * (1. + u) * (1. - w), -0.125 * (1. + u) * (1. - v)}};
        double J[3][3] = {{0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int k = 0; k < 8; ++k) s += xe[k * 3 + i] * dN[k][j];
                J[i][j] = s;
            }
        double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        double Ji[3][3];
        Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        for (int a = 0; a < 8; ++a)
            for (int j = 0; j < 3; ++j)
                dndx[a * 3 + j] = dN[a][0] * Ji[0][j] + dN[a][1] * Ji[1][j] + dN[a][2] * Ji[2][j];
        if (dndx_shear) memcpy(dndx_shear, dndx, 24 * sizeof(double));
        *dV = fabs(det) * 1.0;
        return 0;
    } else if (etype == 2) {
        double c[2] = {-GP2, GP2};
        double ksi = c[gp / 2], eta = c[gp % 2];
        double det, det0;
        quad_dndx(xe, ksi, eta, dndx, &det);
        if (dndx_shear) quad_dndx(xe, 0.0, 0.0, dndx_shear, &det0);
        *dV = fabs(det) * thickness * 1.0;
        return 0;
    } else {
        double x1 = xe[0], x2 = xe[3], x3 = xe[6], x4 = xe[9];
        double y1 = xe[1], y2 = xe[4], y3 = xe[7], y4 = xe[10];
        double z1 = xe[2], z2 = xe[5], z3 = xe[8], z4 = xe[11];
        double detJ = ((x4 - x1) * (y2 - y1) * (z3 - z1) - (x4 - x1) * (y3 - y1) * (z2 - z1) +
                       (x3 - x1) * (y4 - y1) * (z2 - z1) - (x2 - x1) * (y4 - y1) * (z3 - z1) +
                       (x2 - x1) * (y3 - y1) * (z4 - z1) - (x3 - x1) * (y2 - y1) * (z4 - z1));
        if (detJ <= 0.0) return -1;
        double a[12];
        a[0] = -((y3 - y2) * (z4 - z2) - (y4 - y2) * (z3 - z2));
        a[3] = (y4 - y3) * (z1 - z3) - (y1 - y3) * (z4 - z3);
        a[6] = -((y1 - y4) * (z2 - z4) - (y2 - y4) * (z1 - z4));
        a[9] = (y2 - y1) * (z3 - z1) - (y3 - y1) * (z2 - z1);
        a[1] = -((x4 - x2) * (z3 - z2) - (x3 - x2) * (z4 - z2));
        a[4] = (x1 - x3) * (z4 - z3) - (x4 - x3) * (z1 - z3);
        a[7] = -((x2 - x4) * (z1 - z4) - (x1 - x4) * (z2 - z4));
        a[10] = (x3 - x1) * (z2 - z1) - (x2 - x1) * (z3 - z1);
        a[2] = -((x3 - x2) * (y4 - y2) - (x4 - x2) * (y3 - y2));
        a[5] = (x4 - x3) * (y1 - y3) - (x1 - x3) * (y4 - y3);
        a[8] = -((x1 - x4) * (y2 - y4) - (x2 - x4) * (y1 - y4));
        a[11] = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
        double s = 1. / detJ;
        for (int i = 0; i < 12; ++i) dndx[i] = a[i] * s;
        if (dndx_shear) memcpy(dndx_shear, dndx, 12 * sizeof(double));
        *dV = fabs(detJ) * (1.0 / 6.0);
        return 0;
    }
}

/* a6: B matrix (nstress x nloc), row-major.
 * 3-D: Structural3DElement::computeBmatrixAt (structural3delement.C:63-85) /
 *      LSpace::computeBmatrixAt (lspace.C:104-131), rows xx,yy,zz,yz,zx,xy.
 * PS:  PlaneStress2d::computeBmatrixAt (planstrss.C:78-106), rows xx,yy,xy with the
 *      shear row from the centre gradients. */
static void bmatrix(int etype, const double *dndx, const double *dsh, double *B)
{
    int nn = oro_nnpe(etype);
    if (etype == 2) {
        memset(B, 0, 3 * 8 * sizeof(double));
        for (int i = 0; i < 4; ++i) {
            B[0 * 8 + 2 * i] = dndx[i * 2 + 0];
            B[1 * 8 + 2 * i + 1] = dndx[i * 2 + 1];
            B[2 * 8 + 2 * i] = dsh[i * 2 + 1];
            B[2 * 8 + 2 * i + 1] = dsh[i * 2 + 0];
        }
        return;
    }
    int nl = nn * 3;
    memset(B, 0, 6 * nl * sizeof(double));
    for (int i = 0; i < nn; ++i) {
        double gx = dndx[i * 3], gy = dndx[i * 3 + 1], gz = dndx[i * 3 + 2];
        B[0 * nl + 3 * i] = gx;
        B[1 * nl + 3 * i + 1] = gy;
        B[2 * nl + 3 * i + 2] = gz;
        B[3 * nl + 3 * i + 1] = gz; B[3 * nl + 3 * i + 2] = gy;
        B[4 * nl + 3 * i] = gz;     B[4 * nl + 3 * i + 2] = gx;
        B[5 * nl + 3 * i] = gy;     B[5 * nl + 3 * i + 1] = gx;
    }
}

/* a8: NLStructuralElement::computeStiffnessMatrix, small-strain branch
 * (src/sm/Elements/nlstructuralelement.C:345-376): K = sum_gp B^T (D B) dV,
 * upper triangle via plusProductSymmUpper + symmetrized (floatmatrix.C:1243, 1137)
 * when the material tangent is symmetric, full plusProductUnsym (:691) otherwise.
 * Dgp holds d_per_gp ? one D per GP : one D for all GPs. Ke is nloc x nloc row-major. */
void oro_elem_stiffness(int etype, const double *xe, const double *Dgp, int d_per_gp,
                        double thickness, int symmetric, double *Ke)
{
    int nn = oro_nnpe(etype), ndof = oro_ndofpn(etype), ng = oro_ngp(etype);
    int ns = oro_nstress(etype), nl = nn * ndof;
    double dndx[24], dsh[24], dV, B[6 * 24], DB[6 * 24];
    memset(Ke, 0, (size_t)nl * nl * sizeof(double));
    for (int g = 0; g < ng; ++g) {
        oro_gp_gradients(etype, xe, g, thickness, dndx, dsh, &dV);
        bmatrix(etype, dndx, dsh, B);
        const double *D = Dgp + (d_per_gp ? (size_t)g * ns * ns : 0);
        for (int i = 0; i < ns; ++i)
            for (int j = 0; j < nl; ++j) {
                double s = 0;
                for (int k = 0; k < ns; ++k) s += D[i * ns + k] * B[k * nl + j];
                DB[i * nl + j] = s;
            }
        for (int i = 0; i < nl; ++i)
            for (int j = symmetric ? i : 0; j < nl; ++j) {
                double s = 0;
                for (int k = 0; k < ns; ++k) s += B[k * nl + i] * DB[k * nl + j];
                Ke[i * nl + j] += s * dV;
            }
    }
    if (symmetric)
        for (int i = 0; i < nl; ++i)
            for (int j = 0; j < i; ++j) Ke[i * nl + j] = Ke[j * nl + i];
}

/* eps (ngp x nstress) = B u_e per GP (StructuralElement::computeStrainVector,
 * structuralelement.C:723-745 small-strain path). */
void oro_elem_strains(int etype, const double *xe, const double *ue, double *eps)
{
    int nn = oro_nnpe(etype), ndof = oro_ndofpn(etype), ng = oro_ngp(etype);
    int ns = oro_nstress(etype), nl = nn * ndof;
    double dndx[24], dsh[24], dV, B[6 * 24];
    for (int g = 0; g < ng; ++g) {
        oro_gp_gradients(etype, xe, g, 1.0, dndx, dsh, &dV);
        bmatrix(etype, dndx, dsh, B);
        for (int i = 0; i < ns; ++i) {
            double s = 0;
            for (int j = 0; j < nl; ++j) s += B[i * nl + j] * ue[j];
            eps[g * ns + i] = s;
        }
    }
}

/* a9: NLStructuralElement::giveInternalForcesVector, nlGeometry 0
 * (nlstructuralelement.C:151-240): f = sum_gp B^T sigma dV. */
void oro_elem_internal_force(int etype, const double *xe, const double *sig, double thickness,
                             double *fe)
{
    int nn = oro_nnpe(etype), ndof = oro_ndofpn(etype), ng = oro_ngp(etype);
    int ns = oro_nstress(etype), nl = nn * ndof;
    double dndx[24], dsh[24], dV, B[6 * 24];
    memset(fe, 0, (size_t)nl * sizeof(double));
    for (int g = 0; g < ng; ++g) {
        oro_gp_gradients(etype, xe, g, thickness, dndx, dsh, &dV);
        bmatrix(etype, dndx, dsh, B);
        for (int j = 0; j < nl; ++j) {
            double s = 0;
            for (int i = 0; i < ns; ++i) s += B[i * nl + j] * sig[g * ns + i];
            fe[j] += s * dV;
        }
    }
}

void oro_gather_element(int etype, int ndim, const double *coords, const int *conn, int e, double *xe)
{
    int nn = oro_nnpe(etype);
    for (int a = 0; a < nn; ++a)
        for (int d = 0; d < ndim; ++d) xe[a * ndim + d] = coords[(size_t)conn[(size_t)e * nn + a] * ndim + d];
}

/* a14: CompCol::assemble (src/core/compcol.C:275-316): val[pos(i,j)] += Ke(i,j)
 * for every pair of nonzero locations, elements in domain order. */
static void csr_add(const int64_t *rowptr, const int *colind, double *val, int r, int c, double v)
{
    int64_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        if (colind[mid] < c) lo = mid + 1;
        else if (colind[mid] > c) hi = mid - 1;
        else { val[mid] += v; return; }
    }
}

static void material_D(int etype, const double *mat, double *D)
{
    if (etype == 2) oro_isole_dps(mat[1], mat[2], D);
    else oro_isole_d3d(mat[1], mat[2], D);
}

void oro_assemble_linear(int etype, int ndim, int nnodes, const double *coords, int nelem,
                         const int *conn, const int *elem_mat, const double *mats, double thickness,
                         int nloc, const int *loc, int neq, const int64_t *rowptr, const int *colind,
                         double *val)
{
    (void)nnodes; (void)neq;
    double xe[24], D[36], Ke[576];
    memset(val, 0, (size_t)rowptr[neq] * sizeof(double));
    for (int e = 0; e < nelem; ++e) {
        oro_gather_element(etype, ndim, coords, conn, e, xe);
        material_D(etype, mats + 8 * elem_mat[e], D);
        oro_elem_stiffness(etype, xe, D, 0, thickness, 1, Ke);
        const int *l = loc + (size_t)e * nloc;
        for (int j = 0; j < nloc; ++j) {
            if (!l[j]) continue;
            for (int i = 0; i < nloc; ++i)
                if (l[i]) csr_add(rowptr, colind, val, l[i] - 1, l[j] - 1, Ke[i * nloc + j]);
        }
    }
}

/* a16: y = A x (CompCol::times, compcol.C:128-143, on the full symmetric pattern). */
void oro_spmv(int neq, const int64_t *rowptr, const int *colind, const double *val,
              const double *x, double *y)
{
    for (int r = 0; r < neq; ++r) {
        double s = 0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += val[k] * x[colind[k]];
        y[r] = s;
    }
}

static double dot(int n, const double *a, const double *b)
{
    double s = 0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* a17: IML++ CG (iml/cg.h:22-71) with DiagPreconditioner (src/core/iml/diagpre.C:40-67):
 * x0 = incoming x, r = b - A x, stop when ||r_k||/||b|| <= rtol on the recursively
 * updated r; ||b|| = 0 is replaced by 1. Returns 0 when converged, 1 otherwise,
 * -1 on a zero diagonal (the reference raises an error there). */
int oro_pcg(int neq, const int64_t *rowptr, const int *colind, const double *val,
            const double *b, double *x, double rtol, int maxit, int *iters, double *achieved)
{
    double *r = (double *)malloc((size_t)neq * sizeof(double));
    double *z = (double *)malloc((size_t)neq * sizeof(double));
    double *p = (double *)malloc((size_t)neq * sizeof(double));
    double *q = (double *)malloc((size_t)neq * sizeof(double));
    double *dinv = (double *)malloc((size_t)neq * sizeof(double));
    int status = 1;
    for (int i = 0; i < neq; ++i) {
        double d = 0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (colind[k] == i) d = val[k];
        if (d == 0) { status = -1; goto done; }
        dinv[i] = 1. / d;
    }
    {
        double normb = sqrt(dot(neq, b, b));
        oro_spmv(neq, rowptr, colind, val, x, q);
        for (int i = 0; i < neq; ++i) r[i] = b[i] - q[i];
        if (normb == 0.0) normb = 1;
        double resid = sqrt(dot(neq, r, r)) / normb;
        *iters = 0;
        if (resid <= rtol) { *achieved = resid; status = 0; goto done; }
        double rho, rho1 = 0;
        for (int it = 1; it <= maxit; ++it) {
            for (int i = 0; i < neq; ++i) z[i] = r[i] * dinv[i];
            rho = dot(neq, r, z);
            if (it == 1) memcpy(p, z, (size_t)neq * sizeof(double));
            else {
                double beta = rho / rho1;
                for (int i = 0; i < neq; ++i) p[i] = z[i] + beta * p[i];
            }
            oro_spmv(neq, rowptr, colind, val, p, q);
            double alpha = rho / dot(neq, p, q);
            for (int i = 0; i < neq; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            resid = sqrt(dot(neq, r, r)) / normb;
            *iters = it;
            if (resid <= rtol) { *achieved = resid; status = 0; goto done; }
            rho1 = rho;
        }
        *achieved = resid;
        status = 1;
    }
done:
    free(r); free(z); free(p); free(q); free(dinv);
    return status;
}

/* ------------------------------------------------------------------------ */
/* Material point updates. */

/* a12: MisesMat::performPlasticityReturn, 3-D branch (src/sm/Materials/misesmat.C:181-263),
 * htype 0 (computeYieldStress :404-409, prime :426-431), no damage (omega_crit 0 ->
 * computeDamage gives 0, :472-483). Helpers: StructuralMaterial::
 * computeDeviatoricVolumetricSplit / applyDeviatoricElasticStiffness /
 * applyDeviatoricElasticCompliance / computeStressNorm / computeDeviatoricVolumetricSum
 * (structuralmaterial.C:1489-1600). */
static void mises_stress_3d(const double *mat, const double *eps, double *st, double *sig)
{
    double E = mat[1], nu = mat[2], sig0 = mat[3], H = mat[4];
    double G = E / (2.0 * (1. + nu));
    double K = E / (3.0 * (1. - 2. * nu));
    double pl[6];
    for (int i = 0; i < 6; ++i) pl[i] = st[i];
    double kappa = st[6];
    double el[6];
    for (int i = 0; i < 6; ++i) el[i] = eps[i] - pl[i];
    double mean = (el[0] + el[1] + el[2]) / 3.0;
    double dev[6] = {el[0] - mean, el[1] - mean, el[2] - mean, el[3], el[4], el[5]};
    double s[6] = {2. * G * dev[0], 2. * G * dev[1], 2. * G * dev[2], G * dev[3], G * dev[4], G * dev[5]};
    double svol = 3 * K * mean;
    for (int i = 0; i < 6; ++i) st[15 + i] = s[i];
    st[21] = svol;
    double trialS = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
                         2. * s[3] * s[3] + 2. * s[4] * s[4] + 2. * s[5] * s[5]);
    double yieldValue = sqrt(3. / 2.) * trialS - (sig0 + H * kappa);
    if (yieldValue > 0.) {
        double dKappa = yieldValue / (H + 3. * G);
        kappa += dKappa;
        /* applyDeviatoricElasticCompliance(trialStressDev, 0.5) (misesmat.C:244) */
        double dpl[6] = {1. / (2. * 0.5) * s[0], 1. / (2. * 0.5) * s[1], 1. / (2. * 0.5) * s[2],
                         1. / 0.5 * s[3], 1. / 0.5 * s[4], 1. / 0.5 * s[5]};
        double f = sqrt(3. / 2.) * dKappa / trialS;
        for (int i = 0; i < 6; ++i) pl[i] += f * dpl[i];
        double sc = 1. - sqrt(6.) * G * dKappa / trialS;
        for (int i = 0; i < 6; ++i) s[i] *= sc;
    }
    sig[0] = s[0] + svol; sig[1] = s[1] + svol; sig[2] = s[2] + svol;
    sig[3] = s[3]; sig[4] = s[4]; sig[5] = s[5];
    for (int i = 0; i < 6; ++i) st[8 + i] = pl[i];
    st[14] = kappa;
}

/* MisesMat::give3dMaterialStiffnessMatrix (misesmat.C:496-535), TangentStiffness,
 * omega = 0. Reads the committed kappa (st[6]), temp kappa (st[14]) and the stored
 * trial deviator (st[15..20]). */
static void mises_tangent_3d(const double *mat, const double *st, double *D)
{
    double E = mat[1], nu = mat[2], sig0 = mat[3], H = mat[4];
    double G = E / (2.0 * (1. + nu));
    oro_isole_d3d(E, nu, D);
    double kappa = st[6], tempKappa = st[14];
    double dKappa = tempKappa - kappa;
    if (dKappa <= 0.0) return;
    double sigmaY = sig0 + H * kappa;
    const double *s = st + 15;
    double trialS = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
                         2. * s[3] * s[3] + 2. * s[4] * s[4] + 2. * s[5] * s[5]);
    double factor = -2. * sqrt(6.) * G * G / trialS;
    double factor1 = factor * sigmaY / ((H + 3. * G) * trialS * trialS);
    double factor2 = factor * dKappa;
    static const double Idev[36] = {
        2. / 3., -1. / 3., -1. / 3., 0, 0, 0,
        -1. / 3., 2. / 3., -1. / 3., 0, 0, 0,
        -1. / 3., -1. / 3., 2. / 3., 0, 0, 0,
        0, 0, 0, 0.5, 0, 0,
        0, 0, 0, 0, 0.5, 0,
        0, 0, 0, 0, 0, 0.5};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) D[i * 6 + j] += factor1 * s[i] * s[j];
    for (int i = 0; i < 36; ++i) D[i] += factor2 * Idev[i];
}

/* Principal strains of a 3-D strain vector (engineering shears) as
 * StructuralMaterial::computePrincipalValues (structuralmaterial.C:1107-1262) gives
 * them: zeros unless some component exceeds 1e-20 in magnitude; the invariants
 * I1, I2, I3 of the tensor with halved shears; the real roots of
 * -x^3 + I1 x^2 - I2 x + I3 by the trigonometric form of cubic3r
 * (mathfem.C:155-240: a triple root when q and r vanish below 1e-100, the cosine
 * argument clamped to [-1, 1]); sorted in descending order. */
static void principal_strains(const double *e, double *w)
{
    int nonzero = 0;
    for (int i = 0; i < 6; ++i)
        if (fabs(e[i]) > 1.e-20) nonzero = 1;
    w[0] = w[1] = w[2] = 0.0;
    if (!nonzero) return;
    double I1 = e[0] + e[1] + e[2];
    double I2 = e[0] * e[1] + e[1] * e[2] + e[2] * e[0] - 0.25 * (e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
    double I3 = e[0] * e[1] * e[2] + 0.25 * (e[3] * e[4] * e[5] - e[0] * e[3] * e[3] - e[1] * e[4] * e[4] -
                                             e[2] * e[5] * e[5]);
    /* monic form x^3 + a x^2 + b x + c of the cubic with leading coefficient -1 */
    double a = I1 / -1.0, b = -I2 / -1.0, c = I3 / -1.0;
    double q = (a * a - 3.0 * b) / 9.0;
    double r = (2.0 * a * a * a - 9.0 * a * b + 27.0 * c) / 54.0;
    if (fabs(q) < 1.0e-100 && fabs(r) < 1.0e-100) {
        w[0] = w[1] = w[2] = -a / 3.0;
    } else {
        double h = r / sqrt(q * q * q);
        if (fabs(h) > 1.0) h = h > 0 ? 1.0 : -1.0;
        double phi = acos(h), p = sqrt(q);
        w[0] = -2.0 * p * cos(phi / 3.0) - a / 3.0;
        w[1] = -2.0 * p * cos((phi + 2.0 * ORO_PI) / 3.0) - a / 3.0;
        w[2] = -2.0 * p * cos((phi - 2.0 * ORO_PI) / 3.0) - a / 3.0;
    }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            if (w[j + 1] > w[j]) { double t = w[j]; w[j] = w[j + 1]; w[j + 1] = t; }
}

/* Principal values and directions of a symmetric 3x3 matrix as
 * StructuralMaterial::computePrincipalValDir obtains them (structuralmaterial.C:1337-1470
 * with FloatMatrix::jaco_ to 10 significant figures, floatmatrix.C:1953-2120):
 * threshold Jacobi rotations over the pairs (0,1), (0,2), (1,2) in that order; a
 * pair is rotated when |a_pq| exceeds 1e-10 of the sum of the absolute entries of
 * the input, by half of atan2(2 a_pq, a_pp - a_qq); sweeps stop once the rotated
 * entries of a sweep sum to no more than that fraction (51 sweeps at most). The
 * loose stopping rule is part of the result (the crack normal of a damaged point
 * carries it). Values sorted descending with their vectors (columns of V). */
static void principal_dirs(const double *S, double *w, double *V)
{
    double u[3][3];   /* upper triangle is the working matrix, as in jaco_ */
    double ev[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            u[i][j] = S[i * 3 + j];
            V[i * 3 + j] = i == j ? 1.0 : 0.0;
        }
    for (int i = 0; i < 3; ++i) ev[i] = u[i][i];
    const double tol = pow(0.1, 10);
    double sum = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sum += fabs(u[i][j]);
    if (sum > 0.0) {
        int sweeps = 0;
        double ssum;
        do {
            ssum = 0.0;
            for (int j = 1; j < 3; ++j)
                for (int i = 0; i < j; ++i) {
                    if (!(fabs(u[i][j]) / sum > tol)) continue;
                    ssum += fabs(u[i][j]);
                    double ang = atan2(u[i][j] * 2.0, ev[i] - ev[j]) / 2.0;
                    double si = sin(ang), co = cos(ang), t;
                    for (int k = 0; k < i; ++k) {
                        t = u[k][i];
                        u[k][i] = co * t + si * u[k][j];
                        u[k][j] = -si * t + co * u[k][j];
                    }
                    t = ev[i];
                    ev[i] = co * t + si * u[i][j];
                    double aij = -si * t + co * u[i][j];
                    for (int k = i + 1; k < j; ++k) {
                        t = u[i][k];
                        u[i][k] = co * t + si * u[k][j];
                        u[k][j] = -si * t + co * u[k][j];
                    }
                    t = u[i][j];
                    double aji = co * t + si * ev[j];
                    ev[j] = -si * t + co * ev[j];
                    for (int k = j + 1; k < 3; ++k) {
                        t = u[i][k];
                        u[i][k] = co * t + si * u[j][k];
                        u[j][k] = -si * t + co * u[j][k];
                    }
                    for (int k = 0; k < 3; ++k) {
                        t = V[k * 3 + i];
                        V[k * 3 + i] = co * t + si * V[k * 3 + j];
                        V[k * 3 + j] = -si * t + co * V[k * 3 + j];
                    }
                    ev[i] = co * ev[i] + si * aji;
                    ev[j] = -si * aij + co * ev[j];
                    u[i][j] = 0.0;
                }
        } while (++sweeps <= 50 && fabs(ssum) / sum > tol);
    }
    for (int ii = 0; ii < 2; ++ii)
        for (int jj = 0; jj < 2; ++jj)
            if (ev[jj + 1] > ev[jj]) {
                double t = ev[jj]; ev[jj] = ev[jj + 1]; ev[jj + 1] = t;
                for (int k = 0; k < 3; ++k) {
                    t = V[k * 3 + jj]; V[k * 3 + jj] = V[k * 3 + jj + 1]; V[k * 3 + jj + 1] = t;
                }
            }
    for (int i = 0; i < 3; ++i) w[i] = ev[i];
}

/* a13: IsotropicDamageMaterial1 with Mazars equivalent strain (idm1.C:436-470,
 * principal strains of the tensor with halved shears), exponential cohesive-crack
 * softening (damlaw 0 with gf: idm1.C:121-130, 808-911; wf = gf/(E e0), ef = wf/Le,
 * Newton on (1-w)k - e0 exp(-w k/ef) until |R| < e0*1e-9, at most 40 steps),
 * crack-band length on first damage (initDamaged idm1.C:1168-1322: normal = principal
 * direction of the largest principal strain, Le = Element::giveLengthInDir
 * element.C:1162-1183), loading criterion on kappa (isodamagemodel.C:86-160),
 * stress = (1-omega) D eps. State: [0] kappa, [1] omega committed, [2] Le;
 * [8] kappa, [9] omega temp. */
static void idm1_stress_3d(const double *mat, const double *eps, double *st,
                           const double *xe, int nnpe, double *sig)
{
    double E = mat[1], nu = mat[2], e0 = mat[5], gf = mat[6];
    double T[9] = {eps[0], 0.5 * eps[5], 0.5 * eps[4],
                   0.5 * eps[5], eps[1], 0.5 * eps[3],
                   0.5 * eps[4], 0.5 * eps[3], eps[2]};
    double w[3], V[9];
    principal_strains(eps, w);
    double pos = 0;
    for (int i = 0; i < 3; ++i)
        if (w[i] > 0.0) pos += w[i] * w[i];
    double equiv = sqrt(pos);
    double kappa0 = st[0], omega0 = st[1], le = st[2];
    double tempKappa, omega;
    if (equiv - kappa0 <= 0.0) {
        tempKappa = kappa0;
        omega = omega0;
    } else {
        tempKappa = equiv;
        if (tempKappa > e0 && (omega0 == 0.0 || le == 0.0)) {
            principal_dirs(T, w, V);
            int indx = 0;
            for (int i = 1; i < 3; ++i)
                if (w[i] > w[indx]) indx = i;
            double n[3] = {V[0 * 3 + indx], V[1 * 3 + indx], V[2 * 3 + indx]};
            double mx = 0, mn = 0;
            for (int a = 0; a < nnpe; ++a) {
                double d = n[0] * xe[a * 3] + n[1] * xe[a * 3 + 1] + n[2] * xe[a * 3 + 2];
                if (a == 0) mx = mn = d;
                else if (d > mx) mx = d;
                else if (d < mn) mn = d;
            }
            le = mx - mn;
        }
        omega = 0.0;
        if (tempKappa > e0) {
            double wf = gf / E / e0;
            double ef = wf / le;
            int nite = 0;
            double R;
            do {
                nite++;
                double help = omega * tempKappa / ef;
                R = (1. - omega) * tempKappa - e0 * exp(-help);
                double Lhs = tempKappa - e0 * exp(-help) * tempKappa / ef;
                omega += R / Lhs;
                if (nite > 40) break;
            } while (fabs(R) >= e0 * 1e-9);
        }
    }
    double D[36];
    oro_isole_d3d(E, nu, D);
    for (int i = 0; i < 6; ++i) {
        double s = 0;
        for (int k = 0; k < 6; ++k) s += D[i * 6 + k] * eps[k];
        sig[i] = (1.0 - omega) * s;
    }
    st[8] = tempKappa;
    st[9] = omega;
    st[2] = le;   /* the reference stores Le directly in the status (setLe), not as a temp value */
}

void oro_material_stress(int etype, const double *mat, const double *eps, double *state,
                         double le_hint, const double *xe, double *sig)
{
    (void)le_hint;
    int kind = (int)mat[0];
    int ns = oro_nstress(etype);
    if (kind == 2 && etype != 2) {
        mises_stress_3d(mat, eps, state, sig);
    } else if (kind == 3 && etype != 2) {
        idm1_stress_3d(mat, eps, state, xe, oro_nnpe(etype), sig);
    } else {
        double D[36];
        material_D(etype, mat, D);
        for (int i = 0; i < ns; ++i) {
            double s = 0;
            for (int k = 0; k < ns; ++k) s += D[i * ns + k] * eps[k];
            sig[i] = s;
        }
    }
}

void oro_material_tangent(int etype, const double *mat, const double *state, double *D)
{
    int kind = (int)mat[0];
    if (kind == 2 && etype != 2) {
        mises_tangent_3d(mat, state, D);
    } else if (kind == 3 && etype != 2) {
        /* IsotropicDamageMaterial::give3dMaterialStiffnessMatrix (isodamagemodel.C:63-81):
         * (1 - min(omega, maxOmega)) D, maxOmega = 0.999999 (isodamagemodel.h:167). */
        oro_isole_d3d(mat[1], mat[2], D);
        double om = state[9] < 0.999999 ? state[9] : 0.999999;
        for (int i = 0; i < 36; ++i) D[i] *= (1.0 - om);
    } else {
        material_D(etype, mat, D);
    }
}

/* MaterialStatus::updateYourself: temp -> committed. */
void oro_commit_state(int etype, const double *mat, double *st)
{
    (void)etype;
    int kind = (int)mat[0];
    if (kind == 2) {
        for (int i = 0; i < 6; ++i) st[i] = st[8 + i];
        st[6] = st[14];
    } else if (kind == 3) {
        st[0] = st[8]; st[1] = st[9];
    }
}

/* a9/a15: internal forces over all elements (EngngModel::assembleVectorFromElements,
 * engngm.C:1351-1533, with InternalForceAssembler), node-indexed output; enorm
 * (optional, ndofpn) receives the per-DOF-id sums of squared element force
 * entries that NRSolver uses as internalForcesEBENorm. */
void oro_internal_forces(int etype, int ndim, int nnodes, const double *coords, int nelem,
                         const int *conn, const int *elem_mat, const double *mats,
                         double thickness, const double *u_node, double *state,
                         double *f_node, double *gp_stress, double *gp_strain, double *enorm)
{
    int nn = oro_nnpe(etype), ndof = oro_ndofpn(etype), ng = oro_ngp(etype);
    int ns = oro_nstress(etype), nl = nn * ndof;
    double xe[24], ue[24], eps[8 * 6], sig[8 * 6], fe[24];
    memset(f_node, 0, (size_t)nnodes * ndof * sizeof(double));
    if (enorm) memset(enorm, 0, (size_t)ndof * sizeof(double));
    for (int e = 0; e < nelem; ++e) {
        oro_gather_element(etype, ndim, coords, conn, e, xe);
        for (int a = 0; a < nn; ++a)
            for (int d = 0; d < ndof; ++d)
                ue[a * ndof + d] = u_node[(size_t)conn[(size_t)e * nn + a] * ndof + d];
        oro_elem_strains(etype, xe, ue, eps);
        const double *mat = mats + 8 * elem_mat[e];
        for (int g = 0; g < ng; ++g) {
            double *st = state ? state + ((size_t)e * ng + g) * ORO_NSTATE : NULL;
            double dummy[ORO_NSTATE] = {0};
            oro_material_stress(etype, mat, eps + g * ns, st ? st : dummy, 0.0, xe, sig + g * ns);
        }
        if (gp_stress) memcpy(gp_stress + (size_t)e * ng * ns, sig, (size_t)ng * ns * sizeof(double));
        if (gp_strain) memcpy(gp_strain + (size_t)e * ng * ns, eps, (size_t)ng * ns * sizeof(double));
        oro_elem_internal_force(etype, xe, sig, thickness, fe);
        for (int a = 0; a < nn; ++a)
            for (int d = 0; d < ndof; ++d) {
                f_node[(size_t)conn[(size_t)e * nn + a] * ndof + d] += fe[a * ndof + d];
                /* FloatArray::assembleSquared by DOF id (engngm.C:1398-1401) */
                if (enorm) enorm[d] += fe[a * ndof + d] * fe[a * ndof + d];
            }
    }
    (void)nl;
}

/* Threads of the element loop (the reference runs its element loops with OpenMP,
 * engngm.C:900-929, and adds every element matrix inside a critical section). */
int oro_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oro_assemble_tangent(int etype, int ndim, int nnodes, const double *coords, int nelem,
                          const int *conn, const int *elem_mat, const double *mats,
                          double thickness, const double *state, int nloc, const int *loc,
                          int neq, const int64_t *rowptr, const int *colind, double *val)
{
    (void)nnodes;
    const int ng = oro_ngp(etype), ns = oro_nstress(etype);
    /* element matrices of a chunk in parallel, then added in element order: the
     * result does not depend on the thread count */
    enum { CH = 2048 };
    double *kb = (double *)malloc((size_t)CH * 576 * sizeof(double));
    memset(val, 0, (size_t)rowptr[neq] * sizeof(double));
    for (int e0 = 0; e0 < nelem; e0 += CH) {
        const int ne = nelem - e0 < CH ? nelem - e0 : CH;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int k = 0; k < ne; ++k) {
            const int e = e0 + k;
            double xe[24], D[8 * 36];
            oro_gather_element(etype, ndim, coords, conn, e, xe);
            const double *mat = mats + 8 * elem_mat[e];
            for (int g = 0; g < ng; ++g) {
                const double *st = state ? state + ((size_t)e * ng + g) * ORO_NSTATE : NULL;
                double zero[ORO_NSTATE] = {0};
                oro_material_tangent(etype, mat, st ? st : zero, D + (size_t)g * ns * ns);
            }
            oro_elem_stiffness(etype, xe, D, 1, thickness, 1, kb + (size_t)k * 576);
        }
        for (int k = 0; k < ne; ++k) {
            const double *Ke = kb + (size_t)k * 576;
            const int *l = loc + (size_t)(e0 + k) * nloc;
            for (int j = 0; j < nloc; ++j) {
                if (!l[j]) continue;
                for (int i = 0; i < nloc; ++i)
                    if (l[i]) csr_add(rowptr, colind, val, l[i] - 1, l[j] - 1, Ke[i * nloc + j]);
            }
        }
    }
    free(kb);
}
