// Element kernels: Gauss-point gradients, material point updates (K3), element
// stiffness K = sum_gp B^T D B dV (K1) and internal forces f = sum_gp B^T sigma dV
// (K2) for LSpace, PlaneStress2d and LTRSpace, all in FP64.
//
// Thread layout: one block handles EPB = 256/NPE elements. Phase 1 runs one
// thread per (element, Gauss point) and stages gradients, dV (and per-GP
// tangents or weighted stresses) in shared memory; phase 2 runs one thread per
// (element, node a) and produces the a-th block row of the element matrix or
// vector, so no thread holds more than NPE*ND*ND accumulators.
#include "internal.cuh"

namespace ogb {

// 2-point Gauss abscissa as written by the reference (gaussintegrationrule.C:1436-1452).
__device__ __constant__ double c_gp2[2] = {-0.577350269189626, 0.577350269189626};

template <int ET> struct ET_;
template <> struct ET_<OGB_LSPACE> { static constexpr int NPE = 8, NGP = 8, ND = 3, NDIM = 3, NS = 6; };
template <> struct ET_<OGB_PLANESTRESS2D> { static constexpr int NPE = 4, NGP = 4, ND = 2, NDIM = 2, NS = 3; };
template <> struct ET_<OGB_LTRSPACE> { static constexpr int NPE = 4, NGP = 1, ND = 3, NDIM = 3, NS = 6; };

// ------------------------------------------------------------------ gradients
// FEI3dHexaLin::evaldNdxi / evaldNdx (fei3dhexalin.C:126-205); GP order i-j-k
// (gaussintegrationrule.C:190-213); dV = |detJ| (structural3delement.C:330-342).
__device__ void hex_grad(const double (&x)[8][3], int gp, double (&g)[8][3], double &dV)
{
    double u = c_gp2[gp >> 2], v = c_gp2[(gp >> 1) & 1], w = c_gp2[gp & 1];
    double dN[8][3] = {
        {-0.125 * (1. - v) * (1. + w), -0.125 * (1. - u) * (1. + w), 0.125 * (1. - u) * (1. - v)},
        {-0.125 * (1. + v) * (1. + w), 0.125 * (1. - u) * (1. + w), 0.125 * (1. - u) * (1. + v)},
        {0.125 * (1. + v) * (1. + w), 0.125 * (1. + u) * (1. + w), 0.125 * (1. + u) * (1. + v)},
        {0.125 * (1. - v) * (1. + w), -0.125 * (1. + u) * (1. + w), 0.125 * (1. + u) * (1. - v)},
        {-0.125 * (1. - v) * (1. - w), -0.125 * (1. - u) * (1. - w), -0.125 * (1. - u) * (1. - v)},
        {-0.125 * (1. + v) * (1. - w), 0.125 * (1. - u) * (1. - w), -0.125 * (1. - u) * (1. + v)},
        {0.125 * (1. + v) * (1. - w), 0.125 * (1. + u) * (1. - w), -0.125 * (1. + u) * (1. + v)},
        {0.125 * (1. - v) * (1. - w), -0.125 * (1. + u) * (1. - w), -0.125 * (1. + u) * (1. - v)}};
    double J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double s = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) s += x[k][i] * dN[k][j];
            J[i][j] = s;
        }
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    double det = J[0][0] * c00 - J[0][1] * c01 + J[0][2] * c02;
    double Ji[3][3];
    Ji[0][0] = c00 / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][0] = -c01 / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][0] = c02 / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            g[a][j] = dN[a][0] * Ji[0][j] + dN[a][1] * Ji[1][j] + dN[a][2] * Ji[2][j];
    dV = fabs(det);
}

// FEI2dQuadLin::evaldNdxi / evaldNdx (fei2dquadlin.C:80-104, 345-363).
__device__ void quad_grad_at(const double (&x)[4][2], double ksi, double eta, double (&g)[4][2], double &det)
{
    double dn0[4] = {0.25 * (1. + eta), -0.25 * (1. + eta), -0.25 * (1. - eta), 0.25 * (1. - eta)};
    double dn1[4] = {0.25 * (1. + ksi), 0.25 * (1. - ksi), -0.25 * (1. - ksi), -0.25 * (1. + ksi)};
    double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        j00 += dn0[i] * x[i][0]; j01 += dn0[i] * x[i][1];
        j10 += dn1[i] * x[i][0]; j11 += dn1[i] * x[i][1];
    }
    det = j00 * j11 - j01 * j10;
    double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        g[i][0] = i00 * dn0[i] + i01 * dn1[i];
        g[i][1] = i10 * dn0[i] + i11 * dn1[i];
    }
}

// FEI3dTetLin::evaldNdx closed form (fei3dtetlin.C:115-164); w = 1/6.
// Returns false for detJ <= 0 ("negative volume" in the reference).
__device__ bool tet_grad(const double (&x)[4][3], double (&g)[4][3], double &dV)
{
    double x1 = x[0][0], x2 = x[1][0], x3 = x[2][0], x4 = x[3][0];
    double y1 = x[0][1], y2 = x[1][1], y3 = x[2][1], y4 = x[3][1];
    double z1 = x[0][2], z2 = x[1][2], z3 = x[2][2], z4 = x[3][2];
    double detJ = ((x4 - x1) * (y2 - y1) * (z3 - z1) - (x4 - x1) * (y3 - y1) * (z2 - z1) +
                   (x3 - x1) * (y4 - y1) * (z2 - z1) - (x2 - x1) * (y4 - y1) * (z3 - z1) +
                   (x2 - x1) * (y3 - y1) * (z4 - z1) - (x3 - x1) * (y2 - y1) * (z4 - z1));
    double s = 1. / detJ;
    g[0][0] = -((y3 - y2) * (z4 - z2) - (y4 - y2) * (z3 - z2)) * s;
    g[1][0] = ((y4 - y3) * (z1 - z3) - (y1 - y3) * (z4 - z3)) * s;
    g[2][0] = -((y1 - y4) * (z2 - z4) - (y2 - y4) * (z1 - z4)) * s;
    g[3][0] = ((y2 - y1) * (z3 - z1) - (y3 - y1) * (z2 - z1)) * s;
    g[0][1] = -((x4 - x2) * (z3 - z2) - (x3 - x2) * (z4 - z2)) * s;
    g[1][1] = ((x1 - x3) * (z4 - z3) - (x4 - x3) * (z1 - z3)) * s;
    g[2][1] = -((x2 - x4) * (z1 - z4) - (x1 - x4) * (z2 - z4)) * s;
    g[3][1] = ((x3 - x1) * (z2 - z1) - (x2 - x1) * (z3 - z1)) * s;
    g[0][2] = -((x3 - x2) * (y4 - y2) - (x4 - x2) * (y3 - y2)) * s;
    g[1][2] = ((x4 - x3) * (y1 - y3) - (x1 - x3) * (y4 - y3)) * s;
    g[2][2] = -((x1 - x4) * (y2 - y4) - (x2 - x4) * (y1 - y4)) * s;
    g[3][2] = ((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)) * s;
    dV = fabs(detJ) * (1.0 / 6.0);
    return detJ > 0.0;
}

template <int ET>
__device__ __forceinline__ void gather_xe(const double *coords, const int *conn, int e,
                                          double (&x)[ET_<ET>::NPE][ET_<ET>::NDIM])
{
    constexpr int NPE = ET_<ET>::NPE, NDIM = ET_<ET>::NDIM;
#pragma unroll
    for (int a = 0; a < NPE; ++a) {
        int n = __ldg(conn + (size_t)e * NPE + a);
#pragma unroll
        for (int d = 0; d < NDIM; ++d) x[a][d] = __ldg(coords + (size_t)n * NDIM + d);
    }
}

// Gradients of one Gauss point: g (NPE x NDIM), shear-row gradients gs (quad
// only: element centre, planstrss.h:51 / planstrss.C:98-105), dV.
template <int ET>
__device__ __forceinline__ bool gp_grad(const double (&x)[ET_<ET>::NPE][ET_<ET>::NDIM], int gp,
                                        double thickness, double (&g)[ET_<ET>::NPE][ET_<ET>::NDIM],
                                        double (&gs)[ET_<ET>::NPE][ET_<ET>::NDIM], double &dV)
{
    if constexpr (ET == OGB_LSPACE) {
        hex_grad(x, gp, g, dV);
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) gs[a][d] = g[a][d];
        return true;
    } else if constexpr (ET == OGB_PLANESTRESS2D) {
        double det, det0;
        quad_grad_at(x, c_gp2[gp >> 1], c_gp2[gp & 1], g, det);
        quad_grad_at(x, 0.0, 0.0, gs, det0);
        dV = fabs(det) * thickness;
        return true;
    } else {
        bool ok = tet_grad(x, g, dV);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) gs[a][d] = g[a][d];
        return ok;
    }
}

// ------------------------------------------------------------------ materials
// Linear elastic D per material (isolinearelasticmaterial.C:80-88, plane stress
// linearelasticmaterial.C:62-79) is precomputed on the host (capi.cu) into Dmat
// (nmat x 36, row-major NS x NS).

__device__ __forceinline__ double norm_dev(const double (&s)[6])
{
    return sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + 2. * s[3] * s[3] + 2. * s[4] * s[4] +
                2. * s[5] * s[5]);
}

// MisesMat::performPlasticityReturn 3-D branch (misesmat.C:181-263), htype 0, no damage.
// State (24 doubles): [0..5] eps_p, [6] kappa (committed); [8..13] eps_p, [14] kappa (temp);
// [15..20] trial deviatoric stress, [21] trial volumetric stress.
__device__ void mises_stress(const double *mat, const double (&eps)[6], double *st, double (&sig)[6])
{
    double E = mat[1], nu = mat[2], sig0 = mat[3], H = mat[4];
    double G = E / (2.0 * (1. + nu));
    double K = E / (3.0 * (1. - 2. * nu));
    double pl[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) pl[i] = st[i];
    double kappa = st[6];
    double el[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) el[i] = eps[i] - pl[i];
    double mean = (el[0] + el[1] + el[2]) / 3.0;
    double s[6] = {2. * G * (el[0] - mean), 2. * G * (el[1] - mean), 2. * G * (el[2] - mean),
                   G * el[3], G * el[4], G * el[5]};
    double svol = 3 * K * mean;
#pragma unroll
    for (int i = 0; i < 6; ++i) st[15 + i] = s[i];
    st[21] = svol;
    double trialS = norm_dev(s);
    double yieldValue = sqrt(3. / 2.) * trialS - (sig0 + H * kappa);
    if (yieldValue > 0.) {
        double dKappa = yieldValue / (H + 3. * G);
        kappa += dKappa;
        double f = sqrt(3. / 2.) * dKappa / trialS;
        pl[0] += f * (1. / (2. * 0.5) * s[0]);
        pl[1] += f * (1. / (2. * 0.5) * s[1]);
        pl[2] += f * (1. / (2. * 0.5) * s[2]);
        pl[3] += f * (1. / 0.5 * s[3]);
        pl[4] += f * (1. / 0.5 * s[4]);
        pl[5] += f * (1. / 0.5 * s[5]);
        double sc = 1. - sqrt(6.) * G * dKappa / trialS;
#pragma unroll
        for (int i = 0; i < 6; ++i) s[i] *= sc;
    }
    sig[0] = s[0] + svol; sig[1] = s[1] + svol; sig[2] = s[2] + svol;
    sig[3] = s[3]; sig[4] = s[4]; sig[5] = s[5];
#pragma unroll
    for (int i = 0; i < 6; ++i) st[8 + i] = pl[i];
    st[14] = kappa;
}

// MisesMat::give3dMaterialStiffnessMatrix (misesmat.C:496-535), TangentStiffness, omega 0.
__device__ void mises_tangent(const double *mat, const double *st, const double *Del, double (&D)[6][6])
{
    double E = mat[1], nu = mat[2], sig0 = mat[3], H = mat[4];
    double G = E / (2.0 * (1. + nu));
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) D[i][j] = Del[i * 6 + j];
    double kappa = st[6], tempKappa = st[14];
    double dKappa = tempKappa - kappa;
    if (dKappa <= 0.0) return;
    double sigmaY = sig0 + H * kappa;
    double s[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = st[15 + i];
    double trialS = norm_dev(s);
    double factor = -2. * sqrt(6.) * G * G / trialS;
    double factor1 = factor * sigmaY / ((H + 3. * G) * trialS * trialS);
    double factor2 = factor * dKappa;
    const double idev_d = 2. / 3., idev_o = -1. / 3.;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            double idev = (i < 3 && j < 3) ? (i == j ? idev_d : idev_o) : (i == j ? 0.5 : 0.0);
            D[i][j] += factor1 * s[i] * s[j];
            D[i][j] += factor2 * idev;
        }
}

// Principal strains of a 3-D strain vector (engineering shears) as
// StructuralMaterial::computePrincipalValues gives them (structuralmaterial.C:1107-1262):
// zeros unless a component exceeds 1e-20 in magnitude; the invariants of the
// tensor with halved shears; the roots of -x^3 + I1 x^2 - I2 x + I3 in the
// trigonometric form of cubic3r (mathfem.C:155-240: triple root when q and r
// vanish below 1e-100, cosine argument clamped to [-1, 1]); sorted descending.
__device__ void principal_strains(const double (&e)[6], double (&w)[3])
{
    bool nonzero = false;
#pragma unroll
    for (int i = 0; i < 6; ++i) nonzero |= fabs(e[i]) > 1.e-20;
    w[0] = w[1] = w[2] = 0.0;
    if (!nonzero) return;
    const double I1 = e[0] + e[1] + e[2];
    const double I2 = e[0] * e[1] + e[1] * e[2] + e[2] * e[0] - 0.25 * (e[3] * e[3] + e[4] * e[4] + e[5] * e[5]);
    const double I3 = e[0] * e[1] * e[2] +
                      0.25 * (e[3] * e[4] * e[5] - e[0] * e[3] * e[3] - e[1] * e[4] * e[4] - e[2] * e[5] * e[5]);
    // monic form x^3 + a x^2 + b x + c of the cubic with leading coefficient -1
    const double a = I1 / -1.0, b = -I2 / -1.0, c = I3 / -1.0;
    const double q = (a * a - 3.0 * b) / 9.0;
    const double r = (2.0 * a * a * a - 9.0 * a * b + 27.0 * c) / 54.0;
    if (fabs(q) < 1.0e-100 && fabs(r) < 1.0e-100) {
        w[0] = w[1] = w[2] = -a / 3.0;
    } else {
        double h = r / sqrt(q * q * q);
        if (fabs(h) > 1.0) h = h > 0 ? 1.0 : -1.0;
        const double phi = acos(h), p = sqrt(q);
        const double pi = 3.14159265358979323846;
        w[0] = -2.0 * p * cos(phi / 3.0) - a / 3.0;
        w[1] = -2.0 * p * cos((phi + 2.0 * pi) / 3.0) - a / 3.0;
        w[2] = -2.0 * p * cos((phi - 2.0 * pi) / 3.0) - a / 3.0;
    }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            if (w[j + 1] > w[j]) { double t = w[j]; w[j] = w[j + 1]; w[j + 1] = t; }
}

// Principal values and directions of a symmetric 3x3 matrix as
// StructuralMaterial::computePrincipalValDir obtains them (structuralmaterial.C:1337-1470,
// FloatMatrix::jaco_ to 10 significant figures, floatmatrix.C:1953-2120): threshold
// Jacobi rotations over the pairs (0,1), (0,2), (1,2) in that order; a pair is
// rotated when |a_pq| exceeds 1e-10 of the sum of the absolute input entries, by
// half of atan2(2 a_pq, a_pp - a_qq); sweeps stop once the rotated entries of a
// sweep sum to no more than that fraction (51 sweeps at most). The loose stopping
// rule is part of the result: the crack normal of a damaged point carries it.
// Values sorted descending with their vectors (columns of V).
__device__ void principal_dirs(const double (&S)[3][3], double (&w)[3], double (&V)[3][3])
{
    double u[3][3];   // the upper triangle is the working matrix, as in jaco_
    double ev[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            u[i][j] = S[i][j];
            V[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int i = 0; i < 3; ++i) ev[i] = u[i][i];
    const double tol = 1.0e-10;   // 0.1^10
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
                    const double ang = atan2(u[i][j] * 2.0, ev[i] - ev[j]) / 2.0;
                    const double si = sin(ang), co = cos(ang);
                    double t;
                    for (int k = 0; k < i; ++k) {
                        t = u[k][i];
                        u[k][i] = co * t + si * u[k][j];
                        u[k][j] = -si * t + co * u[k][j];
                    }
                    t = ev[i];
                    ev[i] = co * t + si * u[i][j];
                    const double aij = -si * t + co * u[i][j];
                    for (int k = i + 1; k < j; ++k) {
                        t = u[i][k];
                        u[i][k] = co * t + si * u[k][j];
                        u[k][j] = -si * t + co * u[k][j];
                    }
                    t = u[i][j];
                    const double aji = co * t + si * ev[j];
                    ev[j] = -si * t + co * ev[j];
                    for (int k = j + 1; k < 3; ++k) {
                        t = u[i][k];
                        u[i][k] = co * t + si * u[j][k];
                        u[j][k] = -si * t + co * u[j][k];
                    }
                    for (int k = 0; k < 3; ++k) {
                        t = V[k][i];
                        V[k][i] = co * t + si * V[k][j];
                        V[k][j] = -si * t + co * V[k][j];
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
                for (int k = 0; k < 3; ++k) { t = V[k][jj]; V[k][jj] = V[k][jj + 1]; V[k][jj + 1] = t; }
            }
    for (int i = 0; i < 3; ++i) w[i] = ev[i];
}

// IsotropicDamageMaterial1: Mazars equivalent strain (idm1.C:436-470) from the
// principal strains above, exponential
// cohesive crack (idm1.C:808-911, wf = gf/(E e0), ef = wf/Le, Newton until
// |R| < e0*1e-9, at most 40 steps), crack band on first damage (initDamaged
// idm1.C:1168-1322, Element::giveLengthInDir element.C:1162-1183), strain-level
// loading criterion (isodamagemodel.C:86-160). State [0] kappa, [1] omega, [2] Le,
// [8] temp kappa, [9] temp omega.
template <int NPE>
__device__ void idm1_stress(const double *mat, const double (&eps)[6], double *st,
                            const double (&x)[NPE][3], const double *Del, double (&sig)[6])
{
    double E = mat[1], e0 = mat[5], gf = mat[6];
    double T[3][3] = {{eps[0], 0.5 * eps[5], 0.5 * eps[4]},
                      {0.5 * eps[5], eps[1], 0.5 * eps[3]},
                      {0.5 * eps[4], 0.5 * eps[3], eps[2]}};
    double w[3], V[3][3];
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
            double n0 = V[0][indx], n1 = V[1][indx], n2 = V[2][indx];
            double mx = 0, mn = 0;
            for (int a = 0; a < NPE; ++a) {
                double d = n0 * x[a][0] + n1 * x[a][1] + n2 * x[a][2];
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
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double s = 0;
#pragma unroll
        for (int k = 0; k < 6; ++k) s += Del[i * 6 + k] * eps[k];
        sig[i] = (1.0 - omega) * s;
    }
    st[8] = tempKappa;
    st[9] = omega;
    st[2] = le;
}

// ------------------------------------------------------------------ K1 stiffness
// Ke layout: ke[e][a][b][i][j] (ND x ND node blocks, row-major).
template <int ET, bool PER_GP_D>
__global__ void __launch_bounds__(NTHREADS) k_elem_stiffness(
    int nelem, const double *__restrict__ coords, const int *__restrict__ conn,
    const int *__restrict__ emat, const double *__restrict__ mats, const double *__restrict__ Dmat,
    const double *__restrict__ state, double thickness, double *__restrict__ ke, int *status)
{
    using T = ET_<ET>;
    constexpr int NPE = T::NPE, NGP = T::NGP, ND = T::ND, NDIM = T::NDIM, NS = T::NS;
    constexpr int EPB = NTHREADS / NPE;
    constexpr int NSYM = NS * (NS + 1) / 2;
    extern __shared__ double smem[];
    auto s_g = reinterpret_cast<double (*)[NGP][NPE][NDIM]>(smem);
    auto s_gs = reinterpret_cast<double (*)[NPE][NDIM]>(smem + EPB * NGP * NPE * NDIM);
    auto s_dv = reinterpret_cast<double (*)[NGP]>(smem + EPB * NGP * NPE * NDIM + EPB * NPE * NDIM);
    auto s_D = reinterpret_cast<double (*)[NSYM]>(smem + EPB * NGP * NPE * NDIM + EPB * NPE * NDIM + EPB * NGP);

    const int e0 = blockIdx.x * EPB;
    for (int t = threadIdx.x; t < EPB * NGP; t += NTHREADS) {
        int le = t / NGP, gp = t % NGP, e = e0 + le;
        if (e >= nelem) continue;
        double x[NPE][NDIM], g[NPE][NDIM], gs[NPE][NDIM], dV;
        gather_xe<ET>(coords, conn, e, x);
        if (!gp_grad<ET>(x, gp, thickness, g, gs, dV)) atomicCAS(status, DS_OK, DS_NEGVOL);
#pragma unroll
        for (int a = 0; a < NPE; ++a)
#pragma unroll
            for (int d = 0; d < NDIM; ++d) s_g[le][gp][a][d] = g[a][d];
        if constexpr (ET == OGB_PLANESTRESS2D) {
            if (gp == 0)
#pragma unroll
                for (int a = 0; a < NPE; ++a)
#pragma unroll
                    for (int d = 0; d < NDIM; ++d) s_gs[le][a][d] = gs[a][d];
        }
        s_dv[le][gp] = dV;
        if constexpr (PER_GP_D) {
            int m = emat[e];
            const double *mat = mats + 8 * m;
            const double *Del = Dmat + 36 * m;
            const double *st = state + ((size_t)e * NGP + gp) * NSTATE;
            double D[6][6];
            int kind = (int)mat[0];
            if (kind == OGB_MAT_MISES) {
                mises_tangent(mat, st, Del, D);
            } else {
                double f = 1.0;
                if (kind == OGB_MAT_IDM1) {
                    // IsotropicDamageMaterial::give3dMaterialStiffnessMatrix (isodamagemodel.C:63-81):
                    // secant (1 - min(omega, maxOmega)) D, maxOmega 0.999999 (isodamagemodel.h:167).
                    double om = st[9] < 0.999999 ? st[9] : 0.999999;
                    f = 1.0 - om;
                }
                for (int i = 0; i < NS; ++i)
                    for (int j = 0; j < NS; ++j) D[i][j] = f * Del[i * NS + j];
            }
            int k = 0;
            for (int i = 0; i < NS; ++i)
                for (int j = i; j < NS; ++j) s_D[le * NGP + gp][k++] = D[i][j];
        }
    }
    __syncthreads();

    const int le = threadIdx.x / NPE, a = threadIdx.x % NPE, e = e0 + le;
    if (e >= nelem) return;
    if constexpr (ET == OGB_LSPACE && !PER_GP_D) {
        // Isotropic D (D = 2G I_dev + K 1(x)1, isolinearelasticmaterial.C:80-88): with
        // lambda = D_12 and mu = D_44,
        //   K_ab^ij = sum_gp dV [lambda g_a^i g_b^j + mu g_a^j g_b^i + mu delta_ij g_a.g_b]
        // = lambda A_ab^ij + mu A_ab^ji + mu delta_ij tr A_ab,  A_ab^ij = sum_gp dV g_a^i g_b^j,
        // the same B^T D B dV sum in a third of the FP64 operations of the dense product.
        const double *Dm = Dmat + 36 * __ldg(emat + e);
        const double lam = __ldg(Dm + 1), mu = __ldg(Dm + 21);
        double A[NPE][3][3];
#pragma unroll
        for (int b = 0; b < NPE; ++b)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) A[b][i][j] = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < NGP; ++gp) {
            const double dv = s_dv[le][gp];
            const double ga[3] = {dv * s_g[le][gp][a][0], dv * s_g[le][gp][a][1], dv * s_g[le][gp][a][2]};
#pragma unroll
            for (int b = 0; b < NPE; ++b) {
                const double h[3] = {s_g[le][gp][b][0], s_g[le][gp][b][1], s_g[le][gp][b][2]};
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = 0; j < 3; ++j) A[b][i][j] = fma(ga[i], h[j], A[b][i][j]);
            }
        }
        double *out = ke + (((size_t)e * NPE + a) * NPE) * 9;
#pragma unroll
        for (int b = 0; b < NPE; ++b) {
            const double mtr = mu * (A[b][0][0] + A[b][1][1] + A[b][2][2]);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    out[(b * 3 + i) * 3 + j] = lam * A[b][i][j] + mu * A[b][j][i] + (i == j ? mtr : 0.0);
        }
        return;
    }
    double D[NS][NS];
    if constexpr (!PER_GP_D) {
        const double *Dm = Dmat + 36 * __ldg(emat + e);
#pragma unroll
        for (int i = 0; i < NS; ++i)
#pragma unroll
            for (int j = 0; j < NS; ++j) D[i][j] = __ldg(Dm + i * NS + j);
    }
    double K[NPE][ND][ND];
#pragma unroll
    for (int b = 0; b < NPE; ++b)
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int j = 0; j < ND; ++j) K[b][i][j] = 0.0;

#pragma unroll 1
    for (int gp = 0; gp < NGP; ++gp) {
        if constexpr (PER_GP_D) {
            int k = 0;
#pragma unroll
            for (int i = 0; i < NS; ++i)
#pragma unroll
                for (int j = i; j < NS; ++j) {
                    double v = s_D[le * NGP + gp][k++];
                    D[i][j] = v;
                    D[j][i] = v;
                }
        }
        const double dv = s_dv[le][gp];
        // DB_a = D * B_a (NS x ND), B_a sparse (structural3delement.C:76-84 / planstrss.C:92-105)
        double DB[NS][ND];
        if constexpr (NDIM == 3) {
            const double gx = s_g[le][gp][a][0], gy = s_g[le][gp][a][1], gz = s_g[le][gp][a][2];
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                DB[k][0] = D[k][0] * gx + D[k][4] * gz + D[k][5] * gy;
                DB[k][1] = D[k][1] * gy + D[k][3] * gz + D[k][5] * gx;
                DB[k][2] = D[k][2] * gz + D[k][3] * gy + D[k][4] * gx;
            }
#pragma unroll
            for (int b = 0; b < NPE; ++b) {
                const double hx = s_g[le][gp][b][0], hy = s_g[le][gp][b][1], hz = s_g[le][gp][b][2];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    K[b][i][0] += dv * (DB[0][i] * hx + DB[4][i] * hz + DB[5][i] * hy);
                    K[b][i][1] += dv * (DB[1][i] * hy + DB[3][i] * hz + DB[5][i] * hx);
                    K[b][i][2] += dv * (DB[2][i] * hz + DB[3][i] * hy + DB[4][i] * hx);
                }
            }
        } else {
            const double gx = s_g[le][gp][a][0], gy = s_g[le][gp][a][1];
            const double sx = s_gs[le][a][0], sy = s_gs[le][a][1];
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                DB[k][0] = D[k][0] * gx + D[k][2] * sy;
                DB[k][1] = D[k][1] * gy + D[k][2] * sx;
            }
#pragma unroll
            for (int b = 0; b < NPE; ++b) {
                const double hx = s_g[le][gp][b][0], hy = s_g[le][gp][b][1];
                const double tx = s_gs[le][b][0], ty = s_gs[le][b][1];
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    K[b][i][0] += dv * (DB[0][i] * hx + DB[2][i] * ty);
                    K[b][i][1] += dv * (DB[1][i] * hy + DB[2][i] * tx);
                }
            }
        }
    }
    double *out = ke + (((size_t)e * NPE + a) * NPE) * ND * ND;
#pragma unroll
    for (int b = 0; b < NPE; ++b)
#pragma unroll
        for (int i = 0; i < ND; ++i)
#pragma unroll
            for (int j = 0; j < ND; ++j) out[(b * ND + i) * ND + j] = K[b][i][j];
}

// ------------------------------------------------------------------ K2/K3 internal forces
template <int ET>
__global__ void __launch_bounds__(NTHREADS) k_elem_internal_forces(
    int nelem, const double *__restrict__ coords, const int *__restrict__ conn,
    const int *__restrict__ emat, const double *__restrict__ mats, const double *__restrict__ Dmat,
    double thickness, const double *__restrict__ u_node, double *__restrict__ state,
    double *__restrict__ gp_stress, double *__restrict__ gp_strain, double *__restrict__ fe, int *status)
{
    using T = ET_<ET>;
    constexpr int NPE = T::NPE, NGP = T::NGP, ND = T::ND, NDIM = T::NDIM, NS = T::NS;
    constexpr int EPB = NTHREADS / NPE;
    extern __shared__ double smem[];
    auto s_g = reinterpret_cast<double (*)[NGP][NPE][NDIM]>(smem);
    auto s_gs = reinterpret_cast<double (*)[NPE][NDIM]>(smem + EPB * NGP * NPE * NDIM);
    auto s_sig = reinterpret_cast<double (*)[NGP][NS]>(smem + EPB * NGP * NPE * NDIM + EPB * NPE * NDIM);  // sigma*dV

    const int e0 = blockIdx.x * EPB;
    for (int t = threadIdx.x; t < EPB * NGP; t += NTHREADS) {
        int le = t / NGP, gp = t % NGP, e = e0 + le;
        if (e >= nelem) continue;
        double x[NPE][NDIM], g[NPE][NDIM], gs[NPE][NDIM], dV;
        gather_xe<ET>(coords, conn, e, x);
        if (!gp_grad<ET>(x, gp, thickness, g, gs, dV)) atomicCAS(status, DS_OK, DS_NEGVOL);
        double u[NPE][ND];
#pragma unroll
        for (int a = 0; a < NPE; ++a) {
            int n = __ldg(conn + (size_t)e * NPE + a);
#pragma unroll
            for (int d = 0; d < ND; ++d) u[a][d] = u_node[(size_t)n * ND + d];
        }
        // eps = B u_e (StructuralElement::computeStrainVector, structuralelement.C:723-745)
        double eps[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) eps[k] = 0.0;
        if constexpr (NDIM == 3) {
#pragma unroll
            for (int a = 0; a < NPE; ++a) {
                eps[0] += g[a][0] * u[a][0];
                eps[1] += g[a][1] * u[a][1];
                eps[2] += g[a][2] * u[a][2];
                eps[3] += g[a][2] * u[a][1] + g[a][1] * u[a][2];
                eps[4] += g[a][2] * u[a][0] + g[a][0] * u[a][2];
                eps[5] += g[a][1] * u[a][0] + g[a][0] * u[a][1];
            }
        } else {
#pragma unroll
            for (int a = 0; a < NPE; ++a) {
                eps[0] += g[a][0] * u[a][0];
                eps[1] += g[a][1] * u[a][1];
                eps[2] += gs[a][1] * u[a][0] + gs[a][0] * u[a][1];
            }
        }
        int m = emat[e];
        const double *mat = mats + 8 * m;
        const double *Del = Dmat + 36 * m;
        double sig[NS];
        int kind = (int)mat[0];
        double *st = state ? state + ((size_t)e * NGP + gp) * NSTATE : nullptr;
        if constexpr (NDIM == 3) {
            if (kind == OGB_MAT_MISES && st) {
                double e6[6], s6[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) e6[k] = eps[k];
                mises_stress(mat, e6, st, s6);
#pragma unroll
                for (int k = 0; k < 6; ++k) sig[k] = s6[k];
            } else if (kind == OGB_MAT_IDM1 && st) {
                double e6[6], s6[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) e6[k] = eps[k];
                idm1_stress<NPE>(mat, e6, st, x, Del, s6);
#pragma unroll
                for (int k = 0; k < 6; ++k) sig[k] = s6[k];
            } else {
#pragma unroll
                for (int i = 0; i < NS; ++i) {
                    double s = 0;
#pragma unroll
                    for (int k = 0; k < NS; ++k) s += Del[i * NS + k] * eps[k];
                    sig[i] = s;
                }
            }
        } else {
            // LinearElasticMaterial::giveRealStressVector_PlaneStress (linearelasticmaterial.C:167-190)
#pragma unroll
            for (int i = 0; i < NS; ++i) {
                double s = 0;
#pragma unroll
                for (int k = 0; k < NS; ++k) s += Del[i * NS + k] * eps[k];
                sig[i] = s;
            }
        }
        if (gp_stress) {
            size_t o = ((size_t)e * NGP + gp) * NS;
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                gp_stress[o + k] = sig[k];
                gp_strain[o + k] = eps[k];
            }
        }
#pragma unroll
        for (int a = 0; a < NPE; ++a)
#pragma unroll
            for (int d = 0; d < NDIM; ++d) s_g[le][gp][a][d] = g[a][d];
        if constexpr (ET == OGB_PLANESTRESS2D) {
            if (gp == 0)
#pragma unroll
                for (int a = 0; a < NPE; ++a)
#pragma unroll
                    for (int d = 0; d < NDIM; ++d) s_gs[le][a][d] = gs[a][d];
        }
#pragma unroll
        for (int k = 0; k < NS; ++k) s_sig[le][gp][k] = sig[k] * dV;
    }
    __syncthreads();

    const int le = threadIdx.x / NPE, a = threadIdx.x % NPE, e = e0 + le;
    if (e >= nelem) return;
    double f[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) f[d] = 0.0;
#pragma unroll 1
    for (int gp = 0; gp < NGP; ++gp) {
        const double *s = s_sig[le][gp];
        if constexpr (NDIM == 3) {
            const double gx = s_g[le][gp][a][0], gy = s_g[le][gp][a][1], gz = s_g[le][gp][a][2];
            f[0] += gx * s[0] + gz * s[4] + gy * s[5];
            f[1] += gy * s[1] + gz * s[3] + gx * s[5];
            f[2] += gz * s[2] + gy * s[3] + gx * s[4];
        } else {
            const double gx = s_g[le][gp][a][0], gy = s_g[le][gp][a][1];
            const double sx = s_gs[le][a][0], sy = s_gs[le][a][1];
            f[0] += gx * s[0] + sy * s[2];
            f[1] += gy * s[1] + sx * s[2];
        }
    }
    double *out = fe + ((size_t)e * NPE + a) * ND;
#pragma unroll
    for (int d = 0; d < ND; ++d) out[d] = f[d];
}

// ------------------------------------------------------------------ launchers
template <int ET>
constexpr size_t stiff_smem(bool pergp)
{
    using T = ET_<ET>;
    constexpr int EPB = NTHREADS / T::NPE;
    return sizeof(double) * ((size_t)EPB * T::NGP * T::NPE * T::NDIM + EPB * T::NPE * T::NDIM +
                             EPB * T::NGP + (pergp ? (size_t)EPB * T::NGP * (T::NS * (T::NS + 1) / 2) : 0));
}

template <int ET>
constexpr size_t force_smem()
{
    using T = ET_<ET>;
    constexpr int EPB = NTHREADS / T::NPE;
    return sizeof(double) * ((size_t)EPB * T::NGP * T::NPE * T::NDIM + EPB * T::NPE * T::NDIM +
                             (size_t)EPB * T::NGP * T::NS);
}

template <int ET, bool PERGP>
static int run_stiffness(ogb_model *md)
{
    ogb_ctx *ctx = md->ctx;
    constexpr size_t smem = stiff_smem<ET>(PERGP);
    static bool attr_set[64] = {};
    OGB_CUDA(set_smem_limit_once((const void *)k_elem_stiffness<ET, PERGP>, (int)smem, attr_set));
    int nb = (int)ceil_div(md->nelem, NTHREADS / ET_<ET>::NPE);
    k_elem_stiffness<ET, PERGP><<<nb, NTHREADS, smem, ctx->stream>>>(
        md->nelem, md->coords.p, md->conn.p, md->emat.p, md->mats.p, md->Dmat.p, md->state.p, md->thickness,
        md->ke.p, ctx->status.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

template <int ET>
static int run_forces(ogb_model *md, const double *u_node)
{
    ogb_ctx *ctx = md->ctx;
    constexpr size_t smem = force_smem<ET>();
    static bool attr_set[64] = {};
    OGB_CUDA(set_smem_limit_once((const void *)k_elem_internal_forces<ET>, (int)smem, attr_set));
    double *st = md->nonlinear ? md->state.p : nullptr;
    int nb = (int)ceil_div(md->nelem, NTHREADS / ET_<ET>::NPE);
    k_elem_internal_forces<ET><<<nb, NTHREADS, smem, ctx->stream>>>(
        md->nelem, md->coords.p, md->conn.p, md->emat.p, md->mats.p, md->Dmat.p, md->thickness, u_node, st,
        md->gp_stress.p, md->gp_strain.p, md->fe.p, ctx->status.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

int launch_elem_stiffness(ogb_model *md)
{
    const bool pergp = md->nonlinear;
    switch (md->etype) {
    case OGB_LSPACE:
        return pergp ? run_stiffness<OGB_LSPACE, true>(md) : run_stiffness<OGB_LSPACE, false>(md);
    case OGB_PLANESTRESS2D:
        return run_stiffness<OGB_PLANESTRESS2D, false>(md);
    case OGB_LTRSPACE:
        return pergp ? run_stiffness<OGB_LTRSPACE, true>(md) : run_stiffness<OGB_LTRSPACE, false>(md);
    }
    return fail(OGB_E_ARG, "unknown element type");
}

int launch_elem_internal_forces(ogb_model *md, const double *u_node)
{
    switch (md->etype) {
    case OGB_LSPACE: return run_forces<OGB_LSPACE>(md, u_node);
    case OGB_PLANESTRESS2D: return run_forces<OGB_PLANESTRESS2D>(md, u_node);
    case OGB_LTRSPACE: return run_forces<OGB_LTRSPACE>(md, u_node);
    }
    return fail(OGB_E_ARG, "unknown element type");
}

}  // namespace ogb
