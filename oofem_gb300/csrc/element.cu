// Element kernels: Gauss-point gradients, material point updates (K3), element
// stiffness K = sum_gp B^T D B dV (K1) and internal forces f = sum_gp B^T sigma dV
// (K2) for LSpace, PlaneStress2d and LTRSpace, all in FP64.
//
// Thread layout: one block handles EPB = 256/NPE elements. Phase 1 runs one
// thread per (element, Gauss point) and stages gradients, dV (and per-GP
// tangents or weighted stresses) in shared memory; phase 2 runs one thread per
// (element, node a) and produces the a-th block row of the element matrix or
// vector, so no thread holds more than NPE*ND*ND accumulators.
#include <cuda_bf16.h>

#include "internal.cuh"
#include "tcgen05.cuh"

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
template <class R>
__device__ void hex_grad(const R (&x)[8][3], int gp, R (&g)[8][3], R &dV)
{
    const R u = (R)c_gp2[gp >> 2], v = (R)c_gp2[(gp >> 1) & 1], w = (R)c_gp2[gp & 1];
    const R dN[8][3] = {
        {-R(0.125) * (R(1) - v) * (R(1) + w), -R(0.125) * (R(1) - u) * (R(1) + w), R(0.125) * (R(1) - u) * (R(1) - v)},
        {-R(0.125) * (R(1) + v) * (R(1) + w), R(0.125) * (R(1) - u) * (R(1) + w), R(0.125) * (R(1) - u) * (R(1) + v)},
        {R(0.125) * (R(1) + v) * (R(1) + w), R(0.125) * (R(1) + u) * (R(1) + w), R(0.125) * (R(1) + u) * (R(1) + v)},
        {R(0.125) * (R(1) - v) * (R(1) + w), -R(0.125) * (R(1) + u) * (R(1) + w), R(0.125) * (R(1) + u) * (R(1) - v)},
        {-R(0.125) * (R(1) - v) * (R(1) - w), -R(0.125) * (R(1) - u) * (R(1) - w), -R(0.125) * (R(1) - u) * (R(1) - v)},
        {-R(0.125) * (R(1) + v) * (R(1) - w), R(0.125) * (R(1) - u) * (R(1) - w), -R(0.125) * (R(1) - u) * (R(1) + v)},
        {R(0.125) * (R(1) + v) * (R(1) - w), R(0.125) * (R(1) + u) * (R(1) - w), -R(0.125) * (R(1) + u) * (R(1) + v)},
        {R(0.125) * (R(1) - v) * (R(1) - w), -R(0.125) * (R(1) + u) * (R(1) - w), -R(0.125) * (R(1) + u) * (R(1) - v)}};
    R J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R s = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) s += x[k][i] * dN[k][j];
            J[i][j] = s;
        }
    R c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    R c01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
    R c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    R det = J[0][0] * c00 - J[0][1] * c01 + J[0][2] * c02;
    R Ji[3][3];
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
template <class R>
__device__ void quad_grad_at(const R (&x)[4][2], R ksi, R eta, R (&g)[4][2], R &det)
{
    const R q = R(0.25), one = R(1);
    const R dn0[4] = {q * (one + eta), -q * (one + eta), -q * (one - eta), q * (one - eta)};
    const R dn1[4] = {q * (one + ksi), q * (one - ksi), -q * (one - ksi), -q * (one + ksi)};
    R j00 = 0, j01 = 0, j10 = 0, j11 = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        j00 += dn0[i] * x[i][0]; j01 += dn0[i] * x[i][1];
        j10 += dn1[i] * x[i][0]; j11 += dn1[i] * x[i][1];
    }
    det = j00 * j11 - j01 * j10;
    const R i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        g[i][0] = i00 * dn0[i] + i01 * dn1[i];
        g[i][1] = i10 * dn0[i] + i11 * dn1[i];
    }
}

// FEI3dTetLin::evaldNdx closed form (fei3dtetlin.C:115-164); w = 1/6.
// Returns false for detJ <= 0 ("negative volume" in the reference).
template <class R>
__device__ bool tet_grad(const R (&x)[4][3], R (&g)[4][3], R &dV)
{
    const R x1 = x[0][0], x2 = x[1][0], x3 = x[2][0], x4 = x[3][0];
    const R y1 = x[0][1], y2 = x[1][1], y3 = x[2][1], y4 = x[3][1];
    const R z1 = x[0][2], z2 = x[1][2], z3 = x[2][2], z4 = x[3][2];
    const R detJ = ((x4 - x1) * (y2 - y1) * (z3 - z1) - (x4 - x1) * (y3 - y1) * (z2 - z1) +
                   (x3 - x1) * (y4 - y1) * (z2 - z1) - (x2 - x1) * (y4 - y1) * (z3 - z1) +
                   (x2 - x1) * (y3 - y1) * (z4 - z1) - (x3 - x1) * (y2 - y1) * (z4 - z1));
    const R s = R(1) / detJ;
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
    dV = fabs(detJ) * (R(1) / R(6));
    return detJ > R(0);
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
template <int ET, class R = double>
__device__ __forceinline__ bool gp_grad(const R (&x)[ET_<ET>::NPE][ET_<ET>::NDIM], int gp,
                                        R thickness, R (&g)[ET_<ET>::NPE][ET_<ET>::NDIM],
                                        R (&gs)[ET_<ET>::NPE][ET_<ET>::NDIM], R &dV)
{
    if constexpr (ET == OGB_LSPACE) {
        hex_grad(x, gp, g, dV);
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d) gs[a][d] = g[a][d];
        return true;
    } else if constexpr (ET == OGB_PLANESTRESS2D) {
        R det, det0;
        quad_grad_at<R>(x, (R)c_gp2[gp >> 1], (R)c_gp2[gp & 1], g, det);
        quad_grad_at<R>(x, R(0), R(0), gs, det0);
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

// ------------------------------------------------------------------ K1 on tensor cores
// Element stiffness of the mixed-precision tangent on the 5th-generation tensor
// cores: K_e = G^T H with G[(gp, s)][(a, i)] = B_gp[s][(a, i)] and
// H[(gp, s)][(b, j)] = dV_gp (D_gp B_gp)[s][(b, j)] (the sum over Gauss points
// and strain components is the K dimension of one MMA chain,
// NLStructuralElement::computeStiffnessMatrix nlstructuralelement.C:345-376).
// EPT elements share one 128 x 128 tile: element le owns rows and columns
// le*NDOF .. le*NDOF+NDOF-1, and only its diagonal block of the product is read
// back. Split BF16: each FP32 operand is the sum of three BF16 pieces
// (v = v0 + v1 + v2, exact to about 2^-24 |v|); the six products v_i w_j with
// i + j <= 2 are accumulated in FP32 in tensor memory, which gives K_e to FP32
// accuracy. Per CTA (128 threads, persistent over tiles): gradients, dV and the
// material tangent per (element, GP) on the CUDA cores; the split operands in
// shared memory (canonical K-major layout without swizzle); 6 MMAs per 16 of K
// issued by one thread, completion through an mbarrier (bounded wait: a timeout
// sets DS_TIMEOUT and the kernel stops); each warp reads its 32 tensor-memory
// lanes (rows) and writes the element rows in the layout of k_elem_stiffness.
template <int ET>
struct TcTile {
    using T = ET_<ET>;
    static constexpr int NDOF = T::NPE * T::ND;        // 24 hex, 8 quad, 12 tet
    static constexpr int KDIM = T::NGP * T::NS;        // 48, 12, 6
    static constexpr int KP = (KDIM + 15) / 16 * 16;   // K padded to whole MMAs: 48, 16, 16
    static constexpr int EPT = 128 / NDOF;             // elements per tile: 5, 16, 10
    static constexpr int PIECE = 128 * KP * 2;         // bytes of one BF16 operand piece (128 rows)
    static constexpr int OPER = 6 * PIECE;             // A0 A1 A2 (G pieces) B0 B1 B2 (H pieces)
    static constexpr int NGPT = EPT * T::NGP;          // (element, GP) pairs of a tile
    static constexpr int GPF = 2 * T::NPE * T::NDIM + 1 + T::NS * T::NS;   // g, gs, dV, D (FP32)
    static constexpr size_t SMEM = 1024 + OPER + (size_t)NGPT * GPF * 4 + 16;
};

// Store v as three BF16 pieces at (row, k) of pieces p0, p0+1, p0+2.
template <int KP>
__device__ __forceinline__ void store_split3(unsigned char *oper, int piece_bytes, int p0, int row, int k, float v)
{
    const int off = ((((row >> 3) * (KP / 8)) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
    const __nv_bfloat16 h0 = __float2bfloat16_rn(v);
    float rem = v - __bfloat162float(h0);
    const __nv_bfloat16 h1 = __float2bfloat16_rn(rem);
    rem -= __bfloat162float(h1);
    const __nv_bfloat16 h2 = __float2bfloat16_rn(rem);
    *reinterpret_cast<__nv_bfloat16 *>(oper + (p0 + 0) * piece_bytes + off) = h0;
    *reinterpret_cast<__nv_bfloat16 *>(oper + (p0 + 1) * piece_bytes + off) = h1;
    *reinterpret_cast<__nv_bfloat16 *>(oper + (p0 + 2) * piece_bytes + off) = h2;
}

template <int ET>
__global__ void __launch_bounds__(128) k_elem_stiffness_tc(
    int nelem, const double *__restrict__ coords, const int *__restrict__ conn, const int *__restrict__ emat,
    const double *__restrict__ mats, const double *__restrict__ Dmat, const double *__restrict__ state,
    double thickness, double *__restrict__ ke, int *status)
{
    using T = ET_<ET>;
    using L = TcTile<ET>;
    constexpr int NPE = T::NPE, NGP = T::NGP, ND = T::ND, NDIM = T::NDIM, NS = T::NS;
    extern __shared__ unsigned char tc_smem[];
    __shared__ int s_ok;
    const uint32_t raw = tc::smem_u32(tc_smem);
    unsigned char *oper = tc_smem + (((raw + 1023u) & ~1023u) - raw);
    float *gpd = reinterpret_cast<float *>(oper + L::OPER);
    uint64_t *bar = reinterpret_cast<uint64_t *>(gpd + L::NGPT * L::GPF);   // 8-byte aligned: OPER, 4*count even
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;

    // zero the operands: padding rows and K beyond KDIM stay zero for every tile
    for (int i = tid; i < L::OPER / 16; i += 128) reinterpret_cast<uint4 *>(oper)[i] = make_uint4(0, 0, 0, 0);
    if (warp == 0) tc::tmem_alloc(slot, 128);
    if (tid == 0) tc::mbar_init(bar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    const uint32_t abase = tc::smem_u32(oper);
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 128);
    constexpr uint32_t LBO = 128, SBO = (L::KP / 8) * 128;
    constexpr long long WAIT_CYCLES = 2000000000LL;   // about a second
    uint32_t phase = 0;
    bool failed = false;
    const int ntiles = (nelem + L::EPT - 1) / L::EPT;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int e0 = tile * L::EPT;
        // (1) gradients, dV and the material tangent of every (element, GP)
        for (int t = tid; t < L::NGPT; t += 128) {
            const int le = t / NGP, gp = t % NGP, e = e0 + le;
            float *q = gpd + t * L::GPF;
            if (e >= nelem) {
                for (int i = 0; i < L::GPF; ++i) q[i] = 0.f;
                continue;
            }
            // FP32 gradients (this tangent is FP32-accurate) from coordinates relative
            // to the element's first node, which keeps the Jacobian exact to FP32
            // whatever the distance of the element from the origin
            double x[NPE][NDIM];
            gather_xe<ET>(coords, conn, e, x);
            float xl[NPE][NDIM], g[NPE][NDIM], gs[NPE][NDIM], dV;
            for (int a = 0; a < NPE; ++a)
                for (int d = 0; d < NDIM; ++d) xl[a][d] = (float)(x[a][d] - x[0][d]);
            if (!gp_grad<ET, float>(xl, gp, (float)thickness, g, gs, dV)) atomicCAS(status, DS_OK, DS_NEGVOL);
            for (int a = 0; a < NPE; ++a)
                for (int d = 0; d < NDIM; ++d) {
                    q[a * NDIM + d] = g[a][d];
                    q[NPE * NDIM + a * NDIM + d] = gs[a][d];
                }
            q[2 * NPE * NDIM] = dV;
            float *Dq = q + 2 * NPE * NDIM + 1;
            const int m = emat[e];
            const double *mat = mats + 8 * m;
            const double *Del = Dmat + 36 * m;
            const int kind = (int)mat[0];
            if (kind == OGB_MAT_MISES && state) {
                double D[6][6];
                mises_tangent(mat, state + ((size_t)e * NGP + gp) * NSTATE, Del, D);
                for (int i = 0; i < NS; ++i)
                    for (int j = 0; j < NS; ++j) Dq[i * NS + j] = (float)D[i][j];
            } else {
                double f = 1.0;
                if (kind == OGB_MAT_IDM1 && state) {
                    // secant (1 - min(omega, 0.999999)) D (isodamagemodel.C:63-81)
                    const double om = state[((size_t)e * NGP + gp) * NSTATE + 9];
                    f = 1.0 - (om < 0.999999 ? om : 0.999999);
                }
                for (int i = 0; i < NS; ++i)
                    for (int j = 0; j < NS; ++j) Dq[i * NS + j] = (float)(f * Del[i * NS + j]);
            }
        }
        __syncthreads();
        // (2) split operands, one thread per (element, GP, node a): the ND columns
        // (a, i) of B_gp (sparse: gradients of node a) and of dV D_gp B_gp
        for (int t = tid; t < L::NGPT * NPE; t += 128) {
            const int pair = t / NPE, a = t % NPE, le = pair / NGP, gp = pair % NGP;
            const float *q = gpd + pair * L::GPF;
            const float *ga = q + a * NDIM, *gsa = q + NPE * NDIM + a * NDIM;
            const float dv = q[2 * NPE * NDIM];
            const float *Dq = q + 2 * NPE * NDIM + 1;
            float Bc[ND][NS];
            if constexpr (NDIM == 3) {
                // Voigt xx, yy, zz, yz, zx, xy (structural3delement.C:63-85)
                const float gx = ga[0], gy = ga[1], gz = ga[2];
                const float c0[6] = {gx, 0.f, 0.f, 0.f, gz, gy}, c1[6] = {0.f, gy, 0.f, gz, 0.f, gx},
                            c2[6] = {0.f, 0.f, gz, gy, gx, 0.f};
                for (int s = 0; s < 6; ++s) {
                    Bc[0][s] = c0[s];
                    Bc[1][s] = c1[s];
                    Bc[2][s] = c2[s];
                }
            } else {
                // xx, yy, xy with the shear row at the element centre (planstrss.C:78-106)
                Bc[0][0] = ga[0]; Bc[0][1] = 0.f; Bc[0][2] = gsa[1];
                Bc[1][0] = 0.f; Bc[1][1] = ga[1]; Bc[1][2] = gsa[0];
            }
            for (int i = 0; i < ND; ++i) {
                const int row = le * L::NDOF + a * ND + i;
                for (int s = 0; s < NS; ++s) {
                    float h = 0.f;
                    for (int u = 0; u < NS; ++u) h = fmaf(Dq[s * NS + u], Bc[i][u], h);
                    const int k = gp * NS + s;
                    store_split3<L::KP>(oper, L::PIECE, 0, row, k, Bc[i][s]);
                    store_split3<L::KP>(oper, L::PIECE, 3, row, k, h * dv);
                }
            }
        }
        tc::fence_smem_async();
        __syncthreads();
        // (3) one thread issues the split products: A_i B_j with i + j <= 2
        if (tid == 0) {
            tc::fence_after_sync();
            const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
            uint32_t acc = 0;
            for (int ks = 0; ks < L::KP / 16; ++ks)
                for (int pr = 0; pr < 6; ++pr) {
                    const uint64_t ad = tc::smem_desc(abase + pa[pr] * L::PIECE + ks * 256, LBO, SBO);
                    const uint64_t bd = tc::smem_desc(abase + (3 + pb[pr]) * L::PIECE + ks * 256, LBO, SBO);
                    tc::mma_bf16(tmem, ad, bd, idesc, acc);
                    acc = 1;
                }
            tc::mma_commit(bar);
            s_ok = tc::mbar_wait_bounded(bar, phase, WAIT_CYCLES) ? 1 : 0;
        }
        phase ^= 1;
        __syncthreads();
        if (!s_ok) {
            failed = true;
            if (tid == 0) atomicCAS(status, DS_OK, DS_TIMEOUT);
            break;
        }
        tc::fence_after_sync();
        // (4) each warp reads its 32 lanes; thread = row rr = (a, i) of element le.
        // The upper triangle (column >= row) is written to both (rr, c) and (c, rr):
        // B^T D B is symmetric for these materials, and the split products of an
        // entry and of its transpose round differently, so the element matrix is
        // made exactly symmetric as the FP32 operator of the solve assumes (the
        // reference likewise fills the upper triangle and mirrors it,
        // plusProductSymmUpper + symmetrized, nlstructuralelement.C:365-376).
        {
            const int le = tid / L::NDOF, rr = tid % L::NDOF, e = e0 + le;
            const bool valid = le < L::EPT && e < nelem;
            const int a = rr / ND, i = rr % ND;
            const int lo_e = (32 * warp) / L::NDOF;
            const int hi_e = min(L::EPT - 1, (32 * warp + 31) / L::NDOF);
            const int c_lo = (lo_e * L::NDOF) & ~7;
            const int c_hi = min(128, (hi_e + 1) * L::NDOF);
            double *eb = valid ? ke + (size_t)e * NPE * NPE * ND * ND : nullptr;
            for (int c0 = c_lo; c0 < c_hi; c0 += 8) {
                float v[8];
                tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
                for (int qq = 0; qq < 8; ++qq) {
                    const int c = c0 + qq - le * L::NDOF;
                    if (valid && c >= rr && c < L::NDOF) {
                        const int b = c / ND, j = c % ND;
                        const double val = (double)v[qq];
                        eb[((a * NPE + b) * ND + i) * ND + j] = val;   // (rr, c)
                        eb[((b * NPE + a) * ND + j) * ND + i] = val;   // (c, rr)
                    }
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    // a failed tile's MMAs get one more bounded wait before the tensor memory is freed
    if (failed && tid == 0) tc::mbar_wait_bounded(bar, phase ^ 1u, WAIT_CYCLES);
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

template <int ET>
static int run_stiffness_tc(ogb_model *md)
{
    ogb_ctx *ctx = md->ctx;
    constexpr size_t smem = TcTile<ET>::SMEM;
    static bool attr_set[64] = {};
    OGB_CUDA(set_smem_limit_once((const void *)k_elem_stiffness_tc<ET>, (int)smem, attr_set));
    const int ntiles = (int)ceil_div(md->nelem, TcTile<ET>::EPT);
    const int grid = ntiles < num_sms() * 2 ? ntiles : num_sms() * 2;
    if (grid > 0)
        k_elem_stiffness_tc<ET><<<grid, 128, smem, ctx->stream>>>(md->nelem, md->coords.p, md->conn.p, md->emat.p,
                                                                  md->mats.p, md->Dmat.p,
                                                                  md->nonlinear ? md->state.p : nullptr,
                                                                  md->thickness, md->ke.p, ctx->status.p);
    count_launch(ctx);
    OGB_CUDA(cudaGetLastError());
    return OGB_OK;
}

int launch_elem_stiffness_tc(ogb_model *md)
{
    switch (md->etype) {
    case OGB_LSPACE: return run_stiffness_tc<OGB_LSPACE>(md);
    case OGB_PLANESTRESS2D: return run_stiffness_tc<OGB_PLANESTRESS2D>(md);
    case OGB_LTRSPACE: return run_stiffness_tc<OGB_LTRSPACE>(md);
    }
    return fail(OGB_E_ARG, "unknown element type");
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
