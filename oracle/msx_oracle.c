/*
 * msx_oracle.c -- CPU restatement of MuPhiSim v1.1's explicit C3D4 step.
 *
 * TEST INFRASTRUCTURE ONLY (see msx_oracle.h).  Each routine cites the
 * reference file:line it restates and keeps the reference's operation order,
 * so that built with -ffp-contract=off it agrees bit for bit with the
 * reference compiled without FMA contraction.
 */
#include "msx_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/mathematics/maths.cpp:1564-1577 determinantTensor (3x3 branch). */
static double det3(const double *A)
{
    return A[0] * (A[4] * A[8] - A[7] * A[5]) -
           A[1] * (A[3] * A[8] - A[6] * A[5]) +
           A[2] * (A[3] * A[7] - A[6] * A[4]);
}

/* src/mathematics/maths.cpp:2749-2785 inverse (nn == 3 branch). */
static void inverse3(const double *A, double *Ai)
{
    const int nn = 3;
    double det = det3(A);
    double idet = 1.0 / det;
    Ai[0] = idet * (A[nn + 1] * A[nn * 2 + 2] - A[nn * 1 + 2] * A[nn * 2 + 1]);
    Ai[nn] = -idet * (A[nn * 1 + 0] * A[nn * 2 + 2] - A[nn * 1 + 2] * A[nn * 2 + 0]);
    Ai[nn * 2] = idet * (A[nn * 1 + 0] * A[nn * 2 + 1] - A[nn * 1 + 1] * A[nn * 2 + 0]);
    Ai[1] = -idet * (A[nn * 0 + 1] * A[nn * 2 + 2] - A[nn * 0 + 2] * A[nn * 2 + 1]);
    Ai[nn + 1] = idet * (A[nn * 0 + 0] * A[nn * 2 + 2] - A[nn * 0 + 2] * A[nn * 2 + 0]);
    Ai[2 * nn + 1] = -idet * (A[nn * 0 + 0] * A[nn * 2 + 1] - A[nn * 0 + 1] * A[nn * 2 + 0]);
    Ai[2] = idet * (A[nn * 0 + 1] * A[nn * 1 + 2] - A[nn * 0 + 2] * A[nn * 1 + 1]);
    Ai[nn + 2] = -idet * (A[nn * 0 + 0] * A[nn * 1 + 2] - A[nn * 0 + 2] * A[nn * 1 + 0]);
    Ai[2 * nn + 2] = idet * (A[nn * 0 + 0] * A[nn * 1 + 1] - A[nn * 0 + 1] * A[nn * 1 + 0]);
}

/* src/mathematics/geometry.cpp:180-190 crossProduct + :90-136 areaTriangle
 * (ndim == 3): A = v1 - v3, B = v2 - v3, area = 0.5*|A x B|.  The argument
 * layout is the reference's {x1,x2,x3, y1,y2,y3, z1,z2,z3}. */
static double area_triangle(const double *nodes)
{
    double A[3], B[3], C[3];
    for (int i = 0; i < 3; i++) {
        A[i] = nodes[i * 3] - nodes[i * 3 + 2];
        B[i] = nodes[i * 3 + 1] - nodes[i * 3 + 2];
    }
    C[0] = A[1] * B[2] - A[2] * B[1];
    C[1] = A[2] * B[0] - A[0] * B[2];
    C[2] = A[0] * B[1] - A[1] * B[0];
    return 0.5 * sqrt(C[0] * C[0] + C[1] * C[1] + C[2] * C[2]);
}

/* src/mathematics/geometry.cpp:264-301 inscribedSphere, times two as in
 * src/spatialDiscretisation/classLinearTetrahedra.cpp:146-163
 * characteristicLength.  x[a*3+c] = coordinate c of vertex a. */
double orc_char_length(const double *x)
{
    const double *p0 = x, *p1 = x + 3, *p2 = x + 6, *p3 = x + 9;
    double arg[9], s1, s2, s3, s4;
#define TRI(P, Q, R) \
    arg[0] = P[0]; arg[1] = Q[0]; arg[2] = R[0]; \
    arg[3] = P[1]; arg[4] = Q[1]; arg[5] = R[1]; \
    arg[6] = P[2]; arg[7] = Q[2]; arg[8] = R[2];
    TRI(p0, p1, p2) s1 = area_triangle(arg);
    TRI(p1, p2, p3) s2 = area_triangle(arg);
    TRI(p0, p2, p3) s3 = area_triangle(arg);
    TRI(p0, p1, p3) s4 = area_triangle(arg);
#undef TRI
    double A = fabs(s1) + fabs(s2) + fabs(s3) + fabs(s4);
    double M[9] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2],
                   p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2],
                   p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
    double V = 1.0 / 6.0 * fabs(det3(M));
    double r = 3.0 * V / A;
    return 2 * r;
}

/* src/spatialDiscretisation/classLinearTetrahedra.cpp:171-292 defineGPs and
 * getInterpolationParameters; GPsDistribution.cpp:334-342 (1-point rule,
 * weight literal 0.166666666667); classGPs.cpp:24-31 (wJ = w*|J|);
 * maths.cpp:1679-1692 multGeneralMatrices (accumulation from 0). */
int orc_precompute(int64_t nn, int64_t ne, const double *X, const int32_t *conn,
                   double *dphi, double *wJ, double *Lref)
{
    static const double natDev[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0,
                                      0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    const double w = 0.166666666667;
    int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (int64_t e = 0; e < ne; e++) {
        double xyz[12], pts[12], Jac[9], invJ[9];
        for (int k = 0; k < 4; k++) {
            int64_t nd = conn[e * 4 + k];
            if (nd < 0 || nd >= nn) { bad = 1; nd = 0; }
            for (int i = 0; i < 3; i++) {
                xyz[i * 4 + k] = X[i * nn + nd];
                pts[k * 3 + i] = X[i * nn + nd];
            }
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 4; k++) c += xyz[i * 4 + k] * natDev[k * 3 + j];
                Jac[i * 3 + j] = c;
            }
        double J = det3(Jac);
        inverse3(Jac, invJ);
        for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += natDev[a * 3 + k] * invJ[k * 3 + j];
                dphi[e * 12 + a * 3 + j] = c;
            }
        wJ[e] = w * fabs(J);
        Lref[e] = orc_char_length(pts);
    }
    return bad ? ORC_ERR_ARG : ORC_OK;
}

/* constitutiveAlgorithms.cpp:135-206 getLumpedMassVector (generic branch),
 * solverExplicit.cpp:429-459 computeLumpedMassVector (element-order sum). */
int orc_lumped_mass(int64_t nn, int64_t ne, const int32_t *conn, const double *wJ,
                    const int32_t *elem_mat, const orc_material *mats, double *mass)
{
    const double phi = -1.0 * 0.25 - 1.0 * 0.25 - 1.0 * 0.25 + 1.0;
    for (int64_t i = 0; i < nn; i++) mass[i] = 0;
    for (int64_t e = 0; e < ne; e++) {
        double rho = mats[elem_mat ? elem_mat[e] : 0].rho;
        double m = 0;
        for (int b = 0; b < 4; b++) m += wJ[e] * rho * phi * phi;
        for (int a = 0; a < 4; a++) mass[conn[e * 4 + a]] += m;
    }
    return ORC_OK;
}

/* hyperElasticNeoHookean.cpp:51-54, hyperElasticStVenantKirchhoff.cpp:50-55,
 * linearElastic.cpp:43-48. */
double orc_sound_speed(const orc_material *m)
{
    double E = m->young, nu = m->nu;
    if (m->law == ORC_STVK || m->law == ORC_LINEAR_ELASTIC) return sqrt(E / m->rho);
    double lambda = (E * nu) / ((1. + nu) * (1. - 2. * nu));
    double mu = 0.5 * E / (1. + nu);
    return sqrt((lambda + 2 * mu) / m->rho);
}

void orc_stress(const orc_material *m, const double *F, double *P)
{
    double E = m->young, nu = m->nu;
    if (m->law == ORC_COMPRESSIBLE_NH) {
        /* hyperElasticNeoHookean.cpp:221-259; TensorOperations.h:22-75,478-512,215-229 */
        double lambda = (E * nu) / ((1. + nu) * (1. - 2. * nu));
        double mu = 0.5 * E / (1. + nu);
        double J = det3(F), C[9], invC[9], PK2[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = c;
            }
        inverse3(C, invC);
        for (int i = 0; i < 9; i++) PK2[i] = 0;
        for (int i = 0; i < 3; i++) PK2[i * 3 + i] += mu;
        double alpha = lambda * log(J) - mu;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) PK2[i * 3 + j] += alpha * invC[i * 3 + j];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * PK2[k * 3 + j] * 1.;
                P[i * 3 + j] = c;
            }
    } else if (m->law == ORC_LINEAR_ELASTIC) {
        /* linearElastic.cpp:58-82 (E = (F + F^T)/2 - I), :114-145 stress (3D branch):
         * P = E mu2, then P_ii += lam tr(E) */
        double Eg[9], mu2 = E / (1. + nu), lam = E * nu / ((1. + nu) * (1. - (2 * nu))), trE = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Eg[i * 3 + j] = 0.5 * (F[i * 3 + j] + F[j * 3 + i] - 2. * (i == j ? 1. : 0.));
        for (int i = 0; i < 3; i++) trE += Eg[i * 3 + i];
        for (int i = 0; i < 9; i++) P[i] = Eg[i] * mu2;
        for (int i = 0; i < 3; i++) P[i * 3 + i] += lam * trE;
    } else if (m->law == ORC_NEO_HOOKEAN) {
        /* hyperElasticNeoHookean.cpp:23-33 (constants), :70-127 (stress);
         * TensorOperations.h:517-551 leftCauchy, :577-592 dotSecondTranspose */
        double mu = 0.5 * E / (1. + nu);
        double K1 = E / (3 * (1 - 2 * nu));
        double B[9], invF[9], Ca[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * F[j * 3 + k];
                B[i * 3 + j] = c;
            }
        double J = det3(F);
        inverse3(F, invF);
        double traceB = 0;
        for (int i = 0; i < 3; i++) traceB += B[i * 3 + i];
        double fact1 = pow(J, 5.0 / 3.0);
        double fact2 = mu / fact1;
        for (int i = 0; i < 9; i++) Ca[i] = 0;
        for (int i = 0; i < 9; i++) Ca[i] += fact2 * B[i];
        double fact3 = -(mu / 3.0) * traceB / fact1 + K1 * (J - 1.0);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Ca[i * 3 + j] += fact3 * (i == j ? 1.0 : 0.0);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += Ca[i * 3 + k] * invF[j * 3 + k] * J;
                P[i * 3 + j] = c;
            }
    } else {
        /* hyperElasticStVenantKirchhoff.cpp:64-101 stress, :203-227;
         * maths.cpp:1227-1243 computeGL, :1703-1715 multTensorTensor3 */
        double C[9], Eg[9], S[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = c;
            }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Eg[i * 3 + j] = 0.5 * (C[i * 3 + j] - (i == j ? 1.0 : 0.0));
        double mu2 = E / (1. + nu);
        double lam = E * nu / ((1. + nu) * (1. - (2 * nu)));
        double trE = 0;
        for (int i = 0; i < 3; i++) trE += Eg[i * 3 + i];
        for (int i = 0; i < 9; i++) S[i] = Eg[i] * mu2;
        for (int i = 0; i < 3; i++) S[i * 3 + i] += lam * trE;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[i * 3 + k] * S[k * 3 + j];
                P[i * 3 + j] = c;
            }
    }
}

/* solvers.cpp:403-433 updateActivation with the laws' checkActivation
 * (hyperElasticStVenantKirchhoff.cpp:185-194, linearElastic.cpp:230-239): with
 * the *ACTIVATION option a St-Venant-Kirchhoff or linear-elastic Gauss point is
 * active once its first internal variable (the activation time) is <= t; the
 * neo-Hookean laws have no such variable and stay active. */
static int gp_active(const orc_problem *p, int64_t e, double t)
{
    if (!p->activation || !p->act_time) return 1;
    int law = p->mats[p->elem_mat ? p->elem_mat[e] : 0].law;
    if (law != ORC_STVK && law != ORC_LINEAR_ELASTIC) return 1;
    return p->act_time[e] <= t;
}

/* constitutiveManager.cpp:137-164 computeKinematicVariables (F), then the law,
 * then constitutiveAlgorithms.cpp:33-57 getForceVector; fe[a + 4*i]. */
static void element_force(const double *dphi, double wJ, const orc_material *m,
                          const double *ue /* ue[a*3+i] */, double *fe, double *Fo, double *Po)
{
    double F[9], P[9];
    for (int i = 0; i < 9; i++) F[i] = 0.;
    for (int i = 0; i < 3; i++) {
        F[i * 3 + i] += 1.;
        for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dphi[a * 3 + j] * ue[a * 3 + i];
    }
    orc_stress(m, F, P);
    for (int a = 0; a < 4; a++)
        for (int i = 0; i < 3; i++) {
            double f = 0;
            for (int J = 0; J < 3; J++) f += wJ * P[i * 3 + J] * dphi[a * 3 + J];
            fe[a + 4 * i] = 0 + f;
        }
    if (Fo) memcpy(Fo, F, sizeof F);
    if (Po) memcpy(Po, P, sizeof P);
}

/* Output fields: F (constitutiveManager.cpp:151-164); Cauchy = the
 * Neo-Hookean law's sigma (hyperElasticNeoHookean.cpp:113-124) or P F^T / J
 * (maths.cpp:1250-1254 computeCauchy) for the other two laws; Green-Lagrange
 * (maths.cpp:1227-1243); von Mises (maths.cpp:1261-1271). */
int orc_element_fields(int64_t nn, int64_t ne, const int32_t *conn, const double *dphi, const int32_t *elem_mat,
                       const orc_material *mats, const double *u, double *cauchy, double *gl, double *vms)
{
    for (int64_t e = 0; e < ne; e++) {
        const double *dp = dphi + 12 * e;
        const orc_material *m = &mats[elem_mat ? elem_mat[e] : 0];
        double F[9], P[9], S[9], C[9];
        for (int i = 0; i < 9; i++) F[i] = 0.;
        for (int i = 0; i < 3; i++) {
            F[i * 3 + i] += 1.;
            for (int a = 0; a < 4; a++)
                for (int j = 0; j < 3; j++) F[i * 3 + j] += dp[a * 3 + j] * u[conn[e * 4 + a] + i * nn];
        }
        if (m->law == ORC_NEO_HOOKEAN) {
            double E = m->young, nu = m->nu, mu = 0.5 * E / (1. + nu), K1 = E / (3 * (1 - 2 * nu)), B[9];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    double c = 0;
                    for (int k = 0; k < 3; k++) c += F[i * 3 + k] * F[j * 3 + k];
                    B[i * 3 + j] = c;
                }
            double J = det3(F), trB = 0;
            for (int i = 0; i < 3; i++) trB += B[i * 3 + i];
            double fact1 = pow(J, 5.0 / 3.0), fact2 = mu / fact1;
            for (int i = 0; i < 9; i++) S[i] = 0 + fact2 * B[i];
            double fact3 = -(mu / 3.0) * trB / fact1 + K1 * (J - 1.0);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) S[i * 3 + j] += fact3 * (i == j ? 1.0 : 0.0);
        } else {
            orc_stress(m, F, P);
            double detJinv = 1. / det3(F);
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) {
                    double c = 0;
                    for (int k = 0; k < 3; k++) c += P[i * 3 + k] * F[j * 3 + k];
                    S[i * 3 + j] = c;
                }
            for (int i = 0; i < 9; i++) S[i] = S[i] * detJinv;
        }
        /* the compressible neo-Hookean law never updates its Green-Lagrange
         * strain (hyperElasticNeoHookean.cpp:221-289 has no computeGL), so the
         * reference reports it as zero; the linear-elastic law stores its
         * small strain there (linearElastic.cpp:71-76) */
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double c = 0;
                for (int k = 0; k < 3; k++) c += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = m->law == ORC_COMPRESSIBLE_NH ? 0.0
                             : m->law == ORC_LINEAR_ELASTIC ? 0.5 * (F[i * 3 + j] + F[j * 3 + i] - 2. * (i == j ? 1. : 0.))
                                                            : 0.5 * (c - (i == j ? 1.0 : 0.0));
            }
        for (int k = 0; k < 9; k++) {
            if (cauchy) cauchy[e * 9 + k] = S[k];
            if (gl) gl[e * 9 + k] = C[k];
        }
        if (vms)
            vms[e] = sqrt(0.5 * ((S[0] - S[4]) * (S[0] - S[4]) + (S[4] - S[8]) * (S[4] - S[8]) +
                                 (S[8] - S[0]) * (S[8] - S[0]) + 6 * (S[1] * S[1] + S[2] * S[2] + S[5] * S[5])));
    }
    return ORC_OK;
}

/* classSolverExplicit::bulkViscosity (solverExplicit.cpp:514-541): the
 * viscous first Piola stress from the current and previous F of one Gauss
 * point, in the reference's operation order (sumTensorTensor with factor -1,
 * multiSTensorScalar by 1/dt, getTrace, maths.cpp:1169-1175, 1604-1610,
 * 2257-2286).  The quadratic term takes |trD| as fabs; std::min(0., trD) is
 * (trD < 0) ? trD : 0. */
static void bulk_viscosity(double h, double c1, double cl, double c0, const double *F1, const double *F0,
                           double rho, double dt, double *P)
{
    double Fdot[9];
    if (dt == 0) {
        for (int k = 0; k < 9; k++) Fdot[k] = 0.;
    } else {
        for (int k = 0; k < 9; k++) Fdot[k] = F1[k] + (-1) * F0[k];
        for (int k = 0; k < 9; k++) Fdot[k] = Fdot[k] * (1 / dt);
    }
    double trD = 0;
    for (int i = 0; i < 3; i++) trD += Fdot[i * 3 + i];
    double J1 = det3(F1);
    double Rho_1 = rho / J1;
    double qBV = Rho_1 * h * (c1 * c1 * h * fabs(trD) * ((trD < 0.) ? trD : 0.) + cl * c0 * trD);
    double Cv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, iF[9];
    for (int i = 0; i < 3; i++) Cv[i + i * 3] = -1 * qBV;
    inverse3(F1, iF);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            P[i * 3 + j] = 0;
            for (int k = 0; k < 3; k++) P[i * 3 + j] += Cv[i * 3 + k] * iF[j * 3 + k];
        }
    for (int k = 0; k < 9; k++) P[k] = P[k] * (-1 * J1);
}

/* classSolverExplicit::artificialViscosity (solverExplicit.cpp:469-502): its
 * scaled deviatoric rate is never stored in the Cauchy tensor it maps, so the
 * Piola stress is that zero tensor times F^-T, times J (the rest of the
 * routine has no effect on the result). */
static void dev_viscosity(const double *F1, double *P)
{
    double Cv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, iF[9];
    double J1 = det3(F1);
    inverse3(F1, iF);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            P[i * 3 + j] = 0;
            for (int k = 0; k < 3; k++) P[i * 3 + j] += Cv[i * 3 + k] * iF[j * 3 + k];
        }
    for (int k = 0; k < 9; k++) P[k] = P[k] * J1;
}

/* The viscous pass of computeInternalForce (solverExplicit.cpp:381-421): after
 * the elastic scatter, per Gauss point in element order, fint += wJ P_vis dphi
 * term by term.  F1: the elements' current F; F0: their previous F. */
static void viscous_force(const orc_problem *p, const double *dphi, const double *wJ, const double *F1,
                          const double *F0, double dt, double t, double *fint)
{
    const int64_t nn = p->nn;
    for (int64_t e = 0; e < p->ne; e++) {
        if (!gp_active(p, e, t)) continue;
        const orc_material *m = &p->mats[p->elem_mat ? p->elem_mat[e] : 0];
        double P[9];
        if (p->viscosity == 1)
            bulk_viscosity(p->visc_h, p->visc_c1, p->visc_cl, p->visc_c0, F1 + 9 * e, F0 + 9 * e, m->rho, dt, P);
        else
            dev_viscosity(F1 + 9 * e, P);
        const double *dp = dphi + 12 * e;
        for (int a = 0; a < 4; a++)
            for (int i = 0; i < 3; i++) {
                const int64_t d = p->conn[e * 4 + a] + nn * i;
                for (int J = 0; J < 3; J++) fint[d] += wJ[e] * P[i * 3 + J] * dp[a * 3 + J];
            }
    }
}

/* solverExplicit.cpp:363-379 computeInternalForce: scatter in element order. */
static int internal_force(int64_t nn, int64_t ne, const int32_t *conn, const double *dphi,
                          const double *wJ, const int32_t *elem_mat, const orc_material *mats,
                          const double *u, double *fint, double *F_out, double *P_out, int nthreads,
                          const orc_problem *act, double t)
{
    double *fe = (double *)malloc(sizeof(double) * 12 * (size_t)(ne > 0 ? ne : 1));
    if (!fe) return ORC_ERR_ARG;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t e = 0; e < ne; e++) {
        if (act && !gp_active(act, e, t)) continue;   /* solverExplicit.cpp:370-371 */
        double ue[12];
        for (int a = 0; a < 4; a++)
            for (int i = 0; i < 3; i++) ue[a * 3 + i] = u[conn[e * 4 + a] + i * nn];
        element_force(dphi + 12 * e, wJ[e], &mats[elem_mat ? elem_mat[e] : 0], ue, fe + 12 * e,
                      F_out ? F_out + 9 * e : 0, P_out ? P_out + 9 * e : 0);
    }
    (void)nthreads;
    for (int64_t i = 0; i < 3 * nn; i++) fint[i] = 0;
    for (int64_t e = 0; e < ne; e++) {
        if (act && !gp_active(act, e, t)) continue;
        for (int i = 0; i < 3; i++)
            for (int a = 0; a < 4; a++) fint[conn[e * 4 + a] + nn * i] += fe[12 * e + a + 4 * i];
    }
    free(fe);
    return ORC_OK;
}

int orc_internal_force(int64_t nn, int64_t ne, const int32_t *conn, const double *dphi,
                       const double *wJ, const int32_t *elem_mat, const orc_material *mats,
                       const double *u, double *fint, double *F_out, double *P_out, int nthreads)
{
    return internal_force(nn, ne, conn, dphi, wJ, elem_mat, mats, u, fint, F_out, P_out, nthreads, 0, 0.0);
}

/* solvers.cpp:296-320 calculateCriticalTimeStep(nod, elem, uK) without the
 * scale factor; uK == NULL gives the undeformed variant of :276-287. */
static double critical_dt(int64_t nn, int64_t ne, const double *X, const int32_t *conn,
                          const double *Lref, const double *cel, const double *uK, int nthreads)
{
    double best = INFINITY;
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(min : best) num_threads(nthreads > 0 ? nthreads : 1)
#endif
    for (int64_t e = 0; e < ne; e++) {
        double v;
        if (!uK) {
            v = Lref[e] / cel[e];
        } else {
            double x[12];
            for (int a = 0; a < 4; a++)
                for (int k = 0; k < 3; k++) {
                    int64_t nd = conn[e * 4 + a];
                    x[a * 3 + k] = X[k * nn + nd];
                    x[a * 3 + k] += uK[nn * k + nd];
                }
            double dist = orc_char_length(x);
            double m = (dist < Lref[e]) ? dist : Lref[e]; /* std::min(minDist, dist) */
            v = m / cel[e];
        }
        if (v < best) best = v;
    }
    return best;
}

/* src/mathematics/maths.cpp:1550-1557 norm2 */
static double norm2_3(const double *a)
{
    double temp = 0;
    for (int i = 0; i < 3; i++) temp += a[i] * a[i];
    return sqrt(temp);
}

/* src/mathematics/geometry.cpp:180-190 crossProduct */
static void cross3(const double *A, const double *B, double *C)
{
    C[0] = A[1] * B[2] - A[2] * B[1];
    C[1] = A[2] * B[0] - A[0] * B[2];
    C[2] = A[0] * B[1] - A[1] * B[0];
}

/* Face S of a tet: classLinearTetrahedra::getSubElement, classLinearTetrahedra.cpp:30-62. */
static void tet_face(const int32_t *c, int S, int32_t *t)
{
    if (S == 1) { t[0] = c[0]; t[1] = c[1]; t[2] = c[2]; }
    else if (S == 2 || S == 3) { t[0] = c[S - 2]; t[1] = c[3]; t[2] = c[S - 1]; }
    else { t[0] = c[0]; t[1] = c[2]; t[2] = c[S - 1]; }
}

/* The face triangle's one Gauss point: weight * |J| and phi.
 * classLinearTriangles::defineGPs (classLinearTriangles.cpp:194-290) with
 * GPsTriangle2DValues order 1 (GPsDistribution.cpp:149-155), the local basis of
 * createOrthogonalBasisOnPlane (geometry.cpp:363-390), vectorArithmetic
 * (maths.cpp:3107-3117), multGeneralMatrices (maths.cpp:1679-1693) and the
 * triangle's shape functions (classLinearTriangles.cpp:302-317).  xyz = the three
 * face nodes, node-major. */
static void face_rule(const double *xyz, double *wabsJ, double *phi)
{
    const double *p1 = xyz;
    double a[3], b[3], normal[3], xhat[3], yhat[3];
    for (int i = 0; i < 3; i++) {
        a[i] = xyz[3 + i] + (-1.0) * p1[i];
        b[i] = xyz[6 + i] + (-1.0) * p1[i];
    }
    cross3(b, a, normal);
    cross3(a, normal, xhat);
    double magA = norm2_3(a), magX = norm2_3(xhat);
    for (int i = 0; i < 3; i++) {
        yhat[i] = a[i] / magA;
        xhat[i] = xhat[i] / magX;
    }
    double map[6] = {xhat[0], xhat[1], xhat[2], yhat[0], yhat[1], yhat[2]};
    double T[9];   /* T[r*3 + k]: coordinate r of node k, offset by p1 */
    for (int k = 0; k < 3; k++)
        for (int r = 0; r < 3; r++) T[r * 3 + k] = xyz[k * 3 + r] + (-1.0) * p1[r];
    double L[6];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 3; j++) {
            L[i * 3 + j] = 0;
            for (int k = 0; k < 3; k++) L[i * 3 + j] += map[i * 3 + k] * T[k * 3 + j];
        }
    const double natDev[6] = {-1.0 - 0.0 + 0.0, -0.0 - 1.0 + 0.0, 1.0, 0.0, 0.0, 1.0};
    double Jm[4];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            Jm[i * 2 + j] = 0;
            for (int k = 0; k < 3; k++) Jm[i * 2 + j] += L[i * 3 + k] * natDev[k * 2 + j];
        }
    double J = Jm[0] * Jm[3] - Jm[2] * Jm[1];   /* determinantTensor, size 2 */
    double weight = 0.5 * 1.;
    *wabsJ = weight * fabs(J);
    const double x = 0.33333333333333, y = 0.33333333333333;
    phi[0] = -1.0 * x - 1.0 * y + 1.0;
    phi[1] = 1.0 * x;
    phi[2] = 1.0 * y;
}

/* Unit normal of the face triangle: classLinearTriangles::getn0, classLinearTriangles.cpp:19-45. */
static void face_normal(const double *xyz, double *n0)
{
    const double *x1 = xyz, *x2 = xyz + 3, *x3 = xyz + 6;
    for (int i = 0; i < 3; i++) {
        int c1 = i == 0 ? 1 : (i == 1 ? 2 : 0), c2 = i == 0 ? 2 : (i == 1 ? 0 : 1);
        n0[i] = (x2[c1] - x1[c1]) * (x3[c2] - x1[c2]) - (x3[c1] - x1[c1]) * (x2[c2] - x1[c2]);
    }
    double no = norm2_3(n0);
    for (int i = 0; i < 3; i++) n0[i] = n0[i] / no;
}

/* Traction and pressure of one block (boundaryConditions.cpp:218-275 BCsTractionInst/Ramp,
 * :370-505 BCsPressureRamp/Inst, classNeumannBCs.h:57-181 for the amounts).  Pressure
 * follows the face: n = F^-T n0 with F of the bulk tet (classSpatialPoint::getF,
 * classSpatialPoint.cpp:41-66, with the tet's dphi), force w|J| phi_a det(F) P n_i.
 * The ramp variant takes phi and the node list of the bulk tet evaluated at natural
 * coordinates 0 (classLinearTetrahedra::defineShapeOnAPoint, :66-121, :270-292), so
 * phi = (1, 0, 0, 0): the face's force goes to the tet's first node. */
static void surface_block(const orc_problem *p, const orc_load *L, const double *dphi, const double *u,
                          double t, double *fext)
{
    const int64_t nn = p->nn;
    const int ramp = L->kind == ORC_LOAD_TRACTION_RAMP || L->kind == ORC_LOAD_PRESSURE_RAMP;
    const int pressure = L->kind == ORC_LOAD_PRESSURE_INST || L->kind == ORC_LOAD_PRESSURE_RAMP;
    double amount[3] = {0, 0, 0};
    if (t >= L->t0 && t <= L->tf)
        for (int i = 0; i < (pressure ? 1 : 3); i++)
            amount[i] = ramp ? L->value[i] / (L->tf - L->t0) * (t - L->t0) : L->value[i];
    for (int64_t k = 0; k < L->nelems; k++) {
        const int64_t e = L->elems[k];
        const int32_t *c = p->conn + 4 * e;
        int32_t tri[3];
        tet_face(c, L->face, tri);
        double xyz[9], wabsJ, phi[3];
        for (int a = 0; a < 3; a++)
            for (int i = 0; i < 3; i++) xyz[a * 3 + i] = p->X[i * nn + tri[a]];
        face_rule(xyz, &wabsJ, phi);
        if (!pressure) {
            for (int a = 0; a < 3; a++)
                for (int i = 0; i < 3; i++) fext[tri[a] + i * nn] += wabsJ * phi[a] * amount[i];
            continue;
        }
        double n0[3];
        face_normal(xyz, n0);
        double F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < 4; a++) {
            const double *ds = dphi + 12 * e + 3 * a;
            double disp[3];
            for (int i = 0; i < 3; i++) disp[i] = u[c[a] + i * nn];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) F[i * 3 + j] += ds[j] * disp[i];
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) F[i * 3 + j] += (i == j ? 1 : 0);
        double Jac = det3(F), Fi[9], n[3] = {0, 0, 0};
        inverse3(F, Fi);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) n[i] += Fi[j * 3 + i] * n0[j];   /* (F^-1)^T n0 */
        if (ramp) {
            const double phit[4] = {-1.0 * 0 - 1.0 * 0 - 1.0 * 0 + 1.0, 1.0 * 0, 1.0 * 0, 1.0 * 0};
            for (int a = 0; a < 4; a++)
                for (int i = 0; i < 3; i++) fext[c[a] + i * nn] += wabsJ * phit[a] * Jac * amount[0] * n[i];
        } else {
            for (int a = 0; a < 3; a++)
                for (int i = 0; i < 3; i++) fext[tri[a] + i * nn] += wabsJ * phi[a] * Jac * amount[0] * n[i];
        }
    }
}

/* External force at displacement u and time t, src/solvers/boundaryConditions.cpp:75-138
 * (NeumannBCManagement), block by block in the order of the deck: nodal forces
 * (:17-34 BCsNodalForces with classNeumann::getTracAmount, classNodes.h:101-109,
 * slope value/(tf-t0) times the absolute time inside [t0, tf]), gravity
 * (:1146-1171 BCsGravity, -w rho |J| g phi_a on the z DOF, element order),
 * traction and pressure (surface_block). */
static void gravity_block(const orc_problem *p, const double *absJ, double g, double *fext)
{
    const double w = 0.166666666667, phi = -1.0 * 0.25 - 1.0 * 0.25 - 1.0 * 0.25 + 1.0;
    for (int64_t e = 0; e < p->ne; e++) {
        double rho = p->mats[p->elem_mat ? p->elem_mat[e] : 0].rho;
        for (int a = 0; a < 4; a++) fext[p->conn[e * 4 + a] + 2 * p->nn] += -w * rho * absJ[e] * g * phi;
    }
}

static void force_block(const orc_force *fs, int64_t n, double t, double *fext)
{
    for (int64_t k = 0; k < n; k++) {
        const orc_force *f = &fs[k];
        double m = f->value / (f->tf - f->t0);
        double F = (t >= f->t0 && t <= f->tf) ? m * t : 0;
        fext[f->dof] += F;
    }
}

static void external_force(const orc_problem *p, const double *absJ, const double *dphi, const double *u,
                           double t, double *fext)
{
    const int64_t nn = p->nn;
    for (int64_t i = 0; i < 3 * nn; i++) fext[i] = 0;
    if (p->nloads > 0) {
        for (int64_t b = 0; b < p->nloads; b++) {
            const orc_load *L = &p->loads[b];
            if (L->kind == ORC_LOAD_FORCE) force_block(L->forces, L->nforces, t, fext);
            else if (L->kind == ORC_LOAD_GRAVITY) { if (L->value[0] != 0) gravity_block(p, absJ, L->value[0], fext); }
            else surface_block(p, L, dphi, u, t, fext);
        }
        return;
    }
    for (int pass = 0; pass < 2; pass++) {
        int gravity_now = (pass == 0) == (p->gravity_first != 0);
        if (gravity_now) {
            if (p->gravity != 0) gravity_block(p, absJ, p->gravity, fext);
        } else {
            force_block(p->forces, p->nforces, t, fext);
        }
    }
}

/* The explicit solve, src/solvers/solverExplicit.cpp:63-338 (sequential build):
 * time advance with the previous dt (:227-232), dt from the deformed CFL
 * (:267-276), prediction (nonlinearSystem.cpp:1186-1200), Dirichlet
 * (solverExplicit.cpp:545-575), internal force, rhs = -fint (:598-628),
 * a = rhs/m and v += dt*(a_prev + a)/2 (nonlinearSystem.cpp:1034-1117). */
int orc_run(const orc_problem *p, double *u, double *v, double *a,
            double *dt_hist, int64_t max_hist, orc_result *res)
{
    const int64_t nn = p->nn, ne = p->ne, ndof = 3 * nn;
    int rc = ORC_OK;
    double *dphi = malloc(sizeof(double) * 12 * (size_t)ne), *wJ = malloc(sizeof(double) * (size_t)ne);
    double *Lref = malloc(sizeof(double) * (size_t)ne), *cel = malloc(sizeof(double) * (size_t)ne);
    double *mass = malloc(sizeof(double) * (size_t)nn), *fint = malloc(sizeof(double) * (size_t)ndof);
    double *uK = malloc(sizeof(double) * (size_t)ndof), *aprev = malloc(sizeof(double) * (size_t)ndof);
    double *fext = malloc(sizeof(double) * (size_t)ndof), *absJ = malloc(sizeof(double) * (size_t)ne);
    char *cons = calloc((size_t)ndof, 1);
    const int visc = p->viscosity == 1 || p->viscosity == 2;
    double *Fcur = visc ? malloc(sizeof(double) * 9 * (size_t)ne) : NULL;
    int32_t *flag = malloc(sizeof(int32_t) * (size_t)(p->nbc > 0 ? p->nbc : 1));
    double *UU = malloc(sizeof(double) * (size_t)(p->nbc > 0 ? p->nbc : 1));
    if (!dphi || !wJ || !Lref || !cel || !mass || !fint || !uK || !aprev || !cons || !flag || !UU || !fext || !absJ ||
        (visc && (!Fcur || !p->F_prev))) {
        rc = ORC_ERR_ARG;
        goto done;
    }
    if ((rc = orc_precompute(nn, ne, p->X, p->conn, dphi, wJ, Lref)) != ORC_OK) goto done;
    /* |det J| of each element, as classGPs::getJ returns it (classGPs.cpp:24-31) */
    for (int64_t e = 0; e < ne; e++) {
        double M[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) M[i * 3 + j] = p->X[i * nn + p->conn[e * 4 + j + 1]] - p->X[i * nn + p->conn[e * 4]];
        absJ[e] = fabs(det3(M));
    }
    orc_lumped_mass(nn, ne, p->conn, wJ, p->elem_mat, p->mats, mass);
    for (int64_t e = 0; e < ne; e++) cel[e] = orc_sound_speed(&p->mats[p->elem_mat ? p->elem_mat[e] : 0]);
    /* classNodes.cpp:58-74: ramp stores U/duration (flag -1), inst stores U (flag 1) */
    for (int64_t b = 0; b < p->nbc; b++) {
        const orc_bc *bc = &p->bcs[b];
        if (bc->dof < 0 || bc->dof >= ndof) { rc = ORC_ERR_ARG; goto done; }
        cons[bc->dof] = 1;
        if (bc->mode == ORC_BC_RAMP) { flag[b] = -1; UU[b] = bc->value / (p->tf - p->t0); }
        else if (bc->mode == ORC_BC_INST) { flag[b] = 1; UU[b] = bc->value; }
        else { flag[b] = 2; UU[b] = bc->value; }
    }
    /* solverExplicit.cpp:141-149: prev <- current at set-up */
    memcpy(aprev, a, sizeof(double) * (size_t)ndof);
    double t = p->t0, tf = p->tf;
    double dt = critical_dt(nn, ne, p->X, p->conn, Lref, cel, NULL, p->nthreads);
    dt = dt * p->scale_factor;
    if (res) res->dt_init = dt;
    /* :176-177 uK is refreshed from the system only when t0 < 1e-12 */
    if (t < 1E-12 && !p->first_step_zero_uK) memcpy(uK, u, sizeof(double) * (size_t)ndof);
    else memset(uK, 0, sizeof(double) * (size_t)ndof);
    int64_t step = 0;
#ifdef _OPENMP
    double wall0 = omp_get_wtime();
#endif
    while (t < tf - 1E-12) {
        if (p->max_steps > 0 && step >= p->max_steps) break;
        if (t + dt > tf) { dt = tf - t; t = tf; } else { t += dt; }
        dt = critical_dt(nn, ne, p->X, p->conn, Lref, cel, uK, p->nthreads);
        dt = dt * p->scale_factor;
        if (dt < 1E-20) { rc = ORC_ERR_NEG_JACOBIAN; break; }
        step++;
        if (dt_hist && step <= max_hist) dt_hist[step - 1] = dt;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(p->nthreads > 0 ? p->nthreads : 1)
#endif
        for (int64_t j = 0; j < ndof; j++)
            if (!cons[j]) u[j] += dt * v[j] + 0.5 * dt * dt * a[j];
        for (int64_t b = 0; b < p->nbc; b++) {
            double Ud = 0, Vd = UU[b];
            if (flag[b] == 1) { Ud = Vd; flag[b] = 0; }
            else if (flag[b] == -1) { Ud = Vd * dt; }
            else if (flag[b] == 2) {
                double r = p->bcs[b].ramp_steps > 0 && step < p->bcs[b].ramp_steps
                               ? (double)step / (double)p->bcs[b].ramp_steps : 1.0;
                Ud = Vd * r * dt;
            }
            int64_t d = p->bcs[b].dof;
            u[d] += Ud;
            v[d] = Ud;
            a[d] = 0.;
        }
        internal_force(nn, ne, p->conn, dphi, wJ, p->elem_mat, p->mats, u, fint, Fcur, 0, p->nthreads, p, t);
        if (visc) viscous_force(p, dphi, wJ, Fcur, p->F_prev, dt, t, fint);
        external_force(p, absJ, dphi, u, t, fext);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(p->nthreads > 0 ? p->nthreads : 1)
#endif
        for (int64_t j = 0; j < ndof; j++) {
            if (cons[j]) continue;
            double val = -fint[j] + fext[j];
            double rhs = 0;
            rhs += val;
            a[j] = rhs / mass[j % nn];
            v[j] += dt * ((1. - 0.5) * aprev[j] + 0.5 * a[j]);
        }
        memcpy(uK, u, sizeof(double) * (size_t)ndof);
        if (!isfinite(uK[1])) { rc = ORC_ERR_NAN; break; }
        memcpy(aprev, a, sizeof(double) * (size_t)ndof);
        /* solvers.cpp:328-343 nextStep: the Gauss points' previous state <- current */
        if (visc) memcpy(p->F_prev, Fcur, sizeof(double) * 9 * (size_t)ne);
    }
    if (res) {
        res->steps = step; res->t = t; res->dt_last = dt; res->status = rc;
#ifdef _OPENMP
        res->loop_seconds = omp_get_wtime() - wall0;
#else
        res->loop_seconds = 0;
#endif
    }
done:
    free(dphi); free(wJ); free(Lref); free(cel); free(mass); free(fint);
    free(uK); free(aprev); free(cons); free(flag); free(UU); free(fext); free(absJ); free(Fcur);
    return rc;
}

/* One Gauss point's element-extraction value at u, v (q numbered as
 * ExtractData::ElementDataType, solvers/dataExtraction.h:24-27):
 * getValueAtGP (dataExtraction.cpp:508-563) with Cauchy = P F^T / det F
 * (classStates.cpp:309-316; maths.cpp:2257-2290), the laws' defoEnergy
 * (hyperElasticNeoHookean.cpp:291-304, hyperElasticStVenantKirchhoff.cpp:251-274,
 * zero default constitutiveModels.h:91-94), kineticEnergy's density (phi = 0.25
 * at the one-point rule's centroid, dataExtraction.cpp:626-688) and volume's
 * w J det F (:690-748).  The three laws keep at most one internal variable,
 * and getValueAtGP reads INVAR k only past k of them, so INVAR1..6 are 0. */
enum { ORC_Q_FXX = 1, ORC_Q_PXX = 10, ORC_Q_SVM = 19, ORC_Q_KVM = 20, ORC_Q_INVAR1 = 21, ORC_Q_INVAR6 = 26,
       ORC_Q_DEFO = 27, ORC_Q_EXTERNAL = 28, ORC_Q_KIN = 29, ORC_Q_VOLUME = 30 };
enum { ORC_OP_MEAN = 1, ORC_OP_MIN = 2, ORC_OP_MAX = 3, ORC_OP_SUM = 4 };

static double gp_value(const orc_problem *p, const double *dphi, const double *wJ, const double *u, const double *v,
                       int q, int64_t e)
{
    const int64_t nn = p->nn;
    const int32_t *c = p->conn + 4 * e;
    const orc_material *m = &p->mats[p->elem_mat ? p->elem_mat[e] : 0];
    if (!gp_active(p, e, p->time)) return 0.;   /* dataExtraction.cpp:510 (and the energies skip it) */
    if (q >= ORC_Q_INVAR1 && q <= ORC_Q_INVAR6) return 0.;
    if (q == ORC_Q_KIN) {
        double vel[3] = {0., 0., 0.}, val = 0;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) vel[j] += 0.25 * v[c[i] + j * nn];
        for (int j = 0; j < 3; j++) val += 0.5 * m->rho * vel[j] * vel[j];
        return val;
    }
    if (q == ORC_Q_DEFO && m->law == ORC_NEO_HOOKEAN) return 0.;
    if (q == ORC_Q_DEFO && m->law == ORC_LINEAR_ELASTIC) {
        /* linearElastic.cpp:88-101: 0.5 (P:F - P:I), contractions summed from 0 */
        const double *dp = dphi + 12 * e;
        double F[9], P[9], a = 0, b = 0;
        for (int i = 0; i < 9; i++) F[i] = 0.;
        for (int i = 0; i < 3; i++) {
            F[i * 3 + i] += 1.;
            for (int k = 0; k < 4; k++)
                for (int j = 0; j < 3; j++) F[i * 3 + j] += dp[k * 3 + j] * u[c[k] + i * nn];
        }
        orc_stress(m, F, P);
        for (int i = 0; i < 9; i++) a += P[i] * F[i];
        for (int i = 0; i < 9; i++) b += P[i] * ((i % 4) == 0 ? 1. : 0.);
        return 0.5 * (a - b);
    }
    const double *dp = dphi + 12 * e;
    double F[9], P[9], C[9];
    for (int i = 0; i < 9; i++) F[i] = 0.;
    for (int i = 0; i < 3; i++) {
        F[i * 3 + i] += 1.;
        for (int a = 0; a < 4; a++)
            for (int j = 0; j < 3; j++) F[i * 3 + j] += dp[a * 3 + j] * u[c[a] + i * nn];
    }
    if (q >= ORC_Q_FXX && q < ORC_Q_FXX + 9) return F[q - ORC_Q_FXX];
    if (q == ORC_Q_VOLUME) return wJ[e] * det3(F);
    if (q == ORC_Q_DEFO) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int k = 0; k < 3; k++) s += F[k * 3 + i] * F[k * 3 + j];
                C[i * 3 + j] = s;
            }
        if (m->law == ORC_COMPRESSIBLE_NH) {
            double lambda = (m->young * m->nu) / ((1. + m->nu) * (1. - 2. * m->nu));
            double mu = 0.5 * m->young / (1. + m->nu);
            double J = det3(F), tr = 0;
            for (int i = 0; i < 3; i++) tr += C[i * 3 + i];
            return 0.5 * lambda * log(J) * log(J) - mu * log(J) + 0.5 * mu * tr;
        }
        double E[9], S[9], mu2 = m->young / (1. + m->nu);
        double lam = m->young * m->nu / ((1. + m->nu) * (1. - (2 * m->nu))), trE = 0, w = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) E[i * 3 + j] = 0.5 * (C[i * 3 + j] - (i == j ? 1. : 0.));
        for (int i = 0; i < 3; i++) trE += E[i * 3 + i];
        for (int i = 0; i < 9; i++) S[i] = E[i] * mu2;
        for (int i = 0; i < 3; i++) S[i * 3 + i] += lam * trE;
        for (int i = 0; i < 9; i++) w += S[i] * E[i];
        return 0.5 * w;
    }
    orc_stress(m, F, P);
    if (q >= ORC_Q_PXX && q < ORC_Q_PXX + 9) return P[q - ORC_Q_PXX];
    double detJinv = 1. / det3(F), S[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0;
            for (int k = 0; k < 3; k++) s += P[i * 3 + k] * F[j * 3 + k];
            S[i * 3 + j] = s;
        }
    for (int i = 0; i < 9; i++) S[i] = S[i] * detJinv;
    double svm = sqrt(0.5 * ((S[0] - S[4]) * (S[0] - S[4]) + (S[4] - S[8]) * (S[4] - S[8]) +
                             (S[8] - S[0]) * (S[8] - S[0]) + 6 * (S[1] * S[1] + S[2] * S[2] + S[5] * S[5])));
    return q == ORC_Q_KVM ? svm * det3(F) : svm;
}

static int element_setup(const orc_problem *p, double **dphi, double **wJ)
{
    double *Lref = malloc(sizeof(double) * (size_t)(p->ne > 0 ? p->ne : 1));
    *dphi = malloc(sizeof(double) * 12 * (size_t)(p->ne > 0 ? p->ne : 1));
    *wJ = malloc(sizeof(double) * (size_t)(p->ne > 0 ? p->ne : 1));
    int rc = (!Lref || !*dphi || !*wJ) ? ORC_ERR_ARG : orc_precompute(p->nn, p->ne, p->X, p->conn, *dphi, *wJ, Lref);
    free(Lref);
    return rc;
}

int orc_element_values(const orc_problem *p, const double *u, const double *v, int32_t q, const int32_t *elems,
                       int64_t n, double *out)
{
    double *dphi, *wJ;
    int rc = element_setup(p, &dphi, &wJ);
    if (rc == ORC_OK)
        for (int64_t k = 0; k < (elems ? n : p->ne); k++) out[k] = gp_value(p, dphi, wJ, u, v, q, elems ? elems[k] : k);
    free(dphi); free(wJ);
    return rc;
}

/* The value one *EXTRACTION, ELEMENT row holds (dataExtraction.cpp:841-889):
 * the selected Gauss points are those of the listed elements in element order,
 * each once (classElementData::initialise, :441-464); then
 * classElementData::getValue (:338-378) on weights dV/V for F..INVAR,
 * defoEnergy / kineticEnergy / volume (:569-748) for the energies and volume,
 * and u . f_ext over every DOF for the external energy (:853-861). */
int orc_element_reduce(const orc_problem *p, const double *u, const double *v, const double *fext, int32_t q,
                       int32_t op, const int32_t *elems, int64_t n, double *value)
{
    if (q == ORC_Q_EXTERNAL) {
        double energ = 0;
        for (int64_t i = 0; i < 3 * p->nn; i++) energ += u[i] * fext[i];
        *value = energ;
        return ORC_OK;
    }
    double *dphi, *wJ;
    int rc = element_setup(p, &dphi, &wJ);
    unsigned char *sel = calloc((size_t)(p->ne > 0 ? p->ne : 1), 1);
    if (!sel) rc = ORC_ERR_ARG;
    if (rc != ORC_OK) { free(dphi); free(wJ); free(sel); return rc; }
    for (int64_t k = 0; k < (elems ? n : p->ne); k++) sel[elems ? elems[k] : k] = 1;
    double val = 0;
    if (q == ORC_Q_DEFO || q == ORC_Q_KIN || q == ORC_Q_VOLUME) {
        double ener = 0, volume = 0;
        int init = 0;
        for (int64_t e = 0; e < p->ne; e++) {
            if (!sel[e] || !gp_active(p, e, p->time)) continue;
            /* defoEnergy and kineticEnergy weigh the density by dV = wJ;
             * volume's own value is its dV = wJ det F */
            double x = gp_value(p, dphi, wJ, u, v, q, e), dV = q == ORC_Q_VOLUME ? x : wJ[e];
            if (q != ORC_Q_VOLUME) volume += dV;
            if (op == ORC_OP_SUM || op == ORC_OP_MEAN) {
                ener += q == ORC_Q_VOLUME ? dV : x * dV;
            } else if (op == ORC_OP_MAX) {
                if (!init) { init = 1; ener = x; } else if (x > ener) ener = x;
            } else if (op == ORC_OP_MIN) {
                if (!init) { init = 1; ener = x; } else if (x < ener) ener = x;
            }
        }
        val = (op == ORC_OP_MEAN) ? ener / volume : ener;
    } else {
        double V = 0, acc = 0;
        for (int64_t e = 0; e < p->ne; e++)
            if (sel[e]) V += wJ[e];
        int first = 1;
        for (int64_t e = 0; e < p->ne; e++) {
            if (!sel[e]) continue;
            double x = gp_value(p, dphi, wJ, u, v, q, e);
            if (op == ORC_OP_MEAN || op == ORC_OP_SUM) acc += x * (wJ[e] / V);
            else if (first) acc = x;
            else if (op == ORC_OP_MAX ? acc < x : x < acc) acc = x;
            first = 0;
        }
        val = op == ORC_OP_SUM ? V * acc : acc;
    }
    *value = val;
    free(dphi); free(wJ); free(sel);
    return ORC_OK;
}

/* External force of all Neumann blocks at displacement u and time t (test hook). */
int orc_external_force(const orc_problem *p, const double *u, double t, double *fext)
{
    const int64_t nn = p->nn, ne = p->ne;
    double *dphi = malloc(sizeof(double) * 12 * (size_t)ne), *wJ = malloc(sizeof(double) * (size_t)ne);
    double *Lref = malloc(sizeof(double) * (size_t)ne), *absJ = malloc(sizeof(double) * (size_t)ne);
    int rc = ORC_OK;
    if (!dphi || !wJ || !Lref || !absJ) { rc = ORC_ERR_ARG; goto done; }
    if ((rc = orc_precompute(nn, ne, p->X, p->conn, dphi, wJ, Lref)) != ORC_OK) goto done;
    for (int64_t e = 0; e < ne; e++) {
        double M[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) M[i * 3 + j] = p->X[i * nn + p->conn[e * 4 + j + 1]] - p->X[i * nn + p->conn[e * 4]];
        absJ[e] = fabs(det3(M));
    }
    external_force(p, absJ, dphi, u, t, fext);
done:
    free(dphi); free(wJ); free(Lref); free(absJ);
    return rc;
}

/* Cube generator.  Node (i,j,k) has id i + (n+1) j + (n+1)^2 k at (i,j,k)/n;
 * interior nodes move by jitter*h*(2r-1) per coordinate, r from splitmix64
 * seeded with `seed`, drawn in node-id order.  Each hex (i fastest) is split
 * into 6 tets as applications/tools/Hex2Tet-Parallel/Hex2Tet-Partitioning.py
 * :87-110 does for C3D8 node order N1..N8. */
static uint64_t splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

int orc_cube_mesh(int32_t n, uint64_t seed, double jitter, double *X, int32_t *conn)
{
    if (n < 1) return ORC_ERR_ARG;
    const int64_t m = n + 1, nn = m * m * m;
    const double h = 1.0 / (double)n;
    uint64_t s = seed;
    for (int64_t k = 0; k < m; k++)
        for (int64_t j = 0; j < m; j++)
            for (int64_t i = 0; i < m; i++) {
                int64_t id = i + m * j + m * m * k;
                double c[3] = {(double)i / (double)n, (double)j / (double)n, (double)k / (double)n};
                if (i > 0 && i < n && j > 0 && j < n && k > 0 && k < n)
                    for (int d = 0; d < 3; d++) {
                        double r = (double)(splitmix64(&s) >> 11) * 0x1.0p-53;
                        c[d] += (2.0 * r - 1.0) * (jitter * h);
                    }
                for (int d = 0; d < 3; d++) X[d * nn + id] = c[d];
            }
    int64_t e = 0;
    for (int64_t k = 0; k < n; k++)
        for (int64_t j = 0; j < n; j++)
            for (int64_t i = 0; i < n; i++) {
                int32_t N[9];
                N[1] = (int32_t)(i + m * j + m * m * k);
                N[2] = N[1] + 1;
                N[3] = N[1] + 1 + (int32_t)m;
                N[4] = N[1] + (int32_t)m;
                for (int q = 5; q <= 8; q++) N[q] = N[q - 4] + (int32_t)(m * m);
                const int T[6][4] = {{1, 3, 4, 7}, {1, 2, 3, 7}, {4, 1, 7, 8},
                                     {1, 5, 7, 8}, {1, 5, 6, 7}, {2, 1, 6, 7}};
                for (int t = 0; t < 6; t++, e++)
                    for (int q = 0; q < 4; q++) conn[e * 4 + q] = N[T[t][q]];
            }
    return ORC_OK;
}
