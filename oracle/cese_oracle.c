/*
 * CPU oracle of the CESE march -- TEST INFRASTRUCTURE ONLY (see
 * cese_oracle.h).  A restatement of the reference algorithm in plain C, in the
 * reference's operation order, for checking the GPU library.  Never linked
 * into the product.
 */

#include "cese_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CLMFC 6
#define FCMND 4

/* Threads the per-cell loops of the multidim march may use (1 by default,
 * the reference's serial loop).  Every cell's arithmetic is the same either
 * way -- each loop iteration writes only its own cell's rows -- so the
 * results are bit-identical for any count; the checker uses more threads only
 * to reach larger meshes in reasonable time. */
static int g_threads = 1;

void ora_set_threads(int n) { g_threads = n > 0 ? n : 1; }

/* ---- mesh accessors (ghost rows first) --------------------------------- */

static inline double ndcrd(const ora_mesh * m, int64_t i, int d) { return m->ndcrd[(i + m->ngstnode) * m->ndim + d]; }
static inline double fccnd(const ora_mesh * m, int64_t i, int d) { return m->fccnd[(i + m->ngstface) * m->ndim + d]; }
static inline double fcnml(const ora_mesh * m, int64_t i, int d) { return m->fcnml[(i + m->ngstface) * m->ndim + d]; }
static inline double clcnd(const ora_mesh * m, int64_t i, int d) { return m->clcnd[(i + m->ngstcell) * m->ndim + d]; }
static inline int32_t fcnds(const ora_mesh * m, int64_t i, int k) { return m->fcnds[(i + m->ngstface) * 5 + k]; }
static inline int32_t fccls(const ora_mesh * m, int64_t i, int k) { return m->fccls[(i + m->ngstface) * 4 + k]; }
static inline int32_t clfcs(const ora_mesh * m, int64_t i, int k) { return m->clfcs[(i + m->ngstcell) * 7 + k]; }
static inline int32_t cltpn(const ora_mesh * m, int64_t i) { return m->cltpn[i + m->ngstcell]; }
/* StaticMesh::fcrcl (StaticMesh.hpp:355-358). */
static inline int32_t fcrcl(const ora_mesh * m, int32_t ifc, int32_t icl) { return fccls(m, ifc, 0) + fccls(m, ifc, 1) - icl; }

#define NDIMX(e) ((e)->m.ndim)
#define NEQX(e) ((e)->m.ndim + 2)
#define ROW(e, i) ((int64_t)(i) + (e)->m.ngstcell)
#define SO0(a, e, i, k) (a)[ROW(e, i) * NEQX(e) + (k)]
#define SO1(a, e, i, k, d) (a)[(ROW(e, i) * NEQX(e) + (k)) * NDIMX(e) + (d)]
#define CEVOL(e, i, k) (e)->cevol[ROW(e, i) * 7 + (k)]
#define CECND(e, i, k) (e)->cecnd[ROW(e, i) * 7 * NDIMX(e) + (k)]
#define SFCND(e, i, s, d) (e)->sfcnd[((int64_t)(i) * 24 + (s)) * NDIMX(e) + (d)]
#define SFNML(e, i, s, d) (e)->sfnml[((int64_t)(i) * 24 + (s)) * NDIMX(e) + (d)]

/* ---- prepare_ce (euler_ce.cpp:78-347) ----------------------------------- */

static void prepare_ce_2d(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    for (int64_t icl = 0; icl < m->ncell; ++icl)
    {
        int32_t const clnfc = clfcs(m, icl, 0);
        double volc = 0.0, cecnd0 = 0.0, cecnd1 = 0.0;
        double const crdi0 = clcnd(m, icl, 0);
        double const crdi1 = clcnd(m, icl, 1);
        for (int ifl = 1; ifl <= clnfc; ++ifl)
        {
            int32_t const ifc = clfcs(m, icl, ifl);
            int32_t const jcl = fcrcl(m, ifc, (int32_t)icl);
            double const crde0 = clcnd(m, jcl, 0);
            double const crde1 = clcnd(m, jcl, 1);
            int32_t const ind0 = fcnds(m, ifc, 1);
            int32_t const ind1 = fcnds(m, ifc, 2);
            double const crd10 = ndcrd(m, ind0, 0);
            double const crd11 = ndcrd(m, ind0, 1);
            double const crd20 = ndcrd(m, ind1, 0);
            double const crd21 = ndcrd(m, ind1, 1);
            double const cndi0 = (crd10 + crd20 + crdi0) / 3.0;
            double const cndi1 = (crd11 + crd21 + crdi1) / 3.0;
            double const voli = fabs((crd10 - crdi0) * (crd21 - crdi1) - (crd11 - crdi1) * (crd20 - crdi0)) / 2.0;
            double const cnde0 = (crd10 + crd20 + crde0) / 3.0;
            double const cnde1 = (crd11 + crd21 + crde1) / 3.0;
            double const vole = fabs((crd10 - crde0) * (crd21 - crde1) - (crd11 - crde1) * (crd20 - crde0)) / 2.0;
            double const volb = voli + vole;
            CEVOL(e, icl, ifl) = volb;
            CECND(e, icl, ifl * 2 + 0) = (cndi0 * voli + cnde0 * vole) / volb;
            CECND(e, icl, ifl * 2 + 1) = (cndi1 * voli + cnde1 * vole) / volb;
            volc += volb;
            cecnd0 += (cndi0 * voli + cnde0 * vole);
            cecnd1 += (cndi1 * voli + cnde1 * vole);
            int const sb = (ifl - 1) * FCMND;
            double const cross = (crd10 - crde0) * (crd21 - crde1) - (crd11 - crde1) * (crd20 - crde0);
            double const sgn = (cross > 0.0) ? 1.0 : -1.0;
            SFCND(e, icl, sb + 0, 0) = (crde0 + crd10) / 2.0;
            SFCND(e, icl, sb + 0, 1) = (crde1 + crd11) / 2.0;
            SFNML(e, icl, sb + 0, 0) = -(crde1 - crd11) * sgn;
            SFNML(e, icl, sb + 0, 1) = (crde0 - crd10) * sgn;
            SFCND(e, icl, sb + 1, 0) = (crd20 + crde0) / 2.0;
            SFCND(e, icl, sb + 1, 1) = (crd21 + crde1) / 2.0;
            SFNML(e, icl, sb + 1, 0) = -(crd21 - crde1) * sgn;
            SFNML(e, icl, sb + 1, 1) = (crd20 - crde0) * sgn;
        }
        CEVOL(e, icl, 0) = volc;
        CECND(e, icl, 0) = cecnd0 / volc;
        CECND(e, icl, 1) = cecnd1 / volc;
    }
}

static void prepare_ce_3d(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    for (int64_t icl = 0; icl < m->ncell; ++icl)
    {
        int32_t const clnfc = clfcs(m, icl, 0);
        double volc = 0.0, cecnd0 = 0.0, cecnd1 = 0.0, cecnd2 = 0.0;
        double const crdi0 = clcnd(m, icl, 0), crdi1 = clcnd(m, icl, 1), crdi2 = clcnd(m, icl, 2);
        for (int ifl = 1; ifl <= clnfc; ++ifl)
        {
            int32_t const ifc = clfcs(m, icl, ifl);
            int32_t const jcl = fcrcl(m, ifc, (int32_t)icl);
            int32_t const fcnnd = fcnds(m, ifc, 0);
            double const crde0 = clcnd(m, jcl, 0), crde1 = clcnd(m, jcl, 1), crde2 = clcnd(m, jcl, 2);
            double const p0 = fccnd(m, ifc, 0), p1 = fccnd(m, ifc, 1), p2 = fccnd(m, ifc, 2);
            double crd[FCMND + 2][3];
            memset(crd, 0, sizeof(crd));
            for (int inf = 1; inf <= fcnnd; ++inf)
            {
                int32_t const ind = fcnds(m, ifc, inf);
                crd[inf][0] = ndcrd(m, ind, 0);
                crd[inf][1] = ndcrd(m, ind, 1);
                crd[inf][2] = ndcrd(m, ind, 2);
            }
            crd[fcnnd + 1][0] = crd[1][0];
            crd[fcnnd + 1][1] = crd[1][1];
            crd[fcnnd + 1][2] = crd[1][2];
            double volb = 0.0, b0 = 0.0, b1 = 0.0, b2 = 0.0;
            double const voe = (fccls(m, ifc, 0) == icl) ? 0.5 : -0.5;
            int const sb = (ifl - 1) * FCMND;
            for (int inf = 1; inf <= fcnnd; ++inf)
            {
                double const u0 = crd[inf][0] - p0, u1 = crd[inf][1] - p1, u2 = crd[inf][2] - p2;
                double const v0 = crd[inf + 1][0] - p0, v1 = crd[inf + 1][1] - p1, v2 = crd[inf + 1][2] - p2;
                double const t0 = u1 * v2 - u2 * v1;
                double const t1 = u2 * v0 - u0 * v2;
                double const t2 = u0 * v1 - u1 * v0;
                double const voli = fabs(t0 * (crdi0 - p0) + t1 * (crdi1 - p1) + t2 * (crdi2 - p2)) / 6.0;
                double const cndi0 = (crd[inf][0] + crd[inf + 1][0] + p0 + crdi0) / 4.0;
                double const cndi1 = (crd[inf][1] + crd[inf + 1][1] + p1 + crdi1) / 4.0;
                double const cndi2 = (crd[inf][2] + crd[inf + 1][2] + p2 + crdi2) / 4.0;
                double const vole = fabs(t0 * (crde0 - p0) + t1 * (crde1 - p1) + t2 * (crde2 - p2)) / 6.0;
                double const cnde0 = (crd[inf][0] + crd[inf + 1][0] + p0 + crde0) / 4.0;
                double const cnde1 = (crd[inf][1] + crd[inf + 1][1] + p1 + crde1) / 4.0;
                double const cnde2 = (crd[inf][2] + crd[inf + 1][2] + p2 + crde2) / 4.0;
                volb += voli + vole;
                b0 += cndi0 * voli + cnde0 * vole;
                b1 += cndi1 * voli + cnde1 * vole;
                b2 += cndi2 * voli + cnde2 * vole;
                int const si = sb + (inf - 1);
                SFCND(e, icl, si, 0) = (crde0 + crd[inf][0] + crd[inf + 1][0]) / 3.0;
                SFCND(e, icl, si, 1) = (crde1 + crd[inf][1] + crd[inf + 1][1]) / 3.0;
                SFCND(e, icl, si, 2) = (crde2 + crd[inf][2] + crd[inf + 1][2]) / 3.0;
                double const a0 = crd[inf][0] - crde0, a1 = crd[inf][1] - crde1, a2 = crd[inf][2] - crde2;
                double const c0 = crd[inf + 1][0] - crde0, c1 = crd[inf + 1][1] - crde1, c2 = crd[inf + 1][2] - crde2;
                SFNML(e, icl, si, 0) = (a1 * c2 - a2 * c1) * voe;
                SFNML(e, icl, si, 1) = (a2 * c0 - a0 * c2) * voe;
                SFNML(e, icl, si, 2) = (a0 * c1 - a1 * c0) * voe;
            }
            CEVOL(e, icl, ifl) = volb;
            CECND(e, icl, ifl * 3 + 0) = b0 / volb;
            CECND(e, icl, ifl * 3 + 1) = b1 / volb;
            CECND(e, icl, ifl * 3 + 2) = b2 / volb;
            volc += volb;
            cecnd0 += b0;
            cecnd1 += b1;
            cecnd2 += b2;
        }
        CEVOL(e, icl, 0) = volc;
        CECND(e, icl, 0) = cecnd0 / volc;
        CECND(e, icl, 1) = cecnd1 / volc;
        CECND(e, icl, 2) = cecnd2 / volc;
    }
}

void ora_prepare_ce(ora_euler * e)
{
    if (e->m.ndim == 2)
        prepare_ce_2d(e);
    else
        prepare_ce_3d(e);
}

/* ---- flux Jacobian (euler_march.cpp:26-158) ----------------------------- */

typedef struct
{
    double jac[5][5][3]; /* [ieq][jeq][idm] */
    double fcn[5][3];    /* [ieq][idm] */
} jaco_t;

static void jaco_update(jaco_t * J, int nd, double gamma, const double * sol)
{
    double const TINY = 1.e-60;
    double const ga = gamma;
    double const ga1 = ga - 1;
    double const ga3 = ga - 3;
    double const ga1h = ga1 / 2;
    memset(J, 0, sizeof(*J));
    if (nd == 2)
    {
        double const u1 = sol[0] + TINY, u2 = sol[1], u3 = sol[2], u4 = sol[3];
        double const rho2 = u1 * u1;
        double const v1 = u2 / u1;
        double const v1o2 = v1 * v1;
        double const v2 = u3 / u1;
        double const v2o2 = v2 * v2;
        double const ke2 = (u2 * u2 + u3 * u3) / u1;
        double const g1ke2 = ga1 * ke2;
        double const vs = ke2 / u1;
        double const gretot = ga * u4;
        double const getot = gretot / u1;
        double const pr = ga1 * u4 - ga1h * ke2;
        J->fcn[0][0] = u2; J->fcn[0][1] = u3;
        J->fcn[1][0] = pr + u2 * v1; J->fcn[1][1] = u2 * v2;
        J->fcn[2][0] = u3 * v1; J->fcn[2][1] = pr + u3 * v2;
        J->fcn[3][0] = (pr + u4) * v1; J->fcn[3][1] = (pr + u4) * v2;
        J->jac[0][1][0] = 1; J->jac[0][2][1] = 1;
        J->jac[1][0][0] = -v1o2 + ga1h * vs; J->jac[1][0][1] = -v1 * v2;
        J->jac[1][1][0] = -ga3 * v1; J->jac[1][1][1] = v2;
        J->jac[1][2][0] = -ga1 * v2; J->jac[1][2][1] = v1;
        J->jac[1][3][0] = ga1; J->jac[1][3][1] = 0;
        J->jac[2][0][0] = -v2 * v1; J->jac[2][0][1] = -v2o2 + ga1h * vs;
        J->jac[2][1][0] = v2; J->jac[2][1][1] = -ga1 * v1;
        J->jac[2][2][0] = v1; J->jac[2][2][1] = -ga3 * v2;
        J->jac[2][3][0] = 0; J->jac[2][3][1] = ga1;
        J->jac[3][0][0] = (-gretot + g1ke2) * u2 / rho2; J->jac[3][0][1] = (-gretot + g1ke2) * u3 / rho2;
        J->jac[3][1][0] = getot - ga1h * (vs + 2 * v1o2); J->jac[3][1][1] = -ga1 * v1 * v2;
        J->jac[3][2][0] = -ga1 * v2 * v1; J->jac[3][2][1] = getot - ga1h * (vs + 2 * v2o2);
        J->jac[3][3][0] = ga * v1; J->jac[3][3][1] = ga * v2;
    }
    else
    {
        double const u1 = sol[0] + TINY, u2 = sol[1], u3 = sol[2], u4 = sol[3], u5 = sol[4];
        double const rho2 = u1 * u1;
        double const v1 = u2 / u1;
        double const v1o2 = v1 * v1;
        double const v2 = u3 / u1;
        double const v2o2 = v2 * v2;
        double const v3 = u4 / u1;
        double const v3o2 = v3 * v3;
        double const ke2 = (u2 * u2 + u3 * u3 + u4 * u4) / u1;
        double const g1ke2 = ga1 * ke2;
        double const vs = ke2 / u1;
        double const gretot = ga * u5;
        double const getot = gretot / u1;
        double const pr = ga1 * u5 - ga1h * ke2;
        double f[5][3] = {{u2, u3, u4},
                          {pr + u2 * v1, u2 * v2, u2 * v3},
                          {u3 * v1, pr + u3 * v2, u3 * v3},
                          {u4 * v1, u4 * v2, pr + u4 * v3},
                          {(pr + u5) * v1, (pr + u5) * v2, (pr + u5) * v3}};
        double j[5][5][3] = {
            {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 0}},
            {{-v1o2 + ga1h * vs, -v1 * v2, -v1 * v3}, {-ga3 * v1, v2, v3}, {-ga1 * v2, v1, 0}, {-ga1 * v3, 0, v1},
             {ga1, 0, 0}},
            {{-v2 * v1, -v2o2 + ga1h * vs, -v2 * v3}, {v2, -ga1 * v1, 0}, {v1, -ga3 * v2, v3}, {0, -ga1 * v3, v2},
             {0, ga1, 0}},
            {{-v3 * v1, -v3 * v2, -v3o2 + ga1h * vs}, {v3, 0, -ga1 * v1}, {0, v3, -ga1 * v2}, {v1, v2, -ga3 * v3},
             {0, 0, ga1}},
            {{(-gretot + g1ke2) * u2 / rho2, (-gretot + g1ke2) * u3 / rho2, (-gretot + g1ke2) * u4 / rho2},
             {getot - ga1h * (vs + 2 * v1o2), -ga1 * v1 * v2, -ga1 * v1 * v3},
             {-ga1 * v2 * v1, getot - ga1h * (vs + 2 * v2o2), -ga1 * v2 * v3},
             {-ga1 * v3 * v1, -ga1 * v3 * v2, getot - ga1h * (vs + 2 * v3o2)},
             {ga * v1, ga * v2, ga * v3}}};
        memcpy(J->fcn, f, sizeof(f));
        memcpy(J->jac, j, sizeof(j));
    }
}

/* calc_solt_impl (euler_march.cpp:160-191). */
void ora_calc_solt(ora_euler * e)
{
    int const nd = NDIMX(e), neq = NEQX(e);
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int64_t icl = -e->m.ngstcell; icl < e->m.ncell; ++icl)
    {
        jaco_t J;
        double sol[5];
        for (int k = 0; k < neq; ++k)
            sol[k] = SO0(e->so0c, e, icl, k);
        jaco_update(&J, nd, e->gamma[ROW(e, icl)], sol);
        for (int i = 0; i < neq; ++i)
        {
            double val = 0.0;
            for (int d = 0; d < nd; ++d)
                for (int j = 0; j < neq; ++j)
                    val += J.jac[i][j][d] * SO1(e->so1c, e, icl, j, d);
            SO0(e->so0t, e, icl, i) = -val;
        }
    }
}

/* calc_soln_impl (euler_march.cpp:193-303). */
void ora_calc_soln(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e), neq = NEQX(e);
    double const dt = e->dt;
    double const qdt = dt * 0.25;
    double const hdt = dt * 0.5;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int64_t icl = 0; icl < m->ncell; ++icl)
    {
        jaco_t J;
        int32_t const clnfc = clfcs(m, icl, 0);
        double acc[5] = {0, 0, 0, 0, 0};
        for (int ifl = 1; ifl <= clnfc; ++ifl)
        {
            int32_t const ifc = clfcs(m, icl, ifl);
            int32_t const jcl = fcrcl(m, ifc, (int32_t)icl);
            double jce[3], bcnd[3];
            for (int d = 0; d < nd; ++d)
            {
                jce[d] = (jcl >= 0) ? CECND(e, jcl, d) : clcnd(m, jcl, d);
                bcnd[d] = CECND(e, icl, ifl * nd + d);
            }
            double const bvol = CEVOL(e, icl, ifl);
            for (int i = 0; i < neq; ++i)
            {
                double fusp = SO0(e->so0c, e, jcl, i);
                for (int d = 0; d < nd; ++d)
                    fusp += (bcnd[d] - jce[d]) * SO1(e->so1c, e, jcl, i, d);
                acc[i] += fusp * bvol;
            }
            double jsol[5];
            for (int i = 0; i < neq; ++i)
                jsol[i] = SO0(e->so0c, e, jcl, i);
            jaco_update(&J, nd, e->gamma[ROW(e, jcl)], jsol);
            int32_t const fcnnd = fcnds(m, ifc, 0);
            int const sb = (ifl - 1) * FCMND;
            for (int inf = 0; inf < fcnnd; ++inf)
            {
                int const sfi = sb + inf;
                double usfc[5];
                for (int i = 0; i < neq; ++i)
                {
                    usfc[i] = qdt * SO0(e->so0t, e, jcl, i);
                    for (int d = 0; d < nd; ++d)
                        usfc[i] += (SFCND(e, icl, sfi, d) - jce[d]) * SO1(e->so1c, e, jcl, i, d);
                }
                for (int i = 0; i < neq; ++i)
                {
                    double dot = 0.0;
                    for (int d2 = 0; d2 < nd; ++d2)
                    {
                        double dfcn = J.fcn[i][d2];
                        for (int j = 0; j < neq; ++j)
                            dfcn += J.jac[i][j][d2] * usfc[j];
                        dot += dfcn * SFNML(e, icl, sfi, d2);
                    }
                    acc[i] -= hdt * dot;
                }
            }
        }
        double const cvol = CEVOL(e, icl, 0);
        for (int i = 0; i < neq; ++i)
            SO0(e->so0n, e, icl, i) = acc[i] / cvol;
    }
}

/* ---- boundary conditions (euler_bc.cpp:31-320) -------------------------- */

static void normal_matrix(int nd, const double * n, double mat[3][3])
{
    memset(mat, 0, sizeof(double) * 9);
    if (nd == 2)
    {
        mat[0][0] = n[0]; mat[0][1] = n[1];
        mat[1][0] = -n[1]; mat[1][1] = n[0];
        return;
    }
    double axis[3] = {0.0, 0.0, 0.0};
    double const ax = fabs(n[0]), ay = fabs(n[1]), az = fabs(n[2]);
    if (ax <= ay && ax <= az)
        axis[0] = 1.0;
    else if (ay <= az)
        axis[1] = 1.0;
    else
        axis[2] = 1.0;
    double t1[3] = {n[1] * axis[2] - n[2] * axis[1], n[2] * axis[0] - n[0] * axis[2], n[0] * axis[1] - n[1] * axis[0]};
    double const len = sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    t1[0] /= len; t1[1] /= len; t1[2] /= len;
    double const t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    for (int d = 0; d < 3; ++d)
    {
        mat[0][d] = n[d];
        mat[1][d] = t1[d];
        mat[2][d] = t2[d];
    }
}

static void matvec(int nd, double m[3][3], const double * v, double * r)
{
    for (int i = 0; i < nd; ++i)
    {
        r[i] = 0.0;
        for (int j = 0; j < nd; ++j)
            r[i] += m[i][j] * v[j];
    }
}

static void transpose(int nd, double m[3][3], double t[3][3])
{
    memset(t, 0, sizeof(double) * 9);
    for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
            t[i][j] = m[j][i];
}

static void matmat(int nd, double a[3][3], double b[3][3], double r[3][3])
{
    memset(r, 0, sizeof(double) * 9);
    for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
            for (int k = 0; k < nd; ++k)
                r[i][j] += a[i][k] * b[k][j];
}

void ora_bc_soln(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e), neq = NEQX(e);
    for (int32_t ib = 0; ib < e->nbnd; ++ib)
    {
        const double * val = e->bval + (int64_t)ib * (nd + 3);
        for (int64_t k = e->boff[ib]; k < e->boff[ib + 1]; ++k)
        {
            int32_t const ifc = e->bfaces[k];
            int32_t const icl = fccls(m, ifc, 0);
            int32_t const jcl = fccls(m, ifc, 1);
            if (e->bkind[ib] == 0)
            {
                for (int i = 0; i < neq; ++i)
                    SO0(e->so0n, e, jcl, i) = SO0(e->so0n, e, icl, i);
            }
            else if (e->bkind[ib] == 1)
            {
                double n[3], mat[3][3], inv[3][3], mom[3], rot[3], out[3];
                for (int d = 0; d < nd; ++d)
                    n[d] = fcnml(m, ifc, d);
                normal_matrix(nd, n, mat);
                transpose(nd, mat, inv);
                SO0(e->so0n, e, jcl, 0) = SO0(e->so0n, e, icl, 0);
                SO0(e->so0n, e, jcl, neq - 1) = SO0(e->so0n, e, icl, neq - 1);
                for (int d = 0; d < nd; ++d)
                    mom[d] = SO0(e->so0n, e, icl, 1 + d);
                matvec(nd, mat, mom, rot);
                rot[0] = -rot[0];
                matvec(nd, inv, rot, out);
                for (int d = 0; d < nd; ++d)
                    SO0(e->so0n, e, jcl, 1 + d) = out[d];
            }
            else
            {
                double const rho = val[0], p = val[1 + nd], ga = val[2 + nd];
                double vsq = 0.0;
                for (int d = 0; d < nd; ++d)
                    vsq += val[1 + d] * val[1 + d];
                SO0(e->so0n, e, jcl, 0) = rho;
                for (int d = 0; d < nd; ++d)
                    SO0(e->so0n, e, jcl, 1 + d) = rho * val[1 + d];
                SO0(e->so0n, e, jcl, neq - 1) = p / (ga - 1.0) + 0.5 * rho * vsq;
            }
        }
    }
}

void ora_bc_dsoln(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e), neq = NEQX(e);
    for (int32_t ib = 0; ib < e->nbnd; ++ib)
    {
        for (int64_t k = e->boff[ib]; k < e->boff[ib + 1]; ++k)
        {
            int32_t const ifc = e->bfaces[k];
            int32_t const icl = fccls(m, ifc, 0);
            int32_t const jcl = fccls(m, ifc, 1);
            if (e->bkind[ib] == 2)
            {
                for (int i = 0; i < neq; ++i)
                    for (int d = 0; d < nd; ++d)
                        SO1(e->so1n, e, jcl, i, d) = 0.0;
                continue;
            }
            double n[3], mat[3][3], inv[3][3];
            for (int d = 0; d < nd; ++d)
                n[d] = fcnml(m, ifc, d);
            normal_matrix(nd, n, mat);
            transpose(nd, mat, inv);
            if (e->bkind[ib] == 0)
            {
                for (int i = 0; i < neq; ++i)
                {
                    double g[3], rot[3], out[3];
                    for (int d = 0; d < nd; ++d)
                        g[d] = SO1(e->so1c, e, icl, i, d);
                    matvec(nd, mat, g, rot);
                    rot[0] = 0.0;
                    matvec(nd, inv, rot, out);
                    for (int d = 0; d < nd; ++d)
                        SO1(e->so1n, e, jcl, i, d) = out[d];
                }
                continue;
            }
            int const scal[2] = {0, neq - 1};
            for (int s = 0; s < 2; ++s)
            {
                int const i = scal[s];
                double g[3], rot[3], out[3];
                for (int d = 0; d < nd; ++d)
                    g[d] = SO1(e->so1c, e, icl, i, d);
                matvec(nd, mat, g, rot);
                rot[0] = -rot[0];
                matvec(nd, inv, rot, out);
                for (int d = 0; d < nd; ++d)
                    SO1(e->so1n, e, jcl, i, d) = out[d];
            }
            double mg[3][3], t[3][3], uv[3][3], out[3][3];
            memset(mg, 0, sizeof(mg));
            for (int a = 0; a < nd; ++a)
                for (int b = 0; b < nd; ++b)
                    mg[a][b] = SO1(e->so1c, e, icl, 1 + a, b);
            matmat(nd, mat, mg, t);
            matmat(nd, t, inv, uv);
            for (int it = 1; it < nd; ++it)
            {
                uv[0][it] = -uv[0][it];
                uv[it][0] = -uv[it][0];
            }
            matmat(nd, inv, uv, t);
            matmat(nd, t, mat, out);
            for (int a = 0; a < nd; ++a)
                for (int b = 0; b < nd; ++b)
                    SO1(e->so1n, e, jcl, 1 + a, b) = out[a][b];
        }
    }
}

/* ---- calc_cfl (euler_solution.cpp:106-160) ------------------------------ */

void ora_calc_cfl(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e), neq = NEQX(e);
    double const TINY = 1.e-60;
    double const hdt = e->dt / 2.0;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int64_t icl = 0; icl < m->ncell; ++icl)
    {
        int32_t const clnfc = clfcs(m, icl, 0);
        double dist = DBL_MAX;
        for (int ifl = 1; ifl <= clnfc; ++ifl)
        {
            double d2 = 0.0;
            for (int d = 0; d < nd; ++d)
            {
                double const diff = CECND(e, icl, ifl * nd + d) - CECND(e, icl, d);
                d2 += diff * diff;
            }
            double const s = sqrt(d2);
            dist = (s < dist) ? s : dist;
        }
        double const ga = e->gamma[ROW(e, icl)];
        double const ga1 = ga - 1.0;
        double const density = SO0(e->so0n, e, icl, 0);
        double momsq = 0.0;
        for (int d = 0; d < nd; ++d)
        {
            double const mom = SO0(e->so0n, e, icl, 1 + d);
            momsq += mom * mom;
        }
        double const ke = momsq / (2.0 * density);
        double const energy = SO0(e->so0n, e, icl, neq - 1);
        double const pr = ga1 * (energy - ke);
        double const pr_adj = (pr + fabs(pr)) / 2.0;
        double const wspd = sqrt(ga * pr_adj / density) + sqrt(momsq) / density;
        double const cflo = hdt * wspd / dist;
        e->cflo[ROW(e, icl)] = cflo;
        e->cflc[ROW(e, icl)] = (cflo - 1.0) * pr_adj / (pr_adj + TINY) + 1.0;
        SO0(e->so0n, e, icl, neq - 1) = pr_adj / ga1 + ke + TINY;
    }
}

/* ---- GradientElement (GradientElement.cpp:16-290) ----------------------- */

typedef struct
{
    int nfge;
    double nfge_inverse;
    int faces[8][3]; /* 1-based */
} getype_t;

static getype_t getype(int32_t type)
{
    getype_t g;
    memset(&g, 0, sizeof(g));
    static const int quad[4][3] = {{1, 2, -1}, {2, 3, -1}, {3, 4, -1}, {4, 1, -1}};
    static const int tri[3][3] = {{1, 2, -1}, {2, 3, -1}, {3, 1, -1}};
    static const int hex[8][3] = {{2, 3, 5}, {6, 3, 2}, {4, 3, 6}, {5, 3, 4}, {5, 1, 2}, {2, 1, 6}, {6, 1, 4}, {4, 1, 5}};
    static const int tet[4][3] = {{3, 1, 2}, {2, 1, 4}, {4, 1, 3}, {2, 4, 3}};
    static const int pri[6][3] = {{5, 2, 4}, {3, 2, 5}, {4, 2, 3}, {4, 1, 5}, {5, 1, 3}, {3, 1, 4}};
    static const int pyr[6][3] = {{1, 5, 2}, {2, 5, 3}, {3, 5, 4}, {4, 5, 1}, {1, 3, 4}, {3, 1, 2}};
    const int(*t)[3] = NULL;
    switch (type)
    {
    case 3: g.nfge = 4; t = quad; break;
    case 4: g.nfge = 3; t = tri; break;
    case 5: g.nfge = 8; t = hex; break;
    case 6: g.nfge = 4; t = tet; break;
    case 7: g.nfge = 6; t = pri; break;
    case 8: g.nfge = 6; t = pyr; break;
    default: return g;
    }
    g.nfge_inverse = 1.0 / g.nfge;
    memcpy(g.faces, t, sizeof(int) * 3 * (size_t)g.nfge);
    return g;
}

typedef struct
{
    int clnfc;
    getype_t ge;
    int32_t rcl[CLMFC];
    double idis[CLMFC][3];
    double jdis[CLMFC][3];
} gelem_t;

static void gelem_build(const ora_euler * e, int64_t icl, double tau, gelem_t * g)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e);
    memset(g, 0, sizeof(*g));
    g->clnfc = clfcs(m, icl, 0);
    g->ge = getype(cltpn(m, icl));
    double icecnd[3] = {0, 0, 0};
    for (int d = 0; d < nd; ++d)
        icecnd[d] = CECND(e, icl, d);
    double gp[CLMFC][3], jd[CLMFC][3];
    memset(gp, 0, sizeof(gp));
    memset(jd, 0, sizeof(jd));
    for (int ifl = 0; ifl < g->clnfc; ++ifl)
    {
        int32_t const ifc = clfcs(m, icl, ifl + 1);
        int32_t const jcl = fcrcl(m, ifc, (int32_t)icl);
        g->rcl[ifl] = jcl;
        for (int d = 0; d < nd; ++d)
        {
            double const mid = CECND(e, icl, (ifl + 1) * nd + d);
            double const jce = (jcl >= 0) ? CECND(e, jcl, d) : clcnd(m, jcl, d);
            gp[ifl][d] = mid + tau * (jce - mid);
            jd[ifl][d] = gp[ifl][d] - jce;
        }
    }
    double avg[3] = {0, 0, 0};
    for (int ifl = 0; ifl < g->clnfc; ++ifl)
        for (int d = 0; d < nd; ++d)
            avg[d] += gp[ifl][d];
    for (int d = 0; d < nd; ++d)
        avg[d] /= g->clnfc;
    /* calc_gge_centroid (GradientElement.cpp:81-133). */
    double cnd[3] = {0, 0, 0};
    double voc = 0.0;
    for (int isub = 0; isub < g->ge.nfge; ++isub)
    {
        double subcnd[3] = {avg[0], avg[1], avg[2]};
        double dst[3][3];
        memset(dst, 0, sizeof(dst));
        for (int ivx = 0; ivx < nd; ++ivx)
        {
            int const fl = g->ge.faces[isub][ivx] - 1;
            for (int d = 0; d < nd; ++d)
            {
                subcnd[d] += gp[fl][d];
                dst[ivx][d] = gp[fl][d] - avg[d];
            }
        }
        for (int d = 0; d < nd; ++d)
            subcnd[d] /= (double)(nd + 1);
        double vob;
        if (nd == 2)
            vob = dst[0][0] * dst[1][1] - dst[0][1] * dst[1][0];
        else
            vob = dst[0][0] * (dst[1][1] * dst[2][2] - dst[1][2] * dst[2][1]) -
                  dst[0][1] * (dst[1][0] * dst[2][2] - dst[1][2] * dst[2][0]) +
                  dst[0][2] * (dst[1][0] * dst[2][1] - dst[1][1] * dst[2][0]);
        voc += vob;
        for (int d = 0; d < nd; ++d)
            cnd[d] += subcnd[d] * vob;
    }
    for (int d = 0; d < nd; ++d)
        cnd[d] /= voc;
    for (int ifl = 0; ifl < g->clnfc; ++ifl)
        for (int d = 0; d < nd; ++d)
        {
            g->idis[ifl][d] = gp[ifl][d] - cnd[d];
            g->jdis[ifl][d] = jd[ifl][d] + icecnd[d] - cnd[d];
        }
}

static void gelem_solve(const gelem_t * g, int nd, int ifge, const double * udf, double * grad)
{
    double a[3][3];
    memset(a, 0, sizeof(a));
    for (int ivx = 0; ivx < nd; ++ivx)
    {
        int const ifl = g->ge.faces[ifge][ivx] - 1;
        for (int d = 0; d < nd; ++d)
            a[ivx][d] = g->idis[ifl][d];
    }
    double r[3][3];
    memset(r, 0, sizeof(r));
    double det;
    if (nd == 2)
    {
        r[0][0] = a[1][1];
        r[0][1] = -a[0][1];
        r[1][0] = -a[1][0];
        r[1][1] = a[0][0];
        det = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    }
    else
    {
        r[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
        r[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
        r[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
        r[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
        r[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
        r[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
        r[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
        r[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
        r[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
        det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
              a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    }
    double adj[3] = {0, 0, 0};
    for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j)
            adj[i] += r[i][j] * udf[j];
    for (int d = 0; d < nd; ++d)
        grad[d] = adj[d] / det;
}

/* ---- calc_dsoln (euler_gradient.cpp:23-130) ----------------------------- */

void ora_calc_dsoln(ora_euler * e)
{
    const ora_mesh * m = &e->m;
    int const nd = NDIMX(e), neq = NEQX(e);
    double const ALMOST_ZERO = 1.e-200;
    double const hdt = e->dt * 0.5;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
    for (int64_t icl = 0; icl < m->ncell; ++icl)
    {
        double const acfl = fabs(e->cflc[ROW(e, icl)]);
        double const sgm0 = e->sigma0 / acfl;
        double const tau = e->taumin + acfl * e->tauscale;
        gelem_t g;
        gelem_build(e, icl, tau, &g);
        int const nfge = g.ge.nfge;
        double const ofg1 = g.ge.nfge_inverse;
        double grad[8][5][3], widv[8][5], wacc[5] = {0, 0, 0, 0, 0}, sigma_max[5];
        memset(grad, 0, sizeof(grad));
        memset(widv, 0, sizeof(widv));
        for (int ifge = 0; ifge < nfge; ++ifge)
        {
            double udf[5][3];
            memset(udf, 0, sizeof(udf));
            for (int ivx = 0; ivx < nd; ++ivx)
            {
                int const ifl = g.ge.faces[ifge][ivx] - 1;
                int32_t const jcl = g.rcl[ifl];
                for (int i = 0; i < neq; ++i)
                {
                    double val = SO0(e->so0c, e, jcl, i) + hdt * SO0(e->so0t, e, jcl, i) - SO0(e->so0n, e, icl, i);
                    for (int d = 0; d < nd; ++d)
                        val += g.jdis[ifl][d] * SO1(e->so1c, e, jcl, i, d);
                    udf[i][ivx] = val;
                }
            }
            for (int i = 0; i < neq; ++i)
            {
                gelem_solve(&g, nd, ifge, udf[i], grad[ifge][i]);
                double sq = 0.0;
                for (int d = 0; d < nd; ++d)
                    sq += grad[ifge][i][d] * grad[ifge][i][d];
                double const wgt = 1.0 / sqrt(sq + ALMOST_ZERO);
                wacc[i] += wgt;
                widv[ifge][i] = wgt;
            }
        }
        double wpa[5][2];
        memset(wpa, 0, sizeof(wpa));
        for (int ifge = 0; ifge < nfge; ++ifge)
            for (int i = 0; i < neq; ++i)
            {
                double const wgt = widv[ifge][i] / wacc[i] - ofg1;
                widv[ifge][i] = wgt;
                wpa[i][0] = fmax(wpa[i][0], wgt);
                wpa[i][1] = fmin(wpa[i][1], wgt);
            }
        uint8_t fired = 0;
        for (int i = 0; i < neq; ++i)
        {
            double const sm = fmin((1.0 - ofg1) / (wpa[i][0] + ALMOST_ZERO), -ofg1 / (wpa[i][1] - ALMOST_ZERO));
            sigma_max[i] = fmin(sm, sgm0);
            if (sm < sgm0)
                fired |= (uint8_t)(1u << i);
        }
        if (e->limiter)
            e->limiter[icl] = fired;
        for (int i = 0; i < neq; ++i)
            for (int d = 0; d < nd; ++d)
                SO1(e->so1n, e, icl, i, d) = 0.0;
        for (int isub = 0; isub < nfge; ++isub)
            for (int i = 0; i < neq; ++i)
            {
                double const wgt = ofg1 + sigma_max[i] * widv[isub][i];
                for (int d = 0; d < nd; ++d)
                    SO1(e->so1n, e, icl, i, d) += wgt * grad[isub][i][d];
            }
    }
}

/* ---- march (euler.hpp:123-127, euler_march.cpp:339-359) ----------------- */

void ora_update(ora_euler * e)
{
    double * t = e->so0c;
    e->so0c = e->so0n;
    e->so0n = t;
    t = e->so1c;
    e->so1c = e->so1n;
    e->so1n = t;
}

void ora_march_substep(ora_euler * e)
{
    ora_update(e);
    ora_calc_solt(e);
    ora_calc_soln(e);
    ora_bc_soln(e);
    ora_calc_cfl(e);
    ora_calc_dsoln(e);
    ora_bc_dsoln(e);
}

void ora_march(ora_euler * e, int64_t steps)
{
    for (int64_t s = 0; s < steps; ++s)
    {
        ora_march_substep(e);
        ora_march_substep(e);
    }
}

/* ---- 1D Euler (onedim/Euler1DCore.cpp, Euler1DCore.hpp) ----------------- */

typedef struct
{
    double qdt, hdt, ga, x, xctr, xneg, xpos;
    double u[3], ux[3], jac[3][3], f[3], ut[3], ft[3], up[3];
} k1d_t;

/* Euler1DKernel::set_value and derive (Euler1DCore.hpp:193-244). */
static void k1d_set(k1d_t * k, const ora_e1d * e, int64_t ic)
{
    double const tiny = 1.e-100;
    k->hdt = e->dt / 2.0;
    k->qdt = k->hdt / 2.0;
    k->ga = e->gamma[ic];
    k->x = e->coord[ic];
    k->xneg = e->coord[ic - 1];
    k->xpos = e->coord[ic + 1];
    k->xctr = (k->xpos + k->xneg) * 0.5;
    for (int i = 0; i < 3; ++i)
    {
        k->u[i] = e->so0[ic * 3 + i];
        k->ux[i] = e->so1[ic * 3 + i];
    }
    double const ga = k->ga;
    double const * u = k->u;
    k->jac[0][0] = 0.0;
    k->jac[0][1] = 1.0;
    k->jac[0][2] = 0.0;
    k->jac[1][0] = (ga - 3.0) / 2.0 * u[1] * u[1] / (u[0] * u[0] + tiny);
    k->jac[1][1] = -(ga - 3.0) * u[1] / (u[0] + tiny);
    k->jac[1][2] = ga - 1.0;
    k->jac[2][0] = (ga - 1.0) * u[1] * u[1] * u[1] / (u[0] * u[0] * u[0] + tiny) - ga * u[1] * u[2] / (u[0] * u[0] + tiny);
    k->jac[2][1] = ga * u[2] / (u[0] + tiny) - 3.0 / 2.0 * (ga - 1.0) * u[1] * u[1] / (u[0] * u[0] + tiny);
    k->jac[2][2] = ga * u[1] / (u[0] + tiny);
    k->f[0] = u[1];
    k->f[1] = (ga - 1.0) * u[2] + (3.0 - ga) / 2.0 * u[1] * u[1] / (u[0] + tiny);
    k->f[2] = ga * u[1] * u[2] / (u[0] + tiny) - (ga - 1.0) / 2.0 * u[1] * u[1] * u[1] / (u[0] * u[0] + tiny);
    for (int i = 0; i < 3; ++i)
        k->ut[i] = -k->jac[i][0] * k->ux[0] - k->jac[i][1] * k->ux[1] - k->jac[i][2] * k->ux[2];
    for (int i = 0; i < 3; ++i)
        k->ft[i] = k->jac[i][0] * k->ut[0] + k->jac[i][1] * k->ut[1] + k->jac[i][2] * k->ut[2];
    for (int i = 0; i < 3; ++i)
        k->up[i] = u[i] + (k->x - k->xctr) * k->ux[i] + k->hdt * k->ut[i];
}

void ora_e1d_update_cfl(ora_e1d * e, int odd_plane)
{
    int64_t const start = 2 - (odd_plane ? 1 : 0);
    int64_t const stop = e->ncoord - 2 - (odd_plane ? 0 : 1);
    double const hdt = e->dt / 2;
    for (int64_t it = start; it < stop; it += 2)
    {
        double const ga = e->gamma[it];
        double wspd = e->so0[it * 3 + 1];
        wspd *= wspd;
        double const ke = wspd / (2.0 * e->so0[it * 3 + 0]);
        double pr = (ga - 1.0) * (e->so0[it * 3 + 2] - ke);
        pr = (pr + fabs(pr)) / 2.0;
        wspd = sqrt(ga * pr / e->so0[it * 3 + 0]) + sqrt(wspd) / e->so0[it * 3 + 0];
        double const dxpos = e->coord[it + 1] - e->coord[it];
        double const dxneg = e->coord[it] - e->coord[it - 1];
        e->cfl[it] = hdt * wspd / (dxpos < dxneg ? dxpos : dxneg);
    }
}

void ora_e1d_march_half_so0(ora_e1d * e, int odd_plane)
{
    int64_t const start = 2 - (odd_plane ? 1 : 0);
    int64_t const stop = e->ncoord - 2 - (odd_plane ? 0 : 1);
    k1d_t kn, kp;
    k1d_set(&kp, e, start);
    for (int64_t ic = start; ic < stop; ic += 2)
    {
        kn = kp;
        k1d_set(&kp, e, ic + 2);
        double ll[3], lr[3];
        /* calc_flux_ll / calc_flux_lr (Euler1DCore.hpp:246-266). */
        {
            double const deltax = kn.xpos - kn.x;
            double const dxmid = 0.5 * (kn.x + kn.xpos) - kn.xctr;
            double const dxctr = kn.x - kn.xctr;
            for (int i = 0; i < 3; ++i)
                ll[i] = deltax * (kn.u[i] + dxmid * kn.ux[i]) +
                        kn.hdt * (kn.f[i] - (dxctr * kn.ut[i]) + (kn.qdt * kn.ft[i]));
        }
        {
            double const deltax = kp.x - kp.xneg;
            double const dxmid = 0.5 * (kp.x + kp.xneg) - kp.xctr;
            double const dxctr = kp.x - kp.xctr;
            for (int i = 0; i < 3; ++i)
                lr[i] = deltax * (kp.u[i] + dxmid * kp.ux[i]) -
                        kp.hdt * (kp.f[i] - (dxctr * kp.ut[i]) + (kp.qdt * kp.ft[i]));
        }
        double const dx = e->coord[ic + 2] - e->coord[ic];
        for (int i = 0; i < 3; ++i)
            e->so0[(ic + 1) * 3 + i] = (ll[i] + lr[i]) / dx;
    }
}

void ora_e1d_march_half_so1(ora_e1d * e, int odd_plane, int alpha)
{
    int64_t const start = 2 - (odd_plane ? 1 : 0);
    int64_t const stop = e->ncoord - 2 - (odd_plane ? 0 : 1);
    double const tiny = 1.e-100;
    k1d_t kn, kp;
    k1d_set(&kp, e, start);
    for (int64_t ic = start; ic < stop; ic += 2)
    {
        kn = kp;
        k1d_set(&kp, e, ic + 2);
        for (int iv = 0; iv < 3; ++iv)
        {
            double const utp = e->so0[(ic + 1) * 3 + iv];
            double const duxn = (utp - kn.up[iv]) / (kn.xpos - kn.x);
            double const duxp = (kp.up[iv] - utp) / (kp.x - kp.xneg);
            double fan = fabs(duxn), fap = fabs(duxp);
            if (alpha == 2)
            {
                fan = fan * fan;
                fap = fap * fap;
            }
            e->so1[(ic + 1) * 3 + iv] = (fap * duxn + fan * duxp) / (fap + fan + tiny);
        }
    }
}

void ora_e1d_treat_boundary_so0(ora_e1d * e)
{
    int64_t const l = 1, r = e->ncoord - 2;
    for (int i = 0; i < 3; ++i)
    {
        e->so0[l * 3 + i] = e->so0[(l + 1) * 3 + i];
        e->so0[r * 3 + i] = e->so0[(r - 1) * 3 + i];
    }
}

void ora_e1d_treat_boundary_so1(ora_e1d * e)
{
    int64_t const l = 1, r = e->ncoord - 2;
    for (int i = 0; i < 3; ++i)
    {
        e->so1[l * 3 + i] = e->so1[(l + 1) * 3 + i];
        e->so1[r * 3 + i] = e->so1[(r - 1) * 3 + i];
    }
}

/* march_alpha (Euler1DCore.hpp:322-349). */
void ora_e1d_march(ora_e1d * e, int alpha, int64_t steps)
{
    for (int64_t it = 0; it < steps; ++it)
    {
        ora_e1d_march_half_so0(e, 0);
        ora_e1d_update_cfl(e, 0);
        ora_e1d_march_half_so1(e, 0, alpha);
        ora_e1d_treat_boundary_so0(e);
        ora_e1d_treat_boundary_so1(e);
        ora_e1d_march_half_so0(e, 1);
        ora_e1d_update_cfl(e, 1);
        ora_e1d_march_half_so1(e, 1, alpha);
    }
}

/* ---- spacetime scalar solvers (spacetime/core.hpp:946-1036) ------------- */

typedef struct
{
    double x, xneg, xpos, u, ux;
} st_selm_t;

static st_selm_t st_selm(const ora_st * s, int64_t ielm, int odd)
{
    int64_t const xi = 2 + 2 * ielm + odd; /* Grid::xindex_selm */
    st_selm_t e = {s->xcoord[xi], s->xcoord[xi - 1], s->xcoord[xi + 1], s->so0[xi], s->so1[xi]};
    return e;
}

static double st_xctr(const st_selm_t * e) { return (e->xneg + e->xpos) / 2; }

/* LinearScalarSelm / InviscidBurgersSelm xn, xp, tp, so0p
 * (kernel/linear_scalar.hpp:45-80, kernel/inviscid_burgers.hpp:51-100). */
static double st_xn(const st_selm_t * e)
{
    double const disp = 0.5 * (e->x + e->xneg) - st_xctr(e);
    return (e->x - e->xneg) * (e->u + disp * e->ux);
}

static double st_xp(const st_selm_t * e)
{
    double const disp = 0.5 * (e->x + e->xpos) - st_xctr(e);
    return (e->xpos - e->x) * (e->u + disp * e->ux);
}

static double st_tp(const ora_st * s, const st_selm_t * e)
{
    double const hdt = s->dt * 0.5, qdt = s->dt * 0.25;
    double const disp = e->x - st_xctr(e);
    double ret;
    if (s->kind == 0)
    {
        ret = e->u;
        ret += disp * e->ux;
        ret -= qdt * e->ux;
    }
    else
    {
        double const u2 = e->u * e->u;
        ret = 0.5 * u2;
        ret += disp * e->u * e->ux;
        ret -= qdt * u2 * e->ux;
    }
    return hdt * ret;
}

static double st_so0p(const ora_st * s, const st_selm_t * e)
{
    double ret = e->u;
    ret += (e->x - st_xctr(e)) * e->ux;
    ret -= s->dt * 0.5 * e->ux;
    return ret;
}

static void st_update_cfl(ora_st * s, int odd)
{
    for (int64_t ic = odd ? -1 : 0; ic < s->ncelm + 1; ++ic)
    {
        st_selm_t const e = st_selm(s, ic, odd);
        double const dn = e.x - e.xneg, dp = e.xpos - e.x;
        double const hdx = dn < dp ? dn : dp;
        int64_t const xi = 2 + 2 * ic + odd;
        s->cfl[xi] = (s->kind == 0) ? (s->dt * 0.5) / hdx : fabs(e.u) * (s->dt * 0.5) / hdx;
    }
}

static void st_half_so0(ora_st * s, int odd)
{
    for (int64_t ic = odd ? -1 : 0; ic < s->ncelm; ++ic)
    {
        st_selm_t const xn = st_selm(s, ic, odd);
        st_selm_t const xp = st_selm(s, ic + 1, odd);
        double const ll = st_xp(&xn) + st_tp(s, &xn);
        double const ur = st_xn(&xp) - st_tp(s, &xp);
        int64_t const xt = 2 + 2 * (ic + odd) + !odd;
        s->so0[xt] = (ll + ur) / (s->xcoord[xt + 1] - s->xcoord[xt - 1]);
    }
}

static void st_half_so1(ora_st * s, int odd, int alpha)
{
    for (int64_t ic = odd ? -1 : 0; ic < s->ncelm; ++ic)
    {
        st_selm_t const xn = st_selm(s, ic, odd);
        st_selm_t const xp = st_selm(s, ic + 1, odd);
        int64_t const xt = 2 + 2 * (ic + odd) + !odd;
        double const utp = s->so0[xt];
        double const duxn = (utp - st_so0p(s, &xn)) / (xn.xpos - xn.x);
        double const duxp = (st_so0p(s, &xp) - utp) / (xp.x - xp.xneg);
        double fan = fabs(duxn), fap = fabs(duxp);
        if (alpha == 2)
        {
            fan *= fan;
            fap *= fap;
        }
        s->so1[xt] = (fap * duxn + fan * duxp) / (fap + fan + DBL_MIN);
    }
}

static void st_boundary(ora_st * s, double * arr)
{
    int64_t const left_out = 1, left_in = 3;
    int64_t const right_in = 2 * s->ncelm + 1, right_out = 2 * s->ncelm + 3;
    arr[left_out] = arr[right_in];
    arr[right_out] = arr[left_in];
}

void ora_st_march(ora_st * s, int alpha, int64_t steps)
{
    for (int64_t it = 0; it < steps; ++it)
    {
        st_half_so0(s, 0);
        st_boundary(s, s->so0);
        st_update_cfl(s, 1);
        st_half_so1(s, 0, alpha);
        st_boundary(s, s->so1);
        st_half_so0(s, 1);
        st_update_cfl(s, 0);
        st_half_so1(s, 1, alpha);
    }
}

void ora_st_setup(ora_st * s) { st_update_cfl(s, 0); }
