/*
 * CPU oracle of the CESE march -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solvcon algorithm for the path the
 * GPU library implements: the multi-dimensional Euler core
 * (cpp/solvcon/multidim/*.cpp), the 1D Euler core
 * (cpp/solvcon/onedim/Euler1DCore.*) and the 1D spacetime scalar solvers
 * (cpp/solvcon/spacetime/core.hpp, kernel/*.hpp).  Each function cites the
 * reference lines it follows and keeps the reference's operation order, so
 * that on the same inputs it reproduces the reference's results to the last
 * bit or close to it.  Only tests/, the smoke check and bench.py's CPU
 * baseline and reference arm use it, to check and to time against; the
 * product never links it.
 *
 * All tables are whole buffers in the reference layout, ghost rows first.
 */

#ifndef CESE_ORACLE_H
#define CESE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int32_t ndim;
    int64_t nnode, nface, ncell;
    int64_t ngstnode, ngstface, ngstcell;
    const double * ndcrd; /* [ngstnode + nnode][ndim] */
    const double * fccnd; /* [ngstface + nface][ndim] */
    const double * fcnml; /* [ngstface + nface][ndim] */
    const double * clcnd; /* [ngstcell + ncell][ndim] */
    const int32_t * fcnds; /* [..][5] */
    const int32_t * fccls; /* [..][4] */
    const int32_t * clfcs; /* [..][7] */
    const int32_t * cltpn; /* [ngstcell + ncell] */
} ora_mesh;

typedef struct
{
    ora_mesh m;
    double dt, sigma0, taumin, tauscale;
    double * cevol; /* [ngstcell + ncell][7] */
    double * cecnd; /* [ngstcell + ncell][7 * ndim] */
    double * sfcnd; /* [ncell][24][ndim] */
    double * sfnml; /* [ncell][24][ndim] */
    double * so0c, * so0n, * so0t, * stm; /* [ngstcell + ncell][neq] */
    double * so1c, * so1n;               /* [ngstcell + ncell][neq][ndim] */
    double * cflo, * cflc, * gamma;      /* [ngstcell + ncell] */
    uint8_t * limiter;                   /* [ncell] or NULL */
    int32_t nbnd;
    const int32_t * bkind;  /* [nbnd] 0 nonrefl, 1 slipwall, 2 inlet */
    const int64_t * boff;   /* [nbnd + 1] offsets into bfaces */
    const int32_t * bfaces; /* boundary face ids */
    const double * bval;    /* [nbnd][ndim + 3] inlet values */
} ora_euler;

void ora_prepare_ce(ora_euler * e);
void ora_calc_solt(ora_euler * e);
void ora_calc_soln(ora_euler * e);
void ora_bc_soln(ora_euler * e);
void ora_calc_cfl(ora_euler * e);
void ora_calc_dsoln(ora_euler * e);
void ora_bc_dsoln(ora_euler * e);
void ora_update(ora_euler * e);
void ora_march_substep(ora_euler * e);
void ora_march(ora_euler * e, int64_t steps);
/* Threads for the per-cell loops of the multidim march (default 1); the
 * results do not depend on it. */
void ora_set_threads(int n);

/* 1D Euler core (onedim/Euler1DCore.*). */
typedef struct
{
    int64_t ncoord;
    double dt;
    double * coord; /* [ncoord] */
    double * cfl;   /* [ncoord] */
    double * so0;   /* [ncoord][3] */
    double * so1;   /* [ncoord][3] */
    double * gamma; /* [ncoord] */
} ora_e1d;

void ora_e1d_update_cfl(ora_e1d * e, int odd_plane);
void ora_e1d_march_half_so0(ora_e1d * e, int odd_plane);
void ora_e1d_march_half_so1(ora_e1d * e, int odd_plane, int alpha);
void ora_e1d_treat_boundary_so0(ora_e1d * e);
void ora_e1d_treat_boundary_so1(ora_e1d * e);
void ora_e1d_march(ora_e1d * e, int alpha, int64_t steps);

/* 1D spacetime scalar solvers (spacetime/core.hpp, kernel/*.hpp). */
typedef struct
{
    int64_t ncelm;       /* number of conservation elements */
    int32_t kind;        /* 0 linear scalar, 1 inviscid Burgers */
    double dt;
    double * xcoord;     /* [2 * ncelm + 5] (with BOUND_COUNT = 2 padding) */
    double * so0, * so1; /* [2 * ncelm + 5] */
    double * cfl;        /* [2 * ncelm + 5] */
} ora_st;

void ora_st_setup(ora_st * s);
void ora_st_march(ora_st * s, int alpha, int64_t steps);

/* A StaticMesh built on the CPU (mesh_oracle.c): every table whole, ghost
 * rows first, in the reference's layout (StaticMesh.hpp:434-451); widths
 * ndim for ndcrd/fccnd/fcnml/clcnd, 5 fcnds, 4 fccls, 9 clnds, 7 clfcs,
 * 3 bndfcs, 1 for the rest. */
typedef struct
{
    int32_t ndim;
    int64_t nnode, nface, ncell, nbound, ngstnode, ngstface, ngstcell;
    double *ndcrd, *fccnd, *fcnml, *fcara, *clcnd, *clvol;
    int32_t *fctpn, *cltpn, *clgrp, *fcnds, *fccls, *clnds, *clfcs, *bndfcs;
} ora_built_mesh;

/* build_interior (with metrics), build_boundary (no named groups) and
 * build_ghost of a mesh of ncell cells: cltpn[ncell], clnds[ncell][9].
 * Returns 0, or -1 (bad ndim, out of memory).  Free with ora_mesh_free. */
int ora_mesh_build(int ndim, int64_t nnode, int64_t ncell, const double * ndcrd, const int32_t * cltpn,
                   const int32_t * clnds, ora_built_mesh * out);
void ora_mesh_free(ora_built_mesh * m);

#ifdef __cplusplus
}
#endif

#endif
