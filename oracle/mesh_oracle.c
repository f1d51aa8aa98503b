/*
 * StaticMesh build of the CPU oracle -- TEST INFRASTRUCTURE ONLY (see
 * cese_oracle.h).  Never linked into the product.
 *
 * Restates, in the reference's operation order, how solvcon's StaticMesh
 * builds its tables from node coordinates and cell node lists:
 *
 *   build_interior -- FaceBuilder (cpp/solvcon/mesh/StaticMesh_interior.cpp
 *     :17-552): every cell emits its faces in its type's order, faces are
 *     de-duplicated by first sighting, cells and faces are related; then
 *     calc_metric (:616-977): face centroids, normals and areas, cell
 *     centroids and volumes, faces re-oriented to point out of their first
 *     cell;
 *   build_boundary (StaticMesh_boundary.cpp:103-182) with no named groups:
 *     every boundary face, in face order, in one group;
 *   build_ghost / fill_ghost (StaticMesh_boundary.cpp:185-629): one ghost
 *     cell mirrored across every boundary face, its nodes reflected, its
 *     faces copied, the ghost metrics computed.
 *
 * The oracle's march and the benchmark's CPU arm build their meshes with it,
 * so neither needs the GPU library.  It equals the reference's tables entry
 * for entry (golden vectors generated from the reference; tests/test_oracle.py).
 */

#include "cese_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define FCMND 4
#define CLMND 8
#define CLMFC 6
#define FCREL 4
#define BFREL 3

enum
{
    T_NONE = 0,
    T_POINT = 1,
    T_LINE = 2,
    T_QUAD = 3,
    T_TRI = 4,
    T_HEX = 5,
    T_TET = 6,
    T_PRISM = 7,
    T_PYRAMID = 8
};

/* The faces each cell type emits (FaceBuilder::add_*,
 * StaticMesh_interior.cpp:26-310): face type, node count and the 1-based
 * positions of the face's nodes in the cell's node list. */
typedef struct
{
    int type, nnd, pos[4];
} face_def;

static int cell_faces(int type, face_def * f)
{
    static const face_def quad[4] = {{T_LINE, 2, {1, 2}}, {T_LINE, 2, {2, 3}}, {T_LINE, 2, {3, 4}}, {T_LINE, 2, {4, 1}}};
    static const face_def tri[3] = {{T_LINE, 2, {1, 2}}, {T_LINE, 2, {2, 3}}, {T_LINE, 2, {3, 1}}};
    static const face_def hex[6] = {{T_QUAD, 4, {1, 4, 3, 2}}, {T_QUAD, 4, {2, 3, 7, 6}}, {T_QUAD, 4, {5, 6, 7, 8}},
                                    {T_QUAD, 4, {1, 5, 8, 4}}, {T_QUAD, 4, {1, 2, 6, 5}}, {T_QUAD, 4, {3, 4, 8, 7}}};
    static const face_def tet[4] = {{T_TRI, 3, {1, 3, 2}}, {T_TRI, 3, {1, 2, 4}}, {T_TRI, 3, {1, 4, 3}},
                                    {T_TRI, 3, {2, 3, 4}}};
    static const face_def prism[5] = {{T_TRI, 3, {1, 2, 3}}, {T_TRI, 3, {4, 6, 5}}, {T_QUAD, 4, {1, 4, 5, 2}},
                                      {T_QUAD, 4, {1, 3, 6, 4}}, {T_QUAD, 4, {2, 5, 6, 3}}};
    static const face_def pyr[5] = {{T_TRI, 3, {1, 5, 4}}, {T_TRI, 3, {2, 5, 1}}, {T_TRI, 3, {3, 5, 2}},
                                    {T_TRI, 3, {4, 5, 3}}, {T_QUAD, 4, {1, 4, 3, 2}}};
    const face_def * src = NULL;
    int n = 0;
    switch (type)
    {
    case T_QUAD: src = quad; n = 4; break;
    case T_TRI: src = tri; n = 3; break;
    case T_HEX: src = hex; n = 6; break;
    case T_TET: src = tet; n = 4; break;
    case T_PRISM: src = prism; n = 5; break;
    case T_PYRAMID: src = pyr; n = 5; break;
    default: return 0;
    }
    memcpy(f, src, sizeof(face_def) * (size_t)n);
    return n;
}

/* Row-major tables with ghost rows first: row i (negative for ghosts) of a
 * table with ng ghost rows and width w starts at (i + ng) * w. */
#define AT(a, ng, w, i, j) ((a)[((int64_t)(i) + (ng)) * (w) + (j)])

/* ---- build_interior: FaceBuilder ---------------------------------------- */

typedef struct
{
    int64_t mface, nface;
    int32_t *clfcs, *fctpn, *fcnds, *fccls;
} faces_t;

/* The number of nodes of face jfc that are also nodes of face ifc
 * (FaceBuilder::make_dedupmap check_match). */
static int count_match(const int32_t * fcnds, int64_t ifc, int64_t jfc)
{
    int cond = 0;
    int const ni = fcnds[ifc * 5];
    int const nj = fcnds[jfc * 5];
    for (int jn = 1; jn <= nj; ++jn)
    {
        for (int in = 1; in <= ni; ++in)
        {
            if (fcnds[ifc * 5 + in] == fcnds[jfc * 5 + jn])
            {
                ++cond;
                break;
            }
        }
    }
    return cond;
}

static int build_faces(int64_t nnode, int64_t ncell, const int32_t * cltpn, const int32_t * clnds, faces_t * F)
{
    face_def fd[CLMFC];
    int64_t mface = 0;
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        mface += cell_faces(cltpn[icl], fd);
    }
    F->mface = mface;
    F->clfcs = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ncell * 7));
    F->fctpn = (int32_t *)malloc(sizeof(int32_t) * (size_t)(mface > 0 ? mface : 1));
    F->fcnds = (int32_t *)malloc(sizeof(int32_t) * (size_t)(mface > 0 ? mface * 5 : 1));
    F->fccls = (int32_t *)malloc(sizeof(int32_t) * (size_t)(mface > 0 ? mface * 4 : 1));
    int64_t * ndoff = (int64_t *)calloc((size_t)(nnode + 1), sizeof(int64_t));
    int64_t * dedup = (int64_t *)malloc(sizeof(int64_t) * (size_t)(mface > 0 ? mface : 1));
    int64_t * map2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(mface > 0 ? mface : 1));
    if (!F->clfcs || !F->fctpn || !F->fcnds || !F->fccls || !ndoff || !dedup || !map2)
    {
        free(ndoff);
        free(dedup);
        free(map2);
        return -1;
    }
    for (int64_t k = 0; k < ncell * 7; ++k)
        F->clfcs[k] = -1;
    for (int64_t k = 0; k < mface; ++k)
        F->fctpn[k] = -1;
    for (int64_t k = 0; k < mface * 5; ++k)
        F->fcnds[k] = -1;
    for (int64_t k = 0; k < mface * 4; ++k)
        F->fccls[k] = -1;

    /* populate: every cell's faces in its type's order. */
    int64_t ifc = 0;
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        int const nf = cell_faces(cltpn[icl], fd);
        if (nf == 0)
            continue;
        F->clfcs[icl * 7] = nf;
        for (int k = 0; k < nf; ++k, ++ifc)
        {
            F->clfcs[icl * 7 + 1 + k] = (int32_t)ifc;
            F->fctpn[ifc] = fd[k].type;
            F->fcnds[ifc * 5] = fd[k].nnd;
            for (int j = 0; j < fd[k].nnd; ++j)
                F->fcnds[ifc * 5 + 1 + j] = clnds[icl * 9 + fd[k].pos[j]];
        }
    }

    /* make_ndfcs: the faces touching each node, in face order. */
    for (int64_t f = 0; f < mface; ++f)
        for (int j = 1; j <= F->fcnds[f * 5]; ++j)
            ndoff[F->fcnds[f * 5 + j] + 1] += 1;
    for (int64_t n = 0; n < nnode; ++n)
        ndoff[n + 1] += ndoff[n];
    int64_t * ndfcs = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndoff[nnode] > 0 ? ndoff[nnode] : 1));
    int64_t * fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnode > 0 ? nnode : 1));
    if (!ndfcs || !fill)
    {
        free(ndfcs);
        free(fill);
        free(ndoff);
        free(dedup);
        free(map2);
        return -1;
    }
    memcpy(fill, ndoff, sizeof(int64_t) * (size_t)nnode);
    for (int64_t f = 0; f < mface; ++f)
        for (int j = 1; j <= F->fcnds[f * 5]; ++j)
        {
            int32_t const nd = F->fcnds[f * 5 + j];
            ndfcs[fill[nd]++] = f;
        }

    /* make_dedupmap: a face equal to an earlier kept face maps to it. */
    for (int64_t f = 0; f < mface; ++f)
        dedup[f] = f;
    for (int64_t f = 0; f < mface; ++f)
    {
        if (dedup[f] != f)
            continue;
        int32_t const ind = F->fcnds[f * 5 + 1]; /* the face's first node only */
        for (int64_t it = ndoff[ind]; it < ndoff[ind + 1]; ++it)
        {
            int64_t const g = ndfcs[it];
            if (g != f && F->fctpn[g] == F->fctpn[f] && count_match(F->fcnds, f, g) == F->fcnds[g * 5])
                dedup[g] = f;
        }
    }

    /* remap_face: compact the kept faces in order, relate cells and faces. */
    int64_t jfc = 0;
    for (int64_t f = 0; f < mface; ++f)
    {
        if (dedup[f] == f)
        {
            for (int k = 0; k <= FCMND; ++k)
                F->fcnds[jfc * 5 + k] = F->fcnds[f * 5 + k];
            F->fctpn[jfc] = F->fctpn[f];
            map2[f] = jfc;
            ++jfc;
        }
        else
        {
            map2[f] = map2[dedup[f]];
        }
    }
    F->nface = jfc;
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        for (int k = 1; k <= F->clfcs[icl * 7]; ++k)
        {
            int64_t const j = map2[F->clfcs[icl * 7 + k]];
            F->clfcs[icl * 7 + k] = (int32_t)j;
            if (F->fccls[j * 4] == -1)
                F->fccls[j * 4] = (int32_t)icl;
            else if (F->fccls[j * 4 + 1] == -1)
                F->fccls[j * 4 + 1] = (int32_t)icl;
        }
    }
    free(ndfcs);
    free(fill);
    free(ndoff);
    free(dedup);
    free(map2);
    return 0;
}

/* ---- metrics (calc_metric and the ghost part of fill_ghost) ------------- */

/* Centroid of face ifc (2D: the edge's midpoint; 3D: the area-weighted
 * centroid of the triangles fanned from the node average). */
static void face_centroid(ora_built_mesh * m, int64_t ifc)
{
    int const nd = m->ndim;
    int64_t const gn = m->ngstnode, gf = m->ngstface;
    if (nd == 2)
    {
        int32_t ind = AT(m->fcnds, gf, 5, ifc, 1);
        AT(m->fccnd, gf, 2, ifc, 0) = AT(m->ndcrd, gn, 2, ind, 0);
        AT(m->fccnd, gf, 2, ifc, 1) = AT(m->ndcrd, gn, 2, ind, 1);
        ind = AT(m->fcnds, gf, 5, ifc, 2);
        AT(m->fccnd, gf, 2, ifc, 0) += AT(m->ndcrd, gn, 2, ind, 0);
        AT(m->fccnd, gf, 2, ifc, 1) += AT(m->ndcrd, gn, 2, ind, 1);
        AT(m->fccnd, gf, 2, ifc, 0) /= 2;
        AT(m->fccnd, gf, 2, ifc, 1) /= 2;
        return;
    }
    double cfd[FCMND + 2][3];
    cfd[0][0] = cfd[0][1] = cfd[0][2] = 0.0;
    size_t const nnd = (size_t)AT(m->fcnds, gf, 5, ifc, 0);
    for (size_t inf = 1; inf <= nnd; ++inf)
    {
        int32_t const ind = AT(m->fcnds, gf, 5, ifc, inf);
        for (int d = 0; d < 3; ++d)
        {
            cfd[inf][d] = AT(m->ndcrd, gn, 3, ind, d);
            cfd[0][d] += AT(m->ndcrd, gn, 3, ind, d);
        }
    }
    for (int d = 0; d < 3; ++d)
        cfd[nnd + 1][d] = cfd[1][d];
    for (int d = 0; d < 3; ++d)
        cfd[0][d] /= nnd;
    double voc = 0.0;
    double * c = &AT(m->fccnd, gf, 3, ifc, 0);
    c[0] = c[1] = c[2] = 0.0;
    for (size_t inf = 1; inf <= nnd; ++inf)
    {
        double crd[3];
        for (int d = 0; d < 3; ++d)
            crd[d] = (cfd[0][d] + cfd[inf][d] + cfd[inf + 1][d]) / 3;
        double const du0 = cfd[inf][0] - cfd[0][0];
        double const du1 = cfd[inf][1] - cfd[0][1];
        double const du2 = cfd[inf][2] - cfd[0][2];
        double const dv0 = cfd[inf + 1][0] - cfd[0][0];
        double const dv1 = cfd[inf + 1][1] - cfd[0][1];
        double const dv2 = cfd[inf + 1][2] - cfd[0][2];
        double const dw0 = du1 * dv2 - du2 * dv1;
        double const dw1 = du2 * dv0 - du0 * dv2;
        double const dw2 = du0 * dv1 - du1 * dv0;
        double const vob = sqrt(dw0 * dw0 + dw1 * dw1 + dw2 * dw2);
        c[0] += crd[0] * vob;
        c[1] += crd[1] * vob;
        c[2] += crd[2] * vob;
        voc += vob;
    }
    c[0] /= voc;
    c[1] /= voc;
    c[2] /= voc;
}

/* Unit normal and area of face ifc (2D: the edge rotated; 3D: the sum of
 * cross products of the node vectors about the centroid). */
static void face_normal(ora_built_mesh * m, int64_t ifc)
{
    int const nd = m->ndim;
    int64_t const gn = m->ngstnode, gf = m->ngstface;
    double * n = &AT(m->fcnml, gf, nd, ifc, 0);
    double * a = &AT(m->fcara, gf, 1, ifc, 0);
    if (nd == 2)
    {
        int32_t const i1 = AT(m->fcnds, gf, 5, ifc, 1);
        int32_t const i2 = AT(m->fcnds, gf, 5, ifc, 2);
        n[0] = AT(m->ndcrd, gn, 2, i2, 1) - AT(m->ndcrd, gn, 2, i1, 1);
        n[1] = AT(m->ndcrd, gn, 2, i1, 0) - AT(m->ndcrd, gn, 2, i2, 0);
        *a = sqrt(n[0] * n[0] + n[1] * n[1]);
        n[0] /= *a;
        n[1] /= *a;
        return;
    }
    double rv[FCMND][3];
    size_t const nnd = (size_t)AT(m->fcnds, gf, 5, ifc, 0);
    for (size_t inf = 0; inf < nnd; ++inf)
    {
        int32_t const ind = AT(m->fcnds, gf, 5, ifc, inf + 1);
        for (int d = 0; d < 3; ++d)
            rv[inf][d] = AT(m->ndcrd, gn, 3, ind, d) - AT(m->fccnd, gf, 3, ifc, d);
    }
    n[0] = rv[nnd - 1][1] * rv[0][2] - rv[nnd - 1][2] * rv[0][1];
    n[1] = rv[nnd - 1][2] * rv[0][0] - rv[nnd - 1][0] * rv[0][2];
    n[2] = rv[nnd - 1][0] * rv[0][1] - rv[nnd - 1][1] * rv[0][0];
    for (size_t k = 1; k < nnd; ++k)
    {
        n[0] += rv[k - 1][1] * rv[k][2] - rv[k - 1][2] * rv[k][1];
        n[1] += rv[k - 1][2] * rv[k][0] - rv[k - 1][0] * rv[k][2];
        n[2] += rv[k - 1][0] * rv[k][1] - rv[k - 1][1] * rv[k][0];
    }
    *a = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    n[0] /= *a;
    n[1] /= *a;
    n[2] /= *a;
    *a /= 2.0;
}

/* Centroid of cell icl: the node average, then the volume-weighted centroids
 * of the pyramids it forms with the faces. */
static void cell_centroid(ora_built_mesh * m, int64_t icl)
{
    int const nd = m->ndim;
    int64_t const gn = m->ngstnode, gf = m->ngstface, gc = m->ngstcell;
    double crd[3] = {0.0, 0.0, 0.0};
    size_t const nnd = (size_t)AT(m->clnds, gc, 9, icl, 0);
    for (size_t inc = 1; inc <= nnd; ++inc)
    {
        int32_t const ind = AT(m->clnds, gc, 9, icl, inc);
        for (int d = 0; d < nd; ++d)
            crd[d] += AT(m->ndcrd, gn, nd, ind, d);
    }
    for (int d = 0; d < nd; ++d)
        crd[d] /= nnd;
    double voc = 0.0;
    double * c = &AT(m->clcnd, gc, nd, icl, 0);
    for (int d = 0; d < nd; ++d)
        c[d] = 0.0;
    size_t const nfc = (size_t)AT(m->clfcs, gc, 7, icl, 0);
    for (size_t ifl = 1; ifl <= nfc; ++ifl)
    {
        int32_t const ifc = AT(m->clfcs, gc, 7, icl, ifl);
        double const * fc = &AT(m->fccnd, gf, nd, ifc, 0);
        double const * fn = &AT(m->fcnml, gf, nd, ifc, 0);
        double const fa = AT(m->fcara, gf, 1, ifc, 0);
        if (nd == 2)
        {
            double const du0 = crd[0] - fc[0];
            double const du1 = crd[1] - fc[1];
            double const vob = fabs(du0 * fn[0] + du1 * fn[1]) * fa;
            voc += vob;
            double const dv0 = fc[0] + du0 / 3;
            double const dv1 = fc[1] + du1 / 3;
            c[0] += dv0 * vob;
            c[1] += dv1 * vob;
        }
        else
        {
            double const du0 = crd[0] - fc[0];
            double const du1 = crd[1] - fc[1];
            double const du2 = crd[2] - fc[2];
            double const vob = fabs((du0 * fn[0] + du1 * fn[1] + du2 * fn[2]) * fa);
            voc += vob;
            double const dv0 = fc[0] + du0 / 4;
            double const dv1 = fc[1] + du1 / 4;
            double const dv2 = fc[2] + du2 / 4;
            c[0] += dv0 * vob;
            c[1] += dv1 * vob;
            c[2] += dv2 * vob;
        }
    }
    for (int d = 0; d < nd; ++d)
        c[d] /= voc;
}

/* calc_metric's face re-orientation: reverse the node list, flip the normal. */
static void reorder_face(ora_built_mesh * m, int64_t ifc)
{
    int64_t const gf = m->ngstface;
    int const nnd = AT(m->fcnds, gf, 5, ifc, 0);
    int32_t tmp[FCMND];
    for (int j = 0; j < nnd; ++j)
        tmp[j] = AT(m->fcnds, gf, 5, ifc, nnd - j);
    for (int j = 0; j < nnd; ++j)
        AT(m->fcnds, gf, 5, ifc, j + 1) = tmp[j];
    for (int d = 0; d < m->ndim; ++d)
        AT(m->fcnml, gf, m->ndim, ifc, d) = -AT(m->fcnml, gf, m->ndim, ifc, d);
}

/* Volume of cell icl from its faces.  Body cells (calc_metric) re-orient a
 * face to point out of its first cell; ghost cells (fill_ghost) flip only a
 * normal that points into them from a face they own. */
static void cell_volume(ora_built_mesh * m, int64_t icl, int ghost)
{
    int const nd = m->ndim;
    int64_t const gf = m->ngstface, gc = m->ngstcell;
    double * vol = &AT(m->clvol, gc, 1, icl, 0);
    *vol = 0.0;
    int const nfc = AT(m->clfcs, gc, 7, icl, 0);
    for (int it = 1; it <= nfc; ++it)
    {
        int32_t const ifc = AT(m->clfcs, gc, 7, icl, it);
        double v = 0.0;
        for (int d = 0; d < nd; ++d)
            v += (AT(m->fccnd, gf, nd, ifc, d) - AT(m->clcnd, gc, nd, icl, d)) * AT(m->fcnml, gf, nd, ifc, d);
        v *= AT(m->fcara, gf, 1, ifc, 0);
        int64_t const this_fcl = AT(m->fccls, gf, 4, ifc, 0);
        if (ghost)
        {
            if (v < 0.0)
            {
                if (this_fcl == icl)
                    for (int d = 0; d < nd; ++d)
                        AT(m->fcnml, gf, nd, ifc, d) = -AT(m->fcnml, gf, nd, ifc, d);
                v = -v;
            }
        }
        else if (v < 0.0)
        {
            if (this_fcl == icl)
                reorder_face(m, ifc);
            v = -v;
        }
        else if (this_fcl != icl)
        {
            reorder_face(m, ifc);
        }
        *vol += v;
    }
    *vol /= nd;
}

/* ---- the whole build ---------------------------------------------------- */

static int nface_of(int type)
{
    face_def fd[CLMFC];
    return cell_faces(type, fd);
}

void ora_mesh_free(ora_built_mesh * m)
{
    double ** reals[] = {&m->ndcrd, &m->fccnd, &m->fcnml, &m->fcara, &m->clcnd, &m->clvol};
    int32_t ** ints[] = {&m->fctpn, &m->cltpn, &m->clgrp, &m->fcnds, &m->fccls, &m->clnds, &m->clfcs, &m->bndfcs};
    for (size_t k = 0; k < sizeof(reals) / sizeof(reals[0]); ++k)
    {
        free(*reals[k]);
        *reals[k] = NULL;
    }
    for (size_t k = 0; k < sizeof(ints) / sizeof(ints[0]); ++k)
    {
        free(*ints[k]);
        *ints[k] = NULL;
    }
}

static double * real_table(int64_t rows, int w)
{
    return (double *)calloc((size_t)(rows * w > 0 ? rows * w : 1), sizeof(double));
}

static int32_t * int_table(int64_t rows, int w, int32_t init)
{
    int64_t const n = rows * w > 0 ? rows * w : 1;
    int32_t * p = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (p)
        for (int64_t k = 0; k < n; ++k)
            p[k] = init;
    return p;
}

int ora_mesh_build(int ndim, int64_t nnode, int64_t ncell, const double * ndcrd, const int32_t * cltpn,
                   const int32_t * clnds, ora_built_mesh * m)
{
    memset(m, 0, sizeof(*m));
    if (ndim != 2 && ndim != 3)
        return -1;
    faces_t F;
    memset(&F, 0, sizeof(F));
    if (build_faces(nnode, ncell, cltpn, clnds, &F) != 0)
    {
        free(F.clfcs);
        free(F.fctpn);
        free(F.fcnds);
        free(F.fccls);
        return -1;
    }
    int64_t const nface = F.nface;

    /* build_boundary: boundary faces in face order, one group. */
    int64_t nbound = 0;
    for (int64_t f = 0; f < nface; ++f)
        if (F.fccls[f * 4 + 1] < 0)
            ++nbound;

    /* build_ghost: count, then lay every table out with ghost rows first. */
    int64_t ngnode = 0, ngface = 0;
    {
        int64_t ib = 0;
        for (int64_t f = 0; f < nface; ++f)
        {
            if (F.fccls[f * 4 + 1] >= 0)
                continue;
            int32_t const icl = F.fccls[f * 4];
            ngface += nface_of(cltpn[icl]) - 1;
            ngnode += clnds[icl * 9] - F.fcnds[f * 5];
            ++ib;
        }
    }
    m->ndim = ndim;
    m->nnode = nnode;
    m->nface = nface;
    m->ncell = ncell;
    m->nbound = nbound;
    m->ngstnode = ngnode;
    m->ngstface = ngface;
    m->ngstcell = nbound;
    int64_t const tn = ngnode + nnode, tf = ngface + nface, tc = nbound + ncell;
    m->ndcrd = real_table(tn, ndim);
    m->fccnd = real_table(tf, ndim);
    m->fcnml = real_table(tf, ndim);
    m->fcara = real_table(tf, 1);
    m->clcnd = real_table(tc, ndim);
    m->clvol = real_table(tc, 1);
    m->fctpn = int_table(tf, 1, 0);
    m->cltpn = int_table(tc, 1, 0);
    m->clgrp = int_table(tc, 1, -1);
    m->fcnds = int_table(tf, 5, -1);
    m->fccls = int_table(tf, 4, -1);
    m->clnds = int_table(tc, 9, -1);
    m->clfcs = int_table(tc, 7, -1);
    m->bndfcs = int_table(nbound, BFREL, -1);
    if (!m->ndcrd || !m->fccnd || !m->fcnml || !m->fcara || !m->clcnd || !m->clvol || !m->fctpn || !m->cltpn ||
        !m->clgrp || !m->fcnds || !m->fccls || !m->clnds || !m->clfcs || !m->bndfcs)
    {
        ora_mesh_free(m);
        free(F.clfcs);
        free(F.fctpn);
        free(F.fcnds);
        free(F.fccls);
        return -1;
    }
    memcpy(m->ndcrd + ngnode * ndim, ndcrd, sizeof(double) * (size_t)(nnode * ndim));
    memcpy(m->cltpn + nbound, cltpn, sizeof(int32_t) * (size_t)ncell);
    memcpy(m->clnds + nbound * 9, clnds, sizeof(int32_t) * (size_t)(ncell * 9));
    memcpy(m->clfcs + nbound * 7, F.clfcs, sizeof(int32_t) * (size_t)(ncell * 7));
    memcpy(m->fctpn + ngface, F.fctpn, sizeof(int32_t) * (size_t)nface);
    memcpy(m->fcnds + ngface * 5, F.fcnds, sizeof(int32_t) * (size_t)(nface * 5));
    memcpy(m->fccls + ngface * 4, F.fccls, sizeof(int32_t) * (size_t)(nface * 4));
    free(F.clfcs);
    free(F.fctpn);
    free(F.fcnds);
    free(F.fccls);

    /* calc_metric over the body entities (the ghost rows are not yet in
     * use; the reference computes the metrics before the ghost layer). */
    for (int64_t f = 0; f < nface; ++f)
        face_centroid(m, f);
    for (int64_t f = 0; f < nface; ++f)
        face_normal(m, f);
    for (int64_t c = 0; c < ncell; ++c)
        cell_centroid(m, c);
    for (int64_t c = 0; c < ncell; ++c)
        cell_volume(m, c, 0);

    {
        int64_t ib = 0;
        for (int64_t f = 0; f < nface; ++f)
            if (AT(m->fccls, ngface, 4, f, 1) < 0)
            {
                m->bndfcs[ib * 3] = (int32_t)f;
                m->bndfcs[ib * 3 + 1] = 0;
                ++ib;
            }
    }

    /* fill_ghost: mirror the interior cell across each boundary face. */
    int32_t * gstnd = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nnode > 0 ? nnode : 1));
    if (!gstnd)
    {
        ora_mesh_free(m);
        return -1;
    }
    for (int64_t n = 0; n < nnode; ++n)
        gstnd[n] = (int32_t)nnode;
    int32_t ignd = -1, igfc = -1;
    for (int32_t igcl = -1; igcl >= -(int32_t)nbound; --igcl)
    {
        int32_t const ibfc = m->bndfcs[(-igcl - 1) * 3];
        int32_t const icl = AT(m->fccls, ngface, 4, ibfc, 0);
        AT(m->cltpn, nbound, 1, igcl, 0) = AT(m->cltpn, nbound, 1, icl, 0);
        AT(m->clgrp, nbound, 1, igcl, 0) = AT(m->clgrp, nbound, 1, icl, 0);
        for (int k = 0; k <= CLMND; ++k)
            AT(m->clnds, nbound, 9, igcl, k) = AT(m->clnds, nbound, 9, icl, k);
        for (int inl = 1; inl <= AT(m->clnds, nbound, 9, icl, 0); ++inl)
        {
            int32_t const ind = AT(m->clnds, nbound, 9, icl, inl);
            int found = 0;
            for (int inf = 1; inf <= AT(m->fcnds, ngface, 5, ibfc, 0); ++inf)
                if (ind == AT(m->fcnds, ngface, 5, ibfc, inf))
                {
                    found = 1;
                    break;
                }
            if (!found)
            {
                gstnd[ind] = ignd;
                AT(m->clnds, nbound, 9, igcl, inl) = ignd;
                double dist = 0.0;
                for (int d = 0; d < ndim; ++d)
                    dist += (AT(m->fccnd, ngface, ndim, ibfc, d) - AT(m->ndcrd, ngnode, ndim, ind, d)) *
                            AT(m->fcnml, ngface, ndim, ibfc, d);
                for (int d = 0; d < ndim; ++d)
                    AT(m->ndcrd, ngnode, ndim, ignd, d) =
                        AT(m->ndcrd, ngnode, ndim, ind, d) + 2 * dist * AT(m->fcnml, ngface, ndim, ibfc, d);
                ignd -= 1;
            }
        }
        AT(m->fccls, ngface, 4, ibfc, 1) = igcl;
        for (int k = 0; k <= CLMFC; ++k)
            AT(m->clfcs, nbound, 7, igcl, k) = AT(m->clfcs, nbound, 7, icl, k);
        for (int ifl = 1; ifl <= AT(m->clfcs, nbound, 7, icl, 0); ++ifl)
        {
            int32_t const ifc = AT(m->clfcs, nbound, 7, icl, ifl);
            if (ifc == ibfc)
                continue;
            AT(m->fctpn, ngface, 1, igfc, 0) = AT(m->fctpn, ngface, 1, ifc, 0);
            AT(m->fccls, ngface, 4, igfc, 0) = igcl;
            AT(m->clfcs, nbound, 7, igcl, ifl) = igfc;
            for (int k = 0; k <= FCMND; ++k)
                AT(m->fcnds, ngface, 5, igfc, k) = AT(m->fcnds, ngface, 5, ifc, k);
            for (int inf = 1; inf <= AT(m->fcnds, ngface, 5, igfc, 0); ++inf)
            {
                int32_t const ind = AT(m->fcnds, ngface, 5, igfc, inf);
                if (gstnd[ind] != (int32_t)nnode)
                    AT(m->fcnds, ngface, 5, igfc, inf) = gstnd[ind];
            }
            igfc -= 1;
        }
        for (int inl = 1; inl <= AT(m->clnds, nbound, 9, icl, 0); ++inl)
            gstnd[AT(m->clnds, nbound, 9, icl, inl)] = (int32_t)nnode;
    }
    free(gstnd);
    for (int64_t f = -1; f >= -ngface; --f)
        face_centroid(m, f);
    for (int64_t f = -1; f >= -ngface; --f)
        face_normal(m, f);
    for (int64_t c = -1; c >= -nbound; --c)
        cell_centroid(m, c);
    for (int64_t c = -1; c >= -nbound; --c)
        cell_volume(m, c, 1);
    return 0;
}
