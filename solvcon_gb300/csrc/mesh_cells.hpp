#pragma once

/*
 * The faces of each cell type: for every face its type, its node count and
 * the positions of its nodes in the cell's node list, in the order the
 * reference's FaceBuilder emits them (cpp/solvcon/mesh/StaticMesh_interior.cpp
 * :26-310).  The order of the faces and of their nodes decides the face
 * numbering and the face orientation of a built mesh, so both mesh builders
 * (host and device) read this one table.
 */

#include "mesh_host.hpp"

#include <cstdint>

#ifdef __CUDACC__
#define SCG_HD __host__ __device__
#else
#define SCG_HD
#endif

namespace scg
{

struct FaceDef
{
    int32_t type; // face cell type
    int nnd;      // nodes of the face
    int pos[4];   // 1-based positions into the cell's node list
};

struct CellFaces
{
    int nface;
    FaceDef f[CLMFC];
};

SCG_HD inline CellFaces cell_faces(int32_t type)
{
    switch (type)
    {
    case CT_QUAD:
        return {4, {{CT_LINE, 2, {1, 2}}, {CT_LINE, 2, {2, 3}}, {CT_LINE, 2, {3, 4}}, {CT_LINE, 2, {4, 1}}}};
    case CT_TRIANGLE:
        return {3, {{CT_LINE, 2, {1, 2}}, {CT_LINE, 2, {2, 3}}, {CT_LINE, 2, {3, 1}}}};
    case CT_HEX:
        return {6, {{CT_QUAD, 4, {1, 4, 3, 2}}, {CT_QUAD, 4, {2, 3, 7, 6}}, {CT_QUAD, 4, {5, 6, 7, 8}},
                    {CT_QUAD, 4, {1, 5, 8, 4}}, {CT_QUAD, 4, {1, 2, 6, 5}}, {CT_QUAD, 4, {3, 4, 8, 7}}}};
    case CT_TET:
        return {4, {{CT_TRIANGLE, 3, {1, 3, 2}}, {CT_TRIANGLE, 3, {1, 2, 4}}, {CT_TRIANGLE, 3, {1, 4, 3}},
                    {CT_TRIANGLE, 3, {2, 3, 4}}}};
    case CT_PRISM:
        return {5, {{CT_TRIANGLE, 3, {1, 2, 3}}, {CT_TRIANGLE, 3, {4, 6, 5}}, {CT_QUAD, 4, {1, 4, 5, 2}},
                    {CT_QUAD, 4, {1, 3, 6, 4}}, {CT_QUAD, 4, {2, 5, 6, 3}}}};
    case CT_PYRAMID:
        return {5, {{CT_TRIANGLE, 3, {1, 5, 4}}, {CT_TRIANGLE, 3, {2, 5, 1}}, {CT_TRIANGLE, 3, {3, 5, 2}},
                    {CT_TRIANGLE, 3, {4, 5, 3}}, {CT_QUAD, 4, {1, 4, 3, 2}}}};
    case CT_LINE:
        return {2, {{CT_POINT, 1, {1}}, {CT_POINT, 1, {2}}}};
    case CT_POINT:
        return {1, {{CT_NONE, 0, {1}}}};
    default:
        return {0, {}};
    }
}

} // namespace scg
