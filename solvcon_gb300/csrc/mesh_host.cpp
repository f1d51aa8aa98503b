/*
 * Host mesh builder: face extraction with de-duplication, metrics, boundary
 * registration and the mirrored ghost layer.  The step order and the face /
 * node numbering follow the reference StaticMesh exactly (citations inline),
 * because every downstream table of the CESE march is indexed by them.
 */

#include "mesh_host.hpp"
#include "mesh_cells.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>
#include <set>
#include <stdexcept>
#include <thread>
#include <type_traits>
#include <utility>

namespace scg
{

int cell_nface(int32_t type) { return cell_faces(type).nface; }

int cell_ndim(int32_t type)
{
    switch (type)
    {
    case CT_POINT: return 0;
    case CT_LINE: return 1;
    case CT_QUAD:
    case CT_TRIANGLE: return 2;
    case CT_HEX:
    case CT_TET:
    case CT_PRISM:
    case CT_PYRAMID: return 3;
    default: return 0;
    }
}

HostMesh::HostMesh(int ndim_in, int64_t nnode_in, int64_t nface_in, int64_t ncell_in)
    : ndim(ndim_in)
    , nnode(nnode_in)
    , nface(nface_in)
    , ncell(ncell_in)
{
    if (ndim < 2 || ndim > 3)
    {
        throw std::invalid_argument("StaticMesh: ndim must be 2 or 3");
    }
    if (nnode < 0 || nface < 0 || ncell < 0)
    {
        throw std::invalid_argument("StaticMesh: negative size");
    }
    // Shapes of the constructor (StaticMesh.hpp:290-311).
    ndcrd.make(0, nnode, ndim, 0.0);
    fccnd.make(0, nface, ndim, 0.0);
    fcnml.make(0, nface, ndim, 0.0);
    fcara.make(0, nface, 1, 0.0);
    clcnd.make(0, ncell, ndim, 0.0);
    clvol.make(0, ncell, 1, 0.0);
    fctpn.make(0, nface, 1, 0);
    cltpn.make(0, ncell, 1, 0);
    clgrp.make(0, ncell, 1, 0);
    fcnds.make(0, nface, FCMND + 1, -1);
    fccls.make(0, nface, FCREL, -1);
    clnds.make(0, ncell, CLMND + 1, -1);
    clfcs.make(0, ncell, CLMFC + 1, -1);
    ednds.make(0, 0, 2, 0);
    bndfcs.make(0, 0, BFREL, -1);
}

void HostMesh::build_interior(bool do_metric, bool do_edge)
{
    build_faces_from_cells();
    if (do_metric)
    {
        calc_metric();
    }
    if (do_edge)
    {
        build_edge();
    }
}

// Face extraction and de-duplication (FaceBuilder, StaticMesh_interior.cpp:
// 17-543): populate every cell's faces, find duplicates through a
// node-to-face table keyed on each face's first node, compact, and record the
// two cells of each face in ascending cell order.
void HostMesh::validate_cells() const
{
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        int32_t const t = cltpn(icl);
        if (t < CT_POINT || t > CT_PYRAMID)
        {
            throw std::invalid_argument("StaticMesh::build_interior: unknown cell type " + std::to_string(t));
        }
        int const nnd = clnds(icl, 0);
        for (int k = 1; k <= nnd; ++k)
        {
            int32_t const ind = clnds(icl, k);
            if (ind < 0 || ind >= nnode)
            {
                throw std::out_of_range("StaticMesh::build_interior: node " + std::to_string(ind) + " of cell " +
                                        std::to_string(icl) + " out of range");
            }
        }
    }
}

void HostMesh::build_faces_from_cells()
{
    validate_cells();

    int64_t mface = 0;
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        mface += cell_nface(cltpn(icl));
    }

    // populate (StaticMesh_interior.cpp:351-384).
    std::vector<int32_t> tfctpn(static_cast<size_t>(mface), -1);
    std::vector<int32_t> tfcnds(static_cast<size_t>(mface) * (FCMND + 1), -1);
    std::vector<int32_t> tclfcs(static_cast<size_t>(ncell) * (CLMFC + 1), -1);
    {
        int64_t ifc = 0;
        for (int64_t icl = 0; icl < ncell; ++icl)
        {
            CellFaces const cf = cell_faces(cltpn(icl));
            int32_t * cfrow = &tclfcs[static_cast<size_t>(icl) * (CLMFC + 1)];
            cfrow[0] = cf.nface;
            for (int k = 0; k < cf.nface; ++k)
            {
                FaceDef const & fd = cf.f[k];
                int32_t * frow = &tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)];
                tfctpn[ifc] = fd.type;
                frow[0] = fd.nnd;
                for (int j = 0; j < std::max(fd.nnd, 1); ++j)
                {
                    frow[1 + j] = clnds(icl, fd.pos[j]);
                }
                cfrow[1 + k] = static_cast<int32_t>(ifc);
                ++ifc;
            }
        }
    }

    // make_ndfcs (StaticMesh_interior.cpp:388-426): faces touching each node,
    // in ascending face order.
    std::vector<int64_t> ndoff(static_cast<size_t>(nnode) + 1, 0);
    for (int64_t ifc = 0; ifc < mface; ++ifc)
    {
        int32_t const * frow = &tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)];
        for (int j = 1; j <= frow[0]; ++j)
        {
            ndoff[frow[j] + 1] += 1;
        }
    }
    std::partial_sum(ndoff.begin(), ndoff.end(), ndoff.begin());
    std::vector<int32_t> ndfcs(static_cast<size_t>(ndoff.back()));
    {
        std::vector<int64_t> fill(ndoff.begin(), ndoff.end() - 1);
        for (int64_t ifc = 0; ifc < mface; ++ifc)
        {
            int32_t const * frow = &tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)];
            for (int j = 1; j <= frow[0]; ++j)
            {
                ndfcs[fill[frow[j]]++] = static_cast<int32_t>(ifc);
            }
        }
    }

    // make_dedupmap (StaticMesh_interior.cpp:428-477).
    std::vector<int64_t> dedup(static_cast<size_t>(mface));
    std::iota(dedup.begin(), dedup.end(), 0);
    auto count_match = [&](int64_t ifc, int64_t jfc)
    {
        int32_t const * irow = &tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)];
        int32_t const * jrow = &tfcnds[static_cast<size_t>(jfc) * (FCMND + 1)];
        int cond = 0;
        for (int jn = 1; jn <= jrow[0]; ++jn)
        {
            for (int in = 1; in <= irow[0]; ++in)
            {
                if (irow[in] == jrow[jn])
                {
                    ++cond;
                    break;
                }
            }
        }
        return cond;
    };
    for (int64_t ifc = 0; ifc < mface; ++ifc)
    {
        if (dedup[ifc] != ifc)
        {
            continue;
        }
        int32_t const * irow = &tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)];
        if (irow[0] < 1)
        {
            continue;
        }
        int32_t const ind = irow[1];
        for (int64_t it = ndoff[ind]; it < ndoff[ind + 1]; ++it)
        {
            int64_t const jfc = ndfcs[it];
            if (jfc != ifc && tfctpn[jfc] == tfctpn[ifc] &&
                count_match(ifc, jfc) == tfcnds[static_cast<size_t>(jfc) * (FCMND + 1)])
            {
                dedup[jfc] = ifc;
            }
        }
    }

    // remap_face (StaticMesh_interior.cpp:479-528).
    std::vector<int32_t> map2(static_cast<size_t>(mface));
    int64_t nf = 0;
    for (int64_t ifc = 0; ifc < mface; ++ifc)
    {
        if (dedup[ifc] == ifc)
        {
            std::copy_n(&tfcnds[static_cast<size_t>(ifc) * (FCMND + 1)], FCMND + 1,
                        &tfcnds[static_cast<size_t>(nf) * (FCMND + 1)]);
            tfctpn[nf] = tfctpn[ifc];
            map2[ifc] = static_cast<int32_t>(nf);
            ++nf;
        }
        else
        {
            map2[ifc] = map2[dedup[ifc]];
        }
    }
    nface = nf;

    remake(fctpn, 0, nface, 1, -1);
    remake(fcnds, 0, nface, FCMND + 1, -1);
    remake(fccls, 0, nface, FCREL, -1);
    std::copy_n(tfctpn.begin(), nface, fctpn.buf.begin());
    std::copy_n(tfcnds.begin(), nface * (FCMND + 1), fcnds.buf.begin());
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        int32_t * cfrow = &tclfcs[static_cast<size_t>(icl) * (CLMFC + 1)];
        for (int ifl = 1; ifl <= cfrow[0]; ++ifl)
        {
            int32_t const jfc = map2[cfrow[ifl]];
            cfrow[ifl] = jfc;
            if (fccls(jfc, 0) == -1)
            {
                fccls(jfc, 0) = static_cast<int32_t>(icl);
            }
            else if (fccls(jfc, 1) == -1)
            {
                fccls(jfc, 1) = static_cast<int32_t>(icl);
            }
        }
    }
    remake(fccnd, 0, nface, ndim, 0.0);
    remake(fcnml, 0, nface, ndim, 0.0);
    remake(fcara, 0, nface, 1, 0.0);
    remake(clfcs, 0, ncell, CLMFC + 1, -1);
    std::copy(tclfcs.begin(), tclfcs.end(), clfcs.buf.begin());
}

// Unique edges in first-seen order, lower node first (StaticMesh_interior.cpp:
// 566-621).
void HostMesh::build_edge()
{
    std::set<std::pair<int32_t, int32_t>> known;
    std::vector<std::pair<int32_t, int32_t>> edges;
    for (int64_t ifc = 0; ifc < nface; ++ifc)
    {
        int const nnd = fcnds(ifc, 0);
        for (int inf = 1; inf <= nnd; ++inf)
        {
            int const idx1 = (nnd == inf) ? 1 : inf + 1;
            int32_t a = fcnds(ifc, inf);
            int32_t b = fcnds(ifc, idx1);
            if (a > b)
            {
                std::swap(a, b);
            }
            if (known.insert({a, b}).second)
            {
                edges.emplace_back(a, b);
            }
        }
    }
    remake(ednds, 0, static_cast<int64_t>(edges.size()), 2, 0);
    for (size_t i = 0; i < edges.size(); ++i)
    {
        ednds(static_cast<int64_t>(i), 0) = edges[i].first;
        ednds(static_cast<int64_t>(i), 1) = edges[i].second;
    }
}

// Face centroids, unit normals and areas, cell centroids and volumes, with
// face re-orientation so that each face normal points out of fccls[0]
// (StaticMesh_interior.cpp:623-977).
void HostMesh::calc_metric()
{
    if (ndim == 2)
    {
        for (int64_t ifc = 0; ifc < nface; ++ifc)
        {
            int32_t const a = fcnds(ifc, 1);
            int32_t const b = fcnds(ifc, 2);
            fccnd(ifc, 0) = (ndcrd(a, 0) + ndcrd(b, 0)) / 2;
            fccnd(ifc, 1) = (ndcrd(a, 1) + ndcrd(b, 1)) / 2;
        }
    }
    else
    {
        for (int64_t ifc = 0; ifc < nface; ++ifc)
        {
            int const nnd = fcnds(ifc, 0);
            std::array<std::array<double, 3>, FCMND + 2> cfd{};
            for (int inf = 1; inf <= nnd; ++inf)
            {
                int32_t const ind = fcnds(ifc, inf);
                for (int d = 0; d < 3; ++d)
                {
                    cfd[inf][d] = ndcrd(ind, d);
                    cfd[0][d] += ndcrd(ind, d);
                }
            }
            cfd[nnd + 1] = cfd[1];
            for (int d = 0; d < 3; ++d)
            {
                cfd[0][d] /= nnd;
            }
            double voc = 0.0;
            double c0 = 0.0, c1 = 0.0, c2 = 0.0;
            for (int inf = 1; inf <= nnd; ++inf)
            {
                double const m0 = (cfd[0][0] + cfd[inf][0] + cfd[inf + 1][0]) / 3;
                double const m1 = (cfd[0][1] + cfd[inf][1] + cfd[inf + 1][1]) / 3;
                double const m2 = (cfd[0][2] + cfd[inf][2] + cfd[inf + 1][2]) / 3;
                double const u0 = cfd[inf][0] - cfd[0][0];
                double const u1 = cfd[inf][1] - cfd[0][1];
                double const u2 = cfd[inf][2] - cfd[0][2];
                double const v0 = cfd[inf + 1][0] - cfd[0][0];
                double const v1 = cfd[inf + 1][1] - cfd[0][1];
                double const v2 = cfd[inf + 1][2] - cfd[0][2];
                double const w0 = u1 * v2 - u2 * v1;
                double const w1 = u2 * v0 - u0 * v2;
                double const w2 = u0 * v1 - u1 * v0;
                double const ar = std::sqrt(w0 * w0 + w1 * w1 + w2 * w2);
                c0 += m0 * ar;
                c1 += m1 * ar;
                c2 += m2 * ar;
                voc += ar;
            }
            fccnd(ifc, 0) = c0 / voc;
            fccnd(ifc, 1) = c1 / voc;
            fccnd(ifc, 2) = c2 / voc;
        }
    }

    if (ndim == 2)
    {
        for (int64_t ifc = 0; ifc < nface; ++ifc)
        {
            int32_t const a = fcnds(ifc, 1);
            int32_t const b = fcnds(ifc, 2);
            double const n0 = ndcrd(b, 1) - ndcrd(a, 1);
            double const n1 = ndcrd(a, 0) - ndcrd(b, 0);
            double const ar = std::sqrt(n0 * n0 + n1 * n1);
            fcara(ifc) = ar;
            fcnml(ifc, 0) = n0 / ar;
            fcnml(ifc, 1) = n1 / ar;
        }
    }
    else
    {
        for (int64_t ifc = 0; ifc < nface; ++ifc)
        {
            int const nnd = fcnds(ifc, 0);
            std::array<std::array<double, 3>, FCMND> rv{};
            for (int inf = 0; inf < nnd; ++inf)
            {
                int32_t const ind = fcnds(ifc, inf + 1);
                for (int d = 0; d < 3; ++d)
                {
                    rv[inf][d] = ndcrd(ind, d) - fccnd(ifc, d);
                }
            }
            double n0 = rv[nnd - 1][1] * rv[0][2] - rv[nnd - 1][2] * rv[0][1];
            double n1 = rv[nnd - 1][2] * rv[0][0] - rv[nnd - 1][0] * rv[0][2];
            double n2 = rv[nnd - 1][0] * rv[0][1] - rv[nnd - 1][1] * rv[0][0];
            for (int k = 1; k < nnd; ++k)
            {
                n0 += rv[k - 1][1] * rv[k][2] - rv[k - 1][2] * rv[k][1];
                n1 += rv[k - 1][2] * rv[k][0] - rv[k - 1][0] * rv[k][2];
                n2 += rv[k - 1][0] * rv[k][1] - rv[k - 1][1] * rv[k][0];
            }
            double const ar = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
            fcnml(ifc, 0) = n0 / ar;
            fcnml(ifc, 1) = n1 / ar;
            fcnml(ifc, 2) = n2 / ar;
            fcara(ifc) = ar / 2.0;
        }
    }

    // Cell centroids: node average, then the face-pyramid weighted centroid
    // (StaticMesh_interior.cpp:770-925; in-centres are off by default).
    double const frac = (ndim == 2) ? 3.0 : 4.0;
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        std::array<double, 3> crd{0.0, 0.0, 0.0};
        int const nnd = clnds(icl, 0);
        for (int inc = 1; inc <= nnd; ++inc)
        {
            int32_t const ind = clnds(icl, inc);
            for (int d = 0; d < ndim; ++d)
            {
                crd[d] += ndcrd(ind, d);
            }
        }
        for (int d = 0; d < ndim; ++d)
        {
            crd[d] /= nnd;
        }
        std::array<double, 3> acc{0.0, 0.0, 0.0};
        double voc = 0.0;
        int const nfc = clfcs(icl, 0);
        for (int ifl = 1; ifl <= nfc; ++ifl)
        {
            int32_t const ifc = clfcs(icl, ifl);
            std::array<double, 3> du{};
            double dot = 0.0;
            for (int d = 0; d < ndim; ++d)
            {
                du[d] = crd[d] - fccnd(ifc, d);
                dot += du[d] * fcnml(ifc, d);
            }
            double const vob = std::fabs(dot) * fcara(ifc);
            voc += vob;
            for (int d = 0; d < ndim; ++d)
            {
                acc[d] += (fccnd(ifc, d) + du[d] / frac) * vob;
            }
        }
        for (int d = 0; d < ndim; ++d)
        {
            clcnd(icl, d) = acc[d] / voc;
        }
    }

    // Volumes with face re-orientation (StaticMesh_interior.cpp:926-977).
    auto reorder_face = [this](int32_t ifc)
    {
        int const nnd = fcnds(ifc, 0);
        std::array<int32_t, FCMND> tmp{};
        for (int j = 0; j < nnd; ++j)
        {
            tmp[j] = fcnds(ifc, nnd - j);
        }
        for (int j = 0; j < nnd; ++j)
        {
            fcnds(ifc, j + 1) = tmp[j];
        }
        for (int d = 0; d < ndim; ++d)
        {
            fcnml(ifc, d) = -fcnml(ifc, d);
        }
    };
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        double vsum = 0.0;
        int const nfc = clfcs(icl, 0);
        for (int it = 1; it <= nfc; ++it)
        {
            int32_t const ifc = clfcs(icl, it);
            double vol = 0.0;
            for (int d = 0; d < ndim; ++d)
            {
                vol += (fccnd(ifc, d) - clcnd(icl, d)) * fcnml(ifc, d);
            }
            vol *= fcara(ifc);
            bool const own = (fccls(ifc, 0) == icl);
            if (vol < 0.0)
            {
                if (own)
                {
                    reorder_face(ifc);
                }
                vol = -vol;
            }
            else if (!own)
            {
                reorder_face(ifc);
            }
            vsum += vol;
        }
        clvol(icl) = vsum / ndim;
    }
}

void HostMesh::add_bc(std::string const & name, std::vector<int32_t> const & faces)
{
    if (0 != nbound)
    {
        throw std::runtime_error("StaticMesh::add_bc: boundary is already built");
    }
    if (name.empty())
    {
        throw std::invalid_argument("StaticMesh::add_bc: empty name");
    }
    for (auto const & b : bcs)
    {
        if (b.name == name)
        {
            throw std::invalid_argument("StaticMesh::add_bc: duplicated name \"" + name + "\"");
        }
    }
    std::vector<bool> claimed(static_cast<size_t>(nface), false);
    for (auto const & b : bcs)
    {
        for (int64_t i = 0; i < b.nbound(); ++i)
        {
            claimed[b.facn[static_cast<size_t>(i * BFREL)]] = true;
        }
    }
    for (int32_t const ifc : faces)
    {
        if (ifc < 0 || ifc >= nface)
        {
            throw std::invalid_argument("StaticMesh::add_bc: face " + std::to_string(ifc) + " out of range [0, " +
                                        std::to_string(nface) + ")");
        }
        if (fccls(ifc, 1) >= 0)
        {
            throw std::invalid_argument("StaticMesh::add_bc: face " + std::to_string(ifc) + " is not a boundary face");
        }
        if (claimed[ifc])
        {
            throw std::invalid_argument("StaticMesh::add_bc: face " + std::to_string(ifc) + " is already claimed");
        }
        claimed[ifc] = true;
    }
    BcGroup g;
    g.name = name;
    g.facn.assign(faces.size() * BFREL, -1);
    for (size_t i = 0; i < faces.size(); ++i)
    {
        g.facn[i * BFREL] = faces[i];
    }
    bcs.push_back(std::move(g));
}

void HostMesh::build_boundary()
{
    if (0 != nbound)
    {
        throw std::runtime_error("StaticMesh::build_boundary: boundary is already built");
    }
    std::vector<int32_t> allfacn;
    for (int64_t ifc = 0; ifc < nface; ++ifc)
    {
        if (fccls(ifc, 1) < 0)
        {
            allfacn.push_back(static_cast<int32_t>(ifc));
        }
    }
    nbound = static_cast<int64_t>(allfacn.size());
    remake(bndfcs, 0, nbound, BFREL, -1);
    std::vector<int64_t> pos(static_cast<size_t>(nface), -1);
    for (size_t i = 0; i < allfacn.size(); ++i)
    {
        pos[allfacn[i]] = static_cast<int64_t>(i);
    }
    std::vector<bool> specified(allfacn.size(), false);
    int64_t ibfc = 0;
    int64_t nleft = nbound;
    for (size_t ibnd = 0; ibnd < bcs.size(); ++ibnd)
    {
        auto & g = bcs[ibnd];
        for (int64_t k = 0; k < g.nbound(); ++k)
        {
            int32_t const ifc = g.facn[static_cast<size_t>(k * BFREL)];
            bndfcs(ibfc, 0) = ifc;
            bndfcs(ibfc, 1) = static_cast<int32_t>(ibnd);
            g.facn[static_cast<size_t>(k * BFREL + 1)] = static_cast<int32_t>(ibfc);
            if (pos[ifc] >= 0)
            {
                specified[pos[ifc]] = true;
                --nleft;
            }
            ++ibfc;
        }
    }
    if (nleft != 0)
    {
        BcGroup g;
        g.name = "<NONAME>";
        g.facn.assign(static_cast<size_t>(nleft) * BFREL, -1);
        int32_t const ibnd = static_cast<int32_t>(bcs.size());
        int64_t k = 0;
        for (size_t s = 0; s < allfacn.size(); ++s)
        {
            if (!specified[s])
            {
                bndfcs(ibfc, 0) = allfacn[s];
                bndfcs(ibfc, 1) = ibnd;
                g.facn[static_cast<size_t>(k * BFREL)] = allfacn[s];
                g.facn[static_cast<size_t>(k * BFREL + 1)] = static_cast<int32_t>(ibfc);
                ++ibfc;
                ++k;
            }
        }
        bcs.push_back(std::move(g));
    }
}

template <typename T>
void HostMesh::remake(Table<T> & t, int64_t ngst, int64_t nb, int64_t w, T init)
{
    if constexpr (std::is_same_v<T, double>)
        m_retired_real.push_back(std::move(t.buf));
    else
        m_retired_int.push_back(std::move(t.buf));
    t.make(ngst, nb, w, init);
}

template <typename T>
void HostMesh::remake_unset(Table<T> & t, int64_t ngst, int64_t nb, int64_t w)
{
    if constexpr (std::is_same_v<T, double>)
        m_retired_real.push_back(std::move(t.buf));
    else
        m_retired_int.push_back(std::move(t.buf));
    t.make_unset(ngst, nb, w);
}

// Used by the device builder (mesh_device.cu) as well.
template void HostMesh::remake<int32_t>(Table<int32_t> &, int64_t, int64_t, int64_t, int32_t);
template void HostMesh::remake<double>(Table<double> &, int64_t, int64_t, int64_t, double);
template void HostMesh::remake_unset<int32_t>(Table<int32_t> &, int64_t, int64_t, int64_t);
template void HostMesh::remake_unset<double>(Table<double> &, int64_t, int64_t, int64_t);

template <typename T>
void HostMesh::regrow(Table<T> & t, int64_t ngst, T init)
{
    // The ghost rows go first: a new buffer, its ghost rows set to init and
    // the body copied after them, by several threads (one pass over memory
    // instead of a fill and a copy by one thread).
    Table<T> n;
    n.nghost = ngst;
    n.nbody = t.nbody;
    n.width = t.width;
    size_t const head = static_cast<size_t>(ngst * t.width);
    size_t const body = static_cast<size_t>(t.nbody * t.width);
    n.buf.resize(head + body);
    T const * const src = t.buf.data() + static_cast<size_t>(t.nghost * t.width);
    T * const dst = n.buf.data();
    size_t const total = head + body;
    size_t const nthr = std::max<size_t>(
        1, std::min<size_t>(std::thread::hardware_concurrency(), std::min<size_t>(16, total / (1 << 20) + 1)));
    auto work = [&](size_t k) {
        size_t const lo = total * k / nthr;
        size_t const hi = total * (k + 1) / nthr;
        for (size_t i = lo; i < std::min(hi, head); ++i)
        {
            dst[i] = init;
        }
        size_t const b0 = std::max(lo, head);
        if (hi > b0)
        {
            std::copy(src + (b0 - head), src + (hi - head), dst + b0);
        }
    };
    std::vector<std::thread> pool;
    for (size_t k = 1; k < nthr; ++k)
    {
        pool.emplace_back(work, k);
    }
    work(0);
    for (auto & th : pool)
    {
        th.join();
    }
    if constexpr (std::is_same_v<T, double>)
        m_retired_real.push_back(std::move(t.buf));
    else
        m_retired_int.push_back(std::move(t.buf));
    t = std::move(n);
}

void HostMesh::build_ghost()
{
    // count_ghost (StaticMesh_boundary.cpp:248-261).
    int64_t gface = 0, gnode = 0;
    for (int64_t ibfc = 0; ibfc < nbound; ++ibfc)
    {
        int32_t const ifc = bndfcs(ibfc, 0);
        int32_t const icl = fccls(ifc, 0);
        gface += cell_nface(cltpn(icl)) - 1;
        gnode += clnds(icl, 0) - fcnds(ifc, 0);
    }
    ngstnode = gnode;
    ngstface = gface;
    ngstcell = nbound;

    regrow(ndcrd, ngstnode, 0.0);
    regrow(fccnd, ngstface, 0.0);
    regrow(fcnml, ngstface, 0.0);
    regrow(fcara, ngstface, 0.0);
    regrow(clcnd, ngstcell, 0.0);
    regrow(clvol, ngstcell, 0.0);
    regrow(fctpn, ngstface, 0);
    regrow(cltpn, ngstcell, 0);
    regrow(clgrp, ngstcell, -1);
    regrow(fcnds, ngstface, -1);
    regrow(fccls, ngstface, -1);
    regrow(clnds, ngstcell, -1);
    regrow(clfcs, ngstcell, -1);

    fill_ghost();
}

// Mirror each boundary cell across its boundary face into a ghost cell with
// negative ids, then compute the ghost metrics (StaticMesh_boundary.cpp:
// 281-627).
void HostMesh::fill_ghost()
{
    int32_t const nn = static_cast<int32_t>(nnode);
    std::vector<int32_t> gstndmap(static_cast<size_t>(nnode), nn);
    int32_t ignd = -1;
    int32_t igfc = -1;
    for (int32_t igcl = -1; igcl >= -static_cast<int32_t>(ngstcell); --igcl)
    {
        int32_t const ibfc = bndfcs(-igcl - 1, 0);
        int32_t const icl = fccls(ibfc, 0);
        cltpn(igcl) = cltpn(icl);
        clgrp(igcl) = clgrp(icl);
        for (int k = 0; k <= CLMND; ++k)
        {
            clnds(igcl, k) = clnds(icl, k);
        }
        for (int inl = 1; inl <= clnds(icl, 0); ++inl)
        {
            int32_t const ind = clnds(icl, inl);
            bool found = false;
            for (int inf = 1; inf <= fcnds(ibfc, 0); ++inf)
            {
                if (ind == fcnds(ibfc, inf))
                {
                    found = true;
                    break;
                }
            }
            if (!found)
            {
                gstndmap[ind] = ignd;
                clnds(igcl, inl) = ignd;
                double dist = 0.0;
                for (int d = 0; d < ndim; ++d)
                {
                    dist += (fccnd(ibfc, d) - ndcrd(ind, d)) * fcnml(ibfc, d);
                }
                for (int d = 0; d < ndim; ++d)
                {
                    ndcrd(ignd, d) = ndcrd(ind, d) + 2 * dist * fcnml(ibfc, d);
                }
                ignd -= 1;
            }
        }
        fccls(ibfc, 1) = igcl;
        for (int k = 0; k <= CLMFC; ++k)
        {
            clfcs(igcl, k) = clfcs(icl, k);
        }
        for (int ifl = 1; ifl <= clfcs(icl, 0); ++ifl)
        {
            int32_t const ifc = clfcs(icl, ifl);
            if (ifc == ibfc)
            {
                continue;
            }
            fctpn(igfc) = fctpn(ifc);
            fccls(igfc, 0) = igcl;
            clfcs(igcl, ifl) = igfc;
            for (int k = 0; k <= FCMND; ++k)
            {
                fcnds(igfc, k) = fcnds(ifc, k);
            }
            for (int inf = 1; inf <= fcnds(igfc, 0); ++inf)
            {
                int32_t const ind = fcnds(igfc, inf);
                if (gstndmap[ind] != nn)
                {
                    fcnds(igfc, inf) = gstndmap[ind];
                }
            }
            igfc -= 1;
        }
        for (int inl = 1; inl <= clnds(icl, 0); ++inl)
        {
            gstndmap[clnds(icl, inl)] = nn;
        }
    }

    int32_t const ngf = static_cast<int32_t>(ngstface);
    int32_t const ngc = static_cast<int32_t>(ngstcell);
    // Ghost face centroids.
    if (ndim == 2)
    {
        for (int32_t ifc = -1; ifc >= -ngf; --ifc)
        {
            int32_t const a = fcnds(ifc, 1);
            int32_t const b = fcnds(ifc, 2);
            fccnd(ifc, 0) = (ndcrd(a, 0) + ndcrd(b, 0)) / 2;
            fccnd(ifc, 1) = (ndcrd(a, 1) + ndcrd(b, 1)) / 2;
        }
    }
    else
    {
        for (int32_t ifc = -1; ifc >= -ngf; --ifc)
        {
            int const nnd = fcnds(ifc, 0);
            std::array<std::array<double, 3>, FCMND + 2> cfd{};
            for (int inf = 1; inf <= nnd; ++inf)
            {
                int32_t const ind = fcnds(ifc, inf);
                for (int d = 0; d < 3; ++d)
                {
                    cfd[inf][d] = ndcrd(ind, d);
                    cfd[0][d] += ndcrd(ind, d);
                }
            }
            cfd[nnd + 1] = cfd[1];
            for (int d = 0; d < 3; ++d)
            {
                cfd[0][d] /= nnd;
            }
            double voc = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0;
            for (int inf = 1; inf <= nnd; ++inf)
            {
                double const m0 = (cfd[0][0] + cfd[inf][0] + cfd[inf + 1][0]) / 3;
                double const m1 = (cfd[0][1] + cfd[inf][1] + cfd[inf + 1][1]) / 3;
                double const m2 = (cfd[0][2] + cfd[inf][2] + cfd[inf + 1][2]) / 3;
                double const u0 = cfd[inf][0] - cfd[0][0];
                double const u1 = cfd[inf][1] - cfd[0][1];
                double const u2 = cfd[inf][2] - cfd[0][2];
                double const v0 = cfd[inf + 1][0] - cfd[0][0];
                double const v1 = cfd[inf + 1][1] - cfd[0][1];
                double const v2 = cfd[inf + 1][2] - cfd[0][2];
                double const w0 = u1 * v2 - u2 * v1;
                double const w1 = u2 * v0 - u0 * v2;
                double const w2 = u0 * v1 - u1 * v0;
                double const ar = std::sqrt(w0 * w0 + w1 * w1 + w2 * w2);
                c0 += m0 * ar;
                c1 += m1 * ar;
                c2 += m2 * ar;
                voc += ar;
            }
            fccnd(ifc, 0) = c0 / voc;
            fccnd(ifc, 1) = c1 / voc;
            fccnd(ifc, 2) = c2 / voc;
        }
    }
    // Ghost face normals and areas.
    if (ndim == 2)
    {
        for (int32_t ifc = -1; ifc >= -ngf; --ifc)
        {
            int32_t const a = fcnds(ifc, 1);
            int32_t const b = fcnds(ifc, 2);
            double const n0 = ndcrd(b, 1) - ndcrd(a, 1);
            double const n1 = ndcrd(a, 0) - ndcrd(b, 0);
            double const ar = std::sqrt(n0 * n0 + n1 * n1);
            fcara(ifc) = ar;
            fcnml(ifc, 0) = n0 / ar;
            fcnml(ifc, 1) = n1 / ar;
        }
    }
    else
    {
        for (int32_t ifc = -1; ifc >= -ngf; --ifc)
        {
            int const nnd = fcnds(ifc, 0);
            std::array<std::array<double, 3>, FCMND> rv{};
            for (int inf = 0; inf < nnd; ++inf)
            {
                int32_t const ind = fcnds(ifc, inf + 1);
                for (int d = 0; d < 3; ++d)
                {
                    rv[inf][d] = ndcrd(ind, d) - fccnd(ifc, d);
                }
            }
            double n0 = rv[nnd - 1][1] * rv[0][2] - rv[nnd - 1][2] * rv[0][1];
            double n1 = rv[nnd - 1][2] * rv[0][0] - rv[nnd - 1][0] * rv[0][2];
            double n2 = rv[nnd - 1][0] * rv[0][1] - rv[nnd - 1][1] * rv[0][0];
            for (int k = 1; k < nnd; ++k)
            {
                n0 += rv[k - 1][1] * rv[k][2] - rv[k - 1][2] * rv[k][1];
                n1 += rv[k - 1][2] * rv[k][0] - rv[k - 1][0] * rv[k][2];
                n2 += rv[k - 1][0] * rv[k][1] - rv[k - 1][1] * rv[k][0];
            }
            double const ar = std::sqrt(n0 * n0 + n1 * n1 + n2 * n2);
            fcnml(ifc, 0) = n0 / ar;
            fcnml(ifc, 1) = n1 / ar;
            fcnml(ifc, 2) = n2 / ar;
            fcara(ifc) = ar / 2.0;
        }
    }
    // Ghost cell centroids.
    double const frac = (ndim == 2) ? 3.0 : 4.0;
    for (int32_t icl = -1; icl >= -ngc; --icl)
    {
        std::array<double, 3> crd{0.0, 0.0, 0.0};
        int const nnd = clnds(icl, 0);
        for (int inl = 1; inl <= nnd; ++inl)
        {
            int32_t const ind = clnds(icl, inl);
            for (int d = 0; d < ndim; ++d)
            {
                crd[d] += ndcrd(ind, d);
            }
        }
        for (int d = 0; d < ndim; ++d)
        {
            crd[d] /= nnd;
        }
        std::array<double, 3> acc{0.0, 0.0, 0.0};
        double voc = 0.0;
        int const nfc = clfcs(icl, 0);
        for (int ifl = 1; ifl <= nfc; ++ifl)
        {
            int32_t const ifc = clfcs(icl, ifl);
            std::array<double, 3> du{};
            double dot = 0.0;
            for (int d = 0; d < ndim; ++d)
            {
                du[d] = crd[d] - fccnd(ifc, d);
                dot += du[d] * fcnml(ifc, d);
            }
            double const vob = std::fabs(dot * fcara(ifc));
            voc += vob;
            for (int d = 0; d < ndim; ++d)
            {
                acc[d] += (fccnd(ifc, d) + du[d] / frac) * vob;
            }
        }
        for (int d = 0; d < ndim; ++d)
        {
            clcnd(icl, d) = acc[d] / voc;
        }
    }
    // Ghost cell volumes, flipping normals of ghost-owned faces.
    for (int32_t icl = -1; icl >= -ngc; --icl)
    {
        double vsum = 0.0;
        for (int it = 1; it <= clfcs(icl, 0); ++it)
        {
            int32_t const ifc = clfcs(icl, it);
            double vol = 0.0;
            for (int d = 0; d < ndim; ++d)
            {
                vol += (fccnd(ifc, d) - clcnd(icl, d)) * fcnml(ifc, d);
            }
            vol *= fcara(ifc);
            if (vol < 0.0)
            {
                if (fccls(ifc, 0) == icl)
                {
                    for (int d = 0; d < ndim; ++d)
                    {
                        fcnml(ifc, d) = -fcnml(ifc, d);
                    }
                }
                vol = -vol;
            }
            vsum += vol;
        }
        clvol(icl) = vsum / ndim;
    }
}

} // namespace scg
