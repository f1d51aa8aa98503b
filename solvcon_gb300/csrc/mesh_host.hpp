#pragma once

/*
 * Host-side unstructured mesh with mixed element types and a mirrored ghost
 * layer.  Restates the data model and the build steps of solvcon's StaticMesh
 * (cpp/solvcon/mesh/StaticMesh.hpp:264-456, StaticMesh_interior.cpp,
 * StaticMesh_boundary.cpp) so that every connectivity and metric table comes
 * out identical to the reference's, entry for entry; the GPU march consumes
 * these tables.
 *
 * Storage: every table is one contiguous row-major buffer whose first
 * ngst* rows are the ghost rows, so that row r of entity i is at
 * (i + nghost) * width + r, and ghost entities have negative indices -1, -2,
 * ... exactly as in the reference's SimpleArray with nghost set.
 */

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace scg
{

// Cell type ids (StaticMesh.hpp:35-45).
enum CellTypeId : int32_t
{
    CT_NONE = 0,
    CT_POINT = 1,
    CT_LINE = 2,
    CT_QUAD = 3,
    CT_TRIANGLE = 4,
    CT_HEX = 5,
    CT_TET = 6,
    CT_PRISM = 7,
    CT_PYRAMID = 8,
};

constexpr int FCMND = 4; // max nodes per face
constexpr int CLMND = 8; // max nodes per cell
constexpr int CLMFC = 6; // max faces per cell
constexpr int FCREL = 4; // width of fccls
constexpr int BFREL = 3; // width of bndfcs / facn

// Number of faces of a cell type (CellType::nface, StaticMesh.hpp:74,116-124).
int cell_nface(int32_t type);
// Spatial dimension of a cell type.
int cell_ndim(int32_t type);

struct BcGroup
{
    std::string name;
    // [nbound, BFREL]: face in block, face in bndfcs, related block face.
    std::vector<int32_t> facn;
    int64_t nbound() const { return static_cast<int64_t>(facn.size() / BFREL); }
};

// An allocator whose default construction leaves trivial elements
// uninitialised, so a table can be sized without a first pass of zeros
// (the tables of a 24.6M-cell mesh are ~7 GB; build_ghost re-lays all of
// them out with ghost rows first).
template <typename T>
struct NoInit : std::allocator<T>
{
    template <typename U>
    struct rebind
    {
        using other = NoInit<U>;
    };
    NoInit() = default;
    template <typename U>
    NoInit(NoInit<U> const &) noexcept
    {
    }
    template <typename U>
    void construct(U * p) noexcept
    {
        ::new (static_cast<void *>(p)) U;
    }
    template <typename U, typename... Args>
    void construct(U * p, Args &&... args)
    {
        ::new (static_cast<void *>(p)) U(std::forward<Args>(args)...);
    }
};

template <typename T>
using HostVec = std::vector<T, NoInit<T>>;

template <typename T>
struct Table
{
    HostVec<T> buf;
    int64_t nghost = 0;
    int64_t nbody = 0;
    int64_t width = 1; // product of the trailing extents

    void make(int64_t ngst, int64_t nb, int64_t w, T init)
    {
        nghost = ngst;
        nbody = nb;
        width = w;
        buf.assign(static_cast<size_t>((ngst + nb) * w), init);
    }
    // The same shape with the contents left for the caller to write in full.
    void make_unset(int64_t ngst, int64_t nb, int64_t w)
    {
        nghost = ngst;
        nbody = nb;
        width = w;
        buf.clear();
        buf.resize(static_cast<size_t>((ngst + nb) * w));
    }
    T & operator()(int64_t i, int64_t j = 0) { return buf[static_cast<size_t>((i + nghost) * width + j)]; }
    T const & operator()(int64_t i, int64_t j = 0) const { return buf[static_cast<size_t>((i + nghost) * width + j)]; }
    T * data() { return buf.data(); }
};

class HostMesh
{
public:
    HostMesh(int ndim, int64_t nnode, int64_t nface, int64_t ncell);

    // StaticMesh::build_interior (StaticMesh.hpp:363-374).
    void build_interior(bool do_metric, bool do_edge);
    // The same tables built on the GPU (face extraction, de-duplication and
    // numbering, face-cell relations, metrics; mesh_device.cu), entry for
    // entry equal to build_interior's; edges, when asked for, on the host.
    void build_interior_device(bool do_metric, bool do_edge);
    void build_edge();
    // StaticMesh::add_bc (StaticMesh_boundary.cpp:14-78).
    void add_bc(std::string const & name, std::vector<int32_t> const & faces);
    // StaticMesh::build_boundary (StaticMesh_boundary.cpp:103-182).
    void build_boundary();
    // StaticMesh::build_ghost / fill_ghost (StaticMesh_boundary.cpp:185-627).
    void build_ghost();

    int ndim = 0;
    int64_t nnode = 0, nface = 0, ncell = 0, nbound = 0;
    int64_t ngstnode = 0, ngstface = 0, ngstcell = 0;
    bool use_incenter = false;

    Table<double> ndcrd, fccnd, fcnml, fcara, clcnd, clvol;
    Table<int32_t> fctpn, cltpn, clgrp, fcnds, fccls, clnds, clfcs, ednds, bndfcs;
    std::vector<BcGroup> bcs;

    int32_t fcrcl(int32_t ifc, int32_t icl) const { return fccls(ifc, 0) + fccls(ifc, 1) - icl; }

private:
    // Tables replaced by a build step are kept alive until the mesh is
    // destroyed, because Python views of the previous buffers may still exist
    // (the reference keeps a swapped-out buffer alive through its shared
    // ConcreteBuffer for the same reason).
    template <typename T>
    void remake(Table<T> & t, int64_t ngst, int64_t nb, int64_t w, T init);
    template <typename T>
    void regrow(Table<T> & t, int64_t ngst, T init);
    // remake without the fill, for a table the caller overwrites entirely.
    template <typename T>
    void remake_unset(Table<T> & t, int64_t ngst, int64_t nb, int64_t w);
    std::vector<HostVec<double>> m_retired_real;
    std::vector<HostVec<int32_t>> m_retired_int;

    void validate_cells() const;
    void build_faces_from_cells();
    void calc_metric();
    void fill_ghost();
};

} // namespace scg

// The opaque handle behind scg_mesh* in include/scg.h.
struct scg_mesh
{
    scg::HostMesh m;
};
