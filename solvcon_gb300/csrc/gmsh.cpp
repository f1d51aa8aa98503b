/*
 * Gmsh MSH 2.2 (ASCII) reader producing a HostMesh: solvcon's inout::Gmsh
 * (cpp/solvcon/inout/gmsh.hpp:70-285, gmsh.cpp:14-118).
 *
 * The file is a sequence of sections; $MeshFormat, $Nodes and $Elements are
 * required, in that order, with an optional $PhysicalNames before $Nodes
 * (skipped, as the reference does).  Only the elements of the highest
 * dimension present become cells: lower-dimension elements (boundary lines,
 * points) only tag physical groups.  Every node of $Nodes is kept and keeps
 * its 1-based id minus one.  A cell's nodes are the element's corner nodes,
 * reordered into solvcon's order by the element table below; then the mesh
 * runs build_interior (metric and edges), build_boundary and build_ghost.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "mesh_host.hpp"

#include <algorithm>
#include <cstdint>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace
{

// One Gmsh element type: its spatial dimension, solvcon cell type, and where
// each of its first corner nodes goes in the solvcon cell (corner k of the
// Gmsh element is node order[k] of the cell).  The table of
// GmshElementDef::by_id (gmsh.hpp:289-333): which Gmsh types exist, and the
// prism's corner order, define the mesh that is read.
struct ElementType
{
    int id;
    int ndim;
    int cell_type;
    int ncorner;
    int order[8];
};

constexpr ElementType ELEMENT_TYPES[] = {
    // id, dim, cell type, corners, corner order
    {1, 1, scg::CT_LINE, 2, {0, 1}},                      // 2-node line
    {2, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},               // 3-node triangle
    {3, 2, scg::CT_QUAD, 4, {0, 1, 2, 3}},                // 4-node quadrangle
    {4, 3, scg::CT_TET, 4, {0, 1, 2, 3}},                 // 4-node tetrahedron
    {5, 3, scg::CT_HEX, 8, {0, 1, 2, 3, 4, 5, 6, 7}},     // 8-node hexahedron
    {6, 3, scg::CT_PRISM, 6, {0, 2, 1, 3, 5, 4}},         // 6-node prism
    {7, 3, scg::CT_PYRAMID, 5, {0, 1, 2, 3, 4}},          // 5-node pyramid
    {8, 1, scg::CT_LINE, 2, {0, 1}},                      // 3-node line
    {9, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},               // 6-node triangle
    {10, 2, scg::CT_QUAD, 4, {0, 1, 2, 3}},               // 9-node quadrangle
    {11, 3, scg::CT_TET, 4, {0, 1, 2, 3}},                // 10-node tetrahedron
    {12, 3, scg::CT_HEX, 8, {0, 1, 2, 3, 4, 5, 6, 7}},    // 27-node hexahedron
    {13, 3, scg::CT_PRISM, 6, {0, 2, 1, 3, 5, 4}},        // 18-node prism
    {14, 3, scg::CT_PYRAMID, 5, {0, 1, 2, 3, 4}},         // 14-node pyramid
    {15, 0, scg::CT_POINT, 1, {0}},                       // 1-node point
    {16, 2, scg::CT_QUAD, 4, {0, 1, 2, 3}},               // 8-node quadrangle
    {17, 3, scg::CT_HEX, 8, {0, 1, 2, 3, 4, 5, 6, 7}},    // 20-node hexahedron
    {18, 3, scg::CT_PRISM, 6, {0, 2, 1, 3, 5, 4}},        // 15-node prism
    {19, 3, scg::CT_PYRAMID, 5, {0, 1, 2, 3, 4}},         // 13-node pyramid
    {20, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 9-node incomplete triangle
    {21, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 10-node triangle
    {22, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 12-node incomplete triangle
    {23, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 15-node triangle
    {24, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 15-node incomplete triangle
    {25, 2, scg::CT_TRIANGLE, 3, {0, 1, 2}},              // 21-node incomplete triangle
    {26, 1, scg::CT_LINE, 2, {0, 1}},                     // 4-node edge
    {27, 1, scg::CT_LINE, 2, {0, 1}},                     // 5-node edge
    {28, 1, scg::CT_LINE, 2, {0, 1}},                     // 6-node edge
    {29, 3, scg::CT_TET, 4, {0, 1, 2, 3}},                // 20-node tetrahedron
    {30, 3, scg::CT_TET, 4, {0, 1, 2, 3}},                // 35-node tetrahedron
    {31, 3, scg::CT_TET, 4, {0, 1, 2, 3}},                // 56-node tetrahedron
    {92, 3, scg::CT_HEX, 8, {0, 1, 2, 3, 4, 5, 6, 7}},    // 64-node hexahedron
    {93, 3, scg::CT_HEX, 8, {0, 1, 2, 3, 4, 5, 6, 7}},    // 125-node hexahedron
};

// An unknown type reads as a dimension-0 element without nodes, as in the
// reference.
ElementType const & element_type(int id)
{
    static constexpr ElementType NONE = {0, 0, scg::CT_NONE, 0, {0}};
    for (auto const & t : ELEMENT_TYPES)
    {
        if (t.id == id)
        {
            return t;
        }
    }
    return NONE;
}

std::vector<std::string> split(std::string const & line)
{
    std::istringstream is(line);
    std::vector<std::string> out;
    std::string tok;
    while (is >> tok)
    {
        out.push_back(tok);
    }
    return out;
}

struct Element
{
    int ndim;
    int cell_type;
    std::vector<int32_t> nodes; // solvcon order, 0-based
};

class GmshReader
{
public:
    explicit GmshReader(std::string const & data)
    {
        std::string text;
        text.reserve(data.size());
        for (char c : data)
        {
            if (c != '\r')
            {
                text.push_back(c);
            }
        }
        in.str(text);
        bool meta = false, nodes = false, elements = false;
        std::string line;
        while (std::getline(in, line))
        {
            if (line.find('$') == std::string::npos)
            {
                continue;
            }
            // A section keyword out of order, or an unknown one, ends the read.
            if (line == "$MeshFormat" && state == BEGIN)
            {
                read_format();
                meta = true;
            }
            else if (line == "$PhysicalNames" && (state == FORMAT_DONE || state == NAMES_DONE))
            {
                skip_section("$EndPhysicalNames", NAMES_DONE);
            }
            else if (line == "$Nodes" && (state == FORMAT_DONE || state == NAMES_DONE))
            {
                read_nodes();
                nodes = true;
            }
            else if (line == "$Elements" && state == NODES_DONE)
            {
                read_elements();
                elements = true;
            }
            else
            {
                break;
            }
        }
        if (!(meta && nodes && elements))
        {
            throw std::invalid_argument("Incorrect msh file format.");
        }
    }

    scg::HostMesh to_mesh() const
    {
        int topdim = 0;
        for (auto const & e : elems)
        {
            topdim = std::max(topdim, e.ndim);
        }
        if (topdim != 2 && topdim != 3)
        {
            throw std::invalid_argument("Gmsh: the highest element dimension is " + std::to_string(topdim) +
                                        "; a mesh needs 2 or 3");
        }
        int64_t ncell = 0;
        for (auto const & e : elems)
        {
            ncell += e.ndim == topdim ? 1 : 0;
        }
        int64_t const nnode = static_cast<int64_t>(crd.size() / 3);
        scg::HostMesh m(topdim, nnode, 0, ncell);
        for (int64_t i = 0; i < nnode; ++i)
        {
            for (int d = 0; d < topdim; ++d)
            {
                m.ndcrd(i, d) = crd[static_cast<size_t>(i * 3 + d)];
            }
        }
        int64_t icl = 0;
        for (auto const & e : elems)
        {
            if (e.ndim != topdim)
            {
                continue;
            }
            m.cltpn(icl) = e.cell_type;
            m.clnds(icl, 0) = static_cast<int32_t>(e.nodes.size());
            for (size_t k = 0; k < e.nodes.size(); ++k)
            {
                m.clnds(icl, static_cast<int64_t>(k) + 1) = e.nodes[k];
            }
            ++icl;
        }
        m.build_interior(true, true);
        m.build_boundary();
        m.build_ghost();
        return m;
    }

private:
    enum State
    {
        BEGIN,
        FORMAT_DONE,
        NAMES_DONE,
        NODES_DONE,
        ELEMENTS_DONE
    };

    void read_format()
    {
        std::string line;
        while (std::getline(in, line) && line.find('$') == std::string::npos)
        {
            auto const tok = split(line);
            if (tok.empty())
            {
                continue;
            }
            double const ver = std::stod(tok[0]);
            if (ver != 2.2)
            {
                throw std::invalid_argument("solvcon does not support msh file ver " + tok[0] + ".");
            }
        }
        if (line == "$EndMeshFormat")
        {
            state = FORMAT_DONE;
        }
    }

    void skip_section(char const * end, State next)
    {
        std::string line;
        while (std::getline(in, line) && line.find('$') == std::string::npos)
        {
        }
        if (line == end)
        {
            state = next;
        }
    }

    void read_nodes()
    {
        std::string line;
        std::getline(in, line);
        int64_t const nnode = std::stoll(line);
        if (nnode < 0)
        {
            throw std::invalid_argument("Gmsh: negative node count");
        }
        crd.assign(static_cast<size_t>(nnode * 3), 0.0);
        while (std::getline(in, line) && line.find('$') == std::string::npos)
        {
            auto const tok = split(line);
            if (tok.size() < 4)
            {
                continue;
            }
            int64_t const id = std::stoll(tok[0]) - 1;
            if (id < 0 || id >= nnode)
            {
                throw std::out_of_range("Gmsh: node id " + tok[0] + " outside 1.." + std::to_string(nnode));
            }
            for (int d = 0; d < 3; ++d)
            {
                crd[static_cast<size_t>(id * 3 + d)] = std::stod(tok[static_cast<size_t>(1 + d)]);
            }
        }
        if (line == "$EndNodes")
        {
            state = NODES_DONE;
        }
    }

    void read_elements()
    {
        std::string line;
        std::getline(in, line);
        int64_t const nelem = std::stoll(line);
        int64_t const nnode = static_cast<int64_t>(crd.size() / 3);
        elems.reserve(static_cast<size_t>(std::max<int64_t>(nelem, 0)));
        while (static_cast<int64_t>(elems.size()) < nelem && std::getline(in, line) &&
               line.find('$') == std::string::npos)
        {
            auto const tok = split(line);
            if (tok.size() < 3)
            {
                continue;
            }
            ElementType const & t = element_type(std::stoi(tok[1]));
            size_t const first = 3 + static_cast<size_t>(std::stoul(tok[2]));
            if (first + static_cast<size_t>(t.ncorner) > tok.size())
            {
                throw std::invalid_argument("Gmsh: element line with too few nodes: " + line);
            }
            Element e{t.ndim, t.cell_type, std::vector<int32_t>(static_cast<size_t>(t.ncorner), -1)};
            for (int k = 0; k < t.ncorner; ++k)
            {
                int64_t const nd = std::stoll(tok[first + static_cast<size_t>(k)]) - 1;
                if (nd < 0 || nd >= nnode)
                {
                    throw std::out_of_range("Gmsh: element node " + std::to_string(nd + 1) + " outside 1.." +
                                            std::to_string(nnode));
                }
                e.nodes[static_cast<size_t>(t.order[k])] = static_cast<int32_t>(nd);
            }
            elems.push_back(std::move(e));
        }
        if (line == "$EndElements" || static_cast<int64_t>(elems.size()) == nelem)
        {
            state = ELEMENTS_DONE;
        }
    }

    std::istringstream in;
    State state = BEGIN;
    std::vector<double> crd; // [nnode][3]
    std::vector<Element> elems;
};

} // namespace

extern "C"
{

int scg_mesh_from_gmsh(const char * data, int64_t nbyte, scg_mesh ** out)
{
    return scg::guarded([&] {
        if (!data || nbyte < 0 || !out)
        {
            throw std::invalid_argument("scg_mesh_from_gmsh: null argument");
        }
        GmshReader const r(std::string(data, static_cast<size_t>(nbyte)));
        *out = new scg_mesh{r.to_mesh()};
    });
}

} // extern "C"
