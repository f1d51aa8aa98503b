/*
 * Plot3D multi-block structured-grid reader producing a HostMesh of
 * hexahedra: solvcon's inout::Plot3d (cpp/solvcon/inout/plot3d.hpp:22-80,
 * plot3d.cpp:14-155).
 *
 * The file (ASCII) holds the block count, one "ni nj nk" line per block, then
 * for each block the x of all its nodes, then the y, then the z (grid index i
 * fastest).  Each block's nodes keep their order after the previous blocks'
 * nodes; blocks share no nodes.  Every grid cell (i, j, k), i in [1, ni),
 * j in [1, nj), k in [1, nk), becomes one hexahedron whose corners are the
 * grid nodes at the offsets below; then the mesh runs build_interior (metric
 * and edges), build_boundary and build_ghost.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "mesh_host.hpp"

#include <cstdint>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace
{

// Grid offsets (di, dj, dk) of the hexahedron's corners from cell (i, j, k),
// in solvcon's corner order: the x = i - 1 face then the x = i face, each
// around (j, k) (plot3d.cpp:88-96).  The order defines the cells read.
constexpr int HEX_CORNER[8][3] = {{-1, -1, -1}, {-1, 0, -1}, {-1, 0, 0}, {-1, -1, 0},
                                  {0, -1, -1},  {0, 0, -1},  {0, 0, 0},  {0, -1, 0}};

scg::HostMesh read_plot3d(std::string const & data)
{
    std::istringstream in(data);
    std::string line;
    if (!std::getline(in, line))
    {
        throw std::invalid_argument("Plot3d: empty file");
    }
    int64_t const nblock = std::stoll(line);
    if (nblock < 0)
    {
        throw std::invalid_argument("Plot3d: negative block count");
    }
    std::vector<int64_t> ni(static_cast<size_t>(nblock)), nj(ni), nk(ni), offset(ni);
    int64_t nnode = 0, ncell = 0;
    for (int64_t b = 0; b < nblock; ++b)
    {
        if (!std::getline(in, line))
        {
            throw std::invalid_argument("Plot3d: missing block dimensions");
        }
        std::istringstream ls(line);
        int64_t x = 0, y = 0, z = 0;
        if (!(ls >> x >> y >> z) || x < 0 || y < 0 || z < 0)
        {
            throw std::invalid_argument("Plot3d: bad block dimensions: " + line);
        }
        size_t const s = static_cast<size_t>(b);
        ni[s] = x;
        nj[s] = y;
        nk[s] = z;
        offset[s] = nnode;
        nnode += x * y * z;
        if (x > 1 && y > 1 && z > 1)
        {
            ncell += (x - 1) * (y - 1) * (z - 1);
        }
    }
    scg::HostMesh m(3, nnode, 0, ncell);
    for (int64_t b = 0; b < nblock; ++b)
    {
        size_t const s = static_cast<size_t>(b);
        int64_t const size = ni[s] * nj[s] * nk[s];
        for (int d = 0; d < 3; ++d)
        {
            for (int64_t j = 0; j < size; ++j)
            {
                double v = 0.0;
                if (!(in >> v))
                {
                    throw std::invalid_argument("Plot3d: fewer coordinates than the block dimensions need");
                }
                m.ndcrd(offset[s] + j, d) = v;
            }
        }
    }
    int64_t icl = 0;
    for (int64_t b = 0; b < nblock; ++b)
    {
        size_t const s = static_cast<size_t>(b);
        for (int64_t k = 1; k < nk[s]; ++k)
        {
            for (int64_t j = 1; j < nj[s]; ++j)
            {
                for (int64_t i = 1; i < ni[s]; ++i)
                {
                    m.cltpn(icl) = scg::CT_HEX;
                    m.clnds(icl, 0) = 8;
                    for (int v = 0; v < 8; ++v)
                    {
                        int64_t const x = i + HEX_CORNER[v][0];
                        int64_t const y = j + HEX_CORNER[v][1];
                        int64_t const z = k + HEX_CORNER[v][2];
                        m.clnds(icl, v + 1) = static_cast<int32_t>(offset[s] + x + y * ni[s] + z * ni[s] * nj[s]);
                    }
                    ++icl;
                }
            }
        }
    }
    m.build_interior(true, true);
    m.build_boundary();
    m.build_ghost();
    return m;
}

} // namespace

extern "C"
{

int scg_mesh_from_plot3d(const char * data, int64_t nbyte, scg_mesh ** out)
{
    return scg::guarded([&] {
        if (!data || nbyte < 0 || !out)
        {
            throw std::invalid_argument("scg_mesh_from_plot3d: null argument");
        }
        *out = new scg_mesh{read_plot3d(std::string(data, static_cast<size_t>(nbyte)))};
    });
}

} // extern "C"
