/*
 * extern "C" entry points of the mesh and multi-dimensional Euler core
 * (declared in include/scg.h).  Each one converts C++ exceptions into a status
 * code plus a thread-local message.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "euler_core.hpp"
#include "mesh_host.hpp"

#include <cstring>
#include <memory>
#include <string>

namespace scg
{

std::atomic<int64_t> g_launches{0};
std::atomic<int64_t> g_device_allocs{0};

namespace
{
thread_local std::string t_last_error;
}

void set_last_error(std::string const & msg) { t_last_error = msg; }
std::string const & last_error() { return t_last_error; }

} // namespace scg


using scg::guarded;

namespace
{

template <typename T>
T * need(T * p, char const * what)
{
    if (!p)
    {
        throw std::invalid_argument(std::string(what) + ": null handle");
    }
    return p;
}

} // namespace

extern "C"
{

const char * scg_last_error(void) { return scg::last_error().c_str(); }

int64_t scg_launch_count(void) { return scg::g_launches.load(); }
int64_t scg_device_alloc_count(void) { return scg::g_device_allocs.load(); }

const char * scg_version(void) { return "solvcon-gb300 0.1"; }

int scg_mesh_create(int ndim, int64_t nnode, int64_t nface, int64_t ncell, scg_mesh ** out)
{
    return guarded([&] {
        need(out, "scg_mesh_create");
        *out = new scg_mesh{scg::HostMesh(ndim, nnode, nface, ncell)};
    });
}

int scg_mesh_from_tables(const int64_t * sizes, const void * const * tables, scg_mesh ** out)
{
    return guarded([&] {
        need(sizes, "scg_mesh_from_tables");
        need(tables, "scg_mesh_from_tables");
        need(out, "scg_mesh_from_tables");
        int64_t const ndim = sizes[0], nnode = sizes[1], nface = sizes[2], ncell = sizes[3], nbound = sizes[4];
        int64_t const ngnode = sizes[5], ngface = sizes[6], ngcell = sizes[7], nedge = sizes[8];
        for (int k = 1; k < 9; ++k)
        {
            if (sizes[k] < 0)
            {
                throw std::invalid_argument("StaticMesh: negative size in scg_mesh_from_tables");
            }
        }
        auto h = std::make_unique<scg_mesh>(scg_mesh{scg::HostMesh(static_cast<int>(ndim), nnode, nface, ncell)});
        scg::HostMesh & m = h->m;
        m.nbound = nbound;
        m.ngstnode = ngnode;
        m.ngstface = ngface;
        m.ngstcell = ngcell;
        int const nd = static_cast<int>(ndim);
        // Shapes after build_ghost (StaticMesh.hpp:434-451): node, face and
        // cell tables carry their ghost rows first.
        auto take = [&](auto & t, int which, int64_t ngst, int64_t nbody, int64_t width) {
            using T = typename std::decay_t<decltype(t.buf)>::value_type;
            t.make_unset(ngst, nbody, width);
            size_t const n = static_cast<size_t>((ngst + nbody) * width);
            if (n == 0)
            {
                return;
            }
            T const * src = static_cast<T const *>(tables[which]);
            if (!src)
            {
                throw std::invalid_argument("scg_mesh_from_tables: table " + std::to_string(which) + " is null");
            }
            std::copy(src, src + n, t.buf.begin());
        };
        take(m.ndcrd, SCG_MESH_NDCRD, ngnode, nnode, nd);
        take(m.fccnd, SCG_MESH_FCCND, ngface, nface, nd);
        take(m.fcnml, SCG_MESH_FCNML, ngface, nface, nd);
        take(m.fcara, SCG_MESH_FCARA, ngface, nface, 1);
        take(m.clcnd, SCG_MESH_CLCND, ngcell, ncell, nd);
        take(m.clvol, SCG_MESH_CLVOL, ngcell, ncell, 1);
        take(m.fctpn, SCG_MESH_FCTPN, ngface, nface, 1);
        take(m.cltpn, SCG_MESH_CLTPN, ngcell, ncell, 1);
        take(m.clgrp, SCG_MESH_CLGRP, ngcell, ncell, 1);
        take(m.fcnds, SCG_MESH_FCNDS, ngface, nface, scg::FCMND + 1);
        take(m.fccls, SCG_MESH_FCCLS, ngface, nface, scg::FCREL);
        take(m.clnds, SCG_MESH_CLNDS, ngcell, ncell, scg::CLMND + 1);
        take(m.clfcs, SCG_MESH_CLFCS, ngcell, ncell, scg::CLMFC + 1);
        take(m.ednds, SCG_MESH_EDNDS, 0, nedge, 2);
        take(m.bndfcs, SCG_MESH_BNDFCS, 0, nbound, scg::BFREL);
        *out = h.release();
    });
}

int scg_mesh_adopt_bc(scg_mesh * mesh, const char * name, const int32_t * facn, int64_t nbound)
{
    return guarded([&] {
        auto & m = need(mesh, "scg_mesh_adopt_bc")->m;
        need(name, "scg_mesh_adopt_bc");
        if (nbound < 0 || (nbound > 0 && !facn))
        {
            throw std::invalid_argument("scg_mesh_adopt_bc: facn must hold nbound rows");
        }
        scg::BcGroup g;
        g.name = name;
        g.facn.assign(facn, facn + nbound * scg::BFREL);
        m.bcs.push_back(std::move(g));
    });
}

int scg_mesh_destroy(scg_mesh * mesh)
{
    return guarded([&] { delete mesh; });
}

int scg_mesh_sizes(const scg_mesh * mesh, int64_t * out)
{
    return guarded([&] {
        auto const & m = need(mesh, "scg_mesh_sizes")->m;
        out[0] = m.ndim;
        out[1] = m.nnode;
        out[2] = m.nface;
        out[3] = m.ncell;
        out[4] = m.nbound;
        out[5] = m.ngstnode;
        out[6] = m.ngstface;
        out[7] = m.ngstcell;
        out[8] = m.ednds.nbody;
        out[9] = static_cast<int64_t>(m.bcs.size());
    });
}

int scg_mesh_array(scg_mesh * mesh, int which, void ** data, int64_t * shape, int * nd, int64_t * nghost, int * dtype)
{
    return guarded([&] {
        auto & m = need(mesh, "scg_mesh_array")->m;
        auto real = [&](scg::Table<double> & t, bool vec) {
            *data = t.data();
            *dtype = 0;
            *nghost = t.nghost;
            shape[0] = t.nghost + t.nbody;
            shape[1] = t.width;
            *nd = vec ? 2 : 1;
        };
        auto integ = [&](scg::Table<int32_t> & t, bool vec) {
            *data = t.data();
            *dtype = 1;
            *nghost = t.nghost;
            shape[0] = t.nghost + t.nbody;
            shape[1] = t.width;
            *nd = vec ? 2 : 1;
        };
        switch (which)
        {
        case SCG_MESH_NDCRD: real(m.ndcrd, true); break;
        case SCG_MESH_FCCND: real(m.fccnd, true); break;
        case SCG_MESH_FCNML: real(m.fcnml, true); break;
        case SCG_MESH_FCARA: real(m.fcara, false); break;
        case SCG_MESH_CLCND: real(m.clcnd, true); break;
        case SCG_MESH_CLVOL: real(m.clvol, false); break;
        case SCG_MESH_FCTPN: integ(m.fctpn, false); break;
        case SCG_MESH_CLTPN: integ(m.cltpn, false); break;
        case SCG_MESH_CLGRP: integ(m.clgrp, false); break;
        case SCG_MESH_FCNDS: integ(m.fcnds, true); break;
        case SCG_MESH_FCCLS: integ(m.fccls, true); break;
        case SCG_MESH_CLNDS: integ(m.clnds, true); break;
        case SCG_MESH_CLFCS: integ(m.clfcs, true); break;
        case SCG_MESH_EDNDS: integ(m.ednds, true); break;
        case SCG_MESH_BNDFCS: integ(m.bndfcs, true); break;
        default: throw std::invalid_argument("StaticMesh: unknown array id " + std::to_string(which));
        }
    });
}

int scg_mesh_build_interior(scg_mesh * mesh, int do_metric, int do_edge)
{
    return guarded([&] { need(mesh, "scg_mesh_build_interior")->m.build_interior(do_metric != 0, do_edge != 0); });
}

int scg_mesh_build_interior_device(scg_mesh * mesh, int do_metric, int do_edge)
{
    return guarded([&]
                   { need(mesh, "scg_mesh_build_interior_device")->m.build_interior_device(do_metric != 0, do_edge != 0); });
}

int scg_device_count(int * out)
{
    return guarded([&] {
        int n = 0;
        *out = cudaGetDeviceCount(&n) == cudaSuccess ? n : 0;
        cudaGetLastError();
    });
}

int scg_mesh_build_edge(scg_mesh * mesh)
{
    return guarded([&] { need(mesh, "scg_mesh_build_edge")->m.build_edge(); });
}

int scg_mesh_add_bc(scg_mesh * mesh, const char * name, const int32_t * faces, int64_t nface)
{
    return guarded([&] {
        std::vector<int32_t> f(faces, faces + nface);
        need(mesh, "scg_mesh_add_bc")->m.add_bc(std::string(name ? name : ""), f);
    });
}

int scg_mesh_bc(const scg_mesh * mesh, int64_t ibc, char * buf, int64_t buflen, int32_t * facn, int64_t * nbound)
{
    return guarded([&] {
        auto const & m = need(mesh, "scg_mesh_bc")->m;
        if (ibc < 0 || ibc >= static_cast<int64_t>(m.bcs.size()))
        {
            throw std::out_of_range("StaticMesh: bc index " + std::to_string(ibc) + " out of range");
        }
        auto const & g = m.bcs[static_cast<size_t>(ibc)];
        if (buf && buflen > 0)
        {
            std::strncpy(buf, g.name.c_str(), static_cast<size_t>(buflen - 1));
            buf[buflen - 1] = '\0';
        }
        *nbound = g.nbound();
        if (facn)
        {
            std::memcpy(facn, g.facn.data(), g.facn.size() * sizeof(int32_t));
        }
    });
}

int scg_mesh_build_boundary(scg_mesh * mesh)
{
    return guarded([&] { need(mesh, "scg_mesh_build_boundary")->m.build_boundary(); });
}

int scg_mesh_build_ghost(scg_mesh * mesh)
{
    return guarded([&] { need(mesh, "scg_mesh_build_ghost")->m.build_ghost(); });
}

int scg_euler_create(const scg_mesh * mesh, double time_increment, int precision, scg_euler ** out)
{
    return guarded([&] {
        auto const & m = need(mesh, "scg_euler_create")->m;
        auto h = std::make_unique<scg_euler>();
        h->c = scg::make_euler_core(m, time_increment, precision);
        *out = h.release();
    });
}

int scg_euler_destroy(scg_euler * core)
{
    return guarded([&] { delete core; });
}

int scg_euler_info(const scg_euler * core, int64_t * out)
{
    return guarded([&] {
        auto const & c = *need(core, "scg_euler_info")->c;
        out[0] = c.ndim;
        out[1] = c.ncell;
        out[2] = c.ngstcell;
        out[3] = c.neq;
        out[4] = c.precision;
    });
}

int scg_euler_get_param(const scg_euler * core, int which, double * value)
{
    return guarded([&] {
        auto const & c = *need(core, "scg_euler_get_param")->c;
        switch (which)
        {
        case SCG_PARAM_SIGMA0: *value = c.sigma0; break;
        case SCG_PARAM_TAUMIN: *value = c.taumin; break;
        case SCG_PARAM_TAUSCALE: *value = c.tauscale; break;
        case SCG_PARAM_TIME_INCREMENT: *value = c.time_increment; break;
        default: throw std::invalid_argument("EulerCore: unknown parameter " + std::to_string(which));
        }
    });
}

int scg_euler_set_param(scg_euler * core, int which, double value)
{
    return guarded([&] {
        auto & c = *need(core, "scg_euler_set_param")->c;
        switch (which)
        {
        case SCG_PARAM_SIGMA0: c.sigma0 = value; break;
        case SCG_PARAM_TAUMIN: c.taumin = value; break;
        case SCG_PARAM_TAUSCALE: c.tauscale = value; break;
        case SCG_PARAM_TIME_INCREMENT: throw std::invalid_argument("EulerCore: time_increment is read-only");
        default: throw std::invalid_argument("EulerCore: unknown parameter " + std::to_string(which));
        }
    });
}

int scg_euler_array_shape(const scg_euler * core, int which, int64_t * shape, int * nd, int64_t * nghost)
{
    return guarded([&] { need(core, "scg_euler_array_shape")->c->array_shape(which, shape, nd, nghost); });
}

int scg_euler_get(scg_euler * core, int which, double * host, int64_t count)
{
    return guarded([&] {
        auto & c = *need(core, "scg_euler_get")->c;
        if (count != c.array_size(which))
        {
            throw std::invalid_argument("EulerCore: host buffer holds " + std::to_string(count) +
                                        " elements, array has " + std::to_string(c.array_size(which)));
        }
        c.get_array(which, host);
    });
}

int scg_euler_set(scg_euler * core, int which, const double * host, int64_t count)
{
    return guarded([&] {
        auto & c = *need(core, "scg_euler_set")->c;
        if (count != c.array_size(which))
        {
            throw std::invalid_argument("EulerCore: host buffer holds " + std::to_string(count) +
                                        " elements, array has " + std::to_string(c.array_size(which)));
        }
        c.set_array(which, host);
    });
}

int scg_euler_init_solution(scg_euler * core, double gamma, double rho, const double * v, int nv, double p)
{
    return guarded([&] {
        auto & c = *need(core, "scg_euler_init_solution")->c;
        if (nv != c.ndim)
        {
            throw std::invalid_argument("EulerCore::init_solution: velocity size " + std::to_string(nv) +
                                        " must equal ndim " + std::to_string(c.ndim));
        }
        double vv[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < nv; ++d)
        {
            vv[d] = v[d];
        }
        c.init_solution(gamma, rho, vv, p);
    });
}

int scg_euler_add_bc(scg_euler * core, int kind, const int32_t * faces, int64_t nface, const double * value,
                     int64_t nvalue)
{
    return guarded([&] {
        std::vector<int32_t> f(faces, faces + nface);
        std::vector<double> v;
        if (value && nvalue > 0)
        {
            v.assign(value, value + nvalue);
        }
        need(core, "scg_euler_add_bc")->c->add_bc(kind, f, v);
    });
}

int scg_euler_clear_bc(scg_euler * core)
{
    return guarded([&] { need(core, "scg_euler_clear_bc")->c->clear_bc(); });
}

int scg_euler_normal_matrix(const scg_euler * core, int32_t ifc, double * out)
{
    return guarded([&] { need(core, "scg_euler_normal_matrix")->c->normal_matrix(ifc, out); });
}

int scg_euler_op(scg_euler * core, int op)
{
    return guarded([&] { need(core, "scg_euler_op")->c->op(op); });
}

int scg_euler_march(scg_euler * core, int64_t steps)
{
    return guarded([&] {
        if (steps < 0)
        {
            throw std::invalid_argument("EulerCore::march: steps must be >= 0");
        }
        need(core, "scg_euler_march")->c->march(steps);
    });
}

int scg_euler_march_from_host(scg_euler * core, const double * so0n, int64_t n0, const double * so1n,
                              int64_t n1, int64_t steps)
{
    return guarded([&] {
        auto * c = need(core, "scg_euler_march_from_host")->c.get();
        if (steps < 0)
        {
            throw std::invalid_argument("EulerCore::march: steps must be >= 0");
        }
        if (!so0n || !so1n)
        {
            throw std::invalid_argument("scg_euler_march_from_host: null table");
        }
        if (n0 != c->array_size(scg::EA_SO0N) || n1 != c->array_size(scg::EA_SO1N))
        {
            throw std::invalid_argument("scg_euler_march_from_host: table sizes " + std::to_string(n0) + ", " +
                                        std::to_string(n1) + " are not so0n's and so1n's");
        }
        c->march_from_host(so0n, so1n, steps);
    });
}

int scg_euler_deliver(scg_euler * core, int which, double * host, int64_t count)
{
    return guarded([&] { need(core, "scg_euler_deliver")->c->deliver(which, host, count); });
}

int scg_euler_sync(scg_euler * core)
{
    return guarded([&] { need(core, "scg_euler_sync")->c->sync(); });
}

int scg_euler_set_stream(scg_euler * core, void * cuda_stream)
{
    return guarded([&] { need(core, "scg_euler_set_stream")->c->set_stream(static_cast<cudaStream_t>(cuda_stream)); });
}

int scg_euler_limiter_mask(scg_euler * core, uint8_t * out)
{
    return guarded([&] { need(core, "scg_euler_limiter_mask")->c->limiter_mask(out); });
}

int scg_euler_totals(scg_euler * core, double * out)
{
    return guarded([&] { need(core, "scg_euler_totals")->c->totals(out); });
}

int scg_euler_cfl_range(scg_euler * core, double * out)
{
    return guarded([&] { need(core, "scg_euler_cfl_range")->c->cfl_range(out); });
}

int scg_euler_field(scg_euler * core, int which, double * out)
{
    return guarded([&] { need(core, "scg_euler_field")->c->field(which, out); });
}

int scg_euler_device_bytes(const scg_euler * core, int64_t * out)
{
    return guarded([&] { *out = static_cast<int64_t>(need(core, "scg_euler_device_bytes")->c->device_bytes()); });
}

int scg_euler_stream(const scg_euler * core, void ** out)
{
    return guarded([&] { *out = need(core, "scg_euler_stream")->c->get_stream(); });
}

int scg_euler_profile(scg_euler * core, int on)
{
    return guarded([&] { need(core, "scg_euler_profile")->c->profile(on != 0); });
}

int scg_euler_profile_stats(scg_euler * core, double * ms_total, int64_t * launches)
{
    return guarded([&] { need(core, "scg_euler_profile_stats")->c->profile_stats(ms_total, launches); });
}

} // extern "C"
