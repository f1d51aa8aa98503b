/*
 * Test-only C driver over the reference solvcon sources (oracle/_ref).
 *
 * This file is compiled together with the reference's own mesh, multidim and
 * onedim sources (see oracle/Makefile) into oracle/_ref/libsolvcon_ref.so.
 * It only exists so that the tests and the golden-vector generator can run the
 * reference implementation itself from Python through ctypes.  Nothing in the
 * product links or loads it.
 *
 * Every entry point returns 0 on success and -1 on failure; the message of the
 * last failure is available from ref_last_error().
 */

#include <solvcon/inout/gmsh.hpp>
#include <solvcon/inout/plot3d.hpp>
#include <solvcon/mesh/mesh.hpp>
#include <solvcon/multidim/multidim.hpp>
#include <solvcon/onedim/Euler1DCore.hpp>
#include <solvcon/spacetime/kernel/inviscid_burgers.hpp>
#include <solvcon/spacetime/kernel/linear_scalar.hpp>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

using solvcon::EulerBC;
using solvcon::EulerCore;
using solvcon::SimpleArray;
using solvcon::StaticMesh;
using solvcon::onedim::Euler1DCore;
namespace st = solvcon::spacetime;

namespace
{

thread_local std::string g_err;

struct RefMesh
{
    std::shared_ptr<StaticMesh> mesh;
};

struct RefEuler
{
    std::shared_ptr<EulerCore> core;
};

struct RefEuler1D
{
    std::shared_ptr<Euler1DCore> core;
};

// One of the reference's spacetime scalar solvers: kind 0 LinearScalarSolver,
// kind 1 InviscidBurgersSolver.
struct RefSpacetime
{
    int kind = 0;
    std::shared_ptr<st::LinearScalarSolver> linear;
    std::shared_ptr<st::InviscidBurgersSolver> burgers;

    template <typename F>
    void visit(F && f)
    {
        if (kind == 0) f(*linear);
        else f(*burgers);
    }
};

template <typename F>
int guard(F && f)
{
    try
    {
        f();
        return 0;
    }
    catch (std::exception const & e)
    {
        g_err = e.what();
        return -1;
    }
}

// Copy a SimpleArray's whole buffer (ghost rows first) out or in.
template <typename T>
void copy_out(SimpleArray<T> const & arr, T * out)
{
    std::memcpy(out, arr.data(), arr.nbytes());
}

template <typename T>
void copy_in(SimpleArray<T> & arr, T const * in)
{
    std::memcpy(arr.data(), in, arr.nbytes());
}

SimpleArray<double> * euler_array(EulerCore & c, char const * name)
{
    std::string const n(name);
    if (n == "cevol") return &c.cevol();
    if (n == "cecnd") return &c.cecnd();
    if (n == "sfcnd") return &c.sfcnd();
    if (n == "sfnml") return &c.sfnml();
    if (n == "so0c") return &c.so0c();
    if (n == "so0n") return &c.so0n();
    if (n == "so0t") return &c.so0t();
    if (n == "so1c") return &c.so1c();
    if (n == "so1n") return &c.so1n();
    if (n == "stm") return &c.stm();
    if (n == "cflo") return &c.cflo();
    if (n == "cflc") return &c.cflc();
    if (n == "gamma") return &c.gamma();
    throw std::invalid_argument("unknown euler array " + n);
}

} // namespace

extern "C"
{

char const * ref_last_error() { return g_err.c_str(); }

// ---- StaticMesh -----------------------------------------------------------

int ref_mesh_create(int ndim, int nnode, int ncell, double const * ndcrd, int const * cltpn, int const * clnds, void ** out)
{
    return guard([&]
                 {
        auto m = StaticMesh::construct(static_cast<uint8_t>(ndim), nnode, 0, ncell);
        std::memcpy(m->ndcrd().data(), ndcrd, sizeof(double) * nnode * ndim);
        std::memcpy(m->cltpn().data(), cltpn, sizeof(int) * ncell);
        std::memcpy(m->clnds().data(), clnds, sizeof(int) * ncell * (StaticMesh::CLMND + 1));
        *out = new RefMesh{m}; });
}

int ref_mesh_add_bc(void * h, char const * name, int const * faces, int n)
{
    return guard([&]
                 {
        std::vector<int32_t> f(faces, faces + n);
        static_cast<RefMesh *>(h)->mesh->add_bc(std::string(name), f); });
}

// inout::Gmsh(data).to_block(): the mesh of a Gmsh MSH file's contents.
int ref_gmsh_load(char const * data, long long nbyte, void ** out)
{
    return guard([&]
                 {
        solvcon::inout::Gmsh g(std::string(data, static_cast<size_t>(nbyte)));
        *out = new RefMesh{g.to_block()}; });
}

// inout::Plot3d(data).to_block(): the mesh of a Plot3D file's contents.
int ref_plot3d_load(char const * data, long long nbyte, void ** out)
{
    return guard([&]
                 {
        solvcon::inout::Plot3d p(std::string(data, static_cast<size_t>(nbyte)));
        *out = new RefMesh{p.to_block()}; });
}

// stage: 0 build_interior(do_metric=true, do_edge=true), 1 build_boundary,
// 2 build_ghost
int ref_mesh_build(void * h, int stage)
{
    return guard([&]
                 {
        auto & m = *static_cast<RefMesh *>(h)->mesh;
        if (stage == 0) m.build_interior(true, true);
        else if (stage == 1) m.build_boundary();
        else if (stage == 2) m.build_ghost();
        else throw std::invalid_argument("bad stage"); });
}

// sizes: ndim nnode nface ncell nbound ngstnode ngstface ngstcell nedge nbcs
int ref_mesh_sizes(void * h, long long * out)
{
    return guard([&]
                 {
        auto & m = *static_cast<RefMesh *>(h)->mesh;
        out[0] = m.ndim(); out[1] = m.nnode(); out[2] = m.nface(); out[3] = m.ncell();
        out[4] = m.nbound(); out[5] = m.ngstnode(); out[6] = m.ngstface(); out[7] = m.ngstcell();
        out[8] = m.nedge(); out[9] = static_cast<long long>(m.nbcs()); });
}

// Copies the whole buffer (ghost rows first) of a mesh array.  Returns the
// number of elements in *count when out is null.
int ref_mesh_array(void * h, char const * name, void * out, long long * count)
{
    return guard([&]
                 {
        auto & m = *static_cast<RefMesh *>(h)->mesh;
        std::string const n(name);
        auto handle = [&](auto const & arr)
        {
            *count = static_cast<long long>(arr.size());
            if (out) copy_out(arr, static_cast<typename std::decay_t<decltype(arr)>::value_type *>(out));
        };
        if (n == "ndcrd") handle(m.ndcrd());
        else if (n == "fccnd") handle(m.fccnd());
        else if (n == "fcnml") handle(m.fcnml());
        else if (n == "fcara") handle(m.fcara());
        else if (n == "clcnd") handle(m.clcnd());
        else if (n == "clvol") handle(m.clvol());
        else if (n == "fctpn") handle(m.fctpn());
        else if (n == "cltpn") handle(m.cltpn());
        else if (n == "clgrp") handle(m.clgrp());
        else if (n == "fcnds") handle(m.fcnds());
        else if (n == "fccls") handle(m.fccls());
        else if (n == "clnds") handle(m.clnds());
        else if (n == "clfcs") handle(m.clfcs());
        else if (n == "ednds") handle(m.ednds());
        else if (n == "bndfcs") handle(m.bndfcs());
        else throw std::invalid_argument("unknown mesh array " + n); });
}

void ref_mesh_destroy(void * h) { delete static_cast<RefMesh *>(h); }

// ---- EulerCore ------------------------------------------------------------

int ref_euler_create(void * mh, double dt, void ** out)
{
    return guard([&]
                 { *out = new RefEuler{EulerCore::construct(static_cast<RefMesh *>(mh)->mesh, dt)}; });
}

void ref_euler_destroy(void * h) { delete static_cast<RefEuler *>(h); }

int ref_euler_array(void * h, char const * name, double * out, long long * count)
{
    return guard([&]
                 {
        auto * arr = euler_array(*static_cast<RefEuler *>(h)->core, name);
        *count = static_cast<long long>(arr->size());
        if (out) copy_out(*arr, out); });
}

int ref_euler_set_array(void * h, char const * name, double const * in)
{
    return guard([&]
                 { copy_in(*euler_array(*static_cast<RefEuler *>(h)->core, name), in); });
}

int ref_euler_init(void * h, double gamma, double rho, double const * v, double p)
{
    return guard([&]
                 { static_cast<RefEuler *>(h)->core->init_solution(gamma, rho, {v[0], v[1], v[2]}, p); });
}

int ref_euler_params(void * h, double sigma0, double taumin, double tauscale)
{
    return guard([&]
                 {
        auto & c = *static_cast<RefEuler *>(h)->core;
        c.set_sigma0(sigma0); c.set_taumin(taumin); c.set_tauscale(tauscale); });
}

int ref_euler_add_bc(void * h, int kind, int const * faces, int n, double const * value, int nvalue)
{
    return guard([&]
                 {
        std::vector<int32_t> f(faces, faces + n);
        std::vector<double> v(value, value + nvalue);
        static_cast<RefEuler *>(h)->core->add_bc(static_cast<EulerBC>(kind), f, v); });
}

// op: 0 update, 1 calc_solt, 2 calc_soln, 3 bc_soln, 4 calc_cfl, 5 calc_dsoln,
// 6 bc_dsoln, 7 march_substep
int ref_euler_call(void * h, int op)
{
    return guard([&]
                 {
        auto & c = *static_cast<RefEuler *>(h)->core;
        switch (op)
        {
        case 0: c.update(); break;
        case 1: c.calc_solt(); break;
        case 2: c.calc_soln(); break;
        case 3: c.bc_soln(); break;
        case 4: c.calc_cfl(); break;
        case 5: c.calc_dsoln(); break;
        case 6: c.bc_dsoln(); break;
        case 7: c.march_substep(); break;
        default: throw std::invalid_argument("bad op");
        } });
}

int ref_euler_march(void * h, int steps)
{
    return guard([&]
                 { static_cast<RefEuler *>(h)->core->march(steps); });
}

// ---- Euler1DCore ----------------------------------------------------------

int ref_e1d_create(int ncoord, double dt, void ** out)
{
    return guard([&]
                 { *out = new RefEuler1D{Euler1DCore::construct(static_cast<size_t>(ncoord), dt)}; });
}

void ref_e1d_destroy(void * h) { delete static_cast<RefEuler1D *>(h); }

// which: 0 coord, 1 cfl, 2 so0, 3 so1, 4 gamma
int ref_e1d_array(void * h, int which, double * out, double const * in)
{
    return guard([&]
                 {
        auto & c = *static_cast<RefEuler1D *>(h)->core;
        SimpleArray<double> * a = nullptr;
        switch (which)
        {
        case 0: a = &c.coord(); break;
        case 1: a = &c.cfl(); break;
        case 2: a = &c.so0(); break;
        case 3: a = &c.so1(); break;
        case 4: a = &c.gamma(); break;
        default: throw std::invalid_argument("bad array");
        }
        if (in) copy_in(*a, in);
        if (out) copy_out(*a, out); });
}

// op: 0 setup_march, 1 march_alpha1, 2 march_alpha2
int ref_e1d_march(void * h, int op, int steps)
{
    return guard([&]
                 {
        auto & c = *static_cast<RefEuler1D *>(h)->core;
        if (op == 0) c.setup_march();
        else if (op == 1) c.march_alpha<1>(static_cast<size_t>(steps));
        else if (op == 2) c.march_alpha<2>(static_cast<size_t>(steps));
        else throw std::invalid_argument("bad op"); });
}

// ---- spacetime solvers ----------------------------------------------------

// Grid::construct(xloc) (the CE boundaries, ascending) and the solver of the
// given kind on it (kernel/linear_scalar.hpp:32-42, kernel/inviscid_burgers.hpp:30-45).
int ref_st_create(int kind, double const * xloc, long long nloc, double dt, void ** out)
{
    return guard([&]
                 {
        if (kind != 0 && kind != 1) throw std::invalid_argument("bad solver kind");
        st::Grid::array_type loc(solvcon::small_vector<ssize_t>{static_cast<ssize_t>(nloc)});
        for (long long i = 0; i < nloc; ++i) loc[i] = xloc[i];
        auto grid = st::Grid::construct(loc);
        auto * h = new RefSpacetime;
        h->kind = kind;
        if (kind == 0) h->linear = st::LinearScalarSolver::construct(grid, dt);
        else h->burgers = st::InviscidBurgersSolver::construct(grid, dt);
        *out = h; });
}

void ref_st_destroy(void * h) { delete static_cast<RefSpacetime *>(h); }

// which: 0 xcoord, 1 so0, 2 so1, 3 cfl (whole tables, nvar = 1).  *count
// receives the table's element count; out / in may be null.
int ref_st_array(void * h, int which, double * out, double const * in, long long * count)
{
    return guard([&]
                 {
        static_cast<RefSpacetime *>(h)->visit([&](auto & s)
        {
            SimpleArray<double> * a = nullptr;
            switch (which)
            {
            case 0: a = &s.grid().xcoord(); break;
            case 1: a = &s.so0(); break;
            case 2: a = &s.so1(); break;
            case 3: a = &s.cfl(); break;
            default: throw std::invalid_argument("bad array");
            }
            *count = static_cast<long long>(a->size());
            if (in) copy_in(*a, in);
            if (out) copy_out(*a, out);
        }); });
}

// op: 0 setup_march, 1 march_alpha<1>(steps), 2 march_alpha<2>(steps)
// (core.hpp:804-810, 1029-1036).
int ref_st_march(void * h, int op, long long steps)
{
    return guard([&]
                 {
        static_cast<RefSpacetime *>(h)->visit([&](auto & s)
        {
            if (op == 0) s.setup_march();
            else if (op == 1) s.template march_alpha<1>(static_cast<size_t>(steps));
            else if (op == 2) s.template march_alpha<2>(static_cast<size_t>(steps));
            else throw std::invalid_argument("bad op");
        }); });
}

} // extern "C"
