/*
 * GPU spacetime scalar CESE solvers: solvcon's spacetime::SolverBase march
 * (cpp/solvcon/spacetime/core.hpp:946-1036) with the LinearScalar and
 * InviscidBurgers solution-element kernels (kernel/linear_scalar.hpp:45-87,
 * kernel/inviscid_burgers.hpp:51-109), one variable, periodic boundary.
 *
 * Grid layout (core.cpp:52-99): coordinates x[0 .. 2*ncelm+4]; solution
 * element i on plane p sits at x index 2 + 2i + p, conservation element i at
 * 3 + 2i + p.  A half step on plane p computes, for each conservation element
 * ic, so0 then so1 at its top solution element (index 3 + 2ic + p) from its
 * two bottom solution elements (2 + 2ic + p and 4 + 2ic + p), which are all on
 * the other parity: the half step has no dependency between elements.  One
 * thread per conservation element runs so0, the periodic ghost copy, the CFL
 * of the top element and so1 (the order of march_half1_alpha and
 * march_half2_alpha, core.hpp:1006-1025), so a full step is two launches;
 * march_alpha replays a captured CUDA graph of 32 steps.
 */

#include "../../include/scg.h"
#include "common.hpp"

#include <cfloat>
#include <memory>
#include <string>
#include <vector>

namespace
{

struct STArgs
{
    double const * x;
    double * so0;
    double * so1;
    double * cfl;
    int64_t ncelm;
    double hdt, qdt;
};

template <int KIND>
struct Selm
{
    double x, xneg, xpos, u, ux;

    __device__ Selm(STArgs const & a, int64_t xi)
        : x(a.x[xi])
        , xneg(a.x[xi - 1])
        , xpos(a.x[xi + 1])
        , u(a.so0[xi])
        , ux(a.so1[xi])
    {
    }
    __device__ double xctr() const { return (xneg + xpos) / 2; }
    __device__ double dxneg() const { return x - xneg; }
    __device__ double dxpos() const { return xpos - x; }
    __device__ double xn() const { return dxneg() * (u + (0.5 * (x + xneg) - xctr()) * ux); }
    __device__ double xp() const { return dxpos() * (u + (0.5 * (x + xpos) - xctr()) * ux); }
    // Temporal flux of the forward branch (LinearScalarSelm::tp,
    // InviscidBurgersSelm::tp).
    __device__ double tp(STArgs const & a) const
    {
        double const disp = x - xctr();
        if constexpr (KIND == 0)
        {
            double r = u;
            r += disp * ux;
            r -= a.qdt * ux;
            return a.hdt * r;
        }
        else
        {
            double const u2 = u * u;
            double r = 0.5 * u2;
            r += disp * u * ux;
            r -= a.qdt * u2 * ux;
            return a.hdt * r;
        }
    }
    __device__ double so0p(STArgs const & a) const
    {
        double r = u;
        r += (x - xctr()) * ux;
        r -= a.hdt * ux;
        return r;
    }
};

template <int KIND>
__device__ __forceinline__ void cfl_at(STArgs const & a, int64_t xi)
{
    double const dn = a.x[xi] - a.x[xi - 1];
    double const dp = a.x[xi + 1] - a.x[xi];
    double const hdx = dn < dp ? dn : dp;
    if constexpr (KIND == 0)
        a.cfl[xi] = a.hdt / hdx;
    else
        a.cfl[xi] = fabs(a.so0[xi]) * a.hdt / hdx;
}

template <int ALPHA>
__device__ __forceinline__ double wgrad(double duxn, double duxp)
{
    double fan = fabs(duxn), fap = fabs(duxp);
    if constexpr (ALPHA == 2)
    {
        fan *= fan;
        fap *= fap;
    }
    return (fap * duxn + fan * duxp) / (fap + fan + DBL_MIN);
}

// One half step; STAGE bits: 1 so0, 2 cfl of the top element, 4 so1,
// 8 periodic ghost copies (first half only).
template <int KIND, int ALPHA, int STAGE>
__global__ void k_st_half(STArgs a, int odd)
{
    int64_t const ic = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x - (odd ? 1 : 0);
    if (ic >= a.ncelm)
    {
        return;
    }
    int64_t const xn_i = 2 + 2 * ic + odd;
    int64_t const xt = xn_i + 1;
    int64_t const last = 2 * a.ncelm + 1; // selm(ncelm - 1, odd plane)
    Selm<KIND> const sn(a, xn_i);
    Selm<KIND> const sp(a, xn_i + 2);
    double utp;
    if (STAGE & 1)
    {
        double const ll = sn.xp() + sn.tp(a);
        double const ur = sp.xn() - sp.tp(a);
        utp = (ll + ur) / (a.x[xt + 1] - a.x[xt - 1]);
        a.so0[xt] = utp;
        if (STAGE & 8)
        {
            if (xt == last)
                a.so0[1] = utp;
            if (xt == 3)
                a.so0[last + 2] = utp;
        }
    }
    else
    {
        utp = a.so0[xt];
    }
    if (STAGE & 2)
    {
        cfl_at<KIND>(a, xt);
        if (STAGE & 8)
        {
            if (xt == last)
                cfl_at<KIND>(a, 1);
            if (xt == 3)
                cfl_at<KIND>(a, last + 2);
        }
    }
    if (STAGE & 4)
    {
        double const duxn = (utp - sn.so0p(a)) / sn.dxpos();
        double const duxp = (sp.so0p(a) - utp) / sp.dxneg();
        double const g = wgrad<ALPHA>(duxn, duxp);
        a.so1[xt] = g;
        if (STAGE & 8)
        {
            if (xt == last)
                a.so1[1] = g;
            if (xt == 3)
                a.so1[last + 2] = g;
        }
    }
}

template <int KIND>
__global__ void k_st_cfl(STArgs a, int odd)
{
    // update_cfl (core.hpp:962-971): selm(ic, odd) for ic in [-odd, nselm).
    int64_t const ic = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x - (odd ? 1 : 0);
    if (ic <= a.ncelm)
    {
        cfl_at<KIND>(a, 2 + 2 * ic + odd);
    }
}

// treat_boundary_so0 / treat_boundary_so1 (core.hpp:982-1004).
__global__ void k_st_bnd(STArgs a, int which)
{
    double * s = which == 0 ? a.so0 : a.so1;
    int64_t const last = 2 * a.ncelm + 1;
    double const left_in = s[3];
    double const right_in = s[last];
    s[1] = right_in;
    s[last + 2] = left_in;
}

class Spacetime
{
public:
    Spacetime(int kind, double const * xcoord, int64_t ncelm_in, double dt)
        : kind(kind)
        , ncelm(ncelm_in)
    {
        if (kind != 0 && kind != 1)
        {
            throw std::invalid_argument("spacetime: kind must be 0 (linear scalar) or 1 (inviscid Burgers)");
        }
        if (ncelm < 1)
        {
            throw std::invalid_argument("spacetime: ncelm smaller than 1");
        }
        xsize = 2 * ncelm + 5;
        scg::cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        x.alloc(static_cast<size_t>(xsize));
        so0.alloc(static_cast<size_t>(xsize));
        so1.alloc(static_cast<size_t>(xsize));
        cfl.alloc(static_cast<size_t>(xsize));
        put(x.ptr, xcoord);
        std::vector<double> z(static_cast<size_t>(xsize), 0.0);
        put(so0.ptr, z.data());
        put(so1.ptr, z.data());
        put(cfl.ptr, z.data());
        set_dt(dt);
    }

    ~Spacetime()
    {
        if (graph_exec)
            cudaGraphExecDestroy(graph_exec);
        if (stream)
        {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    void set_dt(double dt)
    {
        time_increment = dt;
        if (graph_exec)
        {
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
    }

    STArgs args() { return STArgs{x.ptr, so0.ptr, so1.ptr, cfl.ptr, ncelm, 0.5 * time_increment, 0.25 * time_increment}; }

    double * field(int which)
    {
        switch (which)
        {
        case 0: return x.ptr;
        case 1: return so0.ptr;
        case 2: return so1.ptr;
        case 3: return cfl.ptr;
        default: throw std::invalid_argument("spacetime: unknown array id " + std::to_string(which));
        }
    }

    template <int STAGE>
    void half_t(int alpha, int odd)
    {
        int64_t const n = ncelm + (odd ? 1 : 0);
        unsigned const grid = static_cast<unsigned>((n + 255) / 256);
        if (kind == 0)
        {
            if (alpha == 1)
                k_st_half<0, 1, STAGE><<<grid, 256, 0, stream>>>(args(), odd);
            else
                k_st_half<0, 2, STAGE><<<grid, 256, 0, stream>>>(args(), odd);
        }
        else
        {
            if (alpha == 1)
                k_st_half<1, 1, STAGE><<<grid, 256, 0, stream>>>(args(), odd);
            else
                k_st_half<1, 2, STAGE><<<grid, 256, 0, stream>>>(args(), odd);
        }
        scg::launched(stream, "spacetime_half");
    }

    void step(int alpha)
    {
        half_t<1 | 2 | 4 | 8>(alpha, 0);
        half_t<1 | 2 | 4>(alpha, 1);
    }

    void op(int which, int odd, int alpha)
    {
        switch (which)
        {
        case 0: // update_cfl
        case 5: // setup_march == update_cfl(false)
        {
            int const o = which == 5 ? 0 : odd;
            int64_t const n = ncelm + 1 + o;
            if (kind == 0)
                k_st_cfl<0><<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(args(), o);
            else
                k_st_cfl<1><<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(args(), o);
            scg::launched(stream, "spacetime_cfl");
            break;
        }
        case 1: half_t<1>(alpha, odd); break;
        case 2: half_t<4>(alpha, odd); break;
        case 3:
        case 4:
            k_st_bnd<<<1, 1, 0, stream>>>(args(), which - 3);
            scg::launched(stream, "spacetime_bnd");
            break;
        case 6: // march_half1_alpha
            half_t<1 | 2 | 4 | 8>(alpha, 0);
            break;
        case 7: // march_half2_alpha
            half_t<1 | 2 | 4>(alpha, 1);
            break;
        default: throw std::invalid_argument("spacetime: unknown operation " + std::to_string(which));
        }
        sync();
    }

    void march(int alpha, int64_t steps)
    {
        if (alpha != 1 && alpha != 2)
        {
            throw std::invalid_argument("spacetime: alpha must be 1 or 2");
        }
        int64_t const chunks = steps / GRAPH_STEPS;
        if (chunks > 0)
        {
            if (!graph_exec || graph_alpha != alpha)
            {
                capture(alpha);
            }
            for (int64_t c = 0; c < chunks; ++c)
            {
                scg::cuda_check(cudaGraphLaunch(graph_exec, stream), "cudaGraphLaunch");
                scg::g_launches.fetch_add(2 * GRAPH_STEPS, std::memory_order_relaxed);
            }
        }
        for (int64_t s = chunks * GRAPH_STEPS; s < steps; ++s)
        {
            step(alpha);
        }
    }

    void capture(int alpha)
    {
        sync();
        if (graph_exec)
        {
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        scg::cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "BeginCapture");
        int64_t const before = scg::g_launches.load();
        for (int s = 0; s < GRAPH_STEPS; ++s)
        {
            step(alpha);
        }
        scg::g_launches.store(before);
        scg::cuda_check(cudaStreamEndCapture(stream, &g), "EndCapture");
        scg::cuda_check(cudaGraphInstantiate(&graph_exec, g, 0), "GraphInstantiate");
        cudaGraphDestroy(g);
        graph_alpha = alpha;
    }

    void get(int which, double * host)
    {
        scg::cuda_check(cudaMemcpyAsync(host, field(which), sizeof(double) * static_cast<size_t>(xsize),
                                        cudaMemcpyDeviceToHost, stream),
                        "D2H");
        sync();
    }
    void set(int which, double const * host)
    {
        put(field(which), host);
    }

    void sync() { scg::cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }

    int kind;
    int64_t ncelm, xsize;
    double time_increment = 0.0;
    cudaStream_t stream = nullptr;

private:
    static constexpr int GRAPH_STEPS = 32;

    void put(double * dst, double const * src)
    {
        scg::cuda_check(cudaMemcpyAsync(dst, src, sizeof(double) * static_cast<size_t>(xsize),
                                        cudaMemcpyHostToDevice, stream),
                        "H2D");
        sync();
    }

    scg::DevBuf<double> x, so0, so1, cfl;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_alpha = 0;
};

} // namespace

struct scg_st
{
    std::unique_ptr<Spacetime> c;
};

extern "C"
{

int scg_st_create(int kind, const double * xcoord, int64_t ncelm, double time_increment, scg_st ** out)
{
    return scg::guarded([&] {
        auto h = std::make_unique<scg_st>();
        h->c = std::make_unique<Spacetime>(kind, xcoord, ncelm, time_increment);
        *out = h.release();
    });
}

int scg_st_destroy(scg_st * h)
{
    return scg::guarded([&] { delete h; });
}

int scg_st_set_time_increment(scg_st * h, double time_increment)
{
    return scg::guarded([&] { h->c->set_dt(time_increment); });
}

int scg_st_get(scg_st * h, int which, double * host, int64_t count)
{
    return scg::guarded([&] {
        if (count != h->c->xsize)
            throw std::invalid_argument("spacetime: host buffer size mismatch");
        h->c->get(which, host);
    });
}

int scg_st_set(scg_st * h, int which, const double * host, int64_t count)
{
    return scg::guarded([&] {
        if (count != h->c->xsize)
            throw std::invalid_argument("spacetime: host buffer size mismatch");
        h->c->set(which, host);
    });
}

int scg_st_op(scg_st * h, int op, int odd_plane, int alpha)
{
    return scg::guarded([&] { h->c->op(op, odd_plane, alpha); });
}

int scg_st_march(scg_st * h, int alpha, int64_t steps)
{
    return scg::guarded([&] {
        if (steps < 0)
            throw std::invalid_argument("spacetime: steps must be >= 0");
        h->c->march(alpha, steps);
    });
}

int scg_st_sync(scg_st * h)
{
    return scg::guarded([&] { h->c->sync(); });
}

} // extern "C"
