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
#include "divide.cuh"

#include <cfloat>
#include <memory>
#include <string>
#include <vector>

namespace
{

struct STArgs
{
    double const * x;
    double const * geo; // [G_COUNT][xsize] grid quantities per point
    double * so0;
    double * so1;
    double * cfl;
    int64_t ncelm, xsize;
    double hdt, qdt;
};

// Grid quantities of solution point xi, stored once (k_st_geo) with the very
// expressions the reference evaluates on every half step
// (SolutionElement::xctr/dxneg/dxpos/xn/xp, core.hpp:300-360; the CFL
// half-width and the conservation-element width of
// update_cfl/march_half_so0, core.hpp:962-980), so the march reads them
// instead of recomputing them and its results stay bit-identical.  The four
// divisors of a half step also get their reciprocals (rcp_tab), from which
// div_rcp forms each quotient exactly as the division would.
enum
{
    G_DXNEG = 0, // x - xneg
    G_DXPOS,     // xpos - x
    G_DMNEG,     // 0.5 (x + xneg) - xctr
    G_DMPOS,     // 0.5 (x + xpos) - xctr
    G_DISP,      // x - xctr
    G_HDX,       // min(x - xneg, xpos - x)
    G_WIDTH,     // xpos - xneg (the width of the element whose top is xi)
    G_RDXNEG,    // reciprocals of the four divisors
    G_RDXPOS,
    G_RHDX,
    G_RWIDTH,
    G_CFLLIN,    // the linear solver's CFL number hdt / hdx (set with dt)
    G_COUNT
};

__global__ void k_st_geo(double const * x, int64_t xsize, double * geo)
{
    int64_t const xi = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (xi < 1 || xi >= xsize - 1)
    {
        return;
    }
    double const xm = x[xi - 1], x0 = x[xi], xp = x[xi + 1];
    double const xctr = (xm + xp) / 2;
    double const dn = x0 - xm;
    double const dp = xp - x0;
    geo[G_DXNEG * xsize + xi] = dn;
    geo[G_DXPOS * xsize + xi] = dp;
    geo[G_DMNEG * xsize + xi] = 0.5 * (x0 + xm) - xctr;
    geo[G_DMPOS * xsize + xi] = 0.5 * (x0 + xp) - xctr;
    geo[G_DISP * xsize + xi] = x0 - xctr;
    double const hdx = dn < dp ? dn : dp;
    double const width = xp - xm;
    geo[G_HDX * xsize + xi] = hdx;
    geo[G_WIDTH * xsize + xi] = width;
    geo[G_RDXNEG * xsize + xi] = scg::dev::rcp_tab(dn);
    geo[G_RDXPOS * xsize + xi] = scg::dev::rcp_tab(dp);
    geo[G_RHDX * xsize + xi] = scg::dev::rcp_tab(hdx);
    geo[G_RWIDTH * xsize + xi] = scg::dev::rcp_tab(width);
}

__device__ __forceinline__ double gq(STArgs const & a, int k, int64_t xi) { return a.geo[k * a.xsize + xi]; }

// The parts of solution element xi that the conservation elements on either
// side of it use (LinearScalarSelm / InviscidBurgersSelm, xn, xp, tp, so0p):
// ll = xp + tp (to the element on its right), ur = xn - tp (to the element on
// its left), the value so0p at the next time level and dxneg, dxpos with
// their reciprocals.
template <int KIND>
struct SelmParts
{
    double ll, ur, so0p, dxneg, dxpos, rdxneg, rdxpos;

    __device__ SelmParts(STArgs const & a, int64_t xi)
    {
        double const u = a.so0[xi];
        double const ux = a.so1[xi];
        dxneg = gq(a, G_DXNEG, xi);
        dxpos = gq(a, G_DXPOS, xi);
        rdxneg = gq(a, G_RDXNEG, xi);
        rdxpos = gq(a, G_RDXPOS, xi);
        double const disp = gq(a, G_DISP, xi);
        double const xn = dxneg * (u + gq(a, G_DMNEG, xi) * ux);
        double const xp = dxpos * (u + gq(a, G_DMPOS, xi) * ux);
        double tp;
        if constexpr (KIND == 0)
        {
            double r = u;
            r += disp * ux;
            r -= a.qdt * ux;
            tp = a.hdt * r;
        }
        else
        {
            double const u2 = u * u;
            double r = 0.5 * u2;
            r += disp * u * ux;
            r -= a.qdt * u2 * ux;
            tp = a.hdt * r;
        }
        ll = xp + tp;
        ur = xn - tp;
        double q = u;
        q += disp * ux;
        q -= a.hdt * ux;
        so0p = q;
    }
};

// The linear solver's CFL number at every point, hdt / hdx: it depends on
// the grid and the time increment alone, so it is formed when either is set
// (the same quotient the half step would form) and the half steps copy it.
__global__ void k_st_cfl_tab(double * geo, int64_t xsize, double hdt)
{
    int64_t const xi = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (xi < xsize)
    {
        geo[G_CFLLIN * xsize + xi] = scg::dev::div_rcp(hdt, geo[G_HDX * xsize + xi], geo[G_RHDX * xsize + xi]);
    }
}

template <int KIND>
__device__ __forceinline__ void cfl_at(STArgs const & a, int64_t xi)
{
    if constexpr (KIND == 0)
        a.cfl[xi] = gq(a, G_CFLLIN, xi);
    else
        a.cfl[xi] = scg::dev::div_rcp(fabs(a.so0[xi]) * a.hdt, gq(a, G_HDX, xi), gq(a, G_RHDX, xi));
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

constexpr int BST = 256;

// One half step; STAGE bits: 1 so0, 2 cfl of the top element, 4 so1,
// 8 periodic ghost copies (first half only).  Thread t of a block derives
// the parts of the lower-left solution element of conservation element
// ic = block * BST + t - odd; the element's lower-right solution element is
// the next thread's (or, for the last thread, one extra derived by thread 0),
// shared through shared memory, so each solution element is derived once.
template <int KIND, int ALPHA, int STAGE>
__global__ void __launch_bounds__(BST) k_st_half(STArgs a, int odd)
{
    __shared__ double s_ur[BST + 1];
    __shared__ double s_so0p[BST + 1];
    __shared__ double s_dxneg[BST + 1];
    __shared__ double s_rdxneg[BST + 1];
    int64_t const ic0 = static_cast<int64_t>(blockIdx.x) * BST - (odd ? 1 : 0);
    int64_t const ic = ic0 + threadIdx.x;
    // Solution elements exist for ic <= ncelm (the last one is the
    // lower-right element of conservation element ncelm - 1).
    bool const selm = ic <= a.ncelm;
    double ll = 0.0, so0pn = 0.0, dxposn = 1.0, rdxposn = 1.0;
    if (selm)
    {
        SelmParts<KIND> const sn(a, 2 + 2 * ic + odd);
        ll = sn.ll;
        so0pn = sn.so0p;
        dxposn = sn.dxpos;
        rdxposn = sn.rdxpos;
        s_ur[threadIdx.x] = sn.ur;
        s_so0p[threadIdx.x] = sn.so0p;
        s_dxneg[threadIdx.x] = sn.dxneg;
        s_rdxneg[threadIdx.x] = sn.rdxneg;
    }
    if (threadIdx.x == 0)
    {
        int64_t const ich = ic0 + BST;
        if (ich <= a.ncelm)
        {
            SelmParts<KIND> const sh(a, 2 + 2 * ich + odd);
            s_ur[BST] = sh.ur;
            s_so0p[BST] = sh.so0p;
            s_dxneg[BST] = sh.dxneg;
            s_rdxneg[BST] = sh.rdxneg;
        }
    }
    __syncthreads();
    if (ic >= a.ncelm)
    {
        return;
    }
    int64_t const xt = 3 + 2 * ic + odd;
    int64_t const last = 2 * a.ncelm + 1; // selm(ncelm - 1, odd plane)
    double utp;
    if (STAGE & 1)
    {
        utp = scg::dev::div_rcp(ll + s_ur[threadIdx.x + 1], gq(a, G_WIDTH, xt), gq(a, G_RWIDTH, xt));
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
        double const duxn = scg::dev::div_rcp(utp - so0pn, dxposn, rdxposn);
        double const duxp =
            scg::dev::div_rcp(s_so0p[threadIdx.x + 1] - utp, s_dxneg[threadIdx.x + 1], s_rdxneg[threadIdx.x + 1]);
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
        geo.alloc(static_cast<size_t>(G_COUNT * xsize));
        so0.alloc(static_cast<size_t>(xsize));
        so1.alloc(static_cast<size_t>(xsize));
        cfl.alloc(static_cast<size_t>(xsize));
        put(x.ptr, xcoord);
        make_geo();
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
        make_cfl_tab();
    }

    void make_cfl_tab()
    {
        k_st_cfl_tab<<<static_cast<unsigned>((xsize + 255) / 256), 256, 0, stream>>>(geo.ptr, xsize,
                                                                                     0.5 * time_increment);
        scg::launched(stream, "spacetime_cfl_tab");
        sync();
    }

    STArgs args()
    {
        return STArgs{x.ptr, geo.ptr, so0.ptr, so1.ptr, cfl.ptr, ncelm, xsize, 0.5 * time_increment,
                      0.25 * time_increment};
    }

    // The grid quantities, after the coordinates are set.
    void make_geo()
    {
        scg::cuda_check(cudaMemsetAsync(geo.ptr, 0, geo.bytes(), stream), "memset");
        k_st_geo<<<static_cast<unsigned>((xsize + 255) / 256), 256, 0, stream>>>(x.ptr, xsize, geo.ptr);
        scg::launched(stream, "spacetime_geo");
        make_cfl_tab();
    }

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
        unsigned const grid = static_cast<unsigned>((n + BST - 1) / BST);
        if (kind == 0)
        {
            if (alpha == 1)
                k_st_half<0, 1, STAGE><<<grid, BST, 0, stream>>>(args(), odd);
            else
                k_st_half<0, 2, STAGE><<<grid, BST, 0, stream>>>(args(), odd);
        }
        else
        {
            if (alpha == 1)
                k_st_half<1, 1, STAGE><<<grid, BST, 0, stream>>>(args(), odd);
            else
                k_st_half<1, 2, STAGE><<<grid, BST, 0, stream>>>(args(), odd);
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
        if (which == 0)
        {
            make_geo();
        }
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

    scg::DevBuf<double> x, geo, so0, so1, cfl;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_alpha = 0;
};

// One quotient per thread, by div_rcp from the tabulated reciprocal and by
// the division itself, and the FP64 march's reciprocal of d.
__global__ void k_divide_check(double const * x, double const * d, double * q, double * qdiv, double * rcp,
                               int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        q[i] = scg::dev::div_rcp(x[i], d[i], scg::dev::rcp_tab(d[i]));
        qdiv[i] = x[i] / d[i];
        rcp[i] = scg::dev::recip(d[i]);
    }
}

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

int scg_st_stream(const scg_st * h, void ** out)
{
    return scg::guarded([&] { *out = h->c->stream; });
}

int scg_divide_check(const double * x, const double * d, double * q, double * qdiv, double * rcp, int64_t n)
{
    return scg::guarded([&] {
        if (n < 0 || (n > 0 && (!x || !d || !q || !qdiv || !rcp)))
        {
            throw std::invalid_argument("scg_divide_check: null buffer or negative count");
        }
        if (n == 0)
        {
            return;
        }
        size_t const sz = static_cast<size_t>(n);
        scg::DevBuf<double> dx(sz), dd(sz), dq(sz), dqd(sz), dr(sz);
        scg::cuda_check(cudaMemcpy(dx.ptr, x, dx.bytes(), cudaMemcpyHostToDevice), "H2D");
        scg::cuda_check(cudaMemcpy(dd.ptr, d, dd.bytes(), cudaMemcpyHostToDevice), "H2D");
        k_divide_check<<<static_cast<unsigned>((n + 255) / 256), 256>>>(dx.ptr, dd.ptr, dq.ptr, dqd.ptr, dr.ptr, n);
        scg::launched(nullptr, "divide_check");
        scg::cuda_check(cudaMemcpy(q, dq.ptr, dq.bytes(), cudaMemcpyDeviceToHost), "D2H");
        scg::cuda_check(cudaMemcpy(qdiv, dqd.ptr, dqd.bytes(), cudaMemcpyDeviceToHost), "D2H");
        scg::cuda_check(cudaMemcpy(rcp, dr.ptr, dr.bytes(), cudaMemcpyDeviceToHost), "D2H");
    });
}

} // extern "C"
