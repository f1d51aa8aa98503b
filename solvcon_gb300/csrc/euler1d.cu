/*
 * GPU 1D Euler CESE core: solvcon's onedim::Euler1DCore
 * (cpp/solvcon/onedim/Euler1DCore.hpp:39-349, Euler1DCore.cpp:22-172) on the
 * device.
 *
 * A half step updates the points of one parity from the solution elements
 * ("kernels") at the points of the other parity.  The reference sweeps the
 * points serially with a two-kernel sliding window so that each kernel is
 * derived once; here each thread derives the kernel at one point and shares
 * the quantities its left neighbour needs (flux_lr, up, x - xneg) through
 * shared memory, so each kernel is still derived once per half step.  The
 * first half step also performs the copy-out boundary treatment (it touches
 * only points the half step neither reads nor writes), and update_cfl (which
 * reads only the kernel points) is folded into the same kernel, so a full
 * march_alpha step is two launches.  The fine-grained methods run as separate
 * kernels built from the same device routines.  The FP32 core (Euler1D32,
 * not in the reference) keeps its state split by parity in a layout of its
 * own and updates four outputs per thread; see the comment above it.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "divide.cuh"

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace
{

constexpr int B1D = 256;

// Euler1DKernel::tiny (Euler1DCore.hpp:182) in FP64; it underflows in FP32,
// where the same expressions use the smallest floor that keeps them finite.
template <typename R>
struct Tiny1D;
template <>
struct Tiny1D<double>
{
    static constexpr double V = 1.e-100;
};
template <>
struct Tiny1D<float>
{
    static constexpr float V = 1.e-30f;
};

// The FP64 core's device state: the reference's [n][3] tables.
template <typename R>
struct E1DArgs
{
    double const * coord;
    R const * gamma;
    R * so0; // [n][3]
    R * so1; // [n][3]
    R * cfl;
    int64_t n;
    double hdt, qdt;
    // 1 / (x[i + 1] - x[i]) and 1 / (x[i + 2] - x[i]): the divisions of a
    // half step that depend on the grid alone, formed once per coordinate
    // write by the same expressions (so the same bits) instead of every
    // half step.
    double const * invdx;
    double const * invd2;
    // The solution element's offsets from the grid alone, [5][n]: x - xctr,
    // xpos - x, (x + xpos) / 2 - xctr, x - xneg, (x + xneg) / 2 - xctr with
    // xctr = (xpos + xneg) / 2 (Euler1DCore.hpp:210-244), formed once per
    // coordinate write.
    double const * seo;
};

// The grid's tables of E1DArgs.  The offsets round every operation on its
// own (no contraction), so their bits do not depend on the kernel that
// forms them.
__global__ void k_inv_spacing(double const * coord, int64_t n, double * invdx, double * invd2, double * seo)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        invdx[i] = i + 1 < n ? 1.0 / (coord[i + 1] - coord[i]) : 0.0;
        invd2[i] = i + 2 < n ? 1.0 / (coord[i + 2] - coord[i]) : 0.0;
        double o[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (i > 0 && i + 1 < n)
        {
            double const x = coord[i];
            double const xneg = coord[i - 1];
            double const xpos = coord[i + 1];
            double const xctr = __dmul_rn(__dadd_rn(xpos, xneg), 0.5);
            o[0] = __dsub_rn(x, xctr);
            o[1] = __dsub_rn(xpos, x);
            o[2] = __dsub_rn(__dmul_rn(0.5, __dadd_rn(x, xpos)), xctr);
            o[3] = __dsub_rn(x, xneg);
            o[4] = __dsub_rn(__dmul_rn(0.5, __dadd_rn(x, xneg)), xctr);
        }
        for (int k = 0; k < 5; ++k)
        {
            seo[k * n + i] = o[k];
        }
    }
}

// The solution-element kernel at point ic (Euler1DKernel::set_value and
// derive, Euler1DCore.hpp:193-244): flux f, temporal derivatives ut, ft and
// the value up at the point, plus the two half fluxes of calc_flux_ll/lr
// (Euler1DCore.hpp:246-266).  Reciprocals of rho are formed once: for any
// density above ~1e-50 the reference's denominators rho^k + tiny equal rho^k.
// Its divisions (this one, update_cfl's and the W-alpha weights') multiply
// by scg::dev::recip, a Newton reciprocal within one ulp that takes about
// half the FP64 instructions of a division.
template <typename R>
struct K1D
{
    R r; // 1 / (rho + tiny), shared with update_cfl at the same point
    R up[3];
    R ll[3]; // flux through the lower-left of the CE to the right
    R lr[3]; // flux through the lower-right of the CE to the left
};

template <typename R>
__device__ __forceinline__ void derive(E1DArgs<R> const & a, int64_t ic, K1D<R> & k)
{
    R const ga = a.gamma[ic];
    R u[3], ux[3];
    for (int i = 0; i < 3; ++i)
    {
        u[i] = a.so0[ic * 3 + i];
        ux[i] = a.so1[ic * 3 + i];
    }
    R const r = scg::dev::recip(u[0] + Tiny1D<R>::V);
    k.r = r;
    R const r2 = r * r;
    R const m2r2 = u[1] * u[1] * r2; // u1^2 / u0^2
    R jac[3][3];
    jac[0][0] = R(0);
    jac[0][1] = R(1);
    jac[0][2] = R(0);
    jac[1][0] = (ga - R(3)) / R(2) * m2r2;
    jac[1][1] = -(ga - R(3)) * u[1] * r;
    jac[1][2] = ga - R(1);
    jac[2][0] = (ga - R(1)) * m2r2 * u[1] * r - ga * u[1] * u[2] * r2;
    jac[2][1] = ga * u[2] * r - R(1.5) * (ga - R(1)) * m2r2;
    jac[2][2] = ga * u[1] * r;
    R f[3], ut[3], ft[3];
    f[0] = u[1];
    f[1] = (ga - R(1)) * u[2] + (R(3) - ga) / R(2) * u[1] * u[1] * r;
    f[2] = ga * u[1] * u[2] * r - (ga - R(1)) / R(2) * u[1] * m2r2;
    for (int i = 0; i < 3; ++i)
    {
        ut[i] = -jac[i][0] * ux[0] - jac[i][1] * ux[1] - jac[i][2] * ux[2];
    }
    for (int i = 0; i < 3; ++i)
    {
        ft[i] = jac[i][0] * ut[0] + jac[i][1] * ut[1] + jac[i][2] * ut[2];
    }
    R const hdt = R(a.hdt), qdt = R(a.qdt);
    R const dxctr = R(a.seo[0 * a.n + ic]);
    R const dxl = R(a.seo[1 * a.n + ic]);
    R const dml = R(a.seo[2 * a.n + ic]);
    R const dxr = R(a.seo[3 * a.n + ic]);
    R const dmr = R(a.seo[4 * a.n + ic]);
    for (int i = 0; i < 3; ++i)
    {
        k.up[i] = u[i] + dxctr * ux[i] + hdt * ut[i];
    }
    for (int i = 0; i < 3; ++i)
    {
        R const tf = f[i] - dxctr * ut[i] + qdt * ft[i];
        k.ll[i] = dxl * (u[i] + dml * ux[i]) + hdt * tf;
        k.lr[i] = dxr * (u[i] + dmr * ux[i]) - hdt * tf;
    }
}

// update_cfl at one point (Euler1DCore.cpp:70-94).  The reference's three
// divisions by rho use r = 1 / (rho + tiny), the reciprocal the kernel
// derivation at the same point forms (equal unless rho < ~1e-84, where the
// reference itself overflows).
template <typename R>
__device__ __forceinline__ R rho_recip(E1DArgs<R> const & a, int64_t it)
{
    return scg::dev::recip(a.so0[it * 3 + 0] + Tiny1D<R>::V);
}

__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }

template <typename R>
__device__ __forceinline__ void cfl_at(E1DArgs<R> const & a, int64_t it, double hdt, R r)
{
    R const ga = a.gamma[it];
    R const m = a.so0[it * 3 + 1];
    R const m2 = m * m;
    R const ke = R(0.5) * m2 * r;
    R pr = (ga - R(1)) * (a.so0[it * 3 + 2] - ke);
    pr = (pr + fabs(pr)) / R(2);
    // The reference's sqrt(m * m) is |m| exactly: in binary IEEE arithmetic
    // the square root of a correctly rounded square returns the operand's
    // magnitude (barring overflow or underflow of the square).
    R const wspd = sqrt_r(ga * pr * r) + fabs(m) * r;
    double const dxpos = a.coord[it + 1] - a.coord[it];
    double const dxneg = a.coord[it] - a.coord[it - 1];
    a.cfl[it] = R(hdt) * wspd * scg::dev::recip(R(dxpos < dxneg ? dxpos : dxneg));
}

// The W-alpha gradient (march_half_so1_alpha, Euler1DCore.hpp:284-320).
template <typename R>
__device__ __forceinline__ R wgrad(int alpha, R duxn, R duxp)
{
    R fan = fabs(duxn);
    R fap = fabs(duxp);
    if (alpha == 2)
    {
        fan *= fan;
        fap *= fap;
    }
    return (fap * duxn + fan * duxp) * scg::dev::recip(fap + fan + Tiny1D<R>::V);
}

// What a half step does (k_half's mask): so0, cfl, the copy-out boundary
// treatment, and so1 with the W-alpha weights for alpha = (mask >> 8) > 0.
constexpr unsigned H_SO0 = 1u, H_CFL = 2u, H_BND = 4u;
constexpr unsigned h_alpha(int alpha) { return static_cast<unsigned>(alpha) << 8; }

// Fused half step: so0, cfl and (alpha > 0) so1 at one parity, with the
// copy-out boundary treatment (Euler1DCore.cpp:132-172), each as the mask
// asks.  Output j is point start + 2j + 1 for j < nout; kernels are at
// start + 2j for j <= nout.  The mask is a launch argument, not a template
// parameter: the fine-grained operations (march_half_so0, then
// march_half_so1_alpha on the so0 it stored) and the fused march then run
// the same compiled code and round alike, which the reference requires of
// its two marches; compiled apart, the kernels contracted their
// multiply-adds differently once the divisions became Newton reciprocals.
template <typename R>
__global__ void __launch_bounds__(B1D) k_half(E1DArgs<R> a, int64_t start, int64_t nout, unsigned mask)
{
    {
        int const alpha = static_cast<int>(mask >> 8);
        __shared__ R s_lr[B1D + 1][3];
        __shared__ R s_up[B1D + 1][3];
        __shared__ R s_idxr[B1D + 1]; // 1 / (x - xneg) of each kernel
        int64_t const j0 = static_cast<int64_t>(blockIdx.x) * B1D;
        int64_t const j = j0 + threadIdx.x;
        K1D<R> k;
        bool const have = j <= nout;
        if (have)
        {
            derive(a, start + 2 * j, k);
            for (int i = 0; i < 3; ++i)
            {
                s_lr[threadIdx.x][i] = k.lr[i];
                s_up[threadIdx.x][i] = k.up[i];
            }
            s_idxr[threadIdx.x] = R(a.invdx[start + 2 * j - 1]);
        }
        if (threadIdx.x == 0)
        {
            int64_t const jh = j0 + B1D; // halo kernel on the right
            if (jh <= nout)
            {
                K1D<R> h;
                derive(a, start + 2 * jh, h);
                for (int i = 0; i < 3; ++i)
                {
                    s_lr[B1D][i] = h.lr[i];
                    s_up[B1D][i] = h.up[i];
                }
                s_idxr[B1D] = R(a.invdx[start + 2 * jh - 1]);
            }
        }
        __syncthreads();
        if (have && j < nout)
        {
            int64_t const ic = start + 2 * j;
            R v[3];
            if (mask & H_SO0)
            {
                R const idx = R(a.invd2[ic]);
                for (int i = 0; i < 3; ++i)
                {
                    v[i] = (k.ll[i] + s_lr[threadIdx.x + 1][i]) * idx;
                    a.so0[(ic + 1) * 3 + i] = v[i];
                }
            }
            else
            {
                for (int i = 0; i < 3; ++i)
                {
                    v[i] = a.so0[(ic + 1) * 3 + i];
                }
            }
            if (mask & H_CFL)
            {
                cfl_at(a, ic, a.hdt, k.r);
            }
            if (alpha > 0)
            {
                R const idn = R(a.invdx[ic]);
                R const idp = s_idxr[threadIdx.x + 1];
                for (int i = 0; i < 3; ++i)
                {
                    R const duxn = (v[i] - k.up[i]) * idn;
                    R const duxp = (s_up[threadIdx.x + 1][i] - v[i]) * idp;
                    a.so1[(ic + 1) * 3 + i] = wgrad(alpha, duxn, duxp);
                }
            }
        }
        if ((mask & H_BND) && blockIdx.x == 0 && threadIdx.x == 0)
        {
            int64_t const l = 1, r = a.n - 2;
            for (int i = 0; i < 3; ++i)
            {
                a.so0[l * 3 + i] = a.so0[(l + 1) * 3 + i];
                a.so0[r * 3 + i] = a.so0[(r - 1) * 3 + i];
                a.so1[l * 3 + i] = a.so1[(l + 1) * 3 + i];
                a.so1[r * 3 + i] = a.so1[(r - 1) * 3 + i];
            }
        }

    }
}

// update_cfl alone.
template <typename R>
__global__ void k_cfl1d(E1DArgs<R> a, int64_t start, int64_t nout)
{
    int64_t const j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < nout)
    {
        int64_t const it = start + 2 * j;
        cfl_at(a, it, a.hdt, rho_recip(a, it));
    }
}

// treat_boundary_so0 / treat_boundary_so1.
template <typename R>
__global__ void k_bnd1d(E1DArgs<R> a, int which)
{
    int64_t const l = 1, r = a.n - 2;
    R * s = which == 0 ? a.so0 : a.so1;
    for (int i = 0; i < 3; ++i)
    {
        s[l * 3 + i] = s[(l + 1) * 3 + i];
        s[r * 3 + i] = s[(r - 1) * 3 + i];
    }
}

// What the C ABI calls on a 1D core of either precision.
struct Euler1DBase
{
    virtual ~Euler1DBase() = default;
    virtual std::unique_ptr<Euler1DBase> clone() = 0;
    virtual int64_t count(int which) const = 0;
    virtual void get(int which, double * host) = 0;
    virtual void set(int which, double const * host) = 0;
    virtual void op(int which, int odd, int alpha) = 0;
    virtual void march(int alpha, int64_t steps) = 0;
    virtual void sync() = 0;
    int64_t n = 0;
    double time_increment = 0.0;
    int precision = SCG_FP64;
    cudaStream_t stream = nullptr;
};

// The FP64 core (R = double): the reference's arithmetic on the reference's
// [n][3] device tables.  The FP32 core is Euler1D32 below.
template <typename R>
class Euler1D : public Euler1DBase
{
public:
    Euler1D(int64_t ncoord, double dt)
    {
        n = ncoord;
        time_increment = dt;
        precision = SCG_FP64;
        if (ncoord % 2 == 0)
        {
            throw std::invalid_argument("ncoord cannot be even");
        }
        if (ncoord < 5)
        {
            throw std::invalid_argument("Euler1DCore: ncoord must be at least 5");
        }
        scg::cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        coord.alloc(static_cast<size_t>(n));
        invdx.alloc(static_cast<size_t>(n));
        invd2.alloc(static_cast<size_t>(n));
        seo.alloc(static_cast<size_t>(5 * n));
        for (auto * b : {&cfl, &gamma})
            b->alloc(static_cast<size_t>(n));
        so0.alloc(static_cast<size_t>(n * 3));
        so1.alloc(static_cast<size_t>(n * 3));
        std::vector<double> g(static_cast<size_t>(n), 1.4);
        std::vector<double> z(static_cast<size_t>(n * 3), 0.0);
        set(4, g.data());
        set(0, z.data());
        set(1, z.data());
        set(2, z.data());
        set(3, z.data());
    }

    ~Euler1D() override
    {
        if (graph_exec)
            cudaGraphExecDestroy(graph_exec);
        if (stream)
        {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    std::unique_ptr<Euler1DBase> clone() override
    {
        auto c = std::make_unique<Euler1D<R>>(n, time_increment);
        scg::cuda_check(cudaMemcpyAsync(c->coord.ptr, coord.ptr, sizeof(double) * static_cast<size_t>(n),
                                        cudaMemcpyDeviceToDevice, stream),
                        "copy");
        sync();
        c->spacing();
        for (int k = 1; k < 5; ++k)
        {
            size_t const cnt = static_cast<size_t>(count(k));
            scg::cuda_check(cudaMemcpyAsync(c->state(k), state(k), cnt * sizeof(R), cudaMemcpyDeviceToDevice, stream),
                            "copy");
        }
        sync();
        return c;
    }

    // 0 coord (FP64), 1 cfl, 2 so0, 3 so1, 4 gamma (R)
    R * state(int which)
    {
        switch (which)
        {
        case 1: return cfl.ptr;
        case 2: return so0.ptr;
        case 3: return so1.ptr;
        case 4: return gamma.ptr;
        default: throw std::invalid_argument("Euler1DCore: unknown array id " + std::to_string(which));
        }
    }
    int64_t count(int which) const override { return (which == 2 || which == 3) ? n * 3 : n; }

    void get(int which, double * host) override
    {
        size_t const cnt = static_cast<size_t>(count(which));
        if (which == 0)
        {
            scg::cuda_check(cudaMemcpyAsync(host, coord.ptr, sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream),
                            "D2H");
            sync();
            return;
        }
        scg::cuda_check(cudaMemcpyAsync(host, state(which), sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream),
                        "D2H");
        sync();
    }
    void set(int which, double const * host) override
    {
        size_t const cnt = static_cast<size_t>(count(which));
        if (which == 0)
        {
            put(coord.ptr, host, cnt);
            spacing();
            return;
        }
        put(state(which), host, cnt);
    }

    // The grid's tables (E1DArgs) from the coordinates.
    void spacing()
    {
        k_inv_spacing<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(coord.ptr, n, invdx.ptr, invd2.ptr,
                                                                                   seo.ptr);
        scg::launched(stream, "e1d_inv_spacing");
        sync();
    }

    E1DArgs<R> args()
    {
        return E1DArgs<R>{coord.ptr, gamma.ptr, so0.ptr, so1.ptr, cfl.ptr, n, time_increment / 2.0,
                          time_increment / 4.0, invdx.ptr, invd2.ptr, seo.ptr};
    }

    // Loop bounds of a half step (Euler1DCore.cpp:73-74, 99-100).
    void range(bool odd, int64_t & start, int64_t & nout) const
    {
        start = 2 - (odd ? 1 : 0);
        int64_t const stop = n - 2 - (odd ? 0 : 1);
        nout = stop > start ? (stop - start + 1) / 2 : 0;
    }

    void half(unsigned mask, bool odd)
    {
        int64_t start, nout;
        range(odd, start, nout);
        unsigned const grid = static_cast<unsigned>((nout + B1D) / B1D);
        k_half<R><<<grid, B1D, 0, stream>>>(args(), start, nout, mask);
        scg::launched(stream, "e1d_half");
    }

    void op(int which, int odd, int alpha) override
    {
        switch (which)
        {
        case 0: // update_cfl
        {
            int64_t start, nout;
            range(odd != 0, start, nout);
            if (nout > 0)
            {
                k_cfl1d<R><<<static_cast<unsigned>((nout + 255) / 256), 256, 0, stream>>>(args(), start, nout);
                scg::launched(stream, "e1d_cfl");
            }
            break;
        }
        case 1: // march_half_so0
            half(H_SO0, odd != 0);
            break;
        case 2: // march_half_so1_alpha
            half(h_alpha(alpha == 1 ? 1 : 2), odd != 0);
            break;
        case 3: // treat_boundary_so0
        case 4: // treat_boundary_so1
            k_bnd1d<R><<<1, 1, 0, stream>>>(args(), which - 3);
            scg::launched(stream, "e1d_bnd");
            break;
        case 5: // setup_march
        {
            int64_t start, nout;
            range(false, start, nout);
            if (nout > 0)
            {
                k_cfl1d<R><<<static_cast<unsigned>((nout + 255) / 256), 256, 0, stream>>>(args(), start, nout);
                scg::launched(stream, "e1d_cfl");
            }
            break;
        }
        case 6: // march_half1_alpha: so0, cfl, so1 at the even kernels
            half(H_SO0 | H_CFL | h_alpha(alpha == 1 ? 1 : 2), false);
            break;
        case 7: // march_half2_alpha
            half(H_SO0 | H_CFL | h_alpha(alpha == 1 ? 1 : 2), true);
            break;
        default:
            throw std::invalid_argument("Euler1DCore: unknown operation " + std::to_string(which));
        }
        sync();
    }

    // One march_alpha step (Euler1DCore.hpp:339-349): half 1 with the
    // boundary treatment fused, then half 2.
    void step(int alpha)
    {
        half(H_SO0 | H_CFL | H_BND | h_alpha(alpha), false);
        half(H_SO0 | H_CFL | h_alpha(alpha), true);
    }

    // march_alpha(steps): chunks of GRAPH_STEPS steps replay one captured
    // CUDA graph; the remainder launches directly.
    void march(int alpha, int64_t steps) override
    {
        if (alpha != 1 && alpha != 2)
        {
            throw std::invalid_argument("Euler1DCore: alpha must be 1 or 2");
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
        scg::g_launches.store(before); // captured, not launched
        scg::cuda_check(cudaStreamEndCapture(stream, &g), "EndCapture");
        scg::cuda_check(cudaGraphInstantiate(&graph_exec, g, 0), "GraphInstantiate");
        cudaGraphDestroy(g);
        graph_alpha = alpha;
    }

    void sync() override { scg::cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }

private:
    static constexpr int GRAPH_STEPS = 32;

    template <typename T>
    void put(T * dst, T const * src, size_t cnt)
    {
        scg::cuda_check(cudaMemcpyAsync(dst, src, sizeof(T) * cnt, cudaMemcpyHostToDevice, stream), "H2D");
        sync();
    }

    scg::DevBuf<double> coord;
    scg::DevBuf<double> invdx, invd2, seo; // see E1DArgs
    scg::DevBuf<R> cfl, so0, so1, gamma;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_alpha = 0;
};

// ---------------------------------------------------------------------------
// The FP32 core (not in the reference): FP32 state, cfl and gamma, the
// coordinates kept in FP64 and the spacing between them formed in FP64 and
// rounded once.  It keeps its state in a device layout of its own: every
// quantity split by the parity of the point into two planes (point i -> plane
// i & 1, index i >> 1).  A half step reads the kernel planes of one parity
// and writes the output planes of the other, so every line it fetches is
// used whole, and one thread updates four consecutive outputs with 16-byte
// loads and stores (the planes are padded to a multiple of four).  The host
// sees the reference's [n][3] FP64 tables, converted on the device.

constexpr int B32 = 128;
enum : int
{
    PL_SO0 = 0, // 3 planes: so0 of each variable
    PL_SO1 = 3, // 3 planes: so1
    PL_GAMMA = 6,
    PL_CFL = 7,
    PL_DXM = 8, // x - xneg
    PL_DXP = 9, // xpos - x
    PL_COUNT = 10
};

struct Planes
{
    float * base; // [2][PL_COUNT][P]
    int64_t P;    // plane stride, a multiple of 4
    int64_t n;
    float hdt, qdt;
    __device__ __forceinline__ float * at(int parity, int q) const
    {
        return base + (static_cast<int64_t>(parity) * PL_COUNT + q) * P;
    }
};

// Division in the FP32 core: the approximate quotient (within 2 ulp over the
// normal range; every divisor here is a spacing, a density or a positive sum
// of squares, far inside it).  A correctly rounded FP32 division is a
// multi-instruction sequence, and a half step divides about twelve times per
// output point: 20M-point tube 39.7 -> 88.2 G point-steps/s with it, the
// state within the same bound of the FP64 core as before.
__device__ __forceinline__ float div32(float a, float b) { return __fdividef(a, b); }

// The W-alpha gradient of the FP32 core (wgrad with div32).
template <int ALPHA>
__device__ __forceinline__ float wgrad32(float duxn, float duxp)
{
    float fan = fabsf(duxn);
    float fap = fabsf(duxp);
    if constexpr (ALPHA == 2)
    {
        fan *= fan;
        fap *= fap;
    }
    return div32(fap * duxn + fan * duxp, fap + fan + Tiny1D<float>::V);
}

// The solution-element kernel of one point in FP32 delta form: the state u,
// up - u, and the two half fluxes without their dx * u parts (the caller adds
// those relative to the output point); r = 1 / (rho + tiny) for update_cfl.
struct K32
{
    float u[3], upd[3], llp[3], lrp[3];
    float dm, dp, r, ga;
};

// Euler1DKernel::set_value and derive (Euler1DCore.hpp:193-244) in FP32 from
// the point's state, gamma and spacing dm = x - xneg, dp = xpos - x.
__device__ __forceinline__ void derive32(float const * u, float const * ux, float ga, float dm, float dp, float hdt,
                                         float qdt, K32 & k)
{
    float const r = div32(1.f, u[0] + Tiny1D<float>::V);
    float const r2 = r * r;
    float const m2r2 = u[1] * u[1] * r2;
    float jac[3][3];
    jac[0][0] = 0.f;
    jac[0][1] = 1.f;
    jac[0][2] = 0.f;
    jac[1][0] = (ga - 3.f) / 2.f * m2r2;
    jac[1][1] = -(ga - 3.f) * u[1] * r;
    jac[1][2] = ga - 1.f;
    jac[2][0] = (ga - 1.f) * m2r2 * u[1] * r - ga * u[1] * u[2] * r2;
    jac[2][1] = ga * u[2] * r - 1.5f * (ga - 1.f) * m2r2;
    jac[2][2] = ga * u[1] * r;
    float f[3], ut[3], ft[3];
    f[0] = u[1];
    f[1] = (ga - 1.f) * u[2] + (3.f - ga) / 2.f * u[1] * u[1] * r;
    f[2] = ga * u[1] * u[2] * r - (ga - 1.f) / 2.f * u[1] * m2r2;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        ut[i] = -jac[i][0] * ux[0] - jac[i][1] * ux[1] - jac[i][2] * ux[2];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        ft[i] = jac[i][0] * ut[0] + jac[i][1] * ut[1] + jac[i][2] * ut[2];
    }
    // x - xctr = (dm - dp) / 2, and the BCE midpoints sit at dm / 2 and
    // -dp / 2 from the centre.
    float const dxctr = 0.5f * (dm - dp);
    float const dml = 0.5f * dm;
    float const dmr = -0.5f * dp;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        k.u[i] = u[i];
        k.upd[i] = dxctr * ux[i] + hdt * ut[i];
        float const tf = f[i] - dxctr * ut[i] + qdt * ft[i];
        k.llp[i] = dp * dml * ux[i] + hdt * tf;
        k.lrp[i] = dm * dmr * ux[i] - hdt * tf;
    }
    k.dm = dm;
    k.dp = dp;
    k.r = r;
    k.ga = ga;
}

// update_cfl at a kernel point (Euler1DCore.cpp:70-94) from its derivation.
__device__ __forceinline__ float cfl32(K32 const & k, float hdt)
{
    float const m = k.u[1];
    float const ke = 0.5f * m * m * k.r;
    float pr = (k.ga - 1.f) * (k.u[2] - ke);
    pr = (pr + fabsf(pr)) / 2.f;
    float const wspd = sqrtf(k.ga * pr * k.r) + fabsf(m) * k.r;
    return div32(hdt * wspd, k.dp < k.dm ? k.dp : k.dm);
}

__device__ __forceinline__ float lane(float4 v, int i)
{
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// One half step of the FP32 core, outputs of parity Q from the kernels of the
// other parity.  Output o (1 <= o <= nout) sits between its left and right
// kernels: kernel indices o and o + 1 when the outputs are odd points (the
// first half step), o - 1 and o when they are even.  Thread t updates outputs
// 4t .. 4t + 3 from the four kernels at the same indices (16-byte loads) and
// one more (the next index or the previous one), each derived once per
// thread.  DO_SO0: the new so0 in delta form (each output's old value plus a
// change formed from the kernels' states relative to it, so FP32 rounding
// scales with the change); without it so0 is already new and only so1 is
// formed.  ALPHA > 0: so1 by the W-alpha gradient.  DO_CFL: update_cfl at
// each output's left kernel.  BND: the copy-out boundary treatment of points
// 1 and n - 2, which the half step neither reads nor writes.
template <int ALPHA, bool DO_SO0, bool DO_CFL, bool BND, int Q>
__global__ void __launch_bounds__(B32) k_half32(Planes a, int64_t nout)
{
    constexpr int P = 1 - Q; // parity of the kernels
    if (BND && blockIdx.x == 0 && threadIdx.x == 0)
    {
        int64_t const hi = (a.n - 3) / 2;
        for (int v = 0; v < 3; ++v)
        {
            a.at(1, PL_SO0 + v)[0] = a.at(0, PL_SO0 + v)[1];
            a.at(1, PL_SO0 + v)[hi] = a.at(0, PL_SO0 + v)[hi];
            a.at(1, PL_SO1 + v)[0] = a.at(0, PL_SO1 + v)[1];
            a.at(1, PL_SO1 + v)[hi] = a.at(0, PL_SO1 + v)[hi];
        }
    }
    int64_t const c = 4 * (static_cast<int64_t>(blockIdx.x) * B32 + threadIdx.x);
    if (c > nout)
    {
        return;
    }
    // The five kernels in index order: Q = 1 uses c .. c + 4, Q = 0 uses
    // c - 1 .. c + 3; the one outside the aligned four is the halo.
    int64_t const h = Q == 1 ? c + 4 : c - 1;
    // Index -1 (thread 0 of the second half step) serves only output 0,
    // which is not written: read kernel 0 in its place.
    int64_t const hc = h < 0 ? 0 : h;
    float4 const g4 = *reinterpret_cast<float4 const *>(a.at(P, PL_GAMMA) + c);
    float4 const m4 = *reinterpret_cast<float4 const *>(a.at(P, PL_DXM) + c);
    float4 const p4 = *reinterpret_cast<float4 const *>(a.at(P, PL_DXP) + c);
    float4 u4[3], x4[3];
    float hu[3], hx[3];
#pragma unroll
    for (int v = 0; v < 3; ++v)
    {
        u4[v] = *reinterpret_cast<float4 const *>(a.at(P, PL_SO0 + v) + c);
        x4[v] = *reinterpret_cast<float4 const *>(a.at(P, PL_SO1 + v) + c);
        hu[v] = a.at(P, PL_SO0 + v)[hc];
        hx[v] = a.at(P, PL_SO1 + v)[hc];
    }
    float const hg = a.at(P, PL_GAMMA)[hc];
    float const hm = a.at(P, PL_DXM)[hc];
    float const hp = a.at(P, PL_DXP)[hc];
    // Kernel s (0 .. 4) in index order, derived.
    auto kernel = [&](int s, K32 & k) {
        float u[3], x[3], ga, dm, dp;
        int const l = Q == 1 ? s : s - 1; // lane of the aligned four, or the halo
        if (l < 0 || l > 3)
        {
            for (int v = 0; v < 3; ++v)
            {
                u[v] = hu[v];
                x[v] = hx[v];
            }
            ga = hg;
            dm = hm;
            dp = hp;
        }
        else
        {
            for (int v = 0; v < 3; ++v)
            {
                u[v] = lane(u4[v], l);
                x[v] = lane(x4[v], l);
            }
            ga = lane(g4, l);
            dm = lane(m4, l);
            dp = lane(p4, l);
        }
        derive32(u, x, ga, dm, dp, a.hdt, a.qdt, k);
    };
    // The outputs' so0: their old values (DO_SO0) or the new ones.
    float4 o4[3];
#pragma unroll
    for (int v = 0; v < 3; ++v)
    {
        o4[v] = *reinterpret_cast<float4 const *>(a.at(Q, PL_SO0 + v) + c);
    }
    float nso0[3][4], nso1[3][4], ncfl[4];
    K32 L; // the left kernel of output k; R its right one
    kernel(0, L);
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        K32 R;
        kernel(k + 1, R);
        float const dxl = L.dp;
        float const dxr = R.dm;
        float const idx = div32(1.f, dxl + dxr);
#pragma unroll
        for (int v = 0; v < 3; ++v)
        {
            float const u0 = lane(o4[v], k);
            float d;
            if constexpr (DO_SO0)
            {
                d = (dxl * (L.u[v] - u0) + dxr * (R.u[v] - u0) + L.llp[v] + R.lrp[v]) * idx;
                nso0[v][k] = u0 + d;
            }
            else
            {
                d = 0.f; // u0 is the new value already
                nso0[v][k] = u0;
            }
            if constexpr (ALPHA > 0)
            {
                // The gradient's differences v - up_l and up_r - v from small
                // terms: (u0 - u_l) + d - (up_l - u_l), (u_r - u0) + (up_r - u_r) - d.
                float const duxn = div32((u0 - L.u[v]) + d - L.upd[v], dxl);
                float const duxp = div32((R.u[v] - u0) + R.upd[v] - d, dxr);
                nso1[v][k] = wgrad32<ALPHA>(duxn, duxp);
            }
        }
        if constexpr (DO_CFL)
        {
            ncfl[k] = cfl32(L, a.hdt);
        }
        L = R;
    }
    bool const whole = c >= 1 && c + 3 <= nout;
#pragma unroll
    for (int v = 0; v < 3; ++v)
    {
        float * const s0 = a.at(Q, PL_SO0 + v) + c;
        float * const s1 = a.at(Q, PL_SO1 + v) + c;
        if (whole)
        {
            if constexpr (DO_SO0)
            {
                *reinterpret_cast<float4 *>(s0) = make_float4(nso0[v][0], nso0[v][1], nso0[v][2], nso0[v][3]);
            }
            if constexpr (ALPHA > 0)
            {
                *reinterpret_cast<float4 *>(s1) = make_float4(nso1[v][0], nso1[v][1], nso1[v][2], nso1[v][3]);
            }
        }
        else
        {
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                if (c + k >= 1 && c + k <= nout)
                {
                    if constexpr (DO_SO0)
                    {
                        s0[k] = nso0[v][k];
                    }
                    if constexpr (ALPHA > 0)
                    {
                        s1[k] = nso1[v][k];
                    }
                }
            }
        }
    }
    if constexpr (DO_CFL)
    {
        // The left kernel of output o is kernel o (Q = 1) or o - 1 (Q = 0).
        float * const cf = a.at(P, PL_CFL) + c - (Q == 1 ? 0 : 1);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            if (c + k >= 1 && c + k <= nout)
            {
                cf[k] = ncfl[k];
            }
        }
    }
}

// update_cfl alone at count kernel points of one parity from index i0.
__global__ void k_cfl32(Planes a, int parity, int64_t i0, int64_t count)
{
    int64_t const j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= count)
    {
        return;
    }
    int64_t const i = i0 + j;
    float u[3], x[3];
    for (int v = 0; v < 3; ++v)
    {
        u[v] = a.at(parity, PL_SO0 + v)[i];
        x[v] = a.at(parity, PL_SO1 + v)[i];
    }
    K32 k;
    derive32(u, x, a.at(parity, PL_GAMMA)[i], a.at(parity, PL_DXM)[i], a.at(parity, PL_DXP)[i], a.hdt, a.qdt, k);
    a.at(parity, PL_CFL)[i] = cfl32(k, a.hdt);
}

// treat_boundary_so0 / so1: points 1 and n - 2 from points 2 and n - 3.
__global__ void k_bnd32(Planes a, int q0)
{
    int64_t const hi = (a.n - 3) / 2;
    for (int v = 0; v < 3; ++v)
    {
        a.at(1, q0 + v)[0] = a.at(0, q0 + v)[1];
        a.at(1, q0 + v)[hi] = a.at(0, q0 + v)[hi];
    }
}

// Host table <-> planes.  Table t[i * width + v] of point i (width 3 for so0
// and so1, 1 for cfl and gamma) goes to plane q0 + v of parity i & 1 at
// index i >> 1.
__global__ void k_planes_from_f64(Planes a, int q0, int width, double const * t)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < a.n)
    {
        for (int v = 0; v < width; ++v)
        {
            a.at(static_cast<int>(i & 1), q0 + v)[i >> 1] = float(t[i * width + v]);
        }
    }
}

__global__ void k_planes_to_f64(Planes a, int q0, int width, double * t)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < a.n)
    {
        for (int v = 0; v < width; ++v)
        {
            t[i * width + v] = double(a.at(static_cast<int>(i & 1), q0 + v)[i >> 1]);
        }
    }
}

// The spacing planes from the FP64 coordinates, rounded once (zero where a
// neighbour is missing).
__global__ void k_planes_spacing(Planes a, double const * coord)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < a.n)
    {
        int const p = static_cast<int>(i & 1);
        a.at(p, PL_DXM)[i >> 1] = i > 0 ? float(coord[i] - coord[i - 1]) : 0.f;
        a.at(p, PL_DXP)[i >> 1] = i + 1 < a.n ? float(coord[i + 1] - coord[i]) : 0.f;
    }
}

class Euler1D32 : public Euler1DBase
{
public:
    Euler1D32(int64_t ncoord, double dt)
    {
        n = ncoord;
        time_increment = dt;
        precision = SCG_FP32;
        if (ncoord % 2 == 0)
        {
            throw std::invalid_argument("ncoord cannot be even");
        }
        if (ncoord < 5)
        {
            throw std::invalid_argument("Euler1DCore: ncoord must be at least 5");
        }
        scg::cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        coord.alloc(static_cast<size_t>(n));
        // Each plane holds (n + 1) / 2 points plus room for the last thread's
        // 16-byte accesses past the end.
        P = (((n + 1) / 2 + 8) + 3) / 4 * 4;
        planes.alloc(static_cast<size_t>(2 * PL_COUNT * P));
        scg::cuda_check(cudaMemsetAsync(planes.ptr, 0, planes.bytes(), stream), "memset");
        std::vector<double> g(static_cast<size_t>(n), 1.4);
        set(4, g.data());
        std::vector<double> z(static_cast<size_t>(n), 0.0);
        set(0, z.data());
    }

    ~Euler1D32() override
    {
        if (graph_exec)
            cudaGraphExecDestroy(graph_exec);
        if (stream)
        {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    std::unique_ptr<Euler1DBase> clone() override
    {
        auto c = std::make_unique<Euler1D32>(n, time_increment);
        scg::cuda_check(cudaMemcpyAsync(c->coord.ptr, coord.ptr, sizeof(double) * static_cast<size_t>(n),
                                        cudaMemcpyDeviceToDevice, stream),
                        "copy");
        scg::cuda_check(cudaMemcpyAsync(c->planes.ptr, planes.ptr, planes.bytes(), cudaMemcpyDeviceToDevice, stream),
                        "copy");
        sync();
        return c;
    }

    Planes args() const
    {
        return Planes{planes.ptr, P, n, float(time_increment / 2.0), float(time_increment / 4.0)};
    }

    int64_t count(int which) const override { return (which == 2 || which == 3) ? n * 3 : n; }

    // 1 cfl, 2 so0, 3 so1, 4 gamma -> first plane and width.
    static void plane_of(int which, int & q0, int & width)
    {
        switch (which)
        {
        case 1: q0 = PL_CFL; width = 1; break;
        case 2: q0 = PL_SO0; width = 3; break;
        case 3: q0 = PL_SO1; width = 3; break;
        case 4: q0 = PL_GAMMA; width = 1; break;
        default: throw std::invalid_argument("Euler1DCore: unknown array id " + std::to_string(which));
        }
    }

    void get(int which, double * host) override
    {
        size_t const cnt = static_cast<size_t>(count(which));
        if (which == 0)
        {
            scg::cuda_check(cudaMemcpyAsync(host, coord.ptr, sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream),
                            "D2H");
            sync();
            return;
        }
        int q0, width;
        plane_of(which, q0, width);
        unsigned const grid = static_cast<unsigned>((n + 255) / 256);
        if (double * const dev = static_cast<double *>(scg::mapped_host(host, sizeof(double) * cnt)))
        {
            k_planes_to_f64<<<grid, 256, 0, stream>>>(args(), q0, width, dev);
            scg::launched(stream, "e1d_planes_to_f64");
        }
        else
        {
            double * const tmp = staging(cnt);
            k_planes_to_f64<<<grid, 256, 0, stream>>>(args(), q0, width, tmp);
            scg::launched(stream, "e1d_planes_to_f64");
            scg::cuda_check(cudaMemcpyAsync(host, tmp, sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream), "D2H");
        }
        sync();
    }

    void set(int which, double const * host) override
    {
        size_t const cnt = static_cast<size_t>(count(which));
        unsigned const grid = static_cast<unsigned>((n + 255) / 256);
        if (which == 0)
        {
            scg::cuda_check(cudaMemcpyAsync(coord.ptr, host, sizeof(double) * cnt, cudaMemcpyHostToDevice, stream),
                            "H2D");
            k_planes_spacing<<<grid, 256, 0, stream>>>(args(), coord.ptr);
            scg::launched(stream, "e1d_planes_spacing");
            sync();
            return;
        }
        int q0, width;
        plane_of(which, q0, width);
        if (double const * const dev = static_cast<double const *>(scg::mapped_host(host, sizeof(double) * cnt)))
        {
            k_planes_from_f64<<<grid, 256, 0, stream>>>(args(), q0, width, dev);
            scg::launched(stream, "e1d_planes_from_f64");
        }
        else
        {
            double * const tmp = staging(cnt);
            scg::cuda_check(cudaMemcpyAsync(tmp, host, sizeof(double) * cnt, cudaMemcpyHostToDevice, stream), "H2D");
            k_planes_from_f64<<<grid, 256, 0, stream>>>(args(), q0, width, tmp);
            scg::launched(stream, "e1d_planes_from_f64");
        }
        sync();
    }

    // Grow-only device table for FP64 host data on its way to or from the
    // planes.
    double * staging(size_t cnt)
    {
        if (m_staging.n < cnt)
        {
            sync();
            m_staging.alloc(cnt);
        }
        return m_staging.ptr;
    }

    // Outputs of a half step (Euler1DCore.cpp:97-100): odd = false writes the
    // odd points 3 .. n - 4, odd = true the even points 2 .. n - 3; either
    // way indices 1 .. nout of the output planes.
    int64_t nout_of(bool odd) const { return odd ? (n - 3) / 2 : (n - 5) / 2; }

    template <int ALPHA, bool SO0, bool CFL, bool BND>
    void half(bool odd)
    {
        int64_t const nout = nout_of(odd);
        if (nout <= 0)
        {
            return;
        }
        int64_t const threads = nout / 4 + 1;
        unsigned const grid = static_cast<unsigned>((threads + B32 - 1) / B32);
        if (odd)
        {
            k_half32<ALPHA, SO0, CFL, BND, 0><<<grid, B32, 0, stream>>>(args(), nout);
        }
        else
        {
            k_half32<ALPHA, SO0, CFL, BND, 1><<<grid, B32, 0, stream>>>(args(), nout);
        }
        scg::launched(stream, "e1d_half32");
    }

    // update_cfl(odd_plane) (Euler1DCore.cpp:70-94): the kernel points of the
    // half step, the even points 2 .. n - 5 (indices 1 ..) or the odd points
    // 1 .. n - 4 (indices 0 ..).
    void cfl_plane(bool odd)
    {
        int64_t const count = nout_of(odd);
        if (count > 0)
        {
            k_cfl32<<<static_cast<unsigned>((count + 255) / 256), 256, 0, stream>>>(args(), odd ? 1 : 0, odd ? 0 : 1,
                                                                                  count);
            scg::launched(stream, "e1d_cfl32");
        }
    }

    void op(int which, int odd, int alpha) override
    {
        switch (which)
        {
        case 0: // update_cfl
            cfl_plane(odd != 0);
            break;
        case 1: // march_half_so0
            half<0, true, false, false>(odd != 0);
            break;
        case 2: // march_half_so1_alpha
            if (alpha == 1)
                half<1, false, false, false>(odd != 0);
            else
                half<2, false, false, false>(odd != 0);
            break;
        case 3: // treat_boundary_so0
        case 4: // treat_boundary_so1
            k_bnd32<<<1, 1, 0, stream>>>(args(), which == 3 ? PL_SO0 : PL_SO1);
            scg::launched(stream, "e1d_bnd32");
            break;
        case 5: // setup_march
            cfl_plane(false);
            break;
        case 6: // march_half1_alpha
            if (alpha == 1)
                half<1, true, true, false>(false);
            else
                half<2, true, true, false>(false);
            break;
        case 7: // march_half2_alpha
            if (alpha == 1)
                half<1, true, true, false>(true);
            else
                half<2, true, true, false>(true);
            break;
        default:
            throw std::invalid_argument("Euler1DCore: unknown operation " + std::to_string(which));
        }
        sync();
    }

    // One march_alpha step: half 1 with the boundary treatment fused, half 2.
    void step(int alpha)
    {
        if (alpha == 1)
        {
            half<1, true, true, true>(false);
            half<1, true, true, false>(true);
        }
        else
        {
            half<2, true, true, true>(false);
            half<2, true, true, false>(true);
        }
    }

    void march(int alpha, int64_t steps) override
    {
        if (alpha != 1 && alpha != 2)
        {
            throw std::invalid_argument("Euler1DCore: alpha must be 1 or 2");
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
        scg::g_launches.store(before); // captured, not launched
        scg::cuda_check(cudaStreamEndCapture(stream, &g), "EndCapture");
        scg::cuda_check(cudaGraphInstantiate(&graph_exec, g, 0), "GraphInstantiate");
        cudaGraphDestroy(g);
        graph_alpha = alpha;
    }

    void sync() override { scg::cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }

private:
    static constexpr int GRAPH_STEPS = 32;
    scg::DevBuf<double> coord;
    scg::DevBuf<float> planes;
    int64_t P = 0;
    scg::DevBuf<double> m_staging;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_alpha = 0;
};

} // namespace

struct scg_e1d
{
    std::unique_ptr<Euler1DBase> c;
};

extern "C"
{

int scg_e1d_create(int64_t ncoord, double time_increment, scg_e1d ** out)
{
    return scg_e1d_create_precision(ncoord, time_increment, SCG_FP64, out);
}

int scg_e1d_create_precision(int64_t ncoord, double time_increment, int precision, scg_e1d ** out)
{
    return scg::guarded([&] {
        auto h = std::make_unique<scg_e1d>();
        if (precision == SCG_FP64)
            h->c = std::make_unique<Euler1D<double>>(ncoord, time_increment);
        else if (precision == SCG_FP32)
            h->c = std::make_unique<Euler1D32>(ncoord, time_increment);
        else
            throw std::invalid_argument("Euler1DCore: precision must be SCG_FP64 or SCG_FP32");
        *out = h.release();
    });
}

int scg_e1d_precision(const scg_e1d * h, int * precision)
{
    return scg::guarded([&] { *precision = h->c->precision; });
}

int scg_e1d_destroy(scg_e1d * h)
{
    return scg::guarded([&] { delete h; });
}

int scg_e1d_clone(scg_e1d * h, scg_e1d ** out)
{
    return scg::guarded([&] {
        auto c = std::make_unique<scg_e1d>();
        c->c = h->c->clone();
        *out = c.release();
    });
}

int scg_e1d_info(const scg_e1d * h, int64_t * ncoord, double * time_increment)
{
    return scg::guarded([&] {
        *ncoord = h->c->n;
        *time_increment = h->c->time_increment;
    });
}

int scg_e1d_get(scg_e1d * h, int which, double * host, int64_t count)
{
    return scg::guarded([&] {
        if (count != h->c->count(which))
            throw std::invalid_argument("Euler1DCore: host buffer size mismatch");
        h->c->get(which, host);
    });
}

int scg_e1d_set(scg_e1d * h, int which, const double * host, int64_t count)
{
    return scg::guarded([&] {
        if (count != h->c->count(which))
            throw std::invalid_argument("Euler1DCore: host buffer size mismatch");
        h->c->set(which, host);
    });
}

int scg_e1d_op(scg_e1d * h, int op, int odd_plane, int alpha)
{
    return scg::guarded([&] { h->c->op(op, odd_plane, alpha); });
}

int scg_e1d_march(scg_e1d * h, int alpha, int64_t steps)
{
    return scg::guarded([&] {
        if (steps < 0)
            throw std::invalid_argument("Euler1DCore::march_alpha: steps must be >= 0");
        h->c->march(alpha, steps);
    });
}

int scg_e1d_sync(scg_e1d * h)
{
    return scg::guarded([&] { h->c->sync(); });
}

int scg_e1d_stream(const scg_e1d * h, void ** out)
{
    return scg::guarded([&] { *out = h->c->stream; });
}

} // extern "C"
