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
 * kernels built from the same device routines.
 */

#include "../../include/scg.h"
#include "common.hpp"

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

// Coordinates stay FP64 (the grid); the state, gamma and cfl are R.
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
    // FP32 core: the grid spacing of each point, x - xneg and xpos - x,
    // formed in FP64 from the coordinates once; and dt/2, dt/4 in R.
    float const * dxm;
    float const * dxp;
    R hdt_r, qdt_r;
};

// The solution-element kernel at point ic (Euler1DKernel::set_value and
// derive, Euler1DCore.hpp:193-244): flux f, temporal derivatives ut, ft and
// the value up at the point, plus the two half fluxes of calc_flux_ll/lr
// (Euler1DCore.hpp:246-266).  Reciprocals of rho are formed once: for any
// density above ~1e-50 the reference's denominators rho^k + tiny equal rho^k.
// FP64: distances formed from the coordinates.  FP32: distances formed in
// FP32 from the point's two spacings, each rounded once from FP64.
template <typename R>
struct K1D
{
    double x, xneg, xpos;
    R r; // 1 / (rho + tiny), shared with update_cfl at the same point
    R up[3];
    R ll[3]; // flux through the lower-left of the CE to the right
    R lr[3]; // flux through the lower-right of the CE to the left
    // FP32 delta form: the state u, up - u, and ll / lr without their
    // dx * u parts (the caller adds those relative to the output point).
    R u[3];
    R upd[3];
    R llp[3];
    R lrp[3];
    R dm, dp; // FP32: x - xneg, xpos - x
};

template <typename R>
__device__ __forceinline__ void derive(E1DArgs<R> const & a, int64_t ic, K1D<R> & k)
{
    R const ga = a.gamma[ic];
    double xctr = 0.0;
    if constexpr (sizeof(R) == 8)
    {
        k.x = a.coord[ic];
        k.xneg = a.coord[ic - 1];
        k.xpos = a.coord[ic + 1];
        xctr = (k.xpos + k.xneg) * 0.5;
    }
    else
    {
        k.x = k.xneg = k.xpos = 0.0; // the FP32 path works from dm, dp
    }
    R u[3], ux[3];
    for (int i = 0; i < 3; ++i)
    {
        u[i] = a.so0[ic * 3 + i];
        ux[i] = a.so1[ic * 3 + i];
    }
    R const r = R(1) / (u[0] + Tiny1D<R>::V);
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
    if constexpr (sizeof(R) == 4)
    {
        // All in FP32 from the point's spacing: with dm = x - xneg and
        // dp = xpos - x, x - xctr = (dm - dp) / 2, and the BCE midpoints
        // sit at dm / 2 and -dp / 2 from the centre.
        R const hdt = a.hdt_r, qdt = a.qdt_r;
        R const dm = a.dxm[ic];
        R const dp = a.dxp[ic];
        k.dm = dm;
        k.dp = dp;
        R const dxctr = R(0.5) * (dm - dp);
        R const dxl = dp;
        R const dml = R(0.5) * dm;
        R const dxr = dm;
        R const dmr = R(-0.5) * dp;
        for (int i = 0; i < 3; ++i)
        {
            k.u[i] = u[i];
            k.upd[i] = dxctr * ux[i] + hdt * ut[i];
            k.up[i] = u[i] + k.upd[i]; // for the so1-only half step
            R const tf = f[i] - dxctr * ut[i] + qdt * ft[i];
            k.llp[i] = dxl * dml * ux[i] + hdt * tf;
            k.lrp[i] = dxr * dmr * ux[i] - hdt * tf;
        }
    }
    else
    {
        R const hdt = R(a.hdt), qdt = R(a.qdt);
        R const dxctr = R(k.x - xctr);
        R const dxl = R(k.xpos - k.x);
        R const dml = R(0.5 * (k.x + k.xpos) - xctr);
        R const dxr = R(k.x - k.xneg);
        R const dmr = R(0.5 * (k.x + k.xneg) - xctr);
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
}

// update_cfl at one point (Euler1DCore.cpp:70-94).  The reference's three
// divisions by rho use r = 1 / (rho + tiny), the reciprocal the kernel
// derivation at the same point forms (equal unless rho < ~1e-84, where the
// reference itself overflows).
template <typename R>
__device__ __forceinline__ R rho_recip(E1DArgs<R> const & a, int64_t it)
{
    return R(1) / (a.so0[it * 3 + 0] + Tiny1D<R>::V);
}

__device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__device__ __forceinline__ float sqrt_r(float x) { return sqrtf(x); }

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
    if constexpr (sizeof(R) == 4)
    {
        R const dxpos = a.dxp[it];
        R const dxneg = a.dxm[it];
        a.cfl[it] = a.hdt_r * wspd / (dxpos < dxneg ? dxpos : dxneg);
    }
    else
    {
        double const dxpos = a.coord[it + 1] - a.coord[it];
        double const dxneg = a.coord[it] - a.coord[it - 1];
        a.cfl[it] = R(hdt) * wspd / R(dxpos < dxneg ? dxpos : dxneg);
    }
}

// The W-alpha gradient (march_half_so1_alpha, Euler1DCore.hpp:284-320).
template <int ALPHA, typename R>
__device__ __forceinline__ R wgrad(R duxn, R duxp)
{
    R fan = fabs(duxn);
    R fap = fabs(duxp);
    if constexpr (ALPHA == 2)
    {
        fan *= fan;
        fap *= fap;
    }
    return (fap * duxn + fan * duxp) / (fap + fan + Tiny1D<R>::V);
}

// The FP32 half step in delta form: each new so0 is the old value at the
// point plus the change, formed from the kernels' states relative to it
// (dxl (u_l - u0) + dxr (u_r - u0) + the flux terms, over dxl + dxr), and the
// gradient's differences likewise, so FP32 rounding scales with the changes
// and not with the state.  The copy-out boundary treatment as in k_half.
template <int ALPHA, bool DO_CFL, bool BND>
__device__ __forceinline__ void half_delta(E1DArgs<float> const & a, int64_t start, int64_t nout)
{
    using R = float;
    __shared__ R s_u[B1D + 1][3];
    __shared__ R s_upd[B1D + 1][3];
    __shared__ R s_lrp[B1D + 1][3];
    __shared__ R s_dm[B1D + 1]; // x - xneg of each kernel
    int64_t const j0 = static_cast<int64_t>(blockIdx.x) * B1D;
    int64_t const j = j0 + threadIdx.x;
    K1D<R> k;
    bool const have = j <= nout;
    if (have)
    {
        derive(a, start + 2 * j, k);
        for (int i = 0; i < 3; ++i)
        {
            s_u[threadIdx.x][i] = k.u[i];
            s_upd[threadIdx.x][i] = k.upd[i];
            s_lrp[threadIdx.x][i] = k.lrp[i];
        }
        s_dm[threadIdx.x] = k.dm;
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
                s_u[B1D][i] = h.u[i];
                s_upd[B1D][i] = h.upd[i];
                s_lrp[B1D][i] = h.lrp[i];
            }
            s_dm[B1D] = h.dm;
        }
    }
    __syncthreads();
    if (have && j < nout)
    {
        int64_t const ic = start + 2 * j;
        // The output point ic + 1 between kernels ic (left) and ic + 2.
        R const dxl = k.dp;
        R const dxr = s_dm[threadIdx.x + 1];
        R const idx = R(1) / (dxl + dxr);
        R d[3];
        for (int i = 0; i < 3; ++i)
        {
            R const u0 = a.so0[(ic + 1) * 3 + i];
            d[i] = (dxl * (k.u[i] - u0) + dxr * (s_u[threadIdx.x + 1][i] - u0) + k.llp[i] +
                    s_lrp[threadIdx.x + 1][i]) *
                   idx;
            R const v = u0 + d[i];
            if constexpr (ALPHA > 0)
            {
                // The gradient's differences v - up_l and up_r - v, each
                // from small terms: (u0 - u_l) + d - (up_l - u_l), and
                // (u_r - u0) + (up_r - u_r) - d.
                R const idn = R(1) / dxl;
                R const idp = R(1) / dxr;
                R const duxn = ((u0 - k.u[i]) + d[i] - k.upd[i]) * idn;
                R const duxp = ((s_u[threadIdx.x + 1][i] - u0) + s_upd[threadIdx.x + 1][i] - d[i]) * idp;
                a.so1[(ic + 1) * 3 + i] = wgrad<ALPHA>(duxn, duxp);
            }
            a.so0[(ic + 1) * 3 + i] = v;
        }
        if (DO_CFL)
        {
            cfl_at(a, ic, a.hdt, k.r);
        }
    }
    if (BND && blockIdx.x == 0 && threadIdx.x == 0)
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

// Fused half step: so0, cfl and (when ALPHA > 0) so1 at one parity; with
// BND also the copy-out boundary treatment (Euler1DCore.cpp:132-172).
// Output j is point start + 2j + 1 for j < nout; kernels are at start + 2j for
// j <= nout.
template <int ALPHA, bool DO_SO0, bool DO_CFL, bool BND, typename R>
__global__ void __launch_bounds__(B1D) k_half(E1DArgs<R> a, int64_t start, int64_t nout)
{
    if constexpr (sizeof(R) == 4 && DO_SO0)
    {
        half_delta<ALPHA, DO_CFL, BND>(a, start, nout);
    }
    else
    {
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
            s_idxr[threadIdx.x] = sizeof(R) == 4 ? R(1) / k.dm : R(1.0 / (k.x - k.xneg));
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
                s_idxr[B1D] = sizeof(R) == 4 ? R(1) / h.dm : R(1.0 / (h.x - h.xneg));
            }
        }
        __syncthreads();
        if (have && j < nout)
        {
            int64_t const ic = start + 2 * j;
            R v[3];
            if (DO_SO0)
            {
                R const idx = R(1.0 / (a.coord[ic + 2] - a.coord[ic]));
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
            if (DO_CFL)
            {
                cfl_at(a, ic, a.hdt, k.r);
            }
            if constexpr (ALPHA > 0)
            {
                R const idn = sizeof(R) == 4 ? R(1) / k.dp : R(1.0 / (k.xpos - k.x));
                R const idp = s_idxr[threadIdx.x + 1];
                for (int i = 0; i < 3; ++i)
                {
                    R const duxn = (v[i] - k.up[i]) * idn;
                    R const duxp = (s_up[threadIdx.x + 1][i] - v[i]) * idp;
                    a.so1[(ic + 1) * 3 + i] = wgrad<ALPHA>(duxn, duxp);
                }
            }
        }
        if (BND && blockIdx.x == 0 && threadIdx.x == 0)
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

// FP64 host tables to and from the FP32 state, converted on the device; the
// host side read or written in place when it is a mapped scg_host_alloc
// block, else through a device staging table.
__global__ void k_e1d_from_f64(double const * in, float * out, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = float(in[i]);
    }
}

__global__ void k_e1d_to_f64(float const * in, double * out, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = double(in[i]);
    }
}

// The FP32 core's grid spacing, x - xneg and xpos - x, formed in FP64 from the
// coordinates and rounded once (zero where a neighbour is missing).
__global__ void k_e1d_spacing(double const * coord, float * dxm, float * dxp, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        dxm[i] = i > 0 ? float(coord[i] - coord[i - 1]) : 0.f;
        dxp[i] = i + 1 < n ? float(coord[i + 1] - coord[i]) : 0.f;
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

// R = double: the reference's arithmetic; R = float: FP32 state, cfl and
// gamma, with the coordinates kept in FP64 and the spacing between them
// formed in FP64 and rounded once to FP32 tables (dxm, dxp).
template <typename R>
class Euler1D : public Euler1DBase
{
public:
    Euler1D(int64_t ncoord, double dt)
    {
        n = ncoord;
        time_increment = dt;
        precision = sizeof(R) == 8 ? SCG_FP64 : SCG_FP32;
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
        for (auto * b : {&cfl, &gamma})
            b->alloc(static_cast<size_t>(n));
        so0.alloc(static_cast<size_t>(n * 3));
        so1.alloc(static_cast<size_t>(n * 3));
        if constexpr (sizeof(R) == 4)
        {
            dxm.alloc(static_cast<size_t>(n));
            dxp.alloc(static_cast<size_t>(n));
        }
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
        for (int k = 1; k < 5; ++k)
        {
            size_t const cnt = static_cast<size_t>(count(k));
            scg::cuda_check(cudaMemcpyAsync(c->state(k), state(k), cnt * sizeof(R), cudaMemcpyDeviceToDevice, stream),
                            "copy");
        }
        sync();
        c->spacing();
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
        if constexpr (sizeof(R) == 8)
        {
            scg::cuda_check(cudaMemcpyAsync(host, state(which), sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream),
                            "D2H");
            sync();
        }
        else
        {
            unsigned const grid = static_cast<unsigned>((cnt + 255) / 256);
            if (double * const dev = static_cast<double *>(scg::mapped_host(host, sizeof(double) * cnt)))
            {
                k_e1d_to_f64<<<grid, 256, 0, stream>>>(state(which), dev, static_cast<int64_t>(cnt));
                scg::launched(stream, "e1d_to_f64");
            }
            else
            {
                double * const tmp = staging(cnt);
                k_e1d_to_f64<<<grid, 256, 0, stream>>>(state(which), tmp, static_cast<int64_t>(cnt));
                scg::launched(stream, "e1d_to_f64");
                scg::cuda_check(cudaMemcpyAsync(host, tmp, sizeof(double) * cnt, cudaMemcpyDeviceToHost, stream),
                                "D2H");
            }
            sync();
        }
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
        if constexpr (sizeof(R) == 8)
        {
            put(state(which), host, cnt);
        }
        else
        {
            unsigned const grid = static_cast<unsigned>((cnt + 255) / 256);
            if (double const * const dev =
                    static_cast<double const *>(scg::mapped_host(host, sizeof(double) * cnt)))
            {
                k_e1d_from_f64<<<grid, 256, 0, stream>>>(dev, state(which), static_cast<int64_t>(cnt));
                scg::launched(stream, "e1d_from_f64");
            }
            else
            {
                double * const tmp = staging(cnt);
                scg::cuda_check(cudaMemcpyAsync(tmp, host, sizeof(double) * cnt, cudaMemcpyHostToDevice, stream),
                                "H2D");
                k_e1d_from_f64<<<grid, 256, 0, stream>>>(tmp, state(which), static_cast<int64_t>(cnt));
                scg::launched(stream, "e1d_from_f64");
            }
            sync();
        }
    }

    // The FP32 core's spacing tables from the coordinates, after each write
    // of them.
    void spacing()
    {
        if constexpr (sizeof(R) == 4)
        {
            k_e1d_spacing<<<static_cast<unsigned>((n + 255) / 256), 256, 0, stream>>>(coord.ptr, dxm.ptr, dxp.ptr, n);
            scg::launched(stream, "e1d_spacing");
            sync();
        }
    }

    // Grow-only device table for FP64 host data on its way to or from the
    // FP32 state.
    double * staging(size_t cnt)
    {
        if (m_staging.n < cnt)
        {
            sync();
            m_staging.alloc(cnt);
        }
        return m_staging.ptr;
    }

    E1DArgs<R> args()
    {
        return E1DArgs<R>{coord.ptr,
                          gamma.ptr,
                          so0.ptr,
                          so1.ptr,
                          cfl.ptr,
                          n,
                          time_increment / 2.0,
                          time_increment / 4.0,
                          dxm.ptr,
                          dxp.ptr,
                          R(time_increment / 2.0),
                          R(time_increment / 4.0)};
    }

    // Loop bounds of a half step (Euler1DCore.cpp:73-74, 99-100).
    void range(bool odd, int64_t & start, int64_t & nout) const
    {
        start = 2 - (odd ? 1 : 0);
        int64_t const stop = n - 2 - (odd ? 0 : 1);
        nout = stop > start ? (stop - start + 1) / 2 : 0;
    }

    template <int ALPHA, bool SO0, bool CFL, bool BND>
    void half(bool odd)
    {
        int64_t start, nout;
        range(odd, start, nout);
        unsigned const grid = static_cast<unsigned>((nout + B1D) / B1D);
        k_half<ALPHA, SO0, CFL, BND, R><<<grid, B1D, 0, stream>>>(args(), start, nout);
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

    // One march_alpha step (Euler1DCore.hpp:339-349): half 1 with the
    // boundary treatment fused, then half 2.
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
    scg::DevBuf<R> cfl, so0, so1, gamma;
    scg::DevBuf<float> dxm, dxp; // the FP32 core's grid spacing
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
            h->c = std::make_unique<Euler1D<float>>(ncoord, time_increment);
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
