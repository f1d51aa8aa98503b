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
constexpr double TINY1D = 1.e-100; // Euler1DKernel::tiny (Euler1DCore.hpp:182)

struct E1DArgs
{
    double const * coord;
    double const * gamma;
    double * so0; // [n][3]
    double * so1; // [n][3]
    double * cfl;
    int64_t n;
    double hdt, qdt;
};

// The solution-element kernel at point ic (Euler1DKernel::set_value and
// derive, Euler1DCore.hpp:193-244): flux f, temporal derivatives ut, ft and
// the value up at the point, plus the two half fluxes of calc_flux_ll/lr
// (Euler1DCore.hpp:246-266).  Reciprocals of rho are formed once: for any
// density above ~1e-50 the reference's denominators rho^k + tiny equal rho^k.
struct K1D
{
    double x, xneg, xpos;
    double r; // 1 / (rho + tiny), shared with update_cfl at the same point
    double up[3];
    double ll[3]; // flux through the lower-left of the CE to the right
    double lr[3]; // flux through the lower-right of the CE to the left
};

__device__ __forceinline__ void derive(E1DArgs const & a, int64_t ic, K1D & k)
{
    double const ga = a.gamma[ic];
    k.x = a.coord[ic];
    k.xneg = a.coord[ic - 1];
    k.xpos = a.coord[ic + 1];
    double const xctr = (k.xpos + k.xneg) * 0.5;
    double u[3], ux[3];
    for (int i = 0; i < 3; ++i)
    {
        u[i] = a.so0[ic * 3 + i];
        ux[i] = a.so1[ic * 3 + i];
    }
    double const r = 1.0 / (u[0] + TINY1D);
    k.r = r;
    double const r2 = r * r;
    double const m2r2 = u[1] * u[1] * r2; // u1^2 / u0^2
    double jac[3][3];
    jac[0][0] = 0.0;
    jac[0][1] = 1.0;
    jac[0][2] = 0.0;
    jac[1][0] = (ga - 3.0) / 2.0 * m2r2;
    jac[1][1] = -(ga - 3.0) * u[1] * r;
    jac[1][2] = ga - 1.0;
    jac[2][0] = (ga - 1.0) * m2r2 * u[1] * r - ga * u[1] * u[2] * r2;
    jac[2][1] = ga * u[2] * r - 1.5 * (ga - 1.0) * m2r2;
    jac[2][2] = ga * u[1] * r;
    double f[3], ut[3], ft[3];
    f[0] = u[1];
    f[1] = (ga - 1.0) * u[2] + (3.0 - ga) / 2.0 * u[1] * u[1] * r;
    f[2] = ga * u[1] * u[2] * r - (ga - 1.0) / 2.0 * u[1] * m2r2;
    for (int i = 0; i < 3; ++i)
    {
        ut[i] = -jac[i][0] * ux[0] - jac[i][1] * ux[1] - jac[i][2] * ux[2];
    }
    for (int i = 0; i < 3; ++i)
    {
        ft[i] = jac[i][0] * ut[0] + jac[i][1] * ut[1] + jac[i][2] * ut[2];
    }
    double const dxctr = k.x - xctr;
    for (int i = 0; i < 3; ++i)
    {
        k.up[i] = u[i] + dxctr * ux[i] + a.hdt * ut[i];
    }
    double const dxl = k.xpos - k.x;
    double const dml = 0.5 * (k.x + k.xpos) - xctr;
    double const dxr = k.x - k.xneg;
    double const dmr = 0.5 * (k.x + k.xneg) - xctr;
    for (int i = 0; i < 3; ++i)
    {
        double const tf = f[i] - dxctr * ut[i] + a.qdt * ft[i];
        k.ll[i] = dxl * (u[i] + dml * ux[i]) + a.hdt * tf;
        k.lr[i] = dxr * (u[i] + dmr * ux[i]) - a.hdt * tf;
    }
}

// update_cfl at one point (Euler1DCore.cpp:70-94).  The reference's three
// divisions by rho use r = 1 / (rho + tiny), the reciprocal the kernel
// derivation at the same point forms (equal unless rho < ~1e-84, where the
// reference itself overflows).
__device__ __forceinline__ double rho_recip(E1DArgs const & a, int64_t it)
{
    return 1.0 / (a.so0[it * 3 + 0] + TINY1D);
}

__device__ __forceinline__ void cfl_at(E1DArgs const & a, int64_t it, double hdt, double r)
{
    double const ga = a.gamma[it];
    double const m = a.so0[it * 3 + 1];
    double const m2 = m * m;
    double const ke = 0.5 * m2 * r;
    double pr = (ga - 1.0) * (a.so0[it * 3 + 2] - ke);
    pr = (pr + fabs(pr)) / 2.0;
    // The reference's sqrt(m * m) is |m| exactly: in binary IEEE arithmetic
    // the square root of a correctly rounded square returns the operand's
    // magnitude (barring overflow or underflow of the square).
    double const wspd = sqrt(ga * pr * r) + fabs(m) * r;
    double const dxpos = a.coord[it + 1] - a.coord[it];
    double const dxneg = a.coord[it] - a.coord[it - 1];
    a.cfl[it] = hdt * wspd / (dxpos < dxneg ? dxpos : dxneg);
}

// The W-alpha gradient (march_half_so1_alpha, Euler1DCore.hpp:284-320).
template <int ALPHA>
__device__ __forceinline__ double wgrad(double duxn, double duxp)
{
    double fan = fabs(duxn);
    double fap = fabs(duxp);
    if constexpr (ALPHA == 2)
    {
        fan *= fan;
        fap *= fap;
    }
    return (fap * duxn + fan * duxp) / (fap + fan + TINY1D);
}

// Fused half step: so0, cfl and (when ALPHA > 0) so1 at one parity; with
// BND also the copy-out boundary treatment (Euler1DCore.cpp:132-172).
// Output j is point start + 2j + 1 for j < nout; kernels are at start + 2j for
// j <= nout.
template <int ALPHA, bool DO_SO0, bool DO_CFL, bool BND>
__global__ void __launch_bounds__(B1D) k_half(E1DArgs a, int64_t start, int64_t nout)
{
    __shared__ double s_lr[B1D + 1][3];
    __shared__ double s_up[B1D + 1][3];
    __shared__ double s_idxr[B1D + 1]; // 1 / (x - xneg) of each kernel
    int64_t const j0 = static_cast<int64_t>(blockIdx.x) * B1D;
    int64_t const j = j0 + threadIdx.x;
    K1D k;
    bool const have = j <= nout;
    if (have)
    {
        derive(a, start + 2 * j, k);
        for (int i = 0; i < 3; ++i)
        {
            s_lr[threadIdx.x][i] = k.lr[i];
            s_up[threadIdx.x][i] = k.up[i];
        }
        s_idxr[threadIdx.x] = 1.0 / (k.x - k.xneg);
    }
    if (threadIdx.x == 0)
    {
        int64_t const jh = j0 + B1D; // halo kernel on the right
        if (jh <= nout)
        {
            K1D h;
            derive(a, start + 2 * jh, h);
            for (int i = 0; i < 3; ++i)
            {
                s_lr[B1D][i] = h.lr[i];
                s_up[B1D][i] = h.up[i];
            }
            s_idxr[B1D] = 1.0 / (h.x - h.xneg);
        }
    }
    __syncthreads();
    if (have && j < nout)
    {
        int64_t const ic = start + 2 * j;
        double v[3];
        if (DO_SO0)
        {
            double const idx = 1.0 / (a.coord[ic + 2] - a.coord[ic]);
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
            double const idn = 1.0 / (k.xpos - k.x);
            double const idp = s_idxr[threadIdx.x + 1];
            for (int i = 0; i < 3; ++i)
            {
                double const duxn = (v[i] - k.up[i]) * idn;
                double const duxp = (s_up[threadIdx.x + 1][i] - v[i]) * idp;
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

// update_cfl alone.
__global__ void k_cfl1d(E1DArgs a, int64_t start, int64_t nout)
{
    int64_t const j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < nout)
    {
        int64_t const it = start + 2 * j;
        cfl_at(a, it, a.hdt, rho_recip(a, it));
    }
}

// treat_boundary_so0 / treat_boundary_so1.
__global__ void k_bnd1d(E1DArgs a, int which)
{
    int64_t const l = 1, r = a.n - 2;
    double * s = which == 0 ? a.so0 : a.so1;
    for (int i = 0; i < 3; ++i)
    {
        s[l * 3 + i] = s[(l + 1) * 3 + i];
        s[r * 3 + i] = s[(r - 1) * 3 + i];
    }
}

class Euler1D
{
public:
    Euler1D(int64_t ncoord, double dt)
        : n(ncoord)
        , time_increment(dt)
    {
        if (ncoord % 2 == 0)
        {
            throw std::invalid_argument("ncoord cannot be even");
        }
        if (ncoord < 5)
        {
            throw std::invalid_argument("Euler1DCore: ncoord must be at least 5");
        }
        scg::cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto * b : {&coord, &cfl, &gamma})
            b->alloc(static_cast<size_t>(n));
        so0.alloc(static_cast<size_t>(n * 3));
        so1.alloc(static_cast<size_t>(n * 3));
        std::vector<double> g(static_cast<size_t>(n), 1.4);
        std::vector<double> z(static_cast<size_t>(n * 3), 0.0);
        put(gamma.ptr, g.data(), n);
        put(coord.ptr, z.data(), n);
        put(cfl.ptr, z.data(), n);
        put(so0.ptr, z.data(), n * 3);
        put(so1.ptr, z.data(), n * 3);
        sync();
    }

    ~Euler1D()
    {
        if (graph_exec)
            cudaGraphExecDestroy(graph_exec);
        if (stream)
        {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    std::unique_ptr<Euler1D> clone()
    {
        auto c = std::make_unique<Euler1D>(n, time_increment);
        for (int k = 0; k < 5; ++k)
        {
            double * src = field(k);
            double * dst = c->field(k);
            size_t const cnt = static_cast<size_t>(k >= 2 && k <= 3 ? n * 3 : n);
            scg::cuda_check(cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
        }
        sync();
        return c;
    }

    // 0 coord, 1 cfl, 2 so0, 3 so1, 4 gamma
    double * field(int which)
    {
        switch (which)
        {
        case 0: return coord.ptr;
        case 1: return cfl.ptr;
        case 2: return so0.ptr;
        case 3: return so1.ptr;
        case 4: return gamma.ptr;
        default: throw std::invalid_argument("Euler1DCore: unknown array id " + std::to_string(which));
        }
    }
    int64_t count(int which) const { return (which == 2 || which == 3) ? n * 3 : n; }

    void get(int which, double * host)
    {
        scg::cuda_check(cudaMemcpyAsync(host, field(which), sizeof(double) * static_cast<size_t>(count(which)),
                                        cudaMemcpyDeviceToHost, stream),
                        "D2H");
        sync();
    }
    void set(int which, double const * host)
    {
        put(field(which), host, count(which));
        sync();
    }

    E1DArgs args()
    {
        return E1DArgs{coord.ptr, gamma.ptr, so0.ptr, so1.ptr, cfl.ptr, n, time_increment / 2.0,
                       time_increment / 4.0};
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
        k_half<ALPHA, SO0, CFL, BND><<<grid, B1D, 0, stream>>>(args(), start, nout);
        scg::launched(stream, "e1d_half");
    }

    void op(int which, int odd, int alpha)
    {
        switch (which)
        {
        case 0: // update_cfl
        {
            int64_t start, nout;
            range(odd != 0, start, nout);
            if (nout > 0)
            {
                k_cfl1d<<<static_cast<unsigned>((nout + 255) / 256), 256, 0, stream>>>(args(), start, nout);
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
            k_bnd1d<<<1, 1, 0, stream>>>(args(), which - 3);
            scg::launched(stream, "e1d_bnd");
            break;
        case 5: // setup_march
        {
            int64_t start, nout;
            range(false, start, nout);
            if (nout > 0)
            {
                k_cfl1d<<<static_cast<unsigned>((nout + 255) / 256), 256, 0, stream>>>(args(), start, nout);
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
    void march(int alpha, int64_t steps)
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

    void sync() { scg::cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }

    int64_t n;
    double time_increment;
    cudaStream_t stream = nullptr;

private:
    static constexpr int GRAPH_STEPS = 32;

    void put(double * dst, double const * src, int64_t cnt)
    {
        scg::cuda_check(cudaMemcpyAsync(dst, src, sizeof(double) * static_cast<size_t>(cnt), cudaMemcpyHostToDevice,
                                        stream),
                        "H2D");
        sync();
    }

    scg::DevBuf<double> coord, cfl, so0, so1, gamma;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_alpha = 0;
};

} // namespace

struct scg_e1d
{
    std::unique_ptr<Euler1D> c;
};

extern "C"
{

int scg_e1d_create(int64_t ncoord, double time_increment, scg_e1d ** out)
{
    return scg::guarded([&] {
        auto h = std::make_unique<scg_e1d>();
        h->c = std::make_unique<Euler1D>(ncoord, time_increment);
        *out = h.release();
    });
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
