/*
 * GPU Euler core: device state, the per-operation kernels of the EulerCore
 * surface, and the fused march.
 *
 * Logical arrays of the reference and where they live here (cur/nxt are the
 * two record buffers, swapped by update() just as the reference swaps so0c
 * with so0n and so1c with so1n, euler.hpp:123-127):
 *   so0c = cur.so0, so1c = cur.so1, so0n = nxt.so0, so1n = nxt.so1,
 *   so0t = rec[tbuf].so0t   (so0t is not swapped by update()).
 * The fused march additionally leaves nxt.so0t holding calc_solt of the new
 * state, so the next substep skips its calc_solt pass (see march_substep()).
 */

#include "euler_core.hpp"
#include "euler_kernels.cuh"
#include "euler_setup.cuh"
#include "reduce.cuh"

#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace scg
{

using namespace dev;

namespace
{

constexpr int BLOCK = 128;

inline unsigned grid_for(int64_t n)
{
    return static_cast<unsigned>((n + BLOCK - 1) / BLOCK);
}

// --------------------------------------------------------------------------
// Per-operation kernels (one thread per row or body cell).

template <int ND, typename R>
__global__ void k_solt_rows(R * rec, R const * gamma, int64_t nrow)
{
    constexpr int NEQ = ND + 2;
    int64_t const r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nrow)
    {
        return;
    }
    using RC = Rec<ND, R>;
    R v[RC::NUSED];
    load_rec<ND, R>(rec + r * RC::RS, v);
    R t[NEQ];
    Prim<ND, R> const q(v, gamma[r]);
    solt_prim<ND, R>(q, v, v + 2 * NEQ, t);
    for (int i = 0; i < NEQ; ++i)
    {
        rec[r * RC::RS + NEQ + i] = t[i];
    }
    if constexpr (RC::PRIM)
    {
        q.cache(rec + r * RC::RS + RC::OP);
    }
}

template <int ND, typename R>
__global__ void k_copy_field(R const * src, R * dst, int64_t nrow, int off, int width)
{
    int64_t const r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nrow)
    {
        return;
    }
    for (int k = 0; k < width; ++k)
    {
        dst[r * Rec<ND, R>::RS + off + k] = src[r * Rec<ND, R>::RS + off + k];
    }
}

template <int ND, typename R, typename G>
__global__ void k_soln(MarchArgs<R, G> a)
{
    constexpr int NEQ = ND + 2;
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= a.ncell)
    {
        return;
    }
    R so0n[NEQ];
    int const ct = a.ctype[icl];
    if constexpr (ND == 2)
    {
        if (ct == 4)
            soln_cell<4, R, G>(a, icl, so0n);
        else
            soln_cell<3, R, G>(a, icl, so0n);
    }
    else
    {
        switch (ct)
        {
        case 6: soln_cell<6, R, G>(a, icl, so0n); break;
        case 5: soln_cell<5, R, G>(a, icl, so0n); break;
        case 7: soln_cell<7, R, G>(a, icl, so0n); break;
        default: soln_cell<8, R, G>(a, icl, so0n); break;
        }
    }
    R * out = a.nxt + (icl + a.ngst) * Rec<ND, R>::RS;
    for (int i = 0; i < NEQ; ++i)
    {
        out[i] = so0n[i];
    }
}

template <int ND, typename R, typename G>
__global__ void k_cfl(MarchArgs<R, G> a)
{
    constexpr int NEQ = ND + 2;
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= a.ncell)
    {
        return;
    }
    int64_t const row = icl + a.ngst;
    R * out = a.nxt + row * Rec<ND, R>::RS;
    R s[NEQ];
    for (int i = 0; i < NEQ; ++i)
    {
        s[i] = out[i];
    }
    R rinv;
    cfl_cell<ND, R, G>(a, icl, row, s, rinv);
    out[NEQ - 1] = s[NEQ - 1];
}

template <int ND, typename R, typename G>
__global__ void k_dsoln(MarchArgs<R, G> a)
{
    constexpr int NEQ = ND + 2;
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= a.ncell)
    {
        return;
    }
    int64_t const row = icl + a.ngst;
    R * out = a.nxt + row * Rec<ND, R>::RS;
    R s[NEQ];
    for (int i = 0; i < NEQ; ++i)
    {
        s[i] = out[i];
    }
    R const cflc = a.cflc[row];
    R g[NEQ * ND];
    int const ct = a.ctype[icl];
    if constexpr (ND == 2)
    {
        if (ct == 4)
            dsoln_cell<4, R, G>(a, icl, s, cflc, g);
        else
            dsoln_cell<3, R, G>(a, icl, s, cflc, g);
    }
    else
    {
        switch (ct)
        {
        case 6: dsoln_cell<6, R, G>(a, icl, s, cflc, g); break;
        case 5: dsoln_cell<5, R, G>(a, icl, s, cflc, g); break;
        case 7: dsoln_cell<7, R, G>(a, icl, s, cflc, g); break;
        default: dsoln_cell<8, R, G>(a, icl, s, cflc, g); break;
        }
    }
    for (int i = 0; i < NEQ * ND; ++i)
    {
        out[2 * NEQ + i] = g[i];
    }
}

// bc_soln over every ghost row with a registered condition.
template <int ND, typename R, typename G>
__global__ void k_bc0(MarchArgs<R, G> a, int32_t const * gint)
{
    constexpr int NEQ = ND + 2;
    int64_t const g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= a.ngst || a.gkind[g] < 0)
    {
        return;
    }
    R const * in = a.nxt + static_cast<int64_t>(gint[g]) * Rec<ND, R>::RS;
    R s[NEQ], o[NEQ];
    for (int i = 0; i < NEQ; ++i)
    {
        s[i] = in[i];
    }
    bc0_ghost<ND, R>(a.gkind[g], a.gnml + g * ND, a.gval + g * NEQ, s, o);
    R * out = a.nxt + g * Rec<ND, R>::RS;
    for (int i = 0; i < NEQ; ++i)
    {
        out[i] = o[i];
    }
}

// bc_dsoln over every ghost row with a registered condition.
template <int ND, typename R, typename G>
__global__ void k_bc1(MarchArgs<R, G> a, int32_t const * gint)
{
    constexpr int NEQ = ND + 2;
    int64_t const g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= a.ngst || a.gkind[g] < 0)
    {
        return;
    }
    R const * in = a.cur + static_cast<int64_t>(gint[g]) * Rec<ND, R>::RS + 2 * NEQ;
    R s[NEQ * ND], o[NEQ * ND];
    for (int i = 0; i < NEQ * ND; ++i)
    {
        s[i] = in[i];
    }
    bc1_ghost<ND, R>(a.gkind[g], a.gnml + g * ND, s, o);
    R * out = a.nxt + g * Rec<ND, R>::RS + 2 * NEQ;
    for (int i = 0; i < NEQ * ND; ++i)
    {
        out[i] = o[i];
    }
}

// init_solution (euler_solution.cpp:54-99): so0n body rows and every gamma.
template <int ND, typename R>
__global__ void k_init(R * nxt, R * gamma, int64_t ngst, int64_t nrow, double ga, double rho, double m0, double m1,
                       double m2, double energy)
{
    constexpr int NEQ = ND + 2;
    int64_t const r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nrow)
    {
        return;
    }
    gamma[r] = R(ga);
    if (r >= ngst)
    {
        R * o = nxt + r * Rec<ND, R>::RS;
        o[0] = R(rho);
        o[1] = R(m0);
        o[2] = R(m1);
        if constexpr (ND == 3)
        {
            o[3] = R(m2);
        }
        o[NEQ - 1] = R(energy);
    }
}

// The FP32 state of a body row is its record's so0 plus the rounding residual
// the march carries beside it ([NEQ][ncell], see fused_cell); comp is that
// residual for the so0 table being read or written, else null.
struct Residual
{
    void * comp = nullptr;
    int64_t ngst = 0, ncell = 0;
};

// Value k of row r of a record field in FP64, the residual added.
template <int ND, typename R>
__device__ __forceinline__ double field_value(R const * rec, int64_t r, int off, int k, Residual c)
{
    double v = double(rec[r * Rec<ND, R>::RS + off + k]);
    if (c.comp && r >= c.ngst)
    {
        v += double(static_cast<R const *>(c.comp)[k * c.ncell + (r - c.ngst)]);
    }
    return v;
}

// Store an FP64 value into a record field: the rounded value, and for a body
// row of an FP32 so0 table the part the rounding dropped into the residual.
template <int ND, typename R>
__device__ __forceinline__ void field_store(R * rec, int64_t r, int off, int k, double x, Residual c)
{
    R const t = R(x);
    rec[r * Rec<ND, R>::RS + off + k] = t;
    if (c.comp && r >= c.ngst)
    {
        static_cast<R *>(c.comp)[k * c.ncell + (r - c.ngst)] = R(x - double(t));
    }
}

// Record field <-> FP64 reference-layout table.
template <int ND, typename R>
__global__ void k_get_field(R const * rec, double * out, int64_t nrow, int off, int width, Residual c)
{
    int64_t const r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nrow)
    {
        return;
    }
    for (int k = 0; k < width; ++k)
    {
        out[r * width + k] = field_value<ND, R>(rec, r, off, k, c);
    }
}

template <int ND, typename R>
__global__ void k_set_field(R * rec, double const * in, int64_t nrow, int off, int width, Residual c)
{
    int64_t const r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= nrow)
    {
        return;
    }
    for (int k = 0; k < width; ++k)
    {
        field_store<ND, R>(rec, r, off, k, in[r * width + k], c);
    }
}

// The same record fields read from or written to mapped host memory: one
// thread per pair of consecutive doubles of the host table, so the host side
// is accessed in contiguous 16-byte pieces (vec: the host table is 16-byte
// aligned) and the records are gathered on the device.
template <int ND, typename R>
__global__ void k_get_field_host(R const * rec, double * out, int64_t nrow, int off, int width, bool vec,
                                 Residual c)
{
    int64_t const n = nrow * width;
    int64_t const i = 2 * (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
    if (i >= n)
    {
        return;
    }
    int64_t const r0 = i / width;
    int const k0 = static_cast<int>(i - r0 * width);
    double const v0 = field_value<ND, R>(rec, r0, off, k0, c);
    if (i + 1 >= n)
    {
        out[i] = v0;
        return;
    }
    int64_t const r1 = k0 + 1 < width ? r0 : r0 + 1;
    int const k1 = k0 + 1 < width ? k0 + 1 : 0;
    double const v1 = field_value<ND, R>(rec, r1, off, k1, c);
    if (vec)
    {
        *reinterpret_cast<double2 *>(out + i) = make_double2(v0, v1);
    }
    else
    {
        out[i] = v0;
        out[i + 1] = v1;
    }
}

// Two values per thread (grid-stride: a grid of one pass per pair is the
// usual launch).
template <int ND, typename R>
__global__ void k_set_field_host(R * rec, double const * in, int64_t nrow, int off, int width, bool vec,
                                 Residual c)
{
    int64_t const n = nrow * width;
    int64_t const step = 2 * static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = 2 * (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x); i < n; i += step)
    {
        int64_t const r0 = i / width;
        int const k0 = static_cast<int>(i - r0 * width);
        if (i + 1 >= n)
        {
            field_store<ND, R>(rec, r0, off, k0, in[i], c);
            continue;
        }
        double2 v;
        if (vec)
        {
            v = *reinterpret_cast<double2 const *>(in + i);
        }
        else
        {
            v = make_double2(in[i], in[i + 1]);
        }
        int64_t const r1 = k0 + 1 < width ? r0 : r0 + 1;
        int const k1 = k0 + 1 < width ? k0 + 1 : 0;
        field_store<ND, R>(rec, r0, off, k0, v.x, c);
        field_store<ND, R>(rec, r1, off, k1, v.y, c);
    }
}

// The highest row any cell of each chunk of csize cells reads in a substep
// (its own row and its neighbours' over its cell type's faces), one block per
// chunk: march_from_host launches a chunk's substep once those rows are up.
__global__ void k_chunk_top_row(int32_t const * nbr, int8_t const * ctype, int64_t ncell, int64_t csize,
                                int nslot, int64_t ngst, int64_t * top)
{
    __shared__ int64_t sh[256];
    int64_t const c0 = static_cast<int64_t>(blockIdx.x) * csize;
    int64_t const c1 = c0 + csize < ncell ? c0 + csize : ncell;
    int64_t m = -1;
    for (int64_t t = c0 + threadIdx.x; t < c1; t += blockDim.x)
    {
        int nf;
        switch (ctype[t])
        {
        case CT_TRIANGLE: nf = 3; break;
        case CT_QUAD: nf = 4; break;
        case CT_TET: nf = 4; break;
        case CT_HEX: nf = 6; break;
        default: nf = 5; break; // prism, pyramid
        }
        nf = nf < nslot ? nf : nslot;
        m = m > ngst + t ? m : ngst + t;
        for (int f = 0; f < nf; ++f)
        {
            int64_t const j = nbr[static_cast<int64_t>(f) * ncell + t];
            m = m > j ? m : j;
        }
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1)
    {
        if (static_cast<int>(threadIdx.x) < k)
        {
            sh[threadIdx.x] = sh[threadIdx.x] > sh[threadIdx.x + k] ? sh[threadIdx.x] : sh[threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        top[blockIdx.x] = sh[0];
    }
}

// so1n written from a mapped host table and then calc_solt of each row as
// it now stands (its so0 already in the record): the next march finds so0t
// and the FP64 primitive cache of the new state made, and the Jacobian
// products run while other blocks wait on the host link.  A block copies its
// rows' contiguous stretch of the host table to shared memory in 16-byte
// pieces (vec: the table is 16-byte aligned; a block's stretch starts at a
// multiple of 128 rows, so it is aligned too), then one thread per row
// finishes the row.  The values and the arithmetic are those of
// k_set_field_host followed by k_solt_rows.
template <int ND, typename R>
__global__ void __launch_bounds__(BLOCK) k_set_so1_host_solt(R * rec, double const * in, R const * gamma,
                                                             int64_t nrow, bool vec)
{
    constexpr int NEQ = ND + 2;
    constexpr int W = NEQ * ND;
    using RC = Rec<ND, R>;
    __shared__ double buf[BLOCK * W];
    // Grid-stride over stretches of BLOCK rows (see k_set_field_host).
    for (int64_t r0 = static_cast<int64_t>(blockIdx.x) * BLOCK; r0 < nrow;
         r0 += static_cast<int64_t>(gridDim.x) * BLOCK)
    {
        int64_t const left = nrow - r0;
        int const nr = static_cast<int>(left < BLOCK ? left : BLOCK);
        int const n = nr * W;
        double const * const src = in + r0 * W;
        __syncthreads(); // the previous stretch is done with buf
        for (int i = 2 * static_cast<int>(threadIdx.x); i < n; i += 2 * BLOCK)
        {
            if (vec && i + 1 < n)
            {
                double2 const v = *reinterpret_cast<double2 const *>(src + i);
                buf[i] = v.x;
                buf[i + 1] = v.y;
            }
            else
            {
                buf[i] = src[i];
                if (i + 1 < n)
                {
                    buf[i + 1] = src[i + 1];
                }
            }
        }
        __syncthreads();
        if (static_cast<int>(threadIdx.x) < nr)
        {
            int64_t const r = r0 + threadIdx.x;
            R * const row = rec + r * RC::RS;
            R v[RC::NUSED];
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                v[i] = row[i];
            }
#pragma unroll
            for (int k = 0; k < W; ++k)
            {
                v[2 * NEQ + k] = R(buf[threadIdx.x * W + k]);
            }
            Prim<ND, R> const q(v, gamma[r]);
            R t[NEQ];
            solt_prim<ND, R>(q, v, v + 2 * NEQ, t);
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                row[NEQ + i] = t[i];
            }
#pragma unroll
            for (int k = 0; k < W; ++k)
            {
                row[2 * NEQ + k] = v[2 * NEQ + k];
            }
            if constexpr (RC::PRIM)
            {
                q.cache(row + RC::OP);
            }
        }
    }
}

template <typename R>
__global__ void k_to_f64(R const * in, double * out, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = double(in[i]);
    }
}

template <typename R>
__global__ void k_from_f64(double const * in, R * out, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = R(in[i]);
    }
}

// One scalar field of the newest solution per body cell, in FP64, with the
// formulas of EulerField (solvcon/multidim/euler/_field.py:80-125):
// velocity m / rho, speed |v|, pressure (gamma - 1)(E - rho |v|^2 / 2), Mach
// number |v| / sqrt(gamma p / rho), and the unclamped CFL number cflo.
template <int ND, typename R>
__global__ void k_field(R const * nxt, R const * gamma, R const * cflo, int64_t ngst, int64_t ncell, int which,
                        double * out, Residual c)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= ncell)
    {
        return;
    }
    int64_t const row = icl + ngst;
    double const rho = field_value<ND, R>(nxt, row, 0, 0, c);
    double v[ND];
    double vsq = 0.0;
    for (int d = 0; d < ND; ++d)
    {
        v[d] = field_value<ND, R>(nxt, row, 0, 1 + d, c) / rho;
        vsq += v[d] * v[d];
    }
    double const energy = field_value<ND, R>(nxt, row, 0, ND + 1, c);
    double const ga = double(gamma[row]);
    double r = 0.0;
    switch (which)
    {
    case EF_DENSITY: r = rho; break;
    case EF_VELX: r = v[0]; break;
    case EF_VELY: r = v[1]; break;
    case EF_VELZ: r = v[ND - 1]; break;
    case EF_SPEED: r = sqrt(vsq); break;
    case EF_PRESSURE: r = (ga - 1.0) * (energy - 0.5 * rho * vsq); break;
    case EF_MACH:
    {
        double const p = (ga - 1.0) * (energy - 0.5 * rho * vsq);
        r = sqrt(vsq) / sqrt(ga * p / rho);
        break;
    }
    case EF_TOTAL_ENERGY: r = energy; break;
    default: r = double(cflo[row]); break;
    }
    out[icl] = r;
}

// Per-block FP64 partial sums of so0n[:, i] * clvol (Kahan inside a thread,
// warp shuffles across the block), and min/max of cflo.
template <int ND, typename R>
__global__ void __launch_bounds__(BLOCK) k_totals(R const * nxt, double const * clvol, R const * cflo, int64_t ngst,
                                                  int64_t ncell, double * part, Residual cr)
{
    constexpr int NEQ = ND + 2;
    __shared__ double sh[BLOCK / 32];
    double s[NEQ], c[NEQ];
    for (int i = 0; i < NEQ; ++i)
    {
        s[i] = 0.0;
        c[i] = 0.0;
    }
    double lo = 1.79769313486231570815e+308, hi = -1.79769313486231570815e+308;
    for (int64_t icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; icl < ncell;
         icl += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        int64_t const row = icl + ngst;
        double const v = clvol[row];
        for (int i = 0; i < NEQ; ++i)
        {
            double const y = field_value<ND, R>(nxt, row, 0, i, cr) * v - c[i];
            double const t = s[i] + y;
            c[i] = (t - s[i]) - y;
            s[i] = t;
        }
        double const cf = double(cflo[row]);
        lo = fmin(lo, cf);
        hi = fmax(hi, cf);
    }
    double out[NEQ + 2];
    for (int i = 0; i < NEQ; ++i)
    {
        out[i] = red::block_fold<red::SUM, BLOCK / 32>(s[i], sh);
    }
    out[NEQ] = red::block_fold<red::MIN, BLOCK / 32>(lo, sh);
    out[NEQ + 1] = red::block_fold<red::MAX, BLOCK / 32>(hi, sh);
    if (threadIdx.x == 0)
    {
        for (int i = 0; i < NEQ + 2; ++i)
        {
            part[blockIdx.x * (NEQ + 2) + i] = out[i];
        }
    }
}

} // namespace

// --------------------------------------------------------------------------
// Base-class helpers.

void EulerCoreBase::array_shape(int which, int64_t * shape, int * nd, int64_t * nghost) const
{
    int64_t const tot = ngstcell + ncell;
    *nghost = ngstcell;
    switch (which)
    {
    case EA_CEVOL: shape[0] = tot; shape[1] = 7; *nd = 2; break;
    case EA_CECND: shape[0] = tot; shape[1] = 7 * ndim; *nd = 2; break;
    case EA_SFCND:
    case EA_SFNML:
        shape[0] = ncell; shape[1] = 24; shape[2] = ndim; *nd = 3; *nghost = 0; break;
    case EA_SO0C:
    case EA_SO0N:
    case EA_SO0T:
    case EA_STM: shape[0] = tot; shape[1] = neq; *nd = 2; break;
    case EA_SO1C:
    case EA_SO1N: shape[0] = tot; shape[1] = neq; shape[2] = ndim; *nd = 3; break;
    case EA_CFLO:
    case EA_CFLC:
    case EA_GAMMA: shape[0] = tot; *nd = 1; break;
    default: throw std::invalid_argument("EulerCore: unknown array id " + std::to_string(which));
    }
}

int64_t EulerCoreBase::array_size(int which) const
{
    int64_t shape[3] = {1, 1, 1};
    int nd = 0;
    int64_t ng = 0;
    array_shape(which, shape, &nd, &ng);
    int64_t n = 1;
    for (int k = 0; k < nd; ++k)
    {
        n *= shape[k];
    }
    return n;
}

// add_bc with the reference's validation (euler_bc.cpp:324-391).
void EulerCoreBase::add_bc(int kind, std::vector<int32_t> const & faces, std::vector<double> const & value)
{
    if (kind < BC_NONREFL || kind > BC_INLET)
    {
        throw std::invalid_argument("EulerCore::add_bc: unknown boundary kind " + std::to_string(kind));
    }
    for (int32_t const ifc : faces)
    {
        if (ifc < 0 || ifc >= m_nface)
        {
            throw std::invalid_argument("EulerCore::add_bc: face " + std::to_string(ifc) + " out of range [0, " +
                                        std::to_string(m_nface) + ")");
        }
        if (m_fccls[static_cast<size_t>((ifc + m_ngstface) * 4 + 1)] >= 0)
        {
            throw std::invalid_argument("EulerCore::add_bc: face " + std::to_string(ifc) + " is not a boundary face");
        }
    }
    if (kind == BC_INLET)
    {
        size_t const expect = static_cast<size_t>(ndim) + 3;
        if (value.size() != expect)
        {
            throw std::invalid_argument("EulerCore::add_bc: inlet value size " + std::to_string(value.size()) +
                                        " must equal ndim+3 = " + std::to_string(expect));
        }
        double const rho = value[0];
        double const p = value[1 + ndim];
        double const ga = value[2 + ndim];
        if (ga <= 1.0)
        {
            throw std::invalid_argument("EulerCore::add_bc: inlet gamma " + std::to_string(ga) + " must be > 1");
        }
        if (rho <= 0.0)
        {
            throw std::invalid_argument("EulerCore::add_bc: inlet rho " + std::to_string(rho) + " must be > 0");
        }
        if (p < 0.0)
        {
            throw std::invalid_argument("EulerCore::add_bc: inlet pressure " + std::to_string(p) + " must be >= 0");
        }
    }
    m_bcs.push_back(EulerBoundary{kind, faces, value});
    m_bc_dirty = true;
}

void EulerCoreBase::clear_bc()
{
    m_bcs.clear();
    m_bc_dirty = true;
}

// normal_matrix (euler_bc.cpp:87-128): rows are the outward unit normal and a
// tangent basis.
void EulerCoreBase::normal_matrix(int32_t ifc, double * out) const
{
    if (ifc < 0 || ifc >= m_nface)
    {
        throw std::out_of_range("EulerCore: face " + std::to_string(ifc) + " out of range [0, " +
                                std::to_string(m_nface) + ")");
    }
    double const * n = &m_fcnml[static_cast<size_t>((ifc + m_ngstface) * ndim)];
    if (ndim == 2)
    {
        out[0] = n[0];
        out[1] = n[1];
        out[2] = -n[1];
        out[3] = n[0];
        return;
    }
    double axis[3] = {0.0, 0.0, 0.0};
    double const ax = std::fabs(n[0]), ay = std::fabs(n[1]), az = std::fabs(n[2]);
    if (ax <= ay && ax <= az)
        axis[0] = 1.0;
    else if (ay <= az)
        axis[1] = 1.0;
    else
        axis[2] = 1.0;
    double t1[3] = {n[1] * axis[2] - n[2] * axis[1], n[2] * axis[0] - n[0] * axis[2], n[0] * axis[1] - n[1] * axis[0]};
    double const len = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
    for (double & v : t1)
    {
        v /= len;
    }
    double const t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    for (int d = 0; d < 3; ++d)
    {
        out[d] = n[d];
        out[3 + d] = t1[d];
        out[6 + d] = t2[d];
    }
}

// --------------------------------------------------------------------------
// Templated implementation.

namespace
{

template <int ND, typename R, typename G>
class EulerCoreImpl : public EulerCoreBase
{
public:
    static constexpr int NEQ = ND + 2;
    static constexpr int RS = Rec<ND, R>::RS;
    static constexpr int KF = Geo<ND, G>::KF;

    EulerCoreImpl(HostMesh const & mesh, double dt, int prec)
    {
        ndim = ND;
        neq = NEQ;
        ncell = mesh.ncell;
        ngstcell = mesh.ngstcell;
        time_increment = dt;
        precision = prec;
        nrow = ncell + ngstcell;
        m_nface = mesh.nface;
        m_ngstface = mesh.ngstface;
        m_fccls.assign(mesh.fccls.buf.begin(), mesh.fccls.buf.end());
        m_fcnml.assign(mesh.fcnml.buf.begin(), mesh.fcnml.buf.end());
        m_stm.assign(static_cast<size_t>(nrow * NEQ), 0.0);
        cuda_check(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        stream = own_stream;

        // Mesh tables on the device.
        up(d_ndcrd, mesh.ndcrd.buf);
        up(d_fccnd, mesh.fccnd.buf);
        up(d_clcnd, mesh.clcnd.buf);
        up(d_fcnds, mesh.fcnds.buf);
        up(d_fccls, mesh.fccls.buf);
        up(d_clfcs, mesh.clfcs.buf);
        up(d_cltpn, mesh.cltpn.buf);
        up(d_clvol, mesh.clvol.buf);
        mv.ndim = ND;
        mv.ncell = ncell;
        mv.ngstcell = ngstcell;
        mv.ngstface = mesh.ngstface;
        mv.ngstnode = mesh.ngstnode;
        mv.ndcrd = d_ndcrd.ptr;
        mv.fccnd = d_fccnd.ptr;
        mv.clcnd = d_clcnd.ptr;
        mv.fcnds = d_fcnds.ptr;
        mv.fccls = d_fccls.ptr;
        mv.clfcs = d_clfcs.ptr;
        mv.cltpn = d_cltpn.ptr;

        validate_connectivity(mesh.nface, mesh.nnode);

        nslot = 0;
        for (int64_t icl = 0; icl < ncell; ++icl)
        {
            int32_t const t = mesh.cltpn(icl);
            bool ok = (ND == 2) ? (t == CT_TRIANGLE || t == CT_QUAD)
                                : (t == CT_TET || t == CT_HEX || t == CT_PRISM || t == CT_PYRAMID);
            if (!ok)
            {
                throw std::invalid_argument("EulerCore: cell " + std::to_string(icl) + " has type " +
                                            std::to_string(t) + " unsupported in " + std::to_string(ND) + "D");
            }
            nslot = std::max(nslot, static_cast<int>(mesh.clfcs(icl, 0)));
            single_ct = (icl == 0 || single_ct == t) ? t : -1;
        }

        // Solution state.
        for (auto & r : rec)
        {
            r.alloc(static_cast<size_t>(nrow * RS));
            cuda_check(cudaMemsetAsync(r.ptr, 0, r.bytes(), stream), "memset");
        }
        d_gamma.alloc(nrow);
        d_cflo.alloc(nrow);
        d_cflc.alloc(nrow);
        d_limiter.alloc(std::max<int64_t>(ncell, 1));
        cuda_check(cudaMemsetAsync(d_gamma.ptr, 0, d_gamma.bytes(), stream), "memset");
        cuda_check(cudaMemsetAsync(d_cflo.ptr, 0, d_cflo.bytes(), stream), "memset");
        cuda_check(cudaMemsetAsync(d_cflc.ptr, 0, d_cflc.bytes(), stream), "memset");
        cuda_check(cudaMemsetAsync(d_limiter.ptr, 0, d_limiter.bytes(), stream), "memset");
        if constexpr (sizeof(R) == 4)
        {
            d_comp.alloc(static_cast<size_t>(NEQ) * std::max<int64_t>(ncell, 1));
            cuda_check(cudaMemsetAsync(d_comp.ptr, 0, d_comp.bytes(), stream), "memset");
            comp_live = true;
        }

        // Boundary tables.
        d_gkind.alloc(std::max<int64_t>(ngstcell, 1));
        d_gnml.alloc(std::max<int64_t>(ngstcell * ND, 1));
        d_gval.alloc(std::max<int64_t>(ngstcell * NEQ, 1));
        d_gint.alloc(std::max<int64_t>(ngstcell, 1));

        // Geometry: prepare_ce, then the compact march tables.
        d_fgeo.alloc(static_cast<size_t>(std::max(nslot, 1)) * KF * std::max<int64_t>(ncell, 1));
        d_cgeo.alloc(static_cast<size_t>(Dim<ND>::KC) * std::max<int64_t>(ncell, 1));
        // Slots past a cell's own faces are never written; zero them so the
        // whole tables hold defined values (the FP32 form checks them all).
        cuda_check(cudaMemsetAsync(d_fgeo.ptr, 0, d_fgeo.bytes(), stream), "memset");
        cuda_check(cudaMemsetAsync(d_cgeo.ptr, 0, d_cgeo.bytes(), stream), "memset");
        d_nbr.alloc(static_cast<size_t>(std::max(nslot, 1)) * std::max<int64_t>(ncell, 1));
        d_ctype.alloc(std::max<int64_t>(ncell, 1));
        prepare_ce(true);
        upload_bc();
        sync();
    }

    ~EulerCoreImpl() override
    {
        for (auto & pr : prof_events)
        {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
        if (own_stream)
        {
            cudaStreamSynchronize(own_stream);
            cudaStreamDestroy(own_stream);
        }
        if (m_xfer)
        {
            cudaStreamSynchronize(m_xfer);
            cudaStreamDestroy(m_xfer);
        }
        if (m_side)
        {
            cudaStreamSynchronize(m_side);
            cudaStreamDestroy(m_side);
        }
        if (m_cev)
        {
            cudaEventDestroy(m_cev);
        }
        for (auto & e : m_xev)
        {
            if (e)
            {
                cudaEventDestroy(e);
            }
        }
    }

    size_t device_bytes() const override
    {
        size_t b = 0;
        for (auto const & r : rec)
            b += r.bytes();
        b += d_fgeo.bytes() + d_cgeo.bytes() + d_nbr.bytes() + d_ctype.bytes();
        b += d_gamma.bytes() + d_cflo.bytes() + d_cflc.bytes() + d_comp.bytes();
        b += d_ndcrd.bytes() + d_fccnd.bytes() + d_clcnd.bytes() + d_fcnds.bytes() + d_fccls.bytes() +
             d_clfcs.bytes() + d_cltpn.bytes() + d_clvol.bytes();
        for (auto const & c : ce)
            b += c.bytes();
        return b;
    }

    // Every body cell's faces, their cells and nodes in range, and every face
    // shared with the cell that lists it, so no kernel can index outside a
    // table whatever a caller wrote into the mesh (checked on the device).
    void validate_connectivity(int64_t nface, int64_t nnode)
    {
        if (ncell == 0)
        {
            return;
        }
        DevBuf<unsigned long long> bad(1);
        unsigned long long const none = ~0ull;
        cuda_check(cudaMemcpyAsync(bad.ptr, &none, sizeof(none), cudaMemcpyHostToDevice, stream), "H2D");
        k_validate_mesh<<<grid_for(ncell), BLOCK, 0, stream>>>(mv, nface, nnode, bad.ptr);
        launched(stream, "validate_mesh");
        unsigned long long first = none;
        cuda_check(cudaMemcpyAsync(&first, bad.ptr, sizeof(first), cudaMemcpyDeviceToHost, stream), "D2H");
        sync();
        if (first != none)
        {
            throw std::invalid_argument("EulerCore: mesh connectivity of cell " + std::to_string(first) +
                                        " is inconsistent (a face, face cell or node out of range, or a face "
                                        "that does not have the cell)");
        }
    }

    void set_stream(cudaStream_t s) override
    {
        sync();
        stream = s ? s : own_stream;
    }

    void sync() override
    {
        cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        async_pending = false;
    }

    cudaStream_t get_stream() const override { return stream; }

    void profile(bool on) override
    {
        sync();
        for (auto & pr : prof_events)
        {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
        prof_events.clear();
        profiling = on;
    }

    void profile_stats(double * ms_total, int64_t * launches) override
    {
        sync();
        double tot = 0.0;
        for (auto & pr : prof_events)
        {
            float f = 0.f;
            cuda_check(cudaEventElapsedTime(&f, pr.first, pr.second), "elapsed");
            tot += f;
        }
        *ms_total = tot;
        *launches = static_cast<int64_t>(prof_events.size());
    }

    // ---- geometry -------------------------------------------------------

    // (Re)compute the reference-layout CE tables into ce[] and compact them.
    // When keep is false the big sub-face tables are released afterwards.
    void prepare_ce(bool drop_subface)
    {
        int64_t const tot = nrow;
        size_t const sz[4] = {static_cast<size_t>(tot * 7), static_cast<size_t>(tot * 7 * ND),
                              static_cast<size_t>(ncell * 24 * ND), static_cast<size_t>(ncell * 24 * ND)};
        for (int k = 0; k < 4; ++k)
        {
            if (ce[k].n != sz[k])
            {
                ce[k].alloc(sz[k]);
            }
            if (ce[k].ptr)
            {
                cuda_check(cudaMemsetAsync(ce[k].ptr, 0, ce[k].bytes(), stream), "memset");
            }
        }
        if (ncell > 0)
        {
            CeView v{ce[0].ptr, ce[1].ptr, ce[2].ptr, ce[3].ptr};
            if constexpr (ND == 2)
                k_prepare_ce_2d<<<grid_for(ncell), BLOCK, 0, stream>>>(mv, v);
            else
                k_prepare_ce_3d<<<grid_for(ncell), BLOCK, 0, stream>>>(mv, v);
            launched(stream, "prepare_ce");
        }
        compact();
        if (drop_subface)
        {
            sync();
            ce[2].release();
            ce[3].release();
        }
    }

    void ensure_ce()
    {
        if (!ce[2].ptr && ncell > 0)
        {
            // Recompute the sub-face tables without touching cevol/cecnd,
            // which the caller may have overwritten.
            DevBuf<double> t0(static_cast<size_t>(nrow * 7)), t1(static_cast<size_t>(nrow * 7 * ND));
            ce[2].alloc(static_cast<size_t>(ncell * 24 * ND));
            ce[3].alloc(static_cast<size_t>(ncell * 24 * ND));
            cuda_check(cudaMemsetAsync(ce[2].ptr, 0, ce[2].bytes(), stream), "memset");
            cuda_check(cudaMemsetAsync(ce[3].ptr, 0, ce[3].bytes(), stream), "memset");
            CeView v{t0.ptr, t1.ptr, ce[2].ptr, ce[3].ptr};
            if constexpr (ND == 2)
                k_prepare_ce_2d<<<grid_for(ncell), BLOCK, 0, stream>>>(mv, v);
            else
                k_prepare_ce_3d<<<grid_for(ncell), BLOCK, 0, stream>>>(mv, v);
            launched(stream, "prepare_ce");
            sync();
        }
    }

    void compact()
    {
        m_plan.valid = false;
        if (ncell == 0)
        {
            return;
        }
        ensure_ce();
        k_compact<ND, G><<<grid_for(ncell), BLOCK, 0, stream>>>(mv, ce[0].ptr, ce[1].ptr, ce[2].ptr, ce[3].ptr,
                                                                0.5 * time_increment, std::max(nslot, 1),
                                                                d_fgeo.ptr, d_cgeo.ptr, d_nbr.ptr, d_ctype.ptr);
        launched(stream, "compact");
        if constexpr (sizeof(R) == 4 && sizeof(G) == 8)
        {
            check_geometry_range();
        }
    }

    // The FP32 march rounds its FP64 geometry without range selects
    // (scg::dev::geo_r): refuse tables holding values it does not take.
    void check_geometry_range()
    {
        DevBuf<unsigned long long> bad(1);
        cuda_check(cudaMemsetAsync(bad.ptr, 0, sizeof(unsigned long long), stream), "memset");
        for (auto const * t : {&d_fgeo, &d_cgeo})
        {
            int64_t const n = static_cast<int64_t>(t->bytes() / sizeof(G));
            int64_t const blocks = std::min<int64_t>((n + BLOCK - 1) / BLOCK, 4096);
            k_geo_range<<<static_cast<unsigned>(std::max<int64_t>(blocks, 1)), BLOCK, 0, stream>>>(
                reinterpret_cast<double const *>(t->ptr), n, bad.ptr);
            launched(stream, "geo_range");
        }
        unsigned long long cnt = 0;
        cuda_check(cudaMemcpyAsync(&cnt, bad.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, stream), "D2H");
        sync();
        if (cnt)
        {
            throw std::invalid_argument("EulerCore: precision fp32 keeps FP64 geometry and uses it in FP32; " +
                                        std::to_string(cnt) +
                                        " geometry values of this mesh lie beyond FP32's range (magnitude 2^128 "
                                        "or more, infinite or NaN): use precision fp64, or rescale the mesh");
        }
    }

    // ---- boundary conditions ---------------------------------------------

    void upload_bc()
    {
        if (!m_bc_dirty)
        {
            return;
        }
        std::vector<int8_t> kind(static_cast<size_t>(ngstcell), -1);
        std::vector<double> nml(static_cast<size_t>(ngstcell * ND), 0.0);
        std::vector<double> val(static_cast<size_t>(ngstcell * NEQ), 0.0);
        std::vector<int32_t> gint(static_cast<size_t>(ngstcell), 0);
        // Later registrations override earlier ones for a face, as the
        // reference's sequential trim passes do.
        for (auto const & b : m_bcs)
        {
            double st[NEQ] = {};
            if (b.kind == BC_INLET)
            {
                double const rho = b.value[0];
                double const p = b.value[1 + ND];
                double const ga = b.value[2 + ND];
                double vsq = 0.0;
                for (int d = 0; d < ND; ++d)
                {
                    vsq += b.value[1 + d] * b.value[1 + d];
                }
                st[0] = rho;
                for (int d = 0; d < ND; ++d)
                {
                    st[1 + d] = rho * b.value[1 + d];
                }
                st[NEQ - 1] = p / (ga - 1.0) + 0.5 * rho * vsq;
            }
            for (int32_t const ifc : b.faces)
            {
                int32_t const icl = m_fccls[static_cast<size_t>((ifc + m_ngstface) * 4 + 0)];
                int32_t const jcl = m_fccls[static_cast<size_t>((ifc + m_ngstface) * 4 + 1)];
                int64_t const g = jcl + ngstcell;
                if (g < 0 || g >= ngstcell)
                {
                    throw std::runtime_error("EulerCore: boundary face " + std::to_string(ifc) +
                                             " has no ghost cell; build the ghost layer first");
                }
                if (icl < 0 || icl >= ncell)
                {
                    throw std::invalid_argument("EulerCore: boundary face " + std::to_string(ifc) +
                                                " has no interior cell (fccls[0] = " + std::to_string(icl) + ")");
                }
                kind[g] = static_cast<int8_t>(b.kind);
                gint[g] = static_cast<int32_t>(icl + ngstcell);
                for (int d = 0; d < ND; ++d)
                {
                    nml[g * ND + d] = m_fcnml[static_cast<size_t>((ifc + m_ngstface) * ND + d)];
                }
                for (int i = 0; i < NEQ; ++i)
                {
                    val[g * NEQ + i] = st[i];
                }
            }
        }
        if (ngstcell > 0)
        {
            h2d(d_gkind.ptr, kind.data(), kind.size());
            h2d(d_gnml.ptr, nml.data(), nml.size());
            h2d(d_gval.ptr, val.data(), val.size());
            h2d(d_gint.ptr, gint.data(), gint.size());
            sync();
        }
        m_bc_dirty = false;
        next_valid = false;
    }

    // ---- state access ----------------------------------------------------

    MarchArgs<R, G> args()
    {
        MarchArgs<R, G> a{};
        a.cur = rec[cur].ptr;
        a.nxt = rec[cur ^ 1].ptr;
        a.gamma = d_gamma.ptr;
        a.cflo = d_cflo.ptr;
        a.cflc = d_cflc.ptr;
        a.fgeo = d_fgeo.ptr;
        a.cgeo = d_cgeo.ptr;
        a.nbr = d_nbr.ptr;
        a.ctype = d_ctype.ptr;
        a.gkind = d_gkind.ptr;
        a.gnml = d_gnml.ptr;
        a.gval = d_gval.ptr;
        a.limiter = d_limiter.ptr;
        a.out0 = m_deliver_now ? m_deliver[0].dev : nullptr;
        a.out1 = m_deliver_now ? m_deliver[1].dev : nullptr;
        a.comp = sizeof(R) == 4 ? d_comp.ptr : nullptr;
        a.ncell = ncell;
        a.ngst = ngstcell;
        a.dt = R(time_increment);
        a.hdt = R(time_increment * 0.5);
        a.qdt = R(time_increment * 0.25);
        a.sigma0 = R(sigma0);
        a.taumin = R(taumin);
        a.tauscale = R(tauscale);
        return a;
    }

    void field_of(int which, R *& base, int & off, int & width)
    {
        switch (which)
        {
        case EA_SO0C: base = rec[cur].ptr; off = 0; width = NEQ; break;
        case EA_SO0N: base = rec[cur ^ 1].ptr; off = 0; width = NEQ; break;
        case EA_SO0T: base = rec[tbuf].ptr; off = NEQ; width = NEQ; break;
        case EA_SO1C: base = rec[cur].ptr; off = 2 * NEQ; width = NEQ * ND; break;
        case EA_SO1N: base = rec[cur ^ 1].ptr; off = 2 * NEQ; width = NEQ * ND; break;
        default: throw std::invalid_argument("not a record field");
        }
    }

    void get_array(int which, double * out) override
    {
        upload_bc();
        int64_t const n = array_size(which);
        if (which == EA_STM)
        {
            std::memcpy(out, m_stm.data(), sizeof(double) * static_cast<size_t>(n));
            return;
        }
        if (n == 0)
        {
            return;
        }
        double * const tmp = staging(n);
        size_t const nb = static_cast<size_t>(n) * sizeof(double);
        if (which >= EA_CEVOL && which <= EA_SFNML)
        {
            ensure_ce();
            cuda_check(cudaMemcpyAsync(tmp, ce[which].ptr, nb, cudaMemcpyDeviceToDevice, stream), "copy");
        }
        else if (which == EA_CFLO || which == EA_CFLC || which == EA_GAMMA)
        {
            R const * src = which == EA_CFLO ? d_cflo.ptr : which == EA_CFLC ? d_cflc.ptr : d_gamma.ptr;
            k_to_f64<R><<<grid_for(n), BLOCK, 0, stream>>>(src, tmp, n);
            launched(stream, "to_f64");
        }
        else
        {
            R * base;
            int off, width;
            field_of(which, base, off, width);
            if (double * const dev = static_cast<double *>(mapped_host(out, nb)))
            {
                // Mapped host table: the gather writes it directly.
                k_get_field_host<ND, R><<<grid_for((n + 1) / 2), BLOCK, 0, stream>>>(
                    base, dev, nrow, off, width, reinterpret_cast<uintptr_t>(dev) % 16 == 0, so0_residual(which));
                launched(stream, "get_field_host");
                sync();
                return;
            }
            k_get_field<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(base, tmp, nrow, off, width,
                                                                     so0_residual(which));
            launched(stream, "get_field");
        }
        cuda_check(cudaMemcpyAsync(out, tmp, nb, cudaMemcpyDeviceToHost, stream), "D2H");
        sync();
    }

    void set_array(int which, double const * in) override
    {
        upload_bc();
        int64_t const n = array_size(which);
        if (which == EA_STM)
        {
            std::memcpy(m_stm.data(), in, sizeof(double) * static_cast<size_t>(n));
            return;
        }
        if (n == 0)
        {
            return;
        }
        size_t const nb = static_cast<size_t>(n) * sizeof(double);
        if (which >= EA_SO0C && which <= EA_SO1N)
        {
            if (double const * const dev = static_cast<double const *>(mapped_host(in, nb)))
            {
                // Mapped host table: the scatter reads it directly.
                R * base;
                int off, width;
                field_of(which, base, off, width);
                if (which == EA_SO1N && tbuf != (cur ^ 1))
                {
                    // The new state's so0t can go into its record (the
                    // logical so0t lives in the other buffer): make it now.
                    k_set_so1_host_solt<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(
                        base, dev, d_gamma.ptr, nrow, reinterpret_cast<uintptr_t>(dev) % 16 == 0);
                    launched(stream, "set_so1_host_solt");
                    next_valid = true;
                    next_buf = cur ^ 1;
                }
                else
                {
                    k_set_field_host<ND, R><<<grid_for((n + 1) / 2), BLOCK, 0, stream>>>(
                        base, dev, nrow, off, width, reinterpret_cast<uintptr_t>(dev) % 16 == 0,
                        so0_written(which));
                    launched(stream, "set_field_host");
                    next_valid = false;
                }
                sync();
                return;
            }
        }
        double * const tmp = staging(n);
        cuda_check(cudaMemcpyAsync(tmp, in, nb, cudaMemcpyHostToDevice, stream), "H2D");
        if (which >= EA_CEVOL && which <= EA_SFNML)
        {
            ensure_ce();
            cuda_check(cudaMemcpyAsync(ce[which].ptr, tmp, nb, cudaMemcpyDeviceToDevice, stream), "copy");
            compact();
        }
        else if (which == EA_CFLO || which == EA_CFLC || which == EA_GAMMA)
        {
            R * dst = which == EA_CFLO ? d_cflo.ptr : which == EA_CFLC ? d_cflc.ptr : d_gamma.ptr;
            k_from_f64<R><<<grid_for(n), BLOCK, 0, stream>>>(tmp, dst, n);
            launched(stream, "from_f64");
        }
        else
        {
            R * base;
            int off, width;
            field_of(which, base, off, width);
            k_set_field<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(base, tmp, nrow, off, width,
                                                                     so0_written(which));
            launched(stream, "set_field");
        }
        next_valid = false;
        sync();
    }

    void init_solution(double gamma, double rho, double const * v, double p) override
    {
        if (gamma <= 1.0)
        {
            throw std::invalid_argument("EulerCore::init_solution: gamma " + std::to_string(gamma) + " must be > 1");
        }
        if (rho <= 0.0)
        {
            throw std::invalid_argument("EulerCore::init_solution: rho " + std::to_string(rho) + " must be > 0");
        }
        if (p < 0.0)
        {
            throw std::invalid_argument("EulerCore::init_solution: pressure " + std::to_string(p) +
                                        " must be >= 0");
        }
        double vsq = 0.0;
        for (int d = 0; d < ND; ++d)
        {
            vsq += v[d] * v[d];
        }
        double const energy = p / (gamma - 1.0) + 0.5 * rho * vsq;
        if (nrow > 0)
        {
            k_init<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(rec[cur ^ 1].ptr, d_gamma.ptr, ngstcell, nrow, gamma,
                                                                 rho, rho * v[0], rho * v[1],
                                                                 ND == 3 ? rho * v[2] : 0.0, energy);
            launched(stream, "init_solution");
        }
        comp_live = false;
        next_valid = false;
        sync();
    }

    // ---- operations ------------------------------------------------------

    // Make rec[cur].so0t the logical so0t (copy it over if update() moved
    // the current buffer away from it).
    void so0t_to_cur()
    {
        if (tbuf != cur)
        {
            k_copy_field<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(rec[tbuf].ptr, rec[cur].ptr, nrow, NEQ, NEQ);
            launched(stream, "copy_so0t");
            tbuf = cur;
        }
    }

    void run_solt()
    {
        k_solt_rows<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(rec[cur].ptr, d_gamma.ptr, nrow);
        launched(stream, "calc_solt");
        tbuf = cur;
    }

    void op(int which) override
    {
        upload_bc();
        bool const has_cells = ncell > 0;
        switch (which)
        {
        case EO_PREPARE_CE:
            prepare_ce(false);
            break;
        case EO_UPDATE:
            cur ^= 1;
            comp_live = false; // the residual was so0n's, which is now so0c
            break;
        case EO_CALC_SOLT:
            if (nrow > 0)
                run_solt();
            next_valid = false;
            break;
        case EO_CALC_SOLN:
            so0t_to_cur();
            if (has_cells)
            {
                k_soln<ND, R, G><<<grid_for(ncell), BLOCK, 0, stream>>>(args());
                launched(stream, "calc_soln");
            }
            comp_live = false;
            next_valid = false;
            break;
        case EO_BC_SOLN:
            if (ngstcell > 0)
            {
                k_bc0<ND, R, G><<<grid_for(ngstcell), BLOCK, 0, stream>>>(args(), d_gint.ptr);
                launched(stream, "bc_soln");
            }
            next_valid = false;
            break;
        case EO_CALC_CFL:
            if (has_cells)
            {
                k_cfl<ND, R, G><<<grid_for(ncell), BLOCK, 0, stream>>>(args());
                launched(stream, "calc_cfl");
            }
            comp_live = false; // a rewritten energy no longer has its residual
            next_valid = false;
            break;
        case EO_CALC_DSOLN:
            so0t_to_cur();
            if (has_cells)
            {
                k_dsoln<ND, R, G><<<grid_for(ncell), BLOCK, 0, stream>>>(args());
                launched(stream, "calc_dsoln");
            }
            next_valid = false;
            break;
        case EO_BC_DSOLN:
            if (ngstcell > 0)
            {
                k_bc1<ND, R, G><<<grid_for(ngstcell), BLOCK, 0, stream>>>(args(), d_gint.ptr);
                launched(stream, "bc_dsoln");
            }
            next_valid = false;
            break;
        case EO_MARCH_SUBSTEP:
            march_substep();
            break;
        case EO_RESET_STATE:
            for (auto & r : rec)
            {
                cuda_check(cudaMemsetAsync(r.ptr, 0, r.bytes(), stream), "memset");
            }
            cuda_check(cudaMemsetAsync(d_gamma.ptr, 0, d_gamma.bytes(), stream), "memset");
            cuda_check(cudaMemsetAsync(d_cflo.ptr, 0, d_cflo.bytes(), stream), "memset");
            cuda_check(cudaMemsetAsync(d_cflc.ptr, 0, d_cflc.bytes(), stream), "memset");
            cuda_check(cudaMemsetAsync(d_limiter.ptr, 0, d_limiter.bytes(), stream), "memset");
            std::fill(m_stm.begin(), m_stm.end(), 0.0);
            cur = 0;
            tbuf = 0;
            next_valid = false;
            next_buf = 1;
            comp_live = false;
            break;
        default:
            throw std::invalid_argument("EulerCore: unknown operation " + std::to_string(which));
        }
        sync();
    }

    // march_substep (euler_march.cpp:339-348) as update() plus one fused
    // kernel; calc_solt runs only when the previous fused kernel did not
    // already leave it in the new current buffer.
    void march_substep()
    {
        comp_ready();
        cur ^= 1;
        if (next_valid && next_buf == cur)
        {
            tbuf = cur;
        }
        else if (nrow > 0)
        {
            run_solt();
        }
        if (nrow > 0)
        {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (profiling)
            {
                cuda_check(cudaEventCreate(&e0), "event");
                cuda_check(cudaEventCreate(&e1), "event");
                cuda_check(cudaEventRecord(e0, stream), "record");
            }
            launch_fused();
            launched(stream, "fused_substep");
            if (profiling)
            {
                cuda_check(cudaEventRecord(e1, stream), "record");
                prof_events.emplace_back(e0, e1);
            }
            next_valid = true;
            next_buf = cur ^ 1;
        }
    }

    // The fused kernel specialised to the mesh's cell type when it has only
    // triangles or only tetrahedra (the simplex paths), else the generic one,
    // over rows [t0, t1) of its work order (body cells, then ghost rows).
    void launch_fused(int64_t t0 = 0, int64_t t1 = -1)
    {
        if (t1 < 0)
        {
            t1 = nrow;
        }
        if (t1 <= t0)
        {
            return;
        }
        unsigned const g = grid_for(t1 - t0);
        constexpr int SIMPLEX = (ND == 2) ? CT_TRIANGLE : CT_TET;
        if (single_ct == SIMPLEX)
        {
            constexpr int MINB = min_blocks<ND, R, SIMPLEX, BLOCK, G>();
            if constexpr (MINB > 0)
            {
                k_fused_mb<ND, R, G, SIMPLEX, MINB><<<g, BLOCK, 0, stream>>>(args(), t0, t1);
            }
            else
            {
                k_fused<ND, R, G, SIMPLEX><<<g, BLOCK, 0, stream>>>(args(), t0, t1);
            }
        }
        else
        {
            k_fused<ND, R, G><<<g, BLOCK, 0, stream>>>(args(), t0, t1);
        }
    }

    void march(int64_t steps) override
    {
        upload_bc();
        // FP64: the last substep's kernel writes the rows itself, hidden
        // under its FP64 arithmetic.  FP32: the march is bound by load
        // latency and its per-row host stores would not coalesce into whole
        // lines, so the delivery is a coalesced gather queued after it.
        bool const delivers = steps > 0 && nrow > 0 && revalidate_delivery();
        constexpr bool IN_KERNEL = sizeof(R) == 8;
        for (int64_t s = 0; s < steps; ++s)
        {
            march_substep();
            m_deliver_now = IN_KERNEL && delivers && s + 1 == steps;
            march_substep();
            m_deliver_now = false;
        }
        gather_delivery(delivers);
        async_pending = steps > 0 && nrow > 0;
    }

    // FP32: the registered host blocks receive the state after the march.
    void gather_delivery(bool delivers)
    {
        if constexpr (sizeof(R) == 8)
        {
            (void)delivers;
            return;
        }
        if (!delivers)
        {
            return;
        }
        for (int k = 0; k < 2; ++k)
        {
            Delivery const & d = m_deliver[k];
            if (d.host)
            {
                R * base;
                int off, width;
                field_of(k == 0 ? EA_SO0N : EA_SO1N, base, off, width);
                int64_t const n = static_cast<int64_t>(d.nbytes / sizeof(double));
                k_get_field_host<ND, R><<<grid_for((n + 1) / 2), BLOCK, 0, stream>>>(
                    base, d.dev, nrow, off, width, true, so0_residual(k == 0 ? EA_SO0N : EA_SO1N));
                launched(stream, "get_field_host");
            }
        }
    }

    // set_array(so0n), set_array(so1n) and march(steps), with the state's
    // upload overlapped with the first substep when both tables lie in
    // scg_host_alloc blocks (page-locked): the upload runs in row chunks on a
    // second stream, and the first substep's fused kernel runs in the
    // matching cell chunks, each after the upload of every row its cells read
    // (the chunk plan).  Same values through the same kernels: the state it
    // leaves is set + march's, bit for bit.
    void march_from_host(double const * so0n, double const * so1n, int64_t steps) override
    {
        size_t const nb0 = sizeof(double) * static_cast<size_t>(array_size(EA_SO0N));
        size_t const nb1 = sizeof(double) * static_cast<size_t>(array_size(EA_SO1N));
        double const * const d0 = static_cast<double const *>(mapped_host(so0n, nb0));
        double const * const d1 = static_cast<double const *>(mapped_host(so1n, nb1));
        // FP32: the march takes a fraction of the link's time, so there is
        // nothing to hide the upload under (set_array's mapped scatter is the
        // faster route).
        if (!d0 || !d1 || steps <= 0 || ncell == 0 || sizeof(R) == 4)
        {
            set_array(EA_SO0N, so0n);
            set_array(EA_SO1N, so1n);
            march(steps);
            return;
        }
        upload_bc();
        bool const delivers = revalidate_delivery();
        constexpr bool IN_KERNEL = sizeof(R) == 8;
        plan_chunks();
        int const nch = m_plan.nch;
        // The upload: the copy engine moves each chunk's rows of the two
        // pinned tables into a device table (no SM takes part, so the
        // substep marches beside it), and a scatter at HBM speed puts them
        // into the records, so0t made on the way, as set_array does for a
        // mapped table.
        constexpr int W = NEQ * ND;
        double * const st0 = staging(nrow * (NEQ + W));
        double * const st1 = st0 + nrow * NEQ;
        // The records it writes may still be read by work queued on the
        // core's stream (an earlier march): that goes first.
        cuda_check(cudaEventRecord(m_xev[XCH], stream), "record");
        cuda_check(cudaStreamWaitEvent(m_xfer, m_xev[XCH], 0), "wait");
        R * base;
        int off, width;
        field_of(EA_SO0N, base, off, width);
        bool const solt = tbuf != (cur ^ 1);
        Residual const c = so0_written(EA_SO0N);
        for (int j = 0; j < nch; ++j)
        {
            int64_t const r0 = j == 0 ? 0 : ngstcell + m_plan.cell[j];
            int64_t const r1 = ngstcell + m_plan.cell[j + 1];
            int64_t const nr = r1 - r0;
            double * const in0 = st0 + r0 * NEQ;
            double * const in1 = st1 + r0 * W;
            cuda_check(cudaMemcpyAsync(in0, so0n + r0 * NEQ, sizeof(double) * static_cast<size_t>(nr * NEQ),
                                       cudaMemcpyHostToDevice, m_xfer),
                       "H2D");
            cuda_check(cudaMemcpyAsync(in1, so1n + r0 * W, sizeof(double) * static_cast<size_t>(nr * W),
                                       cudaMemcpyHostToDevice, m_xfer),
                       "H2D");
            k_set_field_host<ND, R><<<grid_for((nr * NEQ + 1) / 2), BLOCK, 0, m_xfer>>>(
                base + r0 * RS, in0, nr, 0, NEQ, reinterpret_cast<uintptr_t>(in0) % 16 == 0,
                Residual{c.comp, c.ngst - r0, c.ncell});
            launched(m_xfer, "set_field_host");
            if (solt)
            {
                k_set_so1_host_solt<ND, R><<<grid_for(nr), BLOCK, 0, m_xfer>>>(
                    base + r0 * RS, in1, d_gamma.ptr + r0, nr, reinterpret_cast<uintptr_t>(in1) % 16 == 0);
                launched(m_xfer, "set_so1_host_solt");
            }
            else
            {
                k_set_field_host<ND, R><<<grid_for((nr * W + 1) / 2), BLOCK, 0, m_xfer>>>(
                    base + r0 * RS, in1, nr, 2 * NEQ, W, reinterpret_cast<uintptr_t>(in1) % 16 == 0, Residual{});
                launched(m_xfer, "set_field_host");
            }
            cuda_check(cudaEventRecord(m_xev[j], m_xfer), "record");
        }
        // What the two sets leave behind.
        next_valid = solt;
        next_buf = cur ^ 1;
        // The first substep, as march_substep with its fused launch in
        // chunks.
        comp_ready();
        cur ^= 1;
        if (next_valid && next_buf == cur)
        {
            tbuf = cur;
        }
        else
        {
            cuda_check(cudaStreamWaitEvent(stream, m_xev[nch - 1], 0), "wait");
            run_solt();
        }
        m_deliver_now = false;
        // The chunks write disjoint rows, so they alternate between the
        // core's stream and a second one: a chunk's last partial wave
        // overlaps the next chunk instead of idling SMs.
        cuda_check(cudaEventRecord(m_cev, stream), "record");
        cuda_check(cudaStreamWaitEvent(m_side, m_cev, 0), "wait");
        cudaStream_t const mine = stream;
        {
            // The core's stream is back to its own even if a launch throws.
            struct Restore
            {
                cudaStream_t & s;
                cudaStream_t v;
                ~Restore() { s = v; }
            } const restore{stream, mine};
            for (int k = 0; k < nch; ++k)
            {
                stream = (k & 1) ? m_side : mine;
                cuda_check(cudaStreamWaitEvent(stream, m_xev[m_plan.need[k]], 0), "wait");
                launch_fused(m_plan.cell[k], m_plan.cell[k + 1]);
                launched(stream, "fused_substep");
            }
        }
        cuda_check(cudaEventRecord(m_cev, m_side), "record");
        cuda_check(cudaStreamWaitEvent(stream, m_cev, 0), "wait");
        cuda_check(cudaStreamWaitEvent(stream, m_xev[nch - 1], 0), "wait");
        if (ngstcell > 0)
        {
            launch_fused(ncell, nrow); // ghost rows without a boundary condition
            launched(stream, "fused_substep");
        }
        next_valid = true;
        next_buf = cur ^ 1;
        // Its second substep and the remaining steps.
        m_deliver_now = IN_KERNEL && delivers && steps == 1;
        march_substep();
        m_deliver_now = false;
        for (int64_t s = 1; s < steps; ++s)
        {
            march_substep();
            m_deliver_now = IN_KERNEL && delivers && s + 1 == steps;
            march_substep();
            m_deliver_now = false;
        }
        gather_delivery(delivers);
        async_pending = true;
    }

    // Cell chunks of the overlapped first substep and, for each, the last
    // upload chunk it must wait for: the one holding the highest row any of
    // its cells reads (its own rows and its neighbours'; ghost rows lie in
    // upload chunk 0).  Made once per mesh on the device.
    void plan_chunks()
    {
        if (m_plan.valid)
        {
            return;
        }
        if (!m_xfer)
        {
            cuda_check(cudaStreamCreateWithFlags(&m_xfer, cudaStreamNonBlocking), "cudaStreamCreate");
            cuda_check(cudaStreamCreateWithFlags(&m_side, cudaStreamNonBlocking), "cudaStreamCreate");
            cuda_check(cudaEventCreateWithFlags(&m_cev, cudaEventDisableTiming), "event");
            for (auto & e : m_xev)
            {
                cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
            }
        }
        int64_t nch = ncell / 65536;
        nch = nch < 1 ? 1 : (nch > XCH ? XCH : nch);
        int64_t csize = (ncell + nch - 1) / nch;
        csize = (csize + BLOCK - 1) / BLOCK * BLOCK;
        nch = (ncell + csize - 1) / csize;
        m_plan.nch = static_cast<int>(nch);
        for (int64_t k = 0; k <= nch; ++k)
        {
            m_plan.cell[k] = k * csize < ncell ? k * csize : ncell;
        }
        DevBuf<int64_t> top(static_cast<size_t>(nch));
        k_chunk_top_row<<<static_cast<unsigned>(nch), 256, 0, stream>>>(d_nbr.ptr, d_ctype.ptr, ncell, csize,
                                                                          std::max(nslot, 1), ngstcell, top.ptr);
        launched(stream, "chunk_top_row");
        int64_t h[XCH];
        cuda_check(cudaMemcpyAsync(h, top.ptr, sizeof(int64_t) * static_cast<size_t>(nch), cudaMemcpyDeviceToHost,
                                   stream),
                   "D2H");
        sync();
        for (int64_t k = 0; k < nch; ++k)
        {
            int64_t const r = h[k] - ngstcell; // a body cell, or < 0: a ghost row
            int64_t const j = r < 0 ? 0 : r / csize;
            m_plan.need[k] = static_cast<int>(std::max(k, std::min(j, nch - 1)));
        }
        m_plan.valid = true;
    }

    bool delivering() override { return revalidate_delivery(); }

    void deliver(int which, double * host, int64_t count) override
    {
        if (which != EA_SO0N && which != EA_SO1N)
        {
            throw std::invalid_argument("EulerCore.deliver: only so0n and so1n are delivered");
        }
        Delivery & d = m_deliver[which == EA_SO0N ? 0 : 1];
        if (!host)
        {
            d = Delivery{};
            return;
        }
        if (count != array_size(which))
        {
            throw std::invalid_argument("EulerCore.deliver: count " + std::to_string(count) + " is not the array's " +
                                        std::to_string(array_size(which)));
        }
        size_t const nb = static_cast<size_t>(count) * sizeof(double);
        uint64_t serial = 0;
        void * const dev = mapped_host(host, nb, &serial);
        if (!dev || reinterpret_cast<uintptr_t>(dev) % 16 != 0)
        {
            throw std::invalid_argument("EulerCore.deliver: host must be a 16-byte aligned range of one "
                                        "scg_host_alloc block");
        }
        d = Delivery{host, static_cast<double *>(dev), nb, serial};
    }

    void limiter_mask(uint8_t * out) override
    {
        if (ncell > 0)
        {
            cuda_check(cudaMemcpyAsync(out, d_limiter.ptr, static_cast<size_t>(ncell), cudaMemcpyDeviceToHost, stream),
                       "D2H");
        }
        sync();
    }

    void reduce(double * part_out, int & nblk)
    {
        nblk = static_cast<int>(std::min<int64_t>(std::max<int64_t>(grid_for(ncell), 1), 1024));
        DevBuf<double> part(static_cast<size_t>(nblk * (NEQ + 2)));
        k_totals<ND, R><<<nblk, BLOCK, 0, stream>>>(rec[cur ^ 1].ptr, d_clvol.ptr, d_cflo.ptr, ngstcell, ncell,
                                                   part.ptr, so0_residual(EA_SO0N));
        launched(stream, "totals");
        std::vector<double> h(static_cast<size_t>(nblk * (NEQ + 2)));
        cuda_check(cudaMemcpyAsync(h.data(), part.ptr, part.bytes(), cudaMemcpyDeviceToHost, stream), "D2H");
        sync();
        for (int i = 0; i < NEQ + 2; ++i)
        {
            part_out[i] = 0.0;
        }
        double c[NEQ] = {};
        part_out[NEQ] = 1.79769313486231570815e+308;
        part_out[NEQ + 1] = -1.79769313486231570815e+308;
        for (int b = 0; b < nblk; ++b)
        {
            for (int i = 0; i < NEQ; ++i)
            {
                double const y = h[static_cast<size_t>(b * (NEQ + 2) + i)] - c[i];
                double const t = part_out[i] + y;
                c[i] = (t - part_out[i]) - y;
                part_out[i] = t;
            }
            part_out[NEQ] = std::fmin(part_out[NEQ], h[static_cast<size_t>(b * (NEQ + 2) + NEQ)]);
            part_out[NEQ + 1] = std::fmax(part_out[NEQ + 1], h[static_cast<size_t>(b * (NEQ + 2) + NEQ + 1)]);
        }
    }

    void totals(double * out) override
    {
        double p[NEQ + 2];
        int nb = 0;
        reduce(p, nb);
        for (int i = 0; i < NEQ; ++i)
        {
            out[i] = p[i];
        }
    }

    void batch_begin() override
    {
        // The batch kernels run on the batch's stream, which is not ordered
        // with this core's: whatever this queues here (boundary tables, the
        // residual's reset, calc_solt) is waited for before returning.
        bool queued = m_bc_dirty;
        upload_bc();
        queued = comp_ready() || queued;
        // Exactly what the first substep of march() does before its fused
        // kernel, minus the buffer swap: so0t of the state in rec[cur ^ 1].
        if (!(next_valid && next_buf == (cur ^ 1)) && nrow > 0)
        {
            k_solt_rows<ND, R><<<grid_for(nrow), BLOCK, 0, stream>>>(rec[cur ^ 1].ptr, d_gamma.ptr, nrow);
            launched(stream, "calc_solt");
            next_valid = true;
            next_buf = cur ^ 1;
            queued = true;
        }
        // A march of this core, or a caller's stream, may also still run.
        if (queued || async_pending || stream != own_stream)
        {
            sync();
        }
    }

    void fill_args(int offset, void * out, size_t size) override
    {
        if (size != sizeof(MarchArgs<R, G>))
        {
            throw std::invalid_argument("EulerCore: argument block size mismatch");
        }
        int const saved = cur;
        cur ^= (offset & 1);
        MarchArgs<R, G> const a = args();
        cur = saved;
        std::memcpy(out, &a, sizeof(a));
    }

    void batch_end(int64_t steps) override
    {
        if (steps > 0)
        {
            // Two substeps per step leave cur unchanged; the second substep's
            // current buffer holds the logical so0t and the fused kernel left
            // the next so0t in the other buffer.
            tbuf = cur;
            next_valid = true;
            next_buf = cur ^ 1;
        }
    }

    StateView state_view() override
    {
        StateView v{};
        v.rec = rec[cur ^ 1].ptr;
        v.rec_stride = RS;
        v.neq = NEQ;
        v.fp32 = sizeof(R) == 4;
        v.clvol = d_clvol.ptr;
        v.ncell = ncell;
        v.ngstcell = ngstcell;
        v.stream = stream;
        v.comp = so0_residual(EA_SO0N).comp;
        return v;
    }

    void cfl_range(double * out) override
    {
        double p[NEQ + 2];
        int nb = 0;
        reduce(p, nb);
        out[0] = p[NEQ];
        out[1] = p[NEQ + 1];
    }

    void field(int which, double * out) override
    {
        if (which < 0 || which >= EF_COUNT || (which == EF_VELZ && ND != 3))
        {
            throw std::invalid_argument("EulerCore: unknown field " + std::to_string(which) + " in " +
                                        std::to_string(ND) + "D");
        }
        if (ncell == 0)
        {
            return;
        }
        double * d = staging(ncell);
        k_field<ND, R><<<grid_for(ncell), BLOCK, 0, stream>>>(rec[cur ^ 1].ptr, d_gamma.ptr, d_cflo.ptr, ngstcell,
                                                             ncell, which, d, so0_residual(EA_SO0N));
        launched(stream, "field");
        cuda_check(cudaMemcpyAsync(out, d, static_cast<size_t>(ncell) * sizeof(double), cudaMemcpyDeviceToHost,
                                   stream),
                   "D2H");
        sync();
    }

private:
    // Grow-only device staging table for get_array/set_array.
    double * staging(int64_t n)
    {
        if (m_staging.n < static_cast<size_t>(n))
        {
            sync();
            m_staging.alloc(static_cast<size_t>(n));
        }
        return m_staging.ptr;
    }

    template <typename T, typename A>
    void up(DevBuf<T> & d, std::vector<T, A> const & h)
    {
        d.alloc(std::max<size_t>(h.size(), 1));
        if (!h.empty())
        {
            h2d(d.ptr, h.data(), h.size());
        }
    }

    template <typename T>
    void h2d(T * dst, T const * src, size_t n)
    {
        cuda_check(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, stream), "H2D");
        cuda_check(cudaStreamSynchronize(stream), "sync");
    }

    int64_t nrow = 0;
    int nslot = 0;
    cudaStream_t own_stream = nullptr;
    // march_from_host: the upload stream, an event per upload chunk (and one
    // for the start), and the chunk plan.
    static constexpr int XCH = 16;
    cudaStream_t m_xfer = nullptr;
    cudaStream_t m_side = nullptr; // the second stream of the chunked substep
    cudaEvent_t m_cev = nullptr;
    cudaEvent_t m_xev[XCH + 1] = {};
    struct ChunkPlan
    {
        bool valid = false;
        int nch = 0;
        int64_t cell[XCH + 1] = {};
        int need[XCH] = {};
    } m_plan;
    cudaStream_t stream = nullptr;
    MeshView mv{};

    DevBuf<double> d_ndcrd, d_fccnd, d_clcnd, d_clvol;
    DevBuf<int32_t> d_fcnds, d_fccls, d_clfcs, d_cltpn;
    DevBuf<double> ce[4]; // cevol, cecnd, sfcnd, sfnml (reference layout)
    DevBuf<G> d_fgeo, d_cgeo;
    DevBuf<int32_t> d_nbr;
    DevBuf<int8_t> d_ctype;
    DevBuf<R> rec[2];
    DevBuf<R> d_gamma, d_cflo, d_cflc;
    // FP32: the rounding residual of so0n's body rows [NEQ][ncell], fed
    // back into each cell's next value by the march (fused_cell) and added to
    // so0n wherever so0n is read; valid while comp_live.  Anything other than
    // a march that changes so0n (or moves it, update()) drops it; the next
    // march starts it again from zero.
    DevBuf<R> d_comp;
    bool comp_live = false;

    Residual so0_residual(int which) const
    {
        Residual c;
        if (sizeof(R) == 4 && comp_live && which == EA_SO0N)
        {
            c.comp = d_comp.ptr;
            c.ngst = ngstcell;
            c.ncell = ncell;
        }
        return c;
    }

    // A write of a whole so0n table also writes the residual of each value.
    Residual so0_written(int which)
    {
        Residual c;
        if (sizeof(R) == 4 && which == EA_SO0N)
        {
            c.comp = d_comp.ptr;
            c.ngst = ngstcell;
            c.ncell = ncell;
            comp_live = true;
        }
        return c;
    }

    // Starts the residual from zero when it is not live; true when that
    // queued a memset on the core's stream.
    bool comp_ready()
    {
        if (sizeof(R) == 4 && !comp_live)
        {
            cuda_check(cudaMemsetAsync(d_comp.ptr, 0, d_comp.bytes(), stream), "memset");
            comp_live = true;
            return true;
        }
        return false;
    }

    // Host blocks a march also writes so0n / so1n into (deliver()).
    struct Delivery
    {
        double * host = nullptr;
        double * dev = nullptr;
        size_t nbytes = 0;
        uint64_t serial = 0;
    };
    Delivery m_deliver[2];
    bool m_deliver_now = false;

    // True when a delivery is registered; a block freed since registration
    // (or a new block at its address) is dropped, never written.
    bool revalidate_delivery()
    {
        bool any = false;
        for (Delivery & d : m_deliver)
        {
            if (!d.host)
            {
                continue;
            }
            uint64_t serial = 0;
            void * const dev = mapped_host(d.host, d.nbytes, &serial);
            if (dev != d.dev || serial != d.serial)
            {
                d = Delivery{};
                continue;
            }
            any = true;
        }
        return any;
    }
    DevBuf<uint8_t> d_limiter;
    DevBuf<int8_t> d_gkind;
    DevBuf<double> d_gnml, d_gval;
    DevBuf<int32_t> d_gint;
    DevBuf<double> m_staging;

    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;

    int cur = 0;           // index of the current (so0c/so1c) record buffer
    int tbuf = 0;          // buffer holding the logical so0t
    bool next_valid = false; // rec[next_buf].so0t (and its primitive cache) == calc_solt of rec[next_buf]
    bool async_pending = false; // march() returned with its kernels possibly still running
    int next_buf = 1;
};

} // namespace

std::unique_ptr<EulerCoreBase> make_euler_core(HostMesh const & mesh, double dt, int prec)
{
    if (mesh.ngstcell != mesh.nbound)
    {
        throw std::invalid_argument("EulerCore: the mesh needs build_boundary() and build_ghost() first");
    }
    if (prec < PREC_FP64 || prec > PREC_FP32)
    {
        throw std::invalid_argument("EulerCore: unknown precision " + std::to_string(prec));
    }
    if (mesh.ndim == 2)
    {
        if (prec == PREC_FP64)
            return std::make_unique<EulerCoreImpl<2, double, double>>(mesh, dt, prec);
        if (prec == PREC_FP32_GEOM64)
            return std::make_unique<EulerCoreImpl<2, float, double>>(mesh, dt, prec);
        return std::make_unique<EulerCoreImpl<2, float, float>>(mesh, dt, prec);
    }
    if (prec == PREC_FP64)
        return std::make_unique<EulerCoreImpl<3, double, double>>(mesh, dt, prec);
    if (prec == PREC_FP32_GEOM64)
        return std::make_unique<EulerCoreImpl<3, float, double>>(mesh, dt, prec);
    return std::make_unique<EulerCoreImpl<3, float, float>>(mesh, dt, prec);
}

} // namespace scg

namespace
{

// One FP64 geometry value per thread, rounded as the FP32 march rounds it.
__global__ void k_geo_round(double const * in, float * out, int64_t n)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = scg::dev::geo_r<float>(in[i]);
    }
}

} // namespace

extern "C" int scg_geometry_round(const double * in, float * out, int64_t n)
{
    return scg::guarded([&] {
        if (n < 0 || (n > 0 && (!in || !out)))
        {
            throw std::invalid_argument("scg_geometry_round: null buffer or negative count");
        }
        if (n == 0)
        {
            return;
        }
        scg::DevBuf<double> din(static_cast<size_t>(n));
        scg::DevBuf<float> dout(static_cast<size_t>(n));
        scg::cuda_check(cudaMemcpy(din.ptr, in, din.bytes(), cudaMemcpyHostToDevice), "H2D");
        int const block = 256;
        int64_t const grid = (n + block - 1) / block;
        k_geo_round<<<static_cast<unsigned>(grid), block>>>(din.ptr, dout.ptr, n);
        scg::launched(nullptr, "geometry_round");
        scg::cuda_check(cudaMemcpy(out, dout.ptr, dout.bytes(), cudaMemcpyDeviceToHost), "D2H");
    });
}
