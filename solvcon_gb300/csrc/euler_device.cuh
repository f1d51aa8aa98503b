#pragma once

/*
 * Device-side building blocks of the multi-dimensional CESE Euler march.
 *
 * The arithmetic is that of the reference EulerCore (cpp/solvcon/multidim/
 * euler_march.cpp, euler_solution.cpp, euler_gradient.cpp, euler_bc.cpp,
 * GradientElement.cpp) rearranged for a GPU whose FP64 pipe, not its HBM, is
 * the scarce resource:
 *
 *  - The flux Jacobian is never formed.  Every product J_d(u) . w the
 *    reference takes (euler_march.cpp:178-189, 280-292) is the directional
 *    derivative of the Euler flux f_d at u along w, evaluated here directly from
 *    primitive variables (jvp_sum).  Same mathematics, about a third of the
 *    operations.
 *  - The sub-face loop of calc_soln (euler_march.cpp:266-294) is linear in the
 *    sub-face centroids and normals, so each face's sub-faces are folded into
 *    two geometric moments at set-up: N = sum_sf n_sf and
 *    M[e][d] = sum_sf (x_sf - x_j)[e] n_sf[d] (pre-scaled by dt/2).
 *  - The gradient element (GradientElement.cpp:137-213) is linear in tau, so
 *    its displacement vectors are idis = P + tau Q - delta and
 *    jdis = R + tau Q - delta with P, Q, R precomputed per face; for simplices
 *    the sub-element centroid shift delta is exactly zero (the fan of a
 *    simplex about its vertex mean has equal sub-volumes).
 *  - Each fundamental gradient element's 2x2/3x3 solve
 *    (GradientElement.cpp:215-290) uses its inverse's rows once per cell,
 *    instead of an adjugate and determinant per equation.
 *
 * Results equal the reference's up to floating-point round-off.
 *
 * Storage (one record per mesh row, ghost rows first, row = icl + ngstcell):
 *   record[row] = { so0[NEQ], so0t[NEQ], so1[NEQ][ND], prim } padded to RS
 * reals, where prim (FP64 records only) caches the primitive variables of so0
 * (1/rho, v, p, E + p, |v|^2).  It is written with so0t, by the same thread
 * and from the same state, so it is valid exactly when so0t is; the fused
 * march then reads a neighbour's primitives instead of re-deriving them for
 * every face (a division and about twenty FP64 operations each).
 */

#include "divide.cuh"

#include <cstdint>

namespace scg
{
namespace dev
{

template <int ND>
struct Dim
{
    static constexpr int NEQ = ND + 2;
    static constexpr int RS = (ND == 2) ? 16 : 32; // record stride in reals
    static constexpr int OT = NEQ;                 // so0t offset
    static constexpr int O1 = 2 * NEQ;             // so1 offset
    // Cell geometry components: 1/cevol[0], hdt/dist.
    static constexpr int KC = 2;
};

// Per-face geometry components, stored as G: bvol, dB[ND] = x_BCE - x_nbr,
// Nh[ND], Mh[ND][ND], then either the gradient-element displacements P[ND],
// Q[ND], R[ND] (FP64 geometry) or mid[ND] = x_BCE - x_cell (FP32 geometry).
// P, Q and R follow from dB and mid with means over the cell's faces:
//   P = mid - mean(mid),  Q = mean(dB) - dB,  R = dB - mean(mid),
// which the memory-bound FP32 march forms in registers for 4 (2D) or 6 (3D)
// fewer stored values per face; the FP64 march, bound by its FP64 pipe,
// reads them.
template <int ND, typename G>
struct Geo
{
    static constexpr bool MID = sizeof(G) == 4;
    static constexpr int K_BVOL = 0;
    static constexpr int K_DB = 1;
    static constexpr int K_NH = 1 + ND;
    static constexpr int K_MH = 1 + 2 * ND;
    static constexpr int K_P = 1 + 2 * ND + ND * ND; // FP64 geometry
    static constexpr int K_Q = K_P + ND;
    static constexpr int K_R = K_Q + ND;
    static constexpr int K_MID = K_P; // FP32 geometry
    static constexpr int KF = MID ? K_MID + ND : K_R + ND;
};

// Record layout per dimension and state precision.
template <int ND, typename R>
struct Rec
{
    static constexpr int NEQ = ND + 2;
    static constexpr int NUSED = 2 * NEQ + NEQ * ND; // so0, so0t, so1: 16 / 25
    // Primitive cache (FP64 only: the FP64 march is bound by the FP64 pipe,
    // the FP32 march by memory, where the extra bytes would cost more).
    static constexpr bool PRIM = sizeof(R) == 8;
    static constexpr int OP = NUSED;    // cache offset: r, v[ND], p, h, vsq
    static constexpr int NPRIM = ND + 4;
    static constexpr int NLOAD = PRIM ? NUSED + NPRIM : NUSED;
    static constexpr int RS = (ND == 2) ? (PRIM ? 24 : 16) : 32;
    static_assert(NLOAD <= RS, "record overflow");
};

// Small constants of the reference, with FP32-safe floors.  The FP64 values
// are the reference's own (euler_march.cpp:30, euler_solution.cpp:108,
// euler_gradient.cpp:28); 1e-60 and 1e-200 underflow in FP32, so the FP32
// march uses the smallest floors that keep the same expressions finite.
template <typename R>
struct Tiny;
template <>
struct Tiny<double>
{
    static constexpr double JAC = 1.e-60;
    static constexpr double CFL = 1.e-60;
    static constexpr double AZ = 1.e-200;
};
template <>
struct Tiny<float>
{
    static constexpr float JAC = 1.e-30f;
    static constexpr float CFL = 1.e-30f;
    static constexpr float AZ = 1.e-37f;
};

// A geometry value (stored G) in the march's precision R.  FP64 geometry read
// by the FP32 march is rounded with integer instructions only: a double ->
// float conversion instruction issues on the FP64 pipe (16 cycles per warp on
// GB300, measured), and the FP32 march converts ~60 geometry values per
// cell-substep, which made that pipe the FP32 march's bottleneck.  In the
// FP32 normal range the result is IEEE round-to-nearest-even: adding
// 2^28 - 1 plus the kept part's lowest bit to the 64-bit pattern carries
// into bit 29 exactly when the 29 bits to be dropped exceed half, or equal
// half with an odd lowest kept bit; the funnel shift then takes bits 29..60,
// the exponent and the top 23 mantissa bits in place, and subtracting
// (1023 - 127) << 23 modulo 2^32 rebiases the exponent (its high bits
// shifted out cancel).  Values below the FP32 normal range (round-off
// residue in the tables) become a signed zero, by one compare and select.
// Larger ones are not taken here: a core of the FP32 form checks its
// geometry tables when it builds them (k_geo_range) and refuses values at
// 2^128 and beyond, infinities and NaNs, so the rounding needs no second
// range select (9 integer instructions per value instead of 15, for ~47
// values per cell-substep in 2D).  Branch-free, so nothing falls back to the
// conversion instruction.
// The geometry values geo_r takes: magnitudes below 2^128 (biased exponent
// up to 1150).
__device__ __forceinline__ bool geo_r_takes(double v)
{
    unsigned const e = (static_cast<unsigned>(__double2hiint(v)) >> 20) & 0x7FFu;
    return e <= 1150u;
}

template <typename R, typename G>
__device__ __forceinline__ R geo_r(G v)
{
    if constexpr (sizeof(R) == 4 && sizeof(G) == 8)
    {
        unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(v));
        unsigned const hi = static_cast<unsigned>(b >> 32);
        unsigned long long const t = b + 0x0FFFFFFFull + ((b >> 29) & 1ull);
        unsigned const r =
            __funnelshift_l(static_cast<unsigned>(t), static_cast<unsigned>(t >> 32), 3) - 0xC0000000u;
        return __uint_as_float(((hi & 0x7FF00000u) >= (897u << 20) ? r : 0u) | (hi & 0x80000000u));
    }
    else
    {
        return R(v);
    }
}

// Reciprocal square root: the library routine for each precision.
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

__device__ __forceinline__ double sqr_t(double x) { return sqrt(x); }
__device__ __forceinline__ float sqr_t(float x) { return sqrtf(x); }


// The march's reciprocals and quotients.  FP64: recip (Newton) and the
// division.  FP32 in 2D: the approximate quotient (div.approx.f32, one
// instruction and within 2 ulp for divisors of magnitude in [2^-126, 2^126];
// a zero divisor gives a signed infinity, or NaN over zero, as the division
// does), where a correctly rounded FP32 division is a multi-instruction
// sequence with a branch and the 2D march divides about a dozen times per
// cell-substep by densities, determinants, weight sums and CFL numbers, all
// far inside that range (2M triangles: 0.2352 -> 0.2155 ms per launch).
// FP32 in 3D: the division (with the approximate quotient the tetrahedron
// kernel ran 6.45 -> 8.59 ms per launch at the same registers, scheduled
// differently).
template <int ND>
__device__ __forceinline__ double mrecip(double d)
{
    return recip(d);
}
template <int ND>
__device__ __forceinline__ float mrecip(float d)
{
    if constexpr (ND == 2)
        return __fdividef(1.0f, d);
    else
        return 1.0f / d;
}
template <int ND>
__device__ __forceinline__ double mquot(double x, double y)
{
    return x / y;
}
template <int ND>
__device__ __forceinline__ float mquot(float x, float y)
{
    if constexpr (ND == 2)
        return __fdividef(x, y);
    else
        return x / y;
}

// Compensated (Kahan) accumulator for the FP32 flux sums; plain sum in FP64.
template <typename R>
struct Acc
{
    R s = R(0);
    __device__ __forceinline__ void add(R x) { s += x; }
    __device__ __forceinline__ R value() const { return s; }
};
template <>
struct Acc<float>
{
    float s = 0.f;
    float c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        float const y = x - c;
        float const t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s; }
};

// Primitive quantities of a conserved state u (with the reference's density
// floor TINY, euler_march.cpp:41).
template <int ND, typename R>
struct Prim
{
    R r;     // 1 / (rho + TINY)
    R v[ND]; // velocity
    R p;     // pressure
    R h;     // E + p
    R ga1;   // gamma - 1
    R vsq;   // |v|^2

    __device__ __forceinline__ Prim(R const * u, R ga) : Prim(u, ga, mrecip<ND>(u[0] + Tiny<R>::JAC)) {}

    // With 1/(rho + TINY) already at hand.
    __device__ __forceinline__ Prim(R const * u, R ga, R rinv)
    {
        constexpr int NEQ = ND + 2;
        r = rinv;
        R ke2 = R(0);
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            v[d] = u[1 + d] * r;
            ke2 += u[1 + d] * v[d];
        }
        vsq = ke2 * r;
        ga1 = ga - R(1);
        p = ga1 * (u[NEQ - 1] - R(0.5) * ke2);
        h = u[NEQ - 1] + p;
    }

    Prim() = default;

    // From a record's primitive cache (see Rec).
    __device__ __forceinline__ static Prim cached(R const * c, R ga)
    {
        Prim q;
        q.r = c[0];
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            q.v[d] = c[1 + d];
        }
        q.p = c[1 + ND];
        q.h = c[2 + ND];
        q.vsq = c[3 + ND];
        q.ga1 = ga - R(1);
        return q;
    }

    __device__ __forceinline__ void cache(R * c) const
    {
        c[0] = r;
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            c[1 + d] = v[d];
        }
        c[1 + ND] = p;
        c[2 + ND] = h;
        c[3 + ND] = vsq;
    }
};

// out[i] = sum_d f_d(u)[i] * n[d]  (the flux of euler_march.cpp:58-61, 120-124).
template <int ND, typename R>
__device__ __forceinline__ void flux_dot(Prim<ND, R> const & q, R const * u, R const * n, R * out)
{
    constexpr int NEQ = ND + 2;
    R mn = R(0);
    R vn = R(0);
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        mn += u[1 + d] * n[d];
        vn += q.v[d] * n[d];
    }
    out[0] = mn;
#pragma unroll
    for (int k = 0; k < ND; ++k)
    {
        out[1 + k] = u[1 + k] * vn + q.p * n[k];
    }
    out[NEQ - 1] = q.h * vn;
}

// out[i] += sum_d (J_d(u) . w[:, d])[i], with w indexed w[i * ND + d].  J_d is
// the analytic Euler flux Jacobian of euler_march.cpp:63-81 / 126-156; its
// product with w is taken as the directional derivative of f_d.
template <int ND, typename R>
__device__ __forceinline__ void jvp_sum(Prim<ND, R> const & q, R const * u, R const * w, R * out)
{
    constexpr int NEQ = ND + 2;
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        R const w0 = w[0 * ND + d];
        R const we = w[(NEQ - 1) * ND + d];
        R vw = R(0);
#pragma unroll
        for (int k = 0; k < ND; ++k)
        {
            vw += q.v[k] * w[(1 + k) * ND + d];
        }
        R const dp = q.ga1 * (we - vw + R(0.5) * q.vsq * w0);
        R const dvd = (w[(1 + d) * ND + d] - q.v[d] * w0) * q.r;
        out[0] += w[(1 + d) * ND + d];
#pragma unroll
        for (int k = 0; k < ND; ++k)
        {
            out[1 + k] += w[(1 + k) * ND + d] * q.v[d] + u[1 + k] * dvd;
        }
        out[1 + d] += dp;
        out[NEQ - 1] += (we + dp) * q.v[d] + q.h * dvd;
    }
}

// so0t = -(J . so1) for one row (euler_march.cpp:160-191), from the row's
// primitives q.
template <int ND, typename R>
__device__ __forceinline__ void solt_prim(Prim<ND, R> const & q, R const * u, R const * g, R * t)
{
    constexpr int NEQ = ND + 2;
    R o[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        o[i] = R(0);
    }
    jvp_sum<ND, R>(q, u, g, o);
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        t[i] = -o[i];
    }
}

template <int ND, typename R>
__device__ __forceinline__ void solt_row(R const * u, R const * g, R ga, R * t)
{
    solt_prim<ND, R>(Prim<ND, R>(u, ga), u, g, t);
}

// Fundamental gradient element tables (1-based in GradientElement.cpp:
// 16-79, 0-based here), per cell type.
template <int CT>
struct CellT;

template <>
struct CellT<4> // triangle
{
    static constexpr int ND = 2, NFC = 3, NFGE = 3;
    static constexpr bool SIMPLEX = true;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        return t[k][v];
    }
};
template <>
struct CellT<3> // quadrilateral
{
    static constexpr int ND = 2, NFC = 4, NFGE = 4;
    static constexpr bool SIMPLEX = false;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
        return t[k][v];
    }
};
template <>
struct CellT<6> // tetrahedron
{
    static constexpr int ND = 3, NFC = 4, NFGE = 4;
    static constexpr bool SIMPLEX = true;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[4][3] = {{2, 0, 1}, {1, 0, 3}, {3, 0, 2}, {1, 3, 2}};
        return t[k][v];
    }
};
template <>
struct CellT<5> // hexahedron
{
    static constexpr int ND = 3, NFC = 6, NFGE = 8;
    static constexpr bool SIMPLEX = false;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[8][3] = {{1, 2, 4}, {5, 2, 1}, {3, 2, 5}, {4, 2, 3},
                                 {4, 0, 1}, {1, 0, 5}, {5, 0, 3}, {3, 0, 4}};
        return t[k][v];
    }
};
template <>
struct CellT<7> // prism
{
    static constexpr int ND = 3, NFC = 5, NFGE = 6;
    static constexpr bool SIMPLEX = false;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[6][3] = {{4, 1, 3}, {2, 1, 4}, {3, 1, 2}, {3, 0, 4}, {4, 0, 2}, {2, 0, 3}};
        return t[k][v];
    }
};
template <>
struct CellT<8> // pyramid
{
    static constexpr int ND = 3, NFC = 5, NFGE = 6;
    static constexpr bool SIMPLEX = false;
    __device__ static constexpr int fge(int k, int v)
    {
        constexpr int t[6][3] = {{0, 4, 1}, {1, 4, 2}, {2, 4, 3}, {3, 4, 0}, {0, 2, 3}, {2, 0, 1}};
        return t[k][v];
    }
};

// Determinant of the rows a, b (, c).
template <int ND, typename R>
__device__ __forceinline__ R det_rows(R const * a, R const * b, R const * c)
{
    if constexpr (ND == 2)
    {
        (void)c;
        return a[0] * b[1] - a[1] * b[0];
    }
    else
    {
        return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
               a[2] * (b[0] * c[1] - b[1] * c[0]);
    }
}

// Kernel argument block shared by the march kernels.
template <typename R, typename G>
struct MarchArgs
{
    R const * cur;        // current records (so0c, so0t, so1c)
    R * nxt;              // new records (so0n, next so0t, so1n)
    R const * gamma;      // [nrow]
    R * cflo;             // [nrow]
    R * cflc;             // [nrow]
    G const * fgeo;       // [NSLOT][KF][ncell]
    G const * cgeo;       // [KC][ncell]
    int32_t const * nbr;  // [NSLOT][ncell] neighbour row
    int8_t const * ctype; // [ncell]
    int8_t const * gkind; // [ngst] BC kind of the ghost row, -1 if none
    double const * gnml;  // [ngst][ND] outward unit normal of the boundary face
    double const * gval;  // [ngst][NEQ] inlet conserved state
    uint8_t * limiter;    // [ncell] W-3/4 firing bits per equation, or null
    // Host blocks (mapped) that also receive every row's new so0n
    // [nrow][NEQ] and so1n [nrow][NEQ][ND] in FP64, or null.
    double * out0;
    double * out1;
    // FP32 march: the rounding residual of each body cell's so0 [NEQ][ncell],
    // fed back into the cell's next value (see fused_cell), or null.
    R * comp;
    int64_t ncell;
    int64_t ngst;
    R dt, hdt, qdt;
    R sigma0, taumin, tauscale;
};

} // namespace dev
} // namespace scg
