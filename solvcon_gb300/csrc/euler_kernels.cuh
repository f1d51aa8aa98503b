#pragma once

/*
 * The CESE march kernels of the multi-dimensional Euler core: per-cell device
 * routines for calc_soln, bc_soln, calc_cfl, calc_dsoln, bc_dsoln and calc_solt,
 * the fused one-kernel substep built from them, and the set-up kernels
 * (prepare_ce and the geometry compaction).  See euler_device.cuh for the data
 * layout and for how the arithmetic relates to the reference's.
 */

#include "euler_device.cuh"

#include <type_traits>

namespace scg
{
namespace dev
{

template <typename T>
__device__ __forceinline__ T ldg(T const * p)
{
    return __ldg(p);
}

// Load the first N reals of a record (default: so0, so0t, so1).
template <int ND, typename R, int N = Rec<ND, R>::NUSED>
__device__ __forceinline__ void load_rec(R const * base, R * out)
{
    if constexpr (sizeof(R) == 8)
    {
        double2 const * p = reinterpret_cast<double2 const *>(base);
#pragma unroll
        for (int k = 0; k < N / 2; ++k)
        {
            double2 const v = __ldg(p + k);
            out[2 * k] = v.x;
            out[2 * k + 1] = v.y;
        }
        if constexpr (N % 2)
        {
            out[N - 1] = __ldg(base + N - 1);
        }
    }
    else
    {
        float4 const * p = reinterpret_cast<float4 const *>(base);
#pragma unroll
        for (int k = 0; k < N / 4; ++k)
        {
            float4 const v = __ldg(p + k);
            out[4 * k] = v.x;
            out[4 * k + 1] = v.y;
            out[4 * k + 2] = v.z;
            out[4 * k + 3] = v.w;
        }
#pragma unroll
        for (int k = (N / 4) * 4; k < N; ++k)
        {
            out[k] = __ldg(base + k);
        }
    }
}

// Store a record: so0, so0t, so1 and (FP64) the primitive cache of so0.
template <int ND, typename R>
__device__ __forceinline__ void store_rec(R * base, R const * so0, R const * so0t, R const * so1,
                                          Prim<ND, R> const & q)
{
    constexpr int NEQ = ND + 2;
    using RC = Rec<ND, R>;
    constexpr int N = RC::NLOAD;
    R v[N];
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        v[i] = so0[i];
        v[NEQ + i] = so0t[i];
    }
#pragma unroll
    for (int i = 0; i < NEQ * ND; ++i)
    {
        v[2 * NEQ + i] = so1[i];
    }
    if constexpr (RC::PRIM)
    {
        q.cache(v + RC::OP);
    }
    else
    {
        (void)q;
    }
    if constexpr (sizeof(R) == 8)
    {
        double2 * p = reinterpret_cast<double2 *>(base);
#pragma unroll
        for (int k = 0; k < N / 2; ++k)
        {
            p[k] = make_double2(v[2 * k], v[2 * k + 1]);
        }
        if constexpr (N % 2)
        {
            base[N - 1] = v[N - 1];
        }
    }
    else
    {
        float4 * p = reinterpret_cast<float4 *>(base);
#pragma unroll
        for (int k = 0; k < N / 4; ++k)
        {
            p[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        }
#pragma unroll
        for (int k = (N / 4) * 4; k < N; ++k)
        {
            base[k] = v[k];
        }
    }
}

// A geometry table value, loaded once per cell-substep and streamed: the
// FP32 3D march (FP64 tables, 816 B per tetrahedron) loads it evict-first,
// which leaves the caches to the neighbour records (measured on 24.6M
// tetrahedra: 7.08 -> 6.84 ms per launch; in 2D, and with L1 no-allocate
// loads, it was slower, so the other marches load it plainly).
template <int ND, typename R, typename G>
__device__ __forceinline__ G geo_ld(G const * p)
{
    if constexpr (ND == 3 && sizeof(R) == 4 && sizeof(G) == 8)
    {
        return __ldcs(p);
    }
    else
    {
        return ldg(p);
    }
}

template <int ND, typename R, typename G>
__device__ __forceinline__ R fg(MarchArgs<R, G> const & a, int f, int k, int64_t icl)
{
    return geo_r<R>(geo_ld<ND, R>(a.fgeo + (static_cast<int64_t>(f) * Geo<ND, G>::KF + k) * a.ncell + icl));
}

// The same rounding (IEEE round-to-nearest-even: the same bits over FP32's
// normal range, where geometry values lie) for the
// few values the FP32 3D march uses last (the gradient-element displacement
// P and the two per-cell scalars): there the conversion instruction, on the
// otherwise idle FP64 pipe, relieves the integer pipe of 14 roundings per
// tetrahedron (6.84 -> 6.70 ms per 24.6M-cell launch; in 2D it was 1% slower,
// so 2D rounds everything with integers).
template <int ND, typename R, typename G>
__device__ __forceinline__ R geo_late(G v)
{
    if constexpr (ND == 3 && sizeof(R) == 4 && sizeof(G) == 8)
    {
        return R(v);
    }
    else
    {
        return geo_r<R>(v);
    }
}

template <int ND, typename R, typename G>
__device__ __forceinline__ R fg_late(MarchArgs<R, G> const & a, int f, int k, int64_t icl)
{
    return geo_late<ND, R>(geo_ld<ND, R>(a.fgeo + (static_cast<int64_t>(f) * Geo<ND, G>::KF + k) * a.ncell + icl));
}

// What calc_soln hands to calc_dsoln of the same cell when the neighbour
// records are not gathered twice (FP32 triangles and tetrahedra; see
// min_blocks for the register budget that makes it pay): the solution change at
// face f's gradient-evaluation point is linear in tau,
//   u_j + hdt ut_j + jdis . g_j - u_i  with  jdis = A_f + tau B_f,
// so calc_soln, holding neighbour j's record, keeps
//   p[f] = u_j + hdt ut_j + A_f . g_j  and  q[f] = B_f . g_j
// per equation.  A_f = dB_f - mean(mid), B_f = mean(dB) - dB_f with FP32
// geometry (R_f and Q_f with FP64 geometry); delta is zero for simplices.
// Whether the fused substep of cell type CT carries calc_soln's neighbour
// terms to calc_dsoln (FP32 simplices) instead of gathering again.
template <typename R, int CT>
__host__ __device__ constexpr bool carries()
{
    return sizeof(R) == 4 && CellT<CT>::SIMPLEX;
}

// Resident blocks of `block` threads to ask of the compiler for a fused
// kernel whose cells carry (0: keep the one-argument launch bound).  The
// carried sums hold 24 (2D) / 40 (3D) more floats; measured at 128 threads,
// 2M triangles: 0.1727 ms per launch without carrying (64 registers), with
// carrying 0.1771 ms at 5 blocks (96 registers), 0.1662 at 6, 0.1555 at 7
// (72 registers, 28 bytes spilled), 0.1557 at 8 (64 registers, 60 bytes
// spilled); 24.6M tetrahedra: 5.92 ms without, 4.75 ms at 5 blocks (96
// registers, 80 bytes spilled), 4.66 ms at 4 (128 registers).  With the
// FP32 delta form (u0, d0 below) 7 blocks stay best in 2D (0.1628 ms; 6:
// 0.1688, 8: 0.1683) and 4 in 3D (4.80 ms).  The budget per thread (72 /
// 128 registers) is kept for other block sizes.  With FP64 geometry tables
// (G = double) the budget is set apart, as the geometry loads and their
// rounding hold more registers: 2D, 980k triangles, 0.2350 / 0.2364 /
// 0.2296 / 0.2175 ms per 2M-cell launch at 64 / 72 / 80 / 96 registers.
#ifndef SCG_CARRY_REGS_2D
#define SCG_CARRY_REGS_2D 72
#endif
#ifndef SCG_CARRY_REGS_2D_G64
#define SCG_CARRY_REGS_2D_G64 96
#endif
#ifndef SCG_CARRY_REGS_3D
#define SCG_CARRY_REGS_3D 128
#endif
#ifndef SCG_CARRY_REGS_3D_G64
#define SCG_CARRY_REGS_3D_G64 128
#endif
template <int ND, typename R, int CT, int BLOCK, typename G = R>
__host__ __device__ constexpr int min_blocks()
{
    if constexpr (!carries<R, CT>())
    {
        return 0;
    }
    else
    {
        constexpr int regs = ND == 3 ? (sizeof(G) == 8 ? SCG_CARRY_REGS_3D_G64 : SCG_CARRY_REGS_3D)
                                     : (sizeof(G) == 8 ? SCG_CARRY_REGS_2D_G64 : SCG_CARRY_REGS_2D);
        return 65536 / (BLOCK * regs);
    }
}

template <int ND, int NFC, typename R>
struct Carry
{
    R mm[ND];
    R mb[ND];
    R p[NFC][ND + 2];
    R q[NFC][ND + 2];
};

// The same sums kept in shared memory instead of registers: one slot per
// thread and component, component-major (SB threads apart), so a warp's
// accesses fall in distinct banks; each thread reads only its own slots, so
// no barrier is needed.  Used for tetrahedra (40 floats per cell), where it
// frees registers at the same budget: 24.6M tetrahedra 6.70 -> 6.44 ms per
// launch at 128 registers (at 96 registers it spills and loses); for
// triangles (24 floats) it was slower at every budget (2D, 2M cells: 0.2356
// ms in registers, 0.2451 / 0.2505 / 0.2734 ms at 96 / 80 / 72 registers).
// The single-mesh and batched kernels carry the same way, so a batched core
// gives the same bits as its own march.
template <int ND>
__host__ __device__ constexpr bool carry_shared()
{
    return ND == 3;
}
template <int ND, int NFC, typename R, int SB>
struct CarrySh
{
    struct Row
    {
        R * b;
        __device__ __forceinline__ R & operator[](int i) const { return b[i * SB]; }
    };
    struct Tab
    {
        R * b;
        __device__ __forceinline__ Row operator[](int f) const { return Row{b + f * (ND + 2) * SB}; }
    };
    R mm[ND];
    R mb[ND];
    Tab p;
    Tab q;
};

// Face means of mid and dB (FP32 geometry; zero with FP64 geometry).
template <int CT, typename R, typename G>
__device__ __forceinline__ void face_means(MarchArgs<R, G> const & a, int64_t icl, R * mm, R * mb)
{
    constexpr int ND = CellT<CT>::ND;
    constexpr int NFC = CellT<CT>::NFC;
    using D = Geo<ND, G>;
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        mm[d] = R(0);
        mb[d] = R(0);
    }
    if constexpr (D::MID)
    {
#pragma unroll
        for (int f = 0; f < NFC; ++f)
        {
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                mm[d] += fg<ND>(a, f, D::K_MID + d, icl);
                mb[d] += fg<ND>(a, f, D::K_DB + d, icl);
            }
        }
        R const inv = R(1) / R(NFC);
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            mm[d] *= inv;
            mb[d] *= inv;
        }
    }
}

// ---------------------------------------------------------------------------
// calc_soln for one body cell (euler_march.cpp:197-303): the CESE flux
// integral over the cell's BCEs, divided by the CCE volume.
//
// With CACHE set (the fused march, where every record's primitive cache is
// valid) a neighbour's primitives come from its record.  With u0 (the cell's
// own current state; the FP32 march) the neighbour values enter as
// differences from u0 and d0 receives so0n - u0: in FP32 the absolute
// rounding then scales with the change, not with the state (the gradients
// calc_dsoln forms from these differences are O(h) of the state).
template <int CT, typename R, typename G, bool CACHE = false,
          typename CA = Carry<CellT<CT>::ND, CellT<CT>::NFC, R>>
__device__ __forceinline__ void soln_cell(MarchArgs<R, G> const & a, int64_t icl, R * so0n, CA * carry = nullptr,
                                          R const * u0 = nullptr, R * d0 = nullptr)
{
    constexpr int ND = CellT<CT>::ND;
    constexpr int NEQ = ND + 2;
    constexpr int NFC = CellT<CT>::NFC;
    using D = Geo<ND, G>;
    using RC = Rec<ND, R>;
    constexpr bool USE = CACHE && RC::PRIM;
    Acc<R> acc[NEQ];
#pragma unroll
    for (int f = 0; f < NFC; ++f)
    {
        int64_t const jr = ldg(a.nbr + f * a.ncell + icl);
        R rec[USE ? RC::NLOAD : RC::NUSED];
        load_rec<ND, R, USE ? RC::NLOAD : RC::NUSED>(a.cur + jr * RC::RS, rec);
        R const * u = rec;
        R const * t = rec + NEQ;
        R const * g = rec + 2 * NEQ;
        R const ga = ldg(a.gamma + jr);

        R const bvol = fg<ND>(a, f, D::K_BVOL, icl);
        R dB[ND], nh[ND], qn[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            dB[d] = fg<ND>(a, f, D::K_DB + d, icl);
            nh[d] = fg<ND>(a, f, D::K_NH + d, icl);
            qn[d] = a.qdt * nh[d];
        }
        if (carry)
        {
            R A[ND], B[ND];
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                if constexpr (D::MID)
                {
                    A[d] = dB[d] - carry->mm[d];
                    B[d] = carry->mb[d] - dB[d];
                }
                else
                {
                    A[d] = fg<ND>(a, f, D::K_R + d, icl);
                    B[d] = fg<ND>(a, f, D::K_Q + d, icl);
                }
            }
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                R pp = (u0 ? u[i] - u0[i] : u[i]) + a.hdt * t[i];
                R qq = R(0);
#pragma unroll
                for (int d = 0; d < ND; ++d)
                {
                    pp += A[d] * g[i * ND + d];
                    qq += B[d] * g[i * ND + d];
                }
                carry->p[f][i] = pp;
                carry->q[f][i] = qq;
            }
        }
        // Spatial flux: neighbour solution at the BCE centroid times its volume.
#pragma unroll
        for (int i = 0; i < NEQ; ++i)
        {
            R s = u0 ? u[i] - u0[i] : u[i];
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                s += dB[d] * g[i * ND + d];
            }
            acc[i].add(s * bvol);
        }
        // Temporal flux: sum over sub-faces folded into Nh and Mh.
        R w[NEQ * ND];
#pragma unroll
        for (int i = 0; i < NEQ; ++i)
        {
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                R s = t[i] * qn[d];
#pragma unroll
                for (int e = 0; e < ND; ++e)
                {
                    s += g[i * ND + e] * fg<ND>(a, f, D::K_MH + e * ND + d, icl);
                }
                w[i * ND + d] = s;
            }
        }
        Prim<ND, R> q;
        if constexpr (USE)
        {
            q = Prim<ND, R>::cached(rec + RC::OP, ga);
        }
        else
        {
            q = Prim<ND, R>(u, ga);
        }
        R fl[NEQ];
        flux_dot<ND, R>(q, u, nh, fl);
        jvp_sum<ND, R>(q, u, w, fl);
#pragma unroll
        for (int i = 0; i < NEQ; ++i)
        {
            acc[i].add(-fl[i]);
        }
    }
    R const ivol = geo_late<ND, R>(geo_ld<ND, R>(a.cgeo + 0 * a.ncell + icl));
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        if (u0)
        {
            // Delta form: the CCE volume is the sum of the BCE volumes, so
            // sum_f bvol_f u0 / cevol = u0 and only the change is summed.
            d0[i] = acc[i].value() * ivol;
            so0n[i] = u0[i] + d0[i];
        }
        else
        {
            so0n[i] = acc[i].value() * ivol;
        }
    }
}

// calc_cfl for one body cell (euler_solution.cpp:106-160): original and
// clamped CFL, and the energy rewritten from the non-negative pressure.  The
// reference's three divisions by rho use one reciprocal 1/(rho + TINY) (the
// floor changes nothing unless rho is below 1e-44 in FP64, 1e-23 in FP32,
// where the reference itself produces inf); it is returned in rinv for the
// primitives of the same state.
template <int ND, typename R, typename G>
__device__ __forceinline__ R cfl_cell(MarchArgs<R, G> const & a, int64_t icl, int64_t row, R * so0n, R & rinv)
{
    constexpr int NEQ = ND + 2;
    R const ga = ldg(a.gamma + row);
    R const ga1 = ga - R(1);
    R const ri = mrecip<ND>(so0n[0] + Tiny<R>::JAC);
    rinv = ri;
    R momsq = R(0);
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        momsq += so0n[1 + d] * so0n[1 + d];
    }
    R const ke = R(0.5) * momsq * ri;
    R const pr = ga1 * (so0n[NEQ - 1] - ke);
    R const pra = (pr + fabs(pr)) / R(2);
    R const wspd = sqr_t(ga * pra * ri) + sqr_t(momsq) * ri;
    R const cflo = wspd * geo_late<ND, R>(geo_ld<ND, R>(a.cgeo + 1 * a.ncell + icl));
    // pra / (pra + TINY) is exactly 1 whenever TINY does not change pra (any
    // pressure above ~1e-44 in FP64), so the division is taken only below.
    R const prt = pra + Tiny<R>::CFL;
    R const cflc = (cflo - R(1)) * (prt == pra ? R(1) : pra / prt) + R(1);
    a.cflo[row] = cflo;
    a.cflc[row] = cflc;
    // The reference stores pra/ga1 + ke + TINY.  For pr > 0 that is exactly
    // E + TINY (= E to working precision); re-forming it would only add a
    // rounding error to the energy every substep, which matters in FP32.
    if (!(pr > R(0)))
    {
        so0n[NEQ - 1] = pra / ga1 + ke + Tiny<R>::CFL;
    }
    return cflc;
}

// calc_dsoln for one body cell (euler_gradient.cpp:23-130 with the gradient
// element of GradientElement.cpp:137-290): per fundamental gradient element
// solve, W-1/2 weights, W-3/4 cap, weighted sum.  The neighbour records are
// gathered a second time (calc_soln just read them, so the loads hit in
// cache); carrying calc_soln's neighbour terms over instead costs more FP64
// operations, but pays in FP32 for simplices (carry != nullptr, see Carry).
template <int CT, typename R, typename G, typename CA = Carry<CellT<CT>::ND, CellT<CT>::NFC, R>>
__device__ __forceinline__ void dsoln_cell(MarchArgs<R, G> const & a, int64_t icl, R const * so0n, R cflc,
                                           R * so1n, CA const * carry = nullptr,
                                           R const * u0 = nullptr, R const * d0 = nullptr)
{
    constexpr int ND = CellT<CT>::ND;
    constexpr int NEQ = ND + 2;
    constexpr int NFC = CellT<CT>::NFC;
    constexpr int NFGE = CellT<CT>::NFGE;
    using D = Geo<ND, G>;

    R const acfl = fabs(cflc);
    R const sgm0 = sizeof(R) == 8 ? R(0) : mquot<ND>(a.sigma0, acfl); // FP32 cap only
    R const tau = a.taumin + acfl * a.tauscale;
    R const ofg1 = R(1) / R(NFGE);

    // Gradient-evaluation displacements: idis = dst - delta, dst = P + tau Q.
    // With FP32 geometry P = mid - mean(mid) and Q = mean(dB) - dB are formed
    // here from the face means (the faces' values are read again rather than
    // held: they hit in L1, and registers bound this kernel's occupancy).
    R mm[ND], mb[ND];
    if (carry)
    {
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            mm[d] = carry->mm[d];
            mb[d] = carry->mb[d];
        }
    }
    else
    {
        face_means<CT, R, G>(a, icl, mm, mb);
    }
    R idis[NFC][ND];
#pragma unroll
    for (int f = 0; f < NFC; ++f)
    {
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            if constexpr (D::MID)
            {
                idis[f][d] = (fg<ND>(a, f, D::K_MID + d, icl) - mm[d]) +
                             tau * (mb[d] - fg<ND>(a, f, D::K_DB + d, icl));
            }
            else
            {
                idis[f][d] = fg_late<ND>(a, f, D::K_P + d, icl) + tau * fg<ND>(a, f, D::K_Q + d, icl);
            }
        }
    }
    R delta[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        delta[d] = R(0);
    }
    if constexpr (!CellT<CT>::SIMPLEX)
    {
        // Sub-element centroid of the gradient element about the vertex mean
        // (calc_gge_centroid, GradientElement.cpp:81-133).
        R voc = R(0);
#pragma unroll
        for (int k = 0; k < NFGE; ++k)
        {
            int const f0 = CellT<CT>::fge(k, 0);
            int const f1 = CellT<CT>::fge(k, 1);
            int const f2 = (ND == 3) ? CellT<CT>::fge(k, ND - 1) : f1;
            R const vob = det_rows<ND, R>(idis[f0], idis[f1], idis[f2]);
            voc += vob;
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                R s = idis[f0][d] + idis[f1][d];
                if constexpr (ND == 3)
                {
                    s += idis[f2][d];
                }
                delta[d] += s * vob;
            }
        }
        R const inv = mrecip<ND>(voc * R(ND + 1));
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            delta[d] *= inv;
        }
#pragma unroll
        for (int f = 0; f < NFC; ++f)
        {
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                idis[f][d] -= delta[d];
            }
        }
    }

    // Solution deltas at the evaluation points: uf[f][i].
    R uf[NFC][NEQ];
    if (carry)
    {
#pragma unroll
        for (int f = 0; f < NFC; ++f)
        {
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                // carry->p already has the cell's own change (d0) or new state
                // taken out (see fused_cell).
                uf[f][i] = carry->p[f][i] + tau * carry->q[f][i];
            }
        }
    }
    else
    {
#pragma unroll
        for (int f = 0; f < NFC; ++f)
        {
            int64_t const jr = ldg(a.nbr + f * a.ncell + icl);
            R rec[Rec<ND, R>::NUSED];
            load_rec<ND, R>(a.cur + jr * Rec<ND, R>::RS, rec);
            R jd[ND];
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                if constexpr (D::MID)
                {
                    R const db = fg<ND>(a, f, D::K_DB + d, icl);
                    jd[d] = (db - mm[d]) + tau * (mb[d] - db) - delta[d];
                }
                else
                {
                    jd[d] = fg<ND>(a, f, D::K_R + d, icl) + tau * fg<ND>(a, f, D::K_Q + d, icl) - delta[d];
                }
            }
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                R s = u0 ? (rec[i] - u0[i]) + a.hdt * rec[NEQ + i] - d0[i] : rec[i] + a.hdt * rec[NEQ + i] - so0n[i];
#pragma unroll
                for (int d = 0; d < ND; ++d)
                {
                    s += jd[d] * rec[2 * NEQ + i * ND + d];
                }
                uf[f][i] = s;
            }
        }
    }

    // Rows of each element's inverse displacement matrix (prescaled by
    // 1/det): grad = sum_v uf[v] * C[k][v].  In FP64 the NFGE reciprocals
    // come from one division by the product of the determinants (prefix
    // products, then peeled off backwards); in FP32 that product could
    // underflow, so each element divides.
    R dets[NFGE];
    R bcx[NFGE][ND == 3 ? 3 : 1]; // 3D: rb x rc, the first row of the adjugate
#pragma unroll
    for (int k = 0; k < NFGE; ++k)
    {
        R const * ra = idis[CellT<CT>::fge(k, 0)];
        R const * rb = idis[CellT<CT>::fge(k, 1)];
        if constexpr (ND == 2)
        {
            dets[k] = ra[0] * rb[1] - ra[1] * rb[0];
        }
        else
        {
            R const * rc = idis[CellT<CT>::fge(k, ND - 1)];
            bcx[k][0] = rb[1] * rc[2] - rb[2] * rc[1];
            bcx[k][1] = rb[2] * rc[0] - rb[0] * rc[2];
            bcx[k][2] = rb[0] * rc[1] - rb[1] * rc[0];
            dets[k] = ra[0] * bcx[k][0] + ra[1] * bcx[k][1] + ra[2] * bcx[k][2];
        }
    }
    R invs[NFGE];
    if constexpr (sizeof(R) == 8)
    {
        R pre[NFGE];
        pre[0] = dets[0];
#pragma unroll
        for (int k = 1; k < NFGE; ++k)
        {
            pre[k] = pre[k - 1] * dets[k];
        }
        R inv = recip(pre[NFGE - 1]);
#pragma unroll
        for (int k = NFGE - 1; k > 0; --k)
        {
            invs[k] = inv * pre[k - 1];
            inv *= dets[k];
        }
        invs[0] = inv;
    }
    else
    {
#pragma unroll
        for (int k = 0; k < NFGE; ++k)
        {
            invs[k] = mrecip<ND>(dets[k]);
        }
    }
    R C[NFGE][ND][ND];
#pragma unroll
    for (int k = 0; k < NFGE; ++k)
    {
        R const * ra = idis[CellT<CT>::fge(k, 0)];
        R const * rb = idis[CellT<CT>::fge(k, 1)];
        R const inv = invs[k];
        if constexpr (ND == 2)
        {
            C[k][0][0] = rb[1] * inv;
            C[k][0][1] = -rb[0] * inv;
            C[k][1][0] = -ra[1] * inv;
            C[k][1][1] = ra[0] * inv;
        }
        else
        {
            R const * rc = idis[CellT<CT>::fge(k, ND - 1)];
            C[k][0][0] = bcx[k][0] * inv;
            C[k][0][1] = bcx[k][1] * inv;
            C[k][0][2] = bcx[k][2] * inv;
            C[k][1][0] = (rc[1] * ra[2] - rc[2] * ra[1]) * inv;
            C[k][1][1] = (rc[2] * ra[0] - rc[0] * ra[2]) * inv;
            C[k][1][2] = (rc[0] * ra[1] - rc[1] * ra[0]) * inv;
            C[k][2][0] = (ra[1] * rb[2] - ra[2] * rb[1]) * inv;
            C[k][2][1] = (ra[2] * rb[0] - ra[0] * rb[2]) * inv;
            C[k][2][2] = (ra[0] * rb[1] - ra[1] * rb[0]) * inv;
        }
    }

    uint8_t fired = 0;
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        R grad[NFGE][ND];
        R wgt[NFGE];
        R wacc = R(0);
#pragma unroll
        for (int k = 0; k < NFGE; ++k)
        {
            R sq = R(0);
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                R s = R(0);
#pragma unroll
                for (int v = 0; v < ND; ++v)
                {
                    s += uf[CellT<CT>::fge(k, v)][i] * C[k][v][d];
                }
                grad[k][d] = s;
                sq += s * s;
            }
            // W-1/2 weighting: inverse gradient magnitude.
            wgt[k] = rsq(sq + Tiny<R>::AZ);
            wacc += wgt[k];
        }
        if constexpr (sizeof(R) == 8)
        {
            // FP64: one division per equation.  With u = w - wacc/n (the
            // deviations scaled by wacc > 0) the reference's weight
            // 1/n + sm (w/wacc - 1/n) is 1/n + (sm/wacc) u, and each of its
            // three caps divided by wacc is a quotient of known sign:
            //   T1 = (1 - 1/n) / (umax + TINY wacc),  T2 = (1/n) / (TINY wacc - umin),
            //   T0 = sigma0 / (|cfl| wacc).
            // The smaller of T1, T2 is chosen by cross-multiplying as in
            // FP32 below; it fires (the W-3/4 cap binds) when it is below
            // T0, again by cross-multiplying, and only the chosen quotient
            // is divided out.
            R const wq = ofg1 * wacc;
            R umax = R(0);
            R umin = R(0);
#pragma unroll
            for (int k = 0; k < NFGE; ++k)
            {
                wgt[k] -= wq;
                umax = fmax(umax, wgt[k]);
                umin = fmin(umin, wgt[k]);
            }
            R const za = Tiny<R>::AZ * wacc;
            R const d1 = umax + za;
            R const d2 = za - umin;
            bool const first = (R(1) - ofg1) * d2 <= ofg1 * d1;
            R const nn = first ? R(1) - ofg1 : ofg1;
            R const dd = first ? d1 : d2;
            R const cw = acfl * wacc;
            bool const fire = nn * cw < a.sigma0 * dd;
            R const c = (fire ? nn : a.sigma0) * recip(fire ? dd : cw);
            if (fire)
            {
                fired |= static_cast<uint8_t>(1u << i);
            }
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                R s = R(0);
#pragma unroll
                for (int k = 0; k < NFGE; ++k)
                {
                    s += (ofg1 + c * wgt[k]) * grad[k][d];
                }
                so1n[i * ND + d] = s;
            }
        }
        else
        {
            R const rw = mrecip<ND>(wacc);
            R wmax = R(0);
            R wmin = R(0);
#pragma unroll
            for (int k = 0; k < NFGE; ++k)
            {
                wgt[k] = wgt[k] * rw - ofg1;
                wmax = fmax(wmax, wgt[k]);
                wmin = fmin(wmin, wgt[k]);
            }
            // W-3/4 cap: sm = min(A / a1, B / a2) with A = 1 - 1/n > 0,
            // a1 = wmax + TINY > 0, B = -1/n < 0, a2 = wmin - TINY < 0.  Both
            // quotients are positive, and A / a1 <= B / a2 exactly when
            // A a2 >= B a1, so the smaller one is chosen first and one
            // division is taken instead of two.
            R const a1 = wmax + Tiny<R>::AZ;
            R const a2 = wmin - Tiny<R>::AZ;
            bool const first = (R(1) - ofg1) * a2 >= -ofg1 * a1;
            R const sm = mquot<ND>(first ? R(1) - ofg1 : -ofg1, first ? a1 : a2);
            R const sig = fmin(sm, sgm0);
            if (sm < sgm0)
            {
                fired |= static_cast<uint8_t>(1u << i);
            }
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                R s = R(0);
#pragma unroll
                for (int k = 0; k < NFGE; ++k)
                {
                    s += (ofg1 + sig * wgt[k]) * grad[k][d];
                }
                so1n[i * ND + d] = s;
            }
        }
    }
    if (a.limiter)
    {
        a.limiter[icl] = fired;
    }
}

// Ghost-row order-0 update of one boundary face (euler_bc.cpp:147-215):
// ghost so0n from the interior's so0n (taken before calc_cfl's rewrite).
template <int ND, typename R>
__device__ __forceinline__ void bc0_ghost(int kind, double const * n, double const * val, R const * in, R * out)
{
    constexpr int NEQ = ND + 2;
    if (kind == 2)
    {
#pragma unroll
        for (int i = 0; i < NEQ; ++i)
        {
            out[i] = R(val[i]);
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < NEQ; ++i)
    {
        out[i] = in[i];
    }
    if (kind == 1)
    {
        // Reflect the momentum: m - 2 (m . n) n.
        R mn = R(0);
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            mn += in[1 + d] * R(n[d]);
        }
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            out[1 + d] = in[1 + d] - R(2) * mn * R(n[d]);
        }
    }
}

// Ghost-row order-1 update of one boundary face (euler_bc.cpp:221-320):
// ghost so1n from the interior's so1c.
template <int ND, typename R>
__device__ __forceinline__ void bc1_ghost(int kind, double const * n, R const * g, R * out)
{
    constexpr int NEQ = ND + 2;
    if (kind == 2)
    {
#pragma unroll
        for (int i = 0; i < NEQ * ND; ++i)
        {
            out[i] = R(0);
        }
        return;
    }
    R nn[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        nn[d] = R(n[d]);
    }
    if (kind == 0)
    {
        // Tangential projection of every gradient: g - (g . n) n.
#pragma unroll
        for (int i = 0; i < NEQ; ++i)
        {
            R gn = R(0);
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                gn += g[i * ND + d] * nn[d];
            }
#pragma unroll
            for (int d = 0; d < ND; ++d)
            {
                out[i * ND + d] = g[i * ND + d] - gn * nn[d];
            }
        }
        return;
    }
    // Slip wall: scalar gradients reflected (I - 2 n n^T) g; momentum
    // gradient tensor reflected on both indices, R G R.
#pragma unroll
    for (int ii = 0; ii < 2; ++ii)
    {
        int const i = ii == 0 ? 0 : NEQ - 1;
        R gn = R(0);
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            gn += g[i * ND + d] * nn[d];
        }
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            out[i * ND + d] = g[i * ND + d] - R(2) * gn * nn[d];
        }
    }
    // RG = G - 2 (G n) n^T then R(RG) = RG - 2 n (n^T RG).
    R gm[ND][ND];
#pragma unroll
    for (int p = 0; p < ND; ++p)
    {
        R gnp = R(0);
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            gnp += g[(1 + p) * ND + d] * nn[d];
        }
#pragma unroll
        for (int d = 0; d < ND; ++d)
        {
            gm[p][d] = g[(1 + p) * ND + d] - R(2) * gnp * nn[d];
        }
    }
#pragma unroll
    for (int d = 0; d < ND; ++d)
    {
        R ntg = R(0);
#pragma unroll
        for (int p = 0; p < ND; ++p)
        {
            ntg += nn[p] * gm[p][d];
        }
#pragma unroll
        for (int p = 0; p < ND; ++p)
        {
            out[(1 + p) * ND + d] = gm[p][d] - R(2) * nn[p] * ntg;
        }
    }
}

// A row's new so0n and so1n, as FP64, into the host blocks of a march that
// delivers them (out0, out1), in the layout of the host arrays: the bytes
// leave over the host link while the march still computes.
template <int ND, typename R, typename G>
__device__ __forceinline__ void deliver_row(MarchArgs<R, G> const & a, int64_t row, R const * so0, R const * so1)
{
    constexpr int NEQ = ND + 2;
    if (a.out0)
    {
        double * const o = a.out0 + row * NEQ;
        if constexpr (NEQ % 2 == 0)
        {
#pragma unroll
            for (int i = 0; i < NEQ; i += 2)
            {
                *reinterpret_cast<double2 *>(o + i) = make_double2(double(so0[i]), double(so0[i + 1]));
            }
        }
        else
        {
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                o[i] = double(so0[i]);
            }
        }
    }
    if (a.out1)
    {
        double * const o = a.out1 + row * (NEQ * ND);
        if constexpr ((NEQ * ND) % 2 == 0)
        {
#pragma unroll
            for (int i = 0; i < NEQ * ND; i += 2)
            {
                *reinterpret_cast<double2 *>(o + i) = make_double2(double(so1[i]), double(so1[i + 1]));
            }
        }
        else
        {
#pragma unroll
            for (int i = 0; i < NEQ * ND; ++i)
            {
                o[i] = double(so1[i]);
            }
        }
    }
}

// One fused CESE substep for one body cell: soln, bc_soln of its boundary
// faces, cfl, dsoln, bc_dsoln of its boundary faces, and calc_solt of the next
// substep for its own row and its ghost rows.  Reads only the current records
// (neighbours' old values) and writes only rows it owns, so one launch covers
// the whole substep with no grid-wide synchronisation.
template <int CT, typename R, typename G, int SB = 0>
__device__ __forceinline__ void fused_cell(MarchArgs<R, G> const & a, int64_t icl)
{
    constexpr int ND = CellT<CT>::ND;
    constexpr int NEQ = ND + 2;
    constexpr int NFC = CellT<CT>::NFC;
    int64_t const row = icl + a.ngst;

    // FP32 simplices hand calc_soln's neighbour terms to calc_dsoln instead
    // of gathering the neighbour records again (see Carry).
    // The choice depends on the cell type and precision only, never on the
    // kernel, so a core's cells give the same bits in every kernel that
    // marches them (single-type or mixed, alone or batched).
    constexpr bool CARRY = carries<R, CT>();
    // SB > 0: the carried sums in shared memory, SB threads per block.
    using CA = std::conditional_t<(SB > 0 && CARRY), CarrySh<ND, NFC, R, SB>, Carry<ND, NFC, R>>;
    CA carry;
    if constexpr (SB > 0 && CARRY)
    {
        __shared__ R s_carry[2 * NFC * NEQ * SB];
        carry.p.b = s_carry + threadIdx.x;
        carry.q.b = s_carry + NFC * NEQ * SB + threadIdx.x;
    }
    if constexpr (CARRY)
    {
        face_means<CT, R, G>(a, icl, carry.mm, carry.mb);
    }
    // FP32: work relative to the cell's own current state (delta form).
    constexpr bool DELTA = sizeof(R) == 4;
    R u0[NEQ], d0[NEQ];
    if constexpr (DELTA)
    {
        load_rec<ND, R, NEQ>(a.cur + row * Rec<ND, R>::RS, u0);
    }
    R so0n[NEQ];
    soln_cell<CT, R, G, true>(a, icl, so0n, CARRY ? &carry : nullptr, DELTA ? u0 : nullptr, d0);
    // FP32 error feedback: what rounding the new so0 to FP32 drops is kept per
    // cell and equation (comp) and added back to the cell's next new value,
    // the rounding taken by an exact two-sum (Knuth) so the kept residual is
    // exactly the part lost.  A CESE cell's new value is formed from its
    // neighbours' stored values, so without this every substep's FP32
    // roundings of the whole state are lost to the totals for good, and they
    // do not average out (measured: the totals of a 3D blast drift ~1e-8 from
    // FP64's in 200 steps, also with FP64 arithmetic on FP32-rounded states);
    // with the residual fed back they cancel over the mesh, and the totals stay
    // within ~1e-10 of FP64's.  Locally the residual re-added is below half an
    // ulp of the state, the size of the rounding itself.  Neighbours read only
    // the rounded so0; the API's so0n and the totals are so0 + comp; d0 becomes
    // the change including the residual.
    R cnew[NEQ];
    if constexpr (DELTA)
    {
        if (a.comp)
        {
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                R const y = d0[i] + a.comp[i * a.ncell + icl];
                R const t = u0[i] + y;
                R const yb = t - u0[i];
                cnew[i] = (u0[i] - (t - yb)) + (y - yb);
                so0n[i] = t;
                d0[i] = y;
            }
        }
    }

    // Boundary faces: ghost so0n (pre-rewrite), so1n and next so0t.
#pragma unroll
    for (int f = 0; f < NFC; ++f)
    {
        int64_t const jr = ldg(a.nbr + f * a.ncell + icl);
        if (jr < a.ngst)
        {
            int const kind = a.gkind[jr];
            if (kind >= 0)
            {
                R own[Rec<ND, R>::NUSED];
                load_rec<ND, R>(a.cur + row * Rec<ND, R>::RS, own);
                R g0[NEQ], g1[NEQ * ND], gt[NEQ];
                bc0_ghost<ND, R>(kind, a.gnml + jr * ND, a.gval + jr * NEQ, so0n, g0);
                bc1_ghost<ND, R>(kind, a.gnml + jr * ND, own + 2 * NEQ, g1);
                Prim<ND, R> const qg(g0, ldg(a.gamma + jr));
                solt_prim<ND, R>(qg, g0, g1, gt);
                store_rec<ND, R>(a.nxt + jr * Rec<ND, R>::RS, g0, gt, g1, qg);
                deliver_row<ND>(a, jr, g0, g1);
            }
        }
    }

    R rinv;
    R const e_soln = so0n[NEQ - 1];
    R const cflc = cfl_cell<ND, R, G>(a, icl, row, so0n, rinv);
    if (DELTA && so0n[NEQ - 1] != e_soln)
    {
        d0[NEQ - 1] = so0n[NEQ - 1] - u0[NEQ - 1]; // calc_cfl rewrote the energy
        cnew[NEQ - 1] = R(0);                      // ... and nothing was dropped
    }
    if constexpr (DELTA)
    {
        if (a.comp)
        {
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                a.comp[i * a.ncell + icl] = cnew[i];
            }
        }
    }
    if constexpr (CARRY)
    {
        // Take the cell's own change (FP32, delta form) or new state out of
        // the carried sums now, so it need not stay live through calc_dsoln.
#pragma unroll
        for (int f = 0; f < NFC; ++f)
        {
#pragma unroll
            for (int i = 0; i < NEQ; ++i)
            {
                carry.p[f][i] -= DELTA ? d0[i] : so0n[i];
            }
        }
    }
    R so1n[NEQ * ND];
    dsoln_cell<CT, R, G>(a, icl, so0n, cflc, so1n, CARRY ? &carry : nullptr, DELTA ? u0 : nullptr, d0);
    R so0t[NEQ];
    Prim<ND, R> const q(so0n, ldg(a.gamma + row), rinv);
    solt_prim<ND, R>(q, so0n, so1n, so0t);
    store_rec<ND, R>(a.nxt + row * Rec<ND, R>::RS, so0n, so0t, so1n, q);
    deliver_row<ND>(a, row, so0n, so1n);
}

// The work of thread t of one substep: body cell t for t < ncell, ghost row
// t - ncell after that.  CT1 = 0 dispatches on each cell's type; a nonzero
// CT1 compiles the one cell type of a single-type mesh, whose kernel then
// needs only that type's registers.
template <int ND, typename R, typename G, int CT1 = 0, int SB = 0>
__device__ __forceinline__ void fused_thread(MarchArgs<R, G> const & a, int64_t t)
{
    if (t < a.ncell)
    {
        int const ct = a.ctype[t];
        if constexpr (CT1 != 0)
        {
            (void)ct;
            fused_cell<CT1, R, G, SB>(a, t);
        }
        else if constexpr (ND == 2)
        {
            if (ct == 4)
                fused_cell<4, R, G>(a, t);
            else
                fused_cell<3, R, G>(a, t);
        }
        else
        {
            switch (ct)
            {
            case 6: fused_cell<6, R, G>(a, t); break;
            case 5: fused_cell<5, R, G>(a, t); break;
            case 7: fused_cell<7, R, G>(a, t); break;
            default: fused_cell<8, R, G>(a, t); break;
            }
        }
    }
    else if (t < a.ncell + a.ngst)
    {
        // A ghost row without a boundary condition keeps its stale state; its
        // next so0t is still the Jacobian product of that state.
        int64_t const g = t - a.ncell;
        if (a.gkind[g] < 0)
        {
            constexpr int NEQ = ND + 2;
            R rec[Rec<ND, R>::NUSED];
            load_rec<ND, R>(a.nxt + g * Rec<ND, R>::RS, rec);
            R tt[NEQ];
            Prim<ND, R> const q(rec, ldg(a.gamma + g));
            solt_prim<ND, R>(q, rec, rec + 2 * NEQ, tt);
            store_rec<ND, R>(a.nxt + g * Rec<ND, R>::RS, rec, tt, rec + 2 * NEQ, q);
            deliver_row<ND>(a, g, rec, rec + 2 * NEQ);
        }
    }
}

// One substep over the rows [t0, t1) of the work order (body cells 0 ..
// ncell - 1, then the ghost rows): the whole substep is [0, ncell + ngst);
// a march that overlaps its state's upload with its first substep launches
// it in ranges.
template <int ND, typename R, typename G, int CT1 = 0>
__global__ void __launch_bounds__(128) k_fused(MarchArgs<R, G> a, int64_t t0, int64_t t1)
{
    int64_t const t = t0 + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t < t1)
    {
        fused_thread<ND, R, G, CT1, carry_shared<ND>() ? 128 : 0>(a, t);
    }
}

// The same kernel asking the compiler for MINB resident blocks of 128
// (min_blocks).  A stated minimum of 1 would instead free the compiler to use
// up to 255 registers, so the kernels that do not carry keep the one-argument
// bound.
template <int ND, typename R, typename G, int CT1, int MINB>
__global__ void __launch_bounds__(128, MINB) k_fused_mb(MarchArgs<R, G> a, int64_t t0, int64_t t1)
{
    int64_t const t = t0 + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t < t1)
    {
        fused_thread<ND, R, G, CT1, carry_shared<ND>() ? 128 : 0>(a, t);
    }
}

} // namespace dev
} // namespace scg
