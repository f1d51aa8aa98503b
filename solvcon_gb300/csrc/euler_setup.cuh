#pragma once

/*
 * Set-up kernels of the multi-dimensional Euler core: the CE geometry of
 * prepare_ce (cpp/solvcon/multidim/euler_ce.cpp:78-347), computed once per
 * mesh on the device, and its compaction into the march's per-face geometric
 * moments (see euler_device.cuh).
 */

#include "euler_device.cuh"

namespace scg
{
namespace dev
{

// Device view of the mesh tables, ghost rows first (row = index + nghost).
struct MeshView
{
    int ndim;
    int64_t ncell, ngstcell, ngstface, ngstnode;
    double const * ndcrd;  // [nrown][ndim]
    double const * fccnd;  // [nrowf][ndim]
    double const * clcnd;  // [nrowc][ndim]
    int32_t const * fcnds; // [nrowf][5]
    int32_t const * fccls; // [nrowf][4]
    int32_t const * clfcs; // [nrowc][7]
    int32_t const * cltpn; // [nrowc]

    __device__ double nd(int64_t i, int d) const { return ndcrd[(i + ngstnode) * ndim + d]; }
    __device__ double fc(int64_t i, int d) const { return fccnd[(i + ngstface) * ndim + d]; }
    __device__ double cc(int64_t i, int d) const { return clcnd[(i + ngstcell) * ndim + d]; }
    __device__ int32_t fnds(int64_t i, int k) const { return fcnds[(i + ngstface) * 5 + k]; }
    __device__ int32_t fcls(int64_t i, int k) const { return fccls[(i + ngstface) * 4 + k]; }
    __device__ int32_t cfcs(int64_t i, int k) const { return clfcs[(i + ngstcell) * 7 + k]; }
    __device__ int32_t rcl(int32_t ifc, int32_t icl) const { return fcls(ifc, 0) + fcls(ifc, 1) - icl; }
};

// Range check of what the set-up and march kernels index through: for body
// cell icl, its face count and faces, each face's two cells (one of them icl)
// and its node count and nodes.  Reads only inside the tables; the first bad
// cell lands in *bad (atomicMin).
// Count the values of an FP64 geometry table that the FP32 march's rounding
// (geo_r) does not take.
__global__ void k_geo_range(double const * g, int64_t n, unsigned long long * bad)
{
    unsigned long long cnt = 0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    {
        cnt += geo_r_takes(g[i]) ? 0ull : 1ull;
    }
    if (cnt)
    {
        atomicAdd(bad, cnt);
    }
}

__global__ void k_validate_mesh(MeshView m, int64_t nface, int64_t nnode, unsigned long long * bad)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= m.ncell)
    {
        return;
    }
    bool ok = true;
    int const nf = m.cfcs(icl, 0);
    ok = nf >= 1 && nf <= 6;
    for (int k = 1; ok && k <= nf; ++k)
    {
        int64_t const ifc = m.cfcs(icl, k);
        if (ifc < -m.ngstface || ifc >= nface)
        {
            ok = false;
            break;
        }
        int64_t const c0 = m.fcls(ifc, 0);
        int64_t const c1 = m.fcls(ifc, 1);
        bool const mine = c0 == icl || c1 == icl;
        int64_t const other = c0 == icl ? c1 : c0;
        ok = mine && other >= -m.ngstcell && other < m.ncell;
        int const nn = m.fnds(ifc, 0);
        ok = ok && nn >= 1 && nn <= 4;
        for (int j = 1; ok && j <= nn; ++j)
        {
            int64_t const ind = m.fnds(ifc, j);
            ok = ind >= -m.ngstnode && ind < nnode;
        }
    }
    if (!ok)
    {
        atomicMin(bad, static_cast<unsigned long long>(icl));
    }
}

// Reference-layout CE geometry (FP64): cevol [nrowc][7], cecnd [nrowc][7*nd],
// sfcnd/sfnml [ncell][24][nd].  Ghost rows of cevol/cecnd stay zero.
struct CeView
{
    double * cevol;
    double * cecnd;
    double * sfcnd;
    double * sfnml;
};

// prepare_ce_2d (euler_ce.cpp:78-176), one thread per body cell.
__global__ void k_prepare_ce_2d(MeshView m, CeView ce)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= m.ncell)
    {
        return;
    }
    int64_t const row = icl + m.ngstcell;
    double * cevol = ce.cevol + row * 7;
    double * cecnd = ce.cecnd + row * 14;
    double * sfcnd = ce.sfcnd + icl * 48;
    double * sfnml = ce.sfnml + icl * 48;
    int const clnfc = m.cfcs(icl, 0);
    double volc = 0.0, cc0 = 0.0, cc1 = 0.0;
    double const ci0 = m.cc(icl, 0);
    double const ci1 = m.cc(icl, 1);
    for (int ifl = 1; ifl <= clnfc; ++ifl)
    {
        int32_t const ifc = m.cfcs(icl, ifl);
        int32_t const jcl = m.rcl(ifc, static_cast<int32_t>(icl));
        double const ce0 = m.cc(jcl, 0);
        double const ce1 = m.cc(jcl, 1);
        int32_t const n0 = m.fnds(ifc, 1);
        int32_t const n1 = m.fnds(ifc, 2);
        double const x10 = m.nd(n0, 0), x11 = m.nd(n0, 1);
        double const x20 = m.nd(n1, 0), x21 = m.nd(n1, 1);
        double const cndi0 = (x10 + x20 + ci0) / 3.0;
        double const cndi1 = (x11 + x21 + ci1) / 3.0;
        double const voli = fabs((x10 - ci0) * (x21 - ci1) - (x11 - ci1) * (x20 - ci0)) / 2.0;
        double const cnde0 = (x10 + x20 + ce0) / 3.0;
        double const cnde1 = (x11 + x21 + ce1) / 3.0;
        double const cross = (x10 - ce0) * (x21 - ce1) - (x11 - ce1) * (x20 - ce0);
        double const vole = fabs(cross) / 2.0;
        double const volb = voli + vole;
        cevol[ifl] = volb;
        cecnd[ifl * 2 + 0] = (cndi0 * voli + cnde0 * vole) / volb;
        cecnd[ifl * 2 + 1] = (cndi1 * voli + cnde1 * vole) / volb;
        volc += volb;
        cc0 += cndi0 * voli + cnde0 * vole;
        cc1 += cndi1 * voli + cnde1 * vole;
        int const sb = (ifl - 1) * 4;
        double const sgn = (cross > 0.0) ? 1.0 : -1.0;
        sfcnd[(sb + 0) * 2 + 0] = (ce0 + x10) / 2.0;
        sfcnd[(sb + 0) * 2 + 1] = (ce1 + x11) / 2.0;
        sfnml[(sb + 0) * 2 + 0] = -(ce1 - x11) * sgn;
        sfnml[(sb + 0) * 2 + 1] = (ce0 - x10) * sgn;
        sfcnd[(sb + 1) * 2 + 0] = (x20 + ce0) / 2.0;
        sfcnd[(sb + 1) * 2 + 1] = (x21 + ce1) / 2.0;
        sfnml[(sb + 1) * 2 + 0] = -(x21 - ce1) * sgn;
        sfnml[(sb + 1) * 2 + 1] = (x20 - ce0) * sgn;
    }
    cevol[0] = volc;
    cecnd[0] = cc0 / volc;
    cecnd[1] = cc1 / volc;
}

// prepare_ce_3d (euler_ce.cpp:178-347), one thread per body cell.
__global__ void k_prepare_ce_3d(MeshView m, CeView ce)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (icl >= m.ncell)
    {
        return;
    }
    int64_t const row = icl + m.ngstcell;
    double * cevol = ce.cevol + row * 7;
    double * cecnd = ce.cecnd + row * 21;
    double * sfcnd = ce.sfcnd + icl * 72;
    double * sfnml = ce.sfnml + icl * 72;
    int const clnfc = m.cfcs(icl, 0);
    double volc = 0.0, cc[3] = {0.0, 0.0, 0.0};
    double ci[3];
    for (int d = 0; d < 3; ++d)
    {
        ci[d] = m.cc(icl, d);
    }
    for (int ifl = 1; ifl <= clnfc; ++ifl)
    {
        int32_t const ifc = m.cfcs(icl, ifl);
        int32_t const jcl = m.rcl(ifc, static_cast<int32_t>(icl));
        int const fcnnd = m.fnds(ifc, 0);
        double ce[3], pf[3];
        for (int d = 0; d < 3; ++d)
        {
            ce[d] = m.cc(jcl, d);
            pf[d] = m.fc(ifc, d);
        }
        double crd[6][3];
        for (int inf = 1; inf <= fcnnd; ++inf)
        {
            int32_t const ind = m.fnds(ifc, inf);
            for (int d = 0; d < 3; ++d)
            {
                crd[inf][d] = m.nd(ind, d);
            }
        }
        for (int d = 0; d < 3; ++d)
        {
            crd[fcnnd + 1][d] = crd[1][d];
        }
        double volb = 0.0, bc[3] = {0.0, 0.0, 0.0};
        double const voe = (m.fcls(ifc, 0) == icl) ? 0.5 : -0.5;
        int const sb = (ifl - 1) * 4;
        for (int inf = 1; inf <= fcnnd; ++inf)
        {
            double const u0 = crd[inf][0] - pf[0], u1 = crd[inf][1] - pf[1], u2 = crd[inf][2] - pf[2];
            double const v0 = crd[inf + 1][0] - pf[0], v1 = crd[inf + 1][1] - pf[1], v2 = crd[inf + 1][2] - pf[2];
            double const t0 = u1 * v2 - u2 * v1;
            double const t1 = u2 * v0 - u0 * v2;
            double const t2 = u0 * v1 - u1 * v0;
            double const voli = fabs(t0 * (ci[0] - pf[0]) + t1 * (ci[1] - pf[1]) + t2 * (ci[2] - pf[2])) / 6.0;
            double const vole = fabs(t0 * (ce[0] - pf[0]) + t1 * (ce[1] - pf[1]) + t2 * (ce[2] - pf[2])) / 6.0;
            volb += voli + vole;
            for (int d = 0; d < 3; ++d)
            {
                double const cndi = (crd[inf][d] + crd[inf + 1][d] + pf[d] + ci[d]) / 4.0;
                double const cnde = (crd[inf][d] + crd[inf + 1][d] + pf[d] + ce[d]) / 4.0;
                bc[d] += cndi * voli + cnde * vole;
            }
            int const si = sb + inf - 1;
            for (int d = 0; d < 3; ++d)
            {
                sfcnd[si * 3 + d] = (ce[d] + crd[inf][d] + crd[inf + 1][d]) / 3.0;
            }
            double const a0 = crd[inf][0] - ce[0], a1 = crd[inf][1] - ce[1], a2 = crd[inf][2] - ce[2];
            double const b0 = crd[inf + 1][0] - ce[0], b1 = crd[inf + 1][1] - ce[1], b2 = crd[inf + 1][2] - ce[2];
            sfnml[si * 3 + 0] = (a1 * b2 - a2 * b1) * voe;
            sfnml[si * 3 + 1] = (a2 * b0 - a0 * b2) * voe;
            sfnml[si * 3 + 2] = (a0 * b1 - a1 * b0) * voe;
        }
        cevol[ifl] = volb;
        for (int d = 0; d < 3; ++d)
        {
            cecnd[ifl * 3 + d] = bc[d] / volb;
            cc[d] += bc[d];
        }
        volc += volb;
    }
    cevol[0] = volc;
    for (int d = 0; d < 3; ++d)
    {
        cecnd[d] = cc[d] / volc;
    }
}

// Compact the reference-layout CE geometry into the march's per-face
// moments and per-cell scalars (layout in euler_device.cuh), in FP64, then
// store them as G.  Also writes the neighbour-row table and the cell types.
template <int ND, typename G>
__global__ void k_compact(MeshView m, double const * cevol, double const * cecnd, double const * sfcnd,
                          double const * sfnml, double hdt, int nslot, G * fgeo, G * cgeo, int32_t * nbr,
                          int8_t * ctype)
{
    using D = Geo<ND, G>;
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t const nc = m.ncell;
    if (icl >= nc)
    {
        return;
    }
    int64_t const row = icl + m.ngstcell;
    int const clnfc = m.cfcs(icl, 0);
    ctype[icl] = static_cast<int8_t>(m.cltpn[row]);
    double ic[ND];
    for (int d = 0; d < ND; ++d)
    {
        ic[d] = cecnd[row * 7 * ND + d];
    }
    double mid[6][ND], ee[6][ND];
    double A[ND], B[ND];
    for (int d = 0; d < ND; ++d)
    {
        A[d] = 0.0;
        B[d] = 0.0;
    }
    double dist = 1.79769313486231570815e+308;
    auto put = [&](int f, int k, double v) { fgeo[(static_cast<int64_t>(f) * D::KF + k) * nc + icl] = G(v); };
    for (int f = 0; f < clnfc; ++f)
    {
        int const ifl = f + 1;
        int32_t const ifc = m.cfcs(icl, ifl);
        int32_t const jcl = m.rcl(ifc, static_cast<int32_t>(icl));
        nbr[f * nc + icl] = static_cast<int32_t>(jcl + m.ngstcell);
        double jce[ND], bc[ND];
        double d2 = 0.0;
        for (int d = 0; d < ND; ++d)
        {
            jce[d] = (jcl >= 0) ? cecnd[(jcl + m.ngstcell) * 7 * ND + d] : m.cc(jcl, d);
            bc[d] = cecnd[row * 7 * ND + ifl * ND + d];
            double const df = bc[d] - ic[d];
            d2 += df * df;
        }
        dist = fmin(dist, sqrt(d2));
        put(f, D::K_BVOL, cevol[row * 7 + ifl]);
        int const fcnnd = m.fnds(ifc, 0);
        double nsum[ND], msum[ND][ND];
        for (int d = 0; d < ND; ++d)
        {
            nsum[d] = 0.0;
            for (int e = 0; e < ND; ++e)
            {
                msum[e][d] = 0.0;
            }
        }
        for (int inf = 0; inf < fcnnd; ++inf)
        {
            int64_t const si = (icl * 24 + f * 4 + inf) * ND;
            for (int d = 0; d < ND; ++d)
            {
                double const n = sfnml[si + d];
                nsum[d] += n;
                for (int e = 0; e < ND; ++e)
                {
                    msum[e][d] += (sfcnd[si + e] - jce[e]) * n;
                }
            }
        }
        for (int d = 0; d < ND; ++d)
        {
            put(f, D::K_DB + d, bc[d] - jce[d]);
            put(f, D::K_NH + d, hdt * nsum[d]);
            for (int e = 0; e < ND; ++e)
            {
                put(f, D::K_MH + e * ND + d, hdt * msum[e][d]);
            }
            mid[f][d] = bc[d] - ic[d];
            ee[f][d] = jce[d] - bc[d];
            A[d] += mid[f][d];
            B[d] += ee[f][d];
        }
    }
    for (int d = 0; d < ND; ++d)
    {
        A[d] /= clnfc;
        B[d] /= clnfc;
    }
    for (int f = 0; f < clnfc; ++f)
    {
        for (int d = 0; d < ND; ++d)
        {
            if constexpr (D::MID)
            {
                put(f, D::K_MID + d, mid[f][d]);
            }
            else
            {
                put(f, D::K_P + d, mid[f][d] - A[d]);
                put(f, D::K_Q + d, ee[f][d] - B[d]);
                put(f, D::K_R + d, -(A[d] + ee[f][d]));
            }
        }
    }
    for (int f = clnfc; f < nslot; ++f)
    {
        nbr[f * nc + icl] = 0;
        for (int k = 0; k < D::KF; ++k)
        {
            put(f, k, 0.0);
        }
    }
    cgeo[0 * nc + icl] = G(1.0 / cevol[row * 7]);
    cgeo[1 * nc + icl] = G(hdt / dist);
}

} // namespace dev
} // namespace scg
