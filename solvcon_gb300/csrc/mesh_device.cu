/*
 * StaticMesh::build_interior on the GPU: the faces of every cell, their
 * de-duplication and numbering, the face-cell relations and the metrics
 * (cpp/solvcon/mesh/StaticMesh_interior.cpp:17-977), giving tables equal to
 * the host builder's (mesh_host.cpp) entry for entry.
 *
 *  1. Every cell writes its faces into consecutive slots (slot order = cell
 *     order, then the cell's face order of mesh_cells.hpp): type, nodes, and
 *     a 128-bit key of the face type and its sorted nodes.
 *  2. Two stable radix sorts (low word, then high word) order the slots by
 *     key, ties by slot; equal keys are one face, and its first slot is the
 *     first time the face was seen.
 *  3. Faces are numbered by the slot of their first sighting (a prefix sum
 *     over slot order), which is the numbering of the reference's
 *     de-duplication; every slot maps to its face, the face keeps the node
 *     order of its first sighting, and its first two cells are its fccls.
 *  4. The metric kernels evaluate the host builder's expressions in the same
 *     order (this file is compiled without FMA contraction, as the host code
 *     is), per face and per cell.  The reference's volume pass turns a face
 *     to point out of its first cell and, in degenerate cells, back again
 *     when its second cell sees it pointing outward too; both decisions
 *     depend only on the two cells' centroids, so each face settles its
 *     orientation on its own.
 */

#include "common.hpp"
#include "mesh_cells.hpp"
#include "mesh_host.hpp"

#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/gather.h>
#include <thrust/scan.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace scg
{

namespace
{

constexpr int TB = 256;

unsigned grid_of(int64_t n) { return static_cast<unsigned>((n + TB - 1) / TB); }

constexpr int64_t W5 = FCMND + 1; // fcnds width
constexpr int64_t W7 = CLMFC + 1; // clfcs width
constexpr int64_t W9 = CLMND + 1; // clnds width

__global__ void k_count(int32_t const * cltpn, int64_t ncell, int64_t * cnt)
{
    int64_t const i = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (i < ncell)
    {
        cnt[i] = cell_faces(cltpn[i]).nface;
    }
}

__global__ void k_emit(int32_t const * cltpn, int32_t const * clnds, int64_t const * off, int64_t ncell,
                       int32_t * tfctpn, int32_t * tfcnds, int32_t * tclfcs, int32_t * slot_cell, uint64_t * khi,
                       uint64_t * klo)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (icl >= ncell)
    {
        return;
    }
    CellFaces const cf = cell_faces(cltpn[icl]);
    int32_t const * row = clnds + icl * W9;
    int32_t * crow = tclfcs + icl * W7;
    crow[0] = cf.nface;
    for (int k = 0; k < cf.nface; ++k)
    {
        FaceDef const fd = cf.f[k];
        int64_t const slot = off[icl] + k;
        int32_t * frow = tfcnds + slot * W5;
        tfctpn[slot] = fd.type;
        frow[0] = fd.nnd;
        uint32_t nd[4] = {0x7fffffffu, 0x7fffffffu, 0x7fffffffu, 0x7fffffffu};
        for (int j = 0; j < (fd.nnd > 1 ? fd.nnd : 1); ++j)
        {
            frow[1 + j] = row[fd.pos[j]];
            if (j < fd.nnd)
            {
                nd[j] = static_cast<uint32_t>(row[fd.pos[j]]);
            }
        }
        // Sorted node ids (at most 4, 31 bits each) and the face type.
        for (int a = 1; a < 4; ++a)
        {
            uint32_t const v = nd[a];
            int b = a - 1;
            while (b >= 0 && nd[b] > v)
            {
                nd[b + 1] = nd[b];
                --b;
            }
            nd[b + 1] = v;
        }
        // Key: 2 bits of face type (line, quadrilateral, triangle), then the
        // four 31-bit node ids.
        uint64_t const t2 = fd.type == CT_LINE ? 0u : (fd.type == CT_QUAD ? 1u : (fd.type == CT_TRIANGLE ? 2u : 3u));
        khi[slot] = (t2 << 62) | (static_cast<uint64_t>(nd[0]) << 31) | nd[1];
        klo[slot] = (static_cast<uint64_t>(nd[2]) << 31) | nd[3];
        crow[1 + k] = static_cast<int32_t>(slot);
        slot_cell[slot] = static_cast<int32_t>(icl);
    }
}

// Group starts: start[p] = p where the key changes, else 0 (max-scanned
// afterwards to the start of p's group).
__global__ void k_starts(uint64_t const * hi, uint64_t const * lo, int64_t n, int64_t * start)
{
    int64_t const p = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (p < n)
    {
        start[p] = (p == 0 || hi[p] != hi[p - 1] || lo[p] != lo[p - 1]) ? p : 0;
    }
}

__global__ void k_heads(int64_t const * start, uint32_t const * idx, int64_t n, int32_t * is_head)
{
    int64_t const p = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (p < n && start[p] == p)
    {
        is_head[idx[p]] = 1;
    }
}

// Face of every slot: the number of its group's first slot.
__global__ void k_map(int64_t const * start, uint32_t const * idx, int32_t const * fid, int64_t n, int32_t * map2)
{
    int64_t const p = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (p < n)
    {
        map2[idx[p]] = fid[idx[start[p]]];
    }
}

// Face tables: type and nodes of the first sighting; fccls = the cells of
// the first two sightings.
__global__ void k_faces(int64_t const * start, uint32_t const * idx, int32_t const * map2, int32_t const * slot_cell,
                        int32_t const * tfctpn, int32_t const * tfcnds, int64_t n, int32_t * fctpn, int32_t * fcnds,
                        int32_t * fccls)
{
    int64_t const p = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (p >= n || start[p] != p)
    {
        return;
    }
    uint32_t const s = idx[p];
    int64_t const f = map2[s];
    fctpn[f] = tfctpn[s];
    for (int j = 0; j < W5; ++j)
    {
        fcnds[f * W5 + j] = tfcnds[s * W5 + j];
    }
    fccls[f * FCREL + 0] = slot_cell[s];
    fccls[f * FCREL + 1] = (p + 1 < n && start[p + 1] == p) ? slot_cell[idx[p + 1]] : -1;
    fccls[f * FCREL + 2] = -1;
    fccls[f * FCREL + 3] = -1;
}

__global__ void k_clfcs(int32_t const * tclfcs, int32_t const * map2, int64_t ncell, int32_t * clfcs)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (icl >= ncell)
    {
        return;
    }
    int32_t const * t = tclfcs + icl * W7;
    int32_t * c = clfcs + icl * W7;
    c[0] = t[0];
    for (int k = 1; k < W7; ++k)
    {
        c[k] = k <= t[0] ? map2[t[k]] : -1;
    }
}

// ---- metrics (mesh_host.cpp calc_metric, same expressions, same order) ----

struct MetricView
{
    int ndim;
    int64_t nface, ncell;
    double const * ndcrd;
    int32_t * fcnds;
    int32_t const * fccls;
    int32_t const * clnds;
    int32_t const * clfcs;
    double * fccnd;
    double * fcnml;
    double * fcara;
    double * clcnd;
    double * clvol;
};

__global__ void k_face_metric(MetricView v)
{
    int64_t const ifc = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (ifc >= v.nface)
    {
        return;
    }
    int32_t const * fn = v.fcnds + ifc * W5;
    double const * x = v.ndcrd;
    if (v.ndim == 2)
    {
        int32_t const a = fn[1], b = fn[2];
        v.fccnd[ifc * 2 + 0] = (x[a * 2 + 0] + x[b * 2 + 0]) / 2;
        v.fccnd[ifc * 2 + 1] = (x[a * 2 + 1] + x[b * 2 + 1]) / 2;
        double const n0 = x[b * 2 + 1] - x[a * 2 + 1];
        double const n1 = x[a * 2 + 0] - x[b * 2 + 0];
        double const ar = sqrt(n0 * n0 + n1 * n1);
        v.fcara[ifc] = ar;
        v.fcnml[ifc * 2 + 0] = n0 / ar;
        v.fcnml[ifc * 2 + 1] = n1 / ar;
        return;
    }
    int const nnd = fn[0];
    double cfd[FCMND + 2][3] = {};
    for (int inf = 1; inf <= nnd; ++inf)
    {
        int32_t const ind = fn[inf];
        for (int d = 0; d < 3; ++d)
        {
            cfd[inf][d] = x[ind * 3 + d];
            cfd[0][d] += x[ind * 3 + d];
        }
    }
    for (int d = 0; d < 3; ++d)
    {
        cfd[nnd + 1][d] = cfd[1][d];
    }
    for (int d = 0; d < 3; ++d)
    {
        cfd[0][d] /= nnd;
    }
    double voc = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0;
    for (int inf = 1; inf <= nnd; ++inf)
    {
        double const m0 = (cfd[0][0] + cfd[inf][0] + cfd[inf + 1][0]) / 3;
        double const m1 = (cfd[0][1] + cfd[inf][1] + cfd[inf + 1][1]) / 3;
        double const m2 = (cfd[0][2] + cfd[inf][2] + cfd[inf + 1][2]) / 3;
        double const u0 = cfd[inf][0] - cfd[0][0];
        double const u1 = cfd[inf][1] - cfd[0][1];
        double const u2 = cfd[inf][2] - cfd[0][2];
        double const v0 = cfd[inf + 1][0] - cfd[0][0];
        double const v1 = cfd[inf + 1][1] - cfd[0][1];
        double const v2 = cfd[inf + 1][2] - cfd[0][2];
        double const w0 = u1 * v2 - u2 * v1;
        double const w1 = u2 * v0 - u0 * v2;
        double const w2 = u0 * v1 - u1 * v0;
        double const ar = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
        c0 += m0 * ar;
        c1 += m1 * ar;
        c2 += m2 * ar;
        voc += ar;
    }
    double cc[3] = {c0 / voc, c1 / voc, c2 / voc};
    for (int d = 0; d < 3; ++d)
    {
        v.fccnd[ifc * 3 + d] = cc[d];
    }
    double rv[FCMND][3] = {};
    for (int inf = 0; inf < nnd; ++inf)
    {
        int32_t const ind = fn[inf + 1];
        for (int d = 0; d < 3; ++d)
        {
            rv[inf][d] = x[ind * 3 + d] - cc[d];
        }
    }
    double n0 = rv[nnd - 1][1] * rv[0][2] - rv[nnd - 1][2] * rv[0][1];
    double n1 = rv[nnd - 1][2] * rv[0][0] - rv[nnd - 1][0] * rv[0][2];
    double n2 = rv[nnd - 1][0] * rv[0][1] - rv[nnd - 1][1] * rv[0][0];
    for (int k = 1; k < nnd; ++k)
    {
        n0 += rv[k - 1][1] * rv[k][2] - rv[k - 1][2] * rv[k][1];
        n1 += rv[k - 1][2] * rv[k][0] - rv[k - 1][0] * rv[k][2];
        n2 += rv[k - 1][0] * rv[k][1] - rv[k - 1][1] * rv[k][0];
    }
    double const ar = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    v.fcnml[ifc * 3 + 0] = n0 / ar;
    v.fcnml[ifc * 3 + 1] = n1 / ar;
    v.fcnml[ifc * 3 + 2] = n2 / ar;
    v.fcara[ifc] = ar / 2.0;
}

__global__ void k_cell_centroid(MetricView v)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (icl >= v.ncell)
    {
        return;
    }
    int const nd = v.ndim;
    double const frac = (nd == 2) ? 3.0 : 4.0;
    double crd[3] = {0.0, 0.0, 0.0};
    int32_t const * cn = v.clnds + icl * W9;
    int const nnd = cn[0];
    for (int inc = 1; inc <= nnd; ++inc)
    {
        for (int d = 0; d < nd; ++d)
        {
            crd[d] += v.ndcrd[cn[inc] * nd + d];
        }
    }
    for (int d = 0; d < nd; ++d)
    {
        crd[d] /= nnd;
    }
    double acc[3] = {0.0, 0.0, 0.0};
    double voc = 0.0;
    int32_t const * cf = v.clfcs + icl * W7;
    for (int ifl = 1; ifl <= cf[0]; ++ifl)
    {
        int64_t const ifc = cf[ifl];
        double du[3] = {};
        double dot = 0.0;
        for (int d = 0; d < nd; ++d)
        {
            du[d] = crd[d] - v.fccnd[ifc * nd + d];
            dot += du[d] * v.fcnml[ifc * nd + d];
        }
        double const vob = fabs(dot) * v.fcara[ifc];
        voc += vob;
        for (int d = 0; d < nd; ++d)
        {
            acc[d] += (v.fccnd[ifc * nd + d] + du[d] / frac) * vob;
        }
    }
    for (int d = 0; d < nd; ++d)
    {
        v.clcnd[icl * nd + d] = acc[d] / voc;
    }
}

// The signed face volume of the host's volume pass, with normal sign s.
__device__ __forceinline__ double face_vol(MetricView const & v, int64_t ifc, int64_t icl, double s)
{
    int const nd = v.ndim;
    double vol = 0.0;
    for (int d = 0; d < nd; ++d)
    {
        vol += (v.fccnd[ifc * nd + d] - v.clcnd[icl * nd + d]) * (s * v.fcnml[ifc * nd + d]);
    }
    return vol * v.fcara[ifc];
}

// Cell volumes: the sum of |face volume| over the cell's faces (the sign of
// a face's normal when its cell is visited does not change the magnitude).
__global__ void k_cell_volume(MetricView v)
{
    int64_t const icl = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (icl >= v.ncell)
    {
        return;
    }
    double vsum = 0.0;
    int32_t const * cf = v.clfcs + icl * W7;
    for (int it = 1; it <= cf[0]; ++it)
    {
        double vol = face_vol(v, cf[it], icl, 1.0);
        if (vol < 0.0)
        {
            vol = -vol;
        }
        vsum += vol;
    }
    v.clvol[icl] = vsum / v.ndim;
}

// Final face orientation: the first cell turns the face outward when its
// volume is negative; the second cell, seeing the face as left by the first,
// turns it when its volume is not negative.
__global__ void k_face_orient(MetricView v)
{
    int64_t const ifc = static_cast<int64_t>(blockIdx.x) * TB + threadIdx.x;
    if (ifc >= v.nface)
    {
        return;
    }
    int32_t const c0 = v.fccls[ifc * FCREL + 0];
    int32_t const c1 = v.fccls[ifc * FCREL + 1];
    bool flip = false;
    if (c0 >= 0 && face_vol(v, ifc, c0, 1.0) < 0.0)
    {
        flip = true;
    }
    if (c1 >= 0 && c1 != c0 && !(face_vol(v, ifc, c1, flip ? -1.0 : 1.0) < 0.0))
    {
        flip = !flip;
    }
    if (flip)
    {
        int32_t * fn = v.fcnds + ifc * W5;
        int const nnd = fn[0];
        int32_t tmp[FCMND];
        for (int j = 0; j < nnd; ++j)
        {
            tmp[j] = fn[nnd - j];
        }
        for (int j = 0; j < nnd; ++j)
        {
            fn[j + 1] = tmp[j];
        }
        for (int d = 0; d < v.ndim; ++d)
        {
            v.fcnml[ifc * v.ndim + d] = -v.fcnml[ifc * v.ndim + d];
        }
    }
}

template <typename T>
T * raw(thrust::device_vector<T> & v)
{
    return thrust::raw_pointer_cast(v.data());
}

template <typename T>
void to_host(thrust::device_vector<T> const & d, T * h, size_t n)
{
    cuda_check(cudaMemcpy(h, thrust::raw_pointer_cast(d.data()), n * sizeof(T), cudaMemcpyDeviceToHost), "D2H");
}

} // namespace

void HostMesh::build_interior_device(bool do_metric, bool do_edge)
{
    validate_cells();
    for (int64_t icl = 0; icl < ncell; ++icl)
    {
        if (cell_ndim(cltpn(icl)) != ndim)
        {
            throw std::invalid_argument("StaticMesh::build_interior: the device builder takes cells of the mesh "
                                        "dimension only; cell " +
                                        std::to_string(icl) + " has type " + std::to_string(cltpn(icl)));
        }
    }
    if (ncell == 0 || ngstnode || ngstface || ngstcell)
    {
        // Nothing to build, or a mesh whose ghost layer exists already: the
        // host builder handles both.
        build_interior(do_metric, do_edge);
        return;
    }
    using thrust::device_vector;
    device_vector<int32_t> d_cltpn(cltpn.buf.begin(), cltpn.buf.end());
    device_vector<int32_t> d_clnds(clnds.buf.begin(), clnds.buf.end());
    device_vector<int64_t> off(static_cast<size_t>(ncell));
    k_count<<<grid_of(ncell), TB>>>(raw(d_cltpn), ncell, raw(off));
    cuda_check(cudaGetLastError(), "k_count");
    int64_t const last_cnt = off[static_cast<size_t>(ncell - 1)];
    thrust::exclusive_scan(thrust::device, off.begin(), off.end(), off.begin());
    int64_t const mface = off[static_cast<size_t>(ncell - 1)] + last_cnt;
    if (mface > INT32_MAX)
    {
        throw std::invalid_argument("StaticMesh::build_interior: too many cell faces for the device builder");
    }

    device_vector<int32_t> tfctpn(static_cast<size_t>(mface), -1);
    device_vector<int32_t> tfcnds(static_cast<size_t>(mface * W5), -1);
    device_vector<int32_t> tclfcs(static_cast<size_t>(ncell * W7), -1);
    device_vector<int32_t> slot_cell(static_cast<size_t>(mface));
    device_vector<uint64_t> khi(static_cast<size_t>(mface)), klo(static_cast<size_t>(mface));
    k_emit<<<grid_of(ncell), TB>>>(raw(d_cltpn), raw(d_clnds), raw(off), ncell, raw(tfctpn), raw(tfcnds), raw(tclfcs),
                                   raw(slot_cell), raw(khi), raw(klo));
    cuda_check(cudaGetLastError(), "k_emit");

    // Order the slots by (key, slot): stable sort by the low word, then by
    // the high word.
    device_vector<uint32_t> idx(static_cast<size_t>(mface));
    thrust::sequence(thrust::device, idx.begin(), idx.end());
    {
        device_vector<uint64_t> k(klo);
        thrust::stable_sort_by_key(thrust::device, k.begin(), k.end(), idx.begin());
        thrust::gather(thrust::device, idx.begin(), idx.end(), khi.begin(), k.begin());
        thrust::stable_sort_by_key(thrust::device, k.begin(), k.end(), idx.begin());
        khi.swap(k);
    }
    {
        device_vector<uint64_t> k(static_cast<size_t>(mface));
        thrust::gather(thrust::device, idx.begin(), idx.end(), klo.begin(), k.begin());
        klo.swap(k);
    }
    device_vector<int64_t> start(static_cast<size_t>(mface));
    k_starts<<<grid_of(mface), TB>>>(raw(khi), raw(klo), mface, raw(start));
    cuda_check(cudaGetLastError(), "k_starts");
    thrust::inclusive_scan(thrust::device, start.begin(), start.end(), start.begin(), thrust::maximum<int64_t>());
    khi.clear();
    khi.shrink_to_fit();
    klo.clear();
    klo.shrink_to_fit();

    device_vector<int32_t> fid(static_cast<size_t>(mface), 0);
    k_heads<<<grid_of(mface), TB>>>(raw(start), raw(idx), mface, raw(fid));
    cuda_check(cudaGetLastError(), "k_heads");
    int32_t const last_head = fid[static_cast<size_t>(mface - 1)];
    thrust::exclusive_scan(thrust::device, fid.begin(), fid.end(), fid.begin());
    nface = static_cast<int64_t>(fid[static_cast<size_t>(mface - 1)]) + last_head;

    device_vector<int32_t> map2(static_cast<size_t>(mface));
    k_map<<<grid_of(mface), TB>>>(raw(start), raw(idx), raw(fid), mface, raw(map2));
    cuda_check(cudaGetLastError(), "k_map");
    device_vector<int32_t> d_fctpn(static_cast<size_t>(nface)), d_fcnds(static_cast<size_t>(nface * W5));
    device_vector<int32_t> d_fccls(static_cast<size_t>(nface * FCREL));
    k_faces<<<grid_of(mface), TB>>>(raw(start), raw(idx), raw(map2), raw(slot_cell), raw(tfctpn), raw(tfcnds), mface,
                                    raw(d_fctpn), raw(d_fcnds), raw(d_fccls));
    cuda_check(cudaGetLastError(), "k_faces");
    device_vector<int32_t> d_clfcs(static_cast<size_t>(ncell * W7));
    k_clfcs<<<grid_of(ncell), TB>>>(raw(tclfcs), raw(map2), ncell, raw(d_clfcs));
    cuda_check(cudaGetLastError(), "k_clfcs");

    // Tables the device results overwrite in full are not filled first.
    remake_unset(fctpn, 0, nface, 1);
    remake_unset(fcnds, 0, nface, FCMND + 1);
    remake_unset(fccls, 0, nface, FCREL);
    remake_unset(clfcs, 0, ncell, CLMFC + 1);
    if (do_metric)
    {
        remake_unset(fccnd, 0, nface, ndim);
        remake_unset(fcnml, 0, nface, ndim);
        remake_unset(fcara, 0, nface, 1);
    }
    else
    {
        remake(fccnd, 0, nface, ndim, 0.0);
        remake(fcnml, 0, nface, ndim, 0.0);
        remake(fcara, 0, nface, 1, 0.0);
    }
    if (do_metric)
    {
        device_vector<double> d_ndcrd(ndcrd.buf.begin(), ndcrd.buf.end());
        device_vector<double> d_fccnd(static_cast<size_t>(nface * ndim)), d_fcnml(static_cast<size_t>(nface * ndim));
        device_vector<double> d_fcara(static_cast<size_t>(nface));
        device_vector<double> d_clcnd(static_cast<size_t>(ncell * ndim)), d_clvol(static_cast<size_t>(ncell));
        MetricView v{ndim,        nface,        ncell,        raw(d_ndcrd), raw(d_fcnds), raw(d_fccls), raw(d_clnds),
                     raw(d_clfcs), raw(d_fccnd), raw(d_fcnml), raw(d_fcara), raw(d_clcnd), raw(d_clvol)};
        k_face_metric<<<grid_of(nface), TB>>>(v);
        k_cell_centroid<<<grid_of(ncell), TB>>>(v);
        k_cell_volume<<<grid_of(ncell), TB>>>(v);
        k_face_orient<<<grid_of(nface), TB>>>(v);
        cuda_check(cudaGetLastError(), "metric kernels");
        to_host(d_fccnd, fccnd.data(), static_cast<size_t>(nface * ndim));
        to_host(d_fcnml, fcnml.data(), static_cast<size_t>(nface * ndim));
        to_host(d_fcara, fcara.data(), static_cast<size_t>(nface));
        to_host(d_clcnd, clcnd.data(), static_cast<size_t>(ncell * ndim));
        to_host(d_clvol, clvol.data(), static_cast<size_t>(ncell));
    }
    to_host(d_fctpn, fctpn.data(), static_cast<size_t>(nface));
    to_host(d_fcnds, fcnds.data(), static_cast<size_t>(nface * W5));
    to_host(d_fccls, fccls.data(), static_cast<size_t>(nface * FCREL));
    to_host(d_clfcs, clfcs.data(), static_cast<size_t>(ncell * W7));
    cuda_check(cudaDeviceSynchronize(), "mesh build");
    if (do_edge)
    {
        build_edge();
    }
}

} // namespace scg

