/*
 * Batched march of many independent Euler cores in one launch per substep.
 *
 * Each core keeps its own device buffers.  The batch holds, per core, the
 * kernel argument block of each of the two substeps of a step (the two
 * differ only in which record buffer is current), and a work list of
 * (core, row tile) pairs covering every core's body cells and ghost rows.
 * The batch kernel walks the work list -- persistently (a grid sized to the
 * resident capacity of the GPU, each block striding over tiles) or one block
 * per tile -- and runs the same per-thread substep as the single-core fused
 * kernel.  One step is two launches (a kernel boundary is the grid-wide
 * barrier between the substeps); they are captured once into a CUDA graph and
 * replayed.  Tile size (the block size) and the grid policy are chosen by the
 * autotuner in solvcon_gb300/batch.py.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "euler_core.hpp"
#include "euler_kernels.cuh"

#include <memory>
#include <string>
#include <vector>

namespace
{

using scg::dev::MarchArgs;

// CT1: the one cell type of every core (then only that type's path is
// compiled and the kernel needs only its registers), or 0 for any mix.
// Every thread of a tile works on the same core, so the tile's argument
// block is staged once in shared memory and read from there as needed, as
// the single-core kernel reads its parameters, instead of being held in
// registers.
template <int ND, typename R, typename G, int B, int CT1>
__device__ __forceinline__ void fused_batch_tiles(MarchArgs<R, G> const * descs, int2 const * tiles, int ntiles)
{
    using Args = MarchArgs<R, G>;
    static_assert(sizeof(Args) % sizeof(int) == 0, "argument block is whole words");
    constexpr int NW = static_cast<int>(sizeof(Args) / sizeof(int));
    static_assert(NW <= B, "one word per thread");
    __shared__ __align__(16) int words[NW];
    Args const & a = *reinterpret_cast<Args const *>(words);
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
        int2 const tl = tiles[t];
        __syncthreads(); // the previous tile is done with the block
        if (threadIdx.x < NW)
        {
            words[threadIdx.x] = reinterpret_cast<int const *>(descs + tl.x)[threadIdx.x];
        }
        __syncthreads();
        scg::dev::fused_thread<ND, R, G, CT1, scg::dev::carry_shared<ND>() ? B : 0>(
            a, static_cast<int64_t>(tl.y) + threadIdx.x);
    }
}

template <int ND, typename R, typename G, int B, int CT1>
__global__ void __launch_bounds__(B) k_fused_batch(MarchArgs<R, G> const * descs, int2 const * tiles, int ntiles)
{
    fused_batch_tiles<ND, R, G, B, CT1>(descs, tiles, ntiles);
}

// The same with the resident-block request of the single-core kernel whose
// cells carry calc_soln's neighbour terms (scg::dev::min_blocks).
template <int ND, typename R, typename G, int B, int CT1, int MINB>
__global__ void __launch_bounds__(B, MINB) k_fused_batch_mb(MarchArgs<R, G> const * descs, int2 const * tiles,
                                                            int ntiles)
{
    fused_batch_tiles<ND, R, G, B, CT1>(descs, tiles, ntiles);
}

template <int ND, typename R, typename G, int B, int CT1>
constexpr int batch_min_blocks()
{
    if constexpr (CT1 == 0)
    {
        return 0;
    }
    else
    {
        return scg::dev::min_blocks<ND, R, CT1, B, G>();
    }
}

template <int ND, typename R, typename G, int B, int CT1>
constexpr auto batch_kernel()
{
    constexpr int MINB = batch_min_blocks<ND, R, G, B, CT1>();
    if constexpr (MINB > 0)
    {
        return &k_fused_batch_mb<ND, R, G, B, CT1, MINB>;
    }
    else
    {
        return &k_fused_batch<ND, R, G, B, CT1>;
    }
}

struct BatchBase
{
    virtual ~BatchBase() = default;
    // Point the batch at another set of cores, keeping its stream, device
    // tables (grown when too small) and occupancy; false (and nothing
    // changed) when the set needs another kernel than this batch's.
    virtual bool retarget(std::vector<scg::EulerCoreBase *> cores) = 0;
    virtual void march(int64_t steps) = 0;
    virtual void sync() = 0;
    virtual cudaStream_t get_stream() const = 0;
    int64_t ncore = 0, ncell = 0, ntiles = 0, grid = 0;
    int block = 0;
    double last_ms = 0.0; // device time of the last march's launches
};

template <int ND, typename R, typename G, int B, int CT1>
class Batch : public BatchBase
{
public:
    using Args = MarchArgs<R, G>;

    Batch(std::vector<scg::EulerCoreBase *> cores_in, bool persistent)
        : cores(std::move(cores_in)), persistent(persistent)
    {
        block = B;
        scg::cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        scg::cuda_check(cudaEventCreate(&ev[0]), "event");
        scg::cuda_check(cudaEventCreate(&ev[1]), "event");
        int dev = 0, nsm = 0, occ = 0;
        scg::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        scg::cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "attr");
        scg::cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel<ND, R, G, B, CT1>(), B, 0),
                        "occupancy");
        resident = static_cast<int64_t>(nsm) * std::max(occ, 1);
        layout();
    }

    // The precision code of the cores this instantiation marches.
    static constexpr int PREC = sizeof(R) == 8 ? scg::PREC_FP64
                                               : (sizeof(G) == 8 ? scg::PREC_FP32_GEOM64 : scg::PREC_FP32);

    bool retarget(std::vector<scg::EulerCoreBase *> cs) override
    {
        if (cs.empty())
        {
            throw std::invalid_argument("EulerBatch: no cores");
        }
        constexpr int SIMPLEX = (ND == 2) ? scg::CT_TRIANGLE : scg::CT_TET;
        bool all = true;
        for (auto * c : cs)
        {
            if (c->ndim != ND || c->precision != PREC)
            {
                return false;
            }
            all = all && c->single_ct == SIMPLEX;
        }
        // make_for_block's choice for the new set must be this kernel.
        if ((CT1 != 0) != all)
        {
            return false;
        }
        sync();
        cores = std::move(cs);
        Args const * const d0 = descs[0].ptr;
        Args const * const d1 = descs[1].ptr;
        int2 const * const t0 = tiles.ptr;
        layout();
        if (graph_exec && (descs[0].ptr != d0 || descs[1].ptr != d1 || tiles.ptr != t0 || !update_graph()))
        {
            drop_graph(); // captured again at the next march
        }
        return true;
    }

    // Point the captured step's two kernel nodes at the new work list (its
    // length and the grid; the device tables did not move) without capturing
    // again.  False when the runtime refuses the update.
    bool update_graph()
    {
        for (cudaGraphNode_t node : graph_nodes)
        {
            cudaKernelNodeParams p{};
            if (cudaGraphKernelNodeGetParams(node, &p) != cudaSuccess || !p.kernelParams)
            {
                (void)cudaGetLastError();
                return false;
            }
            Args const * d = *static_cast<Args const * const *>(p.kernelParams[0]);
            int2 const * t = tiles.ptr;
            int n = static_cast<int>(ntiles);
            void * args[3] = {&d, &t, &n};
            p.gridDim = dim3(static_cast<unsigned>(grid), 1, 1);
            p.kernelParams = args;
            p.extra = nullptr;
            if (cudaGraphExecKernelNodeSetParams(graph_exec, node, &p) != cudaSuccess)
            {
                (void)cudaGetLastError();
                return false;
            }
        }
        return true;
    }

    void drop_graph()
    {
        if (graph_exec)
        {
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
        if (graph)
        {
            cudaGraphDestroy(graph);
            graph = nullptr;
        }
        graph_nodes.clear();
    }

    // The work list of (core, row tile) pairs, the device tables sized for
    // it (grown, never shrunk) and the grid.
    void layout()
    {
        ncore = static_cast<int64_t>(cores.size());
        ncell = 0;
        std::vector<int2> tl;
        for (int64_t c = 0; c < ncore; ++c)
        {
            auto * core = cores[static_cast<size_t>(c)];
            int64_t const nthr = core->ncell + core->ngstcell;
            ncell += core->ncell;
            for (int64_t s = 0; s < nthr; s += B)
            {
                if (s > INT32_MAX - B)
                {
                    throw std::invalid_argument("EulerBatch: a core has too many rows for the work list");
                }
                tl.push_back(make_int2(static_cast<int>(c), static_cast<int>(s)));
            }
        }
        ntiles = static_cast<int64_t>(tl.size());
        if (ntiles > INT32_MAX)
        {
            throw std::invalid_argument("EulerBatch: work list too long");
        }
        if (tiles.n < tl.size() || !tiles.ptr)
        {
            tiles.alloc(std::max<size_t>(tl.size() + tl.size() / 2, 1));
        }
        if (!tl.empty())
        {
            // On the batch's own stream, then waited for: a plain cudaMemcpy
            // from pageable memory returns before its DMA lands and is not
            // ordered with this non-blocking stream, so the next launch could
            // read a work list half old, half new (each thread reads its
            // tile, and the two halves of a block would stage argument words
            // of two different cores).
            scg::cuda_check(cudaMemcpyAsync(tiles.ptr, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                            stream),
                            "H2D");
            sync();
        }
        size_t const nd = static_cast<size_t>(std::max<int64_t>(ncore, 1));
        for (auto & d : descs)
        {
            if (d.n < nd || !d.ptr)
            {
                d.alloc(nd + nd / 2);
            }
        }
        grid = persistent ? std::min<int64_t>(ntiles, resident) : ntiles;
        grid = std::max<int64_t>(grid, 1);
    }

    ~Batch() override
    {
        cudaEventDestroy(ev[0]);
        cudaEventDestroy(ev[1]);
        drop_graph();
        if (stream)
        {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    // Refresh both argument tables from the cores' current state.
    void prepare()
    {
        std::vector<Args> h[2];
        for (int p = 0; p < 2; ++p)
        {
            h[p].resize(static_cast<size_t>(ncore));
        }
        // A batched march never writes a core's registered host blocks (the
        // step graph is shared by all cores); refuse such a core instead of
        // leaving its blocks silently stale.
        for (int64_t c = 0; c < ncore; ++c)
        {
            if (cores[static_cast<size_t>(c)]->delivering())
            {
                throw std::invalid_argument("EulerBatch: core " + std::to_string(c) +
                                            " has host blocks registered with scg_euler_deliver, which batched "
                                            "marches do not write; unregister them first");
            }
        }
        for (int64_t c = 0; c < ncore; ++c)
        {
            auto * core = cores[static_cast<size_t>(c)];
            core->batch_begin();
            core->fill_args(1, &h[0][static_cast<size_t>(c)], sizeof(Args));
            core->fill_args(0, &h[1][static_cast<size_t>(c)], sizeof(Args));
        }
        for (int p = 0; p < 2; ++p)
        {
            if (ncore > 0)
            {
                scg::cuda_check(cudaMemcpyAsync(descs[p].ptr, h[p].data(), sizeof(Args) * h[p].size(),
                                                cudaMemcpyHostToDevice, stream),
                                "H2D");
            }
        }
        sync();
    }

    void launch_step()
    {
        for (int p = 0; p < 2; ++p)
        {
            batch_kernel<ND, R, G, B, CT1>()<<<static_cast<unsigned>(grid), B, 0, stream>>>(
                descs[p].ptr, tiles.ptr, static_cast<int>(ntiles));
            scg::launched(stream, "fused_batch");
        }
    }

    // The step's two launches as a graph; the graph and its kernel nodes are
    // kept for update_graph.
    void capture()
    {
        scg::cuda_check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "BeginCapture");
        int64_t const before = scg::g_launches.load();
        launch_step();
        scg::g_launches.store(before);
        scg::cuda_check(cudaStreamEndCapture(stream, &graph), "EndCapture");
        scg::cuda_check(cudaGraphInstantiate(&graph_exec, graph, 0), "GraphInstantiate");
        size_t n = 0;
        scg::cuda_check(cudaGraphGetNodes(graph, nullptr, &n), "GraphGetNodes");
        graph_nodes.resize(n);
        scg::cuda_check(cudaGraphGetNodes(graph, graph_nodes.data(), &n), "GraphGetNodes");
    }

    void march(int64_t steps) override
    {
        if (steps <= 0 || ntiles == 0)
        {
            return;
        }
        prepare();
        if (!graph_exec)
        {
            capture();
        }
        scg::cuda_check(cudaEventRecord(ev[0], stream), "record");
        for (int64_t s = 0; s < steps; ++s)
        {
            scg::cuda_check(cudaGraphLaunch(graph_exec, stream), "cudaGraphLaunch");
            scg::g_launches.fetch_add(2, std::memory_order_relaxed);
        }
        scg::cuda_check(cudaEventRecord(ev[1], stream), "record");
        sync();
        float ms = 0.f;
        scg::cuda_check(cudaEventElapsedTime(&ms, ev[0], ev[1]), "elapsed");
        last_ms = ms;
        for (auto * core : cores)
        {
            core->batch_end(steps);
        }
    }

    void sync() override { scg::cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }
    cudaStream_t get_stream() const override { return stream; }

private:
    std::vector<scg::EulerCoreBase *> cores;
    bool persistent = true;
    int64_t resident = 1; // SM count x resident blocks of this kernel
    scg::DevBuf<Args> descs[2];
    scg::DevBuf<int2> tiles;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    std::vector<cudaGraphNode_t> graph_nodes;
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

template <int ND, typename R, typename G, int CT1>
std::unique_ptr<BatchBase> make_for_type(std::vector<scg::EulerCoreBase *> cores, int block, bool persistent)
{
    switch (block)
    {
    case 64: return std::make_unique<Batch<ND, R, G, 64, CT1>>(std::move(cores), persistent);
    case 128: return std::make_unique<Batch<ND, R, G, 128, CT1>>(std::move(cores), persistent);
    case 256: return std::make_unique<Batch<ND, R, G, 256, CT1>>(std::move(cores), persistent);
    default: throw std::invalid_argument("EulerBatch: block must be 64, 128 or 256");
    }
}

// The simplex-only kernel when every core has only triangles (2D) or only
// tetrahedra (3D), else the kernel that dispatches on each cell's type.
template <int ND, typename R, typename G>
std::unique_ptr<BatchBase> make_for_block(std::vector<scg::EulerCoreBase *> cores, int block, bool persistent)
{
    constexpr int SIMPLEX = (ND == 2) ? scg::CT_TRIANGLE : scg::CT_TET;
    bool all = true;
    for (auto * c : cores)
    {
        all = all && c->single_ct == SIMPLEX;
    }
    if (all)
    {
        return make_for_type<ND, R, G, SIMPLEX>(std::move(cores), block, persistent);
    }
    return make_for_type<ND, R, G, 0>(std::move(cores), block, persistent);
}

std::unique_ptr<BatchBase> make_batch(std::vector<scg::EulerCoreBase *> cores, int block, bool persistent)
{
    if (cores.empty())
    {
        throw std::invalid_argument("EulerBatch: no cores");
    }
    int const nd = cores[0]->ndim;
    int const prec = cores[0]->precision;
    for (auto * c : cores)
    {
        if (c->ndim != nd || c->precision != prec)
        {
            throw std::invalid_argument("EulerBatch: every core must have the same ndim and precision");
        }
    }
    if (nd == 2)
    {
        if (prec == scg::PREC_FP64)
            return make_for_block<2, double, double>(std::move(cores), block, persistent);
        if (prec == scg::PREC_FP32_GEOM64)
            return make_for_block<2, float, double>(std::move(cores), block, persistent);
        return make_for_block<2, float, float>(std::move(cores), block, persistent);
    }
    if (prec == scg::PREC_FP64)
        return make_for_block<3, double, double>(std::move(cores), block, persistent);
    if (prec == scg::PREC_FP32_GEOM64)
        return make_for_block<3, float, double>(std::move(cores), block, persistent);
    return make_for_block<3, float, float>(std::move(cores), block, persistent);
}

} // namespace

struct scg_batch
{
    std::unique_ptr<BatchBase> b;
};

extern "C"
{

int scg_batch_create(scg_euler * const * cores, int64_t ncore, int block, int persistent, scg_batch ** out)
{
    return scg::guarded([&] {
        std::vector<scg::EulerCoreBase *> v;
        for (int64_t i = 0; i < ncore; ++i)
        {
            if (!cores[i] || !cores[i]->c)
            {
                throw std::invalid_argument("EulerBatch: null core handle");
            }
            v.push_back(cores[i]->c.get());
        }
        auto h = std::make_unique<scg_batch>();
        h->b = make_batch(std::move(v), block, persistent != 0);
        *out = h.release();
    });
}

int scg_batch_retarget(scg_batch * batch, scg_euler * const * cores, int64_t ncore, int * done)
{
    return scg::guarded([&] {
        if (!batch || !done)
        {
            throw std::invalid_argument("scg_batch_retarget: null argument");
        }
        std::vector<scg::EulerCoreBase *> v;
        for (int64_t i = 0; i < ncore; ++i)
        {
            if (!cores[i] || !cores[i]->c)
            {
                throw std::invalid_argument("EulerBatch: null core handle");
            }
            v.push_back(cores[i]->c.get());
        }
        *done = batch->b->retarget(std::move(v)) ? 1 : 0;
    });
}

int scg_batch_destroy(scg_batch * batch)
{
    return scg::guarded([&] { delete batch; });
}

int scg_batch_info(const scg_batch * batch, int64_t * out)
{
    return scg::guarded([&] {
        out[0] = batch->b->ncore;
        out[1] = batch->b->ncell;
        out[2] = batch->b->ntiles;
        out[3] = batch->b->grid;
        out[4] = batch->b->block;
    });
}

int scg_batch_last_ms(const scg_batch * batch, double * ms)
{
    return scg::guarded([&] { *ms = batch->b->last_ms; });
}

int scg_batch_march(scg_batch * batch, int64_t steps)
{
    return scg::guarded([&] {
        if (steps < 0)
            throw std::invalid_argument("EulerBatch::march: steps must be >= 0");
        batch->b->march(steps);
    });
}

int scg_batch_stream(const scg_batch * batch, void ** out)
{
    return scg::guarded([&] { *out = batch->b->get_stream(); });
}

} // extern "C"
