/*
 * scg_euler_totals_noalloc: the conservation totals of scg_euler_totals,
 * computed without allocating anything.
 *
 * Who needs it: a caller that has reserved its device memory up front and
 * must not allocate afterwards -- for example a serving loop that admits
 * solves under a fixed HBM budget and polls the totals of every resident
 * solve each step.  scg_euler_totals allocates a small per-call buffer of
 * per-block partial sums with cudaMalloc and releases it with cudaFree;
 * cudaMalloc can fail once the budget has been handed out, and cudaFree
 * synchronises the whole device, stalling every other solve's stream.
 *
 * How: the per-block partial sums live in one file-scope __device__ array,
 * g_totals_scratch, of fixed size (TOTALS_MAX_BLOCKS rows of 8 doubles plus
 * one result row: 131,136 bytes), which every GPU that loads this library
 * holds until the process exits.  Each block sums a fixed chunk of
 * TOTALS_CHUNK cells, so the entry point accepts at most
 * TOTALS_MAX_BLOCKS * TOTALS_CHUNK = 67,108,864 body cells and rejects larger
 * meshes.  Host code cannot use the array's name as a device address; the
 * address is looked up with cudaGetSymbolAddress once per device, on the
 * first call made with that device current.  Every call copies its result
 * to the host and waits for the core's stream, so no call may be made while
 * that stream is being captured.
 *
 * Every call on a device shares the one array and leaves its contents behind
 * for the next call.  Each call rewrites every partial row it later reads, so
 * nothing has to start at zero.  Two calls whose work overlaps on the GPU
 * (for example two cores on different streams calling at the same time)
 * race on the array and may return wrong totals: issue them one after the
 * other.
 */

#include "../../include/scg.h"
#include "common.hpp"
#include "reduce.cuh"
#include "euler_core.hpp"

#include <mutex>

namespace
{

constexpr int TOTALS_THREADS = 256;
constexpr int64_t TOTALS_CHUNK = 32768;     // body cells summed by one block
constexpr int TOTALS_MAX_BLOCKS = 2048;     // partial-sum rows in the scratch
constexpr int TOTALS_ROW = 8;               // doubles per row: neq <= 5 used, the rest padding
constexpr int MAX_DEVICES = 64;

// Shared by every call on a device; holds the last call's contents.
static __device__ __align__(256) double g_totals_scratch[(TOTALS_MAX_BLOCKS + 1) * TOTALS_ROW];

std::mutex g_setup_mutex;
double * g_scratch_addr[MAX_DEVICES] = {};

// Device address of g_totals_scratch for the current device (set-up on the
// first call per device).
double * scratch_for_current_device()
{
    int dev = 0;
    scg::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= MAX_DEVICES)
    {
        throw std::runtime_error("scg_euler_totals_noalloc: device ordinal out of range");
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev])
    {
        void * p = nullptr;
        scg::cuda_check(cudaGetSymbolAddress(&p, g_totals_scratch), "cudaGetSymbolAddress(g_totals_scratch)");
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    return g_scratch_addr[dev];
}

// Stage 1: block b sums cells [b * CHUNK, (b + 1) * CHUNK) of so0n * clvol
// (compensated per thread, warp shuffles across the block) and writes row b
// of the scratch.  Every row that stage 2 reads is rewritten here, so nothing
// needs clearing.
template <typename R>
__global__ void __launch_bounds__(TOTALS_THREADS) k_totals_part(R const * rec, int rs, int neq,
                                                                double const * clvol, int64_t ngst, int64_t ncell,
                                                                R const * comp, double * scratch)
{
    __shared__ double sh[TOTALS_THREADS / 32];
    double s[5] = {0, 0, 0, 0, 0};
    double c[5] = {0, 0, 0, 0, 0};
    int64_t const begin = static_cast<int64_t>(blockIdx.x) * TOTALS_CHUNK;
    int64_t const end = begin + TOTALS_CHUNK < ncell ? begin + TOTALS_CHUNK : ncell;
    for (int64_t icl = begin + threadIdx.x; icl < end; icl += TOTALS_THREADS)
    {
        int64_t const row = icl + ngst;
        double const v = clvol[row];
        for (int i = 0; i < neq; ++i)
        {
            double q = double(rec[row * rs + i]);
            if (comp)
            {
                q += double(comp[i * ncell + icl]); // the FP32 state's residual
            }
            double const y = q * v - c[i];
            double const t = s[i] + y;
            c[i] = (t - s[i]) - y;
            s[i] = t;
        }
    }
    for (int i = 0; i < neq; ++i)
    {
        double const r = scg::red::block_fold<scg::red::SUM, TOTALS_THREADS / 32>(s[i], sh);
        if (threadIdx.x == 0)
        {
            scratch[blockIdx.x * TOTALS_ROW + i] = r;
        }
    }
}

// Stage 2: one block sums the nblk partial rows (compensated, in block order)
// into the result row after the partial rows.
__global__ void k_totals_final(int nblk, int neq, double * scratch)
{
    if (threadIdx.x >= neq)
    {
        return;
    }
    int const i = threadIdx.x;
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nblk; ++b)
    {
        double const y = scratch[b * TOTALS_ROW + i] - c;
        double const t = s + y;
        c = (t - s) - y;
        s = t;
    }
    scratch[TOTALS_MAX_BLOCKS * TOTALS_ROW + i] = s;
}

} // namespace

extern "C"
{

int scg_euler_totals_noalloc(scg_euler * core, double * out)
{
    return scg::guarded([&] {
        if (!core || !core->c)
        {
            throw std::invalid_argument("scg_euler_totals_noalloc: null handle");
        }
        if (!out)
        {
            throw std::invalid_argument("scg_euler_totals_noalloc: null output");
        }
        scg::EulerCoreBase::StateView const v = core->c->state_view();
        int64_t const max_cells = static_cast<int64_t>(TOTALS_MAX_BLOCKS) * TOTALS_CHUNK;
        if (v.ncell > max_cells)
        {
            throw std::invalid_argument("scg_euler_totals_noalloc: the mesh has " + std::to_string(v.ncell) +
                                        " body cells; this entry point handles at most " +
                                        std::to_string(max_cells) + " (use scg_euler_totals)");
        }
        if (v.neq > 5)
        {
            throw std::invalid_argument("scg_euler_totals_noalloc: neq above 5");
        }
        double * scratch = scratch_for_current_device();
        int const nblk = static_cast<int>((v.ncell + TOTALS_CHUNK - 1) / TOTALS_CHUNK);
        if (nblk > 0)
        {
            if (v.fp32)
                k_totals_part<float><<<nblk, TOTALS_THREADS, 0, v.stream>>>(
                    static_cast<float const *>(v.rec), v.rec_stride, v.neq, v.clvol, v.ngstcell, v.ncell,
                    static_cast<float const *>(v.comp), scratch);
            else
                k_totals_part<double><<<nblk, TOTALS_THREADS, 0, v.stream>>>(
                    static_cast<double const *>(v.rec), v.rec_stride, v.neq, v.clvol, v.ngstcell, v.ncell,
                    static_cast<double const *>(v.comp), scratch);
            scg::launched(v.stream, "totals_noalloc_part");
        }
        k_totals_final<<<1, 32, 0, v.stream>>>(nblk, v.neq, scratch);
        scg::launched(v.stream, "totals_noalloc_final");
        scg::cuda_check(cudaMemcpyAsync(out, scratch + TOTALS_MAX_BLOCKS * TOTALS_ROW, sizeof(double) * v.neq,
                                        cudaMemcpyDeviceToHost, v.stream),
                        "D2H");
        scg::cuda_check(cudaStreamSynchronize(v.stream), "cudaStreamSynchronize");
    });
}

} // extern "C"
