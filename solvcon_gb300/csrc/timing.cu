/*
 * Timing and host-memory helpers of the C ABI: CUDA events recorded on a
 * solver's stream, page-locked host buffers for end-to-end copies, and a
 * probe of the FP64 and FP32 FMA rates of the device (the march's FP64 path
 * is bound by the FP64 pipe, so its roofline needs that peak).
 */

#include "../../include/scg.h"
#include "common.hpp"

#include <cstdint>
#include <map>
#include <mutex>
#include <vector>

namespace
{

// Blocks from scg_host_alloc: host address -> (bytes, device address).
struct HostBlock
{
    size_t nbytes;
    void * dev;
    uint64_t serial; // distinct for every allocation, reused addresses included
};
std::mutex g_blocks_mutex;
std::map<uintptr_t, HostBlock> g_blocks;
uint64_t g_block_serial = 0;

} // namespace

void * scg::mapped_host(void const * p, size_t nbytes, uint64_t * serial)
{
    uintptr_t const a = reinterpret_cast<uintptr_t>(p);
    std::lock_guard<std::mutex> lk(g_blocks_mutex);
    auto it = g_blocks.upper_bound(a);
    if (it == g_blocks.begin())
    {
        return nullptr;
    }
    --it;
    HostBlock const & b = it->second;
    uintptr_t const off = a - it->first;
    if (!b.dev || off > b.nbytes || nbytes > b.nbytes - off)
    {
        return nullptr;
    }
    if (serial)
    {
        *serial = b.serial;
    }
    return static_cast<char *>(b.dev) + off;
}

namespace
{

// A long chain of independent FMAs per thread; 8 accumulators keep the pipe
// full.  Each iteration performs 8 FMAs = 16 flops.
template <typename T>
__global__ void k_fma_probe(T * out, int iters, T a, T b)
{
    T x[8];
    for (int k = 0; k < 8; ++k)
    {
        x[k] = T(threadIdx.x + k) * T(1e-3);
    }
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            x[k] = fma(x[k], a, b);
        }
    }
    T s = T(0);
    for (int k = 0; k < 8; ++k)
    {
        s += x[k];
    }
    if (s == T(12345.678))
    {
        out[0] = s; // keeps the chain live; practically never taken
    }
}

template <typename T>
double probe(int iters)
{
    int dev = 0;
    scg::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    int nsm = 0;
    scg::cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "attr");
    scg::DevBuf<T> out(1);
    unsigned const blocks = static_cast<unsigned>(nsm * 8);
    unsigned const threads = 256;
    cudaEvent_t e0, e1;
    scg::cuda_check(cudaEventCreate(&e0), "event");
    scg::cuda_check(cudaEventCreate(&e1), "event");
    k_fma_probe<T><<<blocks, threads>>>(out.ptr, iters / 10, T(0.999999), T(1e-7));
    scg::launched(nullptr, "fma_probe");
    scg::cuda_check(cudaEventRecord(e0), "record");
    k_fma_probe<T><<<blocks, threads>>>(out.ptr, iters, T(0.999999), T(1e-7));
    scg::launched(nullptr, "fma_probe");
    scg::cuda_check(cudaEventRecord(e1), "record");
    scg::cuda_check(cudaEventSynchronize(e1), "sync");
    float ms = 0.f;
    scg::cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double const flops = double(blocks) * threads * double(iters) * 16.0;
    return flops / (double(ms) * 1e-3) / 1e12;
}

} // namespace

extern "C"
{

int scg_fma_peak(int precision, int iters, double * tflops)
{
    return scg::guarded([&] {
        if (iters <= 0)
        {
            throw std::invalid_argument("scg_fma_peak: iters must be > 0");
        }
        *tflops = precision == SCG_FP64 ? probe<double>(iters) : probe<float>(iters);
    });
}

int scg_host_alloc(int64_t nbytes, void ** out)
{
    return scg::guarded([&] {
        if (nbytes < 0 || !out)
        {
            throw std::invalid_argument("scg_host_alloc: negative size or null out");
        }
        void * p = nullptr;
        cudaError_t rc = cudaHostAlloc(&p, static_cast<size_t>(nbytes), cudaHostAllocMapped);
        if (rc != cudaSuccess)
        {
            (void)cudaGetLastError();
            throw std::bad_alloc();
        }
        void * d = nullptr;
        rc = cudaHostGetDevicePointer(&d, p, 0);
        if (rc != cudaSuccess)
        {
            (void)cudaGetLastError();
            d = nullptr;
        }
        {
            std::lock_guard<std::mutex> lk(g_blocks_mutex);
            g_blocks[reinterpret_cast<uintptr_t>(p)] = {static_cast<size_t>(nbytes), d, ++g_block_serial};
        }
        *out = p;
    });
}

int scg_host_free(void * p)
{
    return scg::guarded([&] {
        {
            std::lock_guard<std::mutex> lk(g_blocks_mutex);
            g_blocks.erase(reinterpret_cast<uintptr_t>(p));
        }
        scg::cuda_check(cudaFreeHost(p), "cudaFreeHost");
    });
}

int scg_event_create(void ** out)
{
    return scg::guarded([&] {
        cudaEvent_t e;
        scg::cuda_check(cudaEventCreate(&e), "cudaEventCreate");
        *out = e;
    });
}

int scg_event_destroy(void * ev)
{
    return scg::guarded([&] { scg::cuda_check(cudaEventDestroy(static_cast<cudaEvent_t>(ev)), "destroy"); });
}

int scg_event_record(void * ev, void * stream)
{
    return scg::guarded([&] {
        scg::cuda_check(cudaEventRecord(static_cast<cudaEvent_t>(ev), static_cast<cudaStream_t>(stream)), "record");
    });
}

int scg_event_elapsed(void * ev0, void * ev1, double * ms)
{
    return scg::guarded([&] {
        scg::cuda_check(cudaEventSynchronize(static_cast<cudaEvent_t>(ev1)), "sync");
        float f = 0.f;
        scg::cuda_check(cudaEventElapsedTime(&f, static_cast<cudaEvent_t>(ev0), static_cast<cudaEvent_t>(ev1)),
                        "elapsed");
        *ms = f;
    });
}

int scg_device_sync(void)
{
    return scg::guarded([&] { scg::cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); });
}

} // extern "C"
