#pragma once

/*
 * Shared plumbing of the C-ABI library: status codes, the thread-local error
 * message, the CUDA error check and the kernel launch counter.
 */

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace scg
{

// Status codes returned by every extern "C" entry point.  They map onto the
// Python exception types the reference raises for the same conditions.
enum Status : int
{
    ST_OK = 0,
    ST_EINVAL = 1,   // std::invalid_argument -> ValueError
    ST_ERANGE = 2,   // std::out_of_range -> IndexError
    ST_ERUNTIME = 3, // std::runtime_error -> RuntimeError
    ST_ECUDA = 4,    // a CUDA runtime failure -> RuntimeError
    ST_ENOMEM = 5,   // device or host allocation failure -> MemoryError
};

struct CudaError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

void set_last_error(std::string const & msg);
std::string const & last_error();

// Count of kernels this library has launched (for the bench's gpu_launches).
extern std::atomic<int64_t> g_launches;
// Count of device allocations made through DevBuf (every device buffer of the
// cores, batches, 1D and spacetime solvers, and per-call scratch).
extern std::atomic<int64_t> g_device_allocs;

// The device address of the host range [p, p + nbytes) when the whole range
// lies inside one block from scg_host_alloc (page-locked and mapped into the
// device's address space), else nullptr.  Kernels may then load and store
// the range directly over the host link, with no staging copy.  With serial
// set it also receives the block's allocation number, which differs between
// two blocks that happen to reuse one address.
void * mapped_host(void const * p, size_t nbytes, uint64_t * serial = nullptr);

inline void cuda_check(cudaError_t rc, char const * what)
{
    if (rc != cudaSuccess)
    {
        throw CudaError(std::string(what) + ": " + cudaGetErrorString(rc));
    }
}

inline void launched(cudaStream_t s, char const * what)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cuda_check(cudaPeekAtLastError(), what);
    (void)s;
}

template <typename F>
int guarded(F && f)
{
    try
    {
        f();
        return ST_OK;
    }
    catch (std::invalid_argument const & e)
    {
        set_last_error(e.what());
        return ST_EINVAL;
    }
    catch (std::out_of_range const & e)
    {
        set_last_error(e.what());
        return ST_ERANGE;
    }
    catch (CudaError const & e)
    {
        set_last_error(e.what());
        return ST_ECUDA;
    }
    catch (std::bad_alloc const & e)
    {
        set_last_error(e.what());
        return ST_ENOMEM;
    }
    catch (std::exception const & e)
    {
        set_last_error(e.what());
        return ST_ERUNTIME;
    }
}

// Owning device buffer.
template <typename T>
struct DevBuf
{
    T * ptr = nullptr;
    size_t n = 0;

    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(DevBuf const &) = delete;
    DevBuf & operator=(DevBuf const &) = delete;
    DevBuf(DevBuf && o) noexcept : ptr(o.ptr), n(o.n) { o.ptr = nullptr; o.n = 0; }
    DevBuf & operator=(DevBuf && o) noexcept
    {
        if (this != &o)
        {
            release();
            ptr = o.ptr;
            n = o.n;
            o.ptr = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }

    void alloc(size_t count)
    {
        release();
        if (count == 0)
        {
            return;
        }
        cudaError_t rc = cudaMalloc(reinterpret_cast<void **>(&ptr), count * sizeof(T));
        if (rc != cudaSuccess)
        {
            ptr = nullptr;
            (void)cudaGetLastError();
            throw std::bad_alloc();
        }
        g_device_allocs.fetch_add(1, std::memory_order_relaxed);
        n = count;
    }
    void release()
    {
        if (ptr)
        {
            cudaFree(ptr);
        }
        ptr = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

} // namespace scg
