// Device memory, launch bookkeeping and error handling for the host side of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nsf
{
    struct Error : std::runtime_error
    {
        int status;
        Error(int s, const std::string & m) : std::runtime_error(m), status(s) {}
    };

    constexpr int ST_OK = 0, ST_INVALID = 1, ST_NONFINITE = 2, ST_MAXITER = 3, ST_BREAKDOWN = 4, ST_CUDA = 5,
                  ST_IO = 6, ST_NOTSUP = 7;

    inline void cudaCheck(cudaError_t e, const char * what)
    {
        if (e != cudaSuccess)
            throw Error(ST_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }

#define NSF_CUDA(x) ::nsf::cudaCheck((x), #x)

    // kernels issued by this library (eager launches plus captured kernels per graph replay)
    inline std::atomic<long long> & launchCounter()
    {
        static std::atomic<long long> c{0};
        return c;
    }

    template <typename T>
    class DevBuf
    {
        T * p_ = nullptr;
        size_t n_ = 0;

    public:
        DevBuf() = default;
        explicit DevBuf(size_t n) { alloc(n); }
        DevBuf(const DevBuf &) = delete;
        DevBuf & operator=(const DevBuf &) = delete;
        DevBuf(DevBuf && o) noexcept : p_(o.p_), n_(o.n_)
        {
            o.p_ = nullptr;
            o.n_ = 0;
        }
        DevBuf & operator=(DevBuf && o) noexcept
        {
            if (this != &o)
            {
                release();
                p_ = o.p_;
                n_ = o.n_;
                o.p_ = nullptr;
                o.n_ = 0;
            }
            return *this;
        }
        ~DevBuf() { release(); }

        void alloc(size_t n)
        {
            release();
            n_ = n;
            if (n > 0)
            {
                NSF_CUDA(cudaMalloc(&p_, n * sizeof(T)));
                NSF_CUDA(cudaMemset(p_, 0, n * sizeof(T)));
            }
        }

        void upload(const T * h, size_t n)
        {
            if (n != n_)
                alloc(n);
            if (n)
                NSF_CUDA(cudaMemcpy(p_, h, n * sizeof(T), cudaMemcpyHostToDevice));
        }

        void upload(const std::vector<T> & h) { upload(h.data(), h.size()); }

        std::vector<T> download() const
        {
            std::vector<T> h(n_);
            if (n_)
                NSF_CUDA(cudaMemcpy(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost));
            return h;
        }

        void release()
        {
            if (p_)
                cudaFree(p_);
            p_ = nullptr;
            n_ = 0;
        }

        T * get() const { return p_; }
        size_t size() const { return n_; }
    };

    // pinned host scratch for small device->host reads
    template <typename T>
    class PinnedBuf
    {
        T * p_ = nullptr;

    public:
        explicit PinnedBuf(size_t n = 1) { NSF_CUDA(cudaMallocHost(&p_, n * sizeof(T))); }
        PinnedBuf(const PinnedBuf &) = delete;
        PinnedBuf & operator=(const PinnedBuf &) = delete;
        ~PinnedBuf()
        {
            if (p_)
                cudaFreeHost(p_);
        }
        T * get() const { return p_; }
    };

    inline int blocksFor(long long threads)
    {
        long long b = (threads + 255) / 256;
        return (int)(b < 1 ? 1 : b);
    }

    // Kernels that end in a grid reduction cap their blocks at 4 per SM (grid-stride loops cover the
    // rest), which keeps the reduction at O(#SM) block sums; plain operators use blocksFor (one row
    // group per row: the rows' dependent loads overlap across the whole grid).
    inline int smCount()
    {
        static int n = 0;
        if (n == 0)
        {
            int dev = 0;
            cudaGetDevice(&dev);
            if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
                n = 152;
        }
        return n;
    }

    inline int cappedBlocks(long long threads)
    {
        const long long cap = 4ll * smCount();
        const long long b = (threads + 255) / 256;
        return (int)(b < 1 ? 1 : (b > cap ? cap : b));
    }

    // lanes per row from the average row length (power of two, 2..32)
    inline int lanesFor(long long nnz, long long rows)
    {
        const double avg = rows > 0 ? (double)nnz / (double)rows : 1.0;
        if (avg <= 3)
            return 2;
        if (avg <= 6)
            return 4;
        if (avg <= 12)
            return 8;
        if (avg <= 24)
            return 16;
        return 32;
    }

    inline void afterLaunch(const char * what)
    {
        launchCounter().fetch_add(1, std::memory_order_relaxed);
        cudaCheck(cudaGetLastError(), what);
    }

    // launch a kernel (through its pointer) with TPB threads per block
    template <typename... KArgs, typename... Args>
    inline void launchKernel(const char * name, void (*k)(KArgs...), int grid, cudaStream_t s, Args &&... a)
    {
        k<<<grid, TPB, 0, s>>>(std::forward<Args>(a)...);
        afterLaunch(name);
    }

    // the same with a 2-D / 3-D grid
    template <typename... KArgs, typename... Args>
    inline void launchKernel(const char * name, void (*k)(KArgs...), dim3 grid, cudaStream_t s, Args &&... a)
    {
        k<<<grid, TPB, 0, s>>>(std::forward<Args>(a)...);
        afterLaunch(name);
    }

#define NSF_LAUNCH(kernel, grid, stream, ...) ::nsf::launchKernel(#kernel, kernel, (grid), (stream), __VA_ARGS__)

    // launch with programmatic stream serialization: the kernel's blocks may start once every block
    // of the preceding kernel in the stream has run griddepcontrol.launch_dependents (or exited), and
    // must run griddepcontrol.wait before they touch anything that kernel writes.  Inside stream
    // capture this becomes a programmatic edge of the graph.
    template <typename... KArgs, typename... Args>
    inline void launchKernelPdl(const char * name, void (*k)(KArgs...), int grid, cudaStream_t s, const Args &... a)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(TPB);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaCheck(cudaLaunchKernelEx(&cfg, k, a...), name);
        launchCounter().fetch_add(1, std::memory_order_relaxed);
    }

#define NSF_LAUNCH_PDL(kernel, grid, stream, ...) \
    ::nsf::launchKernelPdl(#kernel, kernel, (grid), (stream), __VA_ARGS__)

    // launch `clusters` thread-block clusters of cs CTAs of `threads` threads each
    template <typename... KArgs, typename... Args>
    inline void launchClusters(void (*k)(KArgs...), int cs, int clusters, int threads, size_t smem, cudaStream_t s,
                               const Args &... a)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs * clusters);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaCheck(cudaLaunchKernelEx(&cfg, k, a...), "cluster launch");
        launchCounter().fetch_add(1, std::memory_order_relaxed);
    }

    // launch a one-cluster kernel: cs CTAs of `threads` threads forming one thread-block cluster
    template <typename... KArgs, typename... Args>
    inline void launchCluster(void (*k)(KArgs...), int cs, int threads, size_t smem, cudaStream_t s,
                              const Args &... a)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaCheck(cudaLaunchKernelEx(&cfg, k, a...), "cluster launch");
        launchCounter().fetch_add(1, std::memory_order_relaxed);
    }

    // launch a cooperative grid of `blocks` CTAs of 1024 threads, all co-resident
    template <typename... KArgs, typename... Args>
    inline void launchCooperative(void (*k)(KArgs...), int blocks, size_t smem, cudaStream_t s, const Args &... a)
    {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks);
        cfg.blockDim = dim3(1024);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cudaCheck(cudaLaunchKernelEx(&cfg, k, a...), "cooperative launch");
        launchCounter().fetch_add(1, std::memory_order_relaxed);
    }

    inline int envFlag(const char * name)
    {
        const char * v = std::getenv(name);
        return (v && *v && *v != '0') ? 1 : 0;
    }

    inline std::string envStr(const char * name, const char * dflt)
    {
        const char * v = std::getenv(name);
        return (v && *v) ? std::string(v) : std::string(dflt);
    }

// dispatch a lanes-per-row value to a template parameter
#define NSF_LANES(L, ...)                                                                                       \
    do                                                                                                          \
    {                                                                                                           \
        switch (L)                                                                                              \
        {                                                                                                       \
        case 2: { constexpr int LL = 2; __VA_ARGS__; } break;                                                   \
        case 4: { constexpr int LL = 4; __VA_ARGS__; } break;                                                   \
        case 8: { constexpr int LL = 8; __VA_ARGS__; } break;                                                   \
        case 16: { constexpr int LL = 16; __VA_ARGS__; } break;                                                 \
        default: { constexpr int LL = 32; __VA_ARGS__; } break;                                                 \
        }                                                                                                       \
    } while (0)
} // namespace nsf
