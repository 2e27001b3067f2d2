// sm_103a kernels of the Chorin path.  All sparse work is memory/latency bound (no tensor-core
// shape), so the kernels are built around:
//   * SELL-C-sigma (C = 32) for the operators applied once per step (FastConvection, D, G, the
//     library SpMV and the adjoint's transposes): one thread per row, coalesced slice loads and
//     one FMA per entry, because FP64 issues at 1/64 of the FP32 rate on this GPU and the
//     product-plus-sum of a CSR-stream kernel made FP64 SpMV issue-bound (the CSR-stream kernels
//     remain for reference);
//   * row groups of L lanes (L = 2..32) per CSR row for the sweeps and the solver SpMVs;
//   * grids capped at a few blocks per SM (grid-stride loops), and one deterministic reduction per
//     producing kernel: every block writes its block sum, the last block to finish (atomic ticket)
//     sums them in a fixed order into a per-kernel scalar - same bits on every run, O(blocks) work;
//   * device-resident solver scalars and early-exit flags, so solver loops need no host sync and
//     can run inside CUDA graphs (conditional while nodes end the loop on the device);
//   * the iteration counter advanced by that same last block of the last kernel of an iteration,
//     after every block has read it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

namespace nsf
{
    constexpr int TPB = 256;      // threads per block of every kernel here
    constexpr int MAXCH = 2;      // planar channels handled by one solver instance
    constexpr int MAXCOLORS = 64; // colors of a sweep system (smallest-last greedy gives < 10 here)
    constexpr int STREAM_NNZ = 2048; // nnz per block of the CSR-stream kernel (8 per thread)
    constexpr unsigned FULL = 0xffffffffu;

    // the device side of programmatic dependent launch (PTX griddepcontrol, sm_90 and later): let the
    // next kernel of the stream start its blocks / wait until the preceding kernel has completed and
    // its memory operations are visible.  Both are no-ops for a kernel launched without the attribute.
    __device__ __forceinline__ void griddepLaunchDependents()
    {
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    }
    __device__ __forceinline__ void griddepWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

    template <int L>
    struct Group
    {
        int lane, gid, ngroups;
        unsigned mask;

        __device__ __forceinline__ Group() : Group((int)blockIdx.x, (int)gridDim.x) {}

        // block `blk` of `nblk` (batched launches decode their own block index)
        __device__ __forceinline__ Group(int blk, int nblk)
        {
            const int t = blk * blockDim.x + threadIdx.x;
            lane = threadIdx.x & (L - 1);
            gid = t / L;
            ngroups = (nblk * blockDim.x) / L;
            const int w = (threadIdx.x & 31) / L;
            mask = (L == 32) ? FULL : (((1u << L) - 1u) << (w * L));
        }

        template <typename T>
        __device__ __forceinline__ T sum(T v) const
        {
#pragma unroll
            for (int o = L / 2; o > 0; o >>= 1)
                v += __shfl_down_sync(mask, v, o, L);
            return v; // complete in lane 0
        }
    };

    template <typename T>
    __device__ __forceinline__ T ldg(const T * p)
    {
        return __ldg(p);
    }

    // ------------------------------------------------------------------ deterministic reductions

    // Where the totals of a grid reduction go (null entries are dropped).
    template <int K>
    struct Outs
    {
        double * p[K];
    };

    struct NoEpi
    {
        __device__ void operator()() const {}
    };

    // Grid-wide sum of K per-thread values, accumulated in TA (the solve precision: FP64 work runs at
    // ~1/64 of the FP32 rate on this GPU, so an FP32 solve keeps its reductions in FP32).  Block
    // sums go to scratch[k * gridDim.x + block] (scratch holds >= K * gridDim.x values of TA); the
    // last block to take a ticket sums them in a fixed order, writes out.p[k] (as FP64), runs
    // epi() on one thread -- the once-per-grid scalar work that depends on the totals -- resets
    // the ticket and, if tick != null, advances *tick.  Call at most once per kernel, from every
    // thread.
    template <typename TA, int K, typename Epi = NoEpi>
    __device__ __forceinline__ void gridSum(const TA (&v)[K], double * scratchD, const Outs<K> & out,
                                            unsigned * ticket, int * tick, Epi epi = Epi())
    {
        TA * scratch = reinterpret_cast<TA *>(scratchD);
        __shared__ TA sm[TPB / 32][K];
        __shared__ bool lastBlock;
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int k = 0; k < K; k++)
        {
            TA s = v[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0)
                sm[warp][k] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
#pragma unroll
            for (int k = 0; k < K; k++)
            {
                TA s = 0;
                for (int w = 0; w < TPB / 32; w++)
                    s += sm[w][k];
                scratch[k * gridDim.x + blockIdx.x] = s;
            }
            __threadfence();
            const unsigned prev = atomicAdd(ticket, 1u);
            lastBlock = (prev == gridDim.x - 1);
        }
        __syncthreads();
        if (!lastBlock)
            return;
        __threadfence();
#pragma unroll
        for (int k = 0; k < K; k++)
        {
            TA s = 0;
            for (int i = threadIdx.x; i < (int)gridDim.x; i += TPB)
                s += __ldcg(scratch + k * gridDim.x + i);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0)
                sm[warp][k] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
#pragma unroll
            for (int k = 0; k < K; k++)
            {
                TA s = 0;
                for (int w = 0; w < TPB / 32; w++)
                    s += sm[w][k];
                if (out.p[k])
                    *out.p[k] = (double)s;
            }
            epi();
            *ticket = 0;
            if (tick)
                *tick += 1;
            __threadfence();
        }
    }

    // ------------------------------------------------------------------ plain operators

    // y = alpha * A x + beta * y   (beta == 0: y is not read)
    template <typename TM, typename TX, typename TY, typename TA, int L>
    __global__ void __launch_bounds__(TPB) kSpmv(int rows, const int * __restrict__ rs, const int * __restrict__ ci,
                                                  const TM * __restrict__ v, const TX * __restrict__ x,
                                                  TY * __restrict__ y, double alpha, double beta)
    {
        Group<L> g;
        for (int r = g.gid; r < rows; r += g.ngroups)
        {
            const int b = ldg(rs + r), e = ldg(rs + r + 1);
            TA s = 0;
            for (int j = b + g.lane; j < e; j += L)
                s += (TA)ldg(v + j) * (TA)ldg(x + ldg(ci + j));
            s = g.sum(s);
            if (g.lane == 0)
            {
                double out = alpha * (double)s;
                if (beta != 0.0)
                    out += beta * (double)y[r];
                y[r] = (TY)out;
            }
        }
    }

    // planar multi-RHS: Y[c * ldy + r] = sum_j A[r, j] X[c * ldx + j]
    template <typename TM, typename TX, typename TY, typename TA, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kSpmm(int rows, const int * __restrict__ rs, const int * __restrict__ ci,
                                                  const TM * __restrict__ v, const TX * __restrict__ X, int ldx,
                                                  TY * __restrict__ Y, int ldy)
    {
        Group<L> g;
        for (int r = g.gid; r < rows; r += g.ngroups)
        {
            const int b = ldg(rs + r), e = ldg(rs + r + 1);
            TA s[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                s[c] = 0;
            for (int j = b + g.lane; j < e; j += L)
            {
                const TA a = (TA)ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    s[c] += a * (TA)ldg(X + (size_t)c * ldx + col);
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const TA t = g.sum(s[c]);
                if (g.lane == 0)
                    Y[(size_t)c * ldy + r] = (TY)t;
            }
        }
    }

    // A[k] = nu * K[k] + sum_j I[k, j] u[j]   (linearised advection + diffusion), row groups
    template <typename TI, typename TU, typename TK, typename TA, int L>
    __global__ void __launch_bounds__(TPB) kFastConv(int rows, const int * __restrict__ rs, const int * __restrict__ ci,
                                                      const TI * __restrict__ iv, const TU * __restrict__ u,
                                                      const TK * __restrict__ k, TA nu, TK * __restrict__ a)
    {
        Group<L> g;
        for (int r = g.gid; r < rows; r += g.ngroups)
        {
            const int b = ldg(rs + r), e = ldg(rs + r + 1);
            TA s = 0;
            for (int j = b + g.lane; j < e; j += L)
                s += (TA)ldg(iv + j) * (TA)ldg(u + ldg(ci + j));
            s = g.sum(s);
            if (g.lane == 0)
                a[r] = (TK)(nu * (TA)ldg(k + r) + s);
        }
    }

    // CSR-stream form of the same operator.  Block b owns rows [rb[b], rb[b+1]) whose entries form
    // one contiguous chunk of at most STREAM_NNZ nonzeros (rows longer than that are never produced
    // by the row blocking).  Stage 1 streams values and columns with coalesced loads, 8 independent
    // loads and gathers per thread, products into shared memory; stage 2 sums each row in order.
    template <typename TI, typename TU, typename TK, typename TA>
    __global__ void __launch_bounds__(TPB) kFastConvStream(const int * __restrict__ rb, const int * __restrict__ rs,
                                                            const int * __restrict__ ci, const TI * __restrict__ iv,
                                                            const TU * __restrict__ u, const TK * __restrict__ k,
                                                            TA nu, TK * __restrict__ a)
    {
        __shared__ TA prod[STREAM_NNZ];
        const int r0 = ldg(rb + blockIdx.x), r1 = ldg(rb + blockIdx.x + 1);
        const int s = ldg(rs + r0), e = ldg(rs + r1);
        const int cnt = e - s;
        TI vals[STREAM_NNZ / TPB];
        int cols[STREAM_NNZ / TPB];
#pragma unroll
        for (int q = 0; q < STREAM_NNZ / TPB; q++)
        {
            const int j = threadIdx.x + q * TPB;
            vals[q] = j < cnt ? ldg(iv + s + j) : (TI)0;
            cols[q] = j < cnt ? ldg(ci + s + j) : 0;
        }
#pragma unroll
        for (int q = 0; q < STREAM_NNZ / TPB; q++)
        {
            const int j = threadIdx.x + q * TPB;
            if (j < cnt)
                prod[j] = (TA)vals[q] * (TA)ldg(u + cols[q]);
        }
        __syncthreads();
        for (int r = r0 + threadIdx.x; r < r1; r += TPB)
        {
            const int b = ldg(rs + r) - s, en = ldg(rs + r + 1) - s;
            TA acc = 0;
            for (int j = b; j < en; j++)
                acc += prod[j];
            a[r] = (TK)(nu * (TA)ldg(k + r) + acc);
        }
    }

    // y = alpha A x + beta y (beta == 0: y is not read), CSR-stream: block b covers the rows
    // [rb[b], rb[b+1]) whose entries fit in STREAM_NNZ.  Stage 1: coalesced loads of values and
    // columns, STREAM_NNZ / TPB independent loads and gathers per thread, products (rounded) into
    // shared memory; stage 2: one thread per row sums its products in entry order.
    template <typename TM, typename TX, typename TY, typename TA>
    __global__ void __launch_bounds__(TPB) kSpmvStream(const int * __restrict__ rb, const int * __restrict__ rs,
                                                        const int * __restrict__ ci, const TM * __restrict__ v,
                                                        const TX * __restrict__ x, TY * __restrict__ y, double alpha,
                                                        double beta)
    {
        __shared__ TA prod[STREAM_NNZ];
        const int r0 = ldg(rb + blockIdx.x), r1 = ldg(rb + blockIdx.x + 1);
        const int s = ldg(rs + r0), e = ldg(rs + r1);
        const int cnt = e - s;
        TM vals[STREAM_NNZ / TPB];
        int cols[STREAM_NNZ / TPB];
#pragma unroll
        for (int q = 0; q < STREAM_NNZ / TPB; q++)
        {
            const int j = threadIdx.x + q * TPB;
            vals[q] = j < cnt ? ldg(v + s + j) : (TM)0;
            cols[q] = j < cnt ? ldg(ci + s + j) : 0;
        }
#pragma unroll
        for (int q = 0; q < STREAM_NNZ / TPB; q++)
        {
            const int j = threadIdx.x + q * TPB;
            if (j < cnt)
                prod[j] = (TA)vals[q] * (TA)ldg(x + cols[q]);
        }
        __syncthreads();
        for (int r = r0 + threadIdx.x; r < r1; r += TPB)
        {
            const int b = ldg(rs + r) - s, en = ldg(rs + r + 1) - s;
            TA acc = 0;
            for (int j = b; j < en; j++)
                acc += prod[j];
            double out = alpha * (double)acc;
            if (beta != 0.0)
                out += beta * (double)y[r];
            y[r] = (TY)out;
        }
    }

    // ------------------------------------------------------------------ SELL-C-sigma operators
    // SELL-C-sigma with C = 32: the rows, sorted by length inside windows of sigma rows, form slices
    // of 32; slice s stores its rows column-major (entry k of lane l at ss[s] + 32 k + l), padded to
    // the slice's longest row with zero values.  One warp per slice, one thread per row: every
    // value and column load of a warp is one coalesced 32-entry segment, and each stored entry
    // costs one FMA.  (FP64 runs at 1/64 of the FP32 rate on this GPU: the CSR-stream kernels
    // spend a multiply and an add per entry and become FP64-issue-bound.)  Results go to the
    // original row perm[row].  e - b is a multiple of 32, so the unrolled loop is warp-uniform.
    constexpr int SELL_C = 32;

    // Groups of 8 slice columns with predicated loads: all loads of a short row (a 7-point stencil,
    // say) are in flight together, then the gathers, then the FMAs.
    template <typename TM, typename TX, typename TA>
    __device__ __forceinline__ TA sellRow(int b, int e, int lane, const int * __restrict__ ci,
                                          const TM * __restrict__ v, const TX * __restrict__ x)
    {
        constexpr int U = 8;
        TA acc = 0;
        const int w = (e - b) / SELL_C;
        for (int k = 0; k < w; k += U)
        {
            int c[U];
            TM a[U];
#pragma unroll
            for (int t = 0; t < U; t++)
            {
                const int j = b + (k + t) * SELL_C + lane;
                const bool ok = k + t < w;
                c[t] = ok ? ldg(ci + j) : 0;
                a[t] = ok ? ldg(v + j) : (TM)0;
            }
            TX g[U];
#pragma unroll
            for (int t = 0; t < U; t++)
                g[t] = k + t < w ? ldg(x + c[t]) : (TX)0;
#pragma unroll
            for (int t = 0; t < U; t++)
                if (k + t < w)
                    acc += (TA)a[t] * (TA)g[t];
        }
        return acc;
    }

    // y[perm[row]] = alpha * (A x)[row] + beta * y[perm[row]]   (beta == 0: y is not read)
    template <typename TM, typename TX, typename TY, typename TA>
    __device__ __forceinline__ void spmvSellSlice(int slice, int rows, int nSlices, const int * __restrict__ ss,
                                                  const int * __restrict__ perm, const int * __restrict__ ci,
                                                  const TM * __restrict__ v, const TX * __restrict__ x,
                                                  TY * __restrict__ y, double alpha, double beta)
    {
        if (slice >= nSlices)
            return; // whole warps
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int r = row < rows ? ldg(perm + row) : 0; // issued before the row's loads
        const TA acc = sellRow<TM, TX, TA>(ldg(ss + slice), ldg(ss + slice + 1), lane, ci, v, x);
        if (row < rows)
        {
            double out = alpha * (double)acc;
            if (beta != 0.0)
                out += beta * (double)y[r];
            y[r] = (TY)out;
        }
    }

    template <typename TM, typename TX, typename TY, typename TA>
    __global__ void __launch_bounds__(TPB) kSpmvSell(int rows, int nSlices, const int * __restrict__ ss,
                                                      const int * __restrict__ perm, const int * __restrict__ ci,
                                                      const TM * __restrict__ v, const TX * __restrict__ x,
                                                      TY * __restrict__ y, double alpha, double beta)
    {
        const int slice = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        spmvSellSlice<TM, TX, TY, TA>(slice, rows, nSlices, ss, perm, ci, v, x, y, alpha, beta);
    }

    // A[perm[row]] = nu K[perm[row]] + (I u)[row]   (FastConvection with the nu K add fused)
    template <typename TI, typename TU, typename TK, typename TA>
    __global__ void __launch_bounds__(TPB) kFastConvSell(int rows, int nSlices, const int * __restrict__ ss,
                                                          const int * __restrict__ perm, const int * __restrict__ ci,
                                                          const TI * __restrict__ iv, const TU * __restrict__ u,
                                                          const TK * __restrict__ k, TA nu, TK * __restrict__ a)
    {
        const int slice = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        if (slice >= nSlices)
            return;
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int r = row < rows ? ldg(perm + row) : 0;
        const TA kr = row < rows ? (TA)ldg(k + r) : (TA)0;
        const TA acc = sellRow<TI, TU, TA>(ldg(ss + slice), ldg(ss + slice + 1), lane, ci, iv, u);
        if (row < rows)
            a[r] = (TK)(nu * kr + acc);
    }

    // SELL values from CSR values after an update: sv[i] = src[i] >= 0 ? cv[src[i]] : 0
    template <typename T>
    __global__ void __launch_bounds__(TPB) kSellGather(long long stored, const int * __restrict__ src,
                                                        const T * __restrict__ cv, T * __restrict__ sv)
    {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < stored;
             i += (long long)gridDim.x * blockDim.x)
        {
            const int s = src[i];
            sv[i] = s >= 0 ? cv[s] : (T)0;
        }
    }

    // u <- Dirichlet value on boundary rows, u - tau * acc elsewhere (2 planar channels)
    template <typename TA>
    __device__ __forceinline__ void updateVelocityRow(int i, int n, double * __restrict__ u, const TA * __restrict__ acc,
                                                      double tau, const unsigned char * __restrict__ isDir,
                                                      const double * __restrict__ dirVal)
    {
        if (isDir[i])
        {
            u[i] = dirVal[i];
            u[i + n] = 0.0;
        }
        else
        {
            u[i] -= tau * (double)acc[i];
            u[i + n] -= tau * (double)acc[i + n];
        }
    }

    template <typename TA>
    __global__ void __launch_bounds__(TPB) kUpdateVelocity(int n, double * __restrict__ u, const TA * __restrict__ acc,
                                                            double tau, const unsigned char * __restrict__ isDir,
                                                            const double * __restrict__ dirVal)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            updateVelocityRow<TA>(i, n, u, acc, tau, isDir, dirVal);
    }

    // ------------------------------------------------------------------ Chebyshev (mass matrix)
    // Chebyshev iteration with the Jacobi preconditioner for an SPD matrix whose D^-1 A spectrum
    // lies in known bounds (Saad, Iterative Methods, Alg. 12.1): no dot products, one fused kernel
    // per iteration over the SELL copy.  NCH planar channels of n rows each, x starts at 0.
    //   start:  r = b,  d = D^-1 b / theta
    //   step k: q = A d;  x += d;  r -= q;  d' = c1 d + c2 D^-1 r   (c1, c2 from the bounds and k)
    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebStart(int n, const double * __restrict__ b, const double * __restrict__ invD,
                                                       double invTheta, double * __restrict__ r, double * __restrict__ d)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const double id = invD[i];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double bi = b[(size_t)c * n + i];
                r[(size_t)c * n + i] = bi;
                d[(size_t)c * n + i] = bi * id * invTheta;
            }
        }
    }

    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebStep(int n, int nSlices, const int * __restrict__ ss,
                                                      const int * __restrict__ perm, const int * __restrict__ ci,
                                                      const double * __restrict__ v, const double * __restrict__ invD,
                                                      const double * __restrict__ d, double * __restrict__ dn,
                                                      double * __restrict__ x, double * __restrict__ r, double c1,
                                                      double c2, const int * kdev, int it)
    {
        const int slice = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        if (slice >= nSlices || (kdev && it >= *kdev))
            return;
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int b0 = ldg(ss + slice), e0 = ldg(ss + slice + 1);
        // q = A d for every channel; each column / value load serves all channels
        double q[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            q[c] = 0.0;
        const int w = (e0 - b0) / SELL_C;
        for (int k = 0; k < w; k += 4)
        {
            int cc[4];
            double a[4];
#pragma unroll
            for (int t = 0; t < 4; t++)
            {
                const bool ok = k + t < w;
                const int j = b0 + (k + t) * SELL_C + lane;
                cc[t] = ok ? ldg(ci + j) : 0;
                a[t] = ok ? ldg(v + j) : 0.0;
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                double g[4];
#pragma unroll
                for (int t = 0; t < 4; t++)
                    g[t] = k + t < w ? ldg(d + (size_t)c * n + cc[t]) : 0.0;
#pragma unroll
                for (int t = 0; t < 4; t++)
                    if (k + t < w)
                        q[c] += a[t] * g[t];
            }
        }
        if (row >= n)
            return;
        const int i = ldg(perm + row);
        const double id = ldg(invD + i);
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            const size_t o = (size_t)c * n + i;
            const double di = d[o];
            x[o] += di;
            const double ri = r[o] - q[c];
            r[o] = ri;
            dn[o] = c1 * di + c2 * ri * id;
        }
    }

    // ------------------------------------------------------------------ double-float Chebyshev
    // A double-float is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi) / 2): about 48
    // significant bits computed on the FP32 pipes, which run at 64x the FP64 rate on this GPU.  The
    // operations are the error-free transformations of Dekker ("A floating-point technique for
    // extending the available precision", 1971) and Knuth (TAOCP vol. 2, TwoSum); fmaf gives the
    // exact product error.  Vectors and matrix values are float2 = (hi, lo).
    __device__ __forceinline__ float2 dfTwoSum(float a, float b)
    {
        const float s = a + b, bb = s - a;
        return make_float2(s, (a - (s - bb)) + (b - bb));
    }

    __device__ __forceinline__ float2 dfFastTwoSum(float a, float b) // needs |a| >= |b| or a == 0
    {
        const float s = a + b;
        return make_float2(s, b - (s - a));
    }

    __device__ __forceinline__ float2 dfAdd(float2 a, float2 b)
    {
        const float2 s = dfTwoSum(a.x, b.x);
        return dfFastTwoSum(s.x, s.y + (a.y + b.y));
    }

    __device__ __forceinline__ float2 dfMul(float2 a, float2 b)
    {
        const float p = a.x * b.x;
        float e = fmaf(a.x, b.x, -p);
        e = fmaf(a.x, b.y, fmaf(a.y, b.x, e));
        return dfFastTwoSum(p, e);
    }

    __device__ __forceinline__ float2 dfNeg(float2 a) { return make_float2(-a.x, -a.y); }

    // Dot products in double-float, Ogita-Rump-Oishi's Dot2 ("Accurate sum and dot product", SIAM J.
    // Sci. Comput. 26, 2005): the running sum keeps s = acc.x as the FP32 sum of the products' high
    // parts, every rounding error of those additions (TwoSum) and of the products (an exact FMA
    // residual, plus the cross terms of double-float operands) is added into acc.y, and one
    // FastTwoSum normalises the pair at the end (dfDotEnd).  The result is as accurate as a dot
    // product computed in twice the FP32 precision, at 12 instead of 18 operations per term.
    __device__ __forceinline__ float2 dfDotAdd(float2 acc, float2 a, float2 g)
    {
        const float p = a.x * g.x;
        const float e = fmaf(a.x, g.y, fmaf(a.y, g.x, fmaf(a.x, g.x, -p)));
        const float s = acc.x + p, bb = s - acc.x;
        return make_float2(s, acc.y + (((acc.x - (s - bb)) + (p - bb)) + e));
    }

    // the same with a single-float a (FastConvection's FP32 integration values)
    __device__ __forceinline__ float2 dfDotAdd(float2 acc, float a, float2 g)
    {
        const float p = a * g.x;
        const float e = fmaf(a, g.y, fmaf(a, g.x, -p));
        const float s = acc.x + p, bb = s - acc.x;
        return make_float2(s, acc.y + (((acc.x - (s - bb)) + (p - bb)) + e));
    }

    __device__ __forceinline__ float2 dfDotEnd(float2 acc) { return dfFastTwoSum(acc.x, acc.y); }

    __device__ __forceinline__ float2 dfFromDouble(double v)
    {
        const float hi = (float)v;
        return make_float2(hi, (float)(v - (double)hi));
    }

    __device__ __forceinline__ double dfToDouble(float2 a) { return (double)a.x + (double)a.y; }

    // the double-float Chebyshev start: r = b, d = D^-1 b / theta, x = 0 (b and D^-1 from FP64);
    // bOut (may be null) keeps b as double-floats for the check after the solve
    template <int NCH>
    __device__ __forceinline__ void chebStartDfRow(int i, int n, const double * __restrict__ b,
                                                   const float2 * __restrict__ invD, float2 invTheta,
                                                   float2 * __restrict__ r, float2 * __restrict__ d,
                                                   float2 * __restrict__ x, float2 * __restrict__ bOut = nullptr)
    {
        const float2 id = invD[i];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            const size_t o = (size_t)c * n + i;
            const float2 bi = dfFromDouble(b[o]);
            r[o] = bi;
            d[o] = dfMul(dfMul(bi, id), invTheta);
            x[o] = make_float2(0.f, 0.f);
            if (bOut)
                bOut[o] = bi;
        }
    }

    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebStartDf(int n, const double * __restrict__ b,
                                                         const float2 * __restrict__ invD, float2 invTheta,
                                                         float2 * __restrict__ r, float2 * __restrict__ d,
                                                         float2 * __restrict__ x, float2 * __restrict__ bOut)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            chebStartDfRow<NCH>(i, n, b, invD, invTheta, r, d, x, bOut);
    }

    // kChebStep in double-float arithmetic: q = A d; x += d; r -= q; d' = c1 d + c2 D^-1 r
    template <int NCH>
    __device__ __forceinline__ void chebStepDfSlice(int slice, int n, int nSlices, const int * __restrict__ ss,
                                                    const int * __restrict__ perm, const int * __restrict__ ci,
                                                    const float2 * __restrict__ v, const float2 * __restrict__ invD,
                                                    const float2 * __restrict__ d, float2 * __restrict__ dn,
                                                    float2 * __restrict__ x, float2 * __restrict__ r, float2 c1,
                                                    float2 c2)
    {
        if (slice >= nSlices)
            return;
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int b0 = ldg(ss + slice), e0 = ldg(ss + slice + 1);
        float2 q[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            q[c] = make_float2(0.f, 0.f);
        const int w = (e0 - b0) / SELL_C;
        for (int k = 0; k < w; k += 4)
        {
            int cc[4];
            float2 a[4];
#pragma unroll
            for (int t = 0; t < 4; t++)
            {
                const bool ok = k + t < w;
                const int j = b0 + (k + t) * SELL_C + lane;
                cc[t] = ok ? ldg(ci + j) : 0;
                a[t] = ok ? ldg(v + j) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                float2 g[4];
#pragma unroll
                for (int t = 0; t < 4; t++)
                    g[t] = k + t < w ? ldg(d + (size_t)c * n + cc[t]) : make_float2(0.f, 0.f);
#pragma unroll
                for (int t = 0; t < 4; t++)
                    if (k + t < w)
                        q[c] = dfDotAdd(q[c], a[t], g[t]);
            }
        }
        if (row >= n)
            return;
        const int i = ldg(perm + row);
        const float2 id = ldg(invD + i);
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            const size_t o = (size_t)c * n + i;
            const float2 di = d[o];
            x[o] = dfAdd(x[o], di);
            const float2 ri = dfAdd(r[o], dfNeg(dfDotEnd(q[c])));
            r[o] = ri;
            dn[o] = dfAdd(dfMul(c1, di), dfMul(c2, dfMul(ri, id)));
        }
    }

    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebStepDf(int n, int nSlices, const int * __restrict__ ss,
                                                        const int * __restrict__ perm, const int * __restrict__ ci,
                                                        const float2 * __restrict__ v, const float2 * __restrict__ invD,
                                                        const float2 * __restrict__ d, float2 * __restrict__ dn,
                                                        float2 * __restrict__ x, float2 * __restrict__ r, float2 c1,
                                                        float2 c2, const int * kdev, int it)
    {
        const int slice = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        if (kdev && it >= *kdev)
            return;
        chebStepDfSlice<NCH>(slice, n, nSlices, ss, perm, ci, v, invD, d, dn, x, r, c1, c2);
    }

    // The same step with one warp per slice and channel (warps 2s and 2s + 1 take the two channels of
    // slice s, so they read the slice's entries through the same L1): twice the warps in flight for
    // a latency-bound step; per channel the arithmetic and its order are kChebStepDf's.
    // Launched with programmatic stream serialization (NSF_LAUNCH_PDL): each block lets the next
    // iteration's kernel start at once, and loads what no kernel of the solve writes (the slice
    // bounds, the first four stored entries of its row, perm and D^-1) before griddepcontrol.wait, so
    // the next iteration's blocks fill the SMs that this one's last wave leaves idle.  Everything
    // the previous iteration writes (d, x, r) is read after the wait with plain (coherent) loads,
    // and nothing is written before it.  An iteration past a warm solve's count waits and exits
    // without loading anything.
    __global__ void __launch_bounds__(TPB) kChebStepDfSplit(int n, int nSlices, const int * __restrict__ ss,
                                                             const int * __restrict__ perm, const int * __restrict__ ci,
                                                             const float2 * __restrict__ v, const float2 * __restrict__ invD,
                                                             const float2 * d, float2 * dn, float2 * x, float2 * r,
                                                             float2 c1, float2 c2, const int * kdev, int it)
    {
        griddepLaunchDependents();
        // the warm count is written before the solve's first iteration kernel, by a kernel that
        // completed before that one started: it may be read before the wait
        if (kdev && it >= *(volatile const int *)kdev)
        {
            griddepWait();
            return;
        }
        const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        const int slice = w >> 1;
        if (slice >= nSlices)
            return;
        const size_t o = (size_t)(w & 1) * n;
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int b0 = ldg(ss + slice), e0 = ldg(ss + slice + 1);
        const int wd = (e0 - b0) / SELL_C;
        int cc[4];
        float2 a[4];
#pragma unroll
        for (int t = 0; t < 4; t++)
        {
            const bool ok = t < wd;
            const int j = b0 + t * SELL_C + lane;
            cc[t] = ok ? ldg(ci + j) : 0;
            a[t] = ok ? ldg(v + j) : make_float2(0.f, 0.f);
        }
        const bool own = row < n;
        const int i = own ? ldg(perm + row) : 0;
        const float2 id = own ? ldg(invD + i) : make_float2(0.f, 0.f);
        griddepWait();
        const float2 * dc = d + o;
        float2 q = make_float2(0.f, 0.f);
        for (int k = 0; k < wd; k += 4)
        {
            if (k > 0)
            {
#pragma unroll
                for (int t = 0; t < 4; t++)
                {
                    const bool ok = k + t < wd;
                    const int j = b0 + (k + t) * SELL_C + lane;
                    cc[t] = ok ? ldg(ci + j) : 0;
                    a[t] = ok ? ldg(v + j) : make_float2(0.f, 0.f);
                }
            }
            float2 g[4];
#pragma unroll
            for (int t = 0; t < 4; t++)
                g[t] = k + t < wd ? dc[cc[t]] : make_float2(0.f, 0.f);
#pragma unroll
            for (int t = 0; t < 4; t++)
                if (k + t < wd)
                    q = dfDotAdd(q, a[t], g[t]);
        }
        if (!own)
            return;
        const size_t oi = o + i;
        const float2 di = d[oi];
        x[oi] = dfAdd(x[oi], di);
        const float2 ri = dfAdd(r[oi], dfNeg(dfDotEnd(q)));
        r[oi] = ri;
        dn[oi] = dfAdd(dfMul(c1, di), dfMul(c2, dfMul(ri, id)));
    }

    // y = (hi, lo) split of an FP64 vector
    __global__ void __launch_bounds__(TPB) kSplitDf(long long n, const double * __restrict__ x, float2 * __restrict__ y)
    {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            y[i] = dfFromDouble(x[i]);
    }

    // FastConvection in double-float: A[k] = nu K[k] + sum_j I[k, j] u[j] with FP32 values of I (the
    // product I_kj u_j of a float and a double-float is formed exactly up to the last bits), u, K, A
    // and the sums as double-floats.  Same SELL layout and predicated 8-wide load groups as
    // kFastConvSell.
    __device__ __forceinline__ void fastConvSellDfSlice(int slice, int rows, int nSlices, const int * __restrict__ ss,
                                                        const int * __restrict__ perm, const int * __restrict__ ci,
                                                        const float * __restrict__ iv, const float2 * __restrict__ u,
                                                        const float2 * __restrict__ k, float2 nu,
                                                        float2 * __restrict__ a)
    {
        if (slice >= nSlices)
            return;
        const int lane = threadIdx.x & 31;
        const int row = slice * SELL_C + lane;
        const int b0 = ldg(ss + slice), e0 = ldg(ss + slice + 1);
        const int w = (e0 - b0) / SELL_C;
        float2 acc = make_float2(0.f, 0.f);
        constexpr int U = 8;
        for (int kk = 0; kk < w; kk += U)
        {
            int cc[U];
            float av[U];
#pragma unroll
            for (int t = 0; t < U; t++)
            {
                const bool ok = kk + t < w;
                const int j = b0 + (kk + t) * SELL_C + lane;
                cc[t] = ok ? ldg(ci + j) : 0;
                av[t] = ok ? ldg(iv + j) : 0.f;
            }
            float2 g[U];
#pragma unroll
            for (int t = 0; t < U; t++)
                g[t] = kk + t < w ? ldg(u + cc[t]) : make_float2(0.f, 0.f);
#pragma unroll
            for (int t = 0; t < U; t++)
                acc = dfDotAdd(acc, av[t], g[t]);
        }
        if (row >= rows)
            return;
        const int r = ldg(perm + row);
        a[r] = dfAdd(dfMul(nu, ldg(k + r)), dfDotEnd(acc));
    }

    __global__ void __launch_bounds__(TPB) kFastConvSellDf(int rows, int nSlices, const int * __restrict__ ss,
                                                            const int * __restrict__ perm, const int * __restrict__ ci,
                                                            const float * __restrict__ iv, const float2 * __restrict__ u,
                                                            const float2 * __restrict__ k, float2 nu,
                                                            float2 * __restrict__ a)
    {
        const int slice = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
        fastConvSellDfSlice(slice, rows, nSlices, ss, perm, ci, iv, u, k, nu, a);
    }

    // planar multi-RHS in double-float, FP64 result: Y[c ldy + r] = sum_j A[r, j] X[c ldx + j]
    template <int L, int NCH>
    __device__ __forceinline__ void spmmDfRows(const Group<L> & g, int rows, const int * __restrict__ rs,
                                               const int * __restrict__ ci, const float2 * __restrict__ v,
                                               const float2 * __restrict__ X, int ldx, double * __restrict__ Y, int ldy)
    {
        for (int r = g.gid; r < rows; r += g.ngroups)
        {
            const int b = ldg(rs + r), e = ldg(rs + r + 1);
            float2 s[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                s[c] = make_float2(0.f, 0.f);
            for (int j = b + g.lane; j < e; j += L)
            {
                const float2 a = ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    s[c] = dfDotAdd(s[c], a, ldg(X + (size_t)c * ldx + col));
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                float2 t = dfDotEnd(s[c]);
#pragma unroll
                for (int o = L / 2; o > 0; o >>= 1)
                {
                    const float2 other = make_float2(__shfl_down_sync(g.mask, t.x, o, L),
                                                     __shfl_down_sync(g.mask, t.y, o, L));
                    t = dfAdd(t, other);
                }
                if (g.lane == 0)
                    Y[(size_t)c * ldy + r] = dfToDouble(t);
            }
        }
    }

    template <int L, int NCH>
    __global__ void __launch_bounds__(TPB) kSpmmDf(int rows, const int * __restrict__ rs, const int * __restrict__ ci,
                                                    const float2 * __restrict__ v, const float2 * __restrict__ X, int ldx,
                                                    double * __restrict__ Y, int ldy)
    {
        const Group<L> g;
        spmmDfRows<L, NCH>(g, rows, rs, ci, v, X, ldx, Y, ldy);
    }

    // Initial guess of the pressure solve from the last two solutions: before step k the solve
    // starts from 2 p_{k-1} - p_{k-2} once two solved pressures exist (hist >= 2), else from p_{k-1};
    // prev keeps p_{k-1} for the next step.  kHistBump advances the count afterwards (separate
    // launch: every thread here reads the same count).
    __global__ void __launch_bounds__(TPB) kExtrapolate(int n, double * __restrict__ p, double * __restrict__ prev,
                                                         const int * __restrict__ hist)
    {
        const bool two = *hist >= 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const double cur = p[i];
            if (two)
                p[i] = 2.0 * cur - prev[i];
            prev[i] = cur;
        }
    }

    __global__ void kHistBump(int * hist)
    {
        if (threadIdx.x == 0 && blockIdx.x == 0 && *hist < 2)
            *hist += 1;
    }

    // x64 += d (mixed-precision refinement update)
    template <typename TD>
    __global__ void __launch_bounds__(TPB) kAddTo(int n, double * __restrict__ x, const TD * __restrict__ d,
                                                   const int * __restrict__ skip)
    {
        if (skip && *skip)
            return;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i] += (double)d[i];
    }

    // dst[c * n + i] = src[c * n + perm[i]]   (into the color-permuted numbering)
    template <typename T>
    __global__ void __launch_bounds__(TPB) kGatherPerm(int n, int nch, const int * __restrict__ perm,
                                                        const T * __restrict__ src, T * __restrict__ dst)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const int j = perm[i];
            for (int c = 0; c < nch; c++)
                dst[(size_t)c * n + i] = src[(size_t)c * n + j];
        }
    }

    // dst[c * n + perm[i]] = src[c * n + i]   (back to the original numbering)
    template <typename T>
    __global__ void __launch_bounds__(TPB) kScatterPerm(int n, int nch, const int * __restrict__ perm,
                                                         const T * __restrict__ src, T * __restrict__ dst)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const int j = perm[i];
            for (int c = 0; c < nch; c++)
                dst[(size_t)c * n + j] = src[(size_t)c * n + i];
        }
    }

    // ------------------------------------------------------------------ solver state

    // Device-resident scalars of one solve (numCh planar channels).
    struct SolverState
    {
        double rzHist[2][MAXCH];      // r.z of the last two iterations (index = iteration parity)
        double bb[MAXCH];             // ||b||^2
        double lastRR[MAXCH];         // ||r||^2 at the last convergence check
        double rrOut[MAXCOLORS][MAXCH]; // per color phase: ||r||^2 of its rows
        double rzOut[MAXCOLORS][MAXCH]; // per color phase: r.z of its rows
        double pqOut[MAXCH];          // p.Ap of the current iteration
        double bbOut[MAXCH];          // ||b||^2 of the current solve
        double tol2;                  // relative tolerance squared (or absolute RMS^2 * n)
        int absMode;                  // 1: stop on ||r||^2 < tol2 (absolute), 0: ||r||^2 <= tol2 ||b||^2
        int active[MAXCH];
        int iters[MAXCH];
        int status[MAXCH];            // 0 ok / converged, 2 non-finite, 3 max iterations, 4 breakdown
        int iter;                     // iterations started (advanced by the last block of an iteration)
        int maxIters;
        int anyActive;                // 0 once every channel stopped (host polls this)
        unsigned ticket;              // last-block ticket of the grid reductions
        int skip;                     // refinement: 1 once the outer loop has stopped
        int innerTotal[MAXCH];        // refinement: inner iterations summed over passes
        // CG step lengths, computed once per grid by the thread that finishes a reduction and read
        // by every thread in the solve precision
        double alphaD[MAXCH], betaD[MAXCH];
        float alphaF[MAXCH], betaF[MAXCH];
        // refinement: power-of-two scale of the pass's FP32 right-hand side (2^-e, ||r|| ~ 2^e) and
        // its inverse, so that the inner FP32 solve works on O(1) values whatever ||r|| is
        double rscale[MAXCH], rinv[MAXCH];
    };

    __device__ __forceinline__ void loadScalar(float & v, const double *, const float * f, int c) { v = f[c]; }
    __device__ __forceinline__ void loadScalar(double & v, const double * d, const float *, int c) { v = d[c]; }

    __global__ void kSetConfig(SolverState * st, int maxIters, int absMode, double tol2)
    {
        if (threadIdx.x == 0)
        {
            st->maxIters = maxIters;
            st->absMode = absMode;
            st->tol2 = tol2;
        }
    }

    __global__ void kOuterReset(SolverState * st)
    {
        if (threadIdx.x == 0)
        {
            st->skip = 0;
            st->ticket = 0;
            for (int c = 0; c < MAXCH; c++)
            {
                st->status[c] = 0;
                st->iters[c] = 0;
                st->innerTotal[c] = 0;
                st->active[c] = 1;
            }
            st->anyActive = 1;
        }
    }

    // refinement: count the iterations of a preceding FP64 solve (the FP32-preconditioned form) as
    // inner iterations of the solve
    __global__ void kAddInnerIters(SolverState * st, const SolverState * solve, int numCh)
    {
        if (threadIdx.x == 0)
            for (int c = 0; c < numCh && c < MAXCH; c++)
                st->innerTotal[c] += solve->iters[c];
    }

    template <int NCH>
    __device__ __forceinline__ bool anyAct(const bool (&a)[NCH])
    {
        bool r = false;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            r |= a[c];
        return r;
    }

    // sum over the color phases of a per-phase quantity (fixed order)
    __device__ __forceinline__ double phaseSum(const double (*a)[MAXCH], int nColors, int c)
    {
        double s = 0;
        for (int k = 0; k < nColors; k++)
            s += a[k][c];
        return s;
    }

    // ------------------------------------------------------------------ PCG with multicolor SGS
    // Work vectors are planar [ch * n + i] in the color-permuted numbering; color c owns rows
    // [ps[c], ps[c+1]).

    struct PcgPtrs
    {
        int n, nColors;
        double * scratch;        // block sums of the current kernel [2 * MAXCH * maxGrid]
        SolverState * st;
        unsigned long long cond; // graph conditional handle (0: none)
        const int * skip;        // when set and *skip != 0 the solve stops at start (refinement done)
    };

    // r = b - A x (full matrix); ||b||^2
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgInit(PcgPtrs P, const int * __restrict__ rs, const int * __restrict__ ci,
                                                     const T * __restrict__ v, const T * __restrict__ x,
                                                     const T * __restrict__ b, T * __restrict__ r)
    {
        if (P.skip && *P.skip)
            return; // refinement finished: the whole solve is a no-op (same in every block)
        Group<L> g;
        T bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        const int n = P.n;
        for (int i = g.gid; i < n; i += g.ngroups)
        {
            const int s = ldg(rs + i), e = ldg(rs + i + 1);
            T acc[NCH]; // row arithmetic and reductions in the solve precision
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const T a = ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] += a * x[(size_t)c * n + col];
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const T t = g.sum(acc[c]);
                if (g.lane == 0)
                {
                    const T bi = b[(size_t)c * n + i];
                    r[(size_t)c * n + i] = bi - t;
                    bb[c] += bi * bi;
                }
            }
        }
        Outs<NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            o.p[c] = &P.st->bbOut[c];
        gridSum<T, NCH>(bb, P.scratch, o, &P.st->ticket, nullptr);
    }

    // Decision before iteration k, taken by one thread once the SGS sweep that produced the phase
    // sums of ||r||^2 and r.z is complete (end of iteration k - 1, or the initial sweep): stop the
    // channels that converged, went non-finite, broke down or reached the cap; beta of iteration k;
    // end the device loop when nothing is left.
    template <int NCH>
    __device__ void pcgDecide(SolverState * st, int nColors, int numCh, int k, unsigned long long cond)
    {
        int any = 0;
        for (int c = 0; c < NCH; c++)
        {
            const double rr = phaseSum(st->rrOut, nColors, c);
            const double rz = phaseSum(st->rzOut, nColors, c);
            const bool wasActive = c < numCh && st->active[c] && st->status[c] == 0;
            const bool fin = isfinite(rr) && isfinite(rz);
            const bool conv = st->absMode ? (rr < st->tol2) : (rr <= st->tol2 * st->bb[c]);
            const bool act = wasActive && fin && !conv && (k <= st->maxIters);
            const double beta = (k == 1) ? 0.0 : rz / st->rzHist[(k - 1) & 1][c];
            if (c < numCh && st->active[c] && !act)
            {
                st->iters[c] = k - 1;
                st->lastRR[c] = rr;
                if (st->status[c] == 0)
                    st->status[c] = !fin ? 2 : (conv ? 0 : 3);
            }
            st->rzHist[k & 1][c] = rz;
            st->betaD[c] = beta;
            st->betaF[c] = (float)beta;
            st->active[c] = act;
            any |= act;
        }
        st->anyActive = any;
        if (!any && cond)
            cudaGraphSetConditional(cond, 0);
    }

    // Finish the initial state once the SGS of r0 is done: bb, activity, iteration counter, and the
    // decision before the first iteration.
    template <int NCH>
    __global__ void kPcgStart(PcgPtrs P, int numCh)
    {
        if (threadIdx.x != 0)
            return;
        SolverState * st = P.st;
        const bool skipAll = P.skip && *P.skip;
        int any = 0;
        for (int c = 0; c < NCH; c++)
        {
            const double bb = st->bbOut[c];
            const double rr = phaseSum(st->rrOut, P.nColors, c);
            const double rz = phaseSum(st->rzOut, P.nColors, c);
            st->bb[c] = bb;
            st->lastRR[c] = rr;
            st->rzHist[0][c] = rz;
            st->rzHist[1][c] = rz;
            const bool fin = isfinite(rr) && isfinite(bb);
            const bool conv = st->absMode ? (rr < st->tol2) : (rr <= st->tol2 * bb);
            const bool act = c < numCh && fin && !conv && !skipAll;
            st->active[c] = act;
            st->iters[c] = 0;
            st->status[c] = fin ? 0 : 2;
            any |= act;
        }
        st->iter = 1;
        st->ticket = 0;
        st->anyActive = any;
        pcgDecide<NCH>(st, P.nColors, numCh, 1, 0ull);
    }

    // Iteration kernel A: convergence decision from the previous iteration's ||r||^2, beta,
    // p_new = z + beta p_old, q = A p_new, p.q.
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgDirection(PcgPtrs P, int numCh, const int * __restrict__ rs,
                                                          const int * __restrict__ ci, const T * __restrict__ v,
                                                          const T * __restrict__ z, T * __restrict__ pbuf,
                                                          T * __restrict__ q)
    {
        SolverState * st = P.st;
        const int k = st->iter; // stable for the whole iteration
        if (!st->anyActive)
        {
            // every channel stopped at the last decision (same value in every block): end the loop
            if (blockIdx.x == 0 && threadIdx.x == 0 && P.cond)
                cudaGraphSetConditional(P.cond, 0);
            return;
        }
        bool act[NCH];
        T betaT[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            act[c] = c < numCh && st->active[c];
            loadScalar(betaT[c], st->betaD, st->betaF, c);
        }
        T pq[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            pq[c] = 0;
        {
            const int n = P.n;
            const T * pold = pbuf + (size_t)((k - 1) & 1) * NCH * n;
            T * pnew = pbuf + (size_t)(k & 1) * NCH * n;
            Group<L> g;
            for (int i = g.gid; i < n; i += g.ngroups)
            {
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const T a = ldg(v + j);
                    const int col = ldg(ci + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + col;
                            acc[c] += a * (k == 1 ? z[o] : z[o] + betaT[c] * pold[o]);
                        }
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const T t = g.sum(acc[c]);
                    if (g.lane == 0 && act[c])
                    {
                        const size_t o = (size_t)c * n + i;
                        const T pn = k == 1 ? z[o] : z[o] + betaT[c] * pold[o];
                        pnew[o] = pn;
                        q[o] = t;
                        pq[c] += pn * t;
                    }
                }
            }
        }
        Outs<NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            o.p[c] = &st->pqOut[c];
        // once per grid: alpha = r.z / p.q, breakdown when p.q <= 0 (the channel stops at the next decision)
        gridSum<T, NCH>(pq, P.scratch, o, &st->ticket, nullptr, [&]() {
            for (int c = 0; c < NCH; c++)
            {
                const double pqc = st->pqOut[c];
                const double a = st->rzHist[k & 1][c] / pqc;
                st->alphaD[c] = a;
                st->alphaF[c] = (float)a;
                if (c < numCh && st->active[c] && !(pqc > 0))
                    st->status[c] = isfinite(pqc) ? 4 : 2;
            }
        });
    }

    // Forward SGS phase over color rows [r0, r1) using only neighbours of earlier colors
    // (columns < r0; later colors are still zero in a forward sweep from z = 0).
    // init == 0: first x += alpha p, r -= alpha q for these rows.  Writes ||r||^2 of the color
    // (and r.z when this is the last color).  tick: last kernel of an iteration (one color only).
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgForward(PcgPtrs P, int numCh, int init, int color, int r0, int r1,
                                                        int last, int tick, const int * __restrict__ rs,
                                                        const int * __restrict__ ci, const T * __restrict__ v,
                                                        const T * __restrict__ invD, T * __restrict__ x,
                                                        T * __restrict__ r, T * __restrict__ z,
                                                        const T * __restrict__ pbuf, const T * __restrict__ q)
    {
        if (P.skip && *P.skip)
            return;
        SolverState * st = P.st;
        bool act[NCH];
        T alphaT[NCH];
        const int k = st->iter;
        const int n = P.n;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            act[c] = c < numCh && (init || st->active[c]);
            alphaT[c] = 0;
            if (!init)
                loadScalar(alphaT[c], st->alphaD, st->alphaF, c);
        }
        const T * p = pbuf + (size_t)(k & 1) * NCH * n;
        Group<L> g;
        T red[2 * NCH];
#pragma unroll
        for (int c = 0; c < 2 * NCH; c++)
            red[c] = 0;
        if (anyAct<NCH>(act))
            for (int i = r0 + g.gid; i < r1; i += g.ngroups)
            {
                T ri[NCH];
                if (g.lane == 0)
                {
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            T rv = r[o];
                            if (!init)
                            {
                                x[o] = x[o] + alphaT[c] * p[o];
                                rv -= alphaT[c] * q[o];
                                r[o] = rv;
                            }
                            ri[c] = rv;
                        }
                }
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const int col = ldg(ci + j);
                    if (col >= r0)
                        break; // sorted columns: the rest are later colors (zero)
                    const T a = ldg(v + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            acc[c] += a * z[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const T t = g.sum(acc[c]);
                    if (g.lane == 0 && act[c])
                    {
                        const size_t o = (size_t)c * n + i;
                        const T zi = (ri[c] - t) * ldg(invD + i);
                        z[o] = zi;
                        red[c] += ri[c] * ri[c];
                        if (last)
                            red[NCH + c] += ri[c] * zi;
                    }
                }
            }
        Outs<2 * NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            o.p[c] = &st->rrOut[color][c];
            o.p[NCH + c] = last ? &st->rzOut[color][c] : nullptr;
        }
        const bool ends = tick && !init; // last kernel of an iteration: decide the next one
        gridSum<T, 2 * NCH>(red, P.scratch, o, &st->ticket, ends ? &st->iter : nullptr, [&]() {
            if (ends)
                pcgDecide<NCH>(st, P.nColors, numCh, k + 1, P.cond);
        });
    }

    // Backward SGS phase over color rows [r0, r1) with all off-diagonal neighbours; r.z of the
    // color.  tick != 0: this is the last kernel of an iteration (advances the iteration counter).
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgBackward(PcgPtrs P, int numCh, int init, int color, int r0, int r1,
                                                         int tick, const int * __restrict__ rs,
                                                         const int * __restrict__ ci, const T * __restrict__ v,
                                                         const T * __restrict__ invD, const T * __restrict__ r,
                                                         T * __restrict__ z)
    {
        if (P.skip && *P.skip)
            return;
        SolverState * st = P.st;
        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh && (init || st->active[c]);
        const int n = P.n;
        const int k = st->iter;
        Group<L> g;
        T rz[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            rz[c] = 0;
        if (anyAct<NCH>(act))
            for (int i = r0 + g.gid; i < r1; i += g.ngroups)
            {
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const T a = ldg(v + j);
                    const int col = ldg(ci + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            acc[c] += a * z[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const T t = g.sum(acc[c]);
                    if (g.lane == 0 && act[c])
                    {
                        const size_t o = (size_t)c * n + i;
                        const T ri = r[o];
                        const T zi = (ri - t) * ldg(invD + i);
                        z[o] = zi;
                        rz[c] += ri * zi;
                    }
                }
            }
        Outs<NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            o.p[c] = &st->rzOut[color][c];
        const bool ends = tick && !init; // last kernel of an iteration: decide the next one
        gridSum<T, NCH>(rz, P.scratch, o, &st->ticket, ends ? &st->iter : nullptr, [&]() {
            if (ends)
                pcgDecide<NCH>(st, P.nColors, numCh, k + 1, P.cond);
        });
    }

    // ------------------------------------------------------------------ multicolor Gauss-Seidel
    // The reference's "gs" solver: C colored phases per iteration, RMS residual check every
    // `interval` iterations; decision taken at the start of the following iteration.

    struct GsPtrs
    {
        int n;
        double * scratch;
        SolverState * st;
        unsigned long long cond;
        int interval;
    };

    // ||b||^2 (for the relative mode)
    template <typename T, int NCH>
    __global__ void __launch_bounds__(TPB) kGsInit(GsPtrs P, int numCh, const T * __restrict__ b)
    {
        T bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        const int n = P.n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const T t = b[(size_t)c * n + i];
                bb[c] += t * t;
            }
        Outs<NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            o.p[c] = &P.st->bbOut[c];
        gridSum<T, NCH>(bb, P.scratch, o, &P.st->ticket, nullptr);
    }

    template <int NCH>
    __global__ void kGsStart(GsPtrs P, int numCh)
    {
        if (threadIdx.x != 0)
            return;
        SolverState * st = P.st;
        int any = 0;
        for (int c = 0; c < NCH; c++)
        {
            const double bb = st->bbOut[c];
            st->bb[c] = bb;
            st->lastRR[c] = -1;
            st->active[c] = c < numCh && isfinite(bb);
            st->iters[c] = 0;
            st->status[c] = isfinite(bb) ? 0 : 2;
            any |= st->active[c];
        }
        st->iter = 0;
        st->ticket = 0;
        st->anyActive = any;
    }

    // One color phase.  Phase 0 first decides on the residual of the previous check.
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kGsPhase(GsPtrs P, int numCh, int r0, int r1, int first,
                                                     const int * __restrict__ rs, const int * __restrict__ ci,
                                                     const T * __restrict__ v, const T * __restrict__ invD,
                                                     const T * __restrict__ b, T * __restrict__ x)
    {
        SolverState * st = P.st;
        const int k = st->iter; // 0-based iteration about to run
        bool act[NCH];
        if (first)
        {
            const bool checked = k > 0 && ((k - 1) % P.interval) == 0;
            bool stopAll = true;
            bool was[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                was[c] = c < numCh && st->active[c];
                const double rr = checked ? st->rrOut[0][c] : 0.0;
                const bool fin = !checked || isfinite(rr);
                const bool conv = checked && (st->absMode ? (rr < st->tol2) : (rr <= st->tol2 * st->bb[c]));
                act[c] = was[c] && fin;
                // both channels stop together once both meet the target (reference semantics)
                stopAll &= !(was[c] && fin) || conv;
                if (blockIdx.x == 0 && threadIdx.x == 0 && was[c])
                {
                    if (checked)
                        st->lastRR[c] = rr;
                    if (!fin)
                        st->status[c] = 2;
                }
            }
            const bool over = k >= st->maxIters;
            if (stopAll || over)
            {
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    act[c] = false;
            }
            __syncthreads(); // every block has read st->active before block 0 updates it
            if (blockIdx.x == 0 && threadIdx.x == 0)
            {
                int any = 0;
                for (int c = 0; c < NCH; c++)
                {
                    if (was[c] && !act[c])
                    {
                        // index of the last iteration run, or the cap (reference's lastIterations)
                        st->iters[c] = (over && !stopAll) ? k : k - 1;
                        if (over && !stopAll && st->status[c] == 0)
                            st->status[c] = 3;
                    }
                    st->active[c] = act[c];
                    any |= act[c];
                }
                st->anyActive = any;
                if (!any && P.cond)
                    cudaGraphSetConditional(P.cond, 0);
            }
        }
        else
        {
#pragma unroll
            for (int c = 0; c < NCH; c++)
                act[c] = c < numCh && st->active[c];
        }
        if (!anyAct<NCH>(act))
            return;
        const int n = P.n;
        Group<L> g;
        for (int i = r0 + g.gid; i < r1; i += g.ngroups)
        {
            const int s = ldg(rs + i), e = ldg(rs + i + 1);
            T acc[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const T a = ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                        acc[c] += a * x[(size_t)c * n + col];
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const T t = g.sum(acc[c]);
                if (g.lane == 0 && act[c])
                {
                    const size_t o = (size_t)c * n + i;
                    x[o] = (b[o] - t) * ldg(invD + i);
                }
            }
        }
    }

    // residual check (every `interval` iterations) + iteration tick
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kGsCheck(GsPtrs P, int numCh, const int * __restrict__ rs,
                                                     const int * __restrict__ ci, const T * __restrict__ v,
                                                     const T * __restrict__ b, const T * __restrict__ x)
    {
        SolverState * st = P.st;
        const int k = st->iter;
        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh && st->active[c];
        if (!anyAct<NCH>(act))
            return; // the loop is ending; no tick needed
        const bool doCheck = (k % P.interval) == 0;
        T rr[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            rr[c] = 0;
        if (doCheck)
        {
            const int n = P.n;
            Group<L> g;
            for (int i = g.gid; i < n; i += g.ngroups)
            {
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const T a = ldg(v + j);
                    const int col = ldg(ci + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] += a * x[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const T t = g.sum(acc[c]);
                    if (g.lane == 0)
                    {
                        const T d = t - b[(size_t)c * n + i];
                        rr[c] += d * d;
                    }
                }
            }
        }
        Outs<NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            o.p[c] = doCheck ? &st->rrOut[0][c] : nullptr;
        gridSum<T, NCH>(rr, P.scratch, o, &st->ticket, &st->iter);
    }

    // ------------------------------------------------------------------ FP64 refinement

    // r = b - A x in FP64; r is handed to the FP32 inner solve; ||r||^2 and ||b||^2
    template <int L, int NCH>
    __global__ void __launch_bounds__(TPB) kResidual(int n, SolverState * st, double * scratch,
                                                      const int * __restrict__ rs, const int * __restrict__ ci,
                                                      const double * __restrict__ v, const double * __restrict__ x,
                                                      const double * __restrict__ b, float * __restrict__ r32)
    {
        if (st->skip)
            return;
        Group<L> g;
        double red[2 * NCH];
#pragma unroll
        for (int c = 0; c < 2 * NCH; c++)
            red[c] = 0;
        for (int i = g.gid; i < n; i += g.ngroups)
        {
            const int s = ldg(rs + i), e = ldg(rs + i + 1);
            double acc[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const double a = ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] += a * x[(size_t)c * n + col];
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double t = g.sum(acc[c]);
                if (g.lane == 0)
                {
                    const double bi = b[(size_t)c * n + i];
                    const double ri = bi - t;
                    r32[(size_t)c * n + i] = (float)ri;
                    red[c] += ri * ri;
                    red[NCH + c] += bi * bi;
                }
            }
        }
        Outs<2 * NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            o.p[c] = &st->rrOut[0][c];
            o.p[NCH + c] = &st->bbOut[c];
        }
        gridSum<double, 2 * NCH>(red, scratch, o, &st->ticket, nullptr);
    }

    // refinement pass: r32 *= rscale (exact: a power of two), skipped once the loop has stopped
    template <int NCH>
    __global__ void __launch_bounds__(TPB) kScalePass(int n, float * __restrict__ r32, const SolverState * st)
    {
        if (st->skip)
            return;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NCH * n; i += gridDim.x * blockDim.x)
            r32[i] = (float)((double)r32[i] * st->rscale[i / n]);
    }

    // refinement update x64 += d / rscale
    template <int NCH>
    __global__ void __launch_bounds__(TPB) kAddScaled(int n, double * __restrict__ x, const float * __restrict__ d,
                                                       const SolverState * st)
    {
        if (st->skip)
            return;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NCH * n; i += gridDim.x * blockDim.x)
            x[i] += (double)d[i] * st->rinv[i / n];
    }

    // After a Chebyshev solve: ||b - A x||^2 and ||b||^2 per channel in FP64, recorded as the solve's
    // statistics: iters, bb, lastRR, status (0 if within tol2, else 3).
    struct ChebEpi
    {
        SolverState * st;
        int numCh, iters;
        const int * kdev; // the warm solve's device count (else iters)
        __device__ void operator()() const
        {
            const int iters = kdev ? *kdev : this->iters;
            for (int c = 0; c < numCh; c++)
            {
                const double rr = st->rrOut[0][c], bb = st->bbOut[c];
                st->bb[c] = bb;
                st->lastRR[c] = rr;
                st->iters[c] = iters;
                st->innerTotal[c] = iters;
                st->active[c] = 0;
                st->status[c] = !(isfinite(rr) && isfinite(bb)) ? 2 : (rr <= st->tol2 * bb ? 0 : 3);
            }
            st->anyActive = 0;
        }
    };

    // r = b - M x through the SELL copy of M with ||r||^2 and ||b||^2 per channel, reduced over the
    // grid and handed to epi in the last block: the check after a Chebyshev solve (ChebEpi) and the
    // start of a warm solve (ChebWarmEpi, WR: r written).  A warp per slice and channel (warps 2s and
    // 2s + 1 take the two channels of slice s), so the rows of a warp are consecutive stored rows.
    // FP64: M x from the FP64 values, FP64 sums.  DF (after the double-float iterations): FP64
    // arithmetic runs at 1/64 of the FP32 rate on this GPU, so the check stays on the FP32 pipes:
    // M x from the double-float values and solution with Dot2 sums (about 48 bits), r = b - M x in
    // double-float against b kept as double-floats at the solve's start (bDf), and the squares and
    // their sums in FP32 (relative error ~1e-6, ample for a tolerance decision and the reported
    // ratio).  The solution is converted to FP64 here and written to x for the warp's own rows,
    // which replaces a separate conversion pass.
    template <bool DF, bool WR, typename Epi>
    __global__ void __launch_bounds__(TPB) kChebResidualSell(int n, int nSlices, const int * __restrict__ ss,
                                                              const int * __restrict__ perm, const int * __restrict__ ci,
                                                              const double * __restrict__ v, const float2 * __restrict__ vDf,
                                                              const float2 * __restrict__ xDf, double * x,
                                                              const double * __restrict__ b, const float2 * __restrict__ bDf,
                                                              double * __restrict__ r, SolverState * st, double * scratch,
                                                              Epi epi)
    {
        constexpr int NCH = 2;
        using TA = typename std::conditional<DF, float, double>::type;
        TA red[2 * NCH];
#pragma unroll
        for (int c = 0; c < 2 * NCH; c++)
            red[c] = 0;
        const int lane = threadIdx.x & 31;
        const int nw = (int)((gridDim.x * (unsigned)blockDim.x) >> 5);
        for (int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5); w < NCH * nSlices; w += nw)
        {
            const int slice = w >> 1, c = w & 1;
            const size_t co = (size_t)c * n;
            const int row = slice * SELL_C + lane;
            const int b0 = ldg(ss + slice), e0 = ldg(ss + slice + 1);
            const int wd = (e0 - b0) / SELL_C;
            double acc = 0.0;
            float2 q = make_float2(0.f, 0.f);
            for (int k = 0; k < wd; k += 4)
            {
                int cc[4];
#pragma unroll
                for (int t = 0; t < 4; t++)
                    cc[t] = k + t < wd ? ldg(ci + b0 + (k + t) * SELL_C + lane) : 0;
                if (DF)
                {
                    float2 a[4], g[4];
#pragma unroll
                    for (int t = 0; t < 4; t++)
                    {
                        a[t] = k + t < wd ? ldg(vDf + b0 + (k + t) * SELL_C + lane) : make_float2(0.f, 0.f);
                        g[t] = k + t < wd ? ldg(xDf + co + cc[t]) : make_float2(0.f, 0.f);
                    }
#pragma unroll
                    for (int t = 0; t < 4; t++)
                        if (k + t < wd)
                            q = dfDotAdd(q, a[t], g[t]);
                }
                else
                {
                    double a[4], g[4];
#pragma unroll
                    for (int t = 0; t < 4; t++)
                    {
                        a[t] = k + t < wd ? ldg(v + b0 + (k + t) * SELL_C + lane) : 0.0;
                        g[t] = k + t < wd ? ldg(x + co + cc[t]) : 0.0;
                    }
#pragma unroll
                    for (int t = 0; t < 4; t++)
                        acc += a[t] * g[t];
                }
            }
            if (row < n)
            {
                const size_t o = co + ldg(perm + row);
                TA rr, bb;
                if (DF)
                {
                    x[o] = dfToDouble(ldg(xDf + o));
                    const float2 bi = ldg(bDf + o), ri = dfAdd(bi, dfNeg(dfDotEnd(q)));
                    rr = (TA)(ri.x * ri.x);
                    bb = (TA)(bi.x * bi.x);
                }
                else
                {
                    const double bi = ldg(b + o), ri = bi - acc;
                    if (WR)
                        r[o] = ri;
                    rr = (TA)(ri * ri);
                    bb = (TA)(bi * bi);
                }
                red[0] += c == 0 ? rr : (TA)0;
                red[1] += c == 1 ? rr : (TA)0;
                red[NCH] += c == 0 ? bb : (TA)0;
                red[NCH + 1] += c == 1 ? bb : (TA)0;
            }
        }
        Outs<2 * NCH> o;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            o.p[c] = &st->rrOut[0][c];
            o.p[NCH + c] = &st->bbOut[c];
        }
        gridSum<TA, 2 * NCH>(red, scratch, o, &st->ticket, nullptr, epi);
    }

    // Warm-started Chebyshev (mass-solve method 4): x0 is the previous step's solution of the same
    // solve.  Part 1: r0 = b - A x0 (FP64, row groups over the CSR), ||r0||^2 and ||b||^2 per
    // channel; the last block decides per channel whether x0 is a better start than 0 (else that
    // channel starts cold) and the iteration count from the a priori bound
    //   ||r_k|| <= 2 rho^k sqrt(max D / min D) ||r0|| <= tol ||b||,  k <= kmax (the cold count).
    struct ChebWarmEpi
    {
        SolverState * st;
        int * kw; // kw[0]: the iteration count, kw[1 + c]: channel c starts from x0
        int numCh, kmax;
        double lnTarget, lnRho; // log(tol / (2 sqrt(max D / min D))), log(rho)
        __device__ void operator()() const
        {
            int k = 0;
            for (int c = 0; c < numCh; c++)
            {
                const double rr = st->rrOut[0][c], bb = st->bbOut[c];
                int kc;
                if (bb == 0.0)
                {
                    kw[1 + c] = 0; // b = 0: x = 0 is exact, a cold start needs no iteration
                    kc = 0;
                }
                else if (!(rr < bb))
                {
                    kw[1 + c] = 0;
                    kc = kmax;
                }
                else
                {
                    kw[1 + c] = 1;
                    if (!(rr > st->tol2 * bb))
                        kc = 0;
                    else
                    {
                        kc = (int)ceil((lnTarget + 0.5 * log(bb / rr)) / lnRho);
                        kc = kc < 1 ? 1 : (kc > kmax ? kmax : kc);
                    }
                }
                k = kc > k ? kc : k;
            }
            kw[0] = k;
        }
    };

    // Part 2 (FP64 iterations): a warm channel keeps x = x0 and r = r0, a cold one gets x = 0 and
    // r = b; d = D^-1 r / theta
    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebWarmInit(int n, const double * __restrict__ b, const double * __restrict__ invD,
                                                          double invTheta, const int * __restrict__ kw,
                                                          double * __restrict__ x, double * __restrict__ r,
                                                          double * __restrict__ d)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const double id = invD[i];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const size_t o = (size_t)c * n + i;
                double ri = r[o];
                if (!kw[1 + c])
                {
                    ri = b[o];
                    r[o] = ri;
                    x[o] = 0.0;
                }
                d[o] = ri * id * invTheta;
            }
        }
    }

    // Part 2 (double-float iterations): the same into the double-float vectors
    template <int NCH>
    __global__ void __launch_bounds__(TPB) kChebWarmInitDf(int n, const double * __restrict__ b, const double * __restrict__ x0,
                                                            const double * __restrict__ r0, const float2 * __restrict__ invD,
                                                            float2 invTheta, const int * __restrict__ kw,
                                                            float2 * __restrict__ x, float2 * __restrict__ r,
                                                            float2 * __restrict__ d, float2 * __restrict__ bOut)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const float2 id = invD[i];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const size_t o = (size_t)c * n + i;
                const bool warm = kw[1 + c] != 0;
                const float2 bi = dfFromDouble(b[o]);
                const float2 ri = warm ? dfFromDouble(r0[o]) : bi;
                bOut[o] = bi;
                r[o] = ri;
                x[o] = warm ? dfFromDouble(x0[o]) : make_float2(0.f, 0.f);
                d[o] = dfMul(dfMul(ri, id), invTheta);
            }
        }
    }


    // Stop decision of refinement pass `pass` (sticky); stats: iters = refinement updates applied.
    // The next inner solve only has to reach half the remaining distance to the target:
    // inner relative tolerance = max(innerMin, 0.5 * tol * ||b|| / ||r||), written into the inner
    // solver's state (its configuration is not reset by the host between passes).
    template <int NCH>
    __global__ void kOuterDecide(SolverState * st, SolverState * inner, int numCh, int pass, double innerMin,
                                 int innerMaxIters)
    {
        if (threadIdx.x != 0 || st->skip)
            return;
        bool all = true, bad = false, settled = true;
        bool convC[NCH];
        double rr[NCH], bb[NCH];
        for (int c = 0; c < NCH && c < numCh; c++)
        {
            rr[c] = st->rrOut[0][c];
            bb[c] = st->bbOut[c];
            if (pass > 0)
                st->innerTotal[c] += inner->iters[c];
            const bool fin = isfinite(rr[c]) && isfinite(bb[c]);
            const bool conv = rr[c] <= st->tol2 * bb[c];
            // a pass that no longer halves the FP64 residual has reached its rounding floor: further
            // passes would refine noise
            const bool stalled = pass > 0 && rr[c] > 0.25 * st->lastRR[c];
            convC[c] = conv;
            bad |= !fin;
            all &= conv;
            settled &= conv || stalled;
            st->bb[c] = bb[c];
            st->lastRR[c] = rr[c];
            st->iters[c] = pass;
        }
        if (all || bad || settled || pass >= st->maxIters)
        {
            st->skip = 1;
            st->anyActive = 0;
            for (int c = 0; c < NCH; c++)
            {
                st->active[c] = 0;
                st->status[c] = bad ? 2 : ((c >= numCh || convC[c]) ? 0 : 3);
            }
        }
        else
        {
            for (int c = 0; c < NCH; c++)
            {
                int e = 0;
                if (c < numCh && rr[c] > 0)
                    frexp(sqrt(rr[c]), &e);
                st->rscale[c] = ldexp(1.0, -e);
                st->rinv[c] = ldexp(1.0, e);
            }
            // loosest inner tolerance over the channels still above the target
            double need = 1.0;
            for (int c = 0; c < NCH && c < numCh; c++)
                if (rr[c] > st->tol2 * bb[c] && rr[c] > 0)
                    need = fmin(need, 0.5 * sqrt(st->tol2 * bb[c] / rr[c]));
            const double t = fmax(innerMin, need);
            inner->tol2 = t * t;
            inner->absMode = 0;
            inner->maxIters = innerMaxIters;
        }
    }
} // namespace nsf
