// Persistent CG with the multicolor symmetric Gauss-Seidel preconditioner: one launch runs a whole
// solve, the vectors stay in global memory (L2-resident), and the color phases are separated by
// barriers of one of two kinds (the `Sync` policy):
//   * ClusterSync: a single thread-block cluster of CS CTAs (16 where the GPU allows non-portable
//     clusters, else 8).  A cluster barrier costs ~0.3 us on the GB300.
//   * GridSync: a cooperative grid of one 1024-thread CTA per SM with a software grid barrier
//     (arrival counter + generation word, bounded waits).  Slower barriers, but every SM works,
//     which is what a large system (the velocity mass matrix) or an FP64 solve (FP64 runs at ~1/64
//     of the FP32 rate on this GPU) needs.
// CTA k owns chunk k of every color block, so x, r and q are only touched by their owner; z and p
// are read at neighbour rows of other CTAs through L2 (ld.global.cg).
//   * one thread per row; the entries of a row are processed in fixed-width predicated batches so
//     all value loads and neighbour gathers of a row are in flight together;
//   * when the structure of a CTA's rows (row offsets, column indices of the off-diagonal part)
//     fits in shared memory it is copied there at kernel start (SMEM = true), else it is read from
//     global memory;
//   * dot products are reduced in the solve precision with a fixed tree (lanes, warps, CTAs), so
//     every CTA holds bit-identical totals; the iteration scalars (alpha, beta, the stop decisions)
//     are computed from them once per CTA by thread 0, in FP64, and broadcast through shared memory,
//     so every CTA takes identical loop decisions and the barrier count never diverges.
//
// Tolerance, cap and mode are read from the SolverState written by a preceding kernel, so the FP64
// refinement loop can set the inner tolerance on the device.
#pragma once

#include <cooperative_groups.h>

#include <climits>
#include <type_traits>
#include <vector>

#include "kernels.cuh"

namespace nsf
{
    namespace cg = cooperative_groups;

    constexpr int CTPB = 1024;                    // threads per CTA of the persistent solvers
    constexpr size_t kClusterSmemCap = 200 * 1024; // dynamic shared memory ceiling per CTA
    constexpr int RB = 8;                          // entries per predicated batch of a row
    constexpr unsigned kGridSpinLimit = 1u << 22;  // default polls of a grid barrier before it gives up (seconds)

    // T: the CG recurrence (x, r, p, q, the dot products) and the operator A p; TP: the
    // preconditioner (its values, 1/diag and z).  TP = float under T = double keeps the FP64
    // recurrence, and with it the FP64 iteration count, while the sweeps run on the FP32 pipes.
    template <typename T, typename TP = T>
    struct ClusterPcgArgs
    {
        int n, nColors, numCh;
        const int * ps;                  // color starts (device), nColors + 1
        const int *rsO, *ciO;            // off-diagonal part
        const T * vO;
        const T * diag;                  // diagonal values
        const TP * vOP;                  // off-diagonal values of the preconditioner sweeps (vO when TP = T)
        const float * vOLo;              // T = double, TP = float: vO - vOP, so that (vOP, vOLo) is vO as a
                                         // double-float pair (A z on the FP32 pipes)
        const TP * invD;                 // inverses of the diagonal, in the preconditioner's type
        const T * b;
        T *x, *r, *p, *q;
        TP * z;
        SolverState * st;
        const int * skip;                // refinement: stop immediately when *skip != 0
    };

    __device__ __forceinline__ int chunkStart(const int * ps, int c, int rank, int cs)
    {
        const int a = ps[c], len = ps[c + 1] - a;
        return a + (int)(((long long)len * rank) / cs);
    }

    // Shared-memory footprint (bytes) of CTA `rank`: local row offsets (own rows + 1) and the
    // column indices of their off-diagonal entries.  Host and device compute it the same way.
    inline size_t clusterSmemBytes(const std::vector<int> & ps, const std::vector<int> & rsO, int rank, int cs)
    {
        size_t rows = 0, nnz = 0;
        for (size_t c = 0; c + 1 < ps.size(); c++)
        {
            const int len = ps[c + 1] - ps[c];
            const int a0 = ps[c] + (int)(((long long)len * rank) / cs);
            const int a1 = ps[c] + (int)(((long long)len * (rank + 1)) / cs);
            rows += a1 - a0;
            nnz += rsO[a1] - rsO[a0];
        }
        return 4 * (rows + 1 + nnz);
    }

    // Row structure of the CTA's own rows: shared-memory copy (SMEM) or the global CSR itself.
    template <bool SMEM>
    struct RowView;

    template <>
    struct RowView<true>
    {
        const int *lrs, *lci;
        const int *chunkA, *chunkL, *chunkG, *nzBase;
        __device__ __forceinline__ int begin(int, int l) const { return lrs[l]; }
        __device__ __forceinline__ int end(int, int l) const { return lrs[l + 1]; }
        __device__ __forceinline__ int col(int j) const { return lci[j]; }
        __device__ __forceinline__ int gnz(int c, int j) const { return chunkG[c] + (j - nzBase[c]); }
    };

    template <>
    struct RowView<false>
    {
        const int *rsO, *ciO;
        const int *chunkA, *chunkL;
        __device__ __forceinline__ int begin(int c, int l) const { return ldg(rsO + chunkA[c] + (l - chunkL[c])); }
        __device__ __forceinline__ int end(int c, int l) const { return ldg(rsO + chunkA[c] + (l - chunkL[c]) + 1); }
        __device__ __forceinline__ int col(int j) const { return ldg(ciO + j); }
        __device__ __forceinline__ int gnz(int, int j) const { return j; }
    };

    // acc[c] += sum over entries j of the row with col < limit:  a_j * (v0[c][col] + w * v1[c][col])
    // (v1 may be null).  Arithmetic in T; fixed-width predicated batches keep RB loads in flight.
    // The gathers are predicated on the column alone, so they issue together with the value loads.
    template <typename T, typename V0, int NCH, bool SMEM>
    __device__ __forceinline__ void rowGather(const RowView<SMEM> & rv, int color, int jb, int je, int limit,
                                              const T * vO, int n, const V0 * v0, const T * v1, const T * w,
                                              const bool (&act)[NCH], T (&acc)[NCH])
    {
        for (int j0 = jb; j0 < je; j0 += RB)
        {
            int cols[RB];
            bool use[RB];
            T vals[RB];
#pragma unroll
            for (int t = 0; t < RB; t++)
            {
                const int j = j0 + t;
                const bool ok = j < je;
                cols[t] = ok ? rv.col(j) : 0;
                use[t] = ok && cols[t] < limit;
                vals[t] = use[t] ? ldg(vO + rv.gnz(color, j)) : (T)0;
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    T g[RB];
#pragma unroll
                    for (int t = 0; t < RB; t++)
                    {
                        const size_t o = (size_t)c * n + cols[t];
                        g[t] = use[t] ? (T)__ldcg(v0 + o) : (T)0;
                        if (v1 && use[t])
                            g[t] += w[c] * __ldcg(v1 + o);
                    }
#pragma unroll
                    for (int t = 0; t < RB; t++)
                        acc[c] += vals[t] * g[t];
                }
        }
    }

    // LG consecutive lanes of a warp share one row (LG = 1: one thread per row).
    template <int LG>
    struct RowLanes
    {
        int lane, group;
        unsigned mask;
        static constexpr int groups = CTPB / LG;
        __device__ __forceinline__ RowLanes()
        {
            lane = threadIdx.x & (LG - 1);
            group = threadIdx.x / LG;
            const int w = (threadIdx.x & 31) / LG;
            mask = (LG == 32) ? FULL : (((1u << LG) - 1u) << (w * LG));
        }
        // sum over the lanes of the group, valid in every lane (fixed order)
        template <typename T>
        __device__ __forceinline__ T sum(T v) const
        {
#pragma unroll
            for (int o = LG / 2; o > 0; o >>= 1)
                v += __shfl_xor_sync(mask, v, o, LG);
            return v;
        }
    };

    // rowGather for a row shared by LG lanes: lane k takes the entries jb + k, jb + k + LG, ... in
    // predicated batches of 4 (so a row of up to 4 * LG entries has all its loads in flight at
    // once); the caller sums acc over the group.
    template <typename T, typename V0, int NCH, bool SMEM, int LG>
    __device__ __forceinline__ void rowGatherLanes(const RowView<SMEM> & rv, int color, int jb, int je, int limit,
                                                   const T * vO, int n, const V0 * v0, const T * v1, const T * w,
                                                   const bool (&act)[NCH], T (&acc)[NCH], int lane)
    {
        if constexpr (LG == 1)
            rowGather<T, V0, NCH, SMEM>(rv, color, jb, je, limit, vO, n, v0, v1, w, act, acc);
        else
        {
            constexpr int RBL = 4;
            for (int j0 = jb + lane; j0 < je; j0 += RBL * LG)
            {
                int cols[RBL];
                bool use[RBL];
                T vals[RBL];
#pragma unroll
                for (int t = 0; t < RBL; t++)
                {
                    const int j = j0 + t * LG;
                    const bool ok = j < je;
                    cols[t] = ok ? rv.col(j) : 0;
                    use[t] = ok && cols[t] < limit;
                    vals[t] = use[t] ? ldg(vO + rv.gnz(color, j)) : (T)0;
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        T g[RBL];
#pragma unroll
                        for (int t = 0; t < RBL; t++)
                        {
                            const size_t o = (size_t)c * n + cols[t];
                            g[t] = use[t] ? (T)__ldcg(v0 + o) : (T)0;
                            if (v1 && use[t])
                                g[t] += w[c] * __ldcg(v1 + o);
                        }
#pragma unroll
                        for (int t = 0; t < RBL; t++)
                            acc[c] += vals[t] * g[t];
                    }
            }
        }
    }

    // acc[c] += sum over the row's entries of a_j * v[c][col_j], a_j the double-float (vHi, vLo) and
    // v FP32, accumulated as Dot2 (dfDotAdd: exact FMA product residuals, TwoSum of the high parts,
    // errors gathered in acc.y), so the result carries ~48 significant bits computed on the FP32
    // pipes; the caller sums acc.x + acc.y in FP64.  LG lanes share a row as in rowGatherLanes.
    template <int NCH, bool SMEM, int LG>
    __device__ __forceinline__ void rowGatherDf(const RowView<SMEM> & rv, int color, int jb, int je,
                                                const float * vHi, const float * vLo, int n, const float * v,
                                                const bool (&act)[NCH], float2 (&acc)[NCH], int lane)
    {
        constexpr int RBL = LG == 1 ? RB : 4;
        for (int j0 = jb + (LG == 1 ? 0 : lane); j0 < je; j0 += RBL * LG)
        {
            int cols[RBL];
            bool use[RBL];
            float2 a[RBL];
#pragma unroll
            for (int t = 0; t < RBL; t++)
            {
                const int j = j0 + t * LG;
                use[t] = j < je;
                cols[t] = use[t] ? rv.col(j) : 0;
                const int gj = rv.gnz(color, j);
                a[t] = use[t] ? make_float2(__ldg(vHi + gj), __ldg(vLo + gj)) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    float g[RBL];
#pragma unroll
                    for (int t = 0; t < RBL; t++)
                        g[t] = use[t] ? __ldcg(v + (size_t)c * n + cols[t]) : 0.f;
#pragma unroll
                    for (int t = 0; t < RBL; t++)
                        acc[c] = dfDotAdd(acc[c], a[t], make_float2(g[t], 0.f));
                }
        }
    }

    // K per-thread values summed over the CTA in a fixed order; the result is valid in every lane of
    // warp 0.
    template <typename T, int K>
    __device__ __forceinline__ void blockSum(const T (&v)[K], T (&out)[K])
    {
        __shared__ T warpPart[CTPB / 32][K];
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int k = 0; k < K; k++)
        {
            T s = v[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0)
                warpPart[warp][k] = s;
        }
        __syncthreads();
        if (warp == 0)
        {
#pragma unroll
            for (int k = 0; k < K; k++)
            {
                T s = warpPart[lane][k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    s += __shfl_xor_sync(FULL, s, o);
                out[k] = s;
            }
        }
    }

    // One thread-block cluster: hardware cluster barriers; reductions through distributed shared
    // memory (each CTA publishes its block sums in its own shared memory, one warp of every CTA reads
    // all of them after the barrier, lane r <- rank r).
    template <typename T>
    struct ClusterSync
    {
        T (*slot)[8] = nullptr; // two alternating 8-value buffers in the CTA's shared memory
        int buf = 0;
        __device__ __forceinline__ int rank() const { return (int)cg::this_cluster().block_rank(); }
        __device__ __forceinline__ int size() const { return (int)cg::this_cluster().num_blocks(); }
        __device__ __forceinline__ void sync() { cg::this_cluster().sync(); }
        __device__ __forceinline__ bool failed() const { return false; }

        // sum over the cluster of K per-thread values; thread 0 of every CTA runs epi(totals), then
        // the CTA synchronises
        template <int K, typename Epi>
        __device__ __forceinline__ void reduce(const T (&v)[K], Epi && epi)
        {
            cg::cluster_group cl = cg::this_cluster();
            T part[K];
            blockSum<T, K>(v, part);
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            if (warp == 0 && lane == 0)
#pragma unroll
                for (int k = 0; k < K; k++)
                    slot[buf][k] = part[k];
            cl.sync();
            if (warp == 0)
            {
                const int cs = (int)cl.num_blocks();
                const T * remote = cl.map_shared_rank(&slot[buf][0], lane < cs ? lane : 0);
                T tot[K];
#pragma unroll
                for (int k = 0; k < K; k++)
                {
                    T s = lane < cs ? remote[k] : (T)0;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        s += __shfl_xor_sync(FULL, s, o);
                    tot[k] = s;
                }
                if (lane == 0)
                    epi(tot);
            }
            __syncthreads();
            buf ^= 1;
        }

        // no CTA may leave while another can still read its shared memory
        __device__ __forceinline__ void finish() { cg::this_cluster().sync(); }
    };

    __device__ __forceinline__ unsigned ldAcquireGpu(const unsigned * p)
    {
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        return v;
    }

    __device__ __forceinline__ void stReleaseGpu(unsigned * p, unsigned v)
    {
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
    }

    __device__ __forceinline__ unsigned atomAddAcqRelGpu(unsigned * p, unsigned v)
    {
        unsigned old;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
        return old;
    }

    // A cooperative grid (every CTA co-resident): software grid barrier and reductions through
    // global per-CTA slots.  ctl[0] = arrivals, ctl[1] = generation, ctl[2] = abort flag; all zero
    // before the launch.  A wait that polls kGridSpinLimit times without the generation moving sets
    // the abort flag; from then on every barrier returns at once, so the kernel ends (with a
    // failure status) instead of hanging.
    template <typename T>
    struct GridSync
    {
        unsigned * ctl = nullptr;
        T * slots = nullptr; // 2 buffers x 8 values x gridDim.x
        int buf = 0;
        unsigned spinLimit = kGridSpinLimit; // polls of one wait before the barrier gives up
        // Test hook (negative: off): CTA `quietRank` stops arriving at barriers from its
        // `quietAfter`-th barrier on, so that the other CTAs' waits run out.  It waits for nobody
        // either; its loop is bounded like every other CTA's.
        int quietRank = -1;
        unsigned quietAfter = 0;
        unsigned count = 0; // barriers passed by this CTA (per-thread copy, identical in the CTA)
        __device__ __forceinline__ int rank() const { return (int)blockIdx.x; }
        __device__ __forceinline__ int size() const { return (int)gridDim.x; }
        __device__ __forceinline__ bool failed() const { return *(volatile unsigned *)(ctl + 2) != 0u; }

        // The CTA barrier orders every thread's writes before thread 0's arrival, whose release
        // (cumulative) publishes them at GPU scope; the acquire that observes the new generation,
        // followed by the CTA barrier, orders the other CTAs' writes before this CTA's later reads.
        __device__ __forceinline__ void sync()
        {
            __syncthreads();
            const bool quiet = quietRank == (int)blockIdx.x && count >= quietAfter;
            count++;
            if (threadIdx.x == 0 && !quiet && !failed())
            {
                const unsigned gen = ldAcquireGpu(ctl + 1); // read before arriving
                const unsigned prev = atomAddAcqRelGpu(ctl, 1u);
                if (prev == gridDim.x - 1)
                {
                    atomicExch(ctl, 0u);
                    stReleaseGpu(ctl + 1, gen + 1);
                }
                else
                {
                    unsigned polls = 0;
                    while (ldAcquireGpu(ctl + 1) == gen)
                    {
                        if (++polls > spinLimit || failed())
                        {
                            atomicExch(ctl + 2, 1u);
                            break;
                        }
                    }
                }
            }
            __syncthreads();
        }

        template <int K, typename Epi>
        __device__ __forceinline__ void reduce(const T (&v)[K], Epi && epi)
        {
            T part[K];
            blockSum<T, K>(v, part);
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const int G = (int)gridDim.x;
            T * sl = slots + (size_t)buf * 8 * G;
            if (warp == 0 && lane == 0)
#pragma unroll
                for (int k = 0; k < K; k++)
                    sl[k * G + blockIdx.x] = part[k];
            sync();
            if (warp == 0)
            {
                T tot[K];
#pragma unroll
                for (int k = 0; k < K; k++)
                {
                    T s = 0;
                    for (int i = lane; i < G; i += 32)
                        s += __ldcg(sl + k * G + i);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        s += __shfl_xor_sync(FULL, s, o);
                    tot[k] = s;
                }
                if (lane == 0)
                    epi(tot);
            }
            __syncthreads();
            buf ^= 1;
        }

        __device__ __forceinline__ void finish() {}
    };

    // Iteration scalars of a persistent solve, kept by thread 0 of every CTA (all CTAs compute the
    // same values from the same totals) and read by the other threads after a CTA barrier.
    template <typename T, int NCH>
    struct SweepScalars
    {
        T alpha[NCH], beta[NCH];
        int act[NCH], status[NCH], iters[NCH], any;
        double bb[NCH], rr[NCH], rz[NCH], rzPrev[NCH];
    };

    // LG: lanes per row (0: 4 on the grid, 1 in a cluster); TP: the preconditioner's type.
    template <typename T, int NCH, bool SMEM, typename Sync, int LG0 = 0, typename TP = T>
    __global__ void __launch_bounds__(CTPB, 1) kPcgSweep(ClusterPcgArgs<T, TP> A, Sync S)
    {
        extern __shared__ int smemI[];
        __shared__ T slotS[2][8];
        __shared__ int chunkA[MAXCOLORS], chunkL[MAXCOLORS + 1], chunkG[MAXCOLORS], nzBase[MAXCOLORS + 1];
        __shared__ SweepScalars<T, NCH> sc;
        if constexpr (std::is_same<Sync, ClusterSync<T>>::value)
            S.slot = slotS;
        const int rank = S.rank(), cs = S.size();
        SolverState * st = A.st;
        const int n = A.n, C = A.nColors, numCh = A.numCh;
        const int maxIters = st->maxIters;
        if (A.skip && *A.skip)
        {
            if (rank == 0 && threadIdx.x == 0)
                for (int c = 0; c < MAXCH; c++)
                {
                    st->active[c] = 0;
                    st->iters[c] = 0;
                }
            return; // uniform: every CTA reads the same flag before any barrier
        }

        // ---- own rows: chunk `rank` of every color.  Local row l of color c is global row
        // chunkA[c] + (l - chunkL[c]); a color chunk is one contiguous range of the CSR.
        if (threadIdx.x == 0)
        {
            int l = 0, nz = 0;
            for (int c = 0; c < C; c++)
            {
                const int a0 = chunkStart(A.ps, c, rank, cs), a1 = chunkStart(A.ps, c, rank + 1, cs);
                chunkA[c] = a0;
                chunkL[c] = l;
                chunkG[c] = A.rsO[a0];
                nzBase[c] = nz;
                l += a1 - a0;
                nz += A.rsO[a1] - A.rsO[a0];
            }
            chunkL[C] = l;
            nzBase[C] = nz;
        }
        __syncthreads();
        const int R = chunkL[C];
        RowView<SMEM> rv;
        if constexpr (SMEM)
        {
            int * lrs = smemI;
            int * lci = smemI + R + 1;
            for (int c = 0; c < C; c++)
            {
                const int a0 = chunkA[c], nr = chunkL[c + 1] - chunkL[c], cnt = nzBase[c + 1] - nzBase[c];
                for (int t = threadIdx.x; t < nr; t += CTPB)
                    lrs[chunkL[c] + t] = A.rsO[a0 + t] - chunkG[c] + nzBase[c];
                for (int t = threadIdx.x; t < cnt; t += CTPB)
                    lci[nzBase[c] + t] = A.ciO[chunkG[c] + t];
            }
            if (threadIdx.x == 0)
                lrs[R] = nzBase[C];
            __syncthreads();
            rv.lrs = lrs;
            rv.lci = lci;
            rv.chunkA = chunkA;
            rv.chunkL = chunkL;
            rv.chunkG = chunkG;
            rv.nzBase = nzBase;
        }
        else
        {
            rv.rsO = A.rsO;
            rv.ciO = A.ciO;
            rv.chunkA = chunkA;
            rv.chunkL = chunkL;
        }

        bool act[NCH];
        T alpha[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            act[c] = c < numCh;
            alpha[c] = (T)0;
        }

        // rows shared by LG lanes on the grid path (many short phases spread over every SM: one
        // round of gathers per row); one thread per row in a cluster, and on the grid for systems
        // whose colour phases give every thread several rows (more rows, so more loads, in flight)
        constexpr int LG = LG0 > 0 ? LG0 : (std::is_same<Sync, GridSync<T>>::value ? 4 : 1);
        // FP64 recurrence under an FP32 preconditioner: A z from the double-float values (vOP, vOLo)
        constexpr bool DFA = std::is_same<T, double>::value && std::is_same<TP, float>::value;
        const RowLanes<LG> RL;

        // ---- r = b - A x over own rows; ||b||^2
        T bbP[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bbP[c] = (T)0;
        for (int col = 0; col < C; col++)
            for (int l = chunkL[col] + RL.group; l < chunkL[col + 1]; l += RL.groups)
            {
                const int i = chunkA[col] + (l - chunkL[col]);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                rowGatherLanes<T, T, NCH, SMEM, LG>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX, A.vO, n,
                                                    (const T *)A.x, (const T *)nullptr, nullptr, act, acc, RL.lane);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = RL.sum(acc[c]);
                if (RL.lane == 0)
                {
                    const T d = ldg(A.diag + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const T bi = A.b[(size_t)c * n + i];
                            A.r[(size_t)c * n + i] = bi - (d * A.x[(size_t)c * n + i] + acc[c]);
                            bbP[c] += bi * bi;
                        }
                }
            }

        // z = SGS(r) from z = 0.  init: no x / r update.  Forward phases use earlier colors only.
        auto sgs = [&](bool init, const T * pcur, T (&rr)[NCH], T (&rz)[NCH]) {
#pragma unroll
            for (int c = 0; c < NCH; c++)
                rr[c] = rz[c] = (T)0;
            for (int col = 0; col < C; col++)
            {
                const int r0 = A.ps[col];
                for (int l = chunkL[col] + RL.group; l < chunkL[col + 1]; l += RL.groups)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    const int jb = rv.begin(col, l), je = rv.end(col, l);
                    T ri[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        ri[c] = (T)0;
                        if (act[c] && RL.lane == 0)
                        {
                            const size_t o = (size_t)c * n + i;
                            T rvv = A.r[o];
                            if (!init)
                            {
                                A.x[o] = A.x[o] + alpha[c] * pcur[o];
                                rvv -= alpha[c] * A.q[o];
                                A.r[o] = rvv;
                            }
                            ri[c] = rvv;
                        }
                    }
                    TP acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    rowGatherLanes<TP, TP, NCH, SMEM, LG>(rv, col, jb, je, r0, A.vOP, n, (const TP *)A.z,
                                                          (const TP *)nullptr, nullptr, act, acc, RL.lane);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = RL.sum(acc[c]);
                    if (RL.lane == 0)
                    {
                        const TP id = ldg(A.invD + i);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const TP zi = ((TP)ri[c] - acc[c]) * id;
                                A.z[(size_t)c * n + i] = zi;
                                rr[c] += ri[c] * ri[c];
                                if (col == C - 1)
                                    rz[c] += ri[c] * (T)zi;
                            }
                    }
                }
                if (C > 1)
                    S.sync(); // z of this color visible to every CTA
            }
            for (int col = C - 2; col >= 0; col--)
            {
                for (int l = chunkL[col] + RL.group; l < chunkL[col + 1]; l += RL.groups)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    TP acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    rowGatherLanes<TP, TP, NCH, SMEM, LG>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX, A.vOP,
                                                          n, (const TP *)A.z, (const TP *)nullptr, nullptr, act, acc,
                                                          RL.lane);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = RL.sum(acc[c]);
                    if (RL.lane != 0)
                        continue;
                    const TP id = ldg(A.invD + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            const T rvv = A.r[o];
                            const TP zi = ((TP)rvv - acc[c]) * id;
                            A.z[o] = zi;
                            rz[c] += rvv * (T)zi;
                        }
                }
                if (col > 0)
                    S.sync(); // the last phase's barrier is the reduction's
            }
        };

        T rr0[NCH], rz0[NCH];
        sgs(true, A.p, rr0, rz0);
        T red[3 * NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            red[c] = bbP[c];
            red[NCH + c] = rr0[c];
            red[2 * NCH + c] = rz0[c];
        }
        const int absMode = st->absMode;
        const double tol2 = st->tol2;
        // scalar decisions: thread 0 of each CTA, FP64 (identical in every CTA)
        S.template reduce<3 * NCH>(red, [&](const T (&tot)[3 * NCH]) {
            int any = 0;
            for (int c = 0; c < NCH; c++)
            {
                const double bb = (double)tot[c], rr = (double)tot[NCH + c], rz = (double)tot[2 * NCH + c];
                sc.bb[c] = bb;
                sc.rr[c] = rr;
                sc.rz[c] = rz;
                sc.rzPrev[c] = rz;
                const bool fin = isfinite(rr) && isfinite(bb);
                const bool conv = absMode ? (rr < tol2) : (rr <= tol2 * bb);
                sc.status[c] = fin ? 0 : 2;
                sc.iters[c] = 0;
                sc.act[c] = (c < numCh) && fin && !conv;
                sc.alpha[c] = (T)0;
                sc.beta[c] = (T)0;
                any |= sc.act[c];
            }
            sc.any = any;
        });
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = sc.act[c] != 0;

        int k = 1;
        for (; k <= maxIters; k++)
        {
            if (!sc.any)
                break; // same value in every CTA
            // direction: p = z + beta p ; q = A z + beta q (= A p, the previous q being A p_old) ; p.q
            // over own rows of every color.  Only z is gathered, one product per entry.
            T beta[NCH], pq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                beta[c] = sc.beta[c];
                pq[c] = (T)0;
            }
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + RL.group; l < chunkL[col + 1]; l += RL.groups)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    if constexpr (DFA)
                    {
                        float2 accDf[NCH];
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            accDf[c] = make_float2(0.f, 0.f);
                        rowGatherDf<NCH, SMEM, LG>(rv, col, rv.begin(col, l), rv.end(col, l),
                                                   (const float *)A.vOP, A.vOLo, n, (const float *)A.z, act, accDf,
                                                   RL.lane);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            acc[c] = (T)accDf[c].x + (T)accDf[c].y;
                    }
                    else
                        rowGatherLanes<T, TP, NCH, SMEM, LG>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX,
                                                             A.vO, n, (const TP *)A.z, (const T *)nullptr, nullptr,
                                                             act, acc, RL.lane);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = RL.sum(acc[c]);
                    if (RL.lane == 0)
                    {
                        const T d = ldg(A.diag + i);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const size_t o = (size_t)c * n + i;
                                const T zi = (T)A.z[o];
                                T pn = zi, qi = d * zi + acc[c];
                                if (k > 1)
                                {
                                    pn += beta[c] * A.p[o];
                                    qi += beta[c] * A.q[o];
                                }
                                A.p[o] = pn;
                                A.q[o] = qi;
                                pq[c] += pn * qi;
                            }
                    }
                }
            S.template reduce<NCH>(pq, [&](const T (&tot)[NCH]) {
                for (int c = 0; c < NCH; c++)
                {
                    const double pqc = (double)tot[c];
                    sc.rzPrev[c] = sc.rz[c]; // defines this alpha; the previous r.z of the next beta
                    sc.alpha[c] = (T)(sc.rz[c] / pqc);
                    if (sc.act[c] && !(pqc > 0))
                    {
                        sc.status[c] = isfinite(pqc) ? 4 : 2;
                        sc.iters[c] = k - 1;
                        sc.act[c] = 0;
                    }
                }
            });
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                alpha[c] = sc.alpha[c];
                act[c] = sc.act[c] != 0;
            }
            T rrN[NCH], rzN[NCH];
            sgs(false, A.p, rrN, rzN);
            T red2[2 * NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                red2[c] = rrN[c];
                red2[NCH + c] = rzN[c];
            }
            S.template reduce<2 * NCH>(red2, [&](const T (&tot)[2 * NCH]) {
                int any = 0;
                for (int c = 0; c < NCH; c++)
                {
                    if (sc.act[c])
                    {
                        const double rr = (double)tot[c], rz = (double)tot[NCH + c];
                        sc.rr[c] = rr;
                        sc.rz[c] = rz;
                        const bool fin = isfinite(rr) && isfinite(rz);
                        const bool conv = absMode ? (rr < tol2) : (rr <= tol2 * sc.bb[c]);
                        if (!fin || conv)
                        {
                            sc.act[c] = 0;
                            sc.iters[c] = k;
                            sc.status[c] = fin ? 0 : 2;
                        }
                        else
                            sc.beta[c] = (T)(rz / sc.rzPrev[c]);
                    }
                    any |= sc.act[c];
                }
                sc.any = any && !S.failed();
            });
#pragma unroll
            for (int c = 0; c < NCH; c++)
                act[c] = sc.act[c] != 0;
        }
        // results (rank 0 writes; every CTA holds identical values)
        if (rank == 0 && threadIdx.x == 0)
        {
            const bool failed = S.failed();
            for (int c = 0; c < NCH; c++)
            {
                if (sc.act[c])
                {
                    sc.status[c] = 3;
                    sc.iters[c] = maxIters;
                }
                if (failed && c < numCh)
                    sc.status[c] = 5; // a grid barrier gave up waiting: results are not valid
                st->status[c] = c < numCh ? sc.status[c] : 0;
                st->iters[c] = sc.iters[c];
                st->bb[c] = sc.bb[c];
                st->lastRR[c] = sc.rr[c];
                st->active[c] = 0;
            }
            st->iter = k;
            st->anyActive = 0;
        }
        S.finish();
    }

    // Largest cluster (16, else 8, else 0 = unavailable) the device can co-schedule for kernel k
    // with CTPB threads per CTA and `smem` bytes of dynamic shared memory per CTA.
    template <typename K>
    inline int pickClusterSize(K kernel, size_t smemFor16, size_t smemFor8)
    {
        for (int cs : {16, 8})
        {
            const size_t smem = cs == 16 ? smemFor16 : smemFor8;
            if (smem > kClusterSmemCap)
                continue;
            // a fixed ceiling: solvers of different sizes share this kernel instantiation
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmemCap) !=
                cudaSuccess)
            {
                cudaGetLastError();
                continue;
            }
            if (cs > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
            {
                cudaGetLastError();
                continue;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(CTPB);
            cfg.dynamicSmemBytes = smem;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int num = 0;
            if (cudaOccupancyMaxActiveClusters(&num, kernel, &cfg) == cudaSuccess && num >= 1)
                return cs;
            cudaGetLastError();
        }
        return 0;
    }

    // Whether a cooperative grid of one CTA per SM with `smem` bytes of dynamic shared memory can be
    // co-resident (1 = yes).  Sets the kernel's dynamic shared memory ceiling to kClusterSmemCap.
    template <typename K>
    inline bool gridFits(K kernel, size_t smem)
    {
        int dev = 0, coop = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
            smem > kClusterSmemCap ||
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmemCap) !=
                cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, CTPB, smem) != cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
        return nb >= 1;
    }
} // namespace nsf
