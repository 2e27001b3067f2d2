// Cluster-resident CG with the multicolor symmetric Gauss-Seidel preconditioner.
//
// One launch per solve: a single thread-block cluster of CS CTAs (16 where the GPU allows
// non-portable clusters, else 8) x 1024 threads runs the whole iteration loop.  CTA k owns chunk k
// of every color block, so x, r and q are only touched by their owner; z and p are read at
// neighbour rows of other CTAs through L2 (ld.global.cg).
//
// Measured on the GB300: a cluster barrier costs 0.3 us and a dependent L2 load ~150 ns, while a
// kernel boundary with a grid reduction costs >= 3 us.  The kernel is therefore organised for one
// L2 round trip per color phase:
//   * one thread per row; the entries of a row are processed in fixed-width predicated batches so
//     all value loads and neighbour gathers of a row are in flight together;
//   * when the structure of a CTA's rows (row offsets, column indices of the off-diagonal part)
//     fits in shared memory it is copied there at kernel start (SMEM = true), else it is read from
//     global memory (the large mass matrix);
//   * phases end in a hardware cluster barrier; dot products are cluster reductions: each CTA writes
//     its block sum into its own shared memory, after the barrier one warp reads the CS sums
//     through distributed shared memory in parallel (lane r <- rank r) and adds them with a fixed
//     shuffle tree, so all CTAs hold bit-identical scalars and take identical loop decisions (the
//     barrier count can never diverge).  The loop is bounded by the iteration cap.
//
// Tolerance, cap and mode are read from the SolverState written by a preceding kernel, so the FP64
// refinement loop can set the inner tolerance on the device.
#pragma once

#include <cooperative_groups.h>

#include <climits>
#include <vector>

#include "kernels.cuh"

namespace nsf
{
    namespace cg = cooperative_groups;

    constexpr int CTPB = 1024;                    // threads per CTA of the cluster solver
    constexpr size_t kClusterSmemCap = 200 * 1024; // dynamic shared memory ceiling per CTA
    constexpr int RB = 8;                          // entries per predicated batch of a row

    template <typename T>
    struct ClusterPcgArgs
    {
        int n, nColors, numCh;
        const int * ps;                  // color starts (device), nColors + 1
        const int *rsO, *ciO;            // off-diagonal part
        const T * vO;
        const T * diag;                  // diagonal values
        const T * invD;                  // their inverses
        const T * b;
        T *x, *r, *z, *p, *q;            // p holds two planes (ping-pong) of NCH * n
        SolverState * st;
        const int * skip;                // refinement: stop immediately when *skip != 0
    };

    // sum over the cluster of K values per thread; every thread of every CTA gets the totals
    template <int K>
    __device__ __forceinline__ void clusterSum(cg::cluster_group & cl, const double (&v)[K], double (*slot)[8],
                                               int & buf, double (&out)[K])
    {
        __shared__ double warpPart[CTPB / 32][K];
        __shared__ double total[K];
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int k = 0; k < K; k++)
        {
            double s = v[k];
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
                double s = warpPart[lane][k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    s += __shfl_xor_sync(FULL, s, o);
                if (lane == 0)
                    slot[buf][k] = s;
            }
        }
        cl.sync();
        if (warp == 0)
        {
            const int cs = (int)cl.num_blocks();
            double rv[K];
            const double * remote = cl.map_shared_rank(&slot[buf][0], lane < cs ? lane : 0);
#pragma unroll
            for (int k = 0; k < K; k++)
                rv[k] = lane < cs ? remote[k] : 0.0;
#pragma unroll
            for (int k = 0; k < K; k++)
            {
                double s = rv[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    s += __shfl_xor_sync(FULL, s, o);
                if (lane == 0)
                    total[k] = s;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < K; k++)
            out[k] = total[k];
        buf ^= 1;
    }

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
    // (v1 may be null).  Arithmetic in T (FP32 in the inner solver: GB300's FP64 rate is ~1/64 of
    // FP32); fixed-width predicated batches keep RB loads in flight per thread.
    template <typename T, int NCH, bool SMEM>
    __device__ __forceinline__ void rowGather(const RowView<SMEM> & rv, int color, int jb, int je, int limit,
                                              const T * vO, int n, const T * v0, const T * v1, const T * w,
                                              const bool (&act)[NCH], T (&acc)[NCH])
    {
        for (int j0 = jb; j0 < je; j0 += RB)
        {
            int cols[RB];
            T vals[RB];
#pragma unroll
            for (int t = 0; t < RB; t++)
            {
                const int j = j0 + t;
                const bool ok = j < je;
                cols[t] = ok ? rv.col(j) : 0;
                vals[t] = (ok && cols[t] < limit) ? ldg(vO + rv.gnz(color, j)) : (T)0;
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
                        g[t] = vals[t] != (T)0 ? __ldcg(v0 + o) : (T)0;
                        if (v1 && vals[t] != (T)0)
                            g[t] += w[c] * __ldcg(v1 + o);
                    }
#pragma unroll
                    for (int t = 0; t < RB; t++)
                        acc[c] += vals[t] * g[t];
                }
        }
    }

    template <typename T, int NCH, bool SMEM>
    __global__ void __launch_bounds__(CTPB, 1) kPcgCluster(ClusterPcgArgs<T> A)
    {
        extern __shared__ int smemI[];
        cg::cluster_group cl = cg::this_cluster();
        const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
        __shared__ double slot[2][8];
        __shared__ int chunkA[MAXCOLORS], chunkL[MAXCOLORS + 1], chunkG[MAXCOLORS], nzBase[MAXCOLORS + 1];
        int buf = 0;
        SolverState * st = A.st;
        const int n = A.n, C = A.nColors;
        const int maxIters = st->maxIters, absMode = st->absMode;
        const double tol2 = st->tol2;
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
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < A.numCh;

        // ---- r = b - A x over own rows; ||b||^2 (dot products accumulate in FP64)
        double bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        for (int col = 0; col < C; col++)
            for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += CTPB)
            {
                const int i = chunkA[col] + (l - chunkL[col]);
                const T d = ldg(A.diag + i);
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = d * A.x[(size_t)c * n + i];
                rowGather<T, NCH, SMEM>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX, A.vO, n, A.x,
                                        (const T *)nullptr, nullptr, act, acc);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        const T bi = A.b[(size_t)c * n + i];
                        A.r[(size_t)c * n + i] = bi - acc[c];
                        bb[c] += (double)(bi * bi);
                    }
            }

        T alphaT[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            alphaT[c] = 0;
        // z = SGS(r); init: no x/r update.  Forward phases use earlier colors only (limit).
        auto sgs = [&](bool init, const T * pcur, double (&rr)[NCH], double (&rz)[NCH]) {
#pragma unroll
            for (int c = 0; c < NCH; c++)
                rr[c] = rz[c] = 0;
            for (int col = 0; col < C; col++)
            {
                const int r0 = A.ps[col];
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += CTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    const int jb = rv.begin(col, l), je = rv.end(col, l);
                    T ri[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            T rvv = A.r[o];
                            if (!init)
                            {
                                A.x[o] = A.x[o] + alphaT[c] * pcur[o];
                                rvv -= alphaT[c] * A.q[o];
                                A.r[o] = rvv;
                            }
                            ri[c] = rvv;
                        }
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    rowGather<T, NCH, SMEM>(rv, col, jb, je, r0, A.vO, n, A.z, (const T *)nullptr, nullptr, act, acc);
                    const T id = ldg(A.invD + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const T zi = (ri[c] - acc[c]) * id;
                            A.z[(size_t)c * n + i] = zi;
                            rr[c] += (double)(ri[c] * ri[c]);
                            if (col == C - 1)
                                rz[c] += (double)(ri[c] * zi);
                        }
                }
                if (C > 1)
                    cl.sync(); // z of this color visible to the cluster
            }
            for (int col = C - 2; col >= 0; col--)
            {
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += CTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    rowGather<T, NCH, SMEM>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX, A.vO, n, A.z,
                                            (const T *)nullptr, nullptr, act, acc);
                    const T id = ldg(A.invD + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            const T rvv = A.r[o];
                            const T zi = (rvv - acc[c]) * id;
                            A.z[o] = zi;
                            rz[c] += (double)(rvv * zi);
                        }
                }
                if (col > 0)
                    cl.sync(); // the last phase's barrier is the reduction's
            }
        };

        double rr[NCH], rz[NCH], rzPrev[NCH];
        sgs(true, A.p, rr, rz);
        double red[3 * NCH], tot[3 * NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            red[c] = bb[c];
            red[NCH + c] = rr[c];
            red[2 * NCH + c] = rz[c];
        }
        clusterSum<3 * NCH>(cl, red, slot, buf, tot);
        double bbT[NCH], rrT[NCH], rzT[NCH];
        int status[NCH], iters[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            bbT[c] = tot[c];
            rrT[c] = tot[NCH + c];
            rzT[c] = tot[2 * NCH + c];
            rzPrev[c] = rzT[c];
            const bool fin = isfinite(rrT[c]) && isfinite(bbT[c]);
            const bool conv = absMode ? (rrT[c] < tol2) : (rrT[c] <= tol2 * bbT[c]);
            status[c] = fin ? 0 : 2;
            iters[c] = 0;
            act[c] = act[c] && fin && !conv;
        }

        int k = 1;
        for (; k <= maxIters; k++)
        {
            bool any = false;
#pragma unroll
            for (int c = 0; c < NCH; c++)
                any |= act[c];
            if (!any)
                break;
            // direction: p_new = z + beta p_old ; q = A p_new ; p.q   (own rows of every color)
            const T * pold = A.p + (size_t)((k - 1) & 1) * NCH * n;
            T * pnew = A.p + (size_t)(k & 1) * NCH * n;
            T betaT[NCH];
            double pq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                betaT[c] = (k == 1) ? (T)0 : (T)(rzT[c] / rzPrev[c]);
                pq[c] = 0;
            }
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += CTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    const T d = ldg(A.diag + i);
                    T pn[NCH], acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        const size_t o = (size_t)c * n + i;
                        pn[c] = act[c] ? (k == 1 ? A.z[o] : A.z[o] + betaT[c] * pold[o]) : (T)0;
                        acc[c] = d * pn[c];
                    }
                    rowGather<T, NCH, SMEM>(rv, col, rv.begin(col, l), rv.end(col, l), INT_MAX, A.vO, n, A.z,
                                            k == 1 ? (const T *)nullptr : pold, betaT, act, acc);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            pnew[o] = pn[c];
                            A.q[o] = acc[c];
                            pq[c] += (double)(pn[c] * acc[c]);
                        }
                }
            double pqT[NCH];
            clusterSum<NCH>(cl, pq, slot, buf, pqT);
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                rzPrev[c] = rzT[c]; // defines this alpha; the previous r.z of the next beta
                alphaT[c] = (T)(rzT[c] / pqT[c]);
                if (act[c] && !(pqT[c] > 0))
                {
                    status[c] = isfinite(pqT[c]) ? 4 : 2;
                    iters[c] = k - 1;
                    act[c] = false;
                }
            }
            double rrN[NCH], rzN[NCH];
            sgs(false, pnew, rrN, rzN);
            double red2[2 * NCH], tot2[2 * NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                red2[c] = rrN[c];
                red2[NCH + c] = rzN[c];
            }
            clusterSum<2 * NCH>(cl, red2, slot, buf, tot2);
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                if (!act[c])
                    continue;
                rrT[c] = tot2[c];
                rzT[c] = tot2[NCH + c];
                const bool fin = isfinite(rrT[c]) && isfinite(rzT[c]);
                const bool conv = absMode ? (rrT[c] < tol2) : (rrT[c] <= tol2 * bbT[c]);
                if (!fin || conv)
                {
                    act[c] = false;
                    iters[c] = k;
                    status[c] = fin ? 0 : 2;
                }
            }
        }
        // results (rank 0 writes; every CTA holds identical values)
        if (rank == 0 && threadIdx.x == 0)
        {
            for (int c = 0; c < NCH; c++)
            {
                if (act[c])
                {
                    status[c] = 3;
                    iters[c] = maxIters;
                }
                st->status[c] = c < A.numCh ? status[c] : 0;
                st->iters[c] = iters[c];
                st->bb[c] = bbT[c];
                st->lastRR[c] = rrT[c];
                st->active[c] = 0;
            }
            st->iter = k;
            st->anyActive = 0;
        }
        // no CTA may leave while another can still read its shared memory
        cl.sync();
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
} // namespace nsf
