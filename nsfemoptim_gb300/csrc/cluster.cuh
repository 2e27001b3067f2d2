// Cluster-resident CG with the multicolor symmetric Gauss-Seidel preconditioner.
//
// One launch per solve: a single thread-block cluster of CS CTAs (16 where the GPU allows
// non-portable clusters, else 8) x 1024 threads runs the whole iteration loop.  CTA k owns chunk k
// of every color block, so x, r and q are only touched by their owner; z and p are read at
// neighbour rows of other CTAs through L2 (ld.global.cg).  Every color phase ends in a hardware
// cluster barrier (barrier.cluster arrive.release / wait.acquire) instead of a kernel boundary,
// and the dot products are cluster reductions: each CTA writes its block sum into its own shared
// memory, and after the barrier every CTA reads the CS sums through distributed shared memory in
// rank order, so all CTAs hold bit-identical scalars and take identical loop decisions (the
// barrier count can never diverge).  The loop is bounded by maxIters.
//
// The state (tolerance, cap, mode) is read from the SolverState written by a preceding kernel,
// so the FP64 refinement loop can set the inner tolerance on the device.
#pragma once

#include <cooperative_groups.h>

#include "kernels.cuh"

namespace nsf
{
    namespace cg = cooperative_groups;

    constexpr int CTPB = 1024; // threads per CTA of the cluster solver

    template <typename T>
    struct ClusterPcgArgs
    {
        int n, nColors, numCh;
        const int * ps;                  // color starts (device), nColors + 1
        const int *rsF, *ciF;            // full matrix
        const T * vF;
        const int *rsO, *ciO;            // off-diagonal part
        const T * vO;
        const T * invD;
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
        if (threadIdx.x < K)
        {
            double s = 0;
            for (int w = 0; w < CTPB / 32; w++)
                s += warpPart[w][threadIdx.x];
            slot[buf][threadIdx.x] = s;
        }
        cl.sync();
        if (threadIdx.x < K)
        {
            double s = 0;
            const int cs = (int)cl.num_blocks();
            for (int rk = 0; rk < cs; rk++)
                s += cl.map_shared_rank(&slot[buf][0], rk)[threadIdx.x];
            total[threadIdx.x] = s;
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

    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(CTPB, 1) kPcgCluster(ClusterPcgArgs<T> A)
    {
        cg::cluster_group cl = cg::this_cluster();
        const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
        __shared__ double slot[2][8];
        int buf = 0;
        SolverState * st = A.st;
        const int n = A.n, C = A.nColors;
        const int maxIters = st->maxIters, absMode = st->absMode;
        const double tol2 = st->tol2;
        const bool skipAll = A.skip && *A.skip;
        if (skipAll)
        {
            if (rank == 0 && threadIdx.x == 0)
                for (int c = 0; c < MAXCH; c++)
                {
                    st->active[c] = 0;
                    st->iters[c] = 0;
                }
            return; // uniform: every CTA reads the same flag
        }
        const int lane = threadIdx.x & (L - 1);
        const int grp = threadIdx.x / L, ngrp = CTPB / L;
        const unsigned mask = (L == 32) ? FULL : (((1u << L) - 1u) << (((threadIdx.x & 31) / L) * L));
        auto gsum = [&](double v) {
#pragma unroll
            for (int o = L / 2; o > 0; o >>= 1)
                v += __shfl_down_sync(mask, v, o, L);
            return v;
        };

        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < A.numCh;

        // ---- r = b - A x over own rows; ||b||^2
        double bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        for (int col = 0; col < C; col++)
        {
            const int a0 = chunkStart(A.ps, col, rank, cs), a1 = chunkStart(A.ps, col, rank + 1, cs);
            for (int i = a0 + grp; i < a1; i += ngrp)
            {
                const int s = ldg(A.rsF + i), e = ldg(A.rsF + i + 1);
                double acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + lane; j < e; j += L)
                {
                    const double a = (double)ldg(A.vF + j);
                    const int cj = ldg(A.ciF + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] += a * (double)A.x[(size_t)c * n + cj];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const double t = gsum(acc[c]);
                    if (lane == 0)
                    {
                        const double bi = (double)A.b[(size_t)c * n + i];
                        A.r[(size_t)c * n + i] = (T)(bi - t);
                        bb[c] += bi * bi;
                    }
                }
            }
        }

        // ---- z = SGS(r); rr and rz.  init: no x/r update
        double alpha[NCH] = {};
        auto sgs = [&](bool init, const T * pcur, double (&rr)[NCH], double (&rz)[NCH]) {
#pragma unroll
            for (int c = 0; c < NCH; c++)
                rr[c] = rz[c] = 0;
            for (int col = 0; col < C; col++)
            {
                const int r0 = A.ps[col];
                const int a0 = chunkStart(A.ps, col, rank, cs), a1 = chunkStart(A.ps, col, rank + 1, cs);
                for (int i = a0 + grp; i < a1; i += ngrp)
                {
                    double ri[NCH];
                    if (lane == 0)
                    {
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const size_t o = (size_t)c * n + i;
                                double rv = (double)A.r[o];
                                if (!init)
                                {
                                    A.x[o] = (T)((double)A.x[o] + alpha[c] * (double)pcur[o]);
                                    rv -= alpha[c] * (double)A.q[o];
                                    A.r[o] = (T)rv;
                                }
                                ri[c] = (double)(T)rv;
                            }
                    }
                    const int s = ldg(A.rsO + i), e = ldg(A.rsO + i + 1);
                    double acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    for (int j = s + lane; j < e; j += L)
                    {
                        const int cj = ldg(A.ciO + j);
                        if (cj >= r0)
                            break; // later colors: still zero in the forward sweep
                        const double a = (double)ldg(A.vO + j);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                                acc[c] += a * (double)__ldcg(A.z + (size_t)c * n + cj);
                    }
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        const double t = gsum(acc[c]);
                        if (lane == 0 && act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            const T zi = (T)((ri[c] - t) * (double)ldg(A.invD + i));
                            A.z[o] = zi;
                            rr[c] += ri[c] * ri[c];
                            if (col == C - 1)
                                rz[c] += ri[c] * (double)zi;
                        }
                    }
                }
                if (C > 1)
                    cl.sync(); // z of this color visible to the cluster
            }
            for (int col = C - 2; col >= 0; col--)
            {
                const int a0 = chunkStart(A.ps, col, rank, cs), a1 = chunkStart(A.ps, col, rank + 1, cs);
                for (int i = a0 + grp; i < a1; i += ngrp)
                {
                    const int s = ldg(A.rsO + i), e = ldg(A.rsO + i + 1);
                    double acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    for (int j = s + lane; j < e; j += L)
                    {
                        const double a = (double)ldg(A.vO + j);
                        const int cj = ldg(A.ciO + j);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                                acc[c] += a * (double)__ldcg(A.z + (size_t)c * n + cj);
                    }
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        const double t = gsum(acc[c]);
                        if (lane == 0 && act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            const double rv = (double)A.r[o];
                            const T zi = (T)((rv - t) * (double)ldg(A.invD + i));
                            A.z[o] = zi;
                            rz[c] += rv * (double)zi;
                        }
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
            double beta[NCH], pq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                beta[c] = (k == 1) ? 0.0 : rzT[c] / rzPrev[c];
                pq[c] = 0;
            }
            for (int col = 0; col < C; col++)
            {
                const int a0 = chunkStart(A.ps, col, rank, cs), a1 = chunkStart(A.ps, col, rank + 1, cs);
                for (int i = a0 + grp; i < a1; i += ngrp)
                {
                    const int s = ldg(A.rsF + i), e = ldg(A.rsF + i + 1);
                    double acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = 0;
                    for (int j = s + lane; j < e; j += L)
                    {
                        const double a = (double)ldg(A.vF + j);
                        const int cj = ldg(A.ciF + j);
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const size_t o = (size_t)c * n + cj;
                                const double zz = (double)__ldcg(A.z + o);
                                acc[c] += a * (k == 1 ? zz : zz + beta[c] * (double)__ldcg(pold + o));
                            }
                    }
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        const double t = gsum(acc[c]);
                        if (lane == 0 && act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            const double zz = (double)A.z[o];
                            const T pn = (T)(k == 1 ? zz : zz + beta[c] * (double)pold[o]);
                            pnew[o] = pn;
                            A.q[o] = (T)t;
                            pq[c] += (double)pn * t;
                        }
                    }
                }
            }
            double pqT[NCH];
            clusterSum<NCH>(cl, pq, slot, buf, pqT);
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                rzPrev[c] = rzT[c]; // defines this alpha; the previous r.z of the next beta
                alpha[c] = rzT[c] / pqT[c];
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
    // with CTPB threads per CTA.
    template <typename K>
    inline int pickClusterSize(K kernel)
    {
        for (int cs : {16, 8})
        {
            if (cs > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
            {
                cudaGetLastError();
                continue;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(cs);
            cfg.blockDim = dim3(CTPB);
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
