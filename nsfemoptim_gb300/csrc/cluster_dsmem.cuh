// Cluster-resident CG with the multicolor symmetric Gauss-Seidel preconditioner, every vector in
// distributed shared memory.
//
// The variant of the cluster solver for systems whose per-CTA share of the vectors and of the row
// structure fits in shared memory (the pressure Laplacian of the channel meshes).  One thread-block
// cluster of CS CTAs x 1024 threads runs the whole solve; CTA k owns chunk k of every color block.
//   * All CG vectors of a CTA's rows (x, r, q, z, both planes of p) and the diagonal and its
//     inverse live in that CTA's shared memory.  Every CTA uses the same byte layout.
//   * At kernel start the column index of every off-diagonal entry is replaced by the
//     shared::cluster address of that column's z entry in the CTA that owns the column (mapa).
//     The other vectors sit at fixed byte offsets from z in every CTA, so a neighbour gather of any
//     vector is one shared-memory load of the address plus one ld.shared::cluster.
//   * Inside the iteration loop global memory is touched only for the matrix values when they do
//     not fit (VALS = false); x is read at the start and written back at the end.
//   * Row arithmetic and per-thread partial dot products are in T; warp partials are promoted to
//     FP64 and summed across warps and CTAs in a fixed order, so every CTA holds bit-identical
//     scalars and takes the same loop decisions.  (FP64 instructions run at ~1/64 of the FP32 rate
//     on this GPU, so FP64 work is kept to one warp per reduction.)
//   * Phases end in cluster barriers (barrier.cluster arrive.release / wait.acquire), which order
//     the shared-memory stores of one phase before the remote loads of the next.
#pragma once

#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "cluster.cuh"
#include "kernels.cuh"

#ifndef NSF_DS_TPB
#define NSF_DS_TPB 1024
#endif
#ifndef NSF_DS_RB
#define NSF_DS_RB 4 // measured: 4 beats 8 by ~6% per iteration on the pressure system (rows of ~6 entries)
#endif
#ifndef NSF_DS_EXACT
#define NSF_DS_EXACT 0
#endif

namespace nsf
{
    constexpr int DTPB = NSF_DS_TPB; // threads per CTA
    constexpr int DRB = NSF_DS_RB;   // entries per predicated gather batch of a row

    // Byte layout of the dynamic shared memory of one CTA (identical in every CTA of the cluster).
    struct DsLayout
    {
        int stride;                     // elements per vector plane (largest CTA share, rounded up)
        unsigned offZ, offP, offX, offR, offQ, offInvD, offDiag, offRs, offAd, offV, bytes;
        // coarse correction (nAgg > 0): the corrected z (ZF), the CTA's aggregate sums (COwn), every
        // aggregate's sum (CAll), the CTA's coarse values (YOwn), its rows of the coarse inverse
        // (Ainv, aggMax x nAgg) and each local row's aggregate within the CTA (AggL)
        int nAgg, aggMax;
        unsigned offZF, offCOwn, offCAll, offYOwn, offAinv, offAggL;
    };

    inline size_t dsAlign(size_t b) { return (b + 15) & ~(size_t)15; }

    // rows / off-diagonal entries of the largest CTA share; tsize = sizeof(T); vals: values cached too
    inline DsLayout dsLayout(int rowsMax, int nzMax, int nch, int tsize, bool vals, int nAgg = 0, int aggMax = 0)
    {
        DsLayout L{};
        L.stride = (rowsMax + 3) & ~3;
        const size_t plane = (size_t)L.stride * tsize;
        size_t o = 0;
        L.offZ = (unsigned)o;
        o += dsAlign(plane * nch);
        L.offP = (unsigned)o;
        o += dsAlign(plane * nch * 2);
        L.offX = (unsigned)o;
        o += dsAlign(plane * nch);
        L.offR = (unsigned)o;
        o += dsAlign(plane * nch);
        L.offQ = (unsigned)o;
        o += dsAlign(plane * nch);
        L.offInvD = (unsigned)o;
        o += dsAlign(plane);
        L.offDiag = (unsigned)o;
        o += dsAlign(plane);
        L.offRs = (unsigned)o; // packed row starts: local entry offset | (lower-color entries << 24)
        o += dsAlign((size_t)4 * (rowsMax + 1));
        L.offAd = (unsigned)o; // shared::cluster addresses of the z entries of the columns
        o += dsAlign((size_t)4 * nzMax);
        L.offV = (unsigned)o;
        if (vals)
            o += dsAlign((size_t)tsize * nzMax);
        L.nAgg = nAgg;
        L.aggMax = aggMax;
        if (nAgg > 0)
        {
            L.offZF = (unsigned)o;
            o += dsAlign(plane * nch);
            L.offCOwn = (unsigned)o;
            o += dsAlign((size_t)tsize * aggMax);
            L.offCAll = (unsigned)o;
            o += dsAlign((size_t)tsize * nAgg);
            L.offYOwn = (unsigned)o;
            o += dsAlign((size_t)tsize * aggMax);
            L.offAinv = (unsigned)o;
            o += dsAlign((size_t)tsize * aggMax * nAgg);
            L.offAggL = (unsigned)o;
            o += dsAlign((size_t)4 * rowsMax);
        }
        L.bytes = (unsigned)o;
        return L;
    }

    template <typename T>
    struct DsPcgArgs
    {
        int n, nColors, numCh;
        const int * ps;    // color starts, nColors + 1
        const int * rsO;   // off-diagonal part: row offsets, column indices, values
        const int * ciO;
        const T * vO;
        const int * cmap;  // per off-diagonal entry: owner rank << 24 | local row in the owner
        const T * diag;
        const T * invD;
        const T * b;
        T * x;
        SolverState * st;
        const int * skip;
        DsLayout lay;
        // FP64 residual replacement ("reliable updates", T = float only): when ru != 0 the solve is
        // of the FP64 system (values vO64 / diag64 on the same structure) for the FP64 right-hand
        // side b64 and in/out solution x64; the FP32 CG accumulates its increment in shared memory
        // and, whenever the iterated ||r||^2 has dropped by ruDelta2 since the last replacement (or
        // met the tolerance), adds it into x64 and replaces r by b64 - A64 x64 computed in FP64.
        // The solve stops on the FP64 residual.  b and x are unused then.
        int ru;
        double ruDelta2;
        const double * b64;
        const double * vO64;
        const double * diag64;
        double * x64;
        // coarse correction (kernel template CO): z = SGS(r) + P Ac^-1 P^T r over aggregates of
        // rows owned by one CTA each; aggStart[rank] .. aggStart[rank + 1] are the CTA's aggregates,
        // aggOfRow the aggregate of each row (permuted numbering), aggRowStart / aggRows each
        // aggregate's local rows in its CTA, ainv the coarse inverse (nAgg x nAgg, row-major)
        const int * aggStart;
        const int * aggOfRow;
        const int * aggRowStart;
        const int * aggRows;
        const T * ainv;
        // batched instances (one cluster each, launchClusters): the system of instance q, its
        // vectors (b, x, b64, x64) at q * instStride and its state at st + q
        long long instStride;
    };

    __device__ __forceinline__ unsigned dsMapa(unsigned localAddr, int rank)
    {
        unsigned r;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(localAddr), "r"(rank));
        return r;
    }

    __device__ __forceinline__ float dsLoad(unsigned a, float)
    {
        float v;
        asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a));
        return v;
    }

    __device__ __forceinline__ double dsLoad(unsigned a, double)
    {
        double v;
        asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
        return v;
    }

    // acc[c] += sum over local entries [jb, je) of a_j * (V0[c][col_j] + w[c] * V1[c][col_j]), the
    // vectors at byte offsets off0 / off1 from z in the owner CTA (V1 only when TWO).
    template <typename T, int NCH, bool VALS, bool TWO>
    __device__ __forceinline__ void dsGather(const unsigned * lad, const T * lv, const T * vOg, int jb, int je,
                                             unsigned off0, unsigned off1, unsigned chBytes, const T (&w)[NCH],
                                             const bool (&act)[NCH], T (&acc)[NCH])
    {
#if NSF_DS_EXACT
        // exact-length batches: full DRB-wide batches, then one batch of the remaining count
        // (dispatched to a fixed width), no per-entry predicates
        auto batch = [&](int j0, auto width) {
            constexpr int N = decltype(width)::value;
            unsigned ad[N];
            T v[N];
#pragma unroll
            for (int t = 0; t < N; t++)
            {
                ad[t] = lad[j0 + t];
                v[t] = VALS ? lv[j0 + t] : ldg(vOg + j0 + t);
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    T g[N];
#pragma unroll
                    for (int t = 0; t < N; t++)
                    {
                        const unsigned a = ad[t] + c * chBytes;
                        g[t] = dsLoad(a + off0, (T)0);
                        if (TWO)
                            g[t] += w[c] * dsLoad(a + off1, (T)0);
                    }
#pragma unroll
                    for (int t = 0; t < N; t++)
                        acc[c] += v[t] * g[t];
                }
        };
        int j0 = jb;
        for (; j0 + DRB <= je; j0 += DRB)
            batch(j0, std::integral_constant<int, DRB>{});
        switch (je - j0)
        {
        case 1: batch(j0, std::integral_constant<int, 1>{}); break;
        case 2: batch(j0, std::integral_constant<int, 2>{}); break;
        case 3: batch(j0, std::integral_constant<int, 3>{}); break;
        case 4: batch(j0, std::integral_constant<int, 4>{}); break;
        case 5: batch(j0, std::integral_constant<int, 5>{}); break;
        case 6: batch(j0, std::integral_constant<int, 6>{}); break;
        case 7: batch(j0, std::integral_constant<int, 7>{}); break;
        default: break;
        }
        return;
#endif
        for (int j0 = jb; j0 < je; j0 += DRB)
        {
            unsigned ad[DRB];
            T v[DRB];
#pragma unroll
            for (int t = 0; t < DRB; t++)
            {
                const int j = j0 + t;
                const bool ok = j < je;
                ad[t] = ok ? lad[j] : 0u;
                v[t] = ok ? (VALS ? lv[j] : ldg(vOg + j)) : (T)0;
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    T g[DRB];
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                    {
                        g[t] = (T)0;
                        if (j0 + t < je)
                        {
                            const unsigned a = ad[t] + c * chBytes;
                            g[t] = dsLoad(a + off0, (T)0);
                            if (TWO)
                                g[t] += w[c] * dsLoad(a + off1, (T)0);
                        }
                    }
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                        acc[c] += v[t] * g[t];
                }
        }
    }

    // Sum over the cluster of K per-thread values in T with a fixed tree (lanes, then the warps of a
    // CTA, then the CTAs), so every CTA obtains bit-identical totals.  Thread 0 of each CTA then
    // runs epi(totals) -- the scalar work of the iteration, done once per CTA instead of once per
    // thread -- and the CTA synchronises so every thread can read what epi wrote to shared memory.
    // slot: the CTA's two alternating K-slot buffers read by the other CTAs after the barrier.
    template <typename T, int K, typename Epi>
    __device__ __forceinline__ void dsClusterSum(cg::cluster_group & cl, const T (&v)[K], T (*slot)[8], int & buf,
                                                 Epi && epi)
    {
        __shared__ T warpPart[DTPB / 32][K];
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
                T s = lane < DTPB / 32 ? warpPart[lane][k] : (T)0;
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
            T rv[K];
            const T * remote = cl.map_shared_rank(&slot[buf][0], lane < cs ? lane : 0);
#pragma unroll
            for (int k = 0; k < K; k++)
                rv[k] = lane < cs ? remote[k] : (T)0;
            T tot[K];
#pragma unroll
            for (int k = 0; k < K; k++)
            {
                T s = rv[k];
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

    // Iteration scalars of the cluster solver, kept by thread 0 of every CTA (all CTAs compute the
    // same values from the same totals) and read by the other threads after a CTA barrier.
    template <typename T, int NCH>
    struct DsScalars
    {
        T alpha[NCH], beta[NCH];
        int act[NCH], status[NCH], iters[NCH], any;
        double bb[NCH], rr[NCH], rz[NCH], rzPrev[NCH];
        int replace, replacements; // residual replacement due in this iteration; count
        double rrRef[NCH];         // ||r||^2 at the last replacement
        // ru: the FP32 recurrence runs on gsc * (b - A x), gsc = 2^-e with 2^(e-1) <= ||b|| < 2^e:
        // an exact power-of-two scale (the same bits as the unscaled recurrence, shifted), so that
        // the FP32 residual and its dot products stay O(1) instead of underflowing for small ||b||
        // or tight tolerances; the increment is scaled back (igsc) when it is folded into x64
        double gsc[NCH], igsc[NCH];
    };

    // CO: with the coarse correction of DsPcgArgs (NCH == 1, at least three colours)
    template <typename T, int NCH, bool VALS, bool CO = false>
    __global__ void __launch_bounds__(DTPB, 1) kPcgClusterDs(DsPcgArgs<T> Ain)
    {
        extern __shared__ __align__(16) unsigned char dsm[];
        cg::cluster_group cl = cg::this_cluster();
        const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
        DsPcgArgs<T> A = Ain;
        if (A.instStride)
        {
            const long long inst = (long long)(blockIdx.x / (unsigned)cs), off = inst * A.instStride;
            A.b = A.b ? A.b + off : nullptr;
            A.x = A.x ? A.x + off : nullptr;
            A.b64 = A.b64 ? A.b64 + off : nullptr;
            A.x64 = A.x64 ? A.x64 + off : nullptr;
            A.st += inst;
        }
        __shared__ T slot[2][8];
        __shared__ int chunkA[MAXCOLORS], chunkL[MAXCOLORS + 1], chunkG[MAXCOLORS], nzBase[MAXCOLORS + 1];
        __shared__ DsScalars<T, NCH> sc;
        int buf = 0;
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

        // ---- own rows: chunk `rank` of every color (local row l of color c is global row
        // chunkA[c] + (l - chunkL[c])), entries numbered locally in the same order
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
        const DsLayout L = A.lay;
        {
            // vector planes start at zero (padding entries stay finite)
            uint4 * v4 = reinterpret_cast<uint4 *>(dsm);
            const int cnt = (int)(L.offRs / 16);
            for (int t = threadIdx.x; t < cnt; t += DTPB)
                v4[t] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
        const int S = L.stride;
        const unsigned chBytes = (unsigned)(S * sizeof(T));
        T * zs = reinterpret_cast<T *>(dsm + L.offZ);
        T * pl = reinterpret_cast<T *>(dsm + L.offP);
        T * xs = reinterpret_cast<T *>(dsm + L.offX);
        T * rsv = reinterpret_cast<T *>(dsm + L.offR);
        T * qs = reinterpret_cast<T *>(dsm + L.offQ);
        T * invDs = reinterpret_cast<T *>(dsm + L.offInvD);
        T * diags = reinterpret_cast<T *>(dsm + L.offDiag);
        unsigned * lrs = reinterpret_cast<unsigned *>(dsm + L.offRs);
        unsigned * lad = reinterpret_cast<unsigned *>(dsm + L.offAd);
        const T * lv = reinterpret_cast<const T *>(dsm + L.offV);
        const unsigned zBase = (unsigned)__cvta_generic_to_shared(zs);
        const unsigned offX = L.offX - L.offZ, offP0 = L.offP - L.offZ;
        // the direction phase gathers the corrected z when the coarse correction is on
        const unsigned offZF = CO ? L.offZF - L.offZ : 0u;
        const int R = chunkL[C];
        for (int c = 0; c < C; c++)
        {
            const int a0 = chunkA[c], nr = chunkL[c + 1] - chunkL[c], g0 = chunkG[c], nb = nzBase[c];
            const int lo = A.ps[c];
            for (int t = threadIdx.x; t < nr; t += DTPB)
            {
                const int l = chunkL[c] + t, i = a0 + t;
                const int jb = ldg(A.rsO + i), je = ldg(A.rsO + i + 1);
                int sp = jb;
                while (sp < je && ldg(A.ciO + sp) < lo) // sorted columns: earlier colors first
                    sp++;
                lrs[l] = (unsigned)(jb - g0 + nb) | ((unsigned)(sp - jb) << 24);
                invDs[l] = ldg(A.invD + i);
                diags[l] = ldg(A.diag + i);
                if (CO)
                    reinterpret_cast<int *>(dsm + L.offAggL)[l] = ldg(A.aggOfRow + i) - ldg(A.aggStart + rank);
#pragma unroll
                for (int ch = 0; ch < NCH; ch++)
                    xs[ch * S + l] = (ch < numCh && !A.ru) ? A.x[(size_t)ch * n + i] : (T)0; // ru: increment
            }
            const int cnt = nzBase[c + 1] - nb;
            for (int t = threadIdx.x; t < cnt; t += DTPB)
            {
                const int e = ldg(A.cmap + g0 + t);
                lad[nb + t] = dsMapa(zBase + (unsigned)(e & 0xFFFFFF) * (unsigned)sizeof(T), e >> 24);
                if (VALS)
                    reinterpret_cast<T *>(dsm + L.offV)[nb + t] = ldg(A.vO + g0 + t);
            }
        }
        if (threadIdx.x == 0)
            lrs[R] = (unsigned)nzBase[C];
        // coarse correction: the CTA's rows of the coarse inverse into shared memory
        const int nAgg = L.nAgg;
        const int aggA0 = CO ? ldg(A.aggStart + rank) : 0;
        const int nAggOwn = CO ? ldg(A.aggStart + rank + 1) - aggA0 : 0;
        T * zfs = reinterpret_cast<T *>(dsm + L.offZF);
        T * cOwn = reinterpret_cast<T *>(dsm + L.offCOwn);
        T * cAll = reinterpret_cast<T *>(dsm + L.offCAll);
        T * yOwn = reinterpret_cast<T *>(dsm + L.offYOwn);
        T * ainvS = reinterpret_cast<T *>(dsm + L.offAinv);
        const int * aggL = reinterpret_cast<const int *>(dsm + L.offAggL);
        if (CO)
            for (int t = threadIdx.x; t < nAggOwn * nAgg; t += DTPB)
                ainvS[t] = ldg(A.ainv + (size_t)aggA0 * nAgg + t);
        cl.sync(); // every CTA's x and row structure in place

        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh;
        T alpha[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            alpha[c] = (T)0;

        // ---- FP64 residual replacement helpers (ru)
        // x64 += x (the FP32 increment), x = 0, own rows
        auto flushX = [&]() {
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh)
                        {
                            double * px = A.x64 + (size_t)c * n + i;
                            *px = __ldcg(px) + (double)xs[c * S + l] * sc.igsc[c];
                            xs[c * S + l] = (T)0;
                        }
                }
        };
        // r = b64 - A64 x64 in FP64 for own rows (neighbours' x64 through L2), rounded into r;
        // bbAcc += ||b64||^2 when withBb
        auto trueResidual = [&](T (&bbAcc)[NCH], bool withBb) {
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
                    const int jb = ldg(A.rsO + i), je = ldg(A.rsO + i + 1);
                    const double d = ldg(A.diag64 + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh)
                        {
                            const double * xc = A.x64 + (size_t)c * n;
                            double acc = d * __ldcg(xc + i);
                            // predicated batches: all loads of a row in flight together
                            for (int j0 = jb; j0 < je; j0 += DRB)
                            {
                                int cols[DRB];
                                double v[DRB], g[DRB];
#pragma unroll
                                for (int t = 0; t < DRB; t++)
                                {
                                    const bool ok = j0 + t < je;
                                    cols[t] = ok ? ldg(A.ciO + j0 + t) : i;
                                    v[t] = ok ? ldg(A.vO64 + j0 + t) : 0.0;
                                }
#pragma unroll
                                for (int t = 0; t < DRB; t++)
                                    g[t] = __ldcg(xc + cols[t]);
#pragma unroll
                                for (int t = 0; t < DRB; t++)
                                    acc += v[t] * g[t];
                            }
                            const double bi = ldg(A.b64 + (size_t)c * n + i), g = sc.gsc[c];
                            rsv[c * S + l] = (T)((bi - acc) * g);
                            if (withBb)
                                bbAcc[c] += (T)(bi * g) * (T)(bi * g);
                        }
                }
        };

        // ---- r = b - A x over own rows; ||b||^2
        T bbP[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bbP[c] = (T)0;
        if (threadIdx.x == 0)
            for (int c = 0; c < NCH; c++)
                sc.gsc[c] = sc.igsc[c] = 1.0;
        if (A.ru)
        {
            // ||b64||^2 in FP64 over the cluster -> the power-of-two scale of the FP32 recurrence
            __shared__ double dslot[2][8];
            double bq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                bq[c] = 0.0;
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh)
                        {
                            const double bi = ldg(A.b64 + (size_t)c * n + i);
                            bq[c] += bi * bi;
                        }
                }
            dsClusterSum<double, NCH>(cl, bq, dslot, buf, [&](const double (&tot)[NCH]) {
                for (int c = 0; c < NCH; c++)
                    if (tot[c] > 0.0 && isfinite(tot[c]))
                    {
                        int e = 0;
                        frexp(sqrt(tot[c]), &e);
                        sc.gsc[c] = ldexp(1.0, -e);
                        sc.igsc[c] = ldexp(1.0, e);
                    }
            });
            trueResidual(bbP, true);
        }
        else
        for (int col = 0; col < C; col++)
        {
            const T * vOg = A.vO + (chunkG[col] - nzBase[col]);
            for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
            {
                const int i = chunkA[col] + (l - chunkL[col]);
                const int jb = (int)(lrs[l] & 0xFFFFFFu), je = (int)(lrs[l + 1] & 0xFFFFFFu);
                const T d = diags[l];
                T acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = d * xs[c * S + l];
                dsGather<T, NCH, VALS, false>(lad, lv, vOg, jb, je, offX, 0u, chBytes, alpha, act, acc);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        const T bi = A.b[(size_t)c * n + i];
                        rsv[c * S + l] = bi - acc[c];
                        bbP[c] += bi * bi;
                    }
            }
        }

        // z = SGS(r) from z = 0.  init: no x / r update.  Forward phases use earlier colors only.
        auto sgs = [&](bool init, int plane, T (&rr)[NCH], T (&rz)[NCH]) {
            const T * pc = pl + (size_t)plane * NCH * S;
#pragma unroll
            for (int c = 0; c < NCH; c++)
                rr[c] = rz[c] = (T)0;
            for (int col = 0; col < C; col++)
            {
                const T * vOg = A.vO + (chunkG[col] - nzBase[col]);
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const unsigned pk = lrs[l];
                    const int jb = (int)(pk & 0xFFFFFFu), jl = jb + (int)(pk >> 24);
                    T ri[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        ri[c] = (T)0;
                        if (act[c])
                        {
                            const int o = c * S + l;
                            T rv = rsv[o];
                            if (!init)
                            {
                                xs[o] = xs[o] + alpha[c] * pc[o];
                                rv -= alpha[c] * qs[o];
                                rsv[o] = rv;
                            }
                            ri[c] = rv;
                        }
                    }
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    dsGather<T, NCH, VALS, false>(lad, lv, vOg, jb, jl, 0u, 0u, chBytes, alpha, act, acc);
                    const T id = invDs[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const T zi = (ri[c] - acc[c]) * id;
                            zs[c * S + l] = zi;
                            rr[c] += ri[c] * ri[c];
                            if (!CO && col == C - 1)
                                rz[c] += ri[c] * zi;
                        }
                }
                if (C > 1)
                    cl.sync(); // z of this color visible to the cluster
            }
            for (int col = C - 2; col >= 0; col--)
            {
                // plain ifs on CO here: the lambda's discarded if-constexpr branches were not reliably
                // removed from the CO = false kernel
                if (CO)
                {
                    if (col == C - 2)
                    {
                        // r is final on every own row: the CTA's aggregate sums P^T r, a warp per
                        // aggregate in a fixed order, published by this phase's cluster barrier
                        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
                        for (int a = warp; a < nAggOwn; a += DTPB / 32)
                        {
                            const int r0 = ldg(A.aggRowStart + aggA0 + a), r1 = ldg(A.aggRowStart + aggA0 + a + 1);
                            T sum = (T)0;
                            for (int t = r0 + lane; t < r1; t += 32)
                                sum += rsv[ldg(A.aggRows + t)];
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1)
                                sum += __shfl_xor_sync(FULL, sum, o);
                            if (lane == 0)
                                cOwn[a] = sum;
                        }
                    }
                    if (col == 0)
                    {
                        // every aggregate's sum from its CTA, then the CTA's coarse values
                        // y = Ac^-1 (P^T r) for its own aggregates
                        const unsigned cBase = (unsigned)__cvta_generic_to_shared(cOwn);
                        for (int g = threadIdx.x; g < nAgg; g += DTPB)
                        {
                            int rk = 0;
                            while (rk + 1 < cs && ldg(A.aggStart + rk + 1) <= g)
                                rk++;
                            cAll[g] = dsLoad(dsMapa(cBase + (unsigned)(g - ldg(A.aggStart + rk)) * (unsigned)sizeof(T), rk),
                                             (T)0);
                        }
                        __syncthreads();
                        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
                        for (int a = warp; a < nAggOwn; a += DTPB / 32)
                        {
                            const T * row = ainvS + (size_t)a * nAgg;
                            T sum = (T)0;
                            for (int g = lane; g < nAgg; g += 32)
                                sum += row[g] * cAll[g];
#pragma unroll
                            for (int o = 16; o > 0; o >>= 1)
                                sum += __shfl_xor_sync(FULL, sum, o);
                            if (lane == 0)
                                yOwn[a] = sum;
                        }
                        __syncthreads();
                    }
                }
                const T * vOg = A.vO + (chunkG[col] - nzBase[col]);
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int jb = (int)(lrs[l] & 0xFFFFFFu), je = (int)(lrs[l + 1] & 0xFFFFFFu);
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    dsGather<T, NCH, VALS, false>(lad, lv, vOg, jb, je, 0u, 0u, chBytes, alpha, act, acc);
                    const T id = invDs[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const int o = c * S + l;
                            const T rv = rsv[o];
                            const T zi = (rv - acc[c]) * id;
                            zs[o] = zi;
                            if (CO)
                            {
                                if (col == 0)
                                {
                                    const T zf = zi + yOwn[aggL[l]];
                                    zfs[o] = zf;
                                    rz[c] += rv * zf;
                                }
                            }
                            else
                                rz[c] += rv * zi;
                        }
                }
                if (CO && col == 0)
                    // the corrected z of the rows of the later colours (their SGS z is final)
                    for (int l = chunkL[1] + threadIdx.x; l < chunkL[C]; l += DTPB)
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const int o = c * S + l;
                                const T zf = zs[o] + yOwn[aggL[l]];
                                zfs[o] = zf;
                                rz[c] += rsv[o] * zf;
                            }
                if (col > 0)
                    cl.sync(); // the last phase's barrier is the reduction's
            }
        };

        T rr0[NCH], rz0[NCH];
        sgs(true, 0, rr0, rz0);
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
        dsClusterSum<T, 3 * NCH>(cl, red, slot, buf, [&](const T (&tot)[3 * NCH]) {
            int any = 0;
            for (int c = 0; c < NCH; c++)
            {
                const double bb = (double)tot[c], rr = (double)tot[NCH + c], rz = (double)tot[2 * NCH + c];
                sc.bb[c] = bb;
                sc.rr[c] = rr;
                sc.rz[c] = rz;
                sc.rzPrev[c] = rz;
                const bool fin = isfinite(rr) && isfinite(bb);
                const bool conv = absMode ? (rr * sc.igsc[c] * sc.igsc[c] < tol2) : (rr <= tol2 * bb);
                sc.status[c] = fin ? 0 : 2;
                sc.iters[c] = 0;
                sc.act[c] = (c < numCh) && fin && !conv;
                sc.alpha[c] = (T)0;
                sc.beta[c] = (T)0;
                sc.rrRef[c] = rr;
                any |= sc.act[c];
            }
            sc.any = any;
            sc.replace = 0;
            sc.replacements = 0;
        });
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = sc.act[c] != 0;

        int k = 1;
        for (; k <= maxIters; k++)
        {
            if (!sc.any)
                break; // same value in every CTA
            // direction: p_new = z + beta p_old ; q = A p_new ; p.q   (own rows of every color)
            const int po = (k - 1) & 1, pnI = k & 1;
            const T * pold = pl + (size_t)po * NCH * S;
            T * pnew = pl + (size_t)pnI * NCH * S;
            const unsigned offPold = offP0 + (unsigned)po * NCH * chBytes;
            T beta[NCH], pq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                beta[c] = sc.beta[c];
                pq[c] = (T)0;
            }
            for (int col = 0; col < C; col++)
            {
                const T * vOg = A.vO + (chunkG[col] - nzBase[col]);
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int jb = (int)(lrs[l] & 0xFFFFFFu), je = (int)(lrs[l + 1] & 0xFFFFFFu);
                    const T d = diags[l];
                    T pn[NCH], acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                    {
                        const int o = c * S + l;
                        const T zo = CO ? zfs[o] : zs[o];
                        pn[c] = act[c] ? (k == 1 ? zo : zo + beta[c] * pold[o]) : (T)0;
                        acc[c] = d * pn[c];
                    }
                    if (k == 1)
                        dsGather<T, NCH, VALS, false>(lad, lv, vOg, jb, je, offZF, 0u, chBytes, beta, act, acc);
                    else
                        dsGather<T, NCH, VALS, true>(lad, lv, vOg, jb, je, offZF, offPold, chBytes, beta, act, acc);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const int o = c * S + l;
                            pnew[o] = pn[c];
                            qs[o] = acc[c];
                            pq[c] += pn[c] * acc[c];
                        }
                }
            }
            dsClusterSum<T, NCH>(cl, pq, slot, buf, [&](const T (&tot)[NCH]) {
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
            if (A.ru && sc.replace) // same value in every CTA
            {
                // the CG step x += alpha p, folded into x64; r replaced by the FP64 residual
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                        for (int col = 0; col < C; col++)
                            for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                                xs[c * S + l] += alpha[c] * pnew[c * S + l];
                flushX();
                cl.sync(); // every CTA's x64 in global memory
                T unused[NCH];
                trueResidual(unused, false);
                sgs(true, pnI, rrN, rzN);
            }
            else
                sgs(false, pnI, rrN, rzN);
            T red2[2 * NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                red2[c] = rrN[c];
                red2[NCH + c] = rzN[c];
            }
            dsClusterSum<T, 2 * NCH>(cl, red2, slot, buf, [&](const T (&tot)[2 * NCH]) {
                int any = 0;
                const bool replaced = A.ru && sc.replace;
                sc.replace = 0;
                sc.replacements += replaced ? 1 : 0;
                for (int c = 0; c < NCH; c++)
                {
                    if (sc.act[c])
                    {
                        const double rr = (double)tot[c], rz = (double)tot[NCH + c];
                        sc.rr[c] = rr;
                        sc.rz[c] = rz;
                        const bool fin = isfinite(rr) && isfinite(rz);
                        const bool conv =
                            absMode ? (rr * sc.igsc[c] * sc.igsc[c] < tol2) : (rr <= tol2 * sc.bb[c]);
                        // with replacement the solve stops only on an FP64 residual; a converged
                        // or sufficiently reduced iterated residual schedules a replacement
                        const bool stop = !fin || (conv && (!A.ru || replaced));
                        if (replaced)
                            sc.rrRef[c] = rr;
                        else if (A.ru && fin && (conv || rr <= A.ruDelta2 * sc.rrRef[c]))
                            sc.replace = 1;
                        if (stop)
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
                sc.any = any;
            });
#pragma unroll
            for (int c = 0; c < NCH; c++)
                act[c] = sc.act[c] != 0;
        }

        // ---- x back to global memory (own rows); ru: the remaining increment into x64
        if (A.ru)
            flushX();
        else
            for (int col = 0; col < C; col++)
                for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
                {
                    const int i = chunkA[col] + (l - chunkL[col]);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh)
                            A.x[(size_t)c * n + i] = xs[c * S + l];
                }
        // results (rank 0 writes; every CTA holds identical values).  ru: the refinement's view --
        // iters = replacements ("passes"), innerTotal = CG iterations
        if (rank == 0 && threadIdx.x == 0)
        {
            for (int c = 0; c < NCH; c++)
            {
                if (sc.act[c])
                {
                    sc.status[c] = 3;
                    sc.iters[c] = maxIters;
                }
                st->status[c] = c < numCh ? sc.status[c] : 0;
                st->iters[c] = A.ru ? sc.replacements : sc.iters[c];
                if (A.ru)
                    st->innerTotal[c] = sc.iters[c];
                // in the units of b (the ru recurrence runs scaled by gsc)
                st->bb[c] = sc.bb[c] * sc.igsc[c] * sc.igsc[c];
                st->lastRR[c] = sc.rr[c] * sc.igsc[c] * sc.igsc[c];
                st->active[c] = 0;
            }
            st->iter = k;
            st->anyActive = 0;
        }
        // no CTA may leave while another can still read its shared memory
        cl.sync();
    }

    // Per-CTA shares of a color-permuted system split as the cluster kernels split it.
    struct DsShares
    {
        int rowsMax = 0, nzMax = 0;
        std::vector<int> cmap; // per off-diagonal entry: owner rank << 24 | local row in the owner
    };

    // ps: color starts; rsO / ciO: off-diagonal CSR (host); cs: cluster size
    inline DsShares dsShares(const std::vector<int> & ps, const std::vector<int> & rsO, const std::vector<int> & ciO,
                             int cs)
    {
        DsShares D;
        const int C = (int)ps.size() - 1, n = ps.back();
        std::vector<int> owner(n), local(n);
        for (int rk = 0; rk < cs; rk++)
        {
            int l = 0, nz = 0;
            for (int c = 0; c < C; c++)
            {
                const int len = ps[c + 1] - ps[c];
                const int a0 = ps[c] + (int)(((long long)len * rk) / cs);
                const int a1 = ps[c] + (int)(((long long)len * (rk + 1)) / cs);
                for (int i = a0; i < a1; i++)
                {
                    owner[i] = rk;
                    local[i] = l++;
                }
                nz += rsO[a1] - rsO[a0];
            }
            D.rowsMax = std::max(D.rowsMax, l);
            D.nzMax = std::max(D.nzMax, nz);
        }
        D.cmap.resize(ciO.size());
        for (size_t j = 0; j < ciO.size(); j++)
            D.cmap[j] = (owner[ciO[j]] << 24) | local[ciO[j]];
        return D;
    }

    // Whether one cluster of cs CTAs of kernel k with `smem` bytes of dynamic shared memory each can
    // be co-scheduled.  The kernel's dynamic shared memory ceiling is set to the device maximum
    // (minus its static shared memory) once, so solvers of different sizes can share the kernel.
    template <typename K>
    inline bool clusterFits(K kernel, int cs, size_t smem)
    {
        cudaFuncAttributes fa{};
        int dev = 0, optin = 0;
        if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        {
            cudaGetLastError();
            return false;
        }
        if ((size_t)optin <= fa.sharedSizeBytes)
            return false;
        const size_t cap = (size_t)optin - fa.sharedSizeBytes;
        if (smem > cap)
            return false;
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap) != cudaSuccess ||
            (cs > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess))
        {
            cudaGetLastError();
            return false;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(DTPB);
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
            return true;
        cudaGetLastError();
        return false;
    }

    // Whether the per-CTA shares fit the packed encodings (24-bit local offsets, < 256 entries of
    // earlier colors in a row).
    inline bool dsEncodable(const DsShares & D, const std::vector<int> & rsO)
    {
        if (D.rowsMax >= (1 << 24) || D.nzMax >= (1 << 24))
            return false;
        for (size_t i = 0; i + 1 < rsO.size(); i++)
            if (rsO[i + 1] - rsO[i] > 255)
                return false;
        return true;
    }
} // namespace nsf
