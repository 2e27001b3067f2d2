// sm_103a kernels of the Chorin path.  All sparse work is memory/latency bound (no tensor-core
// shape), so the kernels are built around:
//   * row groups of L lanes (L = 2..32) per CSR row: coalesced value/column streams, the
//     row sum finished with width-L shuffles;
//   * deterministic reductions: every block writes one FP64 partial per channel to a fixed
//     slot, consumers sum the slot range in a fixed order (same bits on every run);
//   * device-resident solver scalars and early-exit flags, so solver loops need no host sync
//     and can run inside CUDA graphs (conditional while nodes end the loop on the device);
//   * an iteration counter advanced by the last block of the last kernel of an iteration
//     ("last block done"), so no kernel ever reads a counter that another block is writing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nsf
{
    constexpr int TPB = 256;      // threads per block of every kernel here
    constexpr int MAXCH = 2;      // planar channels handled by one solver instance
    constexpr unsigned FULL = 0xffffffffu;

    template <int L>
    struct Group
    {
        int lane, gid, ngroups;
        unsigned mask;

        __device__ __forceinline__ Group()
        {
            const int t = blockIdx.x * blockDim.x + threadIdx.x;
            lane = threadIdx.x & (L - 1);
            gid = t / L;
            ngroups = (gridDim.x * blockDim.x) / L;
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

    // ------------------------------------------------------------------ reductions

    // Sum v over the block; thread 0 writes it to out[ch * stride + slot].
    template <int NCH>
    __device__ __forceinline__ void blockPartial(double (&v)[NCH], double * out, int stride, int slot)
    {
        __shared__ double sm[TPB / 32][NCH];
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            double s = v[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0)
                sm[warp][c] = s;
        }
        __syncthreads();
        if (warp == 0)
        {
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                double s = lane < (TPB / 32) ? sm[lane][c] : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    s += __shfl_xor_sync(FULL, s, o);
                if (lane == 0 && out)
                    out[c * stride + slot] = s;
            }
        }
        __syncthreads();
    }

    // Every thread of the block gets sum(p[ch * stride + 0 .. n)) per channel (fixed order).
    template <int NCH>
    __device__ __forceinline__ void sumSlots(const double * p, int stride, int n, double (&out)[NCH])
    {
        __shared__ double sm[TPB / 32][NCH];
        __shared__ double res[NCH];
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            double s = 0;
            for (int i = threadIdx.x; i < n; i += blockDim.x)
                s += p[c * stride + i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                s += __shfl_xor_sync(FULL, s, o);
            if (lane == 0)
                sm[warp][c] = s;
        }
        __syncthreads();
        if (warp == 0)
        {
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                double s = lane < (TPB / 32) ? sm[lane][c] : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    s += __shfl_xor_sync(FULL, s, o);
                if (lane == 0)
                    res[c] = s;
            }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < NCH; c++)
            out[c] = res[c];
        __syncthreads();
    }

    // Last block to finish advances *counter (all blocks have read it before they finish).
    __device__ __forceinline__ void lastBlockTick(unsigned * done, int * counter)
    {
        __syncthreads();
        if (threadIdx.x == 0)
        {
            __threadfence();
            const unsigned prev = atomicAdd(done, 1u);
            if (prev == gridDim.x - 1)
            {
                *done = 0;
                *counter += 1;
                __threadfence();
            }
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

    // A[k] = nu * K[k] + sum_j I[k, j] u[j]   (linearised advection + diffusion)
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

    // u <- Dirichlet value on boundary rows, u - tau * acc elsewhere (2 planar channels)
    template <typename TA>
    __global__ void __launch_bounds__(TPB) kUpdateVelocity(int n, double * __restrict__ u, const TA * __restrict__ acc,
                                                            double tau, const unsigned char * __restrict__ isDir,
                                                            const double * __restrict__ dirVal)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
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
    }

    template <typename TS, typename TD>
    __global__ void __launch_bounds__(TPB) kConvert(int n, const TS * __restrict__ s, TD * __restrict__ d)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            d[i] = (TD)s[i];
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

    // ------------------------------------------------------------------ solver state

    // Device-resident scalars of one solve (numCh planar channels).
    struct SolverState
    {
        double rzHist[2][MAXCH]; // r.z of the last two iterations (index = iteration parity)
        double bb[MAXCH];        // ||b||^2
        double lastRR[MAXCH];    // ||r||^2 at the last convergence check
        double tol2;             // relative tolerance squared (or absolute RMS^2 * n for abs mode)
        int absMode;             // 1: stop on ||r||^2 < tol2 (absolute), 0: ||r||^2 <= tol2 * ||b||^2
        int active[MAXCH];
        int iters[MAXCH];
        int status[MAXCH];       // 0 ok / converged, 2 non-finite, 3 max iterations, 4 breakdown
        int iter;                // iterations started (advanced by the last block of an iteration)
        int maxIters;
        int anyActive;           // 0 once every channel stopped (host polls this)
        unsigned done;           // last-block counter
        int skip;                // refinement: 1 once the outer loop has stopped
        int innerTotal[MAXCH];   // refinement: inner iterations summed over passes
    };

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

    template <int NCH>
    __device__ __forceinline__ bool anyAct(const bool (&a)[NCH])
    {
        bool r = false;
#pragma unroll
        for (int c = 0; c < NCH; c++)
            r |= a[c];
        return r;
    }

    // ------------------------------------------------------------------ PCG with multicolor SGS
    // Work vectors are planar [ch * n + i] in the color-permuted numbering; color c owns rows
    // [ps[c], ps[c+1]).  Partial-sum layout: slot ranges per color, same for rr and rz.

    struct PcgPtrs
    {
        int n;
        int slots;        // number of partial slots (sum of blocks over colors)
        double * rrPart;  // [MAXCH][slots]  ||r||^2 partials (forward phases)
        double * rzPart;  // [MAXCH][slots]  r.z partials (last forward phase + backward phases)
        double * pqPart;  // [MAXCH][pqSlots]
        int pqSlots;
        double * bbPart;  // [MAXCH][slots]
        SolverState * st;
        unsigned long long cond; // graph conditional handle (0: none)
        const int * skip;        // when set and *skip != 0 the solve stops at start (refinement done)
    };

    // r = b - A x (full matrix); bb partials; r and x in T
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgInit(PcgPtrs P, const int * __restrict__ rs, const int * __restrict__ ci,
                                                     const T * __restrict__ v, const T * __restrict__ x,
                                                     const T * __restrict__ b, T * __restrict__ r)
    {
        Group<L> g;
        double bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        const int n = P.n;
        for (int i = g.gid; i < n; i += g.ngroups)
        {
            const int s = ldg(rs + i), e = ldg(rs + i + 1);
            double acc[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const double a = (double)ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] += a * (double)x[(size_t)c * n + col];
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double t = g.sum(acc[c]);
                if (g.lane == 0)
                {
                    const double bi = (double)b[(size_t)c * n + i];
                    r[(size_t)c * n + i] = (T)(bi - t);
                    bb[c] += bi * bi;
                }
            }
        }
        blockPartial<NCH>(bb, P.bbPart, P.slots, blockIdx.x);
    }

    // Finish the initial state once the SGS of r0 is done: bb, activity, iteration counter.
    template <int NCH>
    __global__ void kPcgStart(PcgPtrs P, int numCh)
    {
        double bb[NCH], rr[NCH], rz[NCH];
        sumSlots<NCH>(P.bbPart, P.slots, P.slots, bb);
        sumSlots<NCH>(P.rrPart, P.slots, P.slots, rr);
        sumSlots<NCH>(P.rzPart, P.slots, P.slots, rz);
        if (threadIdx.x == 0)
        {
            SolverState * st = P.st;
            const bool skipAll = P.skip && *P.skip;
            int any = 0;
            for (int c = 0; c < NCH; c++)
            {
                st->bb[c] = bb[c];
                st->lastRR[c] = rr[c];
                st->rzHist[0][c] = rz[c];
                st->rzHist[1][c] = rz[c];
                const bool fin = isfinite(rr[c]) && isfinite(bb[c]);
                const bool conv = st->absMode ? (rr[c] < st->tol2) : (rr[c] <= st->tol2 * bb[c]);
                const bool act = c < numCh && fin && !conv && !skipAll;
                st->active[c] = act;
                st->iters[c] = 0;
                st->status[c] = fin ? 0 : 2;
                any |= act;
            }
            st->iter = 1;
            st->done = 0;
            st->anyActive = any;
        }
    }

    // Iteration kernel A: convergence decision from the previous iteration's ||r||^2, beta,
    // p_new = z + beta p_old, q = A p_new, pq partials.
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgDirection(PcgPtrs P, int numCh, const int * __restrict__ rs,
                                                          const int * __restrict__ ci, const T * __restrict__ v,
                                                          const T * __restrict__ z, T * __restrict__ pbuf,
                                                          T * __restrict__ q)
    {
        SolverState * st = P.st;
        const int k = st->iter; // stable for the whole iteration
        double rr[NCH], rz[NCH];
        sumSlots<NCH>(P.rrPart, P.slots, P.slots, rr);
        sumSlots<NCH>(P.rzPart, P.slots, P.slots, rz);
        bool act[NCH];
        double beta[NCH];
        bool stopAll = true;
#pragma unroll
        for (int c = 0; c < NCH; c++)
        {
            const bool wasActive = c < numCh && st->active[c] && st->status[c] == 0;
            const bool fin = isfinite(rr[c]) && isfinite(rz[c]);
            const bool conv = st->absMode ? (rr[c] < st->tol2) : (rr[c] <= st->tol2 * st->bb[c]);
            act[c] = wasActive && fin && !conv && (k <= st->maxIters);
            beta[c] = (k == 1) ? 0.0 : rz[c] / st->rzHist[(k - 1) & 1][c];
            stopAll &= !act[c];
        }
        if (blockIdx.x == 0 && threadIdx.x == 0)
        {
            int any = 0;
            for (int c = 0; c < NCH; c++)
            {
                const bool wasActive = c < numCh && st->active[c];
                if (wasActive && !act[c])
                {
                    st->iters[c] = k - 1;
                    st->lastRR[c] = rr[c];
                    const bool fin = isfinite(rr[c]) && isfinite(rz[c]);
                    const bool conv = st->absMode ? (rr[c] < st->tol2) : (rr[c] <= st->tol2 * st->bb[c]);
                    if (st->status[c] == 0)
                        st->status[c] = !fin ? 2 : (conv ? 0 : 3);
                }
                st->active[c] = act[c];
                st->rzHist[k & 1][c] = rz[c];
                any |= act[c];
            }
            st->anyActive = any;
            if (!any && P.cond)
                cudaGraphSetConditional(P.cond, 0);
        }
        if (stopAll)
            return;
        const int n = P.n;
        const T * pold = pbuf + (size_t)((k - 1) & 1) * NCH * n;
        T * pnew = pbuf + (size_t)(k & 1) * NCH * n;
        Group<L> g;
        double pq[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            pq[c] = 0;
        for (int i = g.gid; i < n; i += g.ngroups)
        {
            const int s = ldg(rs + i), e = ldg(rs + i + 1);
            double acc[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const double a = (double)ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        const size_t o = (size_t)c * n + col;
                        acc[c] += a * (k == 1 ? (double)z[o] : (double)z[o] + beta[c] * (double)pold[o]);
                    }
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double t = g.sum(acc[c]);
                if (g.lane == 0 && act[c])
                {
                    const size_t o = (size_t)c * n + i;
                    const T pn = (T)(k == 1 ? (double)z[o] : (double)z[o] + beta[c] * (double)pold[o]);
                    pnew[o] = pn;
                    q[o] = (T)t;
                    pq[c] += (double)pn * t;
                }
            }
        }
        blockPartial<NCH>(pq, P.pqPart, P.pqSlots, blockIdx.x);
    }

    // Forward SGS phase over color rows [r0, r1) using only neighbours of earlier colors
    // (columns < r0; later colors are still zero in a forward sweep from z = 0).
    // init == 0: first x += alpha p, r -= alpha q for these rows.  Writes rr partials (and the rz
    // partials when this is the last color) at slot base + blockIdx.x.
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgForward(PcgPtrs P, int numCh, int init, int r0, int r1, int last,
                                                        int slotBase, const int * __restrict__ rs,
                                                        const int * __restrict__ ci, const T * __restrict__ v,
                                                        const T * __restrict__ invD, T * __restrict__ x,
                                                        T * __restrict__ r, T * __restrict__ z,
                                                        const T * __restrict__ pbuf, const T * __restrict__ q)
    {
        SolverState * st = P.st;
        bool act[NCH];
        double alpha[NCH];
        const int k = st->iter;
        const int n = P.n;
        if (!init)
        {
            double pq[NCH];
            sumSlots<NCH>(P.pqPart, P.pqSlots, P.pqSlots, pq);
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                act[c] = c < numCh && st->active[c];
                alpha[c] = st->rzHist[k & 1][c] / pq[c];
            }
            if (blockIdx.x == 0 && threadIdx.x == 0)
                for (int c = 0; c < NCH; c++)
                    if (act[c] && !(pq[c] > 0))
                        st->status[c] = isfinite(pq[c]) ? 4 : 2; // reported after the solve
        }
        else
        {
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                act[c] = c < numCh;
                alpha[c] = 0;
            }
        }
        const T * p = pbuf + (size_t)(k & 1) * NCH * n;
        Group<L> g;
        double rr[NCH], rz[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            rr[c] = rz[c] = 0;
        if (anyAct<NCH>(act))
            for (int i = r0 + g.gid; i < r1; i += g.ngroups)
            {
                double ri[NCH];
                if (g.lane == 0)
                {
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const size_t o = (size_t)c * n + i;
                            double rv = (double)r[o];
                            if (!init)
                            {
                                x[o] = (T)((double)x[o] + alpha[c] * (double)p[o]);
                                rv -= alpha[c] * (double)q[o];
                                r[o] = (T)rv;
                            }
                            ri[c] = (double)(T)rv;
                        }
                }
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                double acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const int col = ldg(ci + j);
                    if (col >= r0)
                        break; // sorted columns: the rest are later colors (zero)
                    const double a = (double)ldg(v + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            acc[c] += a * (double)z[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const double t = g.sum(acc[c]);
                    if (g.lane == 0 && act[c])
                    {
                        const size_t o = (size_t)c * n + i;
                        const T zi = (T)((ri[c] - t) * (double)ldg(invD + i));
                        z[o] = zi;
                        rr[c] += ri[c] * ri[c];
                        if (last)
                            rz[c] += ri[c] * (double)zi;
                    }
                }
            }
        blockPartial<NCH>(rr, P.rrPart, P.slots, slotBase + blockIdx.x);
        if (last)
            blockPartial<NCH>(rz, P.rzPart, P.slots, slotBase + blockIdx.x);
    }

    // Backward SGS phase over color rows [r0, r1) with all off-diagonal neighbours; rz partials.
    // tick != 0: this is the last kernel of an iteration (advances the iteration counter).
    template <typename T, int L, int NCH>
    __global__ void __launch_bounds__(TPB) kPcgBackward(PcgPtrs P, int numCh, int init, int r0, int r1, int slotBase,
                                                         int tick, const int * __restrict__ rs,
                                                         const int * __restrict__ ci, const T * __restrict__ v,
                                                         const T * __restrict__ invD, const T * __restrict__ r,
                                                         T * __restrict__ z)
    {
        SolverState * st = P.st;
        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh && (init || st->active[c]);
        const int n = P.n;
        Group<L> g;
        double rz[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            rz[c] = 0;
        if (anyAct<NCH>(act))
            for (int i = r0 + g.gid; i < r1; i += g.ngroups)
            {
                const int s = ldg(rs + i), e = ldg(rs + i + 1);
                double acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const double a = (double)ldg(v + j);
                    const int col = ldg(ci + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            acc[c] += a * (double)z[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const double t = g.sum(acc[c]);
                    if (g.lane == 0 && act[c])
                    {
                        const size_t o = (size_t)c * n + i;
                        const double ri = (double)r[o];
                        const T zi = (T)((ri - t) * (double)ldg(invD + i));
                        z[o] = zi;
                        rz[c] += ri * (double)zi;
                    }
                }
            }
        blockPartial<NCH>(rz, P.rzPart, P.slots, slotBase + blockIdx.x);
        if (tick && !init)
            lastBlockTick(&st->done, &st->iter);
    }

    // single-block tick for systems with one color (no backward phase)
    __global__ void kTick(SolverState * st)
    {
        if (threadIdx.x == 0)
            st->iter += 1;
    }

    // ------------------------------------------------------------------ FP64 refinement

    // r = b - A x in FP64; r is handed to the FP32 inner solve; rr and bb partials
    template <int L, int NCH>
    __global__ void __launch_bounds__(TPB) kResidual(int n, int slots, const SolverState * st,
                                                      const int * __restrict__ rs, const int * __restrict__ ci,
                                                      const double * __restrict__ v, const double * __restrict__ x,
                                                      const double * __restrict__ b, float * __restrict__ r32,
                                                      double * __restrict__ rrPart, double * __restrict__ bbPart)
    {
        if (st->skip)
            return;
        Group<L> g;
        double rr[NCH], bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            rr[c] = bb[c] = 0;
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
                    rr[c] += ri * ri;
                    bb[c] += bi * bi;
                }
            }
        }
        blockPartial<NCH>(rr, rrPart, slots, blockIdx.x);
        blockPartial<NCH>(bb, bbPart, slots, blockIdx.x);
    }

    // stop decision of refinement pass `pass` (sticky); stats: iters = refinement updates applied
    template <int NCH>
    __global__ void kOuterDecide(SolverState * st, const SolverState * inner, int numCh, int slots,
                                 const double * rrPart, const double * bbPart, int pass)
    {
        if (st->skip)
            return;
        double rr[NCH], bb[NCH];
        sumSlots<NCH>(rrPart, slots, slots, rr);
        sumSlots<NCH>(bbPart, slots, slots, bb);
        if (threadIdx.x == 0)
        {
            bool all = true, bad = false;
            for (int c = 0; c < NCH && c < numCh; c++)
            {
                if (pass > 0)
                    st->innerTotal[c] += inner->iters[c];
                const bool fin = isfinite(rr[c]) && isfinite(bb[c]);
                const bool conv = rr[c] <= st->tol2 * bb[c];
                bad |= !fin;
                all &= conv;
                st->bb[c] = bb[c];
                st->lastRR[c] = rr[c];
                st->iters[c] = pass;
            }
            if (all || bad || pass >= st->maxIters)
            {
                st->skip = 1;
                st->anyActive = 0;
                for (int c = 0; c < NCH; c++)
                {
                    st->active[c] = 0;
                    st->status[c] = bad ? 2 : (all ? 0 : 3);
                }
            }
        }
    }

    // ------------------------------------------------------------------ multicolor Gauss-Seidel
    // The reference's "gs" solver: C colored phases per iteration, RMS residual check every
    // `interval` iterations; decision taken at the start of the following iteration.

    struct GsPtrs
    {
        int n;
        int slots;        // residual partial slots
        double * rrPart;  // [MAXCH][slots]
        double * bbPart;  // [MAXCH][slots]
        SolverState * st;
        unsigned long long cond;
        int interval;
    };

    // b norms (for relative mode) and state reset
    template <typename T, int NCH>
    __global__ void __launch_bounds__(TPB) kGsInit(GsPtrs P, int numCh, const T * __restrict__ b)
    {
        double bb[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bb[c] = 0;
        const int n = P.n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double t = (double)b[(size_t)c * n + i];
                bb[c] += t * t;
            }
        blockPartial<NCH>(bb, P.bbPart, P.slots, blockIdx.x);
    }

    template <int NCH>
    __global__ void kGsStart(GsPtrs P, int numCh)
    {
        double bb[NCH];
        sumSlots<NCH>(P.bbPart, P.slots, P.slots, bb);
        if (threadIdx.x == 0)
        {
            SolverState * st = P.st;
            int any = 0;
            for (int c = 0; c < NCH; c++)
            {
                st->bb[c] = bb[c];
                st->lastRR[c] = -1;
                st->active[c] = c < numCh;
                st->iters[c] = 0;
                st->status[c] = isfinite(bb[c]) ? 0 : 2;
                if (!isfinite(bb[c]))
                    st->active[c] = 0;
                any |= st->active[c];
            }
            st->iter = 0;
            st->done = 0;
            st->anyActive = any;
        }
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
            double rr[NCH];
            if (checked)
                sumSlots<NCH>(P.rrPart, P.slots, P.slots, rr);
            bool stopAll = true;
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const bool was = c < numCh && st->active[c];
                bool conv = false, fin = true;
                if (checked)
                {
                    fin = isfinite(rr[c]);
                    conv = st->absMode ? (rr[c] < st->tol2) : (rr[c] <= st->tol2 * st->bb[c]);
                }
                act[c] = was && fin;
                // both channels stop together once both meet the target (reference semantics)
                stopAll &= !(was && fin) || conv;
                if (checked && blockIdx.x == 0 && threadIdx.x == 0)
                    st->lastRR[c] = rr[c];
                if (!fin && blockIdx.x == 0 && threadIdx.x == 0 && was)
                    st->status[c] = 2;
            }
            const bool over = k >= st->maxIters;
            if (stopAll || over)
            {
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    act[c] = false;
            }
            if (blockIdx.x == 0 && threadIdx.x == 0)
            {
                int any = 0;
                for (int c = 0; c < NCH; c++)
                {
                    const bool was = c < numCh && st->active[c];
                    if (was && !act[c])
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
            double acc[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                acc[c] = 0;
            for (int j = s + g.lane; j < e; j += L)
            {
                const double a = (double)ldg(v + j);
                const int col = ldg(ci + j);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                        acc[c] += a * (double)x[(size_t)c * n + col];
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                const double t = g.sum(acc[c]);
                if (g.lane == 0 && act[c])
                {
                    const size_t o = (size_t)c * n + i;
                    x[o] = (T)(((double)b[o] - t) * (double)ldg(invD + i));
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
        const bool doCheck = anyAct<NCH>(act) && (k % P.interval) == 0;
        double rr[NCH];
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
                double acc[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    acc[c] = 0;
                for (int j = s + g.lane; j < e; j += L)
                {
                    const double a = (double)ldg(v + j);
                    const int col = ldg(ci + j);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] += a * (double)x[(size_t)c * n + col];
                }
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    const double t = g.sum(acc[c]);
                    if (g.lane == 0)
                    {
                        const double d = t - (double)b[(size_t)c * n + i];
                        rr[c] += d * d;
                    }
                }
            }
            blockPartial<NCH>(rr, P.rrPart, P.slots, blockIdx.x);
        }
        if (anyAct<NCH>(act))
            lastBlockTick(&st->done, &st->iter);
    }
} // namespace nsf
