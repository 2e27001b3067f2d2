// Initial guess of the pressure solve by projection onto earlier solutions (pressureGuess 2).
//
// Fischer, "Projection techniques for iterative solution of Ax = b with successive right-hand
// sides", Comput. Methods Appl. Mech. Engrg. 163 (1998).  The stepper keeps up to L vectors x_k
// that are orthonormal in the Kp_int inner product.  Before a pressure solve the guess is the
// Kp_int-orthogonal projection of the new solution onto their span,
//     x0 = sum_k a_k x_k,   a_k = x_k . b          (b: the pressure right-hand side),
// which needs no product with the matrix.  After the solve the correction w = x - x0 joins the
// basis: q = A w, beta_k = x_k . q, w' = w - sum_k beta_k x_k, done twice (classical Gram-Schmidt
// with one re-orthogonalisation keeps a basis of hundreds of vectors orthonormal), and
// x_new = w' / sqrt(w' . A w') (the norm from its own product: no cancellation when w lies close to
// the span).  An empty or
// full basis restarts from the solution x and its first and second differences over the last two
// steps, x - x(n-1) and x - 2 x(n-1) + x(n-2): the span then holds the linear and quadratic
// extrapolations (the projection step's pressure carries a two-step oscillation that the
// solution alone misses).  The solve itself, its tolerance and its stopping test are unchanged;
// the guess only shortens it.
//
// Everything stays on the device: the basis size and the restart decision live in ProjState, so
// a captured step replays the same kernels (an update whose "add" is inactive exits at once).
// Dot products of the basis run as PROJ_CHUNKS blocks per vector with a fixed-order final sum:
// the guess is deterministic.
#pragma once

#include "kernels.cuh"
#include "solvers.cuh"

namespace nsf
{
    constexpr int PROJ_MAXL = 256; // basis vectors at most
    constexpr int PROJ_CHUNKS = 8; // blocks per dot product in kProjDots

    struct ProjState
    {
        int m;         // vectors in the basis
        int slot;      // slot of the vector being added (== m)
        int newSlot;   // slot that the last add filled, -1 if it was rejected
        int hist;      // solutions seen since create / set_state (capped at 2)
        int restart;   // this update restarts the basis
        int active[3]; // the adds of this update: correction (or solution), first, second difference
        double g, nn, scale, dot;
        unsigned ticket;
        unsigned dotTicket[PROJ_MAXL];
    };

    // coef[k] = sum_i X[k n + i] v[i] for k < m; grid (PROJ_CHUNKS, L).  The last block of a vector
    // to finish sums its PROJ_CHUNKS partial sums in order.  which >= 0: skipped unless that add is
    // active.
    __global__ void __launch_bounds__(TPB) kProjDots(int n, const double * __restrict__ X, const double * __restrict__ v,
                                                      ProjState * st, double * partial, double * coef, int which)
    {
        {
            const long long q = blockIdx.z; // instance of a batched projection (grid z)
            X += q * gridDim.y * (long long)n;
            v += q * n;
            st += q;
            partial += q * PROJ_MAXL * PROJ_CHUNKS;
            coef += q * PROJ_MAXL;
        }
        if (which >= 0 && !st->active[which])
            return;
        const int k = blockIdx.y;
        if (k >= st->m)
            return;
        const int c = blockIdx.x;
        const int r0 = (int)((long long)n * c / PROJ_CHUNKS), r1 = (int)((long long)n * (c + 1) / PROJ_CHUNKS);
        const double * xk = X + (size_t)k * n;
        double s = 0;
        for (int i = r0 + threadIdx.x; i < r1; i += TPB)
            s += xk[i] * v[i];
        __shared__ double sm[TPB / 32];
        __shared__ bool last;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(FULL, s, o);
        if ((threadIdx.x & 31) == 0)
            sm[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double t = 0;
            for (int w = 0; w < TPB / 32; w++)
                t += sm[w];
            partial[k * PROJ_CHUNKS + c] = t;
            __threadfence();
            last = atomicAdd(&st->dotTicket[k], 1u) == PROJ_CHUNKS - 1;
        }
        __syncthreads();
        if (!last || threadIdx.x != 0)
            return;
        __threadfence();
        double t = 0;
        for (int j = 0; j < PROJ_CHUNKS; j++)
            t += __ldcg(partial + k * PROJ_CHUNKS + j);
        coef[k] = t;
        st->dotTicket[k] = 0;
    }

    // p = sum_k coef[k] X_k over the basis (p unchanged while it is empty); x0 = p
    __global__ void __launch_bounds__(TPB) kProjGuess(int n, int L, const double * __restrict__ X, const double * coef,
                                                       const ProjState * st, double * __restrict__ p,
                                                       double * __restrict__ x0)
    {
        {
            const long long q = blockIdx.y; // instance (grid y)
            X += q * L * (long long)n;
            coef += q * PROJ_MAXL;
            st += q;
            p += q * n;
            x0 += q * n;
        }
        __shared__ double c[PROJ_MAXL];
        const int m = st->m;
        for (int k = threadIdx.x; k < m; k += TPB)
            c[k] = coef[k];
        __syncthreads();
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            double v = p[i];
            if (m > 0)
            {
                v = 0;
                for (int k = 0; k < m; k++)
                    v += c[k] * X[(size_t)k * n + i];
                p[i] = v;
            }
            x0[i] = v;
        }
    }

    // the adds of this update: an empty or full basis restarts (then the differences join too)
    __global__ void kProjDecide(ProjState * st, int L, int B)
    {
        const int q = blockIdx.x * blockDim.x + threadIdx.x; // one thread per instance
        if (q >= B)
            return;
        st += q;
        const int restart = st->m == 0 || st->m >= L;
        if (restart)
            st->m = 0;
        st->restart = restart;
        st->slot = st->m;
        st->active[0] = 1;
        st->active[1] = restart && st->hist >= 1;
        st->active[2] = restart && st->hist >= 2;
    }

    // the vector that add `which` brings: x - x0 (x on a restart), x - x(n-1), x - 2 x(n-1) + x(n-2)
    __global__ void __launch_bounds__(TPB) kProjPrep(int n, int which, const ProjState * st, const double * __restrict__ x,
                                                      const double * __restrict__ x0, const double * __restrict__ prev1,
                                                      const double * __restrict__ prev2, double * __restrict__ w)
    {
        {
            const long long q = blockIdx.y; // instance (grid y)
            st += q;
            x += q * n;
            x0 += q * n;
            prev1 += q * n;
            prev2 += q * n;
            w += q * n;
        }
        if (!st->active[which])
            return;
        const bool restart = st->restart != 0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            double v;
            if (which == 0)
                v = restart ? x[i] : x[i] - x0[i];
            else if (which == 1)
                v = x[i] - prev1[i];
            else
                v = x[i] - 2.0 * prev1[i] + prev2[i];
            w[i] = v;
        }
    }

    // once per grid after kProjSpmvDot: stage 0 keeps g = w . A w; stage 1 accepts the new vector
    // if its A-norm is not lost in rounding, and advances the basis; stage 2 (the product of the
    // re-orthogonalisation) keeps nothing
    struct ProjEpi
    {
        ProjState * st;
        int stage;
        __device__ void operator()() const
        {
            if (stage == 0)
                st->g = st->dot;
            if (stage != 1)
                return;
            const double g = st->g, nn = st->dot;
            const bool ok = g > 0 && nn > 1e-20 * g && isfinite(nn);
            st->nn = nn;
            st->scale = ok ? 1.0 / sqrt(nn) : 0.0;
            st->newSlot = ok ? st->slot : -1;
            if (ok)
            {
                st->m += 1;
                st->slot = st->m;
            }
        }
    };

    // q = A src and src . q (row groups of L lanes over the CSR); stage 0: src = w, stages 1 and 2:
    // src = the slot being filled.  Skipped unless add `which` is active.
    template <int L>
    __global__ void __launch_bounds__(TPB) kProjSpmvDot(int n, int basis, const int * __restrict__ rs,
                                                         const int * __restrict__ ci, const double * __restrict__ v,
                                                         ProjState * st, int which, int stage, const double * w,
                                                         const double * X, double * __restrict__ q, double * scratch)
    {
        {
            const long long b = blockIdx.y; // instance (grid y); its blocks reduce among themselves
            st += b;
            w += b * n;
            X += b * basis * (long long)n;
            q += b * n;
            scratch += b * gridDim.x;
        }
        if (!st->active[which])
            return;
        const double * src = stage == 0 ? w : X + (size_t)st->slot * n;
        Group<L> g;
        double red[1] = {0.0};
        for (int i = g.gid; i < n; i += g.ngroups)
        {
            double acc = 0;
            for (int j = ldg(rs + i) + g.lane; j < ldg(rs + i + 1); j += L)
                acc += ldg(v + j) * src[ldg(ci + j)];
            const double t = g.sum(acc);
            if (g.lane == 0)
            {
                q[i] = t;
                red[0] += src[i] * t;
            }
        }
        gridSum<double, 1>(red, scratch, Outs<1>{{&st->dot}}, &st->ticket, nullptr, ProjEpi{st, stage});
    }

    // X[slot] = w - sum_k beta_k X_k over the basis (w == nullptr: in place, X[slot] -= ...)
    __global__ void __launch_bounds__(TPB) kProjOrth(int n, int L, double * X, const double * beta, const ProjState * st,
                                                      int which, const double * w)
    {
        {
            const long long q = blockIdx.y; // instance (grid y)
            X += q * L * (long long)n;
            beta += q * PROJ_MAXL;
            st += q;
            if (w)
                w += q * n;
        }
        if (!st->active[which])
            return;
        __shared__ double c[PROJ_MAXL];
        const int m = st->m, slot = st->slot;
        for (int k = threadIdx.x; k < m; k += TPB)
            c[k] = beta[k];
        __syncthreads();
        double * dst = X + (size_t)slot * n;
        const double * src = w ? w : dst;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            double v = src[i];
            for (int k = 0; k < m; k++)
                v -= c[k] * X[(size_t)k * n + i];
            dst[i] = v;
        }
    }

    // normalise the vector that the add accepted
    __global__ void __launch_bounds__(TPB) kProjScale(int n, int L, double * X, const ProjState * st, int which)
    {
        {
            const long long q = blockIdx.y; // instance (grid y)
            X += q * L * (long long)n;
            st += q;
        }
        if (!st->active[which] || st->newSlot < 0)
            return;
        const double s = st->scale;
        double * x = X + (size_t)st->newSlot * n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i] *= s;
    }

    // solution history for the restarts: x(n-2) = x(n-1), x(n-1) = x
    __global__ void __launch_bounds__(TPB) kProjShift(int n, ProjState * st, const double * __restrict__ x,
                                                       double * __restrict__ prev1, double * __restrict__ prev2)
    {
        {
            const long long q = blockIdx.y; // instance (grid y)
            st += q;
            x += q * n;
            prev1 += q * n;
            prev2 += q * n;
        }
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            prev2[i] = prev1[i];
            prev1[i] = x[i];
        }
        if (blockIdx.x == 0 && threadIdx.x == 0 && st->hist < 2)
            st->hist += 1;
    }

    // B instances of the same system (batched steppers): every array holds B instance blocks
    // ([B][L][n] basis, [B][n] vectors, B states), each kernel one launch for all instances (the
    // instance in grid y, or z for the dot products whose grid y is the basis vector).
    struct PressureProjection
    {
        int n = 0, L = 60, B = 1;
        const SweepSystem<double> * A = nullptr;
        DevBuf<double> X, x0, w, q, prev1, prev2, coef, partial, scratch;
        DevBuf<ProjState> st;

        void setup(const SweepSystem<double> * a, int basis, int instances = 1)
        {
            A = a;
            n = a->n;
            L = basis;
            B = instances;
            const size_t nb = (size_t)n * B;
            X.alloc((size_t)L * nb);
            x0.alloc(nb);
            w.alloc(nb);
            q.alloc(nb);
            prev1.alloc(nb);
            prev2.alloc(nb);
            coef.alloc((size_t)PROJ_MAXL * B);
            partial.alloc((size_t)PROJ_MAXL * PROJ_CHUNKS * B);
            scratch.alloc((size_t)cappedBlocks(1ll << 40) * B);
            st.alloc(B);
            NSF_CUDA(cudaMemset(st.get(), 0, sizeof(ProjState) * B));
        }

        // a new history (set_state): the basis and the solution history start empty
        void reset(cudaStream_t s, int inst = -1)
        {
            if (inst < 0)
                NSF_CUDA(cudaMemsetAsync(st.get(), 0, sizeof(ProjState) * B, s));
            else
                NSF_CUDA(cudaMemsetAsync(st.get() + inst, 0, sizeof(ProjState), s));
        }

        // p <- the projection of the solution of A p = b onto the basis (p kept while it is empty)
        void guess(cudaStream_t s, const double * b, double * p)
        {
            NSF_LAUNCH(kProjDots, dim3(PROJ_CHUNKS, L, B), s, n, (const double *)X.get(), b, st.get(), partial.get(),
                       coef.get(), -1);
            NSF_LAUNCH(kProjGuess, dim3(blocksFor(n), B), s, n, L, (const double *)X.get(), (const double *)coef.get(),
                       (const ProjState *)st.get(), p, x0.get());
        }

        // after the solve: the basis learns from the solution p
        void update(cudaStream_t s, const double * p)
        {
            const SweepSystem<double> & S = *A;
            const dim3 grid(blocksFor(n), B);
            NSF_LAUNCH(kProjDecide, (B + 127) / 128, s, st.get(), L, B);
            for (int which = 0; which < 3; which++)
            {
                NSF_LAUNCH(kProjPrep, grid, s, n, which, (const ProjState *)st.get(), p, (const double *)x0.get(),
                           (const double *)prev1.get(), (const double *)prev2.get(), w.get());
                // products of w, of the orthogonalised vector (re-orthogonalisation), of the result
                for (int stage : {0, 2, 1})
                {
                    NSF_LANES(S.L, NSF_LAUNCH((kProjSpmvDot<LL>), dim3(S.fullBlocks(), B), s, n, L, S.rsF.get(),
                                              S.ciF.get(), S.vF.get(), st.get(), which, stage, (const double *)w.get(),
                                              (const double *)X.get(), q.get(), scratch.get()));
                    if (stage != 1)
                    {
                        NSF_LAUNCH(kProjDots, dim3(PROJ_CHUNKS, L, B), s, n, (const double *)X.get(),
                                   (const double *)q.get(), st.get(), partial.get(), coef.get(), which);
                        NSF_LAUNCH(kProjOrth, grid, s, n, L, X.get(), (const double *)coef.get(),
                                   (const ProjState *)st.get(), which,
                                   stage == 0 ? (const double *)w.get() : (const double *)nullptr);
                    }
                }
                NSF_LAUNCH(kProjScale, grid, s, n, L, X.get(), (const ProjState *)st.get(), which);
            }
            NSF_LAUNCH(kProjShift, grid, s, n, st.get(), p, prev1.get(), prev2.get());
        }

        int basisKernelsPerStep() const { return 2 + 1 + 3 * 9 + 1; }
    };
} // namespace nsf
