// Discrete adjoint of the FP64 Chorin step, for gradients of a force functional
//   J = sum_n wDrag[n] F_x(u_n, p_n) + wLift[n] F_y(u_n, p_n)
// with respect to the viscosity, the Dirichlet x values and the initial velocity.  The reference
// has no adjoint; this is the exact reverse of the stepper's forward step (capi.cu,
// enqueueStep, after cpp/execs/NavierStokes/src/chorinCuda.cu:236-376) with every linear solve
// taken as exact:
//   lg += lu1[dir, x];  lw = lu1 with Dirichlet rows zeroed
//   x1 = M^-1 (-tau lw);  lpI = lp + G^T x1;  y = Kpi^-1 lpI;  ls = lw - (1/tau) D^T y
//   lg += ls[dir, x];  lv = ls with Dirichlet rows zeroed;  x2 = M^-1 (-tau lv)
//   lu0 = lv + A(u0)^T x2 + I^T lA,  lA[e = (i, j)] = x2_x[i] u0_x[j] + x2_y[i] u0_y[j]
//   lnu += sum_e lA[e] K[e]
// (M and Kpi symmetric: the adjoint solves reuse the stepper's SGS-preconditioned CG on the same
// color-permuted systems).  The transposed operators D^T, G^T and I^T are stored as CSR, built
// once from the stepper's device operators; A^T reads A through the transpose map of the
// symmetric K pattern.  Forward states come from checkpoints every C steps and a recomputation
// of each segment during the reverse sweep (C = 0 keeps every state).
//
// Included at the end of capi.cu (it uses the stepper and force-functional internals).
#pragma once

namespace
{
    // CSR transpose (rows x cols -> cols x rows); src[k] = source entry of transposed entry k.
    // Source rows are visited in order, so each transposed row's columns come out sorted.
    void transposeCsr(int rows, int cols, const std::vector<int> & rs, const std::vector<int> & ci,
                      std::vector<int> & trs, std::vector<int> & tci, std::vector<int> & src)
    {
        const int nnz = rs[rows];
        trs.assign(cols + 1, 0);
        for (int e = 0; e < nnz; e++)
            trs[ci[e] + 1]++;
        for (int c = 0; c < cols; c++)
            trs[c + 1] += trs[c];
        std::vector<int> pos(trs.begin(), trs.end() - 1);
        tci.assign(nnz, 0);
        src.assign(nnz, 0);
        for (int r = 0; r < rows; r++)
            for (int e = rs[r]; e < rs[r + 1]; e++)
            {
                const int k = pos[ci[e]]++;
                tci[k] = r;
                src[k] = e;
            }
    }

    HostCsr<double> transposedOf(const DevCsr<double> & a)
    {
        const std::vector<int> rs = a.rs.download(), ci = a.ci.download();
        const std::vector<double> v = a.v.download();
        HostCsr<double> t;
        t.rows = a.cols;
        t.cols = a.rows;
        std::vector<int> src;
        transposeCsr(a.rows, a.cols, rs, ci, t.rowStart, t.col, src);
        t.val.resize(src.size());
        for (size_t k = 0; k < src.size(); k++)
            t.val[k] = v[src[k]];
        return t;
    }

    // y = alpha A x + beta y through the SELL copy
    void spmvF64(const DevCsr<double> & a, const double * x, double * y, double alpha, double beta, cudaStream_t s)
    {
        sellSpmv<double>(a.sell, x, y, alpha, beta, s);
    }

    // gridSum epilogue: *acc += *total (the total has just been written)
    struct AccumEpi
    {
        const double * total;
        double * acc;
        __device__ void operator()() const { *acc += *total; }
    };

    // Coefficients of the force functional (one thread: fixed order, same bits every run):
    // F_x = nu wV.u_x + wPx.p,  F_y = nu wV.u_y + wPy.p  (stepper numbering; Dirichlet p = 0)
    __global__ void kForceWeights(const ForcePoint * __restrict__ pts, int npts, double * wV, double * wPx,
                                  double * wPy)
    {
        if (blockIdx.x != 0 || threadIdx.x != 0)
            return;
        for (int i = 0; i < npts; i++)
        {
            const ForcePoint & q = pts[i];
            for (int k = 0; k < 6; k++)
                wV[q.v[k]] += q.w * (q.gx[k] * q.nx + q.gy[k] * q.ny);
            for (int k = 0; k < 3; k++)
                if (q.p[k] >= 0)
                {
                    wPx[q.p[k]] -= q.w * q.psi[k] * q.nx;
                    wPy[q.p[k]] -= q.w * q.psi[k] * q.ny;
                }
        }
    }

    // Start of one reverse step: add the functional's seed at the step's output, reverse the final
    // Dirichlet imposition (lDir collects the x rows), and form the first adjoint mass right-hand
    // side rhs = -tau lw and the pressure seed lpI = cx wPx + cy wPy.
    __global__ void __launch_bounds__(TPB) kAdjSeed(int N, int nI, const double * __restrict__ lam,
                                                     double * __restrict__ lw, double * __restrict__ rhs,
                                                     const unsigned char * __restrict__ isDir,
                                                     double * __restrict__ lDir, const double * __restrict__ wV,
                                                     const double * __restrict__ wPx,
                                                     const double * __restrict__ wPy, double * __restrict__ lpI,
                                                     double cxNu, double cyNu, double cx, double cy, double tau)
    {
        const int n = N > nI ? N : nI;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            if (i < N)
            {
                double lx = lam[i] + cxNu * wV[i], ly = lam[N + i] + cyNu * wV[i];
                if (isDir[i])
                {
                    lDir[i] += lx;
                    lx = 0.0;
                    ly = 0.0;
                }
                lw[i] = lx;
                lw[N + i] = ly;
                rhs[i] = -tau * lx;
                rhs[N + i] = -tau * ly;
            }
            if (i < nI)
                lpI[i] = cx * wPx[i] + cy * wPy[i];
        }
    }

    // Reverse of the tentative Dirichlet imposition on ls, and the second mass right-hand side
    __global__ void __launch_bounds__(TPB) kAdjDirichlet(int N, double * __restrict__ ls, double * __restrict__ rhs,
                                                          const unsigned char * __restrict__ isDir,
                                                          double * __restrict__ lDir, double tau)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        {
            double lx = ls[i], ly = ls[N + i];
            if (isDir[i])
            {
                lDir[i] += lx;
                lx = 0.0;
                ly = 0.0;
                ls[i] = 0.0;
                ls[N + i] = 0.0;
            }
            rhs[i] = -tau * lx;
            rhs[N + i] = -tau * ly;
        }
    }

    // Reverse of rhs = A(u0) [ux uy] and A = nu K + I u0 over the symmetric K pattern (row groups):
    //   lam_c[r] = lv_c[r] + sum_{e in row r} A[T[e]] x_c[col e]      (A^T x, T the transpose map)
    //   lA[e]    = x_x[r] u0_x[col e] + x_y[r] u0_y[col e]
    //   *lnu    += sum_e lA[e] K[e]                                     (deterministic grid sum)
    template <int L>
    __global__ void __launch_bounds__(TPB) kAdjConv(int N, const int * __restrict__ rs, const int * __restrict__ ci,
                                                     const int * __restrict__ T, const double * __restrict__ A,
                                                     const double * __restrict__ K, const double * __restrict__ x,
                                                     const double * __restrict__ u0, const double * __restrict__ lv,
                                                     double * __restrict__ lam, double * __restrict__ lA,
                                                     double * scratch, unsigned * ticket, double * total,
                                                     double * lnu)
    {
        Group<L> g;
        double dot = 0.0;
        for (int r = g.gid; r < N; r += g.ngroups)
        {
            const int b = ldg(rs + r), e = ldg(rs + r + 1);
            const double xr0 = ldg(x + r), xr1 = ldg(x + N + r);
            double s0 = 0.0, s1 = 0.0;
            for (int j = b + g.lane; j < e; j += L)
            {
                const int c = ldg(ci + j);
                const double at = ldg(A + ldg(T + j));
                s0 += at * ldg(x + c);
                s1 += at * ldg(x + N + c);
                const double la = xr0 * ldg(u0 + c) + xr1 * ldg(u0 + N + c);
                lA[j] = la;
                dot += la * ldg(K + j);
            }
            s0 = g.sum(s0);
            s1 = g.sum(s1);
            if (g.lane == 0)
            {
                lam[r] = lv[r] + s0;
                lam[N + r] = lv[N + r] + s1;
            }
        }
        const double v[1] = {dot};
        gridSum<double, 1>(v, scratch, Outs<1>{{total}}, ticket, nullptr, AccumEpi{total, lnu});
    }

    // The initial state's Dirichlet rows hold the Dirichlet values too: move their adjoint to lDir
    __global__ void __launch_bounds__(TPB) kAdjFinish(int N, double * __restrict__ lam,
                                                       const unsigned char * __restrict__ isDir,
                                                       double * __restrict__ lDir)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
            if (isDir[i])
            {
                lDir[i] += lam[i];
                lam[i] = 0.0;
                lam[N + i] = 0.0;
            }
    }

    // out[0] += sum_n wD[n] F[4n] + wL[n] F[4n+1] (J), out[1] += sum_n wD[n] F[4n+2] + wL[n] F[4n+3]
    // (the explicit d/dnu of the viscous term); F[4n..4n+3] = (F_x, F_y, V_x, V_y) of step n.
    // One block, fixed summation order.
    __global__ void __launch_bounds__(TPB) kFunctional(int n, const double * __restrict__ F,
                                                        const double * __restrict__ wD,
                                                        const double * __restrict__ wL, double * out)
    {
        __shared__ double part[2][TPB];
        double j = 0.0, v = 0.0;
        for (int i = threadIdx.x; i < n; i += TPB)
        {
            j += wD[i] * F[4 * i] + wL[i] * F[4 * i + 1];
            v += wD[i] * F[4 * i + 2] + wL[i] * F[4 * i + 3];
        }
        part[0][threadIdx.x] = j;
        part[1][threadIdx.x] = v;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double sj = 0.0, sv = 0.0;
            for (int t = 0; t < TPB; t++)
            {
                sj += part[0][t];
                sv += part[1][t];
            }
            out[0] += sj;
            out[1] += sv;
        }
    }

    // tally[0] = max(tally[0], status of every channel); tally[1] += CG iterations when iters is 1
    // (a plain solve's count) or 2 (the inner FP32 iterations of a refinement solve)
    __global__ void kTally(const SolverState * st, int numCh, int * tally, int iters)
    {
        if (blockIdx.x != 0 || threadIdx.x != 0)
            return;
        for (int c = 0; c < numCh; c++)
        {
            if (st->status[c] > tally[0])
                tally[0] = st->status[c];
            if (iters == 1)
                tally[1] += st->iters[c];
            else if (iters == 2)
                tally[1] += st->innerTotal[c];
        }
    }

    // u[dir] = (dirVal, 0) on the Dirichlet rows
    __global__ void __launch_bounds__(TPB) kImposeDirichlet(int N, double * __restrict__ u,
                                                             const unsigned char * __restrict__ isDir,
                                                             const double * __restrict__ dirVal)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
            if (isDir[i])
            {
                u[i] = dirVal[i];
                u[N + i] = 0.0;
            }
    }
} // namespace

struct nsf_adjoint_s
{
    nsf_chorin S = nullptr;
    nsf_forces F = nullptr;
    nsf_adjoint_config cfg{};
    int N = 0, nI = 0, nnzK = 0;
    DevCsr<double> DT, GT, IT; // D^T (2N x nI), G^T (nI x 2N), I^T (2N x nnz K)
    DevBuf<int> T;             // transpose map of the K pattern
    DevBuf<double> wV, wPx, wPy;
    DevBuf<double> lam, lw, rhs, x, lpI, y, A, lA, lDir;
    DevBuf<double> scal;       // [0] J, [1] dJ/dnu, [2] reduction total
    DevBuf<double> redScratch;
    DevBuf<unsigned> ticket;
    DevBuf<int> tally;         // forward (worst status, -), mass (worst, iterations), pressure (worst, iterations)
    DevBuf<double> forcesLog, wD, wL;
    DevBuf<double> ckU, ckP, segU, finU, finP;
    PcgSolver<double, 2> mass;
    PcgSolver<double, 1> pres;
    MixedPcg<2> mmass; // the solves of a NSF_PREC_F64_MIXEDSOLVE stepper: FP32 CG, FP64 residuals
    ChebSolver cmass;  // the mass solve of a velMethod 3 stepper
    MixedPcg<1> mpres;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<double> hwD, hwL;
    double stats[10] = {0};

    ~nsf_adjoint_s()
    {
        for (cudaEvent_t e : ev)
            if (e)
                cudaEventDestroy(e);
    }

    static void ensure(DevBuf<double> & b, size_t n)
    {
        if (b.size() < n)
            b.alloc(n);
    }

    void forwardTallies(cudaStream_t s)
    {
        const SolverState * st[3] = {S->cfg.velMethod == 0 ? S->gsT.st.get() : S->velT.st.get(), S->pres.st.get(),
                                     S->cfg.velMethod == 0 ? S->gsF.st.get() : S->velF.st.get()};
        if (S->mixedSolve)
        {
            st[0] = S->mvelT.st.get();
            st[1] = S->mpres.st.get();
            st[2] = S->mvelF.st.get();
        }
        if (S->cfg.velMethod >= 3)
        {
            st[0] = S->chebT.st.get();
            st[2] = S->chebF.st.get();
        }
        for (int k = 0; k < 3; k++)
            NSF_LAUNCH(kTally, 1, s, st[k], k == 1 ? 1 : 2, tally.get(), 0);
    }

    // M x = rhs (two channels, x from zero) and Kpi y = lpI (y warm), tallied
    void massSolve(cudaStream_t s)
    {
        NSF_CUDA(cudaMemsetAsync(x.get(), 0, sizeof(double) * 2 * N, s));
        if (S->cfg.velMethod == 3)
        {
            cmass.enqueue(s, rhs.get(), x.get(), cfg.maxIters, cfg.tol);
            NSF_LAUNCH(kTally, 1, s, cmass.st.get(), 2, tally.get() + 2, 1);
        }
        else if (S->mixedSolve)
        {
            mmass.enqueue(s, S->body, rhs.get(), x.get(), S->cfg.maxOuter, cfg.tol, cfg.maxIters, S->cfg.innerTol, 1);
            NSF_LAUNCH(kTally, 1, s, mmass.st.get(), 2, tally.get() + 2, 2);
        }
        else
        {
            mass.enqueue(s, S->body, rhs.get(), x.get(), cfg.maxIters, cfg.tol, false, 1);
            NSF_LAUNCH(kTally, 1, s, mass.st.get(), 2, tally.get() + 2, 1);
        }
    }

    void presSolve(cudaStream_t s)
    {
        if (S->mixedSolve)
        {
            mpres.enqueue(s, S->body, lpI.get(), y.get(), S->cfg.maxOuter, cfg.tol, cfg.maxIters, S->cfg.innerTol, 1);
            NSF_LAUNCH(kTally, 1, s, mpres.st.get(), 1, tally.get() + 4, 2);
        }
        else
        {
            pres.enqueue(s, S->body, lpI.get(), y.get(), cfg.maxIters, cfg.tol, false, 1);
            NSF_LAUNCH(kTally, 1, s, pres.st.get(), 1, tally.get() + 4, 1);
        }
    }

    void copyDev(double * dst, const double * src, size_t n, cudaStream_t s)
    {
        NSF_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }

    // one reverse step: lam holds the adjoint of step n's output velocity on entry, of its input
    // velocity u0 on exit
    void reverseStep(int n, const double * u0, cudaStream_t s)
    {
        const double nu = S->cfg.nu, tau = S->cfg.tau;
        const double cx = hwD[n], cy = hwL[n];
        NSF_LAUNCH(kAdjSeed, blocksFor(std::max(N, nI)), s, N, nI, lam.get(), lw.get(), rhs.get(), S->isDir.get(),
                   lDir.get(), wV.get(), wPx.get(), wPy.get(), lpI.get(), cx * nu, cy * nu, cx, cy, tau);
        massSolve(s);
        spmvF64(GT, x.get(), lpI.get(), 1.0, 1.0, s);
        presSolve(s);
        spmvF64(DT, y.get(), lw.get(), -1.0 / tau, 1.0, s);
        NSF_LAUNCH(kAdjDirichlet, blocksFor(N), s, N, lw.get(), rhs.get(), S->isDir.get(), lDir.get(), tau);
        massSolve(s);
        const DevSell<double> & IS = S->I64.sell;
        NSF_LAUNCH((kFastConvSell<double, double, double, double>), IS.blocks(), s, IS.rows, IS.nSlices, IS.ss.get(),
                   IS.perm.get(), IS.ci.get(), IS.v.get(), u0, S->K64.get(), nu, A.get());
        const SweepSystem<double> & M = S->M64;
        NSF_LANES(M.L, NSF_LAUNCH((kAdjConv<LL>), cappedBlocks((long long)N * LL), s, N, M.rsF.get(), M.ciF.get(),
                                  T.get(), A.get(), S->K64.get(), x.get(), u0, lw.get(), lam.get(), lA.get(),
                                  redScratch.get(), ticket.get(), scal.get() + 2, scal.get() + 1));
        spmvF64(IT, lA.get(), lam.get(), 1.0, 1.0, s);
    }

    // ---- binomial checkpointing: the schedule with the fewest recomputed steps for a given number
    // of stored states (the recursion behind Griewank's revolve, solved exactly by dynamic
    // programming): to reverse k steps whose first input state is stored, with s more states
    // available, advance m steps, store that state, reverse the last k - m steps with s - 1 states,
    // restore the first state and reverse the first m steps with s states;
    //   R(1, s) = 0,  R(k, 0) = k (k - 1) / 2,  R(k, s) = min_m  m + R(k - m, s - 1) + R(m, s).
    std::vector<int> binoSplit; // best m for (k, s), row-major over s
    int binoK = 0, binoS = 0;

    void planBinomial(int K, int Smax)
    {
        binoK = K;
        binoS = Smax;
        std::vector<long long> R((size_t)(K + 1) * (Smax + 1), 0);
        binoSplit.assign((size_t)(K + 1) * (Smax + 1), 1);
        auto at = [&](int k, int s) -> long long & { return R[(size_t)s * (K + 1) + k]; };
        for (int k = 1; k <= K; k++)
            at(k, 0) = (long long)k * (k - 1) / 2;
        for (int s = 1; s <= Smax; s++)
            for (int k = 2; k <= K; k++)
            {
                long long best = -1;
                int bm = 1;
                for (int m = 1; m < k; m++)
                {
                    const long long c = m + at(k - m, s - 1) + at(m, s);
                    if (best < 0 || c < best)
                    {
                        best = c;
                        bm = m;
                    }
                }
                at(k, s) = best;
                binoSplit[(size_t)s * (K + 1) + k] = bm;
            }
    }

    void saveState(int slot, cudaStream_t s)
    {
        const size_t twoN = 2 * (size_t)N;
        copyDev(ckU.get() + (size_t)slot * twoN, S->u.get(), twoN, s);
        copyDev(ckP.get() + (size_t)slot * nI, S->pInt.get(), nI, s);
    }

    void restoreState(int slot, cudaStream_t s)
    {
        const size_t twoN = 2 * (size_t)N;
        copyDev(S->u.get(), ckU.get() + (size_t)slot * twoN, twoN, s);
        copyDev(S->pInt.get(), ckP.get() + (size_t)slot * nI, nI, s);
    }

    // reverse steps [l, l + k) with the input state of step l in slot `slot` and in the stepper,
    // s more slots above it free
    void reverseBinomial(int l, int k, int slot, int sFree, cudaStream_t s, long long & recomputed, long long & reversed)
    {
        if (k == 1)
        {
            copyDev(segU.get(), S->u.get(), 2 * (size_t)N, s);
            reverseStep(l, segU.get(), s);
            reversed++;
            return;
        }
        if (sFree == 0)
        {
            for (int n = l + k - 1; n >= l; n--)
            {
                restoreState(slot, s);
                enqueueSteps(S, n - l, s);
                recomputed += n - l;
                copyDev(segU.get(), S->u.get(), 2 * (size_t)N, s);
                reverseStep(n, segU.get(), s);
                reversed++;
            }
            return;
        }
        const int m = binoSplit[(size_t)sFree * (binoK + 1) + k];
        enqueueSteps(S, m, s);
        recomputed += m;
        saveState(slot + 1, s);
        reverseBinomial(l + m, k - m, slot + 1, sFree - 1, s, recomputed, reversed);
        restoreState(slot, s);
        reverseBinomial(l, m, slot, sFree, s, recomputed, reversed);
    }

    void run(int nSteps, cudaStream_t s)
    {
        if (cfg.snapshots > 0)
        {
            runBinomial(nSteps, s);
            return;
        }
        const int C = cfg.checkpointInterval;
        const size_t twoN = 2 * (size_t)N;
        const int nCk = C > 0 ? (nSteps + C - 1) / C : 0;
        const int segLen = C > 0 ? std::min(C, nSteps) : nSteps;
        ensure(ckU, std::max(1, nCk) * twoN);
        ensure(ckP, std::max(1, nCk) * (size_t)nI);
        ensure(segU, std::max(1, segLen) * twoN);
        ensure(forcesLog, 4 * (size_t)std::max(1, nSteps));
        wD.upload(hwD);
        wL.upload(hwL);
        NSF_CUDA(cudaMemsetAsync(tally.get(), 0, 6 * sizeof(int), s));
        NSF_CUDA(cudaMemsetAsync(scal.get(), 0, 3 * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(forcesLog.get(), 0, 4 * sizeof(double) * std::max(1, nSteps), s));
        NSF_CUDA(cudaMemsetAsync(lam.get(), 0, twoN * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(lDir.get(), 0, N * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(y.get(), 0, nI * sizeof(double), s));
        NSF_CUDA(cudaEventRecord(ev[0], s));

        // forward: checkpoints (or every input state), the step, the forces of weighted steps
        for (int n = 0; n < nSteps; n++)
        {
            if (C > 0)
            {
                if (n % C == 0)
                {
                    copyDev(ckU.get() + (size_t)(n / C) * twoN, S->u.get(), twoN, s);
                    copyDev(ckP.get() + (size_t)(n / C) * nI, S->pInt.get(), nI, s);
                }
            }
            else
                copyDev(segU.get() + (size_t)n * twoN, S->u.get(), twoN, s);
            enqueueSteps(S, 1, s);
            forwardTallies(s);
            if (hwD[n] != 0.0 || hwL[n] != 0.0)
                NSF_LAUNCH(kForces, 1, s, F->pts.get(), F->npts, S->u.get(), N, S->pInt.get(), S->cfg.nu,
                           forcesLog.get() + 4 * (size_t)n, forcesLog.get() + 4 * (size_t)n + 2);
        }
        copyDev(finU.get(), S->u.get(), twoN, s);
        copyDev(finP.get(), S->pInt.get(), nI, s);
        NSF_LAUNCH(kFunctional, 1, s, nSteps, forcesLog.get(), wD.get(), wL.get(), scal.get());
        NSF_CUDA(cudaEventRecord(ev[1], s));

        // reverse sweep from the last weighted step (later steps leave lam = 0)
        int last = -1;
        for (int n = 0; n < nSteps; n++)
            if (hwD[n] != 0.0 || hwL[n] != 0.0)
                last = n;
        long long recomputed = 0, reversed = 0;
        if (last >= 0)
        {
            if (C == 0)
                for (int n = last; n >= 0; n--, reversed++)
                    reverseStep(n, segU.get() + (size_t)n * twoN, s);
            else
                for (int seg = last / C; seg >= 0; seg--)
                {
                    const int n0 = seg * C, n1 = std::min(n0 + C, last + 1);
                    copyDev(S->u.get(), ckU.get() + (size_t)seg * twoN, twoN, s);
                    copyDev(S->pInt.get(), ckP.get() + (size_t)seg * nI, nI, s);
                    for (int n = n0; n < n1; n++)
                    {
                        copyDev(segU.get() + (size_t)(n - n0) * twoN, S->u.get(), twoN, s);
                        if (n < n1 - 1)
                        {
                            enqueueSteps(S, 1, s);
                            recomputed++;
                        }
                    }
                    for (int n = n1 - 1; n >= n0; n--, reversed++)
                        reverseStep(n, segU.get() + (size_t)(n - n0) * twoN, s);
                }
        }
        NSF_LAUNCH(kAdjFinish, blocksFor(N), s, N, lam.get(), S->isDir.get(), lDir.get());
        NSF_CUDA(cudaEventRecord(ev[2], s));
        // the stepper keeps the state after the forward run
        copyDev(S->u.get(), finU.get(), twoN, s);
        copyDev(S->pInt.get(), finP.get(), nI, s);

        int t[6];
        NSF_CUDA(cudaMemcpyAsync(t, tally.get(), sizeof t, cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        float msF = 0, msB = 0;
        NSF_CUDA(cudaEventElapsedTime(&msF, ev[0], ev[1]));
        NSF_CUDA(cudaEventElapsedTime(&msB, ev[1], ev[2]));
        stats[0] = nSteps;
        stats[1] = (double)recomputed;
        stats[2] = (double)reversed;
        stats[3] = t[3];
        stats[4] = t[5];
        stats[5] = t[0];
        stats[6] = std::max(t[2], t[4]);
        stats[7] = (double)sizeof(double) * ((double)ckU.size() + ckP.size() + segU.size());
        stats[8] = msF;
        stats[9] = msB;
    }

    // the run with binomial checkpointing: the forward pass stores the initial state only; the
    // reverse sweep recomputes by the binomial schedule with cfg.snapshots further states
    void runBinomial(int nSteps, cudaStream_t s)
    {
        const size_t twoN = 2 * (size_t)N;
        int last = -1;
        for (int n = 0; n < nSteps; n++)
            if (hwD[n] != 0.0 || hwL[n] != 0.0)
                last = n;
        const int K = last + 1, Sfree = cfg.snapshots;
        if (K > 1 && (binoK != K || binoS != Sfree))
            planBinomial(K, Sfree);
        ensure(ckU, (size_t)(Sfree + 1) * twoN);
        ensure(ckP, (size_t)(Sfree + 1) * nI);
        ensure(segU, twoN);
        ensure(forcesLog, 4 * (size_t)std::max(1, nSteps));
        wD.upload(hwD);
        wL.upload(hwL);
        NSF_CUDA(cudaMemsetAsync(tally.get(), 0, 6 * sizeof(int), s));
        NSF_CUDA(cudaMemsetAsync(scal.get(), 0, 3 * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(forcesLog.get(), 0, 4 * sizeof(double) * std::max(1, nSteps), s));
        NSF_CUDA(cudaMemsetAsync(lam.get(), 0, twoN * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(lDir.get(), 0, N * sizeof(double), s));
        NSF_CUDA(cudaMemsetAsync(y.get(), 0, nI * sizeof(double), s));
        NSF_CUDA(cudaEventRecord(ev[0], s));
        saveState(0, s);
        for (int n = 0; n < nSteps; n++)
        {
            enqueueSteps(S, 1, s);
            forwardTallies(s);
            if (hwD[n] != 0.0 || hwL[n] != 0.0)
                NSF_LAUNCH(kForces, 1, s, F->pts.get(), F->npts, S->u.get(), N, S->pInt.get(), S->cfg.nu,
                           forcesLog.get() + 4 * (size_t)n, forcesLog.get() + 4 * (size_t)n + 2);
        }
        copyDev(finU.get(), S->u.get(), twoN, s);
        copyDev(finP.get(), S->pInt.get(), nI, s);
        NSF_LAUNCH(kFunctional, 1, s, nSteps, forcesLog.get(), wD.get(), wL.get(), scal.get());
        NSF_CUDA(cudaEventRecord(ev[1], s));
        long long recomputed = 0, reversed = 0;
        if (K > 0)
        {
            restoreState(0, s);
            reverseBinomial(0, K, 0, Sfree, s, recomputed, reversed);
        }
        NSF_LAUNCH(kAdjFinish, blocksFor(N), s, N, lam.get(), S->isDir.get(), lDir.get());
        NSF_CUDA(cudaEventRecord(ev[2], s));
        copyDev(S->u.get(), finU.get(), twoN, s);
        copyDev(S->pInt.get(), finP.get(), nI, s);
        int t[6];
        NSF_CUDA(cudaMemcpyAsync(t, tally.get(), sizeof t, cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        float msF = 0, msB = 0;
        NSF_CUDA(cudaEventElapsedTime(&msF, ev[0], ev[1]));
        NSF_CUDA(cudaEventElapsedTime(&msB, ev[1], ev[2]));
        stats[0] = nSteps;
        stats[1] = (double)recomputed;
        stats[2] = (double)reversed;
        stats[3] = t[3];
        stats[4] = t[5];
        stats[5] = t[0];
        stats[6] = std::max(t[2], t[4]);
        stats[7] = (double)sizeof(double) * ((double)ckU.size() + ckP.size() + segU.size());
        stats[8] = msF;
        stats[9] = msB;
    }
};

extern "C" int nsf_adjoint_create(nsf_chorin S, nsf_forces f, const nsf_adjoint_config * cfg, nsf_adjoint * out)
{
    return guarded([&] {
        require(S && f && out, "null argument");
        require(f->s == S, "the force functional belongs to another stepper");
        require(!S->mixed, "the adjoint needs FP64 operators (precision NSF_PREC_F64 or NSF_PREC_F64_MIXEDSOLVE)");
        require(!S->extrapolate && !S->project,
                "the adjoint's checkpoints hold (u, p) only: create the stepper with pressureGuess 0");
        require(S->cfg.velMethod != 4,
                "the adjoint's checkpoints hold (u, p) only: warm-started mass solves (velMethod 4) are not supported");
        auto a = std::make_unique<nsf_adjoint_s>();
        if (cfg)
            a->cfg = *cfg;
        require(a->cfg.checkpointInterval >= 0, "checkpointInterval must be >= 0");
        require(a->cfg.snapshots >= 0 && a->cfg.snapshots <= 4096, "snapshots must be in 0..4096");
        if (a->cfg.maxIters <= 0)
            a->cfg.maxIters = 20000;
        if (!(a->cfg.tol > 0))
            a->cfg.tol = 1e-13;
        a->S = S;
        a->F = f;
        const int N = S->N, nI = S->nIntP;
        a->N = N;
        a->nI = nI;
        a->nnzK = (int)S->K64.size();
        a->DT.upload(transposedOf(S->D64), true);
        a->GT.upload(transposedOf(S->G64), true);
        a->IT.upload(transposedOf(S->I64), true);
        {
            const std::vector<int> rs = S->M64.rsF.download(), ci = S->M64.ciF.download();
            std::vector<int> trs, tci, src;
            transposeCsr(N, N, rs, ci, trs, tci, src);
            require(trs == rs && tci == ci, "the K pattern is not structurally symmetric");
            a->T.upload(src);
        }
        a->wV.alloc(N);
        a->wPx.alloc(nI);
        a->wPy.alloc(nI);
        NSF_LAUNCH(kForceWeights, 1, S->stream, f->pts.get(), f->npts, a->wV.get(), a->wPx.get(), a->wPy.get());
        const size_t twoN = 2 * (size_t)N;
        a->lam.alloc(twoN);
        a->lw.alloc(twoN);
        a->rhs.alloc(twoN);
        a->x.alloc(twoN);
        a->lpI.alloc(nI);
        a->y.alloc(nI);
        a->A.alloc(a->nnzK);
        a->lA.alloc(a->nnzK);
        a->lDir.alloc(N);
        a->scal.alloc(3);
        a->redScratch.alloc((size_t)cappedBlocks(1ll << 40));
        a->ticket = DevBuf<unsigned>(1);
        a->tally = DevBuf<int>(6);
        a->finU.alloc(twoN);
        a->finP.alloc(nI);
        if (S->cfg.velMethod >= 3)
            a->cmass.setup(&S->M64, &S->Msell, 2);
        else if (S->mixedSolve)
            a->mmass.setup(&S->M64, &S->M32, 2);
        else
            a->mass.setup(&S->M64, 2);
        if (S->mixedSolve)
        {
            a->mpres.setup(&S->Kpi64, &S->Kpi32, 1);
            S->enablePresCoarse(a->mpres.inner);
        }
        else
            a->pres.setup(&S->Kpi64, 1);
        for (cudaEvent_t & e : a->ev)
            NSF_CUDA(cudaEventCreate(&e));
        NSF_CUDA(cudaStreamSynchronize(S->stream));
        *out = a.release();
    });
}

extern "C" int nsf_adjoint_run(nsf_adjoint a, int nSteps, const double * wDrag, const double * wLift, double * result,
                               double * dJdDir, double * dJdU0, void * stream)
{
    return guarded([&] {
        require(a && nSteps >= 0, "bad argument");
        nsf_chorin S = a->S;
        a->hwD.assign(std::max(1, nSteps), 0.0);
        a->hwL.assign(std::max(1, nSteps), 0.0);
        for (int n = 0; n < nSteps; n++)
        {
            if (wDrag)
                a->hwD[n] = wDrag[n];
            if (wLift)
                a->hwL[n] = wLift[n];
            require(std::isfinite(a->hwD[n]) && std::isfinite(a->hwL[n]), "non-finite functional weight");
        }
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        a->run(nSteps, s);
        const int N = a->N;
        double scal[3];
        NSF_CUDA(cudaMemcpy(scal, a->scal.get(), sizeof scal, cudaMemcpyDeviceToHost));
        if (result)
        {
            result[0] = scal[0];
            result[1] = scal[1];
        }
        if (dJdDir)
        {
            const std::vector<double> l = a->lDir.download();
            for (size_t i = 0; i < S->dirRows.size(); i++)
                dJdDir[i] = l[S->dirRows[i]];
        }
        if (dJdU0)
        {
            const std::vector<double> l = a->lam.download();
            for (int r = 0; r < N; r++)
            {
                dJdU0[S->permV[r]] = l[r];
                dJdU0[N + S->permV[r]] = l[N + r];
            }
        }
        if (a->stats[5] == ST_NONFINITE || a->stats[6] == ST_NONFINITE || !std::isfinite(scal[0]) ||
            !std::isfinite(scal[1]))
            throw Error(ST_NONFINITE, "non-finite value in the forward run or the adjoint sweep");
        // a refinement solve (mixed solves) that used up its passes has reached the FP64 residual
        // floor of a tight tolerance: reported in the stats only
        if (a->stats[6] == ST_MAXITER && !S->mixedSolve)
            throw Error(ST_MAXITER, "an adjoint CG solve reached its iteration cap");
        if (a->stats[6] == ST_BREAKDOWN)
            throw Error(ST_BREAKDOWN, "an adjoint CG solve broke down");
    });
}

extern "C" int nsf_adjoint_stats(nsf_adjoint a, double * stats)
{
    return guarded([&] {
        require(a && stats, "null argument");
        std::copy(a->stats, a->stats + 10, stats);
    });
}

extern "C" void nsf_adjoint_destroy(nsf_adjoint a) { delete a; }

// ---------------------------------------------------------------- stepper parameters

extern "C" int nsf_chorin_set_dirichlet(nsf_chorin S, const double * dirVx, void * stream)
{
    return guarded([&] {
        require(S && dirVx, "null argument");
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        std::vector<double> d = S->dirVal.download();
        for (size_t i = 0; i < S->dirRows.size(); i++)
        {
            require(std::isfinite(dirVx[i]), "non-finite Dirichlet value");
            d[S->dirRows[i]] = dirVx[i];
        }
        NSF_CUDA(cudaStreamSynchronize(s));
        S->dirVal.upload(d);
        NSF_LAUNCH(kImposeDirichlet, blocksFor(S->N), s, S->N, S->u.get(), S->isDir.get(), S->dirVal.get());
        NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_chorin_set_nu(nsf_chorin S, double nu)
{
    return guarded([&] {
        require(S && std::isfinite(nu) && nu >= 0, "nu must be finite and >= 0");
        S->cfg.nu = nu;
        // the captured step holds nu as a kernel argument: capture again at the next step
        if (S->exec)
            NSF_CUDA(cudaGraphExecDestroy(S->exec));
        if (S->graph)
            NSF_CUDA(cudaGraphDestroy(S->graph));
        S->exec = nullptr;
        S->graph = nullptr;
    });
}
