// Batched instances: B flows on one mesh (each with its own viscosity, inflow values and state)
// advanced together, every operation of the time step one launch for all instances.
//
// The operators (I, K, M, D, G, Kp_int and their SELL / double-float copies) are read by the
// instances together: in the operator kernels consecutive blocks are the same rows of consecutive
// instances (instance = blockIdx.x % B), so a block of the FastConvection matrix I -- the only
// operator larger than L2 -- is fetched from HBM once and reused from L2 by the other instances'
// blocks of that row range.  Instance vectors are contiguous per instance ([B][len]).  The pressure
// solves are one launch of B thread-block clusters (kPcgClusterEis with instStride), cluster q
// solving instance q.  Each instance runs exactly the kernels' arithmetic of a single stepper with
// the same configuration (mixed precision, Chebyshev mass solves, any pressure guess), so its
// fields equal that stepper's.
//
// No counterpart in the reference: its loop (chorinCuda.cu:236-376) advances one flow.
#pragma once

namespace nsf
{
    // ---- element-wise kernels: grid (blocks, B), blockIdx.y = instance
    __global__ void __launch_bounds__(TPB) kBSplitDf(long long n, const double * __restrict__ x, float2 * __restrict__ y,
                                                      long long stride)
    {
        const long long off = (long long)blockIdx.y * stride;
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            y[off + i] = dfFromDouble(x[off + i]);
    }

    // u <- Dirichlet value / u - tau acc (vectors stride 2n, Dirichlet values stride n)
    __global__ void __launch_bounds__(TPB) kBUpdateVelocity(int n, double * __restrict__ u, const double * __restrict__ acc,
                                                             double tau, const unsigned char * __restrict__ isDir,
                                                             const double * __restrict__ dirVal)
    {
        const long long off = (long long)blockIdx.y * 2 * n;
        const double * dv = dirVal + (long long)blockIdx.y * n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            updateVelocityRow<double>(i, n, u + off, acc + off, tau, isDir, dv);
    }

    // pressure guess 2 p(n-1) - p(n-2) per instance (kExtrapolate's rule), hist[instance]
    __global__ void __launch_bounds__(TPB) kBExtrapolate(int n, double * __restrict__ p, double * __restrict__ prev,
                                                          const int * __restrict__ hist)
    {
        const long long off = (long long)blockIdx.y * n;
        const bool two = hist[blockIdx.y] >= 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        {
            const double cur = p[off + i];
            if (two)
                p[off + i] = 2.0 * cur - prev[off + i];
            prev[off + i] = cur;
        }
    }

    __global__ void kBHistBump(int B, int * hist)
    {
        const int q = blockIdx.x * blockDim.x + threadIdx.x;
        if (q < B && hist[q] < 2)
            hist[q] += 1;
    }

    __global__ void kBSetConfig(int B, SolverState * st, int maxIters, int absMode, double tol2)
    {
        const int q = blockIdx.x * blockDim.x + threadIdx.x;
        if (q < B)
        {
            st[q].maxIters = maxIters;
            st[q].absMode = absMode;
            st[q].tol2 = tol2;
        }
    }

    // ---- operator kernels: 1-D grid of B x blocks, instance = blockIdx.x % B (instance fastest)
    template <int L>
    __global__ void __launch_bounds__(TPB) kBSpmmDf(int B, int rows, const int * __restrict__ rs, const int * __restrict__ ci,
                                                     const float2 * __restrict__ v, long long sv,
                                                     const float2 * __restrict__ X, long long sx,
                                                     double * __restrict__ Y, long long sy)
    {
        const int q = (int)(blockIdx.x % (unsigned)B), blk = (int)(blockIdx.x / (unsigned)B);
        const Group<L> g(blk, (int)(gridDim.x / (unsigned)B));
        spmmDfRows<L, 2>(g, rows, rs, ci, v + q * sv, X + q * sx, rows, Y + q * sy, rows);
    }

    __global__ void __launch_bounds__(TPB) kBFastConvSellDf(int B, int rows, int nSlices, const int * __restrict__ ss,
                                                             const int * __restrict__ perm, const int * __restrict__ ci,
                                                             const float * __restrict__ iv, const float2 * __restrict__ u,
                                                             long long su, const float2 * __restrict__ k,
                                                             const float2 * __restrict__ nu, float2 * __restrict__ a,
                                                             long long sa)
    {
        const int q = (int)(blockIdx.x % (unsigned)B), blk = (int)(blockIdx.x / (unsigned)B);
        const int slice = (int)((blk * (unsigned)blockDim.x + threadIdx.x) >> 5);
        fastConvSellDfSlice(slice, rows, nSlices, ss, perm, ci, iv, u + q * su, k, nu[q], a + q * sa);
    }

    // ---- the mass solves on instance-interleaved vectors: entry (c, i) of instance q at
    // ((c n + i) B + q), so that the instances' values of one row are contiguous.  The right-hand
    // sides and solutions stay instance-major ([B][2n]); 32 x 32 shared-memory tiles transpose them
    // on the way in and out.

    // r = b, d = D^-1 b / theta, x = 0 (chebStartDfRow per instance) from instance-major b
    __global__ void __launch_bounds__(TPB) kBChebStartIl(int n, int B, const double * __restrict__ b,
                                                         const float2 * __restrict__ invD, float2 invTheta,
                                                         float2 * __restrict__ r, float2 * __restrict__ d,
                                                         float2 * __restrict__ x)
    {
        __shared__ double tile[32][33];
        const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, ny = TPB / 32;
        const long long len = 2ll * n, e0 = (long long)blockIdx.x * 32;
        const int q0 = blockIdx.y * 32;
        for (int qq = ty; qq < 32; qq += ny)
        {
            const int q = q0 + qq;
            const long long e = e0 + tx;
            tile[qq][tx] = (q < B && e < len) ? b[(long long)q * len + e] : 0.0;
        }
        __syncthreads();
        for (int ee = ty; ee < 32; ee += ny)
        {
            const long long e = e0 + ee;
            const int q = q0 + tx;
            if (e < len && q < B)
            {
                const float2 id = invD[(int)(e % n)];
                const float2 bi = dfFromDouble(tile[tx][ee]);
                const long long o = e * B + q;
                r[o] = bi;
                d[o] = dfMul(dfMul(bi, id), invTheta);
                x[o] = make_float2(0.f, 0.f);
            }
        }
    }

    // y (instance-major FP64) = x (interleaved double-float)
    __global__ void __launch_bounds__(TPB) kBDfToDoubleIl(int n, int B, const float2 * __restrict__ x,
                                                          double * __restrict__ y)
    {
        __shared__ double tile[32][33];
        const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, ny = TPB / 32;
        const long long len = 2ll * n, e0 = (long long)blockIdx.x * 32;
        const int q0 = blockIdx.y * 32;
        for (int ee = ty; ee < 32; ee += ny)
        {
            const long long e = e0 + ee;
            const int q = q0 + tx;
            tile[ee][tx] = (e < len && q < B) ? dfToDouble(x[e * B + q]) : 0.0;
        }
        __syncthreads();
        for (int qq = ty; qq < 32; qq += ny)
        {
            const int q = q0 + qq;
            const long long e = e0 + tx;
            if (q < B && e < len)
                y[(long long)q * len + e] = tile[tx][qq];
        }
    }

    // One double-float Chebyshev step of instances q0 .. q0 + Bg - 1 (of B).  A warp takes
    // R = 32 / Q consecutive rows of one SELL slice for Q instances (Q = 2^qLog, min(Bg, 32) rounded
    // up to a power of two): the matrix entries are loaded once per row for Q instances and the
    // gathers of neighbouring lanes read contiguous instance values.  Per instance the arithmetic and
    // its order are chebStepDfSlice's, so the results are bitwise those of the single stepper's
    // kernel.
    __global__ void __launch_bounds__(TPB) kBChebStepIl(int B, int q0, int Bg, int qLog, int n, int nSlices,
                                                        const int * __restrict__ ss, const int * __restrict__ perm,
                                                        const int * __restrict__ ci, const float2 * __restrict__ v,
                                                        const float2 * __restrict__ invD,
                                                        const float2 * __restrict__ d, float2 * __restrict__ dn,
                                                        float2 * __restrict__ x, float2 * __restrict__ r, float2 c1,
                                                        float2 c2)
    {
        const int Q = 1 << qLog, R = SELL_C >> qLog;
        const int groups = (Bg + Q - 1) >> qLog;
        const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
        const int lane = threadIdx.x & 31;
        const long long row = (warp / groups) * R + (lane >> qLog);
        const int qg = (int)(warp % groups) * Q + (lane & (Q - 1)), q = q0 + qg;
        if (row >= (long long)nSlices * SELL_C)
            return; // whole warps: R divides the slice height
        const int slice = (int)(row / SELL_C), l = (int)(row % SELL_C);
        const int b0 = ldg(ss + slice), w = (ldg(ss + slice + 1) - b0) / SELL_C;
        const bool act = qg < Bg && row < n;
        // channel planes of the instance: entry j of channel c at dq[c][j B]
        const float2 * dq0 = d + q;
        const float2 * dq1 = d + (long long)n * B + q;
        float2 acc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll 4
        for (int k = 0; k < w; k++)
        {
            const int e = b0 + k * SELL_C + l;
            const int j = ldg(ci + e);
            const float2 a = ldg(v + e);
            if (act)
            {
                const long long o = (long long)j * B;
                acc[0] = dfDotAdd(acc[0], a, ldg(dq0 + o));
                acc[1] = dfDotAdd(acc[1], a, ldg(dq1 + o));
            }
        }
        if (!act)
            return;
        const int i = ldg(perm + row);
        const float2 id = ldg(invD + i);
#pragma unroll
        for (int c = 0; c < 2; c++)
        {
            const long long o = ((long long)c * n + i) * B + q;
            const float2 di = d[o];
            x[o] = dfAdd(x[o], di);
            const float2 ri = dfAdd(r[o], dfNeg(dfDotEnd(acc[c])));
            r[o] = ri;
            dn[o] = dfAdd(dfMul(c1, di), dfMul(c2, dfMul(ri, id)));
        }
    }

    template <typename TM, typename TX, typename TY, typename TA>
    __global__ void __launch_bounds__(TPB) kBSpmvSell(int B, int rows, int nSlices, const int * __restrict__ ss,
                                                       const int * __restrict__ perm, const int * __restrict__ ci,
                                                       const TM * __restrict__ v, const TX * __restrict__ x, long long sx,
                                                       TY * __restrict__ y, long long sy, double alpha, double beta)
    {
        const int q = (int)(blockIdx.x % (unsigned)B), blk = (int)(blockIdx.x / (unsigned)B);
        const int slice = (int)((blk * (unsigned)blockDim.x + threadIdx.x) >> 5);
        spmvSellSlice<TM, TX, TY, TA>(slice, rows, nSlices, ss, perm, ci, v, x + q * sx, y + q * sy, alpha, beta);
    }

    inline dim3 batchGrid(long long threads, int B)
    {
        return dim3((unsigned)blocksFor(threads), (unsigned)B);
    }
} // namespace nsf

struct nsf_batch_s
{
    nsf_chorin tpl = nullptr; // the shared operators, the solver set-up and the state maps
    int B = 0, N = 0, P = 0, nIntP = 0, chebK = 0;
    // instances per group of the mass solves (NSF_BATCH_CHEB_GROUP; default: a power of two whose
    // four Chebyshev vectors fill at most half of L2)
    int chebGroup = 1;
    nsf_chorin_config cfg{};
    DevBuf<float2> nuDf;
    DevBuf<double> u, rhs, acc, rhsP, pInt, pPrev, dirVal, stage;
    DevBuf<int> hist;
    DevBuf<float2> uDf, ADf, xDf, rDf, d0, d1;
    DevBuf<SolverState> pst;
    PressureProjection proj; // pressureGuess 2: one basis per instance
    // the batch's cluster set-up of the pressure solves (smaller clusters than a single solve uses,
    // so that more instances' clusters are co-resident)
    int pcs = 0, pvals = 0;
    EisLayout play{};
    DevBuf<int> pcmap, pps;
    // two-level pressure preconditioner (as the single stepper's): the classical cluster kernel with
    // the coarse correction, its layout and aggregates held by bpres (NSF_PRES_COARSE=0: off)
    PcgSolver<float, 1> bpres;
    bool bcoarse = false;

    // Cluster size of the batched pressure solves: NSF_BATCH_CLUSTER if set, else the smallest of
    // 4, 8, 16 CTAs whose per-CTA share stays within about 2,700 rows (one row per thread and
    // colour at 4 colours, the size at which a single 16-CTA solve of the finest mesh runs) and fits
    // in shared memory.
    void setupPressureClusters()
    {
        const SweepSystem<float> & S = tpl->Kpi32;
        const int want = std::atoi(envStr("NSF_BATCH_CLUSTER", "0").c_str());
        std::vector<int> sizes = want > 0 ? std::vector<int>{want} : std::vector<int>{4, 8, 16};
        for (int cs : sizes)
        {
            if (want <= 0 && cs < 16 && (S.n + cs - 1) / cs > 2700)
                continue;
            DsShares D = dsShares(S.ps, S.hostRsO, S.hostCiO, cs);
            if (!dsEncodable(D, S.hostRsO))
                continue;
            for (int vals = 1; vals >= 0; vals--)
            {
                const EisLayout lay = eisLayout(D.rowsMax, D.nzMax, 1, (int)sizeof(float), vals != 0);
                const bool fits = vals ? clusterFits(kPcgClusterEis<float, 1, true>, cs, lay.bytes)
                                       : clusterFits(kPcgClusterEis<float, 1, false>, cs, lay.bytes);
                if (fits)
                {
                    pcs = cs;
                    pvals = vals;
                    play = lay;
                    pcmap.upload(D.cmap);
                    pps.upload(S.ps);
                    return;
                }
            }
        }
        throw Error(ST_NOTSUP, "no cluster size fits the batched pressure solves");
    }
    std::unique_ptr<PinnedBuf<SolverState>> stat;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernelsPerCapture = 0;
    std::vector<SolverState> last;

    ~nsf_batch_s()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        if (stream)
            cudaStreamDestroy(stream);
        if (tpl)
            nsf_chorin_destroy(tpl);
    }

    // M acc = b for every instance: double-float Chebyshev with the a priori count (the single
    // stepper's velMethod 3 iterations, without its per-solve residual check)
    void massSolve(cudaStream_t s, const double * b, double * x)
    {
        const ChebSolver & ch = tpl->chebT;
        const DevSell<double> & sell = *ch.sell;
        const long long stride = 2ll * N;
        const double theta = 0.5 * (kMassSpecHi + kMassSpecLo), delta = 0.5 * (kMassSpecHi - kMassSpecLo);
        const double sigma = theta / delta;
        const dim3 tiles((unsigned)((stride + 31) / 32), (unsigned)((B + 31) / 32));
        NSF_LAUNCH(kBChebStartIl, tiles, s, N, B, b, (const float2 *)ch.invDDf.get(),
                   ChebSolver::split(1.0 / theta), rDf.get(), d0.get(), xDf.get());
        // the instances in groups of chebGroup, each group's iterations run back to back so that its
        // vectors stay in L2 between iterations
        const int G = std::min(chebGroup, B);
        int qLog = 0;
        while ((1 << qLog) < std::min(G, 32))
            qLog++;
        for (int q0 = 0; q0 < B; q0 += G)
        {
            const int Bg = std::min(G, B - q0);
            const long long warps =
                ((long long)sell.nSlices * SELL_C >> (5 - qLog)) * ((Bg + (1 << qLog) - 1) >> qLog);
            const int blocks = (int)((warps * 32 + TPB - 1) / TPB);
            float2 * dc = d0.get();
            float2 * dn = d1.get();
            double rh = 1.0 / sigma;
            for (int it = 0; it < chebK; it++)
            {
                const double rhoN = 1.0 / (2.0 * sigma - rh);
                NSF_LAUNCH(kBChebStepIl, blocks, s, B, q0, Bg, qLog, N, sell.nSlices, sell.ss.get(), sell.perm.get(),
                           sell.ci.get(), (const float2 *)ch.vDf.get(), (const float2 *)ch.invDDf.get(),
                           (const float2 *)dc, dn, xDf.get(), rDf.get(), ChebSolver::split(rhoN * rh),
                           ChebSolver::split(2.0 * rhoN / delta));
                rh = rhoN;
                std::swap(dc, dn);
            }
        }
        NSF_LAUNCH(kBDfToDoubleIl, tiles, s, N, B, (const float2 *)xDf.get(), x);
    }

    template <bool VALS>
    void pressureSolve(cudaStream_t s)
    {
        const SweepSystem<float> & S = tpl->Kpi32;
        const SweepSystem<double> & S64 = tpl->Kpi64;
        const double delta = std::atof(envStr("NSF_RU_DELTA", "0.1").c_str());
        NSF_LAUNCH(kBSetConfig, (B + 127) / 128, s, B, pst.get(),
                   cfg.presMaxIters * (cfg.maxOuter > 0 ? cfg.maxOuter : 1), 0, cfg.presTol * cfg.presTol);
        if (bcoarse)
        {
            DsPcgArgs<float> A{S.n,          S.nColors,      1,          bpres.psDev.get(), S.rsO.get(),
                               S.ciO.get(),  S.vO.get(),     bpres.cmapDev.get(), S.diag.get(), S.invD.get(),
                               nullptr,      nullptr,        pst.get(),  nullptr,     bpres.dsLay,
                               1,            delta * delta,  rhsP.get(), S64.vO.get(), S64.diag.get(),
                               pInt.get(),   bpres.aggStartDev.get(), bpres.aggOfRowDev.get(),
                               bpres.aggRowStartDev.get(), bpres.aggRowsDev.get(), bpres.ainvDev.get(),
                               (long long)nIntP};
            if (bpres.dsVals)
                launchClusters(kPcgClusterDs<float, 1, true, true>, bpres.clusterSize, B, DTPB, bpres.dsLay.bytes, s,
                               A);
            else
                launchClusters(kPcgClusterDs<float, 1, false, true>, bpres.clusterSize, B, DTPB, bpres.dsLay.bytes,
                               s, A);
            return;
        }
        EisPcgArgs<float> A{S.n,          S.nColors,     1,              pps.get(),   S.rsO.get(),   S.ciO.get(),
                            S.vO.get(),   pcmap.get(),   S.diag.get(),   S.invD.get(), nullptr,       nullptr,
                            pst.get(),    nullptr,       play,           1,           delta * delta, rhsP.get(),
                            S64.vO.get(), S64.diag.get(), pInt.get(),    (long long)nIntP};
        launchClusters(kPcgClusterEis<float, 1, VALS>, pcs, B, DTPB, play.bytes, s, A);
    }

    // The instance group of the mass solves chosen by measurement (NSF_BATCH_CHEB_GROUP=tune, or
    // NSF_PCG_PATH=tune): every power of two up to B is timed on a mass solve of the (zero)
    // right-hand-side buffer, captured as a graph and replayed (two warm-ups, best of three), and the
    // fastest kept.  The solve reads rhs and writes acc, which hold no state before the first step.
    void tuneChebGroup()
    {
        const long long before = launchCounter().load();
        int best = chebGroup;
        double bestT = 1e30;
        for (int g = 1;; g *= 2)
        {
            const int gg = std::min(g, B);
            chebGroup = gg;
            cudaGraph_t gr = nullptr;
            cudaGraphExec_t ex = nullptr;
            NSF_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            massSolve(stream, rhs.get(), acc.get());
            NSF_CUDA(cudaStreamEndCapture(stream, &gr));
            NSF_CUDA(cudaGraphInstantiate(&ex, gr, 0));
            cudaEvent_t e0, e1;
            NSF_CUDA(cudaEventCreate(&e0));
            NSF_CUDA(cudaEventCreate(&e1));
            double t = 1e30;
            for (int rep = 0; rep < 5; rep++)
            {
                NSF_CUDA(cudaEventRecord(e0, stream));
                NSF_CUDA(cudaGraphLaunch(ex, stream));
                NSF_CUDA(cudaEventRecord(e1, stream));
                NSF_CUDA(cudaStreamSynchronize(stream));
                float ms = 0;
                NSF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep >= 2)
                    t = std::min(t, (double)ms);
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaGraphExecDestroy(ex);
            cudaGraphDestroy(gr);
            if (envFlag("NSF_VERBOSE"))
                std::fprintf(stderr, "[nsf] batch tune: %d instances per mass-solve group: %.1f us\n", gg, 1e3 * t);
            if (t < bestT)
            {
                bestT = t;
                best = gg;
            }
            if (gg == B)
                break;
        }
        chebGroup = best;
        launchCounter().fetch_sub(launchCounter().load() - before); // trial kernels are not work
    }

    void enqueueStep(cudaStream_t s)
    {
        nsf_chorin_s & T = *tpl;
        const long long s2 = 2ll * N;
        // 1. A = nu K + I u (double-float), rhs = A [u_x u_y]
        NSF_LAUNCH(kBSplitDf, batchGrid(s2, B), s, s2, (const double *)u.get(), uDf.get(), s2);
        const DevSell<float> & IS = T.I32.sell;
        const long long nnzK = (long long)T.KDf.size();
        NSF_LAUNCH(kBFastConvSellDf, B * blocksFor((long long)IS.nSlices * SELL_C), s, B, IS.rows, IS.nSlices,
                   IS.ss.get(), IS.perm.get(), IS.ci.get(), IS.v.get(), (const float2 *)uDf.get(), s2,
                   (const float2 *)T.KDf.get(), (const float2 *)nuDf.get(), ADf.get(), nnzK);
        NSF_LANES(T.M32.L, NSF_LAUNCH((kBSpmmDf<LL>), B * blocksFor((long long)N * T.M32.L), s, B, N, T.M32.rsF.get(),
                                      T.M32.ciF.get(), (const float2 *)ADf.get(), nnzK, (const float2 *)uDf.get(), s2,
                                      rhs.get(), s2));
        // 2. M acc = rhs ; u = u - tau acc ; Dirichlet
        massSolve(s, rhs.get(), acc.get());
        NSF_LAUNCH(kBUpdateVelocity, batchGrid(N, B), s, N, u.get(), (const double *)acc.get(), cfg.tau, T.isDir.get(),
                   (const double *)dirVal.get());
        // 3. rhsP = -(1/tau) D u ; Kpi pInt = rhsP
        const DevSell<float> & DS = T.D32.sell;
        NSF_LAUNCH((kBSpmvSell<float, double, double, double>), B * blocksFor((long long)DS.nSlices * SELL_C), s, B,
                   DS.rows, DS.nSlices, DS.ss.get(), DS.perm.get(), DS.ci.get(), DS.v.get(), (const double *)u.get(), s2,
                   rhsP.get(), (long long)nIntP, -1.0 / cfg.tau, 0.0);
        if (cfg.pressureGuess == 1)
        {
            NSF_LAUNCH(kBExtrapolate, batchGrid(nIntP, B), s, nIntP, pInt.get(), pPrev.get(), (const int *)hist.get());
            NSF_LAUNCH(kBHistBump, (B + 127) / 128, s, B, hist.get());
        }
        if (cfg.pressureGuess == 2)
            proj.guess(s, rhsP.get(), pInt.get());
        if (pvals)
            pressureSolve<true>(s);
        else
            pressureSolve<false>(s);
        if (cfg.pressureGuess == 2)
            proj.update(s, pInt.get());
        // 4. M acc = G p ; u = u - tau acc ; Dirichlet
        const DevSell<float> & GS = T.G32.sell;
        NSF_LAUNCH((kBSpmvSell<float, double, double, double>), B * blocksFor((long long)GS.nSlices * SELL_C), s, B,
                   GS.rows, GS.nSlices, GS.ss.get(), GS.perm.get(), GS.ci.get(), GS.v.get(), (const double *)pInt.get(),
                   (long long)nIntP, rhs.get(), s2, 1.0, 0.0);
        massSolve(s, rhs.get(), acc.get());
        NSF_LAUNCH(kBUpdateVelocity, batchGrid(N, B), s, N, u.get(), (const double *)acc.get(), cfg.tau, T.isDir.get(),
                   (const double *)dirVal.get());
    }

    void enqueueSteps(int nSteps, cudaStream_t s)
    {
        if (!cfg.useGraph)
        {
            for (int i = 0; i < nSteps; i++)
                enqueueStep(s);
            return;
        }
        if (!exec)
        {
            const long long before = launchCounter().load();
            NSF_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            try
            {
                enqueueStep(stream);
            }
            catch (...)
            {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(stream, &g);
                if (g)
                    cudaGraphDestroy(g);
                throw;
            }
            NSF_CUDA(cudaStreamEndCapture(stream, &graph));
            NSF_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            kernelsPerCapture = launchCounter().load() - before;
            launchCounter().fetch_sub(kernelsPerCapture);
        }
        for (int i = 0; i < nSteps; i++)
        {
            NSF_CUDA(cudaGraphLaunch(exec, s));
            launchCounter().fetch_add(kernelsPerCapture, std::memory_order_relaxed);
        }
    }
};

extern "C" int nsf_batch_create(nsf_context ctx, const nsf_chorin_config * cfg, int nInst, const double * nu,
                                const double * dirVx, nsf_batch * out)
{
    return guarded([&] {
        require(ctx && cfg && out && nu, "null argument");
        require(nInst >= 1 && nInst <= 65535, "nInst must be in 1..65535");
        require(cfg->precision == NSF_PREC_MIXED, "batched instances run in NSF_PREC_MIXED");
        require(cfg->velMethod == 3, "batched instances use velMethod 3 (Chebyshev mass solves)");
        require(cfg->pressureGuess >= 0 && cfg->pressureGuess <= 2, "pressureGuess must be 0, 1 or 2");
        require(cfg->pressureBasis == 0 || (cfg->pressureBasis >= 3 && cfg->pressureBasis <= PROJ_MAXL),
                "pressureBasis must be 0 (250) or 3..256");
        require(cfg->presTol >= 1e-11, "batched pressure solves need presTol >= 1e-11 (FP64 residual replacement)");
        for (int q = 0; q < nInst; q++)
            require(nu[q] >= 0 && std::isfinite(nu[q]), "viscosities must be finite and >= 0");
        auto b = std::make_unique<nsf_batch_s>();
        nsf_chorin_config c0 = *cfg;
        c0.nu = nu[0];
        tlTemplateStepper = true;
        const int st = nsf_chorin_create(ctx, &c0, &b->tpl);
        tlTemplateStepper = false;
        if (st != NSF_OK)
            throw Error(st, lastError);
        nsf_chorin_s & T = *b->tpl;
        b->cfg = T.cfg;
        {
            PcgSolver<float, 1> & in = T.mpres.inner;
            require(in.path == PcgSolver<float, 1>::DSMEM && in.dsForm == 1 && in.canReplace(),
                    "batched pressure solves need the cluster-resident Eisenstat path (NSF_PCG_PATH auto or dsmem)");
        }
        const int B = nInst, N = T.N;
        b->B = B;
        b->N = N;
        b->P = T.P;
        b->nIntP = T.nIntP;
        b->chebK = std::min(b->cfg.velMaxIters, T.chebT.itersFor(b->cfg.velTol));
        {
            int l2 = 0, dev = 0;
            NSF_CUDA(cudaGetDevice(&dev));
            NSF_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
            const long long perInst = 4ll * 2 * b->N * (long long)sizeof(float2);
            long long g = std::max(1ll, (l2 / 2) / perInst);
            int p2 = 1;
            while (2ll * p2 <= g && p2 < 1024)
                p2 *= 2;
            const int want = std::atoi(envStr("NSF_BATCH_CHEB_GROUP", "0").c_str());
            b->chebGroup = want > 0 ? want : p2;
        }
        std::vector<float2> nd(B);
        for (int q = 0; q < B; q++)
            nd[q] = ChebSolver::split(nu[q]);
        b->nuDf.upload(nd);
        // per-instance Dirichlet values (rows of the colored numbering) and initial states
        const std::vector<double> dv0 = T.dirVal.download();
        const size_t nDir = T.dirRows.size();
        std::vector<double> dv((size_t)B * N, 0.0), u0((size_t)B * 2 * N, 0.0);
        for (int q = 0; q < B; q++)
        {
            double * d = dv.data() + (size_t)q * N;
            if (dirVx)
                for (size_t i = 0; i < nDir; i++)
                    d[T.dirRows[i]] = dirVx[(size_t)q * nDir + i];
            else
                std::copy(dv0.begin(), dv0.end(), d);
            for (size_t i = 0; i < nDir; i++)
                u0[(size_t)q * 2 * N + T.dirRows[i]] = d[T.dirRows[i]];
        }
        b->dirVal.upload(dv);
        b->u.upload(u0);
        const size_t s2 = (size_t)B * 2 * N, sp = (size_t)B * T.nIntP;
        b->rhs.alloc(s2);
        b->acc.alloc(s2);
        b->uDf.alloc(s2);
        b->xDf.alloc(s2);
        b->rDf.alloc(s2);
        b->d0.alloc(s2);
        b->d1.alloc(s2);
        b->ADf.alloc((size_t)B * T.KDf.size());
        b->rhsP.alloc(sp);
        b->pInt.alloc(sp);
        if (b->cfg.pressureGuess == 1)
        {
            b->pPrev.alloc(sp);
            b->hist.alloc(B);
        }
        b->pst.alloc(B);
        b->setupPressureClusters();
        if (envStr("NSF_PRES_COARSE", "1") != "0" && !ctx->c.pXY.empty() && T.Kpi32.nColors >= 3)
        {
            // the coarse correction on mesh cells, with the batch's cluster size (the smallest of
            // 4, 8, 16 that holds the layout, or NSF_BATCH_CLUSTER)
            const int per = std::max(8, std::atoi(envStr("NSF_PRES_COARSE_ROWS", "240").c_str()));
            std::vector<float> xy(2 * (size_t)T.nIntP);
            for (int r = 0; r < T.nIntP; r++)
            {
                const int node = ctx->c.intP[T.permP[r]];
                xy[2 * (size_t)r] = ctx->c.pXY[2 * (size_t)node];
                xy[2 * (size_t)r + 1] = ctx->c.pXY[2 * (size_t)node + 1];
            }
            const int want = std::atoi(envStr("NSF_BATCH_CLUSTER", "0").c_str());
            b->bpres.setup(&T.Kpi32, 1, true, 100);
            b->bcoarse = b->bpres.path == PcgSolver<float, 1>::DSMEM &&
                         b->bpres.enableCoarse(xy, per, want > 0 ? std::vector<int>{want} : std::vector<int>{4, 8, 16});
        }
        if (b->cfg.pressureGuess == 2)
            b->proj.setup(&T.Kpi64, b->cfg.pressureBasis > 0 ? b->cfg.pressureBasis : 250, B);
        b->stage.alloc(2 * (size_t)N + T.P);
        b->stat = std::make_unique<PinnedBuf<SolverState>>(B);
        b->last.resize(B);
        NSF_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        if (envStr("NSF_BATCH_CHEB_GROUP", "0") == "tune" || envStr("NSF_PCG_PATH", "auto") == "tune")
            b->tuneChebGroup();
        NSF_CUDA(cudaDeviceSynchronize());
        *out = b.release();
    });
}

extern "C" int nsf_batch_step(nsf_batch b, int nSteps, void * stream)
{
    return guarded([&] {
        require(b && nSteps >= 0, "bad argument");
        cudaStream_t s = stream ? asStream(stream) : b->stream;
        b->enqueueSteps(nSteps, s);
        if (nSteps == 0)
            return;
        NSF_CUDA(cudaMemcpyAsync(b->stat->get(), b->pst.get(), sizeof(SolverState) * b->B, cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        std::copy(b->stat->get(), b->stat->get() + b->B, b->last.begin());
        for (int q = 0; q < b->B; q++)
            if (b->last[q].status[0] == ST_NONFINITE)
                throw Error(ST_NONFINITE, "non-finite pressure residual in instance " + std::to_string(q));
    });
}

extern "C" int nsf_batch_launch(nsf_batch b, int nSteps, void * stream)
{
    return guarded([&] {
        require(b && nSteps >= 0, "bad argument");
        b->enqueueSteps(nSteps, stream ? asStream(stream) : b->stream);
    });
}

extern "C" int nsf_batch_get_state(nsf_batch b, int inst, double * uOut, double * pOut, void * stream)
{
    return guarded([&] {
        require(b && inst >= 0 && inst < b->B, "bad argument");
        nsf_chorin S = b->tpl;
        cudaStream_t s = stream ? asStream(stream) : b->stream;
        stateMaps(S);
        const int N = b->N;
        double * su = b->stage.get(), * sp = su + 2 * (size_t)N;
        if (uOut)
        {
            NSF_LAUNCH((kScatterPerm<double>), blocksFor(N), s, N, 2, S->permVDev.get(),
                       (const double *)b->u.get() + (size_t)inst * 2 * N, su);
            NSF_CUDA(cudaMemcpyAsync(uOut, su, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, s));
        }
        if (pOut)
        {
            NSF_CUDA(cudaMemsetAsync(sp, 0, sizeof(double) * b->P, s));
            NSF_LAUNCH((kScatterPerm<double>), blocksFor(b->nIntP), s, b->nIntP, 1, S->pIdxDev.get(),
                       (const double *)b->pInt.get() + (size_t)inst * b->nIntP, sp);
            NSF_CUDA(cudaMemcpyAsync(pOut, sp, sizeof(double) * b->P, cudaMemcpyDeviceToHost, s));
        }
        NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_batch_set_state(nsf_batch b, int inst, const double * uIn, const double * pIn, void * stream)
{
    return guarded([&] {
        require(b && inst >= 0 && inst < b->B, "bad argument");
        nsf_chorin S = b->tpl;
        cudaStream_t s = stream ? asStream(stream) : b->stream;
        stateMaps(S);
        const int N = b->N;
        double * su = b->stage.get(), * sp = su + 2 * (size_t)N;
        if (uIn)
        {
            NSF_CUDA(cudaMemcpyAsync(su, uIn, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, s));
            NSF_LAUNCH((kGatherPerm<double>), blocksFor(N), s, N, 2, S->permVDev.get(), (const double *)su,
                       b->u.get() + (size_t)inst * 2 * N);
        }
        if (pIn)
        {
            NSF_CUDA(cudaMemcpyAsync(sp, pIn, sizeof(double) * b->P, cudaMemcpyHostToDevice, s));
            NSF_LAUNCH((kGatherPerm<double>), blocksFor(b->nIntP), s, b->nIntP, 1, S->pIdxDev.get(), (const double *)sp,
                       b->pInt.get() + (size_t)inst * b->nIntP);
        }
        if (b->hist.get()) // a new pressure history for this instance
            NSF_CUDA(cudaMemsetAsync(b->hist.get() + inst, 0, sizeof(int), s));
        if (b->cfg.pressureGuess == 2)
            b->proj.reset(s, inst);
        NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_batch_stats(nsf_batch b, int inst, double * stats)
{
    return guarded([&] {
        require(b && stats && inst >= 0 && inst < b->B, "bad argument");
        const SolverState & L = b->last[inst];
        stats[0] = L.innerTotal[0];
        stats[1] = L.bb[0] > 0 ? std::sqrt(std::max(0.0, L.lastRR[0]) / L.bb[0]) : 0.0;
        stats[2] = L.iters[0];
        stats[3] = L.status[0];
    });
}

extern "C" long long nsf_batch_kernels_per_step(nsf_batch b) { return b ? b->kernelsPerCapture : 0; }

extern "C" void nsf_batch_destroy(nsf_batch b) { delete b; }
