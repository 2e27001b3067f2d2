// Host-side solver objects over the device kernels: a color-permuted sweep system, CG
// preconditioned by multicolor symmetric Gauss-Seidel, the reference's multicolor Gauss-Seidel
// solver, and an FP64 iterative-refinement wrapper around an FP32 inner CG.
//
// Every solve is a sequence of "init" kernels followed by a loop whose body is a fixed kernel
// sequence.  Eagerly the host runs the body in chunks of `checkInterval` iterations and polls one
// device flag; under stream capture the loop becomes a conditional WHILE node whose body the first
// kernel of an iteration ends on the device (cudaGraphSetConditional), so a captured time step
// runs with no host synchronisation at all.
#pragma once

#include "cluster.cuh"
#include "cluster_dsmem.cuh"
#include "cluster_eis.cuh"
#include "device.cuh"
#include "host/setup.hpp"
#include "kernels.cuh"

#include <cmath>
#include <functional>
#include <unordered_map>

namespace nsf
{
    // Run `body(stream, conditionalHandle)` as a device-terminated loop.
    inline void deviceLoop(cudaStream_t s, cudaStream_t bodyStream, SolverState * stDev, int maxIters,
                           int checkInterval, PinnedBuf<int> & flag,
                           const std::function<void(cudaStream_t, unsigned long long)> & body)
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        NSF_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs == cudaStreamCaptureStatusActive)
        {
            cudaGraph_t g = nullptr;
            const cudaGraphNode_t * deps = nullptr;
            size_t nd = 0;
            NSF_CUDA(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd));
            cudaGraphConditionalHandle h;
            NSF_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
            cudaGraphNodeParams prm = {};
            prm.type = cudaGraphNodeTypeConditional;
            prm.conditional.handle = h;
            prm.conditional.type = cudaGraphCondTypeWhile;
            prm.conditional.size = 1;
            cudaGraphNode_t node;
            NSF_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &prm));
            cudaGraph_t bodyGraph = prm.conditional.phGraph_out[0];
            NSF_CUDA(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            NSF_CUDA(cudaStreamBeginCaptureToGraph(bodyStream, bodyGraph, nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeRelaxed));
            body(bodyStream, (unsigned long long)h);
            NSF_CUDA(cudaStreamEndCapture(bodyStream, &bodyGraph));
            return;
        }
        int it = 0;
        const int chunk = checkInterval < 1 ? 1 : checkInterval;
        while (it <= maxIters)
        {
            for (int j = 0; j < chunk && it <= maxIters; j++, it++)
                body(s, 0ull);
            NSF_CUDA(cudaMemcpyAsync(flag.get(), &stDev->anyActive, sizeof(int), cudaMemcpyDeviceToHost, s));
            NSF_CUDA(cudaStreamSynchronize(s));
            if (*flag.get() == 0)
                break;
        }
    }

    template <typename T>
    struct SweepSystem
    {
        int n = 0, nnzFull = 0, nColors = 0, L = 4;
        std::vector<int> ps;      // color starts (host), nColors + 1
        std::vector<int> hostRsO; // off-diagonal row offsets (host copy, sizes the cluster kernel)
        std::vector<int> hostCiO; // off-diagonal column indices (host copy, maps columns to CTAs)
        DevBuf<int> rsF, ciF, rsO, ciO;
        DevBuf<T> vF, vO, invD, diag;

        // a: color-permuted square matrix (rows of color c contiguous), ps: color starts
        void build(const HostCsr<double> & a, const std::vector<int> & partStart)
        {
            n = a.rows;
            ps = partStart;
            nColors = (int)ps.size() - 1;
            if (nColors > MAXCOLORS)
                throw Error(ST_NOTSUP, "more than " + std::to_string(MAXCOLORS) + " colors");
            nnzFull = a.nnz();
            std::vector<int> ro(n + 1, 0), co;
            std::vector<T> vo, vf(a.val.begin(), a.val.end()), id(n), dg(n);
            co.reserve(a.nnz());
            vo.reserve(a.nnz());
            for (int r = 0; r < n; r++)
            {
                bool diag = false;
                for (int j = a.rowStart[r]; j < a.rowStart[r + 1]; j++)
                {
                    if (a.col[j] == r)
                    {
                        if (a.val[j] == 0)
                            throw Error(ST_INVALID, "zero on the diagonal at row " + std::to_string(r));
                        id[r] = (T)(1.0 / a.val[j]);
                        dg[r] = (T)a.val[j];
                        diag = true;
                    }
                    else
                    {
                        co.push_back(a.col[j]);
                        vo.push_back((T)a.val[j]);
                    }
                }
                if (!diag)
                    throw Error(ST_INVALID, "missing diagonal at row " + std::to_string(r));
                ro[r + 1] = (int)co.size();
            }
            rsF.upload(a.rowStart);
            ciF.upload(a.col);
            vF.upload(vf);
            rsO.upload(ro);
            ciO.upload(co);
            vO.upload(vo);
            invD.upload(id);
            diag.upload(dg);
            hostRsO = ro;
            hostCiO = co;
            L = lanesFor(a.nnz(), n);
        }

        // capped grid of the phase kernel of color c and of whole-system kernels
        int phaseBlocks(int c) const { return cappedBlocks((long long)(ps[c + 1] - ps[c]) * L); }
        int fullBlocks() const { return cappedBlocks((long long)n * L); }
    };

    // ------------------------------------------------------------------ PCG with multicolor SGS
    template <typename T, int NCH>
    struct PcgSolver
    {
        const SweepSystem<T> * sys = nullptr;
        int numCh = 1;
        DevBuf<T> r, z, p, q;
        DevBuf<double> scratch;
        DevBuf<SolverState> st;
        PcgPtrs P{};
        PinnedBuf<int> flag{1};
        // How a solve runs (one persistent launch per solve except MULTI):
        //   DSMEM   one thread-block cluster, every vector in distributed shared memory (a CTA's
        //           share of the vectors and of the row structure fits: the pressure system);
        //   GRID    a cooperative grid of one CTA per SM, vectors in L2, grid barriers (large
        //           systems: the velocity mass matrix, FP64 solves);
        //   CLUSTER one thread-block cluster, vectors in L2;
        //   MULTI   one kernel per color phase (no co-residency requirement).
        // Chosen automatically in that order of preference (DSMEM, GRID, MULTI); NSF_PCG_PATH =
        // dsmem | dsmem-novals | grid | grid-global | cluster | cluster-global | multikernel forces
        // one (falling back to MULTI when it cannot run).
        enum Path
        {
            MULTI = 0,
            DSMEM = 1,
            GRID = 2,
            CLUSTER = 3
        };
        int path = MULTI;
        int clusterSize = 0;        // CTAs of the cluster (DSMEM, CLUSTER) or of the grid (GRID)
        bool clusterShared = false; // CLUSTER / GRID: row structure cached in shared memory
        size_t clusterSmem = 0;
        DevBuf<int> psDev;
        // DSMEM: 0 matrix values read from global memory, 1 values in shared memory
        int dsVals = -1;
        DsLayout dsLay{};
        // DSMEM: 1 Eisenstat's form with one reduction per iteration (kPcgClusterEis, systems of at
        // least two colours), 0 the classical form (kPcgClusterDs; NSF_PCG_FORM=classic forces it)
        int dsForm = 0;
        EisLayout eisLay{};
        DevBuf<int> cmapDev;
        // GRID: barrier control words and the per-CTA reduction slots
        DevBuf<unsigned> gridCtl;
        DevBuf<T> gridSlots;
        // GRID: lanes per row, 4 for short colour phases (spread over every SM) or 1 when a phase
        // gives every thread several rows (NSF_GRID_LANES=1|4 forces one)
        int gridLanes = 4;
        // FP32 preconditioner of an FP64 solve on the GRID / CLUSTER path (usePrecondF32): the
        // sweeps run on the FP32 values of the same structure, z in FP32
        const SweepSystem<float> * pre32 = nullptr;
        DevBuf<float> z32;
        DevBuf<float> vOLo; // FP64 off-diagonal values minus their FP32 copy: (FP32 copy, vOLo) is a double-float

        bool setupDsmem(const SweepSystem<T> * s, bool allowVals, int form = -1)
        {
            if (form < 0)
                form = (s->nColors >= 2 && envStr("NSF_PCG_FORM", "eisenstat") != "classic") ? 1 : 0;
            for (int cs : {16, 8})
            {
                DsShares D = dsShares(s->ps, s->hostRsO, s->hostCiO, cs);
                if (!dsEncodable(D, s->hostRsO))
                    return false;
                for (int vals = allowVals ? 1 : 0; vals >= 0; vals--)
                {
                    if (form == 1)
                    {
                        const EisLayout lay = eisLayout(D.rowsMax, D.nzMax, NCH, (int)sizeof(T), vals != 0);
                        const bool fits = vals ? clusterFits(kPcgClusterEis<T, NCH, true>, cs, lay.bytes)
                                               : clusterFits(kPcgClusterEis<T, NCH, false>, cs, lay.bytes);
                        if (fits)
                        {
                            clusterSize = cs;
                            dsVals = vals;
                            dsForm = 1;
                            eisLay = lay;
                            clusterSmem = lay.bytes;
                            cmapDev.upload(D.cmap);
                            return true;
                        }
                        continue;
                    }
                    const DsLayout lay = dsLayout(D.rowsMax, D.nzMax, NCH, (int)sizeof(T), vals != 0);
                    const bool fits = vals ? clusterFits(kPcgClusterDs<T, NCH, true>, cs, lay.bytes)
                                           : clusterFits(kPcgClusterDs<T, NCH, false>, cs, lay.bytes);
                    if (fits)
                    {
                        clusterSize = cs;
                        dsVals = vals;
                        dsForm = 0;
                        dsLay = lay;
                        clusterSmem = lay.bytes;
                        cmapDev.upload(D.cmap);
                        return true;
                    }
                }
            }
            return false;
        }

        static size_t smemFor(const SweepSystem<T> * s, int cs)
        {
            size_t m = 0;
            for (int rk = 0; rk < cs; rk++)
                m = std::max(m, clusterSmemBytes(s->ps, s->hostRsO, rk, cs));
            return m;
        }

        bool setupCluster(const SweepSystem<T> * s, bool shared)
        {
            if (shared)
            {
                const size_t s16 = smemFor(s, 16), s8 = smemFor(s, 8);
                clusterSize = pickClusterSize(kPcgSweep<T, NCH, true, ClusterSync<T>>, s16, s8);
                clusterShared = clusterSize > 0;
                clusterSmem = clusterSize == 16 ? s16 : (clusterSize == 8 ? s8 : 0);
            }
            else
                clusterSize = pickClusterSize(kPcgSweep<T, NCH, false, ClusterSync<T>>, 0, 0);
            return clusterSize > 0;
        }

        bool setupGrid(const SweepSystem<T> * s, bool allowShared)
        {
            // one CTA per SM (NSF_GRID_CTAS overrides, at most one per SM)
            int G = smCount();
            const int want = std::atoi(envStr("NSF_GRID_CTAS", "0").c_str());
            if (want > 0 && want < G)
                G = want;
            const size_t sm = smemFor(s, G);
            if (allowShared && gridFits(kPcgSweep<T, NCH, true, GridSync<T>>, sm))
            {
                clusterShared = true;
                clusterSmem = sm;
            }
            else if (gridFits(kPcgSweep<T, NCH, false, GridSync<T>>, 0))
            {
                clusterShared = false;
                clusterSmem = 0;
            }
            else
                return false;
            clusterSize = G;
            gridCtl.alloc(4);
            gridSlots.alloc((size_t)2 * 8 * G);
            const int lanes = std::atoi(envStr("NSF_GRID_LANES", "0").c_str());
            gridLanes = (lanes == 1 || lanes == 4) ? lanes
                        : ((long long)s->n >= (long long)CTPB * G * std::max(1, s->nColors) ? 1 : 4);
            if (!sweepKernelFits<T>(GRID))
                gridLanes = 4;
            return true;
        }

        // Calls f with the kPcgSweep instantiation that a solve with barrier policy Sync (CLUSTER:
        // ClusterSync, GRID: GridSync) and the current setup launches, for a preconditioner of type TP.
        template <typename TP, typename Sync, typename F>
        void withSweepKernel(F && f) const
        {
            if constexpr (std::is_same<Sync, GridSync<T>>::value)
                if (gridLanes == 1)
                {
                    if (clusterShared)
                        f(kPcgSweep<T, NCH, true, Sync, 1, TP>);
                    else
                        f(kPcgSweep<T, NCH, false, Sync, 1, TP>);
                    return;
                }
            if (clusterShared)
                f(kPcgSweep<T, NCH, true, Sync, 0, TP>);
            else
                f(kPcgSweep<T, NCH, false, Sync, 0, TP>);
        }

        // Whether the kernel withSweepKernel<TP> picks can run as the current setup launches it;
        // sets its shared-memory ceiling (and non-portable cluster size), which every instantiation
        // needs before its first launch.
        template <typename TP>
        bool sweepKernelFits(int pth) const
        {
            bool ok = false;
            const size_t smem = clusterShared ? clusterSmem : 0;
            if (pth == GRID)
                withSweepKernel<TP, GridSync<T>>([&](auto k) { ok = gridFits(k, smem); });
            else
                withSweepKernel<TP, ClusterSync<T>>([&](auto k) {
                    ok = pickClusterSize(k, clusterSize == 16 ? smem : kClusterSmemCap + 1,
                                         clusterSize == 8 ? smem : kClusterSmemCap + 1) == clusterSize;
                });
            return ok;
        }

        // Precondition this FP64 solve with the FP32 copy s32 of the system (same structure and
        // numbering): the CG recurrence, A p and the dot products stay FP64, the SGS sweeps run in
        // FP32.  Only on the GRID and CLUSTER paths; returns whether it took effect.
        bool usePrecondF32(const SweepSystem<float> * s32)
        {
            if constexpr (!std::is_same<T, double>::value)
                return false;
            if ((path != GRID && path != CLUSTER) || s32->n != sys->n || s32->nColors != sys->nColors ||
                !sweepKernelFits<float>(path))
                return false;
            // the low parts against the FP32 values the sweeps read, so that the pair is the FP64
            // value to ~48 bits and A z reads the high parts the preconditioner shares
            const std::vector<T> v = sys->vO.download();
            const std::vector<float> hi = s32->vO.download();
            if (hi.size() != v.size())
                return false;
            std::vector<float> lo(v.size());
            for (size_t k = 0; k < v.size(); k++)
                lo[k] = (float)((double)v[k] - (double)hi[k]);
            vOLo.upload(lo);
            z32.alloc((size_t)NCH * sys->n);
            pre32 = s32;
            return true;
        }

        // ---- autotuning (NSF_PCG_PATH=tune): every path that fits is timed and the fastest kept.
        // A candidate is a path and its variant (DSMEM: values in shared memory or not; CLUSTER /
        // GRID: row structure in shared memory or not).
        // opt: DSMEM -- the form (1 Eisenstat's, 0 classical; -1 the default); GRID -- lanes per row
        // (1 or 4; 0 the default rule).
        bool applyCandidate(const SweepSystem<T> * s, int cpath, int variant, int opt = -1)
        {
            path = MULTI;
            clusterSize = 0;
            clusterShared = false;
            clusterSmem = 0;
            dsVals = -1;
            dsForm = 0;
            bool ok = true;
            if (cpath == DSMEM)
                ok = setupDsmem(s, variant != 0, opt) && dsVals == variant && (opt < 0 || dsForm == opt);
            else if (cpath == CLUSTER)
                ok = setupCluster(s, variant != 0) && clusterShared == (variant != 0);
            else if (cpath == GRID)
            {
                ok = setupGrid(s, variant != 0) && clusterShared == (variant != 0);
                if (ok && opt > 0)
                {
                    gridLanes = opt;
                    ok = sweepKernelFits<T>(GRID);
                }
            }
            if (ok)
                path = cpath;
            else
            {
                clusterSize = 0;
                clusterShared = false;
                clusterSmem = 0;
                dsVals = -1;
            }
            return ok;
        }

        // Seconds of one solve of exactly `iters` iterations (tolerance 0) on b, captured as a
        // graph (as the steppers run it) and replayed; the best of three replays after two warm-ups.
        double trialSolve(int iters, const T * b, T * x, cudaStream_t st, cudaStream_t body)
        {
            const long long before = launchCounter().load();
            cudaGraph_t g = nullptr;
            cudaGraphExec_t e = nullptr;
            NSF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            NSF_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * NCH * (size_t)sys->n, st));
            enqueue(st, body, b, x, iters, 0.0, false, 1);
            NSF_CUDA(cudaStreamEndCapture(st, &g));
            launchCounter().fetch_sub(launchCounter().load() - before); // trial kernels are not work
            NSF_CUDA(cudaGraphInstantiate(&e, g, 0));
            cudaEvent_t e0, e1;
            NSF_CUDA(cudaEventCreate(&e0));
            NSF_CUDA(cudaEventCreate(&e1));
            double best = 1e30;
            for (int rep = 0; rep < 5; rep++)
            {
                NSF_CUDA(cudaEventRecord(e0, st));
                NSF_CUDA(cudaGraphLaunch(e, st));
                NSF_CUDA(cudaEventRecord(e1, st));
                NSF_CUDA(cudaStreamSynchronize(st));
                float ms = 0;
                NSF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (rep >= 2)
                    best = std::min(best, 1e-3 * ms);
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaGraphExecDestroy(e);
            cudaGraphDestroy(g);
            return best;
        }

        // Time every candidate on trial solves of 8 and 24 iterations; keep the one with the least
        // fixed + expectIters x per-iteration time.  The choice can differ between runs when two
        // paths are within timing noise (the paths differ only in summation order).
        void tune(const SweepSystem<T> * s, int expectIters)
        {
            const int n = s->n;
            std::vector<T> hb((size_t)NCH * n);
            for (size_t i = 0; i < hb.size(); i++)
                hb[i] = (T)(std::sin(0.37 * (double)i + 0.11) + 0.5);
            DevBuf<T> b, x;
            b.upload(hb);
            x.alloc(hb.size());
            cudaStream_t st = nullptr, body = nullptr;
            NSF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            NSF_CUDA(cudaStreamCreateWithFlags(&body, cudaStreamNonBlocking));
            // (path, variant, opt): the DSMEM cluster in both forms with or without cached values,
            // the cluster and the grid with or without cached structure, the grid with 4 lanes or one
            // thread per row, the multi-kernel path
            const bool eisOk = s->nColors >= 2;
            const int cands[11][3] = {{DSMEM, 1, 1},   {DSMEM, 0, 1}, {DSMEM, 1, 0}, {DSMEM, 0, 0},
                                      {CLUSTER, 1, -1}, {CLUSTER, 0, -1}, {GRID, 1, 4}, {GRID, 1, 1},
                                      {GRID, 0, 4},    {GRID, 0, 1},    {MULTI, 0, -1}};
            int bestPath = MULTI, bestVar = 0, bestOpt = -1;
            double bestCost = 1e30;
            for (const auto & c : cands)
            {
                if (c[0] == DSMEM && c[2] == 1 && !eisOk)
                    continue;
                if (!applyCandidate(s, c[0], c[1], c[2]))
                    continue;
                const double t8 = trialSolve(8, b.get(), x.get(), st, body);
                const double t24 = trialSolve(24, b.get(), x.get(), st, body);
                const double per = std::max(0.0, (t24 - t8) / 16.0), fixed = std::max(0.0, t8 - 8.0 * per);
                const double cost = fixed + expectIters * per;
                if (envFlag("NSF_VERBOSE"))
                    std::fprintf(stderr, "[nsf] tune n=%d path=%d variant=%d opt=%d: %.2f us/iteration + %.1f us\n",
                                 n, c[0], c[1], c[2], 1e6 * per, 1e6 * fixed);
                if (cost < bestCost)
                {
                    bestCost = cost;
                    bestPath = c[0];
                    bestVar = c[1];
                    bestOpt = c[2];
                }
            }
            cudaStreamDestroy(st);
            cudaStreamDestroy(body);
            applyCandidate(s, bestPath, bestVar, bestOpt);
        }

        // expectIters: a typical iteration count of this system's solves (weighs the autotuner's
        // per-iteration against its fixed cost)
        void setup(const SweepSystem<T> * s, int channels, bool tryPersistent = true, int expectIters = 100)
        {
            sys = s;
            numCh = channels;
            const int n = s->n;
            psDev.upload(s->ps);
            r.alloc((size_t)NCH * n);
            z.alloc((size_t)NCH * n);
            p.alloc((size_t)2 * NCH * n);
            q.alloc((size_t)NCH * n);
            scratch.alloc((size_t)2 * MAXCH * cappedBlocks(1ll << 40));
            st.alloc(1);
            P.n = n;
            P.nColors = s->nColors;
            P.scratch = scratch.get();
            P.st = st.get();
            P.cond = 0;
            path = MULTI;
            clusterSize = 0;
            clusterShared = false;
            clusterSmem = 0;
            dsVals = -1;
            const std::string want = envStr("NSF_PCG_PATH", "auto");
            if (tryPersistent && want == "tune")
                tune(s, expectIters);
            else if (tryPersistent && want != "multikernel")
            {
                // "auto-cluster": never the whole-GPU grid, so that independent solvers (batched
                // instances on separate streams) can run side by side
                const bool any = want == "auto", anyCl = want == "auto-cluster";
                if ((any || anyCl || want == "dsmem" || want == "dsmem-novals") &&
                    setupDsmem(s, want != "dsmem-novals"))
                    path = DSMEM;
                else if ((want == "cluster" || want == "cluster-global") && setupCluster(s, want == "cluster"))
                    path = CLUSTER;
                else if (anyCl && (setupCluster(s, true) || setupCluster(s, false)))
                    path = CLUSTER;
                else if ((any || want == "grid" || want == "grid-global") && setupGrid(s, want != "grid-global"))
                    path = GRID;
                if (path == MULTI)
                {
                    clusterSize = 0;
                    clusterShared = false;
                    clusterSmem = 0;
                }
            }
            if (envFlag("NSF_VERBOSE"))
                std::fprintf(stderr,
                             "[nsf] PCG n=%d nnz=%d colors=%d path=%d ctas=%d shared=%d dsvals=%d form=%d smem=%zu "
                             "lanes=%d\n",
                             n, s->nnzFull, s->nColors, path, clusterSize, (int)clusterShared, dsVals, dsForm,
                             clusterSmem, path == GRID ? gridLanes : 1);
        }

        void sgs(cudaStream_t s, PcgPtrs PP, int init, T * x, bool tickLast)
        {
            const SweepSystem<T> & S = *sys;
            const int C = S.nColors;
            T * pbuf = p.get();
            NSF_LANES(S.L, {
                for (int c = 0; c < C; c++)
                    NSF_LAUNCH((kPcgForward<T, LL, NCH>), S.phaseBlocks(c), s, PP, numCh, init, c, S.ps[c],
                               S.ps[c + 1], c == C - 1 ? 1 : 0, (tickLast && C == 1) ? 1 : 0, S.rsO.get(),
                               S.ciO.get(), S.vO.get(), S.invD.get(), x, r.get(), z.get(), pbuf, q.get());
                for (int c = C - 2; c >= 0; c--)
                    NSF_LAUNCH((kPcgBackward<T, LL, NCH>), S.phaseBlocks(c), s, PP, numCh, init, c, S.ps[c],
                               S.ps[c + 1], (tickLast && c == 0) ? 1 : 0, S.rsO.get(), S.ciO.get(), S.vO.get(),
                               S.invD.get(), r.get(), z.get());
            });
        }

        // Solve A x = b (device, planar numCh * n, x = initial guess).
        // setConfig == false: tolerance and cap are already in the device state (written by a
        // preceding kernel, as the refinement loop does).
        void enqueue(cudaStream_t s, cudaStream_t bodyStream, const T * b, T * x, int maxIters, double tol,
                     bool absolute, int checkInterval, bool setConfig = true)
        {
            const SweepSystem<T> & S = *sys;
            if (setConfig)
                NSF_LAUNCH(kSetConfig, 1, s, st.get(), maxIters, absolute ? 1 : 0,
                           absolute ? tol * tol * (double)S.n : tol * tol);
            if (path == DSMEM && dsForm == 1)
            {
                EisPcgArgs<T> A{S.n,         S.nColors,     numCh,        psDev.get(),  S.rsO.get(), S.ciO.get(),
                                S.vO.get(),  cmapDev.get(), S.diag.get(), S.invD.get(), b,           x,
                                st.get(),    P.skip,        eisLay,       0,            0.0,         nullptr,
                                nullptr,     nullptr,       nullptr};
                if (dsVals)
                    launchCluster(kPcgClusterEis<T, NCH, true>, clusterSize, DTPB, eisLay.bytes, s, A);
                else
                    launchCluster(kPcgClusterEis<T, NCH, false>, clusterSize, DTPB, eisLay.bytes, s, A);
                return;
            }
            if (path == DSMEM)
            {
                DsPcgArgs<T> A{S.n,         S.nColors,    numCh,   psDev.get(), S.rsO.get(), S.ciO.get(),
                               S.vO.get(),  cmapDev.get(), S.diag.get(), S.invD.get(), b,    x,
                               st.get(),    P.skip,       dsLay,   0,     0.0,         nullptr,     nullptr,
                               nullptr,     nullptr};
                launchDs(s, A);
                return;
            }
            if (path == CLUSTER || path == GRID)
            {
                if constexpr (std::is_same<T, double>::value)
                    if (pre32)
                    {
                        ClusterPcgArgs<T, float> A{S.n,         S.nColors,       numCh,       psDev.get(),
                                                   S.rsO.get(), S.ciO.get(),     S.vO.get(),  S.diag.get(),
                                                   pre32->vO.get(), vOLo.get(),  pre32->invD.get(), b,
                                                   x,           r.get(),         p.get(),     q.get(),
                                                   z32.get(),   st.get(),        P.skip};
                        launchSweep(s, A);
                        return;
                    }
                ClusterPcgArgs<T> A{S.n,        S.nColors,    numCh,       psDev.get(), S.rsO.get(), S.ciO.get(),
                                    S.vO.get(), S.diag.get(), S.vO.get(), nullptr,     S.invD.get(), b,
                                    x,          r.get(),      p.get(),     q.get(),     z.get(),     st.get(),
                                    P.skip};
                launchSweep(s, A);
                return;
            }
            NSF_LANES(S.L, NSF_LAUNCH((kPcgInit<T, LL, NCH>), S.fullBlocks(), s, P, S.rsF.get(), S.ciF.get(),
                                      S.vF.get(), x, b, r.get()));
            sgs(s, P, 1, x, false);
            NSF_LAUNCH((kPcgStart<NCH>), 1, s, P, numCh);
            deviceLoop(s, bodyStream, st.get(), maxIters, checkInterval, flag,
                       [&](cudaStream_t bs, unsigned long long cond)
                       {
                           PcgPtrs PP = P;
                           PP.cond = cond;
                           NSF_LANES(S.L, NSF_LAUNCH((kPcgDirection<T, LL, NCH>), S.fullBlocks(), bs, PP, numCh,
                                                     S.rsF.get(), S.ciF.get(), S.vF.get(), z.get(), p.get(),
                                                     q.get()));
                           sgs(bs, PP, 0, x, true);
                       });
        }

        // One persistent solve on the CLUSTER or GRID path (the preconditioner's type from A).
        template <typename TP>
        void launchSweep(cudaStream_t s, const ClusterPcgArgs<T, TP> & A)
        {
            const size_t smem = clusterShared ? clusterSmem : 0;
            if (path == CLUSTER)
            {
                const ClusterSync<T> cs{};
                withSweepKernel<TP, ClusterSync<T>>(
                    [&](auto k) { launchCluster(k, clusterSize, CTPB, smem, s, A, cs); });
                return;
            }
            // barrier words start at zero for every solve (a solve that gave up waiting leaves
            // them in an unknown state)
            NSF_CUDA(cudaMemsetAsync(gridCtl.get(), 0, 4 * sizeof(unsigned), s));
            GridSync<T> gs{};
            gs.ctl = gridCtl.get();
            gs.slots = gridSlots.get();
            // NSF_GRID_SPIN_LIMIT: polls of one barrier wait before the solve gives up (default
            // kGridSpinLimit, seconds).  NSF_GRID_TEST_QUIET_CTA="rank:after": test hook, CTA `rank`
            // stops arriving at barriers after `after` of them, so the other CTAs' waits run out and
            // the solve ends with status 5 (both read at each solve; an enqueue under stream
            // capture fixes them for the graph).
            const long long lim = std::atoll(envStr("NSF_GRID_SPIN_LIMIT", "0").c_str());
            if (lim > 0)
                gs.spinLimit = (unsigned)std::min<long long>(lim, 0xFFFFFFFFll);
            const std::string quiet = envStr("NSF_GRID_TEST_QUIET_CTA", "");
            if (!quiet.empty())
            {
                const size_t colon = quiet.find(':');
                gs.quietRank = std::atoi(quiet.substr(0, colon).c_str());
                gs.quietAfter =
                    colon == std::string::npos ? 0u : (unsigned)std::atoi(quiet.substr(colon + 1).c_str());
                if (gs.quietRank < 1 || gs.quietRank >= clusterSize)
                    throw Error(ST_INVALID, "NSF_GRID_TEST_QUIET_CTA: rank must be in 1.." +
                                                std::to_string(clusterSize - 1));
            }
            withSweepKernel<TP, GridSync<T>>([&](auto k) { launchCooperative(k, clusterSize, smem, s, A, gs); });
        }

        int kernelsPerIteration() const { return 2 * sys->nColors; }
        int initKernels() const { return 3 + 2 * sys->nColors - 1; }

        // Whether solveReplaced can run (the DSMEM path of an FP32 solver).
        bool canReplace() const { return path == DSMEM && sizeof(T) == 4 && envFlag("NSF_NO_RU") == 0; }

        // FP32 CG with FP64 residual replacement on the FP64 system s64 (same structure and
        // numbering): b64, x64 (in/out) planar NCH * n doubles; results and statistics written to
        // stOut, whose tolerance and cap a preceding kernel has set.
        void solveReplaced(cudaStream_t s, const SweepSystem<double> & s64, const double * b64, double * x64,
                           SolverState * stOut, double delta2)
        {
            const SweepSystem<T> & S = *sys;
            if (dsForm == 1)
            {
                EisPcgArgs<T> A{S.n,          S.nColors,     numCh,          psDev.get(),    S.rsO.get(), S.ciO.get(),
                                S.vO.get(),   cmapDev.get(), S.diag.get(),   S.invD.get(),   nullptr,     nullptr,
                                stOut,        nullptr,       eisLay,         1,              delta2,      b64,
                                s64.vO.get(), s64.diag.get(), x64};
                if (dsVals)
                    launchCluster(kPcgClusterEis<T, NCH, true>, clusterSize, DTPB, eisLay.bytes, s, A);
                else
                    launchCluster(kPcgClusterEis<T, NCH, false>, clusterSize, DTPB, eisLay.bytes, s, A);
                return;
            }
            DsPcgArgs<T> A{S.n,          S.nColors,     numCh,          psDev.get(),    S.rsO.get(), S.ciO.get(),
                           S.vO.get(),   cmapDev.get(), S.diag.get(),   S.invD.get(),   nullptr,     nullptr,
                           stOut,        nullptr,       dsLay,          1,              delta2,      b64,
                           s64.vO.get(), s64.diag.get(), x64};
            launchDs(s, A);
        }

        // the classical DSMEM kernel, with the coarse correction when it is on
        void launchDs(cudaStream_t s, DsPcgArgs<T> A)
        {
            if (coarse)
            {
                if constexpr (NCH == 1)
                {
                    A.aggStart = aggStartDev.get();
                    A.aggOfRow = aggOfRowDev.get();
                    A.aggRowStart = aggRowStartDev.get();
                    A.aggRows = aggRowsDev.get();
                    A.ainv = ainvDev.get();
                    if (dsVals)
                        launchCluster(kPcgClusterDs<T, NCH, true, true>, clusterSize, DTPB, dsLay.bytes, s, A);
                    else
                        launchCluster(kPcgClusterDs<T, NCH, false, true>, clusterSize, DTPB, dsLay.bytes, s, A);
                }
                return;
            }
            if (dsVals)
                launchCluster(kPcgClusterDs<T, NCH, true>, clusterSize, DTPB, dsLay.bytes, s, A);
            else
                launchCluster(kPcgClusterDs<T, NCH, false>, clusterSize, DTPB, dsLay.bytes, s, A);
        }

        // ---- two-level preconditioner of the DSMEM solve (enableCoarse)
        bool coarse = false;
        DevBuf<int> aggStartDev, aggOfRowDev, aggRowStartDev, aggRowsDev;
        DevBuf<T> ainvDev;

        // z = SGS(r) + P Ac^-1 P^T r: P is the piecewise-constant prolongation of aggregates of rows
        // -- rows with equal key owned by the same CTA (keys group rows that lie close together,
        // e.g. cells of the mesh) -- and Ac = P^T A P, inverted densely in FP64 on the host.  On the
        // DSMEM path in the classical form, for single-channel systems of at least 3 colours (the
        // aggregate sums are formed in the first backward phase and read in the last, so no barrier
        // is added); returns whether it took effect.  With the aggregates of a Poisson-type system at
        // about 80 rows, CG needs several times fewer iterations (the smooth error components that
        // SGS damps slowly are removed by the coarse solve).
        // xy: coordinates of every row (2 per row, the solver's numbering); the aggregates are
        // square cells of about `per` rows, split by CTA, doubled in size until the cluster's shared
        // memory holds the layout
        bool enableCoarse(const std::vector<float> & xy, int per, const std::vector<int> & sizes = {16, 8})
        {
            if constexpr (NCH != 1)
                return false;
            const SweepSystem<T> & S = *sys;
            const int n = S.n;
            if (path != DSMEM || S.nColors < 3 || (int)xy.size() != 2 * n || n < 1)
                return false;
            float x0 = 1e30f, x1 = -1e30f, y0 = 1e30f, y1 = -1e30f;
            for (int i = 0; i < n; i++)
            {
                x0 = std::min(x0, xy[2 * (size_t)i]);
                x1 = std::max(x1, xy[2 * (size_t)i]);
                y0 = std::min(y0, xy[2 * (size_t)i + 1]);
                y1 = std::max(y1, xy[2 * (size_t)i + 1]);
            }
            for (int tries = 0; tries < 4; tries++, per *= 2)
            {
                const double cell = std::sqrt((double)(x1 - x0) * (double)(y1 - y0) * per / n);
                if (!(cell > 0))
                    return false;
                std::vector<int> key(n);
                for (int i = 0; i < n; i++)
                    key[i] = (int)((xy[2 * (size_t)i] - x0) / cell) * 65536 + (int)((xy[2 * (size_t)i + 1] - y0) / cell);
                if (enableCoarseKeys(key, sizes))
                    return true;
            }
            return false;
        }

        bool enableCoarseKeys(const std::vector<int> & key, const std::vector<int> & sizes)
        {
            const SweepSystem<T> & S = *sys;
            const int n = S.n, C = S.nColors;
            const std::vector<T> vO = S.vO.download(), dg = S.diag.download();
            for (int cs : sizes)
            {
                DsShares D = dsShares(S.ps, S.hostRsO, S.hostCiO, cs);
                if (!dsEncodable(D, S.hostRsO))
                    continue;
                // owner CTA, local row and aggregate of every row; aggregates numbered CTA by CTA
                std::vector<int> aggOfRow(n), aggStart(cs + 1, 0), localOf(n);
                std::vector<std::vector<int>> rowsOf;
                int nAgg = 0, aggMax = 0;
                for (int rk = 0; rk < cs; rk++)
                {
                    aggStart[rk] = nAgg;
                    std::unordered_map<int, int> id;
                    int l = 0;
                    for (int c = 0; c < C; c++)
                    {
                        const int len = S.ps[c + 1] - S.ps[c];
                        const int a0 = S.ps[c] + (int)(((long long)len * rk) / cs);
                        const int a1 = S.ps[c] + (int)(((long long)len * (rk + 1)) / cs);
                        for (int i = a0; i < a1; i++, l++)
                        {
                            auto it = id.find(key[i]);
                            if (it == id.end())
                            {
                                it = id.emplace(key[i], nAgg++).first;
                                rowsOf.emplace_back();
                            }
                            aggOfRow[i] = it->second;
                            localOf[i] = l;
                            rowsOf[it->second].push_back(l);
                        }
                    }
                    aggMax = std::max(aggMax, nAgg - aggStart[rk]);
                }
                aggStart[cs] = nAgg;
                DsLayout lay{};
                int vals = -1;
                for (int v = 1; v >= 0 && vals < 0; v--)
                {
                    lay = dsLayout(D.rowsMax, D.nzMax, NCH, (int)sizeof(T), v != 0, nAgg, aggMax);
                    const bool fits = v ? clusterFits(kPcgClusterDs<T, NCH, true, true>, cs, lay.bytes)
                                        : clusterFits(kPcgClusterDs<T, NCH, false, true>, cs, lay.bytes);
                    if (fits)
                        vals = v;
                }
                if (vals < 0)
                    continue;
                // Ac = P^T A P and its inverse (Cholesky, FP64)
                std::vector<double> ac((size_t)nAgg * nAgg, 0.0);
                for (int i = 0; i < n; i++)
                {
                    const int a = aggOfRow[i];
                    ac[(size_t)a * nAgg + a] += (double)dg[i];
                    for (int e = S.hostRsO[i]; e < S.hostRsO[i + 1]; e++)
                        ac[(size_t)a * nAgg + aggOfRow[S.hostCiO[e]]] += (double)vO[e];
                }
                std::vector<double> inv;
                if (!choleskyInverse(ac, nAgg, inv))
                    return false;
                std::vector<int> rowStart(nAgg + 1, 0), rows;
                rows.reserve(n);
                for (int a = 0; a < nAgg; a++)
                {
                    rowStart[a] = (int)rows.size();
                    rows.insert(rows.end(), rowsOf[a].begin(), rowsOf[a].end());
                }
                rowStart[nAgg] = (int)rows.size();
                std::vector<T> invT(inv.begin(), inv.end());
                aggStartDev.upload(aggStart);
                aggOfRowDev.upload(aggOfRow);
                aggRowStartDev.upload(rowStart);
                aggRowsDev.upload(rows);
                ainvDev.upload(invT);
                clusterSize = cs;
                dsVals = vals;
                dsForm = 0;
                dsLay = lay;
                clusterSmem = lay.bytes;
                cmapDev.upload(D.cmap);
                coarse = true;
                if (envFlag("NSF_VERBOSE"))
                    std::fprintf(stderr, "[nsf] PCG coarse correction: %d aggregates (at most %d per CTA), ctas=%d "
                                 "dsvals=%d smem=%u\n", nAgg, aggMax, cs, vals, lay.bytes);
                return true;
            }
            return false;
        }

        // inverse of the SPD matrix a (n x n, row-major) by Cholesky; false if not positive definite
        static bool choleskyInverse(const std::vector<double> & a, int n, std::vector<double> & inv)
        {
            std::vector<double> L(a);
            for (int j = 0; j < n; j++)
            {
                double d = L[(size_t)j * n + j];
                for (int k = 0; k < j; k++)
                    d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
                if (!(d > 0))
                    return false;
                d = std::sqrt(d);
                L[(size_t)j * n + j] = d;
                for (int i = j + 1; i < n; i++)
                {
                    double v = L[(size_t)i * n + j];
                    for (int k = 0; k < j; k++)
                        v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
                    L[(size_t)i * n + j] = v / d;
                }
            }
            // inv = L^-T L^-1, column by column of the identity
            inv.assign((size_t)n * n, 0.0);
            std::vector<double> y(n);
            for (int c = 0; c < n; c++)
            {
                for (int i = 0; i < n; i++)
                {
                    double v = i == c ? 1.0 : 0.0;
                    for (int k = 0; k < i; k++)
                        v -= L[(size_t)i * n + k] * y[k];
                    y[i] = v / L[(size_t)i * n + i];
                }
                for (int i = n - 1; i >= 0; i--)
                {
                    double v = y[i];
                    for (int k = i + 1; k < n; k++)
                        v -= L[(size_t)k * n + i] * inv[(size_t)k * n + c];
                    inv[(size_t)i * n + c] = v / L[(size_t)i * n + i];
                }
            }
            return true;
        }
    };

    // ------------------------------------------------------------------ multicolor GS ("gs")
    template <typename T, int NCH>
    struct GsSolver
    {
        const SweepSystem<T> * sys = nullptr;
        int numCh = 1, interval = 1;
        DevBuf<double> scratch;
        DevBuf<SolverState> st;
        GsPtrs P{};
        PinnedBuf<int> flag{1};

        void setup(const SweepSystem<T> * s, int channels, int checkInterval)
        {
            sys = s;
            numCh = channels;
            interval = checkInterval < 1 ? 1 : checkInterval;
            scratch.alloc((size_t)2 * MAXCH * cappedBlocks(1ll << 40));
            st.alloc(1);
            P.n = s->n;
            P.scratch = scratch.get();
            P.st = st.get();
            P.cond = 0;
            P.interval = interval;
        }

        void enqueue(cudaStream_t s, cudaStream_t bodyStream, const T * b, T * x, int maxIters, double tol,
                     bool absolute, int hostCheck)
        {
            const SweepSystem<T> & S = *sys;
            const double tol2 = absolute ? tol * tol * (double)S.n : tol * tol;
            NSF_LAUNCH(kSetConfig, 1, s, st.get(), maxIters, absolute ? 1 : 0, tol2);
            NSF_LAUNCH((kGsInit<T, NCH>), cappedBlocks(S.n), s, P, numCh, b);
            NSF_LAUNCH((kGsStart<NCH>), 1, s, P, numCh);
            deviceLoop(s, bodyStream, st.get(), maxIters, hostCheck, flag,
                       [&](cudaStream_t bs, unsigned long long cond)
                       {
                           GsPtrs PP = P;
                           PP.cond = cond;
                           NSF_LANES(S.L, {
                               for (int c = 0; c < S.nColors; c++)
                                   NSF_LAUNCH((kGsPhase<T, LL, NCH>), S.phaseBlocks(c), bs, PP, numCh, S.ps[c],
                                              S.ps[c + 1], c == 0 ? 1 : 0, S.rsO.get(), S.ciO.get(), S.vO.get(),
                                              S.invD.get(), b, x);
                               NSF_LAUNCH((kGsCheck<T, LL, NCH>), S.fullBlocks(), bs, PP, numCh, S.rsF.get(),
                                          S.ciF.get(), S.vF.get(), b, x);
                           });
                       });
        }

        int kernelsPerIteration() const { return sys->nColors + 1; }
        int initKernels() const { return 3; }
    };

    // ------------------------------------------------------------------ FP64 refinement, FP32 inner
    template <int NCH>
    struct MixedPcg
    {
        const SweepSystem<double> * sys64 = nullptr;
        PcgSolver<float, NCH> inner;
        int numCh = 1;
        DevBuf<float> b32, d32;
        DevBuf<double> scratch;
        DevBuf<SolverState> st;
        PinnedBuf<int> flag{1};
        // Systems too large for the cluster-resident residual replacement (one channel on the GRID
        // or CLUSTER path): one CG with the FP64 recurrence and A p and the FP32 SGS preconditioner,
        // followed by the FP64 residual test (and FP32 refinement passes if it stopped short).  FP32
        // values in A p or FP32 vectors delay CG on ill-conditioned systems (1.5-2.9x the FP64
        // iterations on the 1M-row P1 Laplacian family with residual replacement, 2x with restarted
        // passes); an FP32 preconditioner alone does not.  NSF_MIXED_FORM=refine turns it off.
        PcgSolver<double, NCH> pre32Solve;
        bool pre32Form = false;

        void setup(const SweepSystem<double> * s64, const SweepSystem<float> * s32, int channels,
                   int expectIters = 100)
        {
            sys64 = s64;
            numCh = channels;
            inner.setup(s32, channels, true, expectIters);
            b32.alloc((size_t)NCH * s64->n);
            d32.alloc((size_t)NCH * s64->n);
            scratch.alloc((size_t)2 * MAXCH * cappedBlocks(1ll << 40));
            st.alloc(1);
            pre32Form = false;
            if constexpr (NCH == 1)
                if (!inner.canReplace() && (inner.path == inner.GRID || inner.path == inner.CLUSTER) &&
                    envStr("NSF_MIXED_FORM", "auto") != "refine")
                {
                    pre32Solve.setup(s64, channels, true, expectIters);
                    pre32Form = pre32Solve.usePrecondF32(s32);
                }
        }

        // Passes of: r = b - A x in FP64 (also the FP32 inner right-hand side) -> stop decision ->
        // FP32 inner PCG from zero -> x += d in FP64.  The stop decision is a sticky device flag
        // (SolverState::skip) that turns the remaining passes into early exits, so the pass count
        // is fixed at enqueue time and the whole solve can be captured.
        void enqueue(cudaStream_t s, cudaStream_t bodyStream, const double * b, double * x, int maxOuter,
                     double tol, int innerMaxIters, double innerTol, int checkInterval)
        {
            const SweepSystem<double> & S = *sys64;
            const int n = S.n;
            SolverState * sd = st.get();
            // Residual replacement stops only on a replaced FP64 residual.  Below ~1e-11 relative the
            // FP64 residual b - A x of these systems reaches its own rounding floor, so a tighter
            // target would keep it iterating up to the cap; restarted passes stop after maxOuter.
            if (inner.canReplace() && tol >= 1e-11)
            {
                // one launch: FP32 CG whose residual is replaced by the FP64 one whenever it has
                // dropped by a factor 10 (and before stopping), so the Krylov recurrence survives
                // the precision corrections that a restarted refinement pass would discard
                const double delta = std::atof(envStr("NSF_RU_DELTA", "0.1").c_str());
                NSF_LAUNCH(kSetConfig, 1, s, sd, innerMaxIters * (maxOuter > 0 ? maxOuter : 1), 0, tol * tol);
                inner.solveReplaced(s, S, b, x, sd, delta * delta);
                return;
            }
            NSF_LAUNCH(kSetConfig, 1, s, sd, maxOuter, 0, tol * tol);
            NSF_LAUNCH(kOuterReset, 1, s, sd);
            if constexpr (NCH == 1)
                if (pre32Form)
                {
                    pre32Solve.enqueue(s, bodyStream, b, x, innerMaxIters, tol, false, checkInterval);
                    NSF_LAUNCH(kAddInnerIters, 1, s, sd, (const SolverState *)pre32Solve.st.get(), numCh);
                }
            inner.P.skip = &sd->skip;
            for (int pass = 0; pass <= maxOuter; pass++)
            {
                NSF_LANES(S.L, NSF_LAUNCH((kResidual<LL, NCH>), S.fullBlocks(), s, n, sd, scratch.get(), S.rsF.get(),
                                          S.ciF.get(), S.vF.get(), x, b, b32.get()));
                NSF_LAUNCH((kOuterDecide<NCH>), 1, s, sd, inner.st.get(), numCh, pass, innerTol, innerMaxIters);
                if (pass == maxOuter)
                    break;
                NSF_LAUNCH((kScalePass<NCH>), cappedBlocks((long long)NCH * n), s, n, b32.get(), (const SolverState *)sd);
                NSF_CUDA(cudaMemsetAsync(d32.get(), 0, sizeof(float) * NCH * n, s));
                inner.enqueue(s, bodyStream, b32.get(), d32.get(), innerMaxIters, innerTol, false, checkInterval,
                              false);
                NSF_LAUNCH((kAddScaled<NCH>), cappedBlocks((long long)NCH * n), s, n, x, d32.get(),
                           (const SolverState *)sd);
            }
        }
    };
} // namespace nsf
