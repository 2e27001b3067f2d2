// Cluster-resident CG with the multicolor symmetric Gauss-Seidel preconditioner in Eisenstat's
// form, one reduction per iteration, every vector in distributed shared memory.
//
// Same method as kPcgClusterDs (CG on A x = b preconditioned by M = (D+L) D^-1 (D+U), U = L^T, L the
// entries towards earlier colours), same iterates in exact arithmetic, less work and fewer cluster
// barriers per iteration:
//   * Eisenstat (SIAM J. Sci. Stat. Comput. 2, 1981): with W = D + L, CG preconditioned by M on A is
//     CG preconditioned by D^-1 (z = D r~) on A~ = W^-1 A W^-T in the variables x~ = W^T x, and
//     A~ v = t + W^-1 (v - D t) with t = W^-T v, because A = W + W^T - D.  One product with A~ is
//     one backward and one forward colour sweep over half of the off-diagonal entries each; the
//     SpMV of the classical form disappears.  With v = u = D r~ the products simplify to
//       backward  t_i = r~_i - d_i^-1 sum_{j later colour} a_ij t_j
//       forward   f_i = r~_i - t_i - d_i^-1 sum_{j earlier colour} a_ij f_j,  w_i = t_i + f_i,
//     and t of the last colour is r~ itself.
//   * Chronopoulos & Gear (J. Comput. Appl. Math. 25, 1989): s = A~ p is carried by the recurrence
//     s = w + beta s, so gamma = r~.u and delta = w.u are the only dot products and they share one
//     cluster reduction; alpha = gamma / (delta - beta gamma / alpha_prev).
//   * The true residual r = b - A x equals W r~ = D r~ + L r~; its norm (the stopping test, as in the
//     classical form) is accumulated in the forward sweep from the same gathered entries.
// Phases of one iteration with C >= 2 colours (each ends in a cluster barrier, the last in the
// reduction): [update all rows; backward sweep of colour C-2, whose later neighbours (colour C-1)
// are evaluated from their previous r~, w, s and this iteration's alpha, beta] [backward sweeps
// C-3 .. 1] [backward and forward sweep of colour 0] [forward sweeps 1 .. C-1].  Colour C-1 rows
// publish t = r~_new in the first phase and write their own update in the second, so no value is
// read and written in the same phase.  C = 4 (the pressure systems here): 6 phases, against 8
// (2 of them reductions) in the classical form.
// The solve ends with x = x0 + W^-T x~ (one backward sweep).  FP64 residual replacement (T = float)
// as in kPcgClusterDs: the FP32 recurrence runs on gsc * (b - A x64); at a replacement x~ is folded
// into x64 through W^-T, r~ = W^-1 (gsc (b64 - A64 x64)) is recomputed, and alpha is taken from an
// explicit p.A~p reduction (the Krylov direction is kept).
#pragma once

#include "cluster_dsmem.cuh"

namespace nsf
{
    // Byte layout of the dynamic shared memory of one CTA of kPcgClusterEis (the same in every CTA).
    // TF holds t (backward sweeps) and then f (forward sweeps); off-diagonal entries address TF in
    // the owner CTA, the other gathered vector (RT = r~) sits at a fixed offset from it.
    struct EisLayout
    {
        int stride;
        unsigned offTF, offRT, offXT, offP, offS, offW, offInvD, offDiag, offRs, offAd, offV, bytes;
    };

    inline EisLayout eisLayout(int rowsMax, int nzMax, int nch, int tsize, bool vals)
    {
        EisLayout L{};
        L.stride = (rowsMax + 3) & ~3;
        const size_t plane = (size_t)L.stride * tsize;
        size_t o = 0;
        unsigned * vec[6] = {&L.offTF, &L.offRT, &L.offXT, &L.offP, &L.offS, &L.offW};
        for (unsigned * v : vec)
        {
            *v = (unsigned)o;
            o += dsAlign(plane * nch);
        }
        L.offInvD = (unsigned)o;
        o += dsAlign(plane);
        L.offDiag = (unsigned)o;
        o += dsAlign(plane);
        L.offRs = (unsigned)o;
        o += dsAlign((size_t)4 * (rowsMax + 1));
        L.offAd = (unsigned)o;
        o += dsAlign((size_t)4 * nzMax);
        L.offV = (unsigned)o;
        if (vals)
            o += dsAlign((size_t)tsize * nzMax);
        L.bytes = (unsigned)o;
        return L;
    }

    template <typename T>
    struct EisPcgArgs
    {
        int n, nColors, numCh;
        const int * ps;
        const int * rsO;
        const int * ciO;
        const T * vO;
        const int * cmap;
        const T * diag;
        const T * invD;
        const T * b;
        T * x;
        SolverState * st;
        const int * skip;
        EisLayout lay;
        int ru; // FP64 residual replacement (T = float), as DsPcgArgs
        double ruDelta2;
        const double * b64;
        const double * vO64;
        const double * diag64;
        double * x64;
        // several clusters in one launch (batched instances of one system): cluster q solves the
        // system of instance q, its vectors (b, x, b64, x64) at q * instStride and its state at st + q
        long long instStride;
    };

    // The s and r~ updates of one CG step.  The owner of a row and its neighbours (which evaluate the
    // new r~ of a last-colour row from its previous values) call the same function, so both obtain
    // the same bits.
    __device__ __forceinline__ float eisFma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ __forceinline__ double eisFma(double a, double b, double c) { return __fma_rn(a, b, c); }

    template <typename T>
    __device__ __forceinline__ T eisNextS(T w, T s, T beta)
    {
        return eisFma(beta, s, w);
    }

    template <typename T>
    __device__ __forceinline__ T eisNextR(T r, T sNew, T alpha)
    {
        return eisFma(-alpha, sNew, r);
    }

    // acc[c] += sum over local entries [jb, je) of a_j V[c][col_j], V at byte offset `off` from TF
    template <typename T, int NCH, bool VALS>
    __device__ __forceinline__ void eisGather1(const unsigned * lad, const T * lv, const T * vOg, int jb, int je,
                                               unsigned off, unsigned chBytes, const bool (&act)[NCH],
                                               T (&acc)[NCH])
    {
        for (int j0 = jb; j0 < je; j0 += DRB)
        {
            unsigned ad[DRB];
            T v[DRB];
#pragma unroll
            for (int t = 0; t < DRB; t++)
            {
                const bool ok = j0 + t < je;
                ad[t] = ok ? lad[j0 + t] : 0u;
                v[t] = ok ? (VALS ? lv[j0 + t] : ldg(vOg + j0 + t)) : (T)0;
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    T g[DRB];
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                        g[t] = j0 + t < je ? dsLoad(ad[t] + c * chBytes + off, (T)0) : (T)0;
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                        acc[c] += v[t] * g[t];
                }
        }
    }

    // accF[c] += sum a_j TF[c][col_j], accR[c] += sum a_j RT[c][col_j]
    template <typename T, int NCH, bool VALS>
    __device__ __forceinline__ void eisGather2(const unsigned * lad, const T * lv, const T * vOg, int jb, int je,
                                               unsigned offR, unsigned chBytes, const bool (&act)[NCH],
                                               T (&accF)[NCH], T (&accR)[NCH])
    {
        for (int j0 = jb; j0 < je; j0 += DRB)
        {
            unsigned ad[DRB];
            T v[DRB];
#pragma unroll
            for (int t = 0; t < DRB; t++)
            {
                const bool ok = j0 + t < je;
                ad[t] = ok ? lad[j0 + t] : 0u;
                v[t] = ok ? (VALS ? lv[j0 + t] : ldg(vOg + j0 + t)) : (T)0;
            }
#pragma unroll
            for (int c = 0; c < NCH; c++)
                if (act[c])
                {
                    T gf[DRB], gr[DRB];
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                    {
                        const bool ok = j0 + t < je;
                        const unsigned a = ad[t] + c * chBytes;
                        gf[t] = ok ? dsLoad(a, (T)0) : (T)0;
                        gr[t] = ok ? dsLoad(a + offR, (T)0) : (T)0;
                    }
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                    {
                        accF[c] += v[t] * gf[t];
                        accR[c] += v[t] * gr[t];
                    }
                }
        }
    }

    // acc[c] += sum a_j r~new_j with r~new = eisNextR(RT, eisNextS(W, S, beta), alpha) evaluated from the
    // neighbours' previous values (the last-colour t of the first phase)
    template <typename T, int NCH, bool VALS>
    __device__ __forceinline__ void eisGatherNext(const unsigned * lad, const T * lv, const T * vOg, int jb, int je,
                                                  unsigned offR, unsigned offW, unsigned offS, unsigned chBytes,
                                                  const T (&al)[NCH], const T (&be)[NCH], const bool (&act)[NCH],
                                                  T (&acc)[NCH])
    {
        for (int j0 = jb; j0 < je; j0 += DRB)
        {
            unsigned ad[DRB];
            T v[DRB];
#pragma unroll
            for (int t = 0; t < DRB; t++)
            {
                const bool ok = j0 + t < je;
                ad[t] = ok ? lad[j0 + t] : 0u;
                v[t] = ok ? (VALS ? lv[j0 + t] : ldg(vOg + j0 + t)) : (T)0;
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
                            const T r = dsLoad(a + offR, (T)0), w = dsLoad(a + offW, (T)0),
                                    s = dsLoad(a + offS, (T)0);
                            g[t] = eisNextR(r, eisNextS(w, s, be[c]), al[c]);
                        }
                    }
#pragma unroll
                    for (int t = 0; t < DRB; t++)
                        acc[c] += v[t] * g[t];
                }
        }
    }

    // Scalars of the iteration, kept by thread 0 of every CTA (identical in every CTA).
    template <typename T, int NCH>
    struct EisScalars
    {
        T alpha[NCH], beta[NCH];
        int act[NCH], status[NCH], iters[NCH], any;
        double bb[NCH], rr[NCH], gamma[NCH], alphaD[NCH];
        int replace, replacements;
        double rrRef[NCH];
        double gsc[NCH], igsc[NCH];
    };

    template <typename T, int NCH, bool VALS>
    __global__ void __launch_bounds__(DTPB, 1) kPcgClusterEis(EisPcgArgs<T> Ain)
    {
        extern __shared__ __align__(16) unsigned char dsm[];
        cg::cluster_group cl = cg::this_cluster();
        const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
        EisPcgArgs<T> A = Ain;
        {
            const long long inst = (long long)(blockIdx.x / (unsigned)cs), off = inst * A.instStride;
            A.b = A.b ? A.b + off : nullptr;
            A.x = A.x ? A.x + off : nullptr;
            A.b64 = A.b64 ? A.b64 + off : nullptr;
            A.x64 = A.x64 ? A.x64 + off : nullptr;
            A.st += inst;
        }
        __shared__ T slot[2][8];
        __shared__ double dslot[2][8];
        __shared__ int chunkA[MAXCOLORS], chunkL[MAXCOLORS + 1], chunkG[MAXCOLORS], nzBase[MAXCOLORS + 1];
        __shared__ EisScalars<T, NCH> sc;
        int buf = 0, dbuf = 0;
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

        // ---- own rows: chunk `rank` of every colour, as kPcgClusterDs
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
        const EisLayout L = A.lay;
        {
            uint4 * v4 = reinterpret_cast<uint4 *>(dsm);
            const int cnt = (int)(L.offRs / 16);
            for (int t = threadIdx.x; t < cnt; t += DTPB)
                v4[t] = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncthreads();
        const int S = L.stride;
        const unsigned chBytes = (unsigned)(S * sizeof(T));
        T * tf = reinterpret_cast<T *>(dsm + L.offTF);
        T * rt = reinterpret_cast<T *>(dsm + L.offRT);
        T * xt = reinterpret_cast<T *>(dsm + L.offXT);
        T * pv = reinterpret_cast<T *>(dsm + L.offP);
        T * sv = reinterpret_cast<T *>(dsm + L.offS);
        T * wv = reinterpret_cast<T *>(dsm + L.offW);
        T * invDs = reinterpret_cast<T *>(dsm + L.offInvD);
        T * diags = reinterpret_cast<T *>(dsm + L.offDiag);
        unsigned * lrs = reinterpret_cast<unsigned *>(dsm + L.offRs);
        unsigned * lad = reinterpret_cast<unsigned *>(dsm + L.offAd);
        const T * lv = reinterpret_cast<const T *>(dsm + L.offV);
        const unsigned tfBase = (unsigned)__cvta_generic_to_shared(tf);
        const unsigned offR = L.offRT - L.offTF, offW = L.offW - L.offTF, offS = L.offS - L.offTF;
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
                while (sp < je && ldg(A.ciO + sp) < lo) // sorted columns: earlier colours first
                    sp++;
                lrs[l] = (unsigned)(jb - g0 + nb) | ((unsigned)(sp - jb) << 24);
                invDs[l] = ldg(A.invD + i);
                diags[l] = ldg(A.diag + i);
#pragma unroll
                for (int ch = 0; ch < NCH; ch++)
                    rt[ch * S + l] = (ch < numCh && !A.ru) ? A.x[(size_t)ch * n + i] : (T)0; // x0 for r0
            }
            const int cnt = nzBase[c + 1] - nb;
            for (int t = threadIdx.x; t < cnt; t += DTPB)
            {
                const int e = ldg(A.cmap + g0 + t);
                lad[nb + t] = dsMapa(tfBase + (unsigned)(e & 0xFFFFFF) * (unsigned)sizeof(T), e >> 24);
                if (VALS)
                    reinterpret_cast<T *>(dsm + L.offV)[nb + t] = ldg(A.vO + g0 + t);
            }
        }
        if (threadIdx.x == 0)
            lrs[R] = (unsigned)nzBase[C];
        if (threadIdx.x == 0)
            for (int c = 0; c < NCH; c++)
            {
                sc.gsc[c] = sc.igsc[c] = 1.0;
                sc.alpha[c] = sc.beta[c] = (T)0;
            }
        cl.sync(); // every CTA's x0 and row structure in place

        bool act[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh;

        // row loop over the own rows of colour `col`: f(l, i, jb, jl, je, vOg)
        auto rows = [&](int col, auto && f) {
            const T * vOg = A.vO + (chunkG[col] - nzBase[col]);
            for (int l = chunkL[col] + threadIdx.x; l < chunkL[col + 1]; l += DTPB)
            {
                const unsigned pk = lrs[l];
                const int jb = (int)(pk & 0xFFFFFFu), jl = jb + (int)(pk >> 24);
                const int je = (int)(lrs[l + 1] & 0xFFFFFFu);
                f(l, chunkA[col] + (l - chunkL[col]), jb, jl, je, vOg);
            }
        };

        // ---- FP64 residual into TF, scaled by gsc (ru): tf = gsc (b64 - A64 x64), rrAcc += tf^2,
        // bbAcc += (gsc b64)^2 when withBb.  Neighbours' x64 through L2.
        auto trueResidual = [&](T (&rrAcc)[NCH], T (&bbAcc)[NCH], bool withBb) {
            for (int col = 0; col < C; col++)
                rows(col, [&](int l, int i, int, int, int, const T *) {
                    const int jb = ldg(A.rsO + i), je = ldg(A.rsO + i + 1);
                    const double d = ldg(A.diag64 + i);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh && act[c])
                        {
                            const double * xc = A.x64 + (size_t)c * n;
                            double acc = d * __ldcg(xc + i);
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
                            const T ri = (T)((bi - acc) * g);
                            tf[c * S + l] = ri;
                            rrAcc[c] += ri * ri;
                            if (withBb)
                                bbAcc[c] += (T)(bi * g) * (T)(bi * g);
                        }
                });
        };

        // ---- forward solve RT = W^-1 TF (colour by colour, a barrier after each)
        auto forwardSolve = [&]() {
            for (int col = 0; col < C; col++)
            {
                rows(col, [&](int l, int, int jb, int jl, int, const T * vOg) {
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    eisGather1<T, NCH, VALS>(lad, lv, vOg, jb, jl, offR, chBytes, act, acc);
                    const T id = invDs[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            rt[c * S + l] = (tf[c * S + l] - acc[c]) * id;
                });
                cl.sync();
            }
        };

        // ---- backward solve TF = W^-T XT (the accumulated x~ -> x increment), a barrier after each
        // colour
        auto backwardSolveX = [&]() {
            for (int col = C - 1; col >= 0; col--)
            {
                rows(col, [&](int l, int, int, int jl, int je, const T * vOg) {
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    eisGather1<T, NCH, VALS>(lad, lv, vOg, jl, je, 0u, chBytes, act, acc);
                    const T id = invDs[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                            tf[c * S + l] = (xt[c * S + l] - acc[c]) * id;
                });
                cl.sync();
            }
        };

        // ---- one application of A~ to u = D r~ (w = A~ u), preceded by the CG update when upd.
        // Partial sums: gam += r~.u (updated r~), del += w.u, rr += ||W r~||^2.
        auto aPass = [&](bool upd, T (&gam)[NCH], T (&del)[NCH], T (&rr)[NCH]) {
            T al[NCH], be[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                al[c] = upd ? sc.alpha[c] : (T)0;
                be[c] = upd ? sc.beta[c] : (T)0;
                gam[c] = del[c] = rr[c] = (T)0;
            }
            // the CG update of one row (own values only)
            auto update = [&](int l) {
                const T d = diags[l];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        const int o = c * S + l;
                        T r = rt[o];
                        if (upd)
                        {
                            const T sN = eisNextS(wv[o], sv[o], be[c]);
                            const T pN = eisFma(be[c], pv[o], d * r);
                            r = eisNextR(r, sN, al[c]);
                            sv[o] = sN;
                            pv[o] = pN;
                            xt[o] = eisFma(al[c], pN, xt[o]);
                            rt[o] = r;
                        }
                        gam[c] += r * (d * r);
                    }
            };
            // phase A: update colours 0 .. C-2; colour C-1 publishes t = r~_new; backward sweep of
            // colour C-2 (colour 0 merged with its forward sweep when C == 2)
            for (int col = 0; col < C - 1; col++)
                rows(col, [&](int l, int, int, int, int, const T *) { update(l); });
            rows(C - 1, [&](int l, int, int, int, int, const T *) {
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (act[c])
                    {
                        const int o = c * S + l;
                        tf[o] = upd ? eisNextR(rt[o], eisNextS(wv[o], sv[o], be[c]), al[c]) : rt[o];
                    }
            });
            // colour 0 sweep: t_0 from the later colours, f_0 = r~ - t, w = t + f; ||r||^2 from d r~
            auto colour0 = [&](bool onFly) {
                rows(0, [&](int l, int, int, int jl, int je, const T * vOg) {
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    if (onFly)
                        eisGatherNext<T, NCH, VALS>(lad, lv, vOg, jl, je, offR, offW, offS, chBytes, al, be, act, acc);
                    else
                        eisGather1<T, NCH, VALS>(lad, lv, vOg, jl, je, 0u, chBytes, act, acc);
                    const T id = invDs[l], d = diags[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const int o = c * S + l;
                            const T r = rt[o];
                            const T t = r - acc[c] * id;
                            const T f = r - t;
                            const T w = t + f;
                            tf[o] = f;
                            wv[o] = w;
                            const T u = d * r;
                            del[c] += w * u;
                            rr[c] += u * u;
                        }
                });
            };
            // backward sweep of colour col (t = r~ - d^-1 sum over later colours a t)
            auto backward = [&](int col, bool onFly) {
                rows(col, [&](int l, int, int, int jl, int je, const T * vOg) {
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = (T)0;
                    if (onFly)
                        eisGatherNext<T, NCH, VALS>(lad, lv, vOg, jl, je, offR, offW, offS, chBytes, al, be, act, acc);
                    else
                        eisGather1<T, NCH, VALS>(lad, lv, vOg, jl, je, 0u, chBytes, act, acc);
                    const T id = invDs[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const int o = c * S + l;
                            tf[o] = rt[o] - acc[c] * id;
                        }
                });
            };
            // the deferred update of colour C-1 (first thing of the phase after phase A)
            auto deferred = [&]() { rows(C - 1, [&](int l, int, int, int, int, const T *) { update(l); }); };
            if (C == 2)
                colour0(true);
            else
                backward(C - 2, true);
            cl.sync();
            deferred();
            for (int col = C - 3; col >= 1; col--)
            {
                backward(col, false);
                cl.sync();
            }
            if (C >= 3)
            {
                colour0(false);
                cl.sync();
            }
            // forward sweeps of colours 1 .. C-1
            for (int col = 1; col < C; col++)
            {
                rows(col, [&](int l, int, int jb, int jl, int, const T * vOg) {
                    T accF[NCH], accR[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        accF[c] = accR[c] = (T)0;
                    eisGather2<T, NCH, VALS>(lad, lv, vOg, jb, jl, offR, chBytes, act, accF, accR);
                    const T id = invDs[l], d = diags[l];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const int o = c * S + l;
                            const T r = rt[o], t = tf[o];
                            const T f = r - t - accF[c] * id;
                            const T w = t + f;
                            tf[o] = f;
                            wv[o] = w;
                            const T u = d * r;
                            del[c] += w * u;
                            const T ri = u + accR[c];
                            rr[c] += ri * ri;
                        }
                });
                if (col < C - 1)
                    cl.sync(); // the last forward phase's barrier is the reduction's
            }
        };

        const int absMode = st->absMode;
        const double tol2 = st->tol2;

        // ---- r0 = b - A x0 into TF; ||b||^2
        T bbP[NCH], rrT[NCH];
#pragma unroll
        for (int c = 0; c < NCH; c++)
            bbP[c] = rrT[c] = (T)0;
        if (A.ru)
        {
            double bq[NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
                bq[c] = 0.0;
            for (int col = 0; col < C; col++)
                rows(col, [&](int, int i, int, int, int, const T *) {
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (c < numCh)
                        {
                            const double bi = ldg(A.b64 + (size_t)c * n + i);
                            bq[c] += bi * bi;
                        }
                });
            dsClusterSum<double, NCH>(cl, bq, dslot, dbuf, [&](const double (&tot)[NCH]) {
                for (int c = 0; c < NCH; c++)
                    if (tot[c] > 0.0 && isfinite(tot[c]))
                    {
                        int e = 0;
                        frexp(sqrt(tot[c]), &e);
                        sc.gsc[c] = ldexp(1.0, -e);
                        sc.igsc[c] = ldexp(1.0, e);
                    }
            });
            trueResidual(rrT, bbP, true);
        }
        else
        {
            for (int col = 0; col < C; col++)
                rows(col, [&](int l, int i, int jb, int, int je, const T * vOg) {
                    const T d = diags[l];
                    T acc[NCH];
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        acc[c] = d * rt[c * S + l];
                    eisGather1<T, NCH, VALS>(lad, lv, vOg, jb, je, offR, chBytes, act, acc);
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                        if (act[c])
                        {
                            const T bi = A.b[(size_t)c * n + i];
                            tf[c * S + l] = bi - acc[c];
                            bbP[c] += bi * bi;
                        }
                });
        }
        cl.sync(); // every read of x0 (RT) done before the forward solve overwrites it
        forwardSolve();

        // ---- w0 = A~ u0; gamma0, delta0, ||r0||^2
        T g0[NCH], d0[NCH], r0[NCH];
        aPass(false, g0, d0, r0);
        {
            T red[4 * NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                red[c] = bbP[c];
                red[NCH + c] = g0[c];
                red[2 * NCH + c] = d0[c];
                red[3 * NCH + c] = r0[c];
            }
            dsClusterSum<T, 4 * NCH>(cl, red, slot, buf, [&](const T (&tot)[4 * NCH]) {
                int any = 0;
                for (int c = 0; c < NCH; c++)
                {
                    const double bb = (double)tot[c], gm = (double)tot[NCH + c], dl = (double)tot[2 * NCH + c],
                                 rr = (double)tot[3 * NCH + c];
                    sc.bb[c] = bb;
                    sc.rr[c] = rr;
                    sc.gamma[c] = gm;
                    const bool fin = isfinite(rr) && isfinite(bb) && isfinite(gm) && isfinite(dl);
                    const bool conv = absMode ? (rr * sc.igsc[c] * sc.igsc[c] < tol2) : (rr <= tol2 * bb);
                    sc.status[c] = fin ? 0 : 2;
                    sc.iters[c] = 0;
                    sc.act[c] = (c < numCh) && fin && !conv;
                    const double a = gm / dl;
                    if (sc.act[c] && !(dl > 0))
                    {
                        sc.status[c] = isfinite(dl) ? 4 : 2;
                        sc.act[c] = 0;
                    }
                    sc.alphaD[c] = a;
                    sc.alpha[c] = (T)a;
                    sc.beta[c] = (T)0;
                    sc.rrRef[c] = rr;
                    any |= sc.act[c];
                }
                sc.any = any;
                sc.replace = 0;
                sc.replacements = 0;
            });
        }
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = sc.act[c] != 0;

        int k = 1;
        for (; k <= maxIters; k++)
        {
            if (!sc.any)
                break; // same value in every CTA
            T gm[NCH], dl[NCH], rr[NCH];
            aPass(true, gm, dl, rr);
            T red[3 * NCH];
#pragma unroll
            for (int c = 0; c < NCH; c++)
            {
                red[c] = gm[c];
                red[NCH + c] = dl[c];
                red[2 * NCH + c] = rr[c];
            }
            // replaced: this reduction follows a residual replacement (its rr is the FP64 residual's)
            auto decide = [&](const T (&tot)[3 * NCH], bool replaced) {
                int any = 0;
                sc.replace = 0;
                for (int c = 0; c < NCH; c++)
                {
                    if (sc.act[c])
                    {
                        const double g = (double)tot[c], d = (double)tot[NCH + c], r = (double)tot[2 * NCH + c];
                        sc.rr[c] = r;
                        const bool fin = isfinite(r) && isfinite(g) && isfinite(d);
                        const bool conv = absMode ? (r * sc.igsc[c] * sc.igsc[c] < tol2) : (r <= tol2 * sc.bb[c]);
                        const bool stop = !fin || (conv && (!A.ru || replaced));
                        if (replaced)
                            sc.rrRef[c] = r;
                        else if (A.ru && fin && (conv || r <= A.ruDelta2 * sc.rrRef[c]))
                            sc.replace = 1;
                        if (stop)
                        {
                            sc.act[c] = 0;
                            sc.iters[c] = k;
                            sc.status[c] = fin ? 0 : 2;
                        }
                        else
                        {
                            // Chronopoulos-Gear step length (a replacement recomputes it explicitly)
                            const double be = g / sc.gamma[c];
                            const double den = d - be * g / sc.alphaD[c];
                            sc.beta[c] = (T)be;
                            sc.alphaD[c] = g / den;
                            sc.alpha[c] = (T)sc.alphaD[c];
                            sc.gamma[c] = g;
                            if (!replaced && !(den > 0) && !sc.replace)
                            {
                                sc.act[c] = 0;
                                sc.iters[c] = k;
                                sc.status[c] = isfinite(den) ? 4 : 2;
                            }
                        }
                    }
                    any |= sc.act[c];
                }
                sc.any = any;
            };
            // gamma of the previous iteration, needed by a replacement's beta
            double gPrev[NCH];
            if (A.ru)
                for (int c = 0; c < NCH; c++)
                    gPrev[c] = sc.gamma[c];
            dsClusterSum<T, 3 * NCH>(cl, red, slot, buf, [&](const T (&tot)[3 * NCH]) { decide(tot, false); });
#pragma unroll
            for (int c = 0; c < NCH; c++)
                act[c] = sc.act[c] != 0;
            if (A.ru && sc.replace) // same value in every CTA
            {
                // x64 += igsc W^-T x~ ; x~ = 0
                backwardSolveX();
                for (int col = 0; col < C; col++)
                    rows(col, [&](int l, int i, int, int, int, const T *) {
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (c < numCh && act[c])
                            {
                                double * px = A.x64 + (size_t)c * n + i;
                                *px = __ldcg(px) + (double)tf[c * S + l] * sc.igsc[c];
                                xt[c * S + l] = (T)0;
                            }
                    });
                cl.sync(); // every CTA's x64 in global memory
                T rrTrue[NCH], unused[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    rrTrue[c] = unused[c] = (T)0;
                trueResidual(rrTrue, unused, false);
                cl.sync();
                forwardSolve();
                T g2[NCH], d2[NCH], r2[NCH];
                aPass(false, g2, d2, r2);
#pragma unroll
                for (int c = 0; c < NCH; c++)
                {
                    red[c] = g2[c];
                    red[NCH + c] = d2[c];
                    red[2 * NCH + c] = rrTrue[c];
                }
                dsClusterSum<T, 3 * NCH>(cl, red, slot, buf, [&](const T (&tot)[3 * NCH]) {
                    sc.replacements++;
                    for (int c = 0; c < NCH; c++)
                        if (sc.act[c])
                            sc.gamma[c] = gPrev[c];
                    decide(tot, true);
                });
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    act[c] = sc.act[c] != 0;
                // explicit step length of the kept direction: alpha = gamma / (p_new . A~ p_new)
                T pq[NCH];
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    pq[c] = (T)0;
                for (int col = 0; col < C; col++)
                    rows(col, [&](int l, int, int, int, int, const T *) {
                        const T d = diags[l];
#pragma unroll
                        for (int c = 0; c < NCH; c++)
                            if (act[c])
                            {
                                const int o = c * S + l;
                                const T pN = eisFma(sc.beta[c], pv[o], d * rt[o]);
                                const T sN = eisNextS(wv[o], sv[o], sc.beta[c]);
                                pq[c] += pN * sN;
                            }
                    });
                dsClusterSum<T, NCH>(cl, pq, slot, buf, [&](const T (&tot)[NCH]) {
                    for (int c = 0; c < NCH; c++)
                        if (sc.act[c])
                        {
                            const double d = (double)tot[c];
                            if (!(d > 0))
                            {
                                sc.act[c] = 0;
                                sc.iters[c] = k;
                                sc.status[c] = isfinite(d) ? 4 : 2;
                            }
                            else
                            {
                                sc.alphaD[c] = sc.gamma[c] / d;
                                sc.alpha[c] = (T)sc.alphaD[c];
                            }
                        }
                    int any = 0;
                    for (int c = 0; c < NCH; c++)
                        any |= sc.act[c];
                    sc.any = any;
                });
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    act[c] = sc.act[c] != 0;
            }
        }

        // ---- x = x0 + W^-T x~ (ru: the remaining increment into x64)
#pragma unroll
        for (int c = 0; c < NCH; c++)
            act[c] = c < numCh;
        backwardSolveX();
        for (int col = 0; col < C; col++)
            rows(col, [&](int l, int i, int, int, int, const T *) {
#pragma unroll
                for (int c = 0; c < NCH; c++)
                    if (c < numCh)
                    {
                        if (A.ru)
                        {
                            double * px = A.x64 + (size_t)c * n + i;
                            *px = __ldcg(px) + (double)tf[c * S + l] * sc.igsc[c];
                        }
                        else
                        {
                            T * px = A.x + (size_t)c * n + i;
                            *px = *px + tf[c * S + l];
                        }
                    }
            });
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
                st->bb[c] = sc.bb[c] * sc.igsc[c] * sc.igsc[c];
                st->lastRR[c] = sc.rr[c] * sc.igsc[c] * sc.igsc[c];
                st->active[c] = 0;
            }
            st->iter = k;
            st->anyActive = 0;
        }
        cl.sync(); // no CTA may leave while another can still read its shared memory
    }
} // namespace nsf
