// On-device assembly of the channel operators: M, K (P2 mass and stiffness), Kp (P1 stiffness),
// D (divergence, P x 2N), G (gradient, 2N x P) and the FastConvection integration matrix I
// (nnz(K) x 2N), FP64, on patterns built on the host.
//
// The reference assembles element by element with per-thread value bundles summed at the end
// (cpp/libs/Fem/src/chorinCsr.cpp:296-419 over the local matrices of
// cpp/libs/Element/src/triangleIntegrator.cpp:132-293; FastConvection: fastConvection.cpp:52-97).
// Here every output row is one thread that gathers the contributions of its incident elements in
// ascending element order, contracting the element-independent reference tensors (constant memory)
// with the element's adjugate and determinant -- the host assembly's formulation
// (csrc/host/context.cpp) with the same operation order, written with explicitly rounded
// operations (no contraction into FMAs), so the device values equal the host values bit for bit.
#pragma once

namespace nsf
{
    __constant__ AssemblyTables cAsm;

    // adjugate B = adj(m) and det of each element's affine map (float, as the reference stores it)
    struct AsmGeo
    {
        double b00, b01, b10, b11, det, sgn;
    };

    __global__ void __launch_bounds__(TPB) kAsmGeometry(int T, const float * __restrict__ affine, AsmGeo * __restrict__ geo)
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= T)
            return;
        const double m00 = affine[6 * (size_t)t], m01 = affine[6 * (size_t)t + 1], m10 = affine[6 * (size_t)t + 2],
                     m11 = affine[6 * (size_t)t + 3];
        AsmGeo g;
        g.b00 = m11;
        g.b01 = -m10;
        g.b10 = -m01;
        g.b11 = m00;
        g.det = __dadd_rn(__dmul_rn(m00, m11), -__dmul_rn(m10, m01));
        g.sgn = g.det < 0 ? -1.0 : 1.0;
        geo[t] = g;
    }

    __device__ __forceinline__ int asmFind(const int * __restrict__ rs, const int * __restrict__ ci, int r, int c)
    {
        int lo = rs[r], hi = rs[r + 1];
        while (lo < hi)
        {
            const int mid = (lo + hi) >> 1;
            if (ci[mid] < c)
                lo = mid + 1;
            else
                hi = mid;
        }
        return lo; // the pattern holds c
    }

    __device__ __forceinline__ int asmLocal(const int * ids, int n, int v)
    {
        for (int i = 0; i < n; i++)
            if (ids[i] == v)
                return i;
        return -1;
    }

    // the metric t00, t01, t11 of B^T B
    __device__ __forceinline__ void asmMetric(const AsmGeo & g, double & t00, double & t01, double & t11)
    {
        t00 = __dadd_rn(__dmul_rn(g.b00, g.b00), __dmul_rn(g.b10, g.b10));
        t01 = __dadd_rn(__dmul_rn(g.b00, g.b01), __dmul_rn(g.b10, g.b11));
        t11 = __dadd_rn(__dmul_rn(g.b01, g.b01), __dmul_rn(g.b11, g.b11));
    }

    // sgn (a x + b y)
    __device__ __forceinline__ double asmDir(double sgn, double a, double x, double b, double y)
    {
        return __dmul_rn(sgn, __dadd_rn(__dmul_rn(a, x), __dmul_rn(b, y)));
    }

    // rows r of M and K, rows r and r + N of G (one thread per velocity node)
    __global__ void __launch_bounds__(TPB) kAsmVelocity(int N, const int * __restrict__ vStart, const int * __restrict__ vList,
                                                         const int * __restrict__ vElem, const int * __restrict__ pElem,
                                                         const AsmGeo * __restrict__ geo, const int * __restrict__ mrs,
                                                         const int * __restrict__ mci, double * __restrict__ mv,
                                                         double * __restrict__ kv, const int * __restrict__ grs,
                                                         const int * __restrict__ gci, double * __restrict__ gv)
    {
        const int r = blockIdx.x * blockDim.x + threadIdx.x;
        if (r >= N)
            return;
        for (int k = vStart[r]; k < vStart[r + 1]; k++)
        {
            const int t = vList[k];
            const int * ids = vElem + 6 * (size_t)t;
            const AsmGeo g = geo[t];
            const int i = asmLocal(ids, 6, r);
            const double ad = fabs(g.det);
            double t00, t01, t11;
            asmMetric(g, t00, t01, t11);
            for (int j = 0; j < 6; j++)
            {
                const int e = asmFind(mrs, mci, r, ids[j]);
                mv[e] = __dadd_rn(mv[e], __dmul_rn(ad, cAsm.mass[i * 6 + j]));
                const double s = __dadd_rn(__dadd_rn(__dmul_rn(t00, cAsm.sxx[i * 6 + j]),
                                                     __dmul_rn(t01, __dadd_rn(cAsm.sxy[i * 6 + j], cAsm.sxy[j * 6 + i]))),
                                           __dmul_rn(t11, cAsm.syy[i * 6 + j]));
                kv[e] = __dadd_rn(kv[e], __ddiv_rn(s, ad));
            }
            const int * pid = pElem + 3 * (size_t)t;
            for (int q = 0; q < 3; q++)
            {
                const double gx = asmDir(g.sgn, g.b00, cAsm.grdX[i * 3 + q], g.b01, cAsm.grdY[i * 3 + q]);
                const double gy = asmDir(g.sgn, g.b10, cAsm.grdX[i * 3 + q], g.b11, cAsm.grdY[i * 3 + q]);
                const int ex = asmFind(grs, gci, r, pid[q]), ey = asmFind(grs, gci, r + N, pid[q]);
                gv[ex] = __dadd_rn(gv[ex], gx);
                gv[ey] = __dadd_rn(gv[ey], gy);
            }
        }
    }

    // rows r of Kp and D (one thread per pressure node)
    __global__ void __launch_bounds__(TPB) kAsmPressure(int P, int N, const int * __restrict__ pStart,
                                                         const int * __restrict__ pList, const int * __restrict__ pElem,
                                                         const int * __restrict__ vElem, const AsmGeo * __restrict__ geo,
                                                         const int * __restrict__ krs, const int * __restrict__ kci,
                                                         double * __restrict__ kv, const int * __restrict__ drs,
                                                         const int * __restrict__ dci, double * __restrict__ dv)
    {
        const int r = blockIdx.x * blockDim.x + threadIdx.x;
        if (r >= P)
            return;
        for (int k = pStart[r]; k < pStart[r + 1]; k++)
        {
            const int t = pList[k];
            const int * pid = pElem + 3 * (size_t)t;
            const int * vid = vElem + 6 * (size_t)t;
            const AsmGeo g = geo[t];
            const int i = asmLocal(pid, 3, r);
            const double ad = fabs(g.det);
            double t00, t01, t11;
            asmMetric(g, t00, t01, t11);
            for (int j = 0; j < 3; j++)
            {
                const double * ps = cAsm.p1stiff + (i * 3 + j) * 3;
                const double s =
                    __dadd_rn(__dadd_rn(__dmul_rn(t00, ps[0]), __dmul_rn(t01, ps[1])), __dmul_rn(t11, ps[2]));
                const int e = asmFind(krs, kci, r, pid[j]);
                kv[e] = __dadd_rn(kv[e], __ddiv_rn(s, ad));
            }
            for (int a = 0; a < 6; a++)
            {
                const double dx = asmDir(g.sgn, g.b00, cAsm.divX[i * 6 + a], g.b01, cAsm.divY[i * 6 + a]);
                const double dy = asmDir(g.sgn, g.b10, cAsm.divX[i * 6 + a], g.b11, cAsm.divY[i * 6 + a]);
                const int ex = asmFind(drs, dci, r, vid[a]), ey = asmFind(drs, dci, r, vid[a] + N);
                dv[ex] = __dadd_rn(dv[ex], dx);
                dv[ey] = __dadd_rn(dv[ey], dy);
            }
        }
    }

    // row e of I: the FastConvection coefficients of K entry e = (r, c) (one thread per entry)
    __global__ void __launch_bounds__(TPB) kAsmFastConv(int nnzK, int N, const int * __restrict__ entryRow,
                                                         const int * __restrict__ kci, const int * __restrict__ vStart,
                                                         const int * __restrict__ vList, const int * __restrict__ vElem,
                                                         const AsmGeo * __restrict__ geo, const int * __restrict__ irs,
                                                         const int * __restrict__ ici, double * __restrict__ iv)
    {
        const int e = blockIdx.x * blockDim.x + threadIdx.x;
        if (e >= nnzK)
            return;
        const int r = entryRow[e], cc = kci[e];
        for (int k = vStart[r]; k < vStart[r + 1]; k++)
        {
            const int t = vList[k];
            const int * ids = vElem + 6 * (size_t)t;
            const int jl = asmLocal(ids, 6, cc);
            if (jl < 0)
                continue;
            const int il = asmLocal(ids, 6, r);
            const AsmGeo g = geo[t];
            for (int q = 0; q < 6; q++)
            {
                const int a = (il * 6 + jl) * 6 + q;
                const double vx = asmDir(g.sgn, g.b00, cAsm.advX[a], g.b01, cAsm.advY[a]);
                const double vy = asmDir(g.sgn, g.b10, cAsm.advX[a], g.b11, cAsm.advY[a]);
                const int ex = asmFind(irs, ici, e, ids[q]), ey = asmFind(irs, ici, e, ids[q] + N);
                iv[ex] = __dadd_rn(iv[ex], vx);
                iv[ey] = __dadd_rn(iv[ey], vy);
            }
        }
    }

    // M, K, Kp, D, G, I values of a context whose patterns are set, assembled on the device; the
    // internal pressure slice Kpi is taken from Kp afterwards on the host.  Returns the device time
    // of the assembly kernels in ms.
    inline double assembleOnDevice(const Mesh & m, Context & c)
    {
        const AssemblyTables tab = assemblyTables();
        NSF_CUDA(cudaMemcpyToSymbol(cAsm, &tab, sizeof tab));
        const int N = c.N, P = c.P, T = m.numTri();
        std::vector<int> vStart, vList, pStart, pList;
        incidenceOf(N, m.vElem, 6, vStart, vList);
        incidenceOf(P, m.pElem, 3, pStart, pList);
        const int nnzK = c.K.nnz();
        std::vector<int> entryRow(nnzK);
        for (int r = 0; r < N; r++)
            for (int e = c.K.rowStart[r]; e < c.K.rowStart[r + 1]; e++)
                entryRow[e] = r;
        DevBuf<int> dvS, dvL, dpS, dpL, dvE, dpE, dER, mrs, mci, krs, kci, drs, dci, grs, gci, irs, ici;
        DevBuf<float> daf;
        DevBuf<AsmGeo> dgeo(T);
        dvS.upload(vStart);
        dvL.upload(vList);
        dpS.upload(pStart);
        dpL.upload(pList);
        dvE.upload(m.vElem);
        dpE.upload(m.pElem);
        dER.upload(entryRow);
        daf.upload(m.affine);
        mrs.upload(c.M.rowStart);
        mci.upload(c.M.col);
        krs.upload(c.Kp.rowStart);
        kci.upload(c.Kp.col);
        drs.upload(c.D.rowStart);
        dci.upload(c.D.col);
        grs.upload(c.G.rowStart);
        gci.upload(c.G.col);
        irs.upload(c.I.rowStart);
        ici.upload(c.I.col);
        DevBuf<double> mv(c.M.nnz()), kv(c.K.nnz()), kpv(c.Kp.nnz()), dv(c.D.nnz()), gv(c.G.nnz()), iv(c.I.nnz());
        cudaEvent_t e0, e1;
        NSF_CUDA(cudaEventCreate(&e0));
        NSF_CUDA(cudaEventCreate(&e1));
        cudaStream_t s = nullptr;
        NSF_CUDA(cudaEventRecord(e0, s));
        NSF_LAUNCH(kAsmGeometry, blocksFor(T), s, T, (const float *)daf.get(), dgeo.get());
        NSF_LAUNCH(kAsmVelocity, blocksFor(N), s, N, (const int *)dvS.get(), (const int *)dvL.get(),
                   (const int *)dvE.get(), (const int *)dpE.get(), (const AsmGeo *)dgeo.get(), (const int *)mrs.get(),
                   (const int *)mci.get(), mv.get(), kv.get(), (const int *)grs.get(), (const int *)gci.get(), gv.get());
        NSF_LAUNCH(kAsmPressure, blocksFor(P), s, P, N, (const int *)dpS.get(), (const int *)dpL.get(),
                   (const int *)dpE.get(), (const int *)dvE.get(), (const AsmGeo *)dgeo.get(), (const int *)krs.get(),
                   (const int *)kci.get(), kpv.get(), (const int *)drs.get(), (const int *)dci.get(), dv.get());
        NSF_LAUNCH(kAsmFastConv, blocksFor(nnzK), s, nnzK, N, (const int *)dER.get(), (const int *)mci.get(),
                   (const int *)dvS.get(), (const int *)dvL.get(), (const int *)dvE.get(), (const AsmGeo *)dgeo.get(),
                   (const int *)irs.get(), (const int *)ici.get(), iv.get());
        NSF_CUDA(cudaEventRecord(e1, s));
        NSF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        NSF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        c.M.val = mv.download();
        c.K.val = kv.download();
        c.Kp.val = kpv.download();
        c.D.val = dv.download();
        c.G.val = gv.download();
        c.I.val = iv.download();
        c.Kpi = sliceCsr(c.Kp, c.intP, c.intP);
        return ms;
    }
} // namespace nsf
