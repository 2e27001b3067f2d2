// C ABI of the GB300 Chorin path: host setup handles, device CSR operators, solvers and the
// device-resident Chorin stepper.  See include/nsfem_gb300.h for the contract of each call.
#include "../../include/nsfem_gb300.h"

#include "projection.cuh"
#include "solvers.cuh"

#include <algorithm>
#include <climits>
#include <cstring>
#include <memory>
#include <mutex>
#include <utility>
#include <vector>
#include <numeric>
#include <string>

namespace nsf
{
    thread_local std::string lastError;

    template <typename F>
    int guarded(F && f)
    {
        try
        {
            f();
            return ST_OK;
        }
        catch (const Error & e)
        {
            lastError = e.what();
            return e.status;
        }
        catch (const std::bad_alloc & e)
        {
            lastError = std::string("host allocation failed: ") + e.what();
            return ST_INVALID;
        }
        catch (const std::invalid_argument & e)
        {
            lastError = e.what();
            return ST_INVALID;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return ST_IO;
        }
    }

    inline void require(bool ok, const std::string & what)
    {
        if (!ok)
            throw Error(ST_INVALID, what);
    }

    inline cudaStream_t asStream(void * s) { return reinterpret_cast<cudaStream_t>(s); }

    std::vector<int> inverse(const std::vector<int> & perm)
    {
        std::vector<int> inv(perm.size());
        for (size_t i = 0; i < perm.size(); i++)
            inv[perm[i]] = (int)i;
        return inv;
    }

    // re-index rows (rowMap[newRow] = oldRow) and columns (colMap[oldCol] = newCol or -1 to drop)
    HostCsr<double> renumber(const HostCsr<double> & a, const std::vector<int> & rowMap, const std::vector<int> & colMap,
                             int newCols)
    {
        HostCsr<double> out;
        out.rows = (int)rowMap.size();
        out.cols = newCols;
        out.rowStart.assign(out.rows + 1, 0);
        std::vector<std::pair<int, double>> tmp;
        for (int r = 0; r < out.rows; r++)
        {
            tmp.clear();
            const int o = rowMap[r];
            for (int j = a.rowStart[o]; j < a.rowStart[o + 1]; j++)
            {
                const int c = colMap[a.col[j]];
                if (c >= 0)
                    tmp.emplace_back(c, a.val[j]);
            }
            std::sort(tmp.begin(), tmp.end(), [](const auto & x, const auto & y) { return x.first < y.first; });
            for (auto & [c, v] : tmp)
            {
                out.col.push_back(c);
                out.val.push_back(v);
            }
            out.rowStart[r + 1] = (int)out.col.size();
        }
        return out;
    }

    // Row blocks of the CSR-stream kernel: consecutive rows whose entries fit in STREAM_NNZ.
    // Returns an empty vector if some row is longer than STREAM_NNZ (row-group kernel then).
    std::vector<int> streamRowBlocks(const int * rowStart, int rows)
    {
        std::vector<int> rb{0};
        int r = 0;
        while (r < rows)
        {
            const int base = rowStart[r];
            int e = r;
            while (e < rows && rowStart[e + 1] - base <= STREAM_NNZ)
                e++;
            if (e == r)
                return {};
            rb.push_back(e);
            r = e;
        }
        return rb;
    }

    // SELL-C-sigma copy of a CSR matrix for kSpmvSell / kFastConvSell (layout in kernels.cuh).
    // Rows are sorted by length (descending, stable) inside windows of sigma = 256 rows, which
    // keeps the padding of these FEM operators at 1-7% and the scattered result writes inside a
    // window; a padded entry repeats the row's last column with a zero value, so it never
    // gathers a value that the row does not already use.
    template <typename T>
    struct DevSell
    {
        int rows = 0, nSlices = 0;
        long long stored = 0;
        DevBuf<int> ss, perm, ci, src; // src (only with keepSrc): CSR entry of each stored entry, -1 = pad
        DevBuf<T> v;

        void build(int n, const int * rs, const int * col, const double * val, bool keepSrc = false,
                   int sigma = 256)
        {
            rows = n;
            nSlices = (n + SELL_C - 1) / SELL_C;
            std::vector<int> order(n);
            std::iota(order.begin(), order.end(), 0);
            auto len = [&](int r) { return rs[r + 1] - rs[r]; };
            for (int w0 = 0; w0 < n; w0 += sigma)
                std::stable_sort(order.begin() + w0, order.begin() + std::min(n, w0 + sigma),
                                 [&](int a, int b) { return len(a) > len(b); });
            std::vector<long long> start(nSlices + 1, 0);
            for (int s = 0; s < nSlices; s++)
            {
                int w = 0;
                for (int l = 0; l < SELL_C && s * SELL_C + l < n; l++)
                    w = std::max(w, len(order[s * SELL_C + l]));
                start[s + 1] = start[s] + (long long)SELL_C * w;
            }
            stored = start[nSlices];
            if (stored >= INT_MAX)
                throw Error(ST_NOTSUP, "matrix too large for 32-bit SELL offsets");
            std::vector<int> hs(nSlices + 1), hc((size_t)stored), hsrc(keepSrc ? (size_t)stored : 0);
            std::vector<T> hv((size_t)stored);
            for (int s = 0; s <= nSlices; s++)
                hs[s] = (int)start[s];
            for (int s = 0; s < nSlices; s++)
            {
                const int w = (int)((start[s + 1] - start[s]) / SELL_C);
                for (int l = 0; l < SELL_C; l++)
                {
                    const int sr = s * SELL_C + l;
                    const int r = sr < n ? order[sr] : -1;
                    const int m = r >= 0 ? len(r) : 0;
                    const int last = m > 0 ? col[rs[r] + m - 1] : 0;
                    for (int k = 0; k < w; k++)
                    {
                        const size_t i = (size_t)start[s] + (size_t)k * SELL_C + l;
                        const bool real = k < m;
                        hc[i] = real ? col[rs[r] + k] : last;
                        hv[i] = real ? (T)val[rs[r] + k] : (T)0;
                        if (keepSrc)
                            hsrc[i] = real ? rs[r] + k : -1;
                    }
                }
            }
            ss.upload(hs);
            perm.upload(order);
            ci.upload(hc);
            v.upload(hv);
            if (keepSrc)
                src.upload(hsrc);
        }

        int blocks() const { return blocksFor((long long)nSlices * SELL_C); }
    };

    // Chebyshev iteration with the Jacobi preconditioner for the P2 mass matrix (velMethod 3).  The
    // spectrum of D^-1 M lies in [0.392375, 2.059816]: every element matrix is |T| times the same
    // reference matrix (affine P2 triangles, exact quadrature), and those are the extreme generalized
    // eigenvalues of the reference pair (M_ref, diag M_ref), so the bound holds on any mesh.  With
    // kappa = 5.25 the error contracts by rho = (sqrt(kappa) - 1) / (sqrt(kappa) + 1) = 0.392 per
    // iteration: the count for a relative tolerance is fixed in advance (no dot products, one fused
    // kernel per iteration, graph-capturable), and a final FP64 residual gives the statistics.
    constexpr double kMassSpecLo = 0.39237, kMassSpecHi = 2.05982;

    struct ChebSolver
    {
        const SweepSystem<double> * sys = nullptr;
        const DevSell<double> * sell = nullptr;
        int numCh = 2;
        double dratio = 1.0; // max / min of diag(M): the 2-norm factor of the D-scaled error bound
        DevBuf<double> r, d0, d1, scratch;
        DevBuf<SolverState> st;
        // double-float iterations (enableDoubleFloat): the SELL values, D^-1 and the vectors as
        // (hi, lo) float pairs, so the iterations run on the FP32 pipes at about 48-bit precision
        bool df = false;
        // one warp per slice and channel (NSF_CHEB_SPLIT=0: one warp per slice for both channels)
        bool splitChannels = true;
        DevBuf<float2> vDf, invDDf, xDf, rDf, dDf0, dDf1, bDf;
        DevBuf<int> kw; // warm solves: the device count and the per-channel warm flags

        static float2 split(double v)
        {
            const float hi = (float)v;
            return make_float2(hi, (float)(v - (double)hi));
        }

        void enableDoubleFloat()
        {
            df = true;
            splitChannels = numCh == 2 && envStr("NSF_CHEB_SPLIT", "1") != "0";
            const std::vector<double> hv = sell->v.download(), hd = sys->invD.download();
            std::vector<float2> sv(hv.size()), sd(hd.size());
            for (size_t i = 0; i < hv.size(); i++)
                sv[i] = split(hv[i]);
            for (size_t i = 0; i < hd.size(); i++)
                sd[i] = split(hd[i]);
            vDf.upload(sv);
            invDDf.upload(sd);
            const size_t n2 = 2 * (size_t)sys->n;
            xDf.alloc(n2);
            rDf.alloc(n2);
            dDf0.alloc(n2);
            dDf1.alloc(n2);
            bDf.alloc(n2);
        }

        void setup(const SweepSystem<double> * s, const DevSell<double> * sl, int channels)
        {
            sys = s;
            sell = sl;
            numCh = channels;
            const size_t n = (size_t)s->n;
            r.alloc(2 * n);
            d0.alloc(2 * n);
            d1.alloc(2 * n);
            scratch.alloc(std::max((size_t)2 * MAXCH * cappedBlocks(1ll << 40), (size_t)2 * MAXCH * finalBlocks(sl)));
            st.alloc(1);
            kw.alloc(1 + MAXCH);
            const std::vector<double> dg = s->diag.download();
            double lo = 1e300, hi = 0;
            for (double v : dg)
            {
                lo = std::min(lo, std::fabs(v));
                hi = std::max(hi, std::fabs(v));
            }
            dratio = lo > 0 ? hi / lo : 1.0;
        }

        // blocks of the residual kernel (kChebResidualSell): a warp per slice and channel, at most 16
        // blocks per SM
        static int finalBlocks(const DevSell<double> * sl) { return std::min(2 * sl->blocks(), 16 * smCount()); }

        // iterations for ||r|| <= tol ||b||: 2 rho^k sqrt(dratio) <= tol
        int itersFor(double tol) const
        {
            const double kappa = kMassSpecHi / kMassSpecLo;
            const double rho = (std::sqrt(kappa) - 1.0) / (std::sqrt(kappa) + 1.0);
            const double target = tol / (2.0 * std::sqrt(dratio));
            return std::max(1, (int)std::ceil(std::log(target) / std::log(rho)));
        }

        // warm == false: x must be 0 on entry, and the count is the a priori one for x0 = 0.
        // warm == true (mass-solve method 4): x holds the previous step's solution of this solve;
        // a device kernel decides per channel whether it is a better start than 0 and sets the
        // count from the initial residual (at most the cold count); the iterations past it exit
        // at once.
        void enqueue(cudaStream_t s, const double * b, double * x, int maxIters, double tol, bool warm = false)
        {
            const int n = sys->n, k = std::min(maxIters, itersFor(tol));
            NSF_LAUNCH(kSetConfig, 1, s, st.get(), maxIters, 0, tol * tol);
            const double theta = 0.5 * (kMassSpecHi + kMassSpecLo), delta = 0.5 * (kMassSpecHi - kMassSpecLo);
            const double sigma = theta / delta;
            double rho = 1.0 / sigma;
            const int * kdev = nullptr;
            if (warm)
            {
                const double kappa = kMassSpecHi / kMassSpecLo;
                const double lnRho = std::log((std::sqrt(kappa) - 1.0) / (std::sqrt(kappa) + 1.0));
                const ChebWarmEpi epi{st.get(), kw.get(), numCh, k, std::log(tol / (2.0 * std::sqrt(dratio))), lnRho};
                NSF_LAUNCH((kChebResidualSell<false, true, ChebWarmEpi>), finalBlocks(sell), s, n, sell->nSlices,
                           sell->ss.get(), sell->perm.get(), sell->ci.get(), sell->v.get(), (const float2 *)nullptr,
                           (const float2 *)nullptr, x, b, (const float2 *)nullptr, r.get(), st.get(), scratch.get(),
                           epi);
                kdev = kw.get();
            }
            if (df)
            {
                if (warm)
                    NSF_LAUNCH((kChebWarmInitDf<2>), blocksFor(n), s, n, b, (const double *)x, (const double *)r.get(),
                               (const float2 *)invDDf.get(), split(1.0 / theta), kdev, xDf.get(), rDf.get(), dDf0.get(),
                               bDf.get());
                else
                    NSF_LAUNCH((kChebStartDf<2>), blocksFor(n), s, n, b, (const float2 *)invDDf.get(),
                               split(1.0 / theta), rDf.get(), dDf0.get(), xDf.get(), bDf.get());
                float2 * dc = dDf0.get();
                float2 * dn = dDf1.get();
                for (int it = 0; it < k; it++)
                {
                    const double rhoN = 1.0 / (2.0 * sigma - rho);
                    if (splitChannels)
                        NSF_LAUNCH_PDL(kChebStepDfSplit, 2 * sell->blocks(), s, n, sell->nSlices, sell->ss.get(),
                                   sell->perm.get(), sell->ci.get(), (const float2 *)vDf.get(),
                                   (const float2 *)invDDf.get(), (const float2 *)dc, dn, xDf.get(), rDf.get(),
                                   split(rhoN * rho), split(2.0 * rhoN / delta), kdev, it);
                    else
                        NSF_LAUNCH((kChebStepDf<2>), sell->blocks(), s, n, sell->nSlices, sell->ss.get(),
                                   sell->perm.get(), sell->ci.get(), (const float2 *)vDf.get(),
                                   (const float2 *)invDDf.get(), (const float2 *)dc, dn, xDf.get(), rDf.get(),
                                   split(rhoN * rho), split(2.0 * rhoN / delta), kdev, it);
                    rho = rhoN;
                    std::swap(dc, dn);
                }
                NSF_LAUNCH((kChebResidualSell<true, false, ChebEpi>), finalBlocks(sell), s, n, sell->nSlices,
                           sell->ss.get(), sell->perm.get(), sell->ci.get(), (const double *)nullptr,
                           (const float2 *)vDf.get(), (const float2 *)xDf.get(), x, b, (const float2 *)bDf.get(),
                           (double *)nullptr, st.get(), scratch.get(), ChebEpi{st.get(), numCh, k, kdev});
                return;
            }
            else
            {
                if (warm)
                    NSF_LAUNCH((kChebWarmInit<2>), blocksFor(n), s, n, b, sys->invD.get(), 1.0 / theta, kdev, x, r.get(),
                               d0.get());
                else
                    NSF_LAUNCH((kChebStart<2>), blocksFor(n), s, n, b, sys->invD.get(), 1.0 / theta, r.get(),
                               d0.get());
                double * dc = d0.get();
                double * dn = d1.get();
                for (int it = 0; it < k; it++)
                {
                    const double rhoN = 1.0 / (2.0 * sigma - rho);
                    NSF_LAUNCH((kChebStep<2>), sell->blocks(), s, n, sell->nSlices, sell->ss.get(),
                               sell->perm.get(), sell->ci.get(), sell->v.get(), sys->invD.get(), (const double *)dc,
                               dn, x, r.get(), rhoN * rho, 2.0 * rhoN / delta, kdev, it);
                    rho = rhoN;
                    std::swap(dc, dn);
                }
            }
            NSF_LAUNCH((kChebResidualSell<false, false, ChebEpi>), finalBlocks(sell), s, n, sell->nSlices,
                       sell->ss.get(), sell->perm.get(), sell->ci.get(), sell->v.get(), (const float2 *)nullptr,
                       (const float2 *)nullptr, x, b, (const float2 *)nullptr, (double *)nullptr, st.get(),
                       scratch.get(), ChebEpi{st.get(), numCh, k, kdev});
        }
    };

    // y = alpha A x + beta y through the SELL copy (accumulation in TA)
    template <typename TA, typename TM, typename TX, typename TY>
    void sellSpmv(const DevSell<TM> & S, const TX * x, TY * y, double alpha, double beta, cudaStream_t s)
    {
        NSF_LAUNCH((kSpmvSell<TM, TX, TY, TA>), S.blocks(), s, S.rows, S.nSlices, S.ss.get(), S.perm.get(),
                   S.ci.get(), S.v.get(), x, y, alpha, beta);
    }

    template <typename T>
    struct DevCsr
    {
        int rows = 0, cols = 0, nnz = 0, L = 4, nBlocks = 0;
        DevBuf<int> rs, ci, rb;
        DevBuf<T> v;
        DevSell<T> sell;

        void upload(const HostCsr<double> & a, bool stream = false)
        {
            sell.build(a.rows, a.rowStart.data(), a.col.data(), a.val.data());
            rows = a.rows;
            cols = a.cols;
            nnz = a.nnz();
            rs.upload(a.rowStart);
            ci.upload(a.col);
            std::vector<T> tv(a.val.begin(), a.val.end());
            v.upload(tv);
            L = lanesFor(nnz, rows);
            if (stream)
            {
                std::vector<int> b = streamRowBlocks(a.rowStart.data(), rows);
                nBlocks = (int)b.size() - 1;
                if (nBlocks > 0)
                    rb.upload(b);
            }
        }
    };
} // namespace nsf

using namespace nsf;

struct nsf_mesh_s
{
    Mesh m;
};

struct nsf_context_s
{
    Context c;
};

struct nsf_csr_s
{
    int rows = 0, cols = 0, nnz = 0, dtype = NSF_F64, L = 4, nBlocks = 0;
    DevBuf<int> rs, ci, rb;
    DevBuf<double> v64;
    DevBuf<float> v32;
    DevSell<double> s64; // SELL copy used by nsf_spmv / nsf_fastconv_apply (values kept in step
    DevSell<float> s32;  // with nsf_csr_update_values)
};

extern "C" const char * nsf_last_error(void) { return lastError.c_str(); }

extern "C" const char * nsf_status_string(int s)
{
    switch (s)
    {
    case NSF_OK: return "ok";
    case NSF_ERR_INVALID_ARG: return "invalid argument";
    case NSF_ERR_NONFINITE: return "non-finite value";
    case NSF_ERR_MAXITER: return "iteration cap reached";
    case NSF_ERR_BREAKDOWN: return "CG breakdown (matrix not SPD)";
    case NSF_ERR_CUDA: return "CUDA error";
    case NSF_ERR_IO: return "I/O or parse error";
    case NSF_ERR_NOT_SUPPORTED: return "not supported";
    default: return "unknown status";
    }
}

extern "C" int nsf_version(void) { return 1; }

extern "C" long long nsf_kernel_launches(void) { return launchCounter().load(); }

// ============================================================================ host setup

extern "C" int nsf_mesh_load_gmsh(const char * path, nsf_mesh * out)
{
    return guarded([&] {
        require(path && out, "null argument");
        auto h = std::make_unique<nsf_mesh_s>();
        try
        {
            h->m = loadGmsh(path);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
        *out = h.release();
    });
}

extern "C" int nsf_mesh_counts(nsf_mesh h, int * counts)
{
    return guarded([&] {
        require(h && counts, "null argument");
        const Mesh & m = h->m;
        counts[0] = (int)m.cornerXY.size() / 2;
        counts[1] = m.numTri();
        counts[2] = m.numBorder();
        counts[3] = m.N;
        counts[4] = m.P;
        counts[5] = (int)m.groups.size();
    });
}

extern "C" int nsf_mesh_arrays(nsf_mesh h, int * vElem, int * pElem, float * vXY, int * vBorder)
{
    return guarded([&] {
        require(h, "null mesh");
        const Mesh & m = h->m;
        if (vElem)
            std::copy(m.vElem.begin(), m.vElem.end(), vElem);
        if (pElem)
            std::copy(m.pElem.begin(), m.pElem.end(), pElem);
        if (vXY)
            std::copy(m.vXY.begin(), m.vXY.end(), vXY);
        if (vBorder)
            std::copy(m.vBorder.begin(), m.vBorder.end(), vBorder);
    });
}

extern "C" const char * nsf_mesh_group(nsf_mesh h, int i)
{
    if (!h || i < 0 || i >= (int)h->m.groups.size())
        return nullptr;
    return h->m.groups[i].c_str();
}

extern "C" void nsf_mesh_destroy(nsf_mesh h) { delete h; }

extern "C" int nsf_context_build(nsf_mesh mesh, float peak, int nThreads, nsf_context * out)
{
    return guarded([&] {
        require(mesh && out, "null argument");
        auto h = std::make_unique<nsf_context_s>();
        h->c = buildChannelContext(mesh->m, peak, nThreads);
        *out = h.release();
    });
}

// ============================================================ on-device assembly
#include "assembly.cuh"

extern "C" int nsf_context_build_device(nsf_mesh mesh, float peak, int nThreads, nsf_context * out, double * assemblyMs)
{
    return guarded([&] {
        require(mesh && out, "null argument");
        auto h = std::make_unique<nsf_context_s>();
        h->c = buildChannelContextEx(mesh->m, peak, nThreads, false);
        const double ms = assembleOnDevice(mesh->m, h->c);
        if (assemblyMs)
            *assemblyMs = ms;
        *out = h.release();
    });
}

extern "C" int nsf_context_sizes(nsf_context h, int * s)
{
    return guarded([&] {
        require(h && s, "null argument");
        const Context & c = h->c;
        s[0] = c.N;
        s[1] = c.P;
        s[2] = (int)c.dirIds.size();
        s[3] = (int)c.dirPIds.size();
        s[4] = (int)c.intV.size();
        s[5] = (int)c.intP.size();
        s[6] = c.M.nnz();
        s[7] = c.K.nnz();
        s[8] = c.Kp.nnz();
        s[9] = c.Kpi.nnz();
        s[10] = c.D.nnz();
        s[11] = c.G.nnz();
        s[12] = c.I.nnz();
    });
}

static const HostCsr<double> & contextMatrix(const Context & c, int which)
{
    switch (which)
    {
    case 0: return c.M;
    case 1: return c.K;
    case 2: return c.Kp;
    case 3: return c.Kpi;
    case 4: return c.D;
    case 5: return c.G;
    case 6: return c.I;
    default: throw Error(ST_INVALID, "matrix index must be 0..6");
    }
}

extern "C" int nsf_context_matrix(nsf_context h, int which, int * rowStart, int * col, double * val)
{
    return guarded([&] {
        require(h, "null context");
        const HostCsr<double> & a = contextMatrix(h->c, which);
        if (rowStart)
            std::copy(a.rowStart.begin(), a.rowStart.end(), rowStart);
        if (col)
            std::copy(a.col.begin(), a.col.end(), col);
        if (val)
            std::copy(a.val.begin(), a.val.end(), val);
    });
}

extern "C" int nsf_context_lists(nsf_context h, int * dirIds, double * dirVx, int * dirPIds, int * intV, int * intP)
{
    return guarded([&] {
        require(h, "null context");
        const Context & c = h->c;
        if (dirIds)
            std::copy(c.dirIds.begin(), c.dirIds.end(), dirIds);
        if (dirVx)
            std::copy(c.dirVx.begin(), c.dirVx.end(), dirVx);
        if (dirPIds)
            std::copy(c.dirPIds.begin(), c.dirPIds.end(), dirPIds);
        if (intV)
            std::copy(c.intV.begin(), c.intV.end(), intV);
        if (intP)
            std::copy(c.intP.begin(), c.intP.end(), intP);
    });
}

extern "C" void nsf_context_destroy(nsf_context h) { delete h; }

extern "C" int nsf_coloring(int n, const int * rowStart, const int * col, int * perm, int * partStart, int * nColors)
{
    return guarded([&] {
        require(n >= 0 && rowStart && perm && partStart && nColors, "null argument");
        std::string why;
        require(validCsr(n, n, rowStart[n], rowStart, col, why), "invalid CSR: " + why);
        Coloring c = colorGraph(n, rowStart, col);
        std::copy(c.perm.begin(), c.perm.end(), perm);
        std::copy(c.partStart.begin(), c.partStart.end(), partStart);
        *nColors = c.colors();
    });
}

// ============================================================ binary CSR / vector files

extern "C" int nsf_io_csr_info(const char * path, int * info)
{
    return guarded([&] {
        require(path && info, "null argument");
        try
        {
            const BinCsr m = readBinCsr(path);
            info[0] = m.a.rows;
            info[1] = m.a.cols;
            info[2] = m.a.nnz();
            info[3] = m.dtype;
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_io_read_csr(const char * path, int * rowStart, int * col, double * values)
{
    return guarded([&] {
        require(path && rowStart && col && values, "null argument");
        try
        {
            const BinCsr m = readBinCsr(path);
            std::copy(m.a.rowStart.begin(), m.a.rowStart.end(), rowStart);
            std::copy(m.a.col.begin(), m.a.col.end(), col);
            std::copy(m.a.val.begin(), m.a.val.end(), values);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_io_write_csr(const char * path, int rows, int cols, int nnz, const int * rowStart, const int * col,
                                const double * values, int dtype)
{
    return guarded([&] {
        require(path && rowStart && col && values, "null argument");
        require(rows >= 1 && cols >= 1 && nnz >= 1, "rows, cols and nnz must be >= 1");
        std::string why;
        require(validCsr(rows, cols, nnz, rowStart, col, why), "invalid CSR: " + why);
        try
        {
            writeBinCsr(path, rows, cols, nnz, rowStart, col, values, dtype);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_io_vec_info(const char * path, int * info)
{
    return guarded([&] {
        require(path && info, "null argument");
        try
        {
            const BinVec v = readBinVec(path);
            info[0] = (int)v.v.size();
            info[1] = v.dtype;
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_io_read_vec(const char * path, double * values)
{
    return guarded([&] {
        require(path && values, "null argument");
        try
        {
            const BinVec v = readBinVec(path);
            std::copy(v.v.begin(), v.v.end(), values);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_io_write_vec(const char * path, int n, const double * values, int dtype)
{
    return guarded([&] {
        require(path && values, "null argument");
        require(n >= 1, "n must be >= 1");
        try
        {
            writeBinVec(path, n, values, dtype);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

// ============================================================================ device CSR

extern "C" int nsf_csr_create(int rows, int cols, int nnz, const int * rowStart, const int * col, const void * values,
                              int dtype, nsf_csr * out)
{
    return guarded([&] {
        require(out && values, "null argument");
        require(dtype == NSF_F32 || dtype == NSF_F64, "dtype must be NSF_F32 or NSF_F64");
        std::string why;
        require(validCsr(rows, cols, nnz, rowStart, col, why), "invalid CSR: " + why);
        auto h = std::make_unique<nsf_csr_s>();
        h->rows = rows;
        h->cols = cols;
        h->nnz = nnz;
        h->dtype = dtype;
        h->rs.upload(rowStart, rows + 1);
        h->ci.upload(col, nnz);
        if (dtype == NSF_F64)
        {
            const double * v = static_cast<const double *>(values);
            for (int i = 0; i < nnz; i++)
                require(std::isfinite(v[i]), "non-finite CSR value at " + std::to_string(i));
            h->v64.upload(v, nnz);
            h->s64.build(rows, rowStart, col, v, true);
        }
        else
        {
            const float * v = static_cast<const float *>(values);
            for (int i = 0; i < nnz; i++)
                require(std::isfinite(v[i]), "non-finite CSR value at " + std::to_string(i));
            h->v32.upload(v, nnz);
            const std::vector<double> vd(v, v + nnz);
            h->s32.build(rows, rowStart, col, vd.data(), true);
        }
        h->L = lanesFor(nnz, rows);
        std::vector<int> rb = streamRowBlocks(rowStart, rows);
        h->nBlocks = (int)rb.size() - 1;
        if (h->nBlocks > 0)
            h->rb.upload(rb);
        *out = h.release();
    });
}

extern "C" int nsf_csr_update_values(nsf_csr a, const void * values, int onDevice, void * stream)
{
    return guarded([&] {
        require(a && values, "null argument");
        const size_t bytes = (size_t)a->nnz * (a->dtype == NSF_F64 ? 8 : 4);
        void * dst = a->dtype == NSF_F64 ? (void *)a->v64.get() : (void *)a->v32.get();
        NSF_CUDA(cudaMemcpyAsync(dst, values, bytes, onDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 asStream(stream)));
        if (a->dtype == NSF_F64 && a->s64.stored > 0)
            NSF_LAUNCH((kSellGather<double>), cappedBlocks(a->s64.stored), asStream(stream), a->s64.stored,
                       a->s64.src.get(), a->v64.get(), a->s64.v.get());
        else if (a->dtype == NSF_F32 && a->s32.stored > 0)
            NSF_LAUNCH((kSellGather<float>), cappedBlocks(a->s32.stored), asStream(stream), a->s32.stored,
                       a->s32.src.get(), a->v32.get(), a->s32.v.get());
        if (!onDevice)
            NSF_CUDA(cudaStreamSynchronize(asStream(stream)));
    });
}

extern "C" int nsf_csr_device(nsf_csr a, int ** rowStart, int ** col, void ** values)
{
    return guarded([&] {
        require(a, "null csr");
        if (rowStart)
            *rowStart = a->rs.get();
        if (col)
            *col = a->ci.get();
        if (values)
            *values = a->dtype == NSF_F64 ? (void *)a->v64.get() : (void *)a->v32.get();
    });
}

extern "C" void nsf_csr_destroy(nsf_csr a) { delete a; }

extern "C" int nsf_spmv(nsf_csr a, const void * x, void * y, double alpha, double beta, void * stream)
{
    return guarded([&] {
        require(a && x && y, "null argument");
        // SELL-C-sigma: one thread per row, coalesced slice loads, one FMA per stored entry
        cudaStream_t s = asStream(stream);
        if (a->dtype == NSF_F64)
        {
            const DevSell<double> & S = a->s64;
            NSF_LAUNCH((kSpmvSell<double, double, double, double>), S.blocks(), s, S.rows, S.nSlices, S.ss.get(),
                       S.perm.get(), S.ci.get(), S.v.get(), (const double *)x, (double *)y, alpha, beta);
        }
        else
        {
            const DevSell<float> & S = a->s32;
            NSF_LAUNCH((kSpmvSell<float, float, float, float>), S.blocks(), s, S.rows, S.nSlices, S.ss.get(),
                       S.perm.get(), S.ci.get(), S.v.get(), (const float *)x, (float *)y, alpha, beta);
        }
    });
}

extern "C" int nsf_spmm(nsf_csr a, int nrhs, const void * X, int ldx, void * Y, int ldy, void * stream)
{
    return guarded([&] {
        require(a && X && Y && nrhs >= 1, "bad argument");
        require(ldx >= a->cols && ldy >= a->rows, "leading dimensions too small");
        const int grid = blocksFor((long long)a->rows * a->L);
        cudaStream_t s = asStream(stream);
        for (int c0 = 0; c0 < nrhs; c0 += 2)
        {
            const int k = std::min(2, nrhs - c0);
            if (a->dtype == NSF_F64)
            {
                const double * xx = (const double *)X + (size_t)c0 * ldx;
                double * yy = (double *)Y + (size_t)c0 * ldy;
                if (k == 2)
                    NSF_LANES(a->L, NSF_LAUNCH((kSpmm<double, double, double, double, LL, 2>), grid, s, a->rows,
                                               a->rs.get(), a->ci.get(), a->v64.get(), xx, ldx, yy, ldy));
                else
                    NSF_LANES(a->L, NSF_LAUNCH((kSpmm<double, double, double, double, LL, 1>), grid, s, a->rows,
                                               a->rs.get(), a->ci.get(), a->v64.get(), xx, ldx, yy, ldy));
            }
            else
            {
                const float * xx = (const float *)X + (size_t)c0 * ldx;
                float * yy = (float *)Y + (size_t)c0 * ldy;
                if (k == 2)
                    NSF_LANES(a->L, NSF_LAUNCH((kSpmm<float, float, float, float, LL, 2>), grid, s, a->rows,
                                               a->rs.get(), a->ci.get(), a->v32.get(), xx, ldx, yy, ldy));
                else
                    NSF_LANES(a->L, NSF_LAUNCH((kSpmm<float, float, float, float, LL, 1>), grid, s, a->rows,
                                               a->rs.get(), a->ci.get(), a->v32.get(), xx, ldx, yy, ldy));
            }
        }
    });
}

extern "C" int nsf_fastconv_apply_df(nsf_csr I, const float * K, double nu, const float * u, float * A,
                                     void * stream)
{
    return guarded([&] {
        require(I && K && u && A, "null argument");
        require(I->dtype == NSF_F32, "nsf_fastconv_apply_df takes an FP32 FastConvection matrix");
        const DevSell<float> & S = I->s32;
        NSF_LAUNCH(kFastConvSellDf, S.blocks(), asStream(stream), S.rows, S.nSlices, S.ss.get(), S.perm.get(),
                   S.ci.get(), S.v.get(), (const float2 *)u, (const float2 *)K, ChebSolver::split(nu), (float2 *)A);
    });
}

extern "C" int nsf_fastconv_apply(nsf_csr I, const void * K, double nu, const void * u, void * A, void * stream)
{
    return guarded([&] {
        require(I && K && u && A, "null argument");
        cudaStream_t s = asStream(stream);
        if (I->dtype == NSF_F64)
        {
            const DevSell<double> & S = I->s64;
            NSF_LAUNCH((kFastConvSell<double, double, double, double>), S.blocks(), s, S.rows, S.nSlices, S.ss.get(),
                       S.perm.get(), S.ci.get(), S.v.get(), (const double *)u, (const double *)K, nu, (double *)A);
        }
        else
        {
            const DevSell<float> & S = I->s32;
            NSF_LAUNCH((kFastConvSell<float, float, float, float>), S.blocks(), s, S.rows, S.nSlices, S.ss.get(),
                       S.perm.get(), S.ci.get(), S.v.get(), (const float *)u, (const float *)K, (float)nu,
                       (float *)A);
        }
    });
}

// ============================================================ vector helpers (the cu:: call sites)

namespace nsf
{
    template <typename T>
    __global__ void __launch_bounds__(TPB) kAxpy(long long n, T alpha, const T * __restrict__ x, T * __restrict__ y)
    {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            y[i] += alpha * x[i];
    }

    template <typename T>
    __global__ void __launch_bounds__(TPB) kScale(long long n, T alpha, T * __restrict__ x)
    {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            x[i] *= alpha;
    }

    template <typename A, typename B>
    __global__ void __launch_bounds__(TPB) kConvert(long long n, const A * __restrict__ a, B * __restrict__ b)
    {
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            b[i] = (B)a[i];
    }
} // namespace nsf

extern "C" int nsf_axpy(long long n, double alpha, const void * x, void * y, int dtype, void * stream)
{
    return guarded([&] {
        require(n >= 0 && (n == 0 || (x && y)), "bad argument");
        require(dtype == NSF_F32 || dtype == NSF_F64, "unknown dtype");
        if (n == 0)
            return;
        cudaStream_t s = asStream(stream);
        if (dtype == NSF_F32)
            NSF_LAUNCH(kAxpy<float>, blocksFor(n), s, n, (float)alpha, (const float *)x, (float *)y);
        else
            NSF_LAUNCH(kAxpy<double>, blocksFor(n), s, n, alpha, (const double *)x, (double *)y);
    });
}

extern "C" int nsf_scale(long long n, double alpha, void * x, int dtype, void * stream)
{
    return guarded([&] {
        require(n >= 0 && (n == 0 || x), "bad argument");
        require(dtype == NSF_F32 || dtype == NSF_F64, "unknown dtype");
        if (n == 0)
            return;
        cudaStream_t s = asStream(stream);
        if (dtype == NSF_F32)
            NSF_LAUNCH(kScale<float>, blocksFor(n), s, n, (float)alpha, (float *)x);
        else
            NSF_LAUNCH(kScale<double>, blocksFor(n), s, n, alpha, (double *)x);
    });
}

extern "C" int nsf_gather(int n, const int * idx, const void * src, void * dst, int dtype, void * stream)
{
    return guarded([&] {
        require(n >= 0 && (n == 0 || (idx && src && dst)), "bad argument");
        require(dtype == NSF_F32 || dtype == NSF_F64, "unknown dtype");
        if (n == 0)
            return;
        cudaStream_t s = asStream(stream);
        if (dtype == NSF_F32)
            NSF_LAUNCH(kGatherPerm<float>, blocksFor(n), s, n, 1, idx, (const float *)src, (float *)dst);
        else
            NSF_LAUNCH(kGatherPerm<double>, blocksFor(n), s, n, 1, idx, (const double *)src, (double *)dst);
    });
}

extern "C" int nsf_scatter(int n, const int * idx, const void * src, void * dst, int dtype, void * stream)
{
    return guarded([&] {
        require(n >= 0 && (n == 0 || (idx && src && dst)), "bad argument");
        require(dtype == NSF_F32 || dtype == NSF_F64, "unknown dtype");
        if (n == 0)
            return;
        cudaStream_t s = asStream(stream);
        if (dtype == NSF_F32)
            NSF_LAUNCH(kScatterPerm<float>, blocksFor(n), s, n, 1, idx, (const float *)src, (float *)dst);
        else
            NSF_LAUNCH(kScatterPerm<double>, blocksFor(n), s, n, 1, idx, (const double *)src, (double *)dst);
    });
}

// ============================================================================ solvers

struct nsf_solver_s
{
    std::string method;
    int numCh = 1, n = 0, precision = NSF_PREC_F64, maxIters = 200, checkInterval = 1;
    double target = 1e-6;
    Coloring col;
    DevBuf<int> perm;
    SweepSystem<double> s64;
    SweepSystem<float> s32;
    PcgSolver<double, 1> pcg1;
    PcgSolver<double, 2> pcg2;
    GsSolver<double, 1> gs1;
    GsSolver<double, 2> gs2;
    MixedPcg<1> mix1;
    MixedPcg<2> mix2;
    DevBuf<double> bp, xp;
    DevBuf<double> hostB, hostX; // device copies for nsf_solver_solve_host (allocated on first use)
    cudaStream_t body = nullptr;
    PinnedBuf<SolverState> stat{1};
    SolverState last{};
    int lastStatus = 0;

    ~nsf_solver_s()
    {
        if (body)
            cudaStreamDestroy(body);
    }

    const SolverState * devState() const
    {
        if (precision == NSF_PREC_MIXED)
            return numCh == 1 ? mix1.st.get() : mix2.st.get();
        if (method == "gs")
            return numCh == 1 ? gs1.st.get() : gs2.st.get();
        return numCh == 1 ? pcg1.st.get() : pcg2.st.get();
    }
};

extern "C" int nsf_solver_create(const char * method, int numCh, int n, const int * rowStart, const int * col,
                                 const double * values, int precision, int maxIters, double target, int checkInterval,
                                 nsf_solver * out)
{
    return guarded([&] {
        require(method && out && values, "null argument");
        const std::string m(method);
        require(m == "gs" || m == "pcg", "method must be \"gs\" or \"pcg\"");
        require(numCh == 1 || numCh == 2, "numCh must be 1 or 2");
        require(checkInterval >= 1, "checkInterval must be >= 1");
        require(maxIters >= 0, "maxIters must be >= 0");
        require(precision == NSF_PREC_F64 || precision == NSF_PREC_MIXED, "unknown precision");
        require(!(precision == NSF_PREC_MIXED && m == "gs"), "mixed precision is provided for \"pcg\"");
        std::string why;
        require(validCsr(n, n, rowStart ? rowStart[n] : 0, rowStart, col, why), "invalid CSR: " + why);
        auto s = std::make_unique<nsf_solver_s>();
        s->method = m;
        s->numCh = numCh;
        s->n = n;
        s->precision = precision;
        s->maxIters = maxIters;
        s->target = target;
        s->checkInterval = checkInterval;
        HostCsr<double> a;
        a.rows = a.cols = n;
        a.rowStart.assign(rowStart, rowStart + n + 1);
        a.col.assign(col, col + rowStart[n]);
        a.val.assign(values, values + rowStart[n]);
        for (double v : a.val)
            require(std::isfinite(v), "non-finite matrix value");
        s->col = colorGraph(n, a.rowStart.data(), a.col.data());
        HostCsr<double> ap = permuteSym(a, s->col.perm);
        s->perm.upload(s->col.perm);
        s->s64.build(ap, s->col.partStart);
        if (precision == NSF_PREC_MIXED)
        {
            s->s32.build(ap, s->col.partStart);
            if (numCh == 1)
                s->mix1.setup(&s->s64, &s->s32, 1);
            else
                s->mix2.setup(&s->s64, &s->s32, 2);
        }
        else if (m == "gs")
        {
            if (numCh == 1)
                s->gs1.setup(&s->s64, 1, checkInterval);
            else
                s->gs2.setup(&s->s64, 2, checkInterval);
        }
        else
        {
            if (numCh == 1)
                s->pcg1.setup(&s->s64, 1);
            else
                s->pcg2.setup(&s->s64, 2);
        }
        s->bp.alloc((size_t)numCh * n);
        s->xp.alloc((size_t)numCh * n);
        NSF_CUDA(cudaStreamCreateWithFlags(&s->body, cudaStreamNonBlocking));
        *out = s.release();
    });
}

extern "C" int nsf_solver_set(nsf_solver s, int maxIters, double target, int checkInterval)
{
    return guarded([&] {
        require(s && maxIters >= 0 && checkInterval >= 1, "bad argument");
        s->maxIters = maxIters;
        s->target = target;
        s->checkInterval = checkInterval;
        s->gs1.interval = s->gs2.interval = checkInterval;
        s->gs1.P.interval = s->gs2.P.interval = checkInterval;
    });
}

extern "C" int nsf_solver_solve(nsf_solver s, const double * b, double * x, void * stream)
{
    int st = guarded([&] {
        require(s && b && x, "null argument");
        cudaStream_t cs = asStream(stream);
        const int n = s->n, grid = blocksFor(n);
        NSF_LAUNCH(kGatherPerm<double>, grid, cs, n, s->numCh, s->perm.get(), b, s->bp.get());
        NSF_LAUNCH(kGatherPerm<double>, grid, cs, n, s->numCh, s->perm.get(), x, s->xp.get());
        const bool rel = true;
        if (s->precision == NSF_PREC_MIXED)
        {
            const int outer = 6, innerIt = std::max(1, s->maxIters);
            const double innerTol = std::max(1e-5, s->target);
            if (s->numCh == 1)
                s->mix1.enqueue(cs, s->body, s->bp.get(), s->xp.get(), outer, s->target, innerIt, innerTol,
                                s->checkInterval);
            else
                s->mix2.enqueue(cs, s->body, s->bp.get(), s->xp.get(), outer, s->target, innerIt, innerTol,
                                s->checkInterval);
        }
        else if (s->method == "gs")
        {
            // the reference's target is an absolute RMS residual (cu::GaussSeidel)
            if (s->numCh == 1)
                s->gs1.enqueue(cs, s->body, s->bp.get(), s->xp.get(), s->maxIters, s->target, true, 1);
            else
                s->gs2.enqueue(cs, s->body, s->bp.get(), s->xp.get(), s->maxIters, s->target, true, 1);
        }
        else
        {
            if (s->numCh == 1)
                s->pcg1.enqueue(cs, s->body, s->bp.get(), s->xp.get(), s->maxIters, s->target, !rel, s->checkInterval);
            else
                s->pcg2.enqueue(cs, s->body, s->bp.get(), s->xp.get(), s->maxIters, s->target, !rel, s->checkInterval);
        }
        NSF_LAUNCH(kScatterPerm<double>, grid, cs, n, s->numCh, s->perm.get(), s->xp.get(), x);
        NSF_CUDA(cudaMemcpyAsync(s->stat.get(), s->devState(), sizeof(SolverState), cudaMemcpyDeviceToHost, cs));
        NSF_CUDA(cudaStreamSynchronize(cs));
        s->last = *s->stat.get();
        int worst = 0;
        for (int c = 0; c < s->numCh; c++)
            worst = std::max(worst, s->last.status[c]);
        s->lastStatus = worst;
        if (worst != 0)
            throw Error(worst, std::string("solver finished with status ") + nsf_status_string(worst));
    });
    return st;
}

extern "C" int nsf_solver_solve_f32(nsf_solver s, const float * b, float * x, void * stream)
{
    int st = guarded([&] {
        require(s && b && x, "null argument");
        const long long len = (long long)s->numCh * s->n;
        if (!s->hostB.get())
        {
            s->hostB.alloc((size_t)len);
            s->hostX.alloc((size_t)len);
        }
        cudaStream_t cs = asStream(stream);
        NSF_LAUNCH((kConvert<float, double>), blocksFor(len), cs, len, b, s->hostB.get());
        NSF_LAUNCH((kConvert<float, double>), blocksFor(len), cs, len, (const float *)x, s->hostX.get());
    });
    if (st != NSF_OK)
        return st;
    const int solved = nsf_solver_solve(s, s->hostB.get(), s->hostX.get(), stream);
    const std::string err = solved != NSF_OK ? lastError : std::string();
    st = guarded([&] {
        const long long len = (long long)s->numCh * s->n;
        NSF_LAUNCH((kConvert<double, float>), blocksFor(len), asStream(stream), len, (const double *)s->hostX.get(),
                   x);
        NSF_CUDA(cudaStreamSynchronize(asStream(stream)));
    });
    if (st != NSF_OK)
        return st;
    if (solved != NSF_OK)
        lastError = err;
    return solved;
}

extern "C" int nsf_solver_solve_host(nsf_solver s, const double * b, double * x)
{
    int st = guarded([&] {
        require(s && b && x, "null argument");
        const size_t len = (size_t)s->numCh * s->n;
        if (!s->hostB.get())
        {
            s->hostB.alloc(len);
            s->hostX.alloc(len);
        }
        NSF_CUDA(cudaMemcpy(s->hostB.get(), b, sizeof(double) * len, cudaMemcpyHostToDevice));
        NSF_CUDA(cudaMemcpy(s->hostX.get(), x, sizeof(double) * len, cudaMemcpyHostToDevice));
    });
    if (st != NSF_OK)
        return st;
    const int solved = nsf_solver_solve(s, s->hostB.get(), s->hostX.get(), nullptr);
    const std::string err = solved != NSF_OK ? lastError : std::string();
    st = guarded([&] {
        NSF_CUDA(cudaMemcpy(x, s->hostX.get(), sizeof(double) * (size_t)s->numCh * s->n, cudaMemcpyDeviceToHost));
    });
    if (st != NSF_OK)
        return st;
    if (solved != NSF_OK)
        lastError = err;
    return solved;
}

extern "C" int nsf_solver_stats(nsf_solver s, int * iters, double * rms, double * rel)
{
    return guarded([&] {
        require(s, "null solver");
        const SolverState & L = s->last;
        int it = 0;
        for (int c = 0; c < s->numCh; c++)
        {
            const int ci = s->precision == NSF_PREC_MIXED ? L.innerTotal[c] : L.iters[c];
            it = std::max(it, ci);
            if (rms)
                rms[c] = std::sqrt(std::max(0.0, L.lastRR[c]) / (double)s->n);
            if (rel)
                rel[c] = L.bb[c] > 0 ? std::sqrt(std::max(0.0, L.lastRR[c]) / L.bb[c]) : std::sqrt(std::max(0.0, L.lastRR[c]));
        }
        if (iters)
            *iters = it;
    });
}

extern "C" void nsf_solver_destroy(nsf_solver s) { delete s; }

// ============================================================ pure-Neumann Poisson (pin + zero mean)

namespace nsf
{
    // FP64 sum of x[0..n) into out[0]: fixed-order block sums, the last block adds them up.
    __global__ void __launch_bounds__(TPB) kSumVec(int n, const double * __restrict__ x, double * scratch,
                                                    unsigned * ticket, double * out)
    {
        double v[1] = {0.0};
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            v[0] += x[i];
        Outs<1> o;
        o.p[0] = out;
        gridSum<double, 1>(v, scratch, o, ticket, nullptr);
    }

    // Reduced right-hand side: b projected to zero mean (mean = sum / n), the pinned row dropped.
    __global__ void __launch_bounds__(TPB) kNeumannRhs(int n, int pin, const double * __restrict__ b,
                                                        const double * __restrict__ sum, double * __restrict__ bRed)
    {
        const double mean = sum[0] / (double)n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            if (i != pin)
                bRed[i - (i > pin)] = b[i] - mean;
    }

    // Reduced initial guess: x shifted so that the pinned entry is zero, the pinned entry dropped.
    __global__ void __launch_bounds__(TPB) kNeumannGuess(int n, int pin, const double * __restrict__ x,
                                                          double * __restrict__ xRed)
    {
        const double x0 = x[pin];
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            if (i != pin)
                xRed[i - (i > pin)] = x[i] - x0;
    }

    // x = the reduced solution with the pinned entry 0
    __global__ void __launch_bounds__(TPB) kNeumannExpand(int n, int pin, const double * __restrict__ xRed,
                                                           double * __restrict__ x)
    {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i] = i == pin ? 0.0 : xRed[i - (i > pin)];
    }

    // x -= sum / n (the zero-mean representative of the solution)
    __global__ void __launch_bounds__(TPB) kShiftMean(int n, double * __restrict__ x, const double * __restrict__ sum)
    {
        const double mean = sum[0] / (double)n;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            x[i] -= mean;
    }
} // namespace nsf

struct nsf_neumann_s
{
    int n = 0, pin = 0;
    nsf_solver inner = nullptr;
    DevBuf<double> bRed, xRed, scratch, sums;
    DevBuf<unsigned> ticket;
    ~nsf_neumann_s()
    {
        if (inner)
            nsf_solver_destroy(inner);
    }
};

extern "C" int nsf_solver_set_coarse(nsf_solver s, const float * xy, int rowsPerAggregate)
{
    return guarded([&] {
        require(s && xy, "null argument");
        require(rowsPerAggregate >= 8, "rowsPerAggregate must be >= 8");
        require(s->method == "pcg" && s->precision == NSF_PREC_MIXED && s->numCh == 1,
                "the coarse correction is provided for single-channel mixed-precision \"pcg\" solvers");
        // the solver's colour-permuted numbering: row r is input row col.perm[r]
        std::vector<float> p(2 * (size_t)s->n);
        for (int r = 0; r < s->n; r++)
        {
            p[2 * (size_t)r] = xy[2 * (size_t)s->col.perm[r]];
            p[2 * (size_t)r + 1] = xy[2 * (size_t)s->col.perm[r] + 1];
        }
        if (!s->mix1.inner.enableCoarse(p, rowsPerAggregate))
            throw Error(ST_NOTSUP, "the coarse correction needs the cluster-resident path, at least 3 colours and "
                                   "room in the cluster's shared memory");
    });
}

extern "C" int nsf_neumann_create(int n, const int * rowStart, const int * col, const double * values, int pin,
                                  int precision, int maxIters, double target, nsf_neumann * out)
{
    return guarded([&] {
        require(out && rowStart && col && values, "null argument");
        require(n >= 2, "n must be >= 2");
        require(pin >= 0 && pin < n, "pin outside 0..n-1");
        std::string why;
        require(validCsr(n, n, rowStart[n], rowStart, col, why), "invalid CSR: " + why);
        // the system without row and column `pin`
        std::vector<int> rs(1, 0), ci;
        std::vector<double> va;
        ci.reserve(rowStart[n]);
        va.reserve(rowStart[n]);
        for (int i = 0; i < n; i++)
        {
            if (i == pin)
                continue;
            for (int j = rowStart[i]; j < rowStart[i + 1]; j++)
                if (col[j] != pin)
                {
                    ci.push_back(col[j] - (col[j] > pin));
                    va.push_back(values[j]);
                }
            rs.push_back((int)ci.size());
        }
        auto h = std::make_unique<nsf_neumann_s>();
        h->n = n;
        h->pin = pin;
        const int st = nsf_solver_create("pcg", 1, n - 1, rs.data(), ci.data(), va.data(), precision, maxIters, target,
                                         1, &h->inner);
        if (st != NSF_OK)
            throw Error(st, lastError);
        h->bRed.alloc((size_t)n - 1);
        h->xRed.alloc((size_t)n - 1);
        const int g = cappedBlocks(n);
        h->scratch.alloc((size_t)g);
        h->sums.alloc(2);
        h->ticket.alloc(1);
        NSF_CUDA(cudaMemset(h->ticket.get(), 0, sizeof(unsigned)));
        *out = h.release();
    });
}

extern "C" int nsf_neumann_solve(nsf_neumann h, const double * b, double * x, void * stream)
{
    return guarded([&] {
        require(h && b && x, "null argument");
        cudaStream_t s = asStream(stream);
        const int n = h->n, g = cappedBlocks(n), gb = blocksFor(n);
        NSF_LAUNCH(kSumVec, g, s, n, b, h->scratch.get(), h->ticket.get(), h->sums.get());
        NSF_LAUNCH(kNeumannRhs, gb, s, n, h->pin, b, (const double *)h->sums.get(), h->bRed.get());
        NSF_LAUNCH(kNeumannGuess, gb, s, n, h->pin, (const double *)x, h->xRed.get());
        const int st = nsf_solver_solve(h->inner, h->bRed.get(), h->xRed.get(), s);
        NSF_LAUNCH(kNeumannExpand, gb, s, n, h->pin, (const double *)h->xRed.get(), x);
        NSF_LAUNCH(kSumVec, g, s, n, (const double *)x, h->scratch.get(), h->ticket.get(), h->sums.get() + 1);
        NSF_LAUNCH(kShiftMean, gb, s, n, x, (const double *)h->sums.get() + 1);
        if (st != NSF_OK)
            throw Error(st, lastError);
    });
}

extern "C" int nsf_neumann_stats(nsf_neumann h, int * iters, double * rel)
{
    return guarded([&] {
        require(h, "null handle");
        const int st = nsf_solver_stats(h->inner, iters, nullptr, rel);
        if (st != NSF_OK)
            throw Error(st, lastError);
    });
}

extern "C" void nsf_neumann_destroy(nsf_neumann h) { delete h; }

// ============================================================================ Chorin stepper

// set while a batch creates its template stepper (the batched pressure solves run their own
// cluster kernel, with the template's single-level preconditioner layout)
thread_local bool tlTemplateStepper = false;

struct nsf_chorin_s
{
    nsf_chorin_config cfg{};
    bool mixed = false;      // FP32 operators and FP32-inner solves
    bool f32ops = false;     // NSF_PREC_MIXED_F32: the step's products in plain FP32 (mixed is set too)
    bool mixedSolve = false; // FP64 operators, FP32-inner solves (NSF_PREC_F64_MIXEDSOLVE)
    int N = 0, P = 0, nIntP = 0;
    std::vector<int> permV, permP, intP;
    std::vector<int> dirRows; // stepper row of each Dirichlet node (context dirIds order)
    // operators in the color-permuted numbering
    SweepSystem<double> M64, Kpi64;
    SweepSystem<float> M32, Kpi32;
    DevCsr<double> I64, D64, G64;
    DevCsr<float> I32, D32, G32;
    DevBuf<double> K64, A64;
    // state and work vectors
    DevBuf<double> u, pInt, rhs, acc, rhsP;
    // pressure initial guess extrapolated from the last two solutions (cfg.pressureGuess == 1)
    bool extrapolate = false;
    DevBuf<double> pPrev;
    DevBuf<int> pHist;
    // pressure initial guess projected onto earlier solutions (cfg.pressureGuess == 2)
    bool project = false;
    PressureProjection proj;
    // state copies: device staging (original numbering) and the renumbering maps
    DevBuf<double> stateStage;
    DevBuf<int> permVDev, pIdxDev;
    DevBuf<unsigned char> isDir;
    DevBuf<double> dirVal;
    // solvers: separate objects for the tentative and the final mass solve keep both stats
    PcgSolver<double, 2> velT, velF;
    ChebSolver chebT, chebF; // velMethod 3 (FP64 Chebyshev-Jacobi on the SELL copy of M)
    DevBuf<float2> uDf, KDf, ADf; // mixed: u, K and A as double-floats
    DevBuf<float> u32, K32, A32;  // f32ops: u, K and A in FP32
    DevBuf<double> accT, accF;    // velMethod 4: the last tentative and final mass-solve solutions
    DevSell<double> Msell;
    GsSolver<double, 2> gsT, gsF;
    PcgSolver<double, 1> pres;
    MixedPcg<2> mvelT, mvelF;
    MixedPcg<1> mpres;
    cudaStream_t stream = nullptr, body = nullptr;
    // the pressure-basis update runs on `side`, forked after the pressure solve and joined at the
    // end of the step (a parallel branch of the captured graph)
    cudaStream_t side = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernelsPerCapture = 0;
    PinnedBuf<SolverState> stat{5};
    std::unique_ptr<PinnedBuf<double>> stage;
    size_t stageSize = 0;

    double * staging(size_t need)
    {
        if (stageSize < need)
        {
            stage = std::make_unique<PinnedBuf<double>>(need);
            stageSize = need;
        }
        return stage->get();
    }
    double stats[8] = {0};

    // whether a solve of this stepper runs on the whole-GPU cooperative grid
    // internal pressure node coordinates in the solver numbering (empty: no coarse correction)
    std::vector<float> presXY;

    // the two-level pressure preconditioner on an FP32 pressure solver of this stepper: aggregates
    // are mesh cells of about NSF_PRES_COARSE_ROWS (240) internal pressure nodes, split by the CTA
    // that owns the rows
    void enablePresCoarse(PcgSolver<float, 1> & inner) const
    {
        if (presXY.empty())
            return;
        const int per = std::max(8, std::atoi(envStr("NSF_PRES_COARSE_ROWS", "240").c_str()));
        inner.enableCoarse(presXY, per);
    }

    bool usesGrid() const
    {
        using P = PcgSolver<double, 1>;
        return velT.path == P::GRID || velF.path == P::GRID || pres.path == P::GRID ||
               mvelT.inner.path == P::GRID || mvelF.inner.path == P::GRID || mpres.inner.path == P::GRID ||
               (mpres.pre32Form && mpres.pre32Solve.path == P::GRID);
    }

    ~nsf_chorin_s()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        if (body)
            cudaStreamDestroy(body);
        if (side)
            cudaStreamDestroy(side);
        if (evFork)
            cudaEventDestroy(evFork);
        if (evJoin)
            cudaEventDestroy(evJoin);
        if (stream)
            cudaStreamDestroy(stream);
    }

    // returns the buffer that holds the solution
    double * enqueueMassSolve(cudaStream_t s, bool tentative)
    {
        double * b = rhs.get();
        if (cfg.velMethod == 4)
        {
            // warm start from this solve's solution of the previous step (kept in accT / accF)
            double * x = tentative ? accT.get() : accF.get();
            (tentative ? chebT : chebF).enqueue(s, b, x, cfg.velMaxIters, cfg.velTol, true);
            return x;
        }
        double * x = acc.get();
        NSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * 2 * N, s));
        if (cfg.velMethod == 3)
            (tentative ? chebT : chebF).enqueue(s, b, x, cfg.velMaxIters, cfg.velTol);
        else if (mixed || mixedSolve)
            (tentative ? mvelT : mvelF)
                .enqueue(s, body, b, x, cfg.maxOuter, cfg.velTol, cfg.velMaxIters, cfg.innerTol, cfg.checkInterval);
        else if (cfg.velMethod == 0)
            (tentative ? gsT : gsF).enqueue(s, body, b, x, cfg.velMaxIters, cfg.velTol, false, cfg.checkInterval);
        else
            (tentative ? velT : velF).enqueue(s, body, b, x, cfg.velMaxIters, cfg.velTol, false, cfg.checkInterval);
        return x;
    }

    void enqueueStep(cudaStream_t s)
    {
        // 1. A = nu K + I u (SELL copy of the FastConvection matrix) ;  rhs = A [ux uy]
        if (f32ops)
        {
            // the literal FP32 split: FP32 values, vectors and sums, the product rhs widened to FP64
            const DevSell<float> & IS = I32.sell;
            NSF_LAUNCH((kConvert<double, float>), blocksFor(2ll * N), s, 2ll * N, (const double *)u.get(), u32.get());
            NSF_LAUNCH((kFastConvSell<float, float, float, float>), IS.blocks(), s, IS.rows, IS.nSlices, IS.ss.get(),
                       IS.perm.get(), IS.ci.get(), IS.v.get(), (const float *)u32.get(), (const float *)K32.get(),
                       cfg.nu, A32.get());
            NSF_LANES(M32.L, NSF_LAUNCH((kSpmm<float, float, double, float, LL, 2>), blocksFor((long long)N * M32.L), s,
                                        N, M32.rsF.get(), M32.ciF.get(), (const float *)A32.get(),
                                        (const float *)u32.get(), N, rhs.get(), N));
        }
        else if (mixed)
        {
            const DevSell<float> & IS = I32.sell;
            // double-float (FP32 pipes, 48 bits) for the products that feed the divergence
            NSF_LAUNCH(kSplitDf, blocksFor(2ll * N), s, 2ll * N, (const double *)u.get(), uDf.get());
            NSF_LAUNCH(kFastConvSellDf, IS.blocks(), s, IS.rows, IS.nSlices, IS.ss.get(), IS.perm.get(), IS.ci.get(),
                       IS.v.get(), (const float2 *)uDf.get(), (const float2 *)KDf.get(), ChebSolver::split(cfg.nu),
                       ADf.get());
            // double-float sums: FP32 sums would put step-to-step rounding noise into u, which the
            // divergence amplifies in the pressure right-hand side
            NSF_LANES(M32.L, NSF_LAUNCH((kSpmmDf<LL, 2>), blocksFor((long long)N * M32.L), s, N, M32.rsF.get(),
                                        M32.ciF.get(), (const float2 *)ADf.get(), (const float2 *)uDf.get(), N,
                                        rhs.get(), N));
        }
        else
        {
            const DevSell<double> & IS = I64.sell;
            NSF_LAUNCH((kFastConvSell<double, double, double, double>), IS.blocks(), s, IS.rows, IS.nSlices,
                       IS.ss.get(), IS.perm.get(), IS.ci.get(), IS.v.get(), u.get(), K64.get(), cfg.nu, A64.get());
            NSF_LANES(M64.L, NSF_LAUNCH((kSpmm<double, double, double, double, LL, 2>), blocksFor((long long)N * M64.L), s, N,
                                        M64.rsF.get(), M64.ciF.get(), A64.get(), u.get(), N, rhs.get(), N));
        }
        // 2. M acc = rhs ; u = u - tau acc ; Dirichlet
        const double * accT1 = enqueueMassSolve(s, true);
        NSF_LAUNCH(kUpdateVelocity<double>, blocksFor(N), s, N, u.get(), accT1, cfg.tau, isDir.get(), dirVal.get());
        // 3. rhsP = -(1/tau) D u ; Kpi pInt = rhsP (warm start)
        const double invTau = -1.0 / cfg.tau;
        if (extrapolate)
        {
            NSF_LAUNCH(kExtrapolate, blocksFor(nIntP), s, nIntP, pInt.get(), pPrev.get(), (const int *)pHist.get());
            NSF_LAUNCH(kHistBump, 1, s, pHist.get());
        }
        if (mixed)
        {
            // FP32 values, FP64 sums: D u cancels heavily, and FP32 sums would leave rounding noise of
            // ~1e-5 of the result in rhsP that changes from step to step, which the pressure solve
            // then has to remove to its tolerance (no initial guess can predict it)
            if (f32ops)
                sellSpmv<float>(D32.sell, u.get(), rhsP.get(), invTau, 0.0, s);
            else
                sellSpmv<double>(D32.sell, u.get(), rhsP.get(), invTau, 0.0, s);
            if (project)
                proj.guess(s, rhsP.get(), pInt.get());
            mpres.enqueue(s, body, rhsP.get(), pInt.get(), cfg.maxOuter, cfg.presTol, cfg.presMaxIters, cfg.innerTol,
                          cfg.checkInterval);
            if (f32ops)
                sellSpmv<float>(G32.sell, pInt.get(), rhs.get(), 1.0, 0.0, s);
            else
                sellSpmv<double>(G32.sell, pInt.get(), rhs.get(), 1.0, 0.0, s);
        }
        else
        {
            sellSpmv<double>(D64.sell, u.get(), rhsP.get(), invTau, 0.0, s);
            if (project)
                proj.guess(s, rhsP.get(), pInt.get());
            if (mixedSolve)
                mpres.enqueue(s, body, rhsP.get(), pInt.get(), cfg.maxOuter, cfg.presTol, cfg.presMaxIters,
                              cfg.innerTol, cfg.checkInterval);
            else
                pres.enqueue(s, body, rhsP.get(), pInt.get(), cfg.presMaxIters, cfg.presTol, false,
                             cfg.checkInterval);
            sellSpmv<double>(G64.sell, pInt.get(), rhs.get(), 1.0, 0.0, s);
        }
        if (project)
        {
            // the basis update reads only the solved pressure and writes only its own buffers: it runs
            // beside the final mass solve, on the side stream
            NSF_CUDA(cudaEventRecord(evFork, s));
            NSF_CUDA(cudaStreamWaitEvent(side, evFork, 0));
            proj.update(side, pInt.get());
            NSF_CUDA(cudaEventRecord(evJoin, side));
        }
        // 4. M acc = G p ; u = u - tau acc ; Dirichlet
        const double * accF1 = enqueueMassSolve(s, false);
        NSF_LAUNCH(kUpdateVelocity<double>, blocksFor(N), s, N, u.get(), accF1, cfg.tau, isDir.get(), dirVal.get());
        if (project)
            NSF_CUDA(cudaStreamWaitEvent(s, evJoin, 0));
    }

    void collectStats(cudaStream_t s)
    {
        const SolverState * src[3];
        const bool inner = mixed || mixedSolve;
        bool srcInner[3] = {inner, inner, inner};
        if (inner)
        {
            src[0] = mvelT.st.get();
            src[1] = mpres.st.get();
            src[2] = mvelF.st.get();
        }
        else
        {
            src[0] = cfg.velMethod == 0 ? gsT.st.get() : velT.st.get();
            src[1] = pres.st.get();
            src[2] = cfg.velMethod == 0 ? gsF.st.get() : velF.st.get();
        }
        if (cfg.velMethod >= 3)
        {
            src[0] = chebT.st.get();
            src[2] = chebF.st.get();
            srcInner[0] = srcInner[2] = false;
        }
        for (int i = 0; i < 3; i++)
            NSF_CUDA(cudaMemcpyAsync(stat.get() + i, src[i], sizeof(SolverState), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        int worst = 0;
        for (int i = 0; i < 3; i++)
        {
            const SolverState & L = stat.get()[i];
            const int nch = i == 1 ? 1 : 2;
            int it = 0;
            double rel = 0;
            for (int c = 0; c < nch; c++)
            {
                it = std::max(it, srcInner[i] ? L.innerTotal[c] : L.iters[c]);
                const double r = L.bb[c] > 0 ? std::sqrt(std::max(0.0, L.lastRR[c]) / L.bb[c]) : 0.0;
                rel = std::max(rel, r);
                worst = std::max(worst, L.status[c]);
            }
            const int idxIt[3] = {0, 1, 2};
            const int idxRel[3] = {4, 3, 5};
            stats[idxIt[i]] = it;
            stats[idxRel[i]] = rel;
            if (i == 1)
                stats[6] = inner ? L.iters[0] : 0;
        }
        stats[7] = worst;
    }
};

// typical iteration counts of the step's solves (weights for the path autotuner)
constexpr int kMassIters = 30, kPresIters = 400;

static void buildChorin(nsf_chorin_s & S, const Context & c)
{
    const int N = c.N, P = c.P;
    S.N = N;
    S.P = P;
    S.intP = c.intP;
    S.nIntP = (int)c.intP.size();
    require(S.nIntP > 0, "no internal pressure nodes");
    // velocity numbering: coloring of M (shared by K, A); pressure: coloring of Kpi
    Coloring cv = colorGraph(N, c.M.rowStart.data(), c.M.col.data());
    Coloring cp = colorGraph(S.nIntP, c.Kpi.rowStart.data(), c.Kpi.col.data());
    S.permV = cv.perm;
    S.permP = cp.perm;
    if (!c.pXY.empty() && !tlTemplateStepper && envStr("NSF_PRES_COARSE", "1") != "0")
    {
        S.presXY.resize(2 * (size_t)S.nIntP);
        for (int r = 0; r < S.nIntP; r++)
        {
            const int node = c.intP[cp.perm[r]];
            S.presXY[2 * (size_t)r] = c.pXY[2 * (size_t)node];
            S.presXY[2 * (size_t)r + 1] = c.pXY[2 * (size_t)node + 1];
        }
    }
    const std::vector<int> invV = inverse(cv.perm), invP = inverse(cp.perm);
    HostCsr<double> Mp = permuteSym(c.M, cv.perm);
    HostCsr<double> Kp = permuteSym(c.K, cv.perm);
    HostCsr<double> Kpip = permuteSym(c.Kpi, cp.perm);
    // velocity dof map (2N): old (node, ch) -> new
    std::vector<int> dofMap(2 * (size_t)N);
    for (int v = 0; v < N; v++)
    {
        dofMap[v] = invV[v];
        dofMap[v + N] = invV[v] + N;
    }
    std::vector<int> dofRows(2 * (size_t)N);
    for (int r = 0; r < N; r++)
    {
        dofRows[r] = cv.perm[r];
        dofRows[r + N] = cv.perm[r] + N;
    }
    // I: rows follow the entries of the permuted K pattern
    std::vector<int> iRows(Kp.nnz());
    for (int r = 0; r < N; r++)
        for (int e = Kp.rowStart[r]; e < Kp.rowStart[r + 1]; e++)
        {
            const int orow = cv.perm[r], ocol = cv.perm[Kp.col[e]];
            const auto b = c.K.col.begin() + c.K.rowStart[orow], en = c.K.col.begin() + c.K.rowStart[orow + 1];
            auto it = std::lower_bound(b, en, ocol);
            require(it != en && *it == ocol, "K pattern mismatch while permuting I");
            iRows[e] = (int)(it - c.K.col.begin());
        }
    HostCsr<double> Ip = renumber(c.I, iRows, dofMap, 2 * N);
    // D: rows = internal pressure nodes in colored order; cols = velocity dofs
    std::vector<int> dRows(S.nIntP);
    for (int r = 0; r < S.nIntP; r++)
        dRows[r] = c.intP[cp.perm[r]];
    HostCsr<double> Dp = renumber(c.D, dRows, dofMap, 2 * N);
    // G: rows = velocity dofs in colored order; cols = internal pressure (Dirichlet p = 0 dropped)
    std::vector<int> pCol(P, -1);
    for (int i = 0; i < S.nIntP; i++)
        pCol[c.intP[i]] = invP[i];
    HostCsr<double> Gp = renumber(c.G, dofRows, pCol, S.nIntP);

    // velMethod 2: the mass systems as one color, which turns the SGS preconditioner of the PCG
    // kernels into Jacobi (the forward phase of a single color gathers nothing): one parallel phase
    // per iteration instead of 2C - 1 color phases
    const bool cheb = S.cfg.velMethod >= 3;
    const std::vector<int> mParts = S.cfg.velMethod >= 2 ? std::vector<int>{0, N} : cv.partStart;
    S.M64.build(Mp, mParts);
    if (cheb)
    {
        // velMethod 3: the Chebyshev iteration reads M through its SELL copy, with no other solver
        S.Msell.build(N, Mp.rowStart.data(), Mp.col.data(), Mp.val.data());
        S.chebT.setup(&S.M64, &S.Msell, 2);
        S.chebF.setup(&S.M64, &S.Msell, 2);
        if (S.cfg.velMethod == 4)
        {
            S.accT = DevBuf<double>(2 * (size_t)N);
            S.accF = DevBuf<double>(2 * (size_t)N);
            NSF_CUDA(cudaMemset(S.accT.get(), 0, sizeof(double) * 2 * N));
            NSF_CUDA(cudaMemset(S.accF.get(), 0, sizeof(double) * 2 * N));
        }
        if (S.mixed)
        {
            // the mixed stepper iterates in double-float on the FP32 pipes (48 bits: the rounding
            // of the mass solves stays far below their tolerance)
            S.chebT.enableDoubleFloat();
            S.chebF.enableDoubleFloat();
        }
    }
    S.Kpi64.build(Kpip, cp.partStart);
    std::vector<double> knu(Kp.val.begin(), Kp.val.end());
    if (S.mixed)
    {
        // M32 also carries the pattern of the rhs = A u product of the mixed step (M and K share it)
        S.M32.build(Mp, mParts);
        S.Kpi32.build(Kpip, cp.partStart);
        S.I32.upload(Ip, true);
        S.D32.upload(Dp);
        S.G32.upload(Gp);
        std::vector<float2> kdf(knu.size());
        for (size_t i = 0; i < knu.size(); i++)
            kdf[i] = ChebSolver::split(knu[i]);
        S.KDf.upload(kdf);
        S.ADf.alloc(knu.size());
        S.uDf.alloc(2 * (size_t)N);
        if (S.f32ops)
        {
            std::vector<float> k32(knu.begin(), knu.end());
            S.K32.upload(k32);
            S.A32.alloc(knu.size());
            S.u32.alloc(2 * (size_t)N);
        }
        if (!cheb)
        {
            S.mvelT.setup(&S.M64, &S.M32, 2, kMassIters);
            S.mvelF.setup(&S.M64, &S.M32, 2, kMassIters);
        }
        S.mpres.setup(&S.Kpi64, &S.Kpi32, 1, kPresIters);
        S.enablePresCoarse(S.mpres.inner);
    }
    else
    {
        S.I64.upload(Ip, true);
        S.D64.upload(Dp);
        S.G64.upload(Gp);
        S.K64.upload(knu);
        S.A64.alloc(knu.size());
        if (S.mixedSolve)
        {
            // FP64 operators, FP32-inner solves on FP32 copies of the two systems
            S.Kpi32.build(Kpip, cp.partStart);
            if (!cheb)
            {
                S.M32.build(Mp, mParts);
                S.mvelT.setup(&S.M64, &S.M32, 2, kMassIters);
                S.mvelF.setup(&S.M64, &S.M32, 2, kMassIters);
            }
            S.mpres.setup(&S.Kpi64, &S.Kpi32, 1, kPresIters);
            S.enablePresCoarse(S.mpres.inner);
        }
        else
        {
            if (S.cfg.velMethod == 0)
            {
                S.gsT.setup(&S.M64, 2, 1);
                S.gsF.setup(&S.M64, 2, 1);
            }
            else if (!cheb)
            {
                S.velT.setup(&S.M64, 2, true, kMassIters);
                S.velF.setup(&S.M64, 2, true, kMassIters);
            }
            S.pres.setup(&S.Kpi64, 1, true, kPresIters);
        }
    }
    // Dirichlet rows in the colored numbering
    std::vector<unsigned char> isDir(N, 0);
    std::vector<double> dval(N, 0.0);
    for (size_t i = 0; i < c.dirIds.size(); i++)
    {
        isDir[invV[c.dirIds[i]]] = 1;
        dval[invV[c.dirIds[i]]] = c.dirVx[i];
        S.dirRows.push_back(invV[c.dirIds[i]]);
    }
    S.isDir.upload(isDir);
    S.dirVal.upload(dval);
    // initial state: u = 0 with the Dirichlet values, p = 0
    std::vector<double> u0(2 * (size_t)N, 0.0);
    for (int r = 0; r < N; r++)
        if (isDir[r])
            u0[r] = dval[r];
    S.u.upload(u0);
    S.pInt.alloc(S.nIntP);
    S.project = S.cfg.pressureGuess == 2;
    if (S.project)
        S.proj.setup(&S.Kpi64, S.cfg.pressureBasis > 0 ? S.cfg.pressureBasis : 250);
    S.extrapolate = S.cfg.pressureGuess == 1;
    if (S.extrapolate)
    {
        S.pPrev.alloc(S.nIntP);
        S.pHist.alloc(1);
    }
    S.rhs.alloc(2 * (size_t)N);
    S.acc.alloc(2 * (size_t)N);
    S.rhsP.alloc(S.nIntP);
}

extern "C" int nsf_chorin_create(nsf_context ctx, const nsf_chorin_config * cfg, nsf_chorin * out)
{
    return guarded([&] {
        require(ctx && cfg && out, "null argument");
        require(cfg->tau > 0 && cfg->nu >= 0, "tau must be > 0 and nu >= 0");
        require(cfg->precision == NSF_PREC_F64 || cfg->precision == NSF_PREC_MIXED ||
                    cfg->precision == NSF_PREC_F64_MIXEDSOLVE || cfg->precision == NSF_PREC_MIXED_F32,
                "unknown precision");
        require(!(cfg->precision == NSF_PREC_MIXED_F32 && cfg->velMethod != 1 && cfg->velMethod != 2),
                "NSF_PREC_MIXED_F32 runs the mass solves as FP32 PCG: velMethod 1 or 2");
        require(!(cfg->precision == NSF_PREC_F64_MIXEDSOLVE && cfg->velMethod == 0),
                "mixed solves use velMethod 1, 2 (pcg) or 3 (chebyshev)");
        require(cfg->velMethod >= 0 && cfg->velMethod <= 4,
                "velMethod must be 0 (gs), 1 (pcg, SGS preconditioner), 2 (pcg, Jacobi preconditioner), 3 "
                "(chebyshev, Jacobi preconditioner) or 4 (the same warm-started from the last step)");
        require(!(cfg->precision == NSF_PREC_MIXED && cfg->velMethod == 0),
                "mixed precision uses velMethod 1, 2 (pcg) or 3 (chebyshev)");
        require(cfg->velMaxIters >= 1 && cfg->presMaxIters >= 1, "iteration caps must be >= 1");
        require(cfg->pressureGuess >= 0 && cfg->pressureGuess <= 2, "pressureGuess must be 0, 1 or 2");
        require(cfg->pressureBasis == 0 || (cfg->pressureBasis >= 3 && cfg->pressureBasis <= PROJ_MAXL),
                "pressureBasis must be 0 (250) or 3..256");
        auto S = std::make_unique<nsf_chorin_s>();
        S->cfg = *cfg;
        if (S->cfg.checkInterval < 1)
            S->cfg.checkInterval = 1;
        if (S->cfg.maxOuter < 1)
            S->cfg.maxOuter = 4;
        if (!(S->cfg.innerTol > 0))
            S->cfg.innerTol = 1e-4;
        S->mixed = cfg->precision == NSF_PREC_MIXED || cfg->precision == NSF_PREC_MIXED_F32;
        S->f32ops = cfg->precision == NSF_PREC_MIXED_F32;
        S->mixedSolve = cfg->precision == NSF_PREC_F64_MIXEDSOLVE;
        buildChorin(*S, ctx->c);
        NSF_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
        NSF_CUDA(cudaStreamCreateWithFlags(&S->body, cudaStreamNonBlocking));
        NSF_CUDA(cudaStreamCreateWithFlags(&S->side, cudaStreamNonBlocking));
        NSF_CUDA(cudaEventCreateWithFlags(&S->evFork, cudaEventDisableTiming));
        NSF_CUDA(cudaEventCreateWithFlags(&S->evJoin, cudaEventDisableTiming));
        NSF_CUDA(cudaDeviceSynchronize());
        *out = S.release();
    });
}

// Enqueue nSteps time steps on stream s (graph replays when the stepper uses a graph; the
// graph is captured on the first call).
static void enqueueSteps(nsf_chorin S, int nSteps, cudaStream_t s);

extern "C" int nsf_chorin_step(nsf_chorin S, int nSteps, void * stream)
{
    return guarded([&] {
        require(S && nSteps >= 0, "bad argument");
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        enqueueSteps(S, nSteps, s);
        if (nSteps > 0)
            S->collectStats(s);
        if (S->stats[7] == ST_NONFINITE)
            throw Error(ST_NONFINITE, "non-finite solver residual in the time step");
    });
}

extern "C" int nsf_chorin_launch(nsf_chorin S, int nSteps, void * stream)
{
    return guarded([&] {
        require(S && nSteps >= 0, "bad argument");
        require(S->cfg.useGraph, "nsf_chorin_launch needs a graph-captured stepper (useGraph = 1)");
        enqueueSteps(S, nSteps, stream ? asStream(stream) : S->stream);
    });
}

static void enqueueSteps(nsf_chorin S, int nSteps, cudaStream_t s)
{
    {
        if (S->cfg.useGraph)
        {
            if (!S->exec)
            {
                const long long before = launchCounter().load();
                NSF_CUDA(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
                try
                {
                    S->enqueueStep(S->stream);
                }
                catch (...)
                {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(S->stream, &g);
                    if (g)
                        cudaGraphDestroy(g);
                    throw;
                }
                NSF_CUDA(cudaStreamEndCapture(S->stream, &S->graph));
                NSF_CUDA(cudaGraphInstantiate(&S->exec, S->graph, 0));
                S->kernelsPerCapture = launchCounter().load() - before;
                launchCounter().fetch_sub(S->kernelsPerCapture); // counted when replayed
            }
            for (int i = 0; i < nSteps; i++)
            {
                NSF_CUDA(cudaGraphLaunch(S->exec, s));
                // kernel nodes of one replay (a device-terminated loop body, used only by the
                // multi-kernel solver path, is counted once)
                launchCounter().fetch_add(S->kernelsPerCapture, std::memory_order_relaxed);
            }
        }
        else
        {
            for (int i = 0; i < nSteps; i++)
                S->enqueueStep(s);
        }
    }
}

// Device-side renumbering for the state copies: the host arrays (original numbering) are copied
// as they are into a device buffer and permuted there by a kernel, instead of permuting element by
// element on the host (scattered host accesses over MBs).
static void stateMaps(nsf_chorin S)
{
    if (S->permVDev.size() == (size_t)S->N && S->pIdxDev.size() == (size_t)S->nIntP)
        return;
    S->permVDev.upload(S->permV);
    std::vector<int> idx(S->nIntP);
    for (int r = 0; r < S->nIntP; r++)
        idx[r] = S->intP[S->permP[r]];
    S->pIdxDev.upload(idx);
    S->stateStage.alloc(2 * (size_t)S->N + S->P);
}

extern "C" int nsf_chorin_get_state(nsf_chorin S, double * uOut, double * pOut, void * stream)
{
    return guarded([&] {
        require(S, "null stepper");
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        stateMaps(S);
        const int N = S->N;
        double * su = S->stateStage.get(), * sp = su + 2 * (size_t)N;
        if (uOut)
        {
            NSF_LAUNCH((kScatterPerm<double>), blocksFor(N), s, N, 2, S->permVDev.get(), (const double *)S->u.get(),
                       su);
            NSF_CUDA(cudaMemcpyAsync(uOut, su, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, s));
        }
        if (pOut)
        {
            NSF_CUDA(cudaMemsetAsync(sp, 0, sizeof(double) * S->P, s)); // Dirichlet pressure: 0
            NSF_LAUNCH((kScatterPerm<double>), blocksFor(S->nIntP), s, S->nIntP, 1, S->pIdxDev.get(),
                       (const double *)S->pInt.get(), sp);
            NSF_CUDA(cudaMemcpyAsync(pOut, sp, sizeof(double) * S->P, cudaMemcpyDeviceToHost, s));
        }
        NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_chorin_dump(nsf_chorin S, const char * uPath, const char * pPath, int dtype, void * stream)
{
    return guarded([&] {
        require(S, "null stepper");
        require(dtype == NSF_F32 || dtype == NSF_F64, "dtype must be NSF_F32 or NSF_F64");
        std::vector<double> u(uPath ? 2 * (size_t)S->N : 0), p(pPath ? (size_t)S->P : 0);
        const int st = nsf_chorin_get_state(S, uPath ? u.data() : nullptr, pPath ? p.data() : nullptr, stream);
        if (st != NSF_OK)
            throw Error(st, lastError);
        try
        {
            if (uPath)
                writeBinVec(uPath, 2 * S->N, u.data(), dtype);
            if (pPath)
                writeBinVec(pPath, S->P, p.data(), dtype);
        }
        catch (const std::runtime_error & e)
        {
            throw Error(ST_IO, e.what());
        }
    });
}

extern "C" int nsf_chorin_set_state(nsf_chorin S, const double * uIn, const double * pIn, void * stream)
{
    return nsf_chorin_set_state_ex(S, uIn, pIn, 0, stream);
}

extern "C" int nsf_chorin_set_state_ex(nsf_chorin S, const double * uIn, const double * pIn, int flags,
                                       void * stream)
{
    return guarded([&] {
        require((flags & ~(NSF_STATE_KEEP_HISTORY | NSF_STATE_ASYNC)) == 0, "unknown set_state flags");
        require(S, "null stepper");
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        stateMaps(S);
        const int N = S->N;
        double * su = S->stateStage.get(), * sp = su + 2 * (size_t)N;
        if (uIn)
        {
            NSF_CUDA(cudaMemcpyAsync(su, uIn, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, s));
            NSF_LAUNCH((kGatherPerm<double>), blocksFor(N), s, N, 2, S->permVDev.get(), (const double *)su,
                       S->u.get());
        }
        if (pIn)
        {
            NSF_CUDA(cudaMemcpyAsync(sp, pIn, sizeof(double) * S->P, cudaMemcpyHostToDevice, s));
            NSF_LAUNCH((kGatherPerm<double>), blocksFor(S->nIntP), s, S->nIntP, 1, S->pIdxDev.get(),
                       (const double *)sp, S->pInt.get());
        }
        const bool keep = (flags & NSF_STATE_KEEP_HISTORY) != 0;
        if (S->extrapolate && !keep) // a new history starts from the state just set
            NSF_CUDA(cudaMemsetAsync(S->pHist.get(), 0, sizeof(int), s));
        if (S->project && !keep)
            S->proj.reset(s);
        if (S->cfg.velMethod == 4 && !keep) // the mass solves start cold again
        {
            NSF_CUDA(cudaMemsetAsync(S->accT.get(), 0, sizeof(double) * 2 * N, s));
            NSF_CUDA(cudaMemsetAsync(S->accF.get(), 0, sizeof(double) * 2 * N, s));
        }
        if (!(flags & NSF_STATE_ASYNC))
            NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_chorin_mass_solve(nsf_chorin S, const double * b, double * x, double tol, int * iters,
                                     void * stream)
{
    return guarded([&] {
        require(S && b && x, "null argument");
        require(S->cfg.velMethod == 3, "the mass solve is provided for velMethod 3 (Chebyshev) steppers");
        require(tol > 0 && tol < 1, "tol must be in (0, 1)");
        cudaStream_t s = stream ? asStream(stream) : S->stream;
        const int N = S->N;
        NSF_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * 2 * (size_t)N, s));
        S->chebT.enqueue(s, b, x, S->cfg.velMaxIters, tol);
        if (iters)
            *iters = std::min(S->cfg.velMaxIters, S->chebT.itersFor(tol));
        NSF_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int nsf_chorin_stats(nsf_chorin S, double * stats)
{
    return guarded([&] {
        require(S && stats, "null argument");
        std::copy(S->stats, S->stats + 8, stats);
    });
}

extern "C" void nsf_chorin_destroy(nsf_chorin S) { delete S; }

// ============================================================ force functional (drag / lift)

namespace
{
    // One quadrature point on one border edge: P2 velocity dofs and P1 pressure dofs of the
    // adjacent triangle (stepper numbering; pressure -1 = Dirichlet node, p = 0), the physical
    // gradients of the six P2 basis functions and the P1 shape values at the point, the weight
    // (half the edge length) and the unit normal into the fluid.
    struct ForcePoint
    {
        int v[6], p[3];
        double gx[6], gy[6], psi[3], w, nx, ny;
    };

    // F = sum_points w (-p n + nu (grad u) n); one block, fixed summation order.  visc (may be
    // null) receives the viscous integrals sum_points w (grad u) n without the factor nu.
    __global__ void __launch_bounds__(256) kForces(const ForcePoint * __restrict__ pts, int npts,
                                                   const double * __restrict__ u, int N,
                                                   const double * __restrict__ pInt, double nu, double * out,
                                                   double * visc)
    {
        double fx = 0, fy = 0, vx = 0, vy = 0;
        for (int i = threadIdx.x; i < npts; i += blockDim.x)
        {
            const ForcePoint & q = pts[i];
            double uxx = 0, uxy = 0, uyx = 0, uyy = 0, pq = 0;
#pragma unroll
            for (int k = 0; k < 6; k++)
            {
                const double ux = u[q.v[k]], uy = u[N + q.v[k]];
                uxx += ux * q.gx[k];
                uxy += ux * q.gy[k];
                uyx += uy * q.gx[k];
                uyy += uy * q.gy[k];
            }
#pragma unroll
            for (int k = 0; k < 3; k++)
                if (q.p[k] >= 0)
                    pq += pInt[q.p[k]] * q.psi[k];
            fx += q.w * (-pq * q.nx + nu * (uxx * q.nx + uxy * q.ny));
            fy += q.w * (-pq * q.ny + nu * (uyx * q.nx + uyy * q.ny));
            vx += q.w * (uxx * q.nx + uxy * q.ny);
            vy += q.w * (uyx * q.nx + uyy * q.ny);
        }
        __shared__ double part[4][8];
        for (int o = 16; o > 0; o >>= 1)
        {
            fx += __shfl_xor_sync(FULL, fx, o);
            fy += __shfl_xor_sync(FULL, fy, o);
            vx += __shfl_xor_sync(FULL, vx, o);
            vy += __shfl_xor_sync(FULL, vy, o);
        }
        const int warp = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0)
        {
            part[0][warp] = fx;
            part[1][warp] = fy;
            part[2][warp] = vx;
            part[3][warp] = vy;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double s[4] = {0, 0, 0, 0};
            for (int w = 0; w < (int)(blockDim.x >> 5); w++)
                for (int k = 0; k < 4; k++)
                    s[k] += part[k][w];
            out[0] = s[0];
            out[1] = s[1];
            if (visc)
            {
                visc[0] = s[2];
                visc[1] = s[3];
            }
        }
    }
} // namespace

struct nsf_forces_s
{
    nsf_chorin s = nullptr;
    int npts = 0;
    DevBuf<ForcePoint> pts;
    DevBuf<double> out;
    PinnedBuf<double> host{2};
};

extern "C" int nsf_forces_create(nsf_mesh mesh, nsf_chorin S, const char * group, nsf_forces * out)
{
    return guarded([&] {
        require(mesh && S && group && out, "null argument");
        const Mesh & m = mesh->m;
        require(m.N == S->N && m.P == S->P, "mesh and stepper sizes differ");
        const int gid = m.groupId(group);
        require(gid >= 0, "no such border group");
        // stepper numbering of velocity nodes and of pressure nodes (-1: Dirichlet, p = 0)
        const std::vector<int> invV = inverse(S->permV), invP = inverse(S->permP);
        std::vector<int> pCol(S->P, -1);
        for (int i = 0; i < S->nIntP; i++)
            pCol[S->intP[i]] = invP[i];
        const double gq = 0.5 / std::sqrt(3.0);
        const double tq[2] = {0.5 - gq, 0.5 + gq};
        std::vector<ForcePoint> pts;
        for (int b = 0; b < m.numBorder(); b++)
        {
            const int * vb = m.vBorder.data() + 6 * b;
            if (vb[2] != gid)
                continue;
            const int t = vb[0];
            const int * ve = m.vElem.data() + 6 * t;
            const int * pe = m.pElem.data() + 3 * t;
            auto X = [&](int node) { return (double)m.vXY[2 * node]; };
            auto Y = [&](int node) { return (double)m.vXY[2 * node + 1]; };
            const double x0 = X(ve[0]), y0 = Y(ve[0]);
            // reference triangle map J = [[x1-x0, x2-x0], [y1-y0, y2-y0]] (corners c0, c1, c2)
            const double j00 = X(ve[2]) - x0, j01 = X(ve[4]) - x0, j10 = Y(ve[2]) - y0, j11 = Y(ve[4]) - y0;
            const double det = j00 * j11 - j01 * j10;
            const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
            const double ax = X(vb[3]), ay = Y(vb[3]), bx = X(vb[5]), by = Y(vb[5]);
            const double dx = bx - ax, dy = by - ay, len = std::sqrt(dx * dx + dy * dy);
            double nx = dy / len, ny = -dx / len;
            const double cx = (x0 + X(ve[2]) + X(ve[4])) / 3 - 0.5 * (ax + bx);
            const double cy = (y0 + Y(ve[2]) + Y(ve[4])) / 3 - 0.5 * (ay + by);
            if (nx * cx + ny * cy < 0)
            {
                nx = -nx;
                ny = -ny;
            }
            for (int q = 0; q < 2; q++)
            {
                ForcePoint fp{};
                const double px = ax + tq[q] * dx - x0, py = ay + tq[q] * dy - y0;
                const double xi = i00 * px + i01 * py, eta = i10 * px + i11 * py;
                // P2 basis (node order c0, m01, c1, m12, c2, m20): reference gradients
                const double rgx[6] = {-3 + 4 * xi + 4 * eta, 4 - 8 * xi - 4 * eta, -1 + 4 * xi, 4 * eta, 0.0,
                                       -4 * eta};
                const double rgy[6] = {-3 + 4 * eta + 4 * xi, -4 * xi, 0.0, 4 * xi, -1 + 4 * eta,
                                       4 - 8 * eta - 4 * xi};
                for (int k = 0; k < 6; k++)
                {
                    fp.v[k] = invV[ve[k]];
                    fp.gx[k] = i00 * rgx[k] + i10 * rgy[k];
                    fp.gy[k] = i01 * rgx[k] + i11 * rgy[k];
                }
                const double psi[3] = {1 - xi - eta, xi, eta};
                for (int k = 0; k < 3; k++)
                {
                    fp.p[k] = pCol[pe[k]];
                    fp.psi[k] = psi[k];
                }
                fp.w = 0.5 * len;
                fp.nx = nx;
                fp.ny = ny;
                pts.push_back(fp);
            }
        }
        require(!pts.empty(), "the border group has no edges");
        auto f = std::make_unique<nsf_forces_s>();
        f->s = S;
        f->npts = (int)pts.size();
        f->pts.upload(pts);
        f->out.alloc(2);
        *out = f.release();
    });
}

extern "C" int nsf_forces_eval(nsf_forces f, double * forces, int onDevice, void * stream)
{
    return guarded([&] {
        require(f && forces, "null argument");
        cudaStream_t s = stream ? asStream(stream) : f->s->stream;
        double * dst = onDevice ? forces : f->out.get();
        NSF_LAUNCH(kForces, 1, s, f->pts.get(), f->npts, f->s->u.get(), f->s->N, f->s->pInt.get(),
                   f->s->cfg.nu, dst, (double *)nullptr);
        if (!onDevice)
        {
            NSF_CUDA(cudaMemcpyAsync(f->host.get(), dst, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
            NSF_CUDA(cudaStreamSynchronize(s));
            forces[0] = f->host.get()[0];
            forces[1] = f->host.get()[1];
        }
    });
}

extern "C" void nsf_forces_destroy(nsf_forces f) { delete f; }

// ============================================================ allocation-free FP64 residual

namespace
{
    constexpr int kNoAllocMaxBlocks = 1024;                 // grid cap of nsf_residual_noalloc
    constexpr int kNoAllocK = 2 * NSF_NOALLOC_MAX_RHS;      // reduced values per block

    // Scratch of nsf_residual_noalloc: the per-block partial sums of the grid reduction
    // (kNoAllocK x kNoAllocMaxBlocks doubles = 64 KiB) and the last-block counter.  Static device
    // memory: zero when the module loads; each completed call leaves the counter at zero again.
    struct NoAllocScratch
    {
        double part[kNoAllocK * kNoAllocMaxBlocks];
        unsigned ticket;
    };
    static __device__ __align__(256) NoAllocScratch g_noallocScratch;

    // r = b - A x per channel and its squared norms (row groups of L lanes, as the row-group SpMV),
    // then one deterministic grid reduction.
    template <int L>
    __global__ void __launch_bounds__(TPB) kResidualNoAlloc(int rows, const int * __restrict__ rs,
                                                            const int * __restrict__ ci,
                                                            const double * __restrict__ v, int nrhs,
                                                            const double * __restrict__ x,
                                                            const double * __restrict__ b, double * __restrict__ r,
                                                            double * norms2, NoAllocScratch * sc)
    {
        Group<L> g;
        double red[kNoAllocK];
#pragma unroll
        for (int k = 0; k < kNoAllocK; k++)
            red[k] = 0;
        for (int row = g.gid; row < rows; row += g.ngroups)
        {
            const int jb = ldg(rs + row), je = ldg(rs + row + 1);
#pragma unroll
            for (int c = 0; c < NSF_NOALLOC_MAX_RHS; c++)
            {
                if (c >= nrhs)
                    break;
                const double * xc = x + (size_t)c * rows;
                double s = 0;
                for (int j = jb + g.lane; j < je; j += L)
                    s += ldg(v + j) * ldg(xc + ldg(ci + j));
                s = g.sum(s);
                if (g.lane == 0)
                {
                    const double bi = b[(size_t)c * rows + row];
                    const double ri = bi - s;
                    r[(size_t)c * rows + row] = ri;
                    red[c] += ri * ri;
                    red[NSF_NOALLOC_MAX_RHS + c] += bi * bi;
                }
            }
        }
        Outs<kNoAllocK> o;
#pragma unroll
        for (int k = 0; k < kNoAllocK; k++)
        {
            const int c = k % NSF_NOALLOC_MAX_RHS;
            o.p[k] = c < nrhs ? norms2 + (k < NSF_NOALLOC_MAX_RHS ? c : nrhs + c) : nullptr;
        }
        gridSum<double, kNoAllocK>(red, sc->part, o, &sc->ticket, nullptr);
    }

    // Device address of the scratch, looked up once per CUDA context and cached under the
    // context's unique id (cuCtxGetId, reached through the runtime's driver entry points so that the
    // library does not link the driver).  A device reset ends the context; the module is loaded
    // again in the next one, possibly at another address, and the new context's id misses the
    // cache, so the address is looked up again.  If the driver entry points are unavailable the
    // address is looked up on every call (cudaGetSymbolAddress allocates nothing).
    NoAllocScratch * noAllocScratch()
    {
        using GetCurrent = int (*)(void **);                 // CUresult cuCtxGetCurrent(CUcontext *)
        using GetId = int (*)(void *, unsigned long long *); // CUresult cuCtxGetId(CUcontext, u64 *)
        static std::mutex m;
        static GetCurrent getCurrent = nullptr;
        static GetId getId = nullptr;
        static bool looked = false;
        static std::vector<std::pair<unsigned long long, NoAllocScratch *>> cache;
        std::lock_guard<std::mutex> lock(m);
        if (!looked)
        {
            cudaDriverEntryPointQueryResult q1{}, q2{};
            void * f1 = nullptr;
            void * f2 = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
                cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
                q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess)
            {
                getCurrent = reinterpret_cast<GetCurrent>(f1);
                getId = reinterpret_cast<GetId>(f2);
            }
            cudaGetLastError();
            looked = true;
        }
        auto contextId = [&]() -> unsigned long long {
            void * c = nullptr;
            unsigned long long id = 0;
            if (getCurrent && getId && getCurrent(&c) == 0 && c && getId(c, &id) == 0)
                return id;
            return 0;
        };
        unsigned long long id = contextId();
        if (id)
            for (const auto & e : cache)
                if (e.first == id)
                    return e.second;
        NoAllocScratch * ptr = nullptr;
        NSF_CUDA(cudaGetSymbolAddress((void **)&ptr, g_noallocScratch)); // makes the primary context current
        id = contextId();
        if (id)
            cache.emplace_back(id, ptr);
        return ptr;
    }
} // namespace

extern "C" int nsf_residual_noalloc(nsf_csr a, int nrhs, const double * x, const double * b, double * r,
                                    double * norms2, void * stream)
{
    return guarded([&] {
        require(a && x && b && r && norms2, "null argument");
        require(a->dtype == NSF_F64, "nsf_residual_noalloc needs an FP64 matrix");
        require(a->rows == a->cols, "nsf_residual_noalloc needs a square matrix");
        if (nrhs < 1 || nrhs > NSF_NOALLOC_MAX_RHS)
            throw Error(ST_INVALID, "nsf_residual_noalloc: nrhs = " + std::to_string(nrhs) +
                                        " is outside 1.." + std::to_string(NSF_NOALLOC_MAX_RHS) +
                                        " (the static scratch holds the reduction of at most that many channels)");
        NoAllocScratch * sc = noAllocScratch();
        const int grid = std::min(cappedBlocks((long long)a->rows * a->L), kNoAllocMaxBlocks);
        cudaStream_t s = asStream(stream);
        NSF_LANES(a->L, NSF_LAUNCH((kResidualNoAlloc<LL>), grid, s, a->rows, a->rs.get(), a->ci.get(),
                                   a->v64.get(), nrhs, x, b, r, norms2, sc));
    });
}

// ============================================================ discrete adjoint (gradients)
#include "adjoint.cuh"

// ============================================================ batched instances (one launch per operation)
#include "batch.cuh"

// ============================================================ packs of steppers (one graph)
#include "pack.cuh"
