// C++ shims with the class names and methods of the reference's cu:: interface
// (kosyonikolov/NsFemOptim, cpp/libs/CudaUtils/include/cu/), implemented over the C ABI of
// nsfem_gb300.h, so that callers written against cu:: (the reference's solveNsChorinCuda loop,
// cpp/execs/NavierStokes/src/chorinCuda.cu:154-379) build against this library.
//
// Header-only C++17; it needs the CUDA runtime API for the device buffers of cu::vec (cudaMalloc,
// cudaMemcpy), which every user of the reference's cu:: already links.  Errors throw
// std::runtime_error, as the reference's classes do.
//
// What the reference's caller changes (the shims cannot hide these):
//   * the cuBLAS / cuSPARSE handles (cu::Blas, cu::Sparse) are gone: spmv / spmm take no handle
//     and saxpy / scale no Blas object;
//   * C = I u followed by cublasSgeam (A = nu K + C, chorinCuda.cu:243-250) is one call,
//     cu::fastConvection(I, nuK, u, A) (nsf_fastconv_apply with nu = 1 on pre-scaled values);
//   * the Dirichlet scatter and the internal-pressure gather / scatter (chorinCuda.cu:20-150) use
//     cu::scatter / cu::gather;
//   * a matrix whose values the caller overwrites on the device and then applies through cu::spmv
//     calls csrF::valuesChanged() (cu::spmm reads the values as they are).
// The matrix arguments are templates over any type with the members of linalg::CsrMatrix<float>
// (rows, cols, rowStart, column, values as std::vector), the reference's own type included.
#ifndef CU_GB300_SHIMS_HPP
#define CU_GB300_SHIMS_HPP

#include "nsfem_gb300.h"

#include <cuda_runtime_api.h>

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace cu
{
    namespace gb300
    {
        inline void check(int status, const char * what)
        {
            if (status != NSF_OK)
                throw std::runtime_error(std::string(what) + ": " + nsf_status_string(status) + " (" +
                                         nsf_last_error() + ")");
        }

        inline void checkCuda(cudaError_t e, const char * what)
        {
            if (e != cudaSuccess)
                throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
        }

    } // namespace gb300

    // cu::vec (vec.h:16-388): a device buffer, owning (allocated here) or a view of memory owned
    // elsewhere (the X / Y halves of a planar vector, chorinCuda.cu:195-196).
    template <typename T>
    class vec
    {
        T * ptr = nullptr;
        int n = 0;
        bool owns = false;

    public:
        vec() = default;
        explicit vec(int size) : n(size), owns(true)
        {
            if (n > 0)
                gb300::checkCuda(cudaMalloc((void **)&ptr, sizeof(T) * (size_t)n), "cudaMalloc");
        }
        vec(T * p, int size) : ptr(p), n(size), owns(false) {}
        explicit vec(const std::vector<T> & h) : vec((int)h.size()) { upload(h); }
        vec(const vec & o) : vec(o.n)
        {
            if (n > 0)
                gb300::checkCuda(cudaMemcpy(ptr, o.ptr, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice), "copy");
        }
        vec(vec && o) noexcept : ptr(o.ptr), n(o.n), owns(o.owns)
        {
            o.ptr = nullptr;
            o.owns = false;
        }
        vec & operator=(const vec &) = delete;
        vec & operator=(vec && o) noexcept
        {
            if (this != &o)
            {
                if (owns && ptr)
                    cudaFree(ptr);
                ptr = o.ptr;
                n = o.n;
                owns = o.owns;
                o.ptr = nullptr;
                o.owns = false;
            }
            return *this;
        }
        ~vec()
        {
            if (owns && ptr)
                cudaFree(ptr);
        }

        T * get() const { return ptr; }
        int size() const { return n; }
        void memsetZero()
        {
            gb300::checkCuda(cudaMemset(ptr, 0, sizeof(T) * (size_t)n), "cudaMemset");
        }
        void upload(const std::vector<T> & h)
        {
            if ((int)h.size() != n)
                throw std::invalid_argument("cu::vec::upload: size mismatch");
            gb300::checkCuda(cudaMemcpy(ptr, h.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice), "upload");
        }
        void download(std::vector<T> & h) const
        {
            h.resize(n);
            gb300::checkCuda(cudaMemcpy(h.data(), ptr, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost), "download");
        }
        void copyTo(vec & dst) const
        {
            if (dst.n != n)
                throw std::invalid_argument("cu::vec::copyTo: size mismatch");
            gb300::checkCuda(cudaMemcpy(dst.ptr, ptr, sizeof(T) * (size_t)n, cudaMemcpyDeviceToDevice), "copyTo");
        }
    };

    // cu::csrF (csrF.h:12-30): a device FP32 CSR.  `values` views the device CSR values (the target
    // of cu::fastConvection).
    class csrF
    {
    public:
        int rows = 0, cols = 0, nnz = 0;
        nsf_csr h = nullptr;
        vec<float> values;

        template <typename M>
        explicit csrF(const M & m) : rows(m.rows), cols(m.cols), nnz((int)m.values.size())
        {
            std::vector<float> v(m.values.begin(), m.values.end());
            gb300::check(nsf_csr_create(m.rows, m.cols, nnz, m.rowStart.data(), m.column.data(), v.data(), NSF_F32, &h),
                         "nsf_csr_create");
            int * rs = nullptr;
            int * ci = nullptr;
            void * dv = nullptr;
            gb300::check(nsf_csr_device(h, &rs, &ci, &dv), "nsf_csr_device");
            values = vec<float>(static_cast<float *>(dv), nnz);
        }
        csrF(const csrF &) = delete;
        csrF & operator=(const csrF &) = delete;
        ~csrF() { nsf_csr_destroy(h); }

        // after the device values were overwritten: refresh the copies that spmv reads
        void valuesChanged() { gb300::check(nsf_csr_update_values(h, values.get(), 1, nullptr), "nsf_csr_update_values"); }
    };

    // cu::spmv (spmv.h:13-47): b = M x with the default or the supplied operands
    class spmv
    {
    public:
        csrF & mat;
        vec<float> x, b;

        explicit spmv(csrF & m) : mat(m), x(m.cols), b(m.rows) {}
        void compute() { compute(x, b); }
        void compute(vec<float> & ox, vec<float> & ob)
        {
            gb300::check(nsf_spmv(mat.h, ox.get(), ob.get(), 1.0, 0.0, nullptr), "nsf_spmv");
        }
    };

    // cu::spmm (spmm.h:14-49): B = M X for numCh planar channels
    class spmm
    {
    public:
        csrF & mat;
        int numCh;
        vec<float> x, b;

        spmm(csrF & m, int channels) : mat(m), numCh(channels), x(m.cols * channels), b(m.rows * channels) {}
        void compute() { compute(x, b); }
        void compute(vec<float> & ox, vec<float> & ob)
        {
            gb300::check(nsf_spmm(mat.h, numCh, ox.get(), mat.cols, ob.get(), mat.rows, nullptr), "nsf_spmm");
        }
    };

    // cu::saxpy / cu::scale (blas.h:24-26) without the cuBLAS handle: dst += alpha src, x *= alpha
    inline void saxpy(int n, const float * src, float * dst, float alpha)
    {
        gb300::check(nsf_axpy(n, alpha, src, dst, NSF_F32, nullptr), "nsf_axpy");
    }
    inline void scale(int n, float * x, float alpha)
    {
        gb300::check(nsf_scale(n, alpha, x, NSF_F32, nullptr), "nsf_scale");
    }

    // dst[idx[i]] = src[i] / dst[i] = src[idx[i]] for the n entries of the device index vector idx
    inline void scatter(const vec<int> & idx, const float * src, float * dst)
    {
        gb300::check(nsf_scatter(idx.size(), idx.get(), src, dst, NSF_F32, nullptr), "nsf_scatter");
    }
    inline void gather(const vec<int> & idx, const float * src, float * dst)
    {
        gb300::check(nsf_gather(idx.size(), idx.get(), src, dst, NSF_F32, nullptr), "nsf_gather");
    }

    // A = nuK + I u: the FastConvection product and the cublasSgeam of the reference's loop in one
    // call (nuK: the stiffness values already scaled by the viscosity, as the reference keeps them)
    inline void fastConvection(csrF & I, const vec<float> & nuK, const vec<float> & u, vec<float> & A)
    {
        gb300::check(nsf_fastconv_apply(I.h, nuK.get(), 1.0, u.get(), A.get(), nullptr), "nsf_fastconv_apply");
    }

    // cu::AbstractSolver (solvers/abstractSolver.h:8-32)
    class AbstractSolver
    {
    public:
        virtual ~AbstractSolver() = default;
        virtual int getNumCh() const = 0;
        virtual float getLastMse(const int ch = -1) const = 0;
        virtual int getLastIterations() const = 0;
        virtual vec<float> & getRhs() = 0;
        virtual vec<float> & getSol() = 0;
        virtual void solve() = 0;
        virtual void setMaxIters(const int maxIters) = 0;
        virtual void setTargetMse(const float targetMse) = 0;
        virtual void setMseCheckInterval(const int interval) = 0;
    };

    namespace gb300
    {
        // an nsf_solver behind the AbstractSolver interface, with the reference's FP32 IO vectors
        class Solver final : public AbstractSolver
        {
            nsf_solver h = nullptr;
            int numCh, n, maxIters, interval;
            float target;
            vec<float> rhs, sol;

        public:
            template <typename M>
            Solver(const char * method, int channels, const M & m, int maxIt, float targetMse, int checkInterval,
                   int precision)
                : numCh(channels), n(m.rows), maxIters(maxIt), interval(checkInterval), target(targetMse),
                  rhs(channels * m.rows), sol(channels * m.rows)
            {
                std::vector<double> v(m.values.begin(), m.values.end());
                check(nsf_solver_create(method, numCh, n, m.rowStart.data(), m.column.data(), v.data(), precision,
                                        maxIters, target, interval, &h),
                      "nsf_solver_create");
            }
            ~Solver() override { nsf_solver_destroy(h); }

            int getNumCh() const override { return numCh; }
            float getLastMse(const int ch = -1) const override
            {
                double rms[2] = {0, 0};
                check(nsf_solver_stats(h, nullptr, rms, nullptr), "nsf_solver_stats");
                if (ch >= 0)
                    return (float)rms[ch];
                double s = 0;
                for (int c = 0; c < numCh; c++)
                    s += rms[c] * rms[c];
                return (float)std::sqrt(s / numCh);
            }
            int getLastIterations() const override
            {
                int it = 0;
                check(nsf_solver_stats(h, &it, nullptr, nullptr), "nsf_solver_stats");
                return it;
            }
            vec<float> & getRhs() override { return rhs; }
            vec<float> & getSol() override { return sol; }
            void solve() override
            {
                // as the reference's solvers: an iteration cap reached is reported through the MSE
                const int st = nsf_solver_solve_f32(h, rhs.get(), sol.get(), nullptr);
                if (st != NSF_OK && st != NSF_ERR_MAXITER)
                    check(st, "nsf_solver_solve_f32");
            }
            void setMaxIters(const int k) override
            {
                maxIters = k;
                check(nsf_solver_set(h, maxIters, target, interval), "nsf_solver_set");
            }
            void setTargetMse(const float t) override
            {
                target = t;
                check(nsf_solver_set(h, maxIters, target, interval), "nsf_solver_set");
            }
            void setMseCheckInterval(const int k) override
            {
                interval = k;
                check(nsf_solver_set(h, maxIters, target, interval), "nsf_solver_set");
            }
        };
    } // namespace gb300

    // cu::createSolver (solvers/solverFactory.h:13-14): "gs" the multicolor Gauss-Seidel (absolute
    // RMS target), "pcg" (and "cg", "dss") CG with the multicolor SGS preconditioner (relative
    // target); FP64 solves on FP32 IO vectors
    template <typename M>
    std::unique_ptr<AbstractSolver> createSolver(const std::string & name, const int numCh, const M & m,
                                                 const int maxIters, const float targetMse, const int mseCheckInterval)
    {
        const char * method = name == "gs" ? "gs" : "pcg";
        return std::make_unique<gb300::Solver>(method, numCh, m, maxIters, targetMse, mseCheckInterval, NSF_PREC_F64);
    }
} // namespace cu

#endif
