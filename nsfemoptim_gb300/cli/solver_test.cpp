// nsf_solver_test: command-line solver test over the C ABI, with the command line and the output of the
// reference's SolverTest (cpp/tests/SolverTest/src/solverTest.cpp:271-360), so that a system dumped
// by the reference (linalg::write of the matrix and of the right-hand side) can be solved here.
//
//   nsf_solver_test <algo> <matrix> <rhs> [maxIters] [eps]
//
// <matrix>, <rhs>: files of the binary interchange format (float or double).  The right-hand side may
// hold several interleaved channels (xyxy...), as the reference's; its size fixes their count.
// maxIters and eps default to the reference's 100 and 1e-9.
// Algorithms (the GPU ones of the reference, run on this library's solvers):
//   gaussSeidelCuda   multicolor Gauss-Seidel, one channel at a time, RMS target eps (cu::GaussSeidelHost)
//   gaussSeidelCuda2  the same with both channels of a two-channel right-hand side in one solve
//   cgCuda            CG, here preconditioned by multicolor symmetric Gauss-Seidel, stopping at
//                     ||b - A x|| <= eps ||b|| (the reference's cgCuda is unpreconditioned)
//   pcgMixed          the same CG in FP32 with FP64 residual refinement
// The reference's CPU algorithms (cg, cgd, jacobi, gaussSeidel, gaussSeidelCustom) are not provided.
// Output: the reference's lines ("Matrix size = ...", "Final MSE = ..." with MSE the RMS of A x - b,
// as CsrMatrix::mse) plus "Iterations = ..." and "Status = ...".  Exit status 0 unless the input
// cannot be read or the solver cannot be created; a solve that stops at its iteration cap still
// prints its MSE, as the reference's loop does.
#include "../../include/nsfem_gb300.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace
{
    double rmsResidual(int n, const std::vector<int> & rs, const std::vector<int> & ci, const std::vector<double> & v,
                       const double * x, const double * b)
    {
        double sum = 0;
        for (int i = 0; i < n; i++)
        {
            double a = 0;
            for (int j = rs[i]; j < rs[i + 1]; j++)
                a += v[j] * x[ci[j]];
            const double d = a - b[i];
            sum += d * d;
        }
        return std::sqrt(sum / n);
    }

    int fail(const std::string & msg)
    {
        std::fprintf(stderr, "%s\n", msg.c_str());
        return 1;
    }
} // namespace

int main(int argc, char ** argv)
{
    if (argc < 4 || argc > 6)
        return fail("./nsf_solver_test <algo> <matrix> <rhs> [maxIters] [eps]");
    const std::string algo = argv[1], matPath = argv[2], rhsPath = argv[3];
    const int maxIters = argc > 4 ? std::atoi(argv[4]) : 100;
    const double eps = argc > 5 ? std::atof(argv[5]) : 1e-9;

    int info[4];
    if (nsf_io_csr_info(matPath.c_str(), info) != NSF_OK)
        return fail(nsf_last_error());
    const int rows = info[0], cols = info[1], nnz = info[2];
    std::vector<int> rs(rows + 1), ci(nnz);
    std::vector<double> val(nnz);
    if (nsf_io_read_csr(matPath.c_str(), rs.data(), ci.data(), val.data()) != NSF_OK)
        return fail(nsf_last_error());
    int vinfo[2];
    if (nsf_io_vec_info(rhsPath.c_str(), vinfo) != NSF_OK)
        return fail(nsf_last_error());
    std::vector<double> rhs(vinfo[0]);
    if (nsf_io_read_vec(rhsPath.c_str(), rhs.data()) != NSF_OK)
        return fail(nsf_last_error());

    std::printf("Matrix size = %dx%d\n", rows, cols);
    std::printf("RHS size = %zu\n", rhs.size());
    if (rows != cols)
        return fail("Only square matrices supported for now");
    const int n = rows;
    const int numCh = (int)rhs.size() / n;
    if ((size_t)numCh * n != rhs.size())
        return fail("Failed to determine number of channels");
    std::printf("Number of channels = %d\n", numCh);

    std::string method;
    int precision = NSF_PREC_F64, algoCh = 1;
    if (algo == "gaussSeidelCuda")
        method = "gs";
    else if (algo == "gaussSeidelCuda2")
    {
        method = "gs";
        algoCh = 2;
    }
    else if (algo == "cgCuda")
        method = "pcg";
    else if (algo == "pcgMixed")
    {
        method = "pcg";
        precision = NSF_PREC_MIXED;
    }
    else if (algo == "cg" || algo == "cgd" || algo == "jacobi" || algo == "gaussSeidel" || algo == "gaussSeidelCustom")
        return fail("Algorithm " + algo + " is one of the reference's CPU algorithms, not provided here");
    else
        return fail("No algorithm matching " + algo);

    nsf_solver s = nullptr;
    if (nsf_solver_create(method.c_str(), algoCh, n, rs.data(), ci.data(), val.data(), precision, maxIters, eps, 1,
                          &s) != NSF_OK)
        return fail(nsf_last_error());

    // channels: interleaved in the file (xyxy...), planar for the solver
    std::vector<std::vector<double>> ch(numCh, std::vector<double>(n));
    for (int i = 0; i < n; i++)
        for (int c = 0; c < numCh; c++)
            ch[c][i] = rhs[(size_t)i * numCh + c];

    auto report = [&](int status) {
        int it = 0;
        nsf_solver_stats(s, &it, nullptr, nullptr);
        std::printf("Iterations = %d\n", it);
        std::printf("Status = %s\n", nsf_status_string(status));
    };

    if (algoCh == 1)
    {
        std::printf("Single channel solve\n");
        for (int c = 0; c < numCh; c++)
        {
            std::printf("================ Channel %d ================\n", c);
            std::vector<double> x(n, 0.0);
            const int st = nsf_solver_solve_host(s, ch[c].data(), x.data());
            report(st);
            std::printf("Final MSE = %.9g\n", rmsResidual(n, rs, ci, val, x.data(), ch[c].data()));
        }
    }
    else
    {
        std::printf("Two channel solve\n");
        if (numCh != 2)
        {
            nsf_solver_destroy(s);
            return fail("Impossible - input doesn't have 2 channels");
        }
        std::vector<double> b(2 * (size_t)n), x(2 * (size_t)n, 0.0);
        std::copy(ch[0].begin(), ch[0].end(), b.begin());
        std::copy(ch[1].begin(), ch[1].end(), b.begin() + n);
        const int st = nsf_solver_solve_host(s, b.data(), x.data());
        report(st);
        std::printf("Final MSE = %.9g / %.9g\n", rmsResidual(n, rs, ci, val, x.data(), b.data()),
                    rmsResidual(n, rs, ci, val, x.data() + n, b.data() + n));
    }
    nsf_solver_destroy(s);
    return 0;
}
