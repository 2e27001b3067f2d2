// Test program: the time-step loop of the reference's solveNsChorinCuda
// (cpp/execs/NavierStokes/src/chorinCuda.cu:154-379), written against the cu:: shims of
// include/cu_gb300_shims.hpp as a caller of the reference's cu:: interface would be, FP32 vectors and
// operators as the reference's.  Only the call sites that the shim header lists as changed differ:
// FastConvection + geam as one call, the Dirichlet / pressure gather and scatter through
// cu::scatter / cu::gather, no cuBLAS / cuSPARSE handles.
//
//   chorin_loop <mesh.msh> <peak inflow> <nu> <tau> <steps> <vel method> <vel target> <pres target>
//               <u out> <p out>
//
// The context comes from this library's setup (nsf_context_*), in the shape of the reference's
// buildChorinContext.  u (2N planar) and p (P) after the last step go to vector files of the binary
// interchange format (FP64 values of the FP32 fields).
#include "cu_gb300_shims.hpp"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace
{
    // the members of linalg::CsrMatrix<float> that the shims read
    struct CsrMatrixF
    {
        int rows = 0, cols = 0;
        std::vector<int> rowStart, column;
        std::vector<float> values;
    };

    CsrMatrixF contextMatrix(nsf_context ctx, int which, int rows, int cols, int nnz)
    {
        CsrMatrixF m;
        m.rows = rows;
        m.cols = cols;
        m.rowStart.resize(rows + 1);
        m.column.resize(nnz);
        std::vector<double> v(nnz);
        cu::gb300::check(nsf_context_matrix(ctx, which, m.rowStart.data(), m.column.data(), v.data()),
                         "nsf_context_matrix");
        m.values.assign(v.begin(), v.end());
        return m;
    }
} // namespace

int main(int argc, char ** argv)
{
    if (argc != 11)
    {
        std::fprintf(stderr, "chorin_loop <mesh> <peak> <nu> <tau> <steps> <velMethod> <velTarget> <presTarget> "
                             "<uOut> <pOut>\n");
        return 1;
    }
    try
    {
        const float peak = (float)std::atof(argv[2]);
        const float viscosity = (float)std::atof(argv[3]);
        const float tau = (float)std::atof(argv[4]);
        const int numTimeSteps = std::atoi(argv[5]);
        const std::string velMethod = argv[6];
        const float velTarget = (float)std::atof(argv[7]), presTarget = (float)std::atof(argv[8]);

        nsf_mesh mesh = nullptr;
        nsf_context ctx = nullptr;
        cu::gb300::check(nsf_mesh_load_gmsh(argv[1], &mesh), "nsf_mesh_load_gmsh");
        cu::gb300::check(nsf_context_build(mesh, peak, 0, &ctx), "nsf_context_build");
        int sz[13];
        cu::gb300::check(nsf_context_sizes(ctx, sz), "nsf_context_sizes");
        const int N = sz[0], P = sz[1], nDir = sz[2], nIntP = sz[5];
        const CsrMatrixF velocityMass = contextMatrix(ctx, 0, N, N, sz[6]);
        const CsrMatrixF velocityStiffness = contextMatrix(ctx, 1, N, N, sz[7]);
        const CsrMatrixF pressureStiffnessInternal = contextMatrix(ctx, 3, nIntP, nIntP, sz[9]);
        const CsrMatrixF velocityPressureDiv = contextMatrix(ctx, 4, P, 2 * N, sz[10]);
        const CsrMatrixF pressureVelocityDiv = contextMatrix(ctx, 5, 2 * N, P, sz[11]);
        const CsrMatrixF fastConvectionIntegration = contextMatrix(ctx, 6, sz[7], 2 * N, sz[12]);
        std::vector<int> dirIds(nDir), intP(nIntP);
        std::vector<double> dirVx(nDir);
        cu::gb300::check(nsf_context_lists(ctx, dirIds.data(), dirVx.data(), nullptr, nullptr, intP.data()),
                         "nsf_context_lists");

        // ---- chorinCuda.cu:166-230, setup
        cu::csrF velocityStiffnessPlusConvection(velocityStiffness);
        cu::csrF pressureVelocityDivD(pressureVelocityDiv);
        cu::csrF velocityPressureDivD(velocityPressureDiv);
        cu::csrF fastConvection(fastConvectionIntegration);
        cu::vec<float> origVelocityM1Vals(velocityStiffnessPlusConvection.values);
        cu::scale(origVelocityM1Vals.size(), origVelocityM1Vals.get(), viscosity);
        cu::spmm aSpmm(velocityStiffnessPlusConvection, 2);

        cu::vec<float> velocityXy(2 * N);
        velocityXy.memsetZero();
        // DirichletVelocity: x values at the ids, y values 0 at ids + N
        std::vector<int> dIds(2 * (size_t)nDir);
        std::vector<float> dVals(2 * (size_t)nDir, 0.0f);
        for (int i = 0; i < nDir; i++)
        {
            dIds[i] = dirIds[i];
            dVals[i] = (float)dirVx[i];
            dIds[nDir + i] = dirIds[i] + N;
        }
        cu::vec<int> dirIdsD(dIds);
        cu::vec<float> dirValsD(dVals);
        auto impose = [&]() { cu::scatter(dirIdsD, dirValsD.get(), velocityXy.get()); };
        impose();

        auto velocitySolver = cu::createSolver(velMethod, 2, velocityMass, 1000, velTarget, 1);
        auto & accel = velocitySolver->getSol();
        cu::spmv vpdSpmv(velocityPressureDivD);
        auto pressureSolverCore = cu::createSolver("pcg", 1, pressureStiffnessInternal, 20000, presTarget, 1);
        // PressureSolver: dense pressure, internal ids; the solver keeps its solution (warm start)
        cu::vec<float> dense(P);
        cu::vec<int> internalIds(intP);
        cu::spmv pvdSpmv(pressureVelocityDivD);
        auto & nablaPXy = pvdSpmv.b;
        const float invTau = -1.0f / tau;

        for (int iT = 0; iT < numTimeSteps; iT++)
        {
            // ---- chorinCuda.cu:240-251: A = nu M1 + C(u)
            cu::fastConvection(fastConvection, origVelocityM1Vals, velocityXy, velocityStiffnessPlusConvection.values);
            // ---- chorinCuda.cu:262-278: tentative velocity
            auto & accelRhs = velocitySolver->getRhs();
            aSpmm.compute(velocityXy, accelRhs);
            accel.memsetZero();
            velocitySolver->solve();
            cu::saxpy(2 * N, accel.get(), velocityXy.get(), -tau);
            impose();
            // ---- chorinCuda.cu:297-300: pressure (PressureSolver::update)
            vpdSpmv.compute(velocityXy, dense);
            cu::scale(dense.size(), dense.get(), invTau);
            cu::gather(internalIds, dense.get(), pressureSolverCore->getRhs().get());
            pressureSolverCore->solve();
            dense.memsetZero();
            cu::scatter(internalIds, pressureSolverCore->getSol().get(), dense.get());
            // ---- chorinCuda.cu:341-356: final velocity
            pvdSpmv.compute(dense, nablaPXy);
            nablaPXy.copyTo(accelRhs);
            accel.memsetZero();
            velocitySolver->solve();
            cu::saxpy(2 * N, accel.get(), velocityXy.get(), -tau);
            impose();
            std::printf("%d: tent/final iters %d, pressure iters %d, pressure MSE %g\n", iT,
                        velocitySolver->getLastIterations(), pressureSolverCore->getLastIterations(),
                        pressureSolverCore->getLastMse());
        }

        std::vector<float> u, p;
        velocityXy.download(u);
        dense.download(p);
        std::vector<double> ud(u.begin(), u.end()), pd(p.begin(), p.end());
        cu::gb300::check(nsf_io_write_vec(argv[9], (int)ud.size(), ud.data(), NSF_F64), "nsf_io_write_vec");
        cu::gb300::check(nsf_io_write_vec(argv[10], (int)pd.size(), pd.data(), NSF_F64), "nsf_io_write_vec");
        nsf_context_destroy(ctx);
        nsf_mesh_destroy(mesh);
    }
    catch (const std::exception & e)
    {
        std::fprintf(stderr, "chorin_loop: %s\n", e.what());
        return 2;
    }
    return 0;
}
