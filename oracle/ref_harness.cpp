// Test-only harness around the reference's own C++ sources (compiled from the reference tree by
// oracle/Makefile.ref into oracle/_ref/libnsfref.so).  It is the checker's checker: the C oracle
// and the product's host setup are compared against what the reference code itself produces for
// gmsh parsing, P1/P2 numbering, Dirichlet/internal node lists, CSR sparsity prototypes, the
// smallest-last + greedy coloring used by cu::GaussSeidel, CSR slicing and CPU Gauss-Seidel.
//
// Reference entry points driven here:
//   mesh::parseTriangleGmsh        cpp/libs/Mesh/src/io.cpp:65-214
//   mesh::createMesh               cpp/libs/Mesh/src/concreteMesh.cpp:78-293
//   extractDirichletNodes          cpp/execs/NavierStokes/include/NavierStokes/borders.h:12-47
//   extractInternalNodes           cpp/execs/NavierStokes/src/borders.cpp:19-51
//   SparseMatrixPrototypeBuilder   cpp/libs/LinAlg/src/sparseDokBuilder.cpp:310-364
//   buildCsrGraph / buildSmallestLastOrdering / partitionGraphGreedy  cpp/libs/LinAlg/src/graphs.cpp
//   CsrMatrix<float>::slice        cpp/libs/LinAlg/src/csrMatrix.cpp:12-91
//   gaussSeidel2ch<double>         cpp/libs/LinAlg/src/gaussSeidel.cpp:215-230
//   linalg::write / readCsr / readVec   cpp/libs/LinAlg/src/io.cpp:49-192 (binary interchange files)
//   buildChorinCsrMatrices<float>  cpp/libs/Fem/src/chorinCsr.cpp:436-502 (assembled FP32 values)
//   TriangleIntegrator             cpp/libs/Element/src/triangleIntegrator.cpp:113-293 (local matrices)
// Those two files include OpenCV for cv::Mat; they compile here against the test-only stand-in in
// oracle/cvstub.  The element-pattern loops below restate buildPrototypes
// (cpp/libs/Fem/src/chorinCsr.cpp:61-140) and the FastConvection construction
// (cpp/libs/Fem/src/fastConvection.cpp:17-100), whose file needs Eigen, on top of the reference's
// prototype builder and integrator.
#include <algorithm>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include <element/p1.h>
#include <element/p2.h>
#include <element/triangleIntegrator.h>
#include <fem/chorinCsr.h>
#include <linalg/csrMatrix.h>
#include <linalg/gaussSeidel.h>
#include <linalg/io.h>
#include <linalg/graphs.h>
#include <linalg/sparseDokBuilder.h>
#include <mesh/concreteMesh.h>
#include <mesh/io.h>
#include <NavierStokes/borders.h>
#include <NavierStokes/dfgCondtions.h>

namespace
{
    struct RefMesh
    {
        el::P1 p1;
        el::P2 p2;
        mesh::TriangleMesh tri;
        mesh::ConcreteMesh vmesh;
        mesh::ConcreteMesh pmesh;
        std::unique_ptr<fem::ChorinCsrMatrices<float>> mats; // assembled on first use
    };

    constexpr int kIntegrationDegree = 4; // cpp/execs/NavierStokes/src/buildContext.cpp:102

    struct RefCsr
    {
        linalg::CsrMatrix<float> m;
    };

    thread_local std::string lastError;

    template <typename F>
    int refWriteCsr(const char * path, int rows, int cols, int nnz, const int * rs, const int * ci,
                           const double * v)
    {
        linalg::CsrMatrix<F> m;
        m.rows = rows;
        m.cols = cols;
        m.rowStart.assign(rs, rs + rows + 1);
        m.column.assign(ci, ci + nnz);
        m.values.resize(nnz);
        for (int i = 0; i < nnz; i++)
            m.values[i] = (F)v[i];
        linalg::write(std::string(path), m);
        return 0;
    }

    template <typename F>
    int refReadCsr(const char * path, int * dims, int * rs, int * ci, double * v)
    {
        const auto m = linalg::readCsr<F>(std::string(path));
        dims[0] = m.rows;
        dims[1] = m.cols;
        dims[2] = (int)m.column.size();
        if (rs)
        {
            std::copy(m.rowStart.begin(), m.rowStart.end(), rs);
            std::copy(m.column.begin(), m.column.end(), ci);
            for (size_t i = 0; i < m.values.size(); i++)
                v[i] = m.values[i];
        }
        return 0;
    }

}

extern "C"
{
    const char * ref_last_error() { return lastError.c_str(); }

    void * ref_mesh_load(const char * path)
    {
        try
        {
            auto * h = new RefMesh();
            h->tri = mesh::parseTriangleGmsh(std::string(path));
            h->vmesh = mesh::createMesh(h->tri, h->p2);
            h->pmesh = mesh::createMesh(h->tri, h->p1);
            return h;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return nullptr;
        }
    }

    void ref_mesh_free(void * h) { delete static_cast<RefMesh *>(h); }

    // counts[0..5] = corner nodes, triangles, border elements, P2 nodes, P1 nodes, groups
    void ref_mesh_counts(void * hv, int * counts)
    {
        auto * h = static_cast<RefMesh *>(hv);
        counts[0] = (int)h->tri.nodes.size();
        counts[1] = (int)h->tri.elements.size();
        counts[2] = (int)h->tri.borderElements.size();
        counts[3] = (int)h->vmesh.nodes.size();
        counts[4] = (int)h->pmesh.nodes.size();
        counts[5] = (int)h->tri.groups.size();
    }

    const char * ref_mesh_group(void * hv, int i) { return static_cast<RefMesh *>(hv)->tri.groups[i].c_str(); }

    // which: 1 = P1 mesh, 2 = P2 mesh
    void ref_mesh_elements(void * hv, int which, int * out)
    {
        auto * h = static_cast<RefMesh *>(hv);
        const auto & m = which == 2 ? h->vmesh : h->pmesh;
        std::copy(m.elements.begin(), m.elements.end(), out);
    }

    void ref_mesh_nodes(void * hv, int which, float * out)
    {
        auto * h = static_cast<RefMesh *>(hv);
        const auto & m = which == 2 ? h->vmesh : h->pmesh;
        for (size_t i = 0; i < m.nodes.size(); i++)
        {
            out[2 * i] = m.nodes[i].x;
            out[2 * i + 1] = m.nodes[i].y;
        }
    }

    // P2 border elements, (3 + 3) ints each: triangle, side, group, pt0, pt1 (end), pt2 (mid)
    void ref_mesh_border(void * hv, int which, int * out)
    {
        auto * h = static_cast<RefMesh *>(hv);
        const auto & m = which == 2 ? h->vmesh : h->pmesh;
        std::copy(m.borderElements.begin(), m.borderElements.end(), out);
    }

    // Dirichlet lists of the channel problem (buildContext.cpp:64-93): returns counts
    // [nVx, nP, nInternalV, nInternalP]; ids/values written when the out pointers are non-null.
    void ref_dirichlet(void * hv, float peakVelocity, int * counts,
                       int * vxIds, float * vxVals, int * pIds, int * internalV, int * internalP)
    {
        auto * h = static_cast<RefMesh *>(hv);
        DfgConditions cond{0.001f, peakVelocity};
        const auto & vm = h->vmesh;
        const auto & pm = h->pmesh;
        auto zero = [](const mesh::ConcreteMesh &, const int, const int) -> float { return 0.0f; };
        auto vx = [&](const mesh::ConcreteMesh & mesh, const int nodeId, const int borderId) -> float
        {
            if (mesh.groups[borderId] == "Left")
            {
                return cond.calcLeftVelocity(mesh.nodes[nodeId].y);
            }
            return 0.0f;
        };
        const std::vector<int> vIds = {vm.findGroupId("Left"), vm.findGroupId("Top"), vm.findGroupId("Bottom"),
                                       vm.findGroupId("Circle")};
        const std::vector<int> pIdsB = {pm.findGroupId("Right")};
        auto dvx = extractDirichletNodes(vm, vIds, vx);
        auto dp = extractDirichletNodes(pm, pIdsB, zero);
        auto iv = extractInternalNodes((int)vm.nodes.size(), dvx);
        auto ip = extractInternalNodes((int)pm.nodes.size(), dp);
        counts[0] = (int)dvx.size();
        counts[1] = (int)dp.size();
        counts[2] = (int)iv.size();
        counts[3] = (int)ip.size();
        if (vxIds)
        {
            for (size_t i = 0; i < dvx.size(); i++)
            {
                vxIds[i] = dvx[i].id;
                vxVals[i] = dvx[i].value;
            }
            for (size_t i = 0; i < dp.size(); i++)
            {
                pIds[i] = dp[i].id;
            }
            std::copy(iv.begin(), iv.end(), internalV);
            std::copy(ip.begin(), ip.end(), internalP);
        }
    }

    // Sparsity prototypes: which = 0 velocity (N x N), 1 pressure (P x P), 2 D (P x 2N),
    // 3 G (2N x P), 4 FastConvection integration (nnz(velocity) x 2N).
    void * ref_prototype(void * hv, int which)
    {
        auto * h = static_cast<RefMesh *>(hv);
        const auto & vm = h->vmesh;
        const auto & pm = h->pmesh;
        const int N = (int)vm.nodes.size();
        const int P = (int)pm.nodes.size();
        const int nE = vm.numElements;
        std::vector<int> iv(6), ip(3);
        auto * out = new RefCsr();
        using Builder = linalg::SparseMatrixPrototypeBuilder;
        if (which == 0 || which == 4)
        {
            Builder b(N, N);
            for (int e = 0; e < nE; e++)
            {
                vm.getElement(e, iv.data(), nullptr);
                for (int r = 0; r < 6; r++)
                    for (int c = 0; c < 6; c++)
                        b.add(iv[r], iv[c]);
            }
            auto proto = b.buildCsrPrototype2<float>();
            if (which == 0)
            {
                out->m = std::move(proto);
            }
            else
            {
                const int nnz = (int)proto.column.size();
                Builder bi(nnz, 2 * N);
                std::vector<int> offs(6);
                for (int e = 0; e < nE; e++)
                {
                    vm.getElement(e, iv.data(), nullptr);
                    for (int r = 0; r < 6; r++)
                    {
                        proto.findOffsetsUnsorted(iv[r], iv, offs);
                        for (int c = 0; c < 6; c++)
                            for (int k = 0; k < 6; k++)
                            {
                                bi.add(offs[c], iv[k]);
                                bi.add(offs[c], iv[k] + N);
                            }
                    }
                }
                out->m = bi.buildCsrPrototype2<float>();
            }
        }
        else if (which == 1)
        {
            Builder b(P, P);
            for (int e = 0; e < nE; e++)
            {
                pm.getElement(e, ip.data(), nullptr);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++)
                        b.add(ip[r], ip[c]);
            }
            out->m = b.buildCsrPrototype2<float>();
        }
        else
        {
            Builder b(which == 2 ? P : 2 * N, which == 2 ? 2 * N : P);
            for (int e = 0; e < nE; e++)
            {
                vm.getElement(e, iv.data(), nullptr);
                pm.getElement(e, ip.data(), nullptr);
                for (int a = 0; a < 6; a++)
                    for (int q = 0; q < 3; q++)
                    {
                        if (which == 2)
                        {
                            b.add(ip[q], iv[a]);
                            b.add(ip[q], iv[a] + N);
                        }
                        else
                        {
                            b.add(iv[a], ip[q]);
                            b.add(iv[a] + N, ip[q]);
                        }
                    }
            }
            out->m = b.buildCsrPrototype2<float>();
        }
        out->m.values.assign(out->m.column.size(), 0.0f);
        return out;
    }

    void * ref_csr_wrap(int rows, int cols, int nnz, const int * rowStart, const int * column, const float * values)
    {
        auto * out = new RefCsr();
        out->m.rows = rows;
        out->m.cols = cols;
        out->m.rowStart.assign(rowStart, rowStart + rows + 1);
        out->m.column.assign(column, column + nnz);
        if (values)
            out->m.values.assign(values, values + nnz);
        else
            out->m.values.assign(nnz, 0.0f);
        return out;
    }

    void ref_csr_free(void * c) { delete static_cast<RefCsr *>(c); }

    // dims[0..2] = rows, cols, nnz
    void ref_csr_dims(void * cv, int * dims)
    {
        auto & m = static_cast<RefCsr *>(cv)->m;
        dims[0] = m.rows;
        dims[1] = m.cols;
        dims[2] = (int)m.column.size();
    }

    void ref_csr_arrays(void * cv, int * rowStart, int * column, float * values)
    {
        auto & m = static_cast<RefCsr *>(cv)->m;
        std::copy(m.rowStart.begin(), m.rowStart.end(), rowStart);
        std::copy(m.column.begin(), m.column.end(), column);
        if (values)
            std::copy(m.values.begin(), m.values.end(), values);
    }

    void * ref_csr_slice(void * cv, int nRows, const int * rowIds, int nCols, const int * colIds)
    {
        auto & m = static_cast<RefCsr *>(cv)->m;
        auto * out = new RefCsr();
        out->m = m.slice(std::span<const int>(rowIds, nRows), std::span<const int>(colIds, nCols));
        return out;
    }

    // The coloring of cu::GaussSeidel's constructor (gaussSeidel.cu:132-155): smallest-last
    // order, greedy partition, each partition sorted and concatenated.  Returns the number of
    // colors; order[n] receives the concatenated partitions, partStart[nColors + 1] the offsets
    // (partStart may be null to query the color count), slOrder[n] the smallest-last order.
    int ref_coloring(void * cv, int * order, int * partStart, int * slOrder)
    {
        auto & m = static_cast<RefCsr *>(cv)->m;
        auto graph = linalg::buildCsrGraph(m);
        auto sl = linalg::buildSmallestLastOrdering(graph);
        auto parts = linalg::partitionGraphGreedy(graph, sl);
        const int nColors = (int)parts.size();
        int i = 0;
        for (int c = 0; c < nColors; c++)
        {
            auto & p = parts[c];
            std::sort(p.begin(), p.end());
            if (partStart)
                partStart[c] = i;
            if (order)
                std::copy(p.begin(), p.end(), order + i);
            i += (int)p.size();
        }
        if (partStart)
            partStart[nColors] = i;
        if (slOrder)
            std::copy(sl.begin(), sl.end(), slOrder);
        return nColors;
    }

    // Sequential interleaved 2-channel Gauss-Seidel in double (gaussSeidel.cpp:215-230).
    // x is updated in place; returns the iteration-final RMS residuals in res[2].
    void ref_gs2ch_double(int rows, const int * rowStart, const int * column, const double * values,
                          double * x, const double * b, int maxIters, double eps, double * res)
    {
        linalg::CsrMatrix<double> m;
        m.rows = rows;
        m.cols = rows;
        m.rowStart.assign(rowStart, rowStart + rows + 1);
        const int nnz = rowStart[rows];
        m.column.assign(column, column + nnz);
        m.values.assign(values, values + nnz);
        auto [r0, r1] = linalg::gaussSeidel2ch(m, x, b, maxIters, eps);
        res[0] = r0;
        res[1] = r1;
    }

    // CSR x vector in double accumulation (csrMatrix.cpp:224-238, CsrMatrix<double>::rMultD).
    void ref_rmult_double(int rows, int cols, const int * rowStart, const int * column, const double * values,
                          const double * x, double * y)
    {
        linalg::CsrMatrix<double> m;
        m.rows = rows;
        m.cols = cols;
        m.rowStart.assign(rowStart, rowStart + rows + 1);
        const int nnz = rowStart[rows];
        m.column.assign(column, column + nnz);
        m.values.assign(values, values + nnz);
        m.rMultD(x, y);
    }

    // The reference's assembled FP32 operators (buildChorinCsrMatrices, one thread): which = 0 mass
    // M, 1 stiffness K (both N x N), 2 pressure stiffness Kp (P x P), 3 D = velocityPressureDiv
    // (P x 2N), 4 G = pressureVelocityDiv (2N x P).  dims[0..2] = rows, cols, nnz; the arrays are
    // written when rowStart is non-null.  Returns 0, or -1 with ref_last_error().
    int ref_assembled(void * hv, int which, int * dims, int * rowStart, int * column, float * values)
    {
        try
        {
            auto * h = static_cast<RefMesh *>(hv);
            if (!h->mats)
                h->mats = std::make_unique<fem::ChorinCsrMatrices<float>>(
                    fem::buildChorinCsrMatrices<float>(h->vmesh, h->pmesh, kIntegrationDegree, 1));
            const linalg::CsrMatrix<float> * m = nullptr;
            switch (which)
            {
            case 0: m = &h->mats->velocityMass; break;
            case 1: m = &h->mats->velocityStiffness; break;
            case 2: m = &h->mats->pressureStiffness; break;
            case 3: m = &h->mats->velocityPressureDiv; break;
            case 4: m = &h->mats->pressureVelocityDiv; break;
            default: lastError = "ref_assembled: which must be 0..4"; return -1;
            }
            dims[0] = m->rows;
            dims[1] = m->cols;
            dims[2] = (int)m->column.size();
            if (rowStart)
            {
                std::copy(m->rowStart.begin(), m->rowStart.end(), rowStart);
                std::copy(m->column.begin(), m->column.end(), column);
                std::copy(m->values.begin(), m->values.end(), values);
            }
            return 0;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    // Local matrices of element e from the reference's integrator (degree 4), float, row-major:
    // mass[36], stiff[36] (P2), stiffP[9] (P1), divX/divY[18] (swap = false: rows P1, cols P2),
    // gradX/gradY[18] (swap = true: rows P2, cols P1), conv[12 * 36]: the self-convection matrix for
    // the unit velocity of local DOF k (k < 6: x component of node k, else y of node k - 6), as
    // FastConvection's constructor evaluates it.  Any pointer may be null.
    int ref_local_matrices(void * hv, int e, float * mass, float * stiff, float * stiffP, float * divX, float * divY,
                           float * gradX, float * gradY, float * conv)
    {
        try
        {
            auto * h = static_cast<RefMesh *>(hv);
            const auto & vm = h->vmesh;
            const auto & pm = h->pmesh;
            el::TriangleIntegrator vi(vm.baseElement, kIntegrationDegree, pm.baseElement);
            el::TriangleIntegrator pi(pm.baseElement, kIntegrationDegree);
            const auto & t = vm.elementTransforms[e];
            auto put = [](const cv::Mat & m, float * out) {
                if (!out)
                    return;
                for (int r = 0; r < m.rows; r++)
                    for (int c = 0; c < m.cols; c++)
                        out[r * m.cols + c] = m.at<float>(r, c);
            };
            cv::Mat a, b;
            vi.integrateLocalMassMatrix(t, a);
            put(a, mass);
            vi.integrateLocalStiffnessMatrix(t, a);
            put(a, stiff);
            pi.integrateLocalStiffnessMatrix(t, a);
            put(a, stiffP);
            vi.integrateLocalDivergenceMatrix(t, false, a, b);
            put(a, divX);
            put(b, divY);
            vi.integrateLocalDivergenceMatrix(t, true, a, b);
            put(a, gradX);
            put(b, gradY);
            if (conv)
            {
                std::vector<float> lx(6, 0.0f), ly(6, 0.0f);
                for (int k = 0; k < 12; k++)
                {
                    std::vector<float> & lv = k >= 6 ? ly : lx;
                    lv[k % 6] = 1.0f;
                    vi.integrateLocalSelfConvectionMatrix(t, lx.data(), ly.data(), a);
                    lv[k % 6] = 0.0f;
                    put(a, conv + 36 * k);
                }
            }
            return 0;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    // Values of the FastConvection integration matrix in the layout of ref_prototype(hv, 4):
    // fastConvection.cpp:52-97 with the reference's integrator, contributions summed in FP32 in
    // element order (the order of its triplets).  values[nnz(I)].  Returns 0 or -1.
    int ref_fastconv_values(void * hv, float * values)
    {
        try
        {
            auto * h = static_cast<RefMesh *>(hv);
            const auto & vm = h->vmesh;
            const int N = (int)vm.nodes.size();
            std::unique_ptr<RefCsr> vproto(static_cast<RefCsr *>(ref_prototype(hv, 0)));
            std::unique_ptr<RefCsr> iproto(static_cast<RefCsr *>(ref_prototype(hv, 4)));
            const auto & P = vproto->m;
            const auto & I = iproto->m;
            std::fill(values, values + I.column.size(), 0.0f);
            el::TriangleIntegrator vi(vm.baseElement, kIntegrationDegree, h->pmesh.baseElement);
            std::vector<int> iv(6), offs(6);
            std::vector<float> lx(6, 0.0f), ly(6, 0.0f);
            cv::Mat conv;
            for (int e = 0; e < vm.numElements; e++)
            {
                vm.getElement(e, iv.data(), nullptr);
                int rowIdx[6][6];
                for (int r = 0; r < 6; r++)
                {
                    P.findOffsetsUnsorted(iv[r], iv, offs);
                    for (int c = 0; c < 6; c++)
                        rowIdx[r][c] = offs[c];
                }
                for (int k = 0; k < 12; k++)
                {
                    std::vector<float> & lv = k >= 6 ? ly : lx;
                    lv[k % 6] = 1.0f;
                    vi.integrateLocalSelfConvectionMatrix(vm.elementTransforms[e], lx.data(), ly.data(), conv);
                    lv[k % 6] = 0.0f;
                    const int col = k >= 6 ? iv[k - 6] + N : iv[k];
                    for (int r = 0; r < 6; r++)
                        for (int c = 0; c < 6; c++)
                        {
                            const int row = rowIdx[r][c];
                            const int * b0 = I.column.data() + I.rowStart[row];
                            const int * b1 = I.column.data() + I.rowStart[row + 1];
                            const int * it = std::lower_bound(b0, b1, col);
                            if (it == b1 || *it != col)
                            {
                                lastError = "ref_fastconv_values: entry outside the prototype";
                                return -1;
                            }
                            values[it - I.column.data()] += conv.at<float>(r, c);
                        }
                }
            }
            return 0;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    // Binary interchange files through the reference's linalg::write / readCsr / readVec.  dtype 0
    // float, 1 double; values passed as doubles.  Reading with rowStart == null returns the sizes in
    // dims (rows, cols, nnz) only.  0 on success, -1 with ref_last_error().
    int ref_io_write_csr(const char * path, int dtype, int rows, int cols, int nnz, const int * rs, const int * ci,
                         const double * v)
    {
        try
        {
            return dtype == 0 ? refWriteCsr<float>(path, rows, cols, nnz, rs, ci, v)
                              : refWriteCsr<double>(path, rows, cols, nnz, rs, ci, v);
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    int ref_io_read_csr(const char * path, int dtype, int * dims, int * rs, int * ci, double * v)
    {
        try
        {
            return dtype == 0 ? refReadCsr<float>(path, dims, rs, ci, v) : refReadCsr<double>(path, dims, rs, ci, v);
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    int ref_io_write_vec(const char * path, int dtype, int n, const double * v)
    {
        try
        {
            if (dtype == 0)
                linalg::write(std::string(path), std::vector<float>(v, v + n));
            else
                linalg::write(std::string(path), std::vector<double>(v, v + n));
            return 0;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }

    int ref_io_read_vec(const char * path, int dtype, int * n, double * v)
    {
        try
        {
            if (dtype == 0)
            {
                const auto x = linalg::readVec<float>(std::string(path));
                *n = (int)x.size();
                if (v)
                    std::copy(x.begin(), x.end(), v);
            }
            else
            {
                const auto x = linalg::readVec<double>(std::string(path));
                *n = (int)x.size();
                if (v)
                    std::copy(x.begin(), x.end(), v);
            }
            return 0;
        }
        catch (const std::exception & e)
        {
            lastError = e.what();
            return -1;
        }
    }
}
