// Host-side setup of the Chorin path: mesh input, P1/P2 numbering, channel boundary lists,
// FP64 operator assembly, CSR slicing and the Gauss-Seidel coloring.  Integer results
// (numbering, patterns, lists, coloring) are bit-identical to the reference's; values are FP64.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace nsf
{
    template <typename T>
    struct HostCsr
    {
        int rows = 0, cols = 0;
        std::vector<int> rowStart; // rows + 1
        std::vector<int> col;      // sorted within each row
        std::vector<T> val;

        int nnz() const { return (int)col.size(); }
    };

    // Corner mesh + P2 (velocity) and P1 (pressure) numbering.
    struct Mesh
    {
        // corner mesh (cpp/libs/Mesh/include/mesh/triMesh.h:46-52)
        std::vector<float> cornerXY;      // 2 * V
        std::vector<int> tri;             // 3 * T
        std::vector<int> border;          // 3 * B: triangle, side, group
        std::vector<std::string> groups;
        // P2 / P1 (cpp/libs/Mesh/include/mesh/concreteMesh.h:11-58)
        int N = 0, P = 0;
        std::vector<float> vXY;           // 2 * N
        std::vector<int> vElem;           // 6 * T
        std::vector<int> vBorder;         // 6 * B: triangle, side, group, A, mid, B
        std::vector<int> pElem;           // 3 * T
        std::vector<int> pBorder;         // 5 * B
        std::vector<float> affine;        // 6 * T: m00 m01 m10 m11 b0 b1

        int numTri() const { return (int)tri.size() / 3; }
        int numBorder() const { return (int)border.size() / 3; }
        int groupId(const std::string & name) const;
    };

    // throws std::runtime_error with a message on parse errors
    Mesh loadGmsh(const std::string & path);

    struct Context
    {
        int N = 0, P = 0;
        std::vector<int> dirIds;       // sorted Dirichlet velocity nodes (x and y share ids)
        std::vector<double> dirVx;     // inflow values (float-rounded as the reference computes them)
        std::vector<int> dirPIds;      // Dirichlet pressure nodes (Right border)
        std::vector<int> intV, intP;   // complements
        std::vector<float> pXY;        // 2 * P: pressure node coordinates (the mesh corners)
        HostCsr<double> M, K, Kp, Kpi, D, G, I;
    };

    Context buildChannelContext(const Mesh & mesh, float peakVelocity, int nThreads);
    // the same; values == false: patterns and lists only, every operator value 0 (Kpi and I
    // patterns included)
    Context buildChannelContextEx(const Mesh & mesh, float peakVelocity, int nThreads, bool values);

    // Element-independent reference tensors of the P2/P1 operators on straight triangles (degree-4
    // Cowper rule) that the assembly contracts with each element's adjugate and determinant:
    // mass, the stiffness parts sum w g_i g_j (xx, xy, yy), divergence sum w psi_r g_c (x, y),
    // gradient sum w phi_r dpsi_c (x, y), advection [r][c][k] sum w phi_r phi_k g_c (x, y), and the
    // area-weighted P1 stiffness [i][j][t00 | t01 | t11], all row-major.
    struct AssemblyTables
    {
        double mass[36], sxx[36], sxy[36], syy[36];
        double divX[18], divY[18], grdX[18], grdY[18];
        double advX[216], advY[216];
        double p1stiff[27];
    };
    AssemblyTables assemblyTables();
    // node -> incident elements (ascending); elem holds `per` node ids per element
    void incidenceOf(int nNodes, const std::vector<int> & elem, int per, std::vector<int> & start, std::vector<int> & list);

    HostCsr<double> sliceCsr(const HostCsr<double> & a, const std::vector<int> & rows, const std::vector<int> & cols);

    struct Coloring
    {
        std::vector<int> perm;       // new -> old
        std::vector<int> partStart;  // nColors + 1
        int colors() const { return (int)partStart.size() - 1; }
    };

    Coloring colorGraph(int n, const int * rowStart, const int * col);

    // P A P^T for a symmetric permutation perm (new -> old)
    HostCsr<double> permuteSym(const HostCsr<double> & a, const std::vector<int> & perm);

    // validates a CSR: sizes, rowStart monotone, columns sorted/unique/in range
    bool validCsr(int rows, int cols, int nnz, const int * rowStart, const int * col, std::string & why);

    // Binary CSR / vector files in the reference's interchange format (host/io.cpp); values are
    // widened to double on reading, dtype says what the file held (0 float, 1 double).  Errors throw
    // std::runtime_error (I/O, format) or std::invalid_argument (arguments).
    struct BinCsr
    {
        int dtype = 1;
        HostCsr<double> a;
    };
    struct BinVec
    {
        int dtype = 1;
        std::vector<double> v;
    };
    BinCsr readBinCsr(const std::string & path);
    void writeBinCsr(const std::string & path, int rows, int cols, int nnz, const int * rowStart, const int * col,
                     const double * values, int dtype);
    BinVec readBinVec(const std::string & path);
    void writeBinVec(const std::string & path, int n, const double * values, int dtype);
} // namespace nsf
