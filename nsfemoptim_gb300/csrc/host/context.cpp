// Channel-flow context: boundary lists, FP64 operator assembly (threaded, deterministic), the
// internal pressure slice, the FastConvection integration matrix and the GS coloring.
//
// Boundary lists follow buildChorinContext (cpp/execs/NavierStokes/src/buildContext.cpp:64-93)
// with extractDirichletNodes / extractInternalNodes
// (cpp/execs/NavierStokes/include/NavierStokes/borders.h:12-47, src/borders.cpp:19-51) and the
// inflow of DfgConditions (include/NavierStokes/dfgCondtions.h:9-12).
//
// Operators: for straight (affine) triangles every local matrix of the reference integrator
// (cpp/libs/Element/src/triangleIntegrator.cpp:132-293, degree-4 Cowper rule at :27-35) is an
// element-independent reference tensor contracted with the element's adjugate B and det:
//   mass         |det| * sum_q w phi_i phi_j
//   stiffness    1/|det| * sum_q w g_i^T (B^T B) g_j
//   divergence   sgn(det) * (B g_c)_{x|y} * sum_q w psi_r            (D: P1 rows, P2 columns)
//   gradient     sgn(det) * (B g_c)_{x|y} * sum_q w phi_r            (G: P2 rows, P1 columns)
//   advection    sgn(det) * sum_q w phi_r phi_k (B g_c)_{x|y}        (FastConvection, unit u_k)
// The tensors are precomputed once; assembly gathers per CSR row over the incident elements in
// ascending element order, so the sums are deterministic and independent of the thread count.
// Patterns equal the reference's sorted prototypes (cpp/libs/Fem/src/chorinCsr.cpp:142-261,
// cpp/libs/LinAlg/src/sparseDokBuilder.cpp:310-364; fastConvection.cpp:17-80).
#include "setup.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <thread>

namespace nsf
{
    namespace
    {
        // Cowper degree-4 rule on the reference triangle (0,0), (1,0), (0,1); weights sum to 1/2.
        constexpr int NQ = 6;
        constexpr double qa = 9.15762135097710067155318824916321e-02, qb = 8.16847572980457958813360619387822e-01;
        constexpr double qc = 4.45948490915965001235576892213430e-01, qd = 1.08103018168069997528846215573139e-01;
        constexpr double wa = 5.49758718276610602870846378209535e-02, wc = 1.11690794839005624883299105931656e-01;
        constexpr double QP[NQ][3] = {{qa, qa, wa}, {qa, qb, wa}, {qb, qa, wa}, {qc, qc, wc}, {qc, qd, wc}, {qd, qc, wc}};

        // P2 on the reference triangle, nodes c0, m01, c1, m12, c2, m20
        void p2Shape(double x, double y, double * s)
        {
            const double l0 = 1 - x - y;
            s[0] = l0 * (2 * l0 - 1);
            s[1] = 4 * x * l0;
            s[2] = x * (2 * x - 1);
            s[3] = 4 * x * y;
            s[4] = y * (2 * y - 1);
            s[5] = 4 * y * l0;
        }

        void p2Grad(double x, double y, double * gx, double * gy)
        {
            const double l0 = 1 - x - y;
            gx[0] = 1 - 4 * l0;
            gy[0] = 1 - 4 * l0;
            gx[1] = 4 * (l0 - x);
            gy[1] = -4 * x;
            gx[2] = 4 * x - 1;
            gy[2] = 0;
            gx[3] = 4 * y;
            gy[3] = 4 * x;
            gx[4] = 0;
            gy[4] = 4 * y - 1;
            gx[5] = -4 * y;
            gy[5] = 4 * (l0 - y);
        }

        constexpr double P1GX[3] = {-1, 1, 0}, P1GY[3] = {-1, 0, 1};

        struct RefTensors
        {
            double mass[6][6];
            double sxx[6][6], sxy[6][6], syy[6][6]; // sum w g_i g_j per component pair
            double divX[3][6], divY[3][6];           // sum w psi_r g_c
            double grdX[6][3], grdY[6][3];           // sum w phi_r dpsi_c
            double advX[6][6][6], advY[6][6][6];     // [r][c][k] sum w phi_r phi_k g_c
            double p1stiff[3][3][3];                 // [i][j][t00|t01|t11] area-weighted
        };

        RefTensors makeTensors()
        {
            RefTensors T{};
            for (int q = 0; q < NQ; q++)
            {
                const double x = QP[q][0], y = QP[q][1], w = QP[q][2];
                double phi[6], gx[6], gy[6];
                p2Shape(x, y, phi);
                p2Grad(x, y, gx, gy);
                const double psi[3] = {1 - x - y, x, y};
                for (int i = 0; i < 6; i++)
                    for (int j = 0; j < 6; j++)
                    {
                        T.mass[i][j] += w * phi[i] * phi[j];
                        T.sxx[i][j] += w * gx[i] * gx[j];
                        T.sxy[i][j] += w * gx[i] * gy[j];
                        T.syy[i][j] += w * gy[i] * gy[j];
                    }
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 6; c++)
                    {
                        T.divX[r][c] += w * psi[r] * gx[c];
                        T.divY[r][c] += w * psi[r] * gy[c];
                    }
                for (int r = 0; r < 6; r++)
                    for (int c = 0; c < 3; c++)
                    {
                        T.grdX[r][c] += w * phi[r] * P1GX[c];
                        T.grdY[r][c] += w * phi[r] * P1GY[c];
                    }
                for (int r = 0; r < 6; r++)
                    for (int c = 0; c < 6; c++)
                        for (int k = 0; k < 6; k++)
                        {
                            T.advX[r][c][k] += w * phi[r] * phi[k] * gx[c];
                            T.advY[r][c][k] += w * phi[r] * phi[k] * gy[c];
                        }
            }
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                {
                    T.p1stiff[i][j][0] = 0.5 * P1GX[i] * P1GX[j];
                    T.p1stiff[i][j][1] = 0.5 * (P1GX[i] * P1GY[j] + P1GY[i] * P1GX[j]);
                    T.p1stiff[i][j][2] = 0.5 * P1GY[i] * P1GY[j];
                }
            return T;
        }

        struct Geo
        {
            double b00, b01, b10, b11, det, sgn;
        };

        Geo geometry(const float * af)
        {
            // af = m00 m01 m10 m11 (float, as the reference's affine map); B = adj(m)
            const double m00 = af[0], m01 = af[1], m10 = af[2], m11 = af[3];
            Geo g;
            g.b00 = m11;
            g.b01 = -m10;
            g.b10 = -m01;
            g.b11 = m00;
            g.det = m00 * m11 - m10 * m01;
            g.sgn = g.det < 0 ? -1.0 : 1.0;
            return g;
        }

        void parallelFor(int n, int nThreads, const std::function<void(int, int)> & fn)
        {
            nThreads = std::max(1, std::min(nThreads, (n + 1023) / 1024));
            if (nThreads == 1)
            {
                fn(0, n);
                return;
            }
            std::vector<std::thread> th;
            const int chunk = (n + nThreads - 1) / nThreads;
            for (int t = 0; t < nThreads; t++)
            {
                const int a = t * chunk, b = std::min(n, a + chunk);
                if (a < b)
                    th.emplace_back(fn, a, b);
            }
            for (auto & t : th)
                t.join();
        }

        // node -> incident elements (ascending)
        void incidence(int nNodes, const std::vector<int> & elem, int per, std::vector<int> & start, std::vector<int> & list)
        {
            const int T = (int)elem.size() / per;
            start.assign(nNodes + 1, 0);
            for (int v : elem)
                start[v + 1]++;
            for (int i = 0; i < nNodes; i++)
                start[i + 1] += start[i];
            list.resize(elem.size());
            std::vector<int> fill(start.begin(), start.end() - 1);
            for (int t = 0; t < T; t++)
                for (int k = 0; k < per; k++)
                {
                    const int v = elem[(size_t)t * per + k];
                    // an element lists a node once, so each (node, element) pair appears once
                    list[fill[v]++] = t;
                }
        }

        int findCol(const HostCsr<double> & a, int r, int c)
        {
            const auto b = a.col.begin() + a.rowStart[r], e = a.col.begin() + a.rowStart[r + 1];
            auto it = std::lower_bound(b, e, c);
            return (it != e && *it == c) ? (int)(it - a.col.begin()) : -1;
        }

        // rows -> sorted unique column lists built by a callback that appends candidates
        template <typename Gen>
        HostCsr<double> buildPattern(int rows, int cols, int nThreads, Gen gen)
        {
            std::vector<std::vector<int>> rowCols(rows);
            parallelFor(rows, nThreads, [&](int a, int b)
            {
                std::vector<int> tmp;
                for (int r = a; r < b; r++)
                {
                    tmp.clear();
                    gen(r, tmp);
                    std::sort(tmp.begin(), tmp.end());
                    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
                    rowCols[r] = tmp;
                }
            });
            HostCsr<double> out;
            out.rows = rows;
            out.cols = cols;
            out.rowStart.resize(rows + 1);
            out.rowStart[0] = 0;
            for (int r = 0; r < rows; r++)
                out.rowStart[r + 1] = out.rowStart[r] + (int)rowCols[r].size();
            out.col.resize(out.rowStart[rows]);
            for (int r = 0; r < rows; r++)
                std::copy(rowCols[r].begin(), rowCols[r].end(), out.col.begin() + out.rowStart[r]);
            out.val.assign(out.col.size(), 0.0);
            return out;
        }

        float inflow(float peak, float y)
        {
            // the float product, then the remaining factors in double, rounded to float
            const float py = peak * y;
            return (float)((double)py * (0.41 - (double)y) / (0.41 * 0.41));
        }

        struct DNode
        {
            int id;
            float v;
        };

        std::vector<DNode> dirichlet(const Mesh & m, bool p2, const std::vector<int> & groups, int leftGroup, float peak)
        {
            const int per = p2 ? 3 : 2;
            const int stride = p2 ? 6 : 5;
            const auto & bl = p2 ? m.vBorder : m.pBorder;
            const auto & xy = p2 ? m.vXY : m.cornerXY;
            std::vector<char> seen(p2 ? m.N : m.P, 0);
            std::vector<DNode> out;
            for (int i = 0; i < m.numBorder(); i++)
            {
                const int * b = &bl[(size_t)stride * i];
                if (std::find(groups.begin(), groups.end(), b[2]) == groups.end())
                    continue;
                for (int k = 0; k < per; k++)
                {
                    const int id = b[3 + k];
                    if (seen[id])
                        continue;
                    seen[id] = 1;
                    out.push_back({id, b[2] == leftGroup ? inflow(peak, xy[2 * (size_t)id + 1]) : 0.0f});
                }
            }
            std::sort(out.begin(), out.end(), [](const DNode & a, const DNode & b) { return a.id < b.id; });
            return out;
        }

        std::vector<int> complementOf(int n, const std::vector<int> & sortedIds)
        {
            std::vector<int> out;
            out.reserve(n - sortedIds.size());
            size_t j = 0;
            for (int i = 0; i < n; i++)
            {
                while (j < sortedIds.size() && sortedIds[j] < i)
                    j++;
                if (j < sortedIds.size() && sortedIds[j] == i)
                    continue;
                out.push_back(i);
            }
            return out;
        }
    } // namespace

    HostCsr<double> sliceCsr(const HostCsr<double> & a, const std::vector<int> & rows, const std::vector<int> & cols)
    {
        HostCsr<double> out;
        if (rows.empty() || cols.empty())
            return out;
        std::vector<int> map(a.cols, -1);
        for (size_t i = 0; i < cols.size(); i++)
            map.at(cols[i]) = (int)i;
        out.rows = (int)rows.size();
        out.cols = (int)cols.size();
        out.rowStart.push_back(0);
        std::vector<std::pair<int, double>> tmp;
        for (int r : rows)
        {
            tmp.clear();
            for (int j = a.rowStart.at(r); j < a.rowStart[r + 1]; j++)
                if (map[a.col[j]] >= 0)
                    tmp.emplace_back(map[a.col[j]], a.val.empty() ? 0.0 : a.val[j]);
            std::sort(tmp.begin(), tmp.end(), [](const auto & x, const auto & y) { return x.first < y.first; });
            for (auto & [c, v] : tmp)
            {
                out.col.push_back(c);
                out.val.push_back(v);
            }
            out.rowStart.push_back((int)out.col.size());
        }
        return out;
    }

    HostCsr<double> permuteSym(const HostCsr<double> & a, const std::vector<int> & perm)
    {
        return sliceCsr(a, perm, perm);
    }

    Coloring colorGraph(int n, const int * rowStart, const int * col)
    {
        // smallest-last order: repeatedly remove a vertex of least remaining degree; the queue
        // is std::priority_queue with lazy deletion, so ties resolve exactly as in the reference
        struct Item
        {
            int v, deg;
            bool operator<(const Item & o) const { return deg > o.deg; }
        };
        std::vector<int> degree(n);
        std::vector<char> gone(n, 0);
        std::priority_queue<Item> q;
        for (int i = 0; i < n; i++)
        {
            int d = 0;
            for (int j = rowStart[i]; j < rowStart[i + 1]; j++)
                d += col[j] != i;
            degree[i] = d;
            q.push({i, d});
        }
        std::vector<int> order(n);
        for (int k = n - 1; k >= 0; k--)
        {
            int v;
            do
            {
                v = q.top().v;
                q.pop();
            } while (gone[v]);
            order[k] = v;
            gone[v] = 1;
            for (int j = rowStart[v]; j < rowStart[v + 1]; j++)
            {
                const int w = col[j];
                if (w == v || gone[w])
                    continue;
                q.push({w, --degree[w]});
            }
        }
        // greedy first-fit in that order
        std::vector<int> color(n, -1);
        std::vector<char> taken;
        int nColors = 0;
        for (int k = 0; k < n; k++)
        {
            const int v = order[k];
            taken.assign(nColors + 1, 0);
            for (int j = rowStart[v]; j < rowStart[v + 1]; j++)
                if (col[j] != v && color[col[j]] >= 0)
                    taken[color[col[j]]] = 1;
            int c = 0;
            while (taken[c])
                c++;
            color[v] = c;
            nColors = std::max(nColors, c + 1);
        }
        Coloring out;
        out.partStart.assign(nColors + 1, 0);
        for (int v = 0; v < n; v++)
            out.partStart[color[v] + 1]++;
        std::partial_sum(out.partStart.begin(), out.partStart.end(), out.partStart.begin());
        out.perm.resize(n);
        std::vector<int> fill(out.partStart.begin(), out.partStart.end() - 1);
        for (int v = 0; v < n; v++)
            out.perm[fill[color[v]]++] = v;
        return out;
    }

    bool validCsr(int rows, int cols, int nnz, const int * rowStart, const int * col, std::string & why)
    {
        if (rows < 0 || cols < 0 || nnz < 0)
        {
            why = "negative size";
            return false;
        }
        if (!rowStart || (nnz > 0 && !col))
        {
            why = "null array";
            return false;
        }
        if (rowStart[0] != 0 || rowStart[rows] != nnz)
        {
            why = "rowStart must start at 0 and end at nnz";
            return false;
        }
        for (int r = 0; r < rows; r++)
        {
            if (rowStart[r + 1] < rowStart[r])
            {
                why = "rowStart not monotone at row " + std::to_string(r);
                return false;
            }
            for (int j = rowStart[r]; j < rowStart[r + 1]; j++)
            {
                if (col[j] < 0 || col[j] >= cols)
                {
                    why = "column out of range at row " + std::to_string(r);
                    return false;
                }
                if (j > rowStart[r] && col[j] <= col[j - 1])
                {
                    why = "columns not sorted/unique at row " + std::to_string(r);
                    return false;
                }
            }
        }
        return true;
    }

    AssemblyTables assemblyTables()
    {
        static const RefTensors TT = makeTensors();
        AssemblyTables out;
        std::copy(&TT.mass[0][0], &TT.mass[0][0] + 36, out.mass);
        std::copy(&TT.sxx[0][0], &TT.sxx[0][0] + 36, out.sxx);
        std::copy(&TT.sxy[0][0], &TT.sxy[0][0] + 36, out.sxy);
        std::copy(&TT.syy[0][0], &TT.syy[0][0] + 36, out.syy);
        std::copy(&TT.divX[0][0], &TT.divX[0][0] + 18, out.divX);
        std::copy(&TT.divY[0][0], &TT.divY[0][0] + 18, out.divY);
        std::copy(&TT.grdX[0][0], &TT.grdX[0][0] + 18, out.grdX);
        std::copy(&TT.grdY[0][0], &TT.grdY[0][0] + 18, out.grdY);
        std::copy(&TT.advX[0][0][0], &TT.advX[0][0][0] + 216, out.advX);
        std::copy(&TT.advY[0][0][0], &TT.advY[0][0][0] + 216, out.advY);
        std::copy(&TT.p1stiff[0][0][0], &TT.p1stiff[0][0][0] + 27, out.p1stiff);
        return out;
    }

    void incidenceOf(int nNodes, const std::vector<int> & elem, int per, std::vector<int> & start, std::vector<int> & list)
    {
        incidence(nNodes, elem, per, start, list);
    }

    Context buildChannelContext(const Mesh & m, float peakVelocity, int nThreads)
    {
        return buildChannelContextEx(m, peakVelocity, nThreads, true);
    }

    Context buildChannelContextEx(const Mesh & m, float peakVelocity, int nThreads, bool values)
    {
        if (nThreads <= 0)
            nThreads = (int)std::max(1u, std::thread::hardware_concurrency());
        const int left = m.groupId("Left"), right = m.groupId("Right"), top = m.groupId("Top"),
                  bottom = m.groupId("Bottom"), circle = m.groupId("Circle");
        if (left < 0 || right < 0 || top < 0 || bottom < 0 || circle < 0)
            throw std::invalid_argument("channel mesh needs Left/Right/Top/Bottom/Circle border groups");

        Context c;
        c.N = m.N;
        c.P = m.P;
        const int N = m.N, P = m.P, T = m.numTri();
        auto dv = dirichlet(m, true, {left, top, bottom, circle}, left, peakVelocity);
        for (auto & d : dv)
        {
            c.dirIds.push_back(d.id);
            c.dirVx.push_back((double)d.v);
        }
        for (auto & d : dirichlet(m, false, {right}, -1, 0.0f))
            c.dirPIds.push_back(d.id);
        c.intV = complementOf(N, c.dirIds);
        c.intP = complementOf(P, c.dirPIds);
        // pressure node coordinates: the P1 nodes are the mesh corners (pElem holds corner ids)
        if (m.cornerXY.size() == 2 * (size_t)P)
            c.pXY = m.cornerXY;

        // incidence lists
        std::vector<int> vStart, vList, pStart, pList;
        incidence(N, m.vElem, 6, vStart, vList);
        incidence(P, m.pElem, 3, pStart, pList);

        // ---- patterns
        c.M = buildPattern(N, N, nThreads, [&](int r, std::vector<int> & out)
        {
            for (int k = vStart[r]; k < vStart[r + 1]; k++)
                out.insert(out.end(), &m.vElem[6 * (size_t)vList[k]], &m.vElem[6 * (size_t)vList[k]] + 6);
        });
        c.K = c.M;
        c.Kp = buildPattern(P, P, nThreads, [&](int r, std::vector<int> & out)
        {
            for (int k = pStart[r]; k < pStart[r + 1]; k++)
                out.insert(out.end(), &m.pElem[3 * (size_t)pList[k]], &m.pElem[3 * (size_t)pList[k]] + 3);
        });
        c.D = buildPattern(P, 2 * N, nThreads, [&](int r, std::vector<int> & out)
        {
            for (int k = pStart[r]; k < pStart[r + 1]; k++)
                for (int a = 0; a < 6; a++)
                {
                    const int v = m.vElem[6 * (size_t)pList[k] + a];
                    out.push_back(v);
                    out.push_back(v + N);
                }
        });
        c.G = buildPattern(2 * N, P, nThreads, [&](int r, std::vector<int> & out)
        {
            const int v = r < N ? r : r - N;
            for (int k = vStart[v]; k < vStart[v + 1]; k++)
                out.insert(out.end(), &m.pElem[3 * (size_t)vList[k]], &m.pElem[3 * (size_t)vList[k]] + 3);
        });

        // ---- values: gather per row over incident elements in ascending element order
        static const RefTensors TT = makeTensors();
        if (!values)
        {
            // patterns only (the values are assembled elsewhere, e.g. on the device)
            c.Kpi = sliceCsr(c.Kp, c.intP, c.intP);
            const int nnzK = c.K.nnz();
            std::vector<int> entryRow(nnzK);
            for (int r = 0; r < N; r++)
                for (int e = c.K.rowStart[r]; e < c.K.rowStart[r + 1]; e++)
                    entryRow[e] = r;
            c.I = buildPattern(nnzK, 2 * N, nThreads, [&](int e, std::vector<int> & out)
            {
                const int r = entryRow[e], cc = c.K.col[e];
                for (int k = vStart[r]; k < vStart[r + 1]; k++)
                {
                    const int * ids = &m.vElem[6 * (size_t)vList[k]];
                    bool has = false;
                    for (int q = 0; q < 6; q++)
                        has |= ids[q] == cc;
                    if (!has)
                        continue;
                    for (int q = 0; q < 6; q++)
                    {
                        out.push_back(ids[q]);
                        out.push_back(ids[q] + N);
                    }
                }
            });
            return c;
        }
        std::vector<Geo> geo(T);
        parallelFor(T, nThreads, [&](int a, int b)
        {
            for (int t = a; t < b; t++)
                geo[t] = geometry(&m.affine[6 * (size_t)t]);
        });
        auto localIndex = [](const int * ids, int n, int v) -> int
        {
            for (int i = 0; i < n; i++)
                if (ids[i] == v)
                    return i;
            return -1;
        };

        parallelFor(N, nThreads, [&](int a, int b)
        {
            for (int r = a; r < b; r++)
                for (int k = vStart[r]; k < vStart[r + 1]; k++)
                {
                    const int t = vList[k];
                    const int * ids = &m.vElem[6 * (size_t)t];
                    const Geo & g = geo[t];
                    const int i = localIndex(ids, 6, r);
                    const double ad = std::fabs(g.det);
                    const double t00 = g.b00 * g.b00 + g.b10 * g.b10;
                    const double t01 = g.b00 * g.b01 + g.b10 * g.b11;
                    const double t11 = g.b01 * g.b01 + g.b11 * g.b11;
                    for (int j = 0; j < 6; j++)
                    {
                        const int e = findCol(c.M, r, ids[j]);
                        c.M.val[e] += ad * TT.mass[i][j];
                        c.K.val[e] += (t00 * TT.sxx[i][j] + t01 * (TT.sxy[i][j] + TT.sxy[j][i]) + t11 * TT.syy[i][j]) / ad;
                    }
                    // gradient rows r (x) and r + N (y)
                    const int * pid = &m.pElem[3 * (size_t)t];
                    for (int q = 0; q < 3; q++)
                    {
                        const double gx = g.sgn * (g.b00 * TT.grdX[i][q] + g.b01 * TT.grdY[i][q]);
                        const double gy = g.sgn * (g.b10 * TT.grdX[i][q] + g.b11 * TT.grdY[i][q]);
                        c.G.val[findCol(c.G, r, pid[q])] += gx;
                        c.G.val[findCol(c.G, r + N, pid[q])] += gy;
                    }
                }
        });
        parallelFor(P, nThreads, [&](int a, int b)
        {
            for (int r = a; r < b; r++)
                for (int k = pStart[r]; k < pStart[r + 1]; k++)
                {
                    const int t = pList[k];
                    const int * pid = &m.pElem[3 * (size_t)t];
                    const int * vid = &m.vElem[6 * (size_t)t];
                    const Geo & g = geo[t];
                    const int i = localIndex(pid, 3, r);
                    const double ad = std::fabs(g.det);
                    const double t00 = g.b00 * g.b00 + g.b10 * g.b10;
                    const double t01 = g.b00 * g.b01 + g.b10 * g.b11;
                    const double t11 = g.b01 * g.b01 + g.b11 * g.b11;
                    for (int j = 0; j < 3; j++)
                        c.Kp.val[findCol(c.Kp, r, pid[j])] +=
                            (t00 * TT.p1stiff[i][j][0] + t01 * TT.p1stiff[i][j][1] + t11 * TT.p1stiff[i][j][2]) / ad;
                    for (int a2 = 0; a2 < 6; a2++)
                    {
                        const double dx = g.sgn * (g.b00 * TT.divX[i][a2] + g.b01 * TT.divY[i][a2]);
                        const double dy = g.sgn * (g.b10 * TT.divX[i][a2] + g.b11 * TT.divY[i][a2]);
                        c.D.val[findCol(c.D, r, vid[a2])] += dx;
                        c.D.val[findCol(c.D, r, vid[a2] + N)] += dy;
                    }
                }
        });
        c.Kpi = sliceCsr(c.Kp, c.intP, c.intP);

        // ---- FastConvection integration matrix: one row per K entry (i, j)
        const int nnzK = c.K.nnz();
        std::vector<int> entryRow(nnzK);
        for (int r = 0; r < N; r++)
            for (int e = c.K.rowStart[r]; e < c.K.rowStart[r + 1]; e++)
                entryRow[e] = r;
        c.I = buildPattern(nnzK, 2 * N, nThreads, [&](int e, std::vector<int> & out)
        {
            const int r = entryRow[e], cc = c.K.col[e];
            for (int k = vStart[r]; k < vStart[r + 1]; k++)
            {
                const int * ids = &m.vElem[6 * (size_t)vList[k]];
                bool has = false;
                for (int q = 0; q < 6; q++)
                    has |= ids[q] == cc;
                if (!has)
                    continue;
                for (int q = 0; q < 6; q++)
                {
                    out.push_back(ids[q]);
                    out.push_back(ids[q] + N);
                }
            }
        });
        parallelFor(nnzK, nThreads, [&](int a, int b)
        {
            for (int e = a; e < b; e++)
            {
                const int r = entryRow[e], cc = c.K.col[e];
                for (int k = vStart[r]; k < vStart[r + 1]; k++)
                {
                    const int t = vList[k];
                    const int * ids = &m.vElem[6 * (size_t)t];
                    const int jl = localIndex(ids, 6, cc);
                    if (jl < 0)
                        continue;
                    const int il = localIndex(ids, 6, r);
                    const Geo & g = geo[t];
                    for (int q = 0; q < 6; q++)
                    {
                        const double vx = g.sgn * (g.b00 * TT.advX[il][jl][q] + g.b01 * TT.advY[il][jl][q]);
                        const double vy = g.sgn * (g.b10 * TT.advX[il][jl][q] + g.b11 * TT.advY[il][jl][q]);
                        c.I.val[findCol(c.I, e, ids[q])] += vx;
                        c.I.val[findCol(c.I, e, ids[q] + N)] += vy;
                    }
                }
            }
        });
        return c;
    }
} // namespace nsf
