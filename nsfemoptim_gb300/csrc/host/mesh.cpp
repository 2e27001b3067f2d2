// gmsh MSH 4.1 ASCII input and P1/P2 numbering.
//
// Format handling follows the reference reader (cpp/libs/Mesh/src/gmsh.cpp:42-499): text is cut
// into $Section ... $EndSection blocks, Nodes/Elements are read block by block, curve entities
// map to physical groups through their first physical tag, ids are sorted and must be
// contiguous (cpp/libs/Mesh/src/io.cpp:65-101).  2-node elements are border edges claimed by the
// triangle side that matches them in the reference's triangleSides order
// (cpp/libs/Mesh/include/mesh/triMesh.h:17-27, io.cpp:175-208).  P2 side nodes are appended
// edge by edge in the order "lowest vertex id, then first appearance of the edge"
// (cpp/libs/Mesh/src/concreteMesh.cpp:97-154) and each element lists c0, m01, c1, m12, c2, m20.
#include "setup.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string_view>

namespace nsf
{
    namespace
    {
        struct Cursor
        {
            const char * p;
            const char * end;

            bool eol() const { return p >= end; }

            void skipSpace()
            {
                while (p < end && (*p == ' ' || *p == '\t' || *p == '\r'))
                    p++;
            }

            bool readLong(long & v)
            {
                skipSpace();
                if (p >= end)
                    return false;
                char * q = nullptr;
                v = std::strtol(p, &q, 10);
                if (q == p)
                    return false;
                p = q;
                return true;
            }

            bool readDouble(double & v)
            {
                skipSpace();
                if (p >= end)
                    return false;
                char * q = nullptr;
                v = std::strtod(p, &q);
                if (q == p)
                    return false;
                p = q;
                return true;
            }

            void skipToken()
            {
                skipSpace();
                while (p < end && *p != ' ' && *p != '\t' && *p != '\r')
                    p++;
            }
        };

        // one section = the list of its non-empty lines
        using Section = std::vector<std::string_view>;

        std::map<std::string, Section> splitSections(const std::string & text)
        {
            std::map<std::string, Section> out;
            Section * cur = nullptr;
            size_t pos = 0;
            while (pos < text.size())
            {
                size_t nl = text.find('\n', pos);
                if (nl == std::string::npos)
                    nl = text.size();
                std::string_view line(text.data() + pos, nl - pos);
                if (!line.empty() && line.back() == '\r')
                    line.remove_suffix(1);
                pos = nl + 1;
                if (line.empty())
                    continue;
                if (line[0] == '$')
                {
                    if (line.substr(0, 4) == "$End")
                        cur = nullptr;
                    else
                        cur = &out[std::string(line.substr(1))];
                    continue;
                }
                if (cur)
                    cur->push_back(line);
            }
            return out;
        }

        Cursor cursor(std::string_view s) { return Cursor{s.data(), s.data() + s.size()}; }

        struct RawNode
        {
            long id;
            double x, y;
        };

        struct RawElem
        {
            long id, entity;
            int n;
            long v[3];
        };

        [[noreturn]] void fail(const std::string & what) { throw std::runtime_error("gmsh: " + what); }
    } // namespace

    int Mesh::groupId(const std::string & name) const
    {
        for (size_t i = 0; i < groups.size(); i++)
            if (groups[i] == name)
                return (int)i;
        return -1;
    }

    Mesh loadGmsh(const std::string & path)
    {
        std::ifstream f(path, std::ios::binary);
        if (!f)
            fail("cannot open " + path);
        std::stringstream ss;
        ss << f.rdbuf();
        const std::string text = ss.str();
        auto sec = splitSections(text);
        for (const char * need : {"Nodes", "Elements", "Entities", "PhysicalNames"})
            if (!sec.count(need))
                fail(std::string("missing section ") + need);

        // ---- nodes
        std::vector<RawNode> nodes;
        {
            const Section & s = sec["Nodes"];
            long h[4];
            auto c = cursor(s.at(0));
            for (long & v : h)
                if (!c.readLong(v))
                    fail("Nodes header");
            nodes.reserve(h[1]);
            size_t li = 1;
            for (long b = 0; b < h[0]; b++)
            {
                long bh[4];
                if (li >= s.size())
                    fail("node block missing");
                auto cb = cursor(s[li++]);
                for (long & v : bh)
                    if (!cb.readLong(v))
                        fail("node block header");
                const long cnt = bh[3];
                if (li + 2 * cnt > s.size())
                    fail("node block truncated");
                const size_t base = nodes.size();
                nodes.resize(base + cnt);
                for (long j = 0; j < cnt; j++)
                {
                    auto ct = cursor(s[li + j]);
                    if (!ct.readLong(nodes[base + j].id))
                        fail("node tag");
                    auto cc = cursor(s[li + cnt + j]);
                    double z;
                    if (!cc.readDouble(nodes[base + j].x) || !cc.readDouble(nodes[base + j].y) || !cc.readDouble(z))
                        fail("node coordinates");
                }
                li += 2 * cnt;
            }
        }

        // ---- elements
        std::vector<RawElem> elems;
        {
            const Section & s = sec["Elements"];
            long h[4];
            auto c = cursor(s.at(0));
            for (long & v : h)
                if (!c.readLong(v))
                    fail("Elements header");
            elems.reserve(h[1]);
            size_t li = 1;
            for (long b = 0; b < h[0]; b++)
            {
                long bh[4];
                if (li >= s.size())
                    fail("element block missing");
                auto cb = cursor(s[li++]);
                for (long & v : bh)
                    if (!cb.readLong(v))
                        fail("element block header");
                const long cnt = bh[3];
                if (li + cnt > s.size())
                    fail("element block truncated");
                for (long j = 0; j < cnt; j++)
                {
                    auto ce = cursor(s[li + j]);
                    RawElem e{};
                    e.entity = bh[1];
                    if (!ce.readLong(e.id))
                        fail("element tag");
                    long v;
                    while (ce.readLong(v))
                    {
                        if (e.n >= 3)
                            fail("element with more than 3 nodes");
                        e.v[e.n++] = v;
                    }
                    elems.push_back(e);
                }
                li += cnt;
            }
        }

        // ---- physical names: `dim tag "name"`
        std::vector<std::pair<long, std::string>> names;
        {
            const Section & s = sec["PhysicalNames"];
            long cnt;
            auto c = cursor(s.at(0));
            if (!c.readLong(cnt))
                fail("PhysicalNames count");
            for (long i = 0; i < cnt; i++)
            {
                std::string_view line = s.at(1 + i);
                auto cl = cursor(line);
                long dim, tag;
                if (!cl.readLong(dim) || !cl.readLong(tag))
                    fail("physical name line");
                size_t q0 = line.find('"'), q1 = line.rfind('"');
                if (q0 == std::string_view::npos || q1 <= q0)
                    fail("physical name quotes");
                names.emplace_back(tag, std::string(line.substr(q0 + 1, q1 - q0 - 1)));
            }
        }

        // ---- curve entity -> first physical tag
        std::map<long, long> curvePhys;
        {
            const Section & s = sec["Entities"];
            long h[4];
            auto c = cursor(s.at(0));
            for (long & v : h)
                if (!c.readLong(v))
                    fail("Entities header");
            for (long i = 0; i < h[1]; i++)
            {
                auto ce = cursor(s.at(1 + h[0] + i));
                long tag, nPhys;
                if (!ce.readLong(tag))
                    fail("curve entity");
                for (int k = 0; k < 6; k++)
                    ce.skipToken();
                if (!ce.readLong(nPhys))
                    fail("curve physical count");
                long first;
                if (nPhys > 0 && ce.readLong(first))
                    curvePhys[tag] = first;
            }
        }

        auto byId = [](const auto & a, const auto & b) { return a.id < b.id; };
        std::sort(nodes.begin(), nodes.end(), byId);
        std::sort(elems.begin(), elems.end(), byId);
        std::sort(names.begin(), names.end(), [](const auto & a, const auto & b) { return a.first < b.first; });
        for (size_t i = 1; i < nodes.size(); i++)
            if (nodes[i].id != nodes[i - 1].id + 1)
                fail("Node IDs are not contiguous");
        for (size_t i = 1; i < elems.size(); i++)
            if (elems[i].id != elems[i - 1].id + 1)
                fail("Element IDs are not contiguous");
        for (size_t i = 1; i < names.size(); i++)
            if (names[i].first != names[i - 1].first + 1)
                fail("Physical group IDs are not contiguous");
        if (nodes.empty() || names.empty())
            fail("empty mesh");

        const long nodeOff = nodes[0].id, groupOff = names[0].first;
        const int V = (int)nodes.size();
        Mesh m;
        m.cornerXY.resize(2 * (size_t)V);
        for (int i = 0; i < V; i++)
        {
            m.cornerXY[2 * i] = (float)nodes[i].x;
            m.cornerXY[2 * i + 1] = (float)nodes[i].y;
        }
        for (auto & nm : names)
            m.groups.push_back(nm.second);

        // directed border edges per source node, in element order
        std::vector<std::vector<std::pair<int, int>>> out(V); // (to, group)
        size_t nEdge = 0;
        for (const auto & e : elems)
        {
            if (e.n == 2)
            {
                const auto it = curvePhys.find(e.entity);
                const int grp = it == curvePhys.end() ? 0 : (int)(it->second - groupOff);
                out[e.v[0] - nodeOff].emplace_back((int)(e.v[1] - nodeOff), grp);
                nEdge++;
            }
            else if (e.n == 3)
            {
                for (int k = 0; k < 3; k++)
                    m.tri.push_back((int)(e.v[k] - nodeOff));
            }
            else
                fail("Not all elements have been parsed");
        }

        static const int sFrom[6] = {0, 1, 1, 2, 2, 0};
        static const int sTo[6] = {1, 0, 2, 1, 0, 2};
        const int T = m.numTri();
        for (int t = 0; t < T; t++)
            for (int s = 0; s < 6; s++)
            {
                const int a = m.tri[3 * t + sFrom[s]], b = m.tri[3 * t + sTo[s]];
                for (const auto & [to, grp] : out[a])
                    if (to == b)
                    {
                        m.border.insert(m.border.end(), {t, s, grp});
                        break;
                    }
            }
        if ((size_t)m.numBorder() != nEdge)
            fail("border edges not matched one-to-one to triangle sides");

        // ---- P2 numbering: edges keyed by their lower vertex, in first-appearance order
        std::vector<std::vector<std::pair<int, int>>> edgesOf(V); // (higher vertex, midpoint id)
        for (int t = 0; t < T; t++)
            for (int a = 0; a < 3; a++)
            {
                const int u = m.tri[3 * t + a], w = m.tri[3 * t + (a + 1) % 3];
                const int lo = std::min(u, w), hi = std::max(u, w);
                auto & l = edgesOf[lo];
                if (std::find_if(l.begin(), l.end(), [hi](const auto & q) { return q.first == hi; }) == l.end())
                    l.emplace_back(hi, -1);
            }
        m.P = V;
        m.vXY = m.cornerXY;
        int next = V;
        for (int v = 0; v < V; v++)
            for (auto & [hi, mid] : edgesOf[v])
            {
                mid = next++;
                // midpoint in float exactly as 0.5f * a + 0.5f * b
                const float ax = 0.5f * m.cornerXY[2 * v], ay = 0.5f * m.cornerXY[2 * v + 1];
                const float bx = 0.5f * m.cornerXY[2 * hi], by = 0.5f * m.cornerXY[2 * hi + 1];
                m.vXY.push_back(ax + bx);
                m.vXY.push_back(ay + by);
            }
        m.N = next;
        auto midOf = [&](int u, int w) -> int
        {
            const int lo = std::min(u, w), hi = std::max(u, w);
            for (const auto & q : edgesOf[lo])
                if (q.first == hi)
                    return q.second;
            return -1;
        };
        m.vElem.resize(6 * (size_t)T);
        m.pElem.resize(3 * (size_t)T);
        m.affine.resize(6 * (size_t)T);
        for (int t = 0; t < T; t++)
        {
            const int * c = &m.tri[3 * t];
            for (int a = 0; a < 3; a++)
            {
                m.vElem[6 * t + 2 * a] = c[a];
                m.vElem[6 * t + 2 * a + 1] = midOf(c[a], c[(a + 1) % 3]);
                m.pElem[3 * t + a] = c[a];
            }
            const float * p0 = &m.cornerXY[2 * c[0]];
            const float * p1 = &m.cornerXY[2 * c[1]];
            const float * p2 = &m.cornerXY[2 * c[2]];
            float * af = &m.affine[6 * t];
            af[0] = p1[0] - p0[0];
            af[1] = p2[0] - p0[0];
            af[2] = p1[1] - p0[1];
            af[3] = p2[1] - p0[1];
            af[4] = p0[0];
            af[5] = p0[1];
        }
        const int B = m.numBorder();
        m.vBorder.resize(6 * (size_t)B);
        m.pBorder.resize(5 * (size_t)B);
        for (int i = 0; i < B; i++)
        {
            const int t = m.border[3 * i], s = m.border[3 * i + 1], g = m.border[3 * i + 2];
            const int a = m.tri[3 * t + sFrom[s]], b = m.tri[3 * t + sTo[s]];
            int * vb = &m.vBorder[6 * i];
            int * pb = &m.pBorder[5 * i];
            vb[0] = pb[0] = t;
            vb[1] = pb[1] = s;
            vb[2] = pb[2] = g;
            vb[3] = pb[3] = a;
            vb[4] = midOf(a, b);
            vb[5] = pb[4] = b;
        }
        return m;
    }
} // namespace nsf
