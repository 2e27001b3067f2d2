#define _POSIX_C_SOURCE 200809L
/*
 * Oracle, mesh part: gmsh MSH 4.1 ASCII reader, corner-mesh construction, P1/P2 numbering and
 * the channel problem's Dirichlet/internal node lists.  Test infrastructure only.
 *
 * Follows:
 *   section split and Nodes/Elements/Entities/PhysicalNames parsing   cpp/libs/Mesh/src/gmsh.cpp:42-499
 *   id sort, border-edge claiming in triangleSides order             cpp/libs/Mesh/src/io.cpp:65-208
 *   triangleSides                                                    cpp/libs/Mesh/include/mesh/triMesh.h:17-27
 *   P2 side-node creation order and element node order              cpp/libs/Mesh/src/concreteMesh.cpp:78-293
 *   affine map from the reference triangle                           cpp/libs/Element/src/affineTransform.cpp:19-36
 *   Dirichlet lists / internal nodes                                 cpp/execs/NavierStokes/include/NavierStokes/borders.h:12-47,
 *                                                                    cpp/execs/NavierStokes/src/borders.cpp:19-51
 *   inflow profile                                                   cpp/execs/NavierStokes/include/NavierStokes/dfgCondtions.h:9-12
 */
#include "oracle.h"

#include <ctype.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static char g_err[512];

const char *orc_last_error(void) { return g_err; }

static void set_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

/* ------------------------------------------------------------------ text sections */

typedef struct
{
    char **lines;
    int n, cap;
} linelist;

typedef struct
{
    char *name;
    linelist body;
} section;

static void ll_push(linelist *l, char *s)
{
    if (l->n == l->cap)
    {
        l->cap = l->cap ? 2 * l->cap : 64;
        l->lines = (char **)realloc(l->lines, sizeof(char *) * l->cap);
    }
    l->lines[l->n++] = s;
}

typedef struct
{
    section *s;
    int n;
} sections;

static linelist *find_section(sections *ss, const char *name)
{
    for (int i = 0; i < ss->n; i++)
        if (strcmp(ss->s[i].name, name) == 0)
            return &ss->s[i].body;
    return NULL;
}

/* Lines starting with '$' switch sections ("$End..." returns to the unnamed one); empty lines
   are skipped; repeated section names append to the same section (gmsh.cpp:42-99). */
static void split_sections(char *text, sections *ss)
{
    ss->n = 1;
    ss->s = (section *)calloc(1, sizeof(section));
    ss->s[0].name = strdup("");
    int cur = 0;
    char *p = text;
    while (*p)
    {
        char *e = strchr(p, '\n');
        if (e)
            *e = 0;
        size_t len = strlen(p);
        if (len && p[len - 1] == '\r')
            p[--len] = 0;
        if (len > 0)
        {
            if (p[0] == '$')
            {
                if (strncmp(p, "$End", 4) == 0)
                    cur = 0;
                else
                {
                    int found = -1;
                    for (int i = 0; i < ss->n; i++)
                        if (strcmp(ss->s[i].name, p + 1) == 0)
                            found = i;
                    if (found < 0)
                    {
                        ss->s = (section *)realloc(ss->s, sizeof(section) * (ss->n + 1));
                        memset(&ss->s[ss->n], 0, sizeof(section));
                        ss->s[ss->n].name = strdup(p + 1);
                        found = ss->n++;
                    }
                    cur = found;
                }
            }
            else
                ll_push(&ss->s[cur].body, p);
        }
        if (!e)
            break;
        p = e + 1;
    }
}

static void free_sections(sections *ss)
{
    for (int i = 0; i < ss->n; i++)
    {
        free(ss->s[i].name);
        free(ss->s[i].body.lines);
    }
    free(ss->s);
}

/* parse up to max integers from a line; returns the count */
static int parse_ints(const char *s, long *out, int max)
{
    int n = 0;
    char *end;
    while (n < max)
    {
        while (*s && isspace((unsigned char)*s))
            s++;
        if (!*s)
            break;
        long v = strtol(s, &end, 10);
        if (end == s)
            break;
        out[n++] = v;
        s = end;
    }
    return n;
}

static int parse_doubles(const char *s, double *out, int max)
{
    int n = 0;
    char *end;
    while (n < max)
    {
        double v = strtod(s, &end);
        if (end == s)
            break;
        out[n++] = v;
        s = end;
    }
    return n;
}

typedef struct
{
    long id;
    double x, y;
} pnode;

typedef struct
{
    long id;
    long entity;
    int npts;
    long pts[4];
} pelem;

typedef struct
{
    long id;
    char name[128];
} pname;

static int cmp_pnode(const void *a, const void *b)
{
    long x = ((const pnode *)a)->id, y = ((const pnode *)b)->id;
    return (x > y) - (x < y);
}
static int cmp_pelem(const void *a, const void *b)
{
    long x = ((const pelem *)a)->id, y = ((const pelem *)b)->id;
    return (x > y) - (x < y);
}
static int cmp_pname(const void *a, const void *b)
{
    long x = ((const pname *)a)->id, y = ((const pname *)b)->id;
    return (x > y) - (x < y);
}

/* ------------------------------------------------------------------ numbering helpers */

typedef struct
{
    int to;
    int extra; /* id of the side's midpoint node */
} side_t;

typedef struct
{
    side_t *s;
    int n, cap;
} sidelist;

static void side_add(sidelist *g, int a, int b)
{
    int from = a < b ? a : b, to = a < b ? b : a;
    sidelist *l = &g[from];
    for (int i = 0; i < l->n; i++)
        if (l->s[i].to == to)
            return;
    if (l->n == l->cap)
    {
        l->cap = l->cap ? 2 * l->cap : 4;
        l->s = (side_t *)realloc(l->s, sizeof(side_t) * l->cap);
    }
    l->s[l->n].to = to;
    l->s[l->n].extra = -1;
    l->n++;
}

static int side_extra(const sidelist *g, int a, int b)
{
    int from = a < b ? a : b, to = a < b ? b : a;
    const sidelist *l = &g[from];
    for (int i = 0; i < l->n; i++)
        if (l->s[i].to == to)
            return l->s[i].extra;
    return -1;
}

/* ------------------------------------------------------------------ loader */

orc_mesh *orc_mesh_load(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f)
    {
        set_err("cannot open mesh file %s", path);
        return NULL;
    }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *text = (char *)malloc(sz + 1);
    if (fread(text, 1, sz, f) != (size_t)sz)
    {
        fclose(f);
        free(text);
        set_err("read failed");
        return NULL;
    }
    text[sz] = 0;
    fclose(f);

    sections ss;
    split_sections(text, &ss);
    linelist *nodesS = find_section(&ss, "Nodes");
    linelist *elemS = find_section(&ss, "Elements");
    linelist *entS = find_section(&ss, "Entities");
    linelist *physS = find_section(&ss, "PhysicalNames");
    orc_mesh *m = NULL;
    pnode *nodes = NULL;
    pelem *elems = NULL;
    pname *names = NULL;
    long *curveTag = NULL, *curveGroup = NULL;
    int nCurves = 0;
    if (!nodesS || !elemS || !entS || !physS)
    {
        set_err("missing section (need Nodes, Elements, Entities, PhysicalNames)");
        goto fail;
    }

    /* ---- Nodes: numBlocks numNodes minTag maxTag; blocks of tags then coordinates */
    long hdr[4];
    int li = 0;
    if (nodesS->n < 1 || parse_ints(nodesS->lines[0], hdr, 4) != 4)
    {
        set_err("bad Nodes header");
        goto fail;
    }
    li = 1;
    long numNodes = hdr[1];
    nodes = (pnode *)malloc(sizeof(pnode) * (numNodes > 0 ? numNodes : 1));
    long nn = 0;
    for (long b = 0; b < hdr[0]; b++)
    {
        long bh[4];
        if (li >= nodesS->n || parse_ints(nodesS->lines[li++], bh, 4) != 4)
        {
            set_err("bad node block header");
            goto fail;
        }
        long cnt = bh[3];
        if (nn + cnt > numNodes || li + 2 * cnt > nodesS->n)
        {
            set_err("node block overflow");
            goto fail;
        }
        for (long j = 0; j < cnt; j++)
            parse_ints(nodesS->lines[li + j], &nodes[nn + j].id, 1);
        for (long j = 0; j < cnt; j++)
        {
            double xyz[3] = {0, 0, 0};
            parse_doubles(nodesS->lines[li + cnt + j], xyz, 3);
            nodes[nn + j].x = xyz[0];
            nodes[nn + j].y = xyz[1];
        }
        li += 2 * cnt;
        nn += cnt;
    }

    /* ---- Elements */
    if (elemS->n < 1 || parse_ints(elemS->lines[0], hdr, 4) != 4)
    {
        set_err("bad Elements header");
        goto fail;
    }
    long numElems = hdr[1];
    elems = (pelem *)malloc(sizeof(pelem) * (numElems > 0 ? numElems : 1));
    long ne = 0;
    li = 1;
    for (long b = 0; b < hdr[0]; b++)
    {
        long bh[4];
        if (li >= elemS->n || parse_ints(elemS->lines[li++], bh, 4) != 4)
        {
            set_err("bad element block header");
            goto fail;
        }
        long cnt = bh[3];
        if (ne + cnt > numElems || li + cnt > elemS->n)
        {
            set_err("element block overflow");
            goto fail;
        }
        for (long j = 0; j < cnt; j++)
        {
            long v[6];
            int k = parse_ints(elemS->lines[li + j], v, 6);
            if (k < 2 || k > 5)
            {
                set_err("unsupported element line");
                goto fail;
            }
            elems[ne + j].id = v[0];
            elems[ne + j].entity = bh[1];
            elems[ne + j].npts = k - 1;
            for (int q = 1; q < k; q++)
                elems[ne + j].pts[q - 1] = v[q];
        }
        li += cnt;
        ne += cnt;
    }

    /* ---- PhysicalNames: count, then `dim tag "name"` */
    long np_ = 0;
    if (physS->n < 1 || parse_ints(physS->lines[0], &np_, 1) != 1)
    {
        set_err("bad PhysicalNames");
        goto fail;
    }
    names = (pname *)calloc(np_ > 0 ? np_ : 1, sizeof(pname));
    for (long i = 0; i < np_; i++)
    {
        long dt[2];
        const char *ln = physS->lines[1 + i];
        if (parse_ints(ln, dt, 2) != 2)
        {
            set_err("bad physical name line");
            goto fail;
        }
        names[i].id = dt[1];
        const char *q = strchr(ln, '"');
        const char *q2 = q ? strchr(q + 1, '"') : NULL;
        if (!q || !q2 || q2 - q - 1 >= 127)
        {
            set_err("bad physical name");
            goto fail;
        }
        memcpy(names[i].name, q + 1, q2 - q - 1);
        names[i].name[q2 - q - 1] = 0;
    }

    /* ---- Entities: curves' first physical tag (only curves map to border groups, io.cpp:103-108) */
    long eh[4];
    if (entS->n < 1 || parse_ints(entS->lines[0], eh, 4) != 4)
    {
        set_err("bad Entities header");
        goto fail;
    }
    nCurves = (int)eh[1];
    curveTag = (long *)calloc(nCurves > 0 ? nCurves : 1, sizeof(long));
    curveGroup = (long *)calloc(nCurves > 0 ? nCurves : 1, sizeof(long));
    for (int i = 0; i < nCurves; i++)
    {
        const char *ln = entS->lines[1 + eh[0] + i];
        char *end;
        long tag = strtol(ln, &end, 10);
        double bb[6];
        if (parse_doubles(end, bb, 6) != 6)
        {
            set_err("bad curve entity");
            goto fail;
        }
        /* skip tag and 6 doubles, then numPhysicalTags and tags */
        const char *s = ln;
        for (int k = 0; k < 7; k++)
        {
            while (*s && isspace((unsigned char)*s))
                s++;
            while (*s && !isspace((unsigned char)*s))
                s++;
        }
        long v[2];
        int k = parse_ints(s, v, 2);
        curveTag[i] = tag;
        curveGroup[i] = (k >= 2 && v[0] > 0) ? v[1] : -1; /* -1: no physical tag */
    }

    /* ---- sort by id and check contiguity (io.cpp:67-86) */
    qsort(nodes, nn, sizeof(pnode), cmp_pnode);
    qsort(elems, ne, sizeof(pelem), cmp_pelem);
    qsort(names, np_, sizeof(pname), cmp_pname);
    for (long i = 1; i < nn; i++)
        if (nodes[i].id != nodes[i - 1].id + 1)
        {
            set_err("Node IDs are not contiguous");
            goto fail;
        }
    for (long i = 1; i < ne; i++)
        if (elems[i].id != elems[i - 1].id + 1)
        {
            set_err("Element IDs are not contiguous");
            goto fail;
        }
    for (long i = 1; i < np_; i++)
        if (names[i].id != names[i - 1].id + 1)
        {
            set_err("Physical group IDs are not contiguous");
            goto fail;
        }
    long nodeOff = nodes[0].id, groupOff = names[0].id;

    m = (orc_mesh *)calloc(1, sizeof(orc_mesh));
    m->numCorner = (int)nn;
    m->cornerXY = (float *)malloc(sizeof(float) * 2 * nn);
    for (long i = 0; i < nn; i++)
    {
        m->cornerXY[2 * i] = (float)nodes[i].x;
        m->cornerXY[2 * i + 1] = (float)nodes[i].y;
    }
    m->numGroups = (int)np_;
    m->groups = (char **)malloc(sizeof(char *) * np_);
    for (long i = 0; i < np_; i++)
        m->groups[names[i].id - groupOff] = strdup(names[i].name);

    /* border edges as a per-node adjacency list in element-id order (io.cpp:119-140) */
    int *edgeHead = (int *)malloc(sizeof(int) * nn);
    for (long i = 0; i < nn; i++)
        edgeHead[i] = -1;
    int *edgeTo = (int *)malloc(sizeof(int) * (ne + 1));
    int *edgeGroup = (int *)malloc(sizeof(int) * (ne + 1));
    int *edgeNext = (int *)malloc(sizeof(int) * (ne + 1));
    int *edgeTail = (int *)malloc(sizeof(int) * nn);
    int nEdges = 0, nTri = 0;
    for (long i = 0; i < ne; i++)
    {
        if (elems[i].npts == 2)
        {
            int from = (int)(elems[i].pts[0] - nodeOff), to = (int)(elems[i].pts[1] - nodeOff);
            int grp = 0; /* std::map operator[] default for an entity without a physical tag */
            for (int c = 0; c < nCurves; c++)
                if (curveTag[c] == elems[i].entity)
                    grp = curveGroup[c] >= 0 ? (int)(curveGroup[c] - groupOff) : 0;
            edgeTo[nEdges] = to;
            edgeGroup[nEdges] = grp;
            edgeNext[nEdges] = -1;
            if (edgeHead[from] < 0)
                edgeHead[from] = nEdges;
            else
                edgeNext[edgeTail[from]] = nEdges;
            edgeTail[from] = nEdges;
            nEdges++;
        }
        else if (elems[i].npts == 3)
            nTri++;
    }
    if (nEdges + nTri != ne)
    {
        free(edgeHead);
        free(edgeTo);
        free(edgeGroup);
        free(edgeNext);
        free(edgeTail);
        set_err("Not all elements have been parsed");
        goto fail;
    }
    m->numTri = nTri;
    m->tri = (int *)malloc(sizeof(int) * 3 * nTri);
    int t = 0;
    for (long i = 0; i < ne; i++)
        if (elems[i].npts == 3)
        {
            for (int k = 0; k < 3; k++)
                m->tri[3 * t + k] = (int)(elems[i].pts[k] - nodeOff);
            t++;
        }

    /* claim border edges per triangle side in triangleSides order */
    static const int sidesFrom[6] = {0, 1, 1, 2, 2, 0};
    static const int sidesTo[6] = {1, 0, 2, 1, 0, 2};
    m->border = (int *)malloc(sizeof(int) * 3 * (nEdges + 1));
    int nb = 0;
    for (int i = 0; i < nTri; i++)
    {
        const int *pts = m->tri + 3 * i;
        for (int s = 0; s < 6; s++)
        {
            int from = pts[sidesFrom[s]], to = pts[sidesTo[s]];
            for (int e = edgeHead[from]; e >= 0; e = edgeNext[e])
                if (edgeTo[e] == to)
                {
                    if (nb < nEdges)
                    {
                        m->border[3 * nb] = i;
                        m->border[3 * nb + 1] = s;
                        m->border[3 * nb + 2] = edgeGroup[e];
                    }
                    nb++;
                    break;
                }
        }
    }
    free(edgeHead);
    free(edgeTo);
    free(edgeGroup);
    free(edgeNext);
    free(edgeTail);
    if (nb > nEdges)
    {
        set_err("border edge claimed twice");
        goto fail;
    }
    m->numBorder = nb;

    /* ---- P2 numbering (concreteMesh.cpp:78-255): sides in first-seen order per min vertex,
       midpoints appended looping over the min vertex id */
    {
        int V = m->numCorner;
        sidelist *g = (sidelist *)calloc(V, sizeof(sidelist));
        for (int i = 0; i < nTri; i++)
            for (int a = 0; a < 3; a++)
                side_add(g, m->tri[3 * i + a], m->tri[3 * i + (a + 1) % 3]);
        int nSides = 0;
        for (int v = 0; v < V; v++)
            nSides += g[v].n;
        m->numV = V + nSides;
        m->numP = V;
        m->vXY = (float *)malloc(sizeof(float) * 2 * m->numV);
        memcpy(m->vXY, m->cornerXY, sizeof(float) * 2 * V);
        int next = V;
        const float w = 0.5f, cw = 1.0f - 0.5f;
        for (int v = 0; v < V; v++)
            for (int k = 0; k < g[v].n; k++)
            {
                side_t *s = &g[v].s[k];
                const float *fa = m->cornerXY + 2 * v, *fb = m->cornerXY + 2 * s->to;
                volatile float mx = cw * fa[0];
                volatile float my = cw * fa[1];
                volatile float tx = w * fb[0];
                volatile float ty = w * fb[1];
                s->extra = next;
                m->vXY[2 * next] = mx + tx;
                m->vXY[2 * next + 1] = my + ty;
                next++;
            }
        m->vElem = (int *)malloc(sizeof(int) * 6 * nTri);
        m->pElem = (int *)malloc(sizeof(int) * 3 * nTri);
        m->affine = (float *)malloc(sizeof(float) * 6 * nTri);
        for (int i = 0; i < nTri; i++)
        {
            const int *c = m->tri + 3 * i;
            int *e = m->vElem + 6 * i;
            for (int a = 0; a < 3; a++)
            {
                e[2 * a] = c[a];
                e[2 * a + 1] = side_extra(g, c[a], c[(a + 1) % 3]);
                m->pElem[3 * i + a] = c[a];
            }
            const float *p0 = m->cornerXY + 2 * c[0], *p1 = m->cornerXY + 2 * c[1], *p2 = m->cornerXY + 2 * c[2];
            float *af = m->affine + 6 * i;
            af[0] = p1[0] - p0[0];
            af[1] = p2[0] - p0[0];
            af[2] = p1[1] - p0[1];
            af[3] = p2[1] - p0[1];
            af[4] = p0[0];
            af[5] = p0[1];
        }
        /* border elements (concreteMesh.cpp:258-285): P2 as A, mid, B; P1 as A, B */
        m->vBorder = (int *)malloc(sizeof(int) * 6 * (nb + 1));
        m->pBorder = (int *)malloc(sizeof(int) * 5 * (nb + 1));
        for (int i = 0; i < nb; i++)
        {
            int tri = m->border[3 * i], s = m->border[3 * i + 1], grp = m->border[3 * i + 2];
            int A = m->tri[3 * tri + sidesFrom[s]], B = m->tri[3 * tri + sidesTo[s]];
            int *vb = m->vBorder + 6 * i, *pb = m->pBorder + 5 * i;
            vb[0] = pb[0] = tri;
            vb[1] = pb[1] = s;
            vb[2] = pb[2] = grp;
            vb[3] = A;
            vb[4] = side_extra(g, A, B);
            vb[5] = B;
            pb[3] = A;
            pb[4] = B;
        }
        for (int v = 0; v < V; v++)
            free(g[v].s);
        free(g);
    }

    free_sections(&ss);
    free(text);
    free(nodes);
    free(elems);
    free(names);
    free(curveTag);
    free(curveGroup);
    return m;

fail:
    free_sections(&ss);
    free(text);
    free(nodes);
    free(elems);
    free(names);
    free(curveTag);
    free(curveGroup);
    orc_mesh_free(m);
    return NULL;
}

void orc_mesh_free(orc_mesh *m)
{
    if (!m)
        return;
    free(m->cornerXY);
    free(m->tri);
    free(m->border);
    if (m->groups)
        for (int i = 0; i < m->numGroups; i++)
            free(m->groups[i]);
    free(m->groups);
    free(m->vXY);
    free(m->vElem);
    free(m->vBorder);
    free(m->pElem);
    free(m->pBorder);
    free(m->affine);
    free(m);
}

int orc_group_id(const orc_mesh *m, const char *name)
{
    for (int i = 0; i < m->numGroups; i++)
        if (m->groups[i] && strcmp(m->groups[i], name) == 0)
            return i;
    return -1;
}

/* ------------------------------------------------------------------ Dirichlet lists */

/* u = peak * y * (0.41 - y) / 0.41^2 evaluated as the reference does: the float product
   peak*y, then the remaining factors in double, rounded to float on return. */
static float inflow(float peak, float y)
{
    volatile float py = peak * y;
    double v = (double)py * (0.41 - (double)y) / (0.41 * 0.41);
    return (float)v;
}

typedef struct
{
    int id;
    float v;
} dnode;

static int cmp_dnode(const void *a, const void *b)
{
    int x = ((const dnode *)a)->id, y = ((const dnode *)b)->id;
    return (x > y) - (x < y);
}

/* border elements in order, first sight of a node decides its value, then sort by id */
static int extract_dirichlet(const orc_mesh *m, int p2, const int *groups, int nGroups, int leftGroup,
                             float peak, dnode **out)
{
    int nNodes = p2 ? m->numV : m->numP;
    int per = p2 ? 3 : 2;
    char *seen = (char *)calloc(nNodes, 1);
    dnode *r = (dnode *)malloc(sizeof(dnode) * (per * m->numBorder + 1));
    int n = 0;
    for (int i = 0; i < m->numBorder; i++)
    {
        const int *b = p2 ? m->vBorder + 6 * i : m->pBorder + 5 * i;
        int grp = b[2], hit = 0;
        for (int k = 0; k < nGroups; k++)
            if (groups[k] == grp)
                hit = 1;
        if (!hit)
            continue;
        for (int k = 0; k < per; k++)
        {
            int id = b[3 + k];
            if (seen[id])
                continue;
            seen[id] = 1;
            float val = 0.0f;
            if (grp == leftGroup)
            {
                const float *xy = p2 ? m->vXY : m->cornerXY;
                val = inflow(peak, xy[2 * id + 1]);
            }
            r[n].id = id;
            r[n].v = val;
            n++;
        }
    }
    free(seen);
    qsort(r, n, sizeof(dnode), cmp_dnode);
    *out = r;
    return n;
}

static int complement(int n, const dnode *d, int nd, int **out)
{
    int *r = (int *)malloc(sizeof(int) * (n + 1));
    int k = 0, j = 0;
    for (int i = 0; i < n; i++)
    {
        while (j < nd && d[j].id < i)
            j++;
        if (j < nd && d[j].id == i)
            continue;
        r[k++] = i;
    }
    *out = r;
    return k;
}

int orc_channel_bcs(const orc_mesh *m, float peakVelocity, orc_context *ctx)
{
    int left = orc_group_id(m, "Left"), right = orc_group_id(m, "Right"), top = orc_group_id(m, "Top"),
        bottom = orc_group_id(m, "Bottom"), circle = orc_group_id(m, "Circle");
    if (left < 0 || right < 0 || top < 0 || bottom < 0 || circle < 0)
    {
        set_err("channel mesh needs Left/Right/Top/Bottom/Circle groups");
        return 1;
    }
    ctx->N = m->numV;
    ctx->P = m->numP;
    int vg[4] = {left, top, bottom, circle};
    dnode *dv, *dp;
    ctx->nDir = extract_dirichlet(m, 1, vg, 4, left, peakVelocity, &dv);
    ctx->dirIds = (int *)malloc(sizeof(int) * (ctx->nDir + 1));
    ctx->dirVx = (double *)malloc(sizeof(double) * (ctx->nDir + 1));
    for (int i = 0; i < ctx->nDir; i++)
    {
        ctx->dirIds[i] = dv[i].id;
        ctx->dirVx[i] = (double)dv[i].v;
    }
    int pg[1] = {right};
    ctx->nDirP = extract_dirichlet(m, 0, pg, 1, -1, 0.0f, &dp);
    ctx->dirPIds = (int *)malloc(sizeof(int) * (ctx->nDirP + 1));
    for (int i = 0; i < ctx->nDirP; i++)
        ctx->dirPIds[i] = dp[i].id;
    ctx->nIntV = complement(ctx->N, dv, ctx->nDir, &ctx->intV);
    ctx->nIntP = complement(ctx->P, dp, ctx->nDirP, &ctx->intP);
    free(dv);
    free(dp);
    return 0;
}
