/*
 * Oracle, linear-algebra part (FP64).  Test infrastructure only.
 *
 * Follows:
 *   CSR slice                    cpp/libs/LinAlg/src/csrMatrix.cpp:12-91
 *   row-order SpMV (rMultD)      cpp/libs/LinAlg/src/csrMatrix.cpp:224-238
 *   adjacency graph              cpp/libs/LinAlg/src/graphs.cpp:264-284
 *   smallest-last ordering       cpp/libs/LinAlg/src/graphs.cpp:64-121.  Its ties are decided by
 *                                std::priority_queue, i.e. by libstdc++'s binary heap
 *                                (push_heap sift-up; pop_heap moves the last element into the
 *                                root hole after sifting the hole down along the larger child,
 *                                with the odd single-child step); restated here as heap_push /
 *                                heap_pop so the order is bit-identical.
 *   greedy partition             cpp/libs/LinAlg/src/graphs.cpp:123-176
 *   color-contiguous reorder     cpp/libs/CudaUtils/src/gaussSeidel.cu:132-164
 *   GS context (strip diagonal)  cpp/libs/LinAlg/src/gaussSeidel.cpp:9-65
 *   multicolor GS solve          cpp/libs/CudaUtils/src/gaussSeidel.cu:76-119, 224-404
 *   CG recurrence                cpp/libs/CudaUtils/src/conjGradF.cu:20-151
 * The SGS preconditioner composes the multicolor sweep forward and backward (the reference has
 * no preconditioned CG; it is the composition the drop-in specifies).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

void orc_csr_free(orc_csr *a)
{
    free(a->rowStart);
    free(a->col);
    free(a->val);
    a->rowStart = NULL;
    a->col = NULL;
    a->val = NULL;
    a->rows = a->cols = a->nnz = 0;
}

void orc_spmv(const orc_csr *a, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < a->rows; i++)
    {
        double s = 0;
        for (int j = a->rowStart[i]; j < a->rowStart[i + 1]; j++)
            s += a->val[j] * x[a->col[j]];
        y[i] = s;
    }
}

/* y[:, c] = A x[:, c] for two planar channels, with explicit values (A's pattern) */
void orc_spmm2(const orc_csr *a, const double *vals, const double *x, double *y)
{
    const int n = a->rows, m = a->cols;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
    {
        double s0 = 0, s1 = 0;
        for (int j = a->rowStart[i]; j < a->rowStart[i + 1]; j++)
        {
            s0 += vals[j] * x[a->col[j]];
            s1 += vals[j] * x[a->col[j] + m];
        }
        y[i] = s0;
        y[i + n] = s1;
    }
}

typedef struct
{
    int id;
    double v;
} idval;

static int cmp_idval(const void *a, const void *b)
{
    int x = ((const idval *)a)->id, y = ((const idval *)b)->id;
    return (x > y) - (x < y);
}

int orc_slice(const orc_csr *a, int nr, const int *rows, int nc, const int *cols, orc_csr *out)
{
    memset(out, 0, sizeof *out);
    if (nr == 0 || nc == 0)
        return 0;
    int *colMap = (int *)malloc(sizeof(int) * a->cols);
    for (int i = 0; i < a->cols; i++)
        colMap[i] = -1;
    for (int i = 0; i < nc; i++)
        colMap[cols[i]] = i;
    out->rows = nr;
    out->cols = nc;
    out->rowStart = (int *)malloc(sizeof(int) * (nr + 1));
    int cap = 1024, nnz = 0;
    out->col = (int *)malloc(sizeof(int) * cap);
    out->val = (double *)malloc(sizeof(double) * cap);
    idval *tmp = (idval *)malloc(sizeof(idval) * (a->cols + 1));
    for (int i = 0; i < nr; i++)
    {
        out->rowStart[i] = nnz;
        int src = rows[i], k = 0;
        for (int j = a->rowStart[src]; j < a->rowStart[src + 1]; j++)
        {
            int dc = colMap[a->col[j]];
            if (dc < 0)
                continue;
            tmp[k].id = dc;
            tmp[k].v = a->val ? a->val[j] : 0.0;
            k++;
        }
        qsort(tmp, k, sizeof(idval), cmp_idval);
        if (nnz + k > cap)
        {
            while (nnz + k > cap)
                cap *= 2;
            out->col = (int *)realloc(out->col, sizeof(int) * cap);
            out->val = (double *)realloc(out->val, sizeof(double) * cap);
        }
        for (int q = 0; q < k; q++)
        {
            out->col[nnz] = tmp[q].id;
            out->val[nnz] = tmp[q].v;
            nnz++;
        }
    }
    out->rowStart[nr] = nnz;
    out->nnz = nnz;
    free(tmp);
    free(colMap);
    return 0;
}

/* ------------------------------------------------------------------ coloring */

typedef struct
{
    int v, d;
} hent;

/* "a < b" of the queue's element type: smaller degree sorts as larger (min-degree on top) */
static int hless(hent a, hent b) { return a.d > b.d; }

static void heap_sift_up(hent *h, long hole, long top, hent val)
{
    long parent = (hole - 1) / 2;
    while (hole > top && hless(h[parent], val))
    {
        h[hole] = h[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    h[hole] = val;
}

static void heap_push(hent *h, long *n, hent val)
{
    long hole = (*n)++;
    heap_sift_up(h, hole, 0, val);
}

static hent heap_pop(hent *h, long *n)
{
    hent top = h[0];
    long len = *n - 1;
    if (len > 0)
    {
        hent val = h[len];
        h[len] = top;
        long hole = 0, child = 0;
        while (child < (len - 1) / 2)
        {
            child = 2 * (child + 1);
            if (hless(h[child], h[child - 1]))
                child--;
            h[hole] = h[child];
            hole = child;
        }
        if ((len & 1) == 0 && child == (len - 2) / 2)
        {
            child = 2 * (child + 1);
            h[hole] = h[child - 1];
            hole = child - 1;
        }
        heap_sift_up(h, hole, 0, val);
    }
    *n = len;
    return top;
}

int orc_coloring_build(const orc_csr *a, orc_coloring *out)
{
    const int n = a->rows;
    memset(out, 0, sizeof *out);
    out->n = n;
    /* graph without the diagonal, neighbours in column order */
    int *gs = (int *)malloc(sizeof(int) * (n + 1));
    int *gc = (int *)malloc(sizeof(int) * (a->nnz + 1));
    int e = 0;
    for (int r = 0; r < n; r++)
    {
        gs[r] = e;
        for (int j = a->rowStart[r]; j < a->rowStart[r + 1]; j++)
            if (a->col[j] != r)
                gc[e++] = a->col[j];
    }
    gs[n] = e;

    /* smallest-last with lazy deletion */
    int *degree = (int *)malloc(sizeof(int) * (n + 1));
    char *removed = (char *)calloc(n + 1, 1);
    hent *heap = (hent *)malloc(sizeof(hent) * ((long)n + e + 1));
    long hn = 0;
    int *order = (int *)malloc(sizeof(int) * (n + 1));
    for (int i = 0; i < n; i++)
    {
        degree[i] = gs[i + 1] - gs[i];
        hent t = {i, degree[i]};
        heap_push(heap, &hn, t);
    }
    for (int i = 0; i < n; i++)
    {
        int v = -1;
        while (hn > 0)
        {
            hent c = heap_pop(heap, &hn);
            if (removed[c.v])
                continue;
            v = c.v;
            break;
        }
        order[i] = v;
        removed[v] = 1;
        for (int j = gs[v]; j < gs[v + 1]; j++)
        {
            int nv = gc[j];
            if (removed[nv])
                continue;
            degree[nv]--;
            hent t = {nv, degree[nv]};
            heap_push(heap, &hn, t);
        }
    }
    for (int i = 0; i < n / 2; i++)
    {
        int t = order[i];
        order[i] = order[n - 1 - i];
        order[n - 1 - i] = t;
    }
    free(heap);
    free(removed);
    free(degree);

    /* greedy: lowest color unused by already-colored neighbours */
    int *color = (int *)malloc(sizeof(int) * (n + 1));
    for (int i = 0; i < n; i++)
        color[i] = -1;
    int nColors = 0, capC = 16;
    char *used = (char *)calloc(capC, 1);
    if (n > 0)
    {
        color[order[0]] = 0;
        nColors = 1;
    }
    for (int k = 1; k < n; k++)
    {
        int i = order[k];
        memset(used, 0, nColors);
        for (int j = gs[i]; j < gs[i + 1]; j++)
            if (color[gc[j]] >= 0)
                used[color[gc[j]]] = 1;
        int c = 0;
        while (c < nColors && used[c])
            c++;
        if (c == nColors)
        {
            nColors++;
            if (nColors > capC)
            {
                capC *= 2;
                used = (char *)realloc(used, capC);
            }
        }
        color[i] = c;
    }
    free(used);

    /* partitions sorted by id and concatenated: a counting sort by color keeps ids ascending */
    out->nColors = nColors;
    out->partStart = (int *)calloc(nColors + 1, sizeof(int));
    for (int i = 0; i < n; i++)
        out->partStart[color[i] + 1]++;
    for (int c = 0; c < nColors; c++)
        out->partStart[c + 1] += out->partStart[c];
    out->perm = (int *)malloc(sizeof(int) * (n + 1));
    int *fill = (int *)calloc(nColors + 1, sizeof(int));
    for (int i = 0; i < n; i++)
        out->perm[out->partStart[color[i]] + fill[color[i]]++] = i;
    free(fill);
    free(color);
    free(gs);
    free(gc);
    out->slOrder = order;
    return 0;
}

void orc_coloring_free(orc_coloring *c)
{
    free(c->perm);
    free(c->partStart);
    free(c->slOrder);
    memset(c, 0, sizeof *c);
}

int orc_permute(const orc_csr *a, const orc_coloring *c, orc_csr *out)
{
    return orc_slice(a, c->n, c->perm, c->n, c->perm, out);
}

/* ------------------------------------------------------------------ Gauss-Seidel */

typedef struct
{
    orc_csr s;      /* permuted matrix without diagonal */
    double *invD;
    orc_csr full;   /* permuted matrix with diagonal (residuals) */
} gs_ctx;

static int gs_ctx_build(const orc_csr *a, const orc_coloring *c, gs_ctx *g)
{
    orc_permute(a, c, &g->full);
    const int n = g->full.rows;
    g->invD = (double *)malloc(sizeof(double) * (n + 1));
    g->s.rows = g->s.cols = n;
    g->s.rowStart = (int *)malloc(sizeof(int) * (n + 1));
    g->s.col = (int *)malloc(sizeof(int) * (g->full.nnz + 1));
    g->s.val = (double *)malloc(sizeof(double) * (g->full.nnz + 1));
    int k = 0;
    for (int r = 0; r < n; r++)
    {
        g->s.rowStart[r] = k;
        int found = 0;
        for (int j = g->full.rowStart[r]; j < g->full.rowStart[r + 1]; j++)
        {
            if (g->full.col[j] == r)
            {
                if (g->full.val[j] == 0)
                    return 1;
                g->invD[r] = 1.0 / g->full.val[j];
                found = 1;
            }
            else
            {
                g->s.col[k] = g->full.col[j];
                g->s.val[k] = g->full.val[j];
                k++;
            }
        }
        if (!found)
            return 1;
    }
    g->s.rowStart[n] = k;
    g->s.nnz = k;
    return 0;
}

static void gs_ctx_free(gs_ctx *g)
{
    orc_csr_free(&g->s);
    orc_csr_free(&g->full);
    free(g->invD);
}

/* one color phase: rows [r0, r1) of the stripped, permuted system */
static void gs_phase(const gs_ctx *g, int r0, int r1, double *x, const double *b)
{
    /* the rows of one color do not couple: any order, any number of threads */
#pragma omp parallel for schedule(static)
    for (int r = r0; r < r1; r++)
    {
        double s = 0;
        for (int j = g->s.rowStart[r]; j < g->s.rowStart[r + 1]; j++)
            s += g->s.val[j] * x[g->s.col[j]];
        x[r] = (b[r] - s) * g->invD[r];
    }
}

int orc_gs_solve(const orc_csr *a, const orc_coloring *c, int numCh, const double *b, double *x,
                 int maxIters, double targetRms, int checkInterval, double *lastRms, int *lastIter)
{
    return orc_gs_solve_ex(a, c, numCh, b, x, maxIters, targetRms, 0, checkInterval, lastRms, lastIter);
}

int orc_gs_solve_ex(const orc_csr *a, const orc_coloring *c, int numCh, const double *b, double *x,
                    int maxIters, double target, int relative, int checkInterval, double *lastRms, int *lastIter)
{
    const double targetRms = target;
    gs_ctx g;
    memset(&g, 0, sizeof g);
    if (gs_ctx_build(a, c, &g))
    {
        gs_ctx_free(&g);
        return 1;
    }
    const int n = a->rows;
    double *xp = (double *)malloc(sizeof(double) * n * numCh);
    double *bp = (double *)malloc(sizeof(double) * n * numCh);
    double *res = (double *)malloc(sizeof(double) * n);
    for (int ch = 0; ch < numCh; ch++)
        for (int i = 0; i < n; i++)
        {
            xp[ch * n + i] = x[ch * n + c->perm[i]];
            bp[ch * n + i] = b[ch * n + c->perm[i]];
        }
    double bRms[2] = {0, 0};
    for (int ch = 0; ch < numCh && ch < 2; ch++)
    {
        double s = 0;
        for (int i = 0; i < n; i++)
            s += bp[ch * n + i] * bp[ch * n + i];
        bRms[ch] = sqrt(s) / sqrt((double)n);
    }
    for (int ch = 0; ch < numCh; ch++)
        lastRms[ch] = -1;
    int iter = 0;
    for (; iter < maxIters; iter++)
    {
        for (int p = 0; p < c->nColors; p++)
            for (int ch = 0; ch < numCh; ch++)
                gs_phase(&g, c->partStart[p], c->partStart[p + 1], xp + ch * n, bp + ch * n);
        if (iter % checkInterval == 0)
        {
            int done = 1;
            for (int ch = 0; ch < numCh; ch++)
            {
                orc_spmv(&g.full, xp + ch * n, res);
                double s = 0;
                for (int i = 0; i < n; i++)
                {
                    double d = res[i] - bp[ch * n + i];
                    s += d * d;
                }
                lastRms[ch] = sqrt(s) / sqrt((double)n);
                /* absolute: RMS < target (cu::GaussSeidel); relative: ||r|| <= target * ||b|| */
                if (relative ? !(lastRms[ch] <= targetRms * bRms[ch < 2 ? ch : 1]) : !(lastRms[ch] < targetRms))
                    done = 0;
            }
            if (done)
                break;
        }
    }
    *lastIter = iter;
    for (int ch = 0; ch < numCh; ch++)
        for (int i = 0; i < n; i++)
            x[ch * n + c->perm[i]] = xp[ch * n + i];
    free(xp);
    free(bp);
    free(res);
    gs_ctx_free(&g);
    return 0;
}

/* z = SGS(r) in colored order: forward phases 0..C-1 from z = 0, then backward C-2..0 (the
   backward pass over the last color would recompute identical values) */
static void sgs_colored(const gs_ctx *g, const orc_coloring *c, const double *r, double *z)
{
    const int n = g->s.rows;
    for (int i = 0; i < n; i++)
        z[i] = 0;
    for (int p = 0; p < c->nColors; p++)
        gs_phase(g, c->partStart[p], c->partStart[p + 1], z, r);
    for (int p = c->nColors - 2; p >= 0; p--)
        gs_phase(g, c->partStart[p], c->partStart[p + 1], z, r);
}

void orc_sgs_apply(const orc_csr *a, const orc_coloring *c, const double *r, double *z)
{
    gs_ctx g;
    memset(&g, 0, sizeof g);
    gs_ctx_build(a, c, &g);
    const int n = a->rows;
    double *rp = (double *)calloc(n + 1, sizeof(double)), *zp = (double *)calloc(n + 1, sizeof(double));
    for (int i = 0; i < n; i++)
        rp[i] = r[c->perm[i]];
    sgs_colored(&g, c, rp, zp);
    for (int i = 0; i < n; i++)
        z[c->perm[i]] = zp[i];
    free(rp);
    free(zp);
    gs_ctx_free(&g);
}

/* z = preconditioner(r): 0 none, 1 multicolor SGS, 2 Jacobi (z = r / diag) */
static void precond_apply(const gs_ctx *g, const orc_coloring *c, int precond, const double *r, double *z)
{
    const int n = g->s.rows;
    if (precond == 1)
        sgs_colored(g, c, r, z);
    else if (precond == 2)
    {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++)
            z[i] = r[i] * g->invD[i];
    }
    else
        memcpy(z, r, sizeof(double) * n);
}

static double dot(const double *a, const double *b, int n)
{
    double s = 0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int i = 0; i < n; i++)
        s += a[i] * b[i];
    return s;
}

/* PCG in the colored ordering (the system is permuted once at entry and the solution permuted
   back at exit, as cu::GaussSeidel keeps its vectors permuted during a solve). */
static int pcg_core(const gs_ctx *g, const orc_coloring *c, int precond, const double *b, double *x,
                    int maxIters, double relTol, int *iters, double *relRes)
{
    const int n = g->full.rows;
    double *xp = (double *)malloc(sizeof(double) * n), *bp = (double *)malloc(sizeof(double) * n);
    double *r = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
    double *p = (double *)malloc(sizeof(double) * n), *q = (double *)malloc(sizeof(double) * n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
    {
        xp[i] = x[c->perm[i]];
        bp[i] = b[c->perm[i]];
    }
    int status = 3, it = 0;
    double bnorm = sqrt(dot(bp, bp, n));
    orc_spmv(&g->full, xp, q);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        r[i] = bp[i] - q[i];
    double rnorm = sqrt(dot(r, r, n));
    if (!isfinite(rnorm) || !isfinite(bnorm))
        status = 2;
    else if (rnorm <= relTol * bnorm)
        status = 0;
    else
    {
        precond_apply(g, c, precond, r, z);
        memcpy(p, z, sizeof(double) * n);
        double rz = dot(r, z, n);
        for (it = 1; it <= maxIters; it++)
        {
            orc_spmv(&g->full, p, q);
            double pq = dot(p, q, n);
            if (!(pq > 0))
            {
                status = isfinite(pq) ? 4 : 2;
                break;
            }
            double alpha = rz / pq;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++)
            {
                xp[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            rnorm = sqrt(dot(r, r, n));
            if (!isfinite(rnorm))
            {
                status = 2;
                break;
            }
            if (rnorm <= relTol * bnorm)
            {
                status = 0;
                break;
            }
            precond_apply(g, c, precond, r, z);
            double rzNew = dot(r, z, n);
            double beta = rzNew / rz;
            rz = rzNew;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++)
                p[i] = z[i] + beta * p[i];
        }
        if (it > maxIters)
            it = maxIters;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
        x[c->perm[i]] = xp[i];
    *iters = it;
    *relRes = bnorm > 0 ? rnorm / bnorm : rnorm;
    free(xp);
    free(bp);
    free(r);
    free(z);
    free(p);
    free(q);
    return status;
}

int orc_pcg(const orc_csr *a, const orc_coloring *c, int precond, const double *b, double *x,
            int maxIters, double relTol, int *iters, double *relRes)
{
    gs_ctx g;
    memset(&g, 0, sizeof g);
    if (gs_ctx_build(a, c, &g))
    {
        gs_ctx_free(&g);
        return 1;
    }
    const int st = pcg_core(&g, c, precond, b, x, maxIters, relTol, iters, relRes);
    gs_ctx_free(&g);
    return st;
}

/* a system prepared once (color-permuted, diagonal split off) for repeated PCG solves */
struct orc_sys_s
{
    gs_ctx g;
    const orc_coloring *c;
};

orc_sys *orc_sys_create(const orc_csr *a, const orc_coloring *c)
{
    orc_sys *s = (orc_sys *)calloc(1, sizeof *s);
    s->c = c;
    if (gs_ctx_build(a, c, &s->g))
    {
        orc_sys_free(s);
        return NULL;
    }
    return s;
}

void orc_sys_free(orc_sys *s)
{
    if (!s)
        return;
    gs_ctx_free(&s->g);
    free(s);
}

int orc_sys_pcg(const orc_sys *s, int precond, const double *b, double *x, int maxIters, double relTol, int *iters,
                double *relRes)
{
    return pcg_core(&s->g, s->c, precond, b, x, maxIters, relTol, iters, relRes);
}

/* ---------------- Chebyshev-Jacobi solve (mass-solve method 3) ----------------
 * Saad, Iterative Methods for Sparse Linear Systems, Alg. 12.1 with the Jacobi preconditioner and
 * x0 = 0; [lo, hi] bounds the spectrum of D^-1 A.  The iteration count follows the a priori bound
 * ||r_k|| <= 2 rho^k sqrt(max D / min D) ||b||, rho = (sqrt(hi/lo) - 1) / (sqrt(hi/lo) + 1),
 * taken as the smallest k that brings it under relTol (at least 1, at most maxIters). */
static double diag_ratio(const orc_csr *a)
{
    double lo = 1e300, hi = 0;
    for (int i = 0; i < a->rows; i++)
        for (int j = a->rowStart[i]; j < a->rowStart[i + 1]; j++)
            if (a->col[j] == i)
            {
                const double d = fabs(a->val[j]);
                lo = d < lo ? d : lo;
                hi = d > hi ? d : hi;
            }
    return lo > 0 && lo < 1e300 ? hi / lo : 1.0;
}

int orc_cheb_iters(const orc_csr *a, double lo, double hi, double relTol, int maxIters)
{
    const double kappa = hi / lo, rho = (sqrt(kappa) - 1.0) / (sqrt(kappa) + 1.0);
    int k = (int)ceil(log(relTol / (2.0 * sqrt(diag_ratio(a)))) / log(rho));
    if (k < 1)
        k = 1;
    return k < maxIters ? k : maxIters;
}

int orc_cheb_warm_iters(const orc_csr *a, double lo, double hi, const double *b, const double *x0, double relTol,
                        int maxIters)
{
    const int n = a->rows;
    double *q = (double *)malloc(sizeof(double) * n);
    orc_spmv(a, x0, q);
    double rr = 0, bb = 0;
    for (int i = 0; i < n; i++)
    {
        rr += (b[i] - q[i]) * (b[i] - q[i]);
        bb += b[i] * b[i];
    }
    free(q);
    if (bb == 0)
        return -2; /* b = 0: x = 0 is exact, a cold start needs no iteration */
    if (!(rr < bb))
        return -1; /* x0 is no better a start than 0 */
    if (!(rr > relTol * relTol * bb))
        return 0;
    const double kappa = hi / lo, rho = (sqrt(kappa) - 1.0) / (sqrt(kappa) + 1.0);
    int k = (int)ceil(log(relTol * sqrt(bb) / (2.0 * sqrt(diag_ratio(a)) * sqrt(rr))) / log(rho));
    if (k < 1)
        k = 1;
    return k < maxIters ? k : maxIters;
}

int orc_cheb_solve(const orc_csr *a, const double *b, double *x, double lo, double hi, int iters,
                   double relTol, double *relRes)
{
    return orc_cheb_solve_from(a, b, NULL, x, lo, hi, iters, relTol, relRes);
}

int orc_cheb_solve_from(const orc_csr *a, const double *b, const double *x0, double *x, double lo, double hi,
                        int iters, double relTol, double *relRes)
{
    const int n = a->rows;
    double *invD = (double *)malloc(sizeof(double) * n), *r = (double *)malloc(sizeof(double) * n);
    double *d = (double *)malloc(sizeof(double) * n), *q = (double *)malloc(sizeof(double) * n);
    for (int i = 0; i < n; i++)
    {
        invD[i] = 0;
        for (int j = a->rowStart[i]; j < a->rowStart[i + 1]; j++)
            if (a->col[j] == i)
                invD[i] = 1.0 / a->val[j];
    }
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    double rho = 1.0 / sigma;
    if (x0)
        orc_spmv(a, x0, q);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
    {
        x[i] = x0 ? x0[i] : 0.0;
        r[i] = x0 ? b[i] - q[i] : b[i];
        d[i] = r[i] * invD[i] / theta;
    }
    for (int k = 0; k < iters; k++)
    {
        const double rhoN = 1.0 / (2.0 * sigma - rho), c1 = rhoN * rho, c2 = 2.0 * rhoN / delta;
        orc_spmv(a, d, q);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++)
        {
            x[i] += d[i];
            r[i] -= q[i];
            d[i] = c1 * d[i] + c2 * r[i] * invD[i];
        }
        rho = rhoN;
    }
    /* true residual of the result */
    orc_spmv(a, x, q);
    const double bb = dot(b, b, n);
    double rr = 0;
    for (int i = 0; i < n; i++)
        rr += (b[i] - q[i]) * (b[i] - q[i]);
    *relRes = bb > 0 ? sqrt(rr / bb) : sqrt(rr);
    free(invD);
    free(r);
    free(d);
    free(q);
    if (!isfinite(rr))
        return 2;
    return rr <= relTol * relTol * bb ? 0 : 3;
}
