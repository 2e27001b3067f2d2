/*
 * Oracle, FEM part: P1/P2 shape functions, 6-point degree-4 quadrature, local mass, stiffness,
 * divergence and self-convection matrices, serial assembly into sorted CSR patterns and the
 * FastConvection integration matrix.  FP64 arithmetic on the reference's float geometry.
 * Test infrastructure only.
 *
 * Follows:
 *   P2 shape/gradient        cpp/libs/Element/src/p2.cpp:35-84 (node order c0, m01, c1, m12, c2, m20)
 *   P1 shape/gradient        cpp/libs/Element/src/p1.cpp:35-57
 *   quadrature (degree 4)    cpp/libs/Element/src/triangleIntegrator.cpp:27-35
 *   Jacobian, B, det         cpp/libs/Element/src/triangleIntegrator.cpp:84-111
 *   mass                     cpp/libs/Element/src/triangleIntegrator.cpp:132-163
 *   stiffness                cpp/libs/Element/src/triangleIntegrator.cpp:165-190
 *   self-convection          cpp/libs/Element/src/triangleIntegrator.cpp:192-231
 *   divergence (swap=false D, swap=true G)  cpp/libs/Element/src/triangleIntegrator.cpp:233-293
 *   patterns                 cpp/libs/Fem/src/chorinCsr.cpp:142-261, cpp/libs/LinAlg/src/sparseDokBuilder.cpp:310-364
 *   accumulation             cpp/libs/Fem/src/chorinCsr.cpp:296-419 (serial element order here)
 *   internal pressure slice  cpp/execs/NavierStokes/src/buildContext.cpp:120
 *   FastConvection           cpp/libs/Fem/src/fastConvection.cpp:9-100
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Cowper degree-4 rule on the reference triangle (x, y, weight); weights sum to 1/2 */
static const double QX[6] = {9.15762135097710067155318824916321e-02, 9.15762135097710067155318824916321e-02,
                             8.16847572980457958813360619387822e-01, 4.45948490915965001235576892213430e-01,
                             4.45948490915965001235576892213430e-01, 1.08103018168069997528846215573139e-01};
static const double QY[6] = {9.15762135097710067155318824916321e-02, 8.16847572980457958813360619387822e-01,
                             9.15762135097710067155318824916321e-02, 4.45948490915965001235576892213430e-01,
                             1.08103018168069997528846215573139e-01, 4.45948490915965001235576892213430e-01};
static const double QW[6] = {5.49758718276610602870846378209535e-02, 5.49758718276610602870846378209535e-02,
                             5.49758718276610602870846378209535e-02, 1.11690794839005624883299105931656e-01,
                             1.11690794839005624883299105931656e-01, 1.11690794839005624883299105931656e-01};

static void p2_shape(double x, double y, double *s)
{
    s[0] = 1 - 3 * x - 3 * y + 2 * x * x + 2 * y * y + 4 * x * y;
    s[1] = 4 * x - 4 * x * x - 4 * x * y;
    s[2] = -x + 2 * x * x;
    s[3] = 4 * x * y;
    s[4] = -y + 2 * y * y;
    s[5] = 4 * y - 4 * y * y - 4 * x * y;
}

static void p2_grad(double x, double y, double *gx, double *gy)
{
    gx[0] = -3 + 4 * x + 4 * y;
    gy[0] = -3 + 4 * y + 4 * x;
    gx[1] = 4 - 8 * x - 4 * y;
    gy[1] = -4 * x;
    gx[2] = -1 + 4 * x;
    gy[2] = 0;
    gx[3] = 4 * y;
    gy[3] = 4 * x;
    gx[4] = 0;
    gy[4] = -1 + 4 * y;
    gx[5] = -4 * y;
    gy[5] = 4 - 8 * y - 4 * x;
}

static void p1_shape(double x, double y, double *s)
{
    s[0] = 1 - x - y;
    s[1] = x;
    s[2] = y;
}

static const double P1GX[3] = {-1, 1, 0};
static const double P1GY[3] = {-1, 0, 1};

typedef struct
{
    double b00, b01, b10, b11; /* B = [[m11, -m10], [-m01, m00]] */
    double det, sgn;
} geom;

static geom element_geom(const float *af)
{
    /* af = m00 m01 m10 m11 b0 b1 */
    geom g;
    double m00 = af[0], m01 = af[1], m10 = af[2], m11 = af[3];
    g.b00 = m11;
    g.b01 = -m10;
    g.b10 = -m01;
    g.b11 = m00;
    /* J = m^T, det(J) = m00 m11 - m10 m01 */
    g.det = m00 * m11 - m10 * m01;
    g.sgn = g.det < 0 ? -1.0 : 1.0;
    return g;
}

/* local matrices of one element */
typedef struct
{
    double M[6][6], K[6][6], Kp[3][3];
    double Dx[3][6], Dy[3][6]; /* rows P1, cols P2 */
    double Gx[6][3], Gy[6][3]; /* rows P2, cols P1 */
} local_mats;

static void local_matrices(const geom *g, local_mats *L)
{
    memset(L, 0, sizeof *L);
    double adet = fabs(g->det);
    /* B^T B */
    double t00 = g->b00 * g->b00 + g->b10 * g->b10;
    double t01 = g->b00 * g->b01 + g->b10 * g->b11;
    double t11 = g->b01 * g->b01 + g->b11 * g->b11;
    for (int q = 0; q < 6; q++)
    {
        double phi[6], gx[6], gy[6], psi[3];
        p2_shape(QX[q], QY[q], phi);
        p2_grad(QX[q], QY[q], gx, gy);
        p1_shape(QX[q], QY[q], psi);
        double w = QW[q];
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++)
            {
                L->M[i][j] += w * phi[i] * phi[j];
                L->K[i][j] += w * (gx[i] * (t00 * gx[j] + t01 * gy[j]) + gy[i] * (t01 * gx[j] + t11 * gy[j]));
            }
        double ws = w * g->sgn;
        /* global gradients (times det): B * local gradient */
        double Gxv[6], Gyv[6];
        for (int c = 0; c < 6; c++)
        {
            Gxv[c] = g->b00 * gx[c] + g->b01 * gy[c];
            Gyv[c] = g->b10 * gx[c] + g->b11 * gy[c];
        }
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 6; c++)
            {
                L->Dx[r][c] += ws * psi[r] * Gxv[c];
                L->Dy[r][c] += ws * psi[r] * Gyv[c];
            }
        double Pxv[3], Pyv[3];
        for (int c = 0; c < 3; c++)
        {
            Pxv[c] = g->b00 * P1GX[c] + g->b01 * P1GY[c];
            Pyv[c] = g->b10 * P1GX[c] + g->b11 * P1GY[c];
        }
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 3; c++)
            {
                L->Gx[r][c] += ws * phi[r] * Pxv[c];
                L->Gy[r][c] += ws * phi[r] * Pyv[c];
            }
    }
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++)
        {
            L->M[i][j] *= adet;
            L->K[i][j] /= adet;
        }
    /* P1 stiffness: constant gradients, area weight 1/2 */
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            L->Kp[i][j] = 0.5 / adet *
                          (P1GX[i] * (t00 * P1GX[j] + t01 * P1GY[j]) + P1GY[i] * (t01 * P1GX[j] + t11 * P1GY[j]));
}

/* ------------------------------------------------------------------ sparse patterns */

typedef struct
{
    int rows, cols;
    int *cnt, *start, *fill, *col;
} pattern_builder;

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* two passes: count, then fill; rows are then sorted and deduplicated */
static void pb_init(pattern_builder *b, int rows, int cols)
{
    b->rows = rows;
    b->cols = cols;
    b->cnt = (int *)calloc(rows + 1, sizeof(int));
    b->start = NULL;
    b->fill = NULL;
    b->col = NULL;
}

static void pb_alloc(pattern_builder *b)
{
    b->start = (int *)malloc(sizeof(int) * (b->rows + 1));
    b->start[0] = 0;
    for (int r = 0; r < b->rows; r++)
        b->start[r + 1] = b->start[r] + b->cnt[r];
    b->fill = (int *)calloc(b->rows, sizeof(int));
    b->col = (int *)malloc(sizeof(int) * (b->start[b->rows] + 1));
}

static void pb_put(pattern_builder *b, int r, int c)
{
    b->col[b->start[r] + b->fill[r]++] = c;
}

static void pb_finish(pattern_builder *b, orc_csr *out)
{
    out->rows = b->rows;
    out->cols = b->cols;
    out->rowStart = (int *)malloc(sizeof(int) * (b->rows + 1));
    int nnz = 0;
    for (int r = 0; r < b->rows; r++)
    {
        int *c = b->col + b->start[r];
        int n = b->fill[r];
        qsort(c, n, sizeof(int), cmp_int);
        int k = 0;
        for (int i = 0; i < n; i++)
            if (k == 0 || c[i] != c[k - 1])
                c[k++] = c[i];
        b->fill[r] = k;
        nnz += k;
    }
    out->nnz = nnz;
    out->col = (int *)malloc(sizeof(int) * (nnz + 1));
    out->val = (double *)calloc(nnz + 1, sizeof(double));
    int p = 0;
    for (int r = 0; r < b->rows; r++)
    {
        out->rowStart[r] = p;
        memcpy(out->col + p, b->col + b->start[r], sizeof(int) * b->fill[r]);
        p += b->fill[r];
    }
    out->rowStart[b->rows] = p;
    free(b->cnt);
    free(b->start);
    free(b->fill);
    free(b->col);
}

/* position of column c in row r (binary search), -1 if absent */
static int csr_find(const orc_csr *a, int r, int c)
{
    int lo = a->rowStart[r], hi = a->rowStart[r + 1];
    while (lo < hi)
    {
        int mid = (lo + hi) >> 1;
        if (a->col[mid] < c)
            lo = mid + 1;
        else
            hi = mid;
    }
    return (lo < a->rowStart[r + 1] && a->col[lo] == c) ? lo : -1;
}

static int patterns(const orc_mesh *m, orc_context *ctx)
{
    const int N = m->numV, P = m->numP, T = m->numTri;
    pattern_builder bv, bp, bd, bg;
    pb_init(&bv, N, N);
    pb_init(&bp, P, P);
    pb_init(&bd, P, 2 * N);
    pb_init(&bg, 2 * N, P);
    for (int pass = 0; pass < 2; pass++)
    {
        if (pass == 1)
        {
            pb_alloc(&bv);
            pb_alloc(&bp);
            pb_alloc(&bd);
            pb_alloc(&bg);
        }
        for (int e = 0; e < T; e++)
        {
            const int *iv = m->vElem + 6 * e, *ip = m->pElem + 3 * e;
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 6; c++)
                {
                    if (pass)
                        pb_put(&bv, iv[r], iv[c]);
                    else
                        bv.cnt[iv[r]]++;
                }
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++)
                {
                    if (pass)
                        pb_put(&bp, ip[r], ip[c]);
                    else
                        bp.cnt[ip[r]]++;
                }
            for (int a = 0; a < 6; a++)
                for (int q = 0; q < 3; q++)
                {
                    if (pass)
                    {
                        pb_put(&bd, ip[q], iv[a]);
                        pb_put(&bd, ip[q], iv[a] + N);
                        pb_put(&bg, iv[a], ip[q]);
                        pb_put(&bg, iv[a] + N, ip[q]);
                    }
                    else
                    {
                        bd.cnt[ip[q]] += 2;
                        bg.cnt[iv[a]]++;
                        bg.cnt[iv[a] + N]++;
                    }
                }
        }
    }
    pb_finish(&bv, &ctx->M);
    pb_finish(&bp, &ctx->Kp);
    pb_finish(&bd, &ctx->D);
    pb_finish(&bg, &ctx->G);
    /* K shares the velocity pattern */
    ctx->K.rows = ctx->M.rows;
    ctx->K.cols = ctx->M.cols;
    ctx->K.nnz = ctx->M.nnz;
    ctx->K.rowStart = (int *)malloc(sizeof(int) * (N + 1));
    memcpy(ctx->K.rowStart, ctx->M.rowStart, sizeof(int) * (N + 1));
    ctx->K.col = (int *)malloc(sizeof(int) * (ctx->M.nnz + 1));
    memcpy(ctx->K.col, ctx->M.col, sizeof(int) * ctx->M.nnz);
    ctx->K.val = (double *)calloc(ctx->M.nnz + 1, sizeof(double));
    return 0;
}

/* FastConvection integration matrix: row k = k-th entry (r, c) of the convection pattern,
   columns = global velocity DOFs (x block, then y block).  For a unit velocity in local DOF j
   (x or y component), the local self-convection entry is
       C[r][c] = sum_q w sgn(det) phi_r (B^T e phi_j) . grad^ phi_c
   so I[(r,c), j_x] = sum_q w sgn phi_r phi_j (b00 gx_c + b01 gy_c) and
      I[(r,c), j_y] = sum_q w sgn phi_r phi_j (b10 gx_c + b11 gy_c). */
/* Self-convection of one element, linear in the local velocity: Ix[r][c][k] (Iy) is the (r, c) entry
   of the local convection matrix for a unit x (y) velocity at local DOF k, as FastConvection's
   constructor evaluates it (fastConvection.cpp:64-97 over triangleIntegrator.cpp:192-231). */
static void local_convection(const geom *g, double Ix[6][6][6], double Iy[6][6][6])
{
    memset(Ix, 0, sizeof(double) * 216);
    memset(Iy, 0, sizeof(double) * 216);
    for (int q = 0; q < 6; q++)
    {
        double phi[6], gx[6], gy[6];
        p2_shape(QX[q], QY[q], phi);
        p2_grad(QX[q], QY[q], gx, gy);
        double ws = QW[q] * g->sgn;
        for (int c = 0; c < 6; c++)
        {
            double ax = g->b00 * gx[c] + g->b01 * gy[c];
            double ay = g->b10 * gx[c] + g->b11 * gy[c];
            for (int r = 0; r < 6; r++)
                for (int k = 0; k < 6; k++)
                {
                    double f = ws * phi[r] * phi[k];
                    Ix[r][c][k] += f * ax;
                    Iy[r][c][k] += f * ay;
                }
        }
    }
}

void orc_local_matrices(const orc_mesh *m, int e, double *out)
{
    geom g = element_geom(m->affine + 6 * e);
    local_mats L;
    local_matrices(&g, &L);
    double Ix[6][6][6], Iy[6][6][6];
    local_convection(&g, Ix, Iy);
    double *o = out;
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++)
            *o++ = L.M[r][c];
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 6; c++)
            *o++ = L.K[r][c];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            *o++ = L.Kp[r][c];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 6; c++)
            *o++ = L.Dx[r][c];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 6; c++)
            *o++ = L.Dy[r][c];
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 3; c++)
            *o++ = L.Gx[r][c];
    for (int r = 0; r < 6; r++)
        for (int c = 0; c < 3; c++)
            *o++ = L.Gy[r][c];
    for (int k = 0; k < 12; k++)
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++)
                *o++ = k < 6 ? Ix[r][c][k] : Iy[r][c][k - 6];
}

static int fast_convection(const orc_mesh *m, orc_context *ctx)
{
    const int N = m->numV, T = m->numTri;
    const orc_csr *C = &ctx->K; /* convection pattern == velocity pattern */
    pattern_builder bi;
    pb_init(&bi, C->nnz, 2 * N);
    int slot[6][6];
    for (int pass = 0; pass < 2; pass++)
    {
        if (pass == 1)
            pb_alloc(&bi);
        for (int e = 0; e < T; e++)
        {
            const int *iv = m->vElem + 6 * e;
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 6; c++)
                    slot[r][c] = csr_find(C, iv[r], iv[c]);
            for (int r = 0; r < 6; r++)
                for (int c = 0; c < 6; c++)
                    for (int k = 0; k < 6; k++)
                    {
                        if (pass)
                        {
                            pb_put(&bi, slot[r][c], iv[k]);
                            pb_put(&bi, slot[r][c], iv[k] + N);
                        }
                        else
                            bi.cnt[slot[r][c]] += 2;
                    }
        }
    }
    pb_finish(&bi, &ctx->I);
    for (int e = 0; e < T; e++)
    {
        const int *iv = m->vElem + 6 * e;
        geom g = element_geom(m->affine + 6 * e);
        double Ix[6][6][6], Iy[6][6][6];
        local_convection(&g, Ix, Iy);
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++)
            {
                int row = csr_find(C, iv[r], iv[c]);
                for (int k = 0; k < 6; k++)
                {
                    ctx->I.val[csr_find(&ctx->I, row, iv[k])] += Ix[r][c][k];
                    ctx->I.val[csr_find(&ctx->I, row, iv[k] + N)] += Iy[r][c][k];
                }
            }
    }
    return 0;
}

int orc_assemble(const orc_mesh *m, orc_context *ctx, int withConvection)
{
    const int N = m->numV, T = m->numTri;
    patterns(m, ctx);
    for (int e = 0; e < T; e++)
    {
        const int *iv = m->vElem + 6 * e, *ip = m->pElem + 3 * e;
        geom g = element_geom(m->affine + 6 * e);
        local_mats L;
        local_matrices(&g, &L);
        for (int r = 0; r < 6; r++)
            for (int c = 0; c < 6; c++)
            {
                int k = csr_find(&ctx->M, iv[r], iv[c]);
                ctx->M.val[k] += L.M[r][c];
                ctx->K.val[k] += L.K[r][c];
            }
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                ctx->Kp.val[csr_find(&ctx->Kp, ip[r], ip[c])] += L.Kp[r][c];
        for (int a = 0; a < 6; a++)
            for (int q = 0; q < 3; q++)
            {
                ctx->D.val[csr_find(&ctx->D, ip[q], iv[a])] += L.Dx[q][a];
                ctx->D.val[csr_find(&ctx->D, ip[q], iv[a] + N)] += L.Dy[q][a];
                ctx->G.val[csr_find(&ctx->G, iv[a], ip[q])] += L.Gx[a][q];
                ctx->G.val[csr_find(&ctx->G, iv[a] + N, ip[q])] += L.Gy[a][q];
            }
    }
    if (ctx->nIntP > 0)
        orc_slice(&ctx->Kp, ctx->nIntP, ctx->intP, ctx->nIntP, ctx->intP, &ctx->Kpi);
    if (withConvection)
        fast_convection(m, ctx);
    return 0;
}

void orc_context_free(orc_context *ctx)
{
    free(ctx->dirIds);
    free(ctx->dirVx);
    free(ctx->dirPIds);
    free(ctx->intV);
    free(ctx->intP);
    orc_csr_free(&ctx->M);
    orc_csr_free(&ctx->K);
    orc_csr_free(&ctx->Kp);
    orc_csr_free(&ctx->Kpi);
    orc_csr_free(&ctx->D);
    orc_csr_free(&ctx->G);
    orc_csr_free(&ctx->I);
    memset(ctx, 0, sizeof *ctx);
}

/* Force of the flow on the border group `gid` (the cylinder "Circle"):
     F = sum over the group's border edges of  integral ( -p n + nu du/dn ) ds
   with n the unit edge normal pointing into the fluid (towards the adjacent triangle), u the P2
   velocity (planar u[0..N) x, u[N..2N) y) and p the P1 pressure of the adjacent triangle, on each
   straight edge by 2-point Gauss-Legendre quadrature (exact: the integrand is at most quadratic
   along the edge).  New: the reference has no force functional; the definition is the continuum
   one of the DFG benchmark in stress form with the velocity gradient (not symmetrised). */
void orc_forces(const orc_mesh *m, int gid, const double *u, const double *p, double nu, double *out)
{
    const int N = m->numV;
    const double g = 0.5 / sqrt(3.0);
    const double tq[2] = {0.5 - g, 0.5 + g};
    double fx = 0, fy = 0;
    for (int b = 0; b < m->numBorder; b++)
    {
        const int *vb = m->vBorder + 6 * b;
        if (vb[2] != gid)
            continue;
        const int t = vb[0];
        const int *ve = m->vElem + 6 * t, *pe = m->pElem + 3 * t;
        const double x0 = m->vXY[2 * ve[0]], y0 = m->vXY[2 * ve[0] + 1];
        const double x1 = m->vXY[2 * ve[2]], y1 = m->vXY[2 * ve[2] + 1];
        const double x2 = m->vXY[2 * ve[4]], y2 = m->vXY[2 * ve[4] + 1];
        /* J = [[x1-x0, x2-x0], [y1-y0, y2-y0]] maps the reference triangle */
        const double j00 = x1 - x0, j01 = x2 - x0, j10 = y1 - y0, j11 = y2 - y0;
        const double det = j00 * j11 - j01 * j10;
        const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det; /* J^-1 */
        const double ax = m->vXY[2 * vb[3]], ay = m->vXY[2 * vb[3] + 1];
        const double bx = m->vXY[2 * vb[5]], by = m->vXY[2 * vb[5] + 1];
        const double dx = bx - ax, dy = by - ay, len = sqrt(dx * dx + dy * dy);
        double nx = dy / len, ny = -dx / len;
        const double cx = (x0 + x1 + x2) / 3 - 0.5 * (ax + bx), cy = (y0 + y1 + y2) / 3 - 0.5 * (ay + by);
        if (nx * cx + ny * cy < 0)
        {
            nx = -nx;
            ny = -ny;
        }
        for (int q = 0; q < 2; q++)
        {
            const double px = ax + tq[q] * dx - x0, py = ay + tq[q] * dy - y0;
            const double xi = i00 * px + i01 * py, eta = i10 * px + i11 * py;
            double gx[6], gy[6], psi[3];
            p2_grad(xi, eta, gx, gy);
            p1_shape(xi, eta, psi);
            double uxx = 0, uxy = 0, uyx = 0, uyy = 0, pq = 0;
            for (int k = 0; k < 6; k++)
            {
                /* physical gradient = J^-T * reference gradient */
                const double Gx = i00 * gx[k] + i10 * gy[k], Gy = i01 * gx[k] + i11 * gy[k];
                uxx += u[ve[k]] * Gx;
                uxy += u[ve[k]] * Gy;
                uyx += u[N + ve[k]] * Gx;
                uyy += u[N + ve[k]] * Gy;
            }
            for (int k = 0; k < 3; k++)
                pq += p[pe[k]] * psi[k];
            const double w = 0.5 * len;
            fx += w * (-pq * nx + nu * (uxx * nx + uxy * ny));
            fy += w * (-pq * ny + nu * (uyx * nx + uyy * ny));
        }
    }
    out[0] = fx;
    out[1] = fy;
}

/* The same sums as orc_forces, with each nodal value's coefficient collected instead of its
   product: F_x = nu wV.u_x + wPx.p, F_y = nu wV.u_y + wPy.p (the functional is linear). */
void orc_forces_weights(const orc_mesh *m, int gid, double *wV, double *wPx, double *wPy)
{
    const double g = 0.5 / sqrt(3.0);
    const double tq[2] = {0.5 - g, 0.5 + g};
    memset(wV, 0, sizeof(double) * m->numV);
    memset(wPx, 0, sizeof(double) * m->numP);
    memset(wPy, 0, sizeof(double) * m->numP);
    for (int b = 0; b < m->numBorder; b++)
    {
        const int *vb = m->vBorder + 6 * b;
        if (vb[2] != gid)
            continue;
        const int t = vb[0];
        const int *ve = m->vElem + 6 * t, *pe = m->pElem + 3 * t;
        const double x0 = m->vXY[2 * ve[0]], y0 = m->vXY[2 * ve[0] + 1];
        const double x1 = m->vXY[2 * ve[2]], y1 = m->vXY[2 * ve[2] + 1];
        const double x2 = m->vXY[2 * ve[4]], y2 = m->vXY[2 * ve[4] + 1];
        const double j00 = x1 - x0, j01 = x2 - x0, j10 = y1 - y0, j11 = y2 - y0;
        const double det = j00 * j11 - j01 * j10;
        const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
        const double ax = m->vXY[2 * vb[3]], ay = m->vXY[2 * vb[3] + 1];
        const double bx = m->vXY[2 * vb[5]], by = m->vXY[2 * vb[5] + 1];
        const double dx = bx - ax, dy = by - ay, len = sqrt(dx * dx + dy * dy);
        double nx = dy / len, ny = -dx / len;
        const double cx = (x0 + x1 + x2) / 3 - 0.5 * (ax + bx), cy = (y0 + y1 + y2) / 3 - 0.5 * (ay + by);
        if (nx * cx + ny * cy < 0)
        {
            nx = -nx;
            ny = -ny;
        }
        for (int q = 0; q < 2; q++)
        {
            const double px = ax + tq[q] * dx - x0, py = ay + tq[q] * dy - y0;
            const double xi = i00 * px + i01 * py, eta = i10 * px + i11 * py;
            double gx[6], gy[6], psi[3];
            p2_grad(xi, eta, gx, gy);
            p1_shape(xi, eta, psi);
            const double w = 0.5 * len;
            for (int k = 0; k < 6; k++)
            {
                const double Gx = i00 * gx[k] + i10 * gy[k], Gy = i01 * gx[k] + i11 * gy[k];
                wV[ve[k]] += w * (Gx * nx + Gy * ny);
            }
            for (int k = 0; k < 3; k++)
            {
                wPx[pe[k]] -= w * psi[k] * nx;
                wPy[pe[k]] -= w * psi[k] * ny;
            }
        }
    }
}

/* A.values = nu * K.values + I * u  (fastConvection.cpp:102-115 with chorinCuda.cu:243-250) */
void orc_fastconv(const orc_context *ctx, double nu, const double *u, double *Avals)
{
    const orc_csr *I = &ctx->I;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < I->rows; k++)
    {
        double s = 0;
        for (int j = I->rowStart[k]; j < I->rowStart[k + 1]; j++)
            s += I->val[j] * u[I->col[j]];
        Avals[k] = nu * ctx->K.val[k] + s;
    }
}
