/*
 * Oracle, Chorin projection time step in FP64.  Test infrastructure only.
 *
 * Order of operations per step (cpp/execs/NavierStokes/src/chorinCuda.cu:236-376, with the
 * CPU twin cpp/execs/NavierStokes/src/chorinEigen.cpp:272-484):
 *   C.values = I u;  A.values = nu K.values + C.values                 (:243-250)
 *   rhs = A [ux uy];  acc = 0;  solve M acc = rhs (2 channels)         (:264-266)
 *   u = u - tau acc;  impose Dirichlet velocity                        (:275-278)
 *   div = -(1/tau) D u;  rhs_p = div[internal]                          (:297-298, :132-134)
 *   solve Kp_int p_int = rhs_p, warm-started from the previous p_int   (:300; the reference's
 *                                                                       solver keeps ioSol)
 *   p = 0;  p[internal] = p_int                                        (:145-146)
 *   g = G p;  acc = 0;  solve M acc = g;  u = u - tau acc;  Dirichlet   (:341-356)
 * Velocity solves: method 0 is the multicolor Gauss-Seidel solver with an RMS target (the
 * reference's "gs"), method 1 is CG with the multicolor SGS preconditioner to a relative
 * tolerance, method 2 the same CG with the Jacobi preconditioner, method 3 Chebyshev-Jacobi
 * with the a priori iteration count of orc_cheb_iters, method 4 the same started from the
 * previous step's solution of that solve (count from the initial residual, orc_cheb_warm_iters).  Pressure: CG with the multicolor SGS
 * preconditioner to a relative tolerance.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_chorin_s
{
    const orc_context *ctx;
    orc_chorin_cfg cfg;
    orc_coloring colM, colP;
    orc_sys *sysM, *sysP; /* M and Kp_int prepared once for the PCG solves */
    double *u, *p, *pInt, *Avals, *rhs, *acc, *div, *rhsP, *g;
    double *dirVx; /* x values imposed on the Dirichlet nodes (ctx->dirVx unless set) */
    double *pPrev; /* presGuess 1: the pressure solution before the last one */
    int pHist;     /* solved pressures seen since create / set (capped at 2) */
    /* presGuess 2 (Fischer, "Projection techniques for iterative solution of Ax = b with
       successive right-hand sides", CMAME 163, 1998): pX holds pL vectors, the first pM of them
       orthonormal in the Kp_int inner product; the solve starts from their projection of the new
       solution, sum_i (x_i . b) x_i, and its correction is orthogonalised into the basis (a full
       basis restarts from the solution and its last two differences) */
    double *pX, *pX0, *pW, *pQ, *pPrev2; /* pPrev2 (with pPrev, pHist): the last two solutions */
    double *accPrevT, *accPrevF;         /* velMethod 4: the last tentative and final mass solutions */
    int pM, pL;
};

orc_chorin *orc_chorin_create(const orc_context *ctx, const orc_chorin_cfg *cfg)
{
    orc_chorin *s = (orc_chorin *)calloc(1, sizeof *s);
    s->ctx = ctx;
    s->cfg = *cfg;
    orc_coloring_build(&ctx->M, &s->colM);
    orc_coloring_build(&ctx->Kpi, &s->colP);
    s->sysM = orc_sys_create(&ctx->M, &s->colM);
    s->sysP = orc_sys_create(&ctx->Kpi, &s->colP);
    const int N = ctx->N, P = ctx->P;
    s->u = (double *)calloc(2 * N, sizeof(double));
    s->p = (double *)calloc(P, sizeof(double));
    s->pInt = (double *)calloc(ctx->nIntP + 1, sizeof(double));
    s->Avals = (double *)calloc(ctx->K.nnz + 1, sizeof(double));
    s->rhs = (double *)calloc(2 * N, sizeof(double));
    s->acc = (double *)calloc(2 * N, sizeof(double));
    s->div = (double *)calloc(P, sizeof(double));
    s->rhsP = (double *)calloc(ctx->nIntP + 1, sizeof(double));
    s->g = (double *)calloc(2 * N, sizeof(double));
    s->pPrev = (double *)calloc(ctx->nIntP + 1, sizeof(double));
    s->accPrevT = (double *)calloc(2 * (size_t)N + 1, sizeof(double));
    s->accPrevF = (double *)calloc(2 * (size_t)N + 1, sizeof(double));
    s->pL = cfg->presBasis > 0 ? (cfg->presBasis < 256 ? cfg->presBasis : 256) : 250;
    if (cfg->presGuess == 2)
    {
        s->pX = (double *)calloc((size_t)s->pL * ctx->nIntP + 1, sizeof(double));
        s->pX0 = (double *)calloc(ctx->nIntP + 1, sizeof(double));
        s->pW = (double *)calloc(ctx->nIntP + 1, sizeof(double));
        s->pQ = (double *)calloc(ctx->nIntP + 1, sizeof(double));
        s->pPrev2 = (double *)calloc(ctx->nIntP + 1, sizeof(double));
    }
    s->dirVx = (double *)calloc(ctx->nDir + 1, sizeof(double));
    memcpy(s->dirVx, ctx->dirVx, sizeof(double) * ctx->nDir);
    for (int i = 0; i < ctx->nDir; i++)
    {
        s->u[ctx->dirIds[i]] = s->dirVx[i];
        s->u[ctx->dirIds[i] + N] = 0.0;
    }
    return s;
}

void orc_chorin_free(orc_chorin *s)
{
    if (!s)
        return;
    orc_coloring_free(&s->colM);
    orc_coloring_free(&s->colP);
    orc_sys_free(s->sysM);
    orc_sys_free(s->sysP);
    free(s->u);
    free(s->p);
    free(s->pInt);
    free(s->Avals);
    free(s->rhs);
    free(s->acc);
    free(s->div);
    free(s->rhsP);
    free(s->g);
    free(s->dirVx);
    free(s->pPrev);
    free(s->pX);
    free(s->pX0);
    free(s->pW);
    free(s->pQ);
    free(s->pPrev2);
    free(s->accPrevT);
    free(s->accPrevF);
    free(s);
}

void orc_chorin_set_dirichlet(orc_chorin *s, const double *dirVx)
{
    const orc_context *ctx = s->ctx;
    memcpy(s->dirVx, dirVx, sizeof(double) * ctx->nDir);
    for (int i = 0; i < ctx->nDir; i++)
    {
        s->u[ctx->dirIds[i]] = s->dirVx[i];
        s->u[ctx->dirIds[i] + ctx->N] = 0.0;
    }
}

void orc_chorin_get(const orc_chorin *s, double *u, double *p)
{
    if (u)
        memcpy(u, s->u, sizeof(double) * 2 * s->ctx->N);
    if (p)
        memcpy(p, s->p, sizeof(double) * s->ctx->P);
}

void orc_chorin_set(orc_chorin *s, const double *u, const double *p)
{
    const orc_context *ctx = s->ctx;
    if (u)
        memcpy(s->u, u, sizeof(double) * 2 * ctx->N);
    if (p)
    {
        memcpy(s->p, p, sizeof(double) * ctx->P);
        for (int i = 0; i < ctx->nIntP; i++)
            s->pInt[i] = p[ctx->intP[i]];
    }
    s->pHist = 0; /* a new pressure history starts from the state just set */
    s->pM = 0;
    memset(s->accPrevT, 0, sizeof(double) * 2 * ctx->N); /* the mass solves start cold again */
    memset(s->accPrevF, 0, sizeof(double) * 2 * ctx->N);
}

static void impose(orc_chorin *s)
{
    const orc_context *ctx = s->ctx;
    for (int i = 0; i < ctx->nDir; i++)
    {
        s->u[ctx->dirIds[i]] = s->dirVx[i];
        s->u[ctx->dirIds[i] + ctx->N] = 0.0;
    }
}

/* mass solve for both channels; returns iterations (max over channels) and the residual */
static int mass_solve(orc_chorin *s, const double *rhs, double *acc, double *res, int final)
{
    const orc_context *ctx = s->ctx;
    const int N = ctx->N;
    memset(acc, 0, sizeof(double) * 2 * N);
    if (s->cfg.velMethod == 0)
    {
        double rms[2];
        int it = 0;
        orc_gs_solve_ex(&ctx->M, &s->colM, 2, rhs, acc, s->cfg.velMaxIters, s->cfg.velTol, 1, 1, rms, &it);
        *res = rms[0] > rms[1] ? rms[0] : rms[1];
        return it;
    }
    int itMax = 0;
    *res = 0;
    if (s->cfg.velMethod == 4)
    {
        /* warm start from this solve's result of the previous step: the a priori count from the
           initial residual, ||r_k|| <= 2 rho^k sqrt(max D / min D) ||r_0|| <= tol ||b|| */
        double *prev = final ? s->accPrevF : s->accPrevT;
        const int kmax = orc_cheb_iters(&ctx->M, ORC_MASS_SPEC_LO, ORC_MASS_SPEC_HI, s->cfg.velTol, s->cfg.velMaxIters);
        int kUsed = 0, warm[2];
        for (int ch = 0; ch < 2; ch++)
        {
            int k = orc_cheb_warm_iters(&ctx->M, ORC_MASS_SPEC_LO, ORC_MASS_SPEC_HI, rhs + ch * N, prev + ch * N,
                                        s->cfg.velTol, kmax);
            warm[ch] = k >= 0; /* a channel whose previous solution is no better than 0 starts cold */
            if (k == -2)
                k = 0; /* zero right-hand side: cold, x = 0 */
            else if (k < 0)
                k = kmax;
            kUsed = k > kUsed ? k : kUsed;
        }
        for (int ch = 0; ch < 2; ch++)
        {
            double rr = 0;
            orc_cheb_solve_from(&ctx->M, rhs + ch * N, warm[ch] ? prev + ch * N : NULL, acc + ch * N,
                                ORC_MASS_SPEC_LO, ORC_MASS_SPEC_HI, kUsed, s->cfg.velTol, &rr);
            if (rr > *res)
                *res = rr;
        }
        memcpy(prev, acc, sizeof(double) * 2 * N);
        return kUsed;
    }
    if (s->cfg.velMethod == 3)
    {
        const int k = orc_cheb_iters(&ctx->M, ORC_MASS_SPEC_LO, ORC_MASS_SPEC_HI, s->cfg.velTol, s->cfg.velMaxIters);
        for (int ch = 0; ch < 2; ch++)
        {
            double rr = 0;
            orc_cheb_solve(&ctx->M, rhs + ch * N, acc + ch * N, ORC_MASS_SPEC_LO, ORC_MASS_SPEC_HI, k,
                           s->cfg.velTol, &rr);
            if (rr > *res)
                *res = rr;
        }
        return k;
    }
    for (int ch = 0; ch < 2; ch++)
    {
        int it = 0;
        double rr = 0;
        /* velMethod 1: SGS preconditioner, 2: Jacobi */
        int st = orc_sys_pcg(s->sysM, s->cfg.velMethod == 2 ? 2 : 1, rhs + ch * N, acc + ch * N,
                         s->cfg.velMaxIters, s->cfg.velTol, &it, &rr);
        (void)st;
        if (it > itMax)
            itMax = it;
        if (rr > *res)
            *res = rr;
    }
    return itMax;
}

static double dotn(const double *a, const double *b, int n)
{
    double t = 0;
    for (int i = 0; i < n; i++)
        t += a[i] * b[i];
    return t;
}

/* out[k] = X_k . v for k < m: the rows split into one chunk per thread, the chunks' partial sums
   added in thread order */
static void multi_dot(const double *X, int m, int n, const double *v, double *out)
{
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    double *part = (double *)calloc((size_t)nt * m + 1, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        int t = 0, T = 1;
#ifdef _OPENMP
        t = omp_get_thread_num();
        T = omp_get_num_threads();
#endif
        const int i0 = (int)((long long)n * t / T), i1 = (int)((long long)n * (t + 1) / T);
        for (int k = 0; k < m; k++)
        {
            const double *x = X + (size_t)k * n;
            double acc = 0;
            for (int i = i0; i < i1; i++)
                acc += x[i] * v[i];
            part[(size_t)t * m + k] = acc;
        }
    }
    for (int k = 0; k < m; k++)
    {
        double acc = 0;
        for (int t = 0; t < nt; t++)
            acc += part[(size_t)t * m + k];
        out[k] = acc;
    }
    free(part);
}

/* y = base + sign * sum_k c_k X_k for k < m (base may be y) */
static void combine(const double *X, int m, int n, const double *c, const double *base, double sign, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
    {
        double v = 0;
        for (int k = 0; k < m; k++)
            v += c[k] * X[(size_t)k * n + i];
        y[i] = (base ? base[i] : 0.0) + sign * v;
    }
}

/* pressure initial guess x0 = sum_i a_i x_i, a_i = x_i . b, over the basis (the previous solution
   while the basis is empty); x0 is kept for the update */
static void proj_guess(orc_chorin *s)
{
    const int n = s->ctx->nIntP;
    if (s->pM > 0)
    {
        double a[256];
        multi_dot(s->pX, s->pM, n, s->rhsP, a);
        combine(s->pX, s->pM, n, a, NULL, 1.0, s->pInt);
    }
    memcpy(s->pX0, s->pInt, sizeof(double) * n);
}

/* w (in pW) joins the basis: q = A w, beta_k = x_k . q, w' = w - sum_k beta_k x_k, twice
   (classical Gram-Schmidt with one re-orthogonalisation), and w' / |w'|_A with
   |w'|_A^2 = w' . A w' (its own product: no cancellation when w is close to the span) unless w' is
   (numerically) inside the span */
static void proj_add(orc_chorin *s)
{
    const int n = s->ctx->nIntP;
    orc_spmv(&s->ctx->Kpi, s->pW, s->pQ);
    const double g = dotn(s->pW, s->pQ, n);
    double beta[256];
    double *x = s->pX + (size_t)s->pM * n;
    memcpy(x, s->pW, sizeof(double) * n);
    for (int pass = 0; pass < 2; pass++)
    {
        if (pass == 1)
            orc_spmv(&s->ctx->Kpi, x, s->pQ);
        multi_dot(s->pX, s->pM, n, s->pQ, beta);
        combine(s->pX, s->pM, n, beta, x, -1.0, x);
    }
    orc_spmv(&s->ctx->Kpi, x, s->pQ);
    const double nn = dotn(x, s->pQ, n);
    if (!(g > 0) || !(nn > 1e-20 * g))
        return;
    const double inv = 1.0 / sqrt(nn);
    for (int i = 0; i < n; i++)
        x[i] *= inv;
    s->pM++;
}

/* After a solve: the correction x - x0 joins the basis.  An empty or full basis restarts from the
   solution and its first and second differences over the last two steps (the span then holds the
   linear and quadratic extrapolations; the pressure of the projection step carries a two-step
   oscillation that a single vector misses). */
static void proj_update(orc_chorin *s)
{
    const int n = s->ctx->nIntP;
    if (s->pM == 0 || s->pM == s->pL)
    {
        s->pM = 0;
        memcpy(s->pW, s->pInt, sizeof(double) * n);
        proj_add(s);
        if (s->pHist >= 1)
        {
            for (int i = 0; i < n; i++)
                s->pW[i] = s->pInt[i] - s->pPrev[i];
            proj_add(s);
        }
        if (s->pHist >= 2)
        {
            for (int i = 0; i < n; i++)
                s->pW[i] = s->pInt[i] - 2.0 * s->pPrev[i] + s->pPrev2[i];
            proj_add(s);
        }
    }
    else
    {
        for (int i = 0; i < n; i++)
            s->pW[i] = s->pInt[i] - s->pX0[i];
        proj_add(s);
    }
    memcpy(s->pPrev2, s->pPrev, sizeof(double) * n);
    memcpy(s->pPrev, s->pInt, sizeof(double) * n);
    if (s->pHist < 2)
        s->pHist++;
}

int orc_chorin_step(orc_chorin *s, double *stats)
{
    const orc_context *ctx = s->ctx;
    const int N = ctx->N, P = ctx->P;
    const double tau = s->cfg.tau;
    double resT = 0, resF = 0, resP = 0;

    orc_fastconv(ctx, s->cfg.nu, s->u, s->Avals);
    orc_spmm2(&ctx->K, s->Avals, s->u, s->rhs);
    int itT = mass_solve(s, s->rhs, s->acc, &resT, 0);
    for (int i = 0; i < 2 * N; i++)
        s->u[i] -= tau * s->acc[i];
    impose(s);

    orc_spmv(&ctx->D, s->u, s->div);
    const double invTau = -1.0 / tau;
    for (int i = 0; i < P; i++)
        s->div[i] *= invTau;
    for (int i = 0; i < ctx->nIntP; i++)
        s->rhsP[i] = s->div[ctx->intP[i]];
    if (s->cfg.presGuess == 1)
    {
        /* start from 2 p(n-1) - p(n-2) once two solved pressures exist */
        for (int i = 0; i < ctx->nIntP; i++)
        {
            const double cur = s->pInt[i];
            if (s->pHist >= 2)
                s->pInt[i] = 2.0 * cur - s->pPrev[i];
            s->pPrev[i] = cur;
        }
        if (s->pHist < 2)
            s->pHist++;
    }
    if (s->cfg.presGuess == 2)
        proj_guess(s);
    int itP = 0;
    int st = orc_sys_pcg(s->sysP, 1, s->rhsP, s->pInt, s->cfg.presMaxIters, s->cfg.presTol, &itP, &resP);
    if (s->cfg.presGuess == 2)
        proj_update(s);
    memset(s->p, 0, sizeof(double) * P);
    for (int i = 0; i < ctx->nIntP; i++)
        s->p[ctx->intP[i]] = s->pInt[i];

    orc_spmv(&ctx->G, s->p, s->g);
    int itF = mass_solve(s, s->g, s->acc, &resF, 1);
    for (int i = 0; i < 2 * N; i++)
        s->u[i] -= tau * s->acc[i];
    impose(s);

    if (stats)
    {
        stats[0] = itT;
        stats[1] = itP;
        stats[2] = itF;
        stats[3] = resP;
        stats[4] = resT;
        stats[5] = resF;
    }
    for (int i = 0; i < 2 * N; i++)
        if (!isfinite(s->u[i]))
            return 2;
    return st == 2 ? 2 : 0;
}
