/*
 * Oracle, discrete adjoint of the Chorin time step (FP64).  Test infrastructure only: the FP64 CPU
 * reference gradient that the GPU adjoint is checked against, and the CPU baseline of the
 * gradient workload.  The reference has no adjoint, so parity here is pinned only by finite
 * differences of the forward oracle (tests/test_oracle_pins.py).
 *
 * The forward step is orc_chorin_step (cpp/execs/NavierStokes/src/chorinCuda.cu:236-376):
 *   A = nu K + I(u0);  rhs = A u0;  acc = M^-1 rhs;  v = u0 - tau acc;  u* = Dir(v, g)
 *   rhsP = -(1/tau) R D u*;  pI = Kpi^-1 rhsP;  p = R^T pI
 *   gG = G p;  acc2 = M^-1 gG;  w = u* - tau acc2;  u1 = Dir(w, g)
 * with Dir(v, g) = v on free rows and (g, 0) on the Dirichlet rows, R the restriction to the
 * internal pressure nodes.  Taking every solve as exact, the reverse of one step maps the
 * adjoint of its outputs (lu1, lp) to the adjoint of its input lu0:
 *   lg += lu1[dir, x];  lw = lu1 with Dirichlet rows zeroed
 *   x1 = M^-1 (-tau lw);  lpI = R (lp + G^T x1);  y = Kpi^-1 lpI
 *   ls = lw - (1/tau) D^T R^T y;  lg += ls[dir, x];  lv = ls with Dirichlet rows zeroed
 *   x2 = M^-1 (-tau lv);  lu0 = lv + A^T x2 + I^T lA,  lA[e=(i,j)] = sum_c x2_c[i] u0_c[j]
 *   lnu += sum_e lA[e] K[e]
 * (M, Kpi symmetric).  The functional's own contribution at step n is lu_n += c nu wV,
 * lp_n += c wP and lnu += c wV.u_n (orc_forces_weights).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* y += A^T x  (A rows x cols, x rows entries, y cols entries) */
static void spmv_t_add(const orc_csr *a, const double *vals, const double *x, double *y)
{
    for (int i = 0; i < a->rows; i++)
    {
        const double xi = x[i];
        if (xi == 0.0)
            continue;
        for (int e = a->rowStart[i]; e < a->rowStart[i + 1]; e++)
            y[a->col[e]] += vals[e] * xi;
    }
}

static int solve(const orc_sys *s, int n, const double *b, double *x, double tol)
{
    int it = 0;
    double rr = 0;
    memset(x, 0, sizeof(double) * n);
    const int st = orc_sys_pcg(s, 1, b, x, 100000, tol, &it, &rr);
    return st == 0 ? 0 : st;
}

int orc_adjoint_run(const orc_context *ctx, const orc_mesh *m, int gid, const orc_chorin_cfg *cfg,
                    const double *dirVx, const double *u0, const double *p0, int nSteps, const double *wDrag,
                    const double *wLift, double solveTol, double *out, double *dJdDir, double *dJdU0)
{
    const int N = ctx->N, P = ctx->P, nI = ctx->nIntP, nnz = ctx->K.nnz;
    const double nu = cfg->nu, tau = cfg->tau;
    int status = 0;

    double *U = (double *)malloc(sizeof(double) * 2 * N * (size_t)(nSteps + 1));
    double *wV = (double *)calloc(N, sizeof(double)), *wPx = (double *)calloc(P, sizeof(double));
    double *wPy = (double *)calloc(P, sizeof(double));
    double *lam = (double *)calloc(2 * N, sizeof(double)), *ls = (double *)calloc(2 * N, sizeof(double));
    double *rhs = (double *)calloc(2 * N, sizeof(double)), *x = (double *)calloc(2 * N, sizeof(double));
    double *lp = (double *)calloc(P, sizeof(double)), *lpI = (double *)calloc(nI + 1, sizeof(double));
    double *y = (double *)calloc(nI + 1, sizeof(double)), *lDiv = (double *)calloc(P, sizeof(double));
    double *A = (double *)calloc(nnz, sizeof(double)), *lA = (double *)calloc(nnz, sizeof(double));
    double *lg = (double *)calloc(ctx->nDir + 1, sizeof(double)), *pTmp = (double *)calloc(P, sizeof(double));
    orc_forces_weights(m, gid, wV, wPx, wPy);

    /* forward: keep every input state, accumulate J and the explicit nu term */
    double J = 0, lnu = 0;
    {
        orc_chorin *s = orc_chorin_create(ctx, cfg);
        orc_chorin_set(s, u0, p0);
        orc_chorin_set_dirichlet(s, dirVx);
        for (int n = 0; n < nSteps && status == 0; n++)
        {
            orc_chorin_get(s, U + (size_t)2 * N * n, NULL);
            status = orc_chorin_step(s, NULL);
            orc_chorin_get(s, U + (size_t)2 * N * (n + 1), pTmp);
            const double cx = wDrag ? wDrag[n] : 0.0, cy = wLift ? wLift[n] : 0.0;
            if (cx != 0.0 || cy != 0.0)
            {
                double f[2];
                orc_forces(m, gid, U + (size_t)2 * N * (n + 1), pTmp, nu, f);
                J += cx * f[0] + cy * f[1];
                const double *un = U + (size_t)2 * N * (n + 1);
                double vx = 0, vy = 0;
                for (int v = 0; v < N; v++)
                {
                    vx += wV[v] * un[v];
                    vy += wV[v] * un[N + v];
                }
                lnu += cx * vx + cy * vy;
            }
        }
        orc_chorin_free(s);
    }

    orc_coloring colM, colP;
    orc_coloring_build(&ctx->M, &colM);
    orc_coloring_build(&ctx->Kpi, &colP);
    orc_sys *sysM = orc_sys_create(&ctx->M, &colM), *sysP = orc_sys_create(&ctx->Kpi, &colP);
    const double invTau = 1.0 / tau;
    for (int n = nSteps - 1; n >= 0 && status == 0; n--)
    {
        const double *u = U + (size_t)2 * N * n;
        const double cx = wDrag ? wDrag[n] : 0.0, cy = wLift ? wLift[n] : 0.0;
        /* the functional at the output of step n */
        for (int v = 0; v < N; v++)
        {
            lam[v] += cx * nu * wV[v];
            lam[N + v] += cy * nu * wV[v];
        }
        for (int i = 0; i < P; i++)
            lp[i] = cx * wPx[i] + cy * wPy[i];
        /* final Dirichlet imposition */
        for (int d = 0; d < ctx->nDir; d++)
        {
            const int r = ctx->dirIds[d];
            lg[d] += lam[r];
            lam[r] = 0.0;
            lam[N + r] = 0.0;
        }
        /* second mass solve and the gradient */
        for (int i = 0; i < 2 * N; i++)
            rhs[i] = -tau * lam[i];
        status |= solve(sysM, N, rhs, x, solveTol);
        status |= solve(sysM, N, rhs + N, x + N, solveTol);
        spmv_t_add(&ctx->G, ctx->G.val, x, lp);
        for (int i = 0; i < nI; i++)
            lpI[i] = lp[ctx->intP[i]];
        /* pressure solve and the divergence */
        status |= solve(sysP, nI, lpI, y, solveTol);
        memset(lDiv, 0, sizeof(double) * P);
        for (int i = 0; i < nI; i++)
            lDiv[ctx->intP[i]] = -invTau * y[i];
        memcpy(ls, lam, sizeof(double) * 2 * N);
        spmv_t_add(&ctx->D, ctx->D.val, lDiv, ls);
        /* tentative Dirichlet imposition */
        for (int d = 0; d < ctx->nDir; d++)
        {
            const int r = ctx->dirIds[d];
            lg[d] += ls[r];
            ls[r] = 0.0;
            ls[N + r] = 0.0;
        }
        /* first mass solve, A^T and the linearisation */
        for (int i = 0; i < 2 * N; i++)
            rhs[i] = -tau * ls[i];
        status |= solve(sysM, N, rhs, x, solveTol);
        status |= solve(sysM, N, rhs + N, x + N, solveTol);
        orc_fastconv(ctx, nu, u, A);
        memcpy(lam, ls, sizeof(double) * 2 * N);
        spmv_t_add(&ctx->K, A, x, lam);
        spmv_t_add(&ctx->K, A, x + N, lam + N);
        for (int i = 0; i < N; i++)
            for (int e = ctx->K.rowStart[i]; e < ctx->K.rowStart[i + 1]; e++)
            {
                const int j = ctx->K.col[e];
                lA[e] = x[i] * u[j] + x[N + i] * u[N + j];
            }
        for (int e = 0; e < nnz; e++)
            lnu += lA[e] * ctx->K.val[e];
        spmv_t_add(&ctx->I, ctx->I.val, lA, lam);
    }
    orc_coloring_free(&colM);
    orc_coloring_free(&colP);
    orc_sys_free(sysM);
    orc_sys_free(sysP);
    /* the initial state's Dirichlet rows hold (dirVx, 0) as well */
    for (int d = 0; d < ctx->nDir; d++)
    {
        const int r = ctx->dirIds[d];
        lg[d] += lam[r];
        lam[r] = 0.0;
        lam[N + r] = 0.0;
    }

    if (out)
    {
        out[0] = J;
        out[1] = lnu;
    }
    if (dJdDir)
        memcpy(dJdDir, lg, sizeof(double) * ctx->nDir);
    if (dJdU0)
        memcpy(dJdU0, lam, sizeof(double) * 2 * N);
    free(U);
    free(wV);
    free(wPx);
    free(wPy);
    free(lam);
    free(ls);
    free(rhs);
    free(x);
    free(lp);
    free(lpI);
    free(y);
    free(lDiv);
    free(A);
    free(lA);
    free(lg);
    free(pTmp);
    return status;
}
