/*
 * CPU oracle for the Chorin-projection hot path: a plain-C FP64 restatement of the reference's
 * algorithms (kosyonikolov/NsFemOptim).  TEST INFRASTRUCTURE ONLY: it is the checker that the
 * GPU path is compared against, and the CPU baseline that bench.py times.  The product never
 * links or calls it.
 *
 * Parity status: the integer parts (gmsh parse, P1/P2 DOF numbering, Dirichlet and internal
 * node lists, CSR sparsity patterns, smallest-last + greedy coloring, CSR slicing) and the
 * double-precision Gauss-Seidel sweep are pinned against the reference's own C++ compiled from
 * its sources (oracle/_ref).  The local element matrices (the reference computes them with
 * OpenCV, not buildable here) and the Eigen direct solves are restated; their values are
 * checked through physical identities (mass sums to the area, stiffness rows sum to zero,
 * divergence/gradient transpose pair) and parity there is "unpinned".
 */
#ifndef NSF_ORACLE_H
#define NSF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
    int rows, cols, nnz;
    int *rowStart; /* rows + 1 */
    int *col;      /* nnz, sorted within each row */
    double *val;   /* nnz (may be NULL for a pattern) */
} orc_csr;

typedef struct
{
    /* corner mesh (mesh::TriangleMesh) */
    int numCorner, numTri, numBorder, numGroups;
    float *cornerXY;      /* 2 * numCorner */
    int *tri;             /* 3 * numTri */
    int *border;          /* 3 * numBorder: triangle, side, group */
    char **groups;        /* numGroups names */
    /* P2 velocity mesh and P1 pressure mesh (mesh::ConcreteMesh) */
    int numV, numP;
    float *vXY;           /* 2 * numV */
    int *vElem;           /* 6 * numTri: c0, m01, c1, m12, c2, m20 */
    int *vBorder;         /* 6 * numBorder: triangle, side, group, A, mid, B */
    int *pElem;           /* 3 * numTri */
    int *pBorder;         /* 5 * numBorder: triangle, side, group, A, B */
    float *affine;        /* 6 * numTri: m00 m01 m10 m11 b0 b1 (float, as el::AffineTransform) */
} orc_mesh;

typedef struct
{
    int N, P;                 /* velocity nodes per component, pressure nodes */
    int nDir;                 /* Dirichlet velocity nodes (same ids for x and y) */
    int *dirIds;              /* sorted */
    double *dirVx;            /* x values (float-rounded as the reference), y values are 0 */
    int nDirP;
    int *dirPIds;             /* pressure Dirichlet ids (Right border) */
    int nIntV, nIntP;
    int *intV, *intP;         /* internal node lists */
    orc_csr M, K, Kp, Kpi, D, G, I; /* mass, stiffness, pressure stiffness, its internal slice,
                                        divergence P x 2N, gradient 2N x P,
                                        FastConvection integration nnz(K) x 2N */
} orc_context;

typedef struct
{
    int n, nColors;
    int *perm;        /* new -> old row id (concatenated sorted partitions) */
    int *partStart;   /* nColors + 1 */
    int *slOrder;     /* smallest-last order (n) */
} orc_coloring;

/* ---------------- mesh ---------------- */
const char *orc_last_error(void);
orc_mesh *orc_mesh_load(const char *path);
void orc_mesh_free(orc_mesh *m);
int orc_group_id(const orc_mesh *m, const char *name);
/* channel problem lists (buildContext.cpp:64-93); fills N, P and the node lists */
int orc_channel_bcs(const orc_mesh *m, float peakVelocity, orc_context *ctx);

/* ---------------- FEM ---------------- */
/* assembles M, K, Kp, D, G, Kpi and (if withConvection) I; returns 0 on success */
int orc_assemble(const orc_mesh *m, orc_context *ctx, int withConvection);
/* Local matrices of element e, FP64, in the layout of the reference harness's ref_local_matrices:
   mass[36], stiffness[36] (P2), P1 stiffness[9], divergence x/y [3x6] each (rows P1), gradient
   x/y [6x3] each (rows P2), self-convection [12][6][6] (unit velocity of local DOF k: x of node k
   for k < 6, y of node k - 6) -- 585 doubles. */
#define ORC_LOCAL_SIZE 585
void orc_local_matrices(const orc_mesh *m, int e, double *out);
void orc_context_free(orc_context *ctx);

/* ---------------- linear algebra ---------------- */
void orc_csr_free(orc_csr *a);
void orc_spmv(const orc_csr *a, const double *x, double *y);
int orc_slice(const orc_csr *a, int nr, const int *rows, int nc, const int *cols, orc_csr *out);
int orc_coloring_build(const orc_csr *a, orc_coloring *out);
void orc_coloring_free(orc_coloring *c);
/* the color-permuted matrix P A P^T (rows and columns renumbered by coloring->perm) */
int orc_permute(const orc_csr *a, const orc_coloring *c, orc_csr *out);

/* multicolor Gauss-Seidel solve in the reference's cu::GaussSeidel semantics on the
   color-permuted system: numCh planar channels, x in/out (original ordering), RMS residual
   target checked every checkInterval iterations. Returns the last RMS per channel and
   iteration index as cu::GaussSeidel reports it. */
int orc_gs_solve(const orc_csr *a, const orc_coloring *c, int numCh, const double *b, double *x,
                 int maxIters, double targetRms, int checkInterval, double *lastRms, int *lastIter);
/* relative != 0: stop when ||r_c|| <= target * ||b_c|| for every channel */
int orc_gs_solve_ex(const orc_csr *a, const orc_coloring *c, int numCh, const double *b, double *x,
                    int maxIters, double target, int relative, int checkInterval, double *lastRms, int *lastIter);

/* CG preconditioned by symmetric multicolor Gauss-Seidel (forward colors, then backward).
   precond: 0 = none, 1 = multicolor SGS, 2 = Jacobi. Stops when ||r|| <= relTol * ||b||.
   Returns 0 converged, 3 max iterations, 4 breakdown (p^T A p <= 0), 2 non-finite. */
int orc_pcg(const orc_csr *a, const orc_coloring *c, int precond, const double *b, double *x,
            int maxIters, double relTol, int *iters, double *relRes);

/* the same PCG on a system prepared once (color permutation and diagonal split), for repeated
   solves with one matrix; a reference solver object likewise keeps its permuted matrix */
typedef struct orc_sys_s orc_sys;
orc_sys *orc_sys_create(const orc_csr *a, const orc_coloring *c);
void orc_sys_free(orc_sys *s);
int orc_sys_pcg(const orc_sys *s, int precond, const double *b, double *x, int maxIters, double relTol, int *iters,
                double *relRes);

/* Chebyshev iteration with the Jacobi preconditioner from x = 0, for an SPD matrix whose D^-1 A
   spectrum lies in [lo, hi]; orc_cheb_iters gives the a priori count for ||r|| <= relTol ||b||
   (capped at maxIters).  Returns 0 if the true residual meets relTol, 3 if not, 2 non-finite. */
int orc_cheb_iters(const orc_csr *a, double lo, double hi, double relTol, int maxIters);
int orc_cheb_solve(const orc_csr *a, const double *b, double *x, double lo, double hi, int iters,
                   double relTol, double *relRes);
/* the same from x0 (x0 == NULL: from 0); orc_cheb_warm_iters: the a priori count from the initial
   residual, ||r_k|| <= 2 rho^k sqrt(max D / min D) ||b - A x0|| <= relTol ||b|| (0 if x0 already
   meets it; capped at maxIters; -1 if ||b - A x0|| >= ||b||: then start from 0; -2 if b = 0: then
   x = 0 with no iteration) */
int orc_cheb_solve_from(const orc_csr *a, const double *b, const double *x0, double *x, double lo, double hi,
                        int iters, double relTol, double *relRes);
int orc_cheb_warm_iters(const orc_csr *a, double lo, double hi, const double *b, const double *x0, double relTol,
                        int maxIters);
/* spectral bounds of D^-1 M for the P2 mass matrix of affine triangles (any mesh) */
#define ORC_MASS_SPEC_LO 0.39237
#define ORC_MASS_SPEC_HI 2.05982

/* y = (D+L) D^-1 (D+U) inverse applied to r in colored order (the preconditioner alone) */
void orc_sgs_apply(const orc_csr *a, const orc_coloring *c, const double *r, double *z);

/* ---------------- Chorin step ---------------- */
typedef struct
{
    double nu, tau;
    int velMethod;       /* 0 = multicolor GS (RMS target), 1 = PCG-SGS, 2 = PCG-Jacobi, 3 = Chebyshev-
                            Jacobi, 4 = Chebyshev-Jacobi from the previous step's solution of the
                            same solve (relative tol) */
    int velMaxIters;
    double velTol;       /* RMS target for GS, relative tolerance for PCG */
    int presMaxIters;
    double presTol;      /* relative residual */
    int presGuess;       /* 0: start from the previous pressure; 1: from 2 p(n-1) - p(n-2) once two
                            solved pressures exist; 2: the Kp_int-orthogonal projection of the new
                            solution onto the last solutions (Fischer's method, presBasis vectors) */
    int presBasis;       /* presGuess 2: basis size, 3..256 (0 = 250) */
} orc_chorin_cfg;

typedef struct orc_chorin_s orc_chorin;
orc_chorin *orc_chorin_create(const orc_context *ctx, const orc_chorin_cfg *cfg);
void orc_chorin_free(orc_chorin *s);
/* state access: u is planar [ux(N); uy(N)], p has P entries */
void orc_chorin_get(const orc_chorin *s, double *u, double *p);
void orc_chorin_set(orc_chorin *s, const double *u, const double *p);
/* one time step; stats[0..5] = velocity iters (tentative), pressure iters, velocity iters
   (final), pressure relative residual, tentative residual, final residual */
int orc_chorin_step(orc_chorin *s, double *stats);
/* replace the x values of the Dirichlet velocity nodes (nDir, in ctx->dirIds order; y stays 0)
   and impose them on the current state */
void orc_chorin_set_dirichlet(orc_chorin *s, const double *dirVx);

/* the separate stages, exposed for parity tests */
void orc_fastconv(const orc_context *ctx, double nu, const double *u, double *Avals);
/* drag/lift: out[0..1] = integral over border group gid of (-p n + nu du/dn), n into the fluid */
void orc_forces(const orc_mesh *m, int gid, const double *u, const double *p, double nu, double *out);
void orc_spmm2(const orc_csr *a, const double *vals, const double *x, double *y);

/* ---------------- discrete adjoint (no counterpart in the reference) ---------------- */
/* Gradient of the force functional: F_x = nu * wV . u_x + wPx . p and F_y = nu * wV . u_y + wPy . p
   (wV: numV entries, wPx/wPy: numP entries), the same quadrature as orc_forces. */
void orc_forces_weights(const orc_mesh *m, int gid, double *wV, double *wPx, double *wPy);

/* Forward run of nSteps Chorin steps from (u0, p0) with Dirichlet x values dirVx, then the reverse
   sweep of the discrete adjoint (every linear solve taken as exact: PCG to solveTol), for
     J = sum_{n=1..nSteps} wDrag[n-1] F_x(u_n, p_n) + wLift[n-1] F_y(u_n, p_n),
   F the force on border group gid.  u0 (or the rest state if NULL) gets (dirVx, 0) on its
   Dirichlet rows.  out[0] = J, out[1] = dJ/dnu; dJdDir (nDir) = dJ/d dirVx (through the initial
   state and every step's impositions); dJdU0 (2N) = dJ/du0 on the free rows (0 on the Dirichlet
   rows).  Either may be NULL.  Returns 0, or the failing status. */
int orc_adjoint_run(const orc_context *ctx, const orc_mesh *m, int gid, const orc_chorin_cfg *cfg,
                    const double *dirVx, const double *u0, const double *p0, int nSteps, const double *wDrag,
                    const double *wLift, double solveTol, double *out, double *dJdDir, double *dJdU0);

#ifdef __cplusplus
}
#endif

#endif
