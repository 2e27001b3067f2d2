/*
 * nsfem_gb300 — C ABI of the GB300-native Chorin-projection path.
 *
 * Plain C: opaque handles, int32 indices, host or device pointers as documented per call,
 * cudaStream_t passed as void*.  Every call returns an nsf_status; nsf_last_error() gives a
 * one-line message for the calling thread.  Device pointers are owned by the caller unless a
 * handle says otherwise.  Nothing here uses cuSPARSE, cuBLAS or any other vendor math library.
 *
 * Each entry point names the reference interface (kosyonikolov/NsFemOptim, paths inside that
 * project) that it replaces.
 */
#ifndef NSFEM_GB300_H
#define NSFEM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
    NSF_OK = 0,
    NSF_ERR_INVALID_ARG = 1,  /* bad size, pointer, unsorted/out-of-range CSR, missing diagonal */
    NSF_ERR_NONFINITE = 2,    /* a solver residual or the state became NaN/Inf */
    NSF_ERR_MAXITER = 3,      /* the iteration cap was reached before the tolerance */
    NSF_ERR_BREAKDOWN = 4,    /* CG breakdown: p^T A p <= 0 (matrix not SPD) */
    NSF_ERR_CUDA = 5,         /* a CUDA runtime call failed */
    NSF_ERR_IO = 6,           /* file not found / parse error */
    NSF_ERR_NOT_SUPPORTED = 7
} nsf_status;

typedef enum
{
    NSF_F32 = 0,
    NSF_F64 = 1
} nsf_dtype;

typedef enum
{
    NSF_PREC_F64 = 0,   /* everything in FP64 */
    NSF_PREC_MIXED = 1, /* FP32 SpMV/sweeps/inner CG, FP64 residual refinement, dots and state */
    NSF_PREC_F64_MIXEDSOLVE = 2, /* stepper only: FP64 operators and state (the FP64 step), every
                                    solve FP32 CG inside FP64 refinement / residual replacement,
                                    stopping on the same FP64 residual test as NSF_PREC_F64 */
    NSF_PREC_MIXED_F32 = 3 /* stepper only: the literal FP32-inner split -- FastConvection, A u,
                              D u and G p with FP32 values, vectors and sums; the mass and pressure
                              solves FP32 PCG inside FP64 refinement / residual replacement
                              (velMethod 1 or 2); state, residuals and dot-product accumulation of
                              the step lengths in FP64.  NSF_PREC_MIXED keeps FP64-level sums
                              (double-float, FP64) in the products that feed the divergence. */
} nsf_precision;

const char *nsf_last_error(void);
const char *nsf_status_string(int status);
int nsf_version(void);

/* ======================================================================= host setup ===== */

typedef struct nsf_mesh_s *nsf_mesh;

/* gmsh MSH 4.1 ASCII file -> corner mesh -> P2 velocity and P1 pressure numbering.
   Replaces mesh::parseGmsh (cpp/libs/Mesh/src/gmsh.cpp:451), mesh::parseTriangleGmsh
   (cpp/libs/Mesh/src/io.cpp:65) and mesh::createMesh (cpp/libs/Mesh/src/concreteMesh.cpp:78). */
int nsf_mesh_load_gmsh(const char *path, nsf_mesh *out);
/* counts[0..5] = corner nodes, triangles, border elements, P2 nodes (N), P1 nodes (P), groups */
int nsf_mesh_counts(nsf_mesh mesh, int *counts);
/* copies: vElem[6*T] (c0, m01, c1, m12, c2, m20), pElem[3*T], vXY[2*N] float, vBorder[6*B]
   (triangle, side, group, A, mid, B); any pointer may be NULL */
int nsf_mesh_arrays(nsf_mesh mesh, int *vElem, int *pElem, float *vXY, int *vBorder);
/* name of border group i (the string lives as long as the mesh) */
const char *nsf_mesh_group(nsf_mesh mesh, int i);
void nsf_mesh_destroy(nsf_mesh mesh);

typedef struct nsf_context_s *nsf_context;

/* Channel-flow context: Dirichlet velocity on Left/Top/Bottom/Circle with the parabolic inflow
   u = peak*y*(0.41-y)/0.41^2 on Left, Dirichlet pressure on Right, FP64 assembly of the mass M,
   stiffness K, pressure stiffness Kp (and its internal slice), divergence D (P x 2N), gradient
   G (2N x P) and the FastConvection integration matrix I (nnz(K) x 2N).
   Replaces buildChorinContext (cpp/execs/NavierStokes/src/buildContext.cpp:17-142) with
   fem::buildChorinCsrMatrices (cpp/libs/Fem/src/chorinCsr.cpp:437-502) and fem::FastConvection
   (cpp/libs/Fem/src/fastConvection.cpp:9-100).  nThreads <= 0 picks the hardware count. */
int nsf_context_build(nsf_mesh mesh, float peakVelocity, int nThreads, nsf_context *out);
/* nsf_context_build with the operator values assembled on the GPU: the patterns, boundary lists
   and the internal-pressure slice on the host, every value of M, K, Kp, D, G and I by one device
   thread per output row gathering its incident elements in ascending order (the element-parallel
   local matrices of cpp/libs/Element/src/triangleIntegrator.cpp:132-293 and the accumulation of
   cpp/libs/Fem/src/chorinCsr.cpp:296-419 and cpp/libs/Fem/src/fastConvection.cpp:52-97); the values
   equal nsf_context_build's bit for bit.  assemblyMs (may be NULL): device time of the assembly
   kernels. */
int nsf_context_build_device(nsf_mesh mesh, float peakVelocity, int nThreads, nsf_context *out, double *assemblyMs);
/* sizes[0..12] = N, P, nDir, nDirP, nIntV, nIntP, nnz(M), nnz(K), nnz(Kp), nnz(Kpi), nnz(D),
   nnz(G), nnz(I) */
int nsf_context_sizes(nsf_context ctx, int *sizes);
/* which: 0 M, 1 K, 2 Kp, 3 Kpi, 4 D, 5 G, 6 I; copies the host CSR (any pointer may be NULL) */
int nsf_context_matrix(nsf_context ctx, int which, int *rowStart, int *col, double *val);
/* dirIds[nDir] (sorted), dirVx[nDir] (x inflow values; y values are 0), dirPIds[nDirP],
   intV[nIntV], intP[nIntP]; any pointer may be NULL */
int nsf_context_lists(nsf_context ctx, int *dirIds, double *dirVx, int *dirPIds, int *intV, int *intP);
void nsf_context_destroy(nsf_context ctx);

/* Smallest-last + greedy coloring of the adjacency graph of a square CSR pattern, partitions
   sorted by id and concatenated.  perm[n] (new -> old), partStart[n + 1] (first *nColors + 1
   entries used).  Replaces the coloring in cu::GaussSeidel's constructor
   (cpp/libs/CudaUtils/src/gaussSeidel.cu:132-155) over linalg::buildSmallestLastOrdering and
   linalg::partitionGraphGreedy (cpp/libs/LinAlg/src/graphs.cpp:64-176). */
int nsf_coloring(int n, const int *rowStart, const int *col, int *perm, int *partStart, int *nColors);

/* ====================================================== binary CSR / vector interchange files == */

/* The reference's binary format (cpp/libs/LinAlg/src/io.cpp:49-148: linalg::write, linalg::readCsr,
   linalg::readVec): native byte order, CSR = int dtype (0 float, 1 double), int rows, int cols,
   int nnz, values[nnz], column[nnz], rowStart[rows + 1]; vector = int dtype, int n, values[n].
   Values are passed as doubles; dtype says how they are stored in the file.  Reading fails with
   NSF_ERR_IO on what the reference's reader rejects (bad dtype, non-positive sizes, short data,
   rowStart[rows] != nnz) and on unsorted or out-of-range columns. */
/* info[0..3] = rows, cols, nnz, dtype of a CSR file */
int nsf_io_csr_info(const char *path, int *info);
/* rowStart[rows + 1], col[nnz], values[nnz] (sizes from nsf_io_csr_info) */
int nsf_io_read_csr(const char *path, int *rowStart, int *col, double *values);
int nsf_io_write_csr(const char *path, int rows, int cols, int nnz, const int *rowStart, const int *col,
                     const double *values, int dtype);
/* info[0..1] = n, dtype of a vector file */
int nsf_io_vec_info(const char *path, int *info);
int nsf_io_read_vec(const char *path, double *values);
int nsf_io_write_vec(const char *path, int n, const double *values, int dtype);

/* ===================================================================== device CSR ======= */

typedef struct nsf_csr_s *nsf_csr;

/* Upload a host CSR (0-based, rowStart[rows] == nnz, columns sorted and in range, values in
   dtype).  Validated before upload.  Replaces cu::csrF::csrF (cpp/libs/CudaUtils/src/csrF.cu:5-9). */
int nsf_csr_create(int rows, int cols, int nnz, const int *rowStart, const int *col, const void *values,
                   int dtype, nsf_csr *out);
/* replace the values (host pointer when onDevice == 0, else a device pointer) */
int nsf_csr_update_values(nsf_csr a, const void *values, int onDevice, void *stream);
/* device pointers of the stored arrays */
int nsf_csr_device(nsf_csr a, int **rowStart, int **col, void **values);
void nsf_csr_destroy(nsf_csr a);

/* y = alpha A x + beta y on device vectors of the matrix dtype.
   Replaces cu::spmv::compute (cpp/libs/CudaUtils/src/spmv.cu:48-63). */
int nsf_spmv(nsf_csr a, const void *x, void *y, double alpha, double beta, void *stream);
/* Y[:, c] = A X[:, c] for nrhs planar channels (column c starts at c * ld).
   Replaces cu::spmm::compute (cpp/libs/CudaUtils/src/spmm.cu:53-70). */
int nsf_spmm(nsf_csr a, int nrhs, const void *X, int ldx, void *Y, int ldy, void *stream);
/* Avals = nu * Kvals + I u, the linearised advection update fused with the diffusion add.
   Replaces fcSpmv.compute + cublasSgeam (cpp/execs/NavierStokes/src/chorinCuda.cu:243-250). */
int nsf_fastconv_apply(nsf_csr I, const void *Kvals, double nu, const void *u, void *Avals, void *stream);
/* The same with FP32 operator values and double-float vectors and sums: Kvals, u and Avals hold
   (hi, lo) float pairs (value = hi + lo, about 48 significant bits), 2 floats per entry; I has
   dtype NSF_F32.  The FastConvection product of the mixed-precision stepper: the matrix traffic is
   FP32 and the arithmetic runs on the FP32 pipes, while A keeps the precision that the divergence
   needs (it amplifies rounding noise that changes from step to step).  Replaces the same
   reference calls as nsf_fastconv_apply. */
int nsf_fastconv_apply_df(nsf_csr I, const float *Kvals, double nu, const float *u, float *Avals, void *stream);

/* Largest nrhs nsf_residual_noalloc accepts (its scratch is sized for it). */
#define NSF_NOALLOC_MAX_RHS 4

/* FP64 residual with no device allocation: r[c] = b[c] - A x[c] for nrhs planar channels of
   a->rows doubles (device pointers), and the squared norms written to the device array norms2:
   norms2[c] = ||r[c]||^2, norms2[nrhs + c] = ||b[c]||^2 (c < nrhs).  r equals
   nsf_spmv(a, x, y = copy of b, -1, 1) up to the summation order of each row.
   No counterpart in the reference.  It exists for callers that may not allocate device memory
   during the call: code that runs while another component holds the allocator (a caching
   allocator or a memory pool it does not own), real-time loops where an allocation would
   synchronise the device, and embedders with a fixed device-memory budget.  The block partial
   sums of the norm reduction and the last-block counter live in one statically sized device
   array (64 KiB + the counter) inside the library instead of buffers made per handle.
   Limits and rules:
     - a must be FP64 and square; 1 <= nrhs <= NSF_NOALLOC_MAX_RHS, else NSF_ERR_INVALID_ARG;
     - the first call in a CUDA context (on each device, and again after cudaDeviceReset) looks
       the array up (cudaGetSymbolAddress); make that first call before any stream capture;
     - the counter starts at zero when the library is loaded and every completed call leaves it
       at zero; nothing else needs clearing between calls;
     - all calls on one device share the array: calls that overlap in time (other streams or
       host threads) race and give wrong norms.  Order them on one stream. */
int nsf_residual_noalloc(nsf_csr a, int nrhs, const double *x, const double *b, double *r, double *norms2,
                         void *stream);

/* =============================================== vector helpers (the cu:: call sites) ====== */
/* Device vectors of dtype (NSF_F32 / NSF_F64), asynchronous on stream.  They replace the cuBLAS
   calls and the small kernels around the reference's time step: cu::saxpy and cu::scale
   (cpp/libs/CudaUtils/include/cu/blas.h:24-26, used at chorinCuda.cu:275,298,354), the Dirichlet
   value scatter of DirichletVelocity::impose (chorinCuda.cu:59-74) and the internal-node gather /
   scatter of PressureSolver (chorinCuda.cu:109-150). */
/* y += alpha x (n entries) */
int nsf_axpy(long long n, double alpha, const void *x, void *y, int dtype, void *stream);
/* x *= alpha */
int nsf_scale(long long n, double alpha, void *x, int dtype, void *stream);
/* dst[i] = src[idx[i]], i < n (idx on the device) */
int nsf_gather(int n, const int *idx, const void *src, void *dst, int dtype, void *stream);
/* dst[idx[i]] = src[i], i < n (idx on the device) */
int nsf_scatter(int n, const int *idx, const void *src, void *dst, int dtype, void *stream);

/* ======================================================================== solvers ======= */

typedef struct nsf_solver_s *nsf_solver;

/* Linear solver on a square SPD CSR given on the host (FP64 values).
   method "gs": multicolor Gauss-Seidel iterated to an RMS residual target (the reference's
                "gs", cu::GaussSeidel, cpp/libs/CudaUtils/src/gaussSeidel.cu:121-404);
   method "pcg": CG preconditioned by symmetric multicolor Gauss-Seidel, stops at
                ||b - A x|| <= target * ||b||.
   precision NSF_PREC_MIXED runs the sweeps/CG in FP32 inside an FP64 refinement loop.
   Replaces cu::createSolver (cpp/libs/CudaUtils/src/solvers/solverFactory.cu:209-237) and the
   cu::AbstractSolver interface (cpp/libs/CudaUtils/include/cu/solvers/abstractSolver.h:8-32). */
int nsf_solver_create(const char *method, int numCh, int n, const int *rowStart, const int *col,
                      const double *values, int precision, int maxIters, double target, int checkInterval,
                      nsf_solver *out);
/* Solve A x = b for numCh planar channels; b and x are device FP64 vectors of numCh * n
   entries; x holds the initial guess on entry.  Synchronous: returns the solver status. */
int nsf_solver_solve(nsf_solver s, const double *b, double *x, void *stream);
/* Two-level preconditioner for a single-channel NSF_PREC_MIXED "pcg" solver: z = SGS(r) + P Ac^-1 P^T r
   with P the piecewise-constant prolongation of aggregates of rows -- square cells of about
   rowsPerAggregate rows of the coordinates xy (2 floats per row, the solver's row numbering), split by
   the thread-block-cluster CTA that owns the rows -- and Ac = P^T A P inverted densely.  The solve
   runs in the classical form of the cluster kernel; CG needs several times fewer iterations on
   Poisson-type systems.  NSF_ERR_NOT_SUPPORTED when the cluster-resident path, at least 3 colours
   or the shared memory are missing.  No counterpart in the reference (its pressure solve is GS or a
   direct factorisation, cpp/libs/CudaUtils/src/solvers/solverFactory.cu:221-234). */
int nsf_solver_set_coarse(nsf_solver s, const float *xy, int rowsPerAggregate);
/* The same with FP32 device vectors (widened to FP64 around the FP64 solve inside the library):
   the IO vectors of the reference's cu::AbstractSolver are FP32 cu::vec (getRhs / getSol,
   cpp/libs/CudaUtils/include/cu/solvers/abstractSolver.h:8-32).  Synchronous. */
int nsf_solver_solve_f32(nsf_solver s, const float *b, float *x, void *stream);
/* The same with host vectors (numCh * n doubles each; x holds the initial guess and receives the
   solution, also when the solve ends with a non-OK status).  Replaces the host wrappers
   cu::GaussSeidelHost::solve and cu::ConjGradHost::solve (cpp/libs/CudaUtils/src/gaussSeidelHost.cu,
   conjGradHost.cu) that the reference's solver test uses. */
int nsf_solver_solve_host(nsf_solver s, const double *b, double *x);
/* iters: iterations of the last solve; rms[numCh]: RMS residual per channel (getLastMse);
   rel[numCh]: relative residual per channel; any pointer may be NULL */
int nsf_solver_stats(nsf_solver s, int *iters, double *rms, double *rel);
int nsf_solver_set(nsf_solver s, int maxIters, double target, int checkInterval);
void nsf_solver_destroy(nsf_solver s);

/* ============================================== pure-Neumann Poisson: pin and zero mean ======= */

typedef struct nsf_neumann_s *nsf_neumann;

/* A symmetric positive semi-definite system whose null space is the constants (the P1 Laplacian of
   a domain with Neumann conditions everywhere, e.g. the standalone pressure-Poisson benchmark),
   made regular by one Dirichlet pin: row and column `pin` are removed and the rest is solved with
   the "pcg" solver of nsf_solver_create (multicolor SGS preconditioner; precision NSF_PREC_F64 or
   NSF_PREC_MIXED), to ||b' - A' x'|| <= target ||b'|| on the pinned system.  No counterpart in the
   reference (its pressure always has Dirichlet nodes on the outflow, buildContext.cpp:64-93): it
   is the pressure zero-mean / pin correction of the standalone solve, done on the device in FP64. */
int nsf_neumann_create(int n, const int *rowStart, const int *col, const double *values, int pin, int precision,
                       int maxIters, double target, nsf_neumann *out);
/* b, x: device FP64 vectors of n entries; x holds the initial guess.  On the device, in FP64: b is
   projected to zero mean (b - sum(b)/n), the pinned row dropped, the pinned system solved from x
   shifted to x[pin] = 0, the solution expanded with x[pin] = 0 and shifted to zero mean.
   Synchronous: returns the solver status. */
int nsf_neumann_solve(nsf_neumann h, const double *b, double *x, void *stream);
/* iterations and relative residual (of the pinned system) of the last solve; either may be NULL */
int nsf_neumann_stats(nsf_neumann h, int *iters, double *rel);
void nsf_neumann_destroy(nsf_neumann h);

/* ================================================================= Chorin stepper ======= */

typedef struct
{
    double nu;            /* viscosity */
    double tau;           /* time step */
    int precision;        /* nsf_precision */
    int velMethod;        /* mass solves. 0: "gs" (RMS target velTol, relative), 1: "pcg" with the
                             multicolor SGS preconditioner (relative velTol), 2: "pcg" with the
                             Jacobi preconditioner (no reference counterpart: the diagonally
                             scaled P2 mass matrix has condition number ~5.2 whatever h, and each
                             iteration is one parallel phase), 3: Chebyshev iteration with the
                             Jacobi preconditioner over the spectral bounds [0.39237, 2.05982] of
                             D^-1 M (those of every affine P2 element), the iteration count fixed
                             in advance from velTol (relative); one kernel per iteration, no
                             reductions but the final residual check; FP64, or double-float (float
                             pairs on the FP32 pipes) in NSF_PREC_MIXED; 4: the same started from
                             the previous step's solution of that solve, the count set on the
                             device from the initial residual (at most the count of 3); a channel
                             whose previous solution is no better a start than 0 starts cold */
    int velMaxIters;
    double velTol;
    int presMaxIters;
    double presTol;       /* relative pressure residual */
    int checkInterval;    /* eager mode: iterations between device->host convergence checks */
    int useGraph;         /* 1: capture the step once into a CUDA graph whose solver loops are
                             conditional while nodes (no host synchronisation); 0: eager */
    int maxOuter;         /* mixed precision: FP64 refinement passes per solve */
    double innerTol;      /* mixed precision: relative tolerance of each FP32 inner solve */
    int pressureGuess;    /* initial guess of the pressure solve: 0 the previous solution (as the
                             reference's solver keeps it), 1 the linear extrapolation
                             2 p(n-1) - p(n-2) from the last two solutions, 2 the projection of
                             the new solution onto up to pressureBasis earlier solutions,
                             orthonormal in the Kp_int inner product (Fischer 1998: x0 = sum_k
                             (x_k . b) x_k; each solve's correction joins the basis; a full basis
                             restarts from the solution and its last two differences).  1 and 2
                             have no reference counterpart: fewer iterations, the same tolerance */
    int pressureBasis;    /* pressureGuess 2: basis vectors, 3..256 (0: 250) */
} nsf_chorin_config;

typedef struct nsf_chorin_s *nsf_chorin;

/* Device-resident time stepper over a context: uploads the color-permuted operators once.
   Replaces the setup and loop body of solveNsChorinCuda
   (cpp/execs/NavierStokes/src/chorinCuda.cu:154-379). */
int nsf_chorin_create(nsf_context ctx, const nsf_chorin_config *cfg, nsf_chorin *out);
/* advance nSteps time steps on the stepper's stream (stream may be NULL: default stream) */
int nsf_chorin_step(nsf_chorin s, int nSteps, void *stream);
/* enqueue nSteps time steps (graph replays; needs useGraph = 1) and return without waiting, so
   several steppers can advance concurrently on their own streams; nsf_chorin_stats keeps the
   statistics of the last nsf_chorin_step.  No counterpart in the reference (its loop is
   synchronous); used to run independent flow instances side by side. */
int nsf_chorin_launch(nsf_chorin s, int nSteps, void *stream);
/* copy the state to/from host memory in the original numbering: u[2N] planar, p[P] */
int nsf_chorin_get_state(nsf_chorin s, double *u, double *p, void *stream);
int nsf_chorin_set_state(nsf_chorin s, const double *u, const double *p, void *stream);
/* Headless frame output: the state in the original numbering written as two vector files of the
   binary interchange format (nsf_io_*), u (2N planar) to uPath and p (P) to pPath (either may be
   NULL), values as dtype (NSF_F32 or NSF_F64).  Synchronous.  Replaces the solution frames that
   the reference's solver loop renders to images every few steps
   (cpp/execs/NavierStokes/src/navierStokes.cpp:85-119), keeping the fields instead of a picture. */
int nsf_chorin_dump(nsf_chorin s, const char *uPath, const char *pPath, int dtype, void *stream);
/* nsf_chorin_set_state with flags.  NSF_STATE_KEEP_HISTORY: the state continues the stepper's run
   (a host that reads the state, and writes it back, every step), so the pressure-guess history
   (pressureGuess 1 and 2: the earlier solutions) is kept; nsf_chorin_set_state starts a new one.
   The history only shapes the initial guess: the solves reach the same tolerance either way. */
#define NSF_STATE_KEEP_HISTORY 1
/* NSF_STATE_ASYNC: the copies from u and p and their renumbering are enqueued on the stream and the
   call returns at once; u and p must stay unchanged until the stream has passed them (from
   page-locked host memory the copy is asynchronous).  A host loop of set_state (async), a launched
   step and get_state on one stream then waits once per step, in get_state.  Without the flag the
   call returns when the state is set. */
#define NSF_STATE_ASYNC 2
int nsf_chorin_set_state_ex(nsf_chorin s, const double *u, const double *p, int flags, void *stream);
/* stats[0..7] of the last step: tentative iterations, pressure iterations, final iterations,
   pressure relative residual, tentative relative residual, final relative residual,
   pressure refinement sweeps (mixed), status */
int nsf_chorin_stats(nsf_chorin s, double *stats);
/* number of kernels this library launched since the process started */
long long nsf_kernel_launches(void);
void nsf_chorin_destroy(nsf_chorin s);

/* ===================================================================== packs of steppers == */

typedef struct nsf_pack_s *nsf_pack;

/* A pack: one CUDA graph whose branches are the time steps of n steppers (on one mesh or on meshes
   of different resolution), so that one graph launch advances every instance.  No counterpart in
   the reference (its loop drives one flow).  With n > 1 every stepper must keep its solves inside
   thread-block clusters (created with NSF_PCG_PATH=auto-cluster): concurrent branches on the
   whole-GPU cooperative grid could wait on each other's SMs.  The steppers must outlive the pack
   and must not be stepped through their own handles while a pack launch is in flight. */
int nsf_pack_create(const nsf_chorin *steppers, int n, nsf_pack *out);
/* A pack of batches (nsf_batch_create): one graph whose branches are the batched time steps, one
   branch per batch (e.g. one batch per mesh resolution), so one graph launch advances every
   instance of every batch with one kernel per operation and batch.  The batches must outlive the
   pack and must not be stepped through their own handles while a pack launch is in flight.
   Declared here, after nsf_batch. */
int nsf_pack_create_batches(struct nsf_batch_s *const *batches, int n, nsf_pack *out);
/* kernel launches of one pack step */
long long nsf_pack_kernels_per_step(nsf_pack p);
/* enqueue nSteps launches of the pack graph on stream (NULL: the pack's own stream); asynchronous */
int nsf_pack_step(nsf_pack p, int nSteps, void *stream);
void nsf_pack_destroy(nsf_pack p);

/* ================================================================== batched instances == */

typedef struct nsf_batch_s *nsf_batch;

/* nInst flows on the mesh of ctx, each with its own viscosity nu[q] and Dirichlet x values
   dirVx[q * nDir + i] (context dirIds order; NULL: the context's values for every instance),
   advanced together: every operation of the time step is one launch for all instances (the
   operators are read by the instances together, the pressure solves are one launch of nInst
   thread-block clusters).  Each instance computes exactly what an nsf_chorin stepper with the same
   configuration computes.  cfg: NSF_PREC_MIXED, velMethod 3, any pressureGuess (2: one basis per
   instance), presTol >= 1e-11;
   cfg->nu is ignored.  No counterpart in the reference (its loop, chorinCuda.cu:236-376, advances one
   flow): the many-instance workload of the parameter studies. */
int nsf_batch_create(nsf_context ctx, const nsf_chorin_config *cfg, int nInst, const double *nu, const double *dirVx,
                     nsf_batch *out);
/* advance every instance nSteps steps (graph replays when cfg->useGraph), then wait and keep the
   per-instance statistics; NSF_ERR_NONFINITE if a pressure residual became non-finite */
int nsf_batch_step(nsf_batch b, int nSteps, void *stream);
/* the same without waiting (statistics not updated) */
int nsf_batch_launch(nsf_batch b, int nSteps, void *stream);
/* state of instance inst in the original numbering: u[2N] planar, p[P]; synchronous */
int nsf_batch_get_state(nsf_batch b, int inst, double *u, double *p, void *stream);
/* set it (a new pressure history for that instance); synchronous */
int nsf_batch_set_state(nsf_batch b, int inst, const double *u, const double *p, void *stream);
/* stats[0..3] of instance inst after the last nsf_batch_step: pressure CG iterations, pressure
   relative residual, residual replacements, status */
int nsf_batch_stats(nsf_batch b, int inst, double *stats);
/* kernel launches of one captured batch step (0 before the first graph step) */
long long nsf_batch_kernels_per_step(nsf_batch b);
void nsf_batch_destroy(nsf_batch b);

/* ========================================================= force functional (drag/lift) == */

typedef struct nsf_forces_s *nsf_forces;

/* Force of the flow on the border group `group` of mesh ("Circle": the cylinder), evaluated on the
   state of stepper s (created from a context of the same mesh; s must outlive the handle):
     F = sum over the group's edges of integral ( -p n + nu du/dn ) ds,
   n the unit edge normal pointing into the fluid, u the P2 velocity and p the P1 pressure of the
   adjacent triangle, 2-point Gauss-Legendre per edge, FP64.  forces[0] = F_x (drag),
   forces[1] = F_y (lift).  No counterpart in the reference: the DFG benchmark's continuum
   definition in stress form with the velocity gradient, for the drag/lift time series. */
int nsf_forces_create(nsf_mesh mesh, nsf_chorin s, const char *group, nsf_forces *out);
/* onDevice == 0: forces is a host array of 2 doubles and the call synchronises the stream;
   otherwise a device array written asynchronously on stream (NULL: the stepper's stream) */
int nsf_forces_eval(nsf_forces f, double *forces, int onDevice, void *stream);
void nsf_forces_destroy(nsf_forces f);

/* ============================================ parameters and discrete adjoint (gradients) == */
/* None of these has a counterpart in the reference (it has no adjoint and fixes the inflow and
   the viscosity for a run). */

/* Replace the x values of the Dirichlet velocity nodes (one per node, in the context's dirIds
   order; the y values stay 0) and impose them on the current state.  Synchronous. */
int nsf_chorin_set_dirichlet(nsf_chorin s, const double *dirVx, void *stream);
/* Change the viscosity of the following steps (a captured step is captured again). */
int nsf_chorin_set_nu(nsf_chorin s, double nu);
/* M x = b with the stepper's mass solve (velMethod 3: Chebyshev-Jacobi with the a priori count for
   the relative tolerance tol; double-float iterations on an NSF_PREC_MIXED stepper), b and x device
   FP64, planar 2 * N in the stepper's (colour-permuted) numbering, x overwritten; iters (may be
   NULL): the iterations run.  Synchronous.  The solve uses the work buffers of the stepper's
   tentative mass solve: it must not overlap steps of the same stepper, and it replaces that solve's
   statistics until the next step.  The solve of chorinCuda.cu:265-266 on its own (the bench times
   its iterations with it). */
int nsf_chorin_mass_solve(nsf_chorin s, const double *b, double *x, double tol, int *iters, void *stream);

typedef struct
{
    int checkpointInterval; /* steps between stored states; the reverse sweep recomputes each
                               segment from its checkpoint.  0: keep every state (no recomputation) */
    int maxIters;           /* cap of each adjoint CG solve (<= 0: 20000) */
    double tol;             /* relative residual of each adjoint CG solve (<= 0: 1e-13) */
    int snapshots;          /* > 0: binomial checkpointing instead (checkpointInterval ignored):
                               at most this many stored states besides the initial one, placed by
                               the schedule that minimises the recomputed steps for that memory
                               (Griewank's binomial checkpointing, as in revolve); 0: off */
} nsf_adjoint_config;

typedef struct nsf_adjoint_s *nsf_adjoint;

/* Discrete adjoint of an FP64 stepper's time step for the force functional of f (created on s):
     J = sum_{n=1..nSteps} wDrag[n-1] F_x(u_n, p_n) + wLift[n-1] F_y(u_n, p_n),
   u_n, p_n the state after step n.  Every linear solve of the step is taken as exact; the adjoint
   mass and pressure solves are CG with the multicolor SGS preconditioner on the stepper's systems
   (both symmetric); on an NSF_PREC_F64_MIXEDSOLVE stepper they are FP32 CG inside FP64 refinement,
   to the same tolerance, and a refinement solve that used up its passes (the FP64 residual floor of
   a tight tolerance) is reported in the stats, not as an error.  cfg may be NULL (defaults). */
int nsf_adjoint_create(nsf_chorin s, nsf_forces f, const nsf_adjoint_config *cfg, nsf_adjoint *out);
/* Run nSteps steps forward from the stepper's current state (whose Dirichlet rows hold the
   Dirichlet values), then the reverse sweep.  wDrag / wLift: nSteps host weights (NULL = 0).
   result[0] = J, result[1] = dJ/dnu; dJdDir (may be NULL): dJ/d(Dirichlet x value), one per
   Dirichlet node in dirIds order, through the initial state and every step; dJdU0 (may be NULL):
   dJ/du0 in the original numbering, planar [x(N); y(N)], 0 on the Dirichlet rows.  The stepper
   ends in the state after the nSteps steps.  Synchronous. */
int nsf_adjoint_run(nsf_adjoint a, int nSteps, const double *wDrag, const double *wLift, double *result,
                    double *dJdDir, double *dJdU0, void *stream);
/* stats[0..9] of the last run: forward steps, recomputed steps, reverse steps, adjoint mass CG
   iterations (summed over channels and solves), adjoint pressure CG iterations, worst forward solver
   status, worst adjoint solver status, bytes of stored states, forward ms, reverse-sweep ms
   (CUDA events on the run's stream; the reverse sweep includes the recomputation) */
int nsf_adjoint_stats(nsf_adjoint a, double *stats);
void nsf_adjoint_destroy(nsf_adjoint a);

#ifdef __cplusplus
}
#endif

#endif
