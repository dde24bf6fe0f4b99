/*
 * emfa_cuda.h -- C ABI of libemfa_cuda.so, the GB300 (sm_103a) implementation
 * of the surface-integral-equation hot path of xiangwei0909/EMFA: EFIE/CFIE
 * RWG impedance fill, excitation, dense and MLFMA matrix-vector products, the
 * GMRES/BiCGStab iterations that drive them, and the bistatic/monostatic RCS
 * far-field reduction.
 *
 * Plain C: opaque handles, plain pointers and sizes, an emfa_status_t return
 * on every call (no exceptions cross the boundary), and an explicit CUDA
 * stream (passed as void*, a cudaStream_t; NULL = the context's stream).
 * "dev" pointers are device memory, "host" pointers host memory.  Complex
 * arrays are interleaved (re, im): complex64 for EMFA_F32, complex128 for
 * EMFA_F64.  Vectors of several right-hand sides are stored RHS-major:
 * element (r, u) at r * n + u.
 *
 * Each entry point names the reference interface it replaces (file:line in
 * the reference project).
 */
#ifndef EMFA_CUDA_H
#define EMFA_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EMFA_OK = 0,
    EMFA_ERR_INVALID = 1,       /* bad argument; reference: component::ConfigInvalid */
    EMFA_ERR_CUDA = 2,          /* CUDA runtime error; reference: std::runtime_error */
    EMFA_ERR_OOM = 3,           /* device allocation refused (HBM budget)            */
    EMFA_ERR_NOT_CONVERGED = 4, /* Krylov iteration cap reached (reference logs a warning) */
    EMFA_ERR_MESH = 5,          /* mesh not usable; reference: component::FileError  */
    EMFA_ERR_UNSUPPORTED = 6,
    EMFA_ERR_TIMEOUT = 7        /* a device-side wait gave up                        */
} emfa_status_t;

typedef enum { EMFA_F32 = 0, EMFA_F64 = 1 } emfa_precision_t;
typedef enum { EMFA_EFIE = 0, EMFA_CFIE = 1 } emfa_kind_t;
/* EMFA_LU: dense only (emfa_solve, EMFA_F32): FP32 LU of Z (row exchanges
 * within 64-row diagonal blocks; trailing updates on the tensor cores with
 * split-FP16 operands, about 2^-21 of the largest product term), then FP64
 * iterative refinement on the true residual, GMRES-IR if the refinement
 * stalls.  No counterpart in the reference, whose dense solves are iterative
 * (EMSolver/EFIE.cpp:89 has a commented-out Eigen LU). */
typedef enum { EMFA_GMRES = 0, EMFA_BICGSTAB = 1, EMFA_LU = 2 } emfa_method_t;
typedef enum {
    EMFA_MV_AUTO = 0,  /* F64: FP64 SIMT; F32: EMFA_MV_F16X                          */
    EMFA_MV_F64 = 1,   /* FP64 complex GEMM on CUDA cores (plain path)               */
    EMFA_MV_F32 = 2,   /* FP32 complex GEMM on CUDA cores; residual FP32 products    */
                       /* with FP64 chunk sums                                       */
    EMFA_MV_TF32 = 3,  /* tcgen05 TF32 complex GEMM, FP32 accumulation; residual as  */
                       /* EMFA_MV_F32                                                */
    EMFA_MV_F16X = 4   /* tcgen05 split FP16: Z = (Zh + Zl)/s once per solve; inner  */
                       /* product Zh x at the FP16 rate (TF32 accuracy); residual    */
                       /* Zh xh + Zh xl + Zl xh per 64-column block, compensated     */
                       /* FP32 sums across blocks, B - Z x formed in FP64            */
} emfa_matvec_t;

/* Discretisation of the EFIE fill.  EMFA_DISC_REFERENCE: the reference's own,
 * 3 x 3-point regular pairs and singularity extraction on self pairs only
 * (EMSolver/EFIE.cpp:139-160,231-542,655-662).  EMFA_DISC_CONFIG: the
 * discretisation the benchmark configurations state, 7 x 7-point regular
 * pairs and singularity extraction on self and edge-adjacent triangle pairs
 * (closed-form potential integrals for points on or off the source plane);
 * EFIE only.  No counterpart in the reference. */
typedef enum { EMFA_DISC_REFERENCE = 0, EMFA_DISC_CONFIG = 1 } emfa_discretisation_t;

typedef struct emfa_ctx emfa_ctx_t;
typedef struct emfa_geom emfa_geom_t;
typedef struct emfa_mlfma emfa_mlfma_t;

/* Fill parameters: one frequency, one formulation.  Mirrors the members the
 * reference solvers take from ConfigLoader (EMSolver/EFIE.cpp:25-52,
 * EMSolver/CFIE.cpp:25-51). */
typedef struct {
    int kind;           /* emfa_kind_t                                              */
    int precision;      /* EMFA_F32: FP32 regular pairs + FP64 singular self terms; */
                        /* EMFA_F64: everything FP64 (the plain path)               */
    double freq;        /* Hz; k = 2 pi f / c0 in the fill's precision              */
    double alpha;       /* CFIE combination coefficient (alpha:)                    */
    double sigma_re;    /* EFIE surface-impedance term (Sigma:), 0 for PEC          */
    double sigma_im;
    int edm_mode;       /* EFIE pairs farther than 3 lambda: 0 = zero, as in the    */
                        /* matrix the reference solves; 1 = equivalent-dipole value;*/
                        /* 2 = ordinary quadrature (no far-pair branch)             */
    int discretisation; /* emfa_discretisation_t; 0 is the reference's              */
} emfa_fill_params_t;

typedef struct {
    int method;         /* emfa_method_t                                            */
    int restart;        /* GMRES restart length m, 1..255 (reference: 30)           */
    int max_iter;       /* cap on inner iterations per right-hand side              */
    double tol;         /* stop when ||b - Z x|| / ||b|| < tol (or absolute, below) */
    int tol_absolute;   /* 1: ||b - Z x|| < tol, the reference GMRES criterion      */
    int matvec;         /* emfa_matvec_t                                            */
    int max_refine;     /* outer true-residual cycles for EMFA_F32 (GMRES-IR)       */
    int orth;           /* GMRES Gram-Schmidt: 0 = auto (CGS1 for the EMFA_F32     */
                        /* inner solve of the refinement, CGS2 for EMFA_F64),      */
                        /* 1 = CGS1, 2 = CGS2, 3 = CGS1 in separate passes (the    */
                        /* FP32 CGS1 step is otherwise one fused launch for        */
                        /* restarts up to 32, N up to 16384 and n_rhs x ceil(N /   */
                        /* 1024) (at most 8) up to 4 x the SM count), 4 = CGS1     */
                        /* fused whatever n_rhs (restart and N as for 1)           */
    double inner_reduction; /* GMRES refinement with reduced-precision products:  */
                        /* a cycle's inner steps stop once the implicit residual   */
                        /* falls below this fraction of the cycle's starting true  */
                        /* residual, or below the target; 0 = the operator's       */
                        /* default (1e-2 for the tensor-core dense products),      */
                        /* < 0 = iterate to the target                             */
    int basis;          /* GMRES basis storage of the EMFA_F32 inner solve: 0 =    */
                        /* auto (FP16 where the Gram-Schmidt passes run separately */
                        /* and the product packs its operand to FP16, else FP32),  */
                        /* 1 = FP32, 2 = FP16 where possible.  The FP16 basis is   */
                        /* the product's own operand (each vector scaled by a      */
                        /* power of two), so the orthogonalisation sees the        */
                        /* vectors the product multiplied, at half the bytes       */
} emfa_solver_params_t;

typedef struct {
    int iterations;         /* inner iterations performed (max over RHS)            */
    int cycles;             /* outer (restart / refinement) cycles                  */
    int converged;          /* number of RHS that met the tolerance                 */
    double max_rel_residual;/* max over RHS of the last true residual ||b-Zx||/||b||*/
    double seconds;         /* device time of the solve                             */
} emfa_solve_info_t;

/* ---- status and context -------------------------------------------------- */
const char* emfa_status_string(emfa_status_t s);
/* Last error message recorded on ctx (or the process-wide one if ctx NULL). */
const char* emfa_last_error(const emfa_ctx_t* ctx);
const char* emfa_version(void);

/* Creates a context on a CUDA device with an HBM budget (0 = unlimited).
 * Replaces the per-solver resource set-up of EM::init (EMSolver/EM.cpp:24-67)
 * and the MLFMA ThreadPool::init (EMComponent/ThreadPool.cpp:19-29). */
emfa_status_t emfa_ctx_create(int device, size_t hbm_budget_bytes, emfa_ctx_t** out);
emfa_status_t emfa_ctx_destroy(emfa_ctx_t* ctx);
/* Bytes currently held / peak / budget. */
emfa_status_t emfa_ctx_memory(const emfa_ctx_t* ctx, size_t* used, size_t* peak, size_t* budget);
/* Kernels launched through this context since creation. */
emfa_status_t emfa_ctx_launch_count(const emfa_ctx_t* ctx, int64_t* count);
emfa_status_t emfa_ctx_synchronize(emfa_ctx_t* ctx);
/* The context's own CUDA stream (a cudaStream_t), used when a call gets NULL. */
emfa_status_t emfa_ctx_stream(const emfa_ctx_t* ctx, void** stream);

/* Per-kernel timing (the time log of EM::reportTimeInfo, EMSolver/EM.cpp:85-89,
 * at kernel granularity).  While on, every launch of the kernels below is
 * bracketed by a pair of CUDA events on its own stream; turning it on or off
 * clears the records.  emfa_ctx_kernel_time waits for the recorded launches
 * and returns their count, summed device time and summed algorithmic work
 * (work may be NULL): FLOPs for the products (8 n^2 per right-hand side of a
 * complex product), Z entries for the fill. */
typedef enum {
    EMFA_KT_FILL_Z = 0,    /* impedance fill (EFIE/CFIE)                       */
    EMFA_KT_GEMM = 1,      /* tensor-core inner product of the solvers        */
    EMFA_KT_RESIDUAL = 2   /* accurate refinement residual b - Z x             */
} emfa_kernel_timer_t;
emfa_status_t emfa_ctx_set_kernel_timing(emfa_ctx_t* ctx, int on);
emfa_status_t emfa_ctx_kernel_time(emfa_ctx_t* ctx, int kernel, int64_t* launches, double* total_ms,
                                   double* work);

/* Device buffers charged to the context's HBM budget, for callers without
 * CUDA runtime bindings of their own (the C++ front end, FFI users).
 * kind: 0 host->device, 1 device->host, 2 device->device; synchronous. */
emfa_status_t emfa_device_alloc(emfa_ctx_t* ctx, size_t bytes, void** dev);
emfa_status_t emfa_device_free(emfa_ctx_t* ctx, void* dev);
emfa_status_t emfa_memcpy(emfa_ctx_t* ctx, void* dst, const void* src, size_t bytes, int kind);

/* ---- geometry ------------------------------------------------------------- */
/* RWG table of a closed or open triangle mesh, host only (no GPU).  Rows of 6
 * ints: v1 v2 vxp vxm tp tm, in the reference's order and orientation.
 * Replaces CommonEdge::buildCommonEdge (EMComponent/CommonEdge.cpp:74-106,
 * 704-743).  Returns EMFA_ERR_INVALID if capacity rows are too few. */
emfa_status_t emfa_build_rwg(const int* tris_host, int n_tri, int* rwg_host, int capacity, int* n_rwg);

/* Uploads a mesh and its RWG table (host arrays: verts V x 3 double, tris
 * T x 3 int 0-based, rwg N x 6 int).  Replaces the Mesh / CommonEdge members
 * the solvers own (EMSolver/EFIE.h:69-70). */
emfa_status_t emfa_geom_create(emfa_ctx_t* ctx, const double* verts_host, int n_vert, const int* tris_host,
                               int n_tri, const int* rwg_host, int n_rwg, emfa_geom_t** out);
emfa_status_t emfa_geom_destroy(emfa_geom_t* geom);
emfa_status_t emfa_geom_size(const emfa_geom_t* geom, int* n_vert, int* n_tri, int* n_rwg);

/* ---- fill ------------------------------------------------------------------ */
/* Dense impedance matrix, row-major N x N (row = testing RWG f, column =
 * source RWG s) with leading dimension ldz (elements).  Replaces
 * EFIE::fillZ (EMSolver/EFIE.cpp:603-696) and CFIE::fillZ
 * (EMSolver/CFIE.cpp:485-568) with their pair kernels (EFIE.cpp:139-566,
 * EMSolver/Miscellaneous.cpp:6-77). */
emfa_status_t emfa_fill_z(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p, void* Z_dev,
                          size_t ldz, void* stream);

/* Excitation for n_inc plane waves given as (theta, phi, pole) degrees
 * triples (host array), V is n_inc x N.  Replaces EFIE::fillV / eVKernel
 * (EMSolver/EFIE.cpp:568-601,698-722) and CFIE::fillV / cfieVKernel
 * (EMSolver/CFIE.cpp:570-597, EMSolver/Miscellaneous.cpp:152-189), with the
 * incidence vectors of EM::init (EMSolver/EM.cpp:33-38). */
emfa_status_t emfa_fill_v(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p,
                          const double* angles_host, int n_inc, void* V_dev, void* stream);

/* ---- dense products and solvers -------------------------------------------- */
/* Y = Z X for n_rhs vectors (X, Y are n_rhs x n).  Z in precision prec; the
 * vectors are complex128 for EMFA_F64 and complex64 for EMFA_F32.  Replaces
 * the dense products `_A * p1` of iml::BICGSTAB / iml::GMRES
 * (EMIterative/iml.cpp:22,29,186). */
emfa_status_t emfa_matvec(emfa_ctx_t* ctx, int prec, int matvec, const void* Z_dev, int n, const void* X_dev,
                          int n_rhs, void* Y_dev, void* stream);

/* Tile-shape autotuner of the split-FP16 inner product (EMFA_MV_F16X, the
 * mixed dense solver's products).  The first product of a shape bucket
 * (device, ceil(n / 256), ceil(2 n_rhs / 16)) in the process times each
 * candidate tile shape twice with CUDA events on the caller's stream and keeps
 * the fastest for the bucket; every shape gives the same bits.  Shapes:
 * 0 = 64 columns x 128 rows, 1 = 64 x 256, 2 = 144 x 128, 3 = 144 x 256.
 * emfa_autotune_query gives the bucket's choice (-1: not tuned yet) and, in
 * ms[4], the best time of each shape (-1: not a candidate).
 * emfa_autotune_clear forgets every choice.  EMFA_AUTOTUNE=0 in the
 * environment keeps the fixed rule instead (256 x 144 tiles once they fill the
 * SMs).  No counterpart in the reference. */
emfa_status_t emfa_autotune_query(int device, int n, int n_rhs, int* shape, float* ms);
emfa_status_t emfa_autotune_clear(void);

/* Largest n * n_rhs accepted by emfa_matvec_tf32_noalloc (16 MiB of scratch). */
#define EMFA_NOALLOC_MAX_ELEMS 1048576u

/* Y = Z X exactly as emfa_matvec(ctx, EMFA_F32, EMFA_MV_TF32, ...) computes it
 * (complex64 Z row-major n x n, X and Y n_rhs x n, device pointers, Z 16-byte
 * aligned, n even), but the call allocates no device memory: no cudaMalloc,
 * no cudaFree, no allocating library routine.  No counterpart in the
 * reference, which has no device code.
 *
 * Who needs it: a caller whose device memory is all handed out by its own
 * pool (so a library allocation would fail or evict), or a serving loop that
 * shares the GPU with other streams, where cudaFree would synchronise the whole
 * device and stall them.  It needs no context either.
 *
 * Scratch: one fixed static device array per device, sized for
 * n * n_rhs <= EMFA_NOALLOC_MAX_ELEMS; larger products return
 * EMFA_ERR_INVALID with a message saying so (use emfa_matvec for them).
 * The first call on a device, made with that device current, looks the array
 * up and sets the kernels' shared-memory limit; make that first call before
 * any stream capture.  With lazy module loading (the CUDA default) that first
 * call is also when the driver loads this part of the library's device code
 * on the device and reserves the array (16 MiB and one 256-byte line); the
 * array then stays reserved until the process exits, and later calls reserve
 * nothing.  Calls on one device share the array, so two calls that overlap in
 * time (different streams, or different host threads) race and corrupt each
 * other's result: order them.  stream NULL is the default stream; every call
 * copies the kernel's error word to host memory and synchronises `stream`
 * before it returns.  Errors are reported through emfa_last_error(NULL). */
emfa_status_t emfa_matvec_tf32_noalloc(const void* Z_dev, int n, const void* X_dev, int n_rhs, void* Y_dev,
                                       void* stream);

/* R = B - Z X, the accurate residual of mixed-precision iterative refinement,
 * with the residual product of the given matvec mode (EMFA_F32: Z complex64,
 * B complex64; EMFA_F64: Z and B complex128; X and R always complex128,
 * n_rhs x n).  Replaces the residual `r = b - A * x` of iml::BICGSTAB and
 * iml::GMRES (EMIterative/iml.cpp:8,173). */
emfa_status_t emfa_residual(emfa_ctx_t* ctx, int prec, int matvec, const void* Z_dev, int n, const void* X_dev,
                            const void* B_dev, int n_rhs, void* R_dev, void* stream);

/* Solves Z X = B for n_rhs right-hand sides (B complex64 for EMFA_F32,
 * complex128 for EMFA_F64; X always complex128, n_rhs x n).  GMRES(m) or
 * BiCGStab, all right-hand sides in lockstep with one multi-RHS product per
 * step.  For EMFA_F32 the inner products run in reduced precision and each
 * restart recomputes the true residual (iterative refinement); Arnoldi,
 * Givens rotations and norms are FP64.  Replaces iml::GMRES
 * (EMIterative/iml.cpp:156-207) and iml::BICGSTAB (EMIterative/iml.cpp:3-39). */
emfa_status_t emfa_solve(emfa_ctx_t* ctx, int prec, const void* Z_dev, int n, const void* B_dev, int n_rhs,
                         void* X_dev, const emfa_solver_params_t* sp, emfa_solve_info_t* info, void* stream);

/* ---- far field -------------------------------------------------------------- */
/* RCS in dBsm for currents I (complex128, n_rhs x N) and scattering
 * directions (host, unit vectors).  per_rhs_dirs = 0: dirs is n_dir x 3,
 * shared by all RHS (bistatic); 1: dirs is n_rhs x n_dir x 3 (e.g. the
 * monostatic direction of each incidence).  out_host is n_rhs x n_dir.
 * Replaces EFIE::getBiRCS (EMSolver/EFIE.cpp:788-832), CFIE::getBiRCS
 * (EMSolver/CFIE.cpp:643-685) and MLFMA::getBiRCS (EMSolver/MLFMA.cpp:1573-1620)
 * as called by Result::getBistaticRCS / getMonostaticRCS
 * (EMComponent/Result.h:47-155). */
emfa_status_t emfa_rcs(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_fill_params_t* p, const void* I_dev,
                       int n_rhs, const double* dirs_host, int n_dir, int per_rhs_dirs, double* out_host,
                       void* stream);

/* ---- MLFMA ------------------------------------------------------------------- */
/* Multilevel fast multipole CFIE operator.  Replaces MLFMA::init / solve
 * (EMSolver/MLFMA.cpp:23-106): octree and box order (MLFMA.cpp:688-875,
 * MLFMA_Boundary.cpp:15-35), multipoles and interpolation (MLFMA.cpp:877-1002),
 * translation / radiation / receive operators (MLFMA.cpp:1133-1292), near
 * field (MLFMA.cpp:1004-1131) and the mat-vec (MLFMA.cpp:454-686).  Vectors
 * of emfa_mlfma_apply / _fill_v / _solve are in box order (the reference's
 * own unknown order); emfa_mlfma_unpermute maps currents back to RWG order. */
typedef struct {
    double freq;           /* Hz                                                     */
    double alpha;          /* CFIE combination (alpha:)                              */
    double box_threshold;  /* finest box side in wavelengths (mlfma_box_threshold:)  */
    int precond;           /* 1: build the SAI preconditioner (preconditioning:) and  */
                           /* solve P Z x = P b (MLFMA::calculatePreconditioner,      */
                           /* EMSolver/MLFMA.cpp:1294-1391, applied at :407-408,506)  */
    double row_threshold;  /* SAI rows / columns: near unknowns whose centre lies     */
    double col_threshold;  /* within this many finest-box lengths of the box centre   */
                           /* (row_threshold:, col_threshold:; MLFMA.cpp:719-720)     */
    int truncation;        /* multipoles per level from kd = sqrt(3) k box side:      */
                           /* 0 = the reference's int(kd + 6 kd^(1/3))                */
                           /* (MLFMA::getMultipoleNumber, MLFMA.cpp:877-881);         */
                           /* 1 = the configuration's int(kd + 1.8 d0^(2/3) kd^(1/3)) */
                           /* with d0 = 3 digits (no counterpart in the reference)    */
} emfa_mlfma_params_t;

/* Host only (no GPU): the octree plan the operator is built on -- finest
 * level number, boxes per level (level_cap >= levels + 1), multipoles per
 * level 2..L and the box-order permutation (N ints).  MLFMA::init and
 * levelRootsAndWeights (EMSolver/MLFMA.cpp:23-65,688-915). */
emfa_status_t emfa_mlfma_plan(const double* verts_host, int n_vert, const int* rwg_host, int n_rwg,
                              const emfa_mlfma_params_t* p, int* levels, int* level_boxes, int level_cap, int* poles,
                              int* perm);
emfa_status_t emfa_mlfma_create(emfa_ctx_t* ctx, emfa_geom_t* geom, const emfa_mlfma_params_t* p,
                                emfa_mlfma_t** out);
emfa_status_t emfa_mlfma_destroy(emfa_mlfma_t* mlfma);
/* levels = finest level number L (levels 0..L); level_boxes (L+1 ints), poles
 * (L-1 ints, levels 2..L) and perm (N ints: box position -> RWG index) are
 * optional outputs. */
emfa_status_t emfa_mlfma_info(const emfa_mlfma_t* mlfma, int* levels, int* level_boxes, int* poles,
                              size_t* near_nnz, int* perm);
/* y = Z x, complex64, n_rhs vectors of N in box order (MLFMA::matrixVectorMultiply). */
emfa_status_t emfa_mlfma_apply(emfa_mlfma_t* mlfma, const void* x_dev, void* y_dev, int n_rhs, void* stream);
/* One vector, one part of the operator: part 1 = near field only (nearZ_ * x),
 * 2 = far field only (the multipole stages), 0 = both.  For diagnostics. */
emfa_status_t emfa_mlfma_apply_part(emfa_mlfma_t* mlfma, const void* x_dev, void* y_dev, int part, void* stream);
/* CFIE excitation in box order, complex64 (MLFMA::fillVbyBox, MLFMA.cpp:1536-1571). */
emfa_status_t emfa_mlfma_fill_v(emfa_mlfma_t* mlfma, const double* angles_host, int n_inc, void* V_dev,
                                void* stream);
/* GMRES or BiCGStab on the MLFMA operator (MLFMA::iterativeSolve, MLFMA.cpp:402-452);
 * B complex64, X complex128, box order. */
emfa_status_t emfa_mlfma_solve(emfa_mlfma_t* mlfma, const void* B_dev, int n_rhs, void* X_dev,
                               const emfa_solver_params_t* sp, emfa_solve_info_t* info, void* stream);
/* The SAI preconditioner of an operator created with precond = 1: P in CSR
 * over box-order rows (ptr n+1 ints, col and val nnz entries, val complex64);
 * with ptr_host NULL only nnz is returned (0 without a preconditioner). */
emfa_status_t emfa_mlfma_precond_csr(const emfa_mlfma_t* mlfma, size_t* nnz, int* ptr_host, int* col_host,
                                     void* val_host);
/* Its per-box lists: rows and columns (box-order unknowns, CSR by box) and the
 * position of the box's own unknowns in its rows; NULL arrays: sizes only. */
emfa_status_t emfa_mlfma_precond_lists(const emfa_mlfma_t* mlfma, int* nbox, size_t* nrows, size_t* ncols,
                                       int* rptr, int* rows, int* cptr, int* cols, int* own);
/* X_rwg[r][perm[u]] = X_box[r][u], complex128. */
emfa_status_t emfa_mlfma_unpermute(emfa_mlfma_t* mlfma, const void* X_box_dev, int n_rhs, void* X_rwg_dev,
                                   void* stream);

/* ---- end to end ------------------------------------------------------------- */
/* One dense RCS job from host buffers: RWG table, upload, fill, excitation for
 * n_inc incidences, multi-RHS solve, RCS.  rcs_dirs_host/per_rhs_dirs as in
 * emfa_rcs; rcs_out_host is n_inc x n_dir dBsm; I_out_host (optional,
 * complex128 n_inc x N) receives the currents.  This is what
 * solver::invoke_solver<EFIE|CFIE> (EMSolver/Solver.h:20-29) runs:
 * init -> solve -> output.  The job's matrix, excitation and currents stay
 * in the context's workspace after the call (reused by the next job, released
 * with the context; emfa_ctx_memory counts them). */
emfa_status_t emfa_dense_rcs(emfa_ctx_t* ctx, const double* verts_host, int n_vert, const int* tris_host,
                             int n_tri, const emfa_fill_params_t* fp, const double* angles_host, int n_inc,
                             const emfa_solver_params_t* sp, const double* rcs_dirs_host, int n_dir,
                             int per_rhs_dirs, double* rcs_out_host, double* I_out_host,
                             emfa_solve_info_t* info);

/* Diagnostics: sin and cos of pi*x as the FP32 fill evaluates them (its own
 * Taylor-series evaluation), for accuracy tests; n device floats in and out. */
emfa_status_t emfa_diag_sincospi(const float* x_dev, int n, float* s_dev, float* c_dev, void* stream);
/* Diagnostics: the bounded wait of the tensor-core pipelines on a barrier
 * that nothing arrives on, with a 1 ms limit: returns EMFA_ERR_TIMEOUT and
 * *code_out = 42 (the stage code it recorded); the context stays usable.
 * No counterpart in the reference (it has no device code). */
emfa_status_t emfa_diag_wait_timeout(emfa_ctx_t* ctx, int* code_out);

/* ---- binary dumps ------------------------------------------------------------ */
/* Versioned binary dump of a matrix or vector (Z, V, I, operator arrays):
 * a 128-byte header (magic "EMFADUMP", version, dtype, rows, cols,
 * frequency, name, payload size, FNV-1a hash) and the row-major payload.
 * Replaces the Armadillo ASCII dumps of EFIE::writeZIVData
 * (EMSolver/EFIE.cpp:932-950) and CFIE::writeZIVData (EMSolver/CFIE.cpp:797-812).
 * dtype: 1 complex64, 2 complex128, 3 float32, 4 float64, 5 int32.
 * data_on_device: 1 when data is device memory.  Loading checks the header
 * and the payload hash and refuses a destination smaller than the payload. */
emfa_status_t emfa_dump_save(const char* path, const char* name, int dtype, size_t rows, size_t cols, double freq,
                             const void* data, int data_on_device);
emfa_status_t emfa_dump_info(const char* path, char* name_out /* 24 bytes */, int* dtype, size_t* rows,
                             size_t* cols, double* freq);
emfa_status_t emfa_dump_load(const char* path, void* data, size_t capacity_bytes, int data_on_device);

/* ---- batched and served RCS solves ---------------------------------------- */
/* Many independent RCS problems on one GPU.  No counterpart in the reference,
 * which solves one problem per process run (solver::loadSolver,
 * EMSolver/Solver.cpp:45-95).
 *
 * A request is a host mesh plus what to solve.  The engine keeps `lanes`
 * worker lanes, each a host thread with its own context and CUDA stream, so
 * the fills, products and solves of different problems overlap on the
 * device.  Admission: a request becomes visible at its arrival time (all at
 * once when realtime = 0); a free lane takes the oldest visible request whose
 * estimated device memory fits in what the running requests leave of
 * hbm_budget, else the oldest one that fits, so a large request does not
 * block small ones.  Dense CFIE/EFIE with split-FP16 refinement below
 * dense_max unknowns, MLFMA (CFIE, box order) above.  Each problem's
 * operators and Krylov state stay on its lane's device memory until it
 * finishes.  Device memory is stream-ordered per lane (no device-wide
 * synchronisation between lanes). */
typedef struct {
    const double* verts;      /* host, n_vert x 3 */
    int n_vert;
    const int* tris;          /* host, n_tri x 3, 0-based */
    int n_tri;
    int kind;                 /* EMFA_EFIE or EMFA_CFIE                                   */
    int method;               /* 0 auto (dense below dense_max), 1 dense, 2 MLFMA         */
    double freq, alpha;       /* Hz; CFIE combination coefficient                         */
    const double* angles;     /* host, n_inc x (theta, phi, pole) degrees                 */
    int n_inc;
    const double* rcs_dirs;   /* host unit vectors, n_dir x 3 (or n_inc x n_dir x 3)      */
    int n_dir;
    int per_rhs_dirs;
    double tol;               /* relative residual target; 0 = 1e-6 dense CFIE, 1e-5 dense */
                              /* EFIE (GMRES(250)), 1e-3 MLFMA                           */
    int max_iter;
    double box_threshold;     /* MLFMA finest box size in wavelengths                     */
    double arrival_s;         /* seconds after the run starts (realtime mode)             */
    double* rcs_out;          /* host, n_inc x n_dir dBsm, written when the request ends   */
} emfa_request_t;

typedef struct {
    int status;               /* emfa_status_t of the request                            */
    int method;               /* 1 dense, 2 MLFMA                                         */
    int n_rwg;
    int iterations;
    int converged;            /* right-hand sides that met tol                           */
    double max_rel_residual;
    double t_arrive, t_start, t_done;  /* seconds from the run start                      */
    size_t hbm_estimate;      /* bytes the admitter charged                              */
    int lane;
} emfa_request_result_t;

typedef struct {
    int lanes;                /* worker lanes (streams); 0 = 6                            */
    size_t hbm_budget;        /* admission budget in bytes; 0 = 150 GB                    */
    int dense_max;            /* largest dense problem (unknowns); 0 = 10000              */
    int realtime;             /* 1: honour arrival_s on the host clock                   */
    double max_wait_s;        /* a request that has waited this long without fitting the
                                 budget holds later ones back until it fits; 0 = 2 s    */
} emfa_serve_opts_t;

/* Runs every request to completion and fills results (one per request).
 * Returns EMFA_OK when the engine ran; per-request failures are reported in
 * results[i].status. */
emfa_status_t emfa_serve(int device, const emfa_request_t* reqs, int n_req, const emfa_serve_opts_t* opts,
                         emfa_request_result_t* results);

/* The admitter of emfa_serve on the host clock of a simulation (no GPU):
 * requests with given arrival times, durations and memory estimates, and
 * the opts' lanes, budget and realtime flag.  start_out[i] and lane_out[i]
 * receive when and where request i would start. */
emfa_status_t emfa_serve_simulate(const double* arrival, const double* duration, const size_t* bytes, int n,
                                  const emfa_serve_opts_t* opts, double* start_out, int* lane_out);

#ifdef __cplusplus
}
#endif

#endif /* EMFA_CUDA_H */
