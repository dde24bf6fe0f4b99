// End-to-end dense RCS job from host buffers: the work solver::invoke_solver
// runs for EFIE / CFIE (EMSolver/Solver.h:20-29): RWG table, upload, fill,
// excitation, multi-RHS solve, RCS, results back to the host.
#include "emfa_internal.cuh"
#include "gemm.cuh"

#include <vector>

using namespace emfa;

extern "C" emfa_status_t emfa_dense_rcs(emfa_ctx_t* ctx, const double* verts_host, int n_vert, const int* tris_host,
                                        int n_tri, const emfa_fill_params_t* fp, const double* angles_host, int n_inc,
                                        const emfa_solver_params_t* sp, const double* rcs_dirs_host, int n_dir,
                                        int per_rhs_dirs, double* rcs_out_host, double* I_out_host,
                                        emfa_solve_info_t* info)
{
    if (!ctx || !verts_host || !tris_host || !fp || !angles_host || !sp || n_inc <= 0 || n_vert <= 0 || n_tri <= 0) {
        set_error(ctx, "emfa_dense_rcs: bad arguments");
        return EMFA_ERR_INVALID;
    }
    EMFA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    std::vector<int> rwg;
    std::string err;
    int n = build_rwg_host(tris_host, n_tri, rwg, &err);
    if (n <= 0) {
        set_error(ctx, "emfa_dense_rcs: no RWG unknowns (" + err + ")");
        return EMFA_ERR_MESH;
    }
    emfa_geom_t* g = nullptr;
    EMFA_TRY(emfa_geom_create(ctx, verts_host, n_vert, tris_host, n_tri, rwg.data(), n, &g));
    struct GeomGuard {
        emfa_geom_t* g;
        ~GeomGuard() { emfa_geom_destroy(g); }
    } guard{g};
    // Z, V and X stay in the context's workspace for the next job (released
    // with the context): a job then allocates nothing of its size
    const size_t es = fp->precision == EMFA_F64 ? 16 : 8;
    void *Z = nullptr, *V = nullptr, *X = nullptr;
    EMFA_TRY(ctx_workspace(ctx, WS_DENSE_Z, es * (size_t)n * n, &Z));
    EMFA_TRY(ctx_workspace(ctx, WS_DENSE_V, es * (size_t)n * n_inc, &V));
    EMFA_TRY(ctx_workspace(ctx, WS_DENSE_X, 16 * (size_t)n * n_inc, &X));
    EMFA_TRY(launch_fill_z(ctx, g, fp, Z, n, st));
    EMFA_TRY(launch_fill_v(ctx, g, fp, angles_host, n_inc, V, st));
    emfa_status_t ss = solve_dense(ctx, fp->precision, Z, n, V, n_inc, X, sp, info, st);
    if (ss != EMFA_OK && ss != EMFA_ERR_NOT_CONVERGED) return ss;
    if (rcs_dirs_host && n_dir > 0 && rcs_out_host)
        EMFA_TRY(launch_rcs(ctx, g, fp, X, n_inc, rcs_dirs_host, n_dir, per_rhs_dirs, rcs_out_host, st));
    if (I_out_host)
        EMFA_CUDA(ctx, cudaMemcpyAsync(I_out_host, X, 16 * (size_t)n * n_inc, cudaMemcpyDeviceToHost, st));
    EMFA_CUDA(ctx, cudaStreamSynchronize(st));
    return ss;
}
