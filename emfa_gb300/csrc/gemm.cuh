// Launchers of the multi-RHS complex products (gemm.cu, gemm_tc.cu).
#pragma once
#include "emfa_internal.cuh"

namespace emfa {

// Y = Z X on CUDA cores (complex64 / complex128), X and Y RHS-major.
emfa_status_t cgemm_f32(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st);
emfa_status_t cgemm_f64(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st);
// Yd (complex128) = Bsub - Z X (Bsub may be null: Yd = Z X), FP32 products,
// FP64 accumulation of 64-wide K chunks.
emfa_status_t cgemm_f32_chunked(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, const void* Bsub,
                                void* Yd, cudaStream_t st);

}  // namespace emfa

namespace emfa {
// Y = Z X on the tensor cores (tcgen05, TF32 operands, FP32 accumulation).
emfa_status_t cgemm_tf32(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st);
// reads the tensor-core GEMM's error word (synchronises the stream)
emfa_status_t gemm_check_error(Ctx* c, cudaStream_t st);
// dense multi-RHS solve (krylov.cu)
emfa_status_t solve_dense(Ctx* c, int prec, const void* Z, int n, const void* B, int nrhs, void* X,
                          const emfa_solver_params_t* sp, emfa_solve_info_t* info, cudaStream_t st);
}  // namespace emfa
