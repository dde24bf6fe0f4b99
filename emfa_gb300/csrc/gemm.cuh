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

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

namespace emfa {
// driver entry point of cuTensorMapEncodeTiled (null if unavailable)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
// Y = Z X on the tensor cores (tcgen05, TF32 operands, FP32 accumulation).
emfa_status_t cgemm_tf32(Ctx* c, const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, cudaStream_t st);
// reads the tensor-core GEMM's error word (synchronises the stream)
emfa_status_t gemm_check_error(Ctx* c, cudaStream_t st);
// The same product on caller-owned scratch and without a context: bpack holds
// 16 * n * nrhs bytes (16-byte aligned), err is an int the caller has zeroed.
// cgemm_tf32_prepare sets the kernels' shared-memory limit on the current device.
emfa_status_t cgemm_tf32_prepare();
emfa_status_t cgemm_tf32_scratch(const void* Z, size_t ldz, const void* X, int n, int nrhs, void* Y, void* bpack,
                                 int* err, cudaStream_t st);
// Split-FP16 planes of a complex64 matrix Z (gemm_h.cu): Zh = fp16(s Z),
// Zl = fp16(s Z - Zh) with s a power of two (max |s Z| < 2^15), each an
// n x 2n real matrix (re, im interleaved) with rows ldh halves apart.
struct HPlanes {
    const __half* zh = nullptr;
    const __half* zl = nullptr;
    const float* inv_s = nullptr;  // device: 1 / s
    int n = 0;
    size_t ldh = 0;
};
// splits Z into the context's plane workspace (two passes over Z)
emfa_status_t hsplit_prepare(Ctx* c, const void* Z, size_t ldz, int n, HPlanes* out, cudaStream_t st);
// Y (complex64) = Z X (complex64): Zh times an FP16 copy of X scaled per
// right-hand side; accuracy of a TF32 product at the FP16 tensor rate
emfa_status_t hgemm_apply(Ctx* c, const HPlanes& h, const void* X, void* Y, int nrhs, cudaStream_t st);
// Vout = scale[r] W (complex64, the Krylov normalisation), packed to FP16 in
// the same pass, then Y = Z Vout; Y may alias W (W is consumed first)
emfa_status_t hgemm_normalize_apply(Ctx* c, const HPlanes& h, const void* W, const double* scale,
                                    const double* wmax, void* Vout, void* Y, int nrhs, cudaStream_t st);
// The FP16 rows the inner product reads as its B operand: right-hand side r
// is rows 2r = (Re, -Im) and 2r+1 = (Im, Re) of bh, ldh halves apart, scaled
// by t_r = 1 / inv_t[r].  A producer that packs them itself (the fused
// Arnoldi step) then runs the product from them.
struct HPack {
    __half* bh = nullptr;
    float* inv_t = nullptr;
    size_t ldh = 0;
    const int* skip = nullptr;  // optional: a device int; zero when the product starts skips it
};
emfa_status_t hgemm_pack_target(Ctx* c, const HPlanes& h, int nrhs, HPack* out);
emfa_status_t hgemm_apply_packed(Ctx* c, const HPlanes& h, const HPack& p, void* Y, int nrhs, cudaStream_t st);
// packs X (complex64, RHS-major) into the rows p names, with the scale of
// each right-hand side from its max |Re|, |Im| (the packing hgemm_apply does)
emfa_status_t hgemm_pack(Ctx* c, const HPlanes& h, const void* X, const HPack& p, int nrhs, cudaStream_t st);
// exponent e of the FP16 scale t = 2^(14 - e) of v = scale w, from wmax =
// max |Re|, |Im| of w: max |t v| < 2^14 (the FP32 rounding of scale can raise
// max |v| by an ulp, hence the factor)
__device__ __forceinline__ int hpack_exponent(double wmax, double scale)
{
    int e = 0;
    frexpf((float)(wmax * scale) * 1.0000002f, &e);
    return e;
}
// the same from FP32 operands (their product rounds once more: the factor
// covers two ulps)
__device__ __forceinline__ int hpack_exponent_f(float wmax, float scale)
{
    int e = 0;
    frexpf(wmax * scale * 1.0000004f, &e);
    return e;
}
// R (complex128) = B - Z X for X complex128 and B complex64 (f32b) or complex128:
// Zh Xh + Zh Xl + Zl Xh on the tensor cores, FP32 chunk sums reduced in FP64
emfa_status_t hgemm_residual(Ctx* c, const HPlanes& h, const double2* X, const void* B, bool b_is_f32, double2* R,
                             int nrhs, cudaStream_t st);
emfa_status_t hgemm_check_error(Ctx* c, cudaStream_t st);
// the inner product's tile shapes (BN x MS) and the autotuner's record of a
// shape bucket: variant -1 if untuned; ms[v] the best of two timed launches
// of shape v, -1 where v was not a candidate
enum { HV_64_1 = 0, HV_64_2, HV_144_1, HV_144_2, HV_COUNT };
emfa_status_t hgemm_tuned_shape(int device, int n, int nrhs, int* variant, float* ms);
void hgemm_tune_clear();

// Linear operator driven by the batched Krylov solvers (krylov.cu): the
// dense impedance matrix or the MLFMA operator.
struct LinOp {
    int n = 0;
    int prec = EMFA_F32;  // EMFA_F32: iteration vectors complex64; EMFA_F64: complex128
    virtual ~LinOp() {}
    // Y = A X in the iteration precision (nrhs vectors, RHS-major)
    virtual emfa_status_t apply(Ctx* c, const void* X, void* Y, int nrhs, cudaStream_t st) = 0;
    // R = B - A X, accurate: X and R complex128, B in the iteration precision;
    // xt: complex64 scratch of nrhs * n
    virtual emfa_status_t residual(Ctx* c, const double2* X, const void* B, double2* R, int nrhs, float2* xt,
                                   cudaStream_t st) = 0;
    // error word of asynchronous device-side checks (synchronises)
    virtual emfa_status_t check(Ctx*, cudaStream_t) { return EMFA_OK; }
    // fraction of a restart's residual target at which GMRES's inner steps
    // stop: below 1 where apply() is less accurate than residual(), so the
    // implicit residual must undershoot for the true one to meet the target
    virtual double inner_margin() const { return 1.0; }
    // default per-cycle reduction of GMRES-IR's inner solve (0: none, iterate
    // to the target)
    virtual double inner_reduction() const { return 0.0; }
    // Vout = scale[r] W (the Krylov normalisation, iteration precision), then
    // Y = A Vout; Y may alias W.  Operators that pack their input fuse both.
    // wmax (optional): per RHS max |Re|, |Im| of W, known from the pass that produced it
    virtual emfa_status_t normalize_apply(Ctx* c, const void* W, const double* scale, const double* wmax, void* Vout,
                                          void* Y, int nrhs, cudaStream_t st);
    // Operators whose apply() packs its input to FP16 rows: where the rows
    // go (false: the operator does not pack), and Y = A V from rows a
    // producer has written there
    virtual bool pack_target(Ctx*, int, HPack*) { return false; }
    virtual emfa_status_t apply_packed(Ctx*, const HPack&, void*, int, cudaStream_t) { return EMFA_ERR_UNSUPPORTED; }
    // packs X into rows of the layout pack_target gives, at p.bh / p.inv_t
    // (with p.ldh from pack_target): the FP16 basis of GMRES
    virtual emfa_status_t pack(Ctx*, const void*, const HPack&, int, cudaStream_t) { return EMFA_ERR_UNSUPPORTED; }
};

emfa_status_t solve_op(Ctx* c, LinOp& A, const void* B, int nrhs, void* X, const emfa_solver_params_t* sp,
                       emfa_solve_info_t* info, cudaStream_t st);
// dense multi-RHS solve (krylov.cu)
emfa_status_t solve_dense(Ctx* c, int prec, const void* Z, int n, const void* B, int nrhs, void* X,
                          const emfa_solver_params_t* sp, emfa_solve_info_t* info, cudaStream_t st);
}  // namespace emfa
