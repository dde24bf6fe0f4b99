// Dense LU factorisation (lu.cu): the factor object and its solve.
#pragma once
#include "emfa_internal.cuh"

namespace emfa {

constexpr int LU_NB = 64;  // diagonal block of the factorisation

struct LuFactor {
    int n = 0, nblk = 0;
    int lda = 0;  // complex elements between rows of a: n rounded up to even
    DevBuf a;     // complex64 n x n, rows lda apart: unit-lower L below the diagonal, U on and above
    DevBuf perm;  // int n: original row now at each position
    DevBuf linv;  // complex64 [nblk][64][64]: inverses of the unit-lower diagonal blocks
    DevBuf uinv;  // complex64 [nblk][64][64]: inverses of the upper diagonal blocks
    DevBuf info;  // int[0]: 1 + first row whose pivot was exactly zero, 0 if none;
                  // int[1]: error code of a tensor-core update wait that timed out;
                  // int[2]: error code of a triangular-solve wait that timed out
    DevBuf ops;   // trailing-update operands: FP16 hi/lo planes of U12 and L21, and their scales
    void release()
    {
        ops.release();
        a.release();
        perm.release();
        linv.release();
        uinv.release();
        info.release();
    }
};

// Device bytes of a factor of order n.
size_t lu_bytes(int n);
// Factor the row-major complex64 matrix Z (Z may be the factor's own buffer).
emfa_status_t lu_factor(Ctx* c, const void* Z, int n, LuFactor& F, cudaStream_t st);
// First zero pivot (1-based row, 0 if none); synchronises st.  Returns
// EMFA_ERR_TIMEOUT if a wait of the tensor-core update gave up.
emfa_status_t lu_zero_pivot(Ctx* c, const LuFactor& F, int* first, cudaStream_t st);
// Error word of the triangular solves queued so far (synchronises st):
// EMFA_ERR_TIMEOUT if one of their waits gave up.
emfa_status_t lu_check_solves(Ctx* c, const LuFactor& F, cudaStream_t st);
// X = A^-1 B for nrhs complex64 right-hand sides (RHS-major); work holds
// 2 n nrhs complex64.  X may not alias B.
emfa_status_t lu_apply(Ctx* c, const LuFactor& F, const float2* B, int nrhs, float2* X, float2* work,
                       cudaStream_t st);

}  // namespace emfa
