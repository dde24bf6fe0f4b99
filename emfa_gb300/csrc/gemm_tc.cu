// Tensor-core (tcgen05) multi-RHS complex product -- see below.
#include "emfa_internal.cuh"
#include "gemm.cuh"

namespace emfa {

emfa_status_t cgemm_tf32(Ctx* c, const void*, size_t, const void*, int, int, void*, cudaStream_t)
{
    set_error(c, "cgemm_tf32: tensor-core path not built yet");
    return EMFA_ERR_UNSUPPORTED;
}

}  // namespace emfa
