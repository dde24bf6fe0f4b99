// Device state of the batched GMRES solver (krylov.cu).
#pragma once
#include <cuda_runtime.h>

namespace emfa {

struct GmresDev {
    int m, nrhs, tol_abs;
    double tol;
    double inner;    // the Arnoldi steps stop at inner x the restart's threshold,
    double red;      //   or at red x the cycle's starting residual if that is larger
    double2* H;      // nrhs x (m+1) x m, row-major per RHS
    double* cs;      // nrhs x m  Givens cosines
    double2* sn;     // nrhs x m  Givens sines
    double2* g;      // nrhs x (m+1) rotated residual vector
    double2* y;      // m x nrhs  solution of the small system (also CGS scratch)
    double2* hcol;   // (m+1) x nrhs  Arnoldi column being built
    double* bnorm;   // nrhs  ||b||
    double* wmax;    // nrhs  max |Re|, |Im| of the orthogonalised w of the step
    double* scale;   // nrhs  1/beta of the vector being normalised (0 = inactive)
    double* est;     // nrhs  rotated residual estimate
    double* true_res;// nrhs  true relative residual at the last restart
    int* jlen;       // nrhs  basis vectors used in the current cycle
    int* active;     // nrhs
    int* counters;   // [0] active RHS, [1] converged RHS (cycle start); [2], [3] per Arnoldi step
    int* step_cnt;   // the step's count of RHS still active: counters + 2 + (j & 1), so that the
                     //   host's read of step j overlaps step j + 1 (which counts into the other)
};

}  // namespace emfa
