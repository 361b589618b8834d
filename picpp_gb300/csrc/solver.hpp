// solver.hpp -- FP64 Krylov solvers of the implicit Maxwell system on the GPU.
#pragma once
#include <string>
#include <vector>

#include "../../include/picpp_gb300.h"
#include "kernels.hpp"

namespace pic {

// Device workspace, grown on demand and kept for the context's lifetime.
struct Krylov {
    double* V = nullptr;      // basis, cap vectors of length L
    double* Z = nullptr;      // preconditioned directions (flexible GMRES)
    double* w = nullptr;      // scratch vector
    double* mx = nullptr;     // mu x of the operator apply
    double* r = nullptr;      // residual
    double* hdev = nullptr;   // Hessenberg column (device), 2 * (cap + 1)
    double* ydev = nullptr;   // combination coefficients
    double* part = nullptr;   // reduction partials, (cap + 2) * 1024
    double* scal = nullptr;   // scalar results
    int cap = 0;
    int zcap = 0;
    long long L = 0;
    // inner FP32 solve of the mixed-precision preconditioner
    float* mu32 = nullptr;    // FP32 copy of mu (9N)
    float* V32 = nullptr;     // FP32 basis, steps32 + 1 vectors of length L
    float* w32 = nullptr;     // FP32 scratch vector
    float* mx32 = nullptr;    // mu x of the FP32 apply
    double* h32 = nullptr;    // Arnoldi scalars of one inner solve (FP64)
    double* part32 = nullptr; // reduction partials, (steps32 + 2) * 1024
    unsigned* cnt32 = nullptr; // last-block counter of the FP32 reductions (zero between launches)
    int steps32 = 0;
};

class Net;

struct SolveCtx {
    cudaStream_t s;
    const GridP* g;
    const double* mu;
    double* partials;   // >= 8 * 1024 doubles
    int* flag;
    Krylov* k;
    std::string* err;
    Net* net = nullptr;   // learned right preconditioner (PIC_FGMRES_LEARNED)
};

OpCoef make_opcoef(const GridP& g);
pic_status krylov_solve(SolveCtx& c, const double* rhs, double* x, const pic_solve_opts& o, pic_solve_info* info);
void krylov_free(Krylov& k);

}  // namespace pic
