// C++ restatement of the reference's CPU demag solve and energy/gradient entry points.
//
// TEST INFRASTRUCTURE ONLY (oracle).  The reference's own translation unit,
// src/cpp/cpp_mkl_minimizer.cpp of MaMMoS-project/mumag_matrixfree2, is compiled unchanged
// against the MKL-API shim wherever its source is available (oracle/_ref/libcpp_mkl_minimizer.so).
// Where it is not (the GPU host has no copy of the reference), this file provides the entry points
// that the CPU baseline times, with the same C signatures and the same arithmetic, over the same
// shim:
//
//   init_pardiso / free_pardiso / pardiso_solve_direct   cpp_mkl_minimizer.cpp:27-108
//   evaluate_energy_and_grad                              cpp_mkl_minimizer.cpp:178-206
//   solve_poisson                                         cpp_mkl_minimizer.cpp:208-231
//
// A CPU test checks that both libraries give the same results on the same inputs.

#include "mkl.h"

#include <cstdint>
#include <map>
#include <mutex>
#include <vector>

namespace {

struct Factor {
    void* pt[64] = {};
    MKL_INT iparm[64] = {};
    MKL_INT n = 0;
};

std::mutex g_mu;
std::map<int64_t, Factor*> g_factors;
int64_t g_next = 1;

Factor* find(int64_t id) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_factors.find(id);
    return it == g_factors.end() ? nullptr : it->second;
}

MKL_INT call(Factor* f, MKL_INT phase, const double* a, const MKL_INT* ia, const MKL_INT* ja, double* b,
             double* x) {
    const MKL_INT maxfct = 1, mnum = 1, mtype = 2, nrhs = 1, msglvl = 0;
    MKL_INT perm = 0, err = 0;
    pardiso(f->pt, &maxfct, &mnum, &mtype, &phase, &f->n, a, ia, ja, &perm, &nrhs, f->iparm, &msglvl, b, x, &err);
    return err;
}

}  // namespace

extern "C" {

// Factorise the SPD matrix given by its upper triangle (zero-based CSR); a handle > 0, or -error.
int64_t init_pardiso(int n, double* a, int* ia, int* ja) {
    auto* f = new Factor();
    f->n = n;
    f->iparm[0] = 1;
    f->iparm[1] = 2;
    f->iparm[34] = 1;
    const MKL_INT err = call(f, 12, a, ia, ja, nullptr, nullptr);
    if (err != 0) {
        delete f;
        return -static_cast<int64_t>(err);
    }
    std::lock_guard<std::mutex> lk(g_mu);
    const int64_t id = g_next++;
    g_factors[id] = f;
    return id;
}

void free_pardiso(int64_t id) {
    Factor* f = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_factors.find(id);
        if (it == g_factors.end()) return;
        f = it->second;
        g_factors.erase(it);
    }
    call(f, -1, nullptr, nullptr, nullptr, nullptr, nullptr);
    delete f;
}

int pardiso_solve_direct(int64_t id, const double* b, double* x) {
    Factor* f = find(id);
    if (f == nullptr) return -1;
    return call(f, 33, nullptr, nullptr, nullptr, const_cast<double*>(b), x);
}

// g = (K_eff m + G U + g_zee) / V_mag with g_zee_i = -2 M_i B; E = (m . (K_eff m + G U + 2 g_zee)) / (2 V_mag)
void evaluate_energy_and_grad(int N, const double* m, const double* U, const double* B_ext, const double* M_nodal,
                              sparse_matrix_t K_eff, sparse_matrix_t G_sparse, double* E, double* g_total,
                              double inv_Vmag) {
    matrix_descr general{};
    general.type = SPARSE_MATRIX_TYPE_GENERAL;
    mkl_sparse_d_mv(SPARSE_OPERATION_NON_TRANSPOSE, 1.0, K_eff, general, m, 0.0, g_total);
    mkl_sparse_d_mv(SPARSE_OPERATION_NON_TRANSPOSE, 1.0, G_sparse, general, U, 1.0, g_total);
    double twice = 0.0;
#pragma omp parallel for reduction(+ : twice)
    for (int i = 0; i < N; ++i) {
        for (int c = 0; c < 3; ++c) {
            const double gz = -2.0 * M_nodal[i] * B_ext[c];
            g_total[3 * i + c] += gz;
            twice += m[3 * i + c] * (g_total[3 * i + c] + gz);
        }
    }
    *E = 0.5 * twice * inv_Vmag;
    cblas_dscal(3 * N, inv_Vmag, g_total, 1);
}

// U = mask * A^-1 (mask * D m): the demag potential of m with the factorised Poisson operator.
void solve_poisson(int N, const double* m, int64_t pardiso_handle, sparse_matrix_t D_sparse, double* U,
                   const double* boundary_mask) {
    if (pardiso_handle == 0) return;
    matrix_descr general{};
    general.type = SPARSE_MATRIX_TYPE_GENERAL;
    std::vector<double> rhs(N, 0.0);
    mkl_sparse_d_mv(SPARSE_OPERATION_NON_TRANSPOSE, 1.0, D_sparse, general, m, 0.0, rhs.data());
    if (boundary_mask != nullptr)
        for (int i = 0; i < N; ++i) rhs[i] *= boundary_mask[i];
    pardiso_solve_direct(pardiso_handle, rhs.data(), U);
    if (boundary_mask != nullptr)
        for (int i = 0; i < N; ++i) U[i] *= boundary_mask[i];
}

}  // extern "C"
