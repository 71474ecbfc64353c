// MKL-API shim (see mkl.h): sparse BLAS, CBLAS level 1 and a PARDISO stand-in, written for the
// oracle from MKL's public documentation.  TEST INFRASTRUCTURE ONLY: it lets the reference's CPU
// minimizer (src/cpp/cpp_mkl_minimizer.cpp) be compiled unchanged and serves as the timed CPU
// baseline of the demag solve; nothing in the product links it.
//
// Reductions (ddot, dnrm2, idamax and the solver's inner products) are summed over fixed blocks of
// 4096 entries whose partials are combined in block order, so results do not depend on the number
// of OpenMP threads.

#include "mkl.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

struct mkl_shim_csr {
    int rows, cols, base;
    const int* rs;
    const int* re;
    const int* ci;
    const double* v;
};

namespace {

constexpr int64_t kBlock = 4096;

inline int64_t nblocks(int64_t n) { return (n + kBlock - 1) / kBlock; }

double block_dot(int64_t n, const double* x, const double* y) {
    const int64_t nb = nblocks(n);
    std::vector<double> part(nb > 0 ? nb : 1, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t i0 = b * kBlock, i1 = std::min(n, i0 + kBlock);
        double s = 0.0;
        for (int64_t i = i0; i < i1; ++i) s += x[i] * y[i];
        part[b] = s;
    }
    double s = 0.0;
    for (int64_t b = 0; b < nb; ++b) s += part[b];
    return s;
}

// ----------------------------------------------------------------------------------------------
// compressed-row matrices of the solver (zero-based, columns sorted, no duplicates)
// ----------------------------------------------------------------------------------------------
struct Csr {
    int n = 0, m = 0;  // rows, columns
    std::vector<int> p, c;
    std::vector<double> v;
    int64_t nnz() const { return p.empty() ? 0 : p[n]; }
};

void spmv(const Csr& A, const double* x, double* y) {
#pragma omp parallel for schedule(static, 512)
    for (int i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) s += A.v[k] * x[A.c[k]];
        y[i] = s;
    }
}

// y += A x
void spmv_add(const Csr& A, const double* x, double* y) {
#pragma omp parallel for schedule(static, 512)
    for (int i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) s += A.v[k] * x[A.c[k]];
        y[i] += s;
    }
}

Csr transpose(const Csr& A) {
    Csr T;
    T.n = A.m;
    T.m = A.n;
    T.p.assign(T.n + 1, 0);
    for (int64_t k = 0; k < A.nnz(); ++k) T.p[A.c[k] + 1]++;
    for (int i = 0; i < T.n; ++i) T.p[i + 1] += T.p[i];
    T.c.resize(A.nnz());
    T.v.resize(A.nnz());
    std::vector<int> next(T.p.begin(), T.p.end() - 1);
    for (int i = 0; i < A.n; ++i)
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) {
            const int d = next[A.c[k]]++;
            T.c[d] = i;
            T.v[d] = A.v[k];
        }
    return T;  // rows come out with ascending columns because A is traversed by row
}

// C = A B (row-by-row accumulation into a dense scatter row; columns sorted afterwards)
Csr multiply(const Csr& A, const Csr& B) {
    Csr C;
    C.n = A.n;
    C.m = B.m;
    C.p.assign(C.n + 1, 0);
    std::vector<int> mark(B.m, -1);
    std::vector<double> acc(B.m, 0.0);
    std::vector<int> cols;
    for (int i = 0; i < A.n; ++i) {
        cols.clear();
        for (int ka = A.p[i]; ka < A.p[i + 1]; ++ka) {
            const int j = A.c[ka];
            const double a = A.v[ka];
            for (int kb = B.p[j]; kb < B.p[j + 1]; ++kb) {
                const int c = B.c[kb];
                if (mark[c] != i) {
                    mark[c] = i;
                    acc[c] = 0.0;
                    cols.push_back(c);
                }
                acc[c] += a * B.v[kb];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int c : cols) {
            C.c.push_back(c);
            C.v.push_back(acc[c]);
        }
        C.p[i + 1] = static_cast<int>(C.c.size());
    }
    return C;
}

// ----------------------------------------------------------------------------------------------
// smoothed-aggregation hierarchy and the PCG that stands in for PARDISO's direct solve
// ----------------------------------------------------------------------------------------------
constexpr double kTheta = 0.115;   // strength threshold on the finest level
constexpr double kThetaFactor = 0.35;  // each coarser level's threshold relative to the finer one
constexpr double kThetaFallback = 0.1;  // when kTheta gives more than four levels
constexpr double kFilterEps = 0.002;    // weak couplings of the level-1 operator moved into its diagonal
constexpr int kMaxCoarse = 1000;   // the coarsest level is factorised densely
constexpr int kMaxLevels = 10;
constexpr int kMaxIter = 2000;

struct Level {
    Csr A, P, R;
    std::vector<double> sm;  // SPAI0 smoother: a_ii / sum_j a_ij^2
};

struct Solver {
    int n = 0;
    std::vector<Level> lv;
    std::vector<double> chol;  // lower Cholesky factor of the coarsest operator, row-major
    int nc = 0;
};

thread_local int g_last_iters = 0;
thread_local double g_last_relres = 0.0;
double g_tol = 1e-12;

std::vector<double> spai0(const Csr& A) {
    std::vector<double> s(A.n, 0.0);
    for (int i = 0; i < A.n; ++i) {
        double d = 0.0, q = 0.0;
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) {
            q += A.v[k] * A.v[k];
            if (A.c[k] == i) d = A.v[k];
        }
        s[i] = q > 0.0 ? d / q : 0.0;
    }
    return s;
}

// Greedy aggregation over the strong graph: (1) a node whose strong neighbours are all free
// seeds an aggregate with them, (2) free nodes join the aggregate of a strong neighbour from
// pass 1, (3) the rest seed aggregates with their free strong neighbours.  Nodes without strong
// neighbours (Dirichlet rows) stay unaggregated.
int aggregate(const Csr& A, double theta, std::vector<int>& agg) {
    const int n = A.n;
    std::vector<double> diag(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = A.p[i]; k < A.p[i + 1]; ++k)
            if (A.c[k] == i) diag[i] = std::fabs(A.v[k]);
    Csr S;
    S.n = S.m = n;
    S.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) {
            const int j = A.c[k];
            if (j != i && A.v[k] * A.v[k] > theta * theta * diag[i] * diag[j]) S.c.push_back(j);
        }
        S.p[i + 1] = static_cast<int>(S.c.size());
    }
    agg.assign(n, -1);
    int na = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1 || S.p[i] == S.p[i + 1]) continue;
        bool free = true;
        for (int k = S.p[i]; k < S.p[i + 1] && free; ++k) free = agg[S.c[k]] == -1;
        if (!free) continue;
        agg[i] = na;
        for (int k = S.p[i]; k < S.p[i + 1]; ++k) agg[S.c[k]] = na;
        ++na;
    }
    std::vector<int> first(agg);
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        for (int k = S.p[i]; k < S.p[i + 1]; ++k)
            if (first[S.c[k]] != -1) {
                agg[i] = first[S.c[k]];
                break;
            }
    }
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1 || S.p[i] == S.p[i + 1]) continue;
        agg[i] = na;
        for (int k = S.p[i]; k < S.p[i + 1]; ++k)
            if (agg[S.c[k]] == -1) agg[S.c[k]] = na;
        ++na;
    }
    return na;
}

// P = (I - omega D^-1 A) T with T the normalised aggregate indicator and omega = 4 / (3 rho), rho
// 1.05 x the power-method estimate of rho(D^-1 A) after 20 products from a fixed pseudo-random start.
Csr prolongator(const Csr& A, const std::vector<int>& agg, int na) {
    const int n = A.n;
    std::vector<int> size(na, 0);
    for (int i = 0; i < n; ++i)
        if (agg[i] >= 0) size[agg[i]]++;
    Csr T;
    T.n = n;
    T.m = na;
    T.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) {
            T.c.push_back(agg[i]);
            T.v.push_back(1.0 / std::sqrt(static_cast<double>(size[agg[i]])));
        }
        T.p[i + 1] = static_cast<int>(T.c.size());
    }
    std::vector<double> dinv(n, 0.0), x(n), y(n);
    for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int k = A.p[i]; k < A.p[i + 1]; ++k)
            if (A.c[k] == i) d = A.v[k];
        dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
        x[i] = static_cast<double>((static_cast<unsigned long long>(i) * 2654435761ull) % 4294967296ull) /
                   4294967296.0 - 0.5;
    }
    auto norm = [](const std::vector<double>& v) {
        double s = 0.0;
        for (double e : v) s += e * e;
        return std::sqrt(s);
    };
    double nx = norm(x), rho = 0.0;
    for (int it = 0; it < 20 && n > 0; ++it) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int k = A.p[i]; k < A.p[i + 1]; ++k) acc += A.v[k] * x[A.c[k]];
            y[i] = dinv[i] * acc;
        }
        const double ny = norm(y);
        if (!(ny > 0.0 && nx > 0.0)) break;
        rho = ny / nx;
        for (int i = 0; i < n; ++i) x[i] = y[i] / ny;
        nx = 1.0;
    }
    rho *= 1.05;
    const double omega = rho > 0.0 ? 4.0 / (3.0 * rho) : 0.0;
    Csr AT = multiply(A, T);
    Csr P;
    P.n = n;
    P.m = na;
    P.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        int kt = T.p[i], ka = AT.p[i];
        const int et = T.p[i + 1], ea = AT.p[i + 1];
        while (kt < et || ka < ea) {
            const int ct = kt < et ? T.c[kt] : na;
            const int ca = ka < ea ? AT.c[ka] : na;
            const int c = std::min(ct, ca);
            double v = 0.0;
            if (ct == c) v += T.v[kt++];
            if (ca == c) v -= omega * dinv[i] * AT.v[ka++];
            P.c.push_back(c);
            P.v.push_back(v);
        }
        P.p[i + 1] = static_cast<int>(P.c.size());
    }
    return P;
}

// A without its weak off-diagonal couplings, |a_ij| + |a_ji| < 2 eps sqrt(|a_ii a_jj|) (a_ji = 0 when
// not stored), each row's weak values summed from zero in column order and added to its diagonal.
Csr filter_weak(const Csr& A, double eps) {
    const int n = A.n;
    std::vector<double> d(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = A.p[i]; k < A.p[i + 1]; ++k)
            if (A.c[k] == i) d[i] = A.v[k];
    auto value_at = [&](int r, int c) {
        for (int k = A.p[r]; k < A.p[r + 1]; ++k)
            if (A.c[k] == c) return A.v[k];
        return 0.0;
    };
    Csr B;
    B.n = n;
    B.m = A.m;
    B.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        double lump = 0.0;
        const int first = static_cast<int>(B.c.size());
        int diag = -1;
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) {
            const int j = A.c[k];
            if (j != i && std::fabs(A.v[k]) + std::fabs(value_at(j, i)) < 2.0 * eps * std::sqrt(std::fabs(d[i] * d[j]))) {
                lump += A.v[k];
                continue;
            }
            if (j == i) diag = static_cast<int>(B.c.size());
            B.c.push_back(j);
            B.v.push_back(A.v[k]);
        }
        if (diag >= first && diag >= 0) B.v[diag] = B.v[diag] + lump;
        B.p[i + 1] = static_cast<int>(B.c.size());
    }
    return B;
}

bool dense_cholesky(const Csr& A, std::vector<double>& L) {
    const int n = A.n;
    L.assign(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) L[static_cast<size_t>(i) * n + A.c[k]] = A.v[k];
    for (int j = 0; j < n; ++j) {
        double d = L[static_cast<size_t>(j) * n + j];
        for (int k = 0; k < j; ++k) d -= L[static_cast<size_t>(j) * n + k] * L[static_cast<size_t>(j) * n + k];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        L[static_cast<size_t>(j) * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double s = L[static_cast<size_t>(i) * n + j];
            for (int k = 0; k < j; ++k) s -= L[static_cast<size_t>(i) * n + k] * L[static_cast<size_t>(j) * n + k];
            L[static_cast<size_t>(i) * n + j] = s / d;
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) L[static_cast<size_t>(i) * n + j] = 0.0;
    return true;
}

void cholesky_solve(const std::vector<double>& L, int n, const double* b, double* x) {
    for (int i = 0; i < n; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[static_cast<size_t>(i) * n + k] * x[k];
        x[i] = s / L[static_cast<size_t>(i) * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = x[i];
        for (int k = i + 1; k < n; ++k) s -= L[static_cast<size_t>(k) * n + i] * x[k];
        x[i] = s / L[static_cast<size_t>(i) * n + i];
    }
}

// Full symmetric (or general) CSR from PARDISO's input arrays.
bool read_matrix(int n, const double* a, const int* ia, const int* ja, int base, bool upper_only, Csr& A) {
    A.n = A.m = n;
    A.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        for (int k = ia[i] - base; k < ia[i + 1] - base; ++k) {
            const int j = ja[k] - base;
            if (j < 0 || j >= n) return false;
            if (upper_only) {
                if (j < i) continue;
                A.p[i + 1]++;
                if (j != i) A.p[j + 1]++;
            } else {
                A.p[i + 1]++;
            }
        }
    }
    for (int i = 0; i < n; ++i) A.p[i + 1] += A.p[i];
    A.c.resize(A.p[n]);
    A.v.resize(A.p[n]);
    std::vector<int> next(A.p.begin(), A.p.end() - 1);
    for (int i = 0; i < n; ++i) {
        for (int k = ia[i] - base; k < ia[i + 1] - base; ++k) {
            const int j = ja[k] - base;
            if (upper_only && j < i) continue;
            int d = next[i]++;
            A.c[d] = j;
            A.v[d] = a[k];
            if (upper_only && j != i) {
                d = next[j]++;
                A.c[d] = i;
                A.v[d] = a[k];
            }
        }
    }
    // sort each row and sum duplicates
    std::vector<std::pair<int, double>> row;
    Csr B;
    B.n = B.m = n;
    B.p.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        row.clear();
        for (int k = A.p[i]; k < A.p[i + 1]; ++k) row.emplace_back(A.c[k], A.v[k]);
        std::sort(row.begin(), row.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        for (size_t k = 0; k < row.size(); ++k) {
            if (!B.c.empty() && static_cast<int>(B.c.size()) > B.p[i] && B.c.back() == row[k].first)
                B.v.back() += row[k].second;
            else {
                B.c.push_back(row[k].first);
                B.v.push_back(row[k].second);
            }
        }
        B.p[i + 1] = static_cast<int>(B.c.size());
    }
    A = std::move(B);
    return true;
}

Solver* build_solver_theta(const Csr& A0, double theta) {
    auto* s = new Solver();
    s->n = A0.n;
    s->lv.emplace_back();
    s->lv.back().A = A0;
    while (static_cast<int>(s->lv.size()) < kMaxLevels && s->lv.back().A.n > kMaxCoarse) {
        Level& f = s->lv.back();
        std::vector<int> agg;
        const int na = aggregate(f.A, theta, agg);
        theta *= kThetaFactor;
        if (na == 0 || na >= f.A.n) break;
        f.P = prolongator(f.A, agg, na);
        f.R = transpose(f.P);
        Csr AP = multiply(f.A, f.P);
        Csr Ac = multiply(f.R, AP);
        if (s->lv.size() == 1) Ac = filter_weak(Ac, kFilterEps);
        f.sm = spai0(f.A);
        s->lv.emplace_back();
        s->lv.back().A = std::move(Ac);
    }
    Level& c = s->lv.back();
    s->nc = c.A.n;
    if (!dense_cholesky(c.A, s->chol)) {
        delete s;
        return nullptr;
    }
    return s;
}

Solver* build_solver(Csr&& A0) {
    Solver* s = build_solver_theta(A0, kTheta);
    if (s && s->lv.size() > 4) {
        delete s;
        s = build_solver_theta(A0, kThetaFallback);
    }
    return s;
}

struct Work {
    std::vector<std::vector<double>> x, b, r;
};

void vcycle(const Solver& s, Work& w, size_t l) {
    const Level& L = s.lv[l];
    std::vector<double>& x = w.x[l];
    std::vector<double>& b = w.b[l];
    std::vector<double>& r = w.r[l];
    const int n = L.A.n;
    if (l + 1 == s.lv.size()) {
        cholesky_solve(s.chol, n, b.data(), x.data());
        return;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) x[i] = L.sm[i] * b[i];
    spmv(L.A, x.data(), r.data());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
    spmv(L.R, r.data(), w.b[l + 1].data());
    vcycle(s, w, l + 1);
    spmv_add(L.P, w.x[l + 1].data(), x.data());
    spmv(L.A, x.data(), r.data());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) x[i] += L.sm[i] * (b[i] - r[i]);
}

// PCG from x = 0 to ||b - A x|| <= tol ||b|| (the recursive residual's test confirmed on the true
// residual).  Returns the iteration count, or -1 when it did not converge.
int solve(const Solver& s, const double* b, double* x, double tol, double* relres) {
    const int n = s.n;
    const Csr& A = s.lv[0].A;
    Work w;
    for (const Level& L : s.lv) {
        w.x.emplace_back(L.A.n, 0.0);
        w.b.emplace_back(L.A.n, 0.0);
        w.r.emplace_back(L.A.n, 0.0);
    }
    std::vector<double> r(b, b + n), z(n), p(n), q(n);
    std::fill(x, x + n, 0.0);
    const double bn = std::sqrt(block_dot(n, b, b));
    if (bn == 0.0) {
        *relres = 0.0;
        return 0;
    }
    auto precondition = [&](const double* rin, double* zout) {
        std::copy(rin, rin + n, w.b[0].begin());
        vcycle(s, w, 0);
        std::copy(w.x[0].begin(), w.x[0].end(), zout);
    };
    precondition(r.data(), z.data());
    p = z;
    double rz = block_dot(n, r.data(), z.data());
    for (int it = 1; it <= kMaxIter; ++it) {
        spmv(A, p.data(), q.data());
        const double pq = block_dot(n, p.data(), q.data());
        if (!(pq > 0.0)) break;
        const double alpha = rz / pq;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        double rn = std::sqrt(block_dot(n, r.data(), r.data()));
        if (rn <= tol * bn) {
            spmv(A, x, q.data());
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; ++i) r[i] = b[i] - q[i];
            rn = std::sqrt(block_dot(n, r.data(), r.data()));
            if (rn <= tol * bn) {
                *relres = rn / bn;
                return it;
            }
            precondition(r.data(), z.data());  // restart from the true residual
            p = z;
            rz = block_dot(n, r.data(), z.data());
            continue;
        }
        precondition(r.data(), z.data());
        const double rz_new = block_dot(n, r.data(), z.data());
        const double beta = rz_new / rz;
        rz = rz_new;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    spmv(A, x, q.data());
    double rn = 0.0;
    for (int i = 0; i < n; ++i) rn += (b[i] - q[i]) * (b[i] - q[i]);
    *relres = std::sqrt(rn) / bn;
    return -1;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------------
// sparse BLAS
// ---------------------------------------------------------------------------------------------
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t* A, sparse_index_base_t indexing, MKL_INT rows,
                                        MKL_INT cols, MKL_INT* rows_start, MKL_INT* rows_end,
                                        MKL_INT* col_indx, double* values) {
    if (A == nullptr || rows < 0 || cols < 0 || rows_start == nullptr || rows_end == nullptr)
        return SPARSE_STATUS_INVALID_VALUE;
    if (indexing != SPARSE_INDEX_BASE_ZERO && indexing != SPARSE_INDEX_BASE_ONE) return SPARSE_STATUS_INVALID_VALUE;
    auto* h = new (std::nothrow) mkl_shim_csr{rows, cols, indexing == SPARSE_INDEX_BASE_ONE ? 1 : 0,
                                              rows_start, rows_end, col_indx, values};
    if (h == nullptr) return SPARSE_STATUS_ALLOC_FAILED;
    *A = h;
    return SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_optimize(sparse_matrix_t A) {
    return A == nullptr ? SPARSE_STATUS_NOT_INITIALIZED : SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_d_mv(sparse_operation_t operation, double alpha, sparse_matrix_t A,
                                struct matrix_descr descr, const double* x, double beta, double* y) {
    if (A == nullptr) return SPARSE_STATUS_NOT_INITIALIZED;
    if (operation != SPARSE_OPERATION_NON_TRANSPOSE || descr.type != SPARSE_MATRIX_TYPE_GENERAL)
        return SPARSE_STATUS_NOT_SUPPORTED;
    const int base = A->base;
#pragma omp parallel for schedule(static, 512)
    for (int i = 0; i < A->rows; ++i) {
        double s = 0.0;
        for (int k = A->rs[i] - base; k < A->re[i] - base; ++k) s += A->v[k] * x[A->ci[k] - base];
        y[i] = beta == 0.0 ? alpha * s : alpha * s + beta * y[i];
    }
    return SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
    delete A;
    return SPARSE_STATUS_SUCCESS;
}

// ---------------------------------------------------------------------------------------------
// CBLAS level 1
// ---------------------------------------------------------------------------------------------
double cblas_ddot(MKL_INT n, const double* x, MKL_INT incx, const double* y, MKL_INT incy) {
    if (n <= 0) return 0.0;
    if (incx == 1 && incy == 1) return block_dot(n, x, y);
    double s = 0.0;
    const int64_t ix0 = incx >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incx;
    const int64_t iy0 = incy >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incy;
    for (int64_t i = 0; i < n; ++i) s += x[ix0 + i * incx] * y[iy0 + i * incy];
    return s;
}

void cblas_daxpy(MKL_INT n, double a, const double* x, MKL_INT incx, double* y, MKL_INT incy) {
    if (n <= 0) return;
    if (incx == 1 && incy == 1) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
        return;
    }
    const int64_t ix0 = incx >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incx;
    const int64_t iy0 = incy >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incy;
    for (int64_t i = 0; i < n; ++i) y[iy0 + i * incy] += a * x[ix0 + i * incx];
}

void cblas_daxpby(MKL_INT n, double a, const double* x, MKL_INT incx, double b, double* y, MKL_INT incy) {
    if (n <= 0) return;
    if (incx == 1 && incy == 1) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) y[i] = a * x[i] + b * y[i];
        return;
    }
    const int64_t ix0 = incx >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incx;
    const int64_t iy0 = incy >= 0 ? 0 : static_cast<int64_t>(n - 1) * -incy;
    for (int64_t i = 0; i < n; ++i) y[iy0 + i * incy] = a * x[ix0 + i * incx] + b * y[iy0 + i * incy];
}

void cblas_dscal(MKL_INT n, double a, double* x, MKL_INT incx) {
    if (n <= 0 || incx <= 0) return;
    if (incx == 1) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) x[i] *= a;
        return;
    }
    for (int64_t i = 0; i < n; ++i) x[i * incx] *= a;
}

double cblas_dnrm2(MKL_INT n, const double* x, MKL_INT incx) {
    if (n <= 0 || incx <= 0) return 0.0;
    if (incx == 1) return std::sqrt(block_dot(n, x, x));
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += x[i * incx] * x[i * incx];
    return std::sqrt(s);
}

// index (zero-based) of the first entry of largest magnitude
CBLAS_INDEX cblas_idamax(MKL_INT n, const double* x, MKL_INT incx) {
    if (n <= 0 || incx <= 0) return 0;
    if (incx != 1) {
        int64_t best = 0;
        for (int64_t i = 1; i < n; ++i)
            if (std::fabs(x[i * incx]) > std::fabs(x[best * incx])) best = i;
        return static_cast<CBLAS_INDEX>(best);
    }
    const int64_t nb = nblocks(n);
    std::vector<int64_t> arg(nb);
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t i0 = b * kBlock, i1 = std::min<int64_t>(n, i0 + kBlock);
        int64_t best = i0;
        for (int64_t i = i0 + 1; i < i1; ++i)
            if (std::fabs(x[i]) > std::fabs(x[best])) best = i;
        arg[b] = best;
    }
    int64_t best = arg[0];
    for (int64_t b = 1; b < nb; ++b)
        if (std::fabs(x[arg[b]]) > std::fabs(x[best])) best = arg[b];
    return static_cast<CBLAS_INDEX>(best);
}

// ---------------------------------------------------------------------------------------------
// PARDISO stand-in
// ---------------------------------------------------------------------------------------------
void pardiso(void** pt, const MKL_INT* maxfct, const MKL_INT* mnum, const MKL_INT* mtype, const MKL_INT* phase,
             const MKL_INT* n, const void* a, const MKL_INT* ia, const MKL_INT* ja, MKL_INT* perm,
             const MKL_INT* nrhs, MKL_INT* iparm, const MKL_INT* msglvl, void* b, void* x, MKL_INT* error) {
    (void)maxfct;
    (void)mnum;
    (void)perm;
    (void)msglvl;
    if (error == nullptr) return;
    *error = 0;
    if (pt == nullptr || phase == nullptr) {
        *error = -1;
        return;
    }
    auto* s = static_cast<Solver*>(pt[0]);
    const int ph = *phase;
    if (ph == -1 || ph == 0) {
        delete s;
        pt[0] = nullptr;
        return;
    }
    if (n == nullptr || *n <= 0 || (nrhs != nullptr && *nrhs != 1)) {
        *error = -1;
        return;
    }
    if (ph == 12 || ph == 13 || ph == 22 || ph == 23) {
        if (a == nullptr || ia == nullptr || ja == nullptr || mtype == nullptr) {
            *error = -1;
            return;
        }
        const int base = (iparm != nullptr && iparm[34] != 0) ? 0 : 1;
        const bool sym = *mtype == 2 || *mtype == -2 || *mtype == 1;
        Csr A;
        try {
            if (!read_matrix(*n, static_cast<const double*>(a), ia, ja, base, sym, A)) {
                *error = -1;
                return;
            }
            delete s;
            pt[0] = nullptr;
            s = build_solver(std::move(A));
        } catch (const std::bad_alloc&) {
            *error = -2;
            return;
        }
        if (s == nullptr) {
            *error = -4;
            return;
        }
        pt[0] = s;
    } else if (ph == 11) {
        return;  // analysis happens with the numerical phase
    }
    if (ph == 13 || ph == 23 || ph == 33) {
        if (s == nullptr || b == nullptr || x == nullptr || s->n != *n) {
            *error = -1;
            return;
        }
        double rr = 0.0;
        int it;
        try {
            it = solve(*s, static_cast<const double*>(b), static_cast<double*>(x), g_tol, &rr);
        } catch (const std::bad_alloc&) {
            *error = -2;
            return;
        }
        g_last_iters = it;
        g_last_relres = rr;
        if (it < 0) *error = -4;
    }
}

void mkl_shim_set_pardiso_tol(double tol) {
    if (tol > 0.0) g_tol = tol;
}

double mkl_shim_get_pardiso_tol(void) { return g_tol; }

int mkl_shim_last_iterations(void) { return g_last_iters; }

double mkl_shim_last_relres(void) { return g_last_relres; }

int mkl_shim_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int mkl_shim_hierarchy(void** pt, int* rows_out, int max_levels) {
    if (pt == nullptr || pt[0] == nullptr) return 0;
    const auto* s = static_cast<const Solver*>(pt[0]);
    const int L = static_cast<int>(s->lv.size());
    for (int l = 0; l < L && l < max_levels; ++l) rows_out[l] = s->lv[l].A.n;
    return L;
}

}  // extern "C"
