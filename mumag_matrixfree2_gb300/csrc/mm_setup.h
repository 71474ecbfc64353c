// Host-side (C++) setup of the micromagnetic hot path: mesh geometry, Dirichlet mask, Morton
// order, assembly of the compressed-row operators and the smoothed-aggregation hierarchy.
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace mm {

// Allocator whose resize() leaves new elements uninitialised: the large setup arrays are then first
// written (and their pages first touched) by the threads that fill them, in parallel.
template <class T>
struct UninitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <class U>
  UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
};
using dvec = std::vector<double, UninitAlloc<double>>;
using ivec = std::vector<int, UninitAlloc<int>>;

struct HostCSR {
  int n_rows = 0, n_cols = 0;
  std::vector<int> ptr;
  ivec col;
  dvec val;
  int64_t nnz() const { return ptr.empty() ? 0 : ptr.back(); }
};

// Per-magnetic-row operator of the energy, the local Hessian and the demag right-hand side.
// Row r belongs to node rows[r]; entry k couples it to node col[k] through elements of material
// mat[k] (0-based).  For an entry (a, b):
//   w   = sum_e 2 A_e Ve grad(phi_a).grad(phi_b)                    (exchange, K_ex)
//   q   = sum_e 2 K1_e Ve / 20 * (1 + delta_ab)                      (anisotropy, used as -q (k.v_b) k)
//   G   = sum_e 2 Js_e Ve / 4 * grad(phi_b)                          (demag gradient, g_a += G U_b)
//   D   = sum_e Js_e Ve / 4 * grad(phi_a)                            (demag source, b_a += D . m_b)
struct EnergyOp {
  int n_rows = 0;
  std::vector<int> rows, ptr;
  ivec col, mat;
  dvec w, q, gx, gy, gz, dx, dy, dz;
  int n_mat = 0;
  bool single_axis = true;
  std::vector<double> diag_exchange;  // w_aa per node (N)
  // magnetoelastic entries (empty when the term is absent): sum_e 2 (k1me +- k1me_p) Ve / 20 (1 + d_ab),
  // acting on the x (mx) and y (my) components
  dvec mx, my;
};

struct AmgLevel {
  HostCSR A, P, R;
  HostCSR RA;  // R A, the Galerkin product's first factor, kept for the fused restriction (may be freed)
  std::vector<double> spai0, diag;
  std::vector<int> agg;  // aggregate of each row (-1 = none), empty on the coarsest level
};

struct AmgParams {
  int max_levels = 10;
  int max_coarse = 1000;
  // strength threshold on the finest level; 0 (default): 0.115, or 0.1 when 0.115 gives more than
  // four levels (an empirical rule from the 40 / 80 / 120 nm cubes)
  double theta0 = 0.0;
  // the threshold of level l + 1 is theta_factor times level l's: 0.35 keeps the 80 nm cube's 16
  // iterations with a level 2 of 4,673 rows instead of 8,193 (FP64 solve 2.43 -> 2.16 ms)
  double theta_factor = 0.35;
  // weak entries of the level-1 operator dropped into its diagonal (0: none): at 0.002 the 80 nm
  // cube's A_1 keeps 1.65M of 4.40M entries and PCG its 16 iterations
  double filter_eps = 0.002;
  int rho_steps = 20;      // power-method steps of the smoothing's spectral-radius estimate
  double rho_safety = 1.05;
};

// Counts the setups running at once in this process while it lives: each parallel pass of a setup
// takes the host's threads (at most 16) divided by that count, so that many problems set up
// concurrently (one per host thread) share the cores instead of each spawning 16 threads.
struct SetupScope {
  SetupScope();
  ~SetupScope();
  SetupScope(const SetupScope&) = delete;
  SetupScope& operator=(const SetupScope&) = delete;
};

// geometry (src/loop.py:56-102)
void geom_compute(int N, int E, const double* knt, const int* conn_in, int* conn_out, double* volume,
                  double* JinvT, double* grad_phi);
// Dirichlet mask (src/add_shell.py:105-136)
void boundary_mask(int N, int E, const int* conn, double* mask);
// Morton order (src/reorder_mesh.py:19-30,85-100); stable on ties
void morton_order(int N, int E, const double* knt, const int* conn, int* node_perm, int* elem_perm);
// Edge graph of a tetrahedral mesh: node i's neighbours (nodes sharing an edge with it), ascending,
// without i itself
void node_graph(int N, int E, const int* conn, std::vector<int>& ptr, std::vector<int>& col);
// Reverse Cuthill-McKee order of a graph (src/reorder_mesh.py:53-83): unvisited nodes start a
// component in the order `seeds` (nodes by increasing degree); each component is traversed
// breadth-first, the newly reached neighbours of every node ordered by increasing degree (stable, so
// equal degrees keep ascending node order); the visit order reversed is the permutation.
void rcm_order(int N, const std::vector<int>& ptr, const std::vector<int>& col, const int* seeds, int* perm);

// Poisson stiffness with Dirichlet identity rows/columns and regularisation (src/amg_utils.py:21-84)
HostCSR assemble_poisson(int N, int E, const int* conn, const double* volume, const double* grad_phi,
                         const double* mask, double reg);
EnergyOp assemble_energy(int N, int E, const int* conn, const double* volume, const double* grad_phi,
                         const int* mat_id, int n_mat, const double* A, const double* K1, const double* Js,
                         const double* k_easy);

// Magnetoelastic entries of an assembled operator (src/energy_kernels.py:212-224): per element
// Kx_Ve = 2 (k1me + k1me_p) Ve / 20, Ky_Ve = 2 (k1me - k1me_p) Ve / 20 (arrays of length n <= E,
// zero beyond; k1me_p may be null).  Elements with a non-zero constant must belong to the operator.
void assemble_magnetoelastic(EnergyOp& op, int N, int E, const int* conn, const double* volume, const int* mat_id,
                             int n, const double* k1me, const double* k1me_p);

std::vector<AmgLevel> build_amg(const HostCSR& A, const AmgParams& prm);

// R (I - A S), S = diag(s): the restriction of the residual that a pre-smoothing from zero leaves,
// x = S b, r = b - A x, b_c = R r = R (I - A S) b, as one operator (exact zeros dropped, columns sorted)
HostCSR fused_restriction(const HostCSR& R, const HostCSR& A, const std::vector<double>& s);
// the same from the product RA = R A: R - (R A) S, with no second sparse product
HostCSR fused_restriction_ra(const HostCSR& R, const HostCSR& RA, const std::vector<double>& s);
std::vector<double> dense_inverse(const HostCSR& A);  // row-major n x n; throws on singular

}  // namespace mm
