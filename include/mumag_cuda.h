/* C-ABI of libmumag_cuda.so: the GB300 backend of the micromagnetic hot path of
 * MaMMoS-project/mumag_matrixfree2 (energy and gradient, demag Poisson solve, minimizer update).
 *
 * Conventions (those of the reference's own C-ABI, src/cpp/cpp_mkl_minimizer.cpp:26-764):
 *  - caller-owned contiguous arrays; float64; int32 zero-based indices; node vectors are (N,3)
 *    row-major with xyz interleaved (index 3*i+c);
 *  - inputs/outputs through pointers; no exception crosses the ABI;
 *  - every call returns an int status: 0 OK, > 0 a soft condition (MM_MAXITER, MM_NONFINITE,
 *    MM_BREAKDOWN), < 0 an error (see mm_status_str, and mm_last_error for the message);
 *  - host pointers unless the function name ends in _dev (then device pointers on the current
 *    device, e.g. torch tensors' data_ptr());
 *  - one CUDA stream per problem; a problem is not thread-safe, several problems may coexist.
 */
#ifndef MUMAG_CUDA_H
#define MUMAG_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MM_OK 0
#define MM_MAXITER 1
#define MM_NONFINITE 2
#define MM_BREAKDOWN 3
#define MM_ERR_ARG -1
#define MM_ERR_OOM -2
#define MM_ERR_CUDA -3
#define MM_ERR_STATE -4
#define MM_ERR_SETUP -5

#define MM_PRECOND_NONE 0
#define MM_PRECOND_JACOBI 1
#define MM_PRECOND_AMG 2   /* SA-AMG V-cycle, damped-Jacobi smoothing (reference "amg")        */
#define MM_PRECOND_AMGCL 3 /* SA-AMG V-cycle, SPAI0 smoothing (reference "amgcl", the default)  */

#define MM_METHOD_PCOHEN_HS 0
#define MM_METHOD_LBFGS 1
#define MM_METHOD_WG_NP 2
#define MM_METHOD_PLBFGS 3          /* preconditioned L-BFGS (src/minimizers.py:1526-1653)                */
#define MM_METHOD_COHEN 4           /* Cohen CG, PR beta, energy-based initial step (:642-720)            */
#define MM_METHOD_PCG 5             /* preconditioned CG, HS beta, d_prev not re-projected (:828-947)     */
#define MM_METHOD_PCOHEN 6          /* preconditioned Cohen CG, PR beta (:950-1073, beta_type "pr")       */
#define MM_METHOD_PCOHEN_EXACT 7    /* as PCOHEN with Cayley transport of d and g (:1081-1200, "pr")      */
#define MM_METHOD_PCOHEN_HS_EXACT 8 /* as PCOHEN_HS with Cayley transport (:1081-1200, "hs")             */
#define MM_METHOD_DPLBFGS 9         /* damped preconditioned L-BFGS (:1808-1968)                          */
#define MM_METHOD_TN_SPLIT 10       /* split truncated Newton, P d = -g_tan_ext (:1437-1517)              */
#define MM_METHOD_TR 11             /* trust-region Newton-CG on the local Hessian (:1994-2103)           */
#define MM_METHOD_PTR 12            /* preconditioned trust region on the full Hessian (:2129-2320)       */
#define MM_METHOD_AAPG 13           /* Anderson-accelerated preconditioned gradient (:2507-2636)          */
#define MM_METHOD_AAPG_EXACT 14     /* AAPG with Cayley transport of the history (:2395-2504)             */
#define MM_METHOD_PNAG 15           /* preconditioned Nesterov accelerated gradient (:2715-2803)          */
#define MM_METHOD_PCOHEN_LBFGS 16   /* Cohen CG over the L-BFGS-smoothed gradient (:2806-2924)            */
#define MM_METHOD_COUNT 17

typedef struct mm_problem mm_problem;

/* Minimizer parameters; field meanings follow LoopParams (src/hysteresis_loop.py:34-125). */
typedef struct {
  int method;           /* MM_METHOD_* */
  int max_iter;
  int pc_iters;
  int pc_auto;
  int ls_max_evals;     /* 15 in the reference's steps */
  int L;                /* CG restart period; <= 0 means N */
  int memory;           /* L-BFGS history */
  int wg_gamma;         /* BB: number of initial line-search steps */
  double tau_f, eps_a, tau0;
  double ls_eta1, ls_eta2, ls_C, ls_c;
  double pc_force_eta, pc_force_alpha, pc_stagnation_nu, pc_reg;
  double cg_tol;        /* tolerance of the initial Poisson solve */
  double phi_tol;       /* tolerance of the line-search Poisson solves; <= 0: min(cg_tol, 0.1 tau_f) */
  int cg_maxiter;
  int tn_iters;         /* inner iterations of TR / PTR; <= 0 means 5                                */
  double lr;            /* PNAG's initial line-search step; <= 0 means 0.1                           */
  double mu;            /* PNAG's momentum (0.9 in the reference)                                     */
  int phi_extrapolate;  /* PNAG: warm-start the look-ahead solve from 2 U - U_prev                    */
  int cpp_semantics;    /* pcohen_hs / pcohen only: the conventions of the reference's C++ minimizer
                           (--cpp-mkl, run_cpp_pcohen_hs_minimization, src/cpp/cpp_mkl_minimizer.cpp:
                           542-763): an inner solve on the initial state counted in preco_iters, inner
                           trips that stop on curvature or stagnation not counted, and the energy test
                           of the convergence check against the energy two iterations back         */
} mm_min_params;

typedef struct {
  int iters, evals, preco_iters, demag_iters;
  double E, gnorm, seconds;
  int status;
  double demag_seconds;       /* device time of the demag solves (CUDA events around each)            */
  double demag_wall_seconds;  /* host time spent in the demag solve calls (the rest is the minimizer's) */
  int device_loop;            /* 1: the iterations ran as one device graph (MM_OPT_MIN_GRAPH); the two
                                 demag times then cover the solve of the initial state only           */
} mm_min_info;

/* ---- setup helpers ------------------------------------------------------------------------ */

/* Orientation fix (swap local nodes 1,2 where det J < 0), volumes, inv(J)^T (E,3,3) and shape
 * gradients (E,4,3).  Replaces compute_volume_JinvT / compute_grad_phi_from_JinvT,
 * src/loop.py:56-102. */
int mm_geom_compute(int n_nodes, int n_elems, const double* knt, const int* conn_in, int* conn_out,
                    double* volume, double* JinvT, double* grad_phi);

/* Dirichlet mask: 0.0 on nodes of faces owned by one tetrahedron, else 1.0.
 * Replaces find_outer_boundary_mask, src/add_shell.py:105-136. */
int mm_boundary_mask(int n_nodes, int n_elems, const int* conn, double* mask);

/* Morton (10 bits per axis) node and element permutations (stable on equal keys).
 * Replaces the target="gpu" branch of reorder_mesh, src/reorder_mesh.py:19-30,85-100. */
int mm_morton_order(int n_nodes, int n_elems, const double* knt, const int* conn, int* node_perm,
                    int* elem_perm);

/* Degrees of the mesh's edge graph (nodes sharing an edge, the node itself excluded). */
int mm_node_degrees(int n_nodes, int n_elems, const int* conn, int* degree);
/* Reverse Cuthill-McKee node permutation of the mesh's edge graph: unvisited nodes start a
 * breadth-first component in the order `seeds` (the nodes by increasing degree; NULL sorts them
 * stably by degree), the newly reached neighbours of each node are ordered by increasing degree,
 * equal degrees by node number, and the visit order reversed is node_perm.  Replaces the
 * target="cpu" branch of reorder_mesh (src/reorder_mesh.py:53-83), whose call of scipy's
 * reverse_cuthill_mckee passes a keyword scipy does not have; this orders the symmetric edge graph,
 * as scipy.sparse.csgraph.reverse_cuthill_mckee does given the same seed order. */
int mm_rcm_order(int n_nodes, int n_elems, const int* conn, const int* seeds, int* node_perm);

/* ---- host-only setup (no GPU needed): the assembled operators and the SA hierarchy --------- */

typedef struct mm_setup mm_setup;

/* Assemble the energy operator and (when reg >= 0) the Poisson matrix with its SA hierarchy on the
 * host, exactly as mm_create + mm_build_poisson do.  Lets a caller inspect or reuse the setup. */
int mm_setup_create(int n_nodes, int n_elems, const int* conn, const double* volume, const double* grad_phi,
                    const int* mat_id, int n_mat, const double* A_lookup, const double* K1_lookup,
                    const double* Js_lookup, const double* k_easy, const double* boundary_mask, double reg,
                    int max_levels, int max_coarse, mm_setup** out);
int mm_setup_destroy(mm_setup* s);
/* Energy operator: magnetic rows, entries per row (col, material), exchange w, anisotropy q,
 * demag gradient G (3 per entry) and demag source D (3 per entry). */
int mm_setup_energy_info(mm_setup* s, int* n_rows, int64_t* nnz, int* single_axis);
int mm_setup_energy_export(mm_setup* s, int* rows, int* ptr, int* col, int* mat, double* w, double* q,
                           double* G, double* D, double* diag_exchange);
int mm_setup_levels(mm_setup* s, int* n_levels);
int mm_setup_level_info(mm_setup* s, int level, int* n, int64_t* nnz_A, int64_t* nnz_P, int* n_cols_P);
int mm_setup_level_export(mm_setup* s, int level, int* A_ptr, int* A_col, double* A_val, int* P_ptr,
                          int* P_col, double* P_val, int* agg);

/* ---- problem ------------------------------------------------------------------------------ */

/* Upload an oriented mesh with its materials (reduced units) and assemble the energy operator.
 * M_nodal: sum_e Js_e Ve / 4 per node; boundary_mask may be NULL (then the Poisson solve projects
 * out the mean, as make_solve_U does without a mask, src/poisson_solve.py:535-536).
 * The problem lives on the CUDA device current at this call; every entry point taking the problem
 * makes that device current for the call and restores the caller's device on return.
 * Replaces make_energy_kernels (src/energy_kernels.py:82-142) and the operator assembly of
 * src/amg_utils.py:741-789 / src/loop.py:1133-1166. */
int mm_create(int n_nodes, int n_elems, const int* conn, const double* volume, const double* grad_phi,
              const int* mat_id, int n_mat, const double* A_lookup, const double* K1_lookup,
              const double* Js_lookup, const double* k_easy, double V_mag, const double* M_nodal,
              const double* boundary_mask, mm_problem** out);
int mm_destroy(mm_problem* h);

/* Assemble the Poisson matrix (src/amg_utils.py:21-84) and build the preconditioner
 * (src/poisson_solve.py:566-639).  max_levels / max_coarse bound the SA hierarchy. */
int mm_build_poisson(mm_problem* h, double reg, int precond_type, int max_levels, int max_coarse,
                     int* n_levels);
/* Hierarchy introspection (tests): rows, nnz(A), nnz(P) of level l. */
int mm_amg_level_info(mm_problem* h, int level, int* n, int64_t* nnz_A, int64_t* nnz_P);
/* Copy level l's operator (CSR) and aggregates (n, -1 = none; all -1 on the coarsest level). */
int mm_amg_export_level(mm_problem* h, int level, int* A_ptr, int* A_col, double* A_val, int* agg);

/* Energy and gradient: E = 1/2 m.(g + g_z) / V_mag, g = (K m + G U + g_z) / V_mag with
 * g_z = -2 M_nodal (B_ext + B_bias).  B_bias may be NULL.
 * Replaces energy_and_grad (src/energy_kernels.py:147-180,340-459) and the C++
 * evaluate_energy_and_grad (src/cpp/cpp_mkl_minimizer.cpp:178-206). */
int mm_energy_grad(mm_problem* h, const double* m, const double* U, const double* B_ext,
                   const double* B_bias, double* E, double* g);
int mm_energy_grad_dev(mm_problem* h, const double* d_m, const double* d_U, const double* B_ext,
                       const double* d_B_bias, double* E, double* d_g);

/* Energy and gradient for callers that cannot allocate device memory at call time: an application
 * that owns all device memory through a fixed pool reserved at start-up and forbids allocations
 * while it runs (a cudaMalloc there could fail or stall the other work sharing the device).
 * No counterpart in the reference: it is mm_energy_grad_dev with the scratch of its energy
 * reduction (one partial per block of 32 magnetic rows, a ticket counter and the total) held in a
 * file-scope static device array of MM_NOALLOC_SCRATCH_BYTES instead of the problem's workspace,
 * and it calls no allocating routine.  Inputs and outputs are caller-owned device pointers
 * (d_B_bias may be NULL); E is a host pointer, written after the problem's stream is synchronized.
 * Limit: at most MM_NOALLOC_MAX_ROWS magnetic rows (larger problems get MM_ERR_ARG).
 * The work runs on the problem's device (the device current at mm_create, as for every entry point).
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress) for that
 * device; make that first call before any stream capture.  Every call shares the one array (its
 * ticket counter is cleared by each call), so calls that may overlap on the GPU — from different
 * streams or problems — race and must be serialized by the caller. */
#define MM_NOALLOC_MAX_ROWS 1048576
#define MM_NOALLOC_SCRATCH_BYTES 262400
int mm_energy_grad_noalloc(mm_problem* h, const double* d_m, const double* d_U, const double* B_ext,
                           const double* d_B_bias, double* E, double* d_g);

/* Exchange + anisotropy Hessian action C v / V_mag.
 * Replaces local_grad_only (src/energy_kernels.py:190-195,272-338). */
int mm_local_grad(mm_problem* h, const double* v, double* out);

/* Inner preconditioned CG with the Steihaug exit on P y = g_tan_ext (N,3 host arrays; P the projected
 * local Hessian of the state m for the full gradient g_ext, Jacobi preconditioner inv_M_prec of
 * mm_set_node_weights), y = result.  Replaces solve_Py_g, src/cpp/cpp_mkl_minimizer.cpp:233-359
 * (make_preconditioner_op.solve_Py_g, src/minimizers.py:413-490): at most max_iter iterations, stop
 * at r.z <= tol^2 r0.z0, stagnation when 0.5 alpha rho <= stagnation_nu Q, y clipped to 10 |z_fb|,
 * z_fb = g_tan_ext .* inv_M_prec when y is no descent direction.  *iters counts as the C++ function
 * counts (a trip that stops on curvature or stagnation is not counted).  FP32 when the problem's
 * inner precision is FP32. */
int mm_solve_py_g(mm_problem* h, const double* m, const double* g_ext, const double* g_tan_ext, int max_iter,
                  double tol, double reg, double stagnation_nu, double* y, int* iters);

/* Diagonal of the exchange operator / V_mag (src/energy_kernels.py:492-566). */
int mm_exchange_diagonal(mm_problem* h, double* d);

/* Demag right-hand side b = D m (src/poisson_solve.py:173-186,254-280) and b.b. */
int mm_rhs(mm_problem* h, const double* m, double* b, double* bnorm2);

/* Poisson operator y = A U (src/poisson_solve.py:166-171,210-252). */
int mm_apply_A(mm_problem* h, const double* U, double* y);

/* One preconditioner application z = M^-1 r (src/amg_utils.py:491-623). */
int mm_precond(mm_problem* h, const double* r, double* z);

/* Demag solve: b = D m, PCG from U_inout to relative residual tol (recursive residual, as
 * src/poisson_solve.py:422-478), U_inout <- U.  rel_res = sqrt(r.r / b.b).
 * Returns MM_MAXITER when maxiter was reached first.
 * Replaces solve_U (src/poisson_solve.py:748-771) and the C++ solve_poisson
 * (src/cpp/cpp_mkl_minimizer.cpp:208-231). */
int mm_solve_u(mm_problem* h, const double* m, double* U_inout, double tol, int maxiter, int* iters,
               double* rel_res);
int mm_solve_u_dev(mm_problem* h, const double* d_m, double* d_U_inout, double tol, int maxiter,
                   int* iters, double* rel_res);
/* As mm_solve_u with the warm start x0 left untouched and U written to U_out (host arrays; solve_U's
 * (m, x0) -> U of src/poisson_solve.py:748-771 without a host-side copy of x0). */
int mm_solve_u_x0(mm_problem* h, const double* m, const double* x0, double* U_out, double tol, int maxiter,
                  int* iters, double* rel_res);

/* Magnetoelastic anisotropy (src/energy_kernels.py:212-224,319-329,411-426): per element
 * Kx_Ve = 2 (k1me + k1me_p) Ve / 20 and Ky_Ve = 2 (k1me - k1me_p) Ve / 20 (arrays of n <= n_elems
 * entries, zero beyond; k1me_p may be NULL) add g_a,x += Kx_Ve (sum_b m_b,x + m_a,x) and likewise y
 * to the energy gradient and to the local Hessian.  n = 0 removes the term. */
int mm_set_magnetoelastic(mm_problem* h, int n, const double* k1me, const double* k1me_p);

/* Add the multiple of a correction that minimises the energy-norm error of an initial guess:
 * d_U += alpha d_c with alpha = c.(b - A U) / (c.A c), b = D m (never worse than U alone in the A-norm).
 * Used to apply a predicted potential change (the learned warm start) before a solve.  No counterpart
 * in the reference.  alpha may be NULL. */
int mm_scale_correction_dev(mm_problem* h, const double* d_m, double* d_U, const double* d_c, double* alpha);
/* The same correction queued on the problem's stream after the work already queued on `after` (a
 * cudaStream_t, e.g. the network's from mm_unet_predict_dev; NULL = the legacy default stream), with
 * alpha computed and applied on the device: no host wait, so the next solve follows directly. */
int mm_scale_correction_async(mm_problem* h, void* after, const double* d_m, double* d_U, const double* d_c);

/* Override the node weights of the minimizers (default: inv_M_rel = V_mag / M_nodal where
 * M_nodal > 1e-20 else 0; inv_M_prec = 1/d where d > 1e-20 else 1, d the exchange diagonal,
 * src/hysteresis_loop.py:340-353).  Either pointer may be NULL to keep the default. */
int mm_set_node_weights(mm_problem* h, const double* inv_M_rel, const double* inv_M_prec);

/* Per-node bias field (N,3, host) added to the applied field in every energy evaluation of
 * mm_minimize, as sparse_ops["B_bias"] does in the reference (src/minimizers.py:3444-3445,
 * src/energy_kernels.py:169-171); NULL removes it. */
int mm_set_bias_field(mm_problem* h, const double* B_bias);

/* Minimize the energy for one applied field, m_inout and U_inout updated in place.
 * Replaces make_minimizer(...).minimize (src/minimizers.py:2927-4098) for every method of the
 * reference's CLI (MM_METHOD_*), and run_cpp_pcohen_hs_minimization
 * (src/cpp/cpp_mkl_minimizer.cpp:542-763). */
int mm_minimize(mm_problem* h, const double* B_ext, double* m_inout, double* U_inout,
                const mm_min_params* prm, mm_min_info* info);
/* As mm_minimize with the state in device memory (d_m_inout (N,3), d_U_inout (N)), updated in place:
 * a field sweep keeps m and U on the GPU between field steps (B_ext stays a host array of 3). */
int mm_minimize_dev(mm_problem* h, const double* B_ext, double* d_m_inout, double* d_U_inout,
                    const mm_min_params* prm, mm_min_info* info);

/* Time one hot kernel in isolation: `reps` launches on the problem's stream, each preceded by a
 * write of a buffer larger than L2 (so every launch streams its operands from HBM), timed with CUDA
 * events around the launch.  Returns the mean launch time and the algorithmic bytes per launch
 * (every array counted once at its stored width).  kernel: MM_KERNEL_*. */
#define MM_KERNEL_SPMV_A 0   /* level-0 product y = A x                                   */
#define MM_KERNEL_SMOOTH 1   /* level-0 SPAI0 smoothing x' = x + s .* (b - A x)           */
#define MM_KERNEL_ENERGY 2   /* energy + gradient over the magnetic rows                  */
#define MM_KERNEL_HESSIAN 3  /* local Hessian action over the magnetic rows               */
int mm_time_kernel(mm_problem* h, int kernel, int reps, double* ms_per_launch, double* bytes_per_launch);

/* Solver options.  MM_OPT_GRAPH (default 1): run the PCG iterations inside a CUDA graph whose
 * conditional WHILE node loops on the device until convergence; 0 polls the device flag from the
 * host every four iterations (same kernels, same results). */
#define MM_OPT_GRAPH 1
/* MM_OPT_PRECISION (before mm_build_poisson): MM_PRECISION_FP64 (default) is the reference's plain
 * FP64 PCG; MM_PRECISION_MIXED keeps U, the right-hand side and the true residual in FP64 and solves
 * each correction with an FP32 copy of the hierarchy (FP32 products, FP64 inner products), repeating
 * until the FP64 residual meets the same tolerance (iterative refinement). */
#define MM_OPT_PRECISION 2
#define MM_PRECISION_FP64 0
#define MM_PRECISION_MIXED 1
/* MM_PRECISION_FP32_PRECOND: the FP64 PCG of the plain method (iterate, residual, directions, the
 * products with the finest operator and every inner product in FP64, the same stopping test), with
 * the V-cycle preconditioner applied in FP32 on a copy of the hierarchy. */
#define MM_PRECISION_FP32_PRECOND 2
/* MM_OPT_MIXED_ETA_E6: relative residual reduction asked of each FP32 correction solve, in units of
 * 1e-6 (default 10, i.e. 1e-5). */
#define MM_OPT_MIXED_ETA_E6 3
/* MM_OPT_GRID_CAP: largest grid (blocks of 256 threads) of the one-row-per-thread kernels; beyond
 * it they loop (default 4096).  Process-wide; fixed values keep every reduction deterministic. */
#define MM_OPT_GRID_CAP 4
/* MM_OPT_PROFILE (default 0): 1 runs every demag solve with the host-polled loop (synchronising
 * after each direction/step pair, so no launch runs after convergence) and records a CUDA event pair
 * around every solver launch; each launch's device time is added to a slot named by its kind, AMG
 * level and precision.  For measurement only: the loop is slower than the graph. */
#define MM_OPT_PROFILE 5
/* Options 6 and 7 are unused (they selected a one-launch persistent PCG loop, since removed). */
/* MM_OPT_PDL (default 1): launch the solver kernels with programmatic dependent launch, so each
 * kernel is scheduled while its predecessor drains (every solver kernel waits for its predecessor's
 * results at entry); 0 launches them normally.  Same results either way. */
#define MM_OPT_PDL 8
/* MM_OPT_COARSE_FUSE (bit mask, default 1): with 3 or more levels, at most 256 rows on the coarsest
 * level and at most 4Mi entries in the n(L-2) x n(L-1) dense factors (so that they cost little memory
 * and host setup time), the two coarsest levels of the V-cycle (level L-2's residual, restriction,
 * the dense coarsest solve, prolongation and post-smoothing: five dependent kernels) run as two
 * kernels applying the same linear map in factored form, x2 = T b + W (Z b) with T = 2S - S A S,
 * W = (I - S A) P and Z = Ainv R (I - A S) (S the smoother diagonal; T sparse with A's pattern, W and Z
 * dense, formed at mm_build_poisson).  Bit 0: in the FP64 solver, bit 1: in the FP32 solver of the
 * mixed method.  Same V-cycle up to summation order.  (80 nm cube on GB300: the FP64 solve 7 % faster,
 * the FP32 iteration unchanged; mm_autotune measures it per problem.) */
#define MM_OPT_COARSE_FUSE 9
/* MM_OPT_MIN_FP32: precision of the minimizer's inner preconditioner solve (the Steihaug PCG on the
 * local Hessian P y = g of mm_minimize).  -1 (default) follows MM_OPT_PRECISION: FP32 entries, vectors
 * and float-float inner products when the demag solve is MM_PRECISION_MIXED or
 * MM_PRECISION_FP32_PRECOND, FP64 otherwise; 0 always FP64; 1 always FP32.  The energy, the gradient,
 * the outer iteration and the line search stay FP64 in every case. */
#define MM_OPT_MIN_FP32 10
/* MM_OPT_SPLIT_A0 (default 1): in MM_PRECISION_FP32_PRECOND, the finest-level product A0 z of the
 * FP64 PCG (z the FP32 V-cycle's output, exact in FP32) runs on the operator split into FP32 pairs
 * a = hi + lo and sums in float-float (error ~2^-47 sum |a z|) on the FP32 pipes; 0 takes it in FP64. */
#define MM_OPT_SPLIT_A0 11
/* MM_OPT_FUSE_RESTRICT (bit mask, default 3): the V-cycle restricts with R_l (I - A_l S_l), formed
 * once on the host, instead of a residual pass A_l followed by R_l: the pre-smoothing from zero
 * makes x_l = S_l b_l, so b_{l+1} = R_l (b_l - A_l x_l) is one product with one operator (one kernel
 * less per level, and fewer bytes than A_l and R_l together).  Bit 0 the FP64 solver, bit 1 the FP32
 * one; mm_autotune keeps a bit only if the V-cycle is faster with it. */
#define MM_OPT_FUSE_RESTRICT 12
/* MM_OPT_ENERGY_FF: energy and gradient evaluations in float-float (every stored value and the vectors
 * m, U and k.m as FP32 pairs hi + lo, products and row sums on the FP32 pipes with about 2^-48
 * relative error per term; the row totals, gradient and energy sum in FP64).  -1 (default) follows
 * MM_OPT_PRECISION (on in MM_PRECISION_MIXED and MM_PRECISION_FP32_PRECOND), 0 FP64, 1 float-float.
 * Problems with several easy axes or a magnetoelastic term always evaluate in FP64. */
#define MM_OPT_ENERGY_FF 13
/* MM_OPT_MIN_GRAPH (default 1): mm_minimize runs the iterations of pcohen_hs, pcohen and pcg as one
 * CUDA graph: the minimizer loop is a conditional WHILE node, the inner preconditioner solve, the
 * Armijo trials and each trial's demag PCG are WHILE nodes nested in it, and the decisions between
 * kernels (forcing tolerance, clipping and fallback, beta, descent test, step expansion and
 * contraction, the U1-U4 test) are single-thread kernels, so a call waits on the host once.  Same
 * kernels, grids and reductions as the host-driven loop (0), hence the same results; the host loop
 * runs for the other methods, with MM_OPT_PROFILE, without MM_OPT_GRAPH and in MM_PRECISION_MIXED
 * (whose refinement steps are decided on the host). */
#define MM_OPT_MIN_GRAPH 14
/* MM_OPT_ENERGY_FF_LANES: lanes per magnetic row of the float-float energy kernel (1, 2, 4 or 8;
 * default 4; mm_autotune times each with L2 flushed and keeps the fastest). */
#define MM_OPT_ENERGY_FF_LANES 15
/* MM_OPT_COARSE_CYCLE (bit mask, default 0; mm_autotune keeps what is faster): with four levels, the
 * fused restriction at level 1 and the fused coarse correction, the V-cycle runs levels 1 .. 3 (the
 * level-1 restriction, both coarse-correction phases, the level-1 prolongation and post-smoothing)
 * in one cooperative launch with grid barriers instead of five launches; bit-identical results.
 * Bit 0 the FP64 solver, bit 1 the FP32 solver. */
#define MM_OPT_COARSE_CYCLE 16
/* MM_OPT_CSR_LANES (after mm_build_poisson): every compressed-row operator of the hierarchy (coarse
 * levels, R, P and the fused restrictions) read with this many lanes per row (2, 4, 8, 16 or 32);
 * mm_autotune chooses per operator among these and one thread per row. */
#define MM_OPT_CSR_LANES 17
/* MM_OPT_SA_THETA_E3 (before mm_build_poisson): the smoothed-aggregation strength threshold on the
 * finest level in thousandths; 0 (default): 0.115, or 0.1 when 0.115 gives more than four levels. */
#define MM_OPT_SA_THETA_E3 18
/* MM_OPT_SA_FACTOR_E3 (before mm_build_poisson): each coarser level's strength threshold as a
 * multiple of the finer level's, in thousandths; 0 (default): 0.35. */
#define MM_OPT_SA_FACTOR_E3 19
/* MM_OPT_SA_FILTER_E6 (before mm_build_poisson): the level-1 operator's weak couplings
 * (|a_ij| + |a_ji| < 2 eps sqrt(|a_ii a_jj|)) moved into its diagonal, eps in millionths; 0 (default):
 * 0.002; negative: the plain Galerkin operator. */
#define MM_OPT_SA_FILTER_E6 20
int mm_set_option(mm_problem* h, int option, int value);
/* The current value of MM_OPT_COARSE_CYCLE, MM_OPT_FUSE_RESTRICT, MM_OPT_COARSE_FUSE,
 * MM_OPT_ENERGY_FF_LANES or MM_OPT_MIN_GRAPH (after mm_autotune, or after a loop graph that could not
 * hold the cooperative launch turned MM_OPT_COARSE_CYCLE off). */
int mm_get_option(mm_problem* h, int option, int* value);

/* Autotuner (after mm_build_poisson): for every compressed-row operator of the hierarchy (coarse levels,
 * restrictions, prolongations; both precisions) tries 2, 4, 8, 16 and 32 lanes per row, each timed as
 * whole V-cycles so that cache state and neighbouring kernels are those of a solve, and keeps the
 * fastest when it beats the heuristic's shape by more than 3 %; then times the V-cycle with and without the fused coarse correction in each solver and
 * sets MM_OPT_COARSE_FUSE accordingly.  CUDA events on the problem's stream, `reps`
 * launches per candidate.  A JSON report (candidates, times in microseconds, choices) is written to
 * `report` (may be NULL; truncated to report_len - 1 characters).  No counterpart in the reference. */
int mm_autotune(mm_problem* h, int reps, char* report, int report_len);

/* In-solve kernel profile (MM_OPT_PROFILE).  slot = (fp32 * MM_PROF_LEVELS + level) * MM_PROF_KINDS
 * + kind.  No reference counterpart: measurement of this backend's own kernels. */
#define MM_PROF_PCG_DIR 0       /* y = A z ; p = z + beta p ; Ap = y + beta Ap ; p.Ap (level 0)   */
#define MM_PROF_PCG_STEP 1      /* x += alpha p ; r -= alpha Ap ; r.r ; pre-smoothing s .* r      */
#define MM_PROF_VC_RESIDUAL0 2  /* level-0 residual r - A x of the V-cycle                        */
#define MM_PROF_RESIDUAL 3      /* residual b - A x on a coarse level                            */
#define MM_PROF_RESTRICT 4      /* b_c = R res, fused with the coarse pre-smoothing              */
#define MM_PROF_COARSE 5        /* dense coarsest solve x = Ainv b                                */
#define MM_PROF_PROLONG 6       /* x += P e                                                      */
#define MM_PROF_SMOOTH0 7       /* level-0 post-smoothing fused with r.z                          */
#define MM_PROF_SMOOTH 8        /* post-smoothing on a coarse level                              */
#define MM_PROF_INIT_RESIDUAL 9 /* r = b - A x at the start of a PCG solve                        */
#define MM_PROF_COARSE_A 10     /* fused coarse correction: t = T b and z = Z b (level L-2)        */
#define MM_PROF_COARSE_B 11     /* fused coarse correction: x2 = t + W z (level L-2)               */
#define MM_PROF_COARSE_CYCLE 12 /* levels 1 .. 3 in one cooperative launch (MM_OPT_COARSE_CYCLE)   */
#define MM_PROF_KINDS 13
#define MM_PROF_LEVELS 16
#define MM_PROF_SLOTS (2 * MM_PROF_LEVELS * MM_PROF_KINDS)
/* Copy the per-slot totals since the last reset: launches, summed device time [ms] and the
 * algorithmic bytes of one launch (every array counted once at its stored width, padding excluded).
 * Each array holds MM_PROF_SLOTS entries. */
int mm_profile_read(mm_problem* h, int64_t* launches, double* total_ms, double* bytes_per_launch);
int mm_profile_reset(mm_problem* h);
/* Refinement steps (FP32 correction solves) of the last mixed-precision solve. */
int mm_last_refinements(mm_problem* h, int* steps);

/* Device time of the last demag solve (mm_solve_u / mm_solve_u_dev), measured with CUDA events
 * recorded on the problem's stream around all of its kernels (host<->device copies excluded). */
int mm_last_solve_ms(mm_problem* h, double* ms);
/* Number of kernels this problem has launched since it was created. */
int mm_launch_count(mm_problem* h, int64_t* count);

/* ---- learned demag warm start ----------------------------------------------------------------
 * No counterpart in the reference: a 3D U-Net (15 convolutions 3x3x3, 4 levels, 16/32/64/128
 * channels, ReLU, 2x2x2 average pooling, nearest upsampling with added skips) over a G^3 voxel grid
 * maps the voxelised change of magnetisation (3 channels) and the previous potential (1 channel) to
 * the change of the demag potential (output channel 0).  BF16 weights and activations, FP32
 * accumulation, FP32 master weights trained with Adam; convolutions on tcgen05 tensor cores.
 * Parameters are one flat FP32 vector: for each layer in order w[27][c_in][c_out] (tap =
 * (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[c_out].  Voxel arrays are z-major with x fastest. */
#define MM_UNET_LAYERS 15
typedef struct mm_unet mm_unet;
/* grid: level-0 edge G (multiple of 8, 16..256); batch: largest number of samples per call. */
int mm_unet_create(int grid, int batch, mm_unet** out);
int mm_unet_destroy(mm_unet* u);
const char* mm_unet_last_error(mm_unet* u);
int mm_unet_param_count(mm_unet* u, int64_t* n);
int mm_unet_set_params(mm_unet* u, const float* params);  /* also resets the Adam state */
int mm_unet_get_params(mm_unet* u, float* params);
int mm_unet_get_grads(mm_unet* u, float* grads);           /* of the last mm_unet_backward */
/* x: [nb][G^3][4] FP32 host array; y (may be NULL): [nb][G^3] output channel 0. */
int mm_unet_forward(mm_unet* u, const float* x, int nb, float* y);
/* The _dev entry points below read and write the caller's device arrays on the network's own stream
 * after the work queued so far on the legacy default stream (a caller that writes them on another
 * stream synchronises that stream first); every call but the graph forward waits for its results.
 * Device-pointer variant; d_x NULL runs on the input already voxelised by mm_unet_voxelise_dev.  With
 * d_x and d_y both NULL (the in-solve path) the forward runs as a CUDA graph (captured at the second
 * such call for each batch size <= 8) and the call does not wait: a convolution's error is reported
 * by the next waiting call (mm_unet_interp_add_dev, mm_unet_sync). */
int mm_unet_forward_dev(mm_unet* u, const float* d_x, int nb, float* d_y);
/* Mean squared error of output channel 0 against target [nb][G^3] over the samples of the last
 * forward, and the gradient of every parameter. */
int mm_unet_backward(mm_unet* u, const float* target, int nb, double* loss);
int mm_unet_backward_dev(mm_unet* u, const float* d_target, int nb, double* loss);
int mm_unet_adam(mm_unet* u, float lr, float beta1, float beta2, float eps);
/* on = 0: bias gradients are zero, so biases keep the values set (zero biases make the network
 * positively homogeneous, f(a x) = a f(x) for a > 0, which the warm start relies on). */
int mm_unet_set_bias_training(mm_unet* u, int on);
/* Mesh -> grid: input channels of voxel v of `sample` = sum_k w4[v][k] * (scale3 f3[idx4[v][k]][0..2],
 * scale1 f1[idx4[v][k]]) over its 4 nodes (idx < 0 ends the list); device pointers, n_vox = G^3. */
int mm_unet_voxelise_dev(mm_unet* u, int sample, int n_vox, const int* d_idx4, const float* d_w4,
                         const double* d_f3, const double* d_f1, double scale3, double scale1);
/* Grid -> mesh: d_U[node[j]] += scale * sum_k w8[j][k] y0(voxel idx8[j][k]), j < n. */
int mm_unet_interp_add_dev(mm_unet* u, int sample, int n, const int* d_node, const int* d_idx8,
                           const float* d_w8, double scale, double* d_U);
/* Introspection (tests): tensor `which` (0..21, in forward order: input, e0a, s0, pool0, ..., output)
 * lives on level `level` with `channels` channels; read one sample's activations (grad = 0) or their
 * gradients (grad = 1) as FP32 [G_level^3][channels]. */
int mm_unet_tensor_info(int which, int* level, int* channels);
int mm_unet_read_tensor(mm_unet* u, int which, int grad, int sample, float* out);
int mm_unet_sync(mm_unet* u);
/* The in-solve prediction without a host wait (no counterpart in the reference): the network's stream
 * first waits for the work queued on `after` (a cudaStream_t; NULL = the legacy default stream), then
 * voxelises (f3a - f3b, f1) into sample 0 as mm_unet_voxelise_dev does (f3b may be NULL), runs the
 * forward graph, zeroes d_out[0..n_out) and adds the prediction at the grid's nodes as
 * mm_unet_interp_add_dev does.  *stream_out (may be NULL) receives the network's stream so that a
 * consumer can queue after it; convolution errors are reported by the next waiting call. */
int mm_unet_predict_dev(mm_unet* u, void* after, int sample, int n_vox, const int* d_idx4, const float* d_w4,
                        const double* d_f3a, const double* d_f3b, const double* d_f1, double scale3, double scale1,
                        int n, const int* d_node, const int* d_idx8, const float* d_w8, double scale, int n_out,
                        double* d_out, void** stream_out);

/* Wait for the problem's stream. */
int mm_sync(mm_problem* h);
const char* mm_status_str(int status);
const char* mm_last_error(mm_problem* h);
/* Library version string. */
const char* mm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MUMAG_CUDA_H */
