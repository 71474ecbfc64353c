// C-ABI of libmumag_cuda.so: problem handle, device buffers, Poisson PCG with the SA-AMG
// V-cycle, energy operators and the minimizers, all orchestrated on one CUDA stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <mutex>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/mumag_cuda.h"
#include "mm_kernels.cuh"
#include "mm_setup.h"

using mmk::BS;
using mmk::MAXG;

namespace {

struct Fail {
  int code;
  std::string msg;
};

#define CK(x)                                                                                         \
  do {                                                                                                \
    cudaError_t e_ = (x);                                                                             \
    if (e_ != cudaSuccess)                                                                            \
      throw Fail{e_ == cudaErrorMemoryAllocation ? MM_ERR_OOM : MM_ERR_CUDA,                          \
                 std::string(#x) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +           \
                     std::to_string(__LINE__) + ")"};                                                 \
  } while (0)

#define LAUNCH_CHECK()      \
  do {                      \
    ++h->n_launch;          \
    CK(cudaGetLastError()); \
  } while (0)

// Upper bound on the blocks of a one-row-per-thread kernel (grid-stride beyond it); a tunable of
// the problem (MM_OPT_GRID_CAP), fixed per run so reductions stay deterministic.
int g_elem_cap = MAXG;
inline int grid_elem(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + BS - 1) / BS, g_elem_cap));
}
// Blocks of the minimizer's vector kernels (FP64 block reductions): about four per SM with several
// elements per thread, so that the FP64 shuffle trees (a warp-wide FP64 add holds the SM's FP64 pipe
// for 16 cycles) stay a small part of the launch.  Set from the device's SM count at problem creation.
int g_vec_cap = 608;
inline int grid_vec(int64_t n) { return std::min(grid_elem(n), g_vec_cap); }
// grid of the kernels that keep mmk::ILP rows per thread in flight
inline int grid_ilp(int64_t n) {
  const int64_t per = (int64_t)BS * mmk::ILP;
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, g_elem_cap));
}
inline int grid_rows(int64_t n, int tpr) {
  const int rpb = BS / tpr;
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + rpb - 1) / rpb, MAXG));
}

int pick_tpr(int64_t nnz, int64_t rows) {
  const double avg = rows > 0 ? (double)nnz / (double)rows : 1.0;
  if (avg <= 3.0) return 2;
  if (avg <= 10.0) return 4;
  if (avg <= 24.0) return 8;
  if (avg <= 48.0) return 16;
  return 32;
}

// A level operator on the device, in one of two layouts:
//  * sliced ELL, slice height 32, one thread per row (tpr == 1): large matrices with short rows;
//    padding entries carry value 0 and a valid column;
//  * compressed rows with tpr lanes per row (2..32): small matrices with long rows.
template <class T>
struct DevMatT {
  mmk::SellT<T> s{};
  mmk::CsrT<T> c{};
  int tpr = 1;
  int64_t nnz = 0;     // stored non-zeros (without padding)
  int64_t stored = 0;  // entries including padding
};

template <class T>
struct LevelT {
  DevMatT<T> A, P, R;
  DevMatT<T> Rf;     // fused restriction R (I - A S) (levels below the coarsest), empty when not formed
  T* s = nullptr;    // smoother diagonal (SPAI0, or omega/(diag+eps) for Jacobi)
  T* b = nullptr;    // right-hand side (levels >= 1)
  T* x = nullptr;    // iterate (pre-smoothing, prolongation)
  T* x2 = nullptr;   // post-smoothed iterate (levels >= 1)
  T* res = nullptr;  // residual
  int n = 0;
};

// One PCG + preconditioner context in one precision: FP64 for the plain method, FP32 for the inner
// correction solves of the mixed-precision method.  Reductions are always FP64 (Scalars).
template <class T>
struct SolverT {
  bool built = false;
  std::vector<LevelT<T>> lv;
  T* Ainv = nullptr;  // dense inverse of the coarsest level
  int n_coarse = 0;
  T* jac = nullptr;   // Jacobi preconditioner 1/(diag+eps)
  T *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr;
  mmk::Scalars* sc = nullptr;
  cudaGraph_t graph = nullptr;        // the PCG iteration loop, conditional WHILE node
  cudaGraphExec_t exec = nullptr;
  bool graph_failed = false;
  int64_t iter_launches = 0;          // kernels in one loop trip
  int epoch = 0;                      // advanced whenever the loop's launches change (graph dropped)
  // fused coarse correction of levels L-2 .. L-1 (x2 = T b + W (Z b)), when eligible
  bool fused = false;
  mmk::CsrT<T> Tm{};
  T *W = nullptr, *Z = nullptr, *tvec = nullptr, *zvec = nullptr;
  int fn = 0, fc = 0;
  int64_t Tm_nnz = 0;
  // one-launch coarse cycle (levels 1 .. 3): its grid barrier and its co-resident grid
  mmk::GridBar* bar = nullptr;
  int coop_grid = 0;     // blocks of the launch (the autotuner picks 1, 2, 4 or all co-resident per SM)
  int coop_max = 0;      // co-resident blocks of the whole GPU
  int sms = 0;
};

// Layout choice: one thread per row when the rows alone fill the GPU (>= 64Ki rows), else enough
// lanes per row to reach ~256Ki threads, capped by the average row length.
int choose_tpr(int64_t rows, int64_t nnz) {
  if (rows >= 65536) return 1;
  const double avg = rows > 0 ? (double)nnz / (double)rows : 1.0;
  int t = 2;
  while (t < 32 && (rows * t < 262144) && t < avg) t *= 2;
  return t;
}

thread_local std::string g_create_error;

// Pinned host blocks for the problems' scalar read-backs (Scalars, MinScal), kept in a process-wide
// free list and never returned: cudaFreeHost waits for the work of every stream on the device, so
// freeing them with each problem would stall all other problems whenever one is destroyed.
constexpr size_t PINNED_BLOCK = (std::max(sizeof(mmk::Scalars), sizeof(mmk::MinScal)) + 255) / 256 * 256;
std::mutex g_pinned_mu;
std::vector<void*> g_pinned_free;

void* pinned_get() {
  void* p = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    if (!g_pinned_free.empty()) {
      p = g_pinned_free.back();
      g_pinned_free.pop_back();
    }
  }
  if (!p) CK(cudaHostAlloc(&p, PINNED_BLOCK, cudaHostAllocPortable));
  std::memset(p, 0, PINNED_BLOCK);
  return p;
}

void pinned_put(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned_free.push_back(p);
}

}  // namespace

struct mm_problem {
  int device = -1;  // the CUDA device current at mm_create; every entry point runs its work there
  int N = 0, E = 0, n_mat = 0;
  double V_mag = 1.0, inv_Vmag = 1.0;
  cudaStream_t st = nullptr;
  std::vector<void*> allocs;
  std::string err;
  int64_t n_launch = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_solve_ms = 0.0;

  // in-solve kernel profile (MM_OPT_PROFILE): one event pair per tagged launch, folded into the
  // per-slot totals when the solve ends
  struct ProfRec {
    int slot;
    cudaEvent_t a, b;
  };
  bool prof = false;
  std::vector<ProfRec> prof_rec;
  std::vector<cudaEvent_t> prof_pool;
  size_t prof_used = 0;
  int64_t prof_n[MM_PROF_SLOTS] = {};
  double prof_ms[MM_PROF_SLOTS] = {};
  double prof_bytes[MM_PROF_SLOTS] = {};

  // host copies used by the setup
  std::vector<int> conn, mat_id;
  std::vector<double> volume, grad_phi, mask_h;
  bool has_mask = false;

  // energy operator
  mm::EnergyOp eop_h;
  mmk::EnergyDev eop{};
  int eop_tpr = 8;
  mmk::EnergySell eops{};          // the energy operator in sliced-ELL order (the kernels' layout)
  std::vector<int64_t> eops_pos;   // sliced position of every compressed-row entry
  int64_t eops_stored = 0;
  std::vector<double> kax_h;        // easy axes (n_mat, 3)
  mmk::EnergySell32 eops32{};      // FP32 exchange + anisotropy entries for the inner solve (lazy)
  bool eops32_ok = false;          // built and current (a new magnetoelastic term clears it)
  mmk::EnergySellFF eopsff{};      // float-float energy operator (mixed-precision energy evaluations)
  bool eopsff_ok = false;          // built and current (a new magnetoelastic term clears it)
  bool eopsff_failed = false;      // an entry lies outside the range of the float-float pairs
  int energy_ff = -1;              // MM_OPT_ENERGY_FF
  mmk::NodesFF w_ff{};             // the node records it gathers
  int eff_tpr = 4;                 // its lanes per magnetic row (mm_autotune)
  int min_fp32 = -1;               // MM_OPT_MIN_FP32
  double* d_Mn = nullptr;
  double* d_inv_M_rel = nullptr;
  double* d_inv_M_prec = nullptr;
  double* d_diag_ex = nullptr;

  // Poisson
  bool poisson_built = false;
  int precond = MM_PRECOND_AMGCL;
  double reg = 1e-12;
  std::vector<mm::AmgLevel> amg_h;
  SolverT<double> s64;           // plain FP64 method (and the outer residual of the mixed one)
  SolverT<float> s32;            // inner solves of the mixed-precision method
  bool mixed = false;            // MM_OPT_PRECISION = MM_PRECISION_MIXED
  bool fp32_precond = false;     // MM_OPT_PRECISION = MM_PRECISION_FP32_PRECOND
  bool split_a0 = true;          // MM_OPT_SPLIT_A0: FP32_PRECOND's A0 z with the split operator
  mmk::SellDF a0df{};            // A0 = hi + lo in FP32 pairs (built on first use)
  bool a0df_ok = false;
  double mixed_eta = 1e-5;       // relative reduction asked of each inner FP32 solve
  int mixed_max_outer = 12;
  int last_outer = 0;            // refinement steps of the last mixed solve
  double *d_b = nullptr, *d_x = nullptr, *d_r64 = nullptr;
  float *d_r32 = nullptr, *d_d32 = nullptr;
  double* d_part = nullptr;      // NRED x MAXG block partials (shared by every reduction)
  mmk::Scalars* d_sc = nullptr;  // scalars of the FP64 solver, the energy and the minimizer
  mmk::Scalars* d_sc32 = nullptr;
  mmk::Scalars* h_sc = nullptr;  // pinned
  bool use_graph = true;
  bool pdl = true;               // MM_OPT_PDL
  int coarse_fuse = 1;           // MM_OPT_COARSE_FUSE: bit 0 the FP64 solver, bit 1 the FP32 solver
  int fuse_restrict = 3;         // MM_OPT_FUSE_RESTRICT: bit 0 the FP64 solver, bit 1 the FP32 solver
  int coarse_cycle = 0;          // MM_OPT_COARSE_CYCLE: bit 0 the FP64 solver, bit 1 the FP32 solver
  int sa_theta_e3 = 0;           // MM_OPT_SA_THETA_E3 (0: the setup's default)
  int sa_factor_e3 = 0;          // MM_OPT_SA_FACTOR_E3 (0: the setup's default)
  int sa_filter_e6 = 0;          // MM_OPT_SA_FILTER_E6 (0: the setup's default, < 0: no filtering)
  std::vector<mm::HostCSR> rf_host;  // fused restrictions R_l (I - A_l S_l), formed for smoother rf_prec
  int rf_prec = -1;
  // host factors shared by the FP64 and FP32 copies of the hierarchy (formed once, O(nc^3) and
  // O(nc^2 n)): the coarsest level's dense inverse and the fused coarse correction for smoother fc_prec
  std::vector<double> ainv_host;
  struct FusedCoarseHost {
    bool ok = false;
    std::vector<double> tv, W, Z;
  };
  FusedCoarseHost fc_host;
  int fc_prec = -1;
  const std::vector<double>& coarse_inverse() {
    if (ainv_host.empty()) ainv_host = mm::dense_inverse(amg_h.back().A);
    return ainv_host;
  }

  // staging buffers for host-pointer calls
  double *d_m = nullptr, *d_U = nullptr, *d_g = nullptr, *d_v = nullptr, *d_out = nullptr, *d_bias = nullptr;

  // minimizer workspace (allocated on first use)
  bool min_ready = false;
  double *w_gt = nullptr, *w_gte = nullptr, *w_gprev = nullptr, *w_y = nullptr, *w_d = nullptr,
         *w_dprev = nullptr, *w_H = nullptr, *w_mt = nullptr, *w_Ut = nullptr, *w_gt_trial = nullptr,
         *w_graw = nullptr, *w_r3 = nullptr, *w_z3 = nullptr, *w_p3 = nullptr, *w_Ap3 = nullptr,
         *w_tmp = nullptr, *w_mprev = nullptr, *w_gtprev = nullptr, *w_ys = nullptr, *w_x1 = nullptr,
         *w_x2 = nullptr, *w_x3 = nullptr, *w_x4 = nullptr, *w_U2 = nullptr, *w_U3 = nullptr;
  std::vector<double*> w_S, w_Y;
  double* d_lb = nullptr;  // L-BFGS scalars on the device: rho[lb_mem], alpha[lb_mem], gamma
  int lb_mem = 0;
  float *w_r3f = nullptr, *w_z3f = nullptr, *w_p3f = nullptr, *w_Ap3f = nullptr, *w_yf = nullptr;
  struct InnerGraph {              // the inner solve's WHILE graph for one (m, g_ext, y, reg, precision)
    const double* m;
    const double* gext;
    const void* y;
    double reg;
    bool fp32;
    cudaGraph_t g;
    cudaGraphExec_t ex;
  };
  std::vector<InnerGraph> inner_graphs;  // at most 8, oldest replaced first
  bool inner_graph_failed = false;
  bool inner_cpp_count = false;  // solve_Py_g counts its trips as the reference's C++ minimizer does
  void drop_inner_graphs() {  // their launches hold the operator's arrays and the launch attributes
    drop_min_graphs();
    if (inner_graphs.empty()) return;
    if (st) cudaStreamSynchronize(st);
    for (auto& ig : inner_graphs) {
      cudaGraphExecDestroy(ig.ex);
      cudaGraphDestroy(ig.g);
    }
    inner_graphs.clear();
  }
  // device-driven minimizer iterations (MM_OPT_MIN_GRAPH): one graph per set of buffers and settings
  int min_graph = 1;
  bool min_graph_failed = false;
  cudaStream_t aux_st[3] = {nullptr, nullptr, nullptr};  // capture streams of the nested loop bodies
  int cap_depth = 0;
  mmk::MinScal* d_ms = nullptr;
  mmk::MinScal* h_ms = nullptr;  // pinned
  struct MinGraph {
    std::vector<uintptr_t> key;
    cudaGraph_t g;
    cudaGraphExec_t ex;
    int64_t per_outer, per_ls, per_pcg, per_in;  // kernels of one trip of each loop (launch count)
  };
  std::vector<MinGraph> min_graphs;  // at most 4, oldest replaced first
  void drop_min_graphs() {
    if (min_graphs.empty()) return;
    if (st) cudaStreamSynchronize(st);
    for (auto& mg : min_graphs) {
      cudaGraphExecDestroy(mg.ex);
      cudaGraphDestroy(mg.g);
    }
    min_graphs.clear();
  }
  double* d_min_bias = nullptr;    // per-node bias field of the minimizer's energy evaluations (or null)
  double* min_bias_buf = nullptr;  // its storage
  cudaEvent_t ev_after = nullptr;  // ordering point taken on another stream (mm_scale_correction_async)
  cudaStream_t st_copy = nullptr;  // a second copy engine's stream for the host-array solves' initial guess
  cudaEvent_t ev_copy = nullptr;

  // Device buffers come from the device's stream-ordered pool on the problem's stream and go back to
  // it with cudaFreeAsync (mm_destroy): unlike cudaMalloc / cudaFree, neither waits for the work other
  // problems have queued on the device, so problems can be created and destroyed while others run.
  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    if (!st) throw Fail{MM_ERR_CUDA, "device allocation before the problem's stream exists"};
    // an allocation on a capturing stream would become a graph node whose memory lives only while
    // the graph runs: every buffer is made before a capture begins
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) throw Fail{MM_ERR_STATE, "device allocation while the stream captures"};
    CK(cudaMallocAsync(&p, n * sizeof(T), st));
    allocs.push_back(p);
    // zeroed: reused device memory can hold any bit pattern (a NaN in an FP32 view of old FP64 data),
    // and a vector read once with a zero factor (the first direction's beta p) must not carry it in.
    // On the problem's own stream, ahead of any copy into the buffer (that stream does not order with
    // the legacy default stream).
    CK(cudaMemsetAsync(p, 0, n * sizeof(T), st));
    return (T*)p;
  }
  template <class T, class Alloc>
  T* upload(const std::vector<T, Alloc>& v) {
    T* p = alloc<T>(v.size());
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return p;
  }
  template <class T, class Alloc>
  T* upload_as(const std::vector<double, Alloc>& v) {
    std::vector<T> t(v.begin(), v.end());
    return upload(t);
  }
  // a per-entry array of the energy operator in sliced order (padding entries `pad`)
  template <class T, class V>
  T* upload_eop_sell(const V& a, T pad) {
    std::vector<T> out((size_t)eops_stored, pad);
    for (size_t k = 0; k < eops_pos.size(); ++k) out[eops_pos[k]] = (T)a[k];
    return upload(out);
  }
  // the energy operator's sliced-ELL copy (slices of 32 magnetic rows, width = the slice's longest
  // row; padding entries: zero values, the row's own node as column)
  void upload_eop_sell_all() {
    const mm::EnergyOp& o = eop_h;
    const int n = o.n_rows, ns = (n + 31) / 32;
    std::vector<int> sptr(ns + 1, 0);
    for (int sl = 0; sl < ns; ++sl) {
      int w = 0;
      for (int r = 32 * sl; r < std::min(n, 32 * sl + 32); ++r) w = std::max(w, o.ptr[r + 1] - o.ptr[r]);
      sptr[sl + 1] = sptr[sl] + 32 * w;
    }
    eops_stored = sptr[ns];
    eops_pos.assign(o.col.size(), 0);
    std::vector<int> col((size_t)eops_stored, 0);
    for (int r = 0; r < n; ++r) {
      const int sl = r / 32, l = r % 32, w = (sptr[sl + 1] - sptr[sl]) / 32, len = o.ptr[r + 1] - o.ptr[r];
      for (int k = 0; k < w; ++k) {
        const int64_t at = (int64_t)sptr[sl] + 32 * k + l;
        if (k < len) {
          eops_pos[o.ptr[r] + k] = at;
          col[at] = o.col[o.ptr[r] + k];
        } else {
          col[at] = o.rows[r];
        }
      }
    }
    mmk::EnergySell& d = eops;
    d.n_rows = n;
    d.rows = eop.rows;
    d.sptr = upload(sptr);
    d.col = upload(col);
    d.mat = upload_eop_sell<int>(o.mat, 0);
    d.w = upload_eop_sell<double>(o.w, 0.0);
    d.q = upload_eop_sell<double>(o.q, 0.0);
    d.gx = upload_eop_sell<double>(o.gx, 0.0);
    d.gy = upload_eop_sell<double>(o.gy, 0.0);
    d.gz = upload_eop_sell<double>(o.gz, 0.0);
    d.dx = upload_eop_sell<double>(o.dx, 0.0);
    d.dy = upload_eop_sell<double>(o.dy, 0.0);
    d.dz = upload_eop_sell<double>(o.dz, 0.0);
    d.kax = eop.kax;
    d.mex = d.mey = nullptr;
    d.single_axis = eop.single_axis;
    d.axis0 = eop.axis0;
  }
  // whether energy evaluations run in float-float (one easy axis, no magnetoelastic term), building the
  // pairs on first use
  bool use_energy_ff() {
    const bool want = energy_ff < 0 ? (mixed || fp32_precond) : energy_ff != 0;
    if (!want || eop_h.n_rows == 0 || !eops.single_axis || eops.mex) return false;
    if (eopsff_ok) return true;
    if (eopsff_failed) return false;
    double lo = 1e300, hi = 0.0;
    for (const mm::dvec* v : {&eop_h.w, &eop_h.q, &eop_h.gx, &eop_h.gy, &eop_h.gz})
      for (double x : *v)
        if (x != 0.0) lo = std::min(lo, std::fabs(x)), hi = std::max(hi, std::fabs(x));
    if (hi > 0.0 && (lo < 1e-30 || hi > 1e30)) {
      eopsff_failed = true;
      return false;
    }
    auto split = [](double v) {
      const float hi32 = (float)v;
      return make_float2(hi32, (float)(v - (double)hi32));
    };
    auto quads = [&](const mm::dvec& a, const mm::dvec& b) {  // (a_hi, a_lo, b_hi, b_lo) per entry
      std::vector<float4> out((size_t)eops_stored, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
      for (size_t k = 0; k < eops_pos.size(); ++k) {
        const float2 x = split(a[k]), y = split(b[k]);
        out[eops_pos[k]] = make_float4(x.x, x.y, y.x, y.y);
      }
      return upload(out);
    };
    std::vector<float2> gz2((size_t)eops_stored, make_float2(0.0f, 0.0f));
    for (size_t k = 0; k < eops_pos.size(); ++k) gz2[eops_pos[k]] = split(eop_h.gz[k]);
    mmk::EnergySellFF& d = eopsff;
    d.n_rows = eops.n_rows;
    d.rows = eops.rows;
    d.sptr = eops.sptr;
    d.col = eops.col;
    d.wq = quads(eop_h.w, eop_h.q);
    d.gxy = quads(eop_h.gx, eop_h.gy);
    d.gz = upload(gz2);
    d.kx = kax_h[3 * eops.axis0];
    d.ky = kax_h[3 * eops.axis0 + 1];
    d.kz = kax_h[3 * eops.axis0 + 2];
    d.kfx = split(d.kx);
    d.kfy = split(d.ky);
    d.kfz = split(d.kz);
    std::vector<char> seen(N, 0);
    for (int j : eop_h.col) seen[j] = 1;
    std::vector<int> touched;
    for (int i = 0; i < N; ++i)
      if (seen[i]) touched.push_back(i);
    d.n_touched = (int)touched.size();
    d.touched = upload(touched);
    if (!w_ff.hi) {
      w_ff.hi = alloc<float4>(N);
      w_ff.lo = alloc<float4>(N);
      w_ff.u = alloc<float2>(N);
    }
    eopsff_ok = true;
    return true;
  }
  // whether the inner solve runs in FP32, building its entries on first use; false also when an entry
  // of the operator lies outside the range FP32 represents with full precision
  bool inner_fp32() {
    const bool want = min_fp32 < 0 ? (mixed || fp32_precond) : min_fp32 != 0;
    if (!want || eop_h.n_rows == 0) return false;
    if (eops32_ok) return true;
    // 1/V_mag is folded into the FP32 entries (the operator kernel then scales by 1)
    double lo = 1e300, hi = 0.0;
    auto scaled = [&](const mm::dvec& v) {
      std::vector<double> out(v.size());
      for (size_t k = 0; k < v.size(); ++k) {
        out[k] = v[k] * inv_Vmag;
        if (out[k] != 0.0) lo = std::min(lo, std::fabs(out[k])), hi = std::max(hi, std::fabs(out[k]));
      }
      return out;
    };
    const std::vector<double> w32 = scaled(eop_h.w), q32 = scaled(eop_h.q);
    std::vector<double> mx32, my32;
    if (eops.mex) mx32 = scaled(eop_h.mx), my32 = scaled(eop_h.my);
    if (hi > 0.0 && (lo < 1e-30 || hi > 1e30)) return false;
    mmk::EnergySell32& d = eops32;
    d.n_rows = eops.n_rows;
    d.rows = eops.rows;
    d.sptr = eops.sptr;
    d.col = eops.col;
    d.mat = eops.mat;
    d.w = upload_eop_sell<float>(w32, 0.0f);
    d.q = upload_eop_sell<float>(q32, 0.0f);
    d.kax = upload(std::vector<float>(kax_h.begin(), kax_h.end()));
    d.mex = eops.mex ? upload_eop_sell<float>(mx32, 0.0f) : nullptr;
    d.mey = eops.mex ? upload_eop_sell<float>(my32, 0.0f) : nullptr;
    d.single_axis = eops.single_axis;
    d.axis0 = eops.axis0;
    if (!w_yf) {
      const size_t n3 = 3 * (size_t)N;
      for (float** b : {&w_r3f, &w_z3f, &w_p3f, &w_Ap3f, &w_yf}) *b = alloc<float>(n3);
    }
    eops32_ok = true;
    return true;
  }
  // Compressed rows (below 64Ki rows) get a sliced-ELL copy when the autotuner asks for one: one
  // thread per row has no shuffle reductions, whose FP64 adds take a third of the FP64 pipe in the
  // lanes-per-row kernels.
  template <class T>
  DevMatT<T> upload_mat(const mm::HostCSR& A, bool force_sell = false) {
    const int tpr = force_sell ? 1 : choose_tpr(A.n_rows, A.nnz());
    DevMatT<T> d;
    d.tpr = tpr;
    d.nnz = A.nnz();
    if (tpr > 1) {
      d.c.n = A.n_rows;
      d.c.ptr = upload(A.ptr);
      d.c.col = upload(A.col);
      d.c.val = upload_as<T>(A.val);
      d.stored = A.nnz();
      d.s.n = A.n_rows;
      return d;
    }
    upload_sell<T>(A, d);
    return d;
  }
  // sliced ELL (mmk::SellT): slices of 32 rows, entries paired, padding with value 0 and a valid column
  template <class T>
  void upload_sell(const mm::HostCSR& A, DevMatT<T>& d) {
    const int n = A.n_rows;
    const int ns = (n + 31) / 32;
    std::vector<int> sptr(ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
      int w = 0;
      for (int r = 32 * s; r < std::min(n, 32 * s + 32); ++r) w = std::max(w, A.ptr[r + 1] - A.ptr[r]);
      sptr[s + 1] = sptr[s] + 64 * ((w + 1) / 2);  // paired entries (mmk::SellT)
    }
    std::vector<int> col(sptr[ns]);
    std::vector<double> val(sptr[ns], 0.0);
    for (int s = 0; s < ns; ++s) {
      const int w2 = (sptr[s + 1] - sptr[s]) / 32;  // stored entries per row (even)
      for (int l = 0; l < 32; ++l) {
        const int r = 32 * s + l;
        const int len = r < n ? A.ptr[r + 1] - A.ptr[r] : 0;
        for (int k = 0; k < w2; ++k) {
          const size_t at = (size_t)sptr[s] + 64 * (k / 2) + 2 * l + (k % 2);
          if (k < len) {
            col[at] = A.col[A.ptr[r] + k];
            val[at] = A.val[A.ptr[r] + k];
          } else {
            col[at] = r < n ? std::min(r, std::max(A.n_cols - 1, 0)) : 0;
            val[at] = 0.0;
          }
        }
      }
    }
    d.s.n = n;
    d.s.sptr = upload(sptr);
    d.s.col = upload(col);
    d.s.val = upload_as<T>(val);
    if (d.tpr == 1) d.stored = sptr[ns];
  }
  double red(int slot) {
    CK(cudaMemcpyAsync(&h_sc->red[slot], &d_sc->red[slot], sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return h_sc->red[slot];
  }
  // `count` consecutive reduction slots from `first` with one copy and one wait
  const double* red_n(int first, int count) {
    CK(cudaMemcpyAsync(&h_sc->red[first], &d_sc->red[first], count * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return &h_sc->red[first];
  }
  void sync() { CK(cudaStreamSynchronize(st)); }
  // the split copy of the level-0 operator for the FP32-preconditioned PCG (sliced rows only)
  bool use_a0df() {
    if (!split_a0) return false;
    if (a0df_ok) return true;
    const DevMatT<double>& A = s64.lv[0].A;
    if (A.tpr != 1 || A.stored <= 0 || !A.s.val) return false;
    float* hi = alloc<float>((size_t)A.stored);
    float* lo = alloc<float>((size_t)A.stored);
    mmk::k_split_df<<<1024, BS, 0, st>>>(A.stored, A.s.val, hi, lo);
    CK(cudaGetLastError());
    a0df = mmk::SellDF{A.s.n, A.s.sptr, A.s.col, hi, lo};
    a0df_ok = true;
    return true;
  }
  cudaEvent_t prof_event() {
    if (prof_used == prof_pool.size()) {
      cudaEvent_t e = nullptr;
      CK(cudaEventCreate(&e));
      prof_pool.push_back(e);
    }
    return prof_pool[prof_used++];
  }
  // add the recorded launches to the slot totals (the stream must be idle)
  void prof_fold() {
    for (const ProfRec& r : prof_rec) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, r.a, r.b));
      prof_ms[r.slot] += t;
      prof_n[r.slot] += 1;
    }
    prof_rec.clear();
    prof_used = 0;
  }
};

// =============================================================================================
// launch helpers
// =============================================================================================
namespace {

using mmk::R_A;
using mmk::R_B;
using mmk::R_BB;
using mmk::R_BB0;
using mmk::R_C;
using mmk::R_D;
using mmk::R_E;
using mmk::R_MAX;
using mmk::R_PAP;
using mmk::R_R2;
using mmk::R_RZ;
using mmk::R_SUM;

// Launch on the problem's stream with programmatic dependent launch allowed when h->pdl: the
// kernel may be scheduled while its predecessor drains, and waits for the predecessor's results
// itself (pdl_entry at its start).  Arguments are converted to the kernel's parameter types.
template <typename... KArgs, typename... Args>
void launch(mm_problem* h, void (*kern)(KArgs...), dim3 grid, dim3 block, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = h->st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = h->pdl ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...));
}

#define TPR_SWITCH(tpr, ...)                         \
  switch (tpr) {                                     \
    case 2: { constexpr int TP = 2; __VA_ARGS__; } break;   \
    case 4: { constexpr int TP = 4; __VA_ARGS__; } break;   \
    case 8: { constexpr int TP = 8; __VA_ARGS__; } break;   \
    case 16: { constexpr int TP = 16; __VA_ARGS__; } break; \
    default: { constexpr int TP = 32; __VA_ARGS__; } break; \
  }

template <int MODE, class T>
void spmv(mm_problem* h, const DevMatT<T>& A, const T* x, const T* b, const T* s, T* y, const int* done) {
  if (A.tpr == 1) {
    launch(h, mmk::k_sell<MODE, T>, grid_ilp(A.s.n), BS, A.s, x, b, s, y, done);
  } else {
    const int g = grid_rows(A.c.n, A.tpr);
    TPR_SWITCH(A.tpr, (launch(h, mmk::k_csr<TP, MODE, T>, g, BS, A.c, x, b, s, y, done)));
  }
  LAUNCH_CHECK();
}

template <class T>
void dotT(mm_problem* h, int n, const T* x, const T* y, mmk::Scalars* sc, int slot, int post = mmk::POST_NONE) {
  launch(h, mmk::k_dot<T>, std::min(grid_ilp(n), g_vec_cap), BS, n, x, y, sc, h->d_part, slot, post);
  LAUNCH_CHECK();
}

void dot(mm_problem* h, int n, const double* x, const double* y, int slot, int post = mmk::POST_NONE) {
  dotT<double>(h, n, x, y, h->d_sc, slot, post);
}

template <class T>
bool multilevel(mm_problem* h, const SolverT<T>& S) {
  return (h->precond == MM_PRECOND_AMG || h->precond == MM_PRECOND_AMGCL) && S.lv.size() > 1;
}

// In-solve profile: with MM_OPT_PROFILE on, `launch` is bracketed by an event pair whose time goes
// to the slot of (kind, level, precision); `bytes` are the launch's algorithmic bytes.
template <class T, class F>
void tagged(mm_problem* h, int kind, int level, double bytes, F&& launch) {
  if (!h->prof) {
    launch();
    return;
  }
  const int lvl = std::min(level, MM_PROF_LEVELS - 1);
  const int slot = ((sizeof(T) == 4 ? 1 : 0) * MM_PROF_LEVELS + lvl) * MM_PROF_KINDS + kind;
  cudaEvent_t a = h->prof_event(), b = h->prof_event();
  CK(cudaEventRecord(a, h->st));
  launch();
  CK(cudaEventRecord(b, h->st));
  h->prof_bytes[slot] = bytes;
  h->prof_rec.push_back({slot, a, b});
}

// algorithmic bytes of one pass over a stored operator: values + columns of the non-zeros (padding
// excluded) and the slice / row pointers
template <class T>
double mat_bytes(const DevMatT<T>& M) {
  const double ptrs = M.tpr == 1 ? (double)((M.s.n + 31) / 32 + 1) : (double)(M.c.n + 1);
  return (double)M.nnz * (4.0 + sizeof(T)) + 4.0 * ptrs;
}

// ---------------------------------------------------------------------------------------------
// V-cycle (enqueue only).  Level 0's pre-smoothed iterate lv[0].x must already hold s0 .* r.
// in_loop: the level-0 residual is skipped once the solve has converged.
// ---------------------------------------------------------------------------------------------
template <class T>
void enqueue_vcycle(mm_problem* h, SolverT<T>& S, const T* r, T* z, bool in_loop, const int* done,
                    mmk::Scalars* scal = nullptr, double* z64 = nullptr) {
  mmk::Scalars* const sc = scal ? scal : S.sc;  // the PCG's scalars (another solver's with the FP32 preconditioner)
  auto& lv = S.lv;
  const int L = (int)lv.size();
  const double w = sizeof(T);
  const bool fuse = S.fused && ((h->coarse_fuse >> (sizeof(T) == 8 ? 0 : 1)) & 1);
  const int Ld = fuse ? L - 2 : L - 1;  // levels l < Ld compute a residual and restrict it
  const bool fr_on = (h->fuse_restrict >> (sizeof(T) == 8 ? 0 : 1)) & 1;
  // b_{l+1} = R_l res (res = b_l - A_l x_l), and the pre-smoothing x_{l+1} = s_{l+1} b_{l+1} unless
  // level l+1 has none
  auto restrict_into = [&](int l, const DevMatT<T>& M, const T* in, double mbytes) {
    auto& c = lv[l];
    auto& nx = lv[l + 1];
    const bool no_pre = (l + 1 == L - 1) || (fuse && l + 1 == L - 2);
    const double rbytes = mbytes + w * c.n + (no_pre ? 1.0 : 3.0) * w * nx.n;
    tagged<T>(h, MM_PROF_RESTRICT, l, rbytes, [&] {
      if (M.tpr == 1) {
        launch(h, mmk::k_restrict<T>, grid_ilp(nx.n), BS, M.s, in, nx.b, no_pre ? nullptr : nx.s, nx.x, done);
      } else {
        const int g = grid_rows(nx.n, M.tpr);
        TPR_SWITCH(M.tpr, (launch(h, mmk::k_restrict_csr<TP, T>, g, BS, M.c, in, nx.b, no_pre ? nullptr : nx.s,
                                  nx.x, done)));
      }
      LAUNCH_CHECK();
    });
  };
  // levels 1 .. 3 in one cooperative launch when the hierarchy has that shape (four levels, fused
  // restriction at level 1, fused coarse correction, compressed rows on level 1)
  const bool cc_on = ((h->coarse_cycle >> (sizeof(T) == 8 ? 0 : 1)) & 1) && fuse && fr_on && L == 4 &&
                     lv[0].Rf.nnz > 0 && lv[1].Rf.nnz > 0 && lv[1].Rf.tpr > 1 && lv[1].P.tpr > 1 &&
                     lv[1].A.tpr > 1 && S.bar && S.coop_grid > 0;
  for (int l = 0; l < (cc_on ? 1 : Ld); ++l) {
    auto& c = lv[l];
    if (fr_on && c.Rf.nnz > 0) {
      // x_l = s_l b_l (the pre-smoothing from zero, already written), so b_{l+1} = R_l (I - A_l S_l) b_l
      restrict_into(l, c.Rf, l == 0 ? r : c.b, mat_bytes(c.Rf));
      continue;
    }
    if (l == 0 && in_loop) {
      tagged<T>(h, MM_PROF_VC_RESIDUAL0, 0, mat_bytes(c.A) + 3.0 * w * c.n, [&] {
        launch(h, mmk::k_vc_residual0<T>, grid_ilp(c.n), BS, c.A.s, c.x, r, c.res, sc);
        LAUNCH_CHECK();
      });
    } else {
      tagged<T>(h, l == 0 ? MM_PROF_VC_RESIDUAL0 : MM_PROF_RESIDUAL, l, mat_bytes(c.A) + 3.0 * w * c.n,
                [&] { spmv<1, T>(h, c.A, c.x, l == 0 ? r : c.b, nullptr, c.res, done); });
    }
    restrict_into(l, c.R, c.res, mat_bytes(c.R));
  }
  if (cc_on) {
    auto& l1 = lv[1];
    auto& l2 = lv[2];
    mmk::CoarseCycle<T> cc{};
    cc.Rf1 = l1.Rf.c;
    cc.P1 = l1.P.c;
    cc.A1 = l1.A.c;
    cc.Tm = S.Tm;
    cc.tpr_rf1 = l1.Rf.tpr;
    cc.tpr_p1 = l1.P.tpr;
    cc.tpr_a1 = l1.A.tpr;
    cc.b1 = l1.b;
    cc.x1 = l1.x;
    cc.s1 = l1.s;
    cc.x2_1 = l1.x2;
    cc.b2 = l2.b;
    cc.Z = S.Z;
    cc.W = S.W;
    cc.nc = S.fc;
    cc.gT = grid_rows(S.fn, mmk::CA_LANES);
    cc.tvec = S.tvec;
    cc.zvec = S.zvec;
    cc.x2_2 = l2.x2;
    const double bytes = mat_bytes(l1.Rf) + mat_bytes(l1.P) + mat_bytes(l1.A) + 4.0 * ((double)S.Tm.n + 1.0) +
                         (4.0 + w) * (double)S.Tm_nnz + 2.0 * w * (double)S.fc * S.fn + w * 7.0 * l1.n +
                         w * 6.0 * l2.n;
    tagged<T>(h, MM_PROF_COARSE_CYCLE, 1, bytes, [&] {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(S.coop_grid);
      cfg.blockDim = dim3(BS);
      cfg.stream = h->st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      CK(cudaLaunchKernelEx(&cfg, mmk::k_coarse_cycle<T>, cc, S.bar, sc, done));
      LAUNCH_CHECK();
    });
  } else if (fuse) {
    auto& c = lv[L - 2];
    const int n = S.fn, nc = S.fc;
    const double tbytes = (double)S.Tm.n + 1.0;
    tagged<T>(h, MM_PROF_COARSE_A, L - 2,
              4.0 * tbytes + (4.0 + w) * (double)S.Tm_nnz + w * ((double)nc * n + 2.0 * n + nc),
              [&] {
                const int gT = grid_rows(n, mmk::CA_LANES);
                launch(h, mmk::k_coarse_a<T>, gT + nc, BS, S.Tm, S.Z, nc, c.b, S.tvec, S.zvec, gT, done);
                LAUNCH_CHECK();
              });
    tagged<T>(h, MM_PROF_COARSE_B, L - 2, w * ((double)n * nc + 2.0 * n + nc), [&] {
      launch(h, mmk::k_coarse_b<T>, grid_rows(n, mmk::CB_LANES), BS, n, nc, S.W, S.tvec, S.zvec, c.x2, done);
      LAUNCH_CHECK();
    });
  } else {
    auto& c = lv[L - 1];
    tagged<T>(h, MM_PROF_COARSE, L - 1, w * ((double)c.n * c.n + 2.0 * c.n), [&] {
      launch(h, mmk::k_dense_mv<T>, grid_rows(c.n, 32), BS, c.n, S.Ainv, c.b, c.x2, done);
      LAUNCH_CHECK();
    });
  }
  for (int l = (cc_on ? 0 : fuse ? L - 3 : L - 2); l >= 0; --l) {
    auto& c = lv[l];
    tagged<T>(h, MM_PROF_PROLONG, l, mat_bytes(c.P) + w * lv[l + 1].n + 2.0 * w * c.n,
              [&] { spmv<3, T>(h, c.P, lv[l + 1].x2, c.x, nullptr, c.x, done); });  // x += P e
    if (l == 0) {
      tagged<T>(h, MM_PROF_SMOOTH0, 0, mat_bytes(c.A) + 4.0 * w * c.n, [&] {
        launch(h, mmk::k_smooth_dot<T>, grid_ilp(c.n), BS, c.A.s, c.x, r, c.s, z, sc, h->d_part, done, z64);
        LAUNCH_CHECK();
      });
    } else {
      tagged<T>(h, MM_PROF_SMOOTH, l, mat_bytes(c.A) + 4.0 * w * c.n,
                [&] { spmv<2, T>(h, c.A, c.x, c.b, c.s, c.x2, done); });
    }
  }
}

// z = M^-1 r for Jacobi / no preconditioner / a one-level hierarchy (dense solve); r.z -> red[R_RZ]
template <class T>
void apply_M_simple(mm_problem* h, SolverT<T>& S, const T* r, T* z, const int* done) {
  const int N = h->N;
  if (h->precond == MM_PRECOND_JACOBI) {
    launch(h, mmk::k_mul<T>, grid_ilp(N), BS, N, S.jac, r, z);
    LAUNCH_CHECK();
  } else if (h->precond == MM_PRECOND_NONE) {
    CK(cudaMemcpyAsync(z, r, N * sizeof(T), cudaMemcpyDeviceToDevice, h->st));
  } else {
    launch(h, mmk::k_dense_mv<T>, grid_rows(S.n_coarse, 32), BS, S.n_coarse, S.Ainv, r, z, done);
    LAUNCH_CHECK();
  }
  dotT<T>(h, N, r, z, S.sc, R_RZ, mmk::POST_RZ);
}

// preconditioner application outside the PCG loop
template <class T>
void enqueue_precond(mm_problem* h, SolverT<T>& S, const T* r, T* z) {
  if (multilevel(h, S)) {
    launch(h, mmk::k_mul<T>, grid_ilp(h->N), BS, h->N, S.lv[0].s, r, S.lv[0].x);
    LAUNCH_CHECK();
    enqueue_vcycle<T>(h, S, r, z, false, nullptr);
  } else {
    apply_M_simple<T>(h, S, r, z, nullptr);
  }
}

// first half of a PCG iteration: new direction with its operator product, then the step (sets
// `done` on convergence)
template <class T>
void enqueue_dir_step(mm_problem* h, SolverT<T>& S) {
  const int N = h->N;
  const double w = sizeof(T);
  auto& l0 = S.lv[0];
  tagged<T>(h, MM_PROF_PCG_DIR, 0, mat_bytes(l0.A) + 5.0 * w * N, [&] {
    launch(h, mmk::k_pcg_dir<T>, grid_ilp(N), BS, l0.A.s, S.z, S.p, S.Ap, S.sc, h->d_part);
    LAUNCH_CHECK();
  });
  const bool ml = multilevel(h, S);
  tagged<T>(h, MM_PROF_PCG_STEP, 0, (ml ? 8.0 : 6.0) * w * N, [&] {
    launch(h, mmk::k_pcg_step<T>, grid_ilp(N), BS, N, S.x, S.r, S.p, S.Ap, ml ? l0.s : nullptr, l0.x, S.sc,
                                                        h->d_part);
    LAUNCH_CHECK();
  });
}

// second half: z = M^-1 r with r.z
template <class T>
void enqueue_apply_M(mm_problem* h, SolverT<T>& S) {
  if (multilevel(h, S)) enqueue_vcycle<T>(h, S, S.r, S.z, true, &S.sc->done);
  else apply_M_simple<T>(h, S, S.r, S.z, &S.sc->done);
}

// one PCG iteration on x = S.x (all scalars stay on the device)
template <class T>
void enqueue_iteration(mm_problem* h, SolverT<T>& S) {
  enqueue_dir_step<T>(h, S);
  enqueue_apply_M<T>(h, S);
}

// WHILE (condition) { body(handle) } captured from the problem's stream into an instantiated graph.
// Returns false when the driver cannot build conditional graphs (the caller polls on the host then).
template <class Body>
bool capture_while_graph(mm_problem* h, Body&& body, cudaGraph_t* g_out, cudaGraphExec_t* ex_out) {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  cudaGraphConditionalHandle hnd;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
            cudaGraphConditionalHandleCreate(&hnd, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t node;
  if (ok) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hnd;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t inner = cp.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(h->st, inner, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
         cudaSuccess;
    if (ok) {
      try {
        body(hnd);
      } catch (const Fail&) {
        ok = false;
      }
      cudaGraph_t out = nullptr;
      const bool end_ok = cudaStreamEndCapture(h->st, &out) == cudaSuccess;
      ok = ok && end_ok;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();  // clear the error of the failed attempt
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    return false;
  }
  *g_out = g;
  *ex_out = ex;
  return true;
}

// Build the PCG loop graph: WHILE (condition) { iteration; k_set_cond }.
template <class T, class Iter>
bool build_loop_graph(mm_problem* h, SolverT<T>& S, Iter&& iteration) {
  if (S.exec) return true;
  if (S.graph_failed) return false;
  const int64_t saved = h->n_launch;
  const bool ok = capture_while_graph(
      h,
      [&](cudaGraphConditionalHandle hnd) {
        iteration();
        launch(h, mmk::k_set_cond, 1, 32, hnd, S.sc);
      },
      &S.graph, &S.exec);
  S.iter_launches = h->n_launch - saved + 1;
  h->n_launch = saved;
  if (!ok) S.graph_failed = true;
  return ok;
}
template <class T>
bool build_loop_graph(mm_problem* h, SolverT<T>& S) {
  return build_loop_graph(h, S, [&] { enqueue_iteration<T>(h, S); });
}

// the loop graph, or, when it cannot be built with the one-launch coarse cycle in it, without that
template <class T, class Iter>
bool loop_graph_or_retry(mm_problem* h, SolverT<T>& S, Iter&& iteration) {
  if (build_loop_graph(h, S, iteration)) return true;
  if (h->coarse_cycle == 0) return false;
  h->coarse_cycle = 0;
  S.graph_failed = false;
  return build_loop_graph(h, S, iteration);
}

template <class T>
void drop_graph(SolverT<T>& S) {
  if (S.exec) cudaGraphExecDestroy(S.exec);
  if (S.graph) cudaGraphDestroy(S.graph);
  S.exec = nullptr;
  S.graph = nullptr;
  S.graph_failed = false;
  ++S.epoch;
}

// A PCG solve whose final scalars copy is queued but not yet waited for (solve_dev waits once, after
// its own follow-up work, and then reads them with finish_pcg).
struct PcgPending {
  SolverT<double>* S = nullptr;
  bool graph = false;
};

// the one-launch coarse cycle records a grid barrier that gave up waiting in the PCG's scalars
void check_barrier(const mmk::Scalars* sc) {
  if (sc->bar_err) throw Fail{MM_ERR_CUDA, "a grid barrier of the one-launch coarse cycle gave up waiting"};
}

void finish_pcg(mm_problem* h, const PcgPending& pend, int* iters, double* r2_out) {
  check_barrier(h->h_sc);
  if (pend.graph) h->n_launch += (int64_t)h->h_sc->loops * pend.S->iter_launches;
  if (iters) *iters = h->h_sc->it;
  if (r2_out) *r2_out = h->h_sc->red[R_R2];
}

// PCG on S.x (initial guess in, solution out) for the right-hand side S.b; stops on the recursive
// residual r.r <= tol^2 b.b or maxiter (src/poisson_solve.py:422-478).  Returns iterations and r.r.
// the work of a PCG solve before its loop: b.b, the scalars, r0 = b - A x0 and z0 = M^-1 r0
template <class T>
void enqueue_pcg_start(mm_problem* h, SolverT<T>& S, double tol, int maxiter) {
  const int N = h->N;
  dotT<T>(h, N, S.b, (const T*)nullptr, S.sc, R_BB);
  launch(h, mmk::k_pcg_init_scalars, 1, 32, S.sc, tol, maxiter);
  LAUNCH_CHECK();
  const bool ml = multilevel(h, S);
  auto& l0 = S.lv[0];
  const double w = sizeof(T);
  tagged<T>(h, MM_PROF_INIT_RESIDUAL, 0, mat_bytes(l0.A) + 5.0 * w * N, [&] {
    launch(h, mmk::k_init_residual<T>, grid_ilp(N), BS, l0.A.s, S.x, S.b, S.r, ml ? l0.s : nullptr, l0.x, S.sc,
                                                             h->d_part);
    LAUNCH_CHECK();
  });
  if (ml) enqueue_vcycle<T>(h, S, S.r, S.z, false, nullptr);
  else apply_M_simple<T>(h, S, S.r, S.z, nullptr);
}

template <class T>
void run_pcg(mm_problem* h, SolverT<T>& S, double tol, int maxiter, int* iters, double* r2_out,
             PcgPending* pend = nullptr) {
  enqueue_pcg_start<T>(h, S, tol, maxiter);
  const bool graph = h->use_graph && !h->prof && loop_graph_or_retry(h, S, [&] { enqueue_iteration<T>(h, S); });
  if (graph) {
    CK(cudaGraphLaunch(S.exec, h->st));
  } else if (h->prof) {
    // profiled: read `done` after every step so that no launch runs past convergence
    for (int i = 0; i <= maxiter + 2; ++i) {
      enqueue_dir_step<T>(h, S);
      CK(cudaMemcpyAsync(h->h_sc, S.sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
      h->sync();
      if (h->h_sc->done) break;
      enqueue_apply_M<T>(h, S);
    }
  } else {
    for (int i = 0;; ++i) {
      enqueue_iteration<T>(h, S);
      if ((i + 1) % 4 == 0) {
        CK(cudaMemcpyAsync(h->h_sc, S.sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
        h->sync();
        if (h->h_sc->done || i > maxiter + 8) break;
      }
    }
  }
  CK(cudaMemcpyAsync(h->h_sc, S.sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
  if constexpr (std::is_same<T, double>::value) {
    if (pend) {
      *pend = PcgPending{&S, graph};
      return;
    }
  }
  h->sync();
  check_barrier(h->h_sc);
  if (graph) h->n_launch += (int64_t)h->h_sc->loops * S.iter_launches;
  if (iters) *iters = h->h_sc->it;
  if (r2_out) *r2_out = h->h_sc->red[R_R2];
}

// FP64 PCG preconditioned by the FP32 V-cycle (MM_PRECISION_FP32_PRECOND): x, r, p, A p, the
// products with A0 and every inner product in FP64; the V-cycle on the FP32 copy of the hierarchy,
// from fl32(r) (its level-0 pre-smoothing fused into the step) to z in FP32.
// The scalars of the iteration are the FP64 solver's; the last V-cycle kernel also writes z in FP64
// (one conversion per row there, not one per stored entry in the FP64 product with A0).
void enqueue_iteration_mp(mm_problem* h) {
  auto& S = h->s64;
  auto& F = h->s32;
  const int N = h->N;
  auto& l0 = S.lv[0];
  const bool df = h->a0df_ok && h->split_a0;
  if (df) {
    tagged<double>(h, MM_PROF_PCG_DIR, 0, mat_bytes(l0.A) + 4.0 * N + 4.0 * 8.0 * N, [&] {
      launch(h, mmk::k_pcg_dir_df, grid_ilp(N), BS, h->a0df, (const float*)F.z, S.p, S.Ap, S.sc, h->d_part);
      LAUNCH_CHECK();
    });
  } else {
    tagged<double>(h, MM_PROF_PCG_DIR, 0, mat_bytes(l0.A) + 5.0 * 8.0 * N, [&] {
      launch(h, mmk::k_pcg_dir<double>, grid_ilp(N), BS, l0.A.s, S.z, S.p, S.Ap, S.sc, h->d_part);
      LAUNCH_CHECK();
    });
  }
  tagged<double>(h, MM_PROF_PCG_STEP, 0, 6.0 * 8.0 * N + 3.0 * 4.0 * N, [&] {
    launch(h, mmk::k_pcg_step_mp, grid_ilp(N), BS, N, S.x, S.r, S.p, S.Ap, F.lv[0].s, F.r, F.lv[0].x, S.sc,
           h->d_part);
    LAUNCH_CHECK();
  });
  enqueue_vcycle<float>(h, F, F.r, F.z, true, &S.sc->done, S.sc, df ? nullptr : S.z);
}

void enqueue_pcg_mp_start(mm_problem* h, double tol, int maxiter) {
  auto& S = h->s64;
  auto& F = h->s32;
  const int N = h->N;
  const bool df = h->use_a0df();  // z stays FP32 for the split A0 product (no FP64 copy)
  dotT<double>(h, N, S.b, (const double*)nullptr, S.sc, R_BB);
  launch(h, mmk::k_pcg_init_scalars, 1, 32, S.sc, tol, maxiter);
  LAUNCH_CHECK();
  auto& l0 = S.lv[0];
  tagged<double>(h, MM_PROF_INIT_RESIDUAL, 0, mat_bytes(l0.A) + 3.0 * 8.0 * N, [&] {
    launch(h, mmk::k_init_residual<double>, grid_ilp(N), BS, l0.A.s, S.x, S.b, S.r, (const double*)nullptr,
           l0.x, S.sc, h->d_part);
    LAUNCH_CHECK();
  });
  launch(h, mmk::k_split_mp, grid_elem(N), BS, N, S.r, F.lv[0].s, F.r, F.lv[0].x);
  LAUNCH_CHECK();
  enqueue_vcycle<float>(h, F, F.r, F.z, false, nullptr, S.sc, df ? nullptr : S.z);
}

void run_pcg_mp(mm_problem* h, double tol, int maxiter, int* iters, double* r2_out, PcgPending* pend = nullptr) {
  auto& S = h->s64;
  enqueue_pcg_mp_start(h, tol, maxiter);
  const bool graph = h->use_graph && !h->prof && loop_graph_or_retry(h, S, [&] { enqueue_iteration_mp(h); });
  if (graph) {
    CK(cudaGraphLaunch(S.exec, h->st));
  } else {
    // host-polled: read `done` every fourth iteration (every step when profiling)
    const int every = h->prof ? 1 : 4;
    for (int i = 0;; ++i) {
      enqueue_iteration_mp(h);
      if ((i + 1) % every == 0) {
        CK(cudaMemcpyAsync(h->h_sc, S.sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
        h->sync();
        if (h->h_sc->done || i > maxiter + 8) break;
      }
    }
  }
  CK(cudaMemcpyAsync(h->h_sc, S.sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
  if (pend) {
    *pend = PcgPending{&S, graph};
    return;
  }
  h->sync();
  check_barrier(h->h_sc);
  if (graph) h->n_launch += (int64_t)h->h_sc->loops * S.iter_launches;
  if (iters) *iters = h->h_sc->it;
  if (r2_out) *r2_out = h->h_sc->red[R_R2];
}

// b = D m on device (magnetic rows), b.b -> red[R_BB0]
void enqueue_rhs(mm_problem* h, const double* m) {
  const int N = h->N;
  if (!h->has_mask) CK(cudaMemsetAsync(h->d_b, 0, N * sizeof(double), h->st));
  mmk::k_rhs_s<<<grid_elem(h->eops.n_rows), BS, 0, h->st>>>(h->eops, m, h->d_b);
  LAUNCH_CHECK();
  dot(h, N, h->d_b, nullptr, R_BB0);
}

void sub_mean(mm_problem* h, double* x) {
  const int N = h->N;
  mmk::k_mean<<<grid_elem(N), BS, 0, h->st>>>(N, x, h->d_sc, h->d_part, R_SUM);
  LAUNCH_CHECK();
  mmk::k_sub_mean<<<grid_elem(N), BS, 0, h->st>>>(N, x, h->d_sc, R_SUM);
  LAUNCH_CHECK();
}

// Mixed precision: FP64 iterative refinement around FP32 inner PCG solves.  Each step computes the
// true residual r = b - A x in FP64, solves A d = r / |r| with the FP32 hierarchy to a relative
// residual eta (never asking more than the remaining reduction), and adds |r| d to x in FP64.
// Stops when the FP64 residual meets |r| <= tol |b|.  Returns (inner iterations, final r.r).
int run_mixed(mm_problem* h, double tol, int maxiter, int* iters, double* r2_out) {
  const int N = h->N;
  auto& A64 = h->s64.lv[0].A;
  dot(h, N, h->d_b, nullptr, R_BB);
  const double bb = h->red(R_BB);
  int total = 0, outer = 0;
  double rr = 0.0;
  while (true) {
    launch(h, mmk::k_resid64, grid_ilp(N), BS, A64.s, h->d_x, h->d_b, h->d_r64, h->d_sc, h->d_part);
    LAUNCH_CHECK();
    rr = h->red(R_R2);
    if (!(rr > tol * tol * bb) || outer >= h->mixed_max_outer || total >= maxiter || !std::isfinite(rr)) break;
    const double rn = std::sqrt(rr);
    launch(h, mmk::k_to_f32, grid_ilp(N), BS, N, h->d_r64, 1.0 / rn, h->d_r32, h->d_d32);
    LAUNCH_CHECK();
    const double need = tol * std::sqrt(bb) / rn;  // relative reduction still required
    const double eta = std::max(h->mixed_eta, 0.5 * need);
    int it = 0;
    run_pcg<float>(h, h->s32, eta, std::max(1, maxiter - total), &it, nullptr);
    total += it;
    launch(h, mmk::k_add_f32, grid_ilp(N), BS, N, h->d_x, h->d_d32, rn);
    LAUNCH_CHECK();
    ++outer;
  }
  h->last_outer = outer;
  if (iters) *iters = total;
  if (r2_out) *r2_out = rr;
  return outer;
}

// demag solve with the potential in d_U (in/out)
// h_out (host, or null): the potential is also copied there, behind the solve and inside its one wait.
// x0_ready (or null): an event the initial guess d_U waits for (its copy from the host on another
// stream, which then overlaps the right-hand side)
int solve_dev(mm_problem* h, const double* d_m, double* d_U, double tol, int maxiter, int* iters, double* rel_res,
              double* h_out = nullptr, cudaEvent_t x0_ready = nullptr) {
  if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called before a solve"};
  CK(cudaEventRecord(h->ev0, h->st));
  enqueue_rhs(h, d_m);
  if (x0_ready) CK(cudaStreamWaitEvent(h->st, x0_ready, 0));
  if (d_U != h->d_x) CK(cudaMemcpyAsync(h->d_x, d_U, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  const bool zero_mean = !h->has_mask;
  if (zero_mean) {
    sub_mean(h, h->d_b);
    sub_mean(h, h->d_x);
  }
  int it = 0;
  double r2 = 0.0;
  double tol2_ref = 0.0;
  // the PCG paths queue their scalars copy and are read after the one wait below (it carries r.r,
  // the iteration count, tol2 and b.b)
  PcgPending pend;
  if (h->mixed && h->s32.built) {
    run_mixed(h, tol, maxiter, &it, &r2);
    tol2_ref = tol * tol * h->red(R_BB);
  } else if (h->fp32_precond && h->s32.built && multilevel(h, h->s32)) {
    run_pcg_mp(h, tol, maxiter, nullptr, nullptr, &pend);
  } else {
    run_pcg<double>(h, h->s64, tol, maxiter, nullptr, nullptr, &pend);
  }
  if (zero_mean) sub_mean(h, h->d_x);
  if (d_U != h->d_x) CK(cudaMemcpyAsync(d_U, h->d_x, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  CK(cudaEventRecord(h->ev1, h->st));
  if (h_out) {
    CK(cudaMemcpyAsync(h_out, h->d_x, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  } else {
    CK(cudaEventSynchronize(h->ev1));
  }
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
  h->last_solve_ms = ms;
  if (h->prof) h->prof_fold();
  double bb0;
  if (pend.S) {
    finish_pcg(h, pend, &it, &r2);
    tol2_ref = h->h_sc->tol2;
    bb0 = h->h_sc->red[R_BB0];
  } else {
    bb0 = h->red(R_BB0);
  }
  if (iters) *iters = it;
  const double rr = std::sqrt(r2 / (bb0 + 1e-30));
  if (rel_res) *rel_res = rr;
  if (!std::isfinite(rr)) return MM_NONFINITE;
  return (it >= maxiter && r2 > tol2_ref) ? MM_MAXITER : MM_OK;
}

// the float-float operator pass with TP lanes per magnetic row
template <int TP>
void energy_ff_rows(mm_problem* h, const double* d_m, const double* B, const double* d_B, const double* d_bias,
                    double* d_g) {
  const mmk::EnergySellFF& o = h->eopsff;
  const mmk::NodesFF& nf = h->w_ff;
  mmk::k_energy_grad_ff<TP><<<grid_rows(o.n_rows, TP), BS, 0, h->st>>>(o, nf.hi, nf.lo, nf.u, d_m, h->d_Mn, B[0], B[1],
                                                                      B[2], d_B, d_bias, h->inv_Vmag, d_g, h->d_sc,
                                                                      h->d_part);
}

// the launches of one energy and gradient evaluation (m.(g + g_z) into red[R_E]): float-float in the
// mixed-precision problems (MM_OPT_ENERGY_FF), else FP64
void enqueue_energy(mm_problem* h, const double* d_m, const double* d_U, const double* B, const double* d_bias,
                    double* d_g, const double* d_B = nullptr) {
  if (h->use_energy_ff()) {
    const mmk::EnergySellFF& o = h->eopsff;
    const mmk::NodesFF& nf = h->w_ff;
    mmk::k_split_ff<<<grid_elem(o.n_touched), BS, 0, h->st>>>(o.n_touched, o.touched, d_m, d_U, o.kx, o.ky, o.kz,
                                                               nf);
    LAUNCH_CHECK();
    switch (h->eff_tpr) {
      case 1: energy_ff_rows<1>(h, d_m, B, d_B, d_bias, d_g); break;
      case 2: energy_ff_rows<2>(h, d_m, B, d_B, d_bias, d_g); break;
      case 8: energy_ff_rows<8>(h, d_m, B, d_B, d_bias, d_g); break;
      default: energy_ff_rows<4>(h, d_m, B, d_B, d_bias, d_g); break;
    }
    LAUNCH_CHECK();
    return;
  }
  mmk::k_energy_grad_s<<<grid_elem(h->eops.n_rows), BS, 0, h->st>>>(h->eops, d_m, d_U, h->d_Mn, B[0], B[1], B[2],
                                                                     d_B, d_bias, h->inv_Vmag, d_g, h->d_sc,
                                                                     h->d_part);
  LAUNCH_CHECK();
}

double energy_dev(mm_problem* h, const double* d_m, const double* d_U, const double* B, const double* d_bias,
                  double* d_g) {
  enqueue_energy(h, d_m, d_U, B, d_bias, d_g);
  return 0.5 * h->red(R_E) * h->inv_Vmag;
}

void local_grad_dev(mm_problem* h, const double* d_v, double* d_out) {
  mmk::k_local_grad_s<<<grid_elem(h->eops.n_rows), BS, 0, h->st>>>(h->eops, d_v, h->inv_Vmag, d_out);
  LAUNCH_CHECK();
}

// Makes a problem's device current for one entry-point call and restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    int cur = -1;
    if (dev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess)
      prev = cur;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

template <class F>
int guarded(mm_problem* h, F&& f) {
  DeviceGuard device_guard(h ? h->device : -1);
  try {
    return f();
  } catch (const Fail& e) {
    if (h) h->err = e.msg;
    else g_create_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    if (h) h->err = "host allocation failed";
    return MM_ERR_OOM;
  } catch (const std::exception& e) {
    if (h) h->err = e.what();
    else g_create_error = e.what();
    return MM_ERR_SETUP;
  }
}

}  // namespace

// =============================================================================================
// minimizer (host-driven control flow on device vectors, as src/minimizers.py's step functions)
// =============================================================================================
namespace {

struct MinCtx {
  mm_problem* h;
  int N;
  double B[3];
  double phi_tol;
  const mm_min_params* prm;
  int demag = 0, evals = 0, preco = 0;
  double demag_ms = 0.0, demag_wall = 0.0;  // device and host time of the demag solves
};

void ensure_min_buffers(mm_problem* h, int memory) {
  const size_t n3 = 3 * (size_t)h->N;
  if (!h->min_ready) {
    double** bufs[] = {&h->w_gt, &h->w_gte, &h->w_gprev, &h->w_y, &h->w_d, &h->w_dprev, &h->w_H, &h->w_mt,
                       &h->w_gt_trial, &h->w_graw, &h->w_r3, &h->w_z3, &h->w_p3, &h->w_Ap3, &h->w_tmp,
                       &h->w_mprev, &h->w_gtprev, &h->w_ys, &h->w_x1, &h->w_x2, &h->w_x3, &h->w_x4};
    for (double** b : bufs) {
      *b = h->alloc<double>(n3);
      CK(cudaMemsetAsync(*b, 0, n3 * sizeof(double), h->st));
    }
    for (double** b : {&h->w_Ut, &h->w_U2, &h->w_U3}) {
      *b = h->alloc<double>(h->N);
      CK(cudaMemsetAsync(*b, 0, h->N * sizeof(double), h->st));
    }
    h->min_ready = true;
  }
  if (memory > h->lb_mem) {
    h->d_lb = h->alloc<double>(2 * (size_t)memory + 1);
    h->lb_mem = memory;
  }
  while ((int)h->w_S.size() < memory) {
    double* s = h->alloc<double>(n3);
    double* y = h->alloc<double>(n3);
    CK(cudaMemsetAsync(s, 0, n3 * sizeof(double), h->st));
    CK(cudaMemsetAsync(y, 0, n3 * sizeof(double), h->st));
    h->w_S.push_back(s);
    h->w_Y.push_back(y);
  }
}

double dev_dot(mm_problem* h, int n, const double* a, const double* b) {
  dot(h, n, a, b, R_A);
  return h->red(R_A);
}

// reductions read together with one copy sit in consecutive slots
static_assert(mmk::R_A == mmk::R_MAX + 1 && mmk::R_B == mmk::R_MAX + 2 && mmk::R_D == mmk::R_C + 1,
              "consecutive reduction slots");

double dev_absmax(mm_problem* h, int n, const double* a) {
  mmk::k_absmax<<<grid_vec(n), BS, 0, h->st>>>(n, a, h->d_sc, h->d_part);
  LAUNCH_CHECK();
  return h->red(R_MAX);
}

// energy + gradient of (m, U) into g, E returned
double eval(MinCtx& c, const double* m, const double* U, double* g) {
  return energy_dev(c.h, m, U, c.B, c.h->d_min_bias, g);
}

// solve_U(m, U (warm start, in place), tol) -> iterations
int demag_solve(MinCtx& c, const double* m, double* U, double tol) {
  int it = 0;
  double rr = 0.0;
  const int cg_maxiter = c.prm->cg_maxiter > 0 ? c.prm->cg_maxiter : 2000;
  const auto t0 = std::chrono::steady_clock::now();
  solve_dev(c.h, m, U, tol, cg_maxiter, &it, &rr);
  c.demag_wall += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  c.demag_ms += c.h->last_solve_ms;
  return it;
}

// one trip of the device-driven inner solve: P p with alpha and the stop tests, the step with beta
// and the loop test, the new direction
template <class Op, class T>
void enqueue_inner_trip(mm_problem* h, const Op& op, const double* m, const double* gext, T reg, T inv_Vmag, T* r,
                        T* z, T* p, T* Ap, T* y) {
  const int N = h->N;
  launch(h, mmk::k_in_apply<Op, T>, grid_vec(op.n_rows), BS, op, m, gext, p, reg, inv_Vmag, Ap, h->d_sc,
         h->d_part);
  launch(h, mmk::k_in_step<T>, grid_vec(N), BS, N, y, r, p, Ap, h->d_inv_M_prec, z, h->d_sc, h->d_part);
  launch(h, mmk::k_in_xpay<T>, grid_vec(3 * N), BS, 3 * N, z, p, h->d_sc);
}

// The inner PCG loop of solve_Py_g queued without host waits: setup and start, then the WHILE graph
// cached per (m, g_ext, y, reg, precision) (or, without conditional graphs, one wait per trip).  The
// iteration count lands in red[R_D].
template <class Op, class T>
void run_inner(mm_problem* h, const Op& op, const double* m, const double* gext, const double* gte, double tol,
               double reg, T inv_Vmag, T* r, T* z, T* p, T* Ap, T* y, int max_iter, double nu) {
  const int N = h->N;
  launch(h, mmk::k_in_setup, 1, 32, h->d_sc, max_iter, nu, tol * tol, h->inner_cpp_count ? 1 : 0);
  launch(h, mmk::k_in_init<T>, grid_vec(N), BS, N, gte, h->d_inv_M_prec, r, z, p, y, h->d_sc, h->d_part);
  h->n_launch += 2;
  const bool fp32 = std::is_same<T, float>::value;
  const T reg_t = (T)reg;
  auto trip = [&] { enqueue_inner_trip<Op, T>(h, op, m, gext, reg_t, inv_Vmag, r, z, p, Ap, y); };
  cudaGraphExec_t ex = nullptr;
  if (h->use_graph && !h->prof && !h->inner_graph_failed) {
    for (auto& ig : h->inner_graphs)
      if (ig.m == m && ig.gext == gext && ig.y == y && ig.reg == reg && ig.fp32 == fp32) ex = ig.ex;
    if (!ex) {
      mm_problem::InnerGraph ig{m, gext, y, reg, fp32, nullptr, nullptr};
      const bool ok = capture_while_graph(
          h,
          [&](cudaGraphConditionalHandle hnd) {
            trip();
            launch(h, mmk::k_in_cond, 1, 32, hnd, h->d_sc);
          },
          &ig.g, &ig.ex);
      if (ok) {
        if (h->inner_graphs.size() >= 8) {
          CK(cudaStreamSynchronize(h->st));
          cudaGraphExecDestroy(h->inner_graphs.front().ex);
          cudaGraphDestroy(h->inner_graphs.front().g);
          h->inner_graphs.erase(h->inner_graphs.begin());
        }
        h->inner_graphs.push_back(ig);
        ex = ig.ex;
      } else {
        h->inner_graph_failed = true;
      }
    }
  }
  if (ex) {
    CK(cudaGraphLaunch(ex, h->st));
    h->n_launch += 4;  // the trips' kernels are counted by the caller from the iteration count
    return;
  }
  for (int t = 0; t < max_iter + 2; ++t) {
    trip();
    h->n_launch += 3;
    CK(cudaMemcpyAsync(&h->h_sc->in_done, &h->d_sc->in_done, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (h->h_sc->in_done) break;
  }
}

// Inner PCG with Steihaug exit (src/minimizers.py:413-490); y = result; returns iterations.
// max_iter < 0 takes pc_iters, nu < 0 the parameters' stagnation threshold.  The iteration runs on
// the device (alpha, the curvature and stagnation tests, beta and the stopping test are formed by the
// reductions' finishing blocks); the host waits once, for the fallback test.  In the mixed-precision
// modes the operator, the vectors and the inner products are FP32 (float-float sums), the result is
// widened to FP64.
int solve_Py_g(MinCtx& c, const double* m, const double* gext, const double* gte, double tol, double* y,
               double reg, int max_iter = -1, double nu = -1.0) {
  if (max_iter < 0) max_iter = c.prm->pc_iters;
  if (nu < 0) nu = c.prm->pc_stagnation_nu;
  mm_problem* h = c.h;
  const int N = c.N, n3 = 3 * N;
  const int ge = grid_vec(N);
  const bool fp32 = h->inner_fp32();
  // fallback direction z_fb = gte .* inv_M_prec (into w_z3), clipping, descent check: |y|^2, |z_fb|^2
  // and y.gte from one pass, the iteration count beside them, one wait
  if (fp32) {
    run_inner<mmk::EnergySell32, float>(h, h->eops32, m, gext, gte, tol, reg, 1.0f, h->w_r3f, h->w_z3f, h->w_p3f,
                                        h->w_Ap3f, h->w_yf, max_iter, nu);
    mmk::k_fallback_dots32<<<ge, BS, 0, h->st>>>(N, h->w_yf, gte, h->d_inv_M_prec, h->w_z3, h->d_sc, h->d_part);
  } else {
    run_inner<mmk::EnergySell, double>(h, h->eops, m, gext, gte, tol, reg, h->inv_Vmag, h->w_r3, h->w_z3, h->w_p3,
                                       h->w_Ap3, y, max_iter, nu);
    mmk::k_fallback_dots<<<ge, BS, 0, h->st>>>(N, y, gte, h->d_inv_M_prec, h->w_z3, h->d_sc, h->d_part);
  }
  LAUNCH_CHECK();
  const double* f = h->red_n(R_A, 4);
  const double yn = std::sqrt(f[0]), zn = std::sqrt(f[1]);
  double yg = f[2];
  const int it = (int)f[3];
  h->n_launch += 3 * (int64_t)it;
  const bool clip = yn > 10.0 * zn;
  const double cf = clip ? 10.0 * zn / (yn + 1e-30) : 1.0;
  if (fp32) {
    mmk::k_widen_scale<<<grid_vec(n3), BS, 0, h->st>>>(n3, h->w_yf, cf, y);
    LAUNCH_CHECK();
  } else if (clip) {
    mmk::k_scale<<<grid_vec(n3), BS, 0, h->st>>>(n3, cf, y);
    LAUNCH_CHECK();
  }
  if (clip) yg = dev_dot(h, n3, y, gte);  // the clipped direction's slope, as the unfused test computed it
  if (!(yg > 1e-12)) {
    CK(cudaMemcpyAsync(y, h->w_z3, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  }
  return it;
}

// out = P v (the extensive local Hessian, src/minimizers.py:396-411); returns v.out
double apply_P(MinCtx& c, const double* m, const double* gext, const double* v, double reg, double* out) {
  mm_problem* h = c.h;
  mmk::k_apply_P_s<<<grid_vec(h->eops.n_rows), BS, 0, h->st>>>(h->eops, m, gext, v, reg, h->inv_Vmag, out, h->d_sc,
                                                                 h->d_part, R_C);
  LAUNCH_CHECK();
  return h->red(R_C);
}

// sum M_rel a1.b1 and sum M_rel a2.b2
std::pair<double, double> dev_mdot2(mm_problem* h, const double* a1, const double* b1, const double* a2,
                                    const double* b2) {
  mmk::k_mdot2<<<grid_vec(h->N), BS, 0, h->st>>>(h->N, a1, b1, a2, b2, h->d_inv_M_rel, h->d_sc, h->d_part);
  LAUNCH_CHECK();
  const double* v = h->red_n(R_A, 2);
  return {v[0], v[1]};
}

// sum M_rel |y + a p|^2
double dev_mnorm_axpy(mm_problem* h, const double* y, double a, const double* p) {
  mmk::k_mnorm_axpy<<<grid_vec(h->N), BS, 0, h->st>>>(h->N, y, a, p, h->d_inv_M_rel, h->d_sc, h->d_part);
  LAUNCH_CHECK();
  return h->red(R_C);
}

// positive root of a x^2 + b x + c = 0 (the step to the trust-region boundary)
double tr_boundary_step(double a, double b, double c) {
  return (-b + std::sqrt(std::max(0.0, b * b - 4.0 * a * c))) / (2.0 * a);
}

// Steihaug-Toint truncated PCG inside the M_rel-norm ball of radius delta (src/minimizers.py:506-592);
// y = result; returns iterations
int solve_Py_g_tr(MinCtx& c, const double* m, const double* gext, const double* rhs, double delta, int max_iter,
                  double tol, double reg, double* y) {
  mm_problem* h = c.h;
  const int N = c.N, n3 = 3 * N;
  const int ge = grid_vec(N);
  CK(cudaMemsetAsync(y, 0, n3 * sizeof(double), h->st));
  CK(cudaMemcpyAsync(h->w_r3, rhs, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  mmk::k_scale3_dot<<<ge, BS, 0, h->st>>>(N, h->w_r3, h->d_inv_M_prec, h->w_z3, h->d_sc, h->d_part, R_B);
  LAUNCH_CHECK();
  CK(cudaMemcpyAsync(h->w_p3, h->w_z3, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  double rho = h->red(R_B);
  const double target = tol * tol * rho;
  const double d2 = delta * delta;
  int it = 0;
  bool done = false;
  while (it < max_iter && rho > target && rho > 1e-25 && rho < 1e20 && !done) {
    const double pAp = apply_P(c, m, gext, h->w_p3, reg, h->w_Ap3);
    const double alpha = rho / (pAp + 1e-30);
    const auto pp_yp = dev_mdot2(h, h->w_p3, h->w_p3, y, h->w_p3);
    const double yy = dev_mdot2(h, y, y, y, y).first;
    const double a_q = pp_yp.first + 1e-30, b_q = 2.0 * pp_yp.second, c_q = yy - d2;
    const double alpha_tr = tr_boundary_step(a_q, b_q, c_q);
    done = (pAp <= 0.0) || (dev_mnorm_axpy(h, y, alpha, h->w_p3) >= d2);
    mmk::k_inner_step<<<ge, BS, 0, h->st>>>(N, done ? alpha_tr : alpha, alpha, y, h->w_r3, h->w_p3, h->w_Ap3,
                                             h->d_inv_M_prec, h->w_z3, h->d_sc, h->d_part, R_B, 1);
    LAUNCH_CHECK();
    const double rho_next = h->red(R_B);
    if (!done) {
      mmk::k_xpay<<<grid_vec(n3), BS, 0, h->st>>>(n3, h->w_z3, rho_next / (rho + 1e-30), h->w_p3);
      LAUNCH_CHECK();
    }
    rho = rho_next;
    ++it;
  }
  mmk::k_scale3_dot<<<ge, BS, 0, h->st>>>(N, rhs, h->d_inv_M_prec, h->w_z3, h->d_sc, h->d_part, R_B);
  LAUNCH_CHECK();
  const double yn = std::sqrt(dev_dot(h, n3, y, nullptr));
  const double zn = std::sqrt(dev_dot(h, n3, h->w_z3, nullptr));
  if (yn > 10.0 * zn) {
    mmk::k_scale<<<grid_vec(n3), BS, 0, h->st>>>(n3, 10.0 * zn / (yn + 1e-30), y);
    LAUNCH_CHECK();
  }
  const double ym = std::sqrt(dev_mdot2(h, y, y, y, y).first + 1e-30);
  if (ym > delta) {
    mmk::k_scale<<<grid_vec(n3), BS, 0, h->st>>>(n3, delta / ym, y);
    LAUNCH_CHECK();
  }
  return it;
}

struct LSResult {
  double tau, E;
  int evals, demag;
  bool accepted;
};

// Curvilinear Armijo search (src/minimizers.py:265-385).  On acceptance the trial state is in
// (w_mt, w_Ut, w_gt_trial); otherwise the caller keeps (m, U, g_raw).
LSResult armijo(MinCtx& c, const double* m, double pg, const double* H, double E0, const double* U_base, double s0) {
  mm_problem* h = c.h;
  const int N = c.N;
  const mm_min_params* p = c.prm;
  LSResult res{0.0, E0, 0, 0, false};
  if (pg >= 0) return res;
  CK(cudaMemcpyAsync(h->w_Ut, U_base, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  auto D = [&](double s, double& E_t) {
    mmk::k_cayley<<<grid_vec(N), BS, 0, h->st>>>(N, m, H, s, h->w_mt);
    LAUNCH_CHECK();
    res.demag += demag_solve(c, h->w_mt, h->w_Ut, c.phi_tol);
    E_t = eval(c, h->w_mt, h->w_Ut, h->w_gt_trial);
    if (!std::isfinite(E_t)) E_t = 1e20;
    return (E_t - E0) / (s * pg + 1e-30);
  };
  const int max_evals = p->ls_max_evals > 0 ? p->ls_max_evals : 15;
  double s = s0, s_min = 0.0, d_v = 0.0, E_v = E0;
  int it_exp = 0, it_con = 0;
  bool done = false;
  while (it_exp < max_evals && !done) {
    double E_t;
    const double d = D(s, E_t);
    d_v = d;
    E_v = E_t;
    const bool stop = (std::fabs(1.0 - d) >= p->ls_eta2) || (d < 0);
    if (!stop) {
      s_min = s;
      s = p->ls_C * s;
    }
    ++it_exp;
    done = stop;
  }
  done = (d_v >= p->ls_eta1) && (d_v < 1e10);
  while (it_con < max_evals && !done) {
    s = s_min + p->ls_c * (s - s_min);
    double E_t;
    const double d = D(s, E_t);
    d_v = d;
    E_v = E_t;
    done = (d >= p->ls_eta1) && (d < 1e10);
    ++it_con;
  }
  res.evals = it_exp + it_con;
  if (d_v >= 0) {
    res.tau = s;
    res.E = E_v;
    res.accepted = true;
  }
  return res;
}

bool check_conv(int it, double E, double E_prev, double diff_m, double gnorm, const mm_min_params* p) {
  if (it <= 0) return false;
  const bool u1 = (E_prev - E) < p->tau_f * (1.0 + std::fabs(E));
  const bool u2 = diff_m < std::sqrt(p->tau_f) * 2.0;
  const bool u3 = gnorm <= std::pow(p->tau_f, 1.0 / 3.0) * (1.0 + std::fabs(E));
  const bool u4 = gnorm < p->eps_a;
  return (u1 && u2 && u3) || u4;
}

// accept the line-search trial: m <- w_mt, U <- w_Ut, g_raw <- w_gt_trial (buffer swaps)
void accept_trial(mm_problem* h, double*& m, double*& U, double*& graw) {
  std::swap(m, h->w_mt);
  std::swap(U, h->w_Ut);
  std::swap(graw, h->w_gt_trial);
}

// ---------------------------------------------------------------------------------------------
// Device-driven iterations of pcohen_hs, pcohen and pcg (MM_OPT_MIN_GRAPH).  One graph holds the
// minimizer loop as a WHILE node; the inner preconditioner solve, the Armijo trials and each trial's
// demag PCG are WHILE nodes nested in it, and every decision the host loop takes between kernels is
// a k_min_* / k_ls_* kernel over MinScal.  A field step then waits on the host once.  The launches
// and reductions are the host loop's (same grids), so the results are the same to the last bit.
// ---------------------------------------------------------------------------------------------

// WHILE (hnd) { body } appended to the graph that h->st is capturing.  The conditional node takes the
// stream's current dependencies; its body is captured on the auxiliary stream of this nesting depth
// (h->st is swapped for it meanwhile); the node then becomes the stream's only dependency.  The
// first launch after the node is a plain one (a programmatic edge leaves only a kernel node).
template <class Body>
void capture_nested_while(mm_problem* h, cudaGraphConditionalHandle hnd, Body&& body) {
  if (h->cap_depth >= 3) throw Fail{MM_ERR_STATE, "minimizer graph: loops nested too deeply"};
  cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t ndeps = 0;
  CK(cudaStreamGetCaptureInfo(h->st, &status, nullptr, &g, &deps, &edges, &ndeps));
  if (status != cudaStreamCaptureStatusActive) throw Fail{MM_ERR_STATE, "minimizer graph: no capture"};
  std::vector<cudaGraphNode_t> dv(deps, deps + ndeps);
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hnd;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  CK(cudaGraphAddNode(&node, g, dv.empty() ? nullptr : dv.data(), nullptr, dv.size(), &cp));
  cudaStream_t& aux = h->aux_st[h->cap_depth];
  if (!aux) CK(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
  CK(cudaStreamBeginCaptureToGraph(aux, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  cudaStream_t saved = h->st;
  h->st = aux;
  ++h->cap_depth;
  bool ok = true;
  Fail err{MM_OK, ""};
  try {
    body();
  } catch (const Fail& f) {
    ok = false;
    err = f;
  } catch (...) {  // the capture is ended and the stream restored whatever the body threw
    ok = false;
    err = Fail{MM_ERR_STATE, "minimizer graph: capture of a loop body failed"};
  }
  h->st = saved;
  --h->cap_depth;
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(aux, &out);
  if (!ok) throw err;
  CK(e);
  CK(cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
}

// The demag solve of a line-search trial: solve_dev's work, kernels only, with the PCG loop (FP64 or
// FP32-preconditioned) as a nested WHILE node; its iterations go to MinScal.
void enqueue_demag_nested(mm_problem* h, const double* m, double* U, double tol, int maxiter,
                          cudaGraphConditionalHandle hnd, mmk::MinScal* ms, int64_t* per_trip) {
  const int N = h->N;
  mmk::k_copy_vec<<<grid_vec(N), BS, 0, h->st>>>(N, U, h->d_x);
  LAUNCH_CHECK();
  if (!h->has_mask) {
    mmk::k_zero_vec<<<grid_vec(N), BS, 0, h->st>>>(N, h->d_b);
    LAUNCH_CHECK();
  }
  mmk::k_rhs_s<<<grid_elem(h->eops.n_rows), BS, 0, h->st>>>(h->eops, m, h->d_b);
  LAUNCH_CHECK();
  dot(h, N, h->d_b, nullptr, R_BB0);
  if (!h->has_mask) {
    sub_mean(h, h->d_b);
    sub_mean(h, h->d_x);
  }
  auto& S = h->s64;
  const bool mp = h->fp32_precond && h->s32.built && multilevel(h, h->s32);
  if (mp) enqueue_pcg_mp_start(h, tol, maxiter);
  else enqueue_pcg_start<double>(h, S, tol, maxiter);
  mmk::k_cond_set<<<1, 32, 0, h->st>>>(hnd, 1u);  // the loop graph's default: one trip at least
  LAUNCH_CHECK();
  capture_nested_while(h, hnd, [&] {
    const int64_t b0 = h->n_launch;
    if (mp) enqueue_iteration_mp(h);
    else enqueue_iteration<double>(h, S);
    launch(h, mmk::k_set_cond, 1, 32, hnd, S.sc);
    *per_trip = h->n_launch - b0 + 1;
  });
  if (!h->has_mask) sub_mean(h, h->d_x);
  mmk::k_copy_vec<<<grid_vec(N), BS, 0, h->st>>>(N, h->d_x, U);
  LAUNCH_CHECK();
  mmk::k_min_demag<<<1, 32, 0, h->st>>>(S.sc, ms);
  LAUNCH_CHECK();
}

// The inner preconditioner solve P y = g_tan_ext (solve_Py_g) with its forcing tolerance, clipping
// and fallback formed on the device.
template <class Op, class T>
void enqueue_inner_nested(mm_problem* h, const Op& op, const double* m, const double* gext, const double* gte,
                          double reg, T inv_Vmag, T* r, T* z, T* p, T* Ap, T* y, cudaGraphConditionalHandle hnd,
                          mmk::MinScal* ms, int64_t* per_trip) {
  const int N = h->N;
  mmk::k_min_in_setup<<<1, 32, 0, h->st>>>(h->d_sc, ms);
  LAUNCH_CHECK();
  launch(h, mmk::k_in_init<T>, grid_vec(N), BS, N, gte, h->d_inv_M_prec, r, z, p, y, h->d_sc, h->d_part);
  LAUNCH_CHECK();
  mmk::k_cond_set<<<1, 32, 0, h->st>>>(hnd, 1u);
  LAUNCH_CHECK();
  const T reg_t = (T)reg;
  capture_nested_while(h, hnd, [&] {
    enqueue_inner_trip<Op, T>(h, op, m, gext, reg_t, inv_Vmag, r, z, p, Ap, y);
    launch(h, mmk::k_in_cond, 1, 32, hnd, h->d_sc);
  });
  *per_trip = 4;
}

// Runs the iterations of pcohen_hs / pcohen / pcg from the state minimize_dev has set up (it = 0)
// through the cached graph of these buffers and settings.  Returns false, with nothing queued, when
// no graph can be built (the caller then runs its host loop).
uint64_t bits_of(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
}

bool minimize_graph(mm_problem* h, MinCtx& c, double* m, double* U, double E0, bool cpp, int* it_out,
                    double* E_out, double* gnorm_out, bool* conv_out) {
  const mm_min_params* prm = c.prm;
  const int N = h->N, n3 = 3 * N;
  const int meth = prm->method;
  const bool pr = meth == MM_METHOD_PCOHEN;
  const int proj = meth == MM_METHOD_PCG ? 0 : 1;
  const int cg_maxiter = prm->cg_maxiter > 0 ? prm->cg_maxiter : 2000;
  const bool mixed_solve = h->mixed && h->s32.built;  // FP64 refinement steps decided on the host
  if (!h->min_graph || h->min_graph_failed || !h->use_graph || h->prof || mixed_solve || prm->max_iter <= 0)
    return false;
  // lazily built operators first: nothing may allocate while the stream captures
  const bool fp32 = h->inner_fp32();
  const bool ff = h->use_energy_ff();
  const bool mp = h->fp32_precond && h->s32.built && multilevel(h, h->s32);
  if (mp) h->use_a0df();
  if (!h->d_ms) {
    h->d_ms = h->alloc<mmk::MinScal>(1);
    h->h_ms = (mmk::MinScal*)pinned_get();
  }
  double* graw = h->w_graw;
  const std::vector<uintptr_t> key = {
      (uintptr_t)m, (uintptr_t)U, (uintptr_t)graw, (uintptr_t)h->w_gte, (uintptr_t)h->w_gprev,
      (uintptr_t)h->w_y, (uintptr_t)h->w_ys, (uintptr_t)h->w_d, (uintptr_t)h->w_dprev, (uintptr_t)h->w_mt,
      (uintptr_t)h->w_Ut, (uintptr_t)h->w_gt_trial, (uintptr_t)h->d_min_bias, (uintptr_t)pr, (uintptr_t)proj,
      (uintptr_t)fp32, (uintptr_t)ff, (uintptr_t)mp, (uintptr_t)h->pdl, (uintptr_t)h->s64.epoch,
      (uintptr_t)h->s32.epoch, (uintptr_t)cg_maxiter, (uintptr_t)bits_of(c.phi_tol), (uintptr_t)bits_of(prm->pc_reg)};
  mm_problem::MinGraph* mg = nullptr;
  for (auto& x : h->min_graphs)
    if (x.key == key) mg = &x;
  if (!mg) {
    mm_problem::MinGraph ng{key, nullptr, nullptr, 0, 0, 0, 0};
    bool ok = cudaGraphCreate(&ng.g, 0) == cudaSuccess;
    cudaGraphConditionalHandle hnd[4];  // outer loop, inner solve, line search, demag PCG
    for (int i = 0; i < 4 && ok; ++i) ok = cudaGraphConditionalHandleCreate(&hnd[i], ng.g, 0, 0) == cudaSuccess;
    const int64_t saved = h->n_launch;
    if (ok) ok = cudaStreamBeginCaptureToGraph(h->st, ng.g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                 cudaSuccess;
    if (ok) {
      mmk::MinScal* ms = h->d_ms;
      mmk::Scalars* sc = h->d_sc;
      double* part = h->d_part;
      const int ge = grid_vec(N), g3 = grid_vec(n3);
      const int gdot = std::min(grid_ilp(n3), g_vec_cap);
      try {
        mmk::k_min_start<<<1, 32, 0, h->st>>>(hnd[0], ms);
        LAUNCH_CHECK();
        capture_nested_while(h, hnd[0], [&] {
          const int64_t o0 = h->n_launch;
          int64_t ls_body = 0;
          mmk::k_tangent2<<<ge, BS, 0, h->st>>>(N, m, graw, h->d_inv_M_rel, h->w_gt, h->w_gte, sc, part);
          LAUNCH_CHECK();
          // y = P^-1 g_tan_ext with clipping and the z_fb fallback (solve_Py_g)
          if (fp32) {
            enqueue_inner_nested<mmk::EnergySell32, float>(h, h->eops32, m, graw, h->w_gte, prm->pc_reg, 1.0f,
                                                           h->w_r3f, h->w_z3f, h->w_p3f, h->w_Ap3f, h->w_yf, hnd[1],
                                                           ms, &ng.per_in);
            mmk::k_fallback_dots32<<<ge, BS, 0, h->st>>>(N, h->w_yf, h->w_gte, h->d_inv_M_prec, h->w_z3, sc, part);
          } else {
            enqueue_inner_nested<mmk::EnergySell, double>(h, h->eops, m, graw, h->w_gte, prm->pc_reg, h->inv_Vmag,
                                                          h->w_r3, h->w_z3, h->w_p3, h->w_Ap3, h->w_y, hnd[1], ms,
                                                          &ng.per_in);
            mmk::k_fallback_dots<<<ge, BS, 0, h->st>>>(N, h->w_y, h->w_gte, h->d_inv_M_prec, h->w_z3, sc, part);
          }
          LAUNCH_CHECK();
          mmk::k_min_clip<<<1, 32, 0, h->st>>>(sc, ms);
          LAUNCH_CHECK();
          if (fp32) mmk::k_widen_clip<<<g3, BS, 0, h->st>>>(n3, h->w_yf, ms, h->w_y);
          else mmk::k_scale_clip<<<g3, BS, 0, h->st>>>(n3, h->w_y, ms);
          LAUNCH_CHECK();
          mmk::k_dot_flag<<<gdot, BS, 0, h->st>>>(&ms->flag, n3, h->w_y, h->w_gte, sc, part, R_A);
          LAUNCH_CHECK();
          mmk::k_min_fallback<<<1, 32, 0, h->st>>>(sc, ms);
          LAUNCH_CHECK();
          mmk::k_copy_flag<<<g3, BS, 0, h->st>>>(&ms->flag2, n3, h->w_z3, h->w_y);
          LAUNCH_CHECK();
          // beta (HS, or PR over y_prev.g_prev), direction with the descent safeguard, g_raw.d
          mmk::k_absmax<<<grid_vec(n3), BS, 0, h->st>>>(n3, h->w_y, sc, part);
          LAUNCH_CHECK();
          mmk::k_dot2diff<<<g3, BS, 0, h->st>>>(n3, h->w_y, h->w_dprev, h->w_gte, h->w_gprev, sc, part);
          LAUNCH_CHECK();
          if (pr) dot(h, n3, h->w_ys, h->w_gprev, R_C);
          mmk::k_min_beta<<<1, 32, 0, h->st>>>(sc, ms);
          LAUNCH_CHECK();
          mmk::k_direction_ms<<<ge, BS, 0, h->st>>>(N, m, h->w_y, h->w_dprev, ms, h->w_gte, graw, h->w_d, sc, part,
                                                   proj);
          LAUNCH_CHECK();
          mmk::k_min_descent<<<1, 32, 0, h->st>>>(sc, ms);
          LAUNCH_CHECK();
          mmk::k_neg_flag<<<g3, BS, 0, h->st>>>(&ms->flag, n3, h->w_y, h->w_d);
          LAUNCH_CHECK();
          mmk::k_dot_flag<<<gdot, BS, 0, h->st>>>(&ms->flag, n3, graw, h->w_d, sc, part, R_A);
          LAUNCH_CHECK();
          mmk::k_min_pg<<<1, 32, 0, h->st>>>(sc, ms);
          LAUNCH_CHECK();
          mmk::k_cross<<<ge, BS, 0, h->st>>>(N, m, h->w_d, h->w_H);
          LAUNCH_CHECK();
          // curvilinear Armijo search: each trial R(m, H, s), its demag solve (warm-started from the
          // previous trial's potential) and its energy
          mmk::k_copy_vec<<<grid_vec(N), BS, 0, h->st>>>(N, U, h->w_Ut);
          LAUNCH_CHECK();
          mmk::k_ls_init<<<1, 32, 0, h->st>>>(hnd[2], ms);
          LAUNCH_CHECK();
          capture_nested_while(h, hnd[2], [&] {
            const int64_t l0 = h->n_launch;
            int64_t pcg_trip = 0;
            mmk::k_cayley_ms<<<grid_vec(N), BS, 0, h->st>>>(N, m, h->w_H, ms, h->w_mt);
            LAUNCH_CHECK();
            enqueue_demag_nested(h, h->w_mt, h->w_Ut, c.phi_tol, cg_maxiter, hnd[3], ms, &pcg_trip);
            enqueue_energy(h, h->w_mt, h->w_Ut, c.B, h->d_min_bias, h->w_gt_trial, &ms->B[0]);
            mmk::k_ls_decide<<<1, 32, 0, h->st>>>(hnd[2], sc, ms, h->inv_Vmag);
            LAUNCH_CHECK();
            // the kernels of the PCG loop body are counted from the loop's trips, not per trial
            ls_body = h->n_launch - l0;
            ng.per_pcg = pcg_trip;
            ng.per_ls = ls_body - (pcg_trip - 1);
          });
          mmk::k_ls_finish<<<1, 32, 0, h->st>>>(ms);
          LAUNCH_CHECK();
          mmk::k_absmaxdiff<<<g3, BS, 0, h->st>>>(n3, h->w_mt, m, sc, part);
          LAUNCH_CHECK();
          mmk::k_min_advance<<<g3, BS, 0, h->st>>>(n3, N, ms, m, h->w_mt, U, h->w_Ut, graw,
                                                  h->w_gt_trial, h->w_gprev, h->w_gte, h->w_dprev, h->w_d,
                                                  pr ? h->w_ys : nullptr, h->w_y);
          LAUNCH_CHECK();
          mmk::k_min_conv<<<1, 32, 0, h->st>>>(hnd[0], sc, ms);
          LAUNCH_CHECK();
          ng.per_outer = (h->n_launch - o0) - ls_body;
        });
      } catch (...) {
        ok = false;
      }
      cudaGraph_t out = nullptr;
      const bool end_ok = cudaStreamEndCapture(h->st, &out) == cudaSuccess;
      ok = ok && end_ok;
    }
    h->n_launch = saved;
    if (ok) ok = cudaGraphInstantiate(&ng.ex, ng.g, 0) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();  // clear the failed attempt's error; the host loop runs instead
      if (ng.ex) cudaGraphExecDestroy(ng.ex);
      if (ng.g) cudaGraphDestroy(ng.g);
      h->min_graph_failed = true;
      return false;
    }
    if (h->min_graphs.size() >= 4) {
      CK(cudaStreamSynchronize(h->st));
      cudaGraphExecDestroy(h->min_graphs.front().ex);
      cudaGraphDestroy(h->min_graphs.front().g);
      h->min_graphs.erase(h->min_graphs.begin());
    }
    h->min_graphs.push_back(ng);
    mg = &h->min_graphs.back();
  }
  // this call's parameters and starting scalars
  mmk::MinScal& s = *h->h_ms;
  s = mmk::MinScal{};
  s.max_iter = prm->max_iter;
  s.L = prm->L > 0 ? prm->L : N;
  s.pr = pr ? 1 : 0;
  s.pc_auto = prm->pc_auto;
  s.pc_iters = prm->pc_iters;
  s.max_evals = prm->ls_max_evals > 0 ? prm->ls_max_evals : 15;
  s.cpp = cpp ? 1 : 0;
  s.pc_force_eta = prm->pc_force_eta;
  s.pc_force_alpha = prm->pc_force_alpha;
  s.pc_nu = prm->pc_stagnation_nu;
  s.eta1 = prm->ls_eta1;
  s.eta2 = prm->ls_eta2;
  s.C = prm->ls_C;
  s.c = prm->ls_c;
  s.s0 = 1.0;
  s.tau_f = prm->tau_f;
  s.eps_a = prm->eps_a;
  s.u2_bound = std::sqrt(prm->tau_f) * 2.0;
  s.u3_root = std::pow(prm->tau_f, 1.0 / 3.0);
  for (int k = 0; k < 3; ++k) s.B[k] = c.B[k];
  s.E = E0;
  s.E_lag = E0;
  CK(cudaMemcpyAsync(h->d_ms, h->h_ms, sizeof(mmk::MinScal), cudaMemcpyHostToDevice, h->st));
  CK(cudaGraphLaunch(mg->ex, h->st));
  CK(cudaMemcpyAsync(h->h_ms, h->d_ms, sizeof(mmk::MinScal), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->h_sc, h->d_sc, sizeof(mmk::Scalars), cudaMemcpyDeviceToHost, h->st));
  h->sync();
  check_barrier(h->h_sc);
  c.evals += (int)s.evals;
  c.preco += (int)s.preco;
  c.demag += (int)s.demag;
  h->n_launch += 1 + (int64_t)s.outer_loops * mg->per_outer + s.evals * mg->per_ls + s.pcg_trips * mg->per_pcg +
                 s.in_trips * mg->per_in;
  *it_out = s.it;
  *E_out = s.E;
  *gnorm_out = s.gsm;
  *conv_out = s.conv != 0;
  return true;
}

int minimize_dev(mm_problem* h, const double* B, double*& m, double*& U, const mm_min_params* prm,
                 mm_min_info* info) {
  const int N = h->N, n3 = 3 * N;
  const int ge = grid_vec(N), g3 = grid_vec(n3);
  const int meth = prm->method;
  const bool lbfgs = meth == MM_METHOD_LBFGS || meth == MM_METHOD_PLBFGS || meth == MM_METHOD_DPLBFGS ||
                     meth == MM_METHOD_PCOHEN_LBFGS;
  const bool exact = meth == MM_METHOD_PCOHEN_EXACT || meth == MM_METHOD_PCOHEN_HS_EXACT;
  const bool cg_family = meth == MM_METHOD_PCOHEN_HS || meth == MM_METHOD_PCOHEN || meth == MM_METHOD_PCG;
  // the conventions of the reference's C++ minimizer (run_cpp_pcohen_hs_minimization,
  // src/cpp/cpp_mkl_minimizer.cpp:542-763), which implements pcohen_hs and pcohen only
  const bool cpp = prm->cpp_semantics != 0;
  if (cpp && meth != MM_METHOD_PCOHEN_HS && meth != MM_METHOD_PCOHEN)
    throw Fail{MM_ERR_ARG, "cpp_semantics applies to pcohen_hs and pcohen only"};
  struct CountMode {  // restores the inner solve's counting on every exit
    mm_problem* h;
    ~CountMode() { h->inner_cpp_count = false; }
  } count_mode{h};
  h->inner_cpp_count = cpp;
  ensure_min_buffers(h, lbfgs ? std::max(1, prm->memory) : 0);
  MinCtx c{h, N, {B[0], B[1], B[2]}, prm->phi_tol > 0 ? prm->phi_tol : std::min(prm->cg_tol, 0.1 * prm->tau_f), prm};
  const int tn_iters = prm->tn_iters > 0 ? prm->tn_iters : 5;
  const double lr = prm->lr > 0 ? prm->lr : 0.1;
  auto t0 = std::chrono::steady_clock::now();
  double* graw = h->w_graw;
  auto copy3 = [&](double* dst, const double* src) {
    CK(cudaMemcpyAsync(dst, src, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
  };
  auto neg3 = [&](double* dst, const double* src) {  // dst = -src
    mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, src, 0.0, dst);
    LAUNCH_CHECK();
  };
  auto zero3 = [&](double* dst) { CK(cudaMemsetAsync(dst, 0, n3 * sizeof(double), h->st)); };
  mmk::k_normalize<<<ge, BS, 0, h->st>>>(N, m);
  LAUNCH_CHECK();
  c.demag += demag_solve(c, m, U, prm->cg_tol);
  double E = eval(c, m, U, graw);
  mmk::k_tangent2<<<ge, BS, 0, h->st>>>(N, m, graw, h->d_inv_M_rel, h->w_gt, h->w_gte, h->d_sc, h->d_part);
  LAUNCH_CHECK();
  double gnorm = h->red(R_MAX);
  c.evals = 1;
  // initial state of each method (the reference's init_state_fn, src/minimizers.py:2993-3400):
  // g_prev in w_gprev, y_prev / z_prev in w_ys, d_prev / p_prev in w_dprev
  const bool tan_init = meth == MM_METHOD_COHEN || exact;  // these start from g_tan, the others g_tan_ext
  copy3(h->w_gprev, (cg_family || meth == MM_METHOD_COHEN || meth == MM_METHOD_PCOHEN_LBFGS) ? h->w_gte : h->w_gt);
  copy3(h->w_ys, tan_init ? h->w_gt : h->w_gte);
  neg3(h->w_dprev, tan_init ? h->w_gt : h->w_gte);
  copy3(h->w_mprev, m);
  copy3(h->w_gtprev, h->w_gt);
  if (meth == MM_METHOD_PCOHEN_LBFGS) copy3(h->w_x1, h->w_gte);  // z_prev
  if (exact || meth == MM_METHOD_AAPG || meth == MM_METHOD_AAPG_EXACT) {
    zero3(h->w_x1);  // H_prev (exact) or F_prev (aapg)
    zero3(h->w_x2);  // H_prev (aapg_exact)
  }
  if (meth == MM_METHOD_PNAG) {
    zero3(h->w_x4);  // velocity
    CK(cudaMemcpyAsync(h->w_U3, U, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));  // U_prev
  }
  if (meth == MM_METHOD_TN_SPLIT) {
    // TNState is built without the counters, so they start at zero (src/minimizers.py:3198-3203)
    c.evals = 0;
    c.demag = 0;
  }
  double tau_prev = exact ? 1.0 : 0.0;
  double E_last = E;     // cohen: the energy before the previous step
  double delta = 10.0;   // tr / ptr: trust-region radius
  const int L = prm->L > 0 ? prm->L : N;
  const int mem = std::max(1, prm->memory);
  std::vector<double> rho_h(mem, 0.0);
  int hist_it = 0;
  int it = 0;
  bool conv = false;

  // L-BFGS two-loop recursion on g_tan_ext; `initial(q, out)` applies the initial inverse Hessian.
  // The recursion's scalars (rho, alpha, the dots) stay on the device: the history's length and slots
  // are known on the host, so no step waits for a host read.
  double* d_rho = h->d_lb;
  double* d_alpha = h->d_lb ? h->d_lb + h->lb_mem : nullptr;
  double* d_gamma = h->d_lb ? h->d_lb + 2 * h->lb_mem : nullptr;
  auto two_loop = [&](double* out, auto&& initial) {
    const int n_hist = std::min(hist_it, mem);
    double* q = h->w_y;
    copy3(q, h->w_gte);
    for (int i = 0; i < n_hist; ++i) {
      const int idx = ((hist_it - 1 - i) % mem + mem) % mem;
      dot(h, n3, h->w_S[idx], q, R_A);
      mmk::k_lb_first<<<g3, BS, 0, h->st>>>(n3, d_rho + idx, h->d_sc, R_A, d_alpha + idx, h->w_Y[idx], q);
      LAUNCH_CHECK();
    }
    initial(q, out);
    for (int i = 0; i < n_hist; ++i) {
      const int idx = ((hist_it - n_hist + i) % mem + mem) % mem;
      dot(h, n3, h->w_Y[idx], out, R_A);
      mmk::k_lb_second<<<g3, BS, 0, h->st>>>(n3, d_rho + idx, d_alpha + idx, h->d_sc, R_A, h->w_S[idx], out);
      LAUNCH_CHECK();
    }
  };
  // initial Hessian of the plain L-BFGS: gamma q .* inv_M_rel, gamma = s.y / y.(y .* inv_M_rel) clipped
  auto lbfgs_initial = [&](const double* q, double* out, bool clip) {
    const int last = ((hist_it - 1) % mem + mem) % mem;
    if (hist_it > 0) {
      mmk::k_scale3_dot<<<ge, BS, 0, h->st>>>(N, h->w_Y[last], h->d_inv_M_rel, h->w_tmp, h->d_sc, h->d_part, R_B);
      LAUNCH_CHECK();
      dot(h, n3, h->w_S[last], h->w_Y[last], R_A);
    }
    mmk::k_lb_gamma<<<1, 32, 0, h->st>>>(h->d_sc, R_A, R_B, hist_it > 0 ? 1 : 0, clip ? 1 : 0, d_gamma);
    LAUNCH_CHECK();
    mmk::k_scale3_dot<<<ge, BS, 0, h->st>>>(N, q, h->d_inv_M_rel, out, h->d_sc, h->d_part, R_B);
    LAUNCH_CHECK();
    mmk::k_scale_dev<<<g3, BS, 0, h->st>>>(n3, d_gamma, out);
    LAUNCH_CHECK();
  };
  // history update at m_new: s = P(d tau), y = P(g_new) - P(g_tan_ext) (optionally replaced by `y_fix`),
  // all pairs re-projected, the new pair stored if its curvature is positive enough
  auto hist_update = [&](const double* m_new, const double* g_new, const double* dir, double tau, auto&& y_fix) {
    double* s_new = h->w_tmp;
    mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, tau, dir, 0.0, s_new);
    LAUNCH_CHECK();
    mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m_new, s_new, s_new);
    LAUNCH_CHECK();
    mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, 1.0, g_new, 0.0, h->w_r3);
    LAUNCH_CHECK();
    mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_gte, 1.0, h->w_r3);
    LAUNCH_CHECK();
    mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m_new, h->w_r3, h->w_r3);
    LAUNCH_CHECK();
    y_fix(s_new, h->w_r3);
    const double curv = dev_dot(h, n3, h->w_r3, s_new);
    const bool ok = curv > 1e-12 * dev_dot(h, n3, s_new, nullptr);
    for (int i = 0; i < mem; ++i) {
      mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m_new, h->w_S[i], h->w_S[i]);
      LAUNCH_CHECK();
      mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m_new, h->w_Y[i], h->w_Y[i]);
      LAUNCH_CHECK();
    }
    if (ok) {
      const int idx = hist_it % mem;
      copy3(h->w_S[idx], s_new);
      copy3(h->w_Y[idx], h->w_r3);
      rho_h[idx] = 1.0 / (curv + 1e-30);
      if (!d_rho) throw Fail{MM_ERR_STATE, "L-BFGS history without its device scalars"};
      mmk::k_set_value<<<1, 32, 0, h->st>>>(d_rho + idx, rho_h[idx]);
      LAUNCH_CHECK();
      ++hist_it;
    }
  };
  auto no_fix = [](double*, double*) {};
  // d = -y + beta * (P_m) d_prev with the descent safeguard (d = -y when d.g_tan_ext > 0); returns g_raw.d
  auto direction = [&](const double* y, const double* dprev, double beta, int proj) {
    mmk::k_direction<<<ge, BS, 0, h->st>>>(N, m, y, dprev, beta, h->w_gte, graw, h->w_d, h->d_sc, h->d_part, proj);
    LAUNCH_CHECK();
    const double* ab = h->red_n(R_A, 2);
    const double dg = ab[0];
    double pg = ab[1];
    if (dg > 0) {
      neg3(h->w_d, y);
      pg = dev_dot(h, n3, graw, h->w_d);
    }
    return pg;
  };
  // d = -a, replaced by -fallback when not a descent direction; returns g_raw.d
  auto descent_or = [&](const double* a, const double* fallback) {
    neg3(h->w_d, a);
    if (dev_dot(h, n3, h->w_d, h->w_gte) > 0) neg3(h->w_d, fallback);
    return dev_dot(h, n3, graw, h->w_d);
  };
  auto pc_tol_of = [&](double gn) {
    return prm->pc_auto ? std::min(prm->pc_force_eta, std::pow(gn, prm->pc_force_alpha)) : 0.0;
  };
  // trust-region trial R(m, m x d, 1), ratio test, radius update, acceptance (src/minimizers.py:2036-2090)
  auto tr_finish = [&](double pred, double gnorm_inf, int pc_it, int demag_inner) {
    mmk::k_cross<<<ge, BS, 0, h->st>>>(N, m, h->w_d, h->w_H);
    LAUNCH_CHECK();
    mmk::k_cayley<<<ge, BS, 0, h->st>>>(N, m, h->w_H, 1.0, h->w_mt);
    LAUNCH_CHECK();
    CK(cudaMemcpyAsync(h->w_Ut, U, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    const int itd = demag_solve(c, h->w_mt, h->w_Ut, c.phi_tol);
    double E_t = eval(c, h->w_mt, h->w_Ut, h->w_gt_trial);
    if (!std::isfinite(E_t)) E_t = 1e20;
    const double rho_tr = (E - E_t) / (pred + 1e-30);
    const double dnorm = std::sqrt(dev_dot(h, n3, h->w_d, nullptr));
    const double delta_next = rho_tr < 0.25 ? 0.25 * delta
                              : (rho_tr > 0.75 && dnorm >= 0.9 * delta) ? std::min(2.0 * delta, 100.0)
                                                                        : delta;
    const bool accept = rho_tr > 0.01;
    double dm = 0.0;
    if (accept) {
      mmk::k_absmaxdiff<<<g3, BS, 0, h->st>>>(n3, h->w_mt, m, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      dm = h->red(R_MAX);
    }
    const double E_next = accept ? E_t : E;
    conv = check_conv(it, E_next, E, dm, gnorm_inf, prm);
    if (accept) accept_trial(h, m, U, graw);
    delta = delta_next;
    c.evals += 1;
    c.preco += pc_it;
    c.demag += demag_inner + itd;
    E = E_next;
    gnorm = gnorm_inf;
    ++it;
  };

  // C++ conventions: an inner solve on the initial state (its count goes into preco_iters; y_prev and
  // d_prev = -y_prev are unused by the first step, cpp_mkl_minimizer.cpp:606-617), and the energy test
  // of the convergence check against E_lag, the energy before the previous step (:620,723-726)
  double E_lag = E;
  if (cpp) {
    c.preco += solve_Py_g(c, m, graw, h->w_gte, pc_tol_of(gnorm), h->w_ys, prm->pc_reg);
    neg3(h->w_dprev, h->w_ys);
  }
  // pcohen_hs / pcohen / pcg: the iterations as one device graph where it can be built
  const bool on_device = cg_family && minimize_graph(h, c, m, U, E, cpp, &it, &E, &gnorm, &conv);
  while (!on_device && !conv && it < prm->max_iter) {
    const double E_prev = E;
    mmk::k_tangent2<<<ge, BS, 0, h->st>>>(N, m, graw, h->d_inv_M_rel, h->w_gt, h->w_gte, h->d_sc, h->d_part);
    LAUNCH_CHECK();
    const double gnorm_inf = h->red(R_MAX);
    double conv_gnorm = gnorm_inf;
    double pg = 0.0, s0 = 1.0;
    double* H = h->w_H;
    gnorm = gnorm_inf;
    if (cg_family) {
      // preconditioned CG: HS beta (pcohen_hs, pcg) or PR beta (pcohen); pcg keeps d_prev unprojected
      c.preco += solve_Py_g(c, m, graw, h->w_gte, pc_tol_of(gnorm_inf), h->w_y, prm->pc_reg);
      // max|y| (R_MAX) and the two HS sums (R_A, R_B) read with one copy and one wait
      mmk::k_absmax<<<grid_vec(n3), BS, 0, h->st>>>(n3, h->w_y, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      mmk::k_dot2diff<<<g3, BS, 0, h->st>>>(n3, h->w_y, h->w_dprev, h->w_gte, h->w_gprev, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      const double* mab = h->red_n(R_MAX, 3);
      const double gsm = mab[0];
      const double num = mab[1];
      const double den = (meth == MM_METHOD_PCOHEN ? dev_dot(h, n3, h->w_ys, h->w_gprev) : mab[2]) + 1e-30;
      const double beta = (it % L == 0) ? 0.0 : std::max(0.0, num / den);
      pg = direction(h->w_y, h->w_dprev, beta, meth == MM_METHOD_PCG ? 0 : 1);
      conv_gnorm = gnorm = gsm;
    } else if (meth == MM_METHOD_COHEN) {
      // Cohen CG (src/minimizers.py:646-720): y = g_tan, PR beta, energy-based initial step
      mmk::k_dot2diff<<<g3, BS, 0, h->st>>>(n3, h->w_gt, h->w_gt, h->w_gte, h->w_gprev, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      const double num = h->red(R_A);
      const double den = dev_dot(h, n3, h->w_ys, h->w_gprev) + 1e-30;
      const double beta = (it % L == 0) ? 0.0 : std::max(0.0, num / den);
      pg = direction(h->w_gt, h->w_dprev, beta, 1);
      double tau_a = 2.0 * (E - E_last) / (-pg + 1e-30);
      tau_a = std::min(1.0, 1.01 * std::fabs(tau_a));
      tau_a = std::min(std::max(tau_a, 1e-4), 10.0);
      s0 = it > 0 ? tau_a : prm->tau0;
    } else if (exact) {
      // Cohen CG with Cayley transport of d_prev and g_prev (src/minimizers.py:1093-1200)
      c.preco += solve_Py_g(c, m, graw, h->w_gte, pc_tol_of(gnorm_inf), h->w_y, prm->pc_reg);
      const double gsm = dev_absmax(h, n3, h->w_y);
      if (it > 0) {
        mmk::k_transport<<<ge, BS, 0, h->st>>>(N, h->w_dprev, h->w_x1, tau_prev, h->w_x2);
        LAUNCH_CHECK();
        mmk::k_transport<<<ge, BS, 0, h->st>>>(N, h->w_gprev, h->w_x1, tau_prev, h->w_x3);
        LAUNCH_CHECK();
      } else {
        zero3(h->w_x2);
        zero3(h->w_x3);
      }
      mmk::k_dot2diff<<<g3, BS, 0, h->st>>>(n3, h->w_y, h->w_x2, h->w_gte, h->w_x3, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      const double* ab = h->red_n(R_A, 2);
      const double num = ab[0];
      const double den = (meth == MM_METHOD_PCOHEN_HS_EXACT ? ab[1] : dev_dot(h, n3, h->w_ys, h->w_x3)) + 1e-30;
      const double beta = (it % L == 0) ? 0.0 : std::max(0.0, num / den);
      pg = direction(h->w_y, h->w_x2, beta, 0);
      conv_gnorm = gnorm = gsm;
    } else if (meth == MM_METHOD_TN_SPLIT) {
      // split truncated Newton: the Steihaug solve of P d = -g_tan_ext is the step (src/minimizers.py:1448-1517)
      neg3(h->w_tmp, h->w_gte);
      c.preco += solve_Py_g(c, m, graw, h->w_tmp, pc_tol_of(gnorm_inf), h->w_d, prm->pc_reg);
      pg = dev_dot(h, n3, graw, h->w_d);
      s0 = (it == 0) ? prm->tau0 : 1.0;
    } else if (meth == MM_METHOD_PLBFGS || meth == MM_METHOD_DPLBFGS) {
      // preconditioned L-BFGS (src/minimizers.py:1526-1653; damped variant :1820-1968): smoothed gradient
      // y = P^-1 g_tan_ext for the convergence test and the fallback, P^-1 as the initial Hessian
      solve_Py_g(c, m, graw, h->w_gte, 0.0, h->w_ys, 0.0);
      const double gsm = dev_absmax(h, n3, h->w_ys);
      two_loop(h->w_d, [&](const double* q, double* out) { solve_Py_g(c, m, graw, q, 0.0, out, prm->pc_reg); });
      mmk::k_scale<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_d);
      LAUNCH_CHECK();
      if (it == 0 || dev_dot(h, n3, h->w_d, h->w_gte) > 0) neg3(h->w_d, h->w_ys);
      pg = dev_dot(h, n3, graw, h->w_d);
      s0 = (it == 0) ? prm->tau0 : 1.0;
      conv_gnorm = gnorm = gsm;
      c.preco += meth == MM_METHOD_DPLBFGS ? 2 : 1;
    } else if (meth == MM_METHOD_LBFGS) {
      // two-loop recursion on g_tan_ext (src/minimizers.py:1284-1312)
      two_loop(h->w_d, [&](const double* q, double* out) { lbfgs_initial(q, out, true); });
      mmk::k_scale<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_d);
      LAUNCH_CHECK();
      if (it == 0 || dev_dot(h, n3, h->w_d, h->w_gte) > 0) neg3(h->w_d, h->w_gt);
      pg = dev_dot(h, n3, graw, h->w_d);
      s0 = (it == 0) ? prm->tau0 : 1.0;
    } else if (meth == MM_METHOD_PCOHEN_LBFGS) {
      // Cohen CG (PR beta) over the L-BFGS-smoothed gradient z (src/minimizers.py:2816-2924)
      two_loop(h->w_ys, [&](const double* q, double* out) { lbfgs_initial(q, out, false); });
      const double gsm = dev_absmax(h, n3, h->w_ys);
      mmk::k_dot2diff<<<g3, BS, 0, h->st>>>(n3, h->w_ys, h->w_ys, h->w_gte, h->w_gprev, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      const double num = h->red(R_A);
      const double den = dev_dot(h, n3, h->w_gprev, h->w_x1) + 1e-30;
      const double beta = (it % L == 0) ? 0.0 : std::max(0.0, num / den);
      pg = direction(h->w_ys, h->w_dprev, beta, 1);
      conv_gnorm = gnorm = gsm;
    } else if (meth == MM_METHOD_AAPG || meth == MM_METHOD_AAPG_EXACT) {
      // Anderson acceleration of depth one over the previous smoothed gradient (src/minimizers.py:2519-2636),
      // moved by Cayley transport in the exact variant (:2407-2504)
      c.preco += solve_Py_g(c, m, graw, h->w_gte, pc_tol_of(gnorm_inf), h->w_y, prm->pc_reg);
      const double* F_prev = h->w_x1;
      if (meth == MM_METHOD_AAPG_EXACT && it > 0) {
        mmk::k_transport<<<ge, BS, 0, h->st>>>(N, h->w_x1, h->w_x2, tau_prev, h->w_x3);
        LAUNCH_CHECK();
        F_prev = h->w_x3;
      }
      // z_next (w_ys) = z - gamma (z - F_prev) from the third step on, else z
      copy3(h->w_ys, h->w_y);
      if (it > 1 || meth == MM_METHOD_AAPG_EXACT) {
        copy3(h->w_tmp, h->w_y);
        mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, F_prev, 1.0, h->w_tmp);
        LAUNCH_CHECK();
        const double gamma = dev_dot(h, n3, h->w_y, h->w_tmp) / (dev_dot(h, n3, h->w_tmp, nullptr) + 1e-30);
        if (it > 1) {
          mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -gamma, h->w_tmp, 1.0, h->w_ys);
          LAUNCH_CHECK();
        }
      }
      pg = descent_or(h->w_ys, h->w_y);
      conv_gnorm = gnorm = dev_absmax(h, n3, meth == MM_METHOD_AAPG ? h->w_y : h->w_ys);
    } else if (meth == MM_METHOD_PNAG) {
      // Nesterov look-ahead m_look = R(m, -(m x v), mu), smoothed gradient there (src/minimizers.py:2726-2803)
      const double mu = prm->mu;
      mmk::k_cross<<<ge, BS, 0, h->st>>>(N, m, h->w_x4, h->w_x1);
      LAUNCH_CHECK();
      mmk::k_cayley<<<ge, BS, 0, h->st>>>(N, m, h->w_x1, -mu, h->w_x2);
      LAUNCH_CHECK();
      CK(cudaMemcpyAsync(h->w_U2, U, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
      if (prm->phi_extrapolate && it > 0) {
        mmk::k_axpby<<<ge, BS, 0, h->st>>>(N, -1.0, h->w_U3, 2.0, h->w_U2);
        LAUNCH_CHECK();
      }
      c.demag += demag_solve(c, h->w_x2, h->w_U2, c.phi_tol);
      eval(c, h->w_x2, h->w_U2, h->w_x3);
      c.evals += 1;
      mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, h->w_x2, h->w_x3, h->w_tmp);
      LAUNCH_CHECK();
      c.preco += solve_Py_g(c, h->w_x2, h->w_x3, h->w_tmp, 0.0, h->w_y, prm->pc_reg);
      conv_gnorm = gnorm = dev_absmax(h, n3, h->w_y);
      // v_dir = mu P_m(v) - P_m(z)
      mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m, h->w_x4, h->w_d);
      LAUNCH_CHECK();
      mmk::k_tangent<<<ge, BS, 0, h->st>>>(N, m, h->w_y, h->w_tmp);
      LAUNCH_CHECK();
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_tmp, mu, h->w_d);
      LAUNCH_CHECK();
      pg = dev_dot(h, n3, graw, h->w_d);
      s0 = lr;
    } else if (meth == MM_METHOD_TR) {
      // trust-region Newton-CG on the local Hessian (src/minimizers.py:2005-2103)
      neg3(h->w_tmp, h->w_gte);
      const int pc_it = solve_Py_g_tr(c, m, graw, h->w_tmp, delta, tn_iters, pc_tol_of(gnorm_inf), prm->pc_reg,
                                      h->w_d);
      const double dPd = apply_P(c, m, graw, h->w_d, prm->pc_reg, h->w_x1);
      const double pred = -(dev_dot(h, n3, graw, h->w_d) + 0.5 * dPd);
      tr_finish(pred, gnorm_inf, pc_it, 0);
      continue;
    } else if (meth == MM_METHOD_PTR) {
      // preconditioned Steihaug CG on the full Hessian; each product solves the Poisson problem of the
      // direction (src/minimizers.py:2140-2320).  The inner solves use the default stagnation 1e-3.
      const double pc_tol = pc_tol_of(gnorm_inf);
      const double zero_B[3] = {0.0, 0.0, 0.0};
      const double d2 = delta * delta;
      double *d = h->w_d, *r = h->w_x1, *z = h->w_x2, *p = h->w_x3, *Hp = h->w_x4;
      zero3(d);
      copy3(r, h->w_gte);
      int pc_acc = solve_Py_g(c, m, graw, r, pc_tol, z, prm->pc_reg, -1, 1e-3);
      neg3(p, z);
      double rho = dev_dot(h, n3, r, z);
      double q = 0.0;
      CK(cudaMemsetAsync(h->w_U3, 0, N * sizeof(double), h->st));
      int i = 0, dem = 0;
      bool done = false;
      while (i < tn_iters && !done && rho > 0.0) {
        CK(cudaMemcpyAsync(h->w_U2, h->w_U3, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
        const int itd = demag_solve(c, p, h->w_U2, c.phi_tol);
        energy_dev(h, p, h->w_U2, zero_B, h->d_min_bias, h->w_tmp);
        mmk::k_hess_full<<<ge, BS, 0, h->st>>>(N, m, graw, p, h->w_tmp, Hp, h->d_sc, h->d_part);
        LAUNCH_CHECK();
        const double kappa = h->red(R_C);
        const double alpha = rho / (kappa + 1e-30);
        const auto pp_dp = dev_mdot2(h, p, p, d, p);
        const double dd = dev_mdot2(h, d, d, d, d).first;
        const double alpha_tr = tr_boundary_step(pp_dp.first + 1e-30, 2.0 * pp_dp.second, dd - d2);
        const bool done_now = (kappa <= 0.0) || (dev_mnorm_axpy(h, d, alpha, p) >= d2);
        const double af = done_now ? alpha_tr : alpha;
        q = q + af * dev_dot(h, n3, r, p) + 0.5 * af * af * kappa;
        mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, af, p, 1.0, d);
        LAUNCH_CHECK();
        mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, alpha, Hp, 1.0, r);
        LAUNCH_CHECK();
        const int pc_it = solve_Py_g(c, m, graw, r, pc_tol, z, prm->pc_reg, -1, 1e-3);
        const double rho_next = dev_dot(h, n3, r, z);
        const double beta = rho_next / (rho + 1e-30);
        mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, z, beta, p);
        LAUNCH_CHECK();
        mmk::k_axpby<<<ge, BS, 0, h->st>>>(N, beta, h->w_U2, 0.0, h->w_U3);
        LAUNCH_CHECK();
        done = done || done_now || rho_next < 1e-8 || rho <= 0.0;
        rho = rho_next;
        pc_acc += pc_it;
        dem += itd;
        ++i;
      }
      tr_finish(-q, gnorm_inf, pc_acc, dem);
      continue;
    } else {  // wg_np: Barzilai-Borwein (src/minimizers.py:1715-1798)
      // s = m - m_prev ; y = g_tan - g_tan_prev
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, 1.0, m, 0.0, h->w_tmp);
      LAUNCH_CHECK();
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_mprev, 1.0, h->w_tmp);
      LAUNCH_CHECK();
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, 1.0, h->w_gt, 0.0, h->w_y);
      LAUNCH_CHECK();
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, -1.0, h->w_gtprev, 1.0, h->w_y);
      LAUNCH_CHECK();
      const double sty = dev_dot(h, n3, h->w_tmp, h->w_y);
      const double sts = dev_dot(h, n3, h->w_tmp, nullptr);
      const double yty = dev_dot(h, n3, h->w_y, nullptr);
      const double tau1 = sts / (sty + 1e-30), tau2 = sty / (yty + 1e-30);
      double tau_bb = (it % 2 != 0) ? tau1 : tau2;
      tau_bb = std::min(std::max(std::fabs(tau_bb), 1e-6), 1e3);
      // d = -g_tan so that H = m x d = -(m x z) and pg = g_raw . d
      neg3(h->w_d, h->w_gt);
      pg = dev_dot(h, n3, graw, h->w_d);
      if (it >= prm->wg_gamma) {
        mmk::k_cross<<<ge, BS, 0, h->st>>>(N, m, h->w_d, H);
        LAUNCH_CHECK();
        mmk::k_cayley<<<ge, BS, 0, h->st>>>(N, m, H, tau_bb, h->w_mt);
        LAUNCH_CHECK();
        CK(cudaMemcpyAsync(h->w_Ut, U, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
        c.demag += demag_solve(c, h->w_mt, h->w_Ut, c.phi_tol);
        const double E_new = eval(c, h->w_mt, h->w_Ut, h->w_gt_trial);
        c.evals += 1;
        mmk::k_absmaxdiff<<<g3, BS, 0, h->st>>>(n3, h->w_mt, m, h->d_sc, h->d_part);
        LAUNCH_CHECK();
        const double dm = h->red(R_MAX);
        conv = check_conv(it, E_new, E_prev, dm, gnorm_inf, prm);
        copy3(h->w_mprev, m);
        copy3(h->w_gtprev, h->w_gt);
        accept_trial(h, m, U, graw);
        E = E_new;
        ++it;
        continue;
      }
    }
    mmk::k_cross<<<ge, BS, 0, h->st>>>(N, m, h->w_d, H);
    LAUNCH_CHECK();
    LSResult ls = armijo(c, m, pg, H, E_prev, U, s0);
    c.evals += ls.evals;
    c.demag += ls.demag;
    const double tau = ls.accepted ? ls.tau : 0.0;
    if (meth == MM_METHOD_DPLBFGS && !ls.accepted) {
      // m_new = R(m, H, tau) is recomputed by the reference: at tau = 0 that renormalises m
      mmk::k_cayley<<<ge, BS, 0, h->st>>>(N, m, H, 0.0, h->w_mt);
      LAUNCH_CHECK();
    }
    const bool m_moves = ls.accepted || meth == MM_METHOD_DPLBFGS;
    double dm = 0.0;
    if (m_moves) {
      mmk::k_absmaxdiff<<<g3, BS, 0, h->st>>>(n3, h->w_mt, m, h->d_sc, h->d_part);
      LAUNCH_CHECK();
      dm = h->red(R_MAX);
    }
    const double E_new = ls.accepted ? ls.E : E_prev;
    conv = check_conv(it, E_new, cpp ? E_lag : E_prev, dm, conv_gnorm, prm);
    E_lag = E_prev;
    if (lbfgs) {
      const double* m_new = m_moves ? h->w_mt : m;
      const double* g_new = ls.accepted ? h->w_gt_trial : graw;
      if (meth == MM_METHOD_DPLBFGS) {
        // Powell damping against B0 s = P(m_new, g_new) s (src/minimizers.py:1926-1941)
        hist_update(m_new, g_new, h->w_d, tau, [&](const double* s_k, double* y_k) {
          const double sBs = apply_P(c, m_new, g_new, s_k, 0.0, h->w_x1);
          const double sy = dev_dot(h, n3, s_k, y_k);
          const double theta = sy >= 0.2 * sBs ? 1.0 : 0.8 * sBs / (sBs - sy + 1e-30);
          mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, 1.0 - theta, h->w_x1, theta, y_k);
          LAUNCH_CHECK();
        });
      } else {
        hist_update(m_new, g_new, h->w_d, tau, no_fix);
      }
    }
    if (cg_family || meth == MM_METHOD_COHEN || exact || meth == MM_METHOD_PCOHEN_LBFGS) {
      std::swap(h->w_gprev, h->w_gte);  // g_prev <- g_tan_ext
      std::swap(h->w_dprev, h->w_d);    // d_prev <- d
    }
    if (meth == MM_METHOD_PCOHEN || exact) std::swap(h->w_ys, h->w_y);  // y_prev / z_prev <- y / z
    if (meth == MM_METHOD_COHEN) {
      std::swap(h->w_ys, h->w_gt);  // y_prev <- g_tan
      E_last = E_prev;
    }
    if (meth == MM_METHOD_PCOHEN_LBFGS) copy3(h->w_x1, h->w_ys);  // z_prev <- z
    if (exact) {
      copy3(h->w_x1, H);  // H_prev
      tau_prev = tau;
    }
    if (meth == MM_METHOD_AAPG || meth == MM_METHOD_AAPG_EXACT) {
      copy3(h->w_x1, h->w_y);  // F_prev <- z
      if (meth == MM_METHOD_AAPG_EXACT) copy3(h->w_x2, H);
      tau_prev = tau;
    }
    if (meth == MM_METHOD_PNAG) {
      mmk::k_axpby<<<g3, BS, 0, h->st>>>(n3, tau, h->w_d, 0.0, h->w_x4);  // v <- tau v_dir
      LAUNCH_CHECK();
      CK(cudaMemcpyAsync(h->w_U3, U, N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));  // U_prev <- U
    }
    if (meth == MM_METHOD_WG_NP) {
      copy3(h->w_mprev, m);
      copy3(h->w_gtprev, h->w_gt);
    }
    if (ls.accepted) {
      accept_trial(h, m, U, graw);
    } else if (meth == MM_METHOD_DPLBFGS) {
      std::swap(m, h->w_mt);
    }
    E = E_new;
    ++it;
  }
  h->w_graw = graw;
  h->sync();
  auto t1 = std::chrono::steady_clock::now();
  if (info) {
    info->iters = it;
    info->evals = c.evals;
    info->preco_iters = c.preco;
    info->demag_iters = c.demag;
    info->E = E;
    info->gnorm = gnorm;
    info->seconds = std::chrono::duration<double>(t1 - t0).count();
    info->status = (it >= prm->max_iter && !conv) ? MM_MAXITER : MM_OK;
    info->demag_seconds = 1e-3 * c.demag_ms;
    info->demag_wall_seconds = c.demag_wall;
    info->device_loop = on_device ? 1 : 0;
  }
  return std::isfinite(E) ? MM_OK : MM_NONFINITE;
}

}  // namespace

// =============================================================================================
// allocation-free energy + gradient (see mm_energy_grad_noalloc in include/mumag_cuda.h)
// =============================================================================================
namespace {

constexpr int NOALLOC_TPR = 8;                                   // lanes per magnetic row
constexpr int NOALLOC_RPB = BS / NOALLOC_TPR;                    // rows per block (32)
constexpr int NOALLOC_MAX_BLOCKS = MM_NOALLOC_MAX_ROWS / NOALLOC_RPB;
// layout: [0, MAX_BLOCKS) block partials | total | ticket counter (as unsigned) | padding
constexpr int NOALLOC_WORDS = NOALLOC_MAX_BLOCKS + 32;
static_assert(NOALLOC_WORDS * sizeof(double) == MM_NOALLOC_SCRATCH_BYTES, "scratch size");

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_WORDS];

// One block per 32 magnetic rows (no grid-stride loop, so the block count follows the row count).
__global__ void __launch_bounds__(BS) k_energy_grad_noalloc(mmk::EnergyDev op, const double* __restrict__ m,
                                                            const double* __restrict__ U,
                                                            const double* __restrict__ Mn, double Bx, double By,
                                                            double Bz, const double* __restrict__ Bbias,
                                                            double inv_Vmag, double* __restrict__ g,
                                                            double* scratch) {
  constexpr int TPR = NOALLOC_TPR;
  const int lane = threadIdx.x % TPR;
  const int r = blockIdx.x * NOALLOC_RPB + threadIdx.x / TPR;
  const bool valid = r < op.n_rows;
  double ax, ay, az;
  mmk::exch_aniso_row<TPR>(op, r, valid, lane, m, ax, ay, az);
  double ux = 0, uy = 0, uz = 0;
  if (valid) {
    const int s = op.ptr[r], e = op.ptr[r + 1];
    for (int k = s + lane; k < e; k += TPR) {
      const double u = __ldg(U + op.col[k]);
      ux += op.gx[k] * u;
      uy += op.gy[k] * u;
      uz += op.gz[k] * u;
    }
  }
  ux = mmk::group_sum<TPR>(ux);
  uy = mmk::group_sum<TPR>(uy);
  uz = mmk::group_sum<TPR>(uz);
  double en = 0.0;
  if (valid && lane == 0) {
    const int a = op.rows[r];
    double bx = Bx, by = By, bz = Bz;
    if (Bbias) {
      bx += Bbias[3 * a];
      by += Bbias[3 * a + 1];
      bz += Bbias[3 * a + 2];
    }
    const double mn = -2.0 * Mn[a];
    const double zx = mn * bx, zy = mn * by, zz = mn * bz;
    const double gx = (ax + ux) + zx, gy = (ay + uy) + zy, gz = (az + uz) + zz;
    en = m[3 * a] * (gx + zx) + m[3 * a + 1] * (gy + zy) + m[3 * a + 2] * (gz + zz);
    g[3 * a] = gx * inv_Vmag;
    g[3 * a + 1] = gy * inv_Vmag;
    g[3 * a + 2] = gz * inv_Vmag;
  }
  // deterministic reduction: partials in block order, summed by the last block to arrive
  __shared__ unsigned s_last;
  en = mmk::block_sum(en);
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch + NOALLOC_MAX_BLOCKS + 1);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = en;
    __threadfence();
    s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += BS) t += __ldcg(scratch + i);
    t = mmk::block_sum(t);
    if (threadIdx.x == 0) {
      scratch[NOALLOC_MAX_BLOCKS] = t;
      *ticket = 0u;
    }
  }
}

// Device address of g_noalloc_scratch for the current device, looked up once per device (the entry
// point makes the problem's device current first, see guarded()).
double* noalloc_scratch_for_current_device() {
  static std::mutex mu;
  static double* addr[256] = {};
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw Fail{MM_ERR_CUDA, "device ordinal out of range"};
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    addr[dev] = static_cast<double*>(p);
  }
  return addr[dev];
}

}  // namespace

extern "C" int mm_energy_grad_noalloc(mm_problem* h, const double* d_m, const double* d_U, const double* B,
                                      const double* d_bias, double* E, double* d_g) {
  if (!h || !d_m || !d_U || !B || !E || !d_g) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (h->eop.n_rows > MM_NOALLOC_MAX_ROWS)
      throw Fail{MM_ERR_ARG, "mm_energy_grad_noalloc: " + std::to_string(h->eop.n_rows) +
                                 " magnetic rows exceed MM_NOALLOC_MAX_ROWS (" +
                                 std::to_string(MM_NOALLOC_MAX_ROWS) + "); use mm_energy_grad_dev"};
    double* scratch = noalloc_scratch_for_current_device();
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + NOALLOC_MAX_BLOCKS + 1);
    CK(cudaMemsetAsync(ticket, 0, sizeof(unsigned), h->st));                  // must start at zero
    CK(cudaMemsetAsync(scratch + NOALLOC_MAX_BLOCKS, 0, sizeof(double), h->st));  // total (empty mesh)
    CK(cudaMemsetAsync(d_g, 0, 3 * (size_t)h->N * sizeof(double), h->st));
    const int blocks = (h->eop.n_rows + NOALLOC_RPB - 1) / NOALLOC_RPB;
    if (blocks > 0) {
      k_energy_grad_noalloc<<<blocks, BS, 0, h->st>>>(h->eop, d_m, d_U, h->d_Mn, B[0], B[1], B[2], d_bias,
                                                      h->inv_Vmag, d_g, scratch);
      LAUNCH_CHECK();
    }
    double total = 0.0;
    CK(cudaMemcpyAsync(&total, scratch + NOALLOC_MAX_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    *E = 0.5 * total * h->inv_Vmag;
    return std::isfinite(*E) ? MM_OK : MM_NONFINITE;
  });
}

// Factored form of the V-cycle's two coarsest levels, formed in FP64 on the host.  With S the smoother
// diagonal, A, P, R the operators of level L-2 and Ainv the dense inverse of level L-1, the levels
// L-2 .. L-1 map the restricted residual b to the post-smoothed iterate
//   x2 = (I - S A) (S + P Ainv R (I - A S)) b + S b = T b + W (Z b),
//   T = 2S - S A S (A's pattern), W = (I - S A) P (n x nc), Z = Ainv R (I - A S) (nc x n).
// The host factors T, W, Z in FP64 (fc.ok false when a row of A has no stored diagonal).
void form_fused_coarse(mm_problem* h, int precond_type, mm_problem::FusedCoarseHost& fc) {
  const int L = (int)h->amg_h.size();
  const mm::AmgLevel& a = h->amg_h[L - 2];
  const mm::HostCSR &A = a.A, &P = a.P, &R = a.R;
  const int n = A.n_rows, nc = h->amg_h[L - 1].A.n_rows;
  fc = mm_problem::FusedCoarseHost{};
  std::vector<double> sd(n);
  for (int i = 0; i < n; ++i) sd[i] = precond_type == MM_PRECOND_AMGCL ? a.spai0[i] : 0.6667 / (a.diag[i] + 1e-30);
  std::vector<double> tv(A.nnz());
  for (int i = 0; i < n; ++i) {
    bool diag = false;
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
      const int j = A.col[k];
      tv[k] = -sd[i] * A.val[k] * sd[j] + (j == i ? 2.0 * sd[i] : 0.0);
      diag = diag || j == i;
    }
    if (!diag) return;  // a row without a stored diagonal: keep the five-kernel path
  }
  std::vector<double> Wd((size_t)n * nc, 0.0), AP((size_t)n * nc, 0.0);
  for (int i = 0; i < n; ++i)
    for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
      for (int q = P.ptr[A.col[k]]; q < P.ptr[A.col[k] + 1]; ++q) AP[(size_t)i * nc + P.col[q]] += A.val[k] * P.val[q];
  for (int i = 0; i < n; ++i) {
    for (int q = P.ptr[i]; q < P.ptr[i + 1]; ++q) Wd[(size_t)i * nc + P.col[q]] += P.val[q];
    for (int j = 0; j < nc; ++j) Wd[(size_t)i * nc + j] -= sd[i] * AP[(size_t)i * nc + j];
  }
  std::vector<double> M((size_t)nc * n, 0.0);  // R (I - A S)
  for (int r = 0; r < nc; ++r)
    for (int k = R.ptr[r]; k < R.ptr[r + 1]; ++k) {
      M[(size_t)r * n + R.col[k]] += R.val[k];
      const int row = R.col[k];
      for (int q = A.ptr[row]; q < A.ptr[row + 1]; ++q) M[(size_t)r * n + A.col[q]] -= R.val[k] * A.val[q] * sd[A.col[q]];
    }
  const std::vector<double>& Ainv = h->coarse_inverse();
  std::vector<double> Zd((size_t)nc * n, 0.0);
  for (int r = 0; r < nc; ++r)
    for (int q = 0; q < nc; ++q) {
      const double c = Ainv[(size_t)r * nc + q];
      const double* mq = &M[(size_t)q * n];
      double* zr = &Zd[(size_t)r * n];
      for (int j = 0; j < n; ++j) zr[j] += c * mq[j];
    }
  fc.tv = std::move(tv);
  fc.W = std::move(Wd);
  fc.Z = std::move(Zd);
  fc.ok = true;
}

template <class T>
void build_fused_coarse(mm_problem* h, SolverT<T>& S, int precond_type) {
  if (h->fc_prec != precond_type) {
    form_fused_coarse(h, precond_type, h->fc_host);
    h->fc_prec = precond_type;
  }
  const mm_problem::FusedCoarseHost& fc = h->fc_host;
  if (!fc.ok) return;
  const int L = (int)h->amg_h.size();
  const mm::HostCSR& A = h->amg_h[L - 2].A;
  const int n = A.n_rows, nc = h->amg_h[L - 1].A.n_rows;
  S.Tm.n = n;
  S.Tm.ptr = h->upload(A.ptr);
  S.Tm.col = h->upload(A.col);
  S.Tm.val = h->upload_as<T>(fc.tv);
  S.Tm_nnz = A.nnz();
  S.W = h->upload_as<T>(fc.W);
  S.Z = h->upload_as<T>(fc.Z);
  S.tvec = h->alloc<T>(n);
  S.zvec = h->alloc<T>(nc);
  S.fn = n;
  S.fc = nc;
  S.fused = true;
}

// Upload the hierarchy in precision T and allocate the solver's vectors.
template <class T>
void build_solver(mm_problem* h, SolverT<T>& S, const mm::HostCSR& A, bool amg, int precond_type) {
  const int L = (int)h->amg_h.size();
  S.lv.resize(L);
  for (int l = 0; l < L; ++l) {
    const mm::AmgLevel& hl = h->amg_h[l];
    auto& dl = S.lv[l];
    dl.n = hl.A.n_rows;
    dl.A = h->upload_mat<T>(hl.A, l == 0);  // level 0 feeds the fused PCG kernels: always sliced ELL
    if (l < L - 1) {
      dl.P = h->upload_mat<T>(hl.P);
      dl.R = h->upload_mat<T>(hl.R);
    }
    if (amg) {
      std::vector<double> sd(dl.n);
      for (int i = 0; i < dl.n; ++i)
        sd[i] = precond_type == MM_PRECOND_AMGCL ? hl.spai0[i] : 0.6667 / (hl.diag[i] + 1e-30);
      dl.s = h->upload_as<T>(sd);
    }
    dl.b = h->alloc<T>(dl.n);
    dl.x = h->alloc<T>(dl.n);
    dl.x2 = h->alloc<T>(dl.n);
    dl.res = h->alloc<T>(dl.n);
  }
  if (amg && L >= 2) {
    // fused restrictions R_l (I - A_l S_l) with the smoother of this hierarchy, formed once in FP64
    if ((int)h->rf_host.size() != L - 1 || h->rf_prec != precond_type) {
      h->rf_host.assign(L - 1, mm::HostCSR{});
      for (int l = 0; l < L - 1; ++l) {
        const mm::AmgLevel& hl = h->amg_h[l];
        std::vector<double> sd(hl.A.n_rows);
        for (int i = 0; i < hl.A.n_rows; ++i)
          sd[i] = precond_type == MM_PRECOND_AMGCL ? hl.spai0[i] : 0.6667 / (hl.diag[i] + 1e-30);
        // from R A when the setup kept it (no second sparse product), else from R and A
        h->rf_host[l] = hl.RA.ptr.empty() ? mm::fused_restriction(hl.R, hl.A, sd)
                                          : mm::fused_restriction_ra(hl.R, hl.RA, sd);
      }
      h->rf_prec = precond_type;
      for (mm::AmgLevel& hl : h->amg_h) hl.RA = mm::HostCSR{};  // its one use is above
    }
    for (int l = 0; l < L - 1; ++l) S.lv[l].Rf = h->upload_mat<T>(h->rf_host[l]);
  }
  if (amg) {
    const mm::HostCSR& Ac = h->amg_h.back().A;
    S.n_coarse = Ac.n_rows;
    S.Ainv = h->upload_as<T>(h->coarse_inverse());
  } else {
    std::vector<double> jac(h->N, 1.0), dg(h->N, 0.0);
    for (int r = 0; r < A.n_rows; ++r)
      for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
        if (A.col[k] == r) dg[r] = A.val[k];
    for (int i = 0; i < h->N; ++i) jac[i] = 1.0 / (dg[i] + 1e-30);
    S.jac = h->upload_as<T>(jac);
  }
  S.r = h->alloc<T>(h->N);
  S.z = h->alloc<T>(h->N);
  S.p = h->alloc<T>(h->N);
  S.Ap = h->alloc<T>(h->N);
  if (amg && L >= 3) {
    // only where the dense factors stay small: Z = Ainv M costs nc^2 n host FLOPs, W and Z hold n nc each
    const double n = h->amg_h[L - 2].A.n_rows, nc = h->amg_h[L - 1].A.n_rows;
    if (nc <= 256 && n * nc <= 4194304.0) build_fused_coarse<T>(h, S, precond_type);
  }
  if (amg && L == 4 && S.fused) {
    // the one-launch coarse cycle: a grid that is co-resident (the cooperative launch checks it) and
    // the barrier it synchronises on
    int coop = 0, per_sm = 0, sms = 0;
    CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mmk::k_coarse_cycle<T>, BS, 0));
    if (coop && per_sm > 0) {
      S.bar = h->alloc<mmk::GridBar>(1);
      S.coop_max = S.coop_grid = per_sm * sms;
      S.sms = sms;
    }
  }
  S.built = true;
}

// =============================================================================================
// C-ABI
// =============================================================================================
extern "C" {

const char* mm_version(void) { return "mumag_cuda 0.1 (sm_103a)"; }

const char* mm_status_str(int s) {
  switch (s) {
    case MM_OK: return "ok";
    case MM_MAXITER: return "iteration limit reached";
    case MM_NONFINITE: return "non-finite value";
    case MM_BREAKDOWN: return "breakdown";
    case MM_ERR_ARG: return "invalid argument";
    case MM_ERR_OOM: return "out of memory";
    case MM_ERR_CUDA: return "CUDA error";
    case MM_ERR_STATE: return "invalid call order";
    case MM_ERR_SETUP: return "setup failed";
    default: return "unknown status";
  }
}

const char* mm_last_error(mm_problem* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int mm_geom_compute(int N, int E, const double* knt, const int* conn_in, int* conn_out, double* volume,
                    double* JinvT, double* grad_phi) {
  if (N <= 0 || E <= 0 || !knt || !conn_in || !conn_out || !volume || !JinvT || !grad_phi) return MM_ERR_ARG;
  return guarded(nullptr, [&] {
    mm::geom_compute(N, E, knt, conn_in, conn_out, volume, JinvT, grad_phi);
    return MM_OK;
  });
}

int mm_boundary_mask(int N, int E, const int* conn, double* mask) {
  if (N <= 0 || E <= 0 || !conn || !mask) return MM_ERR_ARG;
  return guarded(nullptr, [&] {
    mm::boundary_mask(N, E, conn, mask);
    return MM_OK;
  });
}

int mm_morton_order(int N, int E, const double* knt, const int* conn, int* node_perm, int* elem_perm) {
  if (N <= 0 || E <= 0 || !knt || !conn || !node_perm || !elem_perm) return MM_ERR_ARG;
  return guarded(nullptr, [&] {
    mm::morton_order(N, E, knt, conn, node_perm, elem_perm);
    return MM_OK;
  });
}

int mm_node_degrees(int N, int E, const int* conn, int* degree) {
  if (N <= 0 || E <= 0 || !conn || !degree) return MM_ERR_ARG;
  return guarded(nullptr, [&] {
    for (int64_t k = 0; k < 4 * (int64_t)E; ++k)
      if (conn[k] < 0 || conn[k] >= N) throw Fail{MM_ERR_ARG, "connectivity index out of range"};
    std::vector<int> ptr, col;
    mm::node_graph(N, E, conn, ptr, col);
    for (int i = 0; i < N; ++i) degree[i] = ptr[i + 1] - ptr[i];
    return MM_OK;
  });
}

int mm_rcm_order(int N, int E, const int* conn, const int* seeds, int* node_perm) {
  if (N <= 0 || E <= 0 || !conn || !node_perm) return MM_ERR_ARG;
  return guarded(nullptr, [&] {
    for (int64_t k = 0; k < 4 * (int64_t)E; ++k)
      if (conn[k] < 0 || conn[k] >= N) throw Fail{MM_ERR_ARG, "connectivity index out of range"};
    std::vector<int> ptr, col;
    mm::node_graph(N, E, conn, ptr, col);
    std::vector<int> order(N);
    if (seeds) {
      std::vector<char> hit(N, 0);
      for (int i = 0; i < N; ++i) {
        if (seeds[i] < 0 || seeds[i] >= N || hit[seeds[i]]) throw Fail{MM_ERR_ARG, "seeds is not a permutation"};
        hit[seeds[i]] = 1;
        order[i] = seeds[i];
      }
    } else {
      std::iota(order.begin(), order.end(), 0);
      std::stable_sort(order.begin(), order.end(),
                       [&](int a, int b) { return ptr[a + 1] - ptr[a] < ptr[b + 1] - ptr[b]; });
    }
    mm::rcm_order(N, ptr, col, order.data(), node_perm);
    return MM_OK;
  });
}

struct mm_setup {
  mm::EnergyOp eop;
  std::vector<mm::AmgLevel> amg;
};

int mm_setup_create(int N, int E, const int* conn, const double* volume, const double* grad_phi, const int* mat_id,
                    int n_mat, const double* A_lookup, const double* K1_lookup, const double* Js_lookup,
                    const double* k_easy, const double* boundary_mask, double reg, int max_levels, int max_coarse,
                    mm_setup** out) {
  if (!out || N <= 0 || E <= 0 || n_mat <= 0 || !conn || !volume || !grad_phi || !mat_id || !A_lookup ||
      !K1_lookup || !Js_lookup || !k_easy)
    return MM_ERR_ARG;
  *out = nullptr;
  mm_setup* s = new mm_setup();
  const int rc = guarded(nullptr, [&] {
    mm::SetupScope scope;
    for (int e = 0; e < 4 * E; ++e)
      if (conn[e] < 0 || conn[e] >= N) throw Fail{MM_ERR_ARG, "connectivity index out of range"};
    s->eop = mm::assemble_energy(N, E, conn, volume, grad_phi, mat_id, n_mat, A_lookup, K1_lookup, Js_lookup, k_easy);
    if (reg >= 0) {
      mm::HostCSR A = mm::assemble_poisson(N, E, conn, volume, grad_phi, boundary_mask, reg);
      mm::AmgParams prm;
      prm.max_levels = max_levels > 0 ? max_levels : 10;
      prm.max_coarse = max_coarse > 0 ? max_coarse : 1000;
      s->amg = mm::build_amg(A, prm);
      for (mm::AmgLevel& l : s->amg) l.RA = mm::HostCSR{};
    }
    return MM_OK;
  });
  if (rc != MM_OK) {
    delete s;
    return rc;
  }
  *out = s;
  return MM_OK;
}

int mm_setup_destroy(mm_setup* s) {
  if (!s) return MM_ERR_ARG;
  delete s;
  return MM_OK;
}

int mm_setup_energy_info(mm_setup* s, int* n_rows, int64_t* nnz, int* single_axis) {
  if (!s) return MM_ERR_ARG;
  if (n_rows) *n_rows = s->eop.n_rows;
  if (nnz) *nnz = (int64_t)s->eop.col.size();
  if (single_axis) *single_axis = s->eop.single_axis ? 1 : 0;
  return MM_OK;
}

int mm_setup_energy_export(mm_setup* s, int* rows, int* ptr, int* col, int* mat, double* w, double* q, double* G,
                           double* D, double* diag_exchange) {
  if (!s) return MM_ERR_ARG;
  const mm::EnergyOp& o = s->eop;
  if (rows) std::copy(o.rows.begin(), o.rows.end(), rows);
  if (ptr) std::copy(o.ptr.begin(), o.ptr.end(), ptr);
  if (col) std::copy(o.col.begin(), o.col.end(), col);
  if (mat) std::copy(o.mat.begin(), o.mat.end(), mat);
  if (w) std::copy(o.w.begin(), o.w.end(), w);
  if (q) std::copy(o.q.begin(), o.q.end(), q);
  for (size_t k = 0; k < o.col.size(); ++k) {
    if (G) {
      G[3 * k] = o.gx[k];
      G[3 * k + 1] = o.gy[k];
      G[3 * k + 2] = o.gz[k];
    }
    if (D) {
      D[3 * k] = o.dx[k];
      D[3 * k + 1] = o.dy[k];
      D[3 * k + 2] = o.dz[k];
    }
  }
  if (diag_exchange) std::copy(o.diag_exchange.begin(), o.diag_exchange.end(), diag_exchange);
  return MM_OK;
}

int mm_setup_levels(mm_setup* s, int* n_levels) {
  if (!s || !n_levels) return MM_ERR_ARG;
  *n_levels = (int)s->amg.size();
  return MM_OK;
}

int mm_setup_level_info(mm_setup* s, int level, int* n, int64_t* nnz_A, int64_t* nnz_P, int* n_cols_P) {
  if (!s || level < 0 || level >= (int)s->amg.size()) return MM_ERR_ARG;
  const mm::AmgLevel& L = s->amg[level];
  if (n) *n = L.A.n_rows;
  if (nnz_A) *nnz_A = L.A.nnz();
  if (nnz_P) *nnz_P = L.P.nnz();
  if (n_cols_P) *n_cols_P = L.P.n_cols;
  return MM_OK;
}

int mm_setup_level_export(mm_setup* s, int level, int* A_ptr, int* A_col, double* A_val, int* P_ptr, int* P_col,
                          double* P_val, int* agg) {
  if (!s || level < 0 || level >= (int)s->amg.size()) return MM_ERR_ARG;
  const mm::AmgLevel& L = s->amg[level];
  if (A_ptr) std::copy(L.A.ptr.begin(), L.A.ptr.end(), A_ptr);
  if (A_col) std::copy(L.A.col.begin(), L.A.col.end(), A_col);
  if (A_val) std::copy(L.A.val.begin(), L.A.val.end(), A_val);
  if (P_ptr && !L.P.ptr.empty()) std::copy(L.P.ptr.begin(), L.P.ptr.end(), P_ptr);
  if (P_col) std::copy(L.P.col.begin(), L.P.col.end(), P_col);
  if (P_val) std::copy(L.P.val.begin(), L.P.val.end(), P_val);
  if (agg) {
    if (L.agg.empty()) std::fill(agg, agg + L.A.n_rows, -1);
    else std::copy(L.agg.begin(), L.agg.end(), agg);
  }
  return MM_OK;
}

int mm_create(int N, int E, const int* conn, const double* volume, const double* grad_phi, const int* mat_id,
              int n_mat, const double* A_lookup, const double* K1_lookup, const double* Js_lookup,
              const double* k_easy, double V_mag, const double* M_nodal, const double* boundary_mask,
              mm_problem** out) {
  if (!out || N <= 0 || E <= 0 || n_mat <= 0 || !conn || !volume || !grad_phi || !mat_id || !A_lookup ||
      !K1_lookup || !Js_lookup || !k_easy || !M_nodal || !(V_mag > 0))
    return MM_ERR_ARG;
  *out = nullptr;
  mm_problem* h = new mm_problem();
  int rc = guarded(h, [&] {
    CK(cudaGetDevice(&h->device));
    for (int e = 0; e < 4 * E; ++e)
      if (conn[e] < 0 || conn[e] >= N) throw Fail{MM_ERR_ARG, "connectivity index out of range"};
    h->N = N;
    h->E = E;
    h->n_mat = n_mat;
    h->V_mag = V_mag;
    h->inv_Vmag = 1.0 / V_mag;
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    {
      int dev = 0, sms = 0;
      CK(cudaGetDevice(&dev));
      CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      if (sms > 0) g_vec_cap = std::min(4 * sms, MAXG);
    }
    CK(cudaEventCreate(&h->ev0));
    CK(cudaEventCreate(&h->ev1));
    h->conn.assign(conn, conn + 4 * (size_t)E);
    h->mat_id.assign(mat_id, mat_id + E);
    h->volume.assign(volume, volume + E);
    h->grad_phi.assign(grad_phi, grad_phi + 12 * (size_t)E);
    h->has_mask = boundary_mask != nullptr;
    if (h->has_mask) h->mask_h.assign(boundary_mask, boundary_mask + N);
    mm::SetupScope scope;
    h->eop_h = mm::assemble_energy(N, E, conn, volume, grad_phi, mat_id, n_mat, A_lookup, K1_lookup, Js_lookup,
                                   k_easy);
    const mm::EnergyOp& o = h->eop_h;
    mmk::EnergyDev& d = h->eop;
    d.n_rows = o.n_rows;
    d.rows = h->upload(o.rows);
    d.ptr = h->upload(o.ptr);
    d.col = h->upload(o.col);
    d.mat = h->upload(o.mat);
    d.w = h->upload(o.w);
    d.q = h->upload(o.q);
    d.gx = h->upload(o.gx);
    d.gy = h->upload(o.gy);
    d.gz = h->upload(o.gz);
    d.dx = h->upload(o.dx);
    d.dy = h->upload(o.dy);
    d.dz = h->upload(o.dz);
    h->kax_h.assign(k_easy, k_easy + 3 * (size_t)n_mat);
    d.kax = h->upload(h->kax_h);
    d.single_axis = o.single_axis ? 1 : 0;
    d.axis0 = o.mat.empty() ? 0 : o.mat[0];
    h->eop_tpr = pick_tpr((int64_t)o.col.size(), std::max(1, o.n_rows));
    h->upload_eop_sell_all();
    h->d_Mn = h->upload(std::vector<double>(M_nodal, M_nodal + N));
    // default node weights (src/hysteresis_loop.py:340-353)
    std::vector<double> imr(N), imp(N), dex(N);
    for (int i = 0; i < N; ++i) {
      imr[i] = M_nodal[i] > 1e-20 ? V_mag / M_nodal[i] : 0.0;
      dex[i] = o.diag_exchange[i] * h->inv_Vmag;
      imp[i] = dex[i] > 1e-20 ? 1.0 / dex[i] : 1.0;
    }
    h->d_inv_M_rel = h->upload(imr);
    h->d_inv_M_prec = h->upload(imp);
    h->d_diag_ex = h->upload(dex);
    const size_t n3 = 3 * (size_t)N;
    h->d_m = h->alloc<double>(n3);
    h->d_U = h->alloc<double>(N);
    h->d_g = h->alloc<double>(n3);
    h->d_v = h->alloc<double>(n3);
    h->d_out = h->alloc<double>(n3);
    h->d_b = h->alloc<double>(N);
    CK(cudaMemsetAsync(h->d_g, 0, n3 * sizeof(double), h->st));
    CK(cudaMemsetAsync(h->d_out, 0, n3 * sizeof(double), h->st));
    CK(cudaMemsetAsync(h->d_b, 0, N * sizeof(double), h->st));
    h->d_x = h->alloc<double>(N);
    CK(cudaMemsetAsync(h->d_x, 0, N * sizeof(double), h->st));
    h->d_r64 = h->alloc<double>(N);
    h->d_r32 = h->alloc<float>(N);
    h->d_d32 = h->alloc<float>(N);
    h->d_part = h->alloc<double>((size_t)mmk::NRED * MAXG);
    CK(cudaMemsetAsync(h->d_part, 0, (size_t)mmk::NRED * MAXG * sizeof(double), h->st));
    h->d_sc = h->alloc<mmk::Scalars>(1);
    CK(cudaMemsetAsync(h->d_sc, 0, sizeof(mmk::Scalars), h->st));  // ticket counters start at zero
    h->d_sc32 = h->alloc<mmk::Scalars>(1);
    CK(cudaMemsetAsync(h->d_sc32, 0, sizeof(mmk::Scalars), h->st));
    h->h_sc = (mmk::Scalars*)pinned_get();
    h->sync();
    return MM_OK;
  });
  if (rc != MM_OK) {
    g_create_error = h->err;
    mm_destroy(h);
    return rc;
  }
  *out = h;
  return MM_OK;
}

int mm_destroy(mm_problem* h) {
  if (!h) return MM_ERR_ARG;
  DeviceGuard device_guard(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->s64.exec) cudaGraphExecDestroy(h->s64.exec);
  if (h->s64.graph) cudaGraphDestroy(h->s64.graph);
  if (h->s32.exec) cudaGraphExecDestroy(h->s32.exec);
  if (h->s32.graph) cudaGraphDestroy(h->s32.graph);
  h->drop_inner_graphs();
  for (cudaStream_t a : h->aux_st)
    if (a) cudaStreamDestroy(a);
  // stream-ordered frees behind everything the stream holds (it was synchronized above); the stream
  // is destroyed below without a wait, and the pool takes the memory back when the stream reaches them
  for (void* p : h->allocs) {
    if (h->st) cudaFreeAsync(p, h->st);
    else cudaFree(p);
  }
  pinned_put(h->h_sc);
  pinned_put(h->h_ms);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->ev_after) cudaEventDestroy(h->ev_after);
  if (h->ev_copy) cudaEventDestroy(h->ev_copy);
  if (h->st_copy) cudaStreamDestroy(h->st_copy);
  for (cudaEvent_t e : h->prof_pool) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return MM_OK;
}

int mm_build_poisson(mm_problem* h, double reg, int precond_type, int max_levels, int max_coarse, int* n_levels) {
  if (!h || precond_type < MM_PRECOND_NONE || precond_type > MM_PRECOND_AMGCL) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (h->poisson_built) throw Fail{MM_ERR_STATE, "Poisson operator already built"};
    mm::SetupScope scope;
    h->reg = reg;
    h->precond = precond_type;
    mm::HostCSR A = mm::assemble_poisson(h->N, h->E, h->conn.data(), h->volume.data(), h->grad_phi.data(),
                                         h->has_mask ? h->mask_h.data() : nullptr, reg);
    const bool amg = precond_type == MM_PRECOND_AMG || precond_type == MM_PRECOND_AMGCL;
    if (amg) {
      mm::AmgParams prm;
      prm.max_levels = max_levels > 0 ? max_levels : 10;
      prm.max_coarse = max_coarse > 0 ? max_coarse : 1000;
      if (h->sa_theta_e3 > 0) prm.theta0 = 1e-3 * h->sa_theta_e3;
      if (h->sa_factor_e3 > 0) prm.theta_factor = 1e-3 * h->sa_factor_e3;
      if (h->sa_filter_e6 > 0) prm.filter_eps = 1e-6 * h->sa_filter_e6;
      if (h->sa_filter_e6 < 0) prm.filter_eps = 0.0;
      h->amg_h = mm::build_amg(A, prm);
    } else {
      h->amg_h.clear();
      mm::AmgLevel L0;
      L0.A = A;
      h->amg_h.push_back(L0);
    }
    const int L = (int)h->amg_h.size();
    build_solver<double>(h, h->s64, A, amg, precond_type);
    h->s64.b = h->d_b;
    h->s64.x = h->d_x;
    h->s64.sc = h->d_sc;
    if (h->mixed || h->fp32_precond) {
      build_solver<float>(h, h->s32, A, amg, precond_type);
      h->s32.b = h->d_r32;
      h->s32.x = h->d_d32;
      h->s32.sc = h->d_sc32;
    }
    h->sync();
    h->poisson_built = true;
    if (n_levels) *n_levels = L;
    return MM_OK;
  });
}

int mm_amg_level_info(mm_problem* h, int level, int* n, int64_t* nnz_A, int64_t* nnz_P) {
  if (!h || !h->poisson_built || level < 0 || level >= (int)h->amg_h.size()) return MM_ERR_ARG;
  const mm::AmgLevel& L = h->amg_h[level];
  if (n) *n = L.A.n_rows;
  if (nnz_A) *nnz_A = L.A.nnz();
  if (nnz_P) *nnz_P = L.P.nnz();
  return MM_OK;
}

int mm_amg_export_level(mm_problem* h, int level, int* A_ptr, int* A_col, double* A_val, int* agg) {
  if (!h || !h->poisson_built || level < 0 || level >= (int)h->amg_h.size()) return MM_ERR_ARG;
  const mm::AmgLevel& L = h->amg_h[level];
  if (A_ptr) std::copy(L.A.ptr.begin(), L.A.ptr.end(), A_ptr);
  if (A_col) std::copy(L.A.col.begin(), L.A.col.end(), A_col);
  if (A_val) std::copy(L.A.val.begin(), L.A.val.end(), A_val);
  if (agg) {
    if (L.agg.empty()) std::fill(agg, agg + L.A.n_rows, -1);
    else std::copy(L.agg.begin(), L.agg.end(), agg);
  }
  return MM_OK;
}

int mm_energy_grad(mm_problem* h, const double* m, const double* U, const double* B, const double* B_bias, double* E,
                   double* g) {
  if (!h || !m || !U || !B || !E || !g) return MM_ERR_ARG;
  return guarded(h, [&] {
    const size_t n3 = 3 * (size_t)h->N;
    CK(cudaMemcpyAsync(h->d_m, m, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_U, U, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    const double* dbias = nullptr;
    if (B_bias) {
      if (!h->d_bias) h->d_bias = h->alloc<double>(n3);
      CK(cudaMemcpyAsync(h->d_bias, B_bias, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
      dbias = h->d_bias;
    }
    *E = energy_dev(h, h->d_m, h->d_U, B, dbias, h->d_g);
    CK(cudaMemcpyAsync(g, h->d_g, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return std::isfinite(*E) ? MM_OK : MM_NONFINITE;
  });
}

int mm_energy_grad_dev(mm_problem* h, const double* d_m, const double* d_U, const double* B, const double* d_bias,
                       double* E, double* d_g) {
  if (!h || !d_m || !d_U || !B || !E || !d_g) return MM_ERR_ARG;
  return guarded(h, [&] {
    CK(cudaMemsetAsync(d_g, 0, 3 * (size_t)h->N * sizeof(double), h->st));
    *E = energy_dev(h, d_m, d_U, B, d_bias, d_g);
    return std::isfinite(*E) ? MM_OK : MM_NONFINITE;
  });
}

int mm_local_grad(mm_problem* h, const double* v, double* out) {
  if (!h || !v || !out) return MM_ERR_ARG;
  return guarded(h, [&] {
    const size_t n3 = 3 * (size_t)h->N;
    CK(cudaMemcpyAsync(h->d_v, v, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    local_grad_dev(h, h->d_v, h->d_out);
    CK(cudaMemcpyAsync(out, h->d_out, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return MM_OK;
  });
}

int mm_solve_py_g(mm_problem* h, const double* m, const double* g_ext, const double* g_tan_ext, int max_iter,
                  double tol, double reg, double stagnation_nu, double* y, int* iters) {
  if (!h || !m || !g_ext || !g_tan_ext || !y || !iters || max_iter < 0 || !(stagnation_nu >= 0.0)) return MM_ERR_ARG;
  return guarded(h, [&] {
    ensure_min_buffers(h, 0);
    const size_t n3 = 3 * (size_t)h->N;
    CK(cudaMemcpyAsync(h->w_mt, m, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->w_gt_trial, g_ext, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->w_gte, g_tan_ext, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    mm_min_params prm{};
    prm.pc_iters = max_iter;
    prm.pc_stagnation_nu = stagnation_nu;
    MinCtx c{h, h->N, {0.0, 0.0, 0.0}, 0.0, &prm};
    struct CountMode {
      mm_problem* h;
      ~CountMode() { h->inner_cpp_count = false; }
    } count_mode{h};
    h->inner_cpp_count = true;
    const int it = solve_Py_g(c, h->w_mt, h->w_gt_trial, h->w_gte, tol, h->w_y, reg, max_iter, stagnation_nu);
    CK(cudaMemcpyAsync(y, h->w_y, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    *iters = it;
    return MM_OK;
  });
}

int mm_exchange_diagonal(mm_problem* h, double* d) {
  if (!h || !d) return MM_ERR_ARG;
  return guarded(h, [&] {
    CK(cudaMemcpyAsync(d, h->d_diag_ex, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return MM_OK;
  });
}

int mm_rhs(mm_problem* h, const double* m, double* b, double* bnorm2) {
  if (!h || !m || !b) return MM_ERR_ARG;
  return guarded(h, [&] {
    CK(cudaMemcpyAsync(h->d_m, m, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(h->d_b, 0, h->N * sizeof(double), h->st));
    enqueue_rhs(h, h->d_m);
    const double bb = h->red(R_BB0);
    if (bnorm2) *bnorm2 = bb;
    CK(cudaMemcpyAsync(b, h->d_b, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return MM_OK;
  });
}

int mm_apply_A(mm_problem* h, const double* U, double* y) {
  if (!h || !U || !y) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    CK(cudaMemcpyAsync(h->d_U, U, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    spmv<0, double>(h, h->s64.lv[0].A, h->d_U, nullptr, nullptr, h->d_out, nullptr);
    CK(cudaMemcpyAsync(y, h->d_out, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return MM_OK;
  });
}

int mm_precond(mm_problem* h, const double* r, double* z) {
  if (!h || !r || !z) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    CK(cudaMemcpyAsync(h->d_U, r, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    enqueue_precond<double>(h, h->s64, h->d_U, h->d_out);
    CK(cudaMemcpyAsync(z, h->d_out, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    return MM_OK;
  });
}

// The initial guess's upload on the problem's second copy stream, behind the work already queued on
// its stream (which may still read d_U); returns the event the solve waits on before using it.
static cudaEvent_t upload_x0(mm_problem* h, const double* x0) {
  if (!h->st_copy) CK(cudaStreamCreateWithFlags(&h->st_copy, cudaStreamNonBlocking));
  if (!h->ev_copy) CK(cudaEventCreateWithFlags(&h->ev_copy, cudaEventDisableTiming));
  CK(cudaEventRecord(h->ev_copy, h->st));
  CK(cudaStreamWaitEvent(h->st_copy, h->ev_copy, 0));
  CK(cudaMemcpyAsync(h->d_U, x0, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st_copy));
  CK(cudaEventRecord(h->ev_copy, h->st_copy));
  return h->ev_copy;
}

int mm_solve_u(mm_problem* h, const double* m, double* U, double tol, int maxiter, int* iters, double* rel_res) {
  if (!h || !m || !U || !(tol >= 0) || maxiter < 0) return MM_ERR_ARG;
  return guarded(h, [&] {
    CK(cudaMemcpyAsync(h->d_m, m, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    const cudaEvent_t ready = upload_x0(h, U);
    return solve_dev(h, h->d_m, h->d_U, tol, maxiter, iters, rel_res, U, ready);
  });
}

int mm_solve_u_x0(mm_problem* h, const double* m, const double* x0, double* U_out, double tol, int maxiter,
                  int* iters, double* rel_res) {
  if (!h || !m || !x0 || !U_out || !(tol >= 0) || maxiter < 0) return MM_ERR_ARG;
  return guarded(h, [&] {
    CK(cudaMemcpyAsync(h->d_m, m, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    const cudaEvent_t ready = upload_x0(h, x0);
    return solve_dev(h, h->d_m, h->d_U, tol, maxiter, iters, rel_res, U_out, ready);
  });
}

int mm_solve_u_dev(mm_problem* h, const double* d_m, double* d_U, double tol, int maxiter, int* iters,
                   double* rel_res) {
  if (!h || !d_m || !d_U || !(tol >= 0) || maxiter < 0) return MM_ERR_ARG;
  return guarded(h, [&] { return solve_dev(h, d_m, d_U, tol, maxiter, iters, rel_res); });
}

int mm_set_magnetoelastic(mm_problem* h, int n, const double* k1me, const double* k1me_p) {
  if (!h || n < 0 || n > h->E || (n > 0 && !k1me)) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (n == 0) {
      h->eop.mex = h->eop.mey = nullptr;
      h->eops.mex = h->eops.mey = nullptr;
      h->eops32_ok = false;
      h->eopsff_ok = false;
      h->drop_inner_graphs();
      return MM_OK;
    }
    mm::assemble_magnetoelastic(h->eop_h, h->N, h->E, h->conn.data(), h->volume.data(), h->mat_id.data(), n, k1me,
                                k1me_p);
    h->eop.mex = h->upload(h->eop_h.mx);
    h->eop.mey = h->upload(h->eop_h.my);
    h->eops.mex = h->upload_eop_sell<double>(h->eop_h.mx, 0.0);
    h->eops.mey = h->upload_eop_sell<double>(h->eop_h.my, 0.0);
    h->eops32_ok = false;
      h->eopsff_ok = false;
    h->drop_inner_graphs();
    h->sync();
    return MM_OK;
  });
}

int mm_scale_correction_dev(mm_problem* h, const double* d_m, double* d_U, const double* d_c, double* alpha) {
  if (!h || !d_m || !d_U || !d_c) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    const int N = h->N;
    const auto& A0 = h->s64.lv[0].A;
    enqueue_rhs(h, d_m);                                                      // d_b = D m
    spmv<0, double>(h, A0, d_U, nullptr, nullptr, h->d_out, nullptr);         // A U
    spmv<0, double>(h, A0, d_c, nullptr, nullptr, h->d_r64, nullptr);         // A c
    mmk::k_corr_dots<<<grid_elem(N), BS, 0, h->st>>>(N, d_c, h->d_b, h->d_out, h->d_r64, h->d_sc, h->d_part);
    LAUNCH_CHECK();
    CK(cudaMemcpyAsync(&h->h_sc->red[R_A], &h->d_sc->red[R_A], 2 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    const double num = h->h_sc->red[R_A], cAc = h->h_sc->red[R_B];
    const double a = (cAc > 0.0 && std::isfinite(cAc)) ? num / cAc : 0.0;
    mmk::k_axpby<<<grid_elem(N), BS, 0, h->st>>>(N, a, d_c, 1.0, d_U);
    LAUNCH_CHECK();
    h->sync();
    if (alpha) *alpha = a;
    return MM_OK;
  });
}

int mm_scale_correction_async(mm_problem* h, void* after, const double* d_m, double* d_U, const double* d_c) {
  if (!h || !d_m || !d_U || !d_c) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    const int N = h->N;
    const auto& A0 = h->s64.lv[0].A;
    if (!h->ev_after) CK(cudaEventCreateWithFlags(&h->ev_after, cudaEventDisableTiming));
    CK(cudaEventRecord(h->ev_after, (cudaStream_t)after));
    CK(cudaStreamWaitEvent(h->st, h->ev_after, 0));
    enqueue_rhs(h, d_m);                                                      // d_b = D m
    spmv<0, double>(h, A0, d_U, nullptr, nullptr, h->d_out, nullptr);         // A U
    spmv<0, double>(h, A0, d_c, nullptr, nullptr, h->d_r64, nullptr);         // A c
    mmk::k_corr_dots<<<grid_elem(N), BS, 0, h->st>>>(N, d_c, h->d_b, h->d_out, h->d_r64, h->d_sc, h->d_part);
    LAUNCH_CHECK();
    mmk::k_axpy_ratio<<<grid_elem(N), BS, 0, h->st>>>(N, d_c, d_U, h->d_sc);
    LAUNCH_CHECK();
    return MM_OK;
  });
}

int mm_set_bias_field(mm_problem* h, const double* B_bias) {
  if (!h) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!B_bias) {
      h->d_min_bias = nullptr;  // the buffer stays allocated for a later field
      return MM_OK;
    }
    if (!h->min_bias_buf) h->min_bias_buf = h->alloc<double>(3 * (size_t)h->N);
    CK(cudaMemcpyAsync(h->min_bias_buf, B_bias, 3 * (size_t)h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    h->sync();
    h->d_min_bias = h->min_bias_buf;
    return MM_OK;
  });
}

int mm_set_node_weights(mm_problem* h, const double* inv_M_rel, const double* inv_M_prec) {
  if (!h) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (inv_M_rel)
      CK(cudaMemcpyAsync(h->d_inv_M_rel, inv_M_rel, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    if (inv_M_prec)
      CK(cudaMemcpyAsync(h->d_inv_M_prec, inv_M_prec, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    h->sync();
    return MM_OK;
  });
}

int mm_minimize(mm_problem* h, const double* B, double* m, double* U, const mm_min_params* prm, mm_min_info* info) {
  if (!h || !B || !m || !U || !prm) return MM_ERR_ARG;
  if (prm->method < 0 || prm->method >= MM_METHOD_COUNT || prm->max_iter < 0) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    const size_t n3 = 3 * (size_t)h->N;
    // the minimizer owns d_m / d_U as its state buffers; they may be swapped with its trial buffers
    CK(cudaMemcpyAsync(h->d_m, m, n3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_U, U, h->N * sizeof(double), cudaMemcpyHostToDevice, h->st));
    double* dm = h->d_m;
    double* dU = h->d_U;
    const int rc = minimize_dev(h, B, dm, dU, prm, info);
    CK(cudaMemcpyAsync(m, dm, n3 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(U, dU, h->N * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    h->sync();
    // keep the staging pointers valid whichever buffers ended up holding the state
    h->d_m = dm;
    h->d_U = dU;
    return rc;
  });
}

int mm_minimize_dev(mm_problem* h, const double* B, double* d_m, double* d_U, const mm_min_params* prm,
                    mm_min_info* info) {
  if (!h || !B || !d_m || !d_U || !prm) return MM_ERR_ARG;
  if (prm->method < 0 || prm->method >= MM_METHOD_COUNT || prm->max_iter < 0) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    const size_t n3 = 3 * (size_t)h->N;
    // the minimizer swaps its state with its trial buffers, so it runs on the problem's own buffers;
    // the caller's arrays are copied in and out on the device
    CK(cudaMemcpyAsync(h->d_m, d_m, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_U, d_U, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    double* dm = h->d_m;
    double* dU = h->d_U;
    const int rc = minimize_dev(h, B, dm, dU, prm, info);
    CK(cudaMemcpyAsync(d_m, dm, n3 * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(d_U, dU, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    h->sync();
    h->d_m = dm;
    h->d_U = dU;
    return rc;
  });
}

int mm_time_kernel(mm_problem* h, int kernel, int reps, double* ms, double* bytes) {
  if (!h || reps <= 0 || kernel < MM_KERNEL_SPMV_A || kernel > MM_KERNEL_HESSIAN) return MM_ERR_ARG;
  return guarded(h, [&] {
    if ((kernel == MM_KERNEL_SPMV_A || kernel == MM_KERNEL_SMOOTH) && !h->poisson_built)
      throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    const size_t flush_n = (size_t)256 << 20;  // 256 MiB > L2
    char* flush = nullptr;
    CK(cudaMalloc(&flush, flush_n));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int N = h->N;
    double acc = 0.0, nbytes = 0.0;
    const LevelT<double>* l0 = h->poisson_built ? &h->s64.lv[0] : nullptr;
    auto run_kernel = [&]() {
      if (kernel == MM_KERNEL_SPMV_A) {
        spmv<0, double>(h, l0->A, h->d_U, nullptr, nullptr, h->d_out, nullptr);
      } else if (kernel == MM_KERNEL_SMOOTH) {
        const double* s = l0->s ? l0->s : h->d_U;
        launch(h, mmk::k_smooth_dot<double>, grid_ilp(l0->n), BS, l0->A.s, h->d_U, h->d_b, s, h->d_out, h->d_sc, h->d_part,
                                                                nullptr, (double*)nullptr);
        LAUNCH_CHECK();
      } else if (kernel == MM_KERNEL_ENERGY) {
        const double B[3] = {0.0, 0.0, 1.0};
        enqueue_energy(h, h->d_m, h->d_U, B, nullptr, h->d_g);
      } else {
        local_grad_dev(h, h->d_m, h->d_out);
      }
    };
    const mm::EnergyOp& o = h->eop_h;
    const double nnzE = (double)o.col.size(), nrE = (double)o.n_rows;
    // algorithmic bytes: stored non-zeros (8 B value + 4 B column), slice pointers, vectors once
    if (kernel == MM_KERNEL_SPMV_A) {
      const double nnz = (double)l0->A.nnz;
      nbytes = nnz * 12.0 + ((N + 31) / 32 + 1.0) * 4.0 + N * 8.0 * 2.0;
    } else if (kernel == MM_KERNEL_SMOOTH) {
      const double nnz = (double)l0->A.nnz;
      nbytes = nnz * 12.0 + ((N + 31) / 32 + 1.0) * 4.0 + N * 8.0 * 4.0;
    } else if (kernel == MM_KERNEL_ENERGY && h->use_energy_ff()) {
      // entries: col, (hi, lo) of w, q, G(3); rows: row id, ptr; nodes: m (3), U, M_nodal, g (3);
      // the pair splits of the nodes the rows read: the node list, m (3) and U read, the pairs of m, k.m
      // and U written
      nbytes = nnzE * (4.0 + 8.0 * 5.0) + nrE * 8.0 + nrE * 8.0 * 8.0 +
               (double)h->eopsff.n_touched * (4.0 + 8.0 * 4.0 + 8.0 * 5.0);
    } else if (kernel == MM_KERNEL_ENERGY) {
      // entries: col, mat, w, q, G(3); rows: row id, ptr; nodes: m (3), U, M_nodal, g (3)
      nbytes = nnzE * (4.0 + 4.0 + 8.0 * 5.0) + nrE * 8.0 + nrE * 8.0 * 8.0;
    } else {
      nbytes = nnzE * (4.0 + 4.0 + 8.0 * 2.0) + nrE * 8.0 + nrE * 8.0 * 6.0;
    }
    run_kernel();  // warm-up
    for (int r = 0; r < reps; ++r) {
      CK(cudaMemsetAsync(flush, r & 0xff, flush_n, h->st));
      CK(cudaEventRecord(e0, h->st));
      run_kernel();
      CK(cudaEventRecord(e1, h->st));
      CK(cudaEventSynchronize(e1));
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, e0, e1));
      acc += t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(flush);
    if (ms) *ms = acc / reps;
    if (bytes) *bytes = nbytes;
    return MM_OK;
  });
}

// ---------------------------------------------------------------------------------------------
// autotuner: lanes per row of every compressed-row operator, and which solvers use the fused coarse
// correction, chosen by timing on this GPU (CUDA events on the problem's stream)
// ---------------------------------------------------------------------------------------------
}  // extern "C"

namespace {

template <class T>
float time_ms(mm_problem* h, int reps, const std::function<void()>& f) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  f();  // warm-up
  CK(cudaEventRecord(a, h->st));
  for (int i = 0; i < reps; ++i) f();
  CK(cudaEventRecord(b, h->st));
  CK(cudaEventSynchronize(b));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

// Lanes per row of one compressed-row operator: every candidate is timed in context, as the time of
// whole V-cycles (back to back, so cache state and neighbouring kernels are those of a solve; an
// operator timed alone, L2-hot, prefers fewer lanes than it should), and the fastest is kept.
template <class T>
void tune_csr(mm_problem* h, SolverT<T>& S, DevMatT<T>& M, const mm::HostCSR& host, int reps, const char* tag,
              int level, std::string& rep) {
  if (M.c.n == 0) return;  // sliced ELL only (level 0)
  if (!M.s.sptr) h->upload_sell<T>(host, M);  // the one-thread-per-row candidate
  const int before = M.tpr;
  int best = before;
  float best_ms = 1e30f, before_ms = 1e30f;
  std::string times;
  for (int t : {1, 2, 4, 8, 16, 32}) {
    M.tpr = t;
    const float ms = time_ms<T>(h, reps, [&] { enqueue_precond<T>(h, S, S.r, S.z); });
    times += (times.empty() ? "" : ",") + std::to_string(1e3 * ms);
    if (t == before) before_ms = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
  }
  // keep the heuristic's shape unless another is clearly faster (V-cycle times vary by ~1-2 % run to run)
  if (!(best_ms < 0.97f * before_ms)) best = before;
  M.tpr = best;
  rep += std::string(rep.size() > 1 ? "," : "") + "{\"op\":\"" + tag + "\",\"level\":" + std::to_string(level) +
         ",\"precision\":\"" + (sizeof(T) == 8 ? "fp64" : "fp32") + "\",\"rows\":" + std::to_string(M.c.n) +
         ",\"nnz\":" + std::to_string(M.nnz) + ",\"heuristic_tpr\":" + std::to_string(before) +
         ",\"tpr\":" + std::to_string(best) + ",\"vcycle_us\":[" + times + "]}";
}

template <class T>
void tune_solver(mm_problem* h, SolverT<T>& S, int reps, std::string& rep) {
  if (!S.built || !multilevel(h, S)) return;
  const int L = (int)S.lv.size();
  for (int l = 0; l < L; ++l) {
    auto& c = S.lv[l];
    if (l > 0) tune_csr<T>(h, S, c.A, h->amg_h[l].A, reps, "A", l, rep);
    if (l < L - 1) {
      tune_csr<T>(h, S, c.R, h->amg_h[l].R, reps, "R", l, rep);
      tune_csr<T>(h, S, c.P, h->amg_h[l].P, reps, "P", l, rep);
      if (c.Rf.nnz > 0 && (int)h->rf_host.size() > l) tune_csr<T>(h, S, c.Rf, h->rf_host[l], reps, "Rf", l, rep);
    }
  }
  drop_graph(S);
}

// V-cycle time with and without the fused restrictions in solver S; sets the bit if they win
template <class T>
std::string tune_fuse_restrict(mm_problem* h, SolverT<T>& S, int bit, int reps) {
  if (!S.built || !multilevel(h, S) || S.lv.empty() || S.lv[0].Rf.nnz == 0) return "null";
  const int saved = h->fuse_restrict;
  float ms[2];
  for (int on = 0; on < 2; ++on) {
    h->fuse_restrict = on ? (saved | (1 << bit)) : (saved & ~(1 << bit));
    ms[on] = time_ms<T>(h, reps, [&] { enqueue_precond<T>(h, S, S.r, S.z); });
  }
  h->fuse_restrict = ms[1] < ms[0] ? (saved | (1 << bit)) : (saved & ~(1 << bit));
  drop_graph(S);
  return "{\"unfused_us\":" + std::to_string(1e3 * ms[0]) + ",\"fused_us\":" + std::to_string(1e3 * ms[1]) + "}";
}

// V-cycle time with and without the fused coarse correction in solver S; sets the bit if it wins
template <class T>
std::string tune_fuse(mm_problem* h, SolverT<T>& S, int bit, int reps) {
  if (!S.built || !S.fused || !multilevel(h, S)) return "null";
  T* r = S.r;
  T* z = S.z;
  const int saved = h->coarse_fuse;
  float ms[2];
  for (int on = 0; on < 2; ++on) {
    h->coarse_fuse = on ? (saved | (1 << bit)) : (saved & ~(1 << bit));
    ms[on] = time_ms<T>(h, reps, [&] { enqueue_precond<T>(h, S, r, z); });
  }
  h->coarse_fuse = ms[1] < ms[0] ? (saved | (1 << bit)) : (saved & ~(1 << bit));
  drop_graph(S);
  return "{\"unfused_us\":" + std::to_string(1e3 * ms[0]) + ",\"fused_us\":" + std::to_string(1e3 * ms[1]) + "}";
}

// V-cycle time with levels 1 .. 3 in one cooperative launch and with five; sets the bit if the one
// launch wins by 3 % (a loop graph that cannot hold the cooperative launch turns it off again)
template <class T>
std::string tune_coarse_cycle(mm_problem* h, SolverT<T>& S, int bit, int reps) {
  if (!S.built || !multilevel(h, S) || !S.bar || S.coop_grid <= 0) return "null";
  const int saved = h->coarse_cycle;
  h->coarse_cycle = saved & ~(1 << bit);
  const float ms_off = time_ms<T>(h, reps, [&] { enqueue_precond<T>(h, S, S.r, S.z); });
  // fewer blocks make each grid barrier cheaper and each stage less parallel: 1, 2, 4 per SM or all
  h->coarse_cycle = saved | (1 << bit);
  std::string rep = "{\"five_launches_us\":" + std::to_string(1e3 * ms_off) + ",\"one_launch_us\":{";
  float best = 1e30f;
  int best_grid = S.coop_max;
  for (int per : {1, 2, 4, 0}) {
    const int grid = per ? std::min(per * S.sms, S.coop_max) : S.coop_max;
    S.coop_grid = grid;
    const float ms = time_ms<T>(h, reps, [&] { enqueue_precond<T>(h, S, S.r, S.z); });
    rep += (per != 1 ? ",\"" : "\"") + std::to_string(grid) + "\":" + std::to_string(1e3 * ms);
    if (ms < best) {
      best = ms;
      best_grid = grid;
    }
  }
  S.coop_grid = best_grid;
  // the one launch only when clearly faster (V-cycle times vary by ~1-2 % run to run)
  h->coarse_cycle = best < 0.97f * ms_off ? (saved | (1 << bit)) : (saved & ~(1 << bit));
  drop_graph(S);
  return rep + "}}";
}

// lanes per magnetic row of the float-float energy kernel: each of 1, 2, 4, 8 timed over reps
// evaluations of the current state with L2 flushed before each (in a loop the demag solve between
// two evaluations evicts the operator), the fastest kept
std::string tune_energy_ff(mm_problem* h, int reps) {
  if (!h->use_energy_ff()) return "null";
  const double B[3] = {0.0, 0.0, 1.0};
  const size_t flush_n = (size_t)256 << 20;  // 256 MiB > L2
  char* flush = nullptr;
  CK(cudaMalloc(&flush, flush_n));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  std::string rep = "{\"us\":{";
  float best = 1e30f;
  int best_tpr = h->eff_tpr;
  for (int tpr : {1, 2, 4, 8}) {
    h->eff_tpr = tpr;
    enqueue_energy(h, h->d_m, h->d_U, B, nullptr, h->d_g);  // warm-up
    float ms = 0.f;
    for (int r = 0; r < reps; ++r) {
      CK(cudaMemsetAsync(flush, r & 0xff, flush_n, h->st));
      CK(cudaEventRecord(e0, h->st));
      enqueue_energy(h, h->d_m, h->d_U, B, nullptr, h->d_g);
      CK(cudaEventRecord(e1, h->st));
      CK(cudaEventSynchronize(e1));
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, e0, e1));
      ms += t / reps;
    }
    rep += (tpr > 1 ? ",\"" : "\"") + std::to_string(tpr) + "\":" + std::to_string(1e3 * ms);
    if (ms < best) {
      best = ms;
      best_tpr = tpr;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(flush);
  h->eff_tpr = best_tpr;
  h->drop_min_graphs();  // captured evaluations hold the old launch shape
  return rep + "},\"chosen\":" + std::to_string(best_tpr) + "}";
}

}  // namespace

extern "C" {

int mm_autotune(mm_problem* h, int reps, char* report, int report_len) {
  if (!h || reps < 1) return MM_ERR_ARG;
  return guarded(h, [&] {
    if (!h->poisson_built) throw Fail{MM_ERR_STATE, "mm_build_poisson must be called first"};
    std::string ops = "[";
    tune_solver<double>(h, h->s64, reps, ops);
    tune_solver<float>(h, h->s32, reps, ops);
    ops += "]";
    const std::string f64 = tune_fuse<double>(h, h->s64, 0, reps);
    const std::string f32 = tune_fuse<float>(h, h->s32, 1, reps);
    const std::string r64 = tune_fuse_restrict<double>(h, h->s64, 0, reps);
    const std::string r32 = tune_fuse_restrict<float>(h, h->s32, 1, reps);
    const std::string eff = tune_energy_ff(h, reps);
    const std::string c64 = tune_coarse_cycle<double>(h, h->s64, 0, reps);
    const std::string c32 = tune_coarse_cycle<float>(h, h->s32, 1, reps);
    const std::string rep = "{\"operators\":" + ops + ",\"coarse_fuse\":{\"fp64\":" + f64 + ",\"fp32\":" + f32 +
                            ",\"chosen\":" + std::to_string(h->coarse_fuse) + "},\"fuse_restrict\":{\"fp64\":" +
                            r64 + ",\"fp32\":" + r32 + ",\"chosen\":" + std::to_string(h->fuse_restrict) + "},\"energy_ff\":" + eff +
                            ",\"coarse_cycle\":{\"fp64\":" + c64 + ",\"fp32\":" + c32 +
                            ",\"chosen\":" + std::to_string(h->coarse_cycle) + "}}";
    h->sync();
    if (report && report_len > 0) {
      const size_t n = std::min(rep.size(), (size_t)report_len - 1);
      std::memcpy(report, rep.data(), n);
      report[n] = 0;
    }
    return MM_OK;
  });
}

int mm_get_option(mm_problem* h, int option, int* value) {
  if (!h || !value) return MM_ERR_ARG;
  switch (option) {
    case MM_OPT_COARSE_CYCLE: *value = h->coarse_cycle; return MM_OK;
    case MM_OPT_FUSE_RESTRICT: *value = h->fuse_restrict; return MM_OK;
    case MM_OPT_COARSE_FUSE: *value = h->coarse_fuse; return MM_OK;
    case MM_OPT_ENERGY_FF_LANES: *value = h->eff_tpr; return MM_OK;
    case MM_OPT_MIN_GRAPH: *value = h->min_graph; return MM_OK;
    default: return MM_ERR_ARG;
  }
}

int mm_set_option(mm_problem* h, int option, int value) {
  if (!h) return MM_ERR_ARG;
  if (option == MM_OPT_GRAPH) {
    h->use_graph = value != 0;
    return MM_OK;
  }
  if (option == MM_OPT_PRECISION) {
    if (h->poisson_built) return MM_ERR_STATE;  // the FP32 hierarchy is built by mm_build_poisson
    if (value != MM_PRECISION_FP64 && value != MM_PRECISION_MIXED && value != MM_PRECISION_FP32_PRECOND)
      return MM_ERR_ARG;
    h->mixed = value == MM_PRECISION_MIXED;
    h->fp32_precond = value == MM_PRECISION_FP32_PRECOND;
    return MM_OK;
  }
  if (option == MM_OPT_SPLIT_A0) {
    if (value != 0 && value != 1) return MM_ERR_ARG;
    if (h->split_a0 != (value == 1)) drop_graph(h->s64);  // the captured loop holds the old product
    h->split_a0 = value == 1;
    return MM_OK;
  }
  if (option == MM_OPT_MIN_FP32) {
    if (value < -1 || value > 1) return MM_ERR_ARG;
    h->min_fp32 = value;
    return MM_OK;
  }
  if (option == MM_OPT_GRID_CAP) {
    if (value < 1 || value > MAXG) return MM_ERR_ARG;
    g_elem_cap = value;
    return MM_OK;
  }
  if (option == MM_OPT_PROFILE) {
    if (value != 0 && value != 1) return MM_ERR_ARG;
    h->prof = value == 1;
    return MM_OK;
  }
  if (option == MM_OPT_PDL) {
    if (value != 0 && value != 1) return MM_ERR_ARG;
    if (h->pdl != (value == 1)) {  // captured loop graphs hold the old launches
      drop_graph(h->s64);
      drop_graph(h->s32);
      h->drop_inner_graphs();
    }
    h->pdl = value == 1;
    return MM_OK;
  }
  if (option == MM_OPT_COARSE_FUSE) {
    if (value < 0 || value > 3) return MM_ERR_ARG;
    if (h->coarse_fuse != value) {
      drop_graph(h->s64);
      drop_graph(h->s32);
    }
    h->coarse_fuse = value;
    return MM_OK;
  }
  if (option == MM_OPT_ENERGY_FF) {
    if (value < -1 || value > 1) return MM_ERR_ARG;
    h->energy_ff = value;
    return MM_OK;
  }
  if (option == MM_OPT_FUSE_RESTRICT) {
    if (value < 0 || value > 3) return MM_ERR_ARG;
    if (h->fuse_restrict != value) {
      drop_graph(h->s64);
      drop_graph(h->s32);
    }
    h->fuse_restrict = value;
    return MM_OK;
  }
  if (option == MM_OPT_SA_FACTOR_E3) {
    if (value < 0 || value > 1000) return MM_ERR_ARG;
    if (h->poisson_built) return MM_ERR_STATE;
    h->sa_factor_e3 = value;
    return MM_OK;
  }
  if (option == MM_OPT_SA_FILTER_E6) {
    if (value > 100000) return MM_ERR_ARG;
    if (h->poisson_built) return MM_ERR_STATE;
    h->sa_filter_e6 = value;
    return MM_OK;
  }
  if (option == MM_OPT_SA_THETA_E3) {
    if (value < 0 || value >= 1000) return MM_ERR_ARG;
    if (h->poisson_built) return MM_ERR_STATE;
    h->sa_theta_e3 = value;
    return MM_OK;
  }
  if (option == MM_OPT_CSR_LANES) {
    if (value != 2 && value != 4 && value != 8 && value != 16 && value != 32) return MM_ERR_ARG;
    if (!h->poisson_built) return MM_ERR_STATE;
    auto set_all = [&](auto& S) {
      for (auto& c : S.lv)
        for (auto* M : {&c.A, &c.R, &c.P, &c.Rf})
          if (M->c.n > 0 && M->tpr != 1) M->tpr = value;
      drop_graph(S);
    };
    set_all(h->s64);
    set_all(h->s32);
    h->drop_inner_graphs();
    return MM_OK;
  }
  if (option == MM_OPT_COARSE_CYCLE) {
    if (value < 0 || value > 3) return MM_ERR_ARG;
    if (h->coarse_cycle != value) {
      drop_graph(h->s64);
      drop_graph(h->s32);
    }
    h->coarse_cycle = value;
    return MM_OK;
  }
  if (option == MM_OPT_ENERGY_FF_LANES) {
    if (value != 1 && value != 2 && value != 4 && value != 8) return MM_ERR_ARG;
    if (h->eff_tpr != value) h->drop_min_graphs();
    h->eff_tpr = value;
    return MM_OK;
  }
  if (option == MM_OPT_MIN_GRAPH) {
    if (value != 0 && value != 1) return MM_ERR_ARG;
    h->min_graph = value;
    h->min_graph_failed = false;
    return MM_OK;
  }
  if (option == MM_OPT_MIXED_ETA_E6) {
    if (value <= 0 || value >= 1000000) return MM_ERR_ARG;
    h->mixed_eta = value * 1e-6;
    return MM_OK;
  }
  return MM_ERR_ARG;
}

int mm_profile_read(mm_problem* h, int64_t* launches, double* total_ms, double* bytes_per_launch) {
  if (!h || !launches || !total_ms || !bytes_per_launch) return MM_ERR_ARG;
  for (int i = 0; i < MM_PROF_SLOTS; ++i) {
    launches[i] = h->prof_n[i];
    total_ms[i] = h->prof_ms[i];
    bytes_per_launch[i] = h->prof_bytes[i];
  }
  return MM_OK;
}

int mm_profile_reset(mm_problem* h) {
  if (!h) return MM_ERR_ARG;
  for (int i = 0; i < MM_PROF_SLOTS; ++i) {
    h->prof_n[i] = 0;
    h->prof_ms[i] = 0.0;
    h->prof_bytes[i] = 0.0;
  }
  return MM_OK;
}

int mm_last_refinements(mm_problem* h, int* steps) {
  if (!h || !steps) return MM_ERR_ARG;
  *steps = h->last_outer;
  return MM_OK;
}

int mm_last_solve_ms(mm_problem* h, double* ms) {
  if (!h || !ms) return MM_ERR_ARG;
  *ms = h->last_solve_ms;
  return MM_OK;
}

int mm_launch_count(mm_problem* h, int64_t* count) {
  if (!h || !count) return MM_ERR_ARG;
  *count = h->n_launch;
  return MM_OK;
}

int mm_sync(mm_problem* h) {
  if (!h) return MM_ERR_ARG;
  return guarded(h, [&] {
    h->sync();
    return MM_OK;
  });
}

}  // extern "C"
