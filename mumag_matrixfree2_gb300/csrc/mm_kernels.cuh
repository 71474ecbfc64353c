// Device kernels of the micromagnetic hot path (sm_103a).
//
// Design notes (GB300):
//  * FP64 issue rate is ~1/64 of FP32 on this part, so FP64 instructions are budgeted like memory
//    traffic: every product is one DFMA per stored non-zero, with no shuffle reductions on the
//    fine levels (thread-per-row sliced-ELL storage, slice height 32, columns sorted per row).
//  * Every reduction is deterministic: each block writes one partial (fixed grid, fixed in-block
//    tree); the last block to arrive (atomic ticket) sums the partials in block order and stores
//    the scalar in Scalars::red.  Consumers read one scalar.
//  * Iterative kernels read the device "done" flag first and return when it is set, so queued
//    iterations after convergence cost a launch and nothing else; the PCG loop itself runs inside
//    a CUDA graph whose conditional WHILE node is driven by k_set_cond.
#pragma once

#include <cuda/atomic>
#include <cuda_runtime.h>
#include <type_traits>
#include <stdint.h>

namespace mmk {

constexpr int BS = 256;    // threads per block for every kernel here
constexpr int MAXG = 4096; // upper bound of any grid, and of the partials of one reduction

enum RedSlot { R_BB0, R_BB, R_R2, R_RZ, R_PAP, R_SUM, R_E, R_MAX, R_A, R_B, R_C, R_D, NRED };

struct Scalars {
  double tol2;      // tol^2 * b.b
  double rz;        // current r.z
  double alpha;     // rz / (p.Ap + eps), set when p.Ap is reduced
  double beta;      // rz_new / (rz_old + eps), set when r.z is reduced (0 for the first direction)
  float alpha_f;    // alpha and beta rounded once for the FP32 kernels
  float beta_f;
  int it;           // completed PCG iterations
  int done;         // 1 once converged or out of iterations (set when r.r is reduced)
  int maxiter;
  int loops;        // graph-loop trips (hard stop for the conditional node)
  int rz_valid;     // 0 until the first r.z of a solve is reduced
  int bar_err;      // a grid barrier of the one-launch coarse cycle gave up waiting (sticky)
  double red[NRED];
  unsigned cnt[NRED];
  // the minimizer's inner (preconditioner) solve, driven on the device
  double in_rho;     // current r.z
  double in_target;  // tol^2 * r0.z0
  double in_Q;       // accumulated model decrease
  double in_dq;      // this iteration's decrease 0.5 alpha rho
  double in_alpha;
  double in_beta;
  double in_tol2;
  double in_nu;      // stagnation threshold
  float in_alpha_f;
  float in_beta_f;
  int in_it;         // completed inner iterations
  int in_max;
  int in_stop;       // p.Pp <= 0 or stagnation: this iteration does not update y and r
  int in_done;       // the loop ends after this iteration
  int in_loops;      // graph-loop trips (hard stop for the conditional node)
  int in_cpp;        // 1: a trip that stops on curvature or stagnation is not counted (C++ minimizer)
};

// Scalar follow-ups computed once, by the block that finishes a reduction (so that no thread of
// the consumer kernels spends FP64 divides or compares on them).
enum Post { POST_NONE, POST_PAP, POST_R2_STEP, POST_R2_INIT, POST_RZ, POST_MEAN, POST_IN_INIT, POST_IN_PAP,
            POST_IN_RHO };

// Programmatic dependent launch: wait until the preceding grid in the stream has completed and its
// writes are visible, then allow the next grid to be scheduled (it waits the same way).  Both are
// no-ops when the kernel was launched normally.  Every solver kernel starts with this, so the
// launch latency of a kernel overlaps the drain of its predecessor.
__device__ __forceinline__ void pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ------------------------------------------------------------------------------------------
// deterministic reductions
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Sum (or max) over the block; the result is returned to every thread.  Transposed: the first warp
// folds the block's 256 values eight to a lane, then one shuffle tree, i.e. 12 warp-wide FP64
// instructions per block instead of a tree in every warp (48); a warp-wide FP64 add holds the SM's
// FP64 pipe for 16 cycles on this part, so the trees were a visible share of the FP64 kernels.
template <bool MAX>
__device__ __forceinline__ double block_reduce(double v) {
  __shared__ double s_red[BS];
  __shared__ double s_out;
  __syncthreads();  // the previous reduction of this block has read s_red and s_out
  s_red[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = s_red[threadIdx.x];
#pragma unroll
    for (int k = 1; k < BS / 32; ++k) {
      const double u = s_red[threadIdx.x + 32 * k];
      t = MAX ? fmax(t, u) : t + u;
    }
    t = MAX ? warp_max(t) : warp_sum(t);
    if (threadIdx.x == 0) s_out = t;
  }
  __syncthreads();
  return s_out;
}
__device__ __forceinline__ double block_sum(double v) { return block_reduce<false>(v); }

// Grid reduction of up to two values into sc->red[slot0], sc->red[slot1] (slot1 < 0: one value).
// Partials go to part + slot * MAXG; the ticket counter of slot0 elects the finishing block.
template <bool MAX = false>
__device__ __forceinline__ void grid_finish(double v0, double v1, Scalars* sc, double* part, int slot0,
                                            int slot1 = -1, int post = POST_NONE, double post_arg = 0.0);

template <bool MAX = false>
__device__ __forceinline__ void grid_reduce(double v0, double v1, Scalars* sc, double* part, int slot0,
                                            int slot1 = -1, int post = POST_NONE, double post_arg = 0.0) {
  v0 = block_reduce<MAX>(v0);
  if (slot1 >= 0) v1 = block_reduce<MAX>(v1);
  grid_finish<MAX>(v0, v1, sc, part, slot0, slot1, post, post_arg);
}

// block values v0, v1 (identical in every thread of the block) -> grid total in sc->red.
// Thread 0 publishes the block's partials and takes a ticket with one acquire-release atomic (its
// release orders the partials before the ticket); the block holding the last ticket loads every
// partial at once (independent, unrolled loads), sums them in block order and runs the follow-up.
template <bool MAX>
__device__ __forceinline__ void grid_finish(double v0, double v1, Scalars* sc, double* part, int slot0, int slot1,
                                            int post, double post_arg) {
  __shared__ unsigned s_last;
  if (threadIdx.x == 0) {
    part[(size_t)slot0 * MAXG + blockIdx.x] = v0;
    if (slot1 >= 0) part[(size_t)slot1 * MAXG + blockIdx.x] = v1;
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> ticket(sc->cnt[slot0]);
    const unsigned t = ticket.fetch_add(1u, cuda::memory_order_acq_rel);
    s_last = (t == gridDim.x - 1) ? 1u : 0u;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    const int G = (int)gridDim.x;
    const double* pa = part + (size_t)slot0 * MAXG;
    const double* pb = part + (size_t)(slot1 >= 0 ? slot1 : slot0) * MAXG;
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int k = 0; k < MAXG / BS; ++k) {
      const int i = threadIdx.x + k * BS;
      if (i < G) {
        const double xa = __ldcg(pa + i);
        a = MAX ? fmax(a, xa) : a + xa;
        if (slot1 >= 0) {
          const double xb = __ldcg(pb + i);
          b = MAX ? fmax(b, xb) : b + xb;
        }
      }
    }
    a = block_reduce<MAX>(a);
    if (slot1 >= 0) b = block_reduce<MAX>(b);
    if (threadIdx.x == 0) {
      sc->red[slot0] = a;
      if (slot1 >= 0) sc->red[slot1] = b;
      sc->cnt[slot0] = 0u;
      if (post == POST_PAP) {
        sc->alpha = sc->rz / (a + 1e-30);
        sc->alpha_f = (float)sc->alpha;
      } else if (post == POST_R2_STEP || post == POST_R2_INIT) {
        if (post == POST_R2_STEP) sc->it += 1;
        if (a <= sc->tol2 || sc->it >= sc->maxiter) sc->done = 1;
      } else if (post == POST_RZ) {
        sc->beta = sc->rz_valid ? a / (sc->rz + 1e-30) : 0.0;
        sc->beta_f = (float)sc->beta;
        sc->rz = a;
        sc->rz_valid = 1;
      } else if (post == POST_MEAN) {
        sc->red[slot0] = a / post_arg;
      } else if (post == POST_IN_INIT) {
        sc->in_rho = a;
        sc->in_target = sc->in_tol2 * a;
        sc->in_done = !(sc->in_it < sc->in_max && a > sc->in_target && a > 1e-25 && a < 1e20);
      } else if (post == POST_IN_PAP) {
        const double alpha = sc->in_rho / (a + 1e-30);
        const double dq = 0.5 * alpha * sc->in_rho;
        const bool stag = (sc->in_it > 0) && (dq <= sc->in_nu * sc->in_Q);
        sc->in_alpha = alpha;
        sc->in_alpha_f = (float)alpha;
        sc->in_dq = dq;
        sc->in_stop = (a <= 0.0) || stag;
      } else if (post == POST_IN_RHO) {
        const double rho = a;
        sc->in_beta = rho / (sc->in_rho + 1e-30);
        sc->in_beta_f = (float)sc->in_beta;
        sc->in_rho = rho;
        sc->in_Q = sc->in_Q + sc->in_dq;
        sc->in_it += (sc->in_cpp && sc->in_stop) ? 0 : 1;
        sc->red[R_D] = (double)sc->in_it;  // read by the host with the fallback test's sums
        sc->in_done = sc->in_stop ||
                      !(sc->in_it < sc->in_max && rho > sc->in_target && rho > 1e-25 && rho < 1e20);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------
// Solver kernels, templated on the storage/arithmetic type T of the operator and the vectors:
// T = double for the plain FP64 method, T = float for the inner solves of the mixed-precision
// method.  Inner products and every reduction are accumulated in FP64 in both cases.
// ------------------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T fmaT(T a, T b, T c) { return fma(a, b, c); }

// Inner-product accumulators.  FP64 kernels accumulate in FP64.  FP32 kernels accumulate in
// float-float: the product of two floats is split exactly into hi + lo with one FMA (TwoProd) and
// added with Knuth's TwoSum, so the sum keeps ~48 significant bits while using only FP32 pipes
// (FP64 issue is ~1/64 of FP32 on this GPU); it becomes FP64 once per warp.
template <class T>
struct Acc;
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double warp_total() { return warp_sum(s); }  // valid on lane 0
};
template <>
struct Acc<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ static void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
  }
  __device__ __forceinline__ void add(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);  // exact: a*b = p + pe
    float t, e;
    two_sum(hi, p, t, e);
    hi = t;
    lo += e + pe;
  }
  __device__ __forceinline__ void merge(float h2, float l2) {
    float t, e;
    two_sum(hi, h2, t, e);
    hi = t;
    lo += e + l2;
  }
  __device__ __forceinline__ double warp_total() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_down_sync(0xffffffffu, hi, o);
      const float l2 = __shfl_down_sync(0xffffffffu, lo, o);
      merge(h2, l2);
    }
    return (double)hi + (double)lo;  // valid on lane 0
  }
};

// A scalar in the kernel's precision (the FP32 copy is rounded once, by the reducing block).
template <class T>
__device__ __forceinline__ T scal(double d, float f);
template <>
__device__ __forceinline__ double scal<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float scal<float>(double, float f) { return f; }

// Block total of an accumulator, returned to every thread (FP64 only across the warp leaders; an
// FP64 accumulator takes the transposed block reduction).
template <class T>
__device__ __forceinline__ double block_total(Acc<T>& acc) {
  if constexpr (std::is_same<T, double>::value) {
    return block_reduce<false>(acc.s);
  } else {
    __shared__ double s_w[BS / 32];
    __shared__ double s_out;
    const double w = acc.warp_total();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s_w[wid] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
#pragma unroll
      for (int i = 0; i < BS / 32; ++i) t += s_w[i];
      s_out = t;
    }
    __syncthreads();
    return s_out;
  }
}

// Sliced ELL, slice height 32, entries paired: entry k of row r lives at
// sptr[r/32] + 64 (k/2) + 2 (r%32) + k%2, so a thread loads the columns and values of two consecutive
// entries of its row with one 8-byte (columns, FP32 values) or 16-byte (FP64 values) load, and a warp's
// loads of one pair step are contiguous.  A slice of width w stores 2 ceil(w/2) entries per row; the
// padding holds value 0 and a valid column.
template <class T>
struct SellT {
  int n;
  const int* sptr;
  const int* col;
  const T* val;
};
using Sell = SellT<double>;

template <class T>
struct Pair;
template <>
struct Pair<double> {
  using type = double2;
};
template <>
struct Pair<float> {
  using type = float2;
};

template <class T>
__device__ __forceinline__ T sell_row(const SellT<T>& A, const T* __restrict__ x, int row) {
  const int s = row >> 5;
  const int b0 = __ldg(A.sptr + s);
  const int wp = (__ldg(A.sptr + s + 1) - b0) >> 6;
  const int base = b0 + 2 * (row & 31);
  T acc = T(0);
  for (int j = 0; j < wp; ++j) {
    const int2 c = __ldg(reinterpret_cast<const int2*>(A.col + base + 64 * j));
    const typename Pair<T>::type v = __ldg(reinterpret_cast<const typename Pair<T>::type*>(A.val + base + 64 * j));
    acc = fmaT<T>(v.x, __ldg(x + c.x), acc);
    acc = fmaT<T>(v.y, __ldg(x + c.y), acc);
  }
  return acc;
}

// Rows per thread of the one-row-per-thread kernels.  Each thread keeps ILP rows in flight (their
// loads are issued together), so a kernel over the fine level runs as one balanced wave instead of
// one full wave plus a short second one.
constexpr int ILP = 2;

// Non-zeros per lane loaded together in the compressed-row kernels: the column and value loads of KU
// entries are issued before their gathers; the sum runs over the entries in stored order, so the
// result does not depend on KU.  Measured on the 80 nm cube (GB300): KU = 4 made the PCG iteration
// ~15 % slower than KU = 1 (more registers, fewer resident warps), so 1 is kept.
constexpr int KU = 1;

// Entry pairs of a sliced-ELL row whose column and value loads are issued before their gathers: a
// row of 2 PF entries costs one chain (columns, then gathers) instead of PF chains.  The products
// are summed in stored order whatever PF is.
constexpr int PF = 1;

// x loads: read-only path (the vector is not written during the kernel) or L2 (written by other
// blocks of a persistent launch before the last grid barrier)
template <bool CG, class T>
__device__ __forceinline__ T ldx(const T* x, int c) {
  if constexpr (CG) return __ldcg(x + c);
  else return __ldg(x + c);
}

template <int R, bool CG, class T, class TX = T>
__device__ __forceinline__ void sell_rows_k(const int* __restrict__ sptr, const int* __restrict__ col,
                                            const T* __restrict__ val, int rlim, const TX* x, const int (&row)[R],
                                            T (&acc)[R]) {
  using P2 = typename Pair<T>::type;
  int base[R], wp[R];
  int wmax = 0;
#pragma unroll
  for (int q = 0; q < R; ++q) {
    acc[q] = T(0);
    wp[q] = 0;
    base[q] = 0;
    if (row[q] < rlim) {
      const int s = row[q] >> 5;
      const int b0 = __ldg(sptr + s);
      wp[q] = (__ldg(sptr + s + 1) - b0) >> 6;
      base[q] = b0 + 2 * (row[q] & 31);
    }
    wmax = max(wmax, wp[q]);
  }
  for (int j0 = 0; j0 < wmax; j0 += PF) {
    int2 c[R][PF];
    P2 v[R][PF];
#pragma unroll
    for (int q = 0; q < R; ++q)
#pragma unroll
      for (int u = 0; u < PF; ++u)
        if (j0 + u < wp[q]) {
          c[q][u] = __ldg(reinterpret_cast<const int2*>(col + base[q] + 64 * (j0 + u)));
          v[q][u] = __ldg(reinterpret_cast<const P2*>(val + base[q] + 64 * (j0 + u)));
        }
#pragma unroll
    for (int q = 0; q < R; ++q)
#pragma unroll
      for (int u = 0; u < PF; ++u)
        if (j0 + u < wp[q]) {
          const T x0 = (T)ldx<CG>(x, c[q][u].x), x1 = (T)ldx<CG>(x, c[q][u].y);
          acc[q] = fmaT<T>(v[q][u].x, x0, acc[q]);
          acc[q] = fmaT<T>(v[q][u].y, x1, acc[q]);
        }
  }
}

template <class T>
__device__ __forceinline__ void sell_rows(const SellT<T>& A, const T* __restrict__ x, const int (&row)[ILP],
                                          T (&acc)[ILP]) {
  sell_rows_k<ILP, false, T>(A.sptr, A.col, A.val, A.n, x, row, acc);
}
// row indices of thread threadIdx.x in the block-stride step starting at rb
__device__ __forceinline__ void rows_of(int rb, int (&row)[ILP]) {
#pragma unroll
  for (int q = 0; q < ILP; ++q) row[q] = rb + threadIdx.x + q * BS;
}
#define ROW_LOOP(n) for (int rb = blockIdx.x * BS * ILP; rb < (n); rb += gridDim.x * BS * ILP)

// compressed rows with TPR lanes per row (small levels with long rows, where one thread per row
// would leave most of the GPU idle)
template <class T>
struct CsrT {
  int n;
  const int* ptr;
  const int* col;
  const T* val;
};
using Csr = CsrT<double>;

template <int TPR, class T>
__device__ __forceinline__ T csr_row(const CsrT<T>& A, const T* __restrict__ x, int row, bool valid, int lane) {
  T acc = T(0);
  if (valid) {
    const int s = __ldg(A.ptr + row), e = __ldg(A.ptr + row + 1);
    for (int k = s + lane; k < e; k += KU * TPR) {
      int c[KU];
      T v[KU], xv[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u)
        if (k + u * TPR < e) {
          c[u] = __ldg(A.col + k + u * TPR);
          v[u] = __ldg(A.val + k + u * TPR);
        }
#pragma unroll
      for (int u = 0; u < KU; ++u)
        if (k + u * TPR < e) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < KU; ++u)
        if (k + u * TPR < e) acc = fmaT<T>(v[u], xv[u], acc);
    }
  }
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  return acc;
}

// mode 0: y = A x ; 1: y = b - A x ; 2: y = x + s .* (b - A x) ; 3: y = b + A x (prolongation)
template <int TPR, int MODE, class T>
__global__ void __launch_bounds__(BS) k_csr(CsrT<T> A, const T* __restrict__ x, const T* b, const T* __restrict__ s,
                                            T* y, const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < A.n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < A.n;
    const T ax = csr_row<TPR, T>(A, x, row, valid, lane);
    if (valid && lane == 0) {
      if (MODE == 0) y[row] = ax;
      else if (MODE == 1) y[row] = b[row] - ax;
      else if (MODE == 2) y[row] = x[row] + s[row] * (b[row] - ax);
      else y[row] = b[row] + ax;
    }
  }
}

// restriction with compressed rows, fused with the coarse pre-smoothing from zero
template <int TPR, class T>
__global__ void __launch_bounds__(BS) k_restrict_csr(CsrT<T> R, const T* __restrict__ res, T* __restrict__ bc,
                                                     const T* __restrict__ s_c, T* __restrict__ xc,
                                                     const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < R.n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < R.n;
    const T v = csr_row<TPR, T>(R, res, row, valid, lane);
    if (valid && lane == 0) {
      bc[row] = v;
      if (s_c) xc[row] = s_c[row] * v;
    }
  }
}

template <int MODE, class T>
__global__ void __launch_bounds__(BS) k_sell(SellT<T> A, const T* __restrict__ x, const T* b,
                                             const T* __restrict__ s, T* y, const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  ROW_LOOP(A.n) {
    int row[ILP];
    T ax[ILP];
    rows_of(rb, row);
    sell_rows<T>(A, x, row, ax);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      if (MODE == 0) y[i] = ax[q];
      else if (MODE == 1) y[i] = b[i] - ax[q];
      else if (MODE == 2) y[i] = x[i] + s[i] * (b[i] - ax[q]);
      else y[i] = b[i] + ax[q];
    }
  }
}

// r = b - A x ; r.r -> red[R_R2] ; xv = s .* r (level-0 pre-smoothing from zero)
template <class T>
__global__ void __launch_bounds__(BS) k_init_residual(SellT<T> A, const T* __restrict__ x, const T* __restrict__ b,
                                                      T* __restrict__ r, const T* __restrict__ s, T* __restrict__ xv,
                                                      Scalars* sc, double* part) {
  pdl_entry();
  Acc<T> acc;
  ROW_LOOP(A.n) {
    int row[ILP];
    T ax[ILP];
    rows_of(rb, row);
    sell_rows<T>(A, x, row, ax);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      const T ri = b[i] - ax[q];
      r[i] = ri;
      acc.add(ri, ri);
      if (s) xv[i] = s[i] * ri;
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_R2, -1, POST_R2_INIT);
}

// PCG direction update fused with the operator product:
//   y = A z ; p = z + beta p ; Ap = y + beta Ap ; p.Ap -> red[R_PAP]
// (A p_new = A z + beta A p_old, so the product is taken on z, complete before the launch)
template <class T>
__global__ void __launch_bounds__(BS) k_pcg_dir(SellT<T> A, const T* __restrict__ z, T* __restrict__ p,
                                                T* __restrict__ Ap, Scalars* sc, double* part) {
  pdl_entry();
  if (sc->done) return;
  const T beta = scal<T>(sc->beta, sc->beta_f);
  Acc<T> acc;
  ROW_LOOP(A.n) {
    int row[ILP];
    T az[ILP];
    rows_of(rb, row);
    sell_rows<T>(A, z, row, az);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      // first direction (beta = 0): p = z, Ap = A z, whatever p and Ap held before
      const T pn = beta != T(0) ? z[i] + beta * p[i] : z[i];
      const T apn = beta != T(0) ? az[q] + beta * Ap[i] : az[q];
      p[i] = pn;
      Ap[i] = apn;
      acc.add(pn, apn);
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_PAP, -1, POST_PAP);
}

// ------------------------------------------------------------------------------------------
// The FP64 operator split as a = hi + lo (hi = fl32(a), lo = fl32(a - hi)), sliced-ELL order of SellT,
// for products with FP32 vectors summed in float-float on the FP32 pipes: each entry adds hi z exactly
// (the product's rounding error is recovered with one FMA) and lo z rounded, so a row's sum carries an
// error of about 2^-47 sum |a z|, against 2^-53 in FP64, at 1/64 of the FP64 issue cost per entry.
// ------------------------------------------------------------------------------------------
struct SellDF {
  int n;
  const int* sptr;
  const int* col;
  const float* hi;
  const float* lo;
};

__global__ void k_split_df(int64_t n, const double* __restrict__ a, float* __restrict__ hi, float* __restrict__ lo) {
  for (int64_t i = blockIdx.x * (int64_t)BS + threadIdx.x; i < n; i += (int64_t)gridDim.x * BS) {
    const double v = a[i];
    const float h = (float)v;
    hi[i] = h;
    lo[i] = (float)(v - (double)h);
  }
}

// (sh, sl) += (hi + lo) z
__device__ __forceinline__ void df_madd(float hi, float lo, float z, float& sh, float& sl) {
  const float p = hi * z;
  float e = fmaf(hi, z, -p);  // hi z = p + e exactly
  e = fmaf(lo, z, e);
  float t, err;
  Acc<float>::two_sum(sh, p, t, err);
  sh = t;
  sl += err + e;
}

__device__ __forceinline__ void sell_rows_df(const SellDF& A, const float* __restrict__ z, const int (&row)[ILP],
                                             float (&sh)[ILP], float (&sl)[ILP]) {
  int base[ILP], wp[ILP];
  int wmax = 0;
#pragma unroll
  for (int q = 0; q < ILP; ++q) {
    sh[q] = 0.0f;
    sl[q] = 0.0f;
    wp[q] = 0;
    base[q] = 0;
    if (row[q] < A.n) {
      const int s = row[q] >> 5;
      const int b0 = __ldg(A.sptr + s);
      wp[q] = (__ldg(A.sptr + s + 1) - b0) >> 6;
      base[q] = b0 + 2 * (row[q] & 31);
    }
    wmax = max(wmax, wp[q]);
  }
  for (int j0 = 0; j0 < wmax; j0 += PF) {
    int2 c[ILP][PF];
    float2 vh[ILP][PF], vl[ILP][PF];
#pragma unroll
    for (int q = 0; q < ILP; ++q)
#pragma unroll
      for (int u = 0; u < PF; ++u)
        if (j0 + u < wp[q]) {
          const int e = base[q] + 64 * (j0 + u);
          c[q][u] = __ldg(reinterpret_cast<const int2*>(A.col + e));
          vh[q][u] = __ldg(reinterpret_cast<const float2*>(A.hi + e));
          vl[q][u] = __ldg(reinterpret_cast<const float2*>(A.lo + e));
        }
#pragma unroll
    for (int q = 0; q < ILP; ++q)
#pragma unroll
      for (int u = 0; u < PF; ++u)
        if (j0 + u < wp[q]) {
          df_madd(vh[q][u].x, vl[q][u].x, __ldg(z + c[q][u].x), sh[q], sl[q]);
          df_madd(vh[q][u].y, vl[q][u].y, __ldg(z + c[q][u].y), sh[q], sl[q]);
        }
  }
}

// k_pcg_dir of the FP64 PCG preconditioned by the FP32 V-cycle: the V-cycle's z is exactly FP32, so
// A z is taken with the split operator (FP32 pipes) and only the per-row updates run in FP64:
//   p = z + beta p ; Ap = A z + beta Ap ; p.Ap -> red[R_PAP]
__global__ void __launch_bounds__(BS) k_pcg_dir_df(SellDF A, const float* __restrict__ z, double* __restrict__ p,
                                                   double* __restrict__ Ap, Scalars* sc, double* part) {
  pdl_entry();
  if (sc->done) return;
  const double beta = sc->beta;
  Acc<double> acc;
  ROW_LOOP(A.n) {
    int row[ILP];
    float sh[ILP], sl[ILP];
    rows_of(rb, row);
    sell_rows_df(A, z, row, sh, sl);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      const double az = (double)sh[q] + (double)sl[q];
      const double zi = (double)z[i];
      const double pn = beta != 0.0 ? zi + beta * p[i] : zi;
      const double apn = beta != 0.0 ? az + beta * Ap[i] : az;
      p[i] = pn;
      Ap[i] = apn;
      acc.add(pn, apn);
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_PAP, -1, POST_PAP);
}

// x += alpha p ; r -= alpha Ap ; r.r -> red[R_R2] ; xv = s .* r
template <class T>
__global__ void __launch_bounds__(BS) k_pcg_step(int n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                                 const T* __restrict__ Ap, const T* __restrict__ s0, T* __restrict__ xv,
                                                 Scalars* sc, double* part) {
  pdl_entry();
  if (sc->done) return;
  const T alpha = scal<T>(sc->alpha, sc->alpha_f);
  Acc<T> acc;
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= n) continue;
      x[i] = x[i] + alpha * p[i];
      const T ri = r[i] - alpha * Ap[i];
      r[i] = ri;
      acc.add(ri, ri);
      if (s0) xv[i] = s0[i] * ri;
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_R2, -1, POST_R2_STEP);
}

// FP64 PCG preconditioned by the FP32 V-cycle: x += alpha p ; r -= alpha Ap (FP64) ; r.r -> red[R_R2] ;
// r32 = fl32(r) and xv = s0 .* r32, the FP32 V-cycle's input and its level-0 pre-smoothing
__global__ void __launch_bounds__(BS) k_pcg_step_mp(int n, double* __restrict__ x, double* __restrict__ r,
                                                    const double* __restrict__ p, const double* __restrict__ Ap,
                                                    const float* __restrict__ s0, float* __restrict__ r32,
                                                    float* __restrict__ xv, Scalars* sc, double* part) {
  pdl_entry();
  if (sc->done) return;
  const double alpha = sc->alpha;
  Acc<double> acc;
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= n) continue;
      x[i] = x[i] + alpha * p[i];
      const double ri = r[i] - alpha * Ap[i];
      r[i] = ri;
      acc.add(ri, ri);
      const float rf = (float)ri;
      r32[i] = rf;
      xv[i] = s0[i] * rf;
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_R2, -1, POST_R2_STEP);
}

// r32 = fl32(r), xv = s0 .* r32 (before the first V-cycle of a solve)
__global__ void __launch_bounds__(BS) k_split_mp(int n, const double* __restrict__ r, const float* __restrict__ s0,
                                                 float* __restrict__ r32, float* __restrict__ xv) {
  pdl_entry();
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
    const float rf = (float)r[i];
    r32[i] = rf;
    xv[i] = s0[i] * rf;
  }
}

// level-0 residual res = r - A xv (skipped once the solve has converged)
template <class T>
__global__ void __launch_bounds__(BS) k_vc_residual0(SellT<T> A, const T* __restrict__ xv, const T* __restrict__ r,
                                                     T* __restrict__ res, Scalars* sc) {
  pdl_entry();
  if (sc->done) return;
  ROW_LOOP(A.n) {
    int row[ILP];
    T ax[ILP];
    rows_of(rb, row);
    sell_rows<T>(A, xv, row, ax);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < A.n) res[row[q]] = r[row[q]] - ax[q];
  }
}

// restriction b_c = R res, fused with the coarse pre-smoothing from zero x_c = s_c .* b_c
template <class T>
__global__ void __launch_bounds__(BS) k_restrict(SellT<T> R, const T* __restrict__ res, T* __restrict__ bc,
                                                 const T* __restrict__ s_c, T* __restrict__ xc,
                                                 const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  ROW_LOOP(R.n) {
    int row[ILP];
    T v[ILP];
    rows_of(rb, row);
    sell_rows<T>(R, res, row, v);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= R.n) continue;
      bc[i] = v[q];
      if (s_c) xc[i] = s_c[i] * v[q];
    }
  }
}

// dense coarsest solve x = Ainv b (row-major n x n), one warp per row
template <class T>
__global__ void __launch_bounds__(BS) k_dense_mv(int n, const T* __restrict__ Ainv, const T* __restrict__ b,
                                                 T* __restrict__ x, const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  const int lane = threadIdx.x & 31;
  for (int row = blockIdx.x * (BS / 32) + threadIdx.x / 32; row < n; row += gridDim.x * (BS / 32)) {
    const T* a = Ainv + (size_t)row * n;
    T acc = T(0);
    for (int k = lane; k < n; k += 32) acc = fmaT<T>(a[k], b[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[row] = acc;
  }
}

// Fused coarse correction, first phase.  Block r < nc computes z_r = (Z b)_r for one row of the dense
// nc x n matrix Z = Ainv R (I - A S) with all its threads (fixed-order block sum) - these long dot
// products go first, so that they overlap the rest instead of forming the kernel's tail; blocks
// nc .. nc + gT compute t = T b with CA_LANES lanes per row of T (compressed rows of T = 2S - S A S on
// level L-2, several hundred entries each; a warp per row: eight lanes per row, with fewer FP64
// reduction steps but a quarter of the warps, made the 80 nm cube's kernel 20 -> 24 us slower).
// Both read only b, the restricted residual of level L-2.
// virtual block vb of nc + gT (the kernel's own block, or one of the one-launch coarse cycle's)
constexpr int CA_LANES = 32;

template <class T>
__device__ __forceinline__ void coarse_a_block(const CsrT<T>& Tm, const T* __restrict__ Z, const T* __restrict__ b,
                                               T* __restrict__ t, T* __restrict__ z, int gT, int nc, int vb) {
  const int n = Tm.n;
  if (vb >= nc) {
    constexpr int RPB = BS / CA_LANES;
    const int tb = vb - nc;
    const int lane = threadIdx.x % CA_LANES;
    for (int rb = tb * RPB; rb < n; rb += gT * RPB) {
      const int row = rb + threadIdx.x / CA_LANES;
      const bool valid = row < n;
      const T acc = csr_row<CA_LANES, T>(Tm, b, row, valid, lane);
      if (valid && lane == 0) t[row] = acc;
    }
  } else {
    const int r = vb;
    const T* zr = Z + (size_t)r * n;
    double acc = 0.0;
#pragma unroll 4
    for (int k = threadIdx.x; k < n; k += BS) acc = fma((double)__ldg(zr + k), (double)__ldg(b + k), acc);
    acc = block_sum(acc);
    if (threadIdx.x == 0) z[r] = (T)acc;
  }
}

template <class T>
__global__ void __launch_bounds__(BS) k_coarse_a(CsrT<T> Tm, const T* __restrict__ Z, int nc, const T* __restrict__ b,
                                                 T* __restrict__ t, T* __restrict__ z, int gT,
                                                 const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  coarse_a_block<T>(Tm, Z, b, t, z, gT, nc, (int)blockIdx.x);
}

// Fused coarse correction, second phase: x2 = t + W z (W dense n x nc, row-major, W = (I - S A) P),
// CB_LANES lanes per row (a row of ~250 entries: 31 multiply-adds per lane and three shuffle levels,
// where a warp per row spent as many FP64 issue slots on its five-level reduction as on the row).
// x2 is level L-2's post-smoothed iterate, exactly as the V-cycle's levels L-2 .. L-1 would leave it
// (same linear map, summed in a different order).
constexpr int CB_LANES = 8;

template <class T>
__device__ __forceinline__ void coarse_b_rows(int n, int nc, const T* __restrict__ W, const T* __restrict__ t,
                                              const T* __restrict__ z, T* __restrict__ x2, int vb, int nvb) {
  constexpr int RPB = BS / CB_LANES;
  const int q = threadIdx.x % CB_LANES;
  for (int rb = vb * RPB; rb < n; rb += nvb * RPB) {
    const int row = rb + threadIdx.x / CB_LANES;
    T acc = T(0);
    if (row < n) {
      const T* wr = W + (size_t)row * nc;
#pragma unroll 4
      for (int k = q; k < nc; k += CB_LANES) acc = fmaT<T>(__ldg(wr + k), __ldg(z + k), acc);
    }
#pragma unroll
    for (int o = CB_LANES / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (row < n && q == 0) x2[row] = __ldg(t + row) + acc;
  }
}

template <class T>
__global__ void __launch_bounds__(BS) k_coarse_b(int n, int nc, const T* __restrict__ W, const T* __restrict__ t,
                                                 const T* __restrict__ z, T* __restrict__ x2,
                                                 const int* __restrict__ done) {
  pdl_entry();
  if (done && *done) return;
  coarse_b_rows<T>(n, nc, W, t, z, x2, (int)blockIdx.x, (int)gridDim.x);
}

// ------------------------------------------------------------------------------------------
// The V-cycle's levels 1 .. 3 of a four-level hierarchy in one cooperative launch (fused restriction
// at level 1, fused coarse correction on levels 2 .. 3): b2 = Rf1 b1 | t = T b2, z = Z b2 |
// x2_2 = t + W z | x1 += P1 x2_2 | x2_1 = x1 + s1 (b1 - A1 x1), five stages separated by grid
// barriers instead of five launches.  Every row is computed exactly as by the separate kernels (same
// lanes per row, same order), so the V-cycle's result is bit-identical.
// ------------------------------------------------------------------------------------------
struct GridBar {
  unsigned arrive;  // blocks arrived at the current barrier
  unsigned gen;     // barrier generation
};

// all blocks of the (co-resident, cooperative) grid meet; a wait is bounded: after ~2^22 polls the
// block records the failure in sc->bar_err and goes on (later barriers then do not wait at all), so
// a lost block cannot hang the GPU; the host turns the flag into an error
__device__ __forceinline__ void grid_sync(GridBar* bar, Scalars* sc) {
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(bar->gen), arrive(bar->arrive);
    cuda::atomic_ref<int, cuda::thread_scope_device> err(sc->bar_err);
    const unsigned g = gen.load(cuda::memory_order_relaxed);
    __threadfence();
    if (arrive.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
      arrive.store(0u, cuda::memory_order_relaxed);
      gen.store(g + 1u, cuda::memory_order_release);
    } else if (err.load(cuda::memory_order_relaxed) == 0) {
      unsigned polls = 0;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if (++polls > (1u << 22)) {
          err.store(1, cuda::memory_order_relaxed);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <int TPR, int MODE, class T>
__device__ __forceinline__ void csr_rows(const CsrT<T>& A, const T* __restrict__ x, const T* b,
                                         const T* __restrict__ s, T* y, int vb, int nvb) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = vb * RPB; rb < A.n; rb += nvb * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < A.n;
    const T ax = csr_row<TPR, T>(A, x, row, valid, lane);
    if (valid && lane == 0) {
      if (MODE == 0) y[row] = ax;                                    // restriction into b
      else if (MODE == 2) y[row] = x[row] + s[row] * (b[row] - ax);  // post-smoothing
      else y[row] = b[row] + ax;                                     // prolongation
    }
  }
}

template <int MODE, class T>
__device__ __forceinline__ void csr_rows_tpr(int tpr, const CsrT<T>& A, const T* __restrict__ x, const T* b,
                                             const T* __restrict__ s, T* y) {
  const int vb = blockIdx.x, nvb = gridDim.x;
  switch (tpr) {
    case 2: csr_rows<2, MODE, T>(A, x, b, s, y, vb, nvb); break;
    case 4: csr_rows<4, MODE, T>(A, x, b, s, y, vb, nvb); break;
    case 8: csr_rows<8, MODE, T>(A, x, b, s, y, vb, nvb); break;
    case 16: csr_rows<16, MODE, T>(A, x, b, s, y, vb, nvb); break;
    default: csr_rows<32, MODE, T>(A, x, b, s, y, vb, nvb); break;
  }
}

template <class T>
struct CoarseCycle {
  CsrT<T> Rf1, P1, A1, Tm;
  int tpr_rf1, tpr_p1, tpr_a1;
  const T* b1;  // level-1 right-hand side (the restricted level-0 residual)
  T* x1;        // level-1 iterate (pre-smoothed s1 b1 on entry)
  const T* s1;
  T* x2_1;      // level-1 post-smoothed iterate (the prolongation's input on level 0)
  T* b2;
  const T *Z, *W;
  int nc, gT;
  T *tvec, *zvec, *x2_2;
};

template <class T>
__global__ void __launch_bounds__(BS) k_coarse_cycle(CoarseCycle<T> c, GridBar* bar, Scalars* sc,
                                                     const int* __restrict__ done) {
  if (done && *done) return;  // uniform: every block reads the same flag, set before this launch
  csr_rows_tpr<0, T>(c.tpr_rf1, c.Rf1, c.b1, nullptr, nullptr, c.b2);
  grid_sync(bar, sc);
  for (int vb = blockIdx.x; vb < c.gT + c.nc; vb += gridDim.x)
    coarse_a_block<T>(c.Tm, c.Z, c.b2, c.tvec, c.zvec, c.gT, c.nc, vb);
  grid_sync(bar, sc);
  coarse_b_rows<T>(c.Tm.n, c.nc, c.W, c.tvec, c.zvec, c.x2_2, (int)blockIdx.x, (int)gridDim.x);
  grid_sync(bar, sc);
  csr_rows_tpr<3, T>(c.tpr_p1, c.P1, c.x2_2, c.x1, nullptr, c.x1);
  grid_sync(bar, sc);
  csr_rows_tpr<2, T>(c.tpr_a1, c.A1, c.x1, c.b1, c.s1, c.x2_1);
}

// post-smoothing y = x + s .* (b - A x); with `part` it also reduces b.y into red[R_RZ]
// (level 0: b = r and y = z)
template <class T>
// y64 (may be null): y also widened to FP64 (the FP32 preconditioner's output for the FP64 PCG: N
// conversions here instead of one per stored entry in the next FP64 product)
__global__ void __launch_bounds__(BS) k_smooth_dot(SellT<T> A, const T* __restrict__ x, const T* __restrict__ b,
                                                   const T* __restrict__ s, T* __restrict__ y, Scalars* sc,
                                                   double* part, const int* __restrict__ done,
                                                   double* __restrict__ y64) {
  pdl_entry();
  if (done && *done) return;
  Acc<T> acc;
  ROW_LOOP(A.n) {
    int row[ILP];
    T ax[ILP];
    rows_of(rb, row);
    sell_rows<T>(A, x, row, ax);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      const T yi = x[i] + s[i] * (b[i] - ax[q]);
      y[i] = yi;
      if (y64) y64[i] = (double)yi;
      acc.add(b[i], yi);
    }
  }
  if (part) grid_finish(block_total(acc), 0.0, sc, part, R_RZ, -1, POST_RZ);
}

// condition of the graph's WHILE node: keep looping until done (bounded by maxiter + 2 trips)
__global__ void k_set_cond(cudaGraphConditionalHandle hnd, Scalars* sc) {
  pdl_entry();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    sc->loops += 1;
    const bool more = !sc->done && sc->loops <= sc->maxiter + 2;
    cudaGraphSetConditional(hnd, more ? 1u : 0u);
  }
}

// ------------------------------------------------------------------------------------------
// vector kernels
// ------------------------------------------------------------------------------------------
// x.y (y == nullptr: x.x) -> red[slot], accumulated in FP64
template <class T>
__global__ void __launch_bounds__(BS) k_dot(int n, const T* __restrict__ x, const T* __restrict__ y, Scalars* sc,
                                            double* part, int slot, int post = POST_NONE) {
  pdl_entry();
  Acc<T> acc;
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < n) acc.add(x[row[q]], y ? y[row[q]] : x[row[q]]);
  }
  grid_finish(block_total(acc), 0.0, sc, part, slot, -1, post);
}

// mean of x -> red[slot]
__global__ void __launch_bounds__(BS) k_mean(int n, const double* __restrict__ x, Scalars* sc, double* part, int slot) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) d += x[i];
  grid_reduce(d, 0.0, sc, part, slot, -1, POST_MEAN, (double)n);
}

// x -= red[slot] (a mean computed by k_mean)
__global__ void __launch_bounds__(BS) k_sub_mean(int n, double* __restrict__ x, const Scalars* sc, int slot) {
  const double mean = sc->red[slot];
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) x[i] = x[i] - mean;
}

// out = s .* r
template <class T>
__global__ void __launch_bounds__(BS) k_mul(int n, const T* __restrict__ s, const T* __restrict__ r,
                                            T* __restrict__ out) {
  pdl_entry();
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < n) out[row[q]] = s[row[q]] * r[row[q]];
  }
}

// PCG start: tol2 = tol^2 * red[R_BB]; counters reset
__global__ void k_pcg_init_scalars(Scalars* sc, double tol, int maxiter) {
  pdl_entry();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    sc->tol2 = tol * tol * sc->red[R_BB];
    sc->it = 0;
    sc->done = 0;
    sc->loops = 0;
    sc->maxiter = maxiter;
    sc->rz = 0.0;
    sc->rz_valid = 0;
    sc->alpha = sc->beta = 0.0;
    sc->alpha_f = sc->beta_f = 0.0f;
  }
}

// ------------------------------------------------------------------------------------------
// mixed-precision iterative refinement (FP64 outer residual, FP32 inner correction solve)
// ------------------------------------------------------------------------------------------
// r = b - A x in FP64; r.r -> red[R_R2]
__global__ void __launch_bounds__(BS) k_resid64(Sell A, const double* __restrict__ x, const double* __restrict__ b,
                                                double* __restrict__ r, Scalars* sc, double* part) {
  pdl_entry();
  Acc<double> acc;
  ROW_LOOP(A.n) {
    int row[ILP];
    double ax[ILP];
    rows_of(rb, row);
    sell_rows<double>(A, x, row, ax);
#pragma unroll
    for (int q = 0; q < ILP; ++q) {
      const int i = row[q];
      if (i >= A.n) continue;
      const double ri = b[i] - ax[q];
      r[i] = ri;
      acc.add(ri, ri);
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_R2);
}

// r32 = r * scale (the inner system is solved for a unit-norm right-hand side); d32 = 0
__global__ void __launch_bounds__(BS) k_to_f32(int n, const double* __restrict__ r, double scale,
                                               float* __restrict__ r32, float* __restrict__ d32) {
  pdl_entry();
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < n) {
        r32[row[q]] = (float)(r[row[q]] * scale);
        d32[row[q]] = 0.0f;
      }
  }
}

// x += scale * d32 in FP64
__global__ void __launch_bounds__(BS) k_add_f32(int n, double* __restrict__ x, const float* __restrict__ d32,
                                                double scale) {
  pdl_entry();
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < n) x[row[q]] = fma(scale, (double)d32[row[q]], x[row[q]]);
  }
}

// ------------------------------------------------------------------------------------------
// energy, local Hessian and demag source over the magnetic rows (TPR lanes per row)
// ------------------------------------------------------------------------------------------
struct EnergyDev {
  int n_rows;
  const int* rows;
  const int* ptr;
  const int* col;
  const int* mat;       // material per entry (multi-axis meshes only)
  const double* w;
  const double* q;
  const double* gx;
  const double* gy;
  const double* gz;
  const double* dx;
  const double* dy;
  const double* dz;
  const double* kax;    // (n_mat, 3) easy axes
  const double* mex;    // magnetoelastic entries on m_x, m_y (null: no magnetoelastic term)
  const double* mey;
  int single_axis;
  int axis0;            // material whose axis every entry uses when single_axis
};

template <int TPR>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int TPR>
__device__ __forceinline__ void exch_aniso_row(const EnergyDev& op, int r, bool valid, int lane,
                                               const double* __restrict__ v, double& ax, double& ay, double& az) {
  ax = ay = az = 0.0;
  if (valid) {
    const int s = op.ptr[r], e = op.ptr[r + 1];
    double kx = 0, ky = 0, kz = 0;
    if (op.single_axis) {
      kx = op.kax[3 * op.axis0];
      ky = op.kax[3 * op.axis0 + 1];
      kz = op.kax[3 * op.axis0 + 2];
    }
    for (int k = s + lane; k < e; k += TPR) {
      const int j = op.col[k];
      if (!op.single_axis) {
        const int g = op.mat[k];
        kx = op.kax[3 * g];
        ky = op.kax[3 * g + 1];
        kz = op.kax[3 * g + 2];
      }
      const double vx = __ldg(v + 3 * j), vy = __ldg(v + 3 * j + 1), vz = __ldg(v + 3 * j + 2);
      const double wk = op.w[k];
      const double t = -op.q[k] * (kx * vx + ky * vy + kz * vz);
      ax += wk * vx + t * kx;
      ay += wk * vy + t * ky;
      az += wk * vz + t * kz;
      if (op.mex) {
        ax += op.mex[k] * vx;
        ay += op.mey[k] * vy;
      }
    }
  }
  ax = group_sum<TPR>(ax);
  ay = group_sum<TPR>(ay);
  az = group_sum<TPR>(az);
}

// ------------------------------------------------------------------------------------------
// The energy operator in sliced-ELL order, one thread per magnetic row.  On this part a warp-wide
// FP64 instruction costs 16 SM cycles whatever its active lanes, so lanes-per-row kernels over the
// compressed rows (kept above only for the allocation-free entry point) spend most of their FP64
// issue on idle lanes, shuffle reductions and a one-lane epilogue; here every FP64 instruction does
// useful work for 32 rows and the loads are coalesced across the warp.
// ------------------------------------------------------------------------------------------
// Slices of 32 rows: entry k of lane l of slice s at sptr[s] + 32 k + l; padding entries carry zero
// values and the row's own node as column (the per-node arrays are only read, never indexed out of
// range).
struct EnergySell {
  int n_rows;
  const int* rows;
  const int* sptr;
  const int* col;
  const int* mat;
  const double* w;
  const double* q;
  const double* gx;
  const double* gy;
  const double* gz;
  const double* dx;
  const double* dy;
  const double* dz;
  const double* kax;
  const double* mex;  // null: no magnetoelastic term
  const double* mey;
  int single_axis;
  int axis0;
};

// (exchange + anisotropy + magnetoelastic) v on row r: sum_k w v_j - q (k.v_j) k (+ mex v_j,x, mey v_j,y);
// with a single easy axis the anisotropy sum is accumulated as a scalar and applied once
__device__ __forceinline__ void exch_aniso_sell(const EnergySell& op, int r, const double* __restrict__ v,
                                                double& ax, double& ay, double& az) {
  const int s = r >> 5, l = r & 31;
  const int base = __ldg(op.sptr + s), wd = (__ldg(op.sptr + s + 1) - base) >> 5;
  ax = ay = az = 0.0;
  if (op.single_axis) {
    const double kx = op.kax[3 * op.axis0], ky = op.kax[3 * op.axis0 + 1], kz = op.kax[3 * op.axis0 + 2];
    double t = 0.0;
#pragma unroll 3
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const int j = __ldg(op.col + at);
      const double vx = __ldg(v + 3 * j), vy = __ldg(v + 3 * j + 1), vz = __ldg(v + 3 * j + 2);
      const double wk = __ldg(op.w + at);
      ax = fma(wk, vx, ax);
      ay = fma(wk, vy, ay);
      az = fma(wk, vz, az);
      t = fma(__ldg(op.q + at), fma(kz, vz, fma(ky, vy, kx * vx)), t);
      if (op.mex) {
        ax = fma(__ldg(op.mex + at), vx, ax);
        ay = fma(__ldg(op.mey + at), vy, ay);
      }
    }
    ax = fma(-t, kx, ax);
    ay = fma(-t, ky, ay);
    az = fma(-t, kz, az);
  } else {
#pragma unroll 2
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const int j = __ldg(op.col + at);
      const int g = __ldg(op.mat + at);
      const double kx = op.kax[3 * g], ky = op.kax[3 * g + 1], kz = op.kax[3 * g + 2];
      const double vx = __ldg(v + 3 * j), vy = __ldg(v + 3 * j + 1), vz = __ldg(v + 3 * j + 2);
      const double wk = __ldg(op.w + at);
      const double t = -__ldg(op.q + at) * fma(kz, vz, fma(ky, vy, kx * vx));
      ax = fma(t, kx, fma(wk, vx, ax));
      ay = fma(t, ky, fma(wk, vy, ay));
      az = fma(t, kz, fma(wk, vz, az));
      if (op.mex) {
        ax = fma(__ldg(op.mex + at), vx, ax);
        ay = fma(__ldg(op.mey + at), vy, ay);
      }
    }
  }
}

// g = (K m + G U + g_z) / V_mag on the magnetic rows; m.(g_quad + 2 g_z) -> red[R_E]
__global__ void __launch_bounds__(BS) k_energy_grad_s(EnergySell op, const double* __restrict__ m,
                                                      const double* __restrict__ U, const double* __restrict__ Mn,
                                                      double Bx, double By, double Bz, const double* __restrict__ Bd,
                                                      const double* __restrict__ Bbias, double inv_Vmag,
                                                      double* __restrict__ g, Scalars* sc, double* part) {
  if (Bd) {  // the applied field from device memory (a graph replayed for several fields)
    Bx = Bd[0];
    By = Bd[1];
    Bz = Bd[2];
  }
  double en = 0.0;
  for (int r = blockIdx.x * BS + threadIdx.x; r < op.n_rows; r += gridDim.x * BS) {
    double ax, ay, az;
    exch_aniso_sell(op, r, m, ax, ay, az);
    const int s = r >> 5, l = r & 31;
    const int base = __ldg(op.sptr + s), wd = (__ldg(op.sptr + s + 1) - base) >> 5;
    double ux = 0, uy = 0, uz = 0;
#pragma unroll 3
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const double u = __ldg(U + __ldg(op.col + at));
      ux = fma(__ldg(op.gx + at), u, ux);
      uy = fma(__ldg(op.gy + at), u, uy);
      uz = fma(__ldg(op.gz + at), u, uz);
    }
    const int a = __ldg(op.rows + r);
    double bx = Bx, by = By, bz = Bz;
    if (Bbias) {
      bx += Bbias[3 * a];
      by += Bbias[3 * a + 1];
      bz += Bbias[3 * a + 2];
    }
    const double mn = -2.0 * Mn[a];
    const double zx = mn * bx, zy = mn * by, zz = mn * bz;
    const double gx = (ax + ux) + zx, gy = (ay + uy) + zy, gz = (az + uz) + zz;
    en += m[3 * a] * (gx + zx) + m[3 * a + 1] * (gy + zy) + m[3 * a + 2] * (gz + zz);
    g[3 * a] = gx * inv_Vmag;
    g[3 * a + 1] = gy * inv_Vmag;
    g[3 * a + 2] = gz * inv_Vmag;
  }
  grid_reduce(en, 0.0, sc, part, R_E);
}

// out = C v / V_mag on the magnetic rows
__global__ void __launch_bounds__(BS) k_local_grad_s(EnergySell op, const double* __restrict__ v, double inv_Vmag,
                                                     double* __restrict__ out) {
  for (int r = blockIdx.x * BS + threadIdx.x; r < op.n_rows; r += gridDim.x * BS) {
    double ax, ay, az;
    exch_aniso_sell(op, r, v, ax, ay, az);
    const int a = __ldg(op.rows + r);
    out[3 * a] = ax * inv_Vmag;
    out[3 * a + 1] = ay * inv_Vmag;
    out[3 * a + 2] = az * inv_Vmag;
  }
}

// Pp = C p - (m.Cp) m - (m.g_ext) p + reg p on the magnetic rows; p.Pp -> red[slot]
__global__ void __launch_bounds__(BS) k_apply_P_s(EnergySell op, const double* __restrict__ m,
                                                  const double* __restrict__ gext, const double* __restrict__ p,
                                                  double reg, double inv_Vmag, double* __restrict__ Ap, Scalars* sc,
                                                  double* part, int slot) {
  double d = 0.0;
  for (int r = blockIdx.x * BS + threadIdx.x; r < op.n_rows; r += gridDim.x * BS) {
    double ax, ay, az;
    exch_aniso_sell(op, r, p, ax, ay, az);
    const int a = __ldg(op.rows + r);
    const double cx = ax * inv_Vmag, cy = ay * inv_Vmag, cz = az * inv_Vmag;
    const double mx = m[3 * a], my = m[3 * a + 1], mz = m[3 * a + 2];
    const double mc = mx * cx + my * cy + mz * cz;
    const double mg = mx * gext[3 * a] + my * gext[3 * a + 1] + mz * gext[3 * a + 2];
    const double px = p[3 * a], py = p[3 * a + 1], pz = p[3 * a + 2];
    const double ox = cx - mc * mx - mg * px + reg * px;
    const double oy = cy - mc * my - mg * py + reg * py;
    const double oz = cz - mc * mz - mg * pz + reg * pz;
    Ap[3 * a] = ox;
    Ap[3 * a + 1] = oy;
    Ap[3 * a + 2] = oz;
    d += px * ox + py * oy + pz * oz;
  }
  grid_reduce(d, 0.0, sc, part, slot);
}

// b = D m on the magnetic rows (other rows untouched)
__global__ void __launch_bounds__(BS) k_rhs_s(EnergySell op, const double* __restrict__ m, double* __restrict__ b) {
  for (int r = blockIdx.x * BS + threadIdx.x; r < op.n_rows; r += gridDim.x * BS) {
    const int s = r >> 5, l = r & 31;
    const int base = __ldg(op.sptr + s), wd = (__ldg(op.sptr + s + 1) - base) >> 5;
    double acc = 0.0;
#pragma unroll 3
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const int j = __ldg(op.col + at);
      acc += __ldg(op.dx + at) * __ldg(m + 3 * j) + __ldg(op.dy + at) * __ldg(m + 3 * j + 1) +
             __ldg(op.dz + at) * __ldg(m + 3 * j + 2);
    }
    b[__ldg(op.rows + r)] = acc;
  }
}

// ------------------------------------------------------------------------------------------
// Energy and gradient in float-float for the mixed-precision problems (one easy axis, no magnetoelastic
// term).  Every stored FP64 value a is kept as the pair (fl32(a), fl32(a - fl32(a))), and so are the
// vectors m, U and s = k.m; each product adds hi*hi exactly (TwoProd, one FMA) plus the two cross
// terms, and a row's sums are float-float (TwoSum), all on the FP32 pipes: about 2^-48 of the row's
// sum of |terms| against 2^-53 in FP64.  The row totals, the Zeeman term, the gradient and the energy
// sum are FP64, as in k_energy_grad_s.
// ------------------------------------------------------------------------------------------
struct EnergySellFF {
  int n_rows;
  const int* rows;
  const int* sptr;
  const int* col;
  const float4* wq;   // (w_hi, w_lo, q_hi, q_lo) in the sliced order of EnergySell
  const float4* gxy;  // (gx_hi, gx_lo, gy_hi, gy_lo)
  const float2* gz;   // (gz_hi, gz_lo)
  double kx, ky, kz;  // the easy axis
  float2 kfx, kfy, kfz;  // and its float-float pairs
  int n_touched;         // nodes that magnetic rows read (their columns), the only ones split
  const int* touched;
};

// the float-float node values an entry gathers, in three records (three gathers per entry)
struct NodesFF {
  float4* hi;  // (mx, my, mz, k.m) high parts
  float4* lo;  // their low parts
  float2* u;   // (U_hi, U_lo)
};

// (sh, sl) += (ah + al) (bh + bl), the al bl term dropped
__device__ __forceinline__ void ff_madd(float ah, float al, float bh, float bl, float& sh, float& sl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  float t, err;
  Acc<float>::two_sum(sh, p, t, err);
  sh = t;
  sl += err + e;
}

__device__ __forceinline__ float2 ff_split(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

// (sh, sl) = (ah + al) + (bh + bl)
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float& sh, float& sl) {
  float t, err;
  Acc<float>::two_sum(ah, bh, t, err);
  sh = t;
  sl = (al + bl) + err;
}

// the float-float pairs of m, of s = k.m (formed in FP64 as the FP64 kernel forms k.v) and of U, for
// the nodes the magnetic rows read
__global__ void __launch_bounds__(BS) k_split_ff(int n, const int* __restrict__ nodes, const double* __restrict__ m,
                                                 const double* __restrict__ U, double kx, double ky, double kz,
                                                 NodesFF nf) {
  for (int t = blockIdx.x * BS + threadIdx.x; t < n; t += gridDim.x * BS) {
    const int i = __ldg(nodes + t);
    const double x = m[3 * i], y = m[3 * i + 1], z = m[3 * i + 2];
    const float2 a = ff_split(x), b = ff_split(y), c = ff_split(z), s = ff_split(fma(kz, z, fma(ky, y, kx * x)));
    nf.hi[i] = make_float4(a.x, b.x, c.x, s.x);
    nf.lo[i] = make_float4(a.y, b.y, c.y, s.y);
    nf.u[i] = ff_split(U[i]);
  }
}

// (sh, sl) += (h2, l2) from the lane `o` places down
__device__ __forceinline__ void ff_shfl_add(float& sh, float& sl, int o) {
  const float h2 = __shfl_down_sync(0xffffffffu, sh, o);
  const float l2 = __shfl_down_sync(0xffffffffu, sl, o);
  float t, err;
  Acc<float>::two_sum(sh, h2, t, err);
  sh = t;
  sl += err + l2;
}

// g = (K m + G U + g_z) / V_mag on the magnetic rows; m.(g_quad + 2 g_z) -> red[R_E] (FP64).
// TPR lanes per row (133k magnetic rows would give one thread per row too few warps to hide the
// gather latency): lane q takes entries q, q + TPR, ..., and the row's float-float sums are merged
// over its lanes by a fixed shuffle tree (FP32 shuffles and adds), so the result is deterministic.
template <int TPR>
__global__ void __launch_bounds__(BS) k_energy_grad_ff(EnergySellFF op, const float4* __restrict__ nh,
                                                       const float4* __restrict__ nl, const float2* __restrict__ nu,
                                                       const double* __restrict__ m, const double* __restrict__ Mn,
                                                       double Bx, double By, double Bz, const double* __restrict__ Bd,
                                                       const double* __restrict__ Bbias, double inv_Vmag,
                                                       double* __restrict__ g, Scalars* sc, double* part) {
  static_assert(TPR >= 1 && TPR <= 32 && (TPR & (TPR - 1)) == 0, "TPR: a power of two up to 32");
  if (Bd) {
    Bx = Bd[0];
    By = Bd[1];
    Bz = Bd[2];
  }
  constexpr int RPB = BS / TPR;
  const int q = threadIdx.x % TPR;
  double en = 0.0;
  for (int rb = blockIdx.x * RPB; rb < op.n_rows; rb += gridDim.x * RPB) {
    const int r = rb + threadIdx.x / TPR;
    const bool valid = r < op.n_rows;
    float axh = 0.f, axl = 0.f, ayh = 0.f, ayl = 0.f, azh = 0.f, azl = 0.f, th = 0.f, tl = 0.f;
    float uxh = 0.f, uxl = 0.f, uyh = 0.f, uyl = 0.f, uzh = 0.f, uzl = 0.f;
    if (valid) {
      const int s = r >> 5, l = r & 31;
      const int base = __ldg(op.sptr + s), wd = (__ldg(op.sptr + s + 1) - base) >> 5;
#pragma unroll 2
      for (int k = q; k < wd; k += TPR) {
        const int at = base + (k << 5) + l;
        const int j = __ldg(op.col + at);
        const float4 wq = __ldg(op.wq + at), gxy = __ldg(op.gxy + at);
        const float2 gz = __ldg(op.gz + at);
        const float4 h = __ldg(nh + j), o = __ldg(nl + j);
        const float2 u = __ldg(nu + j);
        ff_madd(wq.x, wq.y, h.x, o.x, axh, axl);
        ff_madd(wq.x, wq.y, h.y, o.y, ayh, ayl);
        ff_madd(wq.x, wq.y, h.z, o.z, azh, azl);
        ff_madd(wq.z, wq.w, h.w, o.w, th, tl);
        ff_madd(gxy.x, gxy.y, u.x, u.y, uxh, uxl);
        ff_madd(gxy.z, gxy.w, u.x, u.y, uyh, uyl);
        ff_madd(gz.x, gz.y, u.x, u.y, uzh, uzl);
      }
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) {
      ff_shfl_add(axh, axl, o);
      ff_shfl_add(ayh, ayl, o);
      ff_shfl_add(azh, azl, o);
      ff_shfl_add(th, tl, o);
      ff_shfl_add(uxh, uxl, o);
      ff_shfl_add(uyh, uyl, o);
      ff_shfl_add(uzh, uzl, o);
    }
    if (valid && q == 0) {
      // a - t k and then + u in float-float; one widening per component (the FP64 pipe issues a
      // warp-wide instruction in 16 cycles whatever its active lanes)
      ff_madd(-th, -tl, op.kfx.x, op.kfx.y, axh, axl);
      ff_madd(-th, -tl, op.kfy.x, op.kfy.y, ayh, ayl);
      ff_madd(-th, -tl, op.kfz.x, op.kfz.y, azh, azl);
      ff_add(axh, axl, uxh, uxl, axh, axl);
      ff_add(ayh, ayl, uyh, uyl, ayh, ayl);
      ff_add(azh, azl, uzh, uzl, azh, azl);
      const double ax = (double)axh + (double)axl, ay = (double)ayh + (double)ayl, az = (double)azh + (double)azl;
      const int a = __ldg(op.rows + r);
      double bx = Bx, by = By, bz = Bz;
      if (Bbias) {
        bx += Bbias[3 * a];
        by += Bbias[3 * a + 1];
        bz += Bbias[3 * a + 2];
      }
      const double mn = -2.0 * Mn[a];
      const double zx = mn * bx, zy = mn * by, zz = mn * bz;
      const double gxr = ax + zx, gyr = ay + zy, gzr = az + zz;
      en += m[3 * a] * (gxr + zx) + m[3 * a + 1] * (gyr + zy) + m[3 * a + 2] * (gzr + zz);
      g[3 * a] = gxr * inv_Vmag;
      g[3 * a + 1] = gyr * inv_Vmag;
      g[3 * a + 2] = gzr * inv_Vmag;
    }
  }
  grid_reduce(en, 0.0, sc, part, R_E);
}

// ------------------------------------------------------------------------------------------
// The minimizer's inner preconditioner solve (the local Hessian P y = g by Steihaug PCG) in FP32, for
// the mixed-precision problems: FP32 copies of the exchange and anisotropy entries in the sliced
// order, FP32 vectors, inner products accumulated in float-float and reduced in FP64.  The energy,
// the gradient, the outer iteration and the line search stay FP64.
// ------------------------------------------------------------------------------------------
struct EnergySell32 {
  int n_rows;
  const int* rows;
  const int* sptr;
  const int* col;
  const int* mat;
  const float* w;
  const float* q;
  const float* kax;   // (n_mat, 3) easy axes
  const float* mex;   // null: no magnetoelastic term
  const float* mey;
  int single_axis;
  int axis0;
};

__device__ __forceinline__ void exch_aniso_sell32(const EnergySell32& op, int r, const float* __restrict__ v,
                                                  float& ax, float& ay, float& az) {
  const int s = r >> 5, l = r & 31;
  const int base = __ldg(op.sptr + s), wd = (__ldg(op.sptr + s + 1) - base) >> 5;
  ax = ay = az = 0.0f;
  if (op.single_axis) {
    const float kx = op.kax[3 * op.axis0], ky = op.kax[3 * op.axis0 + 1], kz = op.kax[3 * op.axis0 + 2];
    float t = 0.0f;
#pragma unroll 3
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const int j = __ldg(op.col + at);
      const float vx = __ldg(v + 3 * j), vy = __ldg(v + 3 * j + 1), vz = __ldg(v + 3 * j + 2);
      const float wk = __ldg(op.w + at);
      ax = fmaf(wk, vx, ax);
      ay = fmaf(wk, vy, ay);
      az = fmaf(wk, vz, az);
      t = fmaf(__ldg(op.q + at), fmaf(kz, vz, fmaf(ky, vy, kx * vx)), t);
      if (op.mex) {
        ax = fmaf(__ldg(op.mex + at), vx, ax);
        ay = fmaf(__ldg(op.mey + at), vy, ay);
      }
    }
    ax = fmaf(-t, kx, ax);
    ay = fmaf(-t, ky, ay);
    az = fmaf(-t, kz, az);
  } else {
#pragma unroll 2
    for (int k = 0; k < wd; ++k) {
      const int at = base + (k << 5) + l;
      const int j = __ldg(op.col + at);
      const int g = __ldg(op.mat + at);
      const float kx = op.kax[3 * g], ky = op.kax[3 * g + 1], kz = op.kax[3 * g + 2];
      const float vx = __ldg(v + 3 * j), vy = __ldg(v + 3 * j + 1), vz = __ldg(v + 3 * j + 2);
      const float wk = __ldg(op.w + at);
      const float t = -__ldg(op.q + at) * fmaf(kz, vz, fmaf(ky, vy, kx * vx));
      ax = fmaf(t, kx, fmaf(wk, vx, ax));
      ay = fmaf(t, ky, fmaf(wk, vy, ay));
      az = fmaf(t, kz, fmaf(wk, vz, az));
      if (op.mex) {
        ax = fmaf(__ldg(op.mex + at), vx, ax);
        ay = fmaf(__ldg(op.mey + at), vy, ay);
      }
    }
  }
}

// the FP32 inner solve's end: |y|^2 -> red[R_A], |z_fb|^2 -> red[R_B], y.g -> red[R_C] with
// z_fb = g .* w computed in FP64 into zf (the fallback direction, as the FP64 solve forms it)
__global__ void __launch_bounds__(BS) k_fallback_dots32(int N, const float* __restrict__ y,
                                                        const double* __restrict__ g, const double* __restrict__ w,
                                                        double* __restrict__ zf, Scalars* sc, double* part) {
  double yy = 0.0, zz = 0.0, yg = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    for (int c = 0; c < 3; ++c) {
      const double gc = g[3 * i + c], yc = (double)y[3 * i + c];
      const double zc = gc * s;
      zf[3 * i + c] = zc;
      yy += yc * yc;
      zz += zc * zc;
      yg += yc * gc;
    }
  }
  grid_reduce(yy, zz, sc, part, R_A, R_B);
  grid_reduce(yg, 0.0, sc, part, R_C);
}

// ------------------------------------------------------------------------------------------
// The inner solve with every decision on the device (Steihaug PCG of src/minimizers.py:413-490):
// the reductions' finishing blocks form alpha, the stagnation and curvature tests, beta and the
// stopping test (POST_IN_*), so an inner solve is one graph launch (WHILE node) and one host wait.
// T = double: the FP64 entries of the energy operator; T = float: the FP32 copy (1/V_mag folded in).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void exch_rows(const EnergySell& op, int r, const double* __restrict__ v, double& ax,
                                          double& ay, double& az) {
  exch_aniso_sell(op, r, v, ax, ay, az);
}
__device__ __forceinline__ void exch_rows(const EnergySell32& op, int r, const float* __restrict__ v, float& ax,
                                          float& ay, float& az) {
  exch_aniso_sell32(op, r, v, ax, ay, az);
}

__global__ void k_in_setup(Scalars* sc, int max_iter, double nu, double tol2, int cpp_count) {
  pdl_entry();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    sc->in_cpp = cpp_count;
    sc->in_max = max_iter;
    sc->in_nu = nu;
    sc->in_tol2 = tol2;
    sc->in_it = 0;
    sc->in_Q = 0.0;
    sc->in_stop = 0;
    sc->in_done = 0;
    sc->in_loops = 0;
    sc->red[R_D] = 0.0;
  }
}

// r = g, z = r .* w, p = z, y = 0; r.z -> in_rho (POST_IN_INIT)
template <class T>
__global__ void __launch_bounds__(BS) k_in_init(int N, const double* __restrict__ g, const double* __restrict__ w,
                                                T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
                                                T* __restrict__ y, Scalars* sc, double* part) {
  pdl_entry();
  Acc<T> acc;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const T s = (T)w[i];
    for (int c = 0; c < 3; ++c) {
      const T rc = (T)g[3 * i + c];
      const T zc = rc * s;
      r[3 * i + c] = rc;
      z[3 * i + c] = zc;
      p[3 * i + c] = zc;
      y[3 * i + c] = T(0);
      acc.add(rc, zc);
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_B, -1, POST_IN_INIT);
}

// Pp on the magnetic rows; p.Pp -> alpha, dq, the stop flag (POST_IN_PAP)
template <class Op, class T>
__global__ void __launch_bounds__(BS) k_in_apply(Op op, const double* __restrict__ m,
                                                 const double* __restrict__ gext, const T* __restrict__ p, T reg,
                                                 T inv_Vmag, T* __restrict__ Ap, Scalars* sc, double* part) {
  pdl_entry();
  if (sc->in_done) return;
  Acc<T> acc;
  for (int r = blockIdx.x * BS + threadIdx.x; r < op.n_rows; r += gridDim.x * BS) {
    T ax, ay, az;
    exch_rows(op, r, p, ax, ay, az);
    const int a = __ldg(op.rows + r);
    const T cx = ax * inv_Vmag, cy = ay * inv_Vmag, cz = az * inv_Vmag;
    const T mx = (T)m[3 * a], my = (T)m[3 * a + 1], mz = (T)m[3 * a + 2];
    const T mc = mx * cx + my * cy + mz * cz;
    const T mg = mx * (T)gext[3 * a] + my * (T)gext[3 * a + 1] + mz * (T)gext[3 * a + 2];
    const T px = p[3 * a], py = p[3 * a + 1], pz = p[3 * a + 2];
    const T ox = cx - mc * mx - mg * px + reg * px;
    const T oy = cy - mc * my - mg * py + reg * py;
    const T oz = cz - mc * mz - mg * pz + reg * pz;
    Ap[3 * a] = ox;
    Ap[3 * a + 1] = oy;
    Ap[3 * a + 2] = oz;
    acc.add(px, ox);
    acc.add(py, oy);
    acc.add(pz, oz);
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_C, -1, POST_IN_PAP);
}

// unless stopped: y += alpha p, r -= alpha Pp; z = r .* w; r.z -> beta, in_rho, the loop test
// (POST_IN_RHO)
template <class T>
__global__ void __launch_bounds__(BS) k_in_step(int N, T* __restrict__ y, T* __restrict__ r,
                                                const T* __restrict__ p, const T* __restrict__ Ap,
                                                const double* __restrict__ w, T* __restrict__ z, Scalars* sc,
                                                double* part) {
  pdl_entry();
  if (sc->in_done) return;
  const bool update = !sc->in_stop;
  const T alpha = scal<T>(sc->in_alpha, sc->in_alpha_f);
  Acc<T> acc;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const T s = (T)w[i];
    for (int c = 0; c < 3; ++c) {
      T rc = r[3 * i + c];
      if (update) {
        y[3 * i + c] = fmaT(alpha, p[3 * i + c], y[3 * i + c]);
        rc = fmaT(-alpha, Ap[3 * i + c], rc);
        r[3 * i + c] = rc;
      }
      const T zc = rc * s;
      z[3 * i + c] = zc;
      acc.add(rc, zc);
    }
  }
  grid_finish(block_total(acc), 0.0, sc, part, R_B, -1, POST_IN_RHO);
}

// p = z + beta p while the loop goes on
template <class T>
__global__ void __launch_bounds__(BS) k_in_xpay(int n, const T* __restrict__ z, T* __restrict__ p, Scalars* sc) {
  pdl_entry();
  if (sc->in_done) return;
  const T beta = scal<T>(sc->in_beta, sc->in_beta_f);
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) p[i] = fmaT(beta, p[i], z[i]);
}

// condition of the inner solve's WHILE node (bounded by max_iter + 2 trips)
__global__ void k_in_cond(cudaGraphConditionalHandle hnd, Scalars* sc) {
  pdl_entry();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    sc->in_loops += 1;
    const bool more = !sc->in_done && sc->in_loops <= sc->in_max + 2;
    cudaGraphSetConditional(hnd, more ? 1u : 0u);
  }
}

// out = c * fl64(y) (the FP32 inner solution, scaled by the clipping factor, widened)
__global__ void __launch_bounds__(BS) k_widen_scale(int n, const float* __restrict__ y, double c,
                                                    double* __restrict__ out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) out[i] = c * (double)y[i];
}

// ------------------------------------------------------------------------------------------
// minimizer vector kernels (3-vectors per node, xyz interleaved)
// ------------------------------------------------------------------------------------------
// g_tan = P_m(g .* inv_M_rel), g_tan_ext = P_m(g); max |g_tan| -> red[R_MAX]
__global__ void __launch_bounds__(BS) k_tangent2(int N, const double* __restrict__ m, const double* __restrict__ g,
                                                 const double* __restrict__ inv_M_rel, double* __restrict__ gt,
                                                 double* __restrict__ gte, Scalars* sc, double* part) {
  double mx_ = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double g0 = g[3 * i], g1 = g[3 * i + 1], g2 = g[3 * i + 2];
    const double w = inv_M_rel[i];
    const double s0 = g0 * w, s1 = g1 * w, s2 = g2 * w;
    const double ds = m0 * s0 + m1 * s1 + m2 * s2;
    const double t0 = s0 - ds * m0, t1 = s1 - ds * m1, t2 = s2 - ds * m2;
    const double de = m0 * g0 + m1 * g1 + m2 * g2;
    gt[3 * i] = t0;
    gt[3 * i + 1] = t1;
    gt[3 * i + 2] = t2;
    gte[3 * i] = g0 - de * m0;
    gte[3 * i + 1] = g1 - de * m1;
    gte[3 * i + 2] = g2 - de * m2;
    mx_ = fmax(mx_, fmax(fabs(t0), fmax(fabs(t1), fabs(t2))));
  }
  grid_reduce<true>(mx_, 0.0, sc, part, R_MAX);
}

// out = P_m(v)
__global__ void __launch_bounds__(BS) k_tangent(int N, const double* __restrict__ m, const double* v, double* out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double v0 = v[3 * i], v1 = v[3 * i + 1], v2 = v[3 * i + 2];
    const double d = m0 * v0 + m1 * v1 + m2 * v2;
    out[3 * i] = v0 - d * m0;
    out[3 * i + 1] = v1 - d * m1;
    out[3 * i + 2] = v2 - d * m2;
  }
}

// Cayley update with renormalisation: out = cayley(m, H, tau)
__device__ __forceinline__ void cayley_rows(int N, const double* __restrict__ m, const double* __restrict__ H,
                                            double tau, double* __restrict__ out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double k0 = 0.5 * tau * H[3 * i], k1 = 0.5 * tau * H[3 * i + 1], k2 = 0.5 * tau * H[3 * i + 2];
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    // FP64 division and square root are long instruction sequences on this part's narrow FP64 pipe:
    // one reciprocal of (1 + k.k) and one of the norm instead of six divisions
    const double kk = k0 * k0 + k1 * k1 + k2 * k2;
    const double iden = 1.0 / (1.0 + kk);
    const double km0 = k1 * m2 - k2 * m1, km1 = k2 * m0 - k0 * m2, km2 = k0 * m1 - k1 * m0;
    const double kd = k0 * m0 + k1 * m1 + k2 * m2;
    const double n0 = ((1.0 - kk) * m0 + 2.0 * km0 + 2.0 * kd * k0) * iden;
    const double n1 = ((1.0 - kk) * m1 + 2.0 * km1 + 2.0 * kd * k1) * iden;
    const double n2 = ((1.0 - kk) * m2 + 2.0 * km2 + 2.0 * kd * k2) * iden;
    const double inr = 1.0 / sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    out[3 * i] = n0 * inr;
    out[3 * i + 1] = n1 * inr;
    out[3 * i + 2] = n2 * inr;
  }
}

__global__ void __launch_bounds__(BS) k_cayley(int N, const double* __restrict__ m, const double* __restrict__ H,
                                               double tau, double* __restrict__ out) {
  cayley_rows(N, m, H, tau, out);
}

// m <- m / |m|
__global__ void __launch_bounds__(BS) k_normalize(int N, double* __restrict__ m) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double a = m[3 * i], b = m[3 * i + 1], c = m[3 * i + 2];
    const double inr = 1.0 / sqrt(a * a + b * b + c * c);
    m[3 * i] = a * inr;
    m[3 * i + 1] = b * inr;
    m[3 * i + 2] = c * inr;
  }
}

// z = r .* w (per node); r.z -> red[slot]
__global__ void __launch_bounds__(BS) k_scale3_dot(int N, const double* __restrict__ r, const double* __restrict__ w,
                                                   double* __restrict__ z, Scalars* sc, double* part, int slot) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    const double z0 = r[3 * i] * s, z1 = r[3 * i + 1] * s, z2 = r[3 * i + 2] * s;
    z[3 * i] = z0;
    z[3 * i + 1] = z1;
    z[3 * i + 2] = z2;
    d += r[3 * i] * z0 + r[3 * i + 1] * z1 + r[3 * i + 2] * z2;
  }
  grid_reduce(d, 0.0, sc, part, slot);
}

// y += ay p ; r -= ar Ap ; z = r .* w ; r.z -> red[slot]   (inner PCG of the local Hessian; the
// trust-region variant moves y by the boundary step ay and r by the Newton step ar)
__global__ void __launch_bounds__(BS) k_inner_step(int N, double ay, double ar, double* __restrict__ y,
                                                   double* __restrict__ r, const double* __restrict__ p,
                                                   const double* __restrict__ Ap, const double* __restrict__ w,
                                                   double* __restrict__ z, Scalars* sc, double* part, int slot,
                                                   int update) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    for (int c = 0; c < 3; ++c) {
      double rc = r[3 * i + c];
      if (update) {
        y[3 * i + c] = y[3 * i + c] + ay * p[3 * i + c];
        rc = rc - ar * Ap[3 * i + c];
        r[3 * i + c] = rc;
      }
      const double zc = rc * s;
      z[3 * i + c] = zc;
      d += rc * zc;
    }
  }
  grid_reduce(d, 0.0, sc, part, slot);
}

// y = x + a * y
__global__ void __launch_bounds__(BS) k_xpay(int n, const double* __restrict__ x, double a, double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = x[i] + a * y[i];
}

__device__ __forceinline__ double axpby_elem(double a, double x, double b, double y) { return a * x + b * y; }

// y = a * x + b * y
__global__ void __launch_bounds__(BS) k_axpby(int n, double a, const double* __restrict__ x, double b,
                                              double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = axpby_elem(a, x[i], b, y[i]);
}

// L-BFGS two-loop recursion with its scalars on the device (no host read between the steps):
// first loop, a = rho * (s.q) from red[slot], stored in *alpha, then q = -a y + q
__global__ void __launch_bounds__(BS) k_lb_first(int n, const double* __restrict__ rho, const Scalars* sc, int slot,
                                                 double* __restrict__ alpha, const double* __restrict__ y,
                                                 double* __restrict__ q) {
  const double a = __dmul_rn(*rho, sc->red[slot]);
  if (blockIdx.x == 0 && threadIdx.x == 0) *alpha = a;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) q[i] = axpby_elem(-a, y[i], 1.0, q[i]);
}

// second loop: c = alpha - rho * (y.out) from red[slot], then out = c s + out
__global__ void __launch_bounds__(BS) k_lb_second(int n, const double* __restrict__ rho,
                                                  const double* __restrict__ alpha, const Scalars* sc, int slot,
                                                  const double* __restrict__ s, double* __restrict__ out) {
  const double c = __dsub_rn(*alpha, __dmul_rn(*rho, sc->red[slot]));
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) out[i] = axpby_elem(c, s[i], 1.0, out[i]);
}

// initial inverse-Hessian scale of the plain L-BFGS: gamma = (s.y) / (y.(M y) + 1e-30) from red[slot_sy]
// and red[slot_ymy] (1 without history), clipped to [1e-3, 1e3] when clip
__global__ void k_lb_gamma(const Scalars* sc, int slot_sy, int slot_ymy, int has_hist, int clip,
                           double* __restrict__ gamma) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double g = 1.0;
  if (has_hist) g = __ddiv_rn(sc->red[slot_sy], __dadd_rn(sc->red[slot_ymy], 1e-30));
  if (clip) {
    g = (g < 1e-3) ? 1e-3 : g;
    g = (1e3 < g) ? 1e3 : g;
  }
  *gamma = g;
}

// y *= *a (a scalar on the device)
__global__ void __launch_bounds__(BS) k_scale_dev(int n, const double* __restrict__ a, double* __restrict__ y) {
  const double s = *a;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = s * y[i];
}

// *dst = v
__global__ void k_set_value(double* __restrict__ dst, double v) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *dst = v;
}

// y *= a
__global__ void __launch_bounds__(BS) k_scale(int n, double a, double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * y[i];
}

// max |x| -> red[R_MAX]
__global__ void __launch_bounds__(BS) k_absmax(int n, const double* __restrict__ x, Scalars* sc, double* part) {
  double v = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) v = fmax(v, fabs(x[i]));
  grid_reduce<true>(v, 0.0, sc, part, R_MAX);
}

// max |x - y| -> red[R_MAX]
__global__ void __launch_bounds__(BS) k_absmaxdiff(int n, const double* __restrict__ x, const double* __restrict__ y,
                                                   Scalars* sc, double* part) {
  double v = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) v = fmax(v, fabs(x[i] - y[i]));
  grid_reduce<true>(v, 0.0, sc, part, R_MAX);
}

// a.(b - c) -> red[R_A] and d.(b - c) -> red[R_B]
// c.(b - y) -> red[R_A] and c.w -> red[R_B] in one pass (the energy-optimal scaling of a correction c)
__global__ void __launch_bounds__(BS) k_corr_dots(int n, const double* __restrict__ c, const double* __restrict__ b,
                                                  const double* __restrict__ y, const double* __restrict__ w,
                                                  Scalars* sc, double* part) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
    s1 = fma(c[i], b[i] - y[i], s1);
    s2 = fma(c[i], w[i], s2);
  }
  grid_reduce(s1, s2, sc, part, R_A, R_B);
}

__global__ void __launch_bounds__(BS) k_dot2diff(int n, const double* __restrict__ a, const double* __restrict__ d,
                                                 const double* __restrict__ b, const double* __restrict__ c,
                                                 Scalars* sc, double* part) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
    const double df = b[i] - c[i];
    s1 = fma(a[i], df, s1);
    s2 = fma(d[i], df, s2);
  }
  grid_reduce(s1, s2, sc, part, R_A, R_B);
}

// d = -y + beta * P_m(d_prev) (d_prev itself when proj == 0); d.gte -> red[R_A]; g_raw.d -> red[R_B]
__device__ __forceinline__ void direction_rows(int N, const double* __restrict__ m, const double* __restrict__ y,
                                               const double* __restrict__ dprev, double beta,
                                               const double* __restrict__ gte, const double* __restrict__ graw,
                                               double* __restrict__ d, Scalars* sc, double* part, int proj) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double a = proj ? m0 * dprev[3 * i] + m1 * dprev[3 * i + 1] + m2 * dprev[3 * i + 2] : 0.0;
    const double dp0 = dprev[3 * i] - a * m0, dp1 = dprev[3 * i + 1] - a * m1, dp2 = dprev[3 * i + 2] - a * m2;
    const double d0 = -y[3 * i] + beta * dp0, d1 = -y[3 * i + 1] + beta * dp1, d2 = -y[3 * i + 2] + beta * dp2;
    d[3 * i] = d0;
    d[3 * i + 1] = d1;
    d[3 * i + 2] = d2;
    s1 += d0 * gte[3 * i] + d1 * gte[3 * i + 1] + d2 * gte[3 * i + 2];
    s2 += graw[3 * i] * d0 + graw[3 * i + 1] * d1 + graw[3 * i + 2] * d2;
  }
  grid_reduce(s1, s2, sc, part, R_A, R_B);
}

__global__ void __launch_bounds__(BS) k_direction(int N, const double* __restrict__ m, const double* __restrict__ y,
                                                  const double* __restrict__ dprev, double beta,
                                                  const double* __restrict__ gte, const double* __restrict__ graw,
                                                  double* __restrict__ d, Scalars* sc, double* part, int proj) {
  direction_rows(N, m, y, dprev, beta, gte, graw, d, sc, part, proj);
}

// H = m x d
__global__ void __launch_bounds__(BS) k_cross(int N, const double* __restrict__ m, const double* __restrict__ d,
                                              double* __restrict__ H) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double d0 = d[3 * i], d1 = d[3 * i + 1], d2 = d[3 * i + 2];
    H[3 * i] = m1 * d2 - m2 * d1;
    H[3 * i + 1] = m2 * d0 - m0 * d2;
    H[3 * i + 2] = m0 * d1 - m1 * d0;
  }
}

// Cayley transport of a tangent vector: out = ((1 - k.k) v + 2 k x v + 2 (k.v) k) / (1 + k.k), k = tau H / 2
// (src/minimizers.py:82-91); out may alias v
__global__ void __launch_bounds__(BS) k_transport(int N, const double* v, const double* __restrict__ H, double tau,
                                                  double* out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double k0 = 0.5 * tau * H[3 * i], k1 = 0.5 * tau * H[3 * i + 1], k2 = 0.5 * tau * H[3 * i + 2];
    const double v0 = v[3 * i], v1 = v[3 * i + 1], v2 = v[3 * i + 2];
    const double kk = k0 * k0 + k1 * k1 + k2 * k2;
    const double iden = 1.0 / (1.0 + kk);
    const double kv0 = k1 * v2 - k2 * v1, kv1 = k2 * v0 - k0 * v2, kv2 = k0 * v1 - k1 * v0;
    const double kd = k0 * v0 + k1 * v1 + k2 * v2;
    out[3 * i] = ((1.0 - kk) * v0 + 2.0 * kv0 + 2.0 * kd * k0) * iden;
    out[3 * i + 1] = ((1.0 - kk) * v1 + 2.0 * kv1 + 2.0 * kd * k1) * iden;
    out[3 * i + 2] = ((1.0 - kk) * v2 + 2.0 * kv2 + 2.0 * kd * k2) * iden;
  }
}

// M_rel-weighted inner products, M_rel = 1 / inv_M_rel where inv_M_rel > 1e-20 (else 0):
// sum M a1.b1 -> red[R_A], sum M a2.b2 -> red[R_B]
__global__ void __launch_bounds__(BS) k_mdot2(int N, const double* __restrict__ a1, const double* __restrict__ b1,
                                              const double* __restrict__ a2, const double* __restrict__ b2,
                                              const double* __restrict__ imr, Scalars* sc, double* part) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double w = imr[i] > 1e-20 ? 1.0 / imr[i] : 0.0;
    s1 += w * (a1[3 * i] * b1[3 * i] + a1[3 * i + 1] * b1[3 * i + 1] + a1[3 * i + 2] * b1[3 * i + 2]);
    s2 += w * (a2[3 * i] * b2[3 * i] + a2[3 * i + 1] * b2[3 * i + 1] + a2[3 * i + 2] * b2[3 * i + 2]);
  }
  grid_reduce(s1, s2, sc, part, R_A, R_B);
}

// sum M_rel |y + a p|^2 -> red[R_C]
__global__ void __launch_bounds__(BS) k_mnorm_axpy(int N, const double* __restrict__ y, double a,
                                                   const double* __restrict__ p, const double* __restrict__ imr,
                                                   Scalars* sc, double* part) {
  double s = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double w = imr[i] > 1e-20 ? 1.0 / imr[i] : 0.0;
    const double u0 = y[3 * i] + a * p[3 * i], u1 = y[3 * i + 1] + a * p[3 * i + 1], u2 = y[3 * i + 2] + a * p[3 * i + 2];
    s += w * (u0 * u0 + u1 * u1 + u2 * u2);
  }
  grid_reduce(s, 0.0, sc, part, R_C);
}

// Riemannian Hessian action from the full gradient operator: out = Cv - ((v.g) m + (m.g) v + (m.Cv) m)
// per node (src/minimizers.py:2155-2162); v.out -> red[R_C]
__global__ void __launch_bounds__(BS) k_hess_full(int N, const double* __restrict__ m, const double* __restrict__ g,
                                                  const double* __restrict__ v, const double* __restrict__ Cv,
                                                  double* __restrict__ out, Scalars* sc, double* part) {
  double s = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double v0 = v[3 * i], v1 = v[3 * i + 1], v2 = v[3 * i + 2];
    const double g0 = g[3 * i], g1 = g[3 * i + 1], g2 = g[3 * i + 2];
    const double c0 = Cv[3 * i], c1 = Cv[3 * i + 1], c2 = Cv[3 * i + 2];
    const double mg = m0 * g0 + m1 * g1 + m2 * g2;
    const double vg = v0 * g0 + v1 * g1 + v2 * g2;
    const double mc = m0 * c0 + m1 * c1 + m2 * c2;
    const double o0 = c0 - (vg * m0 + mg * v0 + mc * m0);
    const double o1 = c1 - (vg * m1 + mg * v1 + mc * m1);
    const double o2 = c2 - (vg * m2 + mg * v2 + mc * m2);
    out[3 * i] = o0;
    out[3 * i + 1] = o1;
    out[3 * i + 2] = o2;
    s += v0 * o0 + v1 * o1 + v2 * o2;
  }
  grid_reduce(s, 0.0, sc, part, R_C);
}

// y += a x with a = red[R_A] / red[R_B] (0 unless the denominator is positive and finite), the
// scaling computed on the device; a -> red[R_C]
__global__ void __launch_bounds__(BS) k_axpy_ratio(int n, const double* __restrict__ x, double* __restrict__ y,
                                                   Scalars* sc) {
  const double num = sc->red[R_A], den = sc->red[R_B];
  const double a = (den > 0.0 && isfinite(den)) ? num / den : 0.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->red[R_C] = a;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * x[i] + y[i];
}

// z = g .* w (per node); |y|^2 -> red[R_A], |z|^2 -> red[R_B], y.g -> red[R_C] (the inner solve's
// fallback direction, clipping and descent test in one pass)
__global__ void __launch_bounds__(BS) k_fallback_dots(int N, const double* __restrict__ y,
                                                      const double* __restrict__ g, const double* __restrict__ w,
                                                      double* __restrict__ z, Scalars* sc, double* part) {
  double yy = 0.0, zz = 0.0, yg = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    for (int c = 0; c < 3; ++c) {
      const double gc = g[3 * i + c], yc = y[3 * i + c];
      const double zc = gc * s;
      z[3 * i + c] = zc;
      yy += yc * yc;
      zz += zc * zc;
      yg += yc * gc;
    }
  }
  grid_reduce(yy, zz, sc, part, R_A, R_B);
  grid_reduce(yg, 0.0, sc, part, R_C);
}

// ------------------------------------------------------------------------------------------
// The preconditioned CG minimizers (pcohen_hs, pcohen, pcg) iterated on the device: every decision
// the host loop takes between kernels (the inner solve's forcing tolerance, clipping and fallback,
// beta, the descent test, the Armijo search's expansion and contraction, the U1-U4 test) restated as
// single-thread kernels over MinScal, so that one CUDA graph with WHILE nodes runs whole iterations:
// the inner preconditioner solve and the line-search trials (each with its demag PCG) are nested
// loops.  Same formulas and the same reduction kernels as the host loop.
// ------------------------------------------------------------------------------------------
struct MinScal {
  // parameters of the call
  int max_iter, L, pr, pc_auto, pc_iters, max_evals, cpp;
  double pc_force_eta, pc_force_alpha, pc_nu, eta1, eta2, C, c, s0;
  double tau_f, eps_a, u2_bound, u3_root;  // sqrt(tau_f) 2 and tau_f^(1/3), formed on the host
  double B[3];
  // outer state
  int it, conv, outer_loops, flag, flag2, accepted, phase, it_exp, it_con, ls_loops;
  double E, E_new, E_lag, gsm, beta, pg, cf;
  // line search
  double s, s_min, d_v, E_v, E0;
  // counters
  long long evals, preco, demag;
  long long in_trips, pcg_trips;  // WHILE trips of the inner solves and of the demag PCG loops
};

__device__ __forceinline__ bool lead_thread() { return threadIdx.x == 0 && blockIdx.x == 0; }

// condition of a WHILE node entered next (a nested node takes no default value per entry)
__global__ void k_cond_set(cudaGraphConditionalHandle hnd, unsigned value) {
  if (lead_thread()) cudaGraphSetConditional(hnd, value);
}

__global__ void __launch_bounds__(BS) k_copy_vec(int n, const double* __restrict__ src, double* __restrict__ dst) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) dst[i] = src[i];
}

__global__ void __launch_bounds__(BS) k_zero_vec(int n, double* __restrict__ dst) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) dst[i] = 0.0;
}

// the outer loop's first trip
__global__ void k_min_start(cudaGraphConditionalHandle hnd, MinScal* ms) {
  if (lead_thread()) {
    ms->outer_loops = 0;
    ms->conv = 0;
    cudaGraphSetConditional(hnd, (ms->it < ms->max_iter) ? 1u : 0u);
  }
}

// the inner solve's start (k_in_setup) with the forcing tolerance min(eta, max|g_tan|^alpha) formed
// here from red[R_MAX] of k_tangent2
__global__ void k_min_in_setup(Scalars* sc, MinScal* ms) {
  if (lead_thread()) {
    const double gn = sc->red[R_MAX];
    const double tol = ms->pc_auto ? fmin(ms->pc_force_eta, pow(gn, ms->pc_force_alpha)) : 0.0;
    sc->in_cpp = ms->cpp;
    sc->in_max = ms->pc_iters;
    sc->in_nu = ms->pc_nu;
    sc->in_tol2 = tol * tol;
    sc->in_it = 0;
    sc->in_Q = 0.0;
    sc->in_stop = 0;
    sc->in_done = 0;
    sc->in_loops = 0;
    sc->red[R_D] = 0.0;
  }
}

// the inner solve's end: clipping factor from |y|^2 and |z_fb|^2 (red[R_A], red[R_B]); its
// iteration count (red[R_D]) into preco
__global__ void k_min_clip(Scalars* sc, MinScal* ms) {
  if (lead_thread()) {
    const double yn = sqrt(sc->red[R_A]), zn = sqrt(sc->red[R_B]);
    const int clip = yn > 10.0 * zn;
    ms->flag = clip;
    ms->cf = clip ? 10.0 * zn / (yn + 1e-30) : 1.0;
    ms->preco += (long long)sc->red[R_D];
    ms->in_trips += sc->in_loops;
  }
}

// y *= cf when clipping (FP64 inner solve)
__global__ void __launch_bounds__(BS) k_scale_clip(int n, double* __restrict__ y, const MinScal* ms) {
  if (!ms->flag) return;
  const double a = ms->cf;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * y[i];
}

// y = cf * fl64(yf) (FP32 inner solve; cf = 1 without clipping)
__global__ void __launch_bounds__(BS) k_widen_clip(int n, const float* __restrict__ yf, const MinScal* ms,
                                                   double* __restrict__ y) {
  const double a = ms->cf;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * (double)yf[i];
}

// k_dot when *flag (the same reduction; nothing, not even the slot, is touched otherwise)
__global__ void __launch_bounds__(BS) k_dot_flag(const int* flag, int n, const double* __restrict__ x,
                                                 const double* __restrict__ y, Scalars* sc, double* part, int slot) {
  if (!*flag) return;
  Acc<double> acc;
  ROW_LOOP(n) {
    int row[ILP];
    rows_of(rb, row);
#pragma unroll
    for (int q = 0; q < ILP; ++q)
      if (row[q] < n) acc.add(x[row[q]], y[row[q]]);
  }
  grid_finish(block_total(acc), 0.0, sc, part, slot, -1, POST_NONE);
}

// not a descent direction (y.g_tan_ext at most 1e-12: red[R_C] of the inner solve's end, or red[R_A]
// recomputed after clipping): fall back to z_fb
__global__ void k_min_fallback(Scalars* sc, MinScal* ms) {
  if (lead_thread()) ms->flag2 = !((ms->flag ? sc->red[R_A] : sc->red[R_C]) > 1e-12);
}

// dst = src when *flag
__global__ void __launch_bounds__(BS) k_copy_flag(const int* flag, int n, const double* __restrict__ src,
                                                  double* __restrict__ dst) {
  if (!*flag) return;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) dst[i] = src[i];
}

// beta: Hestenes-Stiefel y.(g - g_prev) / (d_prev.(g - g_prev) + 1e-30) (red[R_A], red[R_B]) or
// Polak-Ribiere over y_prev.g_prev (red[R_C]); 0 on restarts; max|y| (red[R_MAX]) kept for the test
__global__ void k_min_beta(Scalars* sc, MinScal* ms) {
  if (lead_thread()) {
    ms->gsm = sc->red[R_MAX];
    const double num = sc->red[R_A];
    const double den = (ms->pr ? sc->red[R_C] : sc->red[R_B]) + 1e-30;
    ms->beta = (ms->it % ms->L == 0) ? 0.0 : fmax(0.0, num / den);
  }
}

// k_direction with beta from MinScal
__global__ void __launch_bounds__(BS) k_direction_ms(int N, const double* __restrict__ m, const double* __restrict__ y,
                                                     const double* __restrict__ dprev, const MinScal* ms,
                                                     const double* __restrict__ gte, const double* __restrict__ graw,
                                                     double* __restrict__ d, Scalars* sc, double* part, int proj) {
  direction_rows(N, m, y, dprev, ms->beta, gte, graw, d, sc, part, proj);
}

// d.g_tan_ext > 0 (red[R_A]): d must become -y; g_raw.d from red[R_B]
__global__ void k_min_descent(Scalars* sc, MinScal* ms) {
  if (lead_thread()) {
    ms->flag = sc->red[R_A] > 0.0;
    ms->pg = sc->red[R_B];
  }
}

// d = -1 y + 0 d when *flag (the host loop's k_axpby form)
__global__ void __launch_bounds__(BS) k_neg_flag(const int* flag, int n, const double* __restrict__ y,
                                                 double* __restrict__ d) {
  if (!*flag) return;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) d[i] = -1.0 * y[i] + 0.0 * d[i];
}

// g_raw.d recomputed after the descent fix (red[R_A] of k_dot_flag)
__global__ void k_min_pg(Scalars* sc, MinScal* ms) {
  if (lead_thread() && ms->flag) ms->pg = sc->red[R_A];
}

// Armijo search start (src/minimizers.py:265-385): no search when g_raw.d >= 0
__global__ void k_ls_init(cudaGraphConditionalHandle hnd, MinScal* ms) {
  if (lead_thread()) {
    ms->E0 = ms->E;
    ms->s = ms->s0;
    ms->s_min = 0.0;
    ms->it_exp = ms->it_con = 0;
    ms->d_v = 0.0;
    ms->E_v = ms->E;
    ms->ls_loops = 0;
    ms->accepted = 0;
    ms->phase = (ms->pg >= 0.0) ? 2 : 0;  // 0 expansion, 1 contraction, 2 done
    cudaGraphSetConditional(hnd, ms->phase != 2 ? 1u : 0u);
  }
}

// Cayley update with the trial step from MinScal
__global__ void __launch_bounds__(BS) k_cayley_ms(int N, const double* __restrict__ m, const double* __restrict__ H,
                                                  const MinScal* ms, double* __restrict__ out) {
  cayley_rows(N, m, H, ms->s, out);
}

// the demag PCG iterations of a trial (sc->it) into the counter
__global__ void k_min_demag(const Scalars* sc, MinScal* ms) {
  if (lead_thread()) {
    ms->demag += sc->it;
    ms->pcg_trips += sc->loops;
  }
}

// one trial's test d = (E_t - E0) / (s pg + 1e-30) and the next step: expansion while
// |1 - d| < eta2 and d >= 0 (s_min = s, s *= C), then contraction s = s_min + c (s - s_min) until
// d >= eta1 and d < 1e10; at most max_evals trials each; the loop is bounded besides by its trips
__global__ void k_ls_decide(cudaGraphConditionalHandle hnd, const Scalars* sc, MinScal* ms, double inv_Vmag) {
  if (!lead_thread()) return;
  double E_t = 0.5 * sc->red[R_E] * inv_Vmag;
  if (!isfinite(E_t)) E_t = 1e20;
  const double d = (E_t - ms->E0) / (ms->s * ms->pg + 1e-30);
  ms->d_v = d;
  ms->E_v = E_t;
  ms->ls_loops += 1;
  if (ms->phase == 0) {
    const bool stop = (fabs(1.0 - d) >= ms->eta2) || (d < 0.0);
    if (!stop) {
      ms->s_min = ms->s;
      ms->s = ms->C * ms->s;
    }
    ms->it_exp += 1;
    if (stop || ms->it_exp >= ms->max_evals) {
      const bool ok = (d >= ms->eta1) && (d < 1e10);
      if (ok) {
        ms->phase = 2;
      } else {
        ms->phase = 1;
        ms->s = ms->s_min + ms->c * (ms->s - ms->s_min);
      }
    }
  } else if (ms->phase == 1) {
    ms->it_con += 1;
    const bool ok = (d >= ms->eta1) && (d < 1e10);
    if (ok || ms->it_con >= ms->max_evals) ms->phase = 2;
    else ms->s = ms->s_min + ms->c * (ms->s - ms->s_min);
  }
  const bool more = ms->phase != 2 && ms->ls_loops <= 2 * ms->max_evals + 2;
  cudaGraphSetConditional(hnd, more ? 1u : 0u);
}

// the search's result: the last trial is kept when its d >= 0
__global__ void k_ls_finish(MinScal* ms) {
  if (lead_thread()) {
    const int trials = ms->it_exp + ms->it_con;
    ms->evals += trials;
    ms->accepted = (ms->pg < 0.0 && trials > 0 && ms->d_v >= 0.0) ? 1 : 0;
    ms->E_new = ms->accepted ? ms->E_v : ms->E;
  }
}

// Gill-Murray-Wright U1-U4 on the accepted step (max|m_new - m| in red[R_MAX]) and the next trip's
// condition (src/minimizers.py:160-172)
__global__ void k_min_conv(cudaGraphConditionalHandle hnd, const Scalars* sc, MinScal* ms) {
  if (!lead_thread()) return;
  const double dm = ms->accepted ? sc->red[R_MAX] : 0.0;
  const double E_new = ms->E_new, E_prev = ms->E;
  const double E_ref = ms->cpp ? ms->E_lag : E_prev;  // the C++ minimizer tests against the lagged energy
  bool conv = false;
  if (ms->it > 0) {
    const bool u1 = (E_ref - E_new) < ms->tau_f * (1.0 + fabs(E_new));
    const bool u2 = dm < ms->u2_bound;
    const bool u3 = ms->gsm <= ms->u3_root * (1.0 + fabs(E_new));
    const bool u4 = ms->gsm < ms->eps_a;
    conv = (u1 && u2 && u3) || u4;
  }
  ms->conv = conv ? 1 : 0;
  ms->E_lag = E_prev;
  ms->E = E_new;
  ms->it += 1;
  ms->outer_loops += 1;
  const bool more = !conv && ms->it < ms->max_iter && ms->outer_loops <= ms->max_iter + 2;
  cudaGraphSetConditional(hnd, more ? 1u : 0u);
}

// accepted step: m, U, g_raw <- the trial's; then g_prev <- g_tan_ext, d_prev <- d (y_prev <- y
// when ys != nullptr), the copies that stand for the host loop's buffer swaps
__global__ void __launch_bounds__(BS) k_min_advance(int n3, int N, const MinScal* ms, double* __restrict__ m,
                                                    const double* __restrict__ mt, double* __restrict__ U,
                                                    const double* __restrict__ Ut, double* __restrict__ graw,
                                                    const double* __restrict__ gt, double* __restrict__ gprev,
                                                    const double* __restrict__ gte, double* __restrict__ dprev,
                                                    const double* __restrict__ d, double* __restrict__ ys,
                                                    const double* __restrict__ y) {
  const bool acc = ms->accepted != 0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n3; i += gridDim.x * BS) {
    if (acc) {
      m[i] = mt[i];
      graw[i] = gt[i];
      if (i < N) U[i] = Ut[i];
    }
    gprev[i] = gte[i];
    dprev[i] = d[i];
    if (ys) ys[i] = y[i];
  }
}

}  // namespace mmk
