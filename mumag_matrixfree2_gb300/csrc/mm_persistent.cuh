// Persistent PCG loop: the whole iteration loop of one demag solve (direction, step, V-cycle on
// every level, coarsest dense solve) runs in ONE cooperative launch.
//
// Why: at the sizes of this problem every solver kernel is latency-bound (a chain of three
// dependent loads per row, a launch, a ramp and a tail), so a PCG iteration of ~16 separate
// launches costs far more than its flops or bytes.  Here every block owns a fixed slice of the
// rows of every operator for the whole solve; the phases of an iteration are separated by a grid
// barrier; every block sums the reduction partials itself (fixed order, so all blocks hold the same
// value and the result is deterministic) instead of one finishing block; and the matrices, read
// only, stay cacheable in the SM's L1 from one iteration to the next because the same SM reads the
// same rows every time.
//
// Memory: vectors written inside the kernel are read with ld.global.cg (L2, coherent across SMs)
// after the barrier; matrices and smoother diagonals use the read-only path.
//
// The barrier is this project's own (one arrival counter + a generation word).  Co-residency of all
// blocks is guaranteed by the cooperative launch, and every wait is bounded: after 1 s without
// progress, or when another block has given up, a block sets the error word and returns, and the
// host reports the failure.  The state is cleared by the host before each launch.
#pragma once

#include "mm_kernels.cuh"

namespace mmk {

// operator view: tpr == 1 -> sliced ELL (ptr = slice pointers); tpr in {2..32} -> CSR, tpr lanes/row.
// bp: first slice (ELL) or row (CSR) of every block of the launch, gridDim.x + 1 entries.
template <class T>
struct MatV {
  int n;
  int tpr;
  const int* ptr;
  const int* col;
  const T* val;
  const int* bp;
};

// one level of the hierarchy as the persistent kernel sees it
template <class T>
struct PLev {
  MatV<T> A;  // n x n
  MatV<T> R;  // restriction to level + 1 (n_{l+1} rows); unused on the coarsest level
  MatV<T> P;  // prolongation from level + 1 (n rows); unused on the coarsest level
  const T* s; // smoother diagonal
  T* b;       // right-hand side (levels >= 1)
  T* x;       // pre-smoothed iterate, then prolongation target
  T* x2;      // post-smoothed iterate (levels >= 1; coarsest: dense solution)
  T* res;     // residual
  int n;
};

struct GridBar {
  unsigned count;  // arrivals in the current generation
  unsigned gen;    // completed barriers
  int err;         // 1: a block gave up waiting
  int pad;
};

template <class T>
struct PcgArgs {
  const PLev<T>* lv;
  int L;
  const T* Ainv;  // dense inverse of the coarsest level (row-major nc x nc)
  int nc;
  T* x;
  T* r;
  T* z;
  T* p;
  T* Ap;
  Scalars* sc;
  double* part;  // NRED x MAXG partials
  GridBar* bar;
};

constexpr unsigned long long BAR_TIMEOUT_NS = 1000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier.  Returns false when the wait gave up; the caller must return.
__device__ __forceinline__ bool grid_barrier(GridBar* gb, unsigned& gen_local) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(gb->count);
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(gb->gen);
    cuda::atomic_ref<int, cuda::thread_scope_device> err(gb->err);
    int ok = 1;
    const unsigned g = gen_local;
    __threadfence();
    if (cnt.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
      cnt.store(0u, cuda::memory_order_relaxed);
      gen.store(g + 1u, cuda::memory_order_release);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned spins = 0;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if ((++spins & 31u) == 0u) {
          if (err.load(cuda::memory_order_relaxed) != 0 || global_ns() - t0 > BAR_TIMEOUT_NS) {
            err.store(1, cuda::memory_order_relaxed);
            ok = 0;
            break;
          }
        }
      }
    }
    __threadfence();
    gen_local = g + 1u;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of the gridDim.x partials of one reduction: thread t adds partials t, t + BS, ... (independent
// loads, issued together), then the block's fixed tree.  Every block computes the identical value.
__device__ __forceinline__ double sum_partials(const double* part) {
  const int G = (int)gridDim.x;
  double t = 0.0;
#pragma unroll
  for (int k = 0; k < MAXG / BS; ++k) {
    const int i = threadIdx.x + k * BS;
    if (i < G) t += __ldcg(part + i);
  }
  return block_sum(t);
}

// the rows of an operator owned by this block, from the operator's block bounds (gridDim.x + 1
// entries, balanced by stored entries on the host): sliced ELL in whole slices, CSR in plain rows
template <class T>
__device__ __forceinline__ void owned_rows(const MatV<T>& M, int& r0, int& r1) {
  const int b = blockIdx.x;
  if (M.tpr == 1) {
    r0 = 32 * __ldg(M.bp + b);
    r1 = min(M.n, 32 * __ldg(M.bp + b + 1));
  } else {
    r0 = __ldg(M.bp + b);
    r1 = __ldg(M.bp + b + 1);
  }
}

// (M x)_row for every owned row, f(row, value) called once per row.  Sliced ELL: one thread per
// row, RPT rows in flight per thread; CSR: tpr lanes per row, warp-uniform rounds for the shuffles.
// non-zeros in flight per row in the persistent loop (fewer than the separate kernels: the whole
// iteration lives in one kernel, so registers are scarcer)
constexpr int KUP = 1;

template <int RPT, class T, class F>
__device__ __forceinline__ void mat_rows(const MatV<T>& M, const T* x, F&& f) {
  int r0, r1;
  owned_rows(M, r0, r1);
  if (M.tpr == 1) {
    for (int rb = r0; rb < r1; rb += RPT * BS) {
      int row[RPT];
      T acc[RPT];
#pragma unroll
      for (int q = 0; q < RPT; ++q) row[q] = rb + threadIdx.x + q * BS;
      sell_rows_k<RPT, true, T>(M.ptr, M.col, M.val, r1, x, row, acc);
#pragma unroll
      for (int q = 0; q < RPT; ++q)
        if (row[q] < r1) f(row[q], acc[q]);
    }
  } else {
    const int tpr = M.tpr;
    const int lane = threadIdx.x & (tpr - 1);
    const int grp = threadIdx.x / tpr;
    const int gpb = BS / tpr;
    const int rounds = (r1 - r0 + gpb - 1) / gpb;
    for (int k = 0; k < rounds; ++k) {
      const int row = r0 + grp + k * gpb;
      T acc = T(0);
      if (row < r1) {
        const int e = __ldg(M.ptr + row + 1);
        for (int j = __ldg(M.ptr + row) + lane; j < e; j += KUP * tpr) {
          int c[KUP];
          T v[KUP], xv[KUP];
#pragma unroll
          for (int u = 0; u < KUP; ++u)
            if (j + u * tpr < e) {
              c[u] = __ldg(M.col + j + u * tpr);
              v[u] = __ldg(M.val + j + u * tpr);
            }
#pragma unroll
          for (int u = 0; u < KUP; ++u)
            if (j + u * tpr < e) xv[u] = __ldcg(x + c[u]);
#pragma unroll
          for (int u = 0; u < KUP; ++u)
            if (j + u * tpr < e) acc = fmaT<T>(v[u], xv[u], acc);
        }
      }
      for (int o = tpr >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (row < r1 && lane == 0) f(row, acc);
    }
  }
}

// own rows of a level-0 vector operation (same partition as the level-0 operator)
template <class T, class F>
__device__ __forceinline__ void vec_rows(const MatV<T>& A0, F&& f) {
  int r0, r1;
  owned_rows(A0, r0, r1);
  for (int i = r0 + threadIdx.x; i < r1; i += BS) f(i);
}

template <class T>
__device__ __forceinline__ void put_partial(double* part, int slot, double v) {
  if (threadIdx.x == 0) part[(size_t)slot * MAXG + blockIdx.x] = v;
}

// The PCG loop from the state left by the start of the solve (r, z, p = z not yet formed: the
// first direction uses beta = 0, exactly as the separate kernels do).  Stops on the recursive
// residual r.r <= tol2 or maxiter (src/poisson_solve.py:422-478), then block 0 stores the scalars.
// MINB: blocks per SM the registers are budgeted for; RPT: rows in flight per thread.
template <class T, int MINB, int RPT>
__global__ void __launch_bounds__(BS, MINB) k_pcg_persistent(PcgArgs<T> a) {
  Scalars* sc = a.sc;
  unsigned gen = 0;
  double rz = sc->rz, beta = sc->beta, r2 = sc->red[R_R2], alpha = sc->alpha, pap = 0.0;
  int it = sc->it, done = sc->done;
  const int maxiter = sc->maxiter;
  const double tol2 = sc->tol2;
  const int L = a.L;
  const PLev<T>* lv = a.lv;
  const MatV<T> A0 = lv[0].A;
  const T* s0 = lv[0].s;
  T* xv0 = lv[0].x;
  T* res0 = lv[0].res;
  bool ok = true;

  while (!done) {
    // p = z + beta p ; Ap = A z + beta Ap ; p.Ap
    {
      const T bt = (T)beta;
      Acc<T> acc;
      mat_rows<RPT, T>(A0, a.z, [&](int i, T az) {
        const T pn = bt != T(0) ? __ldcg(a.z + i) + bt * a.p[i] : __ldcg(a.z + i);
        const T apn = bt != T(0) ? az + bt * a.Ap[i] : az;
        a.p[i] = pn;
        a.Ap[i] = apn;
        acc.add(pn, apn);
      });
      put_partial<T>(a.part, R_PAP, block_total(acc));
      if (!(ok = grid_barrier(a.bar, gen))) break;
      pap = sum_partials(a.part + (size_t)R_PAP * MAXG);
      alpha = rz / (pap + 1e-30);
    }
    // x += alpha p ; r -= alpha Ap ; r.r ; xv = s0 .* r
    {
      const T al = (T)alpha;
      Acc<T> acc;
      vec_rows<T>(A0, [&](int i) {
        a.x[i] = a.x[i] + al * a.p[i];
        const T ri = a.r[i] - al * a.Ap[i];
        a.r[i] = ri;
        acc.add(ri, ri);
        xv0[i] = s0[i] * ri;
      });
      put_partial<T>(a.part, R_R2, block_total(acc));
      if (!(ok = grid_barrier(a.bar, gen))) break;
      r2 = sum_partials(a.part + (size_t)R_R2 * MAXG);
      it += 1;
      if (r2 <= tol2 || it >= maxiter) {
        done = 1;
        break;
      }
    }
    // V-cycle, level 0 residual
    mat_rows<RPT, T>(A0, xv0, [&](int i, T ax) { res0[i] = a.r[i] - ax; });
    if (!(ok = grid_barrier(a.bar, gen))) break;
    // down: restrict (fused with the coarse pre-smoothing from zero), coarse residuals
    for (int l = 0; l < L - 1 && ok; ++l) {
      const PLev<T>& c = lv[l];
      const PLev<T>& nx = lv[l + 1];
      const bool coarsest = (l + 1 == L - 1);
      mat_rows<RPT, T>(c.R, c.res, [&](int i, T v) {
        nx.b[i] = v;
        if (!coarsest) nx.x[i] = __ldg(nx.s + i) * v;
      });
      if (!(ok = grid_barrier(a.bar, gen))) break;
      if (!coarsest) {
        mat_rows<RPT, T>(nx.A, nx.x, [&](int i, T ax) { nx.res[i] = __ldcg(nx.b + i) - ax; });
        if (!(ok = grid_barrier(a.bar, gen))) break;
      }
    }
    if (!ok) break;
    // coarsest: x2 = Ainv b, one warp per row
    {
      const PLev<T>& c = lv[L - 1];
      const int nc = a.nc;
      const int lanes = threadIdx.x & 31;
      const int wpb = BS / 32;
      for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < nc; row += gridDim.x * wpb) {
        const T* arow = a.Ainv + (size_t)row * nc;
        T acc = T(0);
        for (int k = lanes; k < nc; k += 32) acc = fmaT<T>(__ldg(arow + k), __ldcg(c.b + k), acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lanes == 0) c.x2[row] = acc;
      }
      if (!(ok = grid_barrier(a.bar, gen))) break;
    }
    // up: prolongate, post-smooth
    for (int l = L - 2; l >= 1 && ok; --l) {
      const PLev<T>& c = lv[l];
      mat_rows<RPT, T>(c.P, lv[l + 1].x2, [&](int i, T e) { c.x[i] = __ldcg(c.x + i) + e; });
      if (!(ok = grid_barrier(a.bar, gen))) break;
      mat_rows<RPT, T>(c.A, c.x, [&](int i, T ax) {
        c.x2[i] = __ldcg(c.x + i) + __ldg(c.s + i) * (__ldcg(c.b + i) - ax);
      });
      if (!(ok = grid_barrier(a.bar, gen))) break;
    }
    if (!ok) break;
    mat_rows<RPT, T>(lv[0].P, lv[1].x2, [&](int i, T e) { xv0[i] = __ldcg(xv0 + i) + e; });
    if (!(ok = grid_barrier(a.bar, gen))) break;
    // level-0 post-smoothing z = x + s0 .* (r - A0 x) ; r.z ; beta
    {
      Acc<T> acc;
      mat_rows<RPT, T>(A0, xv0, [&](int i, T ax) {
        const T ri = a.r[i];
        const T zi = __ldcg(xv0 + i) + s0[i] * (ri - ax);
        a.z[i] = zi;
        acc.add(ri, zi);
      });
      put_partial<T>(a.part, R_RZ, block_total(acc));
      if (!(ok = grid_barrier(a.bar, gen))) break;
      const double rz_new = sum_partials(a.part + (size_t)R_RZ * MAXG);
      beta = rz_new / (rz + 1e-30);
      rz = rz_new;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && ok) {
    sc->it = it;
    sc->done = 1;
    sc->rz = rz;
    sc->alpha = alpha;
    sc->alpha_f = (float)alpha;
    sc->beta = beta;
    sc->beta_f = (float)beta;
    sc->red[R_R2] = r2;
    sc->red[R_PAP] = pap;
    sc->red[R_RZ] = rz;
  }
}

}  // namespace mmk
