// Device kernels of the micromagnetic hot path (sm_103a).
//
// Conventions
//  * Every reduction is deterministic: a kernel writes one partial per block (fixed grid, fixed
//    in-block tree), and its consumers re-reduce the partials in a fixed order (every block of the
//    consumer computes the same value, so no extra launch is needed to finalise a scalar).
//  * Compressed-row kernels map TPR consecutive lanes to one row (TPR = 32 is warp-per-row); lanes
//    stride the row's entries and combine with xor shuffles, so each row sums in a fixed order.
//  * Iterative kernels read a device "done" flag first and return when it is set; a converged
//    solve therefore ignores the launches still queued behind it.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mmk {

constexpr int BS = 256;       // threads per block for every kernel here
constexpr int MAXG = 1216;    // 152 SMs x 8 blocks: upper bound of any grid (and of partial slots)

struct Scalars {              // device-resident solver scalars (one instance per solver context)
  double tol2;                // tol^2 * b.b
  double rz_prev;             // r.z of the previous PCG iteration
  double bnorm2;              // b.b before zero-mean projection
  int it;                     // completed PCG iterations
  int done;                   // 1 once converged or out of iterations
  int maxiter;
  int pad;
};

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

// Sum over the block; the result is returned to every thread.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s_red[BS / 32];
  __shared__ double s_out;
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < BS / 32 ? s_red[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) s_out = t;
  }
  __syncthreads();
  return s_out;
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double s_red[BS / 32];
  __shared__ double s_out;
  v = warp_max(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) s_red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < BS / 32 ? s_red[lane] : 0.0;
    t = warp_max(t);
    if (lane == 0) s_out = t;
  }
  __syncthreads();
  return s_out;
}

// Re-reduce `count` block partials; identical result in every block.
__device__ __forceinline__ double reduce_partials(const double* __restrict__ part, int count) {
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += BS) v += part[i];
  return block_sum(v);
}

__device__ __forceinline__ double reduce_partials_max(const double* __restrict__ part, int count) {
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += BS) v = fmax(v, part[i]);
  return block_max(v);
}

template <int TPR>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum_k val[k] x[col[k]] over one row, TPR lanes; result valid on every lane of the group
template <int TPR>
__device__ __forceinline__ double row_dot(const int* __restrict__ ptr, const int* __restrict__ col,
                                          const double* __restrict__ val, const double* __restrict__ x, int row,
                                          bool valid, int lane) {
  double acc = 0.0;
  if (valid) {
    const int s = ptr[row], e = ptr[row + 1];
    for (int k = s + lane; k < e; k += TPR) acc = fma(val[k], __ldg(x + col[k]), acc);
  }
  return group_sum<TPR>(acc);
}

// ------------------------------------------------------------------------------------------
// compressed-row products used by the PCG and the V-cycle
// ------------------------------------------------------------------------------------------
// mode 0: y = A x ; mode 1: y = b - A x ; mode 2: y = x + s .* (b - A x) ; mode 3: y = x + A e (P e)
template <int TPR, int MODE>
__global__ void __launch_bounds__(BS) k_spmv(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                             const double* __restrict__ val, const double* __restrict__ x,
                                             const double* __restrict__ b, const double* __restrict__ s,
                                             double* __restrict__ y, const int* __restrict__ done) {
  if (done && *done) return;
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double ax = row_dot<TPR>(ptr, col, val, x, row, valid, lane);
    if (valid && lane == 0) {
      if (MODE == 0) y[row] = ax;
      else if (MODE == 1) y[row] = b[row] - ax;
      else if (MODE == 2) y[row] = x[row] + s[row] * (b[row] - ax);
      else y[row] = b[row] + ax;  // prolongation: y = b + P e, with x := e
    }
  }
}

// y = A x and one partial of x.y per block
template <int TPR>
__global__ void __launch_bounds__(BS) k_spmv_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const double* __restrict__ val, const double* __restrict__ x,
                                                 double* __restrict__ y, double* __restrict__ part) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double d = 0.0;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double ax = row_dot<TPR>(ptr, col, val, x, row, valid, lane);
    if (valid && lane == 0) {
      y[row] = ax;
      d = fma(x[row], ax, d);
    }
  }
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// PCG direction update fused with the operator product (iteration i):
//   rz = sum(part_rz); beta = first ? 0 : rz / (rz_prev + eps)
//   y = A z ; p = z + beta p ; Ap = y + beta Ap ; partial p.Ap
// A p_new = A z + beta A p_old, so the product is taken on z, which is complete before the launch.
template <int TPR>
__global__ void __launch_bounds__(BS) k_pcg_dir(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                const double* __restrict__ val, const double* __restrict__ z,
                                                double* __restrict__ p, double* __restrict__ Ap,
                                                const double* __restrict__ part_rz, int n_rz,
                                                const double* __restrict__ part_r2, int n_r2,
                                                double* __restrict__ part_pAp, Scalars* sc, int first) {
  if (sc->done) return;
  const double r2 = reduce_partials(part_r2, n_r2);
  if (r2 <= sc->tol2 || sc->it >= sc->maxiter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = 1;
    return;
  }
  const double rz = reduce_partials(part_rz, n_rz);
  const double beta = first ? 0.0 : rz / (sc->rz_prev + 1e-30);
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double d = 0.0;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double az = row_dot<TPR>(ptr, col, val, z, row, valid, lane);
    if (valid && lane == 0) {
      const double pn = z[row] + beta * p[row];
      const double apn = az + beta * Ap[row];
      p[row] = pn;
      Ap[row] = apn;
      d = fma(pn, apn, d);
    }
  }
  d = block_sum(d);
  if (threadIdx.x == 0) part_pAp[blockIdx.x] = d;
}

// x += alpha p ; r -= alpha Ap ; partial r.r ; V-cycle pre-smoothing from zero: xv = s .* r
__global__ void __launch_bounds__(BS) k_pcg_step(int n, double* __restrict__ x, double* __restrict__ r,
                                                 const double* __restrict__ p, const double* __restrict__ Ap,
                                                 const double* __restrict__ s0, double* __restrict__ xv,
                                                 const double* __restrict__ part_pAp, int n_pap,
                                                 const double* __restrict__ part_rz, int n_rz,
                                                 double* __restrict__ part_r2, Scalars* sc) {
  if (sc->done) return;
  const double pAp = reduce_partials(part_pAp, n_pap);
  const double rz = reduce_partials(part_rz, n_rz);
  const double alpha = rz / (pAp + 1e-30);
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
    x[i] = x[i] + alpha * p[i];
    const double ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    d = fma(ri, ri, d);
    if (s0) xv[i] = s0[i] * ri;
  }
  d = block_sum(d);
  if (threadIdx.x == 0) {
    part_r2[blockIdx.x] = d;
    if (blockIdx.x == 0) {
      sc->rz_prev = rz;
      sc->it += 1;
    }
  }
}

// V-cycle level-0 residual with the convergence test: stops the solve when r.r <= tol2.
template <int TPR>
__global__ void __launch_bounds__(BS) k_vc_residual0(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                     const double* __restrict__ val, const double* __restrict__ xv,
                                                     const double* __restrict__ r, double* __restrict__ res,
                                                     const double* __restrict__ part_r2, int n_r2, Scalars* sc) {
  if (sc->done) return;
  const double r2 = reduce_partials(part_r2, n_r2);
  if (r2 <= sc->tol2 || sc->it >= sc->maxiter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = 1;
    return;
  }
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double ax = row_dot<TPR>(ptr, col, val, xv, row, valid, lane);
    if (valid && lane == 0) res[row] = r[row] - ax;
  }
}

// restriction b_c = R res, fused with the coarse pre-smoothing from zero x_c = s_c .* b_c
template <int TPR>
__global__ void __launch_bounds__(BS) k_restrict(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const double* __restrict__ val, const double* __restrict__ res,
                                                 double* __restrict__ bc, const double* __restrict__ sc_diag,
                                                 double* __restrict__ xc, const int* __restrict__ done) {
  if (done && *done) return;
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double v = row_dot<TPR>(ptr, col, val, res, row, valid, lane);
    if (valid && lane == 0) {
      bc[row] = v;
      if (sc_diag) xc[row] = sc_diag[row] * v;
    }
  }
}

// dense coarsest solve x = Ainv b (row-major n x n), one warp per row
__global__ void __launch_bounds__(BS) k_dense_mv(int n, const double* __restrict__ Ainv, const double* __restrict__ b,
                                                 double* __restrict__ x, const int* __restrict__ done) {
  if (done && *done) return;
  const int lane = threadIdx.x & 31;
  for (int row = blockIdx.x * (BS / 32) + threadIdx.x / 32; row < n; row += gridDim.x * (BS / 32)) {
    const double* a = Ainv + (size_t)row * n;
    double acc = 0.0;
    for (int k = lane; k < n; k += 32) acc = fma(a[k], b[k], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[row] = acc;
  }
}

// post-smoothing that also produces the PCG partial r.z when it writes the level-0 result
template <int TPR>
__global__ void __launch_bounds__(BS) k_smooth_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                   const double* __restrict__ val, const double* __restrict__ x,
                                                   const double* __restrict__ b, const double* __restrict__ s,
                                                   double* __restrict__ y, double* __restrict__ part,
                                                   const int* __restrict__ done) {
  if (done && *done) return;
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double d = 0.0;
  for (int rb = blockIdx.x * RPB; rb < n; rb += gridDim.x * RPB) {
    const int row = rb + threadIdx.x / TPR;
    const bool valid = row < n;
    const double ax = row_dot<TPR>(ptr, col, val, x, row, valid, lane);
    if (valid && lane == 0) {
      const double yi = x[row] + s[row] * (b[row] - ax);
      y[row] = yi;
      d = fma(b[row], yi, d);
    }
  }
  if (part) {
    d = block_sum(d);
    if (threadIdx.x == 0) part[blockIdx.x] = d;
  }
}

// ------------------------------------------------------------------------------------------
// vector kernels
// ------------------------------------------------------------------------------------------
// part = x.y (y == nullptr: x.x)
__global__ void __launch_bounds__(BS) k_dot(int n, const double* __restrict__ x, const double* __restrict__ y,
                                            double* __restrict__ part) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) d = fma(x[i], y ? y[i] : x[i], d);
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

__global__ void __launch_bounds__(BS) k_sum(int n, const double* __restrict__ x, double* __restrict__ part) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) d += x[i];
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// x -= sum(part)/n
__global__ void __launch_bounds__(BS) k_sub_mean(int n, double* __restrict__ x, const double* __restrict__ part,
                                                 int n_part) {
  const double mean = reduce_partials(part, n_part) / (double)n;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) x[i] = x[i] - mean;
}

// PCG initialisation: tol2 = tol^2 * sum(part_bb), bnorm2 stored; x *= mask (optional)
__global__ void k_pcg_init_scalars(Scalars* sc, const double* __restrict__ part_bb, int n_bb, double tol,
                                   int maxiter) {
  const double bb = reduce_partials(part_bb, n_bb);
  if (threadIdx.x == 0) {
    sc->tol2 = tol * tol * bb;
    sc->it = 0;
    sc->done = 0;
    sc->maxiter = maxiter;
    sc->rz_prev = 0.0;
  }
}

// ------------------------------------------------------------------------------------------
// energy, local Hessian and demag source over the magnetic rows
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
  int single_axis;
  int axis0;            // material whose axis every entry uses when single_axis
};

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
    }
  }
  ax = group_sum<TPR>(ax);
  ay = group_sum<TPR>(ay);
  az = group_sum<TPR>(az);
}

// g = (K m + G U + g_z) / V_mag on the magnetic rows; partial of m.(g_quad + 2 g_z)
template <int TPR>
__global__ void __launch_bounds__(BS) k_energy_grad(EnergyDev op, const double* __restrict__ m,
                                                    const double* __restrict__ U, const double* __restrict__ Mn,
                                                    double Bx, double By, double Bz, const double* __restrict__ Bbias,
                                                    double inv_Vmag, double* __restrict__ g,
                                                    double* __restrict__ part) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double en = 0.0;
  for (int rb = blockIdx.x * RPB; rb < op.n_rows; rb += gridDim.x * RPB) {
    const int r = rb + threadIdx.x / TPR;
    const bool valid = r < op.n_rows;
    double ax, ay, az;
    exch_aniso_row<TPR>(op, r, valid, lane, m, ax, ay, az);
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
    ux = group_sum<TPR>(ux);
    uy = group_sum<TPR>(uy);
    uz = group_sum<TPR>(uz);
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
      en += m[3 * a] * (gx + zx) + m[3 * a + 1] * (gy + zy) + m[3 * a + 2] * (gz + zz);
      g[3 * a] = gx * inv_Vmag;
      g[3 * a + 1] = gy * inv_Vmag;
      g[3 * a + 2] = gz * inv_Vmag;
    }
  }
  en = block_sum(en);
  if (threadIdx.x == 0) part[blockIdx.x] = en;
}

// out = C v / V_mag on the magnetic rows
template <int TPR>
__global__ void __launch_bounds__(BS) k_local_grad(EnergyDev op, const double* __restrict__ v, double inv_Vmag,
                                                   double* __restrict__ out) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  for (int rb = blockIdx.x * RPB; rb < op.n_rows; rb += gridDim.x * RPB) {
    const int r = rb + threadIdx.x / TPR;
    const bool valid = r < op.n_rows;
    double ax, ay, az;
    exch_aniso_row<TPR>(op, r, valid, lane, v, ax, ay, az);
    if (valid && lane == 0) {
      const int a = op.rows[r];
      out[3 * a] = ax * inv_Vmag;
      out[3 * a + 1] = ay * inv_Vmag;
      out[3 * a + 2] = az * inv_Vmag;
    }
  }
}

// Inner-PCG operator P p = C p - (m.Cp) m - (m.g_ext) p + reg p on the magnetic rows; partial p.Pp
template <int TPR>
__global__ void __launch_bounds__(BS) k_apply_P(EnergyDev op, const double* __restrict__ m,
                                                const double* __restrict__ gext, const double* __restrict__ p,
                                                double reg, double inv_Vmag, double* __restrict__ Ap,
                                                double* __restrict__ part) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double d = 0.0;
  for (int rb = blockIdx.x * RPB; rb < op.n_rows; rb += gridDim.x * RPB) {
    const int r = rb + threadIdx.x / TPR;
    const bool valid = r < op.n_rows;
    double ax, ay, az;
    exch_aniso_row<TPR>(op, r, valid, lane, p, ax, ay, az);
    if (valid && lane == 0) {
      const int a = op.rows[r];
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
  }
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// b = D m on the magnetic rows (other rows are left untouched), partial b.b
template <int TPR>
__global__ void __launch_bounds__(BS) k_rhs(EnergyDev op, const double* __restrict__ m, double* __restrict__ b,
                                            double* __restrict__ part) {
  constexpr int RPB = BS / TPR;
  const int lane = threadIdx.x % TPR;
  double bb = 0.0;
  for (int rb = blockIdx.x * RPB; rb < op.n_rows; rb += gridDim.x * RPB) {
    const int r = rb + threadIdx.x / TPR;
    const bool valid = r < op.n_rows;
    double acc = 0.0;
    if (valid) {
      const int s = op.ptr[r], e = op.ptr[r + 1];
      for (int k = s + lane; k < e; k += TPR) {
        const int j = op.col[k];
        acc += op.dx[k] * __ldg(m + 3 * j) + op.dy[k] * __ldg(m + 3 * j + 1) + op.dz[k] * __ldg(m + 3 * j + 2);
      }
    }
    acc = group_sum<TPR>(acc);
    if (valid && lane == 0) {
      b[op.rows[r]] = acc;
      bb = fma(acc, acc, bb);
    }
  }
  if (part) {
    bb = block_sum(bb);
    if (threadIdx.x == 0) part[blockIdx.x] = bb;
  }
}

// ------------------------------------------------------------------------------------------
// minimizer vector kernels (3-vectors per node, xyz interleaved)
// ------------------------------------------------------------------------------------------
// g_tan = P_m(g .* inv_M_rel), g_tan_ext = P_m(g); partial max |g_tan|
__global__ void __launch_bounds__(BS) k_tangent2(int N, const double* __restrict__ m, const double* __restrict__ g,
                                                 const double* __restrict__ inv_M_rel, double* __restrict__ gt,
                                                 double* __restrict__ gte, double* __restrict__ part_max) {
  double mx_ = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double g0 = g[3 * i], g1 = g[3 * i + 1], g2 = g[3 * i + 2];
    const double w = inv_M_rel[i];
    const double s0 = g0 * w, s1 = g1 * w, s2 = g2 * w;
    const double ds = m0 * s0 + m1 * s1 + m2 * s2;
    const double t0 = s0 - ds * m0, t1 = s1 - ds * m1, t2 = s2 - ds * m2;
    const double de = m0 * g0 + m1 * g1 + m2 * g2;
    if (gt) {
      gt[3 * i] = t0;
      gt[3 * i + 1] = t1;
      gt[3 * i + 2] = t2;
    }
    gte[3 * i] = g0 - de * m0;
    gte[3 * i + 1] = g1 - de * m1;
    gte[3 * i + 2] = g2 - de * m2;
    mx_ = fmax(mx_, fmax(fabs(t0), fmax(fabs(t1), fabs(t2))));
  }
  mx_ = block_max(mx_);
  if (threadIdx.x == 0) part_max[blockIdx.x] = mx_;
}

// out = P_m(v)
__global__ void __launch_bounds__(BS) k_tangent(int N, const double* __restrict__ m, const double* __restrict__ v,
                                                double* __restrict__ out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double d = m0 * v[3 * i] + m1 * v[3 * i + 1] + m2 * v[3 * i + 2];
    out[3 * i] = v[3 * i] - d * m0;
    out[3 * i + 1] = v[3 * i + 1] - d * m1;
    out[3 * i + 2] = v[3 * i + 2] - d * m2;
  }
}

// Cayley update with renormalisation: m_out = cayley(m, H, tau)
__global__ void __launch_bounds__(BS) k_cayley(int N, const double* __restrict__ m, const double* __restrict__ H,
                                               double tau, double* __restrict__ out) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double k0 = 0.5 * tau * H[3 * i], k1 = 0.5 * tau * H[3 * i + 1], k2 = 0.5 * tau * H[3 * i + 2];
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    const double kk = k0 * k0 + k1 * k1 + k2 * k2;
    const double den = 1.0 + kk;
    const double km0 = k1 * m2 - k2 * m1, km1 = k2 * m0 - k0 * m2, km2 = k0 * m1 - k1 * m0;
    const double kd = k0 * m0 + k1 * m1 + k2 * m2;
    const double n0 = ((1.0 - kk) * m0 + 2.0 * km0 + 2.0 * kd * k0) / den;
    const double n1 = ((1.0 - kk) * m1 + 2.0 * km1 + 2.0 * kd * k1) / den;
    const double n2 = ((1.0 - kk) * m2 + 2.0 * km2 + 2.0 * kd * k2) / den;
    const double nr = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    out[3 * i] = n0 / nr;
    out[3 * i + 1] = n1 / nr;
    out[3 * i + 2] = n2 / nr;
  }
}

// m <- m / |m|
__global__ void __launch_bounds__(BS) k_normalize(int N, double* __restrict__ m) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double a = m[3 * i], b = m[3 * i + 1], c = m[3 * i + 2];
    const double nr = sqrt(a * a + b * b + c * c);
    m[3 * i] = a / nr;
    m[3 * i + 1] = b / nr;
    m[3 * i + 2] = c / nr;
  }
}

// z = r .* w (per node), partial r.z
__global__ void __launch_bounds__(BS) k_scale3_dot(int N, const double* __restrict__ r, const double* __restrict__ w,
                                                   double* __restrict__ z, double* __restrict__ part) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    const double z0 = r[3 * i] * s, z1 = r[3 * i + 1] * s, z2 = r[3 * i + 2] * s;
    z[3 * i] = z0;
    z[3 * i + 1] = z1;
    z[3 * i + 2] = z2;
    d += r[3 * i] * z0 + r[3 * i + 1] * z1 + r[3 * i + 2] * z2;
  }
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// y += a p ; r -= a Ap ; z = r .* w ; partial r.z   (inner PCG of the local Hessian)
__global__ void __launch_bounds__(BS) k_inner_step(int N, double a, double* __restrict__ y, double* __restrict__ r,
                                                   const double* __restrict__ p, const double* __restrict__ Ap,
                                                   const double* __restrict__ w, double* __restrict__ z,
                                                   double* __restrict__ part, int update) {
  double d = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double s = w[i];
    for (int c = 0; c < 3; ++c) {
      double rc = r[3 * i + c];
      if (update) {
        y[3 * i + c] = y[3 * i + c] + a * p[3 * i + c];
        rc = rc - a * Ap[3 * i + c];
        r[3 * i + c] = rc;
      }
      const double zc = rc * s;
      z[3 * i + c] = zc;
      d += rc * zc;
    }
  }
  d = block_sum(d);
  if (threadIdx.x == 0) part[blockIdx.x] = d;
}

// y = x + a * y (axpby with unit x)
__global__ void __launch_bounds__(BS) k_xpay(int n, const double* __restrict__ x, double a, double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = x[i] + a * y[i];
}

// y = a * x + b * y
__global__ void __launch_bounds__(BS) k_axpby(int n, double a, const double* __restrict__ x, double b,
                                              double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * x[i] + b * y[i];
}

// y *= a
__global__ void __launch_bounds__(BS) k_scale(int n, double a, double* __restrict__ y) {
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) y[i] = a * y[i];
}

// partial max |x|
__global__ void __launch_bounds__(BS) k_absmax(int n, const double* __restrict__ x, double* __restrict__ part) {
  double v = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) v = fmax(v, fabs(x[i]));
  v = block_max(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// partial max |x - y|
__global__ void __launch_bounds__(BS) k_absmaxdiff(int n, const double* __restrict__ x, const double* __restrict__ y,
                                                   double* __restrict__ part) {
  double v = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) v = fmax(v, fabs(x[i] - y[i]));
  v = block_max(v);
  if (threadIdx.x == 0) part[blockIdx.x] = v;
}

// d = -y + beta * P_m(d_prev); H = m x d; partials d.gte (slot 0) and g_raw.d (slot 1, stride n_part)
__global__ void __launch_bounds__(BS) k_direction(int N, const double* __restrict__ m, const double* __restrict__ y,
                                                  const double* __restrict__ dprev, double beta,
                                                  const double* __restrict__ gte, const double* __restrict__ graw,
                                                  double* __restrict__ d, double* __restrict__ part_dg,
                                                  double* __restrict__ part_pg) {
  double s1 = 0.0, s2 = 0.0;
  for (int i = blockIdx.x * BS + threadIdx.x; i < N; i += gridDim.x * BS) {
    const double m0 = m[3 * i], m1 = m[3 * i + 1], m2 = m[3 * i + 2];
    double dp0 = 0, dp1 = 0, dp2 = 0;
    if (dprev) {
      const double a = m0 * dprev[3 * i] + m1 * dprev[3 * i + 1] + m2 * dprev[3 * i + 2];
      dp0 = dprev[3 * i] - a * m0;
      dp1 = dprev[3 * i + 1] - a * m1;
      dp2 = dprev[3 * i + 2] - a * m2;
    }
    const double d0 = -y[3 * i] + beta * dp0, d1 = -y[3 * i + 1] + beta * dp1, d2 = -y[3 * i + 2] + beta * dp2;
    d[3 * i] = d0;
    d[3 * i + 1] = d1;
    d[3 * i + 2] = d2;
    s1 += d0 * gte[3 * i] + d1 * gte[3 * i + 1] + d2 * gte[3 * i + 2];
    s2 += graw[3 * i] * d0 + graw[3 * i + 1] * d1 + graw[3 * i + 2] * d2;
  }
  s1 = block_sum(s1);
  s2 = block_sum(s2);
  if (threadIdx.x == 0) {
    part_dg[blockIdx.x] = s1;
    part_pg[blockIdx.x] = s2;
  }
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

}  // namespace mmk
